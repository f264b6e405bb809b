"""Shared test setup: the gpu marker, import paths and cached scenes."""
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "sparse-voxel-octree-raycasting_gb300"))
sys.path.insert(0, os.path.join(ROOT, "oracle"))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")
    config.addinivalue_line("markers", "slow: larger CPU cases")


@pytest.fixture(scope="session")
def svo():
    import svo_gb300

    svo_gb300.load()
    return svo_gb300


@pytest.fixture(scope="session")
def orc():
    import oracle

    oracle.oracle()
    return oracle


_scene_cache = {}


@pytest.fixture(scope="session")
def scene(svo):
    """scene(depth, seed, shell, boxes=0) -> Octree built by the product builder (cached)."""

    def get(depth, seed, shell, boxes=0):
        key = (depth, seed, shell, boxes)
        if key not in _scene_cache:
            _scene_cache[key] = svo.build_terrain(depth, seed, shell, boxes)
        return _scene_cache[key]

    return get


@pytest.fixture(scope="session")
def gpu_ctx(svo):
    ctx = svo.Context(0)
    yield ctx
    ctx.close()
