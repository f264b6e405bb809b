"""The numpy restatement of the benchmark scenes and camera paths
(oracle/scene_gen.py, which the CPU reference arm of bench.py uses so that it
never loads the product library) against the product's own generator: the
same voxels in the same order and the same view bits. No GPU."""
import numpy as np
import pytest


@pytest.mark.parametrize("depth,shell,seed", [(8, True, 11), (8, False, 3), (9, True, 2024)])
def test_terrain_voxels_identical(svo, depth, shell, seed):
    import scene_gen as scene

    want = svo.terrain_voxels(seed, depth, shell)
    got = scene.terrain_voxels(seed, depth, shell)
    for a, b, name in zip(want, got, "xyzc"):
        assert a.size == b.size, name
        assert np.array_equal(np.asarray(a, np.uint32), b), name


@pytest.mark.parametrize("kind", [1, 2])
def test_camera_paths_identical(svo, kind):
    import scene_gen as scene

    for depth in (9, 11):
        for frame in (0, 1, 5, 63, 64, 200, 511):
            v = svo.camera_path(kind, depth, frame, 64, 32)
            pos, m = scene.camera_path(kind, depth, frame)
            assert np.array_equal(v.pos_array.view(np.uint32), pos.view(np.uint32)), (depth, frame)
            assert np.array_equal(v.m_array.view(np.uint32), m.view(np.uint32)), (depth, frame)
