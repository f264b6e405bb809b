"""The product's octree builder (libsvo_gb300.so, host side) against the oracle
builder and the golden fixtures: identical compact words and root word for
the same voxels in the same insertion order (src/octree/octree.h semantics)."""
import json
import os

import numpy as np
import pytest

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def _digest(*arrays):
    import hashlib

    h = hashlib.sha256()
    for a in arrays:
        h.update(np.ascontiguousarray(a).tobytes())
    return h.hexdigest()


def _product(svo, depth, x, y, z, c, initial_words=0):
    b = svo.Builder(depth)
    b.set_voxels(x, y, z, c)
    o = b.finish(initial_words)
    return o.words, o.root


def test_builder_matches_golden(svo):
    with open(os.path.join(GOLDEN, "golden.json")) as f:
        meta = json.load(f)
    for case in meta["builder"]:
        o = svo.build_terrain(case["depth"], case["seed"], case["shell"])
        assert o.words.size == case["n_words"] and o.root == case["root"]
        assert _digest(o.words) == case["words_digest"]
        assert o.voxels == case["voxels"]


@pytest.mark.parametrize("depth", [8, 9, 10, 11, 12])
def test_builder_random_voxels_with_duplicates(svo, orc, depth):
    rng = np.random.default_rng(depth)
    n = 30000
    D = 1 << depth
    # clustered so that blocks share nodes, plus re-insertions with new colours
    cx = rng.integers(0, D, 40)
    cz = rng.integers(0, D, 40)
    k = rng.integers(0, 40, n)
    x = ((cx[k] + rng.integers(0, 48, n)) % D).astype(np.uint32)
    z = ((cz[k] + rng.integers(0, 48, n)) % D).astype(np.uint32)
    y = rng.integers(0, min(D, 96), n).astype(np.uint32)
    c = rng.integers(1, 1 << 32, n, dtype=np.uint64).astype(np.uint32)
    dup = rng.integers(0, n, 4000)
    x, y, z = (np.concatenate([a, a[dup]]) for a in (x, y, z))
    c = np.concatenate([c, (c[dup] * 7) | 1])
    w1, r1 = _product(svo, depth, x, y, z, c)
    w2, r2 = orc.build_octree(depth, x, y, z, c)
    assert r1 == r2 and np.array_equal(w1, w2)


def test_builder_zero_colour_leaves_match_reference_quirk(svo, orc):
    # A zero colour word sets the mask bit but its byte is skipped
    # (octree.h:134); both builders must reproduce that layout.
    rng = np.random.default_rng(7)
    n = 5000
    x, y, z = (rng.integers(0, 256, n).astype(np.uint32) for _ in range(3))
    c = rng.integers(1, 255, n).astype(np.uint32)
    c[::17] = 0
    w1, r1 = _product(svo, 8, x, y, z, c)
    w2, r2 = orc.build_octree(8, x, y, z, c)
    assert r1 == r2 and np.array_equal(w1, w2)


def test_builder_single_voxels_at_corners(svo, orc):
    for depth in (8, 12):
        D = (1 << depth) - 1
        for (x, y, z) in [(0, 0, 0), (D, D, D), (D, 0, 0), (0, D, 0), (0, 0, D), (D // 2, D // 3, 7)]:
            args = [np.array([v], np.uint32) for v in (x, y, z, 0x1234567)]
            w1, r1 = _product(svo, depth, *args)
            w2, r2 = orc.build_octree(depth, *args)
            assert r1 == r2 and np.array_equal(w1, w2), (depth, x, y, z)


def test_builder_empty_scene(svo, orc):
    e = np.zeros(0, np.uint32)
    w1, r1 = _product(svo, 9, e, e, e, e)
    w2, r2 = orc.build_octree(9, e, e, e, e)
    assert r1 == r2 == 0 and np.array_equal(w1, w2)


def test_builder_custom_initial_words(svo, orc):
    x, y, z, c = svo.terrain_voxels(3, 8, True)
    w1, r1 = _product(svo, 8, x, y, z, c, initial_words=4096)
    w2, r2 = orc.build_octree(8, x, y, z, c, initial_words=4096)
    assert r1 == r2 and np.array_equal(w1, w2)
    assert w1.size < 2097152


def test_builder_rejects_bad_input(svo):
    with pytest.raises(svo.SvoError):
        svo.Builder(7)
    with pytest.raises(svo.SvoError):
        svo.Builder(13)
    b = svo.Builder(8)
    with pytest.raises(svo.SvoError):
        b.set_voxel(256, 0, 0, 1)
    b.set_voxel(1, 2, 3, 4)
    b.finish()
    with pytest.raises(svo.SvoError):
        b.finish()


def test_octree_file_round_trip(svo, tmp_path):
    o = svo.build_terrain(8, 21, True)
    p = str(tmp_path / "scene.svo")
    o.save(p)
    o2 = svo.Octree.load_file(p)
    assert o2.root == o.root and o2.depth == o.depth and np.array_equal(o2.words, o.words)
    with pytest.raises(svo.SvoError):
        svo.Octree.load_file(str(tmp_path / "missing.svo"))


@pytest.mark.slow
def test_builder_solid_depth9_terrain_matches_oracle(svo, orc):
    # The plain full raycast configuration's scene: 512^3, solid below the surface.
    x, y, z, c = svo.terrain_voxels(1234, 9, False)
    assert x.size > 30_000_000
    w1, r1 = _product(svo, 9, x, y, z, c)
    w2, r2 = orc.build_octree(9, x, y, z, c)
    assert r1 == r2 and np.array_equal(w1, w2)
