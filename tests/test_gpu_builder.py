"""The GPU octree builder (svo_octree_build) against the host builder, which
the builder tests pin to the reference's set_voxel + convert_tree_blocks:
identical words and root word on terrain, occluder boxes, random voxels with
re-insertions, single-voxel and empty scenes, up to the depth-11 benchmark
terrain."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def _gpu_build(svo, ctx, x, y, z, c, depth, initial_words=0):
    dev = [torch.from_numpy(np.ascontiguousarray(a, np.uint32).view(np.int32)).cuda() for a in (x, y, z, c)]
    torch.cuda.synchronize()
    ctx.build_octree(*(t.data_ptr() for t in dev), len(x), depth, initial_words)
    return ctx.download_octree()


def _host_build(svo, x, y, z, c, depth):
    b = svo.Builder(depth)
    b.set_voxels(x, y, z, c)
    return b.finish()


@pytest.mark.parametrize("depth,seed,shell,boxes", [(8, 31, True, 0), (9, 35, True, 40), (10, 33, False, 0),
                                                    (12, 5, True, 0)])
def test_gpu_builder_matches_host_builder(svo, gpu_ctx, depth, seed, shell, boxes):
    x, y, z, c = svo.terrain_voxels(seed, depth, shell, boxes)
    want = _host_build(svo, x, y, z, c, depth)
    got = _gpu_build(svo, gpu_ctx, x, y, z, c, depth)
    assert got.root == want.root and got.words.size == want.words.size
    assert np.array_equal(got.words, want.words)


def test_gpu_builder_reinsertions_and_order(svo, gpu_ctx):
    rng = np.random.default_rng(3)
    n = 200000
    x = rng.integers(0, 512, n, dtype=np.uint32)
    y = rng.integers(0, 128, n, dtype=np.uint32)
    z = rng.integers(0, 512, n, dtype=np.uint32)
    c = rng.integers(1, 1 << 32, n, dtype=np.uint64).astype(np.uint32)
    c[::97] = 0  # zero leaf colours are skipped in the byte records
    x, y, z = (np.concatenate([a, a[:50000]]) for a in (x, y, z))
    c = np.concatenate([c, (c[:50000] ^ 0x5a5a5a00) | 1])
    want = _host_build(svo, x, y, z, c, 9)
    got = _gpu_build(svo, gpu_ctx, x, y, z, c, 9)
    assert got.root == want.root and np.array_equal(got.words, want.words)


def test_gpu_builder_small_and_empty(svo, gpu_ctx):
    one = [np.array([v], np.uint32) for v in (3, 200, 17, 0x12345678)]
    want = _host_build(svo, *one, 8)
    got = _gpu_build(svo, gpu_ctx, *one, 8)
    assert got.root == want.root and np.array_equal(got.words, want.words)
    e = [np.zeros(0, np.uint32)] * 4
    want = _host_build(svo, *e, 8)
    got = _gpu_build(svo, gpu_ctx, *e, 8, 0)
    assert got.root == want.root == 0 and np.array_equal(got.words, want.words)


def test_gpu_builder_rejects_bad_input(svo, gpu_ctx):
    bad = [np.array([v], np.uint32) for v in (300, 1, 1, 5)]
    with pytest.raises(svo.SvoError):
        _gpu_build(svo, gpu_ctx, *bad, 8)


def test_gpu_built_octree_renders_like_host_built(svo, orc, gpu_ctx):
    x, y, z, c = svo.terrain_voxels(31, 9, True)
    _gpu_build(svo, gpu_ctx, x, y, z, c, 9)
    t = gpu_ctx.target(96, 64)
    v = svo.camera_path(1, 9, 5, 96, 64)
    gpu_ctx.raycast_full(t, v)
    col, _ = t.full()
    words, root = orc.build_octree(9, x, y, z, c)
    ocol, _, _, _ = orc.raycast_full(9, words, root, v.pos_array, v.m_array, 96, 64)
    assert np.array_equal(col, ocol)
    t.close()


def test_gpu_builder_full_size_terrain(svo, gpu_ctx):
    # the depth-11 benchmark scene
    x, y, z, c = svo.terrain_voxels(2024, 11, True)
    want = _host_build(svo, x, y, z, c, 11)
    got = _gpu_build(svo, gpu_ctx, x, y, z, c, 11)
    assert got.root == want.root and np.array_equal(got.words, want.words)
