"""Pins the CPU oracle (oracle/svo_oracle.cpp) to the reference.

Two anchors: the golden fixtures of tests/golden (made by the reference's own
kernel.cl/octree.h compiled for the host, see make_golden.py), which travel
with the repository; and, where the reference tree is present, direct
comparisons against that compiled reference on further seeded cases.
"""
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


@pytest.fixture(scope="module")
def golden():
    with open(os.path.join(GOLDEN, "golden.json")) as f:
        meta = json.load(f)
    arrays = dict(np.load(os.path.join(GOLDEN, "golden.npz")))
    return meta, arrays


@pytest.fixture(scope="module")
def golden_scenes(svo, orc, golden):
    meta, _ = golden
    scenes = {}
    for case in meta["builder"]:
        x, y, z, c = svo.terrain_voxels(case["seed"], case["depth"], case["shell"])
        assert _digest(x, y, z, c) == case["voxel_digest"], "the synthetic terrain generator changed"
        scenes[(case["depth"], case["seed"], case["shell"])] = (x, y, z, c)
    return scenes


def test_log2_known_answer(orc):
    # kernel.cl:202 takes int(log2(float(v))) for v = x0r & (2^depth-1); the
    # oracle and the GPU use 31-clz(v). Equal for every v the walk can form.
    assert orc.log2_kat(1 << 13) == 0


def test_oracle_builder_matches_golden(orc, golden, golden_scenes):
    meta, _ = golden
    for case in meta["builder"]:
        x, y, z, c = golden_scenes[(case["depth"], case["seed"], case["shell"])]
        words, root = orc.build_octree(case["depth"], x, y, z, c)
        assert words.size == case["n_words"] and root == case["root"]
        assert _digest(words) == case["words_digest"]


def test_oracle_full_raycast_matches_golden(orc, golden, golden_scenes):
    meta, arrays = golden
    for case in meta["full"]:
        x, y, z, c = golden_scenes[(case["depth"], case["seed"], case["shell"])]
        words, root = orc.build_octree(case["depth"], x, y, z, c)
        k = case["key"]
        col, xyzw, _, _ = orc.raycast_full(case["depth"], words, root, arrays[k + "_pos"], arrays[k + "_m"],
                                           case["W"], case["H"], case["fov"], case["fov"])
        assert np.array_equal(col, arrays[k + "_colour"])
        assert np.array_equal(np.ascontiguousarray(xyzw[:, :3]).view(np.uint32), arrays[k + "_xyz"].view(np.uint32))


def test_oracle_warp_frames_match_golden(svo, orc, golden, golden_scenes):
    meta, arrays = golden
    for case in meta["warp"]:
        depth = case["depth"]
        x, y, z, c = golden_scenes[(depth, case["seed"], case["shell"])]
        words, root = orc.build_octree(depth, x, y, z, c)
        w = orc.Warp(depth, case["W"], case["H"])
        k = case["key"]
        for f, want in enumerate(case["per_frame"]):
            w.frame(words, root, arrays[f"{k}_f{f}_pos"], arrays[f"{k}_f{f}_m"], f)
            screen, back = w.screen(), w.back()
            ne = screen[2] != svo.EMPTY_PIXEL
            assert w.hole_count() == want["holes"], f"frame {f}"
            assert _digest(w.ids()) == want["ids_digest"], f"frame {f}: hole list"
            assert _digest(screen[0]) == want["plane0_digest"], f"frame {f}: displayed plane"
            assert _digest(screen[2]) == want["plane2_digest"], f"frame {f}: cache plane"
            assert _digest(np.ascontiguousarray(back[2][ne][:, :3])) == want["xyz2_digest"], f"frame {f}: coords"
            assert _digest(w.tex()) == want["tex_digest"], f"frame {f}: BGRX"
        assert np.array_equal(w.screen()[0], arrays[k + "_last_plane0"])
        assert np.array_equal(w.tex(), arrays[k + "_last_tex"])


# ------------------------------------------- against the compiled reference --
needs_ref = pytest.mark.skipif(not __import__("oracle").ref_available(),
                               reason="reference sources not compiled here (oracle/_ref)")


@needs_ref
@pytest.mark.parametrize("depth,seed,shell,boxes", [(8, 31, True, 0), (9, 32, True, 0), (10, 33, True, 0),
                                                    (8, 34, False, 0), (9, 35, True, 40)])
def test_oracle_builder_matches_reference(svo, orc, depth, seed, shell, boxes):
    x, y, z, c = svo.terrain_voxels(seed, depth, shell, boxes)
    rw, rr = orc.build_octree(depth, x, y, z, c, which="reference")
    ow, orr = orc.build_octree(depth, x, y, z, c)
    assert rr == orr and np.array_equal(rw, ow)


@needs_ref
def test_oracle_builder_duplicates_and_order(orc):
    # Re-inserted voxels: leaf keeps the last colour, nodes the first one.
    rng = np.random.default_rng(3)
    n = 20000
    x = rng.integers(0, 256, n, dtype=np.uint32)
    y = rng.integers(0, 64, n, dtype=np.uint32)
    z = rng.integers(0, 256, n, dtype=np.uint32)
    c = rng.integers(1, 1 << 32, n, dtype=np.uint64).astype(np.uint32)
    x = np.concatenate([x, x[:5000]])
    y = np.concatenate([y, y[:5000]])
    z = np.concatenate([z, z[:5000]])
    c = np.concatenate([c, (c[:5000] ^ 0x5a5a5a00) | 1])
    assert np.array_equal(orc.build_octree(8, x, y, z, c, which="reference")[0], orc.build_octree(8, x, y, z, c)[0])


@needs_ref
@pytest.mark.parametrize("depth,seed,shell,kind,frame,W,H,fov", [
    (8, 31, True, 0, 0, 120, 90, 1.1547),
    (9, 32, True, 1, 33, 160, 100, 1.0),
    (10, 33, True, 2, 7, 128, 72, 1.0),
    (8, 34, False, 3, 4, 100, 100, 0.8),
    (9, 35, True, 3, 11, 77, 41, 1.3),
])
def test_oracle_full_raycast_matches_reference(svo, orc, depth, seed, shell, kind, frame, W, H, fov):
    x, y, z, c = svo.terrain_voxels(seed, depth, shell, 40 if seed == 35 else 0)
    words, root = orc.build_octree(depth, x, y, z, c)
    v = svo.camera_path(kind, depth, frame, W, H, fov=fov)
    rc, rx, _, _ = orc.raycast_full(depth, words, root, v.pos_array, v.m_array, W, H, fov, fov, which="reference")
    oc, ox, _, _ = orc.raycast_full(depth, words, root, v.pos_array, v.m_array, W, H, fov, fov)
    assert np.array_equal(rc, oc)
    assert np.array_equal(np.ascontiguousarray(rx[:, :3]).view(np.uint32),
                          np.ascontiguousarray(ox[:, :3]).view(np.uint32))


@needs_ref
@pytest.mark.parametrize("depth,seed,shell,kind,frames,W,H", [
    (8, 31, True, 1, 36, 96, 64),
    (9, 32, True, 2, 8, 112, 80),
    (8, 34, False, 3, 5, 48, 32),
    (8, 31, True, 1, 4, 40, 24),  # ragged tiles on both axes
])
def test_oracle_warp_frames_match_reference(svo, orc, depth, seed, shell, kind, frames, W, H):
    x, y, z, c = svo.terrain_voxels(seed, depth, shell)
    words, root = orc.build_octree(depth, x, y, z, c)
    ref = orc.Warp(depth, W, H, which="reference")
    mine = orc.Warp(depth, W, H)
    for f in range(frames):
        v = svo.camera_path(kind, depth, f, W, H)
        ref.frame(words, root, v.pos_array, v.m_array, f)
        mine.frame(words, root, v.pos_array, v.m_array, f)
        rs, ms = ref.screen(), mine.screen()
        assert np.array_equal(rs, ms), f"frame {f}: colour planes"
        assert ref.hole_count() == mine.hole_count()
        assert np.array_equal(ref.ids(), mine.ids()), f"frame {f}: hole list"
        assert np.array_equal(ref.prefill(), mine.prefill())
        assert np.array_equal(ref.tex(), mine.tex())
        ne = rs[2] != svo.EMPTY_PIXEL
        rb, mb = ref.back(), mine.back()
        assert np.array_equal(np.ascontiguousarray(rb[2][ne][:, :3]).view(np.uint32),
                              np.ascontiguousarray(mb[2][ne][:, :3]).view(np.uint32)), f"frame {f}: coords"


@needs_ref
def test_oracle_alternating_cache_target_matches_reference(svo, orc):
    # raycast.h:395's commented-out target ((frame>>4)%2)+1: both cache planes
    # are projected and the one not copied into keeps its cleared sources.
    depth, W, H = 9, 96, 64
    x, y, z, c = svo.terrain_voxels(41, depth, True)
    words, root = orc.build_octree(depth, x, y, z, c)
    ref = orc.Warp(depth, W, H, which="reference")
    mine = orc.Warp(depth, W, H)
    for f in range(36):
        v = svo.camera_path(2, depth, f, W, H)
        ref.frame(words, root, v.pos_array, v.m_array, f, cache_mode=1)
        mine.frame(words, root, v.pos_array, v.m_array, f, cache_mode=1)
        assert np.array_equal(ref.screen(), mine.screen()), f"frame {f}"
        assert np.array_equal(ref.ids(), mine.ids()) and np.array_equal(ref.tex(), mine.tex())


@needs_ref
@pytest.mark.parametrize("cache_mode", [0, 1])
def test_oracle_coarse_refresh_matches_reference(svo, orc, cache_mode):
    # raycast.h:235-261's disabled raycast_fine pass (one ray per 2x2 block of
    # a quadrant, before the hole gather), alone and with the alternating target.
    depth, W, H = 9, 96, 64
    x, y, z, c = svo.terrain_voxels(43, depth, True)
    words, root = orc.build_octree(depth, x, y, z, c)
    ref = orc.Warp(depth, W, H, which="reference")
    mine = orc.Warp(depth, W, H)
    for f in range(20):
        v = svo.camera_path(2, depth, f, W, H)
        ref.frame(words, root, v.pos_array, v.m_array, f, cache_mode=cache_mode, coarse=True)
        mine.frame(words, root, v.pos_array, v.m_array, f, cache_mode=cache_mode, coarse=True)
        rs, ms = ref.screen(), mine.screen()
        assert np.array_equal(rs, ms), f"frame {f}"
        assert np.array_equal(ref.ids(), mine.ids()) and np.array_equal(ref.tex(), mine.tex()), f"frame {f}"
        ne = rs[2] != svo.EMPTY_PIXEL
        assert np.array_equal(np.ascontiguousarray(ref.back()[2][ne][:, :3]).view(np.uint32),
                              np.ascontiguousarray(mine.back()[2][ne][:, :3]).view(np.uint32)), f"frame {f}"


def test_oracle_coarse_refresh_fills_holes(svo, orc):
    # the coarse pass leaves fewer whole 2x2 holes for the hole gather
    depth, W, H = 8, 64, 48
    x, y, z, c = svo.terrain_voxels(31, depth, True)
    words, root = orc.build_octree(depth, x, y, z, c)
    a, b = orc.Warp(depth, W, H), orc.Warp(depth, W, H)
    for f in range(12):
        v = svo.camera_path(2, depth, f, W, H)
        a.frame(words, root, v.pos_array, v.m_array, f)
        b.frame(words, root, v.pos_array, v.m_array, f, coarse=True)
    assert b.hole_count() <= a.hole_count()


# ------------------------------------------------ the benchmark's own size --
@pytest.mark.parametrize("idx", [0, 1])
def test_oracle_fullsize_matches_golden(svo, orc, golden, idx):
    """1920x1024 at depth 11 (the benchmark's terrain; words from the
    reference builder) and depth 12: one full raycast and four warp frames
    against the reference's digests -- where the compact format's offsets and
    local roots span their full range and horizon rays run to VIEW_DIST_MAX."""
    meta, _ = golden
    case = meta["fullsize"][idx]
    depth, W, H = case["depth"], case["W"], case["H"]
    x, y, z, c = svo.terrain_voxels(case["seed"], depth, case["shell"])
    assert _digest(x, y, z, c) == case["voxel_digest"], "the synthetic terrain generator changed"
    if case["builder"] == "reference":
        words, root = orc.build_octree(depth, x, y, z, c)
    else:
        o = svo.build_terrain(depth, case["seed"], case["shell"])
        words, root = o.words, o.root
    del x, y, z, c
    assert words.size == case["n_words"] and root == case["root"] and _digest(words) == case["words_digest"]
    v = svo.camera_path(1, depth, case["frame"], W, H)
    assert _digest(v.pos_array, v.m_array) == case["camera_digest"]
    col, xyzw, _, st = orc.raycast_full(depth, words, root, v.pos_array, v.m_array, W, H)
    assert _digest(col) == case["colour_digest"], "full raycast colour words"
    assert _digest(np.ascontiguousarray(xyzw[:, :3])) == case["xyz_digest"], "full raycast hit positions"
    w = orc.Warp(depth, W, H)
    for f, want in enumerate(case["warp"]):
        v = svo.camera_path(1, depth, f, W, H)
        assert _digest(v.pos_array, v.m_array) == want["camera_digest"]
        w.frame(words, root, v.pos_array, v.m_array, f)
        screen = w.screen()
        assert w.hole_count() == want["holes"], f"frame {f}"
        assert _digest(w.ids()) == want["ids_digest"], f"frame {f}: hole list"
        assert _digest(screen[0]) == want["plane0_digest"], f"frame {f}: displayed plane"
        assert _digest(screen[2]) == want["plane2_digest"], f"frame {f}: cache plane"
        assert _digest(w.tex()) == want["tex_digest"], f"frame {f}: BGRX"


@needs_ref
def test_oracle_fullsize_depth11_matches_reference_directly(svo, orc):
    """The depth-11 benchmark scene at 1920x1024, oracle against the compiled
    reference itself on a frame the golden set does not hold."""
    depth, W, H = 11, 1920, 1024
    o = svo.build_terrain(depth, 2024, True)
    v = svo.camera_path(1, depth, 131, W, H)
    rc, rx, _, _ = orc.raycast_full(depth, o.words, o.root, v.pos_array, v.m_array, W, H, which="reference")
    oc, ox, _, _ = orc.raycast_full(depth, o.words, o.root, v.pos_array, v.m_array, W, H)
    assert np.array_equal(rc, oc)
    assert np.array_equal(np.ascontiguousarray(rx[:, :3]).view(np.uint32),
                          np.ascontiguousarray(ox[:, :3]).view(np.uint32))
