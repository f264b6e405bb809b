"""GPU parity: the CUDA path against the CPU oracle, bit for bit.

Colour words, hit positions (float bits), hit distances and hit voxels of the
full raycast; every plane, the hole list and the BGRX image of warp frames.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _full_oracle(orc, octree, view):
    return orc.raycast_full(octree.depth, octree.words, octree.root, view.pos_array, view.m_array, view.res_x,
                            view.res_y, view.fovx, view.fovy)


@pytest.mark.parametrize("depth,shell,kind,W,H,fov", [
    (8, True, 0, 160, 120, 1.1547),
    (9, True, 1, 256, 128, 1.0),
    (8, False, 3, 200, 152, 1.0),
    (9, False, 0, 512, 512, 1.1547),   # the plain full raycast configuration: 512^2, depth 9, solid terrain
    (10, True, 2, 160, 96, 1.0),
    (12, True, 1, 128, 80, 1.0),       # the deepest supported octree (4096^3)
])
def test_full_raycast_bit_exact(svo, orc, scene, gpu_ctx, depth, shell, kind, W, H, fov):
    octree = scene(depth, 1234, shell)
    gpu_ctx.upload(octree)
    tgt = gpu_ctx.target(W, H)
    view = svo.camera_path(kind, depth, 5, W, H, fov=fov)
    gpu_ctx.raycast_full(tgt, view)
    gpu_ctx.synchronize()
    col, xyzw = tgt.full()
    vox = tgt.voxels()
    ocol, oxyzw, ovox, stats = _full_oracle(orc, octree, view)
    assert np.array_equal(col, ocol), f"{int((col != ocol).sum())} colour words differ"
    assert np.array_equal(xyzw.view(np.uint32), oxyzw.view(np.uint32)), "hit position/distance bits differ"
    assert np.array_equal(vox, ovox), "hit voxels differ"
    assert np.array_equal(tgt.bgrx(), orc.colorize(ocol))
    if (W, H, depth, shell) == (512, 512, 9, False):
        # the plain full raycast configuration: rays whose hit point lies within
        # 1 ulp of a face of its cell stay under 1e-4 of all rays (and match anyway)
        assert stats[6] < 1e-4 * stats[0], int(stats[6])
    tgt.close()


@pytest.mark.parametrize("dx,dz", [(262244.3, 0.0), (-2000.6, -5000.3), (0.0, 300000.7), (400000.0, -310000.0)])
def test_full_raycast_far_camera_bit_exact(svo, orc, scene, gpu_ctx, dx, dz):
    """Cameras far out in the periodic terrain: rays whose mirrored start point
    lies outside [0, 2^22) raypos units (x or z beyond 262,144 world units, or
    negative) walk with the I2F/F2I conversions instead of the biased
    FMA-pipe coordinates; every ray still matches the oracle bit for bit."""
    octree = scene(9, 1234, True)
    gpu_ctx.upload(octree)
    W, H = 160, 96
    tgt = gpu_ctx.target(W, H)
    view = svo.camera_path(1, 9, 5, W, H)
    view.pos[0] = view.pos[0] + dx
    view.pos[2] = view.pos[2] + dz
    gpu_ctx.raycast_full(tgt, view)
    gpu_ctx.synchronize()
    col, xyzw = tgt.full()
    ocol, oxyzw, ovox, _ = _full_oracle(orc, octree, view)
    assert (ovox >> np.uint64(63)).astype(bool).sum() > W * H // 2  # mostly terrain, not sky
    assert np.array_equal(col, ocol), f"{int((col != ocol).sum())} colour words differ"
    assert np.array_equal(xyzw.view(np.uint32), oxyzw.view(np.uint32)), "hit position/distance bits differ"
    assert np.array_equal(tgt.voxels(), ovox), "hit voxels differ"
    tgt.close()


@pytest.mark.parametrize("depth,shell,kind,W,H,frames", [
    (8, True, 1, 128, 96, 40),    # covers a whole 8x4 refresh cycle
    (9, True, 2, 200, 120, 12),   # ragged: 200x120 is not a multiple of 16
    (8, False, 1, 96, 64, 6),
    (12, True, 2, 96, 64, 6),     # depth 12
])
def test_warp_frames_bit_exact(svo, orc, scene, gpu_ctx, depth, shell, kind, W, H, frames):
    octree = scene(depth, 99, shell)
    gpu_ctx.upload(octree)
    tgt = gpu_ctx.target(W, H)
    warp = orc.Warp(depth, W, H)
    for f in range(frames):
        v = svo.camera_path(kind, depth, f, W, H)
        gpu_ctx.warp_frame(tgt, v, f)
        warp.frame(octree.words, octree.root, v.pos_array, v.m_array, f)
        gpu_ctx.synchronize()
        screen = warp.screen()
        ids, count = tgt.holes()
        assert count == warp.hole_count(), f"frame {f}: hole count"
        assert np.array_equal(ids, warp.ids()), f"frame {f}: hole id buffer"
        assert np.array_equal(tgt.colour(2), screen[2]), f"frame {f}: cache plane (pre-filter colours)"
        assert np.array_equal(tgt.colour(0), screen[0]), f"frame {f}: displayed plane (after the filter)"
        assert np.array_equal(tgt.bgrx(), warp.tex()), f"frame {f}: BGRX"
        ne = screen[2] != svo.EMPTY_PIXEL
        got = tgt.coords(2)[ne]
        want = warp.back()[2][ne]
        assert np.array_equal(got.view(np.uint32), want.view(np.uint32)), f"frame {f}: coordinate buffer"
    tgt.close()


def test_warp_frames_past_the_staged_scan_bit_exact(svo, orc, scene, gpu_ctx):
    """4096x1808 has 256 x 113 = 28,928 hole tiles, more than the hole scan
    stages in shared memory (28,672): it scans in global memory. Frames 0-1
    list every pixel as a hole, frames 2-3 warp; the hole count, the hole id
    buffer, the cache plane and the BGRX image match the oracle's."""
    depth, W, H = 8, 4096, 1808
    assert (W // 16) * (H // 16) > 28 * 1024
    octree = scene(depth, 99, True)
    gpu_ctx.upload(octree)
    tgt = gpu_ctx.target(W, H)
    warp = orc.Warp(depth, W, H)
    for f in range(4):
        v = svo.camera_path(1, depth, f, W, H)
        gpu_ctx.warp_frame(tgt, v, f)
        warp.frame(octree.words, octree.root, v.pos_array, v.m_array, f)
        gpu_ctx.synchronize()
        ids, count = tgt.holes()
        assert count == warp.hole_count(), f"frame {f}: hole count"
        assert np.array_equal(ids, warp.ids()), f"frame {f}: hole id buffer"
        assert np.array_equal(tgt.colour(2), warp.screen()[2]), f"frame {f}: cache plane"
        assert np.array_equal(tgt.bgrx(), warp.tex()), f"frame {f}: BGRX"
    tgt.close()


@pytest.mark.parametrize("depth,kind,W,H,frames", [(9, 2, 160, 96, 40), (8, 1, 128, 64, 36)])
def test_warp_frames_alternating_cache_bit_exact(svo, orc, scene, gpu_ctx, depth, kind, W, H, frames):
    # raycast.h:395's commented-out copy target ((frame>>4)%2)+1: both cache
    # planes live, rejected sources cleared in the plane that is kept.
    octree = scene(depth, 41, True)
    gpu_ctx.upload(octree)
    tgt = gpu_ctx.target(W, H)
    tgt.set_cache_mode(1)
    warp = orc.Warp(depth, W, H)
    for f in range(frames):
        v = svo.camera_path(kind, depth, f, W, H)
        gpu_ctx.warp_frame(tgt, v, f)
        warp.frame(octree.words, octree.root, v.pos_array, v.m_array, f, cache_mode=1)
        gpu_ctx.synchronize()
        screen, back = warp.screen(), warp.back()
        assert np.array_equal(tgt.holes()[0], warp.ids()), f"frame {f}: hole id buffer"
        for plane in (0, 1, 2):
            assert np.array_equal(tgt.colour(plane), screen[plane]), f"frame {f}: plane {plane}"
        for plane in (1, 2):
            ne = screen[plane] != svo.EMPTY_PIXEL
            assert np.array_equal(tgt.coords(plane)[ne][:, :3].view(np.uint32),
                                  back[plane][ne][:, :3].view(np.uint32)), f"frame {f}: coordinates {plane}"
        assert np.array_equal(tgt.bgrx(), warp.tex()), f"frame {f}: BGRX"
    tgt.close()


@pytest.mark.parametrize("cache_mode,graph", [(0, False), (1, True)])
def test_warp_frames_coarse_refresh_bit_exact(svo, orc, scene, gpu_ctx, cache_mode, graph):
    # raycast.h:235-261's disabled raycast_fine pass between reprojection and
    # the hole gather
    depth, W, H = 9, 160, 96
    octree = scene(depth, 43, True)
    gpu_ctx.upload(octree)
    tgt = gpu_ctx.target(W, H)
    tgt.set_cache_mode(cache_mode)
    tgt.set_coarse_refresh(True)
    tgt.use_graph(graph)
    warp = orc.Warp(depth, W, H)
    for f in range(20):
        v = svo.camera_path(2, depth, f, W, H)
        gpu_ctx.warp_frame(tgt, v, f)
        warp.frame(octree.words, octree.root, v.pos_array, v.m_array, f, cache_mode=cache_mode, coarse=True)
        gpu_ctx.synchronize()
        screen, back = warp.screen(), warp.back()
        assert np.array_equal(tgt.holes()[0], warp.ids()), f"frame {f}: hole id buffer"
        for plane in (0, 1, 2):
            assert np.array_equal(tgt.colour(plane), screen[plane]), f"frame {f}: plane {plane}"
        ne = screen[2] != svo.EMPTY_PIXEL
        assert np.array_equal(tgt.coords(2)[ne].view(np.uint32), back[2][ne].view(np.uint32)), f"frame {f}"
        assert np.array_equal(tgt.bgrx(), warp.tex()), f"frame {f}: BGRX"
    tgt.close()
    t2 = gpu_ctx.target(30, 20)
    with pytest.raises(svo.SvoError):
        t2.set_coarse_refresh(True)
    t2.close()
