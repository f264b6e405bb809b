"""GPU tests of the runtime around the kernels: batched views, CUDA-graph
replay, stage timing, fault reporting, edge cases and the reference-named C++
host interface."""
import os
import subprocess

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _oracle_full(orc, octree, v):
    return orc.raycast_full(octree.depth, octree.words, octree.root, v.pos_array, v.m_array, v.res_x, v.res_y,
                            v.fovx, v.fovy)


def test_batched_views_match_single_views(svo, orc, scene, gpu_ctx):
    octree = scene(9, 77, True)
    gpu_ctx.upload(octree)
    sizes = [(64, 48), (200, 120), (33, 17), (128, 128), (320, 180), (8, 4), (1, 1)]
    targets = [gpu_ctx.target(w, h) for w, h in sizes]
    views = [svo.camera_path(3, 9, i, w, h, seed=5) for i, (w, h) in enumerate(sizes)]
    gpu_ctx.raycast_full_batch(targets, views)
    gpu_ctx.synchronize()
    for t, v in zip(targets, views):
        col, xyzw = t.full()
        ocol, oxyzw, ovox, _ = _oracle_full(orc, octree, v)
        assert np.array_equal(col, ocol)
        assert np.array_equal(xyzw.view(np.uint32), oxyzw.view(np.uint32))
        assert np.array_equal(t.voxels(), ovox)
        t.close()


def test_graph_replay_matches_direct_launches(svo, scene, gpu_ctx):
    octree = scene(8, 99, True)
    gpu_ctx.upload(octree)
    a, b = gpu_ctx.target(160, 96), gpu_ctx.target(160, 96)
    b.use_graph(True)
    for f in range(20):
        v = svo.camera_path(2, 8, f, 160, 96)
        gpu_ctx.warp_frame(a, v, f)
        gpu_ctx.warp_frame(b, v, f)
        gpu_ctx.synchronize()
        assert np.array_equal(a.colour(0), b.colour(0)), f
        assert np.array_equal(a.colour(2), b.colour(2)), f
        assert np.array_equal(a.holes()[0], b.holes()[0]), f
    a.close()
    b.close()


@pytest.mark.parametrize("graph", [False, True])
def test_async_readback_matches_blocking_readback(svo, scene, gpu_ctx, graph):
    # svo_read_bgrx_async: each image copied while the next frame renders (the
    # frame's first write to the image waits for the copy) equals the image a
    # blocking readback of a twin target returns -- guided learned frames
    # (the net writes the image), plain warp frames (the filter) and full
    # raycasts, interleaved on the same targets
    torch = pytest.importorskip("torch")
    octree = scene(9, 77, True)
    gpu_ctx.upload(octree)
    net = gpu_ctx.net()
    net.load_file(os.path.join(os.path.dirname(svo.__file__), "net_weights.npy"))
    W, H = 160, 96
    a, b = gpu_ctx.target(W, H), gpu_ctx.target(W, H)
    for t in (a, b):
        t.use_graph(graph)
        t.set_guided(True)
    hosts = [torch.empty(W * H, dtype=torch.int32, pin_memory=True).numpy().view(np.uint32) for _ in range(3)]
    want = []
    for f in range(12):
        v = svo.camera_path(2, 9, f, W, H)
        kind = f % 4
        for t in (a, b):
            if kind == 3:
                gpu_ctx.raycast_full(t, v)
            elif kind == 2:
                gpu_ctx.warp_frame(t, v, f)
            else:
                gpu_ctx.warp_frame_learned(t, v, f, net, 0.5)
        a.bgrx_into_async(hosts[f % 3])
        want.append(b.bgrx())  # blocking
        if f >= 2:  # the copy of frame f - 2 is done once the one of f - 1 is (same stream)
            a.readback_wait()
            assert np.array_equal(hosts[(f - 2) % 3], want[f - 2]), f - 2
    a.readback_wait()
    for f in (10, 11):
        assert np.array_equal(hosts[f % 3], want[f]), f
    a.close()
    b.close()
    net.close()


@pytest.mark.parametrize("graph", [False, True])
def test_stage_timing(svo, scene, gpu_ctx, graph):
    octree = scene(8, 99, True)
    gpu_ctx.upload(octree)
    t = gpu_ctx.target(256, 128)
    t.use_graph(graph)
    t.set_profiling(True)
    for f in range(4):
        gpu_ctx.warp_frame(t, svo.camera_path(1, 8, f, 256, 128), f)
        ms = t.stage_times()
        assert ms.size == 6 and np.all(ms >= 0) and ms.sum() > 0
    gpu_ctx.raycast_full(t, svo.camera_path(1, 8, 0, 256, 128))
    ms = t.stage_times()
    assert ms[4] > 0
    t.close()


def test_launch_count_and_device_outputs(svo, scene, gpu_ctx):
    octree = scene(8, 99, True)
    gpu_ctx.upload(octree)
    t = gpu_ctx.target(64, 64)
    n0 = gpu_ctx.launch_count()
    gpu_ctx.warp_frame(t, svo.camera_path(1, 8, 0, 64, 64), 0)
    gpu_ctx.synchronize()
    assert gpu_ctx.launch_count() - n0 == 7  # params, project, resolve, scan, write, trace, filter
    d = t.device_outputs()
    assert d.bgrx and d.colour and d.full_colour and d.full_xyzw and d.full_voxel
    t.close()


def test_bad_octree_is_rejected_by_validation(svo, gpu_ctx):
    words = np.zeros(64, np.uint32)
    words[0] = (1000 << 9) | 0xFF  # child pointers far past the end
    with pytest.raises(svo.SvoError) as e:
        gpu_ctx.upload(svo.Octree(words, root=0x1, depth=8), validate=True)
    assert e.value.status == 4


def test_bad_octree_raises_device_fault_and_context_survives(svo, orc, scene, gpu_ctx):
    words = np.zeros(4096, np.uint32)
    words[:8] = (0x7FFFF << 9) | 0xFF  # every root child points outside the array
    gpu_ctx.upload(svo.Octree(words, root=0xFF, depth=8), validate=False)
    t = gpu_ctx.target(64, 48)
    gpu_ctx.raycast_full(t, svo.camera_path(0, 8, 0, 64, 48))
    with pytest.raises(svo.SvoError) as e:
        gpu_ctx.synchronize()
    assert e.value.status == 5
    # the flag is cleared and the context keeps working with a good octree
    octree = scene(8, 99, True)
    gpu_ctx.upload(octree)
    v = svo.camera_path(0, 8, 0, 64, 48)
    gpu_ctx.raycast_full(t, v)
    gpu_ctx.synchronize()
    col, _ = t.full()
    assert np.array_equal(col, _oracle_full(orc, octree, v)[0])
    t.close()


def test_empty_and_single_voxel_scenes(svo, orc, gpu_ctx):
    b = svo.Builder(8)
    empty = b.finish()
    b = svo.Builder(8)
    b.set_voxel(128, 60, 128, 0x00AB_CDEF)
    single = b.finish()
    for octree in (empty, single):
        gpu_ctx.upload(octree)
        t = gpu_ctx.target(96, 96)
        pos = np.array([8.0, 10.0, 6.0], np.float32)
        v = svo.view_look_at(pos, [16.0, 3.75, 16.0], 96, 96)
        gpu_ctx.raycast_full(t, v)
        gpu_ctx.synchronize()
        col, xyzw = t.full()
        ocol, oxyzw, ovox, _ = _oracle_full(orc, octree, v)
        assert np.array_equal(col, ocol) and np.array_equal(xyzw.view(np.uint32), oxyzw.view(np.uint32))
        assert np.array_equal(t.voxels(), ovox)
        if octree is empty:
            assert np.all(col == 0xFF000000)
        t.close()


@pytest.mark.parametrize("W,H", [(1, 1), (7, 3), (17, 9), (9, 31)])
def test_tiny_resolutions(svo, orc, scene, gpu_ctx, W, H):
    octree = scene(8, 99, True)
    gpu_ctx.upload(octree)
    t = gpu_ctx.target(W, H)
    v = svo.camera_path(3, 8, 3, W, H)
    gpu_ctx.raycast_full(t, v)
    gpu_ctx.synchronize()
    col, xyzw = t.full()
    ocol, oxyzw, _, _ = _oracle_full(orc, octree, v)
    assert np.array_equal(col, ocol) and np.array_equal(xyzw.view(np.uint32), oxyzw.view(np.uint32))
    t.close()


def test_warp_argument_checks(svo, scene, gpu_ctx):
    octree = scene(8, 99, True)
    gpu_ctx.upload(octree)
    t = gpu_ctx.target(15, 64)
    with pytest.raises(svo.SvoError):
        gpu_ctx.warp_frame(t, svo.camera_path(1, 8, 0, 15, 64), 0)
    t.close()
    t = gpu_ctx.target(64, 64)
    with pytest.raises(svo.SvoError):
        gpu_ctx.warp_frame(t, svo.camera_path(1, 8, 0, 64, 64, fov=1.2), 0)
    with pytest.raises(svo.SvoError):
        gpu_ctx.warp_frame(t, svo.camera_path(1, 8, 0, 32, 64), 0)
    t.close()


def test_warp_frame_numbers_start_anywhere(svo, orc, scene, gpu_ctx):
    # A target with no previous frame behaves like the reference's cleared
    # caches, whatever frame number the caller starts at.
    octree = scene(8, 99, True)
    gpu_ctx.upload(octree)
    t = gpu_ctx.target(96, 64)
    w = orc.Warp(8, 96, 64)
    for i, f in enumerate([5, 6, 7, 40]):
        v = svo.camera_path(1, 8, f, 96, 64)
        gpu_ctx.warp_frame(t, v, f)
        if i == 0:
            # the oracle has no previous frame either: run it at a frame < 2 equivalent
            w.frame(octree.words, octree.root, v.pos_array, v.m_array, 0)
            gpu_ctx.synchronize()
            assert np.array_equal(t.holes()[0][:2 * w.tiles], w.ids()[:2 * w.tiles])
    t.close()


def test_reference_named_cpp_interface(svo, tmp_path):
    exe = str(tmp_path / "raycast_mirror")
    lib_dir = os.path.join(ROOT, "sparse-voxel-octree-raycasting_gb300")
    subprocess.run(["g++", "-std=c++17", "-O2", "-I", os.path.join(ROOT, "include"),
                    os.path.join(ROOT, "tests", "cpp", "raycast_mirror.cpp"), "-o", exe, "-L", lib_dir,
                    "-lsvo_gb300", f"-Wl,-rpath,{lib_dir}"], check=True)
    dump = str(tmp_path / "frames.bin")
    frames, W, H = 6, 256, 160
    out = subprocess.run([exe, str(frames), dump], capture_output=True, text=True, timeout=120)
    assert out.returncode == 0, out.stderr
    assert f"frames={frames}" in out.stdout
    nonblack = int(out.stdout.split("nonblack=")[1])
    assert nonblack > W * H // 4
    # every frame the C++ layer drew equals the oracle's warp frame for the
    # same camera, bit for bit (the layer's default scene: the depth-8 seeded
    # terrain, seed 2024, visible shell)
    import oracle

    octree = svo.build_terrain(8, 2024, True)
    rec = np.fromfile(dump, np.uint32).reshape(frames, 20 + W * H)
    w = oracle.Warp(8, W, H)
    for f in range(frames):
        pos = rec[f, :4].view(np.float32)
        m = rec[f, 4:20].view(np.float32)
        w.frame(octree.words, octree.root, pos, m, f)
        assert np.array_equal(rec[f, 20:], w.tex()), f"frame {f}: BGRX differs from the oracle"


def test_concurrent_camera_streams_share_one_octree(svo, scene, gpu_ctx):
    # One context per camera stream, the octree words uploaded once and shared;
    # frames of all streams in flight together give the same images as one
    # stream at a time.
    torch = pytest.importorskip("torch")
    octree = scene(9, 5, True)
    d_words = torch.from_numpy(octree.words.view(np.int32)).cuda()
    torch.cuda.synchronize()
    ctxs = [svo.Context(0) for _ in range(3)]
    for c in ctxs:
        c.upload_device(d_words.data_ptr(), octree.words.size, octree.root, octree.depth)
    tgts = [c.target(128, 96) for c in ctxs]
    gpu_ctx.upload(octree)
    for f in range(12):
        for k, (c, t) in enumerate(zip(ctxs, tgts)):
            c.warp_frame(t, svo.camera_path(2, 9, 5 * k + f, 128, 96), f)
        for c in ctxs:
            c.synchronize()
    for k, t in enumerate(tgts):
        s2 = gpu_ctx.target(128, 96)
        for f in range(12):
            gpu_ctx.warp_frame(s2, svo.camera_path(2, 9, 5 * k + f, 128, 96), f)
        gpu_ctx.synchronize()
        assert np.array_equal(t.bgrx(), s2.bgrx()) and np.array_equal(t.colour(2), s2.colour(2))
        s2.close()
    for t in tgts:
        t.close()
    for c in ctxs:
        c.close()


def test_context_close_destroys_live_targets(svo, scene):
    # Closing a context first destroys the targets it still owns; closing such
    # a target afterwards is a no-op, and so is the C-level destroy order
    # context-then-nothing.
    octree = scene(8, 99, True)
    ctx = svo.Context(0)
    ctx.upload(octree)
    t = ctx.target(64, 32)
    ctx.raycast_full(t, svo.camera_path(1, 8, 3, 64, 32))
    ctx.synchronize()
    ctx.close()
    t.close()
    lib = svo.load()
    import ctypes
    h, th = ctypes.c_void_p(), ctypes.c_void_p()
    assert lib.svo_context_create(0, ctypes.byref(h)) == 0
    assert lib.svo_target_create(h, 32, 16, ctypes.byref(th)) == 0
    assert lib.svo_context_destroy(h) == 0



def test_trace_configurations_give_identical_frames(svo, scene, gpu_ctx):
    # packet shape, block size and node staging change the schedule only
    octree = scene(9, 77, True)
    gpu_ctx.upload(octree)
    W, H = 200, 120
    full, warp = gpu_ctx.target(W, H), gpu_ctx.target(W, H)
    v = svo.camera_path(1, 9, 3, W, H)
    gpu_ctx.raycast_full(full, v)
    want_col, want_xyz = full.full()
    frames = [svo.camera_path(1, 9, f, W, H) for f in range(6)]
    for f, fv in enumerate(frames):
        gpu_ctx.warp_frame(warp, fv, f)
    want_warp = warp.bgrx()
    for pw in (4, 8, 16, 32):
        for block in (0, 256, 1024):
            for stage in (0, 1):
                gpu_ctx.set_option(svo.OPT_PACKET_WIDTH, pw)
                gpu_ctx.set_option(svo.OPT_TRACE_BLOCK, block)
                gpu_ctx.set_option(svo.OPT_STAGE_NODES, stage)
                gpu_ctx.raycast_full(full, v)
                col, xyz = full.full()
                assert np.array_equal(col, want_col) and np.array_equal(xyz.view(np.uint32),
                                                                         want_xyz.view(np.uint32)), (pw, block, stage)
                t = gpu_ctx.target(W, H)
                for f, fv in enumerate(frames):
                    gpu_ctx.warp_frame(t, fv, f)
                assert np.array_equal(t.bgrx(), want_warp), (pw, block, stage)
                t.close()
    with pytest.raises(svo.SvoError):
        gpu_ctx.set_option(svo.OPT_PACKET_WIDTH, 6)
    full.close()
    warp.close()


def test_learned_trace_configurations_give_identical_frames(svo, scene, gpu_ctx):
    # guided learned frames under every packet shape and learned-tracer block
    # size: the same image (the walk and its start do not depend on them)
    import os
    octree = scene(9, 77, True)
    gpu_ctx.upload(octree)
    W, H = 160, 96
    net = gpu_ctx.net()
    net.load_file(os.path.join(os.path.dirname(svo.__file__), "net_weights.npy"))
    frames = [svo.camera_path(2, 9, f, W, H) for f in range(6)]
    want = None
    for pw in (4, 8, 32):
        for block in (0, 256, 1024):
            gpu_ctx.set_option(svo.OPT_PACKET_WIDTH, pw)
            gpu_ctx.set_option(svo.OPT_LEARNED_TRACE_BLOCK, block)
            t = gpu_ctx.target(W, H)
            t.set_guided(True)
            for f, fv in enumerate(frames):
                gpu_ctx.warp_frame_learned(t, fv, f, net, 0.5)
            img = t.bgrx()
            t.close()
            if want is None:
                want = img
            assert np.array_equal(img, want), (pw, block)
    gpu_ctx.set_option(svo.OPT_PACKET_WIDTH, 8)
    gpu_ctx.set_option(svo.OPT_LEARNED_TRACE_BLOCK, 0)
    with pytest.raises(svo.SvoError):
        gpu_ctx.set_option(svo.OPT_LEARNED_TRACE_BLOCK, 512)
    net.close()


def test_learned_autotune_picks_a_measured_configuration(svo, scene, gpu_ctx):
    import os
    octree = scene(9, 77, True)
    gpu_ctx.upload(octree)
    W, H = 160, 96
    net = gpu_ctx.net()
    net.load_file(os.path.join(os.path.dirname(svo.__file__), "net_weights.npy"))
    t = gpu_ctx.target(W, H)
    t.set_guided(True)
    views = [svo.camera_path(1, 9, f, W, H) for f in range(8)]
    res = gpu_ctx.autotune_learned(t, views, net, 0.5)
    assert len(res) == 8 and all(r["ms"] > 0 for r in res)
    assert {(r["packet_w"], r["block"]) for r in res} == {(w, b) for w in (4, 8, 16, 32) for b in (256, 1024)}
    with pytest.raises(svo.SvoError):
        gpu_ctx.autotune_learned(t, views[:5], net, 0.5)  # needs 6 views at least
    for f, v in enumerate(views):  # frames render with the chosen configuration
        gpu_ctx.warp_frame_learned(t, v, f, net, 0.5)
    gpu_ctx.synchronize()
    gpu_ctx.set_option(svo.OPT_LEARNED_PACKET_WIDTH, 0)
    gpu_ctx.set_option(svo.OPT_LEARNED_TRACE_BLOCK, 0)
    t.close()
    net.close()


def test_autotune_picks_a_measured_configuration(svo, scene, gpu_ctx):
    octree = scene(9, 77, True)
    gpu_ctx.upload(octree)
    t = gpu_ctx.target(256, 160)
    v = svo.camera_path(1, 9, 3, 256, 160)
    res = gpu_ctx.autotune(t, v, repeats=2)
    assert len(res) == 16 and all(r["ms"] > 0 for r in res)
    assert {(r["packet_w"], r["packet_h"]) for r in res} == {(4, 8), (8, 4), (16, 2), (32, 1)}
    gpu_ctx.raycast_full(t, v)  # runs with the chosen configuration
    gpu_ctx.synchronize()
    t.close()
