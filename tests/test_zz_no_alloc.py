"""The allocation-free full raycast (svo_raycast_full_noalloc) against the
regular one (svo_raycast_full), bit for bit, on two calls in a row.

The entry point exists for callers that cannot let the library allocate
device memory (engines with their own allocator or pool, frame loops that may
not allocate after start-up, plugins that may not grow the context): they pass
the octree words and every output buffer themselves, and the trace kernel's
small scratch lives in a static device array. Here the test allocates those
buffers with torch and calls the entry point through the C ABI (ctypes). This
file is collected last so that a failure here comes after every other test.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _frame_buffers(torch, w, h, device):
    n = w * h
    bufs = {
        "colour": torch.zeros(n, dtype=torch.int32, device=device),
        "xyzw": torch.zeros(n * 4, dtype=torch.float32, device=device),
        "voxel": torch.zeros(n, dtype=torch.int64, device=device),
        "bgrx": torch.zeros(n, dtype=torch.int32, device=device),
    }
    return bufs


def _as_struct(svo, bufs):
    return svo.FrameBuffers(bufs["colour"].data_ptr(), bufs["xyzw"].data_ptr(), bufs["voxel"].data_ptr(),
                            bufs["bgrx"].data_ptr())


def _host(torch, bufs):
    torch.cuda.synchronize()
    return (bufs["colour"].cpu().numpy().view(np.uint32), bufs["xyzw"].cpu().numpy(),
            bufs["voxel"].cpu().numpy().view(np.uint64), bufs["bgrx"].cpu().numpy().view(np.uint32))


def test_noalloc_full_raycast_matches_regular_path(svo):
    torch = pytest.importorskip("torch")
    lib = svo.load()
    device = torch.device("cuda", 0)
    torch.cuda.set_device(device)
    octree = svo.build_terrain(9, 4242, True)
    d_words = torch.from_numpy(octree.words.view(np.int32)).to(device)

    # the regular path, through a context that owns its buffers
    ctx = svo.Context(0)
    ctx.upload(octree)
    sizes = [(320, 200), (96, 64)]
    targets = [ctx.target(w, h) for w, h in sizes]

    for call in range(2):  # two calls in a row share (and must clear) the static scratch
        views = [svo.camera_path(3, 9, 10 * call + i, w, h, seed=3) for i, (w, h) in enumerate(sizes)]
        ctx.raycast_full_batch(targets, views)
        ctx.synchronize()
        want = []
        for t in targets:
            col, xyzw = t.full()
            want.append((col, xyzw.reshape(-1), t.voxels(), t.bgrx()))

        bufs = [_frame_buffers(torch, w, h, device) for w, h in sizes]
        varr = (svo.View * len(views))(*views)
        oarr = (svo.FrameBuffers * len(views))(*[_as_struct(svo, b) for b in bufs])
        stream = torch.cuda.current_stream(device).cuda_stream
        rc = lib.svo_raycast_full_noalloc(ctypes.c_void_p(d_words.data_ptr()), octree.words.size, octree.root,
                                          octree.depth, ctypes.cast(varr, ctypes.c_void_p),
                                          ctypes.cast(oarr, ctypes.c_void_p), len(views), ctypes.c_void_p(stream))
        assert rc == 0, svo.STATUS.get(rc, rc)
        for (wc, wx, wv, wb), b in zip(want, bufs):
            col, xyzw, vox, bgrx = _host(torch, b)
            assert np.array_equal(col, wc), f"call {call}: colour words"
            assert np.array_equal(xyzw.view(np.uint32), wx.view(np.uint32)), f"call {call}: hit positions"
            assert np.array_equal(vox, wv), f"call {call}: hit voxels"
            assert np.array_equal(bgrx, wb), f"call {call}: BGRX"

    # more views than the static scratch holds are refused before any work
    n = svo.NOALLOC_MAX_VIEWS + 1
    v = svo.camera_path(3, 9, 0, 8, 8)
    bufs = _frame_buffers(torch, 8, 8, device)
    varr = (svo.View * n)(*([v] * n))
    oarr = (svo.FrameBuffers * n)(*([_as_struct(svo, bufs)] * n))
    rc = lib.svo_raycast_full_noalloc(ctypes.c_void_p(d_words.data_ptr()), octree.words.size, octree.root,
                                      octree.depth, ctypes.cast(varr, ctypes.c_void_p),
                                      ctypes.cast(oarr, ctypes.c_void_p), n, None)
    assert rc == 7  # SVO_ERR_CAPACITY

    # the call synchronises, so it is refused (before any launch) while its
    # stream is being captured; the capture itself stays valid
    side = torch.cuda.Stream(device)
    x = torch.zeros(16, device=device)
    graph = torch.cuda.CUDAGraph()
    with torch.cuda.stream(side):
        with torch.cuda.graph(graph, stream=side):
            x.add_(1.0)
            rc = lib.svo_raycast_full_noalloc(ctypes.c_void_p(d_words.data_ptr()), octree.words.size, octree.root,
                                              octree.depth, ctypes.cast(varr, ctypes.c_void_p),
                                              ctypes.cast(oarr, ctypes.c_void_p), 1, ctypes.c_void_p(side.cuda_stream))
    assert rc == 1  # SVO_ERR_INVALID_ARGUMENT
    graph.replay()
    torch.cuda.synchronize()
    assert float(x[0]) == 1.0
    for t in targets:
        t.close()
    ctx.close()
