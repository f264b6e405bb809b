"""GPU tests of the reconstruction net: the FP32 CUDA-core forward against the
CPU restatement (oracle/net_oracle.py); the training step's gradients -- the
tensor-core forward keeping its activations, then the tensor-core backward
convolutions (data and weight gradients) -- against the restatement's; the
Adam step; the tensor-core inference kernel against the FP32 forward; and
learned warp frames (all pixels requested -> exactly the full raycast; the
feature tap)."""
import numpy as np
import pytest

import net_oracle as no

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def _dev(a):
    t = torch.from_numpy(np.ascontiguousarray(a)).cuda()
    torch.cuda.synchronize()
    return t


def _rand_case(seed, W, H):
    rng = np.random.default_rng(seed)
    params = no.init_params(seed) + (rng.standard_normal(no.NET_PARAMS) * 0.05).astype(np.float32)
    feat = rng.random((8, H, W)).astype(np.float32)
    feat[4] = (feat[4] > 0.7).astype(np.float32)
    feat[6:] *= 0.5
    tgt = rng.integers(0, 1 << 24, H * W, dtype=np.uint32)
    return params.astype(np.float32), feat, tgt


@pytest.fixture
def net(svo, gpu_ctx):
    n = gpu_ctx.net()
    yield n
    n.close()


@pytest.mark.parametrize("W,H", [(37, 29), (64, 8)])
def test_forward_matches_oracle(svo, gpu_ctx, net, W, H):
    params, feat, _ = _rand_case(11, W, H)
    net.set_params(params)
    df = _dev(feat)
    out = torch.empty(4 * W * H, dtype=torch.float32, device="cuda")
    net.forward(df.data_ptr(), W, H, out.data_ptr())
    gpu_ctx.synchronize()
    ref, _ = no.forward(params, feat)
    got = out.cpu().numpy().reshape(4, H, W)
    scale = np.abs(ref).max()
    # FP32 sums vs exact sums: rare one-ulp bf16 flips of hidden activations
    assert np.abs(got - ref).max() < 1e-2 * scale
    assert np.abs(got - ref).mean() < 1e-4 * scale


@pytest.mark.parametrize("W,H", [(45, 31), (130, 70), (200, 124), (5, 3)])
def test_gradients_match_oracle(svo, gpu_ctx, net, W, H):
    # one 62x30 tile of the backward kernels, several ragged tiles, more
    # tiles than a handful of CTAs, and a frame smaller than one 3x3 window
    params, feat, tgt = _rand_case(5, W, H)
    net.set_params(params)
    df, dt = _dev(feat), _dev(tgt.view(np.int32))
    lr, lc = net.backward(df.data_ptr(), dt.data_ptr(), W, H, 0.1, 0.5)
    g = net.grads()
    out, acts = no.forward(params, feat)
    rl, rc, d = no.loss_grad(out, no.target_rgb(tgt, H, W), 0.1, 0.5)
    ref = no.backward(params, acts, d)
    assert abs(lr - rl) < 1e-4 * abs(rl) + 1e-7 and abs(lc - rc) < 1e-4 * abs(rc) + 1e-7
    o = 0
    for ws, bs in no.layer_shapes():
        n = int(np.prod(ws)) + bs[0]
        err = np.linalg.norm(g[o:o + n] - ref[o:o + n]) / np.linalg.norm(ref[o:o + n])
        assert err < 1e-3, (o, err)
        o += n


def test_adam_step_matches_oracle(svo, gpu_ctx, net):
    W, H = 33, 17
    params, feat, tgt = _rand_case(8, W, H)
    net.set_params(params)
    df, dt = _dev(feat), _dev(tgt.view(np.int32))
    p = params.astype(np.float64)
    m = np.zeros_like(p)
    v = np.zeros_like(p)
    for step in range(1, 4):
        net.backward(df.data_ptr(), dt.data_ptr(), W, H, 0.05, 1.0)
        g = net.grads().astype(np.float64)
        net.adam(1e-3)
        p, m, v = no.adam(p, m, v, g, step, 1e-3)
        got = net.params()
        assert np.allclose(got, p, rtol=1e-5, atol=1e-7), step
        p = got.astype(np.float64)  # follow the GPU's rounding of the parameters


@pytest.mark.parametrize("W,H", [(300, 200), (57, 25), (16, 16)])
def test_tensor_core_inference_matches_fp32(svo, gpu_ctx, net, W, H):
    params, feat, _ = _rand_case(21, W, H)
    net.set_params(params)
    df = _dev(feat)
    a = torch.empty(4 * W * H, dtype=torch.float32, device="cuda")
    b = torch.full((4 * W * H,), float("nan"), dtype=torch.float32, device="cuda")
    net.forward(df.data_ptr(), W, H, a.data_ptr())
    net.infer(df.data_ptr(), W, H, b.data_ptr())
    gpu_ctx.synchronize()
    a, b = a.cpu().numpy(), b.cpu().numpy()
    assert not np.isnan(b).any()  # every output pixel written
    scale = np.abs(a).max()
    assert np.abs(a - b).max() < 1e-2 * scale
    assert np.abs(a - b).mean() < 1e-4 * scale


def test_learned_frame_all_requested_equals_full_raycast(svo, scene, gpu_ctx, net):
    # With a threshold no confidence reaches, every pixel is traced: the
    # learned frame must then show exactly the full raycast.
    octree = scene(9, 77, True)
    gpu_ctx.upload(octree)
    W, H = 160, 96
    t, full = gpu_ctx.target(W, H), gpu_ctx.target(W, H)
    for graph in (False, True):
        t.use_graph(graph)
        for f in range(6):
            v = svo.camera_path(2, 9, f, W, H)
            gpu_ctx.warp_frame_learned(t, v, f, net, threshold=0.999999)
            gpu_ctx.raycast_full(full, v)
            gpu_ctx.synchronize()
            assert np.array_equal(t.bgrx(), full.bgrx()), (graph, f)
            assert t.requested() >= W * H - (W // 8 + 16) * (H // 4 + 16)
    t.close()
    full.close()


def test_learned_frame_low_threshold_traces_only_refresh_tile(svo, scene, gpu_ctx, net):
    octree = scene(9, 77, True)
    gpu_ctx.upload(octree)
    W, H = 128, 64
    t = gpu_ctx.target(W, H)
    for f in range(4):
        gpu_ctx.warp_frame_learned(t, svo.camera_path(2, 9, f, W, H), f, net, threshold=1e-6)
        gpu_ctx.synchronize()
        # no cache in the first two frames: every pixel is traced
        assert t.requested() == (W * H if f < 2 else 0)
    t.close()


def test_feature_tap(svo, scene, gpu_ctx, net):
    octree = scene(9, 77, True)
    gpu_ctx.upload(octree)
    W, H = 96, 64
    t = gpu_ctx.target(W, H)
    buf = torch.zeros(8 * W * H, dtype=torch.float32, device="cuda")
    t.set_feature_tap(buf.data_ptr())
    for f in range(5):
        gpu_ctx.warp_frame(t, svo.camera_path(1, 9, f, W, H), f)
        gpu_ctx.synchronize()
        feat = buf.cpu().numpy().reshape(8, H, W)
        hole = feat[4]
        assert set(np.unique(hole)) <= {0.0, 1.0}
        if f < 2:
            assert np.all(hole == 1.0)  # no cache yet: everything is a hole
        else:
            assert hole.mean() < 0.9
        assert np.all(feat[:4, hole == 1.0] == 0.0) and np.all(feat[5:7, hole == 1.0] == 0.0)
        assert np.all((feat[5:] >= 0) & (feat[5:] <= 1))
        if f >= 2:
            # reprojected points land anywhere inside their pixel
            sub = feat[6][hole == 0.0]
            assert 0.1 < sub.mean() < 0.7
        # ray elevation: defined for every pixel, monotonic down the image columns
        elev = feat[7]
        assert np.all(np.diff(elev[:, W // 2]) > 0) or np.all(np.diff(elev[:, W // 2]) < 0)
    t.set_feature_tap(None)
    t.close()


def _learned_quality(svo, ctx, net, octree, W, H, thr, frames=24, kind=2):
    t, full = ctx.target(W, H), ctx.target(W, H)
    mse, traced = [], []
    for f in range(frames):
        v = svo.camera_path(kind, octree.depth, f, W, H)
        if net is None:
            ctx.warp_frame(t, v, f)
        else:
            ctx.warp_frame_learned(t, v, f, net, thr)
        if f >= 8:
            ctx.raycast_full(full, v)
            a = t.bgrx().view(np.uint8).reshape(-1, 4)[:, :3].astype(np.float64)
            b = full.bgrx().view(np.uint8).reshape(-1, 4)[:, :3].astype(np.float64)
            mse.append(((a - b) ** 2).mean())
            traced.append((t.holes()[1] if net is None else t.requested()) / (W * H))
    t.close()
    full.close()
    return 10 * np.log10(255.0 ** 2 / max(np.mean(mse), 1e-9)), float(np.mean(traced))


def test_trained_net_gains_over_the_method_without_it(svo, gpu_ctx):
    # The committed weights against the method without them: (a) the plain
    # warp pipeline (hole filter + hole rays) on the same held-out frames --
    # the net buys several dB; (b) an untrained net at the same threshold --
    # its confidence is uninformative (it traces nearly everything or
    # nothing), the trained one traces a fraction and keeps the quality.
    import os
    octree = svo.build_terrain(10, 2024, shell=True)
    gpu_ctx.upload(octree)
    W, H = 640, 384
    trained = gpu_ctx.net()
    trained.load_file(os.path.join(os.path.dirname(svo.__file__), "net_weights.npy"))
    p_tr, f_tr = _learned_quality(svo, gpu_ctx, trained, octree, W, H, 0.5)
    p_plain, f_plain = _learned_quality(svo, gpu_ctx, None, octree, W, H, 0.5)
    print(f"trained: {p_tr:.2f} dB, {100 * f_tr:.1f}% traced; plain: {p_plain:.2f} dB, {100 * f_plain:.1f}% traced")
    assert p_tr > p_plain + 4.0, (p_tr, p_plain)
    assert p_tr > 34.0 and f_tr < 0.9, (p_tr, f_tr)
    untrained = gpu_ctx.net(seed=3)
    p_un, f_un = _learned_quality(svo, gpu_ctx, untrained, octree, W, H, 0.5)
    print(f"untrained: {p_un:.2f} dB, {100 * f_un:.1f}% traced")
    assert f_un > 0.95 or p_un < p_tr - 4.0, (p_un, f_un)
    trained.close()
    untrained.close()


@pytest.mark.parametrize("W,H", [(37, 29), (100, 50), (130, 17), (57, 25)])
def test_learned_frames_ragged_resolutions(svo, scene, gpu_ctx, net, W, H):
    # ragged net tiles (56x24), ragged 8x4 request packets and ragged 16x16
    # hole tiles: every pixel requested -> the full raycast, bit for bit
    octree = scene(8, 31, True)
    gpu_ctx.upload(octree)
    t, full = gpu_ctx.target(W, H), gpu_ctx.target(W, H)
    t.use_graph(True)
    for f in range(5):
        v = svo.camera_path(2, 8, f, W, H)
        gpu_ctx.warp_frame_learned(t, v, f, net, 0.999999)
        gpu_ctx.raycast_full(full, v)
        gpu_ctx.synchronize()
        assert np.array_equal(t.bgrx(), full.bgrx()), f
        assert t.requested() == W * H
    t.close()
    full.close()
