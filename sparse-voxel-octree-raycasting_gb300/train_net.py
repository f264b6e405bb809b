"""Trains the reconstruction net of learned warp frames on frames the method
itself generates, then evaluates it on a held-out camera path.

Every training step renders one learned warp frame (its input features are
taken through the target's feature tap), the full raycast of the same view
(the target colour), and runs the net's forward, loss, backward and one Adam
step on the GPU (svo_net_backward / svo_net_adam: every convolution on the
tensor cores). The camera alternates,
in stretches of --segment frames, between the orbit (0.5 deg/frame) and the
fast-motion path (2 deg/frame yaw plus 0.05 x extent/frame translation).

    python sparse-voxel-octree-raycasting_gb300/train_net.py --frames 2048 \\
        --out sparse-voxel-octree-raycasting_gb300/net_weights.npy

After training, the confidence is calibrated on a third terrain seed: the
confidence output's bias is shifted (bisection) so that threshold 0.5 reaches
--calib-db on both camera paths. Writes the parameters (.npy) and a JSON
report next to them: the training curve, the calibration shift and, on the
held-out scene (another terrain seed), PSNR against the full raycast and the
fraction of pixels traced, for the learned frames at several confidence
thresholds and for the plain warp pipeline.
"""
from __future__ import annotations

import argparse
import json
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)

import svo_gb300 as svo  # noqa: E402

ORBIT = 1  # camera_path kind: 0.5 deg/frame orbit
FAST_MOTION = 2  # camera_path kind: 2 deg/frame + 0.05 extent/frame


def parse_args(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    ap.add_argument("--frames", type=int, default=2048, help="training frames (one Adam step each)")
    ap.add_argument("--res", default="1920x1024")
    ap.add_argument("--depth", type=int, default=11)
    ap.add_argument("--seed", type=int, default=7, help="terrain seed of the training scene")
    ap.add_argument("--eval-seed", type=int, default=2024, help="terrain seed of the held-out scene")
    ap.add_argument("--eval-frames", type=int, default=96)
    ap.add_argument("--tau", type=float, default=0.015, help="confidence label: all channels within tau")
    ap.add_argument("--lam", type=float, default=0.1, help="weight of the confidence loss")
    ap.add_argument("--lr", type=float, default=1e-3)
    ap.add_argument("--lr-end", type=float, default=5e-5, help="learning rate at the last step (cosine decay)")
    ap.add_argument("--threshold-range", default="0.3,0.9",
                    help="confidence threshold of each training frame, drawn uniformly from this range, so the "
                         "training caches range from mostly reprojected to mostly traced")
    ap.add_argument("--init-seed", type=int, default=1)
    ap.add_argument("--segment", type=int, default=128, help="frames per camera-path stretch")
    ap.add_argument("--epochs", type=int, default=1, help="passes over the --frames camera poses")
    ap.add_argument("--out", default=os.path.join(HERE, "net_weights.npy"))
    ap.add_argument("--calib-seed", type=int, default=1234, help="terrain seed of the calibration scene")
    ap.add_argument("--calib-db", type=float, default=38.5,
                    help="calibrate the confidence so that threshold 0.5 reaches this PSNR on the calibration scene")
    return ap.parse_args(argv)


def evaluate(ctx, net, octree, W, H, frames, thresholds, kind=FAST_MOTION, log=print):
    """PSNR against the full raycast and traced fraction over a camera path,
    for learned frames at each threshold and for the plain warp pipeline."""
    full = ctx.target(W, H)
    res = {}
    runs = [("plain", None)] + [(f"learned@{t:g}", t) for t in thresholds]
    for name, thr in runs:
        tgt = ctx.target(W, H)
        tgt.use_graph(True)
        psnr, traced = [], []
        for f in range(frames):
            v = svo.camera_path(kind, octree.depth, f, W, H)
            if thr is None:
                ctx.warp_frame(tgt, v, f)
            else:
                ctx.warp_frame_learned(tgt, v, f, net, thr)
            if f < 8:
                continue  # caches warming up
            ctx.raycast_full(full, v)
            psnr.append(svo.psnr_bgrx(tgt.bgrx(), full.bgrx()))
            if thr is None:
                traced.append(tgt.holes()[1] / (W * H))
            else:
                traced.append(tgt.requested() / (W * H))
        # frames identical to the full raycast have infinite PSNR: average the
        # MSE instead and convert once
        mse = [255.0 ** 2 / 10 ** (p / 10) if np.isfinite(p) else 0.0 for p in psnr]
        mean_mse = float(np.mean(mse))
        res[name] = {"psnr_db": 10 * np.log10(255.0 ** 2 / mean_mse) if mean_mse > 0 else float("inf"),
                     "psnr_min_db": float(np.min(psnr)), "traced_fraction": float(np.mean(traced))}
        log(f"  {name:16s} psnr {res[name]['psnr_db']:.2f} dB (min {res[name]['psnr_min_db']:.2f})  "
            f"traced {100 * res[name]['traced_fraction']:.1f}% of pixels (+ refresh tile)")
        tgt.close()
    full.close()
    return res


def path_psnr(ctx, net, depth, W, H, kind, frames, threshold=0.5):
    """PSNR of learned frames against the full raycast over one camera path."""
    tgt, full = ctx.target(W, H), ctx.target(W, H)
    tgt.use_graph(True)
    mse = []
    for f in range(frames):
        v = svo.camera_path(kind, depth, f, W, H)
        ctx.warp_frame_learned(tgt, v, f, net, threshold)
        if f >= 8:
            ctx.raycast_full(full, v)
            p = svo.psnr_bgrx(tgt.bgrx(), full.bgrx())
            mse.append(255.0 ** 2 / 10 ** (p / 10) if np.isfinite(p) else 0.0)
    tgt.close()
    full.close()
    m = float(np.mean(mse))
    return 10 * np.log10(255.0 ** 2 / m) if m > 0 else float("inf")


def calibrate(ctx, net, depth, W, H, target_db, frames=48, log=print):
    """Shifts the confidence output's bias so that threshold 0.5 reaches
    target_db on both camera paths of the (already uploaded) calibration
    scene with as few rays as the search finds (bisection on the shift)."""
    params = net.params()
    base = float(params[-1])  # the last value is the confidence bias
    lo, hi = -4.0, 2.0        # shift: lower -> lower confidence -> more rays

    def ok(shift):
        p = params.copy()
        p[-1] = base + shift
        net.set_params(p)
        db = min(path_psnr(ctx, net, depth, W, H, ORBIT, frames), path_psnr(ctx, net, depth, W, H, FAST_MOTION, frames))
        log(f"  confidence shift {shift:+.3f}: {db:.2f} dB")
        return db >= target_db

    if ok(hi):
        lo = hi
    else:
        for _ in range(7):
            mid = 0.5 * (lo + hi)
            if ok(mid):
                lo = mid
            else:
                hi = mid
    p = params.copy()
    p[-1] = base + lo
    net.set_params(p)
    return lo


def main(argv=None):
    import torch

    args = parse_args(argv)
    W, H = (int(v) for v in args.res.split("x"))
    torch.cuda.set_device(0)
    ctx = svo.Context(0)
    t0 = time.perf_counter()
    octree = svo.build_terrain(args.depth, args.seed, shell=True)
    ctx.upload(octree)
    print(f"training scene: depth {args.depth}, seed {args.seed}, {octree.words.size} words "
          f"({time.perf_counter() - t0:.1f} s)", flush=True)
    net = svo.Net(ctx, args.init_seed)
    tgt, full = ctx.target(W, H), ctx.target(W, H)
    tgt.use_graph(True)
    feat = torch.zeros(8 * W * H, dtype=torch.float32, device="cuda")
    torch.cuda.synchronize()
    tgt.set_feature_tap(feat.data_ptr())
    target_bgrx = full.device_outputs().bgrx
    curve = []
    lo, hi = (float(x) for x in args.threshold_range.split(","))
    rng = np.random.default_rng(args.init_seed)
    t0 = time.perf_counter()
    steps = args.frames * args.epochs
    for step in range(steps):
        f = step % args.frames
        seg = f // args.segment
        kind = ORBIT if seg % 2 == 0 else FAST_MOTION
        # each stretch continues its path where the previous stretch of that
        # kind stopped; the frame counter restarts so its caches start empty
        pf = (seg // 2) * args.segment + f % args.segment
        v = svo.camera_path(kind, args.depth, pf, W, H)
        ctx.warp_frame_learned(tgt, v, f % args.segment, net, float(rng.uniform(lo, hi)))
        ctx.raycast_full(full, v)
        lr = args.lr_end + 0.5 * (args.lr - args.lr_end) * (1 + np.cos(np.pi * step / max(1, steps - 1)))
        l_rgb, l_conf = net.backward(feat.data_ptr(), target_bgrx, W, H, args.tau, args.lam)
        net.adam(float(lr))
        if step % 64 == 0 or step == steps - 1:
            req = tgt.requested() / (W * H)
            curve.append({"step": step, "loss_rgb": l_rgb, "loss_conf": l_conf, "requested": req})
            print(f"step {step:5d}  loss rgb {l_rgb:.3e}  conf {l_conf:.4f}  requested {100 * req:5.1f}%  "
                  f"lr {lr:.2e}  ({time.perf_counter() - t0:.1f} s)", flush=True)
    ctx.synchronize()
    train_s = time.perf_counter() - t0
    tgt.set_feature_tap(None)
    tgt.close()
    full.close()
    shift = None
    if args.calib_db > 0:
        print(f"calibration scene: seed {args.calib_seed}", flush=True)
        octree_cal = svo.build_terrain(args.depth, args.calib_seed, shell=True)
        ctx.upload(octree_cal)
        shift = calibrate(ctx, net, args.depth, W, H, args.calib_db)
    params = net.params()
    np.save(args.out, params)

    print(f"held-out scene: seed {args.eval_seed}", flush=True)
    octree_eval = svo.build_terrain(args.depth, args.eval_seed, shell=True)
    ctx.upload(octree_eval)
    evals = {}
    for name, kind in (("orbit", ORBIT), ("fast_motion", FAST_MOTION)):
        print(f" {name}:", flush=True)
        evals[name] = evaluate(ctx, net, octree_eval, W, H, args.eval_frames, [0.3, 0.4, 0.5, 0.6, 0.7], kind)
    report = {"args": vars(args), "train_seconds": train_s, "confidence_shift": shift, "curve": curve, "eval": evals}
    with open(os.path.splitext(args.out)[0] + ".json", "w") as fh:
        json.dump(report, fh, indent=1)
    net.close()
    ctx.close()


if __name__ == "__main__":
    main()
