"""Small, fixed GPU workloads for profiler captures (ncu), one per case:

    learned   8 learned warp frames, 1920x1024, depth-11 benchmark terrain,
              committed net weights, threshold 0.5 (orbit camera)
    guided    the same frames with guided walks
    plain     8 plain warp frames of the same scene and camera
    full      4 full raycasts of the same scene and camera
    build     2 GPU octree builds of the depth-11 benchmark terrain's voxels

    python sparse-voxel-octree-raycasting_gb300/profile_cases.py learned

Each case prints "ok" and exits 0; the inputs are the benchmark's, so a
capture of the n-th launch of a kernel matches the benchmark's steady state.
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)

import svo_gb300 as svo  # noqa: E402

W, H, DEPTH, SEED = 1920, 1024, 11, 2024


def main(case: str) -> None:
    if case == "build":
        import torch

        x, y, z, c = svo.terrain_voxels(SEED, DEPTH, True)
        dev = [torch.from_numpy(np.ascontiguousarray(a, np.uint32).view(np.int32)).cuda() for a in (x, y, z, c)]
        torch.cuda.synchronize()
        ctx = svo.Context(0)
        for _ in range(2):
            ctx.build_octree(*(t.data_ptr() for t in dev), len(x), DEPTH)
        print("ok", ctx.octree_info())
        ctx.close()
        return
    octree = svo.build_terrain(DEPTH, SEED, shell=True)
    ctx = svo.Context(0)
    ctx.upload(octree)
    t = ctx.target(W, H)
    if case in ("learned", "guided"):
        t.set_guided(case == "guided")
        net = svo.Net(ctx)
        net.load_file(os.path.join(HERE, "net_weights.npy"))
        for f in range(8):
            ctx.warp_frame_learned(t, svo.camera_path(1, DEPTH, f, W, H), f, net, 0.5)
        ctx.synchronize()
        print("ok", t.requested())
    elif case == "plain":
        for f in range(8):
            ctx.warp_frame(t, svo.camera_path(1, DEPTH, f, W, H), f)
        ctx.synchronize()
        print("ok", t.holes()[1])
    elif case == "full":
        for f in range(4):
            ctx.raycast_full(t, svo.camera_path(1, DEPTH, 3 + f, W, H))
        ctx.synchronize()
        print("ok")
    else:
        raise SystemExit(f"unknown case {case!r}")
    ctx.close()


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else "learned")
