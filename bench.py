"""Benchmark: warped + learned sparse-voxel-octree frames/s at 1920x1024 on GB300.

Workload (one step = one guided learned warp frame: the reference's
raycast_draw reprojection, start distances from the reprojected depth, the
reconstruction net on the tiles holding a pixel without one, then rays from the
camera for the pixels the net is not confident about and the 8x4 refresh tile
and walks from the start distance for the rest): 1920x1024, depth-11 (2048^3)
seeded fBm terrain octree (visible shell), orbit camera at 1.5x extent, 0.5
degrees yaw per frame, height sinusoid 0.02x extent over 64 frames; the net's
weights are the committed ones (train_net.py). Reported beside it:

* the plain full raycast of the same frames on the same GPU (Mrays/s, frames/s);
* quality over fixed frame windows, independent of --steps: frames 0-255 of
  the orbit and frames 0-511 of the fast-motion path (2 deg/frame yaw + 0.05
  extent/frame), every frame compared with the full raycast of its camera on
  the GPU (PSNR over the window's summed squared error, maximum error), and
  the fast-motion path's 38 dB gate;
* the plain warp pipeline (the reference's algorithm, bit-exact) on the same
  frames, with the CPU reference on those same frames (a like-for-like ratio);
* the plain full raycast configuration: 512x512, depth-9 solid terrain, 60
  degree field of view (Mrays/s, parity against the oracle, the fraction of
  rays with a coordinate within 1 ulp of a cell face);
* per-stage times with L2 and HBM rooflines (the L2 read peak is measured here
  with the library's own read probe over an L2-resident buffer).

Timing: each step is bracketed by CUDA events on the library's stream; the L2
is flushed (256 MiB device write) before every timed step and outside its
events. `value` = frames of all ranks / max over ranks of the summed step
times. `e2e` times the C-ABI calls a user makes with host buffers: camera in,
svo_warp_frame_learned, BGRX8 image out to pinned host memory -- pipelined
(svo_read_bgrx_async: each image's copy overlaps the next frame's first
kernels; host wall time less the L2 flushes), with the blocking readback's
figure beside it.

--impl reference times the reference algorithm on the host CPU cores instead
(oracle/_ref when it was compiled from the reference tree here, else the
oracle port of kernel.cl/raycast.h), with all host threads, on scenes and
cameras from oracle/scene_gen.py: that process never loads the product library.

--profile-case NAME runs one small fixed workload for a profiler capture and
exits (learned, guided, plain, full, build, full512, train).

Multi-GPU: replicas only (the per-frame pipeline does not shard); each rank
renders its own camera path on its own GPU, scaling "weak".
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(ROOT, "sparse-voxel-octree-raycasting_gb300")
ORACLE = os.path.join(ROOT, "oracle")

METRIC = "Mrays/s; 1920x1024 frames/s warped+learned vs full raycast at ≥38 dB PSNR"
WORKLOAD = ("warped + learned pipeline 1920x1024 (guided walks from the reprojected depth, the net on the "
            "unguided pixels), depth-11 terrain octree, 256-frame orbit (0.5 deg/frame), confidence threshold 0.5")
PEAKS_FILE = os.path.join(ROOT, "MEASURED_PEAKS.json")
TRACE_PROFILE = "profiles/k_trace_warp_guided_1920x1024_depth11.md"
PROFILE_CASES = ("learned", "guided", "plain", "full", "build", "full512", "train")


def parse_args(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=60)
    ap.add_argument("--warmup", type=int, default=8)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--res", default="1920x1024")
    ap.add_argument("--depth", type=int, default=11)
    ap.add_argument("--seed", type=int, default=2024)
    ap.add_argument("--cpu-frames", type=int, default=-1, help="oracle frames for the CPU baseline (-1: all)")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline (for profiling runs)")
    ap.add_argument("--graph", type=int, default=1, help="replay each warp frame as a CUDA graph")
    ap.add_argument("--views", type=int, default=8, help="camera streams of the concurrent multi-view measurement")
    ap.add_argument("--threshold", type=float, default=0.5, help="confidence below which learned frames trace a pixel")
    ap.add_argument("--autotune", type=int, default=1, help="pick the trace configuration by measurement first")
    ap.add_argument("--guided", type=int, default=1,
                    help="learned frames walk pixels with a cached surface nearby from just in front of it")
    ap.add_argument("--certify", type=int, default=0,
                    help="guided learned frames certify reprojected pixels whose ray meets a cached face")
    ap.add_argument("--orbit-window", type=int, default=256, help="orbit frames in the quality window")
    ap.add_argument("--fast-window", type=int, default=512, help="fast-motion frames in the quality window")
    ap.add_argument("--extras", type=int, default=1,
                    help="also measure the GPU octree builder, the 64-view batch and the large depth-12 scene")
    ap.add_argument("--weights", default=os.path.join(PKG, "net_weights.npy"))
    ap.add_argument("--profile-case", choices=PROFILE_CASES, default=None,
                    help="run one small fixed workload for a profiler capture and exit")
    return ap.parse_args(argv)


# ------------------------------------------------------------ distributed --
def dist_env():
    return int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1)), int(os.environ.get("LOCAL_RANK", 0))


def reduce_max(value: float, world: int, device=None) -> float:
    """Max over ranks (identity for one rank)."""
    if world <= 1:
        return value
    import torch
    import torch.distributed as dist

    t = torch.tensor([value], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def aggregate(frames_per_rank: int, seconds_per_rank: float, world: int, device=None) -> tuple[float, float]:
    """(value, max seconds): all ranks' frames over the slowest rank's time."""
    t = reduce_max(seconds_per_rank, world, device)
    return frames_per_rank * world / t, t


def barrier(world: int) -> None:
    if world > 1:
        import torch.distributed as dist

        dist.barrier()


# ----------------------------------------------------------------- clocks --
class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled while the timed region runs."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.lines: list[str] = []
        self.reader = None

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
            return
        self.reader = threading.Thread(target=self._read, daemon=True)
        self.reader.start()

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        if self.reader:
            self.reader.join(timeout=2)
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.lines:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for name, flag in zip(names, parts[5:9]):
                if flag.lower() == "active":
                    reasons.add(name)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def _json_default(o):
    """numpy scalars in the JSON line as plain numbers."""
    if hasattr(o, "item"):
        return o.item()
    raise TypeError(f"{type(o).__name__} is not JSON serialisable")


def measured_peaks() -> dict:
    try:
        with open(PEAKS_FILE) as f:
            return json.load(f)
    except OSError:
        return {}


# ------------------------------------------------------------- reference --
def run_reference(args, rank: int, world: int) -> None:
    """Times the reference algorithm on the host cores (rank 0 only). Scenes
    and cameras come from oracle/scene_gen.py (bit-identical to the product's
    generator), so this process loads only the oracle's libraries."""
    if rank != 0:
        return
    sys.path.insert(0, ORACLE)
    import oracle
    import scene_gen

    oracle.build()
    W, H = (int(v) for v in args.res.split("x"))
    which = "reference" if oracle.ref_available() else "oracle"
    x, y, z, c = scene_gen.terrain_voxels(args.seed, args.depth, True)
    words, root = oracle.build_octree(args.depth, x, y, z, c, which=which)
    del x, y, z, c
    warp = oracle.Warp(args.depth, W, H, which=which)
    threads = oracle.max_threads()
    cams = [scene_gen.camera_path(1, args.depth, f) for f in range(args.warmup + args.steps)]
    for f in range(args.warmup):
        warp.frame(words, root, cams[f][0], cams[f][1], f, threads)
    t0 = time.perf_counter()
    for i in range(args.steps):
        f = args.warmup + i
        warp.frame(words, root, cams[f][0], cams[f][1], f, threads)
    dt = time.perf_counter() - t0
    fps = args.steps / dt
    cores = 1 if which == "reference" else threads
    line = {
        "impl": "reference", "metric": METRIC, "value": fps, "unit": "frames/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000.0 * dt / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": WORKLOAD, "res": [W, H], "depth": args.depth, "seed": args.seed},
        "cpu_baseline": {"value": fps, "unit": "frames/s", "cores": cores,
                         "kind": "reference" if which == "reference" else "port",
                         "sample": f"{args.steps} consecutive warped frames (after {args.warmup} untimed) of the "
                                   f"benchmark orbit at {W}x{H}; the reference's own pipeline (reprojection, "
                                   f"hole filter, hole rays): it has no learned stage"},
        "e2e": {"value": fps, "unit": "frames/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


# ------------------------------------------------------- GPU-side helpers --
class _DeviceArray:
    """A device buffer of the library as a torch tensor (no copy), through
    the CUDA array interface."""

    def __init__(self, ptr: int, n: int, typestr: str = "<i4"):
        self.__cuda_array_interface__ = {"shape": (n,), "typestr": typestr, "data": (int(ptr), False),
                                         "version": 3, "strides": None, "stream": None}


def bgrx_tensor(torch, target, device):
    return torch.as_tensor(_DeviceArray(target.device_outputs().bgrx, target.n), device=device)


class ErrorSum:
    """Squared-error sum and maximum error of BGRX frames against reference
    frames, accumulated on the GPU (on the library's stream)."""

    def __init__(self, torch, ext):
        self.torch, self.ext = torch, ext
        self.sse, self.mx, self.frames, self.pixels = [], [], 0, 0

    def add(self, a, b):
        torch = self.torch
        with torch.cuda.stream(self.ext):
            d = (a.view(torch.uint8).reshape(-1, 4)[:, :3].to(torch.int16)
                 - b.view(torch.uint8).reshape(-1, 4)[:, :3].to(torch.int16))
            self.sse.append((d.to(torch.float64) ** 2).sum())
            self.mx.append(d.abs().max())
        self.frames += 1
        self.pixels += a.numel()

    def result(self) -> dict:
        torch = self.torch
        with torch.cuda.stream(self.ext):
            sse = float(torch.stack(self.sse).sum().item())
            mx = int(torch.stack(self.mx).max().item())
        mse = sse / (3.0 * self.pixels)
        return {"psnr_db": 10 * np.log10(255.0 ** 2 / mse) if mse > 0 else float("inf"), "max_abs_error": mx,
                "frames": self.frames}


# ----------------------------------------------------------------- extras --
def measure_builder(svo, torch, octree, depth, seed, device):
    """GPU octree builder on the benchmark scene's voxels vs the host builder's
    words (timed on the device; voxel arrays already resident)."""
    x, y, z, c = svo.terrain_voxels(seed, depth, True)
    dev = [torch.from_numpy(np.ascontiguousarray(a, np.uint32).view(np.int32)).to(device) for a in (x, y, z, c)]
    torch.cuda.synchronize(device)
    ctx = svo.Context(device.index)
    ext = torch.cuda.ExternalStream(ctx.stream, device=device)
    ms = []
    for _ in range(4):
        s_ev, e_ev = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        s_ev.record(ext)
        ctx.build_octree(*(t.data_ptr() for t in dev), len(x), depth)
        e_ev.record(ext)
        e_ev.synchronize()
        ms.append(s_ev.elapsed_time(e_ev))
    built = ctx.download_octree()
    same = bool(built.root == octree.root and np.array_equal(built.words, octree.words))
    ctx.close()
    return {"voxels": int(len(x)), "gpu_ms": float(np.median(ms[1:])), "identical_to_host_builder": same,
            "note": "device events around svo_octree_build (sort, levels, layout, emission; includes its "
                    "host synchronisations)"}


def measure_batch(svo, torch, ctx, depth, device, n_views=64, steps=8):
    """64 cameras at seeded random poses, resolutions log-uniform 256^2..1920x1080,
    all traced by one persistent launch (svo_raycast_full_batch)."""
    rng = np.random.default_rng(64)
    res = []
    for _ in range(n_views):
        w = int(np.exp(rng.uniform(np.log(256), np.log(1920))))
        h = int(np.clip(w * rng.uniform(0.5, 1.0), 256, 1080))
        res.append((w, h))
    targets = [ctx.target(w, h) for w, h in res]
    views = [svo.camera_path(3, depth, k, w, h, seed=11) for k, (w, h) in enumerate(res)]
    ext = torch.cuda.ExternalStream(ctx.stream, device=device)
    for _ in range(2):
        ctx.raycast_full_batch(targets, views)
    ctx.synchronize()
    ms = []
    for _ in range(steps):
        s_ev, e_ev = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        s_ev.record(ext)
        ctx.raycast_full_batch(targets, views)
        e_ev.record(ext)
        e_ev.synchronize()
        ms.append(s_ev.elapsed_time(e_ev))
    rays = sum(w * h for w, h in res)
    for t in targets:
        t.close()
    t_ms = float(np.mean(ms))
    return {"views": n_views, "rays_per_launch": rays, "ms_per_launch": t_ms, "mrays_per_s": rays / t_ms / 1e3,
            "timing": "device events per launch (the batch's working set exceeds L2)"}


def streams_timed(torch, ctxs, go, frames, first, device, flush=None):
    """Device time of `frames` steps in which every context renders one frame
    on its own stream: a start event on the first stream that every other
    stream waits for, an end event per stream, the step's time the latest end.
    The host enqueues every step before reading the events (the first stream
    waits for all ends of a step before the next one starts), so no host
    launch latency falls inside a step; `flush(stream)` enqueues the L2 flush
    ahead of a step's start event."""
    exts = [torch.cuda.ExternalStream(c.stream, device=device) for c in ctxs]
    steps = []
    for i in range(frames):
        f = first + i
        if flush is not None:
            flush(exts[0])
        start = torch.cuda.Event(enable_timing=True)
        start.record(exts[0])
        for e in exts[1:]:
            e.wait_event(start)
        ends = []
        for k in range(len(ctxs)):
            go(k, f)
            ev = torch.cuda.Event(enable_timing=True)
            ev.record(exts[k])
            ends.append(ev)
        for ev in ends[1:]:
            exts[0].wait_event(ev)
        steps.append((start, ends))
    for ev in steps[-1][1]:
        ev.synchronize()
    return sum(max(start.elapsed_time(ev) for ev in ends) for start, ends in steps)


def measure_large(svo, torch, args, device, frames=16, views=8):
    """Depth-12 terrain + 2000 solid boxes (built on the GPU), 3840x2160, fast
    motion, 8 camera streams at once: learned frames/s (all views), plain warp
    frames/s, full raycast frames/s of one view and the learned frames' PSNR."""
    W, H, depth = 3840, 2160, 12
    t0 = time.perf_counter()
    x, y, z, c = svo.terrain_voxels(args.seed, depth, True, 2000)
    gen_s = time.perf_counter() - t0
    dev = [torch.from_numpy(np.ascontiguousarray(a, np.uint32).view(np.int32)).to(device) for a in (x, y, z, c)]
    n = len(x)
    del x, y, z, c
    torch.cuda.synchronize(device)
    base = svo.Context(device.index)
    t0 = time.perf_counter()
    base.build_octree(*(t.data_ptr() for t in dev), n, depth)
    build_s = time.perf_counter() - t0
    del dev
    nw, root, _ = base.octree_info()
    words = base.download_octree().words
    d_words = torch.from_numpy(words.view(np.int32)).to(device)
    torch.cuda.synchronize(device)
    ctxs, tgts, nets = [], [], []
    for k in range(views):
        cx = svo.Context(device.index)
        cx.upload_device(d_words.data_ptr(), nw, root, depth)
        t = cx.target(W, H)
        t.use_graph(True)
        t.set_guided(bool(args.guided))
        t.set_certified(bool(args.certify))
        net = svo.Net(cx)
        net.load_file(args.weights)
        ctxs.append(cx)
        tgts.append(t)
        nets.append(net)

    def vw(k, f):
        return svo.camera_path(2, depth, 64 * k + f, W, H)

    out = {"workload": "depth-12 terrain + 2000 boxes, 3840x2160, fast motion, 8 streams",
           "voxels": int(n), "octree_words": int(nw), "voxel_generation_s": gen_s, "gpu_build_s": build_s,
           "timing": "device events: a start event every stream waits for, the latest stream's end event; "
                     "the 8 views' planes (~2 GB) exceed L2"}
    for mode in ("learned", "plain"):
        def go(k, f):
            if mode == "learned":
                ctxs[k].warp_frame_learned(tgts[k], vw(k, f), f, nets[k], args.threshold)
            else:
                ctxs[k].warp_frame(tgts[k], vw(k, f), f)
        for f in range(4):
            for k in range(views):
                go(k, f)
        for cx in ctxs:
            cx.synchronize()
        ms = streams_timed(torch, ctxs, go, frames, 4, device)
        out[mode + "_frames_per_s"] = views * frames / (ms * 1e-3)
    full = base.target(W, H)
    ext = torch.cuda.ExternalStream(base.stream, device=device)
    base.raycast_full(full, vw(0, 4))
    base.synchronize()
    fms = []
    for f in range(5, 5 + 8):
        s_ev, e_ev = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        s_ev.record(ext)
        base.raycast_full(full, vw(0, f))
        e_ev.record(ext)
        e_ev.synchronize()
        fms.append(s_ev.elapsed_time(e_ev))
    out["full_frames_per_s_one_view"] = 1000.0 / float(np.mean(fms))
    # learned quality on view 0, frames 4-35 against the full raycast
    tq = ctxs[0].target(W, H)
    tq.set_guided(bool(args.guided))
    err = ErrorSum(torch, ext)
    ctxs[0].synchronize()
    for f in range(0, 36):
        v = vw(0, f)
        ctxs[0].warp_frame_learned(tq, v, f, nets[0], args.threshold)
        if f >= 4:
            ctxs[0].synchronize()
            base.raycast_full(full, v)
            err.add(bgrx_tensor(torch, tq, device), bgrx_tensor(torch, full, device))
            base.synchronize()
    q = err.result()
    out["learned_psnr_db"] = q["psnr_db"]
    out["learned_quality_frames"] = "4-35 of view 0"
    tq.close()
    full.close()
    for t in tgts:
        t.close()
    for net in nets:
        net.close()
    for cx in ctxs:
        cx.close()
    base.close()
    del d_words
    return out


def measure_training(svo, torch, args, device, W=1920, H=1024, steps=6):
    """One training step of the net at the benchmark's frame size: the
    tensor-core forward keeping its activations, the loss, the tensor-core
    backward convolutions (data and weight gradients) and Adam, on seeded
    features and targets already on the device; device events per step."""
    ctx = svo.Context(device.index)
    net = svo.Net(ctx)
    net.load_file(args.weights)
    g = torch.Generator(device=device).manual_seed(7)
    feat = torch.rand((8, H, W), generator=g, device=device)
    tgt = torch.randint(0, 1 << 24, (H * W,), generator=g, device=device, dtype=torch.int32)
    torch.cuda.synchronize(device)
    ext = torch.cuda.ExternalStream(ctx.stream, device=device)
    ms = []
    for i in range(steps + 2):
        s_ev, e_ev = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        s_ev.record(ext)
        net.backward(feat.data_ptr(), tgt.data_ptr(), W, H, 0.015, 0.1, read_loss=False)
        net.adam(1e-5)
        e_ev.record(ext)
        e_ev.synchronize()
        if i >= 2:
            ms.append(s_ev.elapsed_time(e_ev))
    net.close()
    ctx.close()
    t = float(np.mean(ms))
    # forward 12,096 + data gradients of layers 3-1 10,368 + weight gradients 12,096 FLOP per pixel
    flops = 34560.0 * W * H
    return {"workload": f"net training step {W}x{H} (forward, loss, backward, Adam)", "ms_per_step": t,
            "tflops_algorithmic": flops / (t * 1e-3) / 1e12,
            "note": "tensor-core forward and backward convolutions; gradients enter the MMAs as two bf16 parts"}


def measure_full_512(svo, torch, device, seed, no_cpu: bool, steps: int = 20):
    """The plain full raycast configuration: 512x512, depth-9 (512^3) solid
    terrain (the GPU builder from the seeded voxels), one camera at 1.5x
    extent looking at the centre, 60 degree vertical field of view."""
    W = H = 512
    depth = 9
    x, y, z, c = svo.terrain_voxels(seed, depth, False)
    dev = [torch.from_numpy(np.ascontiguousarray(a, np.uint32).view(np.int32)).to(device) for a in (x, y, z, c)]
    n = len(x)
    del x, y, z, c
    torch.cuda.synchronize(device)
    ctx = svo.Context(device.index)
    ctx.build_octree(*(t.data_ptr() for t in dev), n, depth)
    del dev
    tgt = ctx.target(W, H)
    view = svo.camera_path(0, depth, 0, W, H, fov=1.1547)
    ext = torch.cuda.ExternalStream(ctx.stream, device=device)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=device)
    # packet shape / block size / node staging for this frame size and octree
    tune = ctx.autotune(tgt, view, repeats=3)
    tuned = min(tune, key=lambda r: r["ms"]) if tune else None
    for _ in range(3):
        ctx.raycast_full(tgt, view)
    ctx.synchronize()
    evs = []
    for _ in range(steps):
        with torch.cuda.stream(ext):  # the flush on the launch's stream: no host latency inside the events
            flush.zero_()
        s_ev, e_ev = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        s_ev.record(ext)
        ctx.raycast_full(tgt, view)
        e_ev.record(ext)
        evs.append((s_ev, e_ev))
    ctx.synchronize()
    ms = [s_ev.elapsed_time(e_ev) for s_ev, e_ev in evs]
    t_ms = float(np.mean(ms))
    out = {"workload": "plain full raycast 512x512, depth-9 solid terrain, 60 deg vertical FOV, one camera",
           "voxels": int(n), "ms_per_frame": t_ms, "mrays_per_s": W * H / t_ms / 1e3,
           "l2": "flushed before every timed launch", "autotune": tuned}
    if not no_cpu:
        sys.path.insert(0, ORACLE)
        import oracle

        oc = ctx.download_octree()
        col, xyzw = tgt.full()
        vox = tgt.voxels()
        ocol, oxyzw, ovox, st = oracle.raycast_full(depth, oc.words, oc.root, view.pos_array, view.m_array, W, H,
                                                    view.fovx, view.fovy, oracle.max_threads())
        out["parity_vs_oracle"] = bool(np.array_equal(col, ocol) and np.array_equal(vox, ovox)
                                       and np.array_equal(xyzw.view(np.uint32), oxyzw.view(np.uint32)))
        out["boundary_ray_fraction"] = float(st[3]) / float(st[0])
        out["boundary_rays"] = int(st[3])
        out["hit_boundary_ray_fraction"] = float(st[6]) / float(st[0])
        out["mismatching_rays"] = int(np.count_nonzero(col != ocol))
    tgt.close()
    ctx.close()
    return out


# ---------------------------------------------------------- profile cases --
def run_profile_case(case: str) -> None:
    """Small, fixed GPU workloads for profiler captures (ncu), one per case:
    learned / guided: 8 learned warp frames (committed weights, threshold
    0.5, orbit) without / with guided walks; plain: 8 plain warp frames;
    full: 4 full raycasts; build: 2 GPU octree builds of the benchmark
    terrain's voxels (all 1920x1024, depth-11 benchmark terrain); full512: 4
    full raycasts of the 512x512 depth-9 solid-terrain configuration; train:
    3 training steps of the net at 1920x1024 on seeded features."""
    sys.path.insert(0, PKG)
    import svo_gb300 as svo

    W, H, DEPTH, SEED = 1920, 1024, 11, 2024
    if case == "train":
        import torch

        ctx = svo.Context(0)
        net = svo.Net(ctx)
        net.load_file(os.path.join(PKG, "net_weights.npy"))
        g = torch.Generator(device="cuda").manual_seed(7)
        feat = torch.rand((8, H, W), generator=g, device="cuda")
        tgt = torch.randint(0, 1 << 24, (H * W,), generator=g, device="cuda", dtype=torch.int32)
        torch.cuda.synchronize()
        for _ in range(3):
            net.backward(feat.data_ptr(), tgt.data_ptr(), W, H, 0.015, 0.1, read_loss=False)
            net.adam(1e-5)
        ctx.synchronize()
        print("ok")
        net.close()
        ctx.close()
        return
    if case in ("build", "full512"):
        import torch

        depth = 9 if case == "full512" else DEPTH
        x, y, z, c = svo.terrain_voxels(SEED, depth, case == "build")
        dev = [torch.from_numpy(np.ascontiguousarray(a, np.uint32).view(np.int32)).cuda() for a in (x, y, z, c)]
        torch.cuda.synchronize()
        ctx = svo.Context(0)
        for _ in range(2 if case == "build" else 1):
            ctx.build_octree(*(t.data_ptr() for t in dev), len(x), depth)
        if case == "full512":
            t = ctx.target(512, 512)
            for _ in range(4):
                ctx.raycast_full(t, svo.camera_path(0, depth, 0, 512, 512, fov=1.1547))
        ctx.synchronize()
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
        net.load_file(os.path.join(PKG, "net_weights.npy"))
        for f in range(8):
            ctx.warp_frame_learned(t, svo.camera_path(1, DEPTH, f, W, H), f, net, 0.5)
        ctx.synchronize()
        print("ok", t.requested())
    elif case == "plain":
        for f in range(8):
            ctx.warp_frame(t, svo.camera_path(1, DEPTH, f, W, H), f)
        ctx.synchronize()
        print("ok", t.holes()[1])
    else:
        for f in range(4):
            ctx.raycast_full(t, svo.camera_path(1, DEPTH, 3 + f, W, H))
        ctx.synchronize()
        print("ok")
    ctx.close()


# ------------------------------------------------------------------- ours --
def run_ours(args, rank: int, world: int, local_rank: int) -> None:
    import torch

    sys.path.insert(0, PKG)
    import svo_gb300 as svo

    torch.cuda.set_device(local_rank)
    device = torch.device("cuda", local_rank)
    W, H = (int(v) for v in args.res.split("x"))
    N = W * H
    depth = args.depth
    t_build = time.perf_counter()
    octree = svo.build_terrain(depth, args.seed, shell=True)
    t_build = time.perf_counter() - t_build
    ctx = svo.Context(local_rank)
    ctx.upload(octree, validate=True)
    net = svo.Net(ctx)
    net.load_file(args.weights)
    thr = args.threshold
    tgt_l, full = ctx.target(W, H), ctx.target(W, H)
    tgt_l.set_guided(bool(args.guided))
    tgt_l.set_certified(bool(args.certify))
    if args.graph:
        tgt_l.use_graph(True)
    ext = torch.cuda.ExternalStream(ctx.stream, device=device)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=device)
    frame_offset = rank * 512  # replicas render different stretches of the orbit

    def view(f, kind=1):
        return svo.camera_path(kind, depth, frame_offset + f, W, H)

    # trace packet shape / block size / node staging: measured on this GPU and scene
    tune = ctx.autotune(full, view(args.warmup), repeats=3) if args.autotune else []
    tuned = min(tune, key=lambda r: r["ms"]) if tune else None
    # and the learned frames' tracer, on 16 learned frames of the same path
    tune_l = []
    if args.autotune:
        tt = ctx.target(W, H)
        tt.set_guided(bool(args.guided))
        tt.set_certified(bool(args.certify))
        tt.use_graph(bool(args.graph))
        tune_l = ctx.autotune_learned(tt, [view(f) for f in range(16)], net, thr)
        tt.close()
    tuned_l = min(tune_l, key=lambda r: r["ms"]) if tune_l else None

    def flush_l2():
        flush.zero_()
        torch.cuda.synchronize(device)

    def flush_on_stream():
        # the L2 flush enqueued on the frames' stream ahead of the next step's
        # start event: the host keeps enqueueing, so each step's events time
        # the device work only (no host launch latency inside them)
        with torch.cuda.stream(ext):
            flush.zero_()

    def new_target(guided=None):
        t = ctx.target(W, H)
        if args.graph:
            t.use_graph(True)
        if guided is not None:
            t.set_guided(guided)
        t.set_certified(bool(args.certify))
        return t

    def plain(t):
        return lambda f, v: ctx.warp_frame(t, v, f)

    def learned(t, th=thr):
        return lambda f, v: ctx.warp_frame_learned(t, v, f, net, th)

    def timed(render, kind=1):
        """Device time (ms) of each of args.steps frames after args.warmup untimed ones."""
        for f in range(args.warmup):
            render(f, view(f, kind))
        ctx.synchronize()
        starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
        ends = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
        for i in range(args.steps):
            f = args.warmup + i
            v = view(f, kind)
            flush_on_stream()
            starts[i].record(ext)
            render(f, v)
            ends[i].record(ext)
        ctx.synchronize()
        return [s_.elapsed_time(e_) for s_, e_ in zip(starts, ends)]

    # ---- headline: learned warp frames, device time per step
    barrier(world)
    torch.cuda.synchronize(device)
    for f in range(args.warmup):
        ctx.warp_frame_learned(tgt_l, view(f), f, net, thr)
    ctx.synchronize()
    clocks = ClockSampler(local_rank)
    clocks.start()
    launches0 = ctx.launch_count()
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    for i in range(args.steps):
        f = args.warmup + i
        v = view(f)
        flush_on_stream()
        starts[i].record(ext)
        ctx.warp_frame_learned(tgt_l, v, f, net, thr)
        ends[i].record(ext)
    ctx.synchronize()
    launches = ctx.launch_count() - launches0
    step_ms = [s_.elapsed_time(e_) for s_, e_ in zip(starts, ends)]
    clock_info = clocks.stop()
    barrier(world)
    torch.cuda.synchronize(device)
    learned_s = sum(step_ms) / 1000.0
    value, _ = aggregate(args.steps, learned_s, world, device if world > 1 else None)
    ms_per_step = 1000.0 * learned_s / args.steps

    # ---- the plain warp pipeline (bit-exact with the reference) on the same frames
    tgt_p = new_target()
    plain_ms = timed(plain(tgt_p))
    plain_fps = 1000.0 / statistics.mean(plain_ms)
    tgt_p.close()

    # ---- per-stage events of both pipelines
    def stage_times(render_target, render, names):
        render_target.set_profiling(True)
        for f in range(args.warmup):
            render(f, view(f))
        ctx.synchronize()
        rows = []
        for i in range(args.steps):
            f = args.warmup + i
            flush_l2()
            render(f, view(f))
            rows.append(render_target.stage_times())
        rows = np.array([r for r in rows if len(r) == len(names)], np.float64)
        if rows.size == 0:
            raise RuntimeError("per-stage CUDA events returned no timings")
        return {n: float(rows[:, k].mean()) for k, n in enumerate(names)}

    t_sp = new_target()
    t_sl = new_target(bool(args.guided))
    stage_ms = stage_times(t_sp, plain(t_sp), ["project", "resolve_gather", "hole_scan", "hole_write", "trace",
                                               "fill_colorize"])
    stage_ms_learned = stage_times(t_sl, learned(t_sl), ["project", "resolve", "net", "trace"])
    t_sp.close()
    t_sl.close()

    # ---- plain full raycast of the same frames
    full_ev = []
    for i in range(args.steps):
        f = args.warmup + i
        v = view(f)
        flush_on_stream()
        s_ev, e_ev = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        s_ev.record(ext)
        ctx.raycast_full(full, v)
        e_ev.record(ext)
        full_ev.append((s_ev, e_ev))
    ctx.synchronize()
    full_ms = [s_ev.elapsed_time(e_ev) for s_ev, e_ev in full_ev]
    full_fps = 1000.0 / statistics.mean(full_ms)
    mrays_full = N * full_fps / 1e6

    # ---- end to end through the C ABI with host buffers (learned frames)
    host_img = torch.empty(N, dtype=torch.int32, pin_memory=True).numpy().view(np.uint32)
    tgt3 = new_target(bool(args.guided))
    for f in range(args.warmup):
        ctx.warp_frame_learned(tgt3, view(f), f, net, thr)
        tgt3.bgrx_into(host_img)
    # blocking: every frame's image read back before the next frame is issued
    e2e_block_s = 0.0
    for i in range(args.steps):
        f = args.warmup + i
        flush_l2()
        t0 = time.perf_counter()
        ctx.warp_frame_learned(tgt3, view(f), f, net, thr)  # camera host -> device inside the call
        tgt3.bgrx_into(host_img)                              # BGRX8 frame device -> pinned host, synchronising
        e2e_block_s += time.perf_counter() - t0
    e2e_block, _ = aggregate(args.steps, e2e_block_s, world, device if world > 1 else None)
    # pipelined, as an application renders: frame i's image is copied to pinned
    # host memory (svo_read_bgrx_async) while frame i + 1 renders -- the copy is
    # issued after the L2 flush that precedes frame i + 1, so it overlaps that
    # frame's first kernels and not the flush; the flushes (device events on the
    # frames' stream) are not counted; the last image is waited for
    hosts = [torch.empty(N, dtype=torch.int32, pin_memory=True).numpy().view(np.uint32) for _ in range(2)]
    base = args.warmup + args.steps  # the orbit continues where the blocking loop stopped
    for i in range(args.warmup):  # the graph with the copy's wait node is captured here
        f = base + i
        ctx.warp_frame_learned(tgt3, view(f), f, net, thr)
        tgt3.bgrx_into_async(hosts[i % 2])
    tgt3.readback_wait()
    ctx.synchronize()
    fl_s = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    fl_e = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    t0 = time.perf_counter()
    for i in range(args.steps):
        f = base + args.warmup + i
        with torch.cuda.stream(ext):
            fl_s[i].record(ext)
            flush.zero_()
            fl_e[i].record(ext)
        if i > 0:
            tgt3.bgrx_into_async(hosts[(i - 1) % 2])  # frame f - 1's image, behind this flush
        ctx.warp_frame_learned(tgt3, view(f), f, net, thr)
    tgt3.bgrx_into_async(hosts[(args.steps - 1) % 2])
    tgt3.readback_wait()
    t1 = time.perf_counter()
    ctx.synchronize()
    flush_s = sum(fl_s[i].elapsed_time(fl_e[i]) for i in range(args.steps)) / 1e3
    e2e_value, _ = aggregate(args.steps, (t1 - t0) - flush_s, world, device if world > 1 else None)
    tgt3.close()

    # ---- quality over fixed windows against the full raycast of the same cameras
    def net_tiles(g):
        # 56x24 net tiles holding an unguided pixel (the tiles k_guide lists)
        tw, th = -(-W // 56), -(-H // 24)
        pad = np.zeros((th * 24, tw * 56), bool)
        pad[:H, :W] = (g == -1.0).reshape(H, W)
        return int(pad.reshape(th, 24, tw, 56).any(axis=(1, 3)).sum())

    def quality(render, t, kind, frames, traced_of, walked=False, sample=4):
        """Frames 0..frames-1 of camera path `kind`, each against the full
        raycast of its camera; the ray fractions on every `sample`-th frame."""
        err = ErrorSum(torch, ext)
        traced, walk, cert, tiles = [], [], [], []
        for f in range(frames):
            v = view(f, kind)
            render(f, v)
            ctx.raycast_full(full, v)
            err.add(bgrx_tensor(torch, t, device), bgrx_tensor(torch, full, device))
            if f % sample == sample - 1:
                traced.append(traced_of(t) / N)
                if walked:
                    g = t.guide()
                    walk.append(float((g >= 0).mean()))
                    cert.append(float((g == -2.0).mean()))
                    tiles.append(net_tiles(g))
        ctx.synchronize()
        out = {**err.result(), "window": f"frames 0-{frames - 1}", "traced_fraction": float(np.mean(traced))}
        if walked:
            out["walked_fraction"] = float(np.mean(walk))
            out["certified_fraction"] = float(np.mean(cert))
            out["net_tiles"] = float(np.mean(tiles))
        return out

    def holes_of(t):
        return t.holes()[1]

    def requested_of(t):
        return t.requested()

    ow, fw = args.orbit_window, args.fast_window
    tq = ctx.target(W, H)
    q_plain = quality(plain(tq), tq, 1, ow, holes_of)
    tq.close()
    tq = new_target(bool(args.guided))
    q_learned = quality(learned(tq), tq, 1, ow, requested_of, bool(args.guided))
    tq.close()
    # the learned frame without guidance (every pixel to the net, low-confidence
    # pixels traced from the camera), for comparison
    unguided = None
    if args.guided:
        tq = new_target(False)
        ms = timed(learned(tq))
        tq.close()
        tq = new_target(False)
        unguided = {"frames_per_s": 1000.0 / statistics.mean(ms), **quality(learned(tq), tq, 1, ow, requested_of)}
        tq.close()
    # fast motion (2 deg/frame + 0.05 extent/frame), the learned configuration
    tq = new_target(bool(args.guided))
    fast_ms = timed(learned(tq), kind=2)
    tq.close()
    tq = new_target(bool(args.guided))
    q_fast = quality(learned(tq), tq, 2, fw, requested_of, bool(args.guided))
    tq.close()
    tq = new_target()
    q_fast_plain = quality(plain(tq), tq, 2, fw, holes_of)
    tq.close()
    # the lowest confidence threshold of {0.5, 0.6, 0.7, 0.8, 0.9} reaching 38 dB
    # over the fast-motion window, and its frame rate
    fast_38 = None
    for th in (0.5, 0.6, 0.7, 0.8, 0.9):
        if th == thr:
            q = q_fast
        else:
            tq = new_target(bool(args.guided))
            q = quality(learned(tq, th), tq, 2, fw, requested_of)
            tq.close()
        if q["psnr_db"] >= 38.0:
            if th == thr:
                ms = fast_ms
            else:
                tq = new_target(bool(args.guided))
                ms = timed(learned(tq, th), kind=2)
                tq.close()
            fast_38 = {"threshold": th, "frames_per_s": 1000.0 / statistics.mean(ms), **q}
            break

    # ---- several camera streams at once: one context (stream) per view, the
    # octree words shared; the warp frames of all views are in flight together
    # so one view's latency tail overlaps the others' work.
    multiview = None
    if args.views > 1:
        d_words = torch.from_numpy(octree.words.view(np.int32)).to(device)
        torch.cuda.synchronize(device)
        ctxs, tgts, nets = [], [], []
        for k in range(args.views):
            c = svo.Context(local_rank)
            c.upload_device(d_words.data_ptr(), octree.words.size, octree.root, octree.depth)
            t = c.target(W, H)
            t.set_guided(bool(args.guided))
            t.set_certified(bool(args.certify))
            n = svo.Net(c)
            n.load_file(args.weights)
            if args.graph:
                t.use_graph(True)
            ctxs.append(c)
            tgts.append(t)
            nets.append(n)

        def mv_view(k, f):
            return svo.camera_path(1, depth, frame_offset + 37 * k + f, W, H)

        def flush_stream(st):
            with torch.cuda.stream(st):
                flush.zero_()

        multiview = {"views": args.views,
                     "timing": "device events: a start event every stream waits for, the latest stream's end "
                               "event, L2 flushed before every step"}
        for mode in ("learned", "plain"):
            def go(k, f):
                if mode == "learned":
                    ctxs[k].warp_frame_learned(tgts[k], mv_view(k, f), f, nets[k], thr)
                else:
                    ctxs[k].warp_frame(tgts[k], mv_view(k, f), f)
            for f in range(args.warmup):
                for k in range(args.views):
                    go(k, f)
            for c in ctxs:
                c.synchronize()
            mv_ms = streams_timed(torch, ctxs, go, args.steps, args.warmup, device, flush_stream)
            multiview[mode] = {"frames_per_s": args.views * args.steps / (mv_ms * 1e-3),
                               "ms_per_step": mv_ms / args.steps}
        for t in tgts:
            t.close()
        for n in nets:
            n.close()
        for c in ctxs:
            c.close()
        del d_words

    # ---- CPU oracle on the same frames: the CPU baseline, parity of the last
    # plain frame, fetch counts for the trace's algorithmic bytes and the
    # boundary-ray fraction of the full raycast.
    cpu = None
    bytes_per_ray = walk_bytes_per_ray = None
    parity = None
    boundary = None
    if not args.no_cpu and rank == 0:
        sys.path.insert(0, ORACLE)
        import oracle

        oracle.build()
        threads = oracle.max_threads()
        warp = oracle.Warp(depth, W, H)
        n_cpu = args.steps if args.cpu_frames < 0 else min(args.cpu_frames, args.steps)
        for f in range(args.warmup):
            v = view(f)
            warp.frame(octree.words, octree.root, v.pos_array, v.m_array, f, threads)
        t0 = time.perf_counter()
        for i in range(n_cpu):
            f = args.warmup + i
            v = view(f)
            warp.frame(octree.words, octree.root, v.pos_array, v.m_array, f, threads)
        cpu_s = time.perf_counter() - t0
        cpu = {"value": n_cpu / cpu_s, "unit": "frames/s", "cores": threads, "kind": "port",
               "sample": f"{n_cpu} consecutive warped frames of the benchmark orbit at {W}x{H} "
                         f"(after {args.warmup} untimed), oracle port of kernel.cl/raycast.h, OpenMP"}
        if n_cpu == args.steps:
            tp = ctx.target(W, H)
            for f in range(args.warmup + args.steps):
                ctx.warp_frame(tp, view(f), f)
            parity = bool(np.array_equal(warp.tex(), tp.bgrx()))
            tp.close()
        # algorithmic bytes per traced ray, counted by the oracle on the full
        # raycast of the last frame: node words + colour word read, float4 +
        # colour word written (4 * fetches + 20)
        v = view(args.warmup + args.steps - 1)
        _, _, _, st = oracle.raycast_full(depth, octree.words, octree.root, v.pos_array, v.m_array, W, H,
                                          1.0, 1.0, threads)
        bytes_per_ray = (4.0 * (float(st[1]) + float(st[2])) + 20.0 * float(st[0])) / float(st[0])
        boundary = {"fraction": float(st[3]) / float(st[0]), "rays": int(st[3]), "of": int(st[0]),
                    "hit_fraction": float(st[6]) / float(st[0]),
                    "definition": "fraction: a step landed a coordinate within 1 ulp of a leaf face; hit_fraction: "
                                  "the hit point lies within 1 ulp of a face of its cell (other than the entry face)",
                    "frame": "full raycast of the last timed orbit frame"}
        if args.guided:
            # the same count for the guided walks of that frame, from the start
            # distances the GPU used (read back after the frame)
            tg = ctx.target(W, H)
            tg.set_guided(True)
            tg.set_certified(bool(args.certify))
            for f in range(args.warmup + args.steps):
                ctx.warp_frame_learned(tg, view(f), f, net, thr)
            g = tg.guide()
            tg.close()
            _, _, stw = oracle.raycast_guided(depth, octree.words, octree.root, v.pos_array, v.m_array, W, H,
                                              np.where(g >= 0, g, -1.0).astype(np.float32), threads, stats=True)
            walk_bytes_per_ray = (4.0 * (float(stw[1]) + float(stw[2])) + 20.0 * float(stw[0])) / max(float(stw[0]), 1.0)

    extras = {}
    if args.extras and rank == 0:
        extras["full_raycast_512x512_depth9"] = measure_full_512(svo, torch, device, args.seed, args.no_cpu)
        extras["net_training"] = measure_training(svo, torch, args, device)
        extras["octree_builder"] = measure_builder(svo, torch, octree, depth, args.seed, device)
        extras["batch_64_views"] = measure_batch(svo, torch, ctx, depth, device)
        extras["large"] = measure_large(svo, torch, args, device)

    # ---- rooflines: algorithmic bytes / stage event time against the L2 read
    # peak measured here and the HBM copy peak measured on this GPU model
    peaks = measured_peaks()
    hbm = peaks.get("hbm_gbs")
    tflops = peaks.get("bf16_tflops")
    l2_buf = torch.empty(48 * 1024 * 1024 // 4, dtype=torch.float32, device=device).fill_(1.0)
    torch.cuda.synchronize(device)
    l2_peak = max(ctx.read_bandwidth(l2_buf.data_ptr(), l2_buf.numel() * 4, 40) for _ in range(3))
    del l2_buf
    hbm_peak = hbm if hbm else 6800.0

    def fracs(algo_bytes, ms):
        gbs = algo_bytes / (ms * 1e-3) / 1e9
        return {"achieved_gbs": gbs, "l2_frac": gbs / l2_peak, "hbm_frac": gbs / hbm_peak,
                "algorithmic_bytes": algo_bytes, "ms": ms}

    stage_rooflines = {
        # every source pixel's colour + float4 read, one 8-byte atomic per
        # cached point (counted for every pixel: holes are few)
        "k_project": fracs(N * (20.0 + 8.0), stage_ms_learned["project"]),
    }
    halo = 340.0 / 256.0  # pixels read per pixel by k_guide's 34x10 halo of a 32x8 block
    if args.guided:
        # k_guide<1>: the halo's keys and winning sources' colour + float4, the
        # block's plane write, the start distance (the tracer clears the keys)
        stage_rooflines["k_guide (gather fused)"] = fracs(N * ((8.0 + 20.0) * halo + 20.0 + 4.0),
                                                          stage_ms_learned["resolve"])
    else:
        # gather: key read + reset, winner colour + float4 read, plane write
        stage_rooflines["k_resolve_gather"] = fracs(N * (8.0 + 8.0 + 20.0 + 20.0), stage_ms_learned["resolve"])
    roofline = None
    roofline_net = None
    # rays of one learned frame's trace launch: the requested pixels and the
    # refresh tile from the camera, plus (guided) the walked pixels
    rays_camera = (q_learned["traced_fraction"] * N + (W // 8 + 15) // 16 * 16 * ((H // 4 + 15) // 16 * 16))
    rays_walked = q_learned.get("walked_fraction", 0.0) * N
    if bytes_per_ray is not None and stage_ms_learned["trace"] > 0 and (walk_bytes_per_ray or not args.guided):
        algo = bytes_per_ray * rays_camera + (walk_bytes_per_ray or 0.0) * rays_walked
        tr = fracs(algo, stage_ms_learned["trace"])
        achieved = tr["achieved_gbs"]
        roofline = {"bound": "issue",
                    "kernel": "k_trace_warp (learned frame: requested pixels, refresh tile"
                              + (", guided walks)" if args.guided else ")"),
                    "achieved": achieved, "peak": hbm_peak, "unit": "GB/s", "frac": achieved / hbm_peak,
                    "peak_source": "measured" if hbm else "fallback",
                    "l2": {"achieved": achieved, "peak": l2_peak, "frac": achieved / l2_peak,
                           "peak_source": "measured in this run: the library's read probe over a 48 MiB "
                                          "L2-resident buffer"},
                    "hbm": {"achieved": achieved, "peak": hbm_peak, "frac": achieved / hbm_peak,
                            "peak_source": "MEASURED_PEAKS.json hbm_gbs (copy)" if hbm else "fallback"},
                    "algorithmic_bytes_per_launch": algo, "bytes_per_ray": bytes_per_ray,
                    "walk_bytes_per_ray": walk_bytes_per_ray,
                    "rays_per_launch": rays_camera + rays_walked, "walked_rays_per_launch": rays_walked,
                    "traffic": None,
                    "traffic_source": f"not captured in this run; DRAM bytes per launch of the same frame: "
                                      f"{TRACE_PROFILE}",
                    "bound_source": f"{TRACE_PROFILE}: issue slots and SIMT lanes (ncu), neither memory roof "
                                    f"binds"}
    if stage_ms_learned["net"] > 0:
        # 2 * 9 * (8*16 + 16*16 + 16*16 + 16*4) per output pixel, over the
        # tiles the net ran on (every tile unless guided)
        net_pixels = q_learned["net_tiles"] * 56 * 24 if "net_tiles" in q_learned else N
        flops = 12096.0 * net_pixels
        ach = flops / (stage_ms_learned["net"] * 1e-3) / 1e12
        peak = tflops if tflops else 1900.0
        roofline_net = {"bound": "tensor", "kernel": "k_net_infer", "achieved": ach, "peak": peak,
                        "unit": "TFLOP/s", "frac": ach / peak, "peak_source": "measured" if tflops else "fallback",
                        **{k: v for k, v in fracs(24.0 * net_pixels, stage_ms_learned["net"]).items()
                           if k in ("achieved_gbs", "l2_frac", "hbm_frac")},
                        "flops_per_launch": flops, "net_pixels_per_launch": net_pixels,
                        "note": ("net stage events: k_net_infer (its warps append the requests)" if args.guided
                                 else "net stage events: k_net_infer plus the request scan")}
    if rank == 0:
        like = None
        if cpu:
            like = {"same_config": True, "workload": f"plain warp frames {args.warmup}-{args.warmup + args.steps - 1} "
                                                     f"of the orbit at {W}x{H} (the reference's algorithm)",
                    "gpu_frames_per_s": plain_fps, "cpu_frames_per_s": cpu["value"], "cpu_cores": cpu["cores"],
                    "ratio": plain_fps / cpu["value"]}
        fast_gate = bool(q_fast["psnr_db"] >= 38.0)
        line = {
            "metric": METRIC, "value": value, "unit": "frames/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_per_step, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32 traversal, bf16 net",
            "data": "synthetic: seeded value-noise fBm terrain (visible shell), seeded orbit camera",
            "config": {"workload": WORKLOAD, "res": [W, H], "depth": depth, "seed": args.seed,
                       "octree_words": int(octree.words.size), "voxels": int(octree.voxels),
                       "confidence_threshold": thr, "weights": os.path.relpath(args.weights, ROOT),
                       "guided_walks": bool(args.guided),
                       "l2": "flushed before every timed step (256 MiB device write, outside the step events)",
                       "cuda_graph": bool(args.graph), "replicas": world},
            "e2e": {"value": e2e_value, "unit": "frames/s", "h2d_bytes_per_step": 4 * 33,
                    "d2h_bytes_per_step": 4 * N,
                    "how": "svo_warp_frame_learned (camera in) then svo_read_bgrx_async of each BGRX8 frame into "
                           "pinned host memory, overlapping the next frame's first kernels; host wall time of the "
                           "steps until the last image is on the host, less the L2 flushes between frames",
                    "blocking": {"value": e2e_block,
                                 "how": "svo_read_bgrx after every frame (the frame and its copy serialised)"}},
            "gpu_launches": int(launches),
            "clocks": clock_info,
            "roofline": roofline,
            "roofline_net": roofline_net,
            "roofline_stages": stage_rooflines,
            "l2_peak_gbs": l2_peak,
            "l2_peak_source": "the library's read probe (svo_measure_read_bandwidth) over a 48 MiB L2-resident "
                              "buffer, 40 passes, best of 3, CUDA events",
            "cpu_baseline": cpu,
            "like_for_like": like,
            "full_raycast": {"frames_per_s": full_fps, "mrays_per_s": mrays_full,
                             "ms_per_frame": statistics.mean(full_ms)},
            "speedup_vs_full": value / world / full_fps,
            "boundary_rays": boundary,
            "learned": q_learned,
            "learned_unguided": unguided,
            "plain_warped": {"frames_per_s": plain_fps, "ms_per_frame": statistics.mean(plain_ms),
                             "speedup_vs_full": plain_fps / full_fps, **q_plain},
            "fast_motion": {"workload": "2 deg/frame yaw + 0.05 extent/frame translation",
                            "learned_frames_per_s": 1000.0 / statistics.mean(fast_ms),
                            "speedup_vs_full": 1000.0 / statistics.mean(fast_ms) / full_fps,
                            "learned": q_fast, "gate_38db": fast_gate,
                            "plain": q_fast_plain, "learned_at_38db": fast_38},
            "stage_ms": stage_ms_learned,
            "stage_ms_plain": stage_ms,
            "multiview": multiview,
            "autotune": {"chosen": tuned, "default_8x4_ms": next((r["ms"] for r in tune if r["packet_w"] == 8 and
                                                                 r["stage_nodes"] == 1 and r["block"] == 256), None),
                         "candidates": len(tune), "applies_to": "full raycasts (warp frames keep the options)"}
            if tune else None,
            "autotune_learned": {"chosen": tuned_l, "ms_per_frame": {f'{r["packet_w"]}x{r["packet_h"]}/{r["block"]}':
                                                                    round(r["ms"], 4) for r in tune_l}}
                                if tune_l else None,
            "parity_plain_vs_oracle": parity,
            "octree_build_s": t_build,
            **extras,
        }
        print(json.dumps(line, default=_json_default), flush=True)
    for t in (tgt_l, full):
        t.close()
    net.close()
    ctx.close()


def main(argv=None):
    args = parse_args(argv)
    if args.profile_case:
        run_profile_case(args.profile_case)
        return
    rank, world, local_rank = dist_env()
    if world > 1:
        import torch
        import torch.distributed as dist

        backend = "nccl" if args.impl == "ours" else "gloo"
        if backend == "nccl":
            torch.cuda.set_device(local_rank)
        dist.init_process_group(backend=backend)
    try:
        if args.impl == "reference":
            run_reference(args, rank, world)
        else:
            run_ours(args, rank, world, local_rank)
    finally:
        if world > 1:
            import torch.distributed as dist

            dist.destroy_process_group()


if __name__ == "__main__":
    main()
