"""Generates tests/golden/golden.npz from the reference itself.

The outputs are produced by the reference's own kernel/kernel.cl and
src/octree/octree.h compiled for the host (oracle/_ref/libsvo_ref.so, built by
oracle/build_ref.sh from the read-only reference tree). Inputs are the seeded
synthetic terrain and camera paths of libsvo_gb300.so; their hashes are stored
so a change of the input generator is reported as such.

Stored per case: SHA-256 digests of the compact octree words, full-raycast
colour words and hit positions, and of every warp frame's planes, hole list
and BGRX image; small cases also keep the raw arrays. Cameras are stored as
float32 bit patterns.

usage: python tests/golden/make_golden.py
"""
from __future__ import annotations

import hashlib
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "sparse-voxel-octree-raycasting_gb300"))
sys.path.insert(0, os.path.join(ROOT, "oracle"))

import oracle  # noqa: E402
import svo_gb300 as svo  # noqa: E402


def digest(*arrays) -> str:
    h = hashlib.sha256()
    for a in arrays:
        h.update(np.ascontiguousarray(a).tobytes())
    return h.hexdigest()


BUILDER_CASES = [
    # depth, seed, shell
    (8, 5, True),
    (8, 6, False),
    (9, 7, True),
]
FULL_CASES = [
    # depth, seed, shell, camera kind, frame, W, H, fov
    (8, 5, True, 0, 0, 64, 48, 1.1547),
    (8, 5, True, 3, 2, 64, 48, 1.0),
    (9, 7, True, 1, 9, 96, 64, 1.0),
    (8, 6, False, 0, 0, 80, 60, 1.1547),
]
WARP_CASES = [
    # depth, seed, shell, camera kind, frames, W, H
    (8, 5, True, 1, 10, 64, 48),
    (9, 7, True, 2, 6, 80, 56),
]
# The benchmark's own size and depths (digests only): the depth-11 terrain of
# the 1920x1024 benchmark, and depth 12 (4096^3), whose terrain needs more
# pointer nodes than the reference builder allows (octree.h:78), so its words
# come from the product builder (their digest is stored) and only the
# raycast and warp frames are the reference's.
FULLSIZE_CASES = [
    # depth, seed, shell, full-raycast frame, warp frames, W, H
    (11, 2024, True, 40, 4, 1920, 1024),
    (12, 2024, True, 40, 4, 1920, 1024),
]


def main() -> None:
    oracle.build()
    if not oracle.ref_available():
        sys.exit("the reference library is not built (is the reference tree present?)")
    out: dict[str, np.ndarray] = {}
    meta: dict = {"builder": [], "full": [], "warp": []}
    scenes = {}
    for depth, seed, shell in BUILDER_CASES:
        x, y, z, c = svo.terrain_voxels(seed, depth, shell)
        words, root = oracle.build_octree(depth, x, y, z, c, which="reference")
        scenes[(depth, seed, shell)] = (words, root)
        meta["builder"].append({"depth": depth, "seed": seed, "shell": shell, "voxels": int(x.size),
                                "voxel_digest": digest(x, y, z, c), "n_words": int(words.size), "root": root,
                                "words_digest": digest(words)})
    for i, (depth, seed, shell, kind, frame, W, H, fov) in enumerate(FULL_CASES):
        words, root = scenes[(depth, seed, shell)]
        v = svo.camera_path(kind, depth, frame, W, H, fov=fov)
        col, xyzw, _, _ = oracle.raycast_full(depth, words, root, v.pos_array, v.m_array, W, H, fov, fov,
                                              which="reference")
        xyz = np.ascontiguousarray(xyzw[:, :3])
        key = f"full{i}"
        out[key + "_pos"] = v.pos_array
        out[key + "_m"] = v.m_array
        out[key + "_colour"] = col
        out[key + "_xyz"] = xyz
        meta["full"].append({"key": key, "depth": depth, "seed": seed, "shell": shell, "kind": kind, "frame": frame,
                             "W": W, "H": H, "fov": fov, "colour_digest": digest(col), "xyz_digest": digest(xyz)})
    for i, (depth, seed, shell, kind, frames, W, H) in enumerate(WARP_CASES):
        words, root = scenes[(depth, seed, shell)]
        w = oracle.Warp(depth, W, H, which="reference")
        key = f"warp{i}"
        per_frame = []
        for f in range(frames):
            v = svo.camera_path(kind, depth, f, W, H)
            out[f"{key}_f{f}_pos"] = v.pos_array
            out[f"{key}_f{f}_m"] = v.m_array
            w.frame(words, root, v.pos_array, v.m_array, f)
            screen = w.screen()
            back = w.back()
            ne = screen[2] != svo.EMPTY_PIXEL
            per_frame.append({
                "holes": w.hole_count(),
                "ids_digest": digest(w.ids()),
                "plane0_digest": digest(screen[0]),
                "plane2_digest": digest(screen[2]),
                "xyz2_digest": digest(np.ascontiguousarray(back[2][ne][:, :3])),
                "tex_digest": digest(w.tex()),
            })
        out[key + "_last_plane0"] = w.screen()[0]
        out[key + "_last_tex"] = w.tex()
        meta["warp"].append({"key": key, "depth": depth, "seed": seed, "shell": shell, "kind": kind,
                             "frames": frames, "W": W, "H": H, "per_frame": per_frame})
    meta["fullsize"] = []
    for depth, seed, shell, frame, frames, W, H in FULLSIZE_CASES:
        x, y, z, c = svo.terrain_voxels(seed, depth, shell)
        if depth <= 11:
            words, root = oracle.build_octree(depth, x, y, z, c, which="reference")
            builder = "reference"
        else:
            o = svo.build_terrain(depth, seed, shell)
            words, root = o.words, o.root
            builder = "product"
        case = {"depth": depth, "seed": seed, "shell": shell, "W": W, "H": H, "voxel_digest": digest(x, y, z, c),
                "builder": builder, "n_words": int(words.size), "root": int(root), "words_digest": digest(words),
                "frame": frame}
        del x, y, z, c
        v = svo.camera_path(1, depth, frame, W, H)
        col, xyzw, _, _ = oracle.raycast_full(depth, words, root, v.pos_array, v.m_array, W, H, 1.0, 1.0,
                                              which="reference")
        case["camera_digest"] = digest(v.pos_array, v.m_array)
        case["colour_digest"] = digest(col)
        case["xyz_digest"] = digest(np.ascontiguousarray(xyzw[:, :3]))
        w = oracle.Warp(depth, W, H, which="reference")
        per_frame = []
        for f in range(frames):
            v = svo.camera_path(1, depth, f, W, H)
            w.frame(words, root, v.pos_array, v.m_array, f)
            screen = w.screen()
            per_frame.append({"camera_digest": digest(v.pos_array, v.m_array), "holes": w.hole_count(),
                              "ids_digest": digest(w.ids()), "plane0_digest": digest(screen[0]),
                              "plane2_digest": digest(screen[2]), "tex_digest": digest(w.tex())})
        case["warp"] = per_frame
        meta["fullsize"].append(case)
        print("fullsize case", depth, "done", flush=True)
    np.savez_compressed(os.path.join(HERE, "golden.npz"), **out)
    with open(os.path.join(HERE, "golden.json"), "w") as f:
        json.dump(meta, f, indent=1)
    print("wrote", os.path.join(HERE, "golden.npz"), "and golden.json")


if __name__ == "__main__":
    main()
