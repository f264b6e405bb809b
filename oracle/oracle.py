"""ctypes bindings of the CPU oracle (libsvo_oracle.so) and, where it was
built, of the reference's own kernel.cl/octree.h compiled for the host
(_ref/libsvo_ref.so).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and the
CPU-baseline leg of bench.py, and only as the checker (or the timed CPU
baseline), never as part of the product path.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE_LIB = os.path.join(HERE, "libsvo_oracle.so")
REF_LIB = os.path.join(HERE, "_ref", "libsvo_ref.so")

_P = ctypes.c_void_p
_orc = None
_ref = None


def _ptr(a):
    return a.ctypes.data_as(_P)


def reference_dir() -> str | None:
    """The reference source tree: SVO_REFERENCE_DIR, else a checkout named
    `reference` beside this repository; None when neither exists."""
    cand = os.environ.get("SVO_REFERENCE_DIR") or os.path.join(os.path.dirname(os.path.dirname(HERE)), "reference")
    return cand if os.path.isfile(os.path.join(cand, "kernel", "kernel.cl")) else None


def build(force: bool = False) -> None:
    """Compiles the oracle restatement (always possible) and, when the
    reference tree is present, the reference's own sources (_ref)."""
    src = os.path.join(HERE, "svo_oracle.cpp")
    if force or not os.path.exists(ORACLE_LIB) or os.path.getmtime(ORACLE_LIB) < os.path.getmtime(src):
        subprocess.run(["bash", os.path.join(HERE, "build_oracle.sh")], check=True, capture_output=True)
    ref_inputs = [os.path.join(HERE, f) for f in ("ref_shim.h", "ref_driver.inc", "ref_capi.inc", "build_ref.sh")]
    if force or not os.path.exists(REF_LIB) or os.path.getmtime(REF_LIB) < max(os.path.getmtime(f) for f in ref_inputs):
        ref = reference_dir()
        if ref:
            subprocess.run(["bash", os.path.join(HERE, "build_ref.sh"), ref], check=True, capture_output=True)


def oracle() -> ctypes.CDLL:
    global _orc
    if _orc is None:
        if not os.path.exists(ORACLE_LIB):
            build()
        lib = ctypes.CDLL(ORACLE_LIB)
        sz, u32, i = ctypes.c_size_t, ctypes.c_uint32, ctypes.c_int
        lib.orc_octree_build.argtypes = [i, _P, _P, _P, _P, sz, sz, ctypes.POINTER(_P)]
        lib.orc_octree_size.restype = sz
        lib.orc_octree_size.argtypes = [_P]
        lib.orc_octree_root.restype = u32
        lib.orc_octree_root.argtypes = [_P]
        lib.orc_octree_copy.argtypes = [_P, _P]
        lib.orc_octree_free.argtypes = [_P]
        lib.orc_raycast_full.argtypes = [i, _P, sz, u32, _P, _P, i, i, ctypes.c_float, ctypes.c_float, _P, _P, _P,
                                         _P, i]
        lib.orc_raycast_guided.argtypes = [i, _P, sz, u32, _P, _P, i, i, _P, _P, _P, _P, i]
        lib.orc_raycast_guided_steps.argtypes = [i, _P, sz, u32, _P, _P, i, i, _P, _P, i]
        lib.orc_guided_create.restype = _P
        lib.orc_guided_create.argtypes = [i, i, i]
        lib.orc_guided_free.argtypes = [_P]
        lib.orc_guided_frame.argtypes = [_P, _P, sz, u32, _P, _P, i, i]
        lib.orc_guided_set_certify.argtypes = [_P, i]
        for name in ("orc_guided_colour", "orc_guided_coords", "orc_guided_guide"):
            getattr(lib, name).restype = _P
            getattr(lib, name).argtypes = [_P]
        lib.orc_warp_create.restype = _P
        lib.orc_warp_create.argtypes = [i, i]
        lib.orc_warp_free.argtypes = [_P]
        lib.orc_warp_frame.argtypes = [_P, i, _P, sz, u32, _P, _P, i, i, i]
        for name in ("screen", "ids", "tex", "prefill"):
            f = getattr(lib, "orc_warp_" + name)
            f.restype = ctypes.POINTER(ctypes.c_uint32)
            f.argtypes = [_P]
        lib.orc_warp_back.restype = ctypes.POINTER(ctypes.c_float)
        lib.orc_warp_back.argtypes = [_P]
        lib.orc_warp_hole_count.argtypes = [_P]
        lib.orc_warp_stats.argtypes = [_P, _P]
        lib.orc_colorize.argtypes = [_P, _P, sz]
        lib.orc_log2_kat.restype = u32
        lib.orc_log2_kat.argtypes = [u32]
        lib.orc_max_threads.restype = i
        lib.orc_max_threads.argtypes = []
        _orc = lib
    return _orc


def ref_available() -> bool:
    return os.path.exists(REF_LIB)


def reference() -> ctypes.CDLL:
    global _ref
    if _ref is None:
        lib = ctypes.CDLL(REF_LIB)
        sz, u32, i = ctypes.c_size_t, ctypes.c_uint32, ctypes.c_int
        lib.ref_octree_build.argtypes = [i, _P, _P, _P, _P, sz, sz, ctypes.POINTER(_P)]
        lib.ref_octree_size.restype = sz
        lib.ref_octree_size.argtypes = [_P]
        lib.ref_octree_root.restype = u32
        lib.ref_octree_root.argtypes = [_P]
        lib.ref_octree_copy.argtypes = [_P, _P]
        lib.ref_octree_free.argtypes = [_P]
        lib.ref_raycast_full.argtypes = [i, _P, sz, u32, _P, _P, i, i, ctypes.c_float, ctypes.c_float, _P, _P]
        lib.ref_warp_create.restype = _P
        lib.ref_warp_create.argtypes = [i, i, i]
        lib.ref_warp_free.argtypes = [_P]
        lib.ref_warp_frame.argtypes = [_P, _P, sz, u32, _P, _P, i, i]
        for name in ("screen", "ids", "tex", "prefill"):
            f = getattr(lib, "ref_warp_" + name)
            f.restype = ctypes.POINTER(ctypes.c_uint32)
            f.argtypes = [_P]
        lib.ref_warp_back.restype = ctypes.POINTER(ctypes.c_float)
        lib.ref_warp_back.argtypes = [_P]
        lib.ref_warp_hole_count.argtypes = [_P]
        _ref = lib
    return _ref


def build_octree(depth, x, y, z, rgba, initial_words: int = 2097152, which: str = "oracle"):
    """Compact octree words and root word from voxels in insertion order."""
    lib = oracle() if which == "oracle" else reference()
    pre = "orc" if which == "oracle" else "ref"
    arrs = [np.ascontiguousarray(a, np.uint32) for a in (x, y, z, rgba)]
    h = _P()
    rc = getattr(lib, pre + "_octree_build")(depth, *[_ptr(a) for a in arrs], arrs[0].size, initial_words,
                                              ctypes.byref(h))
    if rc != 0:
        raise RuntimeError(f"{pre}_octree_build failed: {rc}")
    n = getattr(lib, pre + "_octree_size")(h)
    w = np.empty(n, np.uint32)
    getattr(lib, pre + "_octree_copy")(h, _ptr(w))
    root = getattr(lib, pre + "_octree_root")(h)
    getattr(lib, pre + "_octree_free")(h)
    return w, int(root)


def raycast_full(depth, words, root, pos, m, res_x, res_y, fovx=1.0, fovy=1.0, threads=0, which="oracle"):
    """raycast_fine_2 over the whole frame. Returns colour words, float4 per
    pixel (xyz hit, distance; the reference path leaves w at 0), packed hit
    voxels (oracle only) and [rays, child fetches, colour fetches, boundary rays,
    loop iterations, longest walk, hit-boundary rays]."""
    words = np.ascontiguousarray(words, np.uint32)
    pos = np.ascontiguousarray(pos, np.float32)
    m = np.ascontiguousarray(m, np.float32)
    n = res_x * res_y
    col = np.empty(n, np.uint32)
    xyzw = np.zeros(n * 4, np.float32)
    if which == "oracle":
        vox = np.empty(n, np.uint64)
        st = np.zeros(7, np.uint64)
        rc = oracle().orc_raycast_full(depth, _ptr(words), words.size, root, _ptr(pos), _ptr(m), res_x, res_y, fovx,
                                       fovy, _ptr(col), _ptr(xyzw), _ptr(vox), _ptr(st), threads)
        if rc != 0:
            raise RuntimeError(f"orc_raycast_full failed: {rc}")
        return col, xyzw.reshape(n, 4), vox, st
    rc = reference().ref_raycast_full(depth, _ptr(words), words.size, root, _ptr(pos), _ptr(m), res_x, res_y, fovx,
                                      fovy, _ptr(col), _ptr(xyzw))
    if rc != 0:
        raise RuntimeError(f"ref_raycast_full failed: {rc}")
    return col, xyzw.reshape(n, 4), None, None


def raycast_guided(depth, words, root, pos, m, res_x, res_y, s0, threads=0, stats=False):
    """Guided walks (the product's learned frames): pixel o's ray starts at
    s0[o] raypos units (0: from the camera; < 0: not traced, colour left at
    the empty word and xyzw at 0). Returns colour words and float4 per pixel
    (and, with stats, [rays walked, child fetches, colour fetches])."""
    words = np.ascontiguousarray(words, np.uint32)
    pos = np.ascontiguousarray(pos, np.float32)
    m = np.ascontiguousarray(m, np.float32)
    s0 = np.ascontiguousarray(s0, np.float32)
    n = res_x * res_y
    assert s0.size == n
    col = np.full(n, 0xFFFFFF00, np.uint32)
    xyzw = np.zeros(n * 4, np.float32)
    st = np.zeros(3, np.uint64)
    rc = oracle().orc_raycast_guided(depth, _ptr(words), words.size, root, _ptr(pos), _ptr(m), res_x, res_y, _ptr(s0),
                                     _ptr(col), _ptr(xyzw), _ptr(st), threads)
    if rc != 0:
        raise RuntimeError(f"orc_raycast_guided failed: {rc}")
    if stats:
        return col, xyzw.reshape(n, 4), st
    return col, xyzw.reshape(n, 4)


def raycast_guided_steps(depth, words, root, pos, m, res_x, res_y, s0, threads=0):
    """Loop iterations of each pixel's guided walk (0 where s0 < 0)."""
    words = np.ascontiguousarray(words, np.uint32)
    s0 = np.ascontiguousarray(s0, np.float32)
    steps = np.zeros(res_x * res_y, np.uint32)
    rc = oracle().orc_raycast_guided_steps(depth, _ptr(words), words.size, root,
                                           _ptr(np.ascontiguousarray(pos, np.float32)),
                                           _ptr(np.ascontiguousarray(m, np.float32)), res_x, res_y, _ptr(s0),
                                           _ptr(steps), threads)
    if rc != 0:
        raise RuntimeError(f"orc_raycast_guided_steps failed: {rc}")
    return steps


class Guided:
    """Guided learned frames with every unguided pixel traced (the product's
    learned frames on a guided target with a threshold no confidence reaches):
    reprojection of the last frame's plane re-based by whole periods, start
    distances, rays from the camera and walks. Test infrastructure only."""

    def __init__(self, depth: int, res_x: int, res_y: int, certify: bool = False):
        self.n = res_x * res_y
        self._lib = oracle()
        self._h = self._lib.orc_guided_create(depth, res_x, res_y)
        if not self._h:
            raise ValueError("guided frames: resolution must be at least 16x16")
        self._lib.orc_guided_set_certify(self._h, 1 if certify else 0)

    def frame(self, words, root, pos, m, frame: int, threads: int = 0) -> None:
        words = np.ascontiguousarray(words, np.uint32)
        pos = np.ascontiguousarray(pos, np.float32)
        m = np.ascontiguousarray(m, np.float32)
        rc = self._lib.orc_guided_frame(self._h, _ptr(words), words.size, root, _ptr(pos), _ptr(m), frame, threads)
        if rc != 0:
            raise RuntimeError(f"orc_guided_frame failed: {rc}")

    def colour(self) -> np.ndarray:
        return np.ctypeslib.as_array(ctypes.cast(self._lib.orc_guided_colour(self._h), ctypes.POINTER(ctypes.c_uint32)),
                                     (self.n,)).copy()

    def coords(self) -> np.ndarray:
        return np.ctypeslib.as_array(ctypes.cast(self._lib.orc_guided_coords(self._h), ctypes.POINTER(ctypes.c_float)),
                                     (self.n * 4,)).copy().reshape(self.n, 4)

    def guide(self) -> np.ndarray:
        return np.ctypeslib.as_array(ctypes.cast(self._lib.orc_guided_guide(self._h), ctypes.POINTER(ctypes.c_float)),
                                     (self.n,)).copy()

    def __del__(self):
        if getattr(self, "_h", None):
            self._lib.orc_guided_free(self._h)
            self._h = None


class Warp:
    """Frame state of raycast_draw (4 colour planes, 4 float4 planes, hole
    buffer, BGRX) on the CPU: the oracle restatement or the reference itself."""

    def __init__(self, depth: int, res_x: int, res_y: int, which: str = "oracle"):
        self.which = which
        self.depth, self.res_x, self.res_y = depth, res_x, res_y
        self.n = res_x * res_y
        self.tiles = (res_x // 16) * (res_y // 16)
        if which == "oracle":
            self._lib, self._pre = oracle(), "orc"
            self._h = self._lib.orc_warp_create(res_x, res_y)
        else:
            self._lib, self._pre = reference(), "ref"
            self._h = self._lib.ref_warp_create(depth, res_x, res_y)
        if not self._h:
            raise ValueError("warp state: resolution must be at least 16x16")

    def frame(self, words, root, pos, m, frame: int, threads: int = 0, cache_mode: int = 0,
              coarse: bool = False) -> None:
        """cache_mode 1: alternating copy target; coarse: the raycast_fine pass."""
        cache_mode = (cache_mode & 1) | (2 if coarse else 0)
        words = np.ascontiguousarray(words, np.uint32)
        pos = np.ascontiguousarray(pos, np.float32)
        m = np.ascontiguousarray(m, np.float32)
        if self.which == "oracle":
            rc = self._lib.orc_warp_frame(self._h, self.depth, _ptr(words), words.size, root, _ptr(pos), _ptr(m),
                                          frame, threads, cache_mode)
        else:
            rc = self._lib.ref_warp_frame(self._h, _ptr(words), words.size, root, _ptr(pos), _ptr(m), frame,
                                          cache_mode)
        if rc != 0:
            raise RuntimeError(f"{self._pre}_warp_frame failed: {rc}")

    def _u32(self, name, n):
        return np.ctypeslib.as_array(getattr(self._lib, f"{self._pre}_warp_{name}")(self._h), (n,)).copy()

    def screen(self) -> np.ndarray:
        """4 colour planes, shape (4, n)."""
        return self._u32("screen", 4 * self.n).reshape(4, self.n)

    def back(self) -> np.ndarray:
        """4 float4 planes, shape (4, n, 4)."""
        p = getattr(self._lib, f"{self._pre}_warp_back")(self._h)
        return np.ctypeslib.as_array(p, (16 * self.n,)).copy().reshape(4, self.n, 4)

    def hole_count(self) -> int:
        return int(getattr(self._lib, f"{self._pre}_warp_hole_count")(self._h))

    def ids(self) -> np.ndarray:
        """The hole id buffer up to the last entry (2*tiles + count words)."""
        return self._u32("ids", self.n + 2 * self.tiles)[: 2 * self.tiles + self.hole_count()]

    def tex(self) -> np.ndarray:
        return self._u32("tex", self.n)

    def prefill(self) -> np.ndarray:
        return self._u32("prefill", self.n)

    def stats(self) -> np.ndarray:
        out = np.zeros(4, np.uint64)
        if self.which == "oracle":
            self._lib.orc_warp_stats(self._h, _ptr(out))
        return out

    def __del__(self):
        if getattr(self, "_h", None):
            getattr(self._lib, f"{self._pre}_warp_free")(self._h)
            self._h = None


def colorize(words: np.ndarray) -> np.ndarray:
    words = np.ascontiguousarray(words, np.uint32)
    out = np.empty_like(words)
    oracle().orc_colorize(_ptr(words), _ptr(out), words.size)
    return out


def log2_kat(limit: int) -> int:
    return int(oracle().orc_log2_kat(limit))


def max_threads() -> int:
    return int(oracle().orc_max_threads())
