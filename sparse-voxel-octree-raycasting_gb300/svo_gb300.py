"""Python bindings (ctypes) of libsvo_gb300.so.

The library's C ABI (include/svo_gb300.h) replaces the reference's OpenCL
wrapper src/ocl.h and the buffer plumbing of src/raycast.h. This module is a
thin host-side mirror for Python callers, tests and the benchmark: every call
goes straight to the C ABI, and a failing call raises SvoError carrying the
library's status and message. There is no CPU fallback: without the built
library (or without a GPU for the device calls) the calls fail loudly.
"""
from __future__ import annotations

import atexit
import ctypes
import os
import weakref
from typing import Sequence

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libsvo_gb300.so")

EMPTY_PIXEL = 0xFFFFFF00
OPT_STAGE_NODES = 1
OPT_PACKET_WIDTH = 2
OPT_TRACE_BLOCK = 3
OPT_LEARNED_TRACE_BLOCK = 4
OPT_LEARNED_PACKET_WIDTH = 5
NOALLOC_MAX_VIEWS = 64
DEFAULT_INITIAL_WORDS = 2097152
STATUS = {
    0: "SVO_OK", 1: "SVO_ERR_INVALID_ARGUMENT", 2: "SVO_ERR_CUDA", 3: "SVO_ERR_NO_OCTREE",
    4: "SVO_ERR_BAD_OCTREE", 5: "SVO_ERR_DEVICE_FAULT", 6: "SVO_ERR_OUT_OF_MEMORY",
    7: "SVO_ERR_CAPACITY", 8: "SVO_ERR_NOT_SUPPORTED", 9: "SVO_ERR_IO",
}

# Every symbol include/svo_gb300.h declares.
EXPORTS = [
    "svo_context_create", "svo_context_destroy", "svo_last_error", "svo_context_stream", "svo_synchronize",
    "svo_launch_count", "svo_context_set_option", "svo_octree_upload", "svo_octree_upload_device", "svo_octree_set_l2_window",
    "svo_target_create", "svo_target_destroy", "svo_raycast_full", "svo_raycast_full_batch", "svo_warp_frame",
    "svo_target_use_graph", "svo_target_set_profiling", "svo_target_stage_times", "svo_read_colour",
    "svo_read_coords", "svo_read_holes", "svo_read_bgrx", "svo_read_bgrx_async", "svo_target_readback_wait",
    "svo_read_full", "svo_read_voxels",
    "svo_target_device_outputs", "svo_builder_create", "svo_builder_destroy", "svo_builder_set_voxel",
    "svo_builder_set_voxels", "svo_builder_finish", "svo_builder_copy_words", "svo_builder_stats",
    "svo_octree_save", "svo_octree_load_header", "svo_octree_load_words", "svo_terrain_build",
    "svo_terrain_voxels", "svo_view_from_euler", "svo_view_look_at", "svo_wrap_position", "svo_camera_path",
    "svo_raycast_full_noalloc", "svo_rle4_voxels", "svo_rle4_build", "svo_write_bmp",
    "svo_warp_frame_learned", "svo_read_requested", "svo_target_set_feature_tap", "svo_net_create",
    "svo_net_destroy", "svo_net_init", "svo_net_set_params", "svo_net_get_params", "svo_net_get_grads",
    "svo_net_forward", "svo_net_infer", "svo_net_backward", "svo_net_adam", "svo_target_set_cache_mode",
    "svo_target_set_coarse_refresh", "svo_octree_build", "svo_octree_info", "svo_octree_download",
    "svo_context_autotune", "svo_target_set_guided", "svo_read_guide", "svo_context_autotune_learned",
    "svo_measure_read_bandwidth", "svo_target_set_certified",
]

NET_PARAMS = 6388


class SvoError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__(f"{STATUS.get(status, status)}: {message}")
        self.status = status


class View(ctypes.Structure):
    """svo_view: camera position (world units), row-major view matrix m, fov, resolution."""
    _fields_ = [("pos", ctypes.c_float * 4), ("m", ctypes.c_float * 16), ("fovx", ctypes.c_float),
                ("fovy", ctypes.c_float), ("res_x", ctypes.c_int32), ("res_y", ctypes.c_int32)]

    @property
    def pos_array(self) -> np.ndarray:
        return np.array(self.pos[:], np.float32)

    @property
    def m_array(self) -> np.ndarray:
        return np.array(self.m[:], np.float32)


class TerrainSpec(ctypes.Structure):
    _fields_ = [("seed", ctypes.c_uint32), ("depth", ctypes.c_int32), ("shell", ctypes.c_int32),
                ("boxes", ctypes.c_int32)]


class FrameBuffers(ctypes.Structure):
    """svo_frame_buffers: device output buffers of one view of svo_raycast_full_noalloc."""
    _fields_ = [("colour", ctypes.c_void_p), ("xyzw", ctypes.c_void_p), ("voxel", ctypes.c_void_p),
                ("bgrx", ctypes.c_void_p)]


class TuneResult(ctypes.Structure):
    _fields_ = [("packet_w", ctypes.c_int), ("packet_h", ctypes.c_int), ("block", ctypes.c_int),
                ("stage_nodes", ctypes.c_int), ("ms", ctypes.c_float)]


class DeviceOutputs(ctypes.Structure):
    _fields_ = [("bgrx", ctypes.c_void_p), ("colour", ctypes.c_void_p), ("full_colour", ctypes.c_void_p),
                ("full_xyzw", ctypes.c_void_p), ("full_voxel", ctypes.c_void_p)]


_P = ctypes.c_void_p
_lib = None


def _ptr(a: np.ndarray) -> ctypes.c_void_p:
    return a.ctypes.data_as(_P)


def load(path: str | None = None) -> ctypes.CDLL:
    """Loads the library (building it first when it is missing)."""
    global _lib
    if _lib is not None:
        return _lib
    path = path or LIB_PATH
    if not os.path.exists(path):
        import importlib.util
        spec = importlib.util.spec_from_file_location("svo_gb300_build", os.path.join(HERE, "build.py"))
        mod = importlib.util.module_from_spec(spec)
        spec.loader.exec_module(mod)
        mod.build()
    lib = ctypes.CDLL(path)
    i, u32, sz = ctypes.c_int, ctypes.c_uint32, ctypes.c_size_t
    sigs = {
        "svo_context_create": (i, [i, ctypes.POINTER(_P)]),
        "svo_context_destroy": (i, [_P]),
        "svo_last_error": (ctypes.c_char_p, [_P]),
        "svo_context_stream": (_P, [_P]),
        "svo_target_set_certified": (i, [_P, i]),
        "svo_synchronize": (i, [_P]),
        "svo_measure_read_bandwidth": (i, [_P, _P, ctypes.c_size_t, i, ctypes.POINTER(ctypes.c_double)]),
        "svo_launch_count": (ctypes.c_uint64, [_P]),
        "svo_context_set_option": (i, [_P, i, ctypes.c_int64]),
        "svo_octree_upload": (i, [_P, _P, sz, u32, i, i]),
        "svo_octree_upload_device": (i, [_P, _P, sz, u32, i]),
        "svo_octree_set_l2_window": (i, [_P, sz]),
        "svo_target_create": (i, [_P, i, i, ctypes.POINTER(_P)]),
        "svo_target_destroy": (i, [_P]),
        "svo_raycast_full": (i, [_P, _P, ctypes.POINTER(View)]),
        "svo_raycast_full_batch": (i, [_P, _P, _P, i]),
        "svo_warp_frame": (i, [_P, _P, ctypes.POINTER(View), i]),
        "svo_target_use_graph": (i, [_P, i]),
        "svo_target_set_profiling": (i, [_P, i]),
        "svo_target_stage_times": (i, [_P, _P, i]),
        "svo_read_colour": (i, [_P, i, _P]),
        "svo_read_coords": (i, [_P, i, _P]),
        "svo_read_holes": (i, [_P, _P, sz, ctypes.POINTER(u32)]),
        "svo_read_bgrx": (i, [_P, _P]),
        "svo_read_bgrx_async": (i, [_P, _P]),
        "svo_target_readback_wait": (i, [_P]),
        "svo_read_full": (i, [_P, _P, _P]),
        "svo_read_voxels": (i, [_P, _P]),
        "svo_target_device_outputs": (i, [_P, ctypes.POINTER(DeviceOutputs)]),
        "svo_builder_create": (i, [i, ctypes.POINTER(_P)]),
        "svo_builder_destroy": (i, [_P]),
        "svo_builder_set_voxel": (i, [_P, u32, u32, u32, u32]),
        "svo_builder_set_voxels": (i, [_P, _P, _P, _P, _P, sz]),
        "svo_builder_finish": (i, [_P, sz, ctypes.POINTER(u32), ctypes.POINTER(sz)]),
        "svo_builder_copy_words": (i, [_P, _P]),
        "svo_builder_stats": (i, [_P, ctypes.POINTER(ctypes.c_uint64), ctypes.POINTER(ctypes.c_uint64)]),
        "svo_octree_save": (i, [ctypes.c_char_p, _P, sz, u32, i]),
        "svo_octree_load_header": (i, [ctypes.c_char_p, ctypes.POINTER(sz), ctypes.POINTER(u32),
                                       ctypes.POINTER(i)]),
        "svo_octree_load_words": (i, [ctypes.c_char_p, _P, sz]),
        "svo_terrain_build": (i, [_P, ctypes.POINTER(TerrainSpec)]),
        "svo_terrain_voxels": (i, [ctypes.POINTER(TerrainSpec), _P, _P, _P, _P, sz, ctypes.POINTER(sz)]),
        "svo_view_from_euler": (i, [ctypes.c_float, ctypes.c_float, ctypes.c_float, _P, i, i, ctypes.c_float,
                                    ctypes.POINTER(View)]),
        "svo_view_look_at": (i, [_P, _P, i, i, ctypes.c_float, ctypes.POINTER(View)]),
        "svo_wrap_position": (i, [_P, i]),
        "svo_camera_path": (i, [i, i, i, u32, i, i, ctypes.c_float, ctypes.POINTER(View)]),
        "svo_raycast_full_noalloc": (i, [_P, sz, u32, i, _P, _P, i, _P]),
        "svo_rle4_voxels": (i, [ctypes.c_char_p, i, u32, u32, u32, _P, _P, _P, _P, sz, ctypes.POINTER(sz)]),
        "svo_rle4_build": (i, [_P, ctypes.c_char_p, i, u32, u32, u32]),
        "svo_write_bmp": (i, [ctypes.c_char_p, _P, i, i]),
        "svo_warp_frame_learned": (i, [_P, _P, ctypes.POINTER(View), i, _P, ctypes.c_float]),
        "svo_read_requested": (i, [_P, ctypes.POINTER(u32)]),
        "svo_target_set_feature_tap": (i, [_P, _P]),
        "svo_target_set_cache_mode": (i, [_P, i]),
        "svo_target_set_coarse_refresh": (i, [_P, i]),
        "svo_target_set_guided": (i, [_P, i]),
        "svo_context_autotune_learned": (i, [_P, _P, _P, i, _P, ctypes.c_float, _P, i, ctypes.POINTER(i)]),
        "svo_read_guide": (i, [_P, _P]),
        "svo_octree_build": (i, [_P, _P, _P, _P, _P, sz, i, sz]),
        "svo_octree_info": (i, [_P, ctypes.POINTER(sz), ctypes.POINTER(u32), ctypes.POINTER(i)]),
        "svo_octree_download": (i, [_P, _P, sz]),
        "svo_context_autotune": (i, [_P, _P, ctypes.POINTER(View), i, _P, i, ctypes.POINTER(i)]),
        "svo_net_create": (i, [_P, ctypes.POINTER(_P)]),
        "svo_net_destroy": (i, [_P]),
        "svo_net_init": (i, [_P, ctypes.c_uint64]),
        "svo_net_set_params": (i, [_P, _P, sz]),
        "svo_net_get_params": (i, [_P, _P, sz]),
        "svo_net_get_grads": (i, [_P, _P, sz]),
        "svo_net_forward": (i, [_P, _P, i, i, _P]),
        "svo_net_infer": (i, [_P, _P, i, i, _P]),
        "svo_net_backward": (i, [_P, _P, _P, i, i, ctypes.c_float, ctypes.c_float, _P]),
        "svo_net_adam": (i, [_P, ctypes.c_float, ctypes.c_float, ctypes.c_float, ctypes.c_float]),
    }
    for name, (res, args) in sigs.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def _check(rc: int, ctx=None, what: str = "") -> None:
    if rc != 0:
        msg = what
        if ctx is not None and ctx._h:
            msg = load().svo_last_error(ctx._h).decode(errors="replace") or what
        raise SvoError(rc, msg)


# ----------------------------------------------------------------- scenes --
def terrain_voxels(seed: int, depth: int, shell: bool, boxes: int = 0):
    """Voxels of the seeded terrain in insertion order: (x, y, z, rgba) uint32 arrays."""
    lib = load()
    spec = TerrainSpec(seed, depth, 1 if shell else 0, boxes)
    n = ctypes.c_size_t()
    _check(lib.svo_terrain_voxels(ctypes.byref(spec), None, None, None, None, 0, ctypes.byref(n)))
    x = np.empty(n.value, np.uint32)
    y, z, c = np.empty_like(x), np.empty_like(x), np.empty_like(x)
    _check(lib.svo_terrain_voxels(ctypes.byref(spec), _ptr(x), _ptr(y), _ptr(z), _ptr(c), n.value, ctypes.byref(n)))
    return x, y, z, c


def rle4_voxels(path: str, palette: int = 0, add=(0, 0, 0)):
    """Voxels of map 0 of an .rle4 file in the reference loader's order: (x, y, z, rgba)."""
    lib = load()
    n = ctypes.c_size_t()
    _check(lib.svo_rle4_voxels(path.encode(), palette, add[0], add[1], add[2], None, None, None, None, 0,
                               ctypes.byref(n)), None, f"cannot read {path}")
    x = np.empty(n.value, np.uint32)
    y, z, c = np.empty_like(x), np.empty_like(x), np.empty_like(x)
    _check(lib.svo_rle4_voxels(path.encode(), palette, add[0], add[1], add[2], _ptr(x), _ptr(y), _ptr(z), _ptr(c),
                               n.value, ctypes.byref(n)))
    return x, y, z, c


def write_bmp(path: str, bgrx: np.ndarray, width: int, height: int) -> None:
    img = np.ascontiguousarray(bgrx, np.uint32)
    _check(load().svo_write_bmp(path.encode(), _ptr(img), width, height), None, f"cannot write {path}")


class Octree:
    """A finished compact octree: words (uint32), root word, depth."""

    def __init__(self, words: np.ndarray, root: int, depth: int, voxels: int = 0, nodes: int = 0):
        self.words = np.ascontiguousarray(words, dtype=np.uint32)
        self.root = int(root)
        self.depth = int(depth)
        self.voxels = voxels
        self.nodes = nodes

    def save(self, path: str) -> None:
        _check(load().svo_octree_save(path.encode(), _ptr(self.words), self.words.size, self.root, self.depth))

    @staticmethod
    def load_file(path: str) -> "Octree":
        lib = load()
        n, root, depth = ctypes.c_size_t(), ctypes.c_uint32(), ctypes.c_int()
        _check(lib.svo_octree_load_header(path.encode(), ctypes.byref(n), ctypes.byref(root), ctypes.byref(depth)))
        w = np.empty(n.value, np.uint32)
        _check(lib.svo_octree_load_words(path.encode(), _ptr(w), n.value))
        return Octree(w, root.value, depth.value)


class Builder:
    """set_voxel / convert_tree_blocks (src/octree/octree.h) in one object."""

    def __init__(self, depth: int):
        self._lib = load()
        self._h = _P()
        _check(self._lib.svo_builder_create(depth, ctypes.byref(self._h)))
        self.depth = depth

    def set_voxel(self, x: int, y: int, z: int, rgba: int) -> None:
        _check(self._lib.svo_builder_set_voxel(self._h, x, y, z, rgba))

    def set_voxels(self, x, y, z, rgba) -> None:
        arrs = [np.ascontiguousarray(a, dtype=np.uint32) for a in (x, y, z, rgba)]
        _check(self._lib.svo_builder_set_voxels(self._h, *[_ptr(a) for a in arrs], arrs[0].size))

    def add_rle4(self, path: str, palette: int = 0, add=(0, 0, 0)) -> None:
        _check(self._lib.svo_rle4_build(self._h, path.encode(), palette, add[0], add[1], add[2]), None,
               f"cannot load {path}")

    def add_terrain(self, seed: int, shell: bool, boxes: int = 0) -> None:
        spec = TerrainSpec(seed, self.depth, 1 if shell else 0, boxes)
        _check(self._lib.svo_terrain_build(self._h, ctypes.byref(spec)))

    def finish(self, initial_words: int = 0) -> Octree:
        root, n = ctypes.c_uint32(), ctypes.c_size_t()
        _check(self._lib.svo_builder_finish(self._h, initial_words, ctypes.byref(root), ctypes.byref(n)))
        w = np.empty(n.value, np.uint32)
        _check(self._lib.svo_builder_copy_words(self._h, _ptr(w)))
        vox, nodes = ctypes.c_uint64(), ctypes.c_uint64()
        _check(self._lib.svo_builder_stats(self._h, ctypes.byref(vox), ctypes.byref(nodes)))
        return Octree(w, root.value, self.depth, vox.value, nodes.value)

    def __del__(self):
        if getattr(self, "_h", None):
            self._lib.svo_builder_destroy(self._h)
            self._h = None


def build_terrain(depth: int, seed: int, shell: bool, boxes: int = 0) -> Octree:
    b = Builder(depth)
    b.add_terrain(seed, shell, boxes)
    return b.finish()


# ---------------------------------------------------------------- cameras --
def camera_path(kind: int, depth: int, frame: int, res_x: int, res_y: int, fov: float = 1.0, seed: int = 7) -> View:
    v = View()
    _check(load().svo_camera_path(kind, depth, frame, seed, res_x, res_y, fov, ctypes.byref(v)))
    return v


def view_from_euler(rx: float, ry: float, rz: float, pos, res_x: int, res_y: int, fov: float = 1.0) -> View:
    v = View()
    p = np.ascontiguousarray(pos, np.float32)
    _check(load().svo_view_from_euler(rx, ry, rz, _ptr(p), res_x, res_y, fov, ctypes.byref(v)))
    return v


def view_look_at(pos, target, res_x: int, res_y: int, fov: float = 1.0) -> View:
    v = View()
    p = np.ascontiguousarray(pos, np.float32)
    t = np.ascontiguousarray(target, np.float32)
    _check(load().svo_view_look_at(_ptr(p), _ptr(t), res_x, res_y, fov, ctypes.byref(v)))
    return v


# ------------------------------------------------------------ GPU runtime --
class Context:
    """One device, one stream (ocl_init / raycast_init / raycast_exit)."""

    def __init__(self, device: int = 0):
        self._lib = load()
        self._h = _P()
        self._targets: "weakref.WeakSet[Target]" = weakref.WeakSet()
        self._nets: "weakref.WeakSet[Net]" = weakref.WeakSet()
        _check(self._lib.svo_context_create(device, ctypes.byref(self._h)), None,
               f"svo_context_create(device={device}) failed")
        self.octree: Octree | None = None
        _LIVE_CONTEXTS.add(self)

    @property
    def handle(self):
        return self._h

    @property
    def stream(self) -> int:
        return int(self._lib.svo_context_stream(self._h) or 0)

    def upload(self, octree: Octree, validate: bool = True) -> None:
        _check(self._lib.svo_octree_upload(self._h, _ptr(octree.words), octree.words.size, octree.root, octree.depth,
                                           1 if validate else 0), self)
        self.octree = octree

    def upload_device(self, d_words: int, n_words: int, root: int, depth: int) -> None:
        _check(self._lib.svo_octree_upload_device(self._h, _P(d_words), n_words, root, depth), self)

    def build_octree(self, d_x: int, d_y: int, d_z: int, d_rgba: int, n: int, depth: int,
                     initial_words: int = 0) -> None:
        """Builds the octree on the GPU from device voxel arrays (uint32 each) and installs it."""
        _check(self._lib.svo_octree_build(self._h, _P(d_x), _P(d_y), _P(d_z), _P(d_rgba), n, depth, initial_words),
               self)

    def octree_info(self) -> tuple[int, int, int]:
        """(n_words, root_word, depth) of the installed octree."""
        nw, root, depth = ctypes.c_size_t(), ctypes.c_uint32(), ctypes.c_int()
        _check(self._lib.svo_octree_info(self._h, ctypes.byref(nw), ctypes.byref(root), ctypes.byref(depth)), self)
        return nw.value, root.value, depth.value

    def download_octree(self) -> Octree:
        nw, root, depth = self.octree_info()
        words = np.empty(nw, np.uint32)
        _check(self._lib.svo_octree_download(self._h, _ptr(words), nw), self)
        return Octree(words, root, depth)

    def autotune(self, target: "Target", view: View, repeats: int = 3) -> list[dict]:
        """Times every trace configuration on full raycasts of `view`, keeps the fastest;
        returns the measurements (packet_w, packet_h, block, stage_nodes, ms)."""
        res = (TuneResult * 32)()
        n = ctypes.c_int()
        _check(self._lib.svo_context_autotune(self._h, target._h, ctypes.byref(view), repeats, ctypes.cast(res, _P),
                                              32, ctypes.byref(n)), self)
        return [{"packet_w": r.packet_w, "packet_h": r.packet_h, "block": r.block, "stage_nodes": r.stage_nodes,
                 "ms": r.ms} for r in res[:n.value]]

    def autotune_learned(self, target: "Target", views: Sequence[View], net: "Net",
                         threshold: float = 0.5) -> list[dict]:
        """Times learned frames of `views` (>= 6, rendered as frames 0..n-1 with the
        target's guided setting) for every packet shape and block size of their
        tracer, keeps the fastest; returns the measurements (ms per frame)."""
        arr = (View * len(views))(*views)
        res = (TuneResult * 32)()
        n = ctypes.c_int()
        _check(self._lib.svo_context_autotune_learned(self._h, target._h, ctypes.cast(arr, _P), len(views), net._h,
                                                      threshold, ctypes.cast(res, _P), 32, ctypes.byref(n)), self)
        return [{"packet_w": r.packet_w, "packet_h": r.packet_h, "block": r.block, "stage_nodes": r.stage_nodes,
                 "ms": r.ms} for r in res[:n.value]]

    def set_option(self, option: int, value: int) -> None:
        _check(self._lib.svo_context_set_option(self._h, option, value), self)

    def set_l2_window(self, nbytes: int) -> None:
        _check(self._lib.svo_octree_set_l2_window(self._h, nbytes), self)

    def read_bandwidth(self, d_buf: int, nbytes: int, passes: int = 20) -> float:
        """GB/s of the library's read probe over a device buffer (see
        svo_measure_read_bandwidth); an L2-resident buffer gives the L2 read
        bandwidth."""
        g = ctypes.c_double()
        _check(self._lib.svo_measure_read_bandwidth(self._h, _P(d_buf), nbytes, passes, ctypes.byref(g)), self)
        return g.value

    def synchronize(self) -> None:
        _check(self._lib.svo_synchronize(self._h), self)

    def launch_count(self) -> int:
        return int(self._lib.svo_launch_count(self._h))

    def target(self, res_x: int, res_y: int) -> "Target":
        return Target(self, res_x, res_y)

    def raycast_full(self, target: "Target", view: View) -> None:
        _check(self._lib.svo_raycast_full(self._h, target._h, ctypes.byref(view)), self)

    def raycast_full_batch(self, targets: Sequence["Target"], views: Sequence[View]) -> None:
        n = len(targets)
        tarr = (_P * n)(*[t._h for t in targets])
        varr = (View * n)(*views)
        _check(self._lib.svo_raycast_full_batch(self._h, ctypes.cast(tarr, _P), ctypes.cast(varr, _P), n), self)

    def warp_frame(self, target: "Target", view: View, frame: int) -> None:
        _check(self._lib.svo_warp_frame(self._h, target._h, ctypes.byref(view), frame), self)

    def warp_frame_learned(self, target: "Target", view: View, frame: int, net: "Net",
                           threshold: float = 0.5) -> None:
        _check(self._lib.svo_warp_frame_learned(self._h, target._h, ctypes.byref(view), frame, net._h,
                                                threshold), self)

    def net(self, seed: int = 1) -> "Net":
        return Net(self, seed)

    def close(self) -> None:
        """Destroy the context; its targets and nets still open are closed first."""
        if getattr(self, "_h", None):
            for t in list(getattr(self, "_targets", ())):
                t.close()
            for n in list(getattr(self, "_nets", ())):
                n.close()
            self._lib.svo_context_destroy(self._h)
            self._h = None

    def __del__(self):
        self.close()


# Contexts still open at interpreter exit are closed while every module is
# intact, whatever order the interpreter would finalise the objects in.
_LIVE_CONTEXTS: "weakref.WeakSet[Context]" = weakref.WeakSet()


@atexit.register
def _close_live_contexts() -> None:
    for c in list(_LIVE_CONTEXTS):
        c.close()


class Target:
    """A render target: warp planes, hole buffer, full-raycast outputs, BGRX image."""

    def __init__(self, ctx: Context, res_x: int, res_y: int):
        self.ctx = ctx
        self._lib = ctx._lib
        self._h = _P()
        _check(self._lib.svo_target_create(ctx._h, res_x, res_y, ctypes.byref(self._h)), ctx)
        ctx._targets.add(self)
        self.res_x, self.res_y = res_x, res_y
        self.n = res_x * res_y
        self.tiles = (res_x // 16) * (res_y // 16)

    def use_graph(self, enable: bool = True) -> None:
        _check(self._lib.svo_target_use_graph(self._h, 1 if enable else 0), self.ctx)

    def set_profiling(self, enable: bool = True) -> None:
        _check(self._lib.svo_target_set_profiling(self._h, 1 if enable else 0), self.ctx)

    def stage_times(self) -> np.ndarray:
        ms = np.zeros(8, np.float32)
        k = self._lib.svo_target_stage_times(self._h, _ptr(ms), 8)
        return ms[:k]

    def colour(self, plane: int = 0) -> np.ndarray:
        out = np.empty(self.n, np.uint32)
        _check(self._lib.svo_read_colour(self._h, plane, _ptr(out)), self.ctx)
        return out

    def coords(self, plane: int = 2) -> np.ndarray:
        out = np.empty(self.n * 4, np.float32)
        _check(self._lib.svo_read_coords(self._h, plane, _ptr(out)), self.ctx)
        return out.reshape(self.n, 4)

    def holes(self) -> tuple[np.ndarray, int]:
        cap = self.n + 2 * self.tiles + 4
        out = np.empty(cap, np.uint32)
        cnt = ctypes.c_uint32()
        _check(self._lib.svo_read_holes(self._h, _ptr(out), cap, ctypes.byref(cnt)), self.ctx)
        return out[: 2 * self.tiles + cnt.value], cnt.value

    def bgrx(self) -> np.ndarray:
        out = np.empty(self.n, np.uint32)
        _check(self._lib.svo_read_bgrx(self._h, _ptr(out)), self.ctx)
        return out

    def bgrx_into(self, out: np.ndarray) -> None:
        _check(self._lib.svo_read_bgrx(self._h, _ptr(out)), self.ctx)

    def bgrx_into_async(self, out: np.ndarray) -> None:
        """svo_read_bgrx_async: the copy overlaps the next frame; `out` (pinned)
        is complete after readback_wait()."""
        _check(self._lib.svo_read_bgrx_async(self._h, _ptr(out)), self.ctx)

    def readback_wait(self) -> None:
        _check(self._lib.svo_target_readback_wait(self._h), self.ctx)

    def full(self) -> tuple[np.ndarray, np.ndarray]:
        col = np.empty(self.n, np.uint32)
        xyzw = np.empty(self.n * 4, np.float32)
        _check(self._lib.svo_read_full(self._h, _ptr(col), _ptr(xyzw)), self.ctx)
        return col, xyzw.reshape(self.n, 4)

    def voxels(self) -> np.ndarray:
        out = np.empty(self.n, np.uint64)
        _check(self._lib.svo_read_voxels(self._h, _ptr(out)), self.ctx)
        return out

    def set_cache_mode(self, mode: int) -> None:
        """0: the reference's copy target 2; 1: the alternating target ((frame>>4)%2)+1."""
        _check(self._lib.svo_target_set_cache_mode(self._h, mode), self.ctx)

    def set_coarse_refresh(self, enable: bool = True) -> None:
        """The raycast_fine pass: one ray per 2x2 block of a moving quadrant, before the hole gather."""
        _check(self._lib.svo_target_set_coarse_refresh(self._h, 1 if enable else 0), self.ctx)

    def set_feature_tap(self, d_features: int | None) -> None:
        """Device buffer (8 x res_y x res_x FP32) receiving the net's input
        features of every later frame; None stops it."""
        _check(self._lib.svo_target_set_feature_tap(self._h, _P(d_features) if d_features else None), self.ctx)

    def set_guided(self, enable: bool = True) -> None:
        """Guided learned frames: pixels with a cached surface point nearby are
        walked from just in front of it; only the others go to the net."""
        _check(self._lib.svo_target_set_guided(self._h, 1 if enable else 0), self.ctx)

    def set_certified(self, enable: bool = True) -> None:
        """Certified reprojection in guided learned frames (off by default):
        pixels whose ray provably meets a cached point's face skip the walk."""
        _check(self._lib.svo_target_set_certified(self._h, 1 if enable else 0), self.ctx)

    def guide(self) -> np.ndarray:
        """Start distances of the last guided frame (raypos units; -1 unguided,
        -2 certified)."""
        out = np.empty(self.n, np.float32)
        _check(self._lib.svo_read_guide(self._h, _ptr(out)), self.ctx)
        return out

    def requested(self) -> int:
        """Rays the net requested in the last learned frame."""
        n = ctypes.c_uint32()
        _check(self._lib.svo_read_requested(self._h, ctypes.byref(n)), self.ctx)
        return n.value

    def device_outputs(self) -> DeviceOutputs:
        d = DeviceOutputs()
        _check(self._lib.svo_target_device_outputs(self._h, ctypes.byref(d)), self.ctx)
        return d

    def close(self) -> None:
        if getattr(self, "_h", None):
            if getattr(self.ctx, "_h", None):  # a closed context already destroyed its targets
                self._lib.svo_target_destroy(self._h)
            self._h = None

    def __del__(self):
        self.close()


class Net:
    """The reconstruction net of learned frames (svo_net_*). Feature, output
    and target arguments are device pointers (ints)."""

    def __init__(self, ctx: Context, seed: int = 1):
        self.ctx = ctx
        self._lib = ctx._lib
        self._h = _P()
        _check(self._lib.svo_net_create(ctx._h, ctypes.byref(self._h)), ctx)
        ctx._nets.add(self)
        if seed != 1:
            self.init(seed)

    def init(self, seed: int) -> None:
        _check(self._lib.svo_net_init(self._h, seed), self.ctx)

    def set_params(self, params: np.ndarray) -> None:
        p = np.ascontiguousarray(params, np.float32)
        _check(self._lib.svo_net_set_params(self._h, _ptr(p), p.size), self.ctx)

    def params(self) -> np.ndarray:
        out = np.empty(NET_PARAMS, np.float32)
        _check(self._lib.svo_net_get_params(self._h, _ptr(out), out.size), self.ctx)
        return out

    def grads(self) -> np.ndarray:
        out = np.empty(NET_PARAMS, np.float32)
        _check(self._lib.svo_net_get_grads(self._h, _ptr(out), out.size), self.ctx)
        return out

    def forward(self, d_features: int, w: int, h: int, d_out: int) -> None:
        _check(self._lib.svo_net_forward(self._h, _P(d_features), w, h, _P(d_out)), self.ctx)

    def infer(self, d_features: int, w: int, h: int, d_out: int) -> None:
        _check(self._lib.svo_net_infer(self._h, _P(d_features), w, h, _P(d_out)), self.ctx)

    def backward(self, d_features: int, d_target_bgrx: int, w: int, h: int, tau: float, lam: float,
                 read_loss: bool = True):
        """Gradients of the loss into the net (forward + backward on the tensor
        cores); returns the two loss terms, or None with read_loss=False (no
        host synchronisation)."""
        loss = np.zeros(2, np.float32)
        _check(self._lib.svo_net_backward(self._h, _P(d_features), _P(d_target_bgrx), w, h, tau, lam,
                                          _ptr(loss) if read_loss else None), self.ctx)
        return (float(loss[0]), float(loss[1])) if read_loss else None

    def adam(self, lr: float, beta1: float = 0.9, beta2: float = 0.999, eps: float = 1e-8) -> None:
        _check(self._lib.svo_net_adam(self._h, lr, beta1, beta2, eps), self.ctx)

    def save(self, path: str) -> None:
        np.save(path, self.params())

    def load_file(self, path: str) -> None:
        self.set_params(np.load(path))

    def close(self) -> None:
        if getattr(self, "_h", None):
            if getattr(self.ctx, "_h", None):
                self._lib.svo_net_destroy(self._h)
            self._h = None

    def __del__(self):
        self.close()


def psnr_bgrx(a: np.ndarray, b: np.ndarray) -> float:
    """PSNR (dB) between two BGRX8 images over the three colour channels."""
    av = a.view(np.uint8).reshape(-1, 4)[:, :3].astype(np.float64)
    bv = b.view(np.uint8).reshape(-1, 4)[:, :3].astype(np.float64)
    mse = float(np.mean((av - bv) ** 2))
    return float("inf") if mse == 0 else 10.0 * np.log10(255.0 ** 2 / mse)
