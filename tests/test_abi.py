"""The C ABI library: loads, exports every symbol include/svo_gb300.h declares,
and its host-only entry points behave (cameras, argument checks). No GPU."""
import os
import re
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "svo_gb300.h")


def _declared():
    text = open(HEADER).read()
    return sorted(set(re.findall(r"^\s*(?:const\s+)?[\w\*\s]+?\b(svo_\w+)\s*\(", text, re.M)))


def test_header_declarations_are_exported(svo):
    names = _declared()
    assert len(names) >= 40
    lib = svo.load()
    for n in names:
        assert hasattr(lib, n), n
    out = subprocess.run(["nm", "-D", "--defined-only", svo.LIB_PATH], capture_output=True, text=True).stdout
    exported = set(re.findall(r"\bT (svo_\w+)", out))
    assert set(names) <= exported
    assert set(svo.EXPORTS) == set(names), "bindings and header disagree"


def test_library_is_sm103a_only(svo):
    # The product library carries one cubin target and no PTX fallback.
    text = open(os.path.join(ROOT, "sparse-voxel-octree-raycasting_gb300", "build.py")).read()
    assert "arch=compute_103a,code=sm_103a" in text


def test_context_without_gpu_fails_loudly(svo):
    import torch

    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    with pytest.raises(svo.SvoError):
        svo.Context(0)


def test_null_handles_are_rejected(svo):
    # the guided-frame and autotuner entry points check their handles before
    # touching a device (1 = SVO_ERR_INVALID_ARGUMENT)
    lib = svo.load()
    assert lib.svo_target_set_guided(None, 1) == 1
    assert lib.svo_read_guide(None, None) == 1
    assert lib.svo_context_autotune_learned(None, None, None, 0, None, 0.5, None, 0, None) == 1
    assert lib.svo_context_set_option(None, svo.OPT_LEARNED_PACKET_WIDTH, 8) == 1
    assert lib.svo_read_bgrx_async(None, None) == 1
    assert lib.svo_target_readback_wait(None) == 1


def test_look_at_rows_are_orthonormal_and_aim(svo):
    pos = np.array([10.0, 40.0, -30.0], np.float32)
    tgt = np.array([32.0, 20.0, 32.0], np.float32)
    v = svo.view_look_at(pos, tgt, 640, 480)
    m = v.m_array.reshape(4, 4)[:3, :3].astype(np.float64)
    assert np.allclose(m @ m.T, np.eye(3), atol=1e-6)
    f = (tgt - pos) / np.linalg.norm(tgt - pos)
    assert np.allclose(m[2], f, atol=1e-6)  # row 2 of m is the view direction (raycast.h:126)


def test_euler_matches_reference_rotation_order(svo):
    # m = I.rotate_z(rz).rotate_x(rx).rotate_y(ry) (src/raycast.h:121-124) with
    # _matrix44's row-vector convention.
    rx, ry, rz = 0.3, -1.1, 0.05
    v = svo.view_from_euler(rx, ry, rz, [1, 2, 3], 64, 64)

    def rot(axis, a):
        c, s = np.cos(a), np.sin(a)
        r = np.eye(4)
        i, j = {"x": (1, 2), "y": (0, 2), "z": (0, 1)}[axis]
        if axis == "y":
            r[i, i], r[j, i], r[i, j], r[j, j] = c, s, -s, c
        else:
            r[i, i], r[j, i], r[i, j], r[j, j] = c, -s, s, c
        return r

    want = np.eye(4) @ rot("z", rz) @ rot("x", rx) @ rot("y", ry)
    assert np.allclose(v.m_array.reshape(4, 4), want, atol=1e-6)


def test_camera_paths_are_deterministic_and_inside(svo):
    for kind in range(4):
        for depth in (8, 11):
            a = svo.camera_path(kind, depth, 17, 320, 200)
            b = svo.camera_path(kind, depth, 17, 320, 200)
            assert np.array_equal(a.pos_array, b.pos_array) and np.array_equal(a.m_array, b.m_array)
            extent = (1 << (depth + 1)) / 16
            p = a.pos_array[:3]
            assert np.all(p >= 0) and np.all(p < extent)
    with pytest.raises(svo.SvoError):
        svo.camera_path(9, 8, 0, 10, 10)


def test_golden_cameras_reproduce_bit_for_bit(svo):
    # The golden fixtures store the cameras as float bits; the deterministic
    # trig makes the path generator reproduce them on any IEEE host.
    import json

    meta = json.load(open(os.path.join(ROOT, "tests", "golden", "golden.json")))
    arrays = np.load(os.path.join(ROOT, "tests", "golden", "golden.npz"))
    for case in meta["full"]:
        v = svo.camera_path(case["kind"], case["depth"], case["frame"], case["W"], case["H"], fov=case["fov"])
        assert np.array_equal(v.pos_array.view(np.uint32), arrays[case["key"] + "_pos"].view(np.uint32))
        assert np.array_equal(v.m_array.view(np.uint32), arrays[case["key"] + "_m"].view(np.uint32))


def test_terrain_is_periodic_and_colours_nonzero(svo):
    x, y, z, c = svo.terrain_voxels(9, 8, True)
    assert x.max() < 256 and y.max() < 256 and z.max() < 256
    assert np.all((c & 0xFF) != 0)  # a zero leaf byte would misalign byte records (octree.h:134)
    # every column has its surface voxel
    cols = np.unique(z.astype(np.int64) * 256 + x)
    assert cols.size == 256 * 256


def test_noalloc_rejects_misaligned_pointers_before_any_launch(svo):
    # Caller buffers at an offset (a sub-allocation from the caller's own pool)
    # that are not aligned for the kernel's stores are refused with
    # SVO_ERR_INVALID_ARGUMENT before any CUDA call, so this runs without a
    # GPU: the pointers are never dereferenced.
    import ctypes

    lib = svo.load()
    v = svo.camera_path(3, 9, 0, 16, 16)
    base = 1 << 20  # a fake, suitably aligned device address

    def call(words, colour, xyzw, voxel, bgrx, n_views=1, view=v):
        varr = (svo.View * n_views)(*([view] * n_views))
        fb = svo.FrameBuffers(colour, xyzw, voxel, bgrx)
        oarr = (svo.FrameBuffers * n_views)(*([fb] * n_views))
        return lib.svo_raycast_full_noalloc(ctypes.c_void_p(words), 100, 0, 9, ctypes.cast(varr, ctypes.c_void_p),
                                            ctypes.cast(oarr, ctypes.c_void_p), n_views, None)

    ok = (base, base + 4096, base + 8192, base + 16384, base + 32768)
    for which, off in ((0, 2), (1, 2), (2, 8), (2, 4), (3, 4), (4, 1)):
        args = list(ok)
        args[which] += off
        assert call(*args) == 1, (which, off)
    # a batch whose packet count would wrap the 32-bit work counter
    big = svo.camera_path(3, 9, 0, 65535, 65535)
    assert call(*ok, n_views=svo.NOALLOC_MAX_VIEWS, view=big) == 1
