"""Seeded benchmark scenes and camera paths restated in numpy.

TEST INFRASTRUCTURE ONLY: the reference arm of bench.py builds its inputs
with these, so the timed CPU reference runs without loading the product
library. The product's own generator (svo_terrain_voxels, svo_camera_path in
csrc/svo_host.cpp) is the specification; tests/test_scene.py checks that both
give bit-identical voxels and views.

Terrain: value-noise fBm heightfield over a D x D grid (D = 2^depth), 6
octaves from 4 lattice cells, lacunarity 2, gain 0.5, height 0.35 D + 0.3 D *
fbm, solid below the surface (or, `shell`, only the voxels a column exposes
to its four neighbours); colour byte = material (height band) | intensity
ramp with +-8 hashed noise. Every float operation is one binary32 (or, for
the cameras, binary64) IEEE operation, in the generator's order.
"""
from __future__ import annotations

import math

import numpy as np

_U32 = np.uint32


def hash32(a, b, c, d):
    """The generator's integer hash on uint32 arrays or scalars (wrapping)."""
    a, b, c, d = (np.asarray(v, dtype=np.uint64) for v in (a, b, c, d))
    m = np.uint64(0xFFFFFFFF)
    h = (a * 0x9E3779B1 & m) ^ (((b + 0x7F4A7C15) & m) * 0x85EBCA77 & m)
    h = h ^ (((c + 0x165667B1) & m) * 0xC2B2AE3D & m)
    h = h ^ (((d + 0x27D4EB2F) & m) * 0x27D4EB2D & m)
    h ^= h >> np.uint64(15)
    h = h * 0x2C1B3C6D & m
    h ^= h >> np.uint64(12)
    h = h * 0x297A2D39 & m
    h ^= h >> np.uint64(15)
    return h.astype(_U32)


def _heights(seed: int, depth: int) -> np.ndarray:
    D = 1 << depth
    f32 = np.float32
    x = np.arange(D, dtype=np.uint64)
    total = np.zeros((D, D), f32)
    norm = f32(0.0)
    amp = f32(1.0)
    for o in range(6):
        cells = 4 << o
        u = x * np.uint64(cells)
        i = (u // np.uint64(D)).astype(np.uint64)
        fr = ((u % np.uint64(D)).astype(f32)) / f32(D)
        s = fr * fr * (f32(3.0) - f32(2.0) * fr)
        i1 = (i + np.uint64(1)) % np.uint64(cells)
        # lattice values at (ix, iz) for every column: rows z, columns x
        def lat(ix, iz):
            h = hash32(np.uint64(seed), np.uint64(o), ix[None, :], iz[:, None])
            return (h & _U32(0xFFFFFF)).astype(f32) * f32(1.0 / 8388608.0) - f32(1.0)

        a, b = lat(i, i), lat(i1, i)
        c, d = lat(i, i1), lat(i1, i1)
        sx, sz = s[None, :], s[:, None]
        ab = a + (b - a) * sx
        cd = c + (d - c) * sx
        total = total + amp * (ab + (cd - ab) * sz)
        norm = f32(norm + amp)
        amp = f32(amp * f32(0.5))
    fbm = total / norm
    h = f32(D) * f32(0.35) + f32(D) * f32(0.3) * fbm
    hi = np.trunc(h).astype(np.int64)
    return np.clip(hi, 0, D - 1)  # [z, x]


def _colour(seed: int, D: int, x, y, z) -> np.ndarray:
    x = x.astype(np.uint64)
    y = y.astype(np.uint64)
    z = z.astype(np.uint64)
    band = y * np.uint64(20) // np.uint64(D)
    material = np.where(band < 7, 3, np.where(band < 9, 1, np.where(band < 12, 2, 0))).astype(np.int64)
    noise = (hash32(np.uint64(seed ^ 0xC0105), x, y, z).astype(np.int64) % 17) - 8
    intensity = 72 + (y * np.uint64(170) // np.uint64(D)).astype(np.int64) + noise
    intensity = np.clip(intensity, 4, 252)
    byte = (intensity & 0xFC) | material
    byte = np.where(byte == 0, 4, byte)
    word = byte | ((x ^ z).astype(np.int64) & 0xFF) << 8 | (y.astype(np.int64) & 0xFF) << 16
    return word.astype(_U32)


def terrain_voxels(seed: int, depth: int, shell: bool):
    """(x, y, z, rgba) uint32 arrays in the generator's insertion order:
    columns z outer, x inner, each from its top down."""
    D = 1 << depth
    top = _heights(seed, depth)
    if shell:
        m = np.minimum(np.minimum(np.roll(top, 1, axis=1), np.roll(top, -1, axis=1)),
                       np.minimum(np.roll(top, 1, axis=0), np.roll(top, -1, axis=0)))
        low = np.maximum(0, np.minimum(top, m + 1))
    else:
        low = np.zeros_like(top)
    count = (top - low + 1).reshape(-1)
    n = int(count.sum())
    col = np.repeat(np.arange(D * D, dtype=np.int64), count)
    start = np.cumsum(count) - count
    k = np.arange(n, dtype=np.int64) - np.repeat(start, count)
    zz, xx = np.divmod(col, D)
    yy = top.reshape(-1)[col] - k
    x, y, z = xx.astype(_U32), yy.astype(_U32), zz.astype(_U32)
    return x, y, z, _colour(seed, D, x, y, z)


# ----------------------------------------------------------------- cameras --
def sincos_det(a: float) -> tuple[float, float]:
    """sin and cos from + - * / in binary64 (range reduction by pi/2, Taylor
    series to degree 21), as the generator computes them."""
    pio2_hi, pio2_lo = 1.5707963267948966, 6.123233995736766e-17
    q = a * 0.6366197723675814
    kq = float(int(q + 0.5) if q >= 0 else -int(-(q - 0.5)))
    r = (a - kq * pio2_hi) - kq * pio2_lo
    r2 = r * r
    sn = cs = 0.0
    ts, tc = r, 1.0
    for i in range(1, 12):
        sn += ts
        cs += tc
        ts = -ts * r2 / float((2 * i) * (2 * i + 1))
        tc = -tc * r2 / float((2 * i - 1) * (2 * i))
    k = (int(kq) % 4 + 4) % 4
    return ((sn, cs), (cs, -sn), (-sn, -cs), (-cs, sn))[k]


def _rot_x(m, c, s):
    f = np.float32
    for i in range(4):
        a, b = m[i * 4 + 1], m[i * 4 + 2]
        m[i * 4 + 1] = f(f(a * c) + f(b * f(-s)))
        m[i * 4 + 2] = f(f(a * s) + f(b * c))


def _rot_y(m, c, s):
    f = np.float32
    for i in range(4):
        a, b = m[i * 4 + 0], m[i * 4 + 2]
        m[i * 4 + 0] = f(f(a * c) + f(b * s))
        m[i * 4 + 2] = f(f(a * f(-s)) + f(b * c))


def look_at(pos, target):
    """Row-major 4x4 float32 view matrix (identity, then rotate_x, rotate_y)."""
    f = [float(target[i]) - float(pos[i]) for i in range(3)]
    ln = math.sqrt(f[0] * f[0] + f[1] * f[1] + f[2] * f[2])
    f = [v / ln for v in f]
    cx = math.sqrt(f[0] * f[0] + f[2] * f[2])
    sx = -f[1]
    cy, sy = (f[2] / cx, f[0] / cx) if cx > 0 else (1.0, 0.0)
    m = np.zeros(16, np.float32)
    m[[0, 5, 10, 15]] = 1.0
    _rot_x(m, np.float32(cx), np.float32(sx))
    _rot_y(m, np.float32(cy), np.float32(sy))
    return m


def wrap_position(pos, depth: int) -> np.ndarray:
    dim2 = np.float32(1 << (depth + 1))
    out = np.zeros(4, np.float32)
    for a in range(3):
        p = np.float32(np.float32(pos[a]) * np.float32(16.0))
        while p < 0:
            p = np.float32(p + dim2)
        while p >= dim2:
            p = np.float32(p - dim2)
        out[a] = np.float32(p / np.float32(16.0))
    return out


def camera_path(kind: int, depth: int, frame: int):
    """(pos float32[4], m float32[16]) of frame `frame` of camera path `kind`:
    1 = orbit at 1.5x extent, 0.5 deg/frame, height sinusoid over 64 frames;
    2 = fast motion, 2 deg/frame plus 0.05 extent/frame translation."""
    E = float(1 << (depth + 1)) / 16.0
    pi = 3.14159265358979323846
    cx, cy, cz = 0.5 * E, 0.35 * E, 0.5 * E
    tx, ty, tz = cx, cy, cz
    if kind == 1:
        s, c = sincos_det(0.5 * pi / 180.0 * frame)
        hs, _ = sincos_det(2.0 * pi * (frame % 64) / 64.0)
        px, pz, py = cx + 1.5 * E * c, cz + 1.5 * E * s, 0.8 * E + 0.02 * E * hs
        ty = 0.45 * E
    elif kind == 2:
        s, c = sincos_det(2.0 * pi / 180.0 * frame)
        hs, _ = sincos_det(2.0 * pi * (frame % 64) / 64.0)
        along = 0.05 * E * frame
        px, pz, py = cx + 0.9 * E * c + along, cz + 0.9 * E * s, 0.75 * E + 0.02 * E * hs
        tx, ty = cx + along, 0.4 * E
    else:
        raise ValueError(f"camera path {kind} is not restated here")
    pos = np.array([px, py, pz], np.float32)
    tgt = np.array([tx, ty, tz], np.float32)
    m = look_at(pos, tgt)
    return wrap_position(pos, depth), m
