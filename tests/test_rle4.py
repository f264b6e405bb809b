"""The .rle4 volume loader (svo_rle4_voxels / svo_rle4_build) against the
reference's own RLE4::load (src/octree/Rle4.cpp, compiled for the host in
oracle/_ref): same voxels, same colour words, same insertion order. The
reference's asset (data/Imrodh.rle4) is missing, so seeded synthetic files
are written here in the same format."""
import ctypes
import hashlib
import struct

import numpy as np
import pytest


def write_rle4(path, maps):
    """maps: list of (sx, sy, sz, columns); a column is (slabs, texels) with
    slabs = list of (skip, length) and one uint16 texel per filled voxel."""
    with open(path, "wb") as f:
        f.write(struct.pack("<i", len(maps)))
        for sx, sy, sz, columns in maps:
            words = []
            for slabs, texels in columns:
                words.append(len(slabs))
                words.append(len(texels))
                words.extend((skip & 1023) | (length << 10) for skip, length in slabs)
                words.extend(texels)
            f.write(struct.pack("<4i", sx, sy, sz, len(words)))
            f.write(np.asarray(words, np.uint16).tobytes())


def synthetic_map(rng, sx, sy, sz):
    columns = []
    for _ in range(sx * sz):
        slabs, texels, y = [], [], 0
        for _ in range(int(rng.integers(0, 4))):
            skip = int(rng.integers(0, 40))
            length = int(rng.integers(1, 20))
            slabs.append((skip, length))
            texels.extend(int(t) for t in rng.integers(0, 65536, length))
            y += skip + length
        columns.append((slabs, texels))
    return (sx, sy, sz, columns)


@pytest.fixture(scope="module")
def rle_file(tmp_path_factory):
    rng = np.random.default_rng(77)
    path = str(tmp_path_factory.mktemp("rle") / "scene.rle4")
    # two maps: the loader turns only map 0 into voxels; sy is small enough
    # that some runs reach past the top and are clipped (Rle4.cpp:123)
    write_rle4(path, [synthetic_map(rng, 48, 60, 40), synthetic_map(rng, 24, 30, 20)])
    return path


def _digest(*arrays):
    h = hashlib.sha256()
    for a in arrays:
        h.update(np.ascontiguousarray(a).tobytes())
    return h.hexdigest()


def test_rle4_voxels_are_deterministic(svo, rle_file):
    a = svo.rle4_voxels(rle_file)
    b = svo.rle4_voxels(rle_file)
    assert a[0].size > 1000
    assert _digest(*a) == _digest(*b)
    assert np.all(a[1] < 60) and np.all(a[0] < 48) and np.all(a[2] < 40)


@pytest.mark.skipif(not __import__("oracle").ref_available(), reason="reference sources not compiled here")
@pytest.mark.parametrize("palette,add", [(0, (0, 0, 0)), (1, (3, 5, 7))])
def test_rle4_matches_reference_loader(svo, orc, rle_file, palette, add):
    lib = orc.reference()
    lib.ref_rle4_voxels.restype = ctypes.c_long
    lib.ref_rle4_voxels.argtypes = [ctypes.c_char_p, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                    ctypes.c_void_p, ctypes.c_size_t]
    n = lib.ref_rle4_voxels(rle_file.encode(), palette, *add, None, 0)
    out = np.empty(4 * n, np.uint32)
    lib.ref_rle4_voxels(rle_file.encode(), palette, *add, out.ctypes.data_as(ctypes.c_void_p), out.size)
    ref = out.reshape(-1, 4).T
    mine = svo.rle4_voxels(rle_file, palette, add)
    for r, m in zip(ref, mine):
        assert np.array_equal(r, m)


def test_rle4_octree_matches_oracle_builder(svo, orc, rle_file):
    b = svo.Builder(8)
    b.add_rle4(rle_file, 0, (10, 20, 30))
    mine = b.finish()
    x, y, z, c = svo.rle4_voxels(rle_file, 0, (10, 20, 30))
    words, root = orc.build_octree(8, x, y, z, c)
    assert root == mine.root and np.array_equal(words, mine.words)


def test_rle4_rejects_bad_files(svo, tmp_path):
    with pytest.raises(svo.SvoError):
        svo.rle4_voxels(str(tmp_path / "missing.rle4"))
    bad = tmp_path / "truncated.rle4"
    bad.write_bytes(struct.pack("<i4i", 1, 4, 4, 4, 1000) + b"\x00" * 10)
    with pytest.raises(svo.SvoError):
        svo.rle4_voxels(str(bad))
    # a column whose counts run past the slab array
    bad2 = tmp_path / "overrun.rle4"
    bad2.write_bytes(struct.pack("<i4i", 1, 1, 4, 1, 3) + np.array([5, 9, 0], np.uint16).tobytes())
    with pytest.raises(svo.SvoError):
        svo.rle4_voxels(str(bad2))


def test_bmp_dump(svo, tmp_path):
    w, h = 37, 19
    img = (np.arange(w * h, dtype=np.uint32) * 2654435761) & 0xFFFFFF
    p = str(tmp_path / "frame.bmp")
    svo.write_bmp(p, img, w, h)
    data = open(p, "rb").read()
    assert data[:2] == b"BM"
    size, = struct.unpack_from("<I", data, 2)
    off, = struct.unpack_from("<I", data, 10)
    bw, bh = struct.unpack_from("<ii", data, 18)
    bpp, = struct.unpack_from("<H", data, 28)
    assert size == len(data) == 54 + 4 * w * h and off == 54 and (bw, bh, bpp) == (w, h, 32)
    rows = np.frombuffer(data[54:], np.uint32).reshape(h, w)
    assert np.array_equal(rows[::-1].reshape(-1), img)  # bottom-up rows
