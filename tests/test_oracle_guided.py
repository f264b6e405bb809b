"""CPU checks of the oracle's guided walk (the restatement the GPU's guided
learned frames are compared with): a start distance of 0 is the plain ray,
bit for bit; a start just in front of the true hit finds the same voxel."""
import numpy as np


def test_guided_walk_from_zero_is_the_plain_ray(svo, orc, scene):
    octree = scene(9, 5, True)
    W, H = 96, 64
    for kind, f in ((1, 3), (2, 11)):
        v = svo.camera_path(kind, 9, f, W, H)
        c0, x0, _, _ = orc.raycast_full(9, octree.words, octree.root, v.pos_array, v.m_array, W, H)
        c1, x1 = orc.raycast_guided(9, octree.words, octree.root, v.pos_array, v.m_array, W, H,
                                    np.zeros(W * H, np.float32))
        assert np.array_equal(c0, c1)
        assert np.array_equal(x0.view(np.uint32), x1.view(np.uint32))


def test_guided_walk_from_in_front_of_the_hit(svo, orc, scene):
    octree = scene(9, 5, True)
    W, H = 96, 64
    v = svo.camera_path(1, 9, 7, W, H)
    c0, x0, _, _ = orc.raycast_full(9, octree.words, octree.root, v.pos_array, v.m_array, W, H)
    hit = x0[:, 3] < 20000.0
    s0 = np.where(hit, np.maximum(x0[:, 3] * 16.0 - 8.0, 0.0), -1.0).astype(np.float32)
    c1, x1 = orc.raycast_guided(9, octree.words, octree.root, v.pos_array, v.m_array, W, H, s0)
    # at 96 pixels the level of detail rises every 12 world units; the late
    # start takes the level from its start distance, the plain ray lags by a
    # pop, so a few far pixels land on the neighbouring level
    assert (c1[hit] == c0[hit]).mean() > 0.97
    # the distance is accumulated from the start: within float rounding of
    # the plain ray's wherever the same voxel is hit
    assert np.isclose(x1[hit, 3], x0[hit, 3], rtol=1e-4).mean() > 0.97
    # pixels with s0 < 0 are left alone
    assert np.all(c1[~hit] == 0xFFFFFF00)


def test_oracle_guided_frames(svo, orc, scene):
    # the oracle's guided frames (every unguided pixel traced): frames without a
    # cache are the full raycast; afterwards most pixels are walked and nearly
    # all of them land where the full raycast does
    octree = scene(9, 77, True)
    W, H = 96, 64
    g = orc.Guided(9, W, H)
    for f in range(8):
        v = svo.camera_path(2, 9, f, W, H)
        g.frame(octree.words, octree.root, v.pos_array, v.m_array, f)
        full, _, _, _ = orc.raycast_full(9, octree.words, octree.root, v.pos_array, v.m_array, W, H)
        col, gd = g.colour(), g.guide()
        if f < 2:
            assert np.all(gd == -1.0) and np.array_equal(col, full)
        else:
            assert (gd >= 0).mean() > 0.7
            assert (col == full).mean() > 0.99


def test_oracle_guided_frames_across_camera_wraps(svo, orc, scene):
    # The camera wraps into the periodic volume (src/raycast.h:136-145); the
    # guided frames re-base the cached points by whole periods, so a frame right
    # after a wrap is still guided and still lands on the full raycast's voxels.
    depth, W, H = 9, 96, 64
    octree = scene(depth, 77, True)
    period = 2 ** (depth + 1) / 16
    g = orc.Guided(depth, W, H)
    prev, wraps = None, 0
    for f in range(60):
        v = svo.camera_path(2, depth, f, W, H)
        g.frame(octree.words, octree.root, v.pos_array, v.m_array, f)
        p = v.pos_array[:3]
        if prev is not None and np.any(np.abs(p - prev) > period / 2):
            wraps += 1
            full, _, _, _ = orc.raycast_full(depth, octree.words, octree.root, v.pos_array, v.m_array, W, H)
            assert (g.guide() >= 0).mean() > 0.8, f
            assert (g.colour() == full).mean() > 0.98, f
        prev = p
    assert wraps >= 2


def test_oracle_certified_frames(svo, orc, scene):
    # Certified reprojection in the oracle's guided frames: a pixel whose ray
    # meets the face a cached hit lies on takes that point's colour without a
    # walk. Such pixels are marked -2; their displayed colour is nearly always
    # the full raycast's, and the frame stays as close to it as without them.
    depth, W, H = 10, 240, 128
    octree = scene(depth, 2024, True)
    on = orc.Guided(depth, W, H, certify=True)
    off = orc.Guided(depth, W, H)
    share, wrong = [], []
    for f in range(12):
        v = svo.camera_path(1, depth, f, W, H)
        on.frame(octree.words, octree.root, v.pos_array, v.m_array, f)
        off.frame(octree.words, octree.root, v.pos_array, v.m_array, f)
        full, _, _, _ = orc.raycast_full(depth, octree.words, octree.root, v.pos_array, v.m_array, W, H)
        gd = on.guide()
        c = gd == -2.0
        if f < 2:
            assert not c.any()
            continue
        share.append(c.mean())
        a, b = orc.colorize(on.colour()), orc.colorize(full)
        wrong.append((a[c] != b[c]).mean() if c.any() else 0.0)
        # certified pixels carry their hit code: level in the low 5 bits
        codes = on.coords()[c, 3]
        assert np.all(codes >= 1) and np.all(codes == np.floor(codes))
        # walked pixels are the same with and without certification (same cache)
        if f == 2:
            w = gd >= 0
            assert np.array_equal(on.colour()[w], off.colour()[w])
    assert np.mean(share) > 0.1, np.mean(share)
    assert np.mean(wrong) < 0.02, np.mean(wrong)
