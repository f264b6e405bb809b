// svo_host.cpp -- host side of libsvo_gb300.so: the octree builder, the
// octree file format, the seeded synthetic terrain and the camera helpers.
//
// Builder design. The reference inserts voxels one at a time into a pointer
// octree (src/octree/octree.h:32-89, one 36-byte node per inner node, 24-bit
// node index) and then walks it recursively (octree.h:95-293). This builder
// instead keeps the voxels as a flat list of 3-D Morton keys, radix-sorts them
// (stable, so insertion order is kept among duplicates), and derives every
// tree level by one linear pass over the level below: a node is a run of
// children sharing key>>3. The compact layout is then emitted by the same
// depth-first order as convert_tree_blocks, which fixes every word offset.
// Node colours follow the reference exactly: a node takes the colour of the
// first voxel inserted through it, a leaf the colour of the last insertion of
// that voxel. There is no 2^24 node cap; the limits are those of the compact
// words themselves (23-bit offsets).
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <memory>
#include <string>
#include <thread>
#include <vector>

#include "../../include/svo_gb300.h"

namespace {

inline uint32_t popc8(uint32_t v) { return (uint32_t)__builtin_popcount(v & 0xffu); }

// Morton key, child index bit order (x | y<<1 | z<<2) per level as in
// set_voxel's childbit (octree.h:58).
inline uint64_t spread3(uint32_t v) {
    uint64_t x = v & 0x1fffffu;
    x = (x | x << 32) & 0x1f00000000ffffull;
    x = (x | x << 16) & 0x1f0000ff0000ffull;
    x = (x | x << 8) & 0x100f00f00f00f00full;
    x = (x | x << 4) & 0x10c30c30c30c30c3ull;
    x = (x | x << 2) & 0x1249249249249249ull;
    return x;
}
inline uint64_t morton3(uint32_t x, uint32_t y, uint32_t z) {
    return spread3(x) | (spread3(y) << 1) | (spread3(z) << 2);
}

// Stable LSD radix sort of (key, payload) pairs on the low `bits` key bits.
void radix_sort_pairs(std::vector<uint64_t>& keys, std::vector<uint32_t>& vals, int bits) {
    const size_t n = keys.size();
    if (n < 2) return;
    std::vector<uint64_t> k2(n);
    std::vector<uint32_t> v2(n);
    const int digit = 11;
    const size_t buckets = (size_t)1 << digit;
    unsigned hw = std::max(1u, std::min(16u, std::thread::hardware_concurrency()));
    const size_t nt = n < (1u << 20) ? 1 : hw;
    std::vector<size_t> hist(nt * buckets);
    for (int shift = 0; shift < bits; shift += digit) {
        std::fill(hist.begin(), hist.end(), 0);
        auto chunk = [&](size_t t) { return std::make_pair(n * t / nt, n * (t + 1) / nt); };
        {
            std::vector<std::thread> th;
            for (size_t t = 0; t < nt; ++t)
                th.emplace_back([&, t] {
                    auto [a, b] = chunk(t);
                    size_t* h = &hist[t * buckets];
                    for (size_t i = a; i < b; ++i) ++h[(keys[i] >> shift) & (buckets - 1)];
                });
            for (auto& x : th) x.join();
        }
        // Skip passes where every key shares the digit.
        bool trivial = false;
        for (size_t d = 0; d < buckets; ++d) {
            size_t tot = 0;
            for (size_t t = 0; t < nt; ++t) tot += hist[t * buckets + d];
            if (tot == n) trivial = true;
            if (tot) break;
        }
        if (trivial) continue;
        size_t acc = 0;
        for (size_t d = 0; d < buckets; ++d)
            for (size_t t = 0; t < nt; ++t) {
                size_t c = hist[t * buckets + d];
                hist[t * buckets + d] = acc;
                acc += c;
            }
        {
            std::vector<std::thread> th;
            for (size_t t = 0; t < nt; ++t)
                th.emplace_back([&, t] {
                    auto [a, b] = chunk(t);
                    size_t* h = &hist[t * buckets];
                    for (size_t i = a; i < b; ++i) {
                        size_t p = h[(keys[i] >> shift) & (buckets - 1)]++;
                        k2[p] = keys[i];
                        v2[p] = vals[i];
                    }
                });
            for (auto& x : th) x.join();
        }
        keys.swap(k2);
        vals.swap(v2);
    }
}

struct Level {
    std::vector<uint64_t> key;    // Morton prefix of the node
    std::vector<uint32_t> first;  // smallest insertion index in the subtree
    std::vector<uint32_t> begin;  // first child in the level below (size()+1 entries)
    std::vector<uint8_t> mask;    // child mask
};

}  // namespace

struct svo_builder {
    int depth;
    std::vector<uint64_t> keys;
    std::vector<uint32_t> rgba;
    std::vector<uint32_t> words;
    uint32_t root = 0;
    uint64_t voxels = 0, nodes = 0;
    bool finished = false;
    std::string error;
};

namespace {

struct Emitter {
    const std::vector<Level>& L;       // L[h]: nodes of height h (0 = voxels)
    const std::vector<uint32_t>& leaf;  // leaf colour word per unique voxel
    const std::vector<uint32_t>& rgba;  // input colours by insertion index
    std::vector<uint32_t>& out;
    int depth;
    uint32_t normal_cursor = 0;
    bool overflow = false;

    // The root is pre-pushed with a zero colour and never recoloured
    // (src/raycast.h:15-17, octree.h:44-48); every other node keeps the colour
    // of the voxel that created it, i.e. the first one inserted through it.
    uint32_t colour(int h, uint32_t i) const { return h == depth ? 0u : rgba[L[h].first[i]]; }

    uint32_t rel_word(size_t pos, uint32_t local_root, uint8_t mask) {
        uint64_t rel = pos - local_root;
        if (rel >= (1u << 23)) overflow = true;
        return (uint32_t)(rel << 9) + 256u + mask;
    }

    // convert_tree (octree.h:95-191) for heights 6..2.
    uint32_t block(int h, uint32_t i, uint32_t local_root) {
        const Level& lv = L[h];
        if (h == 2) {
            size_t pos = out.size();
            uint32_t acc = 0, nbytes = 0;
            auto put = [&](uint32_t byte) {
                acc |= (byte & 0xffu) << (8 * (nbytes & 3));
                if ((++nbytes & 3) == 0) {
                    out.push_back(acc);
                    acc = 0;
                }
            };
            put(colour(2, i));
            const Level& l1 = L[1];
            for (uint32_t c = lv.begin[i]; c < lv.begin[i + 1]; ++c) put(l1.mask[c]);
            for (uint32_t c = lv.begin[i]; c < lv.begin[i + 1]; ++c)
                for (uint32_t v = l1.begin[c]; v < l1.begin[c + 1]; ++v)
                    if (leaf[v] != 0) put(leaf[v]);  // zero colour words are skipped (octree.h:134)
            if (nbytes & 3) out.push_back(acc);
            return rel_word(pos, local_root, lv.mask[i]);
        }
        uint32_t cw[8];
        int nc = 0;
        for (uint32_t c = lv.begin[i]; c < lv.begin[i + 1]; ++c) cw[nc++] = block(h - 1, c, local_root);
        size_t pos = out.size();
        out.push_back(colour(h, i));
        for (int k = 0; k < nc; ++k) out.push_back(cw[k]);
        return rel_word(pos, local_root, lv.mask[i]);
    }

    // convert_tree_blocks (octree.h:232-293) for heights depth..7.
    uint32_t normal(int h, uint32_t i) {
        const Level& lv = L[h];
        const Level& lc = L[h - 1];
        uint32_t cw[8] = {0, 0, 0, 0, 0, 0, 0, 0};
        for (uint32_t c = lv.begin[i]; c < lv.begin[i + 1]; ++c) {
            uint32_t j = (uint32_t)(lc.key[c] & 7u);
            if (h - 1 >= 7) {
                cw[j] = normal(h - 1, c);
            } else {
                size_t local_root = (out.size() + 63) / 64 * 64;
                uint32_t entries = popc8(lc.mask[c]) + 1;
                if ((local_root >> 6) >= (1u << 23)) overflow = true;
                out.resize(local_root + entries, 0u);
                cw[j] = (uint32_t)(((local_root >> 6) << 9) | (1u << 8) | lc.mask[c]);
                uint32_t sub = block(h - 1, c, (uint32_t)local_root) >> 9;
                for (uint32_t e = 0; e < entries; ++e) out[local_root + e] = out[local_root + sub + e];
                out.resize(local_root + sub);
            }
        }
        uint32_t at = normal_cursor;
        if ((size_t)at + 10 > out.size()) {
            overflow = true;
            return 0;
        }
        for (int j = 0; j < 8; ++j) out[at + j] = cw[j];
        out[at + 8] = colour(h, i);
        out[at + 9] = colour(h, i);
        normal_cursor += 10;
        if (at >= (1u << 23)) overflow = true;
        return (at << 9) | lv.mask[i];
    }
};

// ---------------------------------------------------------- terrain ------
// Deterministic on any IEEE-754 host: integer hashing plus binary32 + - *
// only (the library is built with -ffp-contract=off).
inline uint32_t hash32(uint32_t a, uint32_t b, uint32_t c, uint32_t d) {
    uint32_t h = a * 0x9e3779b1u ^ (b + 0x7f4a7c15u) * 0x85ebca77u;
    h ^= (c + 0x165667b1u) * 0xc2b2ae3du;
    h ^= (d + 0x27d4eb2fu) * 0x27d4eb2du;
    h ^= h >> 15;
    h *= 0x2c1b3c6du;
    h ^= h >> 12;
    h *= 0x297a2d39u;
    h ^= h >> 15;
    return h;
}
inline float lattice(uint32_t seed, uint32_t oct, uint32_t i, uint32_t k) {
    return (float)(hash32(seed, oct, i, k) & 0xffffffu) * (1.0f / 8388608.0f) - 1.0f;
}

struct Terrain {
    int depth;
    uint32_t D;
    uint32_t seed;
    std::vector<int32_t> height;  // per column, voxel units

    explicit Terrain(const svo_terrain_spec& s) : depth(s.depth), D(1u << s.depth), seed(s.seed), height((size_t)D * D) {
        const int octaves = 6;
        const uint32_t base_cells = 4;
        for (uint32_t z = 0; z < D; ++z)
            for (uint32_t x = 0; x < D; ++x) {
                float sum = 0.0f, amp = 1.0f, norm = 0.0f;
                for (int o = 0; o < octaves; ++o) {
                    uint32_t cells = base_cells << o;  // lacunarity 2
                    uint64_t ux = (uint64_t)x * cells, uz = (uint64_t)z * cells;
                    uint32_t ix = (uint32_t)(ux / D), iz = (uint32_t)(uz / D);
                    float fx = (float)(uint32_t)(ux % D) / (float)D;
                    float fz = (float)(uint32_t)(uz % D) / (float)D;
                    float sx = fx * fx * (3.0f - 2.0f * fx);
                    float sz = fz * fz * (3.0f - 2.0f * fz);
                    uint32_t ix1 = (ix + 1) % cells, iz1 = (iz + 1) % cells;
                    float a = lattice(seed, o, ix, iz), b = lattice(seed, o, ix1, iz);
                    float c = lattice(seed, o, ix, iz1), d = lattice(seed, o, ix1, iz1);
                    float ab = a + (b - a) * sx;
                    float cd = c + (d - c) * sx;
                    sum = sum + amp * (ab + (cd - ab) * sz);
                    norm = norm + amp;
                    amp = amp * 0.5f;  // gain 0.5
                }
                float fbm = sum / norm;
                float h = (float)D * 0.35f + (float)D * 0.3f * fbm;
                int hi = (int)h;
                if (hi < 0) hi = 0;
                if (hi > (int)D - 1) hi = (int)D - 1;
                height[(size_t)z * D + x] = hi;
            }
    }
    int32_t h(int64_t x, int64_t z) const {
        uint32_t xx = (uint32_t)((x % (int64_t)D + D) % D), zz = (uint32_t)((z % (int64_t)D + D) % D);
        return height[(size_t)zz * D + xx];
    }
    // Colour word: low byte = material(2 bits, height band) | intensity ramp
    // +-8 noise (multiple of 4, never 0); upper bytes carry column detail.
    uint32_t colour(uint32_t x, uint32_t y, uint32_t z) const {
        uint32_t band = (uint32_t)((uint64_t)y * 20 / D);  // 0..19 across the volume
        uint32_t material = band < 7 ? 3u : (band < 9 ? 1u : (band < 12 ? 2u : 0u));
        int noise = (int)(hash32(seed ^ 0xc0105u, x, y, z) % 17u) - 8;
        int intensity = 72 + (int)((uint64_t)y * 170 / D) + noise;
        if (intensity < 4) intensity = 4;
        if (intensity > 252) intensity = 252;
        uint32_t byte = ((uint32_t)intensity & 0xfcu) | material;
        if (byte == 0) byte = 4;
        return byte | ((x ^ z) & 0xffu) << 8 | (y & 0xffu) << 16;
    }
    template <class F>
    void for_each_voxel(bool shell, F&& emit) const {
        for (uint32_t z = 0; z < D; ++z)
            for (uint32_t x = 0; x < D; ++x) {
                int32_t top = h(x, z);
                int32_t low = 0;
                if (shell) {
                    int32_t m = std::min(std::min(h((int64_t)x - 1, z), h((int64_t)x + 1, z)),
                                         std::min(h(x, (int64_t)z - 1), h(x, (int64_t)z + 1)));
                    low = std::max(0, std::min(top, m + 1));
                }
                for (int32_t y = top; y >= low; --y) emit(x, (uint32_t)y, z, colour(x, (uint32_t)y, z));
            }
    }
    // Seeded axis-aligned solid boxes (edge 16..256 voxels scaled to the volume).
    template <class F>
    void for_each_box_voxel(int boxes, F&& emit) const {
        for (int b = 0; b < boxes; ++b) {
            uint32_t r0 = hash32(seed, 0xb0c5u, (uint32_t)b, 1), r1 = hash32(seed, 0xb0c5u, (uint32_t)b, 2);
            uint32_t r2 = hash32(seed, 0xb0c5u, (uint32_t)b, 3), r3 = hash32(seed, 0xb0c5u, (uint32_t)b, 4);
            uint32_t emin = std::max<uint32_t>(2, D >> 8), emax = std::max<uint32_t>(emin + 1, D >> 4);
            uint32_t ex = emin + r0 % (emax - emin), ey = emin + (r0 >> 16) % (emax - emin),
                     ez = emin + r1 % (emax - emin);
            uint32_t x0 = r2 % D, z0 = r3 % D;
            int32_t ground = h(x0, z0);
            uint32_t y0 = (uint32_t)std::max(0, ground - (int32_t)(ey / 4));
            for (uint32_t z = z0; z < z0 + ez; ++z)
                for (uint32_t x = x0; x < x0 + ex; ++x)
                    for (uint32_t y = y0 + ey; y-- > y0;) {
                        if (y >= D) continue;
                        uint32_t xx = x % D, zz = z % D;
                        bool surface = x == x0 || z == z0 || x == x0 + ex - 1 || z == z0 + ez - 1 ||
                                       y == y0 || y == y0 + ey - 1;
                        if (!surface) continue;
                        uint32_t byte = (((uint32_t)(96 + (b * 37) % 128) & 0xfcu) | 2u);
                        emit(xx, y, zz, byte | ((uint32_t)b & 0xffu) << 8);
                    }
        }
    }
};

// --------------------------------------------------------- trig ----------
// sin/cos of float camera angles, from +, -, * only (no libm), so camera
// paths agree bit for bit between hosts. Range reduction by multiples of
// pi/2 in double; Taylor series to degree 21 on [-pi/4, pi/4].
void sincos_det(double a, double& s, double& c) {
    const double pio2_hi = 1.5707963267948966, pio2_lo = 6.123233995736766e-17;
    double q = a * 0.6366197723675814;
    double kq = (double)(long long)(q >= 0 ? q + 0.5 : q - 0.5);
    double r = (a - kq * pio2_hi) - kq * pio2_lo;
    double r2 = r * r;
    double sn = 0.0, cs = 0.0, term_s = r, term_c = 1.0;
    for (int i = 1; i <= 11; ++i) {
        sn += term_s;
        cs += term_c;
        term_s = -term_s * r2 / (double)((2 * i) * (2 * i + 1));
        term_c = -term_c * r2 / (double)((2 * i - 1) * (2 * i));
    }
    long long k = ((long long)kq % 4 + 4) % 4;
    switch (k) {
        case 0: s = sn; c = cs; break;
        case 1: s = cs; c = -sn; break;
        case 2: s = -sn; c = -cs; break;
        default: s = -cs; c = sn; break;
    }
}

// The row operations of _matrix44::rotate_x/_y/_z (ext/mathlib/_matrix44.h:
// 529-580) applied to a row-major float matrix, with c and s given.
void rot_x(float* m, float c, float s) {
    for (int i = 0; i < 4; ++i) {
        float a = m[i * 4 + 1], b = m[i * 4 + 2];
        m[i * 4 + 1] = a * c + b * -s;
        m[i * 4 + 2] = a * s + b * c;
    }
}
void rot_y(float* m, float c, float s) {
    for (int i = 0; i < 4; ++i) {
        float a = m[i * 4 + 0], b = m[i * 4 + 2];
        m[i * 4 + 0] = a * c + b * s;
        m[i * 4 + 2] = a * -s + b * c;
    }
}
void rot_z(float* m, float c, float s) {
    for (int i = 0; i < 4; ++i) {
        float a = m[i * 4 + 0], b = m[i * 4 + 1];
        m[i * 4 + 0] = a * c + b * -s;
        m[i * 4 + 1] = a * s + b * c;
    }
}
void identity(float* m) {
    for (int i = 0; i < 16; ++i) m[i] = (i % 5 == 0) ? 1.0f : 0.0f;
}

void fill_view(svo_view* out, const float pos[3], const float* m, int res_x, int res_y, float fov) {
    for (int i = 0; i < 3; ++i) out->pos[i] = pos[i];
    out->pos[3] = 0.0f;
    std::memcpy(out->m, m, sizeof(float) * 16);
    out->fovx = fov;
    out->fovy = fov;
    out->res_x = res_x;
    out->res_y = res_y;
}

// --------------------------------------------------------------- .rle4 ----
// The reference's mip-volume format (src/octree/Rle4.cpp:8-165): int32 map
// count, then per map sx, sy, sz, slabs_size and slabs_size uint16 words. A
// map is sx*sz columns, x fastest; a column is [count, texels, count slab
// words, texels texel words]; a slab word skips (slab & 1023) empty voxels
// and then fills (slab >> 10) voxels, one texel each. Only map 0 is turned
// into voxels (Rle4.cpp:91), column by column (z outer, x inner), top of the
// volume first in y (y = sy-1-y1).
struct Rle4Map {
    int32_t sx = 0, sy = 0, sz = 0;
    std::vector<uint16_t> slabs;
    std::vector<uint32_t> column;  // slab offset of every column
};

bool rle4_read(const char* path, Rle4Map& m0, std::string& why) {
    FILE* f = std::fopen(path, "rb");
    if (!f) {
        why = "cannot open";
        return false;
    }
    auto rd = [&](void* p, size_t bytes) { return std::fread(p, 1, bytes, f) == bytes; };
    int32_t nummaps = 0;
    bool ok = rd(&nummaps, 4) && nummaps >= 1 && nummaps <= 16;
    for (int m = 0; ok && m < nummaps; ++m) {
        int32_t hdr[4];
        ok = rd(hdr, 16) && hdr[0] > 0 && hdr[1] > 0 && hdr[2] > 0 && hdr[3] > 0 &&
             (int64_t)hdr[0] * hdr[2] <= (1ll << 28) && hdr[3] <= (1 << 30);
        if (!ok) break;
        Rle4Map map;
        map.sx = hdr[0];
        map.sy = hdr[1];
        map.sz = hdr[2];
        map.slabs.resize((size_t)hdr[3]);
        ok = rd(map.slabs.data(), map.slabs.size() * 2);
        if (!ok) break;
        // Column offsets (Rle4.cpp:50-73), bounds-checked.
        const size_t cols = (size_t)map.sx * map.sz;
        map.column.resize(cols);
        size_t ofs = 0;
        for (size_t c = 0; c < cols && ok; ++c) {
            if (ofs + 2 > map.slabs.size()) {
                ok = false;
                break;
            }
            map.column[c] = (uint32_t)ofs;
            const size_t count = map.slabs[ofs], texels = map.slabs[ofs + 1];
            if (ofs + 2 + count + texels > map.slabs.size()) ok = false;
            ofs += count + texels + 2;
        }
        if (ok && m == 0) m0 = std::move(map);
    }
    std::fclose(f);
    if (!ok && why.empty()) why = "malformed .rle4 file";
    return ok;
}

// Voxels of map 0 with the reference's colour word (Rle4.cpp:116-160).
template <class F>
void rle4_voxels(const Rle4Map& m, int palette, uint32_t addx, uint32_t addy, uint32_t addz, F&& emit) {
    for (int32_t slice = 0; slice < m.sz; ++slice)
        for (int32_t x = 0; x < m.sx; ++x) {
            const size_t ofs = m.column[(size_t)x + (size_t)m.sx * slice];
            const uint32_t count = m.slabs[ofs];
            const uint32_t texels = m.slabs[ofs + 1];
            const uint16_t* p = m.slabs.data() + ofs + 2;
            const uint16_t* pt = p + count;
            const uint16_t* pt_end = pt + texels;
            uint32_t y1 = 0, y2 = 0;
            for (uint32_t s = 0; s < count; ++s) {
                const uint16_t slab = p[s];
                y1 += slab & 1023u;
                y2 = y1 + (slab >> 10);
                for (; y1 < y2; ++y1, ++pt) {
                    if (y1 >= (uint32_t)m.sy || pt >= pt_end) continue;
                    const uint32_t tcol = *pt;
                    const int material = (int)((tcol >> 8) & 3u);
                    int intensity = (int)((tcol & 255u) * (tcol & 255u) / 255u);
                    if (intensity < 2) intensity = 2;
                    if (intensity > 255) intensity = 255;
                    uint32_t rx = (uint32_t)(material + ((intensity >> 3) << 3)) & 0xffu;
                    if (!palette) rx = (1u + ((255u - (tcol & 255u)) & 0xfcu)) & 0xffu;
                    const uint32_t ry = ((tcol >> 5) << 3) & 0xffu;
                    const uint32_t rz = ((tcol >> 10) << 3) & 0xffu;
                    emit((uint32_t)x + addx, (uint32_t)m.sy - 1u - y1 + addy, (uint32_t)slice + addz,
                         rx | (ry << 8) | (rz << 16));
                }
            }
        }
}

}  // namespace

// ================================================================ C ABI ==
extern "C" {

svo_status svo_builder_create(int depth, svo_builder** out) {
    if (!out || depth < SVO_MIN_DEPTH || depth > SVO_MAX_DEPTH) return SVO_ERR_INVALID_ARGUMENT;
    auto* b = new (std::nothrow) svo_builder;
    if (!b) return SVO_ERR_OUT_OF_MEMORY;
    b->depth = depth;
    *out = b;
    return SVO_OK;
}

svo_status svo_builder_destroy(svo_builder* b) {
    delete b;
    return SVO_OK;
}

svo_status svo_builder_set_voxel(svo_builder* b, uint32_t x, uint32_t y, uint32_t z, uint32_t rgba) {
    if (!b || b->finished) return SVO_ERR_INVALID_ARGUMENT;
    const uint32_t D = 1u << b->depth;
    if (x >= D || y >= D || z >= D) return SVO_ERR_INVALID_ARGUMENT;
    if (b->keys.size() >= 0xffffffffull) return SVO_ERR_CAPACITY;
    b->keys.push_back(morton3(x, y, z));
    b->rgba.push_back(rgba);
    return SVO_OK;
}

svo_status svo_builder_set_voxels(svo_builder* b, const uint32_t* x, const uint32_t* y, const uint32_t* z,
                                  const uint32_t* rgba, size_t n) {
    if (!b || b->finished || (n && (!x || !y || !z || !rgba))) return SVO_ERR_INVALID_ARGUMENT;
    const uint32_t D = 1u << b->depth;
    if (b->keys.size() + n >= 0xffffffffull) return SVO_ERR_CAPACITY;
    b->keys.reserve(b->keys.size() + n);
    b->rgba.reserve(b->rgba.size() + n);
    for (size_t i = 0; i < n; ++i) {
        if (x[i] >= D || y[i] >= D || z[i] >= D) return SVO_ERR_INVALID_ARGUMENT;
        b->keys.push_back(morton3(x[i], y[i], z[i]));
        b->rgba.push_back(rgba[i]);
    }
    return SVO_OK;
}

svo_status svo_builder_finish(svo_builder* b, size_t initial_words, uint32_t* root_word, size_t* n_words) {
    if (!b || b->finished) return SVO_ERR_INVALID_ARGUMENT;
    if (initial_words == 0) initial_words = SVO_DEFAULT_INITIAL_WORDS;
    const int depth = b->depth;
    const size_t n = b->keys.size();
    b->voxels = n;
    std::vector<uint64_t> keys;
    keys.swap(b->keys);
    std::vector<uint32_t> order(n);
    for (size_t i = 0; i < n; ++i) order[i] = (uint32_t)i;
    radix_sort_pairs(keys, order, 3 * depth);

    // Level 0: unique voxels. The sort is stable, so within a run of equal
    // keys the first element is the first insertion and the last the last.
    std::vector<Level> L(depth + 1);
    std::vector<uint32_t> leaf;
    {
        Level& l0 = L[0];
        for (size_t i = 0; i < n;) {
            size_t j = i + 1;
            while (j < n && keys[j] == keys[i]) ++j;
            l0.key.push_back(keys[i]);
            l0.first.push_back(order[i]);
            leaf.push_back(b->rgba[order[j - 1]]);
            i = j;
        }
    }
    std::vector<uint64_t>().swap(keys);
    std::vector<uint32_t>().swap(order);
    for (int h = 1; h <= depth; ++h) {
        const Level& lc = L[h - 1];
        Level& lv = L[h];
        const size_t m = lc.key.size();
        for (size_t i = 0; i < m;) {
            uint64_t k = lc.key[i] >> 3;
            size_t j = i;
            uint32_t first = 0xffffffffu;
            uint8_t mask = 0;
            while (j < m && (lc.key[j] >> 3) == k) {
                first = std::min(first, lc.first[j]);
                mask |= (uint8_t)(1u << (lc.key[j] & 7u));
                ++j;
            }
            lv.key.push_back(k);
            lv.first.push_back(first);
            lv.begin.push_back((uint32_t)i);
            lv.mask.push_back(mask);
            i = j;
        }
        lv.begin.push_back((uint32_t)m);
    }
    uint64_t nodes = 1;  // the root
    for (int h = 1; h < depth; ++h) nodes += L[h].key.size();
    b->nodes = n ? nodes : 1;

    b->words.assign(initial_words, 0u);
    if (n == 0) {
        // Empty scene: an all-zero root node with no children (octree.h:280-292).
        b->root = 0;
        b->finished = true;
        if (root_word) *root_word = 0;
        if (n_words) *n_words = b->words.size();
        return SVO_OK;
    }
    Emitter em{L, leaf, b->rgba, b->words, depth};
    b->root = em.normal(depth, 0);
    if (em.overflow || b->words.size() >= 0xffffffffull) {
        b->words.clear();
        b->error = "octree exceeds the compact format's 23-bit offsets";
        return SVO_ERR_CAPACITY;
    }
    std::vector<uint32_t>().swap(b->rgba);
    b->finished = true;
    if (root_word) *root_word = b->root;
    if (n_words) *n_words = b->words.size();
    return SVO_OK;
}

svo_status svo_builder_copy_words(const svo_builder* b, uint32_t* out) {
    if (!b || !b->finished || !out) return SVO_ERR_INVALID_ARGUMENT;
    std::memcpy(out, b->words.data(), b->words.size() * 4);
    return SVO_OK;
}

svo_status svo_builder_stats(const svo_builder* b, uint64_t* voxels, uint64_t* nodes) {
    if (!b) return SVO_ERR_INVALID_ARGUMENT;
    if (voxels) *voxels = b->finished ? b->voxels : b->keys.size();
    if (nodes) *nodes = b->nodes;
    return SVO_OK;
}

static const uint32_t kFileMagic = 0x4f565353u;  // "SSVO"

svo_status svo_octree_save(const char* path, const uint32_t* words, size_t n_words, uint32_t root_word, int depth) {
    if (!path || (!words && n_words)) return SVO_ERR_INVALID_ARGUMENT;
    FILE* f = std::fopen(path, "wb");
    if (!f) return SVO_ERR_IO;
    uint32_t hdr[4] = {kFileMagic, (uint32_t)depth, root_word, 0};
    uint64_t n = n_words;
    bool ok = std::fwrite(hdr, 4, 4, f) == 4 && std::fwrite(&n, 8, 1, f) == 1 &&
              std::fwrite(words, 4, n_words, f) == n_words;
    ok = (std::fclose(f) == 0) && ok;
    return ok ? SVO_OK : SVO_ERR_IO;
}

svo_status svo_octree_load_header(const char* path, size_t* n_words, uint32_t* root_word, int* depth) {
    if (!path) return SVO_ERR_INVALID_ARGUMENT;
    FILE* f = std::fopen(path, "rb");
    if (!f) return SVO_ERR_IO;
    uint32_t hdr[4];
    uint64_t n = 0;
    bool ok = std::fread(hdr, 4, 4, f) == 4 && std::fread(&n, 8, 1, f) == 1 && hdr[0] == kFileMagic;
    std::fclose(f);
    if (!ok) return SVO_ERR_IO;
    if (n_words) *n_words = (size_t)n;
    if (root_word) *root_word = hdr[2];
    if (depth) *depth = (int)hdr[1];
    return SVO_OK;
}

svo_status svo_octree_load_words(const char* path, uint32_t* words, size_t n_words) {
    if (!path || (!words && n_words)) return SVO_ERR_INVALID_ARGUMENT;
    FILE* f = std::fopen(path, "rb");
    if (!f) return SVO_ERR_IO;
    uint32_t hdr[4];
    uint64_t n = 0;
    bool ok = std::fread(hdr, 4, 4, f) == 4 && std::fread(&n, 8, 1, f) == 1 && hdr[0] == kFileMagic &&
              n == n_words && std::fread(words, 4, n_words, f) == n_words;
    std::fclose(f);
    return ok ? SVO_OK : SVO_ERR_IO;
}

svo_status svo_terrain_build(svo_builder* b, const svo_terrain_spec* spec) {
    if (!b || !spec || spec->depth != b->depth || b->finished) return SVO_ERR_INVALID_ARGUMENT;
    Terrain t(*spec);
    t.for_each_voxel(spec->shell != 0, [&](uint32_t x, uint32_t y, uint32_t z, uint32_t c) {
        b->keys.push_back(morton3(x, y, z));
        b->rgba.push_back(c);
    });
    t.for_each_box_voxel(spec->boxes, [&](uint32_t x, uint32_t y, uint32_t z, uint32_t c) {
        b->keys.push_back(morton3(x, y, z));
        b->rgba.push_back(c);
    });
    return b->keys.size() >= 0xffffffffull ? SVO_ERR_CAPACITY : SVO_OK;
}

svo_status svo_terrain_voxels(const svo_terrain_spec* spec, uint32_t* x, uint32_t* y, uint32_t* z, uint32_t* rgba,
                              size_t cap, size_t* n) {
    if (!spec || !n || spec->depth < SVO_MIN_DEPTH || spec->depth > SVO_MAX_DEPTH) return SVO_ERR_INVALID_ARGUMENT;
    Terrain t(*spec);
    size_t k = 0;
    bool write = x && y && z && rgba;
    auto emit = [&](uint32_t vx, uint32_t vy, uint32_t vz, uint32_t c) {
        if (write && k < cap) {
            x[k] = vx;
            y[k] = vy;
            z[k] = vz;
            rgba[k] = c;
        }
        ++k;
    };
    t.for_each_voxel(spec->shell != 0, emit);
    t.for_each_box_voxel(spec->boxes, emit);
    *n = k;
    return (write && k > cap) ? SVO_ERR_CAPACITY : SVO_OK;
}

svo_status svo_view_from_euler(float rx, float ry, float rz, const float pos[3], int res_x, int res_y, float fov,
                               svo_view* out) {
    if (!pos || !out) return SVO_ERR_INVALID_ARGUMENT;
    float m[16];
    identity(m);
    double s, c;
    sincos_det(rz, s, c);
    rot_z(m, (float)c, (float)s);
    sincos_det(rx, s, c);
    rot_x(m, (float)c, (float)s);
    sincos_det(ry, s, c);
    rot_y(m, (float)c, (float)s);
    fill_view(out, pos, m, res_x, res_y, fov);
    return SVO_OK;
}

svo_status svo_view_look_at(const float pos[3], const float target[3], int res_x, int res_y, float fov,
                            svo_view* out) {
    if (!pos || !target || !out) return SVO_ERR_INVALID_ARGUMENT;
    double f[3] = {(double)target[0] - pos[0], (double)target[1] - pos[1], (double)target[2] - pos[2]};
    double len = std::sqrt(f[0] * f[0] + f[1] * f[1] + f[2] * f[2]);
    if (!(len > 0)) return SVO_ERR_INVALID_ARGUMENT;
    for (double& v : f) v /= len;
    // Row 2 of I.rotate_x(a).rotate_y(b) is (cos a sin b, -sin a, cos a cos b).
    double cx = std::sqrt(f[0] * f[0] + f[2] * f[2]);
    double sx = -f[1];
    double cy = cx > 0 ? f[2] / cx : 1.0, sy = cx > 0 ? f[0] / cx : 0.0;
    float m[16];
    identity(m);
    rot_x(m, (float)cx, (float)sx);
    rot_y(m, (float)cy, (float)sy);
    fill_view(out, pos, m, res_x, res_y, fov);
    return SVO_OK;
}

svo_status svo_wrap_position(float pos[3], int depth) {
    if (!pos || depth < 1 || depth > 20) return SVO_ERR_INVALID_ARGUMENT;
    const float dim2 = (float)(1u << (depth + 1));  // octree_dim*2 (src/raycast.h:138-143)
    for (int a = 0; a < 3; ++a) {
        float p = pos[a] * 16.0f;
        while (p < 0) p += dim2;
        while (p >= dim2) p -= dim2;
        pos[a] = p / 16.0f;
    }
    return SVO_OK;
}

svo_status svo_camera_path(int kind, int depth, int frame, uint32_t seed, int res_x, int res_y, float fov,
                           svo_view* out) {
    if (!out || depth < SVO_MIN_DEPTH || depth > SVO_MAX_DEPTH) return SVO_ERR_INVALID_ARGUMENT;
    const double E = (double)(1u << (depth + 1)) / 16.0;  // extent in world units
    const double pi = 3.14159265358979323846;
    const double cx = 0.5 * E, cy = 0.35 * E, cz = 0.5 * E;
    double px, py, pz, tx = cx, ty = cy, tz = cz;
    switch (kind) {
        case 0: {
            double el = 20.0 * pi / 180.0, s, c;
            sincos_det(el, s, c);
            double ys, yc;
            sincos_det(0.3, ys, yc);
            px = cx + 1.5 * E * c * yc;
            pz = cz + 1.5 * E * c * ys;
            py = cy + 1.5 * E * s;
            break;
        }
        case 1: {
            double yaw = 0.5 * pi / 180.0 * frame, s, c, hs, hc;
            sincos_det(yaw, s, c);
            sincos_det(2.0 * pi * (frame % 64) / 64.0, hs, hc);
            px = cx + 1.5 * E * c;
            pz = cz + 1.5 * E * s;
            py = 0.8 * E + 0.02 * E * hs;
            ty = 0.45 * E;
            break;
        }
        case 2: {
            double yaw = 2.0 * pi / 180.0 * frame, s, c, hs, hc;
            sincos_det(yaw, s, c);
            sincos_det(2.0 * pi * (frame % 64) / 64.0, hs, hc);
            double along = 0.05 * E * frame;
            px = cx + 0.9 * E * c + along;
            pz = cz + 0.9 * E * s;
            py = 0.75 * E + 0.02 * E * hs;
            tx = cx + along;
            ty = 0.4 * E;
            break;
        }
        case 3: {
            uint32_t h0 = hash32(seed, 0x5eedu, (uint32_t)frame, 0), h1 = hash32(seed, 0x5eedu, (uint32_t)frame, 1);
            uint32_t h2 = hash32(seed, 0x5eedu, (uint32_t)frame, 2), h3 = hash32(seed, 0x5eedu, (uint32_t)frame, 3);
            double yaw = (h0 & 0xffffff) / 16777216.0 * 2.0 * pi, s, c;
            sincos_det(yaw, s, c);
            double r = E * (0.6 + 1.2 * ((h1 & 0xffff) / 65536.0));
            px = cx + r * c;
            pz = cz + r * s;
            py = E * (0.72 + 0.2 * ((h2 & 0xffff) / 65536.0));
            tx = cx + E * 0.4 * ((double)(h3 & 0xff) / 255.0 - 0.5);
            tz = cz + E * 0.4 * ((double)((h3 >> 8) & 0xff) / 255.0 - 0.5);
            ty = E * (0.3 + 0.1 * ((h3 >> 16) & 0xff) / 255.0);
            break;
        }
        default:
            return SVO_ERR_INVALID_ARGUMENT;
    }
    float pos[3] = {(float)px, (float)py, (float)pz};
    float tgt[3] = {(float)tx, (float)ty, (float)tz};
    svo_status st = svo_view_look_at(pos, tgt, res_x, res_y, fov, out);
    if (st != SVO_OK) return st;
    // The reference keeps the camera inside the periodic volume (src/raycast.h:136-145).
    svo_wrap_position(out->pos, depth);
    return SVO_OK;
}

svo_status svo_rle4_voxels(const char* path, int palette, uint32_t addx, uint32_t addy, uint32_t addz, uint32_t* x,
                           uint32_t* y, uint32_t* z, uint32_t* rgba, size_t cap, size_t* n) {
    if (!path || !n) return SVO_ERR_INVALID_ARGUMENT;
    Rle4Map m;
    std::string why;
    if (!rle4_read(path, m, why)) return SVO_ERR_IO;
    size_t k = 0;
    const bool write = x && y && z && rgba;
    rle4_voxels(m, palette, addx, addy, addz, [&](uint32_t vx, uint32_t vy, uint32_t vz, uint32_t c) {
        if (write && k < cap) {
            x[k] = vx;
            y[k] = vy;
            z[k] = vz;
            rgba[k] = c;
        }
        ++k;
    });
    *n = k;
    return (write && k > cap) ? SVO_ERR_CAPACITY : SVO_OK;
}

svo_status svo_rle4_build(svo_builder* b, const char* path, int palette, uint32_t addx, uint32_t addy, uint32_t addz) {
    if (!b || !path || b->finished) return SVO_ERR_INVALID_ARGUMENT;
    Rle4Map m;
    std::string why;
    if (!rle4_read(path, m, why)) return SVO_ERR_IO;
    const uint32_t D = 1u << b->depth;
    bool inside = true;
    rle4_voxels(m, palette, addx, addy, addz, [&](uint32_t vx, uint32_t vy, uint32_t vz, uint32_t c) {
        if (vx >= D || vy >= D || vz >= D) {
            inside = false;
            return;
        }
        b->keys.push_back(morton3(vx, vy, vz));
        b->rgba.push_back(c);
    });
    return inside ? SVO_OK : SVO_ERR_CAPACITY;
}

svo_status svo_write_bmp(const char* path, const uint32_t* bgrx, int width, int height) {
    if (!path || !bgrx || width < 1 || height < 1 || (int64_t)width * height > (1ll << 28))
        return SVO_ERR_INVALID_ARGUMENT;
    FILE* f = std::fopen(path, "wb");
    if (!f) return SVO_ERR_IO;
    const uint32_t image = (uint32_t)width * (uint32_t)height * 4u;
    unsigned char h[54] = {'B', 'M'};
    auto put32 = [&](int at, uint32_t v) {
        for (int i = 0; i < 4; ++i) h[at + i] = (unsigned char)(v >> (8 * i));
    };
    put32(2, 54u + image);
    put32(10, 54u);
    put32(14, 40u);
    put32(18, (uint32_t)width);
    put32(22, (uint32_t)height);
    h[26] = 1;
    h[28] = 32;
    put32(34, image);
    bool ok = std::fwrite(h, 1, 54, f) == 54;
    // BMP rows run bottom-up; the frame's row 0 is the top of the image.
    for (int yy = height - 1; ok && yy >= 0; --yy)
        ok = std::fwrite(bgrx + (size_t)yy * width, 4, (size_t)width, f) == (size_t)width;
    ok = (std::fclose(f) == 0) && ok;
    return ok ? SVO_OK : SVO_ERR_IO;
}

}  // extern "C"
