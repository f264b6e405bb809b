// svo_oracle.cpp -- CPU restatement of the reference's sparse-voxel-octree
// raycast + warp path (sp4cerat/Sparse-Voxel-Octree-Raycasting).
//
// TEST INFRASTRUCTURE. This file is the oracle: the parity tests, smoke() and
// the CPU-baseline leg of bench.py are the only users. The product library
// never links or calls it. It restates, in plain C++, what these reference
// sources compute:
//   src/octree/octree.h:32-89    set_voxel (pointer octree, first-voxel colours)
//   src/octree/octree.h:95-191   convert_tree (6-level byte-packed blocks)
//   src/octree/octree.h:232-293  convert_tree_blocks (10-word normal nodes)
//   kernel/kernel.cl:23-112      get_bitcount, fetchChildOffset, fetchColor
//   kernel/kernel.cl:114-214     CAST_RAY
//   kernel/kernel.cl:234-340     raycast_counthole / sumids / writeids
//   kernel/kernel.cl:404-470     raycast_fillhole2
//   kernel/kernel.cl:472-592     raycast_proj
//   kernel/kernel.cl:594-694     raycast_holes
//   kernel/kernel.cl:846-942     raycast_fine_2
//   kernel/kernel.cl:944-974     raycast_colorize
//   src/raycast.h:13-46,147-441  octree_init and the per-frame call sequence
//
// Arithmetic is strict IEEE binary32 (built with -ffp-contract=off). Where the
// reference is racy on a GPU, this file fixes one deterministic meaning:
//   * raycast_proj: targets take the source with the smallest depth key
//     int(z*1000)<<8, ties to the first source in (plane, row, column) order
//     -- the result of running the work-items one after another;
//   * raycast_fillhole2: every pixel reads the image as it was before the
//     filter (snapshot / Jacobi order).
// Its agreement with the reference's own kernel.cl and octree.h, compiled for
// the host (oracle/_ref), is checked by the CPU test suite.
#include <omp.h>

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

namespace {

constexpr uint32_t kEmpty = 0xffffff00u;        // cleared pixel (raycast.h:153,157)
constexpr float kViewDistMax = 400000.0f;       // VIEW_DIST_MAX, kernel.cl:15
constexpr int kHoleThreshold = 4;               // HOLE_PIXEL_THRESHOLD, kernel.cl:21
constexpr size_t kDefaultInitialWords = 2097152;  // raycast.h:38

inline uint32_t popc8(uint32_t v) { return (uint32_t)__builtin_popcount(v & 0xffu); }

// ---------------------------------------------------------------- builder --
// octree.h:4-8: 8 child words plus the colour of the first voxel inserted
// through the node. A child word is (node_index<<8)|child_mask; at the last
// level it is the leaf's raw colour word.
struct PtrNode {
    uint32_t child[8];
    uint32_t colour;
};

struct PtrOctree {
    int depth;
    uint32_t root_mask = 0;         // octree_root (octree.h:24)
    std::vector<PtrNode> nodes;     // octree_array; node 0 is the root (raycast.h:15-17)
    bool overflow = false;          // more than 2^24 nodes: the <<8 index of octree.h:78 would wrap

    explicit PtrOctree(int d) : depth(d) { nodes.push_back(PtrNode{{0, 0, 0, 0, 0, 0, 0, 0}, 0}); }

    // octree.h:32-89
    void set_voxel(uint32_t x, uint32_t y, uint32_t z, uint32_t colour) {
        uint32_t offset = 0, parent_offset = 0, parent_bit = 0, bit_index = 0;
        for (int bit = depth - 1;; --bit) {
            parent_bit = bit_index;
            bit_index = ((x >> bit) & 1u) | (((y >> bit) & 1u) << 1) | (((z >> bit) & 1u) << 2);
            uint32_t existing = nodes[offset >> 8].child[bit_index];
            if (bit < depth - 1)
                nodes[parent_offset >> 8].child[parent_bit] |= 1u << bit_index;
            else
                root_mask |= 1u << bit_index;
            if (bit == 0) {
                nodes[offset >> 8].child[bit_index] = colour;
                return;
            }
            parent_offset = offset;
            if (existing == 0) {
                if (nodes.size() >= (1u << 24)) {
                    overflow = true;
                    return;
                }
                uint32_t fresh = (uint32_t)nodes.size() << 8;
                nodes[offset >> 8].child[bit_index] = fresh;
                nodes.push_back(PtrNode{{0, 0, 0, 0, 0, 0, 0, 0}, colour});
                offset = fresh;
            } else {
                offset = existing;
            }
        }
    }
};

struct Compactor {
    const PtrOctree& t;
    std::vector<uint32_t> out;
    uint32_t normal_cursor = 0;  // octree_normal_offset (octree.h:204)

    Compactor(const PtrOctree& tree, size_t initial_words) : t(tree), out(initial_words, 0u) {}

    // octree.h:95-191. `level` counts from 1 at the root (the reference's
    // _iteration); the byte-packed record sits at level depth-1 (rekursion 2).
    uint32_t block_node(uint32_t ptr, uint32_t local_root, int level) {
        const PtrNode& node = t.nodes[ptr >> 8];
        if (level == t.depth - 1) {
            uint32_t word_pos = (uint32_t)out.size();
            std::vector<uint8_t> bytes;
            bytes.push_back((uint8_t)node.colour);
            for (int j = 0; j < 8; ++j)
                if (node.child[j] > 0) bytes.push_back((uint8_t)node.child[j]);  // leaf-parent masks
            for (int j = 0; j < 8; ++j) {
                if (node.child[j] == 0) continue;
                const PtrNode& lp = t.nodes[node.child[j] >> 8];
                for (int i = 0; i < 8; ++i)
                    if (lp.child[i] > 0) bytes.push_back((uint8_t)lp.child[i]);  // leaf colour bytes
            }
            for (size_t i = 0; i < bytes.size(); i += 4) {
                uint32_t w = 0;
                for (size_t b = 0; b < 4 && i + b < bytes.size(); ++b) w |= (uint32_t)bytes[i + b] << (8 * b);
                out.push_back(w);
            }
            return ((word_pos - local_root) << 9) + 256u + (ptr & 0xffu);
        }
        uint32_t child_words[8];
        for (int j = 0; j < 8; ++j)
            child_words[j] = node.child[j] > 0 ? block_node(node.child[j], local_root, level + 1) : 0u;
        uint32_t pos = (uint32_t)out.size();
        out.push_back(node.colour);
        for (int j = 0; j < 8; ++j)
            if (child_words[j] > 0) out.push_back(child_words[j]);
        return ((pos - local_root) << 9) + 256u + (ptr & 0xffu);
    }

    // octree.h:232-293
    uint32_t normal_node(uint32_t ptr, int level) {
        const PtrNode& node = t.nodes[ptr >> 8];
        uint32_t child_words[8];
        for (int j = 0; j < 8; ++j) {
            uint32_t c = node.child[j];
            child_words[j] = c;
            if (c == 0) continue;
            if (level < t.depth - 6) {
                child_words[j] = normal_node(c, level + 1);
            } else {
                uint32_t local_root = (uint32_t)((out.size() + 63) / 64 * 64);
                uint32_t entries = popc8(c) + 1;
                out.resize(local_root + entries, 0u);
                child_words[j] = ((local_root >> 6) << 9) | (1u << 8) | (c & 0xffu);
                uint32_t sub_root = block_node(c, local_root, level + 1) >> 9;
                // The block root was emitted last (post-order); move it to the
                // reserved slot in front and drop the tail copy.
                for (uint32_t i = 0; i < entries; ++i) out[local_root + i] = out[local_root + sub_root + i];
                out.resize(local_root + sub_root);
            }
        }
        uint32_t at = normal_cursor;
        for (int j = 0; j < 8; ++j) out[at + j] = child_words[j];
        out[at + 8] = node.colour;
        out[at + 9] = node.colour;
        normal_cursor += 10;
        return (at << 9) | (ptr & 0xffu);
    }
};

// ------------------------------------------------------------- traversal --
struct View {
    float pos[3];
    float vx[3], vy[3], vz[3];  // rows of m: raycast_proj's a_mx/a_my/a_mz (raycast.h:160-162)
    float mx[3], my[3], mz[3];  // rows of m^T: the ray kernels' a_mx/a_my/a_mz (raycast.h:322-325)
};

View make_view(const float* pos4, const float* m) {
    View v;
    for (int i = 0; i < 3; ++i) {
        v.pos[i] = pos4[i];
        v.vx[i] = m[0 + i];
        v.vy[i] = m[4 + i];
        v.vz[i] = m[8 + i];
        v.mx[i] = m[4 * i + 0];
        v.my[i] = m[4 * i + 1];
        v.mz[i] = m[4 * i + 2];
    }
    return v;
}

// dot() as the reference's kernels evaluate it: left to right, no fusion.
inline float dot3(const float* a, const float* b) {
    float s = a[0] * b[0];
    s = s + a[1] * b[1];
    s = s + a[2] * b[2];
    return s;
}

struct Ray {
    uint32_t colour;   // the word stored to the screen buffer: 0xff000000 + fetched colour
    float hit[3];      // raypos/16 after the walk (kernel.cl:675,920)
    float dist;        // accumulated distance / 16 (world units)
    uint64_t voxel;    // packed hit cell, see encode_voxel
    uint32_t child_fetches, colour_fetches, steps;
    bool boundary;     // a non-stepping coordinate landed within 1 ulp of an integer
    bool hit_boundary; // the hit point lies within 1 ulp of a face of its hit cell (other than the entry face)
    int level;         // level of the hit cell (its edge is 2^level raypos units), -1 without a hit
    uint32_t signs;    // the ray's direction signs, bit a set when component a < 0
};

struct Tracer {
    const uint32_t* oct;
    size_t n_words;
    uint32_t root;
    int depth;

    uint32_t load(uint32_t i, uint32_t& counter) const {
        ++counter;
        return i < n_words ? oct[i] : 0u;
    }

    // kernel.cl:32-62. Returns the child word; at rekursion 1 the reference
    // reads a word nothing uses (see trace), so that read is not counted.
    uint32_t fetch_child(uint32_t node, uint32_t before, uint32_t& local_root, uint32_t child, uint32_t child_test,
                         int rek, uint32_t& cnt) const {
        uint32_t n = node >> 9, nadd = child;
        if (node & 256u) {
            if (!(before & 256u)) {
                local_root = n << 6;
                n = 0;
            }
            n += local_root;
            nadd = popc8(node & ((child_test << 1) - 1u));
            if (rek == 2) return ((load(n + (nadd >> 2), cnt) >> ((nadd & 3u) << 3)) & 255u) + 256u + (nadd << 9);
            if (rek == 1) return 0u;  // value unused: the walk always stops at rekursion 1
        }
        return load(n + nadd, cnt);
    }

    // kernel.cl:64-112
    uint32_t fetch_colour(uint32_t node, uint32_t before, uint32_t before2, uint32_t& local_root, int rek,
                          uint32_t child_test, uint32_t& cnt) const {
        uint32_t n = node >> 9, nadd = 8;
        if (rek == 1) {
            n = (before >> 9) & 15u;
            uint32_t ofs = (before2 >> 9) + local_root;
            nadd = popc8(before2 & 255u);
            for (uint32_t i = 1; i < n; ++i) nadd += popc8(load(ofs + (i >> 2), cnt) >> ((i & 3u) << 3));
            nadd += popc8(before & ((child_test << 1) - 1u));
            return load(ofs + (nadd >> 2), cnt) >> ((nadd & 3u) << 3);
        }
        if (node & 256u) {
            if (!(before & 256u)) {
                local_root = n << 6;
                n = 0;
            }
            nadd = local_root;
            if (rek == 2) {
                uint32_t ofs = (before >> 9) + local_root;
                nadd = 1 + popc8(before & 255u);
                for (uint32_t i = 1; i < n; ++i) nadd += popc8(load(ofs + (i >> 2), cnt) >> ((i & 3u) << 3));
                return load(ofs + (nadd >> 2), cnt) >> ((nadd & 3u) << 3);
            }
        }
        return load(n + nadd, cnt);
    }

    // Within one ulp of a leaf-cell face (a multiple of 2 in raypos units).
    static bool near_face(float c) {
        float r = 2.0f * std::nearbyint(c * 0.5f);
        float d = std::fabs(c - r);
        float ulp = std::nextafter(std::fabs(c), INFINITY) - std::fabs(c);
        return d <= ulp;
    }

    // Ray setup of raycast_fine_2 / raycast_holes (kernel.cl:883-899, 639-655)
    // followed by CAST_RAY (kernel.cl:114-214) and the colour fetch (:911-921).
    // s0 > 0 (the product's guided walks, not in the reference): the walk
    // starts s0 raypos units along the ray -- at most up to 16 units before
    // the ray leaves the volume's height -- at camera + s0 * (1, g0y, g0z)/len0
    // in the mirrored frame, with the distance at s0 and the level of detail
    // advanced over the lodswitch doublings below s0 (at most to the depth).
    Ray trace(const View& v, int idx, int idy, int res_x, int res_y, float fovx, float fovy, float s0 = 0.0f) const {
        Ray r{};
        const int scale_max = 1 << (depth + 1);
        const int depth_and = (1 << depth) - 1;
        float d1[3];
        d1[0] = (float)((double)(idx - res_x / 2) + 0.5) * fovx / (float)res_y;
        d1[1] = (float)((double)(idy - res_y / 2) + 0.5) * fovy / (float)res_y;
        d1[2] = 1.0f;
        float d[3] = {dot3(d1, v.mx), dot3(d1, v.my), dot3(d1, v.mz)};
        float rp[3] = {v.pos[0] * 16.0f, v.pos[1] * 16.0f, v.pos[2] * 16.0f};

        const float eps = 1.0f / 1048576.0f;  // pow(2,-20), kernel.cl:118
        int sgn[3] = {0, 0, 0};
        for (int a = 0; a < 3; ++a) {
            if (std::fabs(d[a]) < eps) d[a] = (d[a] > 0.0f ? 1.0f : (d[a] < 0.0f ? -1.0f : d[a])) * eps;
        }
        for (int a = 0; a < 3; ++a) {
            if (d[a] < 0.0f) {
                sgn[a] = 1;
                rp[a] = (float)scale_max - rp[a];
                d[a] = -d[a];
            }
        }
        // grad0/1/2 (kernel.cl:127-137) and their lengths (:139-141)
        float g[3][3] = {{1.0f, d[1] / d[0], d[2] / d[0]},
                         {d[0] / d[1], 1.0f, d[2] / d[1]},
                         {d[0] / d[2], d[1] / d[2], 1.0f}};
        float len[3];
        for (int a = 0; a < 3; ++a) len[a] = std::sqrt(dot3(g[a], g[a]));

        int lod = 1;
        float lodswitch = (float)(res_x * 1 * 2);  // LOD_ADJUST=1, kernel.cl:908
        float distance = 0.0f;
        if (s0 > 0.0f) {  // not past the ray's exit through the volume's top (16 raypos units margin)
            const float t_top = ((float)scale_max - rp[1]) * len[1];
            s0 = std::fmin(s0, t_top - 16.0f);
        }
        if (s0 > 0.0f) {  // unit direction (1, g0y, g0z) / len[0]
            const float ux = 1.0f / len[0];
            const float u[3] = {ux, g[0][1] * ux, g[0][2] * ux};
            for (int a = 0; a < 3; ++a) rp[a] = rp[a] + u[a] * s0;
            distance = s0;
            while (distance > lodswitch && lod < depth) {
                lodswitch *= 2.0f;
                ++lod;
            }
        }
        int rpi[3] = {(int)rp[0], (int)rp[1], (int)rp[2]};
        int rek = depth;
        uint32_t nodeid = root, nodeid_before = root, local_root = 0, node_test = 0;
        uint32_t sign_xyz = (uint32_t)(sgn[0] | (sgn[1] << 1) | (sgn[2] << 2));
        int x0ry = 0;
        uint32_t stack[20];  // stack[level]; stack[depth] and above stand for the root
        for (int i = 0; i < 20; ++i) stack[i] = root;
        bool hit = false;
        int hit_cell[3] = {0, 0, 0};
        int last_axis = -1;  // axis of the last step (the hit cell's entry face)
        const uint32_t step_cap = 1u << 22;

        do {
            if (++r.steps > step_cap) break;
            int p0i[3] = {rpi[0] >> rek, rpi[1] >> rek, rpi[2] >> rek};
            uint32_t node_index = ((uint32_t)(p0i[0] & 1) | ((uint32_t)(p0i[1] & 1) << 1) |
                                   ((uint32_t)(p0i[2] & 1) << 2)) ^ sign_xyz;
            node_test = nodeid & (1u << node_index);
            if (node_test) {
                uint32_t parent = nodeid;
                nodeid = fetch_child(nodeid, nodeid_before, local_root, node_index, node_test, rek, r.child_fetches);
                nodeid_before = parent;
                if (rek <= lod) {
                    hit = true;
                    for (int a = 0; a < 3; ++a) hit_cell[a] = p0i[a];
                    const float cell = (float)(1 << rek);
                    for (int a = 0; a < 3; ++a) {
                        if (a == last_axis) continue;
                        const float c = rp[a], f = cell * std::nearbyint(c / cell);
                        if (std::fabs(c - f) <= std::nextafter(std::fabs(c), INFINITY) - std::fabs(c))
                            r.hit_boundary = true;
                    }
                    break;
                }
                --rek;
                stack[rek] = nodeid;
                continue;
            }
            float mul0[3];
            for (int a = 0; a < 3; ++a) mul0[a] = (float)((p0i[a] + 1) << rek) - rp[a];
            int before[3] = {rpi[0], rpi[1], rpi[2]};
            float isec_dist[3] = {mul0[0] * len[0], mul0[1] * len[1], mul0[2] * len[2]};
            int axis = 0;
            if (isec_dist[1] < isec_dist[axis]) axis = 1;
            if (isec_dist[2] < isec_dist[axis]) axis = 2;
            last_axis = axis;
            for (int a = 0; a < 3; ++a) rp[a] = rp[a] + g[axis][a] * mul0[axis];
            for (int a = 0; a < 3; ++a) {
                rpi[a] = (int)rp[a];
                if (a != axis && near_face(rp[a])) r.boundary = true;
            }
            distance = distance + isec_dist[axis];
            int x0rx = before[0] ^ rpi[0];
            x0ry = before[1] ^ rpi[1];
            int x0rz = before[2] ^ rpi[2];
            uint32_t x0r = (uint32_t)((x0rx ^ x0ry ^ x0rz) & depth_and);
            // log2(float(x0r)) truncated (kernel.cl:202) is the index of the top set bit.
            int rek_new = x0r ? 31 - __builtin_clz(x0r) : -1;
            if (distance > kViewDistMax) break;
            if (rek_new < rek) continue;
            rek = rek_new + 1;
            nodeid = stack[rek];
            nodeid_before = stack[rek + 1];
            if (rek == depth) nodeid_before = nodeid = root;
            if (distance > lodswitch) {
                lodswitch *= 2.0f;
                ++lod;
            }
        } while (!(x0ry & (2 * depth_and + 2)));

        for (int a = 0; a < 3; ++a)
            if (sgn[a]) rp[a] = (float)scale_max - rp[a];
        uint32_t col = fetch_colour(nodeid, nodeid_before, stack[rek + 1], local_root, rek, node_test, r.colour_fetches);
        r.colour = 0xff000000u + col;
        for (int a = 0; a < 3; ++a) r.hit[a] = rp[a] / 16.0f;
        r.dist = distance / 16.0f;
        if (hit) {
            // Packed hit cell: voxel coordinates of the cell's low corner, in the
            // unmirrored frame, wrapped to one period; level in bits 48-55;
            // bit 63 marks a hit.
            uint64_t key = (uint64_t)1 << 63 | (uint64_t)(uint32_t)rek << 48;
            uint32_t cells = (uint32_t)scale_max >> rek;
            for (int a = 0; a < 3; ++a) {
                uint32_t c = (uint32_t)hit_cell[a];
                if (sgn[a]) c = cells - 1u - c;
                c &= cells - 1u;
                uint32_t vox = (c << rek) >> 1;
                key |= (uint64_t)(vox & 0xffffu) << (16 * a);
            }
            r.voxel = key;
        }
        r.level = hit ? rek : -1;
        r.signs = sign_xyz;
        return r;
    }
};

// -------------------------------------------------------------- colourise --
// kernel.cl:944-974
inline uint32_t colorize(uint32_t word) {
    static const float tab[4][3] = {{1.0f, 1.0f, 1.0f}, {1.0f, 0.7f, 0.3f}, {1.5f, 0.8f, 0.1f}, {0.2f, 0.8f, 0.2f}};
    int a = (int)word;
    const float* rgb = tab[a & 3];
    float i = (float)(a & (255 - 7));
    int r = (int)(i * rgb[0]);
    if (r > 255) r = 255;
    int g = (int)(i * rgb[1]);
    if (g > 255) g = 255;
    int b = (int)(i * rgb[2]);
    if (b > 255) b = 255;
    return (uint32_t)(b + g * 256 + r * 65536);
}

// ------------------------------------------------------------------ frame --
struct Warp {
    int res_x, res_y;
    size_t N, tiles;
    std::vector<uint32_t> screen;   // 4 colour planes, stride N (raycast.h:85)
    std::vector<float> back;        // 4 float4 planes (raycast.h:82)
    std::vector<uint32_t> ids;      // counts | prefix | hole list (raycast.h:268-270)
    std::vector<uint32_t> tex;      // colourised BGRX
    std::vector<uint32_t> prefill;  // plane 0 before the hole filter
    std::vector<uint64_t> keys;     // per-target depth|source keys for raycast_proj
    uint32_t hole_count = 0;
    uint64_t rays = 0, child_fetches = 0, colour_fetches = 0, boundary_rays = 0;
};

inline void store_ray_plane(uint32_t* col, float* xyz, size_t ofs, const Ray& r) {
    col[ofs] = r.colour;
    xyz[ofs * 4 + 0] = r.hit[0];
    xyz[ofs * 4 + 1] = r.hit[1];
    xyz[ofs * 4 + 2] = r.hit[2];
    xyz[ofs * 4 + 3] = r.dist;
}

inline void store_ray(Warp& w, size_t ofs, const Ray& r) {
    w.screen[ofs] = r.colour;
    w.back[ofs * 4 + 0] = r.hit[0];
    w.back[ofs * 4 + 1] = r.hit[1];
    w.back[ofs * 4 + 2] = r.hit[2];
    w.back[ofs * 4 + 3] = r.dist;  // the reference leaves w untouched here; the contract stores the distance
}

// The screen-space x/y of raycast_proj (kernel.cl:552-553): the unsuffixed
// 0.0 literals make the division and the following add double precision.
inline int proj_coord(float num, float z, float half) {
    double v = (double)num + 0.0;
    v = v / (double)z;
    v = v + (double)half;
    v = v - 0.0;
    return (int)(float)v;
}

// raycast_proj over one cache plane (kernel.cl:472-592). Rejected source
// pixels (behind the camera or off screen) are cleared in that cache plane
// (kernel.cl:549-562), which matters for a plane that is not the copy target.
void proj_plane(Warp& w, const View& v, uint32_t plane) {
    const int res_x = w.res_x, res_y = w.res_y;
    const size_t N = w.N;
    uint32_t* src = w.screen.data() + plane * N;
    const float* sb = w.back.data() + plane * N * 4;
    std::atomic<uint64_t>* keys = reinterpret_cast<std::atomic<uint64_t>*>(w.keys.data());
#pragma omp parallel for schedule(static)
    for (long s = 0; s < (long)N; ++s) {
        uint32_t col = src[s];
        if (col == kEmpty) continue;
        float p[3] = {sb[s * 4 + 0] - v.pos[0], sb[s * 4 + 1] - v.pos[1], sb[s * 4 + 2] - v.pos[2]};
        float ph[3] = {dot3(p, v.vx), dot3(p, v.vy), dot3(p, v.vz)};
        if (ph[2] < 0.05f) {  // (double)z < 0.05 <=> z < 0.05f for binary32 z
            src[s] = kEmpty;
            continue;
        }
        int sx = proj_coord(ph[0] * (float)res_y, ph[2], (float)res_x / 2);
        int sy = proj_coord(ph[1] * (float)res_y, ph[2], (float)res_y / 2);
        if (sx >= res_x - 1 || sx < 0 || sy >= res_y - 1 || sy < 0) {
            src[s] = kEmpty;
            continue;
        }
        size_t t = (size_t)sy * res_x + sx;
        uint32_t sz = (uint32_t)(int)(ph[2] * 1000.0f) << 8;
        if (sz >= kEmpty) continue;  // cannot beat the cleared value (kernel.cl:571)
        uint64_t key = ((uint64_t)sz << 32) | (uint64_t)(plane * N + s);
        uint64_t cur = keys[t].load(std::memory_order_relaxed);
        while (key < cur && !keys[t].compare_exchange_weak(cur, key, std::memory_order_relaxed)) {
        }
    }
}

void proj_resolve(Warp& w, const View& v) {
    const size_t N = w.N;
#pragma omp parallel for schedule(static)
    for (long t = 0; t < (long)N; ++t) {
        uint64_t key = w.keys[t];
        if (key == ~0ull) continue;
        w.keys[t] = ~0ull;
        uint32_t src = (uint32_t)key;
        uint32_t sz = (uint32_t)(key >> 32);
        const float* q = w.back.data() + (size_t)src * 4;
        float p[3] = {q[0] - v.pos[0], q[1] - v.pos[1], q[2] - v.pos[2]};
        float z = dot3(p, v.vz);
        w.screen[t] = sz + (w.screen[src] & 255u);
        w.back[t * 4 + 0] = q[0];
        w.back[t * 4 + 1] = q[1];
        w.back[t * 4 + 2] = q[2];
        w.back[t * 4 + 3] = z;
    }
}

void gather_holes(Warp& w) {
    const int res_x = w.res_x, res_y = w.res_y;
    const int tx_n = res_x / 16, ty_n = res_y / 16;
    const size_t tiles = w.tiles;
    const uint32_t* s = w.screen.data();
    std::vector<uint64_t> masks(tiles, 0);
#pragma omp parallel for schedule(static)
    for (long t = 0; t < (long)tiles; ++t) {
        int x = (int)(t % tx_n) * 16, y = (int)(t / tx_n) * 16;
        uint64_t m = 0;
        for (int j = 0; j < 8; ++j)
            for (int i = 0; i < 8; ++i) {
                size_t o = (size_t)(y + 2 * j) * res_x + x + 2 * i;
                int a = (s[o] == kEmpty) + (s[o + 1] == kEmpty) + (s[o + 1 + res_x] == kEmpty) +
                        (s[o + res_x] == kEmpty);
                if (a >= kHoleThreshold) m |= 1ull << (j * 8 + i);
            }
        masks[t] = m;
        w.ids[t] = 4u * (uint32_t)__builtin_popcountll(m);  // raycast_counthole
    }
    // raycast_sumids (kernel.cl:276-296): exclusive scan, total into ids[0]
    uint32_t acc = 0;
    for (size_t t = 0; t < tiles; ++t) {
        uint32_t len = w.ids[t];
        w.ids[tiles + t] = acc;
        acc += len;
    }
    if (tiles > 0) w.ids[0] = acc;
    w.hole_count = tiles > 0 ? acc : 0;
    // raycast_writeids (kernel.cl:298-340)
#pragma omp parallel for schedule(static)
    for (long t = 0; t < (long)tiles; ++t) {
        int x = (int)(t % tx_n) * 16, y = (int)(t / tx_n) * 16;
        size_t dst = w.ids[tiles + t] + 2 * tiles;
        uint64_t m = masks[t];
        for (int b = 0; b < 64; ++b) {
            if (!(m >> b & 1)) continue;
            int i = b & 7, j = b >> 3;
            uint32_t val = (uint32_t)(x + i * 2) + ((uint32_t)(j * 2 + y) << 16);
            w.ids[dst++] = val;
            w.ids[dst++] = val + 1;
            w.ids[dst++] = val + 1 + (1u << 16);
            w.ids[dst++] = val + (1u << 16);
        }
    }
    (void)ty_n;
}

// raycast_fillhole2 (kernel.cl:404-470) with snapshot reads. `snap` holds
// plane 0 and continues into plane 1, as the reference's linear addressing does.
uint32_t fill_pixel(const uint32_t* snap, size_t lin_limit, int idx, int idy, int res_x, int res_y) {
    size_t ofs = (size_t)idy * res_x + idx;
    uint32_t col = snap[ofs];
    if (idx >= res_x - 1 || idy >= res_y - 1 || idx <= 1 || idy <= 1) return col;
    if (col != kEmpty) return col;
    int c1 = (int)snap[ofs + 1], c2 = (int)snap[ofs - 1], c3 = (int)snap[ofs + res_x], c4 = (int)snap[ofs - res_x];
    bool s1 = (uint32_t)c1 != kEmpty, s2 = (uint32_t)c2 != kEmpty, s3 = (uint32_t)c3 != kEmpty,
         s4 = (uint32_t)c4 != kEmpty;
    if (s1 && s2 && s3 && s4)
        return (uint32_t)((c1 & 3) + ((((c1 & 0xfc) + (c2 & 0xfc) + (c3 & 0xfc) + (c4 & 0xfc)) >> 2) & 0xfc));
    if (s1 && s2) return (uint32_t)((c1 & 3) + ((((c1 & 0xfc) + (c2 & 0xfc)) >> 1) & 0xfc));
    if (s3 && s4) return (uint32_t)((c3 & 3) + ((((c3 & 0xfc) + (c4 & 0xfc)) >> 1) & 0xfc));
    for (int i = 0; i < 4; ++i) {
        col = snap[ofs + (i & 1) + ((i >> 1) & 1) * res_x];
        if (col != kEmpty) break;
    }
    if (col == kEmpty) {
        // 5x5 scan, column offset outer, row offset inner; first non-empty wins.
        for (int i = -2; i < 3 && col == kEmpty; ++i)
            for (int j = -2; j < 3; ++j) {
                long o = (long)ofs + i + (long)j * res_x;
                col = (size_t)o < lin_limit ? snap[o] : kEmpty;
                if (col != kEmpty) break;
            }
    }
    return col;
}

}  // namespace

// ------------------------------------------------------------------ C API --
extern "C" {

struct OrcOctree {
    std::vector<uint32_t> words;
    uint32_t root;
    int depth;
};

// Builds the compact octree from voxels given in insertion order
// (raycast.h:13-39): pointer octree via set_voxel, then convert_tree_blocks.
int orc_octree_build(int depth, const uint32_t* x, const uint32_t* y, const uint32_t* z, const uint32_t* rgba,
                     size_t n, size_t initial_words, void** handle) {
    if (depth < 8 || depth > 16) return -1;
    if (initial_words == 0) initial_words = kDefaultInitialWords;
    PtrOctree t(depth);
    for (size_t i = 0; i < n && !t.overflow; ++i) t.set_voxel(x[i], y[i], z[i], rgba[i]);
    if (t.overflow) return -2;  // 24-bit node index (octree.h:78)
    Compactor c(t, initial_words);
    OrcOctree* o = new OrcOctree;
    o->root = c.normal_node(t.root_mask, 1);
    if ((size_t)c.normal_cursor > initial_words) {
        delete o;
        return -3;  // normal nodes would overrun the pre-sized region
    }
    o->words.swap(c.out);
    o->depth = depth;
    *handle = o;
    return 0;
}
size_t orc_octree_size(void* h) { return static_cast<OrcOctree*>(h)->words.size(); }
uint32_t orc_octree_root(void* h) { return static_cast<OrcOctree*>(h)->root; }
void orc_octree_copy(void* h, uint32_t* out) {
    auto* o = static_cast<OrcOctree*>(h);
    std::memcpy(out, o->words.data(), o->words.size() * 4);
}
void orc_octree_free(void* h) { delete static_cast<OrcOctree*>(h); }

// raycast_fine_2 over the whole frame. Outputs per pixel: colour word, float4
// (hit xyz, distance), packed hit cell and per-ray counters. Any output may be
// null. stats[0..6] = rays, child fetches, colour fetches, boundary rays (a
// step landed a coordinate within 1 ulp of a leaf face), loop iterations,
// longest walk (iterations), hit-boundary rays (the hit point within 1 ulp of
// a face of its hit cell other than the entry face).
int orc_raycast_full(int depth, const uint32_t* words, size_t n_words, uint32_t root, const float* pos4,
                     const float* m16, int res_x, int res_y, float fovx, float fovy, uint32_t* colour, float* xyzw,
                     uint64_t* voxel, uint64_t* stats, int threads) {
    if (res_x <= 0 || res_y <= 0 || res_x > 65535 || res_y > 65535) return -1;
    Tracer tr{words, n_words, root, depth};
    View v = make_view(pos4, m16);
    uint64_t child = 0, col = 0, bnd = 0, hbnd = 0, steps = 0, max_steps = 0;
    if (threads > 0) omp_set_num_threads(threads);
#pragma omp parallel for schedule(dynamic, 4) reduction(+ : child, col, bnd, hbnd, steps) reduction(max : max_steps)
    for (int y = 0; y < res_y; ++y)
        for (int x = 0; x < res_x; ++x) {
            Ray r = tr.trace(v, x, y, res_x, res_y, fovx, fovy);
            size_t o = (size_t)y * res_x + x;
            if (colour) colour[o] = r.colour;
            if (xyzw) {
                xyzw[o * 4 + 0] = r.hit[0];
                xyzw[o * 4 + 1] = r.hit[1];
                xyzw[o * 4 + 2] = r.hit[2];
                xyzw[o * 4 + 3] = r.dist;
            }
            if (voxel) voxel[o] = r.voxel;
            child += r.child_fetches;
            col += r.colour_fetches;
            bnd += r.boundary ? 1 : 0;
            hbnd += r.hit_boundary ? 1 : 0;
            steps += r.steps;
            if (r.steps > max_steps) max_steps = r.steps;
        }
    if (stats) {
        stats[0] = (uint64_t)res_x * res_y;
        stats[1] = child;
        stats[2] = col;
        stats[3] = bnd;
        stats[4] = steps;
        stats[5] = max_steps;
        stats[6] = hbnd;
    }
    return 0;
}

// Guided walks over the whole frame: pixel o starts at s0[o] raypos units
// (0: from the camera); pixels with s0[o] < 0 are not traced (outputs left
// as they are). stats (may be null): [0] rays walked, [1] child fetches,
// [2] colour fetches.
int orc_raycast_guided(int depth, const uint32_t* words, size_t n_words, uint32_t root, const float* pos4,
                       const float* m16, int res_x, int res_y, const float* s0, uint32_t* colour, float* xyzw,
                       uint64_t* stats, int threads) {
    if (res_x <= 0 || res_y <= 0 || res_x > 65535 || res_y > 65535 || !s0) return -1;
    Tracer tr{words, n_words, root, depth};
    View v = make_view(pos4, m16);
    uint64_t rays = 0, child = 0, col = 0;
    if (threads > 0) omp_set_num_threads(threads);
#pragma omp parallel for schedule(dynamic, 4) reduction(+ : rays, child, col)
    for (int y = 0; y < res_y; ++y)
        for (int x = 0; x < res_x; ++x) {
            size_t o = (size_t)y * res_x + x;
            if (s0[o] < 0.0f) continue;
            Ray r = tr.trace(v, x, y, res_x, res_y, 1.0f, 1.0f, s0[o]);
            ++rays;
            child += r.child_fetches;
            col += r.colour_fetches;
            if (colour) colour[o] = r.colour;
            if (xyzw) {
                xyzw[o * 4 + 0] = r.hit[0];
                xyzw[o * 4 + 1] = r.hit[1];
                xyzw[o * 4 + 2] = r.hit[2];
                xyzw[o * 4 + 3] = r.dist;
            }
        }
    if (stats) {
        stats[0] = rays;
        stats[1] = child;
        stats[2] = col;
    }
    return 0;
}

// Loop iterations of every guided walk (s0 as orc_raycast_guided; 0 where
// s0 < 0): the per-lane cost a model of the tracer's warps sums over.
int orc_raycast_guided_steps(int depth, const uint32_t* words, size_t n_words, uint32_t root, const float* pos4,
                             const float* m16, int res_x, int res_y, const float* s0, uint32_t* steps, int threads) {
    if (res_x <= 0 || res_y <= 0 || res_x > 65535 || res_y > 65535 || !s0 || !steps) return -1;
    Tracer tr{words, n_words, root, depth};
    View v = make_view(pos4, m16);
    if (threads > 0) omp_set_num_threads(threads);
#pragma omp parallel for schedule(dynamic, 4)
    for (int y = 0; y < res_y; ++y)
        for (int x = 0; x < res_x; ++x) {
            size_t o = (size_t)y * res_x + x;
            steps[o] = s0[o] < 0.0f ? 0u : tr.trace(v, x, y, res_x, res_y, 1.0f, 1.0f, s0[o]).steps;
        }
    return 0;
}

// ------------------------------------------------ certified reprojection --
// The product's learned frames certify a reprojected colour without a walk
// when the pixel's own ray provably meets a face a cached hit point lies on.
// Every cached point carries its hit code in w: the level L of its hit cell
// (edge s = 2^L raypos units) and the signs of the ray that found it. The hit
// point lies on the cell's entry face: exactly one of its coordinates (raypos
// units) is a multiple of s, and the old ray crossed that plane in the
// direction its sign bit gives. The pixel's ray (the ray kernels' direction,
// not normalised) meets the plane at parameter t; the candidate passes when
// the ray crosses the plane the same way, t > 0, the other two coordinates of
// the meeting point lie inside the cell's face with a margin of s/64, the
// level of detail at the meeting distance is L a thirty-second either side,
// and that distance is at most 2 cells behind the nearest reprojected point of
// the 3x3 neighbourhood (nothing cached lies in front). The candidates are
// the pixel's own cached point and its four neighbours'; the nearest passing
// one (smallest t, the first in row order on a tie) is taken: colour byte,
// meeting point, code. The tests compare cross-multiplied quantities (with n
// = |plane - camera| and A = |d along the face's axis|: t = n/A, the meeting
// distance n*|d|/A compared squared); one division is left, for the winner's
// point. Every operation is one IEEE binary32 operation, as on the GPU.
constexpr float kGuideCertified = -2.0f;

inline float hit_code(const Ray& r) { return r.level < 0 ? -1.0f : (float)(r.level | (int)(r.signs << 5)); }

struct Certified {
    uint32_t colour;
    float xyzw[4];
};

bool certify(const View& v, int res_x, int res_y, int x, int y, const uint32_t* col, const float* xyz, float near_s,
             Certified& out) {
    float d1[3];
    d1[0] = (float)((double)(x - res_x / 2) + 0.5) * 1.0f / (float)res_y;
    d1[1] = (float)((double)(y - res_y / 2) + 0.5) * 1.0f / (float)res_y;
    d1[2] = 1.0f;
    const float d[3] = {dot3(d1, v.mx), dot3(d1, v.my), dot3(d1, v.mz)};
    const float cam[3] = {v.pos[0] * 16.0f, v.pos[1] * 16.0f, v.pos[2] * 16.0f};
    const float dl2 = d[0] * d[0] + d[1] * d[1] + d[2] * d[2];
    const float sw1 = (float)(2 * res_x);
    auto pow2 = [](int e) {
        const uint32_t bits = (uint32_t)(127 + e) << 23;
        float f;
        std::memcpy(&f, &bits, 4);
        return f;
    };
    float bn = 1.0f, ba = 0.0f, bp = 0.0f;  // best t = bn / ba
    int bk = -1, baxis = 0;
    size_t bo = 0;
    // the pixel's own point and its four neighbours', in row order
    static const int kOff[5][2] = {{0, -1}, {-1, 0}, {0, 0}, {1, 0}, {0, 1}};
    for (int k = 0; k < 5; ++k) {
        const int xi = x + kOff[k][0], yj = y + kOff[k][1];
        if (xi < 0 || xi >= res_x || yj < 0 || yj >= res_y) continue;
        const size_t o = (size_t)yj * res_x + xi;
        if (col[o] == kEmpty) continue;
        const float code = xyz[o * 4 + 3];
        if (!(code >= 0.0f)) continue;
        const int ic = (int)code;
        const int L = ic & 31;
        if (L > 23) continue;
        const uint32_t sb = (uint32_t)ic >> 5;
        const float cs = pow2(L), inv = pow2(-L);
        float p[3], f[3];
        int axis = -1, on = 0;
        for (int a = 0; a < 3; ++a) {
            p[a] = xyz[o * 4 + a] * 16.0f;
            f[a] = std::floor(p[a] * inv);
            if (f[a] * cs == p[a]) {
                axis = a;
                ++on;
            }
        }
        if (on != 1) continue;
        const float da = d[axis];
        const bool neg = ((sb >> axis) & 1u) != 0;
        if (neg ? !(da < 0.0f) : !(da > 0.0f)) continue;
        const float num = p[axis] - cam[axis];
        const float n = neg ? -num : num, A = neg ? -da : da;  // t = n / A
        if (!(n > 0.0f)) continue;
        if (!(n * ba < bn * A)) continue;
        // the meeting distance n*|d|/A: gap and level-of-detail tests squared
        const float nd2 = (n * n) * dl2;
        const float gap = (near_s + 2.0f * cs) * A;
        if (!(nd2 <= gap * gap)) continue;
        const float swl = (sw1 * pow2(L - 1)) * A;
        if (!(nd2 * 1.0634765625f <= swl * swl)) continue;  // (1 + 1/32)^2
        if (L > 1) {
            const float swm = (sw1 * pow2(L - 2)) * A;
            if (!(nd2 * 0.9384765625f > swm * swm)) continue;  // (1 - 1/32)^2
        }
        bool inside = true;
        for (int b2 = 0; b2 < 3; ++b2) {
            if (b2 == axis) continue;
            const float u = (cam[b2] - f[b2] * cs) * A + n * d[b2];
            const float sa = cs * A;
            inside = inside && u > sa * 0.015625f && u < sa * 0.984375f;
        }
        if (!inside) continue;
        bn = n;
        ba = A;
        bk = k;
        baxis = axis;
        bp = p[axis];
        bo = o;
    }
    if (bk < 0) return false;
    const int L = (int)xyz[bo * 4 + 3] & 31;
    const float t = bn / ba;
    const uint32_t signs = (d[0] < 0.0f ? 1u : 0u) | (d[1] < 0.0f ? 2u : 0u) | (d[2] < 0.0f ? 4u : 0u);
    out.colour = 0xff000000u | (col[bo] & 255u);
    for (int b2 = 0; b2 < 3; ++b2) out.xyzw[b2] = (b2 == baxis ? bp : cam[b2] + t * d[b2]) * 0.0625f;
    out.xyzw[3] = (float)(L | (int)(signs << 5));
    return true;
}

// Guided learned frames with every unguided pixel traced: the product's
// svo_warp_frame_learned on a guided target with a confidence threshold no
// pixel reaches (the net then decides nothing; the reference has no such
// frame). Two planes: the frame's plane and the last frame's, whose points are
// reprojected after re-basing them by whole periods of the volume (the camera
// wraps into it, src/raycast.h:136-145); then the start distances, then rays
// from the camera for the refresh tile and the unguided pixels and walks for
// the rest. Test infrastructure for the product's guided frames.
struct Guided {
    int res_x = 0, res_y = 0, depth = 0;
    size_t N = 0;
    std::vector<uint32_t> col[2];
    std::vector<float> xyz[2];
    std::vector<uint64_t> keys;
    std::vector<float> guide;
    float cache_pos[3] = {0, 0, 0};
    int cache = -1;  // plane holding the last frame, -1 before the first frame
    bool certify = false;
};

void* orc_guided_create(int depth, int res_x, int res_y) {
    if (res_x < 16 || res_y < 16 || res_x > 65535 || res_y > 65535 || depth < 1 || depth > 20) return nullptr;
    Guided* g = new Guided;
    g->res_x = res_x;
    g->res_y = res_y;
    g->depth = depth;
    g->N = (size_t)res_x * res_y;
    for (int i = 0; i < 2; ++i) {
        g->col[i].assign(g->N, kEmpty);
        g->xyz[i].assign(g->N * 4, 0.0f);
    }
    g->keys.assign(g->N, ~0ull);
    g->guide.assign(g->N, -1.0f);
    return g;
}
void orc_guided_free(void* h) { delete static_cast<Guided*>(h); }
void orc_guided_set_certify(void* h, int enable) { static_cast<Guided*>(h)->certify = enable != 0; }
const uint32_t* orc_guided_colour(void* h) {
    Guided* g = static_cast<Guided*>(h);
    return g->col[g->cache < 0 ? 0 : g->cache].data();
}
const float* orc_guided_coords(void* h) {
    Guided* g = static_cast<Guided*>(h);
    return g->xyz[g->cache < 0 ? 0 : g->cache].data();
}
const float* orc_guided_guide(void* h) { return static_cast<Guided*>(h)->guide.data(); }

int orc_guided_frame(void* h, const uint32_t* words, size_t n_words, uint32_t root, const float* pos4,
                     const float* m16, int frame, int threads) {
    Guided& g = *static_cast<Guided*>(h);
    const int res_x = g.res_x, res_y = g.res_y;
    const size_t N = g.N;
    View v = make_view(pos4, m16);
    Tracer tr{words, n_words, root, g.depth};
    if (threads > 0) omp_set_num_threads(threads);
    const bool have_cache = frame >= 2 && g.cache >= 0;
    const int cur = g.cache == 0 ? 1 : 0;
    std::vector<uint32_t>& col = g.col[cur];
    std::vector<float>& xyz = g.xyz[cur];
    std::fill(col.begin(), col.end(), kEmpty);
    if (have_cache) {
        const std::vector<uint32_t>& sc = g.col[g.cache];
        const std::vector<float>& sx = g.xyz[g.cache];
        const float period = (float)(1u << (g.depth + 1)) / 16.0f;
        float shift[3];
        for (int i = 0; i < 3; ++i)
            shift[i] = (float)std::nearbyint(((double)v.pos[i] - (double)g.cache_pos[i]) / period) * period;
        std::atomic<uint64_t>* keys = reinterpret_cast<std::atomic<uint64_t>*>(g.keys.data());
#pragma omp parallel for schedule(static)
        for (long s0 = 0; s0 < (long)N; ++s0) {
            if (sc[s0] == kEmpty) continue;
            const float q[3] = {sx[s0 * 4 + 0] + shift[0], sx[s0 * 4 + 1] + shift[1], sx[s0 * 4 + 2] + shift[2]};
            float p[3] = {q[0] - v.pos[0], q[1] - v.pos[1], q[2] - v.pos[2]};
            float ph[3] = {dot3(p, v.vx), dot3(p, v.vy), dot3(p, v.vz)};
            if (ph[2] < 0.05f) continue;
            int px = proj_coord(ph[0] * (float)res_y, ph[2], (float)res_x / 2);
            int py = proj_coord(ph[1] * (float)res_y, ph[2], (float)res_y / 2);
            if (px >= res_x - 1 || px < 0 || py >= res_y - 1 || py < 0) continue;
            uint32_t sz = (uint32_t)(int)(ph[2] * 1000.0f) << 8;
            if (sz >= kEmpty) continue;
            // the product reprojects the last frame's plane as cache plane 2 (plane bit 1)
            uint64_t key = ((uint64_t)(sz | 1u) << 32) | (uint64_t)s0;
            size_t t = (size_t)py * res_x + px;
            uint64_t c = keys[t].load(std::memory_order_relaxed);
            while (key < c && !keys[t].compare_exchange_weak(c, key, std::memory_order_relaxed)) {
            }
        }
#pragma omp parallel for schedule(static)
        for (long t = 0; t < (long)N; ++t) {
            uint64_t key = g.keys[t];
            if (key == ~0ull) continue;
            g.keys[t] = ~0ull;
            uint32_t src = (uint32_t)key, hi = (uint32_t)(key >> 32);
            const float q[3] = {sx[(size_t)src * 4 + 0] + shift[0], sx[(size_t)src * 4 + 1] + shift[1],
                                sx[(size_t)src * 4 + 2] + shift[2]};
            float p[3] = {q[0] - v.pos[0], q[1] - v.pos[1], q[2] - v.pos[2]};
            (void)p;
            col[t] = (hi & ~255u) + (sc[src] & 255u);
            xyz[t * 4 + 0] = q[0];
            xyz[t * 4 + 1] = q[1];
            xyz[t * 4 + 2] = q[2];
            xyz[t * 4 + 3] = sx[(size_t)src * 4 + 3];  // the hit code travels with the point
        }
    }
    const int ax = (res_x / 8) * (frame & 7), ay = (res_y / 4) * ((frame >> 3) & 3);
    const int xe = std::min(res_x, ax + (res_x / 8 + 15) / 16 * 16);
    const int ye = std::min(res_y, ay + (res_y / 4 + 15) / 16 * 16);
    std::vector<uint32_t> cert_col(N, 0u);
    std::vector<float> cert_xyz(N * 4, 0.0f);
    // start distances: the 3x3 minimum of the reprojected points' camera
    // distances, less 2 cells of the level of detail there; half that minimum
    // for a pixel with at least 3 holes (pixels of the frame without a point)
    // in its 3x3
    std::vector<float> dist(N);
#pragma omp parallel for schedule(static)
    for (long t = 0; t < (long)N; ++t) {
        float d = INFINITY;
        if (col[t] != kEmpty) {
            const float ax = xyz[t * 4 + 0] - v.pos[0], ay = xyz[t * 4 + 1] - v.pos[1], az = xyz[t * 4 + 2] - v.pos[2];
            d = std::sqrt(ax * ax + ay * ay + az * az);
        }
        dist[t] = d;
    }
#pragma omp parallel for schedule(static)
    for (long t = 0; t < (long)N; ++t) {
        const int x = (int)(t % res_x), y = (int)(t / res_x);
        float m = INFINITY;
        int holes = 0;
        for (int j = -1; j <= 1; ++j)
            for (int i = -1; i <= 1; ++i) {
                const int xi = x + i, yj = y + j;
                if (xi >= 0 && xi < res_x && yj >= 0 && yj < res_y) {
                    const size_t o = (size_t)yj * res_x + xi;
                    m = std::fmin(m, dist[o]);
                    holes += col[o] == kEmpty ? 1 : 0;
                }
            }
        float gd = -1.0f;
        if (m < INFINITY) {
            const float s = m * 16.0f;
            float sw = (float)(2 * res_x);
            int lod = 1;
            while (s > sw && lod < 24) {
                sw *= 2.0f;
                ++lod;
            }
            gd = holes >= 3 ? s * 0.5f : std::fmax(s - 2.0f * (float)(1 << lod), 0.0f);
            const bool rect = x >= ax && x < xe && y >= ay && y < ye;
            if (g.certify && holes == 0 && !rect) {
                Certified c;
                if (certify(v, res_x, res_y, x, y, col.data(), xyz.data(), s, c)) {
                    gd = kGuideCertified;
                    cert_col[t] = c.colour;
                    for (int a = 0; a < 4; ++a) cert_xyz[t * 4 + a] = c.xyzw[a];
                }
            }
        }
        g.guide[t] = gd;
    }
    // rays: the refresh tile (raycast.h:363-366) and the unguided pixels (all of
    // them without a cache) from the camera, every other pixel walked, except
    // the certified ones, which take the certified colour and point
#pragma omp parallel for schedule(dynamic, 4)
    for (int y = 0; y < res_y; ++y)
        for (int x = 0; x < res_x; ++x) {
            const size_t t = (size_t)y * res_x + x;
            const bool rect = x >= ax && x < xe && y >= ay && y < ye;
            if (!rect && have_cache && g.guide[t] == kGuideCertified) {
                col[t] = cert_col[t];
                for (int a = 0; a < 4; ++a) xyz[t * 4 + a] = cert_xyz[t * 4 + a];
                continue;
            }
            const float s0 = (rect || !have_cache || g.guide[t] < 0.0f) ? 0.0f : g.guide[t];
            const Ray r = tr.trace(v, x, y, res_x, res_y, 1.0f, 1.0f, s0);
            store_ray_plane(col.data(), xyz.data(), t, r);
            xyz[t * 4 + 3] = hit_code(r);
        }
    g.cache = cur;
    for (int i = 0; i < 3; ++i) g.cache_pos[i] = v.pos[i];
    return 0;
}

void* orc_warp_create(int res_x, int res_y) {
    if (res_x < 16 || res_y < 16 || res_x > 65535 || res_y > 65535) return nullptr;
    Warp* w = new Warp;
    w->res_x = res_x;
    w->res_y = res_y;
    w->N = (size_t)res_x * res_y;
    w->tiles = (size_t)(res_x / 16) * (res_y / 16);
    w->screen.assign(4 * w->N, kEmpty);
    w->back.assign(4 * w->N * 4, 0.0f);
    w->ids.assign(w->N + 2 * w->tiles, 0u);
    w->tex.assign(w->N, 0u);
    w->prefill.assign(w->N, 0u);
    w->keys.assign(w->N, ~0ull);
    return w;
}
void orc_warp_free(void* h) { delete static_cast<Warp*>(h); }

// raycast_fine (kernel.cl:696-843) as raycast.h:235-261 launches it (a
// block the reference ships disabled): work-items over (res/4 rounded up to
// 16)^2, each owning the 2x2 block at (add + 2*id); it traces the block's
// first empty pixel (order (0,0),(1,0),(0,1),(1,1)), or when none is empty
// the pixel ((frame>>2)&1, (frame>>3)&1) of the block. The quadrant origin
// moves every frame: add = (res/2) * ((frame, frame>>1) & 1). Needs res_x
// and res_y multiples of 4, so that no block crosses the frame edge.
void coarse_refresh(Warp& w, const Tracer& tr, const View& v, int frame, uint64_t& rays, uint64_t& child,
                    uint64_t& col, uint64_t& bnd) {
    const int res_x = w.res_x, res_y = w.res_y;
    const int add_x = (res_x / 2) * (frame & 1), add_y = (res_y / 2) * ((frame >> 1) & 1);
    const int gx = (res_x / 4 + 15) / 16 * 16, gy = (res_y / 4 + 15) / 16 * 16;
#pragma omp parallel for schedule(dynamic, 1) reduction(+ : rays, child, col, bnd)
    for (int j = 0; j < gy; ++j)
        for (int i = 0; i < gx; ++i) {
            const int bx = 2 * i + add_x, by = 2 * j + add_y;
            if (bx >= res_x || by >= res_y) continue;
            int x = bx + ((frame >> 2) & 1), y = by + ((frame >> 3) & 1);
            for (int k = 0; k < 4; ++k) {
                if (w.screen[(size_t)(by + (k >> 1)) * res_x + bx + (k & 1)] == kEmpty) {
                    x = bx + (k & 1);
                    y = by + (k >> 1);
                    break;
                }
            }
            Ray r = tr.trace(v, x, y, res_x, res_y, 1.0f, 1.0f);
            store_ray(w, (size_t)y * res_x + x, r);
            ++rays;
            child += r.child_fetches;
            col += r.colour_fetches;
            bnd += r.boundary;
        }
}

// One raycast_draw (raycast.h:147-441) minus the GL display. options bit 0:
// the commented-out alternating copy target ((frame>>4)%2)+1 instead of the
// shipped target 2 (raycast.h:395); bit 1: the disabled raycast_fine pass
// (raycast.h:235-261) between reprojection and the hole gather.
int orc_warp_frame(void* h, int depth, const uint32_t* words, size_t n_words, uint32_t root, const float* pos4,
                   const float* m16, int frame, int threads, int cache_mode) {
    Warp& w = *static_cast<Warp*>(h);
    if (threads > 0) omp_set_num_threads(threads);
    const int res_x = w.res_x, res_y = w.res_y;
    const size_t N = w.N;
    View v = make_view(pos4, m16);
    Tracer tr{words, n_words, root, depth};
    const float fov = 1.0f;  // raycast.h:109-110

    // raycast.h:150-157
    if (frame < 2) std::fill(w.screen.begin(), w.screen.end(), kEmpty);
    std::fill(w.screen.begin(), w.screen.begin() + N, kEmpty);
    const bool coarse = (cache_mode & 2) != 0;
    if (coarse && (res_x % 4 || res_y % 4)) return -2;
    // raycast.h:176-198: planes 1 then 2 into plane 0
    proj_plane(w, v, 1);
    proj_plane(w, v, 2);
    proj_resolve(w, v);
    uint64_t rays = 0, child = 0, col = 0, bnd = 0;
    if (coarse) coarse_refresh(w, tr, v, frame, rays, child, col, bnd);
    // raycast.h:263-315
    gather_holes(w);
    // raycast.h:330-387
    const size_t tiles = w.tiles;
    const int add_x = (res_x / 8) * (frame & 7), add_y = (res_y / 4) * ((frame >> 3) & 3);
    auto round16 = [](int g) { return (g + 15) / 16 * 16; };
    const int x_end = std::min(res_x, add_x + round16(res_x / 8)), y_end = std::min(res_y, add_y + round16(res_y / 4));
#pragma omp parallel for schedule(dynamic, 64) reduction(+ : rays, child, col, bnd)
    for (long e = 0; e < (long)w.hole_count; ++e) {
        uint32_t xy = w.ids[2 * tiles + e];
        int x = (int)(xy & 0xffffu), y = (int)(xy >> 16);
        if (x >= res_x || y >= res_y) continue;
        Ray r = tr.trace(v, x, y, res_x, res_y, fov, fov);
        store_ray(w, (size_t)y * res_x + x, r);
        ++rays;
        child += r.child_fetches;
        col += r.colour_fetches;
        bnd += r.boundary;
    }
#pragma omp parallel for schedule(dynamic, 1) reduction(+ : rays, child, col, bnd)
    for (int y = add_y; y < y_end; ++y)
        for (int x = add_x; x < x_end; ++x) {
            Ray r = tr.trace(v, x, y, res_x, res_y, fov, fov);
            store_ray(w, (size_t)y * res_x + x, r);
            ++rays;
            child += r.child_fetches;
            col += r.colour_fetches;
            bnd += r.boundary;
        }
    w.rays = rays;
    w.child_fetches = child;
    w.colour_fetches = col;
    w.boundary_rays = bnd;
    // raycast.h:394-405: copy plane 0 to the cache target plane
    const int target = (cache_mode & 1) ? ((frame >> 4) % 2) + 1 : 2;
    std::memcpy(w.screen.data() + (size_t)target * N, w.screen.data(), N * 4);
    std::memcpy(w.back.data() + (size_t)target * N * 4, w.back.data(), N * 16);
    std::memcpy(w.prefill.data(), w.screen.data(), N * 4);
    // raycast.h:411-422 and 429-437
    const uint32_t* snap = w.screen.data();
    std::vector<uint32_t> lin(2 * N);
    std::memcpy(lin.data(), snap, N * 4);
    std::memcpy(lin.data() + N, w.screen.data() + N, N * 4);  // plane 1 follows plane 0 in memory
#pragma omp parallel for schedule(static)
    for (int y = 0; y < res_y; ++y)
        for (int x = 0; x < res_x; ++x) {
            size_t o = (size_t)y * res_x + x;
            uint32_t c = fill_pixel(lin.data(), 2 * N, x, y, res_x, res_y);
            w.screen[o] = c;
            w.tex[o] = colorize(c);
        }
    return 0;
}

uint32_t* orc_warp_screen(void* h) { return static_cast<Warp*>(h)->screen.data(); }
float* orc_warp_back(void* h) { return static_cast<Warp*>(h)->back.data(); }
uint32_t* orc_warp_ids(void* h) { return static_cast<Warp*>(h)->ids.data(); }
uint32_t* orc_warp_tex(void* h) { return static_cast<Warp*>(h)->tex.data(); }
uint32_t* orc_warp_prefill(void* h) { return static_cast<Warp*>(h)->prefill.data(); }
int orc_warp_hole_count(void* h) { return (int)static_cast<Warp*>(h)->hole_count; }
// rays traced, child fetches, colour fetches, boundary rays of the last frame
void orc_warp_stats(void* h, uint64_t* out) {
    Warp& w = *static_cast<Warp*>(h);
    out[0] = w.rays;
    out[1] = w.child_fetches;
    out[2] = w.colour_fetches;
    out[3] = w.boundary_rays;
}

void orc_colorize(const uint32_t* words, uint32_t* out, size_t n) {
    for (size_t i = 0; i < n; ++i) out[i] = colorize(words[i]);
}

// floor(log2f(i)) against the index of the top set bit, for i in [1, limit):
// the known-answer check behind replacing kernel.cl:202's log2 by a bit scan.
// Returns the first mismatching i, or 0 when all agree.
uint32_t orc_log2_kat(uint32_t limit) {
    for (uint32_t i = 1; i < limit; ++i) {
        int a = (int)std::log2((float)i);
        int b = 31 - __builtin_clz(i);
        if (a != b) return i;
    }
    return 0;
}

int orc_max_threads() { return omp_get_max_threads(); }

}  // extern "C"
