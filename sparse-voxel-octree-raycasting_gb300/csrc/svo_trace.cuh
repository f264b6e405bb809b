// svo_trace.cuh -- device-side octree traversal for sm_103a.
//
// One ray = one thread. The walk is the reference's CAST_RAY
// (kernel/kernel.cl:114-214) with its node fetches fetchChildOffset/fetchColor
// (:32-112): the same float operations in the same order, so a GB300 ray
// lands on the same voxel with the same colour word and the same hit
// position bits as the strict-IEEE oracle. Every float operation is an
// explicit round-to-nearest intrinsic (no FMA contraction, IEEE division and
// square root); float->int conversions truncate like OpenCL's convert_int.
//
// GB300 layout choices:
//   * node words are read through the read-only path (__ldg) with a bounds
//     check against the uploaded word count (a bad word raises a fault flag
//     instead of reading outside the allocation);
//   * the per-ray node stack lives in shared memory as [level][thread], so the
//     32 lanes of a warp always hit 32 different banks;
//   * loop state stays in registers; the pop level is the exponent of the
//     exactly converted XOR mask instead of kernel.cl:202's log2 of a float
//     (the same top set bit for every input the walk can produce, pinned by
//     a known-answer test);
//   * every walk is capped at kStepCap steps (fault flag 2) so no input can
//     keep a kernel spinning.
#pragma once
#include <cstdint>

namespace svo {

constexpr uint32_t kEmptyPixel = 0xffffff00u;
constexpr float kViewDistMax = 400000.0f;  // VIEW_DIST_MAX, kernel.cl:15
constexpr uint32_t kStepCap = 1u << 20;
constexpr float kGuideTopMargin = 16.0f;   // raypos units a guided start keeps below the volume's top
constexpr uint32_t kFaultFetch = 1u;       // node word index outside the octree
constexpr uint32_t kFaultSteps = 2u;       // a ray exceeded kStepCap steps
constexpr uint32_t kFaultHoleEntry = 4u;   // hole list entry outside the frame
constexpr uint32_t kFaultStage = 8u;       // staging copy of the node prefix did not complete
constexpr uint32_t kFaultNet = 16u;        // a reconstruction-net tensor-core wait timed out

// Dynamic shared memory of the trace kernels: the per-thread node stack
// ([level][thread]) followed by a staged copy of the octree's first words
// (the normal-node region, see stage_prefix).
extern __shared__ __align__(16) uint32_t svo_dsmem[];

struct Octree {
    const uint32_t* __restrict__ words;
    uint32_t n_words;
    uint32_t root;
    uint32_t n_smem;     // words [0, n_smem) are also in svo_dsmem[smem_base ...]
    uint32_t smem_base;  // word offset of that copy in svo_dsmem
};

// Camera as the ray kernels consume it: position and the rows of m^T.
struct RayCam {
    float px, py, pz;
    float mxx, mxy, mxz;
    float myx, myy, myz;
    float mzx, mzy, mzz;
    float fovx, fovy;
};

struct RayResult {
    uint32_t colour;   // 0xff000000 + fetched colour word (kernel.cl:934)
    float hx, hy, hz;  // raypos/16 (kernel.cl:920)
    float dist;        // distance/16
    uint64_t voxel;    // packed hit cell (bit 63 = hit)
    float code;        // hit code: level | signs << 5 (a float holding an integer), -1 without a hit
};

// Node word fetch: the staged prefix from shared memory, the rest through the
// read-only path, everything bounds-checked against the uploaded word count.
__device__ __forceinline__ uint32_t load_word(const Octree& o, uint32_t i, uint32_t& fault) {
    if (i < o.n_smem) return svo_dsmem[o.smem_base + i];
    if (i < o.n_words) return __ldg(o.words + i);
    fault |= kFaultFetch;
    return 0u;
}

__device__ __forceinline__ uint32_t smem_addr(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ bool mbar_try_wait(uint32_t bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(bar), "r"(parity)
        : "memory");
    return ok != 0;
}

// Programmatic dependent launch (the learned frame's kernel chain): a kernel
// launched with programmatic stream serialisation may start while the kernel
// before it in the stream still runs; it does its independent set-up first,
// then waits here until that kernel has completed and its writes are
// visible (an immediate return for a kernel launched normally).
__device__ __forceinline__ void grid_dep_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
// Lets the next kernel in the stream start its set-up once every block of
// this one has passed this point (called after grid_dep_wait).
__device__ __forceinline__ void grid_dep_launch() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }

__device__ __forceinline__ uint64_t global_ns() {
    uint64_t t;
    asm volatile("mov.u64 %0, %globaltimer;" : "=l"(t));
    return t;
}

// Bounded wait on phase 0 of an mbarrier: gives up after ~0.5 s.
__device__ __forceinline__ bool mbar_wait_bounded(uint32_t bar) {
    if (mbar_try_wait(bar, 0)) return true;
    const uint64_t t0 = global_ns();
    for (;;) {
        if (mbar_try_wait(bar, 0)) return true;
        if (global_ns() - t0 > 500000000ull) return false;
    }
}

// Copies octree words [0, n) into svo_dsmem[base ...] with bulk asynchronous
// copies (the TMA engine), completing on an mbarrier. n*4 rounded up to 16
// bytes must lie inside the octree allocation (checked by the host), the
// source is the 256-byte aligned allocation start and base is a multiple of 4
// words. Every thread of the block must call it. Returns false (and the
// block must not use the copy) if the copy did not complete in time.
__device__ __forceinline__ bool stage_prefix(const uint32_t* src, uint32_t n, uint32_t base, uint64_t* mbar,
                                             uint32_t& fault) {
    const uint32_t bytes = (n * 4u + 15u) & ~15u;
    const uint32_t bar = smem_addr(mbar);
    if (threadIdx.x == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(bar) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
        const uint32_t dst = smem_addr(svo_dsmem + base);
        for (uint32_t off = 0; off < bytes; off += 16384u) {
            const uint32_t chunk = min(16384u, bytes - off);
            asm volatile(
                "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                    dst + off),
                "l"(reinterpret_cast<const char*>(src) + off), "r"(chunk), "r"(bar)
                : "memory");
        }
    }
    const bool ok = __syncthreads_and(mbar_wait_bounded(bar) ? 1 : 0) != 0;
    if (!ok) fault |= kFaultStage;
    return ok;
}

// Before a block that gave up on its staging copy exits: wait (bounded) for
// the copy still in flight so it never lands in released shared memory.
__device__ __forceinline__ void stage_drain(uint64_t* mbar) { (void)mbar_wait_bounded(smem_addr(mbar)); }

// Levels of the per-thread node stack: the walk's levels 0..DEPTH-1 and the
// root twice above them (read by a pop to the top level and by the colour
// fetch of a ray that never descended).
template <int DEPTH>
constexpr int kStackLevels = DEPTH + 2;
// Writes the root into this thread's stack column at levels DEPTH and
// DEPTH + 1; a kernel calls it once, before its first walk.
template <int DEPTH>
__device__ __forceinline__ void stack_init(uint32_t* stk, int stride, uint32_t root) {
    stk[DEPTH * stride] = root;
    stk[(DEPTH + 1) * stride] = root;
}

__device__ __forceinline__ uint32_t popc8(uint32_t v) { return __popc(v & 0xffu); }

// fetchColor (kernel.cl:64-112).
__device__ __forceinline__ uint32_t fetch_colour(const Octree& o, uint32_t node, uint32_t before, uint32_t before2,
                                                 uint32_t local_root, int rek, uint32_t child_test, uint32_t& fault) {
    uint32_t n = node >> 9;
    if (rek == 1) {
        n = (before >> 9) & 15u;
        const uint32_t ofs = (before2 >> 9) + local_root;
        uint32_t nadd = popc8(before2);
        for (uint32_t i = 1; i < n; ++i) nadd += popc8(load_word(o, ofs + (i >> 2), fault) >> ((i & 3u) << 3));
        nadd += popc8(before & ((child_test << 1) - 1u));
        return load_word(o, ofs + (nadd >> 2), fault) >> ((nadd & 3u) << 3);
    }
    uint32_t nadd = 8;
    if (node & 256u) {
        if (!(before & 256u)) {
            local_root = n << 6;
            n = 0;
        }
        nadd = local_root;
        if (rek == 2) {
            const uint32_t ofs = (before >> 9) + local_root;
            nadd = 1u + popc8(before);
            for (uint32_t i = 1; i < n; ++i) nadd += popc8(load_word(o, ofs + (i >> 2), fault) >> ((i & 3u) << 3));
            return load_word(o, ofs + (nadd >> 2), fault) >> ((nadd & 3u) << 3);
        }
    }
    return load_word(o, n + nadd, fault);
}

// Cell coordinates of the walk. On the fast path (coordinates in [0, 2^23))
// a coordinate is carried biased, as the float bits of 2^23 + trunc(x):
// bits(x + 2^23 rounded toward zero) = 0x4B000000 | trunc(x). The low 23 bits
// are the integer itself, so bit tests, the XOR of two coordinates and the
// next cell boundary need no conversion back, and the I2F/F2I instructions
// (a narrow pipe, which throttled the stepping loop) are FMA-pipe adds.
template <bool kFast>
constexpr int kCellBias = kFast ? 0x4B000000 : 0;
template <bool kFast>
__device__ __forceinline__ int float_to_cell(float x) {
    return kFast ? __float_as_int(__fadd_rz(x, 8388608.0f)) : __float2int_rz(x);
}
// (1 << n) - 1 in one instruction.
__device__ __forceinline__ uint32_t low_mask(int n) {
    uint32_t m;
    asm("bmsk.clamp.b32 %0, 0, %1;" : "=r"(m) : "r"(n));
    return m;
}
// The next cell boundary above coordinate r at level rek, as a float, given
// mask = 2^rek - 1: ((r >> rek) + 1) << rek = (r | mask) + 1. On the fast
// path r is biased, so r | mask are the float bits of 2^23 + v with
// v = (unbiased r) | mask < 2^23, and adding 1 - 2^23 (exactly
// representable) gives v + 1 exactly (at most 2^23).
template <bool kFast>
__device__ __forceinline__ float next_boundary(int r, uint32_t mask) {
    if (kFast) return __fadd_rn(__int_as_float((int)((uint32_t)r | mask)), -8388607.0f);
    return (float)(int)(((uint32_t)r | mask) + 1u);
}

struct Walk {
    float rpx, rpy, rpz;
    float distance;
    uint32_t nodeid, nodeid_before, local_root, node_test;
    int rek;
    bool hit;
    int hcx, hcy, hcz;
};

// load_word written as a select chain (no early returns) for the descent loop.
__device__ __forceinline__ uint32_t load_word_sel(const Octree& o, uint32_t i, uint32_t& fault) {
    const bool in_smem = i < o.n_smem;
    const bool in_range = i < o.n_words;
    uint32_t v = 0;
    if (in_smem) v = svo_dsmem[o.smem_base + i];
    else if (in_range) v = __ldg(o.words + i);
    else fault |= kFaultFetch;
    return v;
}

// CAST_RAY's loop (kernel.cl:152-211), arranged for SIMT execution:
//   * descents run in an inner loop, so the lanes of a warp that descend do so
//     together and then all lanes step together (a loop iteration no longer
//     runs both the descend and the step path);
//   * the next level's child index is computed while the node load is in
//     flight; block-node addressing uses selects instead of nested branches;
//   * the descent loop needs no step cap (rek strictly decreases); the view
//     distance and y-exit tests share one branch.
//   * the stack holds the root at levels DEPTH and DEPTH + 1 (written once
//     per thread by the kernel), so a pop reads its node and its parent
//     without testing for the root;
//   * the step cap shares the exit branch (a capped walk has done one more
//     step when it stops; its result is discarded with the fault flag).
// The state changes are those of the reference loop, in the same order.
// kFast: every coordinate of the walk stays in [0, 2^23), checked by the
// caller from the mirrored start point (each step moves a coordinate by at
// most the distance it adds, and the walk stops once the distance passes
// VIEW_DIST_MAX); the cell coordinates are then carried biased
// (float_to_cell).
template <int DEPTH, bool kFast>
__device__ __forceinline__ void walk(const Octree& o, Walk& w, uint32_t sxyz, float g0y, float g0z, float g1x,
                                     float g1z, float g2x, float g2y, float lx, float ly, float lz, float lodswitch,
                                     int lod, uint32_t* stk, int stride, uint32_t& fault) {
    constexpr int kDepthAnd = (1 << DEPTH) - 1;
    constexpr int kTopBit = 2 * kDepthAnd + 2;
    float rpx = w.rpx, rpy = w.rpy, rpz = w.rpz;
    int rix = float_to_cell<kFast>(rpx), riy = float_to_cell<kFast>(rpy), riz = float_to_cell<kFast>(rpz);
    int rek = DEPTH;
    float distance = w.distance;
    const uint32_t root = o.root;
    uint32_t nodeid = root, nodeid_before = root, local_root = 0, node_test = 0;
    uint32_t steps = 0;
    // y and z pre-shifted by 1 and 2, so the child index at level r is three
    // shifts and a bit merge: bit 0 from x >> r, bit 1 from y2 >> r, bit 2
    // from z4 >> r.
    uint32_t ry2 = (uint32_t)riy << 1, rz4 = (uint32_t)riz << 2;
    auto child_index = [&](int r) -> uint32_t {
        const uint32_t a = (uint32_t)rix >> r, b = ry2 >> r, c = rz4 >> r;
        return ((((a & 1u) | (b & ~1u)) & 3u) | (c & 4u)) ^ sxyz;
    };
    uint32_t ni = child_index(rek);
    for (;;) {
        node_test = nodeid & (1u << ni);
        // One exit test per descent: the level-of-detail test of a descent is
        // taken after the next level's child index, stack entry and bit test
        // have been computed; a hit then restores the level and the bit test
        // (the stack entry one level below the hit is never read).
        bool hit = false;
        while (node_test && !hit) {
            const uint32_t parent = nodeid;
            const uint32_t n = nodeid >> 9;
            if (!(nodeid & 256u)) {
                nodeid = load_word_sel(o, n + ni, fault);
            } else {
                const bool enter = !(nodeid_before & 256u);
                local_root = enter ? (n << 6) : local_root;
                const uint32_t base = enter ? local_root : local_root + n;
                const uint32_t nadd = __popc(nodeid & ((node_test << 1) - 1u));
                if (rek > 2) {
                    nodeid = load_word_sel(o, base + nadd, fault);
                } else if (rek == 2) {
                    const uint32_t wd = load_word_sel(o, base + (nadd >> 2), fault);
                    nodeid = ((wd >> ((nadd & 3u) << 3)) & 255u) + 256u + (nadd << 9);
                } else {
                    nodeid = 0u;
                }
            }
            nodeid_before = parent;
            hit = rek <= lod;
            --rek;
            ni = child_index(rek);
            stk[rek * stride] = nodeid;
            node_test = nodeid & (1u << ni);
        }
        if (hit) {
            ++rek;
            node_test = nodeid_before & (1u << child_index(rek));
            w.hit = true;
            w.hcx = (rix - kCellBias<kFast>) >> rek;
            w.hcy = (riy - kCellBias<kFast>) >> rek;
            w.hcz = (riz - kCellBias<kFast>) >> rek;
            break;
        }
        ++steps;
        const uint32_t mask = low_mask(rek);
        const float m0x = __fsub_rn(next_boundary<kFast>(rix, mask), rpx);
        const float m0y = __fsub_rn(next_boundary<kFast>(riy, mask), rpy);
        const float m0z = __fsub_rn(next_boundary<kFast>(riz, mask), rpz);
        float best = __fmul_rn(m0x, lx);
        const float idy_ = __fmul_rn(m0y, ly), idz_ = __fmul_rn(m0z, lz);
        float mm = m0x, gx = 1.0f, gy = g0y, gz = g0z;
        if (idy_ < best) { best = idy_; mm = m0y; gx = g1x; gy = 1.0f; gz = g1z; }
        if (idz_ < best) { best = idz_; mm = m0z; gx = g2x; gy = g2y; gz = 1.0f; }
        rpx = __fadd_rn(rpx, __fmul_rn(gx, mm));
        rpy = __fadd_rn(rpy, __fmul_rn(gy, mm));
        rpz = __fadd_rn(rpz, __fmul_rn(gz, mm));
        const int bx = rix, by = riy, bz = riz;
        rix = float_to_cell<kFast>(rpx);
        riy = float_to_cell<kFast>(rpy);
        riz = float_to_cell<kFast>(rpz);
        ry2 = (uint32_t)riy << 1;
        rz4 = (uint32_t)riz << 2;
        distance = __fadd_rn(distance, best);
        const int x0ry = by ^ riy;
        const uint32_t x0r = (uint32_t)(((bx ^ rix) ^ x0ry ^ (bz ^ riz)) & kDepthAnd);
        const bool far = distance > kViewDistMax;
        if (!far && x0r > mask) {  // x0r >> rek != 0
            // top set bit + 1 (<= DEPTH: x0r has DEPTH bits), from the exponent
            // of float(x0r), exact for x0r < 2^23: shorter latency than clz
            rek = (__float_as_int(__fsub_rn(__int_as_float((int)(0x4B000000u | x0r)), 8388608.0f)) >> 23) - 126;
            nodeid = stk[rek * stride];
            nodeid_before = stk[(rek + 1) * stride];
            if (distance > lodswitch) {
                lodswitch = __fmul_rn(lodswitch, 2.0f);
                ++lod;
            }
        }
        if (far || (x0ry & kTopBit) || steps > kStepCap) break;
        ni = child_index(rek);
    }
    if (steps > kStepCap) fault |= kFaultSteps;
    w.rpx = rpx;
    w.rpy = rpy;
    w.rpz = rpz;
    w.distance = distance;
    w.nodeid = nodeid;
    w.nodeid_before = nodeid_before;
    w.local_root = local_root;
    w.node_test = node_test;
    w.rek = rek;
}

// Ray setup of raycast_fine_2/raycast_holes (kernel.cl:883-899) + CAST_RAY +
// the colour fetch. `stk` points at this thread's column of the shared stack
// (entry for level L at stk[L * stride]); the walk writes levels 0..DEPTH-1,
// levels DEPTH and DEPTH + 1 hold the root (stack_init).
//
// kGuided with s0 > 0: the walk starts s0 (raypos units, 16 per world unit)
// along the ray instead of at the camera -- but at most up to
// kGuideTopMargin before the ray leaves the volume's height -- with the
// distance already at s0 and the level of detail advanced as far as the
// lodswitch doublings below s0 reach. The start point is camera + s0 *
// (1, g0y, g0z)/lx (the unit direction) in the mirrored frame, every
// operation rounded to nearest (the CPU oracle repeats it). Everything the ray passes before s0 is skipped: the caller
// guarantees, or accepts, that nothing lies there.
template <int DEPTH, bool kVoxel, bool kGuided = false>
__device__ __forceinline__ RayResult trace_ray(const Octree& o, const RayCam& c, int idx, int idy, int res_x,
                                               int res_y, uint32_t* stk, int stride, uint32_t& fault,
                                               float s0 = 0.0f) {
    constexpr int kScaleMax = 1 << (DEPTH + 1);
    const float fscale = (float)kScaleMax;

    // delta1 = ((idx-res_x/2+0.5)*fovx/res_y, (idy-res_y/2+0.5)*fovy/res_y, 1)
    const float d1x = __fdiv_rn(__fmul_rn(__fadd_rn((float)(idx - (res_x >> 1)), 0.5f), c.fovx), (float)res_y);
    const float d1y = __fdiv_rn(__fmul_rn(__fadd_rn((float)(idy - (res_y >> 1)), 0.5f), c.fovy), (float)res_y);
    // delta = (dot(delta1, mx), dot(delta1, my), dot(delta1, mz)), left to right
    float dx = __fadd_rn(__fadd_rn(__fmul_rn(d1x, c.mxx), __fmul_rn(d1y, c.mxy)), c.mxz);
    float dy = __fadd_rn(__fadd_rn(__fmul_rn(d1x, c.myx), __fmul_rn(d1y, c.myy)), c.myz);
    float dz = __fadd_rn(__fadd_rn(__fmul_rn(d1x, c.mzx), __fmul_rn(d1y, c.mzy)), c.mzz);
    float rpx = __fmul_rn(c.px, 16.0f), rpy = __fmul_rn(c.py, 16.0f), rpz = __fmul_rn(c.pz, 16.0f);

    const float eps = 9.5367431640625e-07f;  // 2^-20, kernel.cl:118
    if (fabsf(dx) < eps) dx = dx > 0.0f ? eps : (dx < 0.0f ? -eps : dx);
    if (fabsf(dy) < eps) dy = dy > 0.0f ? eps : (dy < 0.0f ? -eps : dy);
    if (fabsf(dz) < eps) dz = dz > 0.0f ? eps : (dz < 0.0f ? -eps : dz);
    uint32_t sxyz = 0;
    if (dx < 0.0f) { sxyz |= 1u; rpx = __fsub_rn(fscale, rpx); dx = -dx; }
    if (dy < 0.0f) { sxyz |= 2u; rpy = __fsub_rn(fscale, rpy); dy = -dy; }
    if (dz < 0.0f) { sxyz |= 4u; rpz = __fsub_rn(fscale, rpz); dz = -dz; }

    const float g0y = __fdiv_rn(dy, dx), g0z = __fdiv_rn(dz, dx);
    const float g1x = __fdiv_rn(dx, dy), g1z = __fdiv_rn(dz, dy);
    const float g2x = __fdiv_rn(dx, dz), g2y = __fdiv_rn(dy, dz);
    const float lx = __fsqrt_rn(__fadd_rn(__fadd_rn(1.0f, __fmul_rn(g0y, g0y)), __fmul_rn(g0z, g0z)));
    const float ly = __fsqrt_rn(__fadd_rn(__fadd_rn(__fmul_rn(g1x, g1x), 1.0f), __fmul_rn(g1z, g1z)));
    const float lz = __fsqrt_rn(__fadd_rn(__fadd_rn(__fmul_rn(g2x, g2x), __fmul_rn(g2y, g2y)), 1.0f));
    float lodswitch = (float)(res_x * 2);  // res_x*LOD_ADJUST*2, kernel.cl:908
    int lod = 1;
    float dist0 = 0.0f;
    if (kGuided && s0 > 0.0f) {
        // lx = |d|/dx and ly = |d|/dy (the walk's step lengths per unit of x
        // and y) give the unit direction (1, g0y, g0z)/lx and the distance
        // to the top of the volume without another square root.
        // Never start past the point where the ray leaves the volume's height
        // (the walk's exit test fires only on the step that crosses it;
        // beyond it the ray would walk the periodic copy above).
        const float t_top = __fmul_rn(__fsub_rn(fscale, rpy), ly);
        s0 = fminf(s0, __fsub_rn(t_top, kGuideTopMargin));
        if (s0 > 0.0f) {
            const float ux = __fdiv_rn(1.0f, lx);
            rpx = __fadd_rn(rpx, __fmul_rn(ux, s0));
            rpy = __fadd_rn(rpy, __fmul_rn(__fmul_rn(g0y, ux), s0));
            rpz = __fadd_rn(rpz, __fmul_rn(__fmul_rn(g0z, ux), s0));
            dist0 = s0;
            while (dist0 > lodswitch && lod < DEPTH) {
                lodswitch = __fmul_rn(lodswitch, 2.0f);
                ++lod;
            }
        }
    }

    Walk w;
    w.rpx = rpx;
    w.rpy = rpy;
    w.rpz = rpz;
    w.distance = dist0;
    w.hit = false;
    w.hcx = w.hcy = w.hcz = 0;
    const float lim = 4194304.0f;  // 2^22
    const bool fast = rpx >= 0.0f && rpx < lim && rpy >= 0.0f && rpy < lim && rpz >= 0.0f && rpz < lim;
    if (fast)
        walk<DEPTH, true>(o, w, sxyz, g0y, g0z, g1x, g1z, g2x, g2y, lx, ly, lz, lodswitch, lod, stk, stride, fault);
    else
        walk<DEPTH, false>(o, w, sxyz, g0y, g0z, g1x, g1z, g2x, g2y, lx, ly, lz, lodswitch, lod, stk, stride, fault);
    rpx = w.rpx;
    rpy = w.rpy;
    rpz = w.rpz;
    const int rek = w.rek;

    if (sxyz & 1u) rpx = __fsub_rn(fscale, rpx);
    if (sxyz & 2u) rpy = __fsub_rn(fscale, rpy);
    if (sxyz & 4u) rpz = __fsub_rn(fscale, rpz);
    const uint32_t before2 = stk[(rek + 1) * stride];
    const uint32_t col = fetch_colour(o, w.nodeid, w.nodeid_before, before2, w.local_root, rek, w.node_test, fault);

    RayResult r;
    r.colour = 0xff000000u + col;
    // x/16 is exact as x*0.0625 (a power-of-two scale)
    r.hx = __fmul_rn(rpx, 0.0625f);
    r.hy = __fmul_rn(rpy, 0.0625f);
    r.hz = __fmul_rn(rpz, 0.0625f);
    r.dist = __fmul_rn(w.distance, 0.0625f);
    r.voxel = 0;
    r.code = w.hit ? (float)(rek | (int)(sxyz << 5)) : -1.0f;
    if (kVoxel && w.hit) {
        const uint32_t cells = (uint32_t)kScaleMax >> rek;
        uint32_t cx = (uint32_t)w.hcx, cy = (uint32_t)w.hcy, cz = (uint32_t)w.hcz;
        if (sxyz & 1u) cx = cells - 1u - cx;
        if (sxyz & 2u) cy = cells - 1u - cy;
        if (sxyz & 4u) cz = cells - 1u - cz;
        cx &= cells - 1u;
        cy &= cells - 1u;
        cz &= cells - 1u;
        r.voxel = (1ull << 63) | ((uint64_t)(uint32_t)rek << 48) | ((uint64_t)(((cz << rek) >> 1) & 0xffffu) << 32) |
                  ((uint64_t)(((cy << rek) >> 1) & 0xffffu) << 16) | (uint64_t)(((cx << rek) >> 1) & 0xffffu);
    }
    return r;
}

// raycast_colorize (kernel.cl:944-974): material a&3 picks an RGB factor,
// intensity a&248, BGRX8 out.
__device__ __forceinline__ uint32_t colorize(uint32_t word) {
    const int a = (int)word;
    const int m = a & 3;
    const float fr = m == 0 ? 1.0f : (m == 1 ? 1.0f : (m == 2 ? 1.5f : 0.2f));
    const float fg = m == 0 ? 1.0f : (m == 1 ? 0.7f : (m == 2 ? 0.8f : 0.8f));
    const float fb = m == 0 ? 1.0f : (m == 1 ? 0.3f : (m == 2 ? 0.1f : 0.2f));
    const float i = (float)(a & (255 - 7));
    int r = __float2int_rz(__fmul_rn(i, fr));
    int g = __float2int_rz(__fmul_rn(i, fg));
    int b = __float2int_rz(__fmul_rn(i, fb));
    r = r > 255 ? 255 : r;
    g = g > 255 ? 255 : g;
    b = b > 255 ? 255 : b;
    return (uint32_t)(b + g * 256 + r * 65536);
}

}  // namespace svo
