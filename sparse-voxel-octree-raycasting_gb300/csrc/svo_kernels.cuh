// svo_kernels.cuh -- the per-frame kernels of the raycast + warp pipeline.
//
// Reference call sequence (src/raycast.h:147-441) and how it maps here:
//   memset plane 0 (+ all planes while frame<2)       } k_project (scatter) +
//   raycast_proj x2 (kernel.cl:472-592)              } k_resolve_gather (gather,
//   raycast_counthole (kernel.cl:234-274)            }   clear and hole count)
//   raycast_sumids + blocking 4-byte readback         -> k_hole_scan (on device)
//   raycast_writeids (kernel.cl:298-340)              -> k_hole_write
//   raycast_holes + raycast_fine_2 (kernel.cl:594-942)-> k_trace<.., kWarp> (one
//                                                         persistent launch)
//   memcpy plane 0 -> plane 2 (raycast.h:390-405)      -> none: the current and
//                                                         cache planes swap roles
//   raycast_fillhole2 + raycast_colorize               -> k_fill_colorize
//
// Determinism: raycast_proj resolves depth ties racily on a GPU; here every
// target takes the source with the smallest (depth key, source index) through
// one 64-bit atomicMin, which is what running the work-items in order gives.
// raycast_fillhole2 reads its neighbours from the unfiltered plane (the
// filter writes a separate displayed plane), i.e. snapshot order.
#pragma once
#include <cstdint>

#include "svo_trace.cuh"

namespace svo {

constexpr uint64_t kKeyEmpty = ~0ull;
constexpr int kWalkBuckets = 4;  // guided walks listed by expected length (k_guide)
static_assert(kWalkBuckets == 4, "k_trace_warp selects among four walk lists");
constexpr int kMaxBatchViews = 256;

// Everything one warp frame needs, written to device memory by k_set_params
// at the start of the frame (so a captured CUDA graph replays unchanged).
struct FrameParams {
    RayCam ray;                 // ray camera (rows of m^T)
    float vx[3], vy[3], vz[3];  // rows of m (raycast_proj's a_mx/a_my/a_mz)
    int frame;
    int cur;            // physical plane (0..2) that receives this frame's plane 0
    int have_cache;     // the source planes hold earlier frames
    int src_plane[2];   // physical planes of the reference's cache planes 1 and 2, -1 = empty
    int clear_rejected; // clear rejected source pixels in their cache plane (kernel.cl:549-562)
    int fill_past;      // physical plane of reference plane 1 after the copy, -1 = empty
    int add_x, add_y, x_end, y_end;  // refresh tile rectangle (raycast.h:363-366)
    int coarse_x, coarse_y;          // quadrant origin of the raycast_fine pass (raycast.h:240-241)
    int pw_shift;                    // ray packets are (1<<pw_shift) x (32>>pw_shift) pixels
    // previous frame's camera (the reconstruction net's motion feature)
    float prev_pos[3], prev_vx[3], prev_vy[3], prev_vz[3];
    int have_prev_view;
    // Learned frames: the camera wraps into the periodic volume, so a cache
    // plane written under an earlier wrap holds points one period off. rebase
    // adds src_shift[r] (whole periods) to the points of source plane r as
    // they are reprojected; plain frames keep the reference's behaviour.
    int rebase;
    float src_shift[2][3];
    uint32_t serial;  // frame serial of the target (stamps the net tile flags)
    int certify;      // guided frames: certified reprojection (k_guide)
    // Guided frames resolve the projection keys inside k_guide<true>, whose
    // blocks read their neighbours' keys as a halo and so cannot clear them;
    // the tracer clears them instead, a 32-key chunk with every packet it
    // pulls, so the stores spread over the launch (one burst of 16 MB at its
    // start cost more than the chunks).
    int clear_keys;
};

// Buffers of one render target.
struct TargetBuffers {
    uint32_t* col[3];   // colour planes: the current one and up to two caches
    float4* xyz[3];     // coordinate planes, likewise
    uint32_t* disp;     // displayed colour plane (after the filter)
    uint32_t* bgrx;     // colourised output
    uint64_t* keys;     // per-pixel projection keys, kKeyEmpty between frames
    uint32_t* ids;      // hole id buffer in the reference layout
    uint64_t* tile_mask;  // per 16x16 tile, bit j*8+i = 2x2 block (i,j) empty
    uint32_t* req_mask;   // learned frames: per 8x4 packet, bit (x&7)+8*(y&3) = ray requested
    int packets_x, packets_y;  // ceil(res/8), ceil(res/4)
    // Guided learned frames: per pixel, the start distance of its walk in
    // raypos units (>= 0) or -1 (unguided: the net decides); per net output
    // tile, the serial of the last frame that needed the net there, and the
    // list of those tiles (count in counters[3]). guide == nullptr: no walks.
    float* guide;
    // Pixel lists k_guide writes (entries x | y << 16, walk_cap = res_x*res_y
    // each): the walks in kWalkBuckets lists by expected length, longest
    // first (walk_list + b * walk_cap, counters[4 + b] entries); the
    // certified pixels in cert_list (counters[4 + kWalkBuckets]), whose
    // colour word and point k_guide leaves in cert_col / cert_xyz for the
    // tracer to commit.
    uint32_t* walk_list;
    uint32_t walk_cap;
    uint32_t* cert_list;
    uint32_t* cert_col;
    float4* cert_xyz;
    uint32_t* net_flags;
    uint32_t* net_list;
    uint32_t* counters;   // [0] trace work counter, [1] hole entries, [2] coarse-pass work counter,
                          // [3] net tiles listed, [4..4+kWalkBuckets) walks listed per bucket,
                          // [4+kWalkBuckets] certified pixels listed
    int res_x, res_y;
    int tiles_x, tiles_y;  // whole 16x16 tiles (res/16)
};

// One view of a (batched) full raycast.
struct FullView {
    RayCam ray;
    int res_x, res_y;
    int packets_x;          // ray packets per row: ceil(res_x / packet width)
    int pw_shift;           // packets are (1<<pw_shift) x (32>>pw_shift) pixels
    uint32_t packet_begin;  // first packet of this view in the batch
    uint32_t* col;
    float4* xyzw;
    uint64_t* vox;
    uint32_t* bgrx;
};

struct FullBatch {
    int n_views;
    uint32_t total_packets;
    FullView v[kMaxBatchViews];
};

// Plane selection without dynamic indexing of the by-value parameter struct
// (which would force a local-memory copy of it).
__device__ __forceinline__ uint32_t* plane_col(const TargetBuffers& B, int i) {
    return i == 0 ? B.col[0] : (i == 1 ? B.col[1] : B.col[2]);
}
__device__ __forceinline__ float4* plane_xyz(const TargetBuffers& B, int i) {
    return i == 0 ? B.xyz[0] : (i == 1 ? B.xyz[1] : B.xyz[2]);
}

__global__ void k_set_params(FrameParams p, FrameParams* dst, uint32_t* counters) {
    *dst = p;
#pragma unroll
    for (int i = 0; i < 5 + kWalkBuckets; ++i) counters[i] = 0;
}

__global__ void k_reset_counter(uint32_t* counter) { *counter = 0; }

// ------------------------------------------------------- reprojection --
// Screen coordinate of raycast_proj (kernel.cl:552-556):
//   trunc(float(double(num)/double(z) + double(half)))
// -- the unsuffixed 0.0 literals make the reference's expression double. The
// float path decides every pixel whose value is further than its error bound
// (2^-22 of the magnitude) from an integer; the rest (about 0.1%) take the
// double path, which is exact.
__device__ __forceinline__ int proj_coord(float num, float z, float half) {
    const float q = __fdiv_rn(num, z);
    const float y = __fadd_rn(q, half);
    const float bound = __fmul_rn(__fadd_rn(__fadd_rn(fabsf(q), fabsf(half)), 1.0f), 2.384185791015625e-07f);
    const float r = rintf(y);
    if (r == 0.0f || fabsf(__fsub_rn(y, r)) > bound) return __float2int_rz(y);
    const double v = __dadd_rn(__ddiv_rn((double)num, (double)z), (double)half);
    return __float2int_rz(__double2float_rn(v));
}

__device__ __forceinline__ float dot3(float ax, float ay, float az, const float* b) {
    return __fadd_rn(__fadd_rn(__fmul_rn(ax, b[0]), __fmul_rn(ay, b[1])), __fmul_rn(az, b[2]));
}

// Scatter: every non-empty pixel of the two cache planes (reference planes 1
// and 2, raycast.h:176-198) proposes itself to the pixel it reprojects to.
// Key = (depth key int(z*1000)<<8 | cache plane bit) << 32 | source pixel:
// the smallest key wins, i.e. the nearest depth key, then plane 1 before
// plane 2, then the lowest source pixel -- the order in which the reference's
// work-items run.
__global__ void __launch_bounds__(256) k_project(const FrameParams* __restrict__ P, TargetBuffers B) {
    grid_dep_wait();
    grid_dep_launch();
    if (!P->have_cache) return;
    const int res_x = B.res_x, res_y = B.res_y;
    const uint32_t N = (uint32_t)res_x * (uint32_t)res_y;
    const float px = P->ray.px, py = P->ray.py, pz = P->ray.pz;
    float vx[3], vy[3], vz[3];
    for (int i = 0; i < 3; ++i) {
        vx[i] = P->vx[i];
        vy[i] = P->vy[i];
        vz[i] = P->vz[i];
    }
    const float hx = (float)res_x / 2.0f, hy = (float)res_y / 2.0f;
    const float fry = (float)res_y;
    const bool clear = P->clear_rejected != 0;
    const bool rebase = P->rebase != 0;
    for (int r = 0; r < 2; ++r) {
        const int phys = P->src_plane[r];
        if (phys < 0) continue;
        uint32_t* __restrict__ col = plane_col(B, phys);
        const float4* __restrict__ xyz = plane_xyz(B, phys);
        const float shx = P->src_shift[r][0], shy = P->src_shift[r][1], shz = P->src_shift[r][2];
        auto project_one = [&](uint32_t s, uint32_t c, float4 q) {
            if (c == kEmptyPixel) return;
            if (rebase) {
                q.x = __fadd_rn(q.x, shx);
                q.y = __fadd_rn(q.y, shy);
                q.z = __fadd_rn(q.z, shz);
            }
            const float ax = __fsub_rn(q.x, px), ay = __fsub_rn(q.y, py), az = __fsub_rn(q.z, pz);
            const float zz = dot3(ax, ay, az, vz);
            if (zz < 0.05f) {  // (double)z < 0.05 <=> z < 0.05f for a binary32 z
                if (clear) col[s] = kEmptyPixel;
                return;
            }
            const int sx = proj_coord(__fmul_rn(dot3(ax, ay, az, vx), fry), zz, hx);
            const int sy = proj_coord(__fmul_rn(dot3(ax, ay, az, vy), fry), zz, hy);
            if (sx >= res_x - 1 || sx < 0 || sy >= res_y - 1 || sy < 0) {
                if (clear) col[s] = kEmptyPixel;
                return;
            }
            const uint32_t sz = (uint32_t)__float2int_rz(__fmul_rn(zz, 1000.0f)) << 8;
            if (sz >= kEmptyPixel) return;  // cannot beat the cleared value (kernel.cl:571)
            const uint32_t t = (uint32_t)sy * (uint32_t)res_x + (uint32_t)sx;
            atomicMin((unsigned long long*)(B.keys + t), (unsigned long long)(((uint64_t)(sz | (uint32_t)r) << 32) | s));
        };
        // four sources per thread and iteration, their loads in flight together
        // (the atomicMin outcome does not depend on the order)
        constexpr int kPer = 4;
        const uint32_t stride = gridDim.x * blockDim.x;
        for (uint32_t s = blockIdx.x * blockDim.x + threadIdx.x; s < N; s += kPer * stride) {
            uint32_t c[kPer];
            float4 q[kPer];
#pragma unroll
            for (int k = 0; k < kPer; ++k) {
                const uint32_t sk = s + (uint32_t)k * stride;
                const bool in = sk < N;
                c[k] = in ? col[sk] : kEmptyPixel;
                q[k] = in ? __ldg(xyz + sk) : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
            }
#pragma unroll
            for (int k = 0; k < kPer; ++k) project_one(s + (uint32_t)k * stride, c[k], q[k]);
        }
    }
}

// raycast_counthole's test (HOLE_PIXEL_THRESHOLD = 4, kernel.cl:262-271) for
// the 16x16 tile of this block: bit j*8+i set when 2x2 block (i,j) is empty.
// Only whole tiles are counted (kernel.cl:243-244). Every thread calls it.
__device__ __forceinline__ void tile_mask_store(const TargetBuffers& B, uint8_t (*empty)[17], uint32_t* halves) {
    __syncthreads();
    if (blockIdx.x >= (unsigned)B.tiles_x || blockIdx.y >= (unsigned)B.tiles_y) return;  // block-uniform
    bool hole = false;
    if (threadIdx.x < 64) {
        const int i = threadIdx.x & 7, j = threadIdx.x >> 3;
        hole = empty[2 * j][2 * i] && empty[2 * j][2 * i + 1] && empty[2 * j + 1][2 * i] && empty[2 * j + 1][2 * i + 1];
    }
    const uint32_t bal = __ballot_sync(0xffffffffu, hole);
    if (threadIdx.x == 0 || threadIdx.x == 32) halves[threadIdx.x >> 5] = bal;
    __syncthreads();
    if (threadIdx.x == 0) {
        const uint32_t tile = blockIdx.y * B.tiles_x + blockIdx.x;
        B.tile_mask[tile] = (uint64_t)halves[0] | ((uint64_t)halves[1] << 32);
    }
}

// The winning source of target pixel t (its 64-bit key, kKeyEmpty for none):
// the colour word (depth key bits + the source's colour byte) and the point,
// re-based by whole periods in learned frames, with the hit code (learned
// frames) or the view depth (plain frames, kernel.cl:585) in w.
__device__ __forceinline__ uint32_t resolve_source(const FrameParams* __restrict__ P, const TargetBuffers& B,
                                                   uint64_t key, float4& q) {
    const uint32_t src = (uint32_t)key;
    const uint32_t hi = (uint32_t)(key >> 32);
    const int phys = (hi & 1u) ? P->src_plane[1] : P->src_plane[0];
    q = plane_xyz(B, phys)[src];
    if (P->rebase) {
        const int r = (int)(hi & 1u);
        q.x = __fadd_rn(q.x, P->src_shift[r][0]);
        q.y = __fadd_rn(q.y, P->src_shift[r][1]);
        q.z = __fadd_rn(q.z, P->src_shift[r][2]);
    } else {
        const float ax = __fsub_rn(q.x, P->ray.px), ay = __fsub_rn(q.y, P->ray.py), az = __fsub_rn(q.z, P->ray.pz);
        q.w = dot3(ax, ay, az, P->vz);
    }
    return (hi & ~255u) + (plane_col(B, phys)[src] & 255u);
}

// Gather + clear + hole count, one 16x16 tile per block: each target pixel
// takes its winning source (or becomes empty), then the block marks the 2x2
// blocks whose four pixels are empty (raycast_counthole's test with
// HOLE_PIXEL_THRESHOLD = 4, kernel.cl:262-271). Only whole tiles are counted
// (kernel.cl:243-244).
__global__ void __launch_bounds__(256) k_resolve_gather(const FrameParams* __restrict__ P, TargetBuffers B) {
    __shared__ uint8_t empty[16][17];
    __shared__ uint32_t halves[2];
    const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
    const int x = blockIdx.x * 16 + tx, y = blockIdx.y * 16 + ty;
    const int res_x = B.res_x, res_y = B.res_y;
    const int cur = P->cur;
    bool is_empty = true;
    if (x < res_x && y < res_y) {
        const uint32_t t = (uint32_t)y * (uint32_t)res_x + (uint32_t)x;
        uint32_t outc = kEmptyPixel;
        if (P->have_cache) {
            const uint64_t key = B.keys[t];
            if (key != kKeyEmpty) {
                B.keys[t] = kKeyEmpty;
                float4 q;
                outc = resolve_source(P, B, key, q);
                plane_xyz(B, cur)[t] = q;
            }
        }
        plane_col(B, cur)[t] = outc;
        is_empty = outc == kEmptyPixel;
    }
    empty[ty][tx] = is_empty;
    tile_mask_store(B, empty, halves);
}

// The hole count of k_resolve_gather alone, for frames whose plane 0 changed
// after the gather (the raycast_fine pass).
__global__ void __launch_bounds__(256) k_hole_mask(const FrameParams* __restrict__ P, TargetBuffers B) {
    __shared__ uint8_t empty[16][17];
    __shared__ uint32_t halves[2];
    const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
    const int x = blockIdx.x * 16 + tx, y = blockIdx.y * 16 + ty;
    bool is_empty = true;
    if (x < B.res_x && y < B.res_y) is_empty = plane_col(B, P->cur)[(size_t)y * B.res_x + x] == kEmptyPixel;
    empty[ty][tx] = is_empty;
    tile_mask_store(B, empty, halves);
}

// raycast_sumids (kernel.cl:276-296) without the single-thread loop or the
// host readback: one block scans the tile counts and leaves the total on the
// device. ids[t] = 4*holes(t) except ids[0] = total; ids[tiles+t] = exclusive
// offset of tile t.
// Tiles whose counts and prefixes the hole scan stages in shared memory
// (8 bytes per tile; beyond it the scan works on global memory).
constexpr uint32_t kScanStageTiles = 28u * 1024u;

// staged: the launch gave 8 bytes of dynamic shared memory per tile. The
// counts are then read and the prefixes written coalesced, and each thread
// scans its contiguous run of tiles in shared memory: a one-block kernel
// whose per-thread runs touched global memory 8 tiles apart spent its time
// in the one SM's scattered loads and stores.
__global__ void __launch_bounds__(1024) k_hole_scan(TargetBuffers B, int staged) {
    __shared__ uint32_t warp_sums[32];
    uint32_t* cnt_s = svo_dsmem;  // [tiles] counts, then [tiles] exclusive prefixes
    const uint32_t tiles = (uint32_t)B.tiles_x * (uint32_t)B.tiles_y;
    uint32_t* pre_s = svo_dsmem + tiles;
    const uint32_t per = (tiles + blockDim.x - 1) / blockDim.x;
    const uint32_t a = threadIdx.x * per, b = min(a + per, tiles);
    if (staged) {
        for (uint32_t t = threadIdx.x; t < tiles; t += blockDim.x) cnt_s[t] = 4u * (uint32_t)__popcll(B.tile_mask[t]);
        __syncthreads();
    }
    uint32_t local = 0;
    for (uint32_t t = a; t < b; ++t) local += staged ? cnt_s[t] : 4u * (uint32_t)__popcll(B.tile_mask[t]);
    // block exclusive scan of `local`
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint32_t incl = local;
    for (int o = 1; o < 32; o <<= 1) {
        uint32_t v = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += v;
    }
    if (lane == 31) warp_sums[warp] = incl;
    __syncthreads();
    if (warp == 0) {
        uint32_t w = lane < (int)(blockDim.x >> 5) ? warp_sums[lane] : 0u;
        for (int o = 1; o < 32; o <<= 1) {
            uint32_t v = __shfl_up_sync(0xffffffffu, w, o);
            if (lane >= o) w += v;
        }
        warp_sums[lane] = w;  // inclusive warp prefix
    }
    __syncthreads();
    uint32_t acc = incl - local + (warp > 0 ? warp_sums[warp - 1] : 0u);
    if (staged) {
        for (uint32_t t = a; t < b; ++t) {
            pre_s[t] = acc;
            acc += cnt_s[t];
        }
        __syncthreads();
        for (uint32_t t = threadIdx.x; t < tiles; t += blockDim.x) {
            B.ids[tiles + t] = pre_s[t];
            if (t > 0) B.ids[t] = cnt_s[t];
        }
    } else {
        for (uint32_t t = a; t < b; ++t) {
            const uint32_t cnt = 4u * (uint32_t)__popcll(B.tile_mask[t]);
            B.ids[tiles + t] = acc;
            if (t > 0) B.ids[t] = cnt;
            acc += cnt;
        }
    }
    if (threadIdx.x == blockDim.x - 1) {
        const uint32_t total = warp_sums[(blockDim.x >> 5) - 1];
        if (tiles > 0) B.ids[0] = total;
        B.counters[1] = total;
        B.counters[0] = 0;
    }
}

// raycast_writeids (kernel.cl:298-340): per tile, per empty 2x2 block (rows
// outer, columns inner) the four entries (x,y),(x+1,y),(x+1,y+1),(x,y+1),
// packed x | y<<16. One warp per tile.
__global__ void __launch_bounds__(256) k_hole_write(TargetBuffers B) {
    const uint32_t tiles = (uint32_t)B.tiles_x * (uint32_t)B.tiles_y;
    const uint32_t tile = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    if (tile >= tiles) return;
    const int lane = threadIdx.x & 31;
    const uint64_t m = B.tile_mask[tile];
    if (m == 0) return;
    const uint32_t base = 2u * tiles + B.ids[tiles + tile];
    const uint32_t x0 = (tile % (uint32_t)B.tiles_x) * 16u, y0 = (tile / (uint32_t)B.tiles_x) * 16u;
    for (int bit = lane; bit < 64; bit += 32) {
        if (!((m >> bit) & 1ull)) continue;
        const uint32_t rank = (uint32_t)__popcll(m & ((1ull << bit) - 1ull));
        const uint32_t i = bit & 7, j = bit >> 3;
        const uint32_t val = (x0 + 2u * i) + ((y0 + 2u * j) << 16);
        uint32_t* dst = B.ids + base + 4u * rank;
        dst[0] = val;
        dst[1] = val + 1u;
        dst[2] = val + 1u + (1u << 16);
        dst[3] = val + (1u << 16);
    }
}

// ----------------------------------------------------------- tracing --
// Persistent ray tracer. Each warp repeatedly takes a 32-ray packet from a
// global atomic work counter. Full mode: packets are 8x4 pixel tiles of the
// batch's views, in view order. Warp mode: first the hole list (32
// consecutive entries = eight neighbouring 2x2 blocks), then the 8x4 tiles of
// the refresh rectangle; holes inside the rectangle are left to it (both
// would store identical values).
//
// Shared memory: the node stack, then (when o.n_smem > 0) a copy of the
// octree's normal-node region, staged once per block by stage_prefix. The
// longest rays of a frame -- horizon rays skimming the periodic terrain up to
// VIEW_DIST_MAX -- fetch nothing else, ~1000 dependent fetches each, so
// their latency (the kernel's tail) drops from L2-hit to shared-memory
// latency per fetch.
template <int DEPTH, int BLOCK>
__device__ __forceinline__ Octree stage_octree(Octree o, uint64_t* mbar, uint32_t& fault, bool& staged) {
    stack_init<DEPTH>(svo_dsmem + threadIdx.x, BLOCK, o.root);
    staged = false;
    if (o.n_smem > 0) {
        o.smem_base = kStackLevels<DEPTH> * BLOCK;
        staged = stage_prefix(o.words, o.n_smem, o.smem_base, mbar, fault);
        if (!staged) o.n_smem = 0;
    }
    return o;
}

template <int DEPTH, int BLOCK, bool kVoxel>
__global__ void __launch_bounds__(BLOCK) k_trace_full(Octree o_in, const FullBatch* __restrict__ batch,
                                                    uint32_t* counter, uint32_t* fault_out) {
    __shared__ uint64_t mbar;
    const int lane = threadIdx.x & 31;
    uint32_t* stk = svo_dsmem + threadIdx.x;
    uint32_t fault = 0;
    bool staged;
    const Octree o = stage_octree<DEPTH, BLOCK>(o_in, &mbar, fault, staged);
    const uint32_t total = batch->total_packets;
    const int nv = batch->n_views;
    for (;;) {
        uint32_t p = 0;
        if (lane == 0) p = atomicAdd(counter, 1u);
        p = __shfl_sync(0xffffffffu, p, 0);
        if (p >= total) break;
        int v = 0;
        {  // view of packet p (views are few; binary search on packet_begin)
            int lo = 0, hi = nv - 1;
            while (lo < hi) {
                const int mid = (lo + hi + 1) >> 1;
                if (batch->v[mid].packet_begin <= p) lo = mid; else hi = mid - 1;
            }
            v = lo;
        }
        const FullView& fv = batch->v[v];
        const uint32_t q = p - fv.packet_begin;
        const int ps = fv.pw_shift;
        const int x = ((int)(q % (uint32_t)fv.packets_x) << ps) + (lane & ((1 << ps) - 1));
        const int y = (int)(q / (uint32_t)fv.packets_x) * (32 >> ps) + (lane >> ps);
        if (x < fv.res_x && y < fv.res_y) {
            const RayCam cam = fv.ray;
            const RayResult r = trace_ray<DEPTH, kVoxel>(o, cam, x, y, fv.res_x, fv.res_y, stk, BLOCK, fault);
            const size_t ofs = (size_t)y * fv.res_x + x;
            fv.col[ofs] = r.colour;
            fv.xyzw[ofs] = make_float4(r.hx, r.hy, r.hz, r.dist);
            if (kVoxel) fv.vox[ofs] = r.voxel;
            fv.bgrx[ofs] = colorize(r.colour);
        }
    }
    if (o_in.n_smem > 0 && !staged) stage_drain(&mbar);
    if (fault) atomicOr(fault_out, fault);
}

// kBgrx (learned frames): also writes the traced pixels' colourised output
// and, in w, the hit code instead of the distance; with a guide buffer it
// walks the pixels k_guide listed after the requested rays and the refresh
// tile, 32 list entries per packet, each ray starting at the pixel's guide
// distance -- the walks k_guide expects to be long (a depth edge nearby: the
// start comes from the near side) first, so the launch does not end on a long
// walk -- and finally commits the certified pixels' colour words and points.
// Requested pixels are unguided and neither walked nor certified, so every
// pixel is written at most once and the walks read nothing the launch writes.
template <int DEPTH, int BLOCK, bool kBgrx>
__global__ void __launch_bounds__(BLOCK) k_trace_warp(Octree o_in, const FrameParams* __restrict__ P,
                                                    TargetBuffers B, uint32_t* fault_out) {
    __shared__ uint64_t mbar;
    const int lane = threadIdx.x & 31;
    uint32_t* stk = svo_dsmem + threadIdx.x;
    uint32_t fault = 0;
    bool staged;
    const Octree o = stage_octree<DEPTH, BLOCK>(o_in, &mbar, fault, staged);  // the octree: no dependency
    grid_dep_wait();
    const int res_x = B.res_x, res_y = B.res_y;
    const uint32_t tiles = (uint32_t)B.tiles_x * (uint32_t)B.tiles_y;
    const uint32_t holes = B.counters[1];
    const uint32_t hole_packets = (holes + 31u) / 32u;
    const int ax = P->add_x, ay = P->add_y, xe = P->x_end, ye = P->y_end;
    const int ps = P->pw_shift, pw = 1 << ps, ph = 32 >> ps;
    const uint32_t rpx = (uint32_t)max(0, (xe - ax + pw - 1) / pw), rpy = (uint32_t)max(0, (ye - ay + ph - 1) / ph);
    const uint32_t fixed = hole_packets + rpx * rpy;
    const float* __restrict__ guide = kBgrx ? B.guide : nullptr;
    uint32_t n_walk[kWalkBuckets], p_walk[kWalkBuckets];
    uint32_t walk_packets = 0;
#pragma unroll
    for (int b = 0; b < kWalkBuckets; ++b) {
        n_walk[b] = guide ? min(B.counters[4 + b], B.walk_cap) : 0u;
        p_walk[b] = (n_walk[b] + 31u) / 32u;
        walk_packets += p_walk[b];
    }
    const uint32_t n_cert = guide ? min(B.counters[4 + kWalkBuckets], B.walk_cap) : 0u;
    const uint32_t p_cert = (n_cert + 31u) / 32u;
    const uint32_t total = fixed + walk_packets + p_cert;
    const RayCam cam = P->ray;
    float4* __restrict__ xyz = plane_xyz(B, P->cur);
    uint32_t* __restrict__ col = plane_col(B, P->cur);
    const size_t n_keys = (size_t)res_x * res_y;
    const uint32_t clear_chunks = (kBgrx && P->clear_keys) ? (uint32_t)((n_keys + 31u) / 32u) : 0u;
    if (clear_chunks && total == 0) {  // no packet to spread the chunks over
        for (size_t i = (size_t)blockIdx.x * BLOCK + threadIdx.x; i < n_keys; i += (size_t)gridDim.x * BLOCK)
            B.keys[i] = kKeyEmpty;
    }
    for (;;) {
        uint32_t p = 0;
        if (lane == 0) p = atomicAdd(B.counters, 1u);
        p = __shfl_sync(0xffffffffu, p, 0);
        if (p >= total) break;
        if (kBgrx && clear_chunks) {
            for (uint32_t c = p; c < clear_chunks; c += total) {
                const size_t i = (size_t)c * 32u + (uint32_t)lane;
                if (i < n_keys) B.keys[i] = kKeyEmpty;
            }
        }
        int x, y;
        bool valid;
        float s0 = 0.0f;
        if (kBgrx && p >= fixed) {
            uint32_t k = p - fixed;
            if (k < walk_packets) {  // the bucket of packet k, longest walks first
                int b = 0;
#pragma unroll
                for (int i = 0; i < kWalkBuckets - 1; ++i)
                    if (b == i && k >= p_walk[i]) {
                        k -= p_walk[i];
                        b = i + 1;
                    }
                const uint32_t e = k * 32u + (uint32_t)lane;
                const uint32_t nb = b == 0 ? n_walk[0] : (b == 1 ? n_walk[1] : (b == 2 ? n_walk[2] : n_walk[3]));
                valid = e < nb;
                const uint32_t xy = valid ? __ldg(B.walk_list + (size_t)b * B.walk_cap + e) : 0u;
                x = (int)(xy & 0xffffu);
                y = (int)(xy >> 16);
                if (valid && (x >= res_x || y >= res_y)) {
                    fault |= kFaultHoleEntry;
                    valid = false;
                }
                if (valid) {
                    s0 = __ldg(guide + (size_t)y * res_x + x);
                    valid = s0 >= 0.0f;
                }
            } else {  // certified pixels: commit the colour word and point k_guide left
                const uint32_t e = (k - walk_packets) * 32u + (uint32_t)lane;
                if (e < n_cert) {
                    const uint32_t xy = __ldg(B.cert_list + e);
                    const size_t ofs = (size_t)(xy >> 16) * res_x + (xy & 0xffffu);
                    if ((xy & 0xffffu) < (uint32_t)res_x && (xy >> 16) < (uint32_t)res_y) {
                        col[ofs] = __ldg(B.cert_col + ofs);
                        xyz[ofs] = __ldg(B.cert_xyz + ofs);
                    } else {
                        fault |= kFaultHoleEntry;
                    }
                }
                continue;
            }
        } else if (p < hole_packets) {
            const uint32_t e = p * 32u + (uint32_t)lane;
            valid = e < holes;
            const uint32_t xy = valid ? B.ids[2u * tiles + e] : 0u;
            x = (int)(xy & 0xffffu);
            y = (int)(xy >> 16);
            if (valid && (x >= res_x || y >= res_y)) {
                fault |= kFaultHoleEntry;
                valid = false;
            }
            if (x >= ax && x < xe && y >= ay && y < ye) valid = false;  // traced by the refresh tile
        } else {
            const uint32_t q = p - hole_packets;
            x = ax + (int)(q % rpx) * pw + (lane & (pw - 1));
            y = ay + (int)(q / rpx) * ph + (lane >> ps);
            valid = x < xe && y < ye;
        }
        if (valid) {
            // s0 = 0: the plain ray from the camera, bit for bit
            const RayResult r = trace_ray<DEPTH, false, kBgrx>(o, cam, x, y, res_x, res_y, stk, BLOCK, fault, s0);
            const size_t ofs = (size_t)y * res_x + x;
            col[ofs] = r.colour;
            xyz[ofs] = make_float4(r.hx, r.hy, r.hz, kBgrx ? r.code : r.dist);
            if (kBgrx) B.bgrx[ofs] = colorize(r.colour);
        }
    }
    if (o_in.n_smem > 0 && !staged) stage_drain(&mbar);
    if (fault) atomicOr(fault_out, fault);
}

// raycast_fine (kernel.cl:696-843) as raycast.h:235-261 would launch it
// (the reference ships the call disabled): work-items over (res/4 rounded up
// to 16) in x and y, each owning the 2x2 block at (coarse + 2*id) and
// tracing its first empty pixel (order (0,0),(1,0),(0,1),(1,1)), else pixel
// ((frame>>2)&1, (frame>>3)&1) of the block. Runs between the gather and the
// hole count. Packets: 8x4 work-items. res_x and res_y are multiples of 4
// (checked by the host), so no block crosses the frame edge.
template <int DEPTH, int BLOCK>
__global__ void __launch_bounds__(BLOCK) k_trace_coarse(Octree o_in, const FrameParams* __restrict__ P,
                                                      TargetBuffers B, uint32_t* fault_out) {
    __shared__ uint64_t mbar;
    const int lane = threadIdx.x & 31;
    uint32_t* stk = svo_dsmem + threadIdx.x;
    uint32_t fault = 0;
    bool staged;
    const Octree o = stage_octree<DEPTH, BLOCK>(o_in, &mbar, fault, staged);
    const int res_x = B.res_x, res_y = B.res_y;
    const int gx = (res_x / 4 + 15) / 16 * 16, gy = (res_y / 4 + 15) / 16 * 16;
    const uint32_t ppx = (uint32_t)gx / 8u, ppy = (uint32_t)gy / 4u;
    const uint32_t total = ppx * ppy;
    const int ax = P->coarse_x, ay = P->coarse_y, frame = P->frame;
    const RayCam cam = P->ray;
    float4* __restrict__ xyz = plane_xyz(B, P->cur);
    uint32_t* __restrict__ col = plane_col(B, P->cur);
    for (;;) {
        uint32_t p = 0;
        if (lane == 0) p = atomicAdd(B.counters + 2, 1u);
        p = __shfl_sync(0xffffffffu, p, 0);
        if (p >= total) break;
        const int bx = ax + 2 * ((int)(p % ppx) * 8 + (lane & 7));
        const int by = ay + 2 * ((int)(p / ppx) * 4 + (lane >> 3));
        if (bx < res_x && by < res_y) {
            int x = bx + ((frame >> 2) & 1), y = by + ((frame >> 3) & 1);
            for (int k = 0; k < 4; ++k) {
                if (col[(size_t)(by + (k >> 1)) * res_x + bx + (k & 1)] == kEmptyPixel) {
                    x = bx + (k & 1);
                    y = by + (k >> 1);
                    break;
                }
            }
            const RayResult r = trace_ray<DEPTH, false>(o, cam, x, y, res_x, res_y, stk, BLOCK, fault);
            const size_t ofs = (size_t)y * res_x + x;
            col[ofs] = r.colour;
            xyz[ofs] = make_float4(r.hx, r.hy, r.hz, r.dist);
        }
    }
    if (o_in.n_smem > 0 && !staged) stage_drain(&mbar);
    if (fault) atomicOr(fault_out, fault);
}

// ----------------------------------------------- filter + colourise ----
// raycast_fillhole2 (kernel.cl:404-470) reading the unfiltered current plane
// and writing the displayed plane, fused with raycast_colorize.
__device__ __forceinline__ uint32_t read_lin(const uint32_t* __restrict__ s, const uint32_t* __restrict__ next,
                                             long long o, long long n) {
    // The reference addresses plane 0 linearly; reads past its end land in
    // plane 1: empty unless the alternating cache target writes it.
    if (o >= 0 && o < n) return __ldg(s + o);
    if (next && o >= n && o < 2 * n) return __ldg(next + (o - n));
    return kEmptyPixel;
}

// The block's 32x8 pixels and a 2-pixel halo are staged in shared memory
// once; the neighbour reads of the filter come from there. A read the tile
// cannot answer -- the reference's linear address running past the end of a
// row (into the next one) or past the last row (into plane 1) -- goes to
// global memory as read_lin has it.
__global__ void __launch_bounds__(256) k_fill_colorize(const FrameParams* __restrict__ P, TargetBuffers B) {
    constexpr int kTW = 32, kTH = 8, kHalo = 2;
    __shared__ uint32_t tile[kTH + 2 * kHalo][kTW + 2 * kHalo];
    const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
    const int x0 = blockIdx.x * kTW, y0 = blockIdx.y * kTH;
    const int idx = x0 + tx, idy = y0 + ty;
    const int res_x = B.res_x, res_y = B.res_y;
    const uint32_t* __restrict__ s = plane_col(B, P->cur);
    const uint32_t* __restrict__ next = P->fill_past >= 0 ? plane_col(B, P->fill_past) : nullptr;
    for (int i = threadIdx.x; i < (kTH + 2 * kHalo) * (kTW + 2 * kHalo); i += 256) {
        const int wx = i % (kTW + 2 * kHalo), wy = i / (kTW + 2 * kHalo);
        const int gx = x0 + wx - kHalo, gy = y0 + wy - kHalo;
        tile[wy][wx] = (gx >= 0 && gx < res_x && gy >= 0 && gy < res_y) ? __ldg(s + (size_t)gy * res_x + gx)
                                                                         : kEmptyPixel;
    }
    __syncthreads();
    if (idx >= res_x || idy >= res_y) return;
    auto at = [&](int dx, int dy) -> uint32_t { return tile[ty + kHalo + dy][tx + kHalo + dx]; };
    const long long n = (long long)res_x * res_y;
    const long long ofs = (long long)idy * res_x + idx;
    uint32_t col = at(0, 0);
    if (col == kEmptyPixel && idx < res_x - 1 && idy < res_y - 1 && idx > 1 && idy > 1) {
        const int c1 = (int)at(1, 0), c2 = (int)at(-1, 0);
        const int c3 = (int)at(0, 1), c4 = (int)at(0, -1);
        const bool s1 = (uint32_t)c1 != kEmptyPixel, s2 = (uint32_t)c2 != kEmptyPixel;
        const bool s3 = (uint32_t)c3 != kEmptyPixel, s4 = (uint32_t)c4 != kEmptyPixel;
        if (s1 && s2 && s3 && s4) {
            col = (uint32_t)((c1 & 3) + ((((c1 & 0xfc) + (c2 & 0xfc) + (c3 & 0xfc) + (c4 & 0xfc)) >> 2) & 0xfc));
        } else if (s1 && s2) {
            col = (uint32_t)((c1 & 3) + ((((c1 & 0xfc) + (c2 & 0xfc)) >> 1) & 0xfc));
        } else if (s3 && s4) {
            col = (uint32_t)((c3 & 3) + ((((c3 & 0xfc) + (c4 & 0xfc)) >> 1) & 0xfc));
        } else {
            for (int i = 0; i < 4; ++i) {  // all four inside the frame here
                col = at(i & 1, (i >> 1) & 1);
                if (col != kEmptyPixel) break;
            }
            if (col == kEmptyPixel) {
                for (int i = -2; i < 3 && col == kEmptyPixel; ++i)
                    for (int j = -2; j < 3; ++j) {
                        const int xi = idx + i, yj = idy + j;
                        col = (xi < res_x && yj < res_y) ? at(i, j)
                                                         : read_lin(s, next, ofs + i + (long long)j * res_x, n);
                        if (col != kEmptyPixel) break;
                    }
            }
        }
    }
    B.disp[ofs] = col;
    B.bgrx[ofs] = colorize(col);
}

}  // namespace svo
