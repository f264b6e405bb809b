// svo_net.cuh -- the learned reconstruction stage of the warp pipeline.
//
// The reference renderer fills the pixels that reprojection left empty with a
// fixed 3x3 filter (raycast_fillhole2, kernel.cl:404-470) and traces every
// 2x2 hole block (raycast_counthole/writeids/holes). The learned stage
// replaces both decisions: a small convolutional net looks at the warped
// frame (colour, depth, hole mask, reprojection motion) and outputs a colour
// plus a confidence per pixel; pixels below the confidence threshold are
// traced exactly like the reference's holes, the rest show the net's colour.
//
// Net: four 3x3 same-size convolutions, zero padding at the frame border,
// channels 8 -> 16 -> 16 -> 16 -> 4, ReLU after the first three; the output's
// first three channels are added to the input colour (a residual), the fourth
// is the confidence logit. Weights, features and hidden activations are
// bfloat16, sums FP32.
//
// Kernels:
//   k_net_features    features of every pixel of the current plane (the
//                     training tap)
//   k_net_infer       the whole net fused per 56x24-pixel tile on the tensor
//                     cores: tcgen05.mma (kind::f16, bf16 x bf16 -> fp32 in
//                     tensor memory) as an implicit GEMM, activations staged
//                     in shared memory between layers
//   k_net_conv_fwd    FP32 CUDA-core forward of one layer (the reference the
//                     tensor-core forward is checked against)
//   k_net_loss, k_net_reduce, k_net_adam
//                     the training loss, a deterministic reduction and Adam;
//                     the backward convolutions are in svo_net_train.cuh
#pragma once
#include <cstdint>
#include <cstring>

#include "svo_kernels.cuh"

namespace svo {

constexpr int kNetLayers = 4;
constexpr int kNetParams = 6388;
__host__ __device__ constexpr int net_cin(int l) { return l == 0 ? 8 : 16; }
__host__ __device__ constexpr int net_cout(int l) { return l == 3 ? 4 : 16; }
// Flat parameter layout: per layer W [9][cin][cout] then b [cout].
__host__ __device__ constexpr int net_w_off(int l) {
    return l == 0 ? 0 : net_w_off(l - 1) + 9 * net_cin(l - 1) * net_cout(l - 1) + net_cout(l - 1);
}
__host__ __device__ constexpr int net_b_off(int l) { return net_w_off(l) + 9 * net_cin(l) * net_cout(l); }
static_assert(net_b_off(3) + 4 == kNetParams, "parameter layout");

// Round to bfloat16, nearest even (finite inputs): the bit pattern and the
// value it stands for.
__host__ __device__ __forceinline__ uint32_t bf16_bits(float x) {
    uint32_t u;
    memcpy(&u, &x, 4);
    return (u + 0x7FFFu + ((u >> 16) & 1u)) >> 16;
}
__host__ __device__ __forceinline__ float bf16_round(float x) {
    const uint32_t u = bf16_bits(x) << 16;
    float r;
    memcpy(&r, &u, 4);
    return r;
}

// --------------------------------------------------------------- features --
// Per pixel of the current plane after reprojection:
//   0-2  colour of the warped pixel (colourised, /255), 0 when empty
//   3    log2(1 + distance from the camera) / 16, 0 when empty
//   4    1 when the pixel is empty (a hole), else 0
//   5    reprojection motion: distance in pixels between where the cached
//        point appears now and where it appeared from the previous camera,
//        clamped to 8 and divided by 8 (1 when it was behind that camera)
//   6    distance in pixels between the pixel centre (which the pixel's own
//        ray passes through) and where the cached point projects now,
//        clamped to 1; 0 when empty
//   7    elevation of the pixel's ray: (1 + world-y of its unit direction)/2,
//        for every pixel (rays above the horizon of the periodic terrain
//        meet nothing)
// (The previous camera travels in FrameParams: prev_pos, prev_vx/vy/vz.)
// net_load fetches what net_compute needs, so callers can issue the loads
// of several pixels before using any of them.
struct NetPixel {
    uint32_t c;
    float4 q;
};

__device__ __forceinline__ NetPixel net_load(const FrameParams& P, const TargetBuffers& B, int x, int y) {
    const size_t ofs = (size_t)y * B.res_x + x;
    NetPixel px;
    px.c = __ldg(plane_col(B, P.cur) + ofs);
    px.q = __ldg(plane_xyz(B, P.cur) + ofs);
    return px;
}

// Fast approximate arithmetic is enough here: the features are rounded to
// bf16 before use, and inference and training compute them with this one
// function.
__device__ __forceinline__ float fast_len(float sq) { return sq * rsqrtf(fmaxf(sq, 1e-30f)); }

__device__ __forceinline__ void net_compute(const FrameParams& P, int res_x, int res_y, int x, int y,
                                            const NetPixel& px, float f[8]) {
#pragma unroll
    for (int i = 0; i < 8; ++i) f[i] = 0.0f;
    const float ry = (float)res_y, inv_ry = __fdividef(1.0f, ry);
    {
        const float d1x = __fmaf_rn((float)(x - (res_x >> 1)) + 0.5f, P.ray.fovx * inv_ry, 0.0f);
        const float d1y = __fmaf_rn((float)(y - (res_y >> 1)) + 0.5f, P.ray.fovy * inv_ry, 0.0f);
        const float dx = __fmaf_rn(d1x, P.ray.mxx, __fmaf_rn(d1y, P.ray.mxy, P.ray.mxz));
        const float dy = __fmaf_rn(d1x, P.ray.myx, __fmaf_rn(d1y, P.ray.myy, P.ray.myz));
        const float dz = __fmaf_rn(d1x, P.ray.mzx, __fmaf_rn(d1y, P.ray.mzy, P.ray.mzz));
        f[7] = __fmaf_rn(0.5f * dy, rsqrtf(__fmaf_rn(dx, dx, __fmaf_rn(dy, dy, dz * dz))), 0.5f);
    }
    if (px.c == kEmptyPixel) {
        f[4] = 1.0f;
        return;
    }
    const uint32_t bgrx = colorize(px.c);
    f[0] = (float)((bgrx >> 16) & 255u) * (1.0f / 255.0f);
    f[1] = (float)((bgrx >> 8) & 255u) * (1.0f / 255.0f);
    f[2] = (float)(bgrx & 255u) * (1.0f / 255.0f);
    const float4 q = px.q;
    const float ax = q.x - P.ray.px, ay = q.y - P.ray.py, az = q.z - P.ray.pz;
    const float d = fast_len(__fmaf_rn(ax, ax, __fmaf_rn(ay, ay, az * az)));
    f[3] = fminf(__log2f(1.0f + d) * (1.0f / 16.0f), 1.0f);
    const float zc = __fmaf_rn(ax, P.vz[0], __fmaf_rn(ay, P.vz[1], az * P.vz[2]));
    float sxc = 0.0f, syc = 0.0f;
    if (zc >= 0.05f) {
        const float iz = __fdividef(ry, zc);
        sxc = __fmaf_rn(ax, P.vx[0], __fmaf_rn(ay, P.vx[1], az * P.vx[2])) * iz;
        syc = __fmaf_rn(ax, P.vy[0], __fmaf_rn(ay, P.vy[1], az * P.vy[2])) * iz;
        const float ex = sxc + 0.5f * (float)res_x - ((float)x + 0.5f);
        const float ey = syc + 0.5f * ry - ((float)y + 0.5f);
        f[6] = fminf(fast_len(__fmaf_rn(ex, ex, ey * ey)), 1.0f);
    }
    float m = 0.0f;
    if (P.have_prev_view) {
        m = 8.0f;
        const float bx = q.x - P.prev_pos[0], by = q.y - P.prev_pos[1], bz = q.z - P.prev_pos[2];
        const float zp = __fmaf_rn(bx, P.prev_vz[0], __fmaf_rn(by, P.prev_vz[1], bz * P.prev_vz[2]));
        if (zp >= 0.05f && zc >= 0.05f) {
            const float iz = __fdividef(ry, zp);
            const float sxp = __fmaf_rn(bx, P.prev_vx[0], __fmaf_rn(by, P.prev_vx[1], bz * P.prev_vx[2])) * iz;
            const float syp = __fmaf_rn(bx, P.prev_vy[0], __fmaf_rn(by, P.prev_vy[1], bz * P.prev_vy[2])) * iz;
            const float ddx = sxc - sxp, ddy = syc - syp;
            m = fminf(fast_len(__fmaf_rn(ddx, ddx, ddy * ddy)), 8.0f);
        }
    }
    f[5] = m * 0.125f;
}

// Training tap: features of every pixel, planar [8][res_y*res_x], FP32.
__global__ void __launch_bounds__(256) k_net_features(const FrameParams* __restrict__ P, TargetBuffers B,
                                                      float* out) {
    const int x = blockIdx.x * 32 + (threadIdx.x & 31), y = blockIdx.y * 8 + (threadIdx.x >> 5);
    if (x >= B.res_x || y >= B.res_y) return;
    const FrameParams p = *P;
    float f[8];
    net_compute(p, B.res_x, B.res_y, x, y, net_load(p, B, x, y), f);
    const size_t n = (size_t)B.res_x * B.res_y, ofs = (size_t)y * B.res_x + x;
#pragma unroll
    for (int i = 0; i < 8; ++i) out[i * n + ofs] = f[i];
}

// ------------------------------------------------- weight preparation --
// From the FP32 master parameters: a bf16-rounded FP32 copy of the weights
// (CUDA-core path) and the tensor-core operand image (bf16, one 512-byte
// block per MMA: [co group 2][ci chunk 2][8 co][8 ci], K-major core matrices).
// Layer 0 has 8 input channels, so one MMA covers two taps (ci chunk 0 = tap
// 2m, chunk 1 = tap 2m+1; the fifth MMA pairs tap 8 with zeros); layers 1-3
// take one tap per MMA; layer 3's 4 output channels are padded to 16.
__host__ __device__ constexpr int net_mmas(int l) { return l == 0 ? 5 : 9; }
__host__ __device__ constexpr int net_mma_base(int l) { return l == 0 ? 0 : 5 + 9 * (l - 1); }
constexpr int kNetMmaTotal = 32;
constexpr int kNetBias = 16 + 16 + 16 + 4;

__global__ void k_net_prepare(const float* __restrict__ params, float* __restrict__ wr, uint16_t* __restrict__ packed,
                              float* __restrict__ bias) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < kNetParams) wr[i] = bf16_round(params[i]);
    if (i < kNetMmaTotal * 256) {
        const int mma = i >> 8, e = i & 255;
        const int ng = e >> 7, kc = (e >> 6) & 1, r = (e >> 3) & 7, k = e & 7;
        int l = 3;
        while (l > 0 && mma < net_mma_base(l)) --l;
        const int m = mma - net_mma_base(l);
        const int co = ng * 8 + r;
        float v = 0.0f;
        if (co < net_cout(l)) {
            int tap, ci;
            if (l == 0) {
                tap = 2 * m + kc;
                ci = k;
            } else {
                tap = m;
                ci = kc * 8 + k;
            }
            if (tap < 9) v = params[net_w_off(l) + (tap * net_cin(l) + ci) * net_cout(l) + co];
        }
        packed[i] = (uint16_t)bf16_bits(v);
    }
    if (i < kNetBias) {
        const int l = i < 16 ? 0 : (i < 32 ? 1 : (i < 48 ? 2 : 3));
        bias[i] = params[net_b_off(l) + (i - 16 * l)];
    }
}

// ------------------------------------------------ tcgen05 primitives --
__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

// Shared-memory matrix descriptor, no swizzle, K-major canonical layout:
// 8-row x 16-byte core matrices; lbo = byte distance between the two core
// matrices of a row group along K, sbo = byte distance between row groups.
__device__ __forceinline__ uint64_t tc_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
    return (uint64_t)((saddr & 0x3FFFFu) >> 4) | ((uint64_t)((lbo & 0x3FFFFu) >> 4) << 16) |
           ((uint64_t)((sbo & 0x3FFFFu) >> 4) << 32) | (1ull << 46);
}

// Instruction descriptor, kind::f16: D f32, A and B bf16, both K-major,
// N = 16, M = 128.
constexpr uint32_t kNetIdesc = (1u << 4) | (1u << 7) | (1u << 10) | ((16u >> 3) << 17) | ((128u >> 4) << 24);

__device__ __forceinline__ void tc_mma(uint32_t d_tmem, uint64_t a, uint64_t b, uint32_t accumulate) {
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}"
        :
        : "r"(d_tmem), "l"(a), "l"(b), "r"(kNetIdesc), "r"(accumulate)
        : "memory");
}

__device__ __forceinline__ void tc_commit(uint32_t mbar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(mbar)
                 : "memory");
}

// 16 columns of this warp's 32 lanes; the registers are valid only after
// tc_wait_ld (so several loads can be in flight together).
__device__ __forceinline__ void tc_ld16_nowait(uint32_t taddr, uint32_t r[16]) {
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr));
}
__device__ __forceinline__ void tc_wait_ld() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }

__device__ __forceinline__ void tc_ld16(uint32_t taddr, float v[16]) {
    uint32_t r[16];
    tc_ld16_nowait(taddr, r);
    tc_wait_ld();
#pragma unroll
    for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

__device__ __forceinline__ void tc_ld4(uint32_t taddr, float v[4]) {
    uint32_t r[4];
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x4.b32 {%0,%1,%2,%3}, [%4];"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
                 : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int i = 0; i < 4; ++i) v[i] = __uint_as_float(r[i]);
}

// try_wait that may suspend the thread for up to ~20 us while the phase is
// incomplete (fewer spinning instructions competing with the MMA issuer).
__device__ __forceinline__ bool mbar_try_wait_sleep(uint32_t bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, 20000;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(bar), "r"(parity)
        : "memory");
    return ok != 0;
}

// Bounded wait on an mbarrier phase (~0.5 s), false on timeout.
__device__ __forceinline__ bool mbar_wait_phase(uint32_t bar, uint32_t parity) {
    if (mbar_try_wait_sleep(bar, parity)) return true;
    const uint64_t t0 = global_ns();
    for (;;) {
        if (mbar_try_wait_sleep(bar, parity)) return true;
        if (global_ns() - t0 > 500000000ull) return false;
    }
}

// Operand-layout self-check, run once per device before the first learned
// frame: one 128x16x16 MMA on small integers laid out exactly as k_net_infer
// lays out its operands (A: two 8-channel planes 2048 bytes apart, B: the
// packed weight block), compared with the CUDA-core product. The A region is
// 64 KB so that every address the descriptors can form stays inside it.
// result[0] = mismatching elements, result[1] = 1 when the wait timed out.
constexpr int kNetProbeSmem = 65536 + 512;

__global__ void __launch_bounds__(128, 1) k_net_probe(uint32_t* result) {
    __shared__ uint64_t mbar;
    __shared__ uint32_t tmem_base_s;
    uint8_t* smem = reinterpret_cast<uint8_t*>(svo_dsmem);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    uint16_t* a = reinterpret_cast<uint16_t*>(smem);
    uint16_t* b = reinterpret_cast<uint16_t*>(smem + 65536);
    for (int i = tid; i < 32768; i += 128) a[i] = 0;
    __syncthreads();
    // A[r][k]: chunk k/8 at byte (k/8)*2048 + r*16 + (k%8)*2
    for (int i = tid; i < 128 * 16; i += 128) {
        const int r = i >> 4, k = i & 15;
        a[((k >> 3) * 2048 + r * 16) / 2 + (k & 7)] = (uint16_t)bf16_bits((float)((r * 3 + k * 5) % 7 - 3));
    }
    // B[n][k] in the packed block layout [n/8][k/8][n%8][k%8]
    for (int i = tid; i < 256; i += 128) {
        const int n = i >> 4, k = i & 15;
        b[(n >> 3) * 128 + (k >> 3) * 64 + (n & 7) * 8 + (k & 7)] = (uint16_t)bf16_bits((float)((n * 2 + k) % 5 - 2));
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_addr(&tmem_base_s)),
                     "r"(32)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    if (tid == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_addr(&mbar)) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    fence_async_smem();
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = tmem_base_s;
    if (tid == 0) {
        tc_mma(tmem, tc_desc(smem_addr(a), 2048u, 128u), tc_desc(smem_addr(b), 128u, 256u), 0u);
        tc_commit(smem_addr(&mbar));
    }
    const bool ok = __syncthreads_and(mbar_wait_phase(smem_addr(&mbar), 0) ? 1 : 0) != 0;
    tc_fence_after();
    uint32_t bad = 0;
    if (ok) {
        float v[16];
        tc_ld16(tmem + ((uint32_t)(32 * warp) << 16), v);
        const int r = 32 * warp + lane;
        for (int n = 0; n < 16; ++n) {
            float e = 0.0f;
            for (int k = 0; k < 16; ++k) e += (float)((r * 3 + k * 5) % 7 - 3) * (float)((n * 2 + k) % 5 - 2);
            if (v[n] != e) ++bad;
        }
    }
    if (bad) atomicAdd(result, bad);
    if (!ok && tid == 0) result[1] = 1;
    tc_fence_before();
    __syncthreads();
    if (warp == 0) {
        tc_fence_after();
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(32) : "memory");
    }
}

// ------------------------------------------------ fused inference --
// One CTA (512 threads) per SM walks 56x24-pixel output tiles. A tile's input
// window is 64x32 positions (a 4-pixel halo for the four 3x3 layers), stored
// as "positions" p = row*64 + col. Activations live in shared memory as
// planes of 8 bf16 channels (16 bytes per position, positions consecutive),
// with a zeroed guard of 16 positions before and after each plane.
//
// Layer l computes output rows [l+1, 31-l) -- (15-l) blocks of 128
// consecutive positions -- as D[128 x 16] = sum over MMAs of A[128 x 16] *
// B[16 x 16]: A for tap (dy,dx) is the input planes read from position
// p + dy*64 + dx, i.e. the same matrix descriptor shifted by that many
// 16-byte rows (an implicit GEMM with no im2col copy). Positions whose column
// wraps into the next row are computed and never used. Each block
// accumulates into its own 16 columns of tensor memory; four threads issue a
// layer's MMAs (blocks round-robin), each committing to its own mbarrier.
// Each group of four warps waits for its issuer's blocks only, reads their
// accumulators back (warp w reads tensor-memory lanes 32*(w%4)..+31), adds
// the bias, applies ReLU, zeroes the positions outside the frame (the border
// padding) and stores bf16 into the other buffer. The last layer writes the
// outputs.
//
// The 8-channel input planes are double-buffered: while the tensor core runs
// a layer's MMAs, every thread computes a quarter of the next tile's input
// features into the other input plane, so the feature loads and arithmetic
// overlap the MMAs.
constexpr int kNetTW = 64, kNetTH = 32, kNetPos = kNetTW * kNetTH;
constexpr int kNetGuard = 16;
constexpr int kNetPlaneBytes = (kNetPos + 2 * kNetGuard) * 16;  // 33280
constexpr int kNetOutW = kNetTW - 8, kNetOutH = kNetTH - 8;      // 56 x 24
constexpr int kNetSmemA = 0;                                     // 2 planes (16 channels)
constexpr int kNetSmemB = 2 * kNetPlaneBytes;                    // 2 planes
constexpr int kNetSmemX = 4 * kNetPlaneBytes;                    // 2 input planes (8 channels each)
constexpr int kNetSmemW = 6 * kNetPlaneBytes;                    // 32 x 512 B
constexpr int kNetSmemBias = kNetSmemW + kNetMmaTotal * 512;     // 52 floats
constexpr int kNetSmemBytes = kNetSmemBias + 256;                // 216320
constexpr int kNetTmemCols = 256;
constexpr int kNetThreads = 512;
constexpr int kNetWarps = kNetThreads / 32;
constexpr int kNetPer = kNetPos / kNetThreads;  // input positions per thread and tile (one per layer)
constexpr int kNetIssuers = 4;                   // threads (lane 0 of warps 0-3) issuing each layer's MMAs
static_assert(kNetPer == kNetLayers, "one slice of the next tile's input per layer");

// ------------------------------------------------- guided walks --
// A guided learned frame walks a pixel's ray from just in front of the
// nearest cached surface around it instead of from the camera: the start
// distance is the smallest camera distance of the reprojected points in the
// pixel's 3x3 neighbourhood, less kGuideMargin cells of the level of detail
// at that distance (half that smallest distance at the edge of a hole region). A cached point that is a ray end rather than a hit (the
// ray left the volume through its top or bottom, or reached the view
// distance limit) bounds its neighbours the same way: their rays are walked
// from just in front of where it ended. A pixel with no cached point around
// it is unguided and left to the net, which colours it or requests a full
// ray. The walk is exact unless a surface the cache has not seen lies in
// front of the start; the refresh tile and the requested rays keep tracing
// from the camera.
// A pixel at the edge of a hole region -- at least kGuideHoleCount of its
// 3x3 neighbourhood are pixels of the frame that reprojection left without a
// point -- is where a surface the cache never saw, newly uncovered by the
// camera's motion, most often lies in front of the cached points, and often
// far in front: its walk starts at half the 3x3 minimum distance instead.
// (Oracle experiment on the fast-motion camera path, 1920x1024, frames 2-21,
// every unguided pixel traced: 35.5 dB against the full raycast without the
// rule, 38.5 dB with it, 39.2 dB when any single hole counts; a wider margin
// of 16 or 32 cells gains nothing. On the orbit the rule costs 4% more node
// fetches, 12% when any single hole -- a splat crack -- counts.)
// The margin: 2 cells cost 7.5% fewer loop iterations than 4 at 0.15 dB on
// the fast-motion path (oracle, 1920x1024, frames 4-19: 37.98 -> 37.83 dB;
// orbit 58.3 -> 56.5 dB); 1 cell, 13% fewer at 0.6 dB; none doubles the
// pixels whose walk misses their voxel.
constexpr float kGuideMargin = 2.0f;        // cells of the start distance's level of detail
constexpr float kGuideNearHole = 0.5f;      // start distance factor at the edge of a hole region
constexpr int kGuideHoleCount = 3;          // holes in the 3x3 that make a hole region
// Walk buckets by the cells between the start and the pixel's own point: a
// depth edge (> kGuideLong, the start taken from the near side; such walks
// cost 4.4x the others in an oracle experiment), then > kGuideMid, >
// kGuideShort and the rest; the tracer runs the buckets in that order, so
// walks of similar length share warps. A pixel without an own point (a hole
// the walk fills) goes to the first bucket too: its length is unknown, and
// near the horizon such walks run through many periods of the terrain
// (150-400 loop iterations against 7.6 on average; an oracle model of the
// persistent tracer's queue put them in its last packets, where one of them
// held an SM for a quarter of the launch).
constexpr float kGuideLong = 64.0f;
constexpr float kGuideMid = 16.0f;
constexpr float kGuideShort = 6.0f;
constexpr int kGuideBW = 32, kGuideBH = 8;  // pixels per block (whole ray packets of every packet shape)

// Certified reprojection: a guided pixel needs no walk when its own ray
// provably meets a face a cached hit point of its neighbourhood lies on.
// Every cached point carries its hit code in w (level L of the hit cell, edge
// s = 2^L raypos units, and the signs of the ray that found it); the point
// lies on the cell's entry face, the one plane of its three coordinates that
// is a multiple of s, which the old ray crossed in the direction of its sign.
// The pixel's ray (the ray kernels' direction, not normalised) meets that
// plane at parameter t; the candidate passes when the ray crosses the plane
// the same way, t > 0, the other two coordinates of the meeting point lie
// inside the face with a margin of s/64, the level of detail at the meeting
// distance is L a thirty-second either side of it, and that distance is at
// most kCertifyGap cells behind the 3x3 minimum distance (nothing cached lies
// in front) -- each test cross-multiplied, see certify_pixel. The candidates are the cached points of the pixel and of its
// four neighbours. The nearest passing candidate (smallest t; the first in row order
// on a tie) gives the pixel's colour word (0xff000000 | colour byte), point
// and code. Only pixels outside the refresh tile with no hole in their 3x3
// are certified. An exact face test alone certified 40% of the orbit's
// pixels, 3.4% of them wrongly (a surface the cache missed in front of the
// face); with the gap test 24-26% on both camera paths, 0.3-0.4% wrongly
// (oracle experiments at 960x512). Every operation is one IEEE binary32
// operation; the CPU oracle repeats them.
constexpr float kGuideCertified = -2.0f;  // guide value of a certified pixel
constexpr float kCertifyGap = 2.0f;       // cells

// The walk's lodswitch doublings in closed form: 1 + the smallest k >= 0
// with s <= sw * 2^k (sw = 2 * res_x), at most 24. For s > sw, with
// s = ms * 2^es and sw = mw * 2^ew (mantissas in [1, 2)), k = es - ew when
// ms <= mw, else es - ew + 1; the mantissas compare as their low 23 bits.
__device__ __forceinline__ int lod_at(float s, int res_x) {
    const float sw = (float)(2 * res_x);
    if (!(s > sw)) return 1;
    const int bs = __float_as_int(s), bw = __float_as_int(sw);
    const int k = ((bs >> 23) - (bw >> 23)) + ((bs & 0x7fffff) > (bw & 0x7fffff) ? 1 : 0);
    return min(1 + k, 24);
}

// Candidate data of the halo, one array per field (conflict-free reads): the
// parts of the face test that do not depend on the pixel's ray, computed once
// per cached point as the halo is loaded.
struct CertHalo {
    uint8_t face[kGuideBH + 2][kGuideBW + 2];  // bit 7: a candidate; bits 0-1 axis; bit 2 the old ray's sign
    uint8_t level[kGuideBH + 2][kGuideBW + 2];
    float plane[kGuideBH + 2][kGuideBW + 2];   // the face's coordinate on its axis (raypos units)
    float lo1[kGuideBH + 2][kGuideBW + 2];     // the cell's low corner on the other two axes, in axis order
    float lo2[kGuideBH + 2][kGuideBW + 2];
    uint32_t col[kGuideBH + 2][kGuideBW + 2];
};

// The entry face of a cached point with hit code `code` (see certify_pixel):
// the one coordinate (raypos units) that is a multiple of the hit cell's
// edge. Writes the halo entry (face byte 0: no candidate).
__device__ __forceinline__ void cert_face(CertHalo& h, int wy, int wx, uint32_t c, float4 q) {
    uint8_t face = 0, lv = 0;
    float pl = 0.0f, l1 = 0.0f, l2 = 0.0f;
    if (c != kEmptyPixel && q.w >= 0.0f) {
        const int ic = (int)q.w;
        const int L = ic & 31;
        const uint32_t sb = (uint32_t)ic >> 5;
        if (L <= 23) {
            const float cs = __int_as_float((127 + L) << 23), inv = __int_as_float((127 - L) << 23);
            const float p[3] = {__fmul_rn(q.x, 16.0f), __fmul_rn(q.y, 16.0f), __fmul_rn(q.z, 16.0f)};
            float f[3];
            int axis = -1, on = 0;
#pragma unroll
            for (int a = 0; a < 3; ++a) {
                f[a] = floorf(__fmul_rn(p[a], inv));
                if (__fmul_rn(f[a], cs) == p[a]) {
                    axis = a;
                    ++on;
                }
            }
            if (on == 1) {
                face = (uint8_t)(0x80u | (uint32_t)axis | (((sb >> axis) & 1u) << 2));
                lv = (uint8_t)L;
                pl = axis == 0 ? p[0] : (axis == 1 ? p[1] : p[2]);
                const int b1 = axis == 0 ? 1 : 0, b2 = axis == 2 ? 1 : 2;
                l1 = __fmul_rn(b1 == 0 ? f[0] : f[1], cs);
                l2 = __fmul_rn(b2 == 1 ? f[1] : f[2], cs);
            }
        }
    }
    h.face[wy][wx] = face;
    h.level[wy][wx] = lv;
    h.plane[wy][wx] = pl;
    h.lo1[wy][wx] = l1;
    h.lo2[wy][wx] = l2;
    h.col[wy][wx] = c;
}

// The candidates are the pixel's own cached point and its four neighbours'
// (the four diagonal neighbours added 3% of the certified pixels for 80% more
// work in an oracle experiment); hx, hy = the pixel's halo position. The tests
// compare cross-multiplied quantities instead of dividing: with n = |plane -
// camera| and A = |d along the face's axis| the meeting parameter is t = n/A,
// the meeting distance n*|d|/A (compared squared), and one division is left,
// for the winner's point. d1x, d1y: the ray kernels' per-column and per-row
// direction terms.
__device__ __forceinline__ bool certify_pixel(const RayCam& cam, int res_x, float d1x, float d1y, const CertHalo& h,
                                              int hx, int hy, float near_s, uint32_t& out_col, float4& out_q) {
    const float d[3] = {__fadd_rn(__fadd_rn(__fmul_rn(d1x, cam.mxx), __fmul_rn(d1y, cam.mxy)), cam.mxz),
                        __fadd_rn(__fadd_rn(__fmul_rn(d1x, cam.myx), __fmul_rn(d1y, cam.myy)), cam.myz),
                        __fadd_rn(__fadd_rn(__fmul_rn(d1x, cam.mzx), __fmul_rn(d1y, cam.mzy)), cam.mzz)};
    const float c16[3] = {__fmul_rn(cam.px, 16.0f), __fmul_rn(cam.py, 16.0f), __fmul_rn(cam.pz, 16.0f)};
    const float dl2 = __fadd_rn(__fadd_rn(__fmul_rn(d[0], d[0]), __fmul_rn(d[1], d[1])), __fmul_rn(d[2], d[2]));
    const float sw1 = (float)(2 * res_x);  // the level-of-detail distance of level 1
    float bn = 1.0f, ba = 0.0f;            // best t = bn / ba (none yet: infinite)
    int bk = -1;
#pragma unroll 1
    for (int k = 0; k < 5; ++k) {  // up, left, own, right, down (row order)
        const int cy = hy + (k == 0 ? -1 : (k == 4 ? 1 : 0)), cx = hx + (k == 1 ? -1 : (k == 3 ? 1 : 0));
        const uint32_t face = h.face[cy][cx];
        if (!(face & 0x80u)) continue;
        const int axis = (int)(face & 3u);
        const bool neg = (face & 4u) != 0;
        const float da = axis == 0 ? d[0] : (axis == 1 ? d[1] : d[2]);
        if (neg ? !(da < 0.0f) : !(da > 0.0f)) continue;
        const float ca = axis == 0 ? c16[0] : (axis == 1 ? c16[1] : c16[2]);
        const float num = __fsub_rn(h.plane[cy][cx], ca);
        const float n = neg ? -num : num, A = neg ? -da : da;  // t = n / A
        if (!(n > 0.0f)) continue;
        if (!(__fmul_rn(n, ba) < __fmul_rn(bn, A))) continue;  // not nearer than the best so far
        const int L = h.level[cy][cx];
        const float cs = __int_as_float((127 + L) << 23);
        // meeting distance n*|d|/A: gap and level-of-detail tests squared
        const float nd2 = __fmul_rn(__fmul_rn(n, n), dl2);
        const float gap = __fmul_rn(__fadd_rn(near_s, __fmul_rn(kCertifyGap, cs)), A);
        if (!(nd2 <= __fmul_rn(gap, gap))) continue;
        const float swl = __fmul_rn(__fmul_rn(sw1, __int_as_float((126 + L) << 23)), A);
        if (!(__fmul_rn(nd2, 1.0634765625f) <= __fmul_rn(swl, swl))) continue;  // (1 + 1/32)^2
        if (L > 1) {
            const float swm = __fmul_rn(__fmul_rn(sw1, __int_as_float((125 + L) << 23)), A);
            if (!(__fmul_rn(nd2, 0.9384765625f) > __fmul_rn(swm, swm))) continue;  // (1 - 1/32)^2
        }
        // the meeting point inside the face, s/64 from its edges: with
        // u = (camera - cell corner) * A + n * d, A * s/64 < u < A * s * 63/64
        const int b1 = axis == 0 ? 1 : 0, b2 = axis == 2 ? 1 : 2;
        const float sa = __fmul_rn(cs, A);
        const float smin = __fmul_rn(sa, 0.015625f), smax = __fmul_rn(sa, 0.984375f);
        const float u1 = __fadd_rn(__fmul_rn(__fsub_rn(b1 == 0 ? c16[0] : c16[1], h.lo1[cy][cx]), A),
                                   __fmul_rn(n, b1 == 0 ? d[0] : d[1]));
        if (!(u1 > smin && u1 < smax)) continue;
        const float u2 = __fadd_rn(__fmul_rn(__fsub_rn(b2 == 1 ? c16[1] : c16[2], h.lo2[cy][cx]), A),
                                   __fmul_rn(n, b2 == 1 ? d[1] : d[2]));
        if (!(u2 > smin && u2 < smax)) continue;
        bn = n;
        ba = A;
        bk = k;
    }
    if (bk < 0) return false;
    const int cy = hy + (bk == 0 ? -1 : (bk == 4 ? 1 : 0)), cx = hx + (bk == 1 ? -1 : (bk == 3 ? 1 : 0));
    const int L = h.level[cy][cx];
    const int baxis = (int)(h.face[cy][cx] & 3u);
    const float t = __fdiv_rn(bn, ba);
    float q[3];
#pragma unroll
    for (int b = 0; b < 3; ++b) q[b] = b == baxis ? h.plane[cy][cx] : __fadd_rn(c16[b], __fmul_rn(t, d[b]));
    const uint32_t signs = (d[0] < 0.0f ? 1u : 0u) | (d[1] < 0.0f ? 2u : 0u) | (d[2] < 0.0f ? 4u : 0u);
    out_col = 0xff000000u | (h.col[cy][cx] & 255u);
    out_q = make_float4(__fmul_rn(q[0], 0.0625f), __fmul_rn(q[1], 0.0625f), __fmul_rn(q[2], 0.0625f),
                        (float)(L | (int)(signs << 5)));
    return true;
}

// Also lists the net tiles (kNetOutW x kNetOutH) holding an unguided pixel:
// the first block to find one in a tile stamps the tile with this frame's
// serial and appends it (a block of 32 x 8 pixels touches at most 2 x 2
// tiles). And it lists, per pixel, what the tracer does with it: a walk (a
// guided pixel outside the refresh tile that is not certified), in the walk
// list of its length bucket -- or a commit of a certified pixel (its colour word and
// point wait in cert_col / cert_xyz: the block cannot write them into the
// plane, which other blocks read as their halo). Each warp appends the
// pixels of one ray packet (pw x ph) of the block, so consecutive list
// entries stay spatial neighbours.
//
// kResolve: the block also resolves the projection keys (k_resolve_gather's
// gather, one launch less): every pixel of its halo takes its winning source
// from the key buffer, and the block writes its own pixels' colour words and
// points into the current plane. The keys stay set (neighbouring blocks read
// them as their halo); the tracer clears them (FrameParams::clear_keys). No
// hole tile masks: learned frames do not use them.
template <bool kResolve>
__global__ void __launch_bounds__(kGuideBW * kGuideBH) k_guide(const FrameParams* __restrict__ P, TargetBuffers B) {
    grid_dep_wait();
    grid_dep_launch();
    constexpr int kHW = kGuideBW + 2, kHH = kGuideBH + 2;
    __shared__ float dist[kHH][kHW];
    __shared__ uint8_t hole[kHH][kHW];  // a pixel of the frame without a point
    __shared__ CertHalo cand;
    __shared__ float d1col[kGuideBW], d1row[kGuideBH];  // the ray kernels' direction terms
    // 0 none, 1..kWalkBuckets a walk (bucket 1: the longest expected), kWalkBuckets+1 certified
    __shared__ uint8_t kind[kGuideBH][kGuideBW];
    __shared__ uint32_t list_cnt[kWalkBuckets + 1][kGuideBH];  // per list and warp: count, then position
    __shared__ uint32_t touched;
    const int res_x = B.res_x, res_y = B.res_y;
    const int x0 = blockIdx.x * kGuideBW, y0 = blockIdx.y * kGuideBH;
    const float cx = P->ray.px, cy = P->ray.py, cz = P->ray.pz;
    const uint32_t* __restrict__ col = plane_col(B, P->cur);
    const float4* __restrict__ xyz = plane_xyz(B, P->cur);
    const bool certify = P->certify != 0;
    if (threadIdx.x == 0) touched = 0;
    if (threadIdx.x < kGuideBW + kGuideBH) {  // as trace_ray computes them
        const bool c = threadIdx.x < kGuideBW;
        const int v = c ? x0 + (int)threadIdx.x : y0 + (int)threadIdx.x - kGuideBW;
        const int half = c ? (res_x >> 1) : (res_y >> 1);
        const float t = __fdiv_rn(__fmul_rn(__fadd_rn((float)(v - half), 0.5f), c ? P->ray.fovx : P->ray.fovy),
                                  (float)res_y);
        if (c) d1col[threadIdx.x] = t;
        else d1row[threadIdx.x - kGuideBW] = t;
    }
    // The halo: with kResolve each thread's (at most two) pixels first load
    // their keys, then both winning sources, so the two dependent loads of
    // each chain overlap the other pixel's instead of following them.
    constexpr int kHalo = kHW * kHH, kPer = (kHalo + kGuideBW * kGuideBH - 1) / (kGuideBW * kGuideBH);
    uint32_t hc[kPer];
    float4 hq[kPer];
    bool hin[kPer];
#pragma unroll
    for (int k = 0; k < kPer; ++k) {
        const int i = threadIdx.x + k * kGuideBW * kGuideBH;
        const int wx = i % kHW, wy = i / kHW;
        const int gx = x0 + wx - 1, gy = y0 + wy - 1;
        hin[k] = i < kHalo && gx >= 0 && gx < res_x && gy >= 0 && gy < res_y;
        hc[k] = kEmptyPixel;
        hq[k] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        if (!kResolve && hin[k]) {
            const size_t o = (size_t)gy * res_x + gx;
            hc[k] = __ldg(col + o);  // both loads in flight together
            hq[k] = __ldg(xyz + o);
        }
    }
    if (kResolve) {
        uint64_t key[kPer];
#pragma unroll
        for (int k = 0; k < kPer; ++k) {
            const int i = threadIdx.x + k * kGuideBW * kGuideBH;
            const int wx = i % kHW, wy = i / kHW;
            key[k] = (hin[k] && P->have_cache) ? B.keys[(size_t)(y0 + wy - 1) * res_x + (x0 + wx - 1)] : kKeyEmpty;
        }
#pragma unroll
        for (int k = 0; k < kPer; ++k)
            if (key[k] != kKeyEmpty) hc[k] = resolve_source(P, B, key[k], hq[k]);
    }
#pragma unroll
    for (int k = 0; k < kPer; ++k) {
        const int i = threadIdx.x + k * kGuideBW * kGuideBH;
        if (i >= kHalo) break;
        const int wx = i % kHW, wy = i / kHW;
        float d = INFINITY;
        uint8_t h = 0;
        uint32_t cc = kEmptyPixel;
        float4 cq = make_float4(0.0f, 0.0f, 0.0f, -1.0f);
        if (hin[k]) {
            const uint32_t c = hc[k];
            const float4 q = hq[k];
            if (kResolve && wx >= 1 && wx <= kGuideBW && wy >= 1 && wy <= kGuideBH) {  // the block's own pixel
                const size_t o = (size_t)(y0 + wy - 1) * res_x + (x0 + wx - 1);
                plane_col(B, P->cur)[o] = c;
                if (c != kEmptyPixel) plane_xyz(B, P->cur)[o] = q;
            }
            // exact IEEE operations, so the CPU oracle finds the same start distances
            const float ax = __fsub_rn(q.x, cx), ay = __fsub_rn(q.y, cy), az = __fsub_rn(q.z, cz);
            if (c != kEmptyPixel) {
                d = __fsqrt_rn(__fadd_rn(__fadd_rn(__fmul_rn(ax, ax), __fmul_rn(ay, ay)), __fmul_rn(az, az)));
                cc = c;
                cq = q;
            } else {
                h = 1;
            }
        }
        dist[wy][wx] = d;
        hole[wy][wx] = h;
        if (certify) cert_face(cand, wy, wx, cc, cq);
    }
    __syncthreads();
    const int tx = threadIdx.x % kGuideBW, ty = threadIdx.x / kGuideBW;
    const int x = x0 + tx, y = y0 + ty;
    uint8_t k_of = 0;
    if (x < res_x && y < res_y) {
        float m = INFINITY;
        int holes = 0;
#pragma unroll
        for (int j = 0; j < 3; ++j)
#pragma unroll
            for (int i = 0; i < 3; ++i) {
                const float d = dist[ty + j][tx + i];
                m = fminf(m, d);
                holes += hole[ty + j][tx + i];
            }
        const float own = dist[ty + 1][tx + 1];
        const size_t ofs = (size_t)y * res_x + x;
        float g = -1.0f;
        if (m < INFINITY) {
            const float s = __fmul_rn(m, 16.0f);  // raypos units
            const int lod = lod_at(s, res_x);
            const float cell = __int_as_float((127 + lod) << 23);  // 2^lod
            g = holes >= kGuideHoleCount ? __fmul_rn(s, kGuideNearHole)
                                         : fmaxf(__fsub_rn(s, __fmul_rn(kGuideMargin, cell)), 0.0f);
            const bool in_tile = x >= P->add_x && x < P->x_end && y >= P->add_y && y < P->y_end;
            uint32_t cc = 0;
            float4 cq;
            if (certify && holes == 0 && !in_tile &&
                certify_pixel(P->ray, res_x, d1col[tx], d1row[ty], cand, tx + 1, ty + 1, s, cc, cq)) {
                g = kGuideCertified;
                B.cert_col[ofs] = cc;
                B.cert_xyz[ofs] = cq;
                B.bgrx[ofs] = colorize(cc);
                k_of = kWalkBuckets + 1;
            } else if (!in_tile) {  // the refresh tile traces its pixels from the camera
                // cells between the start and the pixel's own point; a pixel
                // without one goes with the longest walks
                const float ahead = own < INFINITY ? __fdividef(own * 16.0f - g, cell) : INFINITY;
                k_of = ahead > kGuideLong ? 1 : (ahead > kGuideMid ? 2 : (ahead > kGuideShort ? 3 : 4));
            }
        } else {
            const int ntx = x / kNetOutW - x0 / kNetOutW, nty = y / kNetOutH - y0 / kNetOutH;
            atomicOr(&touched, 1u << (ntx + 2 * nty));
        }
        B.guide[ofs] = g;
    }
    kind[ty][tx] = k_of;
    __syncthreads();
    {  // warp w appends the pixels of packet w of the block, in packet order;
       // one atomic per list and block (not per warp: 8x fewer on three counters)
        const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
        // packets per block row: kGuideBW / pw = 2^rs, packet height ph = 2^rs
        static_assert(kGuideBW == 32, "packet shapes 2^ps x 2^(5-ps) tile a 32-pixel row");
        const int ps = P->pw_shift, pw = 1 << ps, rs = 5 - ps;
        const int bx = ((w & ((1 << rs) - 1)) << ps) + (lane & (pw - 1)), by = ((w >> rs) << rs) + (lane >> ps);
        const int k = kind[by][bx];
        const uint32_t xy = (uint32_t)(x0 + bx) | ((uint32_t)(y0 + by) << 16);
        const uint32_t below = (1u << lane) - 1u;
        uint32_t mine = 0;  // the ballot of this lane's list
#pragma unroll
        for (int kk = 0; kk <= kWalkBuckets; ++kk) {
            const uint32_t bal = __ballot_sync(0xffffffffu, k == kk + 1);
            if (k == kk + 1) mine = bal;
            if (lane == 0) list_cnt[kk][w] = (uint32_t)__popc(bal);
        }
        __syncthreads();
        if (threadIdx.x <= kWalkBuckets) {
            const int kk = (int)threadIdx.x;
            uint32_t total = 0;
            for (int i = 0; i < kGuideBH; ++i) total += list_cnt[kk][i];
            uint32_t at = total ? atomicAdd(B.counters + 4 + kk, total) : 0u;
            for (int i = 0; i < kGuideBH; ++i) {
                const uint32_t c = list_cnt[kk][i];
                list_cnt[kk][i] = at;
                at += c;
            }
        }
        __syncthreads();
        if (k > 0) {
            const uint32_t at = list_cnt[k - 1][w] + (uint32_t)__popc(mine & below);
            if (at < B.walk_cap) {
                if (k <= kWalkBuckets) B.walk_list[(size_t)(k - 1) * B.walk_cap + at] = xy;
                else B.cert_list[at] = xy;
            }
        }
    }
    if (threadIdx.x < 4 && ((touched >> threadIdx.x) & 1u)) {
        const int tiles_x = (res_x + kNetOutW - 1) / kNetOutW;
        const uint32_t tile = (uint32_t)((y0 / kNetOutH + (int)(threadIdx.x >> 1)) * tiles_x + x0 / kNetOutW +
                                         (int)(threadIdx.x & 1));
        if (atomicExch(B.net_flags + tile, P->serial) != P->serial) B.net_list[atomicAdd(B.counters + 3, 1u)] = tile;
    }
}

struct NetInferArgs {
    const uint16_t* packed;  // tensor-core weight image
    const float* bias;       // 52 biases
    // input: either the planes of a target (pipeline) or planar features
    const FrameParams* P;
    TargetBuffers B;
    const float* feat;  // [8][h][w] when not from planes
    float* out;         // [4][h][w] when not from planes
    float* act;         // training: [3][16][h][w] hidden activations (bf16 values), or null
    int w, h;
    int tiles_x, tiles;
    float logit_threshold;  // pipeline: traced when logit < threshold
    uint32_t* fault;
};

// Two floats to a packed bf16 pair, round to nearest even (lo in the low half).
__device__ __forceinline__ uint32_t pack_bf16x2(float lo, float hi) {
    uint32_t r;
    asm("cvt.rn.bf16x2.f32 %0, %1, %2;" : "=r"(r) : "f"(hi), "f"(lo));
    return r;
}

// All MMAs of layer L for the blocks of one tile (issued by one thread).
// MMAs of blocks j0, j0 + jstep, ... (several threads issue a layer's blocks:
// one issuing thread cannot feed the tensor core fast enough with N = 16).
template <int L>
__device__ __forceinline__ void net_issue_layer(uint32_t sbase, uint32_t tmem, uint32_t x_off, int j0, int jstep) {
    constexpr int kMmas = net_mmas(L);
    constexpr int kBlocks = 15 - L;
    constexpr int kFirst = (L + 1) * kNetTW;
    const uint32_t kIn = L == 0 ? x_off : ((L & 1) ? kNetSmemA : kNetSmemB);
    uint64_t ad[kMmas], bd[kMmas];
#pragma unroll
    for (int m = 0; m < kMmas; ++m) {
        int shift, lbo;
        if (L == 0) {
            const int t0 = 2 * m, t1 = 2 * m + 1;
            shift = (t0 / 3 - 1) * kNetTW + (t0 % 3 - 1);
            lbo = t1 < 9 ? ((t1 / 3 - 1) * kNetTW + (t1 % 3 - 1) - shift) * 16 : 16;
        } else {
            shift = (m / 3 - 1) * kNetTW + (m % 3 - 1);
            lbo = kNetPlaneBytes;
        }
        ad[m] = tc_desc(sbase + kIn + (uint32_t)((kNetGuard + kFirst + shift) * 16), (uint32_t)lbo, 128u);
        bd[m] = tc_desc(sbase + kNetSmemW + (uint32_t)((net_mma_base(L) + m) * 512), 128u, 256u);
    }
    for (int j = j0; j < kBlocks; j += jstep) {
        // block j starts 128 positions (2048 bytes, 128 in the address field) later
#pragma unroll
        for (int m = 0; m < kMmas; ++m) tc_mma(tmem + 16u * j, ad[m] + 128ull * j, bd[m], m > 0 ? 1u : 0u);
    }
}

// Input features of one slice of a tile: position p = tid + k * kNetThreads
// of the window at image origin (wx, wy), written bf16 into input plane xoff.
template <bool kPipeline>
__device__ __forceinline__ void net_stage_input(const NetInferArgs& A, const FrameParams& P, uint8_t* smem,
                                                uint32_t xoff, int wx, int wy, int k) {
    const int p = threadIdx.x + k * kNetThreads;
    const int gx = wx + (p & (kNetTW - 1)), gy = wy + (p >> 6);
    float f[8];
#pragma unroll
    for (int i = 0; i < 8; ++i) f[i] = 0.0f;
    if (gx >= 0 && gx < A.w && gy >= 0 && gy < A.h) {
        if (kPipeline) {
            net_compute(P, A.w, A.h, gx, gy, net_load(P, A.B, gx, gy), f);
        } else {
            const size_t n = (size_t)A.w * A.h, ofs = (size_t)gy * A.w + gx;
#pragma unroll
            for (int i = 0; i < 8; ++i) f[i] = __ldg(A.feat + i * n + ofs);
        }
    }
    uint4 v;
    v.x = pack_bf16x2(f[0], f[1]);
    v.y = pack_bf16x2(f[2], f[3]);
    v.z = pack_bf16x2(f[4], f[5]);
    v.w = pack_bf16x2(f[6], f[7]);
    *reinterpret_cast<uint4*>(smem + xoff + (kNetGuard + p) * 16) = v;
}

template <bool kPipeline>
__global__ void __launch_bounds__(kNetThreads, 1) k_net_infer(NetInferArgs A) {
    __shared__ uint64_t mbar[kNetIssuers];  // issuer i's MMAs of a layer: blocks j = i (mod kNetIssuers)
    __shared__ uint32_t tmem_base_s;
    __shared__ FrameParams sP;
    uint8_t* smem = reinterpret_cast<uint8_t*>(svo_dsmem);
    const uint32_t sbase = smem_addr(smem);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int W = A.w, H = A.h;

    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_addr(&tmem_base_s)),
                     "r"(kNetTmemCols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    if (tid < kNetIssuers) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_addr(&mbar[tid])) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    // weights, biases; zero every activation and input plane (guards included)
    {
        const uint4* src = reinterpret_cast<const uint4*>(A.packed);
        uint4* dst = reinterpret_cast<uint4*>(smem + kNetSmemW);
        for (int i = tid; i < kNetMmaTotal * 32; i += kNetThreads) dst[i] = src[i];
        float* b = reinterpret_cast<float*>(smem + kNetSmemBias);
        for (int i = tid; i < kNetBias; i += kNetThreads) b[i] = A.bias[i];
        uint4* z = reinterpret_cast<uint4*>(smem);
        for (int i = tid; i < 6 * kNetPlaneBytes / 16; i += kNetThreads) z[i] = make_uint4(0, 0, 0, 0);
    }
    // everything above is this launch's own set-up; what follows reads the
    // frame's parameters and the kernels before this one
    grid_dep_wait();
    grid_dep_launch();
    if (kPipeline) {
        const uint32_t* src = reinterpret_cast<const uint32_t*>(A.P);
        uint32_t* dst = reinterpret_cast<uint32_t*>(&sP);
        for (int i = tid; i < (int)(sizeof(FrameParams) / 4); i += kNetThreads) dst[i] = src[i];
    }
    __syncthreads();
    // Work: every tile, or (guided frames) the listed tiles.
    const uint32_t* __restrict__ list = kPipeline && A.B.guide ? A.B.net_list : nullptr;
    const int n_work = list ? (int)A.B.counters[3] : A.tiles;
    // the first tile's input
    int item = blockIdx.x;
    if (item < n_work) {
        const int tile = list ? (int)list[item] : item;
        const int wx = (tile % A.tiles_x) * kNetOutW - 4, wy = (tile / A.tiles_x) * kNetOutH - 4;
#pragma unroll
        for (int k = 0; k < kNetPer; ++k) net_stage_input<kPipeline>(A, sP, smem, kNetSmemX, wx, wy, k);
    }
    fence_async_smem();
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = tmem_base_s;
    // the warps of slice s (warp >> 2) read back blocks j = s (mod 4), which
    // issuer s issued and committed to its own barrier
    const uint32_t bar = smem_addr(&mbar[(warp >> 2) % kNetIssuers]);
    const float* bias = reinterpret_cast<const float*>(smem + kNetSmemBias);
    uint32_t phase = 0;
    uint32_t fault = 0;
    bool aborted = false;  // block-uniform: an MMA wait timed out
    int xb = 0;            // which input plane holds this tile's input

    for (; item < n_work; item += gridDim.x, xb ^= 1) {
        const int tile = list ? (int)list[item] : item;
        const int ox = (tile % A.tiles_x) * kNetOutW, oy = (tile / A.tiles_x) * kNetOutH;
        const int wx = ox - 4, wy = oy - 4;  // image position of window position 0
        const uint32_t x_cur = kNetSmemX + (uint32_t)xb * kNetPlaneBytes;
        const uint32_t x_next = kNetSmemX + (uint32_t)(xb ^ 1) * kNetPlaneBytes;
        const int next_item = item + (int)gridDim.x;
        const bool has_next = next_item < n_work;
        const int next = has_next ? (list ? (int)list[next_item] : next_item) : 0;
        const int nwx = (next % A.tiles_x) * kNetOutW - 4, nwy = (next / A.tiles_x) * kNetOutH - 4;

        for (int l = 0; l < kNetLayers; ++l) {
            const int nb = 15 - l;
            const int first = (l + 1) * kNetTW;
            const uint32_t out_off = (l & 1) ? kNetSmemB : kNetSmemA;
            if (lane == 0 && warp < kNetIssuers) {
                tc_fence_after();
                switch (l) {
                    case 0: net_issue_layer<0>(sbase, tmem, x_cur, warp, kNetIssuers); break;
                    case 1: net_issue_layer<1>(sbase, tmem, x_cur, warp, kNetIssuers); break;
                    case 2: net_issue_layer<2>(sbase, tmem, x_cur, warp, kNetIssuers); break;
                    default: net_issue_layer<3>(sbase, tmem, x_cur, warp, kNetIssuers); break;
                }
                tc_commit(smem_addr(&mbar[warp]));
            }
            // while the MMAs run: one slice of the next tile's input
            if (has_next) net_stage_input<kPipeline>(A, sP, smem, x_next, nwx, nwy, l);
            // each warp waits (bounded) for the MMAs of its own blocks only, so the
            // read-back of early blocks overlaps the MMAs of later ones
            const bool ready = mbar_wait_phase(bar, phase);
            phase ^= 1u;
            tc_fence_after();
            const int g = warp & 3;
            if (!ready) {
                // skip this warp's read-back; the block leaves after the barrier below
            } else if (l < kNetLayers - 1) {
                // the (at most 4) blocks of this warp: all loads in flight, one wait
                constexpr int kSlices = kNetWarps / 4;
                uint32_t r[4][16];
#pragma unroll
                for (int k = 0; k < 4; ++k) {
                    const int j = (warp >> 2) + k * kSlices;
                    if (j < nb) tc_ld16_nowait(tmem + ((uint32_t)(32 * g) << 16) + 16u * j, r[k]);
                }
                tc_wait_ld();
                const float* bl = bias + 16 * l;
#pragma unroll
                for (int k = 0; k < 4; ++k) {
                    const int j = (warp >> 2) + k * kSlices;
                    if (j >= nb) continue;
                    const int p = first + 128 * j + 32 * g + lane;  // this thread's position
                    const int gx = wx + (p & (kNetTW - 1)), gy = wy + (p >> 6);
                    const bool inside = gx >= 0 && gx < W && gy >= 0 && gy < H;
                    uint32_t h[8];
#pragma unroll
                    for (int c = 0; c < 16; c += 2) {
                        const float a0 = inside ? fmaxf(__uint_as_float(r[k][c]) + bl[c], 0.0f) : 0.0f;
                        const float a1 = inside ? fmaxf(__uint_as_float(r[k][c + 1]) + bl[c + 1], 0.0f) : 0.0f;
                        h[c >> 1] = pack_bf16x2(a0, a1);
                    }
                    *reinterpret_cast<uint4*>(smem + out_off + (kNetGuard + p) * 16) =
                        make_uint4(h[0], h[1], h[2], h[3]);
                    *reinterpret_cast<uint4*>(smem + out_off + kNetPlaneBytes + (kNetGuard + p) * 16) =
                        make_uint4(h[4], h[5], h[6], h[7]);
                    if (!kPipeline && A.act) {
                        // training: the tile's own positions keep this layer's activations
                        // (the bf16 values the next layer reads) for the backward pass
                        const int col = p & (kNetTW - 1), row = p >> 6;
                        if (inside && col >= 4 && col < 4 + kNetOutW && row >= 4 && row < 4 + kNetOutH) {
                            const size_t n = (size_t)W * H;
                            float* dst = A.act + (size_t)l * 16 * n + (size_t)gy * W + gx;
#pragma unroll
                            for (int c = 0; c < 8; ++c) {
                                dst[(2 * c) * n] = __uint_as_float(h[c] << 16);
                                dst[(2 * c + 1) * n] = __uint_as_float(h[c] & 0xFFFF0000u);
                            }
                        }
                    }
                }
            } else {
                for (int j = warp >> 2; j < nb; j += kNetWarps / 4) {
                    const int p = first + 128 * j + 32 * g + lane;  // this thread's position
                    const int gx = wx + (p & (kNetTW - 1)), gy = wy + (p >> 6);
                    const bool inside = gx >= 0 && gx < W && gy >= 0 && gy < H;
                    float v[4];
                    tc_ld4(tmem + ((uint32_t)(32 * g) << 16) + 16u * j, v);
                    const int col = p & (kNetTW - 1);
                    const bool out = inside && col >= 4 && col < 4 + kNetOutW;  // rows are 4..27 here
                    // the residual colour: the bf16 input channels 0-2 of this position
                    const uint2 in = *reinterpret_cast<const uint2*>(smem + x_cur + (kNetGuard + p) * 16);
                    const float r = v[0] + bias[48] + __uint_as_float(in.x << 16);
                    const float gg = v[1] + bias[49] + __uint_as_float(in.x & 0xFFFF0000u);
                    const float b = v[2] + bias[50] + __uint_as_float(in.y << 16);
                    const float z = v[3] + bias[51];
                    if (kPipeline) {
                        bool req = false;
                        if (out) {
                            const size_t ofs = (size_t)gy * W + gx;
                            const uint32_t ri = (uint32_t)__float2int_rn(fminf(fmaxf(r, 0.0f), 1.0f) * 255.0f);
                            const uint32_t gi = (uint32_t)__float2int_rn(fminf(fmaxf(gg, 0.0f), 1.0f) * 255.0f);
                            const uint32_t bi = (uint32_t)__float2int_rn(fminf(fmaxf(b, 0.0f), 1.0f) * 255.0f);
                            // In guided frames the net decides the unguided pixels only
                            // (guide -1): the others are walked or certified and k_guide
                            // has written the certified pixels' colour already. With no
                            // cache (the first frames) every pixel is traced: pixels the
                            // net fills are not cached, so they would stay unguided.
                            const bool mine = !list || __ldg(A.B.guide + ofs) == -1.0f;
                            if (mine) A.B.bgrx[ofs] = bi + (gi << 8) + (ri << 16);
                            req = !sP.have_cache || (!(z >= A.logit_threshold) && mine);
                        }
                        const uint32_t bal = __ballot_sync(0xffffffffu, req);
                        if (list) {
                            // Guided frames request few rays (the unguided pixels the net is
                            // not confident about): the warp appends them to the hole list
                            // itself, one atomic per warp, instead of the packet masks and
                            // their two compaction kernels. The list's order varies; every
                            // pixel's ray does not depend on it.
                            if (bal) {
                                uint32_t base = 0;
                                if (lane == 0) base = atomicAdd(A.B.counters + 1, (uint32_t)__popc(bal));
                                base = __shfl_sync(0xffffffffu, base, 0);
                                const uint32_t at = base + (uint32_t)__popc(bal & ((1u << lane) - 1u));
                                if (req && at < (uint32_t)W * (uint32_t)H)
                                    A.B.ids[2u * (uint32_t)A.B.tiles_x * (uint32_t)A.B.tiles_y + at] =
                                        (uint32_t)gx | ((uint32_t)gy << 16);
                            }
                        } else if (bal && (lane == 0 || (gx & 7) == 0)) {
                            // Ray requests: bit (x&7) + 8*(y&3) of the pixel's 8x4 packet. The
                            // warp's lanes are consecutive pixels of one row, so the first lane
                            // of each run of one packet ORs the run's bits in one atomic.
                            const int len = min(8 - (gx & 7), 32 - lane);
                            const uint32_t run = (bal >> lane) & ((1u << len) - 1u);
                            if (run)
                                atomicOr(A.B.req_mask + (size_t)(gy >> 2) * A.B.packets_x + (gx >> 3),
                                         run << ((gx & 7) + 8 * (gy & 3)));
                        }
                    } else if (out) {
                        const size_t n = (size_t)W * H, ofs = (size_t)gy * W + gx;
                        A.out[ofs] = r;
                        A.out[n + ofs] = gg;
                        A.out[2 * n + ofs] = b;
                        A.out[3 * n + ofs] = z;
                    }
                }
            }
            fence_async_smem();
            tc_fence_before();
            aborted = __syncthreads_or(ready ? 0 : 1) != 0;  // block-uniform verdict
            tc_fence_after();
            if (aborted) {
                fault |= kFaultNet;
                break;
            }
        }
        if (aborted) break;
    }
    __syncthreads();
    if (warp == 0) {
        tc_fence_after();
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kNetTmemCols) : "memory");
    }
    if (fault) atomicOr(A.fault, fault);
}

// ------------------------------------------------ ray-request list --
// The requests of a learned frame, compacted in 8x4-packet order (packets in
// row-major order, pixels in lane order) into the hole list the tracer reads:
// consecutive entries are spatial neighbours, so the tracer's 32-ray packets
// stay coherent. k_request_scan: per block of 1024 packets, the exclusive
// scan of their request counts and the block's total; k_request_write adds
// the totals of the blocks before it, writes the entries and clears the
// mask words.
constexpr int kReqBlock = 1024;

__device__ __forceinline__ uint32_t block_exclusive_scan(uint32_t v, uint32_t* warp_sums, uint32_t& total) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint32_t incl = v;
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t t = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += t;
    }
    if (lane == 31) warp_sums[warp] = incl;
    __syncthreads();
    if (warp == 0) {
        uint32_t w = lane < (int)(blockDim.x >> 5) ? warp_sums[lane] : 0u;
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t t = __shfl_up_sync(0xffffffffu, w, o);
            if (lane >= o) w += t;
        }
        warp_sums[lane] = w;
    }
    __syncthreads();
    total = warp_sums[(blockDim.x >> 5) - 1];
    return incl - v + (warp > 0 ? warp_sums[warp - 1] : 0u);
}

__global__ void __launch_bounds__(kReqBlock) k_request_scan(TargetBuffers B, uint32_t* __restrict__ offs,
                                                            uint32_t* __restrict__ block_totals) {
    __shared__ uint32_t warp_sums[32];
    const uint32_t n = (uint32_t)B.packets_x * (uint32_t)B.packets_y;
    const uint32_t t = blockIdx.x * kReqBlock + threadIdx.x;
    const uint32_t c = t < n ? (uint32_t)__popc(B.req_mask[t]) : 0u;
    uint32_t total;
    const uint32_t ex = block_exclusive_scan(c, warp_sums, total);
    if (t < n) offs[t] = ex;
    if (threadIdx.x == 0) block_totals[blockIdx.x] = total;
}

__global__ void __launch_bounds__(kReqBlock) k_request_write(TargetBuffers B, const uint32_t* __restrict__ offs,
                                                             const uint32_t* __restrict__ block_totals) {
    __shared__ uint32_t warp_sums[32];
    __shared__ uint32_t prefix_s;
    const uint32_t n = (uint32_t)B.packets_x * (uint32_t)B.packets_y;
    // totals of the blocks before this one
    uint32_t part = 0;
    for (uint32_t k = threadIdx.x; k < blockIdx.x; k += kReqBlock) part += block_totals[k];
    uint32_t sum;
    (void)block_exclusive_scan(part, warp_sums, sum);
    if (threadIdx.x == 0) prefix_s = sum;
    __syncthreads();
    const uint32_t prefix = prefix_s;
    if (blockIdx.x == gridDim.x - 1 && threadIdx.x == 0) {
        B.counters[1] = prefix + block_totals[blockIdx.x];
        B.counters[0] = 0;
    }
    const uint32_t t = blockIdx.x * kReqBlock + threadIdx.x;
    if (t >= n) return;
    uint32_t m = B.req_mask[t];
    if (!m) return;
    B.req_mask[t] = 0;
    const uint32_t x0 = (t % (uint32_t)B.packets_x) * 8u, y0 = (t / (uint32_t)B.packets_x) * 4u;
    uint32_t at = 2u * (uint32_t)B.tiles_x * (uint32_t)B.tiles_y + prefix + offs[t];
    while (m) {
        const uint32_t bit = (uint32_t)__ffs(m) - 1u;
        m &= m - 1u;
        B.ids[at++] = (x0 + (bit & 7u)) | ((y0 + (bit >> 3)) << 16);
    }
}

// ------------------------------------------------ FP32 reference path --
// One layer forward: one thread per pixel, weights (already bf16-rounded) in
// shared memory. kFirst rounds the input features to bf16 on load; hidden
// layers store bf16(ReLU(.)); the last layer stores FP32 plus the residual
// colour.
template <int CIN, int COUT, bool kFirst, bool kLast>
__global__ void __launch_bounds__(256) k_net_conv_fwd(const float* __restrict__ in, const float* __restrict__ wr,
                                                      const float* __restrict__ b, const float* __restrict__ feat,
                                                      float* __restrict__ out, int W, int H) {
    __shared__ float ws[9 * CIN * COUT];
    __shared__ float bs[COUT];
    for (int i = threadIdx.x; i < 9 * CIN * COUT; i += blockDim.x) ws[i] = wr[i];
    if (threadIdx.x < COUT) bs[threadIdx.x] = b[threadIdx.x];
    __syncthreads();
    const int x = blockIdx.x * 32 + (threadIdx.x & 31), y = blockIdx.y * 8 + (threadIdx.x >> 5);
    if (x >= W || y >= H) return;
    const size_t n = (size_t)W * H;
    float acc[COUT];
#pragma unroll
    for (int c = 0; c < COUT; ++c) acc[c] = 0.0f;
    for (int t = 0; t < 9; ++t) {
        const int sx = x + t % 3 - 1, sy = y + t / 3 - 1;
        if (sx < 0 || sx >= W || sy < 0 || sy >= H) continue;
        const size_t o = (size_t)sy * W + sx;
        for (int ci = 0; ci < CIN; ++ci) {
            float a = __ldg(in + ci * n + o);
            if (kFirst) a = bf16_round(a);
            const float* wt = ws + (t * CIN + ci) * COUT;
#pragma unroll
            for (int c = 0; c < COUT; ++c) acc[c] = __fmaf_rn(a, wt[c], acc[c]);
        }
    }
    const size_t o = (size_t)y * W + x;
#pragma unroll
    for (int c = 0; c < COUT; ++c) {
        float v = acc[c] + bs[c];
        if (!kLast) v = bf16_round(fmaxf(v, 0.0f));
        else if (c < 3) v += bf16_round(__ldg(feat + c * n + o));
        out[c * n + o] = v;
    }
}

// Loss and its gradient w.r.t. the four outputs (see net_oracle.loss_grad):
// sum_c (rgb_c - t_c)^2 / 3 + lam * BCE(logit, max_c |rgb_c - t_c| < tau),
// averaged over pixels. Per-block partial sums of the two terms.
__global__ void __launch_bounds__(256) k_net_loss(const float* __restrict__ out, const uint32_t* __restrict__ target,
                                                  float* __restrict__ d_out, float* __restrict__ partial, int n,
                                                  float tau, float lam) {
    __shared__ float red[2][8];
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    float lr = 0.0f, lc = 0.0f;
    if (i < n) {
        const uint32_t w = __ldg(target + i);
        const float t0 = (float)((w >> 16) & 255u) / 255.0f, t1 = (float)((w >> 8) & 255u) / 255.0f,
                    t2 = (float)(w & 255u) / 255.0f;
        const float d0 = out[i] - t0, d1 = out[n + i] - t1, d2 = out[2 * n + i] - t2;
        const float z = out[3 * n + i];
        const float y = fmaxf(fmaxf(fabsf(d0), fabsf(d1)), fabsf(d2)) < tau ? 1.0f : 0.0f;
        const float inv = 1.0f / (float)n;
        lr = (d0 * d0 + d1 * d1 + d2 * d2) / 3.0f;
        lc = fmaxf(z, 0.0f) + log1pf(expf(-fabsf(z))) - y * z;
        const float s = 1.0f / (1.0f + expf(-z));
        d_out[i] = 2.0f / 3.0f * d0 * inv;
        d_out[n + i] = 2.0f / 3.0f * d1 * inv;
        d_out[2 * n + i] = 2.0f / 3.0f * d2 * inv;
        d_out[3 * n + i] = lam * (s - y) * inv;
    }
    for (int o = 16; o > 0; o >>= 1) {
        lr += __shfl_down_sync(0xffffffffu, lr, o);
        lc += __shfl_down_sync(0xffffffffu, lc, o);
    }
    if ((threadIdx.x & 31) == 0) {
        red[0][threadIdx.x >> 5] = lr;
        red[1][threadIdx.x >> 5] = lc;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        float a = 0.0f, c = 0.0f;
        for (int k = 0; k < 8; ++k) {
            a += red[0][k];
            c += red[1][k];
        }
        partial[2 * blockIdx.x] = a;
        partial[2 * blockIdx.x + 1] = c;
    }
}

// grads[i] = sum over blocks of partial[block][i], in block order.
__global__ void k_net_reduce(const float* __restrict__ partial, int blocks, int vals, float* __restrict__ grads) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= vals) return;
    float s = 0.0f;
    for (int k = 0; k < blocks; ++k) s += partial[(size_t)k * vals + i];
    grads[i] = s;
}

__global__ void k_net_adam(float* __restrict__ p, float* __restrict__ m, float* __restrict__ v,
                           const float* __restrict__ g, int n, float lr, float b1, float b2, float eps, float c1,
                           float c2) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float gi = g[i];
    const float mi = b1 * m[i] + (1.0f - b1) * gi;
    const float vi = b2 * v[i] + (1.0f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    p[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
}

}  // namespace svo
