// svo_net_train.cuh -- the reconstruction net's backward pass on the tensor
// cores (training; no reference counterpart).
//
// The forward pass of a training step is k_net_infer (tcgen05, bf16 x bf16 ->
// fp32) writing its hidden activations out; the two kernels here do the
// backward convolutions as implicit GEMMs on the same operand layouts (the
// no-swizzle K-major canonical layout k_net_probe checks):
//
//   k_net_bwd_data_tc    dL/dinput of a layer, times the ReLU mask of the
//                        layer below: D[position, ci] = sum over taps t and
//                        output channels co of g[co][position - off_t] *
//                        W[t][ci][co] -- the gradient planes read through the
//                        same shifted-descriptor trick as the forward pass
//   k_net_bwd_weight_tc  dL/dW[t][ci][co] = sum over positions p of
//                        a[ci][p + off_t] * g[co][p]: a GEMM whose K dimension
//                        is the positions; the rows (t, ci) are gathered per
//                        64-position chunk into shared memory (im2col), the
//                        chunks double-buffered against the MMAs
//
// The gradients are FP32. A bf16 operand keeps 8 bits, too few for them, so
// every gradient enters the MMAs as two bf16 parts, g = hi + lo (hi the
// nearest bf16, lo the nearest bf16 of the rest): two MMAs per product, about
// 16 significant bits. The activations are bf16 values already (the forward
// pass rounds them, the features included), so they enter exactly. Sums are
// FP32 in tensor memory. Every mbarrier wait is bounded (a fault flag, then
// the CTA leaves); tensor memory is always released.
#pragma once
#include <cstdint>

#include "svo_net.cuh"

namespace svo {

constexpr int kBwdOutW = kNetTW - 2, kBwdOutH = kNetTH - 2;  // 62 x 30 positions per tile (halo 1)
constexpr int kBwdThreads = 512;
constexpr int kBwdBlocks = 15;  // 128-position blocks of window rows 1..30

// Packed backward-data weights of layers 1-3, one 512-byte block per tap in
// the layout of k_net_prepare's blocks with the roles of the channels
// swapped: B[n = ci][k = co] = W[t][ci][co] (co past the layer's outputs: 0).
constexpr int kNetBwdBlocks = 27;

__global__ void k_net_prepare_bwd(const float* __restrict__ params, uint16_t* __restrict__ packed) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= kNetBwdBlocks * 256) return;
    const int blk = i >> 8, e = i & 255;
    const int l = 1 + blk / 9, t = blk % 9;
    const int ng = e >> 7, kc = (e >> 6) & 1, r = (e >> 3) & 7, k = e & 7;
    const int ci = ng * 8 + r, co = kc * 8 + k;
    float v = 0.0f;
    if (co < net_cout(l)) v = params[net_w_off(l) + (t * net_cin(l) + ci) * net_cout(l) + co];
    packed[i] = (uint16_t)bf16_bits(v);
}

// hi/lo bf16 parts of an FP32 value.
__device__ __forceinline__ void split_bf16(float v, uint32_t& hi, uint32_t& lo) {
    hi = bf16_bits(v);
    lo = bf16_bits(v - __uint_as_float(hi << 16));
}

// ------------------------------------------------------ backward data --
struct NetBwdDataArgs {
    const float* g;        // [kin][h][w]: gradient w.r.t. the layer's output (pre-activation)
    const uint16_t* wpk;   // the layer's 9 packed backward-data blocks
    const float* act;      // [16][h][w]: the layer's input activation (ReLU mask)
    float* g_in;           // [16][h][w]: gradient w.r.t. the previous layer's pre-activation
    int w, h, tiles_x, tiles;
    uint32_t* fault;
};

// Shared memory: the gradient's hi parts (two planes of 8 channels) and lo
// parts (two planes), each plane laid out as k_net_infer's activation planes,
// then the 9 weight blocks.
constexpr int kBwdDataSmemW = 4 * kNetPlaneBytes;
constexpr int kBwdDataSmem = kBwdDataSmemW + 9 * 512;

template <int KIN>
__global__ void __launch_bounds__(kBwdThreads, 1) k_net_bwd_data_tc(NetBwdDataArgs A) {
    __shared__ uint64_t mbar[kNetIssuers];
    __shared__ uint32_t tmem_base_s;
    uint8_t* smem = reinterpret_cast<uint8_t*>(svo_dsmem);
    const uint32_t sbase = smem_addr(smem);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int W = A.w, H = A.h;
    const size_t n = (size_t)W * H;

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
    {
        const uint4* src = reinterpret_cast<const uint4*>(A.wpk);
        uint4* dst = reinterpret_cast<uint4*>(smem + kBwdDataSmemW);
        for (int i = tid; i < 9 * 32; i += kBwdThreads) dst[i] = src[i];
        uint4* z = reinterpret_cast<uint4*>(smem);
        for (int i = tid; i < kBwdDataSmemW / 16; i += kBwdThreads) z[i] = make_uint4(0, 0, 0, 0);
    }
    __syncthreads();
    const uint32_t tmem = tmem_base_s;
    const uint32_t bar = smem_addr(&mbar[warp >> 2]);
    uint32_t phase = 0, fault = 0;

    for (int item = blockIdx.x; item < A.tiles; item += gridDim.x) {
        const int ox = (item % A.tiles_x) * kBwdOutW, oy = (item / A.tiles_x) * kBwdOutH;
        const int wx = ox - 1, wy = oy - 1;  // image position of window position 0
        // stage the gradient window as hi and lo bf16 planes
        for (int k = 0; k < kNetPos / kBwdThreads; ++k) {
            const int p = tid + k * kBwdThreads;
            const int gx = wx + (p & (kNetTW - 1)), gy = wy + (p >> 6);
            const bool inside = gx >= 0 && gx < W && gy >= 0 && gy < H;
            uint32_t hi[16], lo[16];
#pragma unroll
            for (int c = 0; c < 16; ++c) {
                const float v = (inside && c < KIN) ? __ldg(A.g + c * n + (size_t)gy * W + gx) : 0.0f;
                split_bf16(v, hi[c], lo[c]);
            }
#pragma unroll
            for (int h2 = 0; h2 < 2; ++h2) {
                const int c0 = 8 * h2;
                *reinterpret_cast<uint4*>(smem + h2 * kNetPlaneBytes + (kNetGuard + p) * 16) =
                    make_uint4(hi[c0] | hi[c0 + 1] << 16, hi[c0 + 2] | hi[c0 + 3] << 16, hi[c0 + 4] | hi[c0 + 5] << 16,
                               hi[c0 + 6] | hi[c0 + 7] << 16);
                *reinterpret_cast<uint4*>(smem + (2 + h2) * kNetPlaneBytes + (kNetGuard + p) * 16) =
                    make_uint4(lo[c0] | lo[c0 + 1] << 16, lo[c0 + 2] | lo[c0 + 3] << 16, lo[c0 + 4] | lo[c0 + 5] << 16,
                               lo[c0 + 6] | lo[c0 + 7] << 16);
            }
        }
        fence_async_smem();
        tc_fence_before();
        __syncthreads();
        tc_fence_after();
        if (lane == 0 && warp < kNetIssuers) {
            // blocks j = warp (mod 4): 9 taps x (hi, lo), output rows 1..30
            for (int j = warp; j < kBwdBlocks; j += kNetIssuers) {
#pragma unroll
                for (int t = 0; t < 9; ++t) {
                    const int off = (t / 3 - 1) * kNetTW + (t % 3 - 1);  // position offset of tap t
                    const uint32_t pos = (uint32_t)(kNetGuard + kNetTW + 128 * j - off);
                    const uint64_t bd = tc_desc(sbase + kBwdDataSmemW + (uint32_t)t * 512u, 128u, 256u);
                    tc_mma(tmem + 16u * j, tc_desc(sbase + pos * 16u, kNetPlaneBytes, 128u), bd, t > 0 ? 1u : 0u);
                    tc_mma(tmem + 16u * j, tc_desc(sbase + 2u * kNetPlaneBytes + pos * 16u, kNetPlaneBytes, 128u), bd,
                           1u);
                }
            }
            tc_commit(smem_addr(&mbar[warp]));
        }
        // While the MMAs run: the ReLU masks of this thread's output positions
        // (act > 0 per channel, one bit each), so the read-back below only waits
        // for tensor memory.
        constexpr int kMine = (kBwdBlocks + kNetWarps / 4 - 1) / (kNetWarps / 4);
        uint32_t relu[kMine];
        const int g = warp & 3;
#pragma unroll
        for (int k = 0; k < kMine; ++k) {
            const int j = (warp >> 2) + k * (kNetWarps / 4);
            relu[k] = 0u;
            const int p = kNetTW + 128 * j + 32 * g + lane;
            const int col = p & (kNetTW - 1);
            const int gx = wx + col, gy = wy + (p >> 6);
            if (j < kBwdBlocks && col >= 1 && col <= kBwdOutW && gx < W && gy < H) {
                const size_t o = (size_t)gy * W + gx;
#pragma unroll
                for (int c = 0; c < 16; ++c) relu[k] |= (__ldg(A.act + c * n + o) > 0.0f ? 1u : 0u) << c;
            }
        }
        const bool ready = mbar_wait_phase(bar, phase);
        phase ^= 1u;
        tc_fence_after();
        if (ready) {
#pragma unroll
            for (int k = 0; k < kMine; ++k) {
                const int j = (warp >> 2) + k * (kNetWarps / 4);
                if (j >= kBwdBlocks) continue;
                float v[16];
                tc_ld16(tmem + ((uint32_t)(32 * g) << 16) + 16u * j, v);
                const int p = kNetTW + 128 * j + 32 * g + lane;
                const int col = p & (kNetTW - 1);
                const int gx = wx + col, gy = wy + (p >> 6);
                if (col >= 1 && col <= kBwdOutW && gx < W && gy < H) {
                    const size_t o = (size_t)gy * W + gx;
#pragma unroll
                    for (int c = 0; c < 16; ++c) A.g_in[c * n + o] = ((relu[k] >> c) & 1u) ? v[c] : 0.0f;
                }
            }
        }
        tc_fence_before();
        const bool aborted = __syncthreads_or(ready ? 0 : 1) != 0;
        tc_fence_after();
        if (aborted) {
            fault |= kFaultNet;
            break;
        }
    }
    __syncthreads();
    if (warp == 0) {
        tc_fence_after();
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kNetTmemCols) : "memory");
    }
    if (fault && tid == 0) atomicOr(A.fault, fault);
}

// ---------------------------------------------------- backward weights --
struct NetBwdWeightArgs {
    const float* a;    // [cin][h][w]: the layer's input (the features for layer 0)
    const float* g;    // [kin][h][w]: gradient w.r.t. the layer's output (pre-activation)
    float* partial;    // [gridDim.x][9 * cin * kin + kin]
    int w, h, tiles_x, tiles;
    uint32_t* fault;
};

// Rows of the im2col operand: (tap, input channel) pairs, t * cin + ci; the
// first 128 in one operand, the rest (tap 8 when cin = 16) in a second one
// whose other rows stay zero.
constexpr int kBwdWStages = 4;                          // chunk buffers in flight
constexpr int kBwdWProducers = 512;                     // 16 warps stage the chunks
constexpr int kBwdWThreads = kBwdWProducers + 32;       // + the warp that issues the MMAs
template <int CIN>
struct BwdWeightLayout {
    static constexpr int kRows = 9 * CIN;
    static constexpr int kA1 = kRows > 128;                      // a second 128-row operand
    // bytes of one bf16 channel plane: the positions with their guards, padded
    // to 16 mod 128 so that 16-byte reads of the same slice of consecutive
    // channels fall in different banks
    static constexpr int kWinPlane = ((kNetPos + 2 * kNetGuard) * 2 + 127) / 128 * 128 + 16;
    static constexpr int kWin = CIN * kWinPlane;
    static constexpr int kK = 64;                                // positions per chunk (one window row)
    static constexpr int kABytes = 128 * kK * 2;                 // 16 KB
    static constexpr int kBBytes = 16 * kK * 2;                  // 2 KB
    static constexpr int kBuf = (1 + kA1) * kABytes + 2 * kBBytes;
    static constexpr int kSmem = kWin + kBwdWStages * kBuf;
};

__device__ __forceinline__ void mbar_arrive(uint32_t bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(bar) : "memory");
}
// Barrier 1 among the producer warps only (the issuing warp never joins it).
__device__ __forceinline__ void producers_sync() { asm volatile("bar.sync 1, %0;" ::"n"(kBwdWProducers) : "memory"); }

// Warp-specialised pipeline: 16 producer warps stage one 64-position chunk
// (a window row) at a time -- the im2col rows and the gradient rows -- into
// a ring of kBwdWStages buffers, arriving on the chunk's `full` barrier; one
// issuing thread waits for it, issues the chunk's MMAs and commits them to
// the buffer's `empty` barrier, which the producers wait on before they
// reuse the buffer. So the staging of later chunks runs while the tensor
// core works on earlier ones. Every wait is bounded: a producer or the
// issuer that gives up sets abort_s; after that the producers stop waiting
// (their barriers stay in step), the issuer stops issuing, the CTA waits
// (bounded) for the MMAs it issued, writes nothing and flags the fault.
template <int CIN, int KIN, bool kFirst>
__global__ void __launch_bounds__(kBwdWThreads, 1) k_net_bwd_weight_tc(NetBwdWeightArgs A) {
    using L = BwdWeightLayout<CIN>;
    constexpr int kTmemCols = 32;  // D0 in columns 0-15, D1 in 16-31
    constexpr int S = kBwdWStages;
    __shared__ uint64_t full[S], empty[S];
    __shared__ uint32_t tmem_base_s;
    __shared__ uint32_t abort_s;
    __shared__ float bias_s[kBwdWProducers / 32][8];  // per producer warp: its 8 channels' sums
    uint8_t* smem = reinterpret_cast<uint8_t*>(svo_dsmem);
    const uint32_t sbase = smem_addr(smem);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int W = A.w, H = A.h;
    const size_t n = (size_t)W * H;

    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_addr(&tmem_base_s)),
                     "r"(kTmemCols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    if (tid < S) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(&full[tid])), "n"(kBwdWProducers)
                     : "memory");
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_addr(&empty[tid])) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (tid == 0) abort_s = 0;
    {  // zero everything: window guards and the operand rows staging never writes
        uint4* z = reinterpret_cast<uint4*>(smem);
        for (int i = tid; i < L::kSmem / 16; i += kBwdWThreads) z[i] = make_uint4(0, 0, 0, 0);
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = tmem_base_s;
    int my_tiles = 0;
    for (int item = blockIdx.x; item < A.tiles; item += gridDim.x) ++my_tiles;
    const uint32_t n_chunks = (uint32_t)my_tiles * kBwdOutH;
    uint32_t fault = 0;

    if (warp == kBwdWProducers / 32) {
        // ---- the issuing warp: lane 0 issues every chunk's MMAs
        if (lane == 0) {
            uint32_t issued = 0;
            for (uint32_t c = 0; c < n_chunks; ++c) {
                const uint32_t st = c % S;
                if (!mbar_wait_phase(smem_addr(&full[st]), (c / S) & 1u)) atomicOr(&abort_s, 1u);
                if (*(volatile uint32_t*)&abort_s) break;
                tc_fence_after();
                const uint32_t a0 = sbase + (uint32_t)(L::kWin + st * L::kBuf);
                const uint32_t bhi = a0 + (uint32_t)((1 + L::kA1) * L::kABytes), blo = bhi + (uint32_t)L::kBBytes;
#pragma unroll
                for (int s = 0; s < L::kK / 16; ++s) {
                    const uint32_t acc = (c > 0 || s > 0) ? 1u : 0u;
                    const uint64_t bdh = tc_desc(bhi + (uint32_t)s * 256u, 128u, 1024u);
                    const uint64_t bdl = tc_desc(blo + (uint32_t)s * 256u, 128u, 1024u);
                    const uint64_t ad0 = tc_desc(a0 + (uint32_t)s * 4096u, 2048u, 128u);
                    tc_mma(tmem, ad0, bdh, acc);
                    tc_mma(tmem, ad0, bdl, 1u);
                    if (L::kA1) {
                        const uint64_t ad1 = tc_desc(a0 + (uint32_t)L::kABytes + (uint32_t)s * 4096u, 2048u, 128u);
                        tc_mma(tmem + 16u, ad1, bdh, acc);
                        tc_mma(tmem + 16u, ad1, bdl, 1u);
                    }
                }
                tc_commit(smem_addr(&empty[st]));
                issued = c + 1;
            }
            // the accumulators are complete once the last chunk's MMAs are
            if (issued > 0) {
                const uint32_t last = issued - 1;
                if (!mbar_wait_phase(smem_addr(&empty[last % S]), (last / S) & 1u)) atomicOr(&abort_s, 1u);
            }
            if (issued < n_chunks) atomicOr(&abort_s, 1u);
        }
        __syncwarp();
    } else {
        // ---- the producers
        // This thread's gradient pair: 16 warps x 32 lanes cover the 16 x 64
        // chunk, each warp one 8 x 8 block of the B operand's layout (channel
        // group w >> 3, position group w & 7), so its stores fill 128
        // contiguous bytes (conflict-free).
        const int g_co = (warp >> 3) * 8 + (lane >> 2), g_k = (warp & 7) * 8 + (lane & 3) * 2;
        const int b_idx = (g_co >> 3) * (8 * L::kK) + (g_k >> 3) * 64 + (g_co & 7) * 8 + (g_k & 7);
        // This thread's im2col items (row (t, ci), 8-position group kc): what
        // does not depend on the chunk -- the aligned source offset in the
        // window (a chunk adds its row), how the slice sits in the two
        // aligned 16-byte reads (word offset 0 or 3, shift 0 or 16 bits), and
        // where it goes in the operand.
        constexpr int kItems = L::kRows * (L::kK / 8);
        constexpr int kMaxIt = (kItems + kBwdWProducers - 1) / kBwdWProducers;
        uint32_t it_src[kMaxIt], it_dst[kMaxIt], it_sh[kMaxIt];
        bool it_w3[kMaxIt], it_ok[kMaxIt];
#pragma unroll
        for (int k = 0; k < kMaxIt; ++k) {
            const int it = tid + k * kBwdWProducers;
            it_ok[k] = it < kItems;
            const int kc = it / L::kRows, r = it - kc * L::kRows;
            const int t = r / CIN, ci = r % CIN;
            const int off = (t / 3 - 1) * kNetTW + (t % 3 - 1);
            const int e0 = kNetGuard + kc * 8 + off;  // element index in the plane at row 0
            const int a = e0 & ~7;                    // rows are 64 positions: alignment is the row's
            it_src[k] = (uint32_t)(ci * L::kWinPlane + a * 2);
            it_w3[k] = (e0 - a) == 7;                 // the slice starts in the group's last word
            it_sh[k] = (e0 != a) ? 16u : 0u;
            it_dst[k] = (uint32_t)((r >> 7) * L::kABytes + kc * 2048 + (r & 127) * 16);
        }
        bool stop = false;  // this thread saw the abort: no more waits
        uint32_t c = 0;
        float bias_acc2 = 0.0f;  // g_co's sum over this thread's positions
        for (int item = blockIdx.x; item < A.tiles; item += gridDim.x) {
            const int ox = (item % A.tiles_x) * kBwdOutW, oy = (item / A.tiles_x) * kBwdOutH;
            const int wx = ox - 1, wy = oy - 1;
            producers_sync();  // every producer has read the last tile's window
            // the input window, bf16 channel planes with a guard of kNetGuard
            // positions: 16 loads in flight per thread, then their stores
            constexpr int kPer = CIN * kNetPos / kBwdWProducers;
            static_assert(kPer % 16 == 0, "window staging in groups of 16 loads");
            for (int b = 0; b < kPer; b += 16) {
                float v[16];
#pragma unroll
                for (int j = 0; j < 16; ++j) {
                    const int i = tid + (b + j) * kBwdWProducers;
                    const int ci = i / kNetPos, p = i % kNetPos;
                    const int gx = wx + (p & (kNetTW - 1)), gy = wy + (p >> 6);
                    v[j] = (gx >= 0 && gx < W && gy >= 0 && gy < H) ? __ldg(A.a + ci * n + (size_t)gy * W + gx) : 0.0f;
                }
#pragma unroll
                for (int j = 0; j < 16; ++j) {
                    const int i = tid + (b + j) * kBwdWProducers;
                    const int ci = i / kNetPos, p = i % kNetPos;
                    const float x = kFirst ? bf16_round(v[j]) : v[j];
                    reinterpret_cast<uint16_t*>(smem)[ci * (L::kWinPlane / 2) + kNetGuard + p] =
                        (uint16_t)bf16_bits(x);
                }
            }
            // gradient values of window row r of this tile, zero outside it
            auto load_g = [&](int row, float* out) {
#pragma unroll
                for (int e = 0; e < 2; ++e) {
                    const int kk = g_k + e;
                    const int gx = wx + kk, gy = wy + row;
                    out[e] = (g_co < KIN && kk >= 1 && kk <= kBwdOutW && gx < W && gy < H)
                                 ? __ldg(A.g + g_co * n + (size_t)gy * W + gx)
                                 : 0.0f;
                }
            };
            // gradient values of the next kAhead chunks in flight (registers)
            constexpr int kAhead = 3;
            float gq[kAhead][2];
#pragma unroll
            for (int a = 0; a < kAhead; ++a) load_g(1 + a, gq[a]);
            producers_sync();  // the window is complete
            for (int cr = 0; cr < kBwdOutH; ++cr, ++c) {
                const uint32_t st = c % S;
                const float g0 = gq[0][0], g1 = gq[0][1];
#pragma unroll
                for (int a = 0; a + 1 < kAhead; ++a) {
                    gq[a][0] = gq[a + 1][0];
                    gq[a][1] = gq[a + 1][1];
                }
                if (cr + kAhead < kBwdOutH) {
                    load_g(cr + 1 + kAhead, gq[kAhead - 1]);
                } else {
                    gq[kAhead - 1][0] = gq[kAhead - 1][1] = 0.0f;
                }
                if (!stop && c >= S && !mbar_wait_phase(smem_addr(&empty[st]), (c / S - 1u) & 1u))
                    atomicOr(&abort_s, 1u);
                if (*(volatile uint32_t*)&abort_s) stop = true;
                uint8_t* bufp = smem + L::kWin + st * L::kBuf;
                const uint32_t rofs = (uint32_t)(cr + 1) * (kNetTW * 2);  // this chunk's window row, bytes
                // im2col: two aligned 16-byte reads and a funnel shift per item
#pragma unroll
                for (int k = 0; k < kMaxIt; ++k) {
                    if (!it_ok[k]) continue;
                    const uint4 lo = *reinterpret_cast<const uint4*>(smem + it_src[k] + rofs);
                    const uint4 hi = *reinterpret_cast<const uint4*>(smem + it_src[k] + rofs + 16);
                    const bool w3 = it_w3[k];
                    const uint32_t sh = it_sh[k];
                    uint4 v;
                    v.x = __funnelshift_r(w3 ? lo.w : lo.x, w3 ? hi.x : lo.y, sh);
                    v.y = __funnelshift_r(w3 ? hi.x : lo.y, w3 ? hi.y : lo.z, sh);
                    v.z = __funnelshift_r(w3 ? hi.y : lo.z, w3 ? hi.z : lo.w, sh);
                    v.w = __funnelshift_r(w3 ? hi.z : lo.w, w3 ? hi.w : hi.x, sh);
                    *reinterpret_cast<uint4*>(bufp + it_dst[k]) = v;
                }
                // gradient pair: hi and lo parts (the B operands), one 32-bit store each
                {
                    bias_acc2 += g0 + g1;
                    uint32_t h0, l0, h1, l1;
                    split_bf16(g0, h0, l0);
                    split_bf16(g1, h1, l1);
                    uint16_t* bh = reinterpret_cast<uint16_t*>(bufp + (1 + L::kA1) * L::kABytes);
                    uint16_t* bl = bh + L::kBBytes / 2;
                    *reinterpret_cast<uint32_t*>(bh + b_idx) = h0 | (h1 << 16);
                    *reinterpret_cast<uint32_t*>(bl + b_idx) = l0 | (l1 << 16);
                }
                fence_async_smem();  // the stores reach the tensor core's view of shared memory
                mbar_arrive(smem_addr(&full[st]));
            }
        }
        // biases: the 4 lanes of a channel in this warp, then (below) the 8
        // warps of its channel group, in a fixed order
        float s = bias_acc2;
        s += __shfl_xor_sync(0xffffffffu, s, 1);
        s += __shfl_xor_sync(0xffffffffu, s, 2);
        if ((lane & 3) == 0) bias_s[warp][lane >> 2] = s;
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    constexpr int kVals = 9 * CIN * KIN + KIN;
    float* dst = A.partial + (size_t)blockIdx.x * kVals;
    if (!abort_s) {
        if (warp < 4) {
            float v[16];
            if (n_chunks > 0) {
                tc_ld16(tmem + ((uint32_t)(32 * warp) << 16), v);
            } else {
#pragma unroll
                for (int c = 0; c < 16; ++c) v[c] = 0.0f;
            }
            const int r = 32 * warp + lane;
            if (r < (L::kA1 ? 128 : L::kRows))
#pragma unroll
                for (int c = 0; c < KIN; ++c) dst[r * KIN + c] = v[c];
            if (L::kA1) {
                if (n_chunks > 0) {
                    tc_ld16(tmem + ((uint32_t)(32 * warp) << 16) + 16u, v);
                }
                if (r < L::kRows - 128)
#pragma unroll
                    for (int c = 0; c < KIN; ++c) dst[(128 + r) * KIN + c] = v[c];
            }
        }
        if (tid < KIN) {
            // channel tid: the 8 warps of its group, in order
            float s = 0.0f;
            for (int w = 0; w < 8; ++w) s += bias_s[(tid >> 3) * 8 + w][tid & 7];
            dst[9 * CIN * KIN + tid] = s;
        }
    } else {
        fault |= kFaultNet;
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 0) {
        tc_fence_after();
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kTmemCols) : "memory");
    }
    if (fault && tid == 0) atomicOr(A.fault, fault);
}

}  // namespace svo
