// svo_device.cu -- device runtime of libsvo_gb300.so: context, octree upload,
// render targets, the per-frame launch sequence and its C ABI.
//
// Replaces the reference's OpenCL wrapper (src/ocl.h) and the device half of
// its frame driver (src/raycast.h). One context = one device, one in-order
// stream (the reference's single command queue, src/ocl.h:140). Frames never
// synchronise the host: the hole count that raycast_draw reads back with a
// blocking 4-byte copy (src/raycast.h:298) stays on the device and sizes the
// persistent trace launch's work queue.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/svo_gb300.h"
#include "svo_kernels.cuh"
#include "svo_net.cuh"
#include "svo_net_train.cuh"
#include "svo_build.cuh"

using namespace svo;

struct svo_context {
    int device = 0;
    cudaStream_t stream = nullptr;
    int sm_count = 0;
    uint32_t* d_octree = nullptr;
    bool owns_octree = false;
    size_t n_words = 0;
    uint32_t root = 0;
    int depth = 0;
    uint32_t* d_fault = nullptr;  // device fault flags (kFault*)
    // Batch tables of full raycasts: a ring of pinned staging copies so a call
    // never waits for the GPU unless it laps the ring.
    static constexpr int kRing = 4;
    FullBatch* d_batch[kRing] = {};
    FullBatch* h_batch[kRing] = {};
    cudaEvent_t batch_done[kRing] = {};
    int batch_slot = 0;
    uint32_t* d_counter = nullptr;
    size_t l2_window = 0;
    size_t l2_window_request = ~(size_t)0;  // default: the whole octree
    bool stage_normal = true;               // stage the normal-node region in shared memory
    int pw_shift = 3;                       // ray packets (1<<pw_shift) x (32>>pw_shift): 8x4
    int block_pref = 0;                     // trace block size, 0: chosen by the staging size
    int learned_block_pref = 0;             // the same for learned frames' tracer
    int learned_pw_shift = -1;              // learned frames' ray packets; -1: as pw_shift
    // svo_context_autotune's choice for full raycasts only (-1: as the three
    // options above, which warp frames always follow)
    int full_pw_shift = -1, full_block_pref = -1, full_stage = -1;
    uint64_t config_gen = 0;                // bumped by every option change (captured graphs re-capture)
    uint64_t launches = 0;
    std::vector<svo_target*> targets;  // live targets, destroyed with the context
    std::vector<svo_net*> nets;        // live nets, likewise
    std::string err;
};

// A captured frame and what its capture baked in.
struct FrameGraph {
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    cudaGraphNode_t params_node = nullptr;
    uint64_t launches = 0;  // kernels one replay launches
    bool profiled = false;
    const void* net = nullptr;
    float threshold = 0.0f;
    float* tap = nullptr;
    bool coarse = false;
    bool guided = false;
    bool readback = false;
    uint64_t config_gen = 0;
    void reset() {
        if (exec) cudaGraphExecDestroy(exec);
        if (graph) cudaGraphDestroy(graph);
        exec = nullptr;
        graph = nullptr;
        params_node = nullptr;
    }
};

struct svo_target {
    svo_context* ctx = nullptr;
    int res_x = 0, res_y = 0;
    size_t N = 0, tiles = 0;
    TargetBuffers B{};
    FrameParams* d_params = nullptr;
    uint32_t* full_col = nullptr;
    float4* full_xyzw = nullptr;
    uint64_t* full_vox = nullptr;
    uint64_t frames = 0;      // warp frames issued
    bool have_prev = false;
    // Roles of the three physical planes (see plan_planes): the last frame's
    // plane 0 (reference plane `last_target`), the other cache plane (the
    // reference's plane 3 - last_target, -1 while it is empty).
    int cache_mode = 0;  // 0: copy target 2 (raycast.h:395); 1: ((frame>>4)%2)+1
    bool coarse = false;  // the raycast_fine pass (raycast.h:235-261)
    int last_cur = 0;
    int other = -1;
    int last_target = 2;
    // previous frame's camera (motion feature of learned frames)
    svo_view prev_view{};
    bool have_prev_view = false;
    float* feature_tap = nullptr;  // device [8][N]: features written after reprojection
    uint32_t* req_offs = nullptr;  // learned frames: request offsets per 8x4 packet
    // guided learned frames (walks from the cached depth); buffers in B
    bool guided = false;
    bool certify = false;  // certified reprojection in guided learned frames
    float* d_guide = nullptr;
    // camera position each physical plane's points were written under (the
    // rebase of learned frames across wraps of the periodic volume)
    float plane_pos[3][3] = {};
    // CUDA graphs of one warp frame: [0] plain, [1] learned
    bool use_graph = false;
    FrameGraph graphs[2];
    bool capturing = false;
    // per-stage timing
    bool profiling = false;
    cudaEvent_t ev[8] = {};
    int n_events = 0;
    int last_mode = 0;  // 1 warp, 2 full, 3 learned warp
    // asynchronous BGRX readback: the copy runs on the target's own stream
    // while the next frame renders; that frame's first write to the image
    // waits for it (readback_guard)
    bool async_readback = false;
    cudaStream_t copy_stream = nullptr;
    cudaEvent_t frame_done = nullptr, copy_done = nullptr;
};

// The reconstruction net: FP32 master parameters with Adam moments, their
// bf16 forms for the kernels, and the training buffers (grown on demand).
struct svo_net {
    svo_context* ctx = nullptr;
    float* params = nullptr;
    float* m = nullptr;
    float* v = nullptr;
    float* grads = nullptr;
    float* wr = nullptr;         // bf16-rounded weights, FP32 (CUDA-core path)
    uint16_t* packed = nullptr;  // tensor-core operand image
    uint16_t* packed_bwd = nullptr;  // backward-data operand image (layers 1-3)
    float* bias = nullptr;       // 52 biases
    int step = 0;
    size_t cap = 0;           // pixels the training buffers hold
    float* act = nullptr;     // 3 hidden activations, 16 planes each
    float* out = nullptr;     // 4 planes
    float* dout = nullptr;    // 4 planes
    float* g0 = nullptr;      // 16 planes
    float* g1 = nullptr;      // 16 planes
    float* partial = nullptr;  // weight-gradient partial sums
    size_t partial_cap = 0;    // floats
    float* loss_partial = nullptr;
    size_t loss_cap = 0;  // blocks
};

namespace {

// The persisting-L2 set-aside is one setting of the CUDA context, which every
// svo_context on a device shares; it is released only when the last context
// holding a window gives it up.
std::mutex g_l2_mutex;
int g_l2_users[64] = {};

void l2_window_acquire(int device) {
    std::lock_guard<std::mutex> lock(g_l2_mutex);
    if (device >= 0 && device < 64) ++g_l2_users[device];
}
void l2_window_release(int device) {
    std::lock_guard<std::mutex> lock(g_l2_mutex);
    if (device < 0 || device >= 64 || g_l2_users[device] <= 0) return;
    if (--g_l2_users[device] == 0) {
        cudaCtxResetPersistingL2Cache();
        cudaDeviceSetLimit(cudaLimitPersistingL2CacheSize, 0);
    }
}

const char* status_text(svo_status s) {
    switch (s) {
        case SVO_OK: return "ok";
        case SVO_ERR_INVALID_ARGUMENT: return "invalid argument";
        case SVO_ERR_CUDA: return "CUDA error";
        case SVO_ERR_NO_OCTREE: return "no octree uploaded";
        case SVO_ERR_BAD_OCTREE: return "octree validation failed";
        case SVO_ERR_DEVICE_FAULT: return "device fault flag set";
        case SVO_ERR_OUT_OF_MEMORY: return "out of memory";
        case SVO_ERR_CAPACITY: return "capacity exceeded";
        case SVO_ERR_NOT_SUPPORTED: return "not supported";
        case SVO_ERR_IO: return "I/O error";
    }
    return "unknown";
}

svo_status fail(svo_context* ctx, svo_status s, const std::string& what) {
    if (ctx) ctx->err = std::string(status_text(s)) + ": " + what;
    return s;
}

#define SVO_CUDA(ctx, call)                                                                   \
    do {                                                                                      \
        cudaError_t e_ = (call);                                                              \
        if (e_ != cudaSuccess) {                                                              \
            return fail((ctx), e_ == cudaErrorMemoryAllocation ? SVO_ERR_OUT_OF_MEMORY : SVO_ERR_CUDA, \
                        std::string(#call) + " -> " + cudaGetErrorString(e_));                \
        }                                                                                     \
    } while (0)

#define SVO_LAUNCHED(ctx)                                                                     \
    do {                                                                                      \
        cudaError_t e_ = cudaGetLastError();                                                  \
        if (e_ != cudaSuccess) return fail((ctx), SVO_ERR_CUDA, std::string("launch: ") + cudaGetErrorString(e_)); \
        ++(ctx)->launches;                                                                    \
    } while (0)

RayCam make_raycam(const svo_view& v) {
    // Rows of m^T = columns of m (src/raycast.h:225-228).
    const float* m = v.m;
    RayCam c;
    c.px = v.pos[0];
    c.py = v.pos[1];
    c.pz = v.pos[2];
    c.mxx = m[0];
    c.mxy = m[4];
    c.mxz = m[8];
    c.myx = m[1];
    c.myy = m[5];
    c.myz = m[9];
    c.mzx = m[2];
    c.mzy = m[6];
    c.mzz = m[10];
    c.fovx = v.fovx;
    c.fovy = v.fovy;
    return c;
}

// Host walk of the compact octree in the builder's layout (normal nodes above
// height 6, blocks below). Checks every address the traversal can form.
struct Validator {
    const uint32_t* w;
    size_t n;
    int depth;
    size_t visits = 0, limit;
    std::string why;

    bool fail_at(const char* what, size_t at) {
        char buf[128];
        std::snprintf(buf, sizeof(buf), "%s at word %zu", what, at);
        why = buf;
        return false;
    }
    bool block(size_t local_root, uint32_t word, int h, bool is_root) {
        if (++visits > limit) return fail_at("node visited twice (not a tree)", 0);
        if (!(word & 256u)) return fail_at("block node without block flag", local_root);
        const size_t pos = is_root ? local_root : local_root + (word >> 9);
        const uint32_t mask = word & 0xffu;
        const uint32_t kids = __builtin_popcount(mask);
        if (h == 2) {
            const size_t head = 1 + kids;
            if (pos + (head + 3) / 4 > n) return fail_at("byte record past the end", pos);
            size_t bytes = head;
            for (uint32_t k = 0; k < kids; ++k) {
                const size_t b = 1 + k;
                bytes += __builtin_popcount((w[pos + b / 4] >> (8 * (b & 3))) & 0xffu);
            }
            if (pos + (bytes + 3) / 4 > n) return fail_at("byte record past the end", pos);
            return true;
        }
        if (pos + 1 + kids > n) return fail_at("block node past the end", pos);
        for (uint32_t k = 0; k < kids; ++k)
            if (!block(local_root, w[pos + 1 + k], h - 1, false)) return false;
        return true;
    }
    bool normal(uint32_t word, int h) {
        if (++visits > limit) return fail_at("node visited twice (not a tree)", 0);
        if (word & 256u) return fail_at("normal node with block flag", word >> 9);
        const size_t at = word >> 9;
        if (at + 10 > n) return fail_at("normal node past the end", at);
        for (int j = 0; j < 8; ++j) {
            if (!((word >> j) & 1u)) continue;
            const uint32_t cw = w[at + j];
            if (h - 1 >= 7) {
                if (!normal(cw, h - 1)) return false;
            } else {
                const size_t lr = (size_t)(cw >> 9) << 6;
                if (!block(lr, cw, h - 1, true)) return false;
            }
        }
        return true;
    }
};

// Launch geometry of the trace kernels. The normal-node region (words
// [0, (root>>9)+10), written first by convert_tree_blocks) is staged into
// shared memory when it fits: 256-thread blocks for a small region, 1024-thread
// blocks (one per SM, 32 warps) for a large one; otherwise no staging.
constexpr uint32_t kStageSmallBytes = 48u * 1024u;
constexpr uint32_t kStageMaxBytes = 160u * 1024u;

struct TraceLaunch {
    const void* fn;
    int block;
    size_t smem;
    Octree o;
};

// Trace kernels: full raycast, warp-frame holes + refresh tile, and the same
// for learned frames (which also write the traced pixels' BGRX).
enum TraceKind { kTraceFull = 0, kTraceWarp = 1, kTraceWarpBgrx = 2, kTraceCoarse = 3 };

template <int DEPTH, int BLOCK>
const void* trace_fn(int kind) {
    if (kind == kTraceWarp) return (const void*)k_trace_warp<DEPTH, BLOCK, false>;
    if (kind == kTraceWarpBgrx) return (const void*)k_trace_warp<DEPTH, BLOCK, true>;
    if (kind == kTraceCoarse) return (const void*)k_trace_coarse<DEPTH, BLOCK>;
    return (const void*)k_trace_full<DEPTH, BLOCK, true>;
}

template <int BLOCK>
const void* trace_fn_depth(int depth, int kind) {
    switch (depth) {
        case 8: return trace_fn<8, BLOCK>(kind);
        case 9: return trace_fn<9, BLOCK>(kind);
        case 10: return trace_fn<10, BLOCK>(kind);
        case 11: return trace_fn<11, BLOCK>(kind);
        case 12: return trace_fn<12, BLOCK>(kind);
    }
    return nullptr;
}

// Packet shape of full raycasts: the autotuner's choice, else the option.
int full_pw_shift(const svo_context* ctx) { return ctx->full_pw_shift >= 0 ? ctx->full_pw_shift : ctx->pw_shift; }

svo_status plan_trace(svo_context* ctx, int kind, TraceLaunch& L) {
    L.o = Octree{ctx->d_octree, (uint32_t)ctx->n_words, ctx->root, 0u, 0u};
    uint32_t stage_bytes = 0;
    const bool full = kind == kTraceFull;
    const bool stage = full && ctx->full_stage >= 0 ? ctx->full_stage != 0 : ctx->stage_normal;
    if (stage && !(ctx->root & 256u) && (reinterpret_cast<uintptr_t>(ctx->d_octree) & 15u) == 0) {
        const uint64_t nw = (uint64_t)(ctx->root >> 9) + 10u;
        const uint64_t bytes = (nw * 4u + 15u) & ~15ull;
        if (bytes <= kStageMaxBytes && bytes <= (uint64_t)ctx->n_words * 4u) {
            L.o.n_smem = (uint32_t)nw;
            stage_bytes = (uint32_t)bytes;
        }
    }
    const int pref = kind == kTraceWarpBgrx                ? ctx->learned_block_pref
                     : full && ctx->full_block_pref >= 0 ? ctx->full_block_pref
                                                         : ctx->block_pref;
    L.block = stage_bytes > kStageSmallBytes ? 1024 : 256;
    if (pref == 1024) L.block = 1024;
    if (pref == 256 && L.block == 1024) {  // the staged region does not fit a 256-thread block
        L.block = 256;
        L.o.n_smem = 0;
        stage_bytes = 0;
    }
    L.fn = L.block == 1024 ? trace_fn_depth<1024>(ctx->depth, kind) : trace_fn_depth<256>(ctx->depth, kind);
    if (!L.fn) return fail(ctx, SVO_ERR_NOT_SUPPORTED, "octree depth");
    L.smem = (size_t)(ctx->depth + 2) * L.block * 4u + stage_bytes;  // stack: kStackLevels
    SVO_CUDA(ctx, cudaFuncSetAttribute(L.fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)L.smem));
    return SVO_OK;
}

// Persistent grid: as many blocks as fit on every SM; the access-policy
// window travels with the launch so graph-captured launches keep it.
// Programmatic stream serialisation for a launch of the learned frame's
// kernel chain: the kernel may start its own set-up while the kernel before
// it finishes, and calls grid_dep_wait() before it reads that kernel's output.
void add_chained(cudaLaunchConfig_t& cfg, cudaLaunchAttribute* attr) {
    attr[cfg.numAttrs].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[cfg.numAttrs].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    ++cfg.numAttrs;
}

svo_status launch_trace(svo_context* ctx, const TraceLaunch& L, void** args, bool chained = false) {
    int per_sm = 0;
    SVO_CUDA(ctx, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, L.fn, L.block, L.smem));
    cudaLaunchConfig_t cfg{};
    cfg.gridDim = dim3((unsigned)(std::max(1, per_sm) * ctx->sm_count));
    cfg.blockDim = dim3((unsigned)L.block);
    cfg.dynamicSmemBytes = L.smem;
    cfg.stream = ctx->stream;
    cudaLaunchAttribute attr[2];
    if (ctx->l2_window > 0) {
        attr[0].id = cudaLaunchAttributeAccessPolicyWindow;
        attr[0].val.accessPolicyWindow.base_ptr = ctx->d_octree;
        attr[0].val.accessPolicyWindow.num_bytes = ctx->l2_window;
        attr[0].val.accessPolicyWindow.hitRatio = 1.0f;
        attr[0].val.accessPolicyWindow.hitProp = cudaAccessPropertyPersisting;
        attr[0].val.accessPolicyWindow.missProp = cudaAccessPropertyStreaming;
        cfg.attrs = attr;
        cfg.numAttrs = 1;
    }
    if (chained) add_chained(cfg, attr);
    SVO_CUDA(ctx, cudaLaunchKernelExC(&cfg, L.fn, args));
    ++ctx->launches;
    return SVO_OK;
}

svo_status launch_trace_full(svo_context* ctx, FullBatch* d_batch) {
    TraceLaunch L;
    svo_status st = plan_trace(ctx, kTraceFull, L);
    if (st != SVO_OK) return st;
    void* args[] = {&L.o, &d_batch, &ctx->d_counter, &ctx->d_fault};
    return launch_trace(ctx, L, args);
}

svo_status launch_trace_warp(svo_context* ctx, svo_target* t, int kind = kTraceWarp, bool chained = false) {
    TraceLaunch L;
    svo_status st = plan_trace(ctx, kind, L);
    if (st != SVO_OK) return st;
    void* args[] = {&L.o, &t->d_params, &t->B, &ctx->d_fault};
    return launch_trace(ctx, L, args, chained);
}

// Grid for a grid-stride loop over n items: enough blocks, capped at 32 per SM.
inline unsigned grid_for(size_t n, int threads, int sm_count) {
    return (unsigned)std::max<size_t>(1, std::min<size_t>((n + threads - 1) / threads, (size_t)sm_count * 32));
}

// Before a frame's first write to the BGRX image: wait for the asynchronous
// readback of the previous image (a no-op until svo_read_bgrx_async is used;
// a wait node in a captured graph).
svo_status readback_guard(svo_target* t) {
    if (!t->async_readback || !t->copy_done) return SVO_OK;
    SVO_CUDA(t->ctx, cudaStreamWaitEvent(t->ctx->stream, t->copy_done, t->capturing ? cudaEventWaitExternal : 0));
    return SVO_OK;
}

void record(svo_target* t, int i) {
    if (!t->profiling) return;
    if (t->capturing)
        cudaEventRecordWithFlags(t->ev[i], t->ctx->stream, cudaEventRecordExternal);
    else
        cudaEventRecord(t->ev[i], t->ctx->stream);
}

// Which physical plane plays which role in one frame. The reference keeps
// plane 0 (current) and cache planes 1 and 2, projects both caches into
// plane 0 and copies plane 0 into the target cache at the end. Here plane 0
// is written into a free physical plane and simply becomes the target cache
// (no copy); the other cache keeps its physical plane.
struct PlanePlan {
    int cur, src[2], target, other_after, fill_past;
    bool clear;
};

PlanePlan plan_planes(const svo_target* t, int frame, bool have_cache, int mode) {
    PlanePlan q{};
    q.src[0] = q.src[1] = -1;
    int other = t->other;
    if (have_cache) {
        q.src[t->last_target - 1] = t->last_cur;
        q.src[2 - t->last_target] = other;
    } else {
        other = -1;  // frames 0 and 1 clear every plane (raycast.h:150-154)
    }
    for (int c = 0; c < 3; ++c)
        if ((!have_cache || c != t->last_cur) && c != other) {
            q.cur = c;
            break;
        }
    q.target = mode ? ((frame >> 4) % 2) + 1 : 2;
    q.other_after = -1;
    if (mode) q.other_after = (have_cache && q.target != t->last_target) ? t->last_cur : other;
    q.fill_past = q.target == 1 ? q.cur : q.other_after;
    q.clear = mode != 0;
    return q;
}

void commit_planes(svo_target* t, const PlanePlan& q, const svo_view& v) {
    for (int i = 0; i < 3; ++i) t->plane_pos[q.cur][i] = v.pos[i];
    t->last_cur = q.cur;
    t->other = q.other_after;
    t->last_target = q.target;
}

// Whole periods (of length e) between two wrapped camera positions: a point
// written under camera a lies at point + shift under camera b, assuming the
// camera moved less than half a period between the two.
void period_shift(const float* a, const float* b, float e, float out[3]) {
    for (int i = 0; i < 3; ++i) out[i] = (float)std::nearbyint(((double)b[i] - (double)a[i]) / e) * e;
}

// Guided learned frames resolve the projection keys inside k_guide (one launch
// less), except when the training tap reads the plane between the two.
bool guided_resolve(const svo_target* t, bool learned) { return learned && t->B.guide && !t->feature_tap; }

FrameParams make_params(const svo_target* t, const svo_view& v, int frame, const PlanePlan& q, bool have_cache,
                        bool learned = false) {
    FrameParams p{};
    p.ray = make_raycam(v);
    for (int i = 0; i < 3; ++i) {
        p.vx[i] = v.m[0 + i];
        p.vy[i] = v.m[4 + i];
        p.vz[i] = v.m[8 + i];
    }
    p.frame = frame;
    p.cur = q.cur;
    p.have_cache = have_cache ? 1 : 0;
    p.src_plane[0] = q.src[0];
    p.src_plane[1] = q.src[1];
    p.clear_rejected = q.clear ? 1 : 0;
    p.fill_past = q.fill_past;
    // raycast.h:363-366: tile (frame&7, (frame>>3)&3) of an 8x4 grid; the
    // NDRange of res/8 x res/4 work-items is rounded up to 16 (ocl.h:234-235).
    const int rx = t->res_x, ry = t->res_y;
    p.add_x = (rx / 8) * (frame & 7);
    p.add_y = (ry / 4) * ((frame >> 3) & 3);
    const int gx = (rx / 8 + 15) / 16 * 16, gy = (ry / 4 + 15) / 16 * 16;
    p.x_end = std::min(rx, p.add_x + gx);
    p.y_end = std::min(ry, p.add_y + gy);
    p.pw_shift = (learned && t->ctx->learned_pw_shift >= 0) ? t->ctx->learned_pw_shift : t->ctx->pw_shift;
    p.coarse_x = (rx / 2) * (frame & 1);
    p.coarse_y = (ry / 2) * ((frame >> 1) & 1);
    p.have_prev_view = t->have_prev_view ? 1 : 0;
    for (int i = 0; i < 3; ++i) {
        p.prev_pos[i] = t->prev_view.pos[i];
        p.prev_vx[i] = t->prev_view.m[0 + i];
        p.prev_vy[i] = t->prev_view.m[4 + i];
        p.prev_vz[i] = t->prev_view.m[8 + i];
    }
    p.serial = (uint32_t)(t->frames + 1);
    p.certify = (learned && t->guided && t->certify) ? 1 : 0;
    p.clear_keys = guided_resolve(t, learned) ? 1 : 0;
    if (learned) {
        const float period = (float)(1u << (t->ctx->depth + 1)) / 16.0f;  // world units
        p.rebase = 1;
        for (int r = 0; r < 2; ++r)
            if (q.src[r] >= 0) period_shift(t->plane_pos[q.src[r]], v.pos, period, p.src_shift[r]);
        if (t->have_prev_view) {
            float sh[3];
            period_shift(t->prev_view.pos, v.pos, period, sh);
            for (int i = 0; i < 3; ++i) p.prev_pos[i] = t->prev_view.pos[i] + sh[i];
        }
    }
    return p;
}

// The launch sequence of one warp frame after k_set_params.
svo_status enqueue_warp_body(svo_context* ctx, svo_target* t) {
    cudaStream_t s = ctx->stream;
    const int res_x = t->res_x, res_y = t->res_y;
    record(t, 0);
    {
        const int threads = 256;
        int blocks = (int)std::min<size_t>((t->N + threads - 1) / threads, (size_t)ctx->sm_count * 8);
        k_project<<<blocks, threads, 0, s>>>(t->d_params, t->B);
        SVO_LAUNCHED(ctx);
    }
    record(t, 1);
    k_resolve_gather<<<dim3((res_x + 15) / 16, (res_y + 15) / 16), 256, 0, s>>>(t->d_params, t->B);
    SVO_LAUNCHED(ctx);
    if (t->coarse) {
        svo_status cs = launch_trace_warp(ctx, t, kTraceCoarse);
        if (cs != SVO_OK) return cs;
        k_hole_mask<<<dim3((res_x + 15) / 16, (res_y + 15) / 16), 256, 0, s>>>(t->d_params, t->B);
        SVO_LAUNCHED(ctx);
    }
    if (t->feature_tap) {
        k_net_features<<<dim3((res_x + 31) / 32, (res_y + 7) / 8), 256, 0, s>>>(t->d_params, t->B, t->feature_tap);
        SVO_LAUNCHED(ctx);
    }
    record(t, 2);
    {
        const uint32_t tiles = (uint32_t)t->B.tiles_x * (uint32_t)t->B.tiles_y;
        const int staged = tiles <= kScanStageTiles ? 1 : 0;
        const size_t smem = staged ? (size_t)tiles * 8u : 0u;
        SVO_CUDA(ctx, cudaFuncSetAttribute(k_hole_scan, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        k_hole_scan<<<1, 1024, smem, s>>>(t->B, staged);
        SVO_LAUNCHED(ctx);
    }
    record(t, 3);
    if (t->tiles > 0) {
        k_hole_write<<<(unsigned)((t->tiles + 7) / 8), 256, 0, s>>>(t->B);
        SVO_LAUNCHED(ctx);
    }
    record(t, 4);
    svo_status st = launch_trace_warp(ctx, t);
    if (st != SVO_OK) return st;
    record(t, 5);
    if (svo_status gs = readback_guard(t); gs != SVO_OK) return gs;
    k_fill_colorize<<<dim3((res_x + 31) / 32, (res_y + 7) / 8), 256, 0, s>>>(t->d_params, t->B);
    SVO_LAUNCHED(ctx);
    record(t, 6);
    return SVO_OK;
}

// Tensor-core inference launch: one CTA per SM over the 56x24 output tiles.
svo_status launch_net_infer(svo_context* ctx, const svo_net* net, bool pipeline, NetInferArgs& A) {
    A.packed = net->packed;
    A.bias = net->bias;
    A.tiles_x = (A.w + kNetOutW - 1) / kNetOutW;
    A.tiles = A.tiles_x * ((A.h + kNetOutH - 1) / kNetOutH);
    A.fault = ctx->d_fault;
    const void* fn = pipeline ? (const void*)k_net_infer<true> : (const void*)k_net_infer<false>;
    SVO_CUDA(ctx, cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, kNetSmemBytes));
    const int grid = std::max(1, std::min(A.tiles, ctx->sm_count));
    void* args[] = {&A};
    cudaLaunchConfig_t cfg{};
    cfg.gridDim = dim3((unsigned)grid);
    cfg.blockDim = dim3(kNetThreads);
    cfg.dynamicSmemBytes = kNetSmemBytes;
    cfg.stream = ctx->stream;
    cudaLaunchAttribute attr[1];
    if (pipeline) add_chained(cfg, attr);  // the frame's chain: set-up overlaps k_guide's tail
    SVO_CUDA(ctx, cudaLaunchKernelExC(&cfg, fn, args));
    ++ctx->launches;
    return SVO_OK;
}

// The launch sequence of one learned warp frame after k_set_params:
// reprojection as in the plain frame, then the net (colour for every pixel,
// a ray request for every pixel below the threshold), then the tracer over
// the requests and the refresh tile. Nothing is filtered or copied: the
// current plane keeps reprojected and traced pixels and becomes the cache.
// Guided frames: k_project -> k_guide<true> (the gather, start distances,
// walk lists) -> the net on the listed tiles (it appends its requests) ->
// the tracer (requests, refresh tile, walks); these four launches use
// programmatic stream serialisation, each waiting (griddepcontrol.wait)
// before it reads what the one before wrote.
svo_status enqueue_learned_body(svo_context* ctx, svo_target* t, const svo_net* net, float logit_threshold) {
    cudaStream_t s = ctx->stream;
    const int res_x = t->res_x, res_y = t->res_y;
    record(t, 0);
    {
        const int threads = 256;
        int blocks = (int)std::min<size_t>((t->N + threads - 1) / threads, (size_t)ctx->sm_count * 8);
        cudaLaunchConfig_t cfg{};
        cfg.gridDim = dim3((unsigned)blocks);
        cfg.blockDim = dim3(threads);
        cfg.stream = s;
        cudaLaunchAttribute attr[1];
        add_chained(cfg, attr);
        SVO_CUDA(ctx, cudaLaunchKernelEx(&cfg, k_project, (const FrameParams*)t->d_params, t->B));
        SVO_LAUNCHED(ctx);
    }
    record(t, 1);
    const bool certified = t->B.guide && t->certify;  // k_guide writes certified pixels' BGRX
    if (certified) {
        if (svo_status gs = readback_guard(t); gs != SVO_OK) return gs;
    }
    const dim3 guide_grid((res_x + kGuideBW - 1) / kGuideBW, (res_y + kGuideBH - 1) / kGuideBH);
    if (guided_resolve(t, true)) {
        // the gather happens inside k_guide; the tracer clears the keys
        cudaLaunchConfig_t cfg{};
        cfg.gridDim = guide_grid;
        cfg.blockDim = dim3(kGuideBW * kGuideBH);
        cfg.stream = s;
        cudaLaunchAttribute attr[1];
        add_chained(cfg, attr);
        SVO_CUDA(ctx, cudaLaunchKernelEx(&cfg, k_guide<true>, (const FrameParams*)t->d_params, t->B));
        SVO_LAUNCHED(ctx);
    } else {
        k_resolve_gather<<<dim3((res_x + 15) / 16, (res_y + 15) / 16), 256, 0, s>>>(t->d_params, t->B);
        SVO_LAUNCHED(ctx);
        if (t->feature_tap) {
            k_net_features<<<dim3((res_x + 31) / 32, (res_y + 7) / 8), 256, 0, s>>>(t->d_params, t->B,
                                                                                   t->feature_tap);
            SVO_LAUNCHED(ctx);
        }
        if (t->B.guide) {
            k_guide<false><<<guide_grid, kGuideBW * kGuideBH, 0, s>>>(t->d_params, t->B);
            SVO_LAUNCHED(ctx);
        }
    }
    record(t, 2);
    if (!certified) {  // the net writes the BGRX of the pixels it fills
        if (svo_status gs = readback_guard(t); gs != SVO_OK) return gs;
    }
    NetInferArgs A{};
    A.P = t->d_params;
    A.B = t->B;
    A.w = res_x;
    A.h = res_y;
    A.logit_threshold = logit_threshold;
    svo_status st = launch_net_infer(ctx, net, true, A);
    if (st != SVO_OK) return st;
    if (!t->B.guide) {  // guided frames' requests are appended by the net kernel itself
        const size_t packets = (size_t)t->B.packets_x * t->B.packets_y;
        const unsigned nb = (unsigned)((packets + kReqBlock - 1) / kReqBlock);
        k_request_scan<<<nb, kReqBlock, 0, s>>>(t->B, t->req_offs, t->req_offs + packets);
        SVO_LAUNCHED(ctx);
        k_request_write<<<nb, kReqBlock, 0, s>>>(t->B, t->req_offs, t->req_offs + packets);
        SVO_LAUNCHED(ctx);
    }
    record(t, 3);
    st = launch_trace_warp(ctx, t, kTraceWarpBgrx, true);
    if (st != SVO_OK) return st;
    record(t, 4);
    return SVO_OK;
}

// Runs one frame: k_set_params then `body`, directly or as a CUDA graph that
// is captured once per configuration and replayed with new parameters.
template <class Body>
svo_status run_frame(svo_context* ctx, svo_target* t, const FrameParams& p, FrameGraph& g, const void* net,
                     float threshold, Body body) {
    cudaStream_t s = ctx->stream;
    if (!t->use_graph) {
        k_set_params<<<1, 1, 0, s>>>(p, t->d_params, t->B.counters);
        SVO_LAUNCHED(ctx);
        return body();
    }
    if (!g.exec || g.profiled != t->profiling || g.net != net || g.threshold != threshold || g.tap != t->feature_tap ||
        g.coarse != t->coarse || g.guided != t->guided || g.readback != t->async_readback ||
        g.config_gen != ctx->config_gen) {
        g.reset();
        const uint64_t l0 = ctx->launches;
        SVO_CUDA(ctx, cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
        t->capturing = true;
        k_set_params<<<1, 1, 0, s>>>(p, t->d_params, t->B.counters);
        svo_status st = body();
        t->capturing = false;
        cudaGraph_t gr = nullptr;
        cudaError_t ce = cudaStreamEndCapture(s, &gr);
        g.launches = ctx->launches - l0 + 1;
        ctx->launches = l0;
        if (st != SVO_OK) {
            if (gr) cudaGraphDestroy(gr);
            return st;
        }
        if (ce != cudaSuccess) return fail(ctx, SVO_ERR_CUDA, std::string("capture: ") + cudaGetErrorString(ce));
        g.graph = gr;
        SVO_CUDA(ctx, cudaGraphInstantiate(&g.exec, gr, 0));
        // Find the k_set_params node (the only root of the graph).
        size_t nroots = 0;
        SVO_CUDA(ctx, cudaGraphGetRootNodes(gr, nullptr, &nroots));
        std::vector<cudaGraphNode_t> roots(nroots);
        SVO_CUDA(ctx, cudaGraphGetRootNodes(gr, roots.data(), &nroots));
        for (auto nd : roots) {
            cudaGraphNodeType ty;
            if (cudaGraphNodeGetType(nd, &ty) == cudaSuccess && ty == cudaGraphNodeTypeKernel) {
                cudaKernelNodeParams kp;
                if (cudaGraphKernelNodeGetParams(nd, &kp) == cudaSuccess && kp.func == (void*)k_set_params)
                    g.params_node = nd;
            }
        }
        if (!g.params_node) return fail(ctx, SVO_ERR_CUDA, "graph: parameter node not found");
        g.profiled = t->profiling;
        g.net = net;
        g.threshold = threshold;
        g.tap = t->feature_tap;
        g.coarse = t->coarse;
        g.guided = t->guided;
        g.readback = t->async_readback;
        g.config_gen = ctx->config_gen;
    }
    cudaKernelNodeParams kp;
    SVO_CUDA(ctx, cudaGraphKernelNodeGetParams(g.params_node, &kp));
    FrameParams pc = p;
    FrameParams* dst = t->d_params;
    uint32_t* cnt = t->B.counters;
    void* args[] = {&pc, &dst, &cnt};
    kp.kernelParams = args;
    kp.extra = nullptr;
    SVO_CUDA(ctx, cudaGraphExecKernelNodeSetParams(g.exec, g.params_node, &kp));
    SVO_CUDA(ctx, cudaGraphLaunch(g.exec, s));
    ctx->launches += g.launches;
    return SVO_OK;
}

svo_status net_reserve(svo_net* net, size_t n) {
    svo_context* ctx = net->ctx;
    if (n > net->cap) {
        cudaFree(net->act);
        cudaFree(net->out);
        cudaFree(net->dout);
        cudaFree(net->g0);
        cudaFree(net->g1);
        net->act = net->out = net->dout = net->g0 = net->g1 = nullptr;
        net->cap = 0;
        SVO_CUDA(ctx, cudaMalloc(&net->act, 48 * n * 4));
        SVO_CUDA(ctx, cudaMalloc(&net->out, 4 * n * 4));
        SVO_CUDA(ctx, cudaMalloc(&net->dout, 4 * n * 4));
        SVO_CUDA(ctx, cudaMalloc(&net->g0, 16 * n * 4));
        SVO_CUDA(ctx, cudaMalloc(&net->g1, 16 * n * 4));
        net->cap = n;
    }
    // weight-gradient partial sums: one row per CTA of the backward kernels
    const size_t need = (size_t)std::max(ctx->sm_count, 1) * (9 * 16 * 16 + 16);
    if (need > net->partial_cap) {
        cudaFree(net->partial);
        net->partial = nullptr;
        net->partial_cap = 0;
        SVO_CUDA(ctx, cudaMalloc(&net->partial, need * 4));
        net->partial_cap = need;
    }
    const size_t lb = (n + 255) / 256;
    if (lb > net->loss_cap) {
        cudaFree(net->loss_partial);
        net->loss_partial = nullptr;
        net->loss_cap = 0;
        SVO_CUDA(ctx, cudaMalloc(&net->loss_partial, lb * 2 * 4));
        net->loss_cap = lb;
    }
    return SVO_OK;
}

svo_status net_prepare(svo_net* net) {
    k_net_prepare<<<(kNetMmaTotal * 256 + 255) / 256, 256, 0, net->ctx->stream>>>(net->params, net->wr, net->packed,
                                                                                   net->bias);
    SVO_LAUNCHED(net->ctx);
    k_net_prepare_bwd<<<(kNetBwdBlocks * 256 + 255) / 256, 256, 0, net->ctx->stream>>>(net->params, net->packed_bwd);
    SVO_LAUNCHED(net->ctx);
    return SVO_OK;
}

// FP32 forward of the four layers into net->act / out.
svo_status net_forward_fp32(svo_net* net, const float* feat, int W, int H, float* out) {
    svo_context* ctx = net->ctx;
    cudaStream_t s = ctx->stream;
    const size_t n = (size_t)W * H;
    const dim3 grid((W + 31) / 32, (H + 7) / 8);
    float* a0 = net->act;
    float* a1 = net->act + 16 * n;
    float* a2 = net->act + 32 * n;
    k_net_conv_fwd<8, 16, true, false><<<grid, 256, 0, s>>>(feat, net->wr + net_w_off(0), net->params + net_b_off(0),
                                                            feat, a0, W, H);
    SVO_LAUNCHED(ctx);
    k_net_conv_fwd<16, 16, false, false><<<grid, 256, 0, s>>>(a0, net->wr + net_w_off(1), net->params + net_b_off(1),
                                                              feat, a1, W, H);
    SVO_LAUNCHED(ctx);
    k_net_conv_fwd<16, 16, false, false><<<grid, 256, 0, s>>>(a1, net->wr + net_w_off(2), net->params + net_b_off(2),
                                                              feat, a2, W, H);
    SVO_LAUNCHED(ctx);
    k_net_conv_fwd<16, 4, false, true><<<grid, 256, 0, s>>>(a2, net->wr + net_w_off(3), net->params + net_b_off(3),
                                                            feat, out, W, H);
    SVO_LAUNCHED(ctx);
    return SVO_OK;
}

// Tensor-core backward of one layer (svo_net_train.cuh), over 62x30-position
// tiles, one CTA per SM: the weight and bias gradient (per-CTA partial sums,
// then reduced in CTA order) and, for layers above the first, the gradient
// of the layer below's pre-activation (the ReLU mask of `a` applied).
template <int CIN, int KIN, bool kFirst>
svo_status net_backward_layer(svo_net* net, const float* a, const float* g, float* g_in, int W, int H, int layer) {
    svo_context* ctx = net->ctx;
    const int tiles_x = (W + kBwdOutW - 1) / kBwdOutW;
    const int tiles = tiles_x * ((H + kBwdOutH - 1) / kBwdOutH);
    const int grid = std::max(1, std::min(tiles, ctx->sm_count));
    {
        NetBwdWeightArgs A{a, g, net->partial, W, H, tiles_x, tiles, ctx->d_fault};
        const void* fn = (const void*)k_net_bwd_weight_tc<CIN, KIN, kFirst>;
        constexpr int smem = BwdWeightLayout<CIN>::kSmem;
        SVO_CUDA(ctx, cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
        void* args[] = {&A};
        SVO_CUDA(ctx, cudaLaunchKernel(fn, dim3((unsigned)grid), dim3(kBwdWThreads), args, smem, ctx->stream));
        ++ctx->launches;
        constexpr int vals = 9 * CIN * KIN + KIN;
        k_net_reduce<<<(vals + 255) / 256, 256, 0, ctx->stream>>>(net->partial, grid, vals,
                                                                   net->grads + net_w_off(layer));
        SVO_LAUNCHED(ctx);
    }
    if (g_in) {
        NetBwdDataArgs D{g, net->packed_bwd + (size_t)(layer - 1) * 9 * 256, a, g_in, W, H, tiles_x, tiles,
                         ctx->d_fault};
        const void* fn = (const void*)k_net_bwd_data_tc<KIN>;
        SVO_CUDA(ctx, cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, kBwdDataSmem));
        void* args[] = {&D};
        SVO_CUDA(ctx, cudaLaunchKernel(fn, dim3((unsigned)grid), dim3(kBwdThreads), args, kBwdDataSmem, ctx->stream));
        ++ctx->launches;
    }
    return SVO_OK;
}

// ------------------------------------------------------- GPU builder --
// Device allocations freed when the builder returns.
struct DevScratch {
    std::vector<void*> ptrs;
    ~DevScratch() {
        for (void* p : ptrs) cudaFree(p);
    }
    void release(const void* p) {
        ptrs.erase(std::remove(ptrs.begin(), ptrs.end(), p), ptrs.end());
    }
    template <class T>
    cudaError_t get(T** p, size_t count) {
        void* q = nullptr;
        cudaError_t e = cudaMalloc(&q, std::max<size_t>(count, 1) * sizeof(T));
        if (e == cudaSuccess) ptrs.push_back(q);
        *p = static_cast<T*>(q);
        return e;
    }
};

// Exclusive prefix sum of n uint32 values (in and out may alias); *total
// (host, optional) receives the sum. Synchronises when total is wanted.
svo_status dev_scan(svo_context* ctx, DevScratch& S, const uint32_t* in, uint32_t* out, size_t n, uint32_t* total) {
    cudaStream_t s = ctx->stream;
    if (n == 0) {
        if (total) *total = 0;
        return SVO_OK;
    }
    uint32_t last_in = 0;  // read before the scan: in and out may alias
    if (total) SVO_CUDA(ctx, cudaMemcpyAsync(&last_in, in + n - 1, 4, cudaMemcpyDeviceToHost, s));
    const size_t tiles = (n + kScanTile - 1) / kScanTile;
    uint32_t* sums = nullptr;
    if (tiles > 1) SVO_CUDA(ctx, S.get(&sums, tiles));
    k_scan_tiles<<<(unsigned)tiles, kScanThreads, 0, s>>>(in, out, n, sums);
    SVO_LAUNCHED(ctx);
    if (tiles > 1) {
        svo_status st = dev_scan(ctx, S, sums, sums, tiles, nullptr);
        if (st != SVO_OK) return st;
        k_scan_add<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(out, n, sums);
        SVO_LAUNCHED(ctx);
    }
    if (total) {
        uint32_t a = 0;
        SVO_CUDA(ctx, cudaMemcpyAsync(&a, out + n - 1, 4, cudaMemcpyDeviceToHost, s));
        SVO_CUDA(ctx, cudaStreamSynchronize(s));
        *total = a + last_in;
    }
    return SVO_OK;
}

struct DevLevel {
    uint64_t* key = nullptr;
    uint32_t* first = nullptr;
    uint32_t* begin = nullptr;  // n+1 entries (levels >= 1)
    uint8_t* mask = nullptr;
    uint32_t* size = nullptr;   // subtree words (heights 2-6)
    uint32_t* st = nullptr;     // subtree start (heights 2-5) / block offset (height 6)
    uint32_t* lr = nullptr;     // block start of the node's block (heights 2-5)
    uint32_t* cnt = nullptr;    // normal subtree node count (heights >= 7)
    uint32_t* ps = nullptr;     // post-order start (heights >= 7)
    size_t n = 0;
};

svo_status alloc(svo_context* ctx, void** p, size_t bytes) {
    SVO_CUDA(ctx, cudaMalloc(p, bytes));
    return SVO_OK;
}

}  // namespace

extern "C" {

svo_status svo_context_create(int device, svo_context** out) {
    if (!out) return SVO_ERR_INVALID_ARGUMENT;
    *out = nullptr;
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess || n == 0) return SVO_ERR_CUDA;
    if (device < 0 || device >= n) return SVO_ERR_INVALID_ARGUMENT;
    auto* ctx = new svo_context;
    ctx->device = device;
    auto cleanup = [&](svo_status s) {
        svo_context_destroy(ctx);
        return s;
    };
    if (cudaSetDevice(device) != cudaSuccess) return cleanup(SVO_ERR_CUDA);
    if (cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking) != cudaSuccess) return cleanup(SVO_ERR_CUDA);
    if (cudaDeviceGetAttribute(&ctx->sm_count, cudaDevAttrMultiProcessorCount, device) != cudaSuccess)
        return cleanup(SVO_ERR_CUDA);
    // [0] fault flags, [1] sink word of the read-bandwidth probe
    if (cudaMalloc(&ctx->d_fault, 2 * sizeof(uint32_t)) != cudaSuccess) return cleanup(SVO_ERR_OUT_OF_MEMORY);
    if (cudaMalloc(&ctx->d_counter, sizeof(uint32_t)) != cudaSuccess) return cleanup(SVO_ERR_OUT_OF_MEMORY);
    for (int i = 0; i < svo_context::kRing; ++i) {
        if (cudaMalloc(&ctx->d_batch[i], sizeof(FullBatch)) != cudaSuccess) return cleanup(SVO_ERR_OUT_OF_MEMORY);
        if (cudaMallocHost(&ctx->h_batch[i], sizeof(FullBatch)) != cudaSuccess) return cleanup(SVO_ERR_OUT_OF_MEMORY);
        if (cudaEventCreateWithFlags(&ctx->batch_done[i], cudaEventDisableTiming) != cudaSuccess)
            return cleanup(SVO_ERR_CUDA);
    }
    if (cudaMemsetAsync(ctx->d_fault, 0, 2 * sizeof(uint32_t), ctx->stream) != cudaSuccess) return cleanup(SVO_ERR_CUDA);
    if (cudaStreamSynchronize(ctx->stream) != cudaSuccess) return cleanup(SVO_ERR_CUDA);
    *out = ctx;
    return SVO_OK;
}

svo_status svo_context_destroy(svo_context* ctx) {
    if (!ctx) return SVO_OK;
    while (!ctx->targets.empty()) svo_target_destroy(ctx->targets.back());
    while (!ctx->nets.empty()) svo_net_destroy(ctx->nets.back());
    cudaSetDevice(ctx->device);
    if (ctx->stream) cudaStreamSynchronize(ctx->stream);
    if (ctx->l2_window > 0) l2_window_release(ctx->device);
    if (ctx->owns_octree && ctx->d_octree) cudaFree(ctx->d_octree);
    if (ctx->d_fault) cudaFree(ctx->d_fault);
    if (ctx->d_counter) cudaFree(ctx->d_counter);
    for (int i = 0; i < svo_context::kRing; ++i) {
        if (ctx->d_batch[i]) cudaFree(ctx->d_batch[i]);
        if (ctx->h_batch[i]) cudaFreeHost(ctx->h_batch[i]);
        if (ctx->batch_done[i]) cudaEventDestroy(ctx->batch_done[i]);
    }
    if (ctx->stream) cudaStreamDestroy(ctx->stream);
    delete ctx;
    return SVO_OK;
}

const char* svo_last_error(const svo_context* ctx) { return ctx ? ctx->err.c_str() : "no context"; }

void* svo_context_stream(svo_context* ctx) { return ctx ? (void*)ctx->stream : nullptr; }

uint64_t svo_launch_count(const svo_context* ctx) { return ctx ? ctx->launches : 0; }

svo_status svo_context_set_option(svo_context* ctx, int option, int64_t value) {
    if (!ctx) return SVO_ERR_INVALID_ARGUMENT;
    ++ctx->config_gen;
    switch (option) {
        case SVO_OPT_STAGE_NODES:
            ctx->stage_normal = value != 0;
            ctx->full_pw_shift = ctx->full_block_pref = ctx->full_stage = -1;  // an explicit choice wins
            return SVO_OK;
        case SVO_OPT_PACKET_WIDTH:
            if (value != 4 && value != 8 && value != 16 && value != 32)
                return fail(ctx, SVO_ERR_INVALID_ARGUMENT, "packet width 4, 8, 16 or 32");
            ctx->pw_shift = value == 4 ? 2 : value == 8 ? 3 : value == 16 ? 4 : 5;
            ctx->full_pw_shift = ctx->full_block_pref = ctx->full_stage = -1;
            return SVO_OK;
        case SVO_OPT_TRACE_BLOCK:
            if (value != 0 && value != 256 && value != 1024)
                return fail(ctx, SVO_ERR_INVALID_ARGUMENT, "trace block 0 (auto), 256 or 1024");
            ctx->block_pref = (int)value;
            ctx->full_pw_shift = ctx->full_block_pref = ctx->full_stage = -1;
            return SVO_OK;
        case SVO_OPT_LEARNED_TRACE_BLOCK:
            if (value != 0 && value != 256 && value != 1024)
                return fail(ctx, SVO_ERR_INVALID_ARGUMENT, "learned trace block 0 (auto), 256 or 1024");
            ctx->learned_block_pref = (int)value;
            return SVO_OK;
        case SVO_OPT_LEARNED_PACKET_WIDTH:
            if (value != 0 && value != 4 && value != 8 && value != 16 && value != 32)
                return fail(ctx, SVO_ERR_INVALID_ARGUMENT, "learned packet width 0 (as the others), 4, 8, 16 or 32");
            ctx->learned_pw_shift = value == 0 ? -1 : value == 4 ? 2 : value == 8 ? 3 : value == 16 ? 4 : 5;
            return SVO_OK;
        default:
            return fail(ctx, SVO_ERR_INVALID_ARGUMENT, "unknown option");
    }
}

// Read-bandwidth probe (the L2 roofline's denominator): every block sums
// 16-byte loads over the buffer in a grid-stride loop, `passes` times, with
// L1-bypassing loads, so a buffer that fits in L2 but not in the SMs' L1s is
// read from L2 on every pass. One word per block keeps the loads live.
__global__ void __launch_bounds__(512) k_read_probe(const uint4* __restrict__ p, size_t n16, int passes,
                                                    uint32_t* __restrict__ sink) {
    uint32_t acc = 0;
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    for (int r = 0; r < passes; ++r) {
        size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
        for (; i + 3 * stride < n16; i += 4 * stride) {  // four loads in flight per thread
            const uint4 a = __ldcg(p + i), b = __ldcg(p + i + stride), c = __ldcg(p + i + 2 * stride),
                        d = __ldcg(p + i + 3 * stride);
            acc += a.x ^ b.y ^ c.z ^ d.w;
        }
        for (; i < n16; i += stride) acc += __ldcg(p + i).x;
    }
    acc = __reduce_xor_sync(0xffffffffu, acc);
    if ((threadIdx.x & 31) == 0 && acc == 0x9e3779b9u) atomicAdd(sink, 1u);  // almost never stores
}

svo_status svo_measure_read_bandwidth(svo_context* ctx, const void* d_buf, size_t bytes, int passes, double* gbs) {
    if (!ctx || !d_buf || !gbs || bytes < 16 || passes < 1 || (reinterpret_cast<uintptr_t>(d_buf) & 15u))
        return SVO_ERR_INVALID_ARGUMENT;
    const int sms = ctx->sm_count;
    struct Events {  // released on every return path
        cudaEvent_t e[2] = {nullptr, nullptr};
        ~Events() {
            for (cudaEvent_t x : e)
                if (x) cudaEventDestroy(x);
        }
    } ev;
    SVO_CUDA(ctx, cudaEventCreate(&ev.e[0]));
    SVO_CUDA(ctx, cudaEventCreate(&ev.e[1]));
    cudaEvent_t e0 = ev.e[0], e1 = ev.e[1];
    const size_t n16 = bytes / 16;
    const dim3 grid((unsigned)(sms * 4)), block(512);
    // one untimed launch warms the buffer into L2 (when it fits there)
    k_read_probe<<<grid, block, 0, ctx->stream>>>(static_cast<const uint4*>(d_buf), n16, 1, ctx->d_fault + 1);
    SVO_LAUNCHED(ctx);
    SVO_CUDA(ctx, cudaEventRecord(e0, ctx->stream));
    k_read_probe<<<grid, block, 0, ctx->stream>>>(static_cast<const uint4*>(d_buf), n16, passes, ctx->d_fault + 1);
    SVO_LAUNCHED(ctx);
    SVO_CUDA(ctx, cudaEventRecord(e1, ctx->stream));
    svo_status st = SVO_OK;
    if (cudaEventSynchronize(e1) != cudaSuccess) st = fail(ctx, SVO_ERR_CUDA, "read probe");
    float ms = 0.0f;
    if (st == SVO_OK && cudaEventElapsedTime(&ms, e0, e1) != cudaSuccess) st = fail(ctx, SVO_ERR_CUDA, "read probe events");
    if (st == SVO_OK) *gbs = (double)(n16 * 16) * passes / ((double)ms * 1e-3) / 1e9;
    return st;
}

svo_status svo_synchronize(svo_context* ctx) {
    if (!ctx) return SVO_ERR_INVALID_ARGUMENT;
    SVO_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    uint32_t f = 0;
    SVO_CUDA(ctx, cudaMemcpy(&f, ctx->d_fault, sizeof(f), cudaMemcpyDeviceToHost));
    if (f) {
        SVO_CUDA(ctx, cudaMemset(ctx->d_fault, 0, sizeof(uint32_t)));
        char buf[160];
        std::snprintf(buf, sizeof(buf), "fault flags 0x%x (1: node fetch out of range, 2: ray step limit, "
                      "4: hole entry outside the frame, 8: node staging copy timed out)", f);
        return fail(ctx, SVO_ERR_DEVICE_FAULT, buf);
    }
    return SVO_OK;
}

svo_status svo_octree_upload(svo_context* ctx, const uint32_t* words, size_t n_words, uint32_t root_word, int depth,
                             int validate) {
    if (!ctx || !words || n_words < 10 || n_words >= 0xffffffc0ull) return SVO_ERR_INVALID_ARGUMENT;
    if (depth < SVO_MIN_DEPTH || depth > SVO_MAX_DEPTH) return fail(ctx, SVO_ERR_INVALID_ARGUMENT, "depth");
    if (validate) {
        Validator v{words, n_words, depth, 0, n_words + 16, ""};
        if (!v.normal(root_word, depth)) return fail(ctx, SVO_ERR_BAD_OCTREE, v.why);
    }
    SVO_CUDA(ctx, cudaSetDevice(ctx->device));
    SVO_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    if (ctx->owns_octree && ctx->d_octree) cudaFree(ctx->d_octree);
    ctx->d_octree = nullptr;
    ctx->owns_octree = false;
    void* p = nullptr;
    SVO_CUDA(ctx, cudaMalloc(&p, n_words * 4));
    ctx->d_octree = (uint32_t*)p;
    ctx->owns_octree = true;
    SVO_CUDA(ctx, cudaMemcpyAsync(p, words, n_words * 4, cudaMemcpyHostToDevice, ctx->stream));
    SVO_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    ctx->n_words = n_words;
    ctx->root = root_word;
    ctx->depth = depth;
    // Keep the node words resident in L2 across frames (persisting window over
    // the whole array, clamped to what the device allows).
    return svo_octree_set_l2_window(ctx, ctx->l2_window_request);
}

// ------------------------------------------------------- GPU builder --
svo_status svo_octree_build(svo_context* ctx, const uint32_t* d_x, const uint32_t* d_y, const uint32_t* d_z,
                            const uint32_t* d_rgba, size_t n, int depth, size_t initial_words) {
    if (!ctx || (n && (!d_x || !d_y || !d_z || !d_rgba))) return SVO_ERR_INVALID_ARGUMENT;
    if (depth < SVO_MIN_DEPTH || depth > SVO_MAX_DEPTH) return fail(ctx, SVO_ERR_INVALID_ARGUMENT, "depth");
    if (initial_words == 0) initial_words = SVO_DEFAULT_INITIAL_WORDS;
    if (initial_words < 10 || initial_words >= (1ull << 31)) return fail(ctx, SVO_ERR_INVALID_ARGUMENT, "initial_words");
    SVO_CUDA(ctx, cudaSetDevice(ctx->device));
    cudaStream_t s = ctx->stream;
    const int sms = ctx->sm_count;
    DevScratch S;
    uint32_t* words = nullptr;
    size_t total_words = initial_words;
    uint32_t root = 0;
    if (n == 0) {
        // empty scene: an all-zero root node with no children
        SVO_CUDA(ctx, S.get(&words, initial_words));
        SVO_CUDA(ctx, cudaMemsetAsync(words, 0, initial_words * 4, s));
    } else {
        int ib = 1;
        while (ib < 40 && ((n - 1) >> ib) != 0) ++ib;
        const int key_bits = 3 * depth + ib;
        if (key_bits > 64 || n >= 0xffffffffull)
            return fail(ctx, SVO_ERR_CAPACITY, "too many voxels for 64-bit sort keys at this depth");
        uint32_t* bad = nullptr;
        SVO_CUDA(ctx, S.get(&bad, 4));
        SVO_CUDA(ctx, cudaMemsetAsync(bad, 0, 16, s));
        // ---- keys and sort
        uint64_t *ka = nullptr, *kb = nullptr;
        SVO_CUDA(ctx, S.get(&ka, n));
        SVO_CUDA(ctx, S.get(&kb, n));
        k_bld_keys<<<grid_for(n, 256, sms), 256, 0, s>>>(d_x, d_y, d_z, n, depth, ib, ka, bad);
        SVO_LAUNCHED(ctx);
        const uint32_t nblocks = (uint32_t)((n + kSortTile - 1) / kSortTile);
        uint32_t* counts = nullptr;
        SVO_CUDA(ctx, S.get(&counts, (size_t)256 * nblocks));
        for (int shift = 0; shift < key_bits; shift += 8) {
            k_sort_hist<<<nblocks, kSortThreads, 0, s>>>(ka, n, shift, counts, nblocks);
            SVO_LAUNCHED(ctx);
            svo_status st = dev_scan(ctx, S, counts, counts, (size_t)256 * nblocks, nullptr);
            if (st != SVO_OK) return st;
            k_sort_scatter<<<nblocks, kSortThreads, 0, s>>>(ka, kb, n, shift, counts, nblocks);
            SVO_LAUNCHED(ctx);
            std::swap(ka, kb);
        }
        // ---- levels
        std::vector<DevLevel> L(depth + 1);
        uint32_t *flags = nullptr, *pos = nullptr;
        SVO_CUDA(ctx, S.get(&flags, n));
        SVO_CUDA(ctx, S.get(&pos, n));
        uint32_t* leaf = nullptr;
        {
            k_bld_flags<<<grid_for(n, 256, sms), 256, 0, s>>>(ka, n, ib, flags);
            SVO_LAUNCHED(ctx);
            uint32_t n0 = 0;
            svo_status st = dev_scan(ctx, S, flags, pos, n, &n0);
            if (st != SVO_OK) return st;
            DevLevel& l0 = L[0];
            l0.n = n0;
            SVO_CUDA(ctx, S.get(&l0.key, n0));
            SVO_CUDA(ctx, S.get(&l0.first, n0));
            SVO_CUDA(ctx, S.get(&l0.begin, n0 + 1));
            SVO_CUDA(ctx, S.get(&leaf, n0));
            k_bld_level0<<<grid_for(n, 256, sms), 256, 0, s>>>(ka, n, ib, flags, pos, d_rgba, l0.key, l0.first,
                                                                l0.begin, leaf);
            SVO_LAUNCHED(ctx);
        }
        for (int h = 1; h <= depth; ++h) {
            const DevLevel& c = L[h - 1];
            DevLevel& l = L[h];
            const size_t m = c.n;
            k_bld_flags<<<grid_for(m, 256, sms), 256, 0, s>>>(c.key, m, 3, flags);
            SVO_LAUNCHED(ctx);
            uint32_t np = 0;
            svo_status st = dev_scan(ctx, S, flags, pos, m, &np);
            if (st != SVO_OK) return st;
            l.n = np;
            SVO_CUDA(ctx, S.get(&l.key, np));
            SVO_CUDA(ctx, S.get(&l.first, np));
            SVO_CUDA(ctx, S.get(&l.begin, np + 1));
            SVO_CUDA(ctx, S.get(&l.mask, np));
            k_bld_parents<<<grid_for(m, 256, sms), 256, 0, s>>>(c.key, m, flags, pos, l.key, l.begin);
            SVO_LAUNCHED(ctx);
            const uint32_t mm = (uint32_t)m;
            SVO_CUDA(ctx, cudaMemcpyAsync(l.begin + np, &mm, 4, cudaMemcpyHostToDevice, s));
            k_bld_reduce<<<grid_for(np, 256, sms), 256, 0, s>>>(c.key, c.first, np, l.begin, l.mask, l.first);
            SVO_LAUNCHED(ctx);
            SVO_CUDA(ctx, cudaStreamSynchronize(s));  // mm lives on this frame
        }
        if (L[depth].n != 1) return fail(ctx, SVO_ERR_CUDA, "builder: root level is not a single node");
        // ---- block sizes (heights 2..6) and block offsets
        for (int h = 2; h <= 6; ++h) {
            DevLevel& l = L[h];
            SVO_CUDA(ctx, S.get(&l.size, l.n));
            if (h == 2)
                k_bld_size2<<<grid_for(l.n, 256, sms), 256, 0, s>>>(l.n, l.begin, L[1].begin, leaf, l.size);
            else
                k_bld_size_up<<<grid_for(l.n, 256, sms), 256, 0, s>>>(l.n, l.begin, L[h - 1].size, l.size);
            SVO_LAUNCHED(ctx);
        }
        DevLevel& l6 = L[6];
        SVO_CUDA(ctx, S.get(&l6.st, l6.n));
        k_bld_round64<<<grid_for(l6.n, 256, sms), 256, 0, s>>>(l6.n, l6.size, l6.st);
        SVO_LAUNCHED(ctx);
        uint32_t blocks_total = 0;
        svo_status st = dev_scan(ctx, S, l6.st, l6.st, l6.n, &blocks_total);
        if (st != SVO_OK) return st;
        uint32_t last_off = 0, last_size = 0;
        SVO_CUDA(ctx, cudaMemcpyAsync(&last_off, l6.st + l6.n - 1, 4, cudaMemcpyDeviceToHost, s));
        SVO_CUDA(ctx, cudaMemcpyAsync(&last_size, l6.size + l6.n - 1, 4, cudaMemcpyDeviceToHost, s));
        SVO_CUDA(ctx, cudaStreamSynchronize(s));
        const uint64_t base = (initial_words + 63) / 64 * 64;
        total_words = (size_t)(base + last_off + last_size);
        uint64_t n_normal = 0;
        for (int h = 7; h <= depth; ++h) n_normal += L[h].n;
        if (10 * n_normal > initial_words)
            return fail(ctx, SVO_ERR_CAPACITY, "normal nodes do not fit into initial_words (10 words each)");
        if (total_words >= 0xffffffc0ull || (base >> 6) + ((uint64_t)last_off >> 6) >= (1ull << 23))
            return fail(ctx, SVO_ERR_CAPACITY, "octree exceeds the compact format's 23-bit offsets");
        SVO_CUDA(ctx, S.get(&words, total_words));
        SVO_CUDA(ctx, cudaMemsetAsync(words, 0, total_words * 4, s));
        // ---- blocks, top-down
        for (int h = 5; h >= 2; --h) {
            SVO_CUDA(ctx, S.get(&L[h].st, L[h].n));
            SVO_CUDA(ctx, S.get(&L[h].lr, L[h].n));
        }
        for (int h = 6; h >= 3; --h) {
            DevLevel& l = L[h];
            DevLevel& c = L[h - 1];
            BlockLevel bl{l.begin, l.mask, l.first, l.size}, bc{c.begin, c.mask, c.first, c.size};
            if (h == 6)
                k_bld_emit_block<true><<<grid_for(l.n, 128, sms), 128, 0, s>>>(
                    l.n, bl, bc, false, d_rgba, l.st, nullptr, (uint32_t)base, c.st, c.lr, words, total_words, bad);
            else
                k_bld_emit_block<false><<<grid_for(l.n, 128, sms), 128, 0, s>>>(
                    l.n, bl, bc, h == 3, d_rgba, l.st, l.lr, (uint32_t)base, c.st, c.lr, words, total_words, bad);
            SVO_LAUNCHED(ctx);
        }
        {
            DevLevel& l2 = L[2];
            BlockLevel b2{l2.begin, l2.mask, l2.first, l2.size};
            k_bld_emit_h2<<<grid_for(l2.n, 128, sms), 128, 0, s>>>(l2.n, b2, L[1].begin, L[1].mask, leaf, d_rgba,
                                                                  l2.st, words, total_words, bad);
            SVO_LAUNCHED(ctx);
        }
        // ---- normal nodes
        for (int h = 7; h <= depth; ++h) {
            DevLevel& l = L[h];
            SVO_CUDA(ctx, S.get(&l.cnt, l.n));
            SVO_CUDA(ctx, S.get(&l.ps, l.n));
            k_bld_count_up<<<grid_for(l.n, 256, sms), 256, 0, s>>>(l.n, l.begin, h == 7 ? nullptr : L[h - 1].cnt,
                                                                  l.cnt);
            SVO_LAUNCHED(ctx);
        }
        SVO_CUDA(ctx, cudaMemsetAsync(L[depth].ps, 0, 4, s));
        for (int h = depth; h >= 7; --h) {
            DevLevel& l = L[h];
            DevLevel& c = L[h - 1];
            k_bld_emit_normal<<<grid_for(l.n, 128, sms), 128, 0, s>>>(
                l.n, h, depth, l.begin, l.mask, l.first, l.cnt, l.ps, c.key, c.mask, h - 1 >= 7 ? c.cnt : nullptr,
                h - 1 >= 7 ? c.ps : nullptr, h - 1 == 6 ? c.st : nullptr, (uint32_t)base, d_rgba, words, total_words,
                bad);
            SVO_LAUNCHED(ctx);
        }
        uint8_t root_mask = 0;
        uint32_t flags_host = 0;
        SVO_CUDA(ctx, cudaMemcpyAsync(&root_mask, L[depth].mask, 1, cudaMemcpyDeviceToHost, s));
        SVO_CUDA(ctx, cudaMemcpyAsync(&flags_host, bad, 4, cudaMemcpyDeviceToHost, s));
        SVO_CUDA(ctx, cudaStreamSynchronize(s));
        if (flags_host) {
            if (flags_host & 1u) return fail(ctx, SVO_ERR_INVALID_ARGUMENT, "voxel coordinate outside the volume");
            if (flags_host & 4u) return fail(ctx, SVO_ERR_CUDA, "builder: store outside the word array");
            return fail(ctx, SVO_ERR_CAPACITY, "octree exceeds the compact format's 23-bit offsets");
        }
        root = ((uint32_t)(10 * (n_normal - 1)) << 9) | root_mask;
    }
    SVO_CUDA(ctx, cudaStreamSynchronize(s));
    S.release(words);  // the words outlive the scratch: they become the context's octree
    if (ctx->owns_octree && ctx->d_octree) cudaFree(ctx->d_octree);
    ctx->d_octree = words;
    ctx->owns_octree = true;
    ctx->n_words = total_words;
    ctx->root = root;
    ctx->depth = depth;
    return svo_octree_set_l2_window(ctx, ctx->l2_window_request);
}

svo_status svo_octree_info(const svo_context* ctx, size_t* n_words, uint32_t* root_word, int* depth) {
    if (!ctx || !ctx->d_octree) return SVO_ERR_NO_OCTREE;
    if (n_words) *n_words = ctx->n_words;
    if (root_word) *root_word = ctx->root;
    if (depth) *depth = ctx->depth;
    return SVO_OK;
}

svo_status svo_octree_download(svo_context* ctx, uint32_t* host, size_t n_words) {
    if (!ctx || !host) return SVO_ERR_INVALID_ARGUMENT;
    if (!ctx->d_octree) return fail(ctx, SVO_ERR_NO_OCTREE, "no octree");
    if (n_words != ctx->n_words) return fail(ctx, SVO_ERR_INVALID_ARGUMENT, "n_words differs from the octree's");
    SVO_CUDA(ctx, cudaMemcpyAsync(host, ctx->d_octree, n_words * 4, cudaMemcpyDeviceToHost, ctx->stream));
    SVO_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return SVO_OK;
}

svo_status svo_octree_upload_device(svo_context* ctx, const uint32_t* d_words, size_t n_words, uint32_t root_word,
                                    int depth) {
    if (!ctx || !d_words || n_words < 10 || n_words >= 0xffffffc0ull) return SVO_ERR_INVALID_ARGUMENT;
    if (depth < SVO_MIN_DEPTH || depth > SVO_MAX_DEPTH) return fail(ctx, SVO_ERR_INVALID_ARGUMENT, "depth");
    SVO_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    if (ctx->owns_octree && ctx->d_octree) cudaFree(ctx->d_octree);
    ctx->d_octree = const_cast<uint32_t*>(d_words);
    ctx->owns_octree = false;
    ctx->n_words = n_words;
    ctx->root = root_word;
    ctx->depth = depth;
    return svo_octree_set_l2_window(ctx, ctx->l2_window_request);
}

svo_status svo_octree_set_l2_window(svo_context* ctx, size_t bytes) {
    if (!ctx) return SVO_ERR_INVALID_ARGUMENT;
    ctx->l2_window_request = bytes;
    if (!ctx->d_octree) return SVO_OK;  // applied at the next upload
    cudaStreamAttrValue attr;
    std::memset(&attr, 0, sizeof(attr));
    int max_window = 0, max_persist = 0;
    SVO_CUDA(ctx, cudaDeviceGetAttribute(&max_window, cudaDevAttrMaxAccessPolicyWindowSize, ctx->device));
    SVO_CUDA(ctx, cudaDeviceGetAttribute(&max_persist, cudaDevAttrMaxPersistingL2CacheSize, ctx->device));
    if (max_window <= 0 || max_persist <= 0) bytes = 0;  // no persisting L2 on this device
    if (bytes > 0) {
        bytes = std::min(bytes, std::min(ctx->n_words * 4, (size_t)max_window));
        SVO_CUDA(ctx, cudaDeviceSetLimit(cudaLimitPersistingL2CacheSize, std::min(bytes, (size_t)max_persist)));
        attr.accessPolicyWindow.base_ptr = ctx->d_octree;
        attr.accessPolicyWindow.num_bytes = bytes;
        attr.accessPolicyWindow.hitRatio = 1.0f;
        attr.accessPolicyWindow.hitProp = cudaAccessPropertyPersisting;
        attr.accessPolicyWindow.missProp = cudaAccessPropertyStreaming;
    }
    SVO_CUDA(ctx, cudaStreamSetAttribute(ctx->stream, cudaStreamAttributeAccessPolicyWindow, &attr));
    if (bytes > 0 && ctx->l2_window == 0) l2_window_acquire(ctx->device);
    if (bytes == 0 && ctx->l2_window > 0) l2_window_release(ctx->device);
    ctx->l2_window = bytes;
    return SVO_OK;
}

svo_status svo_target_create(svo_context* ctx, int res_x, int res_y, svo_target** out) {
    if (!ctx || !out || res_x < 1 || res_y < 1 || res_x > 65535 || res_y > 65535) return SVO_ERR_INVALID_ARGUMENT;
    *out = nullptr;
    SVO_CUDA(ctx, cudaSetDevice(ctx->device));
    auto* t = new svo_target;
    t->ctx = ctx;
    t->res_x = res_x;
    t->res_y = res_y;
    t->N = (size_t)res_x * res_y;
    t->B.res_x = res_x;
    t->B.res_y = res_y;
    t->B.tiles_x = res_x / 16;
    t->B.tiles_y = res_y / 16;
    t->tiles = (size_t)t->B.tiles_x * t->B.tiles_y;
    const size_t N = t->N;
    svo_status st = SVO_OK;
    auto A = [&](void** p, size_t bytes) {
        if (st == SVO_OK) st = alloc(ctx, p, bytes);
    };
    A((void**)&t->B.col[0], N * 4);
    A((void**)&t->B.col[1], N * 4);
    A((void**)&t->B.col[2], N * 4);
    A((void**)&t->B.xyz[0], N * 16);
    A((void**)&t->B.xyz[1], N * 16);
    A((void**)&t->B.xyz[2], N * 16);
    A((void**)&t->B.disp, N * 4);
    A((void**)&t->B.bgrx, N * 4);
    A((void**)&t->B.keys, N * 8);
    A((void**)&t->B.ids, (N + 2 * t->tiles + 4) * 4);
    A((void**)&t->B.tile_mask, (t->tiles + 1) * 8);
    t->B.packets_x = (res_x + 7) / 8;
    t->B.packets_y = (res_y + 3) / 4;
    const size_t packets = (size_t)t->B.packets_x * t->B.packets_y;
    A((void**)&t->B.req_mask, packets * 4);
    A((void**)&t->req_offs, (packets + (packets + kReqBlock - 1) / kReqBlock) * 4);  // offsets + block totals
    const size_t net_tiles = (size_t)((res_x + kNetOutW - 1) / kNetOutW) * ((res_y + kNetOutH - 1) / kNetOutH);
    A((void**)&t->d_guide, N * 4);
    // guided frames' pixel lists (walks, certified pixels) and certified results
    t->B.walk_cap = (uint32_t)N;
    A((void**)&t->B.walk_list, N * 4 * kWalkBuckets);
    A((void**)&t->B.cert_list, N * 4);
    A((void**)&t->B.cert_col, N * 4);
    A((void**)&t->B.cert_xyz, N * 16);
    A((void**)&t->B.net_flags, net_tiles * 4);
    A((void**)&t->B.net_list, net_tiles * 4);
    A((void**)&t->B.counters, 64);
    A((void**)&t->d_params, sizeof(FrameParams));
    A((void**)&t->full_col, N * 4);
    A((void**)&t->full_xyzw, N * 16);
    A((void**)&t->full_vox, N * 8);
    if (st != SVO_OK) {
        svo_target_destroy(t);
        return st;
    }
    cudaStream_t s = ctx->stream;
    SVO_CUDA(ctx, cudaMemsetAsync(t->B.keys, 0xff, N * 8, s));
    SVO_CUDA(ctx, cudaMemsetAsync(t->B.col[0], 0xff, N * 4, s));
    SVO_CUDA(ctx, cudaMemsetAsync(t->B.col[1], 0xff, N * 4, s));
    SVO_CUDA(ctx, cudaMemsetAsync(t->B.col[2], 0xff, N * 4, s));
    SVO_CUDA(ctx, cudaMemsetAsync(t->B.xyz[0], 0, N * 16, s));
    SVO_CUDA(ctx, cudaMemsetAsync(t->B.xyz[1], 0, N * 16, s));
    SVO_CUDA(ctx, cudaMemsetAsync(t->B.xyz[2], 0, N * 16, s));
    SVO_CUDA(ctx, cudaMemsetAsync(t->B.ids, 0, (N + 2 * t->tiles + 4) * 4, s));
    SVO_CUDA(ctx, cudaMemsetAsync(t->B.tile_mask, 0, (t->tiles + 1) * 8, s));
    SVO_CUDA(ctx, cudaMemsetAsync(t->B.req_mask, 0, packets * 4, s));
    SVO_CUDA(ctx, cudaMemsetAsync(t->B.net_flags, 0, net_tiles * 4, s));
    SVO_CUDA(ctx, cudaMemsetAsync(t->B.counters, 0, 64, s));
    SVO_CUDA(ctx, cudaMemsetAsync(t->B.bgrx, 0, N * 4, s));
    SVO_CUDA(ctx, cudaMemsetAsync(t->B.disp, 0xff, N * 4, s));
    for (auto& e : t->ev) SVO_CUDA(ctx, cudaEventCreate(&e));
    SVO_CUDA(ctx, cudaStreamSynchronize(s));
    ctx->targets.push_back(t);
    *out = t;
    return SVO_OK;
}

svo_status svo_target_destroy(svo_target* t) {
    if (!t) return SVO_OK;
    svo_context* ctx = t->ctx;
    cudaSetDevice(ctx->device);
    cudaStreamSynchronize(ctx->stream);
    if (t->copy_stream) {
        cudaStreamSynchronize(t->copy_stream);
        cudaStreamDestroy(t->copy_stream);
    }
    if (t->frame_done) cudaEventDestroy(t->frame_done);
    if (t->copy_done) cudaEventDestroy(t->copy_done);
    for (auto& g : t->graphs) g.reset();
    void* ptrs[] = {t->B.col[0], t->B.col[1], t->B.col[2], t->B.xyz[0], t->B.xyz[1], t->B.xyz[2], t->B.disp, t->B.bgrx, t->B.keys, t->B.ids,
                    t->B.tile_mask, t->B.counters, t->d_params, t->full_col, t->full_xyzw, t->full_vox,
                    t->B.req_mask, t->req_offs, t->d_guide, t->B.net_flags, t->B.net_list, t->B.walk_list,
                    t->B.cert_list, t->B.cert_col, t->B.cert_xyz};
    for (void* p : ptrs)
        if (p) cudaFree(p);
    for (auto& e : t->ev)
        if (e) cudaEventDestroy(e);
    auto it = std::find(ctx->targets.begin(), ctx->targets.end(), t);
    if (it != ctx->targets.end()) ctx->targets.erase(it);
    delete t;
    return SVO_OK;
}

svo_status svo_target_use_graph(svo_target* t, int enable) {
    if (!t) return SVO_ERR_INVALID_ARGUMENT;
    t->use_graph = enable != 0;
    if (!t->use_graph)
        for (auto& g : t->graphs) g.reset();
    return SVO_OK;
}

svo_status svo_target_set_profiling(svo_target* t, int enable) {
    if (!t) return SVO_ERR_INVALID_ARGUMENT;
    t->profiling = enable != 0;
    return SVO_OK;
}

int svo_target_stage_times(svo_target* t, float* ms, int cap) {
    if (!t || !ms || t->n_events < 2) return 0;
    if (cudaEventSynchronize(t->ev[t->n_events - 1]) != cudaSuccess) return 0;
    int k = 0;
    if (t->last_mode == 1 || t->last_mode == 3) {
        const int stages = t->last_mode == 1 ? 6 : 4;
        for (int i = 0; i < stages && i < cap; ++i, ++k) {
            float v = 0;
            cudaEventElapsedTime(&v, t->ev[i], t->ev[i + 1]);
            ms[i] = v;
        }
    } else {
        for (int i = 0; i < cap && i < 6; ++i) ms[i] = 0.0f;
        if (cap > 4) cudaEventElapsedTime(&ms[4], t->ev[0], t->ev[1]);
        k = std::min(cap, 6);
    }
    return k;
}

// Largest packet count of one trace launch: the warps' work counter runs past
// the total by at most one increment per resident warp before they stop, and
// must not wrap around 2^32.
constexpr uint64_t kMaxBatchPackets = 0xFF000000ull;

static svo_status check_view(svo_context* ctx, const svo_target* t, const svo_view* v) {
    if (!v) return fail(ctx, SVO_ERR_INVALID_ARGUMENT, "null view");
    if (v->res_x != t->res_x || v->res_y != t->res_y) return fail(ctx, SVO_ERR_INVALID_ARGUMENT, "view resolution differs from the target");
    if (!ctx->d_octree) return fail(ctx, SVO_ERR_NO_OCTREE, "upload an octree first");
    return SVO_OK;
}

svo_status svo_raycast_full_batch(svo_context* ctx, svo_target* const* targets, const svo_view* views, int n) {
    if (!ctx || !targets || !views || n < 1 || n > kMaxBatchViews) return SVO_ERR_INVALID_ARGUMENT;
    if (!ctx->d_octree) return fail(ctx, SVO_ERR_NO_OCTREE, "upload an octree first");
    for (int i = 0; i < n; ++i) {
        if (!targets[i] || targets[i]->ctx != ctx) return fail(ctx, SVO_ERR_INVALID_ARGUMENT, "target");
        svo_status s = check_view(ctx, targets[i], &views[i]);
        if (s != SVO_OK) return s;
    }
    const int slot = ctx->batch_slot;
    ctx->batch_slot = (slot + 1) % svo_context::kRing;
    // The slot's previous copy must have left the staging buffer.
    SVO_CUDA(ctx, cudaEventSynchronize(ctx->batch_done[slot]));
    {  // the packet numbers of the whole batch must fit the 32-bit work counter
        const int pw = 1 << full_pw_shift(ctx), ph = 32 >> full_pw_shift(ctx);
        uint64_t total = 0;
        for (int i = 0; i < n; ++i)
            total += (uint64_t)((views[i].res_x + pw - 1) / pw) * (uint64_t)((views[i].res_y + ph - 1) / ph);
        if (total > kMaxBatchPackets) return fail(ctx, SVO_ERR_INVALID_ARGUMENT, "batch has too many ray packets");
    }
    FullBatch* hb = ctx->h_batch[slot];
    hb->n_views = n;
    uint32_t packets = 0;
    for (int i = 0; i < n; ++i) {
        FullView& fv = hb->v[i];
        const svo_view& v = views[i];
        fv.ray = make_raycam(v);
        fv.res_x = v.res_x;
        fv.res_y = v.res_y;
        const int pw = 1 << full_pw_shift(ctx), ph = 32 >> full_pw_shift(ctx);
        fv.pw_shift = full_pw_shift(ctx);
        fv.packets_x = (v.res_x + pw - 1) / pw;
        fv.packet_begin = packets;
        packets += (uint32_t)fv.packets_x * (uint32_t)((v.res_y + ph - 1) / ph);
        fv.col = targets[i]->full_col;
        fv.xyzw = targets[i]->full_xyzw;
        fv.vox = targets[i]->full_vox;
        fv.bgrx = targets[i]->B.bgrx;
    }
    hb->total_packets = packets;
    const size_t bytes = offsetof(FullBatch, v) + sizeof(FullView) * n;
    svo_target* t0 = targets[0];
    if (t0->profiling) {
        cudaEventRecord(t0->ev[0], ctx->stream);
    }
    SVO_CUDA(ctx, cudaMemcpyAsync(ctx->d_batch[slot], hb, bytes, cudaMemcpyHostToDevice, ctx->stream));
    for (int i = 0; i < n; ++i)
        if (svo_status gs = readback_guard(targets[i]); gs != SVO_OK) return gs;
    k_reset_counter<<<1, 1, 0, ctx->stream>>>(ctx->d_counter);
    SVO_LAUNCHED(ctx);
    svo_status st = launch_trace_full(ctx, ctx->d_batch[slot]);
    SVO_CUDA(ctx, cudaEventRecord(ctx->batch_done[slot], ctx->stream));
    if (st != SVO_OK) return st;
    if (t0->profiling) {
        cudaEventRecord(t0->ev[1], ctx->stream);
        t0->n_events = 2;
        t0->last_mode = 2;
    }
    return SVO_OK;
}

svo_status svo_raycast_full(svo_context* ctx, svo_target* t, const svo_view* view) {
    if (!ctx || !t) return SVO_ERR_INVALID_ARGUMENT;
    return svo_raycast_full_batch(ctx, &t, view, 1);
}

// The autotuners measure the default packet shape (8x4) first and move to
// another configuration only when it is faster by more than this margin:
// configurations within the timing noise of each other keep the default.
constexpr float kTuneMargin = 0.99f;

svo_status svo_context_autotune(svo_context* ctx, svo_target* t, const svo_view* view, int repeats,
                                svo_tune_result* results, int cap, int* n_results) {
    if (!ctx || !t || !view || repeats < 1) return SVO_ERR_INVALID_ARGUMENT;
    svo_status st = check_view(ctx, t, view);
    if (st != SVO_OK) return st;
    struct Cfg {
        int pw, block, stage;
    };
    std::vector<Cfg> cfgs;
    for (int pw : {8, 4, 16, 32})
        for (int stage : {1, 0})
            for (int block : {256, 1024}) cfgs.push_back({pw, block, stage});
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    SVO_CUDA(ctx, cudaEventCreate(&e0));
    SVO_CUDA(ctx, cudaEventCreate(&e1));
    // The candidates and the choice are full-raycast overrides: warp frames
    // keep the options' configuration.
    const int fpw0 = ctx->full_pw_shift, fblock0 = ctx->full_block_pref, fstage0 = ctx->full_stage;
    float best = 1e30f;
    Cfg best_cfg{-1, -1, -1};
    int k = 0;
    for (const Cfg& c : cfgs) {
        ctx->full_pw_shift = c.pw == 4 ? 2 : c.pw == 8 ? 3 : c.pw == 16 ? 4 : 5;
        ctx->full_block_pref = c.block;
        ctx->full_stage = c.stage;
        st = svo_raycast_full(ctx, t, view);  // warm-up
        float ms = 0.0f;
        if (st == SVO_OK && cudaEventRecord(e0, ctx->stream) == cudaSuccess) {
            for (int r = 0; r < repeats && st == SVO_OK; ++r) st = svo_raycast_full(ctx, t, view);
            if (st == SVO_OK && cudaEventRecord(e1, ctx->stream) == cudaSuccess &&
                cudaEventSynchronize(e1) == cudaSuccess && cudaEventElapsedTime(&ms, e0, e1) == cudaSuccess)
                ms /= (float)repeats;
            else if (st == SVO_OK)
                st = fail(ctx, SVO_ERR_CUDA, "autotune timing");
        }
        if (st != SVO_OK) break;
        if (results && k < cap) results[k] = svo_tune_result{c.pw, 32 / c.pw, c.block, c.stage, ms};
        ++k;
        if (ms < best * kTuneMargin) {
            best = ms;
            best_cfg = c;
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (best_cfg.pw > 0) {
        ctx->full_pw_shift = best_cfg.pw == 4 ? 2 : best_cfg.pw == 8 ? 3 : best_cfg.pw == 16 ? 4 : 5;
        ctx->full_block_pref = best_cfg.block;
        ctx->full_stage = best_cfg.stage;
    } else {  // nothing measured: keep what was there
        ctx->full_pw_shift = fpw0;
        ctx->full_block_pref = fblock0;
        ctx->full_stage = fstage0;
    }
    ++ctx->config_gen;
    if (n_results) *n_results = k;
    return st;
}

svo_status svo_context_autotune_learned(svo_context* ctx, svo_target* t, const svo_view* views, int n_views,
                                        const svo_net* net, float threshold, svo_tune_result* results, int cap,
                                        int* n_results) {
    if (!ctx || !t || !views || !net || t->ctx != ctx || net->ctx != ctx || n_views < 6)
        return SVO_ERR_INVALID_ARGUMENT;
    const int pw0 = ctx->learned_pw_shift, block0 = ctx->learned_block_pref;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    SVO_CUDA(ctx, cudaEventCreate(&e0));
    SVO_CUDA(ctx, cudaEventCreate(&e1));
    const int skip = 4;  // frames 0-1 have no cache; two more to settle the cache
    svo_status st = SVO_OK;
    float best = 1e30f;
    int best_pw = pw0, best_block = block0, k = 0;
    for (int pw : {8, 4, 16, 32})
        for (int block : {256, 1024}) {
            ctx->learned_pw_shift = pw == 4 ? 2 : pw == 8 ? 3 : pw == 16 ? 4 : 5;
            ctx->learned_block_pref = block;
            ++ctx->config_gen;
            float ms = 0.0f;
            for (int f = 0; f < n_views && st == SVO_OK; ++f) {
                if (f == skip && cudaEventRecord(e0, ctx->stream) != cudaSuccess)
                    st = fail(ctx, SVO_ERR_CUDA, "autotune timing");
                if (st == SVO_OK) st = svo_warp_frame_learned(ctx, t, &views[f], f, net, threshold);
            }
            if (st == SVO_OK) {
                if (cudaEventRecord(e1, ctx->stream) == cudaSuccess && cudaEventSynchronize(e1) == cudaSuccess &&
                    cudaEventElapsedTime(&ms, e0, e1) == cudaSuccess)
                    ms /= (float)(n_views - skip);
                else
                    st = fail(ctx, SVO_ERR_CUDA, "autotune timing");
            }
            if (st != SVO_OK) break;
            if (results && k < cap) results[k] = svo_tune_result{pw, 32 / pw, block, ctx->stage_normal ? 1 : 0, ms};
            ++k;
            if (ms < best * kTuneMargin) {
                best = ms;
                best_pw = ctx->learned_pw_shift;
                best_block = block;
            }
        }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    ctx->learned_pw_shift = best_pw;
    ctx->learned_block_pref = best_block;
    ++ctx->config_gen;
    if (n_results) *n_results = k;
    return st;
}

svo_status svo_warp_frame(svo_context* ctx, svo_target* t, const svo_view* view, int frame) {
    if (!ctx || !t || t->ctx != ctx) return SVO_ERR_INVALID_ARGUMENT;
    svo_status st = check_view(ctx, t, view);
    if (st != SVO_OK) return st;
    if (t->res_x < 16 || t->res_y < 16)
        return fail(ctx, SVO_ERR_INVALID_ARGUMENT, "warp frames need res >= 16 (the reference's 16x16 hole tiles)");
    if (view->fovx != 1.0f || view->fovy != 1.0f)
        return fail(ctx, SVO_ERR_INVALID_ARGUMENT, "warp frames use fov 1 (raycast_proj has no fov term)");
    if (frame < 0) return fail(ctx, SVO_ERR_INVALID_ARGUMENT, "frame");
    const bool have_cache = frame >= 2 && t->have_prev;
    const PlanePlan q = plan_planes(t, frame, have_cache, t->cache_mode);
    FrameParams p = make_params(t, *view, frame, q, have_cache);
    st = run_frame(ctx, t, p, t->graphs[0], nullptr, 0.0f, [&] { return enqueue_warp_body(ctx, t); });
    if (st != SVO_OK) return st;
    if (t->profiling) {
        t->n_events = 7;
        t->last_mode = 1;
    }
    commit_planes(t, q, *view);
    t->have_prev = true;
    t->prev_view = *view;
    t->have_prev_view = true;
    ++t->frames;
    return SVO_OK;
}

svo_status svo_warp_frame_learned(svo_context* ctx, svo_target* t, const svo_view* view, int frame, const svo_net* net,
                                  float threshold) {
    if (!ctx || !t || t->ctx != ctx || !net || net->ctx != ctx) return SVO_ERR_INVALID_ARGUMENT;
    svo_status st = check_view(ctx, t, view);
    if (st != SVO_OK) return st;
    if (t->res_x < 16 || t->res_y < 16)
        return fail(ctx, SVO_ERR_INVALID_ARGUMENT, "warp frames need res >= 16 (the reference's 16x16 hole tiles)");
    if (view->fovx != 1.0f || view->fovy != 1.0f)
        return fail(ctx, SVO_ERR_INVALID_ARGUMENT, "warp frames use fov 1 (raycast_proj has no fov term)");
    if (frame < 0) return fail(ctx, SVO_ERR_INVALID_ARGUMENT, "frame");
    if (!(threshold > 0.0f && threshold < 1.0f)) return fail(ctx, SVO_ERR_INVALID_ARGUMENT, "threshold in (0, 1)");
    const float logit = std::log(threshold / (1.0f - threshold));
    const bool have_cache = frame >= 2 && t->have_prev;
    // learned frames keep one cache plane (the current plane of the last frame)
    const PlanePlan q = plan_planes(t, frame, have_cache, 0);
    FrameParams p = make_params(t, *view, frame, q, have_cache, true);
    st = run_frame(ctx, t, p, t->graphs[1], net, threshold, [&] { return enqueue_learned_body(ctx, t, net, logit); });
    if (st != SVO_OK) return st;
    if (t->profiling) {
        t->n_events = 5;
        t->last_mode = 3;
    }
    commit_planes(t, q, *view);
    t->have_prev = true;
    t->prev_view = *view;
    t->have_prev_view = true;
    ++t->frames;
    return SVO_OK;
}

svo_status svo_target_set_feature_tap(svo_target* t, float* d_features) {
    if (!t) return SVO_ERR_INVALID_ARGUMENT;
    t->feature_tap = d_features;
    return SVO_OK;
}

svo_status svo_read_requested(svo_target* t, uint32_t* count) {
    if (!t || !count) return SVO_ERR_INVALID_ARGUMENT;
    svo_context* ctx = t->ctx;
    SVO_CUDA(ctx, cudaMemcpyAsync(count, t->B.counters + 1, 4, cudaMemcpyDeviceToHost, ctx->stream));
    SVO_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return SVO_OK;
}

// ------------------------------------------------------------------ net --
// Runs k_net_probe once per device; the verdict is cached for the process.
static std::mutex g_probe_mutex;
static int g_probe_state[64] = {};  // 0 not run, 1 passed, 2 failed

static svo_status net_probe(svo_context* ctx) {
    std::lock_guard<std::mutex> lock(g_probe_mutex);
    const int d = ctx->device;
    if (d >= 0 && d < 64 && g_probe_state[d] == 1) return SVO_OK;
    if (d >= 0 && d < 64 && g_probe_state[d] == 2)
        return fail(ctx, SVO_ERR_NOT_SUPPORTED, "tensor-core operand layout check failed earlier on this device");
    uint32_t* dres = nullptr;
    SVO_CUDA(ctx, cudaMalloc(&dres, 8));
    uint32_t res[2] = {0, 0};
    cudaError_t e = cudaMemsetAsync(dres, 0, 8, ctx->stream);
    if (e == cudaSuccess) e = cudaFuncSetAttribute((const void*)k_net_probe, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                   kNetProbeSmem);
    if (e == cudaSuccess) {
        k_net_probe<<<1, 128, kNetProbeSmem, ctx->stream>>>(dres);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(res, dres, 8, cudaMemcpyDeviceToHost, ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    cudaFree(dres);
    if (e != cudaSuccess) return fail(ctx, SVO_ERR_CUDA, std::string("net probe: ") + cudaGetErrorString(e));
    ++ctx->launches;
    const bool ok = res[0] == 0 && res[1] == 0;
    if (d >= 0 && d < 64) g_probe_state[d] = ok ? 1 : 2;
    if (!ok) {
        char buf[128];
        std::snprintf(buf, sizeof(buf), "tensor-core operand layout check failed (%u mismatches, timeout %u)", res[0],
                      res[1]);
        return fail(ctx, SVO_ERR_NOT_SUPPORTED, buf);
    }
    return SVO_OK;
}

svo_status svo_net_create(svo_context* ctx, svo_net** out) {
    if (!ctx || !out) return SVO_ERR_INVALID_ARGUMENT;
    *out = nullptr;
    SVO_CUDA(ctx, cudaSetDevice(ctx->device));
    {
        const svo_status ps = net_probe(ctx);
        if (ps != SVO_OK) return ps;
    }
    auto* net = new svo_net;
    net->ctx = ctx;
    svo_status st = SVO_OK;
    auto A = [&](void** p, size_t bytes) {
        if (st == SVO_OK) st = alloc(ctx, p, bytes);
    };
    A((void**)&net->params, kNetParams * 4);
    A((void**)&net->m, kNetParams * 4);
    A((void**)&net->v, kNetParams * 4);
    A((void**)&net->grads, kNetParams * 4);
    A((void**)&net->wr, kNetParams * 4);
    A((void**)&net->packed, kNetMmaTotal * 512);
    A((void**)&net->packed_bwd, kNetBwdBlocks * 512);
    A((void**)&net->bias, 64 * 4);
    if (st != SVO_OK) {
        svo_net_destroy(net);
        return st;
    }
    ctx->nets.push_back(net);
    *out = net;
    return svo_net_init(net, 1);
}

svo_status svo_net_destroy(svo_net* net) {
    if (!net) return SVO_OK;
    cudaSetDevice(net->ctx->device);
    cudaStreamSynchronize(net->ctx->stream);
    void* ptrs[] = {net->params, net->m, net->v, net->grads, net->wr, net->packed, net->packed_bwd, net->bias, net->act,
                    net->out, net->dout, net->g0, net->g1, net->partial, net->loss_partial};
    for (void* q : ptrs)
        if (q) cudaFree(q);
    auto& v = net->ctx->nets;
    auto it = std::find(v.begin(), v.end(), net);
    if (it != v.end()) v.erase(it);
    delete net;
    return SVO_OK;
}

svo_status svo_net_set_params(svo_net* net, const float* host, size_t n) {
    if (!net || !host) return SVO_ERR_INVALID_ARGUMENT;
    svo_context* ctx = net->ctx;
    if (n != (size_t)kNetParams) return fail(ctx, SVO_ERR_INVALID_ARGUMENT, "parameter count");
    for (size_t i = 0; i < n; ++i)
        if (!std::isfinite(host[i])) return fail(ctx, SVO_ERR_INVALID_ARGUMENT, "non-finite parameter");
    SVO_CUDA(ctx, cudaMemcpyAsync(net->params, host, n * 4, cudaMemcpyHostToDevice, ctx->stream));
    SVO_CUDA(ctx, cudaMemsetAsync(net->m, 0, n * 4, ctx->stream));
    SVO_CUDA(ctx, cudaMemsetAsync(net->v, 0, n * 4, ctx->stream));
    SVO_CUDA(ctx, cudaMemsetAsync(net->grads, 0, n * 4, ctx->stream));
    net->step = 0;
    svo_status st = net_prepare(net);
    if (st != SVO_OK) return st;
    SVO_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return SVO_OK;
}

// He-normal weights (seeded splitmix64 + Box-Muller), the confidence output's
// weights scaled by 0.1, the colour outputs' weights zero (the net starts as
// the identity on colour), zero biases.
svo_status svo_net_init(svo_net* net, uint64_t seed) {
    if (!net) return SVO_ERR_INVALID_ARGUMENT;
    std::vector<float> p(kNetParams, 0.0f);
    uint64_t state = seed * 0x9E3779B97F4A7C15ull + 0x1234567ull;
    auto next = [&]() {
        uint64_t z = (state += 0x9E3779B97F4A7C15ull);
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        z ^= z >> 31;
        return ((z >> 11) + 0.5) * (1.0 / 9007199254740992.0);
    };
    for (int l = 0; l < kNetLayers; ++l) {
        const double sd = std::sqrt(2.0 / (9.0 * net_cin(l))) * (l == kNetLayers - 1 ? 0.1 : 1.0);
        for (int i = 0; i < 9 * net_cin(l) * net_cout(l); ++i) {
            const double u1 = next(), u2 = next();
            const double w = sd * std::sqrt(-2.0 * std::log(u1)) * std::cos(6.283185307179586 * u2);
            // the colour outputs start as the identity (residual weights 0)
            const bool colour_out = l == kNetLayers - 1 && i % net_cout(l) < 3;
            p[net_w_off(l) + i] = colour_out ? 0.0f : (float)w;
        }
    }
    return svo_net_set_params(net, p.data(), p.size());
}

static svo_status net_copy_out(svo_net* net, const float* dev, float* host, size_t n) {
    svo_context* ctx = net->ctx;
    if (!host) return fail(ctx, SVO_ERR_INVALID_ARGUMENT, "null host buffer");
    if (n != (size_t)kNetParams) return fail(ctx, SVO_ERR_INVALID_ARGUMENT, "parameter count");
    SVO_CUDA(ctx, cudaMemcpyAsync(host, dev, n * 4, cudaMemcpyDeviceToHost, ctx->stream));
    SVO_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return SVO_OK;
}

svo_status svo_net_get_params(svo_net* net, float* host, size_t n) {
    return net ? net_copy_out(net, net->params, host, n) : SVO_ERR_INVALID_ARGUMENT;
}

svo_status svo_net_get_grads(svo_net* net, float* host, size_t n) {
    return net ? net_copy_out(net, net->grads, host, n) : SVO_ERR_INVALID_ARGUMENT;
}

svo_status svo_net_forward(svo_net* net, const float* d_features, int w, int h, float* d_out) {
    if (!net || !d_features || !d_out || w < 1 || h < 1) return SVO_ERR_INVALID_ARGUMENT;
    svo_status st = net_reserve(net, (size_t)w * h);
    if (st != SVO_OK) return st;
    return net_forward_fp32(net, d_features, w, h, d_out);
}

svo_status svo_net_infer(svo_net* net, const float* d_features, int w, int h, float* d_out) {
    if (!net || !d_features || !d_out || w < 1 || h < 1) return SVO_ERR_INVALID_ARGUMENT;
    NetInferArgs A{};
    A.feat = d_features;
    A.out = d_out;
    A.w = w;
    A.h = h;
    return launch_net_infer(net->ctx, net, false, A);
}

svo_status svo_net_backward(svo_net* net, const float* d_features, const uint32_t* d_target_bgrx, int w, int h,
                            float tau, float lambda, float* loss) {
    if (!net || !d_features || !d_target_bgrx || w < 1 || h < 1) return SVO_ERR_INVALID_ARGUMENT;
    svo_context* ctx = net->ctx;
    cudaStream_t s = ctx->stream;
    const size_t n = (size_t)w * h;
    svo_status st = net_reserve(net, n);
    if (st != SVO_OK) return st;
    {  // the forward pass on the tensor cores, keeping the hidden activations
        NetInferArgs A{};
        A.feat = d_features;
        A.out = net->out;
        A.act = net->act;
        A.w = w;
        A.h = h;
        st = launch_net_infer(ctx, net, false, A);
        if (st != SVO_OK) return st;
    }
    const int lb = (int)((n + 255) / 256);
    k_net_loss<<<lb, 256, 0, s>>>(net->out, d_target_bgrx, net->dout, net->loss_partial, (int)n, tau, lambda);
    SVO_LAUNCHED(ctx);
    float* a0 = net->act;
    float* a1 = net->act + 16 * n;
    float* a2 = net->act + 32 * n;
    // layer 3 (4 outputs) .. layer 0 (the features as input, no data gradient)
    st = net_backward_layer<16, 4, false>(net, a2, net->dout, net->g0, w, h, 3);
    if (st == SVO_OK) st = net_backward_layer<16, 16, false>(net, a1, net->g0, net->g1, w, h, 2);
    if (st == SVO_OK) st = net_backward_layer<16, 16, false>(net, a0, net->g1, net->g0, w, h, 1);
    if (st == SVO_OK) st = net_backward_layer<8, 16, true>(net, d_features, net->g0, nullptr, w, h, 0);
    if (st != SVO_OK) return st;
    if (loss) {
        std::vector<float> part(2 * (size_t)lb);
        SVO_CUDA(ctx, cudaMemcpyAsync(part.data(), net->loss_partial, part.size() * 4, cudaMemcpyDeviceToHost, s));
        SVO_CUDA(ctx, cudaStreamSynchronize(s));
        double a = 0.0, c = 0.0;
        for (int i = 0; i < lb; ++i) {
            a += part[2 * i];
            c += part[2 * i + 1];
        }
        loss[0] = (float)(a / (double)n);
        loss[1] = (float)(c / (double)n);
    }
    return SVO_OK;
}

svo_status svo_net_adam(svo_net* net, float lr, float beta1, float beta2, float eps) {
    if (!net || !(lr >= 0.0f) || !(beta1 >= 0.0f && beta1 < 1.0f) || !(beta2 >= 0.0f && beta2 < 1.0f) || !(eps > 0.0f))
        return SVO_ERR_INVALID_ARGUMENT;
    svo_context* ctx = net->ctx;
    ++net->step;
    const float c1 = (float)(1.0 - std::pow((double)beta1, net->step));
    const float c2 = (float)(1.0 - std::pow((double)beta2, net->step));
    k_net_adam<<<(kNetParams + 255) / 256, 256, 0, ctx->stream>>>(net->params, net->m, net->v, net->grads, kNetParams,
                                                                  lr, beta1, beta2, eps, c1, c2);
    SVO_LAUNCHED(ctx);
    return net_prepare(net);
}

static svo_status read_back(svo_target* t, void* host, const void* dev, size_t bytes) {
    svo_context* ctx = t->ctx;
    if (!host) return fail(ctx, SVO_ERR_INVALID_ARGUMENT, "null host buffer");
    SVO_CUDA(ctx, cudaMemcpyAsync(host, dev, bytes, cudaMemcpyDeviceToHost, ctx->stream));
    SVO_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return SVO_OK;
}

svo_status svo_read_colour(svo_target* t, int plane, uint32_t* host) {
    if (!t) return SVO_ERR_INVALID_ARGUMENT;
    if (plane == 0) return read_back(t, host, t->B.disp, t->N * 4);
    if (plane == 1 || plane == 2) {
        const int phys = plane == t->last_target ? t->last_cur : t->other;
        if (phys >= 0) return read_back(t, host, t->B.col[phys], t->N * 4);
        if (!host) return SVO_ERR_INVALID_ARGUMENT;
        for (size_t i = 0; i < t->N; ++i) host[i] = SVO_EMPTY_PIXEL;
        return SVO_OK;
    }
    return fail(t->ctx, SVO_ERR_INVALID_ARGUMENT, "plane");
}

svo_status svo_read_coords(svo_target* t, int plane, float* host) {
    if (!t) return SVO_ERR_INVALID_ARGUMENT;
    if (plane == 0) return read_back(t, host, t->B.xyz[t->last_cur], t->N * 16);
    if (plane == 1 || plane == 2) {
        const int phys = plane == t->last_target ? t->last_cur : t->other;
        if (phys >= 0) return read_back(t, host, t->B.xyz[phys], t->N * 16);
        if (!host) return SVO_ERR_INVALID_ARGUMENT;
        for (size_t i = 0; i < 4 * t->N; ++i) host[i] = 0.0f;
        return SVO_OK;
    }
    return fail(t->ctx, SVO_ERR_INVALID_ARGUMENT, "plane");
}

svo_status svo_target_set_cache_mode(svo_target* t, int mode) {
    if (!t || mode < 0 || mode > 1) return SVO_ERR_INVALID_ARGUMENT;
    t->cache_mode = mode;
    return SVO_OK;
}

svo_status svo_target_set_guided(svo_target* t, int enable) {
    if (!t) return SVO_ERR_INVALID_ARGUMENT;
    t->guided = enable != 0;
    t->B.guide = t->guided ? t->d_guide : nullptr;
    return SVO_OK;
}

svo_status svo_target_set_certified(svo_target* t, int enable) {
    if (!t) return SVO_ERR_INVALID_ARGUMENT;
    t->certify = enable != 0;
    return SVO_OK;
}

svo_status svo_read_guide(svo_target* t, float* host) {
    if (!t || !host) return SVO_ERR_INVALID_ARGUMENT;
    return read_back(t, host, t->d_guide, t->N * 4);
}

svo_status svo_target_set_coarse_refresh(svo_target* t, int enable) {
    if (!t) return SVO_ERR_INVALID_ARGUMENT;
    if (enable && (t->res_x % 4 || t->res_y % 4))
        return fail(t->ctx, SVO_ERR_NOT_SUPPORTED, "the coarse refresh pass needs res_x and res_y multiples of 4");
    t->coarse = enable != 0;
    return SVO_OK;
}

svo_status svo_read_holes(svo_target* t, uint32_t* host, size_t cap_words, uint32_t* count) {
    if (!t || !host) return SVO_ERR_INVALID_ARGUMENT;
    uint32_t total = 0;
    svo_status st = read_back(t, &total, t->B.counters + 1, 4);
    if (st != SVO_OK) return st;
    const size_t words = 2 * t->tiles + total;
    if (count) *count = total;
    if (cap_words < words) return fail(t->ctx, SVO_ERR_INVALID_ARGUMENT, "hole buffer too small");
    return read_back(t, host, t->B.ids, words * 4);
}

svo_status svo_read_bgrx(svo_target* t, uint32_t* host) {
    if (!t) return SVO_ERR_INVALID_ARGUMENT;
    return read_back(t, host, t->B.bgrx, t->N * 4);
}

svo_status svo_read_bgrx_async(svo_target* t, uint32_t* host) {
    if (!t || !host) return SVO_ERR_INVALID_ARGUMENT;
    svo_context* ctx = t->ctx;
    SVO_CUDA(ctx, cudaSetDevice(ctx->device));
    if (!t->copy_stream) SVO_CUDA(ctx, cudaStreamCreateWithFlags(&t->copy_stream, cudaStreamNonBlocking));
    if (!t->frame_done) SVO_CUDA(ctx, cudaEventCreateWithFlags(&t->frame_done, cudaEventDisableTiming));
    if (!t->copy_done) SVO_CUDA(ctx, cudaEventCreateWithFlags(&t->copy_done, cudaEventDisableTiming));
    // the next frame's graph gains the wait on this copy (captured once)
    t->async_readback = true;
    SVO_CUDA(ctx, cudaEventRecord(t->frame_done, ctx->stream));
    SVO_CUDA(ctx, cudaStreamWaitEvent(t->copy_stream, t->frame_done, 0));
    SVO_CUDA(ctx, cudaMemcpyAsync(host, t->B.bgrx, t->N * 4, cudaMemcpyDeviceToHost, t->copy_stream));
    SVO_CUDA(ctx, cudaEventRecord(t->copy_done, t->copy_stream));
    return SVO_OK;
}

svo_status svo_target_readback_wait(svo_target* t) {
    if (!t) return SVO_ERR_INVALID_ARGUMENT;
    if (t->copy_done) SVO_CUDA(t->ctx, cudaEventSynchronize(t->copy_done));
    return SVO_OK;
}

svo_status svo_read_full(svo_target* t, uint32_t* colour, float* xyzw) {
    if (!t) return SVO_ERR_INVALID_ARGUMENT;
    svo_status st = SVO_OK;
    if (colour) st = read_back(t, colour, t->full_col, t->N * 4);
    if (st == SVO_OK && xyzw) st = read_back(t, xyzw, t->full_xyzw, t->N * 16);
    return st;
}

svo_status svo_read_voxels(svo_target* t, uint64_t* host) {
    if (!t) return SVO_ERR_INVALID_ARGUMENT;
    return read_back(t, host, t->full_vox, t->N * 8);
}

svo_status svo_target_device_outputs(svo_target* t, svo_device_outputs* out) {
    if (!t || !out) return SVO_ERR_INVALID_ARGUMENT;
    out->bgrx = t->B.bgrx;
    out->colour = t->B.disp;
    out->full_colour = t->full_col;
    out->full_xyzw = (float*)t->full_xyzw;
    out->full_voxel = t->full_vox;
    return SVO_OK;
}

}  // extern "C"

// ======================================================================
// A full raycast entry point that allocates no memory.
//
// For callers that cannot allocate device memory through this library: host
// engines that hand out all GPU memory from their own allocator or pool, code
// paths that run after start-up in a no-allocation frame budget, and plugins
// that may not create a context or grow its footprint. The caller passes the
// octree words and every output buffer; the only memory the call needs
// besides them -- the trace kernel's work-queue counter, its fault flags and
// the table of views -- lives in the file-scope array below, which exists
// once per device for as long as the library is loaded.
namespace {

// Layout of the scratch array: the counter and fault word in the first 256
// bytes, then a FullBatch header with room for SVO_NOALLOC_MAX_VIEWS views.
constexpr size_t kNoAllocTableOffset = 256;
constexpr size_t kNoAllocTableBytes = offsetof(FullBatch, v) + sizeof(FullView) * SVO_NOALLOC_MAX_VIEWS;
constexpr size_t kNoAllocScratchBytes = kNoAllocTableOffset + kNoAllocTableBytes;
static_assert(SVO_NOALLOC_MAX_VIEWS <= kMaxBatchViews, "view table larger than the kernel's batch layout");

// Device copy of the scratch. In host code this name is only a stand-in for
// the symbol; its device address comes from cudaGetSymbolAddress.
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

// The device address of a __device__ array belongs to the CUDA context that
// was current when it was looked up; a host that makes its own driver-API
// context current, or resets the device, gets another one. So the address is
// cached per context, keyed by the context's process-unique id (a handle
// value can be reused after a context is destroyed).
typedef int (*PfnCtxGetCurrent)(void** ctx);
typedef int (*PfnCtxGetId)(void* ctx, unsigned long long* id);
constexpr int kMaxContexts = 64;
struct ScratchEntry {
    unsigned long long ctx_id;
    unsigned char* ptr;
};
std::mutex g_setup_mutex;
ScratchEntry g_scratch[kMaxContexts] = {};
int g_scratch_used = 0, g_scratch_next = 0;
PfnCtxGetCurrent g_ctx_get_current = nullptr;
PfnCtxGetId g_ctx_get_id = nullptr;

// Device address of g_noalloc_scratch in the current context, looked up the
// first time a context calls (with that context current).
svo_status scratch_address(int device, unsigned char** out) {
    std::lock_guard<std::mutex> lock(g_setup_mutex);
    if (!g_ctx_get_current || !g_ctx_get_id) {
        cudaDriverEntryPointQueryResult q1 = cudaDriverEntryPointSymbolNotFound, q2 = q1;
        void* f1 = nullptr;
        void* f2 = nullptr;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f1, 4000, cudaEnableDefault, &q1) != cudaSuccess ||
            cudaGetDriverEntryPointByVersion("cuCtxGetId", &f2, 12000, cudaEnableDefault, &q2) != cudaSuccess ||
            q1 != cudaDriverEntryPointSuccess || q2 != cudaDriverEntryPointSuccess || !f1 || !f2)
            return SVO_ERR_CUDA;
        g_ctx_get_current = reinterpret_cast<PfnCtxGetCurrent>(f1);
        g_ctx_get_id = reinterpret_cast<PfnCtxGetId>(f2);
    }
    void* ctx = nullptr;
    unsigned long long id = 0;
    if (g_ctx_get_current(&ctx) != 0) return SVO_ERR_CUDA;
    if (!ctx) {
        // No context current on this thread yet: bind the device's primary
        // context, the one the runtime would use.
        if (cudaSetDevice(device) != cudaSuccess || g_ctx_get_current(&ctx) != 0) return SVO_ERR_CUDA;
    }
    if (!ctx || g_ctx_get_id(ctx, &id) != 0) return SVO_ERR_CUDA;
    for (int i = 0; i < g_scratch_used; ++i)
        if (g_scratch[i].ctx_id == id) {
            *out = g_scratch[i].ptr;
            return SVO_OK;
        }
    void* p = nullptr;
    if (cudaGetSymbolAddress(&p, g_noalloc_scratch) != cudaSuccess || !p) return SVO_ERR_CUDA;
    const int slot = g_scratch_used < kMaxContexts ? g_scratch_used++ : (g_scratch_next++ % kMaxContexts);
    g_scratch[slot] = ScratchEntry{id, static_cast<unsigned char*>(p)};
    *out = static_cast<unsigned char*>(p);
    return SVO_OK;
}

template <int BLOCK>
const void* noalloc_kernel(int depth) {
    switch (depth) {
        case 8: return (const void*)k_trace_full<8, BLOCK, true>;
        case 9: return (const void*)k_trace_full<9, BLOCK, true>;
        case 10: return (const void*)k_trace_full<10, BLOCK, true>;
        case 11: return (const void*)k_trace_full<11, BLOCK, true>;
        case 12: return (const void*)k_trace_full<12, BLOCK, true>;
    }
    return nullptr;
}

}  // namespace

extern "C" svo_status svo_raycast_full_noalloc(const uint32_t* d_words, size_t n_words, uint32_t root_word, int depth,
                                               const svo_view* views, const svo_frame_buffers* outputs, int n_views,
                                               void* stream) {
    if (!d_words || n_words < 10 || n_words >= 0xffffffc0ull || !views || !outputs || n_views < 1)
        return SVO_ERR_INVALID_ARGUMENT;
    if (depth < SVO_MIN_DEPTH || depth > SVO_MAX_DEPTH) return SVO_ERR_INVALID_ARGUMENT;
    if (n_views > SVO_NOALLOC_MAX_VIEWS) return SVO_ERR_CAPACITY;
    // Every pointer is checked before any CUDA call: the kernel reads the
    // words as uint32 and stores uint32, uint64 and float4 per pixel, so a
    // caller buffer at an offset (a sub-allocation from its own pool) that is
    // not aligned for those would fault the GPU instead of returning an error.
    if (reinterpret_cast<uintptr_t>(d_words) & 3u) return SVO_ERR_INVALID_ARGUMENT;
    uint64_t packets_total = 0;
    for (int i = 0; i < n_views; ++i) {
        const svo_view& v = views[i];
        const svo_frame_buffers& o = outputs[i];
        if (v.res_x < 1 || v.res_y < 1 || v.res_x > 65535 || v.res_y > 65535) return SVO_ERR_INVALID_ARGUMENT;
        if (!o.colour || !o.xyzw || !o.voxel || !o.bgrx) return SVO_ERR_INVALID_ARGUMENT;
        if ((reinterpret_cast<uintptr_t>(o.xyzw) & 15u) || (reinterpret_cast<uintptr_t>(o.voxel) & 7u) ||
            (reinterpret_cast<uintptr_t>(o.colour) & 3u) || (reinterpret_cast<uintptr_t>(o.bgrx) & 3u))
            return SVO_ERR_INVALID_ARGUMENT;
        packets_total += (uint64_t)((v.res_x + 7) / 8) * (uint64_t)((v.res_y + 3) / 4);
    }
    if (packets_total > kMaxBatchPackets) return SVO_ERR_INVALID_ARGUMENT;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    // The call synchronises and reads the fault word back, which no graph can
    // hold: refuse it while the stream is being captured.
    cudaStreamCaptureStatus capture = cudaStreamCaptureStatusNone;
    if (cudaStreamIsCapturing(s, &capture) != cudaSuccess || capture != cudaStreamCaptureStatusNone)
        return SVO_ERR_INVALID_ARGUMENT;
    int device = 0;
    if (cudaGetDevice(&device) != cudaSuccess) return SVO_ERR_CUDA;
    unsigned char* scratch = nullptr;
    svo_status st = scratch_address(device, &scratch);
    if (st != SVO_OK) return st;

    // View table, built on the host stack and copied into the scratch array.
    struct alignas(16) Table {
        unsigned char bytes[kNoAllocTableBytes];
    } table;
    std::memset(&table, 0, sizeof(table));
    FullBatch* hb = reinterpret_cast<FullBatch*>(table.bytes);
    hb->n_views = n_views;
    uint32_t packets = 0;
    for (int i = 0; i < n_views; ++i) {
        const svo_view& v = views[i];
        FullView& fv = hb->v[i];
        fv.ray.px = v.pos[0];
        fv.ray.py = v.pos[1];
        fv.ray.pz = v.pos[2];
        fv.ray.mxx = v.m[0];
        fv.ray.mxy = v.m[4];
        fv.ray.mxz = v.m[8];
        fv.ray.myx = v.m[1];
        fv.ray.myy = v.m[5];
        fv.ray.myz = v.m[9];
        fv.ray.mzx = v.m[2];
        fv.ray.mzy = v.m[6];
        fv.ray.mzz = v.m[10];
        fv.ray.fovx = v.fovx;
        fv.ray.fovy = v.fovy;
        fv.res_x = v.res_x;
        fv.res_y = v.res_y;
        fv.pw_shift = 3;
        fv.packets_x = (v.res_x + 7) / 8;
        fv.packet_begin = packets;
        packets += (uint32_t)fv.packets_x * (uint32_t)((v.res_y + 3) / 4);
        fv.col = outputs[i].colour;
        fv.xyzw = reinterpret_cast<float4*>(outputs[i].xyzw);
        fv.vox = outputs[i].voxel;
        fv.bgrx = outputs[i].bgrx;
    }
    hb->total_packets = packets;

    // Launch geometry as for the context path: stage the normal-node region in
    // shared memory when it fits and the words are 16-byte aligned.
    Octree o{d_words, (uint32_t)n_words, root_word, 0u, 0u};
    uint32_t stage_bytes = 0;
    if (!(root_word & 256u) && (reinterpret_cast<uintptr_t>(d_words) & 15u) == 0) {
        const uint64_t nw = (uint64_t)(root_word >> 9) + 10u;
        const uint64_t bytes = (nw * 4u + 15u) & ~15ull;
        if (bytes <= 160u * 1024u && bytes <= (uint64_t)n_words * 4u) {
            o.n_smem = (uint32_t)nw;
            stage_bytes = (uint32_t)bytes;
        }
    }
    const int block = stage_bytes > 48u * 1024u ? 1024 : 256;
    const void* fn = block == 1024 ? noalloc_kernel<1024>(depth) : noalloc_kernel<256>(depth);
    const size_t smem = (size_t)(depth + 2) * block * 4u + stage_bytes;  // stack: kStackLevels
    if (cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess)
        return SVO_ERR_CUDA;
    int per_sm = 0, sms = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, block, smem) != cudaSuccess) return SVO_ERR_CUDA;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device) != cudaSuccess) return SVO_ERR_CUDA;

    // The counter and the fault word must start at zero on every call.
    uint32_t* counter = reinterpret_cast<uint32_t*>(scratch);
    uint32_t* fault = counter + 1;
    FullBatch* d_batch = reinterpret_cast<FullBatch*>(scratch + kNoAllocTableOffset);
    if (cudaMemsetAsync(scratch, 0, 8, s) != cudaSuccess) return SVO_ERR_CUDA;
    if (cudaMemcpyAsync(d_batch, table.bytes, kNoAllocTableBytes, cudaMemcpyHostToDevice, s) != cudaSuccess)
        return SVO_ERR_CUDA;
    void* args[] = {&o, &d_batch, &counter, &fault};
    if (cudaLaunchKernel(fn, dim3((unsigned)(std::max(1, per_sm) * sms)), dim3((unsigned)block), args, smem, s) !=
        cudaSuccess)
        return SVO_ERR_CUDA;
    if (cudaStreamSynchronize(s) != cudaSuccess) return SVO_ERR_CUDA;
    uint32_t flags = 0;
    if (cudaMemcpy(&flags, fault, sizeof(flags), cudaMemcpyDeviceToHost) != cudaSuccess) return SVO_ERR_CUDA;
    return flags ? SVO_ERR_DEVICE_FAULT : SVO_OK;
}
