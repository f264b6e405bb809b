/*
 * svo_gb300.h -- C ABI of the GB300-native sparse-voxel-octree raycast and
 * image-warp pipeline (libsvo_gb300.so).
 *
 * This ABI replaces the reference's OpenCL wrapper src/ocl.h and the buffer
 * plumbing of its frame driver src/raycast.h (sp4cerat/Sparse-Voxel-Octree-
 * Raycasting). Every entry point names the reference interface it stands in
 * for. Conventions, as in the reference: one context drives one device through
 * one in-order stream and is not re-entrant; the caller owns host memory.
 * Unlike the reference (which stops the process through error_stop on any
 * failure, src/ocl.h:29-41), every call returns an svo_status.
 *
 * Octree words keep the reference's compact node format (src/octree/octree.h:
 * 95-293, kernel/kernel.cl:32-112): (offset<<9)|(isBlock<<8)|childmask8, ten-
 * word normal nodes for the top depth-6 levels and 64-word-aligned byte-packed
 * blocks for the last six.
 */
#ifndef SVO_GB300_H
#define SVO_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum svo_status {
    SVO_OK = 0,
    SVO_ERR_INVALID_ARGUMENT = 1, /* null pointer, bad size or resolution */
    SVO_ERR_CUDA = 2,             /* a CUDA runtime call failed (see svo_last_error) */
    SVO_ERR_NO_OCTREE = 3,        /* raycast before svo_octree_upload */
    SVO_ERR_BAD_OCTREE = 4,       /* upload validation found an out-of-range node word */
    SVO_ERR_DEVICE_FAULT = 5,     /* a kernel flagged an out-of-range fetch or hit its step limit */
    SVO_ERR_OUT_OF_MEMORY = 6,
    SVO_ERR_CAPACITY = 7,         /* more voxels/nodes than the compact format addresses */
    SVO_ERR_NOT_SUPPORTED = 8,
    SVO_ERR_IO = 9
} svo_status;

/* Empty pixel marker of the colour planes (src/raycast.h:153,157). */
#define SVO_EMPTY_PIXEL 0xffffff00u
/* Pre-sized compact array length of octree_init (src/raycast.h:38). */
#define SVO_DEFAULT_INITIAL_WORDS 2097152u
#define SVO_MIN_DEPTH 8
#define SVO_MAX_DEPTH 12

/*
 * One camera. pos is v0 of src/raycast.h:159 in world units (the kernels
 * trace from pos*16). m is the row-major 4x4 view matrix m of
 * src/raycast.h:121-128 (m[r*4+c]); its rows are the vx/vy/vz handed to
 * raycast_proj (src/raycast.h:160-162) and its columns the mx/my/mz handed to
 * raycast_holes/raycast_fine_2 (src/raycast.h:322-325). fovx/fovy are the
 * kernels' fov arguments (kernel/kernel.cl:640-641; the reference passes 1.0).
 */
typedef struct svo_view {
    float pos[4];
    float m[16];
    float fovx;
    float fovy;
    int32_t res_x;
    int32_t res_y;
} svo_view;

typedef struct svo_context svo_context;
typedef struct svo_target svo_target;
typedef struct svo_builder svo_builder;
typedef struct svo_net svo_net;

/* ----------------------------------------------------------- context -- */

/* Replaces ocl_init (src/ocl.h:57-146) and the device half of raycast_init
 * (src/raycast.h:61-91). Creates a stream on `device`. */
svo_status svo_context_create(int device, svo_context** out);
/* Replaces raycast_exit (src/raycast.h:511-517) and ocl_exit (src/ocl.h:168-174).
 * Also destroys every render target and net of the context still alive;
 * their handles are invalid afterwards. */
svo_status svo_context_destroy(svo_context* ctx);
/* Human-readable text of the last failure on this context (never null). */
const char* svo_last_error(const svo_context* ctx);
/* The cudaStream_t all work of this context is ordered on. */
void* svo_context_stream(svo_context* ctx);
/* Replaces ocl_end_all_kernels' wait (src/ocl.h:253-265): blocks until the
 * stream drains and reports device-side fault flags (SVO_ERR_DEVICE_FAULT). */
svo_status svo_synchronize(svo_context* ctx);
/* Number of kernels this context has launched since creation. */
uint64_t svo_launch_count(const svo_context* ctx);

/* Tuning switches of the trace kernels (no counterpart in the reference).
 * SVO_OPT_STAGE_NODES, SVO_OPT_PACKET_WIDTH and SVO_OPT_TRACE_BLOCK configure
 * the tracer of full raycasts and of plain warp frames; svo_context_autotune
 * overrides them for full raycasts only, until one of the three is set again.
 * SVO_OPT_STAGE_NODES: 1 (default) copies the octree's normal-node region into
 * each trace block's shared memory (when it fits, <= 160 KiB); 0 reads every
 * node word from global memory. */
#define SVO_OPT_STAGE_NODES 1
/* SVO_OPT_PACKET_WIDTH: ray packets of the trace kernels are W x (32/W)
 * pixels, W = 4, 8 (default, the reference's 8x4 refresh tiles), 16 or 32. */
#define SVO_OPT_PACKET_WIDTH 2
/* SVO_OPT_TRACE_BLOCK: threads per trace block, 256 or 1024; 0 (default)
 * picks by the size of the staged node region. */
#define SVO_OPT_TRACE_BLOCK 3
/* SVO_OPT_LEARNED_TRACE_BLOCK: the same for the tracer of learned frames
 * (requested rays, refresh tile, guided walks): 0 (default: 256 threads when
 * the staged node region fits one, as for the benchmark's depth-11 octree,
 * where it beat 1024 by 9% on guided frames), 256 or 1024.
 * svo_context_autotune, which times full raycasts, does not change it. */
#define SVO_OPT_LEARNED_TRACE_BLOCK 4
/* SVO_OPT_LEARNED_PACKET_WIDTH: ray packets of learned frames' tracer (and
 * of their guide's long-walk flags): 0 (default: as SVO_OPT_PACKET_WIDTH),
 * 4, 8, 16 or 32. */
#define SVO_OPT_LEARNED_PACKET_WIDTH 5
svo_status svo_context_set_option(svo_context* ctx, int option, int64_t value);

/* Read-bandwidth probe (no reference counterpart; a measurement aid): reads
 * `bytes` of the device buffer d_buf (16-byte aligned) `passes` times on the
 * context's stream with L1-bypassing 16-byte loads, after one untimed pass,
 * and returns the achieved GB/s (device events around the timed launch). A
 * buffer that fits in L2 measures the L2 read bandwidth the trace and warp
 * kernels' rooflines are quoted against. Synchronises the stream. */
svo_status svo_measure_read_bandwidth(svo_context* ctx, const void* d_buf, size_t bytes, int passes, double* gbs);

/* Autotuner (no reference counterpart): times `repeats` full raycasts of
 * `view` into `t` for every packet shape (8x4 first, then 4x8, 16x2,
 * 32x1), block size (256, 1024) and node staging (on, off), keeps the
 * fastest in the context for full raycasts -- a configuration replaces the
 * best one measured before it only when it is more than 1% faster, so
 * near-ties keep the earlier one; warp frames keep the options' settings,
 * which suit their shorter, hole- and tile-bound launches -- and returns
 * every measurement (up to cap) in results. Results are identical under
 * every setting; only the speed differs. Synchronises. */
typedef struct svo_tune_result {
    int packet_w, packet_h, block, stage_nodes;
    float ms;
} svo_tune_result;
svo_status svo_context_autotune(svo_context* ctx, svo_target* t, const svo_view* view, int repeats,
                                svo_tune_result* results, int cap, int* n_results);
/* The same for learned frames' tracer (no reference counterpart): renders
 * the n_views (>= 6) views as learned frames 0..n_views-1 into `t` (with the
 * target's guided setting, the net and threshold given) for every packet
 * shape and block size, times frames 4.. with CUDA events, and keeps the
 * fastest (with the same 1% rule) as SVO_OPT_LEARNED_PACKET_WIDTH /
 * SVO_OPT_LEARNED_TRACE_BLOCK.
 * results[i].ms = milliseconds per frame. Synchronises. */
svo_status svo_context_autotune_learned(svo_context* ctx, svo_target* t, const svo_view* views, int n_views,
                                        const svo_net* net, float threshold, svo_tune_result* results, int cap,
                                        int* n_results);

/* ------------------------------------------------------------ octree -- */

/* The octree builder on the GPU (no reference counterpart on the device; it
 * produces the words of set_voxel + convert_tree_blocks,
 * src/octree/octree.h:32-293, and of svo_builder_finish): voxel arrays in
 * device memory, array order = insertion order (a voxel inserted twice keeps
 * the last colour, inner nodes the colour of the first voxel through them).
 * The result becomes the context's octree. initial_words as in
 * svo_builder_finish (0: SVO_DEFAULT_INITIAL_WORDS); the normal nodes must fit
 * into it. Synchronises the context stream. */
svo_status svo_octree_build(svo_context* ctx, const uint32_t* d_x, const uint32_t* d_y, const uint32_t* d_z,
                            const uint32_t* d_rgba, size_t n, int depth, size_t initial_words);
/* Size, root word and depth of the context's octree. */
svo_status svo_octree_info(const svo_context* ctx, size_t* n_words, uint32_t* root_word, int* depth);
/* Copies the context's octree words (n_words must equal its size) to host. */
svo_status svo_octree_download(svo_context* ctx, uint32_t* host, size_t n_words);

/* Replaces ocl_malloc(size, &octree_array_compact[0]) of src/raycast.h:68
 * together with the octree_root_normal global (src/octree/octree.h:25).
 * Validates every node word reachable from root_word against n_words
 * (SVO_ERR_BAD_OCTREE) unless validate == 0, then copies the words to the
 * device. depth is OCTREE_DEPTH (kernel/kernel.cl:12), SVO_MIN_DEPTH..SVO_MAX_DEPTH. */
svo_status svo_octree_upload(svo_context* ctx, const uint32_t* words, size_t n_words, uint32_t root_word,
                             int depth, int validate);
/* Flat variant: adopts words already resident on this context's device
 * (nothing is copied; the caller keeps the allocation alive until the next
 * upload or destroy). No validation. */
svo_status svo_octree_upload_device(svo_context* ctx, const uint32_t* d_words, size_t n_words, uint32_t root_word,
                                    int depth);
/* Bytes of the octree (from its start: the normal-node region first) kept in
 * an L2 persisting access-policy window on the context stream, so node words
 * stay resident across frames and other traffic. Default: the whole array,
 * clamped to the device's maximum window and set-aside; 0 disables it and
 * releases the set-aside. Applies to the current and later uploads. */
svo_status svo_octree_set_l2_window(svo_context* ctx, size_t bytes);

/* ------------------------------------------------------- render target -- */

/* A render target holds one camera stream's planes: the cache and current
 * colour/coordinate planes of the warp pipeline (mem_screenbuffer and
 * mem_backbuffer, src/raycast.h:82,85), the hole id buffer (:268-270), the
 * displayed colour plane and the BGRX8 image that replaces the PBO
 * (mem_screenbuffer_tex, :88-89). res_x, res_y <= 65535. */
svo_status svo_target_create(svo_context* ctx, int res_x, int res_y, svo_target** out);
/* Destroy a target before its context (svo_context_destroy destroys the
 * targets left over). */
svo_status svo_target_destroy(svo_target* t);

/* ----------------------------------------------------------- frames ---- */

/* Plain full raycast: raycast_fine_2 (kernel/kernel.cl:846-942) over every
 * pixel, then raycast_colorize (:944-974). Writes the target's "full" planes:
 * colour word 0xff000000+colour, float4 (hit xyz in world units, hit
 * distance in world units), packed hit voxel (svo_read_voxels) and BGRX8.
 * Asynchronous on the context stream. */
svo_status svo_raycast_full(svo_context* ctx, svo_target* t, const svo_view* view);

/* Batched full raycast: n views of any resolution (each into its own target)
 * traced by one persistent launch fed by a global work queue. */
svo_status svo_raycast_full_batch(svo_context* ctx, svo_target* const* targets, const svo_view* views, int n);

/* One warped frame: the body of raycast_draw (src/raycast.h:147-441) without
 * the GL blit. frame is the reference's static frame counter (:104): frames
 * 0 and 1 start from cleared caches, frame selects the 8x4 refresh tile.
 * The view must use fovx = fovy = 1 (raycast_proj has no fov term,
 * kernel/kernel.cl:552-553). No host synchronisation inside (the hole count
 * stays on the device). Asynchronous on the context stream. */
svo_status svo_warp_frame(svo_context* ctx, svo_target* t, const svo_view* view, int frame);

/* Which cache plane a warp frame copies its result into (src/raycast.h:394-
 * 405). mode 0 (default): plane 2, as the reference ships it (plane 1 is
 * never written). mode 1: the alternative the reference leaves commented out
 * at raycast.h:395, ((frame>>4)%2)+1 -- the two cache planes alternate every
 * 16 frames, both are reprojected every frame, and rejected source pixels are
 * cleared in their cache plane (kernel/kernel.cl:549-562). Learned frames
 * always use one cache plane. */
svo_status svo_target_set_cache_mode(svo_target* t, int mode);
/* The raycast_fine pass (kernel/kernel.cl:696-843), launched as the block the
 * reference ships disabled at src/raycast.h:235-261: between reprojection and
 * the hole gather, one ray per 2x2 block of a screen quadrant that moves every
 * frame -- the block's first empty pixel, else a frame-dependent one.
 * Requires res_x and res_y multiples of 4. Plain warp frames only. */
svo_status svo_target_set_coarse_refresh(svo_target* t, int enable);

/* Capture the warp frame of this target as a CUDA graph on first use and
 * replay it on later calls (the per-frame parameters are the arguments of
 * the graph's first kernel node, updated before each replay). Plain and
 * learned frames keep one graph each. enable = 0 returns to direct launches. */
svo_status svo_target_use_graph(svo_target* t, int enable);

/* Per-stage CUDA-event timing of the next frames on this target (replaces
 * the timeGetTime stage array of src/raycast.h:164-166,475-492). */
svo_status svo_target_set_profiling(svo_target* t, int enable);
/* Milliseconds of each stage of the last profiled frame. Warp frames fill
 * [0] project, [1] resolve+gather, [2] scan, [3] hole list, [4] trace,
 * [5] filter+colourise; full raycasts fill [4] trace and [5] colourise;
 * learned frames fill [0] project, [1] resolve, [2] net, [3] trace.
 * Synchronises the stream. Returns the number of stages written. */
int svo_target_stage_times(svo_target* t, float* ms, int cap);

/* -------------------------------------------------------- readbacks ---- */
/* All readbacks synchronise the context stream and copy into host memory of
 * res_x*res_y elements (4 floats per pixel for coordinates). */

/* Warp planes. plane 0: displayed colour words after raycast_fillhole2
 * (reference plane 0 at the end of raycast_draw); planes 1 and 2: the
 * reference's cache planes (colour words before the filter; the memcpy target
 * of :394-405 holds this frame's plane 0). With cache mode 0, plane 1 is never
 * written (all SVO_EMPTY_PIXEL). */
svo_status svo_read_colour(svo_target* t, int plane, uint32_t* host);
/* Coordinate (back) buffer of a plane (0: the last frame's plane 0 before
 * the filter, 1 or 2: the cache planes): x,y,z world hit position; w is the
 * view-space depth for reprojected pixels and the ray distance for traced
 * pixels. Only pixels whose colour is not SVO_EMPTY_PIXEL are defined. */
svo_status svo_read_coords(svo_target* t, int plane, float* host);
/* The hole id buffer of the last warp frame in the reference's layout
 * (kernel/kernel.cl:276-340): [0] total entries, [tiles..2*tiles) exclusive
 * offsets, [2*tiles..) packed x|y<<16 entries. *count receives the total. */
svo_status svo_read_holes(svo_target* t, uint32_t* host, size_t cap_words, uint32_t* count);
/* The BGRX8 image of the last frame (warped or full). */
svo_status svo_read_bgrx(svo_target* t, uint32_t* host);
/* Asynchronous BGRX readback (no reference counterpart; replaces the blocking
 * PBO readback of src/raycast.h:425-441 for hosts that pipeline frames):
 * enqueues the copy of the target's last image into `host` (res_x*res_y words;
 * pinned host memory, or the copy is not asynchronous) on the target's own
 * copy stream and returns at once. The next frame renders meanwhile; its first
 * write to the image (the net, the certified pixels, the filter or a full
 * raycast) waits for the copy. `host` must stay valid, and untouched, until
 * svo_target_readback_wait returns. */
svo_status svo_read_bgrx_async(svo_target* t, uint32_t* host);
/* Returns when the target's last asynchronous readback is complete. */
svo_status svo_target_readback_wait(svo_target* t);
/* Outputs of the last svo_raycast_full on this target. */
svo_status svo_read_full(svo_target* t, uint32_t* colour, float* xyzw);
/* Packed hit voxel of the last full raycast: bits 0-15 x, 16-31 y, 32-47 z
 * (voxel coordinates of the hit cell's low corner), 48-55 hit level
 * (1 = leaf), bit 63 set for a hit; 0 for rays that left the volume. */
svo_status svo_read_voxels(svo_target* t, uint64_t* host);

/* Device pointers of the target's outputs, for zero-copy consumers. */
typedef struct svo_device_outputs {
    uint32_t* bgrx;        /* res_x*res_y BGRX8 */
    uint32_t* colour;      /* displayed colour words (warp) */
    uint32_t* full_colour; /* full raycast colour words */
    float* full_xyzw;      /* full raycast float4 */
    uint64_t* full_voxel;  /* full raycast packed hit voxels */
} svo_device_outputs;
svo_status svo_target_device_outputs(svo_target* t, svo_device_outputs* out);

/* ------------------------------------------- learned reconstruction -- */
/* No counterpart in the reference, which fills reprojection holes with a
 * fixed filter (raycast_fillhole2, kernel/kernel.cl:404-470) and traces every
 * 2x2 hole block (raycast_counthole/writeids/holes, :234-340,594-694). A
 * learned frame reprojects like svo_warp_frame, then a small convolutional
 * net (inputs: warped colour, depth, hole mask, reprojection motion; outputs:
 * colour and a confidence) runs on the tensor cores over the whole frame;
 * pixels whose confidence is below `threshold` (0..1, e.g. 0.5) are traced,
 * together with the 8x4 refresh tile, and show the traced colour; the others
 * show the net's colour. The current plane (reprojected + traced pixels)
 * becomes the next frame's cache. Output: the target's BGRX image.
 * Asynchronous on the context stream. */
svo_status svo_warp_frame_learned(svo_context* ctx, svo_target* t, const svo_view* view, int frame,
                                  const svo_net* net, float threshold);
/* Rays the net requested in the target's last learned frame (synchronises). */
svo_status svo_read_requested(svo_target* t, uint32_t* count);
/* Guided learned frames (enable = 1): after reprojection, every pixel with a
 * cached surface point in its 3x3 neighbourhood is walked from just in front
 * of the nearest such point (2 cells of the level of detail at that
 * distance) instead of from the camera -- the same walk, started late, so it
 * finds the same voxel unless a surface the cache never saw lies in front of
 * the start. Only the remaining (unguided) pixels go to the net, which runs
 * on the 56x24 tiles that hold one; those below `threshold` are traced from
 * the camera, as is the refresh tile. Learned frames also re-base cached
 * points across wraps of the camera into the periodic volume
 * (src/raycast.h:136-145). enable = 0: every pixel goes to the net. */
svo_status svo_target_set_guided(svo_target* t, int enable);
/* The start distances of the last guided frame, res_x*res_y floats in raypos
 * units (16 per world unit; 0 = from the camera, -1 = unguided). */
/* Certified reprojection in guided learned frames (no reference counterpart;
 * off by default -- on a GB300 at 1920x1024 it saves 6% of the trace and
 * costs as much in the start-distance kernel): a guided pixel whose own ray provably meets the face a
 * cached hit point of its 3x3 neighbourhood lies on -- the hit codes the
 * learned frames keep in w of the coordinate planes (level | ray signs << 5,
 * -1 without a hit) name the face -- takes that point's colour and needs no
 * walk (start distance -2 in svo_read_guide), unless a cached point lies more
 * than 2 cells in front of the face, a hole is next to it or it is in the
 * refresh tile. enable = 0 walks every guided pixel. */
svo_status svo_target_set_certified(svo_target* t, int enable);
svo_status svo_read_guide(svo_target* t, float* host);
/* Training tap: when d_features is not NULL, every later frame of the target
 * (plain or learned) writes the net's input features after reprojection to
 * this device buffer, planar [8][res_y*res_x] FP32. */
svo_status svo_target_set_feature_tap(svo_target* t, float* d_features);

/* The net's parameters: SVO_NET_PARAMS FP32 values, per layer l = 0..3 the
 * weights [9 taps (dy+1)*3+(dx+1)][c_in][c_out] then the biases [c_out];
 * channels 8 -> 16 -> 16 -> 16 -> 4. */
#define SVO_NET_PARAMS 6388
/* Creates a net on the context, initialised by svo_net_init(net, 1). */
svo_status svo_net_create(svo_context* ctx, svo_net** out);
svo_status svo_net_destroy(svo_net* net);
/* Seeded He-normal weights; the last layer's colour weights zero (the net
 * starts as the identity on colour) and its confidence weights scaled by
 * 0.1; zero biases. Resets the optimiser. */
svo_status svo_net_init(svo_net* net, uint64_t seed);
/* n must be SVO_NET_PARAMS. set_params resets the optimiser. */
svo_status svo_net_set_params(svo_net* net, const float* host, size_t n);
svo_status svo_net_get_params(svo_net* net, float* host, size_t n);
/* Gradient of the last svo_net_backward. */
svo_status svo_net_get_grads(svo_net* net, float* host, size_t n);
/* Forward passes over a planar feature image (device pointers; features
 * [8][h*w], outputs [4][h*w]: R, G, B, confidence logit). svo_net_forward is
 * an FP32 CUDA-core reference; svo_net_infer is the tensor-core kernel of
 * learned frames and of training. */
svo_status svo_net_forward(svo_net* net, const float* d_features, int w, int h, float* d_out);
svo_status svo_net_infer(svo_net* net, const float* d_features, int w, int h, float* d_out);
/* Forward + loss + backward over one frame: the target is a BGRX8 image
 * (device pointer, e.g. the full raycast of the same view). Loss per pixel:
 * mean squared colour error over R, G, B plus lambda * binary cross-entropy
 * of the confidence against "every colour channel within tau". loss (host,
 * may be NULL) receives the two mean terms. Synchronises when loss != NULL.
 * All convolutions run on the tensor cores: the forward pass as in
 * svo_net_infer (keeping the hidden activations), the data and weight
 * gradients as implicit GEMMs with each FP32 gradient split into two bf16
 * parts; FP32 sums. */
svo_status svo_net_backward(svo_net* net, const float* d_features, const uint32_t* d_target_bgrx, int w, int h,
                            float tau, float lambda, float* loss);
/* One Adam step with the last gradient (asynchronous). */
svo_status svo_net_adam(svo_net* net, float lr, float beta1, float beta2, float eps);

/* ----------------------------------------------- allocation-free call -- */
/* No counterpart in the reference. A full raycast (as svo_raycast_full, one
 * or more views) that allocates nothing, for callers that cannot let this
 * library allocate device memory: engines that hand out all GPU memory from
 * their own allocator or pool, frame loops that may not allocate after
 * start-up, plugins that may not create a context or grow its footprint.
 * The caller passes the octree words already on the current device and, per
 * view, device buffers of res_x*res_y elements for every output. The little
 * scratch the trace needs -- work-queue counter, fault flags and the table
 * of views, 7 KiB -- is a static device array that exists once per device
 * while the library is loaded; the views beyond SVO_NOALLOC_MAX_VIEWS do not
 * fit in it and are rejected with SVO_ERR_CAPACITY.
 * Alignment: d_words 4 bytes, colour and bgrx 4, voxel 8, xyzw 16 (one
 * float4 store per pixel); a misaligned pointer, like a null one, is rejected
 * with SVO_ERR_INVALID_ARGUMENT before any CUDA call.
 * The first call in a CUDA context (normally the device's primary context;
 * a context the host made current through the driver API counts as its own)
 * looks up that array's device address in it. The call is synchronous (it
 * waits for its rays and reads the fault word back), so it cannot be
 * captured into a graph: during an active capture of `stream` it returns
 * SVO_ERR_INVALID_ARGUMENT. Every call shares the array (it keeps the last call's
 * contents; the counter and fault flags are cleared at the start of each
 * call), so calls that overlap on the GPU -- from two host threads or on two
 * streams at once -- race; issue them one after another.
 * The call runs on `stream` (null = the default stream) and returns when the
 * rays are written, with SVO_ERR_DEVICE_FAULT if a kernel flagged an
 * out-of-range node word. */
#define SVO_NOALLOC_MAX_VIEWS 64
typedef struct svo_frame_buffers {
    uint32_t* colour; /* 0xff000000 + colour word */
    float* xyzw;      /* 4 floats per pixel: hit xyz, hit distance (world units) */
    uint64_t* voxel;  /* packed hit voxel, as svo_read_voxels */
    uint32_t* bgrx;   /* colourised BGRX8 */
} svo_frame_buffers;
svo_status svo_raycast_full_noalloc(const uint32_t* d_words, size_t n_words, uint32_t root_word, int depth,
                                    const svo_view* views, const svo_frame_buffers* outputs, int n_views,
                                    void* stream);

/* ------------------------------------------------- host octree builder -- */
/* Replaces set_voxel / convert_tree_blocks (src/octree/octree.h:32-89,
 * 232-293) and octree_init (src/raycast.h:13-46). Produces the same compact
 * words as the reference for the same voxels in the same insertion order:
 * a node takes the colour of the first voxel inserted through it, a leaf the
 * colour of the last insertion of that voxel. */
svo_status svo_builder_create(int depth, svo_builder** out);
svo_status svo_builder_destroy(svo_builder* b);
/* set_voxel(x,y,z,uchar4): rgba is the uchar4 colour read as a little-endian
 * word; only its low byte survives at leaf level (octree.h:117-135) and it
 * must be non-zero. */
svo_status svo_builder_set_voxel(svo_builder* b, uint32_t x, uint32_t y, uint32_t z, uint32_t rgba);
svo_status svo_builder_set_voxels(svo_builder* b, const uint32_t* x, const uint32_t* y, const uint32_t* z,
                                  const uint32_t* rgba, size_t n);
/* convert_tree_blocks(octree_root) after octree_array_compact.resize(initial_words)
 * (initial_words 0 means SVO_DEFAULT_INITIAL_WORDS). */
svo_status svo_builder_finish(svo_builder* b, size_t initial_words, uint32_t* root_word, size_t* n_words);
/* Copies the finished words (n_words of svo_builder_finish). */
svo_status svo_builder_copy_words(const svo_builder* b, uint32_t* out);
/* Voxel count (num_voxels, octree.h:27) and pointer-node count of the built tree. */
svo_status svo_builder_stats(const svo_builder* b, uint64_t* voxels, uint64_t* nodes);

/* Flat octree file: magic, depth, root word, word count, words. Lets deep
 * scenes be built once (the reference rebuilds from .rle4 every start). */
svo_status svo_octree_save(const char* path, const uint32_t* words, size_t n_words, uint32_t root_word, int depth);
svo_status svo_octree_load_header(const char* path, size_t* n_words, uint32_t* root_word, int* depth);
svo_status svo_octree_load_words(const char* path, uint32_t* words, size_t n_words);

/* --------------------------------------------------------- .rle4 files -- */
/* The reference's volume loader RLE4::load (src/octree/Rle4.cpp:8-165): the
 * voxels of map 0 of an .rle4 file with the same colour words and the same
 * insertion order (z outer, x inner, top of each column first), offset by
 * (addx, addy, addz). palette selects the material/intensity colour byte
 * (Rle4.cpp:146); 0 is the reference's default (octree_init passes 0).
 * Malformed files fail with SVO_ERR_IO (the reference reads out of bounds). */
svo_status svo_rle4_voxels(const char* path, int palette, uint32_t addx, uint32_t addy, uint32_t addz, uint32_t* x,
                           uint32_t* y, uint32_t* z, uint32_t* rgba, size_t cap, size_t* n);
/* Inserts those voxels into a builder (SVO_ERR_CAPACITY if one falls outside
 * the builder's 2^depth cube). */
svo_status svo_rle4_build(svo_builder* b, const char* path, int palette, uint32_t addx, uint32_t addy, uint32_t addz);

/* 32-bit BMP of a BGRX8 frame, top row first in the frame (replaces the dead
 * frame dump of src/raycast.h:496-509 and Bmp::save, src/Bmp.cpp:30-60, with
 * a complete header). */
svo_status svo_write_bmp(const char* path, const uint32_t* bgrx, int width, int height);

/* --------------------------------------------------- synthetic scenes -- */
/* Seeded value-noise fBm terrain (6 octaves, lacunarity 2, gain 0.5,
 * amplitude 0.3*extent, base 0.35*extent). shell = 0 inserts every voxel
 * below the surface; shell = 1 only those down to the lowest 4-neighbour
 * surface (the first hit of any ray from above is unchanged). Columns are
 * inserted z-major, x-minor, top voxel first. Colour byte: 2-bit material
 * from the height band | ramp intensity +-8 noise, never 0. */
typedef struct svo_terrain_spec {
    uint32_t seed;
    int32_t depth;
    int32_t shell;
    int32_t boxes;      /* seeded axis-aligned solid boxes added after the terrain (0 = none) */
} svo_terrain_spec;
/* Inserts the terrain into a builder. */
svo_status svo_terrain_build(svo_builder* b, const svo_terrain_spec* spec);
/* Writes the terrain's voxels in insertion order (null arrays: count only). */
svo_status svo_terrain_voxels(const svo_terrain_spec* spec, uint32_t* x, uint32_t* y, uint32_t* z, uint32_t* rgba,
                              size_t cap, size_t* n);

/* ------------------------------------------------------------ cameras -- */
/* m = identity.rotate_z(rz).rotate_x(rx).rotate_y(ry), src/raycast.h:121-124. */
svo_status svo_view_from_euler(float rx, float ry, float rz, const float pos[3], int res_x, int res_y, float fov,
                               svo_view* out);
/* Camera at `pos` looking at `target` (rx/ry chosen so that row 2 of m points
 * at the target, rz = 0). */
svo_status svo_view_look_at(const float pos[3], const float target[3], int res_x, int res_y, float fov,
                            svo_view* out);
/* Wraps pos*16 into [0, 2^(depth+1)) on every axis (src/raycast.h:136-145). */
svo_status svo_wrap_position(float pos[3], int depth);
/* Seeded camera paths over the synthetic terrain.
 * kind 0: still camera at 1.5*extent from the centre, 20 degrees above it,
 *         looking at the centre;
 * kind 1: orbit at radius 1.5*extent, 0.5 degrees yaw per frame, height
 *         sinusoid 0.02*extent over 64 frames, looking at the centre;
 * kind 2: fast motion, 2 degrees yaw and 0.05*extent translation per frame;
 * kind 3: seeded random pose (frame is the view index). */
svo_status svo_camera_path(int kind, int depth, int frame, uint32_t seed, int res_x, int res_y, float fov,
                           svo_view* out);

#ifdef __cplusplus
}
#endif
#endif /* SVO_GB300_H */
