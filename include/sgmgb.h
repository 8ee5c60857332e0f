/* sgmgb.h -- C ABI of the GB300 SGM stereo engine (libsgmgb.so).
 *
 * Plain pointers and sizes only. Every entry point returns SGMGB_OK (0) or a
 * negative SGMGB_ERR_* code; sgmgb_strerror() names the code and
 * sgmgb_last_error() gives the message of the last failure on a context.
 *
 * Algorithms (bit-exact with kylefoxaustin/sgm-bench):
 *   SGMGB_PLAIN       census 9x7 -> Hamming cost (invalid 62) -> 4 or 8 paths,
 *                     P1 = 20, P2 = 192 -> argmin, lowest d on ties
 *                     (common/sgm_ref.c:101-144). D: multiple of 16 in [16, 256].
 *   SGMGB_MULTISCALE  SobelX -> census at 1/2 and full resolution -> averaged
 *                     cost (invalid 63) -> 8 paths with P1 40/20/10, P2 = 200,
 *                     saturating -> argmin at (2x,2y) (multiscale/sgm_ms_ref.c:
 *                     151-200). D = 64 and paths = 8 only; W and H even.
 *                     The output map is (W/2) x (H/2).
 *
 * Reference interfaces each group replaces:
 *   sgmgb_run_frame       the single-frame sgm_run_fn (common/sgm.h:29-31) as
 *                         used by the harness loops (common/harness.c:150-158);
 *                         sgm_gb300.c wraps it as SGM_IMPL.
 *   sgmgb_run_frame_async the device half of cuda_run (cuda/sgm_cuda_opt.cu:
 *                         321-366): inputs already on the device, one stream.
 *   SGMGB_MULTISCALE plans the frame loop of the standalone multi-scale
 *                         binary (multiscale/sgm_ms_ref.c:166-202).
 *   sgmgb_profile_frame   no reference symbol: per-kernel timing for the bench.
 *   sgmgb_set_path_shape, sgmgb_set_schedule, sgmgb_alone_schedule
 *                         no reference symbol: speed knobs, results unchanged.
 *   sgmgb_batch_*         no reference symbol: many frames per launch.
 *   sgmgb_server_*        no reference symbol: a continuous-batching request loop.
 */
#ifndef SGMGB_H
#define SGMGB_H
#include <stdint.h>
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

#define SGMGB_ABI_VERSION 1

enum {
    SGMGB_OK          = 0,
    SGMGB_ERR_ARG     = -1,   /* bad size, D, path count, variant or pointer */
    SGMGB_ERR_NOMEM   = -2,   /* host or device allocation failed */
    SGMGB_ERR_CUDA    = -3,   /* a CUDA call failed; see sgmgb_last_error */
    SGMGB_ERR_NODEV   = -4,   /* no usable CUDA device */
    SGMGB_ERR_BUDGET  = -5,   /* request refused: over the HBM budget or no free slot */
    SGMGB_ERR_TIMEOUT = -6,   /* a bounded device or host wait ran out */
    SGMGB_ERR_STATE   = -7    /* call not valid in the current state */
};

enum { SGMGB_PLAIN = 0, SGMGB_MULTISCALE = 1 };

/* Same layout as sgm_stage_times (include/sgm_plugin.h). */
typedef struct {
    double census_ms;
    double cost_ms;
    double aggregate_ms;
    double argmin_ms;
    double transfer_ms;
    int    threads_used;
} sgmgb_stage_times;

typedef struct {
    int W, H;      /* input size in pixels */
    int D;         /* disparity range */
    int paths;     /* 4 or 8 */
    int variant;   /* SGMGB_PLAIN or SGMGB_MULTISCALE */
} sgmgb_frame_desc;

typedef struct sgmgb_ctx sgmgb_ctx;

/* ---- version, errors, sizes (no GPU needed) ---- */
int         sgmgb_abi_version(void);
const char *sgmgb_strerror(int code);
const char *sgmgb_last_error(const sgmgb_ctx *ctx);
/* Validates a frame description (SGMGB_OK or SGMGB_ERR_ARG). */
int         sgmgb_check_desc(const sgmgb_frame_desc *fd);
/* Output map size: W x H for plain, (W/2) x (H/2) for multi-scale. */
int         sgmgb_out_size(const sgmgb_frame_desc *fd, int *out_w, int *out_h);
/* Device bytes one frame slot of this description holds resident. */
int         sgmgb_workspace_bytes(const sgmgb_frame_desc *fd, size_t *bytes);

/* ---- context ---- */
/* Binds to CUDA device `device`; fails with SGMGB_ERR_NODEV without one. */
int  sgmgb_create(int device, sgmgb_ctx **out);
void sgmgb_destroy(sgmgb_ctx *ctx);
/* Sizes the context's resident single-frame workspace (re-plans on change). */
int  sgmgb_plan(sgmgb_ctx *ctx, const sgmgb_frame_desc *fd);
/* Path-kernel shape of the context's frames: warps per block (1..4) and
 * disparities per lane. 0 (the default) packs two lines per warp into the
 * halves of each register for the scratch and 4-path final passes at D = 32,
 * 64 and 128, and uses the smallest valid value elsewhere; 2, 4 or 8 (raised
 * to the smallest value that fits a line in one warp: 2 up to D = 64, 4 up to
 * 128, 8 up to 256) keeps one line per lane group for every pass. Results do
 * not depend on it, only speed. Drops cached graphs. */
int  sgmgb_set_path_shape(sgmgb_ctx *ctx, int warps_per_block, int disp_per_lane);

/* Frame schedule (no reference symbol; results do not depend on it):
 *   LATENCY     every direction parks its L in a uint8 plane, all directions
 *               side by side, then one streaming pass adds the planes and
 *               takes the argmin: the shortest frame when the GPU is idle;
 *   THROUGHPUT  the last direction (T->B) adds the other directions' planes
 *               to its own L and takes the argmin: one plane less written and
 *               read per frame, for frames that share the GPU;
 *   FUSED       the two horizontal directions split each row in halves: the
 *               first halves compute the matching costs themselves (no cost
 *               pass) and park L; the vertical directions park theirs; the
 *               second halves resume the rows, add the three planes and take
 *               the argmin. Plain variant, 4 paths, D = 32, 64 or 128 in the
 *               default path shape; other frames run THROUGHPUT;
 *   SPLIT       as FUSED, but the costs come from the cost pass and the
 *               first halves of the rows run side by side with the vertical
 *               directions: the shortest critical path of the four. Same
 *               frames as FUSED; other frames run THROUGHPUT;
 *   AUTO        for sgmgb_run_frame: the schedule that runs fastest for a
 *               frame alone, timed once per plan (sgmgb_alone_schedule tells
 *               which); for a server frame with nothing else in flight: SPLIT
 *               on frames of at least 2,000,000 pixels at D >= 64 where it
 *               applies, LATENCY on the others; FUSED (THROUGHPUT where FUSED
 *               does not apply) for sgmgb_run_frame_async and the other server
 *               frames (the default).
 * Drops cached graphs. */
#define SGMGB_SCHED_AUTO       0
#define SGMGB_SCHED_LATENCY    1
#define SGMGB_SCHED_THROUGHPUT 2
#define SGMGB_SCHED_FUSED      3
#define SGMGB_SCHED_SPLIT      4
int  sgmgb_set_schedule(sgmgb_ctx *ctx, int schedule);
/* The schedule sgmgb_run_frame runs for the planned description: the set one,
 * or under AUTO the fastest for a frame alone, timed on the first call after
 * a plan or a shape or schedule change (this call makes that choice if no
 * frame ran yet). */
int  sgmgb_alone_schedule(sgmgb_ctx *ctx, int *schedule);

/* ---- single frame ---- */
/* Host buffers in and out, synchronous: the drop-in call. left/right are
 * W*H bytes, row-major; disp receives the output map (sgmgb_out_size). The
 * images are copied into the planned workspace by the copy engines (faster
 * from page-locked or CUDA-registered memory), the frame runs as one CUDA
 * graph with the schedule of sgmgb_alone_schedule, and the map is copied
 * back. t (may be NULL): the frame's stage times, measured with CUDA events
 * on the first call after a plan or a schedule or shape change and on every
 * 8th call after it (the events cost about 3 us each), the latest measurement
 * returned; census_ms, cost_ms and argmin_ms are -1 (one graph: aggregate_ms
 * is the whole frame on the device). */
int sgmgb_run_frame(sgmgb_ctx *ctx, const uint8_t *left, const uint8_t *right,
                    uint8_t *disp, sgmgb_stage_times *t);
/* Device buffers, enqueued on `stream` (a cudaStream_t, NULL = the context's
 * own stream); returns without waiting. Uses the planned workspace. */
int sgmgb_run_frame_async(sgmgb_ctx *ctx, const uint8_t *d_left, const uint8_t *d_right,
                          uint8_t *d_disp, void *stream);
/* Waits for everything the context enqueued on `stream` (NULL = own stream). */
int sgmgb_sync(sgmgb_ctx *ctx, void *stream);

/* ---- optional post-steps (no reference counterpart) ---- */
/* The reference has no post-steps (common/sgm_params.h:58). These are this
 * engine's, on the plain variant's summed volume S (the frame runs the
 * latency schedule; a second map and S cost an extra 2*W*H*D + 4*W*H bytes of
 * device memory, made on the first call):
 *   SGMGB_POST_LR        left-right consistency check: d_R(x) = argmin_d
 *                        S(x + d, d); a pixel whose d satisfies x - d < 0 or
 *                        |d - d_R(x - d)| > 1 becomes SGMGB_DISP_INVALID (D <= 240);
 *   SGMGB_POST_MEDIAN    3x3 median of the (checked) map, edges replicated;
 *   SGMGB_POST_SUBPIXEL  disp16 (W*H uint16) receives 16*d plus a parabola
 *                        offset (16*(S(d-1) - S(d+1))) / (2*(S(d-1) + S(d+1) -
 *                        2*S(d))) in integer arithmetic; 0xFFFF where checked out.
 * Host buffers, synchronous. flags = 0 gives the plain map. */
#define SGMGB_POST_LR        1
#define SGMGB_POST_MEDIAN    2
#define SGMGB_POST_SUBPIXEL  4
#define SGMGB_DISP_INVALID   255
int sgmgb_run_frame_post(sgmgb_ctx *ctx, const uint8_t *left, const uint8_t *right, uint8_t *disp,
                         uint16_t *disp16, int flags);

/* ---- measurement (no reference symbol) ---- */
typedef struct {
    char   name[24];   /* "census", "cost", "path_rl", ..., "sum_argmin" */
    double ms;         /* mean device time of one launch (CUDA events) */
    double bytes;      /* algorithmic bytes of one launch: inputs read once, outputs written once */
} sgmgb_kernel_stat;
/* Runs `reps` frames of the planned description on device buffers with every
 * kernel alone on the context's stream (no concurrent passes) and CUDA events
 * around each launch; fills up to max_out per-kernel means in launch order and
 * sets *n_out. Synchronous. */
int sgmgb_profile_frame(sgmgb_ctx *ctx, const uint8_t *d_left, const uint8_t *d_right, uint8_t *d_disp,
                        int reps, sgmgb_kernel_stat *out, int max_out, int *n_out);

/* ---- component entry points (parity tests, tools) ---- */
/* 9x7 census of one W x H image on the device; out is W*H uint64. */
int sgmgb_census_async(sgmgb_ctx *ctx, const uint8_t *d_img, uint64_t *d_out, int W, int H,
                       void *stream);

/* ---- a frame that allocates nothing (no reference counterpart) ---- */
/* Size of the static device array sgmgb_run_frame_noalloc works in. */
#define SGMGB_NOALLOC_SCRATCH_BYTES (24u << 20)
/* No counterpart in the reference. Runs one plain-variant frame on device
 * buffers on `stream` (a cudaStream_t; NULL = the legacy default stream),
 * with its whole workspace -- census descriptors, cost volume and three
 * W*H*D planes: 16*W*H + 4*W*H*D bytes in five regions, each rounded up to a
 * multiple of 256 bytes (at most 5*255 bytes more) -- in one static device
 * array of SGMGB_NOALLOC_SCRATCH_BYTES (24 MiB), so it allocates nothing: no
 * device, host or library allocation. It is for callers that must not
 * allocate after start-up, such as a real-time loop with a fixed
 * device-memory budget, where cudaMalloc/cudaFree can block on device-wide
 * synchronisation or fail once another allocator holds the free memory.
 * Limit: the workspace must fit the array, e.g. 320x240 at D=64 (4 or 8
 * paths), 200x200 at D=128, 640x480 at D=16; larger frames return
 * SGMGB_ERR_BUDGET. It runs on the CUDA device current in the calling thread
 * (the buffers must be that device's); note that the context calls above
 * (sgmgb_run_frame, sgmgb_batch_run, ...) make their context's device current
 * and leave it so. The first call on a device looks up the array's address
 * (cudaGetSymbolAddress, with that device current) and sets the path kernels'
 * shared-memory limits (cudaFuncSetAttribute), so make the first call before
 * any stream capture. Every call makes these CUDA runtime calls: cudaGetDevice,
 * then one launch per kernel (6 for 4 paths, 10 for 8), each followed by
 * cudaGetLastError. Nothing in the array needs to start at zero: every byte
 * a call reads is written earlier in the same call, in stream order. All
 * calls on a device share the one array: calls that overlap in time (on
 * other streams or threads) race and corrupt each other's output, so
 * serialise them, e.g. on one stream. Returns SGMGB_OK, SGMGB_ERR_ARG,
 * SGMGB_ERR_BUDGET, SGMGB_ERR_NODEV or SGMGB_ERR_CUDA (launch failure). */
int sgmgb_run_frame_noalloc(const uint8_t *d_left, const uint8_t *d_right, uint8_t *d_disp,
                            int W, int H, int D, int paths, void *stream);

/* ---- batch: many frames of mixed sizes in one run ---- */
/* A batch runs n plain-variant frames of any sizes, disparity ranges and path
 * counts in ONE persistent kernel launch (or as frames in flight: see
 * sgmgb_batch_set_mode): its blocks take work items (census
 * row bands, cost row bands, groups of lines of one direction) from a device
 * queue in phase order and wait, with a bounded spin, on per-frame phase
 * counters. The launch and its counter resets are captured in a CUDA graph on
 * the first run and replayed afterwards. Frames with 4 paths in the
 * two-lines-per-warp layout (D = 32, 64, 128) run the fused schedule's items
 * (SGMGB_SCHED_FUSED), the others the throughput schedule's. Outputs are
 * bit-identical to sgmgb_run_frame on each frame. */
typedef struct sgmgb_batch sgmgb_batch;
/* Plans n frames: one workspace arena, the work-item queue and its phase
 * counters. tune_cache (may be NULL) is an autotuner cache file (see below):
 * each frame takes the path-kernel shape recorded for its description, and the
 * launch the warps per block recorded for the largest frame; otherwise 4 warps
 * and the smallest valid disparities per lane. */
int  sgmgb_batch_create(sgmgb_ctx *ctx, const sgmgb_frame_desc *frames, int n,
                        const char *tune_cache, sgmgb_batch **out);
/* Runs the planned batch on device buffers (host arrays of n device pointers:
 * left/right W*H bytes, disp W*H bytes), enqueued on `stream` (NULL = the
 * context's stream); returns without waiting. */
int  sgmgb_batch_run(sgmgb_batch *b, const uint8_t *const *d_left,
                     const uint8_t *const *d_right, uint8_t *const *d_disp, void *stream);
/* Waits for the last run: SGMGB_OK, or SGMGB_ERR_TIMEOUT when a work item's
 * wait for its inputs ran past the wait limit (the run was abandoned and the
 * outputs are undefined; the context stays usable). */
int  sgmgb_batch_wait(sgmgb_batch *b);
/* Times candidate shapes of the persistent launch (warps per block 2 and 4;
 * disparities per lane 0 -- the two-lines-per-warp layout --, the smallest
 * valid, and twice that) on these buffers, keeps the fastest, and, when
 * tune_cache is not NULL, records it for every frame description; then times
 * the frames-in-flight mode (SGMGB_BATCH_IN_FLIGHT below) on 4, 6 and 8
 * lanes and keeps the faster mode. */
int  sgmgb_batch_autotune(sgmgb_batch *b, const uint8_t *const *d_left,
                          const uint8_t *const *d_right, uint8_t *const *d_disp,
                          const char *tune_cache);
/* Where the last persistent launch's time went (no reference symbol): ms[k]
 * is the time the persistent kernel's blocks spent on work items of kind k,
 * summed over blocks, in milliseconds of the GPU's global timer: k = 0 census, 1 cost,
 * 2 passes that park a direction's L, 3 final passes (planes added, argmin),
 * 4 first halves of split rows with their costs, 5 waiting for an item's
 * inputs (or for the queue to end). n <= 6 entries are filled (more are set
 * to 0); *blocks (may be NULL) receives the launch's block count, so that
 * sum(ms) / blocks is about the launch's time. Waits for the last run;
 * SGMGB_ERR_STATE before the first persistent launch. */
int  sgmgb_batch_busy(sgmgb_batch *b, double *ms, int n, int *blocks);
/* Path-kernel shape used for frame i: warps per block and disparities per lane. */
int  sgmgb_batch_tile_shape(const sgmgb_batch *b, int i, int *warps_per_block,
                            int *disp_per_lane);
/* Failure injection for tests (host side; nothing faults on the device):
 * wait_limit_ms bounds every device-side wait (default 2000); stall_frame >= 0
 * raises that frame's census completion target by one, so the frame's cost
 * items wait until the limit and the next run reports SGMGB_ERR_TIMEOUT.
 * stall_frame = -1 clears it. */
int  sgmgb_batch_set_fault(sgmgb_batch *b, int wait_limit_ms, int stall_frame);
/* How sgmgb_batch_run executes the planned frames (no reference symbol;
 * outputs never change):
 *   SGMGB_BATCH_PERSISTENT  the one persistent launch above (after create);
 *   SGMGB_BATCH_IN_FLIGHT   every frame's own pipeline, as
 *                           sgmgb_run_frame_async runs it with frames in
 *                           flight (the fused schedule where it applies, else
 *                           the throughput one; 4 warps per block, the
 *                           smallest disparities per lane), on `lanes` (1..8)
 *                           concurrent chains of about equal work (frames
 *                           largest first, each onto the least loaded chain);
 *                           the whole run is one CUDA graph, captured again
 *                           when the device pointers differ from the last run's.
 * Runs of either mode on one stream are ordered. The wait limit and the
 * stall of sgmgb_batch_set_fault, and sgmgb_batch_busy, concern the
 * persistent launch. sgmgb_batch_autotune times both modes and keeps the
 * faster (lanes 4, 6 and 8 for the second). */
#define SGMGB_BATCH_PERSISTENT 0
#define SGMGB_BATCH_IN_FLIGHT  1
int  sgmgb_batch_set_mode(sgmgb_batch *b, int mode, int lanes);
int  sgmgb_batch_mode(const sgmgb_batch *b, int *mode, int *lanes);
void sgmgb_batch_destroy(sgmgb_batch *b);

/* ---- autotuner cache (host-only; no GPU needed) ---- */
/* Records / looks up the chosen path-kernel shape for a frame shape. The
 * cache file is a plain text table "W H D paths variant warps dpl us" (dpl 0:
 * two lines per warp); the last matching line wins. */
int sgmgb_tune_lookup(const char *cache_path, const sgmgb_frame_desc *fd,
                      int *warps_per_block, int *disp_per_lane);
int sgmgb_tune_record(const char *cache_path, const sgmgb_frame_desc *fd,
                      int warps_per_block, int disp_per_lane, double us);

/* ---- server: continuous batching of camera frames ---- */
typedef struct sgmgb_server sgmgb_server;
typedef struct {
    size_t hbm_budget_bytes;   /* admission limit for resident workspaces */
    int    max_inflight;       /* frames on the device at once */
    int    streams;            /* CUDA streams the frames are spread over */
} sgmgb_server_config;
typedef struct {
    uint64_t frames_done;
    uint64_t frames_refused;
    double   p50_ms, p99_ms, max_ms;   /* submit -> result on the host */
    double   fps;                      /* frames_done / wall time */
    size_t   resident_bytes;
} sgmgb_server_stats;

int  sgmgb_server_create(sgmgb_ctx *ctx, const sgmgb_server_config *cfg,
                         sgmgb_server **out);
/* Registers a camera: allocates its resident buffers if the budget allows
 * (SGMGB_ERR_BUDGET otherwise). */
int  sgmgb_server_add_camera(sgmgb_server *s, int cam_id, const sgmgb_frame_desc *fd);
/* Makes every camera's resident slots up front, up to slots_per_camera each
 * (at most 4), one per camera in turn while the HBM budget allows, so that
 * no slot is allocated after the first frame is submitted (frames otherwise
 * grow a camera's slots on demand, and an allocation can stall the device).
 * *slots_resident (may be NULL) receives the total number of slots. */
int  sgmgb_server_prepare(sgmgb_server *s, int slots_per_camera, int *slots_resident);
/* Submits one frame (host buffers of W*H bytes, copied before returning).
 * Admitted frames join the device work immediately; *ticket identifies it.
 * SGMGB_ERR_BUDGET when no slot is free for this camera. */
int  sgmgb_server_submit(sgmgb_server *s, int cam_id, const uint8_t *left,
                         const uint8_t *right, uint64_t *ticket);
/* Non-blocking: 1 and the output map (and latency) when done, 0 if pending. */
int  sgmgb_server_poll(sgmgb_server *s, uint64_t ticket, uint8_t *disp, double *latency_ms);
/* Blocks up to timeout_ms for the ticket (SGMGB_ERR_TIMEOUT when it runs out). */
int  sgmgb_server_wait(sgmgb_server *s, uint64_t ticket, uint8_t *disp, double *latency_ms,
                       int timeout_ms);
int  sgmgb_server_stats_get(sgmgb_server *s, sgmgb_server_stats *st);
void sgmgb_server_destroy(sgmgb_server *s);

/* ---- synthetic stereo pairs (host-only, deterministic on every CPU) ---- */
/* Band-limited noise (Gaussian-blurred uniform octaves, sigma 1/4/16),
 * ground truth piecewise planar over 40 Voronoi cells (offsets in [0, D-1],
 * slopes within +-0.02 px/px), right = left warped by the ground truth with
 * occlusions refilled from fresh noise, plus Gaussian noise sigma 2.
 * Writes W*H bytes to each non-NULL output. */
int sgmgb_synth_pair(int W, int H, int D, uint64_t seed, uint8_t *left, uint8_t *right,
                     uint8_t *gt);

#ifdef __cplusplus
}
#endif
#endif
