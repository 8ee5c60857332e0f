// sgmgb_internal.h -- host-side structures shared by the runtime, batch and server files.
#pragma once
#include <cuda_runtime.h>
#include <cstdint>
#include <cstddef>
#include <string>
#include "../../include/sgmgb.h"
#include "sgmgb_kernels.cuh"

// Shape of the path kernels: warps per block and disparities per lane
// (0 = the smallest valid), and the frame schedule (SGMGB_SCHED_*). Only
// speed depends on them.
struct PathShape {
    int wpb = 4;
    int dpl = 0;
    int sched = SGMGB_SCHED_AUTO;
};

// The fused schedule covers the plain variant with 4 paths in the
// two-lines-per-warp layout (D = 32, 64 or 128, no disparities-per-lane
// shape); other frames asking for it run the throughput schedule.
inline bool fused_applies(const sgmgb_frame_desc &fd, const PathShape &s) {
    return fd.variant == SGMGB_PLAIN && fd.paths == 4 && s.dpl == 0 && (fd.D == 32 || fd.D == 64 || fd.D == 128);
}

// The schedule a frame runs with. AUTO becomes FUSED (THROUGHPUT for the
// frames it does not cover) when frames share the GPU, and for a frame that
// has the GPU to itself (the synchronous host-buffer call, a server frame
// with nothing else in flight) SPLIT on frames of at least 2 Mpixel at
// D >= 64, LATENCY on the others. Measured on 1920x1080 frames, ms per frame
// with four in flight, FUSED / THROUGHPUT: D=64 0.251 / 0.259, D=128
// 0.480 / 0.512, D=32 0.185 / 0.197; a frame alone, SPLIT / LATENCY: D=64
// 0.327 / 0.340, D=128 0.639 / 0.697, D=32 0.254 / 0.237, and 1280x720
// D=128 0.374 / 0.329.
inline PathShape resolve_sched(PathShape s, bool alone, const sgmgb_frame_desc &fd) {
    if (s.sched != SGMGB_SCHED_AUTO) return s;
    if (!alone) s.sched = SGMGB_SCHED_FUSED;
    else s.sched = fused_applies(fd, s) && (size_t)fd.W * fd.H >= 2000000 && fd.D >= 64 ? SGMGB_SCHED_SPLIT
                                                                                         : SGMGB_SCHED_LATENCY;
    return s;
}

struct sgmgb_ctx {
    int device = 0;
    int sm_count = 0;
    cudaStream_t stream = nullptr;
    std::string last_error;
    // resident single-frame workspace (sgmgb_plan)
    sgmgb_frame_desc fd{};
    bool planned = false;
    struct FrameSlot *slot = nullptr;
    cudaEvent_t ev[5] = {nullptr, nullptr, nullptr, nullptr, nullptr};
    // CUDA graphs of the planned frame pipeline, one per (left, right, disp)
    // pointer triple seen (a small round-robin cache); replayed by
    // sgmgb_run_frame_async, all dropped when the plan changes.
    static constexpr int kGraphs = 8;
    cudaGraphExec_t graph[kGraphs] = {};
    const void *graph_key[kGraphs][3] = {};
    int graph_next = 0;
    // the synchronous call's frame: a CUDA graph on the slot's own buffers, of
    // the schedule that timed fastest for a frame alone (under AUTO; else the
    // set schedule); made at the first sgmgb_run_frame after a plan or a shape
    // change
    cudaGraphExec_t alone = nullptr;
    int alone_sched = 0;
    // stage times of the synchronous call: measured on the first call after a
    // plan and on every 8th call after it (each CUDA event on the stream costs
    // about 3 us of a 0.38 ms frame), the latest measurement reported
    unsigned timed_calls = 0;
    sgmgb_stage_times last_times{-1, -1, -1, -1, -1, 0};
    PathShape shape;
    // optional post-steps (sgmgb_run_frame_post): their workspace, made on first use
    void *post = nullptr;
    size_t post_bytes = 0;
};

// Device buffers of one frame slot. All pointers are carved from one
// allocation (`base`), 256-byte aligned.
struct FrameSlot {
    sgmgb_frame_desc fd{};
    void *base = nullptr;
    size_t bytes = 0;
    uint8_t *left = nullptr, *right = nullptr, *disp = nullptr;   // inputs / output
    uint64_t *cl = nullptr, *cr = nullptr;                        // full-scale census
    uint8_t *C = nullptr;                                         // W*H*D cost volume
    uint8_t *C1 = nullptr;                                        // half-scale cost volume (multi-scale)
    uint8_t *sc = nullptr;                                        // W*H*D scratch L
    uint16_t *S = nullptr;                                        // W*H*D sum (or two u8 planes)
    uint8_t *xp = nullptr;                                        // 1 (4 paths) or 5 (8 paths) more W*H*D u8 planes
    uint32_t *state = nullptr;                                    // line state of split rows (fused schedule)
    // multi-scale extras
    uint8_t *sobL = nullptr, *sobR = nullptr;                     // full-scale SobelX
    uint8_t *halfL = nullptr, *halfR = nullptr;                   // half-scale images
    uint8_t *hsobL = nullptr, *hsobR = nullptr;                   // half-scale SobelX
    uint64_t *cl1 = nullptr, *cr1 = nullptr;                      // half-scale census
    uint8_t *disp1 = nullptr;                                     // stage-1 argmin (defined work, unused)
    uint8_t *P1 = nullptr;                                        // the half-scale stage's 8 direction planes
    // independent path passes of one frame run on forked streams
    static constexpr int kAux = 7;
    cudaStream_t aux[kAux] = {};
    cudaEvent_t fork = nullptr, join[kAux] = {};
    // multi-scale: the half-scale stage runs on a stream set of its own beside
    // the full-scale one (ms, aux2, fork2, join2); fork_ms hands it the inputs,
    // c1 marks its cost volume (the full-scale cost merge reads it), s1_done its end
    cudaStream_t ms = nullptr, aux2[kAux] = {};
    cudaEvent_t fork2 = nullptr, join2[kAux] = {}, fork_ms = nullptr, c1 = nullptr, s1_done = nullptr;
};

namespace sgmgb {

// Captures the frame on the slot's own buffers (inputs left/right, map disp)
// under shape `sh` into a CUDA graph on stream st (which must be idle).
cudaError_t capture_frame(const FrameSlot &s, cudaStream_t st, const PathShape &sh, cudaGraphExec_t *out);

// Byte layout of a slot for a frame description; total in *bytes.
size_t slot_layout(const sgmgb_frame_desc &fd, FrameSlot *s /* may be null: size only */);
int  slot_alloc(const sgmgb_frame_desc &fd, FrameSlot **out, std::string &err);
void slot_free(FrameSlot *s);

// Per-kernel timing of one enqueued frame: ev[0] before the first launch,
// ev[i+1] after launch i (timing-enabled events, created by the caller).
struct KernelProbe {
    static constexpr int kMax = 32;
    int n = 0;
    cudaEvent_t ev[kMax + 1] = {};
    const char *name[kMax] = {};
    double bytes[kMax] = {};
};

// Enqueues the whole frame pipeline for `s` reading d_left/d_right and
// writing d_disp on `st`. Events ev_census / ev_end (optional) are recorded
// after the cost volume and at the end. With a probe, every kernel runs on
// `st` one after another and the probe's events bracket each launch.
cudaError_t enqueue_frame(const FrameSlot &s, const uint8_t *d_left, const uint8_t *d_right,
                          uint8_t *d_disp, cudaStream_t st, const PathShape &shape,
                          cudaEvent_t ev_census, cudaEvent_t ev_end, KernelProbe *probe = nullptr);

int set_err(sgmgb_ctx *ctx, int code, const std::string &msg);

}  // namespace sgmgb
