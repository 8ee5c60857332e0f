// sgmgb_batch.cu -- many frames of mixed sizes in one persistent launch (or as
// frames in flight in one CUDA graph: SGMGB_BATCH_IN_FLIGHT, at the end).
//
// Work decomposition (plain variant, common/sgm_ref.c semantics per frame):
//   phase 0  census   one item per band of BAND (8) rows (both images)
//   4 paths, two lines per warp (D = 32, 64, 128), the fused schedule:
//            phase 1  the first halves of L->R and R->L with their costs
//                     computed from the census (sgmgb_fused.cuh): the cost
//                     volume, one plane of L and each row's line state
//            phase 2  T->B and B->T into two u8 planes
//            phase 3  the second halves of L->R and R->L add the three planes
//                     to their L and take the argmin
//   otherwise phase 1  cost: one item per band, C[p][d] from its census rows
//   4 paths: phase 2  R->L, B->T, L->R into three u8 planes (all three passes)
//            phase 3  T->B adds the planes to its L and takes the argmin
//   8 paths: phase 2  R->L, L->R, B->T and the four diagonals into seven planes
//            phase 3  T->B adds the seven planes to its L and takes the argmin
// An item of phase k of frame f starts when every item of phase k-1 of f has
// finished. Items are queued phase-major over all frames, so while one frame
// waits at a phase boundary the others keep the SMs busy; every item's
// dependencies sit earlier in the queue, so a block never waits on an item
// that no running block holds.
//
// Cross-block data (census, cost, planes, sums) is read through L2 only
// (cp.async.cg, ld.global.cg), with one exception: the first-half items copy
// the census descriptors with 8-byte cp.async.ca, through L1. That is safe
// because L1 holds no line from before the launch, and no block reads a
// frame's descriptors before every census item of that frame has finished
// (the item's acquire and block barrier) -- after which they do not change.
//
// Every item's busy time and its wait for its inputs are accumulated per item
// kind from global-timer stamps into the control block (sgmgb_batch_busy).
#include "sgmgb_internal.h"
#include "sgmgb_path.cuh"
#include "sgmgb_tiles.cuh"
#include "sgmgb_pair.cuh"
#include "sgmgb_fused.cuh"
#include <algorithm>
#include <cstring>
#include <map>
#include <new>
#include <vector>

namespace sgmgb {

namespace {

constexpr int BAND = tiles::CEN_ROWS;   // rows per census / cost item
constexpr int MAXPH = 4;         // phases per frame: census, cost, scratch passes, final pass

enum ItemKind : int { IT_CENSUS = 0, IT_COST = 1, IT_PATH = 2, IT_HCOST = 3 };
// busy-time kinds (BCtl::busy): census, cost, passes that park L, final
// passes, first halves with costs, and the waits for inputs
enum BusyKind : int { BK_CENSUS = 0, BK_COST = 1, BK_SCRATCH = 2, BK_FINAL = 3, BK_HCOST = 4, BK_WAIT = 5,
                      BK_N = 6 };

struct BFrame {                  // per frame; the user pointers are refreshed per run
    const uint8_t *left, *right;
    uint8_t *disp;
    uint64_t *cl, *cr;
    uint8_t *C;
    int W, H, D;
};

struct BPass {                   // one direction of one frame
    LineParams P;                // C, planes, S, W, H, D, nl/lpl/gpw, dx, dy, p1, p2, nlines, key16
    int frame;
    int mode;
    int dpl;                     // disparities per lane; 0: two lines per warp (sgmgb_pair.cuh)
};

struct BItem {
    int kind;
    int frame;
    int phase;                   // this item's phase
    int arg;                     // band (census, cost) or pass index (path)
    int sub;                     // path: first warp of the item
};

struct BCtl {                    // device control block, reset before every run
    unsigned next;               // queue head
    unsigned abort;              // set on a wait timeout: every block stops taking items
    int err_item;                // item whose wait ran out (-1: none)
    unsigned pad;
    unsigned long long busy[BK_N];   // nanoseconds summed over items, per BusyKind
};

// Nanoseconds of the GPU's global timer (busy-time stamps).
__device__ __forceinline__ unsigned long long gtime_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

__device__ __forceinline__ unsigned ld_acquire(const unsigned *p) {
    unsigned v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

// Thread 0 only: waits until *cnt >= need, the run is aborted, or the limit
// passes (then records the item and aborts the run). Returns false if the
// item must not run.
__device__ bool wait_count(const unsigned *cnt, unsigned need, BCtl *ctl, int item,
                           long long limit_ns) {
    if (ld_acquire(cnt) >= need) return true;
    const unsigned long long t0 = gtime_ns();
    for (unsigned it = 0;; it++) {
        if (ld_acquire(&ctl->abort)) return false;
        if (ld_acquire(cnt) >= need) return true;
        if ((long long)(gtime_ns() - t0) > limit_ns || it > (1u << 26)) {
            atomicCAS(&ctl->err_item, -1, item);
            atomicExch(&ctl->abort, 1u);
            return false;
        }
        __nanosleep(it < 64 ? 64 : 512);
    }
}


// Census 9x7 of rows [y0, y0+BAND) of both images (common/sgm_ref.c:23-41),
// one 128-pixel tile at a time (sgmgb_tiles.cuh).
__device__ void item_census(const BFrame &F, int band, uint8_t *sm) {
    for (int img = 0; img < 2; img++)
        for (int x0 = 0; x0 < F.W; x0 += tiles::CEN_PX)
            tiles::census_tile(img ? F.right : F.left, img ? F.cr : F.cl, F.W, F.H, x0, band * BAND, sm,
                               threadIdx.x, blockDim.x);
}

// Cost C[(y*W + x)*D + d] = popcount(cl[x] ^ cr[x-d]), 62 where x - d < 0
// (common/sgm_ref.c:44-56), for rows [y0, y0+BAND), one 64-pixel tile at a
// time; the descriptors were written by other blocks, so they are read
// through L2 only.
__device__ void item_cost(const BFrame &F, int band, uint8_t *sm) {
    for (int y = band * BAND; y < min(band * BAND + BAND, F.H); y++)
        for (int x0 = 0; x0 < F.W; x0 += tiles::COST_PX)
            tiles::cost_tile<true, false>(F.cl, F.cr, F.C, nullptr, F.W, F.D, kInvalidPlain, y, x0, sm,
                                          threadIdx.x, blockDim.x);
}

// One warp's share of a path item: lines of warp `warp` of pass `bp`.
__device__ __forceinline__ void item_path(const BPass &bp, uint8_t *disp, int warp, uint8_t *ring) {
    LineParams P = bp.P;
    P.disp = disp;
    const bool key16 = P.key16 && P.D <= 64;
    if (bp.dpl == 0) {                           // two lines per warp
        switch ((P.D >> 5) * 8 + bp.mode) {
        case 1 * 8 + MODE_SCRATCH: path_pair<1, MODE_SCRATCH, 0, false>(P, warp, ring); break;
        case 1 * 8 + MODE_STORE:   path_pair<1, MODE_STORE, 0, false>(P, warp, ring); break;
        case 1 * 8 + MODE_ACCUM:   path_pair<1, MODE_ACCUM, 0, false>(P, warp, ring); break;
        case 1 * 8 + MODE_FINAL:   path_pair<1, MODE_FINAL, 0, false>(P, warp, ring); break;
        case 1 * 8 + MODE_FINAL3:  path_pair<1, MODE_FINAL3, 0, true>(P, warp, ring); break;
        case 2 * 8 + MODE_SCRATCH: path_pair<2, MODE_SCRATCH, 0, false>(P, warp, ring); break;
        case 2 * 8 + MODE_STORE:   path_pair<2, MODE_STORE, 0, false>(P, warp, ring); break;
        case 2 * 8 + MODE_ACCUM:   path_pair<2, MODE_ACCUM, 0, false>(P, warp, ring); break;
        case 2 * 8 + MODE_FINAL:   path_pair<2, MODE_FINAL, 0, false>(P, warp, ring); break;
        case 2 * 8 + MODE_FINAL3:  path_pair<2, MODE_FINAL3, 0, true>(P, warp, ring); break;
        case 4 * 8 + MODE_SCRATCH: path_pair<4, MODE_SCRATCH, 0, false>(P, warp, ring); break;
        case 4 * 8 + MODE_STORE:   path_pair<4, MODE_STORE, 0, false>(P, warp, ring); break;
        case 4 * 8 + MODE_ACCUM:   path_pair<4, MODE_ACCUM, 0, false>(P, warp, ring); break;
        case 4 * 8 + MODE_FINAL:   path_pair<4, MODE_FINAL, 0, false>(P, warp, ring); break;
        case 1 * 8 + MODE_FINAL7:  path_pair<1, MODE_FINAL7, 0, false>(P, warp, ring); break;
        case 2 * 8 + MODE_FINAL7:  path_pair<2, MODE_FINAL7, 0, false>(P, warp, ring); break;
        case 4 * 8 + MODE_FINAL7:  path_pair<4, MODE_FINAL7, 0, false>(P, warp, ring); break;
        case 1 * 8 + MODE_FINAL3H: path_pair<1, MODE_FINAL3H, 0, true>(P, warp, ring); break;
        case 2 * 8 + MODE_FINAL3H: path_pair<2, MODE_FINAL3H, 0, true>(P, warp, ring); break;
        case 4 * 8 + MODE_FINAL3H: path_pair<4, MODE_FINAL3H, 0, false>(P, warp, ring); break;
        default:                   path_pair<4, MODE_FINAL3, 0, false>(P, warp, ring); break;
        }
        return;
    }
    switch (bp.dpl * 8 + bp.mode) {
    case 2 * 8 + MODE_SCRATCH: path_warp<2, MODE_SCRATCH, 0, false>(P, warp, ring); break;
    case 2 * 8 + MODE_STORE:   path_warp<2, MODE_STORE, 0, false>(P, warp, ring); break;
    case 2 * 8 + MODE_ACCUM:   path_warp<2, MODE_ACCUM, 0, false>(P, warp, ring); break;
    case 2 * 8 + MODE_FINAL:   path_warp<2, MODE_FINAL, 0, false>(P, warp, ring); break;
    case 2 * 8 + MODE_FINAL7:  path_warp<2, MODE_FINAL7, 0, false>(P, warp, ring); break;
    case 2 * 8 + MODE_FINAL3:
        if (key16) path_warp<2, MODE_FINAL3, 0, true>(P, warp, ring);
        else path_warp<2, MODE_FINAL3, 0, false>(P, warp, ring);
        break;
    case 4 * 8 + MODE_SCRATCH: path_warp<4, MODE_SCRATCH, 0, false>(P, warp, ring); break;
    case 4 * 8 + MODE_STORE:   path_warp<4, MODE_STORE, 0, false>(P, warp, ring); break;
    case 4 * 8 + MODE_ACCUM:   path_warp<4, MODE_ACCUM, 0, false>(P, warp, ring); break;
    case 4 * 8 + MODE_FINAL:   path_warp<4, MODE_FINAL, 0, false>(P, warp, ring); break;
    case 4 * 8 + MODE_FINAL7:  path_warp<4, MODE_FINAL7, 0, false>(P, warp, ring); break;
    case 4 * 8 + MODE_FINAL3:
        if (key16) path_warp<4, MODE_FINAL3, 0, true>(P, warp, ring);
        else path_warp<4, MODE_FINAL3, 0, false>(P, warp, ring);
        break;
    case 8 * 8 + MODE_SCRATCH: path_warp<8, MODE_SCRATCH, 0, false>(P, warp, ring); break;
    case 8 * 8 + MODE_STORE:   path_warp<8, MODE_STORE, 0, false>(P, warp, ring); break;
    case 8 * 8 + MODE_ACCUM:   path_warp<8, MODE_ACCUM, 0, false>(P, warp, ring); break;
    case 8 * 8 + MODE_FINAL:   path_warp<8, MODE_FINAL, 0, false>(P, warp, ring); break;
    case 8 * 8 + MODE_FINAL7:  path_warp<8, MODE_FINAL7, 0, false>(P, warp, ring); break;
    case 8 * 8 + MODE_FINAL3:  path_warp<8, MODE_FINAL3, 0, false>(P, warp, ring); break;
    default: break;
    }
}

// One warp's share of a first-half item: row pair `pair` of pass `bp` (its
// P.dx gives the direction).
__device__ __forceinline__ void item_hcost(const BPass &bp, int pair, uint8_t *ring) {
    uint64_t *ws = (uint64_t *)ring;
    const bool lr = bp.P.dx > 0;
    switch (bp.P.D) {
    case 32:  if (lr) path_hcost<1, 1>(bp.P, pair, ws); else path_hcost<1, -1>(bp.P, pair, ws); break;
    case 64:  if (lr) path_hcost<2, 1>(bp.P, pair, ws); else path_hcost<2, -1>(bp.P, pair, ws); break;
    default:  if (lr) path_hcost<4, 1>(bp.P, pair, ws); else path_hcost<4, -1>(bp.P, pair, ws); break;
    }
}

// The persistent batch kernel: every block loops taking the next queued item
// until the queue is empty or the run is aborted. `ring_bytes`: one warp's
// path ring; the census and cost items use the start of the block's memory.
// At most 128 registers, so that two 256-thread (four 128-thread) blocks fit
// an SM whatever item kinds are inlined.
__global__ void __launch_bounds__(256, 2)
k_batch(const BItem *__restrict__ items, int n_items, const BFrame *__restrict__ frames,
        const BPass *__restrict__ passes, unsigned *done, const unsigned *__restrict__ need,
        BCtl *ctl, int ring_bytes, long long limit_ns) {
    extern __shared__ __align__(16) uint8_t smem[];
    __shared__ int s_item;
    const int wib = threadIdx.x >> 5;
    unsigned long long t_ready = 0;              // thread 0: when the item's inputs were there
    for (;;) {
        if (threadIdx.x == 0) {
            int it = ld_acquire(&ctl->abort) ? n_items : (int)atomicAdd(&ctl->next, 1u);
            const unsigned long long t_take = gtime_ns();
            if (it < n_items) {
                const BItem I = items[it];
                if (I.phase > 0) {
                    const int c = I.frame * MAXPH + I.phase - 1;
                    if (!wait_count(&done[c], need[c], ctl, it, limit_ns)) it = n_items;
                }
            }
            t_ready = gtime_ns();
            atomicAdd(&ctl->busy[BK_WAIT], t_ready - t_take);
            s_item = it;
        }
        __syncthreads();
        const int it = s_item;
        if (it >= n_items) break;
        const BItem I = items[it];
        switch (I.kind) {
        case IT_CENSUS: item_census(frames[I.frame], I.arg, smem); break;
        case IT_COST:   item_cost(frames[I.frame], I.arg, smem); break;
        case IT_HCOST:  item_hcost(passes[I.arg], I.sub + wib, smem + wib * ring_bytes); break;
        default:        item_path(passes[I.arg], frames[I.frame].disp, I.sub + wib, smem + wib * ring_bytes); break;
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            __threadfence();
            atomicAdd(&done[I.frame * MAXPH + I.phase], 1u);
            const int m = I.kind == IT_PATH ? passes[I.arg].mode : -1;
            const int kind = I.kind == IT_CENSUS ? BK_CENSUS : I.kind == IT_COST ? BK_COST
                           : I.kind == IT_HCOST ? BK_HCOST : m == MODE_SCRATCH ? BK_SCRATCH : BK_FINAL;
            atomicAdd(&ctl->busy[kind], gtime_ns() - t_ready);
        }
    }
}

template <int DPL, int MODE> constexpr int ring_of() { return Slot<DPL, MODE>::RING; }

// The pair layout serves every pass at D = 32, 64, 128.
bool pair_ok(int D) { return D == 32 || D == 64 || D == 128; }

template <int NR>
int pair_ring_nr(int mode) {
    switch (mode) {
    case MODE_SCRATCH: return PairSlot<NR, MODE_SCRATCH>::RING;
    case MODE_STORE:   return PairSlot<NR, MODE_STORE>::RING;
    case MODE_ACCUM:   return PairSlot<NR, MODE_ACCUM>::RING;
    case MODE_FINAL:   return PairSlot<NR, MODE_FINAL>::RING;
    case MODE_FINAL7:  return PairSlot<NR, MODE_FINAL7>::RING;
    default:           return PairSlot<NR, MODE_FINAL3>::RING;
    }
}

int pair_ring_bytes(int D, int mode) {
    return D == 32 ? pair_ring_nr<1>(mode) : (D == 64 ? pair_ring_nr<2>(mode) : pair_ring_nr<4>(mode));
}

// Largest per-warp ring a pass of this shape needs.
int ring_bytes_for(int dpl, int mode) {
    switch (dpl * 8 + mode) {
    case 2 * 8 + MODE_SCRATCH: return ring_of<2, MODE_SCRATCH>();
    case 2 * 8 + MODE_STORE:   return ring_of<2, MODE_STORE>();
    case 2 * 8 + MODE_ACCUM:   return ring_of<2, MODE_ACCUM>();
    case 2 * 8 + MODE_FINAL:   return ring_of<2, MODE_FINAL>();
    case 2 * 8 + MODE_FINAL7:  return ring_of<2, MODE_FINAL7>();
    case 2 * 8 + MODE_FINAL3:  return ring_of<2, MODE_FINAL3>();
    case 4 * 8 + MODE_SCRATCH: return ring_of<4, MODE_SCRATCH>();
    case 4 * 8 + MODE_STORE:   return ring_of<4, MODE_STORE>();
    case 4 * 8 + MODE_ACCUM:   return ring_of<4, MODE_ACCUM>();
    case 4 * 8 + MODE_FINAL:   return ring_of<4, MODE_FINAL>();
    case 4 * 8 + MODE_FINAL7:  return ring_of<4, MODE_FINAL7>();
    case 4 * 8 + MODE_FINAL3:  return ring_of<4, MODE_FINAL3>();
    case 8 * 8 + MODE_SCRATCH: return ring_of<8, MODE_SCRATCH>();
    case 8 * 8 + MODE_STORE:   return ring_of<8, MODE_STORE>();
    case 8 * 8 + MODE_ACCUM:   return ring_of<8, MODE_ACCUM>();
    case 8 * 8 + MODE_FINAL:   return ring_of<8, MODE_FINAL>();
    case 8 * 8 + MODE_FINAL7:  return ring_of<8, MODE_FINAL7>();
    case 8 * 8 + MODE_FINAL3:  return ring_of<8, MODE_FINAL3>();
    default: return 0;
    }
}

}  // namespace
}  // namespace sgmgb

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
using namespace sgmgb;

struct sgmgb_batch {
    sgmgb_ctx *ctx = nullptr;
    int n = 0;
    std::vector<sgmgb_frame_desc> fds;
    std::vector<int> dpl;                 // per frame: 0 (pair layout where it applies) or 2, 4, 8
    int wpb = 4;
    // device memory
    void *arena = nullptr;                // all frames' workspaces
    size_t arena_bytes = 0;
    std::vector<FrameSlot> slots;         // carved pointers (host copy)
    void *tables = nullptr;               // frames | passes | items | done | need | ctl
    BFrame *d_frames = nullptr;
    BPass *d_passes = nullptr;
    BItem *d_items = nullptr;
    unsigned *d_done = nullptr, *d_need = nullptr;
    BCtl *d_ctl = nullptr;
    int n_items = 0, n_passes = 0;
    int ring_bytes = 0;
    size_t smem_bytes = 0;
    int grid = 0;
    std::vector<unsigned> need;
    // pinned host staging
    BFrame *h_frames = nullptr;           // pointer table copied in by every run
    BCtl *h_ctl = nullptr;                // [0]: reset image, [1]: read back after the run
    // graph of [table copy, counter reset, kernel, control read-back]
    cudaStream_t cap = nullptr;
    cudaGraphExec_t graph = nullptr;
    cudaEvent_t done_ev = nullptr;
    bool ran = false;
    int wait_limit_ms = 2000;
    int stall_frame = -1;
    // frames in flight (SGMGB_BATCH_IN_FLIGHT): each frame's own pipeline on
    // one of `lanes` chains; a chain is a stream plus the forked streams and events
    // of its frames (FrameSlot fields, no buffers); the run is one graph,
    // keyed by the device pointers it was captured with
    int mode = SGMGB_BATCH_PERSISTENT;
    int lanes = 0;
    std::vector<FrameSlot> chain;
    std::vector<cudaStream_t> chain_st;
    cudaEvent_t lane_fork = nullptr;
    std::vector<cudaEvent_t> lane_join;
    cudaGraphExec_t fgraph = nullptr;
    std::vector<const void *> fkey;
    bool last_persistent = false;         // the last run was the persistent launch
    bool ran_persistent = false;          // h_ctl[1] holds a persistent launch's read-back
};

namespace {

int berr(sgmgb_batch *b, int code, const std::string &msg) { return set_err(b ? b->ctx : nullptr, code, msg); }

void free_tables(sgmgb_batch *b) {
    if (b->graph) { cudaGraphExecDestroy(b->graph); b->graph = nullptr; }
    if (b->tables) { cudaFree(b->tables); b->tables = nullptr; }
}

// Builds passes, items and completion targets for the current shapes and
// uploads them; drops the graph.
int build_plan(sgmgb_batch *b) {
    cudaSetDevice(b->ctx->device);
    if (b->ran) cudaEventSynchronize(b->done_ev);
    free_tables(b);
    std::vector<BPass> passes;
    std::vector<std::vector<BItem>> by_phase(MAXPH);
    b->need.assign((size_t)b->n * MAXPH, 0u);
    int ring = 0;
    for (int f = 0; f < b->n; f++) {
        const sgmgb_frame_desc &fd = b->fds[f];
        const FrameSlot &s = b->slots[f];
        const int nb = (fd.H + BAND - 1) / BAND;
        // 4 paths in the pair layout: the fused schedule (no cost items)
        const bool fused = fd.paths == 4 && b->dpl[f] == 0 && pair_ok(fd.D);
        for (int k = 0; k < nb; k++) {
            by_phase[0].push_back({IT_CENSUS, f, 0, k, 0});
            if (!fused) by_phase[1].push_back({IT_COST, f, 1, k, 0});
        }
        b->need[(size_t)f * MAXPH + 0] = nb;
        b->need[(size_t)f * MAXPH + 1] = fused ? 0 : nb;
        if (fused) {
            const size_t plane = (size_t)fd.W * fd.H * fd.D;
            uint8_t *ph = s.sc, *ptb = (uint8_t *)s.S, *pbt = (uint8_t *)s.S + plane;
            LineParams q{};
            q.C = s.C; q.W = fd.W; q.H = fd.H; q.D = fd.D; q.p1 = 20; q.p2 = 192; q.dpl = 0; q.key16 = fd.D <= 64;
            const int npairs = (fd.H + 1) / 2;
            // phase 1: the first halves of L->R and R->L with their costs
            for (int dx : {1, -1}) {
                BPass bp{};
                bp.P = q;
                bp.P.dx = dx; bp.P.dy = 0; bp.P.hseg = 1; bp.P.cl = s.cl; bp.P.cr = s.cr; bp.P.sc = ph;
                bp.P.state = s.state; bp.P.nlines = fd.H;
                bp.frame = f; bp.mode = MODE_SCRATCH; bp.dpl = 0;
                const int pi = (int)passes.size();
                passes.push_back(bp);
                const int nit = (npairs + b->wpb - 1) / b->wpb;
                for (int j = 0; j < nit; j++) by_phase[1].push_back({IT_HCOST, f, 1, pi, j * b->wpb});
                b->need[(size_t)f * MAXPH + 1] += nit;
            }
            ring = std::max(ring, fd.D == 32 ? HCost<1>::BYTES : fd.D == 64 ? HCost<2>::BYTES : HCost<4>::BYTES);
            // phase 2: T->B and B->T into two planes; phase 3: the second halves
            struct FSpec { int dx, dy, mode, phase, hseg; uint8_t *sc; const uint8_t *sc2, *sc3; };
            const FSpec fs[4] = {{0, 1, MODE_SCRATCH, 2, 0, ptb, nullptr, nullptr},
                                 {0, -1, MODE_SCRATCH, 2, 0, pbt, nullptr, nullptr},
                                 {1, 0, MODE_FINAL3H, 3, 2, ph, ptb, pbt},
                                 {-1, 0, MODE_FINAL3H, 3, 2, ph, ptb, pbt}};
            for (const FSpec &sp : fs) {
                BPass bp{};
                bp.P = q;
                bp.P.dx = sp.dx; bp.P.dy = sp.dy; bp.P.hseg = sp.hseg;
                bp.P.sc = sp.sc; bp.P.sc2 = sp.sc2; bp.P.sc3 = sp.sc3;
                bp.P.state = sp.hseg ? s.state : nullptr;
                bp.P.nlines = lines_for(fd.W, fd.H, sp.dx, sp.dy);
                bp.frame = f; bp.mode = sp.mode; bp.dpl = 0;
                const int pi = (int)passes.size();
                passes.push_back(bp);
                ring = std::max(ring, pair_ring_bytes(fd.D, sp.mode));
                const int warps = (bp.P.nlines + 1) / 2;
                const int nit = (warps + b->wpb - 1) / b->wpb;
                for (int j = 0; j < nit; j++) by_phase[sp.phase].push_back({IT_PATH, f, sp.phase, pi, j * b->wpb});
                b->need[(size_t)f * MAXPH + sp.phase] += nit;
            }
            continue;
        }
        LineParams base{};
        base.C = s.C; base.sc = s.sc; base.S = s.S; base.disp = nullptr;
        base.W = fd.W; base.H = fd.H; base.D = fd.D; base.p1 = 20; base.p2 = 192;
        base.key16 = (fd.paths == 4 && fd.D <= 64) ? 1 : 0;
        const int fdpl = b->dpl[f];                  // 0: pair layout where it applies
        const int dpl = fdpl ? fdpl : path_dpl(fd.D, 0);
        base.dpl = dpl;
        base.nl = fd.D / dpl; base.lpl = base.nl; base.gpw = (32 % base.lpl == 0) ? 32 / base.lpl : 1;
        struct Spec { int dx, dy, mode, phase; uint8_t *sc; const uint8_t *sc2, *sc3; };
        std::vector<Spec> specs;
        const uint8_t *xplanes[4] = {nullptr, nullptr, nullptr, nullptr};
        if (fd.paths == 4) {
            const size_t plane = (size_t)fd.W * fd.H * fd.D;
            uint8_t *pl[3] = {s.sc, (uint8_t *)s.S, (uint8_t *)s.S + plane};
            specs.push_back({-1, 0, MODE_SCRATCH, 2, pl[0], nullptr, nullptr});
            specs.push_back({0, -1, MODE_SCRATCH, 2, pl[1], nullptr, nullptr});
            specs.push_back({1, 0, MODE_SCRATCH, 2, pl[2], nullptr, nullptr});
            specs.push_back({0, 1, MODE_FINAL3, 3, pl[0], pl[1], pl[2]});
        } else {
            // seven directions into seven planes, then T->B sums them (MODE_FINAL7)
            const size_t plane = (size_t)fd.W * fd.H * fd.D;
            uint8_t *pl[7] = {s.sc, (uint8_t *)s.S, (uint8_t *)s.S + plane, s.xp, s.xp + plane, s.xp + 2 * plane,
                              s.xp + 3 * plane};
            static const int dirs[7][2] = {{-1, 0}, {1, 0}, {0, -1}, {-1, -1}, {1, 1}, {1, -1}, {-1, 1}};
            for (int k = 0; k < 7; k++) specs.push_back({dirs[k][0], dirs[k][1], MODE_SCRATCH, 2, pl[k], nullptr, nullptr});
            specs.push_back({0, 1, MODE_FINAL7, 3, pl[0], pl[1], pl[2]});
            xplanes[0] = pl[3]; xplanes[1] = pl[4]; xplanes[2] = pl[5]; xplanes[3] = pl[6];
        }
        for (const Spec &sp : specs) {
            BPass bp{};
            bp.P = base;
            bp.P.dx = sp.dx; bp.P.dy = sp.dy;
            bp.P.sc = sp.sc; bp.P.sc2 = sp.sc2; bp.P.sc3 = sp.sc3;
            for (int q = 0; q < 4; q++) bp.P.xpl[q] = xplanes[q];
            bp.P.nlines = lines_for(fd.W, fd.H, sp.dx, sp.dy);
            const bool pair = fdpl == 0 && pair_ok(fd.D);
            bp.frame = f; bp.mode = sp.mode; bp.dpl = pair ? 0 : dpl;
            const int pi = (int)passes.size();
            passes.push_back(bp);
            ring = std::max(ring, pair ? pair_ring_bytes(fd.D, sp.mode) : ring_bytes_for(dpl, sp.mode));
            const int warps = pair ? (bp.P.nlines + 1) / 2 : (bp.P.nlines + bp.P.gpw - 1) / bp.P.gpw;
            const int nit = (warps + b->wpb - 1) / b->wpb;
            for (int j = 0; j < nit; j++) by_phase[sp.phase].push_back({IT_PATH, f, sp.phase, pi, j * b->wpb});
            b->need[(size_t)f * MAXPH + sp.phase] += nit;
        }
    }
    if (b->stall_frame >= 0 && b->stall_frame < b->n) b->need[(size_t)b->stall_frame * MAXPH + 0] += 1;
    std::vector<BItem> items;
    for (auto &v : by_phase) items.insert(items.end(), v.begin(), v.end());
    b->n_items = (int)items.size();
    b->n_passes = (int)passes.size();
    b->ring_bytes = ring;
    // the census and cost tiles reuse the start of the block's path rings
    size_t smem = (size_t)ring * b->wpb;
    smem = std::max(smem, (size_t)std::max(tiles::CEN_SMEM, tiles::COST_SMEM));
    b->smem_bytes = smem;
    // one device allocation for all tables
    auto al = [](size_t v) { return (v + 255) & ~(size_t)255; };
    const size_t o_fr = 0, o_pa = o_fr + al(sizeof(BFrame) * b->n), o_it = o_pa + al(sizeof(BPass) * passes.size());
    const size_t o_dn = o_it + al(sizeof(BItem) * items.size()), o_nd = o_dn + al(sizeof(unsigned) * b->need.size());
    const size_t o_ct = o_nd + al(sizeof(unsigned) * b->need.size()), total = o_ct + al(sizeof(BCtl));
    cudaError_t e = cudaMalloc(&b->tables, total);
    if (e != cudaSuccess) { cudaGetLastError(); b->tables = nullptr; return berr(b, SGMGB_ERR_NOMEM, "batch tables"); }
    uint8_t *t = (uint8_t *)b->tables;
    b->d_frames = (BFrame *)(t + o_fr); b->d_passes = (BPass *)(t + o_pa); b->d_items = (BItem *)(t + o_it);
    b->d_done = (unsigned *)(t + o_dn); b->d_need = (unsigned *)(t + o_nd); b->d_ctl = (BCtl *)(t + o_ct);
    e = cudaMemcpy(b->d_passes, passes.data(), sizeof(BPass) * passes.size(), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(b->d_items, items.data(), sizeof(BItem) * items.size(), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(b->d_need, b->need.data(), sizeof(unsigned) * b->need.size(), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaFuncSetAttribute(k_batch, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    int per_sm = 0;
    if (e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_batch, 32 * b->wpb, smem);
    if (e != cudaSuccess) { cudaGetLastError(); return berr(b, SGMGB_ERR_CUDA, std::string("batch plan: ") + cudaGetErrorString(e)); }
    if (per_sm < 1) return berr(b, SGMGB_ERR_ARG, "batch shape does not fit on an SM");
    b->grid = per_sm * b->ctx->sm_count;
    return SGMGB_OK;
}

// Fills the pinned pointer table for these buffers.
void fill_frames(sgmgb_batch *b, const uint8_t *const *l, const uint8_t *const *r, uint8_t *const *d) {
    for (int f = 0; f < b->n; f++) {
        const FrameSlot &s = b->slots[f];
        BFrame &F = b->h_frames[f];
        F.left = l[f]; F.right = r[f]; F.disp = d[f];
        F.cl = s.cl; F.cr = s.cr; F.C = s.C;
        F.W = b->fds[f].W; F.H = b->fds[f].H; F.D = b->fds[f].D;
    }
}

int capture_graph(sgmgb_batch *b) {
    cudaError_t e = cudaStreamBeginCapture(b->cap, cudaStreamCaptureModeThreadLocal);
    if (e != cudaSuccess) { cudaGetLastError(); return berr(b, SGMGB_ERR_CUDA, "batch capture"); }
    const long long limit = (long long)b->wait_limit_ms * 1000000LL;   // ns of the global timer
    cudaMemcpyAsync(b->d_frames, b->h_frames, sizeof(BFrame) * b->n, cudaMemcpyHostToDevice, b->cap);
    cudaMemsetAsync(b->d_done, 0, sizeof(unsigned) * b->need.size(), b->cap);
    cudaMemcpyAsync(b->d_ctl, &b->h_ctl[0], sizeof(BCtl), cudaMemcpyHostToDevice, b->cap);
    k_batch<<<b->grid, 32 * b->wpb, b->smem_bytes, b->cap>>>(b->d_items, b->n_items, b->d_frames, b->d_passes,
                                                             b->d_done, b->d_need, b->d_ctl, b->ring_bytes, limit);
    cudaMemcpyAsync(&b->h_ctl[1], b->d_ctl, sizeof(BCtl), cudaMemcpyDeviceToHost, b->cap);
    cudaGraph_t g = nullptr;
    e = cudaStreamEndCapture(b->cap, &g);
    if (e == cudaSuccess) e = cudaGraphInstantiate(&b->graph, g, 0);
    if (g) cudaGraphDestroy(g);
    if (e != cudaSuccess) { cudaGetLastError(); b->graph = nullptr; return berr(b, SGMGB_ERR_CUDA, std::string("batch graph: ") + cudaGetErrorString(e)); }
    return SGMGB_OK;
}

void free_lanes(sgmgb_batch *b) {
    if (b->fgraph) { cudaGraphExecDestroy(b->fgraph); b->fgraph = nullptr; }
    b->fkey.clear();
    for (FrameSlot &c : b->chain) {
        for (auto &a : c.aux) if (a) cudaStreamDestroy(a);
        if (c.fork) cudaEventDestroy(c.fork);
        for (auto &j : c.join) if (j) cudaEventDestroy(j);
    }
    b->chain.clear();
    for (cudaStream_t s : b->chain_st) if (s) cudaStreamDestroy(s);
    b->chain_st.clear();
    for (cudaEvent_t e : b->lane_join) if (e) cudaEventDestroy(e);
    b->lane_join.clear();
    if (b->lane_fork) { cudaEventDestroy(b->lane_fork); b->lane_fork = nullptr; }
    b->lanes = 0;
}

// The streams and events of `lanes` chains (kept while the count stays).
int make_lanes(sgmgb_batch *b, int lanes) {
    if (b->lanes == lanes) return SGMGB_OK;
    free_lanes(b);
    b->chain.resize(lanes);
    b->chain_st.assign(lanes, nullptr);
    b->lane_join.assign(lanes, nullptr);
    b->lanes = lanes;
    cudaError_t e = cudaEventCreateWithFlags(&b->lane_fork, cudaEventDisableTiming);
    for (int k = 0; k < lanes && e == cudaSuccess; k++) {
        FrameSlot &c = b->chain[k];
        e = cudaStreamCreateWithFlags(&b->chain_st[k], cudaStreamNonBlocking);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&b->lane_join[k], cudaEventDisableTiming);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&c.fork, cudaEventDisableTiming);
        for (int i = 0; i < FrameSlot::kAux && e == cudaSuccess; i++) {
            e = cudaStreamCreateWithFlags(&c.aux[i], cudaStreamNonBlocking);
            if (e == cudaSuccess) e = cudaEventCreateWithFlags(&c.join[i], cudaEventDisableTiming);
        }
    }
    if (e != cudaSuccess) {
        cudaGetLastError();
        free_lanes(b);
        return berr(b, SGMGB_ERR_CUDA, std::string("batch lanes: ") + cudaGetErrorString(e));
    }
    return SGMGB_OK;
}

// Captures the frames-in-flight run on these buffers: a fork from the
// capture stream to every chain, each frame's pipeline (enqueue_frame, as
// sgmgb_run_frame_async with frames in flight runs it) on its chain, and the
// chains' joins.
int capture_lanes(sgmgb_batch *b, const uint8_t *const *dl, const uint8_t *const *dr, uint8_t *const *dd) {
    if (b->fgraph) {
        if (b->ran) cudaEventSynchronize(b->done_ev);   // the graph may be running
        cudaGraphExecDestroy(b->fgraph);
        b->fgraph = nullptr;
    }
    b->fkey.clear();
    cudaError_t e = cudaStreamBeginCapture(b->cap, cudaStreamCaptureModeThreadLocal);
    if (e != cudaSuccess) { cudaGetLastError(); return berr(b, SGMGB_ERR_CUDA, "batch capture"); }
    e = cudaEventRecord(b->lane_fork, b->cap);
    for (int k = 0; k < b->lanes && e == cudaSuccess; k++) e = cudaStreamWaitEvent(b->chain_st[k], b->lane_fork, 0);
    PathShape sh;
    sh.sched = SGMGB_SCHED_FUSED;                     // the throughput schedule where it does not apply
    // chains of about equal work: frames largest first, each onto the chain
    // with the least work so far (work ~ W*H*D, 8 paths counted 1.8 times)
    std::vector<int> order(b->n);
    std::vector<double> work(b->n), load(b->lanes, 0.0);
    for (int f = 0; f < b->n; f++) {
        const sgmgb_frame_desc &fd = b->fds[f];
        order[f] = f;
        work[f] = (double)fd.W * fd.H * fd.D * (fd.paths == 8 ? 1.8 : 1.0);
    }
    std::stable_sort(order.begin(), order.end(), [&](int a, int c) { return work[a] > work[c]; });
    for (int f : order) {
        if (e != cudaSuccess) break;
        const int k = (int)(std::min_element(load.begin(), load.end()) - load.begin());
        load[k] += work[f];
        FrameSlot v = b->slots[f];                    // the frame's buffers, its chain's streams
        const FrameSlot &c = b->chain[k];
        std::copy(c.aux, c.aux + FrameSlot::kAux, v.aux);
        std::copy(c.join, c.join + FrameSlot::kAux, v.join);
        v.fork = c.fork;
        e = enqueue_frame(v, dl[f], dr[f], dd[f], b->chain_st[k], sh, nullptr, nullptr);
    }
    for (int k = 0; k < b->lanes && e == cudaSuccess; k++) {
        e = cudaEventRecord(b->lane_join[k], b->chain_st[k]);
        if (e == cudaSuccess) e = cudaStreamWaitEvent(b->cap, b->lane_join[k], 0);
    }
    cudaGraph_t g = nullptr;
    const cudaError_t ee = cudaStreamEndCapture(b->cap, &g);
    if (e == cudaSuccess) e = ee;
    if (e == cudaSuccess) e = cudaGraphInstantiate(&b->fgraph, g, 0);
    if (g) cudaGraphDestroy(g);
    if (e != cudaSuccess) {
        cudaGetLastError();
        b->fgraph = nullptr;
        return berr(b, SGMGB_ERR_CUDA, std::string("batch frames graph: ") + cudaGetErrorString(e));
    }
    for (int f = 0; f < b->n; f++) {
        b->fkey.push_back(dl[f]);
        b->fkey.push_back(dr[f]);
        b->fkey.push_back(dd[f]);
    }
    return SGMGB_OK;
}

bool same_key(const sgmgb_batch *b, const uint8_t *const *dl, const uint8_t *const *dr, uint8_t *const *dd) {
    if (b->fkey.size() != (size_t)3 * b->n) return false;
    for (int f = 0; f < b->n; f++)
        if (b->fkey[3 * f] != dl[f] || b->fkey[3 * f + 1] != dr[f] || b->fkey[3 * f + 2] != dd[f]) return false;
    return true;
}

}  // namespace

extern "C" {

int sgmgb_batch_create(sgmgb_ctx *ctx, const sgmgb_frame_desc *frames, int n, const char *tune_cache,
                       sgmgb_batch **out) {
    if (!ctx || !frames || n < 1 || !out) return SGMGB_ERR_ARG;
    *out = nullptr;
    for (int f = 0; f < n; f++) {
        if (sgmgb_check_desc(&frames[f]) != SGMGB_OK)
            return set_err(ctx, SGMGB_ERR_ARG, "batch frame " + std::to_string(f) + ": invalid description");
        if (frames[f].variant != SGMGB_PLAIN)
            return set_err(ctx, SGMGB_ERR_ARG, "batch frame " + std::to_string(f) + ": batches run the plain variant");
    }
    sgmgb_batch *b = new (std::nothrow) sgmgb_batch();
    if (!b) return SGMGB_ERR_NOMEM;
    b->ctx = ctx;
    b->n = n;
    b->fds.assign(frames, frames + n);
    b->dpl.resize(n);
    size_t biggest = 0;
    for (int f = 0; f < n; f++) {
        const sgmgb_frame_desc &fd = frames[f];
        int w = 0, d = 0;
        const bool hit = tune_cache && sgmgb_tune_lookup(tune_cache, &fd, &w, &d) == SGMGB_OK;
        b->dpl[f] = hit && d ? path_dpl(fd.D, d) : 0;
        const size_t sz = (size_t)fd.W * fd.H * fd.D;
        if (hit && sz > biggest) { biggest = sz; b->wpb = w; }
    }
    cudaSetDevice(ctx->device);
    b->slots.resize(n);
    std::vector<size_t> off(n);
    size_t total = 0;
    for (int f = 0; f < n; f++) { off[f] = total; total += (slot_layout(b->fds[f], nullptr) + 255) & ~(size_t)255; }
    cudaError_t e = cudaMalloc(&b->arena, total);
    if (e != cudaSuccess) {
        cudaGetLastError();
        b->arena = nullptr;
        sgmgb_batch_destroy(b);
        return set_err(ctx, SGMGB_ERR_NOMEM, "batch workspace of " + std::to_string(total) + " bytes");
    }
    b->arena_bytes = total;
    for (int f = 0; f < n; f++) {
        b->slots[f].fd = b->fds[f];
        b->slots[f].base = (uint8_t *)b->arena + off[f];
        slot_layout(b->fds[f], &b->slots[f]);
    }
    e = cudaHostAlloc((void **)&b->h_frames, sizeof(BFrame) * n, cudaHostAllocDefault);
    if (e == cudaSuccess) e = cudaHostAlloc((void **)&b->h_ctl, sizeof(BCtl) * 2, cudaHostAllocDefault);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&b->cap, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&b->done_ev, cudaEventDisableTiming);
    if (e != cudaSuccess) {
        cudaGetLastError();
        sgmgb_batch_destroy(b);
        return set_err(ctx, SGMGB_ERR_CUDA, std::string("batch setup: ") + cudaGetErrorString(e));
    }
    memset(b->h_frames, 0, sizeof(BFrame) * n);
    b->h_ctl[0] = BCtl{0u, 0u, -1, 0u};
    b->h_ctl[1] = BCtl{0u, 0u, -1, 0u};
    const int rc = build_plan(b);
    if (rc) { sgmgb_batch_destroy(b); return rc; }
    *out = b;
    return SGMGB_OK;
}

int sgmgb_batch_run(sgmgb_batch *b, const uint8_t *const *d_left, const uint8_t *const *d_right,
                    uint8_t *const *d_disp, void *stream) {
    if (!b || !d_left || !d_right || !d_disp) return SGMGB_ERR_ARG;
    for (int f = 0; f < b->n; f++)
        if (!d_left[f] || !d_right[f] || !d_disp[f]) return berr(b, SGMGB_ERR_ARG, "batch frame " + std::to_string(f) + ": null buffer");
    cudaSetDevice(b->ctx->device);
    cudaStream_t st = stream ? (cudaStream_t)stream : b->ctx->stream;
    cudaError_t e;
    if (b->mode == SGMGB_BATCH_IN_FLIGHT) {
        if (!b->fgraph || !same_key(b, d_left, d_right, d_disp)) {
            const int rc = capture_lanes(b, d_left, d_right, d_disp);
            if (rc) return rc;
        }
        e = cudaGraphLaunch(b->fgraph, st);
        b->last_persistent = false;
    } else {
        if (b->ran) cudaEventSynchronize(b->done_ev);   // the pinned table is read by the previous run
        fill_frames(b, d_left, d_right, d_disp);
        if (!b->graph) {
            const int rc = capture_graph(b);
            if (rc) return rc;
        }
        e = cudaGraphLaunch(b->graph, st);
        b->last_persistent = b->ran_persistent = true;
    }
    if (e == cudaSuccess) e = cudaEventRecord(b->done_ev, st);
    if (e != cudaSuccess) { cudaGetLastError(); return berr(b, SGMGB_ERR_CUDA, std::string("batch launch: ") + cudaGetErrorString(e)); }
    b->ran = true;
    return SGMGB_OK;
}

int sgmgb_batch_wait(sgmgb_batch *b) {
    if (!b) return SGMGB_ERR_ARG;
    if (!b->ran) return SGMGB_OK;
    cudaSetDevice(b->ctx->device);
    cudaError_t e = cudaEventSynchronize(b->done_ev);
    if (e != cudaSuccess) { cudaGetLastError(); return berr(b, SGMGB_ERR_CUDA, std::string("batch run: ") + cudaGetErrorString(e)); }
    if (b->last_persistent && b->h_ctl[1].err_item != -1)
        return berr(b, SGMGB_ERR_TIMEOUT, "batch item " + std::to_string(b->h_ctl[1].err_item) + " waited past " +
                                              std::to_string(b->wait_limit_ms) + " ms for its inputs; run abandoned");
    return SGMGB_OK;
}

int sgmgb_batch_autotune(sgmgb_batch *b, const uint8_t *const *d_left, const uint8_t *const *d_right,
                         uint8_t *const *d_disp, const char *tune_cache) {
    if (!b) return SGMGB_ERR_ARG;
    cudaSetDevice(b->ctx->device);
    const int saved_wpb = b->wpb, saved_mode = b->mode, saved_lanes = b->lanes;
    const std::vector<int> saved_dpl = b->dpl;
    cudaEvent_t t0 = nullptr, t1 = nullptr;
    if (cudaEventCreate(&t0) != cudaSuccess || cudaEventCreate(&t1) != cudaSuccess) {
        cudaGetLastError();
        if (t0) cudaEventDestroy(t0);
        return berr(b, SGMGB_ERR_CUDA, "autotune events");
    }
    // one untimed run (capture, warm-up), then the best of three on the context's stream
    auto time_runs = [&](float *ms) -> int {
        int r;
        if ((r = sgmgb_batch_run(b, d_left, d_right, d_disp, nullptr)) || (r = sgmgb_batch_wait(b))) return r;
        *ms = 1e30f;
        for (int rep = 0; rep < 3; rep++) {
            cudaEventRecord(t0, b->ctx->stream);
            if ((r = sgmgb_batch_run(b, d_left, d_right, d_disp, nullptr))) return r;
            cudaEventRecord(t1, b->ctx->stream);
            if ((r = sgmgb_batch_wait(b))) return r;
            float t = 0.f;
            cudaEventElapsedTime(&t, t0, t1);
            *ms = std::min(*ms, t);
        }
        return SGMGB_OK;
    };
    float best = -1.f, best_flight = -1.f;
    int best_w = saved_wpb, best_m = 0, best_lanes = 0, rc = SGMGB_OK;
    auto shape_of = [&](int f, int m) {   // m = 0: pair layout; 1, 2: smallest valid and twice that
        return m ? path_dpl(b->fds[f].D, std::min(8, path_dpl(b->fds[f].D, 0) * m)) : 0;
    };
    b->mode = SGMGB_BATCH_PERSISTENT;
    for (int w : {2, 4}) {
        for (int m : {0, 1, 2}) {
            if (rc) break;
            b->wpb = w;
            for (int f = 0; f < b->n; f++) b->dpl[f] = shape_of(f, m);
            float ms = 0.f;
            if ((rc = build_plan(b)) || (rc = time_runs(&ms))) break;
            if (best < 0.f || ms < best) { best = ms; best_w = w; best_m = m; }
        }
    }
    if (!rc) {
        b->wpb = best_w;
        for (int f = 0; f < b->n; f++) b->dpl[f] = shape_of(f, best_m);
        rc = build_plan(b);
    }
    // frames in flight (shapes of their own: the persistent launch's do not apply)
    b->mode = SGMGB_BATCH_IN_FLIGHT;
    for (int lanes : {4, 6, 8}) {
        if (rc) break;
        float ms = 0.f;
        if ((rc = make_lanes(b, lanes)) || (rc = time_runs(&ms))) break;
        if (best_flight < 0.f || ms < best_flight) { best_flight = ms; best_lanes = lanes; }
    }
    cudaEventDestroy(t0);
    cudaEventDestroy(t1);
    if (rc) {
        b->wpb = saved_wpb;
        b->dpl = saved_dpl;
        build_plan(b);
        b->mode = saved_mode;
        if (saved_mode == SGMGB_BATCH_IN_FLIGHT) make_lanes(b, saved_lanes);
        return rc;
    }
    if (best_flight < best) {
        b->mode = SGMGB_BATCH_IN_FLIGHT;
        if ((rc = make_lanes(b, best_lanes))) return rc;
    } else {
        b->mode = SGMGB_BATCH_PERSISTENT;
    }
    if (tune_cache) {
        for (int f = 0; f < b->n; f++) {
            bool seen = false;
            for (int g = 0; g < f && !seen; g++) seen = !memcmp(&b->fds[g], &b->fds[f], sizeof(sgmgb_frame_desc));
            if (!seen && sgmgb_tune_record(tune_cache, &b->fds[f], b->wpb, b->dpl[f], 1000.0 * best) != SGMGB_OK)
                return berr(b, SGMGB_ERR_STATE, std::string("cannot append to tune cache ") + tune_cache);
        }
    }
    return SGMGB_OK;
}

int sgmgb_batch_busy(sgmgb_batch *b, double *ms, int n, int *blocks) {
    if (!b || !ms || n < 1) return SGMGB_ERR_ARG;
    if (!b->ran_persistent) return berr(b, SGMGB_ERR_STATE, "the persistent launch has not run");
    cudaSetDevice(b->ctx->device);
    if (cudaEventSynchronize(b->done_ev) != cudaSuccess) {
        cudaGetLastError();
        return berr(b, SGMGB_ERR_CUDA, "batch run");
    }
    for (int k = 0; k < n; k++) ms[k] = k < BK_N ? (double)b->h_ctl[1].busy[k] * 1e-6 : 0.0;
    if (blocks) *blocks = b->grid;
    return SGMGB_OK;
}

int sgmgb_batch_tile_shape(const sgmgb_batch *b, int i, int *warps_per_block, int *disp_per_lane) {
    if (!b || i < 0 || i >= b->n) return SGMGB_ERR_ARG;
    if (warps_per_block) *warps_per_block = b->wpb;
    if (disp_per_lane) *disp_per_lane = b->dpl[i];
    return SGMGB_OK;
}

int sgmgb_batch_set_mode(sgmgb_batch *b, int mode, int lanes) {
    if (!b || (mode != SGMGB_BATCH_PERSISTENT && mode != SGMGB_BATCH_IN_FLIGHT)) return SGMGB_ERR_ARG;
    if (mode == SGMGB_BATCH_IN_FLIGHT && (lanes < 1 || lanes > 8)) return SGMGB_ERR_ARG;
    cudaSetDevice(b->ctx->device);
    if (mode == SGMGB_BATCH_IN_FLIGHT && lanes != b->lanes) {
        if (b->ran) cudaEventSynchronize(b->done_ev);  // the frames graph may be running
        const int rc = make_lanes(b, lanes);
        if (rc) return rc;
    }
    b->mode = mode;
    return SGMGB_OK;
}

int sgmgb_batch_mode(const sgmgb_batch *b, int *mode, int *lanes) {
    if (!b) return SGMGB_ERR_ARG;
    if (mode) *mode = b->mode;
    if (lanes) *lanes = b->mode == SGMGB_BATCH_IN_FLIGHT ? b->lanes : 0;
    return SGMGB_OK;
}

int sgmgb_batch_set_fault(sgmgb_batch *b, int wait_limit_ms, int stall_frame) {
    if (!b || wait_limit_ms < 1 || wait_limit_ms > 600000 || stall_frame < -1 || stall_frame >= b->n)
        return SGMGB_ERR_ARG;
    b->wait_limit_ms = wait_limit_ms;
    b->stall_frame = stall_frame;
    return build_plan(b);
}

void sgmgb_batch_destroy(sgmgb_batch *b) {
    if (!b) return;
    if (b->ctx) cudaSetDevice(b->ctx->device);
    if (b->ran && b->done_ev) cudaEventSynchronize(b->done_ev);
    free_tables(b);
    free_lanes(b);
    if (b->arena) cudaFree(b->arena);
    if (b->h_frames) cudaFreeHost(b->h_frames);
    if (b->h_ctl) cudaFreeHost(b->h_ctl);
    if (b->cap) cudaStreamDestroy(b->cap);
    if (b->done_ev) cudaEventDestroy(b->done_ev);
    delete b;
}

}  // extern "C"
