// sgmgb_kernels.cuh -- device kernels of the GB300 SGM engine and their launchers.
//
// The semantics are those of kylefoxaustin/sgm-bench (common/sgm_params.h:44-59,
// common/sgm_ref.c, multiscale/sgm_ms_ref.c); the shapes are this engine's own.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace sgmgb {

// Invalid-disparity cost (x - d < 0) of each variant: 62 in the plain method
// (common/sgm_params.h:27-29), 63 in the multi-scale one (multiscale/sgm_ms_ref.c:41).
constexpr int kInvalidPlain = 62, kInvalidMultiscale = 63;

// What a path pass does with its L(p,d) at every pixel it visits.
enum PassMode : int {
    MODE_SCRATCH = 0,   // sc = L
    MODE_STORE   = 1,   // S  = sc + L           (first pair: no memset of S)
    MODE_ACCUM   = 2,   // S += sc + L
    MODE_FINAL   = 3,   // argmin_d(S + sc + L) -> disp, lowest d on ties
    MODE_FINAL3  = 4,   // argmin_d(sc + sc2 + sc3 + L) -> disp: three other directions' planes
    MODE_FINAL7  = 5,   // argmin_d(L + the seven planes sc, sc2, sc3, xpl[0..3]) -> disp (8 paths)
    MODE_FINAL3H = 6    // MODE_FINAL3 along rows (pair layout only): a chunk's disparities of a row
                        // are gathered in registers and leave in one store per row and chunk
};

struct LineParams {
    const uint8_t *C;            // cost volume at this scale, W*H*D
    uint8_t  *sc;                // W*H*D scratch L (written by SCRATCH, read otherwise)
    const uint8_t *sc2, *sc3;    // MODE_FINAL3 / FINAL7: the second and third planes
    const uint8_t *xpl[4];       // MODE_FINAL7: planes four to seven
    uint16_t *S;                 // W*H*D sum
    uint8_t  *disp;              // final passes' output
    int W, H, D;
    int nl;                      // lanes of a line that hold disparities: D / DPL (set by launch_line)
    int lpl, gpw;                // lanes per line, lines per warp (set by launch_line)
    int dx, dy;                  // direction of travel
    int p1, p2;                  // penalties
    int nlines;                  // independent lines for this direction
    int even_only;               // multi-scale full scale: only lines through even (x, y) (nlines from
                                 // lines_for_even), SCRATCH stores and final argmins only at even (x, y),
                                 // the planes compact (pixel (x, y) at (y/2)(W/2) + x/2; SCRATCH and
                                 // FINAL7 only),
                                 // the map (W/2)x(H/2)
    int key16;                   // final: S*64 + d fits 16 bits (4 paths, D <= 64)
    int dpl;                     // disparities per lane: 2, 4 or 8; 0 picks the smallest valid
    // split horizontal lines (the fused schedule): hseg 1 walks the first half
    // of each row (L->R x in [0, W/2), R->L x in [W/2, W)), hseg 2 the second
    // half (L->R [W/2, W), R->L [0, W/2)); 0 the whole line.
    int hseg;
    const uint64_t *cl, *cr;     // census descriptors (the first-half pass computes its costs from them)
    uint32_t *state;             // per warp and lane: L and min at the end of the first half
};

// Disparities per lane of the path kernel: `want` (0, 2, 4 or 8) raised to
// the smallest value that fits a line in one warp (D/DPL <= 32 lanes: 2 up to
// D = 64, 4 up to 128, 8 up to 256); 0 for an invalid D or want. A line takes
// D/DPL lanes and a warp 32/(D/DPL) lines when that divides 32.
int path_dpl(int D, int want);

// Number of independent lines a direction decomposes the image into.
inline int lines_for(int W, int H, int dx, int dy) {
    if (dy == 0) return H;
    if (dx == 0) return W;
    return W + H - 1;
}

// The same with LineParams::even_only (W and H even): the lines that cross a
// pixel with x and y both even -- even rows, even columns, or the diagonals
// with x + y even, counted over the entry rows and then the entry columns.
inline int lines_for_even(int W, int H, int dx, int dy) {
    if (dy == 0) return (H + 1) / 2;
    if (dx == 0) return (W + 1) / 2;
    const int xe = dx > 0 ? 0 : W - 1, ye = dy > 0 ? 0 : H - 1;
    const int n1 = (H - (xe & 1) + 1) / 2;
    const int m0 = ((xe + ye) & 1) ? 1 : 2;          // first entry column offset with xe + m + ye even
    const int n2 = W - 1 >= m0 ? (W - 1 - m0) / 2 + 1 : 0;
    return n1 + n2;
}

// Words of line state the first half of a split horizontal pass leaves for
// the second half: per direction, row pair and lane, the NR packed L
// registers and the packed minimum (NR = D/32, at most 4).
inline size_t hstate_words(int H) { return (size_t)2 * ((H + 1) / 2) * 32 * 5; }

// ---- launchers (all enqueue on `s`, none synchronises) ----
cudaError_t launch_census2(const uint8_t *im0, const uint8_t *im1, uint64_t *out0, uint64_t *out1,
                           int W, int H, cudaStream_t s);
cudaError_t launch_sobel2(const uint8_t *im0, const uint8_t *im1, uint8_t *out0, uint8_t *out1,
                          int W, int H, cudaStream_t s);
cudaError_t launch_half2(const uint8_t *im0, const uint8_t *im1, uint8_t *out0, uint8_t *out1,
                         int W, int H, cudaStream_t s);
// Cost volume (uint8, W*H*D) from census descriptors; C1 != NULL makes the
// multi-scale full-scale cost averaged with the half-scale volume C1.
cudaError_t launch_cost(const uint64_t *cl, const uint64_t *cr, uint8_t *C, const uint8_t *C1,
                        int W, int H, int D, int invalid, cudaStream_t s);
// Sets the kernels' shared-memory limits and carve-out; call once per device
// before the first launch (and outside stream capture). The census, cost,
// prefilter and path kernels ask for the same carve-out (the largest
// shared-memory share), so the side-by-side passes of a frame, and frames in
// flight, can share an SM: kernels that need different L1/shared splits
// cannot (measured: 4 frames in flight 0.305 -> 0.294 ms per frame). The sum
// pass runs alone after the join and streams through L1: it keeps the
// default (the largest shared share measured 90 -> 98 us at 1080p D=64).
cudaError_t prepare_path_kernels();
cudaError_t prepare_frame_kernels();   // census, cost, prefilters (sgmgb_kernels.cu)
template <typename K>
inline cudaError_t set_carveout(K *kernel) {
    return cudaFuncSetAttribute(kernel, cudaFuncAttributePreferredSharedMemoryCarveout,
                                (int)cudaSharedmemCarveoutMaxShared);
}
// One direction's path pass over the cost volume p.C (sgmgb_path.cu).
// saturate: clamp L to 255 (multi-scale). warps_per_block in 1..4.
cudaError_t launch_line(const LineParams &p, int mode, int saturate, int warps_per_block, cudaStream_t s);

// The first half of both horizontal passes of the fused schedule
// (sgmgb_fused.cu): per row pair and direction, the Hamming costs of the half
// row from p.cl / p.cr (stored into p.C), the recurrence (L into the plane
// p.sc) and the line state at the half's end into p.state. D = 32, 64 or 128,
// plain variant. warps_per_block in 1..4.
cudaError_t launch_hcost(const LineParams &p, int warps_per_block, cudaStream_t s);
cudaError_t prepare_fused_kernels();

// Planes of one frame's directions, each W*H*D uint8 in the cost volume's
// layout (16-byte aligned).
struct SumPlanes { const uint8_t *p[8]; };
// disp = argmin_d of the sum of the np (4 or 8) planes, lowest d on ties;
// even_only: at even (x, y) only, from compact planes, into a (W/2)x(H/2) map (sgmgb_sum.cu).
cudaError_t launch_sum(const SumPlanes &pl, int np, uint8_t *disp, int W, int H, int D, int even_only,
                       cudaStream_t s);

}  // namespace sgmgb
