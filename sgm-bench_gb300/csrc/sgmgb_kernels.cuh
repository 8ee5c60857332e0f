// sgmgb_kernels.cuh -- device kernels of the GB300 SGM engine and their launchers.
//
// The semantics are those of kylefoxaustin/sgm-bench (common/sgm_params.h:44-59,
// common/sgm_ref.c, multiscale/sgm_ms_ref.c); the shapes are this engine's own.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace sgmgb {

// How the cost of one (pixel, d) is formed.
enum CostKind : int {
    COST_PLAIN = 0,   // popcount(cl ^ cr), invalid 62              (common/sgm_ref.c:44-56)
    COST_MS1   = 1,   // popcount(cl ^ cr), invalid 63, half scale  (multiscale/sgm_ms_ref.c:66-72)
    COST_MS2   = 2    // (full + half(x/2,y/2,d/2) + 1) >> 1         (multiscale/sgm_ms_ref.c:184-188)
};

// What a path pass does with its L(p,d) at every pixel it visits. Directions
// are run in opposite-direction pairs: the first of a pair parks its L in a
// uint8 scratch plane, the second adds both into the uint16 sum S.
enum PassMode : int {
    MODE_SCRATCH = 0,   // sc = L
    MODE_STORE   = 1,   // S  = sc + L           (first pair: no memset of S)
    MODE_ACCUM   = 2,   // S += sc + L
    MODE_FINAL   = 3    // argmin_d(S + sc + L) -> disp, lowest d on ties
};

struct LineParams {
    const uint64_t *cl, *cr;     // census descriptors at this scale, W*H
    const uint64_t *cl1, *cr1;   // half-scale descriptors (COST_MS2 only), (W/2)*(H/2)
    uint8_t  *sc;                // W*H*D scratch L
    uint16_t *S;                 // W*H*D sum
    uint8_t  *disp;              // MODE_FINAL output
    int W, H, D;
    int nl;                      // active lanes: D / DPL
    int dx, dy;                  // direction of travel
    int p1, p2;                  // penalties
    int nlines;                  // independent lines for this direction
    int even_only;               // MODE_FINAL: argmin only at even (x,y) into a (W/2)x(H/2) map
};

// Disparities per lane for a disparity range: the smallest even count that
// divides D and needs at most 32 lanes.
inline int dpl_for(int D) {
    for (int dpl = 2; dpl <= 8; dpl += 2)
        if (D % dpl == 0 && D / dpl <= 32) return dpl;
    return 0;
}

// Number of independent lines a direction decomposes the image into.
inline int lines_for(int W, int H, int dx, int dy) {
    if (dy == 0) return H;
    if (dx == 0) return W;
    return W + H - 1;
}

// ---- launchers (all enqueue on `s`, none synchronises) ----
cudaError_t launch_census2(const uint8_t *im0, const uint8_t *im1, uint64_t *out0, uint64_t *out1,
                           int W, int H, cudaStream_t s);
cudaError_t launch_sobel2(const uint8_t *im0, const uint8_t *im1, uint8_t *out0, uint8_t *out1,
                          int W, int H, cudaStream_t s);
cudaError_t launch_half2(const uint8_t *im0, const uint8_t *im1, uint8_t *out0, uint8_t *out1,
                         int W, int H, cudaStream_t s);
cudaError_t launch_line(const LineParams &p, int mode, int cost_kind, int saturate,
                        int warps_per_block, cudaStream_t s);

}  // namespace sgmgb
