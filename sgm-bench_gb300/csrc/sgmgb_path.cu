// sgmgb_path.cu -- the per-pass path kernel and its launchers (one launch per
// direction); the recurrence itself is in sgmgb_path.cuh.
#include "sgmgb_path.cuh"
#include "sgmgb_pair.cuh"

namespace sgmgb {

template <int DPL, int MODE, int SAT, bool KEY16, bool EO = false>
__global__ void __launch_bounds__(128)
k_path(const LineParams P) {
    extern __shared__ __align__(16) uint8_t smem[];
    const int wib = threadIdx.x >> 5;
    path_warp<DPL, MODE, SAT, KEY16, EO>(P, blockIdx.x * (blockDim.x >> 5) + wib,
                                         smem + wib * Slot<DPL, MODE>::RING);
}

template <int NR, int MODE, int SAT, bool KEY16>
__global__ void __launch_bounds__(128)
k_pair(const LineParams P) {
    extern __shared__ __align__(16) uint8_t smem[];
    const int wib = threadIdx.x >> 5;
    path_pair<NR, MODE, SAT, KEY16>(P, blockIdx.x * (blockDim.x >> 5) + wib, smem + wib * PairSlot<NR, MODE>::RING);
}

// ---------------------------------------------------------------------------
template <int NR, int MODE, int SAT, bool KEY16>
static cudaError_t prep_pair() {
    cudaError_t e = cudaFuncSetAttribute(k_pair<NR, MODE, SAT, KEY16>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         4 * PairSlot<NR, MODE>::RING);
    if (e == cudaSuccess) e = set_carveout(k_pair<NR, MODE, SAT, KEY16>);
    return e;
}

template <int NR, int SAT>
static cudaError_t prep_pair_modes() {
    cudaError_t e;
    if ((e = prep_pair<NR, MODE_SCRATCH, SAT, false>()) != cudaSuccess) return e;
    if ((e = prep_pair<NR, MODE_STORE, SAT, false>()) != cudaSuccess) return e;
    if ((e = prep_pair<NR, MODE_ACCUM, SAT, false>()) != cudaSuccess) return e;
    if ((e = prep_pair<NR, MODE_FINAL7, SAT, false>()) != cudaSuccess) return e;
    return prep_pair<NR, MODE_FINAL, SAT, false>();
}

template <int NR, int MODE, int SAT, bool KEY16>
static cudaError_t launch_pair_one(const LineParams &p, int wpb, cudaStream_t s) {
    const int warps = (p.nlines + 1) / 2;
    const dim3 b(32 * wpb), g((warps + wpb - 1) / wpb);
    k_pair<NR, MODE, SAT, KEY16><<<g, b, wpb * PairSlot<NR, MODE>::RING, s>>>(p);
    return cudaGetLastError();
}

// The pair layout (two lines per warp in register halves, sgmgb_pair.cuh)
// serves the scratch passes and the eight-plane final at D = 32, 64 and 128
// (the multi-scale ones, saturating, at D = 64) and the plain three-plane
// finals, unless a disparities-per-lane shape was asked for. Alone, a pair
// pass is slower (half the warps: multi-scale full-scale R->L 57 -> 70 us);
// side by side with the other directions its halved instruction count wins
// (configuration C with 4 frames in flight 0.578 -> 0.535 ms). The
// multi-scale full scale's final keeps one line per warp: its even columns
// give a pair final only 480 warps at 1080p (226 against 147 us alone, and
// 0.494 against 0.485 ms per frame with four in flight), and it skips its odd
// rows' argmins (k_path's EO variant). The batch kernel may choose it for any
// mode.
static bool pair_applies(const LineParams &p, int mode, int saturate) {
    if (p.dpl != 0 || (p.D != 32 && p.D != 64 && p.D != 128)) return false;
    if (p.even_only && mode != MODE_SCRATCH) return false;   // its finals read the planes in the full layout
    if (mode == MODE_SCRATCH || mode == MODE_FINAL7) return !saturate || p.D == 64;   // saturating: D = 64
    return (mode == MODE_FINAL3 || mode == MODE_FINAL3H) && !saturate;
}

template <int NR, int SAT>
static cudaError_t launch_pair_nr(const LineParams &p, int mode, int wpb, cudaStream_t s) {
    switch (mode) {
    case MODE_SCRATCH: return launch_pair_one<NR, MODE_SCRATCH, SAT, false>(p, wpb, s);
    case MODE_STORE:   return launch_pair_one<NR, MODE_STORE, SAT, false>(p, wpb, s);
    case MODE_ACCUM:   return launch_pair_one<NR, MODE_ACCUM, SAT, false>(p, wpb, s);
    case MODE_FINAL:   return launch_pair_one<NR, MODE_FINAL, SAT, false>(p, wpb, s);
    case MODE_FINAL7:  return launch_pair_one<NR, MODE_FINAL7, SAT, false>(p, wpb, s);
    default:           return cudaErrorInvalidValue;
    }
}

static cudaError_t launch_pair(const LineParams &p, int mode, int saturate, int wpb, cudaStream_t s) {
    if (saturate) return mode == MODE_FINAL3 ? cudaErrorInvalidValue : launch_pair_nr<2, 1>(p, mode, wpb, s);
    const bool key16 = p.key16 != 0 && p.D <= 64;
    if (mode == MODE_FINAL3) {
        switch (p.D) {
        case 32: return key16 ? launch_pair_one<1, MODE_FINAL3, 0, true>(p, wpb, s)
                              : launch_pair_one<1, MODE_FINAL3, 0, false>(p, wpb, s);
        case 64: return key16 ? launch_pair_one<2, MODE_FINAL3, 0, true>(p, wpb, s)
                              : launch_pair_one<2, MODE_FINAL3, 0, false>(p, wpb, s);
        default: return launch_pair_one<4, MODE_FINAL3, 0, false>(p, wpb, s);
        }
    }
    if (mode == MODE_FINAL3H) {                       // rows only (the fused schedule's second halves)
        if (p.dy != 0) return cudaErrorInvalidValue;
        switch (p.D) {
        case 32: return launch_pair_one<1, MODE_FINAL3H, 0, true>(p, wpb, s);
        case 64: return launch_pair_one<2, MODE_FINAL3H, 0, true>(p, wpb, s);
        default: return launch_pair_one<4, MODE_FINAL3H, 0, false>(p, wpb, s);
        }
    }
    switch (p.D) {
    case 32: return launch_pair_nr<1, 0>(p, mode, wpb, s);
    case 64: return launch_pair_nr<2, 0>(p, mode, wpb, s);
    default: return launch_pair_nr<4, 0>(p, mode, wpb, s);
    }
}

template <int DPL, int MODE, int SAT, bool KEY16, bool EO = false>
static cudaError_t prep_one() {
    cudaError_t e = cudaFuncSetAttribute(k_path<DPL, MODE, SAT, KEY16, EO>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, 4 * Slot<DPL, MODE>::RING);
    if (e == cudaSuccess) e = set_carveout(k_path<DPL, MODE, SAT, KEY16, EO>);
    return e;
}

template <int DPL, int SAT, bool KEY16>
static cudaError_t prep_dpl() {
    cudaError_t e;
    if ((e = prep_one<DPL, MODE_SCRATCH, SAT, false>()) != cudaSuccess) return e;
    if ((e = prep_one<DPL, MODE_STORE, SAT, false>()) != cudaSuccess) return e;
    if ((e = prep_one<DPL, MODE_ACCUM, SAT, false>()) != cudaSuccess) return e;
    if ((e = prep_one<DPL, MODE_FINAL, SAT, false>()) != cudaSuccess) return e;
    if ((e = prep_one<DPL, MODE_FINAL7, SAT, false>()) != cudaSuccess) return e;
    return prep_one<DPL, MODE_FINAL3, SAT, KEY16>();
}

cudaError_t prepare_path_kernels() {
    cudaError_t e;
    if ((e = prepare_frame_kernels()) != cudaSuccess) return e;
    if ((e = prepare_fused_kernels()) != cudaSuccess) return e;
    if ((e = prep_pair_modes<1, 0>()) != cudaSuccess) return e;
    if ((e = prep_pair_modes<2, 0>()) != cudaSuccess) return e;
    if ((e = prep_pair_modes<4, 0>()) != cudaSuccess) return e;
    if ((e = prep_pair_modes<2, 1>()) != cudaSuccess) return e;
    if ((e = prep_pair<1, MODE_FINAL3, 0, true>()) != cudaSuccess) return e;
    if ((e = prep_pair<1, MODE_FINAL3, 0, false>()) != cudaSuccess) return e;
    if ((e = prep_pair<2, MODE_FINAL3, 0, true>()) != cudaSuccess) return e;
    if ((e = prep_pair<2, MODE_FINAL3, 0, false>()) != cudaSuccess) return e;
    if ((e = prep_pair<4, MODE_FINAL3, 0, false>()) != cudaSuccess) return e;
    if ((e = prep_pair<1, MODE_FINAL3H, 0, true>()) != cudaSuccess) return e;
    if ((e = prep_pair<2, MODE_FINAL3H, 0, true>()) != cudaSuccess) return e;
    if ((e = prep_pair<4, MODE_FINAL3H, 0, false>()) != cudaSuccess) return e;
    if ((e = prep_dpl<2, 0, false>()) != cudaSuccess) return e;
    if ((e = prep_dpl<2, 0, true>()) != cudaSuccess) return e;
    if ((e = prep_dpl<4, 0, false>()) != cudaSuccess) return e;
    if ((e = prep_dpl<4, 0, true>()) != cudaSuccess) return e;
    if ((e = prep_dpl<8, 0, false>()) != cudaSuccess) return e;
    if ((e = prep_dpl<2, 1, false>()) != cudaSuccess) return e;
    if ((e = prep_one<2, MODE_FINAL7, 1, false, true>()) != cudaSuccess) return e;   // the multi-scale T->B final
    if ((e = prep_dpl<4, 1, false>()) != cudaSuccess) return e;
    return prep_dpl<8, 1, false>();
}

template <int DPL, int SAT, bool KEY16>
static cudaError_t launch_path_mode(const LineParams &p, int mode, dim3 g, dim3 b, cudaStream_t s) {
    const int w = (int)(b.x / 32);
    switch (mode) {
    case MODE_SCRATCH:
        k_path<DPL, MODE_SCRATCH, SAT, false><<<g, b, w * Slot<DPL, MODE_SCRATCH>::RING, s>>>(p); break;
    case MODE_STORE:
        k_path<DPL, MODE_STORE, SAT, false><<<g, b, w * Slot<DPL, MODE_STORE>::RING, s>>>(p); break;
    case MODE_ACCUM:
        k_path<DPL, MODE_ACCUM, SAT, false><<<g, b, w * Slot<DPL, MODE_ACCUM>::RING, s>>>(p); break;
    case MODE_FINAL:
        k_path<DPL, MODE_FINAL, SAT, false><<<g, b, w * Slot<DPL, MODE_FINAL>::RING, s>>>(p); break;
    case MODE_FINAL3:
        k_path<DPL, MODE_FINAL3, SAT, KEY16><<<g, b, w * Slot<DPL, MODE_FINAL3>::RING, s>>>(p); break;
    case MODE_FINAL7:
        // the multi-scale full scale's T->B final: even columns from row 0, one line per warp
        if (SAT && DPL == 2 && p.even_only && p.gpw == 1 && p.dx == 0 && p.dy == 1)
            k_path<2, MODE_FINAL7, 1, false, true><<<g, b, w * Slot<2, MODE_FINAL7>::RING, s>>>(p);
        else
            k_path<DPL, MODE_FINAL7, SAT, false><<<g, b, w * Slot<DPL, MODE_FINAL7>::RING, s>>>(p);
        break;
    default: return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
}

int path_dpl(int D, int want) {
    if (D < 16 || D > 256 || D % 16) return 0;
    const int lo = D <= 64 ? 2 : (D <= 128 ? 4 : 8);   // at most 32 lanes per line
    if (want != 0 && want != 2 && want != 4 && want != 8) return 0;
    return want < lo ? lo : want;
}

cudaError_t launch_line(const LineParams &p0, int mode, int saturate, int warps_per_block, cudaStream_t s) {
    LineParams p = p0;
    if (warps_per_block < 1 || warps_per_block > 4 || p.nlines < 1 || !p.C) return cudaErrorInvalidValue;
    if (pair_applies(p, mode, saturate)) return launch_pair(p, mode, saturate, warps_per_block, s);
    const int dpl = path_dpl(p.D, p.dpl);
    if (!dpl || p.D % dpl) return cudaErrorInvalidValue;
    p.nl = p.D / dpl;                      // lanes per line that hold disparities
    p.lpl = p.nl;
    p.gpw = (32 % p.lpl == 0) ? 32 / p.lpl : 1;
    const int lines_per_block = warps_per_block * p.gpw;
    const dim3 b(32 * warps_per_block), g((p.nlines + lines_per_block - 1) / lines_per_block);
    const bool key16 = p.key16 != 0 && p.D <= 64;
    if (saturate) {
        switch (dpl) {
        case 2: return launch_path_mode<2, 1, false>(p, mode, g, b, s);
        case 4: return launch_path_mode<4, 1, false>(p, mode, g, b, s);
        case 8: return launch_path_mode<8, 1, false>(p, mode, g, b, s);
        default: return cudaErrorInvalidValue;
        }
    }
    switch (dpl) {
    case 2: return key16 ? launch_path_mode<2, 0, true>(p, mode, g, b, s)
                         : launch_path_mode<2, 0, false>(p, mode, g, b, s);
    case 4: return key16 ? launch_path_mode<4, 0, true>(p, mode, g, b, s)
                         : launch_path_mode<4, 0, false>(p, mode, g, b, s);
    case 8: return launch_path_mode<8, 0, false>(p, mode, g, b, s);
    default: return cudaErrorInvalidValue;
    }
}

}  // namespace sgmgb

