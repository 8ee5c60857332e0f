// sgmgb_path.cu -- the SGM path kernel: groups of lanes walk lines of one direction.
//
// Input: the frame's cost volume C[p][d] (uint8, computed once by k_cost), so
// a path pass does no population counts and needs no image-edge tests.
//
// Layout: a line's D disparities are spread over LPL = D/DPL lanes, DPL per
// lane, held in DPL/2 registers of packed u16 pairs; a warp carries
// G = 32/LPL lines at once (one line per lane group). Lane li of a group owns
// d in [li*DPL, (li+1)*DPL); register j holds (d0 + j, d0 + DPL/2 + j), so the
// d-1 / d+1 neighbours of a register are other registers of the same lane
// except at the two ends, which come from the adjacent lanes by shuffle (the
// group's first and last lanes mask in "no such disparity").
//
// Arithmetic: min.u16x2 runs at the full integer rate on sm_103; additions of
// packed pairs use plain 32-bit IADD because no half can carry (every value
// stays below 0x8000). The reference's saturating adds need no clamps:
// with a = prev[d] <= 255 in the minimum,
//   min(a, sat(lo+P1), sat(hi+P1), sat(mn+P2)) == min(a, lo+P1, hi+P1, mn+P2)
// because any term that would saturate is >= 255 >= a (common/sgm_ref.c:61-72).
// The per-step minimum over d is one group-masked warp REDUX of a packed value
// (v | v << 16), so the result is already the packed pair the next step needs.
// Lanes past the last disparity carry cost 0x3FFF, so they never win a
// minimum. The multi-scale variant clamps L to 255 (multiscale/sgm_ms_ref.c:82).
//
// Memory: every step's inputs (its cost bytes, the planes of other directions,
// the partial sum) are loaded R steps ahead into a register ring.
#include "sgmgb_kernels.cuh"

namespace sgmgb {

namespace {

constexpr uint32_t kFull = 0xFFFFFFFFu;
constexpr uint32_t kPadPk = 0x3FFF3FFFu;   // cost / L of lanes past the last disparity

__device__ __forceinline__ uint32_t vmin2(uint32_t a, uint32_t b) {
    uint32_t r;
    asm("min.u16x2 %0, %1, %2;" : "=r"(r) : "r"(a), "r"(b));
    return r;
}
// min of the two halves, replicated into both halves
__device__ __forceinline__ uint32_t fold2(uint32_t v) { return vmin2(v, __byte_perm(v, v, 0x1032)); }
__device__ __forceinline__ uint32_t pk2(uint32_t v) { return v | (v << 16); }

// half-word k (natural disparity order within the lane) of a register file
template <int NR>
__device__ __forceinline__ uint32_t hw_at(const uint32_t (&r)[NR], int k) {
    return (r[k % NR] >> (16 * (k / NR))) & 0xFFFFu;
}

template <int MODE> struct Planes {   // scratch planes a pass reads
    static constexpr int N = MODE == MODE_SCRATCH ? 0 : (MODE == MODE_FINAL3 ? 3 : 1);
};

template <int DPL, int MODE>
struct StepIn {
    static constexpr int SCW = (DPL + 3) / 4;                      // words per DPL bytes
    uint32_t cw[SCW];                                              // cost bytes d0..d0+DPL-1
    uint32_t pw[Planes<MODE>::N > 0 ? Planes<MODE>::N * SCW : 1];  // plane bytes
    uint32_t sw[DPL / 2];                                          // partial sum, natural u16 pairs
};

template <int DPL>
__device__ __forceinline__ void load_bytes(const uint8_t *src, uint32_t *w) {
    if (DPL == 2) {
        w[0] = *(const uint16_t *)src;
    } else if (DPL == 4) {
        w[0] = *(const uint32_t *)src;
    } else if (DPL == 8) {
        const uint2 v = *(const uint2 *)src;
        w[0] = v.x; w[1] = v.y;
    } else {
#pragma unroll
        for (int k = 0; k < (DPL + 3) / 4; k++) w[k] = 0;
#pragma unroll
        for (int k = 0; k < DPL; k++) w[k / 4] |= (uint32_t)src[k] << (8 * (k % 4));
    }
}

// byte k of a packed byte run
__device__ __forceinline__ uint32_t byte_at(const uint32_t *w, int k) { return (w[k / 4] >> (8 * (k % 4))) & 0xFFu; }

// Loads everything pixel p's step reads.
template <int DPL, int MODE>
__device__ __forceinline__ void fetch(const LineParams &P, int p, int d0, StepIn<DPL, MODE> &s) {
    constexpr int SCW = StepIn<DPL, MODE>::SCW;
    const size_t off = (size_t)p * P.D + d0;
    load_bytes<DPL>(P.C + off, s.cw);
    if (Planes<MODE>::N > 0) {
        load_bytes<DPL>(P.sc + off, s.pw);
        if (MODE == MODE_FINAL3) {
            load_bytes<DPL>(P.sc2 + off, s.pw + SCW);
            load_bytes<DPL>(P.sc3 + off, s.pw + 2 * SCW);
        }
        if (MODE == MODE_ACCUM || MODE == MODE_FINAL) {
            const uint32_t *sp = (const uint32_t *)(P.S + off);
            if (DPL == 4) {
                const uint2 w = *(const uint2 *)sp;
                s.sw[0] = w.x; s.sw[1] = w.y;
            } else if (DPL == 8) {
                const uint4 w = *(const uint4 *)sp;
                s.sw[0] = w.x; s.sw[1] = w.y; s.sw[2] = w.z; s.sw[3] = w.w;
            } else {
#pragma unroll
                for (int i = 0; i < DPL / 2; i++) s.sw[i] = sp[i];
            }
        }
    }
}

// Packed costs, register j = (d0+j, d0+DPL/2+j).
template <int DPL, int MODE>
__device__ __forceinline__ void unpack_cost(const StepIn<DPL, MODE> &s, uint32_t (&c)[DPL / 2]) {
    constexpr int NR = DPL / 2;
    if (DPL == 2) {
        c[0] = __byte_perm(s.cw[0], 0, 0x4140);
    } else if (DPL == 4) {
        c[0] = __byte_perm(s.cw[0], 0, 0x4240);
        c[1] = __byte_perm(s.cw[0], 0, 0x4341);
    } else if (DPL == 8) {
#pragma unroll
        for (int j = 0; j < 4; j++) c[j] = __byte_perm(s.cw[0], s.cw[1], j | ((4 + j) << 8)) & 0x00FF00FFu;
    } else {
#pragma unroll
        for (int j = 0; j < NR; j++) c[j] = byte_at(s.cw, j) | (byte_at(s.cw, j + NR) << 16);
    }
}
// natural-order u16 pair i = (d0+2i, d0+2i+1) of a packed byte run
__device__ __forceinline__ uint32_t byte_pair(const uint32_t *w, int i) {
    return __byte_perm(w[(2 * i) / 4] >> (8 * ((2 * i) % 4)), 0, 0x4140);
}

// What a pass does with L(p, d0..d0+DPL-1). `live`: this lane's line has a
// pixel at this step; `lead`: the group's first lane; `gmask`: the group.
// KEY16: the argmin key S*64 + d fits a packed u16 (4 paths, D <= 64).
template <int DPL, int MODE, bool KEY16>
__device__ __forceinline__ void emit(const LineParams &P, int p, int x, int y, int d0, bool lead,
                                     uint32_t gmask, bool live, const uint32_t (&L)[DPL / 2],
                                     const StepIn<DPL, MODE> &s) {
    constexpr int NR = DPL / 2;
    constexpr int SCW = StepIn<DPL, MODE>::SCW;
    const size_t off = (size_t)p * P.D + d0;
    if (MODE == MODE_SCRATCH) {
        if (!live) return;
        uint8_t *dst = P.sc + off;
        if (DPL == 2) {
            *(uint16_t *)dst = (uint16_t)__byte_perm(L[0], 0, 0x0020);
        } else if (DPL == 4) {
            *(uint32_t *)dst = __byte_perm(L[0], L[1], 0x6240);
        } else if (DPL == 8) {
            const uint32_t t01 = __byte_perm(L[0], L[1], 0x6240), t23 = __byte_perm(L[2], L[3], 0x6240);
            *(uint2 *)dst = make_uint2(__byte_perm(t01, t23, 0x5410), __byte_perm(t01, t23, 0x7632));
        } else {
#pragma unroll
            for (int k = 0; k < DPL; k++) dst[k] = (uint8_t)hw_at<NR>(L, k);
        }
        return;
    }
    // this pass's L plus everything read for this pixel, natural order
    uint32_t tot[NR];
#pragma unroll
    for (int i = 0; i < NR; i++) {
        tot[i] = __byte_perm(L[(2 * i) % NR] >> (16 * ((2 * i) / NR)),
                             L[(2 * i + 1) % NR] >> (16 * ((2 * i + 1) / NR)), 0x5410);
        tot[i] += byte_pair(s.pw, i);
        if (MODE == MODE_FINAL3) tot[i] += byte_pair(s.pw + SCW, i) + byte_pair(s.pw + 2 * SCW, i);
        if (MODE == MODE_ACCUM || MODE == MODE_FINAL) tot[i] += s.sw[i];   // no carry: S <= 2040
    }
    if (MODE == MODE_STORE || MODE == MODE_ACCUM) {
        if (!live) return;
        uint32_t *sp = (uint32_t *)(P.S + off);
        if (DPL == 4) *(uint2 *)sp = make_uint2(tot[0], tot[1]);
        else if (DPL == 8) *(uint4 *)sp = make_uint4(tot[0], tot[1], tot[2], tot[3]);
        else {
#pragma unroll
            for (int i = 0; i < NR; i++) sp[i] = tot[i];
        }
        return;
    }
    // final passes: argmin over d, the lowest d winning ties
    if (P.even_only && ((x | y) & 1)) return;   // uniform within the group
    uint32_t key;
    if (KEY16) {
        uint32_t k = kFull;
#pragma unroll
        for (int i = 0; i < NR; i++) k = vmin2(k, (tot[i] << 6) + pk2((uint32_t)(d0 + 2 * i)) + 0x10000u);
        key = live ? fold2(k) : kFull;
    } else {
        key = kFull;
        if (live) {
#pragma unroll
            for (int i = 0; i < NR; i++) {
                key = min(key, ((tot[i] & 0xFFFFu) << 8) | (uint32_t)(d0 + 2 * i));
                key = min(key, ((tot[i] >> 16) << 8) | (uint32_t)(d0 + 2 * i + 1));
            }
        }
    }
    key = __reduce_min_sync(gmask, key);
    if (lead && live) {
        const uint8_t d = (uint8_t)(KEY16 ? (key & 0x3Fu) : (key & 0xFFu));
        if (P.even_only) P.disp[(size_t)(y >> 1) * (P.W >> 1) + (x >> 1)] = d;
        else P.disp[p] = d;
    }
}

}  // namespace

template <int DPL, int MODE, int SAT, bool KEY16>
__global__ void __launch_bounds__(128)
k_path(const LineParams P) {
    constexpr int NR = DPL / 2;
    constexpr int R = 4;   // input ring: steps whose loads are in flight
    using In = StepIn<DPL, MODE>;
    const int lane = threadIdx.x & 31;
    const int warp = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    const int G = P.gpw, LPL = P.lpl;
    if (warp * G >= P.nlines) return;   // whole warp leaves together
    int g, li;
    uint32_t gmask;
    if (G == 1) { g = 0; li = lane; gmask = kFull; }
    else { g = lane / LPL; li = lane - g * LPL; gmask = ((1u << LPL) - 1u) << (g * LPL); }
    const int line = warp * G + g;
    const bool active = li < P.nl && line < P.nlines;
    const int d0 = li * DPL;
    const bool lead = li == 0;
    const uint32_t m_lo = li == 0 ? 0x00003FFFu : 0u;           // d = -1 does not exist
    const uint32_t m_hi = li == P.nl - 1 ? 0x3FFF0000u : 0u;    // d = D does not exist
    const uint32_t P1 = pk2((uint32_t)P.p1), P2 = pk2((uint32_t)P.p2);
    const int dx = P.dx, dy = P.dy;

    // entry pixel and length of this group's line
    const int xe = dx > 0 ? 0 : P.W - 1, ye = dy > 0 ? 0 : P.H - 1;
    int x, y, len = 0;
    if (dy == 0) { x = xe; y = line; }
    else if (dx == 0) { x = line; y = ye; }
    else if (line < P.H) { x = xe; y = line; }
    else { x = xe + dx * (line - P.H + 1); y = ye; }
    if (active) {
        if (dy == 0) len = P.W;
        else if (dx == 0) len = P.H;
        else len = min(dx > 0 ? P.W - x : x + 1, dy > 0 ? P.H - y : y + 1);
    }
    const int maxlen = __reduce_max_sync(kFull, (uint32_t)len);
    const int step = dy * P.W + dx;
    int p = y * P.W + x;

    In ring[R];
    if (active) {
#pragma unroll
        for (int j = 0; j < R; j++)
            if (j < len) fetch<DPL, MODE>(P, p + j * step, d0, ring[j]);
    }

    // first pixel of the line: L = C
    uint32_t L[NR], c[NR];
#pragma unroll
    for (int j = 0; j < NR; j++) c[j] = kPadPk;
    if (active) unpack_cost<DPL, MODE>(ring[0], c);
    uint32_t t = c[0];
#pragma unroll
    for (int j = 0; j < NR; j++) { L[j] = c[j]; t = vmin2(t, c[j]); }
    uint32_t mn = __reduce_min_sync(gmask, fold2(t));   // packed (mn | mn << 16)
    emit<DPL, MODE, KEY16>(P, p, x, y, d0, lead, gmask, active, L, ring[0]);
    if (active && R < len) fetch<DPL, MODE>(P, p + R * step, d0, ring[0]);

    // One recurrence step on pixel i, whose inputs are in `slot`; the slot is
    // refilled with pixel i+R's inputs once this step is done with it.
    auto body = [&](In &slot, int i) {
        x += dx; y += dy; p += step;
        const bool live = active && i < len;
        if (live) unpack_cost<DPL, MODE>(slot, c);
        const uint32_t up = __shfl_up_sync(kFull, L[NR - 1], 1);
        const uint32_t dn = __shfl_down_sync(kFull, L[0], 1);
        const uint32_t lo0 = __byte_perm(up, L[NR - 1], 0x5432) | m_lo;   // (prev lane's last d, own d0+NR-1)
        const uint32_t hiL = __byte_perm(L[0], dn, 0x5432) | m_hi;        // (own d0+NR, next lane's first d)
        uint32_t w[NR];
#pragma unroll
        for (int j = 0; j < NR; j++) {
            const uint32_t lo = j == 0 ? lo0 : L[j - 1];
            const uint32_t hi = j == NR - 1 ? hiL : L[j + 1];
            w[j] = vmin2(L[j], vmin2(lo, hi) + P1);
        }
        const uint32_t E = mn + P2;
        uint32_t tm = kFull;
#pragma unroll
        for (int j = 0; j < NR; j++) {
            uint32_t v = vmin2(w[j], E) + c[j] - mn;
            if (SAT) v = vmin2(v, 0x00FF00FFu);
            L[j] = v;
            tm = vmin2(tm, v);
        }
        mn = __reduce_min_sync(gmask, fold2(tm));
        emit<DPL, MODE, KEY16>(P, p, x, y, d0, lead, gmask, live, L, slot);
        if (active && i + R < len) fetch<DPL, MODE>(P, p + R * step, d0, slot);
    };

    // pixel i's inputs live in ring[i % R]
    int i = 1;
    for (; i + R - 1 < maxlen; i += R) {
        body(ring[1], i);
        body(ring[2], i + 1);
        body(ring[3], i + 2);
        body(ring[0], i + 3);
    }
    if (i < maxlen) body(ring[1], i);
    if (i + 1 < maxlen) body(ring[2], i + 1);
    if (i + 2 < maxlen) body(ring[3], i + 2);
}

// ---------------------------------------------------------------------------
template <int DPL, int SAT, bool KEY16>
static cudaError_t launch_path_mode(const LineParams &p, int mode, dim3 g, dim3 b, cudaStream_t s) {
    switch (mode) {
    case MODE_SCRATCH: k_path<DPL, MODE_SCRATCH, SAT, false><<<g, b, 0, s>>>(p); break;
    case MODE_STORE:   k_path<DPL, MODE_STORE, SAT, false><<<g, b, 0, s>>>(p); break;
    case MODE_ACCUM:   k_path<DPL, MODE_ACCUM, SAT, false><<<g, b, 0, s>>>(p); break;
    case MODE_FINAL:   k_path<DPL, MODE_FINAL, SAT, false><<<g, b, 0, s>>>(p); break;
    case MODE_FINAL3:  k_path<DPL, MODE_FINAL3, SAT, KEY16><<<g, b, 0, s>>>(p); break;
    default: return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
}

cudaError_t launch_line(const LineParams &p0, int mode, int saturate, int warps_per_block, cudaStream_t s) {
    LineParams p = p0;
    if (warps_per_block < 1 || warps_per_block > 4 || p.nlines < 1 || !p.C) return cudaErrorInvalidValue;
    const int dpl = dpl_for(p.D);
    if (!dpl) return cudaErrorInvalidValue;
    p.nl = p.D / dpl;                      // lanes per line that hold disparities
    p.lpl = p.nl;
    p.gpw = (32 % p.lpl == 0) ? 32 / p.lpl : 1;
    const int lines_per_block = warps_per_block * p.gpw;
    const dim3 b(32 * warps_per_block), g((p.nlines + lines_per_block - 1) / lines_per_block);
    const bool key16 = p.key16 != 0 && dpl == 2;
    if (saturate) {
        if (dpl == 2) return launch_path_mode<2, 1, false>(p, mode, g, b, s);
        return cudaErrorInvalidValue;
    }
    switch (dpl) {
    case 2: return key16 ? launch_path_mode<2, 0, true>(p, mode, g, b, s)
                         : launch_path_mode<2, 0, false>(p, mode, g, b, s);
    case 4: return launch_path_mode<4, 0, false>(p, mode, g, b, s);
    case 8: return launch_path_mode<8, 0, false>(p, mode, g, b, s);
    default: return cudaErrorInvalidValue;
    }
}

}  // namespace sgmgb
