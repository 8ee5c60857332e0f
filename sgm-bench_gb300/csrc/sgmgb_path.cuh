// sgmgb_path.cuh -- the SGM path recurrence: groups of lanes walk lines of one direction.
// Device code shared by the per-pass kernel (sgmgb_path.cu) and the batch
// kernel (sgmgb_batch.cu).
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
// The per-step minimum over d is a warp REDUX of a packed value (v | v << 16)
// per lane group (group_min), so the result is already the packed pair the
// next step needs. Lanes past the last disparity never win a minimum (see the
// ring fill below). The multi-scale variant clamps L to 255
// (multiscale/sgm_ms_ref.c:82).
// The first pixel of a line needs no special case: with L_prev = 0 and
// min_prev = 0 the recurrence gives L = C, which is the reference's start.
//
// Memory: a line's per-step inputs (its cost bytes, the planes of other
// directions, the partial sum) are streamed into a per-warp shared-memory
// ring with cp.async, K steps per chunk and NCH chunks per ring, so NCH-1
// chunks (20-24 steps) are in flight while the lanes consume one. The copies hold no
// registers, which is what lets a pass keep enough bytes in flight per SM when
// only a few lines (warps) run on it -- the case of the horizontal passes.
#pragma once
#include "sgmgb_kernels.cuh"
#include <climits>
#include <type_traits>

namespace sgmgb {

namespace {

constexpr uint32_t kFull = 0xFFFFFFFFu;
constexpr uint32_t kPadPk = 0x3FFF3FFFu;   // cost / L of lanes past the last disparity

// Entry pixel (x, y) and length of line `line` of a pass (len = 0 past
// P.nlines). Lines run along (dx, dy) from the image edge they enter by: rows,
// columns, or diagonals indexed first by entry row, then by entry column.
// P.even_only (multi-scale full scale; W and H even): only the lines that
// cross a pixel with x and y both even are enumerated -- even rows, even
// columns, and the diagonals whose x + y is even (every other diagonal in
// each of the two entry edges).
__device__ __forceinline__ void line_start(const LineParams &P, int line, int &x, int &y, int &len) {
    const int dx = P.dx, dy = P.dy;
    const int xe = dx > 0 ? 0 : P.W - 1, ye = dy > 0 ? 0 : P.H - 1;
    int l = line;
    if (P.even_only) {
        if (dx == 0 || dy == 0) {
            l = 2 * line;
        } else {
            const int n1 = (P.H - (xe & 1) + 1) >> 1;     // entry rows l with xe + l even
            if (line < n1) l = (xe & 1) + 2 * line;
            else l = P.H - 1 + (((xe + ye) & 1) ? 1 : 2) + 2 * (line - n1);   // entry column xe + dx*(l-H+1)
        }
    }
    if (dy == 0) {
        x = xe; y = l; len = P.W;
        if (P.hseg) {                                  // half of the row (split horizontal lines)
            const int m = P.W >> 1;
            const bool first = P.hseg == 1;
            if (dx > 0) { x = first ? 0 : m; len = first ? m : P.W - m; }
            else { x = first ? P.W - 1 : m - 1; len = first ? P.W - m : m; }
        }
    }
    else if (dx == 0) { x = l; y = ye; len = P.H; }
    else {
        if (l < P.H) { x = xe; y = l; }
        else { x = xe + dx * (l - P.H + 1); y = ye; }
        len = min(dx > 0 ? P.W - x : x + 1, dy > 0 ? P.H - y : y + 1);
    }
    if (line >= P.nlines) len = 0;
}

__device__ __forceinline__ uint32_t vmin2(uint32_t a, uint32_t b) {
    uint32_t r;
    asm("min.u16x2 %0, %1, %2;" : "=r"(r) : "r"(a), "r"(b));
    return r;
}
// min(L, early + P1, late + P1) per half (the neighbour terms of the
// recurrence) with two fused add-min operations; `late` (the operand that
// comes from a shuffle) enters last. No half exceeds 0x7FFF, so nothing wraps.
__device__ __forceinline__ uint32_t nbr_min(uint32_t L, uint32_t early, uint32_t late, uint32_t P1) {
    return __viaddmin_u16x2(late, P1, __viaddmin_u16x2(early, P1, L));
}
// min of the two halves, replicated into both halves
__device__ __forceinline__ uint32_t fold2(uint32_t v) { return vmin2(v, __byte_perm(v, v, 0x1032)); }
__device__ __forceinline__ uint32_t pk2(uint32_t v) { return v | (v << 16); }

// half-word k (natural disparity order within the lane) of a register file
template <int NR>
__device__ __forceinline__ uint32_t hw_at(const uint32_t (&r)[NR], int k) {
    return (r[k % NR] >> (16 * (k / NR))) & 0xFFFFu;
}

__device__ __forceinline__ void cp_async16(uint32_t dst_smem, const void *src) {
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(dst_smem), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory"); }

// Minimum of v over this lane's group of lines (G groups of 32/G lanes; g is
// the lane's group, gmask its lanes). For G <= 4 it takes G full-warp
// reductions, each group's lanes contributing and the others passing ~0:
// one reduction per distinct member mask in flight at a time, which keeps the
// warp converged; larger G uses the group-masked form.
__device__ __forceinline__ uint32_t group_min(uint32_t v, int G, int g, uint32_t gmask) {
    if (G == 1) return __reduce_min_sync(kFull, v);
    if (G <= 4) {
        uint32_t r = __reduce_min_sync(kFull, g == 0 ? v : kFull);
        const uint32_t r1 = __reduce_min_sync(kFull, g == 1 ? v : kFull);
        r = g == 1 ? r1 : r;
        if (G == 4) {
            const uint32_t r2 = __reduce_min_sync(kFull, g == 2 ? v : kFull);
            const uint32_t r3 = __reduce_min_sync(kFull, g == 3 ? v : kFull);
            r = g == 2 ? r2 : (g == 3 ? r3 : r);
        }
        return r;
    }
    return __reduce_min_sync(gmask, v);
}

template <int MODE> struct Planes {   // scratch planes a pass reads
    static constexpr int N = MODE == MODE_SCRATCH ? 0 : (MODE == MODE_FINAL3 ? 3 : (MODE == MODE_FINAL7 ? 7 : 1));
};

// Ring geometry of a DPL. A step of one "byte stream" (the cost bytes or a
// plane: D bytes per line) takes SBM = 32*DPL bytes of the ring whatever the
// group shape, so lane l always reads its DPL bytes at l*DPL; the partial sum
// S takes two such units. NGB: 16-byte copies per lane per byte stream per chunk.
template <int DPL, int MODE> struct Ring {
    // steps per chunk: 1 KB of ring per byte stream for the scratch passes
    // (one stream: fewer per-chunk waits, copies and stores per step), 512 B
    // for the modes with more streams (registers for the chunk's inputs)
    static constexpr int K = (MODE == MODE_SCRATCH ? 32 : 16) / DPL;
    static constexpr int NCH = DPL == 2 ? 4 : (DPL == 4 ? 6 : 8);   // ring depth in chunks (NCH-1 in flight)
    static constexpr int SBM = 32 * DPL;
    static constexpr int NGB = K * SBM / 512;      // 2 (scratch) or 1
};
template <int DPL, int MODE> struct Slot {
    static constexpr bool HAS_S = MODE == MODE_ACCUM || MODE == MODE_FINAL;
    static constexpr int U = 1 + Planes<MODE>::N + (HAS_S ? 2 : 0);   // byte-stream units per step
    static constexpr int BYTES = Ring<DPL, MODE>::K * Ring<DPL, MODE>::SBM * U;  // one chunk of a warp
    // ring depth: a chunk of eight streams (FINAL7) already carries 4 KB, so
    // two chunks in flight keep as many bytes moving as deeper rings of one
    static constexpr int NCH = U >= 8 ? 3 : Ring<DPL, MODE>::NCH;
    static constexpr int RING = NCH * BYTES;                          // a warp's whole ring
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
    } else {
        const uint2 v = *(const uint2 *)src;
        w[0] = v.x; w[1] = v.y;
    }
}

// Reads step k's inputs of this lane from the ring chunk at `chunk`.
template <int DPL, int MODE>
__device__ __forceinline__ void ring_read(const uint8_t *chunk, int lane, int k, StepIn<DPL, MODE> &s) {
    constexpr int K = Ring<DPL, MODE>::K, SBM = Ring<DPL, MODE>::SBM, SCW = StepIn<DPL, MODE>::SCW;
    const uint8_t *b = chunk + k * SBM + lane * DPL;
    load_bytes<DPL>(b, s.cw);
#pragma unroll
    for (int q = 0; q < Planes<MODE>::N; q++) load_bytes<DPL>(b + (1 + q) * K * SBM, s.pw + q * SCW);
    if (Slot<DPL, MODE>::HAS_S) {
        const uint8_t *sb = chunk + (1 + Planes<MODE>::N) * K * SBM + k * 2 * SBM + lane * 2 * DPL;
        if (DPL == 2) {
            s.sw[0] = *(const uint32_t *)sb;
        } else if (DPL == 4) {
            const uint2 w = *(const uint2 *)sb;
            s.sw[0] = w.x; s.sw[1] = w.y;
        } else {
            const uint4 w = *(const uint4 *)sb;
            s.sw[0] = w.x; s.sw[1] = w.y; s.sw[2] = w.z; s.sw[3] = w.w;
        }
    }
}

// byte k of a packed byte run
__device__ __forceinline__ uint32_t byte_at(const uint32_t *w, int k) { return (w[k / 4] >> (8 * (k % 4))) & 0xFFu; }

// Packed costs, register j = (d0+j, d0+DPL/2+j).
template <int DPL, int MODE>
__device__ __forceinline__ void unpack_cost(const StepIn<DPL, MODE> &s, uint32_t (&c)[DPL / 2]) {
    if (DPL == 2) {
        c[0] = __byte_perm(s.cw[0], 0, 0x4140);
    } else if (DPL == 4) {
        c[0] = __byte_perm(s.cw[0], 0, 0x4240);
        c[1] = __byte_perm(s.cw[0], 0, 0x4341);
    } else {
#pragma unroll
        for (int j = 0; j < 4; j++) c[j] = __byte_perm(s.cw[0], s.cw[1], j | ((4 + j) << 8)) & 0x00FF00FFu;
    }
}
// natural-order u16 pair i = (d0+2i, d0+2i+1) of a packed byte run
__device__ __forceinline__ uint32_t byte_pair(const uint32_t *w, int i) {
    return __byte_perm(w[(2 * i) / 4] >> (8 * ((2 * i) % 4)), 0, 0x4140);
}

// What a pass does with L(p, d0..d0+DPL-1). `live`: this lane's line has a
// pixel at this step; `lead`: the group's first lane; `gmask`: the group.
// `out` points at this lane's bytes of pixel p in S (STORE, ACCUM), or, for
// SCRATCH, at its bytes of this step in the ring chunk's cost row, which the
// chunk's end copies to the plane (there `live` only excludes pad lanes).
// KEY16: the argmin key S*64 + d fits a packed u16 (4 paths, D <= 64).
template <int DPL, int MODE, bool KEY16, bool ONE>
__device__ __forceinline__ void emit(const LineParams &P, void *out, int p, int x, int y, int d0,
                                     bool lead, int g, uint32_t gmask, bool live, const uint32_t (&L)[DPL / 2],
                                     const StepIn<DPL, MODE> &s) {
    constexpr int NR = DPL / 2;
    constexpr int SCW = StepIn<DPL, MODE>::SCW;
    if (MODE == MODE_SCRATCH) {            // `out`: this lane's bytes in the ring's staging row
        if (!live) return;
        if (DPL == 2) {
            *(uint16_t *)out = (uint16_t)__byte_perm(L[0], 0, 0x0020);
        } else if (DPL == 4) {
            *(uint32_t *)out = __byte_perm(L[0], L[1], 0x6240);
        } else {
            const uint32_t t01 = __byte_perm(L[0], L[1], 0x6240), t23 = __byte_perm(L[2], L[3], 0x6240);
            *(uint2 *)out = make_uint2(__byte_perm(t01, t23, 0x5410), __byte_perm(t01, t23, 0x7632));
        }
        return;
    }
    // this pass's L plus everything read for this pixel, natural order
    uint32_t tot[NR];
#pragma unroll
    for (int i = 0; i < NR; i++) {
        if (NR == 1) tot[i] = L[0];   // register 0 is already (d0, d0+1)
        else tot[i] = __byte_perm(L[(2 * i) % NR] >> (16 * ((2 * i) / NR)),
                                  L[(2 * i + 1) % NR] >> (16 * ((2 * i + 1) / NR)), 0x5410);
        tot[i] += byte_pair(s.pw, i);
#pragma unroll
        for (int q = 1; q < Planes<MODE>::N; q++) tot[i] += byte_pair(s.pw + q * SCW, i);   // FINAL3, FINAL7
        if (MODE == MODE_ACCUM || MODE == MODE_FINAL) tot[i] += s.sw[i];   // no carry: S <= 2040
    }
    if (MODE == MODE_STORE || MODE == MODE_ACCUM) {
        if (!live) return;
        uint32_t *sp = (uint32_t *)out;
        if (DPL == 2) *sp = tot[0];
        else if (DPL == 4) *(uint2 *)sp = make_uint2(tot[0], tot[1]);
        else *(uint4 *)sp = make_uint4(tot[0], tot[1], tot[2], tot[3]);
        return;
    }
    // final passes: argmin over d, the lowest d winning ties. Every lane of the
    // warp reaches group_min (it may reduce over the whole warp); a pixel that
    // is not kept (odd x or y of an even-only map) only skips the store.
    constexpr bool EVEN = MODE == MODE_FINAL || MODE == MODE_FINAL7;   // modes with an even-only map
    const bool keep = live && !(EVEN && P.even_only && ((x | y) & 1));
    uint32_t key;
    if (KEY16) {
        uint32_t k = kFull;
#pragma unroll
        for (int i = 0; i < NR; i++) k = vmin2(k, tot[i] * 64u + (pk2((uint32_t)(d0 + 2 * i)) + 0x10000u));
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
    key = ONE ? __reduce_min_sync(kFull, key) : group_min(key, P.gpw, g, gmask);
    if (lead && keep) {
        const uint8_t d = (uint8_t)(KEY16 ? (key & 0x3Fu) : (key & 0xFFu));
        if (EVEN && P.even_only) P.disp[(size_t)(y >> 1) * (P.W >> 1) + (x >> 1)] = d;
        else P.disp[p] = d;
    }
}

}  // namespace

// Runs warp `warp` of a pass: lines warp*G .. warp*G+G-1 of direction
// (P.dx, P.dy), with P.nl/P.lpl/P.gpw set for DPL. `ring` is this warp's
// Slot<DPL, MODE>::RING bytes of shared memory (16-byte aligned). All 32 lanes
// of the warp must call it.
// EO (FINAL7 only): the even-only final down the even columns from row 0 (the
// multi-scale full scale's T->B final, one line per warp): its odd rows'
// argmins are not kept, so those steps run the recurrence alone (the
// launcher picks EO only for such a pass).
template <int DPL, int MODE, int SAT, bool KEY16, bool EO = false>
__device__ __forceinline__ void path_warp(const LineParams &P, int warp, uint8_t *ring) {
    constexpr int NR = DPL / 2;
    constexpr int K = Ring<DPL, MODE>::K, SBM = Ring<DPL, MODE>::SBM, NGB = Ring<DPL, MODE>::NGB,
                  NCH = Slot<DPL, MODE>::NCH;
    constexpr int NPL = Planes<MODE>::N;
    constexpr bool HAS_S = Slot<DPL, MODE>::HAS_S;
    constexpr int SLOT = Slot<DPL, MODE>::BYTES;
    using In = StepIn<DPL, MODE>;
    const int lane = threadIdx.x & 31;
    const int G = P.gpw, LPL = P.lpl;
    if (warp * G >= P.nlines) return;   // whole warp leaves together
    int g, li;
    uint32_t gmask;
    if (G == 1) { g = 0; li = lane; gmask = kFull; }
    else { g = lane / LPL; li = lane - g * LPL; gmask = ((1u << LPL) - 1u) << (g * LPL); }
    const int line = warp * G + g;
    const bool has_d = li < P.nl;
    const bool active = has_d && line < P.nlines;
    const int d0 = li * DPL;
    const bool lead = li == 0;
    const uint32_t m_lo = li == 0 ? 0x00003FFFu : 0u;           // d = -1 does not exist
    const uint32_t m_hi = li == P.nl - 1 ? 0x3FFF0000u : 0u;    // d = D does not exist
    const uint32_t P1 = pk2((uint32_t)P.p1), P2 = pk2((uint32_t)P.p2);
    const int dx = P.dx, dy = P.dy;

    // entry pixel and length of this group's line
    int x, y, len;
    line_start(P, line, x, y, len);
    if (!active) len = 0;
    const int maxlen = __reduce_max_sync(kFull, (uint32_t)len);
    const int step = dy * P.W + dx;
    int p = y * P.W + x;

    // ---- this lane's share of every chunk's copies ----
    // Byte streams (C and the planes share offsets): 16-byte granule u = lane + 32*j
    // of a chunk covers ring bytes [16u, 16u+16) = step u*16/SBM, lanes' bytes r = u*16 % SBM,
    // which belong to group r/D at byte r%D of its D-byte run.
    const uint32_t ring_s = (uint32_t)__cvta_generic_to_shared(ring);
    const int gD = G * P.D;
    const long long adv = (long long)K * step * P.D;   // element advance per chunk (bytes of C)
    long long goff[NGB];
    int glim[NGB];
#pragma unroll
    for (int j = 0; j < NGB; j++) {
        const int b = (lane + 32 * j) * 16, k = b / SBM, r = b % SBM;
        const int gg = min(r / P.D, 31), o = r - gg * P.D;
        const int pg = __shfl_sync(kFull, p, (gg * LPL) & 31);
        const int lg = __shfl_sync(kFull, len, (gg * LPL) & 31);
        goff[j] = ((long long)pg + (long long)k * step) * P.D + o;
        glim[j] = r < gD ? lg - k : 0;
    }
    // SCRATCH: the plane has the cost volume's layout, so the chunk's L bytes,
    // staged where its cost bytes were, go out by the same 16-byte granules.
    // even_only: only the granules of pixels with x and y even (a chunk is an
    // even number of steps, so a granule's parity is the same in every chunk),
    // into a compact plane: pixel (x, y) at (y/2)(W/2) + x/2, where two steps
    // along any direction move (dy W/2 + dx). The even-only final reads its
    // planes there (poff).
    const long long oadv = P.even_only ? (long long)(K / 2) * (dy * (P.W >> 1) + dx) * P.D : adv;
    long long ooff[NGB], poff[NGB];
    bool ost[NGB];
#pragma unroll
    for (int j = 0; j < NGB; j++) {
        const int b = (lane + 32 * j) * 16, k = b / SBM, gg = min((b % SBM) / P.D, 31), o = b % SBM - gg * P.D;
        const int xg = __shfl_sync(kFull, x, (gg * LPL) & 31) + k * dx;
        const int yg = __shfl_sync(kFull, y, (gg * LPL) & 31) + k * dy;
        ost[j] = !P.even_only || ((xg | yg) & 1) == 0;
        ooff[j] = P.even_only ? ((long long)(yg >> 1) * (P.W >> 1) + (xg >> 1)) * P.D + o : goff[j];
        poff[j] = ooff[j];
    }
    long long soff[HAS_S ? 2 * NGB : 1];
    int slim[HAS_S ? 2 * NGB : 1];
    if (HAS_S) {
#pragma unroll
        for (int j = 0; j < 2 * NGB; j++) {
            const int b = (lane + 32 * j) * 16, k = b / (2 * SBM), r = b % (2 * SBM);
            const int gg = min(r / (2 * P.D), 31), o = r - gg * 2 * P.D;
            const int pg = __shfl_sync(kFull, p, (gg * LPL) & 31);
            const int lg = __shfl_sync(kFull, len, (gg * LPL) & 31);
            soff[j] = ((long long)pg + (long long)k * step) * 2 * P.D + o;
            slim[j] = r < 2 * gD ? lg - k : 0;
        }
    }
    const uint8_t *pl[NPL > 0 ? NPL : 1];
    if (NPL > 0) pl[0] = P.sc;
    if (NPL >= 3) { pl[1] = P.sc2; pl[2] = P.sc3; }
    if (NPL == 7) { pl[3] = P.xpl[0]; pl[4] = P.xpl[1]; pl[5] = P.xpl[2]; pl[6] = P.xpl[3]; }

    // Enqueues chunk c (steps c*K .. c*K+K-1) into ring slot c % NCH.
    auto issue = [&](int c) {
        const uint32_t dst = ring_s + (uint32_t)((c % NCH) * SLOT);
        const int i0 = c * K;
#pragma unroll
        for (int j = 0; j < NGB; j++) {
            if (i0 < glim[j]) {
                const uint32_t db = dst + (uint32_t)((lane + 32 * j) * 16);
                cp_async16(db, P.C + goff[j]);
                // even-only finals: the planes hold values at even (x, y) only, and only
                // those pixels' argmins are kept, so the other granules' planes are not read
                if (ost[j]) {
#pragma unroll
                    for (int q = 0; q < NPL; q++) cp_async16(db + (uint32_t)((1 + q) * K * SBM), pl[q] + poff[j]);
                }
            }
            goff[j] += adv;
            poff[j] += oadv;
        }
        if (HAS_S) {
#pragma unroll
            for (int j = 0; j < 2 * NGB; j++) {
                if (i0 < slim[j])
                    cp_async16(dst + (uint32_t)((1 + NPL) * K * SBM + (lane + 32 * j) * 16),
                               (const uint8_t *)P.S + soff[j]);
                soff[j] += 2 * adv;
            }
        }
        cp_async_commit();
    };

    const int nchunks = (maxlen + K - 1) / K;
#pragma unroll
    for (int c = 0; c < NCH - 1; c++) issue(c);

    // this lane's output for the current pixel: sc bytes (SCRATCH) or S words (STORE, ACCUM)
    uint8_t *out = nullptr;
    long long out_step = 0;
    if (MODE == MODE_STORE || MODE == MODE_ACCUM) {
        out = (uint8_t *)(P.S + (long long)p * P.D + d0); out_step = (long long)step * P.D * 2;
    }

    // Lanes past the last disparity (D/DPL lanes short of a whole warp) read
    // ring bytes that no copy writes: fill them with cost 255 once. Every real
    // L is at most 254 (plain: 62 + P2) or saturated to 255 (multi-scale), and
    // a pad lane's L is at least its cost, so a pad lane never lowers a minimum;
    // its neighbours mask it out as d = D.
    if (!has_d) {
#pragma unroll
        for (int sl = 0; sl < NCH; sl++)
#pragma unroll
            for (int k = 0; k < K; k++)
#pragma unroll
                for (int b = 0; b < DPL; b++) ring[sl * SLOT + k * SBM + lane * DPL + b] = 0xFF;
    }
    __syncwarp();

    // lanes of lines that end before the warp's last step (diagonals)
    const int minlen = (int)__reduce_min_sync(kFull, active ? (uint32_t)len : 0x7FFFFFFFu);

    uint32_t L[NR];
    uint32_t mn = 0;   // L_prev = 0, min_prev = 0: the first step yields L = C
#pragma unroll
    for (int j = 0; j < NR; j++) L[j] = has_d ? 0u : kPadPk;
    x -= dx; y -= dy; p -= step;
    if (MODE == MODE_STORE || MODE == MODE_ACCUM) out -= out_step;

    // One recurrence step on the next pixel of the line; FULL: every line of
    // the warp has this pixel (no per-step length test); ONE: the warp holds
    // one line (a plain full-warp reduction).
    auto step_once = [&](const In &s, int i, uint8_t *stage, auto full_t, auto one_t, auto emit_t) {
        constexpr bool FULL = decltype(full_t)::value;
        constexpr bool ONE = decltype(one_t)::value;
        constexpr bool EMIT = decltype(emit_t)::value;   // false: the recurrence only (no output at this pixel)
        x += dx; y += dy; p += step;
        if (MODE == MODE_STORE || MODE == MODE_ACCUM) out += out_step;
        const bool live = MODE == MODE_SCRATCH ? has_d : (FULL ? active : i < len);
        uint32_t c[NR];
        unpack_cost<DPL, MODE>(s, c);
        uint32_t lo0, hiL;
        if (DPL == 2) {
            // A lane's two disparities are neighbours. At a group's ends the
            // width-limited shuffle returns the lane's own pair, so the missing
            // d-1 (d+1) slot holds the d+1 (d-1) value: a duplicate of the other
            // neighbour, which leaves min(lo, hi) unchanged -- no masks needed.
            // (A pad lane past the last disparity holds L >= 255: also harmless.)
            const uint32_t up = ONE ? __shfl_up_sync(kFull, L[0], 1) : __shfl_up_sync(kFull, L[0], 1, LPL);
            const uint32_t dn = ONE ? __shfl_down_sync(kFull, L[0], 1) : __shfl_down_sync(kFull, L[0], 1, LPL);
            lo0 = __byte_perm(up, L[0], 0x5432);     // (prev lane's d0+1, own d0)
            hiL = __byte_perm(L[0], dn, 0x5432);     // (own d0+1, next lane's d0)
        } else {
            const uint32_t up = __shfl_up_sync(kFull, L[NR - 1], 1);
            const uint32_t dn = __shfl_down_sync(kFull, L[0], 1);
            lo0 = __byte_perm(up, L[NR - 1], 0x5432) | m_lo;   // (prev lane's last d, own d0+NR-1)
            hiL = __byte_perm(L[0], dn, 0x5432) | m_hi;        // (own d0+NR, next lane's first d)
        }
        uint32_t w[NR];
#pragma unroll
        for (int j = 0; j < NR; j++) {
            const uint32_t lo = j == 0 ? lo0 : L[j - 1];
            const uint32_t hi = j == NR - 1 ? hiL : L[j + 1];
            if (NR >= 2)   // measured: faster from DPL = 4 on, slower at DPL = 2
                w[j] = j == 0 ? nbr_min(L[j], hi, lo, P1) : nbr_min(L[j], lo, hi, P1);
            else
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
        mn = ONE ? __reduce_min_sync(kFull, fold2(tm)) : group_min(fold2(tm), G, g, gmask);
        if (EMIT)
            emit<DPL, MODE, KEY16, ONE>(P, MODE == MODE_SCRATCH ? (void *)stage : (void *)out, p, x, y, d0, lead,
                                        g, gmask, live, L, s);
    };

    // EO: the line starts at an even row of an even column and a chunk is an
    // even number of steps, so a chunk's odd steps are the odd rows, whose
    // argmins are not kept; they run the recurrence on the cost alone, without
    // the planes, the sum or the argmin

    // the chunk loop, instantiated for one line per warp and for several
    auto run = [&](auto one_t) {
        for (int ch = 0; ch < nchunks; ch++) {
            cp_async_wait<NCH - 2>();   // chunk ch has landed (this lane's copies)
            __syncwarp();               // ... and every lane's; slot ch-1 is free
            issue(ch + NCH - 1);
            uint8_t *chunk = ring + (ch % NCH) * SLOT;
            if (MODE == MODE_FINAL7) {  // eight input streams: read each step's inputs when it runs
                auto steps = [&](auto full_t) {
#pragma unroll
                    for (int k = 0; k < K; k++) {
                        In s1;
                        if (EO && (k & 1)) {
                            load_bytes<DPL>(chunk + k * SBM + lane * DPL, s1.cw);
                            step_once(s1, ch * K + k, chunk + k * SBM + lane * DPL, full_t, one_t, std::false_type{});
                        } else {
                            ring_read<DPL, MODE>(chunk, lane, k, s1);
                            step_once(s1, ch * K + k, chunk + k * SBM + lane * DPL, full_t, one_t, std::true_type{});
                        }
                    }
                };
                if ((ch + 1) * K <= minlen) steps(std::true_type{});
                else steps(std::false_type{});
                continue;
            }
            In s[K];                    // the chunk's inputs, read before its steps run
#pragma unroll
            for (int k = 0; k < K; k++) ring_read<DPL, MODE>(chunk, lane, k, s[k]);
            if ((ch + 1) * K <= minlen) {
#pragma unroll
                for (int k = 0; k < K; k++)
                    step_once(s[k], ch * K + k, chunk + k * SBM + lane * DPL, std::true_type{}, one_t,
                              std::true_type{});
            } else {
#pragma unroll
                for (int k = 0; k < K; k++)
                    step_once(s[k], ch * K + k, chunk + k * SBM + lane * DPL, std::false_type{}, one_t,
                              std::true_type{});
            }
            if (MODE == MODE_SCRATCH) {
                __syncwarp();           // every lane's L bytes of the chunk are staged
#pragma unroll
                for (int j = 0; j < NGB; j++) {
                    if (ost[j] && ch * K < glim[j])
                        *(uint4 *)(P.sc + ooff[j]) = *(const uint4 *)(chunk + (lane + 32 * j) * 16);
                    ooff[j] += oadv;
                }
            }
        }
    };
    if (G == 1) run(std::true_type{});
    else run(std::false_type{});
    cp_async_wait<0>();   // no copy outlives the kernel
}

}  // namespace sgmgb
