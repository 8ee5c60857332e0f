// sgmgb_pair.cuh -- the path recurrence with two lines per warp packed into
// the halves of each register (every pass mode, D = 32, 64 or 128). Device
// code used by sgmgb_path.cu and sgmgb_batch.cu.
//
// Layout: a warp walks lines A and B of one direction together. Lane l owns
// disparities d = l*NR .. l*NR + NR - 1 (NR = D/32), and register j of the
// lane holds the packed pair (L_A[d], L_B[d]) for d = l*NR + j. Every
// min.u16x2 and 32-bit add then advances both lines at once, the d-1 / d+1
// neighbours of a register are its neighbouring registers (or one shuffle of
// a whole register at the lane's ends) -- no byte permutes on the recurrence
// -- and the minimum over d is a per-register minimum plus one warp reduction
// per line: redux(tm & 0xffff) gives line A's minimum, and redux(tm) gives
// line B's in its high half (the high half is the primary key of an unsigned
// minimum).
//
// Ends of the disparity range: with NR <= 2 the width-32 shuffle returns the
// lane's own register at lanes 0 and 31, so the missing d-1 (d+1) slot holds
// the lane's own d+1 (d-1) value (NR = 2) or d itself (NR = 1): a duplicate
// of the other neighbour or of prev[d], neither of which can lower
// min(prev[d], lo + P1, hi + P1). With NR = 4 the slots are masked to 0x3FFF.
//
// Arithmetic as in sgmgb_path.cuh: no half carries (values < 0x8000), the
// reference's saturations are no-ops (common/sgm_ref.c:61-72), and the first
// pixel of a line starts from L_prev = 0, min_prev = 0, which yields L = C.
//
// Memory: the per-warp shared-memory ring of sgmgb_path.cuh, a step being the
// two lines' D-byte rows [A | B] of each input stream; a chunk is G 16-byte
// cp.async granules per lane of a stream (PairRing). The scratch output is
// staged in the consumed cost rows and leaves by the same granules.
#pragma once
#include "sgmgb_path.cuh"

namespace sgmgb {

namespace {

// A chunk is G 16-byte granules per lane of each input stream: 512 G bytes,
// K = 8 G / NR steps. The scratch passes (one input stream) take chunks of
// 1 KB (2 KB at D = 128): fewer per-chunk waits, copies and stores per step
// (measured at D = 64: 512 B 125 us, 1 KB 94 us, 2 KB 98 us per row pass; at
// D = 128: 1 KB 167 us, 2 KB 143 us). The final-of-planes pass (four input
// streams) takes 1 KB chunks in a ring of three: 166 -> 151 us alone, and the
// ring stays at 48 KB per 4-warp block (a ring of six, 96 KB, had made four
// frames in flight slower: 0.280 -> 0.292 ms per frame; with three, 0.268 ->
// 0.261). The other modes keep 512 bytes.
template <int NR, int MODE> struct PairRing {
    static constexpr bool F3 = MODE == MODE_FINAL3 || MODE == MODE_FINAL3H;
    static constexpr bool F7 = MODE == MODE_FINAL7;                // eight input streams: 512-byte chunks
    static constexpr int G = MODE == MODE_SCRATCH ? (NR == 4 ? 4 : 2) : (F3 ? 2 : 1);
    static constexpr int CB = 512 * G;                             // bytes of one stream per chunk
    static constexpr int K = 8 * G / NR;                           // steps per chunk
    static constexpr int NCH = (F3 || F7) ? 3 : (NR == 1 ? 4 : (NR == 2 ? 6 : 8));   // ring depth
    static constexpr int SB = 64 * NR;                             // bytes of one stream per step: [A | B]
};
// Streams of a chunk slot, in units of CB bytes: the cost bytes, the planes
// the pass reads (one: sc; three for FINAL3; seven for FINAL7), and the
// partial sum S (uint16, two units) for ACCUM and FINAL.
template <int NR, int MODE> struct PairSlot {
    static constexpr int NPL = MODE == MODE_SCRATCH ? 0 : (PairRing<NR, MODE>::F3 ? 3 : (MODE == MODE_FINAL7 ? 7 : 1));
    static constexpr bool HAS_S = MODE == MODE_ACCUM || MODE == MODE_FINAL;
    static constexpr int U = 1 + NPL + (HAS_S ? 2 : 0);
    static constexpr int BYTES = PairRing<NR, MODE>::CB * U;
    static constexpr int RING = PairRing<NR, MODE>::NCH * BYTES;
};

// NR bytes from shared memory, zero-extended into a word (NR = 1, 2) or a word (NR = 4).
template <int NR>
__device__ __forceinline__ uint32_t ld_run(const uint8_t *p) {
    if (NR == 1) return *p;
    if (NR == 2) return *(const uint16_t *)p;
    return *(const uint32_t *)p;
}

// Registers of one stream for one step: out[j] = (A byte j, B byte j) as a u16 pair.
template <int NR>
__device__ __forceinline__ void pair_unpack(uint32_t a, uint32_t b, uint32_t (&out)[NR]) {
    if (NR == 1) {
        out[0] = __byte_perm(a, b, 0x5410);                        // a, b zero-extended bytes
    } else if (NR == 2) {
        out[0] = __byte_perm(a, b, 0x6420);
        out[1] = __byte_perm(a, b, 0x6521);
    } else {
#pragma unroll
        for (int j = 0; j < 4; j++) out[j] = __byte_perm(a, b, j | ((4 + j) << 8)) & 0x00FF00FFu;
    }
}

// The line-A bytes (low halves) or line-B bytes (high halves) of the registers, as NR packed bytes.
template <int NR, bool HI>
__device__ __forceinline__ uint32_t pair_pack(const uint32_t (&L)[NR]) {
    constexpr uint32_t s = HI ? 0x62 : 0x40;                       // byte 0 (2) of x, byte 0 (2) of y
    if (NR == 1) return HI ? (L[0] >> 16) & 0xFFu : L[0] & 0xFFu;
    if (NR == 2) return __byte_perm(L[0], L[1], s);
    return __byte_perm(__byte_perm(L[0], L[1], s), __byte_perm(L[2], L[3], s), 0x5410);
}

// NR uint16 sums of line A (sa) and of line B (sb), as words, into packed (A[d], B[d]) registers.
template <int NR>
__device__ __forceinline__ void pair_unpack16(const uint32_t *sa, const uint32_t *sb, uint32_t (&out)[NR]) {
    if (NR == 1) {
        out[0] = __byte_perm(sa[0], sb[0], 0x5410);
    } else {
#pragma unroll
        for (int w = 0; w < NR / 2; w++) {
            out[2 * w] = __byte_perm(sa[w], sb[w], 0x5410);
            out[2 * w + 1] = __byte_perm(sa[w], sb[w], 0x7632);
        }
    }
}

// The line-A (HI = false) or line-B halves of NR packed registers as NR uint16 values, in words.
template <int NR, bool HI>
__device__ __forceinline__ void pair_pack16(const uint32_t (&t)[NR], uint32_t *w) {
    constexpr uint32_t s = HI ? 0x7632 : 0x5410;
    if (NR == 1) w[0] = HI ? t[0] >> 16 : t[0] & 0xFFFFu;
    else {
#pragma unroll
        for (int i = 0; i < NR / 2; i++) w[i] = __byte_perm(t[2 * i], t[2 * i + 1], s);
    }
}

template <int NR>
__device__ __forceinline__ void st_run(uint8_t *p, uint32_t v) {
    if (NR == 1) *p = (uint8_t)v;
    else if (NR == 2) *(uint16_t *)p = (uint16_t)v;
    else *(uint32_t *)p = v;
}

}  // namespace

// Runs warp `warp` of a pass over lines 2*warp and 2*warp+1, in any mode:
//   SCRATCH  L into the plane P.sc
//   STORE    S = sc + L            ACCUM  S += sc + L
//   FINAL    argmin(S + sc + L)    FINAL3 argmin(L + sc + sc2 + sc3) into P.disp
//   FINAL7   argmin(L + sc + sc2 + sc3 + xpl[0..3]) (8 paths)
// (the even-only map of the multi-scale variant in FINAL and FINAL7). SAT: clamp L to
// 255 (multiscale/sgm_ms_ref.c:82). `ring`: this warp's PairSlot<NR, MODE>::RING
// bytes of shared memory (16-byte aligned). All 32 lanes must call it.
template <int NR, int MODE, int SAT, bool KEY16>
__device__ __forceinline__ void path_pair(const LineParams &P, int warp, uint8_t *ring) {
    using RG = PairRing<NR, MODE>;
    constexpr int K = RG::K, NCH = RG::NCH, SB = RG::SB, G = RG::G, CB = RG::CB;
    constexpr int NPL = PairSlot<NR, MODE>::NPL;
    constexpr bool HAS_S = PairSlot<NR, MODE>::HAS_S;
    constexpr int SLOT = PairSlot<NR, MODE>::BYTES;
    constexpr int D = 32 * NR;
    constexpr bool FIN = MODE == MODE_FINAL || MODE == MODE_FINAL3 || MODE == MODE_FINAL3H || MODE == MODE_FINAL7;
    constexpr int KW = (K + 3) / 4;                   // FINAL3H: words of one row's disparities per chunk
    const int lane = threadIdx.x & 31;
    const int la = 2 * warp;
    if (la >= P.nlines) return;                       // whole warp leaves together
    int xa, ya, lena, xb, yb, lenb;
    line_start(P, la, xa, ya, lena);
    line_start(P, la + 1, xb, yb, lenb);              // lenb = 0 if there is no second line
    const int maxlen = max(lena, lenb), minlen = lenb ? min(lena, lenb) : lena;
    // final passes down or up the columns: the two lines are adjacent columns
    // of equal length, so their two disparities of a step are one 16-bit store
    const bool pair_store = P.dx == 0 && lenb == lena && ((ya * P.W + xa) & 1) == 0 && (P.W & 1) == 0 &&
                            xb == xa + 1 && yb == ya && ((uintptr_t)P.disp & 1) == 0;
    const int dx = P.dx, dy = P.dy, step = dy * P.W + dx;
    int pa = ya * P.W + xa, pb = yb * P.W + xb;
    const uint32_t P1 = pk2((uint32_t)P.p1), P2 = pk2((uint32_t)P.p2);
    const uint32_t mlo = (NR == 4 && lane == 0) ? 0x3FFF3FFFu : 0u;    // d = -1 does not exist
    const uint32_t mhi = (NR == 4 && lane == 31) ? 0x3FFF3FFFu : 0u;   // d = D does not exist

    // this lane's 16-byte granules u = lane + 32 h (h < G) of every chunk.
    // Byte streams (cost, planes): byte b = 16 u is step b / SB, line
    // b % SB / D, byte b % D. The sum S (2 units): granules u < 64 G, step
    // b / (2 SB), line b % (2 SB) / (2D), byte b % (2D).
    const uint32_t ring_s = (uint32_t)__cvta_generic_to_shared(ring);
    const long long adv = (long long)K * step * D;
    // even_only planes are compact: the pixel (x, y), x and y even, at
    // (y/2)(W/2) + x/2; two steps along any direction move (dy W/2 + dx) there
    const long long oadv = P.even_only ? (long long)(K / 2) * (dy * (P.W >> 1) + dx) * D : adv;
    long long goff[G], ooff[G];
    int glim[G];
    bool ost[G];
#pragma unroll
    for (int h = 0; h < G; h++) {
        const int gb = (lane + 32 * h) * 16, gk = gb / SB, gr = gb % SB, gl = gr / D, go = gr - gl * D;
        goff[h] = ((long long)(gl ? pb : pa) + (long long)gk * step) * D + go;
        glim[h] = (gl ? lenb : lena) - gk;
        // scratch output: the same granules, into plane P.sc. even_only: only
        // pixels with x and y both even are stored (a chunk is an even number of
        // steps: a granule's parity is the same in every chunk), compact
        const int gx = (gl ? xb : xa) + gk * dx, gy = (gl ? yb : ya) + gk * dy;
        ost[h] = !P.even_only || ((gx | gy) & 1) == 0;
        ooff[h] = P.even_only ? ((long long)(gy >> 1) * (P.W >> 1) + (gx >> 1)) * D + go : goff[h];
    }
    long long soff[2 * G];
    int slim[2 * G];
#pragma unroll
    for (int h = 0; h < 2 * G; h++) {
        const int b = (lane + 32 * h) * 16, k = b / (2 * SB), r = b % (2 * SB), l = r / (2 * D), o = r - l * 2 * D;
        soff[h] = ((long long)(l ? pb : pa) + (long long)k * step) * 2 * D + o;
        slim[h] = HAS_S ? (l ? lenb : lena) - k : 0;
    }
    const uint8_t *src[1 + NPL];
    src[0] = P.C;
    if (NPL >= 1) src[1] = P.sc;
    if (NPL >= 3) { src[2] = P.sc2; src[3] = P.sc3; }
    if (NPL == 7) { src[4] = P.xpl[0]; src[5] = P.xpl[1]; src[6] = P.xpl[2]; src[7] = P.xpl[3]; }
    auto issue = [&](int c) {
        const uint32_t dst = ring_s + (uint32_t)((c % NCH) * SLOT);
#pragma unroll
        for (int h = 0; h < G; h++) {
            if (c * K < glim[h]) {
#pragma unroll
                for (int q = 0; q <= NPL; q++)
                    cp_async16(dst + (uint32_t)(q * CB + (lane + 32 * h) * 16), src[q] + goff[h]);
            }
            goff[h] += adv;
        }
        if (HAS_S) {
#pragma unroll
            for (int h = 0; h < 2 * G; h++) {
                if (c * K < slim[h])
                    cp_async16(dst + (uint32_t)((1 + NPL) * CB + (lane + 32 * h) * 16), (const uint8_t *)P.S + soff[h]);
                soff[h] += 2 * adv;
            }
        }
        cp_async_commit();
    };
    const int nchunks = (maxlen + K - 1) / K;
#pragma unroll
    for (int c = 0; c < NCH - 1; c++) issue(c);

    uint32_t L[NR];
#pragma unroll
    for (int j = 0; j < NR; j++) L[j] = 0u;
    uint32_t mn = 0;                                  // L_prev = 0, min_prev = 0: the first step yields L = C
    // split rows: the first half (hseg 1) leaves each lane's L and the line
    // minimum at its end, the second half (hseg 2) resumes from them
    uint32_t *const hstate = P.state && P.hseg
        ? P.state + ((size_t)((P.dx > 0 ? 0 : 1) * ((P.nlines + 1) >> 1) + warp) * 32 + lane) * (NR + 1) : nullptr;
    if (hstate && P.hseg == 2) {
#pragma unroll
        for (int j = 0; j < NR; j++) L[j] = hstate[j];
        mn = hstate[NR];
    }
    uint32_t dpk[NR];                                 // (d, d) for the argmin keys
#pragma unroll
    for (int j = 0; j < NR; j++) dpk[j] = pk2((uint32_t)(lane * NR + j));
    // even-only scratch: the steps whose pixels are stored (x and y both even)
    // alternate; when both lines agree on which (a chunk is an even number of
    // steps), the others skip staging their L bytes
    int eoph = -1;
    if (MODE == MODE_SCRATCH && SAT != 0 && P.even_only) {
        const int pha = (xa | ya) & 1, phb = lenb ? (xb | yb) & 1 : pha;
        if (pha == phb) eoph = pha;
    }
    pa -= step; pb -= step; xa -= dx; ya -= dy; xb -= dx; yb -= dy;
    const int hw = P.W >> 1;

    uint32_t dacc[2][KW] = {};                        // FINAL3H: the chunk's disparities of rows A and B, byte k = step k
    // one step of both lines; `row`: this step's cost row in the chunk; kk: the step within the chunk
    // EO (even-only scratch, saturating passes only): -1 stage every step's L;
    // 0 (1) stage the even (odd) steps of a chunk only, the others' pixels
    // being odd and never stored
    auto step_once = [&](const uint32_t (&c)[NR], const uint32_t (&ps)[NR], const uint32_t (&sv)[NR], uint8_t *row,
                         int i, int kk, auto full_t, auto eo_t) {
        constexpr bool FULL = decltype(full_t)::value;
        constexpr int EO = decltype(eo_t)::value;
        if (!FULL && i >= maxlen) return;             // past both lines' ends (warp-uniform): L and mn stay
        pa += step; pb += step; xa += dx; ya += dy; xb += dx; yb += dy;
        const uint32_t up = __shfl_up_sync(kFull, L[NR - 1], 1) | mlo;
        const uint32_t dn = __shfl_down_sync(kFull, L[0], 1) | mhi;
        uint32_t w[NR];
#pragma unroll
        for (int j = 0; j < NR; j++) {
            const uint32_t lo = j == 0 ? up : L[j - 1];
            const uint32_t hi = j == NR - 1 ? dn : L[j + 1];
            if (NR >= 4)   // measured: faster at D = 128, slower at D = 64
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
        const uint32_t ra = __reduce_min_sync(kFull, tm & 0xFFFFu);    // line A: low halves
        const uint32_t rb = __reduce_min_sync(kFull, tm);              // line B: high half of the result
        mn = __byte_perm(ra, rb, 0x7610);
        const bool live_a = FULL ? true : i < lena, live_b = FULL ? lenb > 0 : i < lenb;
        if (MODE == MODE_SCRATCH) {
            if (EO >= 0 && (kk & 1) != EO) return;    // even-only: this step's pixels are not stored
            // stage both lines' L bytes in the consumed cost row of this step
            st_run<NR>(row + lane * NR, pair_pack<NR, false>(L));
            st_run<NR>(row + D + lane * NR, pair_pack<NR, true>(L));
            return;
        }
        uint32_t tot[NR];                             // this pass's L plus what the pass reads, per half <= 8*255
#pragma unroll
        for (int j = 0; j < NR; j++) {
            tot[j] = L[j] + ps[j];
            if (HAS_S) tot[j] += sv[j];
        }
        if (MODE == MODE_STORE || MODE == MODE_ACCUM) {
            uint32_t wa[NR > 1 ? NR / 2 : 1], wb[NR > 1 ? NR / 2 : 1];
            pair_pack16<NR, false>(tot, wa);
            pair_pack16<NR, true>(tot, wb);
            uint16_t *Sa = P.S + (long long)pa * D + lane * NR, *Sb = P.S + (long long)pb * D + lane * NR;
            if (NR == 1) {
                if (live_a) *Sa = (uint16_t)wa[0];
                if (live_b) *Sb = (uint16_t)wb[0];
            } else if (NR == 2) {
                if (live_a) *(uint32_t *)Sa = wa[0];
                if (live_b) *(uint32_t *)Sb = wb[0];
            } else {
                if (live_a) *(uint2 *)Sa = make_uint2(wa[0], wa[1]);
                if (live_b) *(uint2 *)Sb = make_uint2(wb[0], wb[1]);
            }
            return;
        }
        // final passes: argmin over d, the lowest d winning ties; every lane reaches the reductions
        if (MODE == MODE_FINAL3H && KEY16) {
            // gather the chunk's disparities per row: byte kk & 3 of word kk >> 2 takes the low
            // byte of line A's minimal key (d in its low 6 bits) and byte 2 of the packed
            // minimum (line B's key in the high half); the words are masked to 6-bit bytes
            // when the chunk is stored
            uint32_t k = tot[0] * 64u + dpk[0];                    // S*64 + d (S <= 1016)
#pragma unroll
            for (int j = 1; j < NR; j++) k = vmin2(k, tot[j] * 64u + dpk[j]);
            const uint32_t ra = __reduce_min_sync(kFull, k & 0xFFFFu);
            const uint32_t rb = __reduce_min_sync(kFull, k);
            const int q = kk & 3, wq = kk >> 2;
            dacc[0][wq] = q == 0 ? ra : __byte_perm(dacc[0][wq], ra, q == 1 ? 0x3240 : (q == 2 ? 0x3410 : 0x4210));
            dacc[1][wq] = __byte_perm(q == 0 ? rb : dacc[1][wq], rb, q == 0 ? 0x0002 : (q == 1 ? 0x3260 : (q == 2 ? 0x3610 : 0x6210)));
            return;
        }
        uint32_t da, db;
        if (KEY16) {
            uint32_t k = kFull;
#pragma unroll
            for (int j = 0; j < NR; j++) k = vmin2(k, tot[j] * 64u + dpk[j]);       // S*64 + d (S <= 1016)
            da = __reduce_min_sync(kFull, k & 0xFFFFu) & 0x3Fu;
            db = (__reduce_min_sync(kFull, k) >> 16) & 0x3Fu;
        } else {
            uint32_t ka = kFull, kb = kFull;
#pragma unroll
            for (int j = 0; j < NR; j++) {
                const uint32_t d = (uint32_t)(lane * NR + j);
                ka = min(ka, ((tot[j] & 0xFFFFu) << 8) | d);
                kb = min(kb, ((tot[j] >> 16) << 8) | d);
            }
            da = __reduce_min_sync(kFull, ka) & 0xFFu;
            db = __reduce_min_sync(kFull, kb) & 0xFFu;
        }
        if (MODE == MODE_FINAL3H) {                   // every lane holds da and db: gather them per chunk
            dacc[0][kk >> 2] |= da << (8 * (kk & 3));
            dacc[1][kk >> 2] |= db << (8 * (kk & 3));
            return;
        }
        if (lane == 0) {
            if ((MODE == MODE_FINAL || MODE == MODE_FINAL7) && P.even_only) {   // multi-scale: the map at (2x, 2y) only
                if (live_a && !((xa | ya) & 1)) P.disp[(long long)(ya >> 1) * hw + (xa >> 1)] = (uint8_t)da;
                if (live_b && !((xb | yb) & 1)) P.disp[(long long)(yb >> 1) * hw + (xb >> 1)] = (uint8_t)db;
            } else if (pair_store) {
                if (live_a) *(uint16_t *)(P.disp + pa) = (uint16_t)(da | (db << 8));
            } else {
                if (live_a) P.disp[pa] = (uint8_t)da;
                if (live_b) P.disp[pb] = (uint8_t)db;
            }
        }
    };

    for (int ch = 0; ch < nchunks; ch++) {
        cp_async_wait<NCH - 2>();                     // chunk ch has landed (this lane's copies)
        __syncwarp();                                 // ... and every lane's; slot ch-1 is free
        issue(ch + NCH - 1);
        uint8_t *chunk = ring + (ch % NCH) * SLOT;
        // the chunk's inputs, read before its steps run: costs, the sum of the
        // planes the pass reads (off the recurrence: it only enters the total),
        // and the partial sum S
        uint32_t c[K][NR], ps[K][NR], sv[K][NR];
#pragma unroll
        for (int k = 0; k < K; k++) {
            const uint8_t *r = chunk + k * SB + lane * NR;
            pair_unpack<NR>(ld_run<NR>(r), ld_run<NR>(r + D), c[k]);
#pragma unroll
            for (int q = 0; q < NPL; q++) {
                uint32_t pq[NR];
                pair_unpack<NR>(ld_run<NR>(r + (q + 1) * CB), ld_run<NR>(r + (q + 1) * CB + D), pq);
#pragma unroll
                for (int j = 0; j < NR; j++) ps[k][j] = q == 0 ? pq[j] : ps[k][j] + pq[j];
            }
            if (HAS_S) {
                const uint8_t *sr = chunk + (1 + NPL) * CB + k * 2 * SB + lane * 2 * NR;
                uint32_t sa[NR > 1 ? NR / 2 : 1], sb[NR > 1 ? NR / 2 : 1];
                if (NR == 1) { sa[0] = *(const uint16_t *)sr; sb[0] = *(const uint16_t *)(sr + 2 * D); }
                else if (NR == 2) { sa[0] = *(const uint32_t *)sr; sb[0] = *(const uint32_t *)(sr + 2 * D); }
                else {
                    const uint2 a2 = *(const uint2 *)sr, b2 = *(const uint2 *)(sr + 2 * D);
                    sa[0] = a2.x; sa[1] = a2.y; sb[0] = b2.x; sb[1] = b2.y;
                }
                pair_unpack16<NR>(sa, sb, sv[k]);
            }
        }
        const long long pa0 = pa + step, pb0 = pb + step;   // the chunk's first pixel of each line
        if (MODE == MODE_FINAL3H && !KEY16) {
#pragma unroll
            for (int w = 0; w < KW; w++) dacc[0][w] = dacc[1][w] = 0u;
        }
        auto steps = [&](auto eo_t) {
            if ((ch + 1) * K <= minlen) {
#pragma unroll
                for (int k = 0; k < K; k++)
                    step_once(c[k], ps[k], sv[k], chunk + k * SB, ch * K + k, k, std::true_type{}, eo_t);
            } else {
#pragma unroll
                for (int k = 0; k < K; k++)
                    step_once(c[k], ps[k], sv[k], chunk + k * SB, ch * K + k, k, std::false_type{}, eo_t);
            }
        };
        if constexpr (MODE == MODE_SCRATCH && SAT != 0) {
            if (eoph == 0) steps(std::integral_constant<int, 0>{});
            else if (eoph == 1) steps(std::integral_constant<int, 1>{});
            else steps(std::integral_constant<int, -1>{});
        } else {
            steps(std::integral_constant<int, -1>{});
        }
        if (MODE == MODE_FINAL3H && lane == 0) {
            // row r's live steps of the chunk go to disp[p0 + dx*k]: one word store per 4 steps
            // when the chunk is whole and its span word-aligned, byte stores otherwise
#pragma unroll
            for (int r = 0; r < 2; r++) {
                const int n = min(K, (r ? lenb : lena) - ch * K);
                if (n <= 0) continue;
                const long long p0 = r ? pb0 : pa0;
                const long long lo = dx > 0 ? p0 : p0 - (K - 1);     // lowest address of a whole chunk
                constexpr uint32_t dm = KEY16 ? 0x3F3F3F3Fu : 0xFFFFFFFFu;
                if (n == K && K % 4 == 0 && (((uintptr_t)(P.disp + lo)) & 3) == 0) {
#pragma unroll
                    for (int w = 0; w < KW; w++)
                        ((uint32_t *)(P.disp + lo))[w] =
                            dm & (dx > 0 ? dacc[r][w] : __byte_perm(dacc[r][KW - 1 - w], 0, 0x0123));
                } else {
#pragma unroll
                    for (int k = 0; k < K; k++)
                        if (k < n) P.disp[p0 + dx * k] = (uint8_t)((dacc[r][k >> 2] >> (8 * (k & 3))) & dm);
                }
            }
        }
        if (MODE == MODE_SCRATCH) {
            __syncwarp();                             // every lane's L bytes of the chunk are staged
#pragma unroll
            for (int h = 0; h < G; h++) {
                if (ost[h] && ch * K < glim[h])
                    *(uint4 *)(P.sc + ooff[h]) = *(const uint4 *)(chunk + (lane + 32 * h) * 16);
                ooff[h] += oadv;
            }
        }
    }
    cp_async_wait<0>();                               // no copy outlives the kernel
    if (hstate && P.hseg == 1) {
#pragma unroll
        for (int j = 0; j < NR; j++) hstate[j] = L[j];
        hstate[NR] = mn;
    }
}

}  // namespace sgmgb
