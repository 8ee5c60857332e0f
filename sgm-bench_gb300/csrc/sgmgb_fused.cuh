// sgmgb_fused.cuh -- the first half of the horizontal passes of the fused
// schedule, with the matching costs computed on the way. Device code used by
// the per-pass kernel (sgmgb_fused.cu) and the batch kernel (sgmgb_batch.cu).
//
// A warp walks two rows (y, y+1) in one direction over the first half of the
// row: L->R over x in [0, W/2), R->L over x in [W/2, W) from W-1 down. At each
// step it computes the pixel's D Hamming costs from the census descriptors,
// C(x, y, d) = popcount(cl[y][x] ^ cr[y][x-d]), 62 where x - d < 0
// (common/sgm_ref.c:44-56), runs the recurrence of common/sgm_ref.c:61-72 in
// the two-lines-per-warp layout of sgmgb_pair.cuh, and stores both the costs
// (into the cost volume, which the vertical passes and the second halves
// read) and L (into the half-row plane, which the other direction's second
// half reads). At the half's end it leaves each lane's L registers and the
// line minimum for the second half, which resumes there.
//
// The two halves of each direction cover every pixel once, so every cost is
// computed once, as the separate cost kernel would; the population counts
// fill issue slots of this latency-bound pass (a horizontal pass has only H/2
// warps per direction) instead of taking a pass of their own, and the cost
// volume is written without being read first.
//
// Descriptors: the census is L2-resident (16 bytes per pixel). Per chunk of K
// steps a warp copies, with 8-byte cp.async, the K cl descriptors of each row
// and the K cr descriptors that enter the row's sliding window (the window of
// cr[x - D + 1 .. x] a step needs). Lane l reads cr[x - NR*l - j] for its NR
// disparities; as x moves one step only one of them is new (a shift register
// keeps the others). The window is stored with the XOR swizzle
// i ^ ((i >> 4) & (NR - 1)), which makes those reads free of bank conflicts
// for NR = 1, 2 and 4 (checked exhaustively over x and both directions).
#pragma once
#include "sgmgb_path.cuh"
#include "sgmgb_pair.cuh"

namespace sgmgb {

namespace {

template <int NR> struct HCost {
    static constexpr int D = 32 * NR;
    static constexpr int K = 8;                                  // steps per chunk
    static constexpr int NCH = 4;                                // chunks in the ring (NCH - 1 in flight)
    // cr window per row: it must hold the oldest descriptor a chunk reads and
    // the newest one the copies in flight write: NCH*K + D - 1 of them
    static constexpr int CAP = (NCH * K + D - 1) <= 128 ? 128 : 256;
    static constexpr int CL = NCH * 2 * K;                       // cl ring: [chunk][row][step]
    static constexpr int BYTES = (CL + 2 * CAP) * 8;             // one warp's shared memory
};

__device__ __forceinline__ void cp_async8(uint32_t dst_smem, const void *src) {
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"(dst_smem), "l"(src) : "memory");
}

// window slot of descriptor x (any integer x; negative ones are never used for a valid cost)
template <int NR, int CAP>
__device__ __forceinline__ int win_pos(int x) {
    return (x ^ ((x >> 4) & (NR - 1))) & (CAP - 1);
}

template <int NR, int DX>
__device__ __forceinline__ void path_hcost(const LineParams &P, int pair, uint64_t *smem) {
    using HC = HCost<NR>;
    constexpr int D = HC::D, K = HC::K, NCH = HC::NCH, CAP = HC::CAP;
    const int lane = threadIdx.x & 31;
    const int npairs = (P.H + 1) >> 1;
    if (pair >= npairs) return;                                  // whole warp leaves together
    const int W = P.W, m = W >> 1;
    const int ya = 2 * pair, yb = ya + 1;
    const bool has_b = yb < P.H;
    const int x0 = DX > 0 ? 0 : W - 1;                           // first pixel of this direction's half
    const int len = DX > 0 ? m : W - m;
    const uint64_t *cla = P.cl + (size_t)ya * W, *cra_g = P.cr + (size_t)ya * W;
    const uint64_t *clb = P.cl + (size_t)(has_b ? yb : ya) * W, *crb_g = P.cr + (size_t)(has_b ? yb : ya) * W;
    uint64_t *clr = smem;                                        // [NCH][2][K]
    const uint64_t *wa = smem + HC::CL, *wb = wa + CAP;          // cr windows of rows a and b
    const uint32_t clr_s = (uint32_t)__cvta_generic_to_shared(clr);
    const uint32_t win_s = (uint32_t)__cvta_generic_to_shared(smem + HC::CL);
    uint8_t *cost = const_cast<uint8_t *>(P.C);                  // this pass writes the cost volume the others read

    // chunk c: steps [cK, cK + K) of the half. Lanes 0..15 copy the chunk's cl
    // (8 per row); lanes 16..31 the cr descriptors entering the window (8 per
    // row), the first chunk also the window's initial D - 1.
    auto issue = [&](int c) {
        const int s0 = c * K;
        if (s0 < len) {
            const int n = min(K, len - s0);
            const int r = (lane >> 3) & 1, q = lane & 7;
            if (lane < 16) {
                if (q < n)
                    cp_async8(clr_s + (uint32_t)((((c % NCH) * 2 + r) * K + q) * 8), (r ? clb : cla) + (x0 + DX * (s0 + q)));
            } else {
                int lo, hi;
                if (DX > 0) { lo = x0 + s0 - (c == 0 ? D - 1 : 0); hi = x0 + s0 + n - 1; }
                else { lo = x0 - s0 - (n - 1) - (D - 1); hi = c == 0 ? x0 : x0 - s0 - (D - 1); }
                lo = max(lo, 0);
                hi = min(hi, W - 1);
                const uint64_t *g = r ? crb_g : cra_g;
                for (int i = lo + q; i <= hi; i += 8)
                    cp_async8(win_s + (uint32_t)((r * CAP + win_pos<NR, CAP>(i)) * 8), g + i);
            }
        }
        cp_async_commit();
    };
    const int nchunks = (len + K - 1) / K;
#pragma unroll
    for (int c = 0; c < NCH - 1; c++) issue(c);

    const uint32_t P1 = pk2((uint32_t)P.p1), P2 = pk2((uint32_t)P.p2);
    const uint32_t mlo = (NR == 4 && lane == 0) ? 0x3FFF3FFFu : 0u;    // d = -1 does not exist
    const uint32_t mhi = (NR == 4 && lane == 31) ? 0x3FFF3FFFu : 0u;   // d = D does not exist
    uint32_t L[NR];
#pragma unroll
    for (int j = 0; j < NR; j++) L[j] = 0u;
    uint32_t mn = 0;                                             // L_prev = 0, min_prev = 0: the first step yields L = C
    uint64_t ca[NR], cb[NR];                                     // cr[x - NR*lane - j] of rows a and b
    long long offa = ((long long)ya * W + x0) * D + lane * NR;   // this lane's bytes of pixel (x, ya)
    long long offb = ((long long)yb * W + x0) * D + lane * NR;

    // one step of both rows at x: its costs (computed here, stored into the
    // cost volume), the recurrence, and L into the plane; VALID: every x - d
    // of the step is >= 0
    auto step_once = [&](const uint64_t *clc, int k, int x, auto valid_t) {
        constexpr bool VALID = decltype(valid_t)::value;
        if (DX > 0) {
#pragma unroll
            for (int j = NR - 1; j > 0; j--) { ca[j] = ca[j - 1]; cb[j] = cb[j - 1]; }
            const int p = win_pos<NR, CAP>(x - NR * lane);
            ca[0] = wa[p]; cb[0] = wb[p];
        } else {
#pragma unroll
            for (int j = 0; j < NR - 1; j++) { ca[j] = ca[j + 1]; cb[j] = cb[j + 1]; }
            const int p = win_pos<NR, CAP>(x - NR * lane - (NR - 1));
            ca[NR - 1] = wa[p]; cb[NR - 1] = wb[p];
        }
        const uint64_t la = clc[k], lb = clc[K + k];
        uint32_t c[NR];
#pragma unroll
        for (int j = 0; j < NR; j++) {
            uint32_t a = (uint32_t)__popcll(la ^ ca[j]), b = (uint32_t)__popcll(lb ^ cb[j]);
            if (!VALID && x - NR * lane - j < 0) a = b = (uint32_t)kInvalidPlain;
            c[j] = __byte_perm(a, b, 0x5410);
        }
        const uint32_t up = __shfl_up_sync(kFull, L[NR - 1], 1) | mlo;
        const uint32_t dn = __shfl_down_sync(kFull, L[0], 1) | mhi;
        uint32_t w[NR];
#pragma unroll
        for (int j = 0; j < NR; j++) {
            const uint32_t lo = j == 0 ? up : L[j - 1];
            const uint32_t hi = j == NR - 1 ? dn : L[j + 1];
            if (NR >= 4) w[j] = j == 0 ? nbr_min(L[j], hi, lo, P1) : nbr_min(L[j], lo, hi, P1);
            else w[j] = vmin2(L[j], vmin2(lo, hi) + P1);
        }
        const uint32_t E = mn + P2;
        uint32_t tm = kFull;
#pragma unroll
        for (int j = 0; j < NR; j++) {
            const uint32_t v = vmin2(w[j], E) + c[j] - mn;
            L[j] = v;
            tm = vmin2(tm, v);
        }
        const uint32_t ra = __reduce_min_sync(kFull, tm & 0xFFFFu);
        const uint32_t rb = __reduce_min_sync(kFull, tm);
        mn = __byte_perm(ra, rb, 0x7610);
        st_run<NR>(cost + offa, pair_pack<NR, false>(c));
        st_run<NR>(P.sc + offa, pair_pack<NR, false>(L));
        if (has_b) {
            st_run<NR>(cost + offb, pair_pack<NR, true>(c));
            st_run<NR>(P.sc + offb, pair_pack<NR, true>(L));
        }
        offa += DX * D;
        offb += DX * D;
    };

    for (int ch = 0; ch < nchunks; ch++) {
        cp_async_wait<NCH - 2>();                                // chunk ch has landed (this lane's copies)
        __syncwarp();                                            // ... and every lane's; chunk ch-1 is consumed
        issue(ch + NCH - 1);
        const int s0 = ch * K, xc = x0 + DX * s0;
        if (ch == 0) {
            // the descriptors the first step shifts in from "earlier" steps
#pragma unroll
            for (int i = 0; i < NR - 1; i++) {
                const int jd = DX > 0 ? i : i + 1;               // the slot it lands in before the first shift
                const int p = win_pos<NR, CAP>(xc - NR * lane - (DX > 0 ? i + 1 : i));
                ca[jd] = wa[p];
                cb[jd] = wb[p];
            }
        }
        const uint64_t *clc = clr + (ch % NCH) * 2 * K;
        const int n = min(K, len - s0);
        const int xmin = DX > 0 ? xc : xc - (n - 1);
        if (n == K && xmin >= D - 1) {
#pragma unroll
            for (int k = 0; k < K; k++) step_once(clc, k, xc + DX * k, std::true_type{});
        } else {
#pragma unroll
            for (int k = 0; k < K; k++)
                if (k < n) step_once(clc, k, xc + DX * k, std::false_type{});   // past the half's end: the state stays
        }
    }
    cp_async_wait<0>();                                          // no copy outlives the kernel
    uint32_t *st = P.state + ((size_t)((DX > 0 ? 0 : 1) * npairs + pair) * 32 + lane) * (NR + 1);
#pragma unroll
    for (int j = 0; j < NR; j++) st[j] = L[j];
    st[NR] = mn;
}

}  // namespace

}  // namespace sgmgb
