// sgmgb_kernels.cu -- census, prefilters and the generic path kernel.
//
// Path kernel layout: one warp owns one line of one direction. The D
// disparities are spread over the lanes, DPL per lane, held in DPL/2
// registers of packed u16 pairs. Lane l owns d in [l*DPL, (l+1)*DPL); register
// j holds (d0 + j, d0 + DPL/2 + j), so the d-1 / d+1 neighbours of every
// register are other registers of the same lane except at the two ends,
// which come from the adjacent lanes by shuffle.
//
// Packed arithmetic: min.u16x2 runs at the full integer rate on sm_103; the
// additions use plain 32-bit IADD because no half can carry (values stay
// below 0x4000 + 255). The saturating adds of the reference need no
// clamps here: with a = prev[d] <= 255 in the minimum,
//   min(a, sat(lo+P1), sat(hi+P1), sat(mn+P2)) == min(a, lo+P1, hi+P1, mn+P2)
// because any term that saturates is >= 255 >= a (common/sgm_ref.c:61-72).
//
// The per-step minimum over d is a warp REDUX. It is taken one step ahead:
//   mn(x) = min( min_d(c + w), min_d(c) + mn(x-1) + P2 ) - mn(x-1)
// where w = min(prev, nbr + P1) depends only on L(x-1). The reduction for
// pixel x is issued before L(x) is formed and consumed one iteration later,
// so its latency overlaps the next step instead of sitting on the critical
// path. For the multi-scale variant the final clamp to 255 is applied to
// both L and mn (multiscale/sgm_ms_ref.c:82).
#include "sgmgb_kernels.cuh"

namespace sgmgb {

namespace {

constexpr uint32_t kInfPk = 0x3FFF3FFFu;   // "no such disparity": never wins a min
constexpr uint32_t kFull = 0xFFFFFFFFu;

__device__ __forceinline__ uint32_t vmin2(uint32_t a, uint32_t b) {
    uint32_t r;
    asm("min.u16x2 %0, %1, %2;" : "=r"(r) : "r"(a), "r"(b));
    return r;
}
__device__ __forceinline__ uint32_t pk2(uint32_t v) { return v | (v << 16); }
__device__ __forceinline__ uint32_t fold_min(uint32_t v) { return min(v & 0xFFFFu, v >> 16); }
__device__ __forceinline__ int clampi(int v, int lo, int hi) { return v < lo ? lo : (v > hi ? hi : v); }

// half-word k (natural disparity order within the lane) of the register file
template <int NR>
__device__ __forceinline__ uint32_t hw_at(const uint32_t (&r)[NR], int k) {
    return (r[k % NR] >> (16 * (k / NR))) & 0xFFFFu;
}

}  // namespace

// ---------------------------------------------------------------------------
// Census 9x7 of two images at once (blockIdx.z picks the image). A 32x8 tile
// plus its 4/3-pixel halo is staged in shared memory with clamped (edge-
// replicated) coordinates; bit n is set iff the neighbour is darker than the
// centre, n running over dy (outer) then dx, skipping the centre
// (common/sgm_ref.c:23-41).
// ---------------------------------------------------------------------------
constexpr int CT_W = 32, CT_H = 8, CR_X = 4, CR_Y = 3;

__global__ void __launch_bounds__(CT_W * CT_H)
k_census2(const uint8_t *__restrict__ im0, const uint8_t *__restrict__ im1,
          uint64_t *__restrict__ out0, uint64_t *__restrict__ out1, int W, int H) {
    __shared__ uint8_t tile[CT_H + 2 * CR_Y][CT_W + 2 * CR_X];
    const uint8_t *im = blockIdx.z ? im1 : im0;
    uint64_t *out = blockIdx.z ? out1 : out0;
    const int x0 = blockIdx.x * CT_W, y0 = blockIdx.y * CT_H;
    const int tid = threadIdx.y * CT_W + threadIdx.x;
    constexpr int TW = CT_W + 2 * CR_X, TH = CT_H + 2 * CR_Y;
    for (int i = tid; i < TW * TH; i += CT_W * CT_H) {
        const int ty = i / TW, tx = i % TW;
        const int gy = clampi(y0 + ty - CR_Y, 0, H - 1), gx = clampi(x0 + tx - CR_X, 0, W - 1);
        tile[ty][tx] = im[(size_t)gy * W + gx];
    }
    __syncthreads();
    const int x = x0 + threadIdx.x, y = y0 + threadIdx.y;
    if (x >= W || y >= H) return;
    const int cx = threadIdx.x + CR_X, cy = threadIdx.y + CR_Y;
    const uint32_t c = tile[cy][cx];
    uint64_t bits = 0;
    int n = 0;
#pragma unroll
    for (int dy = -CR_Y; dy <= CR_Y; dy++)
#pragma unroll
        for (int dx = -CR_X; dx <= CR_X; dx++) {
            if (dx == 0 && dy == 0) continue;
            bits |= (uint64_t)(tile[cy + dy][cx + dx] < c) << n;
            n++;
        }
    out[(size_t)y * W + x] = bits;
}

// 3x3 horizontal Sobel, clamped coordinates, mapped to clamp(128 + (gx >> 3))
// with an arithmetic shift (multiscale/sgm_ms_ref.c:47-54).
__global__ void k_sobel2(const uint8_t *__restrict__ im0, const uint8_t *__restrict__ im1,
                         uint8_t *__restrict__ out0, uint8_t *__restrict__ out1, int W, int H) {
    const uint8_t *im = blockIdx.z ? im1 : im0;
    uint8_t *out = blockIdx.z ? out1 : out0;
    const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y * blockDim.y + threadIdx.y;
    if (x >= W || y >= H) return;
    const int xm = clampi(x - 1, 0, W - 1), xp = clampi(x + 1, 0, W - 1);
    const uint8_t *rm = im + (size_t)clampi(y - 1, 0, H - 1) * W;
    const uint8_t *r0 = im + (size_t)y * W;
    const uint8_t *rp = im + (size_t)clampi(y + 1, 0, H - 1) * W;
    const int gx = ((int)rm[xp] - rm[xm]) + 2 * ((int)r0[xp] - r0[xm]) + ((int)rp[xp] - rp[xm]);
    out[(size_t)y * W + x] = (uint8_t)clampi(128 + (gx >> 3), 0, 255);
}

// 2x2 box mean with rounding; output (W/2) x (H/2) (multiscale/sgm_ms_ref.c:145-150).
__global__ void k_half2(const uint8_t *__restrict__ im0, const uint8_t *__restrict__ im1,
                        uint8_t *__restrict__ out0, uint8_t *__restrict__ out1, int W, int H) {
    const uint8_t *im = blockIdx.z ? im1 : im0;
    uint8_t *out = blockIdx.z ? out1 : out0;
    const int w = W / 2, h = H / 2;
    const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y * blockDim.y + threadIdx.y;
    if (x >= w || y >= h) return;
    const uint8_t *a = im + (size_t)(2 * y) * W + 2 * x, *b = a + W;
    out[(size_t)y * w + x] = (uint8_t)(((int)a[0] + a[1] + b[0] + b[1] + 2) >> 2);
}

// ---------------------------------------------------------------------------
// Path kernel
// ---------------------------------------------------------------------------
template <int DPL, int CK>
__device__ __forceinline__ void lane_cost(const LineParams &P, int x, int y, int d0,
                                          uint32_t (&c)[DPL / 2]) {
    constexpr int NR = DPL / 2;
    constexpr uint32_t kInvalid = (CK == COST_PLAIN) ? 62u : 63u;
    const uint64_t *rowr = P.cr + (size_t)y * P.W;
    const uint64_t a = __ldg(P.cl + (size_t)y * P.W + x);
    uint32_t v[DPL];
#pragma unroll
    for (int k = 0; k < DPL; k++) {
        const int xr = x - (d0 + k);
        v[k] = xr >= 0 ? (uint32_t)__popcll(a ^ __ldg(rowr + xr)) : kInvalid;
    }
    if (CK == COST_MS2) {
        // half-scale cost at (x/2, y/2, d/2); d0 is even so the pair (d0+k, d0+k+1)
        // shares one half-scale disparity.
        const int hw = P.W >> 1, hx = x >> 1, hy = y >> 1;
        const uint64_t *hrowr = P.cr1 + (size_t)hy * hw;
        const uint64_t a1 = __ldg(P.cl1 + (size_t)hy * hw + hx);
#pragma unroll
        for (int k = 0; k < DPL; k += 2) {
            const int hxr = hx - ((d0 + k) >> 1);
            const uint32_t v1 = hxr >= 0 ? (uint32_t)__popcll(a1 ^ __ldg(hrowr + hxr)) : 63u;
            v[k] = (v[k] + v1 + 1) >> 1;
            v[k + 1] = (v[k + 1] + v1 + 1) >> 1;
        }
    }
#pragma unroll
    for (int j = 0; j < NR; j++) c[j] = v[j] | (v[j + NR] << 16);
}

template <int DPL, int MODE>
__device__ __forceinline__ void emit(const LineParams &P, int x, int y, int d0, int lane, bool active,
                                     const uint32_t (&L)[DPL / 2]) {
    constexpr int NR = DPL / 2;
    const size_t p = (size_t)y * P.W + x;
    const size_t off = p * P.D + d0;
    if (MODE == MODE_SCRATCH) {
        if (!active) return;
        uint8_t *dst = P.sc + off;
        if (DPL == 2) {
            *(uint16_t *)dst = (uint16_t)(hw_at<NR>(L, 0) | (hw_at<NR>(L, 1) << 8));
        } else if (DPL == 4) {
            uint32_t w = 0;
#pragma unroll
            for (int k = 0; k < 4; k++) w |= hw_at<NR>(L, k) << (8 * k);
            *(uint32_t *)dst = w;
        } else if (DPL == 8) {
            uint32_t w0 = 0, w1 = 0;
#pragma unroll
            for (int k = 0; k < 4; k++) {
                w0 |= hw_at<NR>(L, k) << (8 * k);
                w1 |= hw_at<NR>(L, k + 4) << (8 * k);
            }
            *(uint2 *)dst = make_uint2(w0, w1);
        } else {
#pragma unroll
            for (int k = 0; k < DPL; k++) dst[k] = (uint8_t)hw_at<NR>(L, k);
        }
        return;
    }
    // sum of the pair in natural order: tot[i] = (d0+2i, d0+2i+1)
    uint32_t tot[NR];
    if (active) {
        const uint8_t *src = P.sc + off;
        uint32_t scb[DPL];
        if (DPL == 2) {
            const uint32_t w = *(const uint16_t *)src;
            scb[0] = w & 0xFF; scb[1] = w >> 8;
        } else if (DPL == 4) {
            const uint32_t w = *(const uint32_t *)src;
#pragma unroll
            for (int k = 0; k < 4; k++) scb[k] = (w >> (8 * k)) & 0xFF;
        } else if (DPL == 8) {
            const uint2 w = *(const uint2 *)src;
#pragma unroll
            for (int k = 0; k < 4; k++) { scb[k] = (w.x >> (8 * k)) & 0xFF; scb[k + 4] = (w.y >> (8 * k)) & 0xFF; }
        } else {
#pragma unroll
            for (int k = 0; k < DPL; k++) scb[k] = src[k];
        }
#pragma unroll
        for (int i = 0; i < NR; i++)
            tot[i] = (hw_at<NR>(L, 2 * i) + scb[2 * i]) | ((hw_at<NR>(L, 2 * i + 1) + scb[2 * i + 1]) << 16);
        if (MODE == MODE_ACCUM || MODE == MODE_FINAL) {
            const uint32_t *s = (const uint32_t *)(P.S + off);
#pragma unroll
            for (int i = 0; i < NR; i++) tot[i] += s[i];   // u16 pairs, no carry (S <= 2040)
        }
    }
    if (MODE == MODE_STORE || MODE == MODE_ACCUM) {
        if (!active) return;
        uint32_t *s = (uint32_t *)(P.S + off);
#pragma unroll
        for (int i = 0; i < NR; i++) s[i] = tot[i];
        return;
    }
    // MODE_FINAL: argmin over d with the lowest d winning ties.
    if (P.even_only && ((x | y) & 1)) return;
    uint32_t key = kFull;
    if (active) {
#pragma unroll
        for (int i = 0; i < NR; i++) {
            key = min(key, ((tot[i] & 0xFFFFu) << 8) | (uint32_t)(d0 + 2 * i));
            key = min(key, ((tot[i] >> 16) << 8) | (uint32_t)(d0 + 2 * i + 1));
        }
    }
    key = __reduce_min_sync(kFull, key);
    if (lane == 0) {
        if (P.even_only) P.disp[(size_t)(y >> 1) * (P.W >> 1) + (x >> 1)] = (uint8_t)(key & 0xFF);
        else P.disp[p] = (uint8_t)(key & 0xFF);
    }
}

template <int DPL, int MODE, int CK, int SAT>
__global__ void __launch_bounds__(256)
k_line(const LineParams P) {
    constexpr int NR = DPL / 2;
    const int lane = threadIdx.x & 31;
    const int line = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    if (line >= P.nlines) return;   // whole warp leaves together
    const bool active = lane < P.nl;
    const bool last = lane == P.nl - 1;
    const int d0 = lane * DPL;
    const int dx = P.dx, dy = P.dy;

    // entry pixel and length of this line
    const int xe = dx > 0 ? 0 : P.W - 1, ye = dy > 0 ? 0 : P.H - 1;
    int x, y;
    if (dy == 0) { x = xe; y = line; }
    else if (dx == 0) { x = line; y = ye; }
    else if (line < P.H) { x = xe; y = line; }
    else { x = xe + dx * (line - P.H + 1); y = ye; }
    int len;
    if (dy == 0) len = P.W;
    else if (dx == 0) len = P.H;
    else len = min(dx > 0 ? P.W - x : x + 1, dy > 0 ? P.H - y : y + 1);

    const uint32_t P1 = pk2((uint32_t)P.p1);
    const uint32_t p2 = (uint32_t)P.p2;

    uint32_t L[NR], c[NR];
    // first pixel of the line: L = C
    if (active) lane_cost<DPL, CK>(P, x, y, d0, c);
#pragma unroll
    for (int j = 0; j < NR; j++) L[j] = active ? c[j] : kInfPk;
    uint32_t cm = kFull;
    if (active) {
        uint32_t t = c[0];
#pragma unroll
        for (int j = 1; j < NR; j++) t = vmin2(t, c[j]);
        cm = fold_min(t);
    }
    uint32_t mn = __reduce_min_sync(kFull, cm);
    emit<DPL, MODE>(P, x, y, d0, lane, active, L);

    uint32_t pV = 0, pC = 0;
    bool pending = false;
    for (int i = 1; i < len; i++) {
        x += dx; y += dy;
        if (active) lane_cost<DPL, CK>(P, x, y, d0, c);
        else {
#pragma unroll
            for (int j = 0; j < NR; j++) c[j] = 0;
        }
        // neighbours d-1 / d+1 of every register
        const uint32_t up = __shfl_up_sync(kFull, L[NR - 1], 1);
        const uint32_t dn = __shfl_down_sync(kFull, L[0], 1);
        uint32_t lo0 = __byte_perm(up, L[NR - 1], 0x5432);   // (prev lane's last d, own d0+NR-1)
        uint32_t hiL = __byte_perm(L[0], dn, 0x5432);        // (own d0+NR, next lane's d0+DPL)
        if (lane == 0) lo0 = (lo0 & 0xFFFF0000u) | 0x3FFFu;
        if (last) hiL = (hiL & 0x0000FFFFu) | 0x3FFF0000u;
        uint32_t w[NR];
        uint32_t cwm = 0xFFFFFFFFu, ccm = 0xFFFFFFFFu;
#pragma unroll
        for (int j = 0; j < NR; j++) {
            const uint32_t lo = j == 0 ? lo0 : L[j - 1];
            const uint32_t hi = j == NR - 1 ? hiL : L[j + 1];
            w[j] = vmin2(L[j], vmin2(lo, hi) + P1);
            cwm = vmin2(cwm, w[j] + c[j]);
            ccm = vmin2(ccm, c[j]);
        }
        const uint32_t rV = __reduce_min_sync(kFull, active ? fold_min(cwm) : kFull);
        const uint32_t rC = __reduce_min_sync(kFull, active ? fold_min(ccm) : kFull);
        if (pending) {
            uint32_t n = min(pV, pC + mn + p2) - mn;
            if (SAT) n = min(n, 255u);
            mn = n;
        }
        const uint32_t E = pk2(mn + p2), M = pk2(mn);
#pragma unroll
        for (int j = 0; j < NR; j++) {
            uint32_t v = vmin2(w[j], E) + c[j] - M;
            if (SAT) v = vmin2(v, 0x00FF00FFu);
            L[j] = v;
        }
        pV = rV; pC = rC; pending = true;
        emit<DPL, MODE>(P, x, y, d0, lane, active, L);
    }
}

// ---------------------------------------------------------------------------
// launchers
// ---------------------------------------------------------------------------
cudaError_t launch_census2(const uint8_t *im0, const uint8_t *im1, uint64_t *out0, uint64_t *out1,
                           int W, int H, cudaStream_t s) {
    const dim3 b(CT_W, CT_H), g((W + CT_W - 1) / CT_W, (H + CT_H - 1) / CT_H, im1 ? 2 : 1);
    k_census2<<<g, b, 0, s>>>(im0, im1, out0, out1, W, H);
    return cudaGetLastError();
}

cudaError_t launch_sobel2(const uint8_t *im0, const uint8_t *im1, uint8_t *out0, uint8_t *out1,
                          int W, int H, cudaStream_t s) {
    const dim3 b(32, 8), g((W + 31) / 32, (H + 7) / 8, 2);
    k_sobel2<<<g, b, 0, s>>>(im0, im1, out0, out1, W, H);
    return cudaGetLastError();
}

cudaError_t launch_half2(const uint8_t *im0, const uint8_t *im1, uint8_t *out0, uint8_t *out1,
                         int W, int H, cudaStream_t s) {
    const dim3 b(32, 8), g((W / 2 + 31) / 32, (H / 2 + 7) / 8, 2);
    k_half2<<<g, b, 0, s>>>(im0, im1, out0, out1, W, H);
    return cudaGetLastError();
}

template <int DPL, int CK, int SAT>
static cudaError_t launch_line_mode(const LineParams &p, int mode, dim3 g, dim3 b, cudaStream_t s) {
    switch (mode) {
    case MODE_SCRATCH: k_line<DPL, MODE_SCRATCH, CK, SAT><<<g, b, 0, s>>>(p); break;
    case MODE_STORE:   k_line<DPL, MODE_STORE, CK, SAT><<<g, b, 0, s>>>(p); break;
    case MODE_ACCUM:   k_line<DPL, MODE_ACCUM, CK, SAT><<<g, b, 0, s>>>(p); break;
    case MODE_FINAL:   k_line<DPL, MODE_FINAL, CK, SAT><<<g, b, 0, s>>>(p); break;
    default: return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
}

cudaError_t launch_line(const LineParams &p, int mode, int cost_kind, int saturate,
                        int warps_per_block, cudaStream_t s) {
    if (warps_per_block < 1 || warps_per_block > 8 || p.nlines < 1) return cudaErrorInvalidValue;
    const int dpl = p.nl > 0 ? p.D / p.nl : 0;
    const dim3 b(32 * warps_per_block), g((p.nlines + warps_per_block - 1) / warps_per_block);
    if (cost_kind == COST_PLAIN && !saturate) {
        switch (dpl) {
        case 2: return launch_line_mode<2, COST_PLAIN, 0>(p, mode, g, b, s);
        case 4: return launch_line_mode<4, COST_PLAIN, 0>(p, mode, g, b, s);
        case 6: return launch_line_mode<6, COST_PLAIN, 0>(p, mode, g, b, s);
        case 8: return launch_line_mode<8, COST_PLAIN, 0>(p, mode, g, b, s);
        default: return cudaErrorInvalidValue;
        }
    }
    if (saturate && dpl == 2) {
        if (cost_kind == COST_MS1) return launch_line_mode<2, COST_MS1, 1>(p, mode, g, b, s);
        if (cost_kind == COST_MS2) return launch_line_mode<2, COST_MS2, 1>(p, mode, g, b, s);
    }
    return cudaErrorInvalidValue;
}

}  // namespace sgmgb
