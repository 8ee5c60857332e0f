// sgmgb_tiles.cuh -- census and cost of one tile, shared by the per-frame
// kernels (sgmgb_kernels.cu) and the persistent batch kernel (sgmgb_batch.cu).
// Both functions are called by every thread of a block (they synchronise it).
#pragma once
#include <cstdint>
#include "sgmgb_kernels.cuh"

namespace sgmgb {
namespace tiles {

__device__ __forceinline__ int clampi(int v, int lo, int hi) { return v < lo ? lo : (v > hi ? hi : v); }

// ---------------------------------------------------------------------------
// Census 9x7 (common/sgm_ref.c:23-41): bit n is set iff the neighbour is
// darker than the centre, n running over dy (outer) then dx, skipping the
// centre, with clamped (edge-replicated) coordinates.
//
// A thread makes 4 horizontally adjacent pixels with 4-byte SIMD-within-a-
// register compares: for one (dx, dy) offset the 4 neighbour bytes and the 4
// centre bytes are compared at once by a borrow-free per-byte "less than"
// (result in each byte's top bit), and 8 offsets in a row are gathered into
// one word per 8 census bits (byte i = pixel i) by shifting right and OR-ing
// the top bits in. A byte transpose at the end gives each pixel's 62-bit
// descriptor. A tile is CEN_PX x CEN_ROWS pixels plus its 4/3-pixel halo,
// staged in shared memory.
// ---------------------------------------------------------------------------
constexpr int CEN_PX = 128, CEN_ROWS = 8, CEN_TW = CEN_PX + 8;
// shared memory of a tile of R rows, 16-byte aligned by the caller
template <int R> __host__ __device__ constexpr int cen_smem() { return CEN_TW * (R + 6); }
constexpr int CEN_SMEM = cen_smem<CEN_ROWS>();

__device__ __forceinline__ uint32_t bytes_lt(uint32_t n, uint32_t c, uint32_t c7) {
    // per byte: n < c, in the byte's top bit (the other bits are garbage)
    const uint32_t t = (n | 0x80808080u) - c7;       // top bit of a byte: (n & 0x7f) >= (c & 0x7f)
    return (~n & c) | (~(n ^ c) & ~t);
}

// bytes s..s+3 of the 12-byte run w0:w1:w2
__device__ __forceinline__ uint32_t window4(uint32_t w0, uint32_t w1, uint32_t w2, int s) {
    if (s == 0) return w0;
    if (s == 4) return w1;
    if (s == 8) return w2;
    const uint32_t sel = (s & 3) | (((s & 3) + 1) << 4) | (((s & 3) + 2) << 8) | (((s & 3) + 3) << 12);
    return s < 4 ? __byte_perm(w0, w1, sel) : __byte_perm(w1, w2, sel);
}

// The census jobs of a staged CEN_PX x R tile at (x0, y0): word `OFF + w` of
// staged row r holds image bytes x0 - 4 + 4w .. x0 - 1 + 4w of image row
// y0 - 3 + r (clamped), RW words per row. A job makes 4 horizontally adjacent
// pixels. No barrier inside: the caller synchronises around it.
template <int R>
__device__ __forceinline__ void census_jobs(const uint32_t *tile, int RW, int OFF, uint64_t *__restrict__ out,
                                            int W, int H, int x0, int y0, int tid, int nthreads) {
    for (int job = tid; job < 32 * R; job += nthreads) {
        const int tx = job & 31, ty = job >> 5;
        const int x = x0 + 4 * tx, y = y0 + ty;
        if (x >= W || y >= H) continue;
        const uint32_t c = tile[(ty + 3) * RW + OFF + tx + 1], c7 = c & 0x7F7F7F7Fu;
        uint32_t A[8];
        uint32_t acc = 0;
        int n = 0;
#pragma unroll
        for (int dy = -3; dy <= 3; dy++) {
            const uint32_t *r = tile + (ty + 3 + dy) * RW + OFF + tx;
            const uint32_t w0 = r[0], w1 = r[1], w2 = r[2];
#pragma unroll
            for (int dx = -4; dx <= 4; dx++) {
                if (dx == 0 && dy == 0) continue;
                acc = (acc >> 1) | (bytes_lt(window4(w0, w1, w2, 4 + dx), c, c7) & 0x80808080u);
                if ((++n & 7) == 0) { A[(n >> 3) - 1] = acc; acc = 0; }
            }
        }
        A[7] = acc >> 2;                              // bits 56..61: six compares, aligned to bit 0
        uint64_t d[4];
#pragma unroll
        for (int i = 0; i < 4; i++) {
            const uint32_t sel = i | ((i + 4) << 4);
            const uint32_t lo = __byte_perm(__byte_perm(A[0], A[1], sel), __byte_perm(A[2], A[3], sel), 0x5410);
            const uint32_t hi = __byte_perm(__byte_perm(A[4], A[5], sel), __byte_perm(A[6], A[7], sel), 0x5410);
            d[i] = ((uint64_t)hi << 32) | lo;
        }
        uint64_t *o = out + (size_t)y * W + x;
        if (x + 3 < W) {
            if ((((size_t)y * W + x) & 1) == 0) {
                ((ulonglong2 *)o)[0] = make_ulonglong2(d[0], d[1]);
                ((ulonglong2 *)o)[1] = make_ulonglong2(d[2], d[3]);
            } else {
#pragma unroll
                for (int i = 0; i < 4; i++) o[i] = d[i];
            }
        } else {
            for (int i = 0; i < 4 && x + i < W; i++) o[i] = d[i];
        }
    }
}

// Census of the CEN_PX x R tile at (x0, y0) of one W x H image into out
// (W*H uint64). nthreads: a multiple of 32; tid in [0, nthreads). The image
// is read through the read-only path: it is an input, never written during
// the launch. Taller tiles read fewer halo rows per pixel (the 6 rows shared
// with the tiles above and below): (R + 6) / R.
template <int R = CEN_ROWS>
__device__ __forceinline__ void census_tile(const uint8_t *__restrict__ im, uint64_t *__restrict__ out,
                                            int W, int H, int x0, int y0, uint8_t *smem, int tid,
                                            int nthreads) {
    constexpr int CEN_TH = R + 6, CEN_SMEM = cen_smem<R>();
    uint32_t *tile = (uint32_t *)smem;                // [CEN_TH][CEN_TW / 4]
    constexpr int RW = CEN_TW / 4;                    // words per tile row
    if ((W & 15) == 0 && ((uintptr_t)im & 15) == 0 && x0 >= 16 && x0 + CEN_PX + 16 <= W) {
        // interior tile: 16-byte loads of image bytes [x0-16, x0+CEN_PX+16) per
        // row (word j of the row's loads holds tile words 4j-3 .. 4j); a tenth
        // of the loads of byte staging
        constexpr int VPR = (CEN_PX + 32) / 16;       // 16-byte loads per tile row
        for (int i = tid; i < CEN_TH * VPR; i += nthreads) {
            const int ty = i / VPR, j = i - ty * VPR;
            const uint4 v = __ldg((const uint4 *)(im + (size_t)clampi(y0 + ty - 3, 0, H - 1) * W + x0 - 16) + j);
            uint32_t *row = tile + ty * RW;
            const int w = 4 * j - 3;
            if (w >= 0) row[w] = v.x;
            if (w + 1 >= 0 && w + 1 < RW) row[w + 1] = v.y;
            if (w + 2 >= 0 && w + 2 < RW) row[w + 2] = v.z;
            if (w + 3 < RW) row[w + 3] = v.w;
        }
    } else {
        for (int i = tid; i < CEN_SMEM; i += nthreads) {
            const int ty = i / CEN_TW, tx = i - ty * CEN_TW;
            smem[i] = __ldg(im + (size_t)clampi(y0 + ty - 3, 0, H - 1) * W + clampi(x0 + tx - 4, 0, W - 1));
        }
    }
    __syncthreads();
    census_jobs<R>(tile, RW, 0, out, W, H, x0, y0, tid, nthreads);
    __syncthreads();                                  // the tile memory may be reused next
}

// ---------------------------------------------------------------------------
// Cost C[(y*W + x)*D + d], uint8, of COST_PX pixels of row y from x0:
//   plain:        popcount(cl[x] ^ cr[x-d]), `invalid` (62) where x-d < 0   (common/sgm_ref.c:44-56)
//   half scale:   the same with 63                                       (multiscale/sgm_ms_ref.c:66-72)
//   full scale:   (own cost, 63 invalid) averaged with the half-scale cost
//                 at (x/2, y/2, d/2): (c2 + c1 + 1) >> 1                 (multiscale/sgm_ms_ref.c:184-188)
// The row's left descriptors and the right ones from D-1 columns before the
// tile are staged in shared memory. A thread makes 8 consecutive disparities
// of a pixel and stores them as one 8-byte word; a warp covers 4 groups of 8
// disparities (2 when D/8 is not a multiple of 4), so each pixel's 32 bytes of
// the warp are one sector in the store. Interior tiles (most of them) take
// cost_pairs: several adjacent pixels per thread from a swizzled staging
// layout, which cuts the shared-memory loads that share the MIO queue with
// the population counts (2 POPC per cost). Edge tiles (x - d < 0, columns past
// W) take cost_tasks: one pixel per thread, 8 pixels x 4 groups per warp, so
// that its 32 right-descriptor reads for one k are 32 consecutive words.
// ---------------------------------------------------------------------------
constexpr int COST_PX = 128;                          // 16 blocks of 8 pixels, or 8 of 16
constexpr int COST_SLW = COST_PX + COST_PX / 16;      // words of the staged left descriptors (swizzled)
constexpr int COST_SMEM = (COST_SLW + (COST_PX + 256) + (COST_PX + 256) / 16) * 8;   // bytes, 16-byte aligned

// Swizzled shared-memory word of staged descriptor j: one spare word every 16,
// so that reads spaced by even strides spread over all 16 bank pairs.
__device__ __forceinline__ int swz(int j) { return j + (j >> 4); }

// LD_CG: read the descriptors through L2 only (the batch kernel, where other
// blocks of the same launch wrote them); otherwise through the read-only path.
template <bool LD_CG>
__device__ __forceinline__ uint64_t ld_desc(const uint64_t *p) {
    return LD_CG ? __ldcg(p) : __ldg(p);
}

// Bytewise (a + b + 1) >> 1 of four packed bytes: a + b = 2(a | b) - (a ^ b),
// so the rounded-up half is (a | b) - ((a ^ b) >> 1), with the shift kept
// inside each byte; no byte borrows, since (a ^ b) >> 1 <= a | b.
__device__ __forceinline__ uint32_t avg_up_u8x4(uint32_t a, uint32_t b) {
    return (a | b) - (((a ^ b) >> 1) & 0x7F7F7F7Fu);
}

// The multi-scale merge of 8 packed costs d0..d0+7 of a full-scale pixel
// with the half-scale costs at d/2: h holds c1[d0/2 .. d0/2 + 3], and cost
// d0 + k averages with byte k >> 1 (multiscale/sgm_ms_ref.c:184-188).
__device__ __forceinline__ uint2 merge_half(uint32_t lo, uint32_t hi, uint32_t h) {
    return make_uint2(avg_up_u8x4(lo, __byte_perm(h, 0, 0x1100)), avg_up_u8x4(hi, __byte_perm(h, 0, 0x3322)));
}

// One pixel's 8 costs d0..d0+7 from staged descriptors; r[-k] = cr[x - d0 - k].
// EDGE: some x - d0 - k may be negative (the first D columns of a row).
template <bool EDGE>
__device__ __forceinline__ void cost8(uint64_t a, const uint64_t *r, int x, int d0, int invalid, uint32_t (&v)[8]) {
#pragma unroll
    for (int k = 0; k < 8; k++) {
        const uint32_t c = (uint32_t)__popcll(a ^ r[-k]);
        v[k] = EDGE && x - d0 - k < 0 ? (uint32_t)invalid : c;
    }
}

// The tile's compute loop. DG4: D/8 a multiple of 4 (a warp covers 8 pixels x 4
// groups of 8 disparities; otherwise 16 x 2). MS: average with the half-scale
// cost. EDGE / TAIL: the tile has columns x < D - 1 / columns past W.
template <bool DG4, bool MS, bool EDGE, bool TAIL>
__device__ __forceinline__ void cost_tasks(const uint64_t *sl, const uint64_t *sr, uint8_t *__restrict__ row,
                                           const uint8_t *__restrict__ C1, int W, int D, int invalid, int y,
                                           int x0, int tid, int nthreads) {
    constexpr int DG = DG4 ? 4 : 2, PXW = 32 / DG;
    constexpr int LNXB = COST_PX / PXW == 16 ? 4 : (COST_PX / PXW == 8 ? 3 : 2);   // log2(COST_PX / PXW)
    static_assert((1 << LNXB) * PXW == COST_PX, "a tile is a power-of-two number of pixel blocks");
    const int lane = tid & 31;
    const int pxl = lane / DG, dgl = lane & (DG - 1);
    const int ntask = ((D >> 3) / DG) << LNXB;
    const int hw = W >> 1;
    for (int task = tid >> 5; task < ntask; task += nthreads >> 5) {
        const int dgb = task >> LNXB, px = (task & ((1 << LNXB) - 1)) * PXW + pxl;
        const int d0 = (dgb * DG + dgl) * 8, x = x0 + px;
        if (TAIL && x >= W) continue;
        uint32_t v[8];
        cost8<EDGE>(sl[px], sr + px + (D - 1) - d0, x, d0, invalid, v);
        const uint32_t lo = v[0] | (v[1] << 8) | (v[2] << 16) | (v[3] << 24);
        const uint32_t hi = v[4] | (v[5] << 8) | (v[6] << 16) | (v[7] << 24);
        if (MS)     // full scale of the multi-scale variant
            *(uint2 *)(row + (size_t)x * D + d0) =
                merge_half(lo, hi, *(const uint32_t *)(C1 + ((size_t)(y >> 1) * hw + (x >> 1)) * D + (d0 >> 1)));
        else
            *(uint2 *)(row + (size_t)x * D + d0) = make_uint2(lo, hi);
    }
}

// Interior tiles (no x - d < 0, no column past W) with D/8 a multiple of 4:
// a thread makes NPX adjacent pixels x 8 disparities from NPX left and NPX + 7
// right descriptors: 11 shared-memory loads for 16 costs (NPX = 2) or 15 for
// 32 (NPX = 4), where one pixel at a time takes 9 for 8. The loads share the
// MIO queue with the population counts, which binds this kernel. A warp
// covers 8 NPX pixels x 4 groups of 8 disparities; for one load its lanes
// read words NPX p - 8g + c (p < 8, g < 4), which the swizzle (swz) spreads
// over the 16 bank pairs.
template <int NPX, bool MS>
__device__ __forceinline__ void cost_pairs(const uint64_t *sl, const uint64_t *sr, uint8_t *__restrict__ row,
                                           const uint8_t *__restrict__ C1, int W, int D, int y, int x0, int tid,
                                           int nthreads) {
    constexpr int PXW = 8 * NPX;                      // pixels of a warp
    constexpr int LNXB = COST_PX / PXW == 16 ? 4 : COST_PX / PXW == 8 ? 3 : COST_PX / PXW == 4 ? 2 : 1;
    static_assert((1 << LNXB) * PXW == COST_PX, "a tile is a power-of-two number of pixel blocks");
    const int lane = tid & 31, pp = lane >> 2, g = lane & 3;
    const int ntask = ((D >> 3) / 4) << LNXB;
    const int hw = W >> 1;
    for (int task = tid >> 5; task < ntask; task += nthreads >> 5) {
        const int dgb = task >> LNXB, px = (task & ((1 << LNXB) - 1)) * PXW + NPX * pp;
        const int d0 = (dgb * 4 + g) * 8, x = x0 + px;
        uint64_t a[NPX], r[NPX + 7];
#pragma unroll
        for (int i = 0; i < NPX; i++) a[i] = sl[swz(px + i)];
        const int base = px + (D - 1) - d0 - 7;       // r[m] = cr[x - d0 - 7 + m]
#pragma unroll
        for (int m = 0; m < NPX + 7; m++) r[m] = sr[swz(base + m)];
#pragma unroll
        for (int i = 0; i < NPX; i++) {
            uint32_t v[8];
#pragma unroll
            for (int k = 0; k < 8; k++) v[k] = (uint32_t)__popcll(a[i] ^ r[7 + i - k]);
            const uint32_t lo = v[0] | (v[1] << 8) | (v[2] << 16) | (v[3] << 24);
            const uint32_t hi = v[4] | (v[5] << 8) | (v[6] << 16) | (v[7] << 24);
            if (MS)     // full scale of the multi-scale variant: x is even, pixel pairs share (x/2, y/2)
                *(uint2 *)(row + (size_t)(x + i) * D + d0) = merge_half(
                    lo, hi, *(const uint32_t *)(C1 + ((size_t)(y >> 1) * hw + ((x + i) >> 1)) * D + (d0 >> 1)));
            else
                *(uint2 *)(row + (size_t)(x + i) * D + d0) = make_uint2(lo, hi);
        }
    }
}

template <bool LD_CG, bool MS>
__device__ __forceinline__ void cost_tile(const uint64_t *__restrict__ cl, const uint64_t *__restrict__ cr,
                                          uint8_t *__restrict__ C, const uint8_t *__restrict__ C1, int W,
                                          int D, int invalid, int y, int x0, uint8_t *smem, int tid,
                                          int nthreads) {
    uint64_t *sl = (uint64_t *)smem;                  // COST_PX left descriptors
    uint64_t *sr = sl + COST_SLW;                     // descriptor j: cr[x0 - (D-1) + j]
    const uint64_t *rl = cl + (size_t)y * W, *rr = cr + (size_t)y * W;
    const int nr = COST_PX + D - 1;
    const bool dg4 = ((D >> 3) & 3) == 0;
    const bool edge = x0 < D - 1, tail = x0 + COST_PX > W;   // uniform over the block
    const bool pairs = dg4 && !edge && !tail;         // staged swizzled for cost_pairs
    for (int i = tid; i < COST_PX + nr; i += nthreads) {
        if (i < COST_PX) {
            sl[pairs ? swz(i) : i] = x0 + i < W ? ld_desc<LD_CG>(rl + x0 + i) : 0ull;
        } else {
            const int j = i - COST_PX, x = x0 - (D - 1) + j;
            sr[pairs ? swz(j) : j] = (x >= 0 && x < W) ? ld_desc<LD_CG>(rr + x) : 0ull;
        }
    }
    __syncthreads();
    uint8_t *row = C + (size_t)y * W * D;
    if (pairs)
        // measured at 1080p D=64: plain 64.8 (NPX 2) / 63.9 us (NPX 4); the
        // multi-scale merge 37.1 (NPX 2) / 43.8 us (NPX 4, 64 registers)
        cost_pairs<MS ? 2 : 4, MS>(sl, sr, row, C1, W, D, y, x0, tid, nthreads);
    else if (dg4)
        cost_tasks<true, MS, true, true>(sl, sr, row, C1, W, D, invalid, y, x0, tid, nthreads);
    else
        cost_tasks<false, MS, true, true>(sl, sr, row, C1, W, D, invalid, y, x0, tid, nthreads);
    __syncthreads();                                  // the tile memory may be reused next
}

}  // namespace tiles
}  // namespace sgmgb
