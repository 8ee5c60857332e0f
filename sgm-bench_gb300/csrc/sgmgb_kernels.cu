// sgmgb_kernels.cu -- census 9x7 and the multi-scale prefilters (SobelX, 2x2
// box mean). The path kernel is in sgmgb_path.cu.
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
// Census 9x7 of two images at once (blockIdx.z picks the image): bit n is set
// iff the neighbour is darker than the centre, n running over dy (outer) then
// dx, skipping the centre, with clamped (edge-replicated) coordinates
// (common/sgm_ref.c:23-41).
//
// A thread makes 4 horizontally adjacent pixels with 4-byte SIMD-within-a-
// register compares: for one (dx, dy) offset the 4 neighbour bytes and the 4
// centre bytes are compared at once by a borrow-free per-byte "less than"
// (result in each byte's top bit), and 8 offsets in a row are gathered into
// one word per 8 census bits (byte i = pixel i) by shifting right and OR-ing
// the top bits in. A byte transpose at the end gives each pixel's 62-bit
// descriptor. The 128x8-pixel tile plus its 4/3-pixel halo is staged in
// shared memory.
// ---------------------------------------------------------------------------
constexpr int CT_PX = 128, CT_ROWS = 8, CT_TW = CT_PX + 8, CT_TH = CT_ROWS + 6;

__device__ __forceinline__ uint32_t bytes_lt(uint32_t n, uint32_t c, uint32_t c7) {
    // per byte: n < c, in the byte's top bit (other bits are garbage)
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

__global__ void __launch_bounds__(256)
k_census2(const uint8_t *__restrict__ im0, const uint8_t *__restrict__ im1,
          uint64_t *__restrict__ out0, uint64_t *__restrict__ out1, int W, int H) {
    __shared__ __align__(16) uint32_t tile[CT_TH][CT_TW / 4];
    const uint8_t *im = blockIdx.z ? im1 : im0;
    uint64_t *out = blockIdx.z ? out1 : out0;
    const int x0 = blockIdx.x * CT_PX, y0 = blockIdx.y * CT_ROWS;
    uint8_t *tb = (uint8_t *)&tile[0][0];
    for (int i = threadIdx.y * 32 + threadIdx.x; i < CT_TW * CT_TH; i += 256) {
        const int ty = i / CT_TW, tx = i - ty * CT_TW;
        tb[i] = im[(size_t)clampi(y0 + ty - 3, 0, H - 1) * W + clampi(x0 + tx - 4, 0, W - 1)];
    }
    __syncthreads();
    const int tx = threadIdx.x, ty = threadIdx.y;
    const int x = x0 + 4 * tx, y = y0 + ty;
    if (x >= W || y >= H) return;
    const uint32_t c = tile[ty + 3][tx + 1], c7 = c & 0x7F7F7F7Fu;
    uint32_t A[8];
    uint32_t acc = 0;
    int n = 0;
#pragma unroll
    for (int dy = -3; dy <= 3; dy++) {
        const uint32_t w0 = tile[ty + 3 + dy][tx], w1 = tile[ty + 3 + dy][tx + 1], w2 = tile[ty + 3 + dy][tx + 2];
#pragma unroll
        for (int dx = -4; dx <= 4; dx++) {
            if (dx == 0 && dy == 0) continue;
            acc = (acc >> 1) | (bytes_lt(window4(w0, w1, w2, 4 + dx), c, c7) & 0x80808080u);
            if ((++n & 7) == 0) { A[(n >> 3) - 1] = acc; acc = 0; }
        }
    }
    A[7] = acc >> 2;                                  // bits 56..61: six compares, aligned to bit 0
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
// Cost volume C[(y*W + x)*D + d], uint8, computed once per frame and scale:
//   plain:        popcount(cl[x] ^ cr[x-d]), 62 where x-d < 0      (common/sgm_ref.c:44-56)
//   half scale:   the same with 63 for x-d < 0                     (multiscale/sgm_ms_ref.c:66-72)
//   full scale:   (own cost, 63 invalid) averaged with the half-scale
//                 cost at (x/2, y/2, d/2): (c2 + c1 + 1) >> 1      (multiscale/sgm_ms_ref.c:184-188)
// A block makes CT_X pixels of one row: the row's left descriptors and the
// right ones from D-1 columns before the tile are staged in shared memory.
// A thread makes 8 consecutive disparities of one pixel and stores them as one
// 8-byte word. A warp covers 8 pixels x 4 disparity groups (16 x 2 when D/8 is
// not a multiple of 4): its 32 right-descriptor reads for one k are then 32
// consecutive words (no bank conflicts), and each pixel's 32 cost bytes of the
// warp are one contiguous sector in the store. The kernel carries all the
// frame's population counts (2 POPC per cost: the POPC pipe is its bound).
// ---------------------------------------------------------------------------
constexpr int CT_X = 64;

__global__ void __launch_bounds__(256)
k_cost(const uint64_t *__restrict__ cl, const uint64_t *__restrict__ cr, uint8_t *__restrict__ C,
       const uint8_t *__restrict__ C1, int W, int H, int D, int invalid) {
    __shared__ uint64_t sl[CT_X];
    __shared__ uint64_t sr[CT_X + 256];            // sr[j] = cr[x0 - (D-1) + j]
    const int y = blockIdx.y, x0 = blockIdx.x * CT_X;
    const uint64_t *rl = cl + (size_t)y * W, *rr = cr + (size_t)y * W;
    const int nr = CT_X + D - 1;
    for (int i = threadIdx.x; i < CT_X + nr; i += blockDim.x) {
        if (i < CT_X) {
            sl[i] = x0 + i < W ? __ldg(rl + x0 + i) : 0ull;
        } else {
            const int j = i - CT_X, x = x0 - (D - 1) + j;
            sr[j] = (x >= 0 && x < W) ? __ldg(rr + x) : 0ull;
        }
    }
    __syncthreads();
    const int tpp = D >> 3;                        // disparity groups of 8 per pixel
    const int DG = (tpp & 3) ? 2 : 4, PXW = 32 / DG;
    const int lane = threadIdx.x & 31;
    const int pxl = DG == 4 ? lane >> 2 : lane >> 1, dgl = lane & (DG - 1);
    const int nxb = CT_X / PXW, ntask = nxb * (tpp / DG);
    const int hw = W >> 1;
    uint8_t *row = C + (size_t)y * W * D;
    for (int task = threadIdx.x >> 5; task < ntask; task += blockDim.x >> 5) {
        const int dgb = task / nxb, px = (task - dgb * nxb) * PXW + pxl;
        const int d0 = (dgb * DG + dgl) * 8, x = x0 + px;
        if (x >= W) continue;
        const uint64_t a = sl[px];
        const uint64_t *r = sr + px + (D - 1) - d0; // r[-k] = cr[x - d0 - k]
        uint32_t v[8];
        if (x >= d0 + 7) {
#pragma unroll
            for (int k = 0; k < 8; k++) v[k] = (uint32_t)__popcll(a ^ r[-k]);
        } else {
#pragma unroll
            for (int k = 0; k < 8; k++) v[k] = x - d0 - k >= 0 ? (uint32_t)__popcll(a ^ r[-k]) : (uint32_t)invalid;
        }
        if (C1) {   // full scale of the multi-scale variant
            const uint32_t h = *(const uint32_t *)(C1 + ((size_t)(y >> 1) * hw + (x >> 1)) * D + (d0 >> 1));
#pragma unroll
            for (int k = 0; k < 8; k++) v[k] = (v[k] + ((h >> (8 * (k >> 1))) & 0xFFu) + 1) >> 1;
        }
        const uint32_t lo = v[0] | (v[1] << 8) | (v[2] << 16) | (v[3] << 24);
        const uint32_t hi = v[4] | (v[5] << 8) | (v[6] << 16) | (v[7] << 24);
        *(uint2 *)(row + (size_t)x * D + d0) = make_uint2(lo, hi);
    }
}

// ---------------------------------------------------------------------------
// launchers
// ---------------------------------------------------------------------------
cudaError_t launch_cost(const uint64_t *cl, const uint64_t *cr, uint8_t *C, const uint8_t *C1,
                        int W, int H, int D, int invalid, cudaStream_t s) {
    if (D < 16 || D > 256 || D % 16 || W < 1 || H < 1 || H > 65535) return cudaErrorInvalidValue;
    const dim3 g((W + CT_X - 1) / CT_X, H);
    k_cost<<<g, 256, 0, s>>>(cl, cr, C, C1, W, H, D, invalid);
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------
cudaError_t launch_census2(const uint8_t *im0, const uint8_t *im1, uint64_t *out0, uint64_t *out1,
                           int W, int H, cudaStream_t s) {
    const dim3 b(32, CT_ROWS), g((W + CT_PX - 1) / CT_PX, (H + CT_ROWS - 1) / CT_ROWS, im1 ? 2 : 1);
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

}  // namespace sgmgb
