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
// Cost volume C[(y*W + x)*D + d], uint8, computed once per frame and scale:
//   plain (COST_PLAIN):  popcount(cl[x] ^ cr[x-d]), 62 where x-d < 0   (common/sgm_ref.c:44-56)
//   half scale (MS1):    the same with 63 for x-d < 0                  (multiscale/sgm_ms_ref.c:66-72)
//   full scale (MS2):    (own cost, 63 invalid) averaged with the half-scale
//                        cost at (x/2, y/2, d/2): (c2 + c1 + 1) >> 1  (multiscale/sgm_ms_ref.c:184-188)
// Every thread makes 8 consecutive disparities of one pixel and stores them
// as one 8-byte word; the D/8 threads of a pixel are adjacent lanes, so a
// warp writes whole pixels' cost vectors contiguously. This kernel carries
// all the frame's population counts (the POPC pipe is its bound); the path
// passes only read the bytes.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256)
k_cost(const uint64_t *__restrict__ cl, const uint64_t *__restrict__ cr, uint8_t *__restrict__ C,
       const uint8_t *__restrict__ C1, int W, int H, int D, int invalid) {
    const int tpp = D >> 3;                                   // threads per pixel
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const long long p = t / tpp;
    if (p >= (long long)W * H) return;
    const int d0 = (int)(t - p * tpp) * 8;
    const int x = (int)(p % W);
    const uint64_t a = __ldg(cl + p);
    uint32_t v[8];
#pragma unroll
    for (int k = 0; k < 8; k++) {
        const int xr = x - d0 - k;
        v[k] = xr >= 0 ? (uint32_t)__popcll(a ^ __ldg(cr + (p - d0 - k))) : (uint32_t)invalid;
    }
    if (C1) {   // full scale of the multi-scale variant
        const int y = (int)(p / W), hw = W >> 1;
        const uint8_t *c1 = C1 + ((size_t)(y >> 1) * hw + (x >> 1)) * D + (d0 >> 1);
        const uint32_t h = *(const uint32_t *)c1;   // half-scale d0/2 .. d0/2+3
#pragma unroll
        for (int k = 0; k < 8; k++) v[k] = (v[k] + ((h >> (8 * (k >> 1))) & 0xFFu) + 1) >> 1;
    }
    const uint32_t lo = v[0] | (v[1] << 8) | (v[2] << 16) | (v[3] << 24);
    const uint32_t hi = v[4] | (v[5] << 8) | (v[6] << 16) | (v[7] << 24);
    *(uint2 *)(C + p * D + d0) = make_uint2(lo, hi);
}

// ---------------------------------------------------------------------------
// launchers
// ---------------------------------------------------------------------------
cudaError_t launch_cost(const uint64_t *cl, const uint64_t *cr, uint8_t *C, const uint8_t *C1,
                        int W, int H, int D, int invalid, cudaStream_t s) {
    if (D < 16 || D % 16 || W < 1 || H < 1) return cudaErrorInvalidValue;
    const long long threads = (long long)W * H * (D / 8);
    k_cost<<<(unsigned)((threads + 255) / 256), 256, 0, s>>>(cl, cr, C, C1, W, H, D, invalid);
    return cudaGetLastError();
}

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

}  // namespace sgmgb
