// sgmgb_kernels.cu -- the per-frame census and cost kernels (tile code in
// sgmgb_tiles.cuh) and the multi-scale prefilters (SobelX, 2x2 box mean).
// The path kernel is in sgmgb_path.cu.
#include "sgmgb_kernels.cuh"
#include "sgmgb_tiles.cuh"

namespace sgmgb {

namespace {

__device__ __forceinline__ int clampi(int v, int lo, int hi) { return v < lo ? lo : (v > hi ? hi : v); }

}  // namespace

// ---------------------------------------------------------------------------
// Census 9x7 of two images at once (blockIdx.z picks the image); the tile
// code is in sgmgb_tiles.cuh.
// ---------------------------------------------------------------------------
// Tiles of CEN_FRAME_ROWS rows: 1.5 image bytes staged per pixel against 2.2
// with 8-row tiles (the kernel also reads images from page-locked host memory
// across NVLink-C2C when handed such a pointer).
constexpr int CEN_FRAME_ROWS = 32;

__global__ void __launch_bounds__(256)
k_census2(const uint8_t *__restrict__ im0, const uint8_t *__restrict__ im1,
          uint64_t *__restrict__ out0, uint64_t *__restrict__ out1, int W, int H) {
    __shared__ __align__(16) uint8_t smem[tiles::cen_smem<CEN_FRAME_ROWS>()];
    tiles::census_tile<CEN_FRAME_ROWS>(blockIdx.z ? im1 : im0, blockIdx.z ? out1 : out0, W, H,
                                       blockIdx.x * tiles::CEN_PX, blockIdx.y * CEN_FRAME_ROWS, smem,
                                       threadIdx.y * 32 + threadIdx.x, 256);
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
// Cost volume of a frame at one scale, one row tile per block; the tile code
// (and the cost definitions) are in sgmgb_tiles.cuh.
// ---------------------------------------------------------------------------
template <bool MS>
__global__ void __launch_bounds__(256)
k_cost(const uint64_t *__restrict__ cl, const uint64_t *__restrict__ cr, uint8_t *__restrict__ C,
       const uint8_t *__restrict__ C1, int W, int D, int invalid) {
    __shared__ __align__(16) uint8_t smem[tiles::COST_SMEM];
    tiles::cost_tile<false, MS>(cl, cr, C, C1, W, D, invalid, blockIdx.y, blockIdx.x * tiles::COST_PX, smem,
                                threadIdx.x, 256);
}

// ---------------------------------------------------------------------------
// launchers
// ---------------------------------------------------------------------------
cudaError_t launch_cost(const uint64_t *cl, const uint64_t *cr, uint8_t *C, const uint8_t *C1,
                        int W, int H, int D, int invalid, cudaStream_t s) {
    if (D < 16 || D > 256 || D % 16 || W < 1 || H < 1 || H > 65535) return cudaErrorInvalidValue;
    const dim3 g((W + tiles::COST_PX - 1) / tiles::COST_PX, H);
    if (C1) k_cost<true><<<g, 256, 0, s>>>(cl, cr, C, C1, W, D, invalid);
    else k_cost<false><<<g, 256, 0, s>>>(cl, cr, C, nullptr, W, D, invalid);
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------
cudaError_t launch_census2(const uint8_t *im0, const uint8_t *im1, uint64_t *out0, uint64_t *out1,
                           int W, int H, cudaStream_t s) {
    const dim3 b(32, 8),
        g((W + tiles::CEN_PX - 1) / tiles::CEN_PX, (H + CEN_FRAME_ROWS - 1) / CEN_FRAME_ROWS, im1 ? 2 : 1);
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

cudaError_t prepare_frame_kernels() {
    cudaError_t e = set_carveout(k_census2);
    if (e == cudaSuccess) e = set_carveout(k_cost<false>);
    if (e == cudaSuccess) e = set_carveout(k_cost<true>);
    if (e == cudaSuccess) e = set_carveout(k_sobel2);
    if (e == cudaSuccess) e = set_carveout(k_half2);
    return e;
}

}  // namespace sgmgb
