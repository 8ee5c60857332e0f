// sgmgb_post.cu -- optional post-steps on a plain frame: a left-right
// consistency check, a 16x subpixel map and a 3x3 median.
//
// The reference has none of them (common/sgm_params.h:58: "No LR check, no
// subpixel, no median"); their definitions are the oracle's post mode
// (oracle/sgm_oracle.c, sgmo_post), and the maps here are bit-identical to it:
//   d_L(p)  = argmin_d S(p, d), lowest d on ties (the plain map);
//   d16(p)  = 16*d_L + (16*(c0 - c2)) / (2*(c0 + c2 - 2*c1)), c0, c1, c2 =
//             S(d_L - 1), S(d_L), S(d_L + 1), integer division toward zero,
//             when 0 < d_L < D-1 and the denominator is > 0; else 16*d_L;
//   LR      d_R(x, y) = argmin over d with x + d < W of S((x + d, y), d),
//             lowest d on ties; p = (x, y) is invalid (255, d16 0xFFFF)
//             when x - d_L < 0 or |d_L - d_R(x - d_L, y)| > 1;
//   median  the 3x3 median of the checked map, edge-replicated.
// The frame runs the latency schedule, which leaves every direction's L in a
// plane; a streaming pass adds the planes into the uint16 summed volume S,
// which the post kernels read. These passes are simple one-thread-per-pixel
// kernels: the post-steps are an option outside the benchmarked path.
#include "sgmgb_internal.h"
#include <cstring>
#include <new>

using namespace sgmgb;

namespace {

// S (uint16, W*H*D) = the sum of the np planes, 16 bytes of each per thread.
__global__ void __launch_bounds__(256) k_post_sum(SumPlanes pl, int np, uint16_t *__restrict__ S, size_t n16) {
    const size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (i >= n16) return;
    uint32_t acc[8] = {0u, 0u, 0u, 0u, 0u, 0u, 0u, 0u};       // 16 sums as packed u16 pairs
    for (int p = 0; p < np; p++) {
        const uint4 v = ((const uint4 *)pl.p[p])[i];
        const uint32_t w[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
        for (int k = 0; k < 4; k++) {
            acc[2 * k] += __byte_perm(w[k], 0, 0x4140);         // bytes 0, 1 -> the two halves
            acc[2 * k + 1] += __byte_perm(w[k], 0, 0x4342);     // bytes 2, 3
        }
    }
    uint4 *o = (uint4 *)(S + 16 * i);
    o[0] = make_uint4(acc[0], acc[1], acc[2], acc[3]);
    o[1] = make_uint4(acc[4], acc[5], acc[6], acc[7]);
}

// d_R(x, y) = argmin over d with x + d < W of S((x + d, y), d), lowest d on ties.
__global__ void __launch_bounds__(256) k_post_right(const uint16_t *__restrict__ S, uint8_t *__restrict__ dR,
                                                    int W, int D) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y;
    if (x >= W) return;
    const uint16_t *row = S + (size_t)y * W * D;
    const int dmax = min(D, W - x);
    uint32_t best = 0xFFFFFFFFu;
    for (int d = 0; d < dmax; d++) best = min(best, ((uint32_t)row[(size_t)(x + d) * D + d] << 8) | (uint32_t)d);
    dR[(size_t)y * W + x] = (uint8_t)(best & 0xFFu);
}

// d_L, the subpixel map and the left-right check; `out` before the median.
__global__ void __launch_bounds__(256) k_post_left(const uint16_t *__restrict__ S, const uint8_t *__restrict__ dR,
                                                   uint8_t *__restrict__ out, uint16_t *__restrict__ d16, int W,
                                                   int D, int check) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y;
    if (x >= W) return;
    const size_t i = (size_t)y * W + x;
    const uint16_t *s = S + i * D;
    uint32_t best = 0xFFFFFFFFu;
    for (int d = 0; d < D; d++) best = min(best, ((uint32_t)s[d] << 8) | (uint32_t)d);
    const int d = (int)(best & 0xFFu);
    int v16 = 16 * d;
    if (d > 0 && d < D - 1) {
        const int c0 = s[d - 1], c1 = s[d], c2 = s[d + 1], den = c0 + c2 - 2 * c1;
        if (den > 0) v16 += (16 * (c0 - c2)) / (2 * den);
    }
    int o = d;
    if (check) {
        const int xr = x - d;
        if (xr < 0 || abs(d - (int)dR[(size_t)y * W + xr]) > 1) { o = 255; v16 = 0xFFFF; }
    }
    out[i] = (uint8_t)o;
    if (d16) d16[i] = (uint16_t)v16;
}

__device__ __forceinline__ void sort2(uint32_t &a, uint32_t &b) {
    const uint32_t t = min(a, b);
    b = max(a, b);
    a = t;
}

// 3x3 median, edge-replicated: the median-of-nine exchange network (19 exchanges).
__global__ void __launch_bounds__(256) k_post_median(const uint8_t *__restrict__ in, uint8_t *__restrict__ out,
                                                     int W, int H) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y;
    if (x >= W) return;
    uint32_t p[9];
    int k = 0;
#pragma unroll
    for (int dy = -1; dy <= 1; dy++)
#pragma unroll
        for (int dx = -1; dx <= 1; dx++)
            p[k++] = in[(size_t)min(max(y + dy, 0), H - 1) * W + min(max(x + dx, 0), W - 1)];
    sort2(p[1], p[2]); sort2(p[4], p[5]); sort2(p[7], p[8]);
    sort2(p[0], p[1]); sort2(p[3], p[4]); sort2(p[6], p[7]);
    sort2(p[1], p[2]); sort2(p[4], p[5]); sort2(p[7], p[8]);
    sort2(p[0], p[3]); sort2(p[5], p[8]); sort2(p[4], p[7]);
    sort2(p[3], p[6]); sort2(p[1], p[4]); sort2(p[2], p[5]);
    sort2(p[4], p[7]); sort2(p[4], p[2]); sort2(p[6], p[4]);
    sort2(p[4], p[2]);
    out[(size_t)y * W + x] = (uint8_t)p[4];
}

int post_fail(sgmgb_ctx *ctx, cudaError_t e, const char *what) {
    cudaGetLastError();
    return set_err(ctx, SGMGB_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

}  // namespace

extern "C" int sgmgb_run_frame_post(sgmgb_ctx *ctx, const uint8_t *left, const uint8_t *right, uint8_t *disp,
                                    uint16_t *disp16, int flags) {
    if (!ctx || !left || !right || !disp) return SGMGB_ERR_ARG;
    if (!ctx->planned) return set_err(ctx, SGMGB_ERR_STATE, "sgmgb_plan has not been called");
    const sgmgb_frame_desc fd = ctx->fd;
    if (fd.variant != SGMGB_PLAIN) return set_err(ctx, SGMGB_ERR_ARG, "post-steps: plain variant only");
    if (flags & ~(SGMGB_POST_LR | SGMGB_POST_MEDIAN | SGMGB_POST_SUBPIXEL))
        return set_err(ctx, SGMGB_ERR_ARG, "post-steps: unknown flag");
    if ((flags & SGMGB_POST_LR) && fd.D > 240)
        return set_err(ctx, SGMGB_ERR_ARG, "post-steps: the left-right check needs D <= 240 (255 marks invalid)");
    if ((flags & SGMGB_POST_SUBPIXEL) && !disp16)
        return set_err(ctx, SGMGB_ERR_ARG, "post-steps: the subpixel map needs an output buffer");
    cudaSetDevice(ctx->device);
    const size_t N = (size_t)fd.W * fd.H, ND = N * fd.D;
    // post buffers: S (2*N*D), d_R (N), the map before the median (N), the subpixel map (2N)
    const size_t need = 2 * ND + 256 + N + 256 + N + 256 + 2 * N;
    if (ctx->post_bytes < need) {
        if (ctx->post) cudaFree(ctx->post);
        ctx->post = nullptr;
        ctx->post_bytes = 0;
        cudaError_t e = cudaMalloc(&ctx->post, need);
        if (e != cudaSuccess) {
            cudaGetLastError();
            ctx->post = nullptr;
            return set_err(ctx, SGMGB_ERR_NOMEM, "post-steps: workspace of " + std::to_string(need) + " bytes");
        }
        ctx->post_bytes = need;
    }
    auto al = [](size_t v) { return (v + 255) & ~(size_t)255; };
    uint8_t *pb = (uint8_t *)ctx->post;
    uint16_t *S = (uint16_t *)pb;
    uint8_t *dR = pb + al(2 * ND);
    uint8_t *pre = dR + al(N);
    uint16_t *d16 = (uint16_t *)(pre + al(N));
    const FrameSlot &s = *ctx->slot;
    cudaStream_t st = ctx->stream;
    PathShape shape = ctx->shape;
    shape.sched = SGMGB_SCHED_LATENCY;                        // every direction's L in a plane
    cudaError_t e = cudaMemcpyAsync(s.left, left, N, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(s.right, right, N, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = enqueue_frame(s, s.left, s.right, s.disp, st, shape, nullptr, nullptr);
    if (e != cudaSuccess) return post_fail(ctx, e, "post-steps: frame");
    SumPlanes sp{};
    uint8_t *pl[8] = {s.sc, (uint8_t *)s.S, (uint8_t *)s.S + ND, s.xp, s.xp + ND, s.xp + 2 * ND, s.xp + 3 * ND,
                      s.xp + 4 * ND};
    for (int k = 0; k < fd.paths; k++) sp.p[k] = pl[k];
    const size_t n16 = ND / 16;
    k_post_sum<<<(unsigned)((n16 + 255) / 256), 256, 0, st>>>(sp, fd.paths, S, n16);
    const dim3 g((fd.W + 255) / 256, fd.H), b(256);
    if (flags & SGMGB_POST_LR) k_post_right<<<g, b, 0, st>>>(S, dR, fd.W, fd.D);
    k_post_left<<<g, b, 0, st>>>(S, dR, pre, d16, fd.W, fd.D, (flags & SGMGB_POST_LR) ? 1 : 0);
    uint8_t *fin = pre;
    if (flags & SGMGB_POST_MEDIAN) {
        k_post_median<<<g, b, 0, st>>>(pre, s.disp, fd.W, fd.H);
        fin = s.disp;
    }
    e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaMemcpyAsync(disp, fin, N, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess && (flags & SGMGB_POST_SUBPIXEL))
        e = cudaMemcpyAsync(disp16, d16, 2 * N, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return post_fail(ctx, e, "post-steps");
    return SGMGB_OK;
}
