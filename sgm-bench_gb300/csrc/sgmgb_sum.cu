// sgmgb_sum.cu -- the sum over directions and the winner-take-all of a frame
// whose every direction parked its L in a uint8 plane.
//
//   disp(p) = argmin_d sum_r L_r(p, d), the lowest d on ties
//
// as in common/sgm_ref.c:100-117 (S accumulated over the paths, then the
// argmin) and, for the full scale of the multi-scale variant, only at even
// (x, y) into the (W/2)x(H/2) map (multiscale/sgm_ms_ref.c:190-199). The sum
// over directions is order-independent, so adding the planes here, after all
// directions ran side by side, gives the reference's S exactly.
//
// No recurrence is left in this pass: it streams the planes once (HBM-bound).
// A thread takes one 16-byte chunk (16 disparities) of one pixel from each
// plane, adds the planes in u16x2 lanes (even and odd bytes apart), and keeps
// the smallest key S*2^ks + d (u16x2 when it fits 16 bits, else u32 keys
// S*256 + d). The D/16 threads of a pixel are consecutive; they combine their
// keys by shuffles when D/16 divides 32, else through shared memory.
#include <cstdint>
#include <cuda_runtime.h>
#include "sgmgb_kernels.cuh"

namespace sgmgb {

namespace {

__device__ __forceinline__ uint32_t vminu2(uint32_t a, uint32_t b) {
    uint32_t r;
    asm("min.u16x2 %0, %1, %2;" : "=r"(r) : "r"(a), "r"(b));
    return r;
}

// EVEN: only pixels (2ox, 2oy), output (W/2)x(H/2), from compact planes (the
// even-only passes store pixel (2ox, 2oy) at oy*(W/2) + ox). Grid: (ceil(ow / npb), oh).
// lt: log2(D/16) when SHFL (D/16 divides 32); npb: pixels per block.
template <int NP, bool KEY16, bool SHFL, bool EVEN>
__global__ void __launch_bounds__(256) k_sum(SumPlanes pl, uint8_t *__restrict__ disp, int W, int D, int tpp,
                                             int lt, int npb, int ks) {
    __shared__ uint32_t s_key[SHFL ? 1 : 256];
    __shared__ uint8_t s_out[256];
    const int t = threadIdx.x;
    const int ow = EVEN ? W >> 1 : W;
    const int lp = SHFL ? t >> lt : t / tpp, g = t - lp * tpp;
    const int ox = blockIdx.x * npb + lp, oy = blockIdx.y;
    const bool live = lp < npb && ox < ow;
    uint32_t key = 0xFFFFFFFFu;
    if (live) {
        const size_t p = (size_t)oy * ow + ox;   // EVEN: the planes are compact, pixel (2ox, 2oy) at oy*ow + ox
        const size_t off = p * D + 16 * g;
        uint4 v[NP];
#pragma unroll
        for (int r = 0; r < NP; r++) v[r] = __ldg((const uint4 *)(pl.p[r] + off));
        const uint32_t d0 = 16u * g;
        uint32_t m = 0xFFFFFFFFu;
#pragma unroll
        for (int w = 0; w < 4; w++) {
            uint32_t E = 0, O = 0;   // disparities d0+4w+{0,2} and d0+4w+{1,3}
#pragma unroll
            for (int r = 0; r < NP; r++) {
                const uint32_t x = w == 0 ? v[r].x : w == 1 ? v[r].y : w == 2 ? v[r].z : v[r].w;
                E += __byte_perm(x, 0, 0x4240);
                O += __byte_perm(x, 0, 0x4341);
            }
            const uint32_t dE = (d0 + 4 * w) | ((d0 + 4 * w + 2) << 16);
            if (KEY16) {
                m = vminu2(m, (E << ks) + dE);
                m = vminu2(m, (O << ks) + dE + 0x00010001u);
            } else {
                m = min(m, ((E & 0xFFFFu) << 8) | (dE & 0xFFFFu));
                m = min(m, ((E >> 16) << 8) | (dE >> 16));
                m = min(m, ((O & 0xFFFFu) << 8) | ((dE & 0xFFFFu) + 1));
                m = min(m, ((O >> 16) << 8) | ((dE >> 16) + 1));
            }
        }
        key = KEY16 ? min(m & 0xFFFFu, m >> 16) : m;
    }
    if (SHFL) {
        for (int o = 1; o < tpp; o <<= 1) key = min(key, __shfl_xor_sync(0xFFFFFFFFu, key, o));
    } else {
        s_key[t] = key;
        __syncthreads();
        if (live && g == 0)
            for (int i = 1; i < tpp; i++) key = min(key, s_key[t + i]);
    }
    if (live && g == 0) s_out[lp] = (uint8_t)(key & (KEY16 ? (1u << ks) - 1u : 0xFFu));
    __syncthreads();
    // the block's npb outputs are consecutive bytes of one row: one coalesced
    // store per warp (the map may be the caller's pinned host buffer)
    if (t < npb && blockIdx.x * npb + t < ow) disp[(size_t)oy * ow + blockIdx.x * npb + t] = s_out[t];
}

template <int NP, bool KEY16, bool EVEN>
cudaError_t launch_np(const SumPlanes &pl, uint8_t *disp, int W, int H, int D, cudaStream_t s) {
    const int tpp = D / 16;
    const bool shfl = (32 % tpp) == 0;
    int lt = 0;
    while ((1 << lt) < tpp) lt++;
    int ks = 0;
    while ((1 << ks) < D) ks++;
    const int npb = 256 / tpp;
    const int ow = EVEN ? W / 2 : W, oh = EVEN ? H / 2 : H;
    if (ow < 1 || oh < 1) return cudaSuccess;
    const dim3 g((ow + npb - 1) / npb, oh);
    if (shfl)
        k_sum<NP, KEY16, true, EVEN><<<g, 256, 0, s>>>(pl, disp, W, D, tpp, lt, npb, ks);
    else
        k_sum<NP, KEY16, false, EVEN><<<g, 256, 0, s>>>(pl, disp, W, D, tpp, lt, npb, ks);
    return cudaGetLastError();
}

template <int NP>
cudaError_t launch_key(const SumPlanes &pl, uint8_t *disp, int W, int H, int D, bool even, cudaStream_t s) {
    int ks = 0;
    while ((1 << ks) < D) ks++;
    // every plane value is at most 255: the largest key must fit 16 bits
    const bool k16 = ((uint32_t)(NP * 255) << ks) + (1u << ks) - 1u <= 0xFFFFu;
    if (k16) return even ? launch_np<NP, true, true>(pl, disp, W, H, D, s) : launch_np<NP, true, false>(pl, disp, W, H, D, s);
    return even ? launch_np<NP, false, true>(pl, disp, W, H, D, s) : launch_np<NP, false, false>(pl, disp, W, H, D, s);
}

}  // namespace

cudaError_t launch_sum(const SumPlanes &pl, int np, uint8_t *disp, int W, int H, int D, int even_only,
                       cudaStream_t s) {
    if (D < 16 || D > 256 || D % 16 || W < 1 || H < 1) return cudaErrorInvalidValue;
    if (np == 4) return launch_key<4>(pl, disp, W, H, D, even_only != 0, s);
    if (np == 8) return launch_key<8>(pl, disp, W, H, D, even_only != 0, s);
    return cudaErrorInvalidValue;
}

}  // namespace sgmgb
