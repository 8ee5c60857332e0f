// sgmgb_fused.cu -- the kernel and launcher of the first half of the
// horizontal passes of the fused schedule (device code in sgmgb_fused.cuh).
#include "sgmgb_fused.cuh"

namespace sgmgb {

namespace {

template <int NR>
__global__ void __launch_bounds__(128)
k_hcost(const LineParams P) {
    extern __shared__ __align__(16) uint8_t smem[];
    const int wib = threadIdx.x >> 5;
    const int pair = blockIdx.x * (blockDim.x >> 5) + wib;
    uint64_t *ws = (uint64_t *)(smem + wib * HCost<NR>::BYTES);
    if (blockIdx.y == 0) path_hcost<NR, 1>(P, pair, ws);
    else path_hcost<NR, -1>(P, pair, ws);
}

}  // namespace

cudaError_t prepare_fused_kernels() {
    cudaError_t e = set_carveout(k_hcost<1>);
    if (e == cudaSuccess) e = set_carveout(k_hcost<2>);
    if (e == cudaSuccess) e = set_carveout(k_hcost<4>);
    return e;
}

cudaError_t launch_hcost(const LineParams &p, int wpb, cudaStream_t s) {
    if (wpb < 1 || wpb > 4 || p.W < 1 || p.H < 1 || !p.cl || !p.cr || !p.C || !p.sc || !p.state)
        return cudaErrorInvalidValue;
    const int npairs = (p.H + 1) / 2;
    const dim3 g((npairs + wpb - 1) / wpb, 2), b(32 * wpb);
    switch (p.D) {
    case 32: k_hcost<1><<<g, b, wpb * HCost<1>::BYTES, s>>>(p); break;
    case 64: k_hcost<2><<<g, b, wpb * HCost<2>::BYTES, s>>>(p); break;
    case 128: k_hcost<4><<<g, b, wpb * HCost<4>::BYTES, s>>>(p); break;
    default: return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
}

}  // namespace sgmgb
