// sgmgb_noalloc.cu -- a plain-variant frame that allocates nothing.
//
// The frame's workspace (census descriptors, cost volume, three uint8 planes
// or plane + uint16 sum) lives in one file-scope device array of
// SGMGB_NOALLOC_SCRATCH_BYTES; the kernels are the engine's own census, cost
// and path kernels, launched one after another on the caller's stream. Its
// address comes from cudaGetSymbolAddress, looked up once per device (with
// that device current) together with the path kernels' shared-memory limits.
// Every call then makes cudaGetDevice, its kernel launches, and one
// cudaGetLastError after each launch -- no other CUDA runtime call.
#include "sgmgb_internal.h"
#include <mutex>

using namespace sgmgb;

namespace {

static __device__ __align__(256) uint8_t g_noalloc_scratch[SGMGB_NOALLOC_SCRATCH_BYTES];

constexpr int kMaxDevices = 64;
std::mutex g_mu;
uint8_t *g_base[kMaxDevices] = {};

size_t al256(size_t v) { return (v + 255) & ~(size_t)255; }

// Workspace bytes of a frame: census (2 x 8N), cost (N*D), three N*D planes
// (4 paths) or one N*D plane and an N*D uint16 sum (8 paths: also 3*N*D).
size_t noalloc_bytes(const sgmgb_frame_desc &fd) {
    const size_t N = (size_t)fd.W * fd.H, ND = N * fd.D;
    return 2 * al256(8 * N) + al256(ND) + al256(ND) + al256(2 * ND);
}

// The scratch's device address on the current device, set up on first use.
int scratch_base(uint8_t **out) {
    int dev = -1;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) {
        cudaGetLastError();
        return SGMGB_ERR_NODEV;
    }
    std::lock_guard<std::mutex> g(g_mu);
    if (!g_base[dev]) {
        void *p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e == cudaSuccess) e = prepare_path_kernels();
        if (e != cudaSuccess || !p) {
            cudaGetLastError();
            return SGMGB_ERR_CUDA;
        }
        g_base[dev] = (uint8_t *)p;
    }
    *out = g_base[dev];
    return SGMGB_OK;
}

}  // namespace

extern "C" int sgmgb_run_frame_noalloc(const uint8_t *d_left, const uint8_t *d_right, uint8_t *d_disp,
                                       int W, int H, int D, int paths, void *stream) {
    const sgmgb_frame_desc fd = {W, H, D, paths, SGMGB_PLAIN};
    if (!d_left || !d_right || !d_disp || sgmgb_check_desc(&fd) != SGMGB_OK) return SGMGB_ERR_ARG;
    if (noalloc_bytes(fd) > (size_t)SGMGB_NOALLOC_SCRATCH_BYTES) return SGMGB_ERR_BUDGET;
    uint8_t *b = nullptr;
    int rc = scratch_base(&b);
    if (rc) return rc;
    const size_t N = (size_t)W * H, ND = N * D;
    uint64_t *cl = (uint64_t *)b;
    uint64_t *cr = (uint64_t *)(b + al256(8 * N));
    uint8_t *C = b + 2 * al256(8 * N);
    uint8_t *sc = C + al256(ND);
    uint8_t *S8 = sc + al256(ND);                    // 2*N*D bytes: two u8 planes or one u16 sum
    cudaStream_t st = (cudaStream_t)stream;
    const int wpb = 4;
    cudaError_t e = launch_census2(d_left, d_right, cl, cr, W, H, st);
    if (e == cudaSuccess) e = launch_cost(cl, cr, C, nullptr, W, H, D, kInvalidPlain, st);
    LineParams p{};
    p.C = C; p.sc = sc; p.S = (uint16_t *)S8; p.disp = d_disp;
    p.W = W; p.H = H; p.D = D; p.p1 = 20; p.p2 = 192; p.dpl = 0;
    p.key16 = (paths == 4 && D <= 64) ? 1 : 0;
    if (paths == 4) {
        // R->L, B->T, L->R into three planes, then T->B sums them and takes the argmin
        uint8_t *pl[3] = {sc, S8, S8 + ND};
        const int dir[3][2] = {{-1, 0}, {0, -1}, {1, 0}};
        for (int k = 0; k < 3 && e == cudaSuccess; k++) {
            LineParams q = p;
            q.dx = dir[k][0]; q.dy = dir[k][1]; q.sc = pl[k];
            q.nlines = lines_for(W, H, q.dx, q.dy);
            e = launch_line(q, MODE_SCRATCH, 0, wpb, st);
        }
        if (e == cudaSuccess) {
            LineParams q = p;
            q.dx = 0; q.dy = 1; q.sc = pl[0]; q.sc2 = pl[1]; q.sc3 = pl[2];
            q.nlines = lines_for(W, H, 0, 1);
            e = launch_line(q, MODE_FINAL3, 0, wpb, st);
        }
    } else {
        // the pair schedule: the first of each opposite pair parks L in sc, the second adds into S
        static const int sched[8][3] = {{-1, 0, MODE_SCRATCH}, {1, 0, MODE_STORE}, {0, -1, MODE_SCRATCH},
                                        {0, 1, MODE_ACCUM}, {-1, -1, MODE_SCRATCH}, {1, 1, MODE_ACCUM},
                                        {1, -1, MODE_SCRATCH}, {-1, 1, MODE_FINAL}};
        for (int k = 0; k < 8 && e == cudaSuccess; k++) {
            LineParams q = p;
            q.dx = sched[k][0]; q.dy = sched[k][1];
            q.nlines = lines_for(W, H, q.dx, q.dy);
            e = launch_line(q, sched[k][2], 0, wpb, st);
        }
    }
    if (e != cudaSuccess) {
        cudaGetLastError();
        return SGMGB_ERR_CUDA;
    }
    return SGMGB_OK;
}
