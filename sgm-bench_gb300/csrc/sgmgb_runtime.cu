// sgmgb_runtime.cu -- context, resident workspace, frame pipeline and the
// single-frame entry points of the C ABI (include/sgmgb.h).
#include "sgmgb_internal.h"
#include <cstdio>
#include <cstring>
#include <new>
#include <algorithm>
#include <vector>

using namespace sgmgb;

namespace sgmgb {

int set_err(sgmgb_ctx *ctx, int code, const std::string &msg) {
    if (ctx) ctx->last_error = msg;
    return code;
}

static size_t al256(size_t v) { return (v + 255) & ~(size_t)255; }

size_t slot_layout(const sgmgb_frame_desc &fd, FrameSlot *s) {
    const size_t W = (size_t)fd.W, H = (size_t)fd.H, D = (size_t)fd.D, N = W * H;
    size_t off = 0;
    auto take = [&](size_t n) { size_t o = off; off += al256(n); return o; };
    const size_t o_left = take(N), o_right = take(N);
    const size_t out_n = fd.variant == SGMGB_MULTISCALE ? (W / 2) * (H / 2) : N;
    const size_t o_disp = take(out_n);
    const size_t o_cl = take(N * 8), o_cr = take(N * 8);
    const size_t o_C = take(N * D), o_sc = take(N * D), o_S = take(N * D * 2);
    const size_t o_xp = take(N * D * (fd.paths == 8 ? 5 : 1));
    const size_t o_state = fd.variant == SGMGB_PLAIN ? take(hstate_words(fd.H) * 4) : 0;
    size_t o_sobL = 0, o_sobR = 0, o_hL = 0, o_hR = 0, o_hsL = 0, o_hsR = 0, o_cl1 = 0, o_cr1 = 0, o_d1 = 0;
    size_t o_C1 = 0, o_P1 = 0;
    if (fd.variant == SGMGB_MULTISCALE) {
        const size_t Nh = (W / 2) * (H / 2);
        o_sobL = take(N); o_sobR = take(N);
        o_hL = take(Nh); o_hR = take(Nh); o_hsL = take(Nh); o_hsR = take(Nh);
        o_cl1 = take(Nh * 8); o_cr1 = take(Nh * 8);
        o_d1 = take(Nh);
        o_C1 = take(Nh * D);
        o_P1 = take(Nh * D * 8);
    }
    if (s) {
        uint8_t *b = (uint8_t *)s->base;
        s->left = b + o_left; s->right = b + o_right; s->disp = b + o_disp;
        s->cl = (uint64_t *)(b + o_cl); s->cr = (uint64_t *)(b + o_cr);
        s->C = b + o_C; s->sc = b + o_sc; s->S = (uint16_t *)(b + o_S);
        s->xp = b + o_xp;
        s->state = fd.variant == SGMGB_PLAIN ? (uint32_t *)(b + o_state) : nullptr;
        if (fd.variant == SGMGB_MULTISCALE) {
            s->C1 = b + o_C1;
            s->sobL = b + o_sobL; s->sobR = b + o_sobR;
            s->halfL = b + o_hL; s->halfR = b + o_hR; s->hsobL = b + o_hsL; s->hsobR = b + o_hsR;
            s->cl1 = (uint64_t *)(b + o_cl1); s->cr1 = (uint64_t *)(b + o_cr1);
            s->disp1 = b + o_d1;
            s->P1 = b + o_P1;
        }
    }
    return off;
}

int slot_alloc(const sgmgb_frame_desc &fd, FrameSlot **out, std::string &err) {
    FrameSlot *s = new (std::nothrow) FrameSlot();
    if (!s) { err = "host allocation failed"; return SGMGB_ERR_NOMEM; }
    s->fd = fd;
    s->bytes = slot_layout(fd, nullptr);
    cudaError_t e = cudaMalloc(&s->base, s->bytes);
    if (e != cudaSuccess) {
        err = std::string("cudaMalloc of ") + std::to_string(s->bytes) + " bytes: " + cudaGetErrorString(e);
        cudaGetLastError();
        delete s;
        return SGMGB_ERR_NOMEM;
    }
    slot_layout(fd, s);
    for (int i = 0; i < FrameSlot::kAux && e == cudaSuccess; i++)
        e = cudaStreamCreateWithFlags(&s->aux[i], cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&s->fork, cudaEventDisableTiming);
    for (int i = 0; i < FrameSlot::kAux && e == cudaSuccess; i++)
        e = cudaEventCreateWithFlags(&s->join[i], cudaEventDisableTiming);
    if (fd.variant == SGMGB_MULTISCALE) {
        if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&s->ms, cudaStreamNonBlocking);
        for (int i = 0; i < FrameSlot::kAux && e == cudaSuccess; i++)
            e = cudaStreamCreateWithFlags(&s->aux2[i], cudaStreamNonBlocking);
        for (cudaEvent_t *ev : {&s->fork2, &s->fork_ms, &s->c1, &s->s1_done})
            if (e == cudaSuccess) e = cudaEventCreateWithFlags(ev, cudaEventDisableTiming);
        for (int i = 0; i < FrameSlot::kAux && e == cudaSuccess; i++)
            e = cudaEventCreateWithFlags(&s->join2[i], cudaEventDisableTiming);
    }
    if (e != cudaSuccess) {
        err = std::string("stream/event creation: ") + cudaGetErrorString(e);
        cudaGetLastError();
        slot_free(s);
        return SGMGB_ERR_CUDA;
    }
    *out = s;
    return SGMGB_OK;
}

void slot_free(FrameSlot *s) {
    if (!s) return;
    for (auto &a : s->aux) if (a) cudaStreamDestroy(a);
    for (auto &a : s->aux2) if (a) cudaStreamDestroy(a);
    if (s->ms) cudaStreamDestroy(s->ms);
    for (cudaEvent_t ev : {s->fork, s->fork2, s->fork_ms, s->c1, s->s1_done}) if (ev) cudaEventDestroy(ev);
    for (auto &j : s->join) if (j) cudaEventDestroy(j);
    for (auto &j : s->join2) if (j) cudaEventDestroy(j);
    if (s->base) cudaFree(s->base);
    delete s;
}

// Directions and penalties follow common/sgm_ref.c:96-99 (plain, P1 = 20 for
// all) and multiscale/sgm_ms_ref.c:85-87 (P1 40 horizontal, 20 vertical, 10
// diagonal). The sum over directions is order-independent, so the schedule is
// this engine's: every direction parks its L in its own uint8 plane, all of
// them side by side on forked streams, and one streaming pass adds the planes
// and takes the argmin.
static int ms_p1(int dx, int dy) { return dy == 0 ? 40 : (dx == 0 ? 20 : 10); }

namespace {

// Records an event after each launch when a probe is attached: each kernel's
// device time, its name and its algorithmic bytes (every input byte read
// once, every output byte written once).
struct Marker {
    KernelProbe *pr;
    cudaStream_t st;
    cudaError_t start() { return pr ? cudaEventRecord(pr->ev[0], st) : cudaSuccess; }
    cudaError_t operator()(const char *name, double bytes) {
        if (!pr) return cudaSuccess;
        if (pr->n >= KernelProbe::kMax) return cudaErrorInvalidValue;
        pr->name[pr->n] = name;
        pr->bytes[pr->n] = bytes;
        pr->n++;
        return cudaEventRecord(pr->ev[pr->n], st);
    }
};

const char *pass_name(int dx, int dy) {
    if (dy == 0) return dx > 0 ? "path_lr" : "path_rl";
    if (dx == 0) return dy > 0 ? "path_tb" : "path_bt";
    if (dx > 0) return dy > 0 ? "path_diag_tl_br" : "path_diag_bl_tr";
    return dy > 0 ? "path_diag_tr_bl" : "path_diag_br_tl";
}

// The forked streams, events and direction planes of one group of path
// passes: the frame's own (main_fan), or, for the half-scale stage of a
// multi-scale frame, which runs beside the full-scale stage, a set of its own
// (half_fan). `plane`: bytes of one direction's plane at the group's scale.
struct Fan {
    const cudaStream_t *aux;
    cudaEvent_t fork;
    const cudaEvent_t *join;
    uint8_t *pl[8];
};

Fan main_fan(const FrameSlot &s, size_t plane) {
    return Fan{s.aux, s.fork, s.join, {s.sc, (uint8_t *)s.S, (uint8_t *)s.S + plane, s.xp, s.xp + plane,
                                       s.xp + 2 * plane, s.xp + 3 * plane, s.xp + 4 * plane}};
}

Fan half_fan(const FrameSlot &s, size_t plane) {
    Fan f{s.aux2, s.fork2, s.join2, {}};
    for (int k = 0; k < 8; k++) f.pl[k] = s.P1 + k * plane;
    return f;
}

// The THROUGHPUT schedule: every direction but T->B parks its L in its own
// plane (the same planes as run_planes, one fewer), side by side on forked
// streams; then T->B adds them to its own L and takes the argmin
// (MODE_FINAL3 for 4 paths, MODE_FINAL7 for 8). One plane less is written
// and read than with run_planes, at the price of a long pass on the frame's
// critical path.
cudaError_t run_final(const Fan &f, const LineParams &base, int npaths, int sat, bool ms, int wpb,
                      cudaStream_t st, Marker &mark, int even_only, uint8_t *disp, double Nout) {
    const bool serial = mark.pr != nullptr;
    const size_t plane = (size_t)base.W * base.H * base.D;
    uint8_t *const *pl = f.pl;
    static const int dirs[7][2] = {{-1, 0}, {1, 0}, {0, -1}, {-1, -1}, {1, 1}, {1, -1}, {-1, 1}};
    const int nsc = npaths - 1;
    const double ND = (double)plane;
    cudaStream_t ss[7];
    for (int k = 0; k < nsc; k++) ss[k] = (serial || k == 0) ? st : f.aux[k - 1];
    cudaError_t e;
    if (!serial) {
        if ((e = cudaEventRecord(f.fork, st)) != cudaSuccess) return e;
        for (int k = 1; k < nsc; k++)
            if ((e = cudaStreamWaitEvent(ss[k], f.fork, 0)) != cudaSuccess) return e;
    }
    for (int k = 0; k < nsc; k++) {
        LineParams q = base;
        q.dx = dirs[k][0]; q.dy = dirs[k][1]; q.sc = pl[k];
        q.p1 = ms ? ms_p1(q.dx, q.dy) : 20;
        q.nlines = q.even_only ? lines_for_even(q.W, q.H, q.dx, q.dy) : lines_for(q.W, q.H, q.dx, q.dy);
        if ((e = launch_line(q, MODE_SCRATCH, sat, wpb, ss[k])) != cudaSuccess) return e;
        if ((e = mark(pass_name(q.dx, q.dy), 2 * ND)) != cudaSuccess) return e;
    }
    if (!serial) {
        for (int k = 1; k < nsc; k++) {
            if ((e = cudaEventRecord(f.join[k - 1], ss[k])) != cudaSuccess) return e;
            if ((e = cudaStreamWaitEvent(st, f.join[k - 1], 0)) != cudaSuccess) return e;
        }
    }
    LineParams q = base;
    q.dx = 0; q.dy = 1;
    q.sc = pl[0]; q.sc2 = pl[1]; q.sc3 = pl[2];
    for (int k = 0; k < 4; k++) q.xpl[k] = npaths == 8 ? pl[3 + k] : nullptr;
    q.p1 = ms ? ms_p1(0, 1) : 20;
    q.disp = disp;
    q.even_only = even_only;
    q.nlines = even_only ? lines_for_even(q.W, q.H, 0, 1) : lines_for(q.W, q.H, 0, 1);
    q.key16 = (npaths == 4 && base.D <= 64) ? 1 : 0;   // S*64 + d < 2^16
    if ((e = launch_line(q, npaths == 8 ? MODE_FINAL7 : MODE_FINAL3, sat, wpb, st)) != cudaSuccess) return e;
    return mark("path_tb_final", npaths * ND + Nout);
}

// The LATENCY schedule. Every direction (4 or 8 of them, at one scale)
// parks its L in its own uint8 plane: sc, the two halves of S, then xp. The
// directions run side by side on forked streams, longest (horizontal) first;
// one pass then adds the planes and takes the argmin into `disp` (even_only:
// the multi-scale full scale's (W/2)x(H/2) map). `serial` (a probe
// attached): all on `st`, one after another.
cudaError_t run_planes(const Fan &f, const LineParams &base, int npaths, int sat, bool ms, int wpb,
                       cudaStream_t st, Marker &mark, int even_only, uint8_t *disp, double Nout) {
    const bool serial = mark.pr != nullptr;
    const size_t plane = (size_t)base.W * base.H * base.D;   // at this scale (fits the fan's buffers)
    uint8_t *const *pl = f.pl;
    static const int dirs[8][2] = {{-1, 0}, {1, 0}, {0, -1}, {0, 1}, {-1, -1}, {1, 1}, {1, -1}, {-1, 1}};
    const double ND = (double)plane;
    cudaStream_t ss[8];
    for (int k = 0; k < npaths; k++) ss[k] = (serial || k == 0) ? st : f.aux[k - 1];
    cudaError_t e;
    if (!serial) {
        if ((e = cudaEventRecord(f.fork, st)) != cudaSuccess) return e;
        for (int k = 1; k < npaths; k++)
            if ((e = cudaStreamWaitEvent(ss[k], f.fork, 0)) != cudaSuccess) return e;
    }
    SumPlanes sp{};
    for (int k = 0; k < npaths; k++) {
        LineParams q = base;
        q.dx = dirs[k][0]; q.dy = dirs[k][1]; q.sc = pl[k];
        q.p1 = ms ? ms_p1(q.dx, q.dy) : 20;
        q.nlines = q.even_only ? lines_for_even(q.W, q.H, q.dx, q.dy) : lines_for(q.W, q.H, q.dx, q.dy);
        sp.p[k] = pl[k];
        if ((e = launch_line(q, MODE_SCRATCH, sat, wpb, ss[k])) != cudaSuccess) return e;
        if ((e = mark(pass_name(q.dx, q.dy), 2 * ND)) != cudaSuccess) return e;
    }
    if (!serial) {
        for (int k = 1; k < npaths; k++) {
            if ((e = cudaEventRecord(f.join[k - 1], ss[k])) != cudaSuccess) return e;
            if ((e = cudaStreamWaitEvent(st, f.join[k - 1], 0)) != cudaSuccess) return e;
        }
    }
    if ((e = launch_sum(sp, npaths, disp, base.W, base.H, base.D, even_only, st)) != cudaSuccess) return e;
    const double Nsum = even_only ? Nout : (double)base.W * base.H;   // pixels whose planes are read
    return mark("sum_argmin", npaths * Nsum * base.D + Nout);
}

// The FUSED schedule (plain, 4 paths, pair layout; fused_applies), after the
// census: the first halves of both horizontal passes compute the costs from
// the census descriptors into the cost volume and park their L in one plane
// (the two halves are disjoint columns); the vertical passes, side by side,
// park theirs in two more; the second halves of the horizontal passes, side
// by side, resume each row from the first halves' state, add the three
// planes to their own L and take the argmin. One cost pass fewer than the
// other schedules, and its population counts run inside the latency-bound
// horizontal pass; the frame's critical path is census, the first halves,
// the vertical passes and the second halves.
cudaError_t run_fused(const FrameSlot &s, const LineParams &base, int wpb, cudaStream_t st, Marker &mark,
                      uint8_t *disp, double N) {
    const bool serial = mark.pr != nullptr;
    const size_t plane = (size_t)base.W * base.H * base.D;
    const double ND = (double)plane;
    uint8_t *ph = s.sc, *ptb = (uint8_t *)s.S, *pbt = (uint8_t *)s.S + plane;
    cudaError_t e;
    LineParams q = base;
    q.cl = s.cl; q.cr = s.cr; q.sc = ph; q.state = s.state; q.hseg = 1;
    if ((e = launch_hcost(q, wpb, st)) != cudaSuccess) return e;
    if ((e = mark("path_h_first_cost", 16 * N + 2 * ND)) != cudaSuccess) return e;
    // two independent passes side by side (one after the other with a probe)
    auto pair_of = [&](const LineParams &a, const LineParams &b, int mode, const char *na, const char *nb,
                       double bytes) -> cudaError_t {
        cudaStream_t s2 = serial ? st : s.aux[0];
        cudaError_t r;
        if (!serial) {
            if ((r = cudaEventRecord(s.fork, st)) != cudaSuccess) return r;
            if ((r = cudaStreamWaitEvent(s2, s.fork, 0)) != cudaSuccess) return r;
        }
        if ((r = launch_line(a, mode, 0, wpb, st)) != cudaSuccess) return r;
        if ((r = mark(na, bytes)) != cudaSuccess) return r;
        if ((r = launch_line(b, mode, 0, wpb, s2)) != cudaSuccess) return r;
        if ((r = mark(nb, bytes)) != cudaSuccess) return r;
        if (!serial) {
            if ((r = cudaEventRecord(s.join[0], s2)) != cudaSuccess) return r;
            if ((r = cudaStreamWaitEvent(st, s.join[0], 0)) != cudaSuccess) return r;
        }
        return cudaSuccess;
    };
    LineParams tb = base, bt = base;
    tb.dx = 0; tb.dy = 1; tb.sc = ptb; tb.nlines = lines_for(base.W, base.H, 0, 1);
    bt.dx = 0; bt.dy = -1; bt.sc = pbt; bt.nlines = tb.nlines;
    if ((e = pair_of(tb, bt, MODE_SCRATCH, "path_tb", "path_bt", 2 * ND)) != cudaSuccess) return e;
    LineParams lr = base;
    lr.dx = 1; lr.dy = 0; lr.hseg = 2; lr.state = s.state;
    lr.sc = ph; lr.sc2 = ptb; lr.sc3 = pbt; lr.disp = disp;
    lr.nlines = lines_for(base.W, base.H, 1, 0);
    lr.key16 = base.D <= 64 ? 1 : 0;                      // S*64 + d < 2^16 with 4 paths
    LineParams rl = lr;
    rl.dx = -1;
    return pair_of(lr, rl, MODE_FINAL3H, "path_lr_final", "path_rl_final", 2 * ND + N / 2);
}

// The SPLIT schedule (the frames of fused_applies), after census and cost:
// the first halves of both horizontal passes (plain scratch passes over half
// of each row, L into one plane, line state at the half's end) run side by
// side with the two vertical passes; then the second halves resume the rows,
// add the three planes and take the argmin, as in the FUSED schedule. The
// cost pass uses the whole GPU, and the half-rows overlap the vertical
// passes, so the critical path is census, cost, the longer of the vertical
// pass and the half row, and a half row.
cudaError_t run_split(const FrameSlot &s, const LineParams &base, int wpb, cudaStream_t st, Marker &mark,
                      uint8_t *disp, double N) {
    const bool serial = mark.pr != nullptr;
    const size_t plane = (size_t)base.W * base.H * base.D;
    const double ND = (double)plane;
    uint8_t *ph = s.sc, *ptb = (uint8_t *)s.S, *pbt = (uint8_t *)s.S + plane;
    LineParams q[4];
    for (int k = 0; k < 4; k++) q[k] = base;
    q[0].dx = 1; q[0].dy = 0; q[0].hseg = 1; q[0].state = s.state; q[0].sc = ph;
    q[1] = q[0]; q[1].dx = -1;
    q[0].nlines = q[1].nlines = lines_for(base.W, base.H, 1, 0);
    q[2].dx = 0; q[2].dy = 1; q[2].sc = ptb; q[2].nlines = lines_for(base.W, base.H, 0, 1);
    q[3] = q[2]; q[3].dy = -1; q[3].sc = pbt;
    static const char *names[4] = {"path_lr_first", "path_rl_first", "path_tb", "path_bt"};
    const double bytes[4] = {ND, ND, 2 * ND, 2 * ND};
    cudaStream_t ss[4];
    for (int k = 0; k < 4; k++) ss[k] = (serial || k == 0) ? st : s.aux[k - 1];
    cudaError_t e;
    if (!serial) {
        if ((e = cudaEventRecord(s.fork, st)) != cudaSuccess) return e;
        for (int k = 1; k < 4; k++)
            if ((e = cudaStreamWaitEvent(ss[k], s.fork, 0)) != cudaSuccess) return e;
    }
    for (int k : {2, 3, 0, 1}) {                          // the longer vertical passes first
        if ((e = launch_line(q[k], MODE_SCRATCH, 0, wpb, ss[k])) != cudaSuccess) return e;
        if ((e = mark(names[k], bytes[k])) != cudaSuccess) return e;
    }
    if (!serial) {
        for (int k = 1; k < 4; k++) {
            if ((e = cudaEventRecord(s.join[k - 1], ss[k])) != cudaSuccess) return e;
            if ((e = cudaStreamWaitEvent(st, s.join[k - 1], 0)) != cudaSuccess) return e;
        }
    }
    LineParams lr = base;
    lr.dx = 1; lr.dy = 0; lr.hseg = 2; lr.state = s.state;
    lr.sc = ph; lr.sc2 = ptb; lr.sc3 = pbt; lr.disp = disp;
    lr.nlines = lines_for(base.W, base.H, 1, 0);
    LineParams rl = lr;
    rl.dx = -1;
    cudaStream_t s2 = serial ? st : s.aux[0];
    if (!serial) {
        if ((e = cudaEventRecord(s.fork, st)) != cudaSuccess) return e;
        if ((e = cudaStreamWaitEvent(s2, s.fork, 0)) != cudaSuccess) return e;
    }
    if ((e = launch_line(lr, MODE_FINAL3H, 0, wpb, st)) != cudaSuccess) return e;
    if ((e = mark("path_lr_final", 2 * ND + N / 2)) != cudaSuccess) return e;
    if ((e = launch_line(rl, MODE_FINAL3H, 0, wpb, s2)) != cudaSuccess) return e;
    if ((e = mark("path_rl_final", 2 * ND + N / 2)) != cudaSuccess) return e;
    if (!serial) {
        if ((e = cudaEventRecord(s.join[0], s2)) != cudaSuccess) return e;
        if ((e = cudaStreamWaitEvent(st, s.join[0], 0)) != cudaSuccess) return e;
    }
    return cudaSuccess;
}

cudaError_t run_dirs(const PathShape &shape, const Fan &f, const LineParams &base, int npaths, int sat,
                     bool ms, cudaStream_t st, Marker &mark, int even_only, uint8_t *disp, double Nout) {
    if (shape.sched == SGMGB_SCHED_LATENCY)
        return run_planes(f, base, npaths, sat, ms, shape.wpb, st, mark, even_only, disp, Nout);
    return run_final(f, base, npaths, sat, ms, shape.wpb, st, mark, even_only, disp, Nout);
}

}  // namespace

cudaError_t enqueue_frame(const FrameSlot &s, const uint8_t *d_left, const uint8_t *d_right,
                          uint8_t *d_disp, cudaStream_t st, const PathShape &shape,
                          cudaEvent_t ev_census, cudaEvent_t ev_end, KernelProbe *probe) {
    const sgmgb_frame_desc &fd = s.fd;
    Marker mark{probe, st};
    const double N = (double)fd.W * fd.H, ND = N * fd.D;
    cudaError_t e;
    if ((e = mark.start()) != cudaSuccess) return e;
    if (fd.variant == SGMGB_PLAIN && shape.sched == SGMGB_SCHED_FUSED && fused_applies(fd, shape)) {
        if ((e = launch_census2(d_left, d_right, s.cl, s.cr, fd.W, fd.H, st)) != cudaSuccess) return e;
        if ((e = mark("census", 18 * N)) != cudaSuccess) return e;
        if (ev_census && (e = cudaEventRecord(ev_census, st)) != cudaSuccess) return e;
        LineParams p{};
        p.C = s.C; p.W = fd.W; p.H = fd.H; p.D = fd.D; p.dpl = 0; p.p1 = 20; p.p2 = 192;
        if ((e = run_fused(s, p, shape.wpb, st, mark, d_disp, N)) != cudaSuccess) return e;
    } else if (fd.variant == SGMGB_PLAIN && shape.sched == SGMGB_SCHED_SPLIT && fused_applies(fd, shape)) {
        if ((e = launch_census2(d_left, d_right, s.cl, s.cr, fd.W, fd.H, st)) != cudaSuccess) return e;
        if ((e = mark("census", 18 * N)) != cudaSuccess) return e;
        if ((e = launch_cost(s.cl, s.cr, s.C, nullptr, fd.W, fd.H, fd.D, kInvalidPlain, st)) != cudaSuccess)
            return e;
        if ((e = mark("cost", 16 * N + ND)) != cudaSuccess) return e;
        if (ev_census && (e = cudaEventRecord(ev_census, st)) != cudaSuccess) return e;
        LineParams p{};
        p.C = s.C; p.W = fd.W; p.H = fd.H; p.D = fd.D; p.dpl = 0; p.p1 = 20; p.p2 = 192;
        if ((e = run_split(s, p, shape.wpb, st, mark, d_disp, N)) != cudaSuccess) return e;
    } else if (fd.variant == SGMGB_PLAIN) {
        if ((e = launch_census2(d_left, d_right, s.cl, s.cr, fd.W, fd.H, st)) != cudaSuccess) return e;
        if ((e = mark("census", 18 * N)) != cudaSuccess) return e;
        if ((e = launch_cost(s.cl, s.cr, s.C, nullptr, fd.W, fd.H, fd.D, kInvalidPlain, st)) != cudaSuccess)
            return e;
        if ((e = mark("cost", 16 * N + ND)) != cudaSuccess) return e;
        if (ev_census && (e = cudaEventRecord(ev_census, st)) != cudaSuccess) return e;
        LineParams p{};
        p.C = s.C; p.sc = s.sc; p.S = s.S; p.disp = d_disp;
        p.W = fd.W; p.H = fd.H; p.D = fd.D; p.dpl = shape.dpl;
        p.p2 = 192; p.even_only = 0; p.p1 = 20;
        if ((e = run_dirs(shape, main_fan(s, (size_t)ND), p, fd.paths, 0, false, st, mark, 0, d_disp, N)) !=
            cudaSuccess)
            return e;
    } else {
        const int W = fd.W, H = fd.H, hw = W / 2, hh = H / 2;
        const double Nh = (double)hw * hh, NhD = Nh * 64;
        // The half-scale stage (multiscale/sgm_ms_ref.c:168-181) runs on its own
        // stream set beside the full-scale prefilters and stage: the full scale
        // needs only its cost volume, in the cost merge; its map is defined work
        // that nothing reads. With a probe attached everything runs on `st`, in
        // the order below.
        const bool serial = probe != nullptr;
        cudaStream_t sm = serial ? st : s.ms;
        if (!serial) {
            if ((e = cudaEventRecord(s.fork_ms, st)) != cudaSuccess) return e;
            if ((e = cudaStreamWaitEvent(sm, s.fork_ms, 0)) != cudaSuccess) return e;
        }
        if ((e = launch_half2(d_left, d_right, s.halfL, s.halfR, W, H, sm)) != cudaSuccess) return e;
        if ((e = mark("half", 2 * N + 2 * Nh)) != cudaSuccess) return e;
        if ((e = launch_sobel2(s.halfL, s.halfR, s.hsobL, s.hsobR, hw, hh, sm)) != cudaSuccess) return e;
        if ((e = mark("sobel_half", 4 * Nh)) != cudaSuccess) return e;
        if ((e = launch_census2(s.hsobL, s.hsobR, s.cl1, s.cr1, hw, hh, sm)) != cudaSuccess) return e;
        if ((e = mark("census_half", 18 * Nh)) != cudaSuccess) return e;
        if ((e = launch_cost(s.cl1, s.cr1, s.C1, nullptr, hw, hh, 64, kInvalidMultiscale, sm)) != cudaSuccess)
            return e;
        if ((e = mark("cost_half", 16 * Nh + NhD)) != cudaSuccess) return e;
        if (!serial && (e = cudaEventRecord(s.c1, sm)) != cudaSuccess) return e;
        // the full-scale prefilters, beside the half-scale chain
        if ((e = launch_sobel2(d_left, d_right, s.sobL, s.sobR, W, H, st)) != cudaSuccess) return e;
        if ((e = mark("sobel", 4 * N)) != cudaSuccess) return e;
        if ((e = launch_census2(s.sobL, s.sobR, s.cl, s.cr, W, H, st)) != cudaSuccess) return e;
        if ((e = mark("census", 18 * N)) != cudaSuccess) return e;
        if (!serial && (e = cudaStreamWaitEvent(st, s.c1, 0)) != cudaSuccess) return e;
        if ((e = launch_cost(s.cl, s.cr, s.C, s.C1, W, H, 64, kInvalidMultiscale, st)) != cudaSuccess)
            return e;
        if ((e = mark("cost_merge", 16 * N + NhD + ND)) != cudaSuccess) return e;
        if (ev_census && (e = cudaEventRecord(ev_census, st)) != cudaSuccess) return e;
        // stage 1's path passes and map on the half-scale stream set, in its own planes
        LineParams p1{};
        p1.C = s.C1; p1.disp = s.disp1;
        p1.W = hw; p1.H = hh; p1.D = 64; p1.dpl = shape.dpl; p1.p2 = 200; p1.even_only = 0;
        if ((e = run_dirs(shape, half_fan(s, (size_t)NhD), p1, 8, 1, true, sm, mark, 0, s.disp1, Nh)) !=
            cudaSuccess)
            return e;
        if (!serial && (e = cudaEventRecord(s.s1_done, sm)) != cudaSuccess) return e;
        // stage 2: full scale, cost averaged with the half-scale cost (:183-199)
        LineParams p2{};
        p2.C = s.C; p2.sc = s.sc; p2.S = s.S; p2.disp = d_disp;
        p2.W = W; p2.H = H; p2.D = 64; p2.dpl = shape.dpl; p2.p2 = 200; p2.even_only = 1;
        if ((e = run_dirs(shape, main_fan(s, (size_t)ND), p2, 8, 1, true, st, mark, 1, d_disp, Nh)) !=
            cudaSuccess)
            return e;
        if (!serial && (e = cudaStreamWaitEvent(st, s.s1_done, 0)) != cudaSuccess) return e;
    }
    if (ev_end && (e = cudaEventRecord(ev_end, st)) != cudaSuccess) return e;
    return cudaSuccess;
}

cudaError_t capture_frame(const FrameSlot &s, cudaStream_t st, const PathShape &sh, cudaGraphExec_t *out) {
    cudaGraph_t g = nullptr;
    cudaError_t e = cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal);
    if (e != cudaSuccess) return e;
    cudaError_t ee = enqueue_frame(s, s.left, s.right, s.disp, st, sh, nullptr, nullptr);
    e = cudaStreamEndCapture(st, &g);
    if (ee != cudaSuccess) { if (g) cudaGraphDestroy(g); return ee; }
    if (e != cudaSuccess) return e;
    e = cudaGraphInstantiate(out, g, 0);
    cudaGraphDestroy(g);
    return e;
}


}  // namespace sgmgb

// ---------------------------------------------------------------------------
// C ABI
// ---------------------------------------------------------------------------
extern "C" {

static void drop_graph(sgmgb_ctx *ctx);
static cudaError_t alone_graph(sgmgb_ctx *ctx, cudaGraphExec_t *out);
static int cuda_fail(sgmgb_ctx *ctx, cudaError_t e, const char *what);

int sgmgb_abi_version(void) { return SGMGB_ABI_VERSION; }

const char *sgmgb_strerror(int code) {
    switch (code) {
    case SGMGB_OK: return "ok";
    case SGMGB_ERR_ARG: return "invalid argument";
    case SGMGB_ERR_NOMEM: return "out of memory";
    case SGMGB_ERR_CUDA: return "CUDA error";
    case SGMGB_ERR_NODEV: return "no CUDA device";
    case SGMGB_ERR_BUDGET: return "refused: over the HBM budget or no free slot";
    case SGMGB_ERR_TIMEOUT: return "wait timed out";
    case SGMGB_ERR_STATE: return "invalid state";
    default: return "unknown error";
    }
}

const char *sgmgb_last_error(const sgmgb_ctx *ctx) { return ctx ? ctx->last_error.c_str() : ""; }

int sgmgb_check_desc(const sgmgb_frame_desc *fd) {
    if (!fd) return SGMGB_ERR_ARG;
    if (fd->W < 1 || fd->H < 1 || fd->W > 32768 || fd->H > 32768) return SGMGB_ERR_ARG;
    if (fd->variant == SGMGB_PLAIN) {
        if (fd->D < 16 || fd->D > 256 || fd->D % 16) return SGMGB_ERR_ARG;
        if (fd->paths != 4 && fd->paths != 8) return SGMGB_ERR_ARG;
        return SGMGB_OK;
    }
    if (fd->variant == SGMGB_MULTISCALE) {
        if (fd->D != 64 || fd->paths != 8) return SGMGB_ERR_ARG;
        if (fd->W < 2 || fd->H < 2 || (fd->W & 1) || (fd->H & 1)) return SGMGB_ERR_ARG;
        return SGMGB_OK;
    }
    return SGMGB_ERR_ARG;
}

int sgmgb_out_size(const sgmgb_frame_desc *fd, int *out_w, int *out_h) {
    int rc = sgmgb_check_desc(fd);
    if (rc) return rc;
    const bool ms = fd->variant == SGMGB_MULTISCALE;
    if (out_w) *out_w = ms ? fd->W / 2 : fd->W;
    if (out_h) *out_h = ms ? fd->H / 2 : fd->H;
    return SGMGB_OK;
}

int sgmgb_workspace_bytes(const sgmgb_frame_desc *fd, size_t *bytes) {
    int rc = sgmgb_check_desc(fd);
    if (rc) return rc;
    if (bytes) *bytes = slot_layout(*fd, nullptr);
    return SGMGB_OK;
}

int sgmgb_create(int device, sgmgb_ctx **out) {
    if (!out) return SGMGB_ERR_ARG;
    *out = nullptr;
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess || n <= 0) { cudaGetLastError(); return SGMGB_ERR_NODEV; }
    if (device < 0 || device >= n) return SGMGB_ERR_ARG;
    sgmgb_ctx *ctx = new (std::nothrow) sgmgb_ctx();
    if (!ctx) return SGMGB_ERR_NOMEM;
    ctx->device = device;
    cudaError_t e = cudaSetDevice(device);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&ctx->sm_count, cudaDevAttrMultiProcessorCount, device);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking);
    for (int i = 0; i < 5 && e == cudaSuccess; i++) e = cudaEventCreate(&ctx->ev[i]);
    if (e == cudaSuccess) e = prepare_path_kernels();
    if (e != cudaSuccess) {
        cudaGetLastError();
        sgmgb_destroy(ctx);
        return SGMGB_ERR_CUDA;
    }
    *out = ctx;
    return SGMGB_OK;
}

int sgmgb_profile_frame(sgmgb_ctx *ctx, const uint8_t *d_left, const uint8_t *d_right, uint8_t *d_disp,
                        int reps, sgmgb_kernel_stat *out, int max_out, int *n_out) {
    if (!ctx || !d_left || !d_right || !d_disp || reps < 1 || !out || max_out < 1 || !n_out) return SGMGB_ERR_ARG;
    if (!ctx->planned) return set_err(ctx, SGMGB_ERR_STATE, "sgmgb_plan has not been called");
    cudaSetDevice(ctx->device);
    KernelProbe pr;
    cudaError_t e = cudaSuccess;
    for (int i = 0; i <= KernelProbe::kMax && e == cudaSuccess; i++) e = cudaEventCreate(&pr.ev[i]);
    std::vector<double> sum(KernelProbe::kMax, 0.0);
    int n = 0;
    for (int r = 0; r < reps && e == cudaSuccess; r++) {
        pr.n = 0;
        e = enqueue_frame(*ctx->slot, d_left, d_right, d_disp, ctx->stream, resolve_sched(ctx->shape, true, ctx->fd),
                          nullptr, nullptr, &pr);
        if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
        for (int k = 0; k < pr.n && e == cudaSuccess; k++) {
            float ms = 0.f;
            e = cudaEventElapsedTime(&ms, pr.ev[k], pr.ev[k + 1]);
            sum[k] += ms;
        }
        n = pr.n;
    }
    for (int i = 0; i <= KernelProbe::kMax; i++) if (pr.ev[i]) cudaEventDestroy(pr.ev[i]);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "profile_frame");
    *n_out = std::min(n, max_out);
    for (int k = 0; k < *n_out; k++) {
        memset(out[k].name, 0, sizeof out[k].name);
        strncpy(out[k].name, pr.name[k], sizeof out[k].name - 1);
        out[k].ms = sum[k] / reps;
        out[k].bytes = pr.bytes[k];
    }
    return SGMGB_OK;
}

int sgmgb_set_path_shape(sgmgb_ctx *ctx, int warps_per_block, int disp_per_lane) {
    if (!ctx) return SGMGB_ERR_ARG;
    if (warps_per_block < 1 || warps_per_block > 4)
        return set_err(ctx, SGMGB_ERR_ARG, "warps_per_block must be 1..4");
    if (disp_per_lane != 0 && disp_per_lane != 2 && disp_per_lane != 4 && disp_per_lane != 8)
        return set_err(ctx, SGMGB_ERR_ARG, "disp_per_lane must be 0, 2, 4 or 8");
    cudaSetDevice(ctx->device);
    cudaStreamSynchronize(ctx->stream);
    drop_graph(ctx);
    ctx->shape.wpb = warps_per_block;
    ctx->shape.dpl = disp_per_lane;
    return SGMGB_OK;
}

int sgmgb_set_schedule(sgmgb_ctx *ctx, int schedule) {
    if (!ctx) return SGMGB_ERR_ARG;
    if (schedule != SGMGB_SCHED_AUTO && schedule != SGMGB_SCHED_LATENCY && schedule != SGMGB_SCHED_THROUGHPUT &&
        schedule != SGMGB_SCHED_FUSED && schedule != SGMGB_SCHED_SPLIT)
        return set_err(ctx, SGMGB_ERR_ARG, "schedule must be SGMGB_SCHED_AUTO, _LATENCY, _THROUGHPUT, _FUSED or _SPLIT");
    cudaSetDevice(ctx->device);
    cudaStreamSynchronize(ctx->stream);
    drop_graph(ctx);
    ctx->shape.sched = schedule;
    return SGMGB_OK;
}

void sgmgb_destroy(sgmgb_ctx *ctx) {
    if (!ctx) return;
    cudaSetDevice(ctx->device);
    if (ctx->stream) cudaStreamSynchronize(ctx->stream);
    drop_graph(ctx);
    slot_free(ctx->slot);
    if (ctx->post) cudaFree(ctx->post);
    for (auto &e : ctx->ev) if (e) cudaEventDestroy(e);
    if (ctx->stream) cudaStreamDestroy(ctx->stream);
    delete ctx;
}

int sgmgb_plan(sgmgb_ctx *ctx, const sgmgb_frame_desc *fd) {
    if (!ctx) return SGMGB_ERR_ARG;
    int rc = sgmgb_check_desc(fd);
    if (rc) return set_err(ctx, rc, "invalid frame description");
    if (ctx->planned && !memcmp(&ctx->fd, fd, sizeof *fd)) return SGMGB_OK;
    cudaSetDevice(ctx->device);
    if (ctx->slot) {
        cudaStreamSynchronize(ctx->stream);
        drop_graph(ctx);
        slot_free(ctx->slot);
        ctx->slot = nullptr;
        ctx->planned = false;
    }
    std::string err;
    rc = slot_alloc(*fd, &ctx->slot, err);
    if (rc) return set_err(ctx, rc, err);
    ctx->fd = *fd;
    ctx->planned = true;
    // One frame of each schedule on the slot's own zeroed buffers, so every
    // kernel variant the description runs is loaded here (lazy module
    // loading) and not inside the first frame's stage times.
    const FrameSlot &s = *ctx->slot;
    const size_t N = (size_t)fd->W * fd->H;
    cudaError_t e = cudaMemsetAsync(s.left, 0, N, ctx->stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(s.right, 0, N, ctx->stream);
    for (int sched : {SGMGB_SCHED_LATENCY, SGMGB_SCHED_THROUGHPUT, SGMGB_SCHED_FUSED, SGMGB_SCHED_SPLIT}) {
        PathShape sh = ctx->shape;
        sh.sched = sched;
        if ((sched == SGMGB_SCHED_FUSED || sched == SGMGB_SCHED_SPLIT) && !fused_applies(*fd, sh)) continue;
        if (e == cudaSuccess) e = enqueue_frame(s, s.left, s.right, s.disp, ctx->stream, sh, nullptr, nullptr);
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "plan (kernel warm-up)");
    return SGMGB_OK;
}

static int cuda_fail(sgmgb_ctx *ctx, cudaError_t e, const char *what) {
    cudaGetLastError();
    return set_err(ctx, SGMGB_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

int sgmgb_alone_schedule(sgmgb_ctx *ctx, int *schedule) {
    if (!ctx || !schedule) return SGMGB_ERR_ARG;
    if (!ctx->planned) return set_err(ctx, SGMGB_ERR_STATE, "sgmgb_plan has not been called");
    cudaSetDevice(ctx->device);
    cudaGraphExec_t g = nullptr;
    cudaError_t e = alone_graph(ctx, &g);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "frame graph");
    *schedule = ctx->alone_sched;
    return SGMGB_OK;
}

int sgmgb_run_frame(sgmgb_ctx *ctx, const uint8_t *left, const uint8_t *right, uint8_t *disp,
                    sgmgb_stage_times *t) {
    if (!ctx || !left || !right || !disp) return SGMGB_ERR_ARG;
    if (!ctx->planned) return set_err(ctx, SGMGB_ERR_STATE, "sgmgb_plan has not been called");
    cudaSetDevice(ctx->device);
    const FrameSlot &s = *ctx->slot;
    const size_t N = (size_t)s.fd.W * s.fd.H;
    int ow = 0, oh = 0;
    sgmgb_out_size(&s.fd, &ow, &oh);
    const size_t outN = (size_t)ow * oh;
    // The images go into the slot by the copy engines, the frame runs as one
    // CUDA graph (the schedule that timed fastest for a frame alone) and the
    // map comes back by one copy; one stream, one wait at the end. Measured at
    // 1920x1080 D=64 on page-locked buffers: 0.385 ms, against 0.400 ms with
    // the kernels reading the images and writing the map across NVLink-C2C
    // and launched one by one. (Also measured slower: the two images on two
    // streams; the images in two row bands with the census of the top band
    // started early; stage events inside the graph, 17 us. No faster: the
    // copies as nodes of the graph, pointed at each call's page-locked
    // buffers, the images in two row bands with the top band's census and
    // cost beside the bottom band's copy: 0.384 ms against 0.384 at 1080p
    // D=64, 0.376-0.393 against 0.361 at 1280x720 D=128.)
    cudaStream_t st = ctx->stream;
    cudaGraphExec_t g = nullptr;
    cudaError_t e = alone_graph(ctx, &g);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "frame graph");
    cudaEvent_t *ev = ctx->ev;   // 0 start, 3 inputs in, 2 frame done, 4 map out
    const bool timed = t && ctx->timed_calls++ % 8 == 0;
    e = timed ? cudaEventRecord(ev[0], st) : cudaSuccess;
    if (e == cudaSuccess) e = cudaMemcpyAsync(s.left, left, N, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(s.right, right, N, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess && timed) e = cudaEventRecord(ev[3], st);
    if (e == cudaSuccess) e = cudaGraphLaunch(g, st);
    if (e == cudaSuccess && timed) e = cudaEventRecord(ev[2], st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(disp, s.disp, outN, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess && timed) e = cudaEventRecord(ev[4], st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "frame (copies and pipeline)");
    if (timed) {
        // the frame is one graph: census, cost, the passes and the argmin are
        // one phase, aggregate_ms; the others are -1, whose work the
        // reference's cost gate folds into aggregate (common/roofline.h:67-77)
        float agg = 0, in = 0, out = 0;
        cudaEventElapsedTime(&agg, ev[3], ev[2]);
        cudaEventElapsedTime(&in, ev[0], ev[3]);
        cudaEventElapsedTime(&out, ev[2], ev[4]);
        ctx->last_times = sgmgb_stage_times{-1, -1, agg, -1, (double)in + out, 0};
    }
    if (t) *t = ctx->last_times;
    return SGMGB_OK;
}

static void drop_graph(sgmgb_ctx *ctx) {
    for (int i = 0; i < sgmgb_ctx::kGraphs; i++) {
        if (ctx->graph[i]) cudaGraphExecDestroy(ctx->graph[i]);
        ctx->graph[i] = nullptr;
        ctx->graph_key[i][0] = ctx->graph_key[i][1] = ctx->graph_key[i][2] = nullptr;
    }
    ctx->graph_next = 0;
    if (ctx->alone) cudaGraphExecDestroy(ctx->alone);
    ctx->alone = nullptr;
    ctx->timed_calls = 0;   // the next synchronous call measures its stage times
}

// The frame on the slot's own buffers under schedule `sh`. (No stage event
// inside: an event node in the graph measured 17 us slower per 1080p frame.)
static cudaError_t capture_alone(sgmgb_ctx *ctx, const PathShape &sh, cudaGraphExec_t *out) {
    return capture_frame(*ctx->slot, ctx->stream, sh, out);
}

// The synchronous call's graph. Under AUTO each schedule that applies to the
// description is captured and replayed (two untimed runs, then the fastest
// of five timed one at a time, on the slot's current buffers) and the fastest
// is kept: which one wins
// depends on the frame's size, D and variant and on the part (measured on
// one GB300: split at 1920x1080 D=64, latency at 1920x800 multi-scale,
// throughput at 1920x1080 multi-scale).
static cudaError_t alone_graph(sgmgb_ctx *ctx, cudaGraphExec_t *out) {
    if (ctx->alone) { *out = ctx->alone; return cudaSuccess; }
    int cand[4], nc = 0;
    if (ctx->shape.sched != SGMGB_SCHED_AUTO) {
        cand[nc++] = ctx->shape.sched;
    } else {
        for (int sc : {SGMGB_SCHED_LATENCY, SGMGB_SCHED_THROUGHPUT, SGMGB_SCHED_FUSED, SGMGB_SCHED_SPLIT}) {
            PathShape sh = ctx->shape;
            sh.sched = sc;
            if (sc >= SGMGB_SCHED_FUSED && !fused_applies(ctx->fd, sh)) continue;
            cand[nc++] = sc;
        }
    }
    cudaGraphExec_t best = nullptr;
    float best_ms = 0.f;
    int best_sched = cand[0];
    cudaError_t e = cudaSuccess;
    for (int i = 0; i < nc && e == cudaSuccess; i++) {
        PathShape sh = ctx->shape;
        sh.sched = cand[i];
        cudaGraphExec_t g = nullptr;
        e = capture_alone(ctx, sh, &g);
        if (e != cudaSuccess) break;
        float ms = 0.f;
        if (nc > 1) {
            // the fastest of five frames, each alone (the candidates differ by a
            // few per cent, less than one run's spread)
            for (int r = 0; r < 2 && e == cudaSuccess; r++) e = cudaGraphLaunch(g, ctx->stream);
            ms = 1e30f;
            for (int r = 0; r < 5 && e == cudaSuccess; r++) {
                float one = 0.f;
                e = cudaEventRecord(ctx->ev[0], ctx->stream);
                if (e == cudaSuccess) e = cudaGraphLaunch(g, ctx->stream);
                if (e == cudaSuccess) e = cudaEventRecord(ctx->ev[4], ctx->stream);
                if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
                if (e == cudaSuccess) e = cudaEventElapsedTime(&one, ctx->ev[0], ctx->ev[4]);
                ms = std::min(ms, one);
            }
        }
        if (e != cudaSuccess) { cudaGraphExecDestroy(g); break; }
        if (!best || ms < best_ms) {
            if (best) cudaGraphExecDestroy(best);
            best = g; best_ms = ms; best_sched = cand[i];
        } else {
            cudaGraphExecDestroy(g);
        }
    }
    if (e != cudaSuccess) {
        if (best) cudaGraphExecDestroy(best);
        return e;
    }
    ctx->alone = best;
    ctx->alone_sched = best_sched;
    *out = best;
    return cudaSuccess;
}


// Captures the frame pipeline for this pointer triple into a CUDA graph on
// the context's stream (one graph launch per frame afterwards).
static cudaError_t capture_frame_graph(sgmgb_ctx *ctx, const uint8_t *l, const uint8_t *r, uint8_t *d,
                                       cudaGraphExec_t *out) {
    cudaGraph_t g = nullptr;
    cudaError_t e = cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal);
    if (e != cudaSuccess) return e;
    cudaError_t ee = enqueue_frame(*ctx->slot, l, r, d, ctx->stream, resolve_sched(ctx->shape, false, ctx->fd), nullptr,
                                   nullptr);
    e = cudaStreamEndCapture(ctx->stream, &g);
    if (ee != cudaSuccess) { if (g) cudaGraphDestroy(g); return ee; }
    if (e != cudaSuccess) return e;
    e = cudaGraphInstantiate(out, g, 0);
    cudaGraphDestroy(g);
    return e;
}

static cudaError_t frame_graph(sgmgb_ctx *ctx, const uint8_t *l, const uint8_t *r, uint8_t *d,
                               cudaGraphExec_t *out) {
    for (int i = 0; i < sgmgb_ctx::kGraphs; i++)
        if (ctx->graph[i] && ctx->graph_key[i][0] == l && ctx->graph_key[i][1] == r && ctx->graph_key[i][2] == d) {
            *out = ctx->graph[i];
            return cudaSuccess;
        }
    const int k = ctx->graph_next;
    ctx->graph_next = (k + 1) % sgmgb_ctx::kGraphs;
    if (ctx->graph[k]) { cudaGraphExecDestroy(ctx->graph[k]); ctx->graph[k] = nullptr; }
    cudaError_t e = capture_frame_graph(ctx, l, r, d, &ctx->graph[k]);
    if (e != cudaSuccess) { ctx->graph[k] = nullptr; return e; }
    ctx->graph_key[k][0] = l; ctx->graph_key[k][1] = r; ctx->graph_key[k][2] = d;
    *out = ctx->graph[k];
    return cudaSuccess;
}

int sgmgb_run_frame_async(sgmgb_ctx *ctx, const uint8_t *d_left, const uint8_t *d_right,
                          uint8_t *d_disp, void *stream) {
    if (!ctx || !d_left || !d_right || !d_disp) return SGMGB_ERR_ARG;
    if (!ctx->planned) return set_err(ctx, SGMGB_ERR_STATE, "sgmgb_plan has not been called");
    cudaSetDevice(ctx->device);
    cudaStream_t st = stream ? (cudaStream_t)stream : ctx->stream;
    cudaGraphExec_t g = nullptr;
    cudaError_t e = frame_graph(ctx, d_left, d_right, d_disp, &g);
    if (e == cudaSuccess) e = cudaGraphLaunch(g, st);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "frame pipeline");
    return SGMGB_OK;
}

int sgmgb_sync(sgmgb_ctx *ctx, void *stream) {
    if (!ctx) return SGMGB_ERR_ARG;
    cudaSetDevice(ctx->device);
    cudaError_t e = cudaStreamSynchronize(stream ? (cudaStream_t)stream : ctx->stream);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "stream synchronize");
    return SGMGB_OK;
}

int sgmgb_census_async(sgmgb_ctx *ctx, const uint8_t *d_img, uint64_t *d_out, int W, int H,
                       void *stream) {
    if (!ctx || !d_img || !d_out || W < 1 || H < 1) return SGMGB_ERR_ARG;
    cudaSetDevice(ctx->device);
    cudaStream_t st = stream ? (cudaStream_t)stream : ctx->stream;
    cudaError_t e = launch_census2(d_img, nullptr, d_out, nullptr, W, H, st);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "census");
    return SGMGB_OK;
}

}  // extern "C"
