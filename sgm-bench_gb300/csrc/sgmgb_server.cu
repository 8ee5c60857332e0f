// sgmgb_server.cu -- the served form: frames from several cameras admitted
// as they arrive, run concurrently on the device, results collected by ticket.
//
// Per camera:
//   - slots: resident device workspaces (inputs, census, cost, planes, sums,
//     output) sized for the camera's frame description. The first is allocated
//     when the camera is added; sgmgb_server_prepare makes more up front
//     (round-robin over the cameras, within the HBM budget), and otherwise
//     they are added on demand while the budget and the in-flight limit
//     allow. They stay resident.
//   - request buffers: pinned host memory holding one request's two input
//     images and its output map. submit() copies the caller's images into a
//     free one (or refuses the frame when none is free), so the H2D and D2H
//     copies of the frame go straight between pinned memory and the slot.
// A dispatcher thread admits queued requests (per camera, in arrival order)
// into free slots: each admitted frame is H2D, the frame pipeline and D2H on
// the slot's own stream, so frames of different slots overlap on the GPU.
// A host callback after the D2H stamps the completion time and wakes the
// dispatcher, which frees the slot and admits the next request at once.
// Latency = completion - submit, on the host clock.
#include "sgmgb_internal.h"
#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <mutex>
#include <new>
#include <set>
#include <thread>
#include <unordered_map>
#include <vector>

using namespace sgmgb;
using Clock = std::chrono::steady_clock;

namespace {

constexpr int kReqBufsPerCamera = 16;
constexpr int kMaxSlotsPerCamera = 4;

struct Camera;

struct Slot {
    FrameSlot *fs = nullptr;
    cudaStream_t st = nullptr;
    bool busy = false;
    // the frame on this slot's buffers as CUDA graphs: [0] with frames in
    // flight, [1] alone; captured when the slot is made (and again if the
    // context's shape changed since), one launch per frame instead of a
    // launch per kernel and fork on the dispatcher thread
    cudaGraphExec_t g[2] = {nullptr, nullptr};
    PathShape gsh[2];
};

bool same_shape(const PathShape &a, const PathShape &b) {
    return a.sched == b.sched && a.wpb == b.wpb && a.dpl == b.dpl;
}

// The slot's graph for shape sh (captured on the slot's idle stream when
// missing or stale), or null when the capture fails (no lock held).
cudaGraphExec_t slot_graph(Slot &sl, const PathShape &sh, int which) {
    if (sl.g[which] && same_shape(sl.gsh[which], sh)) return sl.g[which];
    if (sl.g[which]) cudaGraphExecDestroy(sl.g[which]);
    sl.g[which] = nullptr;
    cudaGraphExec_t g = nullptr;
    if (capture_frame(*sl.fs, sl.st, sh, &g) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    sl.g[which] = g;
    sl.gsh[which] = sh;
    return g;
}

void slot_release(Slot &sl) {
    for (auto &g : sl.g) if (g) cudaGraphExecDestroy(g);
    if (sl.st) { cudaStreamSynchronize(sl.st); cudaStreamDestroy(sl.st); }
    slot_free(sl.fs);
}

struct Request {
    uint64_t ticket = 0;
    Camera *cam = nullptr;
    int buf = -1;                     // request buffer index in the camera
    int slot = -1;                    // slot while on the device
    Clock::time_point t_submit, t_done;
    int state = 0;                    // 0 queued, 1 on device, 2 done, 3 failed
    struct sgmgb_server *srv = nullptr;
};

struct Camera {
    int id = 0;
    sgmgb_frame_desc fd{};
    size_t n_in = 0, n_out = 0;       // bytes of one image / of the output map
    std::vector<Slot> slots;
    std::vector<uint8_t *> bufs;      // pinned: left | right | out
    std::vector<bool> buf_used;
    std::deque<Request *> queue;      // admitted to the server, waiting for a slot
    int growing = 0;                  // slots being made for it right now
};

}  // namespace

struct sgmgb_server {
    sgmgb_ctx *ctx = nullptr;
    sgmgb_server_config cfg{};
    std::mutex mu;
    std::condition_variable cv_work, cv_done;
    std::thread worker;
    bool stop = false;
    bool kick = false;                // a request arrived: try to admit
    std::map<int, Camera *> cams;
    std::set<int> adding;             // cameras whose first slot is being made
    std::unordered_map<uint64_t, Request *> reqs;
    std::vector<Request *> finished;  // completed on the device, slot not yet released
    uint64_t next_ticket = 1;
    int inflight = 0;
    size_t resident = 0;
    // statistics
    uint64_t done = 0, refused = 0;
    std::vector<double> lat_ms;
    bool have_first = false;
    Clock::time_point first_submit, last_done;
    std::string last_error;
};

namespace {

int serr(sgmgb_server *s, int code, const std::string &m) {
    if (s) s->last_error = m;
    if (s && s->ctx) s->ctx->last_error = m;
    return code;
}

void CUDART_CB on_frame_done(void *p) {
    Request *r = (Request *)p;
    sgmgb_server *s = r->srv;
    // notify under the lock: once the dispatcher can see this request the
    // callback no longer touches the server (which may then be destroyed)
    std::lock_guard<std::mutex> g(s->mu);
    r->t_done = Clock::now();
    s->finished.push_back(r);
    s->cv_work.notify_one();
}

// Device bytes of one more slot for the camera, or 0 if limits forbid it (lock held).
size_t growth_bytes(const sgmgb_server *s, const Camera *c) {
    if ((int)c->slots.size() + c->growing >= kMaxSlotsPerCamera) return 0;
    const size_t need = slot_layout(c->fd, nullptr);
    return s->resident + need <= s->cfg.hbm_budget_bytes ? need : 0;
}

// Allocates one slot and captures its two frame graphs for `shape` (no lock
// held: CUDA calls only run without the lock, so a completion callback
// waiting for the lock can never hold up a CUDA call).
bool make_slot(const sgmgb_frame_desc &fd, const PathShape &shape, Slot *out) {
    Slot sl;
    std::string err;
    if (slot_alloc(fd, &sl.fs, err) != SGMGB_OK) return false;
    if (cudaStreamCreateWithFlags(&sl.st, cudaStreamNonBlocking) != cudaSuccess) {
        cudaGetLastError();
        slot_free(sl.fs);
        return false;
    }
    for (int which = 0; which < 2; which++) slot_graph(sl, resolve_sched(shape, which == 1, fd), which);
    *out = sl;
    return true;
}

// Enqueues request r on slot k of its camera (no lock held). `alone`: the
// frame was admitted with nothing else in flight (under SGMGB_SCHED_AUTO the
// schedule of a frame alone: SPLIT or LATENCY by size).
bool launch(sgmgb_server *s, Request *r, int k, bool alone, std::string &err) {
    Camera *c = r->cam;
    Slot &sl = c->slots[k];
    const FrameSlot &fs = *sl.fs;
    uint8_t *hb = c->bufs[r->buf];
    const PathShape sh = resolve_sched(s->ctx->shape, alone, fs.fd);
    cudaGraphExec_t g = slot_graph(sl, sh, alone ? 1 : 0);   // before the copies: the stream is idle
    cudaError_t e = cudaMemcpyAsync(fs.left, hb, c->n_in, cudaMemcpyHostToDevice, sl.st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(fs.right, hb + c->n_in, c->n_in, cudaMemcpyHostToDevice, sl.st);
    if (e == cudaSuccess)
        e = g ? cudaGraphLaunch(g, sl.st) : enqueue_frame(fs, fs.left, fs.right, fs.disp, sl.st, sh, nullptr, nullptr);
    if (e == cudaSuccess) e = cudaMemcpyAsync(hb + 2 * c->n_in, fs.disp, c->n_out, cudaMemcpyDeviceToHost, sl.st);
    if (e == cudaSuccess) e = cudaLaunchHostFunc(sl.st, on_frame_done, r);
    if (e != cudaSuccess) {
        cudaGetLastError();
        err = std::string("frame launch: ") + cudaGetErrorString(e);
        return false;
    }
    return true;
}

struct Admission {
    Request *r;
    int slot;        // -1: a new slot is to be made for it
    size_t grow;     // bytes reserved for that slot
    bool alone;      // nothing else in flight when it was admitted
};

// Picks queued requests for free slots, oldest head first over the cameras,
// reserving budget for new slots (lock held).
std::vector<Admission> plan_admissions(sgmgb_server *s) {
    std::vector<Admission> out;
    while (s->inflight < s->cfg.max_inflight) {
        Camera *pick = nullptr;
        int pick_k = -1;
        size_t pick_grow = 0;
        for (auto &kv : s->cams) {
            Camera *c = kv.second;
            if (c->queue.empty()) continue;
            if (pick && !(c->queue.front()->t_submit < pick->queue.front()->t_submit)) continue;
            int k = -1;
            for (int i = 0; i < (int)c->slots.size() && k < 0; i++)
                if (!c->slots[i].busy) k = i;
            const size_t g = k < 0 ? growth_bytes(s, c) : 0;
            if (k < 0 && g == 0) continue;      // must wait for one of its slots
            pick = c; pick_k = k; pick_grow = g;
        }
        if (!pick) break;
        Request *r = pick->queue.front();
        pick->queue.pop_front();
        if (pick_k >= 0) pick->slots[pick_k].busy = true;
        else { pick->growing++; s->resident += pick_grow; }
        r->state = 1;
        const bool alone = s->inflight == 0;
        s->inflight++;
        out.push_back({r, pick_k, pick_grow, alone});
    }
    return out;
}

void worker_main(sgmgb_server *s) {
    cudaSetDevice(s->ctx->device);
    std::unique_lock<std::mutex> lk(s->mu);
    for (;;) {
        s->cv_work.wait(lk, [&] { return (s->stop && s->inflight == 0) || s->kick || !s->finished.empty(); });
        s->kick = false;
        for (Request *r : s->finished) {
            r->cam->slots[r->slot].busy = false;
            r->state = 2;
            s->inflight--;
            s->done++;
            s->lat_ms.push_back(std::chrono::duration<double, std::milli>(r->t_done - r->t_submit).count());
            if (r->t_done > s->last_done) s->last_done = r->t_done;
        }
        if (!s->finished.empty()) { s->finished.clear(); s->cv_done.notify_all(); }
        if (s->stop) {
            if (s->inflight == 0) return;
            continue;
        }
        std::vector<Admission> todo = plan_admissions(s);
        if (todo.empty()) continue;
        lk.unlock();
        std::vector<std::pair<Admission, std::string>> failed;
        std::vector<std::pair<Camera *, size_t>> grown;   // (camera, reserved bytes) of made slots
        for (Admission &a : todo) {
            Camera *c = a.r->cam;
            std::string err;
            if (a.slot < 0) {
                Slot sl;
                if (!make_slot(c->fd, s->ctx->shape, &sl)) {
                    failed.push_back({a, "server: slot allocation failed"});
                    continue;
                }
                sl.busy = true;
                {
                    // appended under the lock (sgmgb_server_prepare appends too); the
                    // vector's capacity is reserved, so no slot ever moves
                    std::lock_guard<std::mutex> g(s->mu);
                    c->slots.push_back(sl);
                    a.slot = (int)c->slots.size() - 1;
                }
                grown.push_back({c, a.grow});
            }
            a.r->slot = a.slot;
            if (!launch(s, a.r, a.slot, a.alone, err)) failed.push_back({a, err});
        }
        lk.lock();
        for (auto &g : grown) g.first->growing--;
        for (Admission &a : todo)
            if (a.slot < 0 && a.grow) { a.r->cam->growing--; s->resident -= a.grow; }
        for (auto &f : failed) {
            Request *r = f.first.r;
            if (f.first.slot >= 0) r->cam->slots[f.first.slot].busy = false;
            r->state = 3;
            s->inflight--;
            s->last_error = f.second;
        }
        if (!failed.empty()) s->cv_done.notify_all();
    }
}

// Output map bytes of a description.
size_t out_bytes(const sgmgb_frame_desc &fd) {
    int w = 0, h = 0;
    sgmgb_out_size(&fd, &w, &h);
    return (size_t)w * h;
}

// Hands a finished request's output to the caller and releases it (lock held).
int collect(sgmgb_server *s, Request *r, uint8_t *disp, double *latency_ms) {
    Camera *c = r->cam;
    int rc = SGMGB_OK;
    if (r->state == 3) rc = serr(s, SGMGB_ERR_CUDA, s->last_error.empty() ? "frame failed" : s->last_error);
    else {
        if (disp) memcpy(disp, c->bufs[r->buf] + 2 * c->n_in, c->n_out);
        if (latency_ms) *latency_ms = std::chrono::duration<double, std::milli>(r->t_done - r->t_submit).count();
    }
    c->buf_used[r->buf] = false;
    s->reqs.erase(r->ticket);
    delete r;
    return rc;
}

}  // namespace

extern "C" {

int sgmgb_server_create(sgmgb_ctx *ctx, const sgmgb_server_config *cfg, sgmgb_server **out) {
    if (!ctx || !cfg || !out) return SGMGB_ERR_ARG;
    *out = nullptr;
    if (cfg->hbm_budget_bytes == 0 || cfg->max_inflight < 1)
        return set_err(ctx, SGMGB_ERR_ARG, "server: hbm_budget_bytes > 0 and max_inflight >= 1 required");
    sgmgb_server *s = new (std::nothrow) sgmgb_server();
    if (!s) return SGMGB_ERR_NOMEM;
    s->ctx = ctx;
    s->cfg = *cfg;
    try {
        s->worker = std::thread(worker_main, s);
    } catch (...) {
        delete s;
        return set_err(ctx, SGMGB_ERR_STATE, "server: cannot start the dispatcher thread");
    }
    *out = s;
    return SGMGB_OK;
}

int sgmgb_server_add_camera(sgmgb_server *s, int cam_id, const sgmgb_frame_desc *fd) {
    if (!s || !fd) return SGMGB_ERR_ARG;
    if (sgmgb_check_desc(fd) != SGMGB_OK) return serr(s, SGMGB_ERR_ARG, "server: invalid frame description");
    Camera *c = new (std::nothrow) Camera();
    if (!c) return SGMGB_ERR_NOMEM;
    c->id = cam_id;
    c->fd = *fd;
    c->n_in = (size_t)fd->W * fd->H;
    c->n_out = out_bytes(*fd);
    const size_t need = slot_layout(*fd, nullptr);
    {
        std::lock_guard<std::mutex> g(s->mu);
        if (s->cams.count(cam_id) || s->adding.count(cam_id)) {
            delete c;
            return serr(s, SGMGB_ERR_ARG, "server: camera " + std::to_string(cam_id) + " exists");
        }
        if (s->resident + need > s->cfg.hbm_budget_bytes) {
            delete c;
            return serr(s, SGMGB_ERR_BUDGET, "server: camera " + std::to_string(cam_id) + " needs " +
                                                 std::to_string(need) + " bytes; " + std::to_string(s->resident) +
                                                 " of " + std::to_string(s->cfg.hbm_budget_bytes) + " resident");
        }
        s->resident += need;           // reserved while the slot is made
        s->adding.insert(cam_id);
    }
    cudaSetDevice(s->ctx->device);
    Slot first;
    if (!make_slot(*fd, s->ctx->shape, &first)) {
        std::lock_guard<std::mutex> g(s->mu);
        s->resident -= need;
        s->adding.erase(cam_id);
        delete c;
        return serr(s, SGMGB_ERR_NOMEM, "server: camera " + std::to_string(cam_id) + ": slot allocation failed");
    }
    c->slots.reserve(kMaxSlotsPerCamera);   // slots never move once made
    c->slots.push_back(first);
    for (int i = 0; i < kReqBufsPerCamera; i++) {
        uint8_t *p = nullptr;
        if (cudaHostAlloc((void **)&p, 2 * c->n_in + c->n_out, cudaHostAllocDefault) != cudaSuccess) {
            cudaGetLastError();
            break;
        }
        c->bufs.push_back(p);
    }
    c->buf_used.assign(c->bufs.size(), false);
    if (c->bufs.empty()) {
        slot_release(first);
        std::lock_guard<std::mutex> g(s->mu);
        s->resident -= need;
        s->adding.erase(cam_id);
        delete c;
        return serr(s, SGMGB_ERR_NOMEM, "server: pinned request buffers");
    }
    std::lock_guard<std::mutex> g(s->mu);
    s->adding.erase(cam_id);
    s->cams[cam_id] = c;
    return SGMGB_OK;
}

int sgmgb_server_prepare(sgmgb_server *s, int slots_per_camera, int *slots_resident) {
    if (!s || slots_per_camera < 1) return SGMGB_ERR_ARG;
    const int want = std::min(slots_per_camera, kMaxSlotsPerCamera);
    cudaSetDevice(s->ctx->device);
    // round-robin over the cameras, one slot at a time, so the budget is shared
    for (bool progress = true; progress;) {
        progress = false;
        std::vector<std::pair<Camera *, size_t>> todo;
        {
            std::lock_guard<std::mutex> g(s->mu);
            for (auto &kv : s->cams) {
                Camera *c = kv.second;
                if ((int)c->slots.size() + c->growing >= want) continue;
                const size_t need = growth_bytes(s, c);
                if (!need) continue;
                c->growing++;
                s->resident += need;
                todo.push_back({c, need});
            }
        }
        for (auto &t : todo) {
            Slot sl;
            const bool ok = make_slot(t.first->fd, s->ctx->shape, &sl);
            std::lock_guard<std::mutex> g(s->mu);
            t.first->growing--;
            if (!ok) { s->resident -= t.second; continue; }
            // slots are appended only under the lock while the dispatcher may read them
            t.first->slots.push_back(sl);
            progress = true;
        }
    }
    std::lock_guard<std::mutex> g(s->mu);
    if (slots_resident) {
        int n = 0;
        for (auto &kv : s->cams) n += (int)kv.second->slots.size();
        *slots_resident = n;
    }
    return SGMGB_OK;
}

int sgmgb_server_submit(sgmgb_server *s, int cam_id, const uint8_t *left, const uint8_t *right, uint64_t *ticket) {
    if (!s || !left || !right || !ticket) return SGMGB_ERR_ARG;
    const Clock::time_point now = Clock::now();
    Camera *c;
    int b = -1;
    {
        std::lock_guard<std::mutex> g(s->mu);
        auto it = s->cams.find(cam_id);
        if (it == s->cams.end()) return serr(s, SGMGB_ERR_ARG, "server: unknown camera " + std::to_string(cam_id));
        c = it->second;
        for (int i = 0; i < (int)c->buf_used.size() && b < 0; i++)
            if (!c->buf_used[i]) b = i;
        if (b < 0) {
            s->refused++;
            return serr(s, SGMGB_ERR_BUDGET, "server: camera " + std::to_string(cam_id) + " has no free request buffer");
        }
        c->buf_used[b] = true;
        if (!s->have_first) { s->have_first = true; s->first_submit = now; }
    }
    // the copy runs without the lock: the buffer is ours until the request is collected
    memcpy(c->bufs[b], left, c->n_in);
    memcpy(c->bufs[b] + c->n_in, right, c->n_in);
    Request *r = new (std::nothrow) Request();
    std::lock_guard<std::mutex> g(s->mu);
    if (!r) { c->buf_used[b] = false; return SGMGB_ERR_NOMEM; }
    r->ticket = s->next_ticket++;
    r->cam = c;
    r->buf = b;
    r->t_submit = now;
    r->srv = s;
    s->reqs[r->ticket] = r;
    c->queue.push_back(r);
    s->kick = true;
    *ticket = r->ticket;
    s->cv_work.notify_one();
    return SGMGB_OK;
}

int sgmgb_server_poll(sgmgb_server *s, uint64_t ticket, uint8_t *disp, double *latency_ms) {
    if (!s) return SGMGB_ERR_ARG;
    std::lock_guard<std::mutex> g(s->mu);
    auto it = s->reqs.find(ticket);
    if (it == s->reqs.end()) return serr(s, SGMGB_ERR_ARG, "server: unknown ticket");
    Request *r = it->second;
    if (r->state < 2) return 0;
    const int rc = collect(s, r, disp, latency_ms);
    return rc ? rc : 1;
}

int sgmgb_server_wait(sgmgb_server *s, uint64_t ticket, uint8_t *disp, double *latency_ms, int timeout_ms) {
    if (!s) return SGMGB_ERR_ARG;
    std::unique_lock<std::mutex> lk(s->mu);
    auto it = s->reqs.find(ticket);
    if (it == s->reqs.end()) return serr(s, SGMGB_ERR_ARG, "server: unknown ticket");
    Request *r = it->second;
    const bool ok = s->cv_done.wait_for(lk, std::chrono::milliseconds(timeout_ms < 0 ? 0 : timeout_ms),
                                        [&] { return r->state >= 2; });
    if (!ok) return serr(s, SGMGB_ERR_TIMEOUT, "server: ticket " + std::to_string(ticket) + " not done in time");
    return collect(s, r, disp, latency_ms);
}

int sgmgb_server_stats_get(sgmgb_server *s, sgmgb_server_stats *st) {
    if (!s || !st) return SGMGB_ERR_ARG;
    std::lock_guard<std::mutex> g(s->mu);
    memset(st, 0, sizeof *st);
    st->frames_done = s->done;
    st->frames_refused = s->refused;
    st->resident_bytes = s->resident;
    if (!s->lat_ms.empty()) {
        std::vector<double> v = s->lat_ms;
        std::sort(v.begin(), v.end());
        auto q = [&](double f) { return v[std::min(v.size() - 1, (size_t)(f * (v.size() - 1) + 0.5))]; };
        st->p50_ms = q(0.50);
        st->p99_ms = q(0.99);
        st->max_ms = v.back();
        const double secs = std::chrono::duration<double>(s->last_done - s->first_submit).count();
        st->fps = secs > 0 ? (double)s->done / secs : 0.0;
    }
    return SGMGB_OK;
}

void sgmgb_server_destroy(sgmgb_server *s) {
    if (!s) return;
    {
        std::lock_guard<std::mutex> g(s->mu);
        s->stop = true;
        for (auto &kv : s->cams) {   // queued, never launched: drop
            for (Request *r : kv.second->queue) { s->reqs.erase(r->ticket); delete r; }
            kv.second->queue.clear();
        }
    }
    s->cv_work.notify_all();
    if (s->worker.joinable()) s->worker.join();
    cudaSetDevice(s->ctx->device);
    for (auto &kv : s->cams) {
        Camera *c = kv.second;
        for (Slot &sl : c->slots) slot_release(sl);
        for (uint8_t *p : c->bufs) cudaFreeHost(p);
        delete c;
    }
    for (auto &kv : s->reqs) delete kv.second;
    delete s;
}

}  // extern "C"
