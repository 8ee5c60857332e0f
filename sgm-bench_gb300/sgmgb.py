"""Python binding of the GB300 SGM engine's C ABI (include/sgmgb.h).

Host-side mirror of the reference's plugin interface for Python callers:
`Engine.run_frame(left, right)` is the single-frame call (common/sgm.h:29-31
`sgm_run_fn`: host buffers in, disparity map out, 0 or an error), and
`Plugin` calls the exported `SGM_IMPL` of a built plugin library exactly as
common/harness.c:150-158 does. Device buffers and streams may come from
PyTorch (any object with data_ptr(), or a raw integer address).

The compiled library is required: importing this module without it raises,
and there is no CPU fallback.
"""
import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
LIB_PATH = os.path.join(BUILD, "libsgmgb.so")

PLAIN, MULTISCALE = 0, 1
POST_LR, POST_MEDIAN, POST_SUBPIXEL, DISP_INVALID = 1, 2, 4, 255
SCHED_AUTO, SCHED_LATENCY, SCHED_THROUGHPUT, SCHED_FUSED, SCHED_SPLIT = 0, 1, 2, 3, 4
BATCH_PERSISTENT, BATCH_IN_FLIGHT = 0, 1
OK, ERR_ARG, ERR_NOMEM, ERR_CUDA, ERR_NODEV, ERR_BUDGET, ERR_TIMEOUT, ERR_STATE = 0, -1, -2, -3, -4, -5, -6, -7

# every symbol include/sgmgb.h declares
EXPORTS = [
    "sgmgb_abi_version", "sgmgb_strerror", "sgmgb_last_error", "sgmgb_check_desc", "sgmgb_out_size",
    "sgmgb_workspace_bytes", "sgmgb_create", "sgmgb_destroy", "sgmgb_plan", "sgmgb_set_path_shape",
    "sgmgb_set_schedule", "sgmgb_alone_schedule", "sgmgb_profile_frame",
    "sgmgb_run_frame",
    "sgmgb_run_frame_async", "sgmgb_sync", "sgmgb_census_async", "sgmgb_batch_create", "sgmgb_batch_run",
    "sgmgb_batch_wait", "sgmgb_batch_autotune", "sgmgb_batch_tile_shape", "sgmgb_batch_set_fault",
    "sgmgb_batch_destroy", "sgmgb_tune_lookup", "sgmgb_tune_record",
    "sgmgb_server_create", "sgmgb_server_add_camera", "sgmgb_server_submit", "sgmgb_server_poll",
    "sgmgb_server_wait", "sgmgb_server_stats_get", "sgmgb_server_destroy", "sgmgb_synth_pair",
    "sgmgb_server_prepare", "sgmgb_batch_busy", "sgmgb_run_frame_post",
    "sgmgb_run_frame_noalloc", "sgmgb_batch_set_mode", "sgmgb_batch_mode",
]


class FrameDesc(ctypes.Structure):
    _fields_ = [("W", ctypes.c_int), ("H", ctypes.c_int), ("D", ctypes.c_int),
                ("paths", ctypes.c_int), ("variant", ctypes.c_int)]


class StageTimes(ctypes.Structure):
    _fields_ = [("census_ms", ctypes.c_double), ("cost_ms", ctypes.c_double),
                ("aggregate_ms", ctypes.c_double), ("argmin_ms", ctypes.c_double),
                ("transfer_ms", ctypes.c_double), ("threads_used", ctypes.c_int)]

    def as_dict(self):
        return {f: getattr(self, f) for f, _ in self._fields_}


class KernelStat(ctypes.Structure):
    _fields_ = [("name", ctypes.c_char * 24), ("ms", ctypes.c_double), ("bytes", ctypes.c_double)]


class ServerConfig(ctypes.Structure):
    _fields_ = [("hbm_budget_bytes", ctypes.c_size_t), ("max_inflight", ctypes.c_int),
                ("streams", ctypes.c_int)]


class ServerStats(ctypes.Structure):
    _fields_ = [("frames_done", ctypes.c_uint64), ("frames_refused", ctypes.c_uint64),
                ("p50_ms", ctypes.c_double), ("p99_ms", ctypes.c_double), ("max_ms", ctypes.c_double),
                ("fps", ctypes.c_double), ("resident_bytes", ctypes.c_size_t)]


class SgmError(RuntimeError):
    def __init__(self, code, msg=""):
        super().__init__("%s (%d)%s" % (strerror(code), code, (": " + msg) if msg else ""))
        self.code = code


def _load():
    if not os.path.exists(LIB_PATH):
        raise ImportError("libsgmgb.so is not built (%s); run __graft_entry__.build()" % LIB_PATH)
    lib = ctypes.CDLL(LIB_PATH)
    vp, i, u8p, sz = ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p, ctypes.c_size_t
    fdp = ctypes.POINTER(FrameDesc)
    sig = {
        "sgmgb_abi_version": (i, []),
        "sgmgb_strerror": (ctypes.c_char_p, [i]),
        "sgmgb_last_error": (ctypes.c_char_p, [vp]),
        "sgmgb_check_desc": (i, [fdp]),
        "sgmgb_out_size": (i, [fdp, ctypes.POINTER(i), ctypes.POINTER(i)]),
        "sgmgb_workspace_bytes": (i, [fdp, ctypes.POINTER(sz)]),
        "sgmgb_create": (i, [i, ctypes.POINTER(vp)]),
        "sgmgb_destroy": (None, [vp]),
        "sgmgb_plan": (i, [vp, fdp]),
        "sgmgb_set_path_shape": (i, [vp, i, i]),
        "sgmgb_set_schedule": (i, [vp, i]),
        "sgmgb_alone_schedule": (i, [vp, ctypes.POINTER(i)]),
        "sgmgb_profile_frame": (i, [vp, u8p, u8p, u8p, i, ctypes.POINTER(KernelStat), i, ctypes.POINTER(i)]),
        "sgmgb_run_frame": (i, [vp, u8p, u8p, u8p, ctypes.POINTER(StageTimes)]),
        "sgmgb_run_frame_async": (i, [vp, u8p, u8p, u8p, vp]),
        "sgmgb_run_frame_post": (i, [vp, u8p, u8p, u8p, vp, i]),
        "sgmgb_sync": (i, [vp, vp]),
        "sgmgb_census_async": (i, [vp, u8p, vp, i, i, vp]),
        "sgmgb_batch_create": (i, [vp, fdp, i, ctypes.c_char_p, ctypes.POINTER(vp)]),
        "sgmgb_batch_run": (i, [vp, ctypes.POINTER(vp), ctypes.POINTER(vp), ctypes.POINTER(vp), vp]),
        "sgmgb_batch_wait": (i, [vp]),
        "sgmgb_batch_autotune": (i, [vp, ctypes.POINTER(vp), ctypes.POINTER(vp), ctypes.POINTER(vp),
                                     ctypes.c_char_p]),
        "sgmgb_batch_tile_shape": (i, [vp, i, ctypes.POINTER(i), ctypes.POINTER(i)]),
        "sgmgb_batch_busy": (i, [vp, ctypes.POINTER(ctypes.c_double), i, ctypes.POINTER(i)]),
        "sgmgb_batch_set_fault": (i, [vp, i, i]),
        "sgmgb_batch_set_mode": (i, [vp, i, i]),
        "sgmgb_batch_mode": (i, [vp, ctypes.POINTER(i), ctypes.POINTER(i)]),
        "sgmgb_batch_destroy": (None, [vp]),
        "sgmgb_tune_lookup": (i, [ctypes.c_char_p, fdp, ctypes.POINTER(i), ctypes.POINTER(i)]),
        "sgmgb_tune_record": (i, [ctypes.c_char_p, fdp, i, i, ctypes.c_double]),
        "sgmgb_server_create": (i, [vp, ctypes.POINTER(ServerConfig), ctypes.POINTER(vp)]),
        "sgmgb_server_add_camera": (i, [vp, i, fdp]),
        "sgmgb_server_prepare": (i, [vp, i, ctypes.POINTER(i)]),
        "sgmgb_server_submit": (i, [vp, i, u8p, u8p, ctypes.POINTER(ctypes.c_uint64)]),
        "sgmgb_server_poll": (i, [vp, ctypes.c_uint64, u8p, ctypes.POINTER(ctypes.c_double)]),
        "sgmgb_server_wait": (i, [vp, ctypes.c_uint64, u8p, ctypes.POINTER(ctypes.c_double), i]),
        "sgmgb_server_stats_get": (i, [vp, ctypes.POINTER(ServerStats)]),
        "sgmgb_server_destroy": (None, [vp]),
        "sgmgb_synth_pair": (i, [i, i, i, ctypes.c_uint64, u8p, u8p, u8p]),
        "sgmgb_run_frame_noalloc": (i, [u8p, u8p, u8p, i, i, i, i, vp]),
    }
    for name, (res, args) in sig.items():
        f = getattr(lib, name)
        f.restype = res
        f.argtypes = args
    return lib


lib = _load()


def strerror(code):
    return lib.sgmgb_strerror(code).decode()


def _ptr(x):
    """Address of a numpy array, a torch tensor, or an integer address."""
    if x is None:
        return None
    if isinstance(x, int):
        return x
    if isinstance(x, np.ndarray):
        return x.ctypes.data
    if hasattr(x, "data_ptr"):
        return x.data_ptr()
    raise TypeError("cannot take the address of %r" % type(x))


def _cstr(s):
    return None if s is None else os.fsencode(s)


def _stream(s):
    """cudaStream_t for a torch stream or a raw handle. None selects the
    engine context's own stream; a handle of 0 (torch's default stream) is
    passed as cudaStreamLegacy (1) so the engine orders with it."""
    if s is None:
        return None
    h = s if isinstance(s, int) else getattr(s, "cuda_stream", None)
    if h is None:
        raise TypeError("not a CUDA stream: %r" % (s,))
    return h if h != 0 else 1


def desc(W, H, D=64, paths=4, variant=PLAIN):
    return FrameDesc(W, H, D, paths, variant)


def check_desc(W, H, D=64, paths=4, variant=PLAIN):
    return lib.sgmgb_check_desc(ctypes.byref(desc(W, H, D, paths, variant)))


def out_size(W, H, D=64, paths=4, variant=PLAIN):
    w, h = ctypes.c_int(), ctypes.c_int()
    rc = lib.sgmgb_out_size(ctypes.byref(desc(W, H, D, paths, variant)), ctypes.byref(w), ctypes.byref(h))
    if rc:
        raise SgmError(rc)
    return w.value, h.value


def workspace_bytes(W, H, D=64, paths=4, variant=PLAIN):
    b = ctypes.c_size_t()
    rc = lib.sgmgb_workspace_bytes(ctypes.byref(desc(W, H, D, paths, variant)), ctypes.byref(b))
    if rc:
        raise SgmError(rc)
    return b.value


def synth_pair(W, H, D=64, seed=1):
    """Seeded synthetic pair (left, right, ground truth) as uint8 arrays of shape (H, W)."""
    left = np.empty((H, W), np.uint8)
    right = np.empty((H, W), np.uint8)
    gt = np.empty((H, W), np.uint8)
    rc = lib.sgmgb_synth_pair(W, H, D, seed, left.ctypes.data, right.ctypes.data, gt.ctypes.data)
    if rc:
        raise SgmError(rc)
    return left, right, gt


class Engine:
    """One engine context bound to one CUDA device."""

    def __init__(self, device=0):
        h = ctypes.c_void_p()
        rc = lib.sgmgb_create(device, ctypes.byref(h))
        if rc:
            raise SgmError(rc)
        self.h = h
        self.fd = None

    def close(self):
        if self.h:
            lib.sgmgb_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def _check(self, rc):
        if rc:
            raise SgmError(rc, lib.sgmgb_last_error(self.h).decode())

    def plan(self, W, H, D=64, paths=4, variant=PLAIN):
        self.fd = desc(W, H, D, paths, variant)
        self._check(lib.sgmgb_plan(self.h, ctypes.byref(self.fd)))
        return self

    def set_path_shape(self, warps_per_block=4, disp_per_lane=0):
        """Path-kernel shape (speed only; results are identical)."""
        self._check(lib.sgmgb_set_path_shape(self.h, warps_per_block, disp_per_lane))
        return self

    def set_schedule(self, schedule=SCHED_AUTO):
        """Frame schedule: SCHED_LATENCY, SCHED_THROUGHPUT, SCHED_FUSED,
        SCHED_SPLIT or SCHED_AUTO (speed only; results are identical)."""
        self._check(lib.sgmgb_set_schedule(self.h, schedule))
        return self

    def alone_schedule(self):
        """The schedule run_frame runs (SCHED_*): the set one, or under
        SCHED_AUTO the one that timed fastest for a frame alone."""
        v = ctypes.c_int()
        self._check(lib.sgmgb_alone_schedule(self.h, ctypes.byref(v)))
        return v.value

    def profile_frame(self, d_left, d_right, d_disp, reps=10):
        """Per-kernel mean device time (ms) and algorithmic bytes of the planned
        frame, every kernel timed alone with CUDA events: [(name, ms, bytes)]."""
        out = (KernelStat * 32)()
        n = ctypes.c_int()
        self._check(lib.sgmgb_profile_frame(self.h, _ptr(d_left), _ptr(d_right), _ptr(d_disp), reps, out, 32,
                                            ctypes.byref(n)))
        return [(out[k].name.decode(), out[k].ms, out[k].bytes) for k in range(n.value)]

    def run_frame(self, left, right, times=False, out=None):
        """Host arrays in, host disparity map out (the drop-in call). `out`: a
        C-contiguous uint8 array of the output size to fill (e.g. pinned memory,
        which the copy back writes fastest), else a new array."""
        left = np.ascontiguousarray(left, np.uint8)
        right = np.ascontiguousarray(right, np.uint8)
        H, W = left.shape
        if self.fd is None or (self.fd.W, self.fd.H) != (W, H):
            raise SgmError(ERR_STATE, "plan() this size first")
        ow, oh = out_size(W, H, self.fd.D, self.fd.paths, self.fd.variant)
        if out is None:
            disp = np.empty((oh, ow), np.uint8)
        else:
            if out.dtype != np.uint8 or out.shape != (oh, ow) or not out.flags["C_CONTIGUOUS"]:
                raise SgmError(ERR_ARG, "out must be a C-contiguous uint8 array of shape %r" % ((oh, ow),))
            disp = out
        st = StageTimes()
        self._check(lib.sgmgb_run_frame(self.h, left.ctypes.data, right.ctypes.data, disp.ctypes.data,
                                        ctypes.byref(st) if times else None))
        return (disp, st.as_dict()) if times else disp

    def run_frame_post(self, left, right, flags):
        """The plain frame with optional post-steps (POST_LR, POST_MEDIAN,
        POST_SUBPIXEL): (map, 16x subpixel map or None)."""
        left = np.ascontiguousarray(left, np.uint8)
        right = np.ascontiguousarray(right, np.uint8)
        H, W = left.shape
        disp = np.empty((H, W), np.uint8)
        d16 = np.empty((H, W), np.uint16) if flags & POST_SUBPIXEL else None
        self._check(lib.sgmgb_run_frame_post(self.h, left.ctypes.data, right.ctypes.data, disp.ctypes.data,
                                             d16.ctypes.data if d16 is not None else None, flags))
        return disp, d16

    def run_frame_async(self, d_left, d_right, d_disp, stream=None):
        """Device buffers (torch tensors or addresses), enqueued on `stream`."""
        self._check(lib.sgmgb_run_frame_async(self.h, _ptr(d_left), _ptr(d_right), _ptr(d_disp),
                                              _stream(stream)))

    def sync(self, stream=None):
        self._check(lib.sgmgb_sync(self.h, _stream(stream)))

    def census_async(self, d_img, d_out, W, H, stream=None):
        self._check(lib.sgmgb_census_async(self.h, _ptr(d_img), _ptr(d_out), W, H, _stream(stream)))


class Batch:
    """Many plain-variant frames of mixed shapes planned once and run as one
    persistent launch, or as frames in flight (set_mode), either replayed as a
    CUDA graph."""

    def __init__(self, engine, descs, tune_cache=None):
        self.engine = engine
        self.n = len(descs)
        self.descs = list(descs)
        arr = (FrameDesc * self.n)(*descs)
        h = ctypes.c_void_p()
        engine._check(lib.sgmgb_batch_create(engine.h, arr, self.n, _cstr(tune_cache), ctypes.byref(h)))
        self.h = h

    def _arrays(self, d_lefts, d_rights, d_disps):
        A = ctypes.c_void_p * self.n
        return (A(*[_ptr(x) for x in d_lefts]), A(*[_ptr(x) for x in d_rights]), A(*[_ptr(x) for x in d_disps]))

    def run(self, d_lefts, d_rights, d_disps, stream=None):
        """Enqueues the batch on device buffers; returns without waiting."""
        self.engine._check(lib.sgmgb_batch_run(self.h, *self._arrays(d_lefts, d_rights, d_disps), _stream(stream)))

    def wait(self):
        """Waits for the last run; raises SgmError(ERR_TIMEOUT) if it was abandoned."""
        self.engine._check(lib.sgmgb_batch_wait(self.h))

    def autotune(self, d_lefts, d_rights, d_disps, tune_cache=None):
        self.engine._check(lib.sgmgb_batch_autotune(self.h, *self._arrays(d_lefts, d_rights, d_disps),
                                                    _cstr(tune_cache)))

    BUSY_KINDS = ("census", "cost", "scratch", "final", "first_half_cost", "wait")

    def busy(self):
        """Milliseconds the last persistent launch's blocks spent per work-item
        kind (summed over blocks), and the block count under "blocks"."""
        out = (ctypes.c_double * 6)()
        nb = ctypes.c_int()
        self.engine._check(lib.sgmgb_batch_busy(self.h, out, 6, ctypes.byref(nb)))
        d = {k: out[i] for i, k in enumerate(self.BUSY_KINDS)}
        d["blocks"] = nb.value
        return d

    def tile_shape(self, i):
        """(warps per block, disparities per lane) used for frame i."""
        w, d = ctypes.c_int(), ctypes.c_int()
        self.engine._check(lib.sgmgb_batch_tile_shape(self.h, i, ctypes.byref(w), ctypes.byref(d)))
        return w.value, d.value

    def set_fault(self, wait_limit_ms=2000, stall_frame=-1):
        self.engine._check(lib.sgmgb_batch_set_fault(self.h, wait_limit_ms, stall_frame))

    def set_mode(self, mode, lanes=6):
        """BATCH_PERSISTENT (one persistent launch) or BATCH_IN_FLIGHT (every
        frame's own pipeline on `lanes` concurrent chains, one CUDA graph)."""
        self.engine._check(lib.sgmgb_batch_set_mode(self.h, mode, lanes))

    def mode(self):
        """(mode, lanes); lanes is 0 in the persistent mode."""
        m, k = ctypes.c_int(), ctypes.c_int()
        self.engine._check(lib.sgmgb_batch_mode(self.h, ctypes.byref(m), ctypes.byref(k)))
        return m.value, k.value

    def close(self):
        if self.h:
            lib.sgmgb_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Server:
    """The served form: cameras with resident slots, frames admitted as they
    arrive (HBM budget, in-flight limit), results collected by ticket."""

    def __init__(self, engine, hbm_budget_bytes=40 << 30, max_inflight=8, streams=8):
        self.engine = engine
        cfg = ServerConfig(hbm_budget_bytes, max_inflight, streams)
        h = ctypes.c_void_p()
        engine._check(lib.sgmgb_server_create(engine.h, ctypes.byref(cfg), ctypes.byref(h)))
        self.h = h
        self.cams = {}

    def add_camera(self, cam_id, W, H, D=64, paths=4, variant=PLAIN):
        fd = desc(W, H, D, paths, variant)
        self.engine._check(lib.sgmgb_server_add_camera(self.h, cam_id, ctypes.byref(fd)))
        self.cams[cam_id] = fd

    def prepare(self, slots_per_camera=4):
        """Makes the cameras' slots up front (round-robin, within the budget);
        returns the number of resident slots."""
        n = ctypes.c_int()
        self.engine._check(lib.sgmgb_server_prepare(self.h, slots_per_camera, ctypes.byref(n)))
        return n.value

    def submit(self, cam_id, left, right):
        left = np.ascontiguousarray(left, np.uint8)
        right = np.ascontiguousarray(right, np.uint8)
        t = ctypes.c_uint64()
        self.engine._check(lib.sgmgb_server_submit(self.h, cam_id, left.ctypes.data, right.ctypes.data,
                                                   ctypes.byref(t)))
        return t.value, cam_id

    def _out(self, cam_id):
        fd = self.cams[cam_id]
        ow, oh = out_size(fd.W, fd.H, fd.D, fd.paths, fd.variant)
        return np.empty((oh, ow), np.uint8)

    def poll(self, ticket):
        """(True, disp, latency_ms) when done, else (False, None, None)."""
        t, cam = ticket
        out, lat = self._out(cam), ctypes.c_double()
        rc = lib.sgmgb_server_poll(self.h, t, out.ctypes.data, ctypes.byref(lat))
        if rc < 0:
            self.engine._check(rc)
        return (True, out, lat.value) if rc == 1 else (False, None, None)

    def wait(self, ticket, timeout_ms=10000):
        t, cam = ticket
        out, lat = self._out(cam), ctypes.c_double()
        self.engine._check(lib.sgmgb_server_wait(self.h, t, out.ctypes.data, ctypes.byref(lat), timeout_ms))
        return out, lat.value

    def stats(self):
        st = ServerStats()
        self.engine._check(lib.sgmgb_server_stats_get(self.h, ctypes.byref(st)))
        return {f: getattr(st, f) for f, _ in st._fields_}

    def close(self):
        if self.h:
            lib.sgmgb_server_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Plugin:
    """A built sgm.h plugin library; calls its SGM_IMPL.run like the reference harness."""

    RUN = ctypes.CFUNCTYPE(ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, ctypes.c_int,
                           ctypes.c_void_p, ctypes.c_int, ctypes.POINTER(StageTimes))

    class Impl(ctypes.Structure):
        pass

    Impl._fields_ = [("name", ctypes.c_char_p), ("run", RUN)]

    def __init__(self, D=64, paths=4):
        path = os.path.join(BUILD, "libsgm_gb300_d%d_p%d.so" % (D, paths))
        if not os.path.exists(path):
            raise ImportError("plugin library %s is not built" % path)
        self.lib = ctypes.CDLL(path)
        self.impl = Plugin.Impl.in_dll(self.lib, "SGM_IMPL")
        self.name = self.impl.name.decode()

    def run(self, left, right, threads=0):
        left = np.ascontiguousarray(left, np.uint8)
        right = np.ascontiguousarray(right, np.uint8)
        H, W = left.shape
        disp = np.zeros((H, W), np.uint8)
        st = StageTimes(-1, -1, -1, -1, -1, 0)
        rc = self.impl.run(left.ctypes.data, right.ctypes.data, W, H, disp.ctypes.data, threads,
                           ctypes.byref(st))
        return rc, disp, st.as_dict()
