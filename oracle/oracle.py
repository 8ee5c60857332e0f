"""ctypes binding of the CPU oracle (sgm_oracle.c) and of the reference's own
CPU path built from its sources (oracle/build_ref.sh -> oracle/_ref/).

TEST INFRASTRUCTURE ONLY: the parity tests, the smoke check and the CPU
baseline and reference legs of the benchmark use it, as the checker and as
the timed CPU baseline. The engine never imports it. Building: `build()`
compiles sgm_oracle.c with gcc into oracle/_build/, and, beside it, the
synthetic-pair generator of the benchmark configurations (the package's
csrc/synth.c, compiled into a library of its own so that the CPU-only legs
make the same scenes without loading the engine).
"""
import ctypes
import os
import re
import subprocess
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "libsgm_oracle.so")
SRC = os.path.join(HERE, "sgm_oracle.c")
SYNTH_LIB = os.path.join(OUT, "libsgm_synth.so")
SYNTH_SRC = os.path.join(ROOT, "sgm-bench_gb300", "csrc", "synth.c")
REF_DIR = os.path.join(HERE, "_ref")


def _stale(target, deps):
    return not os.path.exists(target) or any(os.path.getmtime(d) > os.path.getmtime(target) for d in deps)


def build():
    os.makedirs(OUT, exist_ok=True)
    if _stale(LIB, [SRC, os.path.join(HERE, "sgm_oracle.h")]):
        subprocess.run(["gcc", "-O2", "-Wall", "-Wextra", "-fPIC", "-shared", "-ffp-contract=off",
                        SRC, "-o", LIB], check=True)
    hdr = os.path.join(ROOT, "include", "sgmgb.h")
    if _stale(SYNTH_LIB, [SYNTH_SRC, hdr]):
        subprocess.run(["gcc", "-O2", "-Wall", "-Wextra", "-fPIC", "-shared", "-ffp-contract=off",
                        "-I" + os.path.join(ROOT, "include"), SYNTH_SRC, "-o", SYNTH_LIB, "-lm"], check=True)
    return LIB


_lib = None
_synth = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(LIB)
        vp, i = ctypes.c_void_p, ctypes.c_int
        L.sgmo_census.argtypes = [vp, vp, i, i]
        L.sgmo_plain.argtypes = [vp, vp, i, i, i, i, vp, vp]
        L.sgmo_multiscale.argtypes = [vp, vp, i, i, vp]
        L.sgmo_sobelx.argtypes = [vp, vp, i, i]
        L.sgmo_half.argtypes = [vp, vp, i, i]
        L.sgmo_gen_reference.argtypes = [i, i, i, ctypes.c_uint32, vp, vp, vp]
        L.sgmo_post.argtypes = [vp, vp, i, i, i, i, i, vp, vp]
        L.sgmo_fnv1a64.argtypes = [vp, ctypes.c_size_t]
        L.sgmo_fnv1a64.restype = ctypes.c_uint64
        _lib = L
    return _lib


def _p(a):
    return a.ctypes.data


def census(img):
    img = np.ascontiguousarray(img, np.uint8)
    H, W = img.shape
    out = np.empty((H, W), np.uint64)
    assert lib().sgmo_census(_p(img), _p(out), W, H) == 0
    return out


def plain(left, right, D=64, paths=4, with_sum=False):
    left = np.ascontiguousarray(left, np.uint8)
    right = np.ascontiguousarray(right, np.uint8)
    H, W = left.shape
    disp = np.empty((H, W), np.uint8)
    S = np.empty((H, W, D), np.uint16) if with_sum else None
    rc = lib().sgmo_plain(_p(left), _p(right), W, H, D, paths, _p(disp), _p(S) if with_sum else None)
    if rc:
        raise ValueError("oracle rejected W=%d H=%d D=%d paths=%d" % (W, H, D, paths))
    return (disp, S) if with_sum else disp


def multiscale(left, right):
    left = np.ascontiguousarray(left, np.uint8)
    right = np.ascontiguousarray(right, np.uint8)
    H, W = left.shape
    disp = np.empty((H // 2, W // 2), np.uint8)
    rc = lib().sgmo_multiscale(_p(left), _p(right), W, H, _p(disp))
    if rc:
        raise ValueError("oracle rejected multi-scale W=%d H=%d" % (W, H))
    return disp


POST_LR, POST_MEDIAN, POST_SUBPIXEL = 1, 2, 4


def post(left, right, D=64, paths=4, flags=0):
    """The optional post-steps (no reference counterpart; defined in
    sgm_oracle.c): (map, 16x subpixel map or None)."""
    left = np.ascontiguousarray(left, np.uint8)
    right = np.ascontiguousarray(right, np.uint8)
    H, W = left.shape
    disp = np.empty((H, W), np.uint8)
    d16 = np.empty((H, W), np.uint16) if flags & POST_SUBPIXEL else None
    rc = lib().sgmo_post(_p(left), _p(right), W, H, D, paths, flags, _p(disp), _p(d16) if d16 is not None else None)
    if rc:
        raise ValueError("oracle rejected post W=%d H=%d D=%d paths=%d flags=%d" % (W, H, D, paths, flags))
    return disp, d16


def gen_reference(W, H, D, seed):
    """The reference's gen_synthetic scene (left, right, gt)."""
    l, r, g = (np.empty((H, W), np.uint8) for _ in range(3))
    rc = lib().sgmo_gen_reference(W, H, D, seed, _p(l), _p(r), _p(g))
    if rc:
        raise ValueError("generator rejected W=%d H=%d D=%d" % (W, H, D))
    return l, r, g


def fnv1a64(a):
    a = np.ascontiguousarray(a)
    return "%016x" % lib().sgmo_fnv1a64(_p(a), a.nbytes)


def synth_pair(W, H, D, seed):
    """The benchmark configurations' synthetic pair (left, right, gt): the
    same bytes as the engine's sgmgb_synth_pair, from the same source file."""
    global _synth
    if _synth is None:
        build()
        L = ctypes.CDLL(SYNTH_LIB)
        L.sgmgb_synth_pair.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_uint64,
                                       ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
        _synth = L
    l, r, g = (np.empty((H, W), np.uint8) for _ in range(3))
    if _synth.sgmgb_synth_pair(W, H, D, seed, _p(l), _p(r), _p(g)):
        raise ValueError("generator rejected W=%d H=%d D=%d" % (W, H, D))
    return l, r, g


# ---- the reference's own CPU path (built by build_ref.sh; absent without its sources) ----
class _StageTimes(ctypes.Structure):
    _fields_ = [("census_ms", ctypes.c_double), ("cost_ms", ctypes.c_double),
                ("aggregate_ms", ctypes.c_double), ("argmin_ms", ctypes.c_double),
                ("transfer_ms", ctypes.c_double), ("threads_used", ctypes.c_int)]


_RUN_FN = ctypes.CFUNCTYPE(ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, ctypes.c_int,
                           ctypes.c_void_p, ctypes.c_int, ctypes.POINTER(_StageTimes))


class _Impl(ctypes.Structure):
    _fields_ = [("name", ctypes.c_char_p), ("run", _RUN_FN)]


class ReferenceImpl:
    """The reference's sgm_ref.c (compile-time D and path count) as a shared
    library, called through its own SGM_IMPL exactly as common/harness.c:150-158
    calls it. ctypes releases the interpreter lock during the call, and
    ref_run keeps its buffers on the heap, so threads may call it at once."""

    def __init__(self, D=64, paths=4):
        path = os.path.join(REF_DIR, "libsgm_ref_d%d_p%d.so" % (D, paths))
        if not os.path.exists(path):
            raise FileNotFoundError("reference library not built: %s (oracle/build_ref.sh)" % path)
        self.path = path
        self._lib = ctypes.CDLL(path)
        self._impl = _Impl.in_dll(self._lib, "SGM_IMPL")
        self.name = self._impl.name.decode()
        self.D, self.paths = D, paths

    def run(self, left, right, disp=None):
        left = np.ascontiguousarray(left, np.uint8)
        right = np.ascontiguousarray(right, np.uint8)
        H, W = left.shape
        if disp is None:
            disp = np.empty((H, W), np.uint8)
        t = _StageTimes(-1, -1, -1, -1, -1, 0)
        rc = self._impl.run(_p(left), _p(right), W, H, _p(disp), 0, ctypes.byref(t))
        if rc:
            raise RuntimeError("reference run failed (%d)" % rc)
        return disp


def reference_available(D=64, paths=4):
    return os.path.exists(os.path.join(REF_DIR, "libsgm_ref_d%d_p%d.so" % (D, paths)))


def write_pgm(path, a):
    with open(path, "wb") as f:
        f.write(b"P5\n%d %d\n255\n" % (a.shape[1], a.shape[0]))
        f.write(np.ascontiguousarray(a, np.uint8).tobytes())


def reference_multiscale(left, right, reps=1, threads=None):
    """Runs the reference's multi-scale program (multiscale/sgm_ms_ref.c, built
    with OpenMP when the compiler has it) on this pair: `reps` timed frames.
    Returns (median ms as the program prints it, its FNV hash, the OpenMP
    build flag, the team size asked for)."""
    exe = os.path.join(REF_DIR, "sgm_ms_ref")
    if not os.path.exists(exe):
        raise FileNotFoundError("reference multi-scale program not built (oracle/build_ref.sh)")
    threads = threads or (len(os.sched_getaffinity(0)) if hasattr(os, "sched_getaffinity") else os.cpu_count())
    try:
        omp = open(os.path.join(REF_DIR, "sgm_ms_ref.omp")).read().strip()
    except OSError:
        omp = "unknown"
    with tempfile.TemporaryDirectory() as d:
        write_pgm(os.path.join(d, "l.pgm"), left)
        write_pgm(os.path.join(d, "r.pgm"), right)
        p = subprocess.run([exe, os.path.join(d, "l.pgm"), os.path.join(d, "r.pgm"), "-n", str(reps)],
                           capture_output=True, text=True, env=dict(os.environ, OMP_NUM_THREADS=str(threads)))
    m = re.search(r"median ([0-9.]+) ms .* hash ([0-9a-f]{16})", p.stdout)
    if p.returncode != 0 or not m:
        raise RuntimeError("sgm_ms_ref failed: " + p.stdout + p.stderr)
    return float(m.group(1)), m.group(2), omp, threads


# ---- the reference's own CUDA programs (built by build_ref.sh where nvcc is present) ----
def _read_pgm(path):
    with open(path, "rb") as f:
        data = f.read()
    m = re.match(rb"P5\s+(\d+)\s+(\d+)\s+(\d+)\s", data)
    if not m:
        raise ValueError("not a binary PGM: %s" % path)
    W, H = int(m.group(1)), int(m.group(2))
    return np.frombuffer(data[m.end():m.end() + W * H], np.uint8).reshape(H, W).copy()


def reference_cuda_available(what="sgm_cuda_opt_d64"):
    return os.path.exists(os.path.join(REF_DIR, what))


def reference_cuda_plain(left, right, D=64, warm=3, timed=20, timeout=120):
    """Runs the reference's cuda/sgm_cuda_opt.cu (4 paths, compile-time D) in
    the reference's own harness (common/harness.c) on this pair, with the
    harness's cost gate off. Each timed run is the harness's call: its
    pageable buffers copied in, the kernels, the map copied out. Returns
    (dict of the harness's median / p95 / min in ms, the map)."""
    exe = os.path.join(REF_DIR, "sgm_cuda_opt_d%d" % D)
    if not os.path.exists(exe):
        raise FileNotFoundError("reference CUDA program not built: %s (oracle/build_ref.sh)" % exe)
    with tempfile.TemporaryDirectory() as d:
        lp, rp, op = (os.path.join(d, n) for n in ("l.pgm", "r.pgm", "o.pgm"))
        write_pgm(lp, left)
        write_pgm(rp, right)
        p = subprocess.run([exe, lp, rp, "-o", op, "-w", str(warm), "-n", str(timed), "--no-roofline"],
                           capture_output=True, text=True, timeout=timeout)
        m = re.search(r"median\s+([0-9.]+) ms\s+p95\s+([0-9.]+)\s+min\s+([0-9.]+).* hash ([0-9a-f]{16})", p.stdout)
        if p.returncode != 0 or not m:
            raise RuntimeError("sgm_cuda_opt failed: " + p.stdout + p.stderr)
        disp = _read_pgm(op)
    return {"median_ms": float(m.group(1)), "p95_ms": float(m.group(2)), "min_ms": float(m.group(3)),
            "hash": m.group(4), "runs": timed, "warmup": warm}, disp


def reference_cuda_multiscale(left, right, reps=10, timeout=120):
    """Runs the reference's multiscale/sgm_ms_cuda.cu on this pair (its own
    main: the inputs copied once, then per timed frame the kernels and the
    map copied out; 3 warm-up frames). Returns (median ms it prints, its FNV
    hash, the half-resolution map)."""
    exe = os.path.join(REF_DIR, "sgm_ms_cuda")
    if not os.path.exists(exe):
        raise FileNotFoundError("reference multi-scale CUDA program not built (oracle/build_ref.sh)")
    with tempfile.TemporaryDirectory() as d:
        lp, rp, op = (os.path.join(d, n) for n in ("l.pgm", "r.pgm", "o.pgm"))
        write_pgm(lp, left)
        write_pgm(rp, right)
        p = subprocess.run([exe, lp, rp, "-o", op, "-n", str(reps)], capture_output=True, text=True,
                           timeout=timeout)
        m = re.search(r"median ([0-9.]+) ms .* hash ([0-9a-f]{16})", p.stdout)
        if p.returncode != 0 or not m:
            raise RuntimeError("sgm_ms_cuda failed: " + p.stdout + p.stderr)
        disp = _read_pgm(op)
    return float(m.group(1)), m.group(2), disp
