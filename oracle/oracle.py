"""ctypes binding of the CPU oracle (sgm_oracle.c).

TEST INFRASTRUCTURE ONLY: the parity tests, the smoke check and the CPU
baseline leg of the benchmark use it as the checker. The engine never imports
it. Building: `build()` compiles sgm_oracle.c with gcc into oracle/_build/.
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "libsgm_oracle.so")
SRC = os.path.join(HERE, "sgm_oracle.c")


def build():
    os.makedirs(OUT, exist_ok=True)
    if os.path.exists(LIB) and os.path.getmtime(LIB) >= max(os.path.getmtime(SRC),
                                                            os.path.getmtime(os.path.join(HERE, "sgm_oracle.h"))):
        return LIB
    subprocess.run(["gcc", "-O2", "-Wall", "-Wextra", "-fPIC", "-shared", "-ffp-contract=off",
                    SRC, "-o", LIB], check=True)
    return LIB


_lib = None


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
