"""Host-side checks of the C ABI that need no GPU: the library and the sgm.h
plugins load and export every symbol the headers declare, and the host logic
(descriptions, sizes, errors, tune cache, scene generator) behaves."""
import ctypes
import os
import re

import numpy as np
import pytest

import sgmgb

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared(header):
    """Function names declared in a C header (prototypes ending in ';')."""
    src = open(os.path.join(ROOT, "include", header)).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    src = re.sub(r"//[^\n]*", "", src)
    names = set()
    for m in re.finditer(r"\b(sgm\w*)\s*\(([^;{]*)\)\s*;", src):
        names.add(m.group(1))
    return names


def test_every_declared_symbol_is_exported():
    declared = _declared("sgmgb.h")
    assert len(declared) >= 30
    assert declared == set(sgmgb.EXPORTS), declared ^ set(sgmgb.EXPORTS)
    lib = ctypes.CDLL(sgmgb.LIB_PATH)
    for name in declared:
        assert hasattr(lib, name), name


def test_header_constants_match_the_binding():
    """The #define values of the C header and the Python binding's constants
    (variants, schedules, error codes) are the same numbers."""
    src = open(os.path.join(ROOT, "include", "sgmgb.h")).read()
    defines = {m.group(1): int(m.group(2)) for m in re.finditer(r"#define\s+(SGMGB_\w+)\s+(-?\d+)", src)}
    assert defines["SGMGB_SCHED_AUTO"] == sgmgb.SCHED_AUTO
    assert defines["SGMGB_SCHED_LATENCY"] == sgmgb.SCHED_LATENCY
    assert defines["SGMGB_SCHED_THROUGHPUT"] == sgmgb.SCHED_THROUGHPUT
    assert defines["SGMGB_SCHED_FUSED"] == sgmgb.SCHED_FUSED
    assert defines["SGMGB_SCHED_SPLIT"] == sgmgb.SCHED_SPLIT
    enums = {m.group(1): int(m.group(2)) for m in re.finditer(r"(SGMGB_\w+)\s*=\s*(-?\d+)", src)}
    for name, value in (("SGMGB_OK", sgmgb.OK), ("SGMGB_ERR_ARG", sgmgb.ERR_ARG), ("SGMGB_ERR_NOMEM", sgmgb.ERR_NOMEM),
                        ("SGMGB_ERR_CUDA", sgmgb.ERR_CUDA), ("SGMGB_ERR_NODEV", sgmgb.ERR_NODEV),
                        ("SGMGB_ERR_BUDGET", sgmgb.ERR_BUDGET), ("SGMGB_ERR_TIMEOUT", sgmgb.ERR_TIMEOUT),
                        ("SGMGB_ERR_STATE", sgmgb.ERR_STATE), ("SGMGB_PLAIN", sgmgb.PLAIN),
                        ("SGMGB_MULTISCALE", sgmgb.MULTISCALE)):
        assert (enums.get(name) if name in enums else defines.get(name)) == value, name


@pytest.mark.parametrize("D,paths", [(64, 4), (128, 4), (64, 8), (128, 8)])
def test_plugin_exports_sgm_impl(D, paths):
    p = sgmgb.Plugin(D, paths)
    assert p.name.startswith("gb300")
    assert ctypes.cast(p.impl.run, ctypes.c_void_p).value


def test_abi_version_and_errors():
    assert sgmgb.lib.sgmgb_abi_version() >= 1
    for code in (sgmgb.OK, sgmgb.ERR_ARG, sgmgb.ERR_NOMEM, sgmgb.ERR_CUDA, sgmgb.ERR_NODEV, sgmgb.ERR_BUDGET,
                 sgmgb.ERR_TIMEOUT, sgmgb.ERR_STATE):
        assert sgmgb.strerror(code)
    assert sgmgb.strerror(-1000) != sgmgb.strerror(sgmgb.OK)


@pytest.mark.parametrize("args,ok", [
    ((640, 480, 64, 4, 0), True), ((1, 1, 16, 8, 0), True), ((1920, 1080, 256, 4, 0), True),
    ((2, 2, 64, 8, 1), True), ((1920, 800, 64, 8, 1), True),
    ((0, 10, 64, 4, 0), False), ((10, 0, 64, 4, 0), False), ((10, 10, 65, 4, 0), False),
    ((10, 10, 0, 4, 0), False), ((10, 10, 272, 4, 0), False), ((10, 10, 64, 6, 0), False),
    ((11, 10, 64, 8, 1), False), ((10, 10, 128, 8, 1), False), ((10, 10, 64, 4, 1), False),
    ((10, 10, 64, 4, 2), False)])
def test_check_desc(args, ok):
    assert (sgmgb.check_desc(*args) == sgmgb.OK) == ok


def test_out_size_and_workspace():
    assert sgmgb.out_size(1920, 1080, 64, 4) == (1920, 1080)
    assert sgmgb.out_size(1920, 800, 64, 8, sgmgb.MULTISCALE) == (960, 400)
    small, big = sgmgb.workspace_bytes(640, 480, 64, 4), sgmgb.workspace_bytes(1920, 1080, 64, 4)
    N = 1920 * 1080
    assert big >= N * 64 * 5 + 16 * N                 # cost volume, four direction planes, census
    assert big < N * 64 * 5 + 24 * N + (1 << 16)
    assert small < big
    assert sgmgb.workspace_bytes(1920, 1080, 128, 4) > big
    with pytest.raises(sgmgb.SgmError):
        sgmgb.workspace_bytes(10, 10, 65, 4)


def test_create_without_gpu_reports_nodev():
    torch = pytest.importorskip("torch")
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    with pytest.raises(sgmgb.SgmError) as ei:
        sgmgb.Engine(0)
    assert ei.value.code == sgmgb.ERR_NODEV


def test_tune_cache(tmp_path):
    path = str(tmp_path / "cache.txt")
    fd = sgmgb.desc(1920, 1080, 64, 4)
    w, d = ctypes.c_int(), ctypes.c_int()
    look = lambda f: sgmgb.lib.sgmgb_tune_lookup(path.encode(), ctypes.byref(f), ctypes.byref(w), ctypes.byref(d))
    assert look(fd) == sgmgb.ERR_STATE                    # no file yet
    assert sgmgb.lib.sgmgb_tune_record(path.encode(), ctypes.byref(fd), 4, 2, 610.0) == sgmgb.OK
    assert sgmgb.lib.sgmgb_tune_record(path.encode(), ctypes.byref(fd), 2, 4, 590.0) == sgmgb.OK
    assert look(fd) == sgmgb.OK and (w.value, d.value) == (2, 4)    # the last matching line wins
    other = sgmgb.desc(640, 480, 64, 4)
    assert look(other) == sgmgb.ERR_STATE
    for bad in ((0, 2), (5, 2), (4, 3), (4, 16)):
        assert sgmgb.lib.sgmgb_tune_record(path.encode(), ctypes.byref(fd), bad[0], bad[1], 1.0) == sgmgb.ERR_ARG
    with open(path, "a") as f:
        f.write("# comment\ngarbage line\n1920 1080 64 4 0 9 2 1.0\n")   # out-of-range shape is ignored
    assert look(fd) == sgmgb.OK and (w.value, d.value) == (2, 4)


def test_synth_pair_deterministic_and_plausible():
    a = sgmgb.synth_pair(320, 200, 64, 7)
    b = sgmgb.synth_pair(320, 200, 64, 7)
    c = sgmgb.synth_pair(320, 200, 64, 8)
    for x, y in zip(a, b):
        assert np.array_equal(x, y)
    assert not np.array_equal(a[0], c[0])
    left, right, gt = a
    assert gt.max() <= 63 and left.std() > 20
    # right(x - gt) ~ left(x) where the pixel is visible: mostly within the noise
    H, W = left.shape
    ys, xs = np.mgrid[0:H, 0:W]
    ok = xs - gt.astype(int) >= 0
    diff = np.abs(left[ok].astype(int) - right[ys[ok], (xs - gt.astype(int))[ok]].astype(int))
    assert np.median(diff) <= 4
