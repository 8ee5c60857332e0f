"""sgmgb_cli: the reference-style command line (multiscale/sgm_ms_ref.c:151-217
contract for `ms`; `plain` and `gen` beside it). PGM files in and out, the
result line with the FNV hash, exit status 2 on a golden mismatch."""
import json
import os
import re
import subprocess

import numpy as np
import pytest

import oracle
import sgmgb

CLI = os.path.join(os.path.dirname(sgmgb.LIB_PATH), "sgmgb_cli")


def _have_gpu():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


def write_pgm(path, a):
    with open(path, "wb") as f:
        f.write(b"P5\n# written by the test\n%d %d\n255\n" % (a.shape[1], a.shape[0]))
        f.write(np.ascontiguousarray(a, np.uint8).tobytes())


def read_pgm(path):
    d = open(path, "rb").read()
    i, tok = 2, []
    while len(tok) < 3:
        while d[i:i + 1].isspace():
            i += 1
        if d[i:i + 1] == b"#":
            while d[i:i + 1] != b"\n":
                i += 1
            continue
        j = i
        while not d[j:j + 1].isspace():
            j += 1
        tok.append(int(d[i:j]))
        i = j
    w, h, _ = tok
    return np.frombuffer(d[i + 1:i + 1 + w * h], np.uint8).reshape(h, w).copy()


def run(*args):
    return subprocess.run([CLI] + [str(a) for a in args], capture_output=True, text=True)


def test_cli_usage_and_gen(tmp_path):
    assert os.path.exists(CLI)
    assert run().returncode == 1
    assert run("ms").returncode == 1
    p = run("gen", 96, 40, 64, 5, tmp_path)
    assert p.returncode == 0, p.stderr
    l, r, g = sgmgb.synth_pair(96, 40, 64, 5)
    assert np.array_equal(read_pgm(str(tmp_path / "left.pgm")), l)
    assert np.array_equal(read_pgm(str(tmp_path / "right.pgm")), r)
    assert np.array_equal(read_pgm(str(tmp_path / "gt.pgm")), g)
    assert run("gen", 0, 40, 64, 5, tmp_path).returncode == 1


def test_cli_rejects_bad_input(tmp_path):
    (tmp_path / "bad.pgm").write_bytes(b"P2\n2 2\n255\n0 0 0 0\n")
    assert run("plain", tmp_path / "bad.pgm", tmp_path / "bad.pgm").returncode == 1
    assert run("plain", tmp_path / "none.pgm", tmp_path / "none.pgm").returncode == 1


@pytest.mark.skipif(_have_gpu(), reason="a GPU is present")
def test_cli_without_gpu_fails_cleanly(tmp_path):
    a = np.zeros((8, 8), np.uint8)
    write_pgm(str(tmp_path / "a.pgm"), a)
    p = run("plain", tmp_path / "a.pgm", tmp_path / "a.pgm")
    assert p.returncode == 1 and "gb300" in p.stderr


@pytest.mark.gpu
def test_cli_multiscale_golden(tmp_path):
    rng = np.random.default_rng(3)
    l = rng.integers(0, 256, (66, 130), dtype=np.uint8)
    r = rng.integers(0, 256, (66, 130), dtype=np.uint8)
    write_pgm(str(tmp_path / "l.pgm"), l)
    write_pgm(str(tmp_path / "r.pgm"), r)
    want = oracle.multiscale(l, r)
    write_pgm(str(tmp_path / "g.pgm"), want)
    p = run("ms", tmp_path / "l.pgm", tmp_path / "r.pgm", "-g", tmp_path / "g.pgm", "-n", 3,
            "-o", tmp_path / "o.pgm", "-j", tmp_path / "res.jsonl")
    assert p.returncode == 0, p.stdout + p.stderr
    line = p.stdout.strip()
    assert line.startswith("ms_gb300  in 130x66 out 65x33 D=64 paths=8  median ") and line.endswith("GOLDEN OK")
    assert ("hash " + oracle.fnv1a64(want)) in line
    assert np.array_equal(read_pgm(str(tmp_path / "o.pgm")), want)
    rec = json.loads(open(tmp_path / "res.jsonl").read().splitlines()[-1])
    assert rec["impl"] == "ms_gb300" and rec["golden_match"] == 1 and rec["hash"] == oracle.fnv1a64(want)
    bad = want.copy()
    bad[0, 0] ^= 1
    write_pgm(str(tmp_path / "bad.pgm"), bad)
    p = run("ms", tmp_path / "l.pgm", tmp_path / "r.pgm", "-g", tmp_path / "bad.pgm")
    assert p.returncode == 2 and p.stdout.strip().endswith("GOLDEN FAIL")


@pytest.mark.gpu
@pytest.mark.parametrize("D,paths", [(64, 4), (128, 8)])
def test_cli_plain_golden(tmp_path, D, paths):
    l, r, _ = sgmgb.synth_pair(200, 90, D, 8)
    write_pgm(str(tmp_path / "l.pgm"), l)
    write_pgm(str(tmp_path / "r.pgm"), r)
    want = oracle.plain(l, r, D, paths)
    write_pgm(str(tmp_path / "g.pgm"), want)
    p = run("plain", tmp_path / "l.pgm", tmp_path / "r.pgm", "-D", D, "-p", paths, "-g", tmp_path / "g.pgm", "-n", 2,
            "--no-roofline")
    assert p.returncode == 0, p.stdout + p.stderr
    m = HARNESS_LINE.match(p.stdout.splitlines()[0])
    assert m and m.group(1, 2, 3, 4) == ("200", "90", str(D), str(paths)), p.stdout
    assert m.group(16) == "  GOLDEN OK"


HARNESS_LINE = re.compile(
    r"^gb300\s+(\d+)x(\d+) D=(\d+) paths=(\d+) th=(\d+)  median\s+([0-9.]+) ms  p95\s+([0-9.]+)  min\s+([0-9.]+)"
    r"  sd\s+([0-9.]+)  spread ([0-9.]+)/([0-9.]+)( UNSTABLE)?  fps\s+([0-9.]+)  Mpix/s\s+([0-9.]+)  hash ([0-9a-f]{16})"
    r"(  GOLDEN OK|  GOLDEN FAIL)?$")
HARNESS_JSON_KEYS = {"impl", "board", "W", "H", "D", "paths", "census", "P1", "P2", "threads", "threads_requested",
                     "cpu_mask", "warm", "timed", "median_ms", "p95_ms", "min_ms", "rmsd_ms", "spread_hi", "spread_lo",
                     "unstable", "transfer_ms", "threads_used", "fps", "mpix_s", "census_ms", "cost_ms",
                     "aggregate_ms", "argmin_ms", "hash", "golden_match", "roofline_ok", "cflags", "git", "ts"}


@pytest.mark.gpu
def test_cli_plain_harness_line_and_record(tmp_path):
    """`plain` prints the reference harness's result line (common/harness.c:
    197-201) and appends its JSON record (:207-224) with the same fields."""
    l, r, _ = sgmgb.synth_pair(320, 200, 64, 4)
    write_pgm(str(tmp_path / "l.pgm"), l)
    write_pgm(str(tmp_path / "r.pgm"), r)
    want = oracle.plain(l, r, 64, 4)
    write_pgm(str(tmp_path / "g.pgm"), want)
    p = run("plain", tmp_path / "l.pgm", tmp_path / "r.pgm", "-g", tmp_path / "g.pgm", "-w", 2, "-n", 9, "-t", 4,
            "-j", tmp_path / "res.jsonl", "--no-roofline")
    assert p.returncode == 0, p.stdout + p.stderr
    m = HARNESS_LINE.match(p.stdout.splitlines()[0])
    assert m, p.stdout
    assert m.group(1, 2, 3, 4, 5) == ("320", "200", "64", "4", "0")
    med, p95, mn = float(m.group(6)), float(m.group(7)), float(m.group(8))
    assert mn <= med <= p95
    assert m.group(15) == oracle.fnv1a64(want) and m.group(16) == "  GOLDEN OK"
    rec = json.loads(open(tmp_path / "res.jsonl").read().splitlines()[-1])
    assert set(rec) == HARNESS_JSON_KEYS
    assert rec["timed"] == 9 and rec["warm"] == 2 and rec["threads_requested"] == 4 and rec["threads_used"] == 0
    assert rec["golden_match"] == 1 and rec["roofline_ok"] == -1 and rec["hash"] == oracle.fnv1a64(want)
    assert rec["aggregate_ms"] >= 0 and rec["cost_ms"] == -1 and rec["argmin_ms"] == -1


@pytest.mark.gpu
def test_cli_plain_cost_gate(tmp_path):
    """The per-phase cost gate of common/roofline.h: --roofline-calibrate
    writes gb300 rows; the next run arms against them and passes; a planted
    calibration 100x cheaper than the engine fails the run with exit 3 while
    the map stays golden."""
    l, r, _ = sgmgb.synth_pair(320, 200, 64, 6)
    write_pgm(str(tmp_path / "l.pgm"), l)
    write_pgm(str(tmp_path / "r.pgm"), r)
    cal = tmp_path / "roofline.cal"
    p = run("plain", tmp_path / "l.pgm", tmp_path / "r.pgm", "-n", 5, "--board", "testbox", "--roofline-calibrate",
            "--roofline-cal", cal)
    assert p.returncode == 0, p.stderr
    rows = [x.split() for x in open(cal).read().splitlines()]
    assert {x[4] for x in rows} == {"aggregate"}          # the frame is one graph: the other phases are -1
    assert all(x[:4] == ["gb300", "testbox", "320x200", "D64"] and float(x[5]) > 0 for x in rows)
    p = run("plain", tmp_path / "l.pgm", tmp_path / "r.pgm", "-n", 5, "--board", "testbox", "--roofline-cal", cal,
            "--roofline-max", 5, "-j", tmp_path / "a.jsonl")
    assert p.returncode == 0, p.stdout + p.stderr
    assert "roofline:" in p.stdout and "NOT ARMED" not in p.stderr
    assert json.loads(open(tmp_path / "a.jsonl").read())["roofline_ok"] == 1
    planted = tmp_path / "planted.cal"
    planted.write_text("".join("%s %s %s %s %s %.9f\n" % (*x[:5], float(x[5]) / 100) for x in rows))
    p = run("plain", tmp_path / "l.pgm", tmp_path / "r.pgm", "-n", 3, "--board", "testbox", "--roofline-cal", planted)
    assert p.returncode == 3 and "ROOFLINE FAIL" in p.stderr
    p = run("plain", tmp_path / "l.pgm", tmp_path / "r.pgm", "-n", 3, "--board", "other", "--roofline-cal", cal)
    assert p.returncode == 0 and "NOT ARMED" in p.stderr              # no row for this board: says so


@pytest.mark.gpu
def test_cli_plain_default_calibration_arms_on_the_reference_scene(tmp_path):
    """The gb300 calibration rows shipped beside the package (recorded with
    --roofline-calibrate on the reference's calibration scene, gen_synthetic
    1920x1080 seed 1, as its Makefile's roofline-cal target does) arm the gate
    on that scene; the map is the committed golden (FNV 0bc0102058d1505f)."""
    l, r, _ = oracle.gen_reference(1920, 1080, 64, 1)
    write_pgm(str(tmp_path / "l.pgm"), l)
    write_pgm(str(tmp_path / "r.pgm"), r)
    p = run("plain", tmp_path / "l.pgm", tmp_path / "r.pgm", "-w", 2, "-n", 9, "--roofline-max", 2.0,
            "-j", tmp_path / "res.jsonl")
    assert p.returncode == 0, p.stdout + p.stderr
    assert "NOT ARMED" not in p.stderr and "roofline:" in p.stdout
    assert HARNESS_LINE.match(p.stdout.splitlines()[0]).group(15) == "0bc0102058d1505f"
    assert json.loads(open(tmp_path / "res.jsonl").read())["roofline_ok"] == 1
