"""Cross-check of the oracle against the reference's own CPU binaries, built
from the reference's sources by oracle/build_ref.sh into oracle/_ref/
(skipped where they are not built, e.g. on a machine without the reference
checkout)."""
import os
import subprocess

import numpy as np
import pytest

import oracle

REF = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "oracle", "_ref")
pytestmark = pytest.mark.skipif(not os.path.exists(os.path.join(REF, "sgm_ms_ref")),
                                reason="reference binaries not built (oracle/build_ref.sh)")


def write_pgm(path, a):
    with open(path, "wb") as f:
        f.write(b"P5\n%d %d\n255\n" % (a.shape[1], a.shape[0]))
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


@pytest.mark.parametrize("W,H,D,seed", [(320, 200, 64, 5), (257, 91, 128, 2), (160, 120, 256, 9)])
def test_generator_matches_reference_binary(tmp_path, W, H, D, seed):
    subprocess.run([os.path.join(REF, "gen_synthetic_d%d" % D), str(W), str(H), str(tmp_path), str(seed)],
                   check=True, capture_output=True)
    l, r, g = oracle.gen_reference(W, H, D, seed)
    assert np.array_equal(read_pgm(str(tmp_path / "left.pgm")), l)
    assert np.array_equal(read_pgm(str(tmp_path / "right.pgm")), r)
    assert np.array_equal(read_pgm(str(tmp_path / "gt.pgm")), g)


@pytest.mark.parametrize("W,H,D,paths", [(97, 45, 64, 4), (97, 45, 64, 8), (130, 66, 128, 4), (64, 33, 256, 8),
                                         (1, 1, 64, 4), (23, 1, 64, 8)])
def test_plain_matches_reference_binary(tmp_path, W, H, D, paths):
    rng = np.random.default_rng(W * H + D)
    l = rng.integers(0, 256, (H, W), dtype=np.uint8)
    r = rng.integers(0, 256, (H, W), dtype=np.uint8)
    write_pgm(str(tmp_path / "l.pgm"), l)
    write_pgm(str(tmp_path / "r.pgm"), r)
    subprocess.run([os.path.join(REF, "sgm_ref_d%d_p%d" % (D, paths)), str(tmp_path / "l.pgm"),
                    str(tmp_path / "r.pgm"), "-w", "0", "-n", "1", "-o", str(tmp_path / "o.pgm")],
                   check=True, capture_output=True)
    assert np.array_equal(read_pgm(str(tmp_path / "o.pgm")), oracle.plain(l, r, D, paths))


@pytest.mark.parametrize("W,H", [(130, 66), (2, 2), (64, 48)])
def test_multiscale_matches_reference_binary(tmp_path, W, H):
    rng = np.random.default_rng(W + 7 * H)
    l = rng.integers(0, 256, (H, W), dtype=np.uint8)
    r = rng.integers(0, 256, (H, W), dtype=np.uint8)
    write_pgm(str(tmp_path / "l.pgm"), l)
    write_pgm(str(tmp_path / "r.pgm"), r)
    subprocess.run([os.path.join(REF, "sgm_ms_ref"), str(tmp_path / "l.pgm"), str(tmp_path / "r.pgm"), "-n", "1",
                    "-o", str(tmp_path / "o.pgm")], check=True, capture_output=True,
                   env=dict(os.environ, OMP_NUM_THREADS="2"))
    assert np.array_equal(read_pgm(str(tmp_path / "o.pgm")), oracle.multiscale(l, r))


def test_reference_harness_links_the_plugin(tmp_path):
    """The reference's own harness.c, linked against the gb300 SGM_IMPL: on a
    machine without a GPU it must fail the frame cleanly (exit 1, "impl
    failed"), on a GPU it must pass the golden-style comparison."""
    exe = os.path.join(REF, "sgm_gb300_harness_d64_p4")
    if not os.path.exists(exe):
        pytest.skip("plugin harness not linked")
    rng = np.random.default_rng(4)
    l = rng.integers(0, 256, (48, 64), dtype=np.uint8)
    r = rng.integers(0, 256, (48, 64), dtype=np.uint8)
    write_pgm(str(tmp_path / "l.pgm"), l)
    write_pgm(str(tmp_path / "r.pgm"), r)
    want = oracle.plain(l, r, 64, 4)
    write_pgm(str(tmp_path / "g.pgm"), want)
    p = subprocess.run([exe, str(tmp_path / "l.pgm"), str(tmp_path / "r.pgm"), "-g", str(tmp_path / "g.pgm"),
                        "-w", "0", "-n", "1"], capture_output=True, text=True)
    try:
        import torch
        gpu = torch.cuda.is_available()
    except Exception:
        gpu = False
    if gpu:
        assert p.returncode == 0, p.stdout + p.stderr
    else:
        assert p.returncode == 1 and "impl failed" in (p.stdout + p.stderr)
