import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (os.path.join(ROOT, "sgm-bench_gb300"), os.path.join(ROOT, "oracle")):
    if p not in sys.path:
        sys.path.insert(0, p)

GOLDEN_DIR = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (run with -m gpu on the GPU box)")


@pytest.fixture(scope="session")
def engine():
    import sgmgb
    eng = sgmgb.Engine(0)
    yield eng
    eng.close()


@pytest.fixture(scope="session")
def ref_fixtures():
    import json
    with open(os.path.join(GOLDEN_DIR, "reference_scenes.json")) as f:
        return json.load(f)


def reference_plain(left, right, D, paths):
    """The checker's map of a plain frame: the reference's own common/sgm_ref.c
    (built from its sources into oracle/_ref, compile-time D and paths) where it
    is built for this D and path count, else the oracle restating it."""
    import oracle
    if oracle.reference_available(D, paths):
        return oracle.ReferenceImpl(D, paths).run(left, right)
    return oracle.plain(left, right, D, paths)


def reference_multiscale_hash(left, right):
    """The checker's FNV-1a-64 of a multi-scale frame's map: the reference's own
    multiscale/sgm_ms_ref.c (built into oracle/_ref, on all host threads) where
    it is built, else the oracle restating it."""
    import oracle
    try:
        return oracle.reference_multiscale(left, right, reps=1)[1]
    except FileNotFoundError:
        return oracle.fnv1a64(oracle.multiscale(left, right))


# Frames at the sizes of the batched and served configurations: 1920x1080 D=128
# 8-path, 1920x800 D=64 8-path and 1280x720 D=128 4-path.
BASELINE_FRAMES = [(1920, 1080, 128, 8), (1920, 800, 64, 8), (1280, 720, 128, 4)]


@pytest.fixture(scope="session")
def baseline_frames():
    """{(W, H, D, paths): (left, right, checker map)} for BASELINE_FRAMES, the
    checker's maps computed side by side on host threads (the checkers run in
    C with the interpreter lock released)."""
    import concurrent.futures as cf
    import sgmgb
    pairs = {k: sgmgb.synth_pair(k[0], k[1], k[2], seed=k[0] + k[2] + k[3])[:2] for k in BASELINE_FRAMES}
    with cf.ThreadPoolExecutor(max_workers=len(pairs)) as pool:
        futs = {k: pool.submit(reference_plain, l, r, k[2], k[3]) for k, (l, r) in pairs.items()}
        return {k: (pairs[k][0], pairs[k][1], futs[k].result()) for k in pairs}
