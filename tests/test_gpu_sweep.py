"""The disparity-range x resolution grid of the reference's sweep
(scripts/sweep.sh:20-56): D in {32, 64, 128} x {1920x1080, 1280x720, 960x540,
640x480}, 4 paths, each cell on the reference generator's scene for that D
(common/gen_synthetic.c, seed 1, restated in the oracle) with its own golden
from the oracle. As in the reference, a golden gates a cell only if it
discriminates (scripts/check_golden_discriminates.py:59-119): it reaches
d = D-1, has at least 8 distinct values, and at least 0.5 % of its pixels are
in the top decile, so an engine that searched fewer disparities would fail
it. D = 256 runs on the shared scene in test_gpu_parity.test_reference_goldens."""
import numpy as np
import pytest

import oracle
import sgmgb

pytestmark = pytest.mark.gpu

RESOLUTIONS = [(1920, 1080), (1280, 720), (960, 540), (640, 480)]


def discriminates(golden, D):
    top = int(golden.max())
    distinct = len(np.unique(golden))
    cover = 100.0 * np.count_nonzero(golden >= int(D * 0.9)) / golden.size
    return top >= D - 1 and distinct >= 8 and cover >= 0.5, (top, distinct, cover)


@pytest.mark.parametrize("D", [32, 64, 128])
@pytest.mark.parametrize("W,H", RESOLUTIONS)
def test_d_sweep_cell(engine, D, W, H):
    left, right, _ = oracle.gen_reference(W, H, D, 1)
    golden = oracle.plain(left, right, D, 4)
    ok, why = discriminates(golden, D)
    assert ok, "golden for D=%d %dx%d does not discriminate: max %d, %d distinct, %.3f %% top decile" % (
        (D, W, H) + why)
    engine.plan(W, H, D, 4)
    got = engine.run_frame(left, right)
    assert np.array_equal(got, golden), "D=%d %dx%d: %d pixels differ" % (D, W, H, int((got != golden).sum()))
    assert oracle.fnv1a64(got) == oracle.fnv1a64(golden)
