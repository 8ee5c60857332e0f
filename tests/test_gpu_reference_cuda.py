"""The reference's own CUDA programs (cuda/sgm_cuda_opt.cu in the reference's
harness, multiscale/sgm_ms_cuda.cu), built for sm_103a from its sources by
oracle/build_ref.sh, give the same maps as this engine and the oracle on the
same pairs: a third, independent implementation in the parity chain, and the
programs the benchmark's reference arm times on the GPU. Skipped where they
are not built (no reference sources, or no nvcc)."""
import numpy as np
import pytest

import oracle
import sgmgb

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("W,H,D", [(640, 480, 64), (333, 97, 64), (640, 480, 128), (1920, 1080, 64)])
def test_reference_cuda_opt_equals_the_engine(engine, W, H, D):
    if not oracle.reference_cuda_available("sgm_cuda_opt_d%d" % D):
        pytest.skip("reference CUDA program not built (oracle/build_ref.sh)")
    left, right, _ = sgmgb.synth_pair(W, H, D, seed=W + H + D)
    _, ref = oracle.reference_cuda_plain(left, right, D, warm=0, timed=1)
    engine.plan(W, H, D, 4)
    got = engine.run_frame(left, right)
    assert np.array_equal(got, ref), int((got != ref).sum())
    if W * H <= 640 * 480:
        assert np.array_equal(ref, oracle.plain(left, right, D, 4))


@pytest.mark.parametrize("W,H", [(640, 480), (1920, 800)])
def test_reference_ms_cuda_equals_the_engine(engine, W, H):
    if not oracle.reference_cuda_available("sgm_ms_cuda"):
        pytest.skip("reference multi-scale CUDA program not built (oracle/build_ref.sh)")
    left, right, _ = sgmgb.synth_pair(W, H, 64, seed=W + 5)
    _, h, ref = oracle.reference_cuda_multiscale(left, right, reps=1)
    engine.plan(W, H, 64, 8, sgmgb.MULTISCALE)
    got = engine.run_frame(left, right)
    assert got.shape == ref.shape == (H // 2, W // 2)
    assert np.array_equal(got, ref), int((got != ref).sum())
    assert h == oracle.fnv1a64(got)
    if W * H <= 640 * 480:
        assert np.array_equal(ref, oracle.multiscale(left, right))
