"""The optional post-steps: left-right check, 3x3 median, 16x subpixel map.

The reference has none (common/sgm_params.h:58); the definitions are the
oracle's post mode (oracle/sgm_oracle.c, sgmo_post). On the CPU the oracle is
checked against an independent numpy restatement of those definitions; on the
GPU the engine's maps must equal the oracle's byte for byte."""
import numpy as np
import pytest

import oracle
import sgmgb


def _numpy_post(left, right, D, paths, flags):
    """The post-step definitions restated with numpy on the oracle's summed volume."""
    dL, S = oracle.plain(left, right, D, paths, with_sum=True)
    H, W = dL.shape
    S = S.astype(np.int64)
    d = dL.astype(np.int64)
    yy, xx = np.mgrid[0:H, 0:W]
    # subpixel
    inner = (d > 0) & (d < D - 1)
    c0 = S[yy, xx, np.clip(d - 1, 0, D - 1)]
    c1 = S[yy, xx, d]
    c2 = S[yy, xx, np.clip(d + 1, 0, D - 1)]
    den = c0 + c2 - 2 * c1
    num = 16 * (c0 - c2)
    q = np.where(den > 0, np.trunc(num / np.where(den > 0, 2 * den, 1)).astype(np.int64), 0)
    v16 = 16 * d + np.where(inner, q, 0)
    out = d.copy()
    if flags & oracle.POST_LR:
        dR = np.zeros((H, W), np.int64)
        for x in range(W):
            ds = np.arange(min(D, W - x))
            vals = S[:, x + ds, ds]                       # (H, len(ds))
            dR[:, x] = np.argmin(vals, axis=1)            # first minimum: lowest d on ties
        xr = xx - d
        ok = xr >= 0
        bad = ~ok.copy()
        bad[ok] = np.abs(d[ok] - dR[yy[ok], xr[ok]]) > 1
        out[bad] = 255
        v16[bad] = 0xFFFF
    out = out.astype(np.uint8)
    if flags & oracle.POST_MEDIAN:
        p = np.pad(out, 1, mode="edge")
        stack = np.stack([p[dy:dy + H, dx:dx + W] for dy in range(3) for dx in range(3)])
        out = np.sort(stack, axis=0)[4].astype(np.uint8)
    return out, (v16.astype(np.uint16) if flags & oracle.POST_SUBPIXEL else None)


@pytest.mark.parametrize("flags", [0, 1, 2, 3, 4, 5, 6, 7])
@pytest.mark.parametrize("W,H,D,paths", [(64, 24, 32, 4), (97, 33, 64, 8), (40, 17, 16, 4)])
def test_oracle_post_matches_numpy_restatement(W, H, D, paths, flags):
    left, right, _ = oracle.synth_pair(W, H, D, seed=W + D + flags)
    got, g16 = oracle.post(left, right, D, paths, flags)
    want, w16 = _numpy_post(left, right, D, paths, flags)
    assert np.array_equal(got, want)
    if flags & oracle.POST_SUBPIXEL:
        assert np.array_equal(g16, w16)
    if flags == 0:
        assert np.array_equal(got, oracle.plain(left, right, D, paths))


def test_oracle_post_rejects():
    left, right, _ = oracle.synth_pair(32, 8, 16, seed=1)
    with pytest.raises(ValueError):
        oracle.post(left, right, 256, 4, oracle.POST_LR)          # 255 is a disparity at D = 256
    with pytest.raises(ValueError):
        oracle.post(left, right, 64, 4, 8)                         # unknown flag


@pytest.mark.gpu
@pytest.mark.parametrize("W,H,D,paths", [(320, 200, 64, 4), (257, 91, 128, 8), (160, 90, 32, 4), (1, 5, 16, 4),
                                         (1920, 1080, 64, 4)])
def test_post_steps_equal_the_oracle(engine, W, H, D, paths):
    left, right, _ = sgmgb.synth_pair(W, H, min(D, 128), seed=W + H)
    engine.plan(W, H, D, paths)
    for flags in ([0, 1, 2, 3, 4, 5, 6, 7] if W * H < 10 ** 6 else [7]):
        got, g16 = engine.run_frame_post(left, right, flags)
        want, w16 = oracle.post(left, right, D, paths, flags)
        assert np.array_equal(got, want), ("flags", flags, int((got != want).sum()))
        if flags & sgmgb.POST_SUBPIXEL:
            assert np.array_equal(g16, w16), ("subpixel flags", flags)
    # flags 0 is the plain map, as the drop-in call gives it
    assert np.array_equal(engine.run_frame_post(left, right, 0)[0], engine.run_frame(left, right))


@pytest.mark.gpu
def test_post_steps_reject(engine):
    left, right, _ = sgmgb.synth_pair(64, 32, 64, seed=3)
    engine.plan(64, 32, 256, 4)
    with pytest.raises(sgmgb.SgmError):
        engine.run_frame_post(left, right, sgmgb.POST_LR)
    engine.plan(64, 32, 64, 4)
    with pytest.raises(sgmgb.SgmError):
        engine.run_frame_post(left, right, 8)
    assert sgmgb.lib.sgmgb_run_frame_post(engine.h, left.ctypes.data, right.ctypes.data,
                                          np.empty_like(left).ctypes.data, None,
                                          sgmgb.POST_SUBPIXEL) == sgmgb.ERR_ARG   # no subpixel buffer
    engine.plan(64, 32, 64, 8, sgmgb.MULTISCALE)
    with pytest.raises(sgmgb.SgmError):
        engine.run_frame_post(left, right, 0)
