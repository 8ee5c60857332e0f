"""The served form: frames from several cameras admitted as they arrive.

Each result must be byte-identical alone and in the mix, and equal to the
oracle (common/sgm_ref.c, multiscale/sgm_ms_ref.c restated in oracle/)."""
import numpy as np
import pytest

import oracle
import sgmgb

pytestmark = pytest.mark.gpu

CAMS = {0: (160, 96, 64, 4, sgmgb.PLAIN), 1: (200, 120, 128, 4, sgmgb.PLAIN),
        2: (128, 64, 64, 8, sgmgb.PLAIN), 3: (130, 66, 64, 8, sgmgb.MULTISCALE)}


def _want(cam, l, r):
    W, H, D, paths, variant = CAMS[cam]
    return oracle.multiscale(l, r) if variant else oracle.plain(l, r, D, paths)


def _frames(n_per_cam=3):
    out = []
    for k in range(n_per_cam):
        for cam, (W, H, D, paths, variant) in CAMS.items():
            l, r, _ = sgmgb.synth_pair(W, H, min(D, 128), seed=100 + 10 * cam + k)
            out.append((cam, l, r))
    return out


def _server(engine, **kw):
    s = sgmgb.Server(engine, **kw)
    for cam, (W, H, D, paths, variant) in CAMS.items():
        s.add_camera(cam, W, H, D, paths, variant)
    return s


def test_server_alone_equals_mix_equals_oracle(engine):
    frames = _frames()
    s = _server(engine)
    alone = []
    for cam, l, r in frames:                       # one frame on the device at a time
        out, lat = s.wait(s.submit(cam, l, r))
        assert lat > 0
        alone.append(out)
    tickets = [s.submit(cam, l, r) for cam, l, r in frames]   # all at once: they overlap
    mixed = [s.wait(t)[0] for t in tickets]
    for (cam, l, r), a, m in zip(frames, alone, mixed):
        assert np.array_equal(a, m), "camera %d: result differs in the mix" % cam
        assert np.array_equal(a, _want(cam, l, r)), "camera %d: differs from the oracle" % cam
    st = s.stats()
    assert st["frames_done"] == 2 * len(frames) and st["frames_refused"] == 0
    assert 0 < st["p50_ms"] <= st["p99_ms"] <= st["max_ms"]
    assert st["resident_bytes"] <= 40 << 30
    s.close()


def test_server_poll_and_interleaved_collection(engine):
    frames = _frames(2)
    s = _server(engine, max_inflight=2)
    pending = {s.submit(cam, l, r): (cam, l, r) for cam, l, r in frames}
    got = {}
    import time
    deadline = time.time() + 30
    while pending and time.time() < deadline:
        for t in list(pending):
            done, out, lat = s.poll(t)
            if done:
                got[t] = (pending.pop(t), out)
    assert not pending
    for (cam, l, r), out in got.values():
        assert np.array_equal(out, _want(cam, l, r))
    s.close()


def test_server_budget_admission(engine):
    one = sgmgb.workspace_bytes(160, 96, 64, 4)
    s = sgmgb.Server(engine, hbm_budget_bytes=one + one // 2, max_inflight=4)
    s.add_camera(0, 160, 96, 64, 4)
    with pytest.raises(sgmgb.SgmError) as ei:
        s.add_camera(1, 160, 96, 64, 4)            # a second slot would exceed the budget
    assert ei.value.code == sgmgb.ERR_BUDGET
    # frames beyond the one resident slot queue and run in turn, all exact
    l, r, _ = sgmgb.synth_pair(160, 96, 64, seed=7)
    want = oracle.plain(l, r, 64, 4)
    tickets = [s.submit(0, l, r) for _ in range(6)]
    for t in tickets:
        assert np.array_equal(s.wait(t)[0], want)
    assert s.stats()["resident_bytes"] <= one + one // 2
    s.close()


def test_server_refuses_when_request_buffers_run_out(engine):
    s = sgmgb.Server(engine, max_inflight=1)
    s.add_camera(5, 64, 48, 64, 4)
    l, r, _ = sgmgb.synth_pair(64, 48, 64, seed=9)
    tickets = [s.submit(5, l, r) for _ in range(16)]   # 16 request buffers per camera
    with pytest.raises(sgmgb.SgmError) as ei:
        s.submit(5, l, r)
    assert ei.value.code == sgmgb.ERR_BUDGET
    assert s.stats()["frames_refused"] == 1
    for t in tickets:
        s.wait(t)
    s.wait(s.submit(5, l, r))                      # buffers are free again once collected
    with pytest.raises(sgmgb.SgmError):
        s.submit(99, l, r)                         # unknown camera
    s.close()


def test_server_prepare_makes_slots_up_front_within_budget(engine):
    """sgmgb_server_prepare makes each camera's slots before any frame (up to
    4 per camera, one camera at a time while the budget allows), and frames
    submitted afterwards allocate nothing more: the resident bytes stay put."""
    one = sgmgb.workspace_bytes(160, 96, 64, 4)
    s = sgmgb.Server(engine, hbm_budget_bytes=5 * one, max_inflight=8)
    s.add_camera(0, 160, 96, 64, 4)
    s.add_camera(1, 160, 96, 64, 4)
    assert s.stats()["resident_bytes"] == 2 * one
    assert s.prepare(4) == 5                       # 2 + 3 more before the budget stops it, shared in turn
    assert s.stats()["resident_bytes"] == 5 * one
    assert s.prepare(4) == 5                       # nothing left to make
    frames = [(cam, *sgmgb.synth_pair(160, 96, 64, seed=20 + k)[:2]) for k in range(6) for cam in (0, 1)]
    tickets = [s.submit(cam, l, r) for cam, l, r in frames]
    for (cam, l, r), t in zip(frames, tickets):
        assert np.array_equal(s.wait(t)[0], oracle.plain(l, r, 64, 4))
    assert s.stats()["resident_bytes"] == 5 * one
    with pytest.raises(sgmgb.SgmError):
        s.prepare(0)
    s.close()
