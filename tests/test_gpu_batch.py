"""The batched form: many frames of mixed shapes in one persistent launch, or
as frames in flight in one CUDA graph.

Every frame of a batch must equal the oracle (common/sgm_ref.c restated in
oracle/sgm_oracle.c) byte for byte, on the first run and on graph replays with
other buffers; the bounded device-side waits must turn a stalled dependency
into SGMGB_ERR_TIMEOUT with the context still usable."""
import numpy as np
import pytest

import oracle
import sgmgb

pytestmark = pytest.mark.gpu


def _frames(specs, seed0=0):
    """specs: (W, H, D, paths). Returns descs, host pairs, device pairs, device outputs."""
    import torch
    descs, host, dev, outs = [], [], [], []
    for k, (W, H, D, paths) in enumerate(specs):
        l, r, _ = sgmgb.synth_pair(W, H, min(D, 128), seed=seed0 + k + 1)
        descs.append(sgmgb.desc(W, H, D, paths))
        host.append((l, r))
        dev.append((torch.from_numpy(l).cuda(), torch.from_numpy(r).cuda()))
        outs.append(torch.zeros((H, W), dtype=torch.uint8, device="cuda"))
    return descs, host, dev, outs


def _check(host, outs, descs, tag=""):
    for k, ((l, r), o, d) in enumerate(zip(host, outs, descs)):
        got = o.cpu().numpy()
        want = oracle.plain(l, r, d.D, d.paths)
        if not np.array_equal(got, want):
            idx = np.argwhere(got != want)
            y, x = idx[0]
            pytest.fail("%sframe %d (%dx%d D=%d paths=%d): %d pixels differ, first (x=%d,y=%d) got %d want %d"
                        % (tag, k, d.W, d.H, d.D, d.paths, len(idx), x, y, got[y, x], want[y, x]))


MIX = [(160, 96, 64, 4), (97, 45, 64, 8), (320, 200, 128, 4), (61, 40, 16, 4), (200, 33, 128, 8),
       (1, 1, 64, 4), (23, 1, 16, 8), (1, 23, 64, 4), (300, 70, 48, 8), (640, 480, 64, 4)]


def test_batch_mixed_frames_exact(engine):
    import torch
    descs, host, dev, outs = _frames(MIX)
    b = sgmgb.Batch(engine, descs)
    b.run([d[0] for d in dev], [d[1] for d in dev], outs)
    b.wait()
    torch.cuda.synchronize()
    _check(host, outs, descs, "first run: ")
    # graph replay on other buffers: the same frames with left/right swapped roles of two pairs
    for o in outs:
        o.zero_()
    b.run([d[0] for d in dev], [d[1] for d in dev], outs)
    b.wait()
    _check(host, outs, descs, "replay: ")
    b.close()


def test_batch_new_buffers_each_run(engine):
    import torch
    specs = [(128, 64, 64, 4), (96, 80, 64, 8), (64, 48, 128, 4)]
    descs, host1, dev1, outs1 = _frames(specs, seed0=10)
    _, host2, dev2, outs2 = _frames(specs, seed0=20)
    b = sgmgb.Batch(engine, descs)
    for host, dev, outs in ((host1, dev1, outs1), (host2, dev2, outs2), (host1, dev1, outs2)):
        for o in outs:
            o.zero_()
        b.run([d[0] for d in dev], [d[1] for d in dev], outs)
        b.wait()
        torch.cuda.synchronize()
        _check(host, outs, descs)
    b.close()


def test_batch_in_flight_mode_exact(engine):
    """SGMGB_BATCH_IN_FLIGHT: every frame's own pipeline on concurrent chains,
    one CUDA graph; maps equal the oracle's, on a replay and after new output
    buffers (a new capture), and the persistent mode runs after it."""
    import torch
    descs, host, dev, outs = _frames(MIX, seed0=60)
    b = sgmgb.Batch(engine, descs)
    assert b.mode() == (sgmgb.BATCH_PERSISTENT, 0)
    with pytest.raises(sgmgb.SgmError):
        b.busy()                                   # no persistent launch yet
    b.set_mode(sgmgb.BATCH_IN_FLIGHT, 3)
    assert b.mode() == (sgmgb.BATCH_IN_FLIGHT, 3)
    L, R = [d[0] for d in dev], [d[1] for d in dev]
    for tag in ("first run: ", "replay: "):
        for o in outs:
            o.zero_()
        b.run(L, R, outs)
        b.wait()
        torch.cuda.synchronize()
        _check(host, outs, descs, tag)
    outs2 = [torch.zeros_like(o) for o in outs]
    b.run(L, R, outs2)
    b.wait()
    torch.cuda.synchronize()
    _check(host, outs2, descs, "new buffers: ")
    b.set_mode(sgmgb.BATCH_PERSISTENT)
    for o in outs:
        o.zero_()
    b.run(L, R, outs)
    b.wait()
    torch.cuda.synchronize()
    _check(host, outs, descs, "persistent after in flight: ")
    assert b.busy()["blocks"] > 0
    b.close()


def test_batch_autotune_and_cache(engine, tmp_path):
    import torch
    specs = [(320, 240, 64, 4), (256, 128, 128, 8), (320, 240, 64, 4)]
    descs, host, dev, outs = _frames(specs, seed0=30)
    cache = str(tmp_path / "tune.txt")
    b = sgmgb.Batch(engine, descs)
    L, R = [d[0] for d in dev], [d[1] for d in dev]
    b.autotune(L, R, outs, cache)
    shapes = [b.tile_shape(i) for i in range(len(specs))]
    for w, d in shapes:
        assert w in (2, 4) and d in (0, 2, 4, 8)
    mode, lanes = b.mode()
    assert (mode, lanes) == (sgmgb.BATCH_PERSISTENT, 0) or (mode == sgmgb.BATCH_IN_FLIGHT and lanes in (4, 6, 8))
    for o in outs:
        o.zero_()
    b.run(L, R, outs)
    b.wait()
    torch.cuda.synchronize()
    _check(host, outs, descs)
    b.close()
    lines = [l.split() for l in open(cache) if l.strip()]
    assert len(lines) == 2                       # one line per distinct description
    # a new batch planned from the cache takes the recorded shapes
    b2 = sgmgb.Batch(engine, descs, tune_cache=cache)
    assert [b2.tile_shape(i) for i in range(len(specs))] == shapes
    b2.close()


def test_batch_wait_limit_reports_timeout(engine):
    """A frame whose census target can never be met: its cost items' waits run
    out, the run is abandoned with SGMGB_ERR_TIMEOUT, and the batch (and the
    context) run correctly afterwards."""
    import torch
    specs = [(128, 64, 64, 4), (96, 80, 64, 8), (64, 48, 64, 4)]
    descs, host, dev, outs = _frames(specs, seed0=40)
    b = sgmgb.Batch(engine, descs)
    L, R = [d[0] for d in dev], [d[1] for d in dev]
    b.set_fault(wait_limit_ms=200, stall_frame=1)
    b.run(L, R, outs)
    with pytest.raises(sgmgb.SgmError) as ei:
        b.wait()
    assert ei.value.code == sgmgb.ERR_TIMEOUT
    b.set_fault(wait_limit_ms=2000, stall_frame=-1)
    b.run(L, R, outs)
    b.wait()
    torch.cuda.synchronize()
    _check(host, outs, descs)
    b.close()


def test_batch_rejects_bad_input(engine):
    with pytest.raises(sgmgb.SgmError):
        sgmgb.Batch(engine, [sgmgb.desc(64, 48, 64, 8, sgmgb.MULTISCALE)])
    with pytest.raises(sgmgb.SgmError):
        sgmgb.Batch(engine, [sgmgb.desc(64, 48, 65, 4)])
    b = sgmgb.Batch(engine, [sgmgb.desc(16, 16, 64, 4)])
    with pytest.raises(sgmgb.SgmError):
        b.run([0], [0], [0])
    for mode, lanes in ((2, 4), (-1, 4), (sgmgb.BATCH_IN_FLIGHT, 0), (sgmgb.BATCH_IN_FLIGHT, 9)):
        with pytest.raises(sgmgb.SgmError):
            b.set_mode(mode, lanes)
    assert b.mode() == (sgmgb.BATCH_PERSISTENT, 0)
    b.close()


def test_batch_baseline_sizes(engine, baseline_frames):
    """One persistent launch over frames at the batched configuration's sizes
    (1920x1080 D=128 8-path, 1920x800 D=64 8-path, 1280x720 D=128 4-path),
    every map byte for byte against the checker, on two runs, then a run of
    the frames-in-flight mode."""
    import torch
    keys = list(baseline_frames)
    descs = [sgmgb.desc(*k) for k in keys]
    dl = [torch.from_numpy(baseline_frames[k][0]).cuda() for k in keys]
    dr = [torch.from_numpy(baseline_frames[k][1]).cuda() for k in keys]
    outs = [torch.zeros((k[1], k[0]), dtype=torch.uint8, device="cuda") for k in keys]
    b = sgmgb.Batch(engine, descs)
    try:
        for run in range(3):
            if run == 2:                          # the frames-in-flight mode on the same frames
                b.set_mode(sgmgb.BATCH_IN_FLIGHT, 2)
            for o in outs:
                o.zero_()
            b.run(dl, dr, outs)
            b.wait()
            torch.cuda.synchronize()
            for k, o in zip(keys, outs):
                got, want = o.cpu().numpy(), baseline_frames[k][2]
                if not np.array_equal(got, want):
                    y, x = np.argwhere(got != want)[0]
                    pytest.fail("run %d %r: %d pixels differ, first (x=%d,y=%d) got %d want %d"
                                % (run, k, int((got != want).sum()), x, y, got[y, x], want[y, x]))
    finally:
        b.close()


def test_batch_busy_accounts_for_the_run(engine):
    """sgmgb_batch_busy: the blocks' time by item kind. A batch with a fused
    frame (4 paths, D = 64) and an 8-path frame has census, first-half, cost,
    scratch and final work; the kinds' sum per block cannot exceed the run's
    time on the device (blocks that find the queue empty leave at once)."""
    import torch
    specs = [(320, 240, 64, 4), (200, 120, 64, 8)]
    descs, host, dev, outs = _frames(specs, seed0=50)
    b = sgmgb.Batch(engine, descs)
    L, R = [d[0] for d in dev], [d[1] for d in dev]
    b.run(L, R, outs)
    b.wait()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    s = torch.cuda.current_stream()
    e0.record(s)
    b.run(L, R, outs, stream=s)                    # on the stream the events are recorded on
    e1.record(s)
    b.wait()
    torch.cuda.synchronize()
    _check(host, outs, descs)
    busy = b.busy()
    for k in ("census", "cost", "scratch", "final", "first_half_cost"):
        assert busy[k] > 0, (k, busy)
    assert busy["wait"] >= 0 and busy["blocks"] > 0
    per_block = sum(busy[k] for k in sgmgb.Batch.BUSY_KINDS) / busy["blocks"]
    assert 0 < per_block < 1.5 * e0.elapsed_time(e1), (per_block, e0.elapsed_time(e1))
    b.close()
