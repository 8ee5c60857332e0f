"""Bit-exact parity of the CUDA engine with the oracle (common/sgm_ref.c,
multiscale/sgm_ms_ref.c restated in oracle/sgm_oracle.c), through the C ABI.

Integer work: every comparison is byte-for-byte (tolerance 0)."""
import numpy as np
import pytest

import oracle
import sgmgb

pytestmark = pytest.mark.gpu


def _rand(H, W, seed):
    return np.random.default_rng(seed).integers(0, 256, size=(H, W), dtype=np.uint8)


def _first_diff(got, want):
    idx = np.argwhere(got != want)
    if not len(idx):
        return ""
    y, x = idx[0][:2]
    return " first diff at (x=%d,y=%d): got %d want %d; %d differ" % (x, y, got[y, x], want[y, x], len(idx))


# ---- census descriptors (test pattern of common/test_phase1.c:17-62) ----
@pytest.mark.parametrize("W,H", [(1, 1), (5, 3), (9, 7), (33, 10), (640, 480), (1001, 37)])
def test_census_descriptors(engine, W, H):
    import torch
    for img in (_rand(H, W, W * H), sgmgb.synth_pair(max(W, 2), max(H, 2), 64, 3)[0][:H, :W]):
        img = np.ascontiguousarray(img)
        d_img = torch.from_numpy(img).cuda()
        d_out = torch.empty((H, W), dtype=torch.int64, device="cuda")
        engine.census_async(d_img, d_out, W, H)
        engine.sync()
        torch.cuda.synchronize()
        got = d_out.cpu().numpy().view(np.uint64)
        want = oracle.census(img)
        if not np.array_equal(got, want):
            y, x = np.argwhere(got != want)[0]
            xor = int(got[y, x]) ^ int(want[y, x])
            pytest.fail("census diff at (%d,%d): got %016x want %016x lowest bit %d"
                        % (x, y, int(got[y, x]), int(want[y, x]), (xor & -xor).bit_length() - 1))


# ---- plain SGM: edge cases, disparity ranges, path counts ----
@pytest.mark.parametrize("W,H", [(1, 1), (1, 23), (23, 1), (2, 2), (15, 9), (40, 9), (63, 31),
                                 (64, 64), (97, 45), (130, 3)])
@pytest.mark.parametrize("D,paths", [(16, 4), (64, 4), (64, 8), (128, 8)])
def test_plain_small(engine, W, H, D, paths):
    left, right = _rand(H, W, 1), _rand(H, W, 2)
    engine.plan(W, H, D, paths)
    got = engine.run_frame(left, right)
    want = oracle.plain(left, right, D, paths)
    assert np.array_equal(got, want), _first_diff(got, want)


@pytest.mark.parametrize("D", [16, 32, 48, 64, 80, 96, 112, 128, 144, 176, 192, 208, 240, 256])
def test_plain_disparity_ranges(engine, D):
    W, H = 300, 70
    left, right, _ = sgmgb.synth_pair(W, H, min(D, 200), seed=D)
    for paths in (4, 8):
        engine.plan(W, H, D, paths)
        got = engine.run_frame(left, right)
        want = oracle.plain(left, right, D, paths)
        assert np.array_equal(got, want), ("D=%d paths=%d" % (D, paths)) + _first_diff(got, want)


@pytest.mark.parametrize("seed", [1, 2])
def test_plain_640x480_d64(engine, seed):
    """The reference's CPU-runnable configuration: 640x480, D=64, 4 paths."""
    left, right, _ = sgmgb.synth_pair(640, 480, 64, seed)
    engine.plan(640, 480, 64, 4)
    got = engine.run_frame(left, right)
    want = oracle.plain(left, right, 64, 4)
    assert np.array_equal(got, want), _first_diff(got, want)


def test_plain_ties_and_flat(engine):
    """Flat and periodic images make many tied minima: the lowest d must win."""
    W, H = 200, 60
    flat = np.full((H, W), 128, np.uint8)
    stripes = np.tile((np.arange(W) % 7 * 30).astype(np.uint8), (H, 1))
    for l, r in ((flat, flat), (stripes, stripes), (stripes, np.roll(stripes, 3, axis=1))):
        for D, paths in ((64, 4), (64, 8), (128, 4)):
            engine.plan(W, H, D, paths)
            got = engine.run_frame(l, r)
            want = oracle.plain(l, r, D, paths)
            assert np.array_equal(got, want), _first_diff(got, want)


# ---- multi-scale ----
@pytest.mark.parametrize("W,H", [(2, 2), (4, 6), (16, 10), (64, 48), (130, 66), (320, 200)])
def test_multiscale_small(engine, W, H):
    left, right = _rand(H, W, 11), _rand(H, W, 12)
    engine.plan(W, H, 64, 8, sgmgb.MULTISCALE)
    got = engine.run_frame(left, right)
    want = oracle.multiscale(left, right)
    assert np.array_equal(got, want), _first_diff(got, want)


def test_multiscale_synthetic(engine):
    left, right, _ = sgmgb.synth_pair(480, 320, 64, 5)
    engine.plan(480, 320, 64, 8, sgmgb.MULTISCALE)
    got = engine.run_frame(left, right)
    assert np.array_equal(got, oracle.multiscale(left, right))


@pytest.mark.parametrize("sched", ["latency", "throughput"])
def test_multiscale_async_graph(engine, sched):
    """The device-buffer call captures the frame into a CUDA graph, the
    half-scale stage on its own streams beside the full-scale one: the
    captured frame, replayed on two buffer sets, gives the oracle's maps."""
    import torch
    from conftest import reference_multiscale_hash
    engine.set_schedule(SCHEDS[sched])
    try:
        for W, H in ((320, 200), (1920, 800)):
            engine.plan(W, H, 64, 8, sgmgb.MULTISCALE)
            pairs = [sgmgb.synth_pair(W, H, 64, seed=W + k)[:2] for k in range(2)]
            wants = [reference_multiscale_hash(l, r) for l, r in pairs]
            dl = [torch.from_numpy(l).cuda() for l, r in pairs]
            dr = [torch.from_numpy(r).cuda() for l, r in pairs]
            dd = [torch.zeros((H // 2, W // 2), dtype=torch.uint8, device="cuda") for _ in pairs]
            for rep in range(3):                             # capture, then replays
                for k in range(2):
                    engine.run_frame_async(dl[k], dr[k], dd[k])
                engine.sync()
                for k in range(2):
                    assert oracle.fnv1a64(dd[k].cpu().numpy()) == wants[k], (W, H, sched, rep, k)
                    dd[k].zero_()
    finally:
        engine.set_schedule(sgmgb.SCHED_AUTO)


# ---- path-kernel shapes: only speed may depend on them ----
@pytest.mark.parametrize("wpb,dpl", [(1, 2), (2, 4), (3, 8), (4, 4), (4, 8)])
def test_path_shapes(engine, wpb, dpl):
    cases = [((97, 45), 64, 4, sgmgb.PLAIN), ((130, 66), 64, 8, sgmgb.PLAIN), ((61, 40), 16, 4, sgmgb.PLAIN),
             ((300, 70), 48, 8, sgmgb.PLAIN), ((200, 33), 128, 4, sgmgb.PLAIN), ((130, 66), 64, 8, sgmgb.MULTISCALE)]
    try:
        engine.set_path_shape(wpb, dpl)
        for (W, H), D, paths, variant in cases:
            left, right, _ = sgmgb.synth_pair(W, H, D, seed=W + D)
            engine.plan(W, H, D, paths, variant)
            got = engine.run_frame(left, right)
            want = oracle.multiscale(left, right) if variant else oracle.plain(left, right, D, paths)
            assert np.array_equal(got, want), ("%dx%d D=%d paths=%d v=%d" % (W, H, D, paths, variant)
                                               + _first_diff(got, want))
    finally:
        engine.set_path_shape(4, 0)


def test_rejects_bad_path_shape(engine):
    for wpb, dpl in ((0, 2), (5, 2), (4, 3), (4, 16), (4, -1)):
        with pytest.raises(sgmgb.SgmError):
            engine.set_path_shape(wpb, dpl)


def test_rejects_bad_descriptions(engine):
    for args in ((0, 10, 64, 4, 0), (10, 10, 65, 4, 0), (10, 10, 272, 4, 0), (10, 10, 64, 6, 0),
                 (11, 10, 64, 8, 1), (10, 10, 128, 8, 1), (10, 10, 64, 4, 1)):
        with pytest.raises(sgmgb.SgmError) as e:
            engine.plan(*args)
        assert e.value.code == sgmgb.ERR_ARG


# ---- the reference's committed goldens, rebuilt from their generator ----
@pytest.mark.parametrize("golden", ["data/golden/synthetic.pgm", "data/shared/golden_d64.pgm",
                                    "data/shared/golden_d128.pgm", "data/shared/golden_d256.pgm",
                                    "data/multiscale/golden_ms.pgm", "data/multiscale/golden_ms_1080.pgm"])
def test_reference_goldens(engine, ref_fixtures, golden):
    g = ref_fixtures["goldens"][golden]
    s = ref_fixtures["scenes"][g["scene"]]
    left, right, _ = oracle.gen_reference(s["W"], s["H"], s["gen_D"], s["seed"])
    import hashlib
    assert hashlib.sha256(left.tobytes()).hexdigest() == s["sha256_left"]
    assert hashlib.sha256(right.tobytes()).hexdigest() == s["sha256_right"]
    variant = sgmgb.PLAIN if g["variant"] == "plain" else sgmgb.MULTISCALE
    engine.plan(s["W"], s["H"], g["D"], g["paths"], variant)
    got = engine.run_frame(left, right)
    assert got.shape == (g["H"], g["W"])
    assert oracle.fnv1a64(got) == g["fnv1a64"], "%s: FNV mismatch" % golden


# ---- the sgm.h plugin (SGM_IMPL) exactly as the reference harness calls it ----
@pytest.mark.parametrize("D,paths", [(64, 4), (128, 4), (64, 8)])
def test_plugin_sgm_impl(D, paths):
    plug = sgmgb.Plugin(D, paths)
    assert plug.name == "gb300"
    left, right, _ = sgmgb.synth_pair(320, 240, D, 9)
    for _ in range(2):   # second call reuses the resident state
        rc, disp, st = plug.run(left, right, threads=4)
        assert rc == 0
        assert np.array_equal(disp, oracle.plain(left, right, D, paths))
    assert st["aggregate_ms"] > 0 and st["transfer_ms"] >= 0
    # the frame is one graph: its phases are one (aggregate), the fused ones -1
    assert st["census_ms"] == -1 and st["cost_ms"] == -1 and st["argmin_ms"] == -1 and st["threads_used"] == 0
    rc, disp, st = plug.run(left[:100, :150], right[:100, :150])   # resolution change re-plans
    assert rc == 0 and np.array_equal(disp, oracle.plain(left[:100, :150], right[:100, :150], D, paths))


def test_plugin_rejects_empty_frame():
    plug = sgmgb.Plugin(64, 4)
    rc, _, _ = plug.run(np.zeros((0, 5), np.uint8), np.zeros((0, 5), np.uint8))
    assert rc != 0


# ---- full size: 1080p D=64 (configuration A) and the async device path ----
def test_config_a_full_size_async(engine):
    import torch
    left, right, _ = sgmgb.synth_pair(1920, 1080, 64, 1)
    want = oracle.plain(left, right, 64, 4)
    engine.plan(1920, 1080, 64, 4)
    dl, dr = torch.from_numpy(left).cuda(), torch.from_numpy(right).cuda()
    dd = torch.empty((1080, 1920), dtype=torch.uint8, device="cuda")
    s = torch.cuda.current_stream()
    for _ in range(2):
        engine.run_frame_async(dl, dr, dd, stream=s)
    s.synchronize()
    assert np.array_equal(dd.cpu().numpy(), want)
    # host path gives the same bytes
    assert np.array_equal(engine.run_frame(left, right), want)


def test_profile_frame_lists_every_kernel(engine):
    import torch
    W, H = 320, 200
    left, right, _ = sgmgb.synth_pair(W, H, 64, seed=3)
    dl, dr = torch.from_numpy(left).cuda(), torch.from_numpy(right).cuda()
    dd = torch.zeros((H, W), dtype=torch.uint8, device="cuda")
    want = oracle.plain(left, right, 64, 4)
    want_ms = oracle.multiscale(left, right)
    dirs4 = ["census", "cost", "path_rl", "path_lr", "path_bt"]
    fused = ["census", "path_h_first_cost", "path_tb", "path_bt", "path_lr_final", "path_rl_final"]
    cases = [(sgmgb.SCHED_AUTO, dirs4 + ["path_tb", "sum_argmin"], 9),       # a synchronous call: latency
             (sgmgb.SCHED_LATENCY, dirs4 + ["path_tb", "sum_argmin"], 9),
             (sgmgb.SCHED_THROUGHPUT, dirs4 + ["path_tb_final"], 8),
             (sgmgb.SCHED_FUSED, fused, 8),                                 # multi-scale: the throughput schedule
             (sgmgb.SCHED_SPLIT, ["census", "cost", "path_tb", "path_bt", "path_lr_first", "path_rl_first",
                                  "path_lr_final", "path_rl_final"], 8)]
    try:
        for sched, names4, per_scale in cases:
            engine.set_schedule(sched)
            engine.plan(W, H, 64, 4)
            dd.zero_()
            stats = engine.profile_frame(dl, dr, dd, reps=3)
            assert [s[0] for s in stats] == names4
            assert all(ms > 0 and b > 0 for _, ms, b in stats)
            if sched in (sgmgb.SCHED_FUSED, sgmgb.SCHED_SPLIT):
                assert sum(b for n, _, b in stats if n.endswith("_final")) == 4 * W * H * 64 + W * H
            else:
                assert stats[-1][2] == 4 * W * H * 64 + W * H
            assert np.array_equal(dd.cpu().numpy(), want)   # the timed frames are real frames
            engine.plan(W, H, 64, 8, sgmgb.MULTISCALE)
            dd2 = torch.zeros((H // 2, W // 2), dtype=torch.uint8, device="cuda")
            names = [s[0] for s in engine.profile_frame(dl, dr, dd2, reps=2)]
            assert names[:7] == ["half", "sobel_half", "census_half", "cost_half", "sobel", "census", "cost_merge"]
            assert len(names) == 7 + 2 * per_scale
            assert names[-1] == (names4[-1] if sched not in (sgmgb.SCHED_FUSED, sgmgb.SCHED_SPLIT)
                                 else "path_tb_final")
            assert np.array_equal(dd2.cpu().numpy(), want_ms)
    finally:
        engine.set_schedule(sgmgb.SCHED_AUTO)


def test_auto_runs_split_for_a_large_frame_alone(engine):
    """Under AUTO the profile of a frame of at least 2 Mpixel at D >= 64 lists
    the split schedule's kernels (the schedule of a server frame alone), and
    the synchronous call (its own timed choice) returns the checker's map on
    page-locked and on pageable buffers."""
    import torch
    from conftest import reference_plain
    W, H, D = 1920, 1080, 64
    left, right, _ = sgmgb.synth_pair(W, H, D, seed=11)
    want = reference_plain(left, right, D, 4)
    engine.set_schedule(sgmgb.SCHED_AUTO)
    engine.plan(W, H, D, 4)
    dl, dr = torch.from_numpy(left).cuda(), torch.from_numpy(right).cuda()
    dd = torch.zeros((H, W), dtype=torch.uint8, device="cuda")
    names = [s[0] for s in engine.profile_frame(dl, dr, dd, reps=1)]
    assert names == ["census", "cost", "path_tb", "path_bt", "path_lr_first", "path_rl_first", "path_lr_final",
                     "path_rl_final"]
    assert np.array_equal(dd.cpu().numpy(), want)
    hl = torch.from_numpy(left).pin_memory().numpy()
    hr = torch.from_numpy(right).pin_memory().numpy()
    ho = torch.zeros((H, W), dtype=torch.uint8).pin_memory().numpy()
    for _ in range(2):
        engine.run_frame(hl, hr, out=ho)
        assert np.array_equal(ho, want)
        ho[:] = 0
    assert np.array_equal(engine.run_frame(left, right), want)         # pageable: through the copy engines


def test_alone_schedule_is_timed_and_exact(engine):
    """The synchronous call runs one CUDA graph with the schedule that timed
    fastest for a frame alone (under AUTO) or the set one; every choice gives
    the checker's map, and a new plan or schedule makes a new choice."""
    import oracle
    try:
        for (W, H, D, paths, variant) in [(640, 480, 64, 4, sgmgb.PLAIN), (300, 200, 64, 8, sgmgb.MULTISCALE)]:
            left, right, _ = sgmgb.synth_pair(W, H, D, seed=W + 3)
            want = oracle.multiscale(left, right) if variant else oracle.plain(left, right, D, paths)
            engine.set_schedule(sgmgb.SCHED_AUTO)
            engine.plan(W, H, D, paths, variant)
            allowed = {sgmgb.SCHED_LATENCY, sgmgb.SCHED_THROUGHPUT}
            if not variant:
                allowed |= {sgmgb.SCHED_FUSED, sgmgb.SCHED_SPLIT}
            assert engine.alone_schedule() in allowed
            assert np.array_equal(engine.run_frame(left, right), want)
            for sched in sorted(allowed):
                engine.set_schedule(sched)
                assert engine.alone_schedule() == sched
                got, st = engine.run_frame(left, right, times=True)
                assert np.array_equal(got, want), (W, H, variant, sched)
                assert st["census_ms"] == -1 and st["aggregate_ms"] > 0 and st["transfer_ms"] >= 0
    finally:
        engine.set_schedule(sgmgb.SCHED_AUTO)


SCHEDS = {"latency": sgmgb.SCHED_LATENCY, "throughput": sgmgb.SCHED_THROUGHPUT, "fused": sgmgb.SCHED_FUSED,
          "split": sgmgb.SCHED_SPLIT}


@pytest.mark.parametrize("sched", ["latency", "throughput", "fused", "split"])
def test_schedules_agree(engine, sched):
    """Both frame schedules, through the host-buffer call and the device-buffer
    call, on the shapes that take the sum pass's other code paths (D/16 not a
    divisor of 32, 32-bit keys, 8 planes, even-only)."""
    import torch
    engine.set_schedule(SCHEDS[sched])
    try:
        for (W, H, D, paths) in [(300, 70, 48, 4), (301, 71, 128, 4), (160, 90, 32, 8), (200, 64, 64, 8),
                                 (97, 33, 80, 8), (301, 71, 64, 4), (130, 9, 32, 4), (1, 5, 64, 4), (3, 1, 128, 4),
                                 (65, 2, 64, 4), (127, 33, 128, 4)]:
            left, right, _ = sgmgb.synth_pair(W, H, min(D, 128), seed=W + D)
            want = oracle.plain(left, right, D, paths)
            engine.plan(W, H, D, paths)
            assert np.array_equal(engine.run_frame(left, right), want), (W, H, D, paths)
            dl, dr = torch.from_numpy(left).cuda(), torch.from_numpy(right).cuda()
            dd = torch.zeros((H, W), dtype=torch.uint8, device="cuda")
            engine.run_frame_async(dl, dr, dd)
            engine.sync()
            assert np.array_equal(dd.cpu().numpy(), want), (W, H, D, paths, "async")
        left, right, _ = sgmgb.synth_pair(130, 66, 64, seed=5)
        engine.plan(130, 66, 64, 8, sgmgb.MULTISCALE)
        assert np.array_equal(engine.run_frame(left, right), oracle.multiscale(left, right))
    finally:
        engine.set_schedule(sgmgb.SCHED_AUTO)


def test_rejects_bad_schedule(engine):
    with pytest.raises(sgmgb.SgmError):
        engine.set_schedule(5)
    with pytest.raises(sgmgb.SgmError):
        engine.set_schedule(-1)


@pytest.mark.parametrize("pin", ["in", "out", "both"])
def test_pinned_host_buffers(engine, pin):
    """Page-locked host buffers (images, map or both) give the same map as
    pageable ones."""
    import torch
    def pinned(a):
        t = torch.from_numpy(np.ascontiguousarray(a)).pin_memory()
        return t, t.numpy()
    cases = [(320, 200, 64, 4, sgmgb.PLAIN), (301, 77, 128, 8, sgmgb.PLAIN), (130, 66, 64, 8, sgmgb.MULTISCALE)]
    if pin == "both":   # several tiles per block of the streaming census
        cases.append((1920, 1080, 64, 4, sgmgb.PLAIN))
    for (W, H, D, paths, variant) in cases:
        left, right, _ = sgmgb.synth_pair(W, H, min(D, 128), seed=W)
        want = oracle.multiscale(left, right) if variant == sgmgb.MULTISCALE else oracle.plain(left, right, D, paths)
        engine.plan(W, H, D, paths, variant)
        keep = []
        if pin in ("in", "both"):
            (tl, left), (tr, right) = pinned(left), pinned(right)
            keep += [tl, tr]
        out = None
        if pin in ("out", "both"):
            to, out = pinned(np.zeros_like(want))
            keep.append(to)
        for _ in range(2):
            got = engine.run_frame(left, right, out=out)
            assert np.array_equal(got, want), (W, H, D, paths, variant, pin)


# ---- frames at the batched and served configurations' sizes ----
@pytest.mark.parametrize("sched", ["latency", "throughput"])
@pytest.mark.parametrize("frame", [(1920, 1080, 128, 8), (1920, 800, 64, 8)])
def test_baseline_size_8path(engine, baseline_frames, sched, frame):
    """Plain 8-path at full size (long diagonals of up to 1080 steps, the
    eight-plane final pass of the throughput schedule) through the host-buffer
    and the device-buffer calls, byte for byte against the checker."""
    import torch
    left, right, want = baseline_frames[frame]
    W, H, D, paths = frame
    engine.set_schedule(sgmgb.SCHED_LATENCY if sched == "latency" else sgmgb.SCHED_THROUGHPUT)
    try:
        engine.plan(W, H, D, paths)
        got = engine.run_frame(left, right)
        assert np.array_equal(got, want), _first_diff(got, want)
        dl, dr = torch.from_numpy(left).cuda(), torch.from_numpy(right).cuda()
        dd = torch.zeros((H, W), dtype=torch.uint8, device="cuda")
        engine.run_frame_async(dl, dr, dd)
        engine.sync()
        got = dd.cpu().numpy()
        assert np.array_equal(got, want), "async:" + _first_diff(got, want)
    finally:
        engine.set_schedule(sgmgb.SCHED_AUTO)


@pytest.mark.parametrize("frame", [(1920, 1080, 64, 4), (1280, 720, 128, 4), (1920, 1080, 32, 4)])
def test_fused_schedule_full_size(engine, frame):
    """The schedules that split the rows (FUSED: costs computed in the first
    halves; SPLIT: first halves beside the vertical passes) at full size,
    through the host-buffer and the device-buffer calls, against the checker."""
    import torch
    from conftest import reference_plain
    W, H, D, paths = frame
    left, right, _ = sgmgb.synth_pair(W, H, D, seed=W + D + 7)
    want = reference_plain(left, right, D, paths)
    engine.plan(W, H, D, paths)
    try:
        for sched in (sgmgb.SCHED_FUSED, sgmgb.SCHED_SPLIT, sgmgb.SCHED_THROUGHPUT):
            engine.set_schedule(sched)
            got = engine.run_frame(left, right)
            assert np.array_equal(got, want), ("host", sched) + (_first_diff(got, want),)
            dl, dr = torch.from_numpy(left).cuda(), torch.from_numpy(right).cuda()
            dd = torch.zeros((H, W), dtype=torch.uint8, device="cuda")
            for _ in range(2):                                  # graph capture, then replay
                engine.run_frame_async(dl, dr, dd)
            engine.sync()
            got = dd.cpu().numpy()
            assert np.array_equal(got, want), ("async", sched) + (_first_diff(got, want),)
    finally:
        engine.set_schedule(sgmgb.SCHED_AUTO)
