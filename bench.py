#!/usr/bin/env python3
"""Throughput of the GB300 SGM engine on configuration A (1920x1080, D=64,
4 paths, bit-exact), in MDE/s (W*H*D / second), with frames/s beside it.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]
                  [--no-batch] [--no-serve]

One step is one frame through the engine. `value` is measured with the
inputs already resident on the device (one CUDA-graph launch per frame,
round-robin over 8 distinct synthetic pairs whose working set is far larger
than L2); `e2e` is the same metric through the host-buffer call
(sgmgb_run_frame: pinned host inputs copied in, the disparity map copied
back, every step), and `e2e.pageable` through the plugin's SGM_IMPL.run on
pageable buffers, as the reference harness calls it. `roofline` is the
dominant kernel's: its algorithmic bytes per launch over its mean launch time
(CUDA events, kernel alone), against the measured HBM copy bandwidth;
`frame_roofline` relates the modelled minimal bytes of a frame
(2*W*H*D + 3*W*H) to the pipelined frame time. `batched` runs the 96-pair
mixed batch in one persistent launch against 96 sequential drop-in calls;
`served` drives 8 virtual cameras with Poisson arrivals through the server
and reports p50/p99 latency. `multiscale` times configurations B and C (the
multi-scale 8-path variant at 1920x800 and 1920x1080).

The CPU leg runs last: `cpu_baseline` is the reference's own common/sgm_ref.c
(built from its sources by oracle/build_ref.sh and called through its
SGM_IMPL; the oracle port where it is not built) on whole frames, one
thread; the same run checks the GPU's maps (`bit_exact`), the reference's
multi-scale program checks and times configurations B/C on every host thread,
and one frame of each class of the batched mix is checked against the
reference. `--impl reference` times the reference's CPU path on every host
thread, one whole frame per thread per step, with the same `config`.

Multi-GPU: frames are independent, so N GPUs run N replicas (one process per
GPU under torchrun); `value` is the frames of all ranks over the slowest
rank's time. No collective is on the data path.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
for p in (os.path.join(ROOT, "sgm-bench_gb300"), os.path.join(ROOT, "oracle")):
    if p not in sys.path:
        sys.path.insert(0, p)

W, H, D, PATHS = 1920, 1080, 64, 4
WORKLOAD = "configA_1920x1080_D64_4path"
METRIC = "MDE/s (W*H*D per second), 1080p D=64 4-path, bit-exact"
UNIT = "MDE/s"
B_ALG = 2 * W * H * D + 3 * W * H          # modelled minimal bytes per frame
KERNELS_PER_FRAME = 2 + PATHS               # census + cost volume + one pass per direction
SCHED_NAMES = {1: "latency", 2: "throughput", 3: "fused", 4: "split"}


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def committed_profile(kind, kernel):
    """DRAM bytes ("traffic": read + write) or warp-instructions
    ("instructions") of one launch of `kernel` at configuration A, from the
    committed ncu summary (lines "<kind> <kernel> <count>"), or None."""
    path = os.path.join(ROOT, "profiles", "configA_kernel_traffic.txt")
    try:
        for line in open(path):
            f = line.split()
            if len(f) >= 3 and f[0] == kind and f[1] == kernel:
                return int(f[2])
    except Exception:
        pass
    return None


def committed_traffic(kernel):
    return committed_profile("traffic", kernel)


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled while the timed region runs."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index=0):
        self.gpu = gpu_index
        self.rows = []
        self.proc = None

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.Q,
                                          "--format=csv,noheader,nounits", "-lms", "50"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append((time.time(), [x.strip() for x in line.split(",")]))

    def stop(self):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
            self.t.join(timeout=2)

    def summary(self, t0, t1):
        rows = [r for (ts, r) in self.rows if t0 - 0.06 <= ts <= t1 + 0.06] or [r for _, r in self.rows[-2:]]
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"], "samples": 0}
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = set()
        sm = []
        for r in rows:
            try:
                sm.append(float(r[1]))
            except ValueError:
                pass
            for k, n in enumerate(names):
                if len(r) > 5 + k and r[5 + k].lower().startswith("active"):
                    reasons.add(n)
        try:
            smax = float(rows[0][2])
        except ValueError:
            smax = None
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": smax,
                "reasons": sorted(reasons), "samples": len(rows)}


def dist_setup():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def max_over_ranks(v, dist, device):
    """The largest of each rank's v (the slowest rank's time); v itself on one process."""
    if dist is None:
        return float(v)
    import torch
    t = torch.tensor([float(v)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_value(ws, frames_per_rank, seconds):
    """Whole-job MDE/s: every rank's frames over the slowest rank's time."""
    return ws * frames_per_rank * W * H * D / seconds / 1e6


def batched_section(eng_cls, sgmgb, torch, np):
    """The batched form on the 96-pair mix (24 each at 640x480, 1280x720,
    1920x800, 1920x1080; D 64/128 alternating; every 4th pair 8-path) against
    96 sequential plain drop-in calls (host buffers, one pre-planned context
    per frame description, so no re-planning is timed)."""
    sizes = [(640, 480), (1280, 720), (1920, 800), (1920, 1080)]
    specs = [(W, H, 64 if k % 2 == 0 else 128, 8 if k % 4 == 3 else 4) for (W, H) in sizes for k in range(24)]
    scenes = {}
    for (W, H, Dk, P) in specs:
        if (W, H, Dk) not in scenes:
            scenes[(W, H, Dk)] = sgmgb.synth_pair(W, H, Dk, seed=W + Dk)[:2]
    host = [scenes[(W, H, Dk)] for (W, H, Dk, P) in specs]
    dl = [torch.from_numpy(l).cuda() for l, r in host]
    dr = [torch.from_numpy(r).cuda() for l, r in host]
    out = [torch.zeros((H, W), dtype=torch.uint8, device="cuda") for (W, H, Dk, P) in specs]
    eng = eng_cls(0)
    b = sgmgb.Batch(eng, [sgmgb.desc(*sp) for sp in specs])
    b.autotune(dl, dr, out)
    mode, lanes = b.mode()

    def time_batch():
        b.run(dl, dr, out)
        b.wait()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        reps = 5
        s = torch.cuda.current_stream()
        e0.record(s)
        for _ in range(reps):
            b.run(dl, dr, out, stream=s)           # on the stream the events are recorded on
        e1.record(s)
        b.wait()
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / reps

    # both modes, the autotuned one last (its maps are the ones checked)
    other = (sgmgb.BATCH_IN_FLIGHT, 6) if mode == sgmgb.BATCH_PERSISTENT else (sgmgb.BATCH_PERSISTENT, 0)
    b.set_mode(*other)
    other_ms = time_batch()
    b.set_mode(mode, lanes or 6)
    batch_ms = time_batch()
    mode_ms = {mode: batch_ms, other[0]: other_ms}
    engs = {sp: eng_cls(0).plan(*sp) for sp in set(specs)}
    ref = [engs[sp].run_frame(l, r) for sp, (l, r) in zip(specs, host)]        # warm-up and reference maps
    t0 = time.perf_counter()
    for sp, (l, r) in zip(specs, host):
        engs[sp].run_frame(l, r)
    seq_ms = (time.perf_counter() - t0) * 1e3
    maps = [o.cpu().numpy() for o in out]
    same = all(np.array_equal(m, rf) for m, rf in zip(maps, ref))
    shapes = sorted(set(b.tile_shape(i) for i in range(len(specs))))
    busy = b.busy()
    busy_ms = {k: busy[k] for k in sgmgb.Batch.BUSY_KINDS}
    blocks = busy["blocks"]
    for e in engs.values():
        e.close()
    b.close()
    eng.close()
    # one frame of every (size, D, paths) class for the CPU leg's reference
    # check; frames of a class share the class's input pair, so a class whose
    # maps are all identical is covered by its one checked frame
    checks, seen, covered = [], {}, 0
    for sp, (l, r), m in zip(specs, host, maps):
        if sp not in seen:
            seen[sp] = m
            checks.append(sp + (l, r, m))
        covered += int(np.array_equal(m, seen[sp]))
    mde = sum(W * H * Dk for (W, H, Dk, P) in specs)
    return {"frames": len(specs), "ms_per_batch": batch_ms, "fps": 96e3 / batch_ms,
            "mde_per_s": mde / (batch_ms / 1e3) / 1e6,
            "sequential_dropin_ms": seq_ms, "sequential_dropin_fps": 96e3 / seq_ms,
            "speedup_vs_sequential_dropin": seq_ms / batch_ms, "identical_to_dropin": bool(same),
            "frames_equal_to_their_checked_class_frame": covered,
            "block_time_ms": {k: round(v, 3) for k, v in busy_ms.items()},
            "block_time_share": {k: round(v / max(1e-9, sum(busy_ms.values())), 4) for k, v in busy_ms.items()},
            "blocks": blocks,
            "busy_per_block_over_run": sum(busy_ms.values()) / blocks / mode_ms[sgmgb.BATCH_PERSISTENT],
            "block_time_note": "time the persistent kernel's blocks spent per work-item kind in the last run "
                               "(global-timer stamps, summed over blocks); 'wait' is time "
                               "spent waiting for an item's inputs or on an empty queue",
            "mode": "in_flight" if mode == sgmgb.BATCH_IN_FLIGHT else "persistent", "lanes": lanes,
            "persistent_ms": mode_ms[sgmgb.BATCH_PERSISTENT], "in_flight_ms": mode_ms[sgmgb.BATCH_IN_FLIGHT],
            "tile_shapes_warps_dpl": shapes,
            "note": "the mode the autotuner kept: one persistent launch per batch, or every frame's own "
                    "pipeline on concurrent chains (in_flight, 6 lanes timed for the other figure), each a "
                    "CUDA graph per batch; block time is the persistent launch's; batch inputs resident on "
                    "the device; drop-in calls copy host buffers in and out"}, checks


def served_section(eng_cls, sgmgb, np, rates=(2000.0, 3000.0, 4000.0), secs=3.0):
    """8 virtual cameras (sizes from 640x480 / 1280x720 / 1920x1080, D 64/128,
    4-path), Poisson arrivals at each offered rate in turn (the first, 2000
    frames/s, is the configuration's), 40 GB budget. Before each run the
    cameras' slots are made up front (sgmgb_server_prepare), so no device
    allocation falls inside the run; results are collected on one thread per
    camera, so a slow frame of one camera holds no other camera's request
    buffers. Every result is compared with the same frame run alone."""
    import queue
    rng = np.random.default_rng(0)
    sizes = [(640, 480), (1280, 720), (1920, 1080)]
    cams = {c: sizes[rng.integers(0, 3)] + (int(rng.choice([64, 128])), 4) for c in range(8)}
    scenes, want = {}, {}
    for c, (W, H, Dk, P) in cams.items():
        scenes[c] = [sgmgb.synth_pair(W, H, Dk, seed=1000 + 10 * c + k)[:2] for k in range(2)]
        e = eng_cls(0).plan(W, H, Dk, P)
        want[c] = [e.run_frame(l, r) for l, r in scenes[c]]
        e.close()
    eng = eng_cls(0)

    def one_run(rate):
        srv = sgmgb.Server(eng, hbm_budget_bytes=40 << 30, max_inflight=8)
        for c, (W, H, Dk, P) in cams.items():
            srv.add_camera(c, W, H, Dk, P)
        slots = srv.prepare(4)
        qs = {c: queue.Queue() for c in cams}
        refused, bad = [0], [0]
        prng = np.random.default_rng(int(rate))

        def producer():
            t_next = time.perf_counter()
            t_end = t_next + secs
            i = 0
            while True:
                t_next += prng.exponential(1.0 / rate)
                if t_next > t_end:
                    break
                gap = t_next - time.perf_counter()
                if gap > 3e-4:
                    time.sleep(gap - 2e-4)      # sleeping releases the interpreter lock for the collectors
                while time.perf_counter() < t_next:
                    pass
                c = int(prng.integers(0, 8))
                try:
                    qs[c].put((srv.submit(c, *scenes[c][i % 2]), i % 2))
                except sgmgb.SgmError:
                    refused[0] += 1
                i += 1
            for q in qs.values():
                q.put(None)

        def collector(c):
            while True:
                it = qs[c].get()
                if it is None:
                    return
                t, k = it
                o, _ = srv.wait(t, 60000)
                if not np.array_equal(o, want[c][k]):
                    bad[0] += 1

        switch = sys.getswitchinterval()
        sys.setswitchinterval(2e-4)             # the client threads share the interpreter lock finely
        th = [threading.Thread(target=producer)] + [threading.Thread(target=collector, args=(c,)) for c in cams]
        for t in th:
            t.start()
        for t in th:
            t.join()
        sys.setswitchinterval(switch)
        st = srv.stats()
        srv.close()
        return {"offered_fps": rate, "fps": st["fps"], "frames_done": st["frames_done"],
                "frames_refused": st["frames_refused"], "p50_ms": st["p50_ms"],
                "p99_ms": st["p99_ms"], "max_ms": st["max_ms"], "resident_gb": st["resident_bytes"] / 1e9,
                "slots": slots, "results_differing_from_alone": bad[0]}

    runs = [one_run(r) for r in rates]
    eng.close()
    base = runs[0]
    ok = [r for r in runs if r["frames_refused"] == 0 and r["results_differing_from_alone"] == 0]
    return {"cameras": {str(c): "%dx%d D=%d" % v[:3] for c, v in cams.items()}, "offered_fps": base["offered_fps"],
            "seconds": secs, "frames_done": base["frames_done"], "frames_refused": base["frames_refused"],
            "fps": base["fps"], "p50_ms": base["p50_ms"], "p99_ms": base["p99_ms"], "max_ms": base["max_ms"],
            "resident_gb": base["resident_gb"], "slots": base["slots"], "budget_gb": 40 * 2 ** 30 / 1e9,
            "results_differing_from_alone": sum(r["results_differing_from_alone"] for r in runs),
            "load_sweep": runs,
            "capacity_fps": max(r["fps"] for r in ok) if ok else None,
            "capacity_note": "the highest sustained frames/s of the load sweep with no frame refused",
            "latency": "submit (host copy into pinned memory) to result in pinned host memory"}


def cpu_baseline_sample(seconds, left, right, gpu_maps, ms_checks=(), batch_checks=()):
    """The CPU leg, run after every GPU section.

    cpu_baseline: the reference's own common/sgm_ref.c (its SGM_IMPL, built from
    its sources; the oracle port where it was not built), one thread, as the
    reference runs it (single-threaded by design, sgm_ref.c:3), timed on whole
    configuration-A frames -- the pair the GPU timed first -- for at most
    `seconds` (8 frames at most).

    The checker: the GPU's maps of that pair (`gpu_maps`) against that output;
    the multi-scale maps (`ms_checks`: name, left, right, map) against
    multiscale/sgm_ms_ref.c run on every host thread (its FNV hash; that run is
    also the multi-scale CPU baseline), else the oracle; and one frame of every
    (size, D, paths) class of the batched mix (`batch_checks`: W, H, D, paths,
    left, right, map) against the reference for that D and path count, on a
    thread pool."""
    import concurrent.futures as cf
    import oracle
    run, kind = reference_checker(D, PATHS)
    n, t0 = 0, time.perf_counter()
    while True:
        want = run(left, right)
        n += 1
        el = time.perf_counter() - t0
        if el >= seconds or n >= 8:
            break
    exact = all(np.array_equal(m, want) for m in gpu_maps)
    what = "common/sgm_ref.c via SGM_IMPL" if kind == "reference" else "oracle/sgm_oracle.c"
    base = {"value": n * W * H * D / el / 1e6, "unit": UNIT, "cores": 1, "kind": kind,
            "sample": "%d frame(s) of %dx%d D=%d %d-path, %s, 1 thread, %.1f s" % (n, W, H, D, PATHS, what, el)}
    ms = {}
    for name, l, r, m in ms_checks:
        Wm, Hm = l.shape[1], l.shape[0]
        work = ((Wm // 2) * (Hm // 2) + Wm * Hm) * 64
        try:
            med, fnv, omp, thr = oracle.reference_multiscale(l, r, reps=3)
            ms[name] = {"bit_exact_vs_reference": fnv == oracle.fnv1a64(m),
                        "cpu_baseline": {"ms_per_frame": med, "mde_per_s_work": work / (med / 1e3) / 1e6,
                                         "cores": thr, "kind": "reference", "openmp": omp,
                                         "sample": "3 frames, multiscale/sgm_ms_ref.c (median it prints), "
                                                   "OMP_NUM_THREADS=%d" % thr}}
        except FileNotFoundError:
            ms[name] = {"bit_exact_vs_oracle": bool(np.array_equal(m, oracle.multiscale(l, r)))}
    batch = None
    if batch_checks:
        threads = len(os.sched_getaffinity(0)) if hasattr(os, "sched_getaffinity") else (os.cpu_count() or 1)

        def one(c):
            Wc, Hc, Dc, Pc, l, r, m = c
            f, k = reference_checker(Dc, Pc)
            return bool(np.array_equal(f(l, r), m)), k

        with cf.ThreadPoolExecutor(max_workers=min(threads, len(batch_checks))) as pool:
            res = list(pool.map(one, batch_checks))
        batch = {"classes_checked": len(res), "all_exact": all(r[0] for r in res),
                 "kinds": sorted(set(r[1] for r in res)),
                 "failed": ["%dx%d D=%d P=%d" % c[:4] for c, r in zip(batch_checks, res) if not r[0]]}
    return base, exact, ms, batch


def sweep_section(sgmgb, torch, np, warmup=10, frames=60):
    """The reference's disparity-range x resolution grid (scripts/sweep.sh:20-56):
    D in {32, 64, 128} x {1920x1080, 1280x720, 960x540, 640x480}, 4 paths, plus
    D = 256 at 1920x1080, timed like the reference's harness cell (-w 10 -n 60):
    the median wall time of the drop-in call on pinned host buffers, copies in
    and out included. The golden of every cell, with the reference's
    discrimination gate, is checked in tests/test_gpu_sweep.py; here the scene
    is this package's generator at the cell's D."""
    cells = [(D, W, H) for D in (32, 64, 128) for (W, H) in ((1920, 1080), (1280, 720), (960, 540), (640, 480))]
    cells.append((256, 1920, 1080))
    eng = sgmgb.Engine(0)
    out = []
    for D, W, H in cells:
        l, r, _ = sgmgb.synth_pair(W, H, min(D, 200), 1)
        hl = torch.from_numpy(l).pin_memory().numpy()
        hr = torch.from_numpy(r).pin_memory().numpy()
        ho = torch.empty((H, W), dtype=torch.uint8).pin_memory().numpy()
        eng.plan(W, H, D, 4)
        for _ in range(warmup):
            eng.run_frame(hl, hr, out=ho)
        lat = []
        for _ in range(frames):
            t0 = time.perf_counter()
            eng.run_frame(hl, hr, out=ho)
            lat.append(time.perf_counter() - t0)
        med = statistics.median(lat) * 1e3
        out.append({"D": D, "W": W, "H": H, "median_ms": round(med, 4), "fps": round(1e3 / med, 1),
                    "mde_per_s": round(W * H * D / med / 1e3, 1)})
    eng.close()
    return {"cells": out, "paths": 4, "timing": "median of %d drop-in calls after %d warm-up, pinned host "
                                                "buffers" % (frames, warmup)}


def multiscale_section(sgmgb, torch, np, steps=60, inflight=4):
    """Configurations B and C: the multi-scale 8-path variant at 1920x800 and
    1920x1080 (output (W/2)x(H/2)), frames in flight as in the main line;
    MDE/s under the reference's work convention ((W/2)(H/2) + W*H) * 64 per
    second (multiscale/sgm_ms_ref.c:211-216). Returns the section and, per
    configuration, one (left, right, map) for the CPU leg's oracle check."""
    out, checks = {}, []
    for name, (Wm, Hm) in (("configB_1920x800", (1920, 800)), ("configC_1920x1080", (1920, 1080))):
        engs = []
        for _ in range(inflight):
            e = sgmgb.Engine(0)
            e.plan(Wm, Hm, 64, 8, sgmgb.MULTISCALE)
            engs.append(e)
        strs = [torch.cuda.current_stream()] + [torch.cuda.Stream() for _ in range(inflight - 1)]
        pairs = [sgmgb.synth_pair(Wm, Hm, 64, 300 + k) for k in range(inflight)]
        dl = [torch.from_numpy(p[0]).cuda() for p in pairs]
        dr = [torch.from_numpy(p[1]).cuda() for p in pairs]
        dd = [torch.empty((Hm // 2, Wm // 2), dtype=torch.uint8, device="cuda") for _ in range(inflight)]
        for i in range(2 * inflight):                                 # warm-up (graphs captured)
            engs[i % inflight].run_frame_async(dl[i % inflight], dr[i % inflight], dd[i % inflight],
                                               stream=strs[i % inflight])
        torch.cuda.synchronize()
        checks.append((name, pairs[0][0], pairs[0][1], dd[0].cpu().numpy()))
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        s0 = strs[0]
        e0.record(s0)
        for st in strs[1:]:
            st.wait_event(e0)
        for i in range(steps):
            engs[i % inflight].run_frame_async(dl[i % inflight], dr[i % inflight], dd[i % inflight],
                                               stream=strs[i % inflight])
        for st in strs[1:]:
            ev = torch.cuda.Event()
            ev.record(st)
            s0.wait_event(ev)
        e1.record(s0)
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1) / steps
        # one frame at a time, pinned host buffers (the drop-in call)
        hl = torch.from_numpy(pairs[0][0]).pin_memory().numpy()
        hr = torch.from_numpy(pairs[0][1]).pin_memory().numpy()
        ho = torch.empty((Hm // 2, Wm // 2), dtype=torch.uint8).pin_memory().numpy()
        for _ in range(3):
            engs[0].run_frame(hl, hr, out=ho)
        lat = []
        for _ in range(20):
            t0 = time.perf_counter()
            engs[0].run_frame(hl, hr, out=ho)
            lat.append(time.perf_counter() - t0)
        e2e_ms = statistics.median(lat) * 1e3
        work = ((Wm // 2) * (Hm // 2) + Wm * Hm) * 64
        out[name] = {"W": Wm, "H": Hm, "out": [Wm // 2, Hm // 2], "ms_per_frame": ms, "fps": 1e3 / ms,
                     "mde_per_s_work": work / (ms / 1e3) / 1e6, "frames_in_flight": inflight,
                     "e2e_ms_per_frame": e2e_ms, "e2e_fps": 1e3 / e2e_ms}
        for e in engs:
            e.close()
    return out, checks


def workload_config(ws):
    """The `config` both arms print: the workload, not how an arm runs it."""
    return {"workload": WORKLOAD, "W": W, "H": H, "D": D, "paths": PATHS, "variant": "plain",
            "inputs": "8 synthetic pairs (seeds 1..8) round-robin; per-frame working set > L2",
            "parallelism": "replicas" if ws > 1 else "single"}


def reference_checker(Dk, paths):
    """(function left, right -> map, kind): the reference's own sgm_ref.c built
    from its sources (oracle/_ref) where it was built, else the oracle port."""
    import oracle
    if oracle.reference_available(Dk, paths):
        ref = oracle.ReferenceImpl(Dk, paths)
        return ref.run, "reference"
    return (lambda l, r: oracle.plain(l, r, Dk, paths)), "port"


def reference_gpu_section(left, right):
    """The reference's own CUDA programs, built for sm_103a from its sources
    by oracle/build_ref.sh and run on this GPU: cuda/sgm_cuda_opt.cu (4 paths,
    D = 64 and 128) in the reference's harness, timed by the harness on its
    pageable buffers (cuda/sgm_cuda_opt.cu:321-366 copies them in and out
    inside each run), and multiscale/sgm_ms_cuda.cu on configurations B and C
    (its own main and timing, multiscale/sgm_ms_cuda.cu:160-208). A same-GPU
    comparison, not the target. Each map is compared with the reference's CPU
    program on the same pair."""
    import oracle
    out = {"what": "the reference's CUDA programs built for sm_103a (oracle/build_ref.sh), same GPU"}
    if not os.path.exists("/dev/nvidiactl"):
        out["unavailable"] = "no GPU on this host"
        return out
    for Dk in (64, 128):
        name = "cuda_opt_d%d_1920x1080" % Dk
        try:
            t, disp = oracle.reference_cuda_plain(left, right, Dk)
            want, _ = reference_checker(Dk, 4)
            t["equal_to_reference_cpu"] = bool(np.array_equal(disp, want(left, right)))
            t["mde_per_s"] = W * H * Dk / (t["median_ms"] / 1e3) / 1e6
            t["call"] = ("common/harness.c: median of %d runs after %d warm-up, each run copies the pageable "
                         "images in and the map out" % (t["runs"], t["warmup"]))
            out[name] = t
        except Exception as e:                      # not built, or it failed: say so, keep the line
            out[name] = {"unavailable": (str(e).strip().splitlines() or ["?"])[0][:200]}
    for name, (Wm, Hm) in (("ms_cuda_configB_1920x800", (1920, 800)), ("ms_cuda_configC_1920x1080", (1920, 1080))):
        try:
            l2, r2, _ = oracle.synth_pair(Wm, Hm, 64, 300)
            ms, h, _ = oracle.reference_cuda_multiscale(l2, r2)
            _, h_cpu, _, _ = oracle.reference_multiscale(l2, r2, reps=1)
            work = ((Wm // 2) * (Hm // 2) + Wm * Hm) * 64
            out[name] = {"median_ms": ms, "hash": h, "equal_to_reference_cpu": h == h_cpu,
                         "mde_per_s_work": work / (ms / 1e3) / 1e6,
                         "call": "its own main: inputs copied once, each timed frame the kernels and the map "
                                 "copied out, median of 10 after 3 warm-up"}
        except Exception as e:
            out[name] = {"unavailable": (str(e).strip().splitlines() or ["?"])[0][:200]}
    return out


def run_reference(args):
    """The reference's CPU implementation of the path (common/sgm_ref.c through
    its SGM_IMPL, built from its sources by oracle/build_ref.sh; the oracle port
    where it is not built) on every host thread: each step, every thread runs
    one whole configuration-A frame (single-threaded by design, sgm_ref.c:3),
    so a step is `threads` frames. Long runs (steps + warmup > 40) time a band
    of rows per frame instead, to end within minutes. Rank 0 only."""
    ws, rank, _ = dist_setup()
    if rank != 0:
        return 0
    import concurrent.futures as cf
    import oracle
    threads = len(os.sched_getaffinity(0)) if hasattr(os, "sched_getaffinity") else (os.cpu_count() or 1)
    run, kind = reference_checker(D, PATHS)
    total = args.steps + args.warmup
    rows = H if total <= 40 else max(64, int(H * 40 / total))
    pairs = [oracle.synth_pair(W, H, D, k + 1)[:2] for k in range(8)]
    work = [(np.ascontiguousarray(l[:rows]), np.ascontiguousarray(r[:rows])) for l, r in pairs]
    pool = cf.ThreadPoolExecutor(max_workers=threads)

    def step(i):
        list(pool.map(lambda t: run(*work[(i * threads + t) % 8]), range(threads)))

    for i in range(args.warmup):
        step(i)
    t0 = time.perf_counter()
    for i in range(args.steps):
        step(args.warmup + i)
    el = time.perf_counter() - t0
    per_step = el / args.steps
    value = threads * W * rows * D / per_step / 1e6
    what = "common/sgm_ref.c via SGM_IMPL" if kind == "reference" else "oracle port of common/sgm_ref.c"
    sample = "%d threads x one %dx%d D=%d %d-path %s per step (%s)" % (
        threads, W, rows, D, PATHS, "frame" if rows == H else "band of the frame", what)
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": per_step * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "u16", "data": "synthetic",
            "config": workload_config(ws),
            "impl": "reference",
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": kind, "sample": sample},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    if not getattr(args, "no_refgpu", False):
        line["reference_gpu"] = reference_gpu_section(*pairs[0])
    print(json.dumps(line))
    return 0


def run_gb300(args):
    import numpy as np
    import torch
    import sgmgb
    ws, rank, local = dist_setup()
    torch.cuda.set_device(local)
    dist = None
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    dev = torch.device("cuda", local)
    eng = sgmgb.Engine(local)
    eng.plan(W, H, D, PATHS)
    eng.set_path_shape(args.warps_per_block, args.disp_per_lane)
    # frames in flight: each has its own context (resident workspace, stream,
    # cached graph); consecutive frames alternate between them, so one frame's
    # final pass overlaps the next frame's census, cost and first passes
    engines = [eng]
    for _ in range(args.inflight - 1):
        e = sgmgb.Engine(local)
        e.plan(W, H, D, PATHS)
        e.set_path_shape(args.warps_per_block, args.disp_per_lane)
        engines.append(e)
    # 8 distinct resident pairs, round-robin: inputs differ every step and the
    # per-frame working set (about 430 MB of census, scratch and sum planes)
    # is far larger than the 129 MB L2.
    R = 8
    pairs = [sgmgb.synth_pair(W, H, D, 1000 * rank + k + 1) for k in range(R)]
    dl = [torch.from_numpy(p[0]).to(dev) for p in pairs]
    dr = [torch.from_numpy(p[1]).to(dev) for p in pairs]
    dd = [torch.empty((H, W), dtype=torch.uint8, device=dev) for _ in range(R)]
    s = torch.cuda.current_stream(dev)
    streams = [s] + [torch.cuda.Stream(dev) for _ in range(args.inflight - 1)]
    NF = len(engines)
    assert R % NF == 0          # output buffer i % R is always written by the same context and stream

    # what is timed, for the checker in the CPU leg: the first pair through every context
    maps0 = []
    for k, e in enumerate(engines):
        e.run_frame_async(dl[0], dr[0], dd[0], stream=streams[k])
        streams[k].synchronize()
        maps0.append(dd[0].cpu().numpy())

    def run_frames(n, nf):
        for i in range(n):
            engines[i % nf].run_frame_async(dl[i % R], dr[i % R], dd[i % R], stream=streams[i % nf])

    # one frame at a time (a single context and stream), for the frame latency,
    # with the schedule the synchronous call takes under AUTO (the fastest for a
    # frame alone, timed at the first call)
    alone = eng.alone_schedule()
    eng.set_schedule(alone)
    run_frames(3, 1)
    torch.cuda.synchronize(dev)
    e0s, e1s = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    n_serial = max(10, args.steps // 4)
    e0s.record(s)
    run_frames(n_serial, 1)
    e1s.record(s)
    torch.cuda.synchronize(dev)
    serial_ms_per_frame = e0s.elapsed_time(e1s) / n_serial
    eng.set_schedule(sgmgb.SCHED_AUTO)   # frames in flight: the fused schedule
    run_frames(args.warmup, NF)
    torch.cuda.synchronize(dev)

    def barrier():
        if dist is not None:
            dist.barrier()
        torch.cuda.synchronize(dev)

    clocks = ClockSampler(local)
    clocks.start()
    time.sleep(0.3)
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    barrier()
    tw0 = time.time()
    ev0.record(s)
    for st in streams[1:]:
        st.wait_event(ev0)
    run_frames(args.steps, NF)
    for st in streams[1:]:
        ev = torch.cuda.Event()
        ev.record(st)
        s.wait_event(ev)
    ev1.record(s)
    barrier()
    tw1 = time.time()
    clocks.stop()
    ms = max_over_ranks(ev0.elapsed_time(ev1), dist, dev)
    ms_per_step = ms / args.steps
    value = replica_value(ws, args.steps, ms / 1e3)

    # end to end through the host-buffer call: pinned inputs in, the map out
    # into a pinned buffer, every step (copied by the copy engines around the
    # frame's CUDA graph)
    hl = [torch.from_numpy(p[0]).pin_memory().numpy() for p in pairs]
    hr = [torch.from_numpy(p[1]).pin_memory().numpy() for p in pairs]
    ho = [torch.empty((H, W), dtype=torch.uint8).pin_memory().numpy() for _ in range(2)]
    e2e_steps = max(3, min(args.steps, 200))
    for i in range(3):
        eng.run_frame(hl[i % R], hr[i % R], out=ho[i % 2])
    if dist is not None:
        dist.barrier()
    t0 = time.perf_counter()
    lat = []
    for i in range(e2e_steps):
        a = time.perf_counter()
        eng.run_frame(hl[i % R], hr[i % R], out=ho[i % 2])
        lat.append(time.perf_counter() - a)
    e2e_s = max_over_ranks(time.perf_counter() - t0, dist, dev)
    e2e_value = replica_value(ws, e2e_steps, e2e_s)
    ho[0][:] = 0
    eng.run_frame(hl[0], hr[0], out=ho[0])
    e2e_exact = bool(np.array_equal(ho[0], maps0[0]))   # the map that came back is the timed frame's map
    _, st = eng.run_frame(hl[0], hr[0], times=True, out=ho[1])   # a call that measures its stage times
    e2e_exact = e2e_exact and bool(np.array_equal(ho[1], maps0[0]))

    # the drop-in exactly as the reference harness calls it (common/harness.c:
    # 142-158): the plugin's SGM_IMPL.run on ordinary pageable buffers, with a
    # fresh zeroed map per call, so the copies go through the copy engines
    plug = sgmgb.Plugin(D, PATHS)
    pl = [np.array(p[0]) for p in pairs]
    pr = [np.array(p[1]) for p in pairs]
    for i in range(3):
        plug.run(pl[i % R], pr[i % R])
    if dist is not None:
        dist.barrier()
    lat_pg = []
    t0 = time.perf_counter()
    for i in range(e2e_steps):
        a = time.perf_counter()
        rc, pmap, _ = plug.run(pl[i % R], pr[i % R])
        lat_pg.append(time.perf_counter() - a)
        if rc:
            raise RuntimeError("SGM_IMPL.run failed")
    pg_s = max_over_ranks(time.perf_counter() - t0, dist, dev)
    pg_exact = bool(np.array_equal(plug.run(pl[0], pr[0])[1], maps0[0]))

    # per-kernel device time, each kernel alone, CUDA events on the engine's
    # stream: the fused schedule (`value`) and the one of a frame alone (`e2e`)
    eng.set_schedule(sgmgb.SCHED_FUSED)
    kstats = eng.profile_frame(dl[0], dr[0], dd[0], reps=20)
    eng.set_schedule(alone)
    kstats_lat = eng.profile_frame(dl[0], dr[0], dd[0], reps=20)
    eng.set_schedule(sgmgb.SCHED_AUTO)

    if rank != 0:
        for e in engines:
            e.close()
        if dist is not None:
            dist.destroy_process_group()
        return 0
    peak, peak_kind = peaks()
    top = max(kstats, key=lambda k: k[1])
    achieved = top[2] / (top[1] / 1e3) / 1e9
    traffic = committed_traffic(top[0])
    top_inst = committed_profile("instructions", top[0])
    frame_inst = sum(committed_profile("instructions", k[0]) or 0 for k in kstats) or None
    frame_traffic = sum(committed_traffic(k[0]) or 0 for k in kstats) or None
    clk = clocks.summary(tw0, tw1)
    issue_peak = 4 * torch.cuda.get_device_properties(dev).multi_processor_count * (clk["sm_mhz"] or 2070.0) * 1e6
    frame_ms_alone = sum(k[1] for k in kstats)
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_per_step, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "u16", "data": "synthetic",
        "config": workload_config(ws),
        "run": {"frames_in_flight": NF, "schedule": "fused (frames in flight)",
                "inputs": "resident on the device; per-frame working set 570 MB > L2"},
        "frame_latency_ms": serial_ms_per_frame,
        "fps": ws * args.steps / (ms / 1e3),
        "bit_exact": None,
        "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": 2 * W * H, "d2h_bytes_per_step": W * H,
                "fps": ws * e2e_steps / e2e_s, "p50_ms": statistics.median(lat) * 1e3,
                "p99_ms": sorted(lat)[min(len(lat) - 1, int(0.99 * len(lat)))] * 1e3,
                "stage_ms": {k: round(v, 4) for k, v in st.items() if k.endswith("_ms")},
                "schedule": SCHED_NAMES.get(alone, "?") + " (auto: fastest for a frame alone, timed at the "
                            "first call)",
                "transfers": "pinned host buffers: both images copied in and the map copied back by the copy "
                             "engines, the frame between them one CUDA graph, inside the call",
                "same_map_as_device_path": e2e_exact,
                "pageable": {"value": replica_value(ws, e2e_steps, pg_s), "unit": UNIT,
                             "fps": ws * e2e_steps / pg_s, "p50_ms": statistics.median(lat_pg) * 1e3,
                             "p99_ms": sorted(lat_pg)[min(len(lat_pg) - 1, int(0.99 * len(lat_pg)))] * 1e3,
                             "h2d_bytes_per_step": 2 * W * H, "d2h_bytes_per_step": W * H,
                             "call": "SGM_IMPL.run of libsgm_gb300_d64_p4.so, pageable numpy buffers, a new "
                                     "zeroed map per call, as common/harness.c:142-158",
                             "same_map_as_device_path": pg_exact},
                "kernels_alone_ms": {k[0]: round(k[1], 5) for k in kstats_lat}},
        "roofline": {"bound": "hbm", "kernel": top[0], "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "traffic": traffic, "algorithmic_bytes": top[2],
                     "launch_ms": top[1],
                     "note": "dominant kernel of the fused-schedule frame (longest mean launch, timed alone "
                             "with CUDA events); "
                             "achieved = its algorithmic bytes per launch / that time; peak = %s HBM copy "
                             "bandwidth; traffic = ncu dram bytes of one launch (profiles/)" % peak_kind},
        "frame_roofline": {"modelled_bytes": B_ALG, "achieved": B_ALG / (ms_per_step / 1e3) / 1e9,
                           "frac": B_ALG / (ms_per_step / 1e3) / 1e9 / peak, "unit": "GB/s",
                           "measured_bytes": frame_traffic,
                           "measured_over_modelled": frame_traffic / B_ALG if frame_traffic else None,
                           "measured_frac": (frame_traffic / (ms_per_step / 1e3) / 1e9 / peak) if frame_traffic
                           else None,
                           "note": "B_alg = 2*W*H*D + 3*W*H over the pipelined frame time (ms_per_step); "
                                   "measured_bytes: ncu dram bytes of one frame's kernels (profiles/)"},
        "issue_roofline": {"kernel": top[0], "warp_instructions": top_inst,
                           "achieved": top_inst / (top[1] / 1e3) if top_inst else None,
                           "peak": issue_peak, "unit": "warp-instructions/s",
                           "frac": top_inst / (top[1] / 1e3) / issue_peak if top_inst else None,
                           "frame_warp_instructions": frame_inst,
                           "frame_frac": frame_inst / (ms_per_step / 1e3) / issue_peak if frame_inst else None,
                           "note": "the recurrence is 8/16-bit integer work on the issue slots: peak = 4 schedulers "
                                   "x SMs x the SM clock sampled in the timed region; instructions from ncu "
                                   "(profiles/), time from the live CUDA-event timing"},
        "kernels": [{"name": k[0], "ms": round(k[1], 5), "algorithmic_bytes": k[2],
                     "gbs": round(k[2] / (k[1] / 1e3) / 1e9, 1)} for k in kstats],
        "frame_ms_kernels_alone": frame_ms_alone,
        "cpu_baseline": None,
        "clocks": clk,
        "gpu_launches": args.steps * KERNELS_PER_FRAME,
    }
    for e in engines:
        e.close()
    ms_checks, batch_checks = (), ()
    if not args.no_multiscale:
        line["multiscale"], ms_checks = multiscale_section(sgmgb, torch, np)
    if not args.no_sweep:
        line["d_sweep"] = sweep_section(sgmgb, torch, np)
    if not args.no_batch:
        line["batched"], batch_checks = batched_section(sgmgb.Engine, sgmgb, torch, np)
    if not args.no_serve:
        line["served"] = served_section(sgmgb.Engine, sgmgb, np)
    base, exact, ms_res, batch_res = cpu_baseline_sample(args.cpu_seconds, pairs[0][0], pairs[0][1], maps0,
                                                         ms_checks, batch_checks)
    line["cpu_baseline"] = base
    line["bit_exact"] = {"value": exact, "checker": base["kind"],
                         "what": "every timed context's map of the first pair vs the checker's map"}
    for name, r in ms_res.items():
        line["multiscale"][name].update(r)
    if batch_res is not None:
        line["batched"]["reference_check"] = batch_res
    print(json.dumps(line))
    if dist is not None:
        dist.destroy_process_group()
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=2000)
    ap.add_argument("--warmup", type=int, default=50)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--cpu-seconds", type=float, default=12.0)
    ap.add_argument("--warps-per-block", type=int, default=4, help="path-kernel shape (speed only)")
    ap.add_argument("--disp-per-lane", type=int, default=0, help="path-kernel shape: 0, 2, 4 or 8")
    ap.add_argument("--inflight", type=int, default=4,
                    help="frames in flight in the timed region (contexts and streams, round-robin)")
    ap.add_argument("--no-batch", action="store_true", help="skip the batched-form section")
    ap.add_argument("--no-multiscale", action="store_true", help="skip the configurations B/C section")
    ap.add_argument("--no-serve", action="store_true", help="skip the served-form section")
    ap.add_argument("--no-sweep", action="store_true", help="skip the D x resolution grid")
    ap.add_argument("--no-refgpu", action="store_true",
                    help="reference arm: skip the reference's own CUDA programs on this GPU")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.inflight not in (1, 2, 4, 8):
        ap.error("--inflight must be 1, 2, 4 or 8")
    if args.impl == "reference":
        return run_reference(args)
    return run_gb300(args)


if __name__ == "__main__":
    sys.exit(main())
