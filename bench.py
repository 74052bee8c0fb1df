#!/usr/bin/env python3
"""Benchmark of the two-level voxelizer (prints one JSON line on rank 0).

Default workload (one step = one voxelization of one mesh through the plain path): the largest
plain configuration,
  star1310k -- star surface r = 0.3(1 + 0.2 sum a_lm Y_lm), l <= 6, on an icosphere subdivided 8
               times (1,310,720 triangles), scaled 1:1:6 in z; Level1 256^3 over the mesh box
               padded by one cell, Level2 16^3 per boundary voxel.  Seeded synthetic data.
(--workload sphere16k / torus262k run the two smaller plain configurations.)

value    reference-equivalent tri-voxel tests/s on device-resident triangles (results stay on the
         device), timed with CUDA events on the launching stream; L2 is flushed (256 MiB write)
         between steps, outside the timed spans.
e2e      the same metric through the public host API (gpv_voxelize_to_host): H2D of the step's
         triangles from pinned memory, voxelization, D2H of every result array into pinned
         buffers, timed on the host around each step.
tests    = sat1 + sat2 + ray1 + ray2: the tests the reference's algorithm performs on the mesh,
         counted by its definitions (include/gpview.h, gpv_work).  The kernels decide many of them
         in groups without evaluating each, so this is a reference-equivalent rate, not the
         number of predicate evaluations the GPU executes.

--impl reference times the reference's CPU path (the oracle restatement, all host threads) on a
bounded sample of the same workload and reports the same metric and config.  It generates the
mesh with the oracle library's build of the same generator source and never loads the GPU library.
Multi-GPU: replicas only (each rank voxelizes its own copy; the path has no exchange step).
"""
import argparse
import faulthandler
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "tests"))


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=10)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="gpv", choices=["gpv", "reference"])
    p.add_argument("--workload", default="star1310k", choices=["sphere16k", "torus262k", "star1310k"])
    p.add_argument("--tile", type=int, default=0)
    p.add_argument("--level2", type=int, default=0, help="override the workload's Level2 divisions")
    p.add_argument("--chunk", type=int, default=0, help="Level2 chunk of the plain path (0: default)")
    p.add_argument("--level2-mode", default="auto", choices=["auto", "queued", "inline"],
                   help="Level2 SAT organisation of the plain path (default: chosen per launch)")
    p.add_argument("--no-graphs", action="store_true")
    p.add_argument("--slabs", type=int, default=0,
                   help="z slabs of the e2e path's Level2 launch (0: by the Level2 output size)")
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--no-stencil", action="store_true", help="skip the stencil-fill section")
    p.add_argument("--no-shims", action="store_true", help="skip the reference-named shim section")
    p.add_argument("--cpu-seconds", type=float, default=15.0,
                   help="CPU-baseline budget of the GPU arm (the reference arm uses --ref-step-seconds)")
    p.add_argument("--ref-step-seconds", type=float, default=3.0,
                   help="CPU seconds per step of the reference arm's bounded sample")
    p.add_argument("--no-as-written", action="store_true",
                   help="skip the one-thread reference-as-written CPU estimate")
    p.add_argument("--as-written-seconds", type=float, default=12.0)
    p.add_argument("--stencil-cpu", action="store_true",
                   help="also time the oracle's stencil-fill restatement on the host")
    p.add_argument("--batch", type=int, default=4096, help="meshes of the batched workload (0: skip)")
    p.add_argument("--batch-reps", type=int, default=3)
    p.add_argument("--batch-tile", type=int, default=0, help="fixed Level1 tile (0: autotune)")
    p.add_argument("--batch-chunk", type=int, default=0, help="fixed Level2 chunk (0: autotune)")
    p.add_argument("--serve-seconds", type=float, default=60.0, help="served stream length (0: skip)")
    p.add_argument("--serve-pool", type=int, default=256)
    p.add_argument("--serve-rate", type=float, nargs=2, default=(100.0, 5000.0))
    p.add_argument("--serve-tight-seconds", type=float, default=15.0,
                   help="length of the stream under a binding budget (0: skip)")
    p.add_argument("--serve-tight-gb", type=float, default=2.0)
    return p.parse_args()


WORKLOADS = {
    "sphere16k": dict(name="sphere16k", level1=64, level2=4,
                      desc="UV-sphere r=0.4, 128x64 segments, 16,128 triangles, 64^3 / 4^3"),
    "torus262k": dict(name="torus262k", level1=128, level2=8,
                      desc="noisy torus R=0.35 r=0.12, 512x256 segments, 262,144 triangles, 128^3 / 8^3"),
    "star1310k": dict(name="star1310k", level1=256, level2=16,
                      desc="Y_lm star on an 8x subdivided icosphere, 1,310,720 triangles, 1:1:6, 256^3 / 16^3"),
}


class Clocks:
    """nvidia-smi sampling during the timed region."""

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.path = None

    def start(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={q}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        out = {"sm_mhz": None, "sm_max_mhz": None, "reasons": []}
        if not self.proc:
            return out
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sms, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sms.append(float(f[1]))
                mx = float(f[2])
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        os.unlink(self.path)
        out["sm_mhz"] = statistics.median(sms) if sms else None
        out["sm_max_mhz"] = mx
        out["reasons"] = sorted(reasons)
        out["samples"] = len(sms)
        return out


def load_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return json.load(f), "measured"
    except Exception:
        return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "sm_max_mhz": 2070.0}, "fallback"


METRIC = "tri-voxel tests/s (reference-equivalent)"
L2_FLUSH = ("GPU arm: a 256 MiB write between steps, outside the timed spans; "
            "the CPU reference arm has no flush")


def workload_config(cfg, T):
    """The config dict both arms print (identical for the same workload)."""
    return {"workload": cfg["name"], "desc": cfg["desc"], "triangles": int(T),
            "level1": cfg["level1"], "level2": cfg["level2"], "parallelism": "replicas",
            "l2_flush": L2_FLUSH}


def cpu_work(tris, grid, threads):
    """(oracle run, tests per mesh): the reference algorithm's sat1 + ray1 + sat2 + ray2 on the
    mesh, by the oracle's counts (the same definitions the library's gpv_work uses)."""
    from oracle import oracle as orc

    run = orc.Run(tris, grid, fill=orc.FILL_CAND, threads=threads)
    s2, r2 = run.level2_work(threads)
    return run, run.sat1_tests() + run.ray1_candidates() + s2 + r2


def _level2_sample(run, seconds, threads):
    """Level2 of the oracle on an evenly strided sample of the boundary voxels (every part of the
    mesh represented), in one parallel pass per round: a first round of 64 voxels per thread
    measures the cost per voxel, a second round fills the rest of the budget.  Returns (seconds,
    voxels done)."""
    import numpy as np

    B = run.B
    if B == 0:
        return 0.0, 0
    spent, done = 0.0, 0
    n = min(B, 64 * max(threads, 1))
    for rnd in range(2):
        if n <= 0:
            break
        # offset the second round by half a stride so that the two samples interleave
        pick = ((np.arange(n, dtype=np.int64) * B) // n + (rnd * B) // (2 * n)) % B
        pick = np.unique(pick)
        t0 = time.perf_counter()
        run.level2_list(pick, threads)
        spent += time.perf_counter() - t0
        done += pick.size
        per = spent / done
        n = min(B - done, int(max(seconds - spent, 0.0) / per))
    return spent, done


def cpu_sample(tris, grid, work_total, seconds, threads, run=None):
    """One bounded sample of the reference's CPU path as the oracle port restates it, on all
    host threads: Level1 in full (ClassifyTessellation + the candidate-list parity fill) and
    Level2 on an evenly strided sample of the boundary voxels sized to the budget, extrapolated
    to the whole mesh."""
    from oracle import oracle as orc

    t0 = time.perf_counter()
    run = orc.Run(tris, grid, fill=orc.FILL_CAND, threads=threads)
    t_l1 = time.perf_counter() - t0
    t_l2, done = _level2_sample(run, max(seconds - t_l1, 0.2), threads)
    t_full = t_l1 + (t_l2 * run.B / done if done else 0.0)
    return {"value": work_total / t_full, "unit": "tests/s", "cores": threads, "kind": "port",
            "sample": f"Level1 in full + Level2 on an evenly strided sample of {done}/{run.B} "
                      f"boundary voxels, extrapolated ({t_l1 + t_l2:.1f} s of CPU work, "
                      f"est. {t_full:.2f} s per mesh)",
            "sec_per_mesh": t_full}


def cpu_as_written(tris, grid, work_total, seconds, seed=7):
    """The reference's CPU path as it is written, on ONE thread (the reference-as-written baseline):
    ClassifyTessellation and the compaction (timed in full), ClassifyInOutCPU's brute force --
    every voxel centre against every triangle -- on a seeded sample of Level1 columns, and the
    Level2 passes on an evenly strided sample of boundary voxels; the two sampled parts are extrapolated
    to the whole mesh."""
    import numpy as np
    from oracle import oracle as orc

    t0 = time.perf_counter()
    run = orc.Run(tris, grid, fill=orc.FILL_CAND, threads=1)
    t_l1 = time.perf_counter() - t0
    nx, ny = int(run.spec.n[0]), int(run.spec.n[1])
    rng = np.random.default_rng(seed)
    order = rng.permutation(nx * ny)
    t_fill, ncol, k = 0.0, 0, 1
    while t_fill < seconds / 2 and ncol < order.size:
        cols = order[ncol:ncol + k]
        t1 = time.perf_counter()
        run.voxel_fill_columns(cols)
        t_fill += time.perf_counter() - t1
        ncol += cols.size
        k *= 2
    t_l2, done = _level2_sample(run, seconds / 2, 1)
    t_full = t_l1 + t_fill * (nx * ny) / ncol + (t_l2 * run.B / done if done else 0.0)
    return {"value": work_total / t_full, "unit": "tests/s", "cores": 1, "kind": "port",
            "sec_per_mesh": t_full,
            "sample": f"one thread: Level1 SAT + compaction in full ({t_l1:.1f} s), the brute-force "
                      f"parity fill on {ncol}/{nx * ny} seeded columns ({t_fill:.1f} s), Level2 on "
                      f"{done}/{run.B} boundary voxels ({t_l2:.1f} s); extrapolated"}


def batch_bench(gpv, ctx, torch, stream, local, args):
    """The 4096-mesh mixed workload: plain one-mesh-per-launch path vs the batched path."""
    import numpy as np

    import workloads as W

    t0 = time.perf_counter()
    meshes = W.batch4096(args.batch)
    gen_s = time.perf_counter() - t0
    progress(f"batch generated ({len(meshes)} meshes, {gen_s:.1f} s)")
    counts = [t.size // 9 for t, _ in meshes]
    specs = [s for _, s in meshes]
    offs, o = [], 0
    for c in counts:
        offs.append(o)
        o += (c * 9 + 3) // 4 * 4  # keep every mesh 16-byte aligned
    host = np.zeros(max(o, 4), np.float32)
    for (t, _), off in zip(meshes, offs):
        host[off:off + t.size] = t
    dev = torch.from_numpy(host).to(f"cuda:{local}")
    ptrs = [dev.data_ptr() + 4 * off for off in offs]
    sp = stream.cuda_stream
    with torch.cuda.stream(stream):
        if args.batch_tile and args.batch_chunk:
            tile, chunk, tune_ms = args.batch_tile, args.batch_chunk, 0.0
            ctx.set_tile(tile)
            ctx.set_level2_chunk(chunk)
        else:
            # autotuner on a sample of the batch
            ns = min(256, len(ptrs))
            tile, chunk, tune_ms = ctx.autotune(ptrs[:ns], counts[:ns], specs[:ns], sp)
            progress(f"autotuned: tile {tile}, chunk {chunk}")
        # plain path: one voxelization (full launch sequence, host syncs) per mesh
        torch.cuda.synchronize()
        tp = time.perf_counter()
        work = 0
        for p_, c, s_ in zip(ptrs, counts, specs):
            r = ctx.voxelize_device(p_, c, s_, sp)
            work += r.work.total()
            ctx.release(r)
        torch.cuda.synchronize()
        plain_s = time.perf_counter() - tp
        progress(f"plain loop {plain_s:.2f} s")
        # batched path: the first call runs as two graphs and records the sizes; the repeated
        # calls are one graph each (and the same calls as two graphs, for comparison)
        def batched_calls():
            ts, w = [], 0
            for k in range(args.batch_reps + 1):
                torch.cuda.synchronize()
                tb = time.perf_counter()
                res = ctx.voxelize_batch(ptrs, counts, specs, sp)
                torch.cuda.synchronize()
                dt = time.perf_counter() - tb
                w = sum(r.work.total() for r in res)
                for r in res:
                    ctx.release(r)
                if k > 0:
                    ts.append(dt)
            return ts, w

        og0 = ctx.get_debug("one_graph_calls")
        times, bwork = batched_calls()
        og_calls = ctx.get_debug("one_graph_calls") - og0
        ctx.set_graphs(ctx.GRAPHS_TWO)
        times2, bwork2 = batched_calls()
        ctx.set_graphs(True)
        assert bwork2 == bwork, (bwork2, bwork)
        # one more call with host timing on: where the host time of a batch call goes
        ctx.set_timing(True)
        for r in ctx.voxelize_batch(ptrs, counts, specs, sp):
            ctx.release(r)
        torch.cuda.synchronize()
        hcalls, host_ms = ctx.host_times()
        ctx.set_timing(False)
    batch_s = sum(times) / len(times)
    assert bwork == work, (bwork, work)
    n = len(meshes)
    return {"workload": "batch4096", "meshes": n, "triangles": int(sum(counts)),
            "desc": "sphere/noisy torus/superellipsoid, T log-uniform 500-200000, Level1 {32..128}^3, Level2 {2,4,8}^3",
            "tile": tile, "level2_chunk": chunk, "autotune_sample_ms": tune_ms,
            "plain_meshes_per_s": n / plain_s, "batched_meshes_per_s": n / batch_s,
            "batched_graphs": f"one CUDA graph per call ({og_calls} of {args.batch_reps + 1} calls; "
                              "the first records the sizes as two graphs)",
            "batched_two_graph_meshes_per_s": n / (sum(times2) / len(times2)),
            "batched_vs_plain": plain_s / batch_s, "batched_tests_per_s": work / batch_s,
            "plain_s": plain_s, "batched_s": batch_s, "generate_s": gen_s,
            "batched_host_ms_per_call": {k: v / max(hcalls, 1) for k, v in host_ms.items()}}


def poisson_schedule(D, r0, r1, seed):
    """Arrival times of an open-loop Poisson stream whose rate ramps linearly from r0 to r1 over
    D seconds (thinning of a rate-r1 process)."""
    import numpy as np

    rng = np.random.default_rng(seed)
    sched, t = [], 0.0
    while True:
        t += rng.exponential(1.0 / r1)
        if t >= D:
            break
        if rng.random() < (r0 + (r1 - r0) * t / D) / r1:
            sched.append(t)
    return sched, rng


def serve_stream(srv, submit, n_pool, D, r0, r1, seed, shed_limit=2000):
    """Drives one stream against a server: submit(k) enqueues pool mesh k.  A collector thread
    polls and releases results in submission order.  Returns the per-request records and the
    stream's wall time; requests are shed (not submitted) while more than shed_limit wait."""
    import threading
    from collections import deque

    sched, rng = poisson_schedule(D, r0, r1, seed)
    picks = rng.integers(0, n_pool, len(sched))
    q = deque()
    done = []
    shed = [0]
    peak = [0]
    finished = threading.Event()

    def collector():
        while True:
            if not q:
                if finished.is_set():
                    return
                time.sleep(0.0005)
                continue
            tk, ts = q.popleft()
            rc, _, lat, qms = srv.poll(tk, -1)
            done.append((ts, lat, qms, rc))
            srv.release(tk)

    col = threading.Thread(target=collector)
    col.start()
    start = time.perf_counter()
    for ts, k in zip(sched, picks):
        now = time.perf_counter() - start
        if ts > now:
            time.sleep(ts - now)
        st = srv.stats()
        peak[0] = max(peak[0], st["in_use_bytes"])
        if st["pending"] > shed_limit:
            shed[0] += 1
            continue
        tk = submit(int(k))
        if tk is not None:
            q.append((tk, ts))
    finished.set()
    col.join()
    return done, time.perf_counter() - start, len(sched), shed[0], peak[0]


def stream_summary(done, wall, offered, shed, D, r0, r1, nbins=6):
    import numpy as np

    lat = np.array([d[1] for d in done if d[3] == 0])
    ts = np.array([d[0] for d in done if d[3] == 0])
    pct = lambda x, p: float(np.percentile(x, p)) if len(x) else None  # noqa: E731
    bins = []
    for b in range(nbins):
        lo, hi = b * D / nbins, (b + 1) * D / nbins
        m = (ts >= lo) & (ts < hi)
        if m.any():
            bins.append({"rate_req_s": round(r0 + (r1 - r0) * (lo + hi) / 2 / D),
                         "completed": int(m.sum()), "p50_ms": pct(lat[m], 50),
                         "p95_ms": pct(lat[m], 95), "p99_ms": pct(lat[m], 99)})
    return {"offered": offered, "shed": shed, "completed": int(len(lat)),
            "failed": int(sum(1 for d in done if d[3] != 0)), "meshes_per_s": len(lat) / wall,
            "p50_ms": pct(lat, 50), "p95_ms": pct(lat, 95), "p99_ms": pct(lat, 99),
            "queue_p50_ms": pct([d[2] for d in done], 50), "by_rate": bins}


def served_bench(gpv, torch, local, args, tuned):
    """Open-loop Poisson streams against the continuous-batching server; latency = submit to
    results on the device.
      main stream  -- rate ramped 100 -> 5,000 req/s over 60 s, 150 GB budget, the pool's meshes
                      resident on the device (uploaded once, requested by id);
      plain        -- the same pool voxelized one call per mesh on one context (the comparator);
      tight budget -- a shorter stream of host-triangle requests (copied in per request) under a
                      2 GB budget, where admission by predicted footprint binds."""
    import workloads as W

    pool = W.served_pool(args.serve_pool)
    specs = [s for _, s in pool]
    D = args.serve_seconds
    r0, r1 = args.serve_rate
    out = {"workload": "served", "duration_s": D, "rate_req_s": [r0, r1],
           "desc": "Poisson stream, rate ramped linearly; pool of %d meshes (3 families, T log-uniform "
                   "1e3-1e6, Level1 {64,128,256}^3, Level2 {4,8}^3); 150 GB budget; 2 workers; meshes "
                   "resident in the server's device pool" % len(pool)}
    # the comparator: one plain call per pool mesh, device-resident triangles
    dev = [torch.from_numpy(t).to(f"cuda:{local}") for t, _ in pool]
    ctx = gpv.Context(local)
    for d, (t, s) in list(zip(dev, pool))[:8]:
        ctx.release(ctx.voxelize_device(d.data_ptr(), t.size // 9, s))
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for d, (t, s) in zip(dev, pool):
        ctx.release(ctx.voxelize_device(d.data_ptr(), t.size // 9, s))
    torch.cuda.synchronize()
    out["plain_meshes_per_s"] = len(pool) / (time.perf_counter() - t0)
    ctx.close()
    del dev
    # main stream, resident meshes
    srv = gpv.Server(local, budget_bytes=150 << 30, workers=2, max_batch=256)
    srv.set_tunables(*tuned)
    ids = [srv.add_mesh(t) for t, _ in pool]
    out["pool_bytes"] = int(sum(t.size * 4 for t, _ in pool))
    for i in range(8):  # warm-up
        tk = srv.submit_mesh(ids[i], specs[i])
        srv.poll(tk, -1)
        srv.release(tk)
    done, wall, offered, shed, peak = serve_stream(srv, lambda k: srv.submit_mesh(ids[k], specs[k]),
                                                  len(pool), D, r0, r1, 77)
    out["batches"] = srv.stats()["batches"]
    srv.close()
    out.update(stream_summary(done, wall, offered, shed, D, r0, r1))
    out["peak_in_use_gb"] = peak / 2**30
    out["served_vs_plain"] = out["meshes_per_s"] / out["plain_meshes_per_s"]
    # a budget that binds: admission by predicted footprint, host triangles copied per request
    if args.serve_tight_seconds > 0:
        pinned = [torch.from_numpy(t).pin_memory() for t, _ in pool]
        budget = int(args.serve_tight_gb * 2**30)
        srv = gpv.Server(local, budget_bytes=budget, workers=2, max_batch=256)
        srv.set_tunables(*tuned)
        Dt = args.serve_tight_seconds
        refused = [0]

        def submit(k):
            # a request whose predicted footprint exceeds the whole budget is refused at submit
            try:
                return srv.submit(pinned[k], specs[k])
            except gpv.GpvError:
                refused[0] += 1
                return None

        done, wall, offered, shed, peak = serve_stream(srv, submit, len(pool), Dt, 500.0, 500.0, 78)
        tight = stream_summary(done, wall, offered, shed, Dt, 500.0, 500.0, nbins=3)
        tight.update({"budget_gb": budget / 2**30, "duration_s": Dt, "rate_req_s": 500.0,
                      "peak_in_use_gb": peak / 2**30, "batches": srv.stats()["batches"],
                      "refused_as_oversize": refused[0]})
        srv.close()
        out["tight_budget"] = tight
    return out


def run_reference(args):
    """The reference arm: the reference's CPU path (oracle port, all host threads), rank 0 only.
    Each step is one bounded sample (Level1 in full, Level2 on an evenly strided sample of
    boundary voxels), extrapolated to the mesh; value = tests per mesh / mean extrapolated seconds."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    import workloads as W

    cfg = WORKLOADS[args.workload]
    if args.level2:
        cfg = dict(cfg, level2=args.level2)
    tris, grid = W.make(cfg, cpu=True)  # the oracle's generator build: no GPU library loaded
    threads = os.cpu_count() or 1
    _, work_total = cpu_work(tris, grid, threads)
    times = []
    base = None
    for step in range(args.warmup + args.steps):
        base = cpu_sample(tris, grid, work_total, args.ref_step_seconds, threads)
        if step >= args.warmup:
            times.append(base["sec_per_mesh"])
    t = sum(times) / len(times)
    value = work_total / t
    line = {"metric": METRIC, "value": value, "unit": "tests/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": t * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic", "impl": "reference",
            "config": workload_config(cfg, tris.size // 9),
            "tests_per_mesh": work_total,
            "cpu_baseline": {"value": value, "unit": "tests/s", "cores": threads, "kind": "port",
                             "sample": "per step: " + base["sample"]},
            "e2e": {"value": value, "unit": "tests/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    if not args.no_as_written:
        aw = cpu_as_written(tris, grid, work_total, args.as_written_seconds)
        line["cpu_as_written"] = {k: v for k, v in aw.items()}
    print(json.dumps(line))


# Warp instructions one launch of the Level2 kernel executes on each single-mesh workload, from
# a one-launch capture `ncu --metrics smsp__inst_executed.sum,dram__bytes_read.sum,
# dram__bytes_write.sum -k regex:k_level2c -c 1` of this bench on that workload.  The count is a
# property of the kernel's code and the input, not of the clock; it is re-captured whenever the
# kernel changes.
LEVEL2_INST_PER_LAUNCH = {"star1310k": 3465057518, "torus262k": 330108311, "sphere16k": 24003464}
# DRAM bytes read + written by one launch of the Level2 kernel (same captures)
LEVEL2_TRAFFIC = {"star1310k": 128589568 + 1140417024, "torus262k": 30649344 + 4477440,
                  "sphere16k": 2835456 + 0}


def max_over_ranks(seconds, dist, device):
    """Replicas: every rank voxelizes its own copy; the job's time is the slowest rank's."""
    if not dist:
        return seconds
    import torch

    t = torch.tensor([seconds], device=device, dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_value(tests_per_step, steps, world, seconds):
    """Whole-job throughput: the tests all ranks processed over the slowest rank's time."""
    return tests_per_step * steps * world / seconds


def roofline(name, per_call, work, stats, spec, T, peaks, peak_kind, clk):
    """Roofline of the dominant kernel, k_level2c.

    bound "issue": the kernel's throughput is set by instruction issue (4 warp-instructions per
    clock per SM), not by DRAM (it moves ~36 MB per 1 ms launch) and not by one math pipe.
    achieved = warp instructions per launch / the kernel's CUDA-event duration in this run;
    peak = 4 x 152 SMs x the maximum SM clock in MEASURED_PEAKS.json.
    "algorithmic" states the same launch in the reference's terms: the FP32 operations the
    reference's predicates execute on the launch's sat2 + ray2 tests (early exits included,
    per-test averages from tests/golden/op_counts.json) per second, against the FP32 peak
    (128 lanes x 152 SMs x maximum clock).  It exceeds 1 because the kernel decides groups of the
    reference's tests without evaluating each one (plane-slab ranges, column-shared u/v and
    certified parity toggles), so it measures the algorithm, not the hardware use."""
    sm_mhz = float(peaks.get("sm_max_mhz", 2070.0))
    n_sms = 152
    ms = per_call.get("level2_kernel") or per_call.get("level2", 0.0)
    out = {"kernel": "k_level2c", "bound": "issue", "unit": "Gwarp-inst/s",
           "peak": 4 * n_sms * sm_mhz * 1e6 / 1e9, "peak_source":
           f"derived: 4 warp-inst/clk/SM x {n_sms} SMs x sm_max_mhz {sm_mhz:g} ({peak_kind})",
           "kernel_ms": ms, "stage_ms_per_step": per_call}
    inst = LEVEL2_INST_PER_LAUNCH.get(name)
    if inst and ms > 0:
        out["achieved"] = inst / (ms / 1e3) / 1e9
        out["frac"] = out["achieved"] / out["peak"]
        out["inst_per_launch"] = inst
    else:
        out["achieved"] = out["frac"] = None
    cells = spec.ndiv2[0] * spec.ndiv2[1] * spec.ndiv2[2]
    B, P = stats["boundary"], stats["pairs"]
    # DRAM bytes per launch from the ncu capture of the same kernel and workload; the
    # algorithmic bytes are the sorted pairs read once, the triangles (48 B of prepared
    # vertices) gathered once per pair and the Level2 blocks written once.
    out["traffic"] = LEVEL2_TRAFFIC.get(name)
    out["algorithmic_bytes"] = P * 8 + P * 48 + B * cells
    try:
        with open(os.path.join(ROOT, "tests", "golden", "op_counts.json")) as f:
            oc = json.load(f)[name]
        ops = sum(oc[k]["ops"] / oc[k]["tests"] * w for k, w in (("sat2", work[1]), ("ray2", work[3]))
                  if oc[k]["tests"])
        fp32_peak = 128 * n_sms * sm_mhz * 1e6 / 1e12
        out["algorithmic"] = {"ref_fp32_ops_per_launch": ops, "achieved_tops": ops / (ms / 1e3) / 1e12,
                              "fp32_peak_tops": fp32_peak,
                              "frac_of_fp32_peak": ops / (ms / 1e3) / 1e12 / fp32_peak if ms else None}
    except (OSError, KeyError, ZeroDivisionError):
        out["algorithmic"] = None
    return out


def stencil_bench(gpv, ctx, torch, stream, step_device, flush, args, tris, spec, cpu):
    """The same workload with the rasterised stencil fill (GPV_FILL_STENCIL) instead of the ray
    fill: device time per step and per stage, and (cpu) the oracle's restatement on the host."""
    ctx.set_fill(gpv.FILL_STENCIL)
    try:
        with torch.cuda.stream(stream):
            for _ in range(args.warmup):
                ctx.release(step_device())
        torch.cuda.synchronize()
        ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
              for _ in range(args.steps)]
        torch.cuda.synchronize()
        with torch.cuda.stream(stream):
            for k in range(args.steps):
                flush.zero_()
                ev[k][0].record(stream)
                r = step_device()
                ev[k][1].record(stream)
                if k == 0:
                    counts = dict(l1_inside=r.num_level1_inside, l2_inside=r.num_level2_inside,
                                  l2_boundary=r.num_level2_boundary)
                ctx.release(r)
        torch.cuda.synchronize()
        # the stage breakdown from a second pass with the stage events on
        ctx.set_timing(True)
        with torch.cuda.stream(stream):
            for _ in range(2):
                ctx.release(step_device())
        torch.cuda.synchronize()
        ctx.set_timing(True)
        with torch.cuda.stream(stream):
            for k in range(args.steps):
                flush.zero_()
                ctx.release(step_device())
        torch.cuda.synchronize()
        calls, stage_ms = ctx.stage_times()
        ctx.set_timing(False)
    finally:
        ctx.set_fill(gpv.FILL_RAY)
    ms = sum(a.elapsed_time(b) for a, b in ev) / args.steps
    out = {"fill": "stencil (ClassifyInOut2x + ClassifyInOut2xLevel2 as CUDA kernels)",
           "ms_per_step": ms, "meshes_per_s": 1e3 / ms,
           "stage_ms_per_step": {k: v / max(calls, 1) for k, v in stage_ms.items()}, **counts}
    if cpu:
        from oracle import oracle as orc

        t0 = time.perf_counter()
        run = orc.Run(tris, spec, fill=orc.FILL_STENCIL, threads=os.cpu_count() or 1)
        run.level2_state(threads=os.cpu_count() or 1)
        out["cpu_oracle_s_per_mesh"] = time.perf_counter() - t0
        out["cpu_oracle_cores"] = os.cpu_count() or 1
    return out


def shim_bench(gpv, torch, local, args):
    """The reference-named shims driven as GPView's Object drives them, on the mid-size mesh
    (torus262k): CUDAClassifyTessellation into per-voxel id buffers sized to the largest count
    (src/Object.cpp:2116-2183), the host building the flat and column lists (:2146-2180,
    :2560-2577), then CUDAClassifyInOutLevel2 and CUDAClassifyTessellationLevel2 (:2603, :2606).
    Device time of each shim call (CUDA events on the legacy stream, warm), against the native
    call on the same mesh."""
    import ctypes as C

    import numpy as np

    import workloads as W
    from oracle import oracle as orc

    class F3(C.Structure):
        _fields_ = [("x", C.c_float), ("y", C.c_float), ("z", C.c_float)]

    class I3(C.Structure):
        _fields_ = [("x", C.c_int), ("y", C.c_int), ("z", C.c_int)]

    L = gpv.lib()
    vp = C.c_void_p
    L.CUDAClassifyTessellation.argtypes = [vp, C.c_int, vp, vp, vp, F3, F3, F3, I3, C.c_int]
    L.CUDAClassifyTessellationLevel2.argtypes = [vp, vp, vp, vp, vp, vp, vp, vp, C.c_int, I3, F3, F3]
    L.CUDAClassifyInOutLevel2.argtypes = [vp, vp, vp, vp, vp, vp, vp, C.c_int, I3, I3, F3, F3]
    dev = f"cuda:{local}"
    tris, spec = W.make(W.C2)
    T = tris.size // 9
    tab = orc.grid_tables(spec)  # the caller's float grid values (boxExtents, midpoints)
    nd = [int(v) for v in spec.ndiv]
    n2 = [int(v) for v in spec.ndiv2]
    N1 = int(np.prod(nd))
    cells = int(np.prod(n2))
    e1 = F3(*[float(v) for v in tab["e1"]])
    e2 = F3(*[float(v) for v in tab["e2"]])
    d_tris = torch.from_numpy(tris).to(dev)
    s0 = torch.cuda.default_stream(local)

    def timed(fn, reps=5):
        ms = []
        for k in range(reps + 1):
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(s0)
            fn()
            b.record(s0)
            torch.cuda.synchronize()
            if k:
                ms.append(a.elapsed_time(b))
        return sum(ms) / len(ms)

    with torch.cuda.stream(s0):
        inout = torch.zeros(N1, dtype=torch.float32, device=dev)
        cnt = torch.zeros(N1, dtype=torch.int32, device=dev)
        one = torch.zeros(N1, dtype=torch.int32, device=dev)
        L.CUDAClassifyTessellation(d_tris.data_ptr(), T, inout.data_ptr(), cnt.data_ptr(),
                                   one.data_ptr(), F3(*spec.bbox_min), F3(*spec.bbox_max), e1,
                                   I3(*nd), 1)
        buf = int(cnt.max().item())
        idx = torch.zeros(N1 * buf, dtype=torch.int32, device=dev)

        def level1():
            inout.zero_()
            cnt.zero_()
            L.CUDAClassifyTessellation(d_tris.data_ptr(), T, inout.data_ptr(), cnt.data_ptr(),
                                       idx.data_ptr(), F3(*spec.bbox_min), F3(*spec.bbox_max), e1,
                                       I3(*nd), buf)

        l1_ms = timed(level1)
        # the host lists the reference builds between the two levels
        c = cnt.cpu().numpy()
        ids = idx.cpu().numpy().reshape(N1, buf)
        keep = np.arange(buf)[None, :] < c[:, None]
        flat = ids[keep].astype(np.int32)
        flat_index = np.zeros(N1, np.int32)
        flat_index[1:] = np.cumsum(c)[:-1]
        bidx = np.nonzero(inout.cpu().numpy() == 2)[0].astype(np.int32)
        B = bidx.size
        col = (np.repeat(np.arange(N1), c) % (nd[0] * nd[1])).astype(np.int64)
        u = np.unique(col * T + flat)
        ucol, utri = u // T, (u % T).astype(np.int32)
        xcnt = np.bincount(ucol, minlength=nd[0] * nd[1]).astype(np.int32)
        xidx = np.zeros(nd[0] * nd[1], np.int32)
        xidx[1:] = np.cumsum(xcnt)[:-1]
        c1 = tab["c1"]
        ks, rem = np.divmod(bidx, nd[0] * nd[1])
        js, is_ = np.divmod(rem, nd[0])
        mid = np.stack([c1[is_], c1[nd[0] + js], c1[nd[0] + nd[1] + ks]], 1).astype(np.float32)
        t_mid, t_bi = torch.from_numpy(mid.reshape(-1)).to(dev), torch.from_numpy(bidx).to(dev)
        t_cnt, t_fi, t_fl = (torch.from_numpy(x).to(dev) for x in (c.astype(np.int32), flat_index, flat))
        t_xc, t_xi, t_xf = (torch.from_numpy(x).to(dev) for x in (xcnt, xidx, utri))
        l2 = torch.zeros(B * cells, dtype=torch.float32, device=dev)
        nrm = torch.zeros(B * cells * 4, dtype=torch.float32, device=dev)

        def level2_fill():
            l2.zero_()
            L.CUDAClassifyInOutLevel2(d_tris.data_ptr(), l2.data_ptr(), t_mid.data_ptr(), t_bi.data_ptr(),
                                      t_xc.data_ptr(), t_xi.data_ptr(), t_xf.data_ptr(), B, I3(*nd),
                                      I3(*n2), e1, e2)

        def level2_sat():
            nrm.zero_()
            L.CUDAClassifyTessellationLevel2(d_tris.data_ptr(), l2.data_ptr(), nrm.data_ptr(),
                                             t_mid.data_ptr(), t_bi.data_ptr(), t_cnt.data_ptr(),
                                             t_fi.data_ptr(), t_fl.data_ptr(), B, I3(*n2), e1, e2)

        fill_ms = timed(level2_fill, 3)
        sat_ms = timed(level2_sat, 3)
        ctx = gpv.Context(local)
        ref_boundary = None

        def native():
            nonlocal ref_boundary
            r = ctx.voxelize_device(d_tris.data_ptr(), T, spec, s0.cuda_stream)
            ref_boundary = r.num_boundary
            ctx.release(r)

        native_ms = timed(native)
        ctx.close()
    return {"workload": "torus262k", "level1_buffer": buf, "boundary": int(B),
            "boundary_matches_native": int(B) == int(ref_boundary),
            "ms": {"CUDAClassifyTessellation": l1_ms, "CUDAClassifyInOutLevel2": fill_ms,
                   "CUDAClassifyTessellationLevel2": sat_ms},
            "shim_total_ms": l1_ms + fill_ms + sat_ms, "native_ms": native_ms,
            "note": "device time per shim call (legacy stream, CUDA events); the host list "
                    "building between the levels is not included; the native call computes "
                    "both levels' states, prefix, index and Level2 bytes without normals"}


def progress(msg):
    """Section markers on stderr (the JSON line goes to stdout at the end)."""
    print(f"[bench] {msg}", file=sys.stderr, flush=True)


def main():
    faulthandler.enable()
    args = parse()
    if args.impl == "reference":
        run_reference(args)
        return
    import numpy as np
    import torch

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    dist = None
    if world > 1:
        import torch.distributed as dist

        torch.cuda.set_device(local)
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    torch.cuda.set_device(local)

    import gpview_gb300 as gpv
    import workloads as W

    cfg = WORKLOADS[args.workload]
    if args.level2:
        cfg = dict(cfg, level2=args.level2)
    # the recorded per-launch counters of the roofline belong to the workloads as defined
    rname = cfg["name"] + (f"-l2x{args.level2}" if args.level2 else "")
    tris, spec = W.make(cfg)
    T = tris.size // 9
    ctx = gpv.Context(local)
    if args.tile:
        ctx.set_tile(args.tile)
    if args.chunk:
        ctx.set_level2_chunk(args.chunk)
    ctx.set_level2_mode({"auto": gpv.LEVEL2_AUTO, "queued": gpv.LEVEL2_QUEUED,
                         "inline": gpv.LEVEL2_INLINE}[args.level2_mode])
    ctx.set_graphs(not args.no_graphs)
    stream = torch.cuda.Stream(device=local)
    sp = stream.cuda_stream
    d_tris = torch.from_numpy(tris).to(f"cuda:{local}")
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=f"cuda:{local}")

    def step_device():
        res = ctx.voxelize_device(d_tris.data_ptr(), T, spec, sp)
        return res

    # warm-up
    with torch.cuda.stream(stream):
        for _ in range(args.warmup):
            r = step_device()
            ctx.release(r)
    torch.cuda.synchronize()
    peaks, peak_kind = load_peaks()

    # timed region (device-resident inputs), stage timing off: the path as a caller runs it
    clocks = Clocks(local)
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
          for _ in range(args.steps)]
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    clocks.start()
    launches0 = gpv.kernel_launches()
    work = None
    stats = None
    with torch.cuda.stream(stream):
        for k in range(args.steps):
            flush.zero_()
            ev[k][0].record(stream)
            r = step_device()
            ev[k][1].record(stream)
            if work is None:
                work = (r.work.sat1, r.work.sat2, r.work.ray1, r.work.ray2)
                stats = dict(boundary=r.num_boundary, pairs=r.num_pairs,
                             l1_inside=r.num_level1_inside, l2_inside=r.num_level2_inside,
                             l2_boundary=r.num_level2_boundary, level1=r.num_level1)
            ctx.release(r)
    torch.cuda.synchronize()
    launches = gpv.kernel_launches() - launches0
    clk = clocks.stop()
    if dist:
        dist.barrier()
    step_ms = [a.elapsed_time(b) for a, b in ev]
    # the same steps again with the per-stage CUDA events recorded inside the phase graphs: the
    # stage breakdown and the Level2 kernel's own duration (for the roofline).  The event nodes
    # cost ~0.01-0.05 ms per call, so this region is reported beside the headline, not as it.
    ctx.set_timing(True)
    with torch.cuda.stream(stream):
        for _ in range(2):  # the phase graphs are recorded once with the event nodes
            ctx.release(step_device())
    torch.cuda.synchronize()
    ctx.set_timing(True)  # clears the accumulated times
    ev_st = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
             for _ in range(args.steps)]
    torch.cuda.synchronize()
    with torch.cuda.stream(stream):
        for k in range(args.steps):
            flush.zero_()
            ev_st[k][0].record(stream)
            r = step_device()
            ev_st[k][1].record(stream)
            ctx.release(r)
    torch.cuda.synchronize()
    calls, stage_ms = ctx.stage_times()
    hcalls, host_ms = ctx.host_times()
    ctx.set_timing(False)
    staged_ms = sum(a.elapsed_time(b) for a, b in ev_st) / args.steps
    t_total = sum(step_ms) / 1e3
    t_total = max_over_ranks(t_total, dist, f"cuda:{local}")
    tests_per_step = sum(work)
    value = job_value(tests_per_step, args.steps, world, t_total)

    # e2e through the host API: pinned H2D, voxelize, D2H of all outputs
    cells = spec.ndiv2[0] * spec.ndiv2[1] * spec.ndiv2[2]
    h_tris = torch.from_numpy(tris).pin_memory()
    h_l1 = torch.empty(stats["level1"], dtype=torch.uint8).pin_memory()
    h_pre = torch.empty(stats["level1"], dtype=torch.int32).pin_memory()
    h_bi = torch.empty(max(stats["boundary"], 1), dtype=torch.int32).pin_memory()
    h_l2 = torch.empty(max(stats["boundary"] * cells, 1), dtype=torch.uint8).pin_memory()
    e2e_times = []
    for k in range(args.warmup + args.steps):
        with torch.cuda.stream(stream):
            flush.zero_()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        # host triangles in, host outputs out: H2D, voxelization, and the D2H of every output
        # (Level1 arrays as soon as they exist, Level2 slab by slab while later slabs compute)
        rc, res = ctx.voxelize_to_host(h_tris.data_ptr(), T, spec, h_l1.data_ptr(),
                                       h_pre.data_ptr(), h_bi.data_ptr(), h_l2.data_ptr(),
                                       h_l2.numel(), args.slabs, sp)
        if rc:
            raise gpv.GpvError(rc, ctx.error())
        t1 = time.perf_counter()
        ctx.release(res)
        if k >= args.warmup:
            e2e_times.append(t1 - t0)
    e2e_t = sum(e2e_times)
    e2e_t = max_over_ranks(e2e_t, dist, f"cuda:{local}")
    e2e_value = job_value(tests_per_step, args.steps, world, e2e_t)
    h2d = T * 36
    d2h = stats["level1"] * 5 + stats["boundary"] * (4 + cells)

    # roofline of the dominant kernel (the Level2 kernel: instruction-issue-bound integer/FP32 work)
    per_call = {k: v / max(calls, 1) for k, v in stage_ms.items()}
    N1, B = stats["level1"], stats["boundary"]
    roof = roofline(rname, per_call, work, stats, spec, T, peaks, peak_kind, clk)

    line = {"metric": METRIC, "value": value, "unit": "tests/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": t_total * 1e3 / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic", "config": workload_config(cfg, T),
            "work_per_step": dict(zip(("sat1", "sat2", "ray1", "ray2"), work)), "stats": stats,
            "meshes_per_s": args.steps * world / t_total,
            "voxels_per_s": (N1 + B * cells) * args.steps * world / t_total,
            "e2e": {"value": e2e_value, "unit": "tests/s", "h2d_bytes_per_step": h2d,
                    "d2h_bytes_per_step": d2h, "ms_per_step": e2e_t * 1e3 / args.steps},
            "gpu_launches": launches, "roofline": roof, "clocks": clk,
            "ms_per_step_with_stage_events": staged_ms,
            "host_ms_per_call": {k: v / max(hcalls, 1) for k, v in host_ms.items()}}
    tuned = (128, 8)
    progress("plain path done")
    if not args.no_stencil:
        progress("stencil fill section")
        line["stencil_fill"] = stencil_bench(gpv, ctx, torch, stream, step_device, flush, args,
                                             tris, spec, rank == 0 and args.stencil_cpu)
    if args.batch > 0:
        progress("batched section")
        line["batched"] = batch_bench(gpv, ctx, torch, stream, local, args)
        tuned = (line["batched"]["tile"], line["batched"]["level2_chunk"])
    if not args.no_shims:
        progress("shim section")
        line["shims"] = shim_bench(gpv, torch, local, args)
    if args.serve_seconds > 0:
        progress("served section")
        line["served"] = served_bench(gpv, torch, local, args, tuned)
    if rank == 0 and not args.no_cpu_baseline:
        progress("cpu baseline")
        threads = os.cpu_count() or 1
        # the GPU's work counts are the reference algorithm's: the oracle counts the same
        _, work_cpu = cpu_work(tris, spec, threads)
        line["cpu_baseline"] = cpu_sample(tris, spec, tests_per_step, args.cpu_seconds, threads)
        line["cpu_baseline"].pop("sec_per_mesh", None)
        line["cpu_baseline"]["tests_per_mesh_oracle"] = work_cpu
        line["cpu_baseline"]["tests_per_mesh_match"] = work_cpu == tests_per_step
        if not args.no_as_written:
            aw = cpu_as_written(tris, spec, tests_per_step, args.as_written_seconds)
            aw.pop("sec_per_mesh", None)
            line["cpu_baseline"]["as_written"] = aw
    if rank == 0:
        print(json.dumps(line))
    ctx.close()
    if dist:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
