#!/usr/bin/env python3
"""Benchmark of the trace-commitment hot path on GB300.

Workload (default): the plain single-trace BabyBear commit -- a 2^20 x 256
trace of uniform random elements, coset LDE with log_blowup 1 and shift 31
(rows bit-reversed, 2^21 x 256 = 2 GiB of u32), then the Poseidon2-16
(x^7, 8 full + 13 partial rounds, seeded constants) mixed-height MMCS commit
to one root.  A step is one full commit of that trace.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Prints one JSON line (rank 0).  `value` is committed LDE elements/s with the
trace already resident in HBM (device-timed with CUDA events on the launching
stream); `e2e` is the same metric through the C ABI with the trace in pinned
host memory, the host->device copy and the root read-back inside the timed
region.  `--impl reference` times the CPU restatement of the reference path
(the oracle, built from oracle/) on the host cores, on a bounded sample of the
same workload.  Inputs (1 GiB trace, 2 GiB LDE) are larger than L2 (129 MB),
so no L2 flush is needed between steps.
"""
from __future__ import annotations

import argparse
import gc
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

REPO = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(REPO, "plonky3-gpu_gb300"))

METRIC = "committed LDE elements/s on 1 GB300, batched vs plain per-trace; p50/p99 ms"
UNIT = "elements/s"
LOG_H, WIDTH, LOG_B, SHIFT = 20, 256, 1, 31
BB_P = 0x78000001


def peaks():
    p = os.path.join(REPO, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def dist_info():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def job_throughput(units: float, ms: float, device=None):
    """Whole-job throughput of independent replicas: the units every rank
    processed divided by the slowest rank's time.  Returns (units/s, max ms).
    Collective only over the already-initialised process group (NCCL on the
    GPU, gloo in the CPU tests); one rank returns its own figures."""
    import torch
    import torch.distributed as dist
    if dist.is_available() and dist.is_initialized() and dist.get_world_size() > 1:
        t = torch.tensor([ms], dtype=torch.float64, device=device)
        u = torch.tensor([units], dtype=torch.float64, device=device)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        dist.all_reduce(u, op=dist.ReduceOp.SUM)
        ms, units = float(t.item()), float(u.item())
    return units / (ms / 1e3), ms


class ClockSampler:
    """Samples nvidia-smi clocks/throttle reasons while the timed region runs."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        # the raw samples (the JSON line carries their summary); P3G_CLOCKS_DIR keeps them
        self.path = os.path.join(os.environ.get("P3G_CLOCKS_DIR", tempfile.gettempdir()), f"clocks_{device}.csv")

    def __enter__(self):
        os.makedirs(os.path.dirname(self.path), exist_ok=True)
        try:
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=self.f, stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None
        time.sleep(0.3)
        return self

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            self.proc.wait()
            self.f.close()

    def summary(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        rows = []
        with open(self.path) as f:
            for line in f:
                parts = [x.strip() for x in line.split(",")]
                if len(parts) >= 9:
                    rows.append(parts)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[5 + i].lower().startswith("active")})
        loaded = [s for s in sm if s > 0.5 * max(sm)] if sm else []
        return {"sm_mhz": statistics.median(loaded) if loaded else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": reasons, "samples": len(rows)}


def cpu_sample(nthreads: int, log_h: int = 14):
    """The oracle's commit (restated Radix2Dit LDE + Poseidon2 MMCS) on a bounded
    sample of the workload: same width, blowup and hash, height 2^log_h."""
    sys.path.insert(0, os.path.join(REPO, "oracle"))
    import oracle as O

    O.build()
    rng = np.random.default_rng(5)
    t = rng.integers(0, BB_P, size=(1 << log_h, WIDTH), dtype=np.uint32)
    p = O.bb16_params()
    t0 = time.perf_counter()
    lde = O.bb_coset_lde(t, LOG_B, SHIFT, True, nthreads=nthreads)
    O.mmcs_commit(p, [lde], 0, nthreads=nthreads)
    dt = time.perf_counter() - t0
    elems = (1 << (log_h + LOG_B)) * WIDTH
    return elems / dt, dt, f"2^{log_h} x {WIDTH} BabyBear trace, log_blowup 1, LDE + Poseidon2-16 MMCS root"


def run_reference(args):
    ws, rank, _ = dist_info()
    if rank != 0:
        return 0
    nthreads = os.cpu_count() or 1
    for _ in range(args.warmup):
        cpu_sample(nthreads, 12)
    vals, times = [], []
    desc = ""
    for _ in range(args.steps):
        v, dt, desc = cpu_sample(nthreads)
        vals.append(v)
        times.append(dt * 1e3)
    value = statistics.mean(vals)
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": statistics.mean(times),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u32 (BabyBear)",
        "data": "synthetic",
        "config": {"workload": "plain single-trace BabyBear commit, 2^20 x 256, log_blowup 1 (bounded CPU sample)",
                   "sample": desc},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": nthreads, "kind": "port", "sample": desc},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))
    return 0


GL_P = 0xFFFFFFFF00000001


def run_goldilocks(P, torch, ctx, dev, stream, steps: int, warmup: int, log_h: int = 18, width: int = 128,
                   log_b: int = 2, shift: int = 7):
    """Config 2: the plain single-trace Goldilocks commit -- a 2^18 x 128 trace
    of uniform canonical u64 elements, coset LDE with log_blowup 2 and shift 7
    (2^20 x 128 = 1 GiB of u64, rows bit-reversed), Poseidon2-8 (x^7, 8+22)
    MMCS with 4-element digests.  Device-timed with the trace resident; the
    LDE alone is timed beside it for its HBM roofline."""
    sptr = stream.cuda_stream
    h, H = 1 << log_h, 1 << (log_h + log_b)
    rng = np.random.default_rng(2)
    trace = rng.integers(0, GL_P, size=(h, width), dtype=np.uint64)
    d_trace = ctx.to_device(trace)
    ctx.sync()

    def step():
        ctx.commit_traces_device(P.GOLDILOCKS, [(d_trace.ptr, log_h, width, log_b, shift)], 0,
                                 stream=sptr).free(sptr)

    def timed(fn, n):
        evs = [torch.cuda.Event(enable_timing=True) for _ in range(n + 1)]
        torch.cuda.synchronize(dev)
        with torch.cuda.stream(stream):
            for i in range(n):
                evs[i].record(stream)
                fn()
            evs[-1].record(stream)
        torch.cuda.synchronize(dev)
        return [evs[i].elapsed_time(evs[i + 1]) for i in range(n)]

    for _ in range(warmup):
        step()
    l0 = P.kernel_launches()
    st = timed(step, steps)
    launches = (P.kernel_launches() - l0) // max(steps, 1)
    d_lde = ctx.alloc(H * width * 8, sptr)

    def lde():
        ctx.coset_lde_device(P.GOLDILOCKS, d_trace.ptr, log_h, width, log_b, shift, True, d_lde.ptr, sptr)

    for _ in range(2):
        lde()
    lt = timed(lde, 10)
    d_lde.free(sptr)
    torch.cuda.synchronize(dev)
    d_trace.free()
    ms, lde_ms = statistics.mean(st), statistics.mean(lt)
    lde_bytes = 8 * width * (h + H)
    hbm, src = peaks()
    perms = H * ((width + 3) // 4) + (H - 1)
    traffic = None
    tpath = os.path.join(REPO, "profiles", "traffic.json")
    if os.path.exists(tpath):
        with open(tpath) as f:
            traffic = json.load(f).get(f"lde_gl_2p{log_h}x{width}_b{log_b}_bytes")
    return {
        "workload": f"plain single-trace Goldilocks commit: 2^{log_h} x {width} trace, log_blowup {log_b}, "
                    f"shift {shift}, bit-reversed LDE 2^{log_h + log_b} x {width}, Poseidon2-8 (x^7, 8+22) MMCS, "
                    "cap_height 0",
        "value": H * width / (ms / 1e3), "unit": UNIT, "dtype": "u64 (Goldilocks)", "ms_per_step": ms,
        "p50_ms": float(np.percentile(st, 50)), "p99_ms": float(np.percentile(st, 99)),
        "kernels_per_step": int(launches),
        "lde": {"ms": lde_ms, "algorithmic_bytes": lde_bytes, "achieved_gbs": lde_bytes / (lde_ms / 1e3) / 1e9,
                "peak_gbs": hbm, "frac": lde_bytes / (lde_ms / 1e3) / 1e9 / hbm, "peak_source": src,
                "traffic": traffic},
        "merkle": {"ms": ms - lde_ms, "perms": perms, "perms_per_s": perms / ((ms - lde_ms) / 1e3)},
    }


def config3_shapes(seed: int = 3):
    """64 BabyBear traces: log2 height uniform over {12..18}, width uniform in [8, 512]."""
    rng = np.random.default_rng(seed)
    return [(int(rng.integers(12, 19)), int(rng.integers(8, 513))) for _ in range(64)]


def run_batched(P, torch, ctx, dev, stream, steps: int, warmup: int):
    """Config 3: the 64-trace batch committed as one graph-captured plan (one
    mixed-height MMCS) plus a fold of a 2^19-row BabyBear^4 quotient, against
    the same work done per trace (one p3g_commit_traces per trace, then the
    fold) on one stream.  Traces are generated on the device (seeded)."""
    sptr = stream.cuda_stream
    shapes = config3_shapes()
    gen = torch.Generator(device=dev)
    gen.manual_seed(3)
    bufs = [torch.randint(0, BB_P, ((1 << lh) * w,), device=dev, dtype=torch.int64, generator=gen).to(torch.int32)
            for lh, w in shapes]
    fin = torch.randint(0, BB_P, ((1 << 19) * 4,), device=dev, dtype=torch.int64, generator=gen).to(torch.int32)
    fout = torch.empty((1 << 18) * 4, device=dev, dtype=torch.int32)
    beta = [int(x) for x in np.random.default_rng(4).integers(0, BB_P, 4)]
    traces = [(b.data_ptr(), lh, w, 1, SHIFT) for b, (lh, w) in zip(bufs, shapes)]
    elems = sum((1 << (lh + 1)) * w for lh, w in shapes)
    torch.cuda.synchronize(dev)
    t0 = time.perf_counter()
    plan = P.Plan(ctx, P.BABYBEAR, traces, 0, fold=(fin.data_ptr(), fout.data_ptr(), 19, 1, beta), n_streams=0)
    plan_s = time.perf_counter() - t0

    def timed(fn, n):
        evs = [torch.cuda.Event(enable_timing=True) for _ in range(n + 1)]
        torch.cuda.synchronize(dev)
        with torch.cuda.stream(stream):
            for i in range(n):
                evs[i].record(stream)
                fn()
            evs[-1].record(stream)
        torch.cuda.synchronize(dev)
        return [evs[i].elapsed_time(evs[i + 1]) for i in range(n)]

    for _ in range(warmup):
        plan.launch(sptr)
    l0 = P.kernel_launches()
    bt = timed(lambda: plan.launch(sptr), steps)
    b_launches = (P.kernel_launches() - l0) // max(steps, 1)

    def plain():
        for tr in traces:
            ctx.commit_traces_device(P.BABYBEAR, [tr], 0, stream=sptr).free(sptr)
        ctx.fold_matrix_bb4_device(fin.data_ptr(), 19, 1, beta, fout.data_ptr(), stream=sptr)

    for _ in range(warmup):
        plain()
    l0 = P.kernel_launches()
    pt = timed(plain, steps)
    p_launches = (P.kernel_launches() - l0) // max(steps, 1)
    bms, pms = statistics.mean(bt), statistics.mean(pt)
    out = {
        "workload": "64 BabyBear traces, log2 h uniform in {12..18}, width uniform in [8, 512], log_blowup 1, "
                    "one mixed-height Poseidon2-16 MMCS, plus fold_matrix of a 2^19-row BabyBear^4 quotient "
                    "(log_arity 1, seeded beta)",
        "lde_elements": elems,
        "batched": {"value": elems / (bms / 1e3), "unit": UNIT, "ms_per_step": bms,
                    "p50_ms": float(np.percentile(bt, 50)), "p99_ms": float(np.percentile(bt, 99)),
                    "graph_launches_per_step": 1, "kernels_per_step": int(b_launches),
                    "streams": plan.n_streams, "plan_seconds": plan_s},
        "plain_per_trace": {"value": elems / (pms / 1e3), "unit": UNIT, "ms_per_step": pms,
                            "p50_ms": float(np.percentile(pt, 50)), "p99_ms": float(np.percentile(pt, 99)),
                            "kernels_per_step": int(p_launches)},
        "batched_over_plain": pms / bms,
    }
    plan.destroy()
    del bufs
    return out


def run_serving(P, torch, ctx, rates, per_rate: int, slots: int = 8):
    """Config 4: Poisson arrivals of commit+fold requests (log2 h uniform in
    {10..20}, width uniform in [4, 256], log_blowup in {1, 2, 3}) into the
    continuous-batching server; each completed request gets a 32-query
    opening on its resident LDE/tree and is then released.  Latency is from
    the scheduled arrival to the result; elements/s counts committed LDE
    elements over the run.  Request payloads are prefixes of one pinned host
    buffer of random BabyBear elements."""
    import ctypes as C

    max_elems = (1 << 20) * 256
    host = torch.randint(0, BB_P, (max_elems,), dtype=torch.int64).to(torch.int32).pin_memory()
    hptr = host.data_ptr()
    server = P.Server(ctx, max_slots=slots)
    out = []
    rid = 0
    try:
        for lam in rates:
            rng = np.random.default_rng(int(lam))
            reqs = []
            t = 0.0
            for _ in range(per_rate):
                t += rng.exponential(1.0 / lam)
                lh, w, lb = int(rng.integers(10, 21)), int(rng.integers(4, 257)), int(rng.integers(1, 4))
                beta = [int(x) for x in rng.integers(0, BB_P, 4)]
                reqs.append((t, lh, w, lb, beta))
            arrival = {}
            lat, open_ms, elems = [], [], 0
            done = 0
            i = 0
            t0 = time.monotonic_ns()
            while done < len(reqs):
                now = (time.monotonic_ns() - t0) / 1e9
                while i < len(reqs) and reqs[i][0] <= now:
                    tt, lh, w, lb, beta = reqs[i]
                    rid += 1
                    arrival[rid] = (t0 + int(tt * 1e9), lh, w, lb)
                    server.submit(rid, hptr, lh, w, lb, SHIFT, beta)
                    i += 1
                for r in server.poll():
                    a, lh, w, lb = arrival.pop(r.id)
                    if r.status == 0:
                        lat.append((r.t_done_ns - a) / 1e6)
                        elems += (1 << (lh + lb)) * w
                        q = np.random.default_rng(r.id).integers(0, 1 << (lh + lb), 32, dtype=np.uint64)
                        o0 = time.perf_counter()
                        server.open(r.id, q, w, lh + lb + 1)
                        open_ms.append((time.perf_counter() - o0) * 1e3)
                        server.release(r.id)
                    done += 1
                if i < len(reqs):
                    time.sleep(max(0.0, min(0.0005, reqs[i][0] - (time.monotonic_ns() - t0) / 1e9)))
                else:
                    time.sleep(0.0002)
            wall = (time.monotonic_ns() - t0) / 1e9
            out.append({"rate_per_s": lam, "requests": len(reqs), "completed": len(lat),
                        "p50_ms": float(np.percentile(lat, 50)) if lat else None,
                        "p99_ms": float(np.percentile(lat, 99)) if lat else None,
                        "elements_per_s": elems / wall, "wall_s": wall,
                        "open32_p50_ms": float(np.percentile(open_ms, 50)) if open_ms else None})
    finally:
        server.close()
    return {"workload": "Poisson commit+fold requests: log2 h uniform in {10..20}, width uniform in [4, 256], "
                        "log_blowup uniform in {1, 2, 3}; fold of the LDE's first four columns as BabyBear^4; "
                        "32-query opening on the resident tree, then release",
            "slots": slots, "points": out}


def run_ours(args):
    import ctypes as C

    import torch
    import p3g_gb300 as P

    ws, rank, local = dist_info()
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    stream = torch.cuda.Stream(device=dev)
    sptr = stream.cuda_stream

    ctx = P.Context(local)
    ctx.set_default_poseidon2()
    LOG_H, WIDTH = args.log_h, args.width
    h, H = 1 << LOG_H, 1 << (LOG_H + LOG_B)
    elems = H * WIDTH
    rng = np.random.default_rng(1234 + rank)
    trace = rng.integers(0, BB_P, size=(h, WIDTH), dtype=np.uint32)
    d_trace = ctx.to_device(trace)
    ctx.sync()

    def step(cap_out=None):
        tree = ctx.commit_traces_device(P.BABYBEAR, [(d_trace.ptr, LOG_H, WIDTH, LOG_B, SHIFT)], 0,
                                        stream=sptr, cap_out=cap_out)
        tree.free(sptr)

    for _ in range(max(args.warmup, 1)):
        step()
    torch.cuda.synchronize(dev)

    # ---- device-timed region (trace resident in HBM)
    evs = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps + 1)]
    if ws > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize(dev)
    l0 = P.kernel_launches()
    gc.collect()
    gc.disable()
    with ClockSampler(local) as clk:
        with torch.cuda.stream(stream):
            for i in range(args.steps):
                evs[i].record(stream)
                step()
            evs[-1].record(stream)
        torch.cuda.synchronize(dev)
    gc.enable()
    launches = P.kernel_launches() - l0
    step_ms = [evs[i].elapsed_time(evs[i + 1]) for i in range(args.steps)]
    total_ms = evs[0].elapsed_time(evs[-1])
    value, total_ms = job_throughput(float(elems) * args.steps, total_ms, dev)
    ms_per_step = total_ms / args.steps

    # ---- stage breakdown: the LDE alone (roofline) -- same stream, CUDA events
    d_lde = ctx.alloc(elems * 4, sptr)
    reps = 10
    for _ in range(2):
        ctx.coset_lde_device(P.BABYBEAR, d_trace.ptr, LOG_H, WIDTH, LOG_B, SHIFT, True, d_lde.ptr, sptr)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize(dev)
    e0.record(stream)
    for _ in range(reps):
        ctx.coset_lde_device(P.BABYBEAR, d_trace.ptr, LOG_H, WIDTH, LOG_B, SHIFT, True, d_lde.ptr, sptr)
    e1.record(stream)
    torch.cuda.synchronize(dev)
    lde_ms = e0.elapsed_time(e1) / reps
    d_lde.free(sptr)
    torch.cuda.synchronize(dev)

    # ---- end to end through the C ABI with the trace in pinned host memory:
    # p3g_commit_traces_host copies column chunks on a second stream while the
    # earlier chunks' LDEs and row hashes run; the root read-back synchronises
    # the stream
    pinned = torch.empty(h * WIDTH, dtype=torch.int32, pin_memory=True)
    pinned.numpy().view(np.uint32)[:] = trace.reshape(-1)
    cap = np.zeros((1, 8), np.uint32)
    e2e_ms = []
    gc.collect()
    gc.disable()  # the interpreter's collector paused in the timed loop, as the timeit module does
    for i in range(args.warmup + args.steps):
        t0 = time.perf_counter()
        tree = ctx.commit_traces_host(P.BABYBEAR, [(pinned.data_ptr(), LOG_H, WIDTH, LOG_B, SHIFT)], 0,
                                      stream=sptr, cap_out=cap)
        tree.free(sptr)
        dt = (time.perf_counter() - t0) * 1e3
        if i >= args.warmup:
            e2e_ms.append(dt)
    gc.enable()
    torch.cuda.synchronize(dev)
    e2e_value, e2e_mean = job_throughput(float(elems), statistics.mean(e2e_ms), dev)

    prover = {}
    if not args.no_prover:
        # ---- PCS open on the commit's resident bit-reversed LDE (2^21 x 256):
        # opened values at 2 points and the reduced opening into a q vector
        tree = ctx.commit_traces_device(P.BABYBEAR, [(d_trace.ptr, LOG_H, WIDTH, LOG_B, SHIFT)], 0, stream=sptr)
        log_n = LOG_H + LOG_B
        pts = rng.integers(0, BB_P, size=(2, 4), dtype=np.uint32)
        alpha = rng.integers(0, BB_P, size=4, dtype=np.uint32)
        d_q = ctx.alloc(H * 16, sptr)
        ov = ctx.pcs_open_values_device(tree.leaf_ptr(0), log_n, WIDTH, True, SHIFT, pts, stream=sptr)
        ctx.pcs_reduce_device(tree.leaf_ptr(0), log_n, WIDTH, True, SHIFT, pts, ov, alpha, 0, True, d_q.ptr, sptr)
        torch.cuda.synchronize(dev)
        open_reps = 5
        e0.record(stream)
        for _ in range(open_reps):
            ctx.pcs_open_values_device(tree.leaf_ptr(0), log_n, WIDTH, True, SHIFT, pts, stream=sptr)
        e1.record(stream)
        torch.cuda.synchronize(dev)
        open_ms = e0.elapsed_time(e1) / open_reps
        e0.record(stream)
        for _ in range(open_reps):
            ctx.pcs_reduce_device(tree.leaf_ptr(0), log_n, WIDTH, True, SHIFT, pts, ov, alpha, 0, True, d_q.ptr, sptr)
        e1.record(stream)
        torch.cuda.synchronize(dev)
        reduce_ms = e0.elapsed_time(e1) / open_reps
        # ---- prove_fri on that reduced opening (2^21 BabyBear^4), transcript on the
        # device: commit-phase rounds, final polynomial, 16-bit query proof of work,
        # 100 query indices and every round's openings (host clock; the call synchronises)
        fri_params = dict(log_blowup=LOG_B, log_final_poly_len=0, max_log_arity=1, num_queries=100,
                          commit_proof_of_work_bits=0, query_proof_of_work_bits=16)
        st0 = rng.integers(0, BB_P, size=16, dtype=np.uint32)
        ctx.fri_prove_device([(d_q.ptr, log_n)], fri_params, st0, [], [], stream=sptr)
        fri_ms = []
        for _ in range(3):
            t0 = time.perf_counter()
            fri_res = ctx.fri_prove_device([(d_q.ptr, log_n)], fri_params, st0, [], [], stream=sptr)
            fri_ms.append((time.perf_counter() - t0) * 1e3)
        d_q.free(sptr)
        tree.free(sptr)
        torch.cuda.synchronize(dev)

        # ---- FRI fold (p3g_fold_matrix_bb4): the config-3 quotient size (2^19
        # BabyBear^4, L2-resident) and a 2^25-value vector (512 MiB in, larger
        # than L2) for the HBM roofline; CUDA events on the stream
        fold = {}
        for log_f in (19, 25):
            d_in = ctx.to_device(rng.integers(0, BB_P, size=(1 << log_f, 4), dtype=np.uint32))
            d_out = ctx.alloc((1 << log_f) * 16 // 2, sptr)
            beta_f = rng.integers(0, BB_P, size=4, dtype=np.uint32)
            for la in (1, 2, 3):
                ctx.fold_matrix_bb4_device(d_in.ptr, log_f, la, beta_f, d_out.ptr, sptr)
                torch.cuda.synchronize(dev)
                e0.record(stream)
                for _ in range(reps):
                    ctx.fold_matrix_bb4_device(d_in.ptr, log_f, la, beta_f, d_out.ptr, sptr)
                e1.record(stream)
                torch.cuda.synchronize(dev)
                ms = e0.elapsed_time(e1) / reps
                nbytes = 16 * ((1 << log_f) + ((1 << log_f) >> la))
                fold[f"2^{log_f}_arity{1 << la}"] = {"ms": ms, "algorithmic_bytes": nbytes,
                                                     "gbs": nbytes / (ms / 1e3) / 1e9}
            d_out.free(sptr)
            d_in.free()
        torch.cuda.synchronize(dev)

    # ---- permutation ceiling: the same Poseidon2-16 on 2^22 register-resident
    # states (p3g_poseidon2_permute), no sponge or tree around it
    n_states = 1 << 22
    d_states = ctx.to_device(rng.integers(0, BB_P, size=(n_states, 16), dtype=np.uint32))
    perm_once = lambda: P.check(P.load().p3g_poseidon2_permute(ctx.handle, P.BABYBEAR, d_states.ptr, n_states, sptr))
    for _ in range(2):
        perm_once()
    torch.cuda.synchronize(dev)
    e0.record(stream)
    for _ in range(reps):
        perm_once()
    e1.record(stream)
    torch.cuda.synchronize(dev)
    perm_peak = n_states / (e0.elapsed_time(e1) / reps / 1e3)
    d_states.free()

    if not args.no_prover:
        # ---- proof-of-work search (DuplexChallenger::grind, p3g_grind) at 26 bits
        # from 4 random challenger states: candidates searched per second, host
        # clock around each call (the call synchronises)
        grind_bits, grind_cand, grind_s = 26, 0, 0.0
        ctx.grind(P.BABYBEAR, np.zeros(16, np.uint32), [], 8, stream=sptr)
        for k in range(4):
            st = rng.integers(0, BB_P, size=16, dtype=np.uint32)
            t0 = time.perf_counter()
            w = ctx.grind(P.BABYBEAR, st, [int(x) for x in st[:k]], grind_bits, stream=sptr)
            grind_s += time.perf_counter() - t0
            grind_cand += w + 1

    if not args.no_prover:
        prover = {
            "pcs_open": {"workload": f"TwoAdicFriPcs::open passes on the resident bit-reversed LDE 2^{LOG_H + LOG_B} x "
                                     f"{WIDTH}, 2 BabyBear^4 points",
                         "open_values_ms": open_ms, "reduce_ms": reduce_ms,
                         "lde_bytes": elems * 4,
                         "open_values_gbs": elems * 4 / (open_ms / 1e3) / 1e9,
                         "reduce_gbs": elems * 4 / (reduce_ms / 1e3) / 1e9},
            "fri_prove": {"workload": f"prove_fri over the 2^{log_n} BabyBear^4 reduced opening above: "
                                      f"{len(fri_res['log_arities'])} rounds of arity 2, final polynomial of 1, "
                                      "16-bit query proof of work, 100 queries with openings; transcript on the device",
                          "ms": statistics.median(fri_ms), "samples_ms": [round(x, 3) for x in fri_ms]},
            "fold": {"workload": "fold_matrix over BabyBear^4 (p3g_fold_matrix_bb4), arities 2/4/8: 2^19 values "
                                 "(config 3's quotient, L2-resident) and 2^25 values (512 MiB, HBM)",
                     **fold, "hbm_frac_2^25_arity2": fold["2^25_arity2"]["gbs"] / peaks()[0]},
            "pow_grind": {"workload": f"DuplexChallenger::grind, {grind_bits} bits, 4 challenger states "
                                      "(0-3 pending inputs), Poseidon2-16",
                          "candidates": grind_cand, "ms": grind_s * 1e3,
                          "perms_per_s": grind_cand / grind_s,
                          "frac_of_perm_peak": grind_cand / grind_s / perm_peak},
        }
    hbm, src = peaks()
    lde_bytes = 4 * WIDTH * (h + H)
    lde_gbs = lde_bytes / (lde_ms / 1e3) / 1e9
    traffic = None
    tpath = os.path.join(REPO, "profiles", "traffic.json")
    if os.path.exists(tpath):
        with open(tpath) as f:
            traffic = json.load(f).get(f"lde_bb_2p{LOG_H}x{WIDTH}_b{LOG_B}_bytes")
    perms = H * ((WIDTH + 7) // 8) + (H - 1)
    hash_ms = ms_per_step - lde_ms
    result = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_per_step,
        "p50_ms": float(np.percentile(step_ms, 50)), "p99_ms": float(np.percentile(step_ms, 99)),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u32 (BabyBear)",
        "data": "synthetic",
        "config": {"workload": f"plain single-trace BabyBear commit: 2^{LOG_H} x {WIDTH} trace, log_blowup {LOG_B}, "
                               f"shift {SHIFT}, bit-reversed LDE 2^{LOG_H + LOG_B} x {WIDTH}, Poseidon2-16 "
                               "(x^7, 8+13) MMCS, cap_height 0",
                   "trace_rows": h, "trace_cols": WIDTH, "lde_rows": H, "field": "BabyBear",
                   "l2": (f"inputs larger than L2 ({h * WIDTH * 4 / 2**20:.0f} MiB trace, "
                          f"{elems * 4 / 2**20:.0f} MiB LDE); no flush") if h * WIDTH * 4 > 129e6
                         else "inputs smaller than L2 (profiling case)",
                   "parallelism": f"replicas x{ws}"},
        "python_gc": "collected before, paused during the timed loops (as the timeit module does)",
        "e2e": {"value": e2e_value, "unit": UNIT,
                "h2d_bytes_per_step": h * WIDTH * 4, "d2h_bytes_per_step": 32,
                "p50_ms": float(np.percentile(e2e_ms, 50)), "p99_ms": float(np.percentile(e2e_ms, 99)),
                "samples_ms": [round(x, 3) for x in e2e_ms],
                "call": "p3g_commit_traces_host (pinned host trace, root read back)"},
        "gpu_launches": int(launches),
        "clocks": clk.summary(),
        "roofline": {"kernel": "coset LDE (3 passes, k_lde_pass1/2/3)", "bound": "hbm", "achieved": lde_gbs,
                     "peak": hbm, "unit": "GB/s", "frac": lde_gbs / hbm, "traffic": traffic,
                     "peak_source": src, "algorithmic_bytes": lde_bytes, "ms": lde_ms},
        "stages": {"lde_ms": lde_ms, "merkle_ms": hash_ms, "perms": perms,
                   "perms_per_s": perms / (hash_ms / 1e3) if hash_ms > 0 else None},
        "hash_roofline": {"kernel": "Merkle stage (k_hash_groups leaf sponge + k_compress_level)",
                          "bound": "integer multiply pipe (permutation issue)",
                          "achieved": perms / (hash_ms / 1e3) if hash_ms > 0 else None, "unit": "perms/s",
                          "peak": perm_peak,
                          "peak_source": "isolated Poseidon2-16 permutation throughput, same run",
                          "frac": perms / (hash_ms / 1e3) / perm_peak if hash_ms > 0 else None},
    }
    result.update(prover)
    if not args.no_goldilocks:
        result["config2"] = run_goldilocks(P, torch, ctx, dev, stream, max(3, args.steps // 2), args.warmup)
    if not args.no_batched:
        result["config3"] = run_batched(P, torch, ctx, dev, stream, max(3, args.steps // 2), args.warmup)
    if not args.no_serving:
        result["config4"] = run_serving(P, torch, ctx, [50, 100, 200, 500, 1000, 2000], args.serving_requests)
    if rank == 0 and not args.no_cpu:
        v, dt, desc = cpu_sample(os.cpu_count() or 1)
        v1, dt1, desc1 = cpu_sample(1, 12)
        result["cpu_baseline"] = {"value": v, "unit": UNIT, "cores": os.cpu_count() or 1, "kind": "port",
                                  "sample": desc, "seconds": dt,
                                  "single_thread": {"value": v1, "cores": 1, "sample": desc1, "seconds": dt1,
                                                    "note": "the reference's own CPU path is single-threaded"}}
    d_trace.free()
    ctx.close()
    if rank == 0:
        print(json.dumps(result))
    if ws > 1:
        torch.distributed.destroy_process_group()
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline sample")
    ap.add_argument("--no-goldilocks", action="store_true", help="skip the Goldilocks 2^18 x 128 commit")
    ap.add_argument("--no-batched", action="store_true", help="skip the 64-trace batched comparison")
    ap.add_argument("--no-serving", action="store_true", help="skip the serving-loop latency sweep")
    ap.add_argument("--no-prover", action="store_true",
                    help="skip the PCS-open, FRI and proof-of-work measurements (profiling the commit alone)")
    ap.add_argument("--serving-requests", type=int, default=200, help="requests per arrival rate")
    ap.add_argument("--log-h", type=int, default=LOG_H, help="trace log2 height (profiling cases)")
    ap.add_argument("--width", type=int, default=WIDTH, help="trace width (profiling cases)")
    args = ap.parse_args()
    if args.impl == "reference":
        return run_reference(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
