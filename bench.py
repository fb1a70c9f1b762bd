#!/usr/bin/env python3
"""Benchmark of the trace-commitment hot path on GB300.

Headline workload (the metric's configuration): the batched commit of 64
BabyBear traces -- log2 height uniform over {12..18}, width uniform in
[8, 512], log_blowup 1, shift 31 -- as one mixed-height Poseidon2-16 (x^7,
8 full + 13 partial rounds, seeded constants) MMCS, plus fold_matrix of a
2^19-row BabyBear^4 quotient (log_arity 1, seeded beta), all captured in one
CUDA graph (p3g_plan_commit).  A step is one launch of that graph.  The same
work done as plain per-trace commits (one p3g_commit_traces call per trace,
then the fold) is timed beside it.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Prints one JSON line (rank 0).  `value` is committed LDE elements/s of the
batched plan with the traces resident in HBM (CUDA events on the launching
stream); `plain_per_trace` and `batched_over_plain` compare it with the
per-trace commit.  `e2e` is the same metric through the host-input plan
(p3g_plan_commit_host): the traces and the fold input in pinned host memory
are copied in inside every step, and the root and the fold output are read
back.  `config1` (a 2^20 x 256 single trace), `config2` (Goldilocks), the
prover steps and `config4` (serving) are further workloads.  `--impl
reference` times the CPU restatement of the reference path (the oracle,
built from oracle/) on the host cores, on a bounded sample of the same
workload.  The traces (4.2 GB) and LDEs (8.4 GB) exceed L2 (129 MB), so no
flush is needed between steps.
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
BB_P = 0x78000001
GL_P = 0xFFFFFFFF00000001
SHIFT = 31
C3_LOG_B = 1
C3_FOLD_LOG = 19
C1_LOG_H, C1_WIDTH, C1_LOG_B = 20, 256, 1
# the SM count and SMSPs of a GB300 (the issue bound below)
SMSPS = 152 * 4
# batches the end-to-end leg keeps in flight (default of --e2e-depth)
E2E_DEPTH = 3


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


# ------------------------------------------------------------------ workloads
def config3_shapes(seed: int = 3):
    """64 BabyBear traces: (log2 height uniform over {12..18}, width uniform in [8, 512])."""
    rng = np.random.default_rng(seed)
    return [(int(rng.integers(12, 19)), int(rng.integers(8, 513))) for _ in range(64)]


def config3_inputs(seed: int = 3, shrink: int = 0):
    """The batched workload's inputs: the 64 traces (uniform canonical BabyBear
    elements, trace i from default_rng([seed, i])), the 2^19 x 4 quotient
    (default_rng([seed, 64])) and the folding challenge beta.  `shrink` divides
    every height (and the quotient's) by 2^shrink: the bounded CPU samples."""
    shapes = [(lh - shrink, w) for lh, w in config3_shapes(seed)]
    traces = [np.random.default_rng([seed, i]).integers(0, BB_P, size=(1 << lh, w), dtype=np.uint32)
              for i, (lh, w) in enumerate(shapes)]
    fold_in = np.random.default_rng([seed, 64]).integers(0, BB_P, size=(1 << (C3_FOLD_LOG - shrink), 4),
                                                         dtype=np.uint32)
    beta = [int(x) for x in np.random.default_rng([seed, 65]).integers(0, BB_P, 4)]
    return shapes, traces, fold_in, beta


def lde_butterflies(shapes, log_b: int) -> float:
    """Radix-2 butterflies of the coset LDEs: per column an inverse transform
    of size h and 2^b forward ones, (h / 2) log2 h butterflies each."""
    return float(sum(w * (1 + (1 << log_b)) * ((1 << lh) // 2) * lh for lh, w in shapes))


def issue_bound_ms(butterflies: float, sm_mhz: float | None) -> float:
    """The BabyBear LDE's instruction-issue bound: six ALU-pipe instructions per
    butterfly (modular add, lazy difference, the Shoup product's correction),
    16 lanes per SMSP per clock on the ALU pipe, 608 SMSPs."""
    mhz = sm_mhz or 2070.0
    return butterflies * 6 / (SMSPS * 16 * mhz * 1e6) * 1e3


def cpu_sample(nthreads: int, shrink: int):
    """The oracle's batched commit (restated Radix2Dit LDEs, one mixed-height
    Poseidon2 MMCS, fold_matrix) on the config-3 traces with every height
    divided by 2^shrink.  Returns (LDE elements/s, seconds, description)."""
    sys.path.insert(0, os.path.join(REPO, "oracle"))
    import oracle as O

    O.build()
    shapes, traces, fold_in, beta = config3_inputs(3, shrink)
    p = O.bb16_params()
    t0 = time.perf_counter()
    ldes = [O.bb_coset_lde(t, C3_LOG_B, SHIFT, True, nthreads=nthreads) for t in traces]
    O.mmcs_commit(p, ldes, 0, nthreads=nthreads)
    O.fold_matrix_bb4(fold_in, C3_FOLD_LOG - shrink, 1, beta, nthreads=nthreads)
    dt = time.perf_counter() - t0
    elems = sum((1 << (lh + C3_LOG_B)) * w for lh, w in shapes)
    desc = (f"the 64 config-3 traces with every height divided by 2^{shrink} (log2 h in "
            f"{{{12 - shrink}..{18 - shrink}}}, {elems / 1e6:.0f} M LDE elements), one mixed-height Poseidon2-16 "
            f"MMCS, fold of a 2^{C3_FOLD_LOG - shrink} BabyBear^4 quotient")
    return elems / dt, dt, desc


def run_reference(args):
    ws, rank, _ = dist_info()
    if rank != 0:
        return 0
    nthreads = os.cpu_count() or 1
    for _ in range(args.warmup):
        cpu_sample(nthreads, 9)
    vals, times = [], []
    desc = ""
    for _ in range(args.steps):
        v, dt, desc = cpu_sample(nthreads, args.ref_shrink)
        vals.append(v)
        times.append(dt * 1e3)
    value = statistics.mean(vals)
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": statistics.mean(times),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u32 (BabyBear)",
        "data": "synthetic",
        "config": {"workload": "batched commit of the 64 config-3 BabyBear traces + fold (bounded CPU sample)",
                   "sample": desc},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": nthreads, "kind": "port", "sample": desc},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))
    return 0


def events_timed(torch, dev, stream, fn, n):
    """Per-call durations (ms) of n calls of fn, CUDA events on `stream`."""
    evs = [torch.cuda.Event(enable_timing=True) for _ in range(n + 1)]
    torch.cuda.synchronize(dev)
    with torch.cuda.stream(stream):
        for i in range(n):
            evs[i].record(stream)
            fn()
        evs[-1].record(stream)
    torch.cuda.synchronize(dev)
    return [evs[i].elapsed_time(evs[i + 1]) for i in range(n)]


def pinned_copy(torch, a: np.ndarray):
    """A page-locked host copy of a uint32 / uint64 array (a torch tensor that keeps it alive)."""
    dt = torch.int32 if a.dtype == np.uint32 else torch.int64
    t = torch.empty(a.size, dtype=dt, pin_memory=True)
    t.numpy().view(a.dtype)[:] = a.reshape(-1)
    return t


def traffic_of(key: str):
    tpath = os.path.join(REPO, "profiles", "traffic.json")
    if os.path.exists(tpath):
        with open(tpath) as f:
            return json.load(f).get(key)
    return None


# ------------------------------------------------------------------ further workloads
def run_config1(P, torch, ctx, dev, stream, steps: int, warmup: int, log_h: int, width: int, perm_peak: float):
    """Config 1: the plain single-trace BabyBear commit of a 2^20 x 256 trace
    (LDE 2^21 x 256 = 2 GiB), device-timed with the trace resident, its LDE
    alone for the HBM roofline, and end to end through p3g_commit_traces_host
    (pinned host trace, root read back)."""
    sptr = stream.cuda_stream
    h, H = 1 << log_h, 1 << (log_h + C1_LOG_B)
    elems = H * width
    trace = np.random.default_rng(1234).integers(0, BB_P, size=(h, width), dtype=np.uint32)
    d_trace = ctx.to_device(trace)
    ctx.sync()

    def step():
        ctx.commit_traces_device(P.BABYBEAR, [(d_trace.ptr, log_h, width, C1_LOG_B, SHIFT)], 0, stream=sptr).free(sptr)

    for _ in range(max(warmup, 1)):
        step()
    st = events_timed(torch, dev, stream, step, steps)
    ms = statistics.mean(st)
    d_lde = ctx.alloc(elems * 4, sptr)
    lde = lambda: ctx.coset_lde_device(P.BABYBEAR, d_trace.ptr, log_h, width, C1_LOG_B, SHIFT, True, d_lde.ptr, sptr)
    for _ in range(2):
        lde()
    lde_ms = statistics.mean(events_timed(torch, dev, stream, lde, 10))
    d_lde.free(sptr)
    torch.cuda.synchronize(dev)

    pinned = pinned_copy(torch, trace)
    cap = np.zeros((1, 8), np.uint32)
    e2e_ms = []
    for i in range(warmup + steps):
        t0 = time.perf_counter()
        ctx.commit_traces_host(P.BABYBEAR, [(pinned.data_ptr(), log_h, width, C1_LOG_B, SHIFT)], 0,
                               stream=sptr, cap_out=cap).free(sptr)
        if i >= warmup:
            e2e_ms.append((time.perf_counter() - t0) * 1e3)
    torch.cuda.synchronize(dev)
    d_trace.free()
    hbm, src = peaks()
    lde_bytes = 4 * width * (h + H)
    lde_gbs = lde_bytes / (lde_ms / 1e3) / 1e9
    perms = H * ((width + 7) // 8) + (H - 1)
    hash_ms = ms - lde_ms
    bfly = lde_butterflies([(log_h, width)], C1_LOG_B)
    return {
        "workload": f"plain single-trace BabyBear commit: 2^{log_h} x {width} trace, log_blowup {C1_LOG_B}, shift "
                    f"{SHIFT}, bit-reversed LDE 2^{log_h + C1_LOG_B} x {width}, Poseidon2-16 (x^7, 8+13) MMCS, "
                    "cap_height 0",
        "value": elems / (ms / 1e3), "unit": UNIT, "ms_per_step": ms,
        "p50_ms": float(np.percentile(st, 50)), "p99_ms": float(np.percentile(st, 99)),
        "e2e": {"value": elems / (statistics.mean(e2e_ms) / 1e3), "unit": UNIT,
                "h2d_bytes_per_step": h * width * 4, "d2h_bytes_per_step": 32,
                "p50_ms": float(np.percentile(e2e_ms, 50)), "p99_ms": float(np.percentile(e2e_ms, 99)),
                "samples_ms": [round(x, 3) for x in e2e_ms],
                "call": "p3g_commit_traces_host (pinned host trace, root read back)"},
        "roofline": {"kernel": f"coset LDE 2^{log_h} x {width} (k_lde_pass1/2/3)", "bound": "hbm",
                     "achieved": lde_gbs, "peak": hbm, "unit": "GB/s", "frac": lde_gbs / hbm,
                     "traffic": traffic_of(f"lde_bb_2p{log_h}x{width}_b{C1_LOG_B}_bytes"), "peak_source": src,
                     "algorithmic_bytes": lde_bytes, "ms": lde_ms},
        "issue_bound_ms": issue_bound_ms(bfly, None),
        "stages": {"lde_ms": lde_ms, "merkle_ms": hash_ms, "perms": perms,
                   "perms_per_s": perms / (hash_ms / 1e3) if hash_ms > 0 else None},
        "hash_roofline": {"kernel": "Merkle stage (k_hash_groups leaf sponge + compress levels)",
                          "bound": "integer multiply pipe (permutation issue)",
                          "achieved": perms / (hash_ms / 1e3) if hash_ms > 0 else None, "unit": "perms/s",
                          "peak": perm_peak, "peak_source": "isolated Poseidon2-16 permutation throughput, same run",
                          "frac": perms / (hash_ms / 1e3) / perm_peak if hash_ms > 0 else None},
    }


def run_prover(P, torch, ctx, dev, stream, perm_peak: float):
    """The prover steps after the commit on a resident 2^21 x 256 bit-reversed
    LDE: PCS open's two passes, prove_fri on the reduced opening, FRI folds and
    the proof-of-work search."""
    sptr = stream.cuda_stream
    rng = np.random.default_rng(77)
    log_h, width = C1_LOG_H, C1_WIDTH
    log_n = log_h + C1_LOG_B
    H = 1 << log_n
    elems = H * width
    d_trace = ctx.to_device(rng.integers(0, BB_P, size=(1 << log_h, width), dtype=np.uint32))
    tree = ctx.commit_traces_device(P.BABYBEAR, [(d_trace.ptr, log_h, width, C1_LOG_B, SHIFT)], 0, stream=sptr)
    pts = rng.integers(0, BB_P, size=(2, 4), dtype=np.uint32)
    alpha = rng.integers(0, BB_P, size=4, dtype=np.uint32)
    d_q = ctx.alloc(H * 16, sptr)
    ov = ctx.pcs_open_values_device(tree.leaf_ptr(0), log_n, width, True, SHIFT, pts, stream=sptr)
    ctx.pcs_reduce_device(tree.leaf_ptr(0), log_n, width, True, SHIFT, pts, ov, alpha, 0, True, d_q.ptr, sptr)
    open_ms = statistics.mean(events_timed(
        torch, dev, stream, lambda: ctx.pcs_open_values_device(tree.leaf_ptr(0), log_n, width, True, SHIFT, pts,
                                                              stream=sptr), 5))
    reduce_ms = statistics.mean(events_timed(
        torch, dev, stream, lambda: ctx.pcs_reduce_device(tree.leaf_ptr(0), log_n, width, True, SHIFT, pts, ov, alpha,
                                                         0, True, d_q.ptr, sptr), 5))
    fri_params = dict(log_blowup=C1_LOG_B, log_final_poly_len=0, max_log_arity=1, num_queries=100,
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
    d_trace.free(sptr)
    torch.cuda.synchronize(dev)

    fold = {}
    for log_f in (19, 25):
        d_in = ctx.to_device(rng.integers(0, BB_P, size=(1 << log_f, 4), dtype=np.uint32))
        d_out = ctx.alloc((1 << log_f) * 16 // 2, sptr)
        beta_f = rng.integers(0, BB_P, size=4, dtype=np.uint32)
        for la in (1, 2, 3):
            f = lambda: ctx.fold_matrix_bb4_device(d_in.ptr, log_f, la, beta_f, d_out.ptr, sptr)
            f()
            ms = statistics.mean(events_timed(torch, dev, stream, f, 10))
            nbytes = 16 * ((1 << log_f) + ((1 << log_f) >> la))
            fold[f"2^{log_f}_arity{1 << la}"] = {"ms": ms, "algorithmic_bytes": nbytes,
                                                 "gbs": nbytes / (ms / 1e3) / 1e9}
        d_out.free(sptr)
        d_in.free()
    torch.cuda.synchronize(dev)

    grind_bits, grind_cand, grind_s = 26, 0, 0.0
    ctx.grind(P.BABYBEAR, np.zeros(16, np.uint32), [], 8, stream=sptr)
    for k in range(4):
        st = rng.integers(0, BB_P, size=16, dtype=np.uint32)
        t0 = time.perf_counter()
        w = ctx.grind(P.BABYBEAR, st, [int(x) for x in st[:k]], grind_bits, stream=sptr)
        grind_s += time.perf_counter() - t0
        grind_cand += w + 1
    return {
        "pcs_open": {"workload": f"TwoAdicFriPcs::open passes on the resident bit-reversed LDE 2^{log_n} x "
                                 f"{width}, 2 BabyBear^4 points",
                     "open_values_ms": open_ms, "reduce_ms": reduce_ms, "lde_bytes": elems * 4,
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
                      "candidates": grind_cand, "ms": grind_s * 1e3, "perms_per_s": grind_cand / grind_s,
                      "frac_of_perm_peak": grind_cand / grind_s / perm_peak},
    }


def run_goldilocks(P, torch, ctx, dev, stream, steps: int, warmup: int, log_h: int = 18, width: int = 128,
                   log_b: int = 2, shift: int = 7):
    """Config 2: the plain single-trace Goldilocks commit -- a 2^18 x 128 trace
    of uniform canonical u64 elements, coset LDE with log_blowup 2 and shift 7
    (2^20 x 128 = 1 GiB of u64, rows bit-reversed), Poseidon2-8 (x^7, 8+22)
    MMCS with 4-element digests.  Device-timed with the trace resident; the
    LDE alone is timed beside it for its HBM roofline."""
    sptr = stream.cuda_stream
    h, H = 1 << log_h, 1 << (log_h + log_b)
    trace = np.random.default_rng(2).integers(0, GL_P, size=(h, width), dtype=np.uint64)
    d_trace = ctx.to_device(trace)
    ctx.sync()

    def step():
        ctx.commit_traces_device(P.GOLDILOCKS, [(d_trace.ptr, log_h, width, log_b, shift)], 0,
                                 stream=sptr).free(sptr)

    for _ in range(warmup):
        step()
    l0 = P.kernel_launches()
    st = events_timed(torch, dev, stream, step, steps)
    launches = (P.kernel_launches() - l0) // max(steps, 1)
    d_lde = ctx.alloc(H * width * 8, sptr)
    lde = lambda: ctx.coset_lde_device(P.GOLDILOCKS, d_trace.ptr, log_h, width, log_b, shift, True, d_lde.ptr, sptr)
    for _ in range(2):
        lde()
    lt = events_timed(torch, dev, stream, lde, 10)
    d_lde.free(sptr)
    torch.cuda.synchronize(dev)
    d_trace.free()
    ms, lde_ms = statistics.mean(st), statistics.mean(lt)
    lde_bytes = 8 * width * (h + H)
    hbm, src = peaks()
    perms = H * ((width + 3) // 4) + (H - 1)
    return {
        "workload": f"plain single-trace Goldilocks commit: 2^{log_h} x {width} trace, log_blowup {log_b}, "
                    f"shift {shift}, bit-reversed LDE 2^{log_h + log_b} x {width}, Poseidon2-8 (x^7, 8+22) MMCS, "
                    "cap_height 0",
        "value": H * width / (ms / 1e3), "unit": UNIT, "dtype": "u64 (Goldilocks)", "ms_per_step": ms,
        "p50_ms": float(np.percentile(st, 50)), "p99_ms": float(np.percentile(st, 99)),
        "kernels_per_step": int(launches),
        "lde": {"ms": lde_ms, "algorithmic_bytes": lde_bytes, "achieved_gbs": lde_bytes / (lde_ms / 1e3) / 1e9,
                "peak_gbs": hbm, "frac": lde_bytes / (lde_ms / 1e3) / 1e9 / hbm, "peak_source": src,
                "traffic": traffic_of(f"lde_gl_2p{log_h}x{width}_b{log_b}_bytes")},
        "merkle": {"ms": ms - lde_ms, "perms": perms, "perms_per_s": perms / ((ms - lde_ms) / 1e3)},
    }


def run_serving(P, torch, ctx, rates, total: int, slots: int = 8):
    """Config 4: Poisson arrivals of commit+fold requests (log2 h uniform in
    {10..20}, width uniform in [4, 256], log_blowup in {1, 2, 3}) into the
    continuous-batching server; each completed request gets a 32-query
    opening on its resident LDE/tree and is then released.  `total` requests
    are split evenly over the arrival rates.  Latency is from the scheduled
    arrival to the result; elements/s counts committed LDE elements over the
    run.  Request payloads are prefixes of one pinned host buffer of random
    BabyBear elements."""
    max_elems = (1 << 20) * 256
    host = torch.randint(0, BB_P, (max_elems,), dtype=torch.int64).to(torch.int32).pin_memory()
    hptr = host.data_ptr()
    server = P.Server(ctx, max_slots=slots)
    out = []
    rid = 0
    per = [total // len(rates) + (1 if k < total % len(rates) else 0) for k in range(len(rates))]
    try:
        for lam, n_req in zip(rates, per):
            rng = np.random.default_rng(int(lam))
            reqs = []
            t = 0.0
            for _ in range(n_req):
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
            "slots": slots, "requests": sum(per), "completed": sum(p["completed"] for p in out), "points": out}


def run_case(args):
    """One kernel sequence on its own, for profiling: `--case
    lde|commit:bb|gl:LOG_H:WIDTH:LOG_B` runs the coset LDE (bit-reversed rows)
    or the whole commit of one seeded trace, `warmup` untimed and `steps` timed
    calls (CUDA events), and prints their mean; `--case c3lde` runs the
    headline's LDE stage as the bench times it (the 64 config-3 LDEs, one
    p3g_coset_lde call each, on one stream)."""
    import torch
    import p3g_gb300 as P

    if args.case == "c3lde":
        dev = torch.device("cuda", 0)
        torch.cuda.set_device(0)
        stream = torch.cuda.Stream(device=dev)
        sptr = stream.cuda_stream
        ctx = P.Context(0)
        shapes, traces, _, _ = config3_inputs(3, args.c3_shrink)
        d_in = [ctx.to_device(t) for t in traces]
        d_out = [ctx.alloc(t.nbytes << C3_LOG_B) for t in traces]
        ctx.sync()

        def ldes():
            for (lh, w), a, b in zip(shapes, d_in, d_out):
                ctx.coset_lde_device(P.BABYBEAR, a.ptr, lh, w, C3_LOG_B, SHIFT, True, b.ptr, sptr)

        for _ in range(args.warmup):
            ldes()
        ms = statistics.mean(events_timed(torch, dev, stream, ldes, args.steps))
        nbytes = sum(4 * w * ((1 << lh) + (1 << (lh + C3_LOG_B))) for lh, w in shapes)
        print(json.dumps({"case": args.case, "ms": ms, "algorithmic_bytes": nbytes,
                          "algorithmic_gbs": nbytes / (ms / 1e3) / 1e9}))
        for b in d_in + d_out:
            b.free()
        ctx.close()
        return 0
    kind, field, log_h, width, log_b = args.case.split(":")
    log_h, width, log_b = int(log_h), int(width), int(log_b)
    gl = field == "gl"
    fid, shift = (P.GOLDILOCKS, 7) if gl else (P.BABYBEAR, SHIFT)
    dev = torch.device("cuda", 0)
    torch.cuda.set_device(0)
    stream = torch.cuda.Stream(device=dev)
    sptr = stream.cuda_stream
    ctx = P.Context(0)
    ctx.set_default_poseidon2()
    rng = np.random.default_rng(11)
    t = rng.integers(0, GL_P if gl else BB_P, size=(1 << log_h, width), dtype=np.uint64 if gl else np.uint32)
    d_t = ctx.to_device(t)
    H = 1 << (log_h + log_b)
    d_out = ctx.alloc(H * width * t.itemsize)
    ctx.sync()
    if kind == "lde":
        fn = lambda: ctx.coset_lde_device(fid, d_t.ptr, log_h, width, log_b, shift, True, d_out.ptr, sptr)
    else:
        fn = lambda: ctx.commit_traces_device(fid, [(d_t.ptr, log_h, width, log_b, shift)], 0, stream=sptr).free(sptr)
    for _ in range(args.warmup):
        fn()
    ms = statistics.mean(events_timed(torch, dev, stream, fn, args.steps))
    nbytes = t.itemsize * width * ((1 << log_h) + H)
    print(json.dumps({"case": args.case, "ms": ms, "lde_elements_per_s": H * width / (ms / 1e3),
                      "algorithmic_gbs": nbytes / (ms / 1e3) / 1e9 if kind == "lde" else None}))
    d_out.free()
    d_t.free()
    ctx.close()
    return 0


# ------------------------------------------------------------------ headline
def run_ours(args):
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

    # ---- config 3 inputs (host, seeded), device copies for the resident-trace runs
    shapes, traces, fold_in, beta = config3_inputs(3, args.c3_shrink)
    fold_log = C3_FOLD_LOG - args.c3_shrink
    elems = sum((1 << (lh + C3_LOG_B)) * w for lh, w in shapes)
    trace_bytes = sum(t.nbytes for t in traces)
    d_traces = [ctx.to_device(t) for t in traces]
    d_fin = ctx.to_device(fold_in)
    d_fout = ctx.alloc((1 << (fold_log - 1)) * 16)
    ctx.sync()
    dtr = [(b.ptr, lh, w, C3_LOG_B, SHIFT) for b, (lh, w) in zip(d_traces, shapes)]
    t0 = time.perf_counter()
    plan = P.Plan(ctx, P.BABYBEAR, dtr, 0, fold=(d_fin.ptr, d_fout.ptr, fold_log, 1, beta), n_streams=0)
    plan_s = time.perf_counter() - t0

    for _ in range(max(args.warmup, 1)):
        plan.launch(sptr)
    torch.cuda.synchronize(dev)

    # ---- device-timed region: K launches of the batched plan
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
                plan.launch(sptr)
            evs[-1].record(stream)
        torch.cuda.synchronize(dev)
    gc.enable()
    launches = P.kernel_launches() - l0
    step_ms = [evs[i].elapsed_time(evs[i + 1]) for i in range(args.steps)]
    total_ms = evs[0].elapsed_time(evs[-1])
    value, total_ms = job_throughput(float(elems) * args.steps, total_ms, dev)
    ms_per_step = total_ms / args.steps
    clocks = clk.summary()

    # ---- the same work as plain per-trace commits (one call per trace, then the fold)
    plain = None
    if not args.no_plain:
        def plain_step():
            for tr in dtr:
                ctx.commit_traces_device(P.BABYBEAR, [tr], 0, stream=sptr).free(sptr)
            ctx.fold_matrix_bb4_device(d_fin.ptr, fold_log, 1, beta, d_fout.ptr, stream=sptr)

        for _ in range(max(args.warmup, 1)):
            plain_step()
        l1 = P.kernel_launches()
        pt = events_timed(torch, dev, stream, plain_step, args.steps)
        p_launches = (P.kernel_launches() - l1) // max(args.steps, 1)
        pms = statistics.mean(pt)
        plain = {"value": elems / (pms / 1e3), "unit": UNIT, "ms_per_step": pms,
                 "p50_ms": float(np.percentile(pt, 50)), "p99_ms": float(np.percentile(pt, 99)),
                 "kernels_per_step": int(p_launches),
                 "call": "p3g_commit_traces once per trace, then p3g_fold_matrix_bb4, one stream"}

    # ---- LDE stage of the headline workload alone (roofline): the 64 LDEs on
    # one stream into the plan's own LDE buffers, CUDA events
    def ldes():
        for i, (lh, w) in enumerate(shapes):
            ctx.coset_lde_device(P.BABYBEAR, d_traces[i].ptr, lh, w, C3_LOG_B, SHIFT, True, plan.tree.leaf_ptr(i), sptr)

    ldes()
    lde_ms = statistics.mean(events_timed(torch, dev, stream, ldes, 5))
    # restore the plan's commitment inputs (the same values) and check the root is unchanged
    root_dev = plan.tree.layers()[-1].copy()

    # ---- end to end: host-input plans (p3g_plan_commit_host), the traces and
    # the quotient in pinned host memory, copied in by every launch; the root
    # and the fold output are read back after every step.  `depth` plans
    # over the same host inputs (their own device copies, LDEs, trees and fold
    # outputs) take turns on as many streams, so later batches' host-to-device
    # copies overlap the current batch's hashing; the host keeps `depth`
    # batches in flight (it reads back step i after enqueuing step
    # i + depth - 1).  The serial figure (one batch at a time) is reported
    # beside it.
    depth = args.e2e_depth
    pinned = [pinned_copy(torch, t) for t in traces]
    pin_fold = pinned_copy(torch, fold_in)
    htr = [(pt_.data_ptr(), lh, w, C3_LOG_B, SHIFT) for pt_, (lh, w) in zip(pinned, shapes)]
    fouts = [d_fout] + [ctx.alloc((1 << (fold_log - 1)) * 16) for _ in range(depth - 1)]
    plans_h = [P.Plan(ctx, P.BABYBEAR, htr, 0, fold=(pin_fold.data_ptr(), fo.ptr, fold_log, 1, beta), n_streams=0,
                      host=True) for fo in fouts]
    streams_h = [stream] + [torch.cuda.Stream(device=dev) for _ in range(depth - 1)]
    root_ptrs = []
    for ph in plans_h:
        nl = len(ph.tree.info()[0])
        root_ptrs.append(ph.tree.layer_ptr(nl - 1))
    roots = [torch.zeros(8, dtype=torch.int32, pin_memory=True) for _ in range(depth)]
    folds = [torch.zeros((1 << (fold_log - 1)) * 4, dtype=torch.int32, pin_memory=True) for _ in range(depth)]
    lib = P.load()

    def launch(i):
        j = i % depth
        plans_h[j].launch(streams_h[j].cuda_stream)

    def read(i):  # waits for step i, then copies its root and fold output to the host
        j = i % depth
        sp = streams_h[j].cuda_stream
        P.check(lib.p3g_memcpy_d2h(ctx.handle, roots[j].data_ptr(), root_ptrs[j], 32, sp))
        P.check(lib.p3g_memcpy_d2h(ctx.handle, folds[j].data_ptr(), fouts[j].ptr, folds[j].numel() * 4, sp))

    n_e2e = args.warmup + args.steps
    gc.collect()
    gc.disable()  # the interpreter's collector paused in the timed loops, as the timeit module does
    torch.cuda.synchronize(dev)
    done = []
    t_start = time.perf_counter()
    for i in range(min(depth - 1, n_e2e)):
        launch(i)
    for i in range(n_e2e):
        if i + depth - 1 < n_e2e:
            launch(i + depth - 1)
        read(i)
        done.append(time.perf_counter())
    torch.cuda.synchronize(dev)
    root_h = roots[(n_e2e - 1) % depth].numpy().view(np.uint32).copy()
    t0_timed = done[args.warmup - 1] if args.warmup > 0 else t_start
    e2e_total_ms = (done[-1] - t0_timed) * 1e3
    e2e_int = [(done[i] - done[i - 1]) * 1e3 for i in range(max(args.warmup, 1), n_e2e)]
    # serial: one batch at a time (launch, then read back), same host inputs
    serial_ms = []
    for i in range(args.warmup + max(args.steps // 2, 3)):
        t0 = time.perf_counter()
        launch(0)
        read(0)
        if i >= args.warmup:
            serial_ms.append((time.perf_counter() - t0) * 1e3)
    gc.enable()
    torch.cuda.synchronize(dev)
    assert np.array_equal(root_h, root_dev[0]), "host-input plan and device plan commit differently"
    assert np.array_equal(roots[0].numpy().view(np.uint32), root_dev[0])
    e2e_value, _ = job_throughput(float(elems) * args.steps, e2e_total_ms, dev)
    e2e_streams = plans_h[0].n_streams
    for ph in plans_h:
        ph.destroy()
    for fo in fouts[1:]:
        fo.free()
    del pinned, pin_fold
    kernels_per_step = plan.kernels_per_launch
    n_streams = plan.n_streams
    plan.destroy()
    for b in d_traces:
        b.free()
    d_fin.free()
    d_fout.free()
    torch.cuda.synchronize(dev)

    # ---- permutation ceiling: the same Poseidon2-16 on 2^22 register-resident
    # states (p3g_poseidon2_permute), no sponge or tree around it
    rng = np.random.default_rng(9)
    n_states = 1 << 22
    d_states = ctx.to_device(rng.integers(0, BB_P, size=(n_states, 16), dtype=np.uint32))
    perm_once = lambda: P.check(P.load().p3g_poseidon2_permute(ctx.handle, P.BABYBEAR, d_states.ptr, n_states, sptr))
    perm_once()
    perm_peak = n_states / (statistics.mean(events_timed(torch, dev, stream, perm_once, 10)) / 1e3)
    d_states.free()

    hbm, src = peaks()
    lde_bytes = sum(4 * w * ((1 << lh) + (1 << (lh + C3_LOG_B))) for lh, w in shapes)
    lde_gbs = lde_bytes / (lde_ms / 1e3) / 1e9
    bfly = lde_butterflies(shapes, C3_LOG_B)
    perms = sum((1 << (lh + C3_LOG_B)) * ((w + 7) // 8) for lh, w in shapes)
    result = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_per_step,
        "p50_ms": float(np.percentile(step_ms, 50)), "p99_ms": float(np.percentile(step_ms, 99)),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u32 (BabyBear)",
        "data": "synthetic",
        "config": {"workload": "config 3: batched commit of 64 BabyBear traces (log2 h uniform in {12..18}, width "
                               "uniform in [8, 512], log_blowup 1, shift 31, seeded) as one mixed-height "
                               "Poseidon2-16 (x^7, 8+13) MMCS, plus fold_matrix of a 2^19-row BabyBear^4 quotient "
                               "(log_arity 1, seeded beta), one CUDA graph launch per step",
                   "traces": 64, "lde_elements": elems, "trace_bytes": trace_bytes,
                   "height_shrink": args.c3_shrink,
                   "l2": (f"inputs larger than L2 ({trace_bytes / 2**20:.0f} MiB of traces, "
                          f"{elems * 4 / 2**20:.0f} MiB of LDEs); no flush") if trace_bytes > 129e6
                         else "inputs smaller than L2 (profiling case)",
                   "parallelism": f"replicas x{ws}"},
        "batched": {"graph_launches_per_step": 1, "kernels_per_step": int(kernels_per_step), "streams": n_streams,
                    "plan_seconds": plan_s},
        "plain_per_trace": plain,
        "batched_over_plain": (plain["ms_per_step"] / ms_per_step) if plain else None,
        "batched_over_plain_target": 2.0,
        "python_gc": "collected before, paused during the timed loops (as the timeit module does)",
        "e2e": {"value": e2e_value, "unit": UNIT,
                "h2d_bytes_per_step": trace_bytes + fold_in.nbytes,
                "d2h_bytes_per_step": 32 + folds[0].numel() * 4,
                "ms_per_step": e2e_total_ms / args.steps,
                "p50_ms": float(np.percentile(e2e_int, 50)), "p99_ms": float(np.percentile(e2e_int, 99)),
                "intervals_ms": [round(x, 3) for x in e2e_int], "streams": e2e_streams,
                "call": "p3g_plan_launch of p3g_plan_commit_host plans (64 pinned host traces and the quotient "
                        f"copied in by the graph every step), root and fold output read back every step; {args.e2e_depth} "
                        f"batches in flight on {args.e2e_depth} streams (p50/p99 over the intervals between step completions)",
                "serial": {"value": elems / (statistics.mean(serial_ms) / 1e3), "unit": UNIT,
                           "p50_ms": float(np.percentile(serial_ms, 50)),
                           "p99_ms": float(np.percentile(serial_ms, 99)),
                           "samples_ms": [round(x, 3) for x in serial_ms],
                           "note": "one batch at a time: launch, then read back"}},
        "gpu_launches": int(launches),
        "clocks": clocks,
        "roofline": {"kernel": "coset LDE stage of the 64 traces (k_lde_pass1/2/3, one stream)", "bound": "hbm",
                     "achieved": lde_gbs, "peak": hbm, "unit": "GB/s", "frac": lde_gbs / hbm,
                     "traffic": traffic_of("lde_bb_config3_bytes"), "peak_source": src,
                     "algorithmic_bytes": lde_bytes, "ms": lde_ms},
        "issue_bound_ms": {"lde": issue_bound_ms(bfly, clocks.get("sm_mhz")), "butterflies": bfly,
                           "basis": "6 ALU-pipe instructions per radix-2 butterfly, 16 lanes per SMSP per clock, "
                                    "608 SMSPs at the sampled SM clock"},
        "stages": {"lde_ms": lde_ms, "leaf_perms": perms, "perm_peak_per_s": perm_peak,
                   "leaf_hash_ms_at_perm_peak": perms / perm_peak * 1e3},
    }
    if not args.no_config1:
        result["config1"] = run_config1(P, torch, ctx, dev, stream, max(3, args.steps // 2), args.warmup,
                                        args.log_h, args.width, perm_peak)
    if not args.no_prover:
        result.update(run_prover(P, torch, ctx, dev, stream, perm_peak))
    if not args.no_goldilocks:
        result["config2"] = run_goldilocks(P, torch, ctx, dev, stream, max(3, args.steps // 2), args.warmup)
    if not args.no_serving:
        result["config4"] = run_serving(P, torch, ctx, [50, 100, 200, 500, 1000, 2000], args.serving_requests)
    if rank == 0 and not args.no_cpu:
        nt = os.cpu_count() or 1
        v, dt, desc = cpu_sample(nt, args.ref_shrink - 1)
        v1, dt1, desc1 = cpu_sample(1, 8)
        result["cpu_baseline"] = {"value": v, "unit": UNIT, "cores": nt, "kind": "port", "sample": desc,
                                  "seconds": dt,
                                  "single_thread": {"value": v1, "cores": 1, "sample": desc1, "seconds": dt1,
                                                    "note": "the reference's own CPU path is single-threaded"}}
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
    ap.add_argument("--no-plain", action="store_true", help="skip the per-trace comparison of the batched workload")
    ap.add_argument("--no-config1", action="store_true", help="skip the 2^20 x 256 single-trace commit")
    ap.add_argument("--no-goldilocks", action="store_true", help="skip the Goldilocks 2^18 x 128 commit")
    ap.add_argument("--no-serving", action="store_true", help="skip the serving-loop latency sweep")
    ap.add_argument("--no-prover", action="store_true",
                    help="skip the PCS-open, FRI and proof-of-work measurements (profiling the commit alone)")
    ap.add_argument("--serving-requests", type=int, default=10000, help="requests over the whole rate sweep")
    ap.add_argument("--e2e-depth", type=int, default=E2E_DEPTH,
                    help="batches the end-to-end leg keeps in flight (one host-input plan and stream each)")
    ap.add_argument("--c3-shrink", type=int, default=0,
                    help="divide every config-3 height by 2^k (profiling cases)")
    ap.add_argument("--ref-shrink", type=int, default=4,
                    help="the reference arm's CPU sample: config-3 heights divided by 2^k (the all-core "
                         "baseline of the GPU arm uses 2^(k-1))")
    ap.add_argument("--log-h", type=int, default=C1_LOG_H, help="config-1 trace log2 height (profiling cases)")
    ap.add_argument("--width", type=int, default=C1_WIDTH, help="config-1 trace width (profiling cases)")
    ap.add_argument("--case", default="",
                    help="profiling: lde|commit:bb|gl:LOG_H:WIDTH:LOG_B alone, or c3lde (the headline's LDE stage)")
    args = ap.parse_args()
    if args.impl == "reference":
        return run_reference(args)
    if args.case:
        return run_case(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
