"""Benchmark: posterior elements/sec at 43 taxa (FP32 vs FP64 path).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gpu|reference]

A step runs one batch of the 43-taxon workload through the whole per-element
path (M0, M1, M2: Gibbs + Eval2 + output rows, 2,000 iterations each) on the
GPU.  The workload is synthetic with the shapes of the 43-taxon configuration:
Yule tree with total length 2.5 and 8 target taxa in 3 clades; element lengths
log-normal (median 250 bp, sigma 0.6, clipped 50-2000); 10% accelerated
(r2 ~ U[1.5, 4]) and r1 ~ U[0.2, 0.6]; 5% of (taxon, element) pairs missing and
3% gap cells; BURNIN 500 + MCMC 1500.

A step is one batch of E elements (default 1,216, eight per SM) of the
FP32-partial path, served and batched: the W warm-up batches and then the K
timed batches are each submitted at once to a serving context, whose
persistent kernel (one CTA per chain) takes elements from a host-fed queue
as chains finish, so a batch's tail overlaps the next batch.  The kernel's
launch shape (threads per chain, registers a thread, chains per SM) is the
trial-launch tuner's choice, made during the first warm-up batch and
recorded in config.launch_shape.  --serve-sweeps 0 runs the same kernel as
one batched launch per step instead.

value     = K * E / device time of the persistent launch (inputs resident)
e2e       = K * E / wall time through pacc_submit/pacc_poll from host buffers
            (preprocessing, H2D admission, sweeps, D2H of results inside)
fp64      = FP64 partials (the plain path's kernel) on the first E64 (default
            304) elements of the same batch, streamed through the same serving
            machinery for the same K timed and W warm-up steps (value: device
            time, e2e: wall time); the baseline of the FP32/FP64 ratio
error     = FP32 against that FP64 leg on the same elements: posterior
            P(accelerated) per branch and both log Bayes factors (Monte-Carlo
            differences of two chains), and the FP32 likelihood kernel's
            relative error at a fixed state per element
config1   = the 12-taxon configuration (100 elements, BURNIN 500 + MCMC 1000,
            seed 0), FP32 and FP64, K timed steps each, with e2e
serving   = the serving form of the 43-taxon workload: an open-loop Poisson
            stream at 80% of `value` of elements whose lengths are log-normal
            (median 250 bp, sigma 0.6) clipped at 50-5000 (--serve-elements
            distinct elements of the same tree, cycled), admitted against a
            150 GB device-memory budget: p50/p99 latency from arrival to result
gbgc      = the gBGC model's configuration (PhyloAcc-ST-GBGC): 120-taxon Yule
            tree (total length 4.0, 20 targets in 6 clades), elements log-normal
            (median 300 bp, clipped 50-3000) with a GC-bias strength ~ Gamma(2, 1)
            each; BURNIN 200 + MCMC 800 (that program's defaults); M0, M2, M1 with
            Eval2 and the rate / B / Z tables.  A step is one pacc_gbgc_run of
            --gbgc-elements elements from host buffers (value: device time; e2e:
            wall time incl. preprocessing, H2D, D2H of the traces and the host's
            Eval2); FP32 partials served (the K steps' batches submitted at
            once to the persistent kernel, elements admitted as slots free up;
            --gbgc-batched: one launch per step), with an FP64-partial leg on the same batch
            over 40 + 160 iterations, scaled to 1,000; cpu_baseline: the oracle on one element per host core,
            OpenMP over elements, over a bounded chain scaled to 1,000 iterations
cpu_baseline and --impl reference run the CPU oracle (the restatement of
PhyloAcc-ST's path in its own log-space arithmetic) on the host cores over
elements taken from the start of the same batch: one element per core per
step, step s of the reference arm taking elements s*cores..; cpu_baseline is
step 0's sample.
Multi-GPU: replicas (elements are independent; no collective), weak scaling.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "posterior elements/sec at 43 taxa (FP32 vs FP64 path); p50/p99 element latency"
WORKLOAD = ("43-taxon Yule tree (total length 2.5, 8 targets in 3 clades); elements log-normal "
            "(median 250 bp, sigma 0.6, clipped 50-2000), 10% accelerated; BURNIN 500 + MCMC 1500; "
            "M0+M1+M2 with Eval2 and output rows per element")


def dist_init():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if ws > 1:
        import torch.distributed as td
        os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
        td.init_process_group("gloo", rank=rank, world_size=ws)
    return ws, rank, local


def barrier(ws):
    if ws > 1:
        import torch.distributed as td
        td.barrier()


def reduce_max(ws, x):
    if ws == 1:
        return x
    import torch
    import torch.distributed as td
    t = torch.tensor([float(x)], dtype=torch.float64)
    td.all_reduce(t, op=td.ReduceOp.MAX)
    return float(t.item())


class ClockSampler:
    """nvidia-smi clocks and throttle reasons during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.rows = []
        self.p = None

    def start(self):
        try:
            self.p = subprocess.Popen(["nvidia-smi", "-i", str(self.device), "--query-gpu=" + self.Q,
                                       "--format=csv,noheader,nounits", "-lms", "200"],
                                      stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.p = None

    def _read(self):
        for ln in self.p.stdout:
            self.rows.append([x.strip() for x in ln.split(",")])

    def stop(self):
        if self.p is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.p.terminate()
        try:
            self.p.wait(timeout=5)
        except Exception:
            self.p.kill()
        sm = [float(r[1]) for r in self.rows if len(r) >= 9 and r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in self.rows if len(r) >= 9 and r[2].replace(".", "").isdigit()]
        reasons = set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in self.rows:
            if len(r) >= 9:
                for n, v in zip(names, r[5:9]):
                    if v.strip().lower() == "active":
                        reasons.add(n)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def make_workload(n, seed):
    from phyloacc_gb300 import synth
    ds = synth.make_dataset("st43", n_elements=n, seed=seed)
    return ds


ITERS = {"burnin": 500, "mcmc": 1500}


# DRAM bytes per column-node update of chain_kernel<float> in the shape the
# tuner serves with (ncu capture of 608 elements x 60 iterations, 128 threads
# x 128 registers, four chains an SM: 55.1 GB over 1.666e9 updates; the
# 255-register shape moved 28.5 bytes an update)
DRAM_BYTES_PER_UPDATE = 33.1


def hbm_peak_gbs():
    """The measured copy bandwidth of this machine's GPUs, else the fallback."""
    try:
        with open(os.path.join(os.path.dirname(os.path.abspath(__file__)), "MEASURED_PEAKS.json")) as f:
            return float(json.load(f)["hbm_gbs"]), "of measured (MEASURED_PEAKS.json hbm_gbs)"
    except (OSError, KeyError, ValueError):
        return 6800.0, "of fallback (6.8 TB/s)"


def opts_for(precision):
    from phyloacc_gb300 import abi
    o = abi.default_opts()
    o.burnin, o.mcmc, o.seed = ITERS["burnin"], ITERS["mcmc"], 0
    o.precision = precision
    return o


def cpu_baseline(ds, n_sample, threads):
    from oracle import pyoracle
    sub = ds.subset(list(range(n_sample)))
    o = opts_for(0)
    t = time.time()
    pyoracle.run(sub, o, threads=threads)
    dt = time.time() - t
    return n_sample / dt, dt


# The workload every arm measures: the GPU arm's batch (43 taxa, seed 100 for
# rank 0).  The CPU figures take their elements from the start of that batch.
WORKLOAD_SEED = 100


def run_reference(args, ws, rank):
    """The reference's algorithm on the host cores (the oracle, OpenMP over
    elements like main.cpp:452).  Step s runs one element per core: elements
    [s*cores, (s+1)*cores) of the GPU arm's batch (wrapping), so the K timed
    steps together cover the first K*cores elements of that batch and step 0
    is the same sample as the GPU line's cpu_baseline.  value = elements of
    the timed steps / their summed wall time."""
    if rank != 0:
        return
    cores = os.cpu_count() or 1
    E = args.elements
    ds = make_workload(E, seed=WORKLOAD_SEED)
    n_done, t_sum = 0, 0.0
    for step in range(args.warmup + args.steps):
        s = step - args.warmup if step >= args.warmup else step
        idx = [(s * cores + i) % E for i in range(cores)]
        v, dt = cpu_baseline(ds.subset(idx), cores, cores)
        if step >= args.warmup:
            n_done += cores
            t_sum += dt
    v = n_done / t_sum
    ms = t_sum / args.steps * 1e3
    sample = ("%d elements per step (one per host core) of the GPU arm's %d-element batch (seed %d), step s "
              "taking elements s*%d.., %d elements over the timed steps; full 2,000 iterations x 3 models"
              % (cores, E, WORKLOAD_SEED, cores, n_done))
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": "elements/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": WORKLOAD, "elements_per_step": cores, "batch_seed": WORKLOAD_SEED,
                       "parallelism": "OpenMP over elements"},
            "cpu_baseline": {"value": v, "unit": "elements/s", "cores": cores, "kind": "port", "sample": sample},
            "e2e": {"value": v, "unit": "elements/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def time_gpu(ctx, ds, steps, warmup, ws, clocks=None):
    """Returns per-step (kernel_s, wall_s) lists (max over ranks) and the last counters."""
    kern, wall = [], []
    cnt = None
    res = None
    for step in range(warmup + steps):
        timed = step >= warmup
        barrier(ws)
        if timed and clocks is not None and step == warmup:
            clocks.start()
        t = time.perf_counter()
        res = ctx.run(ds)
        dt = time.perf_counter() - t
        c = ctx.counters()
        if timed:
            kern.append(reduce_max(ws, c["kernel_ms"] * 1e-3))
            wall.append(reduce_max(ws, dt))
            cnt = c
    return kern, wall, cnt, res


# device memory the serving form of the workload admits chains against
SERVE_BUDGET_BYTES = 150 * 10**9


def serve_latency(ds, throughput, seconds, sweeps, seed=1):
    """Open-loop serving at 80% of the batch throughput.

    Elements arrive as a Poisson process (rate 0.8 x throughput, cycling
    through ds); the host feeds the persistent kernel's queue as they arrive
    and retires results as chains finish.  Latency = time the result came back
    minus the element's scheduled arrival time, for elements arriving in the
    last two thirds of the window (after the slots have filled)."""
    import phyloacc_gb300 as pg
    from phyloacc_gb300 import abi
    o = opts_for(abi.PACC_FP32)
    o.sweeps_per_launch = sweeps
    o.memory_budget_bytes = SERVE_BUDGET_BYTES
    ctx = pg.Context(ds, o)
    rate = 0.8 * throughput
    rng = np.random.default_rng(seed)
    n_max = int(rate * seconds * 1.5) + 16
    arrive = np.cumsum(rng.exponential(1.0 / rate, n_max))
    arrive = arrive[arrive < seconds]
    E = ds.n_elements
    measured = {k for k in range(len(arrive)) if arrive[k] >= seconds / 3}
    lat = {}
    k_next = 0
    t0 = time.perf_counter()
    while True:
        now = time.perf_counter() - t0
        k_end = int(np.searchsorted(arrive, now, side="right"))
        if k_end > k_next:
            idx = [k % E for k in range(k_next, k_end)]
            ctx.submit(ds.subset(idx), element_no=np.arange(k_next, k_end))
            k_next = k_end
        if ctx.pending() > 0:
            r = ctx.poll(4096, buffers=False)
            t = time.perf_counter() - t0
            for i in range(r.n):
                k = int(r.arr[i].element_no)
                if k in measured:
                    lat[k] = (t - arrive[k]) * 1e3
        else:
            time.sleep(0.001)
        if k_next >= len(arrive) and measured.issubset(lat.keys()):
            break
        if time.perf_counter() - t0 > 6 * seconds + 600:
            break
    wall = time.perf_counter() - t0
    ctx.close()
    v = np.array(list(lat.values()))
    lens = np.array([ds.element(e).shape[1] for e in range(E)])
    return {"load": 0.8, "arrival_rate": rate, "window_s": seconds, "sweeps_per_launch": sweeps,
            "elements": {"distinct": E, "length_median": float(np.median(lens)), "length_max": int(lens.max()),
                         "clip": [50, 5000]},
            "memory_budget_bytes": SERVE_BUDGET_BYTES,
            "elements_measured": int(len(v)), "elements_submitted": int(k_next),
            "p50_ms": float(np.percentile(v, 50)) if len(v) else None,
            "p99_ms": float(np.percentile(v, 99)) if len(v) else None,
            "wall_s": wall}


def serve_stream(ctx, ds, n_batches, ws):
    """Streams n_batches copies of the workload through the serving context
    (submitted at once, longest elements admitted first; chains are admitted
    as slots free up, so no batch waits for another's tail).  Returns (device seconds
    of the sweeps, wall seconds, results)."""
    E = ds.n_elements
    stream = ds.subset(list(range(E)) * n_batches)
    k0 = ctx.counters()["kernel_ms"]
    barrier(ws)
    t = time.perf_counter()
    ctx.submit(stream, element_no=np.arange(n_batches * E))
    got = []
    while ctx.pending() > 0:
        r = ctx.poll(4096, buffers=False)
        if r.n:
            got.append(r)
    wall = time.perf_counter() - t
    dev = (ctx.counters()["kernel_ms"] - k0) * 1e-3
    return reduce_max(ws, dev), reduce_max(ws, wall), got


def by_element(got, n_per_step):
    """element index within the batch -> (Results, row), from the first
    served step (element_no = step * E + e)."""
    out = {}
    for r in got:
        for i in range(r.n):
            no = int(r.arr[i].element_no)
            if no < n_per_step:
                out[no] = (r, i)
    return out


def summary_error(ctx32_res, res64, ds, E64):
    """FP32 against FP64 on the FP64 leg's elements: differences of the
    posterior P(accelerated) per branch and of both log Bayes factors
    (Monte-Carlo differences of two chains), and the relative error of the
    FP32 likelihood kernel at a fixed state per element (each element's M2
    Max_Z of the FP64 run at its median rates), which is deterministic."""
    import phyloacc_gb300 as pg
    from phyloacc_gb300 import abi
    p32, p64, bf1, bf2 = [], [], [], []
    for e in range(E64):
        r, i = ctx32_res[e]
        if r.arr[i].status != abi.PACC_OK or res64.arr[e].status != abi.PACC_OK:
            continue
        a = [r.arr[i].model[m].loglik for m in range(3)]
        b = [res64.arr[e].model[m].loglik for m in range(3)]
        if all(np.isfinite(a)) and all(np.isfinite(b)):
            bf1.append(abs((a[1] - a[0]) - (b[1] - b[0])))
            bf2.append(abs((a[1] - a[2]) - (b[1] - b[2])))
        if r.post_z is not None:
            p32.append(r.post_z[i, 1:, :, 3])
            p64.append(res64.post_z[e, 1:, :, 3])
    out = {"elements": E64, "compared": len(bf1)}
    if p32:
        d = np.abs(np.array(p32) - np.array(p64))
        out["pacc_abs_max"] = float(d.max())
        out["pacc_abs_mean"] = float(d.mean())
    if bf1:
        out["logbf1_abs_max"], out["logbf1_abs_median"] = float(np.max(bf1)), float(np.median(bf1))
        out["logbf2_abs_max"], out["logbf2_abs_median"] = float(np.max(bf2)), float(np.median(bf2))
    # likelihood kernel at a fixed state
    o32, o64 = opts_for(abi.PACC_FP32), opts_for(abi.PACC_FP64)
    n_ll = min(E64, 64)
    sub = ds.subset(list(range(n_ll)))
    c32, c64 = pg.Context(sub, o32), pg.Context(sub, o64)
    rel = []
    for e in range(n_ll):
        if res64.arr[e].status != abi.PACC_OK:
            continue
        z = res64.max_z[e, 2].astype(np.int32)
        m = res64.arr[e].model[2]
        a = c32.loglik(e, z, m.c_rate, m.n_rate).sum()
        b = c64.loglik(e, z, m.c_rate, m.n_rate).sum()
        rel.append(abs(a - b) / abs(b))
    c32.close()
    c64.close()
    if rel:
        out["loglik_rel_max"] = float(np.max(rel))
        out["loglik_rel_p99"] = float(np.percentile(rel, 99))
        out["loglik_elements"] = len(rel)
    out["note"] = ("pacc/logbf: FP32 vs FP64 chains on the same elements and seed (Monte-Carlo differences; the "
                   "GPU tests bound them by the Monte-Carlo error); loglik: the FP32 likelihood kernel against FP64 "
                   "at each element's M2 Max_Z and median rates")
    return out


def run_gpu(args, ws, rank, local):
    import phyloacc_gb300 as pg
    from phyloacc_gb300 import abi
    if not os.path.exists(pg.LIB_PATH):
        from phyloacc_gb300.build import build
        build()
    E, K, W = args.elements, args.steps, args.warmup
    ds = make_workload(E, seed=WORKLOAD_SEED + rank)
    # FP32 served/batched path: a step is one batch of E elements streamed
    # through the persistent chain kernel (continuous batching)
    o32 = opts_for(abi.PACC_FP32)
    o32.device = 0
    o32.sweeps_per_launch = args.serve_sweeps
    o32.trace_iters = 0
    o32.block_threads, o32.register_budget = args.block_threads, args.register_budget
    ctx32 = pg.Context(ds, o32)
    clocks = ClockSampler(local)
    keys = ("edge_updates_internal", "edge_updates_leaf", "tg_draws", "flop")
    first = None
    if args.serve_sweeps > 0:
        serve_stream(ctx32, ds, W, ws)                   # W warm-up steps (the first one tunes the shape)
        clocks.start()
        c0 = ctx32.counters()
        dev, wall, got = serve_stream(ctx32, ds, K, ws)  # K timed steps
        clk = clocks.stop()
        c1 = ctx32.counters()
        cnt = {k: c1[k] - c0[k] for k in keys}
        launches = int(c1["iterations"] - c0["iterations"])
        first = by_element(got, E)
    else:
        # the same kernel without serving: one launch per batch of E elements
        kern, walls, c_last, res = time_gpu(ctx32, ds, K, W, ws, clocks)
        clk = clocks.stop()
        dev, wall, got = float(np.sum(kern)), float(np.sum(walls)), [res]
        cnt = {k: c_last[k] * K for k in keys}          # every step runs the same batch
        launches = K
        first = {e: (res, e) for e in range(E)}
    shape = ctx32.launch_shape()
    value = ws * E * K / dev
    e2e = ws * E * K / wall
    h2d = int(ds.bases.nbytes + ds.lengths.nbytes + ds.offsets.nbytes)
    d2h = int(E * (3 * 9 * 8 + 64))
    dev_ms = np.concatenate([[r.arr[i].device_ms for i in range(r.n)] for r in got])
    # FP32 results with Max_Z / P(Z) buffers for the error comparison: the
    # first E64 elements once more (the chains are deterministic)
    E64 = min(args.fp64_elements, E)
    ds64 = ds.subset(list(range(E64)))
    # FP64 path: the same K timed and W warm-up steps through the same serving
    # stream as the FP32 headline (the persistent kernel taking elements as
    # chains finish), a step E64 elements from host buffers: value = device
    # time, e2e = wall time.  (One launch per small batch would time the
    # batch's longest chain, not the path.)
    fp64 = None
    err = None
    if not args.no_fp64:
        o64 = opts_for(abi.PACC_FP64)
        o64.sweeps_per_launch = max(args.serve_sweeps, 1)
        ctx64 = pg.Context(ds64, o64)
        serve_stream(ctx64, ds64, W, ws)
        k0 = ctx64.counters()
        dev64, wall64, got64 = serve_stream(ctx64, ds64, K, ws)
        k1 = ctx64.counters()
        v64 = ws * E64 * K / dev64
        fp64 = {"value": v64, "unit": "elements/s", "elements_per_step": E64, "steps": K, "warmup": W,
                "path": "FP64 partials (the plain path's kernel), served like the headline",
                "e2e": {"value": ws * E64 * K / wall64, "unit": "elements/s",
                        "h2d_bytes_per_step": int(ds64.bases.nbytes + ds64.lengths.nbytes + ds64.offsets.nbytes),
                        "d2h_bytes_per_step": int(E64 * (3 * 9 * 8 + 64))},
                "shape": ctx64.launch_shape()}
        fp64_flop = k1["flop"] - k0["flop"]
        fp64_s = dev64
        ctx64.close()
        c64b = pg.Context(ds64, opts_for(abi.PACC_FP64))
        res64 = c64b.run(ds64)
        c64b.close()
        c32b = pg.Context(ds64, opts_for(abi.PACC_FP32))
        res32 = c32b.run(ds64)
        c32b.close()
        err = summary_error({e: (res32, e) for e in range(E64)}, res64, ds, E64)
    fp64_peak, fp32_peak = pg.measure_fma_peak(0)
    achieved = cnt["flop"] / dev
    updates = (cnt["edge_updates_internal"] + cnt["edge_updates_leaf"]) / 2
    # DRAM traffic of the launch: bytes per column-node update from one ncu
    # capture of this kernel on a smaller case of the same workload
    # (dram__bytes_read.sum + dram__bytes_write.sum), scaled by the updates
    # this launch made
    traffic = DRAM_BYTES_PER_UPDATE * updates
    hbm_peak, hbm_src = hbm_peak_gbs()
    line = {
        "metric": METRIC, "value": value, "unit": "elements/s", "n_gpus": ws, "steps": K,
        "warmup": W, "ms_per_step": dev / K * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "fp32-partials+fp64", "data": "synthetic",
        "config": {"workload": WORKLOAD, "elements_per_step": E, "batch_seed": WORKLOAD_SEED,
                   "path": ("FP32 partials, served and batched: one CTA per chain, a persistent kernel taking "
                            "elements from a host-fed queue (continuous batching)") if args.serve_sweeps > 0 else
                           "FP32 partials, batched: one CTA per chain, one launch per batch",
                   "launch_shape": shape,
                   "l2": "inputs larger than L2 (resident chain state and partial buffers)",
                   "parallelism": "replicas" if ws > 1 else "single GPU"},
        "e2e": {"value": e2e, "unit": "elements/s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
        "gpu_launches": launches,
        "roofline": {"bound": "fp32", "achieved": achieved / 1e12, "peak": fp32_peak / 1e12, "unit": "TFLOP/s",
                     "frac": achieved / fp32_peak, "traffic": traffic,
                     "work": "36 flop per internal-child edge-column + 4 per leaf-child edge-column (device counters)",
                     "peak_source": "measured FP32 FMA rate of this GPU (pacc_measure_fma_peak)",
                     "traffic_source": "%.1f DRAM bytes per column-node update (ncu, 608 elements x 60 iterations, 128 x 128 shape) "
                                       "x the launch's updates" % DRAM_BYTES_PER_UPDATE,
                     "hbm": {"achieved": traffic / dev / 1e9, "peak": hbm_peak, "unit": "GB/s",
                             "frac": traffic / dev / 1e9 / hbm_peak, "peak_source": hbm_src}},
        "column_node_updates_per_s": updates / dev,
        "element_device_ms": {"p50": float(np.percentile(dev_ms, 50)), "p99": float(np.percentile(dev_ms, 99))},
        "counters": cnt,
        "clocks": clk,
    }
    if fp64 is not None:
        fp64["achieved_tflops"] = fp64_flop / fp64_s / 1e12
        fp64["peak_tflops"] = fp64_peak / 1e12
        fp64["frac"] = fp64_flop / fp64_s / fp64_peak
        line["fp64"] = fp64
        line["fp32_over_fp64"] = value / fp64["value"]
        line["error"] = err
    if not args.no_config1:
        line["config1"] = run_config1(K, W, ws)
    if args.gbgc_elements > 0:
        line["gbgc"] = run_gbgc(args, K, ws, rank)
    if args.serve_seconds > 0:
        from phyloacc_gb300 import synth
        ds_serve = synth.make_dataset("st43_serve", n_elements=args.serve_elements, seed=WORKLOAD_SEED + rank)
        line["serving"] = serve_latency(ds_serve, value / ws, args.serve_seconds, args.serve_sweeps)
        line["latency_ms"] = {"p50": line["serving"]["p50_ms"], "p99": line["serving"]["p99_ms"]}
    if rank == 0 and not args.no_cpu:
        cores = os.cpu_count() or 1
        v, dt = cpu_baseline(ds, cores, cores)
        line["cpu_baseline"] = {"value": v, "unit": "elements/s", "cores": cores, "kind": "port",
                                "sample": "elements 0..%d of this batch (one per host core), %.1f s; the same "
                                          "elements as step 0 of --impl reference" % (cores - 1, dt)}
    if rank == 0:
        print(json.dumps(line), flush=True)


GBGC_WORKLOAD = ("120-taxon Yule tree (total length 4.0, 20 targets in 6 clades); elements log-normal (median 300 "
                 "bp, sigma 0.6, clipped 50-3000), GC-bias strength ~ Gamma(2, 1) on 20% of branches, 10% "
                 "accelerated; '*' gaps 3%, 5% of (taxon, element) pairs missing; BURNIN 200 + MCMC 800; "
                 "M0 + M2 + M1 with Eval2 and tables per element")


def run_gbgc(args, K, ws, rank):
    """The gBGC model's leg: K timed steps (after one small warm-up) of
    --gbgc-elements elements each through pacc_gbgc_run."""
    import phyloacc_gb300 as pg
    from phyloacc_gb300 import abi, synth
    E = args.gbgc_elements
    ds = synth.make_dataset("gbgc120", n_elements=E, seed=WORKLOAD_SEED + rank)
    g = abi.gbgc_default_opts(ds.target)
    g.seed = 1
    if args.gbgc_burnin is not None:
        g.burnin, g.mcmc = args.gbgc_burnin, args.gbgc_mcmc
    out = {"workload": GBGC_WORKLOAD, "metric": "posterior elements/sec (gBGC model, 120 taxa)",
           "unit": "elements/s", "elements_per_step": E, "steps": K,
           "warmup": "served: the 8 longest elements once; batched: one 8-element, 10-iteration run",
           "path": "one CTA per element, persistent kernel fed from a host queue (served) or over one "
                   "batch's queue (batched, longest first); FP64 Pade branch matrices; FP32 partials"}
    # FP32 partials, served: the K steps' batches submitted at once to the
    # serving kernel (elements admitted as slots free up, so no batch waits
    # for another's tail); value = elements / device time of the launches,
    # e2e = elements / wall time from submit to the last poll
    if not args.gbgc_batched:
        o = abi.default_opts()
        o.precision = abi.PACC_FP32
        ctx = pg.Context(ds, o)
        longest = list(np.argsort(-ds.lengths)[:8])
        ctx.gbgc_submit(g, elements=longest)         # warm-up: slots sized for the longest element
        ctx.gbgc_sync()
        ctx.gbgc_poll()
        barrier(ws)
        k0 = ctx.counters()["kernel_ms"]
        f0 = ctx.counters()["flop"]
        ph0 = np.array(ctx.counters()["phase_cycles"])
        t = time.perf_counter()
        for _ in range(K):
            ctx.gbgc_submit(g)
        got = []
        while len(got) < K * E:
            got += ctx.gbgc_poll()
            if len(got) < K * E:
                time.sleep(0.005)
        ctx.gbgc_sync()
        wall = reduce_max(ws, time.perf_counter() - t)
        dev = reduce_max(ws, (ctx.counters()["kernel_ms"] - k0) * 1e-3)
        ph = np.array(ctx.counters()["phase_cycles"]) - ph0
        flop = ctx.counters()["flop"] - f0
        ctx.close()
        fp64_peak, _ = pg.measure_fma_peak(0)
        T = g.burnin + g.mcmc
        lat = np.array([r["device_ms"] for r in got])
        out["fp32"] = {"value": ws * K * E / dev, "unit": "elements/s", "elements_per_step": E, "steps": K,
                       "iterations": T, "ms_per_step": dev / K * 1e3, "path": "served (pacc_gbgc_submit / poll)",
                       "e2e": {"value": ws * K * E / wall, "unit": "elements/s",
                               "h2d_bytes_per_step": int(ds.bases.nbytes + ds.lengths.nbytes + ds.offsets.nbytes),
                               "d2h_bytes_per_step": int(E * 3 * T * (4 * 8 + 2 * ds.tree.n_nodes))},
                       "filtered": int(sum(1 for x in got if x["status"] != 0)) // K,
                       "latency_submit_to_result_ms": {"p50": float(np.percentile(lat, 50)),
                                                       "p99": float(np.percentile(lat, 99))},
                       "roofline": {"bound": "fp64", "achieved": flop / dev / 1e12, "peak": fp64_peak / 1e12,
                                    "unit": "TFLOP/s", "frac": flop / dev / fp64_peak,
                                    "work": "FP64 flops of the Pade solves (34 m + 198 + 128 squarings per branch "
                                            "matrix, device counters); the kernel's other FP64 work is not counted",
                                    "peak_source": "measured FP64 FMA rate of this GPU (pacc_measure_fma_peak)",
                                    "traffic": None},
                       "phase_share": {n: float(v / max(ph.sum(), 1.0)) for n, v in zip(
                           ("monitor_and_setup", "expected_counts", "initial_prob_back", "pade_branch_matrices",
                            "rest_of_sample_rates", "update_zb", "pruning", "elbo_and_mh"), ph)}}
    # FP64 partials: the same batch on chains of a fifth of the length (the
    # cost of an iteration does not change along the chain), scaled to 1,000
    g64 = abi.gbgc_default_opts(ds.target)
    g64.seed, g64.burnin, g64.mcmc = 1, 40, 160
    legs = (("fp32", abi.PACC_FP32, g, K), ("fp64", abi.PACC_FP64, g64, 1))
    if not args.gbgc_batched:
        legs = legs[1:]
    if args.gbgc_fp32_only:
        legs = [l for l in legs if l[0] == "fp32"]
    for name, prec, gg, steps in legs:
        o = abi.default_opts()
        o.precision = prec
        ctx = pg.Context(ds, o)
        gw = abi.gbgc_default_opts(ds.target)
        gw.seed, gw.burnin, gw.mcmc = 1, 2, 8
        ctx.gbgc_run(gw, elements=range(8))            # warm-up: module load, first allocations
        kern, wall = [], []
        for _ in range(steps):
            barrier(ws)
            c0 = ctx.counters()["kernel_ms"]
            t = time.perf_counter()
            r = ctx.gbgc_run(gg)
            dt = time.perf_counter() - t
            kern.append(reduce_max(ws, (ctx.counters()["kernel_ms"] - c0) * 1e-3))
            wall.append(reduce_max(ws, dt))
        ctx.close()
        T = gg.burnin + gg.mcmc
        scale = T / float(g.burnin + g.mcmc)
        leg = {"value": ws * E * steps / float(np.sum(kern)) * scale, "unit": "elements/s", "elements_per_step": E,
               "steps": steps, "iterations": T, "ms_per_step": float(np.mean(kern)) * 1e3,
               "e2e": {"value": ws * E * steps / float(np.sum(wall)) * scale, "unit": "elements/s",
                       "h2d_bytes_per_step": int(ds.bases.nbytes + ds.lengths.nbytes + ds.offsets.nbytes),
                       "d2h_bytes_per_step": int(E * 3 * T * (4 * 8 + 2 * ds.tree.n_nodes))},
               "filtered": int(sum(1 for x in r if x["status"] != 0))}
        if scale != 1.0:
            leg["note"] = "measured on %d-iteration chains, scaled to %d" % (T, g.burnin + g.mcmc)
        out[name] = leg
        if name == "fp64":
            # FP32 against these FP64 chains: the same elements, seed and chain
            # length (the marginal likelihoods are Monte Carlo estimates of two
            # chains that part at the first MH decision FP32 rounding moves)
            o32 = abi.default_opts()
            o32.precision = abi.PACC_FP32
            c32 = pg.Context(ds, o32)
            r32 = c32.gbgc_run(gg)
            c32.close()
            rel = []
            for a, b in zip(r32, r):
                if a["status"] == 0 and b["status"] == 0:
                    for k in ("loglik_null", "loglik_res", "loglik_all"):
                        if np.isfinite(b[k]) and np.isfinite(a[k]):
                            rel.append(abs(a[k] - b[k]) / abs(b[k]))
            rel = np.array(rel) if rel else np.zeros(1)
            out["error"] = {"marginal_loglik_rel_max": float(rel.max()),
                            "marginal_loglik_rel_median": float(np.median(rel)), "values": int(rel.size),
                            "note": "FP32 against FP64 partials, %d elements x 3 models, %d-iteration chains" %
                                    (E, T)}
    out["value"] = out["fp32"]["value"]
    out["e2e"] = out["fp32"]["e2e"]
    if "fp64" in out:
        out["fp32_over_fp64"] = out["fp32"]["value"] / out["fp64"]["value"]
    if rank == 0 and not args.no_cpu:
        from oracle import pyoracle
        cores = os.cpu_count() or 1
        gc = abi.gbgc_default_opts(ds.target)
        gc.seed, gc.burnin, gc.mcmc = 1, 20, 80
        sub = ds.subset(list(range(cores)))
        t = time.time()
        pyoracle.gbgc_run_batch(sub, gc, threads=cores)
        dt = time.time() - t
        scale = (g.burnin + g.mcmc) / float(gc.burnin + gc.mcmc)
        out["cpu_baseline"] = {"value": cores / (dt * scale), "unit": "elements/s", "cores": cores, "kind": "port",
                               "sample": "elements 0..%d of this batch (one per host core), 20 + 80 iterations x 3 "
                                         "models in %.1f s, scaled to 200 + 800 (the chain's cost per iteration "
                                         "does not change along the chain)" % (cores - 1, dt)}
    return out


def run_config1(K, W, ws):
    """The 12-taxon configuration: 100 elements, BURNIN 500 + MCMC 1000,
    seed 0, FP32 and FP64 paths; a step is one launch over the 100 elements
    from host buffers."""
    import phyloacc_gb300 as pg
    from phyloacc_gb300 import abi, synth
    ds = synth.make_dataset("st12", n_elements=100, seed=0)
    out = {"workload": "12-taxon Yule tree (total length 1.2, one outgroup); 100 elements U{100..300} bp, 80 "
                       "conserved (r1 0.35), 20 accelerated (r2 2.5) on a 3-taxon clade; BURNIN 500 + MCMC 1000; "
                       "seed 0", "elements_per_step": 100}
    for name, prec in (("fp32", abi.PACC_FP32), ("fp64", abi.PACC_FP64)):
        o = abi.default_opts()
        o.burnin, o.mcmc, o.seed, o.precision = 500, 1000, 0, prec
        ctx = pg.Context(ds, o)
        kern, wall, _, _ = time_gpu(ctx, ds, K, W, ws)
        out[name] = {"value": ws * 100 * K / float(np.sum(kern)), "unit": "elements/s",
                     "e2e": {"value": ws * 100 * K / float(np.sum(wall)), "unit": "elements/s"},
                     "launch_shape": ctx.launch_shape()}
        ctx.close()
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=2)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gpu", choices=["gpu", "reference"])
    ap.add_argument("--elements", type=int, default=1216,
                    help="elements per step (default: two per resident chain, four chains per SM)")
    ap.add_argument("--fp64-elements", type=int, default=304,
                    help="elements per step of the FP64 leg (the first ones of the batch)")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-fp64", action="store_true")
    ap.add_argument("--no-config1", action="store_true")
    ap.add_argument("--gbgc-elements", type=int, default=760,
                    help="elements per step of the gBGC leg (0: skip; default five chains per SM)")
    ap.add_argument("--gbgc-only", action="store_true", help="profiling: run only the gBGC leg, print it")
    ap.add_argument("--gbgc-fp32-only", action="store_true", help="profiling: skip the gBGC FP64 leg")
    ap.add_argument("--gbgc-batched", action="store_true",
                    help="gBGC FP32 leg as one pacc_gbgc_run per step instead of served (the form ncu replays)")
    ap.add_argument("--gbgc-burnin", type=int, default=None, help="profiling only: shorter gBGC chains")
    ap.add_argument("--gbgc-mcmc", type=int, default=None, help="profiling only: shorter gBGC chains")
    ap.add_argument("--block-threads", type=int, default=0,
                    help="FP32 chain kernel: threads per chain (0: the tuner's choice)")
    ap.add_argument("--register-budget", type=int, default=0,
                    help="FP32 chain kernel: registers a thread, 128/168/255 (0: the tuner's choice)")
    ap.add_argument("--serve-seconds", type=float, default=60.0,
                    help="arrival window of the 80%%-load serving run (0: skip)")
    ap.add_argument("--serve-elements", type=int, default=4096,
                    help="distinct elements of the serving stream (lengths clipped 50-5000), cycled")
    ap.add_argument("--serve-sweeps", type=int, default=64,
                    help="serving on (>0) or off (0: one batched launch per step, the form an ncu "
                         "capture can replay)")
    ap.add_argument("--burnin", type=int, default=500, help="profiling only: shorter chains")
    ap.add_argument("--mcmc", type=int, default=1500, help="profiling only: shorter chains")
    args = ap.parse_args()
    ITERS["burnin"], ITERS["mcmc"] = args.burnin, args.mcmc
    ws, rank, local = dist_init()
    if args.impl == "reference":
        run_reference(args, ws, rank)
    elif args.gbgc_only:
        import phyloacc_gb300 as pg
        if not os.path.exists(pg.LIB_PATH):
            from phyloacc_gb300.build import build
            build()
        out = run_gbgc(args, args.steps, ws, rank)
        if rank == 0:
            print(json.dumps({"gbgc": out}), flush=True)
    else:
        os.environ.setdefault("CUDA_VISIBLE_DEVICES", str(local)) if ws > 1 else None
        run_gpu(args, ws, rank, local)
    if ws > 1:
        import torch.distributed as td
        td.destroy_process_group()


if __name__ == "__main__":
    main()
