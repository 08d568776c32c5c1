"""Benchmark: posterior elements/sec at 43 taxa (FP32 vs FP64 path).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gpu|reference]

A step runs one batch of the 43-taxon workload through the whole per-element
path (M0, M1, M2: Gibbs + Eval2 + output rows, 2,000 iterations each) on the
GPU.  The workload is synthetic with the shapes of the 43-taxon configuration:
Yule tree with total length 2.5 and 8 target taxa in 3 clades; element lengths
log-normal (median 250 bp, sigma 0.6, clipped 50-2000); 10% accelerated
(r2 ~ U[1.5, 4]) and r1 ~ U[0.2, 0.6]; 5% of (taxon, element) pairs missing and
3% gap cells; BURNIN 500 + MCMC 1500.

A step is one batch of E elements (default 1,216: two per resident chain, four
chains per SM) of the FP32-partial path, served and batched: the W warm-up
batches and then the K timed batches are each submitted at once to a serving
context, whose persistent kernel (one CTA per chain) takes elements from a
host-fed queue as chains finish, so a batch's tail overlaps the next batch.
--serve-sweeps 0 runs the same kernel as one batched launch per step instead.

value     = K * E / device time of the persistent launch (inputs resident)
e2e       = K * E / wall time through pacc_submit/pacc_poll from host buffers
            (preprocessing, H2D admission, sweeps, D2H of results inside)
fp64      = the plain FP64 path (one CTA per chain, one launch) on a batch of
            the same workload, the baseline of the FP32/FP64 ratio
serving   = an open-loop Poisson stream at 80% of `value`: p50/p99 latency
--impl reference runs the CPU oracle (the restatement of PhyloAcc-ST's
path; the unmodified reference needs GSL/Armadillo, absent here) on all host
cores over a bounded sample of the same workload.
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


# DRAM bytes per column-node update of chain_kernel<float> (ncu capture of
# 608 elements x 60 iterations: 59.7 GB over 1.666e9 updates)
DRAM_BYTES_PER_UPDATE = 35.8


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


def run_reference(args, ws, rank):
    if rank != 0:
        return
    cores = os.cpu_count() or 1
    ds = make_workload(max(cores, 1) * 2, seed=0)
    vals = []
    for step in range(args.warmup + args.steps):
        sub = ds.subset(list(range((step % 2) * cores, (step % 2) * cores + cores)))
        v, dt = cpu_baseline(sub, cores, cores)
        if step >= args.warmup:
            vals.append((v, dt))
    v = float(np.mean([x[0] for x in vals]))
    ms = float(np.mean([x[1] for x in vals])) * 1e3
    sample = "%d elements per step (one per host core) of the 43-taxon workload, full 2,000 iterations x 3 models" % cores
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": "elements/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": WORKLOAD, "elements_per_step": cores, "parallelism": "OpenMP over elements"},
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


def serve_latency(ds, throughput, seconds, sweeps, seed=1):
    """Open-loop serving at 80% of the batch throughput.

    Elements arrive as a Poisson process (rate 0.8 x throughput, cycling
    through the workload); each poll runs one sweep step of the resident
    chains and retires the finished ones.  Latency = time the result came back
    minus the element's scheduled arrival time, for elements arriving in the
    last two thirds of the window (after the slots have filled)."""
    import phyloacc_gb300 as pg
    from phyloacc_gb300 import abi
    o = opts_for(abi.PACC_FP32)
    o.sweeps_per_launch = sweeps
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
    return {"load": 0.8, "arrival_rate": rate, "window_s": seconds, "sweeps_per_launch": sweeps,
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


def run_gpu(args, ws, rank, local):
    import phyloacc_gb300 as pg
    from phyloacc_gb300 import abi
    if not os.path.exists(pg.LIB_PATH):
        from phyloacc_gb300.build import build
        build()
    E, K, W = args.elements, args.steps, args.warmup
    ds = make_workload(E, seed=100 + rank)
    # FP32 served/batched path: a step is one batch of E elements streamed
    # through the persistent chain kernel (continuous batching)
    o32 = opts_for(abi.PACC_FP32)
    o32.device = 0
    o32.sweeps_per_launch = args.serve_sweeps
    ctx32 = pg.Context(ds, o32)
    clocks = ClockSampler(local)
    keys = ("edge_updates_internal", "edge_updates_leaf", "tg_draws", "flop")
    if args.serve_sweeps > 0:
        serve_stream(ctx32, ds, W, ws)                   # W warm-up steps
        clocks.start()
        c0 = ctx32.counters()
        dev, wall, got = serve_stream(ctx32, ds, K, ws)  # K timed steps
        clk = clocks.stop()
        c1 = ctx32.counters()
        cnt = {k: c1[k] - c0[k] for k in keys}
        launches = int(c1["iterations"] - c0["iterations"])
    else:
        # the same kernel without serving: one launch per batch of E elements
        kern, walls, c_last, res = time_gpu(ctx32, ds, K, W, ws, clocks)
        clk = clocks.stop()
        dev, wall, got = float(np.sum(kern)), float(np.sum(walls)), [res]
        cnt = {k: c_last[k] * K for k in keys}          # every step runs the same batch
        launches = K
    value = ws * E * K / dev
    e2e = ws * E * K / wall
    h2d = int(ds.bases.nbytes + ds.lengths.nbytes + ds.offsets.nbytes)
    d2h = int(E * (3 * 9 * 8 + 64))
    dev_ms = np.concatenate([[r.arr[i].device_ms for i in range(r.n)] for r in got])
    # FP64 plain path (one CTA per chain, all elements in one launch)
    E64 = args.fp64_elements
    if args.no_fp64:
        k64, c64, v64 = [float("nan")], {"flop": float("nan")}, float("nan")
    else:
        ds64 = ds.subset(list(range(E64)))
        ctx64 = pg.Context(ds64, opts_for(abi.PACC_FP64))
        ctx64.run(ds.subset(list(range(152))))           # warm-up on one element per SM
        k64, w64, c64, _ = time_gpu(ctx64, ds64, 1, 0, ws)
        v64 = ws * E64 / float(np.mean(k64))
    fp64_peak, fp32_peak = pg.measure_fma_peak(0)
    achieved = cnt["flop"] / dev
    updates = (cnt["edge_updates_internal"] + cnt["edge_updates_leaf"]) / 2
    # DRAM traffic of the launch: bytes per column-node update from one ncu
    # capture of this kernel on a smaller case of the same workload
    # (dram__bytes_read.sum + dram__bytes_write.sum, 608 elements x 60
    # iterations), scaled by the updates this launch made
    traffic = DRAM_BYTES_PER_UPDATE * updates
    hbm_peak, hbm_src = hbm_peak_gbs()
    line = {
        "metric": METRIC, "value": value, "unit": "elements/s", "n_gpus": ws, "steps": K,
        "warmup": W, "ms_per_step": dev / K * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "fp32-partials+fp64", "data": "synthetic",
        "config": {"workload": WORKLOAD, "elements_per_step": E,
                   "path": ("FP32 partials, served and batched: one CTA per chain, a persistent kernel taking "
                            "elements from a host-fed queue (continuous batching)") if args.serve_sweeps > 0 else
                           "FP32 partials, batched: one CTA per chain, one launch per batch",
                   "l2": "inputs larger than L2 (resident chain state and partial buffers)",
                   "parallelism": "replicas" if ws > 1 else "single GPU"},
        "e2e": {"value": e2e, "unit": "elements/s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
        "gpu_launches": launches,
        "roofline": {"bound": "fp32", "achieved": achieved / 1e12, "peak": fp32_peak / 1e12, "unit": "TFLOP/s",
                     "frac": achieved / fp32_peak, "traffic": traffic,
                     "work": "36 flop per internal-child edge-column + 4 per leaf-child edge-column (device counters)",
                     "peak_source": "measured FP32 FMA rate of this GPU (pacc_measure_fma_peak)",
                     "traffic_source": "%.1f DRAM bytes per column-node update (ncu, 608 elements x 60 iterations) "
                                       "x the launch's updates" % DRAM_BYTES_PER_UPDATE,
                     "hbm": {"achieved": traffic / dev / 1e9, "peak": hbm_peak, "unit": "GB/s",
                             "frac": traffic / dev / 1e9 / hbm_peak, "peak_source": hbm_src}},
        "column_node_updates_per_s": updates / dev,
        "fp64": {"value": v64, "unit": "elements/s", "elements_per_step": E64,
                 "path": "plain FP64, one CTA per chain, one launch",
                 "achieved_tflops": c64["flop"] / float(np.mean(k64)) / 1e12,
                 "peak_tflops": fp64_peak / 1e12,
                 "frac": c64["flop"] / float(np.mean(k64)) / fp64_peak},
        "fp32_over_fp64": value / v64,
        "element_device_ms": {"p50": float(np.percentile(dev_ms, 50)), "p99": float(np.percentile(dev_ms, 99))},
        "counters": cnt,
        "clocks": clk,
    }
    if args.serve_seconds > 0:
        line["serving"] = serve_latency(ds, value / ws, args.serve_seconds, args.serve_sweeps)
        line["latency_ms"] = {"p50": line["serving"]["p50_ms"], "p99": line["serving"]["p99_ms"]}
    if rank == 0 and not args.no_cpu:
        cores = os.cpu_count() or 1
        v, dt = cpu_baseline(ds, cores, cores)
        line["cpu_baseline"] = {"value": v, "unit": "elements/s", "cores": cores, "kind": "port",
                                "sample": "%d elements of the same workload, one per host core, %.1f s" % (cores, dt)}
    if rank == 0:
        print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=2)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gpu", choices=["gpu", "reference"])
    ap.add_argument("--elements", type=int, default=1216,
                    help="elements per step (default: two per resident chain, four chains per SM)")
    ap.add_argument("--fp64-elements", type=int, default=912)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-fp64", action="store_true")
    ap.add_argument("--serve-seconds", type=float, default=60.0,
                    help="arrival window of the 80%%-load serving run (0: skip)")
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
    else:
        os.environ.setdefault("CUDA_VISIBLE_DEVICES", str(local)) if ws > 1 else None
        run_gpu(args, ws, rank, local)
    if ws > 1:
        import torch.distributed as td
        td.destroy_process_group()


if __name__ == "__main__":
    main()
