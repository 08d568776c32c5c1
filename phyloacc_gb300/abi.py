"""ctypes mirror of include/pacc.h (structs and status codes).

The library itself is C/C++/CUDA; this module only describes its data layout
for Python callers (tests, bench.py, the host-side Python API in
phyloacc_gb300/__init__.py)."""
from __future__ import annotations

import ctypes as C

import numpy as np

PACC_OK = 0
PACC_FILTERED = 1
PACC_NAN_LIKELIHOOD = 2
PACC_SAMPLER_ERROR = 3
PACC_OOM = 4
PACC_TIMEOUT = 5
PACC_EINVAL = 6
PACC_ECUDA = 7
PACC_EBUSY = 8
PACC_EUNSUPPORTED = 9

PACC_FP64 = 0
PACC_FP32 = 1
PACC_FP64_BATCHED = 2
PACC_FP32_WARP = 3

_i32p = C.POINTER(C.c_int32)
_f64p = C.POINTER(C.c_double)
_u8p = C.POINTER(C.c_uint8)
_i64p = C.POINTER(C.c_int64)
_i8p = C.POINTER(C.c_int8)


class PaccModel(C.Structure):
    _fields_ = [
        ("n_species", C.c_int32),
        ("children", _i32p),
        ("distances", _f64p),
        ("pi", _f64p),
        ("rate_matrix", _f64p),
        ("outgroup", _i32p),
        ("n_outgroup", C.c_int32),
        ("conserve", _i32p),
        ("n_conserve", C.c_int32),
    ]


class PaccOpts(C.Structure):
    _fields_ = [
        ("burnin", C.c_int32), ("mcmc", C.c_int32), ("adapt_freq", C.c_int32), ("seed", C.c_uint32),
        ("init_conserve_rate", C.c_double), ("init_acce_rate", C.c_double),
        ("conserve_prior_a", C.c_double), ("conserve_prior_b", C.c_double),
        ("acce_prior_a", C.c_double), ("acce_prior_b", C.c_double),
        ("ropt", C.c_int32), ("cub", C.c_double), ("nlb", C.c_double),
        ("init_lrate", C.c_double), ("init_lrate2", C.c_double), ("init_grate", C.c_double),
        ("hyper_lrate_a", C.c_double), ("hyper_lrate_b", C.c_double),
        ("hyper_grate_a", C.c_double), ("hyper_grate_b", C.c_double),
        ("hyper_lrate2_a", C.c_double), ("hyper_lrate2_b", C.c_double),
        ("conserve_prop", C.c_double), ("gap_prop", C.c_double), ("cons_to_mis", C.c_double),
        ("gapchar", C.c_int32), ("prune_tree", C.c_int32), ("trim_gap_percent", C.c_double),
        ("min_len", C.c_int32), ("indel", C.c_double),
        ("precision", C.c_int32), ("device", C.c_int32), ("memory_budget_bytes", C.c_int64),
        ("max_resident", C.c_int32), ("sweeps_per_launch", C.c_int32), ("trace_iters", C.c_int32),
        ("block_threads", C.c_int32), ("use_graphs", C.c_int32), ("columns_per_lane", C.c_int32),
        ("chain", C.c_int32), ("sample_hyper", C.c_int32),
        ("serve_idle_ns", C.c_int64), ("register_budget", C.c_int32), ("reserved0", C.c_int32),
    ]


def default_opts() -> PaccOpts:
    """PhyloAcc-ST defaults (src/PhyloAcc-ST/main.cpp:36-90) plus GPU keys; the
    same values pacc_default_opts() writes."""
    o = PaccOpts()
    o.burnin, o.mcmc, o.adapt_freq, o.seed = 200, 800, 500, 5
    o.init_conserve_rate, o.init_acce_rate = 0.5, 1.0
    o.conserve_prior_a, o.conserve_prior_b = 5.0, 0.04
    o.acce_prior_a, o.acce_prior_b = 10.0, 0.2
    o.ropt, o.cub, o.nlb = 1, 1.0, 0.6
    o.init_lrate, o.init_lrate2, o.init_grate = 0.3, 0.1, 0.5
    o.hyper_lrate_a, o.hyper_lrate_b = 1.0, 9.0
    o.hyper_grate_a, o.hyper_grate_b = 3.0, 1.0
    o.hyper_lrate2_a, o.hyper_lrate2_b = 1.0, 9.0
    o.conserve_prop, o.gap_prop, o.cons_to_mis = 0.8, 0.8, 0.01
    o.gapchar, o.prune_tree, o.trim_gap_percent, o.min_len, o.indel = ord("-"), 0, 1.0, 50, 0.0
    o.precision, o.device, o.memory_budget_bytes = PACC_FP64, 0, 0
    o.max_resident, o.sweeps_per_launch, o.trace_iters = 0, 0, 0
    o.block_threads, o.use_graphs, o.columns_per_lane, o.chain, o.sample_hyper = 0, 1, 0, 0, 0
    o.serve_idle_ns, o.register_budget = 0, 0
    return o


class PaccElementBatch(C.Structure):
    _fields_ = [
        ("n_elements", C.c_int32),
        ("element_no", _i64p),
        ("lengths", _i32p),
        ("offsets", _i64p),
        ("bases", _u8p),
        ("start_z", C.POINTER(C.c_int8)),
        ("start_rates", C.POINTER(C.c_double)),
    ]


class PaccModelResult(C.Structure):
    _fields_ = [
        ("loglik", C.c_double), ("max_loglik", C.c_double),
        ("n_rate", C.c_double), ("c_rate", C.c_double), ("g_rate", C.c_double),
        ("l_rate", C.c_double), ("l2_rate", C.c_double),
        ("failure", C.c_int32), ("n_configs", C.c_int32),
    ]


class PaccTrace(C.Structure):
    _fields_ = [
        ("loglik", _f64p), ("n_rate", _f64p), ("c_rate", _f64p), ("g_rate", _f64p),
        ("l_rate", _f64p), ("l2_rate", _f64p), ("z", _i8p),
    ]


class PaccResult(C.Structure):
    _fields_ = [
        ("element_no", C.c_int64),
        ("status", C.c_int32),
        ("n_nodes", C.c_int32),
        ("model", PaccModelResult * 3),
        ("max_z", _i32p),
        ("post_z", _f64p),
        ("trace", PaccTrace),
        ("latency_ms", C.c_double),
        ("device_ms", C.c_double),
        ("end_z", C.POINTER(C.c_int8)),
        ("end_rates", C.c_double * 5),
    ]


class PaccCounters(C.Structure):
    _fields_ = [(n, C.c_double) for n in (
        "edge_updates_internal", "edge_updates_leaf", "column_loglik", "tg_draws", "z_draws",
        "pmatrix_builds", "iterations", "kernel_ms", "flop")] + [("phase_cycles", C.c_double * 8),
                                                                  ("serve_idle_exits", C.c_double)]


def ptr(a: np.ndarray, ctype):
    return a.ctypes.data_as(C.POINTER(ctype))


class PaccGbgcOpts(C.Structure):
    _fields_ = [
        ("burnin", C.c_int32), ("mcmc", C.c_int32), ("seed", C.c_uint32), ("gapchar", C.c_int32),
        ("conserve_rate", C.c_double), ("acce_rate", C.c_double), ("init_gc", C.c_double),
        ("conserve_prior_a", C.c_double), ("conserve_prior_b", C.c_double),
        ("acce_prior_a", C.c_double), ("acce_prior_b", C.c_double), ("acce_prior_shift", C.c_double),
        ("gc_prior_a", C.c_double), ("gc_prior_b", C.c_double), ("gc_prior_c", C.c_double),
        ("prep_lrate", C.c_double), ("prep_grate", C.c_double),
        ("cons_to_mis", C.c_double), ("ncons_to_mis", C.c_double),
        ("missing_thres", C.c_double), ("conserve_prop", C.c_double),
        ("prop_c", C.c_double), ("prop_n", C.c_double), ("prop_gc", C.c_double),
        ("target", C.POINTER(C.c_int32)), ("n_target", C.c_int32), ("chain", C.c_int32)]


def gbgc_default_opts(target=None) -> PaccGbgcOpts:
    """PhyloAcc-ST-GBGC's defaults (src/PhyloAcc-ST-GBGC/SRC/main.cpp:36-81,
    bpp.cpp:217-219, bpp_c.hpp:365-370); the values pacc_gbgc_default_opts()
    writes.  target: TARGETSPECIES node ids (kept alive on the object)."""
    o = PaccGbgcOpts()
    o.burnin, o.mcmc, o.seed, o.gapchar = 200, 800, 7728, ord("*")
    o.conserve_rate, o.acce_rate, o.init_gc = -2.0, 0.0, 3.0
    o.conserve_prior_a, o.conserve_prior_b = 5.0, 0.4
    o.acce_prior_a, o.acce_prior_b, o.acce_prior_shift = 5.0, 0.4, 2.0
    o.gc_prior_a, o.gc_prior_b, o.gc_prior_c = 4.0, 0.8, 0.2
    o.prep_lrate, o.prep_grate = 0.1, 0.8
    o.cons_to_mis, o.ncons_to_mis = 0.01, 0.1
    o.missing_thres, o.conserve_prop = 0.8, 0.8
    o.prop_c, o.prop_n, o.prop_gc = 1.2, 1.2, 0.2
    set_gbgc_target(o, target or [])
    return o


def set_gbgc_target(o: PaccGbgcOpts, target):
    arr = np.ascontiguousarray(target, dtype=np.int32)
    o._target_keep = arr
    o.target = ptr(arr, C.c_int32)
    o.n_target = len(arr)


class PaccGbgcResult(C.Structure):
    _fields_ = [
        ("element_no", C.c_int64), ("status", C.c_int32), ("root", C.c_int32),
        ("loglik_null", C.c_double), ("loglik_res", C.c_double), ("loglik_all", C.c_double),
        ("max_loglik", C.c_double * 3), ("rates", (C.c_double * 3) * 3), ("device_ms", C.c_double),
        ("max_z", C.POINTER(C.c_int32)), ("max_b", C.POINTER(C.c_int8)), ("post_b", C.POINTER(C.c_double)),
        ("post_z", C.POINTER(C.c_double)), ("trace", C.POINTER(C.c_double))]


class ModelArgs:
    """Keeps the numpy buffers behind a PaccModel alive."""

    def __init__(self, ds):
        t = ds.tree
        self.children = np.ascontiguousarray(t.children.reshape(-1), dtype=np.int32)
        self.distances = np.ascontiguousarray(t.distances, dtype=np.float64)
        self.pi = np.ascontiguousarray(ds.pi, dtype=np.float64)
        self.Q = np.ascontiguousarray(ds.Q.reshape(-1), dtype=np.float64)
        self.outgroup = np.ascontiguousarray(ds.outgroup, dtype=np.int32)
        self.conserve = np.ascontiguousarray(ds.conserve, dtype=np.int32)
        m = PaccModel()
        m.n_species = t.n_species
        m.children = ptr(self.children, C.c_int32)
        m.distances = ptr(self.distances, C.c_double)
        m.pi = ptr(self.pi, C.c_double)
        m.rate_matrix = ptr(self.Q, C.c_double)
        m.outgroup = ptr(self.outgroup, C.c_int32)
        m.n_outgroup = len(self.outgroup)
        m.conserve = ptr(self.conserve, C.c_int32)
        m.n_conserve = len(self.conserve)
        self.model = m


class BatchArgs:
    """Keeps the numpy buffers behind a PaccElementBatch alive."""

    def __init__(self, ds, element_no=None, start_z=None, start_rates=None):
        E = ds.n_elements
        self.element_no = np.ascontiguousarray(np.arange(E) if element_no is None else element_no, dtype=np.int64)
        self.lengths = np.ascontiguousarray(ds.lengths, dtype=np.int32)
        self.offsets = np.ascontiguousarray(ds.offsets, dtype=np.int64)
        self.bases = np.ascontiguousarray(ds.bases, dtype=np.uint8)
        b = PaccElementBatch()
        b.n_elements = E
        b.element_no = ptr(self.element_no, C.c_int64)
        b.lengths = ptr(self.lengths, C.c_int32)
        b.offsets = ptr(self.offsets, C.c_int64)
        b.bases = ptr(self.bases, C.c_uint8)
        self.start_z = None if start_z is None else np.ascontiguousarray(start_z, dtype=np.int8)
        self.start_rates = None if start_rates is None else np.ascontiguousarray(start_rates, dtype=np.float64)
        if self.start_z is not None:
            b.start_z = ptr(self.start_z, C.c_int8)
        if self.start_rates is not None:
            b.start_rates = ptr(self.start_rates, C.c_double)
        self.batch = b


class Results:
    """Result array with caller-owned max_z / post_z / trace buffers."""

    def __init__(self, n: int, n_nodes: int, trace_iters: int = 0, buffers: bool = True):
        self.n = n
        self.N = n_nodes
        self.T = trace_iters
        self.arr = (PaccResult * max(n, 1))()
        if not buffers:      # scalar fields only (max_z / post_z / traces not copied)
            self.max_z = self.post_z = self.tr = self.tr_z = None
            return
        self.max_z = np.zeros((max(n, 1), 3, n_nodes), dtype=np.int32)
        self.post_z = np.zeros((max(n, 1), 3, n_nodes, 4), dtype=np.float64)
        T = max(trace_iters, 1)
        self.tr = {k: np.zeros((max(n, 1), 3, T), dtype=np.float64)
                   for k in ("loglik", "n_rate", "c_rate", "g_rate", "l_rate", "l2_rate")}
        self.tr_z = np.zeros((max(n, 1), 3, T, n_nodes), dtype=np.int8)
        self.end_z = np.zeros((max(n, 1), n_nodes), dtype=np.int8)
        for i in range(n):
            r = self.arr[i]
            r.max_z = ptr(self.max_z[i], C.c_int32)
            r.post_z = ptr(self.post_z[i], C.c_double)
            r.end_z = ptr(self.end_z[i], C.c_int8)
            if trace_iters > 0:
                for k, a in self.tr.items():
                    setattr(r.trace, k, ptr(a[i], C.c_double))
                r.trace.z = ptr(self.tr_z[i], C.c_int8)

    def status(self):
        return np.array([self.arr[i].status for i in range(self.n)])

    def field(self, name: str) -> np.ndarray:
        """[n, 3] array of a pacc_model_result field."""
        return np.array([[getattr(self.arr[i].model[m], name) for m in range(3)] for i in range(self.n)])

    def element_no(self):
        return np.array([self.arr[i].element_no for i in range(self.n)])
