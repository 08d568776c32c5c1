"""phyloacc-gb300: PhyloAcc-ST's per-element Bayesian MCMC on one NVIDIA GB300.

Python access to the C ABI of include/pacc.h (libpaccgpu.so, built in-tree by
phyloacc_gb300/build.py).  The compute path is the CUDA library; there is no
Python or CPU fallback: every call fails with an exception when the library
or a GPU is missing.

    from phyloacc_gb300 import Context, default_opts
    ctx = Context(dataset, opts)          # pacc_create
    res = ctx.run(dataset)                # pacc_run -> abi.Results
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import abi
from .abi import default_opts  # noqa: F401

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libpaccgpu.so")
CLI_PATH = os.path.join(HERE, "_build", "phyloacc-st-gpu")
CLI_GBGC_PATH = os.path.join(os.path.dirname(CLI_PATH), "phyloacc-gbgc-gpu")
_lib = None


def lib():
    """Load libpaccgpu.so (raises if it has not been built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError("libpaccgpu.so is not built; run phyloacc_gb300.build.build() first")
        L = C.CDLL(LIB_PATH)
        L.pacc_default_opts.argtypes = [C.POINTER(abi.PaccOpts)]
        L.pacc_create.argtypes = [C.POINTER(abi.PaccModel), C.POINTER(abi.PaccOpts), C.POINTER(C.c_int)]
        L.pacc_create.restype = C.c_void_p
        L.pacc_submit.argtypes = [C.c_void_p, C.POINTER(abi.PaccElementBatch)]
        L.pacc_poll.argtypes = [C.c_void_p, C.POINTER(abi.PaccResult), C.c_int]
        L.pacc_sync.argtypes = [C.c_void_p]
        L.pacc_pending.argtypes = [C.c_void_p]
        L.pacc_run.argtypes = [C.c_void_p, C.POINTER(abi.PaccElementBatch), C.POINTER(abi.PaccResult)]
        L.pacc_destroy.argtypes = [C.c_void_p]
        L.pacc_last_error.argtypes = [C.c_void_p]
        L.pacc_last_error.restype = C.c_char_p
        L.pacc_get_counters.argtypes = [C.c_void_p, C.POINTER(abi.PaccCounters)]
        L.pacc_debug_pmatrix.argtypes = [C.c_void_p, C.c_int, C.POINTER(C.c_double), C.POINTER(C.c_double),
                                         C.POINTER(C.c_double)]
        L.pacc_pmatrix_noalloc.argtypes = [C.c_void_p, C.c_int, C.POINTER(C.c_double), C.POINTER(C.c_double),
                                           C.POINTER(C.c_double)]
        L.pacc_debug_loglik.argtypes = [C.c_void_p, C.POINTER(C.c_uint8), C.c_int32, C.POINTER(C.c_int32),
                                        C.c_double, C.c_double, C.POINTER(C.c_double), C.POINTER(C.c_int32)]
        L.pacc_debug_encode.argtypes = [C.c_void_p, C.POINTER(C.c_uint8), C.c_int32, C.POINTER(C.c_int8),
                                        C.POINTER(C.c_int32), C.POINTER(C.c_uint8), C.POINTER(C.c_int32),
                                        C.POINTER(C.c_int32)]
        L.pacc_debug_patterns.argtypes = [C.c_void_p, C.POINTER(C.c_uint8), C.c_int32, C.POINTER(C.c_int32),
                                          C.POINTER(C.c_int32), C.POINTER(C.c_int32), C.POINTER(C.c_int32)]
        L.pacc_debug_stream.argtypes = [C.c_uint32, C.c_uint64, C.c_int, C.POINTER(C.c_uint32)]
        L.pacc_measure_fma_peak.argtypes = [C.c_int, C.POINTER(C.c_double), C.POINTER(C.c_double)]
        L.pacc_get_launch_shape.argtypes = [C.c_void_p, C.POINTER(C.c_int32), C.POINTER(C.c_int32),
                                            C.POINTER(C.c_int32), C.POINTER(C.c_double)]
        L.pacc_gbgc_default_opts.argtypes = [C.POINTER(abi.PaccGbgcOpts)]
        L.pacc_gbgc_run.argtypes = [C.c_void_p, C.POINTER(abi.PaccGbgcOpts), C.POINTER(abi.PaccElementBatch),
                                    C.POINTER(abi.PaccGbgcResult)]
        L.pacc_gbgc_submit.argtypes = [C.c_void_p, C.POINTER(abi.PaccGbgcOpts), C.POINTER(abi.PaccElementBatch)]
        L.pacc_gbgc_poll.argtypes = [C.c_void_p, C.POINTER(abi.PaccGbgcResult), C.c_int]
        L.pacc_gbgc_sync.argtypes = [C.c_void_p]
        L.pacc_gbgc_engine.argtypes = [C.c_void_p, C.POINTER(C.c_uint8), C.c_int32, C.c_int32, C.c_double,
                                       C.POINTER(C.c_int32), C.POINTER(C.c_int32), C.c_double, C.c_double,
                                       C.c_double, C.POINTER(C.c_double), C.POINTER(C.c_double),
                                       C.POINTER(C.c_double), C.POINTER(C.c_int32), C.POINTER(C.c_uint8),
                                       C.POINTER(C.c_int32)]
        _lib = L
    return _lib


class PaccError(RuntimeError):
    pass


class Context:
    """A pacc context for one tree / rate matrix / option set."""

    def __init__(self, ds, opts: abi.PaccOpts):
        self.ds = ds
        self.opts = opts
        self._m = abi.ModelArgs(ds)
        st = C.c_int(0)
        self.h = lib().pacc_create(C.byref(self._m.model), C.byref(opts), C.byref(st))
        if not self.h:
            raise PaccError("pacc_create failed (%d): %s" % (st.value, lib().pacc_last_error(None).decode()))

    def close(self):
        if self.h:
            lib().pacc_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _err(self, what, st):
        raise PaccError("%s failed (%d): %s" % (what, st, lib().pacc_last_error(self.h).decode()))

    def run(self, ds=None, element_no=None, start_z=None, start_rates=None) -> abi.Results:
        """Runs a batch to completion.  start_z [n, N] / start_rates [n, 5]:
        the SAMPLE_HYPER start states (opts.sample_hyper)."""
        ds = self.ds if ds is None else ds
        b = abi.BatchArgs(ds, element_no, start_z, start_rates)
        res = abi.Results(ds.n_elements, ds.tree.n_nodes, self.opts.trace_iters)
        st = lib().pacc_run(self.h, C.byref(b.batch), res.arr)
        if st != 0:
            self._err("pacc_run", st)
        return res

    def submit(self, ds, element_no=None):
        b = abi.BatchArgs(ds, element_no)
        st = lib().pacc_submit(self.h, C.byref(b.batch))
        if st != 0:
            self._err("pacc_submit", st)

    def sync(self):
        st = lib().pacc_sync(self.h)
        if st != 0:
            self._err("pacc_sync", st)

    def poll(self, max_n: int, buffers: bool = True) -> abi.Results:
        """Up to max_n finished results.  In serving mode one call also runs
        one sweep step.  buffers=False leaves out max_z / post_z / traces."""
        res = abi.Results(max_n, self.ds.tree.n_nodes, self.opts.trace_iters if buffers else 0, buffers)
        k = lib().pacc_poll(self.h, res.arr, max_n)
        if k < 0:
            self._err("pacc_poll", -k)
        res.n = k
        return res

    def pending(self) -> int:
        """Elements submitted and not yet returned by poll()."""
        return lib().pacc_pending(self.h)

    def counters(self) -> dict:
        c = abi.PaccCounters()
        lib().pacc_get_counters(self.h, C.byref(c))
        out = {n: getattr(c, n) for n, _ in abi.PaccCounters._fields_ if n != "phase_cycles"}
        out["phase_cycles"] = list(c.phase_cycles)
        return out

    def launch_shape(self) -> dict:
        """Threads per chain, registers a thread and chains per SM of the
        CTA kernel (the tuner's choice), and the tuner's trial time in ms."""
        bt, regs, per_sm, ms = C.c_int32(), C.c_int32(), C.c_int32(), C.c_double()
        st = lib().pacc_get_launch_shape(self.h, C.byref(bt), C.byref(regs), C.byref(per_sm), C.byref(ms))
        if st != 0:
            self._err("pacc_get_launch_shape", st)
        return {"block_threads": bt.value, "registers": regs.value, "chains_per_sm": per_sm.value,
                "tuner_trial_ms": ms.value}

    def pmatrix(self, d, r) -> np.ndarray:
        d = np.ascontiguousarray(d, dtype=np.float64)
        r = np.ascontiguousarray(r, dtype=np.float64)
        out = np.zeros((len(d), 16))
        st = lib().pacc_debug_pmatrix(self.h, len(d), abi.ptr(d, C.c_double), abi.ptr(r, C.c_double),
                                      abi.ptr(out, C.c_double))
        if st != 0:
            self._err("pacc_debug_pmatrix", st)
        return out.reshape(-1, 4, 4)

    def pmatrix_noalloc(self, d, r) -> np.ndarray:
        """pmatrix() through the allocation-free entry point (at most
        PACC_NOALLOC_MAX_PAIRS pairs per call)."""
        d = np.ascontiguousarray(d, dtype=np.float64)
        r = np.ascontiguousarray(r, dtype=np.float64)
        out = np.zeros((len(d), 16))
        st = lib().pacc_pmatrix_noalloc(self.h, len(d), abi.ptr(d, C.c_double), abi.ptr(r, C.c_double),
                                        abi.ptr(out, C.c_double))
        if st != 0:
            self._err("pacc_pmatrix_noalloc", st)
        return out.reshape(-1, 4, 4)

    def loglik(self, e: int, z, c_rate: float, n_rate: float) -> np.ndarray:
        blk = np.ascontiguousarray(self.ds.element(e).reshape(-1))
        L = int(self.ds.lengths[e])
        out = np.zeros(L)
        ncol = C.c_int32()
        z = np.ascontiguousarray(z, dtype=np.int32)
        st = lib().pacc_debug_loglik(self.h, abi.ptr(blk, C.c_uint8), L, abi.ptr(z, C.c_int32), c_rate, n_rate,
                                     abi.ptr(out, C.c_double), C.byref(ncol))
        if st != 0:
            self._err("pacc_debug_loglik", st)
        return out[:ncol.value]

    def gbgc_engine(self, e: int, z, b, sel_c: float, sel_n: float, gc_bias: float, gapchar: str = "*",
                    missing_thres: float = 0.8) -> dict:
        """The gBGC model's likelihood engine on element e at one state (Z and
        the gBGC flag B per node, selection sel_c / sel_n, GC bias): the six
        classes' log transition matrices [6][N][4][4], per-column
        log-likelihoods, expected (child, parent) base counts [N][4][4], the
        element's root and missing flags.  A filtered element returns
        {"filtered": 1, "missing": ...}."""
        N = self.ds.tree.n_nodes
        blk = np.ascontiguousarray(self.ds.element(e).reshape(-1))
        L = int(self.ds.lengths[e])
        z = np.ascontiguousarray(z, dtype=np.int32)
        b = np.ascontiguousarray(b, dtype=np.int32)
        logp = np.zeros(6 * N * 16)
        col = np.zeros(L)
        counts = np.zeros(N * 16)
        root = C.c_int32()
        miss = np.zeros(N, np.uint8)
        filt = C.c_int32()
        st = lib().pacc_gbgc_engine(self.h, abi.ptr(blk, C.c_uint8), L, ord(gapchar), missing_thres,
                                    abi.ptr(z, C.c_int32), abi.ptr(b, C.c_int32), sel_c, sel_n, gc_bias,
                                    abi.ptr(logp, C.c_double), abi.ptr(col, C.c_double), abi.ptr(counts, C.c_double),
                                    C.byref(root), abi.ptr(miss, C.c_uint8), C.byref(filt))
        if st == abi.PACC_FILTERED:
            return {"filtered": 1, "missing": miss}
        if st != 0:
            self._err("pacc_gbgc_engine", st)
        return {"logp": logp.reshape(6, N, 4, 4), "col": col, "counts": counts.reshape(N, 4, 4), "root": root.value,
                "missing": miss, "filtered": 0}

    def gbgc_run(self, gopts, elements=None, trace: bool = False, ds=None) -> list:
        """The gBGC model's three chains for the given elements (default: all)
        on the device; one dict per element with the fields of
        pacc_gbgc_result and arrays by model index 0 = M0, 1 = M1, 2 = M2."""
        ds = ds or self.ds
        idx = list(range(ds.n_elements)) if elements is None else list(elements)
        N = ds.tree.n_nodes
        T = gopts.burnin + gopts.mcmc
        sub = ds.subset(idx) if idx != list(range(ds.n_elements)) else ds
        batch = abi.BatchArgs(sub, np.array(idx, np.int64))
        res = (abi.PaccGbgcResult * len(idx))()
        bufs = []
        for k in range(len(idx)):
            b = {"max_z": np.zeros((3, N), np.int32), "max_b": np.zeros((3, N), np.int8),
                 "post_b": np.zeros((3, N)), "post_z": np.zeros((3, N, 4))}
            res[k].max_z = abi.ptr(b["max_z"], C.c_int32)
            res[k].max_b = abi.ptr(b["max_b"], C.c_int8)
            res[k].post_b = abi.ptr(b["post_b"], C.c_double)
            res[k].post_z = abi.ptr(b["post_z"], C.c_double)
            if trace:
                b["trace"] = np.zeros((3, T, 4 + 2 * N))
                res[k].trace = abi.ptr(b["trace"], C.c_double)
            bufs.append(b)
        st = lib().pacc_gbgc_run(self.h, C.byref(gopts), C.byref(batch.batch), res)
        if st != 0:
            self._err("pacc_gbgc_run", st)
        out = []
        for k in range(len(idx)):
            r = res[k]
            d = dict(bufs[k])
            d.update({"element_no": r.element_no, "status": r.status, "root": r.root,
                      "loglik_null": r.loglik_null, "loglik_res": r.loglik_res, "loglik_all": r.loglik_all,
                      "max_loglik": np.array(r.max_loglik[:]), "device_ms": r.device_ms,
                      "rates": np.array([[r.rates[i][j] for j in range(3)] for i in range(3)])})
            out.append(d)
        return out

    def gbgc_submit(self, gopts, elements=None, ds=None):
        """Queue elements for the gBGC serving kernel (pacc_gbgc_submit)."""
        ds = ds or self.ds
        idx = list(range(ds.n_elements)) if elements is None else list(elements)
        sub = ds.subset(idx)
        batch = abi.BatchArgs(sub, np.array(idx, np.int64))
        st = lib().pacc_gbgc_submit(self.h, C.byref(gopts), C.byref(batch.batch))
        if st != 0:
            self._err("pacc_gbgc_submit", st)

    def gbgc_poll(self, max_results: int = 1 << 16) -> list:
        """Finished gBGC elements so far (completion order), as gbgc_run's dicts."""
        N = self.ds.tree.n_nodes
        res = (abi.PaccGbgcResult * max_results)()
        bufs = []
        for k in range(max_results):
            b = {"max_z": np.zeros((3, N), np.int32), "max_b": np.zeros((3, N), np.int8),
                 "post_b": np.zeros((3, N)), "post_z": np.zeros((3, N, 4))}
            res[k].max_z = abi.ptr(b["max_z"], C.c_int32)
            res[k].max_b = abi.ptr(b["max_b"], C.c_int8)
            res[k].post_b = abi.ptr(b["post_b"], C.c_double)
            res[k].post_z = abi.ptr(b["post_z"], C.c_double)
            bufs.append(b)
        n = lib().pacc_gbgc_poll(self.h, res, max_results)
        if n < 0:
            self._err("pacc_gbgc_poll", n)
        out = []
        for k in range(n):
            r = res[k]
            d = dict(bufs[k])
            d.update({"element_no": r.element_no, "status": r.status, "root": r.root,
                      "loglik_null": r.loglik_null, "loglik_res": r.loglik_res, "loglik_all": r.loglik_all,
                      "max_loglik": np.array(r.max_loglik[:]), "device_ms": r.device_ms,
                      "rates": np.array([[r.rates[i][j] for j in range(3)] for i in range(3)])})
            out.append(d)
        return out

    def gbgc_sync(self):
        st = lib().pacc_gbgc_sync(self.h)
        if st != 0:
            self._err("pacc_gbgc_sync", st)

    def patterns(self, e: int):
        """(pattern_of [n_cols], weights [n_patterns]) of element e (host only)."""
        blk = np.ascontiguousarray(self.ds.element(e).reshape(-1))
        L = int(self.ds.lengths[e])
        po = np.zeros(max(L, 1), dtype=np.int32)
        wt = np.zeros(max(L, 1), dtype=np.int32)
        nc, npat = C.c_int32(), C.c_int32()
        st = lib().pacc_debug_patterns(self.h, abi.ptr(blk, C.c_uint8), L, abi.ptr(po, C.c_int32),
                                       abi.ptr(wt, C.c_int32), C.byref(nc), C.byref(npat))
        if st not in (0, abi.PACC_FILTERED):
            self._err("pacc_debug_patterns", st)
        return po[:nc.value], wt[:npat.value]

    def encode(self, e: int):
        blk = np.ascontiguousarray(self.ds.element(e).reshape(-1))
        L = int(self.ds.lengths[e])
        N = self.ds.tree.n_nodes
        tg = np.zeros(L * N, dtype=np.int8)
        ncol = C.c_int32()
        miss = np.zeros(N, dtype=np.uint8)
        root = C.c_int32()
        filt = C.c_int32()
        st = lib().pacc_debug_encode(self.h, abi.ptr(blk, C.c_uint8), L, abi.ptr(tg, C.c_int8), C.byref(ncol),
                                     abi.ptr(miss, C.c_uint8), C.byref(root), C.byref(filt))
        if st != 0:
            self._err("pacc_debug_encode", st)
        return tg[:ncol.value * N].reshape(ncol.value, N), miss, root.value, filt.value


def stream_words(seed: int, w0: int, n: int) -> np.ndarray:
    out = np.zeros(n, dtype=np.uint32)
    st = lib().pacc_debug_stream(seed, w0, n, abi.ptr(out, C.c_uint32))
    if st != 0:
        raise PaccError("pacc_debug_stream failed (%d)" % st)
    return out


def measure_fma_peak(device: int = 0):
    """Measured FP64 and FP32 FMA throughput of the GPU in FLOP/s."""
    a, b = C.c_double(), C.c_double()
    st = lib().pacc_measure_fma_peak(device, C.byref(a), C.byref(b))
    if st != 0:
        raise PaccError("pacc_measure_fma_peak failed (%d)" % st)
    return a.value, b.value
