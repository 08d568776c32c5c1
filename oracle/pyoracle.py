"""TEST INFRASTRUCTURE: ctypes access to oracle/_build/liboracle.so.

Only tests/, __graft_entry__.smoke() and bench.py's CPU baseline call this."""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from phyloacc_gb300 import abi

HERE = os.path.dirname(os.path.abspath(__file__))
_lib = None


def lib():
    global _lib
    if _lib is None:
        path = os.path.join(HERE, "_build", "liboracle.so")
        if not os.path.exists(path):
            from oracle.build_oracle import build_oracle
            build_oracle()
        L = C.CDLL(path)
        L.oracle_run.argtypes = [C.POINTER(abi.PaccModel), C.POINTER(abi.PaccOpts),
                                 C.POINTER(abi.PaccElementBatch), C.POINTER(abi.PaccResult), C.c_int]
        L.oracle_run.restype = C.c_int
        L.oracle_run_chain.argtypes = [C.POINTER(abi.PaccModel), C.POINTER(abi.PaccOpts),
                                       C.POINTER(abi.PaccElementBatch), C.POINTER(abi.PaccResult), C.c_int,
                                       C.c_int]
        L.oracle_run_chain.restype = C.c_int
        L.oracle_run_hyper.argtypes = [C.POINTER(abi.PaccModel), C.POINTER(abi.PaccOpts),
                                       C.POINTER(abi.PaccElementBatch), C.c_int, C.POINTER(abi.PaccResult),
                                       C.POINTER(C.c_double), C.c_int]
        L.oracle_run_hyper.restype = C.c_int
        L.oracle_encode.argtypes = [C.POINTER(abi.PaccModel), C.POINTER(abi.PaccOpts), C.POINTER(C.c_uint8),
                                    C.c_int32, C.POINTER(C.c_int8), C.POINTER(C.c_int32), C.POINTER(C.c_uint8),
                                    C.POINTER(C.c_int32), C.POINTER(C.c_int32)]
        L.oracle_encode.restype = C.c_int
        L.oracle_loglik.argtypes = [C.POINTER(abi.PaccModel), C.POINTER(abi.PaccOpts), C.POINTER(C.c_uint8),
                                    C.c_int32, C.POINTER(C.c_int32), C.c_double, C.c_double,
                                    C.POINTER(C.c_double), C.POINTER(C.c_int32)]
        L.oracle_loglik.restype = C.c_int
        L.oracle_pmatrix.argtypes = [C.POINTER(abi.PaccModel), C.POINTER(abi.PaccOpts), C.c_int,
                                     C.POINTER(C.c_double), C.POINTER(C.c_double), C.POINTER(C.c_double)]
        L.oracle_pmatrix.restype = C.c_int
        L.oracle_stream.argtypes = [C.c_uint32, C.c_uint64, C.c_int, C.POINTER(C.c_uint32)]
        L.oracle_philox.argtypes = [C.POINTER(C.c_uint32), C.POINTER(C.c_uint32), C.POINTER(C.c_uint32)]
        L.oracle_sample_gamma.argtypes = [C.c_uint32, C.c_double, C.c_double, C.c_int, C.POINTER(C.c_double)]
        L.oracle_sample_beta.argtypes = [C.c_uint32, C.c_double, C.c_double, C.c_int, C.POINTER(C.c_double)]
        L.oracle_sample_categorical.argtypes = [C.c_uint32, C.c_int, C.POINTER(C.c_double), C.c_int,
                                                C.POINTER(C.c_int32)]
        L.oracle_eigen.argtypes = [C.POINTER(C.c_double)] * 4
        L.oracle_eigen.restype = C.c_int
        _lib = L
    return _lib


def run(ds, opts: abi.PaccOpts, threads: int = 0, element_no=None, chain: int = 0) -> abi.Results:
    """Every element through M0, M1, M2 on the CPU.  chain > 0: a later chain
    of a CHAIN > 1 run (it starts from Z = 0 on every node)."""
    m = abi.ModelArgs(ds)
    b = abi.BatchArgs(ds, element_no)
    res = abi.Results(ds.n_elements, ds.tree.n_nodes, opts.trace_iters)
    if chain == 0:
        st = lib().oracle_run(C.byref(m.model), C.byref(opts), C.byref(b.batch), res.arr, threads)
    else:
        st = lib().oracle_run_chain(C.byref(m.model), C.byref(opts), C.byref(b.batch), res.arr, threads, chain)
    if st != abi.PACC_OK:
        raise RuntimeError("oracle_run failed: %d" % st)
    return res


def run_hyper(ds, opts: abi.PaccOpts, n_chains: int, threads: int = 0, element_no=None):
    """SAMPLE_HYPER: n_chains chains of M2 over the batch with the
    hyper-parameters drawn between chains.  Returns (results, hyper): results
    holds n_chains * n entries, chain k at [k * n, (k + 1) * n) (model 2
    filled); hyper is [n_chains + 1, 10] (nprior_a, nprior_b, cprior_a,
    cprior_b, prior_l_a, prior_l_b, prior_g_a, prior_g_b, prior_l2_a,
    prior_l2_b), row 0 the starting values."""
    m = abi.ModelArgs(ds)
    b = abi.BatchArgs(ds, element_no)
    res = abi.Results(n_chains * ds.n_elements, ds.tree.n_nodes, opts.trace_iters)
    hyper = np.zeros((n_chains + 1, 10))
    st = lib().oracle_run_hyper(C.byref(m.model), C.byref(opts), C.byref(b.batch), n_chains, res.arr,
                                abi.ptr(hyper, C.c_double), threads)
    if st != abi.PACC_OK:
        raise RuntimeError("oracle_run_hyper failed: %d" % st)
    return res, hyper


def encode(ds, opts, e: int):
    m = abi.ModelArgs(ds)
    blk = np.ascontiguousarray(ds.element(e).reshape(-1))
    L = int(ds.lengths[e])
    N = ds.tree.n_nodes
    tg = np.zeros(L * N, dtype=np.int8)
    ncol = C.c_int32()
    miss = np.zeros(N, dtype=np.uint8)
    root = C.c_int32()
    filt = C.c_int32()
    st = lib().oracle_encode(C.byref(m.model), C.byref(opts), abi.ptr(blk, C.c_uint8), L, abi.ptr(tg, C.c_int8),
                             C.byref(ncol), abi.ptr(miss, C.c_uint8), C.byref(root), C.byref(filt))
    assert st == 0
    return tg[:ncol.value * N].reshape(ncol.value, N), miss, root.value, filt.value


def loglik(ds, opts, e: int, z, c_rate: float, n_rate: float) -> np.ndarray:
    m = abi.ModelArgs(ds)
    blk = np.ascontiguousarray(ds.element(e).reshape(-1))
    L = int(ds.lengths[e])
    out = np.zeros(L, dtype=np.float64)
    ncol = C.c_int32()
    z = np.ascontiguousarray(z, dtype=np.int32)
    st = lib().oracle_loglik(C.byref(m.model), C.byref(opts), abi.ptr(blk, C.c_uint8), L, abi.ptr(z, C.c_int32),
                             c_rate, n_rate, abi.ptr(out, C.c_double), C.byref(ncol))
    assert st == 0, st
    return out[:ncol.value]


def pmatrix(ds, opts, d, r) -> np.ndarray:
    m = abi.ModelArgs(ds)
    d = np.ascontiguousarray(d, dtype=np.float64)
    r = np.ascontiguousarray(r, dtype=np.float64)
    out = np.zeros((len(d), 16))
    st = lib().oracle_pmatrix(C.byref(m.model), C.byref(opts), len(d), abi.ptr(d, C.c_double),
                              abi.ptr(r, C.c_double), abi.ptr(out, C.c_double))
    assert st == 0
    return out.reshape(-1, 4, 4)


def stream(seed: int, w0: int, n: int) -> np.ndarray:
    out = np.zeros(n, dtype=np.uint32)
    lib().oracle_stream(seed, w0, n, abi.ptr(out, C.c_uint32))
    return out


def philox(ctr, key) -> np.ndarray:
    c = np.ascontiguousarray(ctr, dtype=np.uint32)
    k = np.ascontiguousarray(key, dtype=np.uint32)
    out = np.zeros(4, dtype=np.uint32)
    lib().oracle_philox(abi.ptr(c, C.c_uint32), abi.ptr(k, C.c_uint32), abi.ptr(out, C.c_uint32))
    return out


def sample_gamma(seed, a, b, n):
    out = np.zeros(n)
    lib().oracle_sample_gamma(seed, a, b, n, abi.ptr(out, C.c_double))
    return out


def sample_beta(seed, a, b, n):
    out = np.zeros(n)
    lib().oracle_sample_beta(seed, a, b, n, abi.ptr(out, C.c_double))
    return out


def sample_categorical(seed, p, n):
    p = np.ascontiguousarray(p, dtype=np.float64)
    out = np.zeros(n, dtype=np.int32)
    lib().oracle_sample_categorical(seed, len(p), abi.ptr(p, C.c_double), n, abi.ptr(out, C.c_int32))
    return out


def eigen(Q):
    Q = np.ascontiguousarray(Q, dtype=np.float64).reshape(-1)
    lam = np.zeros(4)
    V = np.zeros(16)
    Vi = np.zeros(16)
    st = lib().oracle_eigen(*(abi.ptr(a, C.c_double) for a in (Q, lam, V, Vi)))
    return st, lam, V.reshape(4, 4), Vi.reshape(4, 4)


def gbgc_engine(ds, e, z, b, sc, sn, gb, gapchar="*", missing_thres=0.8, conserve_prop=0.8):
    """The gBGC model's likelihood engine on element e at one state (Z and B
    per node, conserved/accelerated selection sc/sn, GC bias gb): the six
    per-branch log transition matrices [6][N][4][4], per-column
    log-likelihoods, expected (child, parent) base counts [N][4][4], the
    element's root and missing flags (oracle_gbgc.cpp)."""
    L = lib()
    if not hasattr(L, "_gbgc_set"):
        L.oracle_gbgc_engine.argtypes = [C.POINTER(abi.PaccModel), C.POINTER(C.c_uint8), C.c_int32, C.c_int32,
                                         C.c_double, C.c_double, C.POINTER(C.c_int32), C.POINTER(C.c_int32),
                                         C.c_double, C.c_double, C.c_double, C.POINTER(C.c_double),
                                         C.POINTER(C.c_double), C.POINTER(C.c_double), C.POINTER(C.c_int32),
                                         C.POINTER(C.c_uint8), C.POINTER(C.c_int32)]
        L.oracle_gbgc_engine.restype = C.c_int
        L._gbgc_set = True
    m = abi.ModelArgs(ds)
    N = ds.tree.n_nodes
    GG = int(ds.lengths[e])
    blk = np.ascontiguousarray(ds.element(e).reshape(-1))
    z = np.ascontiguousarray(z, dtype=np.int32)
    b = np.ascontiguousarray(b, dtype=np.int32)
    logp = np.zeros(6 * N * 16)
    col = np.zeros(GG)
    counts = np.zeros(N * 16)
    root = C.c_int32()
    miss = np.zeros(N, np.uint8)
    filt = C.c_int32()
    st = L.oracle_gbgc_engine(C.byref(m.model), abi.ptr(blk, C.c_uint8), GG, ord(gapchar), missing_thres,
                              conserve_prop, abi.ptr(z, C.c_int32), abi.ptr(b, C.c_int32), sc, sn, gb,
                              abi.ptr(logp, C.c_double), abi.ptr(col, C.c_double), abi.ptr(counts, C.c_double),
                              C.byref(root), abi.ptr(miss, C.c_uint8), C.byref(filt))
    if st not in (abi.PACC_OK, abi.PACC_FILTERED):
        raise RuntimeError("oracle_gbgc_engine failed: %d" % st)
    return {"logp": logp.reshape(6, N, 4, 4), "col": col, "counts": counts.reshape(N, 4, 4), "root": root.value,
            "missing": miss, "filtered": filt.value}


def gbgc_run(ds, o: abi.PaccGbgcOpts, e: int, trace: bool = True) -> dict:
    """One element through the gBGC model's three chains on the CPU
    (oracle_gbgc.cpp, oracle_gbgc_run_element).  Arrays by model index
    0 = M0, 1 = M1, 2 = M2; trace rows: full loglik, n, c, gBC, B[N], Z[N]."""
    L = lib()
    if not hasattr(L, "_gbgc_run_set"):
        L.oracle_gbgc_run_element.argtypes = [C.POINTER(abi.PaccModel), C.POINTER(abi.PaccGbgcOpts),
                                              C.POINTER(C.c_uint8), C.c_int32, C.POINTER(abi.PaccGbgcResult)]
        L.oracle_gbgc_run_element.restype = C.c_int
        L._gbgc_run_set = True
    m = abi.ModelArgs(ds)
    N = ds.tree.n_nodes
    GG = int(ds.lengths[e])
    T = o.burnin + o.mcmc
    blk = np.ascontiguousarray(ds.element(e).reshape(-1))
    r = abi.PaccGbgcResult()
    out = {"max_z": np.zeros((3, N), np.int32), "max_b": np.zeros((3, N), np.int8),
           "post_b": np.zeros((3, N)), "post_z": np.zeros((3, N, 4))}
    r.max_z = abi.ptr(out["max_z"], C.c_int32)
    r.max_b = abi.ptr(out["max_b"], C.c_int8)
    r.post_b = abi.ptr(out["post_b"], C.c_double)
    r.post_z = abi.ptr(out["post_z"], C.c_double)
    if trace:
        out["trace"] = np.zeros((3, T, 4 + 2 * N))
        r.trace = abi.ptr(out["trace"], C.c_double)
    st = L.oracle_gbgc_run_element(C.byref(m.model), C.byref(o), abi.ptr(blk, C.c_uint8), GG, C.byref(r))
    if st not in (abi.PACC_OK, abi.PACC_FILTERED):
        raise RuntimeError("oracle_gbgc_run_element failed: %d" % st)
    out.update({"status": r.status, "root": r.root, "loglik_null": r.loglik_null, "loglik_res": r.loglik_res,
                "loglik_all": r.loglik_all, "max_loglik": np.array(r.max_loglik[:]),
                "rates": np.array([[r.rates[i][j] for j in range(3)] for i in range(3)])})
    return out


def gbgc_run_batch(ds, o: abi.PaccGbgcOpts, threads: int = 0) -> list:
    """Every element of ds through the gBGC chains on the CPU, OpenMP over
    elements (oracle_gbgc_run); summary fields only."""
    import os as _os
    L = lib()
    if not hasattr(L, "_gbgc_batch_set"):
        L.oracle_gbgc_run.argtypes = [C.POINTER(abi.PaccModel), C.POINTER(abi.PaccGbgcOpts),
                                      C.POINTER(abi.PaccElementBatch), C.POINTER(abi.PaccGbgcResult), C.c_int]
        L.oracle_gbgc_run.restype = C.c_int
        L._gbgc_batch_set = True
    m = abi.ModelArgs(ds)
    b = abi.BatchArgs(ds)
    res = (abi.PaccGbgcResult * ds.n_elements)()
    st = L.oracle_gbgc_run(C.byref(m.model), C.byref(o), C.byref(b.batch), res, threads or (_os.cpu_count() or 1))
    if st != abi.PACC_OK:
        raise RuntimeError("oracle_gbgc_run failed: %d" % st)
    return [{"status": r.status, "loglik_null": r.loglik_null, "loglik_res": r.loglik_res,
             "loglik_all": r.loglik_all} for r in res]
