"""Bit-exact checks of the host preprocessing of the C ABI (column encoding,
trimming, missing taxa, pruning of the outgroup path, bpp_c.hpp:143-476)
against the oracle.  Runs without a GPU: pacc_create serves the host-only
entry points when no device is present."""
import ctypes as C
import os
import re

import numpy as np
import pytest

import phyloacc_gb300 as pg
from golden_io import CASES, load_case
from oracle import pyoracle as po
from phyloacc_gb300 import abi, synth


def _compare(ds, o, elems):
    ctx = pg.Context(ds, o)
    for e in elems:
        a = ctx.encode(e)
        b = po.encode(ds, o, e)
        assert a[3] == b[3], (e, "filtered")
        if a[3]:
            continue
        assert a[0].shape == b[0].shape
        assert (a[0] == b[0]).all(), e
        assert (a[1] == b[1]).all(), e
        assert a[2] == b[2], e


def _edge_dataset(seed=0):
    ds = synth.make_dataset("st12", n_elements=12, seed=seed)
    ds.bases = ds.bases.copy()
    S = ds.tree.n_species
    rng = np.random.default_rng(seed)
    for e in range(ds.n_elements):
        blk = ds.element(e)
        if e == 0:
            blk[ds.outgroup[0]] = ord("-")                 # outgroup missing -> root moves
        if e == 1:
            blk[:, :] = ord("-")                          # everything missing -> filtered by CONSERVE_PROP
        if e == 2:
            for s in ds.conserve[:3]:
                blk[s] = ord("-")
        if e == 3:
            blk[rng.integers(0, S, 40), rng.integers(0, blk.shape[1], 40)] = np.frombuffer(b"rykmsw" * 7, np.uint8)[:40]
        if e == 4:
            blk[:, ::3] = ord("n")
        if e == 5:
            blk[1:, :10] = ord("-")                        # columns nearly all gaps (trimmed when enabled)
        if e == 6:
            blk[[ds.outgroup[0], 1, 2]] = ord("-")
        if e == 7:
            blk[:, :] = np.frombuffer(b"ACGTX*?.", np.uint8)[rng.integers(0, 8, blk.shape)]  # upper case -> other
    return ds


@pytest.mark.parametrize("kv", [
    {},
    {"prune_tree": 1},
    {"trim_gap_percent": 0.5},
    {"gap_prop": 0.05, "conserve_prop": 0.5},
    {"min_len": 160},
    {"gapchar": ord("n")},
])
def test_encode_matches_oracle(kv):
    ds = _edge_dataset()
    o = abi.default_opts()
    for k, v in kv.items():
        setattr(o, k, v)
    _compare(ds, o, range(ds.n_elements))


@pytest.mark.parametrize("case", CASES)
def test_encode_golden_inputs(case):
    ds, o, _ = load_case(case)
    _compare(ds, o, range(ds.n_elements))


def test_encode_43_taxa():
    ds = synth.make_dataset("st43", n_elements=40, seed=2)
    _compare(ds, abi.default_opts(), range(ds.n_elements))


def test_abi_exports_every_declared_symbol(built):
    hdr = open(pg.LIB_PATH.replace("phyloacc_gb300/_build/libpaccgpu.so", "include/pacc.h")).read()
    names = set(re.findall(r"^(?:const\s+)?[a-z_0-9]+\s*\*?\s*(pacc_[a-z_0-9]+)\(", hdr, re.M))
    assert len(names) >= 15
    L = C.CDLL(pg.LIB_PATH)
    for n in sorted(names):
        assert hasattr(L, n), n


def test_default_opts_match_the_library(built):
    """pacc_default_opts writes the same values into the ctypes mirror of
    pacc_opts as abi.default_opts (the two layouts agree field by field)."""
    L = pg.lib()
    a = abi.PaccOpts()
    C.memset(C.byref(a), 0x5A, C.sizeof(a))
    L.pacc_default_opts(C.byref(a))
    b = abi.default_opts()
    for name, _ in abi.PaccOpts._fields_:
        if name == "reserved0":
            continue
        assert getattr(a, name) == getattr(b, name), name


def test_gbgc_default_opts_match_the_library(built):
    """pacc_gbgc_default_opts writes the values abi.gbgc_default_opts gives
    (the gBGC program's defaults) into the ctypes mirror of pacc_gbgc_opts."""
    L = pg.lib()
    a = abi.PaccGbgcOpts()
    C.memset(C.byref(a), 0x5A, C.sizeof(a))
    L.pacc_gbgc_default_opts(C.byref(a))
    b = abi.gbgc_default_opts()
    for name, _ in abi.PaccGbgcOpts._fields_:
        if name in ("target", "n_target"):
            continue
        assert getattr(a, name) == getattr(b, name), name


def test_run_without_gpu_fails_loudly(built):
    import os
    if os.path.exists("/dev/nvidia0"):
        pytest.skip("a GPU is present")
    ds = synth.make_dataset("st12", n_elements=2, seed=0)
    ctx = pg.Context(ds, abi.default_opts())
    with pytest.raises(pg.PaccError):
        ctx.run()


def _patterns_numpy(blk, gapchar=ord("-")):
    """Site patterns restated: encoded columns, distinct ones numbered in order
    of first occurrence, with their column counts."""
    lut = np.full(256, 5, dtype=np.uint8)
    for i, ch in enumerate(b"acgt"):
        lut[ch] = i
    for i, ch in enumerate(b"rykmsw"):
        lut[ch] = 6 + i
    lut[gapchar] = 4
    codes = lut[np.asarray(blk, dtype=np.uint8)]
    ids, of, weights = {}, [], []
    for col in codes.T:
        key = col.tobytes()
        if key not in ids:
            ids[key] = len(ids)
            weights.append(0)
        of.append(ids[key])
        weights[ids[key]] += 1
    return np.array(of, dtype=np.int32), np.array(weights, dtype=np.int32)


@pytest.mark.parametrize("kind", ["edge", "st43"])
def test_site_patterns_bit_exact(kind):
    ds = _edge_dataset(3) if kind == "edge" else synth.make_dataset("st43", n_elements=20, seed=4)
    if kind == "edge":
        blk = ds.element(8)
        blk[:, 1::2] = blk[:, 0:1]        # many repeated columns
    ctx = pg.Context(ds, abi.default_opts())
    n_checked = 0
    for e in range(ds.n_elements):
        of, wt = ctx.patterns(e)
        if len(of) == 0:
            continue                      # filtered
        ref_of, ref_wt = _patterns_numpy(ds.element(e))
        assert np.array_equal(of, ref_of), e
        assert np.array_equal(wt, ref_wt), e
        assert wt.sum() == len(of)
        n_checked += 1
    assert n_checked >= 5


@pytest.mark.parametrize("extra,message", [
    ({"INDEL": "1"}, "INDEL > 0"),
    ({"SAMPLE_HYPER": "1", "GPU_PRECISION": "fp32_warp"}, "SAMPLE_HYPER chains need"),
    ({"CHAIN": "2", "GPU_PRECISION": "fp64_warp"}, "a later chain"),
])
def test_cli_rejects_unbuilt_modes(tmp_path, extra, message):
    """Modes that are not built fail loudly before any device work, instead of
    running something else."""
    import shutil
    import subprocess
    from phyloacc_gb300.build import build, CLI
    build()
    src = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "st12_default")
    for f in ("case.mod", "case.bed", "case.fa"):
        shutil.copy(os.path.join(src, f), tmp_path / f)
    (tmp_path / "out").mkdir()
    lines = [ln for ln in open(os.path.join(src, "case.cfg")).read().splitlines()
             if ln.split(" ")[0] not in extra]
    (tmp_path / "case.cfg").write_text("\n".join(lines + ["%s %s" % kv for kv in extra.items()]) + "\n")
    r = subprocess.run([CLI, "case.cfg"], cwd=tmp_path, capture_output=True, text=True, timeout=120)
    assert r.returncode != 0
    assert message in r.stderr


def test_cli_chain_zero_writes_headers_only(tmp_path):
    """CHAIN 0 (the reference has no default for CHAIN, main.cpp:57): no chain
    runs, so only _hyper.txt, _species_names.txt and the _rate_postZ headers
    are written, as PhyloAcc-ST does; no device is touched."""
    import shutil
    import subprocess
    from phyloacc_gb300.build import build, CLI
    build()
    src = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "st12_default")
    for f in ("case.mod", "case.bed", "case.fa"):
        shutil.copy(os.path.join(src, f), tmp_path / f)
    (tmp_path / "out").mkdir()
    lines = [ln for ln in open(os.path.join(src, "case.cfg")).read().splitlines() if not ln.startswith("CHAIN ")]
    (tmp_path / "case.cfg").write_text("\n".join(lines + ["CHAIN 0"]) + "\n")
    r = subprocess.run([CLI, "case.cfg"], cwd=tmp_path, capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stderr
    assert sorted(os.listdir(tmp_path / "out")) == ["case_hyper.txt", "case_rate_postZ_M0.txt", "case_rate_postZ_M1.txt",
                                                   "case_rate_postZ_M2.txt", "case_species_names.txt"]
    for m in range(3):
        assert len(open(tmp_path / "out" / ("case_rate_postZ_M%d.txt" % m)).read().splitlines()) == 1


def test_gbgc_cli_chain_zero_and_unbuilt_modes(tmp_path):
    """phyloacc-gbgc-gpu: with CHAIN 0 (no default in the reference) only the
    headers, the hyper header and the species names are written and no device
    is touched; INDEL > 0 and SAMPLE_HYPER fail loudly."""
    import shutil
    import subprocess
    from phyloacc_gb300.build import build, CLI_GBGC
    build()
    src = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "gbgc12_default")
    for f in ("case.mod", "case.bed", "case.fa"):
        shutil.copy(os.path.join(src, f), tmp_path / f)
    (tmp_path / "out").mkdir()
    base = [ln for ln in open(os.path.join(src, "case.cfg")).read().splitlines() if not ln.startswith("CHAIN ")]
    # the GPU keys the reference skips as unknown are taken without a device
    gpu_keys = ["GPU_PRECISION fp32", "GPU_DEVICE 0", "GPU_MEMORY_BUDGET_GB 2.5"]
    (tmp_path / "case.cfg").write_text("\n".join(base + ["CHAIN 0"] + gpu_keys) + "\n")
    r = subprocess.run([CLI_GBGC, "case.cfg"], cwd=tmp_path, capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stderr
    assert sorted(os.listdir(tmp_path / "out")) == ["case_hyper.txt", "case_rate_postZ_0.txt", "case_rate_postZ_1.txt",
                                                    "case_rate_postZ_2.txt", "case_species_names.txt"]
    hdr = open(tmp_path / "out" / "case_rate_postZ_1.txt").read().split("\n")[0]
    want = open(os.path.join(src, "out", "case_rate_postZ_1.txt")).read().split("\n")[0]
    assert hdr == want
    for extra, message in ((["INDEL 1"], "INDEL"), (["SAMPLE_HYPER 1"], "SAMPLE_HYPER")):
        (tmp_path / "case.cfg").write_text("\n".join(base + ["CHAIN 1"] + extra) + "\n")
        r = subprocess.run([CLI_GBGC, "case.cfg"], cwd=tmp_path, capture_output=True, text=True, timeout=120)
        assert r.returncode != 0 and message in r.stderr
