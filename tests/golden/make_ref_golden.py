"""Generate the golden fixtures under tests/golden/<case>/.

Each case holds the PhyloAcc-ST inputs (.mod, FASTA, bed, cfg) and the output
tables the unmodified reference wrote for them: the PhyloAcc-ST sources from
the reference checkout compiled against the stand-in GSL/Armadillo headers of
oracle/shim (recipe: oracle/build_oracle.py), run with VERBOSE 1 so that it
also writes its per-iteration traces (_mcmc_trace_M*_*.txt), which are packed
into traces.npz.

    python tests/golden/make_ref_golden.py /path/to/PhyloAcc [case ...]

(all cases, or only the named ones).  Needs the reference checkout; the
fixtures it writes are committed, so the tests that use them run anywhere.
With CHAIN > 1 the reference appends every chain's rows to the same trace
file; they are stored per chain (key M{m}_{e} for the first chain,
M{m}_{e}_c{k} for chain k).
"""
import glob
import os
import shutil
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from phyloacc_gb300 import synth  # noqa: E402
from oracle.build_oracle import build_reference, build_reference_gbgc  # noqa: E402

CASES = {
    # name: (dataset kind, element indices, burnin, mcmc, seed, extra cfg keys)
    "st12_default": ("st12", [0, 1, 2, 3, 85, 90, 91, 99], 100, 300, 0, {}),
    "st12_options": ("st12", [4, 5, 86, 92], 60, 200, 3,
                     {"PRUNE_TREE": 1, "TRIM_GAP_PERCENT": 0.4, "GAP_PROP": 0.3, "ROPT": 2,
                      "HYPER_LRATE2_A": 0, "ADAPT_FREQ": 25, "INIT_CONSERVE_RATE": 0.3}),
    "st43_default": ("st43", [0, 7, 12], 50, 150, 1, {}),
    # non-default priors, hyper-priors, initial values and rate bounds, and a MIN_LEN filter
    "st12_priors": ("st12", [6, 7, 8, 87, 93], 60, 200, 9,
                    {"CONSERVE_PRIOR_A": 4, "CONSERVE_PRIOR_B": 0.08, "ACCE_PRIOR_A": 8, "ACCE_PRIOR_B": 0.3,
                     "HYPER_LRATE_A": 2, "HYPER_LRATE_B": 8, "HYPER_GRATE_A": 2, "HYPER_GRATE_B": 2,
                     "HYPER_LRATE2_A": 2, "HYPER_LRATE2_B": 6, "INIT_LRATE": 0.2, "INIT_GRATE": 0.6,
                     "INIT_LRATE2": 0.2, "INIT_ACCE_RATE": 2.5, "CONSTOMIS": 0.05, "ROPT": 1, "NLB": 0.8,
                     "CUB": 0.9, "MIN_LEN": 150}),
    # missing-species filters: an element whose missing conserved taxa exceed CONSERVE_PROP is
    # filtered; a target taxon 90% gaps is missing
    "st12_filters": ("st12", [9, 10, 11, 88], 60, 150, 11, {"CONSERVE_PROP": 0.2}),
    # two chains: the second starts every element from Z = 0 (main.cpp:445, bpp_c.cpp:150)
    "st12_chain2": ("st12", [0, 85, 90], 60, 150, 2, {"CHAIN": 2}),
    # SAMPLE_HYPER: three chains of M2, hyper-parameters drawn between chains
    "st12_hyper": ("st12", [0, 1, 85, 90], 60, 150, 4, {"CHAIN": 3, "SAMPLE_HYPER": 1}),
    # the gBGC model (src/PhyloAcc-ST-GBGC): same inputs, its own outputs and traces
    "gbgc12_default": ("st12", [0, 1, 85, 90], 20, 60, 0, {}),
    # 43 taxa with missing taxa ('*' rows): the outgroup (root moves), conserved and target leaves
    "gbgc43_missing": ("st43", [0, 7, 12, 20], 30, 90, 5, {}),
    # two chains: a later chain starts every node from Z = 0 (bpp_c.cpp:124-135), which shows on
    # the nodes off the element's tree (a missing outgroup moves the root in element 1)
    "gbgc43_chain2": ("st43", [0, 7], 20, 40, 6, {"CHAIN": 2}),
    # non-default selection coefficients, priors, transition and missing-data options
    "gbgc12_options": ("st12", [2, 3, 86, 91], 20, 60, 8,
                       {"CONSERVE_RATE": -1.5, "ACCE_RATE": 0.5, "CONSERVE_PRIOR_A": 4, "CONSERVE_PRIOR_B": 0.5,
                        "ACCE_PRIOR_A": 6, "ACCE_PRIOR_B": 0.3, "PREP_LRATE": 0.3, "PREP_GRATE": 0.2,
                        "CONSTOMIS": 0.05, "GAP_PROP": 0.5, "CONSERVE_PROP": 0.6}),
    # '-' as the gap character: the 43-taxon data's gap cells and missing taxa count as gaps
    "gbgc43_dash": ("st43", [3, 9, 15], 20, 40, 10, {"GAPCHAR": "-"}),
}
GBGC_CASES = {"gbgc12_default", "gbgc43_missing", "gbgc43_chain2", "gbgc12_options", "gbgc43_dash"}


def mask_taxa(ds, case):
    """Blank some taxa in some elements to exercise missing-taxon handling,
    outgroup collapse and the conserved-species filter."""
    S = ds.tree.n_species
    if case == "st12_options":
        blk = ds.element(1)
        blk[ds.outgroup[0], :] = ord("-")          # outgroup missing -> root moves
        blk = ds.element(2)
        for s in ds.conserve[:2]:
            blk[s, :] = ord("n")
        blk = ds.element(3)
        blk[ds.target[0], : blk.shape[1] // 2] = ord("-")
    if case == "st12_filters":
        blk = ds.element(1)
        for s in ds.conserve[:3]:
            blk[s, :] = ord("-")
        blk = ds.element(2)
        blk[ds.target[0], : (9 * blk.shape[1]) // 10] = ord("-")
    if case == "gbgc43_chain2":
        ds.element(1)[ds.outgroup[0], :] = ord("*")
    if case == "gbgc12_options":
        blk = ds.element(1)
        blk[ds.conserve[0], : (3 * blk.shape[1]) // 5] = ord("*")   # over GAP_PROP 0.5: missing
        ds.element(2)[ds.outgroup[0], :] = ord("*")
    if case == "gbgc43_missing":
        star = ord("*")
        ds.element(1)[ds.outgroup[0], :] = star
        blk = ds.element(2)
        for s in ds.conserve[:3]:
            blk[s, :] = star
        blk = ds.element(3)
        blk[ds.target[0], :] = star
        blk[ds.target[1], : blk.shape[1] // 3] = star      # under the threshold: not missing
    if case == "st43_default":
        blk = ds.element(1)
        blk[0, :] = ord("-")
        blk[S - 1, :] = ord("-")
        blk = ds.element(2)
        blk[:, :5] = ord("r")                     # ambiguity codes in a few columns
        blk[3, 5:9] = ord("y")
    return ds


def read_trace(path):
    rows = [ln.rstrip("\n\t").split("\t") for ln in open(path)][1:]
    a = np.array([[float(x) for x in r] for r in rows])
    return a


def main(ref_root, only=None):
    exe_st = build_reference(ref_root)
    exe_gbgc = build_reference_gbgc(ref_root)
    if exe_st is None or exe_gbgc is None:
        raise SystemExit("reference sources not found under " + ref_root)
    for name, (kind, idx, burn, mcmc, seed, extra) in CASES.items():
        if only and name not in only:
            continue
        exe = exe_gbgc if name in GBGC_CASES else exe_st
        d = os.path.join(HERE, name)
        if os.path.isdir(d):
            shutil.rmtree(d)
        os.makedirs(d)
        ds = synth.make_dataset(kind, seed=0).subset(idx)
        ds.bases = ds.bases.copy()
        ds = mask_taxa(ds, name)
        kv = {"VERBOSE": 1}
        kv.update(extra)
        cfg = synth.write_inputs(ds, d, prefix="case", burnin=burn, mcmc=mcmc, seed=seed, extra=kv,
                                 species_order=list(range(ds.tree.n_species))[::-1])
        # make the cfg relative to the fixture directory
        lines = open(cfg).read().replace(d + "/", "").replace(d, ".")
        open(cfg, "w").write(lines)
        r = subprocess.run([exe, "case.cfg"], cwd=d, capture_output=True, text=True)
        if r.returncode != 0:
            raise SystemExit(r.stdout[-2000:] + r.stderr[-2000:])
        out = os.path.join(d, "out")
        traces = {}
        T = burn + mcmc
        for f in sorted(glob.glob(os.path.join(out, "case_mcmc_trace_*_*.txt"))):
            tag = os.path.basename(f)[len("case_mcmc_trace_"):-4]  # M{m}_{elem} (gBGC: {m}_{elem})
            rows = read_trace(f)
            for k in range(int(extra.get("CHAIN", 1))):
                # the first 200 iterations of each chain are the chain-parity window
                traces[tag + ("_c%d" % k if k else "")] = rows[k * T:k * T + min(T, 200)]
            os.remove(f)
        np.savez_compressed(os.path.join(d, "traces.npz"), **traces)
        if not extra.get("SAMPLE_HYPER"):
            os.remove(os.path.join(out, "case_hyper.txt"))   # only the starting values
        print(name, "ok", sorted(os.listdir(out)))


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else "/root/reference", sys.argv[2:])
