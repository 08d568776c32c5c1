"""Generate tests/golden/gbgc_engine/engine.npz: what the unmodified gBGC
reference (src/PhyloAcc-ST-GBGC/SRC of a PhyloAcc checkout) computes for
chosen latent states and rates on the gbgc12_default inputs: the six
per-branch log transition matrices, per-column log-likelihoods and expected
(child base, parent base) counts.  The harness (gbgc_engine_harness.cpp) is
compiled with the reference sources (without their main.cpp) against the
stand-in GSL/Armadillo headers of oracle/shim.

    python tests/golden/make_gbgc_engine_golden.py /path/to/PhyloAcc
"""
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
CASE = os.path.join(HERE, "gbgc12_default")
SOURCES = ["bpp.cpp", "bpp_c.cpp", "bpp_c2.cpp", "newick.cpp", "profile.cpp", "utils.cpp"]


def build(ref_root, tmp):
    src = os.path.join(ref_root, "src", "PhyloAcc-ST-GBGC", "SRC")
    shim = os.path.join(ROOT, "oracle", "shim")
    exe = os.path.join(tmp, "harness")
    cmd = ["g++", "-O2", "-std=c++14", "-ffp-contract=off", "-fopenmp", "-w", "-I" + shim, "-I" + src,
           "-I" + os.path.join(ROOT, "oracle"), "-I" + os.path.join(ROOT, "phyloacc_gb300", "csrc"),
           os.path.join(HERE, "gbgc_engine_harness.cpp")] + [os.path.join(src, s) for s in SOURCES] + \
          [os.path.join(shim, "shim_impl.cpp"), "-o", exe]
    subprocess.check_call(cmd)
    return exe


def parse(path):
    recs = []
    cur = None
    for line in open(path):
        t = line.split()
        if not t:
            continue
        if t[0] == "N":
            continue
        if t[0] == "element":
            if t[2] == "filtered":
                continue
            cur = {"element": int(t[1]), "state": int(t[3]), "GG": int(t[5]), "root": int(t[7]),
                   "sc": float(t[9]), "sn": float(t[11]), "gb": float(t[13])}
            recs.append(cur)
        elif t[0] == "nodes":
            cur["nodes"] = np.array([int(x) for x in t[2:]], np.int32)
        else:
            key = t[0]
            vals = np.array([float(x) for x in t[1:]])
            cur[key] = vals
    return recs


def main():
    ref = sys.argv[1]
    cfg = dict(ln.split(None, 1) for ln in open(os.path.join(CASE, "case.cfg")) if ln.strip())
    with tempfile.TemporaryDirectory() as tmp:
        exe = build(ref, tmp)
        out = os.path.join(tmp, "dump.txt")
        subprocess.check_call([exe, os.path.join(CASE, "case.mod"), os.path.join(CASE, "case.fa"),
                               os.path.join(CASE, "case.bed"), cfg["TARGETSPECIES"].strip(), cfg["OUTGROUP"].strip(),
                               cfg["CONSERVE"].strip(), out, "3"], cwd=tmp)
        recs = parse(out)
    arrs = {}
    for i, r in enumerate(recs):
        for k, v in r.items():
            arrs["r%d_%s" % (i, k)] = np.asarray(v)
    arrs["n_records"] = np.array(len(recs))
    np.savez_compressed(os.path.join(HERE, "gbgc_engine", "engine.npz"), **arrs)
    print("records:", len(recs))


if __name__ == "__main__":
    main()
