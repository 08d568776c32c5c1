"""TEST INFRASTRUCTURE: build recipe for the oracle (oracle/_build/liboracle.so)
and, where the PhyloAcc sources are present, the reference itself compiled
against the stand-in GSL/Armadillo headers of oracle/shim (oracle/_ref/).

    python oracle/build_oracle.py            # oracle only
    python oracle/build_oracle.py --ref DIR  # also build DIR/src/PhyloAcc-ST and PhyloAcc-ST-GBGC

__graft_entry__.build() builds the reference too when it finds a checkout:
the directory named by the PHYLOACC_REFERENCE environment variable, else a
"reference" directory beside the repository.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CXX = os.environ.get("CXX", "g++")
# -ffp-contract=off: no FMA contraction, so x86 and Arm builds round alike.
FLAGS = ["-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-fopenmp"]


def _newer(out, srcs):
    if not os.path.exists(out):
        return False
    t = os.path.getmtime(out)
    return all(os.path.getmtime(s) <= t for s in srcs)


def build_oracle(force=False):
    out_dir = os.path.join(HERE, "_build")
    os.makedirs(out_dir, exist_ok=True)
    out = os.path.join(out_dir, "liboracle.so")
    srcs = [os.path.join(HERE, "oracle_st.cpp"), os.path.join(HERE, "oracle_gbgc.cpp"),
            os.path.join(HERE, "oracle_rng.h"),
            os.path.join(ROOT, "include", "pacc.h"), os.path.join(ROOT, "phyloacc_gb300", "csrc", "eigen4.h")]
    if not force and _newer(out, srcs):
        return out
    cmd = [CXX] + FLAGS + ["-shared", "-I" + os.path.join(ROOT, "include"), srcs[0], srcs[1], "-o", out + ".tmp"]
    subprocess.check_call(cmd)
    os.replace(out + ".tmp", out)
    return out


REF_SOURCES = ["bpp.cpp", "bpp_c.cpp", "bpp_c2.cpp", "newick.cpp", "profile.cpp", "utils.cpp", "main.cpp"]


def build_reference(ref_root, force=False):
    """Compile the unmodified PhyloAcc-ST sources with the stand-in headers.
    Output: oracle/_ref/PhyloAcc-ST (binary, git-ignored)."""
    src_dir = os.path.join(ref_root, "src", "PhyloAcc-ST")
    if not os.path.isdir(src_dir):
        return None
    out_dir = os.path.join(HERE, "_ref")
    os.makedirs(out_dir, exist_ok=True)
    out = os.path.join(out_dir, "PhyloAcc-ST")
    shim = os.path.join(HERE, "shim")
    srcs = [os.path.join(src_dir, s) for s in REF_SOURCES]
    shim_files = [os.path.join(dp, f) for dp, _, fs in os.walk(shim) for f in fs]
    if not force and _newer(out, srcs + shim_files + [os.path.join(HERE, "oracle_rng.h")]):
        return out
    cmd = [CXX, "-O2", "-std=c++14", "-ffp-contract=off", "-fopenmp", "-w",
           "-I" + shim, "-I" + HERE, "-I" + os.path.join(ROOT, "phyloacc_gb300", "csrc")] + srcs + \
          [os.path.join(shim, "shim_impl.cpp"), "-o", out + ".tmp"]
    subprocess.check_call(cmd)
    os.replace(out + ".tmp", out)
    return out


def build_reference_gbgc(ref_root, force=False):
    """The unmodified PhyloAcc-ST-GBGC sources (the gBGC model) with the same
    stand-in headers.  Output: oracle/_ref/PhyloAcc-gBGC (git-ignored).  The
    prebuilt binary shipped beside those sources is not used."""
    src_dir = os.path.join(ref_root, "src", "PhyloAcc-ST-GBGC", "SRC")
    if not os.path.isdir(src_dir):
        return None
    out_dir = os.path.join(HERE, "_ref")
    os.makedirs(out_dir, exist_ok=True)
    out = os.path.join(out_dir, "PhyloAcc-gBGC")
    shim = os.path.join(HERE, "shim")
    srcs = [os.path.join(src_dir, s) for s in REF_SOURCES]
    shim_files = [os.path.join(dp, f) for dp, _, fs in os.walk(shim) for f in fs]
    if not force and _newer(out, srcs + shim_files + [os.path.join(HERE, "oracle_rng.h")]):
        return out
    cmd = [CXX, "-O2", "-std=c++14", "-ffp-contract=off", "-fopenmp", "-w",
           "-I" + shim, "-I" + HERE, "-I" + os.path.join(ROOT, "phyloacc_gb300", "csrc")] + srcs + \
          [os.path.join(shim, "shim_impl.cpp"), "-o", out + ".tmp"]
    subprocess.check_call(cmd)
    os.replace(out + ".tmp", out)
    return out


if __name__ == "__main__":
    print(build_oracle(force="--force" in sys.argv))
    if "--ref" in sys.argv:
        ref = sys.argv[sys.argv.index("--ref") + 1]
        print(build_reference(ref, force="--force" in sys.argv))
        print(build_reference_gbgc(ref, force="--force" in sys.argv))
