"""Build the CUDA/C++ library in-tree: phyloacc_gb300/_build/libpaccgpu.so and
the command-line drop-ins phyloacc_gb300/_build/phyloacc-st-gpu (PhyloAcc-ST)
and phyloacc_gb300/_build/phyloacc-gbgc-gpu (PhyloAcc-ST-GBGC).

sm_103a only (GB300); nvcc cross-compiles without a GPU."""
import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
NVCC = os.environ.get("NVCC", "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-I" + os.path.join(ROOT, "include"), "-I" + CSRC]

LIB = os.path.join(OUT, "libpaccgpu.so")
CLI = os.path.join(OUT, "phyloacc-st-gpu")
CLI_GBGC = os.path.join(OUT, "phyloacc-gbgc-gpu")


def _deps():
    return [os.path.join(CSRC, f) for f in os.listdir(CSRC)] + [os.path.join(ROOT, "include", "pacc.h")]


def _stale(out):
    if not os.path.exists(out):
        return True
    t = os.path.getmtime(out)
    return any(os.path.getmtime(d) > t for d in _deps())


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed: " + " ".join(cmd) + "\n" + r.stdout + r.stderr)
    return r.stdout + r.stderr


def build(force=False, verbose=False):
    os.makedirs(OUT, exist_ok=True)
    if not force and not _stale(LIB) and not _stale(CLI) and not _stale(CLI_GBGC):
        return LIB
    objs = {
        "pacc_chain.o": [NVCC] + ARCH + COMMON + ["-Xptxas", "-v", "-c", os.path.join(CSRC, "pacc_chain.cu")],
        "pacc_batch.o": [NVCC] + ARCH + COMMON + ["-Xptxas", "-v", "-c", os.path.join(CSRC, "pacc_batch.cu")],
        "pacc_host.o": [NVCC] + ARCH + COMMON + ["-x", "cu", "-c", os.path.join(CSRC, "pacc_host.cpp")],
        "pacc_noalloc.o": [NVCC] + ARCH + COMMON + ["-c", os.path.join(CSRC, "pacc_noalloc.cu")],
        "pacc_gbgc.o": [NVCC] + ARCH + COMMON + ["-Xptxas", "-v", "-c", os.path.join(CSRC, "pacc_gbgc.cu")],
        "pacc_gbgc_chain.o": [NVCC] + ARCH + COMMON + ["-Xptxas", "-v", "-c", os.path.join(CSRC, "pacc_gbgc_chain.cu")],
    }
    cmds = []
    for name, cmd in objs.items():
        cmds.append(cmd + ["-o", os.path.join(OUT, name)])
    with ThreadPoolExecutor(len(cmds)) as ex:
        logs = list(ex.map(_run, cmds))
    if verbose:
        for lg in logs:
            print(lg)
    tmp = LIB + ".tmp"
    _run([NVCC] + ARCH + ["-shared", "-o", tmp] + [os.path.join(OUT, n) for n in objs])
    os.replace(tmp, LIB)
    for src, exe in (("phyloacc_st_gpu.cpp", CLI), ("phyloacc_gbgc_gpu.cpp", CLI_GBGC)):
        tmp = exe + ".tmp"
        # -ffp-contract=off: the host's hyper-parameter MH rounds like the oracle's
        _run(["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-I" + os.path.join(ROOT, "include"), "-I" + CSRC,
              os.path.join(CSRC, src), "-o", tmp, "-L" + OUT, "-lpaccgpu", "-Wl,-rpath,$ORIGIN", "-pthread"])
        os.replace(tmp, exe)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
