"""The ctypes mirrors in phyloacc_gb300/abi.py have the layout of the C
structs in include/pacc.h: a small program compiled against the header
prints every struct's size and every field's offset, which must equal
ctypes' own.  CPU only (needs g++)."""
import ctypes as C
import os
import shutil
import subprocess

import pytest

from phyloacc_gb300 import abi

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

MIRRORS = {
    "pacc_model": abi.PaccModel,
    "pacc_opts": abi.PaccOpts,
    "pacc_element_batch": abi.PaccElementBatch,
    "pacc_model_result": abi.PaccModelResult,
    "pacc_trace": abi.PaccTrace,
    "pacc_result": abi.PaccResult,
    "pacc_counters": abi.PaccCounters,
    "pacc_gbgc_opts": abi.PaccGbgcOpts,
    "pacc_gbgc_result": abi.PaccGbgcResult,
}


@pytest.mark.skipif(shutil.which("g++") is None, reason="needs g++")
def test_ctypes_mirrors_match_the_header(tmp_path):
    lines = ['#include <cstddef>', '#include <cstdio>', '#include "pacc.h"', "int main() {"]
    for cname, cls in MIRRORS.items():
        lines.append('    std::printf("%s size %%zu\\n", sizeof(%s));' % (cname, cname))
        for field, _ in cls._fields_:
            lines.append('    std::printf("%s %s %%zu\\n", offsetof(%s, %s));' % (cname, field, cname, field))
    lines += ["    return 0;", "}"]
    src = tmp_path / "layout.cpp"
    src.write_text("\n".join(lines) + "\n")
    exe = tmp_path / "layout"
    subprocess.run(["g++", "-std=c++17", "-I" + os.path.join(ROOT, "include"), str(src), "-o", str(exe)],
                   check=True, capture_output=True, text=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.split("\n")
    got = {}
    for ln in out:
        w = ln.split()
        if len(w) == 3:
            got[(w[0], w[1])] = int(w[2])
    for cname, cls in MIRRORS.items():
        assert got[(cname, "size")] == C.sizeof(cls), cname
        for field, _ in cls._fields_:
            assert got[(cname, field)] == getattr(cls, field).offset, (cname, field)
