"""The C++ binding (include/seqan_gb300_seqan.h) compiles and links against SeqAn 2.

The program tests/cpp/seqan_binding.cpp calls every overload with the reference's own types;
building it proves the overloads resolve against the reference's headers (no ambiguity with
its Serial/Parallel overloads) and that every engine symbol they use is exported.  The
reference tree is needed (skipped where it is absent); running the program needs a GPU."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REFERENCE = "/root/reference"


@pytest.mark.skipif(not os.path.isdir(os.path.join(REFERENCE, "include", "seqan")),
                    reason="the reference's headers are not present")
@pytest.mark.skipif(shutil.which("g++") is None, reason="no C++ compiler")
def test_binding_compiles_and_links_against_seqan(tmp_path):
    from seqan_gb300 import _native as N
    lib = N.build()
    out = tmp_path / "seqan_binding"
    cmd = ["g++", "-std=c++17", "-O1", "-fopenmp", "-w", "-I", os.path.join(REFERENCE, "include"),
           "-I", os.path.join(ROOT, "include"), os.path.join(ROOT, "tests", "cpp", "seqan_binding.cpp"),
           "-L", os.path.dirname(lib), "-lseqan_gb300", "-Wl,-rpath," + os.path.dirname(lib), "-o", str(out)]
    r = subprocess.run(cmd, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-4000:]
    assert out.exists()
