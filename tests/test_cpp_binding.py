"""The C++ binding (include/seqan_gb300_seqan.h) against SeqAn 2 itself.

tests/cpp/seqan_binding.cpp calls every overload of the binding with the reference's own types.
Building it proves the overloads resolve against the reference's headers (no ambiguity with its
Serial/Parallel overloads) and that every engine symbol they use is exported.  With a GPU the
program runs, and its output -- scores, gapped rows, clip positions and CIGARs of every pair,
extended seeds, records read, SAM text and BAM bytes -- must equal, line by line,
tests/golden/cpp_binding_expected.txt: the same program built with -DGBA_AS_REFERENCE, every call
run by the reference (tests/golden/make_golden.py --only cpp).

The reference's headers come from SEQAN_INCLUDE, else the copy in baseline/_ref/include that the
build step makes where the reference tree exists; without them the tests are skipped."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SEQAN_INCLUDE = os.environ.get("SEQAN_INCLUDE") or os.path.join(ROOT, "baseline", "_ref", "include")
HAVE_HEADERS = os.path.isdir(os.path.join(SEQAN_INCLUDE, "seqan"))


def _build(out):
    from seqan_gb300 import _native as N
    lib = N.build()
    cmd = ["g++", "-std=c++17", "-O1", "-fopenmp", "-w", "-I", SEQAN_INCLUDE,
           "-I", os.path.join(ROOT, "include"), os.path.join(ROOT, "tests", "cpp", "seqan_binding.cpp"),
           "-L", os.path.dirname(lib), "-lseqan_gb300", "-Wl,-rpath," + os.path.dirname(lib), "-o", str(out)]
    r = subprocess.run(cmd, capture_output=True, text=True, timeout=900)
    assert r.returncode == 0, r.stderr[-4000:]
    assert out.exists()


@pytest.mark.skipif(not HAVE_HEADERS, reason="the reference's headers are not present")
@pytest.mark.skipif(shutil.which("g++") is None, reason="no C++ compiler")
def test_binding_compiles_and_links_against_seqan(tmp_path):
    _build(tmp_path / "seqan_binding")


@pytest.mark.gpu
@pytest.mark.skipif(not HAVE_HEADERS, reason="the reference's headers are not present")
@pytest.mark.skipif(shutil.which("g++") is None, reason="no C++ compiler")
def test_binding_output_equals_the_reference(tmp_path):
    exe = tmp_path / "seqan_binding"
    _build(exe)
    r = subprocess.run([str(exe)], capture_output=True, timeout=600)
    assert r.returncode == 0, r.stderr.decode()[-4000:]
    with open(os.path.join(ROOT, "tests", "golden", "cpp_binding_expected.txt"), "rb") as f:
        want = f.read().decode().splitlines()
    got = r.stdout.decode().splitlines()
    for k, (g, w) in enumerate(zip(got, want)):
        assert g == w, f"line {k + 1}: {g!r} != reference {w!r}"
    assert len(got) == len(want)
