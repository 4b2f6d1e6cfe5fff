"""The C-ABI library builds for sm_103a, loads without a GPU, and exports every symbol that
include/*.h declares.  No compute calls are made here."""
import ctypes
import glob
import os
import re

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    names = set()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        with open(h) as f:
            text = f.read()
        names.update(re.findall(r"GBA_API\s+[\w\s\*]+?\b(gba_\w+)\s*\(", text))
    return sorted(names)


def test_library_exports_every_declared_symbol():
    from seqan_gb300 import _native
    path = _native.build()
    lib = ctypes.CDLL(path)
    syms = declared_symbols()
    assert len(syms) >= 19
    missing = [s for s in syms if not hasattr(lib, s)]
    assert not missing, missing
    assert set(syms) <= set(_native.EXPORTED) | set(syms)


def test_status_strings_without_gpu():
    from seqan_gb300 import _native
    lib = _native.lib()
    assert lib.gba_status_string(0) == b"ok"
    assert lib.gba_status_string(3) == b"HBM budget exceeded"


def test_no_cpu_fallback_in_package():
    """The engine package never imports, loads or links the oracle or the reference."""
    pkg = os.path.join(ROOT, "seqan_gb300")
    banned = ("from oracle", "import oracle", "seqan_oracle", "libseqan_ref", "orc_align")
    for path in glob.glob(os.path.join(pkg, "**", "*.*"), recursive=True):
        if path.endswith((".py", ".cu", ".cuh", ".h", ".cpp")):
            with open(path) as f:
                src = f.read()
            assert not any(b in src for b in banned), path
