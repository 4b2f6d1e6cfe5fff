"""Test-only loaders for the oracle (C restatement) and the compiled reference.

This module is TEST INFRASTRUCTURE: only tests/, __graft_entry__.smoke() and bench.py's CPU
baseline leg import it.  The engine (seqan_gb300/) never does.

* ``liboracle``  -- oracle/seqan_oracle.c, the CPU restatement of SeqAn 2's DP, built with gcc
  into oracle/_build/.  Builds on any host (x86 here, aarch64 on the GPU machine).
* ``libseqan_ref`` -- SeqAn 2 itself, compiled from the reference's headers by
  oracle/ref/Makefile into oracle/_ref/.  Only available where the reference tree exists; used
  to pin the restatement and to generate tests/golden fixtures.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from dataclasses import dataclass, field

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
REF_LIB = os.path.join(HERE, "_ref", "libseqan_ref.so")
ORACLE_LIB = os.path.join(BUILD, "libseqan_oracle.so")

FREE_TOP, FREE_LEFT, FREE_RIGHT, FREE_BOTTOM = 1, 2, 4, 8
SEG_DIAGONAL, SEG_HORIZONTAL, SEG_VERTICAL = 1, 2, 4


class OrcParams(C.Structure):
    _fields_ = [("mode", C.c_int32), ("gap_model", C.c_int32), ("free_ends", C.c_int32),
                ("band_on", C.c_int32), ("band_lower", C.c_int32), ("band_upper", C.c_int32),
                ("match", C.c_int32), ("mismatch", C.c_int32), ("gap_open", C.c_int32),
                ("gap_extend", C.c_int32), ("matrix", C.POINTER(C.c_int32)),
                ("alphabet_size", C.c_int32), ("score_bits", C.c_int32), ("traceback", C.c_int32),
                ("xdrop_on", C.c_int32), ("xdrop", C.c_int32), ("trace4", C.c_int32)]


class OrcResult(C.Structure):
    _fields_ = [("score", C.c_int32), ("end_h", C.c_int32), ("end_v", C.c_int32),
                ("begin_h", C.c_int32), ("begin_v", C.c_int32), ("n_segments", C.c_int32),
                ("valid", C.c_int32)]


class RefParams(C.Structure):
    _fields_ = [("mode", C.c_int32), ("free_ends", C.c_int32), ("band_on", C.c_int32),
                ("band_lower", C.c_int32), ("band_upper", C.c_int32), ("match", C.c_int32),
                ("mismatch", C.c_int32), ("gap_open", C.c_int32), ("gap_extend", C.c_int32),
                ("alphabet", C.c_int32), ("blosum62", C.c_int32), ("score_bits", C.c_int32),
                ("threads", C.c_int32)]


class OrcXdropParams(C.Structure):
    _fields_ = [("method", C.c_int32), ("direction", C.c_int32), ("match", C.c_int32),
                ("mismatch", C.c_int32), ("gap", C.c_int32), ("xdrop", C.c_int32),
                ("matrix", C.POINTER(C.c_int32)), ("alphabet_size", C.c_int32)]


class RefGapsOut(C.Structure):
    _fields_ = [("score", C.c_int32), ("h_clip_begin", C.c_int32), ("h_clip_end", C.c_int32),
                ("v_clip_begin", C.c_int32), ("v_clip_end", C.c_int32)]


@dataclass
class Problem:
    """One alignment configuration, in the reference's terms."""
    mode: str = "global"            # "global" | "local"
    free_ends: int = 0              # AlignConfig<TOP,LEFT,RIGHT,BOTTOM> as FREE_* bits
    band: tuple | None = None       # (lower, upper) or None
    match: int = 2
    mismatch: int = -3
    gap_open: int = -5
    gap_extend: int = -5
    matrix: np.ndarray | None = None   # alphabet^2 int32 (row = H code)
    score_bits: int = 32
    alphabet: str = "dna"           # "dna" (Dna5 codes) | "aa" (AminoAcid codes)
    xdrop: int | None = None        # mode "extend": the X-drop terminator's threshold
    trace4: bool = False            # trace values through the 4-bit code before the traceback
    dynamic: bool = False           # DynamicGaps cells (gap open / extend chosen by the neighbour's flag)

    @property
    def affine(self) -> bool:
        # The reference picks Gotoh iff open != extend (align/global_alignment_unbanded.h:801-810).
        return self.gap_open != self.gap_extend


ORACLE_SOURCES = ("seqan_oracle.c", "banded_chain_oracle.c")


def _compile_oracle(force: bool = False) -> str:
    srcs = [os.path.join(HERE, s) for s in ORACLE_SOURCES]
    newest = max(os.path.getmtime(s) for s in srcs + [os.path.join(HERE, "seqan_oracle.h")])
    if force or not os.path.exists(ORACLE_LIB) or os.path.getmtime(ORACLE_LIB) < newest:
        os.makedirs(BUILD, exist_ok=True)
        tmp = ORACLE_LIB + f".tmp{os.getpid()}"
        subprocess.check_call(["gcc", "-O3", "-fopenmp", "-shared", "-fPIC", "-o", tmp] + srcs)
        os.replace(tmp, ORACLE_LIB)
    return ORACLE_LIB


_orc = None
_ref = None


def liboracle():
    global _orc
    if _orc is None:
        _orc = C.CDLL(_compile_oracle())
        _orc.orc_align_batch.argtypes = [C.POINTER(OrcParams), C.c_int64, C.c_void_p, C.c_void_p,
                                         C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                         C.c_void_p, C.c_int32]
        _orc.orc_align_batch.restype = C.c_int
        _orc.orc_extend_seeds.argtypes = [C.POINTER(OrcXdropParams), C.c_int64, C.c_void_p, C.c_void_p,
                                          C.c_int64, C.c_void_p, C.c_void_p, C.c_int64, C.c_void_p,
                                          C.c_void_p, C.c_void_p, C.c_void_p, C.c_int32]
        _orc.orc_extend_seeds.restype = C.c_int
    return _orc


def ref_available() -> bool:
    return os.path.exists(REF_LIB)


REF_BENCH_LIB = os.path.join(HERE, "_ref", "libseqan_ref_bench.so")
REF_HEADERS_COPY = os.path.join(os.path.dirname(HERE), "baseline", "_ref", "include")
_ref_bench = None


def build_ref_bench(include: str | None = None) -> str | None:
    """Builds oracle/_ref/libseqan_ref_bench.so (the reference compiled from its own headers, only
    the benchmark workloads' call shapes) when missing; returns its path, or None when no copy of
    the reference's headers is available (SEQAN_INCLUDE, else baseline/_ref/include)."""
    if os.path.exists(REF_BENCH_LIB):
        return REF_BENCH_LIB
    include = include or os.environ.get("SEQAN_INCLUDE") or REF_HEADERS_COPY
    if not os.path.isdir(os.path.join(include, "seqan")):
        return None
    subprocess.check_call(["make", "-C", os.path.join(HERE, "ref"), "bench", f"-j{os.cpu_count() or 4}",
                           f"SEQAN_INCLUDE={os.path.abspath(include)}"], stdout=subprocess.DEVNULL)
    return REF_BENCH_LIB


def libref_bench():
    """The benchmark-shape reference library (see build_ref_bench), with libref()'s signatures."""
    global _ref_bench
    if _ref_bench is None:
        lib = C.CDLL(REF_BENCH_LIB)
        lib.ref_batch_score.argtypes = [C.POINTER(RefParams), C.c_int64, C.c_void_p, C.c_void_p,
                                        C.c_void_p, C.c_void_p, C.c_void_p]
        lib.ref_batch_gaps.argtypes = [C.POINTER(RefParams), C.c_int64, C.c_void_p, C.c_void_p,
                                       C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                       C.c_void_p, C.c_void_p, C.c_int64]
        lib.ref_has_shape.argtypes = [C.c_int32, C.POINTER(RefParams)]
        lib.ref_simd_bytes.restype = C.c_int32
        _ref_bench = lib
    return _ref_bench


def libref():
    global _ref
    if _ref is None:
        _ref = C.CDLL(REF_LIB)
        _ref.ref_batch_score.argtypes = [C.POINTER(RefParams), C.c_int64, C.c_void_p, C.c_void_p,
                                         C.c_void_p, C.c_void_p, C.c_void_p]
        _ref.ref_batch_gaps.argtypes = [C.POINTER(RefParams), C.c_int64, C.c_void_p, C.c_void_p,
                                        C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                        C.c_void_p, C.c_void_p, C.c_int64]
        _ref.ref_pair_segments.argtypes = [C.POINTER(RefParams), C.c_void_p, C.c_int32, C.c_void_p,
                                           C.c_int32, C.c_void_p, C.c_void_p, C.c_int32, C.c_void_p]
        _ref.ref_has_shape.argtypes = [C.c_int32, C.POINTER(RefParams)]
        if hasattr(_ref, "ref_dynamic_segments"):
            _ref.ref_dynamic_segments.argtypes = [C.POINTER(RefParams), C.c_void_p, C.c_int32, C.c_void_p,
                                                  C.c_int32, C.c_void_p, C.c_void_p, C.c_int32, C.c_void_p]
        _ref.ref_blosum62.argtypes = [C.c_void_p]
        _ref.ref_encode.argtypes = [C.c_int32, C.c_char_p, C.c_int64, C.c_void_p]
        _ref.ref_extend_seeds.argtypes = [C.c_int32] * 8 + [C.c_int64, C.c_void_p, C.c_void_p, C.c_void_p,
                                                             C.c_void_p, C.c_int64, C.c_void_p, C.c_void_p,
                                                             C.c_void_p, C.c_int32]
    return _ref


def concat(seqs):
    """List of uint8 arrays -> (codes, offsets[int64, n+1])."""
    lens = np.array([len(s) for s in seqs], dtype=np.int64)
    off = np.zeros(len(seqs) + 1, dtype=np.int64)
    np.cumsum(lens, out=off[1:])
    codes = np.concatenate([np.asarray(s, dtype=np.uint8) for s in seqs]) if len(seqs) and off[-1] else \
        np.zeros(1, dtype=np.uint8)
    return np.ascontiguousarray(codes), off


def _ptr(a):
    return a.ctypes.data_as(C.c_void_p) if a is not None else None


def _orc_params(pb: Problem, traceback: bool) -> OrcParams:
    p = OrcParams()
    p.mode = {"global": 0, "local": 1, "extend": 2}[pb.mode]
    p.xdrop_on = 0 if pb.xdrop is None else 1
    p.xdrop = 0 if pb.xdrop is None else int(pb.xdrop)
    p.gap_model = 2 if pb.dynamic else (1 if pb.affine else 0)
    p.free_ends = pb.free_ends
    p.band_on = 1 if pb.band is not None else 0
    p.band_lower, p.band_upper = (pb.band if pb.band is not None else (0, 0))
    p.match, p.mismatch, p.gap_open, p.gap_extend = pb.match, pb.mismatch, pb.gap_open, pb.gap_extend
    if pb.matrix is not None:
        mat = np.ascontiguousarray(pb.matrix, dtype=np.int32)
        p._mat_keepalive = mat
        p.matrix = mat.ctypes.data_as(C.POINTER(C.c_int32))
        p.alphabet_size = int(round(np.sqrt(mat.size)))
    p.score_bits = pb.score_bits
    p.traceback = 1 if traceback else 0
    p.trace4 = 1 if pb.trace4 else 0
    return p


@dataclass
class BatchResult:
    score: np.ndarray
    end_h: np.ndarray
    end_v: np.ndarray
    begin_h: np.ndarray | None = None
    begin_v: np.ndarray | None = None
    valid: np.ndarray | None = None
    segments: list = field(default_factory=list)   # per pair: list of (h, v, len, type)
    seg_flat: np.ndarray | None = None             # flat=True: [total, 4] uint32, pairs back to back
    seg_offsets: np.ndarray | None = None          # flat=True: [n + 1] int64


def oracle_batch(pb: Problem, H, V, traceback: bool = False, threads: int = 0, flat: bool = False) -> BatchResult:
    """Runs the C restatement on pairs (H[k], V[k]).

    flat=True returns the segments as one dense array (seg_flat, seg_offsets) in the layout of the
    engine's gba_result instead of per-pair tuple lists (for batches of a million pairs)."""
    lib = liboracle()
    n = len(H)
    sh, oh = concat(H)
    sv, ov = concat(V)
    params = _orc_params(pb, traceback)
    out = (OrcResult * max(n, 1))()
    segs = seg_off = None
    if traceback:
        caps = (oh[1:] - oh[:-1]) + (ov[1:] - ov[:-1]) + 4
        seg_off = np.zeros(n + 1, dtype=np.int64)
        np.cumsum(caps, out=seg_off[1:])
        segs = np.zeros((int(seg_off[-1]) + 1, 4), dtype=np.uint32)
    rc = lib.orc_align_batch(C.byref(params), n, _ptr(sh), _ptr(oh), _ptr(sv), _ptr(ov),
                             C.cast(out, C.c_void_p), _ptr(segs), _ptr(seg_off), threads)
    if rc != 0:
        raise RuntimeError(f"oracle returned {rc}")
    arr = np.frombuffer(out, dtype=np.int32).reshape(-1, 7)[:n]
    res = BatchResult(score=arr[:, 0].copy(), end_h=arr[:, 1].copy(), end_v=arr[:, 2].copy(),
                      begin_h=arr[:, 3].copy(), begin_v=arr[:, 4].copy(), valid=arr[:, 6].copy())
    if traceback and flat:
        cnt = np.maximum(arr[:, 5], 0).astype(np.int64)
        res.seg_offsets = np.zeros(n + 1, dtype=np.int64)
        np.cumsum(cnt, out=res.seg_offsets[1:])
        pair = np.repeat(np.arange(n, dtype=np.int64), cnt)
        local = np.arange(int(res.seg_offsets[-1]), dtype=np.int64) - res.seg_offsets[pair]
        res.seg_flat = segs[seg_off[pair] + local].copy()
    elif traceback:
        for k in range(n):
            cnt = arr[k, 5]
            res.segments.append([tuple(int(x) for x in segs[seg_off[k] + i]) for i in range(max(cnt, 0))])
    return res


def cigar_words_flat(seg_flat, seg_offsets, spliced_gap_thresh: int = 20):
    """CIGARs of many pairs at once, as BAM words (length << 4 | op index into "MIDNSHP=X"), from
    dense TraceSegment_ lists (traceback order): the same operations as cigar_string -- the
    segments from the alignment begin on, runs of one operation joined, D runs of at least
    spliced_gap_thresh as N (bam_io/cigar.h:261-339).  Returns (words, offsets[n + 1])."""
    seg_flat = np.asarray(seg_flat, dtype=np.uint32).reshape(-1, 4)
    off = np.asarray(seg_offsets, dtype=np.int64)
    n = len(off) - 1
    cnt = np.diff(off)
    total = int(off[-1])
    if total == 0:
        return np.zeros(0, np.uint32), np.zeros(n + 1, np.int64)
    pair = np.repeat(np.arange(n, dtype=np.int64), cnt)
    i = np.arange(total, dtype=np.int64)
    rs = seg_flat[2 * off[pair] + cnt[pair] - 1 - i]          # each pair's list reversed
    tp = rs[:, 3]
    op = np.where(tp == SEG_DIAGONAL, 0, np.where(tp == SEG_VERTICAL, 1, 2)).astype(np.int64)
    start = np.ones(total, dtype=bool)
    start[1:] = (op[1:] != op[:-1]) | (pair[1:] != pair[:-1])
    first = np.nonzero(start)[0]
    run_len = np.add.reduceat(rs[:, 2].astype(np.int64), first)
    run_op = op[first]
    run_op = np.where((run_op == 2) & (run_len >= spliced_gap_thresh), 3, run_op)
    words = ((run_len << 4) | run_op).astype(np.uint32)
    coff = np.zeros(n + 1, dtype=np.int64)
    np.cumsum(np.bincount(pair[first], minlength=n), out=coff[1:])
    return words, coff


def _ref_params(pb: Problem, threads: int) -> RefParams:
    p = RefParams()
    p.mode = 1 if pb.mode == "local" else 0
    p.free_ends = pb.free_ends
    p.band_on = 1 if pb.band is not None else 0
    p.band_lower, p.band_upper = (pb.band if pb.band is not None else (0, 0))
    p.match, p.mismatch, p.gap_open, p.gap_extend = pb.match, pb.mismatch, pb.gap_open, pb.gap_extend
    p.alphabet = 0 if pb.alphabet == "dna" else 1
    p.blosum62 = 1 if pb.matrix is not None else 0
    p.score_bits = pb.score_bits
    p.threads = threads
    return p


def ref_has_shape(kind: int, pb: Problem) -> bool:
    p = _ref_params(pb, 1)
    return bool(libref().ref_has_shape(kind, C.byref(p)))


def ref_batch_score(pb: Problem, H, V, threads: int = 1, lib=None) -> np.ndarray:
    lib = lib or libref()
    n = len(H)
    sh, oh = concat(H)
    sv, ov = concat(V)
    out = np.zeros(max(n, 1), dtype=np.int32)
    p = _ref_params(pb, threads)
    rc = lib.ref_batch_score(C.byref(p), n, _ptr(sh), _ptr(oh), _ptr(sv), _ptr(ov), _ptr(out))
    if rc != 0:
        raise RuntimeError(f"reference call shape not instantiated (rc={rc}): {pb}")
    return out[:n]


def ref_batch_gaps(pb: Problem, H, V, threads: int = 1, cigar: bool = False, lib=None, decode: bool = True):
    """Returns (scores, clip[n,4] = hb,he,vb,ve, rows[list of (rowH, rowV)], cigars); decode=False
    skips turning the rows and CIGARs into Python strings (returns None for both)."""
    lib = lib or libref()
    n = len(H)
    sh, oh = concat(H)
    sv, ov = concat(V)
    out = (RefGapsOut * max(n, 1))()
    caps = 2 * ((oh[1:] - oh[:-1]) + (ov[1:] - ov[:-1])) + 4
    row_off = np.zeros(n + 1, dtype=np.int64)
    np.cumsum(caps, out=row_off[1:])
    rows = np.zeros(int(row_off[-1]) + 1, dtype=np.uint8)
    cstride = int(caps.max() if n else 4) * 4 + 16
    cig = np.zeros(n * cstride + 1, dtype=np.uint8) if cigar else None
    p = _ref_params(pb, threads)
    rc = lib.ref_batch_gaps(C.byref(p), n, _ptr(sh), _ptr(oh), _ptr(sv), _ptr(ov),
                            C.cast(out, C.c_void_p), _ptr(rows), _ptr(row_off), _ptr(cig), cstride)
    if rc != 0:
        raise RuntimeError(f"reference call shape not instantiated (rc={rc}): {pb}")
    arr = np.frombuffer(out, dtype=np.int32).reshape(-1, 5)[:n]
    if not decode:
        return arr[:, 0].copy(), arr[:, 1:5].copy(), None, None
    row_strs = []
    for k in range(n):
        raw = bytes(rows[row_off[k]:row_off[k + 1]]).split(b"\0", 1)[0].decode()
        a, b = raw.split("\n")
        row_strs.append((a, b))
    cigars = None
    if cigar:
        cigars = [bytes(cig[k * cstride:(k + 1) * cstride]).split(b"\0", 1)[0].decode() for k in range(n)]
    return arr[:, 0].copy(), arr[:, 1:5].copy(), row_strs, cigars


def ref_pair_segments(pb: Problem, h, v):
    lib = libref()
    h = np.ascontiguousarray(h, dtype=np.uint8)
    v = np.ascontiguousarray(v, dtype=np.uint8)
    cap = len(h) + len(v) + 8
    segs = np.zeros((cap, 4), dtype=np.uint32)
    score = C.c_int32(0)
    nseg = C.c_int32(0)
    p = _ref_params(pb, 1)
    rc = lib.ref_pair_segments(C.byref(p), _ptr(h), len(h), _ptr(v), len(v), C.byref(score),
                               _ptr(segs), cap, C.byref(nseg))
    if rc != 0:
        raise RuntimeError(f"reference call shape not instantiated (rc={rc}): {pb}")
    return score.value, [tuple(int(x) for x in segs[i]) for i in range(nseg.value)]


def ref_dynamic_segments(pb: Problem, h, v):
    """The reference's single-pair DP with DynamicGaps cells: (score, TraceSegment_ list)."""
    lib = libref()
    h = np.ascontiguousarray(h, dtype=np.uint8)
    v = np.ascontiguousarray(v, dtype=np.uint8)
    cap = len(h) + len(v) + 8
    segs = np.zeros((cap, 4), dtype=np.uint32)
    score = C.c_int32(0)
    nseg = C.c_int32(0)
    p = _ref_params(pb, 1)
    rc = lib.ref_dynamic_segments(C.byref(p), _ptr(h), len(h), _ptr(v), len(v), C.byref(score), _ptr(segs), cap,
                                  C.byref(nseg))
    if rc != 0:
        raise RuntimeError(f"reference call shape not instantiated (rc={rc}): {pb}")
    return score.value, [tuple(int(x) for x in segs[i]) for i in range(nseg.value)]


def ref_blosum62() -> np.ndarray:
    out = np.zeros(27 * 27, dtype=np.int32)
    libref().ref_blosum62(_ptr(out))
    return out.reshape(27, 27)


def ref_encode(alphabet: str, text: str) -> np.ndarray:
    b = text.encode()
    out = np.zeros(max(len(b), 1), dtype=np.uint8)
    code = {"dna5": 0, "aa": 1, "dna": 2}[alphabet]
    libref().ref_encode(code, b, len(b), _ptr(out))
    return out[:len(b)]


# ---------------------------------------------------------------------------------------------
# Rendering helpers shared by the tests (segments -> gapped rows / CIGAR), following
# _adaptTraceSegmentsTo (align/dp_traceback_adaptor.h:57-117) and getCigarString
# (bam_io/cigar.h:261-339).
# ---------------------------------------------------------------------------------------------

# ---------------------------------------------------------------------------------------------
# Seed extension: extendSeed(Seed<Simple>, database, query, direction, ...) over a batch
# (seeds/seeds_extension.h).  Seeds are int64 arrays [n, 6] = beginH, beginV, endH, endV,
# lowerDiagonal, upperDiagonal.
# ---------------------------------------------------------------------------------------------

EXTEND_LEFT, EXTEND_RIGHT, EXTEND_BOTH = 1, 2, 3
MATCH_EXTEND, UNGAPPED_XDROP, GAPPED_XDROP = 0, 1, 2


@dataclass
class SeedProblem:
    method: int = GAPPED_XDROP
    direction: int = EXTEND_BOTH
    match: int = 1
    mismatch: int = -1
    gap: int = -1
    xdrop: int = 10
    matrix: np.ndarray | None = None   # alphabet^2 int32, row = first argument of score()
    alphabet: str = "dna"


def seeds_array(seeds):
    """[(beginH, beginV, length)] or [n, 6] -> int64 [n, 6] as Seed(beginH, beginV, length)
    constructs it (seeds/seeds_seed_simple.h:98-104)."""
    a = np.asarray(seeds, dtype=np.int64)
    if a.ndim == 2 and a.shape[1] == 6:
        return np.ascontiguousarray(a.copy())
    a = a.reshape(-1, 3)
    out = np.zeros((len(a), 6), dtype=np.int64)
    out[:, 0], out[:, 1] = a[:, 0], a[:, 1]
    out[:, 2], out[:, 3] = a[:, 0] + a[:, 2], a[:, 1] + a[:, 2]
    out[:, 4] = out[:, 5] = a[:, 0] - a[:, 1]
    return out


def oracle_extend_seeds(sp: SeedProblem, H, V, seeds, pair_of_seed=None, threads: int = 0, seed_h=None,
                        seed_v=None):
    """C restatement over a batch; returns (seeds [n, 6], xscores [n, 2]).  Seed i lies on
    H[seed_h[i]] and V[seed_v[i]]; pair_of_seed sets both."""
    lib = liboracle()
    sh, oh = concat(H)
    sv, ov = concat(V)
    s = seeds_array(seeds)
    xs = np.zeros((max(len(s), 1), 2), dtype=np.int32)
    p = OrcXdropParams(sp.method, sp.direction, sp.match, sp.mismatch, sp.gap, sp.xdrop, None, 0)
    if sp.matrix is not None:
        mat = np.ascontiguousarray(sp.matrix, dtype=np.int32)
        p.matrix = mat.ctypes.data_as(C.POINTER(C.c_int32))
        p.alphabet_size = int(round(np.sqrt(mat.size)))
    if pair_of_seed is not None:
        seed_h = seed_v = pair_of_seed
    ih = None if seed_h is None else np.ascontiguousarray(seed_h, dtype=np.int32)
    iv = None if seed_v is None else np.ascontiguousarray(seed_v, dtype=np.int32)
    rc = lib.orc_extend_seeds(C.byref(p), len(H), _ptr(sh), _ptr(oh), len(V), _ptr(sv), _ptr(ov), len(s),
                              _ptr(ih), _ptr(iv), _ptr(s), _ptr(xs), threads)
    if rc != 0:
        raise RuntimeError(f"oracle returned {rc}")
    return s, xs[:len(s)]


def ref_extend_seeds(sp: SeedProblem, H, V, seeds, pair_of_seed=None, threads: int = 1):
    """The reference's extendSeed over a batch; returns (seeds [n, 6], xscores [n, 2])."""
    lib = libref()
    sh, oh = concat(H)
    sv, ov = concat(V)
    s = seeds_array(seeds)
    xs = np.zeros((max(len(s), 1), 2), dtype=np.int32)
    pos = None if pair_of_seed is None else np.ascontiguousarray(pair_of_seed, dtype=np.int32)
    rc = lib.ref_extend_seeds(sp.method, sp.direction, 0 if sp.alphabet == "dna" else 1,
                              1 if sp.matrix is not None else 0, sp.match, sp.mismatch, sp.gap, sp.xdrop,
                              len(H), _ptr(sh), _ptr(oh), _ptr(sv), _ptr(ov), len(s), _ptr(pos), _ptr(s),
                              _ptr(xs), threads)
    if rc != 0:
        raise RuntimeError(f"reference returned {rc}")
    return s, xs[:len(s)]


# ---------------------------------------------------------------------------------------------
# extendAlignment (align_extend/align_extend.h): an ungapped seed alignment hSeq[hb, he) /
# vSeq[vb, ve) grown to the left on the reversed prefixes and to the right on the suffixes by the
# AlignExtend DP (mode "extend", optional X-drop), then joined around the seed.
# ---------------------------------------------------------------------------------------------

@dataclass
class ExtendResult:
    score: int
    row0: str
    row1: str
    h_begin: int
    h_end: int
    v_begin: int
    v_end: int
    left_score: int = 0
    right_score: int = 0
    left_segments: list = field(default_factory=list)    # prefix coordinates, traceback order
    right_segments: list = field(default_factory=list)   # suffix coordinates, traceback order


def _seg_end(seg):
    hb, vb, ln, tp = seg
    return (hb + (ln if tp in (SEG_DIAGONAL, SEG_HORIZONTAL) else 0),
            vb + (ln if tp in (SEG_DIAGONAL, SEG_VERTICAL) else 0))


def reverse_partial_trace(segments, len_h, len_v):
    """_reversePartialTrace (align_extend/align_extend.h:91-109): begin = length - end, reversed."""
    out = []
    for seg in segments:
        eh, ev = _seg_end(seg)
        out.append((len_h - eh, len_v - ev, seg[2], seg[3]))
    return out[::-1]


def center_score(pb: Problem, row0: str, row1: str, letters="ACGTN") -> int:
    """The aligned part's score as _extendAlignmentImpl computes it when origScore is omitted
    (align_extend/align_extend.h:250-270): gap open for a gap column that starts the row pair's
    gap pattern anew (first column, or either row's gap state changed), gap extend otherwise,
    the substitution score for the rest."""
    code = {ch: k for k, ch in enumerate(letters)}
    sub = (lambda a, b: int(pb.matrix[a, b])) if pb.matrix is not None else \
        (lambda a, b: pb.match if a == b else pb.mismatch)
    total = 0
    for i, (a, b) in enumerate(zip(row0, row1)):
        g0, g1 = a == "-", b == "-"
        if g0 or g1:
            if i == 0 or (row0[i - 1] == "-") != g0 or (row1[i - 1] == "-") != g1:
                total += pb.gap_open
            else:
                total += pb.gap_extend
        else:
            total += sub(code[a], code[b])
    return total


def _wrap32(x: int) -> int:
    return (x + 2 ** 31) % 2 ** 32 - 2 ** 31


def oracle_extend_alignment(pb: Problem, h, v, positions, direction, letters="ACGTN", orig_score=None,
                            center=None) -> ExtendResult:
    """The reference's _extendAlignmentImpl (align_extend/align_extend.h:211-372), restated on the
    oracle's DP (pb.mode must be "extend"; pb.band gives the lowerDiag / upperDiag overloads and
    pb.xdrop the X-drop ones).  center: the aligned part's rows as text with '-' for gaps (None:
    ungapped); orig_score: the origScore argument (None: computed from the rows)."""
    h = np.ascontiguousarray(h, dtype=np.uint8)
    v = np.ascontiguousarray(v, dtype=np.uint8)
    hb, vb, he, ve = (int(x) for x in positions)
    ext_left = bool(direction & EXTEND_LEFT) and hb > 0 and vb > 0
    ext_right = bool(direction & EXTEND_RIGHT) and he < len(h) and ve < len(v)
    text = lambda codes: "".join(letters[int(c)] for c in codes)
    c0, c1 = center if center is not None else (text(h[hb:he]), text(v[vb:ve]))
    center_sc = center_score(pb, c0, c1, letters) if orig_score is None else int(orig_score)
    left = ([], 0)
    if ext_left:
        r = oracle_batch(pb, [h[:hb][::-1].copy()], [v[:vb][::-1].copy()], traceback=True)
        left = (reverse_partial_trace(r.segments[0], hb, vb), int(r.score[0]))
    right = ([], 0)
    if ext_right:
        r = oracle_batch(pb, [h[he:].copy()], [v[ve:].copy()], traceback=True)
        right = (r.segments[0], int(r.score[0]))
    l0, l1 = render_rows(left[0], text(h[:hb]), text(v[:vb]))
    r0, r1 = render_rows(right[0], text(h[he:]), text(v[ve:]))
    lh = sum(s[2] for s in left[0] if s[3] in (SEG_DIAGONAL, SEG_HORIZONTAL))
    lv = sum(s[2] for s in left[0] if s[3] in (SEG_DIAGONAL, SEG_VERTICAL))
    rh = sum(s[2] for s in right[0] if s[3] in (SEG_DIAGONAL, SEG_HORIZONTAL))
    rv = sum(s[2] for s in right[0] if s[3] in (SEG_DIAGONAL, SEG_VERTICAL))
    return ExtendResult(_wrap32(left[1] + center_sc + right[1]), l0 + c0 + r0, l1 + c1 + r1,
                        hb - lh, he + rh, vb - lv, ve + rv, left[1], right[1], left[0], right[0])


def ref_extend_alignment(pb: Problem, h, v, positions, direction, orig_score=None, center=None) -> ExtendResult:
    """The reference's extendAlignment (oracle/ref/units/align_extend.cpp): the overload with
    origScore when orig_score is given, (lowerDiag, upperDiag) with pb.band, xDrop with
    pb.xdrop; center: the aligned part's rows with '-' for gaps (None: ungapped)."""
    lib = libref()
    lib.ref_extend_alignment_ex.argtypes = (
        [C.c_int32] * 6 + [C.c_void_p, C.c_int64, C.c_void_p, C.c_int64, C.c_void_p] + [C.c_int32] * 8 +
        [C.c_char_p, C.c_char_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int64, C.c_void_p])
    h = np.ascontiguousarray(h, dtype=np.uint8)
    v = np.ascontiguousarray(v, dtype=np.uint8)
    pos = np.array(positions, dtype=np.int64)
    cap = 2 * (len(h) + len(v)) + 8
    row0 = C.create_string_buffer(cap)
    row1 = C.create_string_buffer(cap)
    ends = np.zeros(4, dtype=np.int64)
    score = C.c_int32(0)
    lo, up = pb.band if pb.band is not None else (0, 0)
    c0 = center[0].encode() if center is not None else None
    c1 = center[1].encode() if center is not None else None
    rc = lib.ref_extend_alignment_ex(0 if pb.alphabet == "dna" else 1, 1 if pb.matrix is not None else 0, pb.match,
                                     pb.mismatch, pb.gap_open, pb.gap_extend, _ptr(h), len(h), _ptr(v), len(v),
                                     _ptr(pos), int(direction), 0 if pb.band is None else 1, int(lo), int(up),
                                     0 if pb.xdrop is None else 1, 0 if pb.xdrop is None else int(pb.xdrop),
                                     0 if orig_score is None else 1, 0 if orig_score is None else int(orig_score),
                                     c0, c1, C.byref(score), row0, row1, cap, _ptr(ends))
    if rc != 0:
        raise RuntimeError(f"reference returned {rc}")
    return ExtendResult(score.value, row0.value.decode(), row1.value.decode(), int(ends[0]), int(ends[1]),
                        int(ends[2]), int(ends[3]))


# ---------------------------------------------------------------------------------------------
# Waterman-Eggert suboptimal local alignments (LocalAlignmentEnumerator<Score, Unbanded>).
# ---------------------------------------------------------------------------------------------

class OrcWeParams(C.Structure):
    _fields_ = [("match", C.c_int32), ("mismatch", C.c_int32), ("gap", C.c_int32), ("matrix", C.POINTER(C.c_int32)),
                ("alphabet_size", C.c_int32), ("cutoff", C.c_int32)]


@dataclass
class LocalAlignment:
    score: int
    row0: str
    row1: str
    h_begin: int
    h_end: int
    v_begin: int
    v_end: int
    segments: list = field(default_factory=list)   # runs in alignment order (h, v, len, type)


def _we_rows(segments, h_text, v_text):
    r0, r1 = [], []
    for hb, vb, ln, tp in segments:
        if tp == SEG_DIAGONAL:
            r0.append(h_text[hb:hb + ln]); r1.append(v_text[vb:vb + ln])
        elif tp == SEG_HORIZONTAL:
            r0.append(h_text[hb:hb + ln]); r1.append("-" * ln)
        else:
            r0.append("-" * ln); r1.append(v_text[vb:vb + ln])
    return "".join(r0), "".join(r1)


def oracle_local_enumerate(h, v, match=2, mismatch=-1, gap=-2, cutoff=0, matrix=None, max_count=1000,
                           letters="ACGTN", band=None) -> list:
    """Waterman-Eggert alignments of the oracle restatement (orc_waterman_eggert): each with its
    score, gapped rows, clipped source positions and runs of alignment columns.  A trailing None
    marks an enumeration stopped where the reference's next step is undefined."""
    lib = liboracle()
    lib.orc_waterman_eggert.restype = C.c_int32
    lib.orc_waterman_eggert.argtypes = [C.POINTER(OrcWeParams), C.c_void_p, C.c_int32, C.c_void_p, C.c_int32,
                                        C.c_int32, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int64,
                                        C.c_void_p, C.c_void_p]
    h = np.ascontiguousarray(h, dtype=np.uint8)
    v = np.ascontiguousarray(v, dtype=np.uint8)
    p = OrcWeParams(match, mismatch, gap, None, 0, cutoff)
    keep = None
    if matrix is not None:
        keep = np.ascontiguousarray(matrix, dtype=np.int32)
        p.matrix = keep.ctypes.data_as(C.POINTER(C.c_int32))
        p.alphabet_size = int(round(np.sqrt(keep.size)))
    cap = max_count * (len(h) + len(v) + 2) + 8
    scores = np.zeros(max(max_count, 1), np.int32)
    begins = np.zeros(2 * max(max_count, 1), np.int32)
    ends = np.zeros(2 * max(max_count, 1), np.int32)
    segs = np.zeros((cap, 4), np.uint32)
    off = np.zeros(max_count + 1, np.int64)
    undef = C.c_int32(0)
    if band is None:
        k = lib.orc_waterman_eggert(C.byref(p), _ptr(h), len(h), _ptr(v), len(v), max_count, _ptr(scores),
                                    _ptr(begins), _ptr(ends), _ptr(segs), cap, _ptr(off), C.byref(undef))
    else:
        lib.orc_waterman_eggert_banded.restype = C.c_int32
        lib.orc_waterman_eggert_banded.argtypes = [C.POINTER(OrcWeParams), C.c_int32, C.c_int32] + \
            lib.orc_waterman_eggert.argtypes[1:]
        k = lib.orc_waterman_eggert_banded(C.byref(p), int(band[0]), int(band[1]), _ptr(h), len(h), _ptr(v), len(v),
                                           max_count, _ptr(scores), _ptr(begins), _ptr(ends), _ptr(segs), cap,
                                           _ptr(off), C.byref(undef))
    if k < 0:
        raise RuntimeError("segment buffer too small")
    ht = "".join(letters[int(c)] for c in h)
    vt = "".join(letters[int(c)] for c in v)
    out = []
    for i in range(k):
        sg = [tuple(int(x) for x in segs[q]) for q in range(off[i], off[i + 1])]
        r0, r1 = _we_rows(sg, ht, vt)
        # each row's clipped region starts at its first residue (after an alignment whose first
        # column is a gap the two rows differ in length, as the reference prints them)
        r0, r1 = r0.strip("-"), r1.strip("-")
        out.append(LocalAlignment(int(scores[i]), r0, r1, int(begins[2 * i]), int(ends[2 * i]),
                                  int(begins[2 * i + 1]), int(ends[2 * i + 1]), sg))
    del keep
    if undef.value:
        out.append(None)   # marker: asking the reference for another alignment is undefined here
    return out


def ref_local_enumerate(h, v, match=2, mismatch=-1, gap=-2, cutoff=0, blosum62=False, alphabet="dna",
                        max_count=1000, lib=None, band=None) -> list:
    """The reference's LocalAlignmentEnumerator (oracle/ref/units/waterman_eggert.cpp); lib: the
    library to call (default libref(); libref_bench() holds the same entry)."""
    lib = lib or libref()
    lib.ref_local_enumerate.argtypes = [C.c_int32] * 7 + [C.c_void_p, C.c_int64, C.c_void_p, C.c_int64, C.c_int32,
                                                          C.c_void_p, C.c_void_p, C.c_char_p, C.c_int64]
    h = np.ascontiguousarray(h, dtype=np.uint8)
    v = np.ascontiguousarray(v, dtype=np.uint8)
    scores = np.zeros(max(max_count, 1), np.int32)
    pos = np.zeros(4 * max(max_count, 1), np.int32)
    cap = max_count * 2 * (len(h) + len(v) + 2) + 8
    rows = C.create_string_buffer(cap)
    if band is None:
        k = lib.ref_local_enumerate(0 if alphabet == "dna" else 1, 1 if blosum62 else 0, match, mismatch, gap, gap,
                                    cutoff, _ptr(h), len(h), _ptr(v), len(v), max_count, _ptr(scores), _ptr(pos),
                                    rows, cap)
    else:
        lib.ref_local_enumerate_banded.argtypes = [C.c_int32] * 8 + [C.c_void_p, C.c_int64, C.c_void_p, C.c_int64,
                                                                     C.c_int32, C.c_void_p, C.c_void_p, C.c_char_p,
                                                                     C.c_int64]
        k = lib.ref_local_enumerate_banded(0 if alphabet == "dna" else 1, 1 if blosum62 else 0, match, mismatch, gap,
                                           int(band[0]), int(band[1]), cutoff, _ptr(h), len(h), _ptr(v), len(v),
                                           max_count, _ptr(scores), _ptr(pos), rows, cap)
    if k < 0:
        raise RuntimeError("row buffer too small")
    lines = rows.value.decode().split("\n")
    return [LocalAlignment(int(scores[i]), lines[2 * i], lines[2 * i + 1], int(pos[4 * i]), int(pos[4 * i + 1]),
                           int(pos[4 * i + 2]), int(pos[4 * i + 3])) for i in range(k)]


# ---------------------------------------------------------------------------------------------
# SAM lines (bam_io/write_sam.h:126-217) of BamAlignmentRecord fields given as plain lists.
# ---------------------------------------------------------------------------------------------

_TAG_FMT = {"c": ("<b", 1), "C": ("<B", 1), "s": ("<h", 2), "S": ("<H", 2), "i": ("<i", 4), "I": ("<I", 4),
            "f": ("<f", 4)}


def _tag_str(x, ty):
    """A tag number as the reference appends it: integers in decimal, floats as C's "%g" of the
    value (basic/basic_stream.h:1145-1155; a negative NaN prints as "-nan")."""
    if ty != "f":
        return str(x)
    import math
    if math.isnan(x):
        return "-nan" if math.copysign(1.0, x) < 0 else "nan"
    return "%g" % x


def tags_bam_to_sam(t: bytes) -> str:
    """appendTagsBamToSam (bam_io/bam_sam_conversion.h:250-360) of one record's BAM tag bytes."""
    import struct
    out, i = [], 0
    while i < len(t):
        name, ty = t[i:i + 2].decode("latin1"), chr(t[i + 2])
        i += 3
        shown = "i" if ty.lower() in "csi" else ty
        if ty in "ZH":
            j = t.index(0, i)
            val = t[i:j].decode("latin1")
            i = j + 1
        elif ty == "B":
            et = chr(t[i])
            cnt = struct.unpack_from("<I", t, i + 1)[0]
            i += 5
            fmt, sz = _TAG_FMT[et]
            vals = [struct.unpack_from(fmt, t, i + q * sz)[0] for q in range(cnt)]
            i += cnt * sz
            val = et + "".join("," + _tag_str(x, et) for x in vals)
        elif ty == "A":
            val = chr(t[i])
            i += 1
        else:
            fmt, sz = _TAG_FMT[ty]
            val = _tag_str(struct.unpack_from(fmt, t, i)[0], ty)
            i += sz
        out.append(f"{name}:{shown}:{val}")
    return "\t".join(out)


def write_sam(rec) -> str:
    """Restates the reference's SAM record writer for rec (a seqan_gb300.sam.SamRecords)."""
    lines = []
    for k in range(len(rec.qname)):
        rid, rn = int(rec.ref_id[k]), int(rec.next_ref_id[k])
        cig = "".join(f"{int(c) >> 4}{'MIDNSHP=X'[int(c) & 15]}" for c in rec.cigar[k]) or "*"
        seq = "".join(rec.letters[int(x)] for x in rec.seq[k]) or "*"
        qual = (rec.qual[k] if rec.qual is not None else "") or "*"
        tlen = int(rec.tlen[k])
        tags = getattr(rec, "tags", None)
        tail = ("\t" + tags_bam_to_sam(tags[k])) if tags is not None and len(tags[k]) else ""
        lines.append("\t".join([rec.qname[k], str(int(rec.flag[k])), "*" if rid == -1 else rec.contigs[rid],
                                 str(int(rec.pos[k]) + 1), str(int(rec.mapq[k])), cig,
                                 "*" if rn == -1 else ("=" if rn == rid else rec.contigs[rn]),
                                 str(int(rec.next_pos[k]) + 1), "0" if tlen == 0 else str(tlen), seq, qual]) + tail
                     + "\n")
    return "".join(lines)


def sam_arrays(rec):
    """The records as the flat arrays of the C writers (engine and oracle)."""
    n = len(rec.qname)
    enc = [q.encode() for q in rec.qname]
    qoff = np.zeros(n + 1, np.int64)
    np.cumsum([len(x) for x in enc], out=qoff[1:])
    cig = np.concatenate([np.asarray(c, np.uint32) for c in rec.cigar] + [np.zeros(1, np.uint32)])
    coff = np.zeros(n + 1, np.int64)
    np.cumsum([len(c) for c in rec.cigar], out=coff[1:])
    seq = np.concatenate([np.asarray(s, np.uint8) for s in rec.seq] + [np.zeros(1, np.uint8)])
    soff = np.zeros(n + 1, np.int64)
    np.cumsum([len(s) for s in rec.seq], out=soff[1:])
    qb = [q.encode() for q in (rec.qual if rec.qual is not None else [""] * n)]
    quoff = np.zeros(n + 1, np.int64)
    np.cumsum([len(x) for x in qb], out=quoff[1:])
    cb = [c.encode() for c in rec.contigs]
    cnoff = np.zeros(len(cb) + 1, np.int64)
    np.cumsum([len(x) for x in cb], out=cnoff[1:])
    letters = np.zeros(32, np.uint8)
    letters[:len(rec.letters)] = np.frombuffer(rec.letters.encode(), np.uint8)
    tg = getattr(rec, "tags", None)
    tags, toff = None, None
    if tg is not None:
        toff = np.zeros(n + 1, np.int64)
        np.cumsum([len(x) for x in tg], out=toff[1:])
        tags = np.frombuffer(b"".join(bytes(x) for x in tg) + b"\0", np.uint8)
    return dict(tags=tags, toff=toff, qname=np.frombuffer(b"".join(enc) + b"\0", np.uint8), qoff=qoff,
                flag=np.ascontiguousarray(rec.flag, np.uint16), rid=np.ascontiguousarray(rec.ref_id, np.int32),
                pos=np.ascontiguousarray(rec.pos, np.int32), mapq=np.ascontiguousarray(rec.mapq, np.uint8),
                cigar=cig, coff=coff, rnext=np.ascontiguousarray(rec.next_ref_id, np.int32),
                pnext=np.ascontiguousarray(rec.next_pos, np.int32), tlen=np.ascontiguousarray(rec.tlen, np.int32),
                seq=seq, soff=soff, letters=letters, qual=np.frombuffer(b"".join(qb) + b"\0", np.uint8),
                quoff=quoff, cnames=np.frombuffer(b"".join(cb) + b"\0", np.uint8), cnoff=cnoff)


def oracle_write_sam_c(rec, threads: int = 0, arrays=None) -> str:
    """The C restatement of the SAM writer (OpenMP), for timing the CPU path."""
    lib = liboracle()
    lib.orc_write_sam.restype = C.c_int64
    a = arrays or sam_arrays(rec)
    n = len(rec.qname)
    args = [C.c_int64(n), _ptr(a["qname"]), _ptr(a["qoff"]), _ptr(a["flag"]), _ptr(a["rid"]), _ptr(a["pos"]),
            _ptr(a["mapq"]), _ptr(a["cigar"]), _ptr(a["coff"]), _ptr(a["rnext"]), _ptr(a["pnext"]), _ptr(a["tlen"]),
            _ptr(a["seq"]), _ptr(a["soff"]), _ptr(a["letters"]), _ptr(a["qual"]), _ptr(a["quoff"]),
            C.c_int64(len(rec.contigs)), _ptr(a["cnames"]), _ptr(a["cnoff"]), _ptr(a["tags"]), _ptr(a["toff"])]
    total = lib.orc_write_sam(*args, None, C.c_int64(0), C.c_int32(threads))
    if total < 0:
        raise ValueError("tags the restatement does not write")
    out = np.zeros(total + 1, np.uint8)
    lib.orc_write_sam(*args, _ptr(out), C.c_int64(total + 1), C.c_int32(threads))
    return bytes(out[:total]).decode()


_TAG_KEEP = []


def _tags_ptrs(rec, n):
    """(tags, offsets) pointers of rec.tags for the C writers, or (None, None)."""
    tg = getattr(rec, "tags", None)
    if tg is None:
        return None, None
    toff = np.zeros(n + 1, np.int64)
    np.cumsum([len(x) for x in tg], out=toff[1:])
    buf = np.frombuffer(b"".join(bytes(x) for x in tg) + b"\0", np.uint8)
    _TAG_KEEP[:] = [toff, buf]
    return _ptr(buf), _ptr(toff)


def ref_write_sam(rec) -> str:
    """The reference's SAM writer on the same records (oracle/ref/units/sam.cpp)."""
    lib = libref()
    lib.ref_write_sam.restype = C.c_int64
    n = len(rec.qname)
    enc = lambda parts: [p.encode() for p in parts]
    qn = enc(rec.qname)
    qoff = np.zeros(n + 1, np.int64)
    np.cumsum([len(x) for x in qn], out=qoff[1:])
    qname = b"".join(qn) or b"\0"
    cig = np.concatenate([np.asarray(c, np.uint32) for c in rec.cigar] + [np.zeros(1, np.uint32)])
    coff = np.zeros(n + 1, np.int64)
    np.cumsum([len(c) for c in rec.cigar], out=coff[1:])
    seqs = enc(["".join(rec.letters[int(x)] for x in s) for s in rec.seq])
    soff = np.zeros(n + 1, np.int64)
    np.cumsum([len(x) for x in seqs], out=soff[1:])
    quals = enc(rec.qual if rec.qual is not None else [""] * n)
    quoff = np.zeros(n + 1, np.int64)
    np.cumsum([len(x) for x in quals], out=quoff[1:])
    cn = enc(rec.contigs)
    cnoff = np.zeros(len(cn) + 1, np.int64)
    np.cumsum([len(x) for x in cn], out=cnoff[1:])
    arr = lambda a, t: np.ascontiguousarray(a, t)
    flag, rid, pos = arr(rec.flag, np.uint16), arr(rec.ref_id, np.int32), arr(rec.pos, np.int32)
    mapq, rn, pn, tl = arr(rec.mapq, np.uint8), arr(rec.next_ref_id, np.int32), arr(rec.next_pos, np.int32), \
        arr(rec.tlen, np.int32)
    tp, to = _tags_ptrs(rec, n)
    cap = 8 * sum(len(x) for x in (getattr(rec, "tags", None) or [])) + int(qoff[-1] + soff[-1] + quoff[-1] + 64 * n + 16 * int(coff[-1]) + 1024)
    out = C.create_string_buffer(cap)
    args = [C.c_int64(n), C.c_char_p(qname), _ptr(qoff), _ptr(flag), _ptr(rid), _ptr(pos), _ptr(mapq), _ptr(cig),
            _ptr(coff), _ptr(rn), _ptr(pn), _ptr(tl), C.c_char_p(b"".join(seqs) or b"\0"), _ptr(soff),
            C.c_char_p(b"".join(quals) or b"\0"), _ptr(quoff), C.c_int64(len(cn)), C.c_char_p(b"".join(cn) or b"\0"),
            _ptr(cnoff), tp, to, out, C.c_int64(cap)]
    length = lib.ref_write_sam(*args)
    return out.raw[:length].decode()


def render_rows(segments, h_text: str, v_text: str):
    """Gapped rows of the clipped alignment view, as operator<< on Gaps prints them."""
    if not segments:
        return "", ""
    hb, vb = segments[-1][0], segments[-1][1]
    rh, rv = [], []
    ch, cv = hb, vb
    for (_, _, ln, tp) in reversed(segments):
        if tp == SEG_DIAGONAL:
            rh.append(h_text[ch:ch + ln]); rv.append(v_text[cv:cv + ln]); ch += ln; cv += ln
        elif tp == SEG_VERTICAL:
            rh.append("-" * ln); rv.append(v_text[cv:cv + ln]); cv += ln
        else:
            rh.append(h_text[ch:ch + ln]); rv.append("-" * ln); ch += ln
    return "".join(rh), "".join(rv)


def segments_clip(segments):
    """(h_begin, h_end, v_begin, v_end) as clippedBegin/EndPosition report them after
    _adaptTraceSegmentsTo: the end is set to begin + the alignment's view length
    (align/dp_traceback_adaptor.h:114-115), for both rows."""
    if not segments:
        return (0, 0, 0, 0)
    hb, vb = segments[-1][0], segments[-1][1]
    view = sum(s[2] for s in segments)
    return (hb, hb + view, vb, vb + view)


def cigar_string(segments) -> str:
    ops = []
    for (_, _, ln, tp) in reversed(segments):
        op = "M" if tp == SEG_DIAGONAL else ("I" if tp == SEG_VERTICAL else "D")
        if ops and ops[-1][0] == op:
            ops[-1][1] += ln
        else:
            ops.append([op, ln])
    return "".join(f"{n}{'N' if (o == 'D' and n >= 20) else o}" for o, n in ops)


# --- FASTA / FASTQ records (seq_io/fasta_fastq.h readRecord loop) ------------------------------

SEQIO_ALPHABETS = {"dna": 4, "dna5": 5, "aa": 27}


class SeqParseError(Exception):
    """ParseError (kind "parse") or UnexpectedEnd (kind "end") at text offset `offset`."""

    def __init__(self, kind, offset):
        super().__init__(f"{kind} at {offset}")
        self.kind, self.offset = kind, offset


def oracle_read_records(text: bytes, fmt: str, alphabet: str = "dna5", raw: bool = False):
    """Records of FASTA ("fasta") or FASTQ ("fastq") text through the C restatement of the
    reference's readRecord loop: a list of (id bytes, residue codes uint8, quality bytes), or with
    raw the arrays (num, id_begin, id_end, seq_off, codes)."""
    lib = liboracle()
    lib.orc_read_records.restype = C.c_int32
    text = bytes(text)
    n = len(text)
    rec_cap = text.count(b"@" if fmt == "fastq" else b">") + 2
    res_cap = n + 1
    ib, ie, so, qe = (np.zeros(rec_cap, np.int64) for _ in range(4))
    codes = np.zeros(res_cap, np.uint8)
    quals = np.zeros(res_cap, np.uint8)
    num, res, err = C.c_int64(), C.c_int64(), C.c_int64()
    buf = C.create_string_buffer(text, n + 1)
    rc = lib.orc_read_records(C.c_int32(1 if fmt == "fastq" else 0), C.c_int32(SEQIO_ALPHABETS[alphabet]), buf,
                              C.c_int64(n), C.c_int64(rec_cap), _ptr(ib), _ptr(ie), _ptr(so), _ptr(qe),
                              C.c_int64(res_cap), _ptr(codes), _ptr(quals), C.byref(num), C.byref(res), C.byref(err))
    if rc == -1:
        raise SeqParseError("parse", err.value)
    if rc == -2:
        raise SeqParseError("end", err.value)
    assert rc == 0, rc
    if raw:
        k = num.value
        return k, ib[:k], ie[:k], so[:k + 1], codes[:res.value]
    out = []
    for k in range(num.value):
        out.append((text[ib[k]:ie[k]], codes[so[k]:so[k + 1]].copy(), bytes(quals[so[k]:qe[k]])))
    return out


def ref_read_records(text: bytes, fmt: str, alphabet: str = "dna5"):
    """The reference's readRecord loop on the same text (oracle/ref/units/seqio.cpp)."""
    lib = libref()
    lib.ref_read_records.restype = C.c_int64
    text = bytes(text)
    cap = 3 * len(text) + 64
    out = C.create_string_buffer(cap)
    nrec = C.c_int64()
    r = lib.ref_read_records(C.c_int32({"fasta": 0, "fastq": 1, "raw": 2}[fmt]), C.c_int32(SEQIO_ALPHABETS[alphabet]),
                             C.c_char_p(text), C.c_int64(len(text)), out, C.c_int64(cap), C.byref(nrec))
    if r == -1:
        raise SeqParseError("parse", None)
    if r == -2:
        raise SeqParseError("end", None)
    assert r >= 0, r
    raw, p, recs = out.raw[:r], 0, []
    while p < r:
        parts = []
        for _ in range(3):
            L = int.from_bytes(raw[p:p + 4], "little")
            parts.append(raw[p + 4:p + 4 + L])
            p += 4 + L
        recs.append((parts[0], np.frombuffer(parts[1], np.uint8).copy(), parts[2]))
    return recs


def ref_char_table(alphabet: str):
    """The reference's IsInAlphabet / conversion per character: code or -1."""
    lib = libref()
    t = np.zeros(256, np.int16)
    lib.ref_char_table(C.c_int32(SEQIO_ALPHABETS[alphabet]), _ptr(t))
    return t


# --- BAM records (bam_io/write_bam.h) ------------------------------------------------------------

def oracle_write_bam_c(rec, threads: int = 0, arrays=None) -> bytes:
    """The C restatement of the BAM record writer (OpenMP): the uncompressed record blocks."""
    lib = liboracle()
    lib.orc_write_bam.restype = C.c_int64
    a = arrays or sam_arrays(rec)
    n = len(rec.qname)
    args = [C.c_int64(n), _ptr(a["qname"]), _ptr(a["qoff"]), _ptr(a["flag"]), _ptr(a["rid"]), _ptr(a["pos"]),
            _ptr(a["mapq"]), _ptr(a["cigar"]), _ptr(a["coff"]), _ptr(a["rnext"]), _ptr(a["pnext"]), _ptr(a["tlen"]),
            _ptr(a["seq"]), _ptr(a["soff"]), _ptr(a["letters"]), _ptr(a["qual"]), _ptr(a["quoff"]),
            _ptr(a["tags"]), _ptr(a["toff"])]
    total = lib.orc_write_bam(*args, None, C.c_int64(0), C.c_int32(threads))
    out = np.zeros(total + 1, np.uint8)
    lib.orc_write_bam(*args, _ptr(out), C.c_int64(total + 1), C.c_int32(threads))
    return bytes(out[:total])


def ref_write_bam(rec) -> bytes:
    """The reference's BAM writer on the same records (oracle/ref/units/bam.cpp)."""
    lib = libref()
    lib.ref_write_bam.restype = C.c_int64
    n = len(rec.qname)
    enc = lambda parts: [p.encode("latin1") for p in parts]
    qn = enc(rec.qname)
    qoff = np.zeros(n + 1, np.int64)
    np.cumsum([len(x) for x in qn], out=qoff[1:])
    cig = np.concatenate([np.asarray(c, np.uint32) for c in rec.cigar] + [np.zeros(1, np.uint32)])
    coff = np.zeros(n + 1, np.int64)
    np.cumsum([len(c) for c in rec.cigar], out=coff[1:])
    seqs = enc(["".join(rec.letters[int(x)] for x in s) for s in rec.seq])
    soff = np.zeros(n + 1, np.int64)
    np.cumsum([len(x) for x in seqs], out=soff[1:])
    quals = enc(rec.qual if rec.qual is not None else [""] * n)
    quoff = np.zeros(n + 1, np.int64)
    np.cumsum([len(x) for x in quals], out=quoff[1:])
    cn = enc(rec.contigs)
    cnoff = np.zeros(len(cn) + 1, np.int64)
    np.cumsum([len(x) for x in cn], out=cnoff[1:])
    arr = lambda a, t: np.ascontiguousarray(a, t)
    flag, rid, pos = arr(rec.flag, np.uint16), arr(rec.ref_id, np.int32), arr(rec.pos, np.int32)
    mapq, rn, pn, tl = arr(rec.mapq, np.uint8), arr(rec.next_ref_id, np.int32), arr(rec.next_pos, np.int32), \
        arr(rec.tlen, np.int32)
    tp, to = _tags_ptrs(rec, n)
    cap = 8 * sum(len(x) for x in (getattr(rec, "tags", None) or [])) + int(qoff[-1] + 2 * soff[-1] + quoff[-1] + 40 * n + 4 * int(coff[-1]) + 64)
    out = C.create_string_buffer(cap)
    args = [C.c_int64(n), C.c_char_p(b"".join(qn) or b"\0"), _ptr(qoff), _ptr(flag), _ptr(rid), _ptr(pos),
            _ptr(mapq), _ptr(cig), _ptr(coff), _ptr(rn), _ptr(pn), _ptr(tl), C.c_char_p(b"".join(seqs) or b"\0"),
            _ptr(soff), C.c_char_p(b"".join(quals) or b"\0"), _ptr(quoff), C.c_int64(len(cn)),
            C.c_char_p(b"".join(cn) or b"\0"), _ptr(cnoff), tp, to, out, C.c_int64(cap)]
    length = lib.ref_write_bam(*args)
    assert length <= cap
    return out.raw[:length]


def ref_iupac_table():
    """ordValue(Iupac(c)) of the reference for each of the 256 characters."""
    lib = libref()
    t = np.zeros(256, np.uint8)
    lib.ref_iupac_table(_ptr(t))
    return t


# ---------------------------------------------------------------------------------------------
# Banded chain alignment (seeds/banded_chain_alignment.h:184-214).
# ---------------------------------------------------------------------------------------------

class OrcSimpleScore(C.Structure):
    _fields_ = [("match", C.c_int32), ("mismatch", C.c_int32), ("gap_extend", C.c_int32), ("gap_open", C.c_int32)]


class OrcChainParams(C.Structure):
    _fields_ = [("anchor", OrcSimpleScore), ("gap", OrcSimpleScore), ("free_ends", C.c_int32),
                ("band_extension", C.c_int32)]


@dataclass
class ChainResult:
    status: int            # 0 ok, 1 the reference throws (no glue point), 2 undefined in the reference
    score: int
    segments: list         # TraceSegment_ runs (h, v, length, type) in the reference's order
    n_traces: int
    rows: tuple | None = None


def _chain_seeds(seeds):
    return np.ascontiguousarray(np.asarray(seeds, dtype=np.int32).reshape(-1, 4))


def oracle_banded_chain(h, v, seeds, anchor, gap=None, free_ends=0, k=15) -> ChainResult:
    """The restatement (oracle/banded_chain_oracle.c).  anchor / gap: (match, mismatch, gap_extend,
    gap_open); seeds: (beginH, beginV, endH, endV) per seed in chain order."""
    lib = liboracle()
    lib.orc_banded_chain.argtypes = [C.POINTER(OrcChainParams), C.c_void_p, C.c_int32, C.c_void_p, C.c_int32,
                                     C.c_int32, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int32, C.c_void_p,
                                     C.c_void_p]
    gap = gap or anchor
    p = OrcChainParams(OrcSimpleScore(*anchor), OrcSimpleScore(*gap), free_ends, k)
    h = np.ascontiguousarray(h, dtype=np.uint8)
    v = np.ascontiguousarray(v, dtype=np.uint8)
    sd = _chain_seeds(seeds)
    cap = 4 * (len(h) + len(v)) + 64
    segs = np.zeros((cap, 4), np.uint32)
    out = np.zeros(3, np.int32)
    rc = lib.orc_banded_chain(C.byref(p), _ptr(h), len(h), _ptr(v), len(v), len(sd), _ptr(sd), _ptr(out[0:]),
                              _ptr(segs), cap, _ptr(out[1:]), _ptr(out[2:]))
    if rc < 0:
        raise RuntimeError("segment buffer too small")
    return ChainResult(int(rc), int(out[0]), [tuple(int(x) for x in s) for s in segs[:out[1]]], int(out[2]))


def ref_banded_chain(h, v, seeds, anchor, gap=None, free_ends=0, k=15, lib=None) -> ChainResult:
    """The reference's bandedChainAlignment (oracle/ref/units/banded_chain.cpp): score, the first
    trace of its trace set, the number of traces and the Align rows it prints."""
    lib = lib or libref()
    lib.ref_banded_chain.argtypes = [C.c_void_p, C.c_void_p, C.c_int32, C.c_int32, C.c_void_p, C.c_int64,
                                     C.c_void_p, C.c_int64, C.c_int32, C.c_void_p, C.c_void_p, C.c_void_p,
                                     C.c_int32, C.c_void_p, C.c_void_p, C.c_char_p, C.c_int64]
    gap = gap or anchor
    a = np.asarray(anchor, np.int32)
    g = np.asarray(gap, np.int32)
    h = np.ascontiguousarray(h, dtype=np.uint8)
    v = np.ascontiguousarray(v, dtype=np.uint8)
    sd = _chain_seeds(seeds)
    cap = 4 * (len(h) + len(v)) + 64
    segs = np.zeros((cap, 4), np.uint32)
    out = np.zeros(3, np.int32)
    tcap = 4 * (len(h) + len(v)) + 16
    rows = C.create_string_buffer(tcap)
    rc = lib.ref_banded_chain(_ptr(a), _ptr(g), free_ends, k, _ptr(h), len(h), _ptr(v), len(v), len(sd), _ptr(sd),
                              _ptr(out[0:]), _ptr(segs), cap, _ptr(out[1:]), _ptr(out[2:]), rows, tcap)
    if rc < 0:
        raise RuntimeError(f"ref_banded_chain failed ({rc})")
    r = rows.value.decode().split("\n")
    return ChainResult(int(rc), int(out[0]), [tuple(int(x) for x in s) for s in segs[:out[1]]], int(out[2]),
                       (r[0], r[1]) if rc == 0 else None)
