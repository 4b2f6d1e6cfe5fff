"""Host-side mirror of SeqAn 2's batch alignment interface over the GB300 engine.

The functions keep the reference's names, argument order and meaning:

* ``globalAlignmentScore(setH, setV, score, config=AlignConfig(), lower=None, upper=None)``
  -- align_parallel/parallel_align_interface.h:330-340, align/global_alignment_unbanded.h:739-821,
  banded align/global_alignment_banded.h:558-652.
* ``localAlignmentScore(setH, setV, score, lower=None, upper=None)``
  -- align/local_alignment_unbanded.h:554-572, align/local_alignment_banded.h:252.
* ``globalAlignment(gapsH, gapsV, score, config, lower, upper)`` and ``localAlignment(...)``
  over lists of :class:`Gaps` (overwritten in place, scores returned) --
  align/global_alignment_unbanded.h:831-888, align/local_alignment_unbanded.h:367-399.
* ``getCigarString(gapsRef, gapsRead)`` -- bam_io/cigar.h:261-339.

An optional ``execution_policy`` first argument is accepted (and ignored: the whole batch runs
on the GPU), as the reference's ``ExecutionPolicy<Parallel, Vectorial>`` overloads take one.
Like the reference, invalid pairs (empty sequence, band outside the matrix) score
``numeric_limits<T>::min()``.  Every call goes through the C-ABI; nothing runs on the CPU.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

from . import _native as N
from .alphabet import encode
from .scoring import Blosum62, Score  # noqa: F401  (re-exported)


@dataclass(frozen=True)
class AlignConfig:
    """AlignConfig<TOP, LEFT, RIGHT, BOTTOM> (align/align_config.h:52-94)."""
    top: bool = False
    left: bool = False
    right: bool = False
    bottom: bool = False

    @property
    def bits(self) -> int:
        return (N.GBA_FREE_TOP if self.top else 0) | (N.GBA_FREE_LEFT if self.left else 0) | \
            (N.GBA_FREE_RIGHT if self.right else 0) | (N.GBA_FREE_BOTTOM if self.bottom else 0)


class ExecutionPolicy:
    """Accepted for call-surface parity with ExecutionPolicy<Parallel, Vectorial>."""

    def __init__(self, parallel: str = "Parallel", vectorial: str = "Vectorial", threads: int = 1):
        self.parallel, self.vectorial, self.threads = parallel, vectorial, threads


class Gaps:
    """A gapped view of one sequence, filled by globalAlignment/localAlignment.

    Holds the clipped begin/end (source positions) and the gapped row, like
    Gaps<String<T>, ArrayGaps> after _adaptTraceSegmentsTo (align/dp_traceback_adaptor.h:57-117).
    """

    def __init__(self, source, alphabet: str = "dna5"):
        self.text = source if isinstance(source, str) else None
        self.codes = encode(source, alphabet)
        self.alphabet = alphabet
        self.clipped_begin = 0
        self.clipped_end = len(self.codes)
        self.gap_runs: list[tuple[int, int]] = []   # (view position, length)
        self.segments = []                          # the pair's TraceSegment_ list

    def __len__(self):
        return self.clipped_end - self.clipped_begin + sum(l for _, l in self.gap_runs)

    def row(self) -> str:
        """The gapped row as operator<< prints it (clipped part, '-' for gaps)."""
        txt = self.text if self.text is not None else _decode(self.codes, self.alphabet)
        out = []
        src = self.clipped_begin
        view = 0
        for pos, ln in self.gap_runs:
            take = pos - view
            out.append(txt[src:src + take]); src += take; view += take
            out.append("-" * ln); view += ln
        out.append(txt[src:self.clipped_end])
        return "".join(out)

    def __str__(self):
        return self.row()


def _decode(codes, alphabet):
    from .alphabet import decode
    return decode(codes, alphabet)


def _split_policy(args):
    if args and isinstance(args[0], ExecutionPolicy):
        return args[1:]
    return args


def _as_codes(seqs, alphabet):
    return [encode(s, alphabet) for s in seqs]


def _concat(codes):
    lens = np.fromiter((len(c) for c in codes), dtype=np.int64, count=len(codes))
    off = np.zeros(len(codes) + 1, dtype=np.int64)
    np.cumsum(lens, out=off[1:])
    flat = np.concatenate(codes).astype(np.uint8, copy=False) if off[-1] else np.zeros(1, np.uint8)
    return np.ascontiguousarray(flat), off


def _vp(a):
    return a.ctypes.data_as(C.c_void_p) if a is not None else None


def make_params(score, mode: int, config: AlignConfig | None, band, outputs: int,
                alphabet_size: int = 0, flags: int = 0, gaps: int = N.GBA_GAPS_AUTO) -> N.GbaParams:
    p = N.GbaParams()
    p.mode = mode
    p.gap_model = gaps
    p.free_ends = config.bits if (config is not None and mode == N.GBA_GLOBAL) else 0
    if band is not None:
        p.band_on, p.band_lower, p.band_upper = 1, int(band[0]), int(band[1])
    p.match, p.mismatch = score.match, score.mismatch
    p.gap_open, p.gap_extend = score.gap_open, score.gap_extend
    p.alphabet_size = alphabet_size
    if score.matrix is not None:
        p.matrix = score.matrix.ctypes.data_as(C.c_void_p)
        p.alphabet_size = score.matrix.shape[0]
    p.score_bits = score.bits
    p.outputs = outputs
    p.flags = flags
    return p


@dataclass
class BatchOutput:
    score: np.ndarray
    end_h: np.ndarray
    end_v: np.ndarray
    status: np.ndarray
    begin_h: np.ndarray | None = None
    begin_v: np.ndarray | None = None
    segments: np.ndarray | None = None         # [total, 4] uint32
    segment_offsets: np.ndarray | None = None  # [n+1]
    cigar: np.ndarray | None = None            # [total] uint32 (len << 4 | op)
    cigar_offsets: np.ndarray | None = None

    def pair_segments(self, k):
        s = self.segments[self.segment_offsets[k]:self.segment_offsets[k + 1]]
        return [tuple(int(x) for x in row) for row in s]

    def pair_cigar(self, k) -> str:
        ops = "MIDNSHP=X"
        c = self.cigar[self.cigar_offsets[k]:self.cigar_offsets[k + 1]]
        return "".join(f"{int(x) >> 4}{ops[int(x) & 15]}" for x in c)


ALPHABET_SIZE = {"dna": 4, "dna5": 5, "aa": 27}


def align_codes(codes_h, codes_v, score, mode=N.GBA_GLOBAL, config=None, band=None,
                traceback=False, cigar=False, h_shared=False, ctx: N.Context | None = None,
                alphabet_size: int | None = None, flags: int = 0, packed_bits: int | None = None,
                fasta_texts=None, tile_variant: int = 0, gaps: int = N.GBA_GAPS_AUTO) -> BatchOutput:
    """Aligns lists of code arrays through gba_align_batch.

    alphabet_size bounds the codes (the reference's ValueSize of the alphabet); when None it is
    taken from the codes themselves.  packed_bits (2 Dna, 3 Dna5, 5 AminoAcid) sends the sequences
    as String<TValue, Packed<>> host words through gba_align_packed instead.  gaps selects the gap
    cost model (N.GBA_GAPS_DYNAMIC: the reference's DynamicGaps cells)."""
    ctx = ctx or N.default_context()
    n = len(codes_v)
    sh, oh = _concat(codes_h)
    sv, ov = _concat(codes_v)
    outputs = N.GBA_OUT_SCORE | N.GBA_OUT_END
    if traceback:
        outputs |= N.GBA_OUT_SEGMENTS
    if cigar:
        outputs |= N.GBA_OUT_CIGAR | N.GBA_OUT_SEGMENTS
    if alphabet_size is None:
        alphabet_size = int(max(sh.max(initial=0), sv.max(initial=0))) + 1 if n else 0
    params = make_params(score, mode, config, band, outputs, alphabet_size, flags, gaps)
    params.tile_variant = tile_variant
    b = N.GbaBatch(n, _vp(sh), _vp(oh), _vp(sv), _vp(ov), 1 if h_shared else 0, 0)
    res = BatchOutput(score=np.zeros(n, np.int32), end_h=np.zeros(n, np.int32), end_v=np.zeros(n, np.int32),
                      status=np.zeros(n, np.int32))
    r = N.GbaResult()
    r.score, r.end_h, r.end_v, r.pair_status = _vp(res.score), _vp(res.end_h), _vp(res.end_v), _vp(res.status)
    if traceback or cigar:
        lh = np.full(n, oh[1] - oh[0], np.int64) if h_shared else (oh[1:] - oh[:-1])
        cap = int((lh + (ov[1:] - ov[:-1]) + 4).sum()) + 1
        res.begin_h, res.begin_v = np.zeros(n, np.int32), np.zeros(n, np.int32)
        res.segments = np.zeros((cap, 4), np.uint32)
        res.segment_offsets = np.zeros(n + 1, np.int64)
        r.begin_h, r.begin_v = _vp(res.begin_h), _vp(res.begin_v)
        r.segments, r.segment_capacity, r.segment_offsets = _vp(res.segments), cap, _vp(res.segment_offsets)
        if cigar:
            res.cigar = np.zeros(cap, np.uint32)
            res.cigar_offsets = np.zeros(n + 1, np.int64)
            r.cigar, r.cigar_capacity, r.cigar_offsets = _vp(res.cigar), cap, _vp(res.cigar_offsets)
    if fasta_texts is not None:
        th, tv, alph = fasta_texts
        bh, bv = np.frombuffer(bytes(th) or b"\0", np.uint8), np.frombuffer(bytes(tv) or b"\0", np.uint8)
        npairs = C.c_int64()
        ctx.check(N.lib().gba_align_fasta(ctx.handle, C.byref(params), _vp(bh), len(th), _vp(bv), len(tv), alph,
                                          1 if h_shared else 0, n, C.byref(npairs), C.byref(r)), "gba_align_fasta")
        return res
    if packed_bits:
        from . import packed as P
        hw, hoff = P.pack_set(codes_h[:1] if h_shared else codes_h, packed_bits)
        vw, voff = P.pack_set(codes_v, packed_bits)
        ph = N.GbaPackedSet(len(hoff) - 1, _vp(hw), _vp(hoff), packed_bits, 0)
        pv = N.GbaPackedSet(len(voff) - 1, _vp(vw), _vp(voff), packed_bits, 0)
        ctx.check(N.lib().gba_align_packed(ctx.handle, C.byref(params), C.byref(ph), C.byref(pv),
                                           1 if h_shared else 0, C.byref(r)), "gba_align_packed")
        return res
    ctx.check(N.lib().gba_align_batch(ctx.handle, C.byref(params), C.byref(b), C.byref(r)), "gba_align_batch")
    return res


def align_codes_resident(codes_h, codes_v, score, mode=N.GBA_GLOBAL, config=None, band=None, traceback=False,
                         cigar=False, alphabet_size: int | None = None, flags: int = 0, tile_variant: int = 0,
                         runs: int = 2, ctx: N.Context | None = None) -> BatchOutput:
    """align_codes on the device-resident path: the codes are copied to HBM once, a plan is built
    from the host offsets (gba_plan_create) and run `runs` times on the device buffers
    (gba_plan_execute; from the second run on, a CUDA-graph replay unless GBA_FLAG_NO_GRAPH), and
    the last run's results are copied back (gba_plan_fetch for segments and CIGARs)."""
    ctx = ctx or N.default_context()
    L = N.lib()
    h = ctx.handle
    n = len(codes_v)
    sh, oh = _concat(codes_h)
    sv, ov = _concat(codes_v)
    outputs = N.GBA_OUT_SCORE | N.GBA_OUT_END
    if traceback or cigar:
        outputs |= N.GBA_OUT_SEGMENTS
    if cigar:
        outputs |= N.GBA_OUT_CIGAR
    if alphabet_size is None:
        alphabet_size = int(max(sh.max(initial=0), sv.max(initial=0))) + 1 if n else 0
    params = make_params(score, mode, config, band, outputs, alphabet_size, flags)
    params.tile_variant = tile_variant
    host_batch = N.GbaBatch(n, _vp(sh), _vp(oh), _vp(sv), _vp(ov), 0, 0)
    bufs = []

    def dev(nbytes):
        ptr = C.c_void_p()
        ctx.check(L.gba_device_alloc(h, C.byref(ptr), max(int(nbytes), 16)), "gba_device_alloc")
        bufs.append(ptr)
        return ptr

    plan = C.c_void_p()
    try:
        d_sh, d_sv = dev(sh.nbytes), dev(sv.nbytes)
        ctx.check(L.gba_copy_to_device(h, d_sh, _vp(sh), sh.nbytes), "copy")
        ctx.check(L.gba_copy_to_device(h, d_sv, _vp(sv), sv.nbytes), "copy")
        d_score, d_eh, d_ev = dev(4 * n), dev(4 * n), dev(4 * n)
        ctx.check(L.gba_plan_create(h, C.byref(params), C.byref(host_batch), C.byref(plan)), "gba_plan_create")
        dev_batch = N.GbaBatch(n, d_sh, None, d_sv, None, 0, 0)
        dres = N.GbaResult()
        dres.score, dres.end_h, dres.end_v = d_score, d_eh, d_ev
        for _ in range(max(1, runs)):
            ctx.check(L.gba_plan_execute(h, plan, C.byref(dev_batch), C.byref(dres)), "gba_plan_execute")
        ctx.check(L.gba_synchronize(h), "gba_synchronize")
        res = BatchOutput(score=np.zeros(n, np.int32), end_h=np.zeros(n, np.int32), end_v=np.zeros(n, np.int32),
                          status=np.zeros(n, np.int32))
        for arr, ptr in ((res.score, d_score), (res.end_h, d_eh), (res.end_v, d_ev)):
            ctx.check(L.gba_copy_to_host(h, _vp(arr), ptr, 4 * n), "copy")
        if traceback or cigar:
            cap = int(((oh[1:] - oh[:-1]) + (ov[1:] - ov[:-1]) + 4).sum()) + 1
            res.begin_h, res.begin_v = np.zeros(n, np.int32), np.zeros(n, np.int32)
            res.segments = np.zeros((cap, 4), np.uint32)
            res.segment_offsets = np.zeros(n + 1, np.int64)
            r = N.GbaResult()
            r.begin_h, r.begin_v = _vp(res.begin_h), _vp(res.begin_v)
            r.segments, r.segment_capacity, r.segment_offsets = _vp(res.segments), cap, _vp(res.segment_offsets)
            if cigar:
                res.cigar = np.zeros(cap, np.uint32)
                res.cigar_offsets = np.zeros(n + 1, np.int64)
                r.cigar, r.cigar_capacity, r.cigar_offsets = _vp(res.cigar), cap, _vp(res.cigar_offsets)
            ctx.check(L.gba_plan_fetch(h, plan, C.byref(r)), "gba_plan_fetch")
        return res
    finally:
        if plan:
            L.gba_plan_destroy(h, plan)
        for ptr in bufs:
            L.gba_device_free(h, ptr)


def _band(args):
    if len(args) >= 2 and args[0] is not None:
        return (int(args[0]), int(args[1]))
    return None


def globalAlignmentScore(*args, alphabet: str = "dna5", **kw):
    """globalAlignmentScore([policy,] setH, setV, score[, config][, lower, upper]) -> scores."""
    args = _split_policy(args)
    setH, setV, score = args[0], args[1], args[2]
    rest = list(args[3:])
    config = rest.pop(0) if rest and isinstance(rest[0], AlignConfig) else kw.get("config", AlignConfig())
    band = _band(rest) or kw.get("band")
    h_shared = not isinstance(setH, (list, tuple))
    codes_h = [encode(setH, alphabet)] if h_shared else _as_codes(setH, alphabet)
    out = align_codes(codes_h, _as_codes(setV, alphabet), score, N.GBA_GLOBAL, config, band, h_shared=h_shared,
                      alphabet_size=ALPHABET_SIZE[alphabet])
    return out.score.astype(score.dtype)


def localAlignmentScore(*args, alphabet: str = "dna5", **kw):
    """localAlignmentScore([policy,] setH, setV, score[, lower, upper]) -> scores."""
    args = _split_policy(args)
    setH, setV, score = args[0], args[1], args[2]
    band = _band(list(args[3:])) or kw.get("band")
    h_shared = not isinstance(setH, (list, tuple))
    codes_h = [encode(setH, alphabet)] if h_shared else _as_codes(setH, alphabet)
    out = align_codes(codes_h, _as_codes(setV, alphabet), score, N.GBA_LOCAL, None, band, h_shared=h_shared,
                      alphabet_size=ALPHABET_SIZE[alphabet])
    return out.score.astype(score.dtype)


def _apply_segments(gH: Gaps, gV: Gaps, segs):
    """_adaptTraceSegmentsTo (align/dp_traceback_adaptor.h:57-117)."""
    gH.segments = gV.segments = segs
    gH.gap_runs, gV.gap_runs = [], []
    if not segs:
        gH.clipped_begin = gH.clipped_end = gV.clipped_begin = gV.clipped_end = 0
        return
    hb, vb = segs[-1][0], segs[-1][1]
    view = 0
    ch, cv = hb, vb
    for (_, _, ln, tp) in reversed(segs):
        if tp == N.GBA_SEG_HORIZONTAL:
            _add_run(gV.gap_runs, view, ln); ch += ln
        elif tp == N.GBA_SEG_VERTICAL:
            _add_run(gH.gap_runs, view, ln); cv += ln
        else:
            ch += ln; cv += ln
        view += ln
    gH.clipped_begin, gH.clipped_end = hb, ch
    gV.clipped_begin, gV.clipped_end = vb, cv


def _add_run(runs, pos, ln):
    if runs and runs[-1][0] + runs[-1][1] == pos:
        runs[-1] = (runs[-1][0], runs[-1][1] + ln)
    else:
        runs.append((pos, ln))


def _align_gaps(mode, args, kw):
    args = _split_policy(args)
    gapsH, gapsV, score = args[0], args[1], args[2]
    rest = list(args[3:])
    config = rest.pop(0) if rest and isinstance(rest[0], AlignConfig) else kw.get("config", AlignConfig())
    band = _band(rest) or kw.get("band")
    out = align_codes([g.codes for g in gapsH], [g.codes for g in gapsV], score, mode,
                      config if mode == N.GBA_GLOBAL else None, band, traceback=True)
    for k, (gH, gV) in enumerate(zip(gapsH, gapsV)):
        _apply_segments(gH, gV, out.pair_segments(k))
    return out.score.astype(score.dtype)


def globalAlignment(*args, **kw):
    """globalAlignment([policy,] gapsH, gapsV, score[, config][, lower, upper]) -> scores."""
    return _align_gaps(N.GBA_GLOBAL, args, kw)


def localAlignment(*args, **kw):
    """localAlignment([policy,] gapsH, gapsV, score[, lower, upper]) -> scores."""
    return _align_gaps(N.GBA_LOCAL, args, kw)


def getCigarString(gapsRef: Gaps, gapsRead: Gaps, spliced_gap_thresh: int = 20) -> str:
    """CIGAR of an aligned pair (bam_io/cigar.h:261-339): M/I/D, D runs >= thresh as N."""
    ops = []
    for (_, _, ln, tp) in reversed(gapsRef.segments):
        op = "M" if tp == N.GBA_SEG_DIAGONAL else ("I" if tp == N.GBA_SEG_VERTICAL else "D")
        if ops and ops[-1][0] == op:
            ops[-1][1] += ln
        else:
            ops.append([op, ln])
    return "".join(f"{n}{'N' if (o == 'D' and n >= spliced_gap_thresh) else o}" for o, n in ops)


def align_fasta(text_h: bytes, text_v: bytes, score, alphabet: str = "dna5", **kw) -> BatchOutput:
    """Aligns the records of two FASTA texts pairwise (record k of text_h with record k of text_v,
    or the single record of text_h with every record of text_v when h_shared) through
    gba_align_fasta: both texts are parsed on the device and aligned from the codes left there.
    The records are read once more here, only to size the result arrays."""
    from . import seq_io as S
    codes_h, codes_v = S.read_fasta(text_h, alphabet).seqs, S.read_fasta(text_v, alphabet).seqs
    kw.setdefault("alphabet_size", S.ALPHABETS[alphabet])
    return align_codes(codes_h, codes_v, score, fasta_texts=(text_h, text_v, S.ALPHABETS[alphabet]), **kw)
