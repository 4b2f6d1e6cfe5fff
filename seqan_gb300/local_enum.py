"""Waterman-Eggert suboptimal local alignments with the reference's call surface
(align/local_alignment_enumeration_unbanded.h, align/local_alignment_enumeration_banded.h).

:func:`local_enumerate` runs the enumeration for a batch of pairs in one GPU call
(``gba_local_enumerate``): per pair, up to ``max_count`` alignments, each with the enumerator's
score (getScore), the gapped rows as the reference prints them, the clipped source positions and
the alignment's columns as runs.  :class:`LocalAlignmentEnumerator` with :func:`nextLocalAlignment`
is the reference's stateful form for one pair: each call gives the next alignment or False.
With ``band=(lowerDiag, upperDiag)`` both run LocalAlignmentEnumerator<Score, Banded>
(``gba_local_enumerate_banded``).
Linear gaps only, as the reference's Waterman-Eggert is: every gap column costs the scheme's gap
extension score.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _native as N
from .alphabet import decode, encode


class LocalAlignment:
    """One suboptimal local alignment: the enumerator's score, the clipped source positions and
    the alignment's columns as runs (h, v, length, type) in alignment order.  The two gapped rows
    (``row0`` / ``row1``, as the reference prints them) are rendered on first access."""
    __slots__ = ("score", "h_begin", "h_end", "v_begin", "v_end", "segments", "_texts", "_rows")

    def __init__(self, score, h_begin, h_end, v_begin, v_end, segments, texts):
        self.score, self.h_begin, self.h_end, self.v_begin, self.v_end = score, h_begin, h_end, v_begin, v_end
        self.segments = segments
        self._texts = texts          # (H text, V text) or a callable giving them
        self._rows = None

    def _render(self):
        if self._rows is None:
            t = self._texts() if callable(self._texts) else self._texts
            self._rows = _rows(self.segments, t[0], t[1])
        return self._rows

    @property
    def row0(self):
        return self._render()[0]

    @property
    def row1(self):
        return self._render()[1]

    def __repr__(self):
        return (f"LocalAlignment(score={self.score}, h=[{self.h_begin},{self.h_end}), "
                f"v=[{self.v_begin},{self.v_end}), segments={len(self.segments)})")


class PairEnumeration:
    """The enumeration of one pair.  ``alignments`` is built from the call's output arrays on first
    access; ``undefined_next``: stopped where the reference's next step is undefined."""

    def __init__(self, batch, k, undefined_next=False):
        self._batch, self._k, self.undefined_next = batch, k, undefined_next
        self._alignments = None

    @property
    def alignments(self):
        if self._alignments is None:
            self._alignments = self._batch.alignments_of(self._k)
        return self._alignments


def _rows(segments, h_text, v_text):
    r0, r1 = [], []
    for hb, vb, ln, tp in segments:
        if tp == N.GBA_SEG_DIAGONAL:
            r0.append(h_text[hb:hb + ln]); r1.append(v_text[vb:vb + ln])
        elif tp == N.GBA_SEG_HORIZONTAL:
            r0.append(h_text[hb:hb + ln]); r1.append("-" * ln)
        else:
            r0.append("-" * ln); r1.append(v_text[vb:vb + ln])
    # each row's clipped region runs from its first to its last residue
    return "".join(r0).strip("-"), "".join(r1).strip("-")


def local_enumerate(H, V, score, cutoff: int = 0, max_count: int = 25, alphabet: str = "dna5",
                    context=None, band=None) -> list:
    """One GPU call: up to max_count Waterman-Eggert alignments per pair (H[k], V[k]); band =
    (lowerDiag, upperDiag) for the banded enumerator."""
    ch = [np.ascontiguousarray(encode(s, alphabet), dtype=np.uint8) for s in H]
    cv = [np.ascontiguousarray(encode(s, alphabet), dtype=np.uint8) for s in V]
    n = len(ch)
    oh = np.zeros(n + 1, np.int64)
    ov = np.zeros(n + 1, np.int64)
    np.cumsum([len(c) for c in ch], out=oh[1:])
    np.cumsum([len(c) for c in cv], out=ov[1:])
    sh = np.concatenate(ch + [np.zeros(1, np.uint8)])
    sv = np.concatenate(cv + [np.zeros(1, np.uint8)])
    p = N.GbaEnumParams()
    p.match, p.mismatch, p.gap, p.cutoff, p.max_count = score.match, score.mismatch, score.gap_extend, cutoff, max_count
    keep = None
    if score.matrix is not None:
        keep = np.ascontiguousarray(score.matrix, dtype=np.int32)
        p.matrix = keep.ctypes.data
        p.alphabet_size = int(round(np.sqrt(keep.size)))
    b = N.GbaBatch(n, sh.ctypes.data, oh.ctypes.data, sv.ctypes.data, ov.ctypes.data, 0, 0)
    na = max(n * max_count, 1)
    count = np.zeros(max(n, 1), np.int32)
    status = np.zeros(max(n, 1), np.int32)
    arrs = [np.zeros(na, np.int32) for _ in range(5)]
    cap = int(sum(max_count * (len(a) + len(c) + 1) for a, c in zip(ch, cv))) + 8
    segs = np.zeros((cap, 4), np.uint32)
    off = np.zeros(na + 1, np.int64)
    r = N.GbaEnumResult(count.ctypes.data, status.ctypes.data, *[a.ctypes.data for a in arrs], segs.ctypes.data,
                        cap, off.ctypes.data)
    ctx = context or N.default_context()
    if band is None:
        ctx.check(N.lib().gba_local_enumerate(ctx.handle, C.byref(p), C.byref(b), C.byref(r)), "gba_local_enumerate")
    else:
        ctx.check(N.lib().gba_local_enumerate_banded(ctx.handle, C.byref(p), int(band[0]), int(band[1]), C.byref(b),
                                                     C.byref(r)), "gba_local_enumerate_banded")
    del keep
    out = _Batch(ch, cv, alphabet, max_count, count, arrs, segs, off)
    return [PairEnumeration(out, k, int(status[k]) == N.GBA_ENUM_UNDEFINED_NEXT) for k in range(n)]


class _Batch:
    """Output arrays of one gba_local_enumerate call, turned into LocalAlignment objects per pair on
    demand."""

    def __init__(self, ch, cv, alphabet, max_count, count, arrs, segs, off):
        self.ch, self.cv, self.alphabet, self.max_count = ch, cv, alphabet, max_count
        self.count, self.arrs, self.segs, self.off = count, arrs, segs, off

    def alignments_of(self, k):
        sc, bh, eh, bv, ev = self.arrs
        texts = _Texts(self, k)
        als = []
        for i in range(int(self.count[k])):
            g = k * self.max_count + i
            sg = [tuple(x) for x in self.segs[self.off[g]:self.off[g + 1]].tolist()]
            als.append(LocalAlignment(int(sc[g]), int(bh[g]), int(eh[g]), int(bv[g]), int(ev[g]), sg, texts))
        return als


class _Texts:
    """The decoded texts of pair k, decoded once for all its alignments."""

    def __init__(self, batch, k):
        self.batch, self.k, self.t = batch, k, None

    def __call__(self):
        if self.t is None:
            b = self.batch
            self.t = (decode(b.ch[self.k], b.alphabet), decode(b.cv[self.k], b.alphabet))
        return self.t


class LocalAlignmentEnumerator:
    """LocalAlignmentEnumerator<Score, Unbanded>(score[, cutoff]) for one pair of sequences, or
    LocalAlignmentEnumerator<Score, Banded>(score, lowerDiag, upperDiag[, cutoff]) when both
    diagonals are given."""

    def __init__(self, score, *args, alphabet: str = "dna5", context=None):
        if len(args) >= 2:
            self.band, self.cutoff = (int(args[0]), int(args[1])), int(args[2]) if len(args) > 2 else 0
        else:
            self.band, self.cutoff = None, int(args[0]) if args else 0
        self.score_scheme, self.alphabet, self.context = score, alphabet, context
        self._pair = None
        self._done = []
        self._next = 0
        self._exhausted = False
        self.current = None

    def _fill(self, h, v, want):
        e = local_enumerate([h], [v], self.score_scheme, self.cutoff, want, self.alphabet, self.context,
                            band=self.band)[0]
        self._done = e.alignments
        self._exhausted = len(e.alignments) < want

    def next(self, h, v):
        key = (bytes(encode(h, self.alphabet)), bytes(encode(v, self.alphabet)))
        if key != self._pair:
            self._pair, self._next = key, 0
            self._fill(h, v, 32)
        if self._next >= len(self._done) and not self._exhausted:
            self._fill(h, v, 4 * len(self._done))   # the enumeration is deterministic: redo it longer
        if self._next >= len(self._done):
            self.current = None
            return None
        self.current = self._done[self._next]
        self._next += 1
        return self.current

    def getScore(self):
        return self.current.score if self.current else 0


def nextLocalAlignment(h, v, enumerator: LocalAlignmentEnumerator):
    """The next suboptimal local alignment of (h, v), or None once the enumeration ends (the
    reference returns false)."""
    return enumerator.next(h, v)
