"""Waterman-Eggert suboptimal local alignments with the reference's call surface
(align/local_alignment_enumeration_unbanded.h).

:func:`local_enumerate` runs the enumeration for a batch of pairs in one GPU call
(``gba_local_enumerate``): per pair, up to ``max_count`` alignments, each with the enumerator's
score (getScore), the gapped rows as the reference prints them, the clipped source positions and
the alignment's columns as runs.  :class:`LocalAlignmentEnumerator` with :func:`nextLocalAlignment`
is the reference's stateful form for one pair: each call gives the next alignment or False.
Linear gaps only, as the reference's Waterman-Eggert is: every gap column costs the scheme's gap
extension score.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field

import numpy as np

from . import _native as N
from .alphabet import decode, encode


@dataclass
class LocalAlignment:
    score: int
    row0: str
    row1: str
    h_begin: int
    h_end: int
    v_begin: int
    v_end: int
    segments: list = field(default_factory=list)   # runs in alignment order (h, v, length, type)


@dataclass
class PairEnumeration:
    alignments: list
    undefined_next: bool = False   # stopped where the reference's next step is undefined


def _rows(segments, h_text, v_text):
    r0, r1 = [], []
    for hb, vb, ln, tp in segments:
        if tp == N.GBA_SEG_DIAGONAL:
            r0.append(h_text[hb:hb + ln]); r1.append(v_text[vb:vb + ln])
        elif tp == N.GBA_SEG_HORIZONTAL:
            r0.append(h_text[hb:hb + ln]); r1.append("-" * ln)
        else:
            r0.append("-" * ln); r1.append(v_text[vb:vb + ln])
    # each row's clipped region starts at its first residue
    return "".join(r0).lstrip("-"), "".join(r1).lstrip("-")


def local_enumerate(H, V, score, cutoff: int = 0, max_count: int = 25, alphabet: str = "dna5",
                    context=None) -> list:
    """One GPU call: up to max_count Waterman-Eggert alignments per pair (H[k], V[k])."""
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
    ctx.check(N.lib().gba_local_enumerate(ctx.handle, C.byref(p), C.byref(b), C.byref(r)), "gba_local_enumerate")
    del keep
    sc, bh, eh, bv, ev = arrs
    out = []
    for k in range(n):
        ht, vt = decode(ch[k], alphabet), decode(cv[k], alphabet)
        als = []
        for i in range(int(count[k])):
            g = k * max_count + i
            sg = [tuple(int(x) for x in segs[q]) for q in range(off[g], off[g + 1])]
            r0, r1 = _rows(sg, ht, vt)
            als.append(LocalAlignment(int(sc[g]), r0, r1, int(bh[g]), int(eh[g]), int(bv[g]), int(ev[g]), sg))
        out.append(PairEnumeration(als, int(status[k]) == N.GBA_ENUM_UNDEFINED_NEXT))
    return out


class LocalAlignmentEnumerator:
    """LocalAlignmentEnumerator<Score, Unbanded>(score[, cutoff]) for one pair of sequences."""

    def __init__(self, score, cutoff: int = 0, alphabet: str = "dna5", context=None):
        self.score_scheme, self.cutoff, self.alphabet, self.context = score, cutoff, alphabet, context
        self._pair = None
        self._done = []
        self._next = 0
        self._exhausted = False
        self.current = None

    def _fill(self, h, v, want):
        e = local_enumerate([h], [v], self.score_scheme, self.cutoff, want, self.alphabet, self.context)[0]
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
