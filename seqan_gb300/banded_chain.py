"""Banded chain alignment with the reference's call surface (seeds/banded_chain_alignment.h).

:func:`bandedChainAlignment` aligns a batch of pairs, each around its own seed chain, in one GPU
call (``gba_banded_chain``): the rectangle before the first anchor, a band of the anchor's diagonals
widened by ``bandExtension`` around every anchor and the rectangle to the next anchor, then the
rectangle to the end of the matrix, each grid started from the cells the previous grid's
traceback reached.  ``scoreAnchor`` scores the bands, ``scoreGap`` the rectangles (the reference's
two-scheme overloads; one scheme serves both when ``scoreGap`` is omitted).  Per pair the result
holds the score, the two gapped rows (the reference's Align rows after _adaptTraceSegmentsTo), the
TraceSegment_ runs they come from and the number of co-optimal traces the reference's trace set
held.  A pair whose chain is empty scores numeric_limits<int>::min() and keeps its rows ungapped,
as the reference does.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _native as N
from .align import AlignConfig, Gaps, _apply_segments
from .alphabet import encode


class ChainError(RuntimeError):
    """A pair where the reference does not return: it throws (no glue point between two grids'
    traces) or its behaviour is undefined."""


class ChainAlignment:
    def __init__(self, score, status, num_traces, segments, gapsH: Gaps, gapsV: Gaps):
        self.score, self.status, self.num_traces, self.segments = score, status, num_traces, segments
        self.gapsH, self.gapsV = gapsH, gapsV

    @property
    def row0(self):
        return self.gapsH.row()

    @property
    def row1(self):
        return self.gapsV.row()


def _seed_array(chain):
    a = np.asarray(chain, dtype=np.int32)
    return a.reshape(-1, 4) if a.size else np.zeros((0, 4), np.int32)


def banded_chain_codes(codes_h, codes_v, chains, score_anchor, score_gap=None, config: AlignConfig | None = None,
                       band_extension: int = 15, max_traces: int = 0, context=None):
    """One GPU call over code arrays; returns (score, status, num_traces, segment lists)."""
    score_gap = score_gap or score_anchor
    for s in (score_anchor, score_gap):
        if s.matrix is not None:
            raise ValueError("bandedChainAlignment takes Score<int, Simple> schemes")
    n = len(codes_h)
    if len(codes_v) != n or len(chains) != n:
        raise ValueError("H, V and the chains must have one entry per pair")
    ch = [np.ascontiguousarray(c, dtype=np.uint8) for c in codes_h]
    cv = [np.ascontiguousarray(c, dtype=np.uint8) for c in codes_v]
    oh = np.zeros(n + 1, np.int64)
    ov = np.zeros(n + 1, np.int64)
    np.cumsum([len(c) for c in ch], out=oh[1:])
    np.cumsum([len(c) for c in cv], out=ov[1:])
    sh = np.concatenate(ch + [np.zeros(1, np.uint8)])
    sv = np.concatenate(cv + [np.zeros(1, np.uint8)])
    sa = [_seed_array(c) for c in chains]
    so = np.zeros(n + 1, np.int64)
    np.cumsum([len(a) for a in sa], out=so[1:])
    seeds = np.ascontiguousarray(np.concatenate(sa + [np.zeros((1, 4), np.int32)]), dtype=np.int32)
    p = N.GbaChainParams()
    p.anchor = N.GbaSimpleScore(score_anchor.match, score_anchor.mismatch, score_anchor.gap_extend,
                                score_anchor.gap_open)
    p.gap = N.GbaSimpleScore(score_gap.match, score_gap.mismatch, score_gap.gap_extend, score_gap.gap_open)
    p.free_ends = (config or AlignConfig()).bits
    p.band_extension = band_extension
    p.max_traces = max_traces
    b = N.GbaBatch(n, sh.ctypes.data, oh.ctypes.data, sv.ctypes.data, ov.ctypes.data, 0, 0)
    sd = N.GbaChainSeeds(seeds.ctypes.data, so.ctypes.data)
    score = np.zeros(max(n, 1), np.int32)
    status = np.zeros(max(n, 1), np.int32)
    ntr = np.zeros(max(n, 1), np.int32)
    cap = int(oh[-1] + ov[-1]) + 8 * n + 8
    segs = np.zeros((cap, 4), np.uint32)
    off = np.zeros(n + 1, np.int64)
    r = N.GbaChainResult(score.ctypes.data, status.ctypes.data, ntr.ctypes.data, segs.ctypes.data, cap, off.ctypes.data)
    ctx = context or N.default_context()
    ctx.check(N.lib().gba_banded_chain(ctx.handle, C.byref(p), C.byref(b), C.byref(sd), C.byref(r)),
              "gba_banded_chain")
    return score[:n], status[:n], ntr[:n], SegmentLists(segs, off, n)


class SegmentLists:
    """The pairs' TraceSegment_ runs of one call: item k is pair k's list of (h, v, length, type)
    tuples, built from the call's output arrays when first read."""

    def __init__(self, segs, off, n):
        self._segs, self._off, self._n = segs, off, n
        self._cache = {}

    def __len__(self):
        return self._n

    def __getitem__(self, k):
        if isinstance(k, slice):
            return [self[i] for i in range(*k.indices(self._n))]
        if k < 0:
            k += self._n
        if not 0 <= k < self._n:
            raise IndexError(k)
        got = self._cache.get(k)
        if got is None:
            got = [tuple(x) for x in self._segs[self._off[k]:self._off[k + 1]].tolist()]
            self._cache[k] = got
        return got

    def __iter__(self):
        return (self[k] for k in range(self._n))

    def __eq__(self, other):
        return list(self) == list(other)


def bandedChainAlignment(seqsH, seqsV, chains, scoreAnchor, scoreGap=None, alignConfig: AlignConfig | None = None,
                         bandExtension: int = 15, alphabet: str = "dna5", max_traces: int = 0, context=None):
    """bandedChainAlignment(align, seedChain, scoreAnchor[, scoreGap][, alignConfig][, bandExtension])
    for a batch: seqsH[k], seqsV[k] with chains[k] = [(beginH, beginV, endH, endV), ...] in chain
    order.  Returns one ChainAlignment per pair; raises ChainError for a pair the reference does
    not complete."""
    codes_h = [encode(s, alphabet) for s in seqsH]
    codes_v = [encode(s, alphabet) for s in seqsV]
    score, status, ntr, segs = banded_chain_codes(codes_h, codes_v, chains, scoreAnchor, scoreGap, alignConfig,
                                                  bandExtension, max_traces, context)
    out = []
    for k in range(len(codes_h)):
        if status[k] != N.GBA_CHAIN_OK:
            raise ChainError(f"pair {k}: " + {N.GBA_CHAIN_NO_GLUE: "no glue point between two grids' traces",
                                              N.GBA_CHAIN_UNDEFINED: "undefined in the reference",
                                              N.GBA_CHAIN_CAPACITY: "more co-optimal traces than max_traces"}
                             .get(int(status[k]), "failed"))
        gH = Gaps(seqsH[k], alphabet)
        gV = Gaps(seqsV[k], alphabet)
        if segs[k]:
            _apply_segments(gH, gV, segs[k])
        out.append(ChainAlignment(int(score[k]), int(status[k]), int(ntr[k]), segs[k], gH, gV))
    return out
