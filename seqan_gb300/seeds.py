"""Seed extension with the reference's call surface (seeds/seeds_extension.h).

* :class:`Seed` -- Seed<Simple, DefaultSeedConfig> (seeds/seeds_seed_simple.h:78-132): begin and
  end positions in the database (H) and the query (V), lower/upper diagonal (H - V).
* :func:`extendSeed` -- ``extendSeed(seed, database, query, direction, MatchExtend())`` and
  ``extendSeed(seed, database, query, direction, score, scoreDropOff, UnGappedXDrop() |
  GappedXDrop())`` (seeds/seeds_extension.h:181-218, 283-360, 780-835), one seed.
* :func:`extend_seeds` -- the same over a batch in one GPU call (``gba_extend_seeds``): seeds
  as an int64 array [n, 6] or a list of :class:`Seed`, each on database ``seed_h[k]`` and query
  ``seed_v[k]`` (default: database k / query k).

The extension runs on the GPU only; a missing engine library raises.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _native as N
from .alphabet import encode

EXTEND_NONE, EXTEND_LEFT, EXTEND_RIGHT, EXTEND_BOTH = 0, 1, 2, 3


class MatchExtend:
    """Tag: extend while the residues match (no scoring scheme)."""
    method = N.GBA_MATCH_EXTEND


class UnGappedXDrop:
    """Tag: ungapped x-drop extension along the seed's diagonal."""
    method = N.GBA_UNGAPPED_XDROP


class GappedXDrop:
    """Tag: gapped x-drop extension (anti-diagonal DP with a drop-off bound)."""
    method = N.GBA_GAPPED_XDROP


class Seed:
    """Seed<Simple>: ``Seed(beginH, beginV, length)`` or ``Seed(beginH, beginV, endH, endV)``;
    the diagonals start as the reference's constructors set them."""

    __slots__ = ("begin_h", "begin_v", "end_h", "end_v", "lower_diagonal", "upper_diagonal")

    def __init__(self, begin_h=0, begin_v=0, end_h_or_length=0, end_v=None):
        self.begin_h, self.begin_v = int(begin_h), int(begin_v)
        if end_v is None:
            self.end_h = self.begin_h + int(end_h_or_length)
            self.end_v = self.begin_v + int(end_h_or_length)
            self.lower_diagonal = self.upper_diagonal = self.begin_h - self.begin_v
        else:
            self.end_h, self.end_v = int(end_h_or_length), int(end_v)
            d0, d1 = self.begin_h - self.begin_v, self.end_h - self.end_v
            self.lower_diagonal, self.upper_diagonal = min(d0, d1), max(d0, d1)

    @property
    def begin_diagonal(self) -> int:
        return self.begin_h - self.begin_v

    @property
    def end_diagonal(self) -> int:
        return self.end_h - self.end_v

    def as_row(self):
        return [self.begin_h, self.begin_v, self.end_h, self.end_v, self.lower_diagonal, self.upper_diagonal]

    @classmethod
    def from_row(cls, row):
        s = cls()
        (s.begin_h, s.begin_v, s.end_h, s.end_v, s.lower_diagonal, s.upper_diagonal) = (int(x) for x in row)
        return s

    def __eq__(self, other):
        return isinstance(other, Seed) and self.as_row() == other.as_row()

    def __repr__(self):
        return (f"Seed(H {self.begin_h}..{self.end_h}, V {self.begin_v}..{self.end_v}, "
                f"diagonals [{self.lower_diagonal}, {self.upper_diagonal}])")


def _concat(seqs, alphabet):
    codes = [np.ascontiguousarray(encode(s, alphabet), dtype=np.uint8) for s in seqs]
    off = np.zeros(len(codes) + 1, dtype=np.int64)
    np.cumsum([len(c) for c in codes], out=off[1:])
    flat = np.concatenate(codes) if len(codes) and off[-1] else np.zeros(1, dtype=np.uint8)
    return np.ascontiguousarray(flat), off


def _params(method, direction, score, score_drop_off):
    p = N.GbaExtendParams()
    p.method = int(method)
    p.direction = int(direction)
    p.score_drop_off = int(score_drop_off)
    keep = None
    if score is not None:
        if method == N.GBA_GAPPED_XDROP and score.gap_open != score.gap_extend:
            raise ValueError("GappedXDrop needs a linear gap score (gap open == gap extend)")
        p.match, p.mismatch, p.gap = score.match, score.mismatch, score.gap_extend
        if score.matrix is not None:
            keep = np.ascontiguousarray(score.matrix, dtype=np.int32)
            p.matrix = keep.ctypes.data
            p.alphabet_size = int(round(np.sqrt(keep.size)))
    return p, keep


def _method_of(tag):
    return tag.method if hasattr(tag, "method") else int(tag)


def extend_seeds(seeds, databases, queries, direction=EXTEND_BOTH, score=None, score_drop_off=0,
                 method=GappedXDrop, seed_h=None, seed_v=None, alphabet="dna5", return_scores=False,
                 context=None):
    """Extends a batch of seeds on the GPU; returns the grown seeds as int64 [n, 6]
    (beginH, beginV, endH, endV, lowerDiagonal, upperDiagonal), plus the gapped left/right
    extension scores [n, 2] when ``return_scores``."""
    method = _method_of(method)
    if isinstance(seeds, np.ndarray) and seeds.ndim == 2 and seeds.shape[1] == 6:
        arr = np.ascontiguousarray(seeds, dtype=np.int64).copy()
    else:
        arr = np.array([s.as_row() for s in seeds], dtype=np.int64).reshape(-1, 6)
    sh, oh = _concat(databases, alphabet)
    sv, ov = _concat(queries, alphabet)
    ids_h = None if seed_h is None else np.ascontiguousarray(seed_h, dtype=np.int32)
    ids_v = None if seed_v is None else np.ascontiguousarray(seed_v, dtype=np.int32)
    p, keep = _params(method, direction, score if method != N.GBA_MATCH_EXTEND else None, score_drop_off)
    b = N.GbaSeedBatch(len(oh) - 1, sh.ctypes.data, oh.ctypes.data, len(ov) - 1, sv.ctypes.data, ov.ctypes.data,
                       len(arr), None if ids_h is None else ids_h.ctypes.data,
                       None if ids_v is None else ids_v.ctypes.data, 0)
    scores = np.zeros((max(len(arr), 1), 2), dtype=np.int32) if return_scores else None
    ctx = context or N.default_context()
    rc = N.lib().gba_extend_seeds(ctx.handle, C.byref(p), C.byref(b), arr.ctypes.data if len(arr) else None,
                                  None if scores is None else scores.ctypes.data)
    ctx.check(rc, "gba_extend_seeds")
    del keep
    return (arr, scores[:len(arr)]) if return_scores else arr


def extendSeed(seed, database, query, direction, *args, alphabet="dna5", context=None):
    """extendSeed(seed, database, query, direction, MatchExtend()) or
    extendSeed(seed, database, query, direction, score, scoreDropOff, UnGappedXDrop() |
    GappedXDrop()); grows ``seed`` in place like the reference."""
    if len(args) == 1:
        score, drop, tag = None, 0, args[0]
    elif len(args) == 3:
        score, drop, tag = args
    else:
        raise TypeError("extendSeed(seed, database, query, direction, MatchExtend()) or "
                        "(..., score, scoreDropOff, UnGappedXDrop()/GappedXDrop())")
    out = extend_seeds([seed], [database], [query], direction, score, drop, tag, alphabet=alphabet,
                       context=context)
    (seed.begin_h, seed.begin_v, seed.end_h, seed.end_v, seed.lower_diagonal,
     seed.upper_diagonal) = (int(x) for x in out[0])
    return seed
