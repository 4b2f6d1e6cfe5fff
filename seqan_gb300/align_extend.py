"""Alignment extension with the reference's call surface (align_extend/align_extend.h).

:func:`extend_alignments` extends a batch of aligned parts -- hSeq[beginH, endH) over
vSeq[beginV, endV), given as int64 [n, 4] or [n, 6] position rows -- to the left and right with
the AlignExtend DP (optionally X-drop terminated, optionally banded) in one GPU call
(``gba_extend_alignments``) and returns, per alignment, the two sides' scores and TraceSegment_
lists.  :func:`extendAlignment` is ``extendAlignment(align, [origScore,] hSeq, vSeq, positions,
direction, [lowerDiag, upperDiag,] [xDrop,] score)``: it returns the reference's score (left +
aligned part + right) and the extended rows with their begin and end positions; the aligned
part may carry gaps (``center`` rows).
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field

import numpy as np

from . import _native as N
from .alphabet import decode, encode

EXTEND_LEFT, EXTEND_RIGHT, EXTEND_BOTH = 1, 2, 3
SEG_DIAGONAL, SEG_HORIZONTAL, SEG_VERTICAL = 1, 2, 4


@dataclass
class SideExtension:
    left_score: int
    right_score: int
    left_segments: list = field(default_factory=list)    # prefix coordinates, traceback order
    right_segments: list = field(default_factory=list)   # suffix coordinates, traceback order


def _concat(seqs, alphabet):
    codes = [np.ascontiguousarray(encode(s, alphabet), dtype=np.uint8) for s in seqs]
    off = np.zeros(len(codes) + 1, dtype=np.int64)
    np.cumsum([len(c) for c in codes], out=off[1:])
    flat = np.concatenate(codes) if len(codes) and off[-1] else np.zeros(1, dtype=np.uint8)
    return np.ascontiguousarray(flat), off, codes


def extend_alignments(databases, queries, positions, direction, score, xdrop=None, seed_h=None, seed_v=None,
                      alphabet="dna5", context=None, band=None):
    """One GPU call for a batch; positions rows are (beginH, beginV, endH, endV[, ...]); band =
    (lowerDiag, upperDiag) for the banded overloads.  A side whose band misses its matrix gets
    the reference's invalid value (INT32_MIN) and no segments."""
    pos = np.asarray(positions, dtype=np.int64).reshape(len(positions), -1)
    seeds = np.zeros((len(pos), 6), dtype=np.int64)
    seeds[:, :4] = pos[:, :4]
    sh, oh, _ = _concat(databases, alphabet)
    sv, ov, _ = _concat(queries, alphabet)
    p = N.GbaExtendAlignParams()
    p.direction = int(direction)
    p.xdrop_on = 0 if xdrop is None else 1
    p.xdrop = 0 if xdrop is None else int(xdrop)
    p.match, p.mismatch = score.match, score.mismatch
    p.gap_open, p.gap_extend = score.gap_open, score.gap_extend
    if band is not None:
        p.band_on = 1
        p.band_lower, p.band_upper = int(band[0]), int(band[1])
    keep = None
    if score.matrix is not None:
        keep = np.ascontiguousarray(score.matrix, dtype=np.int32)
        p.matrix = keep.ctypes.data
        p.alphabet_size = int(round(np.sqrt(keep.size)))
    ids_h = None if seed_h is None else np.ascontiguousarray(seed_h, dtype=np.int32)
    ids_v = None if seed_v is None else np.ascontiguousarray(seed_v, dtype=np.int32)
    b = N.GbaSeedBatch(len(oh) - 1, sh.ctypes.data, oh.ctypes.data, len(ov) - 1, sv.ctypes.data, ov.ctypes.data,
                       len(seeds), None if ids_h is None else ids_h.ctypes.data,
                       None if ids_v is None else ids_v.ctypes.data, 0)
    n = len(seeds)
    ls = np.zeros(max(n, 1), dtype=np.int32)
    rs = np.zeros(max(n, 1), dtype=np.int32)
    # a side's segments are at most its computed columns + rows + 2
    hl = (oh[1:] - oh[:-1]) if ids_h is None else (oh[1:] - oh[:-1])[ids_h]
    vl = (ov[1:] - ov[:-1]) if ids_v is None else (ov[1:] - ov[:-1])[ids_v]
    cap = int((hl + vl).sum() + 8 * n + 8)
    segs = np.zeros((cap, 4), dtype=np.uint32)
    offs = np.zeros(2 * n + 1, dtype=np.int64)
    r = N.GbaExtendAlignResult(ls.ctypes.data, rs.ctypes.data, segs.ctypes.data, cap, offs.ctypes.data)
    ctx = context or N.default_context()
    rc = N.lib().gba_extend_alignments(ctx.handle, C.byref(p), C.byref(b), seeds.ctypes.data, C.byref(r))
    ctx.check(rc, "gba_extend_alignments")
    del keep
    out = []
    for k in range(n):
        left = [tuple(int(x) for x in segs[q]) for q in range(offs[2 * k], offs[2 * k + 1])]
        right = [tuple(int(x) for x in segs[q]) for q in range(offs[2 * k + 1], offs[2 * k + 2])]
        out.append(SideExtension(int(ls[k]), int(rs[k]), left, right))
    return out


def _render(segments, h_text, v_text):
    """Gapped rows of a TraceSegment_ list in traceback order (last = begin)."""
    if not segments:
        return "", "", 0, 0
    ch, cv = segments[-1][0], segments[-1][1]
    rh, rv = [], []
    lh = lv = 0
    for (_, _, ln, tp) in reversed(segments):
        if tp == SEG_DIAGONAL:
            rh.append(h_text[ch:ch + ln]); rv.append(v_text[cv:cv + ln]); ch += ln; cv += ln; lh += ln; lv += ln
        elif tp == SEG_VERTICAL:
            rh.append("-" * ln); rv.append(v_text[cv:cv + ln]); cv += ln; lv += ln
        else:
            rh.append(h_text[ch:ch + ln]); rv.append("-" * ln); ch += ln; lh += ln
    return "".join(rh), "".join(rv), lh, lv


@dataclass
class ExtendedAlignment:
    score: int
    row0: str
    row1: str
    h_begin: int
    h_end: int
    v_begin: int
    v_end: int


def _center_score(row0, row1, score, alphabet):
    """The aligned part's score when origScore is omitted (align_extend/align_extend.h:250-270):
    a gap column opens a gap when it is the first column or either row's gap state changes there,
    and extends one otherwise; other columns score their residues."""
    total = 0
    for i, (a, b) in enumerate(zip(row0, row1)):
        g0, g1 = a == "-", b == "-"
        if g0 or g1:
            fresh = i == 0 or (row0[i - 1] == "-") != g0 or (row1[i - 1] == "-") != g1
            total += score.gap_open if fresh else score.gap_extend
        else:
            x, y = int(encode(a, alphabet)[0]), int(encode(b, alphabet)[0])
            total += int(score.matrix[x, y]) if score.matrix is not None else \
                (score.match if x == y else score.mismatch)
    return total


def _int32(x):
    return (x + 2 ** 31) % 2 ** 32 - 2 ** 31


def assemble(ext: SideExtension, h, v, positions, score, alphabet="dna5", orig_score=None,
             center=None) -> ExtendedAlignment:
    """Joins the sides around the aligned part as _extendAlignmentImpl does
    (align_extend/align_extend.h:264-369): rows, begin/end positions and the returned score
    (left + origScore, or the part's own score, + right, in the reference's int arithmetic).
    center: the part's rows with '-' for gaps (None: ungapped)."""
    h = encode(h, alphabet)
    v = encode(v, alphabet)
    hb, vb, he, ve = (int(x) for x in positions[:4])
    text = lambda c: decode(c, alphabet)
    c0, c1 = center if center is not None else (text(h[hb:he]), text(v[vb:ve]))
    mid = _center_score(c0, c1, score, alphabet) if orig_score is None else int(orig_score)
    l0, l1, llh, llv = _render(ext.left_segments, text(h[:hb]), text(v[:vb]))
    r0, r1, rlh, rlv = _render(ext.right_segments, text(h[he:]), text(v[ve:]))
    return ExtendedAlignment(_int32(ext.left_score + mid + ext.right_score), l0 + c0 + r0, l1 + c1 + r1,
                             hb - llh, he + rlh, vb - llv, ve + rlv)


def extendAlignment(h, v, positions, direction, *args, orig_score=None, center=None, alphabet="dna5",
                    context=None):
    """extendAlignment(align, [origScore,] hSeq, vSeq, positions, direction, [lowerDiag,
    upperDiag,] [xDrop,] score) on the aligned part hSeq[positions[0], positions[2]) /
    vSeq[positions[1], positions[3]); origScore as orig_score=, the part's gapped rows as
    center=(row0, row1)."""
    if len(args) == 1:
        band, xdrop, score = None, None, args[0]
    elif len(args) == 2:
        band, (xdrop, score) = None, args
    elif len(args) == 3:
        band, xdrop, score = (args[0], args[1]), None, args[2]
    elif len(args) == 4:
        band, xdrop, score = (args[0], args[1]), args[2], args[3]
    else:
        raise TypeError("extendAlignment(h, v, positions, direction, [lowerDiag, upperDiag,] [xDrop,] score)")
    ext = extend_alignments([h], [v], [list(positions)[:4]], direction, score, xdrop, alphabet=alphabet,
                            context=context, band=band)[0]
    return assemble(ext, h, v, positions, score, alphabet, orig_score=orig_score, center=center)
