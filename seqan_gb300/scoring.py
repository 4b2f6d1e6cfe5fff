"""Scoring schemes of the reference's batch interface.

* :class:`Score` -- Score<T, Simple> (score/score_simple.h:54-98).  The constructor keeps the
  reference's argument order ``(match, mismatch, gap)`` or ``(match, mismatch, gapExtend,
  gapOpen)``: a gap of length k costs gapOpen + (k - 1) * gapExtend.
* :class:`Blosum62` -- Score<T, ScoreMatrix<AminoAcid, ScoreSpecBlosum62>> with constructor
  ``(gapExtend, gapOpen)`` (score/score_matrix.h:112-115).

``dtype`` is the reference's TScoreValue (np.int16 or np.int32); it sets the engine's cell
width semantics (int16 "infinity" -16384, numeric min for invalid pairs).
"""
from __future__ import annotations

import numpy as np

# BLOSUM62 over the 27-letter AminoAcid alphabet (A B C D E F G H I J K L M N O P Q R S T U V W
# Y Z X *), row = first (H) residue.  The values must equal the reference's table
# (score/score_matrix_data.h:311-400) for scores to match; tests/test_oracle_golden.py checks
# them against a fixture dumped from the compiled reference (tests/golden/blosum62.json).
BLOSUM62_AA27 = np.array([
    [ 4, -2,  0, -2, -1, -2,  0, -2, -1, -1, -1, -1, -1, -2,  0, -1, -1, -1,  1,  0,  0,  0, -3, -2, -1,  0, -4],
    [-2,  4, -3,  4,  1, -3, -1,  0, -3, -4,  0, -4, -3,  3, -1, -2,  0, -1,  0, -1, -1, -3, -4, -3,  1, -1, -4],
    [ 0, -3,  9, -3, -4, -2, -3, -3, -1, -1, -3, -1, -1, -3, -2, -3, -3, -3, -1, -1, -2, -1, -2, -2, -3, -2, -4],
    [-2,  4, -3,  6,  2, -3, -1, -1, -3, -4, -1, -4, -3,  1, -1, -1,  0, -2,  0, -1, -1, -3, -4, -3,  1, -1, -4],
    [-1,  1, -4,  2,  5, -3, -2,  0, -3, -3,  1, -3, -2,  0, -1, -1,  2,  0,  0, -1, -1, -2, -3, -2,  4, -1, -4],
    [-2, -3, -2, -3, -3,  6, -3, -1,  0,  0, -3,  0,  0, -3, -1, -4, -3, -3, -2, -2, -1, -1,  1,  3, -3, -1, -4],
    [ 0, -1, -3, -1, -2, -3,  6, -2, -4, -4, -2, -4, -3,  0, -1, -2, -2, -2,  0, -2, -1, -3, -2, -3, -2, -1, -4],
    [-2,  0, -3, -1,  0, -1, -2,  8, -3, -3, -1, -3, -2,  1, -1, -2,  0,  0, -1, -2, -1, -3, -2,  2,  0, -1, -4],
    [-1, -3, -1, -3, -3,  0, -4, -3,  4,  3, -3,  2,  1, -3, -1, -3, -3, -3, -2, -1, -1,  3, -3, -1, -3, -1, -4],
    [-1, -4, -1, -4, -3,  0, -4, -3,  3,  3, -3,  3,  2, -3, -1, -3, -3, -3, -2, -1, -1,  2, -3, -1, -3, -1, -4],
    [-1,  0, -3, -1,  1, -3, -2, -1, -3, -3,  5, -2, -1,  0, -1, -1,  1,  2,  0, -1, -1, -2, -3, -2,  1, -1, -4],
    [-1, -4, -1, -4, -3,  0, -4, -3,  2,  3, -2,  4,  2, -3, -1, -3, -2, -2, -2, -1, -1,  1, -2, -1, -3, -1, -4],
    [-1, -3, -1, -3, -2,  0, -3, -2,  1,  2, -1,  2,  5, -2, -1, -2,  0, -1, -1, -1, -1,  1, -1, -1, -1, -1, -4],
    [-2,  3, -3,  1,  0, -3,  0,  1, -3, -3,  0, -3, -2,  6, -1, -2,  0,  0,  1,  0, -1, -3, -4, -2,  0, -1, -4],
    [ 0, -1, -2, -1, -1, -1, -1, -1, -1, -1, -1, -1, -1, -1, -1, -2, -1, -1,  0,  0, -1, -1, -2, -1, -1, -1, -4],
    [-1, -2, -3, -1, -1, -4, -2, -2, -3, -3, -1, -3, -2, -2, -2,  7, -1, -2, -1, -1, -2, -2, -4, -3, -1, -2, -4],
    [-1,  0, -3,  0,  2, -3, -2,  0, -3, -3,  1, -2,  0,  0, -1, -1,  5,  1,  0, -1, -1, -2, -2, -1,  3, -1, -4],
    [-1, -1, -3, -2,  0, -3, -2,  0, -3, -3,  2, -2, -1,  0, -1, -2,  1,  5, -1, -1, -1, -3, -3, -2,  0, -1, -4],
    [ 1,  0, -1,  0,  0, -2,  0, -1, -2, -2,  0, -2, -1,  1,  0, -1,  0, -1,  4,  1,  0, -2, -3, -2,  0,  0, -4],
    [ 0, -1, -1, -1, -1, -2, -2, -2, -1, -1, -1, -1, -1,  0,  0, -1, -1, -1,  1,  5,  0,  0, -2, -2, -1,  0, -4],
    [ 0, -1, -2, -1, -1, -1, -1, -1, -1, -1, -1, -1, -1, -1, -1, -2, -1, -1,  0,  0, -1, -1, -2, -1, -1, -1, -4],
    [ 0, -3, -1, -3, -2, -1, -3, -3,  3,  2, -2,  1,  1, -3, -1, -2, -2, -3, -2,  0, -1,  4, -3, -1, -2, -1, -4],
    [-3, -4, -2, -4, -3,  1, -2, -2, -3, -3, -3, -2, -1, -4, -2, -4, -2, -3, -3, -2, -2, -3, 11,  2, -3, -2, -4],
    [-2, -3, -2, -3, -2,  3, -3,  2, -1, -1, -2, -1, -1, -2, -1, -3, -1, -2, -2, -2, -1, -1,  2,  7, -2, -1, -4],
    [-1,  1, -3,  1,  4, -3, -2,  0, -3, -3,  1, -3, -1,  0, -1, -1,  3,  0,  0, -1, -1, -2, -3, -2,  4, -1, -4],
    [ 0, -1, -2, -1, -1, -1, -1, -1, -1, -1, -1, -1, -1, -1, -1, -2, -1, -1,  0,  0, -1, -1, -2, -1, -1, -1, -4],
    [-4, -4, -4, -4, -4, -4, -4, -4, -4, -4, -4, -4, -4, -4, -4, -4, -4, -4, -4, -4, -4, -4, -4, -4, -4, -4,  1]
], dtype=np.int32)


class Score:
    """Score<T, Simple>(match, mismatch, gap) / (match, mismatch, gapExtend, gapOpen)."""

    matrix = None

    def __init__(self, match=0, mismatch=-1, gap_extend=-1, gap_open=None, dtype=np.int32):
        self.match = int(match)
        self.mismatch = int(mismatch)
        self.gap_extend = int(gap_extend)
        self.gap_open = int(gap_extend if gap_open is None else gap_open)
        self.dtype = np.dtype(dtype)
        if self.dtype not in (np.dtype(np.int16), np.dtype(np.int32)):
            raise ValueError("score dtype must be int16 or int32")

    @property
    def bits(self) -> int:
        return 16 if self.dtype == np.dtype(np.int16) else 32

    def __repr__(self):
        return (f"Score({self.match}, {self.mismatch}, {self.gap_extend}, {self.gap_open}, "
                f"dtype={self.dtype.name})")


class Blosum62(Score):
    """Score<T, ScoreMatrix<AminoAcid, ScoreSpecBlosum62>>(gapExtend, gapOpen)."""

    def __init__(self, gap_extend=-1, gap_open=None, dtype=np.int32):
        super().__init__(0, 0, gap_extend, gap_open, dtype)
        self.matrix = np.ascontiguousarray(BLOSUM62_AA27)

    def __repr__(self):
        return f"Blosum62({self.gap_extend}, {self.gap_open}, dtype={self.dtype.name})"
