"""The oracle's DynamicGaps cells against the reference (CPU).

tests/golden/dynamic_cases.json holds seeded pairs aligned by the reference's own single-pair DP with
DynamicGaps cells (align/dp_cell_dynamic.h, align/dp_formula_dynamic.h), made by
tests/golden/make_golden.py --only dynamic from the reference compiled here: every AlignConfig shape
it instantiates, local mode, int16 and int32 cells, Simple and Blosum62 scores.  The oracle must give
the same score and the same raw TraceSegment_ list for every pair."""
import dataclasses

import numpy as np
import pytest

import golden_cases as G
from oracle import oracle as O

CASES = G.load("dynamic_cases.json")["cases"]


def _problem(p):
    return dataclasses.replace(G.oracle_problem(p), dynamic=True)


@pytest.mark.parametrize("case", CASES, ids=[G.case_id({"kind": "dynamic", "problem": c["problem"]}) for c in CASES])
def test_oracle_dynamic_gaps_match_reference(case):
    p = case["problem"]
    H, V = G.codes(case["H"], p["alphabet"]), G.codes(case["V"], p["alphabet"])
    out = O.oracle_batch(_problem(p), H, V, traceback=True)
    for k, want in enumerate(case["results"]):
        assert out.score[k] == want["score"], k
        assert [list(s) for s in out.segments[k]] == want["segments"], k


def test_oracle_refuses_banded_dynamic_gaps():
    with pytest.raises(RuntimeError):
        O.oracle_batch(O.Problem("global", 0, (-3, 3), 2, -3, -5, -1, dynamic=True), [np.array([0, 1], np.uint8)],
                       [np.array([0], np.uint8)])
