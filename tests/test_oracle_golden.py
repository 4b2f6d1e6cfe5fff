"""The oracle (C restatement) against the reference's own outputs stored as fixtures.

This pins the oracle: every score, gapped row, clip position, CIGAR and raw TraceSegment_
list in tests/golden/reference_cases.json came from SeqAn 2 compiled from its headers
(tests/golden/make_golden.py)."""
import numpy as np
import pytest

import golden_cases as G
from oracle import oracle as O

SCORE_CASES = G.cases("score")
GAPS_CASES = G.cases("gaps")
SEG_CASES = G.cases("segments")


@pytest.mark.parametrize("case", SCORE_CASES, ids=[G.case_id(c) for c in SCORE_CASES])
def test_oracle_scores_match_reference(case):
    p = case["problem"]
    H, V = G.codes(case["H"], p["alphabet"]), G.codes(case["V"], p["alphabet"])
    res = O.oracle_batch(G.oracle_problem(p), H, V)
    assert res.score.tolist() == case["scores"]


@pytest.mark.parametrize("case", GAPS_CASES, ids=[G.case_id(c) for c in GAPS_CASES])
def test_oracle_gaps_match_reference(case):
    p = case["problem"]
    H, V = G.codes(case["H"], p["alphabet"]), G.codes(case["V"], p["alphabet"])
    res = O.oracle_batch(G.oracle_problem(p), H, V, traceback=True)
    assert res.score.tolist() == case["scores"]
    for k in range(len(H)):
        segs = res.segments[k]
        assert list(O.render_rows(segs, case["H"][k], case["V"][k])) == case["rows"][k], k
        assert list(O.segments_clip(segs)) == case["clip"][k], k
        assert O.cigar_string(segs) == case["cigar"][k], k


@pytest.mark.parametrize("case", SEG_CASES, ids=[G.case_id(c) for c in SEG_CASES])
def test_oracle_segments_match_reference(case):
    p = case["problem"]
    H, V = G.codes(case["H"], p["alphabet"]), G.codes(case["V"], p["alphabet"])
    res = O.oracle_batch(G.oracle_problem(p), H, V, traceback=True)
    assert res.score.tolist() == case["scores"]
    for k in range(len(H)):
        assert [list(s) for s in res.segments[k]] == case["segments"][k], k


def test_blosum62_table_matches_reference():
    from seqan_gb300.scoring import BLOSUM62_AA27
    assert np.array_equal(BLOSUM62_AA27, np.array(G.load("blosum62.json")["matrix"]))


@pytest.mark.parametrize("alphabet", ["dna5", "dna", "aa"])
def test_alphabet_maps_match_reference(alphabet):
    from seqan_gb300.alphabet import encode
    d = G.load("alphabets.json")
    assert encode(d["chars"], alphabet).tolist() == d[alphabet]


def test_invalid_pairs_score_numeric_min():
    pb = O.Problem(score_bits=16)
    res = O.oracle_batch(pb, [np.zeros(0, np.uint8), np.array([1, 2], np.uint8)],
                         [np.array([1], np.uint8), np.zeros(0, np.uint8)])
    assert res.score.tolist() == [-32768, -32768]
    res = O.oracle_batch(O.Problem(score_bits=32), [np.zeros(0, np.uint8)], [np.array([1], np.uint8)])
    assert res.score.tolist() == [-(2 ** 31)]
