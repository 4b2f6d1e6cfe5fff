"""extendAlignment oracle (CPU): the AlignExtend DP with and without the X-drop terminator,
pinned to the reference's own known answers (tests/align_extend/test_align_extend.h) and to
extendAlignment outputs of the compiled reference (tests/golden/extend_cases.json)."""
import numpy as np
import pytest

from oracle import oracle as O
from tests import golden_cases as G

B62 = np.array(G.load("blosum62.json")["matrix"], dtype=np.int32)
AA = "ABCDEFGHIJKLMNOPQRSTUVWYZX*"

# test_align_extend_simple (:44-112), the cases whose center is an ungapped seed: Score<int>(2, -1,
# -2), EXTEND_BOTH, no X-drop.  (H, V, seed positions, expected rows, clipped begin / end of row 0
# and row 1 in view positions, score.)
KNOWN = [
    ("NNNNNNNNNNTTCCGGGAC" "GGTA" "CACACACGGGGGGGGGG", "CTCGGGAC" "GGTA" "CAGGCACGGTTTTTTTT", (19, 8, 23, 12),
     "CGGGAC" "GGTA" "CACACACGG", "CGGGAC" "GGTA" "CAGGCACGG", (13, 32, 2, 21), 12 + 8 + 12),
    ("NNNNNNNNNNTTCCGGGA" "GGTA" "CACACACGGGGGGGGGG", "CTCGGGAC" "GGTA" "AGGCACGGTTTTTTTT", (18, 8, 22, 12),
     "CGGGA-" "GGTA" "CACACACGG", "CGGGAC" "GGTA" "-AGGCACGG", (13, 32, 2, 21), 8 + 8 + 8),
]


@pytest.mark.parametrize("case", KNOWN, ids=["no_gaps", "gaps_in_extensions"])
def test_known_answers_of_the_reference_tests(case):
    h, v, pos, row0, row1, clips, score = case
    pb = O.Problem("extend", 0, None, 2, -1, -2, -2, None, 32, "dna")
    r = O.oracle_extend_alignment(pb, G.codes([h], "dna")[0], G.codes([v], "dna")[0], pos, O.EXTEND_BOTH)
    assert (r.row0, r.row1) == (row0, row1)
    assert (r.h_begin, r.h_begin + len(r.row0), r.v_begin, r.v_begin + len(r.row1)) == clips
    assert r.score == score


EXTEND_CASES = G.load("extend_cases.json")["cases"]


def extend_problem(c):
    return O.Problem("extend", 0, None, c["match"], c["mismatch"], c["gap_open"], c["gap_extend"],
                     B62 if c["blosum62"] else None, 32, c["alphabet"], c["xdrop"])


@pytest.mark.parametrize("chunk", range(0, len(EXTEND_CASES), 60))
def test_oracle_matches_reference_fixtures(chunk):
    for c in EXTEND_CASES[chunk:chunk + 60]:
        pb = extend_problem(c)
        alph = "aa" if c["alphabet"] == "aa" else "dna"
        h, v = G.codes([c["H"]], alph)[0], G.codes([c["V"]], alph)[0]
        r = O.oracle_extend_alignment(pb, h, v, c["positions"], c["direction"],
                                      letters=AA if alph == "aa" else "ACGTN")
        assert (r.score, r.row0, r.row1, [r.h_begin, r.h_end, r.v_begin, r.v_end]) == \
            (c["score"], c["row0"], c["row1"], c["ends"]), c


def test_fixtures_cover_xdrop_and_gap_models():
    assert any(c["xdrop"] is None for c in EXTEND_CASES)
    assert any(c["xdrop"] == 0 for c in EXTEND_CASES)
    assert any(c["gap_open"] != c["gap_extend"] for c in EXTEND_CASES)
    assert any(c["blosum62"] for c in EXTEND_CASES)
    assert {c["direction"] for c in EXTEND_CASES} == {1, 2, 3}
    # some extensions stopped by the drop-off before a sequence end
    assert any(c["xdrop"] is not None and c["ends"][1] < len(c["H"]) and c["ends"][3] < len(c["V"])
               for c in EXTEND_CASES)


@pytest.mark.skipif(not O.ref_available(), reason="compiled reference not present")
def test_oracle_matches_live_reference_random():
    from seqan_gb300 import workloads as W
    rng = np.random.default_rng(91)
    for trial in range(300):
        L = int(rng.integers(2, 80))
        h = rng.integers(0, 4, L).astype(np.uint8)
        v = W.mutate(rng, h, 0.2, 0.05)
        sl = int(rng.integers(1, min(len(h), len(v), 8) + 1))
        hb = int(rng.integers(0, len(h) - sl + 1))
        vb = min(hb, len(v) - sl)
        go = int(rng.integers(-6, 0))
        pb = O.Problem("extend", 0, None, 2, -3, go, int(rng.choice([go, -1])), None, 32, "dna",
                       None if trial % 2 else int(rng.integers(0, 20)))
        d = int(rng.integers(1, 4))
        a = O.ref_extend_alignment(pb, h, v, (hb, vb, hb + sl, vb + sl), d)
        b = O.oracle_extend_alignment(pb, h, v, (hb, vb, hb + sl, vb + sl), d)
        assert (a.score, a.row0, a.row1, a.h_begin, a.h_end, a.v_begin, a.v_end) == \
            (b.score, b.row0, b.row1, b.h_begin, b.h_end, b.v_begin, b.v_end), trial


# --- The other overloads: (lowerDiag, upperDiag), origScore, aligned parts with gaps -----------

BANDED_CASES = G.load("extend_banded_cases.json")["cases"]


def banded_problem(c):
    return O.Problem("extend", 0, tuple(c["band"]), c["match"], c["mismatch"], c["gap_open"], c["gap_extend"],
                     B62 if c["blosum62"] else None, 32, c["alphabet"], c["xdrop"])


@pytest.mark.parametrize("chunk", range(0, len(BANDED_CASES), 100))
def test_oracle_matches_reference_banded_origscore_gapped_fixtures(chunk):
    """The banded AlignExtend DP (the band phases of align/dp_algorithm_impl.h:586-967 with every
    cell tracked, the X-drop checks at the reference's column boundaries), origScore and the
    aligned part's gap score (align_extend/align_extend.h:250-270) against the compiled
    reference's extendAlignment overloads."""
    for c in BANDED_CASES[chunk:chunk + 100]:
        pb = banded_problem(c)
        alph = "aa" if c["alphabet"] == "aa" else "dna"
        h, v = G.codes([c["H"]], alph)[0], G.codes([c["V"]], alph)[0]
        r = O.oracle_extend_alignment(pb, h, v, c["positions"], c["direction"],
                                      letters=AA if alph == "aa" else "ACGTN", orig_score=c["orig_score"],
                                      center=c["center"])
        assert (r.score, r.row0, r.row1, [r.h_begin, r.h_end, r.v_begin, r.v_end]) == \
            (c["score"], c["row0"], c["row1"], c["ends"]), c


def test_banded_fixtures_cover_the_overloads():
    bands = [tuple(c["band"]) for c in BANDED_CASES]
    assert any(lo == up == 0 for lo, up in bands)                      # one diagonal
    assert any(lo > 0 for lo, up in bands)                             # band misses the matrices
    assert any(up - lo > 200 for lo, up in bands)                      # wider than the matrices
    assert any(c["xdrop"] is not None for c in BANDED_CASES) and any(c["xdrop"] is None for c in BANDED_CASES)
    assert any(c["orig_score"] is not None for c in BANDED_CASES)
    assert any(c["center"] is not None for c in BANDED_CASES)
    assert any(c["blosum62"] for c in BANDED_CASES)
    assert {c["direction"] for c in BANDED_CASES} == {0, 1, 2, 3}
    # the band changes the result against the unbanded extension for some cases
    changed = 0
    for c in BANDED_CASES[:300]:
        alph = "aa" if c["alphabet"] == "aa" else "dna"
        h, v = G.codes([c["H"]], alph)[0], G.codes([c["V"]], alph)[0]
        pb = banded_problem(c)
        pb.band = None
        r = O.oracle_extend_alignment(pb, h, v, c["positions"], c["direction"],
                                      letters=AA if alph == "aa" else "ACGTN", orig_score=c["orig_score"],
                                      center=c["center"])
        changed += (r.row0, r.row1) != (c["row0"], c["row1"])
    assert changed > 20


@pytest.mark.skipif(not O.ref_available(), reason="compiled reference not present")
def test_oracle_matches_live_reference_banded_random():
    from seqan_gb300 import workloads as W
    rng = np.random.default_rng(93)
    for trial in range(400):
        L = int(rng.integers(2, 120))
        h = rng.integers(0, 4, L).astype(np.uint8)
        v = W.mutate(rng, h, 0.2, 0.05)
        sl = int(rng.integers(1, min(len(h), len(v), 8) + 1))
        hb = int(rng.integers(0, len(h) - sl + 1))
        vb = min(hb, len(v) - sl)
        go = int(rng.integers(-6, 0))
        band = (-int(rng.integers(0, 12)), int(rng.integers(0, 12)))
        pb = O.Problem("extend", 0, band, 2, -3, go, int(rng.choice([go, -1])), None, 32, "dna",
                       None if trial % 2 else int(rng.integers(0, 20)))
        d = int(rng.integers(1, 4))
        a = O.ref_extend_alignment(pb, h, v, (hb, vb, hb + sl, vb + sl), d)
        b = O.oracle_extend_alignment(pb, h, v, (hb, vb, hb + sl, vb + sl), d)
        assert (a.score, a.row0, a.row1, a.h_begin, a.h_end, a.v_begin, a.v_end) == \
            (b.score, b.row0, b.row1, b.h_begin, b.h_end, b.v_begin, b.v_end), trial
