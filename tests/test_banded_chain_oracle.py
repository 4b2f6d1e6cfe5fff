"""Banded chain alignment, oracle (CPU): the restatement of bandedChainAlignment
(seeds/banded_chain_alignment*.h, oracle/banded_chain_oracle.c) pinned to the reference test file's
known answers (tests/seeds/test_align_banded_chain_impl.cpp) and to 440 chains run through the
compiled reference (tests/golden/banded_chain_cases.json)."""
import numpy as np
import pytest

from oracle import oracle as O
from tests import golden_cases as G

CASES = G.load("banded_chain_cases.json")["cases"]
LIN, AFF = (5, -3, -5, -5), (5, -3, -1, -5)
FULL = 15   # AlignConfig<true, true, true, true>

_A = "AAAAAAAAAAATTTTTTTTTTCCCCCCCC"
_B = "AAAAAAAAAAAGGGGGGGGGGCCCCCCCC"
_T3H = "TTTTTTTTTTGGGGGGGGGGGAAAAAAAAAAAGGGGGGTTCCCCCCCC"
_T3V = "AAAAAAAAAAAGGGGGGGGGGCCCCCCCCAAAAAAAAAAATTTTTTTTGGGGGGGGGGGG"
_T3S = [(10, 11, 21, 21), (21, 29, 32, 40), (38, 40, 40, 48)]
_C5H, _C5V = "CCCCCGTGTGAAAAAAAAAAATCGAT", "CGTGCAAAAAAAAAAAGTAGCGGGGG"

# (H, V, chain, bandExtension, scheme, score, row0, row1) from the reference's test file
KNOWN = [
    ("AAAAAAAAAAA", "AAAAAAAAAAA", [(0, 0, 11, 11)], 5, LIN, 55, "AAAAAAAAAAA", "AAAAAAAAAAA"),
    ("AAAAAAAAAAA", "AAAAAAAAAAA", [(0, 0, 11, 11)], 5, AFF, 55, "AAAAAAAAAAA", "AAAAAAAAAAA"),
    ("CCCCCAAAAAAAAAAATTTTT", "GGGGGAAAAAAAAAAAGGGGG", [(5, 5, 16, 16)], 5, AFF, 37,
     "CCCCC-----AAAAAAAAAAA-----TTTTT", "-----GGGGGAAAAAAAAAAAGGGGG-----"),
    ("CCCCCAAAAAAAAAAATTTTT", "GGGGGAAAAAAAAAAAGGGGG", [(5, 5, 16, 16)], 5, LIN, 25,
     "CCCCCAAAAAAAAAAATTTTT", "GGGGGAAAAAAAAAAAGGGGG"),
    ("CCCCCGTGTGAAAAAAAAAAATCGATTTTTT", "GGGGGCGTGCAAAAAAAAAAAGTAGCGGGGG", [(10, 10, 21, 21)], 5, AFF, 56,
     "-----CCCCCGTGTG-AAAAAAAAAAA-T--CG----ATTTTTT", "GGGGGC------GTGCAAAAAAAAAAAGTAGCGGGGG-------"),
    ("CCCCCGTGTGAAAAAAAAAAATCGATTTTTT", "GGGGGCGTGCAAAAAAAAAAAGTAGCGGGGG", [(10, 10, 21, 21)], 5, LIN, 43,
     "-CCCCCGTGTGAAAAAAAAAAA-T--CGATTTTTT", "GGGGGCGTG-CAAAAAAAAAAAGTAGCGGGGG---"),
    ("CCCCCAAAAAAAAAAATCGATTTTTT", "GGGGGCGTGCAAAAAAAAAAAGTAGCGGGGG", [(5, 10, 16, 21)], 5, AFF, 52,
     "-----CCCCCAAAAAAAAAAA-T--CG----ATTTTTT", "GGGGGCGTGCAAAAAAAAAAAGTAGCGGGGG-------"),
    ("CCCCCAAAAAAAAAAATCGATTTTTT", "GGGGGCGTGCAAAAAAAAAAAGTAGCGGGGG", [(5, 10, 16, 21)], 5, LIN, 44,
     "-----CCCCCAAAAAAAAAAA-T--CGATTTTTT", "GGGGGCGTGCAAAAAAAAAAAGTAGCGGGGG---"),
    (_C5H, _C5V, [(10, 5, 21, 16)], 5, AFF, 66, "CCCCCGTGTGAAAAAAAAAAATCGAT--------", "----CGTG-CAAAAAAAAAAA--G-TAGCGGGGG"),
    (_C5H, _C5V, [(10, 5, 21, 16)], 5, LIN, 63, "CCCCCGTGTGAAAAAAAAAAA-TCGAT----", "----CGTG-CAAAAAAAAAAAGTAGCGGGGG"),
    (_C5H, _C5V, [(12, 5, 19, 16)], 5, AFF, 66, "CCCCCGTGTGAAAAAAAAAAATCGAT--------", "----CGTG-CAAAAAAAAAAA--G-TAGCGGGGG"),
    (_C5H, _C5V, [(12, 5, 19, 16)], 5, LIN, 63, "CCCCCGTGTGAAAAAAAAAAA-TCGAT----", "----CGTG-CAAAAAAAAAAAGTAGCGGGGG"),
    (_C5H, _C5V, [(5, 12, 16, 14)], 5, AFF, 64, "CCCCCGTGTGAAAAAAAAAA--ATCGAT----", "----CGTGCAAAAAAAAAAAGTAGCG--GGGG"),
    (_C5H, _C5V, [(5, 12, 16, 14)], 5, LIN, 62, "CCCCCGTGTGAAAAAAAAAAATCGAT----", "----CGTGCAAAAAAAAAAAGTAGCGGGGG"),
    (_C5H, _C5V, [(12, 5, 19, 16)], 8, AFF, 66, "CCCCCGTGTGAAAAAAAAAAATCGAT--------", "----CGTG-CAAAAAAAAAAA--G-TAGCGGGGG"),
    (_C5H, _C5V, [(12, 5, 19, 16)], 8, LIN, 63, "CCCCCGTGTGAAAAAAAAAAA-TCGAT----", "----CGTG-CAAAAAAAAAAAGTAGCGGGGG"),
    (_C5V, _C5H, [(5, 12, 16, 19)], 8, AFF, 66, "----CGTG-CAAAAAAAAAAA--G-TAGCGGGGG", "CCCCCGTGTGAAAAAAAAAAATCGAT--------"),
    (_C5V, _C5H, [(5, 12, 16, 19)], 8, LIN, 63, "----CGTG-CAAAAAAAAAAAGTAGCGGGGG", "CCCCCGTGTGAAAAAAAAAAA-TCGAT----"),
    (_A, _B, [(0, 2, 11, 11), (21, 21, 26, 29)], 5, LIN, 65, _A, _B),
    (_A, _B, [(0, 2, 11, 11), (21, 21, 26, 29)], 5, AFF, 67,
     "AAAAAAAAAAATTTTTTTTTT----------CCCCCCCC", "AAAAAAAAAAA----------GGGGGGGGGGCCCCCCCC"),
    (_A, _B, [(2, 6, 17, 15), (17, 15, 29, 29)], 5, LIN, 65, _A, _B),
    (_A, _B, [(2, 6, 17, 15), (17, 15, 29, 29)], 5, AFF, 55,
     "AAAAAAAAAAATTTTTTTTTTCC----------CCCCCC--", "AAAAAAAAAAA------------GGGGGGGGGGCCCCCCCC"),
    (_A, _B, [(2, 6, 17, 15), (17, 15, 29, 29)], 7, AFF, 67,
     "AAAAAAAAAAATTTTTTTTTT----------CCCCCCCC", "AAAAAAAAAAA----------GGGGGGGGGGCCCCCCCC"),
    (_A, _B, [(2, 6, 17, 15), (17, 15, 29, 29)], 1, AFF, 61,
     "AAAAAAAAAAA----TTTTTTTT----TTCCCCCCCC", "AAAAAAAAAAAGGGG--------GGGGGGCCCCCCCC"),
    (_T3H, _T3V, _T3S, 1, LIN, 5, "-TTTTTTTTTTGGGGGGGGGG-------GAAAAAAAAAAAGGGGGGTTCCCCCCCC----", _T3V),
    (_T3H, _T3V, _T3S, 1, AFF, 65,
     "-----------TTTTTTTTTTGGGGGGGGGG-------GAAAAAAAAAAAGGGGGGTTCCCCCCCC------------------",
     "AAAAAAAAAAA----------GGGGGGGGGGCCCCCCCCAAAAAAAAAAA------TT--------TTTTTTGGGGGGGGGGGG"),
    (_T3H, _T3V, _T3S, 15, LIN, 109,
     "TTTTTTTTTTGGGGGGGGGGGAAAAAAAAAAAGGGG--GGTTCCCCCCCC-------------------------------",
     "---------------------AAAAAAAAAAAGGGGGGGGGGCCCCCCCCAAAAAAAAAAATTTTTTTTGGGGGGGGGGGG"),
    (_T3H, _T3V, _T3S, 15, AFF, 113,
     "TTTTTTTTTTGGGGGGGGGGGAAAAAAAAAAAGGGG--GGTTCCCCCCCC-------------------------------",
     "---------------------AAAAAAAAAAAGGGGGGGGGGCCCCCCCCAAAAAAAAAAATTTTTTTTGGGGGGGGGGGG"),
    (_T3H, _T3V, _T3S, 6, LIN, 3, "-TTTTTTTTTTGGGGGGGGGG-------GAAAAAAAAAAA-------GGGGGGTTCCCCCCCC",
     "AAAAAAAAAAAGGGGGGGGGGCCCCCCCCAAAAAAAAAAATTTTTTTTGGGGGGGGGGGG---"),
]
KNOWN_IDS = [f"known{i}" for i in range(len(KNOWN))]


def codes(text):
    return G.codes([text], "dna")[0]


def rows_of(segments, h, v):
    """The two rows _adaptTraceSegmentsTo builds from a trace that runs from (0, 0) to the end."""
    r0, r1 = [], []
    for hb, vb, ln, tp in reversed(segments):
        if tp == O.SEG_DIAGONAL:
            r0.append(h[hb:hb + ln]); r1.append(v[vb:vb + ln])
        elif tp == O.SEG_HORIZONTAL:
            r0.append(h[hb:hb + ln]); r1.append("-" * ln)
        else:
            r0.append("-" * ln); r1.append(v[vb:vb + ln])
    return "".join(r0), "".join(r1)


@pytest.mark.parametrize("case", KNOWN, ids=KNOWN_IDS)
def test_known_answers_of_the_reference_tests(case):
    h, v, chain, k, sc, score, row0, row1 = case
    r = O.oracle_banded_chain(codes(h), codes(v), chain, sc, sc, FULL, k)
    assert r.status == 0
    assert r.score == score
    assert rows_of(r.segments, h, v) == (row0, row1)


def test_empty_chain_scores_numeric_min():
    r = O.oracle_banded_chain(codes("ACGATCGATCGACTGACT"), codes("ACGATCGATCGACTGACT"), [], LIN, LIN, FULL, 5)
    assert r.status == 0 and r.score == -2 ** 31 and r.segments == []


@pytest.mark.parametrize("chunk", range(0, len(CASES), 110))
def test_oracle_matches_reference_fixtures(chunk):
    for c in CASES[chunk:chunk + 110]:
        r = O.oracle_banded_chain(codes(c["H"]), codes(c["V"]), c["seeds"], c["anchor"], c["gap"], c["free_ends"],
                                  c["k"])
        assert r.status == c["status"], c
        if c["status"] == 0:
            assert (r.score, r.n_traces) == (c["score"], c["n_traces"]), c
            assert [list(s) for s in r.segments] == c["segments"], c
            assert list(rows_of(r.segments, c["H"], c["V"])) == c["rows"], c


def test_fixtures_cover_the_cases():
    ok = [c for c in CASES if c["status"] == 0]
    assert any(c["status"] == 1 for c in CASES)                            # the reference throws
    assert {c["free_ends"] for c in ok} == set(range(16))                   # every AlignConfig
    assert any(c["anchor"] != c["gap"] for c in ok)                         # two schemes
    assert any(c["anchor"][2] != c["anchor"][3] for c in ok) and any(c["anchor"][2] == c["anchor"][3] for c in ok)
    assert any(c["n_traces"] > 1 for c in ok)                               # co-optimal traces
    assert any(len(c["seeds"]) >= 10 for c in ok)
    assert {c["k"] for c in ok} >= {1, 15}
    assert any(len(c["H"]) >= 800 for c in ok)


@pytest.mark.skipif(not O.ref_available(), reason="compiled reference not present")
def test_oracle_matches_live_reference_random():
    from tests.golden.make_golden import chain_case
    rng = np.random.Generator(np.random.PCG64(991))
    for trial in range(200):
        h, v, seeds, a, g, fe, k = chain_case(rng)
        o = O.oracle_banded_chain(h, v, seeds, a, g, fe, k)
        r = O.ref_banded_chain(h, v, seeds, a, g, fe, k)
        assert o.status == r.status, trial
        if r.status == 0:
            assert (o.score, o.segments, o.n_traces) == (r.score, r.segments, r.n_traces), trial
