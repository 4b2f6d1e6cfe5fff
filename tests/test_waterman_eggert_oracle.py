"""Waterman-Eggert suboptimal local alignments, oracle (CPU): the restatement of the reference's
LocalAlignmentEnumerator<Score, Unbanded> (align/local_alignment_enumeration_unbanded.h,
align/local_alignment_waterman_eggert_impl.h) pinned to the reference test file's known answers
(tests/align/test_align_local_alignment.h:225-330) and to enumerations of the compiled reference
(tests/golden/waterman_eggert_cases.json)."""
import numpy as np
import pytest

from oracle import oracle as O
from tests import golden_cases as G

B62 = np.array(G.load("blosum62.json")["matrix"], dtype=np.int32)
AA = "ABCDEFGHIJKLMNOPQRSTUVWYZX*"
CASES = G.load("waterman_eggert_cases.json")["cases"]

# SimpleScore(2, -1, -2, -2), cutoff 5: (H, V, [(score, row0, row1), ...])
KNOWN = [
    ("ATAAGCGTCTCG", "TCATAGAGTTGC", [(9, "ATAAGCGT", "ATA-GAGT"), (5, "TC-TCG", "TCATAG")]),
    ("GGGGCTTAAGCTTGGGG", "AAAACTTAGCTCTAAAA",
     [(12, "CTTAAGCT", "CTTA-GCT"), (10, "GCT-TAA", "GCTCTAA"), (10, "AAGCTTGG", "AAACTTAG"), (7, "CTTAA", "CTAAA"),
      (5, "AAGCTTG", "AACTTAG")]),
]


def _codes(text, alphabet="dna"):
    return G.codes([text], alphabet)[0]


@pytest.mark.parametrize("case", KNOWN, ids=["testLocalAlign2", "testBandedLocalAlign_1"])
def test_known_answers_of_the_reference_tests(case):
    h, v, want = case
    got = O.oracle_local_enumerate(_codes(h), _codes(v), 2, -1, -2, 5)
    assert [(a.score, a.row0, a.row1) for a in got] == want


def test_third_known_answer():
    # the second example of testBandedLocalAlign: SimpleScore(1, -9, -9, -9), cutoff 7, one alignment
    h = "GCAGAATTAAGGAGGATTACAAGTGGGAATTTGAAGAGCTTTTGAAATCC"
    v = "CGGTTGAGCAGAACTTGGGCTACGAGACTCCCCCCGAGGAATTTGAAGGCTTTCTTCAAATCCAAAAGCA"
    got = O.oracle_local_enumerate(_codes(h), _codes(v), 1, -9, -9, 7)
    assert [(a.score, a.row0, a.row1) for a in got] == [(11, "GGAATTTGAAG", "GGAATTTGAAG")]


def _run(c):
    alph = c["alphabet"]
    h, v = _codes(c["H"], alph), _codes(c["V"], alph)
    return O.oracle_local_enumerate(h, v, c["match"], c["mismatch"], c["gap"], c["cutoff"],
                                    matrix=B62 if c["blosum62"] else None, max_count=c["max_count"],
                                    letters=AA if alph == "aa" else "ACGTN")


@pytest.mark.parametrize("chunk", range(0, len(CASES), 50))
def test_oracle_matches_reference_fixtures(chunk):
    for c in CASES[chunk:chunk + 50]:
        got = _run(c)
        undefined = bool(got) and got[-1] is None
        if undefined:
            got = got[:-1]
        assert undefined == c["undefined_next"], c
        assert [[a.score, a.row0, a.row1, a.h_begin, a.h_end, a.v_begin, a.v_end] for a in got] == c["alignments"], c


def test_fixtures_cover_the_enumeration():
    assert sum(len(c["alignments"]) for c in CASES) > 1000
    assert any(len(c["alignments"]) == c["max_count"] for c in CASES)       # stopped by the count
    assert any(0 < len(c["alignments"]) < c["max_count"] and not c["undefined_next"] for c in CASES)  # exhausted
    assert any(len(c["alignments"]) == 0 for c in CASES)                     # nothing above cutoff
    assert any(c["undefined_next"] for c in CASES)
    assert any(c["blosum62"] for c in CASES) and any(c["cutoff"] <= 0 for c in CASES)
    # alignments with gaps in both rows
    assert any("-" in a[1] and "-" in a[2] for c in CASES for a in c["alignments"])


@pytest.mark.skipif(not O.ref_available(), reason="compiled reference not present")
def test_oracle_matches_live_reference_random():
    from seqan_gb300 import workloads as W
    rng = np.random.default_rng(97)
    for trial in range(150):
        L = int(rng.integers(1, 50))
        h = rng.integers(0, 4, L).astype(np.uint8)
        v = W.mutate(rng, h, 0.2, 0.05) if trial % 2 else rng.integers(0, 4, int(rng.integers(1, 50))).astype(np.uint8)
        mt, mm, gap, cutoff = int(rng.integers(1, 4)), -int(rng.integers(1, 4)), -int(rng.integers(1, 5)), int(rng.integers(0, 9))
        o = O.oracle_local_enumerate(h, v, mt, mm, gap, cutoff, max_count=30)
        truncated = bool(o) and o[-1] is None
        if truncated:
            o = o[:-1]
        r = O.ref_local_enumerate(h, v, mt, mm, gap, cutoff, max_count=len(o) if truncated else 30)
        assert [(a.score, a.row0, a.row1, a.h_begin, a.h_end, a.v_begin, a.v_end) for a in o] == \
            [(a.score, a.row0, a.row1, a.h_begin, a.h_end, a.v_begin, a.v_end) for a in r], trial
