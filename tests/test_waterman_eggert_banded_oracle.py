"""Banded Waterman-Eggert suboptimal local alignments, oracle (CPU): the restatement of the
reference's LocalAlignmentEnumerator<Score, Banded> (align/local_alignment_enumeration_banded.h,
align/local_alignment_banded_waterman_eggert_impl.h) pinned to the reference test file's known
answers (tests/align/test_align_local_alignment.h:470-580) and to enumerations of the compiled
reference (tests/golden/waterman_eggert_banded_cases.json)."""
import numpy as np
import pytest

from oracle import oracle as O
from tests import golden_cases as G

B62 = np.array(G.load("blosum62.json")["matrix"], dtype=np.int32)
AA = "ABCDEFGHIJKLMNOPQRSTUVWYZX*"
CASES = G.load("waterman_eggert_banded_cases.json")["cases"]

# (H, V, score (match, mismatch, gap), cutoff, band, accepted answers: [(score, row0, row1), ...])
KNOWN = [
    ("ATAAGCGTCTCG", "TCATAGAGTTGC", (2, -1, -2), 5, (-4, 4),
     [[(9, "ATAAGCGT", "ATA-GAGT")], [(9, "ATAAGCGT", "AT-AGAGT")]]),
    ("GGGGCTTAAGCTTGGGG", "AAAACTTAGCTCTAAAA", (2, -1, -2), 5, (-10, 10),
     [[(12, "CTTAAGCT", v), (10, "AAGCTTGG", "AAACTTAG"), (10, "GCT-TAA", "GCTCTAA"), (7, "CTTAA", "CTAAA"),
       (5, "AAGCTTG", "AACTTAG")] for v in ("CTTA-GCT", "CTT-AGCT")]),
    ("GCAGAATTAAGGAGGATTACAAGTGGGAATTTGAAGAGCTTTTGAAATCC",
     "CGGTTGAGCAGAACTTGGGCTACGAGACTCCCCCCGAGGAATTTGAAGGCTTTCTTCAAATCCAAAAGCA", (1, -9, -9), 7, (-20, 0),
     [[(11, "GGAATTTGAAG", "GGAATTTGAAG")]]),
]


def _codes(text, alphabet="dna"):
    return G.codes([text], alphabet)[0]


@pytest.mark.parametrize("case", KNOWN, ids=["banded_align_1", "banded_align_2", "banded_align_3"])
def test_known_answers_of_the_reference_tests(case):
    h, v, (mt, mm, gap), cutoff, band, accepted = case
    got = O.oracle_local_enumerate(_codes(h), _codes(v), mt, mm, gap, cutoff, band=band)
    assert [(a.score, a.row0, a.row1) for a in got] in accepted


def _run(c):
    alph = c["alphabet"]
    h, v = _codes(c["H"], alph), _codes(c["V"], alph)
    return O.oracle_local_enumerate(h, v, c["match"], c["mismatch"], c["gap"], c["cutoff"],
                                    matrix=B62 if c["blosum62"] else None, max_count=c["max_count"],
                                    letters=AA if alph == "aa" else "ACGTN", band=tuple(c["band"]))


@pytest.mark.parametrize("chunk", range(0, len(CASES), 50))
def test_oracle_matches_reference_fixtures(chunk):
    for c in CASES[chunk:chunk + 50]:
        got = _run(c)
        undefined = bool(got) and got[-1] is None
        if undefined:
            got = got[:-1]
        assert undefined == c["undefined_next"], c
        assert [[a.score, a.row0, a.row1, a.h_begin, a.h_end, a.v_begin, a.v_end] for a in got] == c["alignments"], c


def test_full_band_equals_unbanded_scores():
    """A band covering the whole matrix finds the same best local score as the unbanded
    enumerator (the two fill the matrix from opposite ends, so later alignments may differ)."""
    rng = np.random.default_rng(5)
    for _ in range(40):
        h = rng.integers(0, 4, int(rng.integers(1, 50))).astype(np.uint8)
        v = rng.integers(0, 4, int(rng.integers(1, 50))).astype(np.uint8)
        a = O.oracle_local_enumerate(h, v, 2, -1, -2, 1, max_count=1)
        b = O.oracle_local_enumerate(h, v, 2, -1, -2, 1, max_count=1, band=(-len(v), len(h)))
        assert [x.score for x in a if x] == [x.score for x in b if x]


def test_band_outside_the_matrix_gives_nothing():
    h, v = _codes("ACGTACGT"), _codes("ACGT")
    assert O.oracle_local_enumerate(h, v, 2, -1, -2, 1, band=(8, 12)) == []
    assert O.oracle_local_enumerate(h, v, 2, -1, -2, 1, band=(-9, -4)) == []


@pytest.mark.skipif(not O.ref_available(), reason="compiled reference (oracle/_ref) not built")
def test_oracle_matches_reference_random():
    rng = np.random.default_rng(77)
    for t in range(60):
        h = rng.integers(0, 4, int(rng.integers(1, 40))).astype(np.uint8)
        v = rng.integers(0, 4, int(rng.integers(1, 40))).astype(np.uint8)
        lo = int(rng.integers(-len(v) + 1, len(h)))
        up = int(rng.integers(max(lo, -len(v) + 1), len(h) + 4))
        mt, mm, gap, cutoff = int(rng.integers(1, 4)), -int(rng.integers(1, 4)), -int(rng.integers(1, 5)), 2
        o = O.oracle_local_enumerate(h, v, mt, mm, gap, cutoff, max_count=20, band=(lo, up))
        truncated = bool(o) and o[-1] is None
        if truncated:
            o = o[:-1]
        r = O.ref_local_enumerate(h, v, mt, mm, gap, cutoff, max_count=len(o) if truncated else 20, band=(lo, up))
        assert [(a.score, a.row0, a.row1, a.h_begin, a.h_end, a.v_begin, a.v_end) for a in o] == \
               [(a.score, a.row0, a.row1, a.h_begin, a.h_end, a.v_begin, a.v_end) for a in r]
