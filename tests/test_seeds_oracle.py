"""Seed extension oracle (CPU): pinned to the reference's own known answers
(tests/seeds/test_seeds_extension.cpp) and to extendSeed outputs of the compiled reference
(tests/golden/seed_cases.json); where the compiled reference is present, also checked live on
random seeds."""
import numpy as np
import pytest

from oracle import oracle as O
from tests import golden_cases as G

B62 = np.array(G.load("blosum62.json")["matrix"], dtype=np.int32)

# Known answers of tests/seeds/test_seeds_extension.cpp: (method, direction, H, V, seed
# (beginH, beginV, length), (match, mismatch, gap) or "b62" with gap, drop-off, expected
# (beginH, beginV, endH, endV[, lower, upper])).  The UnGappedXDrop cases pass the string named
# "query" as the database argument, as the reference test does.
ME, UX, GX = O.MATCH_EXTEND, O.UNGAPPED_XDROP, O.GAPPED_XDROP
L, R, B = O.EXTEND_LEFT, O.EXTEND_RIGHT, O.EXTEND_BOTH
ED = (0, -1, -1)   # Score<int, EditDistance>
KNOWN = [
    # testSeedsExtensionMatchExtension (:48-113)
    (ME, L, "CCCCCCCCC", "AAACCCCCCAA", (4, 5, 2), None, 0, (2, 3, 6, 7)),
    (ME, L, "CCCCCCCCC", "AAAAACCCCAA", (4, 5, 2), None, 0, (4, 5, 6, 7)),
    (ME, R, "AAAAAAAAACC", "AAAAAAAAA", (5, 4, 2), None, 0, (5, 4, 9, 8)),
    (ME, R, "AAAAAACC", "AAAAAAAAAA", (4, 5, 2), None, 0, (4, 5, 6, 7)),
    (ME, B, "GGCCCCCCAA", "AAACCCCCCC", (4, 5, 2), None, 0, (2, 3, 8, 9)),
    (ME, B, "GGCCCCAAAA", "AAACCCCCCC", (4, 5, 2), None, 0, (2, 3, 6, 7)),
    (ME, B, "GGCCCCCCAA", "AAAAACCCCC", (4, 5, 2), None, 0, (4, 5, 8, 9)),
    (ME, B, "CCCCAACCC", "AAAAAAAAAAA", (4, 5, 2), None, 0, (4, 5, 6, 7)),
    # testSeedsExtensionUnGappedXDropExtension (:118-188)
    (UX, L, "AAACACCCCAA", "CCCCCCCCC", (5, 4, 2), ED, 2, (3, 2, 7, 6)),
    (UX, L, "AAAAACCACAA", "CCCCCCCCC", (5, 4, 2), ED, 2, (5, 4, 7, 6)),
    (UX, R, "AAAAAAACACC", "AAAAAAAAA", (5, 4, 2), ED, 2, (5, 4, 9, 8)),
    (UX, R, "AAAAAAAAAA", "AAAAAACC", (5, 4, 2), ED, 2, (5, 4, 7, 6)),
    (UX, B, "AAACCCCCCC", "GGCCCCCCAA", (5, 4, 2), ED, 2, (3, 2, 9, 8)),
    (UX, B, "AAACCCCCCC", "GGCCCCAAAA", (5, 4, 2), ED, 2, (3, 2, 7, 6)),
    (UX, B, "AAAAACCCCC", "GGCCCCCCAA", (5, 4, 2), ED, 2, (5, 4, 9, 8)),
    (UX, B, "AAAAAAAAAAA", "CCCCAACCC", (5, 4, 2), ED, 2, (5, 4, 7, 6)),
    # testSeedsExtensionGappedXDropExtension (:193-460): expected (bH, bV, eH, eV, lower, upper)
    (GX, B, "AACCCCTTTGGTGAAAAA", "AAACCCTTTGGGTTTTT", (4, 4, 3), (2, -1, -1), 1, (0, 0, 14, 13, -2, 2)),
    (GX, B, "ttttcgatcgatgcttttt", "aaaacgatcgatgc", (4, 4, 9), (2, -1, -1), 1, (3, 3, 15, 14, 0, 1)),
    (GX, B, "ttttcgatcgatgcttttt", "aaaacgatcgatgc", (5, 5, 7), (2, -1, -1), 1, (3, 3, 15, 14, -1, 1)),
    (GX, B, "ttttcgatcgatgcttttt", "aaaacgatcgatgc", (6, 6, 6), (2, -1, -1), 0, (4, 4, 14, 14, 0, 0)),
    (GX, B, "ttttcgatcgatgc", "cgatcgatgcaaaaaaaaa", (5, 1, 5), (2, -1, -1), 1, (3, 0, 14, 11, 3, 5)),
    (GX, B, "cgatcgatgccaact", "aaaaaaaaacgatcgatgcaaaaaaaaa", (2, 11, 4), (2, -1, -1), 1,
     (0, 8, 14, 23, -10, -7)),
    (GX, B, "ccccagctgatcgtttgcccccc", "ttttagtgacgttttaaaaaa", (11, 9, 5), (1, -5, -5), 7, (4, 4, 17, 15, 0, 2)),
    (GX, B, "ccccccgtttgctagtcgacccc", "aaaaaattttgcagtgatttt", (7, 7, 5), (1, -5, -5), 7, (6, 6, 19, 17, 0, 2)),
    (GX, B, "ttttagtgacgttttaaaaaa", "ccccagctgatcgtttgcccccc", (9, 11, 5), (1, -5, -5), 7,
     (4, 4, 15, 17, -2, 0)),
    (GX, B, "AGCAGCAAACAGTAAGCCAGCAGCCT", "CTGACAGCGAGAAACAGTAACCAGCTAGCCT", (21, 26, 5), (1, -9, -9), 45,
     (0, 1, 26, 31, -9, 0)),
    (GX, B, "CSNNHKMMMMAAGGW", "CSNNHKMMMMAAGGW", (6, 6, 3), ("b62", -9), 1, (0, 0, 15, 15, 0, 0)),
    (GX, B, "CSNNHKMMMMAAGGW", "CSNNHMMMMAAGGW", (6, 5, 3), ("b62", -9), 10, (0, 0, 15, 14, -1, 2)),
    (GX, B, "CSNNHKMMMMAAGGW", "CSNNHRMLMLAAGGW", (6, 6, 3), ("b62", -9), 10, (0, 0, 15, 15, -1, 1)),
    (GX, B, "CSNNHKMMMMAAGGW", "WWNNHKMMMMAAGLV", (6, 6, 3), ("b62", -9), 10, (0, 0, 15, 15, -1, 1)),
    (GX, B, "CSNNHKMMMMAAGGW", "WSNNHMLMWAAGLV", (6, 5, 3), ("b62", -9), 10, (0, 0, 15, 14, -1, 2)),
    (GX, B, "CSNNHKMMMMAGWW", "WSNNHMLMWAARGWW", (6, 5, 3), ("b62", -9), 10, (0, 0, 14, 13, -1, 2)),
]


def known_problem(case):
    method, direction, h, v, seed, sc, x, want = case
    if sc is not None and sc[0] == "b62":
        sp = O.SeedProblem(method, direction, 0, 0, sc[1], x, B62, "aa")
        alph = "aa"
    else:
        mt, mm, g = sc if sc is not None else (0, -1, -1)
        sp = O.SeedProblem(method, direction, mt, mm, g, x)
        alph = "dna5"
    return sp, G.codes([h], alph)[0], G.codes([v], alph)[0], seed, want


@pytest.mark.parametrize("case", KNOWN, ids=[f"{c[0]}-{c[1]}-{c[2][:8]}-{c[4]}" for c in KNOWN])
def test_oracle_matches_reference_known_answers(case):
    sp, h, v, seed, want = known_problem(case)
    got, _ = O.oracle_extend_seeds(sp, [h], [v], [seed])
    assert tuple(got[0][:len(want)]) == tuple(want)


def seed_case_inputs(c):
    alph = c["alphabet"]
    H = G.codes(c["H"], alph)
    V = G.codes(c["V"], alph)
    sp = O.SeedProblem(c["method"], c["direction"], c["match"], c["mismatch"], c["gap"], c["xdrop"],
                       B62 if c["blosum62"] else None, alph)
    return sp, H, V


SEED_CASES = G.load("seed_cases.json")["cases"]


def seed_case_id(c):
    return (f"m{c['method']}-d{c['direction']}-{c['alphabet']}-{c['match']},{c['mismatch']},{c['gap']}"
            f"-x{c['xdrop']}{'-b62' if c['blosum62'] else ''}")


@pytest.mark.parametrize("case", SEED_CASES, ids=[seed_case_id(c) for c in SEED_CASES])
def test_oracle_matches_reference_fixtures(case):
    sp, H, V = seed_case_inputs(case)
    got, xs = O.oracle_extend_seeds(sp, H, V, np.array(case["seeds"], dtype=np.int64), case["pair_of_seed"])
    assert got.tolist() == case["extended"]
    if case["xscores"] is not None:
        assert xs.tolist() == case["xscores"]


def test_fixtures_cover_every_method_direction_and_edge():
    kinds = {(c["method"], c["direction"]) for c in SEED_CASES}
    assert kinds == {(m, d) for m in (0, 1, 2) for d in (1, 2, 3)}
    assert any(c["blosum62"] for c in SEED_CASES)
    total = sum(len(c["seeds"]) for c in SEED_CASES)
    assert total > 2000
    # empty seeds, seeds at both sequence ends, empty sequences
    edge = [c for c in SEED_CASES if "" in c["H"] or "" in c["V"]]
    assert edge and any(s[2] == s[0] for c in edge for s in c["seeds"])


@pytest.mark.skipif(not O.ref_available(), reason="compiled reference not present")
def test_oracle_matches_live_reference_random():
    rng = np.random.default_rng(77)
    for trial in range(300):
        aa = trial % 3 == 0
        A = 20 if aa else 4
        h = rng.integers(0, A, int(rng.integers(1, 120))).astype(np.uint8)
        v = h.copy()
        sub = rng.random(len(v)) < 0.15
        v[sub] = (v[sub] + 1) % A
        if aa:
            from seqan_gb300.workloads import AA20_CODES
            h, v = AA20_CODES[h], AA20_CODES[v]
        method = int(rng.integers(0, 3))
        if aa:
            sp = O.SeedProblem(method, int(rng.integers(1, 4)), 0, 0, -9, int(rng.integers(0, 40)), B62, "aa")
        else:
            g = int(rng.integers(-5, 0))
            sp = O.SeedProblem(method, int(rng.integers(1, 4)), int(rng.integers(1, 4)), int(rng.integers(g, 1)), g,
                               int(rng.integers(0, 30)))
        L = int(rng.integers(0, min(len(h), len(v)) + 1))
        bh = int(rng.integers(0, len(h) - L + 1))
        bv = min(bh, len(v) - L)
        if L == 0 and method == UX:
            continue
        ref, rx = O.ref_extend_seeds(sp, [h], [v], [(bh, bv, L)])
        orc, ox = O.oracle_extend_seeds(sp, [h], [v], [(bh, bv, L)])
        assert ref.tolist() == orc.tolist(), (trial, sp)
        if method == GX:
            assert rx.tolist() == ox.tolist(), (trial, sp)
