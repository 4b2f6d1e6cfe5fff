"""Waterman-Eggert suboptimal local alignments on the GPU through gba_local_enumerate: identical
to the reference's LocalAlignmentEnumerator (fixtures from the compiled reference, the reference
test file's known answers) and to the oracle on seeded batches (DNA and protein, related and
unrelated pairs, cutoffs at and below zero, enumerations cut where the reference's next step is
undefined)."""
import numpy as np
import pytest

from oracle import oracle as O
from tests import golden_cases as G
from tests.test_waterman_eggert_oracle import AA, B62, CASES, KNOWN

pytestmark = pytest.mark.gpu


def _score(match, mismatch, gap, blosum62=False):
    import seqan_gb300 as sg
    if blosum62:
        return sg.Blosum62(gap, gap)
    return sg.Score(match, mismatch, gap, gap)


def _key(a):
    return (a.score, a.row0, a.row1, a.h_begin, a.h_end, a.v_begin, a.v_end)


@pytest.mark.parametrize("case", KNOWN, ids=["testLocalAlign2", "testBandedLocalAlign_1"])
def test_known_answers(engine, case):
    from seqan_gb300 import local_enum as LE
    h, v, want = case
    got = LE.local_enumerate([h], [v], _score(2, -1, -2), cutoff=5, max_count=50)[0]
    assert [(a.score, a.row0, a.row1) for a in got.alignments] == want
    e = LE.LocalAlignmentEnumerator(_score(2, -1, -2), 5)
    seen = []
    while LE.nextLocalAlignment(h, v, e):
        seen.append((e.getScore(), e.current.row0, e.current.row1))
    assert seen == want


@pytest.mark.parametrize("chunk", range(0, len(CASES), 100))
def test_fixtures_through_c_abi(engine, chunk):
    from seqan_gb300 import local_enum as LE
    for c in CASES[chunk:chunk + 100]:
        alph = "aa" if c["alphabet"] == "aa" else "dna5"
        got = LE.local_enumerate([c["H"]], [c["V"]], _score(c["match"], c["mismatch"], c["gap"], c["blosum62"]),
                                 c["cutoff"], c["max_count"], alphabet=alph)[0]
        assert got.undefined_next == c["undefined_next"], c
        assert [list(_key(a)) for a in got.alignments] == c["alignments"], c


@pytest.mark.parametrize("cutoff", [0, 6, -1])
def test_seeded_dna_batch_vs_oracle(engine, cutoff):
    """1,500 pairs of 40-160 bp (half related), up to 12 alignments each, one call."""
    from seqan_gb300 import local_enum as LE
    from seqan_gb300 import workloads as W
    rng = np.random.default_rng(51 + cutoff)
    H, V = [], []
    for k in range(1500):
        h = rng.integers(0, 4, int(rng.integers(40, 160))).astype(np.uint8)
        v = W.mutate(rng, h, 0.1, 0.02) if k % 2 else rng.integers(0, 4, int(rng.integers(40, 160))).astype(np.uint8)
        H.append(h)
        V.append(v)
    got = LE.local_enumerate(H, V, _score(2, -3, -2), cutoff, 12, alphabet="dna5")
    for k in range(len(H)):
        ref = O.oracle_local_enumerate(H[k], V[k], 2, -3, -2, cutoff, max_count=12)
        undefined = bool(ref) and ref[-1] is None
        ref = ref[:-1] if undefined else ref
        assert got[k].undefined_next == undefined, k
        assert [_key(a) for a in got[k].alignments] == [_key(a) for a in ref], k
        assert [a.segments for a in got[k].alignments] == [a.segments for a in ref], k


def test_protein_blosum62_batch_vs_oracle(engine):
    from seqan_gb300 import local_enum as LE
    from seqan_gb300 import workloads as W
    H, V = W.protein_pairs(300, seed=61, related=0.8, identity=0.5)
    H, V = [h[:150] for h in H], [v[:150] for v in V]
    got = LE.local_enumerate(H, V, _score(0, 0, -4, True), 10, 8, alphabet="aa")
    for k in range(len(H)):
        ref = O.oracle_local_enumerate(H[k], V[k], 0, 0, -4, 10, matrix=B62, max_count=8, letters=AA)
        undefined = bool(ref) and ref[-1] is None
        ref = ref[:-1] if undefined else ref
        assert [_key(a) for a in got[k].alignments] == [_key(a) for a in ref], k
