"""Banded Waterman-Eggert suboptimal local alignments on the GPU through
gba_local_enumerate_banded: identical to the reference's LocalAlignmentEnumerator<Score, Banded>
(fixtures from the compiled reference, the reference test file's known answers) and to the
oracle on seeded batches (DNA and protein, narrow, wide and off-centre bands, bands that miss the
matrix, enumerations whose heap outgrows the first launch's room)."""
import numpy as np
import pytest

from oracle import oracle as O
from tests.test_waterman_eggert_banded_oracle import AA, B62, CASES, KNOWN

pytestmark = pytest.mark.gpu


def _score(match, mismatch, gap, blosum62=False):
    import seqan_gb300 as sg
    if blosum62:
        return sg.Blosum62(gap, gap)
    return sg.Score(match, mismatch, gap, gap)


def _key(a):
    return (a.score, a.row0, a.row1, a.h_begin, a.h_end, a.v_begin, a.v_end)


def _oracle(h, v, mt, mm, gap, cutoff, band, max_count, matrix=None, letters="ACGTN"):
    ref = O.oracle_local_enumerate(h, v, mt, mm, gap, cutoff, matrix=matrix, max_count=max_count, letters=letters,
                                   band=band)
    undefined = bool(ref) and ref[-1] is None
    return (ref[:-1] if undefined else ref), undefined


@pytest.mark.parametrize("case", KNOWN, ids=["banded_align_1", "banded_align_2", "banded_align_3"])
def test_known_answers(engine, case):
    from seqan_gb300 import local_enum as LE
    h, v, (mt, mm, gap), cutoff, band, accepted = case
    got = LE.local_enumerate([h], [v], _score(mt, mm, gap), cutoff=cutoff, max_count=50, band=band)[0]
    assert [(a.score, a.row0, a.row1) for a in got.alignments] in accepted
    e = LE.LocalAlignmentEnumerator(_score(mt, mm, gap), band[0], band[1], cutoff)
    seen = []
    while LE.nextLocalAlignment(h, v, e):
        seen.append((e.getScore(), e.current.row0, e.current.row1))
    assert seen in accepted


@pytest.mark.parametrize("chunk", range(0, len(CASES), 100))
def test_fixtures_through_c_abi(engine, chunk):
    from seqan_gb300 import local_enum as LE
    for c in CASES[chunk:chunk + 100]:
        alph = "aa" if c["alphabet"] == "aa" else "dna5"
        got = LE.local_enumerate([c["H"]], [c["V"]], _score(c["match"], c["mismatch"], c["gap"], c["blosum62"]),
                                 c["cutoff"], c["max_count"], alphabet=alph, band=tuple(c["band"]))[0]
        assert got.undefined_next == c["undefined_next"], c
        assert [list(_key(a)) for a in got.alignments] == c["alignments"], c


@pytest.mark.parametrize("band", [(-8, 8), (-30, 2), (0, 40), (-3, -1)])
def test_seeded_dna_batch_vs_oracle(engine, band):
    """1,000 pairs of 40-160 bp (half related), up to 12 alignments each, one call per band."""
    from seqan_gb300 import local_enum as LE
    from seqan_gb300 import workloads as W
    rng = np.random.default_rng(71 + band[0])
    H, V = [], []
    for k in range(1000):
        h = rng.integers(0, 4, int(rng.integers(40, 160))).astype(np.uint8)
        v = W.mutate(rng, h, 0.1, 0.02) if k % 2 else rng.integers(0, 4, int(rng.integers(40, 160))).astype(np.uint8)
        H.append(h)
        V.append(v)
    got = LE.local_enumerate(H, V, _score(2, -3, -2), 4, 12, alphabet="dna5", band=band)
    for k in range(len(H)):
        ref, undefined = _oracle(H[k], V[k], 2, -3, -2, 4, band, 12)
        assert got[k].undefined_next == undefined, k
        assert [_key(a) for a in got[k].alignments] == [_key(a) for a in ref], k
        assert [a.segments for a in got[k].alignments] == [a.segments for a in ref], k


def test_protein_blosum62_batch_vs_oracle(engine):
    from seqan_gb300 import local_enum as LE
    from seqan_gb300 import workloads as W
    H, V = W.protein_pairs(300, seed=62, related=0.8, identity=0.5)
    H, V = [h[:150] for h in H], [v[:150] for v in V]
    got = LE.local_enumerate(H, V, _score(0, 0, -4, True), 10, 8, alphabet="aa", band=(-20, 20))
    for k in range(len(H)):
        ref, undefined = _oracle(H[k], V[k], 0, 0, -4, 10, (-20, 20), 8, matrix=B62, letters=AA)
        assert got[k].undefined_next == undefined, k
        assert [_key(a) for a in got[k].alignments] == [_key(a) for a in ref], k


def test_heap_rerun_and_ragged_batch(engine):
    """Low cutoffs and many alignments push declumped cells again and again: pairs whose heap
    outgrows the first launch's room are rerun; empty bands and one-residue pairs sit between."""
    from seqan_gb300 import local_enum as LE
    rng = np.random.default_rng(9)
    H, V = [], []
    for k in range(200):
        n = 1 if k % 17 == 0 else int(rng.integers(20, 90))
        H.append(rng.integers(0, 4, int(rng.integers(1, 90))).astype(np.uint8))
        V.append(rng.integers(0, 4, n).astype(np.uint8))
    for band in [(-40, 40), (-2, 2), (5, 7), (-100, -95)]:
        got = LE.local_enumerate(H, V, _score(1, -1, -1), 1, 40, alphabet="dna5", band=band)
        for k in range(len(H)):
            ref, undefined = _oracle(H[k], V[k], 1, -1, -1, 1, band, 40)
            assert got[k].undefined_next == undefined, (band, k)
            assert [_key(a) for a in got[k].alignments] == [_key(a) for a in ref], (band, k)


def test_argument_errors(engine):
    import ctypes as C
    from seqan_gb300 import _native as N
    ctx = N.default_context()
    p = N.GbaEnumParams()
    p.match, p.mismatch, p.gap, p.cutoff, p.max_count = 2, -1, -2, 0, 4
    b = N.GbaBatch(0, None, None, None, None, 0, 0)
    off = np.zeros(1, np.int64)
    one = np.zeros(1, np.int32)
    r = N.GbaEnumResult(one.ctypes.data, one.ctypes.data, one.ctypes.data, one.ctypes.data, one.ctypes.data,
                        one.ctypes.data, one.ctypes.data, None, 0, off.ctypes.data)
    assert N.lib().gba_local_enumerate_banded(ctx.handle, C.byref(p), 3, 2, C.byref(b), C.byref(r)) == N.GBA_EINVAL
    assert N.lib().gba_local_enumerate_banded(ctx.handle, C.byref(p), -2, 2, C.byref(b), C.byref(r)) == N.GBA_OK
