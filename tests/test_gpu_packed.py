"""Packed input on the GPU (gba_align_packed): String<TValue, Packed<>> host words uploaded as is
and unpacked on the device give the same results as the same sequences sent as codes."""
import numpy as np
import pytest

from tests import golden_cases as G

pytestmark = pytest.mark.gpu


def _same(a, b, traceback=False):
    assert np.array_equal(a.score, b.score) and np.array_equal(a.end_h, b.end_h) and \
        np.array_equal(a.end_v, b.end_v) and np.array_equal(a.status, b.status)
    if traceback:
        assert np.array_equal(a.segment_offsets, b.segment_offsets)
        n = int(a.segment_offsets[-1])
        assert np.array_equal(a.segments[:n], b.segments[:n])


@pytest.mark.parametrize("bits,alphabet", [(2, 4), (3, 5), (5, 27)])
@pytest.mark.parametrize("mode,tb", [(0, False), (0, True), (1, True)])
def test_packed_equals_codes(engine, bits, alphabet, mode, tb):
    import seqan_gb300 as sg
    from seqan_gb300 import align as A
    from seqan_gb300 import workloads as W
    rng = np.random.default_rng(bits * 10 + mode)
    H, V = [], []
    for k in range(3000):
        L = int(rng.integers(0, 300)) if k % 50 else 0
        h = rng.integers(0, alphabet, L).astype(np.uint8)
        v = W.mutate(rng, h, 0.1, 0.02, alphabet=alphabet) if k % 3 else \
            rng.integers(0, alphabet, int(rng.integers(0, 300))).astype(np.uint8)
        H.append(h)
        V.append(v)
    score = sg.Blosum62(-1, -11, dtype=np.int16) if alphabet == 27 else sg.Score(2, -4, -1, -6, dtype=np.int16)
    a = A.align_codes(H, V, score, mode=mode, traceback=tb, alphabet_size=alphabet)
    b = A.align_codes(H, V, score, mode=mode, traceback=tb, alphabet_size=alphabet, packed_bits=bits)
    _same(a, b, tb)


def test_packed_banded_cigar_and_shared(engine):
    import seqan_gb300 as sg
    from seqan_gb300 import align as A
    from seqan_gb300 import workloads as W
    wins, reads = W.read_windows(20000, ref_len=1_000_000, seed=8)
    score = sg.Score(2, -4, -1, -6, dtype=np.int16)
    cfg = sg.AlignConfig(True, False, False, True)
    a = A.align_codes(wins, reads, score, config=cfg, band=(-6, 26), cigar=True, alphabet_size=4)
    b = A.align_codes(wins, reads, score, config=cfg, band=(-6, 26), cigar=True, alphabet_size=4, packed_bits=2)
    _same(a, b, True)
    assert np.array_equal(a.cigar[:int(a.cigar_offsets[-1])], b.cigar[:int(b.cigar_offsets[-1])])
    H = [wins[0]]
    a = A.align_codes(H, reads[:5000], score, h_shared=True, alphabet_size=4)
    b = A.align_codes(H, reads[:5000], score, h_shared=True, alphabet_size=4, packed_bits=3)
    _same(a, b)


def test_large_batch_chunked(engine):
    """450,000 short pairs: the chunked score path on unpacked codes."""
    import seqan_gb300 as sg
    from seqan_gb300 import align as A
    from seqan_gb300 import workloads as W
    H, V = W.mutated_dna_pairs(450_000, 20, 60, seed=12)
    score = sg.Score(2, -4, -1, -6, dtype=np.int16)
    a = A.align_codes(H, V, score, alphabet_size=4)
    b = A.align_codes(H, V, score, alphabet_size=4, packed_bits=2)
    _same(a, b)


def test_reference_packed_words_as_input(engine):
    """The reference's own host words (fixtures) as input, aligned against themselves."""
    import ctypes as C
    import seqan_gb300 as sg
    from seqan_gb300 import _native as N
    from seqan_gb300 import align as A
    cases = [c for c in G.load("packed_cases.json")["cases"] if c["alphabet"] == "dna5" and c["codes"]]
    words = [np.array([int(w, 16) for w in c["words"]], dtype=np.uint64) for c in cases]
    codes = [np.array(c["codes"], dtype=np.uint8) for c in cases]
    off = np.zeros(len(words) + 1, dtype=np.int64)
    np.cumsum([len(w) for w in words], out=off[1:])
    allw = np.concatenate(words)
    score = sg.Score(2, -3, -5, dtype=np.int32)
    ref = A.align_codes(codes, codes[::-1], score, traceback=True, alphabet_size=5)
    rw = [words[k] for k in range(len(words))][::-1]
    roff = np.zeros(len(rw) + 1, dtype=np.int64)
    np.cumsum([len(w) for w in rw], out=roff[1:])
    rall = np.concatenate(rw)
    params = A.make_params(score, 0, None, None, N.GBA_OUT_SCORE | N.GBA_OUT_END, 5, 0)
    n = len(codes)
    sc, eh, ev, stt = (np.zeros(n, np.int32) for _ in range(4))
    r = N.GbaResult()
    r.score, r.end_h, r.end_v, r.pair_status = (x.ctypes.data for x in (sc, eh, ev, stt))
    ph = N.GbaPackedSet(n, allw.ctypes.data, off.ctypes.data, 3, 0)
    pv = N.GbaPackedSet(n, rall.ctypes.data, roff.ctypes.data, 3, 0)
    ctx = engine
    ctx.check(N.lib().gba_align_packed(ctx.handle, C.byref(params), C.byref(ph), C.byref(pv), 0, C.byref(r)), "packed")
    assert np.array_equal(sc, ref.score) and np.array_equal(eh, ref.end_h) and np.array_equal(ev, ref.end_v)
