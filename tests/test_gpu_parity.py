"""GPU parity: the engine (through the C-ABI) against the reference's fixtures and the oracle.

Everything is integer arithmetic, so every comparison is exact: scores, best-cell positions,
raw TraceSegment_ lists, begin positions and CIGARs."""
import numpy as np
import pytest

import golden_cases as G
from oracle import oracle as O

pytestmark = pytest.mark.gpu

SCORE_CASES = G.cases("score")
GAPS_CASES = G.cases("gaps")
SEG_CASES = G.cases("segments")


def run_engine(p, H, V, traceback=False, cigar=False):
    import seqan_gb300 as sg
    score, mode, cfg, band = G.engine_args(p)
    return sg.align_codes(H, V, score, mode=mode, config=cfg, band=band, traceback=traceback, cigar=cigar)


@pytest.mark.parametrize("case", SCORE_CASES, ids=[G.case_id(c) for c in SCORE_CASES])
def test_scores_match_reference_fixture(engine, case):
    p = case["problem"]
    H, V = G.codes(case["H"], p["alphabet"]), G.codes(case["V"], p["alphabet"])
    out = run_engine(p, H, V)
    assert out.score.tolist() == case["scores"]


@pytest.mark.parametrize("case", GAPS_CASES, ids=[G.case_id(c) for c in GAPS_CASES])
def test_gaps_and_cigar_match_reference_fixture(engine, case):
    p = case["problem"]
    H, V = G.codes(case["H"], p["alphabet"]), G.codes(case["V"], p["alphabet"])
    out = run_engine(p, H, V, traceback=True, cigar=True)
    assert out.score.tolist() == case["scores"]
    for k in range(len(H)):
        segs = out.pair_segments(k)
        assert list(O.render_rows(segs, case["H"][k], case["V"][k])) == case["rows"][k], k
        assert list(O.segments_clip(segs)) == case["clip"][k], k
        assert out.pair_cigar(k) == case["cigar"][k], k


@pytest.mark.parametrize("case", SEG_CASES, ids=[G.case_id(c) for c in SEG_CASES])
def test_segments_match_reference_fixture(engine, case):
    p = case["problem"]
    H, V = G.codes(case["H"], p["alphabet"]), G.codes(case["V"], p["alphabet"])
    out = run_engine(p, H, V, traceback=True)
    assert out.score.tolist() == case["scores"]
    for k in range(len(H)):
        assert [list(s) for s in out.pair_segments(k)] == case["segments"][k], k


def _random_pairs(seed, n, lo, hi, alpha=4):
    rng = np.random.default_rng(seed)
    H = [rng.integers(0, alpha, rng.integers(lo, hi + 1)).astype(np.uint8) for _ in range(n)]
    V = []
    for h in H:
        if rng.random() < 0.5:
            v = h.copy()
            m = rng.random(len(v)) < 0.1
            v[m] = (v[m] + 1) % alpha
            V.append(v)
        else:
            V.append(rng.integers(0, alpha, rng.integers(lo, hi + 1)).astype(np.uint8))
    return H, V


SCHEMES = [(2, -3, -5, -5), (2, -4, -6, -1), (4, -2, -10, -4), (1, -1, -2, -2), (3, -2, -4, -4)]


@pytest.mark.parametrize("fe", range(16))
@pytest.mark.parametrize("scheme", SCHEMES)
def test_all_free_end_configs_against_oracle(engine, fe, scheme):
    import seqan_gb300 as sg
    mt, mm, go, ge = scheme
    H, V = _random_pairs(100 + fe, 150, 1, 90)
    cfg = sg.AlignConfig(bool(fe & 1), bool(fe & 2), bool(fe & 4), bool(fe & 8))
    for bits, dtype in ((16, np.int16), (32, np.int32)):
        out = sg.align_codes(H, V, sg.Score(mt, mm, ge, go, dtype=dtype), config=cfg, traceback=True, cigar=True)
        ref = O.oracle_batch(O.Problem("global", fe, None, mt, mm, go, ge, None, bits), H, V, traceback=True)
        assert np.array_equal(out.score, ref.score)
        assert np.array_equal(out.end_h, ref.end_h) and np.array_equal(out.end_v, ref.end_v)
        for k in range(len(H)):
            assert out.pair_segments(k) == ref.segments[k], k
            assert out.pair_cigar(k) == O.cigar_string(ref.segments[k]), k


@pytest.mark.parametrize("scheme", SCHEMES)
def test_local_against_oracle(engine, scheme):
    import seqan_gb300 as sg
    mt, mm, go, ge = scheme
    H, V = _random_pairs(7, 300, 1, 160)
    out = sg.align_codes(H, V, sg.Score(mt, mm, ge, go, dtype=np.int16), mode=1, traceback=True)
    ref = O.oracle_batch(O.Problem("local", 0, None, mt, mm, go, ge, None, 16), H, V, traceback=True)
    assert np.array_equal(out.score, ref.score)
    assert np.array_equal(out.end_h, ref.end_h) and np.array_equal(out.end_v, ref.end_v)
    for k in range(len(H)):
        assert out.pair_segments(k) == ref.segments[k], k


def test_blosum62_local_protein_against_oracle(engine):
    import seqan_gb300 as sg
    from seqan_gb300 import workloads as W
    H, V = W.protein_pairs(60, median=200, seed=11)
    sc = sg.Blosum62(-1, -11, dtype=np.int16)
    out = sg.align_codes(H, V, sc, mode=1, traceback=True)
    ref = O.oracle_batch(O.Problem("local", 0, None, 0, 0, -11, -1, sc.matrix, 16, "aa"), H, V, traceback=True)
    assert np.array_equal(out.score, ref.score)
    for k in range(len(H)):
        assert out.pair_segments(k) == ref.segments[k], k


def test_invalid_pairs_and_empty_batch(engine):
    import seqan_gb300 as sg
    e = np.zeros(0, np.uint8)
    a = np.array([0, 1, 2, 3], np.uint8)
    out = sg.align_codes([e, a, a], [a, e, a], sg.Score(2, -3, -5, dtype=np.int16), traceback=True, cigar=True)
    assert out.score.tolist()[:2] == [-32768, -32768]
    assert out.score[2] == 8
    assert out.status.tolist()[:2] == [1, 1]
    assert out.pair_segments(0) == [] and out.pair_cigar(1) == ""
    out = sg.align_codes([], [], sg.Score(2, -3, -5))
    assert len(out.score) == 0


def test_int16_promotion_is_exact(engine):
    """Pairs whose values can leave the exact int16 range run with 32-bit cells; pairs inside it
    keep 16-bit semantics.  Score(2,-4,-1,-6): 9,000+ bp pairs can fall below the int16
    "infinity" (-16384), 300 bp pairs cannot."""
    import seqan_gb300 as sg
    Hl, Vl = _random_pairs(5, 3, 9000, 10000)
    Hs, Vs = _random_pairs(6, 3, 200, 300)
    H, V = Hl + Hs, Vl + Vs
    out = sg.align_codes(H, V, sg.Score(2, -4, -1, -6, dtype=np.int16))
    ref = O.oracle_batch(O.Problem("global", 0, None, 2, -4, -6, -1, None, 32), H, V)
    assert np.array_equal(out.score, ref.score)
    assert out.status.tolist() == [2, 2, 2, 0, 0, 0]


def test_one_vs_many(engine):
    import seqan_gb300 as sg
    H, V = _random_pairs(9, 50, 20, 80)
    h = H[0]
    got = sg.globalAlignmentScore("".join("ACGT"[c] for c in h), ["".join("ACGT"[c] for c in v) for v in V],
                                  sg.Score(2, -3, -5))
    ref = O.oracle_batch(O.Problem(), [h] * len(V), V)
    assert got.tolist() == ref.score.tolist()


def test_python_interface_gaps(engine):
    """globalAlignment over Gaps fills rows like the reference's KAT (AlignConfig<>, NW)."""
    import seqan_gb300 as sg
    gH, gV = sg.Gaps("ATGT"), sg.Gaps("ATAGAT")
    sc = sg.globalAlignment([gH], [gV], sg.Score(2, -1, -1))
    assert int(sc[0]) == 6
    assert (gH.row(), gV.row()) == ("AT-G-T", "ATAGAT")


# packed kernel: 32-row strips (split slots for the 320 longest pairs, the rest two per thread),
# 16-row strips, every pair split (32- and 16-row strips), no split slots; then the warp kernel
@pytest.mark.parametrize("flags", [32, 2, 32 | 64, 2 | 64, 32 | 128, 0])
@pytest.mark.parametrize("fe", [0, 1, 2, 4, 8, 9, 6, 15, 5, 10])
def test_packed_kernel_against_oracle(engine, flags, fe):
    """The packed 16-bit kernel: two-pair slots (uneven lengths in one slot, odd pair count) and
    split slots (one pair, two strips at once), Dna5 codes (N = 4), both gap models, every
    tracked-cell rule."""
    import seqan_gb300 as sg
    rng = np.random.default_rng(1000 + fe)
    H = [rng.integers(0, 5, rng.integers(1, 260)).astype(np.uint8) for _ in range(333)]
    V = [np.where(rng.random(len(h)) < 0.15, rng.integers(0, 5, len(h)), h).astype(np.uint8)
         if rng.random() < 0.6 else rng.integers(0, 5, rng.integers(1, 260)).astype(np.uint8) for h in H]
    cfg = sg.AlignConfig(bool(fe & 1), bool(fe & 2), bool(fe & 4), bool(fe & 8))
    for (mt, mm, go, ge) in [(2, -4, -6, -1), (2, -3, -5, -5), (5, -4, -10, -1)]:
        for dtype, bits in ((np.int16, 16), (np.int32, 32)):
            sc = sg.Score(mt, mm, ge, go, dtype=dtype)
            out = sg.align_codes(H, V, sc, config=cfg, alphabet_size=5, flags=flags)
            gen = sg.align_codes(H, V, sc, config=cfg, alphabet_size=5, flags=1)
            ref = O.oracle_batch(O.Problem("global", fe, None, mt, mm, go, ge, None, bits), H, V)
            assert np.array_equal(out.score, ref.score) and np.array_equal(gen.score, ref.score)
            assert np.array_equal(out.end_h, ref.end_h) and np.array_equal(out.end_v, ref.end_v)
            assert np.array_equal(out.status, gen.status)


@pytest.mark.parametrize("flags", [4, 8, 1 | 8])
def test_plain_buckets_and_direct_launch(engine, flags):
    """The plain per-bucket form and direct (non-graph) launches give the same results."""
    import seqan_gb300 as sg
    H, V = _random_pairs(77, 500, 1, 300)
    sc = sg.Score(2, -4, -1, -6, dtype=np.int16)
    out = sg.align_codes(H, V, sc, alphabet_size=4, flags=flags)
    ref = O.oracle_batch(O.Problem("global", 0, None, 2, -4, -6, -1, None, 16), H, V)
    assert np.array_equal(out.score, ref.score)
    assert np.array_equal(out.end_h, ref.end_h) and np.array_equal(out.end_v, ref.end_v)


def test_device_resident_plan_replays_graph(engine):
    """gba_plan_execute twice on the same device buffers (the second run replays the captured
    graph) gives the oracle's scores both times."""
    import ctypes as C
    import seqan_gb300 as sg
    from seqan_gb300 import _native as N
    L, h = N.lib(), engine.handle
    H, V = _random_pairs(78, 700, 50, 300)
    sh, oh = sg.align._concat(H)
    sv, ov = sg.align._concat(V)
    n = len(H)
    params = sg.align.make_params(sg.Score(2, -4, -1, -6, dtype=np.int16), 0, None, None,
                                  N.GBA_OUT_SCORE | N.GBA_OUT_END, alphabet_size=4)
    hb = N.GbaBatch(n, sh.ctypes.data, oh.ctypes.data, sv.ctypes.data, ov.ctypes.data, 0, 0)
    ptrs = []

    def dev(nbytes, src=None):
        p = C.c_void_p()
        engine.check(L.gba_device_alloc(h, C.byref(p), nbytes), "alloc")
        if src is not None:
            engine.check(L.gba_copy_to_device(h, p, src.ctypes.data, nbytes), "h2d")
        ptrs.append(p)
        return p

    d_sh, d_sv = dev(sh.nbytes, sh), dev(sv.nbytes, sv)
    d_sc, d_eh, d_ev = dev(4 * n), dev(4 * n), dev(4 * n)
    plan = C.c_void_p()
    engine.check(L.gba_plan_create(h, C.byref(params), C.byref(hb), C.byref(plan)), "plan")
    db = N.GbaBatch(n, d_sh, None, d_sv, None, 0, 0)
    dr = N.GbaResult()
    dr.score, dr.end_h, dr.end_v = d_sc, d_eh, d_ev
    ref = O.oracle_batch(O.Problem("global", 0, None, 2, -4, -6, -1, None, 16), H, V)
    for _ in range(2):
        engine.check(L.gba_plan_execute(h, plan, C.byref(db), C.byref(dr)), "execute")
        got = np.zeros(n, np.int32)
        engine.check(L.gba_copy_to_host(h, got.ctypes.data, d_sc, 4 * n), "d2h")
        assert np.array_equal(got, ref.score)
    L.gba_plan_destroy(h, plan)
    for p in ptrs:
        L.gba_device_free(h, p)


def _band_cases(seed, count):
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(count):
        m, n = int(rng.integers(1, 45)), int(rng.integers(1, 45))
        h = rng.integers(0, 4, m).astype(np.uint8)
        v = h[:n].copy() if (n <= m and rng.random() < 0.5) else rng.integers(0, 4, n).astype(np.uint8)
        lo = int(rng.integers(-n - 2, m + 2))
        up = lo + int(rng.choice([1, 2, 3, 5, 8, 13, 33, 60])) - 1
        out.append((h, v, lo, up))
    return out


@pytest.mark.parametrize("mode,fe", [("global", f) for f in (0, 1, 2, 4, 8, 9, 6, 15)] + [("local", 0)])
@pytest.mark.parametrize("scheme", [(2, -3, -5, -5), (2, -4, -6, -1), (1, -1, -2, -1)])
def test_banded_against_oracle(engine, mode, fe, scheme):
    """Banded DP: every band phase (top, middle, full, bottom, final), one-diagonal bands and
    the single-cell bands; scores, best cells, segment lists and CIGARs."""
    import seqan_gb300 as sg
    mt, mm, go, ge = scheme
    cfg = sg.AlignConfig(bool(fe & 1), bool(fe & 2), bool(fe & 4), bool(fe & 8))
    md = 1 if mode == "local" else 0
    for (h, v, lo, up) in _band_cases(hash((mode, fe, scheme)) % 1000, 60):
        out = sg.align_codes([h], [v], sg.Score(mt, mm, ge, go, dtype=np.int32), mode=md, config=cfg,
                             band=(lo, up), traceback=True, cigar=True)
        ref = O.oracle_batch(O.Problem(mode, fe, (lo, up), mt, mm, go, ge, None, 32), [h], [v], traceback=True)
        assert out.score[0] == ref.score[0], (lo, up, len(h), len(v))
        if ref.valid[0]:
            assert (out.end_h[0], out.end_v[0]) == (ref.end_h[0], ref.end_v[0]), (lo, up, len(h), len(v))
            assert out.pair_segments(0) == ref.segments[0], (lo, up, len(h), len(v))
            assert out.pair_cigar(0) == O.cigar_string(ref.segments[0])


def test_banded_read_mapping_batch(engine):
    """The read-to-reference verification shape: 150 bp reads with substitutions and indels
    against 170 bp windows, band (-6, 26), free reference overhang, int16, CIGARs."""
    import seqan_gb300 as sg
    from seqan_gb300 import workloads as W
    wins, reads = W.read_windows(2000, ref_len=1_000_000, seed=21)
    sc = sg.Score(2, -4, -1, -6, dtype=np.int16)
    out = sg.align_codes(wins, reads, sc, config=sg.AlignConfig(True, False, False, True), band=(-6, 26),
                         traceback=True, cigar=True)
    ref = O.oracle_batch(O.Problem("global", 9, (-6, 26), 2, -4, -6, -1, None, 16), wins, reads, traceback=True)
    assert np.array_equal(out.score, ref.score)
    for k in range(len(wins)):
        assert out.pair_cigar(k) == O.cigar_string(ref.segments[k]), k


@pytest.mark.parametrize("mode,fe", [("global", 0), ("global", 9), ("global", 6), ("global", 15), ("local", 0)])
def test_warp_kernel_multiband_traceback(engine, mode, fe):
    """One warp per pair over several 256-row bands (lengths up to 1200), with tracebacks;
    against the oracle and against the one-pair-per-thread kernel."""
    import seqan_gb300 as sg
    H, V = _random_pairs(300 + fe, 40, 1, 1200)
    cfg = sg.AlignConfig(bool(fe & 1), bool(fe & 2), bool(fe & 4), bool(fe & 8))
    md = 1 if mode == "local" else 0
    for (mt, mm, go, ge) in [(2, -4, -6, -1), (2, -3, -5, -5)]:
        sc = sg.Score(mt, mm, ge, go, dtype=np.int32)
        out = sg.align_codes(H, V, sc, mode=md, config=cfg, traceback=True, cigar=True)
        gen = sg.align_codes(H, V, sc, mode=md, config=cfg, traceback=True, flags=1)
        ref = O.oracle_batch(O.Problem(mode, fe, None, mt, mm, go, ge, None, 32), H, V, traceback=True)
        assert np.array_equal(out.score, ref.score) and np.array_equal(gen.score, ref.score)
        assert np.array_equal(out.end_h, ref.end_h) and np.array_equal(out.end_v, ref.end_v)
        for k in range(len(H)):
            assert out.pair_segments(k) == ref.segments[k], k
            assert gen.pair_segments(k) == ref.segments[k], k
            assert out.pair_cigar(k) == O.cigar_string(ref.segments[k]), k


def test_warp_kernel_protein_local(engine):
    import seqan_gb300 as sg
    from seqan_gb300 import workloads as W
    H, V = W.protein_pairs(150, seed=31)
    sc = sg.Blosum62(-1, -11, dtype=np.int16)
    out = sg.align_codes(H, V, sc, mode=1, traceback=True)
    ref = O.oracle_batch(O.Problem("local", 0, None, 0, 0, -11, -1, sc.matrix, 16, "aa"), H, V, traceback=True)
    assert np.array_equal(out.score, ref.score)
    for k in range(len(H)):
        assert out.pair_segments(k) == ref.segments[k], k


def _long_mix(seed):
    """A few long related pairs (1,000-6,000 bp and one 10,000 bp pair) mixed with short ones."""
    from seqan_gb300 import workloads as W
    rng = np.random.default_rng(seed)
    H, V = [], []
    for L in [10_000] + list(rng.integers(1000, 6001, 5)) + list(rng.integers(1, 400, 20)):
        h = rng.integers(0, 4, int(L)).astype(np.uint8)
        H.append(h)
        V.append(W.mutate(rng, h, 0.05, 0.01))
    order = rng.permutation(len(H))
    return [H[i] for i in order], [V[i] for i in order]


@pytest.mark.parametrize("mode,fe", [("global", 0), ("global", 9), ("global", 15), ("local", 0)])
def test_long_pairs_pipelined_bands_and_warp_traceback(engine, mode, fe):
    """Pairs of up to 40 bands, whose bands run on different warps and whose tracebacks are
    walked by a warp through shared-memory tiles, mixed with short pairs; against the oracle."""
    import seqan_gb300 as sg
    H, V = _long_mix(700 + fe)
    cfg = sg.AlignConfig(bool(fe & 1), bool(fe & 2), bool(fe & 4), bool(fe & 8))
    md = 1 if mode == "local" else 0
    for (mt, mm, go, ge), bits in [((2, -4, -6, -1), 16), ((2, -3, -5, -5), 32)]:
        sc = sg.Score(mt, mm, ge, go, dtype=np.int16 if bits == 16 else np.int32)
        out = sg.align_codes(H, V, sc, mode=md, config=cfg, traceback=True, cigar=True)
        # int16 scoring: pairs past the exact int16 range (the 10,000 bp one) are promoted to
        # 32-bit cells, the others keep exact 16-bit values -- both equal 32-bit arithmetic.
        ref = O.oracle_batch(O.Problem(mode, fe, None, mt, mm, go, ge, None, 32), H, V, traceback=True)
        assert np.array_equal(out.score, ref.score)
        assert np.array_equal(out.end_h, ref.end_h) and np.array_equal(out.end_v, ref.end_v)
        for k in range(len(H)):
            assert out.pair_segments(k) == ref.segments[k], k
            assert out.pair_cigar(k) == O.cigar_string(ref.segments[k]), k
        score_only = sg.align_codes(H, V, sc, mode=md, config=cfg)
        assert np.array_equal(score_only.score, ref.score)


@pytest.mark.parametrize("mode,fe", [("global", 0), ("global", 9), ("local", 0)])
def test_many_narrow_multiband_pairs_run_bands_in_order(engine, mode, fe):
    """20,000 pairs of 257-330 bp (two bands each): more pairs than twice the resident warps at
    any occupancy, so each pair's warp runs its bands in order; against the oracle (scores and
    ends of all pairs, segments of every 40th)."""
    import seqan_gb300 as sg
    rng = np.random.default_rng(900 + fe)
    H = [rng.integers(0, 4, int(L)).astype(np.uint8) for L in rng.integers(257, 331, 20000)]
    V = [h.copy() for h in H]
    for v in V:
        sub = rng.random(len(v)) < 0.08
        v[sub] = (v[sub] + 1) % 4
    cfg = sg.AlignConfig(bool(fe & 1), bool(fe & 2), bool(fe & 4), bool(fe & 8))
    md = 1 if mode == "local" else 0
    sc = sg.Score(2, -4, -1, -6, dtype=np.int32)
    out = sg.align_codes(H, V, sc, mode=md, config=cfg, traceback=True)
    pb = O.Problem(mode, fe, None, 2, -4, -6, -1, None, 32)
    ref = O.oracle_batch(pb, H, V)
    assert np.array_equal(out.score, ref.score)
    assert np.array_equal(out.end_h, ref.end_h) and np.array_equal(out.end_v, ref.end_v)
    sub_idx = list(range(0, len(H), 40))
    reft = O.oracle_batch(pb, [H[k] for k in sub_idx], [V[k] for k in sub_idx], traceback=True)
    for i, k in enumerate(sub_idx):
        assert out.pair_segments(k) == reft.segments[i], k


@pytest.mark.parametrize("fe", [0, 9])
def test_chunked_large_score_batch(engine, fe):
    """450,000 pairs, score only: gba_align_batch plans and runs the batch as contiguous chunks
    (each planned while the previous one runs); scores, ends and statuses against the oracle,
    including a few pairs that need 32-bit cells."""
    import seqan_gb300 as sg
    rng = np.random.default_rng(1200 + fe)
    H = [rng.integers(0, 4, int(L)).astype(np.uint8) for L in rng.integers(20, 41, 450000)]
    V = [h.copy() for h in H]
    for v in V[::3]:
        sub = rng.random(len(v)) < 0.1
        v[sub] = (v[sub] + 1) % 4
    for k in (5, 230000, 449999):         # past the exact int16 range: promoted
        H[k] = rng.integers(0, 4, 9500).astype(np.uint8)
        V[k] = rng.integers(0, 4, 9400).astype(np.uint8)
    cfg = sg.AlignConfig(bool(fe & 1), bool(fe & 2), bool(fe & 4), bool(fe & 8))
    out = sg.align_codes(H, V, sg.Score(2, -4, -1, -6, dtype=np.int16), config=cfg, alphabet_size=4)
    ref = O.oracle_batch(O.Problem("global", fe, None, 2, -4, -6, -1, None, 32), H, V)
    assert np.array_equal(out.score, ref.score)
    assert np.array_equal(out.end_h, ref.end_h) and np.array_equal(out.end_v, ref.end_v)
    assert out.status[[5, 230000, 449999]].tolist() == [2, 2, 2] and (out.status == 2).sum() == 3
