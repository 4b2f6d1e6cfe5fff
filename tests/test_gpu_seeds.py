"""Seed extension on the GPU through gba_extend_seeds: identical to the reference's extendSeed
(fixtures and known answers) and to the oracle on large seeded batches, including seeds whose
x-drop band outgrows the shared-memory ring (fallback kernel), shared databases, and the
device-pointer entry point."""
import ctypes as C

import numpy as np
import pytest

from oracle import oracle as O
from tests import golden_cases as G
from tests.test_seeds_oracle import KNOWN, SEED_CASES, known_problem, seed_case_id, seed_case_inputs

pytestmark = pytest.mark.gpu

B62 = np.array(G.load("blosum62.json")["matrix"], dtype=np.int32)


def engine_score(sp):
    import seqan_gb300 as sg
    if sp.matrix is not None:
        return sg.Blosum62(sp.gap, sp.gap)
    return sg.Score(sp.match, sp.mismatch, sp.gap)


def run_gpu(sp, H, V, seeds, seed_h=None, seed_v=None, scores=False):
    from seqan_gb300 import seeds as S
    return S.extend_seeds(np.asarray(seeds, dtype=np.int64).reshape(-1, 6), H, V, sp.direction,
                          engine_score(sp), sp.xdrop, sp.method, seed_h=seed_h, seed_v=seed_v,
                          alphabet="aa" if sp.alphabet == "aa" else "dna5", return_scores=scores)


@pytest.mark.parametrize("case", SEED_CASES, ids=[seed_case_id(c) for c in SEED_CASES])
def test_fixtures_through_c_abi(engine, case):
    sp, H, V = seed_case_inputs(case)
    pos = case["pair_of_seed"]
    got, xs = run_gpu(sp, H, V, case["seeds"], pos, pos, scores=True)
    assert got.tolist() == case["extended"]
    if case["xscores"] is not None:
        assert xs.tolist() == case["xscores"]


@pytest.mark.parametrize("case", KNOWN, ids=[f"{c[0]}-{c[1]}-{c[2][:8]}-{c[4]}" for c in KNOWN])
def test_known_answers_with_extendSeed(engine, case):
    from seqan_gb300 import seeds as S
    sp, h, v, seed, want = known_problem(case)
    s = S.Seed(*seed)
    tag = {O.MATCH_EXTEND: S.MatchExtend(), O.UNGAPPED_XDROP: S.UnGappedXDrop(), O.GAPPED_XDROP: S.GappedXDrop()}
    if sp.method == O.MATCH_EXTEND:
        S.extendSeed(s, h, v, sp.direction, tag[sp.method])
    else:
        S.extendSeed(s, h, v, sp.direction, engine_score(sp), sp.xdrop, tag[sp.method],
                     alphabet="aa" if sp.alphabet == "aa" else "dna5")
    assert tuple(s.as_row()[:len(want)]) == tuple(want)


@pytest.mark.parametrize("method", [O.MATCH_EXTEND, O.UNGAPPED_XDROP, O.GAPPED_XDROP])
@pytest.mark.parametrize("direction", [O.EXTEND_LEFT, O.EXTEND_RIGHT, O.EXTEND_BOTH])
def test_read_mapping_batch_against_oracle(engine, method, direction):
    """60,000 read seeds (150 bp reads, 250 bp windows, 19-mers): every seed equals the oracle."""
    from seqan_gb300 import workloads as W
    wins, reads, seeds, pos = W.seed_windows(60_000, ref_len=2_000_000, seed=11)
    sp = O.SeedProblem(method, direction, 1, -2, -2, 20)
    arr = O.seeds_array(seeds)
    got, xs = run_gpu(sp, wins, reads, arr, scores=True)
    ref, rx = O.oracle_extend_seeds(sp, wins, reads, arr)
    assert np.array_equal(got, ref)
    if method == O.GAPPED_XDROP:
        assert np.array_equal(xs, rx)
        # the seeds really grew across the reads (one side only for LEFT / RIGHT)
        assert (got[:, 2] - got[:, 0]).mean() > (100 if direction == O.EXTEND_BOTH else 60)


@pytest.mark.parametrize("xdrop,gap,mismatch,match,fallback", [
    (20, -1, -1, 2, None), (30, -1, -1, 2, None), (45, -1, -1, 2, None), (60, -3, -2, 2, None),
    (120, -1, -1, 2, "all"),   # X / |gap| > 48: every seed on the global-memory ring
    (20, -1, -1, 3, "some"),   # positive expected score: live ranges outgrow the 32-slot ring
])
def test_wide_bands_use_the_fallback_exactly(engine, xdrop, gap, mismatch, match, fallback):
    """Drop-offs whose band outgrows the 32- or 64-slot ring on some seeds, and one whose band
    runs every seed on the global fallback: results stay identical to the oracle."""
    import seqan_gb300 as sg
    from seqan_gb300 import workloads as W
    rng = np.random.default_rng(xdrop)
    H, V, seeds = [], [], []
    for k in range(4000):
        L = int(rng.integers(50, 400))
        h = rng.integers(0, 4, L).astype(np.uint8)
        v = W.mutate(rng, h, float(rng.uniform(0.0, 0.35)), float(rng.uniform(0.0, 0.08)))
        if k % 5 == 0:
            v = rng.integers(0, 4, int(rng.integers(30, 400))).astype(np.uint8)
        H.append(h)
        V.append(v)
        sl = int(rng.integers(0, min(len(h), len(v), 20) + 1))
        bh = int(rng.integers(0, len(h) - sl + 1))
        bv = min(bh, len(v) - sl)
        seeds.append((bh, bv, sl))
    sp = O.SeedProblem(O.GAPPED_XDROP, O.EXTEND_BOTH, match, mismatch, gap, xdrop)
    arr = O.seeds_array(seeds)
    got, xs = run_gpu(sp, H, V, arr, scores=True)
    st = sg.default_context().stats()
    ref, rx = O.oracle_extend_seeds(sp, H, V, arr)
    assert np.array_equal(got, ref)
    assert np.array_equal(xs, rx)
    if fallback == "all":
        assert st.seed_ring == 0 and st.seed_fallbacks == len(arr)
    else:
        assert st.seed_ring == (32 if xdrop // -gap <= 20 else 64)
        if fallback == "some":
            assert 0 < st.seed_fallbacks < len(arr)


def test_protein_blosum62_batch(engine):
    from seqan_gb300 import workloads as W
    H, V = W.protein_pairs(3000, seed=21, related=0.8, identity=0.6)
    rng = np.random.default_rng(4)
    seeds = []
    for h, v in zip(H, V):
        sl = int(rng.integers(0, min(len(h), len(v), 8) + 1))
        bh = int(rng.integers(0, min(len(h), len(v)) - sl + 1))
        seeds.append((bh, bh, sl))
    for gap, x in ((-9, 10), (-11, 25), (-4, 60)):
        sp = O.SeedProblem(O.GAPPED_XDROP, O.EXTEND_BOTH, 0, 0, gap, x, B62, "aa")
        arr = O.seeds_array(seeds)
        got, xs = run_gpu(sp, H, V, arr, scores=True)
        ref, rx = O.oracle_extend_seeds(sp, H, V, arr)
        assert np.array_equal(got, ref) and np.array_equal(xs, rx), (gap, x)


def test_shared_database_many_queries(engine):
    """One 200 kbp database, 20,000 reads with seeds at their origins (seed_h all 0)."""
    from seqan_gb300 import workloads as W
    rng = np.random.default_rng(8)
    genome = rng.integers(0, 4, 200_000).astype(np.uint8)
    origins = rng.integers(0, len(genome) - 200, 20_000)
    reads = [W.mutate(rng, genome[o:o + 150], 0.04, 0.004) for o in origins]
    seeds = [(int(o) + 60, 60, 15) for o in origins]
    sp = O.SeedProblem(O.GAPPED_XDROP, O.EXTEND_BOTH, 1, -1, -1, 12)
    arr = O.seeds_array(seeds)
    sh = np.zeros(len(arr), np.int32)
    sv = np.arange(len(arr), dtype=np.int32)
    got, xs = run_gpu(sp, [genome], reads, arr, seed_h=sh, seed_v=sv, scores=True)
    ref, rx = O.oracle_extend_seeds(sp, [genome], reads, arr, seed_h=sh, seed_v=sv)
    assert np.array_equal(got, ref) and np.array_equal(xs, rx)


def test_refusals(engine):
    import seqan_gb300 as sg
    from seqan_gb300 import _native as N
    from seqan_gb300 import seeds as S
    h = np.array([0, 1, 2, 3], np.uint8)
    with pytest.raises(N.GbaError) as e:       # seed past the end
        S.extend_seeds([S.Seed(3, 0, 2)], [h], [h], S.EXTEND_BOTH, sg.Score(1, -1, -1), 5, S.GappedXDrop)
    assert e.value.status == N.GBA_EINVAL
    with pytest.raises(N.GbaError) as e:       # mismatch below gap: the reference overflows int
        S.extend_seeds([S.Seed(1, 1, 1)], [h], [h], S.EXTEND_BOTH, sg.Score(1, -3, -2), 5, S.GappedXDrop)
    assert e.value.status == N.GBA_EUNSUPPORTED
    with pytest.raises(N.GbaError) as e:       # UnGappedXDrop's left walk would start past the end
        S.extend_seeds([S.Seed(4, 4, 0)], [h], [h], S.EXTEND_LEFT, sg.Score(1, -1, -1), 5, S.UnGappedXDrop)
    assert e.value.status == N.GBA_EINVAL
    with pytest.raises(ValueError):            # GappedXDrop asserts gap open == extend
        S.extend_seeds([S.Seed(1, 1, 1)], [h], [h], S.EXTEND_BOTH, sg.Score(1, -1, -1, -3), 5, S.GappedXDrop)
    # the context stays usable
    out = S.extend_seeds([S.Seed(1, 1, 1)], [h], [h], S.EXTEND_BOTH, sg.Score(1, -1, -1), 5, S.GappedXDrop)
    assert out.tolist() == [[0, 0, 4, 4, -1, 1]]


def test_device_entry_point(engine):
    """gba_extend_seeds_device on device buffers equals the host call; a seed outside its
    sequences is reported by gba_synchronize."""
    from seqan_gb300 import _native as N
    from seqan_gb300 import workloads as W
    L = N.lib()
    ctx = engine
    wins, reads, seeds, pos = W.seed_windows(5000, ref_len=1_000_000, seed=3)
    arr = O.seeds_array(seeds)
    sh, oh = O.concat(wins)
    sv, ov = O.concat(reads)
    bufs = []

    def dev(a):
        p = C.c_void_p()
        ctx.check(L.gba_device_alloc(ctx.handle, C.byref(p), max(a.nbytes, 1)), "alloc")
        ctx.check(L.gba_copy_to_device(ctx.handle, p, a.ctypes.data, a.nbytes), "h2d")
        bufs.append(p)
        return p

    try:
        d_sh, d_oh, d_sv, d_ov, d_seeds = dev(sh), dev(oh), dev(sv), dev(ov), dev(arr)
        d_sc = dev(np.zeros((len(arr), 2), np.int32))
        b = N.GbaSeedBatch(len(wins), d_sh, d_oh, len(reads), d_sv, d_ov, len(arr), None, None,
                           int(max(len(r) for r in reads)))
        p = N.GbaExtendParams(N.GBA_GAPPED_XDROP, N.GBA_EXTEND_BOTH, 20, 1, -2, -2, None, 0, 0)
        ctx.check(L.gba_extend_seeds_device(ctx.handle, C.byref(p), C.byref(b), d_seeds, d_sc), "extend")
        ctx.check(L.gba_synchronize(ctx.handle), "sync")
        out = np.zeros_like(arr)
        sc = np.zeros((len(arr), 2), np.int32)
        ctx.check(L.gba_copy_to_host(ctx.handle, out.ctypes.data, d_seeds, out.nbytes), "d2h")
        ctx.check(L.gba_copy_to_host(ctx.handle, sc.ctypes.data, d_sc, sc.nbytes), "d2h")
        ref, rx = O.oracle_extend_seeds(O.SeedProblem(O.GAPPED_XDROP, O.EXTEND_BOTH, 1, -2, -2, 20), wins, reads,
                                        arr)
        assert np.array_equal(out, ref) and np.array_equal(sc, rx)
        bad = arr.copy()
        bad[7, 2] = 10_000          # end past its window
        ctx.check(L.gba_copy_to_device(ctx.handle, d_seeds, bad.ctypes.data, bad.nbytes), "h2d")
        ctx.check(L.gba_extend_seeds_device(ctx.handle, C.byref(p), C.byref(b), d_seeds, d_sc), "extend")
        assert L.gba_synchronize(ctx.handle) == N.GBA_EINVAL
        ctx.check(L.gba_synchronize(ctx.handle), "sync after error")
    finally:
        for p_ in bufs:
            L.gba_device_free(ctx.handle, p_)
