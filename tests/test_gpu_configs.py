"""GPU parity on the benchmark configurations at their stated sizes.

Each test builds the seeded workload the benchmark times (same generators, same seeds), runs it
through the C-ABI and compares every pair's results with the oracle: scores and best cells, and
where the configuration asks for them begin positions, the raw TraceSegment_ lists and the CIGAR
words.  Integer arithmetic throughout, so every comparison is exact.  The routing the timed runs
take (packed kernel with split slots and each tiling variant, graph replay of a device-resident
plan, the plain per-bucket form, the warp kernel's band pipeline, the banded kernel) runs at the
same batch shapes as in the benchmark, because the routing depends on the batch size and the
length distribution.

Reference rules the results follow: first maximum in column-major order
(align/dp_scout.h:166-180), traceback order and head/tail segments
(align/dp_traceback_impl.h:489-546), CIGAR of the Gaps (bam_io/cigar.h:261-339).
"""
import time

import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu


def _flags():
    from seqan_gb300 import _native as N
    return N


def _assert_scores(out, ref, what):
    bad = np.nonzero((out.score != ref.score) | (out.end_h != ref.end_h) | (out.end_v != ref.end_v))[0]
    assert bad.size == 0, f"{what}: {bad.size} pairs differ, first {bad[:5].tolist()}"


def _assert_segments(out, ref, what):
    n = len(out.score)
    assert np.array_equal(out.segment_offsets, ref.seg_offsets), f"{what}: segment counts differ"
    total = int(ref.seg_offsets[-1])
    got = out.segments[:total]
    if not np.array_equal(got, ref.seg_flat):
        row = int(np.nonzero((got != ref.seg_flat).any(axis=1))[0][0])
        pair = int(np.searchsorted(ref.seg_offsets, row, side="right") - 1)
        raise AssertionError(f"{what}: segments differ, first at pair {pair} of {n}")


# --- Plain global score, 1024 pairs of 150 bp uniform DNA, Score<int,Simple>(2,-3,-5), int32 ---

def test_linear_dna_1024x150(engine):
    import seqan_gb300 as sg
    from seqan_gb300 import workloads as W
    N = _flags()
    H, V = W.uniform_dna_pairs(1024, 150, seed=1)
    score = sg.Score(2, -3, -5, dtype=np.int32)
    ref = O.oracle_batch(O.Problem("global", 0, None, 2, -3, -5, -5, None, 32), H, V)
    for flags in (0, N.GBA_FLAG_GENERAL_KERNEL, N.GBA_FLAG_PLAIN_BUCKETS):
        out = sg.align_codes(H, V, score, alphabet_size=4, flags=flags)
        _assert_scores(out, ref, f"flags {flags}")
    out = sg.align.align_codes_resident(H, V, score, alphabet_size=4)
    _assert_scores(out, ref, "device-resident plan")


# --- Batched affine global DNA, 100,000 pairs of 100-300 bp, Score<int16_t,Simple>(2,-4,-1,-6) ---

@pytest.fixture(scope="module")
def affine_100k():
    from seqan_gb300 import workloads as W
    H, V = W.mutated_dna_pairs(100_000, 100, 300, 0.05, 0.01, seed=2)
    ref = O.oracle_batch(O.Problem("global", 0, None, 2, -4, -6, -1, None, 16), H, V)
    return H, V, ref


def test_affine_dna_100k_autotuned_graph_replay(engine, affine_100k):
    """The timed path of the headline benchmark: a device-resident plan with GBA_FLAG_AUTOTUNE
    (every tiling variant runs once at the first execution), then a graph replay."""
    import seqan_gb300 as sg
    N = _flags()
    H, V, ref = affine_100k
    score = sg.Score(2, -4, -1, -6, dtype=np.int16)
    out = sg.align.align_codes_resident(H, V, score, alphabet_size=4, flags=N.GBA_FLAG_AUTOTUNE, runs=3)
    _assert_scores(out, ref, "autotuned plan")
    st = sg.default_context().stats()
    assert st.dp_kernels & N.GBA_KERNEL_PACKED
    out = sg.align_codes(H, V, score, alphabet_size=4, flags=N.GBA_FLAG_AUTOTUNE)
    _assert_scores(out, ref, "gba_align_batch")
    assert (out.status == 0).all()


@pytest.mark.parametrize("variant", range(1, 6))
def test_affine_dna_100k_each_tiling_variant(engine, affine_100k, variant):
    import seqan_gb300 as sg
    H, V, ref = affine_100k
    out = sg.align_codes(H, V, sg.Score(2, -4, -1, -6, dtype=np.int16), alphabet_size=4, tile_variant=variant)
    _assert_scores(out, ref, f"tiling variant {variant}")
    assert sg.default_context().stats().tile_rows in (16, 24, 32)


@pytest.mark.parametrize("which", ["split_all", "no_split", "plain_buckets", "plain_general"])
def test_affine_dna_100k_forms(engine, affine_100k, which):
    import seqan_gb300 as sg
    N = _flags()
    H, V, ref = affine_100k
    flags = {"split_all": N.GBA_FLAG_PACKED_SPLIT, "no_split": N.GBA_FLAG_PACKED_NO_SPLIT,
             "plain_buckets": N.GBA_FLAG_PLAIN_BUCKETS | N.GBA_FLAG_NO_GRAPH,
             "plain_general": N.GBA_FLAG_PLAIN_BUCKETS | N.GBA_FLAG_GENERAL_KERNEL | N.GBA_FLAG_NO_GRAPH}[which]
    out = sg.align_codes(H, V, sg.Score(2, -4, -1, -6, dtype=np.int16), alphabet_size=4, flags=flags)
    _assert_scores(out, ref, which)
    kernels = sg.default_context().stats().dp_kernels
    assert kernels & (N.GBA_KERNEL_STRIP if which == "plain_general" else N.GBA_KERNEL_PACKED)


# --- Local protein with traceback, 20,000 pairs, Blosum62(-1,-11), int16 ---

def test_protein_local_traceback_20k(engine):
    import seqan_gb300 as sg
    from seqan_gb300 import workloads as W
    N = _flags()
    H, V = W.protein_pairs(20_000, seed=3)
    score = sg.Blosum62(-1, -11, dtype=np.int16)
    ref = O.oracle_batch(O.Problem("local", 0, None, 0, 0, -11, -1, score.matrix, 16, "aa"), H, V,
                         traceback=True, flat=True)
    for flags in (0, N.GBA_FLAG_PLAIN_BUCKETS):
        out = sg.align_codes(H, V, score, mode=1, traceback=True, alphabet_size=27, flags=flags)
        _assert_scores(out, ref, f"flags {flags}")
        assert np.array_equal(out.begin_h, ref.begin_h) and np.array_equal(out.begin_v, ref.begin_v)
        _assert_segments(out, ref, f"flags {flags}")
        assert sg.default_context().stats().dp_kernels & (N.GBA_KERNEL_WARP | N.GBA_KERNEL_WARP16)


# --- Banded semi-global read verification, 1,000,000 reads vs 170 bp windows, band (-6, 26) ---

def test_banded_reads_1m_cigar(engine):
    import seqan_gb300 as sg
    from seqan_gb300 import workloads as W
    N = _flags()
    wins, reads = W.read_windows(1_000_000, seed=4)
    score = sg.Score(2, -4, -1, -6, dtype=np.int16)
    cfg = sg.AlignConfig(True, False, False, True)
    ref = O.oracle_batch(O.Problem("global", cfg.bits, (-6, 26), 2, -4, -6, -1, None, 16), wins, reads,
                         traceback=True, flat=True)
    out = sg.align_codes(wins, reads, score, config=cfg, band=(-6, 26), traceback=True, cigar=True, alphabet_size=4)
    _assert_scores(out, ref, "banded")
    _assert_segments(out, ref, "banded")
    words, coff = O.cigar_words_flat(ref.seg_flat, ref.seg_offsets)
    assert np.array_equal(out.cigar_offsets, coff)
    assert np.array_equal(out.cigar[:len(words)], words)
    assert sg.default_context().stats().dp_kernels & N.GBA_KERNEL_BANDED


# --- Serving: Poisson arrivals at 50,000 req/s, mixed lengths incl. 10,000 x 10,000 bp ---

def test_serving_mixed_stream_with_10kbp_pairs(engine):
    """2,000 requests of the serving workload's length mix (90% 100-500 bp, 9% 1-5 kbp, 1%
    10 kbp) arrive at 50,000 req/s through the server with traceback; every result equals the
    oracle's.  The 10 kbp pairs leave the exact int16 range and come back promoted to 32-bit
    cells (their reference result is Score<int32_t, ...>'s)."""
    import threading
    import seqan_gb300 as sg
    from seqan_gb300 import workloads as W
    from seqan_gb300.serving import Server
    n = 2000
    rng = np.random.Generator(np.random.PCG64(7))
    lens = W.serving_lengths(n, seed=7)
    lens[:3] = 10_000   # at least a few 10 kbp pairs in this short stream
    H, V = [], []
    for L in lens:
        h = rng.integers(0, 4, size=int(L), dtype=np.uint8)
        H.append(h)
        V.append(W.mutate(rng, h, 0.05, 0.01))
    gaps = np.random.Generator(np.random.PCG64(8)).exponential(1 / 50_000, size=n)
    at = np.cumsum(gaps) - gaps[0]
    done = {}
    with Server(sg.Score(2, -4, -1, -6, dtype=np.int16), traceback=True, streams=8, max_batch_pairs=4096,
                hbm_budget_bytes=64 << 30) as srv:
        rc = []
        th = threading.Thread(target=lambda: rc.append(srv.submit_schedule(H, V, at)))
        th.start()
        t0 = time.time()
        while len(done) < n:
            for r in srv.poll():
                done[r.tag] = r
            assert time.time() - t0 < 300, f"{len(done)} of {n} requests finished"
            time.sleep(0.001)
        th.join()
    assert rc == [0]
    ref = O.oracle_batch(O.Problem("global", 0, None, 2, -4, -6, -1, None, 32), H, V, traceback=True)
    for k in range(n):
        r = done[k]
        long_pair = len(H[k]) >= 10_000
        assert r.status == (2 if long_pair else 0), k
        assert (r.score, r.end_h, r.end_v) == (ref.score[k], ref.end_h[k], ref.end_v[k]), k
        assert r.segments == ref.segments[k], k
