"""GPU parity of the packed 16-bit warp kernel (k_dp_warp2: 64 strips per warp in int16x2 halves,
4-bit trace) against the oracle.

GBA_FLAG_WARP16 routes every eligible pair (16-bit cells in the exact int16 range, fewer than 1024
columns, at most 4096 rows) to it even in small batches, so every AlignConfig, local mode, linear and
affine gaps, Simple and Blosum62 scores and multi-band pairs (256-row bands; last bands of 64, 128 or
256 rows) are covered; the same batches through the 32-bit warp kernel (GBA_FLAG_NO_WARP16) must give
identical results.  Exact comparisons: scores, best cells, begin positions, TraceSegment_ lists,
CIGARs."""
import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu

SCHEMES = [(2, -3, -5, -5), (2, -4, -6, -1), (4, -2, -10, -4), (1, -1, -2, -2), (3, -2, -4, -1)]


def _pairs(seed, n, lo, hi, alpha=4, codes=None):
    rng = np.random.default_rng(seed)
    draw = (lambda k: rng.integers(0, alpha, k)) if codes is None else (lambda k: codes[rng.integers(0, len(codes), k)])
    H, V = [], []
    for _ in range(n):
        h = draw(rng.integers(lo, hi + 1)).astype(np.uint8)
        if rng.random() < 0.6:
            v = h.copy()
            msk = rng.random(len(v)) < 0.12
            v[msk] = draw(int(msk.sum()))
            cut = int(rng.integers(0, 6))
            v = v[cut:] if len(v) > cut + 1 else v
        else:
            v = draw(rng.integers(lo, hi + 1)).astype(np.uint8)
        H.append(h)
        V.append(v.astype(np.uint8))
    return H, V


def _check(score, H, V, mode, cfg, pb, alphabet_size):
    import seqan_gb300 as sg
    from seqan_gb300 import _native as N
    ref = O.oracle_batch(pb, H, V, traceback=True)
    out = sg.align_codes(H, V, score, mode=mode, config=cfg, traceback=True, cigar=True, alphabet_size=alphabet_size,
                         flags=N.GBA_FLAG_WARP16)
    assert sg.default_context().stats().dp_kernels & N.GBA_KERNEL_WARP16
    assert out.score.tolist() == ref.score.tolist()
    assert out.end_h.tolist() == ref.end_h.tolist() and out.end_v.tolist() == ref.end_v.tolist()
    for k in range(len(H)):
        assert out.pair_segments(k) == ref.segments[k], k
        assert out.pair_cigar(k) == O.cigar_string(ref.segments[k]), k
    old = sg.align_codes(H, V, score, mode=mode, config=cfg, traceback=True, cigar=True, alphabet_size=alphabet_size,
                         flags=N.GBA_FLAG_NO_WARP16)
    assert not (sg.default_context().stats().dp_kernels & N.GBA_KERNEL_WARP16)
    assert np.array_equal(old.score, out.score) and np.array_equal(old.segments, out.segments)


@pytest.mark.parametrize("fe", range(16))
@pytest.mark.parametrize("scheme", SCHEMES)
def test_warp16_global_all_configs(engine, fe, scheme):
    import seqan_gb300 as sg
    mt, mm, go, ge = scheme
    H, V = _pairs(500 + fe * 11 - go, 120, 1, 300)
    cfg = sg.AlignConfig(bool(fe & 1), bool(fe & 2), bool(fe & 4), bool(fe & 8))
    _check(sg.Score(mt, mm, ge, go, dtype=np.int16), H, V, 0, cfg,
           O.Problem("global", fe, None, mt, mm, go, ge, None, 16), 4)


@pytest.mark.parametrize("scheme", SCHEMES)
def test_warp16_local(engine, scheme):
    import seqan_gb300 as sg
    mt, mm, go, ge = scheme
    H, V = _pairs(700 - ge, 200, 1, 400)
    _check(sg.Score(mt, mm, ge, go, dtype=np.int16), H, V, 1, None,
           O.Problem("local", 0, None, mt, mm, go, ge, None, 16), 4)


@pytest.mark.parametrize("mode", ["local", "global"])
def test_warp16_blosum62_protein(engine, mode):
    import seqan_gb300 as sg
    from seqan_gb300 import workloads as W
    score = sg.Blosum62(-1, -11, dtype=np.int16)
    H, V = _pairs(17, 300, 20, 700, codes=W.AA20_CODES)
    _check(score, H, V, 1 if mode == "local" else 0, sg.AlignConfig() if mode == "global" else None,
           O.Problem(mode, 0, None, 0, 0, -11, -1, score.matrix, 16, "aa"), 27)


@pytest.mark.parametrize("rows", [255, 256, 257, 300, 320, 384, 385, 512, 700, 1000, 4096])
def test_warp16_band_boundaries(engine, rows):
    """Pairs whose row counts sit at and around the band sizes (last bands of 64 / 128 / 256 rows)."""
    import seqan_gb300 as sg
    rng = np.random.default_rng(rows)
    H = [rng.integers(0, 4, int(rng.integers(1, 1023))).astype(np.uint8) for _ in range(12)]
    V = [rng.integers(0, 4, rows).astype(np.uint8) for _ in range(12)]
    for k in range(0, 12, 2):
        V[k][: min(len(H[k]), rows)] = H[k][: min(len(H[k]), rows)]
    for mode, fe in (("local", 0), ("global", 0), ("global", 9), ("global", 6)):
        cfg = sg.AlignConfig(bool(fe & 1), bool(fe & 2), bool(fe & 4), bool(fe & 8))
        _check(sg.Score(2, -4, -1, -6, dtype=np.int16), H, V, 1 if mode == "local" else 0,
               cfg if mode == "global" else None, O.Problem(mode, fe, None, 2, -4, -6, -1, None, 16), 4)


def test_warp16_routing_keeps_other_pairs_exact(engine):
    """A batch mixing eligible pairs with pairs the packed warp kernel does not take (1,024 columns and
    more, more than 4,096 rows, and pairs past the exact int16 range) gives the oracle's results for
    all of them; the kernels share one call."""
    import seqan_gb300 as sg
    from seqan_gb300 import _native as N
    H, V = _pairs(23, 60, 50, 400)
    rng = np.random.default_rng(5)
    for L in (1024, 1500):
        h = rng.integers(0, 4, L).astype(np.uint8)
        H.append(h)
        V.append(h[: L - 10].copy())
    h = rng.integers(0, 4, 300).astype(np.uint8)
    H.append(h)
    V.append(np.concatenate([h] * 14)[:4200].astype(np.uint8))
    h = rng.integers(0, 4, 900).astype(np.uint8)
    H.append(h)
    V.append(rng.integers(0, 4, 4000).astype(np.uint8))
    score = sg.Score(2, -4, -3, -6, dtype=np.int16)   # extension -3: long global pairs leave the exact range
    for mode in ("global", "local"):
        ref = O.oracle_batch(O.Problem(mode, 0, None, 2, -4, -6, -3, None, 32 if mode == "global" else 16), H, V,
                             traceback=True)
        out = sg.align_codes(H, V, score, mode=0 if mode == "global" else 1, traceback=True, alphabet_size=4,
                             flags=N.GBA_FLAG_WARP16)
        kernels = sg.default_context().stats().dp_kernels
        assert kernels & N.GBA_KERNEL_WARP16 and kernels & N.GBA_KERNEL_WARP
        assert out.score.tolist() == ref.score.tolist()
        for k in range(len(H)):
            assert out.pair_segments(k) == ref.segments[k], k
