"""The 4-bit trace code keeps every traceback decision (oracle, CPU).

Each cell's trace needs 4 bits: the source of S (none, diagonal, MAX_FROM_V, MAX_FROM_H) and one
open/extend bit for each of E and F (SingleTrace sets exactly one of each pair in inner cells,
align/dp_formula.h:179-181).  Here the oracle passes every trace byte through that code before
its traceback (_doTraceback, align/dp_traceback_impl.h:376-450, with the start-cell correction
of align/dp_algorithm_impl.h:1188-1205 and the head/tail segments of :489-546) and the
TraceSegment_ lists must equal the 8-bit run's exactly, over every AlignConfig, local mode,
linear and affine gaps, both cell widths, bands (whose edge cells lack an open/extend pair) and
Blosum62 -- and over the reference's own fixture cases."""
import numpy as np
import pytest

import golden_cases as G
from oracle import oracle as O


def _pairs(seed, n, lo, hi, alpha=4):
    rng = np.random.default_rng(seed)
    H = [rng.integers(0, alpha, rng.integers(lo, hi + 1)).astype(np.uint8) for _ in range(n)]
    V = []
    for h in H:
        if rng.random() < 0.6:
            v = h.copy()
            m = rng.random(len(v)) < 0.15
            v[m] = rng.integers(0, alpha, int(m.sum()))
            cut = rng.integers(0, 4)
            V.append(v[cut:len(v) - rng.integers(0, 4)] if len(v) > 8 else v)
        else:
            V.append(rng.integers(0, alpha, rng.integers(lo, hi + 1)).astype(np.uint8))
    return H, V


def _same(pb, H, V):
    import dataclasses
    full = O.oracle_batch(pb, H, V, traceback=True)
    q = O.oracle_batch(dataclasses.replace(pb, trace4=True), H, V, traceback=True)
    assert np.array_equal(full.score, q.score)
    for k in range(len(H)):
        assert q.segments[k] == full.segments[k], (pb, k)


SCHEMES = [(2, -3, -5, -5), (2, -4, -6, -1), (4, -2, -10, -4), (1, -1, -2, -2), (3, -2, -4, -1)]


@pytest.mark.parametrize("fe", range(16))
@pytest.mark.parametrize("scheme", SCHEMES)
def test_trace4_global_all_configs(fe, scheme):
    mt, mm, go, ge = scheme
    H, V = _pairs(fe * 7 - go, 120, 1, 70)
    for bits in (16, 32):
        _same(O.Problem("global", fe, None, mt, mm, go, ge, None, bits), H, V)


@pytest.mark.parametrize("scheme", SCHEMES)
def test_trace4_local(scheme):
    mt, mm, go, ge = scheme
    H, V = _pairs(100 - ge, 200, 1, 90)
    for bits in (16, 32):
        _same(O.Problem("local", 0, None, mt, mm, go, ge, None, bits), H, V)


@pytest.mark.parametrize("band", [(-6, 26), (-3, 3), (0, 0), (-10, 2), (5, 30), (-20, -2)])
@pytest.mark.parametrize("fe", [0, 9, 6, 15])
def test_trace4_banded(band, fe):
    H, V = _pairs(300 + fe + band[0] + 40, 150, 20, 60)
    for scheme in ((2, -4, -6, -1), (2, -3, -5, -5)):
        mt, mm, go, ge = scheme
        pb = O.Problem("global", fe, band, mt, mm, go, ge, None, 16)
        keep = [k for k in range(len(H)) if O.oracle_batch(pb, [H[k]], [V[k]]).valid[0]]
        _same(pb, [H[k] for k in keep], [V[k] for k in keep])
    pbl = O.Problem("local", 0, band, 2, -4, -6, -1, None, 32)
    _same(pbl, H, V)


def test_trace4_blosum62():
    b62 = np.array(G.load("blosum62.json")["matrix"], dtype=np.int32)
    H, V = _pairs(7, 200, 5, 150, alpha=24)
    for mode in ("local", "global"):
        _same(O.Problem(mode, 0, None, 0, 0, -11, -1, b62, 16, "aa"), H, V)


def test_trace4_reference_fixture_cases():
    for case in G.cases("segments") + G.cases("gaps"):
        p = case["problem"]
        pb = G.oracle_problem(p)
        H, V = G.codes(case["H"], p["alphabet"]), G.codes(case["V"], p["alphabet"])
        _same(pb, H, V)
