"""GPU parity of DynamicGaps cells (k_dp_dynamic) against the reference's fixtures and the oracle.

The reference's third gap-cost model keeps one score and two gap flags per cell and extends a gap
when the neighbour's flag for its direction is set (align/dp_cell_dynamic.h,
align/dp_formula_dynamic.h); the traceback walks one cell at a time and corrects the start cell from
the best cell's flags (align/dp_traceback_impl.h:190-370, align/dp_algorithm_impl.h:1235-1249).
Exact comparisons of scores, best cells and TraceSegment_ lists."""
import dataclasses

import numpy as np
import pytest

import golden_cases as G
from oracle import oracle as O

pytestmark = pytest.mark.gpu

CASES = G.load("dynamic_cases.json")["cases"]


def _run(p, H, V, traceback=True, flags=0):
    import seqan_gb300 as sg
    from seqan_gb300 import _native as N
    score, mode, cfg, band = G.engine_args(p)
    return sg.align_codes(H, V, score, mode=mode, config=cfg, band=band, traceback=traceback,
                          alphabet_size=27 if p["alphabet"] == "aa" else 5, gaps=N.GBA_GAPS_DYNAMIC, flags=flags)


@pytest.mark.parametrize("case", CASES, ids=[G.case_id({"kind": "dynamic", "problem": c["problem"]}) for c in CASES])
def test_dynamic_gaps_match_reference_fixture(engine, case):
    p = case["problem"]
    H, V = G.codes(case["H"], p["alphabet"]), G.codes(case["V"], p["alphabet"])
    out = _run(p, H, V)
    for k, want in enumerate(case["results"]):
        assert out.score[k] == want["score"], k
        assert [list(s) for s in out.pair_segments(k)] == want["segments"], k


SCHEMES = [(2, -3, -5, -5), (2, -4, -6, -1), (4, -2, -10, -4), (2, -3, -1, -7)]


def _pairs(seed, n, lo, hi, alpha=4):
    rng = np.random.default_rng(seed)
    H = [rng.integers(0, alpha, rng.integers(lo, hi + 1)).astype(np.uint8) for _ in range(n)]
    V = []
    for h in H:
        if rng.random() < 0.6:
            v = h.copy()
            msk = rng.random(len(v)) < 0.12
            v[msk] = rng.integers(0, alpha, int(msk.sum()))
            V.append(v[: max(1, len(v) - int(rng.integers(0, 6)))])
        else:
            V.append(rng.integers(0, alpha, rng.integers(lo, hi + 1)).astype(np.uint8))
    return H, V


@pytest.mark.parametrize("fe", range(16))
@pytest.mark.parametrize("scheme", SCHEMES)
def test_dynamic_gaps_all_configs_against_oracle(engine, fe, scheme):
    mt, mm, go, ge = scheme
    H, V = _pairs(900 + fe * 13 - go, 150, 1, 120)
    H[3] = np.zeros(0, np.uint8)          # an empty pair: numeric min, no segments
    for bits in (16, 32):
        p = {"mode": "global", "free_ends": fe, "band": None, "match": mt, "mismatch": mm, "gap_open": go,
             "gap_extend": ge, "blosum62": False, "score_bits": bits, "alphabet": "dna"}
        ref = O.oracle_batch(dataclasses.replace(G.oracle_problem(p), dynamic=True), H, V, traceback=True)
        out = _run(p, H, V)
        assert out.score.tolist() == ref.score.tolist()
        assert out.end_h.tolist() == ref.end_h.tolist() and out.end_v.tolist() == ref.end_v.tolist()
        for k in range(len(H)):
            assert out.pair_segments(k) == ref.segments[k], k


@pytest.mark.parametrize("alphabet", ["dna", "aa"])
def test_dynamic_gaps_local_and_long_pairs(engine, alphabet):
    """Local mode, Blosum62, and pairs long enough to leave the exact int16 range (promoted to 32-bit
    cells, whose reference result is the int32 one)."""
    b62 = alphabet == "aa"
    H, V = _pairs(77, 120, 10, 600, alpha=24 if b62 else 4)
    for L in (3000, 5200):
        rng = np.random.default_rng(L)
        h = rng.integers(0, 24 if b62 else 4, L).astype(np.uint8)
        H.append(h)
        V.append(h[:: 1 + (L % 3)].copy())
    for mode in ("local", "global"):
        p = {"mode": mode, "free_ends": 0, "band": None, "match": 2, "mismatch": -3, "gap_open": -11 if b62 else -6,
             "gap_extend": -3, "blosum62": b62, "score_bits": 16, "alphabet": alphabet}
        out = _run(p, H, V)
        p32 = dict(p, score_bits=32)
        ref = O.oracle_batch(dataclasses.replace(G.oracle_problem(p32), dynamic=True), H, V, traceback=True)
        assert out.score.tolist() == ref.score.tolist()
        for k in range(len(H)):
            assert out.pair_segments(k) == ref.segments[k], k


def test_dynamic_gaps_refuses_a_band(engine):
    import seqan_gb300 as sg
    from seqan_gb300 import _native as N
    with pytest.raises(N.GbaError) as e:
        sg.align_codes([np.zeros(5, np.uint8)], [np.zeros(5, np.uint8)], sg.Score(2, -3, -1, -5), band=(-2, 2),
                       gaps=N.GBA_GAPS_DYNAMIC)
    assert e.value.status == N.GBA_EUNSUPPORTED
