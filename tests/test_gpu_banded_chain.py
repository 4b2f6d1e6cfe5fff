"""Banded chain alignment on the GPU through gba_banded_chain: identical to the reference's
bandedChainAlignment on its test file's known answers and on 440 fixture chains from the compiled
reference, and to the oracle on seeded batches (random colinear chains over every AlignConfig and
scheme; genomic pairs with exact-match anchors at the benchmark's shape)."""
import numpy as np
import pytest

from oracle import oracle as O
from tests.test_banded_chain_oracle import CASES, FULL, KNOWN, KNOWN_IDS, codes, rows_of

pytestmark = pytest.mark.gpu


def _text(c):
    return "".join("ACGTN"[int(x)] for x in c)


def _score(t):
    import seqan_gb300 as sg
    return sg.Score(t[0], t[1], t[2], t[3])


@pytest.mark.parametrize("case", KNOWN, ids=KNOWN_IDS)
def test_known_answers(engine, case):
    import seqan_gb300 as sg
    from seqan_gb300.banded_chain import bandedChainAlignment
    h, v, chain, k, sc, score, row0, row1 = case
    r = bandedChainAlignment([h], [v], [chain], _score(sc), alignConfig=sg.AlignConfig(True, True, True, True),
                             bandExtension=k)[0]
    assert (r.score, r.row0, r.row1) == (score, row0, row1)


def test_empty_chain_keeps_rows(engine):
    from seqan_gb300.banded_chain import bandedChainAlignment
    r = bandedChainAlignment(["ACGATCGATCGACTGACT"], ["ACGATCGATCGACTGACT"], [[]], _score((5, -3, -5, -5)),
                             bandExtension=5)[0]
    assert r.score == -2 ** 31 and r.row0 == "ACGATCGATCGACTGACT" and r.segments == []


def _run(cases, max_traces=0):
    from seqan_gb300.banded_chain import banded_chain_codes
    from seqan_gb300 import AlignConfig
    # one call per (schemes, free ends, k) group
    groups = {}
    for i, c in enumerate(cases):
        groups.setdefault((tuple(c["anchor"]), tuple(c["gap"]), c["free_ends"], c["k"]), []).append(i)
    out = [None] * len(cases)
    for (a, g, fe, k), idx in groups.items():
        cfg = AlignConfig(bool(fe & 1), bool(fe & 2), bool(fe & 4), bool(fe & 8))
        sc, st, nt, segs = banded_chain_codes([codes(cases[i]["H"]) for i in idx], [codes(cases[i]["V"]) for i in idx],
                                              [cases[i]["seeds"] for i in idx], _score(a), _score(g), cfg, k,
                                              max_traces)
        for j, i in enumerate(idx):
            out[i] = (int(st[j]), int(sc[j]), int(nt[j]), segs[j])
    return out


def test_fixtures_through_c_abi(engine):
    got = _run(CASES)
    for c, (st, sc, nt, segs) in zip(CASES, got):
        assert st == c["status"], c
        if st == 0:
            assert (sc, nt) == (c["score"], c["n_traces"]), c
            assert [list(s) for s in segs] == c["segments"], c
            assert list(rows_of(segs, c["H"], c["V"])) == c["rows"], c


@pytest.mark.parametrize("seed", [1, 2])
def test_seeded_random_chains_vs_oracle(engine, seed):
    """1,500 random colinear chains (lengths 5-300, up to 12 seeds) in grouped calls."""
    from tests.golden.make_golden import chain_case
    rng = np.random.Generator(np.random.PCG64(4000 + seed))
    cases = []
    for t in range(1500):
        h, v, seeds, a, g, fe, k = chain_case(rng, 300, 12, 40)
        cases.append({"H": _text(h), "V": _text(v), "seeds": seeds, "anchor": a, "gap": g, "free_ends": fe, "k": k})
    got = _run(cases)
    for c, (st, sc, nt, segs) in zip(cases, got):
        o = O.oracle_banded_chain(codes(c["H"]), codes(c["V"]), c["seeds"], c["anchor"], c["gap"], c["free_ends"],
                                  c["k"])
        assert st == o.status, c
        if st == 0:
            assert (sc, nt, segs) == (o.score, o.n_traces, o.segments), c


def test_genomic_chains_vs_oracle(engine):
    """2,000 pairs of 1-3 kbp with exact-match anchors (the benchmark's shape), affine, k = 15."""
    from seqan_gb300 import workloads as W
    from seqan_gb300.banded_chain import banded_chain_codes
    H, V, chains = W.chain_pairs(2000, 1000, 3000, seed=501)
    sc_ = _score((2, -3, -1, -5))
    score, status, nt, segs = banded_chain_codes(H, V, chains, sc_, sc_, None, 15)
    for k in range(len(H)):
        o = O.oracle_banded_chain(H[k], V[k], chains[k], (2, -3, -1, -5), (2, -3, -1, -5), 0, 15)
        assert int(status[k]) == o.status, k
        if o.status == 0:
            assert (int(score[k]), int(nt[k]), segs[k]) == (o.score, o.n_traces, o.segments), k


def test_trace_capacity_is_reported(engine):
    """A chain whose grids hold more co-optimal traces than max_traces comes back with
    GBA_CHAIN_CAPACITY, never a wrong trace."""
    from seqan_gb300 import _native as N
    multi = [c for c in CASES if c["status"] == 0 and c["n_traces"] >= 2][:20]
    got = _run(multi, max_traces=1)
    assert all(st in (0, N.GBA_CHAIN_CAPACITY) for st, *_ in got)
    assert any(st == N.GBA_CHAIN_CAPACITY for st, *_ in got)
    for c, (st, sc, nt, segs) in zip(multi, got):
        if st == 0:
            assert [list(s) for s in segs] == c["segments"]
