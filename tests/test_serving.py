"""Serving loop: results identical alone and in the mix, HBM-budget admission, overlap."""
import time

import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu


def _pairs(seed, lengths):
    from seqan_gb300 import workloads as W
    rng = np.random.default_rng(seed)
    H, V = [], []
    for L in lengths:
        h = rng.integers(0, 4, int(L)).astype(np.uint8)
        H.append(h)
        V.append(W.mutate(rng, h, 0.05, 0.01))
    return H, V


def _drain(srv, want, timeout=120.0):
    done = {}
    t0 = time.time()
    while len(done) < want:
        for r in srv.poll():
            done[r.tag] = r
        assert time.time() - t0 < timeout, f"{len(done)} of {want} requests finished"
        time.sleep(0.001)
    return done


def _key(r):
    return (r.score, r.end_h, r.end_v, r.begin_h, r.begin_v, r.status, tuple(r.segments))


@pytest.mark.parametrize("mode", [0, 1])
def test_results_same_alone_and_in_the_mix(engine, mode):
    """Probe requests (one of them 5,000 bp, several bands) run alone, one request per batch,
    then again interleaved with 600 background requests of 20-3,000 bp on 4 streams; every
    probe's score, positions and segment list are identical both ways and equal the oracle."""
    import seqan_gb300 as sg
    from seqan_gb300.serving import Server
    score = sg.Score(2, -4, -1, -6, dtype=np.int16)
    Hp, Vp = _pairs(1, [5000, 300, 1, 150, 2500, 777, 64, 1200])
    Hb, Vb = _pairs(2, np.random.default_rng(3).integers(20, 3001, 600))

    with Server(score, mode=mode, traceback=True, streams=1, max_batch_pairs=1) as srv:
        alone = {}
        for i, (h, v) in enumerate(zip(Hp, Vp)):
            assert srv.submit(i, h, v) == 0
            alone.update(_drain(srv, 1))
    with Server(score, mode=mode, traceback=True, streams=4, max_batch_pairs=64) as srv:
        tag = 0
        probes = {}
        for k, (h, v) in enumerate(zip(Hb, Vb)):
            assert srv.submit(1000 + k, h, v) == 0
            if k % 75 == 0 and tag < len(Hp):
                probes[tag] = True
                assert srv.submit(tag, Hp[tag], Vp[tag]) == 0
                tag += 1
        while tag < len(Hp):
            assert srv.submit(tag, Hp[tag], Vp[tag]) == 0
            tag += 1
        mix = _drain(srv, len(Hb) + len(Hp))
        st = srv.stats()
        assert st.batches > 4 and st.completed == len(Hb) + len(Hp)

    pb = O.Problem("local" if mode else "global", 0, None, 2, -4, -6, -1, None, 32)
    ref = O.oracle_batch(pb, Hp, Vp, traceback=True)
    for i in range(len(Hp)):
        assert _key(alone[i]) == _key(mix[i]), i
        assert alone[i].score == ref.score[i] and alone[i].segments == ref.segments[i], i
        assert (alone[i].end_h, alone[i].end_v) == (ref.end_h[i], ref.end_v[i]), i
    refb = O.oracle_batch(pb, Hb, Vb)
    assert [mix[1000 + k].score for k in range(len(Hb))] == refb.score.tolist()


def test_budget_admission(engine):
    """A 4 MiB budget: a pair that alone needs more is refused with GBA_EBUDGET; the others run,
    and the device bytes in flight never exceed the budget."""
    import seqan_gb300 as sg
    from seqan_gb300 import _native as N
    from seqan_gb300.serving import Server
    score = sg.Score(2, -4, -1, -6, dtype=np.int16)
    budget = 4 << 20
    H, V = _pairs(5, [400] * 200)
    Hbig, Vbig = _pairs(6, [3000])
    with Server(score, traceback=True, streams=8, max_batch_pairs=256, hbm_budget_bytes=budget) as srv:
        assert srv.submit(99999, Hbig[0], Vbig[0]) == N.GBA_EBUDGET
        for k, (h, v) in enumerate(zip(H, V)):
            assert srv.submit(k, h, v) == 0
        done = _drain(srv, len(H))
        st = srv.stats()
        assert 0 < st.hbm_in_flight_peak <= budget
        assert st.hbm_in_flight == 0 and st.submitted == len(H)
        assert st.batches > 1   # the budget split the queue
    ref = O.oracle_batch(O.Problem("global", 0, None, 2, -4, -6, -1, None, 32), H, V)
    assert [done[k].score for k in range(len(H))] == ref.score.tolist()
    assert all(done[k].status == 0 for k in range(len(H)))


def test_latency_timestamps_and_empty_pairs(engine):
    """Empty pairs come back invalid with numeric_limits<int16>::min(); timestamps are ordered."""
    import seqan_gb300 as sg
    from seqan_gb300.serving import Server
    with Server(sg.Score(2, -4, -1, -6, dtype=np.int16), traceback=True, streams=2) as srv:
        t0 = srv.clock()
        assert srv.submit(1, np.zeros(0, np.uint8), np.array([1, 2], np.uint8)) == 0
        assert srv.submit(2, np.array([0, 1, 2, 3], np.uint8), np.array([0, 1, 2, 3], np.uint8)) == 0
        done = _drain(srv, 2)
    assert done[1].status == 1 and done[1].score == -32768 and done[1].segments == []
    assert done[2].score == 8 and done[2].segments == [(0, 0, 4, 1)]
    for r in done.values():
        assert t0 <= r.t_submit <= r.t_done


def test_native_submit_schedule(engine):
    """A request trace replayed by gba_server_submit_schedule at its arrival times (native
    thread) while Python polls; every result equals the oracle's and each was submitted no
    earlier than its scheduled time."""
    import threading
    import seqan_gb300 as sg
    from seqan_gb300.serving import Server
    H, V = _pairs(9, np.random.default_rng(10).integers(50, 1500, 300))
    at = np.sort(np.random.default_rng(11).uniform(0, 0.06, len(H)))
    with Server(sg.Score(2, -4, -1, -6, dtype=np.int16), traceback=True, streams=4) as srv:
        t0 = srv.clock()
        rc = []
        th = threading.Thread(target=lambda: rc.append(srv.submit_schedule(H, V, at, first_tag=5000)))
        th.start()
        done = _drain(srv, len(H))
        th.join()
    assert rc == [0]
    ref = O.oracle_batch(O.Problem("global", 0, None, 2, -4, -6, -1, None, 32), H, V, traceback=True)
    for k in range(len(H)):
        r = done[5000 + k]
        assert r.score == ref.score[k] and r.segments == ref.segments[k], k
        assert r.t_submit >= t0 + at[k] - 1e-3
