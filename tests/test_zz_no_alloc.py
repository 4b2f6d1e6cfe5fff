"""gba_align_score_noalloc against gba_align_batch, through the C-ABI.

The allocation-free entry point serves callers that cannot allocate device memory on their
call path (hosts that own all device memory through their own pool, and latency-bound
request loops that keep cudaMalloc/cudaFree out of their requests).  The test allocates the
inputs and outputs itself, as such a caller would, then checks calls in a row against the
regular entry point: global, local and Blosum62 scoring, int16 and int32 cells, pairs past
the exact int16 range, pairs over the caller's length bound.  Integer results, so the
tolerance is zero: every score, end position and status must be identical.  Each call uses a
different batch, so a stale scratch array from the call before would show up as a mismatch.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _device_sync():
    cuda = C.CDLL("libcuda.so.1")
    assert cuda.cuCtxSynchronize() == 0


def _free_device_bytes():
    cuda = C.CDLL("libcuda.so.1")
    free, total = C.c_size_t(), C.c_size_t()
    assert cuda.cuMemGetInfo_v2(C.byref(free), C.byref(total)) == 0
    return free.value


def _regular(score, H, V, mode, config):
    import seqan_gb300 as sg
    return sg.align_codes(H, V, score, mode=mode, config=config)


def _noalloc(ctx, score, H, V, mode, config, max_h_len, free_bytes=None):
    import seqan_gb300 as sg
    from seqan_gb300 import _native as N
    L, h = N.lib(), ctx.handle
    sh, oh = sg.align._concat(H)
    sv, ov = sg.align._concat(V)
    n = len(H)
    bufs = []

    def dev(arr):
        p = C.c_void_p()
        ctx.check(L.gba_device_alloc(h, C.byref(p), max(arr.nbytes, 16)), "alloc")
        ctx.check(L.gba_copy_to_device(h, p, arr.ctypes.data_as(C.c_void_p), arr.nbytes), "h2d")
        bufs.append(p)
        return p

    d_sh, d_oh, d_sv, d_ov = dev(sh), dev(oh), dev(sv), dev(ov)
    outs = [dev(np.zeros(n, np.int32)) for _ in range(4)]
    ctx.check(L.gba_synchronize(h), "sync")
    params = sg.align.make_params(score, mode, config, None, N.GBA_OUT_SCORE | N.GBA_OUT_END)
    batch = N.GbaNoAllocBatch(n, d_sh, d_oh, d_sv, d_ov, max_h_len, 0)
    _device_sync()
    before = _free_device_bytes()
    rc = L.gba_align_score_noalloc(C.byref(params), C.byref(batch), *outs, None)
    assert rc == N.GBA_OK
    _device_sync()
    if free_bytes is not None:
        free_bytes.append((before, _free_device_bytes()))
    res = []
    for p in outs:
        a = np.zeros(n, np.int32)
        ctx.check(L.gba_copy_to_host(h, a.ctypes.data_as(C.c_void_p), p, a.nbytes), "d2h")
        res.append(a)
    for p in bufs:
        L.gba_device_free(h, p)
    return res


def _pairs(seed, n, lo, hi, alpha=4, codes=None):
    rng = np.random.default_rng(seed)
    draw = (lambda k: rng.integers(0, alpha, k)) if codes is None else (lambda k: codes[rng.integers(0, len(codes), k)])
    H = [draw(rng.integers(lo, hi + 1)).astype(np.uint8) for _ in range(n)]
    V = [np.where(rng.random(len(x)) < 0.3, draw(len(x)), x).astype(np.uint8) for x in H]
    return H, V


AA20 = np.array([0, 2, 3, 4, 5, 6, 7, 8, 10, 11, 12, 13, 15, 16, 17, 18, 19, 21, 22, 23], np.uint8)


def _cases():
    import seqan_gb300 as sg
    b62 = sg.Blosum62(-1, -11, dtype=np.int16)
    return [
        ("affine global int16", sg.Score(2, -4, -1, -6, dtype=np.int16), _pairs(1, 3000, 100, 300), 0,
         sg.AlignConfig(), 300),
        ("linear global int32, free first/last row", sg.Score(2, -3, -5, dtype=np.int32), _pairs(2, 1500, 1, 120), 0,
         sg.AlignConfig(True, False, False, True), 400),
        ("affine local int16", sg.Score(2, -4, -1, -6, dtype=np.int16), _pairs(3, 2000, 20, 250), 1, None, 250),
        ("Blosum62 local int16", b62, _pairs(4, 1200, 30, 400, codes=AA20), 1, None, 400),
        ("Blosum62 global int16", b62, _pairs(5, 1200, 30, 400, codes=AA20), 0, sg.AlignConfig(), 400),
        # With gap extension -3, 3,000 x 3,000 bp global pairs can reach values below the int16
        # "infinity" (all-gap paths cost 3 * (m + n)): promoted to 32-bit cells.
        ("int16 past the exact bound", sg.Score(2, -4, -3, -6, dtype=np.int16), _pairs(6, 40, 2900, 3000), 0,
         sg.AlignConfig(), 3000),
    ]


def test_noalloc_matches_regular_entry_point_twice(engine):
    """Every case calls the allocation-free entry point twice in a row on the shared scratch and
    compares both results with gba_align_batch with zero tolerance.  The second call of a case must
    leave the device's free memory unchanged: the first call of a scoring shape may still load that
    shape's kernel code onto the device (CUDA's lazy module loading), a repeated call allocates
    nothing."""
    for name, score, (H, V), mode, cfg, max_h in _cases():
        ref = _regular(score, H, V, mode, cfg)
        free = []
        for call in range(2):
            got_score, got_eh, got_ev, got_status = _noalloc(engine, score, H, V, mode, cfg, max_h, free)
            assert np.array_equal(got_score, ref.score), (name, call)
            assert np.array_equal(got_eh, ref.end_h) and np.array_equal(got_ev, ref.end_v), (name, call)
            assert np.array_equal(got_status, ref.status), (name, call)
            if name.startswith("int16 past"):
                assert (got_status == 2).all(), name
        before, after = free[1]
        assert after == before, f"{name}: a repeated call changed the device's free memory"


def test_noalloc_pairs_over_the_bound_are_skipped(engine):
    """Pairs with |H| above max_h_len are not computed: numeric min and GBA_PAIR_SKIPPED; empty
    pairs keep GBA_PAIR_INVALID; every other pair equals gba_align_batch."""
    import seqan_gb300 as sg
    from seqan_gb300 import _native as N
    score = sg.Score(2, -4, -1, -6, dtype=np.int16)
    H, V = _pairs(7, 500, 50, 200)
    H[17] = np.zeros(0, np.uint8)
    for k in (3, 250, 499):
        H[k] = np.random.default_rng(k).integers(0, 4, 260).astype(np.uint8)
    ref = _regular(score, H, V, 0, sg.AlignConfig())
    got_score, got_eh, got_ev, got_status = _noalloc(engine, score, H, V, 0, sg.AlignConfig(), 200)
    over = np.array([len(h) > 200 for h in H])
    assert (got_status[over] == N.GBA_PAIR_SKIPPED).all() and (got_score[over] == -32768).all()
    assert got_status[17] == N.GBA_PAIR_INVALID == ref.status[17] and got_score[17] == ref.score[17]
    ok = ~over
    assert np.array_equal(got_score[ok], ref.score[ok]) and np.array_equal(got_status[ok], ref.status[ok])
    assert np.array_equal(got_eh[ok], ref.end_h[ok]) and np.array_equal(got_ev[ok], ref.end_v[ok])


def test_noalloc_rejects_bound_beyond_scratch(engine):
    import seqan_gb300 as sg
    from seqan_gb300 import _native as N
    params = sg.align.make_params(sg.Score(2, -3, -5), 0, sg.AlignConfig(), None, N.GBA_OUT_SCORE)
    too_long = N.GBA_NOALLOC_SCRATCH_BYTES // (32 * 8)
    batch = N.GbaNoAllocBatch(1, 1, 1, 1, 1, too_long, 0)
    dummy = C.c_void_p(1)
    assert N.lib().gba_align_score_noalloc(C.byref(params), C.byref(batch), dummy, None, None, None,
                                           None) == N.GBA_ECAPACITY
