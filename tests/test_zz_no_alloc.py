"""gba_align_score_noalloc against gba_align_batch, through the C-ABI.

The allocation-free entry point serves callers that cannot allocate device memory on their
call path (hosts that own all device memory through their own pool, and latency-bound
request loops that keep cudaMalloc/cudaFree out of their requests).  The test allocates the
inputs and outputs itself, as such a caller would, then checks two calls in a row against
the regular entry point.  Integer results, so the tolerance is zero: every score and end
position must be identical.  The second call uses a different batch, so a stale scratch
array from the first call would show up as a mismatch.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _device_sync():
    cuda = C.CDLL("libcuda.so.1")
    assert cuda.cuCtxSynchronize() == 0


def _regular(score, H, V, mode, config):
    import seqan_gb300 as sg
    return sg.align_codes(H, V, score, mode=mode, config=config)


def _noalloc(ctx, score, H, V, mode, config, max_h_len):
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
    rc = L.gba_align_score_noalloc(C.byref(params), C.byref(batch), *outs, None)
    assert rc == N.GBA_OK
    _device_sync()
    res = []
    for p in outs:
        a = np.zeros(n, np.int32)
        ctx.check(L.gba_copy_to_host(h, a.ctypes.data_as(C.c_void_p), p, a.nbytes), "d2h")
        res.append(a)
    for p in bufs:
        L.gba_device_free(h, p)
    return res


def _pairs(seed, n, lo, hi):
    rng = np.random.default_rng(seed)
    H = [rng.integers(0, 4, rng.integers(lo, hi + 1)).astype(np.uint8) for _ in range(n)]
    V = [np.where(rng.random(len(x)) < 0.1, (x + 1) % 4, x).astype(np.uint8) for x in H]
    return H, V


def test_noalloc_matches_regular_entry_point_twice(engine):
    import seqan_gb300 as sg
    cases = [
        (sg.Score(2, -4, -1, -6, dtype=np.int16), _pairs(1, 3000, 100, 300), 0, sg.AlignConfig(), 300),
        (sg.Score(2, -3, -5, dtype=np.int32), _pairs(2, 1500, 1, 120), 0,
         sg.AlignConfig(True, False, False, True), 400),
    ]
    for score, (H, V), mode, cfg, max_h in cases:
        ref = _regular(score, H, V, mode, cfg)
        got_score, got_eh, got_ev, got_status = _noalloc(engine, score, H, V, mode, cfg, max_h)
        assert np.array_equal(got_score, ref.score)
        assert np.array_equal(got_eh, ref.end_h) and np.array_equal(got_ev, ref.end_v)
        assert np.array_equal(got_status, ref.status)


def test_noalloc_rejects_bound_beyond_scratch(engine):
    import seqan_gb300 as sg
    from seqan_gb300 import _native as N
    params = sg.align.make_params(sg.Score(2, -3, -5), 0, sg.AlignConfig(), None, N.GBA_OUT_SCORE)
    too_long = N.GBA_NOALLOC_SCRATCH_BYTES // (32 * 8)
    batch = N.GbaNoAllocBatch(1, 1, 1, 1, 1, too_long, 0)
    dummy = C.c_void_p(1)
    assert N.lib().gba_align_score_noalloc(C.byref(params), C.byref(batch), dummy, None, None, None,
                                           None) == N.GBA_ECAPACITY
