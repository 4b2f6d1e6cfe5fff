"""Serving loop: requests submitted one pair at a time, batched continuously on the GPU.

A thin wrapper over the engine's gba_server_* entry points (include/seqan_gb300.h).  The
reference has no request loop -- its batch call blocks until the whole StringSet is aligned --
so this is the only interface here without a SeqAn counterpart; a request's result is the one
globalAlignment / localAlignment returns for that pair (the same kernels as the batch call).

    srv = Server(Score(2, -4, -1, -6), traceback=True)
    srv.submit(tag, h_codes, v_codes)
    for r in srv.poll():          # non-blocking; completion order
        r.tag, r.score, r.segments, r.t_done - r.t_submit
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field

import numpy as np

from . import _native as N
from .align import AlignConfig, _concat, make_params


@dataclass
class RequestResult:
    tag: int
    score: int
    end_h: int
    end_v: int
    begin_h: int
    begin_v: int
    status: int
    t_submit: float
    t_done: float
    segments: list = field(default_factory=list)   # TraceSegment_ tuples (h_begin, v_begin, length, type)


class Server:
    """One scoring scheme, `streams` batches in flight, FIFO admission under `max_batch_pairs`
    and an HBM budget (bytes of the batches in flight; 0 = none)."""

    def __init__(self, score, mode: int = N.GBA_GLOBAL, config: AlignConfig | None = None, band=None,
                 traceback: bool = True, streams: int = 8, max_batch_pairs: int = 4096,
                 hbm_budget_bytes: int = 0, device: int = 0, alphabet_size: int = 0):
        L = N.lib()
        outputs = N.GBA_OUT_SCORE | N.GBA_OUT_END | (N.GBA_OUT_SEGMENTS if traceback else 0)
        self._score = score   # keeps a matrix alive while the params are built
        params = make_params(score, mode, config, band, outputs, alphabet_size)
        cfg = N.GbaServerConfig(device, streams, max_batch_pairs, hbm_budget_bytes)
        self._h = C.c_void_p()
        rc = L.gba_server_create(C.byref(self._h), C.byref(cfg), C.byref(params))
        if rc != N.GBA_OK:
            raise N.GbaError(rc, f"gba_server_create failed: {L.gba_status_string(rc).decode()}")
        self._results = (N.GbaRequestResult * 4096)()
        self._segs = np.zeros((1 << 20, 4), dtype=np.uint32)

    def _error(self) -> str:
        buf = C.create_string_buffer(512)
        N.lib().gba_server_last_error(self._h, buf, 512)
        return buf.value.decode()

    def submit(self, tag: int, h: np.ndarray, v: np.ndarray) -> int:
        """Queues one pair of code arrays; returns the status (GBA_EBUDGET when the pair alone
        does not fit the budget)."""
        h = np.ascontiguousarray(h, dtype=np.uint8)
        v = np.ascontiguousarray(v, dtype=np.uint8)
        return N.lib().gba_server_submit(self._h, tag, h.ctypes.data, len(h), v.ctypes.data, len(v))

    def submit_schedule(self, H, V, at_seconds, first_tag: int = 0) -> int:
        """Submits pair k with tag first_tag + k at at_seconds[k] after the call starts, from
        native code (no Python between submits); blocks until all are submitted.  Call it from
        a thread to poll meanwhile: the call does not hold the GIL."""
        sh, oh = _concat(H)
        sv, ov = _concat(V)
        at = np.ascontiguousarray(at_seconds, dtype=np.float64)
        if len(at) != len(H) or len(H) != len(V):
            raise ValueError("H, V and at_seconds differ in length")
        b = N.GbaBatch(len(H), sh.ctypes.data, oh.ctypes.data, sv.ctypes.data, ov.ctypes.data, 0, 0)
        return N.lib().gba_server_submit_schedule(self._h, C.byref(b), at.ctypes.data, first_tag)

    def poll(self, segments: bool = True) -> list[RequestResult]:
        """Finished requests (completion order); never waits.  segments=False skips building
        the per-request segment lists."""
        L = N.lib()
        out = []
        while True:
            nr, ns = C.c_int64(), C.c_int64()
            rc = L.gba_server_poll(self._h, self._results, len(self._results), self._segs.ctypes.data,
                                   len(self._segs), C.byref(nr), C.byref(ns))
            if rc == N.GBA_ECAPACITY:
                self._segs = np.zeros((2 * len(self._segs), 4), dtype=np.uint32)
                continue
            if rc != N.GBA_OK:
                raise N.GbaError(rc, f"gba_server_poll: {self._error()}")
            for i in range(nr.value):
                r = self._results[i]
                segs = self._segs[r.segment_offset:r.segment_offset + r.n_segments]
                out.append(RequestResult(r.tag, r.score, r.end_h, r.end_v, r.begin_h, r.begin_v, r.status,
                                         r.t_submit, r.t_done,
                                         [tuple(int(x) for x in s) for s in segs] if segments else []))
            if nr.value < len(self._results):
                return out

    def stats(self) -> N.GbaServerStats:
        s = N.GbaServerStats()
        N.lib().gba_server_get_stats(self._h, C.byref(s))
        return s

    @staticmethod
    def clock() -> float:
        return N.lib().gba_clock_seconds()

    def close(self):
        if self._h:
            N.lib().gba_server_destroy(self._h)
            self._h = C.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
