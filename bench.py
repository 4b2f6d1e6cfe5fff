#!/usr/bin/env python3
"""Benchmark of the batch alignment hot path on one GB300 (per rank).

Default workload: batched affine global DNA alignment, uneven lengths -- 100,000 pairs, read
length uniform in [100, 300], partner = read with 5% substitutions and 1% single-base indels,
Score(match=2, mismatch=-4, gapExtend=-1, gapOpen=-6), 16-bit cells, outputs score + end
position.  A step is one pass of the engine over the whole batch.

* ``value``: GCUPS with inputs resident in HBM (gba_plan_execute), CUDA events around each
  step on the engine's stream, L2 flushed (256 MiB write) between steps outside the events.
* ``e2e``: the same metric through gba_align_batch with pinned HOST buffers: host->device copy
  of the codes and offsets, the kernels, and the device->host copy of scores and end positions
  are inside the timed region (wall clock around the blocking call).
* ``roofline``: the DP kernel against the measured 32-bit integer add/max rate (the DP is
  integer-issue bound; algorithmic ops per cell are stated in the design doc).
* ``cpu_baseline``: the oracle (CPU restatement of the reference, OpenMP over all host cores)
  timed on a sample of the same workload.
``--impl reference`` times that CPU implementation alone, in the same JSON shape.
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import os
import statistics
import subprocess
import sys
import tempfile
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

WORKLOADS = {
    # name: (description, generator kwargs)
    "affine_dna_100k": "100000 pairs, uniform length in [100,300], partner 5% subs + 1% indels, "
                       "Score(2,-4,-1,-6) int16, global, score + end position",
    "linear_dna_1024x150": "1024 pairs of uniform ACGT, both length 150, Score(2,-3,-5) int32, global, score",
}
OPS_PER_CELL = {"affine_global": 9, "linear_global": 5, "affine_local": 10, "linear_local": 6}


def make_workload(name: str, seed_offset: int = 0):
    import seqan_gb300 as sg
    from seqan_gb300 import workloads as W
    if name == "affine_dna_100k":
        H, V = W.mutated_dna_pairs(100_000, 100, 300, 0.05, 0.01, seed=2 + seed_offset)
        return H, V, sg.Score(2, -4, -1, -6, dtype=np.int16), 0, "affine_global"
    if name == "linear_dna_1024x150":
        H, V = W.uniform_dna_pairs(1024, 150, seed=1 + seed_offset)
        return H, V, sg.Score(2, -3, -5, dtype=np.int32), 0, "linear_global"
    raise SystemExit(f"unknown workload {name}")


class ClockSampler:
    """Samples nvidia-smi clocks and throttle reasons while the timed region runs."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.path = None

    def start(self):
        fd, self.path = tempfile.mkstemp(prefix="clocks", suffix=".csv")
        os.close(fd)
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.device}", f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except (FileNotFoundError, OSError):
            self.proc = None

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.15)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        with open(self.path) as f:
            for line in f:
                parts = [x.strip() for x in line.split(",")]
                if len(parts) < 9:
                    continue
                try:
                    sm.append(float(parts[1]))
                    smax.append(float(parts[2]))
                except ValueError:
                    continue
                for nm, val in zip(names, parts[5:9]):
                    if val.lower() == "active":
                        reasons.add(nm)
        os.unlink(self.path)
        busy = [x for x in sm if smax and x > 0.5 * max(smax)] or sm
        return {"sm_mhz": statistics.median(busy) if busy else None,
                "sm_max_mhz": max(smax) if smax else None, "reasons": sorted(reasons), "samples": len(sm)}


def concat(seqs):
    lens = np.fromiter((len(s) for s in seqs), dtype=np.int64, count=len(seqs))
    off = np.zeros(len(seqs) + 1, dtype=np.int64)
    np.cumsum(lens, out=off[1:])
    return np.concatenate(seqs).astype(np.uint8), off


def cpu_baseline(H, V, score, kind: str, seconds_target: float = 10.0):
    """Times the oracle (CPU restatement, all host threads) on a sample of the workload."""
    from oracle import oracle as O
    pb = O.Problem("global", 0, None, score.match, score.mismatch, score.gap_open, score.gap_extend, None,
                   score.bits)
    threads = os.cpu_count() or 1
    n = min(len(H), 2000)
    t0 = time.perf_counter()
    O.oracle_batch(pb, H[:n], V[:n], threads=threads)
    dt = time.perf_counter() - t0
    # Grow the sample to about seconds_target of wall time, bounded by the workload.
    n = int(min(len(H), max(n, n * seconds_target / max(dt, 1e-3) / 3)))
    best = None
    for _ in range(2):
        t0 = time.perf_counter()
        O.oracle_batch(pb, H[:n], V[:n], threads=threads)
        dt = time.perf_counter() - t0
        best = dt if best is None else min(best, dt)
    cells = int(sum(len(h) * len(v) for h, v in zip(H[:n], V[:n])))
    return {"value": cells / best / 1e9, "unit": "GCUPS", "cores": threads, "kind": "port",
            "sample": f"first {n} pairs of the workload, oracle/seqan_oracle.c with OpenMP over {threads} "
                      f"threads, best of 2", "cells": cells, "seconds": best}


def run_reference(args, rank):
    if rank != 0:
        return
    H, V, score, _, _ = make_workload(args.workload)
    from oracle import oracle as O
    pb = O.Problem("global", 0, None, score.match, score.mismatch, score.gap_open, score.gap_extend, None,
                   score.bits)
    threads = os.cpu_count() or 1
    n = min(len(H), args.ref_pairs)
    cells = int(sum(len(h) * len(v) for h, v in zip(H[:n], V[:n])))
    for _ in range(args.warmup):
        O.oracle_batch(pb, H[:n], V[:n], threads=threads)
    times = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        O.oracle_batch(pb, H[:n], V[:n], threads=threads)
        times.append(time.perf_counter() - t0)
    total = sum(times)
    gcups = cells * len(times) / total / 1e9
    line = {"metric": "GCUPS, batched affine DNA align", "value": gcups, "unit": "GCUPS", "n_gpus": 1,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * total / len(times),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "int16" if score.bits == 16 else "int32",
            "data": "synthetic", "impl": "reference",
            "config": {"workload": args.workload, "pairs_per_step": n, "description": WORKLOADS[args.workload]},
            "cpu_baseline": {"value": gcups, "unit": "GCUPS", "cores": threads, "kind": "port",
                             "sample": f"first {n} pairs of the workload per step; the reference's own SIMD "
                                       "path is x86-only and cannot build on the Arm host, so its CPU "
                                       "restatement (oracle/seqan_oracle.c) runs with OpenMP"},
            "e2e": {"value": gcups, "unit": "GCUPS", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--workload", default="affine_dna_100k", choices=sorted(WORKLOADS))
    ap.add_argument("--ref-pairs", type=int, default=20000)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-plain", action="store_true", help="skip the plain per-bucket comparison")
    ap.add_argument("--kernel", default="auto", choices=["auto", "general", "packed16", "plain"],
                    help="auto: persistent packed 16-bit kernel (32-row strips), graph-replayed; "
                         "plain: general kernel, one launch per length bucket")
    args = ap.parse_args()

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))
    dist = None
    if world > 1:
        import torch
        import torch.distributed as dist
        os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    if args.impl == "reference":
        run_reference(args, rank)
        if dist:
            dist.barrier()
        return

    import seqan_gb300 as sg
    from seqan_gb300 import _native as N
    N.build()
    L = N.lib()
    ctx = N.Context(local_rank)
    h = ctx.handle

    H, V, score, mode, kind = make_workload(args.workload, seed_offset=rank)
    sh, oh = concat(H)
    sv, ov = concat(V)
    npairs = len(H)
    cells = int(((oh[1:] - oh[:-1]) * (ov[1:] - ov[:-1])).sum())

    def pinned(nbytes):
        p = C.c_void_p()
        ctx.check(L.gba_host_alloc(h, C.byref(p), nbytes), "gba_host_alloc")
        return p

    def device(nbytes):
        p = C.c_void_p()
        ctx.check(L.gba_device_alloc(h, C.byref(p), nbytes), "gba_device_alloc")
        return p

    def as_np(ptr, count, dtype):
        return np.ctypeslib.as_array(C.cast(ptr, C.POINTER(np.ctypeslib.as_ctypes_type(dtype))), shape=(count,))

    # Pinned host copies of the inputs and outputs (the e2e path's host buffers).
    p_sh, p_sv = pinned(sh.nbytes), pinned(sv.nbytes)
    p_oh, p_ov = pinned(oh.nbytes), pinned(ov.nbytes)
    as_np(p_sh, sh.size, np.uint8)[:] = sh
    as_np(p_sv, sv.size, np.uint8)[:] = sv
    as_np(p_oh, oh.size, np.int64)[:] = oh
    as_np(p_ov, ov.size, np.int64)[:] = ov
    p_score, p_eh, p_ev = pinned(npairs * 4), pinned(npairs * 4), pinned(npairs * 4)

    flags = {"auto": N.GBA_FLAG_AUTOTUNE, "general": N.GBA_FLAG_GENERAL_KERNEL, "packed16": N.GBA_FLAG_STRIP16,
             "plain": N.GBA_FLAG_PLAIN_BUCKETS | N.GBA_FLAG_NO_GRAPH}[args.kernel]
    params = sg.align.make_params(score, mode, None, None, N.GBA_OUT_SCORE | N.GBA_OUT_END,
                                  alphabet_size=4, flags=flags)
    host_batch = N.GbaBatch(npairs, p_sh, p_oh, p_sv, p_ov, 0, 0)

    # Device-resident inputs for `value`.
    d_sh, d_sv = device(sh.nbytes), device(sv.nbytes)
    ctx.check(L.gba_copy_to_device(h, d_sh, p_sh, sh.nbytes), "copy")
    ctx.check(L.gba_copy_to_device(h, d_sv, p_sv, sv.nbytes), "copy")
    d_score, d_eh, d_ev = device(npairs * 4), device(npairs * 4), device(npairs * 4)
    dev_batch = N.GbaBatch(npairs, d_sh, None, d_sv, None, 0, 0)
    dev_res = N.GbaResult()
    dev_res.score, dev_res.end_h, dev_res.end_v = d_score, d_eh, d_ev
    plan = C.c_void_p()
    ctx.check(L.gba_plan_create(h, C.byref(params), C.byref(host_batch), C.byref(plan)), "gba_plan_create")

    flush_bytes = 256 << 20
    d_flush = device(flush_bytes)
    p_flush = pinned(flush_bytes)

    def flush_l2():
        ctx.check(L.gba_copy_to_device(h, d_flush, p_flush, flush_bytes), "flush")
        ctx.check(L.gba_synchronize(h), "sync")

    def barrier():
        if dist:
            dist.barrier()

    for _ in range(args.warmup):
        ctx.check(L.gba_plan_execute(h, plan, C.byref(dev_batch), C.byref(dev_res)), "execute")
        ctx.check(L.gba_synchronize(h), "sync")

    sampler = ClockSampler(local_rank)
    barrier()
    ctx.check(L.gba_synchronize(h), "sync")
    sampler.start()
    step_ms, dp_ms, launches = [], [], 0
    ms = C.c_float()
    tile = None
    for _ in range(args.steps):
        flush_l2()
        ctx.check(L.gba_timer_start(h), "timer")
        ctx.check(L.gba_plan_execute(h, plan, C.byref(dev_batch), C.byref(dev_res)), "execute")
        ctx.check(L.gba_timer_stop(h, C.byref(ms)), "timer")
        step_ms.append(ms.value)
        st = ctx.stats()
        dp_ms.append(st.dp_kernel_ms)
        launches += st.kernel_launches
        tile = {"rows_per_strip": st.tile_rows, "min_blocks_per_sm": st.tile_min_blocks}
    ctx.check(L.gba_synchronize(h), "sync")
    barrier()
    clocks = sampler.stop()
    total_ms = sum(step_ms)
    if dist:
        import torch
        t = torch.tensor([total_ms], dtype=torch.float64, device=f"cuda:{local_rank}")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        total_ms = float(t.item())
    value = cells * world * args.steps / (total_ms * 1e-3) / 1e9

    # The plain GPU form on the same device-resident batch: the general one-pair-per-thread
    # kernel, one launch per 8-residue length bucket (comparison for the persistent form).
    plain = None
    if args.kernel == "auto" and not args.no_plain:
        pparams = sg.align.make_params(score, mode, None, None, N.GBA_OUT_SCORE | N.GBA_OUT_END, alphabet_size=4,
                                       flags=N.GBA_FLAG_PLAIN_BUCKETS | N.GBA_FLAG_NO_GRAPH)
        pplan = C.c_void_p()
        ctx.check(L.gba_plan_create(h, C.byref(pparams), C.byref(host_batch), C.byref(pplan)), "plain plan")
        ctx.check(L.gba_plan_execute(h, pplan, C.byref(dev_batch), C.byref(dev_res)), "plain")
        ctx.check(L.gba_synchronize(h), "sync")
        pms = []
        for _ in range(2):
            flush_l2()
            ctx.check(L.gba_timer_start(h), "timer")
            ctx.check(L.gba_plan_execute(h, pplan, C.byref(dev_batch), C.byref(dev_res)), "plain")
            ctx.check(L.gba_timer_stop(h, C.byref(ms)), "timer")
            pms.append(ms.value)
        plain_launches = ctx.stats().kernel_launches
        L.gba_plan_destroy(h, pplan)
        pg = cells / (sum(pms) / len(pms) * 1e-3) / 1e9
        plain = {"value": pg, "unit": "GCUPS", "launches_per_step": plain_launches,
                 "speedup_of_value": value / pg,
                 "form": "general one-pair-per-thread kernel, one launch per 8-residue length bucket"}

    # End to end through the public C-ABI call with host buffers.
    host_res = N.GbaResult()
    host_res.score, host_res.end_h, host_res.end_v = p_score, p_eh, p_ev
    for _ in range(max(1, args.warmup)):
        ctx.check(L.gba_align_batch(h, C.byref(params), C.byref(host_batch), C.byref(host_res)), "e2e")
    e2e_s = []
    for _ in range(args.steps):
        flush_l2()
        t0 = time.perf_counter()
        ctx.check(L.gba_align_batch(h, C.byref(params), C.byref(host_batch), C.byref(host_res)), "e2e")
        e2e_s.append(time.perf_counter() - t0)
    est = ctx.stats()
    e2e_launches = est.kernel_launches
    e2e_breakdown = {"host_plan_ms": est.host_plan_ms, "dp_kernel_ms": est.dp_kernel_ms, "call_ms": est.call_ms}
    e2e_gcups = cells * world * len(e2e_s) / sum(e2e_s) / 1e9
    h2d = sh.nbytes + sv.nbytes
    d2h = 3 * npairs * 4

    # Roofline of the DP kernel: integer add/max ops against the measured integer rate.
    peak = C.c_double()
    ctx.check(L.gba_measure_int_peak(h, C.byref(peak)), "int peak")
    dp_avg_ms = sum(dp_ms) / len(dp_ms)
    ops = cells * OPS_PER_CELL[kind]
    achieved = ops / (dp_avg_ms * 1e-3) / 1e12
    roofline = {"bound": "int32", "achieved": achieved, "peak": peak.value, "unit": "Tops/s",
                "frac": achieved / peak.value if peak.value else None, "traffic": None,
                "kernel": "k_dp_strip (one pair per thread, int32)" if args.kernel == "general" else
                          "k_pack16 + k_dp16x2 (two pairs per thread, DPX int16x2)", "ops_per_cell": OPS_PER_CELL[kind],
                "dp_kernel_ms": dp_avg_ms,
                "peak_source": "measured live by gba_measure_int_peak (32-bit add+max issue rate)"}

    line = {"metric": "GCUPS, batched affine DNA align", "value": value, "unit": "GCUPS", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": total_ms / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "int16" if score.bits == 16 else "int32", "data": "synthetic",
            "config": {"workload": args.workload, "description": WORKLOADS[args.workload], "pairs": npairs,
                       "cells_per_step": cells, "l2": "flushed (256 MiB write) between timed steps",
                       "kernel": args.kernel,
                       "parallelism": f"replicas x{world} (pairs are independent)"},
            "e2e": {"value": e2e_gcups, "unit": "GCUPS", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                    "ms_per_step": 1e3 * sum(e2e_s) / len(e2e_s), "last_call": e2e_breakdown},
            "gpu_launches": launches, "roofline": roofline, "clocks": clocks}
    if tile:
        line["config"]["tiling"] = tile
    if plain:
        line["plain_gpu_form"] = plain
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(H, V, score, kind)
    L.gba_plan_destroy(h, plan)
    for p in (d_sh, d_sv, d_score, d_eh, d_ev, d_flush):
        L.gba_device_free(h, p)
    for p in (p_sh, p_sv, p_oh, p_ov, p_score, p_eh, p_ev, p_flush):
        L.gba_host_free(h, p)
    if rank == 0:
        print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
