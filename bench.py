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
  integer-issue bound; add and max each count one op: affine global 9 ops per cell, affine
  local 10, linear global 5, linear local 6).
* ``plain_gpu_form``: the same kernels launched once per 8-residue length bucket (no sorting
  across buckets, no split slots, no autotune, no graph) -- what the persistent, length-sorted,
  graph-replayed batch is compared with.
* ``parity``: every pair of the timed runs (device-resident and end to end) compared with the
  oracle, outside the timed regions; the run exits non-zero when any result differs.
* ``cpu_baseline``: the oracle (CPU restatement of the reference, OpenMP over all host cores)
  timed on a sample of the same workload.
``--impl reference`` times the reference's own batch call (SeqAn compiled from its headers on
this host) when its headers are available, else the CPU restatement, in the same JSON shape.
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
    "affine_dna_100k": "100000 pairs, read length uniform in [100,300], partner 5% subs + 1% indels, "
                       "Score(2,-4,-1,-6) int16, global, score + end position",
    "linear_dna_1024x150": "1024 pairs of uniform ACGT, both length 150, Score(2,-3,-5) int32, global, score",
    "protein_local_tb_20k": "20000 protein pairs, log-normal lengths (median 300, sigma 0.5, [50,1000]), 30% "
                            "related at 40% identity, Blosum62(-1,-11) int16, local, score + begin/end + "
                            "trace segments (Gaps)",
    "banded_reads_1m": "1000000 reads of 150 bp (2% subs, 0.2% indels) vs 170 bp windows of a 10 Mbp "
                       "reference, AlignConfig<true,false,false,true>, band [-6,26], Score(2,-4,-1,-6) int16, "
                       "score + CIGAR",
    "xdrop_reads_1m": "1000000 seeds: 150 bp reads (3% subs, 0.3% indels) vs 250 bp windows of a 10 Mbp "
                      "reference, one 19-mer seed per read on its true diagonal; extendSeed EXTEND_BOTH, "
                      "GappedXDrop, Score<int,Simple>(1,-2,-2), scoreDropOff 20; seeds + extension scores",
}
SEED_WORKLOADS = {"xdrop_reads_1m"}
WORKLOADS["extend_reads_250k"] = ("250000 read alignments: 150 bp reads (3% subs, 0.3% indels) in 250 bp windows of a "
                                  "10 Mbp reference, the aligned part a 19-mer seed on the true diagonal; "
                                  "extendAlignment EXTEND_BOTH, xDrop 20, Score<int,Simple>(2,-4,-1,-6); scores + "
                                  "trace segments of both sides")
EXTEND_WORKLOADS = {"extend_reads_250k"}
WORKLOADS["waterman_eggert_10k"] = ("10000 DNA pairs of 100-200 bp (half related: 10% subs, 2% indels), "
                                    "LocalAlignmentEnumerator<Score<int,Simple>(2,-1,-2,-2), Unbanded>, cutoff 10, "
                                    "up to 10 suboptimal local alignments per pair (scores, rows, positions)")
WORKLOADS["waterman_eggert_banded_10k"] = ("the same 10000 DNA pairs, LocalAlignmentEnumerator<Score<int,Simple>"
                                           "(2,-1,-2,-2), Banded> over diagonals -16..16, cutoff 10, up to 10 "
                                           "suboptimal local alignments per pair")
WE_WORKLOADS = {"waterman_eggert_10k", "waterman_eggert_banded_10k"}
WE_BAND = {"waterman_eggert_banded_10k": (-16, 16)}
WORKLOADS["banded_chain_20k"] = ("20000 genomic pairs of 1-3 kbp (5% subs, 1% indels) with LAGAN-style anchor chains (the "
                                 "exact matches of >= 20 bp on the true alignment, at most 64 per pair, 35 on average), "
                                 "bandedChainAlignment(align, chain, Score<int,Simple>(2,-3,-1,-5), AlignConfig<>(), 15): "
                                 "score + trace segments (the Align rows) per pair")
CHAIN_WORKLOADS = {"banded_chain_20k"}
CHAIN_SCORE, CHAIN_K = (2, -3, -1, -5), 15
WORKLOADS["sam_records_1m"] = ("1000000 SAM records of read alignments: names read<k>, flag 0/16, one contig, "
                               "positions < 10^7, MAPQ 60, 1-3 CIGAR operations, 150 bp SEQ and QUAL; "
                               "BamAlignmentRecord -> SAM text as the reference's writer")
SAM_WORKLOADS = {"sam_records_1m"}
WORKLOADS["fasta_reads_2m"] = ("FASTA text of 2000000 reads of 150 bp (ids 'read<k> len=150', sequences in lines of 80 "
                               "columns, 3% lower case, 0.1% N), about 345 MB; readRecord loop into Dna5 codes + "
                               "record offsets")
FASTA_WORKLOADS = {"fasta_reads_2m"}
WORKLOADS["dynamic_dna_tb_100k"] = ("the 100000 pairs of affine_dna_100k with DynamicGaps cells (one score and two gap "
                                    "flags per cell; align/dp_formula_dynamic.h), Score(2,-4,-1,-6) int16, global, score + "
                                    "end position + trace segments")
WORKLOADS["bam_records_1m"] = ("the 1000000 records of sam_records_1m as uncompressed BAM blocks "
                               "(write(target, record, context, Bam()), no tags); the line's bgzf key times the "
                               "blocks' BGZF compression")
BAM_WORKLOADS = {"bam_records_1m"}


def run_bam_bench(args, rank, world, local_rank, dist):
    from seqan_gb300 import _native as N
    from oracle import oracle as O
    N.build()
    L = N.lib()
    ctx = N.Context(local_rank)
    h = ctx.handle
    n = args.pairs or 1_000_000
    rec = make_sam_records(n, seed=21 + rank)
    a = O.sam_arrays(rec)
    pinned_bufs = {}
    for key, arr in a.items():
        if arr is None:   # no tags: the records struct's tag fields stay NULL
            continue
        p = C.c_void_p()
        ctx.check(L.gba_host_alloc(h, C.byref(p), max(arr.nbytes, 1)), "alloc")
        C.memmove(p, arr.ctypes.data, arr.nbytes)
        pinned_bufs[key] = p
    P = pinned_bufs
    r = N.GbaSamRecords(n, P["qname"], P["qoff"], P["flag"], P["rid"], P["pos"], P["mapq"], P["cigar"], P["coff"],
                        P["rnext"], P["pnext"], P["tlen"], P["seq"], P["soff"], P["letters"], P["qual"], P["quoff"],
                        P["cnames"], P["cnoff"], len(rec.contigs))
    rec_off = np.zeros(n + 1, np.int64)
    L.gba_format_bam(h, C.byref(r), None, 0, rec_off.ctypes.data)
    total = int(rec_off[-1])
    p_out = C.c_void_p()
    ctx.check(L.gba_host_alloc(h, C.byref(p_out), total + 16), "alloc")

    def call():
        ctx.check(L.gba_format_bam(h, C.byref(r), p_out, total + 16, rec_off.ctypes.data), "bam")

    for _ in range(args.warmup):
        call()
    sampler = ClockSampler(local_rank)
    sampler.start()
    wall, kern = [], []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        call()
        wall.append(time.perf_counter() - t0)
        kern.append(ctx.stats().dp_kernel_ms)
    clocks = sampler.stop()
    data = C.string_at(p_out, total)
    threads = os.cpu_count() or 1
    parity = data == O.oracle_write_bam_c(rec, threads=threads, arrays=a)
    kernel_ms = sum(kern) / len(kern)
    value = n * world / (kernel_ms * 1e-3) / 1e6
    e2e = n * world * len(wall) / sum(wall) / 1e6
    hbm = measured_hbm_gbs()
    in_bytes = sum(int(x.nbytes) for x in a.values() if x is not None)
    line = {"metric": "M BAM records/s, device formatting", "value": value, "unit": "M records/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": kernel_ms, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "u8", "data": "synthetic",
            "config": {"workload": args.workload, "description": WORKLOADS[args.workload], "records": n,
                       "bam_bytes": total, "parallelism": f"replicas x{world}"},
            "e2e": {"value": e2e, "unit": "M records/s", "h2d_bytes_per_step": in_bytes,
                    "d2h_bytes_per_step": total + 8 * (n + 1), "ms_per_step": 1e3 * sum(wall) / len(wall)},
            "gpu_launches": args.steps * 4,
            "roofline": {"bound": "hbm", "achieved": (in_bytes + total) / (kernel_ms * 1e-3) / 1e9,
                         "peak": hbm, "unit": "GB/s",
                         "frac": ((in_bytes + total) / (kernel_ms * 1e-3) / 1e9 / hbm) if hbm else None,
                         "traffic": None, "kernel": "k_bam_lengths + CUB scan + k_bam_write",
                         "algorithmic_bytes": "record fields read once + BAM blocks written once",
                         "peak_source": "MEASURED_PEAKS.json hbm_gbs (of measured)"},
            "clocks": clocks, "parity_vs_oracle": parity}
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        best = None
        for _ in range(2):
            t0 = time.perf_counter()
            O.oracle_write_bam_c(rec, threads=threads, arrays=a)
            dt = time.perf_counter() - t0
            best = dt if best is None else min(best, dt)
        line["cpu_baseline"] = {"value": n / best / 1e6, "unit": "M records/s", "cores": threads, "kind": "port",
                                "sample": f"all {n} records, orc_write_bam (oracle/seqan_oracle.c, the reference's "
                                          f"BAM writer restated) with OpenMP over {threads} threads, best of 2",
                                "seconds": best}
    line["bgzf"] = bgzf_measure(ctx, data, args, threads)
    for p in list(pinned_bufs.values()) + [p_out]:
        L.gba_host_free(h, p)
    if rank == 0:
        print(json.dumps(line), flush=True)


def bgzf_measure(ctx, data: bytes, args, threads: int) -> dict:
    """The BAM blocks as a BGZF file (gba_bgzf_compress, the BgzfFile stream under BamFileOut):
    device kernel rate, the whole call from host buffers, the size ratio, whether every member
    inflates to its page, and zlib level 1 (the reference's deflateInit2(Z_BEST_SPEED) per 65,505-byte
    page) on the host threads as the CPU side."""
    import gzip
    import zlib
    from concurrent.futures import ThreadPoolExecutor
    from seqan_gb300 import _native as N
    L = N.lib()
    n = len(data)
    src = np.frombuffer(data, np.uint8)
    cap = n + 64 * (n // 65505 + 2) + 64
    out = np.zeros(cap, np.uint8)
    olen = C.c_int64()

    def call():
        ctx.check(L.gba_bgzf_compress(ctx.handle, src.ctypes.data, n, 1, out.ctypes.data, cap, C.byref(olen)), "bgzf")

    for _ in range(max(args.warmup, 1)):
        call()
    wall, kern = [], []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        call()
        wall.append(time.perf_counter() - t0)
        kern.append(ctx.stats().dp_kernel_ms)
    z = bytes(out[:olen.value])
    res = {"value": n / (sum(kern) / len(kern) * 1e-3) / 1e9, "unit": "GB/s of BAM bytes", "input_bytes": n,
           "output_bytes": len(z), "ratio": len(z) / max(n, 1), "e2e_gbs": n * len(wall) / sum(wall) / 1e9,
           "kernel": "k_bgzf_members (one warp per member) + k_bgzf_pack", "inflates_equal": gzip.decompress(z) == data,
           "timing": "CUDA events around k_bgzf_members; e2e = the whole call from host buffers"}
    if not args.no_cpu_baseline:
        pages = [data[i:i + 65505] for i in range(0, n, 65505)]

        def deflate(page):
            c = zlib.compressobj(1, zlib.DEFLATED, -15, 8)
            return c.compress(page) + c.flush()

        with ThreadPoolExecutor(threads) as ex:
            t0 = time.perf_counter()
            zs = list(ex.map(deflate, pages))
            dt = time.perf_counter() - t0
        res["cpu_zlib_level1"] = {"value": n / dt / 1e9, "unit": "GB/s", "cores": threads,
                                  "ratio": (sum(len(x) for x in zs) + 26 * len(pages) + 28) / max(n, 1),
                                  "sample": "every page through zlib level 1 (Python's zlib, threads over pages)"}
    return res


def run_bam_reference(args):
    from oracle import oracle as O
    n = min(args.pairs or 1_000_000, 1_000_000)
    rec = make_sam_records(n)
    a = O.sam_arrays(rec)
    threads = os.cpu_count() or 1
    for _ in range(args.warmup):
        O.oracle_write_bam_c(rec, threads=threads, arrays=a)
    times = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        O.oracle_write_bam_c(rec, threads=threads, arrays=a)
        times.append(time.perf_counter() - t0)
    rate = n * len(times) / sum(times) / 1e6
    print(json.dumps({"metric": "M BAM records/s, device formatting", "value": rate, "unit": "M records/s",
                      "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
                      "ms_per_step": 1e3 * sum(times) / len(times), "higher_is_better": True, "scaling": "weak",
                      "vs_baseline": None, "dtype": "u8", "data": "synthetic", "impl": "reference",
                      "config": {"workload": args.workload, "records_per_step": n,
                                 "description": WORKLOADS[args.workload]},
                      "cpu_baseline": {"value": rate, "unit": "M records/s", "cores": threads, "kind": "port",
                                       "sample": f"{n} records per step, the reference's BAM writer restated in C "
                                                 "(orc_write_bam), OpenMP"},
                      "e2e": {"value": rate, "unit": "M records/s", "h2d_bytes_per_step": 0,
                              "d2h_bytes_per_step": 0}}), flush=True)


def fasta_reads_text(n, seed=3):
    """FASTA text of n random 150 bp reads, each sequence wrapped into lines of 80 + 70 columns."""
    rng = np.random.default_rng(seed)
    codes = rng.integers(0, 4, (n, 150), dtype=np.uint8)
    codes[rng.random((n, 150)) < 0.001] = 4
    letters = np.frombuffer(b"ACGTN", np.uint8)[codes]
    letters[rng.random((n, 150)) < 0.03] += 32
    rows = np.empty((n, 152), np.uint8)
    rows[:, :80] = letters[:, :80]
    rows[:, 80] = 10
    rows[:, 81:151] = letters[:, 80:]
    rows[:, 151] = 10
    heads = [b">read%d len=150\n" % k for k in range(n)]
    hl = np.fromiter((len(h) for h in heads), np.int64, n)
    out = np.empty(int(hl.sum()) + 152 * n, np.uint8)
    starts = np.zeros(n, np.int64)
    np.cumsum(hl[:-1] + 152, out=starts[1:])
    hb = np.frombuffer(b"".join(heads), np.uint8)
    hoff = np.zeros(n, np.int64)
    np.cumsum(hl[:-1], out=hoff[1:])
    idx = np.repeat(starts - hoff, hl) + np.arange(len(hb))
    out[idx] = hb
    ridx = (starts + hl)[:, None] + np.arange(152)[None, :]
    out[ridx.ravel()] = rows.ravel()
    return out.tobytes(), codes


def fastq_reads_text(codes, seed=4):
    """FASTQ text of the reads (one sequence line, '+', one quality line per record)."""
    rng = np.random.default_rng(seed)
    n, L = codes.shape
    letters = np.frombuffer(b"ACGTN", np.uint8)[codes]
    quals = rng.integers(33, 74, (n, L), dtype=np.uint8)
    heads = [b"@read%d\n" % k for k in range(n)]
    hl = np.fromiter((len(h) for h in heads), np.int64, n)
    body = 2 * L + 4   # sequence, '\n+\n', qualities, '\n'
    rows = np.empty((n, body), np.uint8)
    rows[:, :L] = letters
    rows[:, L:L + 3] = np.frombuffer(b"\n+\n", np.uint8)
    rows[:, L + 3:2 * L + 3] = quals
    rows[:, 2 * L + 3] = 10
    out = np.empty(int(hl.sum()) + body * n, np.uint8)
    starts = np.zeros(n, np.int64)
    np.cumsum(hl[:-1] + body, out=starts[1:])
    hb = np.frombuffer(b"".join(heads), np.uint8)
    hoff = np.zeros(n, np.int64)
    np.cumsum(hl[:-1], out=hoff[1:])
    out[np.repeat(starts - hoff, hl) + np.arange(len(hb))] = hb
    out[((starts + hl)[:, None] + np.arange(body)[None, :]).ravel()] = rows.ravel()
    return out.tobytes()


def time_fastq_host(L, text, n_reads, reps=3):
    """gba_read_fastq (the host FASTQ reader) on the text: GB/s of text, best of reps."""
    from seqan_gb300 import _native as N
    n = len(text)
    buf = np.frombuffer(text, np.uint8)
    ib, ie, so, qe = (np.zeros(n_reads + 1, np.int64) for _ in range(4))
    codes = np.zeros(n, np.uint8)
    quals = np.zeros(n, np.uint8)
    r = N.GbaSeqRecords(n_reads + 1, n, ib.ctypes.data, ie.ctypes.data, so.ctypes.data, qe.ctypes.data,
                        codes.ctypes.data, quals.ctypes.data, 0, 0, -1)
    best = None
    for _ in range(reps):
        t0 = time.perf_counter()
        rc = L.gba_read_fastq(None, buf.ctypes.data, n, 5, C.byref(r))
        dt = time.perf_counter() - t0
        best = dt if best is None else min(best, dt)
    return (n / best / 1e9 if rc == N.GBA_OK and r.num == n_reads else None), codes[:r.residues]


def run_fasta_bench(args, rank, world, local_rank, dist):
    from seqan_gb300 import _native as N
    from oracle import oracle as O
    N.build()
    L = N.lib()
    ctx = N.Context(local_rank)
    h = ctx.handle
    n_reads = args.pairs or 2_000_000
    text, codes = fasta_reads_text(n_reads, seed=3 + rank)
    n = len(text)

    def pinned(nbytes):
        p = C.c_void_p()
        ctx.check(L.gba_host_alloc(h, C.byref(p), max(nbytes, 16)), "alloc")
        return p

    p_text = pinned(n)
    C.memmove(p_text, text, n)
    cap = n_reads + 1
    p_ib, p_ie, p_so, p_codes = pinned(8 * cap), pinned(8 * cap), pinned(8 * cap), pinned(n)
    r = N.GbaSeqRecords(cap, n, p_ib, p_ie, p_so, None, p_codes, None, 0, 0, -1)

    def call():
        ctx.check(L.gba_read_fasta(h, p_text, n, 5, C.byref(r)), "gba_read_fasta")

    for _ in range(args.warmup):
        call()
    sampler = ClockSampler(local_rank)
    sampler.start()
    wall, kern = [], []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        call()
        wall.append(time.perf_counter() - t0)
        kern.append(ctx.stats().dp_kernel_ms)
    clocks = sampler.stop()
    got = np.ctypeslib.as_array(C.cast(p_codes, C.POINTER(C.c_uint8)), (r.residues,))
    so = np.ctypeslib.as_array(C.cast(p_so, C.POINTER(C.c_int64)), (r.num + 1,))
    parity = bool(r.num == n_reads and np.array_equal(got, codes.ravel()) and np.array_equal(
        so, np.arange(n_reads + 1, dtype=np.int64) * 150))
    k = min(n_reads, 20_000)
    cut = text.index(b">read%d " % k) if k < n_reads else n
    want = O.oracle_read_records(text[:cut], "fasta", "dna5")
    ib = np.ctypeslib.as_array(C.cast(p_ib, C.POINTER(C.c_int64)), (k,))
    ie = np.ctypeslib.as_array(C.cast(p_ie, C.POINTER(C.c_int64)), (k,))
    parity = parity and all(text[ib[j]:ie[j]] == want[j][0] for j in range(k))
    kernel_ms = sum(kern) / len(kern)
    gb = n * world / 1e9
    value = gb / (kernel_ms * 1e-3)
    e2e = gb * len(wall) / sum(wall)
    hbm = measured_hbm_gbs()
    out_bytes = int(r.residues) + 24 * int(r.num)
    achieved = (n + out_bytes) / (kernel_ms * 1e-3) / 1e9
    line = {"metric": "GB/s of FASTA text read into records", "value": value, "unit": "GB/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": kernel_ms, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "u8", "data": "synthetic",
            "config": {"workload": args.workload, "description": WORKLOADS[args.workload], "records": n_reads,
                       "text_bytes": n, "residues": int(r.residues), "parallelism": f"replicas x{world}",
                       "l2": "text larger than L2"},
            "e2e": {"value": e2e, "unit": "GB/s", "h2d_bytes_per_step": n, "d2h_bytes_per_step": out_bytes,
                    "ms_per_step": 1e3 * sum(wall) / len(wall)},
            "gpu_launches": args.steps * 4,
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": hbm, "unit": "GB/s",
                         "frac": achieved / hbm if hbm else None, "traffic": None,
                         "kernel": "k_fasta_summary + k_fasta_scan_tiles + k_fasta_scan_top + k_fasta_write",
                         "algorithmic_bytes": "text read once + codes and 3 x 8 B per record written once",
                         "peak_source": "MEASURED_PEAKS.json hbm_gbs (of measured)"},
            "clocks": clocks, "parity_vs_generated_codes_and_oracle_ids": parity}
    fq = fastq_reads_text(codes)
    fq_gbs, fq_codes = time_fastq_host(L, fq, n_reads)
    line["fastq_host"] = {"value": fq_gbs, "unit": "GB/s", "text_bytes": len(fq), "cores": os.cpu_count() or 1,
                          "reader": "gba_read_fastq (host threads: speculative record starts per slice, each "
                                    "checked against the previous slice's reading, sequential fallback)",
                          "parity_vs_generated_codes": bool(np.array_equal(fq_codes, codes.ravel()))}
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        best = None
        for _ in range(2):
            t0 = time.perf_counter()
            O.oracle_read_records(text, "fasta", "dna5", raw=True)
            dt = time.perf_counter() - t0
            best = dt if best is None else min(best, dt)
        line["cpu_baseline"] = {"value": n / best / 1e9, "unit": "GB/s", "cores": 1, "kind": "port",
                                "sample": f"the whole {n} byte text, orc_read_records (oracle/seqan_oracle.c, the "
                                          "reference's readRecord loop restated; sequential as the reference's "
                                          "reader), best of 2",
                                "seconds": best}
    for p in (p_text, p_ib, p_ie, p_so, p_codes):
        L.gba_host_free(h, p)
    if rank == 0:
        print(json.dumps(line), flush=True)


def run_fasta_reference(args):
    from oracle import oracle as O
    n_reads = args.pairs or 2_000_000
    text, _ = fasta_reads_text(n_reads)
    for _ in range(args.warmup):
        O.oracle_read_records(text, "fasta", "dna5", raw=True)
    times = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        O.oracle_read_records(text, "fasta", "dna5", raw=True)
        times.append(time.perf_counter() - t0)
    rate = len(text) * len(times) / sum(times) / 1e9
    print(json.dumps({"metric": "GB/s of FASTA text read into records", "value": rate, "unit": "GB/s",
                      "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
                      "ms_per_step": 1e3 * sum(times) / len(times), "higher_is_better": True, "scaling": "weak",
                      "vs_baseline": None, "dtype": "u8", "data": "synthetic", "impl": "reference",
                      "config": {"workload": args.workload, "text_bytes": len(text),
                                 "description": WORKLOADS[args.workload]},
                      "cpu_baseline": {"value": rate, "unit": "GB/s", "cores": 1, "kind": "port",
                                       "sample": "the whole text per step, the reference's readRecord loop restated "
                                                 "in C (orc_read_records), sequential as the reference's reader"},
                      "e2e": {"value": rate, "unit": "GB/s", "h2d_bytes_per_step": 0,
                              "d2h_bytes_per_step": 0}}), flush=True)


def make_sam_records(n, seed=21):
    from seqan_gb300 import sam as S
    rng = np.random.Generator(np.random.PCG64(seed))
    L = 150
    seqs = list(rng.integers(0, 4, size=(n, L), dtype=np.uint8))
    qual_chars = rng.integers(33, 75, size=(n, L), dtype=np.uint8)
    quals = [bytes(q).decode() for q in qual_chars]
    cig = []
    for k in range(n):
        if k % 3 == 0:
            cig.append(np.array([(L << 4) | 0], np.uint32))
        else:
            a = int(rng.integers(20, 120))
            cig.append(np.array([(a << 4) | 0, (1 << 4) | (1 + k % 2), ((L - a - (1 if k % 2 else 0)) << 4) | 0],
                                np.uint32))
    return S.SamRecords([f"read{k}" for k in range(n)], rng.choice([0, 16], n).astype(np.uint16),
                        np.zeros(n, np.int32), rng.integers(0, 10_000_000, n).astype(np.int32),
                        np.full(n, 60, np.uint8), cig, np.full(n, -1, np.int32), np.full(n, -1, np.int32),
                        np.zeros(n, np.int32), seqs, quals, ["chrSim"])


def run_sam_bench(args, rank, world, local_rank, dist):
    from seqan_gb300 import _native as N
    from oracle import oracle as O
    N.build()
    L = N.lib()
    ctx = N.Context(local_rank)
    h = ctx.handle
    n = args.pairs or 1_000_000
    rec = make_sam_records(n, seed=21 + rank)
    a = O.sam_arrays(rec)
    pinned_bufs = {}
    for key, arr in a.items():
        if arr is None:   # no tags: the records struct's tag fields stay NULL
            continue
        p = C.c_void_p()
        ctx.check(L.gba_host_alloc(h, C.byref(p), max(arr.nbytes, 1)), "alloc")
        C.memmove(p, arr.ctypes.data, arr.nbytes)
        pinned_bufs[key] = p
    P = pinned_bufs
    r = N.GbaSamRecords(n, P["qname"], P["qoff"], P["flag"], P["rid"], P["pos"], P["mapq"], P["cigar"], P["coff"],
                        P["rnext"], P["pnext"], P["tlen"], P["seq"], P["soff"], P["letters"], P["qual"], P["quoff"],
                        P["cnames"], P["cnoff"], len(rec.contigs))
    line_off = np.zeros(n + 1, np.int64)
    rc = L.gba_format_sam(h, C.byref(r), None, 0, line_off.ctypes.data)
    total = int(line_off[-1])
    p_out = C.c_void_p()
    ctx.check(L.gba_host_alloc(h, C.byref(p_out), total + 16), "alloc")

    def call():
        ctx.check(L.gba_format_sam(h, C.byref(r), p_out, total + 16, line_off.ctypes.data), "sam")

    for _ in range(args.warmup):
        call()
    sampler = ClockSampler(local_rank)
    sampler.start()
    wall, kern = [], []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        call()
        wall.append(time.perf_counter() - t0)
        kern.append(ctx.stats().dp_kernel_ms)
    clocks = sampler.stop()
    text = C.string_at(p_out, total).decode()
    k = min(n, 20_000)
    parity = text[:int(line_off[k])] == O.write_sam(type(rec)(rec.qname[:k], rec.flag[:k], rec.ref_id[:k], rec.pos[:k],
                                                               rec.mapq[:k], rec.cigar[:k], rec.next_ref_id[:k],
                                                               rec.next_pos[:k], rec.tlen[:k], rec.seq[:k],
                                                               rec.qual[:k], rec.contigs))
    kernel_ms = sum(kern) / len(kern)
    value = n * world / (kernel_ms * 1e-3) / 1e6
    e2e = n * world * len(wall) / sum(wall) / 1e6
    hbm = measured_hbm_gbs()
    in_bytes = sum(int(x.nbytes) for x in a.values() if x is not None)
    line = {"metric": "M SAM records/s, device formatting", "value": value, "unit": "M records/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": kernel_ms, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "u8", "data": "synthetic",
            "config": {"workload": args.workload, "description": WORKLOADS[args.workload], "records": n,
                       "text_bytes": total, "parallelism": f"replicas x{world}"},
            "e2e": {"value": e2e, "unit": "M records/s", "h2d_bytes_per_step": in_bytes, "d2h_bytes_per_step": total + 8 * (n + 1),
                    "ms_per_step": 1e3 * sum(wall) / len(wall)},
            "gpu_launches": args.steps * 4,
            "roofline": {"bound": "hbm", "achieved": (in_bytes + total) / (kernel_ms * 1e-3) / 1e9,
                         "peak": hbm, "unit": "GB/s",
                         "frac": ((in_bytes + total) / (kernel_ms * 1e-3) / 1e9 / hbm) if hbm else None,
                         "traffic": None, "kernel": "k_sam_lengths + CUB scan + k_sam_write",
                         "algorithmic_bytes": "record fields read once + SAM text written once",
                         "peak_source": "MEASURED_PEAKS.json hbm_gbs (of measured)"},
            "clocks": clocks, "parity_first_20000_vs_oracle": parity}
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        threads = os.cpu_count() or 1
        best = None
        for _ in range(2):
            t0 = time.perf_counter()
            O.oracle_write_sam_c(rec, threads=threads, arrays=a)
            dt = time.perf_counter() - t0
            best = dt if best is None else min(best, dt)
        line["cpu_baseline"] = {"value": n / best / 1e6, "unit": "M records/s", "cores": threads, "kind": "port",
                                "sample": f"all {n} records, orc_write_sam (oracle/seqan_oracle.c, the reference's "
                                          f"SAM writer restated) with OpenMP over {threads} threads, best of 2",
                                "seconds": best}
    for p in list(pinned_bufs.values()) + [p_out]:
        L.gba_host_free(h, p)
    if rank == 0:
        print(json.dumps(line), flush=True)


def run_sam_reference(args):
    from oracle import oracle as O
    n = min(args.pairs or 1_000_000, 1_000_000)
    rec = make_sam_records(n)
    a = O.sam_arrays(rec)
    threads = os.cpu_count() or 1
    for _ in range(args.warmup):
        O.oracle_write_sam_c(rec, threads=threads, arrays=a)
    times = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        O.oracle_write_sam_c(rec, threads=threads, arrays=a)
        times.append(time.perf_counter() - t0)
    rate = n * len(times) / sum(times) / 1e6
    print(json.dumps({"metric": "M SAM records/s, device formatting", "value": rate, "unit": "M records/s",
                      "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
                      "ms_per_step": 1e3 * sum(times) / len(times), "higher_is_better": True, "scaling": "weak",
                      "vs_baseline": None, "dtype": "u8", "data": "synthetic", "impl": "reference",
                      "config": {"workload": args.workload, "records_per_step": n,
                                 "description": WORKLOADS[args.workload]},
                      "cpu_baseline": {"value": rate, "unit": "M records/s", "cores": threads, "kind": "port",
                                       "sample": f"{n} records per step, the reference's SAM writer restated in C "
                                                 "(orc_write_sam), OpenMP"},
                      "e2e": {"value": rate, "unit": "M records/s", "h2d_bytes_per_step": 0,
                              "d2h_bytes_per_step": 0}}), flush=True)
# Integer ops of one x-drop cell: max(up, left) + gap, diagonal + score, the max of the two, the
# drop-off compare and the anti-diagonal best (add and max each count one).
XDROP_OPS_PER_CELL = 6
# Algorithmic integer ops per cell (add and max each count one): affine global 9
# (E: 2 adds + 1 max, F: 2 + 1, S: 1 add + 2 max), affine local 10 (+ max with 0),
# linear global 5, linear local 6.
OPS_PER_CELL = {"affine_global": 9, "linear_global": 5, "affine_local": 10, "linear_local": 6,
                # DynamicGaps: two flag-selected gap adds, the gap max, the diagonal add and max
                "dynamic_global": 5}


# DRAM traffic and ALU-pipe share of the DP kernel from the committed ncu captures (a bench run
# cannot profile itself): bytes read + written per algorithmic cell of the captured launch, scaled
# to the timed launch's cells for roofline.traffic.  Workloads without a capture report None.
CAPTURED = {
    "affine_dna_100k": {"dram_bytes_per_cell": (143.7e6 + 361.7e6) / 4.336e9, "alu_pipe_pct": 80.8,
                        "profile": "profiles/k_dp16x2_affine_dna_100k.md"},
    "banded_reads_1m": {"dram_bytes_per_cell": (367.6e6 + 837.0e6) / 9.816e8, "alu_pipe_pct": 57.5,
                        "profile": "profiles/k_dp_banded_reads_1m.md"},
    "protein_local_tb_20k": {"dram_bytes_per_cell": (13.5e6 + 626.4e6) / 9.732e8, "alu_pipe_pct": 78.9,
                             "profile": "profiles/k_dp_warp2_protein_local_tb.md"},
}

KERNEL_NAMES = [(2, "k_pack16 + k_dp16x2 (two pairs per thread, DPX int16x2)"),
                (16, "k_dp_warp2 (64 strips per warp in int16x2 halves, 4-bit trace)"),
                (4, "k_dp_warp (one warp per 256-row band, anti-diagonal front)"),
                (8, "k_dp_banded (one pair per thread, band in per-thread slots)"),
                (1, "k_dp_strip (one pair per thread, int32)"),
                (32, "k_dp_dynamic (DynamicGaps cells, one pair per thread, int32)")]


def measured_hbm_gbs():
    """The measured HBM copy rate of this GPU pool (MEASURED_PEAKS.json at the repo root), or None."""
    try:
        with open(os.path.join(os.path.dirname(os.path.abspath(__file__)), "MEASURED_PEAKS.json")) as f:
            return float(json.load(f)["hbm_gbs"])
    except (OSError, KeyError, ValueError):
        return None


def kernel_label(bits: int) -> str:
    """Names of the DP kernels a run launched (gba_stats.dp_kernels), the main one first."""
    return " + ".join(name for bit, name in KERNEL_NAMES if bits & bit) or "none"


class Spec:
    def __init__(self, H, V, score, mode, kind, config=None, band=None, traceback=False, cigar=False,
                 alphabet_size=4, dynamic=False):
        self.H, self.V, self.score, self.mode, self.kind = H, V, score, mode, kind
        self.config, self.band, self.traceback, self.cigar = config, band, traceback, cigar
        self.alphabet_size = alphabet_size
        self.dynamic = dynamic      # DynamicGaps cells

    @property
    def gaps(self):
        from seqan_gb300 import _native as N
        return N.GBA_GAPS_DYNAMIC if self.dynamic else N.GBA_GAPS_AUTO


def make_workload(name: str, seed_offset: int = 0) -> Spec:
    import seqan_gb300 as sg
    from seqan_gb300 import workloads as W
    if name == "affine_dna_100k":
        H, V = W.mutated_dna_pairs(100_000, 100, 300, 0.05, 0.01, seed=2 + seed_offset)
        return Spec(H, V, sg.Score(2, -4, -1, -6, dtype=np.int16), 0, "affine_global")
    if name == "linear_dna_1024x150":
        H, V = W.uniform_dna_pairs(1024, 150, seed=1 + seed_offset)
        return Spec(H, V, sg.Score(2, -3, -5, dtype=np.int32), 0, "linear_global")
    if name == "protein_local_tb_20k":
        H, V = W.protein_pairs(20_000, seed=3 + seed_offset)
        return Spec(H, V, sg.Blosum62(-1, -11, dtype=np.int16), 1, "affine_local", traceback=True,
                    alphabet_size=27)
    if name == "banded_reads_1m":
        wins, reads = W.read_windows(1_000_000, seed=4 + seed_offset)
        return Spec(wins, reads, sg.Score(2, -4, -1, -6, dtype=np.int16), 0, "affine_global",
                    config=sg.AlignConfig(True, False, False, True), band=(-6, 26), traceback=True, cigar=True)
    if name == "dynamic_dna_tb_100k":
        H, V = W.mutated_dna_pairs(100_000, 100, 300, 0.05, 0.01, seed=2 + seed_offset)
        return Spec(H, V, sg.Score(2, -4, -1, -6, dtype=np.int16), 0, "dynamic_global", traceback=True, dynamic=True)
    raise SystemExit(f"unknown workload {name}")


def oracle_problem(spec: Spec):
    from oracle import oracle as O
    fe = spec.config.bits if spec.config is not None else 0
    return O.Problem("local" if spec.mode == 1 else "global", fe, spec.band, spec.score.match,
                     spec.score.mismatch, spec.score.gap_open, spec.score.gap_extend, spec.score.matrix,
                     spec.score.bits, "aa" if spec.alphabet_size > 5 else "dna", dynamic=spec.dynamic)


def algorithmic_cells(spec: Spec) -> int:
    """m * n per pair; in-band cells (1 <= i <= n, 1 <= j <= m, lower <= j - i <= upper) when banded."""
    lh = np.fromiter((len(h) for h in spec.H), dtype=np.int64, count=len(spec.H))
    lv = np.fromiter((len(v) for v in spec.V), dtype=np.int64, count=len(spec.V))
    if spec.band is None:
        return int((lh * lv).sum())
    lo, up = spec.band
    total = 0
    for dg in range(lo, up + 1):
        total += np.clip(np.minimum(lv, lh - dg) - np.maximum(1, 1 - dg) + 1, 0, None).sum()
    return int(total)


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


def fetch_results(L, ctx, plan, npairs, d_score, d_eh, d_ev, spec, oh, ov):
    """Copies a device-resident run's results back: scores and best cells from the device
    buffers, begin positions, segments and CIGARs from the plan (gba_plan_fetch)."""
    h = ctx.handle
    out = {}
    for key, ptr in (("score", d_score), ("end_h", d_eh), ("end_v", d_ev)):
        a = np.zeros(npairs, np.int32)
        ctx.check(L.gba_copy_to_host(h, a.ctypes.data, ptr, 4 * npairs), "copy")
        out[key] = a
    if spec.traceback:
        from seqan_gb300 import _native as N
        cap = int(((oh[1:] - oh[:-1]) + (ov[1:] - ov[:-1]) + 4).sum()) + 1
        r = N.GbaResult()
        out["begin_h"], out["begin_v"] = np.zeros(npairs, np.int32), np.zeros(npairs, np.int32)
        out["segments"] = np.zeros((cap, 4), np.uint32)
        out["segment_offsets"] = np.zeros(npairs + 1, np.int64)
        r.begin_h, r.begin_v = out["begin_h"].ctypes.data, out["begin_v"].ctypes.data
        r.segments, r.segment_capacity = out["segments"].ctypes.data, cap
        r.segment_offsets = out["segment_offsets"].ctypes.data
        if spec.cigar:
            out["cigar"] = np.zeros(cap, np.uint32)
            out["cigar_offsets"] = np.zeros(npairs + 1, np.int64)
            r.cigar, r.cigar_capacity, r.cigar_offsets = out["cigar"].ctypes.data, cap, out["cigar_offsets"].ctypes.data
        ctx.check(L.gba_plan_fetch(h, plan, C.byref(r)), "gba_plan_fetch")
        out["segments"] = out["segments"][:int(out["segment_offsets"][-1])]
        if spec.cigar:
            out["cigar"] = out["cigar"][:int(out["cigar_offsets"][-1])]
    return out


def host_results(res, npairs, spec, as_np):
    """Copies of the results gba_align_batch (or a sibling call) left in pinned host buffers."""
    out = {k: as_np(getattr(res, k), npairs, np.int32).copy() for k in ("score", "end_h", "end_v")}
    if spec.traceback:
        out["begin_h"] = as_np(res.begin_h, npairs, np.int32).copy()
        out["begin_v"] = as_np(res.begin_v, npairs, np.int32).copy()
        out["segment_offsets"] = as_np(res.segment_offsets, npairs + 1, np.int64).copy()
        tot = int(out["segment_offsets"][-1])
        out["segments"] = as_np(res.segments, 4 * tot, np.uint32).reshape(-1, 4).copy()
        if spec.cigar:
            out["cigar_offsets"] = as_np(res.cigar_offsets, npairs + 1, np.int64).copy()
            out["cigar"] = as_np(res.cigar, int(out["cigar_offsets"][-1]), np.uint32).copy()
    return out


def results_equal(a, b) -> bool:
    return a.keys() == b.keys() and all(np.array_equal(a[k], b[k]) for k in a)


def check_parity(spec: Spec, runs: dict):
    """Compares every pair of the timed batch with the oracle (all host threads): scores and best
    cells, and for traceback workloads begin positions, TraceSegment_ lists and CIGAR words.  Runs
    outside every timed region."""
    from oracle import oracle as O
    t0 = time.perf_counter()
    ref = O.oracle_batch(oracle_problem(spec), spec.H, spec.V, traceback=spec.traceback,
                         threads=os.cpu_count() or 1, flat=True)
    want = {"score": ref.score, "end_h": ref.end_h, "end_v": ref.end_v}
    if spec.traceback:
        want.update(begin_h=ref.begin_h, begin_v=ref.begin_v, segments=ref.seg_flat, segment_offsets=ref.seg_offsets)
        if spec.cigar:
            want["cigar"], want["cigar_offsets"] = O.cigar_words_flat(ref.seg_flat, ref.seg_offsets)
    out = {"pairs_checked": len(spec.H), "checked": sorted(want), "oracle_s": round(time.perf_counter() - t0, 2)}
    ok = True
    for name, got in runs.items():
        diff = [k for k in want if not np.array_equal(np.asarray(got[k]), np.asarray(want[k]).astype(got[k].dtype))]
        bad = int(np.count_nonzero((got["score"] != want["score"]) | (got["end_h"] != want["end_h"]) |
                                   (got["end_v"] != want["end_v"])))
        out[name] = {"equal": not diff, "fields_differing": diff, "pairs_with_score_or_end_differing": bad}
        ok = ok and not diff
    out["equal"] = ok
    return out


def cpu_baseline(spec: Spec, seconds_target: float = 10.0):
    """Times the oracle (CPU restatement, all host threads) on a sample of the workload."""
    from oracle import oracle as O
    pb = oracle_problem(spec)
    threads = os.cpu_count() or 1
    H, V = spec.H, spec.V
    n = min(len(H), 2000)
    t0 = time.perf_counter()
    O.oracle_batch(pb, H[:n], V[:n], traceback=spec.traceback, threads=threads)
    dt = time.perf_counter() - t0
    # Grow the sample to about seconds_target of wall time, bounded by the workload.
    n = int(min(len(H), max(n, n * seconds_target / max(dt, 1e-3) / 3)))
    best = None
    for _ in range(2):
        t0 = time.perf_counter()
        O.oracle_batch(pb, H[:n], V[:n], traceback=spec.traceback, threads=threads)
        dt = time.perf_counter() - t0
        best = dt if best is None else min(best, dt)
    sub = Spec(H[:n], V[:n], spec.score, spec.mode, spec.kind, spec.config, spec.band)
    cells = algorithmic_cells(sub)
    return {"value": cells / best / 1e9, "unit": "GCUPS", "cores": threads, "kind": "port",
            "sample": f"first {n} pairs of the workload, oracle/seqan_oracle.c with OpenMP over {threads} "
                      f"threads{' with traceback' if spec.traceback else ''}, best of 2",
            "cells": cells, "seconds": best}


def _reference_call(spec: Spec, H, V, threads: int, lib):
    """One call of the reference's own batch interface, compiled from its headers on this host:
    globalAlignmentScore(ExecutionPolicy<Parallel, Vectorial>, ...) for score-only workloads,
    globalAlignment / localAlignment over StringSet<Gaps> (+ getCigarString) for the others."""
    from oracle import oracle as O
    pb = oracle_problem(spec)
    if spec.traceback:
        return O.ref_batch_gaps(pb, H, V, threads=threads, cigar=spec.cigar, lib=lib, decode=False)[0]
    return O.ref_batch_score(pb, H, V, threads=threads, lib=lib)


def run_reference(args, rank):
    """The reference arm: SeqAn's own batch call on all host cores when its headers are available
    (compiled here by oracle/ref/Makefile's bench target), else the CPU restatement."""
    if rank != 0:
        return
    import platform
    spec = make_workload(args.workload)
    from oracle import oracle as O
    threads = os.cpu_count() or 1
    lib = None
    why = None
    try:
        if spec.dynamic:
            why = "no public batch function of the reference selects DynamicGaps cells"
        elif O.build_ref_bench():
            lib = O.libref_bench()
        else:
            why = "no copy of the reference's headers (baseline/_ref/include) on this host"
    except (subprocess.CalledProcessError, OSError) as e:
        why = f"compiling the reference failed: {e}"
    pb = oracle_problem(spec)
    N = len(spec.H)

    def call(n):
        if lib is not None:
            return _reference_call(spec, spec.H[:n], spec.V[:n], threads, lib)
        return O.oracle_batch(pb, spec.H[:n], spec.V[:n], traceback=spec.traceback, threads=threads).score

    # Size a step to about 4 s of host work: the whole workload when it fits.
    n0 = min(N, 4000)
    t0 = time.perf_counter()
    call(n0)
    dt = time.perf_counter() - t0
    cells0 = algorithmic_cells(Spec(spec.H[:n0], spec.V[:n0], spec.score, spec.mode, spec.kind, spec.config,
                                    spec.band))
    rate = cells0 / max(dt, 1e-6)
    n = N
    if algorithmic_cells(spec) / rate > 4.0:
        n = int(min(N, max(n0, N * 4.0 * rate / algorithmic_cells(spec))))
    H, V = spec.H[:n], spec.V[:n]
    cells = algorithmic_cells(Spec(H, V, spec.score, spec.mode, spec.kind, spec.config, spec.band))
    for _ in range(args.warmup):
        call(n)
    times = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        got = call(n)
        times.append(time.perf_counter() - t0)
    total = sum(times)
    gcups = cells * len(times) / total / 1e9
    # The reference's scores on a sample against the oracle (outside the timed steps).
    m = min(n, 2000)
    agrees = bool(np.array_equal(np.asarray(got[:m], np.int32), O.oracle_batch(pb, H[:m], V[:m], threads=threads).score))
    if lib is not None:
        simd = int(lib.ref_simd_bytes())
        kind = "reference"
        sample = (f"SeqAn compiled from its own headers on this host ({platform.machine()}, g++ -O3, "
                  f"{'SIMD vectors of ' + str(simd) + ' bytes' if simd else 'no SIMD: the Vectorial policy runs its scalar DP'}"
                  f"), ExecutionPolicy<Parallel, Vectorial> with {threads} threads, "
                  f"{'globalAlignment/localAlignment over StringSet<Gaps>' + (' + getCigarString' if spec.cigar else '') if spec.traceback else 'globalAlignmentScore'}"
                  f"; {n} of {N} pairs per step")
    else:
        kind = "port"
        sample = (f"the reference could not run here ({why}); its CPU restatement oracle/seqan_oracle.c with OpenMP "
                  f"over {threads} threads; {n} of {N} pairs per step")
    line = {"metric": "GCUPS, batched affine DNA align", "value": gcups, "unit": "GCUPS", "n_gpus": 1,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * total / len(times),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "int16" if spec.score.bits == 16 else "int32", "data": "synthetic", "impl": "reference",
            "config": {"workload": args.workload, "pairs_per_step": n, "same_config": n == N,
                       "description": WORKLOADS[args.workload]},
            "cpu_baseline": {"value": gcups, "unit": "GCUPS", "cores": threads, "kind": kind, "sample": sample,
                             "scores_agree_with_oracle_on_first_pairs": {"pairs": m, "equal": agrees}},
            "e2e": {"value": gcups, "unit": "GCUPS", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def make_seed_workload(name: str, seed_offset: int = 0):
    from seqan_gb300 import workloads as W
    if name == "xdrop_reads_1m":
        wins, reads, seeds, _ = W.seed_windows(1_000_000, seed=6 + seed_offset)
        return wins, reads, seeds
    raise SystemExit(f"unknown seed workload {name}")


def seed_problem():
    from oracle import oracle as O
    return O.SeedProblem(O.GAPPED_XDROP, O.EXTEND_BOTH, 1, -2, -2, 20)


def seed_cpu_time(wins, reads, seeds, n, threads):
    from oracle import oracle as O
    arr = O.seeds_array(seeds[:n])
    t0 = time.perf_counter()
    O.oracle_extend_seeds(seed_problem(), wins[:n], reads[:n], arr, threads=threads)
    return time.perf_counter() - t0


def seed_cpu_baseline(wins, reads, seeds, seconds_target: float = 10.0):
    """The oracle's seed extension (OpenMP over all host threads) on a sample of the seeds."""
    threads = os.cpu_count() or 1
    n = min(len(seeds), 20_000)
    dt = seed_cpu_time(wins, reads, seeds, n, threads)
    n = int(min(len(seeds), max(n, n * seconds_target / max(dt, 1e-3) / 3)))
    best = min(seed_cpu_time(wins, reads, seeds, n, threads) for _ in range(2))
    return {"value": n / best / 1e6, "unit": "Mseeds/s", "cores": threads, "kind": "port",
            "sample": f"first {n} seeds of the workload, orc_extend_seeds (oracle/seqan_oracle.c) with OpenMP "
                      f"over {threads} threads, best of 2", "seeds": n, "seconds": best}


def run_seed_reference(args):
    wins, reads, seeds = make_seed_workload(args.workload)
    threads = os.cpu_count() or 1
    n = min(len(seeds), args.ref_pairs * 10)
    for _ in range(args.warmup):
        seed_cpu_time(wins, reads, seeds, n, threads)
    times = [seed_cpu_time(wins, reads, seeds, n, threads) for _ in range(args.steps)]
    rate = n * len(times) / sum(times) / 1e6
    line = {"metric": "Mseeds/s, batched gapped x-drop seed extension", "value": rate, "unit": "Mseeds/s",
            "n_gpus": 1, "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * sum(times) / len(times),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "int32",
            "data": "synthetic", "impl": "reference",
            "config": {"workload": args.workload, "seeds_per_step": n, "description": WORKLOADS[args.workload]},
            "cpu_baseline": {"value": rate, "unit": "Mseeds/s", "cores": threads, "kind": "port",
                             "sample": f"first {n} seeds of the workload per step; the reference's extendSeed "
                                       "restated in oracle/seqan_oracle.c (pinned to the compiled reference), "
                                       "OpenMP over the host threads"},
            "e2e": {"value": rate, "unit": "Mseeds/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def run_seed_bench(args, rank, world, local_rank, dist):
    """Seed extension: value with seeds and sequences resident in HBM (gba_extend_seeds_device),
    e2e through gba_extend_seeds with pinned host buffers."""
    from seqan_gb300 import _native as N
    N.build()
    L = N.lib()
    ctx = N.Context(local_rank)
    h = ctx.handle
    from oracle import oracle as O
    wins, reads, seeds = make_seed_workload(args.workload, seed_offset=rank)
    if args.pairs:
        wins, reads, seeds = wins[:args.pairs], reads[:args.pairs], seeds[:args.pairs]
    arr = O.seeds_array(seeds)
    ns = len(arr)
    sh, oh = concat(wins)
    sv, ov = concat(reads)
    max_v = int((ov[1:] - ov[:-1]).max())
    sp = seed_problem()
    params = N.GbaExtendParams(sp.method, sp.direction, sp.xdrop, sp.match, sp.mismatch, sp.gap, None, 0, 0)

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

    host = {}
    for name, a in (("sh", sh), ("oh", oh), ("sv", sv), ("ov", ov), ("seeds", arr)):
        host[name] = pinned(a.nbytes)
        as_np(host[name], a.size, a.dtype)[:] = a.reshape(-1)
    host["io"] = pinned(arr.nbytes)
    host["scores"] = pinned(ns * 8)
    dev = {name: device(a.nbytes) for name, a in (("sh", sh), ("oh", oh), ("sv", sv), ("ov", ov), ("seeds0", arr),
                                                    ("seeds", arr))}
    dev["scores"] = device(ns * 8)
    for name in ("sh", "oh", "sv", "ov"):
        ctx.check(L.gba_copy_to_device(h, dev[name], host[name], {"sh": sh, "oh": oh, "sv": sv, "ov": ov}[name].nbytes),
                  "copy")
    ctx.check(L.gba_copy_to_device(h, dev["seeds0"], host["seeds"], arr.nbytes), "copy")
    dbatch = N.GbaSeedBatch(len(wins), dev["sh"], dev["oh"], len(reads), dev["sv"], dev["ov"], ns, None, None, max_v)
    hbatch = N.GbaSeedBatch(len(wins), host["sh"], host["oh"], len(reads), host["sv"], host["ov"], ns, None, None, 0)
    flush_bytes = 256 << 20
    d_flush, p_flush = device(flush_bytes), pinned(flush_bytes)

    def reset_and_flush():
        ctx.check(L.gba_copy_to_device(h, d_flush, p_flush, flush_bytes), "flush")
        ctx.check(L.gba_copy_to_device(h, dev["seeds"], host["seeds"], arr.nbytes), "seeds")
        ctx.check(L.gba_synchronize(h), "sync")

    def run_device():
        ctx.check(L.gba_extend_seeds_device(h, C.byref(params), C.byref(dbatch), dev["seeds"], dev["scores"]), "ext")

    for _ in range(args.warmup):
        reset_and_flush()
        run_device()
        ctx.check(L.gba_synchronize(h), "sync")
    sampler = ClockSampler(local_rank)
    if dist:
        dist.barrier()
    sampler.start()
    step_ms = []
    ms = C.c_float()
    for _ in range(args.steps):
        reset_and_flush()
        ctx.check(L.gba_timer_start(h), "timer")
        run_device()
        ctx.check(L.gba_timer_stop(h, C.byref(ms)), "timer")
        step_ms.append(ms.value)
    ctx.check(L.gba_synchronize(h), "sync")
    if dist:
        dist.barrier()
    clocks = sampler.stop()
    total_ms = sum(step_ms)
    if dist:
        import torch
        t = torch.tensor([total_ms], dtype=torch.float64, device=f"cuda:{local_rank}")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        total_ms = float(t.item())
    value = ns * world * args.steps / (total_ms * 1e-3) / 1e6
    # Parity spot check of the device run against the oracle (first 20,000 seeds).
    out = np.zeros_like(arr)
    ctx.check(L.gba_copy_to_host(h, out.ctypes.data, dev["seeds"], arr.nbytes), "d2h")
    k = min(ns, 20_000)
    ref, _ = O.oracle_extend_seeds(sp, wins[:k], reads[:k], arr[:k])
    parity = bool(np.array_equal(out[:k], ref))

    # e2e: the host-buffer C-ABI call, seeds copied in and back every step.
    def run_host():
        io = as_np(host["io"], arr.size, np.int64)
        io[:] = arr.reshape(-1)
        t0 = time.perf_counter()
        ctx.check(L.gba_extend_seeds(h, C.byref(params), C.byref(hbatch), host["io"], host["scores"]), "e2e")
        return time.perf_counter() - t0

    for _ in range(max(1, args.warmup)):
        run_host()
    e2e_s = []
    for _ in range(args.steps):
        reset_and_flush()
        e2e_s.append(run_host())
    st = ctx.stats()
    e2e = ns * world * len(e2e_s) / sum(e2e_s) / 1e6
    peak = C.c_double()
    ctx.check(L.gba_measure_int_peak(h, C.byref(peak)), "int peak")
    kernel_ms = st.dp_kernel_ms
    ops = st.cells * XDROP_OPS_PER_CELL
    achieved = ops / (kernel_ms * 1e-3) / 1e12
    line = {"metric": "Mseeds/s, batched gapped x-drop seed extension", "value": value, "unit": "Mseeds/s",
            "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": total_ms / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "int32", "data": "synthetic",
            "config": {"workload": args.workload if not args.pairs else f"{args.workload} (first {ns} seeds)",
                       "description": WORKLOADS[args.workload], "seeds": ns, "cells_per_step": int(st.cells),
                       "l2": "flushed (256 MiB write) between timed steps; seeds restored before each step",
                       "parallelism": f"replicas x{world} (seeds are independent)",
                       "shared_memory_ring": int(st.seed_ring), "fallback_seeds": int(st.seed_fallbacks)},
            "e2e": {"value": e2e, "unit": "Mseeds/s", "h2d_bytes_per_step": int(sh.nbytes + sv.nbytes + oh.nbytes +
                                                                               ov.nbytes + arr.nbytes),
                    "d2h_bytes_per_step": int(arr.nbytes + ns * 8), "ms_per_step": 1e3 * sum(e2e_s) / len(e2e_s),
                    "last_call": {"kernel_ms": kernel_ms, "call_ms": st.call_ms}},
            "gpu_launches": args.steps * int(st.kernel_launches),
            "roofline": {"bound": "int32", "achieved": achieved, "peak": peak.value, "unit": "Tops/s",
                         "frac": achieved / peak.value if peak.value else None, "traffic": None,
                         "kernel": f"k_extend_gapped<{int(st.seed_ring)}> (persistent, one seed per thread, "
                                   "anti-diagonal and residue rings in shared memory) + fallback levels + "
                                   "k_apply_gapped",
                         "ops_per_cell": XDROP_OPS_PER_CELL, "gcups": st.cells / (kernel_ms * 1e-3) / 1e9,
                         "kernel_ms": kernel_ms,
                         "peak_source": "measured live by gba_measure_int_peak (32-bit add+max issue rate)"},
            "clocks": clocks, "parity_first_20000_vs_oracle": parity}
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        line["cpu_baseline"] = seed_cpu_baseline(wins, reads, seeds)
    for p in list(dev.values()) + [d_flush]:
        L.gba_device_free(h, p)
    for p in list(host.values()) + [p_flush]:
        L.gba_host_free(h, p)
    if rank == 0:
        print(json.dumps(line), flush=True)


def extend_sides(wins, reads, seeds):
    """The side tasks of extendAlignment: reversed prefixes (left) and suffixes (right)."""
    H, V = [], []
    for w, r, s in zip(wins, reads, seeds):
        bh, bv, L = (int(x) for x in s)
        if bh > 0 and bv > 0:
            H.append(np.ascontiguousarray(w[:bh][::-1]))
            V.append(np.ascontiguousarray(r[:bv][::-1]))
        if bh + L < len(w) and bv + L < len(r):
            H.append(np.ascontiguousarray(w[bh + L:]))
            V.append(np.ascontiguousarray(r[bv + L:]))
    return H, V


def extend_cpu_time(H, V, threads):
    from oracle import oracle as O
    pb = O.Problem("extend", 0, None, 2, -4, -6, -1, None, 32, "dna", 20)
    t0 = time.perf_counter()
    O.oracle_batch(pb, H, V, traceback=True, threads=threads)
    return time.perf_counter() - t0


def run_extend_bench(args, rank, world, local_rank, dist):
    import seqan_gb300 as sg
    from seqan_gb300 import _native as N
    N.build()
    L = N.lib()
    ctx = N.Context(local_rank)
    h = ctx.handle
    from seqan_gb300 import workloads as W
    n_al = args.pairs or 250_000
    wins, reads, seeds, _ = W.seed_windows(n_al, seed=16 + rank)
    sh, oh = concat(wins)
    sv, ov = concat(reads)
    pos = np.zeros((n_al, 6), dtype=np.int64)
    pos[:, 0], pos[:, 1] = seeds[:, 0], seeds[:, 1]
    pos[:, 2], pos[:, 3] = seeds[:, 0] + seeds[:, 2], seeds[:, 1] + seeds[:, 2]

    def pinned(a):
        p = C.c_void_p()
        ctx.check(L.gba_host_alloc(h, C.byref(p), max(a.nbytes, 1)), "gba_host_alloc")
        C.memmove(p, a.ctypes.data, a.nbytes)
        return p

    p_sh, p_oh, p_sv, p_ov, p_pos = pinned(sh), pinned(oh), pinned(sv), pinned(ov), pinned(pos)
    score = sg.Score(2, -4, -1, -6)
    params = N.GbaExtendAlignParams(3, 1, 20, score.match, score.mismatch, score.gap_open, score.gap_extend,
                                    None, 0, 0)
    batch = N.GbaSeedBatch(n_al, p_sh, p_oh, n_al, p_sv, p_ov, n_al, None, None, 0)
    cap = int(len(sh) + len(sv) + 8 * n_al)
    segs = np.zeros((cap, 4), dtype=np.uint32)
    offs = np.zeros(2 * n_al + 1, dtype=np.int64)
    ls = np.zeros(n_al, dtype=np.int32)
    rs = np.zeros(n_al, dtype=np.int32)
    res = N.GbaExtendAlignResult(ls.ctypes.data, rs.ctypes.data, segs.ctypes.data, cap, offs.ctypes.data)

    def call():
        ctx.check(L.gba_extend_alignments(h, C.byref(params), C.byref(batch), p_pos, C.byref(res)), "extend")

    for _ in range(args.warmup):
        call()
    sampler = ClockSampler(local_rank)
    if dist:
        dist.barrier()
    sampler.start()
    wall, kern, dpk = [], [], []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        call()
        wall.append(time.perf_counter() - t0)
        st = ctx.stats()
        kern.append(st.dp_kernel_ms + st.traceback_kernel_ms)
        dpk.append(st.dp_kernel_ms)
    if dist:
        dist.barrier()
    clocks = sampler.stop()
    st = ctx.stats()
    kernel_ms = sum(kern) / len(kern)
    value = n_al * world / (kernel_ms * 1e-3) / 1e6
    e2e = n_al * world * len(wall) / sum(wall) / 1e6
    # parity spot check: the first 2,000 alignments against the oracle
    from seqan_gb300 import align_extend as X
    from oracle import oracle as O
    pb = O.Problem("extend", 0, None, 2, -4, -6, -1, None, 32, "dna", 20)
    parity = True
    for k in range(min(n_al, 2000)):
        ext = X.SideExtension(int(ls[k]), int(rs[k]),
                              [tuple(int(x) for x in segs[q]) for q in range(offs[2 * k], offs[2 * k + 1])],
                              [tuple(int(x) for x in segs[q]) for q in range(offs[2 * k + 1], offs[2 * k + 2])])
        ref = O.oracle_extend_alignment(pb, wins[k], reads[k], pos[k, :4], 3)
        if (ext.left_score, ext.right_score, ext.left_segments, ext.right_segments) != \
                (ref.left_score, ref.right_score, ref.left_segments, ref.right_segments):
            parity = False
            break
    peak = C.c_double()
    ctx.check(L.gba_measure_int_peak(h, C.byref(peak)), "int peak")
    dp_ms = sum(dpk) / len(dpk)
    ops = 2 * st.cells * OPS_PER_CELL["affine_global"]     # score pass + trace pass over the same cells
    achieved = ops / (dp_ms * 1e-3) / 1e12
    line = {"metric": "M alignments/s, batched extendAlignment (X-drop)", "value": value, "unit": "M alignments/s",
            "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": kernel_ms,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "int32", "data": "synthetic",
            "config": {"workload": args.workload, "description": WORKLOADS[args.workload], "alignments": n_al,
                       "cells_per_step": int(st.cells), "rows_per_band": int(st.tile_rows),
                       "value_timing": "CUDA events around the score pass, trace pass and traceback inside "
                                       "gba_extend_alignments (inputs in HBM)",
                       "parallelism": f"replicas x{world}"},
            "e2e": {"value": e2e, "unit": "M alignments/s",
                    "h2d_bytes_per_step": int(sh.nbytes + sv.nbytes + oh.nbytes + ov.nbytes + pos.nbytes),
                    "d2h_bytes_per_step": int(offs[-1]) * 16 + int(offs.nbytes) + 2 * n_al * 4,
                    "ms_per_step": 1e3 * sum(wall) / len(wall), "last_call_ms": st.call_ms},
            "gpu_launches": args.steps * int(st.kernel_launches),
            "roofline": {"bound": "int32", "achieved": achieved, "peak": peak.value, "unit": "Tops/s",
                         "frac": achieved / peak.value if peak.value else None, "traffic": None,
                         "kernel": "k_extend_dp<affine> (score and trace passes) + k_extend_traceback",
                         "ops_per_cell": OPS_PER_CELL["affine_global"], "dp_kernel_ms": dp_ms,
                         "gcups_per_pass": st.cells / (dp_ms / 2 * 1e-3) / 1e9,
                         "peak_source": "measured live by gba_measure_int_peak (32-bit add+max issue rate)"},
            "clocks": clocks, "parity_first_2000_vs_oracle": parity}
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        threads = os.cpu_count() or 1
        n = min(n_al, 50_000)
        Hs, Vs = extend_sides(wins[:n], reads[:n], seeds[:n])
        best = min(extend_cpu_time(Hs, Vs, threads) for _ in range(2))
        line["cpu_baseline"] = {"value": n / best / 1e6, "unit": "M alignments/s", "cores": threads, "kind": "port",
                                "sample": f"both sides of the first {n} alignments: the oracle's extension DP with "
                                          f"X-drop and traceback (oracle/seqan_oracle.c), OpenMP over {threads} "
                                          "threads, best of 2", "seconds": best}
    for p in (p_sh, p_oh, p_sv, p_ov, p_pos):
        L.gba_host_free(h, p)
    if rank == 0:
        print(json.dumps(line), flush=True)


def run_extend_reference(args):
    from seqan_gb300 import workloads as W
    n_al = min(args.pairs or 250_000, 50_000)
    wins, reads, seeds, _ = W.seed_windows(n_al, seed=16)
    Hs, Vs = extend_sides(wins, reads, seeds)
    threads = os.cpu_count() or 1
    for _ in range(args.warmup):
        extend_cpu_time(Hs, Vs, threads)
    times = [extend_cpu_time(Hs, Vs, threads) for _ in range(args.steps)]
    rate = n_al * len(times) / sum(times) / 1e6
    print(json.dumps({"metric": "M alignments/s, batched extendAlignment (X-drop)", "value": rate,
                      "unit": "M alignments/s", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
                      "ms_per_step": 1e3 * sum(times) / len(times), "higher_is_better": True, "scaling": "weak",
                      "vs_baseline": None, "dtype": "int32", "data": "synthetic", "impl": "reference",
                      "config": {"workload": args.workload, "alignments_per_step": n_al,
                                 "description": WORKLOADS[args.workload]},
                      "cpu_baseline": {"value": rate, "unit": "M alignments/s", "cores": threads, "kind": "port",
                                       "sample": f"both sides of {n_al} alignments per step, the oracle's extension "
                                                 "DP with X-drop and traceback, OpenMP"},
                      "e2e": {"value": rate, "unit": "M alignments/s", "h2d_bytes_per_step": 0,
                              "d2h_bytes_per_step": 0}}), flush=True)


def we_pairs(n: int, seed: int):
    """The Waterman-Eggert workload's pairs: 100-200 bp, every other one a mutated copy."""
    from seqan_gb300 import workloads as W
    rng = np.random.Generator(np.random.PCG64(seed))
    H, V = [], []
    for k in range(n):
        h = rng.integers(0, 4, int(rng.integers(100, 201))).astype(np.uint8)
        v = W.mutate(rng, h, 0.1, 0.02) if k % 2 else rng.integers(0, 4, int(rng.integers(100, 201))).astype(np.uint8)
        H.append(h)
        V.append(v)
    return H, V


WE_SCORE, WE_CUTOFF, WE_COUNT = (2, -1, -2), 10, 10


def we_cpu_time(H, V, kind, lib=None, band=None):
    """Seconds for the enumeration of every pair: the oracle ("port") or the compiled reference
    ("reference", through lib), one pair after another, as the reference's enumerator runs."""
    from oracle import oracle as O
    t0 = time.perf_counter()
    for h, v in zip(H, V):
        if kind == "reference":
            O.ref_local_enumerate(h, v, *WE_SCORE, WE_CUTOFF, max_count=WE_COUNT, lib=lib, band=band)
        else:
            O.oracle_local_enumerate(h, v, *WE_SCORE, WE_CUTOFF, max_count=WE_COUNT, band=band)
    return time.perf_counter() - t0


def we_band_cells(m, n, band):
    """Cells of the banded enumerator's band storage that lie in the matrix (1 <= column <= m)."""
    lo, up = band
    return sum(max(0, min(m, r + up) - max(1, r + lo) + 1) for r in range(1, n + 1))


def we_metric(band):
    if band:
        return "pairs/s, banded Waterman-Eggert enumeration (LocalAlignmentEnumerator<Score, Banded>)"
    return "pairs/s, Waterman-Eggert enumeration (LocalAlignmentEnumerator)"


def run_we_bench(args, rank, world, local_rank, dist):
    import seqan_gb300 as sg
    from seqan_gb300 import _native as N
    from seqan_gb300 import local_enum as LE
    N.build()
    L = N.lib()
    ctx = N.Context(local_rank)
    n = args.pairs or 10_000
    H, V = we_pairs(n, 70 + rank)
    band = WE_BAND.get(args.workload)
    if band is None:
        cells = int(sum(len(h) * len(v) for h, v in zip(H, V)))
    else:
        cells = int(sum(we_band_cells(len(h), len(v), band) for h, v in zip(H, V)))
    score = sg.Score(WE_SCORE[0], WE_SCORE[1], WE_SCORE[2], WE_SCORE[2])

    def call():
        return LE.local_enumerate(H, V, score, WE_CUTOFF, WE_COUNT, alphabet="dna5", context=ctx, band=band)

    for _ in range(args.warmup):
        out = call()
    sampler = ClockSampler(local_rank)
    if dist:
        dist.barrier()
    sampler.start()
    wall, kern = [], []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        out = call()
        wall.append(time.perf_counter() - t0)
        kern.append(ctx.stats().dp_kernel_ms)
    if dist:
        dist.barrier()
    clocks = sampler.stop()
    st = ctx.stats()
    kernel_ms = sum(kern) / len(kern)
    value = n * world / (kernel_ms * 1e-3)
    e2e = n * world * len(wall) / sum(wall)
    alignments = sum(len(e.alignments) for e in out)
    # parity: the first 300 pairs against the oracle
    from oracle import oracle as O
    parity = True
    for k in range(min(n, 300)):
        ref = O.oracle_local_enumerate(H[k], V[k], *WE_SCORE, WE_CUTOFF, max_count=WE_COUNT, band=band)
        und = bool(ref) and ref[-1] is None
        ref = ref[:-1] if und else ref
        if out[k].undefined_next != und or [(a.score, a.row0, a.row1, a.h_begin, a.h_end, a.v_begin, a.v_end)
                                             for a in out[k].alignments] != \
                [(a.score, a.row0, a.row1, a.h_begin, a.h_end, a.v_begin, a.v_end) for a in ref]:
            parity = False
            break
    peak = C.c_double()
    ctx.check(L.gba_measure_int_peak(ctx.handle, C.byref(peak)), "int peak")
    # the initial fill alone: linear local, 6 ops per cell (two gap adds, diagonal add, two maxima,
    # the zero floor); the heap, the traces and the declumping come on top
    achieved = cells * OPS_PER_CELL["linear_local"] / (kernel_ms * 1e-3) / 1e12
    kname = "k_waterman_eggert_banded" if band else "k_waterman_eggert"
    line = {"metric": we_metric(band), "value": value,
            "unit": "pairs/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": kernel_ms,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "int32", "data": "synthetic",
            "config": {"workload": args.workload, "description": WORKLOADS[args.workload], "pairs": n,
                       "alignments_per_step": alignments, "cells_per_step": cells,
                       "value_timing": "CUDA events around the enumeration kernel inside gba_local_enumerate "
                                       "(inputs in HBM)", "parallelism": f"replicas x{world}"},
            "e2e": {"value": e2e, "unit": "pairs/s", "h2d_bytes_per_step": int(sum(len(h) + len(v) for h, v in zip(H, V))),
                    "d2h_bytes_per_step": int(alignments * 5 * 4 + sum(len(a.segments) for e in out
                                                                       for a in e.alignments) * 16),
                    "ms_per_step": 1e3 * sum(wall) / len(wall), "last_call_ms": st.call_ms},
            "gpu_launches": args.steps * int(st.kernel_launches),
            "roofline": {"bound": "latency", "achieved": achieved, "peak": peak.value, "unit": "Tops/s",
                         "frac": achieved / peak.value if peak.value else None, "traffic": None,
                         "kernel": kname + " (one thread per pair: heap, traces and declumping are sequential "
                                           "per pair) + k_enum_pack",
                         "ops_per_cell": OPS_PER_CELL["linear_local"], "dp_kernel_ms": kernel_ms,
                         "note": "achieved counts the initial matrix fill only" +
                                 (" (the band's cells inside the matrix)" if band else ""),
                         "peak_source": "measured live by gba_measure_int_peak (32-bit add+max issue rate)"},
            "clocks": clocks, "parity_first_300_vs_oracle": parity}
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        k = min(n, 1000)
        t = we_cpu_time(H[:k], V[:k], "port", band=band)
        line["cpu_baseline"] = {"value": k / t, "unit": "pairs/s", "cores": 1, "kind": "port",
                                "sample": f"the first {k} pairs, the oracle's enumeration one pair after another",
                                "seconds": t}
    if rank == 0:
        print(json.dumps(line), flush=True)


def run_we_reference(args):
    from oracle import oracle as O
    n = min(args.pairs or 10_000, 4000)
    H, V = we_pairs(n, 70)
    if O.ref_available():
        lib = O.libref()
    elif O.build_ref_bench():
        lib = O.libref_bench()
    else:
        print(json.dumps({"impl": "reference", "unavailable": "the reference's headers are not on this host "
                                                              "(baseline/_ref/include)"}), flush=True)
        return
    band = WE_BAND.get(args.workload)
    lib.ref_local_enumerate_batch.argtypes = [C.c_int32] * 4 + [C.c_int64, C.c_void_p, C.c_void_p, C.c_void_p,
                                                                C.c_void_p, C.c_int32, C.c_void_p, C.c_int32]
    lib.ref_local_enumerate_banded_batch.argtypes = [C.c_int32] * 6 + [C.c_int64, C.c_void_p, C.c_void_p, C.c_void_p,
                                                                       C.c_void_p, C.c_int32, C.c_void_p, C.c_int32]
    sh, oh = O.concat(H)
    sv, ov = O.concat(V)
    count = np.zeros(n, np.int32)
    threads = os.cpu_count() or 1

    def step(k):
        if band:
            lib.ref_local_enumerate_banded_batch(WE_SCORE[0], WE_SCORE[1], WE_SCORE[2], band[0], band[1], WE_CUTOFF,
                                                 k, sh.ctypes.data, oh.ctypes.data, sv.ctypes.data, ov.ctypes.data,
                                                 WE_COUNT, count.ctypes.data, threads)
        else:
            lib.ref_local_enumerate_batch(WE_SCORE[0], WE_SCORE[1], WE_SCORE[2], WE_CUTOFF, k, sh.ctypes.data,
                                          oh.ctypes.data, sv.ctypes.data, ov.ctypes.data, WE_COUNT, count.ctypes.data,
                                          threads)

    for _ in range(args.warmup):
        step(min(n, 200))
    times = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        step(n)
        times.append(time.perf_counter() - t0)
    rate = n * len(times) / sum(times)
    print(json.dumps({"metric": we_metric(band), "value": rate,
                      "unit": "pairs/s", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
                      "ms_per_step": 1e3 * sum(times) / len(times), "higher_is_better": True, "scaling": "weak",
                      "vs_baseline": None, "dtype": "int32", "data": "synthetic", "impl": "reference",
                      "config": {"workload": args.workload, "pairs_per_step": n, "description": WORKLOADS[args.workload]},
                      "cpu_baseline": {"value": rate, "unit": "pairs/s", "cores": threads, "kind": "reference",
                                       "sample": f"the first {n} pairs of the workload per step through the compiled "
                                                 f"reference's LocalAlignmentEnumerator{'<.., Banded>' if band else ''}, "
                                                 f"{threads} OpenMP threads over the pairs"},
                      "e2e": {"value": rate, "unit": "pairs/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}),
          flush=True)


def chain_data(n: int, seed: int):
    from seqan_gb300 import workloads as W
    return W.chain_pairs(n, 1000, 3000, seed=seed)


def run_chain_bench(args, rank, world, local_rank, dist):
    import seqan_gb300 as sg
    from seqan_gb300 import _native as N
    from seqan_gb300.banded_chain import banded_chain_codes
    N.build()
    L = N.lib()
    ctx = N.Context(local_rank)
    n = args.pairs or 20_000
    H, V, chains = chain_data(n, 90 + rank)
    sc = sg.Score(*CHAIN_SCORE)

    def call():
        return banded_chain_codes(H, V, chains, sc, sc, None, CHAIN_K, context=ctx)

    for _ in range(max(args.warmup, 1)):
        out = call()
    sampler = ClockSampler(local_rank)
    if dist:
        dist.barrier()
    sampler.start()
    wall, kern = [], []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        out = call()
        wall.append(time.perf_counter() - t0)
        kern.append(ctx.stats().dp_kernel_ms)
    if dist:
        dist.barrier()
    clocks = sampler.stop()
    st = ctx.stats()
    kernel_ms = sum(kern) / len(kern)
    value = n * world / (kernel_ms * 1e-3)
    e2e = n * world * len(wall) / sum(wall)
    score, status, ntr, segs = out
    cells = int(st.cells)
    parity = None
    if not args.no_parity:
        from oracle import oracle as O
        parity = True
        for k in range(min(n, 300)):
            o = O.oracle_banded_chain(H[k], V[k], chains[k], CHAIN_SCORE, CHAIN_SCORE, 0, CHAIN_K)
            if (int(status[k]), int(score[k]), int(ntr[k]), segs[k]) != (o.status, o.score, o.n_traces, o.segments):
                parity = False
                break
    peak = C.c_double()
    ctx.check(L.gba_measure_int_peak(ctx.handle, C.byref(peak)), "int peak")
    achieved = cells * OPS_PER_CELL["affine_global"] / (kernel_ms * 1e-3) / 1e12
    line = {"metric": "pairs/s, banded chain alignment (bandedChainAlignment)", "value": value, "unit": "pairs/s",
            "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": kernel_ms,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "int32", "data": "synthetic",
            "config": {"workload": args.workload, "description": WORKLOADS[args.workload], "pairs": n,
                       "seeds": int(sum(len(c) for c in chains)), "cells_per_step": cells,
                       "gcups": cells / (kernel_ms * 1e-3) / 1e9, "trace_bytes_per_step": int(st.trace_bytes),
                       "l2": "not flushed: each step's scratch (trace matrices, score columns, traces; several GB) "
                             "is far larger than L2",
                       "value_timing": "CUDA events around k_banded_chain inside gba_banded_chain (inputs in HBM)",
                       "parallelism": f"replicas x{world}"},
            "e2e": {"value": e2e, "unit": "pairs/s",
                    "h2d_bytes_per_step": int(sum(len(h) + len(v) for h, v in zip(H, V)) +
                                              16 * sum(len(c) for c in chains)),
                    "d2h_bytes_per_step": int(12 * n + 16 * sum(len(x) for x in segs)),
                    "ms_per_step": 1e3 * sum(wall) / len(wall), "last_call_ms": st.call_ms},
            "gpu_launches": args.steps * int(st.kernel_launches),
            "roofline": {"bound": "latency", "achieved": achieved, "peak": peak.value, "unit": "Tops/s",
                         "frac": achieved / peak.value if peak.value else None, "traffic": None,
                         "kernel": "k_banded_chain (one thread per chain: its grids, tracebacks and glue in order) "
                                   "+ k_chain_pack",
                         "ops_per_cell": OPS_PER_CELL["affine_global"], "dp_kernel_ms": kernel_ms,
                         "peak_source": "measured live by gba_measure_int_peak (32-bit add+max issue rate)"},
            "clocks": clocks, "parity_first_300_vs_oracle": parity,
            "statuses": {str(k): int(v) for k, v in zip(*np.unique(status, return_counts=True))}}
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        from oracle import oracle as O
        k = min(n, 2000)
        t0 = time.perf_counter()
        for q in range(k):
            O.oracle_banded_chain(H[q], V[q], chains[q], CHAIN_SCORE, CHAIN_SCORE, 0, CHAIN_K)
        t = time.perf_counter() - t0
        line["cpu_baseline"] = {"value": k / t, "unit": "pairs/s", "cores": 1, "kind": "port",
                                "sample": f"the first {k} pairs, the oracle's banded chain alignment one pair after "
                                          "another", "seconds": t}
    if rank == 0:
        print(json.dumps(line), flush=True)


def run_chain_reference(args):
    from oracle import oracle as O
    n = min(args.pairs or 20_000, 4000)
    H, V, chains = chain_data(n, 90)
    if O.ref_available():
        lib = O.libref()
    elif O.build_ref_bench():
        lib = O.libref_bench()
    else:
        print(json.dumps({"impl": "reference", "unavailable": "the reference's headers are not on this host "
                                                              "(baseline/_ref/include)"}), flush=True)
        return
    lib.ref_banded_chain_batch.argtypes = [C.c_void_p, C.c_void_p, C.c_int32, C.c_int32, C.c_int64, C.c_void_p,
                                           C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                           C.c_void_p, C.c_int32]
    sh, oh = O.concat(H)
    sv, ov = O.concat(V)
    so = np.zeros(n + 1, np.int64)
    np.cumsum([len(c) for c in chains], out=so[1:])
    seeds = np.ascontiguousarray(np.concatenate(chains + [np.zeros((1, 4), np.int32)]), dtype=np.int32)
    a = np.array(CHAIN_SCORE, np.int32)
    score = np.zeros(n, np.int32)
    status = np.zeros(n, np.int32)
    threads = os.cpu_count() or 1

    def step(k):
        lib.ref_banded_chain_batch(a.ctypes.data, a.ctypes.data, 0, CHAIN_K, k, sh.ctypes.data, oh.ctypes.data,
                                   sv.ctypes.data, ov.ctypes.data, seeds.ctypes.data, so.ctypes.data,
                                   score.ctypes.data, status.ctypes.data, threads)

    for _ in range(args.warmup):
        step(min(n, 200))
    times = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        step(n)
        times.append(time.perf_counter() - t0)
    rate = n * len(times) / sum(times)
    print(json.dumps({"metric": "pairs/s, banded chain alignment (bandedChainAlignment)", "value": rate,
                      "unit": "pairs/s", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
                      "ms_per_step": 1e3 * sum(times) / len(times), "higher_is_better": True, "scaling": "weak",
                      "vs_baseline": None, "dtype": "int32", "data": "synthetic", "impl": "reference",
                      "config": {"workload": args.workload, "pairs_per_step": n, "description": WORKLOADS[args.workload]},
                      "cpu_baseline": {"value": rate, "unit": "pairs/s", "cores": threads, "kind": "reference",
                                       "sample": f"the first {n} pairs of the workload per step through the compiled "
                                                 f"reference's bandedChainAlignment, {threads} OpenMP threads"},
                      "e2e": {"value": rate, "unit": "pairs/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}),
          flush=True)


def serving_requests(n: int, seed: int):
    """Mixed-length affine DNA requests: 90% U[100,500], 9% U[1000,5000], 1% 10,000 bp; the
    partner has 5% substitutions and 1% indels."""
    from seqan_gb300 import workloads as W
    rng = np.random.Generator(np.random.PCG64(seed))
    lens = W.serving_lengths(n, seed=seed)
    H, V = [], []
    for L in lens:
        h = rng.integers(0, 4, size=int(L), dtype=np.uint8)
        H.append(h)
        V.append(W.mutate(rng, h, 0.05, 0.01))
    return H, V


def run_serving(rate: float, duration: float, seed: int = 7, streams: int = 8):
    """Open-loop Poisson arrivals at `rate` for `duration` seconds through the server; returns
    throughput and latency percentiles of the completed requests."""
    import seqan_gb300 as sg
    from seqan_gb300.serving import Server
    rng = np.random.Generator(np.random.PCG64(seed + 1))
    n = max(1, int(rate * duration))
    gaps = rng.exponential(1.0 / rate, size=n)
    arrivals = np.cumsum(gaps) - gaps[0]
    H, V = serving_requests(n, seed)
    cells = int(sum(len(h) * len(v) for h, v in zip(H, V)))
    srv = Server(sg.Score(2, -4, -1, -6, dtype=np.int16), traceback=True, streams=streams,
                 max_batch_pairs=4096, hbm_budget_bytes=64 << 30)
    done = {}
    try:
        # The arrival process runs in native code on its own thread (the call releases the
        # GIL); this thread collects results meanwhile.
        rc = []
        t0 = srv.clock()
        feeder = threading.Thread(target=lambda: rc.append(srv.submit_schedule(H, V, arrivals)))
        feeder.start()
        while len(done) < n:
            for r in srv.poll(segments=False):
                done[r.tag] = r
            if not feeder.is_alive() and rc and rc[0] != 0:
                raise RuntimeError(f"submit_schedule failed with status {rc[0]}")
            time.sleep(0.0005)
        feeder.join()
        t_end = max(r.t_done for r in done.values())
        st = srv.stats()
    finally:
        srv.close()
    lat = np.array([done[i].t_done - done[i].t_submit for i in range(n)]) * 1e3
    span = t_end - t0
    bad = sum(1 for r in done.values() if r.status not in (0, 2))
    return {"offered_req_s": rate, "requests": n, "arrival_window_s": duration,
            "throughput_req_s": n / span, "gcups": cells / span / 1e9, "p50_ms": float(np.percentile(lat, 50)),
            "p99_ms": float(np.percentile(lat, 99)), "max_ms": float(lat.max()), "batches": int(st.batches),
            "streams": streams, "hbm_in_flight_peak_bytes": int(st.hbm_in_flight_peak), "failed": bad}


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
    ap.add_argument("--pairs", type=int, default=0, help="use only the first N pairs (small profiling cases)")
    ap.add_argument("--no-serving", action="store_true", help="skip the serving-loop measurement")
    ap.add_argument("--no-parity", action="store_true", help="skip the oracle comparison of the timed results")
    ap.add_argument("--tile-variant", type=int, default=0,
                    help="packed kernel tiling variant 1..5 instead of the autotuned one (profiling captures)")
    ap.add_argument("--kernel", default="auto", choices=["auto", "general", "packed16", "plain", "warp32"],
                    help="auto: the engine's routing (packed 16-bit kernels), graph-replayed; "
                         "plain: the same kernels, one launch per length bucket; "
                         "warp32: the 32-bit warp kernel instead of the packed 16-bit warp kernel")
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
        if args.workload in BAM_WORKLOADS:
            if rank == 0:
                run_bam_reference(args)
        elif args.workload in FASTA_WORKLOADS:
            if rank == 0:
                run_fasta_reference(args)
        elif args.workload in SAM_WORKLOADS:
            if rank == 0:
                run_sam_reference(args)
        elif args.workload in EXTEND_WORKLOADS:
            if rank == 0:
                run_extend_reference(args)
        elif args.workload in WE_WORKLOADS:
            if rank == 0:
                run_we_reference(args)
        elif args.workload in CHAIN_WORKLOADS:
            if rank == 0:
                run_chain_reference(args)
        elif args.workload in SEED_WORKLOADS:
            if rank == 0:
                run_seed_reference(args)
        else:
            run_reference(args, rank)
        if dist:
            dist.barrier()
        return
    if args.workload in SEED_WORKLOADS:
        run_seed_bench(args, rank, world, local_rank, dist)
        if dist:
            dist.destroy_process_group()
        return
    if args.workload in EXTEND_WORKLOADS:
        run_extend_bench(args, rank, world, local_rank, dist)
        if dist:
            dist.destroy_process_group()
        return
    if args.workload in WE_WORKLOADS:
        run_we_bench(args, rank, world, local_rank, dist)
        if dist:
            dist.destroy_process_group()
        return
    if args.workload in CHAIN_WORKLOADS:
        run_chain_bench(args, rank, world, local_rank, dist)
        if dist:
            dist.destroy_process_group()
        return
    if args.workload in BAM_WORKLOADS:
        run_bam_bench(args, rank, world, local_rank, dist)
        if dist:
            dist.destroy_process_group()
        return
    if args.workload in FASTA_WORKLOADS:
        run_fasta_bench(args, rank, world, local_rank, dist)
        if dist:
            dist.destroy_process_group()
        return
    if args.workload in SAM_WORKLOADS:
        run_sam_bench(args, rank, world, local_rank, dist)
        if dist:
            dist.destroy_process_group()
        return

    import seqan_gb300 as sg
    from seqan_gb300 import _native as N
    N.build()
    L = N.lib()
    ctx = N.Context(local_rank)
    h = ctx.handle

    spec = make_workload(args.workload, seed_offset=rank)
    if args.pairs:
        spec.H, spec.V = spec.H[:args.pairs], spec.V[:args.pairs]
    H, V, score, mode, kind = spec.H, spec.V, spec.score, spec.mode, spec.kind
    sh, oh = concat(H)
    sv, ov = concat(V)
    npairs = len(H)
    cells = algorithmic_cells(spec)
    outputs = N.GBA_OUT_SCORE | N.GBA_OUT_END
    if spec.traceback:
        outputs |= N.GBA_OUT_SEGMENTS
    if spec.cigar:
        outputs |= N.GBA_OUT_CIGAR

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
             "plain": N.GBA_FLAG_PLAIN_BUCKETS | N.GBA_FLAG_NO_GRAPH,
             "warp32": N.GBA_FLAG_AUTOTUNE | N.GBA_FLAG_NO_WARP16}[args.kernel]
    params = sg.align.make_params(score, mode, spec.config, spec.band, outputs, gaps=spec.gaps,
                                  alphabet_size=spec.alphabet_size, flags=flags)
    params.tile_variant = args.tile_variant
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
    step_ms, dp_ms, tb_ms, launches = [], [], [], 0
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
        tb_ms.append(st.traceback_kernel_ms)
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
    # The timed runs' results (outside the timed region), for the parity check against the oracle.
    value_out = fetch_results(L, ctx, plan, npairs, d_score, d_eh, d_ev, spec, oh, ov)

    # The plain GPU form on the same device-resident batch (comparison for the persistent form):
    # the same kernels, launched once per 8-residue length bucket of max(|H|, |V|), pairs in input
    # order inside a bucket, no split slots, default tiling, no autotune, no CUDA graph.  A second
    # plain form runs the one-pair-per-thread 32-bit kernel per bucket (the form of a first GPU
    # port).  Each must give the same results as the timed runs.
    plain = plain_strip = None
    if args.kernel == "auto" and not args.no_plain and spec.band is None:
        def time_plain(extra_flags):
            pparams = sg.align.make_params(score, mode, spec.config, None, outputs, gaps=spec.gaps,
                                           alphabet_size=spec.alphabet_size,
                                           flags=N.GBA_FLAG_PLAIN_BUCKETS | N.GBA_FLAG_NO_GRAPH | extra_flags)
            pplan = C.c_void_p()
            ctx.check(L.gba_plan_create(h, C.byref(pparams), C.byref(host_batch), C.byref(pplan)), "plain plan")
            ctx.check(L.gba_plan_execute(h, pplan, C.byref(dev_batch), C.byref(dev_res)), "plain")
            ctx.check(L.gba_synchronize(h), "sync")
            pms, pdp = [], []
            for _ in range(3):
                flush_l2()
                ctx.check(L.gba_timer_start(h), "timer")
                ctx.check(L.gba_plan_execute(h, pplan, C.byref(dev_batch), C.byref(dev_res)), "plain")
                ctx.check(L.gba_timer_stop(h, C.byref(ms)), "timer")
                pms.append(ms.value)
                pdp.append(ctx.stats().dp_kernel_ms)
            pst = ctx.stats()
            same = results_equal(fetch_results(L, ctx, pplan, npairs, d_score, d_eh, d_ev, spec, oh, ov), value_out)
            L.gba_plan_destroy(h, pplan)
            pg = cells / (sum(pms) / len(pms) * 1e-3) / 1e9
            return {"value": pg, "unit": "GCUPS", "ms_per_step": sum(pms) / len(pms),
                    "dp_kernel_ms": sum(pdp) / len(pdp), "launches_per_step": pst.kernel_launches,
                    "kernel": kernel_label(pst.dp_kernels), "speedup_of_value": value / pg,
                    "results_equal_timed_runs": same}
        plain = time_plain(0)
        plain["form"] = ("the same kernels as the timed runs, one launch per 8-residue bucket of max(|H|,|V|), input "
                         "order inside a bucket, no split slots, default tiling, no autotune, no CUDA graph")
        if not spec.traceback:
            plain_strip = time_plain(N.GBA_FLAG_GENERAL_KERNEL)
            plain_strip["form"] = "one-pair-per-thread int32 kernel (k_dp_strip), one launch per 8-residue bucket"
        # Restore the timed results in the device buffers (the plain runs wrote the same values).

    # End to end through the public C-ABI call with host buffers.
    host_res = N.GbaResult()
    host_res.score, host_res.end_h, host_res.end_v = p_score, p_eh, p_ev
    seg_cap = int((oh[1:] - oh[:-1]).sum() + (ov[1:] - ov[:-1]).sum() + 4 * npairs) if spec.traceback else 0
    extra_pinned = []
    if spec.traceback:
        p_seg = pinned(seg_cap * 16)
        p_segoff = pinned((npairs + 1) * 8)
        p_bh, p_bv = pinned(npairs * 4), pinned(npairs * 4)
        extra_pinned += [p_seg, p_segoff, p_bh, p_bv]
        host_res.segments, host_res.segment_capacity, host_res.segment_offsets = p_seg, seg_cap, p_segoff
        host_res.begin_h, host_res.begin_v = p_bh, p_bv
    if spec.cigar:
        p_cig = pinned(seg_cap * 4)
        p_cigoff = pinned((npairs + 1) * 8)
        extra_pinned += [p_cig, p_cigoff]
        host_res.cigar, host_res.cigar_capacity, host_res.cigar_offsets = p_cig, seg_cap, p_cigoff
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
    e2e_out = host_results(host_res, npairs, spec, as_np)
    # The same call on String<Dna, Packed<>> host words (2 bits per residue) from pinned memory:
    # gba_align_packed uploads the words and unpacks them on the device.
    e2e_packed = None
    if spec.alphabet_size <= 4 and not spec.traceback:
        from seqan_gb300 import packed as P
        hw, hwo = P.pack_set(H, 2)
        vw, vwo = P.pack_set(V, 2)
        pk = [pinned(a.nbytes) for a in (hw, hwo, vw, vwo)]
        for p_, a_ in zip(pk, (hw, hwo, vw, vwo)):
            C.memmove(p_, a_.ctypes.data, a_.nbytes)
        ph = N.GbaPackedSet(len(hwo) - 1, pk[0], pk[1], 2, 0)
        pv = N.GbaPackedSet(len(vwo) - 1, pk[2], pk[3], 2, 0)
        for _ in range(max(1, args.warmup)):
            ctx.check(L.gba_align_packed(h, C.byref(params), C.byref(ph), C.byref(pv), 0, C.byref(host_res)), "pk")
        pk_s = []
        for _ in range(args.steps):
            flush_l2()
            t0 = time.perf_counter()
            ctx.check(L.gba_align_packed(h, C.byref(params), C.byref(ph), C.byref(pv), 0, C.byref(host_res)), "pk")
            pk_s.append(time.perf_counter() - t0)
        pk_same = results_equal(host_results(host_res, npairs, spec, as_np), e2e_out)
        e2e_packed = {"value": cells * world * len(pk_s) / sum(pk_s) / 1e9, "unit": "GCUPS",
                      "results_equal_codes_path": pk_same,
                      "h2d_bytes_per_step": int(hw.nbytes + vw.nbytes + hwo.nbytes + vwo.nbytes),
                      "d2h_bytes_per_step": 3 * npairs * 4, "ms_per_step": 1e3 * sum(pk_s) / len(pk_s),
                      "input": "String<Dna, Packed<>> host words (gba_align_packed)"}
        extra_pinned += pk
    # The same pairs as two FASTA texts (60-column lines) from pinned memory: gba_align_fasta reads
    # both on the device and aligns from the codes left in HBM.
    e2e_fasta = None
    if spec.alphabet_size <= 5 and not spec.traceback and not getattr(spec, "h_shared", False):
        from seqan_gb300 import workloads as Wl
        th = Wl.records_text(H, "fasta", width=60, seed=7, id_prefix="h")
        tv = Wl.records_text(V, "fasta", width=60, seed=8, id_prefix="v")
        ft = [pinned(len(th)), pinned(len(tv))]
        C.memmove(ft[0], th, len(th))
        C.memmove(ft[1], tv, len(tv))
        npairs_out = C.c_int64()
        fa_call = lambda: ctx.check(L.gba_align_fasta(h, C.byref(params), ft[0], len(th), ft[1], len(tv), 5, 0, npairs,
                                                      C.byref(npairs_out), C.byref(host_res)), "fa")
        for _ in range(max(1, args.warmup)):
            fa_call()
        fa_s = []
        for _ in range(args.steps):
            flush_l2()
            t0 = time.perf_counter()
            fa_call()
            fa_s.append(time.perf_counter() - t0)
        fa_same = npairs_out.value == npairs and results_equal(host_results(host_res, npairs, spec, as_np), e2e_out)
        e2e_fasta = {"value": cells * world * len(fa_s) / sum(fa_s) / 1e9, "unit": "GCUPS",
                     "results_equal_codes_path": fa_same,
                     "h2d_bytes_per_step": len(th) + len(tv), "d2h_bytes_per_step": 3 * npairs * 4,
                     "ms_per_step": 1e3 * sum(fa_s) / len(fa_s),
                     "input": "two FASTA texts, 60-column lines (gba_align_fasta)"}
        extra_pinned += ft
    e2e_breakdown = {"host_plan_ms": est.host_plan_ms, "dp_kernel_ms": est.dp_kernel_ms, "call_ms": est.call_ms}
    e2e_gcups = cells * world * len(e2e_s) / sum(e2e_s) / 1e9
    h2d = sh.nbytes + sv.nbytes + oh.nbytes + ov.nbytes
    d2h = 3 * npairs * 4
    if spec.traceback:
        segoff = as_np(p_segoff, npairs + 1, np.int64)
        d2h += int(segoff[-1]) * 16 + (npairs + 1) * 8 + 2 * npairs * 4
    if spec.cigar:
        cigoff = as_np(p_cigoff, npairs + 1, np.int64)
        d2h += int(cigoff[-1]) * 4 + (npairs + 1) * 8

    # Roofline of the DP kernel: integer add/max ops against the measured integer rate.
    peak = C.c_double()
    ctx.check(L.gba_measure_int_peak(h, C.byref(peak)), "int peak")
    dp_avg_ms = sum(dp_ms) / len(dp_ms)
    tb_avg_ms = sum(tb_ms) / len(tb_ms)
    st_last = ctx.stats()
    ops = cells * OPS_PER_CELL[kind]
    achieved = ops / (dp_avg_ms * 1e-3) / 1e12
    cap = CAPTURED.get(args.workload) if not args.pairs and not args.tile_variant else None
    roofline = {"bound": "int32", "achieved": achieved, "peak": peak.value, "unit": "Tops/s",
                "frac": achieved / peak.value if peak.value else None,
                "traffic": int(cap["dram_bytes_per_cell"] * cells) if cap else None,
                "kernel": kernel_label(st_last.dp_kernels), "ops_per_cell": OPS_PER_CELL[kind],
                "dp_kernel_ms": dp_avg_ms,
                "peak_source": "measured live by gba_measure_int_peak (32-bit add+max issue rate)"}
    if cap:
        # k_int_peak counts an add and a max as two ops; a DPX add-max on int16x2 halves does four
        # algorithmic ops in one ALU instruction, so the captured ALU-pipe share is the direct
        # measure of how busy the bound unit is.
        roofline["traffic_source"] = f"dram__bytes_read.sum + dram__bytes_write.sum per cell of {cap['profile']}"
        roofline["alu_pipe_pct_captured"] = cap["alu_pipe_pct"]

    if spec.traceback:
        roofline["trace_bytes_per_launch"] = int(st_last.trace_bytes)
        roofline["trace_write_gbs"] = st_last.trace_bytes / (dp_avg_ms * 1e-3) / 1e9
        # Traceback configs also count the algorithmic trace (0.5 byte per cell: a 2-bit source
        # of S and one open/extend bit each for E and F) against the measured HBM copy rate;
        # the bound is whichever fraction is larger.
        hbm = measured_hbm_gbs()
        if hbm:
            tr_frac = 0.5 * cells / (dp_avg_ms * 1e-3) / 1e9 / hbm
            roofline["trace_hbm"] = {"algorithmic_bytes_per_cell": 0.5, "achieved_gbs": 0.5 * cells / (dp_avg_ms * 1e-3) / 1e9,
                                     "peak_gbs": hbm, "frac": tr_frac,
                                     "peak_source": "MEASURED_PEAKS.json hbm_gbs (of measured)"}
            roofline["frac_traceback_max"] = max(roofline["frac"] or 0.0, tr_frac)
        roofline["traceback_and_output_ms"] = tb_avg_ms
    line = {"metric": "GCUPS, batched affine DNA align", "value": value, "unit": "GCUPS", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": total_ms / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "int16" if score.bits == 16 else "int32", "data": "synthetic",
            "config": {"workload": args.workload if not args.pairs else f"{args.workload} (first {npairs} pairs)",
                       "description": WORKLOADS[args.workload], "pairs": npairs,
                       "cells_per_step": cells, "l2": "flushed (256 MiB write) between timed steps",
                       "kernel": args.kernel,
                       "parallelism": f"replicas x{world} (pairs are independent)"},
            "e2e": {"value": e2e_gcups, "unit": "GCUPS", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                    "ms_per_step": 1e3 * sum(e2e_s) / len(e2e_s), "last_call": e2e_breakdown},
            "gpu_launches": launches, "roofline": roofline, "clocks": clocks}
    if tile:
        line["config"]["tiling"] = tile
    if e2e_packed:
        line["e2e_packed"] = e2e_packed
    if e2e_fasta:
        line["e2e_fasta"] = e2e_fasta
    if plain:
        line["plain_gpu_form"] = plain
    if plain_strip:
        line["plain_strip_form"] = plain_strip
    if rank == 0 and not args.no_parity:
        line["parity"] = check_parity(spec, {"value_runs": value_out, "e2e_runs": e2e_out})
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(spec)
    if rank == 0 and world == 1 and args.workload == "affine_dna_100k" and not args.no_serving and not args.pairs:
        # Serving: the stated load (50,000 req/s, mixed lengths incl. 1% 10 kbp x 10 kbp, global
        # affine with traceback) for a 2 s arrival window (100,000 requests), then the capacity.
        stated = run_serving(50_000.0, 2.0)
        # Capacity: 20,000 requests offered at once.
        saturated = run_serving(1e9, 20_000 / 1e9, seed=13)
        line["serving"] = {"workload": "Poisson arrivals; lengths 90% U[100,500], 9% U[1000,5000], 1% 10000; "
                                       "5% subs + 1% indels; Score(2,-4,-1,-6) int16 (10 kbp pairs promoted to "
                                       "int32); global; score + traceback; 64 GB HBM admission budget; "
                                       "8 batches in flight",
                           "stated_load": stated, "capacity": saturated}
    L.gba_plan_destroy(h, plan)
    for p in (d_sh, d_sv, d_score, d_eh, d_ev, d_flush):
        L.gba_device_free(h, p)
    for p in [p_sh, p_sv, p_oh, p_ov, p_score, p_eh, p_ev, p_flush] + extra_pinned:
        L.gba_host_free(h, p)
    if rank == 0:
        print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()
    mismatches = [k for k, v in (("parity", line.get("parity")), ("plain_gpu_form", plain), ("plain_strip_form", plain_strip),
                                 ("e2e_packed", e2e_packed), ("e2e_fasta", e2e_fasta))
                  if v and not v.get("equal", v.get("results_equal_timed_runs", v.get("results_equal_codes_path", True)))]
    if mismatches:
        print(f"results differ: {mismatches}", file=sys.stderr, flush=True)
        sys.exit(1)


if __name__ == "__main__":
    main()
