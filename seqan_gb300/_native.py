"""ctypes binding of the engine's C-ABI (include/seqan_gb300.h) and its in-tree build.

The shared library is built in-tree into seqan_gb300/_lib/ by :func:`build` (nvcc for
sm_103a).  Loading fails loudly when it is missing: there is no CPU fallback.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
import threading

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
LIB_DIR = os.path.join(PKG, "_lib")
LIB_PATH = os.path.join(LIB_DIR, "libseqan_gb300.so")
CSRC = os.path.join(PKG, "csrc")
INCLUDE = os.path.join(ROOT, "include")

NVCC_FLAGS = ["-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-lineinfo", "-std=c++17",
              "-Xcompiler", "-fPIC", "-Xcompiler", "-fopenmp"]

# Status codes (include/seqan_gb300.h)
GBA_OK, GBA_EINVAL, GBA_ENOMEM, GBA_EBUDGET, GBA_ECUDA, GBA_ETIMEOUT, GBA_EUNSUPPORTED, GBA_ECAPACITY, GBA_EPARSE = \
    range(9)
GBA_PAIR_OK, GBA_PAIR_INVALID, GBA_PAIR_PROMOTED, GBA_PAIR_FAILED, GBA_PAIR_SKIPPED = 0, 1, 2, 3, 4
GBA_GLOBAL, GBA_LOCAL, GBA_ALIGN_EXTEND = 0, 1, 2
GBA_GAPS_AUTO, GBA_GAPS_LINEAR, GBA_GAPS_AFFINE, GBA_GAPS_DYNAMIC = 0, 1, 2, 3
GBA_FREE_TOP, GBA_FREE_LEFT, GBA_FREE_RIGHT, GBA_FREE_BOTTOM = 1, 2, 4, 8
GBA_OUT_SCORE, GBA_OUT_END, GBA_OUT_SEGMENTS, GBA_OUT_CIGAR = 1, 2, 4, 8
GBA_SEG_DIAGONAL, GBA_SEG_HORIZONTAL, GBA_SEG_VERTICAL = 1, 2, 4
GBA_NOALLOC_SCRATCH_BYTES = 64 << 20
GBA_FLAG_GENERAL_KERNEL, GBA_FLAG_STRIP16, GBA_FLAG_PLAIN_BUCKETS, GBA_FLAG_NO_GRAPH, GBA_FLAG_AUTOTUNE = 1, 2, 4, 8, 16
GBA_FLAG_PACKED = 32
GBA_FLAG_PACKED_SPLIT, GBA_FLAG_PACKED_NO_SPLIT, GBA_FLAG_NO_WARP16, GBA_FLAG_WARP16 = 64, 128, 256, 512
GBA_FLAG_XDROP = 1024
GBA_KERNEL_STRIP, GBA_KERNEL_PACKED, GBA_KERNEL_WARP, GBA_KERNEL_BANDED, GBA_KERNEL_WARP16 = 1, 2, 4, 8, 16
GBA_KERNEL_DYNAMIC = 32
GBA_MATCH_EXTEND, GBA_UNGAPPED_XDROP, GBA_GAPPED_XDROP = 0, 1, 2
GBA_EXTEND_NONE, GBA_EXTEND_LEFT, GBA_EXTEND_RIGHT, GBA_EXTEND_BOTH = 0, 1, 2, 3

# Every symbol include/seqan_gb300.h declares.
EXPORTED = ["gba_create", "gba_destroy", "gba_status_string", "gba_last_error", "gba_align_batch",
            "gba_plan_create", "gba_plan_destroy", "gba_plan_execute", "gba_plan_fetch",
            "gba_device_alloc", "gba_device_free", "gba_host_alloc", "gba_host_free",
            "gba_copy_to_device", "gba_copy_to_host", "gba_synchronize", "gba_timer_start",
            "gba_timer_stop", "gba_get_stats", "gba_measure_int_peak", "gba_align_score_noalloc",
            "gba_server_create", "gba_server_submit", "gba_server_poll", "gba_server_get_stats",
            "gba_server_last_error", "gba_server_destroy", "gba_clock_seconds", "gba_server_submit_schedule",
            "gba_extend_seeds", "gba_extend_seeds_device", "gba_extend_alignments", "gba_align_packed",
            "gba_format_sam", "gba_read_fasta", "gba_read_fastq", "gba_format_bam",
            "gba_align_fasta", "gba_bgzf_compress"]


class GbaConfig(C.Structure):
    _fields_ = [("device", C.c_int32), ("hbm_budget_bytes", C.c_int64)]


class GbaParams(C.Structure):
    _fields_ = [("mode", C.c_int32), ("gap_model", C.c_int32), ("free_ends", C.c_int32),
                ("band_on", C.c_int32), ("band_lower", C.c_int32), ("band_upper", C.c_int32),
                ("match", C.c_int32), ("mismatch", C.c_int32), ("gap_open", C.c_int32),
                ("gap_extend", C.c_int32), ("matrix", C.c_void_p), ("alphabet_size", C.c_int32),
                ("score_bits", C.c_int32), ("outputs", C.c_int32), ("flags", C.c_int32),
                ("tile_variant", C.c_int32), ("xdrop", C.c_int32)]


class GbaBatch(C.Structure):
    _fields_ = [("num_pairs", C.c_int64), ("seq_h", C.c_void_p), ("off_h", C.c_void_p),
                ("seq_v", C.c_void_p), ("off_v", C.c_void_p), ("h_shared", C.c_int32),
                ("reserved", C.c_int32)]


class GbaResult(C.Structure):
    _fields_ = [("score", C.c_void_p), ("end_h", C.c_void_p), ("end_v", C.c_void_p),
                ("begin_h", C.c_void_p), ("begin_v", C.c_void_p), ("pair_status", C.c_void_p),
                ("segments", C.c_void_p), ("segment_capacity", C.c_int64),
                ("segment_offsets", C.c_void_p), ("cigar", C.c_void_p),
                ("cigar_capacity", C.c_int64), ("cigar_offsets", C.c_void_p)]


class GbaNoAllocBatch(C.Structure):
    _fields_ = [("num_pairs", C.c_int64), ("seq_h", C.c_void_p), ("off_h", C.c_void_p),
                ("seq_v", C.c_void_p), ("off_v", C.c_void_p), ("max_h_len", C.c_int32),
                ("reserved", C.c_int32)]


class GbaStats(C.Structure):
    _fields_ = [("dp_kernel_ms", C.c_float), ("traceback_kernel_ms", C.c_float),
                ("kernel_launches", C.c_int32), ("cells", C.c_int64), ("trace_bytes", C.c_int64),
                ("tile_rows", C.c_int32), ("tile_min_blocks", C.c_int32), ("host_plan_ms", C.c_float),
                ("call_ms", C.c_float), ("dp_kernels", C.c_int32), ("seed_ring", C.c_int32),
                ("seed_fallbacks", C.c_int64)]


class GbaServerConfig(C.Structure):
    _fields_ = [("device", C.c_int32), ("streams", C.c_int32), ("max_batch_pairs", C.c_int64),
                ("hbm_budget_bytes", C.c_int64)]


class GbaRequestResult(C.Structure):
    _fields_ = [("tag", C.c_uint64), ("score", C.c_int32), ("end_h", C.c_int32), ("end_v", C.c_int32),
                ("begin_h", C.c_int32), ("begin_v", C.c_int32), ("status", C.c_int32),
                ("n_segments", C.c_int32), ("segment_offset", C.c_int64), ("t_submit", C.c_double),
                ("t_done", C.c_double)]


class GbaServerStats(C.Structure):
    _fields_ = [("submitted", C.c_int64), ("completed", C.c_int64), ("pending", C.c_int64),
                ("batches", C.c_int64), ("cells", C.c_int64), ("hbm_in_flight", C.c_int64),
                ("hbm_in_flight_peak", C.c_int64)]


class GbaSeed(C.Structure):
    _fields_ = [("begin_h", C.c_int64), ("begin_v", C.c_int64), ("end_h", C.c_int64), ("end_v", C.c_int64),
                ("lower_diagonal", C.c_int64), ("upper_diagonal", C.c_int64)]


class GbaExtendParams(C.Structure):
    _fields_ = [("method", C.c_int32), ("direction", C.c_int32), ("score_drop_off", C.c_int32),
                ("match", C.c_int32), ("mismatch", C.c_int32), ("gap", C.c_int32), ("matrix", C.c_void_p),
                ("alphabet_size", C.c_int32), ("reserved", C.c_int32)]


class GbaSeedBatch(C.Structure):
    _fields_ = [("num_h", C.c_int64), ("seq_h", C.c_void_p), ("off_h", C.c_void_p),
                ("num_v", C.c_int64), ("seq_v", C.c_void_p), ("off_v", C.c_void_p),
                ("num_seeds", C.c_int64), ("seed_h", C.c_void_p), ("seed_v", C.c_void_p),
                ("max_v_len", C.c_int64)]


class GbaExtendAlignParams(C.Structure):
    _fields_ = [("direction", C.c_int32), ("xdrop_on", C.c_int32), ("xdrop", C.c_int32), ("match", C.c_int32),
                ("mismatch", C.c_int32), ("gap_open", C.c_int32), ("gap_extend", C.c_int32),
                ("matrix", C.c_void_p), ("alphabet_size", C.c_int32), ("band_on", C.c_int32),
                ("band_lower", C.c_int32), ("band_upper", C.c_int32)]


class GbaEnumParams(C.Structure):
    _fields_ = [("match", C.c_int32), ("mismatch", C.c_int32), ("gap", C.c_int32), ("cutoff", C.c_int32),
                ("matrix", C.c_void_p), ("alphabet_size", C.c_int32), ("max_count", C.c_int32)]


class GbaEnumResult(C.Structure):
    _fields_ = [("count", C.c_void_p), ("status", C.c_void_p), ("score", C.c_void_p), ("begin_h", C.c_void_p),
                ("end_h", C.c_void_p), ("begin_v", C.c_void_p), ("end_v", C.c_void_p), ("segments", C.c_void_p),
                ("segment_capacity", C.c_int64), ("segment_offsets", C.c_void_p)]


GBA_ENUM_DONE, GBA_ENUM_UNDEFINED_NEXT = 0, 1


class GbaSimpleScore(C.Structure):
    _fields_ = [("match", C.c_int32), ("mismatch", C.c_int32), ("gap_extend", C.c_int32), ("gap_open", C.c_int32)]


class GbaChainParams(C.Structure):
    _fields_ = [("anchor", GbaSimpleScore), ("gap", GbaSimpleScore), ("free_ends", C.c_int32),
                ("band_extension", C.c_int32), ("max_traces", C.c_int32)]


class GbaChainSeeds(C.Structure):
    _fields_ = [("seeds", C.c_void_p), ("seed_offsets", C.c_void_p)]


class GbaChainResult(C.Structure):
    _fields_ = [("score", C.c_void_p), ("status", C.c_void_p), ("num_traces", C.c_void_p), ("segments", C.c_void_p),
                ("segment_capacity", C.c_int64), ("segment_offsets", C.c_void_p)]


GBA_CHAIN_OK, GBA_CHAIN_NO_GLUE, GBA_CHAIN_UNDEFINED, GBA_CHAIN_CAPACITY = 0, 1, 2, 3


class GbaExtendAlignResult(C.Structure):
    _fields_ = [("left_score", C.c_void_p), ("right_score", C.c_void_p), ("segments", C.c_void_p),
                ("segment_capacity", C.c_int64), ("segment_offsets", C.c_void_p)]


class GbaPackedSet(C.Structure):
    _fields_ = [("num", C.c_int64), ("words", C.c_void_p), ("word_off", C.c_void_p),
                ("bits_per_value", C.c_int32), ("reserved", C.c_int32)]


class GbaSamRecords(C.Structure):
    _fields_ = [("num", C.c_int64), ("qname", C.c_void_p), ("qname_off", C.c_void_p), ("flag", C.c_void_p),
                ("ref_id", C.c_void_p), ("pos", C.c_void_p), ("mapq", C.c_void_p), ("cigar", C.c_void_p),
                ("cigar_off", C.c_void_p), ("next_ref_id", C.c_void_p), ("next_pos", C.c_void_p),
                ("tlen", C.c_void_p), ("seq", C.c_void_p), ("seq_off", C.c_void_p), ("seq_letters", C.c_void_p),
                ("qual", C.c_void_p), ("qual_off", C.c_void_p), ("contig_names", C.c_void_p),
                ("contig_off", C.c_void_p), ("num_contigs", C.c_int64), ("tags", C.c_void_p),
                ("tags_off", C.c_void_p)]


class GbaSeqRecords(C.Structure):
    _fields_ = [("record_capacity", C.c_int64), ("residue_capacity", C.c_int64), ("id_begin", C.c_void_p),
                ("id_end", C.c_void_p), ("seq_off", C.c_void_p), ("qual_end", C.c_void_p), ("codes", C.c_void_p),
                ("quals", C.c_void_p), ("num", C.c_int64), ("residues", C.c_int64), ("error_offset", C.c_int64)]


def _sources():
    return [os.path.join(CSRC, f) for f in sorted(os.listdir(CSRC)) if f.endswith((".cu", ".cuh", ".h"))] + \
        [os.path.join(INCLUDE, "seqan_gb300.h")]


def build(force: bool = False, verbose: bool = False) -> str:
    """Compiles the engine for sm_103a into seqan_gb300/_lib/ (no-op when up to date): each
    translation unit to an object file in parallel, then one link."""
    srcs = _sources()
    newest = max(os.path.getmtime(s) for s in srcs)
    if not force and os.path.exists(LIB_PATH) and os.path.getmtime(LIB_PATH) >= newest:
        return LIB_PATH
    os.makedirs(LIB_DIR, exist_ok=True)
    tag = f"tmp{os.getpid()}"
    units = [os.path.join(CSRC, f) for f in sorted(os.listdir(CSRC)) if f.endswith(".cu")]
    objs = [os.path.join(LIB_DIR, os.path.basename(u)[:-3] + f".{tag}.o") for u in units]
    procs = []
    try:
        for u, o in zip(units, objs):
            cmd = ["nvcc", *NVCC_FLAGS, "-c", "-o", o, u]
            if verbose:
                print(" ".join(cmd))
            procs.append((cmd, subprocess.Popen(cmd)))
        failed = [cmd for cmd, pr in procs if pr.wait() != 0]
        if failed:
            raise subprocess.CalledProcessError(1, failed[0])
        tmp = LIB_PATH + f".{tag}"
        link = ["nvcc", "-gencode", "arch=compute_103a,code=sm_103a", "-shared", "-o", tmp, *objs, "-lgomp"]
        if verbose:
            print(" ".join(link))
        subprocess.check_call(link)
        os.replace(tmp, LIB_PATH)
    finally:
        for cmd, pr in procs:
            if pr.poll() is None:
                pr.wait()
        for o in objs:
            if os.path.exists(o):
                os.remove(o)
    return LIB_PATH


_lib = None
_lock = threading.Lock()


def lib():
    """Loads the engine library; raises if it has not been built."""
    global _lib
    with _lock:
        if _lib is None:
            if not os.path.exists(LIB_PATH):
                raise RuntimeError(f"seqan_gb300 engine library missing ({LIB_PATH}); run "
                                   "seqan_gb300._native.build() -- there is no CPU fallback")
            L = C.CDLL(LIB_PATH)
            vp, i64, i32 = C.c_void_p, C.c_int64, C.c_int32
            L.gba_create.argtypes = [C.POINTER(vp), C.POINTER(GbaConfig)]
            L.gba_destroy.argtypes = [vp]
            L.gba_status_string.argtypes = [C.c_int]
            L.gba_status_string.restype = C.c_char_p
            L.gba_last_error.argtypes = [vp, C.c_char_p, C.c_size_t]
            L.gba_align_batch.argtypes = [vp, C.POINTER(GbaParams), C.POINTER(GbaBatch), C.POINTER(GbaResult)]
            L.gba_plan_create.argtypes = [vp, C.POINTER(GbaParams), C.POINTER(GbaBatch), C.POINTER(vp)]
            L.gba_plan_destroy.argtypes = [vp, vp]
            L.gba_plan_execute.argtypes = [vp, vp, C.POINTER(GbaBatch), C.POINTER(GbaResult)]
            L.gba_plan_fetch.argtypes = [vp, vp, C.POINTER(GbaResult)]
            L.gba_device_alloc.argtypes = [vp, C.POINTER(vp), C.c_size_t]
            L.gba_device_free.argtypes = [vp, vp]
            L.gba_host_alloc.argtypes = [vp, C.POINTER(vp), C.c_size_t]
            L.gba_host_free.argtypes = [vp, vp]
            L.gba_copy_to_device.argtypes = [vp, vp, vp, C.c_size_t]
            L.gba_copy_to_host.argtypes = [vp, vp, vp, C.c_size_t]
            L.gba_synchronize.argtypes = [vp]
            L.gba_timer_start.argtypes = [vp]
            L.gba_timer_stop.argtypes = [vp, C.POINTER(C.c_float)]
            L.gba_get_stats.argtypes = [vp, C.POINTER(GbaStats)]
            L.gba_measure_int_peak.argtypes = [vp, C.POINTER(C.c_double)]
            L.gba_align_score_noalloc.argtypes = [C.POINTER(GbaParams), C.POINTER(GbaNoAllocBatch), vp, vp,
                                                  vp, vp, vp]
            L.gba_server_create.argtypes = [C.POINTER(vp), C.POINTER(GbaServerConfig), C.POINTER(GbaParams)]
            L.gba_server_submit.argtypes = [vp, C.c_uint64, vp, i64, vp, i64]
            L.gba_server_poll.argtypes = [vp, C.POINTER(GbaRequestResult), i64, vp, i64, C.POINTER(i64),
                                          C.POINTER(i64)]
            L.gba_server_get_stats.argtypes = [vp, C.POINTER(GbaServerStats)]
            L.gba_server_submit_schedule.argtypes = [vp, C.POINTER(GbaBatch), vp, C.c_uint64]
            L.gba_server_last_error.argtypes = [vp, C.c_char_p, C.c_size_t]
            L.gba_server_destroy.argtypes = [vp]
            L.gba_extend_seeds.argtypes = [vp, C.POINTER(GbaExtendParams), C.POINTER(GbaSeedBatch), vp, vp]
            L.gba_extend_seeds_device.argtypes = [vp, C.POINTER(GbaExtendParams), C.POINTER(GbaSeedBatch), vp, vp]
            L.gba_extend_alignments.argtypes = [vp, C.POINTER(GbaExtendAlignParams), C.POINTER(GbaSeedBatch), vp,
                                                C.POINTER(GbaExtendAlignResult)]
            L.gba_local_enumerate.argtypes = [vp, C.POINTER(GbaEnumParams), C.POINTER(GbaBatch),
                                              C.POINTER(GbaEnumResult)]
            L.gba_local_enumerate_banded.argtypes = [vp, C.POINTER(GbaEnumParams), C.c_int32, C.c_int32,
                                                     C.POINTER(GbaBatch), C.POINTER(GbaEnumResult)]
            L.gba_banded_chain.argtypes = [vp, C.POINTER(GbaChainParams), C.POINTER(GbaBatch),
                                           C.POINTER(GbaChainSeeds), C.POINTER(GbaChainResult)]
            L.gba_align_packed.argtypes = [vp, C.POINTER(GbaParams), C.POINTER(GbaPackedSet),
                                           C.POINTER(GbaPackedSet), C.c_int32, C.POINTER(GbaResult)]
            L.gba_format_sam.argtypes = [vp, C.POINTER(GbaSamRecords), vp, i64, vp]
            L.gba_format_bam.argtypes = [vp, C.POINTER(GbaSamRecords), vp, i64, vp]
            L.gba_bgzf_compress.argtypes = [vp, vp, i64, C.c_int32, vp, i64, vp]
            L.gba_align_fasta.argtypes = [vp, C.POINTER(GbaParams), vp, i64, vp, i64, i32, i32, i64,
                                          C.POINTER(i64), C.POINTER(GbaResult)]
            L.gba_read_fasta.argtypes = [vp, vp, i64, i32, C.POINTER(GbaSeqRecords)]
            L.gba_read_fastq.argtypes = [vp, vp, i64, i32, C.POINTER(GbaSeqRecords)]
            L.gba_clock_seconds.argtypes = []
            L.gba_clock_seconds.restype = C.c_double
            _lib = L
    return _lib


class GbaError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__(f"{message} [status {status}]")
        self.status = status


class Context:
    """Owns a gba_context (device, stream, cached device buffers)."""

    def __init__(self, device: int = 0, hbm_budget_bytes: int = 0):
        L = lib()
        self._h = C.c_void_p()
        cfg = GbaConfig(device, hbm_budget_bytes)
        rc = L.gba_create(C.byref(self._h), C.byref(cfg))
        if rc != GBA_OK:
            raise GbaError(rc, f"gba_create failed: {L.gba_status_string(rc).decode()}")

    @property
    def handle(self):
        return self._h

    def check(self, rc: int, what: str):
        if rc != GBA_OK:
            buf = C.create_string_buffer(512)
            lib().gba_last_error(self._h, buf, 512)
            raise GbaError(rc, f"{what}: {lib().gba_status_string(rc).decode()}: {buf.value.decode()}")

    def stats(self) -> GbaStats:
        s = GbaStats()
        self.check(lib().gba_get_stats(self._h, C.byref(s)), "gba_get_stats")
        return s

    def close(self):
        if self._h:
            lib().gba_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


_default_ctx = None


def default_context() -> Context:
    global _default_ctx
    if _default_ctx is None:
        _default_ctx = Context(0)
    return _default_ctx
