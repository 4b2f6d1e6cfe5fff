"""SAM output on the device (``gba_format_sam``): BamAlignmentRecord fields -> SAM lines as the
reference's SAM writer writes them (bam_io/write_sam.h:126-217); ``gba_format_bam``: the same
records as uncompressed BAM blocks (bam_io/write_bam.h:100-271).

:class:`SamRecords` holds the fields as arrays (0-based positions, -1 for none, BAM-packed CIGARs
as ``gba_result.cigar`` returns them); :func:`format_sam` returns the text.
:func:`records_from_read_alignments` fills the records of a read-to-window batch (the reference
window's start on its contig plus the alignment's begin in the window).
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

from . import _native as N

CIGAR_OPS = "MIDNSHP=X"


def _off(parts):
    off = np.zeros(len(parts) + 1, dtype=np.int64)
    np.cumsum([len(p) for p in parts], out=off[1:])
    return off


def _cat(parts, dtype):
    return np.concatenate([np.asarray(p, dtype=dtype) for p in parts]) if parts and sum(len(p) for p in parts) \
        else np.zeros(1, dtype=dtype)


@dataclass
class SamRecords:
    qname: list            # str per record
    flag: np.ndarray       # uint16
    ref_id: np.ndarray     # int32, -1 = '*'
    pos: np.ndarray        # int32, 0-based, -1 = none
    mapq: np.ndarray       # uint8
    cigar: list            # per record: uint32 BAM-packed ops
    next_ref_id: np.ndarray
    next_pos: np.ndarray
    tlen: np.ndarray
    seq: list              # per record: residue codes
    qual: list | None      # per record: str, or None for '*'
    contigs: list          # contig names
    letters: str = "ACGTN"
    tags: list | None = None   # per record: BamAlignmentRecord.tags bytes (BAM form), or None


def _tags(rec: SamRecords):
    if rec.tags is None:
        return None, None
    tb = [bytes(t) for t in rec.tags]
    return _cat([np.frombuffer(t, np.uint8) for t in tb], np.uint8), _off(tb)


def _records_struct(rec: SamRecords):
    """The gba_sam_records of rec and the arrays it points into (kept alive by the caller)."""
    n = len(rec.qname)
    qn = [q.encode("latin1") for q in rec.qname]
    qname, qoff = _cat([np.frombuffer(q, np.uint8) for q in qn], np.uint8), _off(qn)
    cig, coff = _cat(rec.cigar, np.uint32), _off(rec.cigar)
    seq, soff = _cat(rec.seq, np.uint8), _off(rec.seq)
    letters = np.zeros(32, dtype=np.uint8)
    letters[:len(rec.letters)] = np.frombuffer(rec.letters.encode(), np.uint8)
    if rec.qual is not None:
        qb = [q.encode("latin1") for q in rec.qual]
        qual, quoff = _cat([np.frombuffer(q, np.uint8) for q in qb], np.uint8), _off(qb)
    else:
        qual = quoff = None
    cb = [c.encode() for c in rec.contigs]
    cnames, cnoff = _cat([np.frombuffer(c, np.uint8) for c in cb], np.uint8), _off(cb)
    arrs = dict(flag=np.ascontiguousarray(rec.flag, np.uint16), ref_id=np.ascontiguousarray(rec.ref_id, np.int32),
                pos=np.ascontiguousarray(rec.pos, np.int32), mapq=np.ascontiguousarray(rec.mapq, np.uint8),
                next_ref_id=np.ascontiguousarray(rec.next_ref_id, np.int32),
                next_pos=np.ascontiguousarray(rec.next_pos, np.int32), tlen=np.ascontiguousarray(rec.tlen, np.int32))
    p = lambda a: None if a is None else a.ctypes.data
    r = N.GbaSamRecords(n, p(qname), p(qoff), p(arrs["flag"]), p(arrs["ref_id"]), p(arrs["pos"]), p(arrs["mapq"]),
                        p(cig), p(coff), p(arrs["next_ref_id"]), p(arrs["next_pos"]), p(arrs["tlen"]), p(seq),
                        p(soff), p(letters), p(qual), p(quoff), p(cnames), p(cnoff), len(rec.contigs))
    tags, toff = _tags(rec)
    r.tags, r.tags_off = p(tags), p(toff)
    keep = [qname, qoff, cig, coff, seq, soff, letters, qual, quoff, cnames, cnoff, arrs, tags, toff]
    return r, keep


def format_bam(rec: SamRecords, ctx=None) -> bytes:
    """The records' uncompressed BAM blocks as the reference's BAM writer writes them
    (bam_io/write_bam.h:100-271, tags appended as they are), formatted on the device (gba_format_bam)."""
    ctx = ctx or N.default_context()
    n = len(rec.qname)
    r, keep = _records_struct(rec)
    rec_off = np.zeros(n + 1, dtype=np.int64)
    rc = N.lib().gba_format_bam(ctx.handle, C.byref(r), None, 0, rec_off.ctypes.data)
    if rc not in (N.GBA_OK, N.GBA_ECAPACITY):
        ctx.check(rc, "gba_format_bam")
    out = np.zeros(int(rec_off[-1]) + 1, dtype=np.uint8)
    ctx.check(N.lib().gba_format_bam(ctx.handle, C.byref(r), out.ctypes.data, len(out), rec_off.ctypes.data),
              "gba_format_bam")
    del keep
    return bytes(out[:int(rec_off[-1])])


def bgzf_compress(data: bytes, eof_marker: bool = True, ctx=None) -> bytes:
    """``data`` as a BGZF file, compressed on the device (gba_bgzf_compress): the reference's member
    partition (65,505 bytes per member), headers, CRC-32s and sizes, this engine's deflate data, and
    the end-of-file member when eof_marker."""
    ctx = ctx or N.default_context()
    buf = np.frombuffer(bytes(data), np.uint8) if len(data) else np.zeros(1, np.uint8)
    cap = len(data) + 64 * (len(data) // 65505 + 2) + 64
    out = np.zeros(cap, np.uint8)
    n = C.c_int64()
    ctx.check(N.lib().gba_bgzf_compress(ctx.handle, buf.ctypes.data, len(data), 1 if eof_marker else 0, out.ctypes.data,
                                        cap, C.byref(n)), "gba_bgzf_compress")
    return bytes(out[:n.value])


def write_bam_file(rec: SamRecords, header: bytes = b"", ctx=None) -> bytes:
    """A BAM file's bytes: the given BAM header bytes (magic, text and reference list, as the
    reference's writer lays them out) and the records' blocks, BGZF-compressed on the device."""
    return bgzf_compress(bytes(header) + format_bam(rec, ctx), True, ctx)


def format_sam(rec: SamRecords, ctx=None) -> str:
    ctx = ctx or N.default_context()
    n = len(rec.qname)
    qn = [q.encode() for q in rec.qname]
    qname, qoff = _cat([np.frombuffer(q, np.uint8) for q in qn], np.uint8), _off(qn)
    cig, coff = _cat(rec.cigar, np.uint32), _off(rec.cigar)
    seq, soff = _cat(rec.seq, np.uint8), _off(rec.seq)
    letters = np.zeros(32, dtype=np.uint8)
    letters[:len(rec.letters)] = np.frombuffer(rec.letters.encode(), np.uint8)
    if rec.qual is not None:
        qb = [q.encode() for q in rec.qual]
        qual, quoff = _cat([np.frombuffer(q, np.uint8) for q in qb], np.uint8), _off(qb)
    else:
        qual = quoff = None
    cb = [c.encode() for c in rec.contigs]
    cnames, cnoff = _cat([np.frombuffer(c, np.uint8) for c in cb], np.uint8), _off(cb)
    arrs = dict(flag=np.ascontiguousarray(rec.flag, np.uint16), ref_id=np.ascontiguousarray(rec.ref_id, np.int32),
                pos=np.ascontiguousarray(rec.pos, np.int32), mapq=np.ascontiguousarray(rec.mapq, np.uint8),
                next_ref_id=np.ascontiguousarray(rec.next_ref_id, np.int32),
                next_pos=np.ascontiguousarray(rec.next_pos, np.int32), tlen=np.ascontiguousarray(rec.tlen, np.int32))
    p = lambda a: None if a is None else a.ctypes.data
    r = N.GbaSamRecords(n, p(qname), p(qoff), p(arrs["flag"]), p(arrs["ref_id"]), p(arrs["pos"]), p(arrs["mapq"]),
                        p(cig), p(coff), p(arrs["next_ref_id"]), p(arrs["next_pos"]), p(arrs["tlen"]), p(seq),
                        p(soff), p(letters), p(qual), p(quoff), p(cnames), p(cnoff), len(rec.contigs))
    tags, toff = _tags(rec)
    r.tags, r.tags_off = p(tags), p(toff)
    line_off = np.zeros(n + 1, dtype=np.int64)
    rc = N.lib().gba_format_sam(ctx.handle, C.byref(r), None, 0, line_off.ctypes.data)
    if rc not in (N.GBA_OK, N.GBA_ECAPACITY):
        ctx.check(rc, "gba_format_sam")
    out = np.zeros(int(line_off[-1]) + 1, dtype=np.uint8)
    ctx.check(N.lib().gba_format_sam(ctx.handle, C.byref(r), out.ctypes.data, len(out), line_off.ctypes.data),
              "gba_format_sam")
    return bytes(out[:int(line_off[-1])]).decode()


def records_from_read_alignments(names, reads, window_starts, out, contig_id=0, contigs=("ref",), mapq=255,
                                 qual=None) -> SamRecords:
    """Records of reads aligned to reference windows by the batch calls with GBA_OUT_CIGAR:
    POS = window start + the alignment's begin in the window, CIGAR from out.cigar."""
    n = len(reads)
    cig = [out.cigar[out.cigar_offsets[k]:out.cigar_offsets[k + 1]] for k in range(n)]
    pos = np.asarray(window_starts, dtype=np.int64) + np.asarray(out.begin_h, dtype=np.int64)
    return SamRecords(list(names), np.zeros(n, np.uint16), np.full(n, contig_id, np.int32), pos.astype(np.int32),
                      np.full(n, mapq, np.uint8), cig, np.full(n, -1, np.int32), np.full(n, -1, np.int32),
                      np.zeros(n, np.int32), list(reads), qual, list(contigs))
