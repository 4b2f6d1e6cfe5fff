"""FASTA / FASTQ input into the engine's record layout.

:func:`read_records` returns every record of a text as the reference's loop
``while (!atEnd(iter)) readRecord(id, seq, qual, iter, Fasta | Fastq)`` reads them
(seq_io/fasta_fastq.h:265-283 FASTA, :354-392 FASTQ; seq a String<Dna|Dna5|AminoAcid>, qual a
CharString).  FASTA parses on the device (``gba_read_fasta``), FASTQ on the host
(``gba_read_fastq``).  The records' residue codes and offsets are the arrays
``gba_align_batch`` takes, so :meth:`SeqRecords.seqs` feeds :func:`seqan_gb300.align.align_codes`
without conversion.  Text outside the format raises :class:`SeqParseError` where the reference
raises ParseError / UnexpectedEnd.
"""
from __future__ import annotations

import ctypes as C
import os
from dataclasses import dataclass

import numpy as np

from . import _native as N

ALPHABETS = {"dna": 4, "dna5": 5, "aa": 27}


class SeqParseError(ValueError):
    """The text is not in the format: ``offset`` is where the reader stopped (the offending
    character, or the text's length when a record start / '+' line is missing)."""

    def __init__(self, message: str, offset: int):
        super().__init__(message)
        self.offset = offset


@dataclass
class SeqRecords:
    text: bytes
    id_begin: np.ndarray    # int64 [num]
    id_end: np.ndarray      # int64 [num]
    seq_off: np.ndarray     # int64 [num + 1]
    qual_end: np.ndarray    # int64 [num]
    codes: np.ndarray       # uint8 [residues]
    quals: np.ndarray       # uint8 [residues] (FASTQ)

    def __len__(self):
        return len(self.id_begin)

    def id(self, k: int) -> bytes:
        return self.text[self.id_begin[k]:self.id_end[k]]

    def seq(self, k: int) -> np.ndarray:
        return self.codes[self.seq_off[k]:self.seq_off[k + 1]]

    def qual(self, k: int) -> bytes:
        return bytes(self.quals[self.seq_off[k]:self.qual_end[k]])

    @property
    def ids(self):
        return [self.id(k) for k in range(len(self))]

    @property
    def seqs(self):
        return [self.seq(k) for k in range(len(self))]

    @property
    def quals_list(self):
        return [self.qual(k) for k in range(len(self))]


def read_records(text: bytes, fmt: str = "fasta", alphabet: str = "dna5", ctx: N.Context | None = None) -> SeqRecords:
    """Reads every record of ``text`` (bytes) in format "fasta" or "fastq"."""
    if fmt not in ("fasta", "fastq"):
        raise ValueError("fmt must be 'fasta' or 'fastq'")
    text = bytes(text)
    n = len(text)
    buf = np.frombuffer(text, np.uint8) if n else np.zeros(1, np.uint8)
    start = ord(">") if fmt == "fasta" else ord("@")
    rec_cap = int(np.count_nonzero(buf[:n] == start)) + 1
    res_cap = max(n, 1)
    ib, ie, so, qe = (np.zeros(rec_cap, np.int64) for _ in range(4))
    codes = np.zeros(res_cap, np.uint8)
    quals = np.zeros(res_cap if fmt == "fastq" else 1, np.uint8)
    r = N.GbaSeqRecords(rec_cap, res_cap, ib.ctypes.data, ie.ctypes.data, so.ctypes.data, qe.ctypes.data,
                        codes.ctypes.data, quals.ctypes.data if fmt == "fastq" else None, 0, 0, -1)
    if fmt == "fasta":
        ctx = ctx or N.default_context()
        rc = N.lib().gba_read_fasta(ctx.handle, buf.ctypes.data, n, ALPHABETS[alphabet], C.byref(r))
    else:
        rc = N.lib().gba_read_fastq(ctx.handle if ctx else None, buf.ctypes.data, n, ALPHABETS[alphabet],
                                    C.byref(r))
    if rc == N.GBA_EPARSE:
        raise SeqParseError(f"{fmt} text not in the format at offset {r.error_offset}", r.error_offset)
    if rc != N.GBA_OK:
        if ctx is not None:
            ctx.check(rc, f"gba_read_{fmt}")
        raise N.GbaError(rc, f"gba_read_{fmt}")
    k = r.num
    return SeqRecords(text, ib[:k], ie[:k], so[:k + 1], qe[:k], codes[:r.residues], quals[:r.residues])


def read_raw(text: bytes, alphabet: str = "dna5", ctx: N.Context | None = None) -> SeqRecords:
    """Every line of ``text`` as one record with an empty id, as the reference's readRecord(Raw)
    reads them (seq_io/fasta_fastq.h:235-261: the residues up to the line end with FASTA's ignore
    / assert rule, then skipLine: "\r\n", "\r" and "\n" end a line).  The lines are framed as
    FASTA records (">" + newline before each) and read by the device FASTA reader.  A '>' starts a
    record anywhere in FASTA but is a residue that fails the assert in Raw, so it is handed to the
    reader as '!', which no alphabet holds; error offsets refer to ``text``."""
    import re
    text = bytes(text)
    starts, ends = [], []
    pos = 0
    for mt in re.finditer(rb"\r\n|\r|\n", text):
        starts.append(pos)
        ends.append(mt.start())
        pos = mt.end()
    if pos < len(text):
        starts.append(pos)
        ends.append(len(text))
    parts, conv_starts = [], []
    q = 0
    for a, b in zip(starts, ends):
        line = text[a:b].replace(b">", b"!")
        parts.append(b">\n" + line + b"\n")
        conv_starts.append(q + 2)
        q += len(line) + 3
    fasta = b"".join(parts)
    try:
        rec = read_records(fasta, "fasta", alphabet, ctx)
    except SeqParseError as e:
        i = max(0, int(np.searchsorted(np.asarray(conv_starts, np.int64), e.offset, side="right")) - 1)
        off = starts[i] + (e.offset - conv_starts[i]) if starts else 0
        raise SeqParseError(f"raw text not in the format at offset {off}", off) from None
    return SeqRecords(text, np.zeros(len(rec), np.int64), np.zeros(len(rec), np.int64), rec.seq_off, rec.qual_end,
                      rec.codes, rec.quals)


def read_fasta(text: bytes, alphabet: str = "dna5", ctx: N.Context | None = None) -> SeqRecords:
    return read_records(text, "fasta", alphabet, ctx)


def read_fastq(text: bytes, alphabet: str = "dna5", ctx: N.Context | None = None) -> SeqRecords:
    return read_records(text, "fastq", alphabet, ctx)


def readRecords(ids: list, seqs: list, *args, fmt: str = "fasta", alphabet: str = "dna5"):
    """``readRecords(ids, seqs[, quals], text)``: appends every record's id (bytes), residue codes
    and, when a quals list is given, qualities (bytes), as the reference's readRecords fills its
    StringSets."""
    quals, text = (args[0], args[1]) if len(args) == 2 else (None, args[0])
    rec = read_records(text, fmt, alphabet)
    ids.extend(rec.ids)
    seqs.extend(rec.seqs)
    if quals is not None:
        quals.extend(rec.quals_list)
    return rec


# --- SeqFileIn: format and compression guessing --------------------------------------------------
# The reference's FormattedFile<Fastq, Input> opens a file through a VirtualStream that recognises
# a compressed stream by its magic bytes (stream/stream_base.h:99-148: gzip 1f 8b 08, bzip2 "BZh";
# BGZF is gzip members with an extra field), then picks the record format from the file name with
# the compression extension removed (stream/formatted_file.h:700-730, guessFormatFromFilename) and
# raises UnknownExtensionError when no format claims the extension; a pipe or an open stream is
# recognised by its first bytes instead, the formats tried in SeqInFormats order (guessFormat,
# MagicHeader: '@' FASTQ, '>' FASTA; Raw has no magic header and takes any other text;
# seq_io/fasta_fastq.h:79-143, seq_io/sequence_file.h:86-97, stream/stream_base.h:196-230).  Decompression runs on the host (Python's zlib / bz2 modules, as the
# reference's streams call zlib / libbz2); the records are then read as read_records reads them.

FASTA_EXTENSIONS = (".fa", ".fasta", ".faa", ".ffn", ".fna", ".frn", ".fas")
FASTQ_EXTENSIONS = (".fq", ".fastq")
RAW_EXTENSIONS = (".raw",)
COMPRESSION_EXTENSIONS = {"gzip": (".gz",), "bgzf": (".bgzf", ".bam", ".vcf.gz", ".bed.gz", ".tbi"),
                          "bzip2": (".bz2",)}


class UnknownFileFormat(ValueError):
    """No record format claims the file name's extension, or the text's first character."""


def guess_compression(data: bytes) -> str | None:
    """'bgzf', 'gzip', 'bzip2' or None from the stream's first bytes."""
    if data[:3] == b"\x1f\x8b\x08":
        # BGZF: FEXTRA set with the "BC" subfield first (SAM/BAM specification, section 4.1)
        if len(data) >= 18 and data[3] & 4 and data[12:14] == b"BC":
            return "bgzf"
        return "gzip"
    if data[:3] == b"BZh":
        return "bzip2"
    return None


def guess_format_from_filename(name: str, compression: str | None = None) -> str | None:
    """'fasta' / 'fastq' from a file name whose compression extension (of the detected
    compression) is removed first; None when no format claims the extension."""
    low = name.lower()
    if compression is not None:
        exts = COMPRESSION_EXTENSIONS["gzip"] + COMPRESSION_EXTENSIONS["bgzf"] if compression in ("gzip", "bgzf") \
            else COMPRESSION_EXTENSIONS[compression]
        for ext in sorted(exts, key=len, reverse=True):
            if low.endswith(ext):
                low = low[:-len(ext)]
                break
    if low.endswith(FASTA_EXTENSIONS):
        return "fasta"
    if low.endswith(FASTQ_EXTENSIONS):
        return "fastq"
    if low.endswith(RAW_EXTENSIONS):
        return "raw"
    return None


def guess_format(text: bytes) -> str:
    """'fastq' / 'fasta' from the first character of the (uncompressed) text, else 'raw'.
    EMBL ("ID ") and GenBank ("LOCUS ") texts, which the reference recognises before Raw
    (seq_io/read_embl.h:73, read_genbank.h:82), are refused: their readers are not built."""
    if text[:1] == b"@":
        return "fastq"
    if text[:1] == b">":
        return "fasta"
    if text[:3] == b"ID " or text[:6] == b"LOCUS ":
        raise UnknownFileFormat("EMBL / GenBank input is not supported")
    return "raw"


def decompress(data: bytes, compression: str | None) -> bytes:
    if compression in ("gzip", "bgzf"):
        import gzip
        return gzip.decompress(data)   # every member, as BGZF files hold many
    if compression == "bzip2":
        import bz2
        return bz2.decompress(data)
    return data


class SeqFileIn:
    """SeqFileIn(fileName) / SeqFileIn(stream): a FASTA, FASTQ or Raw file, plain, gzip, BGZF or
    bzip2 compressed, read into the engine's record layout (FASTA and Raw on the device, FASTQ on
    the host)."""

    def __init__(self, source, alphabet: str = "dna5", ctx: N.Context | None = None):
        if isinstance(source, (str, os.PathLike)):
            with open(source, "rb") as f:
                raw = f.read()
            self.compression = guess_compression(raw)
            self.format = guess_format_from_filename(str(source), self.compression)
            if self.format is None:
                raise UnknownFileFormat(f"unknown file extension of {source!r}")
            self.text = decompress(raw, self.compression)
        else:
            raw = source.read() if hasattr(source, "read") else bytes(source)
            self.compression = guess_compression(raw)
            self.text = decompress(raw, self.compression)
            self.format = guess_format(self.text)
        self.alphabet, self.ctx = alphabet, ctx
        self._records = None
        self._next = 0

    def records(self) -> SeqRecords:
        if self._records is None:
            if self.format == "raw":
                self._records = read_raw(self.text, self.alphabet, self.ctx)
            else:
                self._records = read_records(self.text, self.format, self.alphabet, self.ctx)
        return self._records

    def atEnd(self) -> bool:
        return self._next >= len(self.records())

    def readRecord(self):
        """(id, codes, qual) of the next record (qual b"" for FASTA)."""
        rec = self.records()
        if self._next >= len(rec):
            raise EOFError("no record left")
        k = self._next
        self._next += 1
        return rec.id(k), rec.seq(k), rec.qual(k) if self.format == "fastq" else b""

    def readRecords(self, ids: list, seqs: list, quals: list | None = None, max_records: int | None = None):
        """Appends up to max_records (all by default) of the remaining records."""
        rec = self.records()
        end = len(rec) if max_records is None else min(len(rec), self._next + max_records)
        for k in range(self._next, end):
            ids.append(rec.id(k))
            seqs.append(rec.seq(k))
            if quals is not None:
                quals.append(rec.qual(k) if self.format == "fastq" else b"")
        self._next = end
        return end
