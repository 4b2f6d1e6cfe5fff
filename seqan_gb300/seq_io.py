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
