"""SeqFileIn format and compression guessing (CPU): the reference's FormattedFile<Fastq, Input>
picks the compression by the stream's magic bytes (stream/stream_base.h:99-148), the record format
by the file name without the compression extension (stream/formatted_file.h:700-730,
seq_io/fasta_fastq.h:104-132) and, for a stream, by its first character (MagicHeader, :79-93).
FASTQ files (plain, gzip, BGZF, bzip2) read through the host reader equal the plain text's
records; FASTA files through the device reader are in the GPU test."""
import bz2
import gzip
import struct
import zlib

import numpy as np
import pytest

from seqan_gb300 import seq_io as S

FASTQ = b"@r1 first\nACGTNACGT\n+\nIIIIIIIII\n@r2\nGGGTTTAAAC\n+r2\n#########!\n@r3\n\n+\n\n"


def bgzf(data: bytes, block: int = 7) -> bytes:
    """BGZF members: raw deflate blocks in gzip members with the "BC" extra field (SAM/BAM
    specification, section 4.1), then the empty end-of-file member."""
    out = b""
    for i in range(0, len(data) + 1, block):
        chunk = data[i:i + block]
        if not chunk and i < len(data):
            continue
        co = zlib.compressobj(6, zlib.DEFLATED, -15)
        body = co.compress(chunk) + co.flush()
        bsize = len(body) + 25
        out += (b"\x1f\x8b\x08\x04" + b"\0" * 4 + b"\0\xff" + struct.pack("<H", 6) + b"BC" + struct.pack("<HH", 2, bsize)
                + body + struct.pack("<II", zlib.crc32(chunk), len(chunk)))
        if not chunk:
            break
    return out


@pytest.mark.parametrize("name,comp,fmt", [
    ("reads.fa", None, "fasta"), ("reads.fasta", None, "fasta"), ("x.faa", None, "fasta"), ("x.ffn", None, "fasta"),
    ("x.fna", None, "fasta"), ("x.frn", None, "fasta"), ("x.fas", None, "fasta"), ("READS.FQ", None, "fastq"),
    ("reads.fastq", None, "fastq"), ("reads.fq.gz", "gzip", "fastq"), ("reads.fa.gz", "gzip", "fasta"),
    ("reads.fa.bgzf", "bgzf", "fasta"), ("reads.fq.bz2", "bzip2", "fastq"), ("reads.txt", None, None),
    ("reads.fq.gz", None, None), ("reads.sam", None, None), ("reads.raw", None, "raw"), ("r.raw.gz", "gzip", "raw")])
def test_format_from_file_name(name, comp, fmt):
    assert S.guess_format_from_filename(name, comp) == fmt


def test_compression_from_magic_bytes():
    assert S.guess_compression(gzip.compress(FASTQ)) == "gzip"
    assert S.guess_compression(bgzf(FASTQ)) == "bgzf"
    assert S.guess_compression(bz2.compress(FASTQ)) == "bzip2"
    assert S.guess_compression(FASTQ) is None
    assert S.guess_format(FASTQ) == "fastq" and S.guess_format(b">x\nAC\n") == "fasta"
    # Raw has no magic header: any other text is Raw (EMBL and GenBank come first and are refused)
    assert S.guess_format(b"ACGT") == "raw" and S.guess_format(b"") == "raw" and S.guess_format(b"IDLE") == "raw"
    for t in (b"ID   X; SV 1\n", b"LOCUS       X\n"):
        with pytest.raises(S.UnknownFileFormat):
            S.guess_format(t)


def _recs(f):
    ids, seqs, quals = [], [], []
    f.readRecords(ids, seqs, quals)
    return ids, [s.tolist() for s in seqs], quals


@pytest.mark.parametrize("comp", [None, "gzip", "bgzf", "bzip2"])
def test_fastq_files_read_as_the_plain_text(tmp_path, comp):
    data = {None: FASTQ, "gzip": gzip.compress(FASTQ), "bgzf": bgzf(FASTQ), "bzip2": bz2.compress(FASTQ)}[comp]
    ext = {None: "", "gzip": ".gz", "bgzf": ".bgzf", "bzip2": ".bz2"}[comp]
    p = tmp_path / f"reads.fastq{ext}"
    p.write_bytes(data)
    f = S.SeqFileIn(str(p))
    assert f.format == "fastq" and f.compression == comp
    want = S.read_fastq(FASTQ)
    ids, seqs, quals = _recs(f)
    assert ids == want.ids and seqs == [s.tolist() for s in want.seqs] and quals == want.quals_list
    assert f.atEnd()
    # a stream is recognised by its content
    g = S.SeqFileIn(data)
    assert g.format == "fastq"
    assert g.readRecord()[0] == b"r1 first"


def test_unknown_extension_and_content(tmp_path):
    p = tmp_path / "reads.txt"
    p.write_bytes(FASTQ)
    with pytest.raises(S.UnknownFileFormat):
        S.SeqFileIn(str(p))
    assert S.SeqFileIn(b"ACGT\n").format == "raw"


def test_records_in_parts(tmp_path):
    rng = np.random.default_rng(3)
    text = b"".join(b"@q%d\n%s\n+\n%s\n" % (k, rng.choice(list(b"ACGTN"), 30).astype(np.uint8).tobytes(), b"I" * 30) for k in range(50))
    p = tmp_path / "many.fq.gz"
    p.write_bytes(gzip.compress(text))
    f = S.SeqFileIn(str(p))
    ids, seqs = [], []
    while not f.atEnd():
        f.readRecords(ids, seqs, max_records=7)
    assert len(ids) == 50 and ids[-1] == b"q49"
