"""BGZF compression on the device (gba_bgzf_compress): every member inflates (Python's zlib) to its
page, the member partition (65,505 input bytes), the 18-byte header with its "BC" size field, the
CRC-32 and input size are the reference's BgzfFile stream's (stream/stream_compressor.h:60-130,
325-375), and the end-of-file member is the reference's 28 bytes.  A BAM file of the fixture
records inflates to the reference's BAM record bytes."""
import base64
import gzip
import struct
import zlib

import numpy as np
import pytest

from tests.test_sam_tags import tag_records

pytestmark = pytest.mark.gpu

EOF_MARKER = bytes([0x1f, 0x8b, 0x08, 0x04, 0, 0, 0, 0, 0, 0xff, 0x06, 0, 0x42, 0x43, 0x02, 0, 0x1b, 0, 0x03, 0,
                    0, 0, 0, 0, 0, 0, 0, 0])
HEADER = bytes([0x1f, 0x8b, 0x08, 4, 0, 0, 0, 0, 0, 0xff, 6, 0, ord("B"), ord("C"), 2, 0])


def _members(z: bytes, data: bytes):
    p, k = 0, 0
    while p < len(z):
        assert z[p:p + 16] == HEADER
        size = struct.unpack_from("<H", z, p + 16)[0] + 1
        crc, isize = struct.unpack_from("<II", z, p + size - 8)
        page = data[k * 65505:(k + 1) * 65505]
        assert isize == len(page) and crc == zlib.crc32(page)
        assert zlib.decompress(z[p + 18:p + size - 8], -15) == page
        p += size
        k += 1
    return k


@pytest.mark.parametrize("kind", ["empty", "one", "page", "page+1", "random", "dna", "repeats", "zeros"])
def test_round_trip_and_framing(engine, kind):
    from seqan_gb300 import sam as S
    rng = np.random.default_rng(5)
    data = {"empty": b"", "one": b"A", "page": bytes(rng.integers(65, 70, 65505, dtype=np.uint8)),
            "page+1": bytes(rng.integers(65, 70, 65506, dtype=np.uint8)),
            "random": bytes(rng.integers(0, 256, 400_000, dtype=np.uint8)),
            "dna": bytes(np.frombuffer(b"ACGT", np.uint8)[rng.integers(0, 4, 1_000_000)]),
            "repeats": b"ACGTTGCAAC" * 50_000, "zeros": bytes(300_000)}[kind]
    z = S.bgzf_compress(data)
    assert z.endswith(EOF_MARKER)
    assert _members(z[:-28], data) == (len(data) + 65504) // 65505
    assert gzip.decompress(z) == data
    assert S.bgzf_compress(data, eof_marker=False) == z[:-28]


def test_bam_file_of_fixture_records(engine):
    from seqan_gb300 import sam as S
    rec, _, data = tag_records()
    many = data * 40
    z = S.bgzf_compress(many)
    assert gzip.decompress(z) == many
    f = S.write_bam_file(rec, header=b"BAM\1" + struct.pack("<i", 0) + struct.pack("<i", 0))
    assert gzip.decompress(f)[12:] == data
    assert len(z) < len(many)
