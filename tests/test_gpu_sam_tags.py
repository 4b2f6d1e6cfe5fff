"""SAM / BAM tags on the GPU (gba_format_sam / gba_format_bam with gba_sam_records.tags): byte-
identical to the reference's writers on the fixture records with tags, and to the oracle on
50,000 random records, float values included; malformed tags are refused for SAM."""
import struct

import numpy as np
import pytest

from oracle import oracle as O
from tests.test_sam_tags import tag_records

pytestmark = pytest.mark.gpu


def test_sam_tags_match_reference_fixture(engine):
    from seqan_gb300 import sam as S
    rec, text, _ = tag_records()
    assert S.format_sam(rec) == text


def test_bam_tags_match_reference_fixture(engine):
    from seqan_gb300 import sam as S
    rec, _, data = tag_records()
    assert S.format_bam(rec) == data


def test_float_tags_match_reference_fixture(engine):
    from seqan_gb300 import sam as S
    rec, text, data = tag_records("sam_float_tag_cases.json")
    assert S.format_sam(rec) == text
    assert S.format_bam(rec) == data


def test_every_float_exponent_vs_oracle(engine):
    """One record per float exponent and sign with edge and random mantissas in B:f arrays."""
    from seqan_gb300 import sam as S
    from tests.golden.make_golden import sam_records
    rng = np.random.Generator(np.random.PCG64(31))
    rec = sam_records(rng, 512)
    tags = []
    for k in range(512):
        sign, ex = k >> 8, k & 255
        mants = [0, 1, 0x7fffff, 0x400000] + [int(x) for x in rng.integers(0, 1 << 23, 60)]
        words = [(sign << 31) | (ex << 23) | mt for mt in mants]
        tags.append(b"XFBf" + struct.pack("<I", len(words)) + b"".join(struct.pack("<I", w) for w in words) +
                    b"YFf" + struct.pack("<I", words[-1]))
    rec.tags = tags
    assert S.format_sam(rec) == O.oracle_write_sam_c(rec)


def test_random_records_with_tags_vs_oracle(engine):
    from seqan_gb300 import sam as S
    from tests.golden.make_golden import random_tags, sam_records
    rng = np.random.Generator(np.random.PCG64(4242))
    rec = sam_records(rng, 50_000)
    rec.tags = [random_tags(rng, floats=k % 2 == 1) for k in range(len(rec.qname))]
    assert S.format_sam(rec) == O.oracle_write_sam_c(rec)
    assert S.format_bam(rec) == O.oracle_write_bam_c(rec)


def test_malformed_tags_refused_for_sam(engine):
    from seqan_gb300 import _native as N
    from seqan_gb300 import sam as S
    rec, _, _ = tag_records()
    rec.tags = list(rec.tags)
    rec.tags[5] = b"XZZabc"   # a string without its NUL
    with pytest.raises(N.GbaError) as e:
        S.format_sam(rec)
    assert e.value.status == N.GBA_EINVAL
    # BAM writes the bytes as they are
    rec.tags[5] = b"XFf" + struct.pack("<f", 0.25)
    assert S.format_bam(rec) == O.oracle_write_bam_c(rec)
