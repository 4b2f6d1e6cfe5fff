"""SAM / BAM tags (CPU): the oracle's writers against the reference's appendTagsBamToSam SAM lines
and raw-tag BAM records (bam_io/bam_sam_conversion.h:250-360, bam_io/write_bam.h:202-203) on 300
fixture records with tags of every integer, character, string and array type
(tests/golden/sam_tag_cases.json) and 300 with float values of every kind, printed as the
reference's appendNumber(float) prints them: "%g" (tests/golden/sam_float_tag_cases.json)."""
import base64
import struct

import numpy as np
import pytest

from oracle import oracle as O
from tests import golden_cases as G


def tag_records(name="sam_tag_cases.json"):
    from seqan_gb300.sam import SamRecords
    d = G.load(name)
    rec = SamRecords(d["qname"], np.array(d["flag"], np.uint16), np.array(d["ref_id"], np.int32),
                     np.array(d["pos"], np.int32), np.array(d["mapq"], np.uint8),
                     [np.array(c, np.uint32) for c in d["cigar"]], np.array(d["next_ref_id"], np.int32),
                     np.array(d["next_pos"], np.int32), np.array(d["tlen"], np.int32),
                     [np.array(s, np.uint8) for s in d["seq"]], d["qual"], d["contigs"],
                     tags=[base64.b64decode(t) for t in d["tags"]])
    return rec, d["text"], base64.b64decode(d["bam"])


def test_fixtures_cover_every_tag_type():
    rec, text, _ = tag_records()
    types = set()
    for t in rec.tags:
        i = 0
        while i < len(t):
            ty = chr(t[i + 2])
            types.add(ty)
            i += 3
            if ty in "ZH":
                i = t.index(0, i) + 1
            elif ty == "B":
                types.add("B" + chr(t[i]))
                cnt = struct.unpack_from("<I", t, i + 1)[0]
                i += 5 + cnt * {"c": 1, "C": 1, "s": 2, "S": 2, "i": 4, "I": 4}[chr(t[i])]
            else:
                i += {"A": 1, "c": 1, "C": 1, "s": 2, "S": 2, "i": 4, "I": 4}[ty]
    assert set("AcCsSiIZHB") <= types and {"Bc", "BC", "Bs", "BS", "Bi", "BI"} <= types
    assert any(len(t) == 0 for t in rec.tags) and "\t" in text


def test_sam_with_tags_matches_reference_fixture():
    rec, text, _ = tag_records()
    assert O.write_sam(rec) == text
    assert O.oracle_write_sam_c(rec, threads=2) == text


def test_bam_with_tags_matches_reference_fixture():
    rec, _, data = tag_records()
    assert O.oracle_write_bam_c(rec, threads=2) == data


def test_float_tags_match_reference_fixture():
    rec, text, data = tag_records("sam_float_tag_cases.json")
    assert any(b"f" == t[2:3] for t in rec.tags if len(t) > 2)
    for special in ("nan", "-nan", "inf", "-inf", "e-", "e+"):
        assert special in text
    assert O.write_sam(rec) == text
    assert O.oracle_write_sam_c(rec, threads=2) == text
    assert O.oracle_write_bam_c(rec, threads=2) == data


def test_malformed_tags_are_refused_by_the_sam_restatement():
    rec, _, _ = tag_records()
    rec.tags = [t for t in rec.tags]
    rec.tags[3] = b"XZZabc"   # a string without its NUL
    with pytest.raises(ValueError):
        O.oracle_write_sam_c(rec)


@pytest.mark.skipif(not O.ref_available(), reason="compiled reference not present")
def test_live_reference_random_tags():
    from tests.golden.make_golden import random_tags, sam_records
    rng = np.random.Generator(np.random.PCG64(77))
    rec = sam_records(rng, 200)
    rec.tags = [random_tags(rng, floats=True) for _ in rec.qname]
    assert O.oracle_write_sam_c(rec) == O.ref_write_sam(rec)
    assert O.oracle_write_bam_c(rec) == O.ref_write_bam(rec)
