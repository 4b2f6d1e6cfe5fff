"""SAM output oracle (CPU): the restated SAM record writer equals the reference's writer on the
committed fixture (tests/golden/sam_cases.json) and, where the compiled reference exists, on
fresh random records."""
import numpy as np
import pytest

from oracle import oracle as O
from tests import golden_cases as G


def fixture_records():
    from seqan_gb300 import sam as S
    d = G.load("sam_cases.json")
    rec = S.SamRecords(d["qname"], np.array(d["flag"], np.uint16), np.array(d["ref_id"], np.int32),
                       np.array(d["pos"], np.int32), np.array(d["mapq"], np.uint8),
                       [np.array(c, np.uint32) for c in d["cigar"]], np.array(d["next_ref_id"], np.int32),
                       np.array(d["next_pos"], np.int32), np.array(d["tlen"], np.int32),
                       [np.array(s, np.uint8) for s in d["seq"]], d["qual"], d["contigs"])
    return rec, d["text"]


def test_oracle_writer_matches_reference_fixture():
    rec, text = fixture_records()
    assert O.write_sam(rec) == text
    assert O.oracle_write_sam_c(rec, threads=2) == text
    lines = text.splitlines()
    assert len(lines) == len(rec.qname)
    assert any("\t=\t" in ln for ln in lines) and any("\t*\t*\t" in ln for ln in lines)


@pytest.mark.skipif(not O.ref_available(), reason="compiled reference not present")
def test_oracle_writer_matches_live_reference():
    import sys
    import os
    sys.path.insert(0, os.path.join(os.path.dirname(__file__), "golden"))
    from make_golden import sam_records
    rec = sam_records(np.random.Generator(np.random.PCG64(5)), 300)
    assert O.write_sam(rec) == O.ref_write_sam(rec)
