"""SAM output on the GPU (gba_format_sam): byte-identical to the reference's SAM writer on the
fixture records, to the oracle writer on large random batches, and through the read-mapping path
(banded alignment with CIGARs on the device -> SAM)."""
import numpy as np
import pytest

from oracle import oracle as O
from tests.test_sam import fixture_records

pytestmark = pytest.mark.gpu


def test_fixture_records(engine):
    from seqan_gb300 import sam as S
    rec, text = fixture_records()
    assert S.format_sam(rec) == text


def test_large_random_batch(engine):
    import os
    import sys
    from seqan_gb300 import sam as S
    sys.path.insert(0, os.path.join(os.path.dirname(__file__), "golden"))
    from make_golden import sam_records
    rec = sam_records(np.random.Generator(np.random.PCG64(77)), 50_000)
    assert S.format_sam(rec) == O.write_sam(rec)


def test_read_alignments_to_sam(engine):
    import seqan_gb300 as sg
    from seqan_gb300 import align as A
    from seqan_gb300 import sam as S
    from seqan_gb300 import workloads as W
    wins, reads = W.read_windows(20_000, ref_len=2_000_000, seed=19)
    out = A.align_codes(wins, reads, sg.Score(2, -4, -1, -6, dtype=np.int16), config=sg.AlignConfig(True, False, False, True),
                        band=(-6, 26), cigar=True, alphabet_size=4)
    starts = np.arange(len(reads)) * 1000
    names = [f"r{k}" for k in range(len(reads))]
    quals = ["I" * len(r) for r in reads]
    rec = S.records_from_read_alignments(names, reads, starts, out, contigs=("chrSim",), qual=quals)
    text = S.format_sam(rec)
    assert text == O.write_sam(rec)
    first = text.split("\n", 1)[0].split("\t")
    assert first[0] == "r0" and first[2] == "chrSim" and int(first[3]) == 1 + int(out.begin_h[0])


def test_refuses_unknown_contig(engine):
    from seqan_gb300 import _native as N
    from seqan_gb300 import sam as S
    rec, _ = fixture_records()
    rec.ref_id[3] = 17
    with pytest.raises(N.GbaError) as e:
        S.format_sam(rec)
    assert e.value.status == N.GBA_EINVAL
