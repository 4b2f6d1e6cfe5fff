"""BAM records formatted on the GPU through gba_format_bam: byte-identical to the reference's BAM
writer on the fixture records and to the oracle on a large random batch; the fields the core
cannot hold are refused."""
import numpy as np
import pytest

from oracle import oracle as O
from tests.test_bam import BAM, case_records

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("k", range(len(BAM["cases"])))
def test_fixture_records(engine, k):
    from seqan_gb300 import sam as S
    rec, data = case_records(BAM["cases"][k])
    assert S.format_bam(rec) == data


def test_large_random_batch(engine):
    import sys
    from seqan_gb300 import sam as S
    from tests import golden_cases as G
    sys.path.insert(0, G.HERE)
    import make_golden as MG
    rng = np.random.Generator(np.random.PCG64(9))
    rec = MG.sam_records(rng, 50_000)
    rec.qual = [q if k % 4 else q[:len(q) // 3] for k, q in enumerate(rec.qual)]
    assert S.format_bam(rec) == O.oracle_write_bam_c(rec)


def test_sam_and_bam_of_read_alignments(engine):
    """Reads aligned to windows with device CIGARs, written as BAM: the oracle's bytes."""
    import seqan_gb300 as sg
    from seqan_gb300 import align as A
    from seqan_gb300 import sam as S
    from seqan_gb300 import workloads as W
    wins, reads = W.read_windows(2000, ref_len=500_000, seed=4)
    out = A.align_codes(list(wins), list(reads), sg.Score(2, -4, -1, -6), config=sg.AlignConfig(True, False, False, True),
                        traceback=True, cigar=True, alphabet_size=5)
    rec = S.records_from_read_alignments([f"read{k}" for k in range(len(reads))], list(reads),
                                         np.arange(len(reads)) * 300, out)
    assert S.format_bam(rec) == O.oracle_write_bam_c(rec)


def test_refusals(engine):
    from seqan_gb300 import _native as N
    from seqan_gb300 import sam as S
    rec, _ = case_records(BAM["cases"][0])
    long_name = S.SamRecords(["x" * 255], rec.flag[:1], rec.ref_id[:1], rec.pos[:1], rec.mapq[:1], rec.cigar[:1],
                             rec.next_ref_id[:1], rec.next_pos[:1], rec.tlen[:1], [np.zeros(3, np.uint8)], ["III"],
                             rec.contigs)
    with pytest.raises(N.GbaError) as e:
        S.format_bam(long_name)
    assert e.value.status == N.GBA_EINVAL
    long_qual = S.SamRecords(["r"], rec.flag[:1], rec.ref_id[:1], rec.pos[:1], rec.mapq[:1], rec.cigar[:1],
                             rec.next_ref_id[:1], rec.next_pos[:1], rec.tlen[:1], [np.zeros(2, np.uint8)], ["III"],
                             rec.contigs)
    with pytest.raises(N.GbaError):
        S.format_bam(long_qual)
