"""BAM record output (CPU): the oracle's restatement of the reference's BAM writer against the
bytes the compiled reference wrote for the fixture records (tests/golden/bam_cases.json: the SAM
fixture records plus unmapped records, positions on every bin level, short qualities, every CIGAR
operation, Iupac letters) and against the reference's char-to-Iupac table."""
import base64

import numpy as np
import pytest

from oracle import oracle as O
from tests import golden_cases as G

BAM = G.load("bam_cases.json")


def case_records(c):
    from seqan_gb300 import sam as S
    rec = S.SamRecords(c["qname"], np.array(c["flag"], np.uint16), np.array(c["ref_id"], np.int32),
                       np.array(c["pos"], np.int32), np.array(c["mapq"], np.uint8),
                       [np.array(x, np.uint32) for x in c["cigar"]], np.array(c["next_ref_id"], np.int32),
                       np.array(c["next_pos"], np.int32), np.array(c["tlen"], np.int32),
                       [np.array(s, np.uint8) for s in c["seq"]], c["qual"], c["contigs"])
    rec.letters = c["letters"]
    return rec, base64.b64decode(c["bam"])


@pytest.mark.parametrize("k", range(len(BAM["cases"])))
def test_oracle_writer_matches_reference_fixture(k):
    rec, data = case_records(BAM["cases"][k])
    assert O.oracle_write_bam_c(rec, threads=2) == data


def test_fixture_covers_the_bam_fields():
    rec, data = case_records(BAM["cases"][0])
    assert -1 in rec.pos.tolist() and max(rec.pos) >= 1 << 29
    assert any(0 < len(q) < len(s) for q, s in zip(rec.qual, rec.seq))
    assert any(len(s) % 2 for s in rec.seq) and any(len(s) == 0 for s in rec.seq)
    assert any(sorted(int(x) & 15 for x in c) == list(range(9)) for c in rec.cigar)
    assert "U" in BAM["cases"][1]["letters"] and "a" in BAM["cases"][1]["letters"]


def test_oracle_iupac_matches_reference_table():
    """Each printable character as a one-residue record: the high nibble of its sequence byte is
    the reference's ordValue(Iupac(c))."""
    from seqan_gb300 import sam as S
    table = BAM["iupac"]
    chars = [chr(c) for c in range(33, 127)]
    for i in range(0, len(chars), 32):
        letters = "".join(chars[i:i + 32])
        n = len(letters)
        rec = S.SamRecords([f"r{j}" for j in range(n)], np.zeros(n, np.uint16), np.full(n, -1, np.int32),
                           np.full(n, -1, np.int32), np.zeros(n, np.uint8), [np.zeros(0, np.uint32)] * n,
                           np.full(n, -1, np.int32), np.full(n, -1, np.int32), np.zeros(n, np.int32),
                           [np.array([j], np.uint8) for j in range(n)], [""] * n, [])
        rec.letters = letters
        data = O.oracle_write_bam_c(rec)
        p = 0
        for j in range(n):
            size = int.from_bytes(data[p:p + 4], "little")
            lq = data[p + 12]
            seq_byte = data[p + 36 + lq]
            assert seq_byte >> 4 == table[ord(letters[j])], letters[j]
            p += 4 + size


@pytest.mark.skipif(not O.ref_available(), reason="compiled reference not present")
def test_oracle_matches_live_reference_random():
    import sys
    sys.path.insert(0, G.HERE)
    import make_golden as MG
    rng = np.random.Generator(np.random.PCG64(123))
    for rec in MG.bam_records(rng):
        assert O.oracle_write_bam_c(rec) == O.ref_write_bam(rec)
