"""FASTA / FASTQ records (CPU): the oracle's restatement of the reference's readRecord loop and the
engine's host FASTQ reader (gba_read_fastq, no GPU), against readRecord outputs of the compiled
reference (tests/golden/seqio_cases.json: the reference's seq_io test files, edge cases, seeded
random texts) and the reference's IsInAlphabet tables."""
import base64

import numpy as np
import pytest

from oracle import oracle as O
from tests import golden_cases as G

SEQIO = G.load("seqio_cases.json")
CASES = SEQIO["cases"]


def expected(c):
    return [(i.encode("latin1"), np.asarray(s, np.uint8), q.encode("latin1")) for i, s, q in c["records"]]


def same(got, want):
    return len(got) == len(want) and all(a[0] == b[0] and np.array_equal(a[1], b[1]) and a[2] == b[2]
                                         for a, b in zip(got, want))


def test_fixtures_cover_the_formats_and_errors():
    assert {(c["format"], c["alphabet"]) for c in CASES} == {(f, a) for f in ("fasta", "fastq")
                                                            for a in ("dna5", "dna", "aa")}
    assert any(c.get("error") == "parse" for c in CASES) and any(c.get("error") == "end" for c in CASES)
    assert any(c["source"].startswith("tests/seq_io/") and "records" in c for c in CASES)


@pytest.mark.parametrize("chunk", range(0, len(CASES), 150))
def test_oracle_matches_reference_fixtures(chunk):
    for c in CASES[chunk:chunk + 150]:
        text = base64.b64decode(c["text"])
        if "error" in c:
            with pytest.raises(O.SeqParseError) as e:
                O.oracle_read_records(text, c["format"], c["alphabet"])
            assert e.value.kind == c["error"], c["source"]
        else:
            assert same(O.oracle_read_records(text, c["format"], c["alphabet"]), expected(c)), c["source"]


@pytest.mark.parametrize("alphabet", ["dna5", "dna", "aa"])
def test_oracle_alphabet_matches_reference_tables(alphabet):
    """Every byte value as a one-residue FASTA sequence: its code where the reference's
    IsInAlphabet accepts it, skipped as whitespace, a new record for '>', else ParseError."""
    table = SEQIO["char_tables"][alphabet]
    for c in range(256):
        text = b">x\n" + bytes([c])
        if c in b" \t\r\n":
            assert len(O.oracle_read_records(text, "fasta", alphabet)[0][1]) == 0
        elif c == ord(">"):
            assert len(O.oracle_read_records(text, "fasta", alphabet)) == 2
        elif table[c] >= 0:
            assert O.oracle_read_records(text, "fasta", alphabet)[0][1].tolist() == [table[c]], c
        else:
            with pytest.raises(O.SeqParseError):
                O.oracle_read_records(text, "fasta", alphabet)


def test_fastq_host_reader_matches_reference_fixtures():
    from seqan_gb300 import _native
    from seqan_gb300 import seq_io as S
    _native.build()
    for c in CASES:
        if c["format"] != "fastq":
            continue
        text = base64.b64decode(c["text"])
        if "error" in c:
            with pytest.raises(S.SeqParseError):
                S.read_fastq(text, c["alphabet"])
        else:
            rec = S.read_fastq(text, c["alphabet"])
            assert same(list(zip(rec.ids, rec.seqs, rec.quals_list)), expected(c)), c["source"]


def test_fastq_host_reader_error_offsets_match_oracle():
    from seqan_gb300 import _native
    from seqan_gb300 import seq_io as S
    _native.build()
    for c in CASES:
        if c["format"] != "fastq" or "error" not in c:
            continue
        text = base64.b64decode(c["text"])
        with pytest.raises(O.SeqParseError) as want:
            O.oracle_read_records(text, "fastq", c["alphabet"])
        with pytest.raises(S.SeqParseError) as got:
            S.read_fastq(text, c["alphabet"])
        assert got.value.offset == want.value.offset, c["source"]


def test_fastq_host_reader_capacity_and_arguments():
    import ctypes as C
    from seqan_gb300 import _native as N
    N.build()
    text = b"@r1\nACGT\n+\nIIII\n@r2\nAC\n+\n!!\n"
    r = N.GbaSeqRecords(1, 2, None, None, None, None, None, None, 0, 0, -1)
    buf = np.frombuffer(text, np.uint8)
    assert N.lib().gba_read_fastq(None, buf.ctypes.data, len(text), 5, C.byref(r)) == N.GBA_ECAPACITY
    assert (r.num, r.residues) == (2, 6)
    assert N.lib().gba_read_fastq(None, buf.ctypes.data, len(text), 7, C.byref(r)) == N.GBA_EINVAL
    assert N.lib().gba_read_fastq(None, None, 5, 5, C.byref(r)) == N.GBA_EINVAL


@pytest.mark.skipif(not O.ref_available(), reason="compiled reference not present")
def test_oracle_matches_live_reference_random():
    import sys
    sys.path.insert(0, G.HERE)
    import make_golden as MG
    rng = np.random.Generator(np.random.PCG64(77))
    for k in range(600):
        fmt, alph = ("fasta", "fastq")[k % 2], ("dna5", "dna", "aa")[k % 3]
        t = MG.seqio_random_text(rng, fmt, alph)
        try:
            want = O.ref_read_records(t, fmt, alph)
        except O.SeqParseError as e:
            with pytest.raises(O.SeqParseError) as got:
                O.oracle_read_records(t, fmt, alph)
            assert got.value.kind == e.kind
            continue
        assert same(O.oracle_read_records(t, fmt, alph), want), t


def _big_fastq(seed, n_records, adversarial):
    rng = np.random.default_rng(seed)
    parts = []
    for k in range(n_records):
        L = int(rng.integers(0, 120))
        seq = bytes(np.frombuffer(b"ACGTN", np.uint8)[rng.integers(0, 5, L)])
        q = bytearray(rng.integers(33, 74, L).astype(np.uint8).tobytes())
        if adversarial and L and rng.random() < 0.3:
            q[0] = ord("@")                      # quality lines that start like a record
        if adversarial and rng.random() < 0.1 and L > 10:
            seq = seq[:L // 2] + b"\n" + seq[L // 2:]   # records over several lines
            q = q[:L // 3] + b"\n" + q[L // 3:]
        parts.append(b"@r%d x\n" % k + seq + b"\n+\n" + bytes(q) + b"\n")
    return b"".join(parts)


@pytest.mark.parametrize("adversarial", [False, True])
def test_fastq_host_reader_large_texts_match_oracle(adversarial):
    """Texts above the size where the host reader splits the work across threads (speculative
    record starts, checked against the previous slice's reading, sequential fallback)."""
    from seqan_gb300 import _native
    from seqan_gb300 import seq_io as S
    _native.build()
    text = _big_fastq(3 if adversarial else 4, 70_000, adversarial)
    assert len(text) > 4 << 20
    rec = S.read_fastq(text)
    assert same(list(zip(rec.ids, rec.seqs, rec.quals_list)), O.oracle_read_records(text, "fastq", "dna5"))
    bad = bytearray(text)
    pos = bytes(bad).index(b"\n+\n", len(bad) * 3 // 4)
    while bad[pos - 1] not in b"ACGTN":   # the last residue of a record's sequence
        pos = bytes(bad).index(b"\n+\n", pos + 1)
    pos -= 1
    for ch in (b"X", b"@"):
        t = bytes(bad[:pos] + ch + bad[pos + 1:])
        with pytest.raises(O.SeqParseError) as want:
            O.oracle_read_records(t, "fastq", "dna5")
        with pytest.raises(S.SeqParseError) as got:
            S.read_fastq(t)
        assert got.value.offset == want.value.offset
