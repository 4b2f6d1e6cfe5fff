"""FASTA on the GPU through gba_read_fasta: identical to the reference's readRecord loop on the
fixtures (the reference's seq_io test files, edge cases, seeded random texts) and to the oracle on
multi-megabyte texts whose headers and sequences cross the device's 128-byte chunks and 16 KB
blocks; parse errors at the reference's offset; the records align as the codes they came from."""
import base64

import numpy as np
import pytest

from oracle import oracle as O
from tests import golden_cases as G
from tests.test_seqio import CASES, expected, same

pytestmark = pytest.mark.gpu


def records(rec):
    return list(zip(rec.ids, rec.seqs, rec.quals_list))


@pytest.mark.parametrize("chunk", range(0, len(CASES), 150))
def test_fasta_fixtures_through_c_abi(engine, chunk):
    from seqan_gb300 import seq_io as S
    for c in CASES[chunk:chunk + 150]:
        if c["format"] != "fasta":
            continue
        text = base64.b64decode(c["text"])
        if "error" in c:
            with pytest.raises(S.SeqParseError) as got:
                S.read_fasta(text, c["alphabet"])
            with pytest.raises(O.SeqParseError) as want:
                O.oracle_read_records(text, "fasta", c["alphabet"])
            assert got.value.offset == want.value.offset, c["source"]
        else:
            assert same(records(S.read_fasta(text, c["alphabet"])), expected(c)), c["source"]


def random_fasta(rng, size, alphabet):
    """Records with headers of 0-400 bytes (some with '>' or tabs), sequences of 0-40k residues in
    lines of random width, blank lines, CR / CRLF / LF ends, lower case, '>' starting a record
    mid-line."""
    letters = {"dna5": b"ACGTNacgtn", "dna": b"ACGTacgt", "aa": b"ACDEFGHIKLMNPQRSTVWYXBZJOU*acdx"}[alphabet]
    out, total = [], 0
    while total < size:
        hl = int(rng.choice([0, 5, 30, 140, 400]))
        head = bytes(rng.choice(np.frombuffer(b"abcXYZ 012>\t|_", np.uint8), hl))
        L = int(rng.choice([0, 1, 50, 150, 1000, 20000, 40000]))
        body = np.frombuffer(letters, np.uint8)[rng.integers(0, len(letters), L)].tobytes()
        w = int(rng.choice([0, 60, 61, 80, 127, 128, 129]))
        nl = [b"\n", b"\r\n", b"\r"][int(rng.integers(3))]
        if w:
            body = nl.join(body[i:i + w] for i in range(0, len(body), w))
        rec = b">" + head + nl + body + (nl if rng.random() < 0.8 else b"") + (nl if rng.random() < 0.1 else b"")
        out.append(rec)
        total += len(rec)
    return b"".join(out)


@pytest.mark.parametrize("alphabet", ["dna5", "dna", "aa"])
def test_multi_megabyte_texts_match_oracle(engine, alphabet):
    from seqan_gb300 import seq_io as S
    rng = np.random.default_rng({"dna5": 1, "dna": 2, "aa": 3}[alphabet])
    for size in (3_000_000, 300_001):
        text = random_fasta(rng, size, alphabet)
        assert same(records(S.read_fasta(text, alphabet)), O.oracle_read_records(text, "fasta", alphabet))


def test_leading_text_and_unterminated_header(engine):
    from seqan_gb300 import seq_io as S
    rng = np.random.default_rng(9)
    body = random_fasta(rng, 200_000, "dna5")
    for text in (b"free text before the records\n" * 700 + body, body + b">last header without a newline" * 10):
        assert same(records(S.read_fasta(text)), O.oracle_read_records(text, "fasta"))


def test_parse_error_deep_in_the_text(engine):
    from seqan_gb300 import seq_io as S
    rng = np.random.default_rng(5)
    text = bytearray(random_fasta(rng, 2_000_000, "dna"))
    seq_bytes = [i for i in range(1_500_000, len(text)) if text[i] in b"ACGTacgt"]
    for planted in (seq_bytes[0], seq_bytes[-1]):
        t = bytes(text[:planted] + b"N" + text[planted + 1:])
        with pytest.raises(O.SeqParseError) as want:
            O.oracle_read_records(t, "fasta", "dna")
        with pytest.raises(S.SeqParseError) as got:
            S.read_fasta(t, "dna")
        assert got.value.offset == want.value.offset


def test_reads_and_windows_align_as_their_codes(engine):
    """Windows and reads written as FASTA, read back on the device and aligned: the same scores as
    aligning the codes they were written from."""
    import seqan_gb300 as sg
    from seqan_gb300 import align as A
    from seqan_gb300 import seq_io as S
    from seqan_gb300 import workloads as W
    wins, reads = W.read_windows(4000, ref_len=1_000_000, seed=12)
    tw = W.records_text(wins, "fasta", width=60, seed=1, lowercase=0.1, id_prefix="win")
    tr = W.records_text(reads, "fasta", width=0, seed=2, crlf=True)
    rw, rr = S.read_fasta(tw), S.read_fasta(tr)
    assert [bytes(x).split()[0] for x in rw.ids[:3]] == [b"win0", b"win1", b"win2"]
    assert all(np.array_equal(a, b) for a, b in zip(rw.seqs, wins))
    sc = sg.Score(2, -3, -1, -5)
    cfg = sg.AlignConfig(True, False, False, True)
    a = A.align_codes(rw.seqs, rr.seqs, sc, config=cfg, alphabet_size=5)
    b = A.align_codes(list(wins), list(reads), sc, config=cfg, alphabet_size=5)
    assert np.array_equal(a.score, b.score)


def test_empty_text_capacity_and_arguments(engine):
    import ctypes as C
    from seqan_gb300 import _native as N
    from seqan_gb300 import seq_io as S
    assert len(S.read_fasta(b"")) == 0
    with pytest.raises(S.SeqParseError) as e:
        S.read_fasta(b"no record here\n")
    assert e.value.offset == len(b"no record here\n")
    text = np.frombuffer(b">a\nACGT\n>b\nAC\n", np.uint8)
    r = N.GbaSeqRecords(2, 6, None, None, None, None, None, None, 0, 0, -1)
    assert N.lib().gba_read_fasta(engine.handle, text.ctypes.data, len(text), 5, C.byref(r)) == N.GBA_ECAPACITY
    assert (r.num, r.residues) == (2, 6)
    assert N.lib().gba_read_fasta(engine.handle, text.ctypes.data, len(text), 3, C.byref(r)) == N.GBA_EINVAL


@pytest.mark.parametrize("h_shared", [False, True])
def test_align_fasta_equals_align_of_codes(engine, h_shared):
    """gba_align_fasta (both texts parsed on the device, aligned from the codes left in HBM): the
    scores, ends, trace segments and CIGARs of aligning the same records as code arrays."""
    import seqan_gb300 as sg
    from seqan_gb300 import align as A
    from seqan_gb300 import workloads as W
    wins, reads = W.read_windows(3000, ref_len=1_000_000, seed=21)
    H = [wins[0]] if h_shared else list(wins)
    th = W.records_text(H, "fasta", width=70, seed=5, lowercase=0.05, id_prefix="win")
    tv = W.records_text(reads, "fasta", width=0, seed=6, crlf=True)
    sc = sg.Score(2, -4, -1, -6)
    cfg = sg.AlignConfig(True, False, False, True)
    got = A.align_fasta(th, tv, sc, config=cfg, traceback=True, cigar=True, h_shared=h_shared)
    want = A.align_codes(H, list(reads), sc, config=cfg, traceback=True, cigar=True, h_shared=h_shared,
                         alphabet_size=5)
    assert np.array_equal(got.score, want.score) and np.array_equal(got.end_h, want.end_h)
    assert np.array_equal(got.end_v, want.end_v)
    assert np.array_equal(got.segment_offsets, want.segment_offsets)
    assert np.array_equal(got.segments[:got.segment_offsets[-1]], want.segments[:want.segment_offsets[-1]])
    assert np.array_equal(got.cigar[:got.cigar_offsets[-1]], want.cigar[:want.cigar_offsets[-1]])


def test_align_fasta_refuses_mismatched_texts(engine):
    import seqan_gb300 as sg
    from seqan_gb300 import _native as N
    from seqan_gb300 import align as A
    with pytest.raises(N.GbaError) as e:
        A.align_codes([np.zeros(3, np.uint8)] * 2, [np.zeros(3, np.uint8)], sg.Score(1, -1, -1),
                      fasta_texts=(b">a\nACG\n>b\nACG\n", b">c\nACG\n", 5), alphabet_size=5)
    assert e.value.status == N.GBA_EINVAL
