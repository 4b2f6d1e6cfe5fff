"""SeqFileIn on the GPU machine: gzip, BGZF and bzip2 FASTA files read through the device FASTA reader
give the records of the plain text (format from the file name, compression from the magic bytes);
Raw texts (one sequence per line) give the records of the reference's readRecord(Raw)
(tests/golden/seqio_raw_cases.json)."""
import bz2
import gzip

import numpy as np
import pytest

from tests import golden_cases as G
from tests.test_seq_file_in import bgzf

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("comp", [None, "gzip", "bgzf", "bzip2"])
def test_fasta_files(engine, tmp_path, comp):
    from seqan_gb300 import seq_io as S
    rng = np.random.default_rng(11)
    text = b"".join(b">s%d desc\n%s\n" % (k, b"\n".join(
        rng.choice(list(b"ACGTN"), int(rng.integers(1, 300))).astype(np.uint8).tobytes()[q:q + 60]
        for q in range(0, 300, 60)).rstrip(b"\n")) for k in range(400))
    data = {None: text, "gzip": gzip.compress(text), "bgzf": bgzf(text, 4096), "bzip2": bz2.compress(text)}[comp]
    p = tmp_path / ("reads.fa" + {None: "", "gzip": ".gz", "bgzf": ".bgzf", "bzip2": ".bz2"}[comp])
    p.write_bytes(data)
    f = S.SeqFileIn(str(p))
    assert f.format == "fasta" and f.compression == comp
    ids, seqs = [], []
    f.readRecords(ids, seqs)
    want = S.read_fasta(text)
    assert ids == want.ids
    assert [s.tolist() for s in seqs] == [s.tolist() for s in want.seqs]


def test_raw_texts_match_reference(engine, tmp_path):
    from seqan_gb300 import seq_io as S
    cases = G.load("seqio_raw_cases.json")["cases"]
    for i, c in enumerate(cases):
        text = c["text"].encode("latin1")
        p = tmp_path / f"t{i}.raw"
        p.write_bytes(gzip.compress(text) if i % 3 == 0 else text)
        f = S.SeqFileIn(str(p), alphabet=c["alphabet"])
        assert f.format == "raw"
        if c["error"]:
            with pytest.raises(S.SeqParseError):
                f.records()
            continue
        ids, seqs = [], []
        f.readRecords(ids, seqs)
        assert [[x.decode("latin1"), s.tolist()] for x, s in zip(ids, seqs)] == c["records"], c
