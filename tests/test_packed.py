"""Packed strings (CPU): the restated String<TValue, Packed<>> layout equals the reference's host
words (tests/golden/packed_cases.json, bits that hold no value masked) for Dna, Dna5, AminoAcid."""
import numpy as np
import pytest

from tests import golden_cases as G

CASES = G.load("packed_cases.json")["cases"]


@pytest.mark.parametrize("case", CASES, ids=[f"{c['alphabet']}-{len(c['codes'])}" for c in CASES])
def test_pack_matches_reference_words(case):
    from seqan_gb300 import packed as P
    codes = np.array(case["codes"], dtype=np.uint8)
    want = np.array([int(w, 16) for w in case["words"]], dtype=np.uint64)
    mine = P.pack(codes, case["bits"])
    assert len(mine) == len(want)
    assert np.array_equal(mine & P.used_mask(len(codes), case["bits"]), want)
    assert np.array_equal(P.unpack(want, case["bits"]), codes)


def test_values_per_word():
    from seqan_gb300 import packed as P
    assert [P.values_per_word(b) for b in (2, 3, 5)] == [32, 21, 12]
