"""Residue codes of the reference's alphabets (ordValue of Dna, Dna5 and AminoAcid).

Character conversion follows the reference's translation tables
(basic/alphabet_residue_tabs.h): Dna5 maps A C G T/U to 0..3 and anything else to N = 4;
Dna maps anything else to A = 0; AminoAcid uses the 27-letter order
A B C D E F G H I J K L M N O P Q R S T U V W Y Z X * (basic/alphabet_residue.h:526-556),
case-insensitive, with unknown characters mapped to X = 25.
"""
from __future__ import annotations

import numpy as np

AA_LETTERS = "ABCDEFGHIJKLMNOPQRSTUVWYZX*"
DNA5_LETTERS = "ACGTN"


def _table(alphabet: str) -> np.ndarray:
    t = np.zeros(256, dtype=np.uint8)
    if alphabet in ("dna5", "dna"):
        t[:] = 4 if alphabet == "dna5" else 0
        for ch, code in (("A", 0), ("C", 1), ("G", 2), ("T", 3), ("U", 3)):
            t[ord(ch)] = code
            t[ord(ch.lower())] = code
    elif alphabet == "aa":
        t[:] = AA_LETTERS.index("X")
        for code, ch in enumerate(AA_LETTERS):
            t[ord(ch)] = code
            if ch.isalpha():
                t[ord(ch.lower())] = code
    else:
        raise ValueError(f"unknown alphabet {alphabet!r}")
    return t


_TABLES = {a: _table(a) for a in ("dna5", "dna", "aa")}


def encode(seq, alphabet: str = "dna5") -> np.ndarray:
    """Text (str/bytes) -> uint8 codes; arrays of codes pass through unchanged."""
    if isinstance(seq, str):
        seq = seq.encode()
    if isinstance(seq, (bytes, bytearray)):
        return _TABLES[alphabet][np.frombuffer(bytes(seq), dtype=np.uint8)]
    return np.ascontiguousarray(seq, dtype=np.uint8)


def decode(codes, alphabet: str = "dna5") -> str:
    letters = AA_LETTERS if alphabet == "aa" else DNA5_LETTERS
    return "".join(letters[int(c)] for c in codes)
