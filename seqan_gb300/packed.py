"""SeqAn's packed strings: String<TValue, Packed<>> (sequence/string_packed.h).

The host string of a packed string is a 64-bit length word followed by data words; data word w
holds values w*N .. w*N+N-1 with N = 64 // bits (bits = BitsPerValue<TValue>: 2 for Dna, 3 for
Dna5, 5 for AminoAcid), value i of a word in bits (N-1-i)*bits .. (N-i)*bits-1, i.e. the first
value in the most significant used bits (string_packed.h:185-191, 600-635).  :func:`pack` builds
those words from residue codes, as `assign` on a packed string does; the engine uploads such
words and unpacks them on the device (``gba_align_packed``).
"""
from __future__ import annotations

import numpy as np

BITS = {"dna": 2, "dna5": 3, "aa": 5}


def values_per_word(bits: int) -> int:
    return 64 // bits


def pack(codes, bits: int) -> np.ndarray:
    """uint64 host words (length word first) of String<TValue, Packed<>> holding codes; an empty
    string has no host words, as in the reference.  Unused bits are zero (the reference leaves them
    undefined; readers ignore them)."""
    codes = np.asarray(codes, dtype=np.uint64)
    n = len(codes)
    if n == 0:
        return np.zeros(0, dtype=np.uint64)
    N = values_per_word(bits)
    nw = (n + N - 1) // N
    padded = np.zeros(nw * N, dtype=np.uint64)
    padded[:n] = codes
    shifts = ((N - 1 - np.arange(N)) * bits).astype(np.uint64)
    data = np.bitwise_or.reduce(padded.reshape(nw, N) << shifts[None, :], axis=1) if nw else \
        np.zeros(0, dtype=np.uint64)
    return np.concatenate([np.array([n], dtype=np.uint64), data.astype(np.uint64)])


def used_mask(n: int, bits: int) -> np.ndarray:
    """Per host word, the bits that hold values of a packed string of length n."""
    N = values_per_word(bits)
    if n == 0:
        return np.zeros(0, dtype=np.uint64)
    nw = (n + N - 1) // N
    full = np.uint64(((1 << (N * bits)) - 1) << (64 - N * bits)) >> np.uint64(64 - N * bits)
    m = np.full(nw + 1, full, dtype=np.uint64)
    m[0] = np.uint64(0xFFFFFFFFFFFFFFFF)
    rest = n - (nw - 1) * N
    m[-1] = np.uint64(((1 << (rest * bits)) - 1) << ((N - rest) * bits))
    return m


def unpack(words, bits: int) -> np.ndarray:
    words = np.asarray(words, dtype=np.uint64)
    if len(words) == 0:
        return np.zeros(0, dtype=np.uint8)
    n = int(words[0])
    N = values_per_word(bits)
    shifts = ((N - 1 - np.arange(N)) * bits).astype(np.uint64)
    vals = (words[1:, None] >> shifts[None, :]) & np.uint64((1 << bits) - 1)
    return vals.reshape(-1)[:n].astype(np.uint8)


def pack_set(seqs, bits: int):
    """(words, word_offsets) of a set of packed strings stored back to back."""
    parts = [pack(s, bits) for s in seqs]
    off = np.zeros(len(parts) + 1, dtype=np.int64)
    np.cumsum([len(p) for p in parts], out=off[1:])
    words = np.concatenate(parts) if parts else np.zeros(1, dtype=np.uint64)
    return np.ascontiguousarray(words), off
