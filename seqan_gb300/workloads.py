"""Seeded synthetic workloads with the shapes of the benchmark configurations.

There is no public dataset for this path; these generators stand in for it:

* ``uniform_dna_pairs``   -- independent uniform ACGT pairs (the plain 1024 x 150 bp case).
* ``mutated_dna_pairs``   -- reads of uniform length in [lo, hi]; the partner is the read with
  per-position substitutions (to one of the 3 other bases) and single-base indels (50/50
  insertion/deletion, inserted base uniform).
* ``protein_pairs``       -- log-normal lengths (median 300, sigma 0.5, clipped to [50, 1000]),
  residues i.i.d. from BACKGROUND_AA; a fraction of pairs is derived by substitution to a target
  identity.
* ``read_windows``        -- reads sampled from a random reference with substitutions and indels,
  each paired with a reference window around its true origin.
* ``serving_lengths``     -- the mixed length distribution of the serving workload.
* ``seed_windows``        -- read-mapping seeds: reads against reference windows with one exact
  k-mer seed per read on the read's true diagonal (or the best-matching k-mer near it).
All generators use numpy's PCG64 with the given seed.
"""
from __future__ import annotations

import numpy as np

# Residue composition used for i.i.d. protein sequences over the 20 standard amino acids, as
# AminoAcid codes (A=0 ... Y=23).  Stand-in for "standard background frequencies": the counts
# are the residue composition of the protein FASTA files shipped with the reference's
# T-Coffee app tests, counted by tests/golden/make_golden.py.
AA20_CODES = np.array([0, 2, 3, 4, 5, 6, 7, 8, 10, 11, 12, 13, 15, 16, 17, 18, 19, 21, 22, 23], dtype=np.uint8)
BACKGROUND_AA_COUNTS = None  # filled from tests/golden/aa_background.json by load_background()


def _rng(seed):
    return np.random.Generator(np.random.PCG64(seed))


def uniform_dna_pairs(n: int, length: int, seed: int = 1):
    rng = _rng(seed)
    H = rng.integers(0, 4, size=(n, length), dtype=np.uint8)
    V = rng.integers(0, 4, size=(n, length), dtype=np.uint8)
    return list(H), list(V)


def mutate(rng, seq: np.ndarray, sub_rate: float, indel_rate: float, alphabet: int = 4) -> np.ndarray:
    """Substitutions to a different symbol and single-symbol insertions/deletions."""
    s = seq.copy()
    L = len(s)
    subs = rng.random(L) < sub_rate
    if subs.any():
        shift = rng.integers(1, alphabet, size=int(subs.sum()), dtype=np.uint8)
        s[subs] = (s[subs] + shift) % alphabet
    ev = rng.random(L) < indel_rate
    if not ev.any():
        return s
    ins = rng.random(L) < 0.5
    out = []
    prev = 0
    for pos in np.nonzero(ev)[0]:
        out.append(s[prev:pos])
        if ins[pos]:
            out.append(rng.integers(0, alphabet, size=1, dtype=np.uint8))
            out.append(s[pos:pos + 1])
        prev = pos + 1
    out.append(s[prev:])
    return np.concatenate(out).astype(np.uint8)


def mutated_dna_pairs(n: int, lo: int = 100, hi: int = 300, sub_rate: float = 0.05,
                      indel_rate: float = 0.01, seed: int = 2):
    rng = _rng(seed)
    lens = rng.integers(lo, hi + 1, size=n)
    H, V = [], []
    for L in lens:
        h = rng.integers(0, 4, size=int(L), dtype=np.uint8)
        H.append(h)
        V.append(mutate(rng, h, sub_rate, indel_rate))
    return H, V


def load_background():
    import json
    import os
    here = os.path.dirname(os.path.abspath(__file__))
    path = os.path.join(os.path.dirname(here), "tests", "golden", "aa_background.json")
    with open(path) as f:
        d = json.load(f)
    counts = np.array([d["counts"][c] for c in "ACDEFGHIKLMNPQRSTVWY"], dtype=np.float64)
    return counts / counts.sum()


def protein_pairs(n: int, median: int = 300, sigma: float = 0.5, lo: int = 50, hi: int = 1000,
                  related: float = 0.3, identity: float = 0.4, seed: int = 3, background=None):
    rng = _rng(seed)
    p = load_background() if background is None else background

    def draw_len():
        return int(np.clip(np.round(np.exp(np.log(median) + sigma * rng.standard_normal())), lo, hi))

    H, V = [], []
    for _ in range(n):
        h = AA20_CODES[rng.choice(20, size=draw_len(), p=p)]
        if rng.random() < related:
            v = h.copy()
            subs = rng.random(len(v)) >= identity
            v[subs] = AA20_CODES[rng.choice(20, size=int(subs.sum()), p=p)]
        else:
            v = AA20_CODES[rng.choice(20, size=draw_len(), p=p)]
        H.append(h)
        V.append(v)
    return H, V


def read_windows(n_reads: int, ref_len: int = 10_000_000, read_len: int = 150, flank: int = 10,
                 sub_rate: float = 0.02, indel_rate: float = 0.002, seed: int = 4):
    """Reads with their reference windows ref[o - flank, o + read_len + flank).

    Substitutions are applied to all reads at once; the few reads that draw an indel are
    rebuilt one by one."""
    rng = _rng(seed)
    ref = rng.integers(0, 4, size=ref_len, dtype=np.uint8)
    origins = rng.integers(flank, ref_len - read_len - flank, size=n_reads)
    win_len = read_len + 2 * flank
    windows = ref[(origins - flank)[:, None] + np.arange(win_len)[None, :]]
    reads = ref[origins[:, None] + np.arange(read_len)[None, :]].copy()
    subs = rng.random(reads.shape) < sub_rate
    reads[subs] = (reads[subs] + rng.integers(1, 4, size=int(subs.sum()), dtype=np.uint8)) % 4
    indel = rng.random(reads.shape) < indel_rate
    out = list(reads)
    for k in np.nonzero(indel.any(axis=1))[0]:
        r, pieces, prev = reads[k], [], 0
        for pos in np.nonzero(indel[k])[0]:
            pieces.append(r[prev:pos])
            if rng.random() < 0.5:
                pieces.append(rng.integers(0, 4, size=1, dtype=np.uint8))
                pieces.append(r[pos:pos + 1])
            prev = pos + 1
        pieces.append(r[prev:])
        out[k] = np.concatenate(pieces).astype(np.uint8)
    return list(windows), out


def seed_windows(n_reads: int, ref_len: int = 10_000_000, read_len: int = 150, flank: int = 50, k: int = 19,
                 sub_rate: float = 0.03, indel_rate: float = 0.003, seed: int = 6, tries: int = 8):
    """(windows, reads, seeds [(beginH, beginV, k)], pair_of_seed) for seed extension.

    Each read comes from ref[o, o + read_len) (with substitutions and indels) and is paired with
    the window ref[o - flank, o + read_len + flank).  Its seed is the first of `tries` random
    read k-mers that occurs in the window on the true diagonal shifted by 0, -1 or +1 (indels
    move it); a read without one gets the true-diagonal k-mer at its first tried start."""
    wins, reads = read_windows(n_reads, ref_len, read_len, flank, sub_rate, indel_rate, seed)
    rng = _rng(seed + 1)
    n = len(reads)
    W = np.stack(wins)
    lens = np.array([len(r) for r in reads], dtype=np.int64)
    R = np.full((n, int(lens.max()) + 2), 255, dtype=np.uint8)
    for i, r in enumerate(reads):
        R[i, :len(r)] = r
    found = np.zeros(n, dtype=bool)
    bh = np.zeros(n, dtype=np.int64)
    bv = np.zeros(n, dtype=np.int64)
    rows = np.arange(n)
    span = np.arange(k)
    for t in range(tries):
        start = rng.integers(0, np.maximum(lens - k, 0) + 1)
        if t == 0:
            bv[:] = start
            bh[:] = np.minimum(start + flank, W.shape[1] - k)
        for shift in (0, -1, 1):
            h0 = np.clip(start + flank + shift, 0, W.shape[1] - k)
            eq = (R[rows[:, None], start[:, None] + span] == W[rows[:, None], h0[:, None] + span]).all(axis=1)
            new = eq & ~found
            bh[new], bv[new] = h0[new], start[new]
            found |= new
    seeds = np.stack([bh, bv, np.minimum(k, lens - bv)], axis=1)
    return list(W), reads, seeds, np.arange(n, dtype=np.int32)


def serving_lengths(n: int, seed: int = 5):
    rng = _rng(seed)
    u = rng.random(n)
    lens = np.where(u < 0.90, rng.integers(100, 501, size=n),
                    np.where(u < 0.99, rng.integers(1000, 5001, size=n), 10_000))
    return lens


def records_text(seqs, fmt: str = "fasta", letters: str = "ACGTN", width: int = 0, seed: int = 0,
                 lowercase: float = 0.0, crlf: bool = False, id_prefix: str = "read") -> bytes:
    """FASTA or FASTQ text of code arrays: ids "<id_prefix><k> ...", sequences wrapped at `width`
    columns (0: one line) with a fraction `lowercase` of lower-case letters, FASTQ qualities of the
    sequence's length on one line, '\\n' or '\\r\\n' line ends."""
    rng = _rng(seed)
    nl = b"\r\n" if crlf else b"\n"
    lut_up = np.frombuffer(letters.encode(), np.uint8)
    lut_lo = np.frombuffer(letters.lower().encode(), np.uint8)
    parts = []
    for k, s in enumerate(seqs):
        s = np.asarray(s, np.uint8)
        chars = lut_up[s]
        if lowercase:
            low = rng.random(len(s)) < lowercase
            chars = np.where(low, lut_lo[s], chars)
        body = chars.tobytes()
        if width and len(body) > width:
            body = nl.join(body[i:i + width] for i in range(0, len(body), width))
        if fmt == "fasta":
            parts.append(b">%s%d len=%d" % (id_prefix.encode(), k, len(s)) + nl + body + nl)
        else:
            qual = (rng.integers(33, 74, len(s)).astype(np.uint8)).tobytes()
            parts.append(b"@%s%d" % (id_prefix.encode(), k) + nl + body + nl + b"+" + nl + qual + nl)
    return b"".join(parts)


def chain_pairs(n: int, lo: int = 1000, hi: int = 3000, sub_rate: float = 0.05, indel_rate: float = 0.01,
                min_seed: int = 20, max_seeds: int = 64, seed: int = 31):
    """Genomic pairs with seed chains for banded chain alignment (LAGAN-style anchors): H random of
    lo..hi bp, V = H with substitutions and single-base indels, and per pair the exact matches of at
    least min_seed bp along the true alignment as Seed<Simple>(beginH, beginV, endH, endV), in chain
    order (colinear, non-overlapping), at most max_seeds evenly picked.  Returns (H, V, chains)."""
    rng = _rng(seed)
    H, V, chains = [], [], []
    for _ in range(n):
        m = int(rng.integers(lo, hi + 1))
        h = rng.integers(0, 4, m).astype(np.uint8)
        r = rng.random(m)
        dele = r < indel_rate / 2                       # h[i] dropped
        ins = (r >= indel_rate / 2) & (r < indel_rate)  # a random base before h[i]
        kept = ~dele
        sub = rng.random(m) < sub_rate
        hv = np.where(sub, (h + rng.integers(1, 4, m)) % 4, h).astype(np.uint8)
        width = kept.astype(np.int64) + ins.astype(np.int64)
        start = np.concatenate([[0], np.cumsum(width)[:-1]])
        vpos = np.where(kept, start + ins, -1)         # V position of each kept residue
        v = np.empty(int(width.sum()) or 1, np.uint8)
        v[:] = rng.integers(0, 4, v.size)               # inserted bases (and a filler for an empty V)
        v[vpos[kept]] = hv[kept]
        # maximal runs of equal residues on one diagonal of the true alignment
        match = kept & ~sub
        cont = match[:-1] & match[1:] & (vpos[1:] == vpos[:-1] + 1)
        seeds = []
        if match.any():
            starts = np.flatnonzero(match & ~np.concatenate([[False], cont]))
            ends = np.flatnonzero(match & ~np.concatenate([cont, [False]]))
            for i, j in zip(starts, ends):
                if j - i + 1 >= min_seed:
                    seeds.append((int(i), int(vpos[i]), int(j) + 1, int(vpos[j]) + 1))
        if len(seeds) > max_seeds:
            pick = np.linspace(0, len(seeds) - 1, max_seeds).round().astype(int)
            seeds = [seeds[q] for q in pick]
        H.append(h)
        V.append(v)
        chains.append(np.array(seeds, np.int32).reshape(-1, 4))
    return H, V, chains
