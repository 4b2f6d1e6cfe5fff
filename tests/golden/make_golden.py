"""Generates the golden fixtures in tests/golden/ from the compiled reference.

Run where the reference tree exists (it builds oracle/_ref/ from its headers):
    python tests/golden/make_golden.py [--only seeds|extend|extend_banded|waterman_eggert|waterman_eggert_banded|raw|packed|sam|seqio|bam|cpp|dynamic|banded_chain|tags]
Outputs (all small, committed):
  reference_cases.json  seeded inputs with the reference's outputs: batch scores through
                        ExecutionPolicy<Parallel, Vectorial>, batch Gaps rows / clip positions /
                        CIGARs, and raw TraceSegment_ lists of the single-pair DP.
  blosum62.json         the reference's 27x27 Blosum62 table (score/score_matrix_data.h).
  alphabets.json        the reference's char -> ordValue maps for Dna5, Dna and AminoAcid.
  seed_cases.json       seeds extended by the reference's extendSeed (MatchExtend, UnGappedXDrop,
                        GappedXDrop; seeds/seeds_extension.h) with the gapped extension scores.
  sam_cases.json        BamAlignmentRecord fields and the SAM text the reference's writer makes of them.
  sam_tag_cases.json, sam_float_tag_cases.json  records with BAM tags (integer, character, string
                        and array values; the second set with float values of every kind) and the
                        SAM lines / BAM records the reference's writers make of them.
  packed_cases.json     host words of String<Dna|Dna5|AminoAcid, Packed<>> built by the reference
                        (the bits that hold no value, undefined there, masked to zero).
  extend_cases.json     ungapped seed alignments grown by the reference's extendAlignment
                        (align_extend/align_extend.h) with and without X-drop: score and rows.
  extend_banded_cases.json  the other extendAlignment overloads: (lowerDiag, upperDiag) with and
                        without xDrop, origScore, aligned parts with gaps.
  waterman_eggert_cases.json  suboptimal local alignments of the reference's
                        LocalAlignmentEnumerator<Score, Unbanded> (scores, rows, positions).
  waterman_eggert_banded_cases.json  the same for LocalAlignmentEnumerator<Score, Banded> with
                        random diagonal bands.
  seqio_raw_cases.json  Raw texts (one sequence per line; LF, CR LF and CR line ends, empty lines,
                        blanks, invalid characters) read by the reference's readRecord(Raw).
  dynamic_cases.json    pairs aligned by the reference's single-pair DP with DynamicGaps cells
                        (score and raw TraceSegment_ list) for the shapes oracle/ref/units/dynamic_*.cpp
                        instantiate.
  cpp_binding_expected.txt  the output of tests/cpp/seqan_binding.cpp built with
                        -DGBA_AS_REFERENCE: the binding's calls run by the reference itself.
  aa_background.json    residue counts of the reference's T-Coffee test FASTA files, the
                        stand-in for background amino-acid frequencies.
"""
from __future__ import annotations

import collections
import glob
import json
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
REFERENCE = os.environ.get("SEQAN_REF_ROOT", "/root/reference")

from oracle import oracle as O  # noqa: E402

DNA = "ACGTN"
AA = "ABCDEFGHIJKLMNOPQRSTUVWYZX*"


def text(codes, alphabet):
    letters = AA if alphabet == "aa" else DNA
    return "".join(letters[int(c)] for c in codes)


def problem_dict(pb: O.Problem):
    return {"mode": pb.mode, "free_ends": pb.free_ends, "band": list(pb.band) if pb.band else None,
            "match": pb.match, "mismatch": pb.mismatch, "gap_open": pb.gap_open,
            "gap_extend": pb.gap_extend, "blosum62": pb.matrix is not None,
            "score_bits": pb.score_bits, "alphabet": pb.alphabet}


def rand_pairs(rng, n, lo, hi, alphabet, related=0.5):
    H, V = [], []
    for _ in range(n):
        if alphabet == "dna":
            h = rng.integers(0, 4, rng.integers(lo, hi + 1)).astype(np.uint8)
        else:
            h = rng.choice(np.array([0, 2, 3, 4, 5, 6, 7, 8, 10, 11, 12, 13, 15, 16, 17, 18, 19, 21, 22, 23],
                                    dtype=np.uint8), rng.integers(lo, hi + 1))
        if rng.random() < related:
            v = h.copy()
            sub = rng.random(len(v)) < 0.15
            v[sub] = (v[sub] + 1) % (4 if alphabet == "dna" else 20)
            if len(v) > 4 and rng.random() < 0.7:
                a = rng.integers(0, len(v) - 2)
                v = np.concatenate([v[:a], v[a + rng.integers(1, 3):]]) if rng.random() < 0.5 else \
                    np.concatenate([v[:a], h[:rng.integers(1, 4)], v[a:]])
        else:
            lv = rng.integers(lo, hi + 1)
            v = rng.integers(0, 4, lv).astype(np.uint8) if alphabet == "dna" else \
                rng.integers(0, 20, lv).astype(np.uint8)
        H.append(h.astype(np.uint8))
        V.append(v.astype(np.uint8))
    return H, V


DNA_SCORES = [(2, -3, -5, -5), (2, -4, -6, -1), (4, -2, -10, -4), (2, -1, -1, -1)]  # match, mismatch, open, extend
FREE_END_SETS = [0, 15, 9, 6]


def main():
    if not os.path.isdir(REFERENCE):
        sys.exit("the reference tree is needed to generate fixtures")
    if not O.ref_available():
        subprocess.check_call(["make", "-C", os.path.join(ROOT, "oracle", "ref"), f"-j{os.cpu_count()}",
                               f"SEQAN_INCLUDE={os.path.join(REFERENCE, 'include')}"])
    b62 = O.ref_blosum62()
    only = sys.argv[sys.argv.index("--only") + 1] if "--only" in sys.argv else None
    if only == "seeds":
        write_seeds(b62)
        return
    if only == "extend":
        write_extend(b62)
        return
    if only == "extend_banded":
        write_extend_banded(b62)
        return
    if only == "waterman_eggert":
        write_waterman_eggert(b62)
        return
    if only == "waterman_eggert_banded":
        write_waterman_eggert_banded(b62)
        return
    if only == "raw":
        write_raw_cases()
        return
    if only == "packed":
        write_packed()
        return
    if only == "sam":
        write_sam_cases()
        return
    if only == "seqio":
        write_seqio()
        return
    if only == "bam":
        write_bam_cases()
        return
    if only == "cpp":
        write_cpp_binding()
        return
    if only == "dynamic":
        write_dynamic_cases(b62)
        return
    if only == "banded_chain":
        write_banded_chain()
        return
    if only == "tags":
        write_tag_cases()
        return
    rng = np.random.Generator(np.random.PCG64(20261203))
    cases = []

    def add(kind, pb, H, V):
        alph = pb.alphabet
        case = {"kind": kind, "problem": problem_dict(pb),
                "H": [text(h, alph) for h in H], "V": [text(v, alph) for v in V]}
        if kind == "score":
            case["scores"] = [int(x) for x in O.ref_batch_score(pb, H, V, threads=2)]
        elif kind == "gaps":
            sc, clip, rows, cig = O.ref_batch_gaps(pb, H, V, threads=2, cigar=True)
            case["scores"] = [int(x) for x in sc]
            case["clip"] = [[int(x) for x in c] for c in clip]
            case["rows"] = [list(r) for r in rows]
            case["cigar"] = cig
        else:
            segs, scores = [], []
            for h, v in zip(H, V):
                s, sg = O.ref_pair_segments(pb, h, v)
                scores.append(int(s))
                segs.append([list(x) for x in sg])
            case["scores"] = scores
            case["segments"] = segs
        cases.append(case)

    # Batch scores (SIMD batch path).
    for bits in (16, 32):
        for (mt, mm, go, ge) in DNA_SCORES:
            H, V = rand_pairs(rng, 48, 1, 70, "dna")
            for fe in FREE_END_SETS:
                add("score", O.Problem("global", fe, None, mt, mm, go, ge, None, bits, "dna"), H, V)
            add("score", O.Problem("local", 0, None, mt, mm, go, ge, None, bits, "dna"), H, V)
    for fe in FREE_END_SETS:
        H, V = rand_pairs(rng, 32, 1, 90, "aa")
        add("score", O.Problem("global", fe, None, 0, 0, -11, -1, b62, 16, "aa"), H, V)
    H, V = rand_pairs(rng, 32, 1, 90, "aa")
    add("score", O.Problem("local", 0, None, 0, 0, -11, -1, b62, 16, "aa"), H, V)
    # Batch Gaps (SIMD batch path with traceback) + CIGAR.
    for (mt, mm, go, ge) in DNA_SCORES[:3]:
        H, V = rand_pairs(rng, 32, 1, 60, "dna")
        for fe in FREE_END_SETS:
            add("gaps", O.Problem("global", fe, None, mt, mm, go, ge, None, 16, "dna"), H, V)
        add("gaps", O.Problem("local", 0, None, mt, mm, go, ge, None, 16, "dna"), H, V)
        add("gaps", O.Problem("global", 0, None, mt, mm, go, ge, None, 32, "dna"), H, V)
    for fe in FREE_END_SETS:
        H, V = rand_pairs(rng, 24, 1, 80, "aa")
        add("gaps", O.Problem("global", fe, None, 0, 0, -11, -1, b62, 16, "aa"), H, V)
    H, V = rand_pairs(rng, 24, 1, 80, "aa")
    add("gaps", O.Problem("local", 0, None, 0, 0, -11, -1, b62, 16, "aa"), H, V)
    # Raw segment lists (single-pair DP), all 16 AlignConfigs.
    for (mt, mm, go, ge) in DNA_SCORES:
        H, V = rand_pairs(rng, 12, 1, 40, "dna")
        for fe in range(16):
            add("segments", O.Problem("global", fe, None, mt, mm, go, ge, None, 32, "dna"), H, V)
        add("segments", O.Problem("local", 0, None, mt, mm, go, ge, None, 32, "dna"), H, V)

    # Banded: random bands that meet the matrix.  Shapes the reference cannot run are left out:
    # bands that start in the last column or end in the first one (its traceback does not
    # terminate there) and one-diagonal bands whose diagonal leaves the matrix through the
    # bottom row with m < -2 * lower (its diagonal-only path reads past the end of V).
    def band_ok(m, n, lo, up):
        hb = max(0, min(m - 1, lo))
        hbot = max(0, min(m, up + n) - 1)
        if hb == m - 1 or hbot == 0:
            return False
        if lo == up and max(0, min(n - 1, -lo)) > min(n - 1, lo + m):
            return False
        return True

    def band_pairs(count, widths):
        out = []
        while len(out) < count:
            H, V = rand_pairs(rng, 1, 2, 40, "dna")
            m, n = len(H[0]), len(V[0])
            lo = int(rng.integers(-n - 1, m + 1))
            up = lo + int(rng.choice(widths)) - 1
            if up < -n or lo > m or not band_ok(m, n, lo, up):
                continue
            out.append((H[0], V[0], lo, up))
        return out

    # The reference's SIMD batch traceback path with a band hangs or drops residues on several
    # shapes, so banded tracebacks come from its scalar single-pair path ("segments"), and
    # banded scores from single-pair batches.
    for kind, bits_list, fes in (("score", (16, 32), (0, 9)), ("segments", (32,), (0, 9, 15, 6))):
        for bits in bits_list:
            for mode in ("global", "local"):
                for fe in (fes if mode == "global" else (0,)):
                    for (mt, mm, go, ge) in DNA_SCORES[:3]:
                        added = 0
                        while added < 6:
                            (h, v, lo, up), = band_pairs(1, (1, 2, 3, 5, 8, 13, 33))
                            pb = O.Problem(mode, fe, (lo, up), mt, mm, go, ge, None, bits, "dna")
                            if not O.ref_has_shape({"score": 0, "gaps": 1, "segments": 2}[kind], pb):
                                break
                            # Tracebacks only for bands _checkBandProperties accepts: for the others
                            # the reference leaves the Gaps rows inconsistent.
                            if kind != "score" and not O.oracle_batch(pb, [h], [v]).valid[0]:
                                continue
                            add(kind, pb, [h], [v])
                            added += 1

    # Read-to-reference verification shape: 150 bp reads (substitutions only, so the batch has
    # equal lengths -- the reference's SIMD batch path with a band only works then) against
    # 170 bp windows, free reference overhang, band (-6, 26), affine (2,-4,-1,-6), with CIGARs.
    from seqan_gb300 import workloads as W
    wins, reads = W.read_windows(48, ref_len=100_000, sub_rate=0.03, indel_rate=0.0, seed=12)
    reads = [r[:150] for r in reads]
    add("gaps", O.Problem("global", 9, (-6, 26), 2, -4, -6, -1, None, 16, "dna"), wins, reads)
    add("score", O.Problem("global", 9, (-6, 26), 2, -4, -6, -1, None, 16, "dna"), wins, reads)

    with open(os.path.join(HERE, "reference_cases.json"), "w") as f:
        json.dump({"generator": "tests/golden/make_golden.py", "seed": 20261203,
                   "ref_simd_bytes": int(O.libref().ref_simd_bytes()), "cases": cases}, f, separators=(",", ":"))
    with open(os.path.join(HERE, "blosum62.json"), "w") as f:
        json.dump({"alphabet": AA, "matrix": b62.tolist()}, f)
    printable = "".join(chr(i) for i in range(32, 127))
    with open(os.path.join(HERE, "alphabets.json"), "w") as f:
        json.dump({"chars": printable,
                   "dna5": O.ref_encode("dna5", printable).tolist(),
                   "dna": O.ref_encode("dna", printable).tolist(),
                   "aa": O.ref_encode("aa", printable).tolist()}, f)
    files = sorted(glob.glob(os.path.join(REFERENCE, "apps/seqan_tcoffee/tests/*.fa")) +
                   glob.glob(os.path.join(REFERENCE, "apps/seqan_tcoffee/tests/*.fasta")))
    cnt = collections.Counter()
    for fn in files:
        with open(fn) as fh:
            for line in fh:
                if not line.startswith(">"):
                    cnt.update(c for c in line.strip().upper() if c in "ACDEFGHIKLMNPQRSTVWY")
    with open(os.path.join(HERE, "aa_background.json"), "w") as f:
        json.dump({"source": "apps/seqan_tcoffee/tests/*.fa, *.fasta of the reference tree",
                   "files": len(files), "counts": {c: cnt[c] for c in "ACDEFGHIKLMNPQRSTVWY"}}, f)
    print(f"{len(cases)} alignment cases written")
    write_seeds(b62)
    write_extend(b62)
    write_extend_banded(b62)
    write_waterman_eggert(b62)
    write_waterman_eggert_banded(b62)
    write_raw_cases()
    write_packed()
    write_sam_cases()


def sam_records(rng, n):
    from seqan_gb300 import sam as S
    contigs = ["chr1", "chr2", "scaffold_17", "X"]
    names, cig, seq, qual = [], [], [], []
    for k in range(n):
        names.append(f"read{k}" + ("" if k % 7 else "/1"))
        ops = []
        for _ in range(int(rng.integers(0, 6)) if k % 11 else 0):
            ops.append((int(rng.integers(1, 300)) << 4) | int(rng.integers(0, 9)))
        cig.append(ops)
        L = 0 if k % 13 == 0 else int(rng.integers(1, 160))
        seq.append(rng.integers(0, 5, L).astype(np.uint8))
        qual.append("" if k % 5 == 0 else "".join(chr(33 + int(x)) for x in rng.integers(0, 42, L)))
    rid = rng.integers(-1, len(contigs), n).astype(np.int32)
    rn = np.where(rng.random(n) < 0.3, rid, rng.integers(-1, len(contigs), n)).astype(np.int32)
    return S.SamRecords(names, rng.choice([0, 4, 16, 99, 147, 256, 2048, 65535], n).astype(np.uint16), rid,
                        rng.integers(-1, 250_000_000, n).astype(np.int32), rng.choice([0, 1, 60, 255], n).astype(np.uint8),
                        cig, rn, rng.integers(-1, 250_000_000, n).astype(np.int32),
                        np.where(rng.random(n) < 0.3, 0, rng.integers(-800, 800, n)).astype(np.int32), seq, qual,
                        contigs)


def write_sam_cases():
    rng = np.random.Generator(np.random.PCG64(20261207))
    rec = sam_records(rng, 400)
    text = O.ref_write_sam(rec)
    with open(os.path.join(HERE, "sam_cases.json"), "w") as f:
        json.dump({"generator": "tests/golden/make_golden.py", "seed": 20261207, "contigs": rec.contigs,
                   "qname": rec.qname, "flag": rec.flag.tolist(), "ref_id": rec.ref_id.tolist(),
                   "pos": rec.pos.tolist(), "mapq": rec.mapq.tolist(), "cigar": [list(c) for c in rec.cigar],
                   "next_ref_id": rec.next_ref_id.tolist(), "next_pos": rec.next_pos.tolist(),
                   "tlen": rec.tlen.tolist(), "seq": [s.tolist() for s in rec.seq], "qual": rec.qual,
                   "text": text}, f, separators=(",", ":"))
    print(f"{len(rec.qname)} SAM records written")


def random_tags(rng, floats=False):
    """BAM-form tag bytes: 0-5 tags of every type the SAM conversion writes (A, c, C, s, S, i, I,
    Z, H, B arrays of integers; f and B:f when floats)."""
    import struct
    out = b""
    kinds = list("AcCsSiIZHB") + (["f", "Bf"] if floats else [])
    for _ in range(int(rng.integers(0, 6))):
        name = bytes([int(rng.integers(65, 91)), int(rng.integers(48, 91))])
        kd = kinds[int(rng.integers(0, len(kinds)))]
        if kd == "A":
            out += name + b"A" + bytes([int(rng.integers(33, 127))])
        elif kd in "cCsSiI":
            fmt = {"c": "<b", "C": "<B", "s": "<h", "S": "<H", "i": "<i", "I": "<I"}[kd]
            lo, hi = {"c": (-128, 128), "C": (0, 256), "s": (-32768, 32768), "S": (0, 65536),
                      "i": (-2 ** 31, 2 ** 31), "I": (0, 2 ** 32)}[kd]
            out += name + kd.encode() + struct.pack(fmt, int(rng.integers(lo, hi)))
        elif kd in "ZH":
            ln = int(rng.integers(0, 12))
            alphabet = b"0123456789ABCDEF" if kd == "H" else bytes(range(33, 127))
            out += name + kd.encode() + bytes(alphabet[int(x)] for x in rng.integers(0, len(alphabet), ln)) + b"\0"
        elif kd == "f":
            out += name + b"f" + random_float_bytes(rng)
        else:
            et = "f" if kd == "Bf" else "cCsSiI"[int(rng.integers(0, 6))]
            cnt = int(rng.integers(0, 6))
            fmt = {"c": "<b", "C": "<B", "s": "<h", "S": "<H", "i": "<i", "I": "<I", "f": "<f"}[et]
            lim = {"c": 127, "C": 255, "s": 32767, "S": 65535, "i": 2 ** 31 - 1, "I": 2 ** 32 - 1, "f": 1}[et]
            if et == "f":
                body = b"".join(random_float_bytes(rng) for _ in range(cnt))
            else:
                body = b"".join(struct.pack(fmt, int(rng.integers(0 if et.isupper() else -lim, lim)))
                                for _ in range(cnt))
            out += name + b"B" + et.encode() + struct.pack("<I", cnt) + body
    return out


def random_float_bytes(rng):
    """A little-endian float32 for a tag: normal values, any bit pattern (denormals, infinities,
    NaNs of either sign), halves and decimal powers whose %g rounding ties."""
    import struct
    r = int(rng.integers(0, 4))
    if r == 0:
        return struct.pack("<f", float(rng.normal()) * 10.0 ** int(rng.integers(-8, 9)))
    if r == 1:
        if rng.random() < 0.3:   # infinities, NaNs of both signs, -0, the smallest denormal, the largest float
            return struct.pack("<I", [0x7f800000, 0xff800000, 0x7fc00000, 0xffc00000, 0x80000000, 1,
                                      0x7f7fffff][int(rng.integers(0, 7))])
        return struct.pack("<I", int(rng.integers(0, 2 ** 32)))
    if r == 2:
        return struct.pack("<f", int(rng.integers(-4_000_000, 4_000_000)) * 0.5)
    return struct.pack("<f", min(float(10.0 ** int(rng.integers(-40, 38))) * int(rng.integers(1, 20)), 3.0e38))


def write_tag_cases():
    """SAM lines and BAM records with tags, through the reference's writers (appendTagsBamToSam and
    the raw tag bytes of write_bam.h)."""
    import base64
    rng = np.random.Generator(np.random.PCG64(20261211))
    rec = sam_records(rng, 300)
    rec.tags = [random_tags(rng) for _ in rec.qname]
    text = O.ref_write_sam(rec)
    data = O.ref_write_bam(rec)
    with open(os.path.join(HERE, "sam_tag_cases.json"), "w") as f:
        json.dump({"generator": "tests/golden/make_golden.py --only tags", "seed": 20261211, "contigs": rec.contigs,
                   "qname": rec.qname, "flag": rec.flag.tolist(), "ref_id": rec.ref_id.tolist(),
                   "pos": rec.pos.tolist(), "mapq": rec.mapq.tolist(), "cigar": [list(map(int, c)) for c in rec.cigar],
                   "next_ref_id": rec.next_ref_id.tolist(), "next_pos": rec.next_pos.tolist(),
                   "tlen": rec.tlen.tolist(), "seq": [s.tolist() for s in rec.seq], "qual": rec.qual,
                   "tags": [base64.b64encode(t).decode() for t in rec.tags], "text": text,
                   "bam": base64.b64encode(data).decode()}, f, separators=(",", ":"))
    print(f"{len(rec.qname)} SAM/BAM records with tags written")
    rng = np.random.Generator(np.random.PCG64(20261213))
    rec = sam_records(rng, 300)
    rec.tags = [random_tags(rng, floats=True) for _ in rec.qname]
    text = O.ref_write_sam(rec)
    data = O.ref_write_bam(rec)
    with open(os.path.join(HERE, "sam_float_tag_cases.json"), "w") as f:
        json.dump({"generator": "tests/golden/make_golden.py --only tags", "seed": 20261213, "contigs": rec.contigs,
                   "qname": rec.qname, "flag": rec.flag.tolist(), "ref_id": rec.ref_id.tolist(),
                   "pos": rec.pos.tolist(), "mapq": rec.mapq.tolist(), "cigar": [list(map(int, c)) for c in rec.cigar],
                   "next_ref_id": rec.next_ref_id.tolist(), "next_pos": rec.next_pos.tolist(),
                   "tlen": rec.tlen.tolist(), "seq": [s.tolist() for s in rec.seq], "qual": rec.qual,
                   "tags": [base64.b64encode(t).decode() for t in rec.tags], "text": text,
                   "bam": base64.b64encode(data).decode()}, f, separators=(",", ":"))
    print(f"{len(rec.qname)} SAM/BAM records with float tags written")


def write_packed():
    import ctypes as C
    from seqan_gb300 import packed as P
    lib = O.libref()
    lib.ref_pack_string.argtypes = [C.c_int32, C.c_void_p, C.c_int64, C.c_void_p, C.c_int64]
    lib.ref_pack_string.restype = C.c_int64
    rng = np.random.Generator(np.random.PCG64(20261206))
    cases = []
    for alph, name, A in ((2, "dna", 4), (0, "dna5", 5), (1, "aa", 27)):
        bits = P.BITS[name]
        for n in [0, 1, 2, P.values_per_word(bits) - 1, P.values_per_word(bits), P.values_per_word(bits) + 1] + \
                [int(x) for x in rng.integers(3, 400, 20)]:
            codes = rng.integers(0, A, n).astype(np.uint8)
            out = np.zeros(n // P.values_per_word(bits) + 4, dtype=np.uint64)
            nw = lib.ref_pack_string(alph, codes.ctypes.data, n, out.ctypes.data, len(out))
            words = out[:nw] & P.used_mask(n, bits)
            cases.append({"alphabet": name, "bits": bits, "codes": codes.tolist(),
                          "words": [format(int(w), "016x") for w in words]})
    with open(os.path.join(HERE, "packed_cases.json"), "w") as f:
        json.dump({"generator": "tests/golden/make_golden.py", "seed": 20261206, "cases": cases}, f,
                  separators=(",", ":"))
    print(f"{len(cases)} packed-string cases written")


def write_extend(b62):
    """extendAlignment on ungapped seeds: random DNA and protein pairs (linear and affine gaps,
    X-drop off and 0..30), plus read-mapping shapes (150 bp reads in 250 bp windows)."""
    from seqan_gb300 import workloads as W
    rng = np.random.Generator(np.random.PCG64(20261205))
    cases = []

    def add(pb, h, v, pos, d):
        r = O.ref_extend_alignment(pb, h, v, pos, d)
        cases.append({"alphabet": pb.alphabet, "blosum62": pb.matrix is not None, "match": pb.match,
                      "mismatch": pb.mismatch, "gap_open": pb.gap_open, "gap_extend": pb.gap_extend,
                      "xdrop": pb.xdrop, "H": text(h, pb.alphabet), "V": text(v, pb.alphabet),
                      "positions": [int(x) for x in pos], "direction": int(d), "score": r.score,
                      "row0": r.row0, "row1": r.row1, "ends": [r.h_begin, r.h_end, r.v_begin, r.v_end]})

    for trial in range(600):
        aa = trial % 4 == 3
        A = 20 if aa else 4
        L = int(rng.integers(2, 120))
        h = rng.integers(0, A, L).astype(np.uint8)
        v = W.mutate(rng, h, float(rng.uniform(0, 0.3)), float(rng.uniform(0, 0.08)), alphabet=A)
        if trial % 5 == 0:
            v = rng.integers(0, A, int(rng.integers(2, 120))).astype(np.uint8)
        if aa:
            h, v = W.AA20_CODES[h], W.AA20_CODES[v]
        sl = int(rng.integers(1, min(len(h), len(v), 12) + 1))
        hb = int(rng.integers(0, len(h) - sl + 1))
        vb = min(max(hb + int(rng.integers(-3, 4)), 0), len(v) - sl)
        xd = None if trial % 3 == 0 else int(rng.integers(0, 31))
        if aa:
            go = int(rng.choice([-11, -9, -4]))
            pb = O.Problem("extend", 0, None, 0, 0, go, int(rng.choice([-1, go])), b62, 32, "aa", xd)
        else:
            go = int(rng.integers(-8, 0))
            pb = O.Problem("extend", 0, None, int(rng.integers(1, 4)), int(rng.integers(-4, 0)), go,
                           int(rng.choice([go, -1, -2])), None, 32, "dna", xd)
        add(pb, h, v, (hb, vb, hb + sl, vb + sl), int(rng.integers(1, 4)))
    wins, reads, seeds, _ = W.seed_windows(60, seed=15)
    for k in range(60):
        bh, bv, sl = (int(x) for x in seeds[k])
        pb = O.Problem("extend", 0, None, 1, -2, -4 if k % 2 else -2, -1 if k % 2 else -2, None, 32, "dna",
                       None if k % 3 == 0 else 20)
        add(pb, wins[k], reads[k], (bh, bv, bh + sl, bv + sl), 3)
    with open(os.path.join(HERE, "extend_cases.json"), "w") as f:
        json.dump({"generator": "tests/golden/make_golden.py", "seed": 20261205, "cases": cases}, f,
                  separators=(",", ":"))
    print(f"{len(cases)} extendAlignment cases written")


def write_extend_banded(b62):
    """extendAlignment's other overloads: (lowerDiag, upperDiag) with and without xDrop, origScore,
    and aligned parts with gaps (rows given as text).  Bands include one-diagonal bands, bands
    wider than the matrices and bands that miss a side's matrix (lowerDiag > 0: the reference's
    invalid value; the aligned part's score is then set high enough that the reference's int sum
    stays in range)."""
    from seqan_gb300 import workloads as W
    rng = np.random.Generator(np.random.PCG64(20261207))
    cases = []
    for trial in range(700):
        aa = trial % 5 == 4
        A = 20 if aa else 4
        L = int(rng.integers(2, 160))
        h = rng.integers(0, A, L).astype(np.uint8)
        v = W.mutate(rng, h, float(rng.uniform(0, 0.3)), float(rng.uniform(0, 0.08)), alphabet=A)
        if trial % 6 == 0:
            v = rng.integers(0, A, int(rng.integers(2, 160))).astype(np.uint8)
        if aa:
            h, v = W.AA20_CODES[h], W.AA20_CODES[v]
        letters = "ABCDEFGHIJKLMNOPQRSTUVWYZX*" if aa else "ACGTN"
        sl = int(rng.integers(0, min(len(h), len(v), 14) + 1))
        hb = int(rng.integers(0, len(h) - sl + 1))
        vb = min(max(hb + int(rng.integers(-3, 4)), 0), len(v) - sl)
        pos = (hb, vb, hb + sl, vb + sl)
        kind = trial % 8
        if kind == 0:
            band = (0, 0)
        elif kind == 1:
            band = (-int(rng.integers(0, 3)), int(rng.integers(0, 3)))
        elif kind == 2:
            band = (int(rng.integers(1, 4)), int(rng.integers(4, 9)))          # misses the matrices
        elif kind == 3:
            band = (-int(rng.integers(40, 300)), int(rng.integers(40, 300)))   # wider than them
        else:
            band = (-int(rng.integers(0, 25)), int(rng.integers(0, 25)))
        xd = None if trial % 3 == 0 else int(rng.integers(0, 31))
        if aa:
            go = int(rng.choice([-11, -9, -4]))
            pb = O.Problem("extend", 0, band, 0, 0, go, int(rng.choice([-1, go])), b62, 32, "aa", xd)
        else:
            go = int(rng.integers(-8, 0))
            pb = O.Problem("extend", 0, band, int(rng.integers(1, 4)), int(rng.integers(-4, 0)), go,
                           int(rng.choice([go, -1, -2])), None, 32, "dna", xd)
        center = None
        if trial % 4 == 1 and sl >= 2:
            t0 = "".join(letters[c] for c in h[hb:hb + sl])
            t1 = "".join(letters[c] for c in v[vb:vb + sl])
            i, g = int(rng.integers(1, sl)), int(rng.integers(1, 4))
            if rng.random() < 0.5:
                t0 = t0[:i] + "-" * g + t0[i:]
                j = int(rng.integers(0, len(t1) + 1))
                t1 = t1[:j] + "-" * g + t1[j:]
            else:
                t1 = t1[:i] + "-" * g + t1[i:]
                j = int(rng.integers(0, len(t0) + 1))
                t0 = t0[:j] + "-" * g + t0[j:]
            center = [t0, t1]
        orig = None if trial % 3 != 2 else int(rng.integers(-40, 60))
        if kind == 2:
            orig = 1 << 20
        d = int(rng.integers(0, 4))
        r = O.ref_extend_alignment(pb, h, v, pos, d, orig_score=orig, center=center)
        cases.append({"alphabet": pb.alphabet, "blosum62": pb.matrix is not None, "match": pb.match,
                      "mismatch": pb.mismatch, "gap_open": pb.gap_open, "gap_extend": pb.gap_extend,
                      "xdrop": pb.xdrop, "band": list(band), "orig_score": orig, "center": center,
                      "H": text(h, pb.alphabet), "V": text(v, pb.alphabet), "positions": [int(x) for x in pos],
                      "direction": d, "score": r.score, "row0": r.row0, "row1": r.row1,
                      "ends": [r.h_begin, r.h_end, r.v_begin, r.v_end]})
    with open(os.path.join(HERE, "extend_banded_cases.json"), "w") as f:
        json.dump({"generator": "tests/golden/make_golden.py", "seed": 20261207, "cases": cases}, f,
                  separators=(",", ":"))
    print(f"{len(cases)} banded / origScore / gapped extendAlignment cases written")


def write_waterman_eggert(b62):
    """Suboptimal local alignments from the reference's LocalAlignmentEnumerator<Score, Unbanded>:
    random DNA and protein pairs (related and unrelated), several scores, gap costs and cutoffs,
    up to 25 alignments each (enumerations the reference cannot continue -- after an alignment
    whose first column is a gap -- are cut where the oracle stops)."""
    from seqan_gb300 import workloads as W
    rng = np.random.Generator(np.random.PCG64(20261208))
    cases = []
    for trial in range(300):
        aa = trial % 4 == 3
        A = 20 if aa else 4
        m = int(rng.integers(1, 60))
        h = rng.integers(0, A, m).astype(np.uint8)
        if rng.random() < 0.6:
            v = W.mutate(rng, h, float(rng.uniform(0, 0.3)), float(rng.uniform(0, 0.08)), alphabet=A)
        else:
            v = rng.integers(0, A, int(rng.integers(1, 60))).astype(np.uint8)
        if trial % 5 == 0 and len(v) > 4:
            v = np.concatenate([v[:len(v) // 2], h[:len(h) // 2], v[len(v) // 2:]])
        if aa:
            h, v = W.AA20_CODES[h], W.AA20_CODES[v]
            mt, mm, gap = 0, 0, -int(rng.integers(1, 12))
            letters = "ABCDEFGHIJKLMNOPQRSTUVWYZX*"
        else:
            mt, mm, gap = int(rng.integers(1, 4)), -int(rng.integers(1, 4)), -int(rng.integers(1, 5))
            letters = "ACGTN"
        cutoff = int(rng.integers(-1, 12))
        o = O.oracle_local_enumerate(h, v, mt, mm, gap, cutoff, matrix=b62 if aa else None, max_count=25,
                                     letters=letters)
        truncated = bool(o) and o[-1] is None
        if truncated:
            o = o[:-1]
        r = O.ref_local_enumerate(h, v, mt, mm, gap, cutoff, blosum62=aa, alphabet="aa" if aa else "dna",
                                  max_count=len(o) if truncated else 25)
        cases.append({"alphabet": "aa" if aa else "dna", "blosum62": aa, "match": mt, "mismatch": mm, "gap": gap,
                      "cutoff": cutoff, "H": text(h, "aa" if aa else "dna"), "V": text(v, "aa" if aa else "dna"),
                      "max_count": 25, "undefined_next": truncated,
                      "alignments": [[a.score, a.row0, a.row1, a.h_begin, a.h_end, a.v_begin, a.v_end] for a in r]})
    with open(os.path.join(HERE, "waterman_eggert_cases.json"), "w") as f:
        json.dump({"generator": "tests/golden/make_golden.py", "seed": 20261208, "cases": cases}, f,
                  separators=(",", ":"))
    print(f"{len(cases)} Waterman-Eggert cases written")


def write_waterman_eggert_banded(b62):
    """Suboptimal local alignments from the reference's LocalAlignmentEnumerator<Score, Banded>:
    random DNA and protein pairs with random bands [lowerDiag, upperDiag] that cross the matrix
    (lowerDiag < len(H), upperDiag > -len(V): the reference crashes on a band outside it), up to 25
    alignments each, cut where the oracle marks the reference's next step undefined."""
    from seqan_gb300 import workloads as W
    rng = np.random.Generator(np.random.PCG64(20261212))
    cases = []
    for trial in range(300):
        aa = trial % 4 == 3
        A = 20 if aa else 4
        m = int(rng.integers(1, 60))
        h = rng.integers(0, A, m).astype(np.uint8)
        if rng.random() < 0.6:
            v = W.mutate(rng, h, float(rng.uniform(0, 0.3)), float(rng.uniform(0, 0.08)), alphabet=A)
        else:
            v = rng.integers(0, A, int(rng.integers(1, 60))).astype(np.uint8)
        if len(v) == 0:
            v = rng.integers(0, A, 1).astype(np.uint8)
        lo = int(rng.integers(-len(v) + 1, len(h)))
        up = int(rng.integers(max(lo, -len(v) + 1), len(h) + 6))
        if trial % 7 == 0:
            lo, up = -len(v) - int(rng.integers(0, 5)), len(h) + int(rng.integers(0, 5))
        if aa:
            h, v = W.AA20_CODES[h], W.AA20_CODES[v]
            mt, mm, gap = 0, 0, -int(rng.integers(1, 12))
            letters = "ABCDEFGHIJKLMNOPQRSTUVWYZX*"
        else:
            mt, mm, gap = int(rng.integers(1, 4)), -int(rng.integers(1, 4)), -int(rng.integers(1, 5))
            letters = "ACGTN"
        cutoff = int(rng.integers(-1, 12))
        o = O.oracle_local_enumerate(h, v, mt, mm, gap, cutoff, matrix=b62 if aa else None, max_count=25,
                                     letters=letters, band=(lo, up))
        truncated = bool(o) and o[-1] is None
        if truncated:
            o = o[:-1]
        r = O.ref_local_enumerate(h, v, mt, mm, gap, cutoff, blosum62=aa, alphabet="aa" if aa else "dna",
                                  max_count=len(o) if truncated else 25, band=(lo, up))
        cases.append({"alphabet": "aa" if aa else "dna", "blosum62": aa, "match": mt, "mismatch": mm, "gap": gap,
                      "cutoff": cutoff, "band": [lo, up], "H": text(h, "aa" if aa else "dna"),
                      "V": text(v, "aa" if aa else "dna"), "max_count": 25, "undefined_next": truncated,
                      "alignments": [[a.score, a.row0, a.row1, a.h_begin, a.h_end, a.v_begin, a.v_end] for a in r]})
    with open(os.path.join(HERE, "waterman_eggert_banded_cases.json"), "w") as f:
        json.dump({"generator": "tests/golden/make_golden.py --only waterman_eggert_banded", "seed": 20261212,
                   "cases": cases}, f, separators=(",", ":"))
    print(f"{len(cases)} banded Waterman-Eggert cases written")


def write_raw_cases():
    """Raw texts through the reference's `while (!atEnd(iter)) readRecord(id, seq, qual, iter, Raw())`
    for the three alphabets: records (empty ids) or the ParseError."""
    rng = np.random.Generator(np.random.PCG64(20261214))
    letters = {"dna": b"ACGTacgt", "dna5": b"ACGTNacgtn", "aa": b"ACDEFGHIKLMNPQRSTVWYXacdefghik*"}
    ends = [b"\n", b"\r\n", b"\r"]
    cases = []
    fixed = [b"", b"\n", b"ACGT", b"ACGT\n", b"ACGT\n\n", b"\n\nAC\n", b"AC\rGT\r\nTT\n", b"A C\tG T\n",
             b">ACGT\n", b"AC>GT\n", b"AC\nG1T\n", b"acgtn\nNNNN", b"AC GT \r\n\r\nGG"]
    for alph in ("dna5", "dna", "aa"):
        for t in fixed:
            cases.append((alph, t))
        for _ in range(60):
            lines = []
            for _ in range(int(rng.integers(0, 8))):
                ln = bytes(letters[alph][int(x)] for x in rng.integers(0, len(letters[alph]), int(rng.integers(0, 40))))
                if rng.random() < 0.15:
                    i = int(rng.integers(0, len(ln) + 1))
                    ln = ln[:i] + bytes([b" \t"[int(rng.integers(0, 2))]]) + ln[i:]
                if rng.random() < 0.05:
                    i = int(rng.integers(0, len(ln) + 1))
                    ln = ln[:i] + bytes([b"#>1@"[int(rng.integers(0, 4))]]) + ln[i:]
                lines.append(ln + ends[int(rng.integers(0, 3))])
            t = b"".join(lines)
            if t and rng.random() < 0.3:
                t = t.rstrip(b"\r\n")
            cases.append((alph, t))
    out = []
    for alph, t in cases:
        try:
            recs = O.ref_read_records(t, "raw", alph)
            out.append({"alphabet": alph, "text": t.decode("latin1"), "error": None,
                        "records": [[r[0].decode("latin1"), r[1].tolist()] for r in recs]})
        except O.SeqParseError:
            out.append({"alphabet": alph, "text": t.decode("latin1"), "error": "parse", "records": None})
    with open(os.path.join(HERE, "seqio_raw_cases.json"), "w") as f:
        json.dump({"generator": "tests/golden/make_golden.py --only raw", "seed": 20261214, "cases": out}, f,
                  separators=(",", ":"))
    print(f"{len(out)} Raw texts written ({sum(c['error'] is not None for c in out)} with a ParseError)")


def chain_case(rng, max_len=200, max_seeds=8, max_seed_len=30):
    """A random pair with a random colinear seed chain (seeds need not match the sequences)."""
    m = int(rng.integers(5, max_len))
    h = rng.integers(0, 4, m).astype(np.uint8)
    v = []
    for x in h:
        r = rng.random()
        if r < 0.05:
            continue
        if r < 0.10:
            v.append(int(rng.integers(0, 4)))
        v.append(int(x) if rng.random() > 0.08 else int(rng.integers(0, 4)))
    v = np.array(v if v else [0], np.uint8)
    n = len(v)
    k = int(rng.integers(1, 16))
    ns = int(rng.integers(1, max_seeds + 1))
    seeds, ph, pv = [], 0, 0
    for _ in range(ns):
        if ph >= m - 2 or pv >= n - 2:
            break
        bh = int(rng.integers(ph, min(m - 1, ph + max(2, m // ns))))
        bv = int(rng.integers(pv, min(n - 1, pv + max(2, n // ns))))
        ln = int(rng.integers(1, 1 + max(1, min(m - bh, n - bv, max_seed_len))))
        eh = min(m, bh + ln + int(rng.integers(0, 3)))
        ev = min(n, bv + ln + int(rng.integers(0, 3)))
        if eh <= bh or ev <= bv:
            break
        seeds.append((bh, bv, eh, ev))
        ph, pv = eh, ev
    if not seeds:
        seeds = [(0, 0, 1, 1)]
    schemes = [(2, -1, -2, -2), (5, -3, -1, -5), (1, -1, -1, -1), (2, -3, -1, -4), (5, -3, -5, -5)]
    a = schemes[int(rng.integers(0, len(schemes)))]
    g = schemes[int(rng.integers(0, len(schemes)))] if rng.random() < 0.3 else a
    return h, v, seeds, a, g, int(rng.integers(0, 16)), k


def write_banded_chain():
    """bandedChainAlignment through the compiled reference: random pairs with random colinear
    chains (every AlignConfig, linear and affine schemes, separate anchor / gap schemes, band
    extensions 1..15, chains whose grids the reference cannot glue), and genomic pairs with the
    exact-match anchors of workloads.chain_pairs."""
    from seqan_gb300 import workloads as W
    rng = np.random.Generator(np.random.PCG64(20261210))
    cases = []

    def add(h, v, seeds, a, g, fe, k):
        r = O.ref_banded_chain(h, v, seeds, a, g, fe, k)
        cases.append({"H": text(h, "dna"), "V": text(v, "dna"), "seeds": [list(map(int, s)) for s in seeds],
                      "anchor": list(a), "gap": list(g), "free_ends": fe, "k": k, "status": r.status,
                      "score": r.score if r.status == 0 else None,
                      "segments": [list(s) for s in r.segments] if r.status == 0 else None,
                      "n_traces": r.n_traces if r.status == 0 else None,
                      "rows": list(r.rows) if r.status == 0 else None})

    for trial in range(360):
        add(*chain_case(rng, 60 if trial % 3 == 0 else 200, 12 if trial % 3 == 0 else 8,
                        8 if trial % 3 == 0 else 30))
    for trial in range(40):
        add(*chain_case(rng, 1200, 20, 120))
    H, V, chains = W.chain_pairs(40, 300, 900, min_seed=12, seed=77)
    for k in range(40):
        add(H[k], V[k], [tuple(s) for s in chains[k]], (2, -3, -1, -5), (2, -3, -1, -5), [0, 15, 5, 10][k % 4],
            [15, 5, 10, 3][k % 4])
    with open(os.path.join(HERE, "banded_chain_cases.json"), "w") as f:
        json.dump({"generator": "tests/golden/make_golden.py --only banded_chain", "seed": 20261210,
                   "cases": cases}, f, separators=(",", ":"))
    print(f"{len(cases)} banded chain cases written ({sum(c['status'] == 1 for c in cases)} where the reference "
          f"throws)")


def write_seeds(b62):
    seeds = seed_cases(b62)
    with open(os.path.join(HERE, "seed_cases.json"), "w") as f:
        json.dump({"generator": "tests/golden/make_golden.py", "seed": 20261204, "cases": seeds}, f,
                  separators=(",", ":"))
    print(f"{len(seeds)} seed cases written")


def seed_cases(b62):
    """Batches of seeds through the reference's extendSeed.  Gapped cases keep every substitution
    score >= the gap score: below that the reference adds a score to its `undefined` sentinel
    (INT_MIN - gap) and overflows int."""
    rng = np.random.Generator(np.random.PCG64(20261204))
    out = []

    def related(n, A, sub, indel):
        h = rng.integers(0, A, n).astype(np.uint8)
        v = h.copy()
        s = rng.random(n) < sub
        v[s] = (v[s] + rng.integers(1, A, int(s.sum()))) % A
        for _ in range(int(rng.poisson(indel * n))):
            if len(v) < 4:
                break
            a = int(rng.integers(0, len(v) - 2))
            v = np.delete(v, slice(a, a + int(rng.integers(1, 3)))) if rng.random() < 0.5 else \
                np.insert(v, a, rng.integers(0, A, int(rng.integers(1, 3))).astype(np.uint8))
        return h, v.astype(np.uint8)

    def add(sp, H, V, seeds, pos):
        alph = sp.alphabet
        s, xs = O.ref_extend_seeds(sp, H, V, seeds, pos, threads=4)
        out.append({"method": sp.method, "direction": sp.direction, "match": sp.match,
                    "mismatch": sp.mismatch, "gap": sp.gap, "xdrop": sp.xdrop,
                    "blosum62": sp.matrix is not None, "alphabet": alph,
                    "H": [text(h, alph) for h in H], "V": [text(v, alph) for v in V],
                    "pair_of_seed": None if pos is None else [int(x) for x in pos],
                    "seeds": O.seeds_array(seeds).tolist(), "extended": s.tolist(),
                    "xscores": xs.tolist() if sp.method == O.GAPPED_XDROP else None})

    def batch(sp, count, lo, hi, A, seeds_per_pair=1):
        H, V, seeds, pos = [], [], [], []
        for k in range(count):
            h, v = related(int(rng.integers(lo, hi + 1)), A, rng.uniform(0.0, 0.3), rng.uniform(0, 0.05))
            if rng.random() < 0.2:
                v = rng.integers(0, A, int(rng.integers(lo, hi + 1))).astype(np.uint8)
            if A == 20:
                h, v = AA_CODES[h], AA_CODES[v]
            H.append(h)
            V.append(v)
            m, n = len(h), len(v)
            for _ in range(seeds_per_pair):
                L = int(rng.integers(0, min(m, n, 24) + 1))
                bh = int(rng.integers(0, m - L + 1))
                # mostly on the pair's own diagonal (a true seed), sometimes anywhere
                bv = min(max(bh + int(rng.integers(-3, 4)), 0), n - L) if rng.random() < 0.7 else \
                    int(rng.integers(0, n - L + 1))
                if sp.method == O.UNGAPPED_XDROP and (sp.direction & 1) and bh > 0 and bv > 0 and \
                        (bh >= m or bv >= n):
                    continue   # the left walk scores database[beginH], past the end for such seeds
                seeds.append((bh, bv, L))
                pos.append(k)
        add(sp, H, V, seeds, pos)

    AA_CODES = np.array([0, 2, 3, 4, 5, 6, 7, 8, 10, 11, 12, 13, 15, 16, 17, 18, 19, 21, 22, 23], dtype=np.uint8)
    dna_scores = [(1, -1, -1), (2, -1, -1), (1, -2, -2), (2, -3, -5), (1, -5, -5), (1, -9, -9), (3, 0, -2)]
    for method in (O.MATCH_EXTEND, O.UNGAPPED_XDROP, O.GAPPED_XDROP):
        for direction in (O.EXTEND_LEFT, O.EXTEND_RIGHT, O.EXTEND_BOTH):
            for (mt, mm, g) in dna_scores:
                if method == O.GAPPED_XDROP and mm < g:
                    continue
                for xdrop in ((0, 1, 5, 20) if method else (0,)):
                    batch(O.SeedProblem(method, direction, mt, mm, g, xdrop), 6, 1, 90, 4, 2)
            if method:
                for (g, xdrop) in ((-9, 1), (-9, 10), (-11, 25), (-4, 8)):
                    batch(O.SeedProblem(method, direction, 0, 0, g, xdrop, b62, "aa"), 6, 1, 90, 20, 2)
    # Read-mapping shape: 150 bp reads against 250 bp windows, 19-mer seeds on the true diagonal.
    from seqan_gb300 import workloads as W
    wins, reads, seeds, pos = W.seed_windows(40, seed=5)
    for method in (O.UNGAPPED_XDROP, O.GAPPED_XDROP):
        add(O.SeedProblem(method, O.EXTEND_BOTH, 1, -2, -2, 20), wins, reads, seeds, pos)
    # Edges: seeds touching the sequence ends, empty seeds, one-letter sequences.
    H = [np.array([0], np.uint8), np.array([1, 2, 3], np.uint8), np.array([2, 2, 2, 2], np.uint8),
         np.zeros(0, np.uint8), np.array([3, 1], np.uint8)]
    V = [np.array([0], np.uint8), np.array([1, 2, 3], np.uint8), np.array([2, 2], np.uint8),
         np.array([1, 1], np.uint8), np.zeros(0, np.uint8)]
    seeds = [(0, 0, 1), (0, 0, 0), (1, 1, 0), (3, 3, 0), (0, 0, 3), (2, 0, 2), (4, 2, 0), (0, 0, 0), (0, 1, 0),
             (0, 0, 0), (2, 0, 0)]
    pos = [0, 0, 1, 1, 1, 2, 2, 2, 3, 4, 4]
    for direction in (O.EXTEND_LEFT, O.EXTEND_RIGHT, O.EXTEND_BOTH):
        add(O.SeedProblem(O.GAPPED_XDROP, direction, 1, -1, -1, 3), H, V, seeds, pos)
        add(O.SeedProblem(O.MATCH_EXTEND, direction), H, V, seeds, pos)
    return out



# FASTA / FASTQ: the reference's readRecord loop (oracle/ref/units/seqio.cpp) on the reference's own
# seq_io test files, hand-made edge cases and seeded random texts.
SEQIO_LETTERS = {"dna5": "ACGTNacgtn", "dna": "ACGTacgt", "aa": "ACDEFGHIKLMNPQRSTVWYXBZJOU*acdx"}
SEQIO_EDGE = [
    ("fasta", b""), ("fasta", b"  \n"), ("fasta", b">"), ("fasta", b">id only"), ("fasta", b">a\r\nAC GT\n\nNN>b c>d\rAC\n"),
    ("fasta", b"junk XX\n>x\nACGT\n"), ("fasta", b">x\nAC\n>y\n"), ("fasta", b">x\nACGU\n"), ("fasta", b">x\nac\tgt\r\n"),
    ("fasta", b">x y\n\n\nACGT\n\n>z\n\n"), ("fasta", b">>>\n>\n>"), ("fasta", b"\xff>x\nA\xffC\n"),
    ("fastq", b""), ("fastq", b"@r1\nACGT\n+\nIIII\n@r2\nAC\nGT\n+r2\nII\nI@\n"), ("fastq", b"@r\nACGT\n+\nII\n"),
    ("fastq", b"@r\nAC\n+\nI I\n"), ("fastq", b"@r\nAC\n+\nII\n\n  @s\n\n+\n"), ("fastq", b"@r\nAC\n+\nIIX\n"),
    ("fastq", b"@r\nAC"), ("fastq", b"@r\nAC\n+"), ("fastq", b"  "), ("fastq", b"@r\r\nAC\r\n+\r\n@@\r\n"),
    ("fastq", b"@r\nA>C\n+\nII\n"), ("fastq", b"@r\nAC\n+\nII\xff"), ("fastq", b"x@r\n\n+\n@s\nA\n+\n+\n"),
]


def seqio_random_text(rng, fmt, alphabet):
    letters = SEQIO_LETTERS[alphabet]
    pick = lambda s: s[int(rng.integers(len(s)))]
    parts = []
    for _ in range(int(rng.integers(0, 6))):
        if fmt == "fasta":
            parts.append(">" + "".join(pick("ab >\t") for _ in range(int(rng.integers(0, 7)))) +
                         pick(["\n", "\r\n", "\r", ""]))
            out = []
            for _ in range(int(rng.integers(0, 40))):
                out.append(pick(letters))
                if rng.random() < 0.15:
                    out.append(pick(["\n", "\r\n", " ", "\t"]))
            parts.append("".join(out))
        else:
            parts.append("@" + "".join(pick("ab @+") for _ in range(int(rng.integers(0, 5)))) + pick(["\n", "\r\n"]))
            L = int(rng.integers(0, 20))
            seq = "".join(pick(letters) for _ in range(L))
            parts.append(seq + pick(["\n", "\r\n"]) + "+" + pick(["", "x"]) + "\n")
            q = "".join(pick("I#@+ !") for _ in range(max(0, L + pick([0, 0, 0, 1, -1]))))
            parts.append(q + pick(["\n", "\n\n", "\r\n", ""]))
    t = "".join(parts)
    if rng.random() < 0.2 and t:
        i = int(rng.integers(len(t)))
        t = t[:i] + pick(" \t\r\n>@+X-1\xff") + t[i:]
    return t.encode("latin1")


def write_seqio():
    import base64
    rng = np.random.Generator(np.random.PCG64(20261208))
    texts = []
    for name, fmt in (("test_dna.fa", "fasta"), ("test_dna.fq", "fastq"), ("adeno_genome.fa", "fasta")):
        with open(os.path.join(REFERENCE, "tests", "seq_io", name), "rb") as f:
            data = f.read()
        for alph in ("dna5", "dna", "aa"):
            texts.append((f"tests/seq_io/{name}", fmt, alph, data))
    for k, (fmt, t) in enumerate(SEQIO_EDGE):
        for alph in ("dna5", "dna", "aa"):
            texts.append((f"edge {k}", fmt, alph, t))
    for k in range(360):
        fmt = ("fasta", "fastq")[k % 2]
        alph = ("dna5", "dna", "aa")[(k // 2) % 3]
        texts.append((f"random {k}", fmt, alph, seqio_random_text(rng, fmt, alph)))
    cases = []
    for src, fmt, alph, t in texts:
        case = {"source": src, "format": fmt, "alphabet": alph, "text": base64.b64encode(t).decode()}
        try:
            recs = O.ref_read_records(t, fmt, alph)
            case["records"] = [[i.decode("latin1"), c.tolist(), q.decode("latin1")] for i, c, q in recs]
        except O.SeqParseError as e:
            case["error"] = e.kind
        cases.append(case)
    tables = {a: O.ref_char_table(a).tolist() for a in ("dna5", "dna", "aa")}
    with open(os.path.join(HERE, "seqio_cases.json"), "w") as f:
        json.dump({"generator": "tests/golden/make_golden.py --only seqio", "seed": 20261208, "char_tables": tables,
                   "cases": cases}, f, separators=(",", ":"))
    print(f"{len(cases)} FASTA/FASTQ cases written ({sum('error' in c for c in cases)} errors)")



def bam_records(rng):
    """SAM fixture records plus the BAM writer's own cases: unmapped records at position -1,
    positions on every bin level, qualities shorter than the sequence, odd lengths, every CIGAR
    operation, and Iupac letters (lower case, 'U', characters outside the alphabet)."""
    rec = sam_records(rng, 400)
    n = len(rec.qname)
    pos = rec.pos.copy()
    edges = [-1, 0, 1, (1 << 14) - 1, 1 << 14, (1 << 17) - 3, 1 << 20, (1 << 23) + 5, (1 << 26) - 2, (1 << 29) - 7,
             2_000_000_000]
    for j, e in enumerate(edges):
        pos[j * 7] = e
    quals = list(rec.qual)
    for k in range(0, n, 9):
        quals[k] = quals[k][:len(rec.seq[k]) // 2]
    cig = list(rec.cigar)
    for k in range(3, n, 17):
        cig[k] = [(int(rng.integers(1, 50)) << 4) | op for op in range(9)]
    rec.pos, rec.qual, rec.cigar = pos, quals, cig
    rec2 = sam_records(rng, 120)
    rec2.letters = "=ACMGRSVTWYHKDBNacgtuUX*n-"
    rec2.seq = [rng.integers(0, len(rec2.letters), len(s)).astype(np.uint8) for s in rec2.seq]
    return rec, rec2


def write_bam_cases():
    import base64
    rng = np.random.Generator(np.random.PCG64(20261209))
    cases = []
    for rec in bam_records(rng):
        data = O.ref_write_bam(rec)
        cases.append({"contigs": rec.contigs, "letters": rec.letters, "qname": rec.qname, "flag": rec.flag.tolist(),
                      "ref_id": rec.ref_id.tolist(), "pos": rec.pos.tolist(), "mapq": rec.mapq.tolist(),
                      "cigar": [list(map(int, c)) for c in rec.cigar], "next_ref_id": rec.next_ref_id.tolist(),
                      "next_pos": rec.next_pos.tolist(), "tlen": rec.tlen.tolist(),
                      "seq": [s.tolist() for s in rec.seq], "qual": rec.qual,
                      "bam": base64.b64encode(data).decode()})
    with open(os.path.join(HERE, "bam_cases.json"), "w") as f:
        json.dump({"generator": "tests/golden/make_golden.py --only bam", "seed": 20261209,
                   "iupac": O.ref_iupac_table().tolist(), "cases": cases}, f, separators=(",", ":"))
    print(f"{sum(len(c['qname']) for c in cases)} BAM records written")


def write_dynamic_cases(b62):
    """Seeded pairs through the reference's DP with DynamicGaps cells, for every instantiated shape."""
    rng = np.random.Generator(np.random.PCG64(20261205))
    shapes = [("global", fe, 32, "dna") for fe in (0, 15, 9, 6)] + [("local", 0, 32, "dna"), ("global", 0, 16, "dna"),
                                                                   ("local", 0, 16, "dna"), ("local", 0, 16, "aa"),
                                                                   ("global", 0, 16, "aa")]
    schemes = [(2, -3, -5, -5), (2, -4, -6, -1), (4, -2, -10, -4), (1, -1, -2, -2), (3, -2, -4, -1), (2, -3, -1, -7)]
    cases = []
    for mode, fe, bits, alph in shapes:
        for sc in schemes if alph == "dna" else [(0, 0, -11, -1), (0, 0, -8, -2)]:
            mt, mm, go, ge = sc
            mat = b62 if alph == "aa" else None
            pb = O.Problem(mode, fe, None, mt, mm, go, ge, mat, bits, alph, dynamic=True)
            H, V = rand_pairs(rng, 25, 1, 70, alph)
            out = []
            for h, v in zip(H, V):
                score, segs = O.ref_dynamic_segments(pb, h, v)
                out.append({"score": score, "segments": [list(x) for x in segs]})
            cases.append({"problem": problem_dict(pb), "H": [text(h, alph) for h in H], "V": [text(v, alph) for v in V],
                          "results": out})
    with open(os.path.join(HERE, "dynamic_cases.json"), "w") as f:
        json.dump({"generator": "tests/golden/make_golden.py --only dynamic", "seed": 20261205, "cases": cases}, f,
                  separators=(",", ":"))
    print(f"{sum(len(c['results']) for c in cases)} DynamicGaps pairs written")


def write_cpp_binding():
    """Builds tests/cpp/seqan_binding.cpp against the reference's headers with -DGBA_AS_REFERENCE
    (every call run by the reference) and records its output."""
    import tempfile
    with tempfile.TemporaryDirectory() as tmp:
        exe = os.path.join(tmp, "binding_ref")
        subprocess.check_call(["g++", "-std=c++17", "-O1", "-fopenmp", "-w", "-DGBA_AS_REFERENCE",
                               "-I", os.path.join(REFERENCE, "include"), "-I", os.path.join(ROOT, "include"),
                               os.path.join(ROOT, "tests", "cpp", "seqan_binding.cpp"), "-o", exe])
        out = subprocess.run([exe], check=True, capture_output=True).stdout
    with open(os.path.join(HERE, "cpp_binding_expected.txt"), "wb") as f:
        f.write(out)
    print(f"{out.count(b'\n')} lines of reference output written")


if __name__ == "__main__":
    main()
