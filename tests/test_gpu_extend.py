"""extendAlignment on the GPU through gba_extend_alignments: identical to the reference's
extendAlignment (fixtures, known answers) and to the oracle on seeded batches -- read seeds,
queries taller than one 256-row band, long databases cut short by the X-drop terminator, Blosum62,
linear and affine gaps."""
import numpy as np
import pytest

from oracle import oracle as O
from tests import golden_cases as G
from tests.test_extend_oracle import BANDED_CASES, EXTEND_CASES, KNOWN, banded_problem, extend_problem

pytestmark = pytest.mark.gpu

AA = "ABCDEFGHIJKLMNOPQRSTUVWYZX*"


def engine_score(pb):
    import seqan_gb300 as sg
    if pb.matrix is not None:
        return sg.Blosum62(pb.gap_extend, pb.gap_open)
    return sg.Score(pb.match, pb.mismatch, pb.gap_extend, pb.gap_open)


def check_batch(pb, H, V, positions, direction, letters="ACGTN", alphabet="dna5", seed_h=None):
    from seqan_gb300 import align_extend as X
    exts = X.extend_alignments(H, V, positions, direction, engine_score(pb), pb.xdrop, seed_h=seed_h,
                               alphabet=alphabet, band=pb.band)
    for k, ext in enumerate(exts):
        h = H[seed_h[k]] if seed_h is not None else H[k]
        got = X.assemble(ext, h, V[k], positions[k], engine_score(pb), alphabet)
        ref = O.oracle_extend_alignment(pb, h, V[k], positions[k], direction, letters=letters)
        assert (got.score, got.row0, got.row1, got.h_begin, got.h_end, got.v_begin, got.v_end) == \
            (ref.score, ref.row0, ref.row1, ref.h_begin, ref.h_end, ref.v_begin, ref.v_end), k
        assert ext.left_segments == ref.left_segments and ext.right_segments == ref.right_segments, k
    return exts


@pytest.mark.parametrize("chunk", range(0, len(EXTEND_CASES), 110))
def test_fixtures_through_c_abi(engine, chunk):
    from seqan_gb300 import align_extend as X
    for c in EXTEND_CASES[chunk:chunk + 110]:
        pb = extend_problem(c)
        alph = "aa" if c["alphabet"] == "aa" else "dna5"
        got = X.extendAlignment(c["H"], c["V"], c["positions"], c["direction"],
                                *(() if c["xdrop"] is None else (c["xdrop"],)), engine_score(pb), alphabet=alph)
        assert (got.score, got.row0, got.row1, [got.h_begin, got.h_end, got.v_begin, got.v_end]) == \
            (c["score"], c["row0"], c["row1"], c["ends"]), c


@pytest.mark.parametrize("case", KNOWN, ids=["no_gaps", "gaps_in_extensions"])
def test_known_answers(engine, case):
    import seqan_gb300 as sg
    from seqan_gb300 import align_extend as X
    h, v, pos, row0, row1, clips, score = case
    got = X.extendAlignment(h, v, pos, X.EXTEND_BOTH, sg.Score(2, -1, -2))
    assert (got.row0, got.row1, got.score) == (row0, row1, score)
    assert (got.h_begin, got.h_begin + len(got.row0), got.v_begin, got.v_begin + len(got.row1)) == clips


@pytest.mark.parametrize("gaps", [(-2, -2), (-5, -1)])
@pytest.mark.parametrize("xdrop", [None, 20, 3])
def test_read_seeds_batch(engine, gaps, xdrop):
    """3,000 read seeds (150 bp reads in 250 bp windows), both sides extended."""
    from seqan_gb300 import workloads as W
    wins, reads, seeds, _ = W.seed_windows(3000, ref_len=1_000_000, seed=31)
    pos = [(int(s[0]), int(s[1]), int(s[0] + s[2]), int(s[1] + s[2])) for s in seeds]
    pb = O.Problem("extend", 0, None, 1, -2, gaps[0], gaps[1], None, 32, "dna", xdrop)
    check_batch(pb, wins, reads, pos, O.EXTEND_BOTH)


def test_tall_queries_use_several_bands(engine):
    """Queries of 300-900 residues: the left / right sides have more than 256 rows."""
    from seqan_gb300 import workloads as W
    rng = np.random.default_rng(17)
    H, V, pos = [], [], []
    for k in range(300):
        L = int(rng.integers(300, 900))
        h = rng.integers(0, 4, L).astype(np.uint8)
        v = W.mutate(rng, h, 0.08, 0.02)
        sl = 12
        hb = int(rng.integers(0, min(len(h), len(v)) - sl))
        H.append(h)
        V.append(v)
        pos.append((hb, hb, hb + sl, hb + sl))
    for xdrop in (None, 15):
        pb = O.Problem("extend", 0, None, 2, -3, -5, -2, None, 32, "dna", xdrop)
        check_batch(pb, H, V, pos, O.EXTEND_BOTH)


def test_narrow_groups_with_tall_minority(engine):
    """70 bp reads (task heights <= 64: eight lanes per task) plus 5% reads of 300 bp whose sides
    span several 64-row bands."""
    from seqan_gb300 import workloads as W
    rng = np.random.default_rng(29)
    H, V, pos = [], [], []
    for k in range(1500):
        L = 300 if k % 20 == 0 else 70
        o = int(rng.integers(0, 40))
        win = rng.integers(0, 4, L + 80).astype(np.uint8)
        read = W.mutate(rng, win[o + 10:o + 10 + L], 0.04, 0.01)
        sl = min(11, len(read) - 1)
        s0 = int(rng.integers(0, len(read) - sl))
        H.append(win)
        V.append(read)
        pos.append((o + 10 + s0, s0, o + 10 + s0 + sl, s0 + sl))
    for xdrop in (None, 12):
        pb = O.Problem("extend", 0, None, 2, -3, -5, -1, None, 32, "dna", xdrop)
        check_batch(pb, H, V, pos, O.EXTEND_BOTH)


def test_long_database_cut_short_by_xdrop(engine):
    """Reads seeded inside a 200 kbp database shared by all alignments: the extension over the
    database prefix / suffix stops where the X-drop terminator stops the reference."""
    from seqan_gb300 import workloads as W
    rng = np.random.default_rng(23)
    genome = rng.integers(0, 4, 200_000).astype(np.uint8)
    origins = rng.integers(1000, len(genome) - 1200, 400)
    reads = [W.mutate(rng, genome[o:o + 150], 0.03, 0.003) for o in origins]
    pos = [(int(o) + 60, 60, int(o) + 75, 75) for o in origins]
    pb = O.Problem("extend", 0, None, 1, -2, -4, -1, None, 32, "dna", 10)
    exts = check_batch(pb, [genome], reads, pos, O.EXTEND_BOTH, seed_h=np.zeros(len(pos), np.int32))
    assert all(sum(s[2] for s in e.left_segments) < 1000 for e in exts)


def test_protein_blosum62(engine):
    from seqan_gb300 import workloads as W
    B62 = np.array(G.load("blosum62.json")["matrix"], dtype=np.int32)
    H, V = W.protein_pairs(400, seed=41, related=0.9, identity=0.6)
    pos = []
    for h, v in zip(H, V):
        L = min(len(h), len(v))
        b = L // 3
        pos.append((b, b, b + 4, b + 4))
    for go, ge, xd in ((-11, -1, None), (-11, -1, 25), (-9, -9, 12)):
        pb = O.Problem("extend", 0, None, 0, 0, go, ge, B62, 32, "aa", xd)
        check_batch(pb, H, V, pos, O.EXTEND_BOTH, letters=AA, alphabet="aa")


def test_refusals(engine):
    import seqan_gb300 as sg
    from seqan_gb300 import _native as N
    from seqan_gb300 import align_extend as X
    with pytest.raises(N.GbaError) as e:
        X.extend_alignments(["ACGT"], ["ACGT"], [(2, 2, 5, 5)], X.EXTEND_BOTH, sg.Score(1, -1, -1))
    assert e.value.status == N.GBA_EINVAL
    out = X.extendAlignment("ACGTACGT", "ACGTACGT", (3, 3, 5, 5), X.EXTEND_BOTH, sg.Score(1, -1, -1))
    assert (out.score, out.row0, out.h_begin, out.h_end) == (8, "ACGTACGT", 0, 8)


# --- The other overloads: (lowerDiag, upperDiag), origScore, aligned parts with gaps -----------

@pytest.mark.parametrize("chunk", range(0, len(BANDED_CASES), 140))
def test_banded_origscore_gapped_fixtures_through_c_abi(engine, chunk):
    """The reference's extendAlignment overloads with (lowerDiag, upperDiag) [and xDrop], with
    origScore and with gapped aligned parts: one gba_extend_alignments call per case (the banded
    kernel in its AlignExtend_ mode, GBA_ALIGN_EXTEND)."""
    from seqan_gb300 import align_extend as X
    for c in BANDED_CASES[chunk:chunk + 140]:
        pb = banded_problem(c)
        alph = "aa" if c["alphabet"] == "aa" else "dna5"
        args = tuple(c["band"]) + (() if c["xdrop"] is None else (c["xdrop"],)) + (engine_score(pb),)
        got = X.extendAlignment(c["H"], c["V"], c["positions"], c["direction"], *args, alphabet=alph,
                                orig_score=c["orig_score"],
                                center=None if c["center"] is None else tuple(c["center"]))
        assert (got.score, got.row0, got.row1, [got.h_begin, got.h_end, got.v_begin, got.v_end]) == \
            (c["score"], c["row0"], c["row1"], c["ends"]), c


@pytest.mark.parametrize("band", [(-10, 10), (-3, 3), (0, 0), (-30, 5), (-200, 200)])
@pytest.mark.parametrize("xdrop", [None, 8])
def test_banded_read_seeds_batch(engine, band, xdrop):
    """3,000 read seeds in 250 bp windows, both sides extended inside a band, vs the oracle."""
    from seqan_gb300 import workloads as W
    wins, reads, seeds, _ = W.seed_windows(3000, ref_len=1_000_000, seed=37)
    pos = [(int(s[0]), int(s[1]), int(s[0] + s[2]), int(s[1] + s[2])) for s in seeds]
    pb = O.Problem("extend", 0, band, 1, -2, -4, -1, None, 32, "dna", xdrop)
    check_batch(pb, wins, reads, pos, O.EXTEND_BOTH)
    assert _kernels() & _flags().GBA_KERNEL_BANDED


def test_banded_protein_and_invalid_bands(engine):
    """Blosum62 sides in a band, and a band that misses the sides' matrices (lowerDiag > 0): the
    side scores are the reference's invalid value and no segments."""
    from seqan_gb300 import align_extend as X
    from seqan_gb300 import workloads as W
    B62 = np.array(G.load("blosum62.json")["matrix"], dtype=np.int32)
    H, V = W.protein_pairs(300, seed=43, related=0.9, identity=0.6)
    pos = []
    for h, v in zip(H, V):
        b = min(len(h), len(v)) // 3
        pos.append((b, b, b + 4, b + 4))
    for band, xd in (((-15, 15), None), ((-15, 15), 25), ((-2, 6), 12)):
        pb = O.Problem("extend", 0, band, 0, 0, -11, -1, B62, 32, "aa", xd)
        check_batch(pb, H, V, pos, O.EXTEND_BOTH, letters=AA, alphabet="aa")
    exts = X.extend_alignments(H[:5], V[:5], pos[:5], X.EXTEND_BOTH, engine_score(
        O.Problem("extend", 0, None, 0, 0, -11, -1, B62, 32, "aa")), band=(1, 4), alphabet="aa")
    for e in exts:
        assert e.left_score == e.right_score == -2 ** 31
        assert e.left_segments == [] and e.right_segments == []


def _flags():
    from seqan_gb300 import _native as N
    return N


def _kernels():
    import seqan_gb300 as sg
    return sg.default_context().stats().dp_kernels
