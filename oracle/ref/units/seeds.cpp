// Seed extension through the UNMODIFIED reference (test infrastructure, see ref_common.h).
// Calls extendSeed(Seed<Simple>, database, query, direction, ...) with MatchExtend,
// UnGappedXDrop and GappedXDrop (seeds/seeds_extension.h:181-218, 283-360, 780-835) over a
// batch of seeds, and the one-direction gapped routine (:613-775) on copies of the seeds for
// the scores that extendSeed itself discards.
#include "../ref_common.h"

#include <seqan/seeds.h>

namespace seqan_ref {
namespace {

template <typename TAlph, typename TScore>
int extend_all(int32_t method, int32_t direction, TScore const & sc, int32_t xdrop, int64_t n_seeds,
               StringSet<String<TAlph>> const & setH, StringSet<String<TAlph>> const & setV,
               const int32_t * pair_of_seed, int64_t * seeds, int32_t * xscores, int32_t threads)
{
    typedef Seed<Simple> TSeed;
#pragma omp parallel for schedule(dynamic, 64) num_threads(threads > 0 ? threads : 1)
    for (int64_t i = 0; i < n_seeds; ++i)
    {
        const int64_t k = pair_of_seed ? pair_of_seed[i] : i;
        String<TAlph> const & db = setH[k];
        String<TAlph> const & q = setV[k];
        int64_t * s = seeds + 6 * i;
        TSeed seed(s[0], s[1], s[2], s[3]);
        setLowerDiagonal(seed, s[4]);
        setUpperDiagonal(seed, s[5]);
        const TSeed before = seed;
        const ExtensionDirection dir = static_cast<ExtensionDirection>(direction);
        if (method == 0)
            extendSeed(seed, db, q, dir, MatchExtend());
        else if (method == 1)
            extendSeed(seed, db, q, dir, sc, (int)xdrop, UnGappedXDrop());
        else
        {
            extendSeed(seed, db, q, dir, sc, (int)xdrop, GappedXDrop());
            if (xscores)
            {
                TSeed tmp = before;
                xscores[2 * i] = 0;
                xscores[2 * i + 1] = 0;
                if (direction & 1)
                    xscores[2 * i] = _extendSeedGappedXDropOneDirection(
                        tmp, prefix(q, beginPositionV(before)), prefix(db, beginPositionH(before)), EXTEND_LEFT,
                        sc, (int)xdrop);
                if (direction & 2)
                    xscores[2 * i + 1] = _extendSeedGappedXDropOneDirection(
                        tmp, suffix(q, endPositionV(before)), suffix(db, endPositionH(before)), EXTEND_RIGHT,
                        sc, (int)xdrop);
            }
        }
        s[0] = beginPositionH(seed);
        s[1] = beginPositionV(seed);
        s[2] = endPositionH(seed);
        s[3] = endPositionV(seed);
        s[4] = lowerDiagonal(seed);
        s[5] = upperDiagonal(seed);
    }
    return 0;
}

template <typename TAlph>
int extend_alph(int32_t method, int32_t direction, int32_t blosum62, int32_t match, int32_t mismatch, int32_t gap,
                int32_t xdrop, int64_t n_pairs, const uint8_t * sh, const int64_t * oh, const uint8_t * sv,
                const int64_t * ov, int64_t n_seeds, const int32_t * pair_of_seed, int64_t * seeds,
                int32_t * xscores, int32_t threads)
{
    StringSet<String<TAlph>> setH, setV;
    build_set(setH, n_pairs, sh, oh);
    build_set(setV, n_pairs, sv, ov);
    if (blosum62)
    {
        Score<int, ScoreMatrix<AminoAcid, ScoreSpecBlosum62>> sc(gap, gap);
        return extend_all(method, direction, sc, xdrop, n_seeds, setH, setV, pair_of_seed, seeds, xscores, threads);
    }
    Score<int, Simple> sc(match, mismatch, gap);
    return extend_all(method, direction, sc, xdrop, n_seeds, setH, setV, pair_of_seed, seeds, xscores, threads);
}

}  // namespace
}  // namespace seqan_ref

extern "C" {

// seeds: 6 int64 per seed (beginH, beginV, endH, endV, lowerDiagonal, upperDiagonal), extended in
// place.  pair_of_seed: the (H, V) pair each seed lies on (NULL: seed i on pair i).  xscores:
// optional 2 per seed, the gapped left/right extension scores.  alphabet 0 = Dna5, 1 = AminoAcid.
int ref_extend_seeds(int32_t method, int32_t direction, int32_t alphabet, int32_t blosum62, int32_t match,
                     int32_t mismatch, int32_t gap, int32_t xdrop, int64_t n_pairs, const uint8_t * sh,
                     const int64_t * oh, const uint8_t * sv, const int64_t * ov, int64_t n_seeds,
                     const int32_t * pair_of_seed, int64_t * seeds, int32_t * xscores, int32_t threads)
{
    if (alphabet == 1)
        return seqan_ref::extend_alph<AminoAcid>(method, direction, blosum62, match, mismatch, gap, xdrop, n_pairs,
                                                 sh, oh, sv, ov, n_seeds, pair_of_seed, seeds, xscores, threads);
    return seqan_ref::extend_alph<Dna5>(method, direction, blosum62, match, mismatch, gap, xdrop, n_pairs, sh, oh, sv,
                                        ov, n_seeds, pair_of_seed, seeds, xscores, threads);
}

}  // extern "C"
