// Waterman-Eggert suboptimal local alignments through the UNMODIFIED reference (test
// infrastructure, see ref_common.h): LocalAlignmentEnumerator<Score, Unbanded> with
// nextLocalAlignment / getScore (align/local_alignment_enumeration_unbanded.h).
#include "../ref_common.h"

#include <seqan/align.h>

#include <sstream>
#include <string>
#include <vector>

#include <omp.h>

namespace seqan_ref {
namespace {

template <typename TAlph, typename TEnumerator>
int enumerate_with(TEnumerator & enumerator, const uint8_t * h, int64_t m, const uint8_t * v, int64_t n,
                   int32_t max_count, int32_t * scores, int32_t * pos, char * out_rows, int64_t cap);

template <typename TAlph, typename TScore>
int enumerate(TScore const & sc, int32_t cutoff, const uint8_t * h, int64_t m, const uint8_t * v, int64_t n,
              int32_t max_count, int32_t * scores, int32_t * pos, char * out_rows, int64_t cap)
{
    LocalAlignmentEnumerator<TScore, Unbanded> enumerator(sc, cutoff);
    return enumerate_with<TAlph>(enumerator, h, m, v, n, max_count, scores, pos, out_rows, cap);
}

template <typename TAlph, typename TEnumerator>
int enumerate_with(TEnumerator & enumerator, const uint8_t * h, int64_t m, const uint8_t * v, int64_t n,
                   int32_t max_count, int32_t * scores, int32_t * pos, char * out_rows, int64_t cap)
{
    typedef String<TAlph> TStr;
    TStr hs, vs;
    resize(hs, m);
    resize(vs, n);
    for (int64_t i = 0; i < m; ++i) assignValue(hs, i, TAlph(unsigned(h[i])));
    for (int64_t i = 0; i < n; ++i) assignValue(vs, i, TAlph(unsigned(v[i])));
    Align<TStr> align;
    resize(rows(align), 2);
    assignSource(row(align, 0), hs);
    assignSource(row(align, 1), vs);
    std::string text;
    int32_t k = 0;
    for (; k < max_count && nextLocalAlignment(align, enumerator); ++k)
    {
        scores[k] = getScore(enumerator);
        pos[4 * k + 0] = int32_t(beginPosition(row(align, 0)));
        pos[4 * k + 1] = int32_t(endPosition(row(align, 0)));
        pos[4 * k + 2] = int32_t(beginPosition(row(align, 1)));
        pos[4 * k + 3] = int32_t(endPosition(row(align, 1)));
        std::stringstream s0, s1;
        s0 << row(align, 0);
        s1 << row(align, 1);
        text += s0.str() + "\n" + s1.str() + "\n";
    }
    if (int64_t(text.size()) + 1 > cap) return -1;
    std::memcpy(out_rows, text.c_str(), text.size() + 1);
    return k;
}

}  // namespace
}  // namespace seqan_ref

extern "C" {

// Up to max_count alignments: scores, pos = (H begin, H end, V begin, V end) source positions of
// the clipped rows, rows = the two rows of each alignment as text lines.  Returns the count.
int ref_local_enumerate(int32_t alphabet, int32_t blosum62, int32_t match, int32_t mismatch, int32_t gap_extend,
                        int32_t gap_open, int32_t cutoff, const uint8_t * h, int64_t m, const uint8_t * v, int64_t n,
                        int32_t max_count, int32_t * scores, int32_t * pos, char * out_rows, int64_t cap)
{
    if (alphabet == 1)
    {
        if (blosum62)
        {
            Score<int, ScoreMatrix<AminoAcid, ScoreSpecBlosum62>> sc(gap_extend, gap_open);
            return seqan_ref::enumerate<AminoAcid>(sc, cutoff, h, m, v, n, max_count, scores, pos, out_rows, cap);
        }
        Score<int, Simple> sc(match, mismatch, gap_extend, gap_open);
        return seqan_ref::enumerate<AminoAcid>(sc, cutoff, h, m, v, n, max_count, scores, pos, out_rows, cap);
    }
    Score<int, Simple> sc(match, mismatch, gap_extend, gap_open);
    return seqan_ref::enumerate<Dna5>(sc, cutoff, h, m, v, n, max_count, scores, pos, out_rows, cap);
}

// The banded enumerator LocalAlignmentEnumerator<Score, Banded>(score, lowerDiag, upperDiag, cutoff)
// (align/local_alignment_enumeration_banded.h), outputs as ref_local_enumerate.
int ref_local_enumerate_banded(int32_t alphabet, int32_t blosum62, int32_t match, int32_t mismatch, int32_t gap,
                               int32_t lower, int32_t upper, int32_t cutoff, const uint8_t * h, int64_t m,
                               const uint8_t * v, int64_t n, int32_t max_count, int32_t * scores, int32_t * pos,
                               char * out_rows, int64_t cap)
{
    if (alphabet == 1 && blosum62)
    {
        typedef Score<int, ScoreMatrix<AminoAcid, ScoreSpecBlosum62>> TSc;
        LocalAlignmentEnumerator<TSc, Banded> e(TSc(gap, gap), lower, upper, cutoff);
        return seqan_ref::enumerate_with<AminoAcid>(e, h, m, v, n, max_count, scores, pos, out_rows, cap);
    }
    Score<int, Simple> sc(match, mismatch, gap, gap);
    LocalAlignmentEnumerator<Score<int, Simple>, Banded> e(sc, lower, upper, cutoff);
    if (alphabet == 1)
        return seqan_ref::enumerate_with<AminoAcid>(e, h, m, v, n, max_count, scores, pos, out_rows, cap);
    return seqan_ref::enumerate_with<Dna5>(e, h, m, v, n, max_count, scores, pos, out_rows, cap);
}

// A batch of pairs (codes concatenated with offsets) on `threads` OpenMP threads (<= 0: all):
// the enumeration of every pair as above; count[k] = the alignments pair k gave.
int ref_local_enumerate_batch(int32_t match, int32_t mismatch, int32_t gap, int32_t cutoff, int64_t n_pairs,
                              const uint8_t * seq_h, const int64_t * off_h, const uint8_t * seq_v,
                              const int64_t * off_v, int32_t max_count, int32_t * count, int32_t threads)
{
    const int nt = threads > 0 ? threads : omp_get_max_threads();
    Score<int, Simple> sc(match, mismatch, gap, gap);
#pragma omp parallel num_threads(nt)
    {
        std::vector<int32_t> scores(size_t(max_count > 0 ? max_count : 1)), pos(size_t(4 * (max_count > 0 ? max_count : 1)));
        std::vector<char> rows;
#pragma omp for schedule(dynamic, 8)
        for (int64_t k = 0; k < n_pairs; ++k)
        {
            const int64_t m = off_h[k + 1] - off_h[k], n = off_v[k + 1] - off_v[k];
            rows.resize(size_t(max_count) * size_t(2 * (m + n + 2)) + 8);
            count[k] = seqan_ref::enumerate<Dna5>(sc, cutoff, seq_h + off_h[k], m, seq_v + off_v[k], n, max_count,
                                                  scores.data(), pos.data(), rows.data(), int64_t(rows.size()));
        }
    }
    return 0;
}

// The same batch through LocalAlignmentEnumerator<Score, Banded>(sc, lower, upper, cutoff).
int ref_local_enumerate_banded_batch(int32_t match, int32_t mismatch, int32_t gap, int32_t lower, int32_t upper,
                                     int32_t cutoff, int64_t n_pairs, const uint8_t * seq_h, const int64_t * off_h,
                                     const uint8_t * seq_v, const int64_t * off_v, int32_t max_count, int32_t * count,
                                     int32_t threads)
{
    const int nt = threads > 0 ? threads : omp_get_max_threads();
#pragma omp parallel num_threads(nt)
    {
        std::vector<int32_t> scores(size_t(max_count > 0 ? max_count : 1)), pos(size_t(4 * (max_count > 0 ? max_count : 1)));
        std::vector<char> rows;
#pragma omp for schedule(dynamic, 8)
        for (int64_t k = 0; k < n_pairs; ++k)
        {
            const int64_t m = off_h[k + 1] - off_h[k], n = off_v[k + 1] - off_v[k];
            rows.resize(size_t(max_count) * size_t(2 * (m + n + 2)) + 8);
            count[k] = ref_local_enumerate_banded(0, 0, match, mismatch, gap, lower, upper, cutoff, seq_h + off_h[k], m,
                                                  seq_v + off_v[k], n, max_count, scores.data(), pos.data(),
                                                  rows.data(), int64_t(rows.size()));
        }
    }
    return 0;
}

}  // extern "C"
