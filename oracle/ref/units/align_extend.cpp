// extendAlignment through the UNMODIFIED reference (test infrastructure, see ref_common.h).
// Builds an Align over the infixes hSeq[hb, he) / vSeq[vb, ve) (ungapped, the seed), calls
// extendAlignment(align, hSeq, vSeq, positions, direction, [xDrop,] scoreScheme)
// (align_extend/align_extend.h:494-600) and reports the returned score and the extended rows.
#include "../ref_common.h"

#include <seqan/align_extend.h>

#include <vector>

namespace seqan_ref {
namespace {

template <typename TRow>
void write_row(TRow const & row, char const * letters, char * out, int64_t cap, int64_t * src_begin,
               int64_t * src_end)
{
    *src_begin = int64_t(beginPosition(row));
    *src_end = int64_t(endPosition(row));
    int64_t k = 0;
    for (auto it = begin(row); it != end(row) && k + 1 < cap; ++it, ++k)
        out[k] = isGap(it) ? '-' : letters[ordValue(getValue(it))];
    out[k] = 0;
}

template <typename TAlph, typename TScore>
int extend_one(TScore const & sc, const uint8_t * h, int64_t m, const uint8_t * v, int64_t n, const int64_t * pos,
               int32_t direction, int32_t xdrop_on, int32_t xdrop, int32_t * score, char * row0, char * row1,
               int64_t cap, int64_t * ends)
{
    typedef String<TAlph> TStr;
    typedef typename Infix<TStr const>::Type TInf;
    TStr hs, vs;
    resize(hs, m);
    resize(vs, n);
    for (int64_t i = 0; i < m; ++i) assignValue(hs, i, TAlph(unsigned(h[i])));
    for (int64_t i = 0; i < n; ++i) assignValue(vs, i, TAlph(unsigned(v[i])));
    TStr const & hc = hs;
    TStr const & vc = vs;
    Align<TInf> align;
    resize(rows(align), 2);
    assignSource(row(align, 0), infix(hc, pos[0], pos[2]));
    assignSource(row(align, 1), infix(vc, pos[1], pos[3]));
    Tuple<unsigned, 4> positions;
    positions[0] = unsigned(pos[0]);
    positions[1] = unsigned(pos[1]);
    positions[2] = unsigned(pos[2]);
    positions[3] = unsigned(pos[3]);
    const ExtensionDirection dir = static_cast<ExtensionDirection>(direction);
    if (xdrop_on)
        *score = extendAlignment(align, hc, vc, positions, dir, int(xdrop), sc);
    else
        *score = extendAlignment(align, hc, vc, positions, dir, sc);
    char const * letters = std::is_same<TAlph, AminoAcid>::value ? "ABCDEFGHIJKLMNOPQRSTUVWYZX*" : "ACGTN";
    write_row(row(align, 0), letters, row0, cap, ends + 0, ends + 1);
    write_row(row(align, 1), letters, row1, cap, ends + 2, ends + 3);
    return 0;
}

// The general form: any of the public overloads (align_extend/align_extend.h:494-620) -- with or
// without origScore, the band (lowerDiag, upperDiag) and xDrop -- on an aligned part whose rows
// may hold gaps: c0 / c1 give the part's rows as text with '-' for a gap (NULL: ungapped).
template <typename TAlph, typename TScore>
int extend_ex(TScore const & sc, const uint8_t * h, int64_t m, const uint8_t * v, int64_t n, const int64_t * pos,
              int32_t direction, int32_t band_on, int32_t lower, int32_t upper, int32_t xdrop_on, int32_t xdrop,
              int32_t orig_on, int32_t orig_score, const char * c0, const char * c1, int32_t * score, char * row0,
              char * row1, int64_t cap, int64_t * ends)
{
    typedef String<TAlph> TStr;
    typedef typename Infix<TStr const>::Type TInf;
    TStr hs, vs;
    resize(hs, m);
    resize(vs, n);
    for (int64_t i = 0; i < m; ++i) assignValue(hs, i, TAlph(unsigned(h[i])));
    for (int64_t i = 0; i < n; ++i) assignValue(vs, i, TAlph(unsigned(v[i])));
    TStr const & hc = hs;
    TStr const & vc = vs;
    Align<TInf> align;
    resize(rows(align), 2);
    assignSource(row(align, 0), infix(hc, pos[0], pos[2]));
    assignSource(row(align, 1), infix(vc, pos[1], pos[3]));
    if (c0 && c1)
    {
        for (int64_t i = 0; c0[i]; ++i)
            if (c0[i] == '-') insertGap(row(align, 0), i);
        for (int64_t i = 0; c1[i]; ++i)
            if (c1[i] == '-') insertGap(row(align, 1), i);
    }
    Tuple<unsigned, 4> positions;
    positions[0] = unsigned(pos[0]);
    positions[1] = unsigned(pos[1]);
    positions[2] = unsigned(pos[2]);
    positions[3] = unsigned(pos[3]);
    const ExtensionDirection dir = static_cast<ExtensionDirection>(direction);
    const int os = orig_score;
    if (orig_on)
    {
        if (band_on && xdrop_on)
            *score = extendAlignment(align, os, hc, vc, positions, dir, int(lower), int(upper), int(xdrop), sc);
        else if (band_on)
            *score = extendAlignment(align, os, hc, vc, positions, dir, int(lower), int(upper), sc);
        else if (xdrop_on)
            *score = extendAlignment(align, os, hc, vc, positions, dir, int(xdrop), sc);
        else
            *score = extendAlignment(align, os, hc, vc, positions, dir, sc);
    }
    else
    {
        if (band_on && xdrop_on)
            *score = extendAlignment(align, hc, vc, positions, dir, int(lower), int(upper), int(xdrop), sc);
        else if (band_on)
            *score = extendAlignment(align, hc, vc, positions, dir, int(lower), int(upper), sc);
        else if (xdrop_on)
            *score = extendAlignment(align, hc, vc, positions, dir, int(xdrop), sc);
        else
            *score = extendAlignment(align, hc, vc, positions, dir, sc);
    }
    char const * letters = std::is_same<TAlph, AminoAcid>::value ? "ABCDEFGHIJKLMNOPQRSTUVWYZX*" : "ACGTN";
    write_row(row(align, 0), letters, row0, cap, ends + 0, ends + 1);
    write_row(row(align, 1), letters, row1, cap, ends + 2, ends + 3);
    return 0;
}

}  // namespace
}  // namespace seqan_ref

extern "C" {

// One extension.  pos = hBegin, vBegin, hEnd, vEnd of the seed (an ungapped alignment of equal
// lengths).  Outputs the returned score, the rows of the extended (clipped) alignment as text
// ('-' for gaps), and ends = row 0 begin/end, row 1 begin/end source positions.
int ref_extend_alignment(int32_t alphabet, int32_t blosum62, int32_t match, int32_t mismatch, int32_t gap_open,
                         int32_t gap_extend, const uint8_t * h, int64_t m, const uint8_t * v, int64_t n,
                         const int64_t * pos, int32_t direction, int32_t xdrop_on, int32_t xdrop, int32_t * score,
                         char * row0, char * row1, int64_t cap, int64_t * ends)
{
    if (alphabet == 1)
    {
        if (blosum62)
        {
            Score<int, ScoreMatrix<AminoAcid, ScoreSpecBlosum62>> sc(gap_extend, gap_open);
            return seqan_ref::extend_one<AminoAcid>(sc, h, m, v, n, pos, direction, xdrop_on, xdrop, score, row0, row1,
                                                     cap, ends);
        }
        Score<int, Simple> sc(match, mismatch, gap_extend, gap_open);
        return seqan_ref::extend_one<AminoAcid>(sc, h, m, v, n, pos, direction, xdrop_on, xdrop, score, row0, row1,
                                                 cap, ends);
    }
    Score<int, Simple> sc(match, mismatch, gap_extend, gap_open);
    return seqan_ref::extend_one<Dna5>(sc, h, m, v, n, pos, direction, xdrop_on, xdrop, score, row0, row1, cap, ends);
}

// extend_ex above: band_on with (lower, upper), xdrop_on with xdrop, orig_on with orig_score,
// c0 / c1 the aligned part's rows with gaps (or NULL).
int ref_extend_alignment_ex(int32_t alphabet, int32_t blosum62, int32_t match, int32_t mismatch, int32_t gap_open,
                            int32_t gap_extend, const uint8_t * h, int64_t m, const uint8_t * v, int64_t n,
                            const int64_t * pos, int32_t direction, int32_t band_on, int32_t lower, int32_t upper,
                            int32_t xdrop_on, int32_t xdrop, int32_t orig_on, int32_t orig_score, const char * c0,
                            const char * c1, int32_t * score, char * row0, char * row1, int64_t cap, int64_t * ends)
{
#define SEQAN_REF_EXT_ARGS h, m, v, n, pos, direction, band_on, lower, upper, xdrop_on, xdrop, orig_on, orig_score, \
                           c0, c1, score, row0, row1, cap, ends
    if (alphabet == 1)
    {
        if (blosum62)
        {
            Score<int, ScoreMatrix<AminoAcid, ScoreSpecBlosum62>> sc(gap_extend, gap_open);
            return seqan_ref::extend_ex<AminoAcid>(sc, SEQAN_REF_EXT_ARGS);
        }
        Score<int, Simple> sc(match, mismatch, gap_extend, gap_open);
        return seqan_ref::extend_ex<AminoAcid>(sc, SEQAN_REF_EXT_ARGS);
    }
    Score<int, Simple> sc(match, mismatch, gap_extend, gap_open);
    return seqan_ref::extend_ex<Dna5>(sc, SEQAN_REF_EXT_ARGS);
#undef SEQAN_REF_EXT_ARGS
}

}  // extern "C"
