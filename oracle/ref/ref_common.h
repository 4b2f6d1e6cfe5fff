#pragma once
// ref_common.h -- shared templates of the extern "C" wrapper that runs the UNMODIFIED SeqAn 2 alignment code.
//
// TEST INFRASTRUCTURE ONLY.  Built by oracle/ref/Makefile from the reference's own headers
// into oracle/_ref/libseqan_ref.so; used to pin the C restatement (oracle/seqan_oracle.c)
// and to generate golden fixtures (tests/golden/make_golden.py).  The GPU engine never
// links it.  Calls made here:
//   globalAlignmentScore / localAlignmentScore / globalAlignment / localAlignment with
//   ExecutionPolicy<Parallel, Vectorial> (align_parallel/parallel_align_interface.h:288-365),
//   banded StringSet overloads (align/global_alignment_banded.h:558-700,
//   align/local_alignment_banded.h), the internal single-pair _setUpAndRunAlignment
//   (align/dp_setup.h:266-326) for raw TraceSegment_ lists, and getCigarString
//   (bam_io/cigar.h:261-339).
#include <seqan/align.h>
#include <seqan/align_parallel.h>
#include <seqan/bam_io.h>

#include <cstdint>
#include <cstring>
#include <sstream>
#include <string>
#include <map>

using namespace seqan2;

extern "C" {

struct ref_params {
    int32_t mode;          // 0 global, 1 local
    int32_t free_ends;     // TOP=1 LEFT=2 RIGHT=4 BOTTOM=8 (AlignConfig order)
    int32_t band_on, band_lower, band_upper;
    int32_t match, mismatch, gap_open, gap_extend;
    int32_t alphabet;      // 0 = Dna5, 1 = AminoAcid
    int32_t blosum62;      // 1: Score<T, ScoreMatrix<AminoAcid, ScoreSpecBlosum62>>
    int32_t score_bits;    // 16 or 32
    int32_t threads;       // ExecutionPolicy<Parallel, Vectorial> threads; 0 = plain StringSet call
};

struct ref_gaps_out {      // per pair, for Gaps-producing calls
    int32_t score;
    int32_t h_clip_begin, h_clip_end, v_clip_begin, v_clip_end;
};

}  // extern "C"

namespace seqan_ref {

template <typename TAlph>
void build_set(StringSet<String<TAlph>> & set, int64_t n, const uint8_t * seq, const int64_t * off)
{
    resize(set, n);
    for (int64_t k = 0; k < n; ++k)
    {
        String<TAlph> & s = set[k];
        resize(s, off[k + 1] - off[k]);
        for (int64_t i = off[k]; i < off[k + 1]; ++i)
            assignValue(s, i - off[k], TAlph(static_cast<unsigned>(seq[i])));
    }
}

template <typename TScoreValue, typename TAlph, bool B62>
struct ScoreOf;
template <typename TScoreValue, typename TAlph>
struct ScoreOf<TScoreValue, TAlph, false>
{
    using Type = Score<TScoreValue, Simple>;
    static Type make(ref_params const & p)
    {
        return Type(p.match, p.mismatch, p.gap_extend, p.gap_open);
    }
};
template <typename TScoreValue, typename TAlph>
struct ScoreOf<TScoreValue, TAlph, true>
{
    using Type = Score<TScoreValue, ScoreMatrix<AminoAcid, ScoreSpecBlosum62>>;
    static Type make(ref_params const & p)
    {
        return Type(p.gap_extend, p.gap_open);
    }
};

template <bool T, bool L, bool R, bool B, typename TScoreValue, typename TAlph, bool B62>
int run_score(ref_params const & p, int64_t n, const uint8_t * sh, const int64_t * oh,
              const uint8_t * sv, const int64_t * ov, int32_t * out)
{
    StringSet<String<TAlph>> setH, setV;
    build_set(setH, n, sh, oh);
    build_set(setV, n, sv, ov);
    auto score = ScoreOf<TScoreValue, TAlph, B62>::make(p);
    String<TScoreValue> res;
    ExecutionPolicy<Parallel, Vectorial> exec;
    setNumThreads(exec, p.threads > 0 ? p.threads : 1);
    if (p.mode == 0)
    {
        AlignConfig<T, L, R, B> cfg;
        if (p.band_on)
        {
            if (p.threads > 0)
                res = globalAlignmentScore(exec, setH, setV, score, cfg, p.band_lower, p.band_upper);
            else
                res = globalAlignmentScore(setH, setV, score, cfg, p.band_lower, p.band_upper);
        }
        else
        {
            if (p.threads > 0)
                res = globalAlignmentScore(exec, setH, setV, score, cfg);
            else
                res = globalAlignmentScore(setH, setV, score, cfg);
        }
    }
    else
    {
        if (p.band_on)
        {
            if (p.threads > 0)
                res = localAlignmentScore(exec, setH, setV, score, p.band_lower, p.band_upper);
            else
                res = localAlignmentScore(setH, setV, score, p.band_lower, p.band_upper);
        }
        else
        {
            if (p.threads > 0)
                res = localAlignmentScore(exec, setH, setV, score);
            else
                res = localAlignmentScore(setH, setV, score);
        }
    }
    for (int64_t k = 0; k < n; ++k)
        out[k] = static_cast<int32_t>(res[k]);
    return 0;
}

// Gapped rows are written the way the reference's tests print them (operator<< on Gaps).
template <bool T, bool L, bool R, bool B, typename TScoreValue, typename TAlph, bool B62>
int run_gaps(ref_params const & p, int64_t n, const uint8_t * sh, const int64_t * oh,
             const uint8_t * sv, const int64_t * ov, ref_gaps_out * out,
             char * rows, const int64_t * row_off, char * cigar, int64_t cigar_stride)
{
    typedef String<TAlph> TSeq;
    typedef Gaps<TSeq, ArrayGaps> TGaps;
    StringSet<TSeq> setH, setV;
    build_set(setH, n, sh, oh);
    build_set(setV, n, sv, ov);
    StringSet<TGaps> gapsH, gapsV;
    resize(gapsH, n);
    resize(gapsV, n);
    for (int64_t k = 0; k < n; ++k)
    {
        gapsH[k] = TGaps(setH[k]);
        gapsV[k] = TGaps(setV[k]);
    }
    auto score = ScoreOf<TScoreValue, TAlph, B62>::make(p);
    String<TScoreValue> res;
    ExecutionPolicy<Parallel, Vectorial> exec;
    setNumThreads(exec, p.threads > 0 ? p.threads : 1);
    if (p.mode == 0)
    {
        AlignConfig<T, L, R, B> cfg;
        if (p.band_on)
        {
            if (p.threads > 0)
                res = globalAlignment(exec, gapsH, gapsV, score, cfg, p.band_lower, p.band_upper);
            else
                res = globalAlignment(gapsH, gapsV, score, cfg, p.band_lower, p.band_upper);
        }
        else
        {
            if (p.threads > 0)
                res = globalAlignment(exec, gapsH, gapsV, score, cfg);
            else
                res = globalAlignment(gapsH, gapsV, score, cfg);
        }
    }
    else
    {
        if (p.band_on)
        {
            if (p.threads > 0)
                res = localAlignment(exec, gapsH, gapsV, score, p.band_lower, p.band_upper);
            else
                res = localAlignment(gapsH, gapsV, score, p.band_lower, p.band_upper);
        }
        else
        {
            if (p.threads > 0)
                res = localAlignment(exec, gapsH, gapsV, score);
            else
                res = localAlignment(gapsH, gapsV, score);
        }
    }
    for (int64_t k = 0; k < n; ++k)
    {
        out[k].score = static_cast<int32_t>(res[k]);
        out[k].h_clip_begin = static_cast<int32_t>(clippedBeginPosition(gapsH[k]));
        out[k].h_clip_end = static_cast<int32_t>(clippedEndPosition(gapsH[k]));
        out[k].v_clip_begin = static_cast<int32_t>(clippedBeginPosition(gapsV[k]));
        out[k].v_clip_end = static_cast<int32_t>(clippedEndPosition(gapsV[k]));
        if (rows)
        {
            std::stringstream ssH, ssV;
            ssH << gapsH[k];
            ssV << gapsV[k];
            std::string s = ssH.str() + "\n" + ssV.str();
            int64_t cap = row_off[k + 1] - row_off[k];
            int64_t len = static_cast<int64_t>(s.size());
            if (len >= cap)
                len = cap - 1;
            std::memcpy(rows + row_off[k], s.data(), len);
            rows[row_off[k] + len] = 0;
        }
        if (cigar)
        {
            CharString c;
            getCigarString(c, gapsH[k], gapsV[k]);
            int64_t len = static_cast<int64_t>(length(c));
            if (len >= cigar_stride)
                len = cigar_stride - 1;
            for (int64_t i = 0; i < len; ++i)
                cigar[k * cigar_stride + i] = c[i];
            cigar[k * cigar_stride + len] = 0;
        }
    }
    return 0;
}

// Raw TraceSegment_ list of the scalar single-pair DP (what _adaptTraceSegmentsTo consumes).
template <bool T, bool L, bool R, bool B, typename TScoreValue, typename TAlph, bool B62>
int run_segments(ref_params const & p, const uint8_t * h, int32_t m, const uint8_t * v, int32_t n,
                 int32_t * score_out, uint32_t * segs, int32_t cap, int32_t * nseg)
{
    typedef String<TAlph> TSeq;
    TSeq sH, sV;
    resize(sH, m);
    resize(sV, n);
    for (int32_t i = 0; i < m; ++i) assignValue(sH, i, TAlph(static_cast<unsigned>(h[i])));
    for (int32_t i = 0; i < n; ++i) assignValue(sV, i, TAlph(static_cast<unsigned>(v[i])));
    auto score = ScoreOf<TScoreValue, TAlph, B62>::make(p);
    typedef TraceSegment_<unsigned, unsigned> TSeg;
    String<TSeg> trace;
    DPScoutState_<Default> state;
    TScoreValue res;
    bool affine = score.data_gap_open != score.data_gap_extend;
    if (p.mode == 0)
    {
        typedef typename SubstituteAlignConfig_<AlignConfig<T, L, R, B>>::Type TFree;
        if (p.band_on)
        {
            typedef AlignConfig2<DPGlobal, DPBandConfig<BandOn>, TFree> TCfg;
            TCfg cfg(p.band_lower, p.band_upper);
            res = affine ? _setUpAndRunAlignment(trace, state, sH, sV, score, cfg, AffineGaps())
                         : _setUpAndRunAlignment(trace, state, sH, sV, score, cfg, LinearGaps());
        }
        else
        {
            typedef AlignConfig2<DPGlobal, DPBandConfig<BandOff>, TFree> TCfg;
            res = affine ? _setUpAndRunAlignment(trace, state, sH, sV, score, TCfg(), AffineGaps())
                         : _setUpAndRunAlignment(trace, state, sH, sV, score, TCfg(), LinearGaps());
        }
    }
    else
    {
        if (p.band_on)
        {
            typedef AlignConfig2<DPLocal, DPBandConfig<BandOn>, FreeEndGaps_<>> TCfg;
            TCfg cfg(p.band_lower, p.band_upper);
            res = affine ? _setUpAndRunAlignment(trace, state, sH, sV, score, cfg, AffineGaps())
                         : _setUpAndRunAlignment(trace, state, sH, sV, score, cfg, LinearGaps());
        }
        else
        {
            typedef AlignConfig2<DPLocal, DPBandConfig<BandOff>, FreeEndGaps_<>> TCfg;
            res = affine ? _setUpAndRunAlignment(trace, state, sH, sV, score, TCfg(), AffineGaps())
                         : _setUpAndRunAlignment(trace, state, sH, sV, score, TCfg(), LinearGaps());
        }
    }
    *score_out = static_cast<int32_t>(res);
    int32_t ns = static_cast<int32_t>(length(trace));
    *nseg = ns;
    for (int32_t i = 0; i < ns && i < cap; ++i)
    {
        segs[4 * i + 0] = trace[i]._horizontalBeginPos;
        segs[4 * i + 1] = trace[i]._verticalBeginPos;
        segs[4 * i + 2] = trace[i]._length;
        segs[4 * i + 3] = trace[i]._traceValue;
    }
    return 0;
}

}  // namespace seqan_ref

namespace seqan_ref {

// Unit registry: each translation unit instantiates a few SeqAn call shapes (SeqAn's SIMD
// templates take ~30 s each to compile, so units are built in parallel).
typedef int (*score_fn)(ref_params const &, int64_t, const uint8_t *, const int64_t *,
                        const uint8_t *, const int64_t *, int32_t *);
typedef int (*gaps_fn)(ref_params const &, int64_t, const uint8_t *, const int64_t *,
                       const uint8_t *, const int64_t *, ref_gaps_out *, char *, const int64_t *,
                       char *, int64_t);
typedef int (*seg_fn)(ref_params const &, const uint8_t *, int32_t, const uint8_t *, int32_t,
                      int32_t *, uint32_t *, int32_t, int32_t *);

// key = kind(0 score,1 gaps,2 segments) | mode<<2 | band<<3 | variant<<4 | free_ends<<8
void register_unit(int key, void * fn);
inline int variant_of(ref_params const & p)
{
    int v = (p.alphabet == 0) ? 0 : 2;
    return v + (p.score_bits == 16 ? 0 : 1);
}
inline int make_key(int kind, ref_params const & p)
{
    int fe = (p.mode == 1) ? 0 : (p.free_ends & 15);
    return kind | (p.mode << 2) | ((p.band_on ? 1 : 0) << 3) | (variant_of(p) << 4) | (fe << 8);
}

struct Registrar
{
    Registrar(int key, void * fn) { register_unit(key, fn); }
};

}  // namespace seqan_ref

// variant: 0 Dna5/int16, 1 Dna5/int32, 2 AminoAcid-Blosum62/int16, 3 AminoAcid-Blosum62/int32
// kind: 0 run_score, 1 run_gaps, 2 run_segments.
#define SEQAN_REF_UNIT(NAME, KIND, FN, MODE, BAND, VARIANT, FE, T, L, R, B, TV, TA, BB)      \
    namespace {                                                                             \
    seqan_ref::Registrar reg_##NAME(                                                        \
        (KIND) | ((MODE) << 2) | ((BAND) << 3) | ((VARIANT) << 4) | ((FE) << 8),              \
        (void *)&seqan_ref::FN<T, L, R, B, TV, TA, BB>);                                     \
    }
