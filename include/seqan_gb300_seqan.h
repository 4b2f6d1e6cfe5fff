// seqan_gb300_seqan.h -- SeqAn 2 call surface on the GB300 engine (header-only C++ binding).
//
// Include after <seqan/align.h> (and <seqan/align_parallel.h>) in code built against SeqAn 2
// and link libseqan_gb300.so.  It adds a parallel policy tag `GB300` and overloads of the four
// batch functions of align_parallel/parallel_align_interface.h:288-365 for
// ExecutionPolicy<GB300, TVectorization>, with the reference's argument lists:
//
//   globalAlignmentScore(exec, setH, setV, score [, AlignConfig] [, lowerDiag, upperDiag])
//   globalAlignmentScore(exec, seqH, setV, score [, AlignConfig])        (one vs many)
//   localAlignmentScore (exec, setH, setV, score [, lowerDiag, upperDiag])
//   globalAlignment     (exec, gapsSetH, gapsSetV, score [, AlignConfig] [, lowerDiag, upperDiag])
//   localAlignment      (exec, gapsSetH, gapsSetV, score [, lowerDiag, upperDiag])
//   globalAlignment     (exec, alignSet, score [, AlignConfig] [, lowerDiag, upperDiag])
//   localAlignment      (exec, alignSet, score [, lowerDiag, upperDiag])   (StringSet<Align>:
//                        row 0 = H, row 1 = V; align/global_alignment_unbanded.h:894-952,
//                        align/local_alignment_unbanded.h:405-439)
//
// and batch forms of extendSeed (seeds/seeds_extension.h:181-218, 283-360, 780-835), whose
// reference form extends one Seed<Simple> per call:
//
//   extendSeed(exec, seeds, databases, queries, direction, MatchExtend())
//   extendSeed(exec, seeds, databases, queries, direction, score, scoreDropOff,
//              UnGappedXDrop() | GappedXDrop())
//
// seeds[k] lies on databases[k] / queries[k] (StringSets), or on the one database String and
// queries[k];
//
// so switching a call from ExecutionPolicy<Parallel, Vectorial> is a change of the policy
// type only.  Sequences go to the engine as ordValue codes (the layout of
// StringSet<..., Owner<ConcatDirect<>>>); Score<T, Simple> passes its four values and
// Score<T, ScoreMatrix<...>> its table; T = int16_t selects 16-bit cells as the reference's
// SIMD path does (pairs that could leave the exact int16 range run with 32-bit cells).  The
// Gaps results are rebuilt by the reference's own _adaptTraceSegmentsTo
// (align/dp_traceback_adaptor.h:57-117) from the engine's TraceSegment_ lists, so Gaps parity
// is structural.  Errors throw std::runtime_error with the engine's message (the reference's
// functions have no error channel).
#ifndef SEQAN_GB300_SEQAN_H_
#define SEQAN_GB300_SEQAN_H_

#include <seqan/align.h>
#include <seqan/bam_io.h>
#include <seqan/seeds.h>
#include <seqan/seq_io.h>

#include <algorithm>
#include <cstdint>
#include <cstring>
#include <stdexcept>
#include <string>
#include <type_traits>
#include <vector>

#include "seqan_gb300.h"

namespace seqan2 {

struct GB300_;
typedef Tag<GB300_> GB300;   // parallel policy: the GB300 batch engine

namespace gb300_impl {

// One engine context per process (device 0), created on first use.
inline gba_context *context()
{
    static gba_context *ctx = [] {
        gba_context *c = nullptr;
        gba_config cfg{0, 0};
        const int rc = gba_create(&c, &cfg);
        if (rc != GBA_OK) throw std::runtime_error(std::string("gba_create: ") + gba_status_string(rc));
        return c;
    }();
    return ctx;
}

inline void check(int rc, char const *what)
{
    if (rc == GBA_OK) return;
    char buf[512] = {0};
    gba_last_error(context(), buf, sizeof(buf));
    throw std::runtime_error(std::string(what) + ": " + gba_status_string(rc) + ": " + buf);
}

// Concatenated ordValue codes and offsets of a set of sequences.
struct Codes {
    std::vector<uint8_t> seq;
    std::vector<int64_t> off{0};
    template <typename TSeq>
    void add(TSeq const &s)
    {
        for (auto it = begin(s, Standard()); it != end(s, Standard()); ++it) seq.push_back(uint8_t(ordValue(*it)));
        off.push_back(int64_t(seq.size()));
    }
};

template <typename TSet>
Codes flatten(TSet const &set)
{
    Codes c;
    for (size_t k = 0; k < length(set); ++k) c.add(set[k]);
    return c;
}

template <typename TGapsSet>
Codes flatten_gaps(TGapsSet const &set)
{
    Codes c;
    for (size_t k = 0; k < length(set); ++k) c.add(source(set[k]));
    return c;
}

// Scoring scheme -> engine parameters.
template <typename TValue, typename TAlphabet>
void set_score(gba_params &p, std::vector<int32_t> &, Score<TValue, Simple> const &sc)
{
    p.match = scoreMatch(sc);
    p.mismatch = scoreMismatch(sc);
    p.gap_open = scoreGapOpen(sc);
    p.gap_extend = scoreGapExtend(sc);
    p.alphabet_size = int32_t(ValueSize<TAlphabet>::VALUE);
}

template <typename TValue, typename TAlphabet, typename TSeqValue, typename TSpec>
void set_score(gba_params &p, std::vector<int32_t> &table, Score<TValue, ScoreMatrix<TSeqValue, TSpec>> const &sc)
{
    const int A = int(ValueSize<TAlphabet>::VALUE);
    table.resize(size_t(A) * A);
    for (int i = 0; i < A; ++i)
        for (int j = 0; j < A; ++j) table[i * A + j] = int32_t(score(sc, TAlphabet(i), TAlphabet(j)));
    p.matrix = table.data();
    p.alphabet_size = A;
    p.gap_open = scoreGapOpen(sc);
    p.gap_extend = scoreGapExtend(sc);
}

template <typename TScoreValue>
constexpr int score_bits()
{
    static_assert(sizeof(TScoreValue) == 2 || sizeof(TScoreValue) == 4,
                  "the GB300 engine computes with 16- or 32-bit score values");
    return sizeof(TScoreValue) == 2 ? 16 : 32;
}

template <bool TOP, bool LEFT, bool RIGHT, bool BOTTOM, typename TACSpec>
int free_ends(AlignConfig<TOP, LEFT, RIGHT, BOTTOM, TACSpec> const &)
{
    return (TOP ? GBA_FREE_TOP : 0) | (LEFT ? GBA_FREE_LEFT : 0) | (RIGHT ? GBA_FREE_RIGHT : 0) |
           (BOTTOM ? GBA_FREE_BOTTOM : 0);
}

struct Band {
    bool on = false;
    int lower = 0, upper = 0;
};

// Runs one batch; returns the scores and, with `segments`, fills each pair's TraceSegment_ list.
template <typename TScoreValue, typename TAlphabet, typename TScoreSpec>
String<TScoreValue> run(Codes const &h, Codes const &v, bool h_shared, Score<TScoreValue, TScoreSpec> const &sc,
                        int mode, int fe, Band band,
                        std::vector<String<TraceSegment_<unsigned, unsigned>>> *segments)
{
    gba_params p{};
    std::vector<int32_t> table;
    set_score<TScoreValue, TAlphabet>(p, table, sc);
    p.mode = mode;
    p.gap_model = GBA_GAPS_AUTO;
    p.free_ends = mode == GBA_GLOBAL ? fe : 0;
    p.band_on = band.on;
    p.band_lower = band.lower;
    p.band_upper = band.upper;
    p.score_bits = score_bits<TScoreValue>();
    p.outputs = GBA_OUT_SCORE | GBA_OUT_END | (segments ? GBA_OUT_SEGMENTS : 0);
    const int64_t n = int64_t(v.off.size()) - 1;
    gba_batch b{};
    b.num_pairs = n;
    b.seq_h = h.seq.data();
    b.off_h = h.off.data();
    b.seq_v = v.seq.data();
    b.off_v = v.off.data();
    b.h_shared = h_shared ? 1 : 0;
    std::vector<int32_t> score(size_t(n) + 1);
    std::vector<gba_segment> segs;
    std::vector<int64_t> seg_off(size_t(n) + 1);
    gba_result r{};
    r.score = score.data();
    if (segments) {
        // At most m + n + 4 segments per pair.
        int64_t cap = 4 * n;
        for (int64_t k = 0; k < n; ++k)
            cap += (h_shared ? h.off[1] - h.off[0] : h.off[k + 1] - h.off[k]) + v.off[k + 1] - v.off[k];
        segs.resize(size_t(cap) + 1);
        r.segments = segs.data();
        r.segment_capacity = cap;
        r.segment_offsets = seg_off.data();
    }
    check(gba_align_batch(context(), &p, &b, &r), "gba_align_batch");
    String<TScoreValue> out;
    resize(out, size_t(n));
    for (int64_t k = 0; k < n; ++k) out[k] = TScoreValue(score[k]);
    if (segments) {
        segments->resize(size_t(n));
        for (int64_t k = 0; k < n; ++k) {
            auto &dst = (*segments)[k];
            clear(dst);
            for (int64_t q = seg_off[k]; q < seg_off[k + 1]; ++q)
                appendValue(dst, TraceSegment_<unsigned, unsigned>(segs[q].h_begin, segs[q].v_begin, segs[q].length,
                                                                    uint8_t(segs[q].type)));
        }
    }
    return out;
}

template <typename TSet>
using AlphabetOf = typename Value<typename Value<TSet>::Type>::Type;

template <typename TGapsSet>
using GapsAlphabetOf = typename Value<typename Source<typename Value<TGapsSet>::Type>::Type>::Type;

// Aligns pair k = (source(rowH(k)), source(rowV(k))) for k < count and rebuilds both Gaps rows.
template <typename TScoreValue, typename TScoreSpec, typename TAlphabet, typename TRowH, typename TRowV>
String<TScoreValue> run_rows(size_t count, TRowH rowH, TRowV rowV, Score<TScoreValue, TScoreSpec> const &sc, int mode,
                             int fe, Band band)
{
    Codes h, v;
    for (size_t k = 0; k < count; ++k) {
        h.add(source(rowH(k)));
        v.add(source(rowV(k)));
    }
    std::vector<String<TraceSegment_<unsigned, unsigned>>> segs;
    String<TScoreValue> out = run<TScoreValue, TAlphabet>(h, v, false, sc, mode, fe, band, &segs);
    for (size_t k = 0; k < count; ++k) _adaptTraceSegmentsTo(rowH(k), rowV(k), segs[k]);
    return out;
}

template <typename TScoreValue, typename TScoreSpec, typename TGapsSetH, typename TGapsSetV>
String<TScoreValue> run_gaps(TGapsSetH &gapsH, TGapsSetV &gapsV, Score<TScoreValue, TScoreSpec> const &sc, int mode,
                             int fe, Band band)
{
    if (length(gapsH) != length(gapsV)) throw std::runtime_error("gapsH and gapsV differ in length");
    return run_rows<TScoreValue, TScoreSpec, GapsAlphabetOf<TGapsSetH>>(
        length(gapsH), [&](size_t k) -> decltype(gapsH[0]) & { return gapsH[k]; },
        [&](size_t k) -> decltype(gapsV[0]) & { return gapsV[k]; }, sc, mode, fe, band);
}

// StringSet<Align>: row 0 is H, row 1 is V (align/global_alignment_unbanded.h:894-952).
template <typename TScoreValue, typename TScoreSpec, typename TSeq, typename TAlignSpec, typename TSetSpec>
String<TScoreValue> run_aligns(StringSet<Align<TSeq, TAlignSpec>, TSetSpec> &set, Score<TScoreValue, TScoreSpec> const &sc,
                               int mode, int fe, Band band)
{
    return run_rows<TScoreValue, TScoreSpec, typename Value<TSeq>::Type>(
        length(set), [&](size_t k) -> decltype(row(set[0], 0)) & { return row(set[k], 0); },
        [&](size_t k) -> decltype(row(set[0], 1)) & { return row(set[k], 1); }, sc, mode, fe, band);
}

}  // namespace gb300_impl

// ---- globalAlignmentScore ---------------------------------------------------------------

template <typename TVec, typename TSetH, typename TSetV, typename TScoreValue, typename TScoreSpec, bool TOP,
          bool LEFT, bool RIGHT, bool BOTTOM, typename TACSpec>
SEQAN_FUNC_ENABLE_IF(And<Is<ContainerConcept<typename Value<TSetH>::Type>>,
                         Is<ContainerConcept<typename Value<TSetV>::Type>>>,
                     String<TScoreValue>)
globalAlignmentScore(ExecutionPolicy<GB300, TVec> const &, TSetH const &setH, TSetV const &setV,
                     Score<TScoreValue, TScoreSpec> const &sc, AlignConfig<TOP, LEFT, RIGHT, BOTTOM, TACSpec> const &ac,
                     int lowerDiag, int upperDiag)
{
    if (length(setH) != length(setV)) throw std::runtime_error("setH and setV differ in length");
    return gb300_impl::run<TScoreValue, gb300_impl::AlphabetOf<TSetH>>(
        gb300_impl::flatten(setH), gb300_impl::flatten(setV), false, sc, GBA_GLOBAL, gb300_impl::free_ends(ac),
        gb300_impl::Band{true, lowerDiag, upperDiag}, nullptr);
}

template <typename TVec, typename TSetH, typename TSetV, typename TScoreValue, typename TScoreSpec, bool TOP,
          bool LEFT, bool RIGHT, bool BOTTOM, typename TACSpec>
SEQAN_FUNC_ENABLE_IF(And<Is<ContainerConcept<typename Value<TSetH>::Type>>,
                         Is<ContainerConcept<typename Value<TSetV>::Type>>>,
                     String<TScoreValue>)
globalAlignmentScore(ExecutionPolicy<GB300, TVec> const &, TSetH const &setH, TSetV const &setV,
                     Score<TScoreValue, TScoreSpec> const &sc, AlignConfig<TOP, LEFT, RIGHT, BOTTOM, TACSpec> const &ac)
{
    if (length(setH) != length(setV)) throw std::runtime_error("setH and setV differ in length");
    return gb300_impl::run<TScoreValue, gb300_impl::AlphabetOf<TSetH>>(
        gb300_impl::flatten(setH), gb300_impl::flatten(setV), false, sc, GBA_GLOBAL, gb300_impl::free_ends(ac),
        gb300_impl::Band{}, nullptr);
}

template <typename TVec, typename TSetH, typename TSetV, typename TScoreValue, typename TScoreSpec>
SEQAN_FUNC_ENABLE_IF(And<Is<ContainerConcept<typename Value<TSetH>::Type>>,
                         Is<ContainerConcept<typename Value<TSetV>::Type>>>,
                     String<TScoreValue>)
globalAlignmentScore(ExecutionPolicy<GB300, TVec> const &exec, TSetH const &setH, TSetV const &setV,
                     Score<TScoreValue, TScoreSpec> const &sc, int lowerDiag, int upperDiag)
{
    return globalAlignmentScore(exec, setH, setV, sc, AlignConfig<>(), lowerDiag, upperDiag);
}

template <typename TVec, typename TSetH, typename TSetV, typename TScoreValue, typename TScoreSpec>
SEQAN_FUNC_ENABLE_IF(And<Is<ContainerConcept<typename Value<TSetH>::Type>>,
                         Is<ContainerConcept<typename Value<TSetV>::Type>>>,
                     String<TScoreValue>)
globalAlignmentScore(ExecutionPolicy<GB300, TVec> const &exec, TSetH const &setH, TSetV const &setV,
                     Score<TScoreValue, TScoreSpec> const &sc)
{
    return globalAlignmentScore(exec, setH, setV, sc, AlignConfig<>());
}

// One vs many (align/global_alignment_unbanded.h:766-821).
template <typename TVec, typename TString1, typename TString2, typename TSpec, typename TScoreValue,
          typename TScoreSpec, bool TOP, bool LEFT, bool RIGHT, bool BOTTOM, typename TACSpec>
SEQAN_FUNC_DISABLE_IF(Is<ContainerConcept<typename Value<TString1>::Type>>, String<TScoreValue>)
globalAlignmentScore(ExecutionPolicy<GB300, TVec> const &, TString1 const &seqH, StringSet<TString2, TSpec> const &setV,
                     Score<TScoreValue, TScoreSpec> const &sc, AlignConfig<TOP, LEFT, RIGHT, BOTTOM, TACSpec> const &ac)
{
    gb300_impl::Codes h;
    h.add(seqH);
    return gb300_impl::run<TScoreValue, typename Value<TString1>::Type>(
        h, gb300_impl::flatten(setV), true, sc, GBA_GLOBAL, gb300_impl::free_ends(ac), gb300_impl::Band{}, nullptr);
}

template <typename TVec, typename TString1, typename TString2, typename TSpec, typename TScoreValue,
          typename TScoreSpec>
SEQAN_FUNC_DISABLE_IF(Is<ContainerConcept<typename Value<TString1>::Type>>, String<TScoreValue>)
globalAlignmentScore(ExecutionPolicy<GB300, TVec> const &exec, TString1 const &seqH,
                     StringSet<TString2, TSpec> const &setV, Score<TScoreValue, TScoreSpec> const &sc)
{
    return globalAlignmentScore(exec, seqH, setV, sc, AlignConfig<>());
}

// ---- localAlignmentScore ----------------------------------------------------------------

template <typename TVec, typename TSetH, typename TSetV, typename TScoreValue, typename TScoreSpec>
String<TScoreValue> localAlignmentScore(ExecutionPolicy<GB300, TVec> const &, TSetH const &setH, TSetV const &setV,
                                        Score<TScoreValue, TScoreSpec> const &sc, int lowerDiag, int upperDiag)
{
    if (length(setH) != length(setV)) throw std::runtime_error("setH and setV differ in length");
    return gb300_impl::run<TScoreValue, gb300_impl::AlphabetOf<TSetH>>(
        gb300_impl::flatten(setH), gb300_impl::flatten(setV), false, sc, GBA_LOCAL, 0,
        gb300_impl::Band{true, lowerDiag, upperDiag}, nullptr);
}

template <typename TVec, typename TSetH, typename TSetV, typename TScoreValue, typename TScoreSpec>
String<TScoreValue> localAlignmentScore(ExecutionPolicy<GB300, TVec> const &, TSetH const &setH, TSetV const &setV,
                                        Score<TScoreValue, TScoreSpec> const &sc)
{
    if (length(setH) != length(setV)) throw std::runtime_error("setH and setV differ in length");
    return gb300_impl::run<TScoreValue, gb300_impl::AlphabetOf<TSetH>>(
        gb300_impl::flatten(setH), gb300_impl::flatten(setV), false, sc, GBA_LOCAL, 0, gb300_impl::Band{}, nullptr);
}

// ---- globalAlignment / localAlignment over StringSet<Gaps> -------------------------------

template <typename TVec, typename TGapsSetH, typename TGapsSetV, typename TScoreValue, typename TScoreSpec, bool TOP,
          bool LEFT, bool RIGHT, bool BOTTOM, typename TACSpec>
String<TScoreValue> globalAlignment(ExecutionPolicy<GB300, TVec> const &, TGapsSetH &gapsH, TGapsSetV &gapsV,
                                    Score<TScoreValue, TScoreSpec> const &sc,
                                    AlignConfig<TOP, LEFT, RIGHT, BOTTOM, TACSpec> const &ac, int lowerDiag,
                                    int upperDiag)
{
    return gb300_impl::run_gaps(gapsH, gapsV, sc, GBA_GLOBAL, gb300_impl::free_ends(ac),
                                gb300_impl::Band{true, lowerDiag, upperDiag});
}

template <typename TVec, typename TGapsSetH, typename TGapsSetV, typename TScoreValue, typename TScoreSpec, bool TOP,
          bool LEFT, bool RIGHT, bool BOTTOM, typename TACSpec>
String<TScoreValue> globalAlignment(ExecutionPolicy<GB300, TVec> const &, TGapsSetH &gapsH, TGapsSetV &gapsV,
                                    Score<TScoreValue, TScoreSpec> const &sc,
                                    AlignConfig<TOP, LEFT, RIGHT, BOTTOM, TACSpec> const &ac)
{
    return gb300_impl::run_gaps(gapsH, gapsV, sc, GBA_GLOBAL, gb300_impl::free_ends(ac), gb300_impl::Band{});
}

template <typename TVec, typename TGapsSetH, typename TGapsSetV, typename TScoreValue, typename TScoreSpec>
String<TScoreValue> globalAlignment(ExecutionPolicy<GB300, TVec> const &exec, TGapsSetH &gapsH, TGapsSetV &gapsV,
                                    Score<TScoreValue, TScoreSpec> const &sc, int lowerDiag, int upperDiag)
{
    return globalAlignment(exec, gapsH, gapsV, sc, AlignConfig<>(), lowerDiag, upperDiag);
}

template <typename TVec, typename TGapsSetH, typename TGapsSetV, typename TScoreValue, typename TScoreSpec>
String<TScoreValue> globalAlignment(ExecutionPolicy<GB300, TVec> const &exec, TGapsSetH &gapsH, TGapsSetV &gapsV,
                                    Score<TScoreValue, TScoreSpec> const &sc)
{
    return globalAlignment(exec, gapsH, gapsV, sc, AlignConfig<>());
}

template <typename TVec, typename TGapsSetH, typename TGapsSetV, typename TScoreValue, typename TScoreSpec>
String<TScoreValue> localAlignment(ExecutionPolicy<GB300, TVec> const &, TGapsSetH &gapsH, TGapsSetV &gapsV,
                                   Score<TScoreValue, TScoreSpec> const &sc, int lowerDiag, int upperDiag)
{
    return gb300_impl::run_gaps(gapsH, gapsV, sc, GBA_LOCAL, 0, gb300_impl::Band{true, lowerDiag, upperDiag});
}

template <typename TVec, typename TGapsSetH, typename TGapsSetV, typename TScoreValue, typename TScoreSpec>
String<TScoreValue> localAlignment(ExecutionPolicy<GB300, TVec> const &, TGapsSetH &gapsH, TGapsSetV &gapsV,
                                   Score<TScoreValue, TScoreSpec> const &sc)
{
    return gb300_impl::run_gaps(gapsH, gapsV, sc, GBA_LOCAL, 0, gb300_impl::Band{});
}

// ---- globalAlignment / localAlignment over StringSet<Align> ------------------------------

template <typename TVec, typename TSeq, typename TAlignSpec, typename TSetSpec, typename TScoreValue, typename TScoreSpec,
          bool TOP, bool LEFT, bool RIGHT, bool BOTTOM, typename TACSpec>
String<TScoreValue> globalAlignment(ExecutionPolicy<GB300, TVec> const &, StringSet<Align<TSeq, TAlignSpec>, TSetSpec> &aligns,
                                    Score<TScoreValue, TScoreSpec> const &sc,
                                    AlignConfig<TOP, LEFT, RIGHT, BOTTOM, TACSpec> const &ac, int lowerDiag,
                                    int upperDiag)
{
    return gb300_impl::run_aligns(aligns, sc, GBA_GLOBAL, gb300_impl::free_ends(ac),
                                  gb300_impl::Band{true, lowerDiag, upperDiag});
}

template <typename TVec, typename TSeq, typename TAlignSpec, typename TSetSpec, typename TScoreValue, typename TScoreSpec,
          bool TOP, bool LEFT, bool RIGHT, bool BOTTOM, typename TACSpec>
String<TScoreValue> globalAlignment(ExecutionPolicy<GB300, TVec> const &, StringSet<Align<TSeq, TAlignSpec>, TSetSpec> &aligns,
                                    Score<TScoreValue, TScoreSpec> const &sc,
                                    AlignConfig<TOP, LEFT, RIGHT, BOTTOM, TACSpec> const &ac)
{
    return gb300_impl::run_aligns(aligns, sc, GBA_GLOBAL, gb300_impl::free_ends(ac), gb300_impl::Band{});
}

template <typename TVec, typename TSeq, typename TAlignSpec, typename TSetSpec, typename TScoreValue, typename TScoreSpec>
String<TScoreValue> globalAlignment(ExecutionPolicy<GB300, TVec> const &exec,
                                    StringSet<Align<TSeq, TAlignSpec>, TSetSpec> &aligns,
                                    Score<TScoreValue, TScoreSpec> const &sc, int lowerDiag, int upperDiag)
{
    return globalAlignment(exec, aligns, sc, AlignConfig<>(), lowerDiag, upperDiag);
}

template <typename TVec, typename TSeq, typename TAlignSpec, typename TSetSpec, typename TScoreValue, typename TScoreSpec>
String<TScoreValue> globalAlignment(ExecutionPolicy<GB300, TVec> const &exec,
                                    StringSet<Align<TSeq, TAlignSpec>, TSetSpec> &aligns,
                                    Score<TScoreValue, TScoreSpec> const &sc)
{
    return globalAlignment(exec, aligns, sc, AlignConfig<>());
}

template <typename TVec, typename TSeq, typename TAlignSpec, typename TSetSpec, typename TScoreValue, typename TScoreSpec>
String<TScoreValue> localAlignment(ExecutionPolicy<GB300, TVec> const &, StringSet<Align<TSeq, TAlignSpec>, TSetSpec> &aligns,
                                   Score<TScoreValue, TScoreSpec> const &sc, int lowerDiag, int upperDiag)
{
    return gb300_impl::run_aligns(aligns, sc, GBA_LOCAL, 0, gb300_impl::Band{true, lowerDiag, upperDiag});
}

template <typename TVec, typename TSeq, typename TAlignSpec, typename TSetSpec, typename TScoreValue, typename TScoreSpec>
String<TScoreValue> localAlignment(ExecutionPolicy<GB300, TVec> const &, StringSet<Align<TSeq, TAlignSpec>, TSetSpec> &aligns,
                                   Score<TScoreValue, TScoreSpec> const &sc)
{
    return gb300_impl::run_aligns(aligns, sc, GBA_LOCAL, 0, gb300_impl::Band{});
}

// ---- Seed extension ------------------------------------------------------------------------

namespace gb300_impl {

// The reference declares its tags as `typedef Tag<X_> const X`.
template <typename T>
struct is_gapped : std::is_same<T, typename std::remove_const<GappedXDrop>::type> {};
template <typename T>
struct is_xdrop_tag
    : std::integral_constant<bool, is_gapped<T>::value ||
                                       std::is_same<T, typename std::remove_const<UnGappedXDrop>::type>::value> {};

template <typename TAlphabet, typename TScoreValue>
void set_seed_score(gba_extend_params &p, std::vector<int32_t> &, Score<TScoreValue, Simple> const &sc)
{
    p.match = scoreMatch(sc);
    p.mismatch = scoreMismatch(sc);
    p.gap = scoreGapExtend(sc);
    if (p.method == GBA_GAPPED_XDROP && scoreGapOpen(sc) != scoreGapExtend(sc))
        throw std::runtime_error("GappedXDrop needs gap open == gap extend (seeds/seeds_extension.h:792-794)");
}

template <typename TAlphabet, typename TScoreValue, typename TSeqValue, typename TSpec>
void set_seed_score(gba_extend_params &p, std::vector<int32_t> &table,
                    Score<TScoreValue, ScoreMatrix<TSeqValue, TSpec>> const &sc)
{
    const int A = int(ValueSize<TAlphabet>::VALUE);
    table.resize(size_t(A) * A);
    for (int i = 0; i < A; ++i)
        for (int j = 0; j < A; ++j) table[i * A + j] = int32_t(score(sc, TAlphabet(i), TAlphabet(j)));
    p.matrix = table.data();
    p.alphabet_size = A;
    p.gap = scoreGapExtend(sc);
    if (p.method == GBA_GAPPED_XDROP && scoreGapOpen(sc) != scoreGapExtend(sc))
        throw std::runtime_error("GappedXDrop needs gap open == gap extend (seeds/seeds_extension.h:792-794)");
}

// Runs a batch; shared_db: every seed lies on databases[0].
template <typename TConfig>
void run_seeds(String<Seed<Simple, TConfig>> &seeds, Codes const &db, Codes const &qs, bool shared_db,
               gba_extend_params const &p)
{
    const size_t n = length(seeds);
    std::vector<gba_seed> es(n);
    for (size_t k = 0; k < n; ++k) {
        Seed<Simple, TConfig> const &s = seeds[k];
        es[k] = gba_seed{int64_t(beginPositionH(s)), int64_t(beginPositionV(s)), int64_t(endPositionH(s)),
                         int64_t(endPositionV(s)), int64_t(lowerDiagonal(s)), int64_t(upperDiagonal(s))};
    }
    std::vector<int32_t> ids_h(shared_db ? n : 0, 0);
    gba_seed_batch b{};
    b.num_h = int64_t(db.off.size()) - 1;
    b.seq_h = db.seq.data();
    b.off_h = db.off.data();
    b.num_v = int64_t(qs.off.size()) - 1;
    b.seq_v = qs.seq.data();
    b.off_v = qs.off.data();
    b.num_seeds = int64_t(n);
    b.seed_h = shared_db ? ids_h.data() : nullptr;
    check(gba_extend_seeds(context(), &p, &b, es.data(), nullptr), "gba_extend_seeds");
    for (size_t k = 0; k < n; ++k) {
        Seed<Simple, TConfig> &s = seeds[k];
        setBeginPositionH(s, es[k].begin_h);
        setBeginPositionV(s, es[k].begin_v);
        setEndPositionH(s, es[k].end_h);
        setEndPositionV(s, es[k].end_v);
        setLowerDiagonal(s, es[k].lower_diagonal);
        setUpperDiagonal(s, es[k].upper_diagonal);
    }
}

template <typename TSeq>
Codes flatten_one(TSeq const &s)
{
    Codes c;
    c.add(s);
    return c;
}

template <typename TAlphabet, typename TConfig, typename TScore>
void extend_batch(String<Seed<Simple, TConfig>> &seeds, Codes const &db, Codes const &qs, bool shared_db,
                  ExtensionDirection dir, int method, TScore const *sc, int dropOff)
{
    gba_extend_params p{};
    p.method = method;
    p.direction = int32_t(dir);
    p.score_drop_off = dropOff;
    std::vector<int32_t> table;
    if (sc) set_seed_score<TAlphabet>(p, table, *sc);
    run_seeds(seeds, db, qs, shared_db, p);
}

}  // namespace gb300_impl

// Per-seed databases and queries (StringSets).
template <typename TVec, typename TConfig, typename TDb, typename TDbSpec, typename TQ, typename TQSpec>
void extendSeed(ExecutionPolicy<GB300, TVec> const &, String<Seed<Simple, TConfig>> &seeds,
                StringSet<TDb, TDbSpec> const &databases, StringSet<TQ, TQSpec> const &queries,
                ExtensionDirection direction, MatchExtend const &)
{
    typedef typename Value<TQ>::Type TAlphabet;
    gb300_impl::extend_batch<TAlphabet>(seeds, gb300_impl::flatten(databases), gb300_impl::flatten(queries), false,
                                        direction, GBA_MATCH_EXTEND, (Score<int, Simple> const *)nullptr, 0);
}

template <typename TVec, typename TConfig, typename TDb, typename TDbSpec, typename TQ, typename TQSpec,
          typename TScoreValue, typename TScoreSpec, typename TXDropTag>
void extendSeed(ExecutionPolicy<GB300, TVec> const &, String<Seed<Simple, TConfig>> &seeds,
                StringSet<TDb, TDbSpec> const &databases, StringSet<TQ, TQSpec> const &queries,
                ExtensionDirection direction, Score<TScoreValue, TScoreSpec> const &sc, TScoreValue scoreDropOff,
                TXDropTag const &)
{
    static_assert(gb300_impl::is_xdrop_tag<TXDropTag>::value, "x-drop tag must be UnGappedXDrop or GappedXDrop");
    typedef typename Value<TQ>::Type TAlphabet;
    gb300_impl::extend_batch<TAlphabet>(seeds, gb300_impl::flatten(databases), gb300_impl::flatten(queries), false,
                                        direction,
                                        gb300_impl::is_gapped<TXDropTag>::value ? GBA_GAPPED_XDROP
                                                                                    : GBA_UNGAPPED_XDROP,
                                        &sc, int(scoreDropOff));
}

// One database shared by every seed; seeds[k] lies on queries[k].
template <typename TVec, typename TConfig, typename TAlph, typename TDbSpec, typename TQ, typename TQSpec>
void extendSeed(ExecutionPolicy<GB300, TVec> const &, String<Seed<Simple, TConfig>> &seeds,
                String<TAlph, TDbSpec> const &database, StringSet<TQ, TQSpec> const &queries,
                ExtensionDirection direction, MatchExtend const &)
{
    gb300_impl::extend_batch<TAlph>(seeds, gb300_impl::flatten_one(database), gb300_impl::flatten(queries), true,
                                    direction, GBA_MATCH_EXTEND, (Score<int, Simple> const *)nullptr, 0);
}

template <typename TVec, typename TConfig, typename TAlph, typename TDbSpec, typename TQ, typename TQSpec,
          typename TScoreValue, typename TScoreSpec, typename TXDropTag>
void extendSeed(ExecutionPolicy<GB300, TVec> const &, String<Seed<Simple, TConfig>> &seeds,
                String<TAlph, TDbSpec> const &database, StringSet<TQ, TQSpec> const &queries,
                ExtensionDirection direction, Score<TScoreValue, TScoreSpec> const &sc, TScoreValue scoreDropOff,
                TXDropTag const &)
{
    static_assert(gb300_impl::is_xdrop_tag<TXDropTag>::value, "x-drop tag must be UnGappedXDrop or GappedXDrop");
    gb300_impl::extend_batch<TAlph>(seeds, gb300_impl::flatten_one(database), gb300_impl::flatten(queries), true,
                                    direction,
                                    gb300_impl::is_gapped<TXDropTag>::value ? GBA_GAPPED_XDROP
                                                                                : GBA_UNGAPPED_XDROP,
                                    &sc, int(scoreDropOff));
}

// ---- FASTA / FASTQ input: readRecord loop of seq_io/fasta_fastq.h (:265-283, :354-392) ----------
// readRecords(GB300, ids, seqs[, quals], text, Fasta() | Fastq()) reads every record of an
// in-memory text as `while (!atEnd(iter)) readRecord(id, seq[, qual], iter, tag)` does, with seq a
// String<Dna | Dna5 | AminoAcid>; ParseError / UnexpectedEnd are thrown where the reference throws
// them.  FASTA is parsed on the device, FASTQ on the host.
namespace gb300_impl {

template <typename TAlph>
struct ReaderAlphabet;
template <>
struct ReaderAlphabet<Dna> { static const int32_t VALUE = 4; };
template <>
struct ReaderAlphabet<Dna5> { static const int32_t VALUE = 5; };
template <>
struct ReaderAlphabet<AminoAcid> { static const int32_t VALUE = 27; };

template <typename TIdSet, typename TSeqSet, typename TQualSet>
void read_records(bool fastq, TIdSet &ids, TSeqSet &seqs, TQualSet *quals, std::string const &text)
{
    typedef typename Value<TSeqSet>::Type TSeq;
    typedef typename Value<TSeq>::Type TAlph;
    const int64_t n = int64_t(text.size());
    const int64_t rcap = int64_t(std::count(text.begin(), text.end(), fastq ? '@' : '>')) + 1;
    const size_t cap = static_cast<size_t>(rcap);
    std::vector<int64_t> ib(cap), ie(cap), so(cap), qe(cap);
    std::vector<uint8_t> codes(size_t(n) + 1);
    std::vector<char> qual(fastq ? size_t(n) + 1 : 1);
    gba_seq_records r{rcap, n + 1, ib.data(), ie.data(), so.data(), qe.data(), codes.data(),
                      fastq ? qual.data() : nullptr, 0, 0, -1};
    const int rc = fastq ? gba_read_fastq(context(), text.data(), n, ReaderAlphabet<TAlph>::VALUE, &r)
                         : gba_read_fasta(context(), text.data(), n, ReaderAlphabet<TAlph>::VALUE, &r);
    if (rc == GBA_EPARSE) {
        if (r.error_offset >= n) throw UnexpectedEnd();
        throw ParseError("record text not in the format at offset " + std::to_string(r.error_offset));
    }
    check(rc, fastq ? "gba_read_fastq" : "gba_read_fasta");
    for (int64_t k = 0; k < r.num; ++k) {
        appendValue(ids, CharString(text.substr(size_t(ib[k]), size_t(ie[k] - ib[k]))));
        TSeq s;
        resize(s, size_t(so[k + 1] - so[k]));
        for (int64_t i = so[k]; i < so[k + 1]; ++i) s[size_t(i - so[k])] = TAlph(unsigned(codes[size_t(i)]));
        appendValue(seqs, s);
        if (quals) appendValue(*quals, CharString(std::string(qual.data() + so[k], qual.data() + qe[k])));
    }
}

// ---- SAM / BAM output of BamAlignmentRecords (bam_io/write_sam.h:126-217, write_bam.h:100-271) ---

struct RecordArrays {
    std::vector<char> qname, seq_letters, qual, cnames;
    std::vector<int64_t> qoff{0}, coff{0}, soff{0}, quoff{0}, cnoff{0};
    std::vector<uint16_t> flag;
    std::vector<int32_t> rid, pos, rnext, pnext, tlen;
    std::vector<uint8_t> mapq, seq;
    std::vector<uint32_t> cigar;
    gba_sam_records rec{};
};

template <typename TNameStore, typename TNameStoreCache, typename TStorageSpec>
void record_arrays(RecordArrays &a, String<BamAlignmentRecord> const &records,
                   BamIOContext<TNameStore, TNameStoreCache, TStorageSpec> &context)
{
    static char const ops[] = "MIDNSHP=X";
    for (size_t k = 0; k < length(records); ++k) {
        BamAlignmentRecord const &r = records[k];
        if (!empty(r.tags)) throw std::runtime_error("GB300 SAM/BAM output: records with tags are not supported");
        for (size_t i = 0; i < length(r.qName); ++i) a.qname.push_back(r.qName[i]);
        a.qoff.push_back(int64_t(a.qname.size()));
        a.flag.push_back(uint16_t(r.flag));
        a.rid.push_back(r.rID);
        a.pos.push_back(r.beginPos);
        a.mapq.push_back(uint8_t(r.mapQ));
        for (size_t i = 0; i < length(r.cigar); ++i) {
            char const *op = std::strchr(ops, r.cigar[i].operation);
            if (!op || !*op) throw std::runtime_error("GB300 SAM/BAM output: CIGAR operation outside MIDNSHP=X");
            a.cigar.push_back((uint32_t(r.cigar[i].count) << 4) | uint32_t(op - ops));
        }
        a.coff.push_back(int64_t(a.cigar.size()));
        a.rnext.push_back(r.rNextId);
        a.pnext.push_back(r.pNext);
        a.tlen.push_back(r.tLen);
        for (size_t i = 0; i < length(r.seq); ++i) a.seq.push_back(uint8_t(ordValue(r.seq[i])));
        a.soff.push_back(int64_t(a.seq.size()));
        for (size_t i = 0; i < length(r.qual); ++i) a.qual.push_back(r.qual[i]);
        a.quoff.push_back(int64_t(a.qual.size()));
    }
    for (size_t c = 0; c < length(contigNames(context)); ++c) {
        for (size_t i = 0; i < length(contigNames(context)[c]); ++i) a.cnames.push_back(contigNames(context)[c][i]);
        a.cnoff.push_back(int64_t(a.cnames.size()));
    }
    a.seq_letters.assign(32, 'N');
    for (unsigned v = 0; v < 16; ++v) a.seq_letters[v] = convert<char>(Iupac(v));   // IupacString letters
    for (auto *v : {&a.qname, &a.qual, &a.cnames}) v->push_back(0);
    a.seq.push_back(0);
    a.cigar.push_back(0);
    const int64_t n = int64_t(length(records));
    a.rec = gba_sam_records{n, a.qname.data(), a.qoff.data(), a.flag.data(), a.rid.data(), a.pos.data(), a.mapq.data(),
                            a.cigar.data(), a.coff.data(), a.rnext.data(), a.pnext.data(), a.tlen.data(),
                            a.seq.data(), a.soff.data(), a.seq_letters.data(), a.qual.data(), a.quoff.data(),
                            a.cnames.data(), a.cnoff.data(), int64_t(length(contigNames(context)))};
}

}  // namespace gb300_impl

template <typename TVec, typename TIdSet, typename TSeqSet>
void readRecords(ExecutionPolicy<GB300, TVec> const &, TIdSet &ids, TSeqSet &seqs, std::string const &text, Fasta)
{
    gb300_impl::read_records(false, ids, seqs, static_cast<TIdSet *>(nullptr), text);
}

template <typename TVec, typename TIdSet, typename TSeqSet, typename TQualSet>
void readRecords(ExecutionPolicy<GB300, TVec> const &, TIdSet &ids, TSeqSet &seqs, TQualSet &quals,
                 std::string const &text, Fastq)
{
    gb300_impl::read_records(true, ids, seqs, &quals, text);
}

// Appends the SAM lines of the records (no header) to target, as write(target, record, context,
// Sam()) for each record does.
template <typename TVec, typename TTarget, typename TNameStore, typename TNameStoreCache, typename TStorageSpec>
void write(ExecutionPolicy<GB300, TVec> const &, TTarget &target, String<BamAlignmentRecord> const &records,
           BamIOContext<TNameStore, TNameStoreCache, TStorageSpec> &context, Sam const &)
{
    gb300_impl::RecordArrays a;
    gb300_impl::record_arrays(a, records, context);
    std::vector<int64_t> off(length(records) + 1);
    int rc = gba_format_sam(gb300_impl::context(), &a.rec, nullptr, 0, off.data());
    if (rc != GBA_ECAPACITY) gb300_impl::check(rc, "gba_format_sam");
    std::vector<char> text(size_t(off.back()) + 1);
    gb300_impl::check(gba_format_sam(gb300_impl::context(), &a.rec, text.data(), int64_t(text.size()), off.data()),
                      "gba_format_sam");
    for (int64_t i = 0; i < off.back(); ++i) appendValue(target, text[size_t(i)]);
}

// Appends the BAM record blocks (uncompressed, no header) to target, as write(target, record,
// context, Bam()) for each record does.
template <typename TVec, typename TTarget, typename TNameStore, typename TNameStoreCache, typename TStorageSpec>
void write(ExecutionPolicy<GB300, TVec> const &, TTarget &target, String<BamAlignmentRecord> const &records,
           BamIOContext<TNameStore, TNameStoreCache, TStorageSpec> &context, Bam const &)
{
    gb300_impl::RecordArrays a;
    gb300_impl::record_arrays(a, records, context);
    std::vector<int64_t> off(length(records) + 1);
    int rc = gba_format_bam(gb300_impl::context(), &a.rec, nullptr, 0, off.data());
    if (rc != GBA_ECAPACITY) gb300_impl::check(rc, "gba_format_bam");
    std::vector<char> bytes(size_t(off.back()) + 1);
    gb300_impl::check(gba_format_bam(gb300_impl::context(), &a.rec, bytes.data(), int64_t(bytes.size()), off.data()),
                      "gba_format_bam");
    for (int64_t i = 0; i < off.back(); ++i) appendValue(target, bytes[size_t(i)]);
}

}  // namespace seqan2

#endif  // SEQAN_GB300_SEQAN_H_
