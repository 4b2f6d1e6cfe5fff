// Banded chain alignment through the UNMODIFIED reference (test infrastructure, see ref_common.h):
// bandedChainAlignment(align, seedChain, scoreAnchor, scoreGap, alignConfig, bandExtension)
// (seeds/banded_chain_alignment.h:184-214) and the TraceSegment_ lists it is built from
// (_setupAndRunBandedChainAlignment, seeds/banded_chain_alignment_profile.h).
#include "../ref_common.h"

#include <seqan/align.h>
#include <seqan/seeds.h>

#include <sstream>
#include <stdexcept>
#include <string>
#include <vector>

#include <omp.h>

namespace seqan_ref {
namespace {

template <bool T, bool L, bool R, bool B>
int chain_run(Score<int, Simple> const & sa, Score<int, Simple> const & sg, int32_t band_ext, const uint8_t * h,
              int64_t m, const uint8_t * v, int64_t n, int32_t n_seeds, const int32_t * seeds, int32_t * score,
              uint32_t * segs, int32_t seg_cap, int32_t * n_segs, int32_t * n_traces, char * out_rows, int64_t cap)
{
    typedef String<Dna5> TStr;
    TStr hs, vs;
    resize(hs, m);
    resize(vs, n);
    for (int64_t i = 0; i < m; ++i) assignValue(hs, i, Dna5(unsigned(h[i])));
    for (int64_t i = 0; i < n; ++i) assignValue(vs, i, Dna5(unsigned(v[i])));
    String<Seed<Simple>> chain;
    for (int32_t k = 0; k < n_seeds; ++k)
        appendValue(chain, Seed<Simple>(seeds[4 * k], seeds[4 * k + 1], seeds[4 * k + 2], seeds[4 * k + 3]));

    // The traces the public call adapts its rows from (the same call it makes).
    typedef StringSet<String<TraceSegment_<size_t, size_t>>> TTraceSet;
    TTraceSet traces;
    *score = _setupAndRunBandedChainAlignment(traces, chain, hs, vs, sa, sg, AlignConfig<T, L, R, B>(),
                                              unsigned(band_ext), GapsLeft());
    *n_traces = int32_t(length(traces));
    *n_segs = 0;
    if (!empty(traces))
    {
        String<TraceSegment_<size_t, size_t>> const & t = traces[0];
        if (int64_t(length(t)) > seg_cap) return -1;
        for (size_t q = 0; q < length(t); ++q)
        {
            segs[4 * q + 0] = uint32_t(t[q]._horizontalBeginPos);
            segs[4 * q + 1] = uint32_t(t[q]._verticalBeginPos);
            segs[4 * q + 2] = uint32_t(t[q]._length);
            segs[4 * q + 3] = uint32_t(t[q]._traceValue);
        }
        *n_segs = int32_t(length(t));
    }

    // The public call itself: score and rows.
    Align<TStr> align;
    resize(rows(align), 2);
    assignSource(row(align, 0), hs);
    assignSource(row(align, 1), vs);
    int s2 = bandedChainAlignment(align, chain, sa, sg, AlignConfig<T, L, R, B>(), unsigned(band_ext));
    if (s2 != *score) return -2;
    std::stringstream s0, s1;
    s0 << row(align, 0);
    s1 << row(align, 1);
    std::string text = s0.str() + "\n" + s1.str() + "\n";
    if (int64_t(text.size()) + 1 > cap) return -1;
    std::memcpy(out_rows, text.c_str(), text.size() + 1);
    return 0;
}

typedef int (*chain_fn)(Score<int, Simple> const &, Score<int, Simple> const &, int32_t, const uint8_t *, int64_t,
                        const uint8_t *, int64_t, int32_t, const int32_t *, int32_t *, uint32_t *, int32_t, int32_t *,
                        int32_t *, char *, int64_t);

// AlignConfig<TOP, LEFT, RIGHT, BOTTOM> from the free-end bits TOP=1 LEFT=2 RIGHT=4 BOTTOM=8.
const chain_fn kChain[16] = {
    chain_run<false, false, false, false>, chain_run<true, false, false, false>,
    chain_run<false, true, false, false>,  chain_run<true, true, false, false>,
    chain_run<false, false, true, false>,  chain_run<true, false, true, false>,
    chain_run<false, true, true, false>,   chain_run<true, true, true, false>,
    chain_run<false, false, false, true>,  chain_run<true, false, false, true>,
    chain_run<false, true, false, true>,   chain_run<true, true, false, true>,
    chain_run<false, false, true, true>,   chain_run<true, false, true, true>,
    chain_run<false, true, true, true>,    chain_run<true, true, true, true>,
};

}  // namespace
}  // namespace seqan_ref

extern "C" {

// One banded chain alignment of Dna5 codes.  sa / sg: (match, mismatch, gap_extend, gap_open) of
// the anchor and gap scoring schemes; seeds: n_seeds x (beginH, beginV, endH, endV) in chain
// order.  Outputs: the score, the first trace of the trace set as (h, v, length, trace value)
// segments in the reference's order, the number of traces, and the two rows as text lines.
// Returns 0, 1 when the reference throws (no glue point between two grids' traces), -1 when an
// output does not fit, -2 when the public call's score differs from the trace-set call's.
int ref_banded_chain(const int32_t * sa, const int32_t * sg, int32_t free_ends, int32_t band_ext, const uint8_t * h,
                     int64_t m, const uint8_t * v, int64_t n, int32_t n_seeds, const int32_t * seeds, int32_t * score,
                     uint32_t * segs, int32_t seg_cap, int32_t * n_segs, int32_t * n_traces, char * out_rows,
                     int64_t cap)
{
    Score<int, Simple> a(sa[0], sa[1], sa[2], sa[3]);
    Score<int, Simple> g(sg[0], sg[1], sg[2], sg[3]);
    try
    {
        return seqan_ref::kChain[free_ends & 15](a, g, band_ext, h, m, v, n, n_seeds, seeds, score, segs, seg_cap,
                                                 n_segs, n_traces, out_rows, cap);
    }
    catch (std::logic_error const &)
    {
        return 1;
    }
}

// A batch of chains (codes concatenated with offsets, seeds with per-chain offsets) on `threads`
// OpenMP threads (<= 0: all), as the reference's per-pair calls: scores and statuses per chain.
int ref_banded_chain_batch(const int32_t * sa, const int32_t * sg, int32_t free_ends, int32_t band_ext,
                           int64_t n_pairs, const uint8_t * seq_h, const int64_t * off_h, const uint8_t * seq_v,
                           const int64_t * off_v, const int32_t * seeds, const int64_t * seed_off, int32_t * score,
                           int32_t * status, int32_t threads)
{
    Score<int, Simple> a(sa[0], sa[1], sa[2], sa[3]);
    Score<int, Simple> g(sg[0], sg[1], sg[2], sg[3]);
    const int nt = threads > 0 ? threads : omp_get_max_threads();
#pragma omp parallel num_threads(nt)
    {
        std::vector<uint32_t> segs;
        std::vector<char> rows;
#pragma omp for schedule(dynamic, 4)
        for (int64_t k = 0; k < n_pairs; ++k)
        {
            const int64_t m = off_h[k + 1] - off_h[k], n = off_v[k + 1] - off_v[k];
            const int64_t cap = 4 * (m + n) + 64;
            segs.resize(size_t(4 * cap));
            rows.resize(size_t(4 * (m + n) + 16));
            int32_t ns = 0, ntr = 0;
            try
            {
                status[k] = seqan_ref::kChain[free_ends & 15](
                    a, g, band_ext, seq_h + off_h[k], m, seq_v + off_v[k], n, int32_t(seed_off[k + 1] - seed_off[k]),
                    seeds + 4 * seed_off[k], &score[k], segs.data(), int32_t(cap), &ns, &ntr, rows.data(),
                    int64_t(rows.size()));
            }
            catch (std::logic_error const &)
            {
                status[k] = 1;
            }
        }
    }
    return 0;
}

}  // extern "C"
