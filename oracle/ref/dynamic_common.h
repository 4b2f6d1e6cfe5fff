#pragma once
// dynamic_common.h -- DynamicGaps cells through the UNMODIFIED reference (test infrastructure, see
// ref_common.h): the single-pair DP _setUpAndRunAlignment (align/dp_setup.h:266-326) with the
// DynamicGaps gap-cost tag (align/dp_cell_dynamic.h, align/dp_formula_dynamic.h) instead of
// LinearGaps / AffineGaps.  No public alignment function selects this cell type; the reference's own
// DP tests reach it the same way.  Returns the score and the raw TraceSegment_ list.
#include "ref_common.h"

namespace seqan_ref {

template <bool T, bool L, bool R, bool B, typename TScoreValue, typename TAlph, bool B62>
int run_dynamic(ref_params const & p, const uint8_t * h, int32_t m, const uint8_t * v, int32_t n,
                int32_t * score_out, uint32_t * segs, int32_t cap, int32_t * nseg)
{
    String<TAlph> sH, sV;
    resize(sH, m);
    resize(sV, n);
    for (int32_t i = 0; i < m; ++i) assignValue(sH, i, TAlph(static_cast<unsigned>(h[i])));
    for (int32_t i = 0; i < n; ++i) assignValue(sV, i, TAlph(static_cast<unsigned>(v[i])));
    auto score = ScoreOf<TScoreValue, TAlph, B62>::make(p);
    String<TraceSegment_<unsigned, unsigned>> trace;
    DPScoutState_<Default> state;
    TScoreValue res;
    if (p.mode == 0)
    {
        typedef typename SubstituteAlignConfig_<AlignConfig<T, L, R, B>>::Type TFree;
        typedef AlignConfig2<DPGlobal, DPBandConfig<BandOff>, TFree> TCfg;
        res = _setUpAndRunAlignment(trace, state, sH, sV, score, TCfg(), DynamicGaps());
    }
    else
    {
        typedef AlignConfig2<DPLocal, DPBandConfig<BandOff>, FreeEndGaps_<>> TCfg;
        res = _setUpAndRunAlignment(trace, state, sH, sV, score, TCfg(), DynamicGaps());
    }
    *score_out = static_cast<int32_t>(res);
    const int32_t ns = static_cast<int32_t>(length(trace));
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

