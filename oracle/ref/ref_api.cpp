// ref_api.cpp -- extern "C" entry points of the reference wrapper (test infrastructure).
// Each call is routed to the translation unit that instantiated that call shape; a shape
// that no unit instantiated returns -1 (the tests only use instantiated shapes).
#include "ref_common.h"

#include <map>
#include <mutex>

namespace seqan_ref {

static std::map<int, void *> & registry()
{
    static std::map<int, void *> r;
    return r;
}

void register_unit(int key, void * fn)
{
    registry()[key] = fn;
}

static void * find(int kind, ref_params const & p)
{
    auto it = registry().find(make_key(kind, p));
    return it == registry().end() ? nullptr : it->second;
}

}  // namespace seqan_ref

extern "C" {

int ref_batch_score(const ref_params * pp, int64_t n, const uint8_t * sh, const int64_t * oh,
                    const uint8_t * sv, const int64_t * ov, int32_t * out)
{
    void * f = seqan_ref::find(0, *pp);
    if (!f) return -1;
    return reinterpret_cast<seqan_ref::score_fn>(f)(*pp, n, sh, oh, sv, ov, out);
}

int ref_batch_gaps(const ref_params * pp, int64_t n, const uint8_t * sh, const int64_t * oh,
                   const uint8_t * sv, const int64_t * ov, ref_gaps_out * out,
                   char * rows, const int64_t * row_off, char * cigar, int64_t cigar_stride)
{
    void * f = seqan_ref::find(1, *pp);
    if (!f) return -1;
    return reinterpret_cast<seqan_ref::gaps_fn>(f)(*pp, n, sh, oh, sv, ov, out, rows, row_off,
                                                   cigar, cigar_stride);
}

int ref_pair_segments(const ref_params * pp, const uint8_t * h, int32_t m, const uint8_t * v, int32_t n,
                      int32_t * score, uint32_t * segs, int32_t cap, int32_t * nseg)
{
    void * f = seqan_ref::find(2, *pp);
    if (!f) return -1;
    return reinterpret_cast<seqan_ref::seg_fn>(f)(*pp, h, m, v, n, score, segs, cap, nseg);
}

// DynamicGaps cells (kind 3): score and raw TraceSegment_ list of the single-pair DP.
int ref_dynamic_segments(const ref_params * pp, const uint8_t * h, int32_t m, const uint8_t * v, int32_t n,
                         int32_t * score, uint32_t * segs, int32_t cap, int32_t * nseg)
{
    void * f = seqan_ref::find(3, *pp);
    if (!f) return -1;
    return reinterpret_cast<seqan_ref::seg_fn>(f)(*pp, h, m, v, n, score, segs, cap, nseg);
}

// 1 if the call shape is instantiated.
int ref_has_shape(int32_t kind, const ref_params * pp)
{
    return seqan_ref::find(kind, *pp) != nullptr;
}

// Blosum62 over the 27-letter AminoAcid alphabet, row = first argument of score().
void ref_blosum62(int32_t * out)
{
    Score<int, ScoreMatrix<AminoAcid, ScoreSpecBlosum62>> sc;
    for (unsigned i = 0; i < 27; ++i)
        for (unsigned j = 0; j < 27; ++j)
            out[i * 27 + j] = score(sc, AminoAcid(i), AminoAcid(j));
}

// Character -> ordValue conversion of the reference's alphabets (0 = Dna5, 1 = AminoAcid, 2 = Dna).
void ref_encode(int32_t alphabet, const char * in, int64_t n, uint8_t * out)
{
    for (int64_t i = 0; i < n; ++i)
    {
        if (alphabet == 0)
            out[i] = static_cast<uint8_t>(ordValue(Dna5(in[i])));
        else if (alphabet == 1)
            out[i] = static_cast<uint8_t>(ordValue(AminoAcid(in[i])));
        else
            out[i] = static_cast<uint8_t>(ordValue(Dna(in[i])));
    }
}

// The widest SIMD vector (bytes) the reference was compiled for; 0 = scalar build.
int32_t ref_simd_bytes()
{
#if defined(SEQAN_SIMD_ENABLED) && defined(SEQAN_SIZEOF_MAX_VECTOR)
    return SEQAN_SIZEOF_MAX_VECTOR;
#else
    return 0;
#endif
}

}  // extern "C"
