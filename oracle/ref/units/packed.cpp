// String<TValue, Packed<>> host words through the UNMODIFIED reference (test infrastructure, see
// ref_common.h): the layout the packed upload reads (sequence/string_packed.h).
#include "../ref_common.h"

namespace seqan_ref {
namespace {

template <typename TAlph>
int64_t pack_one(const uint8_t * codes, int64_t n, uint64_t * out, int64_t cap)
{
    String<TAlph, Packed<>> s;
    resize(s, n);
    for (int64_t i = 0; i < n; ++i) assignValue(s, i, TAlph(unsigned(codes[i])));
    auto const & h = host(s);
    const int64_t words = int64_t(length(h));
    for (int64_t w = 0; w < words && w < cap; ++w) out[w] = h[w].i;
    return words;
}

}  // namespace
}  // namespace seqan_ref

extern "C" {

// Packs codes[0..n) as String<Dna|Dna5|AminoAcid, Packed<>> (alphabet 2 / 0 / 1) and copies its
// host words (the length word, then the data words) to out; returns the number of host words.
int64_t ref_pack_string(int32_t alphabet, const uint8_t * codes, int64_t n, uint64_t * out, int64_t cap)
{
    if (alphabet == 1) return seqan_ref::pack_one<AminoAcid>(codes, n, out, cap);
    if (alphabet == 2) return seqan_ref::pack_one<Dna>(codes, n, out, cap);
    return seqan_ref::pack_one<Dna5>(codes, n, out, cap);
}

// BitsPerValue of the reference's alphabets (2 Dna, 3 Dna5, 5 AminoAcid).
int32_t ref_bits_per_value(int32_t alphabet)
{
    if (alphabet == 1) return int32_t(BitsPerValue<AminoAcid>::VALUE);
    if (alphabet == 2) return int32_t(BitsPerValue<Dna>::VALUE);
    return int32_t(BitsPerValue<Dna5>::VALUE);
}

}  // extern "C"
