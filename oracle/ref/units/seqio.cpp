// FASTA / FASTQ records through the UNMODIFIED reference's readRecord (test infrastructure, see
// ref_common.h): the loop `while (!atEnd(iter)) readRecord(id, seq, qual, iter, Fasta|Fastq)` over
// an in-memory stream (seq_io/fasta_fastq.h:265-283, :354-392), seq a String<Dna|Dna5|AminoAcid>,
// qual a CharString.
#include "../ref_common.h"

#include <seqan/seq_io.h>

#include <sstream>
#include <string>

namespace seqan_ref {
namespace {

void put_u32(std::string & out, uint32_t v) { out.append(reinterpret_cast<const char *>(&v), 4); }

template <typename TAlph>
int64_t read_all(int32_t format, const char * text, int64_t n, char * out, int64_t cap, int64_t * nrec)
{
    std::istringstream ss(std::string(text, size_t(n)));
    auto iter = directionIterator(ss, Input());
    CharString id, qual;
    String<TAlph> seq;
    std::string buf;
    *nrec = 0;
    try {
        while (!atEnd(iter)) {
            if (format == 1) readRecord(id, seq, qual, iter, Fastq());
            else if (format == 2) readRecord(id, seq, qual, iter, Raw());
            else readRecord(id, seq, qual, iter, Fasta());
            put_u32(buf, uint32_t(length(id)));
            buf.append(toCString(id), length(id));
            put_u32(buf, uint32_t(length(seq)));
            for (size_t i = 0; i < length(seq); ++i) buf.push_back(char(ordValue(seq[i])));
            put_u32(buf, uint32_t(length(qual)));
            buf.append(toCString(qual), length(qual));
            ++*nrec;
        }
    } catch (UnexpectedEnd const &) {
        return -2;
    } catch (ParseError const &) {
        return -1;
    }
    if (int64_t(buf.size()) > cap) return -3;
    memcpy(out, buf.data(), buf.size());
    return int64_t(buf.size());
}

template <typename TAlph>
void char_table(int16_t * out)
{
    IsInAlphabet<TAlph> in;
    for (int c = 0; c < 256; ++c) {
        const char ch = char(c);
        out[c] = in(ch) ? int16_t(ordValue(TAlph(ch))) : int16_t(-1);
    }
}

}  // namespace
}  // namespace seqan_ref

extern "C" {

// Reads every record of text[0..n) (format 0 FASTA, 1 FASTQ; alphabet 4 Dna, 5 Dna5, 27
// AminoAcid) and serialises them to out as (u32 id length, id, u32 residues, codes, u32 quality
// length, qualities) per record.  Returns the bytes written, -1 on ParseError, -2 on
// UnexpectedEnd, -3 when cap is too small; *nrec = records read before the return.
int64_t ref_read_records(int32_t format, int32_t alphabet, const char * text, int64_t n, char * out, int64_t cap,
                         int64_t * nrec)
{
    if (alphabet == 27) return seqan_ref::read_all<AminoAcid>(format, text, n, out, cap, nrec);
    if (alphabet == 4) return seqan_ref::read_all<Dna>(format, text, n, out, cap, nrec);
    return seqan_ref::read_all<Dna5>(format, text, n, out, cap, nrec);
}

// For each of the 256 characters: the residue code TAlph(c) when IsInAlphabet<TAlph>(c), else -1.
void ref_char_table(int32_t alphabet, int16_t * out)
{
    if (alphabet == 27) seqan_ref::char_table<AminoAcid>(out);
    else if (alphabet == 4) seqan_ref::char_table<Dna>(out);
    else seqan_ref::char_table<Dna5>(out);
}

}  // extern "C"
