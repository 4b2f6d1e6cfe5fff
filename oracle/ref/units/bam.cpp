// BAM records through the UNMODIFIED reference's writer (test infrastructure, see ref_common.h):
// BamAlignmentRecord fields from arrays, written by write(target, record, context, Bam())
// (bam_io/write_bam.h:100-271): the uncompressed record blocks a BGZF stream would carry.
#include "../ref_common.h"

#include <seqan/bam_io.h>

extern "C" {

// Fields as ref_write_sam takes them (seq as letters).  Writes the records' bytes to out when they
// fit in cap; returns their total length.
int64_t ref_write_bam(int64_t n, const char * qname, const int64_t * qoff, const uint16_t * flag,
                      const int32_t * rid, const int32_t * pos, const uint8_t * mapq, const uint32_t * cigar,
                      const int64_t * coff, const int32_t * rnext, const int32_t * pnext, const int32_t * tlen,
                      const char * seq, const int64_t * soff, const char * qual, const int64_t * quoff,
                      int64_t ncontigs, const char * cnames, const int64_t * cnoff, const char * tags,
                      const int64_t * toff, char * out, int64_t cap)
{
    typedef StringSet<CharString> TNameStore;
    typedef NameStoreCache<TNameStore> TNameStoreCache;
    TNameStore names;
    for (int64_t c = 0; c < ncontigs; ++c)
        appendValue(names, CharString(std::string(cnames + cnoff[c], cnames + cnoff[c + 1])));
    TNameStoreCache cache(names);
    BamIOContext<TNameStore, TNameStoreCache> context(names, cache);
    CharString bytes;
    static char const ops[] = "MIDNSHP=X";
    for (int64_t k = 0; k < n; ++k)
    {
        BamAlignmentRecord r;
        r.qName = std::string(qname + qoff[k], qname + qoff[k + 1]);
        r.flag = flag[k];
        r.rID = rid[k];
        r.beginPos = pos[k];
        r.mapQ = mapq[k];
        for (int64_t i = coff[k]; i < coff[k + 1]; ++i)
            appendValue(r.cigar, CigarElement<>(ops[cigar[i] & 15u], cigar[i] >> 4));
        r.rNextId = rnext[k];
        r.pNext = pnext[k];
        r.tLen = tlen[k];
        r.seq = std::string(seq + soff[k], seq + soff[k + 1]);
        r.qual = std::string(qual + quoff[k], qual + quoff[k + 1]);
        if (toff) r.tags = std::string(tags + toff[k], tags + toff[k + 1]);
        write(bytes, r, context, Bam());
    }
    const int64_t len = int64_t(length(bytes));
    if (len <= cap)
        for (int64_t i = 0; i < len; ++i) out[i] = bytes[i];
    return len;
}

// ordValue(Iupac(c)) for each of the 256 characters.
void ref_iupac_table(uint8_t * out)
{
    for (int c = 0; c < 256; ++c) out[c] = uint8_t(ordValue(Iupac(char(c))));
}

}  // extern "C"
