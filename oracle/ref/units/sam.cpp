// SAM records through the UNMODIFIED reference's writer (test infrastructure, see ref_common.h):
// BamAlignmentRecord fields from arrays, written by write(target, record, context, Sam())
// (bam_io/write_sam.h:126-217) with a BamIOContext that names the contigs.
#include "../ref_common.h"

#include <seqan/bam_io.h>

extern "C" {

// Fields of record k: qname chars [qoff[k], qoff[k+1]), flag, rid, pos (0-based), mapq, cigar
// (BAM-packed length << 4 | op into "MIDNSHP=X") [coff[k], coff[k+1]), rnext, pnext, tlen, seq
// letters [soff[k], soff[k+1]), qual [quoff[k], quoff[k+1]), BAM tag bytes [toff[k], toff[k+1]) (toff
// NULL: none).  Contig names back to back.  Writes
// the SAM lines to out (NUL-terminated if it fits); returns their total length.
int64_t ref_write_sam(int64_t n, const char * qname, const int64_t * qoff, const uint16_t * flag,
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
    CharString text;
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
        write(text, r, context, Sam());
    }
    const int64_t len = int64_t(length(text));
    if (len < cap)
    {
        for (int64_t i = 0; i < len; ++i) out[i] = text[i];
        out[len] = 0;
    }
    return len;
}

}  // extern "C"
