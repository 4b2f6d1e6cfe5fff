// sam_host.cuh -- gba_format_sam: SAM lines of alignment records, formatted on the device as the
// reference's SAM writer formats a BamAlignmentRecord (bam_io/write_sam.h:126-217); included at
// the end of engine.cu.
//
// A length pass (one thread per record) sizes every line, a device scan places them, and a
// write pass (one warp per record) writes each line: the numeric fields and CIGAR operations by one
// lane, the name, sequence and qualities by all lanes.
#pragma once

namespace gba {

struct SamArgs {
    int64_t num;
    const char *qname;
    const int64_t *qname_off;
    const uint16_t *flag;
    const int32_t *ref_id, *pos, *next_ref_id, *next_pos, *tlen;
    const uint8_t *mapq;
    const uint32_t *cigar;
    const int64_t *cigar_off;
    const uint8_t *seq;
    const int64_t *seq_off;
    const char *letters;        // 32 letters for the residue codes
    const char *qual;
    const int64_t *qual_off;    // null: every qual is '*'
    const char *cnames;
    const int64_t *cname_off;
    int64_t num_contigs;
    const char *tags;           // BAM-form tag bytes of every record, back to back
    const int64_t *tags_off;    // null: no record has tags
};

__device__ __forceinline__ int dec_digits_u(uint64_t v)
{
    int d = 1;
    while (v >= 10) {
        v /= 10;
        ++d;
    }
    return d;
}

__device__ __forceinline__ int dec_len(int64_t v) { return v < 0 ? 1 + dec_digits_u(uint64_t(-v)) : dec_digits_u(uint64_t(v)); }

__device__ __forceinline__ char *dec_write(char *p, int64_t v)
{
    if (v < 0) {
        *p++ = '-';
        v = -v;
    }
    const int d = dec_digits_u(uint64_t(v));
    for (int i = d - 1; i >= 0; --i) {
        p[i] = char('0' + v % 10);
        v /= 10;
    }
    return p + d;
}

// --- tags: appendTagsBamToSam (bam_io/bam_sam_conversion.h:250-360) ---------------------------
__host__ __device__ __forceinline__ int tag_size(char t)
{
    switch (t) {
    case 'A': case 'c': case 'C': return 1;
    case 's': case 'S': return 2;
    case 'i': case 'I': case 'f': return 4;
    default: return 0;
    }
}

__host__ __device__ __forceinline__ int64_t tag_value(const char *q, char t)
{
    const unsigned char *u = reinterpret_cast<const unsigned char *>(q);
    const uint32_t v = uint32_t(u[0]) | (uint32_t(u[1]) << 8) | (uint32_t(u[2]) << 16) | (uint32_t(u[3]) << 24);
    switch (t) {
    case 'c': return int8_t(u[0]);
    case 'C': return u[0];
    case 's': return int16_t(uint16_t(u[0] | (u[1] << 8)));
    case 'S': return uint16_t(u[0] | (u[1] << 8));
    case 'i': return int32_t(v);
    default: return v;   // 'I'
    }
}

// A float tag value as C's printf "%g" prints the value (the reference's appendNumber(float),
// basic/basic_stream.h:1145-1155): six significant digits, correctly rounded with ties to even,
// %e style when the decimal exponent is below -4 or at least 6, trailing zeros removed; "inf",
// "nan" with the sign.  The value M * 2^E is written exactly as D * 10^-k (D = M * 5^k for
// E = -k < 0, D = M * 2^E otherwise) in 32-bit limbs, D's decimal digits are produced by
// division by 10^9, and the rounding works on those digits.  w == nullptr only counts.
__host__ __device__ inline int tag_float_text(uint32_t bits, char *w)
{
    int n = 0;
    auto put = [&](char c) {
        if (w) w[n] = c;
        ++n;
    };
    const uint32_t ex = (bits >> 23) & 0xffu, fr = bits & 0x7fffffu;
    if (bits >> 31) put('-');
    if (ex == 255) {
        const char *t = fr ? "nan" : "inf";
        for (int i = 0; i < 3; ++i) put(t[i]);
        return n;
    }
    const uint32_t M = ex ? (fr | 0x800000u) : fr;
    const int E = ex ? int(ex) - 150 : -149;
    if (M == 0) {
        put('0');
        return n;
    }
    uint32_t D[13];   // M * 5^149 < 2^370
    int nl = 1, k = 0;
    D[0] = M;
    auto mul = [&](uint32_t f) {
        uint64_t c = 0;
        for (int i = 0; i < nl; ++i) {
            const uint64_t t = uint64_t(D[i]) * f + c;
            D[i] = uint32_t(t);
            c = t >> 32;
        }
        if (c) D[nl++] = uint32_t(c);
    };
    if (E >= 0) {
        for (int e = E; e > 0; e -= 16) mul(1u << (e < 16 ? e : 16));
    } else {
        k = -E;
        for (int e = k; e > 0; e -= 13) {
            uint32_t f = 1;
            for (int i = 0; i < (e < 13 ? e : 13); ++i) f *= 5u;
            mul(f);
        }
    }
    // decimal digits of D, most significant first
    char dig[120];
    int nd = 0;
    {
        char rev[126];
        int nr = 0;
        while (nl > 0) {
            uint64_t r = 0;
            for (int i = nl - 1; i >= 0; --i) {
                const uint64_t t = (r << 32) | D[i];
                D[i] = uint32_t(t / 1000000000u);
                r = t % 1000000000u;
            }
            while (nl > 0 && D[nl - 1] == 0) --nl;
            for (int q = 0; q < 9; ++q) {
                rev[nr++] = char('0' + r % 10);
                r /= 10;
            }
        }
        while (nr > 1 && rev[nr - 1] == '0') --nr;
        for (int i = nr - 1; i >= 0; --i) dig[nd++] = rev[i];
    }
    int X = nd - k - 1;   // decimal exponent of the first digit
    char s[6];
    for (int i = 0; i < 6; ++i) s[i] = i < nd ? dig[i] : '0';
    if (nd > 6) {
        bool up;
        if (dig[6] != '5') {
            up = dig[6] > '5';
        } else {
            bool rest = false;
            for (int i = 7; i < nd; ++i) rest |= dig[i] != '0';
            up = rest || ((s[5] - '0') & 1);
        }
        if (up) {
            int i = 5;
            while (i >= 0 && s[i] == '9') s[i--] = '0';
            if (i >= 0) {
                ++s[i];
            } else {
                s[0] = '1';
                ++X;
            }
        }
    }
    int last = 5;   // last significant digit kept after removing trailing zeros
    while (last > 0 && s[last] == '0') --last;
    if (X < -4 || X >= 6) {
        put(s[0]);
        if (last > 0) {
            put('.');
            for (int i = 1; i <= last; ++i) put(s[i]);
        }
        put('e');
        put(X < 0 ? '-' : '+');
        const int ax = X < 0 ? -X : X;
        put(char('0' + ax / 10));
        put(char('0' + ax % 10));
    } else if (X >= 0) {
        for (int i = 0; i <= X; ++i) put(s[i]);
        if (last > X) {
            put('.');
            for (int i = X + 1; i <= last; ++i) put(s[i]);
        }
    } else {
        put('0');
        put('.');
        for (int i = 0; i < -X - 1; ++i) put('0');
        for (int i = 0; i <= last; ++i) put(s[i]);
    }
    return n;
}

// 0 when t[0, len) are tags the SAM writer formats here; 1 malformed.
inline int tags_check(const char *t, int64_t len)
{
    int64_t i = 0;
    while (i < len) {
        if (i + 3 > len) return 1;
        const char ty = t[i + 2];
        i += 3;
        if (ty == 'Z' || ty == 'H') {
            while (i < len && t[i] != 0) ++i;
            if (i >= len) return 1;
            ++i;
        } else if (ty == 'B') {
            if (i + 5 > len) return 1;
            const char et = t[i];
            const int sz = tag_size(et);
            if (sz == 0 || et == 'A') return 1;
            const int64_t cnt = tag_value(t + i + 1, 'I');
            i += 5;
            if (cnt * sz > len - i) return 1;
            i += cnt * sz;
        } else {
            const int sz = tag_size(ty);
            if (sz == 0 || i + sz > len) return 1;
            i += sz;
        }
    }
    return 0;
}

// The SAM text of checked tags; w == nullptr only counts.
__device__ int64_t sam_tags_text(const char *t, int64_t len, char *w)
{
    int64_t n = 0, i = 0;
    auto put = [&](char c) {
        if (w) w[n] = c;
        ++n;
    };
    auto num = [&](int64_t v) {
        if (w) dec_write(w + n, v);
        n += dec_len(v);
    };
    while (i < len) {
        put(t[i]);
        put(t[i + 1]);
        put(':');
        const char ty = t[i + 2];
        const char lo = (ty >= 'A' && ty <= 'Z') ? char(ty + 32) : ty;
        put((lo == 'c' || lo == 's' || lo == 'i') ? 'i' : ty);
        put(':');
        i += 3;
        if (ty == 'Z' || ty == 'H') {
            while (t[i] != 0) put(t[i++]);
            ++i;
        } else if (ty == 'B') {
            const char et = t[i];
            const int sz = tag_size(et);
            put(et);
            const int64_t cnt = tag_value(t + i + 1, 'I');
            i += 5;
            for (int64_t e = 0; e < cnt; ++e) {
                put(',');
                if (et == 'f') n += tag_float_text(uint32_t(tag_value(t + i, 'I')), w ? w + n : nullptr);
                else num(tag_value(t + i, et));
                i += sz;
            }
        } else if (ty == 'A') {
            put(t[i]);
            i += 1;
        } else if (ty == 'f') {
            n += tag_float_text(uint32_t(tag_value(t + i, 'I')), w ? w + n : nullptr);
            i += 4;
        } else {
            num(tag_value(t + i, ty));
            i += tag_size(ty);
        }
        if (i < len) put('\t');
    }
    return n;
}

__device__ __forceinline__ int64_t contig_len(const SamArgs &a, int32_t id)
{
    return (id < 0 || id >= a.num_contigs) ? 1 : a.cname_off[id + 1] - a.cname_off[id];
}

// Byte length of record k's line, in the writer's field order.
__device__ int64_t sam_line_len(const SamArgs &a, int64_t k)
{
    int64_t n = a.qname_off[k + 1] - a.qname_off[k] + 1;
    n += dec_len(a.flag[k]) + 1;
    n += contig_len(a, a.ref_id[k]) + 1;
    n += dec_len(int64_t(a.pos[k]) + 1) + 1;
    n += dec_len(a.mapq[k]) + 1;
    const int64_t c0 = a.cigar_off[k], c1 = a.cigar_off[k + 1];
    if (c0 == c1) n += 1;
    for (int64_t i = c0; i < c1; ++i) n += dec_len(a.cigar[i] >> 4) + 1;
    n += 1;
    const int32_t rn = a.next_ref_id[k];
    n += (rn < 0 || rn == a.ref_id[k]) ? 1 : contig_len(a, rn);
    n += 1;
    n += dec_len(int64_t(a.next_pos[k]) + 1) + 1;
    n += (a.tlen[k] == 0 ? 1 : dec_len(a.tlen[k])) + 1;
    const int64_t sl = a.seq_off[k + 1] - a.seq_off[k];
    n += (sl == 0 ? 1 : sl) + 1;
    const int64_t ql = a.qual_off ? a.qual_off[k + 1] - a.qual_off[k] : 0;
    n += (ql == 0 ? 1 : ql) + 1;
    if (a.tags_off) {
        const int64_t t0 = a.tags_off[k], tl = a.tags_off[k + 1] - t0;
        if (tl) n += 1 + sam_tags_text(a.tags + t0, tl, nullptr);
    }
    return n;
}

__global__ void __launch_bounds__(128) k_sam_lengths(SamArgs a, int64_t *len)
{
    const int64_t k = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (k < a.num) len[k] = sam_line_len(a, k);
}

__global__ void __launch_bounds__(128) k_sam_write(SamArgs a, const int64_t *line_off, char *out)
{
    const int64_t k = (int64_t(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (k >= a.num) return;
    char *p = out + line_off[k];
    const unsigned FULL = 0xffffffffu;
    // QNAME (all lanes)
    const int64_t q0 = a.qname_off[k], ql = a.qname_off[k + 1] - q0;
    for (int64_t i = lane; i < ql; i += 32) p[i] = a.qname[q0 + i];
    p += ql;
    // FLAG .. TLEN (lane 0), then the others learn where SEQ starts
    int64_t seq_at = 0;
    if (lane == 0) {
        char *w = p;
        *w++ = '\t';
        w = dec_write(w, a.flag[k]);
        *w++ = '\t';
        const int32_t rid = a.ref_id[k];
        if (rid < 0 || rid >= a.num_contigs) {
            *w++ = '*';
        } else {
            for (int64_t i = a.cname_off[rid]; i < a.cname_off[rid + 1]; ++i) *w++ = a.cnames[i];
        }
        *w++ = '\t';
        w = dec_write(w, int64_t(a.pos[k]) + 1);
        *w++ = '\t';
        w = dec_write(w, a.mapq[k]);
        *w++ = '\t';
        const int64_t c0 = a.cigar_off[k], c1 = a.cigar_off[k + 1];
        if (c0 == c1) *w++ = '*';
        for (int64_t i = c0; i < c1; ++i) {
            w = dec_write(w, a.cigar[i] >> 4);
            *w++ = "MIDNSHP=X"[a.cigar[i] & 15u];
        }
        *w++ = '\t';
        const int32_t rn = a.next_ref_id[k];
        if (rn < 0 || rn >= a.num_contigs) {
            *w++ = '*';
        } else if (rn == rid) {
            *w++ = '=';
        } else {
            for (int64_t i = a.cname_off[rn]; i < a.cname_off[rn + 1]; ++i) *w++ = a.cnames[i];
        }
        *w++ = '\t';
        w = dec_write(w, int64_t(a.next_pos[k]) + 1);
        *w++ = '\t';
        if (a.tlen[k] == 0) *w++ = '0';
        else w = dec_write(w, a.tlen[k]);
        *w++ = '\t';
        seq_at = w - p;
    }
    seq_at = __shfl_sync(FULL, seq_at, 0);
    p += seq_at;
    // SEQ, QUAL (all lanes)
    const int64_t s0 = a.seq_off[k], sl = a.seq_off[k + 1] - s0;
    if (sl == 0) {
        if (lane == 0) p[0] = '*';
        p += 1;
    } else {
        for (int64_t i = lane; i < sl; i += 32) p[i] = a.letters[a.seq[s0 + i] & 31];
        p += sl;
    }
    if (lane == 0) p[0] = '\t';
    p += 1;
    const int64_t u0 = a.qual_off ? a.qual_off[k] : 0, ul = a.qual_off ? a.qual_off[k + 1] - u0 : 0;
    if (ul == 0) {
        if (lane == 0) p[0] = '*';
        p += 1;
    } else {
        for (int64_t i = lane; i < ul; i += 32) p[i] = a.qual[u0 + i];
        p += ul;
    }
    if (lane == 0) {
        if (a.tags_off && a.tags_off[k + 1] > a.tags_off[k]) {
            *p++ = '\t';
            p += sam_tags_text(a.tags + a.tags_off[k], a.tags_off[k + 1] - a.tags_off[k], p);
        }
        p[0] = '\n';
    }
}

// --- BAM: write(target, record, context, Bam()) without tags (bam_io/write_bam.h:100-271) --------
// A record is block_size, the 32-byte core (rID, beginPos, l_qname | mapQ << 8 | bin << 16,
// n_cigar | flag << 16, l_qseq, rNextId, pNext, tLen), the name and a NUL, the CIGAR words, the
// sequence as Iupac codes two per byte (high nibble first), the qualities minus '!' (0xFF where
// missing), little-endian.  bin = reg2bin(beginPos, beginPos + max(1, l)) in uint32 arithmetic,
// l the CIGAR's length in the reference (operations other than S, H, I: bam_io/cigar.h:601-612),
// kept to its 16-bit field.

struct BamArgs {
    SamArgs s;
    uint8_t iupac[32];   // Iupac code of each residue code's letter
};

__host__ __device__ __forceinline__ uint32_t bam_reg2bin(uint32_t beg, uint32_t end)
{
    --end;
    if (beg >> 14 == end >> 14) return 4681 + (beg >> 14);
    if (beg >> 17 == end >> 17) return 585 + (beg >> 17);
    if (beg >> 20 == end >> 20) return 73 + (beg >> 20);
    if (beg >> 23 == end >> 23) return 9 + (beg >> 23);
    if (beg >> 26 == end >> 26) return 1 + (beg >> 26);
    return 0;
}

__device__ __forceinline__ void bam_put32(char *p, uint32_t v)
{
    p[0] = char(v & 0xffu);
    p[1] = char((v >> 8) & 0xffu);
    p[2] = char((v >> 16) & 0xffu);
    p[3] = char(v >> 24);
}

__global__ void __launch_bounds__(128) k_bam_lengths(BamArgs b, int64_t *len)
{
    const int64_t k = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (k >= b.s.num) return;
    const int64_t lq = b.s.qname_off[k + 1] - b.s.qname_off[k];
    const int64_t nc = b.s.cigar_off[k + 1] - b.s.cigar_off[k];
    const int64_t ls = b.s.seq_off[k + 1] - b.s.seq_off[k];
    const int64_t lt = b.s.tags_off ? b.s.tags_off[k + 1] - b.s.tags_off[k] : 0;
    len[k] = 36 + lq + 1 + 4 * nc + (ls + 1) / 2 + ls + lt;
}

__global__ void __launch_bounds__(128) k_bam_write(BamArgs b, const int64_t *rec_off, char *out)
{
    __shared__ uint8_t iu[32];
    if (threadIdx.x < 32) iu[threadIdx.x] = b.iupac[threadIdx.x];
    __syncthreads();
    const int64_t k = (int64_t(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (k >= b.s.num) return;
    char *p = out + rec_off[k];
    const int64_t q0 = b.s.qname_off[k], lq = b.s.qname_off[k + 1] - q0;
    const int64_t c0 = b.s.cigar_off[k], nc = b.s.cigar_off[k + 1] - c0;
    const int64_t s0 = b.s.seq_off[k], ls = b.s.seq_off[k + 1] - s0;
    const int64_t u0 = b.s.qual_off ? b.s.qual_off[k] : 0;
    const int64_t lqual = b.s.qual_off ? b.s.qual_off[k + 1] - u0 : 0;
    const int64_t t0 = b.s.tags_off ? b.s.tags_off[k] : 0, lt = b.s.tags_off ? b.s.tags_off[k + 1] - t0 : 0;
    if (lane == 0) {
        uint32_t l = 0;
        for (int64_t i = c0; i < c0 + nc; ++i) {
            const uint32_t op = b.s.cigar[i] & 15u;
            if (op != 1u && op != 4u && op != 5u) l += b.s.cigar[i] >> 4;
        }
        const uint32_t beg = uint32_t(b.s.pos[k]);
        const uint32_t bin = bam_reg2bin(beg, beg + (l > 1u ? l : 1u)) & 0xffffu;
        bam_put32(p, uint32_t(32 + ((lq + 1) & 0xff) + 4 * (nc & 0xffff) + (ls + 1) / 2 + ls + lt));
        bam_put32(p + 4, uint32_t(b.s.ref_id[k]));
        bam_put32(p + 8, beg);
        bam_put32(p + 12, uint32_t((lq + 1) & 0xff) | (uint32_t(b.s.mapq[k]) << 8) | (bin << 16));
        bam_put32(p + 16, uint32_t(nc & 0xffff) | (uint32_t(b.s.flag[k]) << 16));
        bam_put32(p + 20, uint32_t(ls));
        bam_put32(p + 24, uint32_t(b.s.next_ref_id[k]));
        bam_put32(p + 28, uint32_t(b.s.next_pos[k]));
        bam_put32(p + 32, uint32_t(b.s.tlen[k]));
        p[36 + lq] = 0;
    }
    char *q = p + 36;
    for (int64_t i = lane; i < lq; i += 32) q[i] = b.s.qname[q0 + i];
    q += lq + 1;
    for (int64_t i = lane; i < nc; i += 32) bam_put32(q + 4 * i, b.s.cigar[c0 + i]);
    q += 4 * nc;
    const int64_t pairs = (ls + 1) / 2;
    for (int64_t j = lane; j < pairs; j += 32) {
        const uint32_t hi = iu[b.s.seq[s0 + 2 * j] & 31u];
        const uint32_t lo = 2 * j + 1 < ls ? iu[b.s.seq[s0 + 2 * j + 1] & 31u] : 0u;
        q[j] = char((hi << 4) | lo);
    }
    q += pairs;
    for (int64_t i = lane; i < ls; i += 32) q[i] = i < lqual ? char(b.s.qual[u0 + i] - '!') : char(0xff);
    q += ls;
    for (int64_t i = lane; i < lt; i += 32) q[i] = b.s.tags[t0 + i];   // the tags as they are
}

// ordValue(Iupac(c)): the position of the upper-cased letter in "=ACMGRSVTWYHKDBN", 'U' as '=',
// anything else N (the reference's char-to-Iupac conversion).
inline uint8_t bam_iupac(char c)
{
    static const char iu[] = "=ACMGRSVTWYHKDBN";
    const char u = (c >= 'a' && c <= 'z') ? char(c - 32) : c;
    if (u == 'U') return 0;
    for (int k = 0; k < 16; ++k)
        if (iu[k] == u) return uint8_t(k);
    return 15;
}

// Validates the records and uploads their fields into one device buffer; a holds the device
// pointers.  Shared by the SAM and BAM writers.
inline int sam_upload(gba_context *ctx, const gba_sam_records *r, SamArgs &a)
{
    const int64_t n = r->num;
    if (!r->qname_off || !r->flag || !r->ref_id || !r->pos || !r->mapq || !r->cigar_off || !r->next_ref_id ||
        !r->next_pos || !r->tlen || !r->seq_off || !r->seq_letters || (r->num_contigs > 0 && !r->contig_off))
        return fail(ctx, GBA_EINVAL, "null record field");
    // ids the writer can name (the reference indexes contigNames with them) and CIGAR operations
    for (int64_t k = 0; k < n; ++k) {
        if (r->ref_id[k] < -1 || r->ref_id[k] >= r->num_contigs || r->next_ref_id[k] < -1 ||
            r->next_ref_id[k] >= r->num_contigs)
            return fail(ctx, GBA_EINVAL, "record %lld: reference id outside the contigs", (long long)k);
    }
    if (r->cigar_off[n] > 0 && !r->cigar) return fail(ctx, GBA_EINVAL, "null cigar");
    for (int64_t i = 0; i < r->cigar_off[n]; ++i)
        if ((r->cigar[i] & 15u) > 8u) return fail(ctx, GBA_EINVAL, "CIGAR operation index above 8");
    cudaStream_t st = ctx->stream;
    // uploads: one buffer per field (the host arrays are the caller's)
    struct Up {
        const void *src;
        size_t bytes;
    };
    const int64_t qn = r->qname_off[n], cn = r->cigar_off[n], sn = r->seq_off[n];
    const int64_t un = r->qual_off ? r->qual_off[n] : 0;
    const int64_t nc = r->num_contigs, cnb = nc ? r->contig_off[nc] : 0;
    const int64_t tn = r->tags_off ? r->tags_off[n] : 0;
    if (tn > 0 && !r->tags) return fail(ctx, GBA_EINVAL, "null tags");
    const Up ups[] = {{r->qname, size_t(qn)},           {r->qname_off, size_t(n + 1) * 8},
                      {r->flag, size_t(n) * 2},         {r->ref_id, size_t(n) * 4},
                      {r->pos, size_t(n) * 4},          {r->next_ref_id, size_t(n) * 4},
                      {r->next_pos, size_t(n) * 4},     {r->tlen, size_t(n) * 4},
                      {r->mapq, size_t(n)},             {r->cigar, size_t(cn) * 4},
                      {r->cigar_off, size_t(n + 1) * 8}, {r->seq, size_t(sn)},
                      {r->seq_off, size_t(n + 1) * 8},  {r->seq_letters, 32},
                      {r->qual, size_t(un)},            {r->qual_off, r->qual_off ? size_t(n + 1) * 8 : 0},
                      {r->contig_names, size_t(cnb)},   {r->contig_off, nc ? size_t(nc + 1) * 8 : 0},
                      {r->tags, size_t(tn)},            {r->tags_off, r->tags_off ? size_t(n + 1) * 8 : 0}};
    size_t total = 0;
    size_t at[sizeof(ups) / sizeof(ups[0])];
    for (size_t i = 0; i < sizeof(ups) / sizeof(ups[0]); ++i) {
        at[i] = total;
        total += (ups[i].bytes + 15) & ~size_t(15);
    }
    GBA_CUDA(ctx, ctx->sam_in.ensure(total + 16));
    char *base = ctx->sam_in.as<char>();
    for (size_t i = 0; i < sizeof(ups) / sizeof(ups[0]); ++i)
        if (ups[i].bytes && ups[i].src)
            GBA_CUDA(ctx, cudaMemcpyAsync(base + at[i], ups[i].src, ups[i].bytes, cudaMemcpyHostToDevice, st));
    a = SamArgs{};
    a.num = n;
    a.qname = base + at[0];
    a.qname_off = reinterpret_cast<const int64_t *>(base + at[1]);
    a.flag = reinterpret_cast<const uint16_t *>(base + at[2]);
    a.ref_id = reinterpret_cast<const int32_t *>(base + at[3]);
    a.pos = reinterpret_cast<const int32_t *>(base + at[4]);
    a.next_ref_id = reinterpret_cast<const int32_t *>(base + at[5]);
    a.next_pos = reinterpret_cast<const int32_t *>(base + at[6]);
    a.tlen = reinterpret_cast<const int32_t *>(base + at[7]);
    a.mapq = reinterpret_cast<const uint8_t *>(base + at[8]);
    a.cigar = reinterpret_cast<const uint32_t *>(base + at[9]);
    a.cigar_off = reinterpret_cast<const int64_t *>(base + at[10]);
    a.seq = reinterpret_cast<const uint8_t *>(base + at[11]);
    a.seq_off = reinterpret_cast<const int64_t *>(base + at[12]);
    a.letters = base + at[13];
    a.qual = base + at[14];
    a.qual_off = r->qual_off ? reinterpret_cast<const int64_t *>(base + at[15]) : nullptr;
    a.cnames = base + at[16];
    a.cname_off = reinterpret_cast<const int64_t *>(base + at[17]);
    a.num_contigs = nc;
    a.tags = base + at[18];
    a.tags_off = r->tags_off ? reinterpret_cast<const int64_t *>(base + at[19]) : nullptr;
    return GBA_OK;
}

}  // namespace gba

extern "C" {

GBA_API int gba_format_sam(gba_context *ctx, const gba_sam_records *r, char *out, int64_t capacity, int64_t *line_off)
{
    if (!ctx || !r || !line_off) return GBA_EINVAL;
    GBA_CUDA(ctx, cudaSetDevice(ctx->device));
    const int64_t n = r->num;
    if (n < 0) return fail(ctx, GBA_EINVAL, "negative record count");
    line_off[0] = 0;
    if (n == 0) return GBA_OK;
    if (r->tags_off) {
        for (int64_t k = 0; k < n; ++k) {
            if (r->tags_off[k + 1] < r->tags_off[k]) return fail(ctx, GBA_EINVAL, "record %lld: bad tag offsets", (long long)k);
            const int c = r->tags ? tags_check(r->tags + r->tags_off[k], r->tags_off[k + 1] - r->tags_off[k]) : 0;
            if (c == 1) return fail(ctx, GBA_EINVAL, "record %lld: malformed tags", (long long)k);
        }
    }
    SamArgs a{};
    if (int rc = sam_upload(ctx, r, a)) return rc;
    cudaStream_t st = ctx->stream;
    // lengths, offsets (exclusive scan), text
    GBA_CUDA(ctx, ctx->sam_len.ensure(size_t(n + 1) * 8 * 2));
    int64_t *len = ctx->sam_len.as<int64_t>();
    int64_t *off = len + (n + 1);
    GBA_CUDA(ctx, cudaMemsetAsync(len + n, 0, 8, st));
    GBA_CUDA(ctx, cudaEventRecord(ctx->ev[0], st));
    k_sam_lengths<<<unsigned((n + 127) / 128), 128, 0, st>>>(a, len);
    GBA_CUDA(ctx, cudaGetLastError());
    size_t tmp_bytes = 0;
    GBA_CUDA(ctx, cub::DeviceScan::ExclusiveSum(nullptr, tmp_bytes, len, off, n + 1, st));
    GBA_CUDA(ctx, ctx->sam_tmp.ensure(tmp_bytes + 16));
    GBA_CUDA(ctx, cub::DeviceScan::ExclusiveSum(ctx->sam_tmp.ptr, tmp_bytes, len, off, n + 1, st));
    GBA_CUDA(ctx, cudaMemcpyAsync(line_off, off, size_t(n + 1) * 8, cudaMemcpyDeviceToHost, st));
    GBA_CUDA(ctx, cudaStreamSynchronize(st));
    const int64_t bytes = line_off[n];
    if (bytes > capacity || !out) return fail(ctx, GBA_ECAPACITY, "SAM text needs %lld bytes", (long long)bytes);
    GBA_CUDA(ctx, ctx->sam_out.ensure(size_t(bytes) + 16));
    k_sam_write<<<unsigned((n * 32 + 127) / 128), 128, 0, st>>>(a, off, ctx->sam_out.as<char>());
    GBA_CUDA(ctx, cudaGetLastError());
    GBA_CUDA(ctx, cudaEventRecord(ctx->ev[1], st));
    GBA_CUDA(ctx, cudaMemcpyAsync(out, ctx->sam_out.ptr, size_t(bytes), cudaMemcpyDeviceToHost, st));
    GBA_CUDA(ctx, cudaStreamSynchronize(st));
    float ms = 0;
    GBA_CUDA(ctx, cudaEventElapsedTime(&ms, ctx->ev[0], ctx->ev[1]));
    ctx->stats = gba_stats{};
    ctx->stats.dp_kernel_ms = ms;
    ctx->stats.kernel_launches = 4;
    return GBA_OK;
}

}  // extern "C"

extern "C" {

GBA_API int gba_format_bam(gba_context *ctx, const gba_sam_records *r, char *out, int64_t capacity, int64_t *rec_off)
{
    if (!ctx || !r || !rec_off) return GBA_EINVAL;
    GBA_CUDA(ctx, cudaSetDevice(ctx->device));
    const int64_t n = r->num;
    if (n < 0) return fail(ctx, GBA_EINVAL, "negative record count");
    rec_off[0] = 0;
    if (n == 0) return GBA_OK;
    if (r->qname_off && r->cigar_off && r->seq_off) {
        for (int64_t k = 0; k < n; ++k) {
            // the core's l_qname (8 bits) and n_cigar (16 bits) fields; the reference's qualities
            // may not outnumber the residues
            if (r->qname_off[k + 1] - r->qname_off[k] > 254)
                return fail(ctx, GBA_EINVAL, "record %lld: name longer than 254", (long long)k);
            if (r->cigar_off[k + 1] - r->cigar_off[k] > 65535)
                return fail(ctx, GBA_EINVAL, "record %lld: more than 65535 CIGAR operations", (long long)k);
            if (r->qual_off && r->qual_off[k + 1] - r->qual_off[k] > r->seq_off[k + 1] - r->seq_off[k])
                return fail(ctx, GBA_EINVAL, "record %lld: more qualities than residues", (long long)k);
        }
    }
    BamArgs b{};
    if (int rc = sam_upload(ctx, r, b.s)) return rc;
    for (int c = 0; c < 32; ++c) b.iupac[c] = bam_iupac(r->seq_letters[c]);
    cudaStream_t st = ctx->stream;
    GBA_CUDA(ctx, ctx->sam_len.ensure(size_t(n + 1) * 8 * 2));
    int64_t *len = ctx->sam_len.as<int64_t>();
    int64_t *off = len + (n + 1);
    GBA_CUDA(ctx, cudaMemsetAsync(len + n, 0, 8, st));
    GBA_CUDA(ctx, cudaEventRecord(ctx->ev[0], st));
    k_bam_lengths<<<unsigned((n + 127) / 128), 128, 0, st>>>(b, len);
    GBA_CUDA(ctx, cudaGetLastError());
    size_t tmp_bytes = 0;
    GBA_CUDA(ctx, cub::DeviceScan::ExclusiveSum(nullptr, tmp_bytes, len, off, n + 1, st));
    GBA_CUDA(ctx, ctx->sam_tmp.ensure(tmp_bytes + 16));
    GBA_CUDA(ctx, cub::DeviceScan::ExclusiveSum(ctx->sam_tmp.ptr, tmp_bytes, len, off, n + 1, st));
    GBA_CUDA(ctx, cudaMemcpyAsync(rec_off, off, size_t(n + 1) * 8, cudaMemcpyDeviceToHost, st));
    GBA_CUDA(ctx, cudaStreamSynchronize(st));
    const int64_t bytes = rec_off[n];
    if (bytes > capacity || !out) return fail(ctx, GBA_ECAPACITY, "BAM records need %lld bytes", (long long)bytes);
    GBA_CUDA(ctx, ctx->sam_out.ensure(size_t(bytes) + 16));
    k_bam_write<<<unsigned((n * 32 + 127) / 128), 128, 0, st>>>(b, off, ctx->sam_out.as<char>());
    GBA_CUDA(ctx, cudaGetLastError());
    GBA_CUDA(ctx, cudaEventRecord(ctx->ev[1], st));
    GBA_CUDA(ctx, cudaMemcpyAsync(out, ctx->sam_out.ptr, size_t(bytes), cudaMemcpyDeviceToHost, st));
    GBA_CUDA(ctx, cudaStreamSynchronize(st));
    float ms = 0;
    GBA_CUDA(ctx, cudaEventElapsedTime(&ms, ctx->ev[0], ctx->ev[1]));
    ctx->stats = gba_stats{};
    ctx->stats.dp_kernel_ms = ms;
    ctx->stats.kernel_launches = 4;
    return GBA_OK;
}

}  // extern "C"
