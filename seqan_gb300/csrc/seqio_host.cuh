// FASTA / FASTQ input into the engine's record layout (residue codes back to back with n + 1
// offsets, the form gba_align_batch reads).  Semantics: the loop
// `while (!atEnd(iter)) readRecord(id, seq, qual, iter, Fasta|Fastq)` of seq_io/fasta_fastq.h
// (:265-283 FASTA, :354-392 FASTQ), seq a String<Dna|Dna5|AminoAcid>, qual a CharString.
//
// FASTA runs on the device.  Reading it is a three-state automaton over the bytes: BEFORE the
// first record (skipUntil '>'), in a HEADER line (readLine: up to '\r' or '\n'), in a SEQUENCE
// (readUntil '>': whitespace skipped, every other byte a residue or a ParseError).  A '>' outside a
// header starts a record; a newline ends a header.  Each thread summarises a 128-byte chunk for all
// three start states at once (one pass: the BEFORE and HEADER runs join the SEQUENCE run at the
// chunk's first '>' / first newline), a block scan and a two-level scan over the 16 KB blocks'
// summaries compose them, and a second pass re-reads each chunk from its known state, record and residue
// index to write codes and record bounds (the first pass keeps each chunk's summary in one word, so
// the second reads it back instead of recomputing it).
//
// FASTQ runs on the host: where a record ends depends on counting its quality characters from the
// record's start ('@' is also a quality value), so the text does not split into independent chunks.
#pragma once

namespace gba {

constexpr int kFaChunk = 128;      // bytes per thread
constexpr int kFaThreads = 128;    // threads per block: 16 KB of text per block
constexpr int kFaTile = 256;       // block summaries per tile of the summary scan

enum : int8_t { FA_GT = -4, FA_NL = -3, FA_WS = -2, FA_BAD = -1 };
enum : int32_t { FA_BEFORE = 0, FA_HEADER = 1, FA_SEQ = 2 };

struct alignas(16) FaSum {
    int64_t rec[3];   // records started in the chunk, per start state
    int64_t res[3];   // residues (valid or not) read in the chunk, per start state
    int32_t end[3];   // state after the chunk, per start state
    int32_t pad;
};

// v[m] for a state m in 0..2 through selects (runtime indexing would put the summary in local
// memory); any other m reads v[2].
template <typename T>
__host__ __device__ __forceinline__ T fa_pick(const T (&v)[3], int m)
{
    return m == 0 ? v[0] : m == 1 ? v[1] : v[2];
}

struct FaCompose {
    __host__ __device__ FaSum operator()(const FaSum &a, const FaSum &b) const
    {
        FaSum r;
#pragma unroll
        for (int s = 0; s < 3; ++s) {
            const int m = a.end[s];
            r.end[s] = fa_pick(b.end, m);
            r.rec[s] = a.rec[s] + fa_pick(b.rec, m);
            r.res[s] = a.res[s] + fa_pick(b.res, m);
        }
        r.pad = 0;
        return r;
    }
};

__host__ __device__ inline FaSum fa_identity()
{
    FaSum r{};
    r.end[0] = 0;
    r.end[1] = 1;
    r.end[2] = 2;
    return r;
}

// A chunk's summary in one word: per start state 8 bits of records, 8 of residues (a chunk of 128
// bytes holds at most 128 of either) and 2 of end state.
__device__ __forceinline__ unsigned long long fa_pack(const FaSum &v)
{
    unsigned long long w = 0;
#pragma unroll
    for (int s = 0; s < 3; ++s)
        w |= (static_cast<unsigned long long>(v.rec[s]) | (static_cast<unsigned long long>(v.res[s]) << 8) |
              (static_cast<unsigned long long>(v.end[s]) << 16)) << (18 * s);
    return w;
}

__device__ __forceinline__ FaSum fa_unpack(unsigned long long w)
{
    FaSum v;
    v.pad = 0;
#pragma unroll
    for (int s = 0; s < 3; ++s) {
        const unsigned long long f = w >> (18 * s);
        v.rec[s] = int64_t(f & 0xffu);
        v.res[s] = int64_t((f >> 8) & 0xffu);
        v.end[s] = int32_t((f >> 16) & 3u);
    }
    return v;
}

struct FaArgs {
    const uint8_t *text;
    int64_t n;
    int8_t cls[256];          // residue code, or FA_GT / FA_NL / FA_WS / FA_BAD
    FaSum *block_sum;         // [blocks]: after the scans, inclusive within tiles of kFaTile blocks
    const FaSum *tile_sum;    // [tiles]: inclusive over the tiles
    const unsigned long long *chunk_sum;   // [chunks]: each chunk's summary from the first pass
    uint8_t *codes;
    int64_t *id_begin, *id_end, *seq_off;
    unsigned long long *error;   // smallest offset of a ParseError byte
    int64_t nrec, nres;          // totals of the scan: bounds of the second pass's writes
    unsigned int *bounds;        // set when a write falls outside them (skipped)
};

// Byte classes of a 32-byte group as bit masks (bit i = byte i): '>' (g), '\n' or '\r' (l), residue
// candidates (r: neither '>', a newline, ' ' nor '\t').  __vcmpeq4 compares four bytes at once;
// the multiply gathers the low bit of each byte into four adjacent bits.
struct FaMasks {
    uint32_t g, l, r;
};

__device__ __forceinline__ uint32_t fa_bits4(uint32_t eq) { return ((eq & 0x01010101u) * 0x01020408u) >> 24; }

__device__ __forceinline__ FaMasks fa_masks(const uint32_t (&x)[8])
{
    FaMasks m{0u, 0u, 0u};
#pragma unroll
    for (int q = 0; q < 8; ++q) {
        const uint32_t g = __vcmpeq4(x[q], 0x3e3e3e3eu);
        const uint32_t l = __vcmpeq4(x[q], 0x0a0a0a0au) | __vcmpeq4(x[q], 0x0d0d0d0du);
        const uint32_t w = l | __vcmpeq4(x[q], 0x20202020u) | __vcmpeq4(x[q], 0x09090909u);
        m.g |= fa_bits4(g) << (4 * q);
        m.l |= fa_bits4(l) << (4 * q);
        m.r |= fa_bits4(~(g | w)) << (4 * q);
    }
    return m;
}

// Header state after each byte of a group, all 32 at once.  Header-or-not is a set ('>') / reset
// (newline) flip-flop.  In each run of non-newline bytes the state is "not header" from the run's
// start up to its first '>' (or the whole run): adding one at every run start to the run's
// non-'>' bytes carries through exactly those bytes, which the sum clears.  A run that starts the
// group inherits hdr_in, so it gets no carry when hdr_in is set.
__device__ __forceinline__ uint32_t fa_after(uint32_t g, uint32_t l, bool hdr_in)
{
    const uint32_t z = ~l;
    const uint32_t m = z & ~g;
    uint32_t starts = z & ~(z << 1);
    if (hdr_in) starts &= ~1u;
    const uint32_t not_yet = m & ~(m + starts);
    return z & ~not_yet;
}

__device__ __forceinline__ void fa_group_words(const uint4 (&w)[kFaChunk / 16], int grp, uint32_t (&x)[8])
{
    const uint4 a = w[2 * grp], b = w[2 * grp + 1];
    x[0] = a.x; x[1] = a.y; x[2] = a.z; x[3] = a.w;
    x[4] = b.x; x[5] = b.y; x[6] = b.z; x[7] = b.w;
}

// The SEQUENCE run over one byte, without branches: '>' starts a record outside a header, a
// newline ends a header, any other non-whitespace byte is a residue outside a header.
struct FaRun {
    bool hdr = false, seen_gt = false, seen_nl = false;
    int32_t rec = 0, res = 0, gt_res = 0, nl_rec = 0, nl_res = 0;
    __device__ __forceinline__ void step(uint32_t c)
    {
        const bool g = c == '>';
        const bool l = c == '\n' || c == '\r';
        const bool r = !(g || l || c == ' ' || c == '\t');
        gt_res = (g && !seen_gt) ? res : gt_res;
        nl_rec = (l && !seen_nl) ? rec : nl_rec;
        nl_res = (l && !seen_nl) ? res : nl_res;
        seen_gt |= g;
        seen_nl |= l;
        rec += (g && !hdr) ? 1 : 0;
        res += (r && !hdr) ? 1 : 0;
        hdr = g || (hdr && !l);
    }
    // The same run over a 32-byte group given as masks.
    __device__ __forceinline__ void group(const FaMasks &m)
    {
        const uint32_t after = fa_after(m.g, m.l, hdr);
        const uint32_t before = (after << 1) | (hdr ? 1u : 0u);
        const uint32_t starts = m.g & ~before, counted = m.r & ~before;
        if (!seen_gt && m.g) {
            const uint32_t below = (1u << (__ffs(m.g) - 1)) - 1u;
            gt_res = res + __popc(counted & below);
            seen_gt = true;
        }
        if (!seen_nl && m.l) {
            const uint32_t below = (1u << (__ffs(m.l) - 1)) - 1u;
            nl_rec = rec + __popc(starts & below);
            nl_res = res + __popc(counted & below);
            seen_nl = true;
        }
        rec += __popc(starts);
        res += __popc(counted);
        hdr = (after >> 31) != 0;
    }
    __device__ __forceinline__ FaSum summary() const
    {
        FaSum o;
        o.pad = 0;
        const int s = hdr ? FA_HEADER : FA_SEQ;
        o.end[FA_SEQ] = s;
        o.rec[FA_SEQ] = rec;
        o.res[FA_SEQ] = res;
        // From BEFORE: nothing counts until the first '>', where the run joins the SEQUENCE run.
        o.end[FA_BEFORE] = seen_gt ? s : FA_BEFORE;
        o.rec[FA_BEFORE] = seen_gt ? rec : 0;
        o.res[FA_BEFORE] = seen_gt ? res - gt_res : 0;
        // From HEADER: nothing counts until the first newline, after which both runs are in SEQUENCE.
        o.end[FA_HEADER] = seen_nl ? s : FA_HEADER;
        o.rec[FA_HEADER] = seen_nl ? rec - nl_rec : 0;
        o.res[FA_HEADER] = seen_nl ? res - nl_res : 0;
        return o;
    }
};

// Summary of the chunk at base: a full chunk through 16-byte loads kept in registers, the text's
// last partial chunk through byte loads.
__device__ __forceinline__ FaSum fa_summary_at(const uint8_t *text, int64_t n, int64_t base, uint4 (&w)[kFaChunk / 16],
                                               bool &full)
{
    FaRun run;
    full = n - base >= kFaChunk;
    if (full) {
        const uint4 *src = reinterpret_cast<const uint4 *>(text + base);
#pragma unroll
        for (int i = 0; i < kFaChunk / 16; ++i) w[i] = __ldg(src + i);
#pragma unroll
        for (int grp = 0; grp < kFaChunk / 32; ++grp) {
            uint32_t x[8];
            fa_group_words(w, grp, x);
            run.group(fa_masks(x));
        }
    } else {
        for (int64_t i = base; i < n; ++i) run.step(text[i]);
    }
    return run.summary();
}

__global__ void __launch_bounds__(kFaThreads) k_fasta_summary(const uint8_t *__restrict__ text, int64_t n,
                                                              FaSum *__restrict__ block_sum,
                                                              unsigned long long *__restrict__ chunk_sum)
{
    using Scan = cub::BlockScan<FaSum, kFaThreads, cub::BLOCK_SCAN_WARP_SCANS>;
    __shared__ typename Scan::TempStorage tmp;
    const int64_t base = (int64_t(blockIdx.x) * kFaThreads + threadIdx.x) * kFaChunk;
    FaSum mine = fa_identity();
    if (base < n) {
        uint4 w[kFaChunk / 16];
        bool full;
        mine = fa_summary_at(text, n, base, w, full);
        chunk_sum[int64_t(blockIdx.x) * kFaThreads + threadIdx.x] = fa_pack(mine);
    }
    FaSum incl;
    Scan(tmp).InclusiveScan(mine, incl, FaCompose());
    if (threadIdx.x == kFaThreads - 1) block_sum[blockIdx.x] = incl;
}

// One byte of the record pass: record bounds go to global memory (rare), residue codes to the
// block's shared staging buffer at their offset from the block's first residue.
struct FaWriter {
    const int8_t *cls;
    uint8_t *stage;
    int64_t stage_base, nrec, nres;
    int64_t *id_begin, *id_end, *seq_off;
    unsigned long long *error;
    unsigned int *bounds;
    int s;
    int64_t rec, res;
    int64_t first_bad;   // first byte outside the alphabet seen by the bit path, or -1
    __device__ __forceinline__ void step(uint32_t c, int64_t pos)
    {
        const int k = cls[c];
        if (k == FA_GT) {
            if (s != FA_HEADER) {
                ++rec;
                s = FA_HEADER;
                if (rec >= 0 && rec < nrec) {
                    id_begin[rec] = pos + 1;
                    seq_off[rec] = res;
                } else {
                    atomicOr(bounds, 1u);
                }
            }
        } else if (k == FA_NL) {
            if (s == FA_HEADER) {
                if (rec >= 0 && rec < nrec) id_end[rec] = pos;
                else atomicOr(bounds, 1u);
                s = FA_SEQ;
            }
        } else if (k != FA_WS && s == FA_SEQ) {
            if (k == FA_BAD) atomicMin(error, static_cast<unsigned long long>(pos));
            const int64_t o = res - stage_base;
            if (res < nres && o >= 0 && o < kFaThreads * kFaChunk) stage[o] = k == FA_BAD ? uint8_t(0) : uint8_t(k);
            else atomicOr(bounds, 2u);
            ++res;
        }
    }
};

// The record pass over a full 32-byte group at text offset pos0: record starts and header ends
// (rare) by walking their bits, residue codes into the staging buffer with the group's bytes at
// compile-time positions.
__device__ __forceinline__ void fa_write_group(FaWriter &wr, const uint32_t (&x)[8], int64_t pos0)
{
    const FaMasks m = fa_masks(x);
    const bool hdr = wr.s == FA_HEADER;
    const uint32_t after = fa_after(m.g, m.l, hdr);
    const uint32_t before = (after << 1) | (hdr ? 1u : 0u);
    uint32_t counted = m.r & ~before;
    const uint32_t starts = m.g & ~before, ends = m.l & before;
    bool still_before = false;
    if (wr.s == FA_BEFORE) {   // nothing counts before the text's first '>'
        counted &= m.g ? ~((1u << (__ffs(m.g) - 1)) - 1u) : 0u;
        still_before = m.g == 0;
    }
    for (uint32_t ev = starts | ends; ev; ev &= ev - 1) {
        const int i = __ffs(ev) - 1;
        const int64_t pos = pos0 + i;
        if ((starts >> i) & 1u) {
            ++wr.rec;
            if (wr.rec >= 0 && wr.rec < wr.nrec) {
                wr.id_begin[wr.rec] = pos + 1;
                wr.seq_off[wr.rec] = wr.res + __popc(counted & ((1u << i) - 1u));
            } else {
                atomicOr(wr.bounds, 1u);
            }
        } else {
            if (wr.rec >= 0 && wr.rec < wr.nrec) wr.id_end[wr.rec] = pos;
            else atomicOr(wr.bounds, 1u);
        }
    }
    const int cnt = __popc(counted);
    int64_t o = wr.res - wr.stage_base;
    if (o < 0 || o + cnt > kFaThreads * kFaChunk || wr.res + cnt > wr.nres) {
        if (cnt) atomicOr(wr.bounds, 2u);
    } else {
        // Predicated per byte: the store and the advance only for counted bytes; the first byte
        // outside the alphabet is kept in a register (one atomic per chunk, by the caller).
        uint32_t bad = 0;
#pragma unroll
        for (int q = 0; q < 8; ++q) {
            uint32_t xq = x[q];
#pragma unroll
            for (int b = 0; b < 4; ++b) {
                const bool take = (counted >> (4 * q + b)) & 1u;
                const int k = wr.cls[xq & 0xffu];
                if (take) wr.stage[o] = uint8_t(k < 0 ? 0 : k);
                o += take ? 1 : 0;
                bad |= (take && k == FA_BAD) ? (1u << (4 * q + b)) : 0u;
                xq >>= 8;
            }
        }
        if (bad && wr.first_bad < 0) wr.first_bad = pos0 + (__ffs(bad) - 1);
    }
    wr.res += cnt;
    wr.s = still_before ? FA_BEFORE : ((after >> 31) ? FA_HEADER : FA_SEQ);
}

__global__ void __launch_bounds__(kFaThreads) k_fasta_write(FaArgs a)
{
    using Scan = cub::BlockScan<FaSum, kFaThreads, cub::BLOCK_SCAN_WARP_SCANS>;
    __shared__ typename Scan::TempStorage tmp;
    __shared__ int8_t cls[256];
    __shared__ uint8_t stage[kFaThreads * kFaChunk];
    for (int i = threadIdx.x; i < 256; i += blockDim.x) cls[i] = a.cls[i];
    __syncthreads();
    const int64_t base = (int64_t(blockIdx.x) * kFaThreads + threadIdx.x) * kFaChunk;
    uint4 w[kFaChunk / 16];
    const bool full = a.n - base >= kFaChunk;
    FaSum mine = fa_identity();
    if (base < a.n) {
        mine = fa_unpack(a.chunk_sum[int64_t(blockIdx.x) * kFaThreads + threadIdx.x]);
        if (full) {
            const uint4 *src = reinterpret_cast<const uint4 *>(a.text + base);
#pragma unroll
            for (int i = 0; i < kFaChunk / 16; ++i) w[i] = __ldg(src + i);
        }
    }
    FaSum before;
    Scan(tmp).ExclusiveScan(mine, before, fa_identity(), FaCompose());
    // Prefix of the blocks before this one: the tiles before this block's tile, then the blocks
    // before it in its tile.
    const unsigned tile = blockIdx.x / kFaTile;
    const FaSum tile_before = tile ? a.tile_sum[tile - 1] : fa_identity();
    const FaSum blk = blockIdx.x % kFaTile ? FaCompose()(tile_before, a.block_sum[blockIdx.x - 1]) : tile_before;
    const int64_t blk_res = blk.res[FA_BEFORE];
    if (base < a.n) {
        // State, records started and residues read before this chunk, from the start of the text.
        const int mid = blk.end[FA_BEFORE];
        FaWriter wr{cls, stage, blk_res, a.nrec, a.nres, a.id_begin, a.id_end, a.seq_off, a.error, a.bounds,
                    fa_pick(before.end, mid), blk.rec[FA_BEFORE] + fa_pick(before.rec, mid) - 1,
                    blk_res + fa_pick(before.res, mid), -1};
        if (full) {
#pragma unroll
            for (int grp = 0; grp < kFaChunk / 32; ++grp) {
                uint32_t x[8];
                fa_group_words(w, grp, x);
                fa_write_group(wr, x, base + 32 * grp);
            }
            if (wr.first_bad >= 0) atomicMin(a.error, static_cast<unsigned long long>(wr.first_bad));
        } else {
            for (int64_t i = base; i < a.n; ++i) wr.step(a.text[i], i);
        }
    }
    __syncthreads();
    // The block's residues are one contiguous range of the output: copy it out coalesced.
    const int64_t cnt = FaCompose()(tile_before, a.block_sum[blockIdx.x]).res[FA_BEFORE] - blk_res;
    uint8_t *out = a.codes + blk_res;
    for (int64_t i = threadIdx.x; i < cnt && i < kFaThreads * kFaChunk && blk_res + i < a.nres; i += kFaThreads)
        out[i] = stage[i];
}

// Scan of the block summaries in two levels.  k_fasta_scan_tiles: one block of kFaTile threads per
// tile of kFaTile consecutive block summaries (coalesced loads, one summary per thread) rewrites them
// as inclusive prefixes within the tile and writes the tile's total.  k_fasta_scan_top: one block
// scans the tile totals in place (thread t composes a contiguous range, a block scan gives each
// range its prefix).  The record pass composes the two.
__global__ void __launch_bounds__(kFaTile) k_fasta_scan_tiles(FaSum *sums, int64_t nb, FaSum *tile_sum)
{
    using Scan = cub::BlockScan<FaSum, kFaTile, cub::BLOCK_SCAN_WARP_SCANS>;
    __shared__ typename Scan::TempStorage tmp;
    const int64_t i = int64_t(blockIdx.x) * kFaTile + threadIdx.x;
    const FaSum mine = i < nb ? sums[i] : fa_identity();
    FaSum incl;
    Scan(tmp).InclusiveScan(mine, incl, FaCompose());
    if (i < nb) sums[i] = incl;
    if (threadIdx.x == kFaTile - 1) tile_sum[blockIdx.x] = incl;
}

__global__ void __launch_bounds__(kFaTile) k_fasta_scan_top(FaSum *sums, int64_t nt)
{
    using Scan = cub::BlockScan<FaSum, kFaTile, cub::BLOCK_SCAN_WARP_SCANS>;
    __shared__ typename Scan::TempStorage tmp;
    const int64_t per = (nt + kFaTile - 1) / kFaTile;
    const int64_t lo = int64_t(threadIdx.x) * per;
    const int64_t hi = lo + per < nt ? lo + per : nt;
    const FaCompose op;
    FaSum agg = fa_identity();
    for (int64_t i = lo; i < hi; ++i) agg = op(agg, sums[i]);
    FaSum pre;
    Scan(tmp).ExclusiveScan(agg, pre, fa_identity(), op);
    for (int64_t i = lo; i < hi; ++i) {
        pre = op(pre, sums[i]);
        sums[i] = pre;
    }
}

// Residue code per character: the reference's IsInAlphabet<T>(c) ? ordValue(T(c)) : ParseError.
inline bool seqio_classes(int32_t alphabet, int8_t *cls)
{
    if (alphabet != 4 && alphabet != 5 && alphabet != 27) return false;
    for (int c = 0; c < 256; ++c) cls[c] = FA_BAD;
    if (alphabet == 27) {
        static const char aa[] = "ABCDEFGHIJKLMNOPQRSTUVWYZX*";
        for (int k = 0; k < 27; ++k) {
            cls[uint8_t(aa[k])] = int8_t(k);
            if (aa[k] >= 'A' && aa[k] <= 'Z') cls[uint8_t(aa[k] + 32)] = int8_t(k);
        }
    } else {
        const char *dna = alphabet == 5 ? "ACGTN" : "ACGT";
        for (int k = 0; dna[k]; ++k) {
            cls[uint8_t(dna[k])] = int8_t(k);
            cls[uint8_t(dna[k] + 32)] = int8_t(k);
        }
    }
    cls[uint8_t(' ')] = FA_WS;
    cls[uint8_t('\t')] = FA_WS;
    cls[uint8_t('\n')] = FA_NL;
    cls[uint8_t('\r')] = FA_NL;
    cls[uint8_t('>')] = FA_GT;
    return true;
}

inline int seqio_check(gba_context *ctx, const char *text, int64_t n, int32_t alphabet, gba_seq_records *r,
                       int8_t *cls)
{
    if (!r || n < 0 || (n > 0 && !text)) return fail(ctx, GBA_EINVAL, "null text or records, or negative length");
    if (!seqio_classes(alphabet, cls)) return fail(ctx, GBA_EINVAL, "alphabet must be 4 (Dna), 5 (Dna5) or 27 (AminoAcid)");
    r->num = 0;
    r->residues = 0;
    r->error_offset = -1;
    return GBA_OK;
}

// ---- FASTQ on the host ------------------------------------------------------------------------

struct FqResult {
    int status = GBA_OK;
    int64_t err_at = -1;
    const char *what = "";
    int64_t end = 0;   // parser position after the last record read: the next '@' or the end
};

// Writes records straight into the caller's buffers (counting past their capacities).
struct FqCallerSink {
    gba_seq_records *r;
    bool write;
    int64_t rec = 0, res = 0, qe = 0;
    void code(uint8_t k)
    {
        if (write && res < r->residue_capacity) r->codes[res] = k;
        ++res;
    }
    void qual_begin() { qe = seq_begin; }
    void qual(char c)
    {
        if (write && r->quals && qe < r->residue_capacity) r->quals[qe] = c;
        ++qe;
    }
    int64_t seq_begin = 0;
    void record_begin() { seq_begin = res; }
    void record(int64_t ib, int64_t ie)
    {
        if (write && rec < r->record_capacity) {
            r->id_begin[rec] = ib;
            r->id_end[rec] = ie;
            r->seq_off[rec] = seq_begin;
            if (r->qual_end) r->qual_end[rec] = qe;
        }
        ++rec;
    }
};

// Collects one thread's records (residue and quality offsets local to the thread).
struct FqLocalSink {
    std::vector<int64_t> ib, ie, sb, qe;
    std::vector<uint8_t> codes;
    std::vector<char> quals;
    int64_t seq_begin = 0;
    void code(uint8_t k) { codes.push_back(k); }
    void qual_begin() { quals.resize(size_t(seq_begin)); }
    void qual(char c) { quals.push_back(c); }
    void record_begin() { seq_begin = int64_t(codes.size()); }
    void record(int64_t b, int64_t e)
    {
        ib.push_back(b);
        ie.push_back(e);
        sb.push_back(seq_begin);
        qe.push_back(int64_t(quals.size()));
        quals.resize(codes.size());   // keep qualities at their residues' offsets
    }
};

// The reference's readRecord loop for FASTQ from position p: records are read while the next one
// starts before stop (a record's start is the '@' that skipUntil reaches).
template <typename Sink>
FqResult fastq_parse(const uint8_t *t, int64_t n, int64_t p, int64_t stop, const int8_t *cls, Sink &sink)
{
    FqResult out;
    auto nl = [](uint8_t c) { return c == '\n' || c == '\r'; };
    auto ws = [](uint8_t c) { return c == ' ' || c == '\t' || c == '\n' || c == '\r'; };
    auto err = [&](int64_t at, const char *what) {
        out.status = GBA_EPARSE;
        out.err_at = at;
        out.what = what;
        out.end = at;
        return out;
    };
    while (p < n) {
        const void *at = memchr(t + p, '@', size_t(n - p));   // skipUntil '@'
        if (!at) return err(n, "no '@' record start before the end");
        if (static_cast<const uint8_t *>(at) - t >= stop) {
            out.end = static_cast<const uint8_t *>(at) - t;
            return out;
        }
        p = static_cast<const uint8_t *>(at) - t + 1;
        const int64_t ib = p;                                  // readLine(id)
        while (p < n && !nl(t[p])) ++p;
        const int64_t ie = p;
        if (p < n && t[p] == '\r') ++p;
        if (p < n && t[p] == '\n') ++p;
        sink.record_begin();
        int64_t len = 0;
        for (; p < n && t[p] != '+'; ++p) {                    // readUntil(seq, '+')
            const int k = cls[t[p]];
            if (k == FA_WS || k == FA_NL) continue;
            if (k < 0) return err(p, "character outside the alphabet");
            sink.code(uint8_t(k));
            ++len;
        }
        if (p >= n) return err(n, "no '+' line before the end");
        ++p;
        while (p < n && !nl(t[p])) ++p;                        // skipLine
        if (p < n && t[p] == '\r') ++p;
        if (p < n && t[p] == '\n') ++p;
        sink.qual_begin();
        for (int64_t need = len; p < n && need > 0; ++p) {     // counted qualities
            if (nl(t[p])) continue;
            sink.qual(char(t[p]));
            --need;
        }
        while (p < n && ws(t[p])) ++p;
        if (p < n && t[p] != '@' && t[p] != 0xFF) return err(p, "quality string not as long as the sequence");
        sink.record(ib, ie);
    }
    out.end = n;
    return out;
}

// A plausible record start at or after from: '@' at a line start, then a line, a line, a line
// starting with '+', and a line as long as the second.
inline int64_t fastq_sync(const uint8_t *t, int64_t n, int64_t from)
{
    auto line_end = [&](int64_t q) {
        while (q < n && t[q] != '\n') ++q;
        return q;
    };
    for (int64_t p = from; p < n; ++p) {
        if (t[p] != '@' || (p > 0 && t[p - 1] != '\n')) continue;
        const int64_t e1 = line_end(p);
        const int64_t e2 = line_end(e1 + 1);
        if (e2 >= n || t[e2 + 1] != '+') continue;
        const int64_t e3 = line_end(e2 + 1);
        const int64_t e4 = line_end(e3 + 1);
        if (e4 - (e3 + 1) == e2 - (e1 + 1)) return p;
    }
    return n;
}

// Reads a large text with the threads of the host: each thread starts at a plausible record start
// in its slice and reads until the next thread's start.  The result stands only if every thread's
// reading ends exactly on the next thread's start (thread 0 starts where the reference starts, so
// each start is then a true record start) and no thread met an error; otherwise it returns false
// and the caller reads the text sequentially.
template <typename Sink>
bool fastq_read_parallel(const uint8_t *t, int64_t n, const int8_t *cls, Sink &sink, FqResult &result)
{
    const int threads = omp_get_max_threads();
    if (threads < 2 || n < (int64_t(4) << 20)) return false;
    std::vector<int64_t> start(size_t(threads) + 1);
    start[0] = 0;
    start[size_t(threads)] = n;
#pragma omp parallel for num_threads(threads)
    for (int k = 1; k < threads; ++k) start[size_t(k)] = fastq_sync(t, n, n / threads * k);
    for (int k = 1; k <= threads; ++k)
        if (start[size_t(k)] < start[size_t(k - 1)]) start[size_t(k)] = start[size_t(k - 1)];
    std::vector<FqLocalSink> local(static_cast<size_t>(threads));
    std::vector<FqResult> res(static_cast<size_t>(threads));
#pragma omp parallel for num_threads(threads)
    for (int k = 0; k < threads; ++k) {
        const size_t slice = size_t(start[size_t(k + 1)] - start[size_t(k)]) + 4096;
        FqLocalSink &l = local[size_t(k)];
        l.codes.reserve(slice);
        l.quals.reserve(slice);
        for (auto *v : {&l.ib, &l.ie, &l.sb, &l.qe}) v->reserve(slice / 64 + 16);
        res[size_t(k)] = fastq_parse(t, n, start[size_t(k)], k + 1 < threads ? start[size_t(k + 1)] : INT64_MAX, cls,
                                     l);
    }
    for (int k = 0; k < threads; ++k) {
        if (res[size_t(k)].status) return false;
        if (k + 1 < threads && res[size_t(k)].end != start[size_t(k + 1)]) return false;
    }
    // Concatenate the threads' records in order into the caller's buffers, each thread its part.
    std::vector<int64_t> rec0(size_t(threads) + 1, 0), res0(size_t(threads) + 1, 0);
    for (int k = 0; k < threads; ++k) {
        rec0[size_t(k + 1)] = rec0[size_t(k)] + int64_t(local[size_t(k)].ib.size());
        res0[size_t(k + 1)] = res0[size_t(k)] + int64_t(local[size_t(k)].codes.size());
    }
    const int64_t nrec = rec0[size_t(threads)], nres = res0[size_t(threads)];
    if (sink.write && nrec <= sink.r->record_capacity && nres <= sink.r->residue_capacity) {
        gba_seq_records *r = sink.r;
#pragma omp parallel for num_threads(threads)
        for (int k = 0; k < threads; ++k) {
            const FqLocalSink &l = local[size_t(k)];
            const int64_t b = res0[size_t(k)], q = rec0[size_t(k)];
            memcpy(r->codes + b, l.codes.data(), l.codes.size());
            if (r->quals) memcpy(r->quals + b, l.quals.data(), std::min(l.quals.size(), l.codes.size()));
            for (size_t j = 0; j < l.ib.size(); ++j) {
                r->id_begin[q + int64_t(j)] = l.ib[j];
                r->id_end[q + int64_t(j)] = l.ie[j];
                r->seq_off[q + int64_t(j)] = b + l.sb[j];
                if (r->qual_end) r->qual_end[q + int64_t(j)] = b + l.qe[j];
            }
        }
    }
    sink.rec = nrec;
    sink.res = nres;
    result = FqResult{};
    result.end = n;
    return true;
}

}  // namespace gba

extern "C" {

}  // extern "C"

namespace gba {

// Host arrays for the record bounds that fasta_parse sizes itself once the scan has counted the
// records (one reading of the text instead of a counting call and a reading call).
struct FaHostRecords {
    std::vector<int64_t> id_begin, id_end, seq_off;
};

// gba_read_fasta's work; with dst the residue codes also go to that device buffer (from offset 0)
// and r->codes may be null; with grow the record arrays are grow's, sized to the records found.
int fasta_parse(gba_context *ctx, const char *text, int64_t n, int32_t alphabet, gba_seq_records *r, DevBuf *dst,
                FaHostRecords *grow = nullptr)
{
    if (!ctx) return GBA_EINVAL;
    FaArgs a{};
    if (int rc = seqio_check(ctx, text, n, alphabet, r, a.cls)) return rc;
    if (n == 0) {
        if (grow) {
            grow->seq_off.assign(1, 0);
            r->seq_off = grow->seq_off.data();
            r->record_capacity = 1;
        }
        if (r->record_capacity < 1 || !r->seq_off) return fail(ctx, GBA_ECAPACITY, "seq_off needs 1 entry");
        r->seq_off[0] = 0;
        if (dst) GBA_CUDA(ctx, dst->ensure(16));
        return GBA_OK;
    }
    GBA_CUDA(ctx, cudaSetDevice(ctx->device));
    cudaStream_t st = ctx->stream;
    const int64_t chunks = (n + kFaChunk - 1) / kFaChunk;
    const int64_t blocks = (chunks + kFaThreads - 1) / kFaThreads;
    if (blocks > INT32_MAX) return fail(ctx, GBA_EINVAL, "text too long");
    GBA_CUDA(ctx, ctx->fa_text.ensure(size_t(n) + 16));
    const int64_t tiles = (blocks + kFaTile - 1) / kFaTile;
    GBA_CUDA(ctx, ctx->fa_sum.ensure(size_t(blocks + tiles) * sizeof(FaSum) + 16));
    GBA_CUDA(ctx, cudaEventRecord(ctx->ev[0], st));
    GBA_CUDA(ctx, cudaMemcpyAsync(ctx->fa_text.ptr, text, size_t(n), cudaMemcpyHostToDevice, st));
    a.text = ctx->fa_text.as<uint8_t>();
    a.n = n;
    a.block_sum = ctx->fa_sum.as<FaSum>();
    GBA_CUDA(ctx, cudaEventRecord(ctx->ev[2], st));
    GBA_CUDA(ctx, ctx->fa_chunk.ensure(size_t(blocks) * kFaThreads * 8 + 16));
    a.chunk_sum = ctx->fa_chunk.as<unsigned long long>();
    k_fasta_summary<<<unsigned(blocks), kFaThreads, 0, st>>>(a.text, a.n, a.block_sum,
                                                           ctx->fa_chunk.as<unsigned long long>());
    GBA_CUDA(ctx, cudaGetLastError());
    FaSum *tile_sum = a.block_sum + blocks;
    a.tile_sum = tile_sum;
    k_fasta_scan_tiles<<<unsigned(tiles), kFaTile, 0, st>>>(a.block_sum, blocks, tile_sum);
    GBA_CUDA(ctx, cudaGetLastError());
    k_fasta_scan_top<<<1, kFaTile, 0, st>>>(tile_sum, tiles);
    GBA_CUDA(ctx, cudaGetLastError());
    GBA_CUDA(ctx, ctx->fa_tmp.ensure(64));
    FaSum total;
    GBA_CUDA(ctx, cudaMemcpyAsync(&total, tile_sum + (tiles - 1), sizeof(FaSum), cudaMemcpyDeviceToHost, st));
    GBA_CUDA(ctx, cudaStreamSynchronize(st));
    const int64_t nrec = total.rec[FA_BEFORE], nres = total.res[FA_BEFORE];
    r->num = nrec;
    r->residues = nres;
    if (nrec == 0) {   // readRecord's skipOne('>') at the end of the text: UnexpectedEnd
        r->error_offset = n;
        return fail(ctx, GBA_EPARSE, "no '>' record start in the text");
    }
    if (grow) {
        const size_t cap = static_cast<size_t>(nrec) + 1;
        grow->id_begin.assign(cap, 0);
        grow->id_end.assign(cap, 0);
        grow->seq_off.assign(cap, 0);
        r->id_begin = grow->id_begin.data();
        r->id_end = grow->id_end.data();
        r->seq_off = grow->seq_off.data();
        r->record_capacity = int64_t(cap);
    }
    if (nrec + 1 > r->record_capacity || (!dst && (nres > r->residue_capacity || !r->codes)) || !r->id_begin ||
        !r->id_end || !r->seq_off)
        return fail(ctx, GBA_ECAPACITY, "records need %lld record and %lld residue entries", (long long)nrec + 1,
                    (long long)nres);
    const size_t idx_bytes = (size_t(nrec) + 1) * 8;
    GBA_CUDA(ctx, ctx->fa_out.ensure(size_t(nres) + 3 * idx_bytes + 64));
    char *o = ctx->fa_out.as<char>();
    a.id_begin = reinterpret_cast<int64_t *>(o);
    a.id_end = reinterpret_cast<int64_t *>(o + idx_bytes);
    a.seq_off = reinterpret_cast<int64_t *>(o + 2 * idx_bytes);
    a.codes = reinterpret_cast<uint8_t *>(o + 3 * idx_bytes);
    a.error = reinterpret_cast<unsigned long long *>(ctx->fa_tmp.ptr);
    a.bounds = reinterpret_cast<unsigned int *>(ctx->fa_tmp.as<char>() + 8);
    a.nrec = nrec;
    a.nres = nres;
    GBA_CUDA(ctx, cudaMemsetAsync(a.error, 0xff, 8, st));
    GBA_CUDA(ctx, cudaMemsetAsync(a.bounds, 0, 4, st));
    k_fasta_write<<<unsigned(blocks), kFaThreads, 0, st>>>(a);
    GBA_CUDA(ctx, cudaGetLastError());
    GBA_CUDA(ctx, cudaEventRecord(ctx->ev[3], st));
    unsigned long long err = 0;
    unsigned int bounds = 0;
    GBA_CUDA(ctx, cudaMemcpyAsync(&err, a.error, 8, cudaMemcpyDeviceToHost, st));
    GBA_CUDA(ctx, cudaMemcpyAsync(&bounds, a.bounds, 4, cudaMemcpyDeviceToHost, st));
    GBA_CUDA(ctx, cudaMemcpyAsync(r->id_begin, a.id_begin, size_t(nrec) * 8, cudaMemcpyDeviceToHost, st));
    GBA_CUDA(ctx, cudaMemcpyAsync(r->id_end, a.id_end, size_t(nrec) * 8, cudaMemcpyDeviceToHost, st));
    GBA_CUDA(ctx, cudaMemcpyAsync(r->seq_off, a.seq_off, size_t(nrec) * 8, cudaMemcpyDeviceToHost, st));
    if (nres && r->codes && nres <= r->residue_capacity)
        GBA_CUDA(ctx, cudaMemcpyAsync(r->codes, a.codes, size_t(nres), cudaMemcpyDeviceToHost, st));
    if (dst) {
        GBA_CUDA(ctx, dst->ensure(size_t(nres) + 16));
        if (nres) GBA_CUDA(ctx, cudaMemcpyAsync(dst->ptr, a.codes, size_t(nres), cudaMemcpyDeviceToDevice, st));
    }
    GBA_CUDA(ctx, cudaEventRecord(ctx->ev[1], st));
    GBA_CUDA(ctx, cudaStreamSynchronize(st));
    r->seq_off[nrec] = nres;
    if (total.end[FA_BEFORE] == FA_HEADER) r->id_end[nrec - 1] = n;   // last header runs to the end
    if (r->qual_end)
        for (int64_t k = 0; k < nrec; ++k) r->qual_end[k] = r->seq_off[k];
    float ms = 0, call = 0;
    GBA_CUDA(ctx, cudaEventElapsedTime(&ms, ctx->ev[2], ctx->ev[3]));
    GBA_CUDA(ctx, cudaEventElapsedTime(&call, ctx->ev[0], ctx->ev[1]));
    ctx->stats = gba_stats{};
    ctx->stats.dp_kernel_ms = ms;
    ctx->stats.call_ms = call;
    ctx->stats.kernel_launches = 4;
    if (bounds) return fail(ctx, GBA_ECUDA, "FASTA record pass wrote outside the scanned totals (%u)", bounds);
    if (err != ~0ull) {
        r->error_offset = int64_t(err);
        return fail(ctx, GBA_EPARSE, "character outside the alphabet at offset %lld", (long long)err);
    }
    return GBA_OK;
}

}  // namespace gba

extern "C" {

GBA_API int gba_read_fasta(gba_context *ctx, const char *text, int64_t n, int32_t alphabet, gba_seq_records *r)
{
    return gba::fasta_parse(ctx, text, n, alphabet, r, nullptr);
}

GBA_API int gba_align_fasta(gba_context *ctx, const gba_params *params, const char *text_h, int64_t len_h,
                            const char *text_v, int64_t len_v, int32_t alphabet, int32_t h_shared,
                            int64_t pair_capacity, int64_t *num_pairs, gba_result *result)
{
    using namespace gba;
    if (!ctx || !params || !num_pairs || !result) return GBA_EINVAL;
    FaHostRecords rec[2];
    const char *texts[2] = {text_h, text_v};
    const int64_t lens[2] = {len_h, len_v};
    DevBuf *dst[2] = {&ctx->seq_h, &ctx->seq_v};
    for (int side = 0; side < 2; ++side) {
        gba_seq_records r{};
        if (int rc = fasta_parse(ctx, texts[side], lens[side], alphabet, &r, dst[side], &rec[side])) return rc;
    }
    std::vector<int64_t> off[2] = {std::move(rec[0].seq_off), std::move(rec[1].seq_off)};
    const int64_t nh = int64_t(off[0].size()) - 1, nv = int64_t(off[1].size()) - 1;
    *num_pairs = nv;
    if (h_shared ? nh != 1 : nh != nv)
        return fail(ctx, GBA_EINVAL, "FASTA texts hold %lld and %lld records", (long long)nh, (long long)nv);
    if (nv > pair_capacity) return fail(ctx, GBA_ECAPACITY, "%lld pairs, result arrays hold %lld", (long long)nv,
                                        (long long)pair_capacity);
    gba_batch b{};
    b.num_pairs = nv;
    b.off_h = off[0].data();
    b.off_v = off[1].data();
    b.h_shared = h_shared;
    ctx->device_codes = true;
    const int rc = gba_align_batch(ctx, params, &b, result);
    ctx->device_codes = false;
    return rc;
}

GBA_API int gba_read_fastq(gba_context *ctx, const char *text, int64_t n, int32_t alphabet, gba_seq_records *r)
{
    using namespace gba;
    int8_t cls[256];
    {
        const int rc = seqio_check(ctx, text, n, alphabet, r, cls);
        if (rc) return rc;
    }
    cls[uint8_t('>')] = FA_BAD;
    const uint8_t *t = reinterpret_cast<const uint8_t *>(text);
    FqCallerSink sink{r, r->codes && r->id_begin && r->id_end && r->seq_off};
    FqResult res;
    if (!fastq_read_parallel(t, n, cls, sink, res)) res = fastq_parse(t, n, 0, INT64_MAX, cls, sink);
    if (res.status) {
        r->error_offset = res.err_at;
        return ctx ? fail(ctx, res.status, "%s at offset %lld", res.what, (long long)res.err_at) : res.status;
    }
    const int64_t rec = sink.rec, nres = sink.res;
    r->num = rec;
    r->residues = nres;
    if (!sink.write || rec + 1 > r->record_capacity || nres > r->residue_capacity) {
        return ctx ? fail(ctx, GBA_ECAPACITY, "records need %lld record and %lld residue entries",
                          (long long)rec + 1, (long long)nres)
                   : GBA_ECAPACITY;
    }
    r->seq_off[rec] = nres;
    return GBA_OK;
}

}  // extern "C"
