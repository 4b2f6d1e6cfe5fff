// bgzf_host.cuh -- BGZF compression of a byte stream on the device (included at the end of
// engine.cu): gba_bgzf_compress.
//
// The reference's BamFileOut writes its BAM bytes through a BGZF stream
// (stream/stream_compressor.h:60-130, 325-375): pages of 65,505 input bytes, each compressed into
// one gzip member with the 18-byte BGZF header (extra field "BC" holding the member size - 1),
// the raw deflate data, the CRC-32 and the input size, and a 28-byte empty member at the end of the
// file.  The members here have the same partition, header, CRC-32 and sizes; the deflate data is
// this engine's own (zlib's level-1 matcher and its Huffman trees are not restated), so the
// compressed bytes differ while every member inflates to the same page.
//
// One warp per member, one lane per 2,048-byte segment of its page: greedy LZ77 over the segment
// (a 512-entry table of the last position of each 3-byte hash, in shared memory; matches of 3..258
// bytes inside the segment) coded with the fixed Huffman codes of RFC 1951 section 3.2.6 in a
// non-final block closed by an empty stored block, which ends it on a byte boundary (the flush
// marker 00 00 ff ff), so the lanes' bytes concatenate; an empty final fixed block (03 00) ends
// the stream.  A page whose coded form would not be smaller than one stored block (RFC 1951
// section 3.2.4) is written as that stored block.  Lane 0 computes the page's CRC-32.
#pragma once

namespace {

constexpr int kBgzfPage = 65505;                 // input bytes per member
constexpr int kBgzfMember = 65536;               // bytes reserved per member in the slots
constexpr int kBgzfHashBits = 9;
constexpr int kBgzfSegment = 2048;               // input bytes per lane
constexpr int kBgzfLaneCap = 2320;               // coded bytes a lane may produce (9 bits per byte + 16)

struct BgzfBits {
    uint8_t *out;
    int cap, n;
    uint64_t acc;
    int nacc;
    bool over;
    __host__ __device__ void put(uint32_t v, int bits)   // LSB first
    {
        acc |= uint64_t(v) << nacc;
        nacc += bits;
        while (nacc >= 8) {
            if (n < cap) out[n] = uint8_t(acc);
            else over = true;
            ++n;
            acc >>= 8;
            nacc -= 8;
        }
    }
    __host__ __device__ void flush()
    {
        if (nacc > 0) put(0, 8 - nacc);
    }
};

__host__ __device__ inline uint32_t bgzf_rev(uint32_t code, int len)
{
#ifdef __CUDA_ARCH__
    return __brev(code) >> (32 - len);
#else
    uint32_t r = 0;
    for (int i = 0; i < len; ++i) r |= ((code >> i) & 1u) << (len - 1 - i);
    return r;
#endif
}

__host__ __device__ inline int bgzf_log2(uint32_t x)   // x > 0
{
#ifdef __CUDA_ARCH__
    return 31 - __clz(x);
#else
    int r = 0;
    while (x >>= 1) ++r;
    return r;
#endif
}

// Fixed literal / length code v (0..287), bit-reversed for the LSB-first stream.
__host__ __device__ inline void bgzf_litlen(BgzfBits &b, int v)
{
    if (v < 144) b.put(bgzf_rev(0x30u + v, 8), 8);
    else if (v < 256) b.put(bgzf_rev(0x190u + (v - 144), 9), 9);
    else if (v < 280) b.put(bgzf_rev(uint32_t(v - 256), 7), 7);
    else b.put(bgzf_rev(0xC0u + (v - 280), 8), 8);
}

// A match of len 3..258 at distance 1..32768 (RFC 1951 section 3.2.5): the length code 257..285
// and the distance code 0..29 follow from the bit length of len - 3 and dist - 1 (four codes per
// extra bit for lengths, two for distances), their extra bits are the low bits.
__host__ __device__ inline void bgzf_match(BgzfBits &b, int len, int dist)
{
    const uint32_t l = uint32_t(len - 3);
    if (len == 258) {
        bgzf_litlen(b, 285);
    } else if (l < 8) {
        bgzf_litlen(b, 257 + int(l));
    } else {
        const int e = bgzf_log2(l) - 2;
        bgzf_litlen(b, 257 + 4 * e + int(l >> e));
        b.put(l & ((1u << e) - 1u), e);
    }
    const uint32_t d = uint32_t(dist - 1);
    if (d < 4) {
        b.put(bgzf_rev(d, 5), 5);
    } else {
        const int e = bgzf_log2(d) - 1;
        b.put(bgzf_rev(uint32_t(2 * e) + 2u + ((d >> e) & 1u), 5), 5);
        b.put(d & ((1u << e) - 1u), e);
    }
}

__host__ __device__ inline uint32_t bgzf_crc32(const uint8_t *p, int n, const uint32_t *table)
{
    uint32_t c = 0xffffffffu;
    for (int i = 0; i < n; ++i) c = table[(c ^ p[i]) & 0xffu] ^ (c >> 8);
    return c ^ 0xffffffffu;
}

__host__ __device__ inline void bgzf_put16(uint8_t *p, uint32_t v)
{
    p[0] = uint8_t(v);
    p[1] = uint8_t(v >> 8);
}
__host__ __device__ inline void bgzf_put32(uint8_t *p, uint32_t v)
{
    for (int i = 0; i < 4; ++i) p[i] = uint8_t(v >> (8 * i));
}

// The coded bytes of in[0, n) (n <= kBgzfSegment) as one non-final fixed-code block closed by an
// empty stored block (byte aligned); 0 bytes for n == 0.  table: 1 << kBgzfHashBits entries.
__host__ __device__ inline int bgzf_segment(const uint8_t *in, int n, uint8_t *out, uint16_t *table)
{
    if (n == 0) return 0;
    BgzfBits b{out, kBgzfLaneCap, 0, 0, 0, false};
    for (int i = 0; i < (1 << kBgzfHashBits); ++i) table[i] = 0xffffu;
    b.put(0u, 1);   // BFINAL 0
    b.put(1u, 2);   // BTYPE 01: fixed Huffman codes
    int pos = 0;
    while (pos < n) {
        if (pos + 3 <= n) {
            const uint32_t key = uint32_t(in[pos]) | (uint32_t(in[pos + 1]) << 8) | (uint32_t(in[pos + 2]) << 16);
            const uint32_t h = (key * 2654435761u) >> (32 - kBgzfHashBits);
            const int cand = table[h];
            table[h] = uint16_t(pos);
            if (cand != 0xffff && in[cand] == in[pos] && in[cand + 1] == in[pos + 1] && in[cand + 2] == in[pos + 2]) {
                int len = 3;
                while (len < 258 && pos + len < n && in[cand + len] == in[pos + len]) ++len;
                bgzf_match(b, len, pos - cand);
                pos += len;
                continue;
            }
        }
        bgzf_litlen(b, in[pos]);
        ++pos;
    }
    bgzf_litlen(b, 256);
    b.put(0u, 3);   // BFINAL 0, BTYPE 00: an empty stored block
    b.flush();
    b.put(0u, 16);
    b.put(0xffffu, 16);
    return b.n;
}

// Member framing around clen coded bytes already at out + 18.
__host__ __device__ inline int bgzf_frame(uint8_t *out, int clen, uint32_t crc, int n)
{
    const uint8_t head[18] = {0x1f, 0x8b, 0x08, 4, 0, 0, 0, 0, 0, 0xff, 6, 0, 'B', 'C', 2, 0, 0, 0};
    for (int i = 0; i < 16; ++i) out[i] = head[i];
    const int size = 18 + clen + 8;
    bgzf_put16(out + 16, uint32_t(size - 1));
    bgzf_put32(out + 18 + clen, crc);
    bgzf_put32(out + 18 + clen + 4, uint32_t(n));
    return size;
}

struct BgzfArgs {
    const uint8_t *in;
    int64_t n;
    int64_t members;
    uint8_t *slots;        // kBgzfMember bytes per member
    uint8_t *scratch;      // 32 x kBgzfLaneCap bytes per member
    int32_t *sizes;
    const uint32_t *crc_table;
};

// One warp per member, one member per block (32 x 1 KiB of hash tables in shared memory).
__global__ void __launch_bounds__(32) k_bgzf_members(BgzfArgs a)
{
    __shared__ uint16_t table[32][1 << kBgzfHashBits];
    __shared__ uint32_t crc[256];
    for (int i = threadIdx.x; i < 256; i += blockDim.x) crc[i] = a.crc_table[i];
    __syncthreads();
    const int lane = threadIdx.x & 31;
    const int64_t m = blockIdx.x;
    if (m >= a.members) return;
    const int64_t off = m * kBgzfPage;
    const int n = int(a.n - off < kBgzfPage ? a.n - off : kBgzfPage);
    const uint8_t *page = a.in + off;
    uint8_t *scr = a.scratch + m * (32 * int64_t(kBgzfLaneCap)) + lane * kBgzfLaneCap;
    const int s0 = lane * kBgzfSegment < n ? lane * kBgzfSegment : n;
    const int s1 = s0 + kBgzfSegment < n ? s0 + kBgzfSegment : n;
    const int len = bgzf_segment(page + s0, s1 - s0, scr, table[threadIdx.x]);
    // exclusive prefix of the lanes' byte counts
    int pre = len;
    for (int d = 1; d < 32; d <<= 1) {
        const int v = __shfl_up_sync(0xffffffffu, pre, d);
        if (lane >= d) pre += v;
    }
    const int total = __shfl_sync(0xffffffffu, pre, 31) + 2;   // + the final empty block
    pre -= len;
    uint8_t *out = a.slots + m * kBgzfMember;
    int clen;
    if (total <= n + 5) {
        for (int i = 0; i < len; ++i) out[18 + pre + i] = scr[i];
        if (lane == 31) {
            out[18 + total - 2] = 0x03;   // BFINAL 1, BTYPE 01, end of block
            out[18 + total - 1] = 0x00;
        }
        clen = total;
    } else {
        // one stored block: BFINAL 1, BTYPE 00, byte-aligned LEN and NLEN, the bytes
        for (int i = lane; i < n; i += 32) out[18 + 5 + i] = page[i];
        if (lane == 0) {
            out[18] = 1;
            bgzf_put16(out + 19, uint32_t(n));
            bgzf_put16(out + 21, uint32_t(~n & 0xffff));
        }
        clen = n + 5;
    }
    __syncwarp();
    if (lane == 0) a.sizes[m] = bgzf_frame(out, clen, bgzf_crc32(page, n, crc), n);
}

__global__ void __launch_bounds__(128) k_bgzf_pack(const uint8_t *slots, const int32_t *sizes, const int64_t *offs,
                                                   uint8_t *out, int64_t members)
{
    // one block per member, its threads copy the member's bytes
    const int64_t m = blockIdx.x;
    if (m >= members) return;
    const uint8_t *src = slots + m * kBgzfMember;
    uint8_t *dst = out + offs[m];
    for (int i = threadIdx.x; i < sizes[m]; i += blockDim.x) dst[i] = src[i];
}

}  // namespace

extern "C" {

GBA_API int gba_bgzf_compress(gba_context *ctx, const uint8_t *data, int64_t n, int32_t eof_marker, uint8_t *out,
                              int64_t capacity, int64_t *out_len)
{
    if (!ctx || !out_len || n < 0 || (n > 0 && !data)) return GBA_EINVAL;
    const auto t0 = std::chrono::steady_clock::now();
    GBA_CUDA(ctx, cudaSetDevice(ctx->device));
    cudaStream_t st = ctx->stream;
    const int64_t members = (n + kBgzfPage - 1) / kBgzfPage;
    static const uint8_t eof[28] = {0x1f, 0x8b, 0x08, 0x04, 0, 0, 0, 0, 0, 0xff, 0x06, 0, 0x42, 0x43, 0x02, 0,
                                    0x1b, 0, 0x03, 0, 0, 0, 0, 0, 0, 0, 0, 0};
    int64_t total = 0;
    float ms = 0;
    int launches = 0;
    std::vector<int64_t> offs(size_t(members) + 1, 0);
    if (members > 0) {
        uint32_t crc_table[256];
        for (uint32_t i = 0; i < 256; ++i) {   // CRC-32, reflected polynomial 0xEDB88320
            uint32_t c = i;
            for (int k = 0; k < 8; ++k) c = (c & 1u) ? 0xEDB88320u ^ (c >> 1) : c >> 1;
            crc_table[i] = c;
        }
        GBA_CUDA(ctx, ctx->bz_in.ensure(size_t(n) + 16));
        GBA_CUDA(ctx, ctx->bz_slots.ensure(size_t(members) * kBgzfMember));
        GBA_CUDA(ctx, ctx->bz_scratch.ensure(size_t(members) * 32 * kBgzfLaneCap));
        GBA_CUDA(ctx, ctx->bz_meta.ensure(size_t(members) * 4 + 1024 + size_t(members + 1) * 8 + 16));
        uint32_t *dcrc = ctx->bz_meta.as<uint32_t>();
        int32_t *dsizes = reinterpret_cast<int32_t *>(dcrc + 256);
        int64_t *doffs = reinterpret_cast<int64_t *>(ctx->bz_meta.as<uint8_t>() + ((1024 + size_t(members) * 4 + 7) & ~size_t(7)));
        GBA_CUDA(ctx, cudaMemcpyAsync(ctx->bz_in.ptr, data, size_t(n), cudaMemcpyHostToDevice, st));
        GBA_CUDA(ctx, cudaMemcpyAsync(dcrc, crc_table, sizeof(crc_table), cudaMemcpyHostToDevice, st));
        BgzfArgs a{ctx->bz_in.as<uint8_t>(), n, members, ctx->bz_slots.as<uint8_t>(), ctx->bz_scratch.as<uint8_t>(),
                   dsizes, dcrc};
        GBA_CUDA(ctx, cudaEventRecord(ctx->ev[0], st));
        k_bgzf_members<<<unsigned(members), 32, 0, st>>>(a);
        GBA_CUDA(ctx, cudaGetLastError());
        GBA_CUDA(ctx, cudaEventRecord(ctx->ev[1], st));
        ++launches;
        std::vector<int32_t> sizes(static_cast<size_t>(members));
        GBA_CUDA(ctx, cudaMemcpyAsync(sizes.data(), dsizes, size_t(members) * 4, cudaMemcpyDeviceToHost, st));
        GBA_CUDA(ctx, cudaStreamSynchronize(st));
        GBA_CUDA(ctx, cudaEventElapsedTime(&ms, ctx->ev[0], ctx->ev[1]));
        for (int64_t m = 0; m < members; ++m) offs[m + 1] = offs[m] + sizes[m];
        total = offs[members];
    }
    const int64_t need = total + (eof_marker ? 28 : 0);
    *out_len = need;
    if (need > capacity || (need > 0 && !out)) return fail(ctx, GBA_ECAPACITY, "bgzf output needs %lld bytes", (long long)need);
    if (members > 0) {
        int64_t *doffs = reinterpret_cast<int64_t *>(ctx->bz_meta.as<uint8_t>() + ((1024 + size_t(members) * 4 + 7) & ~size_t(7)));
        int32_t *dsizes = reinterpret_cast<int32_t *>(ctx->bz_meta.as<uint32_t>() + 256);
        GBA_CUDA(ctx, ctx->bz_out.ensure(size_t(total) + 16));
        GBA_CUDA(ctx, cudaMemcpyAsync(doffs, offs.data(), size_t(members) * 8, cudaMemcpyHostToDevice, st));
        k_bgzf_pack<<<unsigned(members), 128, 0, st>>>(ctx->bz_slots.as<uint8_t>(), dsizes, doffs,
                                                       ctx->bz_out.as<uint8_t>(), members);
        GBA_CUDA(ctx, cudaGetLastError());
        ++launches;
        GBA_CUDA(ctx, cudaMemcpyAsync(out, ctx->bz_out.ptr, size_t(total), cudaMemcpyDeviceToHost, st));
        GBA_CUDA(ctx, cudaStreamSynchronize(st));
    }
    if (eof_marker) std::memcpy(out + total, eof, 28);
    ctx->stats = gba_stats{};
    ctx->stats.dp_kernel_ms = ms;
    ctx->stats.kernel_launches = launches;
    ctx->stats.call_ms = std::chrono::duration<float, std::milli>(std::chrono::steady_clock::now() - t0).count();
    return GBA_OK;
}

}  // extern "C"
