// packed_host.cuh -- gba_align_packed: packed strings (String<TValue, Packed<>>, sequence/
// string_packed.h) uploaded as their host words and unpacked on the device into the engine's code
// buffers, then aligned by gba_align_batch (included at the end of engine.cu).
#pragma once

namespace gba {

// One warp per packed string: lanes take its data words in turn and write the N values of each.
__global__ void __launch_bounds__(128) k_unpack_packed(const uint64_t *words, const int64_t *word_off,
                                                       const int64_t *res_off, int64_t num, int bits,
                                                       uint8_t *codes)
{
    const int64_t k = (int64_t(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (k >= num) return;
    const int64_t len = res_off[k + 1] - res_off[k];
    if (len == 0) return;
    const int N = 64 / bits;
    const uint64_t mask = (uint64_t(1) << bits) - 1;
    const uint64_t *data = words + word_off[k] + 1;
    uint8_t *out = codes + res_off[k];
    const int64_t nw = (len + N - 1) / N;
    for (int64_t w = lane; w < nw; w += 32) {
        const uint64_t x = data[w];
        const int64_t base = w * N;
        const int cnt = len - base < N ? int(len - base) : N;
        for (int i = 0; i < cnt; ++i) out[base + i] = uint8_t((x >> ((N - 1 - i) * bits)) & mask);
    }
}

}  // namespace gba

namespace {

// Reads the strings' lengths from their length words into residue offsets and checks the sizes.
int packed_offsets(gba_context *ctx, const gba_packed_set *s, std::vector<int64_t> &off)
{
    if (!s || s->num < 0 || (s->num > 0 && !s->word_off)) return fail(ctx, GBA_EINVAL, "bad packed set");
    if (s->bits_per_value != 2 && s->bits_per_value != 3 && s->bits_per_value != 5)
        return fail(ctx, GBA_EINVAL, "bits_per_value must be 2, 3 or 5");
    const int N = 64 / s->bits_per_value;
    if (s->num > 0 && s->word_off[s->num] > s->word_off[0] && !s->words)
        return fail(ctx, GBA_EINVAL, "null packed words");
    off.assign(size_t(s->num) + 1, 0);
    // lengths from the length words (in parallel: one host word read per string), then the offsets
    int64_t bad = -1;
    const int threads = plan_threads(s->num * 4);
#pragma omp parallel for num_threads(threads) schedule(static) reduction(max : bad)
    for (int64_t k = 0; k < s->num; ++k) {
        const int64_t nw = s->word_off[k + 1] - s->word_off[k];
        int64_t len = 0;
        if (nw > 0) len = int64_t(s->words[s->word_off[k]]);
        if (nw < 0 || len < 0 || (nw > 0 && nw != 1 + (len + N - 1) / N)) bad = std::max(bad, k);
        off[k + 1] = len;
    }
    if (bad >= 0) return fail(ctx, GBA_EINVAL, "packed string %lld: its words do not hold its length", (long long)bad);
    for (int64_t k = 0; k < s->num; ++k) off[k + 1] += off[k];
    return GBA_OK;
}

// Queues the words' copy and their unpacking on the context stream; nothing waits, so the copies
// overlap the host's planning as gba_align_batch's own upload does.  (Pageable offsets are staged
// by cudaMemcpyAsync before it returns.)
int packed_copy_words(gba_context *ctx, const gba_packed_set *s, size_t words_at)
{
    const int64_t nw = s->num ? s->word_off[s->num] - s->word_off[0] : 0;
    if (nw > 0)
        GBA_CUDA(ctx, cudaMemcpyAsync(ctx->pk_words.as<char>() + words_at, s->words + s->word_off[0], size_t(nw) * 8,
                                      cudaMemcpyHostToDevice, ctx->stream));
    return GBA_OK;
}

int packed_upload(gba_context *ctx, const gba_packed_set *s, const std::vector<int64_t> &off, DevBuf &codes,
                  DevBuf &offbuf, size_t words_at)
{
    cudaStream_t st = ctx->stream;
    const int64_t nw = s->num ? s->word_off[s->num] - s->word_off[0] : 0;
    GBA_CUDA(ctx, codes.ensure(size_t(off.back()) + 16));
    if (nw == 0) return GBA_OK;
    char *wbase = ctx->pk_words.as<char>() + words_at;
    // word offsets rebased to the copied words, then residue offsets, in the offsets buffer
    std::vector<int64_t> wo(size_t(s->num) + 1);
    for (int64_t k = 0; k <= s->num; ++k) wo[k] = s->word_off[k] - s->word_off[0];
    GBA_CUDA(ctx, offbuf.ensure(size_t(2 * (s->num + 1)) * 8));
    int64_t *dwo = offbuf.as<int64_t>();
    int64_t *dro = dwo + (s->num + 1);
    GBA_CUDA(ctx, cudaMemcpyAsync(dwo, wo.data(), wo.size() * 8, cudaMemcpyHostToDevice, st));
    GBA_CUDA(ctx, cudaMemcpyAsync(dro, off.data(), off.size() * 8, cudaMemcpyHostToDevice, st));
    const unsigned grid = unsigned((s->num * 32 + 127) / 128);
    k_unpack_packed<<<grid, 128, 0, st>>>(reinterpret_cast<const uint64_t *>(wbase), dwo, dro, s->num,
                                          s->bits_per_value, codes.as<uint8_t>());
    GBA_CUDA(ctx, cudaGetLastError());
    return GBA_OK;
}

}  // namespace

extern "C" {

GBA_API int gba_align_packed(gba_context *ctx, const gba_params *params, const gba_packed_set *h,
                             const gba_packed_set *v, int32_t h_shared, gba_result *result)
{
    if (!ctx || !params || !h || !v || !result) return GBA_EINVAL;
    GBA_CUDA(ctx, cudaSetDevice(ctx->device));
    if (h->num < 0 || v->num < 0 || (h->num && !h->word_off) || (v->num && !v->word_off))
        return fail(ctx, GBA_EINVAL, "bad packed set");
    const int64_t hw = h->num ? h->word_off[h->num] - h->word_off[0] : 0;
    const int64_t vw = v->num ? v->word_off[v->num] - v->word_off[0] : 0;
    if (hw < 0 || vw < 0) return fail(ctx, GBA_EINVAL, "packed word offsets decrease");
    if ((hw && !h->words) || (vw && !v->words)) return fail(ctx, GBA_EINVAL, "null packed words");
    // the words' copies first: they run while the host reads the lengths
    GBA_CUDA(ctx, ctx->pk_words.ensure(size_t(hw + vw) * 8 + 16));
    if (int rc = packed_copy_words(ctx, h, 0)) return rc;
    if (int rc = packed_copy_words(ctx, v, size_t(hw) * 8)) return rc;
    std::vector<int64_t> off_h, off_v;
    if (int rc = packed_offsets(ctx, h, off_h)) return rc;
    if (int rc = packed_offsets(ctx, v, off_v)) return rc;
    const int64_t N = v->num;
    if (h_shared ? h->num != 1 : h->num != N) return fail(ctx, GBA_EINVAL, "packed sets of different sizes");
    if (int rc = packed_upload(ctx, h, off_h, ctx->seq_h, ctx->pk_off_h, 0)) return rc;
    if (int rc = packed_upload(ctx, v, off_v, ctx->seq_v, ctx->pk_off_v, size_t(hw) * 8)) return rc;
    gba_batch b{};
    b.num_pairs = N;
    b.seq_h = nullptr;
    b.off_h = off_h.data();
    b.seq_v = nullptr;
    b.off_v = off_v.data();
    b.h_shared = h_shared;
    ctx->device_codes = true;
    const int rc = gba_align_batch(ctx, params, &b, result);
    ctx->device_codes = false;
    return rc;
}

}  // extern "C"
