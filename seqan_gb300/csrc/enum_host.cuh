// enum_host.cuh -- host side of gba_local_enumerate (included at the end of engine.cu).
//
// Each pair gets its own scratch in HBM (score matrix, forbidden flags, heap, trace steps and
// segment slots, about 17 bytes per matrix cell plus the slots); pairs are processed in chunks
// whose scratch fits kEnumScratchBudget.  After the kernel the per-alignment segment counts come
// back, the host lays out the dense output and a pack kernel copies the used slots.
#pragma once

#include "enum_kernels.cuh"

namespace {

constexpr size_t kEnumScratchBudget = size_t(6) << 30;

__global__ void __launch_bounds__(128) k_enum_pack(const uint32_t *slots, const int64_t *slot_off,
                                                   const int32_t *count, const int64_t *dense_off, uint32_t *dense,
                                                   int64_t num)
{
    const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= num) return;
    const int32_t c = count[i];
    const uint32_t *src = slots + 4 * slot_off[i];
    uint32_t *dst = dense + 4 * dense_off[i];
    for (int32_t q = 0; q < 4 * c; ++q) dst[q] = src[q];
}

// Band storage of LocalAlignmentEnumerator<Score, Banded> for an m x n pair: cells of the
// stored matrix (diagonalWidth x rows, _initLocalAlignmentFinder), 0 when the band misses it.
int64_t enum_band_cells(int64_t m, int64_t n, int64_t lower, int64_t upper)
{
    const int64_t W = upper - lower + 1, lo_row = upper <= 0 ? -upper : 0;
    int64_t hi_init = n + 1, hi_fill = n;
    if (m - lower >= 0 && m - lower < hi_init) hi_init = m - lower;
    if (m - lower >= 0 && m - lower < hi_fill) hi_fill = m - lower;
    if (m <= 0 || n <= 0 || hi_init - lo_row + 1 <= 0 || hi_fill - lo_row + 1 <= 0) return 0;
    return W * (hi_init - lo_row + 1);
}

// gba_local_enumerate (band == nullptr) and gba_local_enumerate_banded (band = {lower, upper}).
int enumerate_impl(gba_context *ctx, const gba_enum_params *params, const int32_t *band, const gba_batch *b,
                   gba_enum_result *res)
{
    if (!ctx || !params || !b || !res) return GBA_EINVAL;
    const auto t0 = std::chrono::steady_clock::now();
    GBA_CUDA(ctx, cudaSetDevice(ctx->device));
    const int64_t N = b->num_pairs;
    const int32_t K = params->max_count;
    if (N < 0) return fail(ctx, GBA_EINVAL, "negative num_pairs");
    if (K < 1 || K > 65536) return fail(ctx, GBA_EINVAL, "max_count must be in 1..65536");
    const int lim = 1 << 20;
    if (std::abs(params->match) > lim || std::abs(params->mismatch) > lim || std::abs(params->gap) > lim ||
        std::abs(params->cutoff) > lim)
        return fail(ctx, GBA_EUNSUPPORTED, "scores beyond +-2^20");
    if (band) {
        if (band[1] < band[0]) return fail(ctx, GBA_EINVAL, "upper_diag below lower_diag");
        if (std::abs(band[0]) > (1 << 30) || std::abs(band[1]) > (1 << 30))
            return fail(ctx, GBA_EUNSUPPORTED, "diagonals beyond +-2^30");
    }
    std::vector<int32_t> mat;
    if (params->matrix) {
        if (params->alphabet_size < 1 || params->alphabet_size > 32)
            return fail(ctx, GBA_EINVAL, "matrix alphabet_size must be 1..32");
        mat.assign(params->matrix, params->matrix + params->alphabet_size * params->alphabet_size);
        for (int32_t x : mat)
            if (std::abs(x) > lim) return fail(ctx, GBA_EUNSUPPORTED, "matrix scores beyond +-2^20");
    }
    if (!res->count || !res->status || !res->score || !res->begin_h || !res->end_h || !res->begin_v ||
        !res->end_v || !res->segment_offsets)
        return fail(ctx, GBA_EINVAL, "null result array");
    res->segment_offsets[0] = 0;
    if (N == 0) return GBA_OK;
    if (!b->off_h || !b->off_v || !b->seq_h || !b->seq_v) return fail(ctx, GBA_EINVAL, "null sequence or offset pointer");
    cudaStream_t st = ctx->stream;
    const int64_t hbytes = b->h_shared ? b->off_h[1] : b->off_h[N], vbytes = b->off_v[N];
    GBA_CUDA(ctx, ctx->seq_h.ensure(size_t(hbytes) + 16));
    GBA_CUDA(ctx, ctx->seq_v.ensure(size_t(vbytes) + 16));
    if (hbytes) GBA_CUDA(ctx, cudaMemcpyAsync(ctx->seq_h.ptr, b->seq_h, hbytes, cudaMemcpyHostToDevice, st));
    if (vbytes) GBA_CUDA(ctx, cudaMemcpyAsync(ctx->seq_v.ptr, b->seq_v, vbytes, cudaMemcpyHostToDevice, st));
    if (!mat.empty()) {
        GBA_CUDA(ctx, ctx->xs_matrix.ensure(mat.size() * 4));
        GBA_CUDA(ctx, cudaMemcpyAsync(ctx->xs_matrix.ptr, mat.data(), mat.size() * 4, cudaMemcpyHostToDevice, st));
    }
    std::vector<EnumPair> pairs(static_cast<size_t>(N));
    std::vector<size_t> need(static_cast<size_t>(N));
    std::vector<int64_t> cells_of(static_cast<size_t>(N));
    for (int64_t k = 0; k < N; ++k) {
        const int64_t h0 = b->h_shared ? b->off_h[0] : b->off_h[k], h1 = b->h_shared ? b->off_h[1] : b->off_h[k + 1];
        const int64_t v0 = b->off_v[k], v1 = b->off_v[k + 1];
        if (h0 < 0 || v0 < 0 || h1 < h0 || v1 < v0) return fail(ctx, GBA_EINVAL, "bad offsets of pair %lld", (long long)k);
        const int64_t m = h1 - h0, n = v1 - v0;
        if (m > (int64_t(1) << 30) || n > (int64_t(1) << 30))
            return fail(ctx, GBA_EUNSUPPORTED, "pair %lld: sequence of more than 2^30 residues", (long long)k);
        const int64_t cells = band ? enum_band_cells(m, n, band[0], band[1]) : (m + 1) * (n + 1);
        if (cells > (int64_t(1) << 31) - 1)
            return fail(ctx, GBA_EUNSUPPORTED, "pair %lld: matrix of more than 2^31 cells", (long long)k);
        EnumPair &d = pairs[k];
        d.h_off = h0;
        d.v_off = v0;
        d.m = int32_t(m);
        d.n = int32_t(n);
        // banded: the fill pushes each cell once, a declump at most each cell again, so
        // max_count pushes per cell bound the heap; the first launch gives room for up to 16 per
        // cell, and a pair that needs more (max_count > 16) is rerun with the bound
        d.heap_cap = band ? int64_t(K < 16 ? K : 16) * cells + 16 : m * n;
        cells_of[k] = cells;
        need[k] = size_t(cells) * 5 + size_t(d.heap_cap) * 8 + size_t(2 * (m + n + 5)) * 4 +
                  size_t(K) * size_t(m + n + 1) * 16 + 64;
        if (need[k] > kEnumScratchBudget) return fail(ctx, GBA_EUNSUPPORTED, "pair %lld needs more scratch than one chunk", (long long)k);
    }
    std::vector<int64_t> slot_off(size_t(N) * K, 0);
    int64_t w = 0;   // segments written to the result
    float dp_ms = 0;
    int launches = 0;
    int64_t c0 = 0;
    while (c0 < N) {
        // one chunk: consecutive pairs whose scratch fits the budget
        int64_t c1 = c0;
        size_t tot = 0;
        while (c1 < N && tot + need[c1] <= kEnumScratchBudget) tot += need[c1++];
        const int64_t nc = c1 - c0, na = nc * K;
        int32_t *o = nullptr;
        std::vector<int32_t> outh(size_t(na) * 6 + size_t(nc) * 2);
        for (int attempt = 0;; ++attempt) {
        int64_t mo = 0, fo = 0, ho = 0, so = 0, go = 0;
        for (int64_t k = c0; k < c1; ++k) {
            EnumPair &d = pairs[k];
            const int64_t cells = cells_of[k];
            d.mat_off = mo;
            mo += cells;
            d.forb_off = fo;
            fo += cells;
            d.heap_off = ho;
            ho += d.heap_cap;
            d.step_off = so;
            so += 2 * int64_t(d.m + d.n + 5);
            d.seg_off = go;
            for (int32_t i = 0; i < K; ++i) slot_off[k * K + i] = go + int64_t(i) * (d.m + d.n + 1);
            go += int64_t(K) * (d.m + d.n + 1);
        }
        GBA_CUDA(ctx, ctx->en_pairs.ensure(size_t(nc) * sizeof(EnumPair)));
        GBA_CUDA(ctx, ctx->en_mat.ensure(size_t(mo) * 4 + 16));
        GBA_CUDA(ctx, ctx->en_forb.ensure(size_t(fo) + 16));
        GBA_CUDA(ctx, ctx->en_heap.ensure(size_t(ho) * 8 + 16));
        GBA_CUDA(ctx, ctx->en_steps.ensure(size_t(so) * 4 + 16));
        GBA_CUDA(ctx, ctx->en_slots.ensure(size_t(go) * 16 + 16));
        GBA_CUDA(ctx, ctx->en_out.ensure(size_t(na) * 6 * 4 + size_t(nc) * 2 * 4 + 64));
        GBA_CUDA(ctx, cudaMemcpyAsync(ctx->en_pairs.ptr, pairs.data() + c0, size_t(nc) * sizeof(EnumPair),
                                      cudaMemcpyHostToDevice, st));
        if (band) {   // the band storage starts zeroed, as the reference's matrix does
            GBA_CUDA(ctx, cudaMemsetAsync(ctx->en_mat.ptr, 0, size_t(mo) * 4, st));
            GBA_CUDA(ctx, cudaMemsetAsync(ctx->en_forb.ptr, 0, size_t(fo), st));
        }
        o = ctx->en_out.as<int32_t>();
        EnumArgs a{};
        a.seq_h = ctx->seq_h.as<uint8_t>();
        a.seq_v = ctx->seq_v.as<uint8_t>();
        a.pairs = ctx->en_pairs.as<EnumPair>();
        a.num_pairs = nc;
        a.mat = ctx->en_mat.as<int32_t>();
        a.forb = ctx->en_forb.as<uint8_t>();
        a.heap = ctx->en_heap.as<int2>();
        a.steps = ctx->en_steps.as<int32_t>();
        a.seg_slots = ctx->en_slots.as<uint32_t>();
        a.score = o;
        a.begin_h = o + na;
        a.end_h = o + 2 * na;
        a.begin_v = o + 3 * na;
        a.end_v = o + 4 * na;
        a.seg_count = o + 5 * na;
        a.count = o + 6 * na;
        a.status = o + 6 * na + nc;
        a.matrix = mat.empty() ? nullptr : ctx->xs_matrix.as<int32_t>();
        a.alphabet = mat.empty() ? 0 : params->alphabet_size;
        a.match = params->match;
        a.mismatch = params->mismatch;
        a.gap = params->gap;
        a.cutoff = params->cutoff;
        a.max_count = K;
        GBA_CUDA(ctx, cudaMemsetAsync(a.seg_count, 0, size_t(na) * 4, st));
        GBA_CUDA(ctx, cudaEventRecord(ctx->ev[0], st));
        {
            // Each pair is one thread's sequential enumeration whose heap and declump steps take
            // data-dependent branches, so the lanes of a warp diverge and run one after another.
            // A warp therefore takes few pairs -- the smallest power of two that still fits
            // the batch into the resident warps (measured on 10,000 pairs of 100-200 bp: 2 pairs
            // per warp 2.4x faster than 32, 4 per warp 2.0x) -- and blocks are one warp each.
            // "Fits" allows two warps per resident warp slot.
            const void *fn = band ? reinterpret_cast<const void *>(&k_waterman_eggert_banded)
                                  : reinterpret_cast<const void *>(&k_waterman_eggert);
            const int64_t resident = persistent_grid(ctx, fn) * (kBlock / 32);
            a.lanes = 2;
            while (a.lanes < 32 && 2 * int64_t(a.lanes) * resident < nc) a.lanes *= 2;
            const int64_t warps = (nc + a.lanes - 1) / a.lanes;
            if (band)
                k_waterman_eggert_banded<<<unsigned(warps), 32, 0, st>>>(a, band[0], band[1]);
            else
                k_waterman_eggert<<<unsigned(warps), 32, 0, st>>>(a);
        }
        GBA_CUDA(ctx, cudaGetLastError());
        GBA_CUDA(ctx, cudaEventRecord(ctx->ev[1], st));
        ++launches;
        // results of the chunk
        GBA_CUDA(ctx, cudaMemcpyAsync(outh.data(), o, outh.size() * 4, cudaMemcpyDeviceToHost, st));
        GBA_CUDA(ctx, cudaStreamSynchronize(st));
        {
            float ms = 0;
            GBA_CUDA(ctx, cudaEventElapsedTime(&ms, ctx->ev[0], ctx->ev[1]));
            dp_ms += ms;
        }
        bool rerun = false;
        for (int64_t k = 0; k < nc; ++k)
            if (outh[size_t(6 * na + nc + k)] == 2) {
                EnumPair &d = pairs[c0 + k];
                const int64_t bound = int64_t(K) * cells_of[c0 + k] + 16;
                if (attempt > 0 || d.heap_cap >= bound)
                    return fail(ctx, GBA_EUNSUPPORTED, "pair %lld: heap beyond its bound", (long long)(c0 + k));
                d.heap_cap = bound;
                rerun = true;
            }
        if (!rerun) break;
        }
        std::vector<int64_t> dense(size_t(na) + 1, 0), src(size_t(na), 0);
        for (int64_t i = 0; i < na; ++i) {
            const int64_t pk = c0 + i / K, ik = i % K;
            const int32_t cnt = outh[size_t(6 * na + i / K)];
            const int32_t c = ik < cnt ? outh[size_t(5 * na + i)] : 0;
            dense[i + 1] = dense[i] + c;
            src[i] = slot_off[pk * K + ik];
            const int64_t gi = pk * K + ik;
            res->score[gi] = ik < cnt ? outh[size_t(i)] : 0;
            res->begin_h[gi] = ik < cnt ? outh[size_t(na + i)] : 0;
            res->end_h[gi] = ik < cnt ? outh[size_t(2 * na + i)] : 0;
            res->begin_v[gi] = ik < cnt ? outh[size_t(3 * na + i)] : 0;
            res->end_v[gi] = ik < cnt ? outh[size_t(4 * na + i)] : 0;
        }
        for (int64_t k = 0; k < nc; ++k) {
            res->count[c0 + k] = outh[size_t(6 * na + k)];
            res->status[c0 + k] = outh[size_t(6 * na + nc + k)];
        }
        const int64_t total = dense[na];
        if (w + total > res->segment_capacity || (total && !res->segments))
            return fail(ctx, GBA_ECAPACITY, "segment_capacity too small");
        if (total) {
            GBA_CUDA(ctx, ctx->en_dense.ensure(size_t(total) * 16 + 16));
            GBA_CUDA(ctx, ctx->en_offs.ensure(size_t(2 * na + 1) * 8 + 16));
            GBA_CUDA(ctx, ctx->en_cnt.ensure(size_t(na) * 4 + 16));
            int64_t *doff = ctx->en_offs.as<int64_t>();
            GBA_CUDA(ctx, cudaMemcpyAsync(doff, src.data(), size_t(na) * 8, cudaMemcpyHostToDevice, st));
            GBA_CUDA(ctx, cudaMemcpyAsync(doff + na, dense.data(), size_t(na) * 8, cudaMemcpyHostToDevice, st));
            std::vector<int32_t> cnts(static_cast<size_t>(na));
            for (int64_t i = 0; i < na; ++i) cnts[i] = int32_t(dense[i + 1] - dense[i]);
            GBA_CUDA(ctx, cudaMemcpyAsync(ctx->en_cnt.ptr, cnts.data(), size_t(na) * 4, cudaMemcpyHostToDevice, st));
            k_enum_pack<<<unsigned((na + 127) / 128), 128, 0, st>>>(ctx->en_slots.as<uint32_t>(), doff,
                                                                     ctx->en_cnt.as<int32_t>(), doff + na,
                                                                     ctx->en_dense.as<uint32_t>(), na);
            GBA_CUDA(ctx, cudaGetLastError());
            ++launches;
            GBA_CUDA(ctx, cudaMemcpyAsync(res->segments + w, ctx->en_dense.ptr, size_t(total) * 16,
                                          cudaMemcpyDeviceToHost, st));
            GBA_CUDA(ctx, cudaStreamSynchronize(st));
        }
        for (int64_t i = 0; i < na; ++i) res->segment_offsets[c0 * K + i + 1] = w + dense[i + 1];
        w += total;
        c0 = c1;
    }
    ctx->stats = gba_stats{};
    ctx->stats.dp_kernel_ms = dp_ms;
    ctx->stats.kernel_launches = launches;
    ctx->stats.call_ms = std::chrono::duration<float, std::milli>(std::chrono::steady_clock::now() - t0).count();
    return GBA_OK;
}

}  // namespace

extern "C" {

GBA_API int gba_local_enumerate(gba_context *ctx, const gba_enum_params *params, const gba_batch *batch,
                                gba_enum_result *result)
{
    return enumerate_impl(ctx, params, nullptr, batch, result);
}

GBA_API int gba_local_enumerate_banded(gba_context *ctx, const gba_enum_params *params, int32_t lower_diag,
                                       int32_t upper_diag, const gba_batch *batch, gba_enum_result *result)
{
    const int32_t band[2] = {lower_diag, upper_diag};
    return enumerate_impl(ctx, params, band, batch, result);
}

}  // extern "C"
