// seeds_host.cuh -- host side of gba_extend_seeds / gba_extend_seeds_device (included at the end
// of engine.cu, which defines gba_context).
//
// One call extends a whole batch: the seeds go to the device, one thread per seed runs the
// reference's extension (seed_kernels.cuh), and the seeds come back grown in place.  Gapped
// x-drop seeds first run with a 32- or 64-slot shared-memory ring per thread, picked from the
// band width the drop-off allows (X / |gap| columns on each side of the seed's diagonal); the
// few whose live range outgrows it are re-run by the fallback kernel with a global ring that
// holds the longest query, right after on the same stream (no host round trip).
#pragma once

namespace {

constexpr int64_t kSeedMaxGappedLen = int64_t(1) << 29;   // 2 * max(rows, cols) must fit int
constexpr int32_t kSeedMaxWideRing = 1 << 20;             // widest live range the fallback holds
constexpr size_t kSeedWideScratch = size_t(64) << 20;     // fallback scratch budget
// Work words: overflow counts of levels 1 and 2, error, work counters of levels 1-3, cells.
constexpr size_t kSeedWorkHeader = 32;
// Resident blocks per SM of the shared-memory ring kernels (at most; 5 fit with 16-slot rings),
// with the carveout sized to them so the rest of the SM's memory stays L1.  Measured on the 1M
// read-seed batch (16-slot rings): 2 blocks 7.7 ms, 3 6.1, 4 5.4, 5 5.2.
constexpr int kSeedBlocksPerSM = 5;

// Parameter checks shared by both entry points; the matrix is copied to `mat`.
int seeds_check_params(gba_context *ctx, const gba_extend_params *p, std::vector<int32_t> &mat)
{
    if (!p) return fail(ctx, GBA_EINVAL, "null params");
    if (p->method < GBA_MATCH_EXTEND || p->method > GBA_GAPPED_XDROP)
        return fail(ctx, GBA_EINVAL, "unknown extension method %d", p->method);
    if (p->direction < GBA_EXTEND_NONE || p->direction > GBA_EXTEND_BOTH)
        return fail(ctx, GBA_EINVAL, "unknown extension direction %d", p->direction);
    if (p->method != GBA_MATCH_EXTEND && (p->score_drop_off >= (1 << 30) || p->score_drop_off <= -(1 << 30)))
        return fail(ctx, GBA_EINVAL, "score_drop_off out of range");
    mat.clear();
    if (p->matrix) {
        if (p->alphabet_size < 1 || p->alphabet_size > 32)
            return fail(ctx, GBA_EINVAL, "matrix alphabet_size must be 1..32");
        mat.assign(p->matrix, p->matrix + p->alphabet_size * p->alphabet_size);
    }
    if (p->method == GBA_GAPPED_XDROP) {
        if (p->gap >= 0) return fail(ctx, GBA_EUNSUPPORTED, "GappedXDrop needs a negative gap score");
        const int lowest = mat.empty() ? std::min(p->match, p->mismatch) : *std::min_element(mat.begin(), mat.end());
        if (lowest < p->gap)
            return fail(ctx, GBA_EUNSUPPORTED,
                        "GappedXDrop with a substitution score (%d) below the gap score (%d): the reference "
                        "overflows int on such schemes",
                        lowest, p->gap);
    }
    return GBA_OK;
}

int64_t pow2_at_least(int64_t v)
{
    int64_t r = 32;
    while (r < v) r <<= 1;
    return r;
}

// Blocks of a persistent level at a dynamic shared-memory size (cached per context): at most
// kSeedBlocksPerSM per SM for shared-memory rings, with the carveout sized to them.
int seeds_resident(gba_context *ctx, const void *fn, size_t smem, bool ring_in_smem)
{
    const auto key = std::make_pair(fn, smem);
    auto it = ctx->xs_grid.find(key);
    if (it != ctx->xs_grid.end()) return int(it->second);
    int nb = 0;
    if (cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem)) != cudaSuccess ||
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, fn, kSeedBlock, smem) != cudaSuccess || nb < 1)
        nb = 1;
    if (ring_in_smem) {
        nb = std::min(nb, kSeedBlocksPerSM);
        int max_smem = 0;
        cudaDeviceGetAttribute(&max_smem, cudaDevAttrMaxSharedMemoryPerMultiprocessor, ctx->device);
        if (max_smem > 0) {
            const size_t want = size_t(nb) * (smem + 1024);
            const int pct = int(std::min<size_t>(100, (want * 100 + max_smem - 1) / size_t(max_smem)));
            cudaFuncSetAttribute(fn, cudaFuncAttributePreferredSharedMemoryCarveout, pct);
        }
    }
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, ctx->device);
    const int64_t blocks = int64_t(nb) * std::max(sms, 1);
    ctx->xs_grid[key] = blocks;
    return int(blocks);
}

template <int RING, int STRIDE>
int seeds_launch_level(gba_context *ctx, bool matrix, size_t mat_bytes, const SeedArgs &a, const XLevel &lv,
                       int64_t max_threads)
{
    const size_t smem = (STRIDE == 1 ? 0 : size_t(seed_ring_words(RING)) * kSeedBlock * 4) + (matrix ? 32 * 32 * 4 : 0);
    const void *fn = matrix ? reinterpret_cast<const void *>(k_extend_gapped<RING, STRIDE, true>)
                            : reinterpret_cast<const void *>(k_extend_gapped<RING, STRIDE, false>);
    (void)mat_bytes;
    const int64_t resident = seeds_resident(ctx, fn, smem, STRIDE != 1);
    const int64_t blocks = std::max<int64_t>(1, std::min(resident, (max_threads + kSeedBlock - 1) / kSeedBlock));
    if (matrix)
        k_extend_gapped<RING, STRIDE, true><<<unsigned(blocks), kSeedBlock, smem, ctx->stream>>>(a, lv);
    else
        k_extend_gapped<RING, STRIDE, false><<<unsigned(blocks), kSeedBlock, smem, ctx->stream>>>(a, lv);
    GBA_CUDA(ctx, cudaGetLastError());
    return GBA_OK;
}

// Launches the extension of `a` (device pointers) on the context stream.
int seeds_enqueue(gba_context *ctx, const gba_extend_params *p, const std::vector<int32_t> &mat, SeedArgs a,
                  int64_t max_v_len, int *launches, int *ring_used)
{
    cudaStream_t s = ctx->stream;
    const int64_t n = a.num_seeds;
    GBA_CUDA(ctx, ctx->xs_work.ensure(kSeedWorkHeader + size_t(std::max<int64_t>(n, 1)) * 8));
    char *work = ctx->xs_work.as<char>();
    int32_t *hdr = reinterpret_cast<int32_t *>(work);
    int32_t *list1 = reinterpret_cast<int32_t *>(work + kSeedWorkHeader);
    int32_t *list2 = list1 + std::max<int64_t>(n, 1);
    a.error = hdr + 2;
    a.cells = reinterpret_cast<unsigned long long *>(work + 24);
    GBA_CUDA(ctx, cudaMemsetAsync(work, 0, kSeedWorkHeader, s));
    a.matrix = nullptr;
    a.alphabet_size = p->alphabet_size;
    if (!mat.empty()) {
        GBA_CUDA(ctx, ctx->xs_matrix.ensure(mat.size() * 4));
        GBA_CUDA(ctx, cudaMemcpyAsync(ctx->xs_matrix.ptr, mat.data(), mat.size() * 4, cudaMemcpyHostToDevice, s));
        a.matrix = ctx->xs_matrix.as<int32_t>();
    }
    a.method = p->method;
    a.direction = p->direction;
    a.xdrop = p->score_drop_off;
    a.match = p->match;
    a.mismatch = p->mismatch;
    a.gap = p->gap;
    const bool matrix = !mat.empty();
    *launches = 0;
    *ring_used = 0;
    GBA_CUDA(ctx, cudaEventRecord(ctx->ev[0], s));
    if (n > 0 && p->direction != GBA_EXTEND_NONE) {
        if (p->method != GBA_GAPPED_XDROP) {
            const unsigned grid = unsigned((n + kSeedBlock - 1) / kSeedBlock);
            if (matrix) k_extend_simple<true><<<grid, kSeedBlock, 0, s>>>(a);
            else k_extend_simple<false><<<grid, kSeedBlock, 0, s>>>(a);
            GBA_CUDA(ctx, cudaGetLastError());
            *launches = 1;
        } else {
            // Columns of a live anti-diagonal: about X / |gap| + 4 (each gap moves the trace one
            // diagonal and costs |gap|), so the first ring is sized from the drop-off.
            GBA_CUDA(ctx, ctx->xs_results.ensure(size_t(n) * sizeof(XResult)));
            a.results = ctx->xs_results.as<XResult>();
            GBA_CUDA(ctx, cudaMemsetAsync(a.results, 0, size_t(n) * sizeof(XResult), s));
            const int64_t reach = int64_t(std::abs(p->score_drop_off)) / int64_t(-p->gap);
            const int ring = reach <= 12 ? 16 : (reach <= 28 ? 32 : (reach <= 60 ? 64 : 0));
            *ring_used = ring;
            XLevel lv{};
            const int32_t *pending = nullptr, *pending_count = nullptr;   // input of the next level
            if (ring) {
                lv.out_list = list1;
                lv.out_count = hdr + 0;
                lv.next = hdr + 3;
                int rc = ring == 16 ? seeds_launch_level<16, kSeedBlock>(ctx, matrix, 0, a, lv, n)
                         : ring == 32 ? seeds_launch_level<32, kSeedBlock>(ctx, matrix, 0, a, lv, n)
                                      : seeds_launch_level<64, kSeedBlock>(ctx, matrix, 0, a, lv, n);
                if (rc) return rc;
                *launches += 1;
                pending = list1;
                pending_count = hdr + 0;
                if (ring < 64) {
                    XLevel l2{};
                    l2.in_list = list1;
                    l2.in_count = hdr + 0;
                    l2.out_list = list2;
                    l2.out_count = hdr + 1;
                    l2.next = hdr + 4;
                    if (int rc2 = seeds_launch_level<64, kSeedBlock>(ctx, matrix, 0, a, l2, std::max<int64_t>(n / 8, 1)))
                        return rc2;
                    *launches += 1;
                    pending = list2;
                    pending_count = hdr + 1;
                }
            }
            // Last level: a global-memory ring that holds the whole query segment (a live range
            // spans at most query + 2 columns).
            const int64_t wring = pow2_at_least(max_v_len + 2);
            if (wring > kSeedMaxWideRing)
                return fail(ctx, GBA_EUNSUPPORTED, "queries longer than %d residues", kSeedMaxWideRing - 2);
            const size_t per_thread = size_t(seed_ring_words(int(wring))) * 4;
            int64_t threads = int64_t(std::max(kSeedWideScratch, per_thread * 32) / per_thread);
            threads = std::min<int64_t>(threads, int64_t(152) * 8 * kSeedBlock);
            threads = std::min<int64_t>(threads, ring ? std::max<int64_t>(n / 64, kSeedBlock) : n);
            threads = (std::max<int64_t>(threads, 1) + 31) / 32 * 32;   // whole warps
            GBA_CUDA(ctx, ctx->xs_scratch.ensure(size_t(threads) * per_thread));
            XLevel l3{};
            l3.in_list = pending;
            l3.in_count = pending_count;
            l3.next = hdr + 5;
            l3.scratch = ctx->xs_scratch.as<int32_t>();
            l3.ring = int32_t(wring);
            l3.threads = int32_t(threads);
            if (int rc3 = seeds_launch_level<1, 1>(ctx, matrix, 0, a, l3, threads)) return rc3;
            k_apply_gapped<<<unsigned((n + kSeedBlock - 1) / kSeedBlock), kSeedBlock, 0, s>>>(a);
            GBA_CUDA(ctx, cudaGetLastError());
            *launches += 2;
        }
    }
    GBA_CUDA(ctx, cudaEventRecord(ctx->ev[1], s));
    ctx->xs_check = true;
    return GBA_OK;
}

// Reads the error word of the last enqueued extension (stream already synchronized).
int seeds_read_error(gba_context *ctx, int64_t *cells, int64_t *fallbacks)
{
    if (!ctx->xs_check) return GBA_OK;
    ctx->xs_check = false;
    int32_t hdr[8] = {};
    GBA_CUDA(ctx, cudaMemcpy(hdr, ctx->xs_work.ptr, sizeof(hdr), cudaMemcpyDeviceToHost));
    if (cells) std::memcpy(cells, hdr + 6, 8);
    if (fallbacks) *fallbacks = hdr[0];
    if (hdr[2] & 1) return fail(ctx, GBA_EINVAL, "a seed lies outside its sequences");
    if (hdr[2] & 2) return fail(ctx, GBA_EUNSUPPORTED, "an x-drop band wider than the fallback ring");
    return GBA_OK;
}

}  // namespace

int seeds_check_error(gba_context *ctx)
{
    return seeds_read_error(ctx, nullptr, nullptr);
}

extern "C" {

GBA_API int gba_extend_seeds(gba_context *ctx, const gba_extend_params *params, const gba_seed_batch *b,
                             gba_seed *seeds, int32_t *scores)
{
    if (!ctx || !b) return GBA_EINVAL;
    const auto t0 = std::chrono::steady_clock::now();
    GBA_CUDA(ctx, cudaSetDevice(ctx->device));
    std::vector<int32_t> mat;
    if (int rc = seeds_check_params(ctx, params, mat)) return rc;
    const int64_t ns = b->num_seeds;
    if (ns < 0 || b->num_h < 0 || b->num_v < 0) return fail(ctx, GBA_EINVAL, "negative count");
    if (ns > INT32_MAX / 2) return fail(ctx, GBA_EUNSUPPORTED, "more than 2^30 seeds in one call");
    if (ns == 0) return GBA_OK;
    if (!seeds || !b->off_h || !b->off_v) return fail(ctx, GBA_EINVAL, "null seeds or offsets");
    for (int64_t k = 0; k < b->num_h; ++k)
        if (b->off_h[k + 1] < b->off_h[k]) return fail(ctx, GBA_EINVAL, "database offsets decrease at %lld", (long long)k);
    for (int64_t k = 0; k < b->num_v; ++k)
        if (b->off_v[k + 1] < b->off_v[k]) return fail(ctx, GBA_EINVAL, "query offsets decrease at %lld", (long long)k);
    if (b->off_h[0] < 0 || b->off_v[0] < 0) return fail(ctx, GBA_EINVAL, "negative offset");
    const int64_t hb = b->off_h[b->num_h], vb = b->off_v[b->num_v];
    if ((hb && !b->seq_h) || (vb && !b->seq_v)) return fail(ctx, GBA_EINVAL, "null sequence codes");
    // Seeds: on their sequences, as the reference's prefix/suffix calls require.
    int64_t max_v = 0;
    const bool gapped = params->method == GBA_GAPPED_XDROP;
    const bool ungapped_left = params->method == GBA_UNGAPPED_XDROP && (params->direction & GBA_EXTEND_LEFT) &&
                               params->score_drop_off > 0;
    for (int64_t i = 0; i < ns; ++i) {
        const int64_t hi = b->seed_h ? b->seed_h[i] : i, vi = b->seed_v ? b->seed_v[i] : i;
        if (hi < 0 || hi >= b->num_h || vi < 0 || vi >= b->num_v)
            return fail(ctx, GBA_EINVAL, "seed %lld names a missing sequence", (long long)i);
        const int64_t m = b->off_h[hi + 1] - b->off_h[hi], n = b->off_v[vi + 1] - b->off_v[vi];
        const gba_seed &s = seeds[i];
        if (!(0 <= s.begin_h && s.begin_h <= s.end_h && s.end_h <= m && 0 <= s.begin_v && s.begin_v <= s.end_v &&
              s.end_v <= n))
            return fail(ctx, GBA_EINVAL, "seed %lld lies outside its sequences", (long long)i);
        if (ungapped_left && s.begin_h >= 1 && s.begin_v >= 1 && (s.begin_h >= m || s.begin_v >= n))
            return fail(ctx, GBA_EINVAL, "seed %lld: empty UnGappedXDrop seed at a sequence end", (long long)i);
        if (gapped && (m > kSeedMaxGappedLen || n > kSeedMaxGappedLen))
            return fail(ctx, GBA_EUNSUPPORTED, "GappedXDrop on sequences longer than 2^29");
        max_v = std::max(max_v, n);
    }
    cudaStream_t st = ctx->stream;
    // Uploads: codes, offsets, seed indices, seeds.
    GBA_CUDA(ctx, ctx->xs_seq_h.ensure(size_t(hb) + 16));
    GBA_CUDA(ctx, ctx->xs_seq_v.ensure(size_t(vb) + 16));
    if (hb) GBA_CUDA(ctx, cudaMemcpyAsync(ctx->xs_seq_h.ptr, b->seq_h, hb, cudaMemcpyHostToDevice, st));
    if (vb) GBA_CUDA(ctx, cudaMemcpyAsync(ctx->xs_seq_v.ptr, b->seq_v, vb, cudaMemcpyHostToDevice, st));
    GBA_CUDA(ctx, ctx->xs_off_h.ensure(size_t(b->num_h + 1) * 8));
    GBA_CUDA(ctx, ctx->xs_off_v.ensure(size_t(b->num_v + 1) * 8));
    const uint8_t *dseq_h = ctx->xs_seq_h.as<uint8_t>();
    const uint8_t *dseq_v = ctx->xs_seq_v.as<uint8_t>();
    GBA_CUDA(ctx, cudaMemcpyAsync(ctx->xs_off_h.ptr, b->off_h, size_t(b->num_h + 1) * 8, cudaMemcpyHostToDevice, st));
    GBA_CUDA(ctx, cudaMemcpyAsync(ctx->xs_off_v.ptr, b->off_v, size_t(b->num_v + 1) * 8, cudaMemcpyHostToDevice, st));
    const size_t ids = size_t(ns) * 4;
    GBA_CUDA(ctx, ctx->xs_ids.ensure(2 * ids));
    if (b->seed_h) GBA_CUDA(ctx, cudaMemcpyAsync(ctx->xs_ids.ptr, b->seed_h, ids, cudaMemcpyHostToDevice, st));
    if (b->seed_v)
        GBA_CUDA(ctx, cudaMemcpyAsync(ctx->xs_ids.as<char>() + ids, b->seed_v, ids, cudaMemcpyHostToDevice, st));
    GBA_CUDA(ctx, ctx->xs_seeds.ensure(size_t(ns) * sizeof(gba_seed)));
    GBA_CUDA(ctx, cudaMemcpyAsync(ctx->xs_seeds.ptr, seeds, size_t(ns) * sizeof(gba_seed), cudaMemcpyHostToDevice, st));
    if (scores) GBA_CUDA(ctx, ctx->xs_scores.ensure(size_t(ns) * 8));
    SeedArgs a{};
    a.seq_h = dseq_h;
    a.seq_v = dseq_v;
    a.off_h = ctx->xs_off_h.as<int64_t>();
    a.off_v = ctx->xs_off_v.as<int64_t>();
    a.seed_h = b->seed_h ? ctx->xs_ids.as<int32_t>() : nullptr;
    a.seed_v = b->seed_v ? reinterpret_cast<const int32_t *>(ctx->xs_ids.as<char>() + ids) : nullptr;
    a.num_h = b->num_h;
    a.num_v = b->num_v;
    a.seeds = ctx->xs_seeds.as<SeedDev>();
    a.scores = scores ? ctx->xs_scores.as<int32_t>() : nullptr;
    a.num_seeds = int32_t(ns);
    int launches = 0, ring = 0;
    if (int rc = seeds_enqueue(ctx, params, mat, a, max_v, &launches, &ring)) return rc;
    GBA_CUDA(ctx, cudaMemcpyAsync(seeds, ctx->xs_seeds.ptr, size_t(ns) * sizeof(gba_seed), cudaMemcpyDeviceToHost, st));
    if (scores) GBA_CUDA(ctx, cudaMemcpyAsync(scores, ctx->xs_scores.ptr, size_t(ns) * 8, cudaMemcpyDeviceToHost, st));
    GBA_CUDA(ctx, cudaStreamSynchronize(st));
    int64_t cells = 0, fallbacks = 0;
    int rc = seeds_read_error(ctx, &cells, &fallbacks);
    float ms = 0;
    GBA_CUDA(ctx, cudaEventElapsedTime(&ms, ctx->ev[0], ctx->ev[1]));
    ctx->stats = gba_stats{};
    ctx->stats.dp_kernel_ms = ms;
    ctx->stats.kernel_launches = launches;
    ctx->stats.cells = cells;
    ctx->stats.seed_ring = ring;
    ctx->stats.seed_fallbacks = (params->method == GBA_GAPPED_XDROP && ring == 0) ? ns : fallbacks;
    ctx->stats.call_ms = std::chrono::duration<float, std::milli>(std::chrono::steady_clock::now() - t0).count();
    return rc;
}

GBA_API int gba_extend_seeds_device(gba_context *ctx, const gba_extend_params *params, const gba_seed_batch *b,
                                    gba_seed *dev_seeds, int32_t *dev_scores)
{
    if (!ctx || !b) return GBA_EINVAL;
    GBA_CUDA(ctx, cudaSetDevice(ctx->device));
    std::vector<int32_t> mat;
    if (int rc = seeds_check_params(ctx, params, mat)) return rc;
    if (b->num_seeds < 0 || b->num_h < 0 || b->num_v < 0 || b->max_v_len < 0)
        return fail(ctx, GBA_EINVAL, "negative count");
    if (b->num_seeds > INT32_MAX / 2) return fail(ctx, GBA_EUNSUPPORTED, "more than 2^30 seeds in one call");
    if (b->num_seeds == 0) return GBA_OK;
    if (!dev_seeds || !b->off_h || !b->off_v) return fail(ctx, GBA_EINVAL, "null seeds or offsets");
    if (params->method == GBA_GAPPED_XDROP && b->max_v_len > kSeedMaxGappedLen)
        return fail(ctx, GBA_EUNSUPPORTED, "GappedXDrop on sequences longer than 2^29");
    SeedArgs a{};
    a.seq_h = b->seq_h;
    a.seq_v = b->seq_v;
    a.off_h = b->off_h;
    a.off_v = b->off_v;
    a.seed_h = b->seed_h;
    a.seed_v = b->seed_v;
    a.num_h = b->num_h;
    a.num_v = b->num_v;
    a.seeds = reinterpret_cast<SeedDev *>(dev_seeds);
    a.scores = dev_scores;
    a.num_seeds = int32_t(b->num_seeds);
    int launches = 0, ring = 0;
    return seeds_enqueue(ctx, params, mat, a, b->max_v_len, &launches, &ring);
}

}  // extern "C"
