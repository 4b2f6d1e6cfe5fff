// extend_host.cuh -- host side of gba_extend_alignments (included at the end of engine.cu).
//
// Each alignment contributes up to two tasks (its left side on the reversed prefixes, its right
// side on the suffixes).  A score pass runs the AlignExtend DP with the X-drop terminator and
// finds each task's best cell and last computed column; the host then sizes the trace
// (last column + 1 columns of round8(rows + 1) bytes per task) and the segment slots, and a trace
// pass recomputes exactly those columns with trace, followed by the traceback.  Tasks are cut
// into chunks whose trace fits kExtTraceBudget.  With a band, both sides run as one
// GBA_ALIGN_EXTEND batch on the banded kernel instead (ext_banded).
#pragma once

namespace {

constexpr size_t kExtTraceBudget = size_t(4) << 30;
constexpr int64_t kExtMaxLen = int64_t(1) << 28;

int ext_check_params(gba_context *ctx, const gba_extend_align_params *p, std::vector<int32_t> &mat)
{
    if (!p) return fail(ctx, GBA_EINVAL, "null params");
    if (p->direction < GBA_EXTEND_NONE || p->direction > GBA_EXTEND_BOTH)
        return fail(ctx, GBA_EINVAL, "unknown extension direction %d", p->direction);
    const int lim = 1 << 20;
    if (std::abs(p->gap_open) > lim || std::abs(p->gap_extend) > lim || std::abs(p->match) > lim ||
        std::abs(p->mismatch) > lim || (p->xdrop_on && std::abs(p->xdrop) >= (1 << 30)))
        return fail(ctx, GBA_EUNSUPPORTED, "scores beyond +-2^20 (cells are int, infinity -2^30)");
    mat.clear();
    if (p->matrix) {
        if (p->alphabet_size < 1 || p->alphabet_size > 32)
            return fail(ctx, GBA_EINVAL, "matrix alphabet_size must be 1..32");
        mat.assign(p->matrix, p->matrix + p->alphabet_size * p->alphabet_size);
        for (int32_t x : mat)
            if (std::abs(x) > lim) return fail(ctx, GBA_EUNSUPPORTED, "matrix scores beyond +-2^20");
    }
    return GBA_OK;
}

template <bool AFFINE, bool MATRIX, bool TRACE, int W>
int ext_launch_dp(gba_context *ctx, const ExtArgs &a)
{
    const void *fn = reinterpret_cast<const void *>(k_extend_dp<AFFINE, MATRIX, TRACE, W>);
    int nb = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, fn, 128, 0) != cudaSuccess || nb < 1) nb = 1;
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, ctx->device);
    const int64_t threads_needed = int64_t(a.num_tasks) * W;
    const int64_t blocks = std::max<int64_t>(1, std::min<int64_t>(int64_t(nb) * sms, (threads_needed + 127) / 128));
    k_extend_dp<AFFINE, MATRIX, TRACE, W><<<unsigned(blocks), 128, 0, ctx->stream>>>(a);
    GBA_CUDA(ctx, cudaGetLastError());
    return GBA_OK;
}

template <int W>
int ext_dp_w(gba_context *ctx, bool affine, bool matrix, bool trace, const ExtArgs &a)
{
    if (affine) {
        if (matrix)
            return trace ? ext_launch_dp<true, true, true, W>(ctx, a) : ext_launch_dp<true, true, false, W>(ctx, a);
        return trace ? ext_launch_dp<true, false, true, W>(ctx, a) : ext_launch_dp<true, false, false, W>(ctx, a);
    }
    if (matrix) return trace ? ext_launch_dp<false, true, true, W>(ctx, a) : ext_launch_dp<false, true, false, W>(ctx, a);
    return trace ? ext_launch_dp<false, false, true, W>(ctx, a) : ext_launch_dp<false, false, false, W>(ctx, a);
}

// Lanes per task: 8 rows per lane, so a group of W lanes covers 8W rows per band; W follows the
// batch's 90th-percentile task height (read halves of ~75 rows fill 8 or 16 lanes, not 32).
int ext_dp(gba_context *ctx, int W, bool affine, bool matrix, bool trace, const ExtArgs &a)
{
    if (W == 8) return ext_dp_w<8>(ctx, affine, matrix, trace, a);
    if (W == 16) return ext_dp_w<16>(ctx, affine, matrix, trace, a);
    return ext_dp_w<32>(ctx, affine, matrix, trace, a);
}

// Resident groups of W lanes (an upper bound on the groups that need scratch).
int64_t ext_max_groups(gba_context *ctx, int W)
{
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, ctx->device);
    return int64_t(std::max(sms, 1)) * 2048 / W;   // 2,048 resident threads per SM at most
}

// The banded overloads (lowerDiag, upperDiag): each side is one pair of a GBA_ALIGN_EXTEND batch
// -- the reversed prefixes for the left side, the suffixes for the right one -- aligned by the
// banded kernel in its AlignExtend_ mode with the engine's traceback; the left side's segments
// are then mapped back as _reversePartialTrace does.
int ext_banded(gba_context *ctx, const gba_extend_align_params *params, const std::vector<int32_t> &mat,
               const gba_seed_batch *b, const gba_seed *seeds, gba_extend_align_result *res)
{
    const int64_t ns = b->num_seeds;
    std::vector<uint8_t> hcat, vcat;
    std::vector<int64_t> hoff(1, 0), voff(1, 0);
    std::vector<int64_t> task_of(size_t(ns) * 2, -1);
    int64_t cap = 0;
    for (int64_t k = 0; k < ns; ++k) {
        const int64_t hi = b->seed_h ? b->seed_h[k] : k, vi = b->seed_v ? b->seed_v[k] : k;
        if (hi < 0 || hi >= b->num_h || vi < 0 || vi >= b->num_v)
            return fail(ctx, GBA_EINVAL, "alignment %lld names a missing sequence", (long long)k);
        const int64_t m = b->off_h[hi + 1] - b->off_h[hi], n = b->off_v[vi + 1] - b->off_v[vi];
        if (m > kExtMaxLen || n > kExtMaxLen) return fail(ctx, GBA_EUNSUPPORTED, "sequences longer than 2^28");
        const gba_seed &sd = seeds[k];
        if (!(0 <= sd.begin_h && sd.begin_h <= sd.end_h && sd.end_h <= m && 0 <= sd.begin_v &&
              sd.begin_v <= sd.end_v && sd.end_v <= n))
            return fail(ctx, GBA_EINVAL, "alignment %lld lies outside its sequences", (long long)k);
        const uint8_t *h = b->seq_h + b->off_h[hi], *v = b->seq_v + b->off_v[vi];
        if ((params->direction & GBA_EXTEND_LEFT) && sd.begin_h > 0 && sd.begin_v > 0) {
            task_of[2 * k] = int64_t(hoff.size()) - 1;
            for (int64_t i = sd.begin_h - 1; i >= 0; --i) hcat.push_back(h[i]);
            for (int64_t i = sd.begin_v - 1; i >= 0; --i) vcat.push_back(v[i]);
            hoff.push_back(int64_t(hcat.size()));
            voff.push_back(int64_t(vcat.size()));
            cap += sd.begin_h + sd.begin_v + 2;
        }
        if ((params->direction & GBA_EXTEND_RIGHT) && sd.end_h < m && sd.end_v < n) {
            task_of[2 * k + 1] = int64_t(hoff.size()) - 1;
            hcat.insert(hcat.end(), h + sd.end_h, h + m);
            vcat.insert(vcat.end(), v + sd.end_v, v + n);
            hoff.push_back(int64_t(hcat.size()));
            voff.push_back(int64_t(vcat.size()));
            cap += (m - sd.end_h) + (n - sd.end_v) + 2;
        }
    }
    const int64_t nt = int64_t(hoff.size()) - 1;
    std::vector<int32_t> score(size_t(std::max<int64_t>(nt, 1))), status(size_t(std::max<int64_t>(nt, 1)));
    std::vector<gba_segment> segs(size_t(std::max<int64_t>(cap, 1)));
    std::vector<int64_t> seg_off(size_t(nt) + 1, 0);
    if (nt > 0) {
        if (hcat.empty()) hcat.push_back(0);
        if (vcat.empty()) vcat.push_back(0);
        gba_params gp{};
        gp.mode = GBA_ALIGN_EXTEND;
        gp.gap_model = GBA_GAPS_AUTO;   // Gotoh iff open != extend, as _extendAlignmentImpl picks
        // Diagonals beyond every side's matrix change nothing the banded DP decides (its phase
        // tests, the tracked cells, which cells are in the band), so a band wider than the
        // matrices is narrowed to up' = min(up, max over sides of max(m, n + lo + 1)) and then
        // lo' = max(lo, min over sides of min(-n, up' - n - 1)): each test on (lo, up) --
        // up < 0, lo >= 0, lo > -n, up > n + lo, up == m - n, up >= m, lo + n vs m -- and the
        // band's validity keep their value for every side.
        int64_t lo = params->band_lower, up = params->band_upper;
        int64_t U = INT64_MIN;
        for (int64_t t = 0; t < nt; ++t)
            U = std::max(U, std::max(hoff[t + 1] - hoff[t], (voff[t + 1] - voff[t]) + lo + 1));
        if (up > U && U > lo) up = U;
        int64_t L = INT64_MAX;
        for (int64_t t = 0; t < nt; ++t) {
            const int64_t n = voff[t + 1] - voff[t];
            L = std::min(L, std::min(-n, up - n - 1));
        }
        if (lo < L) lo = L;
        if (up - lo + 1 > int64_t(1) << 20)
            return fail(ctx, GBA_EUNSUPPORTED, "band wider than the engine's band slots");
        gp.band_on = 1;
        gp.band_lower = int32_t(lo);
        gp.band_upper = int32_t(up);
        gp.match = params->match;
        gp.mismatch = params->mismatch;
        gp.gap_open = params->gap_open;
        gp.gap_extend = params->gap_extend;
        gp.matrix = mat.empty() ? nullptr : mat.data();
        gp.alphabet_size = mat.empty() ? 0 : params->alphabet_size;
        gp.score_bits = 32;
        gp.outputs = GBA_OUT_SCORE | GBA_OUT_END | GBA_OUT_SEGMENTS;
        gp.flags = params->xdrop_on ? GBA_FLAG_XDROP : 0;
        gp.xdrop = params->xdrop;
        gba_batch gb{};
        gb.num_pairs = nt;
        gb.seq_h = hcat.data();
        gb.off_h = hoff.data();
        gb.seq_v = vcat.data();
        gb.off_v = voff.data();
        gba_result gr{};
        gr.score = score.data();
        gr.pair_status = status.data();
        gr.segments = segs.data();
        gr.segment_capacity = cap;
        gr.segment_offsets = seg_off.data();
        if (int rc = gba_align_batch(ctx, &gp, &gb, &gr)) return rc;
    }
    int64_t w = 0;
    for (int64_t k = 0; k < ns; ++k) {
        for (int side = 0; side < 2; ++side) {
            const int64_t t = task_of[2 * k + side];
            int32_t sc = 0;
            if (t >= 0) {
                sc = score[t];   // INT32_MIN with no segments for a band outside the side's matrix
                const int64_t c = seg_off[t + 1] - seg_off[t];
                if (w + c > res->segment_capacity || (c && !res->segments))
                    return fail(ctx, GBA_ECAPACITY, "segment_capacity too small");
                const gba_segment *sg = segs.data() + seg_off[t];
                if (side == 1) {
                    for (int64_t q = 0; q < c; ++q) res->segments[w + q] = sg[q];
                } else {
                    const uint32_t lh = uint32_t(hoff[t + 1] - hoff[t]), lv = uint32_t(voff[t + 1] - voff[t]);
                    for (int64_t q = 0; q < c; ++q) {
                        const gba_segment &x = sg[c - 1 - q];
                        const uint32_t eh = x.h_begin + ((x.type == GBA_SEG_DIAGONAL || x.type == GBA_SEG_HORIZONTAL) ? x.length : 0);
                        const uint32_t ev = x.v_begin + ((x.type == GBA_SEG_DIAGONAL || x.type == GBA_SEG_VERTICAL) ? x.length : 0);
                        res->segments[w + q] = gba_segment{lh - eh, lv - ev, x.length, x.type};
                    }
                }
                w += c;
            }
            if (side == 0 && res->left_score) res->left_score[k] = sc;
            if (side == 1 && res->right_score) res->right_score[k] = sc;
            res->segment_offsets[2 * k + side + 1] = w;
        }
    }
    return GBA_OK;
}

}  // namespace

extern "C" {

GBA_API int gba_extend_alignments(gba_context *ctx, const gba_extend_align_params *params,
                                  const gba_seed_batch *b, const gba_seed *seeds, gba_extend_align_result *res)
{
    if (!ctx || !b || !res) return GBA_EINVAL;
    const auto t0 = std::chrono::steady_clock::now();
    GBA_CUDA(ctx, cudaSetDevice(ctx->device));
    std::vector<int32_t> mat;
    if (int rc = ext_check_params(ctx, params, mat)) return rc;
    const int64_t ns = b->num_seeds;
    if (ns < 0 || b->num_h < 0 || b->num_v < 0) return fail(ctx, GBA_EINVAL, "negative count");
    if (ns > (int64_t(1) << 30)) return fail(ctx, GBA_EUNSUPPORTED, "more than 2^30 alignments in one call");
    if (!res->segment_offsets) return fail(ctx, GBA_EINVAL, "null segment_offsets");
    res->segment_offsets[0] = 0;
    if (ns == 0) return GBA_OK;
    if (!seeds || !b->off_h || !b->off_v) return fail(ctx, GBA_EINVAL, "null seeds or offsets");
    for (int64_t k = 0; k < b->num_h; ++k)
        if (b->off_h[k + 1] < b->off_h[k]) return fail(ctx, GBA_EINVAL, "database offsets decrease");
    for (int64_t k = 0; k < b->num_v; ++k)
        if (b->off_v[k + 1] < b->off_v[k]) return fail(ctx, GBA_EINVAL, "query offsets decrease");
    const int64_t hb_total = b->off_h[b->num_h], vb_total = b->off_v[b->num_v];
    if (b->off_h[0] < 0 || b->off_v[0] < 0) return fail(ctx, GBA_EINVAL, "negative offset");
    if ((hb_total && !b->seq_h) || (vb_total && !b->seq_v)) return fail(ctx, GBA_EINVAL, "null sequence codes");
    if (params->band_on) {
        if (params->band_lower > params->band_upper) return fail(ctx, GBA_EINVAL, "band_lower > band_upper");
        return ext_banded(ctx, params, mat, b, seeds, res);
    }
    const bool affine = params->gap_open != params->gap_extend;
    const bool matrix = !mat.empty();
    cudaStream_t st = ctx->stream;

    GBA_CUDA(ctx, ctx->seq_h.ensure(size_t(hb_total) + 16));
    GBA_CUDA(ctx, ctx->seq_v.ensure(size_t(vb_total) + 16));
    if (hb_total) GBA_CUDA(ctx, cudaMemcpyAsync(ctx->seq_h.ptr, b->seq_h, hb_total, cudaMemcpyHostToDevice, st));
    if (vb_total) GBA_CUDA(ctx, cudaMemcpyAsync(ctx->seq_v.ptr, b->seq_v, vb_total, cudaMemcpyHostToDevice, st));
    const uint8_t *dh = ctx->seq_h.as<uint8_t>(), *dv = ctx->seq_v.as<uint8_t>();

    // Tasks: (alignment, side) in alignment order; task_of[2k + side] = task index or -1.
    std::vector<ExtTask> tasks;
    tasks.reserve(size_t(ns) * 2);
    std::vector<int64_t> task_of(size_t(ns) * 2, -1);
    int64_t max_n = 0;
    for (int64_t k = 0; k < ns; ++k) {
        const int64_t hi = b->seed_h ? b->seed_h[k] : k, vi = b->seed_v ? b->seed_v[k] : k;
        if (hi < 0 || hi >= b->num_h || vi < 0 || vi >= b->num_v)
            return fail(ctx, GBA_EINVAL, "alignment %lld names a missing sequence", (long long)k);
        const int64_t m = b->off_h[hi + 1] - b->off_h[hi], n = b->off_v[vi + 1] - b->off_v[vi];
        if (m > kExtMaxLen || n > kExtMaxLen) return fail(ctx, GBA_EUNSUPPORTED, "sequences longer than 2^28");
        const gba_seed &s = seeds[k];
        if (!(0 <= s.begin_h && s.begin_h <= s.end_h && s.end_h <= m && 0 <= s.begin_v && s.begin_v <= s.end_v &&
              s.end_v <= n))
            return fail(ctx, GBA_EINVAL, "alignment %lld lies outside its sequences", (long long)k);
        const uint8_t *h = dh + b->off_h[hi], *v = dv + b->off_v[vi];
        if ((params->direction & GBA_EXTEND_LEFT) && s.begin_h > 0 && s.begin_v > 0) {
            task_of[2 * k] = int64_t(tasks.size());
            tasks.push_back(ExtTask{h + s.begin_h, v + s.begin_v, int32_t(s.begin_h), int32_t(s.begin_v), -1, -1, 0, 0,
                                    0});
            max_n = std::max<int64_t>(max_n, s.begin_v);
        }
        if ((params->direction & GBA_EXTEND_RIGHT) && s.end_h < m && s.end_v < n) {
            task_of[2 * k + 1] = int64_t(tasks.size());
            tasks.push_back(ExtTask{h + s.end_h - 1, v + s.end_v - 1, int32_t(m - s.end_h), int32_t(n - s.end_v), 1, 1,
                                    0, 0, 0});
            max_n = std::max<int64_t>(max_n, n - s.end_v);
        }
    }
    const int64_t nt = int64_t(tasks.size());
    int W = 32;
    if (nt > 0) {
        std::vector<int32_t> heights(static_cast<size_t>(nt), 0);
        for (int64_t t = 0; t < nt; ++t) heights[t] = tasks[t].n + 1;
        const size_t q = size_t(nt) * 9 / 10;
        std::nth_element(heights.begin(), heights.begin() + q, heights.end());
        const int p90 = heights[q];
        W = p90 <= 8 * 8 ? 8 : (p90 <= 8 * 16 ? 16 : 32);
    }
    std::vector<ExtOut> outs(size_t(std::max<int64_t>(nt, 1)));
    std::vector<int32_t> counts;
    std::vector<ExtSegment> segs_host;
    std::vector<int64_t> seg_off_host, packed_off;
    int launches = 0;
    float dp_ms = 0, tb_ms = 0;
    int64_t cells = 0;
    if (nt > 0) {
        GBA_CUDA(ctx, ctx->xa_tasks.ensure(size_t(nt) * sizeof(ExtTask)));
        GBA_CUDA(ctx, ctx->xa_out.ensure(size_t(nt) * sizeof(ExtOut)));
        GBA_CUDA(ctx, ctx->xa_next.ensure(16));
        GBA_CUDA(ctx, cudaMemcpyAsync(ctx->xa_tasks.ptr, tasks.data(), size_t(nt) * sizeof(ExtTask),
                                      cudaMemcpyHostToDevice, st));
        if (matrix) {
            GBA_CUDA(ctx, ctx->xs_matrix.ensure(mat.size() * 4));
            GBA_CUDA(ctx, cudaMemcpyAsync(ctx->xs_matrix.ptr, mat.data(), mat.size() * 4, cudaMemcpyHostToDevice, st));
        }
        ExtArgs a{};
        a.tasks = ctx->xa_tasks.as<ExtTask>();
        a.out = ctx->xa_out.as<ExtOut>();
        a.num_tasks = int32_t(nt);
        a.next = ctx->xa_next.as<int32_t>();
        a.match = params->match;
        a.mismatch = params->mismatch;
        a.gap_open = params->gap_open;
        a.gap_extend = params->gap_extend;
        a.matrix = matrix ? ctx->xs_matrix.as<int32_t>() : nullptr;
        a.asize = params->alphabet_size;
        a.xdrop_on = params->xdrop_on;
        a.xdrop = params->xdrop;
        if (max_n + 1 > 8 * W) {
            a.scratch_stride = 2 * (max_n + 1);
            GBA_CUDA(ctx, ctx->xa_scratch.ensure(size_t(ext_max_groups(ctx, W)) * size_t(a.scratch_stride) * 4));
            a.scratch = ctx->xa_scratch.as<int32_t>();
        }
        // score pass
        GBA_CUDA(ctx, cudaMemsetAsync(a.next, 0, 4, st));
        GBA_CUDA(ctx, cudaEventRecord(ctx->ev[0], st));
        if (int rc = ext_dp(ctx, W, affine, matrix, false, a)) return rc;
        GBA_CUDA(ctx, cudaEventRecord(ctx->ev[1], st));
        ++launches;
        GBA_CUDA(ctx, cudaMemcpyAsync(outs.data(), a.out, size_t(nt) * sizeof(ExtOut), cudaMemcpyDeviceToHost, st));
        GBA_CUDA(ctx, cudaStreamSynchronize(st));
        {
            float ms = 0;
            GBA_CUDA(ctx, cudaEventElapsedTime(&ms, ctx->ev[0], ctx->ev[1]));
            dp_ms += ms;
        }
        // trace layout and segment slots
        seg_off_host.assign(size_t(nt) + 1, 0);
        std::vector<int64_t> trace_end(static_cast<size_t>(nt), 0);
        int64_t toff = 0;
        for (int64_t t = 0; t < nt; ++t) {
            ExtTask &tk = tasks[t];
            tk.col_limit = outs[t].last_col;
            tk.trace_off = toff;
            toff += int64_t(outs[t].last_col + 1) * ext_trace_stride(tk.n);
            trace_end[t] = toff;
            seg_off_host[t + 1] = seg_off_host[t] + int64_t(outs[t].last_col) + tk.n + 2;
            cells += int64_t(outs[t].last_col + 1) * (tk.n + 1);
        }
        GBA_CUDA(ctx, ctx->xa_segoff.ensure(size_t(nt + 1) * 8));
        GBA_CUDA(ctx, ctx->xa_segcnt.ensure(size_t(nt) * 4));
        GBA_CUDA(ctx, ctx->xa_segs.ensure(size_t(seg_off_host[nt]) * sizeof(ExtSegment)));
        GBA_CUDA(ctx, cudaMemcpyAsync(ctx->xa_segoff.ptr, seg_off_host.data(), size_t(nt + 1) * 8,
                                      cudaMemcpyHostToDevice, st));
        // trace pass and traceback, in chunks of tasks whose trace fits the budget
        int64_t c0 = 0;
        while (c0 < nt) {
            int64_t c1 = c0 + 1;
            const int64_t base = tasks[c0].trace_off;
            while (c1 < nt && size_t(trace_end[c1] - base) <= kExtTraceBudget) ++c1;
            const size_t tbytes = size_t(trace_end[c1 - 1] - base);
            GBA_CUDA(ctx, ctx->xa_trace.ensure(tbytes + 16));
            std::vector<ExtTask> chunk(tasks.begin() + c0, tasks.begin() + c1);
            for (ExtTask &tk : chunk) tk.trace_off -= base;
            GBA_CUDA(ctx, cudaMemcpyAsync(ctx->xa_tasks.ptr, chunk.data(), chunk.size() * sizeof(ExtTask),
                                          cudaMemcpyHostToDevice, st));
            ExtArgs at = a;
            at.num_tasks = int32_t(c1 - c0);
            at.out = a.out + c0;
            at.trace = ctx->xa_trace.as<uint8_t>();
            GBA_CUDA(ctx, cudaMemsetAsync(a.next, 0, 4, st));
            GBA_CUDA(ctx, cudaEventRecord(ctx->ev[0], st));
            if (int rc = ext_dp(ctx, W, affine, matrix, true, at)) return rc;
            GBA_CUDA(ctx, cudaEventRecord(ctx->ev[1], st));
            const unsigned grid = unsigned((c1 - c0 + 127) / 128);
            if (affine)
                k_extend_traceback<true><<<grid, 128, 0, st>>>(at.tasks, at.out, at.num_tasks, at.trace,
                                                               ctx->xa_segs.as<ExtSegment>(),
                                                               ctx->xa_segoff.as<int64_t>() + c0,
                                                               ctx->xa_segcnt.as<int32_t>() + c0);
            else
                k_extend_traceback<false><<<grid, 128, 0, st>>>(at.tasks, at.out, at.num_tasks, at.trace,
                                                                ctx->xa_segs.as<ExtSegment>(),
                                                                ctx->xa_segoff.as<int64_t>() + c0,
                                                                ctx->xa_segcnt.as<int32_t>() + c0);
            GBA_CUDA(ctx, cudaGetLastError());
            GBA_CUDA(ctx, cudaEventRecord(ctx->ev[2], st));
            launches += 2;
            GBA_CUDA(ctx, cudaStreamSynchronize(st));
            float ms1 = 0, ms2 = 0;
            GBA_CUDA(ctx, cudaEventElapsedTime(&ms1, ctx->ev[0], ctx->ev[1]));
            GBA_CUDA(ctx, cudaEventElapsedTime(&ms2, ctx->ev[1], ctx->ev[2]));
            dp_ms += ms1;
            tb_ms += ms2;
            c0 = c1;
        }
        // pack the used part of each slot, then copy only that back
        counts.resize(size_t(nt));
        GBA_CUDA(ctx, cudaMemcpyAsync(counts.data(), ctx->xa_segcnt.ptr, size_t(nt) * 4, cudaMemcpyDeviceToHost, st));
        GBA_CUDA(ctx, cudaStreamSynchronize(st));
        packed_off.assign(size_t(nt) + 1, 0);
        for (int64_t t = 0; t < nt; ++t) {
            if (counts[t] < 0) return fail(ctx, GBA_ECUDA, "traceback slot overflow (internal)");
            packed_off[t + 1] = packed_off[t] + counts[t];
        }
        GBA_CUDA(ctx, ctx->xa_packoff.ensure(size_t(nt + 1) * 8));
        GBA_CUDA(ctx, ctx->xa_packed.ensure(size_t(std::max<int64_t>(packed_off[nt], 1)) * sizeof(ExtSegment)));
        GBA_CUDA(ctx, cudaMemcpyAsync(ctx->xa_packoff.ptr, packed_off.data(), size_t(nt + 1) * 8,
                                      cudaMemcpyHostToDevice, st));
        k_extend_pack<<<unsigned((nt + 127) / 128), 128, 0, st>>>(
            ctx->xa_segs.as<ExtSegment>(), ctx->xa_segoff.as<int64_t>(), ctx->xa_segcnt.as<int32_t>(),
            ctx->xa_packoff.as<int64_t>(), ctx->xa_packed.as<ExtSegment>(), int(nt));
        GBA_CUDA(ctx, cudaGetLastError());
        ++launches;
        segs_host.resize(size_t(packed_off[nt]));
        if (packed_off[nt])
            GBA_CUDA(ctx, cudaMemcpyAsync(segs_host.data(), ctx->xa_packed.ptr, segs_host.size() * sizeof(ExtSegment),
                                          cudaMemcpyDeviceToHost, st));
        GBA_CUDA(ctx, cudaStreamSynchronize(st));
    }
    // Results: scores and segment lists; the left side's trace is mapped back from the reversed
    // prefixes (_reversePartialTrace: begin = length - end, order reversed).
    int64_t w = 0;
    for (int64_t k = 0; k < ns; ++k) {
        for (int side = 0; side < 2; ++side) {
            const int64_t t = task_of[2 * k + side];
            int32_t score = 0;
            if (t >= 0) {
                score = outs[t].score;
                const int32_t c = counts[t];
                const ExtSegment *sg = segs_host.data() + packed_off[t];
                if (w + c > res->segment_capacity || (c && !res->segments))
                    return fail(ctx, GBA_ECAPACITY, "segment_capacity too small");
                if (side == 1) {
                    for (int32_t q = 0; q < c; ++q)
                        res->segments[w + q] = gba_segment{sg[q].h_begin, sg[q].v_begin, sg[q].length, sg[q].type};
                } else {
                    const uint32_t lh = uint32_t(tasks[t].m), lv = uint32_t(tasks[t].n);
                    for (int32_t q = 0; q < c; ++q) {
                        const ExtSegment &x = sg[c - 1 - q];
                        const uint32_t eh = x.h_begin + ((x.type == GBA_SEG_DIAGONAL || x.type == GBA_SEG_HORIZONTAL) ? x.length : 0);
                        const uint32_t ev = x.v_begin + ((x.type == GBA_SEG_DIAGONAL || x.type == GBA_SEG_VERTICAL) ? x.length : 0);
                        res->segments[w + q] = gba_segment{lh - eh, lv - ev, x.length, x.type};
                    }
                }
                w += c;
            }
            if (side == 0 && res->left_score) res->left_score[k] = score;
            if (side == 1 && res->right_score) res->right_score[k] = score;
            res->segment_offsets[2 * k + side + 1] = w;
        }
    }
    ctx->stats = gba_stats{};
    ctx->stats.dp_kernel_ms = dp_ms;
    ctx->stats.traceback_kernel_ms = tb_ms;
    ctx->stats.kernel_launches = launches;
    ctx->stats.cells = cells;
    ctx->stats.tile_rows = 8 * W;      // rows per band (lanes per task x 8)
    ctx->stats.call_ms = std::chrono::duration<float, std::milli>(std::chrono::steady_clock::now() - t0).count();
    return GBA_OK;
}

}  // extern "C"
