// server.cuh -- continuous-batching request loop (gba_server_* in include/seqan_gb300.h).
//
// Included at the end of engine.cu: a batch slot is a gba_context (its own stream, events and
// grow-only device buffers) plus a gba_plan, and a launch is build_plan + run_plan on the
// slot's inputs, exactly the path of gba_align_batch, so a request's result does not depend on
// the other requests of its batch.  Outputs come back with asynchronous copies into the slot's
// pinned buffers; one worker thread launches batches into free slots and harvests finished ones
// by cudaEventQuery, so batches launched while others run overlap on the device.
#include <condition_variable>
#include <deque>
#include <mutex>
#include <thread>

namespace {

double clock_seconds()
{
    return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

// Pinned host buffer that only grows (by half again, so growth is rare).
struct PinnedBuf {
    void *ptr = nullptr;
    size_t cap = 0;
    cudaError_t ensure(size_t bytes)
    {
        if (bytes <= cap) return cudaSuccess;
        const size_t want = std::max<size_t>(std::max(bytes, cap + cap / 2), 4096);
        if (ptr) cudaFreeHost(ptr);
        ptr = nullptr;
        cap = 0;
        const cudaError_t e = cudaMallocHost(&ptr, want);
        if (e == cudaSuccess) cap = want;
        return e;
    }
    void release()
    {
        if (ptr) cudaFreeHost(ptr);
        ptr = nullptr;
        cap = 0;
    }
    template <typename T> T *as() const { return static_cast<T *>(ptr); }
};

struct SrvRequest {
    uint64_t tag = 0;
    std::vector<uint8_t> h, v;
    double t_submit = 0;
    int64_t bytes = 0;   // device bytes it adds to a batch
};

struct SrvDone {
    gba_request_result r{};
    std::vector<gba_segment> segs;
};

struct SrvSlot {
    gba_context *ctx = nullptr;
    gba_plan plan;
    std::vector<SrvRequest> reqs;
    int64_t bytes = 0;
    bool busy = false;
    bool check_err = false;
    cudaEvent_t done = nullptr;
    std::vector<int64_t> off_h, off_v;
    PinnedBuf seq_h, seq_v, out, segs;
    DevBuf dseq_h, dseq_v, dscore;
};

}  // namespace

struct gba_server {
    gba_params params{};
    std::vector<int32_t> matrix;
    int device = 0;
    int64_t max_batch = 1;
    int64_t budget = 0;
    std::vector<std::unique_ptr<SrvSlot>> slots;
    std::thread worker;
    std::mutex mu;                       // guards everything below
    std::condition_variable cv;
    bool stop = false;
    std::deque<SrvRequest> pending;
    std::deque<SrvDone> completed;
    gba_server_stats stats{};
    std::string last_error;
};

namespace {

// Device bytes one pair adds to a batch: inputs, per-pair records, row buffers, trace and
// segment slots (the terms build_plan allocates for it).
int64_t request_bytes(const gba_params &p, int64_t m, int64_t n)
{
    int64_t b = m + n + int64_t(sizeof(PairDesc)) + 128;
    if (p.outputs & GBA_OUT_SEGMENTS) {
        if (p.band_on) b += (m + 1) * band_col_bytes(p.band_upper - p.band_lower + 1) / 32;
        else b += warp_trace_bytes(int(m), int(n), kWarpRows);
        b += (m + n + 4) * 16 * 2;
    }
    if (!p.band_on && n > 32 * kWarpRows) b += 2 * (m + 1) * 8 + ((n + 255) / 256) * int64_t(sizeof(BandState));
    return b;
}

void srv_fail_batch(gba_server *s, SrvSlot &sl, const std::string &why)
{
    const double now = clock_seconds();
    std::lock_guard<std::mutex> lk(s->mu);
    s->last_error = why;
    for (const SrvRequest &q : sl.reqs) {
        SrvDone d;
        d.r.tag = q.tag;
        d.r.status = GBA_PAIR_FAILED;
        d.r.t_submit = q.t_submit;
        d.r.t_done = now;
        s->completed.push_back(std::move(d));
    }
    s->stats.completed += int64_t(sl.reqs.size());
    s->stats.hbm_in_flight -= sl.bytes;
    sl.reqs.clear();
    sl.bytes = 0;
    sl.busy = false;
}

// Launches sl.reqs on the slot: pack codes into pinned buffers, plan, copy in, run, copy out.
int srv_launch(gba_server *s, SrvSlot &sl)
{
    gba_context *ctx = sl.ctx;
    const int64_t N = int64_t(sl.reqs.size());
    sl.off_h.assign(N + 1, 0);
    sl.off_v.assign(N + 1, 0);
    for (int64_t k = 0; k < N; ++k) {
        sl.off_h[k + 1] = sl.off_h[k] + int64_t(sl.reqs[k].h.size());
        sl.off_v[k + 1] = sl.off_v[k] + int64_t(sl.reqs[k].v.size());
    }
    GBA_CUDA(ctx, sl.seq_h.ensure(size_t(sl.off_h[N]) + 16));
    GBA_CUDA(ctx, sl.seq_v.ensure(size_t(sl.off_v[N]) + 16));
    for (int64_t k = 0; k < N; ++k) {
        if (!sl.reqs[k].h.empty())
            std::memcpy(sl.seq_h.as<uint8_t>() + sl.off_h[k], sl.reqs[k].h.data(), sl.reqs[k].h.size());
        if (!sl.reqs[k].v.empty())
            std::memcpy(sl.seq_v.as<uint8_t>() + sl.off_v[k], sl.reqs[k].v.data(), sl.reqs[k].v.size());
    }
    gba_batch b{};
    b.num_pairs = N;
    b.seq_h = sl.seq_h.as<uint8_t>();
    b.off_h = sl.off_h.data();
    b.seq_v = sl.seq_v.as<uint8_t>();
    b.off_v = sl.off_v.data();
    int rc = build_plan(ctx, &s->params, &b, &sl.plan);
    if (rc) return rc;
    GBA_CUDA(ctx, sl.dseq_h.ensure(size_t(sl.plan.seq_h_bytes) + 16));
    GBA_CUDA(ctx, sl.dseq_v.ensure(size_t(sl.plan.seq_v_bytes) + 16));
    GBA_CUDA(ctx, sl.dscore.ensure(size_t(N) * 4 + 16));
    if (sl.plan.seq_h_bytes)
        GBA_CUDA(ctx, cudaMemcpyAsync(sl.dseq_h.ptr, b.seq_h, sl.plan.seq_h_bytes, cudaMemcpyHostToDevice,
                                      ctx->stream));
    if (sl.plan.seq_v_bytes)
        GBA_CUDA(ctx, cudaMemcpyAsync(sl.dseq_v.ptr, b.seq_v, sl.plan.seq_v_bytes, cudaMemcpyHostToDevice,
                                      ctx->stream));
    rc = run_plan(ctx, &sl.plan, sl.dseq_h.as<uint8_t>(), sl.dseq_v.as<uint8_t>(), sl.dscore.as<int32_t>(), nullptr,
                  nullptr, false);
    if (rc) return rc;
    ctx->stats_pending = false;
    sl.check_err = ctx->check_err != 0;
    ctx->check_err = 0;
    // Outputs: 6 int32 per pair (score, end_h, end_v, begin_h, begin_v, segment count), the
    // error word, then the per-pair segment slots.
    const bool tb = sl.plan.traceback;
    GBA_CUDA(ctx, sl.out.ensure(size_t(6 * N + 4) * 4));
    int32_t *o = sl.out.as<int32_t>();
    auto d2h = [&](void *dst, const void *src, size_t bytes) {
        return cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, ctx->stream);
    };
    GBA_CUDA(ctx, d2h(o, sl.dscore.ptr, N * 4));
    GBA_CUDA(ctx, d2h(o + N, sl.plan.end_h.ptr, N * 4));
    GBA_CUDA(ctx, d2h(o + 2 * N, sl.plan.end_v.ptr, N * 4));
    o[6 * N] = 0;
    if (sl.check_err) GBA_CUDA(ctx, d2h(o + 6 * N, ctx->err_word.ptr, 4));
    if (tb) {
        GBA_CUDA(ctx, d2h(o + 3 * N, sl.plan.begin_h.ptr, N * 4));
        GBA_CUDA(ctx, d2h(o + 4 * N, sl.plan.begin_v.ptr, N * 4));
        GBA_CUDA(ctx, d2h(o + 5 * N, sl.plan.seg_count.ptr, N * 4));
        GBA_CUDA(ctx, sl.segs.ensure(size_t(std::max<int64_t>(sl.plan.seg_slots_total, 1)) * 16));
        if (sl.plan.seg_slots_total > 0)
            GBA_CUDA(ctx, d2h(sl.segs.ptr, sl.plan.seg_slots.ptr, size_t(sl.plan.seg_slots_total) * 16));
    }
    GBA_CUDA(ctx, cudaEventRecord(sl.done, ctx->stream));
    return GBA_OK;
}

// Moves a finished slot's results to the completed queue.
void srv_harvest(gba_server *s, SrvSlot &sl)
{
    const double now = clock_seconds();
    const int64_t N = int64_t(sl.reqs.size());
    const int32_t *o = sl.out.as<const int32_t>();
    const bool tb = sl.plan.traceback;
    const bool failed = o[6 * N] != 0;
    std::vector<SrvDone> done(N);
    for (int64_t k = 0; k < N; ++k) {
        SrvDone &d = done[k];
        d.r.tag = sl.reqs[k].tag;
        d.r.t_submit = sl.reqs[k].t_submit;
        d.r.t_done = now;
        if (failed) {
            d.r.status = GBA_PAIR_FAILED;
            continue;
        }
        d.r.score = o[k];
        d.r.end_h = o[N + k];
        d.r.end_v = o[2 * N + k];
        d.r.status = sl.plan.status[k];
        if (tb) {
            d.r.begin_h = o[3 * N + k];
            d.r.begin_v = o[4 * N + k];
            const int64_t cnt = o[5 * N + k];
            const int64_t cap = sl.plan.seg_off_host[k + 1] - sl.plan.seg_off_host[k];
            if (cnt > 0 && cnt <= cap) {
                const gba_segment *src = sl.segs.as<const gba_segment>() + sl.plan.seg_off_host[k];
                d.segs.assign(src, src + cnt);
            }
            d.r.n_segments = int32_t(d.segs.size());
        }
    }
    std::lock_guard<std::mutex> lk(s->mu);
    if (failed) s->last_error = "a wait between the bands of a pair ran out";
    for (SrvDone &d : done) s->completed.push_back(std::move(d));
    s->stats.completed += N;
    s->stats.hbm_in_flight -= sl.bytes;
    sl.reqs.clear();
    sl.bytes = 0;
    sl.busy = false;
}

void srv_loop(gba_server *s)
{
    cudaSetDevice(s->device);
    for (;;) {
        bool progress = false;
        bool any_busy = false;
        for (auto &slp : s->slots) {
            SrvSlot &sl = *slp;
            if (!sl.busy) continue;
            const cudaError_t q = cudaEventQuery(sl.done);
            if (q == cudaSuccess) {
                srv_harvest(s, sl);
                progress = true;
            } else if (q != cudaErrorNotReady) {
                cudaGetLastError();
                srv_fail_batch(s, sl, std::string("batch failed: ") + cudaGetErrorString(q));
                progress = true;
            } else {
                any_busy = true;
            }
        }
        for (auto &slp : s->slots) {
            SrvSlot &sl = *slp;
            if (sl.busy) continue;
            {
                // Admission: arrival order, up to the pair cap and the HBM budget.
                std::lock_guard<std::mutex> lk(s->mu);
                int64_t add = 0;
                while (!s->pending.empty() && int64_t(sl.reqs.size()) < s->max_batch) {
                    const int64_t rb = s->pending.front().bytes;
                    if (s->budget > 0 && s->stats.hbm_in_flight + add + rb > s->budget) break;
                    add += rb;
                    sl.reqs.push_back(std::move(s->pending.front()));
                    s->pending.pop_front();
                }
                if (sl.reqs.empty()) break;
                sl.bytes = add;
                sl.busy = true;
                s->stats.pending = int64_t(s->pending.size());
                s->stats.hbm_in_flight += add;
                s->stats.hbm_in_flight_peak = std::max(s->stats.hbm_in_flight_peak, s->stats.hbm_in_flight);
                s->stats.batches += 1;
            }
            const int rc = srv_launch(s, sl);
            if (rc) {
                cudaStreamSynchronize(sl.ctx->stream);
                srv_fail_batch(s, sl, sl.ctx->last_error);
            } else {
                std::lock_guard<std::mutex> lk(s->mu);
                s->stats.cells += sl.plan.cells;
            }
            progress = true;
            any_busy = true;
        }
        std::unique_lock<std::mutex> lk(s->mu);
        if (s->stop && s->pending.empty() && !any_busy) break;
        if (!progress) {
            // Idle or waiting for the GPU: sleep briefly, or until a submit arrives.
            s->cv.wait_for(lk, std::chrono::microseconds(any_busy ? 20 : 200));
        }
    }
}

}  // namespace

extern "C" {

GBA_API double gba_clock_seconds(void) { return clock_seconds(); }

GBA_API int gba_server_create(gba_server **out, const gba_server_config *cfg, const gba_params *params)
{
    if (!out || !cfg || !params) return GBA_EINVAL;
    *out = nullptr;
    if (cfg->streams < 1 || cfg->streams > 16 || cfg->max_batch_pairs < 1 || cfg->hbm_budget_bytes < 0)
        return GBA_EINVAL;
    if ((params->outputs & GBA_OUT_CIGAR) || (params->band_on && params->band_lower > params->band_upper))
        return GBA_EINVAL;
    std::unique_ptr<gba_server> s(new gba_server());
    s->params = *params;
    if (params->matrix) {
        if (params->alphabet_size <= 0 || params->alphabet_size > 32) return GBA_EINVAL;
        s->matrix.assign(params->matrix, params->matrix + params->alphabet_size * params->alphabet_size);
        s->params.matrix = s->matrix.data();
    }
    s->params.flags &= GBA_FLAG_GENERAL_KERNEL;   // no graphs, no packed/autotune paths
    s->params.flags |= GBA_FLAG_NO_GRAPH;
    s->device = cfg->device;
    s->max_batch = cfg->max_batch_pairs;
    s->budget = cfg->hbm_budget_bytes;
    gba_config cc{};
    cc.device = cfg->device;
    for (int i = 0; i < cfg->streams; ++i) {
        std::unique_ptr<SrvSlot> sl(new SrvSlot());
        int rc = gba_create(&sl->ctx, &cc);
        if (rc) {
            for (auto &x : s->slots) gba_destroy(x->ctx);
            return rc;
        }
        for (DevBuf *db : {&sl->dseq_h, &sl->dseq_v, &sl->dscore}) db->bind(sl->ctx->stream);
        // Pinned staging sized for a few thousand requests up front (growing it later can
        // synchronize the device).
        if (sl->seq_h.ensure(4u << 20) != cudaSuccess || sl->seq_v.ensure(4u << 20) != cudaSuccess ||
            sl->out.ensure(1u << 20) != cudaSuccess || sl->segs.ensure(32u << 20) != cudaSuccess) {
            gba_destroy(sl->ctx);
            for (auto &x : s->slots) gba_destroy(x->ctx);
            return GBA_ENOMEM;
        }
        if (cudaEventCreateWithFlags(&sl->done, cudaEventDisableTiming) != cudaSuccess) {
            gba_destroy(sl->ctx);
            for (auto &x : s->slots) gba_destroy(x->ctx);
            return GBA_ECUDA;
        }
        s->slots.push_back(std::move(sl));
    }
    gba_server *raw = s.get();
    s->worker = std::thread(srv_loop, raw);
    *out = s.release();
    return GBA_OK;
}

GBA_API int gba_server_submit(gba_server *s, uint64_t tag, const uint8_t *h, int64_t m, const uint8_t *v, int64_t n)
{
    if (!s || m < 0 || n < 0 || (m > 0 && !h) || (n > 0 && !v)) return GBA_EINVAL;
    if (m > (1 << 30) || n > (1 << 30)) return GBA_EINVAL;
    SrvRequest q;
    q.tag = tag;
    q.bytes = request_bytes(s->params, m, n);
    if (s->budget > 0 && q.bytes > s->budget) {
        std::lock_guard<std::mutex> lk(s->mu);
        s->last_error = "request needs " + std::to_string(q.bytes) + " device bytes, budget is " +
                        std::to_string(s->budget);
        return GBA_EBUDGET;
    }
    q.h.assign(h, h + m);
    q.v.assign(v, v + n);
    q.t_submit = clock_seconds();
    {
        std::lock_guard<std::mutex> lk(s->mu);
        s->pending.push_back(std::move(q));
        s->stats.submitted += 1;
        s->stats.pending = int64_t(s->pending.size());
    }
    s->cv.notify_one();
    return GBA_OK;
}

GBA_API int gba_server_submit_schedule(gba_server *s, const gba_batch *req, const double *at, uint64_t first_tag)
{
    if (!s || !req || (req->num_pairs > 0 && (!at || !req->off_h || !req->off_v || !req->seq_h || !req->seq_v)))
        return GBA_EINVAL;
    const double t0 = clock_seconds();
    for (int64_t k = 0; k < req->num_pairs; ++k) {
        while (clock_seconds() - t0 < at[k]) {
        }
        const int64_t h0 = req->h_shared ? req->off_h[0] : req->off_h[k];
        const int64_t h1 = req->h_shared ? req->off_h[1] : req->off_h[k + 1];
        const int rc = gba_server_submit(s, first_tag + uint64_t(k), req->seq_h + h0, h1 - h0,
                                         req->seq_v + req->off_v[k], req->off_v[k + 1] - req->off_v[k]);
        if (rc) return rc;
    }
    return GBA_OK;
}

GBA_API int gba_server_poll(gba_server *s, gba_request_result *results, int64_t max_results, gba_segment *segments,
                            int64_t segment_capacity, int64_t *num_results, int64_t *num_segments)
{
    if (!s || !num_results || (max_results > 0 && !results)) return GBA_EINVAL;
    *num_results = 0;
    if (num_segments) *num_segments = 0;
    std::lock_guard<std::mutex> lk(s->mu);
    int64_t nr = 0, ns = 0;
    while (nr < max_results && !s->completed.empty()) {
        SrvDone &d = s->completed.front();
        const int64_t cnt = int64_t(d.segs.size());
        if (cnt > 0 && (!segments || ns + cnt > segment_capacity)) {
            if (nr == 0) {
                s->last_error = "segment buffer too small for the next result";
                return GBA_ECAPACITY;
            }
            break;
        }
        results[nr] = d.r;
        results[nr].segment_offset = ns;
        results[nr].n_segments = int32_t(cnt);
        if (cnt > 0) std::memcpy(segments + ns, d.segs.data(), size_t(cnt) * sizeof(gba_segment));
        ns += cnt;
        ++nr;
        s->completed.pop_front();
    }
    *num_results = nr;
    if (num_segments) *num_segments = ns;
    return GBA_OK;
}

GBA_API int gba_server_get_stats(gba_server *s, gba_server_stats *stats)
{
    if (!s || !stats) return GBA_EINVAL;
    std::lock_guard<std::mutex> lk(s->mu);
    *stats = s->stats;
    stats->pending = int64_t(s->pending.size());
    return GBA_OK;
}

GBA_API int gba_server_last_error(gba_server *s, char *buf, size_t size)
{
    if (!s || !buf || size == 0) return GBA_EINVAL;
    std::lock_guard<std::mutex> lk(s->mu);
    std::snprintf(buf, size, "%s", s->last_error.c_str());
    return GBA_OK;
}

GBA_API int gba_server_destroy(gba_server *s)
{
    if (!s) return GBA_OK;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        s->stop = true;
        s->pending.clear();
    }
    s->cv.notify_one();
    if (s->worker.joinable()) s->worker.join();
    cudaSetDevice(s->device);
    for (auto &sl : s->slots) {
        if (sl->ctx) cudaStreamSynchronize(sl->ctx->stream);
        sl->plan.release();
        sl->dseq_h.release();
        sl->dseq_v.release();
        sl->dscore.release();
        sl->seq_h.release();
        sl->seq_v.release();
        sl->out.release();
        sl->segs.release();
        if (sl->done) cudaEventDestroy(sl->done);
        gba_destroy(sl->ctx);
    }
    delete s;
    return GBA_OK;
}

}  // extern "C"
