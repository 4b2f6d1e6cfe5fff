// chain_host.cuh -- host side of gba_banded_chain (included at the end of engine.cu).
//
// A host pass runs every chain's driver in plan mode (grid geometry only) to size its scratch;
// chains are then processed in chunks whose scratch fits kChainArenaBudget: one thread per chain
// runs the whole chain (k_banded_chain), the per-chain trace lengths come back, the host lays out
// the dense output and k_chain_pack copies each chain's first trace there.
#pragma once

#include "chain_kernels.cuh"

namespace {

constexpr size_t kChainArenaBudget = size_t(24) << 30;

}  // namespace

extern "C" {

GBA_API int gba_banded_chain(gba_context *ctx, const gba_chain_params *params, const gba_batch *b,
                             const gba_chain_seeds *sd, gba_chain_result *res)
{
    if (!ctx || !params || !b || !sd || !res) return GBA_EINVAL;
    const auto t0 = std::chrono::steady_clock::now();
    GBA_CUDA(ctx, cudaSetDevice(ctx->device));
    const int64_t N = b->num_pairs;
    if (N < 0) return fail(ctx, GBA_EINVAL, "negative num_pairs");
    if (params->band_extension < 1 || params->band_extension > (1 << 20))
        return fail(ctx, GBA_EINVAL, "band_extension must be in 1..2^20");
    const int32_t T = params->max_traces ? params->max_traces : 8;
    if (T < 1 || T > 32) return fail(ctx, GBA_EINVAL, "max_traces must be in 1..32");
    const int lim = 1 << 20;
    for (const gba_simple_score *s : {&params->anchor, &params->gap})
        if (std::abs(s->match) > lim || std::abs(s->mismatch) > lim || std::abs(s->gap_extend) > lim ||
            std::abs(s->gap_open) > lim)
            return fail(ctx, GBA_EUNSUPPORTED, "scores beyond +-2^20");
    if (!res->score || !res->status || !res->segment_offsets) return fail(ctx, GBA_EINVAL, "null result array");
    res->segment_offsets[0] = 0;
    if (N == 0) return GBA_OK;
    if (!b->off_h || !b->off_v || !b->seq_h || !b->seq_v) return fail(ctx, GBA_EINVAL, "null sequence or offset pointer");
    if (!sd->seed_offsets || (sd->seed_offsets[N] > 0 && !sd->seeds)) return fail(ctx, GBA_EINVAL, "null seed array");
    if (sd->seed_offsets[0] != 0) return fail(ctx, GBA_EINVAL, "seed_offsets[0] must be 0");
    cudaStream_t st = ctx->stream;

    chain::Scheme anchor{params->anchor.match, params->anchor.mismatch, params->anchor.gap_extend,
                         params->anchor.gap_open};
    chain::Scheme gap{params->gap.match, params->gap.mismatch, params->gap.gap_extend, params->gap.gap_open};
    // affine cells when either scheme opens gaps at another cost than it extends them
    // (seeds/banded_chain_alignment_profile.h:235-262)
    const int affine = (anchor.ext != anchor.open) || (gap.ext != gap.open);

    // ---- plan pass: per-chain scratch sizes from the grids' geometry ----
    std::vector<chain::ChainDesc> desc(static_cast<size_t>(N));
    std::vector<int64_t> bytes(static_cast<size_t>(N));
    const int64_t nseeds = sd->seed_offsets[N];
    for (int64_t k = 0; k < N; ++k) {
        const int64_t h0 = b->h_shared ? b->off_h[0] : b->off_h[k], h1 = b->h_shared ? b->off_h[1] : b->off_h[k + 1];
        const int64_t v0 = b->off_v[k], v1 = b->off_v[k + 1];
        const int64_t s0 = sd->seed_offsets[k], s1 = sd->seed_offsets[k + 1];
        if (h0 < 0 || v0 < 0 || h1 < h0 || v1 < v0 || s1 < s0 || s1 > nseeds)
            return fail(ctx, GBA_EINVAL, "bad offsets of pair %lld", (long long)k);
        if (h1 - h0 > (1 << 28) || v1 - v0 > (1 << 28) || s1 - s0 > (1 << 28))
            return fail(ctx, GBA_EUNSUPPORTED, "pair %lld: sequences or chain beyond 2^28", (long long)k);
        chain::ChainDesc &d = desc[k];
        d = chain::ChainDesc{};
        d.h_off = h0;
        d.v_off = v0;
        d.seed_off = s0;
        d.m = int32_t(h1 - h0);
        d.n = int32_t(v1 - v0);
        d.n_seeds = int32_t(s1 - s0);
    }
#pragma omp parallel for schedule(dynamic, 64)
    for (int64_t k = 0; k < N; ++k) {
        chain::ChainDesc &d = desc[k];
        chain::Plan &pl = d.plan;
        pl = chain::Plan{};
        pl.gseg_cap = d.m + d.n + 8;
        chain::Engine e{};
        e.plan = true;
        e.warp = false;
        e.lane = 0;
        e.anchor = anchor;
        e.gap = gap;
        e.fe = params->free_ends;
        e.affine = affine;
        e.k = params->band_extension;
        e.max_traces = T;
        e.h = nullptr;
        e.v = nullptr;
        e.m = d.m;
        e.n = d.n;
        e.pl = &pl;
        e.run(sd->seeds + 4 * d.seed_off, d.n_seeds);
        pl.status = e.err;
        if (pl.set_cap < pl.mp_cap) pl.set_cap = pl.mp_cap;
        if (pl.col_rows < 1) pl.col_rows = 1;
        bytes[k] = chain::layout(pl, T, nullptr, nullptr) + 16;
    }
    for (int64_t k = 0; k < N; ++k)
        if (size_t(bytes[k]) > kChainArenaBudget)
            return fail(ctx, GBA_EUNSUPPORTED, "pair %lld needs more scratch than one chunk", (long long)k);

    // ---- inputs ----
    const int64_t hbytes = b->h_shared ? b->off_h[1] : b->off_h[N], vbytes = b->off_v[N];
    GBA_CUDA(ctx, ctx->seq_h.ensure(size_t(hbytes) + 16));
    GBA_CUDA(ctx, ctx->seq_v.ensure(size_t(vbytes) + 16));
    if (hbytes) GBA_CUDA(ctx, cudaMemcpyAsync(ctx->seq_h.ptr, b->seq_h, hbytes, cudaMemcpyHostToDevice, st));
    if (vbytes) GBA_CUDA(ctx, cudaMemcpyAsync(ctx->seq_v.ptr, b->seq_v, vbytes, cudaMemcpyHostToDevice, st));
    GBA_CUDA(ctx, ctx->bc_seeds.ensure(size_t(nseeds) * 16 + 16));
    if (nseeds) GBA_CUDA(ctx, cudaMemcpyAsync(ctx->bc_seeds.ptr, sd->seeds, size_t(nseeds) * 16, cudaMemcpyHostToDevice, st));

    int64_t cells = 0, trace_total = 0;
    for (const chain::ChainDesc &d : desc) {
        cells += d.plan.cells;
        trace_total += d.plan.trace_total;
    }
    int64_t wseg = 0;
    float dp_ms = 0;
    int launches = 0;
    int64_t c0 = 0;
    while (c0 < N) {
        int64_t c1 = c0, tot = 0;
        while (c1 < N && size_t(tot + bytes[c1]) <= kChainArenaBudget) {
            desc[c1].arena_off = tot;
            tot += bytes[c1++];
        }
        const int64_t nc = c1 - c0;
        GBA_CUDA(ctx, ctx->bc_desc.ensure(size_t(nc) * sizeof(chain::ChainDesc)));
        GBA_CUDA(ctx, ctx->bc_arena.ensure(size_t(tot) + 16));
        GBA_CUDA(ctx, ctx->bc_out.ensure(size_t(nc) * 16 + 64));
        GBA_CUDA(ctx, cudaMemcpyAsync(ctx->bc_desc.ptr, desc.data() + c0, size_t(nc) * sizeof(chain::ChainDesc),
                                      cudaMemcpyHostToDevice, st));
        int32_t *o = ctx->bc_out.as<int32_t>();
        ChainArgs a{};
        a.seq_h = ctx->seq_h.as<uint8_t>();
        a.seq_v = ctx->seq_v.as<uint8_t>();
        a.seeds = ctx->bc_seeds.as<int32_t>();
        a.chains = ctx->bc_desc.as<chain::ChainDesc>();
        a.num_chains = nc;
        a.arena = ctx->bc_arena.as<uint8_t>();
        a.anchor = anchor;
        a.gap = gap;
        a.free_ends = params->free_ends;
        a.band_ext = params->band_extension;
        a.affine = affine;
        a.max_traces = T;
        a.score = o;
        a.status = o + nc;
        a.n_traces = o + 2 * nc;
        a.seg_count = o + 3 * nc;
        GBA_CUDA(ctx, cudaEventRecord(ctx->ev[0], st));
        launch_banded_chain(a, st);
        GBA_CUDA(ctx, cudaGetLastError());
        GBA_CUDA(ctx, cudaEventRecord(ctx->ev[1], st));
        ++launches;
        std::vector<int32_t> outh(size_t(nc) * 4);
        GBA_CUDA(ctx, cudaMemcpyAsync(outh.data(), o, outh.size() * 4, cudaMemcpyDeviceToHost, st));
        GBA_CUDA(ctx, cudaStreamSynchronize(st));
        {
            float ms = 0;
            GBA_CUDA(ctx, cudaEventElapsedTime(&ms, ctx->ev[0], ctx->ev[1]));
            dp_ms += ms;
        }
        std::vector<int64_t> dense(size_t(nc) + 1, 0);
        for (int64_t i = 0; i < nc; ++i) {
            res->score[c0 + i] = outh[size_t(i)];
            res->status[c0 + i] = outh[size_t(nc + i)];
            if (res->num_traces) res->num_traces[c0 + i] = outh[size_t(2 * nc + i)];
            dense[i + 1] = dense[i] + outh[size_t(3 * nc + i)];
        }
        const int64_t total = dense[nc];
        if (wseg + total > res->segment_capacity || (total && !res->segments))
            return fail(ctx, GBA_ECAPACITY, "segment_capacity too small");
        if (total) {
            GBA_CUDA(ctx, ctx->bc_dense.ensure(size_t(total) * 16 + 16));
            GBA_CUDA(ctx, ctx->bc_offs.ensure(size_t(nc) * 8 + 16));
            GBA_CUDA(ctx, cudaMemcpyAsync(ctx->bc_offs.ptr, dense.data(), size_t(nc) * 8, cudaMemcpyHostToDevice, st));
            launch_chain_pack(a.chains, nc, a.arena, T, a.seg_count, ctx->bc_offs.as<int64_t>(),
                              ctx->bc_dense.as<chain::Seg>(), st);
            GBA_CUDA(ctx, cudaGetLastError());
            ++launches;
            GBA_CUDA(ctx, cudaMemcpyAsync(res->segments + wseg, ctx->bc_dense.ptr, size_t(total) * 16,
                                          cudaMemcpyDeviceToHost, st));
            GBA_CUDA(ctx, cudaStreamSynchronize(st));
        }
        for (int64_t i = 0; i < nc; ++i) res->segment_offsets[c0 + i + 1] = wseg + dense[i + 1];
        wseg += total;
        c0 = c1;
    }
    // With the default trace budget, chains that held more co-optimal traces at once run again with
    // 32 trace slots (only those chains; their outputs are spliced into place).
    std::vector<int64_t> retry;
    if (params->max_traces == 0)
        for (int64_t k = 0; k < N; ++k)
            if (res->status[k] == chain::ST_CAPACITY) retry.push_back(k);
    if (!retry.empty()) {
        const int64_t R = int64_t(retry.size());
        std::vector<uint8_t> rh, rv;
        std::vector<int64_t> roh(size_t(R) + 1, 0), rov(size_t(R) + 1, 0), rso(size_t(R) + 1, 0);
        std::vector<int32_t> rseeds;
        for (int64_t i = 0; i < R; ++i) {
            const chain::ChainDesc &d = desc[retry[i]];
            rh.insert(rh.end(), b->seq_h + d.h_off, b->seq_h + d.h_off + d.m);
            rv.insert(rv.end(), b->seq_v + d.v_off, b->seq_v + d.v_off + d.n);
            rseeds.insert(rseeds.end(), sd->seeds + 4 * d.seed_off, sd->seeds + 4 * (d.seed_off + d.n_seeds));
            roh[i + 1] = int64_t(rh.size());
            rov[i + 1] = int64_t(rv.size());
            rso[i + 1] = rso[i] + d.n_seeds;
        }
        rh.push_back(0);
        rv.push_back(0);
        rseeds.resize(rseeds.size() + 4);
        gba_batch b2{R, rh.data(), roh.data(), rv.data(), rov.data(), 0, 0};
        gba_chain_seeds s2{rseeds.data(), rso.data()};
        gba_chain_params p2 = *params;
        p2.max_traces = 32;
        std::vector<int32_t> sc2(static_cast<size_t>(R)), st2(static_cast<size_t>(R)), nt2(static_cast<size_t>(R));
        std::vector<int64_t> off2(static_cast<size_t>(R) + 1);
        const int64_t cap2 = roh[R] + rov[R] + 8 * R + 8;
        std::vector<gba_segment> seg2(static_cast<size_t>(cap2));
        gba_chain_result r2{sc2.data(), st2.data(), nt2.data(), seg2.data(), cap2, off2.data()};
        const int rc = gba_banded_chain(ctx, &p2, &b2, &s2, &r2);
        if (rc != GBA_OK) return rc;
        dp_ms += ctx->stats.dp_kernel_ms;
        launches += ctx->stats.kernel_launches;
        // splice: the retried chains' segments replace their empty slots
        std::vector<gba_segment> old(res->segments, res->segments + wseg);
        std::vector<int64_t> oldoff(res->segment_offsets, res->segment_offsets + N + 1);
        int64_t total = 0;
        for (int64_t i = 0; i < R; ++i) total += off2[i + 1] - off2[i];
        if (wseg + total > res->segment_capacity || (total && !res->segments))
            return fail(ctx, GBA_ECAPACITY, "segment_capacity too small");
        int64_t w = 0, ri = 0;
        for (int64_t k = 0; k < N; ++k) {
            if (ri < R && retry[ri] == k) {
                const int64_t c = off2[ri + 1] - off2[ri];
                std::copy(seg2.begin() + off2[ri], seg2.begin() + off2[ri + 1], res->segments + w);
                res->score[k] = sc2[ri];
                res->status[k] = st2[ri];
                if (res->num_traces) res->num_traces[k] = nt2[ri];
                w += c;
                ++ri;
            } else {
                const int64_t c = oldoff[k + 1] - oldoff[k];
                std::copy(old.begin() + oldoff[k], old.begin() + oldoff[k + 1], res->segments + w);
                w += c;
            }
            res->segment_offsets[k + 1] = w;
        }
    }
    ctx->stats = gba_stats{};
    ctx->stats.dp_kernel_ms = dp_ms;
    ctx->stats.kernel_launches = launches;
    ctx->stats.cells = cells;
    ctx->stats.trace_bytes = trace_total;
    ctx->stats.call_ms = std::chrono::duration<float, std::milli>(std::chrono::steady_clock::now() - t0).count();
    return GBA_OK;
}

}  // extern "C"
