// engine.cu -- the C-ABI of the GB300 batch alignment engine (include/seqan_gb300.h).
//
// A call runs: validate -> plan (lengths, int16 range check, length-binned order, scratch
// and trace offsets) -> upload -> DP kernel -> [traceback kernel -> compaction] -> download.
// There is no CPU fallback: every alignment is computed by the kernels in this file.
#include "../../include/seqan_gb300.h"

#include "dp_common.cuh"
#include "dp_kernels.cuh"
#include "traceback_kernels.cuh"
#include "dp16x2_kernels.cuh"
#include "banded_launch.cuh"
#include "dp_banded_kernels.cuh"
#include "dp_warp_kernels.cuh"
#include "dp_warp2_kernels.cuh"
#include "dp_dynamic_kernels.cuh"
#include "seed_kernels.cuh"
#include "extend_kernels.cuh"
#include "int_peak.cuh"

#include <cub/device/device_scan.cuh>
#include <cuda_runtime.h>
#include <omp.h>

#include <algorithm>
#include <chrono>
#include <cstdarg>
#include <cstdlib>
#include <cstdio>
#include <cstring>
#include <functional>
#include <map>
#include <memory>
#include <string>
#include <vector>

using namespace gba;

namespace {

// ------------------------------------------------------------------------------------
// Device buffer that only grows.  Bound to a stream, it is allocated and freed in stream
// order (cudaMallocAsync / cudaFreeAsync): growing it does not synchronize the device, so
// batches in flight on other streams keep running.  The buffer is idle whenever it grows.
// ------------------------------------------------------------------------------------
struct DevBuf {
    void *ptr = nullptr;
    size_t cap = 0;
    cudaStream_t stream = nullptr;
    bool async = false;
    void bind(cudaStream_t s)
    {
        if (ptr && async != true) release();
        stream = s;
        async = true;
    }
    cudaError_t ensure(size_t bytes)
    {
        if (bytes <= cap) return cudaSuccess;
        release();
        size_t want = std::max<size_t>(bytes, 256);
        cudaError_t e = async ? cudaMallocAsync(&ptr, want, stream) : cudaMalloc(&ptr, want);
        if (e == cudaSuccess) cap = want;
        else ptr = nullptr;
        return e;
    }
    void release()
    {
        if (ptr) {
            if (async) cudaFreeAsync(ptr, stream);
            else cudaFree(ptr);
        }
        ptr = nullptr;
        cap = 0;
    }
    template <typename T> T *as() const { return static_cast<T *>(ptr); }
};

}  // namespace

struct gba_plan {
    // host side
    int64_t num_pairs = 0;
    int64_t num_slots = 0;          // valid pairs
    bool traceback = false;
    bool cigar = false;
    bool affine = false;
    bool dynamic = false;           // DynamicGaps cells (dp_dynamic_kernels.cuh)
    bool local = false;
    bool extend = false;            // GBA_ALIGN_EXTEND (banded kernel in its AlignExtend_ mode)
    bool matrix = false;
    int32_t free_ends = 0;
    gba_params params{};
    std::vector<int32_t> matrix_host;
    std::vector<int32_t> status;    // per pair GBA_PAIR_*
    std::vector<int32_t> invalid_score;  // per invalid pair
    int64_t cells = 0;
    int64_t trace_total = 0;
    int64_t seg_slots_total = 0;
    int64_t cigar_slots_total = 0;
    int64_t scratch_total = 0;      // int2 elements
    int64_t seq_h_bytes = 0, seq_v_bytes = 0;
    // device side
    DevBuf pairs, order, warp_scratch, scratch, trace, best_e, best_f, matrix_dev;
    DevBuf end_h, end_v, score_tmp, begin_h, begin_v;
    DevBuf seg_slots, seg_slot_off, seg_count, seg_dense_off, seg_dense, seg_count64;
    DevBuf cig_slots, cig_slot_off, cig_count, cig_dense_off, cig_dense, cig_count64;
    DevBuf cub_tmp;
    size_t cub_tmp_bytes = 0;
    // Packed two-pairs-per-thread path (dp16x2_kernels.cuh).
    int64_t num16 = 0;              // slots (two pairs each)
    int rows16 = 32;                // rows per register strip
    int64_t codes_total = 0, bnd16_total = 0;
    DevBuf slots16, warp_codes, warp_hwords, codes16, warp_bnd16, bnd16, counter16;
    int32_t tasks16 = 0;
    // Warp-per-pair path (dp_warp_kernels.cuh).
    bool use_warp = false;
    int warp_rows = 8;
    int64_t grid_warp = 0;
    DevBuf rowbuf, rowbuf_off, counter_warp, tasks_warp, band_base, band_state;
    // Packed 16-bit warp path (dp_warp2_kernels.cuh): pairs in cost order, one task each.
    int64_t num_w2 = 0;             // pairs
    int64_t num_w2_tasks = 0;       // (pair, band) tasks
    int64_t num_w2_states = 0;      // bands of pipelined pairs
    int64_t grid_w2 = 0;
    DevBuf tasks_w2, order_w2, rowbuf_w2, rowbuf_w2_off, counter_w2, band_w2, band_w2_base;
    std::vector<int2> h_w2tasks;
    std::vector<int64_t> w2b_start, w2b_count;   // plain form: task ranges per length bucket
    int64_t num_warp_tasks = 0;     // (pair, band) work items
    int64_t num_band_states = 0;    // bands of pairs that span more than one band
    int64_t num_tiled_tb = 0;       // leading slots whose traceback a whole warp walks
    int64_t grid16[8] = {};         // resident blocks of each packed-kernel variant
    int variant16 = 0;              // chosen tiling variant
    bool tune_pending = false;      // autotune at the first run
    int64_t tune_key = 0;
    int32_t launches = 0;           // kernels one run launches
    int err_slot = 0;               // word of the context's error buffer this plan's kernels use
    // Plain per-bucket mode: one launch per 8-residue length bucket.  bucket_*: slot ranges of
    // the one-pair-per-thread kernel; b16_*: slot ranges of the packed kernel; wb_*: task
    // ranges of the warp kernel.
    std::vector<int64_t> bucket_start, bucket_count, b16_start, b16_count, wb_start, wb_count;
    // Captured launch sequence (replayed while the device pointers stay the same).
    cudaGraphExec_t graph = nullptr;
    const void *graph_key[5] = {};
    int64_t seg_dense_total = -1, cig_dense_total = -1;
    std::vector<int64_t> seg_off_host;   // per-pair segment slot offsets (num_pairs + 1)
    // Host-side planning arrays, reused by the next build of this plan.
    std::vector<PairDesc> h_desc;
    std::vector<uint32_t> h_keys16, h_keys, h_key, h_keys2;
    std::vector<int32_t> h_idx16, h_idx, h_idx2;
    std::vector<uint8_t> h_cls;
    std::vector<Slot16> h_slots16;
    bool owned = true;
    void release()
    {
        DevBuf *all[] = {&pairs, &order, &warp_scratch, &scratch, &trace, &best_e, &best_f, &matrix_dev,
                         &end_h, &end_v, &score_tmp, &begin_h, &begin_v, &seg_slots, &seg_slot_off,
                         &seg_count, &seg_dense_off, &seg_dense, &seg_count64, &cig_slots,
                         &cig_slot_off, &cig_count, &cig_dense_off, &cig_dense, &cig_count64, &cub_tmp,
                         &slots16, &warp_codes, &warp_hwords, &codes16, &warp_bnd16, &bnd16, &counter16,
                         &rowbuf, &rowbuf_off, &counter_warp, &tasks_warp, &band_base, &band_state,
                         &tasks_w2, &order_w2, &rowbuf_w2, &rowbuf_w2_off, &counter_w2, &band_w2, &band_w2_base};
        for (DevBuf *b : all) b->release();
        drop_graph();
    }
    void bind(cudaStream_t s)
    {
        DevBuf *all[] = {&pairs, &order, &warp_scratch, &scratch, &trace, &best_e, &best_f, &matrix_dev,
                         &end_h, &end_v, &score_tmp, &begin_h, &begin_v, &seg_slots, &seg_slot_off,
                         &seg_count, &seg_dense_off, &seg_dense, &seg_count64, &cig_slots,
                         &cig_slot_off, &cig_count, &cig_dense_off, &cig_dense, &cig_count64, &cub_tmp,
                         &slots16, &warp_codes, &warp_hwords, &codes16, &warp_bnd16, &bnd16, &counter16,
                         &rowbuf, &rowbuf_off, &counter_warp, &tasks_warp, &band_base, &band_state,
                         &tasks_w2, &order_w2, &rowbuf_w2, &rowbuf_w2_off, &counter_w2, &band_w2, &band_w2_base};
        for (DevBuf *b : all)
            if (!b->async || b->stream != s) b->bind(s);
    }
    void drop_graph()
    {
        if (graph) cudaGraphExecDestroy(graph);
        graph = nullptr;
        for (auto &k : graph_key) k = nullptr;
    }
    size_t device_bytes() const
    {
        const DevBuf *all[] = {&pairs, &order, &warp_scratch, &scratch, &trace, &best_e, &best_f,
                               &matrix_dev, &end_h, &end_v, &score_tmp, &begin_h, &begin_v, &seg_slots,
                               &seg_slot_off, &seg_count, &seg_dense_off, &seg_dense, &seg_count64,
                               &cig_slots, &cig_slot_off, &cig_count, &cig_dense_off, &cig_dense,
                               &cig_count64, &cub_tmp, &slots16, &warp_codes, &warp_hwords, &codes16,
                               &warp_bnd16, &bnd16, &counter16, &rowbuf, &rowbuf_off, &counter_warp,
                               &tasks_warp, &band_base, &band_state, &tasks_w2, &order_w2, &rowbuf_w2,
                               &rowbuf_w2_off, &counter_w2, &band_w2, &band_w2_base};
        size_t s = 0;
        for (const DevBuf *b : all) s += b->cap;
        return s;
    }
};

struct gba_context {
    std::map<int64_t, int> tuning;  // batch shape -> packed-kernel variant (autotuner results)
    std::map<const void *, int64_t> grid_cache;   // kernel -> resident blocks on this device
    int device = 0;
    int64_t budget = 0;
    cudaStream_t stream = nullptr;
    cudaEvent_t ev[6] = {};
    std::string last_error;
    gba_stats stats{};
    bool stats_pending = false;     // events of the last run not read yet
    gba_plan oneshot;               // buffers reused by gba_align_batch
    DevBuf seq_h, seq_v;            // device copies of the inputs for gba_align_batch
    DevBuf out_score, out_end_h, out_end_v;
    DevBuf err_word;                // one word per plan slot, set by a kernel whose bounded wait ran out
    uint32_t check_err = 0;         // slots of err_word the runs since the last check can set
    std::vector<std::unique_ptr<gba_plan>> chunk_plans;   // gba_align_batch chunks 1.. (0 = oneshot)
    std::vector<cudaEvent_t> chunk_ev;                    // 3 per chunk
    // seed extension: device copies of a host batch, the kernels' work words and scratch
    DevBuf xs_seq_h, xs_seq_v, xs_off_h, xs_off_v, xs_ids, xs_seeds, xs_scores, xs_matrix, xs_work, xs_scratch,
        xs_results;
    bool xs_check = false;          // a device seed-extension run whose error word is unread
    std::map<std::pair<const void *, size_t>, int64_t> xs_grid;   // (kernel, smem) -> resident blocks
    // alignment extension: tasks, per-task results, trace, segments, scratch
    DevBuf xa_tasks, xa_out, xa_trace, xa_segs, xa_segoff, xa_segcnt, xa_scratch, xa_next, xa_packoff, xa_packed;
    DevBuf en_pairs, en_mat, en_forb, en_heap, en_steps, en_slots, en_out, en_dense, en_offs, en_cnt;   // gba_local_enumerate
    DevBuf bc_seeds, bc_desc, bc_arena, bc_out, bc_dense, bc_offs;   // gba_banded_chain
    DevBuf bz_in, bz_slots, bz_scratch, bz_meta, bz_out;             // gba_bgzf_compress
    // packed input: the codes are already in seq_h / seq_v (gba_align_packed unpacked them)
    bool device_codes = false;
    DevBuf pk_words, pk_off_h, pk_off_v;
    DevBuf sam_in, sam_len, sam_tmp, sam_out;   // gba_format_sam
    DevBuf fa_text, fa_sum, fa_tmp, fa_out, fa_chunk;   // gba_read_fasta
};

// Banded kernel launchers (banded_launch_*.cu, translation units of their own).
BandLauncher pick_banded(bool a, bool l, bool m, bool t)
{
    return a ? (l ? pick_banded_affine_local(m, t) : pick_banded_affine_global(m, t))
             : (l ? pick_banded_linear_local(m, t) : pick_banded_linear_global(m, t));
}
BandLauncher pick_banded_ext(bool a, bool m, bool t)
{
    return a ? pick_banded_ext_affine(m, t) : pick_banded_ext_linear(m, t);
}

namespace {

int fail(gba_context *ctx, int code, const char *fmt, ...)
{
    if (ctx) {
        char buf[512];
        va_list ap;
        va_start(ap, fmt);
        vsnprintf(buf, sizeof(buf), fmt, ap);
        va_end(ap);
        ctx->last_error = buf;
    }
    return code;
}

#define GBA_CUDA(ctx, call)                                                                  \
    do {                                                                                     \
        cudaError_t e_ = (call);                                                             \
        if (e_ != cudaSuccess) {                                                             \
            int code_ = (e_ == cudaErrorMemoryAllocation) ? GBA_ENOMEM : GBA_ECUDA;          \
            return fail(ctx, code_, "%s failed: %s (%s:%d)", #call, cudaGetErrorString(e_),  \
                        __FILE__, __LINE__);                                                 \
        }                                                                                    \
    } while (0)

constexpr int kBlock = 128;
constexpr int kMaxBandWidth = 512;   // band slots a thread keeps (local memory)
// Below this many pairs two-pairs-per-thread leaves most SMs idle; one warp per pair fills them.
constexpr int64_t kPackedMinPairs = 32768;
// gba_align_batch splits large score-only batches into up to kMaxChunks contiguous chunks of at
// least kChunkPairs pairs: each chunk is planned on the host while the previous one runs.  A
// chunk must still fill the GPU on its own (100,000 short pairs split in two ran 37% slower).
constexpr int kMaxChunks = 8;
constexpr int64_t kChunkPairs = 200000;
// Pairs at least this wide pipeline their bands across warps even in large batches: the ~130
// steps a pipelined band waits before its first column are then a small share of its work.
constexpr int kPipelineMinCols = 1024;
// The packed 16-bit warp kernel takes pairs narrower than kPipelineMinCols with at most kW2MaxRows
// rows, in batches of at least kW2MinPairs pairs (it runs each pair's bands in order on one warp).
constexpr int kW2MaxRows = 4096;
// Pairs of at least this many 256-row bands pipeline their bands across warps.
constexpr int kW2PipeBands = 3;
constexpr int64_t kW2MinPairs = 4096;

// _checkBandProperties (align/dp_algorithm_impl.h:193-234): the band must meet the matrix and
// may leave it only across sides whose end gaps are free.
// Trace bytes of one band column for the 32 lanes of a warp: 4-bit codes for bands of at most
// kBandFastW diagonals, otherwise one byte per slot.
int band_col_bytes(int W) { return band_trace4(W) ? band4_col_bytes(W) : band_trace_stride(W) * 32; }

bool band_valid(const gba_params &p, int64_t m, int64_t n, int fe)
{
    const int64_t lo = p.band_lower, up = p.band_upper;
    if (up < -n || lo > m) return false;
    if (up < 0 && !(fe & GBA_FREE_LEFT)) return false;
    if (lo > 0 && !(fe & GBA_FREE_TOP)) return false;
    if (up + n < m && !(fe & GBA_FREE_BOTTOM)) return false;
    if (lo + n > m && !(fe & GBA_FREE_RIGHT)) return false;
    return true;
}

// In-band cells (i, j), 1 <= i <= n, 1 <= j <= m, lower <= j - i <= upper.
int64_t band_cells(int64_t m, int64_t n, int64_t lo, int64_t up)
{
    int64_t c = 0;
    for (int64_t dg = std::max(lo, 1 - n); dg <= std::min(up, m - 1); ++dg)
        c += std::min(n, m - dg) - std::max<int64_t>(1, 1 - dg) + 1;
    return c;
}

bool is_affine(const gba_params &p)
{
    if (p.gap_model == GBA_GAPS_LINEAR || p.gap_model == GBA_GAPS_DYNAMIC) return false;
    if (p.gap_model == GBA_GAPS_AFFINE) return true;
    return p.gap_open != p.gap_extend;
}

int max_sub_abs(const gba_params &p, const std::vector<int32_t> &mat, int *max_pos)
{
    int mx = 0, mp = 0;
    if (!mat.empty()) {
        for (int32_t v : mat) {
            mx = std::max(mx, std::abs(v));
            mp = std::max(mp, int(v));
        }
    } else {
        mx = std::max(std::abs(p.match), std::abs(p.mismatch));
        mp = std::max(std::max(p.match, p.mismatch), 0);
    }
    *max_pos = mp;
    return mx;
}

// True when every real cell value of an m x n problem stays inside the range where the
// reference's wrapping int16 cells equal exact arithmetic: the best score is at most
// max_pos * min(m, n) <= 32767, and no value falls to the int16 "infinity" of -16384
// (align/dp_cell.h:143-146).  Scores are bounded below by the all-gap path.
bool int16_exact(const gba_params &p, int max_pos, int64_t m, int64_t n, bool local)
{
    const int64_t open = std::abs(p.gap_open), ext = std::abs(p.gap_extend);
    const int64_t upper = int64_t(max_pos) * std::min(m, n);
    if (upper > 32767 - 64) return false;
    if (local) return true;
    const int64_t lower = -(3 * open + ext * (m + n + 2));
    return lower > -16384 + 2 * (open + ext) + 64;
}

int validate(gba_context *ctx, const gba_params *p, const gba_batch *b)
{
    if (!p || !b) return fail(ctx, GBA_EINVAL, "null params or batch");
    if (p->mode != GBA_GLOBAL && p->mode != GBA_LOCAL && p->mode != GBA_ALIGN_EXTEND)
        return fail(ctx, GBA_EINVAL, "bad mode %d", p->mode);
    if (p->mode == GBA_ALIGN_EXTEND) {
        if (!p->band_on)
            return fail(ctx, GBA_EUNSUPPORTED, "GBA_ALIGN_EXTEND is banded only (unbanded: gba_extend_alignments)");
        if (p->score_bits != 32) return fail(ctx, GBA_EUNSUPPORTED, "GBA_ALIGN_EXTEND runs 32-bit cells");
        if (p->gap_model == GBA_GAPS_DYNAMIC)
            return fail(ctx, GBA_EUNSUPPORTED, "DynamicGaps cells are not an extension profile");
        if ((p->flags & GBA_FLAG_XDROP) && std::abs(int64_t(p->xdrop)) >= (int64_t(1) << 30))
            return fail(ctx, GBA_EUNSUPPORTED, "xdrop beyond +-2^30");
    } else if (p->flags & GBA_FLAG_XDROP) {
        return fail(ctx, GBA_EINVAL, "GBA_FLAG_XDROP needs mode GBA_ALIGN_EXTEND");
    }
    if (p->gap_model < 0 || p->gap_model > 3) return fail(ctx, GBA_EINVAL, "bad gap model");
    if (p->gap_model == GBA_GAPS_DYNAMIC && p->band_on)
        return fail(ctx, GBA_EUNSUPPORTED, "DynamicGaps cells are supported unbanded only");
    if (p->score_bits != 16 && p->score_bits != 32) return fail(ctx, GBA_EINVAL, "score_bits must be 16 or 32");
    if (p->free_ends & ~15) return fail(ctx, GBA_EINVAL, "bad free_ends bits");
    if (p->matrix && (p->alphabet_size <= 0 || p->alphabet_size > 32))
        return fail(ctx, GBA_EINVAL, "alphabet_size must be in 1..32");
    if (b->num_pairs < 0) return fail(ctx, GBA_EINVAL, "negative num_pairs");
    // Pair indices are 32-bit (slot orders, task lists) and the output scans count num_pairs + 1
    // items in an int.
    if (b->num_pairs > int64_t(INT32_MAX) - 1) return fail(ctx, GBA_EINVAL, "more than 2^31 - 2 pairs in one batch");
    if (b->num_pairs > 0 && (!b->off_h || !b->off_v || ((!b->seq_h || !b->seq_v) && !ctx->device_codes)))
        return fail(ctx, GBA_EINVAL, "null sequence or offset pointer");
    if (p->band_on) {
        if (p->band_lower > p->band_upper) return fail(ctx, GBA_EINVAL, "band_lower > band_upper");
        if (int64_t(p->band_upper) - p->band_lower + 1 > kMaxBandWidth)
            return fail(ctx, GBA_EUNSUPPORTED, "band wider than %d diagonals", kMaxBandWidth);
    }
    if (p->tile_variant < 0 || p->tile_variant > GBA_TILE_VARIANTS)
        return fail(ctx, GBA_EINVAL, "tile_variant must be in 0..%d", GBA_TILE_VARIANTS);
    if ((p->outputs & GBA_OUT_CIGAR) && !(p->outputs & GBA_OUT_SEGMENTS))
        return fail(ctx, GBA_EINVAL, "GBA_OUT_CIGAR requires GBA_OUT_SEGMENTS");
    return GBA_OK;
}

int plan_threads(int64_t work);

// Stable sort of (key, index) by key descending; keys < 2^32.  Small key ranges (the strip
// costs of short pairs) take one counting pass, others two 16-bit LSD radix passes.
void sort_desc(std::vector<uint32_t> &keys, std::vector<int32_t> &idx)
{
    const size_t n = idx.size();
    if (n == 0) return;
    const uint32_t kmax = *std::max_element(keys.begin(), keys.end());
    const int nth = kmax < 65536 ? plan_threads(int64_t(n)) : 1;
    if (nth > 1) {
        // Per-thread histograms of contiguous chunks; bucket-major, thread-minor offsets keep
        // the sort stable.
        const size_t K = size_t(kmax) + 1;
        std::vector<uint32_t> hist(size_t(nth) * K, 0);
        std::vector<uint32_t> k2(n);
        std::vector<int32_t> i2(n);
#pragma omp parallel num_threads(nth)
        {
            const int t = omp_get_thread_num();
            const size_t a = n * t / nth, b = n * (t + 1) / nth;
            uint32_t *h = hist.data() + size_t(t) * K;
            for (size_t i = a; i < b; ++i) ++h[kmax - keys[i]];
#pragma omp barrier
#pragma omp single
            {
                uint32_t run = 0;
                for (size_t q = 0; q < K; ++q)
                    for (int u = 0; u < nth; ++u) {
                        const uint32_t c = hist[size_t(u) * K + q];
                        hist[size_t(u) * K + q] = run;
                        run += c;
                    }
            }
            for (size_t i = a; i < b; ++i) {
                const size_t d = h[kmax - keys[i]]++;
                k2[d] = keys[i];
                i2[d] = idx[i];
            }
        }
        keys.swap(k2);
        idx.swap(i2);
        return;
    }
    if (kmax < std::max<uint64_t>(65536, 4 * uint64_t(n))) {
        std::vector<uint32_t> cnt(size_t(kmax) + 2, 0);
        for (size_t i = 0; i < n; ++i) ++cnt[size_t(kmax - keys[i]) + 1];
        for (size_t i = 1; i < cnt.size(); ++i) cnt[i] += cnt[i - 1];
        std::vector<uint32_t> k2(n);
        std::vector<int32_t> i2(n);
        for (size_t i = 0; i < n; ++i) {
            const size_t d = cnt[kmax - keys[i]]++;
            k2[d] = keys[i];
            i2[d] = idx[i];
        }
        keys.swap(k2);
        idx.swap(i2);
        return;
    }
    std::vector<uint32_t> k2(n);
    std::vector<int32_t> i2(n);
    for (int pass = 0; pass < 2; ++pass) {
        const int shift = 16 * pass;
        std::vector<size_t> cnt(65537, 0);
        for (size_t i = 0; i < n; ++i) ++cnt[(0xffffu - ((keys[i] >> shift) & 0xffffu)) + 1];
        for (size_t i = 1; i < cnt.size(); ++i) cnt[i] += cnt[i - 1];
        for (size_t i = 0; i < n; ++i) {
            size_t d = cnt[0xffffu - ((keys[i] >> shift) & 0xffffu)]++;
            k2[d] = keys[i];
            i2[d] = idx[i];
        }
        keys.swap(k2);
        idx.swap(i2);
    }
}

template <typename T>
int upload(gba_context *ctx, DevBuf &buf, const std::vector<T> &v)
{
    GBA_CUDA(ctx, buf.ensure(v.size() * sizeof(T) + 16));
    if (!v.empty())
        GBA_CUDA(ctx, cudaMemcpyAsync(buf.ptr, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice,
                                      ctx->stream));
    return GBA_OK;
}

// Tiling variants of the packed kernel: rows per register strip x minimum resident blocks per
// SM (which caps registers per thread).  The autotuner times them on the real batch.
struct Variant16 {
    int rows, minb;
};
constexpr Variant16 kVariants16[] = {{32, 2}, {32, 3}, {24, 3}, {24, 4}, {16, 4}};
constexpr int kNumVariants16 = int(sizeof(kVariants16) / sizeof(kVariants16[0]));
static_assert(kNumVariants16 == GBA_TILE_VARIANTS, "tiling variants and the header disagree");

const void *dp16_fn(int v, bool affine)
{
#define GBA_V16(R, B) (affine ? (const void *)k_dp16x2<true, R, B> : (const void *)k_dp16x2<false, R, B>)
    switch (v) {
    case 0: return GBA_V16(32, 2);
    case 1: return GBA_V16(32, 3);
    case 2: return GBA_V16(24, 3);
    case 3: return GBA_V16(24, 4);
    default: return GBA_V16(16, 4);
    }
#undef GBA_V16
}

void launch_dp16(int v, bool affine, int grid, const Dp16Args &a, cudaStream_t st)
{
#define GBA_L16(R, B)                                                         \
    do {                                                                      \
        if (affine) k_dp16x2<true, R, B><<<grid, kBlock, 0, st>>>(a);         \
        else k_dp16x2<false, R, B><<<grid, kBlock, 0, st>>>(a);               \
    } while (0)
    switch (v) {
    case 0: GBA_L16(32, 2); break;
    case 1: GBA_L16(32, 3); break;
    case 2: GBA_L16(24, 3); break;
    case 3: GBA_L16(24, 4); break;
    default: GBA_L16(16, 4); break;
    }
#undef GBA_L16
}

// Resident blocks of a persistent kernel on this device (all SMs x blocks per SM); the
// occupancy queries are cached per context (they do not change).
int64_t persistent_grid(gba_context *ctx, const void *fn)
{
    auto it = ctx->grid_cache.find(fn);
    if (it != ctx->grid_cache.end()) return it->second;
    int sms = 0, per_sm = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, ctx->device);
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, kBlock, 0) != cudaSuccess || per_sm < 1)
        per_sm = 1;
    const int64_t g = int64_t(sms) * per_sm;
    ctx->grid_cache.emplace(fn, g);
    return g;
}

const void *warp_fn(bool a, bool l, bool m, bool t);
const void *warp2_fn(bool a, bool l, bool m, bool t);

// Host threads for a planning loop over `work` items: serial below 16,384 items.
int plan_threads(int64_t work)
{
    if (work < 16384) return 1;
    return int(std::max<int64_t>(1, std::min<int64_t>({int64_t(omp_get_max_threads()), 16, work / 4096})));
}

// Phase timer of build_plan: with GBA_PLAN_PROFILE set in the environment, each plan prints
// its phases' host milliseconds to stderr (diagnostics only).
struct PlanTimer {
    bool on = std::getenv("GBA_PLAN_PROFILE") != nullptr;
    std::chrono::steady_clock::time_point t0 = std::chrono::steady_clock::now(), last = t0;
    std::string line;
    void mark(const char *what)
    {
        if (!on) return;
        const auto now = std::chrono::steady_clock::now();
        char buf[64];
        std::snprintf(buf, sizeof(buf), " %s=%.3f", what, std::chrono::duration<double, std::milli>(now - last).count());
        line += buf;
        last = now;
    }
    ~PlanTimer()
    {
        if (on)
            std::fprintf(stderr, "[gba plan] total=%.3f ms:%s\n",
                         std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count(),
                         line.c_str());
    }
};

// Builds a plan from host offsets.  `plan` buffers are (re)used.
int build_plan(gba_context *ctx, const gba_params *p, const gba_batch *b, gba_plan *plan)
{
    PlanTimer timer;
    int rc = validate(ctx, p, b);
    if (rc) return rc;
    const int64_t N = b->num_pairs;
    plan->bind(ctx->stream);
    plan->params = *p;
    plan->num_pairs = N;
    plan->affine = is_affine(*p);
    plan->dynamic = p->gap_model == GBA_GAPS_DYNAMIC;
    plan->local = p->mode == GBA_LOCAL;
    plan->extend = p->mode == GBA_ALIGN_EXTEND;
    // AlignExtend_ has a free last row and column (align_extend/align_extend_base.h:75-81).
    plan->free_ends = plan->extend ? (GBA_FREE_RIGHT | GBA_FREE_BOTTOM) : p->free_ends;
    plan->traceback = (p->outputs & GBA_OUT_SEGMENTS) != 0;
    plan->cigar = (p->outputs & GBA_OUT_CIGAR) != 0;
    plan->matrix = p->matrix != nullptr;
    plan->matrix_host.clear();
    if (p->matrix) plan->matrix_host.assign(p->matrix, p->matrix + p->alphabet_size * p->alphabet_size);
    int max_pos = 0;
    max_sub_abs(*p, plan->matrix_host, &max_pos);

    plan->status.assign(N, GBA_PAIR_OK);
    // The packed 16-bit path: global score-only runs with equality scoring over an alphabet of
    // at most 8 codes (the caller's alphabet_size), table entries that fit a byte, and gaps that
    // keep int16 arithmetic exact (checked per pair below).
    const bool plain = (p->flags & GBA_FLAG_PLAIN_BUCKETS) != 0;
    const bool packed_ok = !plan->local && !plan->traceback && !plan->matrix && !p->band_on && !plan->dynamic &&
                           !(p->flags & GBA_FLAG_GENERAL_KERNEL) &&
                           (N >= kPackedMinPairs || (p->flags & (GBA_FLAG_STRIP16 | GBA_FLAG_PACKED))) &&
                           p->alphabet_size >= 1 &&
                           p->alphabet_size <= 8 && p->match >= -128 && p->match <= 127 &&
                           p->mismatch >= -128 && p->mismatch <= 127 && std::abs(p->gap_open) <= 1024 &&
                           std::abs(p->gap_extend) <= 1024;
    plan->rows16 = 32;
    // Pairs that are neither banded nor on the packed path run one warp per pair, unless the
    // one-pair-per-thread kernel is forced.
    plan->use_warp = !p->band_on && !(p->flags & GBA_FLAG_GENERAL_KERNEL) && !plan->dynamic;
    plan->warp_rows = 8;
    // The packed 16-bit warp path: 16-bit cells, a batch large enough to fill the GPU with one
    // warp per pair, equality scoring over at most 8 codes (PRMT lookup) or a table whose entries
    // fit int16, and gap scores small enough for the int16 range checks.
    bool w2_ok = plan->use_warp && p->score_bits == 16 && (N >= kW2MinPairs || (p->flags & GBA_FLAG_WARP16)) &&
                 !(p->flags & GBA_FLAG_NO_WARP16) &&
                 std::abs(p->gap_open) <= 1024 && std::abs(p->gap_extend) <= 1024;
    if (w2_ok && plan->matrix) {
        for (int32_t v : plan->matrix_host) w2_ok = w2_ok && v >= -1024 && v <= 1024;
    } else if (w2_ok) {
        w2_ok = p->alphabet_size >= 1 && p->alphabet_size <= 8 && p->match >= -128 && p->match <= 127 &&
                p->mismatch >= -128 && p->mismatch <= 127;
    }
    // Host arrays live in the plan and keep their capacity between builds (no zero fill).
    auto &keys16 = plan->h_keys16;
    auto &idx16 = plan->h_idx16;
    auto &keys2 = plan->h_keys2;
    auto &idx2 = plan->h_idx2;
    auto &desc = plan->h_desc;
    auto &keys = plan->h_keys;
    auto &idx = plan->h_idx;
    desc.resize(std::max<int64_t>(N, 1));
    plan->cells = 0;
    int64_t trace_off = 0;
    const int64_t hs0 = b->h_shared ? b->off_h[0] : 0;
    const int64_t hs1 = b->h_shared ? b->off_h[1] : 0;
    plan->seq_h_bytes = N ? (b->h_shared ? b->off_h[1] : b->off_h[N]) : 0;
    plan->seq_v_bytes = N ? b->off_v[N] : 0;
    // Per-pair pass, in parallel over contiguous chunks of pairs: descriptor, status, class
    // (packed path / other / invalid), sort key and trace bytes.  Then each chunk appends its
    // pairs to the class lists and assigns trace offsets at its prefix-summed position, so the
    // lists are in input order exactly as a serial pass makes them.
    timer.mark("setup");
    const int nth = plan_threads(N);
    auto &cls = plan->h_cls;
    auto &key = plan->h_key;
    cls.resize(N);
    key.resize(N);
    std::vector<int64_t> tbytes(plan->traceback ? N : 0);
    std::vector<int64_t> c16(nth + 1, 0), cot(nth + 1, 0), ctr(nth + 1, 0), cw2(nth + 1, 0);
    int64_t first_bad = N, cells = 0;
    double cells16 = 0;   // cells of the packed-path pairs
    const int fe_all = plan->local ? 15 : plan->free_ends;
#pragma omp parallel num_threads(nth) reduction(+ : cells, cells16) reduction(min : first_bad)
    {
        const int t = omp_get_thread_num();
        const int64_t k0 = N * t / nth, k1 = N * (t + 1) / nth;
        std::map<uint64_t, int64_t> band_cache;
        int64_t n16 = 0, not16 = 0, nw2 = 0, tsum = 0;
        for (int64_t k = k0; k < k1; ++k) {
            const int64_t h0 = b->h_shared ? hs0 : b->off_h[k];
            const int64_t h1 = b->h_shared ? hs1 : b->off_h[k + 1];
            const int64_t v0 = b->off_v[k], v1 = b->off_v[k + 1];
            PairDesc &d = desc[k];
            cls[k] = 0;
            if (h0 < 0 || v0 < 0 || h1 < h0 || v1 < v0 || h1 - h0 > (1 << 30) || v1 - v0 > (1 << 30)) {
                first_bad = std::min(first_bad, k);
                d.invalid = 1;
                continue;
            }
            d.h_off = h0;
            d.v_off = v0;
            d.m = int32_t(h1 - h0);
            d.n = int32_t(v1 - v0);
            d.trace_off = 0;
            d.invalid = 0;
            const bool exact16 = p->score_bits == 16 && int16_exact(*p, max_pos, d.m, d.n, plan->local);
            d.inf = exact16 ? -16384 : -(1 << 30);
            plan->status[k] = (p->score_bits == 16 && !exact16) ? GBA_PAIR_PROMOTED : GBA_PAIR_OK;
            if (d.m == 0 || d.n == 0 || (p->band_on && !band_valid(*p, d.m, d.n, fe_all))) {
                plan->status[k] = GBA_PAIR_INVALID;
                d.invalid = 1;
                continue;
            }
            if (p->band_on) {
                const uint64_t ck = (uint64_t(d.m) << 32) | uint32_t(d.n);
                auto it = band_cache.find(ck);
                if (it == band_cache.end())
                    it = band_cache.emplace(ck, band_cells(d.m, d.n, p->band_lower, p->band_upper)).first;
                cells += it->second;
            } else {
                cells += int64_t(d.m) * d.n;
            }
            // (packed_ok excludes local mode, so exact16 is the global-mode check here)
            if (packed_ok && (p->score_bits == 16 ? exact16 : int16_exact(*p, max_pos, d.m, d.n, false))) {
                const int64_t strips = (d.n + plan->rows16 - 1) / plan->rows16;
                key[k] = uint32_t(std::min<int64_t>(strips * (d.m + 1), 0xffffffffLL));
                cls[k] = 1;
                ++n16;
                cells16 += double(d.m) * d.n;
            } else if (w2_ok && exact16 && d.m < kPipelineMinCols && d.n <= kW2MaxRows) {
                const int64_t bands = (d.n + kW2BandRows - 1) / kW2BandRows;
                key[k] = uint32_t(std::min<int64_t>(bands * (d.m + 64), 0xffffffffLL));
                cls[k] = 3;
                ++nw2;
            } else {
                const int64_t strips = (d.n + STRIP_ROWS - 1) / STRIP_ROWS;
                key[k] = uint32_t(std::min<int64_t>(strips * (d.m + 1), 0xffffffffLL));
                cls[k] = 2;
                ++not16;
            }
            if (plan->traceback) {
                tbytes[k] = p->band_on ? int64_t(d.m + 1) * band_col_bytes(p->band_upper - p->band_lower + 1) / 32
                            : cls[k] == 3 ? warp2_trace_bytes(d.m, d.n)
                            : plan->use_warp ? warp_trace_bytes(d.m, d.n, plan->warp_rows)
                                             : trace_bytes(d.m, d.n);
                tsum += tbytes[k];
            }
        }
        c16[t + 1] = n16;
        cot[t + 1] = not16;
        cw2[t + 1] = nw2;
        ctr[t + 1] = tsum;
#pragma omp barrier
#pragma omp single
        for (int i = 0; i < nth; ++i) {
            c16[i + 1] += c16[i];
            cot[i + 1] += cot[i];
            cw2[i + 1] += cw2[i];
            ctr[i + 1] += ctr[i];
        }
#pragma omp single
        {
            keys16.resize(c16[nth]);
            idx16.resize(c16[nth]);
            keys.resize(cot[nth]);
            idx.resize(cot[nth]);
            keys2.resize(cw2[nth]);
            idx2.resize(cw2[nth]);
        }
        int64_t q16 = c16[t], qot = cot[t], qw2 = cw2[t], toff = ctr[t];
        for (int64_t k = k0; k < k1; ++k) {
            if (cls[k] == 1) {
                keys16[q16] = key[k];
                idx16[q16++] = int32_t(k);
            } else if (cls[k] == 2) {
                keys[qot] = key[k];
                idx[qot++] = int32_t(k);
            } else if (cls[k] == 3) {
                keys2[qw2] = key[k];
                idx2[qw2++] = int32_t(k);
            }
            if (plan->traceback && cls[k] != 0) {
                desc[k].trace_off = toff;
                toff += tbytes[k];
            }
        }
    }
    if (first_bad < N)
        return fail(ctx, GBA_EINVAL, "negative, decreasing or too long offsets at pair %lld", (long long)first_bad);
    plan->cells = cells;
    trace_off = ctr[nth];
    plan->trace_total = trace_off;
    timer.mark("pairs");
    plan->bucket_start.clear();
    plan->bucket_count.clear();
    if (plain) {
        // The plain GPU form: pairs grouped into 8-residue buckets of max(m, n), in input order
        // inside a bucket, one launch per bucket.  Buckets start on a warp boundary (padding
        // slots hold -1).
        std::vector<std::vector<int32_t>> buckets;
        for (int32_t k : idx) {
            const int b = std::max(desc[k].m, desc[k].n) / 8;
            if (b >= int(buckets.size())) buckets.resize(b + 1);
            buckets[b].push_back(k);
        }
        idx.clear();
        for (auto &bk : buckets) {
            if (bk.empty()) continue;
            plan->bucket_start.push_back(int64_t(idx.size()));
            plan->bucket_count.push_back(int64_t(bk.size()));
            idx.insert(idx.end(), bk.begin(), bk.end());
            while (idx.size() % 32) idx.push_back(-1);
        }
    } else {
        sort_desc(keys, idx);
    }
    plan->num_slots = int64_t(idx.size());
    // Banded traces are interleaved by lane within each warp of 32 slots (see band_trace_pos and
    // band4_pos): a warp's region holds (its largest m + 1) columns of band_col_bytes(W) bytes
    // for the 32 lanes, rounded up to 512 bytes so that a pair's lane is (trace_off >> 4) & 31.
    if (p->band_on && plan->traceback && plan->num_slots > 0) {
        const int CB = band_col_bytes(p->band_upper - p->band_lower + 1);
        const int64_t nw = (plan->num_slots + 31) / 32;
        std::vector<int64_t> wsize(nw + 1, 0);
#pragma omp parallel for num_threads(plan_threads(plan->num_slots)) schedule(static)
        for (int64_t w = 0; w < nw; ++w) {
            int maxm = -1;
            for (int64_t s = 32 * w; s < std::min(plan->num_slots, 32 * w + 32); ++s)
                if (idx[s] >= 0) maxm = std::max(maxm, desc[idx[s]].m);
            wsize[w + 1] = maxm < 0 ? 0 : (int64_t(maxm + 1) * CB + 511) / 512 * 512;
        }
        for (int64_t w = 0; w < nw; ++w) wsize[w + 1] += wsize[w];
#pragma omp parallel for num_threads(plan_threads(plan->num_slots)) schedule(static)
        for (int64_t s = 0; s < plan->num_slots; ++s)
            if (idx[s] >= 0) desc[idx[s]].trace_off = wsize[s / 32] + (s % 32) * 16;
        trace_off = wsize[nw];
        plan->trace_total = trace_off;
    }
    // Large pairs of the warp layout (a prefix of the cost-sorted order) get the warp-walked
    // traceback; the key is strips of STRIP_ROWS rows x (m + 1) columns.
    plan->num_tiled_tb = 0;
    if (plan->use_warp && plan->traceback && !(p->flags & GBA_FLAG_PLAIN_BUCKETS))
        while (plan->num_tiled_tb < int64_t(keys.size()) &&
               keys[plan->num_tiled_tb] >= uint32_t(kTiledTraceCells / STRIP_ROWS))
            ++plan->num_tiled_tb;

    // Packed path: neighbours in the length-sorted order share a thread; per warp, the code
    // words (4 residues per word, both pairs' codes per byte) and the boundary row are
    // interleaved by lane.
    if (!plain) sort_desc(keys16, idx16);
    timer.mark("sort");
    // Split slots: a thread holds two pairs, so its time is set by its larger pair; pairs whose
    // cells exceed the batch's average work per resident thread (the batch cannot finish before
    // its longest thread) run one per thread as a split slot, two strips at once.  They are a
    // prefix of the length-sorted order, rounded down to whole warps.
    int64_t nsplit = 0;
    if (!idx16.empty() && !plain && !(p->flags & GBA_FLAG_PACKED_NO_SPLIT)) {
        if (p->flags & GBA_FLAG_PACKED_SPLIT) {
            nsplit = int64_t(idx16.size());
        } else {
            const double resident = double(persistent_grid(ctx, dp16_fn(0, plan->affine))) * kBlock;
            // keys16 (descending) are strips of rows16 rows x (m + 1) columns: about a slot's
            // cells / rows16, so the split prefix ends at the first key below that threshold.
            const double per_thread = cells16 / 2 / resident;
            const uint32_t kthr = uint32_t(std::min<double>(per_thread / plan->rows16, 4e9));
            nsplit = int64_t(std::upper_bound(keys16.begin(), keys16.end(), kthr, std::greater<uint32_t>()) -
                             keys16.begin());
            nsplit -= nsplit % 32;
        }
    }
    const int64_t rest16 = int64_t(idx16.size()) - nsplit;
    auto &slots16 = plan->h_slots16;
    plan->b16_start.clear();
    plan->b16_count.clear();
    if (plain) {
        // Plain form: two pairs per slot inside each 8-residue bucket (input order), each
        // bucket's slots padded to whole warps (padding slots have pa = -1 and are never run).
        std::vector<std::vector<int32_t>> bk;
        for (int32_t k : idx16) {
            const int b = std::max(desc[k].m, desc[k].n) / 8;
            if (b >= int(bk.size())) bk.resize(b + 1);
            bk[b].push_back(k);
        }
        slots16.clear();
        for (auto &v : bk) {
            if (v.empty()) continue;
            const int64_t start = int64_t(slots16.size());
            for (size_t i = 0; i < v.size(); i += 2) {
                Slot16 sl{};
                sl.pa = v[i];
                sl.pb = i + 1 < v.size() ? v[i + 1] : -1;
                sl.split = 0;
                sl.m = desc[sl.pa].m;
                sl.n = desc[sl.pa].n;
                if (sl.pb >= 0) {
                    sl.m = std::max(sl.m, desc[sl.pb].m);
                    sl.n = std::max(sl.n, desc[sl.pb].n);
                }
                slots16.push_back(sl);
            }
            plan->b16_start.push_back(start);
            plan->b16_count.push_back(int64_t(slots16.size()) - start);
            while (slots16.size() % 32) slots16.push_back(Slot16{-1, -1, 0, 0, 0});
        }
    } else {
        slots16.resize(size_t(nsplit + (rest16 + 1) / 2));
    }
#pragma omp parallel for num_threads(plan_threads(int64_t(slots16.size()))) schedule(static)
    for (size_t q = 0; q < (plain ? size_t(0) : slots16.size()); ++q) {
        Slot16 &sl = slots16[q];
        if (int64_t(q) < nsplit) {
            sl.pa = idx16[q];
            sl.pb = -1;
            sl.m = desc[sl.pa].m + 1;   // steps: the high strip runs one column behind
            sl.n = desc[sl.pa].n;
            sl.split = 1;
            continue;
        }
        const size_t u = size_t(nsplit) + 2 * (q - size_t(nsplit));
        sl.pa = idx16[u];
        sl.pb = u + 1 < idx16.size() ? idx16[u + 1] : -1;
        sl.split = 0;
        sl.m = desc[sl.pa].m;
        sl.n = desc[sl.pa].n;
        if (sl.pb >= 0) {
            sl.m = std::max(sl.m, desc[sl.pb].m);
            sl.n = std::max(sl.n, desc[sl.pb].n);
        }
    }
    plan->num16 = int64_t(slots16.size());
    const int64_t warps16 = (plan->num16 + 31) / 32;
    std::vector<int64_t> wcodes(std::max<int64_t>(warps16, 1)), wbnd(std::max<int64_t>(warps16, 1));
    std::vector<int32_t> whw(std::max<int64_t>(warps16, 1));
    std::vector<int32_t> wmaxm(std::max<int64_t>(warps16, 1)), wmaxn(std::max<int64_t>(warps16, 1));
#pragma omp parallel for num_threads(plan_threads(warps16 * 32)) schedule(static)
    for (int64_t w = 0; w < warps16; ++w) {
        int maxm = 0, maxn = 0;
        for (int64_t q = w * 32; q < std::min(plan->num16, (w + 1) * 32); ++q) {
            maxm = std::max(maxm, slots16[q].m);
            maxn = std::max(maxn, slots16[q].n);
        }
        wmaxm[w] = maxm;
        wmaxn[w] = maxn;
    }
    int64_t ctot = 0, btot = 0;
    for (int64_t w = 0; w < warps16; ++w) {
        const int hw = (wmaxm[w] + 3) / 4, vw = (wmaxn[w] + 3) / 4;
        wcodes[w] = ctot;
        whw[w] = hw;
        ctot += int64_t(hw + vw) * 32;
        wbnd[w] = btot;
        btot += int64_t(wmaxm[w] + 1) * 32;
    }
    plan->codes_total = ctot;
    plan->bnd16_total = btot;
    plan->tasks16 = int32_t(warps16);
    timer.mark("slots16");

    // Warp path: tasks in the length-sorted pair order.  A pair's bands run as separate,
    // pipelined tasks (pair, b) when the pair is wide or the batch too small to fill the GPU
    // otherwise; else the pair is one task (pair, -1) whose warp runs its bands in order.  A
    // pair of more than one band gets two row slots of m + 1 int2; a pipelined one also a
    // BandState per band.
    std::vector<int64_t> rboff, bbase;
    std::vector<int2> wtasks;
    int64_t rbtot = 0, nstates = 0;
    if (plan->use_warp && !idx.empty()) {
        plan->grid_warp = persistent_grid(ctx, warp_fn(plan->affine, plan->local, plan->matrix, plan->traceback));
        const bool few_pairs = int64_t(idx.size()) < 2 * plan->grid_warp * (kBlock / 32);
        rboff.assign(N + 1, 0);
        bbase.assign(N + 1, 0);
        const int band_rows = 32 * plan->warp_rows;
        wtasks.reserve(idx.size());
        plan->wb_start.clear();
        plan->wb_count.clear();
        int last_bucket = -1;
        for (int32_t k : idx) {
            if (k < 0) continue;   // plain-form padding slot
            if (plain) {
                const int bucket = std::max(desc[k].m, desc[k].n) / 8;
                if (bucket != last_bucket) {
                    if (!plan->wb_start.empty()) plan->wb_count.back() = int64_t(wtasks.size()) - plan->wb_start.back();
                    plan->wb_start.push_back(int64_t(wtasks.size()));
                    plan->wb_count.push_back(0);
                    last_bucket = bucket;
                }
            }
            const int nb = (desc[k].n + band_rows - 1) / band_rows;
            const bool pipe = nb > 1 && (few_pairs || desc[k].m >= kPipelineMinCols);
            if (pipe) {
                for (int bb = 0; bb < nb; ++bb) wtasks.push_back(make_int2(k, bb));
                bbase[k] = nstates;
                nstates += nb;
            } else {
                wtasks.push_back(make_int2(k, nb > 1 ? -1 : 0));
            }
            if (nb > 1) {
                rboff[k] = rbtot;
                rbtot += 2 * (int64_t(desc[k].m) + 1);
            }
        }
        if (!plan->wb_start.empty()) plan->wb_count.back() = int64_t(wtasks.size()) - plan->wb_start.back();
    }
    plan->num_warp_tasks = int64_t(wtasks.size());
    plan->num_band_states = nstates;

    // Packed 16-bit warp path: one task per pair, costliest first (plain form: 8-residue buckets
    // of max(m, n) in input order); a pair of more than one band gets a row buffer of m + 1 words.
    plan->w2b_start.clear();
    plan->w2b_count.clear();
    if (plain && !idx2.empty()) {
        std::vector<std::vector<int32_t>> bk;
        for (int32_t k : idx2) {
            const int bb = std::max(desc[k].m, desc[k].n) / 8;
            if (bb >= int(bk.size())) bk.resize(bb + 1);
            bk[bb].push_back(k);
        }
        idx2.clear();
        for (auto &v : bk) {
            if (v.empty()) continue;
            plan->w2b_start.push_back(int64_t(idx2.size()));
            plan->w2b_count.push_back(int64_t(v.size()));
            idx2.insert(idx2.end(), v.begin(), v.end());
        }
    } else {
        sort_desc(keys2, idx2);
    }
    plan->num_w2 = int64_t(idx2.size());
    // Tasks: (pair, -1) runs the pair's bands in order on one warp; a pair of at least
    // kW2PipeBands bands, or of two or more in a batch too small to keep the GPU busy otherwise,
    // becomes one task per band, pipelined across warps.  Row buffers: one slot of m + 1 words for
    // in-order pairs, two for pipelined ones; pipelined bands get a BandState each.
    std::vector<int64_t> rb2off, bs2base;
    std::vector<int2> &w2tasks = plan->h_w2tasks;
    w2tasks.clear();
    int64_t rb2tot = 0, ns2 = 0;
    if (plan->num_w2 > 0) {
        plan->grid_w2 = persistent_grid(ctx, warp2_fn(plan->affine, plan->local, plan->matrix, plan->traceback));
        const bool few = plan->num_w2 < 2 * plan->grid_w2 * (kBlock / 32);
        rb2off.assign(N + 1, 0);
        bs2base.assign(N + 1, 0);
        std::vector<int64_t> bstart(plan->w2b_start.size() + 1, 0);
        size_t bk = 0;
        for (int64_t q = 0; q < plan->num_w2; ++q) {
            if (!plan->w2b_start.empty()) {
                while (bk < plan->w2b_start.size() && plan->w2b_start[bk] + plan->w2b_count[bk] <= q) ++bk;
                if (q == plan->w2b_start[bk]) bstart[bk] = int64_t(w2tasks.size());
            }
            const int32_t k = idx2[q];
            const int nb = (desc[k].n + kW2BandRows - 1) / kW2BandRows;
            const bool pipe = nb >= kW2PipeBands || (nb > 1 && few);
            if (pipe) {
                for (int bb = 0; bb < nb; ++bb) w2tasks.push_back(make_int2(k, bb));
                bs2base[k] = ns2;
                ns2 += nb;
            } else {
                w2tasks.push_back(make_int2(k, -1));
            }
            if (nb > 1) {
                rb2off[k] = rb2tot;
                rb2tot += (pipe ? 2 : 1) * (int64_t(desc[k].m) + 1);
            }
        }
        // Plain form: task ranges per bucket.
        if (!plan->w2b_start.empty()) {
            bstart[plan->w2b_start.size()] = int64_t(w2tasks.size());
            for (size_t i = 0; i < plan->w2b_start.size(); ++i) {
                plan->w2b_start[i] = bstart[i];
                plan->w2b_count[i] = bstart[i + 1] - bstart[i];
            }
        }
    }
    plan->num_w2_tasks = int64_t(w2tasks.size());
    plan->num_w2_states = ns2;
    // Per-warp interleaved boundary rows: warp w holds 32 lanes x (max m + 1) int2.
    // (only the one-pair-per-thread strip kernel uses these boundary rows)
    const int64_t warps = (plan->use_warp || p->band_on) ? 0 : (plan->num_slots + 31) / 32;
    std::vector<int64_t> wscr(std::max<int64_t>(warps, 1));
    int64_t scr = 0;
    for (int64_t w = 0; w < warps; ++w) {
        int maxm = 0;
        for (int64_t s = w * 32; s < std::min(plan->num_slots, (w + 1) * 32); ++s)
            if (idx[s] >= 0) maxm = std::max(maxm, desc[idx[s]].m);
        wscr[w] = scr;
        scr += int64_t(maxm + 1) * 32;
    }
    plan->scratch_total = scr;

    timer.mark("warp+strip");
    // Segment / CIGAR slots: at most m + n + 4 records per pair.
    std::vector<int64_t> seg_off(plan->traceback ? N + 1 : 0, 0), cig_off;
    plan->seg_slots_total = 0;
    plan->cigar_slots_total = 0;
    if (plan->traceback) {
        for (int64_t k = 0; k < N; ++k) {
            const int64_t cap = plan->status[k] == GBA_PAIR_INVALID ? 0 : int64_t(desc[k].m) + desc[k].n + 4;
            seg_off[k + 1] = seg_off[k] + cap;
        }
        plan->seg_slots_total = seg_off[N];
        plan->seg_off_host = seg_off;
        if (plan->cigar) {
            cig_off = seg_off;
            plan->cigar_slots_total = seg_off[N];
        }
    }

    // HBM budget: everything this plan keeps on the device plus the input codes.
    const int64_t need = int64_t(sizeof(PairDesc)) * N + 4 * N * 8 + scr * 8 + plan->trace_total +
                         plan->codes_total * 4 + plan->bnd16_total * 8 + plan->num16 * int64_t(sizeof(Slot16)) +
                         plan->seg_slots_total * 16 * 2 + plan->cigar_slots_total * 4 * 2 +
                         plan->seq_h_bytes + plan->seq_v_bytes + rbtot * 8 + nstates * int64_t(sizeof(BandState)) +
                         plan->num_warp_tasks * 8 + rb2tot * 4 + plan->num_w2 * 12 + plan->num_w2_tasks * 8 +
                         ns2 * int64_t(sizeof(BandState));
    if (ctx->budget > 0 && need > ctx->budget)
        return fail(ctx, GBA_EBUDGET, "batch needs %lld bytes of HBM, budget is %lld", (long long)need,
                    (long long)ctx->budget);

    timer.mark("layout");
    if ((rc = upload(ctx, plan->pairs, desc))) return rc;
    if ((rc = upload(ctx, plan->order, idx))) return rc;
    if ((rc = upload(ctx, plan->warp_scratch, wscr))) return rc;
    GBA_CUDA(ctx, plan->scratch.ensure(size_t(std::max<int64_t>(scr, 1)) * sizeof(int2)));
    if (plan->use_warp && plan->num_slots > 0) {
        if ((rc = upload(ctx, plan->rowbuf_off, rboff))) return rc;
        if ((rc = upload(ctx, plan->band_base, bbase))) return rc;
        if ((rc = upload(ctx, plan->tasks_warp, wtasks))) return rc;
        GBA_CUDA(ctx, plan->rowbuf.ensure(size_t(std::max<int64_t>(rbtot, 1)) * sizeof(int2)));
        GBA_CUDA(ctx, plan->band_state.ensure(size_t(std::max<int64_t>(nstates, 1)) * sizeof(BandState)));
        GBA_CUDA(ctx, ctx->err_word.ensure(kMaxChunks * sizeof(int32_t)));
        GBA_CUDA(ctx, plan->counter_warp.ensure(std::max<size_t>(16, plan->wb_start.size() * sizeof(int32_t))));
    }
    if (plan->num_w2 > 0) {
        if ((rc = upload(ctx, plan->tasks_w2, w2tasks))) return rc;
        if ((rc = upload(ctx, plan->order_w2, idx2))) return rc;
        if ((rc = upload(ctx, plan->rowbuf_w2_off, rb2off))) return rc;
        if ((rc = upload(ctx, plan->band_w2_base, bs2base))) return rc;
        GBA_CUDA(ctx, plan->rowbuf_w2.ensure(size_t(std::max<int64_t>(rb2tot, 1)) * sizeof(uint32_t)));
        GBA_CUDA(ctx, plan->band_w2.ensure(size_t(std::max<int64_t>(ns2, 1)) * sizeof(BandState)));
        GBA_CUDA(ctx, plan->counter_w2.ensure(std::max<size_t>(16, plan->w2b_start.size() * sizeof(int32_t))));
        GBA_CUDA(ctx, ctx->err_word.ensure(kMaxChunks * sizeof(int32_t)));
    }
    if (plan->num16 > 0) {
        if ((rc = upload(ctx, plan->slots16, slots16))) return rc;
        if ((rc = upload(ctx, plan->warp_codes, wcodes))) return rc;
        if ((rc = upload(ctx, plan->warp_hwords, whw))) return rc;
        if ((rc = upload(ctx, plan->warp_bnd16, wbnd))) return rc;
        GBA_CUDA(ctx, plan->codes16.ensure(size_t(std::max<int64_t>(ctot, 1)) * 4));
        GBA_CUDA(ctx, plan->bnd16.ensure(size_t(std::max<int64_t>(btot, 1)) * sizeof(int2)));
        GBA_CUDA(ctx, plan->counter16.ensure(std::max<size_t>(16, plan->b16_start.size() * sizeof(int32_t))));
        for (int v = 0; v < kNumVariants16; ++v) plan->grid16[v] = persistent_grid(ctx, dp16_fn(v, plan->affine));
        // Variant: forced by flags, else the context's tuning table for this batch shape, else
        // the default; GBA_FLAG_AUTOTUNE times all variants at the first run.
        int64_t summ = 0, sumn = 0;
        for (const Slot16 &sl : slots16) { summ += sl.m; sumn += sl.n; }
        const int64_t mm = summ / plan->num16, mn = sumn / plan->num16;
        plan->tune_key = (int64_t(plan->affine) << 40) | ((mm / 32) << 20) | (mn / 32);
        plan->variant16 = 0;
        plan->tune_pending = false;
        if (p->tile_variant >= 1 && p->tile_variant <= kNumVariants16) {
            plan->variant16 = p->tile_variant - 1;
        } else if (p->flags & GBA_FLAG_STRIP16) {
            plan->variant16 = kNumVariants16 - 1;
        } else if (plain) {
            plan->variant16 = 0;
        } else {
            auto it = ctx->tuning.find(plan->tune_key);
            if (it != ctx->tuning.end()) plan->variant16 = it->second;
            else if (p->flags & GBA_FLAG_AUTOTUNE) plan->tune_pending = true;
        }
    }
    plan->drop_graph();
    if (plan->matrix) {
        if ((rc = upload(ctx, plan->matrix_dev, plan->matrix_host))) return rc;
    }
    GBA_CUDA(ctx, plan->end_h.ensure(size_t(N + 1) * 4));
    GBA_CUDA(ctx, plan->end_v.ensure(size_t(N + 1) * 4));
    GBA_CUDA(ctx, plan->score_tmp.ensure(size_t(N + 1) * 4));
    if (plan->traceback) {
        GBA_CUDA(ctx, plan->trace.ensure(size_t(std::max<int64_t>(plan->trace_total, 16))));
        GBA_CUDA(ctx, plan->best_e.ensure(size_t(N + 1) * 4));
        GBA_CUDA(ctx, plan->best_f.ensure(size_t(N + 1) * 4));
        GBA_CUDA(ctx, plan->begin_h.ensure(size_t(N + 1) * 4));
        GBA_CUDA(ctx, plan->begin_v.ensure(size_t(N + 1) * 4));
        if ((rc = upload(ctx, plan->seg_slot_off, seg_off))) return rc;
        GBA_CUDA(ctx, plan->seg_slots.ensure(size_t(std::max<int64_t>(plan->seg_slots_total, 1)) * 16));
        GBA_CUDA(ctx, plan->seg_count.ensure(size_t(N + 1) * 4));
        GBA_CUDA(ctx, plan->seg_count64.ensure(size_t(N + 1) * 8));
        GBA_CUDA(ctx, plan->seg_dense_off.ensure(size_t(N + 1) * 8));
        GBA_CUDA(ctx, plan->seg_dense.ensure(size_t(std::max<int64_t>(plan->seg_slots_total, 1)) * 16));
        if (plan->cigar) {
            if ((rc = upload(ctx, plan->cig_slot_off, cig_off))) return rc;
            GBA_CUDA(ctx, plan->cig_slots.ensure(size_t(std::max<int64_t>(plan->cigar_slots_total, 1)) * 4));
            GBA_CUDA(ctx, plan->cig_count.ensure(size_t(N + 1) * 4));
            GBA_CUDA(ctx, plan->cig_count64.ensure(size_t(N + 1) * 8));
            GBA_CUDA(ctx, plan->cig_dense_off.ensure(size_t(N + 1) * 8));
            GBA_CUDA(ctx, plan->cig_dense.ensure(size_t(std::max<int64_t>(plan->cigar_slots_total, 1)) * 4));
        }
        size_t tmp = 0;
        cub::DeviceScan::ExclusiveSum(nullptr, tmp, (int64_t *)nullptr, (int64_t *)nullptr, int(N + 1));
        plan->cub_tmp_bytes = tmp;
        GBA_CUDA(ctx, plan->cub_tmp.ensure(tmp + 16));
    }
    plan->seg_dense_total = -1;
    plan->cig_dense_total = -1;
    timer.mark("upload+alloc");
    return GBA_OK;
}

template <bool A, bool L, bool M, bool T>
void launch_dp(const DpArgs &args, int grid, size_t smem, cudaStream_t s)
{
    k_dp_strip<A, L, M, T><<<grid, kBlock, smem, s>>>(args);
}

using DpLauncher = void (*)(const DpArgs &, int, size_t, cudaStream_t);


constexpr int kWarpRows = 8;
template <bool A, bool L, bool M, bool T>
void launch_warp(const WarpArgs &args, int grid, size_t smem, cudaStream_t s)
{
    k_dp_warp<A, L, M, T, kWarpRows><<<grid, kBlock, smem, s>>>(args);
}
using WarpLauncher = void (*)(const WarpArgs &, int, size_t, cudaStream_t);

WarpLauncher pick_warp(bool a, bool l, bool m, bool t)
{
    static const WarpLauncher table[16] = {
        launch_warp<false, false, false, false>, launch_warp<false, false, false, true>,
        launch_warp<false, false, true, false>,  launch_warp<false, false, true, true>,
        launch_warp<false, true, false, false>,  launch_warp<false, true, false, true>,
        launch_warp<false, true, true, false>,   launch_warp<false, true, true, true>,
        launch_warp<true, false, false, false>,  launch_warp<true, false, false, true>,
        launch_warp<true, false, true, false>,   launch_warp<true, false, true, true>,
        launch_warp<true, true, false, false>,   launch_warp<true, true, false, true>,
        launch_warp<true, true, true, false>,    launch_warp<true, true, true, true>};
    return table[(a ? 8 : 0) | (l ? 4 : 0) | (m ? 2 : 0) | (t ? 1 : 0)];
}

template <bool A, bool L, bool M, bool T>
void launch_warp2(const Warp2Args &args, int grid, cudaStream_t s)
{
    k_dp_warp2<A, L, M, T><<<grid, kBlock, 0, s>>>(args);
}
using Warp2Launcher = void (*)(const Warp2Args &, int, cudaStream_t);

Warp2Launcher pick_warp2(bool a, bool l, bool m, bool t)
{
    static const Warp2Launcher table[16] = {
        launch_warp2<false, false, false, false>, launch_warp2<false, false, false, true>,
        launch_warp2<false, false, true, false>,  launch_warp2<false, false, true, true>,
        launch_warp2<false, true, false, false>,  launch_warp2<false, true, false, true>,
        launch_warp2<false, true, true, false>,   launch_warp2<false, true, true, true>,
        launch_warp2<true, false, false, false>,  launch_warp2<true, false, false, true>,
        launch_warp2<true, false, true, false>,   launch_warp2<true, false, true, true>,
        launch_warp2<true, true, false, false>,   launch_warp2<true, true, false, true>,
        launch_warp2<true, true, true, false>,    launch_warp2<true, true, true, true>};
    return table[(a ? 8 : 0) | (l ? 4 : 0) | (m ? 2 : 0) | (t ? 1 : 0)];
}

const void *warp2_fn(bool a, bool l, bool m, bool t)
{
#define GBA_W2F(A, L, M, T) (const void *)k_dp_warp2<A, L, M, T>
    const void *table[16] = {GBA_W2F(false, false, false, false), GBA_W2F(false, false, false, true),
                             GBA_W2F(false, false, true, false),  GBA_W2F(false, false, true, true),
                             GBA_W2F(false, true, false, false),  GBA_W2F(false, true, false, true),
                             GBA_W2F(false, true, true, false),   GBA_W2F(false, true, true, true),
                             GBA_W2F(true, false, false, false),  GBA_W2F(true, false, false, true),
                             GBA_W2F(true, false, true, false),   GBA_W2F(true, false, true, true),
                             GBA_W2F(true, true, false, false),   GBA_W2F(true, true, false, true),
                             GBA_W2F(true, true, true, false),    GBA_W2F(true, true, true, true)};
#undef GBA_W2F
    return table[(a ? 8 : 0) | (l ? 4 : 0) | (m ? 2 : 0) | (t ? 1 : 0)];
}

const void *warp_fn(bool a, bool l, bool m, bool t)
{
#define GBA_WF(A, L, M, T) (const void *)k_dp_warp<A, L, M, T, kWarpRows>
    const void *table[16] = {GBA_WF(false, false, false, false), GBA_WF(false, false, false, true),
                             GBA_WF(false, false, true, false),  GBA_WF(false, false, true, true),
                             GBA_WF(false, true, false, false),  GBA_WF(false, true, false, true),
                             GBA_WF(false, true, true, false),   GBA_WF(false, true, true, true),
                             GBA_WF(true, false, false, false),  GBA_WF(true, false, false, true),
                             GBA_WF(true, false, true, false),   GBA_WF(true, false, true, true),
                             GBA_WF(true, true, false, false),   GBA_WF(true, true, false, true),
                             GBA_WF(true, true, true, false),    GBA_WF(true, true, true, true)};
#undef GBA_WF
    return table[(a ? 8 : 0) | (l ? 4 : 0) | (m ? 2 : 0) | (t ? 1 : 0)];
}

DpLauncher pick_dp(bool a, bool l, bool m, bool t)
{
    static const DpLauncher table[16] = {
        launch_dp<false, false, false, false>, launch_dp<false, false, false, true>,
        launch_dp<false, false, true, false>,  launch_dp<false, false, true, true>,
        launch_dp<false, true, false, false>,  launch_dp<false, true, false, true>,
        launch_dp<false, true, true, false>,   launch_dp<false, true, true, true>,
        launch_dp<true, false, false, false>,  launch_dp<true, false, false, true>,
        launch_dp<true, false, true, false>,   launch_dp<true, false, true, true>,
        launch_dp<true, true, false, false>,   launch_dp<true, true, false, true>,
        launch_dp<true, true, true, false>,    launch_dp<true, true, true, true>};
    return table[(a ? 8 : 0) | (l ? 4 : 0) | (m ? 2 : 0) | (t ? 1 : 0)];
}

template <bool L, bool M, bool T>
void launch_dynamic(const DpArgs &args, int grid, size_t smem, cudaStream_t s)
{
    k_dp_dynamic<L, M, T><<<grid, kBlock, smem, s>>>(args);
}

DpLauncher pick_dynamic(bool l, bool m, bool t)
{
    static const DpLauncher table[8] = {launch_dynamic<false, false, false>, launch_dynamic<false, false, true>,
                                        launch_dynamic<false, true, false>,  launch_dynamic<false, true, true>,
                                        launch_dynamic<true, false, false>,  launch_dynamic<true, false, true>,
                                        launch_dynamic<true, true, false>,   launch_dynamic<true, true, true>};
    return table[(l ? 4 : 0) | (m ? 2 : 0) | (t ? 1 : 0)];
}

__global__ void k_widen(const int32_t *src, int64_t *dst, int64_t n)
{
    int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i < n) dst[i] = src[i];
    if (i == n) dst[i] = 0;
}

// Invalid pairs: numeric_limits<T>::min() and an empty alignment
// (align/dp_algorithm_impl.h:1399-1400).
__global__ void k_fill_invalid(const PairDesc *pairs, int64_t n, int32_t minval, int32_t *score,
                               int32_t *end_h, int32_t *end_v, int32_t *begin_h, int32_t *begin_v,
                               int32_t *seg_count, int32_t *cig_count)
{
    int64_t k = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (k >= n) return;
    if (!pairs[k].invalid) return;
    score[k] = minval;
    if (end_h) end_h[k] = 0;
    if (end_v) end_v[k] = 0;
    if (begin_h) begin_h[k] = 0;
    if (begin_v) begin_v[k] = 0;
    if (seg_count) seg_count[k] = 0;
    if (cig_count) cig_count[k] = 0;
}

// Enqueues the kernels of a plan on device inputs.  Scores/end positions go to the given
// device pointers; segments and CIGARs stay in the plan's device buffers.
int enqueue_plan(gba_context *ctx, gba_plan *plan, const uint8_t *dseq_h, const uint8_t *dseq_v,
                 int32_t *dscore, int32_t *dend_h, int32_t *dend_v, bool capturing)
{
    // Inside a capture the timing events must be graph nodes (external records).
    const unsigned evflags = capturing ? cudaEventRecordExternal : cudaEventRecordDefault;
    const int64_t N = plan->num_pairs;
    int32_t *end_h = dend_h ? dend_h : plan->end_h.as<int32_t>();
    int32_t *end_v = dend_v ? dend_v : plan->end_v.as<int32_t>();
    const int32_t minval = plan->params.score_bits == 16 ? -32768 : INT32_MIN;
    int launches = 0;

    // The error word of this plan's bounded waits between bands (both warp kernels).
    if ((plan->use_warp && plan->num_band_states > 0) || plan->num_w2_states > 0)
        GBA_CUDA(ctx, cudaMemsetAsync(ctx->err_word.as<int32_t>() + plan->err_slot, 0, sizeof(int32_t), ctx->stream));
    GBA_CUDA(ctx, cudaEventRecordWithFlags(ctx->ev[0], ctx->stream, evflags));
    if (plan->num16 > 0) {
        Dp16Args a{};
        a.seq_h = dseq_h;
        a.seq_v = dseq_v;
        a.pairs = plan->pairs.as<PairDesc>();
        a.slots = plan->slots16.as<Slot16>();
        a.warp_codes = plan->warp_codes.as<int64_t>();
        a.warp_hwords = plan->warp_hwords.as<int32_t>();
        a.codes = plan->codes16.as<uint32_t>();
        a.warp_bnd = plan->warp_bnd16.as<int64_t>();
        a.bnd = plan->bnd16.as<int2>();
        a.score = dscore;
        a.end_h = end_h;
        a.end_v = end_v;
        a.num_slots = plan->num16;
        a.match = plan->params.match;
        a.mismatch = plan->params.mismatch;
        a.gap_open = plan->params.gap_open;
        a.gap_extend = plan->params.gap_extend;
        a.free_ends = plan->free_ends;
        a.num_tasks = plan->tasks16;
        a.task_counter = plan->counter16.as<int32_t>();
        a.rows = kVariants16[plan->variant16].rows;
        const size_t nb16 = plan->b16_start.size();
        GBA_CUDA(ctx, cudaMemsetAsync(plan->counter16.ptr, 0, sizeof(int32_t) * std::max<size_t>(nb16, 1),
                                      ctx->stream));
        k_pack16<<<int((plan->num16 + kBlock - 1) / kBlock), kBlock, 0, ctx->stream>>>(a);
        ++launches;
        if (nb16 == 0) {
            const int grid = int(std::min<int64_t>(plan->grid16[plan->variant16],
                                                    (int64_t(plan->tasks16) * 32 + kBlock - 1) / kBlock));
            launch_dp16(plan->variant16, plan->affine, grid, a, ctx->stream);
            ++launches;
        } else {
            // Plain form: one launch per length bucket (its slots start on a warp boundary).
            for (size_t b = 0; b < nb16; ++b) {
                Dp16Args ab = a;
                const int64_t w0 = plan->b16_start[b] / 32;
                ab.slots = a.slots + plan->b16_start[b];
                ab.warp_codes = a.warp_codes + w0;
                ab.warp_hwords = a.warp_hwords + w0;
                ab.warp_bnd = a.warp_bnd + w0;
                ab.num_slots = plan->b16_count[b];
                ab.num_tasks = int32_t((plan->b16_count[b] + 31) / 32);
                ab.task_counter = a.task_counter + b;
                const int grid = int(std::min<int64_t>(plan->grid16[plan->variant16],
                                                        (int64_t(ab.num_tasks) * 32 + kBlock - 1) / kBlock));
                launch_dp16(plan->variant16, plan->affine, grid, ab, ctx->stream);
                ++launches;
            }
        }
        GBA_CUDA(ctx, cudaGetLastError());
    }
    if (plan->num_w2 > 0) {
        Warp2Args w{};
        w.seq_h = dseq_h;
        w.seq_v = dseq_v;
        w.pairs = plan->pairs.as<PairDesc>();
        w.tasks = plan->tasks_w2.as<int2>();
        w.rowbuf = plan->rowbuf_w2.as<uint32_t>();
        w.rowbuf_off = plan->rowbuf_w2_off.as<int64_t>();
        w.bands = plan->band_w2.as<BandState>();
        w.band_base = plan->band_w2_base.as<int64_t>();
        w.error = ctx->err_word.as<int32_t>() + plan->err_slot;
        w.trace = plan->traceback ? plan->trace.as<uint8_t>() : nullptr;
        w.score = dscore;
        w.end_h = end_h;
        w.end_v = end_v;
        w.best_e = plan->traceback ? plan->best_e.as<int32_t>() : nullptr;
        w.best_f = plan->traceback ? plan->best_f.as<int32_t>() : nullptr;
        w.matrix = plan->matrix ? plan->matrix_dev.as<int32_t>() : nullptr;
        w.task_counter = plan->counter_w2.as<int32_t>();
        w.num_tasks = int32_t(plan->num_w2_tasks);
        w.match = plan->params.match;
        w.mismatch = plan->params.mismatch;
        w.gap_open = plan->params.gap_open;
        w.gap_extend = plan->params.gap_extend;
        w.free_ends = plan->free_ends;
        w.alphabet = plan->matrix ? plan->params.alphabet_size : 0;
        const size_t nb2 = plan->w2b_start.size();
        GBA_CUDA(ctx, cudaMemsetAsync(plan->counter_w2.ptr, 0, sizeof(int32_t) * std::max<size_t>(nb2, 1), ctx->stream));
        if (plan->num_w2_states > 0)
            GBA_CUDA(ctx, cudaMemsetAsync(plan->band_w2.ptr, 0, plan->num_w2_states * sizeof(BandState), ctx->stream));
        const Warp2Launcher wl = pick_warp2(plan->affine, plan->local, plan->matrix, plan->traceback);
        if (nb2 == 0) {
            wl(w, int(std::min<int64_t>(plan->grid_w2, (plan->num_w2_tasks * 32 + kBlock - 1) / kBlock)), ctx->stream);
            ++launches;
        } else {
            // Plain form: one launch per length bucket.
            for (size_t b = 0; b < nb2; ++b) {
                Warp2Args wb = w;
                wb.tasks = w.tasks + plan->w2b_start[b];
                wb.num_tasks = int32_t(plan->w2b_count[b]);
                wb.task_counter = w.task_counter + b;
                wl(wb, int(std::min<int64_t>(plan->grid_w2, (plan->w2b_count[b] * 32 + kBlock - 1) / kBlock)),
                   ctx->stream);
                ++launches;
            }
        }
        GBA_CUDA(ctx, cudaGetLastError());
    }
    if (plan->num_slots > 0 && plan->params.band_on) {
        BandArgs b{};
        b.seq_h = dseq_h;
        b.seq_v = dseq_v;
        b.pairs = plan->pairs.as<PairDesc>();
        b.order = plan->order.as<int32_t>();
        b.trace = plan->traceback ? plan->trace.as<uint8_t>() : nullptr;
        b.score = dscore;
        b.end_h = end_h;
        b.end_v = end_v;
        b.best_e = plan->traceback ? plan->best_e.as<int32_t>() : nullptr;
        b.best_f = plan->traceback ? plan->best_f.as<int32_t>() : nullptr;
        b.matrix = plan->matrix ? plan->matrix_dev.as<int32_t>() : nullptr;
        b.num_slots = plan->num_slots;
        b.match = plan->params.match;
        b.mismatch = plan->params.mismatch;
        b.gap_open = plan->params.gap_open;
        b.gap_extend = plan->params.gap_extend;
        b.free_ends = plan->free_ends;
        b.alphabet = plan->matrix ? plan->params.alphabet_size : 0;
        b.lower = plan->params.band_lower;
        b.upper = plan->params.band_upper;
        b.xdrop_on = plan->extend && (plan->params.flags & GBA_FLAG_XDROP) ? 1 : 0;
        b.xdrop = plan->params.xdrop;
        const int grid = int((plan->num_slots + kBlock - 1) / kBlock);
        const size_t smem = plan->matrix ? size_t(32 * 32) * sizeof(int) : 0;
        if (plan->extend)
            pick_banded_ext(plan->affine, plan->matrix, plan->traceback)(b, grid, smem, ctx->stream);
        else
            pick_banded(plan->affine, plan->local, plan->matrix, plan->traceback)(b, grid, smem, ctx->stream);
        GBA_CUDA(ctx, cudaGetLastError());
        ++launches;
    } else if (plan->num_slots > 0 && plan->use_warp) {
        WarpArgs w{};
        w.seq_h = dseq_h;
        w.seq_v = dseq_v;
        w.pairs = plan->pairs.as<PairDesc>();
        w.tasks = plan->tasks_warp.as<int2>();
        w.rowbuf = plan->rowbuf.as<int2>();
        w.rowbuf_off = plan->rowbuf_off.as<int64_t>();
        w.bands = plan->band_state.as<BandState>();
        w.band_base = plan->band_base.as<int64_t>();
        w.error = ctx->err_word.as<int32_t>() + plan->err_slot;
        w.trace = plan->traceback ? plan->trace.as<uint8_t>() : nullptr;
        w.score = dscore;
        w.end_h = end_h;
        w.end_v = end_v;
        w.best_e = plan->traceback ? plan->best_e.as<int32_t>() : nullptr;
        w.best_f = plan->traceback ? plan->best_f.as<int32_t>() : nullptr;
        w.matrix = plan->matrix ? plan->matrix_dev.as<int32_t>() : nullptr;
        w.task_counter = plan->counter_warp.as<int32_t>();
        w.num_tasks = int32_t(plan->num_warp_tasks);
        w.match = plan->params.match;
        w.mismatch = plan->params.mismatch;
        w.gap_open = plan->params.gap_open;
        w.gap_extend = plan->params.gap_extend;
        w.free_ends = plan->free_ends;
        w.alphabet = plan->matrix ? plan->params.alphabet_size : 0;
        const size_t nbw = plan->wb_start.size();
        GBA_CUDA(ctx, cudaMemsetAsync(plan->counter_warp.ptr, 0, sizeof(int32_t) * std::max<size_t>(nbw, 1),
                                      ctx->stream));
        if (plan->num_band_states > 0)
            GBA_CUDA(ctx, cudaMemsetAsync(plan->band_state.ptr, 0, plan->num_band_states * sizeof(BandState),
                                          ctx->stream));
        const size_t smem = plan->matrix ? size_t(32 * 32) * sizeof(int) : 0;
        const WarpLauncher wl = pick_warp(plan->affine, plan->local, plan->matrix, plan->traceback);
        if (nbw == 0) {
            const int grid =
                int(std::min<int64_t>(plan->grid_warp, (plan->num_warp_tasks * 32 + kBlock - 1) / kBlock));
            wl(w, grid, smem, ctx->stream);
            ++launches;
        } else {
            // Plain form: one launch per length bucket over that bucket's tasks.
            for (size_t b = 0; b < nbw; ++b) {
                WarpArgs wb = w;
                wb.tasks = w.tasks + plan->wb_start[b];
                wb.num_tasks = int32_t(plan->wb_count[b]);
                wb.task_counter = w.task_counter + b;
                const int grid =
                    int(std::min<int64_t>(plan->grid_warp, (plan->wb_count[b] * 32 + kBlock - 1) / kBlock));
                wl(wb, grid, smem, ctx->stream);
                ++launches;
            }
        }
        GBA_CUDA(ctx, cudaGetLastError());
    } else if (plan->num_slots > 0) {
        DpArgs a{};
        a.seq_h = dseq_h;
        a.seq_v = dseq_v;
        a.pairs = plan->pairs.as<PairDesc>();
        a.order = plan->order.as<int32_t>();
        a.warp_scratch = plan->warp_scratch.as<int64_t>();
        a.scratch = plan->scratch.as<int2>();
        a.trace = plan->traceback ? plan->trace.as<uint8_t>() : nullptr;
        a.score = dscore;
        a.end_h = end_h;
        a.end_v = end_v;
        a.best_e = plan->traceback ? plan->best_e.as<int32_t>() : nullptr;
        a.best_f = plan->traceback ? plan->best_f.as<int32_t>() : nullptr;
        a.matrix = plan->matrix ? plan->matrix_dev.as<int32_t>() : nullptr;
        a.num_slots = plan->num_slots;
        a.match = plan->params.match;
        a.mismatch = plan->params.mismatch;
        a.gap_open = plan->params.gap_open;
        a.gap_extend = plan->params.gap_extend;
        a.free_ends = plan->free_ends;
        a.alphabet = plan->matrix ? plan->params.alphabet_size : 0;
        const size_t smem = plan->matrix ? size_t(32 * 32) * sizeof(int) : 0;
        DpLauncher launch = plan->dynamic ? pick_dynamic(plan->local, plan->matrix, plan->traceback)
                                          : pick_dp(plan->affine, plan->local, plan->matrix, plan->traceback);
        if (!plan->bucket_start.empty()) {
            for (size_t b = 0; b < plan->bucket_start.size(); ++b) {
                DpArgs ab = a;
                ab.order = a.order + plan->bucket_start[b];
                ab.warp_scratch = a.warp_scratch + plan->bucket_start[b] / 32;
                ab.num_slots = plan->bucket_count[b];
                launch(ab, int((ab.num_slots + kBlock - 1) / kBlock), smem, ctx->stream);
                ++launches;
            }
            --launches;
        } else {
            launch(a, int((plan->num_slots + kBlock - 1) / kBlock), smem, ctx->stream);
        }
        GBA_CUDA(ctx, cudaGetLastError());
        ++launches;
    }
    GBA_CUDA(ctx, cudaEventRecordWithFlags(ctx->ev[1], ctx->stream, evflags));
    {
        const int grid = int((N + 255) / 256);
        k_fill_invalid<<<grid, 256, 0, ctx->stream>>>(
            plan->pairs.as<PairDesc>(), N, minval, dscore, end_h, end_v,
            plan->traceback ? plan->begin_h.as<int32_t>() : nullptr,
            plan->traceback ? plan->begin_v.as<int32_t>() : nullptr,
            plan->traceback ? plan->seg_count.as<int32_t>() : nullptr,
            plan->cigar ? plan->cig_count.as<int32_t>() : nullptr);
        GBA_CUDA(ctx, cudaGetLastError());
        ++launches;
    }
    if (plan->traceback) {
        if (plan->num_slots > 0) {
            TraceArgs t{};
            t.pairs = plan->pairs.as<PairDesc>();
            t.order = plan->order.as<int32_t>();
            t.trace = plan->trace.as<uint8_t>();
            t.score = dscore;
            t.end_h = end_h;
            t.end_v = end_v;
            t.best_e = plan->best_e.as<int32_t>();
            t.best_f = plan->best_f.as<int32_t>();
            t.begin_h = plan->begin_h.as<int32_t>();
            t.begin_v = plan->begin_v.as<int32_t>();
            t.seg_slots = plan->seg_slots.as<uint32_t>();
            t.seg_slot_off = plan->seg_slot_off.as<int64_t>();
            t.seg_count = plan->seg_count.as<int32_t>();
            t.cigar_slots = plan->cigar ? plan->cig_slots.as<uint32_t>() : nullptr;
            t.cigar_slot_off = plan->cigar ? plan->cig_slot_off.as<int64_t>() : nullptr;
            t.cigar_count = plan->cigar ? plan->cig_count.as<int32_t>() : nullptr;
            t.num_slots = plan->num_slots;
            t.affine = plan->affine;
            t.local = plan->local;
            t.extend = plan->extend;
            t.band_w = plan->params.band_on ? plan->params.band_upper - plan->params.band_lower + 1 : 0;
            t.band_upper = plan->params.band_upper;
            t.warp_rows = plan->use_warp ? plan->warp_rows : 0;
            t.warp2 = 0;
            t.dynamic = plan->dynamic;
            const int64_t L = plan->num_tiled_tb;
            if (L > 0) {
                TraceArgs tl = t;
                tl.num_slots = L;
                k_traceback_tiled<kWarpRows><<<int((L + 1) / 2), 64, 0, ctx->stream>>>(tl);
                ++launches;
            }
            if (plan->num_slots > L) {
                TraceArgs ts = t;
                ts.order = t.order + L;
                ts.num_slots = plan->num_slots - L;
                k_traceback<<<int((ts.num_slots + kBlock - 1) / kBlock), kBlock, 0, ctx->stream>>>(ts);
                ++launches;
            }
            GBA_CUDA(ctx, cudaGetLastError());
        }
        if (plan->num_w2 > 0) {
            TraceArgs t{};
            t.pairs = plan->pairs.as<PairDesc>();
            t.order = plan->order_w2.as<int32_t>();
            t.trace = plan->trace.as<uint8_t>();
            t.score = dscore;
            t.end_h = end_h;
            t.end_v = end_v;
            t.best_e = plan->best_e.as<int32_t>();
            t.best_f = plan->best_f.as<int32_t>();
            t.begin_h = plan->begin_h.as<int32_t>();
            t.begin_v = plan->begin_v.as<int32_t>();
            t.seg_slots = plan->seg_slots.as<uint32_t>();
            t.seg_slot_off = plan->seg_slot_off.as<int64_t>();
            t.seg_count = plan->seg_count.as<int32_t>();
            t.cigar_slots = plan->cigar ? plan->cig_slots.as<uint32_t>() : nullptr;
            t.cigar_slot_off = plan->cigar ? plan->cig_slot_off.as<int64_t>() : nullptr;
            t.cigar_count = plan->cigar ? plan->cig_count.as<int32_t>() : nullptr;
            t.num_slots = plan->num_w2;
            t.affine = plan->affine;
            t.local = plan->local;
            t.warp2 = 1;
            k_traceback<<<int((plan->num_w2 + kBlock - 1) / kBlock), kBlock, 0, ctx->stream>>>(t);
            ++launches;
            GBA_CUDA(ctx, cudaGetLastError());
        }
        // Dense packing: exclusive scan of the counts, then a copy per pair.
        const int g1 = int((N + 1 + 255) / 256);
        k_widen<<<g1, 256, 0, ctx->stream>>>(plan->seg_count.as<int32_t>(), plan->seg_count64.as<int64_t>(), N);
        size_t tmp = plan->cub_tmp_bytes;
        GBA_CUDA(ctx, cub::DeviceScan::ExclusiveSum(plan->cub_tmp.ptr, tmp, plan->seg_count64.as<int64_t>(),
                                                    plan->seg_dense_off.as<int64_t>(), int(N + 1), ctx->stream));
        k_compact_u32<<<int((N + 7) / 8), 256, 0, ctx->stream>>>(
            plan->seg_slots.as<uint32_t>(), plan->seg_slot_off.as<int64_t>(), plan->seg_count.as<int32_t>(),
            plan->seg_dense_off.as<int64_t>(), plan->seg_dense.as<uint32_t>(), N, 4);
        launches += 3;
        if (plan->cigar) {
            k_widen<<<g1, 256, 0, ctx->stream>>>(plan->cig_count.as<int32_t>(), plan->cig_count64.as<int64_t>(), N);
            tmp = plan->cub_tmp_bytes;
            GBA_CUDA(ctx, cub::DeviceScan::ExclusiveSum(plan->cub_tmp.ptr, tmp, plan->cig_count64.as<int64_t>(),
                                                        plan->cig_dense_off.as<int64_t>(), int(N + 1), ctx->stream));
            k_compact_u32<<<int((N + 7) / 8), 256, 0, ctx->stream>>>(
                plan->cig_slots.as<uint32_t>(), plan->cig_slot_off.as<int64_t>(), plan->cig_count.as<int32_t>(),
                plan->cig_dense_off.as<int64_t>(), plan->cig_dense.as<uint32_t>(), N, 1);
            launches += 3;
        }
        GBA_CUDA(ctx, cudaGetLastError());
    }
    GBA_CUDA(ctx, cudaEventRecordWithFlags(ctx->ev[2], ctx->stream, evflags));
    plan->launches = launches;
    return GBA_OK;
}

// Runs a plan: the first run with a given set of device pointers captures the launch sequence
// into a CUDA graph; later runs with the same pointers replay it with one graph launch.
int run_plan(gba_context *ctx, gba_plan *plan, const uint8_t *dseq_h, const uint8_t *dseq_v,
             int32_t *dscore, int32_t *dend_h, int32_t *dend_v, bool allow_graph = true)
{
    ctx->stats = gba_stats{};
    ctx->stats.cells = plan->cells;
    ctx->stats.trace_bytes = plan->trace_total;
    plan->seg_dense_total = -1;
    plan->cig_dense_total = -1;
    if (plan->num_pairs == 0) return GBA_OK;
    if (plan->tune_pending) {
        // Autotune: run every tiling variant once on this batch (each run computes the same
        // results), keep the fastest for this context and batch shape.
        float best_ms = 1e30f;
        int best_v = 0;
        for (int v = 0; v < kNumVariants16; ++v) {
            plan->variant16 = v;
            const int rc = enqueue_plan(ctx, plan, dseq_h, dseq_v, dscore, dend_h, dend_v, false);
            if (rc) return rc;
            GBA_CUDA(ctx, cudaEventSynchronize(ctx->ev[1]));
            float ms = 0;
            GBA_CUDA(ctx, cudaEventElapsedTime(&ms, ctx->ev[0], ctx->ev[1]));
            if (ms < best_ms) { best_ms = ms; best_v = v; }
        }
        plan->variant16 = best_v;
        plan->tune_pending = false;
        ctx->tuning[plan->tune_key] = best_v;
        plan->drop_graph();
    }
    const void *key[5] = {dseq_h, dseq_v, dscore, dend_h, dend_v};
    const bool use_graph = allow_graph && !(plan->params.flags & (GBA_FLAG_NO_GRAPH | GBA_FLAG_PLAIN_BUCKETS));
    if (use_graph && plan->graph && std::equal(key, key + 5, plan->graph_key)) {
        GBA_CUDA(ctx, cudaGraphLaunch(plan->graph, ctx->stream));
    } else if (use_graph) {
        plan->drop_graph();
        GBA_CUDA(ctx, cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal));
        const int rc = enqueue_plan(ctx, plan, dseq_h, dseq_v, dscore, dend_h, dend_v, true);
        cudaGraph_t g = nullptr;
        const cudaError_t ec = cudaStreamEndCapture(ctx->stream, &g);
        if (rc) {
            if (g) cudaGraphDestroy(g);
            return rc;
        }
        if (ec != cudaSuccess) return fail(ctx, GBA_ECUDA, "graph capture failed: %s", cudaGetErrorString(ec));
        cudaGraphExec_t exec = nullptr;
        const cudaError_t ei = cudaGraphInstantiate(&exec, g, 0);
        cudaGraphDestroy(g);
        if (ei != cudaSuccess) return fail(ctx, GBA_ECUDA, "graph instantiate failed: %s", cudaGetErrorString(ei));
        plan->graph = exec;
        std::copy(key, key + 5, plan->graph_key);
        GBA_CUDA(ctx, cudaGraphLaunch(plan->graph, ctx->stream));
    } else {
        const int rc = enqueue_plan(ctx, plan, dseq_h, dseq_v, dscore, dend_h, dend_v, false);
        if (rc) return rc;
    }
    if ((plan->use_warp && plan->num_band_states > 0) || plan->num_w2_states > 0) ctx->check_err |= 1u << plan->err_slot;
    ctx->stats.kernel_launches = plan->launches;
    ctx->stats.tile_rows = plan->num16 ? kVariants16[plan->variant16].rows : 0;
    ctx->stats.tile_min_blocks = plan->num16 ? kVariants16[plan->variant16].minb : 0;
    ctx->stats.dp_kernels = (plan->num16 > 0 ? GBA_KERNEL_PACKED : 0) | (plan->num_w2 > 0 ? GBA_KERNEL_WARP16 : 0) |
                            (plan->num_slots > 0 ? (plan->params.band_on ? GBA_KERNEL_BANDED
                                                    : plan->use_warp ? GBA_KERNEL_WARP
                                                    : plan->dynamic ? GBA_KERNEL_DYNAMIC : GBA_KERNEL_STRIP)
                                                 : 0);
    ctx->stats_pending = true;
    return GBA_OK;
}

// Reads the error words of the plan slots whose runs can set them.
int check_wait_errors(gba_context *ctx)
{
    if (!ctx->check_err) return GBA_OK;
    const uint32_t mask = ctx->check_err;
    ctx->check_err = 0;
    int32_t e[kMaxChunks] = {};
    GBA_CUDA(ctx, cudaMemcpyAsync(e, ctx->err_word.ptr, sizeof(e), cudaMemcpyDeviceToHost, ctx->stream));
    GBA_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    for (int i = 0; i < kMaxChunks; ++i)
        if ((mask >> i & 1u) && e[i]) return fail(ctx, GBA_ETIMEOUT, "a wait between the bands of a pair ran out");
    return GBA_OK;
}

int finish_stats(gba_context *ctx)
{
    if (!ctx->stats_pending) return GBA_OK;
    ctx->stats_pending = false;
    GBA_CUDA(ctx, cudaEventSynchronize(ctx->ev[2]));
    if (int rc = check_wait_errors(ctx)) return rc;
    float a = 0, b = 0;
    GBA_CUDA(ctx, cudaEventElapsedTime(&a, ctx->ev[0], ctx->ev[1]));
    GBA_CUDA(ctx, cudaEventElapsedTime(&b, ctx->ev[1], ctx->ev[2]));
    ctx->stats.dp_kernel_ms = a;
    ctx->stats.traceback_kernel_ms = b;
    return GBA_OK;
}

// Copies segment/CIGAR outputs of a finished plan to host result buffers.
int fetch_outputs(gba_context *ctx, gba_plan *plan, gba_result *r)
{
    const int64_t N = plan->num_pairs;
    if (!plan->traceback || N == 0) {
        if (plan->traceback && r->segment_offsets) r->segment_offsets[0] = 0;
        if (plan->cigar && r->cigar_offsets) r->cigar_offsets[0] = 0;
        return GBA_OK;
    }
    std::vector<int64_t> off(N + 1);
    GBA_CUDA(ctx, cudaMemcpyAsync(off.data(), plan->seg_dense_off.ptr, (N + 1) * 8, cudaMemcpyDeviceToHost,
                                  ctx->stream));
    GBA_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    const int64_t total = off[N];
    if (r->segment_offsets) std::memcpy(r->segment_offsets, off.data(), (N + 1) * 8);
    if (r->segments) {
        if (total > r->segment_capacity)
            return fail(ctx, GBA_ECAPACITY, "segment buffer holds %lld, need %lld", (long long)r->segment_capacity,
                        (long long)total);
        if (total > 0)
            GBA_CUDA(ctx, cudaMemcpyAsync(r->segments, plan->seg_dense.ptr, total * 16, cudaMemcpyDeviceToHost,
                                          ctx->stream));
    }
    if (r->begin_h)
        GBA_CUDA(ctx, cudaMemcpyAsync(r->begin_h, plan->begin_h.ptr, N * 4, cudaMemcpyDeviceToHost, ctx->stream));
    if (r->begin_v)
        GBA_CUDA(ctx, cudaMemcpyAsync(r->begin_v, plan->begin_v.ptr, N * 4, cudaMemcpyDeviceToHost, ctx->stream));
    if (plan->cigar) {
        std::vector<int64_t> coff(N + 1);
        GBA_CUDA(ctx, cudaMemcpyAsync(coff.data(), plan->cig_dense_off.ptr, (N + 1) * 8, cudaMemcpyDeviceToHost,
                                      ctx->stream));
        GBA_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
        const int64_t ctotal = coff[N];
        if (r->cigar_offsets) std::memcpy(r->cigar_offsets, coff.data(), (N + 1) * 8);
        if (r->cigar) {
            if (ctotal > r->cigar_capacity)
                return fail(ctx, GBA_ECAPACITY, "cigar buffer holds %lld, need %lld", (long long)r->cigar_capacity,
                            (long long)ctotal);
            if (ctotal > 0)
                GBA_CUDA(ctx, cudaMemcpyAsync(r->cigar, plan->cig_dense.ptr, ctotal * 4, cudaMemcpyDeviceToHost,
                                              ctx->stream));
        }
    }
    GBA_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return GBA_OK;
}

}  // namespace

// Score-only batch of at least 2 * kChunkPairs pairs, in contiguous chunks: chunk c + 1 is
// planned on the host while chunk c runs on the device (each chunk's pairs are length-sorted
// within the chunk).  The input copies are already enqueued on ctx->stream.
int align_batch_chunked(gba_context *ctx, const gba_params *params, const gba_batch *batch, gba_result *result,
                        std::chrono::steady_clock::time_point t0)
{
    const int64_t N = batch->num_pairs;
    const int K = int(std::min<int64_t>(kMaxChunks, N / kChunkPairs));
    while (int(ctx->chunk_plans.size()) < K - 1) ctx->chunk_plans.emplace_back(new gba_plan());
    while (int(ctx->chunk_ev.size()) < 3 * K) {
        cudaEvent_t e = nullptr;
        GBA_CUDA(ctx, cudaEventCreate(&e));
        ctx->chunk_ev.push_back(e);
    }
    GBA_CUDA(ctx, ctx->out_score.ensure(size_t(N) * 4));
    cudaEvent_t saved[3] = {ctx->ev[0], ctx->ev[1], ctx->ev[2]};
    std::vector<int64_t> k0(K + 1);
    for (int c = 0; c <= K; ++c) k0[c] = N * c / K;
    gba_stats total{};
    float plan_ms = 0;
    int rc = GBA_OK;
    for (int c = 0; c < K && rc == GBA_OK; ++c) {
        gba_plan *plan = c == 0 ? &ctx->oneshot : ctx->chunk_plans[c - 1].get();
        plan->err_slot = c;
        gba_batch sub = *batch;
        sub.num_pairs = k0[c + 1] - k0[c];
        if (!batch->h_shared) sub.off_h = batch->off_h + k0[c];
        sub.off_v = batch->off_v + k0[c];
        const auto tp = std::chrono::steady_clock::now();
        rc = build_plan(ctx, params, &sub, plan);
        plan_ms += std::chrono::duration<float, std::milli>(std::chrono::steady_clock::now() - tp).count();
        if (rc) break;
        for (int i = 0; i < 3; ++i) ctx->ev[i] = ctx->chunk_ev[3 * c + i];
        rc = run_plan(ctx, plan, ctx->seq_h.as<uint8_t>(), ctx->seq_v.as<uint8_t>(),
                      ctx->out_score.as<int32_t>() + k0[c], nullptr, nullptr, false);
        total.cells += plan->cells;
        total.kernel_launches += plan->launches;
        total.trace_bytes += plan->trace_total;
        total.dp_kernels |= ctx->stats.dp_kernels;
        total.tile_rows = ctx->stats.tile_rows;
        total.tile_min_blocks = ctx->stats.tile_min_blocks;
    }
    for (int i = 0; i < 3; ++i) ctx->ev[i] = saved[i];
    ctx->stats_pending = false;
    if (rc) {
        cudaStreamSynchronize(ctx->stream);
        return rc;
    }
    if (result->score)
        GBA_CUDA(ctx, cudaMemcpyAsync(result->score, ctx->out_score.ptr, N * 4, cudaMemcpyDeviceToHost, ctx->stream));
    for (int c = 0; c < K; ++c) {
        gba_plan *plan = c == 0 ? &ctx->oneshot : ctx->chunk_plans[c - 1].get();
        const int64_t n = k0[c + 1] - k0[c];
        if (result->end_h)
            GBA_CUDA(ctx, cudaMemcpyAsync(result->end_h + k0[c], plan->end_h.ptr, n * 4, cudaMemcpyDeviceToHost,
                                          ctx->stream));
        if (result->end_v)
            GBA_CUDA(ctx, cudaMemcpyAsync(result->end_v + k0[c], plan->end_v.ptr, n * 4, cudaMemcpyDeviceToHost,
                                          ctx->stream));
    }
    GBA_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    for (int c = 0; c < K; ++c) {
        gba_plan *plan = c == 0 ? &ctx->oneshot : ctx->chunk_plans[c - 1].get();
        if (result->pair_status) std::memcpy(result->pair_status + k0[c], plan->status.data(), (k0[c + 1] - k0[c]) * 4);
        float a = 0, b = 0;
        GBA_CUDA(ctx, cudaEventElapsedTime(&a, ctx->chunk_ev[3 * c], ctx->chunk_ev[3 * c + 1]));
        GBA_CUDA(ctx, cudaEventElapsedTime(&b, ctx->chunk_ev[3 * c + 1], ctx->chunk_ev[3 * c + 2]));
        total.dp_kernel_ms += a;
        total.traceback_kernel_ms += b;
    }
    if ((rc = check_wait_errors(ctx))) return rc;
    total.host_plan_ms = plan_ms;
    total.call_ms = std::chrono::duration<float, std::milli>(std::chrono::steady_clock::now() - t0).count();
    ctx->stats = total;
    return GBA_OK;
}

// =======================================================================================
// C-ABI
// =======================================================================================
extern "C" {

GBA_API const char *gba_status_string(int s)
{
    switch (s) {
    case GBA_OK: return "ok";
    case GBA_EINVAL: return "invalid argument";
    case GBA_ENOMEM: return "out of memory";
    case GBA_EBUDGET: return "HBM budget exceeded";
    case GBA_ECUDA: return "CUDA error";
    case GBA_ETIMEOUT: return "timeout";
    case GBA_EUNSUPPORTED: return "unsupported";
    case GBA_ECAPACITY: return "output buffer too small";
    case GBA_EPARSE: return "input text not in the format";
    default: return "unknown status";
    }
}

GBA_API int gba_create(gba_context **out, const gba_config *cfg)
{
    if (!out) return GBA_EINVAL;
    *out = nullptr;
    std::unique_ptr<gba_context> ctx(new gba_context());
    ctx->device = cfg ? cfg->device : 0;
    ctx->budget = cfg ? cfg->hbm_budget_bytes : 0;
    int ndev = 0;
    cudaError_t e = cudaGetDeviceCount(&ndev);
    if (e != cudaSuccess || ndev == 0) return GBA_ECUDA;
    if (ctx->device < 0 || ctx->device >= ndev) return GBA_EINVAL;
    if (cudaSetDevice(ctx->device) != cudaSuccess) return GBA_ECUDA;
    if (cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking) != cudaSuccess) return GBA_ECUDA;
    // Stream-ordered buffers: keep freed blocks in the device's pool for reuse instead of
    // unmapping them at every synchronization (a setting of this process only).
    cudaMemPool_t pool = nullptr;
    if (cudaDeviceGetDefaultMemPool(&pool, ctx->device) == cudaSuccess) {
        uint64_t keep = UINT64_MAX;
        cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
    }
    for (DevBuf *b : {&ctx->seq_h, &ctx->seq_v, &ctx->out_score, &ctx->out_end_h, &ctx->out_end_v, &ctx->err_word})
        b->bind(ctx->stream);
    for (auto &ev : ctx->ev)
        if (cudaEventCreate(&ev) != cudaSuccess) return GBA_ECUDA;
    *out = ctx.release();
    return GBA_OK;
}

GBA_API int gba_destroy(gba_context *ctx)
{
    if (!ctx) return GBA_OK;
    cudaSetDevice(ctx->device);
    cudaStreamSynchronize(ctx->stream);
    ctx->oneshot.release();
    for (auto &cp : ctx->chunk_plans) cp->release();
    for (cudaEvent_t e : ctx->chunk_ev) cudaEventDestroy(e);
    ctx->seq_h.release();
    ctx->seq_v.release();
    ctx->out_score.release();
    ctx->out_end_h.release();
    ctx->out_end_v.release();
    ctx->err_word.release();
    cudaStreamSynchronize(ctx->stream);   // the stream-ordered frees above
    for (auto &ev : ctx->ev)
        if (ev) cudaEventDestroy(ev);
    if (ctx->stream) cudaStreamDestroy(ctx->stream);
    delete ctx;
    return GBA_OK;
}

GBA_API int gba_last_error(gba_context *ctx, char *buf, size_t size)
{
    if (!ctx || !buf || size == 0) return GBA_EINVAL;
    std::snprintf(buf, size, "%s", ctx->last_error.c_str());
    return GBA_OK;
}

GBA_API int gba_align_batch(gba_context *ctx, const gba_params *params, const gba_batch *batch,
                            gba_result *result)
{
    if (!ctx || !result) return GBA_EINVAL;
    GBA_CUDA(ctx, cudaSetDevice(ctx->device));
    gba_plan *plan = &ctx->oneshot;
    const auto t0 = std::chrono::steady_clock::now();
    // Inputs: the concatenated codes as given.  Their copies are issued before planning so the
    // transfer overlaps the host work.
    if (!ctx->device_codes && batch && batch->num_pairs > 0 && batch->off_h && batch->off_v && batch->seq_h &&
        batch->seq_v) {
        const int64_t N0 = batch->num_pairs;
        const int64_t hb = batch->h_shared ? batch->off_h[1] : batch->off_h[N0];
        const int64_t vb = batch->off_v[N0];
        if (hb < 0 || vb < 0) return fail(ctx, GBA_EINVAL, "negative sequence length");
        GBA_CUDA(ctx, ctx->seq_h.ensure(size_t(hb) + 16));
        GBA_CUDA(ctx, ctx->seq_v.ensure(size_t(vb) + 16));
        if (hb) GBA_CUDA(ctx, cudaMemcpyAsync(ctx->seq_h.ptr, batch->seq_h, hb, cudaMemcpyHostToDevice, ctx->stream));
        if (vb) GBA_CUDA(ctx, cudaMemcpyAsync(ctx->seq_v.ptr, batch->seq_v, vb, cudaMemcpyHostToDevice, ctx->stream));
    }
    if (params && batch && !(params->outputs & GBA_OUT_SEGMENTS) && !(params->flags & GBA_FLAG_PLAIN_BUCKETS) &&
        batch->num_pairs >= 2 * kChunkPairs)
        return align_batch_chunked(ctx, params, batch, result, t0);
    plan->err_slot = 0;
    int rc = build_plan(ctx, params, batch, plan);
    if (rc) return rc;
    const float plan_ms = std::chrono::duration<float, std::milli>(std::chrono::steady_clock::now() - t0).count();
    const int64_t N = batch->num_pairs;
    if (N == 0) {
        if (plan->traceback && result->segment_offsets) result->segment_offsets[0] = 0;
        if (plan->cigar && result->cigar_offsets) result->cigar_offsets[0] = 0;
        return GBA_OK;
    }
    GBA_CUDA(ctx, ctx->out_score.ensure(size_t(N) * 4));
    // A one-shot batch is planned anew on every call, so a captured graph would never be
    // replayed: launch directly.
    rc = run_plan(ctx, plan, ctx->seq_h.as<uint8_t>(), ctx->seq_v.as<uint8_t>(), ctx->out_score.as<int32_t>(),
                  nullptr, nullptr, false);
    if (rc) return rc;
    if (result->score)
        GBA_CUDA(ctx, cudaMemcpyAsync(result->score, ctx->out_score.ptr, N * 4, cudaMemcpyDeviceToHost, ctx->stream));
    if (result->end_h)
        GBA_CUDA(ctx, cudaMemcpyAsync(result->end_h, plan->end_h.ptr, N * 4, cudaMemcpyDeviceToHost, ctx->stream));
    if (result->end_v)
        GBA_CUDA(ctx, cudaMemcpyAsync(result->end_v, plan->end_v.ptr, N * 4, cudaMemcpyDeviceToHost, ctx->stream));
    rc = fetch_outputs(ctx, plan, result);
    if (rc) return rc;
    GBA_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    if (result->pair_status) std::memcpy(result->pair_status, plan->status.data(), N * 4);
    rc = finish_stats(ctx);
    ctx->stats.host_plan_ms = plan_ms;
    ctx->stats.call_ms = std::chrono::duration<float, std::milli>(std::chrono::steady_clock::now() - t0).count();
    return rc;
}

GBA_API int gba_plan_create(gba_context *ctx, const gba_params *params, const gba_batch *host_batch,
                            gba_plan **out)
{
    if (!ctx || !out) return GBA_EINVAL;
    GBA_CUDA(ctx, cudaSetDevice(ctx->device));
    std::unique_ptr<gba_plan> plan(new gba_plan());
    int rc = build_plan(ctx, params, host_batch, plan.get());
    if (rc) {
        plan->release();
        return rc;
    }
    GBA_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    *out = plan.release();
    return GBA_OK;
}

GBA_API int gba_plan_destroy(gba_context *ctx, gba_plan *plan)
{
    if (!plan) return GBA_OK;
    if (ctx) {
        cudaSetDevice(ctx->device);
        cudaStreamSynchronize(ctx->stream);
        plan->release();
        cudaStreamSynchronize(ctx->stream);
    } else {
        // Without its context the plan's stream may be gone: free in order on the default stream.
        cudaDeviceSynchronize();
        plan->bind(nullptr);
        plan->release();
        cudaDeviceSynchronize();
    }
    delete plan;
    return GBA_OK;
}

GBA_API int gba_plan_execute(gba_context *ctx, gba_plan *plan, const gba_batch *dev_batch, gba_result *dev_result)
{
    if (!ctx || !plan || !dev_batch || !dev_result) return GBA_EINVAL;
    if (dev_batch->num_pairs != plan->num_pairs) return fail(ctx, GBA_EINVAL, "batch size differs from plan");
    if (plan->num_pairs > 0 && !dev_result->score) return fail(ctx, GBA_EINVAL, "score output required");
    return run_plan(ctx, plan, dev_batch->seq_h, dev_batch->seq_v, dev_result->score, dev_result->end_h,
                    dev_result->end_v);
}

GBA_API int gba_plan_fetch(gba_context *ctx, gba_plan *plan, gba_result *host_result)
{
    if (!ctx || !plan || !host_result) return GBA_EINVAL;
    int rc = fetch_outputs(ctx, plan, host_result);
    if (rc) return rc;
    if (host_result->pair_status && plan->num_pairs)
        std::memcpy(host_result->pair_status, plan->status.data(), plan->num_pairs * 4);
    return finish_stats(ctx);
}

GBA_API int gba_device_alloc(gba_context *ctx, void **ptr, size_t bytes)
{
    if (!ctx || !ptr) return GBA_EINVAL;
    GBA_CUDA(ctx, cudaSetDevice(ctx->device));
    GBA_CUDA(ctx, cudaMalloc(ptr, std::max<size_t>(bytes, 16)));
    return GBA_OK;
}

GBA_API int gba_device_free(gba_context *ctx, void *ptr)
{
    if (!ctx) return GBA_EINVAL;
    if (ptr) GBA_CUDA(ctx, cudaFree(ptr));
    return GBA_OK;
}

GBA_API int gba_host_alloc(gba_context *ctx, void **ptr, size_t bytes)
{
    if (!ctx || !ptr) return GBA_EINVAL;
    GBA_CUDA(ctx, cudaMallocHost(ptr, std::max<size_t>(bytes, 16)));
    return GBA_OK;
}

GBA_API int gba_host_free(gba_context *ctx, void *ptr)
{
    if (!ctx) return GBA_EINVAL;
    if (ptr) GBA_CUDA(ctx, cudaFreeHost(ptr));
    return GBA_OK;
}

GBA_API int gba_copy_to_device(gba_context *ctx, void *dst, const void *src, size_t bytes)
{
    if (!ctx) return GBA_EINVAL;
    if (bytes) GBA_CUDA(ctx, cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, ctx->stream));
    return GBA_OK;
}

GBA_API int gba_copy_to_host(gba_context *ctx, void *dst, const void *src, size_t bytes)
{
    if (!ctx) return GBA_EINVAL;
    if (bytes) GBA_CUDA(ctx, cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, ctx->stream));
    GBA_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return GBA_OK;
}

int seeds_check_error(gba_context *ctx);   // seeds_host.cuh

GBA_API int gba_synchronize(gba_context *ctx)
{
    if (!ctx) return GBA_EINVAL;
    GBA_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return seeds_check_error(ctx);
}

GBA_API int gba_timer_start(gba_context *ctx)
{
    if (!ctx) return GBA_EINVAL;
    GBA_CUDA(ctx, cudaEventRecord(ctx->ev[4], ctx->stream));
    return GBA_OK;
}

GBA_API int gba_timer_stop(gba_context *ctx, float *ms)
{
    if (!ctx || !ms) return GBA_EINVAL;
    GBA_CUDA(ctx, cudaEventRecord(ctx->ev[5], ctx->stream));
    GBA_CUDA(ctx, cudaEventSynchronize(ctx->ev[5]));
    GBA_CUDA(ctx, cudaEventElapsedTime(ms, ctx->ev[4], ctx->ev[5]));
    return GBA_OK;
}

GBA_API int gba_measure_int_peak(gba_context *ctx, double *tops)
{
    if (!ctx || !tops) return GBA_EINVAL;
    GBA_CUDA(ctx, cudaSetDevice(ctx->device));
    int sms = 0;
    GBA_CUDA(ctx, cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, ctx->device));
    DevBuf out;
    GBA_CUDA(ctx, out.ensure(64));
    const int blocks = sms * 8, threads = 256, iters = 4096;
    k_int_peak<<<blocks, threads, 0, ctx->stream>>>(out.as<int32_t>(), iters, 5);  // warm-up
    GBA_CUDA(ctx, cudaEventRecord(ctx->ev[4], ctx->stream));
    k_int_peak<<<blocks, threads, 0, ctx->stream>>>(out.as<int32_t>(), iters, 7);
    GBA_CUDA(ctx, cudaEventRecord(ctx->ev[5], ctx->stream));
    GBA_CUDA(ctx, cudaEventSynchronize(ctx->ev[5]));
    float ms = 0;
    GBA_CUDA(ctx, cudaEventElapsedTime(&ms, ctx->ev[4], ctx->ev[5]));
    out.release();
    // 16 accumulators x 2 updates x (add + max) per iteration.
    const double ops = double(blocks) * threads * iters * 16.0 * 2.0 * 2.0;
    *tops = ops / (ms * 1e-3) / 1e12;
    return GBA_OK;
}

GBA_API int gba_get_stats(gba_context *ctx, gba_stats *stats)
{
    if (!ctx || !stats) return GBA_EINVAL;
    int rc = finish_stats(ctx);
    if (rc) return rc;
    *stats = ctx->stats;
    return GBA_OK;
}

}  // extern "C"

#include "server.cuh"
#include "seeds_host.cuh"
#include "extend_host.cuh"
#include "enum_host.cuh"
#include "chain_host.cuh"
#include "bgzf_host.cuh"
#include "packed_host.cuh"
#include "sam_host.cuh"
#include "seqio_host.cuh"
