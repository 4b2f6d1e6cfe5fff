// noalloc.cu -- gba_align_score_noalloc: batch alignment scores with no device allocation.
//
// Some callers cannot allocate device memory on the path that calls the aligner: hosts that
// own every byte of device memory through their own pool (a database or plugin host that
// hands out buffers), and latency-bound request loops that keep cudaMalloc/cudaFree -- which
// can synchronize the device and take unbounded time -- off their request path.  They still
// allocate their inputs and outputs themselves and pass device pointers here.  This entry
// point therefore needs no gba_context and never calls cudaMalloc, cudaFree or any allocating
// library routine: the DP kernel's scratch (the boundary row that one register strip of
// rows hands to the next) lives in the file-scope array below, which every GPU that loads
// this library holds until the process exits.
//
// Set-up: the first call on each device looks up that device's address of the array with
// cudaGetSymbolAddress (the device must be current).  With CUDA's lazy module loading (the
// default) that lookup is also when this file's module is loaded on the device and the array's
// 64 MiB are committed, and the first call of each scoring shape (affine or linear, global or
// local, table or not) loads that kernel's code, so first calls may allocate and synchronize: make
// one per shape at start-up (or run with CUDA_MODULE_LOADING=EAGER), before any stream capture
// starts and before a host pool reserves the GPU's memory.  Repeated calls allocate nothing.  All
// calls share the array and it keeps the previous call's
// contents; the kernel writes every scratch element before reading it, so nothing has to be
// cleared.  Calls that overlap on the GPU (on different streams, or from several threads)
// race on the array and must be serialized by the caller.
//
// The DP is the one-pair-per-thread strip sweep of dp_kernels.cuh (same recurrences, tie rules
// and best-cell choice as the reference: align/dp_formula_affine.h:66-330,
// align/dp_formula_linear.h:62-258, align/dp_meta_info.h:178-221, align/dp_scout.h:166-180),
// restricted to scores and end positions, reading lengths from device offsets and visiting
// pairs grid-stride so a bounded number of lanes shares the fixed scratch.
#include "../../include/seqan_gb300.h"

#include "dp_common.cuh"

#include <cuda_runtime.h>

#include <climits>
#include <cstdlib>
#include <mutex>

namespace {

using namespace gba;

constexpr size_t kScratchBytes = GBA_NOALLOC_SCRATCH_BYTES;
constexpr int64_t kScratchElems = int64_t(kScratchBytes / sizeof(int2));

static __device__ __align__(256) int2 g_noalloc_scratch[kScratchElems];

struct NoAllocArgs {
    const uint8_t *seq_h;
    const int64_t *off_h;
    const uint8_t *seq_v;
    const int64_t *off_v;
    int2 *scratch;             // device address of g_noalloc_scratch
    int32_t *score, *end_h, *end_v, *status;
    int64_t num_pairs;
    int64_t num_slots;         // lanes that own a scratch column (multiple of 32)
    int32_t max_h_len;
    int32_t match, mismatch, gap_open, gap_extend;
    int32_t free_ends;
    int32_t score_bits;
    int32_t max_pos;           // largest positive substitution score (int16 range check)
    int32_t alphabet;
    int8_t matrix[32 * 32];    // substitution table by value (row = H code), zero padded
};

__device__ __forceinline__ bool exact16(const NoAllocArgs &a, int64_t m, int64_t n, bool local)
{
    const int64_t open = abs(a.gap_open), ext = abs(a.gap_extend);
    if (int64_t(a.max_pos) * (m < n ? m : n) > 32767 - 64) return false;
    if (local) return true;
    return -(3 * open + ext * (m + n + 2)) > -16384 + 2 * (open + ext) + 64;
}

template <bool AFFINE, bool LOCAL, bool MATRIX>
__global__ void __launch_bounds__(128) k_dp_noalloc(NoAllocArgs a)
{
    const int64_t slot = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (slot >= a.num_slots) return;
    int2 *bnd = a.scratch + (slot >> 5) * int64_t(32) * (a.max_h_len + 1) + (slot & 31);
    const int fe = LOCAL ? (FREE_TOP | FREE_LEFT | FREE_RIGHT | FREE_BOTTOM) : a.free_ends;
    const bool fTop = fe & FREE_TOP, fLeft = fe & FREE_LEFT;
    const bool fRight = fe & FREE_RIGHT, fBottom = fe & FREE_BOTTOM;
    const int OPEN = AFFINE ? a.gap_open : a.gap_extend;
    const int EXT = a.gap_extend;

    for (int64_t p = slot; p < a.num_pairs; p += a.num_slots) {
        const int64_t h0 = a.off_h[p], v0 = a.off_v[p];
        const int64_t m64 = a.off_h[p + 1] - h0, n64 = a.off_v[p + 1] - v0;
        const int32_t minval = a.score_bits == 16 ? -32768 : INT_MIN;
        if (m64 <= 0 || n64 <= 0 || m64 > a.max_h_len || n64 > (int64_t(1) << 30)) {
            // Empty pairs score numeric min like the reference (GBA_PAIR_INVALID); pairs longer
            // than the caller's bound are not computed -- their scratch column would not fit --
            // and get numeric min with GBA_PAIR_SKIPPED, so the two cases stay apart.
            const bool empty = m64 <= 0 || n64 <= 0;
            a.score[p] = minval;
            if (a.end_h) a.end_h[p] = 0;
            if (a.end_v) a.end_v[p] = 0;
            if (a.status) a.status[p] = empty ? GBA_PAIR_INVALID : GBA_PAIR_SKIPPED;
            continue;
        }
        const int m = int(m64), n = int(n64);
        const bool e16 = a.score_bits == 16 && exact16(a, m, n, LOCAL);
        const int INF = e16 ? -16384 : -(1 << 30);
        if (a.status) a.status[p] = (a.score_bits == 16 && !e16) ? GBA_PAIR_PROMOTED : GBA_PAIR_OK;
        const uint8_t *H = a.seq_h + h0;
        const uint8_t *V = a.seq_v + v0;

        int bs = INF, bcol = 0, brow = 0;
        auto offer = [&](int s, int col, int row) {
            if (s >= bs && (s > bs || col < bcol || (col == bcol && row < brow))) {
                bs = s; bcol = col; brow = row;
            }
        };

        // Row 0.
        {
            int s = 0, e = INF;
            bnd[0] = make_int2(0, INF);
            if (LOCAL) offer(0, 0, 0);
            for (int j = 1; j <= m; ++j) {
                if (!fTop) {
                    if (AFFINE) {
                        const int ext = e + EXT, opn = s + OPEN;
                        e = ext < opn ? opn : ext;
                        s = e;
                    } else {
                        s = s + EXT;
                    }
                }
                bnd[int64_t(j) * 32] = make_int2(s, INF);
                if (LOCAL || (j == m && fRight)) offer(s, j, 0);
            }
        }
        for (int i0 = 1; i0 <= n; i0 += STRIP_ROWS) {
            uint8_t vc[STRIP_ROWS];
#pragma unroll
            for (int r = 0; r < STRIP_ROWS; ++r) vc[r] = (i0 + r <= n) ? V[i0 + r - 1] : 0;
            int Sp[STRIP_ROWS], Ep[STRIP_ROWS];
            const bool lastStrip = (i0 + STRIP_ROWS > n);
            int diagNext;
            {
                const int2 up = bnd[0];
                int sUp = up.x, fUp = up.y;
                diagNext = sUp;
#pragma unroll
                for (int r = 0; r < STRIP_ROWS; ++r) {
                    int s, f = fUp;
                    if (fLeft) {
                        s = 0;
                    } else if (AFFINE) {
                        const int ext = fUp + EXT, opn = sUp + OPEN;
                        f = ext < opn ? opn : ext;
                        s = f;
                    } else {
                        s = sUp + EXT;
                    }
                    Sp[r] = s;
                    Ep[r] = INF;
                    sUp = s;
                    fUp = f;
                    const int i = i0 + r;
                    if (i <= n && (LOCAL || (i == n && fBottom))) offer(s, 0, i);
                }
                bnd[0] = make_int2(sUp, fUp);
            }
            for (int j = 1; j <= m; ++j) {
                const int hc = H[j - 1];
                const int2 up = bnd[int64_t(j) * 32];
                int sUp = up.x, fUp = up.y;
                int diag = diagNext;
                diagNext = sUp;
                const bool trackCol = LOCAL || (j == m && fRight);
#pragma unroll
                for (int r = 0; r < STRIP_ROWS; ++r) {
                    const int sub = MATRIX ? int(a.matrix[((hc & 31) << 5) | (vc[r] & 31)])
                                           : (hc == vc[r] ? a.match : a.mismatch);
                    const int inter = diag + sub;
                    diag = Sp[r];
                    int s, e = Ep[r], f = fUp;
                    if (AFFINE) {
                        const int eExt = Ep[r] + EXT, eOpn = Sp[r] + OPEN;
                        e = eExt < eOpn ? eOpn : eExt;
                        const int fExt = fUp + EXT, fOpn = sUp + OPEN;
                        f = fExt < fOpn ? fOpn : fExt;
                        const int g = f < e ? e : f;
                        s = inter < g ? g : inter;
                    } else {
                        const int gv = sUp + EXT, gh = Sp[r] + EXT;
                        const int g = gv < gh ? gh : gv;
                        s = inter < g ? g : inter;
                    }
                    if (LOCAL && s <= 0) s = 0;
                    Sp[r] = s;
                    Ep[r] = e;
                    sUp = s;
                    fUp = f;
                    if (!lastStrip || i0 + r <= n) {
                        if (trackCol || (lastStrip && i0 + r == n && (j == m || fBottom))) offer(s, j, i0 + r);
                    }
                }
                bnd[int64_t(j) * 32] = make_int2(sUp, fUp);
            }
        }
        a.score[p] = bs;
        if (a.end_h) a.end_h[p] = bcol;
        if (a.end_v) a.end_v[p] = brow;
    }
}

template <bool A, bool L, bool M>
void launch(const NoAllocArgs &a, int grid, cudaStream_t s)
{
    k_dp_noalloc<A, L, M><<<grid, 128, 0, s>>>(a);
}

std::mutex g_setup_mutex;
void *g_scratch_addr[256] = {};

}  // namespace

extern "C" GBA_API int gba_align_score_noalloc(const gba_params *params, const gba_noalloc_batch *batch,
                                               int32_t *score, int32_t *end_h, int32_t *end_v,
                                               int32_t *pair_status, void *stream)
{
    if (!params || !batch || (batch->num_pairs > 0 && !score)) return GBA_EINVAL;
    if (batch->num_pairs < 0) return GBA_EINVAL;
    if (params->mode != GBA_GLOBAL && params->mode != GBA_LOCAL) return GBA_EINVAL;
    if (params->score_bits != 16 && params->score_bits != 32) return GBA_EINVAL;
    if (params->gap_model < 0 || params->gap_model > GBA_GAPS_AFFINE) return GBA_EUNSUPPORTED;
    if (params->free_ends & ~15) return GBA_EINVAL;
    if (params->band_on || (params->outputs & (GBA_OUT_SEGMENTS | GBA_OUT_CIGAR))) return GBA_EUNSUPPORTED;
    if (batch->max_h_len < 1) return GBA_EINVAL;
    // One warp keeps 32 scratch columns of max_h_len + 1 cells; refuse bounds that do not fit.
    const int64_t warp_elems = int64_t(32) * (int64_t(batch->max_h_len) + 1);
    if (warp_elems > kScratchElems) return GBA_ECAPACITY;
    if (batch->num_pairs == 0) return GBA_OK;
    if (!batch->seq_h || !batch->seq_v || !batch->off_h || !batch->off_v) return GBA_EINVAL;

    NoAllocArgs a{};
    const bool affine = params->gap_model == GBA_GAPS_AFFINE ||
                        (params->gap_model == GBA_GAPS_AUTO && params->gap_open != params->gap_extend);
    int max_pos = 0;
    if (params->matrix) {
        if (params->alphabet_size <= 0 || params->alphabet_size > 32) return GBA_EINVAL;
        const int asz = params->alphabet_size;
        for (int r = 0; r < asz; ++r)
            for (int c = 0; c < asz; ++c) {
                const int v = params->matrix[r * asz + c];
                if (v < -128 || v > 127) return GBA_EUNSUPPORTED;  // the table travels as int8
                a.matrix[(r << 5) | c] = int8_t(v);
                max_pos = v > max_pos ? v : max_pos;
            }
        a.alphabet = asz;
    } else {
        max_pos = params->match > params->mismatch ? params->match : params->mismatch;
        max_pos = max_pos > 0 ? max_pos : 0;
    }

    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 256) return GBA_ECUDA;
    {
        std::lock_guard<std::mutex> lock(g_setup_mutex);
        if (!g_scratch_addr[dev]) {
            void *ptr = nullptr;
            if (cudaGetSymbolAddress(&ptr, g_noalloc_scratch) != cudaSuccess || !ptr) return GBA_ECUDA;
            g_scratch_addr[dev] = ptr;
        }
        a.scratch = static_cast<int2 *>(g_scratch_addr[dev]);
    }

    a.seq_h = batch->seq_h;
    a.off_h = batch->off_h;
    a.seq_v = batch->seq_v;
    a.off_v = batch->off_v;
    a.score = score;
    a.end_h = end_h;
    a.end_v = end_v;
    a.status = pair_status;
    a.num_pairs = batch->num_pairs;
    a.max_h_len = batch->max_h_len;
    a.match = params->match;
    a.mismatch = params->mismatch;
    a.gap_open = params->gap_open;
    a.gap_extend = params->gap_extend;
    a.free_ends = params->free_ends;
    a.score_bits = params->score_bits;
    a.max_pos = max_pos;
    const int64_t warps_fit = kScratchElems / warp_elems;
    const int64_t warps_need = (batch->num_pairs + 31) / 32;
    a.num_slots = 32 * (warps_fit < warps_need ? warps_fit : warps_need);
    const int grid = int((a.num_slots + 127) / 128);
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    const bool local = params->mode == GBA_LOCAL, mat = params->matrix != nullptr;
    using Fn = void (*)(const NoAllocArgs &, int, cudaStream_t);
    static const Fn table[8] = {launch<false, false, false>, launch<false, false, true>,
                                launch<false, true, false>,  launch<false, true, true>,
                                launch<true, false, false>,  launch<true, false, true>,
                                launch<true, true, false>,   launch<true, true, true>};
    // An error already pending on this thread (the caller's own) is left in place for the caller
    // and reported as GBA_ECUDA without launching; only this call's launch error is consumed.
    if (cudaPeekAtLastError() != cudaSuccess) return GBA_ECUDA;
    table[(affine ? 4 : 0) | (local ? 2 : 0) | (mat ? 1 : 0)](a, grid, s);
    return cudaGetLastError() == cudaSuccess ? GBA_OK : GBA_ECUDA;
}
