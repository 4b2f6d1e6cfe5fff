// dp_warp_kernels.cuh -- intra-pair parallel DP: one warp per pair (anti-diagonal wavefront).
//
// The 32 lanes of a warp own consecutive strips of R rows of V (a "band" of 32 * R rows).  At
// step t lane l computes column t - l of its strip, so the lanes form an anti-diagonal front:
// the bottom row of lane l - 1's strip for column j (its S and F) is handed to lane l by
// __shfl_up_sync one step later, and the previous hand-off is the diagonal of lane l's first
// row.  Matrices taller than one band pass the band's bottom row to the next band through a
// per-pair row buffer in global memory.  Row 0 is computed by lane 0 of the first band as the
// front passes.  Warps take pairs from a length-sorted queue (longest first).
//
// The per-cell code is the one-pair-per-thread strip kernel's (dp_kernels.cuh): recurrences,
// tie rules, directions and tracked cells of the reference (align/dp_formula_affine.h:66-330,
// align/dp_formula_linear.h:62-258, align/dp_meta_info.h:178-221).  Every lane keeps its own
// best cell with the (column, row) order of the reference's column-major scout
// (align/dp_scout.h:166-180) and the warp reduces the 32 candidates with the same order.
//
// Trace (optional): one byte per cell in step-major order -- for band b and step t the 32
// lanes' R bytes are contiguous, so each step is one coalesced 32 * R byte store per warp.
#pragma once

#include "dp_common.cuh"

namespace gba {

struct WarpArgs {
    const uint8_t *seq_h;
    const uint8_t *seq_v;
    const PairDesc *pairs;
    const int32_t *order;          // work item -> pair index (longest first)
    int2 *rowbuf;                  // per pair at rowbuf_off[p]: (m + 1) int2 band boundary
    const int64_t *rowbuf_off;
    uint8_t *trace;
    int32_t *score, *end_h, *end_v, *best_e, *best_f;
    const int32_t *matrix;
    int32_t *task_counter;
    int32_t num_tasks;
    int32_t match, mismatch, gap_open, gap_extend;
    int32_t free_ends;
    int32_t alphabet;
};

// Trace bytes of one pair in the warp layout: row 0 (m + 1 bytes, padded), then for each band
// (m + 32) steps x 32 lanes x R bytes.
__host__ __device__ inline int64_t warp_trace_bytes(int m, int n, int R)
{
    const int64_t band_rows = 32 * R;
    const int64_t bands = (n + band_rows - 1) / band_rows;
    return align16(m + 1) + bands * int64_t(m + 32) * 32 * R;
}

__device__ __forceinline__ uint8_t trace_at_warp(const uint8_t *base, int m, int R, int col, int row)
{
    if (row == 0) return base[col];
    const int r0 = row - 1;
    const int band_rows = 32 * R;
    const int b = r0 / band_rows;
    const int within = r0 - b * band_rows;
    const int lane = within / R;
    const int r = within - lane * R;
    const int t = col + lane;
    return base[align16(m + 1) + ((int64_t(b) * (m + 32) + t) * 32 + lane) * R + r];
}

struct WarpBest {
    int s, e, f, col, row;
    __device__ __forceinline__ void offer(int cs, int ce, int cf, int ccol, int crow)
    {
        if (cs >= s && (cs > s || ccol < col || (ccol == col && crow < row))) {
            s = cs; e = ce; f = cf; col = ccol; row = crow;
        }
    }
};

template <int R>
__device__ __forceinline__ void store_trace(uint8_t *dst, const uint32_t (&tw)[R / 4])
{
    if (R == 4) *reinterpret_cast<uint32_t *>(dst) = tw[0];
    else if (R == 8) *reinterpret_cast<uint2 *>(dst) = make_uint2(tw[0], tw[1 % (R / 4)]);
    else {
#pragma unroll
        for (int q = 0; q < R / 16; ++q)
            reinterpret_cast<uint4 *>(dst)[q] =
                make_uint4(tw[4 * q], tw[(4 * q + 1) % (R / 4)], tw[(4 * q + 2) % (R / 4)], tw[(4 * q + 3) % (R / 4)]);
    }
}

template <bool AFFINE, bool LOCAL, bool MATRIX, bool TRACE, int R>
__device__ void warp_pair(const WarpArgs &a, const int *smat, int p, int lane)
{
    const PairDesc d = a.pairs[p];
    const int m = d.m, n = d.n;
    const int INF = d.inf;
    const uint8_t *H = a.seq_h + d.h_off;
    const uint8_t *V = a.seq_v + d.v_off;
    uint8_t *T = TRACE ? a.trace + d.trace_off : nullptr;
    int2 *rowbuf = a.rowbuf + a.rowbuf_off[p];
    const int fe = LOCAL ? (FREE_TOP | FREE_LEFT | FREE_RIGHT | FREE_BOTTOM) : a.free_ends;
    const bool fTop = fe & FREE_TOP, fLeft = fe & FREE_LEFT;
    const bool fRight = fe & FREE_RIGHT, fBottom = fe & FREE_BOTTOM;
    const int OPEN = AFFINE ? a.gap_open : a.gap_extend;
    const int EXT = a.gap_extend;
    const int band_rows = 32 * R;
    const int bands = (n + band_rows - 1) / band_rows;
    const int64_t row0Bytes = align16(m + 1);

    WarpBest best{INF, INF, INF, 0, 0};
    if (LOCAL && lane == 0) best.offer(0, INF, INF, 0, 0);

    for (int b = 0; b < bands; ++b) {
        const int i0 = b * band_rows + lane * R + 1;      // first row of this lane's strip
        const bool active = i0 <= n;
        const bool lastStrip = i0 + R > n;                // the strip holds row n (or lies below it)
        uint8_t vc[R];
#pragma unroll
        for (int r = 0; r < R; ++r) vc[r] = (i0 + r <= n) ? V[i0 + r - 1] : 0;
        int Sp[R], Ep[R];
#pragma unroll
        for (int r = 0; r < R; ++r) { Sp[r] = INF; Ep[r] = INF; }
        int s0 = 0, e0 = INF;            // row 0 (lane 0, band 0): S(0, j - 1), E(0, j - 1)
        int outS = INF, outF = INF;      // this lane's hand-off from the previous step
        int diagNext = INF;
        uint8_t *Tband = TRACE ? T + row0Bytes + int64_t(b) * (m + 32) * 32 * R + int64_t(lane) * R : nullptr;
        for (int t = 0; t <= m + 31; ++t) {
            const int j = t - lane;
            const int inS = __shfl_up_sync(0xffffffffu, outS, 1);
            const int inF = __shfl_up_sync(0xffffffffu, outF, 1);
            if (j < 0 || j > m) continue;
            // S and F of the row above this strip, column j.
            int upS, upF;
            if (lane > 0) {
                upS = inS;
                upF = inF;
            } else if (b > 0) {
                const int2 bb = rowbuf[j];
                upS = bb.x;
                upF = bb.y;
            } else {
                // Row 0 cell (0, j): Zero at (0, 0) and with a free first row, else Horizontal.
                uint8_t tv0 = TV_NONE;
                if (j > 0 && !fTop) {
                    if (AFFINE) {
                        const int ex = e0 + EXT, op = s0 + OPEN;
                        if (ex < op) { e0 = op; tv0 = TV_HO | TV_MFH; } else { e0 = ex; tv0 = TV_H | TV_MFH; }
                        s0 = e0;
                    } else {
                        s0 = s0 + EXT;
                        tv0 = TV_H | TV_MFH;
                    }
                }
                if (TRACE) T[j] = tv0;
                if (j > 0 && (LOCAL || (j == m && fRight))) best.offer(s0, fTop ? INF : e0, INF, j, 0);
                upS = s0;
                upF = INF;
            }
            if (!active) {
                outS = INF;
                outF = INF;
                continue;
            }
            uint32_t tw[R / 4];
            int sUp = upS, fUp = upF;
            if (j == 0) {
                // Column 0: Vertical, or Zero with a free first column.
                diagNext = sUp;
#pragma unroll
                for (int r = 0; r < R; ++r) {
                    const int i = i0 + r;
                    uint8_t tv = TV_NONE;
                    int s, f = fUp;
                    if (fLeft) {
                        s = 0;
                    } else if (AFFINE) {
                        const int ex = fUp + EXT, op = sUp + OPEN;
                        if (ex < op) { f = op; tv = TV_VO | TV_MFV; } else { f = ex; tv = TV_V | TV_MFV; }
                        s = f;
                    } else {
                        s = sUp + EXT;
                        tv = TV_V | TV_MFV;
                    }
                    Sp[r] = s;
                    Ep[r] = INF;
                    sUp = s;
                    fUp = f;
                    if (TRACE) {
                        if ((r & 3) == 0) tw[r >> 2] = 0;
                        tw[r >> 2] |= uint32_t(tv) << (8 * (r & 3));
                    }
                    if (i <= n && (LOCAL || (i == n && fBottom))) best.offer(s, INF, f, 0, i);
                }
            } else {
                const int hc = H[j - 1];
                int diag = diagNext;
                diagNext = sUp;
                const bool trackCol = LOCAL || (j == m && fRight);
#pragma unroll
                for (int r = 0; r < R; ++r) {
                    const int sub = MATRIX ? smat[((hc & 31) << 5) | (vc[r] & 31)] : (hc == vc[r] ? a.match : a.mismatch);
                    const int inter = diag + sub;
                    diag = Sp[r];
                    int s, e = Ep[r], f = fUp;
                    uint8_t tv;
                    if (AFFINE) {
                        uint8_t tvE, tvF, tm;
                        const int eExt = Ep[r] + EXT, eOpn = Sp[r] + OPEN;
                        if (eExt < eOpn) { e = eOpn; tvE = TV_HO; } else { e = eExt; tvE = TV_H; }
                        const int fExt = fUp + EXT, fOpn = sUp + OPEN;
                        if (fExt < fOpn) { f = fOpn; tvF = TV_VO; } else { f = fExt; tvF = TV_V; }
                        int g;
                        if (f < e) { g = e; tm = TV_MFH; } else { g = f; tm = TV_MFV; }
                        if (inter < g) { s = g; tv = tm | tvE | tvF; } else { s = inter; tv = TV_DIAG | tvE | tvF; }
                    } else {
                        const int gv = sUp + EXT, gh = Sp[r] + EXT;
                        int g;
                        uint8_t tg;
                        if (gv < gh) { g = gh; tg = TV_H | TV_MFH; } else { g = gv; tg = TV_V | TV_MFV; }
                        if (inter < g) { s = g; tv = tg; } else { s = inter; tv = TV_DIAG; }
                    }
                    if (LOCAL) {
                        if (s <= 0) { s = 0; tv = TV_NONE; }
                    }
                    Sp[r] = s;
                    Ep[r] = e;
                    sUp = s;
                    fUp = f;
                    if (TRACE) {
                        if ((r & 3) == 0) tw[r >> 2] = 0;
                        tw[r >> 2] |= uint32_t(tv) << (8 * (r & 3));
                    }
                    if (!lastStrip || i0 + r <= n) {
                        if (trackCol || (lastStrip && i0 + r == n && (j == m || fBottom)))
                            best.offer(s, e, f, j, i0 + r);
                    }
                }
            }
            if (TRACE) store_trace<R>(Tband + int64_t(t) * 32 * R, tw);
            outS = sUp;
            outF = fUp;
            if (lane == 31 && b + 1 < bands) rowbuf[j] = make_int2(sUp, fUp);
        }
        // The next band's lane 0 reads what lane 31 stored.
        __syncwarp();
    }

    // Warp reduction of the 32 best cells in the reference's column-major order.
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
        const int os = __shfl_down_sync(0xffffffffu, best.s, off);
        const int oe = __shfl_down_sync(0xffffffffu, best.e, off);
        const int of = __shfl_down_sync(0xffffffffu, best.f, off);
        const int oc = __shfl_down_sync(0xffffffffu, best.col, off);
        const int orr = __shfl_down_sync(0xffffffffu, best.row, off);
        if (lane + off < 32) best.offer(os, oe, of, oc, orr);
    }
    if (lane == 0) {
        a.score[p] = best.s;
        if (a.end_h) a.end_h[p] = best.col;
        if (a.end_v) a.end_v[p] = best.row;
        if (a.best_e) a.best_e[p] = best.e;
        if (a.best_f) a.best_f[p] = best.f;
    }
}

template <bool AFFINE, bool LOCAL, bool MATRIX, bool TRACE, int R>
__global__ void __launch_bounds__(128) k_dp_warp(WarpArgs a)
{
    extern __shared__ int smat[];
    if (MATRIX) {
        for (int i = threadIdx.x; i < 32 * 32; i += blockDim.x) {
            const int r = i >> 5, c = i & 31;
            smat[i] = (r < a.alphabet && c < a.alphabet) ? a.matrix[r * a.alphabet + c] : 0;
        }
        __syncthreads();
    }
    const int lane = threadIdx.x & 31;
    for (;;) {
        int task = 0;
        if (lane == 0) task = atomicAdd(a.task_counter, 1);
        task = __shfl_sync(0xffffffffu, task, 0);
        if (task >= a.num_tasks) break;
        warp_pair<AFFINE, LOCAL, MATRIX, TRACE, R>(a, smat, a.order[task], lane);
    }
}

}  // namespace gba
