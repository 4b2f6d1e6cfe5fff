// dp_warp_kernels.cuh -- intra-pair parallel DP: bands of 32 * R rows, one warp per band.
//
// The 32 lanes of a warp own consecutive strips of R rows of V (a "band" of 32 * R rows).  At
// step t lane l computes column t - l of its strip, so the lanes form an anti-diagonal front:
// the bottom row of lane l - 1's strip for column j (its S and F) is handed to lane l by
// __shfl_up_sync one step later, and the previous hand-off is the diagonal of lane l's first
// row.  Row 0 is computed by lane 0 of band 0 as the front passes.
//
// The unit of work is one band of one pair.  Warps take (pair, band) tasks from a queue that
// lists the pairs longest first and each pair's bands in order, so the bands of a long pair run
// at the same time on different warps as a pipeline: band b reads band b - 1's bottom row
// (S, F per column) from a two-slot row buffer in global memory, 32 columns at a time, once
// band b - 1 has published that it has written them (a release/acquire counter per band).  Every
// band a warp waits on was taken from the queue before its own band, by a warp that is running,
// so the waits end; each wait still has an iteration limit after which the kernel records an
// error and carries on.  A pipelined band idles for about 130 steps before its first column,
// so when there is enough other work (many pairs) a narrow pair is instead one task (band -1)
// whose warp runs its bands in order, with no waits.  Band b + 2 reuses band b's row slot: it writes column j only after
// band b + 1 has produced column j, which band b + 1 does only after reading column j of band b.
//
// The per-cell code is the one-pair-per-thread strip kernel's (dp_kernels.cuh): recurrences,
// tie rules, directions and tracked cells of the reference (align/dp_formula_affine.h:66-330,
// align/dp_formula_linear.h:62-258, align/dp_meta_info.h:178-221).  Every lane keeps its own
// best cell with the (column, row) order of the reference's column-major scout
// (align/dp_scout.h:166-180); the warp reduces the 32 candidates and the bands of a pair
// combine theirs in band order with the same (total) order.
//
// Trace (optional): one byte per cell in step-major order -- for band b and step t the 32
// lanes' R bytes are contiguous, so each step is one coalesced 32 * R byte store per warp.
#pragma once

#include "dp_common.cuh"

namespace gba {

// Cross-band state of one band of a multi-band pair (zeroed before every run).
struct BandState {
    int progress;                  // columns of the band's bottom row written to the row buffer
    int done;                      // 1 once s..row hold the best cell of bands 0..b
    int s, e, f, col, row, pad;
};

struct WarpArgs {
    const uint8_t *seq_h;
    const uint8_t *seq_v;
    const PairDesc *pairs;
    const int2 *tasks;             // work item -> (pair, band); pairs longest first, bands in order
    int2 *rowbuf;                  // per multi-band pair at rowbuf_off[p]: 2 x (m + 1) int2
    const int64_t *rowbuf_off;
    BandState *bands;              // per multi-band pair at band_base[p]: one per band
    const int64_t *band_base;
    int32_t *error;                // set to 1 when a wait ran out
    uint8_t *trace;
    int32_t *score, *end_h, *end_v, *best_e, *best_f;
    const int32_t *matrix;
    int32_t *task_counter;
    int32_t num_tasks;
    int32_t match, mismatch, gap_open, gap_extend;
    int32_t free_ends;
    int32_t alphabet;
};

// Bands are 32 lanes x R rows (R = 8: 256 rows), except that a pair's last band holding at most
// half that many rows runs with R / 2 rows per lane: its idle rows would otherwise cost as much
// as busy ones.  Rows per lane of the last band of an n-row pair:
__host__ __device__ inline int warp_last_rows(int n, int R)
{
    const int rem = n - ((n - 1) / (32 * R)) * (32 * R);
    return rem <= 16 * R ? R / 2 : R;
}

// Trace bytes of one pair in the warp layout: row 0 (m + 1 bytes, padded), then for each band
// (m + 32) steps x 32 lanes x (its rows per lane) bytes.
__host__ __device__ inline int64_t warp_trace_bytes(int m, int n, int R)
{
    if (n <= 0) return align16(m + 1);
    const int64_t bands = (n + 32 * R - 1) / (32 * R);
    return align16(m + 1) + ((bands - 1) * R + warp_last_rows(n, R)) * int64_t(m + 32) * 32;
}

// Byte offset of band b's trace within the pair's trace, and its rows per lane.
__host__ __device__ inline int64_t warp_band_trace_off(int m, int b, int R)
{
    return align16(m + 1) + int64_t(b) * (m + 32) * 32 * R;
}

__device__ __forceinline__ uint8_t trace_at_warp(const uint8_t *base, int m, int n, int R, int col, int row)
{
    if (row == 0) return base[col];
    const int r0 = row - 1;
    const int b = r0 / (32 * R);
    const int Rb = (b == (n - 1) / (32 * R)) ? warp_last_rows(n, R) : R;
    const int within = r0 - b * 32 * R;
    const int lane = within / Rb;
    const int r = within - lane * Rb;
    const int t = col + lane;
    return base[warp_band_trace_off(m, b, R) + (int64_t(t) * 32 + lane) * Rb + r];
}

struct WarpBest {
    int s, e, f, col, row;
    __device__ __forceinline__ void offer(int cs, int ce, int cf, int ccol, int crow)
    {
        if (cs >= s && (cs > s || ccol < col || (ccol == col && crow < row))) {
            s = cs; e = ce; f = cf; col = ccol; row = crow;
        }
    }
    // For candidates visited in column-major order: a later cell wins only with a higher score.
    __device__ __forceinline__ void offer_later(int cs, int ce, int cf, int ccol, int crow)
    {
        if (cs > s) {
            s = cs; e = ce; f = cf; col = ccol; row = crow;
        }
    }
};

// Maximum of a strip's R values with 3-way max instructions.
template <int R>
__device__ __forceinline__ int strip_max(const int (&v)[R])
{
    int m = v[0];
    int r = 1;
#pragma unroll
    for (; r + 1 < R; r += 2) m = __vimax3_s32(m, v[r], v[r + 1]);
#pragma unroll
    for (; r < R; ++r) m = max(m, v[r]);
    return m;
}

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

__device__ __forceinline__ int ld_acquire_gpu(const int *p)
{
    int v;
    asm volatile("ld.acquire.gpu.global.s32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

__device__ __forceinline__ void st_release_gpu(int *p, int v)
{
    asm volatile("st.release.gpu.global.s32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

// Warp-wide wait until *p >= need, seen by every lane (each lane's own acquire orders its later
// loads).  Gives up after about a second of polling, or at once when another wait already gave
// up, recording the error.
__device__ __forceinline__ void warp_wait_at_least(const int *p, int need, int32_t *error)
{
    for (int it = 0;; ++it) {
        if (__all_sync(0xffffffffu, ld_acquire_gpu(p) >= need)) return;
        if ((it & 1023) == 1023 && __any_sync(0xffffffffu, *(volatile int32_t *)error != 0)) return;
        if (it > (1 << 22)) {
            if ((threadIdx.x & 31) == 0) atomicExch(error, 1);
            return;
        }
        __nanosleep(256);
    }
}

constexpr int kRowChunk = 32;   // columns per row-buffer hand-off between bands

// One band of pair p with R rows per lane; RF is the rows per lane of the pair's full bands.
template <bool AFFINE, bool LOCAL, bool MATRIX, bool TRACE, int RF, int R>
__device__ void warp_band(const WarpArgs &a, const int *smat, int2 *rb, int p, int b, int lane, bool seq,
                          WarpBest &carry)
{
    const PairDesc d = a.pairs[p];
    const int m = d.m, n = d.n;
    const int INF = d.inf;
    const uint8_t *H = a.seq_h + d.h_off;
    const uint8_t *V = a.seq_v + d.v_off;
    uint8_t *T = TRACE ? a.trace + d.trace_off : nullptr;
    const int fe = LOCAL ? (FREE_TOP | FREE_LEFT | FREE_RIGHT | FREE_BOTTOM) : a.free_ends;
    const bool fTop = fe & FREE_TOP, fLeft = fe & FREE_LEFT;
    const bool fRight = fe & FREE_RIGHT, fBottom = fe & FREE_BOTTOM;
    const int OPEN = AFFINE ? a.gap_open : a.gap_extend;
    const int EXT = a.gap_extend;
    const int band_rows = 32 * RF;
    const int bands = (n + band_rows - 1) / band_rows;

    WarpBest best{INF, INF, INF, 0, 0};
    if (LOCAL && lane == 0 && b == 0) best.offer(0, INF, INF, 0, 0);
    // Row buffers: band b writes slot b & 1 and reads slot (b - 1) & 1.
    int2 *rowOut = nullptr;
    const int2 *rowIn = nullptr;
    BandState *st = nullptr;
    if (bands > 1) {
        rowOut = a.rowbuf + a.rowbuf_off[p] + int64_t(b & 1) * (m + 1);
        rowIn = a.rowbuf + a.rowbuf_off[p] + int64_t((b + 1) & 1) * (m + 1);
        st = a.bands + a.band_base[p] + b;
    }
    int2 pre = make_int2(0, 0);   // lane k: entry c + k of the band above, for the next chunk c
    auto fetch = [&](int c0) {
        if (!seq) warp_wait_at_least(&st[-1].progress, min(c0 + kRowChunk, m + 1), a.error);
        if (c0 + lane <= m) pre = __ldcg(rowIn + c0 + lane);
    };
    if (b > 0) fetch(0);

    {
        const int i0 = b * band_rows + lane * R + 1;      // first row of this lane's strip
        const int rvalid = n - i0 + 1;                     // rows of this strip inside the matrix
        const int rowN = (rvalid >= 1 && rvalid <= R) ? rvalid - 1 : -1;   // row n, if here
        const bool trackRowN = !LOCAL && fBottom && rowN >= 0;
        uint8_t vc[R];
#pragma unroll
        for (int r = 0; r < R; ++r) vc[r] = (i0 + r <= n) ? V[i0 + r - 1] : 0;
        int Sp[R], Ep[R];
#pragma unroll
        for (int r = 0; r < R; ++r) { Sp[r] = INF; Ep[r] = INF; }
        int s0 = 0, e0 = INF;            // row 0 (lane 0, band 0): S(0, j - 1), E(0, j - 1)
        int outS = INF, outF = INF;      // this lane's hand-off from the previous step
        int diagNext = INF;
        int hnext = H[0];
        uint8_t *Tband = TRACE ? T + warp_band_trace_off(m, b, RF) + int64_t(lane) * R : nullptr;
        // One loop body for every step.  Lane l holds column j = t - l; lanes with j outside
        // [0, m] (the fill and drain of the front) compute values nothing reads: their trace
        // bytes lie at steps the traceback never visits, their hand-off reaches only lanes that
        // are idle too, and they offer no best cell.  Column 0 and column m take short branches.
        // The recurrences run on max / add-max / 3-way max, which equal the reference's
        // compare-and-select values, ties included; the trace bits come from comparisons of the
        // chain's own values, off the dependency chain down the column.
        // Full-height bands also get a lean copy of the cell code for the steady steps (all
        // lanes in columns 1 .. m - 1: no edge tests, shorter per-step latency), except the
        // matrix-scored traceback variant, whose code with that copy no longer fits the
        // instruction cache next to the short band's (measured 5% slower).
        constexpr bool kLeanSteady = R == RF && !(MATRIX && TRACE);
        for (int t = 0; t <= m + 31; ++t) {
            if (kLeanSteady && t == 32 && m - 1 >= 32) {
                // Steady phase, steps 32 .. m - 1: every lane's column lies in [1, m - 1], so
                // there is no column 0, no last column and no idle lane; lane 0's input is a
                // select.  The recurrences run on max / add-max / 3-way max (the values equal the
                // compare-and-select form of the other steps, ties included), and the trace bits
                // come from comparisons off the dependency chain down the column.  Each lane
                // meets its cells in column-major order.
                const int rvalid = n - i0 + 1;             // rows of this strip inside the matrix
                const int rowN = (rvalid >= 1 && rvalid <= R) ? rvalid - 1 : -1;   // row n, if here
                const bool trackRowN = !LOCAL && fBottom && rowN >= 0;
                // hnext already holds H[31 - lane], this lane's column at step 32; the steady
                // loop leaves in it the code the drain steps start from.
                for (; t <= m - 1; ++t) {
                    const int j = t - lane;
                    if (b > 0 && (t & (kRowChunk - 1)) == 0) {
                        __syncwarp();
                        rb[lane] = pre;
                        __syncwarp();
                        if (t + kRowChunk <= m) fetch(t + kRowChunk);
                    }
                    const int inS = __shfl_up_sync(0xffffffffu, outS, 1);
                    const int inF = __shfl_up_sync(0xffffffffu, outF, 1);
                    const int hc = hnext;
                    hnext = H[j];                          // column j + 1 at the next step
                    int2 bb;
                    if (b == 0) {
                        // Row 0, column j (lane 0's; the other lanes' copies go unused).
                        uint8_t tv0 = TV_NONE;
                        if (!fTop) {
                            if (AFFINE) {
                                const int ex = e0 + EXT, op = s0 + OPEN;
                                tv0 = ex < op ? (TV_HO | TV_MFH) : (TV_H | TV_MFH);
                                e0 = max(ex, op);
                                s0 = e0;
                            } else {
                                s0 = s0 + EXT;
                                tv0 = TV_H | TV_MFH;
                            }
                        }
                        if (TRACE && lane == 0) T[j] = tv0;
                        bb = make_int2(s0, INF);
                    } else {
                        bb = rb[j & (kRowChunk - 1)];
                    }
                    int sUp = lane ? inS : bb.x;
                    int fUp = lane ? inF : bb.y;
                    int diag = diagNext;
                    diagNext = sUp;
                    const int hrow = MATRIX ? ((hc & 31) << 5) : hc;
                    uint32_t tw[R / 4];
                    int Fp[R];                             // F of each row (for the best cell)
#pragma unroll
                    for (int r = 0; r < R; ++r) {
                        const int sub = MATRIX ? smat[hrow | (vc[r] & 31)] : (hc == vc[r] ? a.match : a.mismatch);
                        const int inter = diag + sub;
                        diag = Sp[r];
                        int s, e = Ep[r], f = fUp;
                        uint32_t tv = 0;
                        if (AFFINE) {
                            const int eExt = Ep[r] + EXT, eOpn = Sp[r] + OPEN;
                            e = max(eExt, eOpn);
                            const int fExt = fUp + EXT;
                            f = __viaddmax_s32(sUp, OPEN, fExt);
                            s = LOCAL ? __vimax3_s32_relu(inter, e, f) : __vimax3_s32(inter, e, f);
                            if (TRACE) {
                                // s == inter: the diagonal wins (ties included); e != eExt: the
                                // gap opened (eExt < eOpn); f != fExt: likewise for F.  With the
                                // local zero floor, s == 0 overrides everything below.
                                tv = s == inter ? TV_DIAG : (f < e ? TV_MFH : TV_MFV);
                                tv |= e != eExt ? TV_HO : TV_H;
                                tv |= f != fExt ? TV_VO : TV_V;
                            }
                        } else {
                            const int gv = sUp + EXT, gh = Sp[r] + EXT;
                            s = LOCAL ? __vimax3_s32_relu(inter, gv, gh) : __vimax3_s32(inter, gv, gh);
                            if (TRACE)
                                tv = s == inter ? TV_DIAG : (gv < gh ? (TV_H | TV_MFH) : (TV_V | TV_MFV));
                        }
                        if (TRACE && LOCAL && s == 0) tv = TV_NONE;
                        Sp[r] = s;
                        Ep[r] = e;
                        Fp[r] = f;
                        sUp = s;
                        fUp = f;
                        if (TRACE) {
                            if ((r & 3) == 0) tw[r >> 2] = 0;
                            tw[r >> 2] |= tv << (8 * (r & 3));
                        }
                    }
                    if (LOCAL) {
                        // Column j's best row of this strip: the first row holding the strip's
                        // maximum, taken only when it beats every earlier column.
                        if (rvalid >= R) {
                            const int mx = strip_max<R>(Sp);
                            if (mx > best.s) {
#pragma unroll
                                for (int r = 0; r < R; ++r)
                                    if (Sp[r] == mx) {
                                        best.offer_later(Sp[r], Ep[r], Fp[r], j, i0 + r);
                                        break;
                                    }
                            }
                        } else {
#pragma unroll
                            for (int r = 0; r < R; ++r)
                                if (r < rvalid) best.offer_later(Sp[r], Ep[r], Fp[r], j, i0 + r);
                        }
                    } else if (trackRowN) {
#pragma unroll
                        for (int r = 0; r < R; ++r)
                            if (r == rowN) best.offer_later(Sp[r], Ep[r], Fp[r], j, i0 + r);
                    }
                    if (TRACE) store_trace<R>(Tband + int64_t(t) * 32 * R, tw);
                    outS = sUp;
                    outF = fUp;
                    if (lane == 31 && b + 1 < bands) {
                        rowOut[j] = make_int2(sUp, fUp);
                        if (!seq && (j & (kRowChunk - 1)) == kRowChunk - 1) st_release_gpu(&st->progress, j + 1);
                    }
                }
            }
            const int j = t - lane;
            // Fill and drain steps (some lane outside [1, m - 1]); the same for the whole warp.
            const bool edge = t < 32 || t >= m;
            if (b > 0 && (t & (kRowChunk - 1)) == 0 && t <= m) {
                // Stage chunk t of the band above, then prefetch chunk t + 32.
                __syncwarp();
                rb[lane] = pre;
                __syncwarp();
                if (t + kRowChunk <= m) fetch(t + kRowChunk);
            }
            const int inS = __shfl_up_sync(0xffffffffu, outS, 1);
            const int inF = __shfl_up_sync(0xffffffffu, outF, 1);
            const int hc = hnext;
            hnext = H[edge ? min(max(j, 0), m - 1) : j];      // column j + 1 at the next step
            // S and F of the row above this strip, column j (lane 0: row 0 or the band above).
            int2 bb;
            if (b == 0) {
                // Row 0: Zero at (0, 0) and with a free first row, else Horizontal.  Lane 0's
                // values; the other lanes' copies go unused.
                uint8_t tv0 = TV_NONE;
                if (t >= 1 && !fTop) {
                    if (AFFINE) {
                        const int ex = e0 + EXT, op = s0 + OPEN;
                        tv0 = ex < op ? (TV_HO | TV_MFH) : (TV_H | TV_MFH);
                        e0 = max(ex, op);
                        s0 = e0;
                    } else {
                        s0 = s0 + EXT;
                        tv0 = TV_H | TV_MFH;
                    }
                }
                if (lane == 0 && t <= m) {
                    if (TRACE) T[t] = tv0;
                    if (!LOCAL && t == m && fRight && t > 0) best.offer_later(s0, fTop ? INF : e0, INF, t, 0);
                }
                bb = make_int2(s0, INF);
            } else {
                bb = rb[j & (kRowChunk - 1)];
            }
            int sUp = lane ? inS : bb.x;
            int fUp = lane ? inF : bb.y;
            uint32_t tw[R / 4];
            if (edge && j == 0) {
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
                int diag = diagNext;
                diagNext = sUp;
                const int hrow = MATRIX ? ((hc & 31) << 5) : hc;
                int Fp[R];                                 // F of each row (for the best cell)
#pragma unroll
                for (int r = 0; r < R; ++r) {
                    const int sub = MATRIX ? smat[hrow | (vc[r] & 31)] : (hc == vc[r] ? a.match : a.mismatch);
                    const int inter = diag + sub;
                    diag = Sp[r];
                    int s, e = Ep[r], f = fUp;
                    uint32_t tv = 0;
                    if (AFFINE) {
                        const int eExt = Ep[r] + EXT, eOpn = Sp[r] + OPEN;
                        e = max(eExt, eOpn);
                        const int fExt = fUp + EXT;
                        f = __viaddmax_s32(sUp, OPEN, fExt);
                        s = LOCAL ? __vimax3_s32_relu(inter, e, f) : __vimax3_s32(inter, e, f);
                        if (TRACE) {
                            // s == inter: the diagonal wins (ties included); e != eExt: the gap
                            // opened (eExt < eOpn); f != fExt: likewise for F.  With the local
                            // zero floor, s == 0 overrides everything below.
                            tv = s == inter ? TV_DIAG : (f < e ? TV_MFH : TV_MFV);
                            tv |= e != eExt ? TV_HO : TV_H;
                            tv |= f != fExt ? TV_VO : TV_V;
                        }
                    } else {
                        const int gv = sUp + EXT, gh = Sp[r] + EXT;
                        s = LOCAL ? __vimax3_s32_relu(inter, gv, gh) : __vimax3_s32(inter, gv, gh);
                        if (TRACE)
                            tv = s == inter ? TV_DIAG : (gv < gh ? (TV_H | TV_MFH) : (TV_V | TV_MFV));
                    }
                    if (TRACE && LOCAL && s == 0) tv = TV_NONE;
                    Sp[r] = s;
                    Ep[r] = e;
                    Fp[r] = f;
                    sUp = s;
                    fUp = f;
                    if (TRACE) {
                        if ((r & 3) == 0) tw[r >> 2] = 0;
                        tw[r >> 2] |= tv << (8 * (r & 3));
                    }
                }
                // Best cells of column j (1 <= j <= m) in column-major order.
                if (!edge || (j >= 1 && j <= m)) {
                    if (LOCAL) {
                        // The first row holding the strip's maximum, taken only when it beats
                        // every earlier column.
                        if (rvalid >= R) {
                            const int mx = strip_max<R>(Sp);
                            if (mx > best.s) {
#pragma unroll
                                for (int r = 0; r < R; ++r)
                                    if (Sp[r] == mx) {
                                        best.offer_later(Sp[r], Ep[r], Fp[r], j, i0 + r);
                                        break;
                                    }
                            }
                        } else {
#pragma unroll
                            for (int r = 0; r < R; ++r)
                                if (r < rvalid) best.offer_later(Sp[r], Ep[r], Fp[r], j, i0 + r);
                        }
                    } else if (edge && j == m && (fRight || rowN >= 0)) {
                        // Last column: every row with a free last column, else row n only.
#pragma unroll
                        for (int r = 0; r < R; ++r)
                            if (r < rvalid && (fRight || r == rowN)) best.offer_later(Sp[r], Ep[r], Fp[r], j, i0 + r);
                    } else if (trackRowN) {
#pragma unroll
                        for (int r = 0; r < R; ++r)
                            if (r == rowN) best.offer_later(Sp[r], Ep[r], Fp[r], j, i0 + r);
                    }
                }
            }
            if (TRACE) store_trace<R>(Tband + int64_t(t) * 32 * R, tw);
            outS = sUp;
            outF = fUp;
            if (lane == 31 && b + 1 < bands && (!edge || (j >= 0 && j <= m))) {
                rowOut[j] = make_int2(sUp, fUp);
                if (!seq && ((j & (kRowChunk - 1)) == kRowChunk - 1 || j == m)) st_release_gpu(&st->progress, j + 1);
            }
        }
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
    if (bands > 1 && seq) {
        // One warp runs all bands of the pair in order: combine in registers.
        if (lane == 0) carry.offer(best.s, best.e, best.f, best.col, best.row);
        if (b + 1 < bands) return;
        best = carry;
    } else if (bands > 1) {
        // Chain the bands' best cells in band order.
        if (b > 0) {
            warp_wait_at_least(&st[-1].done, 1, a.error);
            if (lane == 0) {
                const BandState *q = st - 1;
                best.offer(__ldcg(&q->s), __ldcg(&q->e), __ldcg(&q->f), __ldcg(&q->col), __ldcg(&q->row));
            }
        }
        if (b + 1 < bands) {
            if (lane == 0) {
                st->s = best.s;
                st->e = best.e;
                st->f = best.f;
                st->col = best.col;
                st->row = best.row;
                st_release_gpu(&st->done, 1);
            }
            return;
        }
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
__global__ void __launch_bounds__(128, 4) k_dp_warp(WarpArgs a)
// R: rows per lane of full bands; a short last band runs with R / 2.
{
    extern __shared__ int smat[];
    if (MATRIX) {
        for (int i = threadIdx.x; i < 32 * 32; i += blockDim.x) {
            const int r = i >> 5, c = i & 31;
            smat[i] = (r < a.alphabet && c < a.alphabet) ? a.matrix[r * a.alphabet + c] : 0;
        }
        __syncthreads();
    }
    __shared__ int2 rbuf[4][kRowChunk];
    static_assert(kRowChunk == 32, "one row-buffer entry per lane");
    const int lane = threadIdx.x & 31;
    int2 *rb = rbuf[(threadIdx.x >> 5) & 3];
    for (;;) {
        int task = 0;
        if (lane == 0) task = atomicAdd(a.task_counter, 1);
        task = __shfl_sync(0xffffffffu, task, 0);
        if (task >= a.num_tasks) break;
        const int2 pb = a.tasks[task];
        const PairDesc d = a.pairs[pb.x];
        const int bands = (d.n + 32 * R - 1) / (32 * R);
        const bool halfLast = warp_last_rows(d.n, R) < R;
        WarpBest carry{d.inf, d.inf, d.inf, 0, 0};
        auto run = [&](int b, bool seq) {
            if (halfLast && b == bands - 1)
                warp_band<AFFINE, LOCAL, MATRIX, TRACE, R, R / 2>(a, smat, rb, pb.x, b, lane, seq, carry);
            else
                warp_band<AFFINE, LOCAL, MATRIX, TRACE, R, R>(a, smat, rb, pb.x, b, lane, seq, carry);
        };
        if (pb.y >= 0) {
            run(pb.y, false);
        } else {
            // Band -1: this warp runs every band of the pair in order (no waits between bands).
            for (int b = 0; b < bands; ++b) {
                run(b, true);
                __syncwarp();
            }
        }
        __syncwarp();
    }
}

}  // namespace gba
