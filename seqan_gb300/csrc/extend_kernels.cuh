// extend_kernels.cuh -- the DP of extendAlignment (align_extend/align_extend.h:115-206): the
// AlignExtend_ profile (align_extend/align_extend_base.h) -- a gap-initialised first row and
// column, every cell tracked, no zero floor -- with the optional X-drop terminator
// (align_extend/dp_scout_xdrop.h), and its traceback to the origin.
//
// A group of W lanes (W = 8, 16 or 32; 32 / W groups per warp) per extension task (one side of
// one alignment), column-synchronous: lane L of the group owns rows 8L..8L+7 of each 8W-row band,
// and a column is finished by all lanes before the next starts,
// so the column maximum (the X-drop rule) and the first maximum in column-major order (the
// scout) are exact at every column and the DP stops exactly where the reference stops.  The
// vertical gap chain of a column is a max-plus prefix scan: with X_i the best of the diagonal and
// horizontal candidates of row i,
//     affine:  F_{i+1} = max(F_i + max(ext, open), X_i + open),  S_i = max(X_i, F_i)
//     linear:  S_i     = max(X_i, S_{i-1} + ext)
// (max(F + ext, max(X, F) + open) = max(F + max(ext, open), X + open)), so each lane folds its
// 8 rows, the group scans the lane aggregates with log2(W) shuffles, and each lane replays its
// rows.  Groups of one warp run different tasks; their shuffles and ballots use the group's lanes
// only, so a group that finishes a task fetches the next while the others continue.
// Trace bits follow the reference's comparisons cell by cell (align/dp_formula_affine.h:66-125,
// dp_formula_linear.h:62-106, the left operand winning ties).  Scores are int (the reference's
// TScoreValue for Score<int, ...>); "infinity" is -2^30 (align/dp_cell.h:143-146).
#pragma once

#include <cstdint>
#include <climits>

namespace gba {

constexpr int kExtRows = 8;                    // rows per lane
constexpr int kExtInf = -(1 << 30);

enum : uint8_t { XT_DIAG = 1, XT_H = 2, XT_V = 4, XT_HO = 8, XT_VO = 16, XT_MFH = 32, XT_MFV = 64 };

struct ExtTask {
    const uint8_t *h;          // residue of column j (1..m): h[hstep * j]
    const uint8_t *v;          // residue of row i (1..n): v[vstep * i]
    int32_t m, n, hstep, vstep;
    int32_t col_limit;         // trace pass: the last column the score pass computed
    int32_t pad;
    int64_t trace_off;         // trace pass: the task's column-major trace, column stride round8(n + 1)
};

struct ExtOut {                // the best cell (first maximum in column-major order) and its E, F
    int32_t score, col, row, e, f;
    int32_t last_col;          // the last column computed
    int32_t pad[2];
};

struct ExtArgs {
    const ExtTask *tasks;
    ExtOut *out;
    int32_t num_tasks;
    int32_t *next;             // work counter
    int32_t match, mismatch, gap_open, gap_extend;
    const int32_t *matrix;     // alphabet^2 table (row = H residue) or null
    int32_t asize;
    int32_t xdrop_on, xdrop;
    uint8_t *trace;
    int32_t *scratch;          // per group: 2 * (max n + 1) ints (tasks with more than one band)
    int64_t scratch_stride;
};

__host__ __device__ inline int ext_trace_stride(int n) { return (n + 1 + 7) & ~7; }

struct ExtSegment {
    uint32_t h_begin, v_begin, length, type;
};

template <bool MATRIX>
__device__ __forceinline__ int ext_sub(const ExtArgs &a, const int32_t *smat, int hc, int vc)
{
    if (MATRIX) return smat[hc * a.asize + vc];
    return hc == vc ? a.match : a.mismatch;
}

template <bool AFFINE, bool MATRIX, bool TRACE, int W>
__global__ void __launch_bounds__(128) k_extend_dp(ExtArgs a)
{
    __shared__ int32_t smat[32 * 32];
    if (MATRIX) {
        for (int t = threadIdx.x; t < a.asize * a.asize; t += blockDim.x) smat[t] = a.matrix[t];
    }
    __syncthreads();
    constexpr int kExtBand = W * kExtRows;             // rows per band
    const int lane = threadIdx.x & (W - 1);            // lane within the group
    const unsigned FULL = W == 32 ? 0xffffffffu : (((1u << W) - 1u) << ((threadIdx.x & 31) & ~(W - 1)));
    const int group_global = (blockIdx.x * blockDim.x + threadIdx.x) / W;
    int32_t *const scr = a.scratch ? a.scratch + (size_t)group_global * a.scratch_stride : nullptr;
    const int open = a.gap_open, ext = a.gap_extend;
    const int g = AFFINE ? max(ext, open) : ext;       // the vertical chain's per-row step
    const int g8 = kExtRows * g;

    for (;;) {
        int t = 0;
        if (lane == 0) t = atomicAdd(a.next, 1);
        t = __shfl_sync(FULL, t, 0, W);
        if (t >= a.num_tasks) break;
        const ExtTask tk = a.tasks[t];
        const int m = tk.m, n = tk.n;
        const int nb = (n + 1 + kExtBand - 1) / kExtBand;
        const int limit = TRACE ? tk.col_limit : m;
        const int nt = ext_trace_stride(n);
        uint8_t *const tr = TRACE ? a.trace + tk.trace_off : nullptr;
        int Sp[kExtRows], Ep[kExtRows];     // previous column, this lane's rows of the current band
        int vc[kExtRows];
#pragma unroll
        for (int r = 0; r < kExtRows; ++r) {
            Sp[r] = kExtInf;
            Ep[r] = kExtInf;
        }
        int bestS = kExtInf, bestC = 0, bestR = 0, bestE = kExtInf, bestF = kExtInf;
        bool flag = false;
        int lastCol = limit;
        int hnext = limit >= 1 ? tk.h[tk.hstep] : 0;   // column residues are loaded one column ahead
        for (int j = 0; j <= limit; ++j) {
            const int hc = j > 0 ? hnext : 0;
            if (j >= 1 && j < limit) hnext = tk.h[tk.hstep * (j + 1)];
            int bandF = kExtInf;        // affine: F of the band's first row; linear: S of the row above it
            int bandDiag = kExtInf;     // previous column's S of the row above the band
            int colMax = INT_MIN, cbS = INT_MIN, cbR = 0, cbE = 0, cbF = 0;
            int aboveF = kExtInf, aboveS = kExtInf;   // final F, S of the row above the band (this column)
            for (int b = 0; b < nb; ++b) {
                const int r0 = b * kExtBand + lane * kExtRows;
                if (nb > 1) {
#pragma unroll
                    for (int r = 0; r < kExtRows; ++r) {
                        const int i = r0 + r;
                        Sp[r] = (j > 0 && i <= n) ? scr[i] : kExtInf;
                        Ep[r] = (j > 0 && i <= n) ? scr[n + 1 + i] : kExtInf;
                    }
                }
                if (nb > 1 || j == 0) {
#pragma unroll
                    for (int r = 0; r < kExtRows; ++r) {
                        const int i = r0 + r;
                        vc[r] = (i >= 1 && i <= n) ? tk.v[tk.vstep * i] : 0;
                    }
                }
                // previous column's S of the row above each of this lane's rows
                int up = __shfl_up_sync(FULL, Sp[kExtRows - 1], 1, W);
                if (lane == 0) up = bandDiag;
                const int lastOld = __shfl_sync(FULL, Sp[kExtRows - 1], W - 1, W);
                // X (best of diagonal and horizontal), E and their bits
                int X[kExtRows], E[kExtRows];
                uint8_t bits[kExtRows];
#pragma unroll
                for (int r = 0; r < kExtRows; ++r) {
                    const int i = r0 + r;
                    const int dS = r == 0 ? up : Sp[r - 1];
                    int x, e = Ep[r];
                    uint8_t bt = 0;
                    if (j == 0) {
                        x = (i == 0) ? 0 : kExtInf;           // zero cell, then the vertical column
                        if (i > 0) e = kExtInf;
                    } else if (i == 0) {                       // first row: horizontal
                        if (AFFINE) {
                            const int a1 = Ep[r] + ext, a2 = Sp[r] + open;
                            e = a1 < a2 ? a2 : a1;
                            bt = (a1 < a2 ? XT_HO : XT_H) | XT_MFH;
                            x = e;
                        } else {
                            x = Sp[r] + ext;
                            bt = XT_H | XT_MFH;
                        }
                    } else {
                        const int inter = dS + ext_sub<MATRIX>(a, smat, hc, vc[r]);
                        if (AFFINE) {
                            const int a1 = Ep[r] + ext, a2 = Sp[r] + open;
                            e = a1 < a2 ? a2 : a1;
                            bt = a1 < a2 ? XT_HO : XT_H;
                            x = max(inter, e);
                        } else {
                            x = max(inter, Sp[r] + ext);
                        }
                    }
                    X[r] = x;
                    E[r] = e;
                    bits[r] = bt;
                }
                // lane aggregate of the vertical chain and the exclusive scan over lanes
                int agg = INT_MIN / 2;
#pragma unroll
                for (int r = 0; r < kExtRows; ++r) {
                    const int contrib = AFFINE ? X[r] + open : X[r];
                    agg = max(agg + g, contrib);
                }
                // agg = max_r (contrib_r + (7 - r) g): the chain value one past the lane's last row
                // (affine F) or at its last row (linear S) when nothing enters from above.
                int bnorm = agg - lane * g8;
                int pre = bnorm;
#pragma unroll
                for (int o = 1; o < W; o <<= 1) {
                    const int q = __shfl_up_sync(FULL, pre, o, W);
                    if (lane >= o) pre = max(pre, q);
                }
                int excl = __shfl_up_sync(FULL, pre, 1, W);
                int in = bandF + lane * g8;               // what enters the band's first row, carried down
                if (lane > 0) in = max(in, excl + (lane - 1) * g8);
                // replay the lane's rows
                int S[kExtRows], F[kExtRows];
                if (AFFINE) {
                    int f = in;                             // F of row r0
#pragma unroll
                    for (int r = 0; r < kExtRows; ++r) {
                        F[r] = f;
                        S[r] = max(X[r], f);
                        f = max(f + g, X[r] + open);
                    }
                } else {
                    int sa = in;                            // S of the row above row r0
#pragma unroll
                    for (int r = 0; r < kExtRows; ++r) {
                        S[r] = max(X[r], sa + ext);
                        F[r] = kExtInf;
                        sa = S[r];
                    }
                }
                // the row above each row, final values of this column (for the trace bits)
                int upF = __shfl_up_sync(FULL, F[kExtRows - 1], 1, W);
                int upS = __shfl_up_sync(FULL, S[kExtRows - 1], 1, W);
                if (lane == 0) {
                    upF = aboveF;
                    upS = aboveS;
                }
                if (TRACE) {
#pragma unroll
                    for (int r = 0; r < kExtRows; ++r) {
                        const int i = r0 + r;
                        const int pF = r == 0 ? upF : F[r - 1];
                        const int pS = r == 0 ? upS : S[r - 1];
                        uint8_t bt = bits[r];
                        if (j == 0) {
                            if (i > 0) {
                                if (AFFINE) bt = ((pF + ext < pS + open) ? XT_VO : XT_V) | XT_MFV;
                                else bt = XT_V | XT_MFV;
                            }
                        } else if (i > 0) {
                            const int inter = (r == 0 ? up : Sp[r - 1]) + ext_sub<MATRIX>(a, smat, hc, vc[r]);
                            if (AFFINE) {
                                bt |= (pF + ext < pS + open) ? XT_VO : XT_V;
                                const int f = F[r], e = E[r];
                                const uint8_t t2 = f < e ? XT_MFH : XT_MFV;
                                const int s1 = f < e ? e : f;
                                bt |= inter < s1 ? t2 : XT_DIAG;
                            } else {
                                const int vv = pS + ext, hh = Sp[r] + ext;
                                const uint8_t t1 = vv < hh ? (XT_H | XT_MFH) : (XT_V | XT_MFV);
                                const int s1 = vv < hh ? hh : vv;
                                bt = inter < s1 ? t1 : XT_DIAG;
                            }
                        }
                        bits[r] = bt;
                    }
                    if (r0 <= n) {
                        uint2 w;
                        w.x = bits[0] | (bits[1] << 8) | (bits[2] << 16) | ((uint32_t)bits[3] << 24);
                        w.y = bits[4] | (bits[5] << 8) | (bits[6] << 16) | ((uint32_t)bits[7] << 24);
                        *reinterpret_cast<uint2 *>(tr + (size_t)j * nt + r0) = w;
                    }
                }
                // column statistics over this band: maximum, first row holding it, its E and F
                int lmax = INT_MIN, lrow = 0, le = 0, lf = 0;
#pragma unroll
                for (int r = 0; r < kExtRows; ++r) {
                    const int i = r0 + r;
                    if (i <= n && S[r] > lmax) {
                        lmax = S[r];
                        lrow = i;
                        le = E[r];
                        lf = AFFINE ? F[r] : kExtInf;
                    }
                }
                int wmax = lmax;
#pragma unroll
                for (int o = W / 2; o > 0; o >>= 1) wmax = max(wmax, __shfl_xor_sync(FULL, wmax, o, W));
                const unsigned holders = __ballot_sync(FULL, lmax == wmax && lmax != INT_MIN) & FULL;
                if (holders) {
                    const int src = (__ffs(holders) - 1) & (W - 1);
                    const int brow = __shfl_sync(FULL, lrow, src, W);
                    const int be = __shfl_sync(FULL, le, src, W);
                    const int bf = __shfl_sync(FULL, lf, src, W);
                    if (wmax > cbS) {       // earlier bands keep ties (smaller rows)
                        cbS = wmax;
                        cbR = brow;
                        cbE = be;
                        cbF = bf;
                    }
                    colMax = max(colMax, wmax);
                }
                // carries into the next band
                bandDiag = lastOld;
                if (AFFINE) {
                    const int fNext = max(F[kExtRows - 1] + g, X[kExtRows - 1] + open);
                    bandF = __shfl_sync(FULL, fNext, W - 1, W);
                } else {
                    bandF = __shfl_sync(FULL, S[kExtRows - 1], W - 1, W);
                }
                aboveF = __shfl_sync(FULL, F[kExtRows - 1], W - 1, W);
                aboveS = __shfl_sync(FULL, S[kExtRows - 1], W - 1, W);
#pragma unroll
                for (int r = 0; r < kExtRows; ++r) {
                    Sp[r] = S[r];
                    Ep[r] = E[r];
                }
                if (nb > 1) {
#pragma unroll
                    for (int r = 0; r < kExtRows; ++r) {
                        const int i = r0 + r;
                        if (i <= n) {
                            scr[i] = S[r];
                            scr[n + 1 + i] = E[r];
                        }
                    }
                    __syncwarp(FULL);
                }
            }
            // the scout: first maximum in column-major order
            if (cbS > bestS) {
                bestS = cbS;
                bestC = j;
                bestR = cbR;
                bestE = cbE;
                bestF = cbF;
            }
            // the X-drop terminator: flag at the column's end, tested after inner columns
            if (!TRACE && a.xdrop_on) {
                if (bestS - colMax >= a.xdrop) flag = true;
                if (flag && j >= 1 && j < m) {
                    lastCol = j;
                    break;
                }
            }
        }
        if (lane == 0) {
            ExtOut o;
            o.score = bestS;
            o.col = bestC;
            o.row = bestR;
            o.e = bestE;
            o.f = bestF;
            o.last_col = lastCol;
            o.pad[0] = o.pad[1] = 0;
            a.out[t] = o;
        }
        __syncwarp(FULL);
    }
}

// Copies each task's segments from its traceback slot to the packed output (one thread per task).
__global__ void __launch_bounds__(128) k_extend_pack(const ExtSegment *slots, const int64_t *slot_off,
                                                     const int32_t *count, const int64_t *packed_off,
                                                     ExtSegment *packed, int num_tasks)
{
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= num_tasks) return;
    const int c = count[t];
    const ExtSegment *src = slots + slot_off[t];
    ExtSegment *dst = packed + packed_off[t];
    for (int q = 0; q < c; ++q) dst[q] = src[q];
}

// Traceback of one task from its best cell to the origin (align/dp_traceback_impl.h:190-546 with
// the AlignExtend_ profile: TraceTail_ false, TraceHead_ true), one thread per task.  Segments in
// traceback order (last = alignment begin) go to segs[seg_off[t] ...]; seg_count[t] gets their
// number (-1 if the slot was too small).
__device__ inline void ext_record(ExtSegment *s, int cap, int &cnt, int hb, int vb, int len, int tv)
{
    if (len == 0) return;
    int type;
    if (tv & XT_DIAG) type = 1;
    else if (tv & XT_V) type = 4;
    else if (tv & XT_H) type = 2;
    else return;
    if (cnt >= cap) {
        cnt = cap + 1;
        return;
    }
    s[cnt++] = ExtSegment{(uint32_t)hb, (uint32_t)vb, (uint32_t)len, (uint32_t)type};
}

template <bool AFFINE>
__global__ void __launch_bounds__(128) k_extend_traceback(const ExtTask *tasks, const ExtOut *outs, int num_tasks,
                                                          const uint8_t *trace, ExtSegment *segs,
                                                          const int64_t *seg_off, int32_t *seg_count)
{
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= num_tasks) return;
    const ExtTask tk = tasks[t];
    const ExtOut o = outs[t];
    const int nt = ext_trace_stride(tk.n);
    const uint8_t *T = trace + tk.trace_off;
    ExtSegment *s = segs + seg_off[t];
    const int cap = (int)(seg_off[t + 1] - seg_off[t]);
    int cnt = 0;
    int col = o.col, row = o.row;
    int tv = T[(size_t)col * nt + row];
    // _correctTraceValue (align/dp_algorithm_impl.h:1188-1205), affine only
    if (AFFINE) {
        if (o.f == o.score) tv = (tv & ~XT_DIAG) | XT_MFV;
        else if (o.e == o.score) tv = (tv & ~XT_DIAG) | XT_MFH;
    }
    int last;
    if (AFFINE) {
        if (tv & XT_MFV) {
            tv &= (XT_V | XT_VO | XT_MFV);
            last = XT_V;
        } else if (tv & XT_MFH) {
            tv &= (XT_H | XT_HO | XT_MFH);
            last = XT_H;
        } else {
            last = XT_DIAG;
        }
    } else {
        if (tv & XT_DIAG) last = XT_DIAG;
        else if (tv & (XT_V | XT_MFV)) last = XT_V;
        else if (tv & (XT_H | XT_MFH)) last = XT_H;
        else last = 0;
    }
    int frag = 0;
#define XTAT(cc, rr) T[(size_t)(cc) * nt + (rr)]
    while (!(col <= 0 || row <= 0) && tv != 0) {
        if (tv & XT_DIAG) {
            if (!(last & XT_DIAG)) {
                ext_record(s, cap, cnt, col, row, frag, last);
                last = XT_DIAG;
                frag = 0;
            }
            --col;
            --row;
            tv = XTAT(col, row);
            ++frag;
        } else if ((tv & XT_MFV) && (tv & XT_V)) {
            if (!(last & XT_V)) {
                ext_record(s, cap, cnt, col, row, frag, last);
                last = XT_V;
                frag = 0;
            }
            if (AFFINE) {
                while ((!(tv & XT_VO) || (tv & XT_V)) && row != 1) {
                    --row;
                    tv = XTAT(col, row);
                    ++frag;
                }
            }
            --row;
            tv = XTAT(col, row);
            ++frag;
        } else if ((tv & XT_MFV) && (tv & XT_VO)) {
            if (!(last & XT_V)) {
                ext_record(s, cap, cnt, col, row, frag, last);
                last = XT_V;
                frag = 0;
            }
            --row;
            tv = XTAT(col, row);
            ++frag;
        } else if ((tv & XT_MFH) && (tv & XT_H)) {
            if (!(last & XT_H)) {
                ext_record(s, cap, cnt, col, row, frag, last);
                last = XT_H;
                frag = 0;
            }
            if (AFFINE) {
                while ((!(tv & XT_HO) || (tv & XT_H)) && col != 1) {
                    --col;
                    tv = XTAT(col, row);
                    ++frag;
                }
            }
            --col;
            tv = XTAT(col, row);
            ++frag;
        } else if ((tv & XT_MFH) && (tv & XT_HO)) {
            if (!(last & XT_H)) {
                ext_record(s, cap, cnt, col, row, frag, last);
                last = XT_H;
                frag = 0;
            }
            --col;
            tv = XTAT(col, row);
            ++frag;
        } else {
            break;
        }
    }
#undef XTAT
    ext_record(s, cap, cnt, col, row, frag, last);
    // TraceHead_ (:538-545)
    if (row != 0) ext_record(s, cap, cnt, 0, 0, row, XT_V);
    if (col != 0) ext_record(s, cap, cnt, 0, 0, col, XT_H);
    seg_count[t] = cnt > cap ? -1 : cnt;
}

}  // namespace gba
