// dp_dynamic_kernels.cuh -- DP with DynamicGaps cells, one pair per thread.
//
// The reference's third gap-cost model (align/dp_cell_dynamic.h, align/dp_formula_dynamic.h): a cell
// holds one score and two flags saying whether its best path ends in a vertical or a horizontal gap.
// A gap from a neighbour is extended (gap_extend) when the neighbour's flag for that direction is set
// and opened (gap_open) otherwise; there are no separate E / F matrices.  Per inner cell:
//   tmp = S_left + (flagH(left) ? ext : open)         trace H or H_OPEN
//   act = S_up + (flagV(up) ? ext : open)             trace V or V_OPEN
//   act < tmp ? (act = tmp, flags = H, MAX_FROM_H) : (flags = V, MAX_FROM_V)
//   act <= diag + sub ? (S = diag + sub, flags = 0, DIAGONAL | gap bits) : (S = act, gap bits | max bit)
//   local: S <= 0 becomes 0 with trace NONE (flags kept)
// Row 0 cells are horizontal gaps (flag H) and column 0 cells vertical gaps (flag V) unless that side
// is free (Zero cells: score 0, no flags).  Tracked cells and the first-maximum rule are those of the
// other kernels (align/dp_meta_info.h:178-221, align/dp_scout.h:166-180); the best cell's flags go to
// best_e for the start-cell correction of the traceback (align/dp_algorithm_impl.h:1235-1249).
//
// Layout: the one-pair-per-thread strips of dp_kernels.cuh -- STRIP_ROWS rows in registers, the strip's
// bottom row (S, flags) in the per-warp interleaved boundary buffer, the trace in the strip layout
// (trace_at), so the common traceback kernel reads it.
#pragma once

#include "dp_common.cuh"
#include "dp_kernels.cuh"

namespace gba {

constexpr int DYN_FLAG_V = 1, DYN_FLAG_H = 2;   // MASK_VERTICAL_GAP, MASK_HORIZONTAL_GAP

template <bool LOCAL, bool MATRIX, bool TRACE>
__global__ void __launch_bounds__(128) k_dp_dynamic(DpArgs a)
{
    extern __shared__ int smat[];
    if (MATRIX) {
        for (int i = threadIdx.x; i < 32 * 32; i += blockDim.x) {
            const int r = i >> 5, c = i & 31;
            smat[i] = (r < a.alphabet && c < a.alphabet) ? a.matrix[r * a.alphabet + c] : 0;
        }
        __syncthreads();
    }
    const int64_t slot = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (slot >= a.num_slots) return;
    const int p = a.order[slot];
    if (p < 0) return;
    const PairDesc d = a.pairs[p];
    const int m = d.m, n = d.n;
    const int INF = d.inf;
    const uint8_t *H = a.seq_h + d.h_off;
    const uint8_t *V = a.seq_v + d.v_off;
    int2 *bnd = a.scratch + a.warp_scratch[slot >> 5] + (slot & 31);
    uint8_t *T = TRACE ? a.trace + d.trace_off : nullptr;

    const int fe = LOCAL ? (FREE_TOP | FREE_LEFT | FREE_RIGHT | FREE_BOTTOM) : a.free_ends;
    const bool fTop = fe & FREE_TOP, fLeft = fe & FREE_LEFT;
    const bool fRight = fe & FREE_RIGHT, fBottom = fe & FREE_BOTTOM;
    const int OPEN = a.gap_open, EXT = a.gap_extend;

    // best.e carries the best cell's flags.
    Scout<LOCAL> best;
    best.init(INF);

    // ---- Row 0: Zero at (0, 0); horizontal gaps, or Zero cells with a free first row.
    {
        int s = 0, fl = 0;
        bnd[0] = make_int2(0, 0);
        if (TRACE) T[0] = TV_NONE;
        if (LOCAL) best.offer(0, 0, INF, 0, 0);
        for (int j = 1; j <= m; ++j) {
            uint8_t tv = TV_NONE;
            if (!fTop) {
                if (fl & DYN_FLAG_H) { s += EXT; tv = TV_H | TV_MFH; }
                else { s += OPEN; tv = TV_HO | TV_MFH; }
                fl = DYN_FLAG_H;
            }
            bnd[int64_t(j) * 32] = make_int2(s, fl);
            if (TRACE) T[j] = tv;
            if (LOCAL || (j == m && fRight)) best.offer(s, fl, INF, j, 0);
        }
    }

    // ---- Strips of rows 1..n.
    const int64_t row0Bytes = align16(m + 1);
    for (int i0 = 1, strip = 0; i0 <= n; i0 += STRIP_ROWS, ++strip) {
        uint8_t vc[STRIP_ROWS];
#pragma unroll
        for (int r = 0; r < STRIP_ROWS; ++r) vc[r] = (i0 + r <= n) ? V[i0 + r - 1] : 0;
        int Sp[STRIP_ROWS], Fl[STRIP_ROWS];
        uint32_t tw[STRIP_ROWS / 4];
        const bool lastStrip = (i0 + STRIP_ROWS > n);

        // Column 0: vertical gaps, or Zero cells with a free first column.
        int diagNext;
        {
            const int2 up = bnd[0];
            int sUp = up.x, flUp = up.y;
            diagNext = sUp;
#pragma unroll
            for (int r = 0; r < STRIP_ROWS; ++r) {
                const int i = i0 + r;
                uint8_t tv = TV_NONE;
                int s = 0, fl = 0;
                if (!fLeft) {
                    if (flUp & DYN_FLAG_V) { s = sUp + EXT; tv = TV_V | TV_MFV; }
                    else { s = sUp + OPEN; tv = TV_VO | TV_MFV; }
                    fl = DYN_FLAG_V;
                }
                Sp[r] = s;
                Fl[r] = fl;
                sUp = s;
                flUp = fl;
                if (TRACE) {
                    if ((r & 3) == 0) tw[r >> 2] = 0;
                    tw[r >> 2] |= uint32_t(tv) << (8 * (r & 3));
                }
                if (i <= n && (LOCAL || (i == n && fBottom))) best.offer(s, fl, INF, 0, i);
            }
            bnd[0] = make_int2(sUp, flUp);
            if (TRACE)
                *reinterpret_cast<uint4 *>(T + row0Bytes + (int64_t(strip) * (m + 1)) * STRIP_ROWS) =
                    make_uint4(tw[0], tw[1], tw[2], tw[3]);
        }

        // Columns 1..m.
        for (int j = 1; j <= m; ++j) {
            const int hc = H[j - 1];
            const int2 up = bnd[int64_t(j) * 32];
            int sUp = up.x, flUp = up.y;
            int diag = diagNext;
            diagNext = sUp;
            const bool trackCol = LOCAL || (j == m && fRight);
#pragma unroll
            for (int r = 0; r < STRIP_ROWS; ++r) {
                const int inter = diag + sub_score<MATRIX>(a, smat, hc, vc[r]);
                diag = Sp[r];
                int tmp, act, fl;
                uint8_t tvG, tm, tv;
                if (Fl[r] & DYN_FLAG_H) { tmp = Sp[r] + EXT; tvG = TV_H; }
                else { tmp = Sp[r] + OPEN; tvG = TV_HO; }
                if (flUp & DYN_FLAG_V) { act = sUp + EXT; tvG |= TV_V; }
                else { act = sUp + OPEN; tvG |= TV_VO; }
                if (act < tmp) { act = tmp; fl = DYN_FLAG_H; tm = TV_MFH; }
                else { fl = DYN_FLAG_V; tm = TV_MFV; }
                if (act <= inter) { act = inter; fl = 0; tv = TV_DIAG | tvG; }
                else tv = tvG | tm;
                if (LOCAL && !(0 < act)) { act = 0; tv = TV_NONE; }
                Sp[r] = act;
                Fl[r] = fl;
                sUp = act;
                flUp = fl;
                if (TRACE) {
                    if ((r & 3) == 0) tw[r >> 2] = 0;
                    tw[r >> 2] |= uint32_t(tv) << (8 * (r & 3));
                }
                if (!lastStrip || i0 + r <= n) {
                    if (trackCol || (lastStrip && i0 + r == n && (j == m || fBottom)))
                        best.offer(act, fl, INF, j, i0 + r);
                }
            }
            bnd[int64_t(j) * 32] = make_int2(sUp, flUp);
            if (TRACE)
                *reinterpret_cast<uint4 *>(T + row0Bytes + (int64_t(strip) * (m + 1) + j) * STRIP_ROWS) =
                    make_uint4(tw[0], tw[1], tw[2], tw[3]);
        }
    }

    a.score[p] = best.s;
    if (a.end_h) a.end_h[p] = best.col;
    if (a.end_v) a.end_v[p] = best.row;
    if (a.best_e) a.best_e[p] = best.e;
    if (a.best_f) a.best_f[p] = best.f;
}

}  // namespace gba
