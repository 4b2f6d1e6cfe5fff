// dp_kernels.cuh -- one-pair-per-thread DP kernels (inter-pair parallelism).
//
// Each thread owns one pair and sweeps its DP matrix in horizontal strips of STRIP_ROWS
// rows of V.  Inside a strip the thread walks the columns of H left to right with the
// strip's S and E values in registers; the bottom row of the strip (S, F) is passed to the
// next strip through a per-warp interleaved boundary buffer in global memory, so a warp
// reads and writes 256 contiguous bytes per column.
//
// The recurrences, their tie rules and the per-cell directions follow the reference's
// column-major DP exactly (align/dp_formula_affine.h:66-330, align/dp_formula_linear.h:62-258,
// align/dp_meta_info.h:178-221).  The visiting order differs (strips), so the best-cell
// search compares (column, row) on equal scores to return the cell the reference's
// column-major scout with strict '>' finds (align/dp_scout.h:166-180).
#pragma once

#include "dp_common.cuh"

namespace gba {

template <bool LOCAL>
struct Scout {
    int s, e, f, col, row;
    __device__ __forceinline__ void init(int inf)
    {
        s = inf; e = inf; f = inf; col = 0; row = 0;
    }
    __device__ __forceinline__ void offer(int cs, int ce, int cf, int ccol, int crow)
    {
        if (cs >= s) {
            if (cs > s || ccol < col || (ccol == col && crow < row)) {
                s = cs; e = ce; f = cf; col = ccol; row = crow;
            }
        }
    }
};

template <bool MATRIX>
__device__ __forceinline__ int sub_score(const DpArgs &a, const int *smat, int hc, int vc)
{
    // The table is staged as 32 x 32 with zero padding; masking keeps every index in bounds.
    if (MATRIX) return smat[((hc & 31) << 5) | (vc & 31)];
    return hc == vc ? a.match : a.mismatch;
}

template <bool AFFINE, bool LOCAL, bool MATRIX, bool TRACE>
__global__ void __launch_bounds__(128) k_dp_strip(DpArgs a)
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
    if (p < 0) return;   // padding slot (per-bucket launches start on a warp boundary)
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
    const int OPEN = AFFINE ? a.gap_open : a.gap_extend;
    const int EXT = a.gap_extend;

    Scout<LOCAL> best;
    best.init(INF);

    // ---- Row 0: Zero at (0,0); Horizontal or Zero (free first row) elsewhere.
    {
        int s = 0, e = INF;
        bnd[0] = make_int2(0, INF);
        if (TRACE) T[0] = TV_NONE;
        if (LOCAL) best.offer(0, INF, INF, 0, 0);
        for (int j = 1; j <= m; ++j) {
            uint8_t tv = TV_NONE;
            if (!fTop) {
                if (AFFINE) {
                    int ext = e + EXT, opn = s + OPEN;
                    if (ext < opn) { e = opn; tv = TV_HO | TV_MFH; } else { e = ext; tv = TV_H | TV_MFH; }
                    s = e;
                } else {
                    s = s + EXT;
                    tv = TV_H | TV_MFH;
                }
            }
            bnd[int64_t(j) * 32] = make_int2(s, INF);
            if (TRACE) T[j] = tv;
            if (LOCAL || (j == m && fRight)) best.offer(s, fTop ? INF : e, INF, j, 0);
        }
    }

    // ---- Strips of rows 1..n.
    const int64_t row0Bytes = align16(m + 1);
    for (int i0 = 1, strip = 0; i0 <= n; i0 += STRIP_ROWS, ++strip) {
        uint8_t vc[STRIP_ROWS];
#pragma unroll
        for (int r = 0; r < STRIP_ROWS; ++r) vc[r] = (i0 + r <= n) ? V[i0 + r - 1] : 0;
        int Sp[STRIP_ROWS], Ep[STRIP_ROWS];
        uint32_t tw[STRIP_ROWS / 4];
        const bool lastStrip = (i0 + STRIP_ROWS > n);

        // Column 0: Vertical, or Zero with a free first column.
        int diagNext;
        {
            int2 up = bnd[0];
            int sUp = up.x, fUp = up.y;
            diagNext = sUp;
#pragma unroll
            for (int r = 0; r < STRIP_ROWS; ++r) {
                const int i = i0 + r;
                uint8_t tv = TV_NONE;
                int s, f = fUp;
                if (fLeft) {
                    s = 0;
                } else if (AFFINE) {
                    int ext = fUp + EXT, opn = sUp + OPEN;
                    if (ext < opn) { f = opn; tv = TV_VO | TV_MFV; } else { f = ext; tv = TV_V | TV_MFV; }
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
            bnd[0] = make_int2(sUp, fUp);
            if (TRACE)
                *reinterpret_cast<uint4 *>(T + row0Bytes + (int64_t(strip) * (m + 1)) * STRIP_ROWS) =
                    make_uint4(tw[0], tw[1], tw[2], tw[3]);
        }

        // Columns 1..m: every cell uses all three directions.
        for (int j = 1; j <= m; ++j) {
            const int hc = H[j - 1];
            int2 up = bnd[int64_t(j) * 32];
            int sUp = up.x, fUp = up.y;
            int diag = diagNext;
            diagNext = sUp;
            const bool trackCol = LOCAL || (j == m && fRight);
#pragma unroll
            for (int r = 0; r < STRIP_ROWS; ++r) {
                const int inter = diag + sub_score<MATRIX>(a, smat, hc, vc[r]);
                diag = Sp[r];
                int s, e = Ep[r], f = fUp;
                uint8_t tv;
                if (AFFINE) {
                    uint8_t tvE, tvF, tm;
                    int eExt = Ep[r] + EXT, eOpn = Sp[r] + OPEN;
                    if (eExt < eOpn) { e = eOpn; tvE = TV_HO; } else { e = eExt; tvE = TV_H; }
                    int fExt = fUp + EXT, fOpn = sUp + OPEN;
                    if (fExt < fOpn) { f = fOpn; tvF = TV_VO; } else { f = fExt; tvF = TV_V; }
                    int g;
                    if (f < e) { g = e; tm = TV_MFH; } else { g = f; tm = TV_MFV; }
                    if (inter < g) { s = g; tv = tm | tvE | tvF; } else { s = inter; tv = TV_DIAG | tvE | tvF; }
                } else {
                    int gv = sUp + EXT, gh = Sp[r] + EXT;
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
            bnd[int64_t(j) * 32] = make_int2(sUp, fUp);
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
