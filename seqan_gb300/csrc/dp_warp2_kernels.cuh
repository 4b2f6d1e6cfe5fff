// dp_warp2_kernels.cuh -- packed 16-bit warp bands: 64 strips per warp, 4-bit trace.
//
// For pairs whose every cell value stays inside the exact int16 range (the bound the engine uses
// to honour 16-bit cells), one warp computes a band of 64 strips of R rows (R = 4: 256 rows) of
// one pair.  Lane l owns strip l in the low 16-bit halves of its registers and strip 32 + l in the
// high halves, so every max/add instruction advances two cells (DPX __viaddmax_s16x2 and
// __vimax_s16x2_relu, __vimax3_s16x2, __vimin3_u16x2).  The strips form an anti-diagonal front:
// at step t the low half of lane l
// is at column t - l and the high half at column t - l - 32; each step lane l receives the bottom
// row (S, F) of lane l - 1 by one rotating shuffle, and lane 0's high half receives lane 31's low
// half (strip 31 is the strip above strip 32).  A band therefore takes m + 64 steps.  The bottom
// row of a band (strip 63: lane 31, high half) goes to the next band through global memory.  Most
// pairs run their bands in order on one warp with a one-row buffer (column c is read by the next
// band at its step c and overwritten by it at step c + 63); a pair of many bands instead runs them
// as separate tasks on different warps at the same time, band b following band b - 1 through a
// two-slot row buffer and a progress counter (bounded waits, as in the 32-bit warp kernel), which
// cuts the pair's critical path from bands x (m + 64) steps to about m + 64 + 96 x (bands - 1).
// The last band of a pair holds 64 strips of R = 2 rows when its rows fit (128 rows).
//
// Recurrences, tie rules and tracked cells are the reference's (align/dp_formula_affine.h:66-330,
// align/dp_formula_linear.h:62-258, align/dp_meta_info.h:178-221, align/dp_scout.h:166-180), in
// the max / add-max form whose values equal the compare-and-select ones, ties included:
//   E = max(E_left + ext, S_left + open)   (extend wins ties)
//   F = max(F_up + ext, S_up + open)       (extend wins ties)
//   G = max(E, F), S = max(diag + sub, G)  (F wins ties against E, the diagonal against G)
// and for linear gaps G = max(S_left + g, S_up + g) (vertical wins ties).  Local mode floors S at 0.
//
// Trace: 4 bits per cell -- the TraceBitMap_ byte of the reference (align/dp_profile.h:121-135)
// reduced to what _doTraceback reads (align/dp_traceback_impl.h:376-450): the source of S (none,
// diagonal, MAX_FROM_V, MAX_FROM_H) and one open/extend bit for E and for F.  The oracle checks
// (tests/test_trace4_oracle.py) that this code gives the reference's traceback on every
// configuration.  Bits per cell, each a 0/1 computed for both halves at once:
//   nd = S != diag + sub, h = G != F (E > F), eo = E != E_left + ext, fo = F != F_up + ext
//   none = (local and S == 0) or (free first column and column 0)
//   b0 = nd & ~none, b1 = (nd & h) | none:  (b1, b0) = 00 DIAG, 01 MAX_FROM_V, 11 MAX_FROM_H, 10 NONE
// stored as bit planes: in the word of one lane and step, the half of strip s holds b0 of its R
// rows in bits 0..R-1, b1 in R..2R-1, eo in 2R..3R-1 and fo in 3R..4R-1 (low half strip l, high
// half strip 32 + l).  Row 0 is stored as TraceBitMap_ bytes, as in the other layouts.
#pragma once

#include "dp_common.cuh"
#include "dp16x2_kernels.cuh"
#include "dp_warp_kernels.cuh"

#include <type_traits>

namespace gba {

constexpr int kW2Rows = 4;                    // rows per half-strip of a full band
constexpr int kW2BandRows = 64 * kW2Rows;     // 256 rows per full band

// Rows per half-strip of the last band of an n-row pair (2 or 4).
__host__ __device__ inline int warp2_last_rows(int n)
{
    const int rem = n - ((n - 1) / kW2BandRows) * kW2BandRows;
    return rem <= 128 ? 2 : 4;
}

__host__ __device__ inline int64_t warp2_band_off(int m, int b)
{
    return align16(m + 1) + int64_t(b) * (m + 64) * 32 * kW2Rows;
}

// Trace bytes of one pair: row 0 (m + 1 bytes, padded), then per band (m + 64) steps x 32 lanes x
// R bytes (R rows x 2 halves x 4 bits).
__host__ __device__ inline int64_t warp2_trace_bytes(int m, int n)
{
    if (n <= 0) return align16(m + 1);
    const int bands = (n + kW2BandRows - 1) / kW2BandRows;
    return warp2_band_off(m, bands - 1) + int64_t(m + 64) * 32 * warp2_last_rows(n);
}

// TraceBitMap_ byte of cell (col, row) from the 4-bit planes.
__device__ __forceinline__ uint8_t trace_at_warp2(const uint8_t *base, int m, int n, bool affine, int col, int row)
{
    if (row == 0) return base[col];
    const int r0 = row - 1;
    const int b = r0 / kW2BandRows;
    const int Rb = (b == (n - 1) / kW2BandRows) ? warp2_last_rows(n) : kW2Rows;
    const int within = r0 - b * kW2BandRows;
    const int s = within / Rb, r = within - s * Rb;
    const int lane = s & 31, h = s >> 5;
    const int t = col + lane + 32 * h;
    const uint8_t *w = base + warp2_band_off(m, b) + (int64_t(t) * 32 + lane) * Rb;
    const uint32_t word = Rb == 4 ? *reinterpret_cast<const uint32_t *>(w)
                                  : (Rb == 2 ? uint32_t(*reinterpret_cast<const uint16_t *>(w)) : uint32_t(*w));
    const int sh = h * 4 * Rb + r;
    const int b0 = (word >> sh) & 1, b1 = (word >> (sh + Rb)) & 1;
    const int eo = (word >> (sh + 2 * Rb)) & 1, fo = (word >> (sh + 3 * Rb)) & 1;
    if (b1 && !b0) return TV_NONE;
    if (!affine) return !b0 ? TV_DIAG : (b1 ? (TV_H | TV_MFH) : (TV_V | TV_MFV));
    const int src = !b0 ? TV_DIAG : (b1 ? TV_MFH : TV_MFV);
    return uint8_t(src | (eo ? TV_HO : TV_H) | (fo ? TV_VO : TV_V));
}

struct Warp2Args {
    const uint8_t *seq_h;
    const uint8_t *seq_v;
    const PairDesc *pairs;
    const int2 *tasks;             // (pair, band): band -1 = all bands of the pair in order on one warp
    uint32_t *rowbuf;              // per multi-band pair at rowbuf_off[p] (uint32): 1 (in order) or 2
                                   // (pipelined) slots of m + 1 packed (S, F)
    const int64_t *rowbuf_off;
    BandState *bands;              // pipelined pairs at band_base[p]: one per band (zeroed per run)
    const int64_t *band_base;
    int32_t *error;                // set to 1 when a wait between bands ran out
    uint8_t *trace;
    int32_t *score, *end_h, *end_v, *best_e, *best_f;
    const int32_t *matrix;
    int32_t *task_counter;
    int32_t num_tasks;
    int32_t match, mismatch, gap_open, gap_extend;
    int32_t free_ends;
    int32_t alphabet;
};

// Best cell of one half-strip (column-major first maximum).
struct Best1 {
    int s, e, f, col, row;
    __device__ __forceinline__ void offer(int cs, int ce, int cf, int ccol, int crow)
    {
        if (cs >= s && (cs > s || ccol < col || (ccol == col && crow < row))) {
            s = cs; e = ce; f = cf; col = ccol; row = crow;
        }
    }
    // For candidates that arrive in column-major order: a later cell wins only with a higher score.
    __device__ __forceinline__ void offer_later(int cs, int ce, int cf, int ccol, int crow)
    {
        if (cs > s) { s = cs; e = ce; f = cf; col = ccol; row = crow; }
    }
};

__device__ __forceinline__ uint32_t w2_sel(uint32_t x, uint32_t mask, uint32_t y)
{
    return (x & ~mask) | (y & mask);   // one LOP3
}

// 0/1 per half: a != b (one XOR and one DPX 3-way minimum).
__device__ __forceinline__ uint32_t w2_ne(uint32_t a, uint32_t b)
{
    return __vimin3_u16x2(a ^ b, 0x00010001u, 0x00010001u);
}

// Packed signed 16-bit maximum as a DPX 3-way maximum.
__device__ __forceinline__ uint32_t w2_max(uint32_t a, uint32_t b)
{
    return __vimax3_s16x2(a, b, b);
}

// S(0, j) of row 0 (Horizontal gaps, or Zero with a free first row); E(0, j) equals it for j >= 1.
__device__ __forceinline__ int w2_row0(int j, bool fTop, bool affine, int open, int ext)
{
    if (fTop || j == 0) return 0;
    return affine ? open + (j - 1) * max(ext, open) : j * ext;
}

// Per-lane state of one band: lane l holds strip l (low halves) and strip 32 + l (high halves).
template <bool AFFINE, bool LOCAL, bool MATRIX, bool TRACE, int R>
struct W2Lane {
    uint32_t vsel[R];              // !MATRIX: PRMT selectors of the two halves' row codes
    int vlo[R], vhi[R];            // MATRIX: row codes of the low / high strip
    uint32_t rowmask[R];           // 0xffff in the halves whose row r lies inside the matrix
    bool partial;                  // some row of this lane lies beyond n
    int i0lo, i0hi;                // first rows of the two strips
    int rowNlo, rowNhi;            // index of row n in each strip, or -1
    uint32_t Sp[R], Ep[R], Fp[R];
    uint32_t diagNext, outS, outF, hcode;
    uint32_t bestS2;               // bl.s and bh.s packed (LOCAL)
    Best1 bl, bh;

    // One step t.  EDGE: some half may be at column 0 or outside [1, m - 1] (fill and drain).
    template <bool EDGE>
    __device__ __forceinline__ void step(const int *smat, int t, int lane, int m, int n, uint32_t above,
                                         const uint8_t *H, uint32_t *tstore, uint32_t T0, uint32_t T1,
                                         uint32_t OPEN2, uint32_t EXT2, bool fLeft, bool fRight, bool fBottom)
    {
        const uint32_t NEG2 = 0x80008000u, INF2 = pack2(-16384, -16384), ONE2 = 0x00010001u;
        // Hand-off: lane l takes lane l - 1's bottom row; lane 0 takes the row above the band (low
        // half) and lane 31's low half (high half).  Column codes rotate the same way.
        const uint32_t rotS = __shfl_sync(0xffffffffu, outS, (lane + 31) & 31);
        const uint32_t rotF = __shfl_sync(0xffffffffu, outF, (lane + 31) & 31);
        const uint32_t rotH = __shfl_sync(0xffffffffu, hcode, (lane + 31) & 31);
        uint32_t sUp = lane ? rotS : prmt(above, rotS, 0x5410);
        uint32_t fUp = lane ? rotF : prmt(above, rotF, 0x5432);
        const uint32_t hcur = hcode;
        {
            const int c = H[min(t, m - 1)];
            const uint32_t hnew = MATRIX ? uint32_t((c & 31) << 5) : uint32_t((c & 7) * 0x11u);
            hcode = lane ? rotH : (MATRIX ? prmt(hnew, rotH, 0x5410) : prmt(hnew, rotH, 0x1140));
        }
        const int jlo = t - lane, jhi = jlo - 32;
        uint32_t m0 = 0, none0 = 0;     // halves at column 0; those whose column-0 cells are NONE
        if (EDGE) {
            m0 = (jlo == 0 ? 0x0000ffffu : 0u) | (jhi == 0 ? 0xffff0000u : 0u);
            if (fLeft || LOCAL) none0 = m0 & ONE2;
        }
        uint32_t diag = diagNext;
        diagNext = sUp;
        const int hrlo = int(hcur & 0xffffu), hrhi = int(hcur >> 16);
        uint32_t acc = 0;
#pragma unroll
        for (int r = 0; r < R; ++r) {
            uint32_t sub;
            if (MATRIX) sub = prmt(uint32_t(smat[hrlo + vlo[r]]), uint32_t(smat[hrhi + vhi[r]]), 0x5410);
            else sub = prmt(T0, T1, hcur ^ vsel[r]);
            uint32_t inter = __viaddmax_s16x2(diag, sub, NEG2);
            if (EDGE) inter = w2_sel(inter, m0, NEG2);
            diag = Sp[r];
            uint32_t s, g, e = 0, f, eExt = 0, fExt = 0, gv = 0;
            if (AFFINE) {
                eExt = __viaddmax_s16x2(Ep[r], EXT2, NEG2);
                e = __viaddmax_s16x2(Sp[r], OPEN2, eExt);
                if (EDGE) {
                    eExt = w2_sel(eExt, m0, INF2);
                    e = w2_sel(e, m0, INF2);
                }
                fExt = __viaddmax_s16x2(fUp, EXT2, NEG2);
                f = __viaddmax_s16x2(sUp, OPEN2, fExt);
                g = w2_max(e, f);
            } else {
                gv = __viaddmax_s16x2(sUp, EXT2, NEG2);
                g = __viaddmax_s16x2(Sp[r], EXT2, gv);
                if (EDGE) g = w2_sel(g, m0, gv);          // column 0: vertical only
                f = gv;
            }
            s = LOCAL ? __vimax_s16x2_relu(inter, g) : w2_max(inter, g);
            if (EDGE && (LOCAL || fLeft)) {
                s = s & ~m0;                               // Zero cells of a free first column
                if (AFFINE) f = w2_sel(f, m0, fUp);        // F passes through unchanged
            }
            if (TRACE) {
                const uint32_t nd = w2_ne(s, inter);
                const uint32_t h = AFFINE ? w2_ne(g, f) : w2_ne(g, gv);
                uint32_t none = 0;
                if (LOCAL) none = w2_ne(s, 0u) ^ ONE2;
                if (EDGE) none |= none0;
                acc += (nd & ~none) << r;
                acc += ((nd & h) | none) << (R + r);
                if (AFFINE) {
                    acc += w2_ne(e, eExt) << (2 * R + r);
                    acc += w2_ne(f, fExt) << (3 * R + r);
                }
            }
            Sp[r] = s;
            if (AFFINE) Ep[r] = e;
            Fp[r] = f;
            sUp = s;
            fUp = f;
        }
        if (TRACE) {
            if (R == 4) tstore[0] = acc;
            else if (R == 2) *reinterpret_cast<uint16_t *>(tstore) = uint16_t(prmt(acc, 0u, 0x4420));
            else *reinterpret_cast<uint8_t *>(tstore) = uint8_t((acc | (acc >> 12)) & 0xffu);
        }
        outS = sUp;
        outF = fUp;

        // Tracked cells.
        if (LOCAL) {
            uint32_t mx;
            if (partial) {
                mx = w2_sel(NEG2, rowmask[0], Sp[0]);
#pragma unroll
                for (int r = 1; r < R; ++r) mx = w2_max(mx, w2_sel(NEG2, rowmask[r], Sp[r]));
            } else if (R == 4) {
                mx = __vimax3_s16x2(__vimax3_s16x2(Sp[0], Sp[1 % R], Sp[2 % R]), Sp[3 % R], Sp[3 % R]);
            } else if (R == 2) {
                mx = w2_max(Sp[0], Sp[1 % R]);
            } else {
                mx = Sp[0];
            }
            if (EDGE) {
                const uint32_t vmask = (jlo >= 1 && jlo <= m ? 0x0000ffffu : 0u) | (jhi >= 1 && jhi <= m ? 0xffff0000u : 0u);
                mx = w2_sel(NEG2, vmask, mx);
            }
            if (w2_max(mx, bestS2) != bestS2) {
                // The first row holding each half's maximum, with its E and F, found for both halves
                // at once (bottom up, so the first matching row is the last one selected).
                uint32_t ridx = 0, es = 0, fs = 0;
#pragma unroll
                for (int r = R - 1; r >= 0; --r) {
                    uint32_t eq = (w2_ne(Sp[r], mx) ^ ONE2) * 0xffffu;
                    if (partial) eq &= rowmask[r];
                    ridx = w2_sel(ridx, eq, uint32_t(r) * ONE2);
                    es = w2_sel(es, eq, Ep[r]);
                    fs = w2_sel(fs, eq, Fp[r]);
                }
                const int mlo = lo16(mx), mhi = hi16(mx);
                if (mlo > bl.s) bl.offer_later(mlo, lo16(es), lo16(fs), jlo, i0lo + int(ridx & 0xffffu));
                if (mhi > bh.s) bh.offer_later(mhi, hi16(es), hi16(fs), jhi, i0hi + int(ridx >> 16));
                bestS2 = pack2(bl.s, bh.s);
            }
        } else {
            // Global: the last column (every row with a free last column, else row n) and, with a
            // free last row, row n of every column (column 0 included).
            const bool lastLo = jlo == m, lastHi = jhi == m;
            if (lastLo || lastHi || (fBottom && (rowNlo >= 0 || rowNhi >= 0))) {
#pragma unroll
                for (int r = 0; r < R; ++r) {
                    if (jlo >= 0 && jlo <= m && i0lo + r <= n &&
                        ((lastLo && (fRight || r == rowNlo)) || (fBottom && r == rowNlo)))
                        bl.offer_later(lo16(Sp[r]), jlo == 0 ? -16384 : lo16(Ep[r]), lo16(Fp[r]), jlo, i0lo + r);
                    if (jhi >= 0 && jhi <= m && i0hi + r <= n &&
                        ((lastHi && (fRight || r == rowNhi)) || (fBottom && r == rowNhi)))
                        bh.offer_later(hi16(Sp[r]), jhi == 0 ? -16384 : hi16(Ep[r]), hi16(Fp[r]), jhi, i0hi + r);
                }
            }
        }
    }
};

// Band b of pair p (all lanes).  RB: rows per half-strip of this band.  seq: the pair's bands run
// in order on this warp (best cell carried in `carry`); else this band is a pipelined task.
template <bool AFFINE, bool LOCAL, bool MATRIX, bool TRACE, int RB>
__device__ __forceinline__ void warp2_band(const Warp2Args &a, const int *smat, int p, int b, int lane, bool seq,
                                        Best1 &carry)
{
    const PairDesc d = a.pairs[p];
    const int m = d.m, n = d.n;
    const int bands = (n + kW2BandRows - 1) / kW2BandRows;
    const uint8_t *H = a.seq_h + d.h_off;
    const uint8_t *V = a.seq_v + d.v_off;
    uint8_t *T = TRACE ? a.trace + d.trace_off : nullptr;
    const int fe = LOCAL ? (FREE_TOP | FREE_LEFT | FREE_RIGHT | FREE_BOTTOM) : a.free_ends;
    const bool fTop = fe & FREE_TOP, fLeft = fe & FREE_LEFT;
    const bool fRight = fe & FREE_RIGHT, fBottom = fe & FREE_BOTTOM;
    const int OPEN = AFFINE ? a.gap_open : a.gap_extend;
    const int EXT = a.gap_extend;
    const uint32_t OPEN2 = pack2(OPEN, OPEN), EXT2 = pack2(EXT, EXT);
    const uint32_t T0 = (uint32_t(a.match) & 0xffu) | ((uint32_t(a.mismatch) & 0xffu) * 0x01010100u);
    const uint32_t T1 = (uint32_t(a.mismatch) & 0xffu) * 0x01010101u;
    const int INF = -16384;
    const uint32_t INF2 = pack2(INF, INF);

    W2Lane<AFFINE, LOCAL, MATRIX, TRACE, RB> w;
    const int rowBase = b * kW2BandRows;
    w.i0lo = rowBase + lane * RB + 1;
    w.i0hi = rowBase + (32 + lane) * RB + 1;
    w.partial = w.i0hi + RB - 1 > n;       // the high strip ends last
    w.rowNlo = (n >= w.i0lo && n < w.i0lo + RB) ? n - w.i0lo : -1;
    w.rowNhi = (n >= w.i0hi && n < w.i0hi + RB) ? n - w.i0hi : -1;
#pragma unroll
    for (int r = 0; r < RB; ++r) {
        const bool inlo = w.i0lo + r <= n, inhi = w.i0hi + r <= n;
        const int clo = inlo ? V[w.i0lo + r - 1] : 0;
        const int chi = inhi ? V[w.i0hi + r - 1] : 0;
        if (MATRIX) {
            w.vlo[r] = clo & 31;
            w.vhi[r] = chi & 31;
        } else {
            w.vsel[r] = vsel_of(uint32_t(clo & 7) | (uint32_t(chi & 7) << 4));
        }
        w.rowmask[r] = (inlo ? 0x0000ffffu : 0u) | (inhi ? 0xffff0000u : 0u);
        w.Sp[r] = INF2;
        w.Ep[r] = INF2;
        w.Fp[r] = INF2;
    }
    w.diagNext = INF2;
    w.outS = INF2;
    w.outF = INF2;
    w.hcode = 0;
    w.bl = Best1{INF, INF, INF, 0, 0};
    w.bh = Best1{INF, INF, INF, 0, 0};
    Best1 row0{INF, INF, INF, 0, 0};       // candidates of row 0 (not in column-major order here)
    if (b == 0) {
        if (LOCAL && lane == 0) row0.offer(0, INF, INF, 0, 0);
        if (!LOCAL && fRight && lane == 0)
            row0.offer(w2_row0(m, fTop, AFFINE, OPEN, EXT), fTop ? INF : w2_row0(m, fTop, AFFINE, OPEN, EXT), INF, m, 0);
        if (TRACE) {
            // Row 0: Zero at (0, 0) and with a free first row, else Horizontal (open at column 1).
            for (int c = lane; c <= m; c += 32) {
                uint8_t tv = TV_NONE;
                if (c >= 1 && !fTop)
                    tv = AFFINE ? ((c == 1 || EXT < OPEN) ? (TV_HO | TV_MFH) : (TV_H | TV_MFH)) : (TV_H | TV_MFH);
                T[c] = tv;
            }
        }
    }
    w.bestS2 = pack2(w.bl.s, w.bh.s);

    // Row buffers.  In order: one slot, read and rewritten in place.  Pipelined: band b writes slot
    // b & 1 and reads slot (b - 1) & 1 after band b - 1 has published the columns.
    uint32_t *rowOut = nullptr;
    const uint32_t *rowIn = nullptr;
    BandState *st = nullptr;
    if (bands > 1) {
        uint32_t *base = a.rowbuf + a.rowbuf_off[p];
        if (seq) {
            rowOut = base;
            rowIn = base;
        } else {
            rowOut = base + int64_t(b & 1) * (m + 1);
            rowIn = base + int64_t((b + 1) & 1) * (m + 1);
            st = a.bands + a.band_base[p] + b;
        }
    }
    uint32_t pre = 0, preNext = 0;          // columns 32c + lane of the row above, chunks c and c + 1
    if (b > 0) {
        if (!seq) warp_wait_at_least(&st[-1].progress, min(64, m + 1), a.error);
        if (lane <= m) pre = __ldcg(rowIn + lane);
        if (32 + lane <= m) preNext = __ldcg(rowIn + 32 + lane);
    }
    uint8_t *Tb = TRACE ? T + warp2_band_off(m, b) + int64_t(lane) * RB : nullptr;
    const bool publish = b + 1 < bands && lane == 31;
    const int last = m + 63;

#define GBA_W2_STEP(EDGE)                                                                               \
    do {                                                                                                \
        uint32_t above;                                                                                 \
        if (b == 0) {                                                                                   \
            above = pack2(w2_row0(t, fTop, AFFINE, OPEN, EXT), INF);                                    \
        } else {                                                                                        \
            above = __shfl_sync(0xffffffffu, pre, t & 31);                                              \
            if ((t & 31) == 31) {                                                                       \
                pre = preNext;                                                                          \
                const int c0 = t + 33;                                                                  \
                if (!seq && c0 <= m) warp_wait_at_least(&st[-1].progress, min(c0 + 32, m + 1), a.error); \
                preNext = c0 + lane <= m ? __ldcg(rowIn + c0 + lane) : 0u;                              \
            }                                                                                           \
        }                                                                                               \
        w.template step<EDGE>(smat, t, lane, m, n, above, H,                                            \
                              TRACE ? reinterpret_cast<uint32_t *>(Tb + int64_t(t) * 32 * RB) : nullptr, T0, \
                              T1, OPEN2, EXT2, fLeft, fRight, fBottom);                                 \
        if (publish) {                                                                                  \
            const int jh = t - 63;                                                                      \
            if (jh >= 0 && jh <= m) {                                                                   \
                rowOut[jh] = prmt(w.outS, w.outF, 0x7632);                                              \
                if (!seq && ((jh & 31) == 31 || jh == m)) st_release_gpu(&st->progress, jh + 1);        \
            }                                                                                           \
        }                                                                                               \
    } while (0)

    // Steps 64 .. m - 1 have every half in columns 1 .. m - 1 (no column 0, no last column);
    // the fill and drain steps around them take the edge path.
    for (int t = 0; t <= last; ++t) {
        if (t >= 64 && t < m) GBA_W2_STEP(false);
        else GBA_W2_STEP(true);
    }
#undef GBA_W2_STEP

    // Combine this lane's candidates, then the warp's, in the reference's order.
    Best1 best = w.bl;
    best.offer(w.bh.s, w.bh.e, w.bh.f, w.bh.col, w.bh.row);
    best.offer(row0.s, row0.e, row0.f, row0.col, row0.row);
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

template <bool AFFINE, bool LOCAL, bool MATRIX, bool TRACE>
__global__ void __launch_bounds__(128, 6) k_dp_warp2(Warp2Args a)
{
    __shared__ int smat[MATRIX ? 32 * 32 : 1];
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
        const int2 pb = a.tasks[task];
        const PairDesc d = a.pairs[pb.x];
        const int bands = (d.n + kW2BandRows - 1) / kW2BandRows;
        const int rl = warp2_last_rows(d.n);
        Best1 carry{d.inf, d.inf, d.inf, 0, 0};
        const int b0 = pb.y < 0 ? 0 : pb.y, b1 = pb.y < 0 ? bands : pb.y + 1;
        for (int b = b0; b < b1; ++b) {
            const int rb = b + 1 < bands ? kW2Rows : rl;
            if (rb == 4) warp2_band<AFFINE, LOCAL, MATRIX, TRACE, 4>(a, smat, pb.x, b, lane, pb.y < 0, carry);
            else warp2_band<AFFINE, LOCAL, MATRIX, TRACE, 2>(a, smat, pb.x, b, lane, pb.y < 0, carry);
            __syncwarp();
        }
    }
}

}  // namespace gba
