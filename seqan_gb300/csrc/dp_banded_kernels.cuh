// dp_banded_kernels.cuh -- banded DP (DPBandConfig<BandOn>), one pair per thread.
//
// Follows the reference's banded column phases exactly (align/dp_algorithm_impl.h:586-967):
// an initial column, columns attached to the top of the matrix, middle or full columns,
// columns attached to the bottom, and the final column, each computed as a "track" of rows
// [r0, r1] whose first, inner and last cells take the recursion direction and tracking flag
// of DPMetaColumn_ (align/dp_meta_info.h:178-370); band width 1 runs the reference's
// diagonal-only path (:970-1110).  The extra best-cell offers at phase boundaries are made
// with the F value the reference's band storage holds for that cell (the column of the band is
// stored one slot per diagonal, so a slot keeps the F of the last tracked cell on its
// diagonal unless the call site refreshes it).
//
// XT: the AlignExtend_ profile of extendAlignment's banded overloads
// (align_extend/align_extend.h:137-206, align_extend/align_extend_base.h): global directions with a
// free last row and column, every cell tracked, no zero floor, and with xdrop_on the X-drop
// terminator (align_extend/dp_scout_xdrop.h:127-143): every offer raises the column maximum, an
// offer with IsLastRow (a track's last cell, and the reference's extra offers that pass it) ends
// the DP when best - column maximum >= xdrop and resets the maximum otherwise, and the DP stops
// at the reference's column checks (after the initial column and after each column of the three
// band phases, align/dp_algorithm_impl.h:746-836).
//
// Band state: per thread, slot k = upper - col + row (one per diagonal) of S, E and the stored
// F, in per-thread arrays (local memory).  Trace: for bands of at most kBandFastW diagonals the
// 4-bit trace code of each cell (trace4_encode: 0.5 byte per band slot per column, band4_pos),
// for wider bands one byte per band slot per column (the reference's TraceBitMap_ bits), columns
// band_trace_stride(W) = W rounded up to 16 bytes apart; both interleaved by lane per warp so a
// warp's column stores coalesce.
//
// Middle phase fast path: the columns whose track covers all W slots (first cell Upper, inner
// cells All, last cell Lower, every cell tracked in local mode and none otherwise) are most of
// a banded alignment.  For W <= kBandFastW they run with slots 0 .. W-2 in register arrays
// (static indices), the last slot in scalars, a window of V codes packed four per register
// and shifted one code per column, and the column's 4-bit trace codes packed into registers and
// written with one 16-byte store (and a 4-byte one for W > 32); the per-cell rules are the
// generic cell()'s, ties included.  (A form with every phase in register arrays was measured
// slower: its per-phase unrolled column code overflowed the instruction cache.)
#pragma once

#include "dp_common.cuh"

namespace gba {

struct BandArgs {
    const uint8_t *seq_h;
    const uint8_t *seq_v;
    const PairDesc *pairs;
    const int32_t *order;
    uint8_t *trace;                // per pair at PairDesc::trace_off: (m + 1) * W bytes
    int32_t *score, *end_h, *end_v, *best_e, *best_f;
    const int32_t *matrix;
    int64_t num_slots;
    int32_t match, mismatch, gap_open, gap_extend;
    int32_t free_ends;
    int32_t alphabet;
    int32_t lower, upper;
    int32_t xdrop_on, xdrop;       // XT instances only
};

constexpr int kBandFastW = 40;   // widest band of the middle-phase fast path

// Bytes of a trace column of a band of W slots (W rounded up to 16).
__host__ __device__ inline int band_trace_stride(int W) { return (W + 15) & ~15; }

// Banded trace layout, interleaved by lane: the 32 pairs of a warp share one region, in which
// 16-byte chunk q of column col of the pair in lane l lies at ((col * Wt / 16 + q) * 32 + l) * 16,
// so a warp writes a chunk of its 32 columns with one 512-byte store.  A pair's trace_off points
// at its lane's first chunk; relative to it, byte k of column col is at:
__host__ __device__ inline int64_t band_trace_pos(int Wt, int col, int k)
{
    return (int64_t(col) * (Wt >> 4) + (k >> 4)) * 512 + (k & 15);
}

// 4-bit banded trace (bands of at most kBandFastW diagonals): each column holds the pair's W
// trace4 codes, code k = band slot k, slots 0..31 in a 16-byte chunk and slots 32..39 in a 4-byte
// word.  Per warp region a column takes the 32 lanes' chunks (512 bytes) followed, for W > 32, by
// their words (128 bytes); regions start at multiples of 512 bytes, so a pair's lane is
// (trace_off >> 4) & 31.  Relative to trace_off (its lane's first chunk), the byte of slot k of
// column col is at:
__host__ __device__ inline bool band_trace4(int W) { return W <= kBandFastW; }
__host__ __device__ inline int band4_col_bytes(int W) { return W > 32 ? 640 : 512; }
__host__ __device__ inline int64_t band4_pos(int W, int lane, int col, int k)
{
    const int64_t c = int64_t(col) * band4_col_bytes(W);
    return k < 32 ? c + (k >> 1) : c + 512 - 12 * lane + ((k - 32) >> 1);
}

enum { BCOL_INITIAL = 0, BCOL_INNER = 1, BCOL_FINAL = 2 };
enum { BLOC_FULL = 0, BLOC_TOP = 1, BLOC_MIDDLE = 2, BLOC_BOTTOM = 3 };
enum { BDIR_ZERO = 0, BDIR_ALL, BDIR_HORIZONTAL, BDIR_VERTICAL, BDIR_UPPER, BDIR_LOWER };

template <bool AFFINE, bool LOCAL, bool MATRIX, bool TRACE, int WMAX, bool XT = false>
struct BandedPair {
    static constexpr bool TRK = LOCAL || XT;   // every cell tracked
    const BandArgs &a;
    const int *smat;
    const uint8_t *H, *V;
    uint8_t *T;
    int m, n, W, Wt, lower, upper, INF;
    int lane;          // the pair's lane in its trace region (4-bit layout)
    bool fTop, fLeft, fRight, fBottom;
    int OPEN, EXT;
    int S[WMAX], E[WMAX], Fs[WMAX];
    // caches of the current track
    int dS, vS, vF, lastF;
    // scout (strict '>' in the reference's visiting order)
    int bs, be, bf, bcol, brow;
    // X-drop terminator (XT)
    int colmax;
    bool term;

    __device__ BandedPair(const BandArgs &args, const int *sm) : a(args), smat(sm) {}

    __device__ __forceinline__ int sub(int col, int row) const
    {
        const int hc = H[col - 1], vc = V[row - 1];
        if (MATRIX) return smat[((hc & 31) << 5) | (vc & 31)];
        return hc == vc ? a.match : a.mismatch;
    }
    __device__ __forceinline__ void scout(int s, int e, int f, int col, int row)
    {
        if (s > bs) { bs = s; be = e; bf = f; bcol = col; brow = row; }
    }
    // An offer of the X-drop scout; last_row: the reference's IsLastRow (termination check).
    __device__ __forceinline__ void offer(int s, int e, int f, int col, int row, bool last_row)
    {
        scout(s, e, f, col, row);
        if (XT && a.xdrop_on) {
            colmax = max(colmax, s);
            if (last_row) {
                if (bs - colmax >= a.xdrop) term = true;
                else colmax = INT_MIN;
            }
        }
    }
    __device__ __forceinline__ int slot(int col, int row) const { return upper - col + row; }
    // One trace value: a byte, or its 4-bit code in the 4-bit layout (the other half of the byte
    // kept; each pair owns its bytes).
    __device__ __forceinline__ void put_trace(int col, int k, int tv)
    {
        if (band_trace4(W)) {
            uint8_t *b = T + band4_pos(W, lane, col, k);
            const uint32_t c = trace4_encode(uint32_t(tv));
            *b = uint8_t((k & 1) ? ((*b & 0x0fu) | (c << 4)) : ((*b & 0xf0u) | c));
        } else {
            T[band_trace_pos(Wt, col, k)] = uint8_t(tv);
        }
    }
    __device__ __forceinline__ bool in_slots(int k) const { return k >= 0 && k < W; }

    // One cell; the horizontal neighbour (row, col - 1) is slot k + 1 of the previous column,
    // which still holds it because slots are overwritten in increasing k within a column.
    __device__ void cell(int dir, int col, int row, bool tracked, bool last_row = false)
    {
        const int k = slot(col, row);
        const int hS = in_slots(k + 1) ? S[k + 1] : INF;
        const int hE = in_slots(k + 1) ? E[k + 1] : INF;
        const int eStored = in_slots(k) ? E[k] : INF;
        int s, e = INF, f = vF, tv = TV_NONE;
        switch (dir) {
        case BDIR_ZERO:
            s = 0;
            e = eStored;       // stays as stored
            dS = 0;
            vS = 0;
            f = vF;
            break;
        case BDIR_ALL: {
            const int inter = dS + sub(col, row);
            dS = hS;
            if (AFFINE) {
                int tE, tF, tm;
                if (hE + EXT < hS + OPEN) { e = hS + OPEN; tE = TV_HO; } else { e = hE + EXT; tE = TV_H; }
                if (vF + EXT < vS + OPEN) { f = vS + OPEN; tF = TV_VO; } else { f = vF + EXT; tF = TV_V; }
                int g;
                if (f < e) { g = e; tm = TV_MFH; } else { g = f; tm = TV_MFV; }
                if (inter < g) { s = g; tv = tm | tE | tF; } else { s = inter; tv = TV_DIAG | tE | tF; }
                vF = f;
            } else {
                const int gv = vS + EXT, gh = hS + EXT;
                int g, tg;
                if (gv < gh) { g = gh; tg = TV_H | TV_MFH; } else { g = gv; tg = TV_V | TV_MFV; }
                if (inter < g) { s = g; tv = tg; } else { s = inter; tv = TV_DIAG; }
                e = hE;
            }
            break;
        }
        case BDIR_HORIZONTAL:
            dS = hS;
            if (AFFINE) {
                if (hE + EXT < hS + OPEN) { e = hS + OPEN; tv = TV_HO | TV_MFH; } else { e = hE + EXT; tv = TV_H | TV_MFH; }
                vF = INF;
                f = INF;
                s = e;
            } else {
                s = hS + EXT;
                tv = TV_H | TV_MFH;
                e = hE;
            }
            break;
        case BDIR_VERTICAL:
            if (AFFINE) {
                if (vF + EXT < vS + OPEN) { f = vS + OPEN; tv = TV_VO | TV_MFV; } else { f = vF + EXT; tv = TV_V | TV_MFV; }
                vF = f;
                e = INF;
                s = f;
            } else {
                s = vS + EXT;
                tv = TV_V | TV_MFV;
                e = hE;
            }
            break;
        case BDIR_UPPER: {
            const int inter = dS + sub(col, row);
            dS = hS;
            if (AFFINE) {
                int tE;
                if (hE + EXT < hS + OPEN) { e = hS + OPEN; tE = TV_HO; } else { e = hE + EXT; tE = TV_H; }
                vF = INF;
                f = INF;
                if (inter < e) { s = e; tv = tE | TV_MFH; } else { s = inter; tv = tE | TV_DIAG; }
            } else {
                const int gh = hS + EXT;
                if (inter < gh) { s = gh; tv = TV_H | TV_MFH; } else { s = inter; tv = TV_DIAG; }
                e = hE;
            }
            break;
        }
        default: {  // BDIR_LOWER
            const int inter = dS + sub(col, row);
            if (AFFINE) {
                int tF;
                if (vF + EXT < vS + OPEN) { f = vS + OPEN; tF = TV_VO; } else { f = vF + EXT; tF = TV_V; }
                vF = f;
                e = INF;
                if (inter < f) { s = f; tv = tF | TV_MFV; } else { s = inter; tv = tF | TV_DIAG; }
            } else {
                const int gv = vS + EXT;
                if (inter < gv) { s = gv; tv = TV_V | TV_MFV; } else { s = inter; tv = TV_DIAG; }
                e = hE;
            }
            break;
        }
        }
        if (LOCAL && dir != BDIR_ZERO) {
            if (s <= 0) { s = 0; tv = TV_NONE; }
        }
        if (dir != BDIR_LOWER) vS = s;
        lastF = f;
        // Only the degenerate single-cell bands can produce a cell outside the band; it is
        // scouted but not stored.
        const bool inside = in_slots(k);
        if (inside) {
            S[k] = s;
            E[k] = e;
            if (TRACE) put_trace(col, k, tv);
        }
        if (tracked) {
            if (inside) Fs[k] = f;
            offer(s, e, f, col, row, last_row);
        }
    }

    // The reference's extra best-cell offers at phase boundaries (see the file comment).
    // last_row: the reference's call passes IsLastRow (an X-drop check in XT mode).
    __device__ void retrack(int col, int row, bool set_f, bool last_row = true)
    {
        const int k = slot(col, row);
        if (!in_slots(k)) {
            // A degenerate single-cell band whose one cell lies outside the band: the cell
            // just computed (direction Zero) is offered with its values.
            offer(0, INF, INF, col, row, last_row);
            return;
        }
        if (set_f) Fs[k] = lastF;
        offer(S[k], E[k], Fs[k], col, row, last_row);
    }

    // Middle-phase columns hIt + 1 .. hMid with every track covering slots 0 .. W - 1 (first
    // row in slot 0); advances hIt, vb and ve as the generic loop does.  Same per-cell rules as
    // cell(): Upper for slot 0, All for slots 1 .. W - 2, Lower for slot W - 1.
    __device__ void middle_fast(int &hIt, const int hMid, int &vb, int &ve)
    {
        constexpr int FW = kBandFastW;
        constexpr int NW = FW / 4;                    // V window words (4 codes each)
        constexpr int NT = (FW + 7) / 8;              // trace words of one column (8 codes each)
        static_assert(FW % 4 == 0, "whole window words");
        const int WL = W - 1;                         // register slots 0 .. W - 2
        int Sr[FW], Er[FW];
#pragma unroll
        for (int k = 0; k < FW - 1; ++k)
            if (k < WL) {
                Sr[k] = S[k];
                Er[k] = AFFINE ? E[k] : INF;
            }
        int sLast = S[WL], eLast = E[WL];
        // V window of the next column: code k = V[first row - 1 + k] (0 past the end of V).
        uint32_t vw[NW];
#pragma unroll
        for (int q = 0; q < NW; ++q) {
            uint32_t w = 0;
#pragma unroll
            for (int c = 0; c < 4; ++c) {
                const int idx = vb + 4 * q + c;
                w |= uint32_t(idx < n ? V[idx] : 0) << (8 * c);
            }
            vw[q] = w;
        }
        // Codes of the next column are loaded one column ahead (their latency hides behind a
        // column of W cells): H, the last row's V code and the window's incoming V code.
        int hcN = H[hIt];
        int vLowN = V[ve];                               // V[ve + 1 - 1] of the first fast column
        int vInN = (vb + FW < n) ? V[vb + FW] : 0;       // incoming window code after it
        for (; hIt != hMid; ++hIt) {
            ++vb;
            ++ve;
            const int col = hIt + 1;
            const int hc = hcN;
            const int vLow = vLowN;
            const int vIn = vInN;
            if (col < hMid) {
                hcN = H[col];
                vLowN = ve < n ? V[ve] : 0;
                vInN = (vb + FW < n) ? V[vb + FW] : 0;
            }
            const int hrow = MATRIX ? ((hc & 31) << 5) : hc;
            int dS = Sr[0];
            int vS = INF, vF = INF;
            uint32_t tw[NT];
#pragma unroll
            for (int q = 0; q < NT; ++q) tw[q] = 0;
#pragma unroll
            for (int k = 0; k < FW - 1; ++k) {
                if (k >= WL) break;
                const int vc = int((vw[k >> 2] >> (8 * (k & 3))) & 0xffu);
                const int sub = MATRIX ? smat[hrow | (vc & 31)] : (hc == vc ? a.match : a.mismatch);
                const int inter = dS + sub;
                const int hS = (k + 1 < WL) ? Sr[k + 1] : sLast;   // S(row, col - 1): slot k + 1
                const int hE = (k + 1 < WL) ? Er[k + 1] : eLast;
                dS = hS;
                int s, e, f = INF;
                uint32_t tv = 0;
                if (k == 0) {
                    // Upper: diagonal or horizontal.
                    if (AFFINE) {
                        const int eExt = hE + EXT, eOpn = hS + OPEN;
                        // DPX max with its comparison as a predicate: pe = eExt >= eOpn (the
                        // extension wins ties), pd = inter >= e (the diagonal wins ties)
                        bool pe, pd;
                        e = __vibmax_s32(eExt, eOpn, &pe);
                        s = __vibmax_s32(inter, e, &pd);
                        tv = (pe ? 0u : 4u) | (pd ? 1u : 3u);
                        vF = INF;
                    } else {
                        const int gh = hS + EXT;
                        s = max(inter, gh);
                        tv = inter < gh ? 3u : 1u;
                        e = hE;
                    }
                } else {
                    // All directions.
                    if (AFFINE) {
                        const int eExt = hE + EXT, eOpn = hS + OPEN;
                        const int fExt = vF + EXT, fOpn = vS + OPEN;
                        if (TRACE) {
                            // pe / pf: the extension wins; pfe: f >= e (vertical over
                            // horizontal); pd: inter >= max(e, f), i.e. s == inter
                            bool pe, pf, pfe, pd;
                            e = __vibmax_s32(eExt, eOpn, &pe);
                            f = __vibmax_s32(fExt, fOpn, &pf);
                            s = __vibmax_s32(inter, __vibmax_s32(f, e, &pfe), &pd);
                            tv = (pe ? 0u : 4u) | (pf ? 0u : 8u) | (pd ? 1u : (pfe ? 2u : 3u));
                        } else {
                            e = max(eExt, eOpn);
                            f = max(fExt, fOpn);
                            s = __vimax3_s32(inter, e, f);
                        }
                        vF = f;
                    } else {
                        const int gv = vS + EXT, gh = hS + EXT;
                        if (TRACE) {
                            bool pvh, pd;
                            s = __vibmax_s32(inter, __vibmax_s32(gv, gh, &pvh), &pd);
                            tv = pd ? 1u : (pvh ? 2u : 3u);
                        } else {
                            s = __vimax3_s32(inter, gv, gh);
                        }
                        e = hE;
                    }
                }
                if (LOCAL && s <= 0) {
                    s = 0;
                    tv = 0u;
                }
                vS = s;
                Sr[k] = s;
                if (AFFINE) Er[k] = e;
                if (TRACE) tw[k >> 3] |= tv << (4 * (k & 7));
                if (LOCAL) {
                    Fs[k] = f;
                    scout(s, e, f, col, vb + k);
                }
            }
            // Lower: diagonal or vertical (slot W - 1, row ve).
            {
                const int vc = vLow;
                const int sub = MATRIX ? smat[hrow | (vc & 31)] : (hc == vc ? a.match : a.mismatch);
                const int inter = dS + sub;
                int s, f = INF;
                uint32_t tv;
                if (AFFINE) {
                    const int fExt = vF + EXT, fOpn = vS + OPEN;
                    bool pf, pd;
                    f = __vibmax_s32(fExt, fOpn, &pf);
                    s = __vibmax_s32(inter, f, &pd);
                    tv = (pf ? 0u : 8u) | (pd ? 1u : 2u);
                } else {
                    const int gv = vS + EXT;
                    bool pd;
                    s = __vibmax_s32(inter, gv, &pd);
                    tv = pd ? 1u : 2u;
                }
                if (LOCAL && s <= 0) {
                    s = 0;
                    tv = 0u;
                }
                sLast = s;
                eLast = INF;
                lastF = f;
                if (LOCAL) {
                    Fs[WL] = f;
                    scout(s, INF, f, col, ve);
                }
                if (TRACE) {
                    // The last slot's code into its word, then the column: codes 0..31 as a 16-byte
                    // chunk, 32..39 as a 4-byte word (band4_pos).
#pragma unroll
                    for (int q = 0; q < NT; ++q)
                        if (q == (WL >> 3)) tw[q] |= tv << (4 * (WL & 7));
                    uint8_t *c = T + int64_t(col) * band4_col_bytes(W);
                    *reinterpret_cast<uint4 *>(c) = make_uint4(tw[0], tw[1], NT > 2 ? tw[2] : 0u, NT > 3 ? tw[3] : 0u);
                    if (NT > 4 && W > 32) *reinterpret_cast<uint32_t *>(c + 512 - 12 * lane) = tw[NT > 4 ? 4 : 0];
                }
            }
            // Shift the V window by one row: code k <- code k + 1, the new last code from V.
#pragma unroll
            for (int q = 0; q < NW - 1; ++q) vw[q] = __funnelshift_r(vw[q], vw[q + 1], 8);
            vw[NW - 1] = (vw[NW - 1] >> 8) | (uint32_t(vIn) << 24);   // V[vb + FW - 1]
        }
#pragma unroll
        for (int k = 0; k < FW - 1; ++k)
            if (k < WL) {
                S[k] = Sr[k];
                if (AFFINE) E[k] = Er[k];
            }
        S[WL] = sLast;
        E[WL] = eLast;
    }

    __device__ int first_dir(int type, int loc) const
    {
        if (type == BCOL_INITIAL) return BDIR_ZERO;
        if (loc == BLOC_FULL || loc == BLOC_TOP) return fTop ? BDIR_ZERO : BDIR_HORIZONTAL;
        return BDIR_UPPER;
    }
    __device__ int inner_dir(int type) const
    {
        if (type == BCOL_INITIAL) return fLeft ? BDIR_ZERO : BDIR_VERTICAL;
        return BDIR_ALL;
    }
    __device__ int last_dir(int type, int loc) const
    {
        if (type == BCOL_INITIAL) return fLeft ? BDIR_ZERO : BDIR_VERTICAL;
        return (loc == BLOC_TOP || loc == BLOC_MIDDLE) ? BDIR_LOWER : BDIR_ALL;
    }
    __device__ bool track_flag(int type, int loc, int which) const
    {
        if (TRK) return true;
        const bool lastColFree = type == BCOL_FINAL && fRight;
        if (which < 2) return lastColFree;
        if (loc == BLOC_FULL || loc == BLOC_BOTTOM) return type == BCOL_FINAL || fBottom;
        return lastColFree;
    }

    __device__ void track(int col, int type, int loc, int r0, int r1)
    {
        dS = INF; vS = INF; vF = INF;
        if (type != BCOL_INITIAL && (loc == BLOC_MIDDLE || loc == BLOC_BOTTOM) && r0 > 0 && col > 0) {
            const int kd = slot(col - 1, r0 - 1);
            dS = in_slots(kd) ? S[kd] : INF;
        }
        cell(first_dir(type, loc), col, r0, track_flag(type, loc, 0));
        for (int i = r0 + 1; i < r1; ++i) cell(inner_dir(type), col, i, track_flag(type, loc, 1));
        cell(last_dir(type, loc), col, r1, track_flag(type, loc, 2), true);
    }

    __device__ void single(int dir, int col, int row, int diag_from_col, int diag_from_row, bool tracked)
    {
        dS = INF; vS = INF; vF = INF;
        if (diag_from_col >= 0) {
            const int kd = slot(diag_from_col, diag_from_row);
            dS = in_slots(kd) ? S[kd] : INF;
        }
        cell(dir, col, row, tracked);
    }

    __device__ void run()
    {
        for (int k = 0; k < W; ++k) { S[k] = INF; E[k] = INF; Fs[k] = INF; }
        bs = INF; be = INF; bf = INF; bcol = 0; brow = 0;
        lastF = INF;
        colmax = INT_MIN;
        term = false;
        const int lo = lower, up = upper;
        if (up == lo) {
            // Band of one diagonal (align/dp_algorithm_impl.h:970-1110).
            int ih = max(0, min(m - 1, up)), ihEnd = min(m - 1, up + n);
            int iv = max(0, min(n - 1, -lo)), ivEnd = min(n - 1, lo + m);
            int col = up >= 0 ? min(m, up) : 0;
            int row = up >= 0 ? 0 : min(n, -up);
            // _computeHammingDistance offers its cells without IsLastRow (no X-drop check).
            single(BDIR_ZERO, col, row, -1, 0, false);
            if (up < 0) {
                if (up == -n) { if (TRK || fBottom) retrack(col, row, false, false); return; }
                if (TRK) retrack(col, row, false, false);
            } else if (lo > 0) {
                if (lo == m) { if (TRK || fRight) retrack(col, row, false, false); return; }
                if (TRK) retrack(col, row, false, false);
            } else {
                if (TRK) retrack(col, row, false, false);
            }
            int prev = 0;
            while (ih != ihEnd && iv != ivEnd) {
                ++col; ++row;
                int s = prev + (MATRIX ? smat[((H[ih] & 31) << 5) | (V[iv] & 31)] : (H[ih] == V[iv] ? a.match : a.mismatch));
                int tv = TV_DIAG;
                if (LOCAL && s <= 0) { s = 0; tv = TV_NONE; }
                if (TRACE) put_trace(col, 0, tv);
                if (TRK) offer(s, INF, INF, col, row, false);
                prev = s;
                ++ih; ++iv;
            }
            if (ih > m - 1 || iv > n - 1 || col + 1 > m || row + 1 > n) return;
            ++col; ++row;
            int s = prev + (MATRIX ? smat[((H[ih] & 31) << 5) | (V[iv] & 31)] : (H[ih] == V[iv] ? a.match : a.mismatch));
            int tv = TV_DIAG;
            if (LOCAL && s <= 0) { s = 0; tv = TV_NONE; }
            if (TRACE) put_trace(col, 0, tv);
            if (ih == ihEnd) {
                if (iv == ivEnd) offer(s, INF, INF, col, row, false);
                if (TRK || fBottom) offer(s, INF, INF, col, row, false);
            } else {
                if (TRK || fRight) offer(s, INF, INF, col, row, false);
            }
            return;
        }

        int vb = -min(0, 1 + up);
        int ve = -min(0, max(-n, lo));
        const int hb = max(0, min(m - 1, lo));
        int hTop = min(m - 1, max(0, up));
        int hMid = min(m - 1, max(0, n + lo));
        if (up > n + lo) { const int t = hTop; hTop = hMid; hMid = t; }
        const int hBot = max(0, min(m, up + n) - 1);

        if (hb == m - 1) {
            const int col = max(0, min(m, lo));
            single(BDIR_ZERO, col, 0, -1, 0, TRK);
            if (TRK || fRight) retrack(col, 0, false, false);   // (IsLastColumn, not IsLastRow)
            return;
        }
        if (hBot == 0) {
            const int row = min(n, -up);
            single(BDIR_ZERO, 0, row, -1, 0, TRK);
            if (TRK || fBottom) retrack(0, row, false);
            return;
        }
        if (up < 0) {
            ++vb;
            track(0, BCOL_INITIAL, lo > -n ? BLOC_MIDDLE : BLOC_BOTTOM, vb, ve);
        } else if (lo >= 0) {
            single(BDIR_ZERO, hb, 0, -1, 0, TRK);
            if (TRK) retrack(hb, 0, false, false);
        } else {
            track(0, BCOL_INITIAL, lo <= -n ? BLOC_FULL : BLOC_TOP, vb, ve);
        }
        if (XT && term) return;
        int hIt = hb;
        for (; hIt != hTop; ++hIt) {
            ++ve;
            track(hIt + 1, BCOL_INNER, BLOC_TOP, vb, ve);
            if (XT && term) return;
        }
        if (up > n + lo) {
            if (TRK || fBottom) retrack(hIt, ve, false);
            for (; hIt != hMid; ++hIt) {
                track(hIt + 1, BCOL_INNER, BLOC_FULL, vb, ve);
                if (XT && term) return;
            }
        } else {
            if (!XT && W >= 2 && W <= kBandFastW && hIt != hMid && ve - vb + 1 == W &&
                upper - (hIt + 1) + (vb + 1) == 0)
                middle_fast(hIt, hMid, vb, ve);
            for (; hIt != hMid; ++hIt) {
                ++vb; ++ve;
                track(hIt + 1, BCOL_INNER, BLOC_MIDDLE, vb, ve);
                if (XT && term) return;
            }
            if ((TRK || fBottom) && lo + n < m) retrack(hIt, ve, false);
        }
        for (; hIt != hBot; ++hIt) {
            ++vb;
            track(hIt + 1, BCOL_INNER, BLOC_BOTTOM, vb, ve);
            if (XT && term) return;
        }
        if (hIt < m - 1) {
            single(BDIR_UPPER, hIt + 1, vb + 1, hIt, vb, TRK);
            if (TRK || fBottom) retrack(hIt + 1, vb + 1, true);
        } else if (hIt == m - 1) {
            if (up == m - n) {
                single(BDIR_UPPER, m, vb + 1, hIt, vb, TRK || fRight);
                retrack(m, vb + 1, true);
            } else if (up >= m) {
                if (lo + n > m) {
                    ++ve;
                    track(m, BCOL_FINAL, BLOC_TOP, vb, ve);
                } else if (lo + n + 1 > m) {
                    ++ve;
                    track(m, BCOL_FINAL, BLOC_TOP, vb, ve);
                    retrack(m, ve, true);
                } else {
                    track(m, BCOL_FINAL, BLOC_FULL, vb, ve);
                }
            } else {
                ++vb;
                if (lo + n <= m) {
                    if (lo + n == m) {
                        ++ve;
                        track(m, BCOL_FINAL, BLOC_MIDDLE, vb, ve);
                        retrack(m, ve, true);
                    } else {
                        track(m, BCOL_FINAL, BLOC_BOTTOM, vb, ve);
                    }
                } else {
                    ++ve;
                    track(m, BCOL_FINAL, BLOC_MIDDLE, vb, ve);
                }
            }
        }
    }
};

template <bool AFFINE, bool LOCAL, bool MATRIX, bool TRACE, int WMAX, bool XT = false>
__global__ void __launch_bounds__(128) k_dp_banded(BandArgs a)
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
    const int W = a.upper - a.lower + 1;
    const int fe = LOCAL ? (FREE_TOP | FREE_LEFT | FREE_RIGHT | FREE_BOTTOM)
                         : XT ? (FREE_RIGHT | FREE_BOTTOM) : a.free_ends;
    const int lane = int((d.trace_off >> 4) & 31);
    BandedPair<AFFINE, LOCAL, MATRIX, TRACE, WMAX, XT> bp(a, smat);
    bp.lane = lane;
    bp.m = d.m;
    bp.n = d.n;
    bp.W = W;
    bp.Wt = band_trace_stride(bp.W);
    bp.lower = a.lower;
    bp.upper = a.upper;
    bp.INF = d.inf;
    bp.H = a.seq_h + d.h_off;
    bp.V = a.seq_v + d.v_off;
    bp.T = TRACE ? a.trace + d.trace_off : nullptr;
    bp.fTop = fe & FREE_TOP;
    bp.fLeft = fe & FREE_LEFT;
    bp.fRight = fe & FREE_RIGHT;
    bp.fBottom = fe & FREE_BOTTOM;
    bp.OPEN = AFFINE ? a.gap_open : a.gap_extend;
    bp.EXT = a.gap_extend;
    bp.run();
    a.score[p] = bp.bs;
    if (a.end_h) a.end_h[p] = bp.bcol;
    if (a.end_v) a.end_v[p] = bp.brow;
    if (a.best_e) a.best_e[p] = bp.be;
    if (a.best_f) a.best_f[p] = bp.bf;
}

// Trace byte of (col, row) in a banded trace matrix; cells outside the band read as NONE.  base
// is the pair's trace_off (whose lane the 4-bit layout needs).
__device__ __forceinline__ uint8_t trace_at_band(const uint8_t *base, int64_t trace_off, int W, int upper, bool affine,
                                                 int col, int row)
{
    const int k = upper - col + row;
    if (k < 0 || k >= W) return TV_NONE;
    if (band_trace4(W)) {
        const uint32_t b = base[band4_pos(W, int((trace_off >> 4) & 31), col, k)];
        return trace4_decode((k & 1) ? (b >> 4) : (b & 15u), affine);
    }
    return base[band_trace_pos(band_trace_stride(W), col, k)];
}

}  // namespace gba
