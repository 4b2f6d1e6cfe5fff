// dp16x2_kernels.cuh -- packed 16-bit DP: two pairs per thread, DPX max/add.
//
// For global alignments with equality scoring (Score<T, Simple>) whose every cell value
// stays inside the exact int16 range (the same bound the engine uses to honour 16-bit
// cells), each thread runs TWO pairs in the two 16-bit halves of 32-bit registers.  The
// max/add steps are the sm_90+ DPX instructions __viaddmax_s16x2 (max(a + b, c)) and
// __vimax3_s16x2, so one instruction advances two cells; the substitution score of both
// halves comes from one PRMT lookup in a byte table.
//
// Scores and end positions are exactly those of the reference's DP: the recurrence values
// are the same integers (align/dp_formula_affine.h:66-330, align/dp_formula_linear.h:62-258;
// border cells align/dp_meta_info.h:178-221), and the tracked cells and the first-max rule
// of the scout (align/dp_scout.h:166-180) are applied per half.
//
// Layout (all per warp, interleaved by lane so each warp access is 128 contiguous bytes):
//   codes:    one 32-bit word per 4 columns of H and per 4 rows of V; byte k of a word holds
//             the two pairs' residue codes (pair A in the low nibble, pair B in the high nibble)
//   boundary: per column, the strip's bottom row (S2, F2) as one int2
#pragma once

#include "dp_common.cuh"

namespace gba {

// Slot = two pairs sharing one thread, or (split slot) one pair whose rows run as two strips
// at once, one per 16-bit half.
struct Slot16 {
    int32_t pa, pb;        // pair indices (pb = -1: no second pair)
    int32_t m, n;          // max columns / rows over the two pairs (split slot: m + 1 steps, n)
    int32_t split;         // 1: split slot (pb = -1)
};

struct Dp16Args {
    const uint8_t *seq_h;
    const uint8_t *seq_v;
    const PairDesc *pairs;
    const Slot16 *slots;
    const int64_t *warp_codes;    // per warp: word offset of its code region
    const int32_t *warp_hwords;   // per warp: words of H codes per lane (the V codes follow)
    uint32_t *codes;
    const int64_t *warp_bnd;      // per warp: int2 offset of its boundary region
    int2 *bnd;
    int32_t *score, *end_h, *end_v;
    int64_t num_slots;
    int32_t match, mismatch, gap_open, gap_extend;
    int32_t free_ends;
    int32_t num_tasks;            // warp-sized work items (32 consecutive slots each)
    int32_t *task_counter;        // next work item; zeroed before each launch
    int32_t rows;                 // rows per strip of the launched variant (split slot packing)
};

// ---- packing: residue codes of the two pairs -> interleaved nibble words -------------
// Each lane packs its own slot into its column of the warp's code region and is the only
// reader of that column, so no synchronisation is needed.
__device__ __forceinline__ void pack_slot(const Dp16Args &a, const Slot16 &sl, int64_t task, int lane)
{
    uint32_t *base = a.codes + a.warp_codes[task] + lane;
    const int hw = a.warp_hwords[task];
    const PairDesc A = a.pairs[sl.pa];
    if (sl.split) {
        // Split slot: H byte j holds H[j] (low nibble, lower strip at column j + 1) and H[j - 1]
        // (high nibble, upper strip one column behind); V byte i holds V[i] and V[i + rows].
        const uint8_t *h = a.seq_h + A.h_off, *v = a.seq_v + A.v_off;
        const int R = a.rows;
        for (int q = 0; q < (A.m + 1 + 3) >> 2; ++q) {
            uint32_t word = 0;
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                const int j = 4 * q + k;
                const uint32_t lo = j < A.m ? (h[j] & 7u) : 0u;
                const uint32_t hi = (j >= 1 && j <= A.m) ? (h[j - 1] & 7u) : 0u;
                word |= (lo | (hi << 4)) << (8 * k);
            }
            base[int64_t(q) * 32] = word;
        }
        for (int q = 0; q < (A.n + 3) >> 2; ++q) {
            uint32_t word = 0;
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                const int i = 4 * q + k;
                const uint32_t lo = i < A.n ? (v[i] & 7u) : 0u;
                const uint32_t hi = i + R < A.n ? (v[i + R] & 7u) : 0u;
                word |= (lo | (hi << 4)) << (8 * k);
            }
            base[int64_t(hw + q) * 32] = word;
        }
        return;
    }
    PairDesc B = A;
    int mb = 0, nb = 0;
    if (sl.pb >= 0) { B = a.pairs[sl.pb]; mb = B.m; nb = B.n; }
    const uint8_t *ha = a.seq_h + A.h_off, *hb = a.seq_h + B.h_off;
    const uint8_t *va = a.seq_v + A.v_off, *vb = a.seq_v + B.v_off;
    const int hq = (sl.m + 3) >> 2;
    for (int q = 0; q < hq; ++q) {
        uint32_t word = 0;
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            const int j = 4 * q + k;
            const uint32_t ca = j < A.m ? (ha[j] & 7u) : 0u;
            const uint32_t cb = j < mb ? (hb[j] & 7u) : 0u;
            word |= (ca | (cb << 4)) << (8 * k);
        }
        base[int64_t(q) * 32] = word;
    }
    const int vw = (sl.n + 3) >> 2;
    for (int q = 0; q < vw; ++q) {
        uint32_t word = 0;
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            const int i = 4 * q + k;
            const uint32_t ca = i < A.n ? (va[i] & 7u) : 0u;
            const uint32_t cb = i < nb ? (vb[i] & 7u) : 0u;
            word |= (ca | (cb << 4)) << (8 * k);
        }
        base[int64_t(hw + q) * 32] = word;
    }
}

__device__ __forceinline__ uint32_t pack2(int lo, int hi)
{
    return (uint32_t(lo) & 0xffffu) | (uint32_t(hi) << 16);
}
__device__ __forceinline__ int lo16(uint32_t x) { return int(int16_t(x & 0xffffu)); }
__device__ __forceinline__ int hi16(uint32_t x) { return int(int16_t(x >> 16)); }

__device__ __forceinline__ uint32_t prmt(uint32_t a, uint32_t b, uint32_t sel)
{
    uint32_t d;
    asm("prmt.b32 %0, %1, %2, %3;" : "=r"(d) : "r"(a), "r"(b), "r"(sel));
    return d;
}

// Selector half for a row code v (3 bits): byte nibble v, then 8|v (sign replicate).
__device__ __forceinline__ uint32_t vsel_of(uint32_t byte)
{
    const uint32_t a = byte & 7u, b = (byte >> 4) & 7u;
    return a | ((a | 8u) << 4) | (b << 8) | ((b | 8u) << 12);
}
__device__ __forceinline__ uint32_t hsel_of(uint32_t byte)
{
    const uint32_t a = byte & 7u, b = (byte >> 4) & 7u;
    return (a * 0x11u) | ((b * 0x11u) << 8);
}

struct Best2 {
    int s[2], col[2], row[2];
    __device__ __forceinline__ void init()
    {
        s[0] = s[1] = -16384; col[0] = col[1] = 0; row[0] = row[1] = 0;
    }
    __device__ __forceinline__ void offer(int h, int cs, int ccol, int crow)
    {
        if (cs >= s[h] && (cs > s[h] || ccol < col[h] || (ccol == col[h] && crow < row[h]))) {
            s[h] = cs; col[h] = ccol; row[h] = crow;
        }
    }
};

// Packs every slot's codes (one thread per slot, full occupancy) before the DP runs.
__global__ void __launch_bounds__(128) k_pack16(Dp16Args a)
{
    const int64_t s = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (s >= a.num_slots) return;
    const Slot16 sl = a.slots[s];
    if (sl.pa < 0) return;   // padding slot of the plain per-bucket form
    pack_slot(a, sl, s >> 5, int(s & 31));
}

constexpr int kBndAhead = 4;   // columns between a boundary load and its use

// Split slot: one pair whose rows run in double strips of 2R.  The low 16-bit half computes rows
// i0 .. i0+R-1 at column j while the high half computes rows i0+R .. i0+2R-1 at column j - 1,
// taking as its row above the low half's bottom row of the previous step (kept in registers),
// so the pair's sequence of steps is half as long as in a two-pair slot.  Recurrences and
// tracked cells are dp16x2_slot's; every instruction still advances two cells.
template <bool AFFINE, int R>
__device__ __forceinline__ void dp16x2_split(const Dp16Args &a, const Slot16 &sl, const uint32_t *codes, int hw,
                                             int2 *bnd)
{
    const PairDesc A = a.pairs[sl.pa];
    const int m = A.m, n = A.n;
    const int fe = a.free_ends;
    const bool fTop = fe & FREE_TOP, fLeft = fe & FREE_LEFT;
    const bool fRight = fe & FREE_RIGHT, fBottom = fe & FREE_BOTTOM;
    const int INF = -16384;
    const uint32_t INF2 = pack2(INF, INF);
    const uint32_t EXT2 = pack2(a.gap_extend, a.gap_extend);
    const uint32_t OPEN2 = AFFINE ? pack2(a.gap_open, a.gap_open) : EXT2;
    const int emax = max(a.gap_extend, a.gap_open);
    const uint32_t EMAX2 = pack2(emax, emax);
    const uint32_t NEG2 = pack2(-32768, -32768);
    const uint32_t T0 = (uint32_t(a.match) & 0xffu) | ((uint32_t(a.mismatch) & 0xffu) * 0x01010100u);
    const uint32_t T1 = (uint32_t(a.mismatch) & 0xffu) * 0x01010101u;
    Best2 best;
    best.init();

    // Row 0 (both halves carry the same values).
    {
        uint32_t s2 = 0, e2 = INF2;
        bnd[0] = make_int2(0, int(AFFINE ? __viaddmax_s16x2(INF2, EXT2, __viaddmax_s16x2(s2, OPEN2, NEG2)) : INF2));
        for (int j = 1; j <= m; ++j) {
            if (!fTop) {
                if (AFFINE) {
                    e2 = __viaddmax_s16x2(e2, EXT2, __viaddmax_s16x2(s2, OPEN2, NEG2));
                    s2 = e2;
                } else {
                    s2 = __viaddmax_s16x2(s2, EXT2, NEG2);
                }
            }
            const uint32_t f1 = AFFINE ? __viaddmax_s16x2(INF2, EXT2, __viaddmax_s16x2(s2, OPEN2, NEG2)) : INF2;
            bnd[int64_t(j) * 32] = make_int2(int(s2), int(f1));
            if (fRight && j == m) best.offer(0, lo16(s2), j, 0);
        }
    }

    for (int i0 = 1; i0 <= n; i0 += 2 * R) {
        uint32_t vs[R];
#pragma unroll
        for (int q = 0; q < R / 4; ++q) {
            const int wq = (i0 - 1) / 4 + q;
            const uint32_t word = (4 * wq < n) ? codes[int64_t(hw + wq) * 32] : 0u;
#pragma unroll
            for (int k = 0; k < 4; ++k) vs[4 * q + k] = vsel_of(word >> (8 * k));
        }
        uint32_t Sp[R], Ep[R];
        const int rLo = n - i0, rHi = n - i0 - R;      // row n's index in each strip
        const bool endLo = rLo >= 0 && rLo < R, endHi = rHi >= 0 && rHi < R;

        // Column 0 of a strip from the S and (advanced) F above it; hi = the high strip, whose
        // values go to the high halves.  Both halves of the inputs are equal.
        auto col0 = [&](uint32_t &sUp, uint32_t &fUp, bool hi, bool track) {
#pragma unroll
            for (int r = 0; r < R; ++r) {
                uint32_t s2, ep;
                if (fLeft) {
                    s2 = 0;
                } else if (AFFINE) {
                    s2 = fUp;
                } else {
                    s2 = __viaddmax_s16x2(sUp, EXT2, NEG2);
                }
                if (AFFINE) {
                    const uint32_t so = __viaddmax_s16x2(s2, OPEN2, NEG2);
                    fUp = __viaddmax_s16x2(fUp, EXT2, so);
                    ep = __viaddmax_s16x2(INF2, EXT2, so);
                } else {
                    ep = INF2;
                }
                Sp[r] = hi ? prmt(Sp[r], s2, 0x7610) : s2;
                Ep[r] = hi ? prmt(Ep[r], ep, 0x7610) : ep;
                sUp = s2;
                if (track && fBottom && ((!hi && endLo && r == rLo) || (hi && endHi && r == rHi)))
                    best.offer(0, lo16(s2), 0, n);
            }
        };
        const int2 up0 = bnd[0];
        uint32_t sUp = uint32_t(up0.x), fUp = uint32_t(up0.y);
        col0(sUp, fUp, false, true);
        const uint32_t sLo0 = sUp, fLo0 = fUp;          // low strip's bottom, column 0
        col0(sUp, fUp, true, true);
        bnd[0] = make_int2(int(sUp), int(fUp));         // high strip's bottom, column 0

        uint32_t hword = codes[0];
        uint32_t hnext = m + 1 > 4 ? codes[32] : 0u;
        int2 upq[kBndAhead];
#pragma unroll
        for (int d = 0; d < kBndAhead; ++d) upq[d] = (1 + d <= m) ? bnd[int64_t(1 + d) * 32] : make_int2(0, 0);
        uint32_t diagLo = uint32_t(up0.x);              // S above the low strip, previous column
        uint32_t loS1 = sLo0, loF1 = fLo0, loS2 = sLo0;  // low strip's bottom, one / two steps back
        // Step j: low strip column j (j <= m), high strip column j - 1 (j >= 2).
        for (int j = 1; j <= m + 1; ++j) {
            const uint32_t hsel = hsel_of(hword >> (8 * ((j - 1) & 3)));
            const int2 upLo = upq[0];
#pragma unroll
            for (int d = 0; d + 1 < kBndAhead; ++d) upq[d] = upq[d + 1];
            if (j + kBndAhead <= m) upq[kBndAhead - 1] = bnd[int64_t(j + kBndAhead) * 32];
            if ((j & 3) == 0) {
                hword = hnext;
                if (4 * ((j >> 2) + 1) < m + 1) hnext = codes[int64_t((j >> 2) + 1) * 32];
            }
            sUp = prmt(uint32_t(upLo.x), loS1, 0x5410);
            fUp = prmt(uint32_t(upLo.y), loF1, 0x5410);
            uint32_t diag = prmt(diagLo, loS2, 0x5410);
            diagLo = uint32_t(upLo.x);
#pragma unroll
            for (int r = 0; r < R; ++r) {
                const uint32_t sub = prmt(T0, T1, hsel ^ vs[r]);
                uint32_t s2;
                if (AFFINE) {
                    const uint32_t X = __viaddmax_s16x2(diag, sub, Ep[r]);
                    const uint32_t XO = __viaddmax_s16x2(X, OPEN2, NEG2);
                    s2 = __vimax3_s16x2(X, fUp, fUp);
                    const uint32_t so = __viaddmax_s16x2(s2, OPEN2, NEG2);
                    Ep[r] = __viaddmax_s16x2(Ep[r], EXT2, so);
                    fUp = __viaddmax_s16x2(fUp, EMAX2, XO);
                } else {
                    const uint32_t Y = __viaddmax_s16x2(diag, sub, __viaddmax_s16x2(Sp[r], EXT2, NEG2));
                    s2 = __viaddmax_s16x2(sUp, EXT2, Y);
                }
                diag = Sp[r];
                Sp[r] = s2;
                sUp = s2;
            }
            if (j == 1) {
                // The high strip has no column to compute yet: put its column-0 state back.
                uint32_t s0 = sLo0, f0 = fLo0;
                const uint32_t sKeep = sUp, fKeep = fUp;
                col0(s0, f0, true, false);
                sUp = sKeep;
                fUp = fKeep;
            } else {
                bnd[int64_t(j - 1) * 32] = make_int2(int(prmt(sUp, sUp, 0x3232)), int(prmt(fUp, fUp, 0x3232)));
            }
            loS2 = loS1;
            loS1 = sUp;
            loF1 = fUp;
            // Tracking: the low strip is at column j, the high strip at column j - 1.
            const int jh = j - 1;
            if (j == m || jh == m) {
#pragma unroll
                for (int r = 0; r < R; ++r) {
                    const int il = i0 + r, ih = i0 + R + r;
                    if (j == m && il <= n && (fRight || il == n)) best.offer(0, lo16(Sp[r]), m, il);
                    if (jh == m && ih <= n && (fRight || ih == n)) best.offer(0, hi16(Sp[r]), m, ih);
                }
            }
            if (fBottom && (endLo || endHi)) {
#pragma unroll
                for (int r = 0; r < R; ++r) {
                    if (endLo && r == rLo && j < m) best.offer(0, lo16(Sp[r]), j, n);
                    if (endHi && r == rHi && jh >= 1 && jh < m) best.offer(0, hi16(Sp[r]), jh, n);
                }
            }
        }
    }
    a.score[sl.pa] = best.s[0];
    if (a.end_h) a.end_h[sl.pa] = best.col[0];
    if (a.end_v) a.end_v[sl.pa] = best.row[0];
}

// One pair-of-pairs per thread.  R rows per register strip.
template <bool AFFINE, int R>
__device__ __forceinline__ void dp16x2_slot(const Dp16Args &a, int64_t w, int lane)
{
    const int64_t s = w * 32 + lane;
    if (s >= a.num_slots) return;
    const Slot16 sl = a.slots[s];
    const uint32_t *codes = a.codes + a.warp_codes[w] + lane;
    const int hw = a.warp_hwords[w];
    int2 *bnd = a.bnd + a.warp_bnd[w] + lane;

    if (sl.split) {
        dp16x2_split<AFFINE, R>(a, sl, codes, hw, bnd);
        return;
    }
    const PairDesc A = a.pairs[sl.pa];
    const bool hasB = sl.pb >= 0;
    int mB = 0, nB = 0;
    if (hasB) { const PairDesc B = a.pairs[sl.pb]; mB = B.m; nB = B.n; }
    const int mA = A.m, nA = A.n;
    const int M = sl.m, N = sl.n;

    const int fe = a.free_ends;
    const bool fTop = fe & FREE_TOP, fLeft = fe & FREE_LEFT;
    const bool fRight = fe & FREE_RIGHT, fBottom = fe & FREE_BOTTOM;
    const int INF = -16384;
    const uint32_t INF2 = pack2(INF, INF);
    const uint32_t EXT2 = pack2(a.gap_extend, a.gap_extend);
    const uint32_t OPEN2 = AFFINE ? pack2(a.gap_open, a.gap_open) : EXT2;
    const int emax = max(a.gap_extend, a.gap_open);
    const uint32_t EMAX2 = pack2(emax, emax);
    const uint32_t NEG2 = pack2(-32768, -32768);
    // Byte table for PRMT: entry d = code_h XOR code_v, 0 -> match, 1..7 -> mismatch.
    const uint32_t T0 = (uint32_t(a.match) & 0xffu) | ((uint32_t(a.mismatch) & 0xffu) * 0x01010100u);
    const uint32_t T1 = (uint32_t(a.mismatch) & 0xffu) * 0x01010101u;

    Best2 best;
    best.init();
    const int mh[2] = {mA, mB}, nh[2] = {nA, nB};
    const int halves = hasB ? 2 : 1;

    // ---- Row 0.  The boundary holds, per column, S of the row above the next strip and F of
    // that strip's first row (already advanced: F(i, j) = max(F(i-1, j) + ext, S(i-1, j) + open)).
    {
        uint32_t s2 = 0, e2 = INF2;
        bnd[0] = make_int2(0, int(AFFINE ? __viaddmax_s16x2(INF2, EXT2, __viaddmax_s16x2(s2, OPEN2, NEG2)) : INF2));
        for (int j = 1; j <= M; ++j) {
            if (!fTop) {
                if (AFFINE) {
                    e2 = __viaddmax_s16x2(e2, EXT2, __viaddmax_s16x2(s2, OPEN2, NEG2));
                    s2 = e2;
                } else {
                    s2 = __viaddmax_s16x2(s2, EXT2, NEG2);
                }
            }
            const uint32_t f1 = AFFINE ? __viaddmax_s16x2(INF2, EXT2, __viaddmax_s16x2(s2, OPEN2, NEG2)) : INF2;
            bnd[int64_t(j) * 32] = make_int2(int(s2), int(f1));
            if (fRight) {
                if (j == mA) best.offer(0, lo16(s2), j, 0);
                if (hasB && j == mB) best.offer(1, hi16(s2), j, 0);
            }
        }
    }

    // ---- Strips.
    for (int i0 = 1; i0 <= N; i0 += R) {
        uint32_t vs[R];
#pragma unroll
        for (int q = 0; q < R / 4; ++q) {
            const int wq = (i0 - 1) / 4 + q;
            const uint32_t word = (4 * wq < N) ? codes[int64_t(hw + wq) * 32] : 0u;
#pragma unroll
            for (int k = 0; k < 4; ++k) vs[4 * q + k] = vsel_of(word >> (8 * k));
        }
        uint32_t Sp[R], Ep[R];
        // Rows of each half that end inside this strip (for end-row tracking).
        const int rA = nA - i0, rB = nB - i0;
        const bool endA = rA >= 0 && rA < R, endB = hasB && rB >= 0 && rB < R;

        // Column 0: Vertical (or Zero with a free first column); E enters column 1 as
        // E(i, 1) = max(E(i, 0) + ext, S(i, 0) + open) with E(i, 0) = infinity.
        uint32_t diagNext;
        {
            const int2 up = bnd[0];
            uint32_t sUp = uint32_t(up.x), fUp = uint32_t(up.y);
            diagNext = sUp;
#pragma unroll
            for (int r = 0; r < R; ++r) {
                uint32_t s2;
                if (fLeft) {
                    s2 = 0;
                } else if (AFFINE) {
                    s2 = fUp;
                } else {
                    s2 = __viaddmax_s16x2(sUp, EXT2, NEG2);
                }
                if (AFFINE) {
                    const uint32_t so = __viaddmax_s16x2(s2, OPEN2, NEG2);
                    fUp = __viaddmax_s16x2(fUp, EXT2, so);
                    Ep[r] = __viaddmax_s16x2(INF2, EXT2, so);
                } else {
                    Ep[r] = INF2;
                }
                Sp[r] = s2;
                sUp = s2;
                if (fBottom) {
                    if (endA && r == rA) best.offer(0, lo16(s2), 0, nA);
                    if (endB && r == rB) best.offer(1, hi16(s2), 0, nB);
                }
            }
            bnd[0] = make_int2(int(sUp), int(fUp));
        }

        // Columns 1..M.  Boundary entries are loaded kBndAhead columns ahead and code words one
        // word ahead, so their latency (an L2 round trip) hides behind several columns of R
        // rows.  An entry is read before this strip overwrites it (at its own column).
        uint32_t hword = codes[0];
        uint32_t hnext = M > 4 ? codes[32] : 0u;
        int2 upq[kBndAhead];
#pragma unroll
        for (int d = 0; d < kBndAhead; ++d) upq[d] = (1 + d <= M) ? bnd[int64_t(1 + d) * 32] : make_int2(0, 0);
        for (int j = 1; j <= M; ++j) {
            const uint32_t hsel = hsel_of(hword >> (8 * ((j - 1) & 3)));
            const int2 up = upq[0];
            uint32_t sUp = uint32_t(up.x), fUp = uint32_t(up.y);
#pragma unroll
            for (int d = 0; d + 1 < kBndAhead; ++d) upq[d] = upq[d + 1];
            if (j + kBndAhead <= M) upq[kBndAhead - 1] = bnd[int64_t(j + kBndAhead) * 32];
            if ((j & 3) == 0) {
                hword = hnext;
                if (4 * ((j >> 2) + 1) < M) hnext = codes[int64_t((j >> 2) + 1) * 32];
            }
            uint32_t diag = diagNext;
            diagNext = sUp;
#pragma unroll
            for (int r = 0; r < R; ++r) {
                const uint32_t sub = prmt(T0, T1, hsel ^ vs[r]);
                uint32_t s2;
                if (AFFINE) {
                    // S = max(X, F) with X = max(diag + sub, E); E(i, j+1) from S + open.  The
                    // next row's F = max(F + ext, S + open) = max(F + max(ext, open), X + open):
                    // X + open does not depend on F, so the chain down the column is one
                    // add-max per row.  (All values stay in the exact int16 range here, so the
                    // two forms give the same integers.)
                    const uint32_t X = __viaddmax_s16x2(diag, sub, Ep[r]);
                    const uint32_t XO = __viaddmax_s16x2(X, OPEN2, NEG2);
                    s2 = __vimax3_s16x2(X, fUp, fUp);
                    const uint32_t so = __viaddmax_s16x2(s2, OPEN2, NEG2);
                    Ep[r] = __viaddmax_s16x2(Ep[r], EXT2, so);
                    fUp = __viaddmax_s16x2(fUp, EMAX2, XO);
                } else {
                    // S = max(diag + sub, left + gap, up + gap): only up + gap is on the chain.
                    const uint32_t Y = __viaddmax_s16x2(diag, sub, __viaddmax_s16x2(Sp[r], EXT2, NEG2));
                    s2 = __viaddmax_s16x2(sUp, EXT2, Y);
                }
                diag = Sp[r];
                Sp[r] = s2;
                sUp = s2;
            }
            bnd[int64_t(j) * 32] = make_int2(int(sUp), int(fUp));
            // Tracking: last column of each half, and its last row when the last row is free.
            if (j == mA || (hasB && j == mB)) {
#pragma unroll
                for (int r = 0; r < R; ++r) {
                    const int i = i0 + r;
                    if (j == mA && i <= nA && (fRight || i == nA)) best.offer(0, lo16(Sp[r]), j, i);
                    if (hasB && j == mB && i <= nB && (fRight || i == nB)) best.offer(1, hi16(Sp[r]), j, i);
                }
            }
            if (fBottom && (endA || endB)) {
#pragma unroll
                for (int r = 0; r < R; ++r) {
                    if (endA && r == rA && j < mA) best.offer(0, lo16(Sp[r]), j, nA);
                    if (endB && r == rB && j < mB) best.offer(1, hi16(Sp[r]), j, nB);
                }
            }
        }
    }
    for (int h = 0; h < halves; ++h) {
        const int p = h == 0 ? sl.pa : sl.pb;
        a.score[p] = best.s[h];
        if (a.end_h) a.end_h[p] = best.col[h];
        if (a.end_v) a.end_v[p] = best.row[h];
    }
    (void)mh;
    (void)nh;
}

// Persistent kernel: each warp takes the next work item (32 slots of the length-sorted order,
// longest first) from an atomic counter until the queue is empty.
template <bool AFFINE, int R, int MINB>
__global__ void __launch_bounds__(128, MINB) k_dp16x2(Dp16Args a)
{
    const int lane = threadIdx.x & 31;
    for (;;) {
        int t = 0;
        if (lane == 0) t = atomicAdd(a.task_counter, 1);
        t = __shfl_sync(0xffffffffu, t, 0);
        if (t >= a.num_tasks) break;
        dp16x2_slot<AFFINE, R>(a, t, lane);
    }
}

}  // namespace gba
