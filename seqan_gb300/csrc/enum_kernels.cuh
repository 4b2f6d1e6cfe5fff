// enum_kernels.cuh -- Waterman-Eggert suboptimal local alignments on the device.
//
// The reference's LocalAlignmentEnumerator<Score, Unbanded> (align/local_alignment_enumeration_
// unbanded.h) with _smithWaterman / _smithWatermanGetNext (align/local_alignment_waterman_eggert_
// impl.h): linear gaps (the scheme's gap extension score); the score matrix filled from the
// sequence ends, every cell of value >= cutoff pushed on a binary heap ordered by score
// (misc/priority_type_heap.h), each alignment traced forward from the heap's current maximum, and
// the last alignment's residue pairs forbidden and their neighbourhood recomputed ("declumping")
// before the next maximum is taken (stale heap entries are refreshed lazily).  Ties between equal
// scores go where the reference's heap puts them, so the heap's push / pop / adjust-top steps are
// the reference's.
//
// One thread per pair: an enumeration is sequential (each alignment depends on the declumped
// matrix of the previous one, and the heap's tie order on the exact sequence of pushes), so the
// batch's pairs run in parallel.  Each pair's scratch -- the (m+1) x (n+1) score matrix, the
// forbidden flags, the heap (at most m * n entries) and the trace steps -- sits in HBM at offsets
// the host assigns.
#pragma once

#include "dp_common.cuh"

namespace gba {

struct EnumPair {
    int64_t h_off, v_off;
    int64_t mat_off;       // int32 score matrix, (m + 1) * (n + 1)
    int64_t forb_off;      // uint8 flags, (m + 1) * (n + 1)
    int64_t heap_off;      // int2 {score, position}, m * n
    int64_t step_off;      // int32 steps: H then V, 2 * (m + n + 1)
    int64_t seg_off;       // segment slots: max_count * (m + n + 1)
    int64_t heap_cap;      // banded enumeration: heap entries this pair may hold
    int32_t m, n;
};

struct EnumArgs {
    const uint8_t *seq_h, *seq_v;
    const EnumPair *pairs;
    int64_t num_pairs;
    int32_t *mat;
    uint8_t *forb;
    int2 *heap;
    int32_t *steps;
    uint32_t *seg_slots;   // 4 words per segment
    int32_t *seg_count;    // [num_pairs * max_count]
    int32_t *count, *status;
    int32_t *score, *begin_h, *end_h, *begin_v, *end_v;   // [num_pairs * max_count]
    const int32_t *matrix;
    int32_t alphabet;
    int32_t match, mismatch, gap, cutoff, max_count;
    int32_t lanes;         // pairs per warp (lanes 0 .. lanes - 1 of each warp take one pair each)
};

// The pair of this thread, or -1: warp w takes pairs w * lanes .. w * lanes + lanes - 1.
__device__ __forceinline__ int64_t enum_pair_of_thread(const EnumArgs &a)
{
    const int lane = int(threadIdx.x & 31u);
    const int64_t warp = (int64_t(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
    if (lane >= a.lanes) return -1;
    const int64_t p = warp * a.lanes + lane;
    return p < a.num_pairs ? p : -1;
}

struct WeState {
    const EnumArgs *a;
    const uint8_t *H, *V;
    int32_t m, n, W;
    int32_t *M;
    uint8_t *F;
    int2 *hp;             // heap entries: x = score, y = matrix position
    int64_t hn;           // heap size
    int32_t *stepH, *stepV;
    int64_t T, bH, bV;
    int32_t x0, y0, endH, endV;
    int32_t best_end, best_begin;

    __device__ __forceinline__ int sc(int x, int y) const
    {
        if (a->matrix) return a->matrix[x * a->alphabet + y];
        return x == y ? a->match : a->mismatch;
    }

    // push + _adjustHeapTowardRoot
    __device__ void push(int2 e)
    {
        int64_t h = hn++;
        while (h > 0) {
            const int64_t i = (h - 1) / 2;
            if (hp[i].x < e.x) { hp[h] = hp[i]; h = i; }
            else break;
        }
        hp[h] = e;
    }
    // _adjustHeapTowardLeaves
    __device__ void toward_leaves(int2 e, int64_t h, int64_t i)
    {
        while (i < hn) {
            if (e.x < hp[i].x) {
                if (hp[i - 1].x < hp[i].x) { hp[h] = hp[i]; h = i; }
                else { hp[h] = hp[i - 1]; h = i - 1; }
            } else if (e.x < hp[i - 1].x) {
                hp[h] = hp[i - 1]; h = i - 1;
            } else {
                break;
            }
            i = 2 * (h + 1);
        }
        if (i == hn && e.x < hp[i - 1].x) { hp[h] = hp[i - 1]; h = i - 1; }
        hp[h] = e;
    }
    __device__ void pop()
    {
        const int2 e = hp[hn - 1];
        hn -= 1;
        if (hn > 0) toward_leaves(e, 0, 2);
    }

    // _smithWatermanGetMatrix (:112-175)
    __device__ int32_t fill()
    {
        const int32_t gap = a->gap, cutoff = a->cutoff;
        for (int32_t x = 0; x <= m; ++x) M[x + int64_t(n) * W] = 0;
        for (int32_t y = n - 1; y >= 0; --y) {
            const int cy = V[y];
            int32_t hh = 0, vv = 0;
            M[m + int64_t(y) * W] = vv;
            for (int32_t x = m - 1; x >= 0; --x) {
                const int64_t f1 = x + int64_t(y) * W, f2 = f1 + W;
                const int hx = H[x];
                const int32_t cs = sc(hx, cy);
                if (hx == cy) {
                    vv = hh + cs;
                    hh = M[f2];
                } else {
                    const int32_t s1 = hh + cs;
                    hh = M[f2];
                    const int32_t s2 = gap + (hh > vv ? hh : vv);
                    vv = s1 > s2 ? s1 : s2;
                    if (vv < 0) vv = 0;
                }
                M[f1] = vv;
                if (vv >= cutoff) push(make_int2(vv, int32_t(f1)));
            }
        }
        if (hn > 0) {
            best_end = hp[0].y;
            return M[best_end];
        }
        return 0;
    }

    // _smithWatermanTrace (:300-371)
    __device__ int32_t trace(int32_t src)
    {
        const int32_t gap = a->gap;
        int32_t i0 = src % W, i1 = src / W;
        int64_t t = 0;
        x0 = i0;
        y0 = i1;
        while (M[src] != 0 && i0 != m && i1 != n) {
            const bool forb = F[src] != 0;
            bool gv, gh;
            if (H[i0] == V[i1] && !forb) {
                gv = gh = true;
            } else {
                const int32_t vr = M[src + 1] + gap;
                const int32_t d = forb ? 0 : M[src + 1 + W] + sc(H[i0], V[i1]);
                const int32_t hd = M[src + W] + gap;
                gv = (vr >= hd) | (d >= hd);
                gh = (hd > vr) | (d >= vr);
            }
            stepH[t] = gv ? i0 : -1;
            stepV[t] = gh ? i1 : -1;
            if (gv) { ++i0; src += 1; }
            if (gh) { ++i1; src += W; }
            ++t;
        }
        T = t;
        bH = 0;
        while (bH < t && stepH[bH] < 0) ++bH;
        bV = 0;
        while (bV < t && stepV[bV] < 0) ++bV;
        endH = i0;
        endV = i1;
        return src;
    }

    __device__ __forceinline__ bool is_gap(const int32_t *step, int64_t q) const { return q >= 0 && step[q] < 0; }

    // _smithWatermanDeclump (:176-299); false where the reference's walk leaves its arrays.
    __device__ bool declump()
    {
        const int32_t gap = a->gap;
        int64_t a0 = T, a1 = T;
        const int64_t s0 = bH, s1 = bV;
        int64_t finger0, finger1, end_col, forb;
        int32_t xe = endH - 1, x_stop;
        bool forbidden_reached = true, end_reached = false, skip_row = false;
        finger0 = end_col = finger1 = forb = best_begin;
        x_stop = xe;
        for (int32_t y = endV - 1; y != -1; --y) {
            bool different = true;
            if (forbidden_reached && !end_reached) {
                if (a0 == s0 && a1 == s1) end_reached = true;
                if (!end_reached) {
                    --a0;
                    forb -= W;
                    if (x0 + a0 < 0 || y0 + a1 < 0 || forb < 0) return false;
                    while (is_gap(stepH, a0) && a0 != s0) {
                        skip_row = true;
                        --a0;
                        --a1;
                        forb -= W;
                        if (x0 + a0 < 0 || y0 + a1 < 0 || forb < 0) return false;
                    }
                    --a1;
                    forb -= 1;
                    if (x0 + a0 < 0 || y0 + a1 < 0 || forb < 0) return false;
                    while (is_gap(stepV, a1) && a1 != s1) {
                        --a1;
                        --a0;
                        forb -= 1;
                        if (x0 + a0 < 0 || y0 + a1 < 0 || forb < 0) return false;
                    }
                    F[forb] = 1;
                    forbidden_reached = false;
                }
            }
            const int cy = V[y];
            int32_t hh = M[end_col];
            finger1 = end_col;
            end_col -= W;
            finger0 = end_col;
            int32_t vv = M[finger0];
            int32_t x = xe;
            while (x != -1 && different) {
                --finger0;
                --finger1;
                const int hx = H[x];
                const int32_t cs = sc(hx, cy);
                if (hx == cy && !F[finger0]) {
                    vv = hh + cs;
                    hh = M[finger1];
                } else {
                    int32_t sa;
                    if (finger0 == forb) {
                        skip_row = false;
                        forbidden_reached = true;
                        sa = 0;
                    } else {
                        sa = F[finger0] ? 0 : hh + cs;
                    }
                    hh = M[finger1];
                    const int32_t sb = gap + (hh > vv ? hh : vv);
                    vv = sa > sb ? sa : sb;
                    if (vv < 0) vv = 0;
                }
                if (M[finger0] == vv) {
                    if (x < x_stop) {
                        different = false;
                    } else if (x == xe && ((!forbidden_reached && !skip_row) || end_reached)) {
                        --xe;
                        end_col -= 1;
                    }
                }
                if (x < x_stop) x_stop = x;
                M[finger0] = vv;
                --x;
            }
            if (xe == -1) break;
        }
        return true;
    }

    // _getNextBestEndPosition (:372-403); 0 means none (also for the real position 0).
    __device__ int32_t next_end()
    {
        int32_t top = 0;
        if (hn > 0) top = M[hp[0].y];
        if (hn > 0) {
            while (hp[0].x != top) {
                if (top >= a->cutoff) {
                    hp[0].x = top;
                    toward_leaves(hp[0], 0, 2);
                } else {
                    pop();
                }
                if (hn > 0) top = M[hp[0].y];
                else break;
            }
        }
        if (hn == 0) return 0;
        const int32_t ret = hp[0].y;
        best_end = ret;
        pop();
        return ret;
    }
};

__device__ __forceinline__ uint32_t we_type(int32_t sh, int32_t sv)
{
    return (sh >= 0 && sv >= 0) ? uint32_t(TV_DIAG) : (sh >= 0 ? uint32_t(TV_H) : uint32_t(TV_V));
}

__global__ void __launch_bounds__(128) k_waterman_eggert(EnumArgs a)
{
    const int64_t p = enum_pair_of_thread(a);
    if (p < 0) return;
    const EnumPair d = a.pairs[p];
    WeState w;
    w.a = &a;
    w.H = a.seq_h + d.h_off;
    w.V = a.seq_v + d.v_off;
    w.m = d.m;
    w.n = d.n;
    w.W = d.m + 1;
    w.M = a.mat + d.mat_off;
    w.F = a.forb + d.forb_off;
    w.hp = a.heap + d.heap_off;
    w.hn = 0;
    w.stepH = a.steps + d.step_off;
    w.stepV = w.stepH + (d.m + d.n + 1);
    int32_t k = 0, status = 0;
    if (d.m > 0 && d.n > 0) {
        const int64_t cells = int64_t(d.m + 1) * (d.n + 1);
        for (int64_t q = 0; q < cells; ++q) w.F[q] = 0;
        for (; k < a.max_count; ++k) {
            int32_t s;
            if (k == 0) {
                s = w.fill();
                if (s == 0) break;
                w.best_begin = w.trace(w.hp[0].y);
                w.pop();
            } else {
                if (!w.declump()) {
                    status = 1;
                    break;
                }
                const int32_t e = w.next_end();
                if (e == 0) break;
                w.best_begin = w.trace(e);
                s = w.M[e];
                if (s == 0) break;
            }
            const int64_t o = p * a.max_count + k;
            a.score[o] = w.M[w.best_end];
            a.begin_h[o] = w.bH < w.T ? w.stepH[w.bH] : w.endH;
            a.begin_v[o] = w.bV < w.T ? w.stepV[w.bV] : w.endV;
            a.end_h[o] = w.endH;
            a.end_v[o] = w.endV;
            // the columns as runs in alignment order, from the earlier of the two rows' begins
            uint32_t *out = a.seg_slots + 4 * (d.seg_off + int64_t(k) * (d.m + d.n + 1));
            int32_t ns = 0;
            int64_t t = w.bH < w.bV ? w.bH : w.bV;
            int32_t nextH = w.endH, nextV = w.endV;   // next residue of each row from step t on
            for (int64_t q = w.T - 1; q >= t; --q) {
                if (w.stepH[q] >= 0) nextH = w.stepH[q];
                if (w.stepV[q] >= 0) nextV = w.stepV[q];
            }
            while (t < w.T) {
                const uint32_t type = we_type(w.stepH[t], w.stepV[t]);
                int64_t u = t + 1;
                while (u < w.T && we_type(w.stepH[u], w.stepV[u]) == type) ++u;
                out[4 * ns + 0] = uint32_t(nextH);
                out[4 * ns + 1] = uint32_t(nextV);
                out[4 * ns + 2] = uint32_t(u - t);
                out[4 * ns + 3] = type;
                ++ns;
                const uint32_t len = uint32_t(u - t);
                if (type != TV_V) nextH += int32_t(len);
                if (type != TV_H) nextV += int32_t(len);
                t = u;
            }
            a.seg_count[o] = ns;
        }
    }
    a.count[p] = k;
    a.status[p] = status;
}

// --- LocalAlignmentEnumerator<Score, Banded> ------------------------------------------------
// align/local_alignment_banded_waterman_eggert_impl.h: the score matrix kept as band storage (one
// stored row per matrix row, diagonalWidth = upper - lower + 1 columns, a step to the next stored
// row moving one diagonal), filled forward from the sequence begins with every cell >= cutoff
// pushed on the heap (_alignBandedSmithWaterman), each alignment traced backward from the heap's
// maximum into a list of (size, direction) runs as _alignTracePrint appends them
// (_alignBandedSmithWatermanTrace), its diagonal cells forbidden and the rows below re-filled
// while values change, with every changed cell >= cutoff pushed again
// (_alignBandedSmithWatermanDeclump).  The heap's entries are refreshed lazily from the matrix
// as in the unbanded enumerator.  A walk that reads outside the band storage, or a character
// outside a sequence, is undefined in the reference: the enumeration stops with status 1.

enum { WB_DIAG = 0, WB_HORI = 1, WB_VERT = 2, WB_STOP = 3 };

struct WbState {
    const EnumArgs *a;
    const uint8_t *H, *V;
    int64_t len1, len2, lo, W, lo_row, height_fill, cells;
    int32_t *M;
    uint8_t *F;
    int2 *hp;
    int64_t hn, hcap;
    int32_t *tsz;           // trace runs: sizes
    int32_t *ttv;           // trace runs: directions
    int64_t nt;
    int64_t best_end, best_begin;
    int64_t aCol, eCol, aRow, eRow;
    int status;             // 0, 1 undefined next step, 2 heap capacity

    __device__ __forceinline__ int sc(int64_t x, int64_t y) const
    {
        const int hx = H[x], vy = V[y];
        if (a->matrix) return a->matrix[hx * a->alphabet + vy];
        return hx == vy ? a->match : a->mismatch;
    }
    __device__ void push(int2 e)
    {
        if (hn >= hcap) { status = 2; return; }
        int64_t h = hn++;
        while (h > 0) {
            const int64_t i = (h - 1) / 2;
            if (hp[i].x < e.x) { hp[h] = hp[i]; h = i; }
            else break;
        }
        hp[h] = e;
    }
    __device__ void toward_leaves(int2 e, int64_t h, int64_t i)
    {
        while (i < hn) {
            if (e.x < hp[i].x) {
                if (hp[i - 1].x < hp[i].x) { hp[h] = hp[i]; h = i; }
                else { hp[h] = hp[i - 1]; h = i - 1; }
            } else if (e.x < hp[i - 1].x) {
                hp[h] = hp[i - 1]; h = i - 1;
            } else {
                break;
            }
            i = 2 * (h + 1);
        }
        if (i == hn && e.x < hp[i - 1].x) { hp[h] = hp[i - 1]; h = i - 1; }
        hp[h] = e;
    }
    __device__ void pop()
    {
        const int2 e = hp[hn - 1];
        hn -= 1;
        if (hn > 0) toward_leaves(e, 0, 2);
    }
    __device__ __forceinline__ void print(int64_t size, int tv)
    {
        tsz[nt] = int32_t(size);
        ttv[nt] = tv;
        ++nt;
    }

    // _alignBandedSmithWaterman (:69-200): the heap's top score, or 0
    __device__ int32_t fill()
    {
        const int32_t gap = a->gap, cutoff = a->cutoff;
        int64_t it = W, it2 = 0;
        for (int64_t row = 1; row < height_fill; ++row) {
            const int64_t ar = row + lo_row;
            int32_t hori = 0;
            for (int64_t col = 0; col < W; ++col, ++it) {
                const int64_t ac = col + lo + ar;
                if (ac < 0 || ac > len1) { ++it2; continue; }
                if (ac != 0) {
                    int32_t val = M[it2] + sc(ac - 1, ar - 1);
                    ++it2;
                    if (col < W - 1) { const int32_t vv = M[it2] + gap; if (vv > val) val = vv; }
                    if (col > 0) { hori += gap; if (hori > val) val = hori; }
                    if (val < 0) val = 0;
                    M[it] = val;
                    if (val >= cutoff) push(make_int2(val, int32_t(it)));
                } else {
                    ++it2;
                }
                hori = M[it];
            }
        }
        if (hn > 0) { best_end = hp[0].y; return hp[0].x; }
        return 0;
    }

    // _alignBandedSmithWatermanTrace (:369-468) from best_end
    __device__ void trace()
    {
        const int32_t gap = a->gap;
        int64_t it = best_end, it2 = best_end - W;
        int64_t row = it / W, col = it % W, ar, ac, segLen = 0;
        int tv, next;
        nt = 0;
        eRow = row + lo_row;
        eCol = col + lo + eRow;
        ar = eRow;
        ac = eCol;
        if (ac == 0 || ar == 0) { aCol = eCol = aRow = eRow = 0; return; }
        if (ac < len1) print(len1 - ac, WB_HORI);
        if (ar < len2) print(len2 - ar, WB_VERT);
        next = WB_HORI;
        while (next != WB_STOP) {
            tv = next;
            if (it < 0 || it >= cells) { status = 1; return; }
            if (M[it] == 0) {
                next = WB_STOP;
            } else if (it2 < 0 || it2 + 1 >= cells || ac <= 0 || ar <= 0 || ac > len1 || ar > len2) {
                status = 1;
                return;
            } else if (M[it] == M[it2] + sc(ac - 1, ar - 1)) {
                next = WB_DIAG;
                --ar; --ac; --row;
                it -= W; it2 -= W;
            } else if (M[it] == M[it2 + 1] + gap) {
                next = WB_VERT;
                --ar; --row; ++col;
                it += 1 - W; it2 += 1 - W;
            } else {
                next = WB_HORI;
                --ac; --col;
                it -= 1; it2 -= 1;
            }
            if (tv == next) ++segLen;
            else { print(segLen, tv); segLen = 1; }
        }
        if (ac != 0) print(ac, WB_HORI);
        if (ar != 0) print(ar, WB_VERT);
        best_begin = it + W;
        aCol = ac;
        aRow = ar;
    }

    // _alignBandedSmithWatermanDeclump (:203-362)
    __device__ void declump()
    {
        const int32_t gap = a->gap, cutoff = a->cutoff;
        int64_t it = best_begin, it2;
        int64_t minCol = W, newMinCol = W, maxCol = 0, newMaxCol = 0;
        int64_t row = it / W, col = it % W, traceCol = col, tracePos = nt, traceSize;
        int traceValue;
        it -= col;
        while (tracePos > 0 && ttv[tracePos - 1] != WB_DIAG) --tracePos;
        if (tracePos == 0) return;
        traceSize = tsz[tracePos - 1];
        traceValue = ttv[tracePos - 1];
        while (row < height_fill && (maxCol > minCol || tracePos > 0)) {
            const int64_t ar = row + lo_row;
            while (traceSize == 0 && tracePos > 1) {
                --tracePos;
                traceValue = ttv[tracePos - 1];
                if (traceValue == WB_HORI) traceCol += tsz[tracePos - 1];
                else traceSize = tsz[tracePos - 1];
            }
            if (tracePos > 0) {
                if (traceValue == WB_DIAG) {
                    const int64_t f = row * W + traceCol;
                    --traceSize;
                    if (f < 0 || f >= cells) { status = 1; return; }
                    F[f] = 1;
                    if (traceCol < minCol) minCol = traceCol;
                    if (traceCol + 1 > maxCol) maxCol = traceCol + 1;
                } else if (traceValue == WB_VERT) {
                    if (traceCol > 0) --traceCol;
                    --traceSize;
                }
                if (traceCol >= maxCol) maxCol = traceCol + 1;
            }
            if (maxCol > minCol) {
                col = minCol;
                it += col;
                it2 = it - W;
                while (col < maxCol) {
                    const int64_t ac = col + lo + ar;   // unsigned in the reference: negative ends the row
                    int32_t nv = 0;
                    if (ac < 0 || ac > len1) break;
                    if (it < 0 || it >= cells || it2 < 0 || it2 + 1 >= cells) { status = 1; return; }
                    if (!F[it]) {
                        if (ac == 0) { status = 1; return; }   // the reference reads H[-1]
                        const int32_t d = M[it2] + sc(ac - 1, ar - 1);
                        if (d > nv) nv = d;
                    }
                    ++it2;
                    if (col > 0) { const int32_t hh = M[it - 1] + gap; if (hh > nv) nv = hh; }
                    if (col + 1 < maxCol) { const int32_t vv = M[it2] + gap; if (vv > nv) nv = vv; }
                    if (nv != M[it]) {
                        M[it] = nv;
                        maxCol = maxCol > col + 2 ? maxCol : col + 2;
                        if (maxCol > W) maxCol = W;
                        if (col + 1 > newMaxCol) newMaxCol = col + 1;
                        newMinCol = col != 0 ? (newMinCol < col - 1 ? newMinCol : col - 1) : 0;
                        if (nv >= cutoff) push(make_int2(nv, int32_t(it)));
                    } else if (col == minCol) {
                        ++minCol;
                    }
                    ++col;
                    ++it;
                }
                it += W - col;
            } else {
                it += W;
            }
            minCol = newMinCol > 0 ? newMinCol : 0;
            maxCol = newMaxCol < W ? newMaxCol : W;
            newMinCol = W;
            newMaxCol = 0;
            ++row;
        }
    }

    // _getNextBestEndPosition; 0 means none
    __device__ int64_t next_end()
    {
        int32_t top = 0;
        if (hn > 0) top = M[hp[0].y];
        if (hn > 0) {
            while (hp[0].x != top) {
                if (top >= a->cutoff) {
                    hp[0].x = top;
                    toward_leaves(hp[0], 0, 2);
                } else {
                    pop();
                }
                if (hn > 0) top = M[hp[0].y];
                else break;
            }
        }
        if (hn == 0) return 0;
        const int64_t ret = hp[0].y;
        best_end = ret;
        pop();
        return ret;
    }

    // The alignment's columns (the trace runs in alignment order, _pumpTraceToGaps) clipped to
    // the union of the two rows' views: from the column of the first residue at or after
    // (aCol, aRow) of each row to the column after its residue eCol - 1 / eRow - 1.
    __device__ int32_t emit(uint32_t *out) const
    {
        int64_t vh0 = -1, vh1 = 0, vv0 = -1, vv1 = 0, t = 0, ch = 0, cv = 0;
        for (int64_t i = nt; i > 0; --i) {
            const int64_t sz = tsz[i - 1];
            const int tv = ttv[i - 1];
            if (tv != WB_VERT) {   // h residues ch .. ch + sz - 1 at columns t .. t + sz - 1
                if (vh0 < 0 && aCol >= ch && aCol < ch + sz) vh0 = t + (aCol - ch);
                if (eCol - 1 >= ch && eCol - 1 < ch + sz) vh1 = t + (eCol - 1 - ch) + 1;
                ch += sz;
            }
            if (tv != WB_HORI) {
                if (vv0 < 0 && aRow >= cv && aRow < cv + sz) vv0 = t + (aRow - cv);
                if (eRow - 1 >= cv && eRow - 1 < cv + sz) vv1 = t + (eRow - 1 - cv) + 1;
                cv += sz;
            }
            t += sz;
        }
        if (vh0 < 0) vh0 = vh1;
        if (vv0 < 0) vv0 = vv1;
        const int64_t lo_t = vh0 < vv0 ? vh0 : vv0, hi_t = vh1 > vv1 ? vh1 : vv1;
        int32_t ns = 0;
        uint32_t cur = 0xffffffffu;
        t = 0;
        ch = 0;
        cv = 0;
        for (int64_t i = nt; i > 0; --i) {
            const int64_t sz = tsz[i - 1];
            const int tv = ttv[i - 1];
            const int64_t s0 = t > lo_t ? t : lo_t, s1 = t + sz < hi_t ? t + sz : hi_t;
            if (s1 > s0) {
                const uint32_t type = tv == WB_DIAG ? uint32_t(TV_DIAG) : (tv == WB_HORI ? uint32_t(TV_H) : uint32_t(TV_V));
                if (type == cur) {
                    out[4 * (ns - 1) + 2] += uint32_t(s1 - s0);
                } else {
                    out[4 * ns + 0] = uint32_t(ch + (tv != WB_VERT ? s0 - t : 0));
                    out[4 * ns + 1] = uint32_t(cv + (tv != WB_HORI ? s0 - t : 0));
                    out[4 * ns + 2] = uint32_t(s1 - s0);
                    out[4 * ns + 3] = type;
                    ++ns;
                    cur = type;
                }
            }
            if (tv != WB_VERT) ch += sz;
            if (tv != WB_HORI) cv += sz;
            t += sz;
        }
        return ns;
    }
};

// One thread per pair.  status: 0 done, 1 the reference's next step is undefined, 2 the heap
// needs more than heap_cap entries (the host reruns the pair with the exact bound).
__global__ void __launch_bounds__(128) k_waterman_eggert_banded(EnumArgs a, int32_t lower, int32_t upper)
{
    const int64_t p = enum_pair_of_thread(a);
    if (p < 0) return;
    const EnumPair d = a.pairs[p];
    WbState w;
    w.a = &a;
    w.H = a.seq_h + d.h_off;
    w.V = a.seq_v + d.v_off;
    w.len1 = d.m;
    w.len2 = d.n;
    w.lo = lower;
    w.W = int64_t(upper) - lower + 1;
    w.lo_row = upper <= 0 ? -int64_t(upper) : 0;
    int64_t hi_init = int64_t(d.n) + 1, hi_fill = d.n;
    if (int64_t(d.m) - lower >= 0 && int64_t(d.m) - lower < hi_init) hi_init = int64_t(d.m) - lower;
    if (int64_t(d.m) - lower >= 0 && int64_t(d.m) - lower < hi_fill) hi_fill = int64_t(d.m) - lower;
    const int64_t height_init = hi_init - w.lo_row + 1;
    w.height_fill = hi_fill - w.lo_row + 1;
    w.cells = w.W * height_init;
    w.M = a.mat + d.mat_off;
    w.F = a.forb + d.forb_off;
    w.hp = a.heap + d.heap_off;
    w.hn = 0;
    w.hcap = d.heap_cap;
    w.tsz = a.steps + d.step_off;
    w.ttv = w.tsz + (d.m + d.n + 5);
    w.nt = 0;
    w.status = 0;
    int32_t k = 0;
    if (d.m > 0 && d.n > 0 && height_init > 0 && w.height_fill > 0) {
        for (; k < a.max_count; ++k) {
            if (k == 0) {
                const int32_t s = w.fill();
                if (w.status || s < a.cutoff || s == 0) break;
                w.trace();
                w.pop();
            } else {
                w.declump();
                if (w.status) break;
                const int64_t e = w.next_end();
                if (e == 0 || w.M[e] == 0) break;
                w.trace();
            }
            if (w.status) break;
            const int64_t o = p * a.max_count + k;
            a.score[o] = w.M[w.best_end];
            a.begin_h[o] = int32_t(w.aCol);
            a.begin_v[o] = int32_t(w.aRow);
            a.end_h[o] = int32_t(w.eCol);
            a.end_v[o] = int32_t(w.eRow);
            a.seg_count[o] = w.emit(a.seg_slots + 4 * (d.seg_off + int64_t(k) * (d.m + d.n + 1)));
        }
    }
    a.count[p] = k;
    a.status[p] = w.status;
}

}  // namespace gba
