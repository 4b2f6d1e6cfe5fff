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
};

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
    const int64_t p = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (p >= a.num_pairs) return;
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

}  // namespace gba
