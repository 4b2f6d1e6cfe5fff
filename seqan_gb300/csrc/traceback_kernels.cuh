// traceback_kernels.cuh -- device traceback: trace matrix -> TraceSegment_ list -> CIGAR.
//
// One thread per pair walks back from the best cell exactly as the reference does:
//   start-cell correction          align/dp_algorithm_impl.h:1188-1205 (affine only)
//   initial direction              align/dp_traceback_impl.h:456-483 (PreferGapsAtEnd_ for affine)
//   tail / head gap segments       align/dp_traceback_impl.h:522-545 (global only; the
//                                  AlignExtend_ profile records the head only)
//   walk order and gap walkers     align/dp_traceback_impl.h:190-450 (GapsLeft)
//   segment recording              align/dp_trace_segment.h:318-337
// and writes the segments in the reference's order (traceback order).  Pairs of the warp layout
// with at least kTiledTraceCells cells are walked by a whole warp instead: every lane runs the
// same walk, and the trace is read from a shared-memory tile of kTraceTileSteps steps of the
// current band that the warp reloads together (coalesced) when the walk leaves it; lane 0
// writes the outputs.  The CIGAR is the
// run-length form of the same alignment columns that getCigarString iterates
// (bam_io/cigar.h:261-339): DIAGONAL -> M, VERTICAL (gap in H) -> I, HORIZONTAL -> D, and a
// D run of at least 20 becomes N.
#pragma once

#include "dp_common.cuh"
#include "dp_banded_kernels.cuh"
#include "dp_warp_kernels.cuh"
#include "dp_warp2_kernels.cuh"

namespace gba {

struct SegWriter {
    uint32_t *out;
    int cap;
    int n;
    bool leader;       // writes the records (all lanes of a warp walk keep the count)
    __device__ __forceinline__ void record(int hb, int vb, int len, int tv)
    {
        if (len == 0) return;
        uint32_t type;
        if (tv & TV_DIAG) type = TV_DIAG;
        else if (tv & TV_V) type = TV_V;
        else if (tv & TV_H) type = TV_H;
        else return;
        if (leader && n < cap) {
            uint32_t *o = out + 4 * int64_t(n);
            o[0] = uint32_t(hb);
            o[1] = uint32_t(vb);
            o[2] = uint32_t(len);
            o[3] = type;
        }
        ++n;
    }
};

// Walks pair p back from its best cell; TAT(col, row) reads one trace byte.  With leader false
// the walk only counts (the other lanes of a warp walk).
template <typename Cell>
__device__ __forceinline__ void traceback_pair(const TraceArgs &a, int p, Cell &TAT, bool leader)
{
    const PairDesc d = a.pairs[p];
    const int m = d.m, n = d.n;
    int col = a.end_h[p], row = a.end_v[p];
    const bool affine = a.affine != 0;
    const bool global = a.local == 0;

    SegWriter w;
    w.out = a.seg_slots + 4 * a.seg_slot_off[p];
    w.cap = int(a.seg_slot_off[p + 1] - a.seg_slot_off[p]);
    w.n = 0;
    w.leader = leader;

    int tv = TAT(col, row);
    if (affine) {
        const int s = a.score[p];
        if (a.best_f[p] == s) { tv &= ~TV_DIAG; tv |= TV_MFV; }
        else if (a.best_e[p] == s) { tv &= ~TV_DIAG; tv |= TV_MFH; }
    } else if (a.dynamic) {
        // DynamicGaps: the best cell's flags (vertical first) decide
        // (align/dp_algorithm_impl.h:1235-1249).
        const int fl = a.best_e[p];
        if (fl & 1) { tv &= ~TV_DIAG; tv |= TV_MFV; }
        else if (fl & 2) { tv &= ~TV_DIAG; tv |= TV_MFH; }
    }
    int last;
    if (affine) {
        if (tv & TV_MFV) { tv &= (TV_V | TV_VO | TV_MFV); last = TV_V; }
        else if (tv & TV_MFH) { tv &= (TV_H | TV_HO | TV_MFH); last = TV_H; }
        else last = TV_DIAG;
    } else {
        if (tv & TV_DIAG) last = TV_DIAG;
        else if (tv & (TV_V | TV_MFV)) last = TV_V;
        else if (tv & (TV_H | TV_MFH)) last = TV_H;
        else last = TV_NONE;
    }
    if (global && !a.extend) {
        if (row != n) w.record(m, row, n - row, TV_V);
        if (col != m) w.record(col, row, m - col, TV_H);
    }
    int frag = 0;
    // Every step moves left or up, so the walk ends after at most m + n steps.
    while (!(col <= 0 || row <= 0) && tv != TV_NONE) {
        if (tv & TV_DIAG) {
            if (!(last & TV_DIAG)) { w.record(col, row, frag, last); last = TV_DIAG; frag = 0; }
            --col; --row; tv = TAT(col, row); ++frag;
        } else if ((tv & TV_MFV) && (tv & TV_V)) {
            if (!(last & TV_V)) { w.record(col, row, frag, last); last = TV_V; frag = 0; }
            if (affine) {
                while ((!(tv & TV_VO) || (tv & TV_V)) && row != 1) {
                    --row; tv = TAT(col, row); ++frag;
                }
            }
            --row; tv = TAT(col, row); ++frag;
        } else if ((tv & TV_MFV) && (tv & TV_VO)) {
            if (!(last & TV_V)) { w.record(col, row, frag, last); last = TV_V; frag = 0; }
            --row; tv = TAT(col, row); ++frag;
        } else if ((tv & TV_MFH) && (tv & TV_H)) {
            if (!(last & TV_H)) { w.record(col, row, frag, last); last = TV_H; frag = 0; }
            if (affine) {
                while ((!(tv & TV_HO) || (tv & TV_H)) && col != 1) {
                    --col; tv = TAT(col, row); ++frag;
                }
            }
            --col; tv = TAT(col, row); ++frag;
        } else if ((tv & TV_MFH) && (tv & TV_HO)) {
            if (!(last & TV_H)) { w.record(col, row, frag, last); last = TV_H; frag = 0; }
            --col; tv = TAT(col, row); ++frag;
        } else {
            break;
        }
    }
    w.record(col, row, frag, last);
    if (global) {
        if (row != 0) w.record(0, 0, row, TV_V);
        if (col != 0) w.record(0, 0, col, TV_H);
    }
    if (!leader) return;
    a.seg_count[p] = w.n;
    if (w.n > 0 && w.n <= w.cap) {
        const uint32_t *lastSeg = w.out + 4 * int64_t(w.n - 1);
        a.begin_h[p] = int32_t(lastSeg[0]);
        a.begin_v[p] = int32_t(lastSeg[1]);
    } else {
        a.begin_h[p] = 0;
        a.begin_v[p] = 0;
    }

    // CIGAR: walk the segments in alignment order (reverse of the list).
    if (a.cigar_slots && w.n <= w.cap) {
        uint32_t *co = a.cigar_slots + a.cigar_slot_off[p];
        const int ccap = int(a.cigar_slot_off[p + 1] - a.cigar_slot_off[p]);
        int nc = 0;
        int curOp = -1;
        uint32_t curLen = 0;
        for (int k = w.n - 1; k >= -1; --k) {
            int op = -1;
            uint32_t len = 0;
            if (k >= 0) {
                const uint32_t *sg = w.out + 4 * int64_t(k);
                len = sg[2];
                op = sg[3] == TV_DIAG ? 0 : (sg[3] == TV_V ? 1 : 2);  // M, I, D
            }
            if (op != curOp) {
                if (curLen > 0) {
                    int emit = (curOp == 2 && curLen >= 20) ? 3 : curOp;  // N
                    if (nc < ccap) co[nc] = (curLen << 4) | uint32_t(emit);
                    ++nc;
                }
                curOp = op;
                curLen = 0;
            }
            curLen += len;
        }
        a.cigar_count[p] = nc;
    } else if (a.cigar_slots) {
        a.cigar_count[p] = 0;
    }
}

__global__ void __launch_bounds__(128) k_traceback(TraceArgs a)
{
    const int64_t slot = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (slot >= a.num_slots) return;
    const int p = a.order[slot];
    if (p < 0) return;   // padding slot
    const PairDesc d = a.pairs[p];
    const int m = d.m;
    const uint8_t *T = a.trace + d.trace_off;
    const int bw = a.band_w, bu = a.band_upper, wr = a.warp_rows;
    const bool w2 = a.warp2 != 0, affine = a.affine != 0;
    auto TAT = [&](int c, int r) -> int {
        if (w2) return int(trace_at_warp2(T, m, d.n, affine, c, r));
        if (wr) return int(trace_at_warp(T, m, d.n, wr, c, r));
        return bw ? int(trace_at_band(T, d.trace_off, bw, bu, affine, c, r)) : int(trace_at(T, m, c, r));
    };
    traceback_pair(a, p, TAT, true);
}

constexpr int kTraceTileSteps = 64;             // steps of one band held in shared memory
constexpr int64_t kTiledTraceCells = 1 << 20;   // pairs at least this large are walked by a warp

// Trace reader of the warp layout (dp_warp_kernels.cuh) through a shared-memory tile: steps
// [t0, t0 + kTraceTileSteps) of band tb, each step 32 * Rb bytes (Rb: the band's rows per lane,
// R or, for a short last band, R / 2).  Called by all 32 lanes with the same cell; a miss
// reloads the tile ending at the requested step (the walk only moves to earlier steps).
template <int R>
struct TileCell {
    const uint8_t *T;
    int m, n;
    uint4 *tile;
    int tb, t0;
    __device__ __forceinline__ int operator()(int col, int row)
    {
        if (row == 0) return T[col];
        const int r0 = row - 1;
        const int b = r0 / (32 * R);
        const int Rb = (b == (n - 1) / (32 * R)) ? warp_last_rows(n, R) : R;
        const int within = r0 - b * 32 * R;
        const int ln = within / Rb;
        const int t = col + ln;
        if (b != tb || t < t0 || t >= t0 + kTraceTileSteps) {
            tb = b;
            t0 = max(0, t - kTraceTileSteps + 1);
            const int steps = min(kTraceTileSteps, m + 32 - t0);
            const uint4 *src = reinterpret_cast<const uint4 *>(T + warp_band_trace_off(m, b, R) + int64_t(t0) * 32 * Rb);
            const int lane = threadIdx.x & 31;
            __syncwarp();
            for (int q = lane; q < steps * 2 * Rb; q += 32) tile[q] = __ldcs(src + q);
            __syncwarp();
        }
        return reinterpret_cast<const uint8_t *>(tile)[(t - t0) * 32 * Rb + within];
    }
};

template <int R>
__global__ void __launch_bounds__(64) k_traceback_tiled(TraceArgs a)
{
    __shared__ uint4 tiles[2][kTraceTileSteps * 2 * R];
    const int64_t slot = int64_t(blockIdx.x) * 2 + (threadIdx.x >> 5);
    if (slot >= a.num_slots) return;
    const int p = a.order[slot];
    if (p < 0) return;
    const PairDesc d = a.pairs[p];
    TileCell<R> cell{a.trace + d.trace_off, d.m, d.n, tiles[threadIdx.x >> 5], -1, 0};
    traceback_pair(a, p, cell, (threadIdx.x & 31) == 0);
}

// Packs per-pair slot outputs densely: dst[off[k] ..] = src[slot_off[k] .. + count[k]].
__global__ void k_compact_u32(const uint32_t *src, const int64_t *slot_off, const int32_t *count,
                              const int64_t *dense_off, uint32_t *dst, int64_t num_pairs, int words)
{
    const int64_t p = int64_t(blockIdx.x) * (blockDim.x / 32) + (threadIdx.x / 32);
    if (p >= num_pairs) return;
    const int lane = threadIdx.x & 31;
    const int64_t cnt = int64_t(count[p]) * words;
    const uint32_t *s = src + slot_off[p] * words;
    uint32_t *d = dst + dense_off[p] * words;
    for (int64_t i = lane; i < cnt; i += 32) d[i] = s[i];
}

}  // namespace gba
