// dp_common.cuh -- shared definitions of the GB300 alignment kernels.
//
// Trace values are the reference's TraceBitMap_ bits (align/dp_profile.h:121-135) so the
// device traceback makes exactly the reference's decisions.
#pragma once

#include <climits>
#include <cstdint>
#include <cuda_runtime.h>

namespace gba {

constexpr uint8_t TV_NONE = 0;
constexpr uint8_t TV_DIAG = 1;
constexpr uint8_t TV_H = 2;
constexpr uint8_t TV_V = 4;
constexpr uint8_t TV_HO = 8;
constexpr uint8_t TV_VO = 16;
constexpr uint8_t TV_MFH = 32;
constexpr uint8_t TV_MFV = 64;

// The 4-bit trace code: bits 0-1 the source of S (0 none, 1 diagonal, 2 MAX_FROM_V, 3
// MAX_FROM_H), bit 2 "E opened" (H_OPEN without H), bit 3 "F opened" (V_OPEN without V).  With
// SingleTrace exactly one bit of each open/extend pair is set in inner cells (align/dp_formula.h:
// 179-181), and _doTraceback (align/dp_traceback_impl.h:376-450) reads nothing else, so decoding
// gives back every decision it makes; border and band-edge cells, which lack a pair, decode with
// "extend" for it.
__host__ __device__ __forceinline__ uint32_t trace4_encode(uint32_t tv)
{
    const uint32_t src = (tv & TV_DIAG) ? 1u : (tv & TV_MFV) ? 2u : (tv & TV_MFH) ? 3u : 0u;
    const uint32_t eo = ((tv & TV_HO) && !(tv & TV_H)) ? 4u : 0u;
    const uint32_t fo = ((tv & TV_VO) && !(tv & TV_V)) ? 8u : 0u;
    return src | eo | fo;
}
__host__ __device__ __forceinline__ uint8_t trace4_decode(uint32_t code, bool affine)
{
    const uint32_t src = code & 3u;
    if (src == 0) return TV_NONE;
    if (!affine) return src == 1 ? TV_DIAG : (src == 2 ? uint8_t(TV_V | TV_MFV) : uint8_t(TV_H | TV_MFH));
    const uint8_t sb = src == 1 ? TV_DIAG : (src == 2 ? TV_MFV : TV_MFH);
    return uint8_t(sb | ((code & 4u) ? TV_HO : TV_H) | ((code & 8u) ? TV_VO : TV_V));
}

constexpr int FREE_TOP = 1, FREE_LEFT = 2, FREE_RIGHT = 4, FREE_BOTTOM = 8;

// Rows per register strip of the one-pair-per-thread kernels.  16 trace bytes per strip
// column make one 16-byte store.
constexpr int STRIP_ROWS = 16;

// Per-pair descriptor (device).  Offsets index the device code buffers.
struct PairDesc {
    int64_t h_off;
    int64_t v_off;
    int64_t trace_off;   // byte offset of this pair's trace matrix (16-byte aligned)
    int32_t m;           // |H| (columns)
    int32_t n;           // |V| (rows)
    int32_t inf;         // DPCellDefaultInfinity of the cell width the pair runs with
    int32_t invalid;     // 1: empty sequence or band outside the matrix (score = numeric min)
};

// Arguments of the DP kernels, passed by value.
struct DpArgs {
    const uint8_t *seq_h;
    const uint8_t *seq_v;
    const PairDesc *pairs;
    const int32_t *order;          // thread slot -> pair index (length-binned order)
    const int64_t *warp_scratch;   // per warp: int2 offset of its interleaved boundary rows
    int2 *scratch;
    uint8_t *trace;
    int32_t *score;
    int32_t *end_h;
    int32_t *end_v;
    int32_t *best_e;               // E and F of the best cell (start-cell trace correction)
    int32_t *best_f;
    const int32_t *matrix;         // alphabet^2 table or nullptr
    int64_t num_slots;
    int32_t match, mismatch, gap_open, gap_extend;
    int32_t free_ends;
    int32_t alphabet;
};

struct TraceArgs {
    const PairDesc *pairs;
    const int32_t *order;
    const uint8_t *trace;
    const int32_t *score;
    const int32_t *end_h;
    const int32_t *end_v;
    const int32_t *best_e;
    const int32_t *best_f;
    int32_t *begin_h;
    int32_t *begin_v;
    uint32_t *seg_slots;           // 4 words per segment, slot of pair k at seg_slot_off[k]
    const int64_t *seg_slot_off;
    int32_t *seg_count;
    uint32_t *cigar_slots;
    const int64_t *cigar_slot_off;
    int32_t *cigar_count;
    int64_t num_slots;
    int32_t affine;
    int32_t local;
    int32_t band_w;        // banded layout: slots per column (0: not banded)
    int32_t band_upper;
    int32_t warp_rows;     // warp layout: rows per lane strip (0: not the warp layout)
    int32_t warp2;         // 1: the packed 16-bit warp layout with 4-bit cells (dp_warp2_kernels.cuh)
    int32_t dynamic;       // 1: DynamicGaps cells; best_e holds the best cell's gap flags
    int32_t extend;        // 1: AlignExtend_ (TraceHead_ but no TraceTail_, align_extend_base.h:67-73)
};

__host__ __device__ inline int64_t align16(int64_t x) { return (x + 15) & ~int64_t(15); }

// Trace layout of one pair: row 0 as m+1 bytes (padded to 16), then rows 1..n in strips of
// STRIP_ROWS rows; strip s stores column j's STRIP_ROWS bytes contiguously at
// (s * (m + 1) + j) * STRIP_ROWS.
__host__ __device__ inline int64_t trace_bytes(int m, int n)
{
    int64_t strips = (n + STRIP_ROWS - 1) / STRIP_ROWS;
    return align16(m + 1) + strips * int64_t(m + 1) * STRIP_ROWS;
}

__device__ __forceinline__ uint8_t trace_at(const uint8_t *base, int m, int col, int row)
{
    if (row == 0) return base[col];
    int r = row - 1;
    int s = r / STRIP_ROWS;
    int k = r - s * STRIP_ROWS;
    return base[align16(m + 1) + (int64_t(s) * (m + 1) + col) * STRIP_ROWS + k];
}

}  // namespace gba
