/*
 * seqan_oracle.c -- CPU restatement of SeqAn 2's pairwise DP.
 *
 * TEST INFRASTRUCTURE ONLY: this is the checker the GPU engine is compared against and
 * the CPU baseline timed beside it.  Nothing in seqan_gb300/ links or calls it.
 *
 * What is restated, with the reference lines each part follows (paths are relative to
 * the SeqAn 2 source tree):
 *   - column-major DP with one sparse score column and per-column diagonal/vertical
 *     caches: align/dp_algorithm_impl.h:334-429 (_computeTrack) and :483-579
 *     (unbanded _computeAlignmentImpl); banded columns :586-967.
 *   - affine recurrences per recursion direction: align/dp_formula_affine.h:66-330;
 *     linear: align/dp_formula_linear.h:62-258; Zero/Diagonal: align/dp_formula.h:249-309.
 *   - tie rule of _maxScore with SingleTrace (left operand wins ties):
 *     align/dp_formula.h:171-182.
 *   - which cell uses which direction and which cells are tracked:
 *     align/dp_meta_info.h:178-370.
 *   - "infinity" = lowest()/2 of the cell type: align/dp_cell.h:126-146.
 *   - best-cell scout with strict '>': align/dp_scout.h:166-180.
 *   - start-cell trace correction: align/dp_algorithm_impl.h:1188-1205.
 *   - traceback walk, initial direction and head/tail segments:
 *     align/dp_traceback_impl.h:190-546; segment recording align/dp_trace_segment.h:318-337.
 *   - invalid settings return numeric_limits<T>::min(): align/dp_algorithm_impl.h:183-256,
 *     :1399-1400.
 * With score_bits == 16 every sum is wrapped to int16, as the reference's int16 SIMD lanes
 * do (simd/simd_base_seqan_impl_avx2.h add_epi16 semantics).
 */
#include "seqan_oracle.h"

#include <limits.h>
#include <stdlib.h>
#include <stdio.h>
#include <string.h>
#include <omp.h>

#define TV_NONE 0
#define TV_DIAG 1
#define TV_H 2
#define TV_V 4
#define TV_HO 8
#define TV_VO 16
#define TV_MFH 32
#define TV_MFV 64

enum { DIR_ZERO, DIR_ALL, DIR_HORIZONTAL, DIR_VERTICAL, DIR_UPPER, DIR_LOWER };

typedef struct {
    int bits16;
    int inf;
    int local;
    int extend;     /* AlignExtend_: every cell tracked, no zero floor */
    int complete;   /* CompleteTrace: ties keep every source's trace bits (dp_formula.h:205-220) */
    int affine;
    int dynamic;    /* DynamicGaps: one score and two gap-extension flags per cell */
    int ext, open;
    int match, mismatch;
    const int32_t *mat;
    int asz;
} ctx_t;

static inline int wr(const ctx_t *c, long x)
{
    return c->bits16 ? (int)(int16_t)(uint16_t)(x & 0xffff) : (int)x;
}

static inline int sub_score(const ctx_t *c, uint8_t hv, uint8_t vv)
{
    if (c->mat) return c->mat[(int)hv * c->asz + (int)vv];
    return hv == vv ? c->match : c->mismatch;
}

/* _maxScore with SingleTrace: the left operand wins ties (align/dp_formula.h:171-182); with
 * CompleteTrace a tie keeps the left value and the union of both traces (:205-220). */
#define MAXTL(target, tv, left, right, tl, tr) \
    do { if ((left) < (right)) { (target) = (right); (tv) = (tr); } \
         else if (c->complete && (left) == (right)) { (target) = (left); (tv) = (tl) | (tr); } \
         else { (target) = (left); (tv) = (tl); } } while (0)

/* Per-column caches and the one sparse column (align/dp_matrix.h:137-147). */
typedef struct {
    int dS;          /* cacheDiag._score */
    int vS, vF;      /* cacheVert._score, cacheVert._verticalScore */
} caches_t;

/* DynamicGaps cell flags (align/dp_cell_dynamic.h: MASK_VERTICAL_GAP, MASK_HORIZONTAL_GAP). */
#define DYN_V 1
#define DYN_H 2

/* One DynamicGaps cell (align/dp_formula_dynamic.h, scalar SingleTrace overloads).  A cell holds a
 * score and two flags telling whether it ends in a vertical / horizontal gap; a gap from a
 * neighbour is extended when the neighbour's flag for that direction is set, else opened.
 * colS/colE hold the previous column's score and flags at row i; k->vS / k->vF the cell above. */
static inline int compute_cell_dynamic(const ctx_t *c, int dir, int *colS, int *colE, caches_t *k,
                                       uint8_t hv, uint8_t vv, int *fOut)
{
    int tv = TV_NONE, s = 0, fl = 0, tmp, tvGap;
    const int hS = *colS, hF = *colE;
    switch (dir) {
    case DIR_ZERO:   /* align/dp_formula_dynamic.h: RecursionDirectionZero */
        *colS = 0;
        *colE = 0;
        k->dS = 0;
        k->vS = 0;
        k->vF = 0;
        *fOut = 0;
        return TV_NONE;
    case DIR_ALL: {  /* _computeScore [RecursionDirectionAll, DynamicGaps] */
        int inter = wr(c, (long)k->dS + sub_score(c, hv, vv));
        k->dS = hS;
        if (hF & DYN_H) { tmp = wr(c, (long)hS + c->ext); tvGap = TV_H; }
        else { tmp = wr(c, (long)hS + c->open); tvGap = TV_HO; }
        if (k->vF & DYN_V) { s = wr(c, (long)k->vS + c->ext); tvGap |= TV_V; }
        else { s = wr(c, (long)k->vS + c->open); tvGap |= TV_VO; }
        if (s < tmp) { s = tmp; fl = DYN_H; tv = TV_MFH; }
        else { fl = DYN_V; tv = TV_MFV; }
        if (s <= inter) { s = inter; fl = 0; tv = TV_DIAG | tvGap; }
        else tv = tvGap | tv;
        break;
    }
    case DIR_HORIZONTAL:   /* row 0: extend when the left cell ended in a horizontal gap */
        k->dS = hS;
        fl = DYN_H;
        if (hF & DYN_H) { s = wr(c, (long)hS + c->ext); tv = TV_H; }
        else { s = wr(c, (long)hS + c->open); tv = TV_HO; }
        tv |= TV_MFH;
        *colS = s;
        *colE = fl;
        k->vS = s;
        k->vF = fl;
        *fOut = fl;
        return tv;         /* no zero floor in this overload */
    case DIR_VERTICAL:     /* column 0 */
        fl = DYN_V;
        if (k->vF & DYN_V) { s = wr(c, (long)k->vS + c->ext); tv = TV_V; }
        else { s = wr(c, (long)k->vS + c->open); tv = TV_VO; }
        tv |= TV_MFV;
        break;
    case DIR_UPPER: {      /* banded: no vertical predecessor */
        int inter = wr(c, (long)k->dS + sub_score(c, hv, vv));
        k->dS = hS;
        if (hF & DYN_H) { s = wr(c, (long)hS + c->ext); tv = TV_H; }
        else { s = wr(c, (long)hS + c->open); tv = TV_HO; }
        fl = DYN_H;
        if (s <= inter) { s = inter; fl = 0; tv = TV_DIAG | tv; }
        else tv = tv | TV_MFH;
        break;
    }
    default: {             /* DIR_LOWER: no horizontal predecessor; the cell above is kept */
        if (k->vF & DYN_V) { s = wr(c, (long)k->vS + c->ext); tv = TV_V; }
        else { s = wr(c, (long)k->vS + c->open); tv = TV_VO; }
        fl = DYN_V;
        tmp = wr(c, (long)k->dS + sub_score(c, hv, vv));
        if (s <= tmp) { s = tmp; fl = 0; tv = TV_DIAG | tv; }
        else tv = tv | TV_MFV;
        break;
    }
    }
    if (c->local) {
        /* _maxScore(score, NONE, score, NONE, tv): 0 wins ties; the flags stay as they are. */
        if (!(0 < s)) { s = 0; tv = TV_NONE; }
    }
    *colS = s;
    *colE = fl;
    if (dir != DIR_LOWER) { k->vS = s; k->vF = fl; }
    *fOut = fl;
    return tv;
}

/* Computes one cell in place.  colS/colE hold the previous column's S/E at row i on entry
 * (the sparse matrix cell) and this column's on exit.  Returns the trace value. */
static inline int compute_cell(const ctx_t *c, int dir, int *colS, int *colE, caches_t *k,
                               uint8_t hv, uint8_t vv, int *fOut)
{
    int tv = TV_NONE, t2, s, e, f;
    int hS = *colS, hE = *colE;   /* previous horizontal cell (same row, previous column) */

    if (c->dynamic) return compute_cell_dynamic(c, dir, colS, colE, k, hv, vv, fOut);
    switch (dir) {
    case DIR_ZERO:
        /* align/dp_formula.h:295-309: score 0; E of the cell and F of cacheVert stay. */
        s = 0;
        *colS = 0;
        k->dS = 0;
        k->vS = 0;
        *fOut = k->vF;
        return TV_NONE;
    case DIR_ALL:
        if (c->affine) {
            int inter = wr(c, (long)k->dS + sub_score(c, hv, vv));
            k->dS = hS;
            MAXTL(e, tv, wr(c, (long)hE + c->ext), wr(c, (long)hS + c->open), TV_H, TV_HO);
            MAXTL(f, t2, wr(c, (long)k->vF + c->ext), wr(c, (long)k->vS + c->open), TV_V, TV_VO);
            tv |= t2;
            {
                int tmp2;
                MAXTL(s, tmp2, f, e, TV_MFV, TV_MFH);
                MAXTL(s, tv, inter, s, TV_DIAG | tv, tmp2 | tv);
            }
            k->vF = f;
        } else {
            int inter = wr(c, (long)k->dS + sub_score(c, hv, vv));
            k->dS = hS;
            MAXTL(s, tv, wr(c, (long)k->vS + c->ext), wr(c, (long)hS + c->ext),
                  TV_V | TV_MFV, TV_H | TV_MFH);
            MAXTL(s, tv, inter, s, TV_DIAG, tv);
            e = hE;
        }
        break;
    case DIR_HORIZONTAL:
        if (c->affine) {
            k->dS = hS;
            MAXTL(e, tv, wr(c, (long)hE + c->ext), wr(c, (long)hS + c->open), TV_H, TV_HO);
            tv |= TV_MFH;
            k->vF = c->inf;
            s = e;
        } else {
            k->dS = hS;
            s = wr(c, (long)hS + c->ext);
            tv = TV_H | TV_MFH;
            e = hE;
        }
        break;
    case DIR_VERTICAL:
        if (c->affine) {
            MAXTL(f, tv, wr(c, (long)k->vF + c->ext), wr(c, (long)k->vS + c->open), TV_V, TV_VO);
            tv |= TV_MFV;
            k->vF = f;
            e = c->inf;
            s = f;
        } else {
            s = wr(c, (long)k->vS + c->ext);
            tv = TV_V | TV_MFV;
            e = hE;
        }
        break;
    case DIR_UPPER:
        if (c->affine) {
            int inter = wr(c, (long)k->dS + sub_score(c, hv, vv));
            k->dS = hS;
            MAXTL(e, tv, wr(c, (long)hE + c->ext), wr(c, (long)hS + c->open), TV_H, TV_HO);
            k->vF = c->inf;
            MAXTL(s, tv, inter, e, tv | TV_DIAG, tv | TV_MFH);
        } else {
            int inter = wr(c, (long)k->dS + sub_score(c, hv, vv));
            k->dS = hS;
            MAXTL(s, tv, inter, wr(c, (long)hS + c->ext), TV_DIAG, TV_H | TV_MFH);
            e = hE;
        }
        break;
    default: /* DIR_LOWER */
        if (c->affine) {
            MAXTL(f, tv, wr(c, (long)k->vF + c->ext), wr(c, (long)k->vS + c->open), TV_V, TV_VO);
            k->vF = f;
            e = c->inf;
            MAXTL(s, tv, wr(c, (long)k->dS + sub_score(c, hv, vv)), f, tv | TV_DIAG, tv | TV_MFV);
        } else {
            MAXTL(s, tv, wr(c, (long)k->dS + sub_score(c, hv, vv)), wr(c, (long)k->vS + c->ext),
                  TV_DIAG, TV_V | TV_MFV);
            e = hE;
        }
        break;
    }
    if (c->local) {
        /* align/dp_formula_affine.h:113-122: max(0, S) with 0 winning ties. */
        int t3;
        MAXTL(s, t3, 0, s, TV_NONE, tv);
        tv = t3;
    }
    *colS = s;
    *colE = e;
    /* cacheVert follows the current cell, except in LowerDiagonal, which leaves it
     * (align/dp_formula_affine.h:196-238, dp_formula_linear.h:154-186). */
    if (dir != DIR_LOWER) k->vS = s;
    *fOut = k->vF;
    return tv;
}

typedef struct {
    int s, e, f;
    int col, row;
} best_t;

static inline void scout(best_t *b, int s, int e, int f, int col, int row)
{
    if (s > b->s) { b->s = s; b->e = e; b->f = f; b->col = col; b->row = row; }
}

/* ---------------------------------------------------------------------------------
 * Traceback (align/dp_traceback_impl.h:190-546).
 * ------------------------------------------------------------------------------- */

typedef struct {
    orc_segment *segs;
    int cap, n, overflow;
} segbuf_t;

static void record(segbuf_t *sb, int hb, int vb, int len, int tv)
{
    int type;
    if (len == 0) return;
    if (tv & TV_DIAG) type = ORC_SEG_DIAGONAL;
    else if (tv & TV_V) type = ORC_SEG_VERTICAL;
    else if (tv & TV_H) type = ORC_SEG_HORIZONTAL;
    else return;
    if (sb->n >= sb->cap) { sb->overflow = 1; return; }
    sb->segs[sb->n].h_begin = (uint32_t)hb;
    sb->segs[sb->n].v_begin = (uint32_t)vb;
    sb->segs[sb->n].length = (uint32_t)len;
    sb->segs[sb->n].type = (uint32_t)type;
    sb->n++;
}

/* Banded traceback bookkeeping of TracebackCoordinator_ (align/dp_traceback_impl.h:57-171)
 * is not needed here because the trace matrix is stored dense in (column, row). */
static void traceback(const ctx_t *c, const uint8_t *T, int n, int m, int col, int row,
                      segbuf_t *sb, int tail, int head)
{
#define TAT(cc, rr) T[(size_t)(cc) * (size_t)(n + 1) + (size_t)(rr)]
    int tv = TAT(col, row);
    int last;
    int frag = 0;

    /* _retrieveInitialTraceDirection (:456-483); PreferGapsAtEnd_ is true for affine. */
    if (c->affine) {
        if (tv & TV_MFV) { tv &= (TV_V | TV_VO | TV_MFV); last = TV_V; }
        else if (tv & TV_MFH) { tv &= (TV_H | TV_HO | TV_MFH); last = TV_H; }
        else last = TV_DIAG;
    } else {
        if (tv & TV_DIAG) last = TV_DIAG;
        else if (tv & (TV_V | TV_MFV)) last = TV_V;
        else if (tv & (TV_H | TV_MFH)) last = TV_H;
        else last = TV_NONE;
    }

    if (tail) { /* TraceTail_ (:522-530) */
        if (row != n) record(sb, m, row, n - row, TV_V);
        if (col != m) record(sb, col, row, m - col, TV_H);
    }

    while (!(col <= 0 || row <= 0) && tv != TV_NONE) {
        if (tv & TV_DIAG) {
            if (!(last & TV_DIAG)) { record(sb, col, row, frag, last); last = TV_DIAG; frag = 0; }
            --col; --row; tv = TAT(col, row); ++frag;
        } else if ((tv & TV_MFV) && (tv & TV_V)) {
            if (!(last & TV_V)) { record(sb, col, row, frag, last); last = TV_V; frag = 0; }
            if (c->affine) {
                while ((!(tv & TV_VO) || (tv & TV_V)) && row != 1) {
                    --row; tv = TAT(col, row); ++frag;
                }
            }
            --row; tv = TAT(col, row); ++frag;
        } else if ((tv & TV_MFV) && (tv & TV_VO)) {
            if (!(last & TV_V)) { record(sb, col, row, frag, last); last = TV_V; frag = 0; }
            --row; tv = TAT(col, row); ++frag;
        } else if ((tv & TV_MFH) && (tv & TV_H)) {
            if (!(last & TV_H)) { record(sb, col, row, frag, last); last = TV_H; frag = 0; }
            if (c->affine) {
                while ((!(tv & TV_HO) || (tv & TV_H)) && col != 1) {
                    --col; tv = TAT(col, row); ++frag;
                }
            }
            --col; tv = TAT(col, row); ++frag;
        } else if ((tv & TV_MFH) && (tv & TV_HO)) {
            if (!(last & TV_H)) { record(sb, col, row, frag, last); last = TV_H; frag = 0; }
            --col; tv = TAT(col, row); ++frag;
        } else {
            break;  /* NONE, or a value the reference asserts on */
        }
    }
    record(sb, col, row, frag, last);
    if (head) { /* TraceHead_ (:538-545) */
        if (row != 0) record(sb, 0, 0, row, TV_V);
        if (col != 0) record(sb, 0, 0, col, TV_H);
    }
#undef TAT
}

/* ---------------------------------------------------------------------------------
 * Band validity (align/dp_algorithm_impl.h:193-234).
 * ------------------------------------------------------------------------------- */
static int band_valid(const orc_params *p, int m, int n, int fe)
{
    long lo = p->band_lower, up = p->band_upper;
    if (!p->band_on) return 1;
    if (up < -(long)n || lo > (long)m) return 0;
    if (up < 0 && !(fe & ORC_FREE_LEFT)) return 0;
    if (lo > 0 && !(fe & ORC_FREE_TOP)) return 0;
    if (up + n < m && !(fe & ORC_FREE_BOTTOM)) return 0;
    if (lo + n > m && !(fe & ORC_FREE_RIGHT)) return 0;
    return 1;
}

/* ---------------------------------------------------------------------------------
 * Banded DP (align/dp_algorithm_impl.h:586-967).  Cells are stored densely by (column, row);
 * the reference's band-indexed storage only changes addressing.  A "track" computes rows
 * [r0, r1] of one column like _computeTrack (:334-429): first cell, inner cells, last cell,
 * with the recursion direction and tracking flag of each cell taken from DPMetaColumn_
 * (align/dp_meta_info.h:178-370) for the column's type and location.
 * ------------------------------------------------------------------------------- */
enum { COL_INITIAL, COL_INNER, COL_FINAL };
enum { LOC_FULL, LOC_TOP, LOC_MIDDLE, LOC_BOTTOM };

typedef struct {
    const ctx_t *c;
    int fe, m, n;
    const uint8_t *h, *v;
    int *S, *E;          /* dense (m+1) x (n+1), column-major */
    uint8_t *T;
    best_t *b;
    caches_t k;          /* caches of the current track */
    int lastF;           /* cacheVert F after the last computed cell */
    int upper;
    int *Fslot;          /* F field of the band column's storage, one slot per diagonal */
    int nslots;
    int trk;             /* every cell tracked: local, or the AlignExtend_ profile */
    /* X-drop terminator of an AlignExtend_ DP (align_extend/dp_scout_xdrop.h:127-143): every
     * offer raises colmax; an offer of a column's last cell (and the reference's extra offers
     * made with IsLastRow) sets term when best - colmax >= xdrop and resets colmax otherwise. */
    int xd_on, xd, colmax, term;
} band_t;

#define BAT(bt, arr, col, row) (bt)->arr[(size_t)(col) * (size_t)((bt)->n + 1) + (size_t)(row)]

static int first_dir(const band_t *bt, int type, int loc)
{
    if (type == COL_INITIAL) return DIR_ZERO;
    if (loc == LOC_FULL || loc == LOC_TOP) return (bt->fe & ORC_FREE_TOP) ? DIR_ZERO : DIR_HORIZONTAL;
    return DIR_UPPER;
}
static int inner_dir(const band_t *bt, int type)
{
    if (type == COL_INITIAL) return (bt->fe & ORC_FREE_LEFT) ? DIR_ZERO : DIR_VERTICAL;
    return DIR_ALL;
}
static int last_dir(const band_t *bt, int type, int loc)
{
    if (type == COL_INITIAL) return (bt->fe & ORC_FREE_LEFT) ? DIR_ZERO : DIR_VERTICAL;
    return (loc == LOC_TOP || loc == LOC_MIDDLE) ? DIR_LOWER : DIR_ALL;
}
/* Tracking flags of DPMetaColumn_ for first / inner / last cells (every cell for local and for
 * AlignExtend_, align_extend/align_extend_base.h:86-190). */
static int track_flag(const band_t *bt, int type, int loc, int which /* 0 first 1 inner 2 last */)
{
    if (bt->trk) return 1;
    int lastColFree = (type == COL_FINAL) && (bt->fe & ORC_FREE_RIGHT);
    if (which < 2) return lastColFree;
    if (loc == LOC_FULL || loc == LOC_BOTTOM) return (type == COL_FINAL) || (bt->fe & ORC_FREE_BOTTOM);
    return lastColFree;
}

/* One offer to the scout; last_row: the XDrop scout's IsLastRow (termination check). */
static void band_offer(band_t *bt, int s, int e, int f, int col, int row, int last_row)
{
    scout(bt->b, s, e, f, col, row);
    if (!bt->xd_on) return;
    if (s > bt->colmax) bt->colmax = s;
    if (last_row) {
        if (bt->b->s - bt->colmax >= bt->xd) bt->term = 1;
        else bt->colmax = INT_MIN;
    }
}

static void band_cell_x(band_t *bt, int dir, int col, int row, int tracked, int last_row);
static void band_cell(band_t *bt, int dir, int col, int row, int tracked)
{
    band_cell_x(bt, dir, col, row, tracked, 0);
}

static void band_cell_x(band_t *bt, int dir, int col, int row, int tracked, int last_row)
{
    int f;
    /* The horizontal neighbour (row, col-1): its S/E are read through the dense arrays. */
    int sh = col > 0 ? BAT(bt, S, col - 1, row) : bt->c->inf;
    int eh = col > 0 ? BAT(bt, E, col - 1, row) : bt->c->inf;
    int tv = compute_cell(bt->c, dir, &sh, &eh, &bt->k,
                          col > 0 ? bt->h[col - 1] : 0, row > 0 ? bt->v[row - 1] : 0, &f);
    if (dir == DIR_ZERO) {
        /* Zero leaves the cell's stored E as it was (never written: infinity). */
        eh = BAT(bt, E, col, row);
    }
    BAT(bt, S, col, row) = sh;
    BAT(bt, E, col, row) = eh;
    if (bt->T) BAT(bt, T, col, row) = (uint8_t)tv;
    bt->lastF = f;
    if (tracked) {
        /* _computeCell stores cacheVert's F into the tracked cell before scouting it
         * (align/dp_algorithm_impl.h:303-311). */
        int slot = bt->upper - col + row;
        if (slot >= 0 && slot < bt->nslots) bt->Fslot[slot] = f;
        band_offer(bt, sh, eh, f, col, row, last_row);
    }
}

/* One track: rows r0..r1 of column col (r1 > r0). */
static void band_track(band_t *bt, int col, int type, int loc, int r0, int r1)
{
    int i;
    bt->k.dS = bt->c->inf; bt->k.vS = bt->c->inf; bt->k.vF = bt->c->inf;
    /* _preInitCacheDiagonal: partial columns that start below row 0 read the diagonal
     * neighbour of their first cell (dp_matrix_navigator_score_matrix.h:358-392). */
    if (type != COL_INITIAL && (loc == LOC_MIDDLE || loc == LOC_BOTTOM) && r0 > 0 && col > 0)
        bt->k.dS = BAT(bt, S, col - 1, r0 - 1);
    band_cell(bt, first_dir(bt, type, loc), col, r0, track_flag(bt, type, loc, 0));
    for (i = r0 + 1; i < r1; ++i) band_cell(bt, inner_dir(bt, type), col, i, track_flag(bt, type, loc, 1));
    band_cell_x(bt, last_dir(bt, type, loc), col, r1, track_flag(bt, type, loc, 2), 1);
}

/* Re-offers the last computed cell to the scout (the reference's extra _scoutBestScore calls
 * at phase boundaries).  The scout copies the stored cell: its F is what the band column's
 * slot holds (written only by tracked cells of that diagonal), unless the call site refreshes
 * it from cacheVert first (set_f). */
static void band_retrack_x(band_t *bt, int col, int row, int set_f, int last_row)
{
    int slot = bt->upper - col + row;
    int inside = slot >= 0 && slot < bt->nslots;
    if (set_f && inside) bt->Fslot[slot] = bt->lastF;
    band_offer(bt, BAT(bt, S, col, row), BAT(bt, E, col, row), inside ? bt->Fslot[slot] : bt->c->inf, col, row,
               last_row);
}
#define band_retrack_f(bt, col, row, set_f) band_retrack_x((bt), (col), (row), (set_f), 1)
#define band_retrack(bt, col, row) band_retrack_x((bt), (col), (row), 0, 1)
#define band_retrack_nocheck(bt, col, row) band_retrack_x((bt), (col), (row), 0, 0)

static void dp_banded_impl(const ctx_t *c, int fe, const uint8_t *h, int m, const uint8_t *v, int n,
                           int lower, int upper, int *S, int *E, uint8_t *T, best_t *b, int *Fslot,
                           int xdrop_on, int xdrop)
{
    band_t bt;
    int hb, hTop, hMid, hBot, hIt, vb, ve, tmp;
    bt.c = c; bt.fe = fe; bt.m = m; bt.n = n; bt.h = h; bt.v = v; bt.S = S; bt.E = E; bt.T = T; bt.b = b;
    bt.lastF = c->inf;
    bt.upper = upper;
    bt.Fslot = Fslot;
    bt.nslots = upper - lower + 1;
    bt.trk = c->local || c->extend;
    bt.xd_on = xdrop_on;
    bt.xd = xdrop;
    bt.colmax = INT_MIN;
    bt.term = 0;
    {
        size_t cells = (size_t)(m + 1) * (size_t)(n + 1), q;
        for (q = 0; q < cells; ++q) { S[q] = c->inf; E[q] = c->inf; }
    }
#define MIN(a, b) ((a) < (b) ? (a) : (b))
#define MAX(a, b) ((a) > (b) ? (a) : (b))
    if (upper == lower) {
        /* Band of one diagonal: _computeHammingDistance (:970-1110). */
        int ih = MAX(0, MIN(m - 1, upper)), ihEnd = MIN(m - 1, upper + n);
        int iv = MAX(0, MIN(n - 1, -lower)), ivEnd = MIN(n - 1, lower + m);
        int col = ih + (upper >= 0 ? 0 : 0), row;
        int tr;
        /* The first cell of the diagonal gets direction Zero. */
        col = upper >= 0 ? MIN(m, upper) : 0;
        row = upper >= 0 ? 0 : MIN(n, -upper);
        bt.k.dS = c->inf; bt.k.vS = c->inf; bt.k.vF = c->inf;
        band_cell(&bt, DIR_ZERO, col, row, 0);
        /* _computeHammingDistance offers cells with no IsLastRow: no X-drop check here. */
        if (upper < 0) {
            if (upper == -n) { if (bt.trk || (fe & ORC_FREE_BOTTOM)) band_retrack_nocheck(&bt, col, row); return; }
            if (bt.trk) band_retrack_nocheck(&bt, col, row);
        } else if (lower > 0) {
            if (lower == m) { if (bt.trk || (fe & ORC_FREE_RIGHT)) band_retrack_nocheck(&bt, col, row); return; }
            if (bt.trk) band_retrack_nocheck(&bt, col, row);
        } else {
            if (bt.trk) band_retrack_nocheck(&bt, col, row);
        }
        tr = bt.trk;
        while (ih != ihEnd && iv != ivEnd) {
            int prev = BAT(&bt, S, col, row);
            ++col; ++row;
            {
                int s = wr(c, (long)prev + sub_score(c, h[ih], v[iv]));
                int t = TV_DIAG;
                if (c->local) { if (s <= 0) { s = 0; t = TV_NONE; } }
                BAT(&bt, S, col, row) = s;
                if (T) BAT(&bt, T, col, row) = (uint8_t)t;
            }
            if (tr) band_offer(&bt, BAT(&bt, S, col, row), c->inf, c->inf, col, row, 0);
            ++ih; ++iv;
        }
        /* The reference computes one more diagonal cell here.  When the diagonal leaves the
         * matrix through its bottom row with m < -2 * lower, its end iterators let that cell
         * read past the end of V (undefined behaviour); the restatement stops at the matrix edge
         * instead, so parity excludes that case. */
        if (ih > m - 1 || iv > n - 1 || col + 1 > m || row + 1 > n) return;
        {
            int prev = BAT(&bt, S, col, row);
            int s, t = TV_DIAG;
            ++col; ++row;
            s = wr(c, (long)prev + sub_score(c, h[ih], v[iv]));
            if (c->local) { if (s <= 0) { s = 0; t = TV_NONE; } }
            BAT(&bt, S, col, row) = s;
            if (T) BAT(&bt, T, col, row) = (uint8_t)t;
            if (ih == ihEnd) {
                if (iv == ivEnd) band_offer(&bt, s, c->inf, c->inf, col, row, 0);   /* final column, last cell: always */
                if (bt.trk || (fe & ORC_FREE_BOTTOM)) band_offer(&bt, s, c->inf, c->inf, col, row, 0);
            } else {
                if (bt.trk || (fe & ORC_FREE_RIGHT)) band_offer(&bt, s, c->inf, c->inf, col, row, 0);
            }
        }
        return;
    }

    /* Positions of seqVBegin / seqVEnd and of the H iterators (0-based character positions). */
    vb = -MIN(0, 1 + upper);
    ve = -MIN(0, MAX(-n, lower));
    hb = MAX(0, MIN(m - 1, lower));
    hTop = MIN(m - 1, MAX(0, upper));
    hMid = MIN(m - 1, MAX(0, n + lower));
    if (upper > n + lower) { tmp = hTop; hTop = hMid; hMid = tmp; }
    hBot = MAX(0, MIN(m, upper + n) - 1);

    /* Bands that start in the last column or end in the first one: the reference computes a
     * single cell (direction Zero) and stops, even when the band holds a second cell.  Its
     * traceback does not terminate on these shapes, so they take part in score parity only;
     * the cell is placed at the band's first cell. */
    if (hb == m - 1) {
        int col = MAX(0, MIN(m, lower));
        bt.k.dS = c->inf; bt.k.vS = c->inf; bt.k.vF = c->inf;
        band_cell(&bt, DIR_ZERO, col, 0, bt.trk);
        if (bt.trk || (fe & ORC_FREE_RIGHT)) band_retrack_nocheck(&bt, col, 0);   /* (True, False) */
        return;
    }
    if (hBot == 0) {
        int row = MIN(n, -upper);
        bt.k.dS = c->inf; bt.k.vS = c->inf; bt.k.vF = c->inf;
        band_cell(&bt, DIR_ZERO, 0, row, bt.trk);
        if (bt.trk || (fe & ORC_FREE_BOTTOM)) band_retrack(&bt, 0, row);
        return;
    }

    if (upper < 0) {
        ++vb;
        band_track(&bt, 0, COL_INITIAL, lower > -n ? LOC_MIDDLE : LOC_BOTTOM, vb, ve);
    } else if (lower >= 0) {
        bt.k.dS = c->inf; bt.k.vS = c->inf; bt.k.vF = c->inf;
        band_cell(&bt, DIR_ZERO, hb, 0, bt.trk);
        if (bt.trk) band_retrack_nocheck(&bt, hb, 0);
    } else {
        band_track(&bt, 0, COL_INITIAL, lower <= -n ? LOC_FULL : LOC_TOP, vb, ve);
    }
    /* _computeAlignmentHelperCheckTerminate after the initial column and after each column of
     * the three band phases (align/dp_algorithm_impl.h:746-836). */
    if (bt.term) return;

    hIt = hb;
    for (; hIt != hTop; ++hIt) {
        ++ve;
        band_track(&bt, hIt + 1, COL_INNER, LOC_TOP, vb, ve);
        if (bt.term) return;
    }
    if (upper > n + lower) {
        if (bt.trk || (fe & ORC_FREE_BOTTOM)) band_retrack(&bt, hIt, ve);
        for (; hIt != hMid; ++hIt) {
            band_track(&bt, hIt + 1, COL_INNER, LOC_FULL, vb, ve);
            if (bt.term) return;
        }
    } else {
        for (; hIt != hMid; ++hIt) {
            ++vb; ++ve;
            band_track(&bt, hIt + 1, COL_INNER, LOC_MIDDLE, vb, ve);
            if (bt.term) return;
        }
        if ((bt.trk || (fe & ORC_FREE_BOTTOM)) && lower + n < m) band_retrack(&bt, hIt, ve);
    }
    for (; hIt != hBot; ++hIt) {
        ++vb;
        band_track(&bt, hIt + 1, COL_INNER, LOC_BOTTOM, vb, ve);
        if (bt.term) return;
    }

    /* Last band column. */
    if (hIt < m - 1) {
        /* The band ends before the final column: one cell (first cell of a bottom column). */
        bt.k.dS = BAT(&bt, S, hIt, vb); bt.k.vS = c->inf; bt.k.vF = c->inf;
        band_cell(&bt, DIR_UPPER, hIt + 1, vb + 1, bt.trk);
        if (bt.trk || (fe & ORC_FREE_BOTTOM)) band_retrack_f(&bt, hIt + 1, vb + 1, 1);
    } else if (hIt == m - 1) {
        if (upper == m - n) {
            bt.k.dS = BAT(&bt, S, hIt, vb); bt.k.vS = c->inf; bt.k.vF = c->inf;
            band_cell(&bt, DIR_UPPER, m, vb + 1, bt.trk || (fe & ORC_FREE_RIGHT));
            band_retrack_f(&bt, m, vb + 1, 1);
        } else if (upper >= m) {
            if (lower + n > m) {
                ++ve;
                band_track(&bt, m, COL_FINAL, LOC_TOP, vb, ve);
            } else if (lower + n + 1 > m) {
                ++ve;
                band_track(&bt, m, COL_FINAL, LOC_TOP, vb, ve);
                band_retrack_f(&bt, m, ve, 1);
            } else {
                band_track(&bt, m, COL_FINAL, LOC_FULL, vb, ve);
            }
        } else {
            ++vb;
            if (lower + n <= m) {
                if (lower + n == m) {
                    ++ve;
                    band_track(&bt, m, COL_FINAL, LOC_MIDDLE, vb, ve);
                    band_retrack_f(&bt, m, ve, 1);
                } else {
                    band_track(&bt, m, COL_FINAL, LOC_BOTTOM, vb, ve);
                }
            } else {
                ++ve;
                band_track(&bt, m, COL_FINAL, LOC_MIDDLE, vb, ve);
            }
        }
    }
#undef MIN
#undef MAX
}

static void dp_banded(const ctx_t *c, int fe, const uint8_t *h, int m, const uint8_t *v, int n,
                      int lower, int upper, int *S, int *E, uint8_t *T, best_t *b, int xdrop_on, int xdrop)
{
    int slots = upper - lower + 1, q;
    int *Fslot = (int *)malloc(sizeof(int) * (size_t)(slots > 0 ? slots : 1));
    for (q = 0; q < slots; ++q) Fslot[q] = c->inf;
    dp_banded_impl(c, fe, h, m, v, n, lower, upper, S, E, T, b, Fslot, xdrop_on, xdrop);
    free(Fslot);
}

/* ---------------------------------------------------------------------------------
 * Unbanded DP (align/dp_algorithm_impl.h:483-579 with dp_meta_info.h:178-221).
 * ------------------------------------------------------------------------------- */
/* xdrop_on (ORC_EXTEND): the X-drop terminator of align_extend/dp_scout_xdrop.h:127-143 sets its
 * flag at the last cell of a column when best - columnMax >= xdrop (columnMax: the column's
 * maximum S; it is reset only when the flag is not set), and the column loop of
 * _computeAlignmentImpl (align/dp_algorithm_impl.h:535-557) tests the flag after each inner
 * column 1..m-1 only: a flag set in column 0 stops the DP after column 1, and the last column
 * is computed whenever the loop runs out. */
static void dp_unbanded(const ctx_t *c, int fe, const uint8_t *h, int m, const uint8_t *v, int n,
                        int *colS, int *colE, uint8_t *T, best_t *b, int xdrop_on, int xdrop)
{
    int i, j;
    int terminated = 0, colmax = INT_MIN;
    for (i = 0; i <= n; ++i) { colS[i] = c->inf; colE[i] = c->dynamic ? 0 : c->inf; }
    for (j = 0; j <= m; ++j) {
        caches_t k;
        int finalCol = (j == m);
        k.dS = c->inf; k.vS = c->inf; k.vF = c->dynamic ? 0 : c->inf;
        for (i = 0; i <= n; ++i) {
            int dir, tv, f;
            int tracked;
            if (i == 0)
                dir = (j == 0 || (fe & ORC_FREE_TOP)) ? DIR_ZERO : DIR_HORIZONTAL;
            else if (j == 0)
                dir = (fe & ORC_FREE_LEFT) ? DIR_ZERO : DIR_VERTICAL;
            else
                dir = DIR_ALL;
            tv = compute_cell(c, dir, &colS[i], &colE[i], &k,
                              j > 0 ? h[j - 1] : 0, i > 0 ? v[i - 1] : 0, &f);
            if (T) T[(size_t)j * (size_t)(n + 1) + (size_t)i] = (uint8_t)tv;
            if (c->local || c->extend)
                tracked = 1;
            else if (i < n)
                tracked = finalCol && (fe & ORC_FREE_RIGHT);
            else
                tracked = finalCol || (fe & ORC_FREE_BOTTOM);
            if (tracked) scout(b, colS[i], colE[i], f, j, i);
            if (xdrop_on && colS[i] > colmax) colmax = colS[i];
        }
        if (xdrop_on) {
            if (b->s - colmax >= xdrop) terminated = 1;
            else colmax = INT_MIN;
            if (terminated && j >= 1 && j < m) break;
        }
    }
}

/* 4-bit trace code (see seqan_oracle.h).  _doTraceback (align/dp_traceback_impl.h:376-450) reads
 * DIAGONAL, MAX_FROM_V with VERTICAL / VERTICAL_OPEN and MAX_FROM_H with HORIZONTAL /
 * HORIZONTAL_OPEN, and its gap walks continue while !(open) || (extend) (:242-255, :320-332);
 * SingleTrace sets exactly one bit of each open/extend pair in inner cells (dp_formula.h:179-181). */
uint8_t orc_trace4_encode(uint8_t tv)
{
    int src = (tv & TV_DIAG) ? 1 : (tv & TV_MFV) ? 2 : (tv & TV_MFH) ? 3 : 0;
    int eo = (tv & TV_HO) && !(tv & TV_H);
    int fo = (tv & TV_VO) && !(tv & TV_V);
    return (uint8_t)(src | (eo << 2) | (fo << 3));
}

uint8_t orc_trace4_decode(uint8_t code, int32_t affine)
{
    static const uint8_t src_bits[4] = {TV_NONE, TV_DIAG, TV_MFV, TV_MFH};
    int src = code & 3;
    if (src == 0) return TV_NONE;
    if (!affine) return (uint8_t)(src == 1 ? TV_DIAG : src == 2 ? (TV_V | TV_MFV) : (TV_H | TV_MFH));
    return (uint8_t)(src_bits[src] | ((code & 4) ? TV_HO : TV_H) | ((code & 8) ? TV_VO : TV_V));
}

static int align_pair_impl(const orc_params *p, int complete,
                           const uint8_t *h, int32_t m,
                           const uint8_t *v, int32_t n,
                           orc_result *out, orc_segment *segs, int32_t seg_cap)
{
    ctx_t c;
    int fe;
    int *colS, *colE;
    uint8_t *T = NULL;
    best_t b;

    memset(out, 0, sizeof(*out));
    c.bits16 = (p->score_bits == 16);
    c.inf = c.bits16 ? -16384 : -(1 << 30);
    c.local = (p->mode == ORC_LOCAL);
    c.extend = (p->mode == ORC_EXTEND);
    c.complete = complete;
    c.affine = (p->gap_model == ORC_AFFINE);
    c.dynamic = (p->gap_model == ORC_DYNAMIC);
    c.ext = p->gap_extend;
    c.open = p->gap_open;
    c.match = p->match;
    c.mismatch = p->mismatch;
    c.mat = p->matrix;
    c.asz = p->alphabet_size;
    /* AlignExtend_ has free last row and column (align_extend/align_extend_base.h:75-81): they
     * only decide band validity and the extra offers, since it tracks every cell anyway. */
    fe = c.local ? (ORC_FREE_TOP | ORC_FREE_LEFT | ORC_FREE_RIGHT | ORC_FREE_BOTTOM)
                 : (c.extend ? (ORC_FREE_RIGHT | ORC_FREE_BOTTOM) : p->free_ends);
    if (c.dynamic && (p->band_on || c.extend)) return -1;   /* DynamicGaps: unbanded global / local */

    if (m <= 0 || n <= 0 || !band_valid(p, m, n, fe)) {
        out->score = c.bits16 ? -32768 : INT_MIN;
        out->valid = 0;
        out->n_segments = 0;
        return 0;
    }
    out->valid = 1;
    colS = (int *)malloc(sizeof(int) * (size_t)(n + 1) * 2);
    colE = colS + (n + 1);
    if (p->traceback) T = (uint8_t *)calloc((size_t)(m + 1) * (size_t)(n + 1), 1);
    b.s = c.inf; b.e = c.inf; b.f = c.inf; b.col = 0; b.row = 0;

    if (p->band_on) {
        int *S = (int *)malloc(sizeof(int) * (size_t)(m + 1) * (size_t)(n + 1) * 2);
        if (!T) T = NULL;
        dp_banded(&c, fe, h, m, v, n, p->band_lower, p->band_upper, S, S + (size_t)(m + 1) * (size_t)(n + 1), T, &b,
                  c.extend && p->xdrop_on, p->xdrop);
        free(S);
    } else {
        dp_unbanded(&c, fe, h, m, v, n, colS, colE, T, &b, c.extend && p->xdrop_on, p->xdrop);
    }

    out->score = b.s;
    out->end_h = b.col;
    out->end_v = b.row;
    if (T) {
        segbuf_t sb;
        uint8_t *cell = &T[(size_t)b.col * (size_t)(n + 1) + (size_t)b.row];
        if (p->trace4) {
            size_t q, cells = (size_t)(m + 1) * (size_t)(n + 1);
            for (q = 0; q < cells; ++q) T[q] = orc_trace4_decode(orc_trace4_encode(T[q]), c.affine);
        }
        /* _correctTraceValue (align/dp_algorithm_impl.h:1188-1205) for affine cells; for DynamicGaps
         * cells the best cell's flags decide (:1235-1249; the scout keeps the flags in b.e). */
        if (c.complete) {
            /* CompleteTrace: _finishAlignment corrects no trace value (dp_algorithm_impl.h:1352). */
        } else if (c.affine) {
            if (b.f == b.s) { *cell &= (uint8_t)~TV_DIAG; *cell |= TV_MFV; }
            else if (b.e == b.s) { *cell &= (uint8_t)~TV_DIAG; *cell |= TV_MFH; }
        } else if (c.dynamic) {
            if (b.e & DYN_V) { *cell &= (uint8_t)~TV_DIAG; *cell |= TV_MFV; }
            else if (b.e & DYN_H) { *cell &= (uint8_t)~TV_DIAG; *cell |= TV_MFH; }
        }
        sb.segs = segs; sb.cap = segs ? seg_cap : 0; sb.n = 0; sb.overflow = 0;
        traceback(&c, T, n, m, b.col, b.row, &sb, !c.local && !c.extend, !c.local);
        out->n_segments = sb.overflow ? -1 : sb.n;
        if (sb.n > 0 && !sb.overflow) {
            out->begin_h = (int32_t)segs[sb.n - 1].h_begin;
            out->begin_v = (int32_t)segs[sb.n - 1].v_begin;
        } else {
            out->begin_h = 0;
            out->begin_v = 0;
        }
        free(T);
    }
    free(colS);
    return 0;
}

int orc_align_pair(const orc_params *p,
                   const uint8_t *h, int32_t m,
                   const uint8_t *v, int32_t n,
                   orc_result *out, orc_segment *segs, int32_t seg_cap)
{
    return align_pair_impl(p, 0, h, m, v, n, out, segs, seg_cap);
}

int orc_align_pair_complete(const orc_params *p,
                            const uint8_t *h, int32_t m,
                            const uint8_t *v, int32_t n,
                            orc_result *out, orc_segment *segs, int32_t seg_cap)
{
    return align_pair_impl(p, 1, h, m, v, n, out, segs, seg_cap);
}

int orc_align_batch(const orc_params *p, int64_t n_pairs,
                    const uint8_t *seq_h, const int64_t *off_h,
                    const uint8_t *seq_v, const int64_t *off_v,
                    orc_result *out, orc_segment *segs, const int64_t *seg_off,
                    int32_t threads)
{
    int64_t k;
    int rc = 0;
    int nt = threads > 0 ? threads : omp_get_max_threads();
#pragma omp parallel for schedule(dynamic, 16) reduction(| : rc) num_threads(nt)
    for (k = 0; k < n_pairs; ++k) {
        orc_segment *sp = NULL;
        int32_t cap = 0;
        if (p->traceback && segs && seg_off) {
            sp = segs + seg_off[k];
            cap = (int32_t)(seg_off[k + 1] - seg_off[k]);
        }
        rc |= orc_align_pair(p, seq_h + off_h[k], (int32_t)(off_h[k + 1] - off_h[k]),
                             seq_v + off_v[k], (int32_t)(off_v[k + 1] - off_v[k]),
                             &out[k], sp, cap);
    }
    return rc;
}

/* ===================================================================================== */
/* Seed extension                                                                        */
/* ===================================================================================== */

static int xs_score(const orc_xdrop_params *p, int a, int b)
{
    if (p->matrix) return p->matrix[a * p->alphabet_size + b];
    return a == b ? p->match : p->mismatch;
}

/* extendSeed [UnGappedXDrop] seeds/seeds_extension.h:283-360.  The left walk scores the pair
 * at (posH, posV) while it tests (posH - 1, posV - 1) for a match, as the reference does. */
/* extendSeed [MatchExtend] seeds/seeds_extension.h:181-218. */
static void xs_match(const orc_xdrop_params *p, orc_seed *s, const uint8_t *db, uint64_t m, const uint8_t *q,
                     uint64_t n)
{
    if (p->direction & ORC_EXTEND_LEFT) {
        uint64_t posH = (uint64_t)s->begin_h, posV = (uint64_t)s->begin_v;
        while (posH >= 1 && posV >= 1 && db[posH - 1] == q[posV - 1]) {
            --posH;
            --posV;
        }
        s->begin_h = (int64_t)posH;
        s->begin_v = (int64_t)posV;
    }
    if (p->direction & ORC_EXTEND_RIGHT) {
        uint64_t posH = (uint64_t)s->end_h, posV = (uint64_t)s->end_v;
        while (posH < m && posV < n && db[posH] == q[posV]) {
            ++posH;
            ++posV;
        }
        s->end_h = (int64_t)posH;
        s->end_v = (int64_t)posV;
    }
}

static void xs_ungapped(const orc_xdrop_params *p, orc_seed *s, const uint8_t *db, uint64_t m, const uint8_t *q,
                        uint64_t n)
{
    const int drop = -p->xdrop;
    if (p->direction & ORC_EXTEND_LEFT) {
        int tmp = 0;
        uint64_t posH = (uint64_t)s->begin_h, posV = (uint64_t)s->begin_v, mism = 0;
        while (posH >= 1 && posV >= 1 && tmp > drop) {
            tmp += xs_score(p, db[posH], q[posV]);
            if (db[posH - 1] == q[posV - 1]) {
                mism = 0;
                if (tmp > 0) tmp = 0;
            } else {
                mism += 1;
            }
            --posH;
            --posV;
        }
        s->begin_h = (int64_t)(posH + mism);
        s->begin_v = (int64_t)(posV + mism);
    }
    if (p->direction & ORC_EXTEND_RIGHT) {
        int tmp = 0;
        uint64_t posH = (uint64_t)s->end_h, posV = (uint64_t)s->end_v, mism = 0;
        while (posH < m && posV < n && tmp > drop) {
            tmp += xs_score(p, db[posH], q[posV]);
            if (db[posH] == q[posV]) {
                mism = 0;
                if (tmp > 0) tmp = 0;
            } else {
                mism += 1;
            }
            ++posH;
            ++posV;
        }
        s->end_h = (int64_t)(posH - mism);
        s->end_v = (int64_t)(posV - mism);
    }
}

/* _extendSeedGappedXDropOneDirection, seeds/seeds_extension.h:613-775, with _initAntiDiags
 * (:457-481), _initAntiDiag3 (:498-520), _calcExtendedLowerDiag/UpperDiag (:522-545) and
 * _updateExtendedSeed (:547-579).  qs/ds: the query (V) and database (H) segments; `left`
 * reads them backwards from their ends.  Index arithmetic in size_t, diagonals signed, scores
 * int, as in the reference. */
static int xs_gapped_one(const orc_xdrop_params *p, orc_seed *s, const uint8_t *qs, uint64_t qlen,
                         const uint8_t *ds, uint64_t dlen, int left)
{
    const uint64_t cols = qlen + 1, rows = dlen + 1;
    if (rows == 1 || cols == 1) return 0;
    const int len = 2 * (int)(cols > rows ? cols : rows);
    const int minErr = INT_MIN / len;
    const int gap = p->gap > minErr ? p->gap : minErr;
    const int undefined = INT_MIN - gap;
    const int xdrop = p->xdrop;
    /* Score<int, Simple>: the mismatch score is raised to minErr too (:603-609). */
    orc_xdrop_params sp = *p;
    if (!p->matrix && sp.mismatch < minErr) sp.mismatch = minErr;
    p = &sp;
    /* anti-diagonal buffers: at most cols + 1 entries each */
    int *buf = (int *)malloc(sizeof(int) * 3 * (size_t)(cols + 2));
    int *ad1 = buf, *ad2 = buf + (cols + 2), *ad3 = buf + 2 * (cols + 2);
    uint64_t len1 = 0, len2 = 1, len3 = 2;
    ad2[0] = 0;
    if (-gap > xdrop) {
        ad3[0] = undefined;
        ad3[1] = undefined;
    } else {
        ad3[0] = gap;
        ad3[1] = gap;
    }
    uint64_t minCol = 1, maxCol = 2;
    uint64_t off1 = 0, off2 = 0, off3 = 0;
    uint64_t antiDiagNo = 1;
    int best = 0;
    int64_t lowerDiag = 0, upperDiag = 0;
    while (minCol < maxCol) {
        ++antiDiagNo;
        int *t = ad1;
        ad1 = ad2;
        ad2 = ad3;
        ad3 = t;
        len1 = len2;
        len2 = len3;
        off1 = off2;
        off2 = off3;
        off3 = minCol - 1;
        /* _initAntiDiag3 */
        len3 = maxCol + 1 - off3;
        ad3[0] = undefined;
        ad3[maxCol - off3] = undefined;
        if ((int)antiDiagNo * gap > best - xdrop) {
            if (off3 == 0) ad3[0] = (int)(antiDiagNo * (uint64_t)(int64_t)gap);
            if (antiDiagNo - maxCol == 0) ad3[maxCol - off3] = (int)(antiDiagNo * (uint64_t)(int64_t)gap);
        }
        int antiDiagBest = (int)(antiDiagNo * (uint64_t)(int64_t)gap);
        for (uint64_t col = minCol; col < maxCol; ++col) {
            const uint64_t i3 = col - off3, i2 = col - off2, i1 = col - off1;
            uint64_t queryPos, dbPos;
            if (!left) {
                queryPos = col - 1;
                dbPos = antiDiagNo - col - 1;
            } else {
                queryPos = cols - 1 - col;
                dbPos = rows - 1 + col - antiDiagNo;
            }
            int tmp = (ad2[i2 - 1] > ad2[i2] ? ad2[i2 - 1] : ad2[i2]) + gap;
            const int d = ad1[i1 - 1] + xs_score(p, qs[queryPos], ds[dbPos]);
            tmp = tmp > d ? tmp : d;
            if (tmp < best - xdrop) {
                ad3[i3] = undefined;
            } else {
                ad3[i3] = tmp;
                if (tmp > antiDiagBest) antiDiagBest = tmp;
            }
        }
        if (antiDiagBest > best) best = antiDiagBest;
        while (minCol - off3 < len3 && ad3[minCol - off3] == undefined && minCol - off2 - 1 < len2 &&
               ad2[minCol - off2 - 1] == undefined)
            ++minCol;
        while (maxCol - off3 > 0 && ad3[maxCol - off3 - 1] == undefined && ad2[maxCol - off2 - 1] == undefined)
            --maxCol;
        ++maxCol;
        {
            const uint64_t minRow = antiDiagNo - minCol;
            if ((int64_t)minCol - (int64_t)minRow < lowerDiag) lowerDiag = (int64_t)minCol - (int64_t)minRow;
        }
        {
            const uint64_t mc = maxCol - 1;
            const uint64_t maxRow = antiDiagNo + 1 - mc;
            if ((int64_t)mc - 1 - (int64_t)maxRow > upperDiag) upperDiag = (int64_t)(mc - 1 - maxRow);
        }
        {
            const int a = (int)minCol, b = (int)antiDiagNo + 2 - (int)rows;
            minCol = (uint64_t)(a > b ? a : b);
        }
        if (maxCol > cols) maxCol = cols;
    }
    /* Position of the longest extension. */
    uint64_t lcol = len3 + off3 - 2;
    uint64_t lrow = antiDiagNo - lcol;
    int lscore = ad3[lcol - off3];
    if (lscore == undefined) {
        if (ad2[len2 - 2] != undefined) {
            lcol = len2 + off2 - 2;
            lrow = antiDiagNo - 1 - lcol;
            lscore = ad2[lcol - off2];
        } else if (len2 > 2 && ad2[len2 - 3] != undefined) {
            lcol = len2 + off2 - 3;
            lrow = antiDiagNo - 1 - lcol;
            lscore = ad2[lcol - off2];
        }
    }
    if (lscore == undefined) {
        for (uint64_t i = 0; i < len1; ++i) {
            if (ad1[i] > lscore) {
                lscore = ad1[i];
                lcol = i + off1;
                lrow = antiDiagNo - 2 - lcol;
            }
        }
    }
    free(buf);
    if (lscore != undefined) {
        if (left) {
            const int64_t beginDiag = s->begin_h - s->begin_v;
            if (s->lower_diag > beginDiag + lowerDiag) s->lower_diag = beginDiag + lowerDiag;
            if (s->upper_diag < beginDiag + upperDiag) s->upper_diag = beginDiag + upperDiag;
            s->begin_h = (int64_t)((uint64_t)s->begin_h - lrow);
            s->begin_v = (int64_t)((uint64_t)s->begin_v - lcol);
        } else {
            const int64_t endDiag = s->end_h - s->end_v;
            if (s->upper_diag < endDiag - lowerDiag) s->upper_diag = endDiag - lowerDiag;
            if (s->lower_diag > endDiag - upperDiag) s->lower_diag = endDiag - upperDiag;
            s->end_h = (int64_t)((uint64_t)s->end_h + lrow);
            s->end_v = (int64_t)((uint64_t)s->end_v + lcol);
        }
    }
    return lscore;
}

/* extendSeed [GappedXDrop] seeds/seeds_extension.h:780-835: left on the prefixes before the
 * seed, right on the suffixes after it. */
int orc_extend_seed(const orc_xdrop_params *p, orc_seed *seed, const uint8_t *db, int64_t m, const uint8_t *q,
                    int64_t n, int32_t *xscore)
{
    if (!p || !seed) return -1;
    if (xscore) xscore[0] = xscore[1] = 0;
    if (p->method == ORC_MATCH_EXTEND) {
        xs_match(p, seed, db, (uint64_t)m, q, (uint64_t)n);
        return 0;
    }
    if (p->method == ORC_XDROP_UNGAPPED) {
        xs_ungapped(p, seed, db, (uint64_t)m, q, (uint64_t)n);
        return 0;
    }
    if (p->direction & ORC_EXTEND_LEFT) {
        const int sc = xs_gapped_one(p, seed, q, (uint64_t)seed->begin_v, db, (uint64_t)seed->begin_h, 1);
        if (xscore) xscore[0] = sc;
    }
    if (p->direction & ORC_EXTEND_RIGHT) {
        const uint64_t eh = (uint64_t)seed->end_h, ev = (uint64_t)seed->end_v;
        const int sc = xs_gapped_one(p, seed, q + ev, (uint64_t)n - ev, db + eh, (uint64_t)m - eh, 0);
        if (xscore) xscore[1] = sc;
    }
    return 0;
}

int orc_extend_seeds(const orc_xdrop_params *p, int64_t n_h, const uint8_t *seq_h, const int64_t *off_h,
                     int64_t n_v, const uint8_t *seq_v, const int64_t *off_v, int64_t n_seeds,
                     const int32_t *seed_h, const int32_t *seed_v, orc_seed *seeds, int32_t *xscores,
                     int32_t threads)
{
    if (!p || n_seeds < 0 || (n_seeds > 0 && !seeds)) return -1;
    if (threads <= 0) threads = omp_get_max_threads();
#pragma omp parallel for schedule(dynamic, 64) num_threads(threads)
    for (int64_t i = 0; i < n_seeds; ++i) {
        const int64_t kh = seed_h ? seed_h[i] : i, kv = seed_v ? seed_v[i] : i;
        if (kh < 0 || kh >= n_h || kv < 0 || kv >= n_v) continue;
        orc_extend_seed(p, &seeds[i], seq_h + off_h[kh], off_h[kh + 1] - off_h[kh], seq_v + off_v[kv],
                        off_v[kv + 1] - off_v[kv], xscores ? xscores + 2 * i : NULL);
    }
    return 0;
}

/* ===================================================================================== */
/* SAM output                                                                            */
/* ===================================================================================== */

static int sam_num(char *p, int64_t v)
{
    char tmp[24];
    int n = 0, k = 0;
    uint64_t u = v < 0 ? (uint64_t)(-v) : (uint64_t)v;
    do { tmp[n++] = (char)('0' + u % 10); u /= 10; } while (u);
    if (v < 0) { if (p) p[k] = '-'; ++k; }
    while (n) { if (p) p[k] = tmp[n - 1]; ++k; --n; }
    return k;
}

/* appendTagsBamToSam (bam_io/bam_sam_conversion.h:250-360) on one record's BAM tag bytes: per tag
 * the two name characters, ':', the type ('c', 's', 'i', 'C', 'S', 'I' all written as 'i'), ':'
 * and the value -- Z and H strings up to their NUL, B arrays as the element type and ","-prefixed
 * values, numbers in decimal, A as the character; tags separated by tabs.  p == NULL only counts.
 * Float values (f, B:f) as the reference's appendNumber(float) prints them: snprintf "%g" of the
 * value (basic/basic_stream.h:1145-1155).  Returns -1 for bytes that are not well-formed tags. */
static int64_t tag_size(char t)
{
    switch (t) {
    case 'A': case 'c': case 'C': return 1;
    case 's': case 'S': return 2;
    case 'i': case 'I': case 'f': return 4;
    default: return 0;
    }
}

static int64_t tag_num(const char *q, char t)
{
    const unsigned char *u = (const unsigned char *)q;
    const uint32_t v = (uint32_t)u[0] | ((uint32_t)u[1] << 8) | ((uint32_t)u[2] << 16) | ((uint32_t)u[3] << 24);
    switch (t) {
    case 'c': return (int8_t)u[0];
    case 'C': return u[0];
    case 's': return (int16_t)(uint16_t)(u[0] | (u[1] << 8));
    case 'S': return (uint16_t)(u[0] | (u[1] << 8));
    case 'i': return (int32_t)v;
    default: return v;   /* 'I' */
    }
}

static int64_t tag_float(char *p, const char *q)
{
    const unsigned char *u = (const unsigned char *)q;
    const uint32_t v = (uint32_t)u[0] | ((uint32_t)u[1] << 8) | ((uint32_t)u[2] << 16) | ((uint32_t)u[3] << 24);
    float f;
    char buf[32];
    int n;
    memcpy(&f, &v, 4);
    n = snprintf(buf, sizeof(buf), "%g", (double)f);
    if (p) memcpy(p, buf, (size_t)n);
    return n;
}

static int64_t sam_tags(char *p, const char *t, int64_t len)
{
    int64_t w = 0, i = 0;
#define TPUT(c) do { if (p) p[w] = (c); ++w; } while (0)
    while (i < len) {
        char ty, lo;
        if (i + 3 > len) return -1;
        TPUT(t[i]);
        TPUT(t[i + 1]);
        TPUT(':');
        ty = t[i + 2];
        lo = (ty >= 'A' && ty <= 'Z') ? (char)(ty + 32) : ty;
        TPUT((lo == 'c' || lo == 's' || lo == 'i') ? 'i' : ty);
        TPUT(':');
        i += 3;
        if (ty == 'Z' || ty == 'H') {
            while (i < len && t[i] != 0) { TPUT(t[i]); ++i; }
            if (i >= len) return -1;
            ++i;
        } else if (ty == 'B') {
            char et;
            uint32_t cnt, e;
            int64_t sz;
            if (i + 5 > len) return -1;
            et = t[i];
            sz = tag_size(et);
            if (sz == 0 || et == 'A') return -1;
            TPUT(et);
            cnt = (uint32_t)tag_num(t + i + 1, 'I');
            i += 5;
            if ((int64_t)cnt * sz > len - i) return -1;
            for (e = 0; e < cnt; ++e) {
                TPUT(',');
                if (et == 'f') w += tag_float(p ? p + w : NULL, t + i);
                else w += sam_num(p ? p + w : NULL, tag_num(t + i, et));
                i += sz;
            }
        } else {
            const int64_t sz = tag_size(ty);
            if (sz == 0 || i + sz > len) return -1;
            if (ty == 'A') TPUT(t[i]);
            else if (ty == 'f') w += tag_float(p ? p + w : NULL, t + i);
            else w += sam_num(p ? p + w : NULL, tag_num(t + i, ty));
            i += sz;
        }
        if (i < len) TPUT('\t');
    }
#undef TPUT
    return w;
}

/* write(target, record, context, Sam()) of bam_io/write_sam.h:126-217; p == NULL only counts. */
static int64_t sam_line(char *p, int64_t k, const char *qname, const int64_t *qoff, const uint16_t *flag,
                        const int32_t *rid, const int32_t *pos, const uint8_t *mapq, const uint32_t *cigar,
                        const int64_t *coff, const int32_t *rnext, const int32_t *pnext, const int32_t *tlen,
                        const uint8_t *seq, const int64_t *soff, const char *letters, const char *qual,
                        const int64_t *quoff, const char *cnames, const int64_t *cnoff, const char *tags,
                        const int64_t *toff)
{
    int64_t w = 0, i;
#define PUT(c) do { if (p) p[w] = (c); ++w; } while (0)
#define NUM(v) do { w += sam_num(p ? p + w : NULL, (int64_t)(v)); } while (0)
    for (i = qoff[k]; i < qoff[k + 1]; ++i) PUT(qname[i]);
    PUT('\t');
    NUM(flag[k]);
    PUT('\t');
    if (rid[k] == -1) PUT('*');
    else for (i = cnoff[rid[k]]; i < cnoff[rid[k] + 1]; ++i) PUT(cnames[i]);
    PUT('\t');
    NUM((int64_t)pos[k] + 1);
    PUT('\t');
    NUM(mapq[k]);
    PUT('\t');
    if (coff[k] == coff[k + 1]) PUT('*');
    for (i = coff[k]; i < coff[k + 1]; ++i) { NUM(cigar[i] >> 4); PUT("MIDNSHP=X"[cigar[i] & 15u]); }
    PUT('\t');
    if (rnext[k] == -1) PUT('*');
    else if (rnext[k] == rid[k]) PUT('=');
    else for (i = cnoff[rnext[k]]; i < cnoff[rnext[k] + 1]; ++i) PUT(cnames[i]);
    PUT('\t');
    NUM((int64_t)pnext[k] + 1);
    PUT('\t');
    if (tlen[k] == 0) PUT('0');
    else NUM(tlen[k]);
    PUT('\t');
    if (soff[k] == soff[k + 1]) PUT('*');
    for (i = soff[k]; i < soff[k + 1]; ++i) PUT(letters[seq[i] & 31]);
    PUT('\t');
    if (!quoff || quoff[k] == quoff[k + 1]) PUT('*');
    else for (i = quoff[k]; i < quoff[k + 1]; ++i) PUT(qual[i]);
    if (toff && toff[k + 1] > toff[k]) {
        int64_t tl;
        PUT('\t');
        tl = sam_tags(p ? p + w : NULL, tags + toff[k], toff[k + 1] - toff[k]);
        if (tl < 0) return -1;
        w += tl;
    }
    PUT('\n');
#undef PUT
#undef NUM
    return w;
}

int64_t orc_write_sam(int64_t n, const char *qname, const int64_t *qoff, const uint16_t *flag, const int32_t *rid,
                      const int32_t *pos, const uint8_t *mapq, const uint32_t *cigar, const int64_t *coff,
                      const int32_t *rnext, const int32_t *pnext, const int32_t *tlen, const uint8_t *seq,
                      const int64_t *soff, const char *letters, const char *qual, const int64_t *quoff,
                      int64_t ncontigs, const char *cnames, const int64_t *cnoff, const char *tags,
                      const int64_t *toff, char *out, int64_t cap, int32_t threads)
{
    int64_t k, total;
    int64_t *off;
    int bad = 0;
    (void)ncontigs;
    if (n < 0) return -1;
    if (threads <= 0) threads = omp_get_max_threads();
    off = (int64_t *)malloc(sizeof(int64_t) * (size_t)(n + 1));
    off[0] = 0;
#pragma omp parallel for schedule(static) num_threads(threads)
    for (k = 0; k < n; ++k)
        off[k + 1] = sam_line(NULL, k, qname, qoff, flag, rid, pos, mapq, cigar, coff, rnext, pnext, tlen, seq,
                              soff, letters, qual, quoff, cnames, cnoff, tags, toff);
    for (k = 0; k < n; ++k) {
        if (off[k + 1] < 0) bad = 1;
        off[k + 1] += off[k];
    }
    if (bad) { free(off); return -1; }
    total = off[n];
    if (out && total <= cap) {
#pragma omp parallel for schedule(static) num_threads(threads)
        for (k = 0; k < n; ++k)
            sam_line(out + off[k], k, qname, qoff, flag, rid, pos, mapq, cigar, coff, rnext, pnext, tlen, seq, soff,
                     letters, qual, quoff, cnames, cnoff, tags, toff);
    }
    free(off);
    return total;
}


/* ---------------------------------------------------------------------------------------------
 * FASTA / FASTQ records: the loop `while (!atEnd(iter)) readRecord(id, seq, qual, iter, Fasta|Fastq)`
 * of seq_io/fasta_fastq.h, seq a String<Dna|Dna5|AminoAcid>, qual a CharString.
 *   Fasta (:265-283): skipUntil '>', skipOne, readLine(id), readUntil(seq, '>') ignoring
 *     IsWhitespace (' ', '\t', '\n', '\r') and asserting IsInAlphabet on the rest.
 *   Fastq (:354-392): skipUntil '@', skipOne, readLine(id), readUntil(seq, '+') as above,
 *     skipOne '+' (UnexpectedEnd at the end of the text), skipLine, then as many non-newline
 *     quality characters as the sequence has residues (fewer at the end of the text), skip
 *     whitespace; the next character must be '@', 0xFF or the end, else ParseError.
 * readLine (stream/tokenization.h:430-450) stops at '\r' or '\n' and consumes "\r\n", "\r" or "\n".
 * IsInAlphabet<T>(c) is convert<char>(T(c)) == toupper(c) (stream/tokenization.h:51-63). */

static int orc_residue_code(int32_t alphabet, unsigned char c)
{
    const unsigned char u = (c >= 'a' && c <= 'z') ? (unsigned char)(c - 32) : c;
    if (alphabet == 27) {
        static const char aa[] = "ABCDEFGHIJKLMNOPQRSTUVWYZX*";
        for (int k = 0; k < 27; ++k)
            if (aa[k] == (char)u) return k;
        return -1;
    }
    switch (u) {
    case 'A': return 0;
    case 'C': return 1;
    case 'G': return 2;
    case 'T': return 3;
    case 'N': return alphabet == 5 ? 4 : -1;
    default: return -1;
    }
}

static int orc_is_nl(unsigned char c) { return c == '\n' || c == '\r'; }
static int orc_is_ws(unsigned char c) { return c == ' ' || c == '\t' || c == '\n' || c == '\r'; }

int32_t orc_read_records(int32_t format, int32_t alphabet, const char *text_, int64_t n, int64_t rec_cap,
                         int64_t *id_begin, int64_t *id_end, int64_t *seq_off, int64_t *qual_end,
                         int64_t res_cap, uint8_t *codes, char *quals, int64_t *num, int64_t *residues,
                         int64_t *err_off)
{
    const unsigned char *t = (const unsigned char *)text_;
    const unsigned char start = format == 1 ? '@' : '>';
    int16_t table[256];   /* the conversion as a table, as TranslateTableCharToDna5_ and the like */
    for (int c = 0; c < 256; ++c) table[c] = (int16_t)orc_residue_code(alphabet, (unsigned char)c);
    int64_t p = 0, rec = 0, res = 0;
    int status = 0;
    *err_off = -1;
    while (p < n) {
        while (p < n && t[p] != start) ++p;                     /* skipUntil */
        if (p >= n) { *err_off = n; status = -2; break; }       /* skipOne at the end */
        ++p;
        const int64_t ib = p;                                   /* readLine(id) */
        while (p < n && !orc_is_nl(t[p])) ++p;
        const int64_t ie = p;
        if (p < n && t[p] == '\r') ++p;
        if (p < n && t[p] == '\n') ++p;
        const int64_t sb = res;
        const unsigned char stop = format == 1 ? '+' : '>';
        for (; p < n && t[p] != stop; ++p) {                    /* readUntil(seq, stop) */
            if (orc_is_ws(t[p])) continue;
            const int code = table[t[p]];
            if (code < 0) { *err_off = p; status = -1; break; }
            if (res < res_cap) codes[res] = (uint8_t)code;
            ++res;
        }
        if (status) break;
        int64_t qe = sb;                                        /* FASTA: no qualities */
        if (format == 1) {
            if (p >= n) { *err_off = n; status = -2; break; }   /* skipOne('+') */
            ++p;
            while (p < n && !orc_is_nl(t[p])) ++p;              /* skipLine */
            if (p < n && t[p] == '\r') ++p;
            if (p < n && t[p] == '\n') ++p;
            int64_t need = res - sb;
            qe = sb;
            for (; p < n && need > 0; ++p) {                    /* counted qualities */
                if (orc_is_nl(t[p])) continue;
                if (qe < res_cap && quals) quals[qe] = (char)t[p];
                ++qe;
                --need;
            }
            while (p < n && orc_is_ws(t[p])) ++p;
            if (p < n && t[p] != '@' && t[p] != 0xFF) { *err_off = p; status = -1; break; }
        }
        if (rec < rec_cap) {
            id_begin[rec] = ib;
            id_end[rec] = ie;
            seq_off[rec] = sb;
            if (qual_end) qual_end[rec] = qe;
        }
        ++rec;
    }
    *num = rec;
    *residues = res;
    if (status) return status;
    if (rec + 1 > rec_cap || res > res_cap) return -3;
    seq_off[rec] = res;
    return 0;
}

/* ---------------------------------------------------------------------------------------------
 * BAM records: write(target, record, context, Bam()) for a BamAlignmentRecord without tags
 * (bam_io/write_bam.h:100-271): block_size, the 32-byte core (rID, beginPos, l_qname | mapQ << 8 |
 * bin << 16, n_cigar | flag << 16, l_qseq, rNextId, pNext, tLen), the name and a NUL, the CIGAR
 * words, the sequence as Iupac codes two per byte (high nibble first), the qualities minus '!'
 * (0xFF for the ones missing), all little-endian.  bin = reg2bin(beginPos, beginPos + max(1, l)) in
 * uint32 arithmetic, l the CIGAR's length in the reference (every operation but S, H and I:
 * bam_io/cigar.h:601-612), kept to its 16-bit field. */

static uint8_t orc_iupac(unsigned char c)
{
    static const char iu[] = "=ACMGRSVTWYHKDBN";
    const unsigned char u = (c >= 'a' && c <= 'z') ? (unsigned char)(c - 32) : c;
    if (u == 'U') return 0;
    for (int k = 0; k < 16; ++k)
        if (iu[k] == (char)u) return (uint8_t)k;
    return 15;
}

static uint32_t orc_reg2bin(uint32_t beg, uint32_t end)
{
    --end;
    if (beg >> 14 == end >> 14) return 4681 + (beg >> 14);
    if (beg >> 17 == end >> 17) return 585 + (beg >> 17);
    if (beg >> 20 == end >> 20) return 73 + (beg >> 20);
    if (beg >> 23 == end >> 23) return 9 + (beg >> 23);
    if (beg >> 26 == end >> 26) return 1 + (beg >> 26);
    return 0;
}

static void orc_put32(char *p, uint32_t v)
{
    p[0] = (char)(v & 0xff);
    p[1] = (char)((v >> 8) & 0xff);
    p[2] = (char)((v >> 16) & 0xff);
    p[3] = (char)(v >> 24);
}

int64_t orc_write_bam(int64_t n, const char *qname, const int64_t *qoff, const uint16_t *flag, const int32_t *rid,
                      const int32_t *pos, const uint8_t *mapq, const uint32_t *cigar, const int64_t *coff,
                      const int32_t *rnext, const int32_t *pnext, const int32_t *tlen, const uint8_t *seq,
                      const int64_t *soff, const char *letters, const char *qual, const int64_t *quoff,
                      const char *tags, const int64_t *toff, char *out, int64_t cap, int32_t threads)
{
    int64_t k, total;
    int64_t *off;
    uint8_t iu[32];
    if (n < 0) return -1;
    if (threads <= 0) threads = omp_get_max_threads();
    for (k = 0; k < 32; ++k) iu[k] = orc_iupac((unsigned char)letters[k]);
    off = (int64_t *)malloc(sizeof(int64_t) * (size_t)(n + 1));
    off[0] = 0;
    for (k = 0; k < n; ++k) {
        const int64_t lq = qoff[k + 1] - qoff[k], nc = coff[k + 1] - coff[k], ls = soff[k + 1] - soff[k];
        const int64_t lt = toff ? toff[k + 1] - toff[k] : 0;
        off[k + 1] = off[k] + 4 + 32 + lq + 1 + 4 * nc + (ls + 1) / 2 + ls + lt;
    }
    total = off[n];
    if (out && total <= cap) {
#pragma omp parallel for num_threads(threads) schedule(static)
        for (k = 0; k < n; ++k) {
            char *p = out + off[k];
            const int64_t lq = qoff[k + 1] - qoff[k], nc = coff[k + 1] - coff[k], ls = soff[k + 1] - soff[k];
            const int64_t lqual = quoff ? quoff[k + 1] - quoff[k] : 0;
            const int64_t lt = toff ? toff[k + 1] - toff[k] : 0;
            uint32_t l = 0, bin;
            int64_t i;
            for (i = coff[k]; i < coff[k + 1]; ++i) {
                const uint32_t op = cigar[i] & 15u;
                if (op != 1 && op != 4 && op != 5) l += cigar[i] >> 4;
            }
            bin = orc_reg2bin((uint32_t)pos[k], (uint32_t)pos[k] + (l > 1 ? l : 1u)) & 0xffffu;
            orc_put32(p, (uint32_t)(32 + ((lq + 1) & 0xff) + 4 * (nc & 0xffff) + (ls + 1) / 2 + ls + lt));
            orc_put32(p + 4, (uint32_t)rid[k]);
            orc_put32(p + 8, (uint32_t)pos[k]);
            orc_put32(p + 12, (uint32_t)((lq + 1) & 0xff) | ((uint32_t)mapq[k] << 8) | (bin << 16));
            orc_put32(p + 16, (uint32_t)(nc & 0xffff) | ((uint32_t)flag[k] << 16));
            orc_put32(p + 20, (uint32_t)ls);
            orc_put32(p + 24, (uint32_t)rnext[k]);
            orc_put32(p + 28, (uint32_t)pnext[k]);
            orc_put32(p + 32, (uint32_t)tlen[k]);
            p += 36;
            memcpy(p, qname + qoff[k], (size_t)lq);
            p += lq;
            *p++ = 0;
            for (i = coff[k]; i < coff[k + 1]; ++i, p += 4) orc_put32(p, cigar[i]);
            for (i = 0; i + 1 < ls; i += 2)
                *p++ = (char)((iu[seq[soff[k] + i] & 31] << 4) | iu[seq[soff[k] + i + 1] & 31]);
            if (ls & 1) *p++ = (char)(iu[seq[soff[k] + ls - 1] & 31] << 4);
            for (i = 0; i < ls; ++i) *p++ = i < lqual ? (char)(qual[quoff[k] + i] - '!') : (char)0xff;
            if (lt) memcpy(p, tags + toff[k], (size_t)lt);   /* the tags as they are (write_bam.h:202-203) */
        }
    }
    free(off);
    return total;
}

/* ===================================================================================== */
/* Waterman-Eggert suboptimal local alignments                                            */
/* ===================================================================================== */

/* The reference's binary heap (misc/priority_type_heap.h) of (score, matrix position) entries,
 * ordered by score only (ScoreAndID::operator<, align/local_alignment_waterman_eggert_impl.h:
 * 62-100): the maximum on top; ties fall where push / pop / adjustTop put them. */
typedef struct { int32_t value; int64_t id; } we_entry;
typedef struct { we_entry *a; int64_t n, cap; } we_heap;

static void we_reserve(we_heap *hp, int64_t need)
{
    if (need <= hp->cap) return;
    hp->cap = need > 2 * hp->cap ? need : 2 * hp->cap;
    hp->a = (we_entry *)realloc(hp->a, sizeof(we_entry) * (size_t)hp->cap);
}

static void we_push(we_heap *hp, we_entry e)   /* push + _adjustHeapTowardRoot */
{
    int64_t h;
    we_reserve(hp, hp->n + 1);
    h = hp->n++;
    while (h > 0) {
        const int64_t i = (h - 1) / 2;
        if (hp->a[i].value < e.value) { hp->a[h] = hp->a[i]; h = i; }
        else break;
    }
    hp->a[h] = e;
}

static void we_toward_leaves(we_heap *hp, we_entry e, int64_t h, int64_t i)   /* _adjustHeapTowardLeaves */
{
    const int64_t n = hp->n;
    while (i < n) {
        if (e.value < hp->a[i].value) {
            if (hp->a[i - 1].value < hp->a[i].value) { hp->a[h] = hp->a[i]; h = i; }
            else { hp->a[h] = hp->a[i - 1]; h = i - 1; }
        } else if (e.value < hp->a[i - 1].value) {
            hp->a[h] = hp->a[i - 1]; h = i - 1;
        } else {
            break;
        }
        i = 2 * (h + 1);
    }
    if (i == n && e.value < hp->a[i - 1].value) { hp->a[h] = hp->a[i - 1]; h = i - 1; }
    hp->a[h] = e;
}

static void we_pop(we_heap *hp)
{
    const we_entry e = hp->a[hp->n - 1];
    hp->n -= 1;
    if (hp->n > 0) we_toward_leaves(hp, e, 0, 2);
}

typedef struct {
    const orc_we_params *p;
    const uint8_t *h, *v;
    int32_t m, n;
    int64_t W;            /* row stride of the matrix: m + 1 (dimension 0 is H) */
    int32_t *M;           /* (m + 1) x (n + 1) scores, position x + y * W */
    uint8_t *F;           /* forbidden cells */
    we_heap pq;
    int64_t best_end;     /* bestEndPos */
    int64_t best_begin;   /* bestBeginPos (where the last trace stopped) */
    /* the last alignment: per trace step, the H / V source index or -1 (a gap) */
    int32_t *stepH, *stepV;
    int64_t T;            /* trace steps */
    int64_t bH, bV;       /* first step of each row's clipped region */
    int32_t x0, y0;       /* the trace's start cell: step t of the H row is view position x0 + t */
    int32_t endH, endV;   /* clipped end source positions */
} we_t;

static int we_score(const we_t *w, int a, int b)
{
    if (w->p->matrix) return w->p->matrix[a * w->p->alphabet_size + b];
    return a == b ? w->p->match : w->p->mismatch;
}

/* _smithWatermanGetMatrix (:112-175): the matrix from the sequence ends, every cell of value
 * >= cutoff pushed. */
static int32_t we_matrix(we_t *w)
{
    const int32_t gap = w->p->gap, cutoff = w->p->cutoff;
    int32_t x, y;
    for (x = 0; x <= w->m; ++x) w->M[x + (int64_t)w->n * w->W] = 0;
    for (y = w->n - 1; y >= 0; --y) {
        const int cy = w->v[y];
        int32_t hh = 0, vv = 0;
        w->M[w->m + (int64_t)y * w->W] = vv;
        for (x = w->m - 1; x >= 0; --x) {
            const int64_t f1 = x + (int64_t)y * w->W, f2 = f1 + w->W;
            const int32_t cs = we_score(w, w->h[x], cy);
            if (w->h[x] == cy) {
                vv = hh + cs;
                hh = w->M[f2];
            } else {
                const int32_t s1 = hh + cs;
                int32_t s2;
                hh = w->M[f2];
                s2 = gap + (hh > vv ? hh : vv);
                vv = s1 > s2 ? s1 : s2;
                if (vv < 0) vv = 0;
            }
            w->M[f1] = vv;
            if (vv >= cutoff) { we_entry e; e.value = vv; e.id = f1; we_push(&w->pq, e); }
        }
    }
    if (w->pq.n > 0) {
        w->best_end = w->pq.a[0].id;
        return w->M[w->best_end];
    }
    return 0;
}

/* _smithWatermanTrace (:300-371): forward from src while the cell is non-zero and both sequences
 * have residues left; a gap is inserted in the row that does not advance.  Records the steps and
 * each row's clipped region (begin = the view position of its first residue, end = the view
 * position after the last step). */
static int64_t we_trace(we_t *w, int64_t src)
{
    const int32_t gap = w->p->gap;
    int32_t i0 = (int32_t)(src % w->W), i1 = (int32_t)(src / w->W);
    int64_t t = 0;
    w->x0 = i0;
    w->y0 = i1;
    while (w->M[src] != 0 && i0 != w->m && i1 != w->n) {
        const int forb = w->F[src];
        int gv, gh;
        if (w->h[i0] == w->v[i1] && !forb) {
            gv = gh = 1;
        } else {
            const int32_t vr = w->M[src + 1] + gap;
            const int32_t d = forb ? 0 : w->M[src + 1 + w->W] + we_score(w, w->h[i0], w->v[i1]);
            const int32_t hd = w->M[src + w->W] + gap;
            gv = (vr >= hd) | (d >= hd);
            gh = (hd > vr) | (d >= vr);
        }
        w->stepH[t] = gv ? i0 : -1;
        w->stepV[t] = gh ? i1 : -1;
        if (gv) { ++i0; src += 1; }
        if (gh) { ++i1; src += w->W; }
        ++t;
    }
    w->T = t;
    w->bH = 0;
    while (w->bH < t && w->stepH[w->bH] < 0) ++w->bH;
    w->bV = 0;
    while (w->bV < t && w->stepV[w->bV] < 0) ++w->bV;
    w->endH = i0;
    w->endV = i1;
    return src;
}

/* isGap of a row iterator at step index a (view positions before the trace's start are
 * residues). */
static int we_is_gap(const int32_t *step, int64_t a) { return a >= 0 && step[a] < 0; }

/* _smithWatermanDeclump (:176-299): forbids the last alignment's residue pairs, walking it from
 * its end, and recomputes the rows from the alignment's last V residue upwards, each from its
 * right end leftwards until a recomputed cell left of every earlier stop keeps its value. */
static int we_declump(we_t *w)
{
    const int32_t gap = w->p->gap;
    int64_t a0 = w->T, a1 = w->T;
    const int64_t s0 = w->bH, s1 = w->bV;
    int64_t finger0, finger1, end_col, forb;
    int32_t xe = w->endH - 1, ye = w->endV - 1, x_stop, y;
    int different, forbidden_reached = 1, end_reached = 0, skip_row = 0;
    finger0 = end_col = finger1 = forb = w->best_begin;
    (void)finger1;
    x_stop = xe;
    for (y = ye; y != -1; --y) {
        int32_t hh, vv, x;
        int cy;
        different = 1;
        if (forbidden_reached && !end_reached) {
            if (a0 == s0 && a1 == s1) end_reached = 1;
            if (!end_reached) {
                /* The walk stops only where both rows' clipped regions start; when they start at
                 * different steps (an alignment whose first column is a gap) it runs on into the
                 * rows' unaligned prefixes, and past their first view position the reference's
                 * iterators (and its forbidden-cell write) leave their arrays: undefined. */
#define WE_CHECK() do { if (w->x0 + a0 < 0 || w->y0 + a1 < 0 || forb < 0) return -1; } while (0)
                --a0;
                forb -= w->W;
                WE_CHECK();
                while (we_is_gap(w->stepH, a0) && a0 != s0) {
                    skip_row = 1;
                    --a0;
                    --a1;
                    forb -= w->W;
                    WE_CHECK();
                }
                --a1;
                forb -= 1;
                WE_CHECK();
                while (we_is_gap(w->stepV, a1) && a1 != s1) {
                    --a1;
                    --a0;
                    forb -= 1;
                    WE_CHECK();
                }
#undef WE_CHECK
                w->F[forb] = 1;
                forbidden_reached = 0;
            }
        }
        cy = w->v[y];
        hh = w->M[end_col];
        finger1 = end_col;
        end_col -= w->W;
        finger0 = end_col;
        vv = w->M[finger0];
        x = xe;
        while (x != -1 && different) {
            int32_t cs;
            --finger0;
            --finger1;
            cs = we_score(w, w->h[x], cy);
            if (w->h[x] == cy && !w->F[finger0]) {
                vv = hh + cs;
                hh = w->M[finger1];
            } else {
                int32_t sa, sb;
                if (finger0 == forb) {
                    skip_row = 0;
                    forbidden_reached = 1;
                    sa = 0;
                } else {
                    sa = w->F[finger0] ? 0 : hh + cs;
                }
                hh = w->M[finger1];
                sb = gap + (hh > vv ? hh : vv);
                vv = sa > sb ? sa : sb;
                if (vv < 0) vv = 0;
            }
            if (w->M[finger0] == vv) {
                if (x < x_stop) {
                    different = 0;
                } else if (x == xe && ((!forbidden_reached && !skip_row) || end_reached)) {
                    --xe;
                    end_col -= 1;
                }
            }
            if (x < x_stop) x_stop = x;
            w->M[finger0] = vv;
            --x;
        }
        if (xe == -1) break;
    }
    return 0;
}

/* _getNextBestEndPosition (:372-403): lazily refreshes the heap's top until its entry holds the
 * cell's current score (dropping cells below cutoff); 0 (also a real position!) means none. */
static int64_t we_next_end(we_t *w)
{
    int32_t top_score = 0;
    if (w->pq.n > 0) top_score = w->M[w->pq.a[0].id];
    if (w->pq.n > 0) {
        while (w->pq.a[0].value != top_score) {
            if (top_score >= w->p->cutoff) {
                w->pq.a[0].value = top_score;
                we_toward_leaves(&w->pq, w->pq.a[0], 0, 2);
            } else {
                we_pop(&w->pq);
            }
            if (w->pq.n > 0) top_score = w->M[w->pq.a[0].id];
            else break;
        }
    }
    if (w->pq.n == 0) return 0;
    {
        const int64_t ret = w->pq.a[0].id;
        w->best_end = ret;
        we_pop(&w->pq);
        return ret;
    }
}

int32_t orc_waterman_eggert(const orc_we_params *p, const uint8_t *h, int32_t m, const uint8_t *v, int32_t n,
                            int32_t max_count, int32_t *scores, int32_t *begins, int32_t *ends,
                            orc_segment *segs, int64_t seg_cap, int64_t *seg_off, int32_t *undefined_next)
{
    we_t w;
    int32_t k = 0, ret = 0;
    int64_t ns = 0;
    if (seg_off) seg_off[0] = 0;
    if (undefined_next) *undefined_next = 0;
    if (m <= 0 || n <= 0 || max_count <= 0) return 0;
    memset(&w, 0, sizeof(w));
    w.p = p; w.h = h; w.v = v; w.m = m; w.n = n; w.W = (int64_t)m + 1;
    w.M = (int32_t *)malloc(sizeof(int32_t) * (size_t)w.W * (size_t)(n + 1));
    w.F = (uint8_t *)calloc((size_t)w.W * (size_t)(n + 1), 1);
    w.stepH = (int32_t *)malloc(sizeof(int32_t) * (size_t)(m + n + 2));
    w.stepV = (int32_t *)malloc(sizeof(int32_t) * (size_t)(m + n + 2));
    for (k = 0; k < max_count; ++k) {
        int32_t sc;
        int64_t t, t0;
        if (k == 0) {
            /* _smithWaterman (:404-432) */
            sc = we_matrix(&w);
            if (sc == 0) break;
            w.best_begin = we_trace(&w, w.pq.a[0].id);
            we_pop(&w.pq);
        } else {
            /* _smithWatermanGetNext (:433-456) */
            int64_t e;
            if (we_declump(&w)) {
                if (undefined_next) *undefined_next = 1;
                break;
            }
            e = we_next_end(&w);
            if (e == 0) break;
            w.best_begin = we_trace(&w, e);
            sc = w.M[e];
            if (sc == 0) break;   /* nextLocalAlignment's bool */
        }
        scores[k] = w.M[w.best_end];
        begins[2 * k] = w.bH < w.T ? w.stepH[w.bH] : w.endH;
        begins[2 * k + 1] = w.bV < w.T ? w.stepV[w.bV] : w.endV;
        ends[2 * k] = w.endH;
        ends[2 * k + 1] = w.endV;
        /* the columns as runs in alignment order, from the earlier of the two rows' begins */
        t0 = w.bH < w.bV ? w.bH : w.bV;
        for (t = t0; t < w.T;) {
            const int type = (w.stepH[t] >= 0 && w.stepV[t] >= 0) ? ORC_SEG_DIAGONAL
                             : (w.stepH[t] >= 0 ? ORC_SEG_HORIZONTAL : ORC_SEG_VERTICAL);
            int64_t u = t + 1;
            uint32_t hb = 0, vb = 0;
            int64_t q;
            while (u < w.T) {
                const int ty = (w.stepH[u] >= 0 && w.stepV[u] >= 0) ? ORC_SEG_DIAGONAL
                               : (w.stepH[u] >= 0 ? ORC_SEG_HORIZONTAL : ORC_SEG_VERTICAL);
                if (ty != type) break;
                ++u;
            }
            /* run start positions: the next residue of each row at step t */
            for (q = t; q < w.T && w.stepH[q] < 0; ++q) {}
            hb = (uint32_t)(q < w.T ? w.stepH[q] : w.endH);
            for (q = t; q < w.T && w.stepV[q] < 0; ++q) {}
            vb = (uint32_t)(q < w.T ? w.stepV[q] : w.endV);
            if (ns >= seg_cap) { ret = -1; goto done; }
            segs[ns].h_begin = hb;
            segs[ns].v_begin = vb;
            segs[ns].length = (uint32_t)(u - t);
            segs[ns].type = (uint32_t)type;
            ++ns;
            t = u;
        }
        if (seg_off) seg_off[k + 1] = ns;
    }
    ret = k;
done:
    free(w.M);
    free(w.F);
    free(w.stepH);
    free(w.stepV);
    free(w.pq.a);
    return ret;
}

/* ===================================================================================== */
/* Banded Waterman-Eggert (LocalAlignmentEnumerator<Score, Banded>)                        */
/* ===================================================================================== */

/* align/local_alignment_banded_waterman_eggert_impl.h: the matrix in band storage (diagonalWidth
 * columns per row, row r covers H positions col + lowerDiag + r + lo_row), filled forward row by row
 * (_alignBandedSmithWaterman :68-151), traced back from the maximum into a (size, direction) trace
 * (_alignBandedSmithWatermanTrace :368-470), declumped forward from where that trace stopped
 * (_alignBandedSmithWatermanDeclump :175-350), the next maximum taken from the same heap as the
 * unbanded enumerator (_getNextBestEndPosition, local_alignment_waterman_eggert_impl.h:643-676). */
enum { WB_DIAG = 0, WB_HORI = 1, WB_VERT = 2, WB_STOP = 3 };

typedef struct {
    const orc_we_params *p;
    const uint8_t *h, *v;
    int64_t len1, len2;      /* |H|, |V| */
    int64_t lo, up;          /* lowerDiag, upperDiag */
    int64_t W, lo_row;       /* diagonalWidth, first row */
    int64_t height_fill;     /* rows the fill and the declump visit */
    int64_t cells;           /* matrix size */
    int32_t *M;
    uint8_t *F;
    we_heap pq;
    int64_t best_end, best_begin;
    int64_t *tsz;            /* the trace: sizes and directions in the order _alignTracePrint appends */
    uint8_t *ttv;
    int64_t nt, tcap;
    int64_t aCol, eCol, aRow, eRow;   /* alignmentPositions */
    int undef;
} wb_t;

static int wb_score(const wb_t *w, int64_t a, int64_t b)
{
    if (w->p->matrix) return w->p->matrix[(int)w->h[a] * w->p->alphabet_size + (int)w->v[b]];
    return w->h[a] == w->v[b] ? w->p->match : w->p->mismatch;
}

static void wb_print(wb_t *w, int64_t size, int tv)
{
    if (w->nt == w->tcap) {
        w->tcap = w->tcap ? 2 * w->tcap : 64;
        w->tsz = (int64_t *)realloc(w->tsz, sizeof(int64_t) * (size_t)w->tcap);
        w->ttv = (uint8_t *)realloc(w->ttv, (size_t)w->tcap);
    }
    w->tsz[w->nt] = size;
    w->ttv[w->nt] = (uint8_t)tv;
    w->nt++;
}

/* _alignBandedSmithWaterman: returns the heap's top score or 0 */
static int32_t wb_fill(wb_t *w)
{
    const int32_t gap = w->p->gap, cutoff = w->p->cutoff;
    int64_t row, col, it = w->W, it2 = 0;
    for (row = 1; row < w->height_fill; ++row) {
        const int64_t ar = row + w->lo_row;
        int32_t hori = 0;
        for (col = 0; col < w->W; ++col, ++it) {
            int64_t ac;
            if (col + w->lo + ar < 0) { ++it2; continue; }
            ac = col + w->lo + ar;
            if (ac > w->len1) { ++it2; continue; }
            if (ac != 0) {
                int32_t val = w->M[it2] + wb_score(w, ac - 1, ar - 1);
                ++it2;
                if (col < w->W - 1) { const int32_t vv = w->M[it2] + gap; if (vv > val) val = vv; }
                if (col > 0) { hori = hori + gap; if (hori > val) val = hori; }
                if (0 > val) val = 0;
                w->M[it] = val;
                if (val >= cutoff) { we_entry e; e.value = val; e.id = it; we_push(&w->pq, e); }
            } else {
                ++it2;
            }
            hori = w->M[it];
        }
    }
    if (w->pq.n > 0) { w->best_end = w->pq.a[0].id; return w->pq.a[0].value; }
    return 0;
}

/* _alignBandedSmithWatermanTrace from best_end; sets the alignment positions and best_begin */
static void wb_trace(wb_t *w)
{
    const int32_t gap = w->p->gap;
    int64_t it = w->best_end, it2 = w->best_end - w->W;
    int64_t row = it / w->W, col = it % w->W;
    int64_t ar, ac, segLen = 0;
    int tv, next;
    w->nt = 0;
    w->eRow = row + w->lo_row;
    w->eCol = col + w->lo + w->eRow;
    ar = w->eRow;
    ac = w->eCol;
    if (ac == 0 || ar == 0) { w->aCol = w->eCol = w->aRow = w->eRow = 0; return; }
    if (ac < w->len1) wb_print(w, w->len1 - ac, WB_HORI);
    if (ar < w->len2) wb_print(w, w->len2 - ar, WB_VERT);
    tv = WB_STOP;
    next = WB_HORI;
    while (next != WB_STOP) {
        tv = next;
        if (it < 0 || it >= w->cells) { w->undef = 1; return; }
        if (w->M[it] == 0) {
            next = WB_STOP;
        } else if (it2 < 0 || it2 + 1 >= w->cells || ac <= 0 || ar <= 0 || ac > w->len1 || ar > w->len2) {
            /* the reference reads outside the band storage, or a character before a sequence's
             * begin or after its end: a step at the band's last column wraps into the next stored
             * row, and the declump can write one cell past a row's last column */
            w->undef = 1;
            return;
        } else if (w->M[it] == w->M[it2] + wb_score(w, ac - 1, ar - 1)) {
            next = WB_DIAG;
            --ar; --ac; --row;
            it -= w->W; it2 -= w->W;
        } else if (w->M[it] == w->M[it2 + 1] + gap) {
            next = WB_VERT;
            --ar; --row; ++col;
            it += 1 - w->W; it2 += 1 - w->W;
        } else {
            next = WB_HORI;
            --ac; --col;
            it -= 1; it2 -= 1;
        }
        if (tv == next) ++segLen;
        else { wb_print(w, segLen, tv); segLen = 1; }
    }
    if (ac != 0) wb_print(w, ac, WB_HORI);
    if (ar != 0) wb_print(w, ar, WB_VERT);
    w->best_begin = it + w->W;
    w->aCol = ac;
    w->aRow = ar;
}

/* _alignBandedSmithWatermanDeclump */
static void wb_declump(wb_t *w)
{
    const int32_t gap = w->p->gap, cutoff = w->p->cutoff;
    const int64_t W = w->W;
    int64_t it = w->best_begin, it2;
    int64_t minCol = W, newMinCol = W, maxCol = 0, newMaxCol = 0;
    int64_t row = it / W, col = it % W, traceCol, tracePos, traceSize;
    int traceValue;
    traceCol = col;
    it -= col;
    tracePos = w->nt;
    while (tracePos > 0 && w->ttv[tracePos - 1] != WB_DIAG) --tracePos;
    if (tracePos == 0) return;
    traceSize = w->tsz[tracePos - 1];
    traceValue = w->ttv[tracePos - 1];
    while (row < w->height_fill && (maxCol > minCol || tracePos > 0)) {
        const int64_t ar = row + w->lo_row;
        while (traceSize == 0 && tracePos > 1) {
            --tracePos;
            traceValue = w->ttv[tracePos - 1];
            if (traceValue == WB_HORI) traceCol += w->tsz[tracePos - 1];
            else traceSize = w->tsz[tracePos - 1];
        }
        if (tracePos > 0) {
            if (traceValue == WB_DIAG) {
                const int64_t f = row * W + traceCol;
                --traceSize;
                if (f < 0 || f >= w->cells) { w->undef = 1; return; }
                w->F[f] = 1;
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
                const int64_t ac = col + w->lo + ar;   /* unsigned in the reference: negative reads as huge */
                int32_t nv = 0;
                if (ac < 0 || ac > w->len1) break;
                if (it < 0 || it >= w->cells || it2 < 0 || it2 + 1 >= w->cells) { w->undef = 1; return; }
                if (!w->F[it]) {
                    int32_t d;
                    if (ac == 0) { w->undef = 1; return; }   /* the reference reads H[-1] */
                    d = w->M[it2] + wb_score(w, ac - 1, ar - 1);
                    if (d > nv) nv = d;
                }
                ++it2;
                if (col > 0) { const int32_t hh = w->M[it - 1] + gap; if (hh > nv) nv = hh; }
                if (col + 1 < maxCol) { const int32_t vv = w->M[it2] + gap; if (vv > nv) nv = vv; }
                if (nv != w->M[it]) {
                    w->M[it] = nv;
                    maxCol = (maxCol > col + 2 ? maxCol : col + 2);
                    if (maxCol > W) maxCol = W;
                    if (col + 1 > newMaxCol) newMaxCol = col + 1;
                    newMinCol = col != 0 ? (newMinCol < col - 1 ? newMinCol : col - 1) : 0;
                    if (nv >= cutoff) { we_entry e; e.value = nv; e.id = it; we_push(&w->pq, e); }
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

static int64_t wb_next_end(wb_t *w)   /* _getNextBestEndPosition */
{
    int32_t top_score = 0;
    if (w->pq.n > 0) top_score = w->M[w->pq.a[0].id];
    if (w->pq.n > 0) {
        while (w->pq.a[0].value != top_score) {
            if (top_score >= w->p->cutoff) {
                w->pq.a[0].value = top_score;
                we_toward_leaves(&w->pq, w->pq.a[0], 0, 2);
            } else {
                we_pop(&w->pq);
            }
            if (w->pq.n > 0) top_score = w->M[w->pq.a[0].id];
            else break;
        }
    }
    if (w->pq.n == 0) return 0;
    {
        const int64_t ret = w->pq.a[0].id;
        w->best_end = ret;
        we_pop(&w->pq);
        return ret;
    }
}

/* The alignment's columns from the trace (_pumpTraceToGaps, align/gaps_base.h:979-1016) and the
 * two rows' clipped views (toViewPosition of the begin and of the end with rightOfGaps false):
 * the runs over the union of both views, as orc_waterman_eggert gives them. */
static int wb_emit(const wb_t *w, orc_segment *segs, int64_t seg_cap, int64_t *ns)
{
    int64_t total = 0, i, t, vh0 = -1, vh1 = 0, vv0 = -1, vv1 = 0, lo, hi;
    int64_t *sh, *sv, ch = 0, cv = 0;
    for (i = 0; i < w->nt; ++i) total += w->tsz[i];
    sh = (int64_t *)malloc(sizeof(int64_t) * (size_t)(total + 1));
    sv = (int64_t *)malloc(sizeof(int64_t) * (size_t)(total + 1));
    t = 0;
    for (i = w->nt; i > 0; --i) {
        const int64_t sz = w->tsz[i - 1];
        const int tv = w->ttv[i - 1];
        int64_t q;
        for (q = 0; q < sz; ++q, ++t) {
            sh[t] = (tv == WB_VERT) ? -1 : ch++;
            sv[t] = (tv == WB_HORI) ? -1 : cv++;
        }
    }
    /* view positions of the begins (the column of the source character) and the ends (after the
     * previous character) */
    for (t = 0; t < total; ++t) {
        if (sh[t] == w->aCol && vh0 < 0) vh0 = t;
        if (sv[t] == w->aRow && vv0 < 0) vv0 = t;
        if (sh[t] >= 0 && sh[t] == w->eCol - 1) vh1 = t + 1;
        if (sv[t] >= 0 && sv[t] == w->eRow - 1) vv1 = t + 1;
    }
    if (vh0 < 0) vh0 = vh1;
    if (vv0 < 0) vv0 = vv1;
    lo = vh0 < vv0 ? vh0 : vv0;
    hi = vh1 > vv1 ? vh1 : vv1;
    for (t = lo; t < hi;) {
        const int type = (sh[t] >= 0 && sv[t] >= 0) ? ORC_SEG_DIAGONAL : (sh[t] >= 0 ? ORC_SEG_HORIZONTAL : ORC_SEG_VERTICAL);
        int64_t u = t + 1, q;
        while (u < hi) {
            const int ty = (sh[u] >= 0 && sv[u] >= 0) ? ORC_SEG_DIAGONAL : (sh[u] >= 0 ? ORC_SEG_HORIZONTAL : ORC_SEG_VERTICAL);
            if (ty != type) break;
            ++u;
        }
        if (*ns >= seg_cap) { free(sh); free(sv); return -1; }
        for (q = t; q < total && sh[q] < 0; ++q) {}
        segs[*ns].h_begin = (uint32_t)(q < total ? sh[q] : w->len1);
        for (q = t; q < total && sv[q] < 0; ++q) {}
        segs[*ns].v_begin = (uint32_t)(q < total ? sv[q] : w->len2);
        segs[*ns].length = (uint32_t)(u - t);
        segs[*ns].type = (uint32_t)type;
        ++*ns;
        t = u;
    }
    free(sh);
    free(sv);
    return 0;
}

int32_t orc_waterman_eggert_banded(const orc_we_params *p, int32_t lower, int32_t upper, const uint8_t *h, int32_t m,
                                   const uint8_t *v, int32_t n, int32_t max_count, int32_t *scores, int32_t *begins,
                                   int32_t *ends, orc_segment *segs, int64_t seg_cap, int64_t *seg_off,
                                   int32_t *undefined_next)
{
    wb_t w;
    int32_t k = 0, ret = 0;
    int64_t ns = 0, hi_init, hi_fill, height_init;
    if (seg_off) seg_off[0] = 0;
    if (undefined_next) *undefined_next = 0;
    if (m <= 0 || n <= 0 || max_count <= 0 || upper < lower) return 0;
    memset(&w, 0, sizeof(w));
    w.p = p; w.h = h; w.v = v; w.len1 = m; w.len2 = n; w.lo = lower; w.up = upper;
    /* _initLocalAlignmentFinder [BandedWatermanEggert] (:480-505) and the fill's own row bound */
    w.lo_row = upper <= 0 ? -(int64_t)upper : 0;
    hi_init = (int64_t)n + 1;
    if ((int64_t)m - lower >= 0 && (int64_t)m - lower < hi_init) hi_init = (int64_t)m - lower;
    height_init = hi_init - w.lo_row + 1;
    hi_fill = n;
    if ((int64_t)m - lower >= 0 && (int64_t)m - lower < hi_fill) hi_fill = (int64_t)m - lower;
    w.height_fill = hi_fill - w.lo_row + 1;
    w.W = (int64_t)upper - lower + 1;
    if (height_init <= 0 || w.height_fill <= 0) return 0;
    w.cells = w.W * height_init;
    w.M = (int32_t *)calloc((size_t)w.cells, sizeof(int32_t));
    w.F = (uint8_t *)calloc((size_t)w.cells, 1);
    for (k = 0; k < max_count; ++k) {
        int32_t sc;
        if (k == 0) {
            sc = wb_fill(&w);
            if (sc < p->cutoff || sc == 0) break;    /* _localAlignment returns 0: false */
            wb_trace(&w);
            we_pop(&w.pq);
        } else {
            int64_t e;
            wb_declump(&w);
            if (w.undef) { if (undefined_next) *undefined_next = 1; break; }
            e = wb_next_end(&w);
            if (e == 0) break;
            sc = w.M[e];
            if (sc == 0) break;
            wb_trace(&w);
        }
        if (w.undef) { if (undefined_next) *undefined_next = 1; break; }
        scores[k] = w.M[w.best_end];
        begins[2 * k] = (int32_t)w.aCol;
        begins[2 * k + 1] = (int32_t)w.aRow;
        ends[2 * k] = (int32_t)w.eCol;
        ends[2 * k + 1] = (int32_t)w.eRow;
        if (wb_emit(&w, segs, seg_cap, &ns)) { ret = -1; goto done; }
        if (seg_off) seg_off[k + 1] = ns;
    }
    ret = k;
done:
    free(w.M);
    free(w.F);
    free(w.tsz);
    free(w.ttv);
    free(w.pq.a);
    return ret;
}
