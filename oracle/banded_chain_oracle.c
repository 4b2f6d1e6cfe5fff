/*
 * banded_chain_oracle.c -- CPU restatement of SeqAn 2's banded chain alignment
 * (bandedChainAlignment over a seed chain, seeds/banded_chain_alignment*.h).
 *
 * TEST INFRASTRUCTURE ONLY: the checker the GPU engine's gba_banded_chain is compared against.
 * Nothing in seqan_gb300/ links or calls it.
 *
 * What is restated (paths relative to the SeqAn 2 source tree):
 *   - the chain driver: _computeAlignment (seeds/banded_chain_alignment_impl.h:1250-1330),
 *     _findFirstAnchor / _findLastAnchor (:660-722), _initializeBandedChain (:800-966) with
 *     _initiaizeBeginningOfBandedChain (:748-794), _computeGapArea (:972-1024),
 *     _computeAnchorArea (:1030-1090), _finishBandedChain (:1096-1230), the band shifts
 *     (:195-245);
 *   - the scout state and its initialisation cells (seeds/banded_chain_alignment_scout.h:60-240):
 *     a std::set of (i1, i2, cell) whose cells of one key always compare equivalent (the cells'
 *     operator< compares scores, and one key always names the same stored cell), so the first
 *     insert of a key wins;
 *   - the grid DP: the unbanded and banded column loops of align/dp_algorithm_impl.h:483-579 and
 *     :586-967 with the BandedChainAlignment_ cell overrides (seeds/banded_chain_alignment_impl.h:
 *     409-705: initial-column and first-row cells taken from the init vectors), its recursion
 *     directions (seeds/banded_chain_alignment_profile.h:80-160), CompleteTrace ties
 *     (align/dp_formula.h:205-220), the tracking options (:260-390) and the scout
 *     (banded_chain_alignment_scout.h:212-240: >= keeps every position of the maximum);
 *   - the trace matrix as the reference stores it: band storage of L rows per column with the
 *     trace navigator's lane leaps (align/dp_matrix_navigator_trace_matrix.h:77-330), the
 *     TracebackCoordinator_ (align/dp_traceback_impl.h:57-186) and _doTraceback with GapsLeft
 *     (:196-455), the chain's traceback with its init-cell hand-off (seeds/
 *     banded_chain_alignment_traceback.h:250-370), _glueTracebacks / _smoothGluePoint (:95-200).
 * A grid that spans the whole matrix runs the GlobalAlignment_ profile with CompleteTrace
 * (orc_align_pair_complete in seqan_oracle.c).
 */
#include "seqan_oracle.h"

#include <limits.h>
#include <stdlib.h>
#include <string.h>

#define INF (INT_MIN / 2)   /* DPCellDefaultInfinity<DPCell_<int, ..>> (align/dp_cell.h:136-146) */

/* TraceBitMap_ (align/dp_profile.h) */
#define T_NONE 0
#define T_DIAG 1
#define T_H 2
#define T_V 4
#define T_HO 8
#define T_VO 16
#define T_MFH 32
#define T_MFV 64

enum { KIND_INITIAL, KIND_INNER, KIND_FINAL };     /* BandedChain{Initial,Inner,Final}DPMatrix */
enum { COL_INITIAL, COL_INNER, COL_FINAL };
enum { LOC_FULL, LOC_TOP, LOC_MIDDLE, LOC_BOTTOM };
enum { CELL_FIRST, CELL_INNER, CELL_LAST };
enum { DIR_ALL, DIR_UPPER, DIR_LOWER };

#define ERR_GLUE 1      /* the reference throws std::logic_error (no glue point) */
#define ERR_UNDEF 2     /* outside what the reference defines (an index past its vectors) */

typedef struct { int s, e, f; } cell_t;   /* score, horizontal (E), vertical (F) */
static const cell_t CELL_DEFAULT = {INF, INF, INF};

/* ---------------------------------------------------------------------------------------------
 * Traces: growable TraceSegment_ lists, stored as the reference stores them (the segment nearest
 * the end of the sequences first).
 * ------------------------------------------------------------------------------------------- */
typedef struct { orc_segment *a; int n, cap; } trace_t;
typedef struct { trace_t *t; int n, cap; } traceset_t;

static void tr_push(trace_t *t, long h, long v, long len, int type)
{
    if (t->n == t->cap) {
        t->cap = t->cap ? 2 * t->cap : 16;
        t->a = (orc_segment *)realloc(t->a, sizeof(orc_segment) * (size_t)t->cap);
    }
    t->a[t->n].h_begin = (uint32_t)h;
    t->a[t->n].v_begin = (uint32_t)v;
    t->a[t->n].length = (uint32_t)len;
    t->a[t->n].type = (uint32_t)type;
    t->n++;
}

/* _recordSegment (align/dp_trace_segment.h:318-337). */
static void record(trace_t *t, long h, long v, long len, int tv)
{
    if (len == 0) return;
    if (tv & T_DIAG) tr_push(t, h, v, len, T_DIAG);
    else if (tv & T_V) tr_push(t, h, v, len, T_V);
    else if (tv & T_H) tr_push(t, h, v, len, T_H);
}

static void ts_append(traceset_t *s, trace_t t)
{
    if (s->n == s->cap) {
        s->cap = s->cap ? 2 * s->cap : 4;
        s->t = (trace_t *)realloc(s->t, sizeof(trace_t) * (size_t)s->cap);
    }
    s->t[s->n++] = t;
}

static trace_t tr_copy(const trace_t *t)
{
    trace_t c = {NULL, 0, 0};
    if (t->n) {
        c.cap = t->n;
        c.a = (orc_segment *)malloc(sizeof(orc_segment) * (size_t)t->n);
        memcpy(c.a, t->a, sizeof(orc_segment) * (size_t)t->n);
        c.n = t->n;
    }
    return c;
}

static void ts_free(traceset_t *s)
{
    int i;
    for (i = 0; i < s->n; ++i) free(s->t[i].a);
    free(s->t);
    s->t = NULL;
    s->n = s->cap = 0;
}

static long seg_end_h(const orc_segment *g)
{
    return (g->type & (T_H | T_DIAG)) ? (long)g->h_begin + g->length : (long)g->h_begin;
}
static long seg_end_v(const orc_segment *g)
{
    return (g->type & (T_V | T_DIAG)) ? (long)g->v_begin + g->length : (long)g->v_begin;
}

/* _adaptLocalTracesToGlobalGrid (seeds/banded_chain_alignment_traceback.h:95-113). */
static void ts_adapt(traceset_t *s, long gh, long gv)
{
    int i, q;
    for (i = 0; i < s->n; ++i)
        for (q = 0; q < s->t[i].n; ++q) {
            s->t[i].a[q].h_begin = (uint32_t)((long)s->t[i].a[q].h_begin + gh);
            s->t[i].a[q].v_begin = (uint32_t)((long)s->t[i].a[q].v_begin + gv);
        }
}

/* _smoothGluePoint (:119-133): the first old segment absorbs the last new one of the same kind. */
static void smooth(trace_t *t, int old_n)
{
    int io = t->n - old_n, in = io - 1;
    if (in < 0 || io >= t->n) return;
    if (t->a[io].type == t->a[in].type) {
        t->a[io].length += t->a[in].length;
        memmove(&t->a[in], &t->a[in + 1], sizeof(orc_segment) * (size_t)(t->n - in - 1));
        t->n--;
    }
}

/* _glueTracebacks (:139-200).  Returns ERR_GLUE where the reference throws. */
static int glue(traceset_t *g, traceset_t *l)
{
    int j, i, glued = 0, n0, old_total;
    int *erase, ne = 0;
    if (g->n == 0) {
        for (i = 0; i < l->n; ++i) ts_append(g, tr_copy(&l->t[i]));
        return 0;
    }
    n0 = g->n;
    old_total = n0;
    erase = (int *)malloc(sizeof(int) * (size_t)n0);
    for (j = 0; j < n0; ++j) {
        orc_segment gend;
        if (g->t[j].n == 0) { free(erase); return ERR_UNDEF; }   /* the reference reads past an empty trace */
        gend = g->t[j].a[0];
        int cur_n = g->t[j].n, added = 0, connected = 0, id;
        for (i = 0; i < l->n; ++i) {
            const orc_segment *lb = &l->t[i].a[l->t[i].n - 1];
            if (seg_end_h(&gend) == (long)lb->h_begin && seg_end_v(&gend) == (long)lb->v_begin) {
                int add = l->t[i].n;
                if (connected) {
                    trace_t nt = {NULL, 0, 0};
                    nt.cap = cur_n + add;
                    nt.a = (orc_segment *)malloc(sizeof(orc_segment) * (size_t)nt.cap);
                    memcpy(nt.a, l->t[i].a, sizeof(orc_segment) * (size_t)add);
                    memcpy(nt.a + add, g->t[j].a + (g->t[j].n - cur_n), sizeof(orc_segment) * (size_t)cur_n);
                    nt.n = cur_n + add;
                    ts_append(g, nt);
                    ++added;
                    continue;
                }
                {
                    trace_t *t = &g->t[j];
                    if (t->cap < cur_n + add) {
                        t->cap = cur_n + add;
                        t->a = (orc_segment *)realloc(t->a, sizeof(orc_segment) * (size_t)t->cap);
                    }
                    memmove(t->a + add, t->a, sizeof(orc_segment) * (size_t)cur_n);
                    memcpy(t->a, l->t[i].a, sizeof(orc_segment) * (size_t)add);
                    t->n = cur_n + add;
                }
                glued = 1;
                connected = 1;
            }
        }
        if (!connected) {
            erase[ne++] = j;
        } else {
            smooth(&g->t[j], cur_n);
            for (id = old_total; id < old_total + added; ++id) smooth(&g->t[id], cur_n);
            old_total += added;
        }
    }
    if (!glued) { free(erase); return ERR_GLUE; }
    for (i = ne; i > 0; --i) {
        int at = erase[i - 1];
        free(g->t[at].a);
        memmove(&g->t[at], &g->t[at + 1], sizeof(trace_t) * (size_t)(g->n - at - 1));
        g->n--;
    }
    free(erase);
    return 0;
}

/* ---------------------------------------------------------------------------------------------
 * Scout state: origins of the next grid, the four init vectors and the init-cell set.
 * ------------------------------------------------------------------------------------------- */
typedef struct { long i1, i2; cell_t c; } initcell_t;

typedef struct {
    long hNext, vNext;
    cell_t *v4[4];         /* horizontal current, vertical current, horizontal next, vertical next */
    long n4[4];
    initcell_t *set;
    int nset, capset;
    int fe, affine;
    int err;
} state_t;

enum { HCUR, VCUR, HNXT, VNXT };

static int set_insert(state_t *st, long i1, long i2, cell_t c)
{
    int lo = 0, hi = st->nset;
    while (lo < hi) {
        int mid = (lo + hi) / 2;
        const initcell_t *e = &st->set[mid];
        if (e->i1 < i1 || (e->i1 == i1 && e->i2 < i2)) lo = mid + 1;
        else hi = mid;
    }
    if (lo < st->nset && st->set[lo].i1 == i1 && st->set[lo].i2 == i2) return 0;
    if (st->nset == st->capset) {
        st->capset = st->capset ? 2 * st->capset : 64;
        st->set = (initcell_t *)realloc(st->set, sizeof(initcell_t) * (size_t)st->capset);
    }
    memmove(&st->set[lo + 1], &st->set[lo], sizeof(initcell_t) * (size_t)(st->nset - lo));
    st->set[lo].i1 = i1;
    st->set[lo].i2 = i2;
    st->set[lo].c = c;
    st->nset++;
    return 1;
}

/* _reinitScoutState (banded_chain_alignment_scout.h:150-190): the vectors keep their largest
 * length, are reset to default cells and the init cells are planted into the current pair. */
static void reinit(state_t *st, long oh, long ov, long ch, long cv, long nh, long nv)
{
    long want[4];
    int k, i;
    want[HCUR] = ch; want[VCUR] = cv; want[HNXT] = nh; want[VNXT] = nv;
    if (oh < 0 || ov < 0 || ch < 0 || cv < 0 || nh < 0 || nv < 0) { st->err = ERR_UNDEF; return; }
    st->hNext = oh;
    st->vNext = ov;
    for (k = 0; k < 4; ++k) {
        long q;
        if (st->n4[k] < want[k]) {
            st->v4[k] = (cell_t *)realloc(st->v4[k], sizeof(cell_t) * (size_t)want[k]);
            st->n4[k] = want[k];
        }
        for (q = 0; q < st->n4[k]; ++q) st->v4[k][q] = CELL_DEFAULT;
    }
    for (i = 0; i < st->nset; ++i) {
        const initcell_t *e = &st->set[i];
        if (e->i1 == 0) {
            if (e->i2 >= st->n4[VCUR]) { st->err = ERR_UNDEF; return; }
            st->v4[VCUR][e->i2] = e->c;
        }
        if (e->i2 == 0) {
            if (e->i1 >= st->n4[HCUR]) { st->err = ERR_UNDEF; return; }
            st->v4[HCUR][e->i1] = e->c;
        }
    }
}

/* ---------------------------------------------------------------------------------------------
 * One grid's DP.
 * ------------------------------------------------------------------------------------------- */
typedef struct {
    int match, mismatch, ext, open;
} scheme_t;

typedef struct {
    state_t *st;
    const scheme_t *sc;
    int affine, kind, fe;
    const uint8_t *h, *v;
    long m, n;
    int banded;
    long lower, upper;
    long L, Hlen;
    uint8_t *T;
    long pos, leap;
    /* the two latest score columns (the reference's sparse column); a row outside a column's
     * computed range reads as the default cell, as an untouched dense matrix would */
    int *cS[2], *cE[2];
    long lo[2], hi[2];
    int dS, vS, vF;   /* cacheDiag score, cacheVert score and vertical score */
    int maxS;
    long *mp;
    int nmp, cmp;
} grid_t;

static inline int g_sub(const grid_t *g, uint8_t a, uint8_t b)
{
    return a == b ? g->sc->match : g->sc->mismatch;
}

/* CompleteTrace _maxScore (align/dp_formula.h:205-220). */
static inline int mx(int *target, int left, int right, int tl, int tr)
{
    if (left == right) { *target = left; return tl | tr; }
    if (left < right) { *target = right; return tr; }
    *target = left;
    return tl;
}

static inline int prevS(const grid_t *g, long col, long row)
{
    int k = (int)((col - 1) & 1);
    if (col < 1 || row < g->lo[k] || row > g->hi[k]) return INF;
    return g->cS[k][row];
}
static inline int prevE(const grid_t *g, long col, long row)
{
    int k = (int)((col - 1) & 1);
    if (col < 1 || row < g->lo[k] || row > g->hi[k]) return INF;
    return g->cE[k][row];
}

/* _goNextCell of the trace navigator (align/dp_matrix_navigator_trace_matrix.h:140-330). */
static void nav_move(grid_t *g, int coltype, int loc, int cellk)
{
    if (!g->banded) {
        if (cellk == CELL_FIRST) { if (coltype != COL_INITIAL) g->pos += g->leap; }
        else g->pos += 1;
        return;
    }
    if (cellk == CELL_FIRST) {
        if (coltype == COL_INITIAL) return;
        if (loc == LOC_TOP) { g->leap -= 1; g->pos += g->leap; }
        else g->pos += g->leap;
    } else if (cellk == CELL_INNER) {
        g->pos += 1;
    } else {
        g->pos += 1;
        if (loc == LOC_BOTTOM && coltype != COL_INITIAL) g->leap += 1;
    }
}

/* _determineTrackingOptions + _scoutBestScore (seeds/banded_chain_alignment_impl.h:260-390,
 * banded_chain_alignment_scout.h:212-240). */
static void g_track(grid_t *g, int coltype, int loc, int cellk, const cell_t *cur)
{
    state_t *st = g->st;
    long cH = g->pos / g->L, cV = g->pos % g->L;
    int storeRow = 0, storeCol = 0, lastCol = 0, lastRow = 0;
    int finalM = (g->kind == KIND_FINAL);
    if (cH >= st->hNext) {
        if (loc == LOC_BOTTOM) { if (cV + g->leap == st->vNext) storeRow = 1; }
        else if (cV == st->vNext) storeRow = 1;
        if (cH == st->hNext && cV >= st->vNext) storeCol = 1;
        if (cellk == CELL_LAST) {
            if (!finalM || (g->fe & ORC_FREE_BOTTOM)) lastRow = 1;
        }
        if (coltype == COL_FINAL) {
            if (cellk == CELL_LAST) { lastCol = 1; lastRow = 1; }
            else if (loc != LOC_FULL || cV >= st->vNext) {
                if (!finalM || (g->fe & ORC_FREE_RIGHT)) lastCol = 1;
            }
        }
    }
    if (storeCol) {
        long q = cV - st->vNext;
        if (q >= st->n4[VNXT]) { st->err = ERR_UNDEF; return; }
        st->v4[VNXT][q] = *cur;
    }
    if (storeRow) {
        long q = cH - st->hNext;
        if (q >= st->n4[HNXT]) { st->err = ERR_UNDEF; return; }
        st->v4[HNXT][q] = *cur;
    }
    if ((lastCol || lastRow) && cur->s >= g->maxS) {
        if (cur->s != g->maxS) { g->nmp = 0; g->maxS = cur->s; }
        if (g->nmp == g->cmp) {
            g->cmp = g->cmp ? 2 * g->cmp : 16;
            g->mp = (long *)realloc(g->mp, sizeof(long) * (size_t)g->cmp);
        }
        g->mp[g->nmp++] = g->pos;
    }
}

/* One cell: navigator step, the cell (chain override or recursion), trace value, tracking. */
static void g_cell(grid_t *g, int coltype, int loc, int cellk, long col, long row)
{
    state_t *st = g->st;
    cell_t cur;
    int tv = T_NONE, k = (int)(col & 1);
    int hS, hE;
    if (st->err) return;
    nav_move(g, coltype, loc, cellk);
    if (g->pos < 0 || g->pos >= g->L * g->Hlen) { st->err = ERR_UNDEF; return; }
    hS = prevS(g, col, row);
    hE = prevE(g, col, row);
    if (coltype == COL_INITIAL) {
        /* _computeCell [BandedChainAlignment, DPInitialColumn] (:455-490) */
        long idx = (g->pos % g->L) - (g->leap - 1);
        if (idx < 0 || idx >= st->n4[VCUR]) { st->err = ERR_UNDEF; return; }
        g->dS = hS;
        cur = st->v4[VCUR][idx];
        g->vS = cur.s;
        g->vF = cur.f;
    } else if (cellk == CELL_FIRST && (loc == LOC_TOP || loc == LOC_FULL)) {
        /* _computeHorizontalInitCell (:495-510) for the first cell of full / top columns */
        long idx = g->pos / g->L;
        if (idx >= st->n4[HCUR]) { st->err = ERR_UNDEF; return; }
        g->dS = hS;
        cur = st->v4[HCUR][idx];
        g->vS = cur.s;
        g->vF = cur.f;
    } else {
        int dir = (cellk == CELL_INNER) ? DIR_ALL
                : (cellk == CELL_FIRST) ? DIR_UPPER
                : (loc == LOC_TOP || loc == LOC_MIDDLE) ? DIR_LOWER : DIR_ALL;
        int sub = g_sub(g, g->h[col - 1], g->v[row - 1]);
        const scheme_t *sc = g->sc;
        if (g->affine) {
            /* align/dp_formula_affine.h:66-238 */
            if (dir == DIR_ALL) {
                int inter = g->dS + sub, t2, s;
                g->dS = hS;
                tv = mx(&cur.e, hE + sc->ext, hS + sc->open, T_H, T_HO);
                tv |= mx(&g->vF, g->vF + sc->ext, g->vS + sc->open, T_V, T_VO);
                t2 = mx(&s, g->vF, cur.e, T_MFV, T_MFH);
                tv = mx(&cur.s, inter, s, T_DIAG | tv, t2 | tv);
                g->vS = cur.s;
            } else if (dir == DIR_UPPER) {
                int inter = g->dS + sub;
                g->dS = hS;
                tv = mx(&cur.e, hE + sc->ext, hS + sc->open, T_H, T_HO);
                g->vF = INF;
                tv = mx(&cur.s, inter, cur.e, tv | T_DIAG, tv | T_MFH);
                g->vS = cur.s;
            } else {
                tv = mx(&g->vF, g->vF + sc->ext, g->vS + sc->open, T_V, T_VO);
                cur.e = INF;
                tv = mx(&cur.s, g->dS + sub, g->vF, tv | T_DIAG, tv | T_MFV);
            }
            cur.f = g->vF;   /* _setVerticalScoreOfCell(current, vertical) before tracking */
        } else {
            /* align/dp_formula_linear.h:62-190 */
            if (dir == DIR_ALL) {
                int inter = g->dS + sub, s;
                g->dS = hS;
                tv = mx(&s, g->vS + sc->ext, hS + sc->ext, T_V | T_MFV, T_H | T_MFH);
                tv = mx(&cur.s, inter, s, T_DIAG, tv);
                g->vS = cur.s;
            } else if (dir == DIR_UPPER) {
                int inter = g->dS + sub;
                g->dS = hS;
                tv = mx(&cur.s, inter, hS + sc->ext, T_DIAG, T_H | T_MFH);
                g->vS = cur.s;
            } else {
                tv = mx(&cur.s, g->dS + sub, g->vS + sc->ext, T_DIAG, T_V | T_MFV);
            }
            cur.e = INF;
            cur.f = INF;
        }
    }
    if (row < g->lo[k]) g->lo[k] = row;
    if (row > g->hi[k]) g->hi[k] = row;
    g->cS[k][row] = cur.s;
    g->cE[k][row] = cur.e;
    g->T[g->pos] = (uint8_t)tv;
    g_track(g, coltype, loc, cellk, &cur);
}

static void g_new_col(grid_t *g, long col)
{
    int k = (int)(col & 1);
    g->lo[k] = LONG_MAX;
    g->hi[k] = -1;
}

/* _computeTrack (align/dp_algorithm_impl.h:334-429): rows r0..r1 of column col. */
static void g_track_col(grid_t *g, long col, int coltype, int loc, long r0, long r1)
{
    long i;
    g_new_col(g, col);
    g->dS = INF; g->vS = INF; g->vF = INF;
    /* _preInitCacheDiagonal: middle and bottom columns start below their diagonal neighbour */
    if (coltype != COL_INITIAL && (loc == LOC_MIDDLE || loc == LOC_BOTTOM) && r0 > 0 && col > 0)
        g->dS = prevS(g, col, r0 - 1);
    g_cell(g, coltype, loc, CELL_FIRST, col, r0);
    for (i = r0 + 1; i < r1; ++i) g_cell(g, coltype, loc, CELL_INNER, col, i);
    g_cell(g, coltype, loc, CELL_LAST, col, r1);
}

#define MIN(a, b) ((a) < (b) ? (a) : (b))
#define MAX(a, b) ((a) > (b) ? (a) : (b))

static void g_run_unbanded(grid_t *g)
{
    long col;
    g_track_col(g, 0, COL_INITIAL, LOC_FULL, 0, g->n);
    for (col = 1; col < g->m; ++col) g_track_col(g, col, COL_INNER, LOC_FULL, 0, g->n);
    g_track_col(g, g->m, COL_FINAL, LOC_FULL, 0, g->n);
}

/* The banded column loop (align/dp_algorithm_impl.h:586-967). */
static void g_run_banded(grid_t *g)
{
    long m = g->m, n = g->n, lower = g->lower, upper = g->upper;
    long vb = -MIN(0, 1 + upper), ve = -MIN(0, MAX(-n, lower));
    long hb = MAX(0, MIN(m - 1, lower));
    long hTop = MIN(m - 1, MAX(0, upper)), hMid = MIN(m - 1, MAX(0, n + lower)), hBot, hIt, t;
    if (upper > n + lower) { t = hTop; hTop = hMid; hMid = t; }
    hBot = MAX(0, MIN(m, upper + n) - 1);
    if (hb == m - 1) {
        long col = MAX(0, MIN(m, lower));
        g_new_col(g, col);
        g->dS = INF; g->vS = INF; g->vF = INF;
        g_cell(g, COL_INITIAL, LOC_TOP, CELL_FIRST, col, 0);
        return;
    }
    if (hBot == 0) {
        g_new_col(g, 0);
        g->dS = INF; g->vS = INF; g->vF = INF;
        g_cell(g, COL_INITIAL, LOC_BOTTOM, CELL_FIRST, 0, MIN(n, -upper));
        return;
    }
    if (upper < 0) {
        ++vb;
        g_track_col(g, 0, COL_INITIAL, lower > -n ? LOC_MIDDLE : LOC_BOTTOM, vb, ve);
    } else if (lower >= 0) {
        g_new_col(g, hb);
        g->dS = INF; g->vS = INF; g->vF = INF;
        g_cell(g, COL_INITIAL, LOC_TOP, CELL_FIRST, hb, 0);
    } else {
        g_track_col(g, 0, COL_INITIAL, lower <= -n ? LOC_FULL : LOC_TOP, vb, ve);
    }
    hIt = hb;
    for (; hIt != hTop; ++hIt) {
        ++ve;
        g_track_col(g, hIt + 1, COL_INNER, LOC_TOP, vb, ve);
    }
    if (upper > n + lower) {
        for (; hIt != hMid; ++hIt) g_track_col(g, hIt + 1, COL_INNER, LOC_FULL, vb, ve);
    } else {
        for (; hIt != hMid; ++hIt) {
            ++vb; ++ve;
            g_track_col(g, hIt + 1, COL_INNER, LOC_MIDDLE, vb, ve);
        }
    }
    for (; hIt != hBot; ++hIt) {
        ++vb;
        g_track_col(g, hIt + 1, COL_INNER, LOC_BOTTOM, vb, ve);
    }
    if (hIt < m - 1) {
        /* The band ends before the final column: one bottom cell. */
        g_new_col(g, hIt + 1);
        g->dS = prevS(g, hIt + 1, vb); g->vS = INF; g->vF = INF;
        g_cell(g, COL_INNER, LOC_BOTTOM, CELL_FIRST, hIt + 1, vb + 1);
    } else if (hIt == m - 1) {
        if (upper == m - n) {
            g_new_col(g, m);
            g->dS = prevS(g, m, vb); g->vS = INF; g->vF = INF;
            g_cell(g, COL_FINAL, LOC_BOTTOM, CELL_FIRST, m, vb + 1);
        } else if (upper >= m) {
            if (lower + n > m) { ++ve; g_track_col(g, m, COL_FINAL, LOC_TOP, vb, ve); }
            else if (lower + n + 1 > m) { ++ve; g_track_col(g, m, COL_FINAL, LOC_TOP, vb, ve); }
            else g_track_col(g, m, COL_FINAL, LOC_FULL, vb, ve);
        } else {
            ++vb;
            if (lower + n <= m) {
                if (lower + n == m) { ++ve; g_track_col(g, m, COL_FINAL, LOC_MIDDLE, vb, ve); }
                else g_track_col(g, m, COL_FINAL, LOC_BOTTOM, vb, ve);
            } else {
                ++ve;
                g_track_col(g, m, COL_FINAL, LOC_MIDDLE, vb, ve);
            }
        }
    }
}

/* ---------------------------------------------------------------------------------------------
 * Traceback over the band storage.
 * ------------------------------------------------------------------------------------------- */
typedef struct { long cc, cr, ec, er, bp1, bp2; int band; } coord_t;

/* TracebackCoordinator_ with _initTracebackCoordinator (align/dp_traceback_impl.h:57-171). */
static void coord_init(coord_t *c, const grid_t *g, long cc, long cr, long ec, long er)
{
    c->cc = cc; c->cr = cr; c->ec = ec; c->er = er; c->bp1 = 0; c->bp2 = 0; c->band = 0;
    if (g->banded) {
        long b;
        if (g->lower >= 0) c->cc += g->lower;
        if (c->cc > g->upper) c->cr += c->cc - g->upper;
        if (c->ec > g->upper) c->er += c->ec - g->upper;
        c->bp1 = MIN(g->m, MAX(0, g->upper));
        c->bp2 = MIN(g->m, MAX(0, g->n + g->lower));
        b = MIN(c->bp1, c->bp2);
        if (c->cc < b) c->cr -= b - c->cc;
        c->band = 1;
    }
}
static int reached_end(const coord_t *c) { return c->cc <= c->ec || c->cr <= c->er; }
static int in_band(const coord_t *c) { return c->band && (c->cc > c->bp1 || c->cc <= c->bp2); }

/* _retrieveInitialTraceDirection (:456-483). */
static int initial_dir(int *tv, int prefer_gaps_at_end)
{
    if (prefer_gaps_at_end) {
        if (*tv & T_MFV) { *tv &= (T_V | T_VO | T_MFV); return T_V; }
        if (*tv & T_MFH) { *tv &= (T_H | T_HO | T_MFH); return T_H; }
        return T_DIAG;
    }
    if (*tv & T_DIAG) return T_DIAG;
    if (*tv & (T_V | T_MFV)) return T_V;
    if (*tv & (T_H | T_MFH)) return T_H;
    return T_NONE;
}

typedef struct { grid_t *g; long pos; int tv, last; long frag; coord_t c; int bad; } walk_t;

static void w_step(walk_t *w, long delta)
{
    if (delta <= 0) { w->bad = 1; w->tv = T_NONE; return; }   /* a one-row band: the walk would not move */
    w->pos -= delta;
    if (w->pos < 0 || w->pos >= w->g->L * w->g->Hlen) { w->bad = 1; w->tv = T_NONE; return; }
    w->tv = w->g->T[w->pos];
}
static void w_switch(walk_t *w, trace_t *t, int dirbit)
{
    if (!(w->last & dirbit)) {
        record(t, w->c.cc, w->c.cr, w->frag, w->last);
        w->last = dirbit;
        w->frag = 0;
    }
}

/* _doTraceback with GapsLeft (:376-415) and its moves (:196-373). */
static void do_trace(walk_t *w, trace_t *t)
{
    long L = w->g->L;
    int tv = w->tv;
    if (tv & T_DIAG) {
        w_switch(w, t, T_DIAG);
        w_step(w, in_band(&w->c) ? L : L + 1);
        --w->c.cc; --w->c.cr; ++w->frag;
    } else if ((tv & T_MFV) && (tv & T_V)) {
        w_switch(w, t, T_V);
        if (w->g->affine) {
            while ((!(w->tv & T_VO) || (w->tv & T_V)) && w->c.cr != 1 && !w->bad) {
                w_step(w, 1);
                --w->c.cr; ++w->frag;
            }
        }
        w_step(w, 1);
        --w->c.cr; ++w->frag;
    } else if ((tv & T_MFV) && (tv & T_VO)) {
        w_switch(w, t, T_V);
        w_step(w, 1);
        --w->c.cr; ++w->frag;
    } else if ((tv & T_MFH) && (tv & T_H)) {
        w_switch(w, t, T_H);
        if (w->g->affine) {
            while ((!(w->tv & T_HO) || (w->tv & T_H)) && w->c.cc != 1 && !w->bad) {
                w_step(w, in_band(&w->c) ? L - 1 : L);
                --w->c.cc; ++w->frag;
            }
        }
        w_step(w, in_band(&w->c) ? L - 1 : L);
        --w->c.cc; ++w->frag;
    } else if ((tv & T_MFH) && (tv & T_HO)) {
        w_switch(w, t, T_H);
        w_step(w, in_band(&w->c) ? L - 1 : L);
        --w->c.cc; ++w->frag;
    } else {
        /* a value the reference asserts on: with NDEBUG its walk never ends */
        w->bad = 1;
        w->tv = T_NONE;
    }
}

static int prefer_end(const grid_t *g) { return g->affine && g->kind == KIND_FINAL; }

/* The generic _computeTraceback of a BandedChainAlignment_ profile (no head, no tail;
 * align/dp_traceback_impl.h:489-546) from the navigator's position. */
static int generic_trace(grid_t *g, trace_t *t, long *pos)
{
    walk_t w;
    w.g = g; w.pos = *pos; w.bad = 0; w.frag = 0;
    w.tv = g->T[*pos];
    w.last = initial_dir(&w.tv, prefer_end(g));
    coord_init(&w.c, g, *pos / g->L, *pos % g->L, 0, 0);
    while (!reached_end(&w.c) && w.tv != T_NONE && !w.bad) do_trace(&w, t);
    record(t, w.c.cc, w.c.cr, w.frag, w.last);
    *pos = w.pos;
    return w.bad ? ERR_UNDEF : 0;
}

/* _correctDPCellForAffineGaps (seeds/banded_chain_alignment_traceback.h:206-228). */
static void correct_cell(cell_t *c, int last, int affine)
{
    if (!affine) return;
    if (last & T_DIAG) { c->f = INF; c->e = INF; }
    else if (last & T_V) c->e = INF;
    else c->f = INF;
}

/* The chain's _computeTraceback for one maximum (:250-355). */
static int chain_trace_one(grid_t *g, long maxpos, traceset_t *out)
{
    state_t *st = g->st;
    trace_t tgt = {NULL, 0, 0}, tmp = {NULL, 0, 0};
    walk_t w;
    long hip, vip;
    int ins, rc = 0;
    w.g = g; w.pos = maxpos; w.bad = 0; w.frag = 0;
    w.tv = g->T[maxpos];
    w.last = initial_dir(&w.tv, prefer_end(g));
    coord_init(&w.c, g, maxpos / g->L, maxpos % g->L, st->hNext, st->vNext);
    if (g->kind == KIND_FINAL) {
        long pos = maxpos;
        if (w.c.cr != g->n) record(&tgt, g->m, w.c.cr, g->n - w.c.cr, T_V);
        if (w.c.cc != g->m) record(&tgt, w.c.cc, w.c.cr, g->m - w.c.cc, T_H);
        rc = generic_trace(g, &tgt, &pos);
        if (tgt.n) ts_append(out, tgt); else free(tgt.a);
        return rc;
    }
    while (!reached_end(&w.c) && w.tv != T_NONE && !w.bad) do_trace(&w, &tmp);
    free(tmp.a);
    if (w.bad) { free(tgt.a); return ERR_UNDEF; }
    hip = w.c.cc - w.c.ec;
    vip = w.c.cr - w.c.er;
    if (vip <= 0) {
        if (hip < 0 || hip >= st->n4[HNXT]) { free(tgt.a); return ERR_UNDEF; }
        correct_cell(&st->v4[HNXT][hip], w.last, g->affine);
        ins = set_insert(st, hip, 0, st->v4[HNXT][hip]);
    } else {
        if (vip >= st->n4[VNXT]) { free(tgt.a); return ERR_UNDEF; }
        correct_cell(&st->v4[VNXT][vip], w.last, g->affine);
        ins = set_insert(st, 0, vip, st->v4[VNXT][vip]);
    }
    if (ins) {
        if (vip < 0) record(&tgt, w.c.cc, w.c.cr, -vip, w.last);
        else if (hip < 0) record(&tgt, w.c.cc, w.c.cr, -hip, w.last);
        rc = generic_trace(g, &tgt, &w.pos);
    }
    if (g->kind == KIND_INITIAL) {
        long cc = w.pos / g->L, cr = w.pos % g->L;
        if (g->banded && g->upper > 0 && cc < w.c.bp1 && cc < w.c.bp2) cr -= g->L - 1 + g->lower - cc;
        if (cr != 0) record(&tgt, 0, 0, cr, T_V);
        if (cc != 0) record(&tgt, 0, 0, cc, T_H);
    }
    if (tgt.n) ts_append(out, tgt); else free(tgt.a);
    return rc;
}

/* _computeAlignment of one grid with the BandedChainAlignment_ profile: returns the score and
 * appends the grid's traces to out (align/dp_algorithm_impl.h:1371-1445, _finishAlignment
 * :1330-1355 with CompleteTrace). */
static int run_grid(state_t *st, const scheme_t *sc, int kind, int banded, long lower, long upper,
                    const uint8_t *h, long m, const uint8_t *v, long n, traceset_t *out)
{
    grid_t g;
    int q, score;
    if (st->err) return INT_MIN;
    if (m <= 0 || n <= 0) return INT_MIN;
    if (banded) {
        /* _checkBandProperties with the chain's free ends (align/dp_algorithm_impl.h:193-234) */
        if (upper < -n || lower > m) return INT_MIN;
        if (upper < 0 && !(st->fe & ORC_FREE_LEFT)) return INT_MIN;
        if (lower > 0 && !(st->fe & ORC_FREE_TOP)) return INT_MIN;
        if (upper + n < m && !(st->fe & ORC_FREE_BOTTOM)) return INT_MIN;
        if (lower + n > m && !(st->fe & ORC_FREE_RIGHT)) return INT_MIN;
    }
    memset(&g, 0, sizeof(g));
    g.st = st; g.sc = sc; g.affine = st->affine; g.kind = kind; g.fe = st->fe;
    g.h = h; g.v = v; g.m = m; g.n = n; g.banded = banded; g.lower = lower; g.upper = upper;
    if (banded) {
        long bs = MIN(m, upper) - MAX(lower, -n) + 1;
        g.L = MIN(n + 1, bs);
        g.Hlen = m + 1 - MAX(0, lower);
        if (lower >= 0) { g.leap = MIN(g.L, upper - lower + 1); g.pos = g.L - 1; }
        else if (upper <= 0) { g.leap = 1; g.pos = 0; }
        else { long lp = MAX(-(g.L - 1), lower); g.leap = g.L + lp; g.pos = g.leap - 1; }
    } else {
        g.L = n + 1;
        g.Hlen = m + 1;
        g.leap = 1;
        g.pos = 0;
    }
    g.T = (uint8_t *)calloc((size_t)(g.L * g.Hlen), 1);
    for (q = 0; q < 2; ++q) {
        g.cS[q] = (int *)malloc(sizeof(int) * (size_t)(n + 1));
        g.cE[q] = (int *)malloc(sizeof(int) * (size_t)(n + 1));
        g.lo[q] = LONG_MAX;
        g.hi[q] = -1;
    }
    g.maxS = INF;
    if (banded && upper == lower) st->err = ERR_UNDEF;   /* never built by a chain */
    else if (banded) g_run_banded(&g);
    else g_run_unbanded(&g);
    score = g.maxS;
    if (!st->err) {
        /* _computeTraceback [BandedChainAlignment, global interface] (:360-385) */
        int i;
        st->nset = 0;
        for (i = 0; i < g.nmp && !st->err; ++i) {
            int rc = chain_trace_one(&g, g.mp[i], out);
            if (rc) st->err = rc;
        }
    }
    free(g.T);
    for (q = 0; q < 2; ++q) { free(g.cS[q]); free(g.cE[q]); }
    free(g.mp);
    return score;
}

/* A grid that spans the whole matrix: GlobalAlignment_ with CompleteTrace, banded
 * (seeds/banded_chain_alignment_impl.h:929-936). */
static int run_global_grid(state_t *st, const scheme_t *sc, long lower, long upper, const uint8_t *h, long m,
                           const uint8_t *v, long n, traceset_t *out)
{
    orc_params p;
    orc_result r;
    orc_segment *segs;
    trace_t t = {NULL, 0, 0};
    int cap = (int)(2 * (m + n) + 16), q;
    memset(&p, 0, sizeof(p));
    p.mode = ORC_GLOBAL;
    p.gap_model = st->affine ? ORC_AFFINE : ORC_LINEAR;
    p.free_ends = st->fe;
    p.band_on = 1;
    p.band_lower = (int32_t)lower;
    p.band_upper = (int32_t)upper;
    p.match = sc->match; p.mismatch = sc->mismatch; p.gap_open = sc->open; p.gap_extend = sc->ext;
    p.score_bits = 32;
    p.traceback = 1;
    segs = (orc_segment *)malloc(sizeof(orc_segment) * (size_t)cap);
    orc_align_pair_complete(&p, h, (int32_t)m, v, (int32_t)n, &r, segs, cap);
    if (r.n_segments < 0) { st->err = ERR_UNDEF; free(segs); return INT_MIN; }
    for (q = 0; q < r.n_segments; ++q) tr_push(&t, segs[q].h_begin, segs[q].v_begin, segs[q].length, (int)segs[q].type);
    ts_append(out, t);   /* localTraceSet[0], empty or not */
    free(segs);
    return r.score;
}

/* ---------------------------------------------------------------------------------------------
 * The chain driver.
 * ------------------------------------------------------------------------------------------- */
typedef struct { long bh, bv, eh, ev, lo, up; } seed_t;   /* Seed<Simple> */

typedef struct {
    state_t st;
    scheme_t anchor, gap;
    const uint8_t *h, *v;
    long m, n, k;
    traceset_t global;
} chain_t;

static long hshift_begin(const seed_t *s) { return s->up - (s->bh - s->bv); }
static long vshift_begin(const seed_t *s) { return (s->bh - s->bv) - s->lo; }
static long hshift_end(const seed_t *s) { return s->eh - s->ev - s->lo; }
static long vshift_end(const seed_t *s) { return s->up - s->eh + s->ev; }

static int glue_local(chain_t *ch, traceset_t *local, long gh, long gv, int check_empty)
{
    int rc = 0;
    ts_adapt(local, gh, gv);
    if (!check_empty || local->n) rc = glue(&ch->global, local);
    ts_free(local);
    if (rc && !ch->st.err) ch->st.err = rc;
    return rc;
}

/* _initiaizeBeginningOfBandedChain (:748-794). */
static void init_beginning(chain_t *ch, long sizeH, long sizeV, const scheme_t *sc)
{
    state_t *st = &ch->st;
    cell_t c = {0, INF, INF}, cv;
    long i;
    set_insert(st, 0, 0, c);
    for (i = 1; i < sizeH; ++i) {
        cell_t prev = c;
        if (st->fe & ORC_FREE_TOP) {
            c.s = 0;
        } else if (st->affine) {
            mx(&c.e, prev.e + sc->ext, prev.s + sc->open, 0, 0);
            c.s = c.e;
        } else {
            c.s = prev.s + sc->ext;
        }
        set_insert(st, i, 0, c);
    }
    cv.s = 0; cv.e = INF; cv.f = INF;
    for (i = 1; i < sizeV; ++i) {
        if (st->fe & ORC_FREE_LEFT) {
            cv.s = 0;
        } else if (st->affine) {
            mx(&cv.f, cv.f + sc->ext, cv.s + sc->open, 0, 0);
            cv.s = cv.f;
        } else {
            cv.s = cv.s + sc->ext;
        }
        set_insert(st, 0, i, cv);
    }
}

static int initialize_chain(chain_t *ch, const seed_t *s)
{
    state_t *st = &ch->st;
    long k = ch->k, m = ch->m, n = ch->n;
    long hs = hshift_begin(s), vs = vshift_begin(s);
    long hN = MAX(0, s->bh + 1 - k), vN = MAX(0, s->bv + 1 - k);
    long upper = MIN(m, hN + 2 * k + hs + MAX(0, k - s->bv - 1) + MIN(0, s->bh + 1 - k));
    long lower = -MIN(n, vN + 2 * k + vs + MAX(0, k - s->bh - 1) + MIN(0, s->bv + 1 - k));
    long gbh, gbv, geh, gev, lh, lv, hN2, vN2;
    int score = 0;
    traceset_t local = {NULL, 0, 0};
    if (hN != 0 || vN != 0) {
        init_beginning(ch, upper + 1, 1 - lower, &ch->gap);
        reinit(st, hN, vN, 1 + upper, 1 - lower, 1 + upper - hN, 1 - lower - vN);
        score = run_grid(st, &ch->gap, KIND_INITIAL, 0, 0, 0, ch->h, upper, ch->v, -lower, &ch->global);
    } else {
        init_beginning(ch, upper, -lower, &ch->anchor);
    }
    gbh = hN; gbv = vN;
    geh = MIN(m, s->eh + k);
    gev = MIN(n, s->ev + k);
    lh = geh - gbh;
    lv = gev - gbv;
    hN2 = MAX(0, s->eh - k - hshift_end(s) - MAX(0, s->ev + k - n) - gbh);
    vN2 = MAX(0, s->ev - k - vshift_end(s) - MAX(0, s->eh + k - m) - gbv);
    upper -= gbh;
    lower += gbv;
    if (lv + lower > upper) vN2 -= (lv + lower) - upper;
    reinit(st, hN2, vN2, upper + 1, 1 - lower, lh - hN2 + 1, lv - vN2 + 1);
    if (gbh == 0 && gbv == 0) {
        if (geh == m && gev == n)
            score = run_global_grid(st, &ch->gap, lower, upper, ch->h, lh, ch->v, lv, &local);
        else
            score = run_grid(st, &ch->gap, KIND_INITIAL, 1, lower, upper, ch->h, lh, ch->v, lv, &local);
    } else {
        score = run_grid(st, &ch->gap, (geh == m && gev == n) ? KIND_FINAL : KIND_INNER, 1, lower, upper,
                         ch->h + gbh, lh, ch->v + gbv, lv, &local);
    }
    if (gbh != 0 || gbv != 0) {
        glue_local(ch, &local, gbh, gbv, 1);
    } else {
        ts_free(&ch->global);
        ch->global = local;
    }
    st->hNext += gbh;
    st->vNext += gbv;
    if (lv + lower > upper) st->vNext += (lv + lower) - upper;
    return score;
}

static void gap_area(chain_t *ch, const seed_t *s)
{
    state_t *st = &ch->st;
    long k = ch->k;
    long gbh = st->hNext, gbv = st->vNext;
    long geh = s->bh + 1 + k + hshift_begin(s), gev = s->bv + 1 + k + vshift_begin(s);
    long hN = s->bh + 1 - k - gbh, vN = s->bv + 1 - k - gbv;
    traceset_t local = {NULL, 0, 0};
    if (geh > ch->m || gev > ch->n || gbh > geh || gbv > gev) { st->err = ERR_UNDEF; return; }
    reinit(st, hN, vN, geh - gbh + 1, gev - gbv + 1, geh - gbh + 1 - hN, gev - gbv + 1 - vN);
    run_grid(st, &ch->gap, KIND_INNER, 0, 0, 0, ch->h + gbh, geh - gbh, ch->v + gbv, gev - gbv, &local);
    glue_local(ch, &local, gbh, gbv, 1);
    st->hNext += gbh;
    st->vNext += gbv;
}

static void anchor_area(chain_t *ch, const seed_t *s)
{
    state_t *st = &ch->st;
    long k = ch->k;
    long gbh = st->hNext, gbv = st->vNext;
    long geh = s->eh + k, gev = s->ev + k;
    long lh = geh - gbh, lv = gev - gbv;
    long hN = s->eh - k - hshift_end(s) - gbh, vN = s->ev - k - vshift_end(s) - gbv;
    long lower = -2 * k - vshift_begin(s), upper = 2 * k + hshift_begin(s), relV = vN;
    traceset_t local = {NULL, 0, 0};
    if (geh > ch->m || gev > ch->n || lh < 0 || lv < 0) { st->err = ERR_UNDEF; return; }
    if (lv + lower > upper) relV -= (lv + lower) - upper;
    reinit(st, hN, relV, upper + 1, 1 - lower, lh - hN + 1, lv - vN + 1);
    run_grid(st, &ch->anchor, KIND_INNER, 1, lower, upper, ch->h + gbh, lh, ch->v + gbv, lv, &local);
    glue_local(ch, &local, gbh, gbv, 1);
    st->hNext += gbh;
    st->vNext += gbv;
    if (lv + lower > upper) st->vNext += (lv + lower) - upper;
}

static int finish_chain(chain_t *ch, const seed_t *s)
{
    state_t *st = &ch->st;
    long k = ch->k, m = ch->m, n = ch->n;
    long gbh = st->hNext, gbv = st->vNext;
    long hs = hshift_begin(s), vs = vshift_begin(s);
    long geh = MIN(m, s->bh + 1 + k + hs), gev = MIN(n, s->bv + 1 + k + vs);
    long lh = geh - gbh, lv = gev - gbv;
    long hN = MAX(0, s->bh + 1 - k - gbh), vN = MAX(0, s->bv + 1 - k - gbv);
    long lower, upper;
    int score;
    traceset_t local = {NULL, 0, 0};
    if (lh < 0 || lv < 0) { st->err = ERR_UNDEF; return INT_MIN; }
    /* Part A: the rectangle between the last two anchors */
    reinit(st, hN, vN, lh + 1, lv + 1, lh - hN + 1, lv - vN + 1);
    run_grid(st, &ch->gap, KIND_INNER, 0, 0, 0, ch->h + gbh, lh, ch->v + gbv, lv, &local);
    glue_local(ch, &local, gbh, gbv, 1);
    /* Part B: the last anchor */
    gbh += hN;
    gbv += vN;
    geh = MIN(m, s->eh + k);
    gev = MIN(n, s->ev + k);
    lh = geh - gbh;
    lv = gev - gbv;
    if (lh < 0 || lv < 0) { st->err = ERR_UNDEF; return INT_MIN; }
    if (geh == m && gev == n) {
        lower = -(gev - gbv);
        upper = geh - gbh;
        reinit(st, 0, 0, upper + 1, 1 - lower, upper + 1, 1 - lower);
        score = run_grid(st, &ch->anchor, KIND_FINAL, 1, lower, upper, ch->h + gbh, lh, ch->v + gbv, lv, &local);
        glue_local(ch, &local, gbh, gbv, 1);
        return score;
    }
    lower = -2 * k - vs;
    upper = 2 * k + hs;
    hN = MAX(0, s->eh - k - hshift_end(s) - gbh - MAX(0, s->ev + k - n));
    vN = MAX(0, s->ev - k - vshift_end(s) - gbv - MAX(0, s->eh + k - m));
    if (lv + lower > upper) vN -= (lv + lower) - upper;
    reinit(st, hN, vN, upper + 1, 1 - lower, lh - hN + 1, lv - vN + 1);
    run_grid(st, &ch->anchor, KIND_INNER, 1, lower, upper, ch->h + gbh, lh, ch->v + gbv, lv, &local);
    glue_local(ch, &local, gbh, gbv, 1);
    /* the gap between the last anchor and the end of the matrix */
    gbh += hN;
    if (lv + lower > upper) vN += (lv + lower) - upper;
    gbv += vN;
    if (gbh > m || gbv > n) { st->err = ERR_UNDEF; return INT_MIN; }
    reinit(st, 0, 0, m - gbh + 1, n - gbv + 1, m - gbh + 1, n - gbv + 1);
    score = run_grid(st, &ch->gap, KIND_FINAL, 0, 0, 0, ch->h + gbh, m - gbh, ch->v + gbv, n - gbv, &local);
    glue_local(ch, &local, gbh, gbv, 1);
    return score;
}

int32_t orc_banded_chain(const orc_chain_params *p, const uint8_t *h, int32_t m, const uint8_t *v, int32_t n,
                         int32_t n_seeds, const int32_t *seeds, int32_t *score, orc_segment *segs,
                         int32_t seg_cap, int32_t *n_segs, int32_t *n_traces)
{
    chain_t ch;
    seed_t *sd;
    long i, it, itEnd, N = n_seeds, k = p->band_extension;
    int sc = 0, rc = 0, q;
    memset(&ch, 0, sizeof(ch));
    *n_segs = 0;
    *n_traces = 0;
    /* the profile: affine cells when either scheme opens gaps at another cost than it extends
     * them (seeds/banded_chain_alignment_profile.h:235-262) */
    ch.anchor.match = p->anchor.match; ch.anchor.mismatch = p->anchor.mismatch;
    ch.anchor.ext = p->anchor.gap_extend; ch.anchor.open = p->anchor.gap_open;
    ch.gap.match = p->gap.match; ch.gap.mismatch = p->gap.mismatch;
    ch.gap.ext = p->gap.gap_extend; ch.gap.open = p->gap.gap_open;
    ch.st.affine = (ch.anchor.ext != ch.anchor.open) || (ch.gap.ext != ch.gap.open);
    ch.st.fe = p->free_ends;
    ch.h = h; ch.v = v; ch.m = m; ch.n = n; ch.k = k;
    if (N < 1) { *score = INT_MIN; return 0; }
    if (m <= 0 || n <= 0 || k < 1) return ERR_UNDEF;
    sd = (seed_t *)malloc(sizeof(seed_t) * (size_t)N);
    for (i = 0; i < N; ++i) {
        sd[i].bh = seeds[4 * i]; sd[i].bv = seeds[4 * i + 1];
        sd[i].eh = seeds[4 * i + 2]; sd[i].ev = seeds[4 * i + 3];
        sd[i].lo = MIN(sd[i].bh - sd[i].bv, sd[i].eh - sd[i].ev);
        sd[i].up = MAX(sd[i].bh - sd[i].bv, sd[i].eh - sd[i].ev);
    }
    /* _findFirstAnchor / _findLastAnchor */
    it = 0;
    while (it != N - 1) {
        const seed_t *s = &sd[++it];
        if (s->bh - k <= 0) continue;
        if (s->bv - k <= 0) continue;
        --it;
        break;
    }
    itEnd = N - 1;
    while (itEnd != it) {
        const seed_t *s = &sd[--itEnd];
        if (s->eh + k >= m) continue;
        if (s->ev + k >= n) continue;
        break;
    }
    sc = initialize_chain(&ch, &sd[it]);
    if (!ch.st.err && (N == 1 || (it == itEnd && itEnd == N - 1))) {
        if (sd[it].eh + k < m || sd[it].ev + k < n) {
            long gbh = ch.st.hNext, gbv = ch.st.vNext;
            traceset_t local = {NULL, 0, 0};
            reinit(&ch.st, 0, 0, m + 1 - gbh, n + 1 - gbv, m + 1 - gbh, n + 1 - gbv);
            sc = run_grid(&ch.st, &ch.gap, KIND_FINAL, 0, 0, 0, h + gbh, m - gbh, v + gbv, n - gbv, &local);
            glue_local(&ch, &local, gbh, gbv, 0);
        }
    } else if (!ch.st.err) {
        while (it != itEnd && !ch.st.err) {
            ++it;
            gap_area(&ch, &sd[it]);
            anchor_area(&ch, &sd[it]);
        }
        if (!ch.st.err) sc = finish_chain(&ch, &sd[++it]);
    }
    rc = ch.st.err;
    *score = sc;
    *n_traces = ch.global.n;
    if (!rc && ch.global.n > 0) {
        const trace_t *t = &ch.global.t[0];
        if (t->n > seg_cap) rc = -1;
        else {
            for (q = 0; q < t->n; ++q) segs[q] = t->a[q];
            *n_segs = t->n;
        }
    }
    ts_free(&ch.global);
    for (q = 0; q < 4; ++q) free(ch.st.v4[q]);
    free(ch.st.set);
    free(sd);
    return rc;
}
