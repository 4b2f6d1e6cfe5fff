// chain_kernels.cuh -- banded chain alignment (bandedChainAlignment over a seed chain,
// seeds/banded_chain_alignment*.h), one chain per thread.
//
// A chain is a sequence of grids -- the rectangle before the first anchor, then per anchor a band
// around it and the rectangle to the next anchor, then the rectangle to the matrix end -- each a
// DP whose first row and column come from cells the previous grid's traceback picked.  The grids
// of one chain depend on each other; chains are independent, so a batch runs one chain per thread
// with the chain's scratch (trace matrix of the current grid, two score columns, the four init
// vectors, the init-cell set, the positions of the maximum and the trace sets) in its own slice of
// an HBM arena.  The same code runs on the host in plan mode: the grids' geometry depends only on
// the seeds, the band extension and the sequence lengths, so a host pass sizes every chain's
// slice before the kernel runs.
//
// Semantics followed (reference lines):
//   chain driver          seeds/banded_chain_alignment_impl.h:660-722, 748-1330
//   scout state, set      seeds/banded_chain_alignment_scout.h:60-240 (first insert of a key wins:
//                         the cells of one key compare equivalent)
//   grid DP               align/dp_algorithm_impl.h:483-579 (unbanded), :586-967 (banded), with
//                         the chain's first-row / first-column overrides (impl.h:409-705), its
//                         recursion directions (banded_chain_alignment_profile.h:80-160) and
//                         CompleteTrace ties (align/dp_formula.h:205-220)
//   tracking              seeds/banded_chain_alignment_impl.h:260-390; scout >= keeps every
//                         position of the maximum (scout.h:212-240)
//   trace storage / walk  align/dp_matrix_navigator_trace_matrix.h:77-330 (band storage, lane
//                         leaps), align/dp_traceback_impl.h:57-455 (coordinator, GapsLeft walk)
//   chain traceback       seeds/banded_chain_alignment_traceback.h:206-385
//   glue / smooth         seeds/banded_chain_alignment_traceback.h:95-200
// A grid that spans the whole matrix runs the GlobalAlignment_ profile (standard tracking with the
// extra offers at band-phase boundaries, strict > scout, head and tail gaps).
#pragma once

#include <climits>
#include <cstdint>

namespace chain {

constexpr int INF = INT_MIN / 2;   // DPCellDefaultInfinity<DPCell_<int, ..>>

enum : int { T_NONE = 0, T_DIAG = 1, T_H = 2, T_V = 4, T_HO = 8, T_VO = 16, T_MFH = 32, T_MFV = 64 };
enum : int { KIND_INITIAL, KIND_INNER, KIND_FINAL, KIND_GLOBAL };
enum : int { COL_INITIAL, COL_INNER, COL_FINAL };
enum : int { LOC_FULL, LOC_TOP, LOC_MIDDLE, LOC_BOTTOM };
enum : int { CELL_FIRST, CELL_INNER, CELL_LAST };
enum : int { DIR_ZERO, DIR_ALL, DIR_UPPER, DIR_LOWER, DIR_HORIZONTAL, DIR_VERTICAL };
enum : int { FREE_TOP = 1, FREE_LEFT = 2, FREE_RIGHT = 4, FREE_BOTTOM = 8 };

// status per chain (mirrors GBA_CHAIN_* in the C ABI)
enum : int { ST_OK = 0, ST_NO_GLUE = 1, ST_UNDEFINED = 2, ST_CAPACITY = 3 };

struct Cell { int s, e, f; };
struct Seg { uint32_t h, v, len, type; };
struct InitCell { int i1, i2; Cell c; };
struct Scheme { int match, mismatch, ext, open; };

// Sizes of one chain's scratch (plan pass maxima).
struct Plan {
    int64_t trace_bytes;   // largest L * Hlen of its grids
    int32_t col_rows;      // largest n + 1
    int32_t vlen[4];       // largest lengths of the four init vectors
    int32_t set_cap;       // init-cell set entries
    int32_t mp_cap;        // positions of the maximum of one grid
    int32_t gseg_cap;      // segments of one global trace (m + n + 8)
    int32_t lseg_cap;      // segments of one local trace (largest grid m + n + 8)
    int32_t col_cap;       // largest m + 1 (columns of one grid)
    int32_t status;        // ST_UNDEFINED when the geometry leaves the sequences
    int64_t cells;         // DP cells of all grids (in-band cells for a band)
    int64_t trace_total;   // trace bytes of all grids
};

// One column of a grid as the reference's loop visits it: rows r0..r1 (r1 = r0 for a single
// cell), its column type and location, the trace navigator's position at its first cell and the
// lane leap its cells see.
struct ColDesc {
    int r0, r1;
    int64_t pos0;
    int leap;
    int hcol, vrow0;   // storage column and storage row of the first cell (a column never wraps)
    int8_t type, loc, single, present;
};

// One chain's scratch slices (device or host memory) and its inputs.
struct Work {
    uint8_t *T;
    int *cS0, *cS1, *cE0, *cE1;
    Cell *v4[4];
    InitCell *set;
    int *mp;
    Seg *gseg;      // global traces: slot q at gseg + q * gseg_cap, stored reversed (reference's last first)
    int *glen;      // [traces]
    int *gorder;    // [traces] slot ids in set order
    Seg *lseg;      // local traces: slot q at lseg + q * lseg_cap, reference order
    int *llen;      // [traces]
    int *erase;     // [traces]
    // warp-cooperative fill: per-column descriptors, three rolling anti-diagonals of (S, E, F)
    // indexed by column, candidate cells for the maximum (last cell per column, the final column)
    ColDesc *cols;
    int *aS, *aE, *aF;       // [3 * col_cap]
    int *ccS, *ccP, *ccF;    // [col_cap]
    int *fcS, *fcP, *fcF;    // [col_rows]
};


struct ChainDesc {
    int64_t h_off, v_off, seed_off;   // into the batch's codes and seeds (4 int32 per seed)
    int32_t m, n, n_seeds;
    int32_t pad;
    int64_t arena_off;                // byte offset of the chain's scratch
    Plan plan;
};

template <typename T> __host__ __device__ inline T cmin(T a, T b) { return a < b ? a : b; }
template <typename T> __host__ __device__ inline T cmax(T a, T b) { return a > b ? a : b; }

// CompleteTrace _maxScore: a tie keeps the left value and the union of both traces.
__host__ __device__ inline int mxc(int &target, int left, int right, int tl, int tr)
{
    if (left == right) { target = left; return tl | tr; }
    if (left < right) { target = right; return tr; }
    target = left;
    return tl;
}

struct Engine {
    // ---- configuration ----
    bool plan;                  // plan mode: geometry only
    bool warp;                  // one warp per chain: grids filled by anti-diagonals across the lanes
    int lane;                   // this thread's lane (0 on the host)
    Scheme anchor, gap;
    int fe, affine, k;
    int max_traces;
    const uint8_t *h, *v;
    int m, n;
    Work w;
    Plan *pl;                   // plan mode: maxima go here; run mode: capacities
    int err;

    // ---- scout state ----
    int64_t hNext, vNext;
    int n4[4];
    int nset;
    // ---- trace sets ----
    int ng;                     // global traces in order
    uint32_t gused;
    int nl;                     // local traces

    // ---- current grid ----
    const Scheme *sc;
    int kind, banded;
    int gm, gn;                 // grid sizes
    const uint8_t *gh, *gv;
    int lower, upper;
    int64_t L, Hlen, pos, leap;
    int lo0, hi0, lo1, hi1;
    int dS, vS, vF;
    int maxS, nmp;
    // standard scout of a GlobalAlignment_ grid
    int bestS, bestCol, bestRow;
    int64_t bestPos;
    Cell bestCell;

    __host__ __device__ void fail(int code) { if (!err) err = code; }

    // =========================== init-cell set ===========================
    __host__ __device__ bool set_insert(int i1, int i2, Cell c)
    {
        if (plan) return true;
        int lo = 0, hi = nset;
        while (lo < hi) {
            const int mid = (lo + hi) >> 1;
            const InitCell &e = w.set[mid];
            if (e.i1 < i1 || (e.i1 == i1 && e.i2 < i2)) lo = mid + 1;
            else hi = mid;
        }
        if (lo < nset && w.set[lo].i1 == i1 && w.set[lo].i2 == i2) return false;
        if (nset >= pl->set_cap) { fail(ST_CAPACITY); return false; }
        for (int q = nset; q > lo; --q) w.set[q] = w.set[q - 1];
        w.set[lo].i1 = i1;
        w.set[lo].i2 = i2;
        w.set[lo].c = c;
        ++nset;
        return true;
    }

    // _reinitScoutState
    __host__ __device__ void reinit(int64_t oh, int64_t ov, int64_t ch, int64_t cv, int64_t nh, int64_t nv)
    {
        if (err) return;
        const int64_t want[4] = {ch, cv, nh, nv};
        if (oh < 0 || ov < 0 || ch < 0 || cv < 0 || nh < 0 || nv < 0) { fail(ST_UNDEFINED); return; }
        if (ch > (1 << 30) || cv > (1 << 30) || nh > (1 << 30) || nv > (1 << 30)) { fail(ST_UNDEFINED); return; }
        hNext = oh;
        vNext = ov;
        for (int q = 0; q < 4; ++q) {
            if (n4[q] < want[q]) n4[q] = int(want[q]);
            if (plan) {
                if (pl->vlen[q] < n4[q]) pl->vlen[q] = n4[q];
                continue;
            }
#ifdef __CUDA_ARCH__
            if (warp) {
                for (int i = lane; i < n4[q]; i += 32) w.v4[q][i] = Cell{INF, INF, INF};
                continue;
            }
#endif
            for (int i = 0; i < n4[q]; ++i) w.v4[q][i] = Cell{INF, INF, INF};
        }
#ifdef __CUDA_ARCH__
        if (warp) __syncwarp();
#endif
        if (plan) return;
        for (int i = 0; i < nset; ++i) {
            const InitCell &e = w.set[i];
            if (e.i1 == 0) {
                if (e.i2 >= n4[1]) { fail(ST_UNDEFINED); return; }
                w.v4[1][e.i2] = e.c;
            }
            if (e.i2 == 0) {
                if (e.i1 >= n4[0]) { fail(ST_UNDEFINED); return; }
                w.v4[0][e.i1] = e.c;
            }
        }
    }

    // =========================== traces ===========================
    __host__ __device__ Seg *lslot(int q) { return w.lseg + int64_t(q) * pl->lseg_cap; }
    __host__ __device__ Seg *gslot(int q) { return w.gseg + int64_t(q) * pl->gseg_cap; }

    // _recordSegment into local trace q (q < 0: discarded)
    __host__ __device__ void record(int q, int64_t hp, int64_t vp, int64_t len, int tv)
    {
        if (len == 0 || q < 0) return;
        int type;
        if (tv & T_DIAG) type = T_DIAG;
        else if (tv & T_V) type = T_V;
        else if (tv & T_H) type = T_H;
        else return;
        if (w.llen[q] >= pl->lseg_cap) { fail(ST_CAPACITY); return; }
        Seg &s = lslot(q)[w.llen[q]++];
        s.h = uint32_t(hp);
        s.v = uint32_t(vp);
        s.len = uint32_t(len);
        s.type = uint32_t(type);
    }

    __host__ __device__ int new_local()
    {
        if (nl >= max_traces) { fail(ST_CAPACITY); return -1; }
        w.llen[nl] = 0;
        return nl++;
    }

    __host__ __device__ int new_global()
    {
        for (int q = 0; q < max_traces; ++q)
            if (!(gused & (1u << q))) {
                if (ng >= max_traces) break;
                gused |= 1u << q;
                w.glen[q] = 0;
                w.gorder[ng++] = q;
                return q;
            }
        fail(ST_CAPACITY);
        return -1;
    }

    // reversed append of local trace l onto global slot g (prepends it in reference order)
    __host__ __device__ bool g_prepend(int g, const Seg *ls, int ln)
    {
        if (w.glen[g] + ln > pl->gseg_cap) { fail(ST_CAPACITY); return false; }
        Seg *gs = gslot(g);
        for (int i = ln - 1; i >= 0; --i) gs[w.glen[g]++] = ls[i];
        return true;
    }

    static __host__ __device__ int64_t end_h(const Seg &s)
    {
        return (s.type & (T_H | T_DIAG)) ? int64_t(s.h) + s.len : int64_t(s.h);
    }
    static __host__ __device__ int64_t end_v(const Seg &s)
    {
        return (s.type & (T_V | T_DIAG)) ? int64_t(s.v) + s.len : int64_t(s.v);
    }

    // _smoothGluePoint on a reversed global trace whose first old_n entries are the old part
    __host__ __device__ void smooth(int g, int old_n)
    {
        Seg *gs = gslot(g);
        const int n_ = w.glen[g];
        const int io = old_n - 1, in = old_n;   // reversed indices of the old end and the new begin
        if (io < 0 || in >= n_) return;
        if (gs[io].type == gs[in].type) {
            gs[io].len += gs[in].len;
            for (int q = in; q + 1 < n_; ++q) gs[q] = gs[q + 1];
            w.glen[g] = n_ - 1;
        }
    }

    // _adaptLocalTracesToGlobalGrid + _glueTracebacks (check_empty: skip an empty local set)
    __host__ __device__ void glue_local(int64_t gbh, int64_t gbv, bool check_empty)
    {
        if (plan || err) return;
        for (int i = 0; i < nl; ++i) {
            Seg *ls = lslot(i);
            for (int q = 0; q < w.llen[i]; ++q) {
                ls[q].h = uint32_t(int64_t(ls[q].h) + gbh);
                ls[q].v = uint32_t(int64_t(ls[q].v) + gbv);
            }
        }
        if (check_empty && nl == 0) return;
        if (ng == 0) {
            for (int i = 0; i < nl; ++i) {
                const int g = new_global();
                if (g < 0) return;
                g_prepend(g, lslot(i), w.llen[i]);
            }
            nl = 0;
            return;
        }
        const int n0 = ng;
        int old_total = n0, ne = 0;
        bool glued = false;
        for (int j = 0; j < n0; ++j) {
            const int gj = w.gorder[j];
            if (w.glen[gj] == 0) { fail(ST_UNDEFINED); return; }   // the reference reads past an empty trace
            const Seg gend = gslot(gj)[w.glen[gj] - 1];
            const int cur_n = w.glen[gj];
            int added = 0;
            bool connected = false;
            for (int i = 0; i < nl; ++i) {
                const Seg &lb = lslot(i)[w.llen[i] - 1];
                if (end_h(gend) == int64_t(lb.h) && end_v(gend) == int64_t(lb.v)) {
                    if (connected) {
                        const int g = new_global();
                        if (g < 0) return;
                        if (cur_n > pl->gseg_cap) { fail(ST_CAPACITY); return; }
                        for (int q = 0; q < cur_n; ++q) gslot(g)[q] = gslot(gj)[q];
                        w.glen[g] = cur_n;
                        if (!g_prepend(g, lslot(i), w.llen[i])) return;
                        ++added;
                        continue;
                    }
                    if (!g_prepend(gj, lslot(i), w.llen[i])) return;
                    glued = true;
                    connected = true;
                }
            }
            if (!connected) {
                w.erase[ne++] = j;
            } else {
                smooth(gj, cur_n);
                for (int id = old_total; id < old_total + added; ++id) smooth(w.gorder[id], cur_n);
                old_total += added;
            }
        }
        nl = 0;
        if (!glued) { fail(ST_NO_GLUE); return; }
        for (int i = ne; i > 0; --i) {
            const int at = w.erase[i - 1];
            gused &= ~(1u << w.gorder[at]);
            for (int q = at; q + 1 < ng; ++q) w.gorder[q] = w.gorder[q + 1];
            --ng;
        }
    }

    // globalTraceSet = localTraceSet
    __host__ __device__ void assign_global_from_local()
    {
        if (plan || err) return;
        ng = 0;
        gused = 0;
        for (int i = 0; i < nl; ++i) {
            const int g = new_global();
            if (g < 0) return;
            g_prepend(g, lslot(i), w.llen[i]);
        }
        nl = 0;
    }

    // =========================== grid DP ===========================
    __host__ __device__ int sub(int col, int row) const
    {
        return gh[col - 1] == gv[row - 1] ? sc->match : sc->mismatch;
    }
    __host__ __device__ int prev_s(int col, int row) const
    {
        if (col < 1) return INF;
        const bool odd = ((col - 1) & 1) != 0;
        const int lo = odd ? lo1 : lo0, hi = odd ? hi1 : hi0;
        if (row < lo || row > hi) return INF;
        return odd ? w.cS1[row] : w.cS0[row];
    }
    __host__ __device__ int prev_e(int col, int row) const
    {
        if (col < 1) return INF;
        const bool odd = ((col - 1) & 1) != 0;
        const int lo = odd ? lo1 : lo0, hi = odd ? hi1 : hi0;
        if (row < lo || row > hi) return INF;
        return odd ? w.cE1[row] : w.cE0[row];
    }
    __host__ __device__ void new_col(int col)
    {
        if (col & 1) { lo1 = INT_MAX; hi1 = -1; }
        else { lo0 = INT_MAX; hi0 = -1; }
    }

    __host__ __device__ void nav_move(int coltype, int loc, int cellk)
    {
        if (!banded) {
            if (cellk == CELL_FIRST) { if (coltype != COL_INITIAL) pos += leap; }
            else pos += 1;
            return;
        }
        if (cellk == CELL_FIRST) {
            if (coltype == COL_INITIAL) return;
            if (loc == LOC_TOP) { leap -= 1; pos += leap; }
            else pos += leap;
        } else {
            pos += 1;
            if (cellk == CELL_LAST && loc == LOC_BOTTOM && coltype != COL_INITIAL) leap += 1;
        }
    }

    // the chain's tracking options and scout
    __host__ __device__ void track_chain(int coltype, int loc, int cellk, const Cell &cur)
    {
        const int64_t cH = pos / L, cV = pos % L;
        bool storeRow = false, storeCol = false, lastCol = false, lastRow = false;
        const bool finalM = kind == KIND_FINAL;
        if (cH >= hNext) {
            if (loc == LOC_BOTTOM) { if (cV + leap == vNext) storeRow = true; }
            else if (cV == vNext) storeRow = true;
            if (cH == hNext && cV >= vNext) storeCol = true;
            if (cellk == CELL_LAST && (!finalM || (fe & FREE_BOTTOM))) lastRow = true;
            if (coltype == COL_FINAL) {
                if (cellk == CELL_LAST) { lastCol = true; lastRow = true; }
                else if (loc != LOC_FULL || cV >= vNext) {
                    if (!finalM || (fe & FREE_RIGHT)) lastCol = true;
                }
            }
        }
        if (storeCol) {
            const int64_t q = cV - vNext;
            if (q >= n4[3]) { fail(ST_UNDEFINED); return; }
            w.v4[3][q] = cur;
        }
        if (storeRow) {
            const int64_t q = cH - hNext;
            if (q >= n4[2]) { fail(ST_UNDEFINED); return; }
            w.v4[2][q] = cur;
        }
        if ((lastCol || lastRow) && cur.s >= maxS) {
            if (cur.s != maxS) { nmp = 0; maxS = cur.s; }
            if (nmp >= pl->mp_cap) { fail(ST_CAPACITY); return; }
            w.mp[nmp++] = int(pos);
        }
    }

    // the standard tracking of a GlobalAlignment_ grid (DPMetaColumn_ flags) and its scout
    __host__ __device__ void track_global(int coltype, int loc, int cellk, int col, int row, const Cell &cur)
    {
        bool t;
        const bool lastColFree = coltype == COL_FINAL && (fe & FREE_RIGHT);
        if (cellk < CELL_LAST) t = lastColFree;
        else if (loc == LOC_FULL || loc == LOC_BOTTOM) t = coltype == COL_FINAL || (fe & FREE_BOTTOM);
        else t = lastColFree;
        if (t) offer_global(cur, col, row);
    }
    __host__ __device__ void offer_global(const Cell &c, int col, int row)
    {
        if (c.s > bestS) { bestS = c.s; bestCell = c; bestCol = col; bestRow = row; bestPos = pos; }
    }

    // one cell: navigator step, value, trace byte, tracking
    __host__ __device__ void cell(int coltype, int loc, int cellk, int col, int row)
    {
        if (err) return;
        nav_move(coltype, loc, cellk);
        if (pos < 0 || pos >= L * Hlen) { fail(ST_UNDEFINED); return; }
        const int hS = prev_s(col, row), hE = prev_e(col, row);
        Cell cur{INF, INF, INF};
        int tv = T_NONE;
        const bool chainProfile = kind != KIND_GLOBAL;
        int dir;
        if (chainProfile && coltype == COL_INITIAL) {
            const int64_t idx = (pos % L) - (leap - 1);
            if (idx < 0 || idx >= n4[1]) { fail(ST_UNDEFINED); return; }
            dS = hS;
            cur = w.v4[1][idx];
            vS = cur.s;
            vF = cur.f;
            dir = -1;
        } else if (chainProfile && cellk == CELL_FIRST && (loc == LOC_TOP || loc == LOC_FULL)) {
            const int64_t idx = pos / L;
            if (idx >= n4[0]) { fail(ST_UNDEFINED); return; }
            dS = hS;
            cur = w.v4[0][idx];
            vS = cur.s;
            vF = cur.f;
            dir = -1;
        } else if (chainProfile) {
            dir = (cellk == CELL_INNER) ? DIR_ALL
                : (cellk == CELL_FIRST) ? DIR_UPPER
                : (loc == LOC_TOP || loc == LOC_MIDDLE) ? DIR_LOWER : DIR_ALL;
        } else {
            // GlobalAlignment_ meta columns (align/dp_meta_info.h:178-370)
            if (coltype == COL_INITIAL)
                dir = cellk == CELL_FIRST ? DIR_ZERO : ((fe & FREE_LEFT) ? DIR_ZERO : DIR_VERTICAL);
            else if (cellk == CELL_FIRST)
                dir = (loc == LOC_FULL || loc == LOC_TOP) ? ((fe & FREE_TOP) ? DIR_ZERO : DIR_HORIZONTAL) : DIR_UPPER;
            else if (cellk == CELL_INNER)
                dir = DIR_ALL;
            else
                dir = (loc == LOC_TOP || loc == LOC_MIDDLE) ? DIR_LOWER : DIR_ALL;
        }
        if (dir >= 0) tv = compute(dir, col, row, hS, hE, cur, dS, vS, vF);
        const int k1 = col & 1;
        if (k1) { if (row < lo1) lo1 = row; if (row > hi1) hi1 = row; w.cS1[row] = cur.s; w.cE1[row] = cur.e; }
        else { if (row < lo0) lo0 = row; if (row > hi0) hi0 = row; w.cS0[row] = cur.s; w.cE0[row] = cur.e; }
        w.T[pos] = uint8_t(tv);
        if (chainProfile) track_chain(coltype, loc, cellk, cur);
        else track_global(coltype, loc, cellk, col, row, cur);
        lastCell = cur;
    }
    Cell lastCell;

    // the recurrences (align/dp_formula_affine.h, dp_formula_linear.h, dp_formula.h Zero) with
    // CompleteTrace ties; cur.f gets cacheVert's vertical score (_setVerticalScoreOfCell)
    __host__ __device__ int compute(int dir, int col, int row, int hS, int hE, Cell &cur, int &dS, int &vS, int &vF) const
    {
        int tv = T_NONE;
        const int ext = sc->ext, open = sc->open;
        if (dir == DIR_ZERO) {
            cur.s = 0;
            cur.e = INF;   // Zero never writes E: a border cell keeps the default
            dS = 0;
            vS = 0;
            cur.f = vF;
            if (!affine) { cur.e = INF; cur.f = INF; }
            return T_NONE;
        }
        if (affine) {
            switch (dir) {
            case DIR_ALL: {
                const int inter = dS + sub(col, row);
                int s, t2;
                dS = hS;
                tv = mxc(cur.e, hE + ext, hS + open, T_H, T_HO);
                tv |= mxc(vF, vF + ext, vS + open, T_V, T_VO);
                t2 = mxc(s, vF, cur.e, T_MFV, T_MFH);
                tv = mxc(cur.s, inter, s, T_DIAG | tv, t2 | tv);
                vS = cur.s;
                break;
            }
            case DIR_UPPER: {
                const int inter = dS + sub(col, row);
                dS = hS;
                tv = mxc(cur.e, hE + ext, hS + open, T_H, T_HO);
                vF = INF;
                tv = mxc(cur.s, inter, cur.e, tv | T_DIAG, tv | T_MFH);
                vS = cur.s;
                break;
            }
            case DIR_LOWER:
                tv = mxc(vF, vF + ext, vS + open, T_V, T_VO);
                cur.e = INF;
                tv = mxc(cur.s, dS + sub(col, row), vF, tv | T_DIAG, tv | T_MFV);
                break;
            case DIR_HORIZONTAL:
                dS = hS;
                tv = mxc(cur.e, hE + ext, hS + open, T_H, T_HO) | T_MFH;
                vF = INF;
                cur.s = cur.e;
                vS = cur.s;
                break;
            default:   // DIR_VERTICAL
                tv = mxc(vF, vF + ext, vS + open, T_V, T_VO) | T_MFV;
                cur.e = INF;
                cur.s = vF;
                vS = cur.s;
                break;
            }
            cur.f = vF;
        } else {
            switch (dir) {
            case DIR_ALL: {
                const int inter = dS + sub(col, row);
                int s;
                dS = hS;
                tv = mxc(s, vS + ext, hS + ext, T_V | T_MFV, T_H | T_MFH);
                tv = mxc(cur.s, inter, s, T_DIAG, tv);
                vS = cur.s;
                break;
            }
            case DIR_UPPER: {
                const int inter = dS + sub(col, row);
                dS = hS;
                tv = mxc(cur.s, inter, hS + ext, T_DIAG, T_H | T_MFH);
                vS = cur.s;
                break;
            }
            case DIR_LOWER:
                tv = mxc(cur.s, dS + sub(col, row), vS + ext, T_DIAG, T_V | T_MFV);
                break;
            case DIR_HORIZONTAL:
                dS = hS;
                cur.s = hS + ext;
                tv = T_H | T_MFH;
                vS = cur.s;
                break;
            default:
                cur.s = vS + ext;
                tv = T_V | T_MFV;
                vS = cur.s;
                break;
            }
            cur.e = INF;
            cur.f = INF;
        }
        return tv;
    }

    __host__ __device__ void track_col(int col, int coltype, int loc, int r0, int r1)
    {
        new_col(col);
        dS = INF; vS = INF; vF = INF;
        if (coltype != COL_INITIAL && (loc == LOC_MIDDLE || loc == LOC_BOTTOM) && r0 > 0 && col > 0)
            dS = prev_s(col, r0 - 1);
        cell(coltype, loc, CELL_FIRST, col, r0);
        for (int i = r0 + 1; i < r1 && !err; ++i) cell(coltype, loc, CELL_INNER, col, i);
        cell(coltype, loc, CELL_LAST, col, r1);
    }

    // an extra scout offer of the last computed cell (GlobalAlignment_ grids only; the chain's
    // scout ignores these calls), optionally with cacheVert's F stored first
    __host__ __device__ void retrack(int col, int row, bool set_f)
    {
        if (kind != KIND_GLOBAL || err) return;
        Cell c = lastCell;
        if (set_f) c.f = vF;
        (void)set_f;
        offer_global(c, col, row);
    }

    __host__ __device__ void run_unbanded()
    {
        track_col(0, COL_INITIAL, LOC_FULL, 0, gn);
        for (int col = 1; col < gm && !err; ++col) track_col(col, COL_INNER, LOC_FULL, 0, gn);
        if (!err) track_col(gm, COL_FINAL, LOC_FULL, 0, gn);
    }

    __host__ __device__ void single_init(int col, int coltype, int loc, int row)
    {
        new_col(col);
        dS = INF; vS = INF; vF = INF;
        cell(coltype, loc, CELL_FIRST, col, row);
    }

    __host__ __device__ void run_banded()
    {
        const int mm = gm, nn = gn, lw = lower, up = upper;
        const bool glob = kind == KIND_GLOBAL;
        int vb = -cmin(0, 1 + up), ve = -cmin(0, cmax(-nn, lw));
        const int hb = cmax(0, cmin(mm - 1, lw));
        int hTop = cmin(mm - 1, cmax(0, up)), hMid = cmin(mm - 1, cmax(0, nn + lw));
        if (up > nn + lw) { const int t = hTop; hTop = hMid; hMid = t; }
        const int hBot = cmax(0, cmin(mm, up + nn) - 1);
        if (hb == mm - 1) {
            const int col = cmax(0, cmin(mm, lw));
            single_init(col, COL_INITIAL, LOC_TOP, 0);
            if (glob && (fe & FREE_RIGHT)) retrack(col, 0, false);
            return;
        }
        if (hBot == 0) {
            const int row = cmin(nn, -up);
            single_init(0, COL_INITIAL, LOC_BOTTOM, row);
            if (glob && (fe & FREE_BOTTOM)) retrack(0, row, false);
            return;
        }
        if (up < 0) {
            ++vb;
            track_col(0, COL_INITIAL, lw > -nn ? LOC_MIDDLE : LOC_BOTTOM, vb, ve);
        } else if (lw >= 0) {
            single_init(hb, COL_INITIAL, LOC_TOP, 0);
        } else {
            track_col(0, COL_INITIAL, lw <= -nn ? LOC_FULL : LOC_TOP, vb, ve);
        }
        int hIt = hb;
        for (; hIt != hTop && !err; ++hIt) {
            ++ve;
            track_col(hIt + 1, COL_INNER, LOC_TOP, vb, ve);
        }
        if (up > nn + lw) {
            if (glob && (fe & FREE_BOTTOM)) retrack(hIt, ve, false);
            for (; hIt != hMid && !err; ++hIt) track_col(hIt + 1, COL_INNER, LOC_FULL, vb, ve);
        } else {
            for (; hIt != hMid && !err; ++hIt) {
                ++vb; ++ve;
                track_col(hIt + 1, COL_INNER, LOC_MIDDLE, vb, ve);
            }
            if (glob && (fe & FREE_BOTTOM) && lw + nn < mm) retrack(hIt, ve, false);
        }
        for (; hIt != hBot && !err; ++hIt) {
            ++vb;
            track_col(hIt + 1, COL_INNER, LOC_BOTTOM, vb, ve);
        }
        if (err) return;
        if (hIt < mm - 1) {
            new_col(hIt + 1);
            dS = prev_s(hIt + 1, vb); vS = INF; vF = INF;
            cell(COL_INNER, LOC_BOTTOM, CELL_FIRST, hIt + 1, vb + 1);
            if (glob && (fe & FREE_BOTTOM)) retrack(hIt + 1, vb + 1, true);
        } else if (hIt == mm - 1) {
            if (up == mm - nn) {
                new_col(mm);
                dS = prev_s(mm, vb); vS = INF; vF = INF;
                cell(COL_FINAL, LOC_BOTTOM, CELL_FIRST, mm, vb + 1);
                if (glob) retrack(mm, vb + 1, true);
            } else if (up >= mm) {
                if (lw + nn > mm) { ++ve; track_col(mm, COL_FINAL, LOC_TOP, vb, ve); }
                else if (lw + nn + 1 > mm) {
                    ++ve;
                    track_col(mm, COL_FINAL, LOC_TOP, vb, ve);
                    if (glob) retrack(mm, ve, true);
                } else track_col(mm, COL_FINAL, LOC_FULL, vb, ve);
            } else {
                ++vb;
                if (lw + nn <= mm) {
                    if (lw + nn == mm) {
                        ++ve;
                        track_col(mm, COL_FINAL, LOC_MIDDLE, vb, ve);
                        if (glob) retrack(mm, ve, true);
                    } else track_col(mm, COL_FINAL, LOC_BOTTOM, vb, ve);
                } else {
                    ++ve;
                    track_col(mm, COL_FINAL, LOC_MIDDLE, vb, ve);
                }
            }
        }
    }

    // ---------------- traceback over the band storage ----------------
    struct Walk {
        int64_t pos, cc, cr, ec, er, bp1, bp2;
        int tv, last;
        int64_t frag;
        bool band, bad;
    };

    __host__ __device__ void coord_init(Walk &wk, int64_t cc, int64_t cr, int64_t ec, int64_t er) const
    {
        wk.cc = cc; wk.cr = cr; wk.ec = ec; wk.er = er; wk.bp1 = 0; wk.bp2 = 0; wk.band = false;
        if (banded) {
            if (lower >= 0) wk.cc += lower;
            if (wk.cc > upper) wk.cr += wk.cc - upper;
            if (wk.ec > upper) wk.er += wk.ec - upper;
            wk.bp1 = cmin<int64_t>(gm, cmax<int64_t>(0, upper));
            wk.bp2 = cmin<int64_t>(gm, cmax<int64_t>(0, int64_t(gn) + lower));
            const int64_t b = cmin(wk.bp1, wk.bp2);
            if (wk.cc < b) wk.cr -= b - wk.cc;
            wk.band = true;
        }
    }
    static __host__ __device__ bool reached_end(const Walk &wk) { return wk.cc <= wk.ec || wk.cr <= wk.er; }
    static __host__ __device__ bool in_band(const Walk &wk) { return wk.band && (wk.cc > wk.bp1 || wk.cc <= wk.bp2); }

    static __host__ __device__ int initial_dir(int &tv, bool prefer)
    {
        if (prefer) {
            if (tv & T_MFV) { tv &= (T_V | T_VO | T_MFV); return T_V; }
            if (tv & T_MFH) { tv &= (T_H | T_HO | T_MFH); return T_H; }
            return T_DIAG;
        }
        if (tv & T_DIAG) return T_DIAG;
        if (tv & (T_V | T_MFV)) return T_V;
        if (tv & (T_H | T_MFH)) return T_H;
        return T_NONE;
    }

    __host__ __device__ void w_step(Walk &wk, int64_t d) const
    {
        if (d <= 0) { wk.bad = true; wk.tv = T_NONE; return; }   // a one-row band: the walk would not move
        wk.pos -= d;
        if (wk.pos < 0 || wk.pos >= L * Hlen) { wk.bad = true; wk.tv = T_NONE; return; }
        wk.tv = w.T[wk.pos];
    }
    __host__ __device__ void w_switch(Walk &wk, int q, int bit)
    {
        if (!(wk.last & bit)) {
            record(q, wk.cc, wk.cr, wk.frag, wk.last);
            wk.last = bit;
            wk.frag = 0;
        }
    }
    // _doTraceback with GapsLeft
    __host__ __device__ void do_trace(Walk &wk, int q)
    {
        const int tv = wk.tv;
        if (tv & T_DIAG) {
            w_switch(wk, q, T_DIAG);
            w_step(wk, in_band(wk) ? L : L + 1);
            --wk.cc; --wk.cr; ++wk.frag;
        } else if ((tv & T_MFV) && (tv & T_V)) {
            w_switch(wk, q, T_V);
            if (affine)
                while ((!(wk.tv & T_VO) || (wk.tv & T_V)) && wk.cr != 1 && !wk.bad) {
                    w_step(wk, 1);
                    --wk.cr; ++wk.frag;
                }
            w_step(wk, 1);
            --wk.cr; ++wk.frag;
        } else if ((tv & T_MFV) && (tv & T_VO)) {
            w_switch(wk, q, T_V);
            w_step(wk, 1);
            --wk.cr; ++wk.frag;
        } else if ((tv & T_MFH) && (tv & T_H)) {
            w_switch(wk, q, T_H);
            if (affine)
                while ((!(wk.tv & T_HO) || (wk.tv & T_H)) && wk.cc != 1 && !wk.bad) {
                    w_step(wk, in_band(wk) ? L - 1 : L);
                    --wk.cc; ++wk.frag;
                }
            w_step(wk, in_band(wk) ? L - 1 : L);
            --wk.cc; ++wk.frag;
        } else if ((tv & T_MFH) && (tv & T_HO)) {
            w_switch(wk, q, T_H);
            w_step(wk, in_band(wk) ? L - 1 : L);
            --wk.cc; ++wk.frag;
        } else {
            wk.bad = true;   // a trace value the reference asserts on: its walk never ends
            wk.tv = T_NONE;
        }
    }

    __host__ __device__ bool prefer_end() const
    {
        return affine && (kind == KIND_FINAL || kind == KIND_GLOBAL);
    }

    // the generic _computeTraceback from position *p (no head / tail for the chain profile)
    __host__ __device__ void generic_trace(int q, int64_t &p)
    {
        Walk wk;
        wk.pos = p; wk.bad = false; wk.frag = 0;
        wk.tv = w.T[p];
        wk.last = initial_dir(wk.tv, prefer_end());
        coord_init(wk, p / L, p % L, 0, 0);
        while (!reached_end(wk) && wk.tv != T_NONE && !wk.bad && !err) do_trace(wk, q);
        record(q, wk.cc, wk.cr, wk.frag, wk.last);
        p = wk.pos;
        if (wk.bad) fail(ST_UNDEFINED);
    }

    __host__ __device__ static void correct_cell(Cell &c, int last, bool aff)
    {
        if (!aff) return;
        if (last & T_DIAG) { c.f = INF; c.e = INF; }
        else if (last & T_V) c.e = INF;
        else c.f = INF;
    }

    // the chain's traceback from one position of the maximum
    __host__ __device__ void chain_trace_one(int64_t maxpos)
    {
        const int q = new_local();
        if (q < 0) return;
        Walk wk;
        wk.pos = maxpos; wk.bad = false; wk.frag = 0;
        wk.tv = w.T[maxpos];
        wk.last = initial_dir(wk.tv, prefer_end());
        coord_init(wk, maxpos / L, maxpos % L, hNext, vNext);
        if (kind == KIND_FINAL) {
            int64_t p = maxpos;
            if (wk.cr != gn) record(q, gm, wk.cr, gn - wk.cr, T_V);
            if (wk.cc != gm) record(q, wk.cc, wk.cr, gm - wk.cc, T_H);
            generic_trace(q, p);
            if (w.llen[q] == 0) --nl;
            return;
        }
        while (!reached_end(wk) && wk.tv != T_NONE && !wk.bad) do_trace(wk, -1);
        if (wk.bad) { fail(ST_UNDEFINED); return; }
        const int64_t hip = wk.cc - wk.ec, vip = wk.cr - wk.er;
        bool ins;
        if (vip <= 0) {
            if (hip < 0 || hip >= n4[2]) { fail(ST_UNDEFINED); return; }
            correct_cell(w.v4[2][hip], wk.last, affine);
            ins = set_insert(int(hip), 0, w.v4[2][hip]);
        } else {
            if (vip >= n4[3]) { fail(ST_UNDEFINED); return; }
            correct_cell(w.v4[3][vip], wk.last, affine);
            ins = set_insert(0, int(vip), w.v4[3][vip]);
        }
        if (err) return;
        if (ins) {
            if (vip < 0) record(q, wk.cc, wk.cr, -vip, wk.last);
            else if (hip < 0) record(q, wk.cc, wk.cr, -hip, wk.last);
            generic_trace(q, wk.pos);
        }
        if (kind == KIND_INITIAL) {
            const int64_t cc = wk.pos / L;
            int64_t cr = wk.pos % L;
            if (banded && upper > 0 && cc < wk.bp1 && cc < wk.bp2) cr -= L - 1 + lower - cc;
            if (cr != 0) record(q, 0, 0, cr, T_V);
            if (cc != 0) record(q, 0, 0, cc, T_H);
        }
        if (w.llen[q] == 0) --nl;
    }

    // the standard traceback of a GlobalAlignment_ grid (head and tail, no start-cell correction)
    __host__ __device__ void global_trace()
    {
        const int q = new_local();
        if (q < 0) return;
        Walk wk;
        wk.pos = bestPos; wk.bad = false; wk.frag = 0;
        wk.tv = w.T[bestPos];
        wk.last = initial_dir(wk.tv, prefer_end());
        coord_init(wk, bestPos / L, bestPos % L, 0, 0);
        if (wk.cr != gn) record(q, gm, wk.cr, gn - wk.cr, T_V);
        if (wk.cc != gm) record(q, wk.cc, wk.cr, gm - wk.cc, T_H);
        while (!reached_end(wk) && wk.tv != T_NONE && !wk.bad && !err) do_trace(wk, q);
        record(q, wk.cc, wk.cr, wk.frag, wk.last);
        if (wk.cr != 0) record(q, 0, 0, wk.cr, T_V);
        if (wk.cc != 0) record(q, 0, 0, wk.cc, T_H);
        if (wk.bad) fail(ST_UNDEFINED);
    }

    // _computeAlignment of one grid; local traces go to the local set (appended)
    __host__ __device__ int run_grid(const Scheme *s, int kd, bool bd, int lw, int up, const uint8_t *ph, int64_t pm,
                                     const uint8_t *pv, int64_t pn)
    {
        if (err) return INT_MIN;
        if (pm <= 0 || pn <= 0) return INT_MIN;
        if (pm > (1 << 28) || pn > (1 << 28)) { fail(ST_UNDEFINED); return INT_MIN; }
        if (bd) {
            if (up < -pn || lw > pm) return INT_MIN;
            if (up < 0 && !(fe & FREE_LEFT)) return INT_MIN;
            if (lw > 0 && !(fe & FREE_TOP)) return INT_MIN;
            if (up + pn < pm && !(fe & FREE_BOTTOM)) return INT_MIN;
            if (lw + pn > pm && !(fe & FREE_RIGHT)) return INT_MIN;
            if (up == lw) { fail(ST_UNDEFINED); return INT_MIN; }
        }
        sc = s; kind = kd; banded = bd; lower = lw; upper = up;
        gh = ph; gv = pv; gm = int(pm); gn = int(pn);
        if (bd) {
            const int64_t bs = cmin<int64_t>(pm, up) - cmax<int64_t>(lw, -pn) + 1;
            L = cmin<int64_t>(pn + 1, bs);
            Hlen = pm + 1 - cmax(0, lw);
            if (lw >= 0) { leap = cmin<int64_t>(L, int64_t(up) - lw + 1); pos = L - 1; }
            else if (up <= 0) { leap = 1; pos = 0; }
            else { const int64_t lp = cmax<int64_t>(-(L - 1), lw); leap = L + lp; pos = leap - 1; }
        } else {
            L = pn + 1;
            Hlen = pm + 1;
            leap = 1;
            pos = 0;
        }
        if (L * Hlen >= (int64_t(1) << 31)) { fail(ST_CAPACITY); return INT_MIN; }   // positions are 32-bit
        if (plan) {
            if (bd) {
                for (int64_t j = 0; j <= pm; ++j) {
                    const int64_t r0 = cmax<int64_t>(0, j - up), r1 = cmin<int64_t>(pn, j - lw);
                    if (r1 >= r0) pl->cells += r1 - r0 + 1;
                }
            } else {
                pl->cells += (pm + 1) * (pn + 1);
            }
            pl->trace_total += L * Hlen;
            if (pl->trace_bytes < L * Hlen) pl->trace_bytes = L * Hlen;
            if (pl->col_rows < pn + 1) pl->col_rows = int32_t(pn + 1);
            const int64_t mpb = pm + L + 4;
            if (pl->mp_cap < mpb) pl->mp_cap = int32_t(mpb);
            if (pl->lseg_cap < pm + pn + 8) pl->lseg_cap = int32_t(pm + pn + 8);
            if (pl->col_cap < pm + 1) pl->col_cap = int32_t(pm + 1);
            return 0;
        }
        if (L * Hlen > pl->trace_bytes || pn + 1 > pl->col_rows) { fail(ST_CAPACITY); return INT_MIN; }
        if (!warp || kd == KIND_GLOBAL) {
            for (int64_t q = 0; q < L * Hlen; ++q) w.T[q] = 0;
        }
        lo0 = lo1 = INT_MAX;
        hi0 = hi1 = -1;
        maxS = INF;
        nmp = 0;
        bestS = INF;
        bestPos = 0;
        bestCol = bestRow = 0;
        if (warp && kd != KIND_GLOBAL) fill_warp();
        else if (bd) run_banded();
        else run_unbanded();
        if (err) return INT_MIN;
        if (kd == KIND_GLOBAL) {
            global_trace();
            return bestS;
        }
        nset = 0;
        for (int i = 0; i < nmp && !err; ++i) chain_trace_one(w.mp[i]);
        return maxS;
    }

    // ---------------- warp-cooperative fill ----------------
    // The cells of one anti-diagonal (c + r = d) depend only on the two before it, so the lanes of a
    // warp take the cells of a diagonal together.  Every cell gets the inputs the column-major loop
    // gives it -- the horizontal and diagonal neighbours from the previous column's computed rows,
    // the cell above as cacheVert (none for a column's first cell), the diagonal preset of middle /
    // bottom columns -- so values, trace bytes and init-vector stores are the loop's.  The candidates
    // for the maximum are kept per column and scanned afterwards in column-major order, which gives
    // the scout's list of positions in the loop's order.

    static __host__ __device__ int64_t floor2(int64_t a) { return a >= 0 ? a / 2 : -((-a + 1) / 2); }

    __host__ __device__ void desc_col(int col, int coltype, int loc, int r0, int r1, bool single, int64_t &p,
                                      int64_t &lp)
    {
        if (col < 0 || col > gm || col >= pl->col_cap) { fail(ST_UNDEFINED); return; }
        if (!single && r1 <= r0) { fail(ST_UNDEFINED); return; }   // the reference's track needs two cells
        if (coltype != COL_INITIAL) {
            if (banded && loc == LOC_TOP) { lp -= 1; p += lp; }
            else p += lp;
        }
        ColDesc &d = w.cols[col];
        d.r0 = r0;
        d.r1 = single ? r0 : r1;
        d.pos0 = p;
        d.leap = int(lp);
        d.hcol = int(p / L);
        d.vrow0 = int(p % L);
        if (!single && d.vrow0 + (r1 - r0) >= L) { fail(ST_UNDEFINED); return; }
        d.type = int8_t(coltype);
        d.loc = int8_t(loc);
        d.single = single;
        d.present = 1;
        if (!single) {
            p += r1 - r0;
            if (banded && loc == LOC_BOTTOM && coltype != COL_INITIAL) lp += 1;
        }
    }

    // the columns of run_banded / run_unbanded, with the navigator's positions
    __host__ __device__ void describe(int &cfirst, int &clast)
    {
        int64_t p = pos, lp = leap;
        cfirst = 0;
        clast = gm;
        if (!banded) {
            desc_col(0, COL_INITIAL, LOC_FULL, 0, gn, false, p, lp);
            for (int c = 1; c < gm; ++c) desc_col(c, COL_INNER, LOC_FULL, 0, gn, false, p, lp);
            desc_col(gm, COL_FINAL, LOC_FULL, 0, gn, false, p, lp);
            return;
        }
        const int mm = gm, nn = gn, lw = lower, up = upper;
        int vb = -cmin(0, 1 + up), ve = -cmin(0, cmax(-nn, lw));
        const int hb = cmax(0, cmin(mm - 1, lw));
        int hTop = cmin(mm - 1, cmax(0, up)), hMid = cmin(mm - 1, cmax(0, nn + lw));
        if (up > nn + lw) { const int t = hTop; hTop = hMid; hMid = t; }
        const int hBot = cmax(0, cmin(mm, up + nn) - 1);
        if (hb == mm - 1) {
            const int col = cmax(0, cmin(mm, lw));
            cfirst = clast = col;
            desc_col(col, COL_INITIAL, LOC_TOP, 0, 0, true, p, lp);
            return;
        }
        if (hBot == 0) {
            const int row = cmin(nn, -up);
            cfirst = clast = 0;
            desc_col(0, COL_INITIAL, LOC_BOTTOM, row, row, true, p, lp);
            return;
        }
        if (up < 0) {
            ++vb;
            desc_col(0, COL_INITIAL, lw > -nn ? LOC_MIDDLE : LOC_BOTTOM, vb, ve, false, p, lp);
        } else if (lw >= 0) {
            cfirst = hb;
            desc_col(hb, COL_INITIAL, LOC_TOP, 0, 0, true, p, lp);
        } else {
            desc_col(0, COL_INITIAL, lw <= -nn ? LOC_FULL : LOC_TOP, vb, ve, false, p, lp);
        }
        int hIt = hb;
        for (; hIt != hTop && !err; ++hIt) { ++ve; desc_col(hIt + 1, COL_INNER, LOC_TOP, vb, ve, false, p, lp); }
        if (up > nn + lw) {
            for (; hIt != hMid && !err; ++hIt) desc_col(hIt + 1, COL_INNER, LOC_FULL, vb, ve, false, p, lp);
        } else {
            for (; hIt != hMid && !err; ++hIt) {
                ++vb; ++ve;
                desc_col(hIt + 1, COL_INNER, LOC_MIDDLE, vb, ve, false, p, lp);
            }
        }
        for (; hIt != hBot && !err; ++hIt) { ++vb; desc_col(hIt + 1, COL_INNER, LOC_BOTTOM, vb, ve, false, p, lp); }
        clast = hIt;
        if (hIt < mm - 1) {
            clast = hIt + 1;
            desc_col(hIt + 1, COL_INNER, LOC_BOTTOM, vb + 1, vb + 1, true, p, lp);
        } else if (hIt == mm - 1) {
            clast = mm;
            if (up == mm - nn) desc_col(mm, COL_FINAL, LOC_BOTTOM, vb + 1, vb + 1, true, p, lp);
            else if (up >= mm) {
                if (lw + nn > mm) { ++ve; desc_col(mm, COL_FINAL, LOC_TOP, vb, ve, false, p, lp); }
                else if (lw + nn + 1 > mm) { ++ve; desc_col(mm, COL_FINAL, LOC_TOP, vb, ve, false, p, lp); }
                else desc_col(mm, COL_FINAL, LOC_FULL, vb, ve, false, p, lp);
            } else {
                ++vb;
                if (lw + nn <= mm) {
                    if (lw + nn == mm) { ++ve; desc_col(mm, COL_FINAL, LOC_MIDDLE, vb, ve, false, p, lp); }
                    else desc_col(mm, COL_FINAL, LOC_BOTTOM, vb, ve, false, p, lp);
                } else {
                    ++ve;
                    desc_col(mm, COL_FINAL, LOC_MIDDLE, vb, ve, false, p, lp);
                }
            }
        }
    }

    // the cells of anti-diagonal d that lane l takes; k3 / k1 / k2: the rolling slots of d, d - 1, d - 2
    __host__ __device__ void fill_diag(int d, int l, int cfirst, int clast, int k3, int k1, int k2)
    {
        const int cap = pl->col_cap, gnn = gn;
        const int hN = int(hNext), vN = int(vNext);
        const bool finalM = kind == KIND_FINAL;
        const bool freeB = (fe & FREE_BOTTOM) != 0, freeR = (fe & FREE_RIGHT) != 0;
        const ColDesc *cols = w.cols;
        int *aS = w.aS, *aE = w.aE, *aF = w.aF;
        int clo = cmax(cfirst, d - gnn), chi = cmin(clast, d);
        if (banded) {
            clo = cmax(clo, int(-floor2(-(int64_t(d) + lower))));
            chi = cmin(chi, int(floor2(int64_t(d) + upper)));
        }
        for (int c = clo + l; c <= chi; c += 32) {
            const int r = d - c;
            const ColDesc cd = cols[c];
            if (!cd.present || r < cd.r0 || r > cd.r1) continue;
            const int cellk = (r == cd.r0) ? CELL_FIRST : (r == cd.r1 ? CELL_LAST : CELL_INNER);
            const int dr = r - cd.r0;
            const int p = int(cd.pos0) + dr;
            const int lp = cd.leap + ((cellk == CELL_LAST && cd.loc == LOC_BOTTOM && cd.type != COL_INITIAL) ? 1 : 0);
            // the previous column's computed rows
            bool hv = false, dv = false;
            if (c > cfirst) {
                const ColDesc &pc = cols[c - 1];
                hv = pc.present && r >= pc.r0 && r <= pc.r1;
                dv = pc.present && r - 1 >= pc.r0 && r - 1 <= pc.r1;
            }
            const int hS = hv ? aS[k1 * cap + c - 1] : INF, hE = hv ? aE[k1 * cap + c - 1] : INF;
            int kdS = INF, kvS = INF, kvF = INF;
            if (cellk != CELL_FIRST) {
                kvS = aS[k1 * cap + c];
                kvF = aF[k1 * cap + c];
                if (dv) kdS = aS[k2 * cap + c - 1];
            } else if (cd.type != COL_INITIAL && (cd.loc == LOC_MIDDLE || cd.loc == LOC_BOTTOM) && r > 0 && dv) {
                kdS = aS[k2 * cap + c - 1];
            }
            Cell cur{INF, INF, INF};
            int tv = T_NONE;
            const int cV = cd.vrow0 + dr, cH = cd.hcol;
            if (cd.type == COL_INITIAL) {
                const int idx = cV - (lp - 1);
                if (idx < 0 || idx >= n4[1]) { fail(ST_UNDEFINED); continue; }
                cur = w.v4[1][idx];
            } else if (cellk == CELL_FIRST && (cd.loc == LOC_TOP || cd.loc == LOC_FULL)) {
                if (cH >= n4[0]) { fail(ST_UNDEFINED); continue; }
                cur = w.v4[0][cH];
            } else {
                const int dir = (cellk == CELL_INNER) ? DIR_ALL
                              : (cellk == CELL_FIRST) ? DIR_UPPER
                              : (cd.loc == LOC_TOP || cd.loc == LOC_MIDDLE) ? DIR_LOWER : DIR_ALL;
                tv = compute(dir, c, r, hS, hE, cur, kdS, kvS, kvF);
            }
            aS[k3 * cap + c] = cur.s;
            aE[k3 * cap + c] = cur.e;
            aF[k3 * cap + c] = cur.f;
            w.T[p] = uint8_t(tv);
            if (cH < hN) continue;
            // the chain's tracking options
            bool storeRow, lastCol = false, lastRow = false;
            if (cd.loc == LOC_BOTTOM) storeRow = cV + lp == vN;
            else storeRow = cV == vN;
            const bool storeCol = cH == hN && cV >= vN;
            if (cellk == CELL_LAST && (!finalM || freeB)) lastRow = true;
            if (cd.type == COL_FINAL) {
                if (cellk == CELL_LAST) { lastCol = true; lastRow = true; }
                else if ((cd.loc != LOC_FULL || cV >= vN) && (!finalM || freeR)) lastCol = true;
            }
            if (storeCol) {
                const int q = cV - vN;
                if (q >= n4[3]) { fail(ST_UNDEFINED); continue; }
                w.v4[3][q] = cur;
            }
            if (storeRow) {
                const int q = cH - hN;
                if (q >= n4[2]) { fail(ST_UNDEFINED); continue; }
                w.v4[2][q] = cur;
            }
            if (lastCol || lastRow) {
                if (cd.type == COL_FINAL) {
                    w.fcS[r] = cur.s;
                    w.fcP[r] = p;
                    w.fcF[r] = 1;
                } else {
                    w.ccS[c] = cur.s;
                    w.ccP[c] = p;
                    w.ccF[c] = 1;
                }
            }
        }
    }

    __host__ __device__ void offer_chain(int s_, int p_)
    {
        if (s_ >= maxS) {
            if (s_ != maxS) { nmp = 0; maxS = s_; }
            if (nmp >= pl->mp_cap) { fail(ST_CAPACITY); return; }
            w.mp[nmp++] = p_;
        }
    }

    __host__ __device__ void fill_warp()
    {
        if (gm + 1 > pl->col_cap || gn + 1 > pl->col_rows) { fail(ST_CAPACITY); return; }
        const int64_t cells = L * Hlen;
#ifdef __CUDA_ARCH__
        for (int64_t q = lane; q < cells; q += 32) w.T[q] = 0;
        for (int c = lane; c <= gm; c += 32) { w.cols[c].present = 0; w.ccF[c] = 0; }
        for (int r = lane; r <= gn; r += 32) w.fcF[r] = 0;
        __syncwarp();
#else
        for (int64_t q = 0; q < cells; ++q) w.T[q] = 0;
        for (int c = 0; c <= gm; ++c) { w.cols[c].present = 0; w.ccF[c] = 0; }
        for (int r = 0; r <= gn; ++r) w.fcF[r] = 0;
#endif
        int cfirst = 0, clast = 0;
        describe(cfirst, clast);   // every lane writes the same descriptors
#ifdef __CUDA_ARCH__
        __syncwarp();
#endif
        if (err) return;
        int64_t dmin = INT64_MAX, dmax = -1;
        for (int c = cfirst; c <= clast; ++c) {
            const ColDesc &cd = w.cols[c];
            if (!cd.present) continue;
            dmin = cmin<int64_t>(dmin, int64_t(c) + cd.r0);
            dmax = cmax<int64_t>(dmax, int64_t(c) + cd.r1);
        }
        int k3 = int(dmin % 3), k1 = (k3 + 2) % 3, k2 = (k3 + 1) % 3;
        for (int d = int(dmin); d <= int(dmax); ++d) {
#ifdef __CUDA_ARCH__
            fill_diag(d, lane, cfirst, clast, k3, k1, k2);
            __syncwarp();
#else
            for (int l = 0; l < 32; ++l) fill_diag(d, l, cfirst, clast, k3, k1, k2);
#endif
            const int t = k2;   // d + 1: its d - 1 is this d, its d - 2 this d - 1
            k2 = k1;
            k1 = k3;
            k3 = t;
        }
#ifdef __CUDA_ARCH__
        err = __reduce_max_sync(0xffffffffu, err);
#endif
        if (err) return;
        // the scout's positions of the maximum, in the loop's order
        for (int c = cfirst; c <= clast && !err; ++c) {
            const ColDesc &cd = w.cols[c];
            if (!cd.present) continue;
            if (cd.type == COL_FINAL) {
                for (int r = cd.r0; r <= cd.r1; ++r)
                    if (w.fcF[r]) offer_chain(w.fcS[r], w.fcP[r]);
            } else if (w.ccF[c]) {
                offer_chain(w.ccS[c], w.ccP[c]);
            }
        }
    }

    // ---------------- the chain driver ----------------
    struct Seed { int64_t bh, bv, eh, ev, lo, up; };

    __host__ __device__ static int64_t hsb(const Seed &s) { return s.up - (s.bh - s.bv); }
    __host__ __device__ static int64_t vsb(const Seed &s) { return (s.bh - s.bv) - s.lo; }
    __host__ __device__ static int64_t hse(const Seed &s) { return s.eh - s.ev - s.lo; }
    __host__ __device__ static int64_t vse(const Seed &s) { return s.up - s.eh + s.ev; }

    __host__ __device__ void init_beginning(int64_t sizeH, int64_t sizeV, const Scheme &s)
    {
        Cell c{0, INF, INF};
        set_insert(0, 0, c);
        for (int64_t i = 1; i < sizeH && !err; ++i) {
            const Cell prev = c;
            if (fe & FREE_TOP) c.s = 0;
            else if (affine) { mxc(c.e, prev.e + s.ext, prev.s + s.open, 0, 0); c.s = c.e; }
            else c.s = prev.s + s.ext;
            set_insert(int(i), 0, c);
        }
        Cell cv{0, INF, INF};
        for (int64_t i = 1; i < sizeV && !err; ++i) {
            if (fe & FREE_LEFT) cv.s = 0;
            else if (affine) { mxc(cv.f, cv.f + s.ext, cv.s + s.open, 0, 0); cv.s = cv.f; }
            else cv.s = cv.s + s.ext;
            set_insert(0, int(i), cv);
        }
        if (plan && pl->set_cap < sizeH + sizeV + 4) pl->set_cap = int32_t(sizeH + sizeV + 4);
    }

    __host__ __device__ int initialize(const Seed &s)
    {
        const int64_t hN = cmax<int64_t>(0, s.bh + 1 - k), vN = cmax<int64_t>(0, s.bv + 1 - k);
        int64_t up = cmin<int64_t>(m, hN + 2 * k + hsb(s) + cmax<int64_t>(0, k - s.bv - 1) + cmin<int64_t>(0, s.bh + 1 - k));
        int64_t lw = -cmin<int64_t>(n, vN + 2 * k + vsb(s) + cmax<int64_t>(0, k - s.bh - 1) + cmin<int64_t>(0, s.bv + 1 - k));
        int score = 0;
        if (hN != 0 || vN != 0) {
            init_beginning(up + 1, 1 - lw, gap);
            reinit(hN, vN, 1 + up, 1 - lw, 1 + up - hN, 1 - lw - vN);
            nl = 0;
            score = run_grid(&gap, KIND_INITIAL, false, 0, 0, h, up, v, -lw);
            // the initial gap area writes into the global set directly
            if (!plan && !err) {
                for (int i = 0; i < nl; ++i) {
                    const int g = new_global();
                    if (g < 0) break;
                    g_prepend(g, lslot(i), w.llen[i]);
                }
                nl = 0;
            }
        } else {
            init_beginning(up, -lw, anchor);
        }
        const int64_t gbh = hN, gbv = vN;
        const int64_t geh = cmin<int64_t>(m, s.eh + k), gev = cmin<int64_t>(n, s.ev + k);
        const int64_t lh = geh - gbh, lv = gev - gbv;
        int64_t hN2 = cmax<int64_t>(0, s.eh - k - hse(s) - cmax<int64_t>(0, s.ev + k - n) - gbh);
        int64_t vN2 = cmax<int64_t>(0, s.ev - k - vse(s) - cmax<int64_t>(0, s.eh + k - m) - gbv);
        up -= gbh;
        lw += gbv;
        if (lv + lw > up) vN2 -= (lv + lw) - up;
        reinit(hN2, vN2, up + 1, 1 - lw, lh - hN2 + 1, lv - vN2 + 1);
        if (lh < 0 || lv < 0) { fail(ST_UNDEFINED); return INT_MIN; }
        nl = 0;
        if (gbh == 0 && gbv == 0) {
            if (geh == m && gev == n) score = run_grid(&gap, KIND_GLOBAL, true, int(lw), int(up), h, lh, v, lv);
            else score = run_grid(&gap, KIND_INITIAL, true, int(lw), int(up), h, lh, v, lv);
        } else {
            score = run_grid(&gap, (geh == m && gev == n) ? KIND_FINAL : KIND_INNER, true, int(lw), int(up), h + gbh, lh,
                             v + gbv, lv);
        }
        if (gbh != 0 || gbv != 0) glue_local(gbh, gbv, true);
        else assign_global_from_local();
        hNext += gbh;
        vNext += gbv;
        if (lv + lw > up) vNext += (lv + lw) - up;
        return score;
    }

    __host__ __device__ void gap_area(const Seed &s)
    {
        const int64_t gbh = hNext, gbv = vNext;
        const int64_t geh = s.bh + 1 + k + hsb(s), gev = s.bv + 1 + k + vsb(s);
        const int64_t hN = s.bh + 1 - k - gbh, vN = s.bv + 1 - k - gbv;
        if (geh > m || gev > n || gbh > geh || gbv > gev) { fail(ST_UNDEFINED); return; }
        reinit(hN, vN, geh - gbh + 1, gev - gbv + 1, geh - gbh + 1 - hN, gev - gbv + 1 - vN);
        nl = 0;
        run_grid(&gap, KIND_INNER, false, 0, 0, h + gbh, geh - gbh, v + gbv, gev - gbv);
        glue_local(gbh, gbv, true);
        hNext += gbh;
        vNext += gbv;
    }

    __host__ __device__ void anchor_area(const Seed &s)
    {
        const int64_t gbh = hNext, gbv = vNext;
        const int64_t geh = s.eh + k, gev = s.ev + k;
        const int64_t lh = geh - gbh, lv = gev - gbv;
        const int64_t hN = s.eh - k - hse(s) - gbh, vN = s.ev - k - vse(s) - gbv;
        const int64_t lw = -2 * k - vsb(s), up = 2 * k + hsb(s);
        int64_t relV = vN;
        if (geh > m || gev > n || lh < 0 || lv < 0) { fail(ST_UNDEFINED); return; }
        if (lv + lw > up) relV -= (lv + lw) - up;
        reinit(hN, relV, up + 1, 1 - lw, lh - hN + 1, lv - vN + 1);
        nl = 0;
        run_grid(&anchor, KIND_INNER, true, int(lw), int(up), h + gbh, lh, v + gbv, lv);
        glue_local(gbh, gbv, true);
        hNext += gbh;
        vNext += gbv;
        if (lv + lw > up) vNext += (lv + lw) - up;
    }

    __host__ __device__ int finish(const Seed &s)
    {
        int64_t gbh = hNext, gbv = vNext;
        const int64_t hs = hsb(s), vs = vsb(s);
        int64_t geh = cmin<int64_t>(m, s.bh + 1 + k + hs), gev = cmin<int64_t>(n, s.bv + 1 + k + vs);
        int64_t lh = geh - gbh, lv = gev - gbv;
        int64_t hN = cmax<int64_t>(0, s.bh + 1 - k - gbh), vN = cmax<int64_t>(0, s.bv + 1 - k - gbv);
        int score;
        if (lh < 0 || lv < 0) { fail(ST_UNDEFINED); return INT_MIN; }
        reinit(hN, vN, lh + 1, lv + 1, lh - hN + 1, lv - vN + 1);
        nl = 0;
        run_grid(&gap, KIND_INNER, false, 0, 0, h + gbh, lh, v + gbv, lv);
        glue_local(gbh, gbv, true);
        gbh += hN;
        gbv += vN;
        geh = cmin<int64_t>(m, s.eh + k);
        gev = cmin<int64_t>(n, s.ev + k);
        lh = geh - gbh;
        lv = gev - gbv;
        if (lh < 0 || lv < 0) { fail(ST_UNDEFINED); return INT_MIN; }
        if (geh == m && gev == n) {
            const int64_t lw = -(gev - gbv), up = geh - gbh;
            reinit(0, 0, up + 1, 1 - lw, up + 1, 1 - lw);
            nl = 0;
            score = run_grid(&anchor, KIND_FINAL, true, int(lw), int(up), h + gbh, lh, v + gbv, lv);
            glue_local(gbh, gbv, true);
            return score;
        }
        const int64_t lw = -2 * k - vs, up = 2 * k + hs;
        hN = cmax<int64_t>(0, s.eh - k - hse(s) - gbh - cmax<int64_t>(0, s.ev + k - n));
        vN = cmax<int64_t>(0, s.ev - k - vse(s) - gbv - cmax<int64_t>(0, s.eh + k - m));
        if (lv + lw > up) vN -= (lv + lw) - up;
        reinit(hN, vN, up + 1, 1 - lw, lh - hN + 1, lv - vN + 1);
        nl = 0;
        run_grid(&anchor, KIND_INNER, true, int(lw), int(up), h + gbh, lh, v + gbv, lv);
        glue_local(gbh, gbv, true);
        gbh += hN;
        if (lv + lw > up) vN += (lv + lw) - up;
        gbv += vN;
        if (gbh > m || gbv > n) { fail(ST_UNDEFINED); return INT_MIN; }
        reinit(0, 0, m - gbh + 1, n - gbv + 1, m - gbh + 1, n - gbv + 1);
        nl = 0;
        score = run_grid(&gap, KIND_FINAL, false, 0, 0, h + gbh, m - gbh, v + gbv, n - gbv);
        glue_local(gbh, gbv, true);
        return score;
    }

    // The whole chain; returns the score (status in err).
    __host__ __device__ int run(const int32_t *seeds, int ns)
    {
        err = 0;
        hNext = vNext = 0;
        n4[0] = n4[1] = n4[2] = n4[3] = 0;
        nset = 0;
        ng = 0;
        gused = 0;
        nl = 0;
        if (ns < 1) return INT_MIN;
        if (m <= 0 || n <= 0 || k < 1) { fail(ST_UNDEFINED); return INT_MIN; }
        auto seed = [&](int i) {
            Seed s;
            s.bh = seeds[4 * i]; s.bv = seeds[4 * i + 1]; s.eh = seeds[4 * i + 2]; s.ev = seeds[4 * i + 3];
            s.lo = cmin(s.bh - s.bv, s.eh - s.ev);
            s.up = cmax(s.bh - s.bv, s.eh - s.ev);
            return s;
        };
        int it = 0;
        while (it != ns - 1) {
            const Seed s = seed(++it);
            if (s.bh - k <= 0) continue;
            if (s.bv - k <= 0) continue;
            --it;
            break;
        }
        int itEnd = ns - 1;
        while (itEnd != it) {
            const Seed s = seed(--itEnd);
            if (s.eh + k >= m) continue;
            if (s.ev + k >= n) continue;
            break;
        }
        int score = initialize(seed(it));
        if (err) return score;
        if (ns == 1 || (it == itEnd && itEnd == ns - 1)) {
            const Seed s = seed(it);
            if (s.eh + k < m || s.ev + k < n) {
                const int64_t gbh = hNext, gbv = vNext;
                reinit(0, 0, m + 1 - gbh, n + 1 - gbv, m + 1 - gbh, n + 1 - gbv);
                nl = 0;
                score = run_grid(&gap, KIND_FINAL, false, 0, 0, h + gbh, m - gbh, v + gbv, n - gbv);
                glue_local(gbh, gbv, false);
            }
            return score;
        }
        while (it != itEnd && !err) {
            ++it;
            const Seed s = seed(it);
            gap_area(s);
            anchor_area(s);
        }
        if (err) return score;
        return finish(seed(++it));
    }
};

}  // namespace chain

struct ChainArgs {
    const uint8_t *seq_h, *seq_v;
    const int32_t *seeds;
    const chain::ChainDesc *chains;
    int64_t num_chains;
    uint8_t *arena;
    chain::Scheme anchor, gap;
    int32_t free_ends, band_ext, affine, max_traces;
    int32_t *score, *status, *n_traces, *seg_count;
};

namespace chain {

// Scratch layout of one chain inside its arena slice (shared by the host sizing and the kernel).
__host__ __device__ inline int64_t align16(int64_t x) { return (x + 15) & ~int64_t(15); }

__host__ __device__ inline int64_t layout(const Plan &p, int max_traces, uint8_t *base, Work *w)
{
    int64_t o = 0;
    auto take = [&](int64_t bytes) { const int64_t at = o; o = align16(o + bytes); return base ? base + at : nullptr; };
    uint8_t *T = take(p.trace_bytes);
    int *c0 = reinterpret_cast<int *>(take(int64_t(p.col_rows) * 4));
    int *c1 = reinterpret_cast<int *>(take(int64_t(p.col_rows) * 4));
    int *e0 = reinterpret_cast<int *>(take(int64_t(p.col_rows) * 4));
    int *e1 = reinterpret_cast<int *>(take(int64_t(p.col_rows) * 4));
    Cell *v4[4];
    for (int q = 0; q < 4; ++q) v4[q] = reinterpret_cast<Cell *>(take(int64_t(p.vlen[q]) * int64_t(sizeof(Cell))));
    InitCell *set = reinterpret_cast<InitCell *>(take(int64_t(p.set_cap) * int64_t(sizeof(InitCell))));
    int *mp = reinterpret_cast<int *>(take(int64_t(p.mp_cap) * 4));
    Seg *gseg = reinterpret_cast<Seg *>(take(int64_t(max_traces) * p.gseg_cap * int64_t(sizeof(Seg))));
    int *glen = reinterpret_cast<int *>(take(int64_t(max_traces) * 4));
    int *gorder = reinterpret_cast<int *>(take(int64_t(max_traces) * 4));
    Seg *lseg = reinterpret_cast<Seg *>(take(int64_t(max_traces) * p.lseg_cap * int64_t(sizeof(Seg))));
    int *llen = reinterpret_cast<int *>(take(int64_t(max_traces) * 4));
    int *erase = reinterpret_cast<int *>(take(int64_t(max_traces) * 4));
    ColDesc *cols = reinterpret_cast<ColDesc *>(take(int64_t(p.col_cap) * int64_t(sizeof(ColDesc))));
    int *aS = reinterpret_cast<int *>(take(int64_t(p.col_cap) * 12));
    int *aE = reinterpret_cast<int *>(take(int64_t(p.col_cap) * 12));
    int *aF = reinterpret_cast<int *>(take(int64_t(p.col_cap) * 12));
    int *ccS = reinterpret_cast<int *>(take(int64_t(p.col_cap) * 4));
    int *ccP = reinterpret_cast<int *>(take(int64_t(p.col_cap) * 4));
    int *ccF = reinterpret_cast<int *>(take(int64_t(p.col_cap) * 4));
    int *fcS = reinterpret_cast<int *>(take(int64_t(p.col_rows) * 4));
    int *fcP = reinterpret_cast<int *>(take(int64_t(p.col_rows) * 4));
    int *fcF = reinterpret_cast<int *>(take(int64_t(p.col_rows) * 4));
    if (w) {
        w->cols = cols; w->aS = aS; w->aE = aE; w->aF = aF;
        w->ccS = ccS; w->ccP = ccP; w->ccF = ccF; w->fcS = fcS; w->fcP = fcP; w->fcF = fcF;
        w->T = T; w->cS0 = c0; w->cS1 = c1; w->cE0 = e0; w->cE1 = e1;
        for (int q = 0; q < 4; ++q) w->v4[q] = v4[q];
        w->set = set; w->mp = mp; w->gseg = gseg; w->glen = glen; w->gorder = gorder;
        w->lseg = lseg; w->llen = llen; w->erase = erase;
    }
    return o;
}

}  // namespace chain

// Launchers of the two kernels below (defined in chain.cu, their own translation unit).
void launch_banded_chain(const ChainArgs &a, cudaStream_t st);
void launch_chain_pack(const chain::ChainDesc *chains, int64_t num_chains, const uint8_t *arena, int32_t max_traces,
                       const int32_t *seg_count, const int64_t *dense_off, chain::Seg *dense, cudaStream_t st);

#ifdef SEQAN_GB300_CHAIN_KERNELS
__global__ void __launch_bounds__(128) k_banded_chain(ChainArgs a)
{
    const int64_t c = (int64_t(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
    const int lane = int(threadIdx.x & 31);
    if (c >= a.num_chains) return;   // whole warps leave together
    const chain::ChainDesc &d = a.chains[c];
    chain::Plan pl = d.plan;
    chain::Engine e;
    e.plan = false;
    e.warp = true;
    e.lane = lane;
    e.anchor = a.anchor;
    e.gap = a.gap;
    e.fe = a.free_ends;
    e.affine = a.affine;
    e.k = a.band_ext;
    e.max_traces = a.max_traces;
    e.h = a.seq_h + d.h_off;
    e.v = a.seq_v + d.v_off;
    e.m = d.m;
    e.n = d.n;
    e.pl = &pl;
    chain::layout(pl, a.max_traces, a.arena + d.arena_off, &e.w);
    int score = INT_MIN;
    if (pl.status == chain::ST_OK) score = e.run(a.seeds + 4 * d.seed_off, d.n_seeds);
    else e.err = pl.status;
    __syncwarp();
    if (lane == 0) {
        a.score[c] = score;
        a.status[c] = e.err;
        a.n_traces[c] = e.ng;
        a.seg_count[c] = (!e.err && e.ng > 0) ? e.w.glen[e.w.gorder[0]] : 0;
    }
}

// Copies the first trace of each chain's set (kept reversed in its scratch) to the dense output in
// the reference's order.
__global__ void __launch_bounds__(128) k_chain_pack(const chain::ChainDesc *chains, int64_t num_chains,
                                                    const uint8_t *arena, int32_t max_traces,
                                                    const int32_t *seg_count, const int64_t *dense_off,
                                                    chain::Seg *dense)
{
    const int64_t c = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (c >= num_chains) return;
    const int32_t cnt = seg_count[c];
    if (cnt <= 0) return;
    const chain::ChainDesc &d = chains[c];
    chain::Work w;
    chain::layout(d.plan, max_traces, const_cast<uint8_t *>(arena) + d.arena_off, &w);
    const chain::Seg *src = w.gseg + int64_t(w.gorder[0]) * d.plan.gseg_cap;
    chain::Seg *dst = dense + dense_off[c];
    for (int32_t q = 0; q < cnt; ++q) dst[q] = src[cnt - 1 - q];
}
#endif
