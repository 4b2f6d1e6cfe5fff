// seed_kernels.cuh -- seed extension: extendSeed(Seed<Simple>, database, query, direction, ...)
// with MatchExtend, UnGappedXDrop and GappedXDrop (seeds/seeds_extension.h:181-218, 283-360,
// 613-835) over a batch of seeds.
//
// GappedXDrop runs the reference's anti-diagonal DP (_extendSeedGappedXDropOneDirection): each
// anti-diagonal holds the columns [minCol - 1, maxCol]; cells below best - X become `undefined`
// (INT_MIN - gap) and the live column range shrinks from both ends where two consecutive
// anti-diagonals are undefined.  One thread owns one seed at a time and keeps the three
// anti-diagonals a cell reads in a ring of RING slots indexed by column (slot = column mod
// RING), in shared memory interleaved by thread (slot s of thread t is word s * blockDim + t, so
// a warp's accesses hit 32 different banks whatever the columns).  The kernel is persistent:
// every loop iteration steps the thread's current seed by one anti-diagonal, and a thread that
// finishes a direction or a seed starts the next one in the same iteration, so lanes do not
// idle while their warp-mates finish longer extensions.  A seed whose live range outgrows the
// ring is queued for the next level (a 64-slot ring, then a ring in global memory that holds
// the whole query), which re-runs it from the start.
#pragma once

#include <cstdint>
#include <climits>

namespace gba {

constexpr int kSeedBlock = 128;

struct SeedDev {               // gba_seed: Seed<Simple, DefaultSeedConfig>
    int64_t begin_h, begin_v, end_h, end_v;
    int64_t lower_diag, upper_diag;
};

struct SeedArgs {
    const uint8_t *seq_h, *seq_v;
    const int64_t *off_h, *off_v;
    const int32_t *seed_h, *seed_v;   // per seed: database / query index (null: the seed's own index)
    int64_t num_h, num_v;
    SeedDev *seeds;
    int32_t *scores;                  // null or 2 per seed (gapped: left, right extension score)
    int32_t num_seeds;
    int32_t method, direction, xdrop;
    int32_t match, mismatch, gap;
    const int32_t *matrix;            // device alphabet^2 table or null
    int32_t alphabet_size;
    int32_t *error;                   // bit 0: a seed outside its sequences; bit 1: a live range
                                      // wider than the last level's ring
    unsigned long long *cells;        // DP cells computed (gapped)
    struct XResult *results;          // gapped: per seed, applied by k_apply_gapped
};

// One gapped seed's extension in both directions (rows grow the database side, columns the
// query side; diagonals relative to the seed end each direction starts from).
struct XResult {
    int32_t l_row, l_col, l_lower, l_upper;
    int32_t r_row, r_col, r_lower, r_upper;
    int32_t l_score, r_score;
    int32_t flags;                    // 1: left grew, 2: right grew, 4: done
    int32_t pad;
};

// One level of the gapped cascade.
struct XLevel {
    const int32_t *in_list, *in_count;   // seeds to run (null: every seed)
    int32_t *out_list, *out_count;       // seeds that outgrew the ring (null: an error)
    int32_t *next;                       // work counter of the persistent loop
    int32_t *scratch;                    // global ring (STRIDE 1): 3 * ring ints per thread
    int32_t ring;                        // global ring slots (power of two)
    int32_t threads;                     // threads that own global scratch
};

template <bool MATRIX>
struct XdropScore {
    const int32_t *mat;   // shared-memory table (matrix schemes)
    int32_t asize, match, mismatch;
    __device__ __forceinline__ int operator()(int a, int b) const
    {
        if (MATRIX) return mat[a * asize + b];
        return a == b ? match : mismatch;
    }
};

template <bool MATRIX>
__device__ __forceinline__ XdropScore<MATRIX> load_score(const SeedArgs &a, int32_t *smat)
{
    XdropScore<MATRIX> sc{smat, a.alphabet_size, a.match, a.mismatch};
    if (MATRIX) {
        const int cnt = a.alphabet_size * a.alphabet_size;
        for (int t = threadIdx.x; t < cnt; t += blockDim.x) smat[t] = a.matrix[t];
    }
    __syncthreads();
    return sc;
}

// Locates seed i's sequences and checks it lies on them.
__device__ __forceinline__ bool seed_sequences(const SeedArgs &a, int64_t i, const SeedDev &s, const uint8_t *&db,
                                               int64_t &m, const uint8_t *&q, int64_t &n)
{
    const int64_t hi = a.seed_h ? a.seed_h[i] : i;
    const int64_t vi = a.seed_v ? a.seed_v[i] : i;
    if (hi < 0 || hi >= a.num_h || vi < 0 || vi >= a.num_v) return false;
    db = a.seq_h + a.off_h[hi];
    m = a.off_h[hi + 1] - a.off_h[hi];
    q = a.seq_v + a.off_v[vi];
    n = a.off_v[vi + 1] - a.off_v[vi];
    if (!(0 <= s.begin_h && s.begin_h <= s.end_h && s.end_h <= m && 0 <= s.begin_v && s.begin_v <= s.end_v &&
          s.end_v <= n))
        return false;
    // GappedXDrop: 2 * max(rows, cols) must fit int, as the reference computes it.
    if (a.method == 2 && (m > (int64_t(1) << 29) || n > (int64_t(1) << 29))) return false;
    // UnGappedXDrop's left walk first scores database[beginH] / query[beginV]: past the end for
    // an empty seed at the end of a sequence, so such seeds are refused.
    if (a.method == 1 && (a.direction & 1) && a.xdrop > 0 && s.begin_h >= 1 && s.begin_v >= 1 &&
        (s.begin_h >= m || s.begin_v >= n))
        return false;
    return true;
}

// MatchExtend (:181-218) and UnGappedXDrop (:283-360).
template <bool MATRIX>
__device__ void simple_seed(const SeedArgs &a, XdropScore<MATRIX> sc, SeedDev &s, const uint8_t *db, int64_t m,
                            const uint8_t *q, int64_t n)
{
    const bool ungapped = a.method == 1;
    const int drop = -a.xdrop;
    if (a.direction & 1) {
        int64_t ph = s.begin_h, pv = s.begin_v, mism = 0;
        int tmp = 0;
        if (!ungapped) {
            while (ph >= 1 && pv >= 1 && db[ph - 1] == q[pv - 1]) { --ph; --pv; }
        } else {
            while (ph >= 1 && pv >= 1 && tmp > drop) {
                tmp += sc(db[ph], q[pv]);   // the pair at the walk's position, as the reference scores it
                if (db[ph - 1] == q[pv - 1]) {
                    mism = 0;
                    if (tmp > 0) tmp = 0;
                } else {
                    ++mism;
                }
                --ph;
                --pv;
            }
        }
        s.begin_h = ph + mism;
        s.begin_v = pv + mism;
    }
    if (a.direction & 2) {
        int64_t ph = s.end_h, pv = s.end_v, mism = 0;
        int tmp = 0;
        if (!ungapped) {
            while (ph < m && pv < n && db[ph] == q[pv]) { ++ph; ++pv; }
        } else {
            while (ph < m && pv < n && tmp > drop) {
                tmp += sc(db[ph], q[pv]);
                if (db[ph] == q[pv]) {
                    mism = 0;
                    if (tmp > 0) tmp = 0;
                } else {
                    ++mism;
                }
                ++ph;
                ++pv;
            }
        }
        s.end_h = ph - mism;
        s.end_v = pv - mism;
    }
}

// MatchExtend / UnGappedXDrop: one thread per seed.
template <bool MATRIX>
__global__ void __launch_bounds__(kSeedBlock) k_extend_simple(SeedArgs a)
{
    __shared__ int32_t smat[32 * 32];
    const XdropScore<MATRIX> sc = load_score<MATRIX>(a, smat);
    const int64_t i = (int64_t)blockIdx.x * kSeedBlock + threadIdx.x;
    if (i >= a.num_seeds) return;
    SeedDev s = a.seeds[i];
    const uint8_t *db, *q;
    int64_t m, n;
    if (!seed_sequences(a, i, s, db, m, q, n)) {
        atomicOr(a.error, 1);
        return;
    }
    simple_seed(a, sc, s, db, m, q, n);
    a.seeds[i] = s;
}

template <int RING> struct XMinBlocks { static constexpr int value = RING <= 16 ? 5 : (RING <= 32 ? 3 : 2); };

constexpr int kRefillLanes = 8;   // idle lanes that trigger a warp refill

// Rings per thread, one word per slot: anti-diagonals k-2, k-1, k, then the query residues by
// column and the database residues by row.  Both residue windows only slide forward: per
// anti-diagonal at most one new column (maxCol grows by one at most) and one new row
// (k - minCol) enter, so each step loads the next residue of each stream from global memory into
// a register and stores it into its ring at the following step, when the load has completed.
// (Residues packed four to a word let 7 blocks reside instead of 5 but ran 6% slower: the byte
// addressing costs more issue slots than the extra warps recover.)
__host__ __device__ constexpr int seed_ring_words(int ring) { return 5 * ring; }

// GappedXDrop, one level of the cascade.  RING slots in shared memory (STRIDE = kSeedBlock), or
// lv.ring slots of global scratch per thread (STRIDE = 1; lv.threads is a multiple of 32).
template <int RING, int STRIDE, bool MATRIX>
__global__ void __launch_bounds__(kSeedBlock, STRIDE == 1 ? 4 : XMinBlocks<RING>::value)
    k_extend_gapped(SeedArgs a, XLevel lv)
{
    extern __shared__ int32_t smem[];
    int32_t *smat = STRIDE == 1 ? smem : smem + seed_ring_words(RING) * kSeedBlock;
    const XdropScore<MATRIX> sc0 = load_score<MATRIX>(a, smat);
    const int tglob = blockIdx.x * kSeedBlock + threadIdx.x;
    if (STRIDE == 1 && tglob >= lv.threads) return;   // whole warps
    const unsigned FULL = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    int32_t *const base =
        STRIDE == 1 ? lv.scratch + (size_t)tglob * seed_ring_words(lv.ring) : smem + threadIdx.x;
    const int ring = STRIDE == 1 ? lv.ring : RING;
    const int rmask = ring - 1;
    int32_t *const qres = base + 3 * ring * STRIDE;   // query residue of column c
    int32_t *const dres = base + 4 * ring * STRIDE;   // database residue of row r
    const int count = lv.in_list ? *lv.in_count : a.num_seeds;
    const int xdrop = a.xdrop;

    bool idle = true, drained = false;
    // the current seed: index, the right side prepared at fetch, the left side's result
    int i = 0, dir = 0;
    const uint8_t *qR = nullptr, *dR = nullptr;
    int qlenR = 0, dlenR = 0;
    int l_row = 0, l_col = 0, l_lower = 0, l_upper = 0, l_score = 0, l_flag = 0;
    // the current direction
    XdropScore<MATRIX> sc = sc0;
    const uint8_t *qbase = nullptr, *dbase = nullptr;
    int step = 1, rows = 0, cols = 0, gap = 0, U = 0;
    int k = 0, minCol = 0, maxCol = 0, best = 0, lowerDiag = 0, upperDiag = 0;
    int lo1 = 0, hi1 = 0, lo2 = 0, hi2 = 0, lo3 = 0, hi3 = 0;
    int qnext = 0, dnext = 0;             // next column / row whose residue is not loaded yet
    int qpend = -1, dpend = -1;           // residues loaded at the previous step, stored at this one
    uint64_t cells = 0;
#define XR(r, c) (r)[((c) & rmask) * STRIDE]
#define XB(r, c) XR(r, c)

    // Starts direction `dir` on (qb, db, qlen, dlen); false when that side is empty (score 0,
    // seed unchanged, :626-627).
    auto start = [&](const uint8_t *qb, const uint8_t *dbp, int qlen, int dlen, int stp) -> bool {
        qbase = qb;
        dbase = dbp;
        step = stp;
        cols = qlen + 1;
        rows = dlen + 1;
        if (rows == 1 || cols == 1) return false;
        // minimal error score, gap and mismatch limits, `undefined` (:629-637)
        const int len = 2 * (cols > rows ? cols : rows);
        const int minErr = INT_MIN / len;
        gap = a.gap > minErr ? a.gap : minErr;
        sc = sc0;
        if (!MATRIX && sc.mismatch < minErr) sc.mismatch = minErr;
        U = INT_MIN - gap;
        // _initAntiDiags (:451-477): anti-diagonal 0 in ring 1, anti-diagonal 1 in ring 2
        lo2 = 0; hi2 = 0;
        lo3 = 0; hi3 = 1;
        base[(1 * ring) * STRIDE] = 0;
        const int g0 = (-gap > xdrop) ? U : gap;
        base[(2 * ring) * STRIDE] = g0;
        base[(2 * ring + 1) * STRIDE] = g0;
        minCol = 1;
        maxCol = 2;
        k = 1;
        best = 0;
        lowerDiag = 0;
        upperDiag = 0;
        // residues of columns 1..2 and rows 1..2 (the first anti-diagonals)
        XB(qres, 1) = qbase[step];
        XB(dres, 1) = dbase[step];
        if (qlen >= 2) XB(qres, 2) = qbase[2 * step];
        if (dlen >= 2) XB(dres, 2) = dbase[2 * step];
        qnext = 3;
        dnext = 3;
        qpend = -1;
        dpend = -1;
        return true;
    };
    // Records the finished direction (score, and the extension when `grew`) and moves on: to
    // the right side, or the seed is done and the lane idles.
    auto finish = [&](int score, bool grew, int row, int col) {
        for (;;) {
            if (dir == 0) {
                l_score = score;
                l_flag = grew ? 1 : 0;
                l_row = row;
                l_col = col;
                l_lower = lowerDiag;
                l_upper = upperDiag;
                if (a.direction & 2) {
                    dir = 1;
                    if (start(qR, dR, qlenR, dlenR, 1)) return;
                    score = 0;
                    grew = false;
                    continue;
                }
            }
            XResult r;
            r.l_row = l_row;
            r.l_col = l_col;
            r.l_lower = l_lower;
            r.l_upper = l_upper;
            r.r_row = row;
            r.r_col = col;
            r.r_lower = lowerDiag;
            r.r_upper = upperDiag;
            r.l_score = l_score;
            r.r_score = dir == 1 ? score : 0;
            r.flags = 4 | l_flag | ((dir == 1 && grew) ? 2 : 0);
            r.pad = 0;
            a.results[i] = r;
            idle = true;
            return;
        }
    };

    for (;;) {
        const unsigned want = __ballot_sync(FULL, idle && !drained);
        const unsigned busy = __ballot_sync(FULL, !idle);
        if (!want && !busy) break;
        if (want && (__popc(want) >= kRefillLanes || !busy)) {
            const int leader = __ffs(want) - 1;
            int first = 0;
            if (lane == leader) first = atomicAdd(lv.next, __popc(want));
            first = __shfl_sync(FULL, first, leader);
            if (idle && !drained) {
                const int j = first + __popc(want & ((1u << lane) - 1));
                if (j >= count) {
                    drained = true;
                } else {
                    i = lv.in_list ? lv.in_list[j] : j;
                    const SeedDev s = a.seeds[i];
                    const uint8_t *db, *q;
                    int64_t m, n;
                    if (!seed_sequences(a, i, s, db, m, q, n)) {
                        atomicOr(a.error, 1);
                    } else {
                        // prefix(query, beginV) / prefix(database, beginH) read backwards, the
                        // suffixes from endV / endH forwards (seeds/seeds_extension.h:800-830)
                        qR = q + s.end_v - 1;
                        dR = db + s.end_h - 1;
                        qlenR = (int)(n - s.end_v);
                        dlenR = (int)(m - s.end_h);
                        idle = false;
                        l_flag = 0;
                        l_score = 0;
                        if (a.direction & 1) {
                            dir = 0;
                            if (!start(q + s.begin_v, db + s.begin_h, (int)s.begin_v, (int)s.begin_h, -1))
                                finish(0, false, 0, 0);
                        } else {
                            dir = 1;
                            if (!start(qR, dR, qlenR, dlenR, 1)) finish(0, false, 0, 0);
                        }
                    }
                }
            }
        }
        if (idle) continue;
        // one anti-diagonal
        ++k;
        lo1 = lo2; hi1 = hi2;
        lo2 = lo3; hi2 = hi3;
        lo3 = minCol - 1; hi3 = maxCol;
        if (hi3 - lo3 + 1 > ring) {
            // live range wider than the ring: the next level re-runs the seed
            if (lv.out_list) lv.out_list[atomicAdd(lv.out_count, 1)] = i;
            else atomicOr(a.error, 2);
            idle = true;
            continue;
        }
        // anti-diagonals k-2, k-1, k live in rings (k-1) % 3, k % 3, (k+1) % 3
        const int km = k % 3;
        int32_t *const r1 = base + (km == 0 ? 2 : km - 1) * ring * STRIDE;
        int32_t *const r2 = base + km * ring * STRIDE;
        int32_t *const r3 = base + (km == 2 ? 0 : km + 1) * ring * STRIDE;
        const int thr = best - xdrop;
        const int kg = k * gap;
        // _initAntiDiag3 (:492-513)
        int blo = U, bhi = U;
        if (kg > thr) {
            if (lo3 == 0) blo = kg;
            if (k == maxCol) bhi = kg;
        }
        XR(r3, lo3) = blo;
        XR(r3, hi3) = bhi;
        cells += (uint64_t)(maxCol - minCol);
        // residues: store last step's loads (columns < maxCol and rows <= k - minCol are then
        // all in their rings), then load the next column / row this anti-diagonal may add
        if (qpend >= 0) XB(qres, qnext - 1) = qpend;
        if (dpend >= 0) XB(dres, dnext - 1) = dpend;
        qpend = -1;
        dpend = -1;
        if (qnext <= maxCol && qnext < cols) {
            qpend = qbase[step * qnext];
            ++qnext;
        }
        if (dnext <= k + 1 - minCol && dnext < rows) {
            dpend = dbase[step * dnext];
            ++dnext;
        }
        int dbest = kg;
        int up = XR(r2, lo3);
        // The reference's minCol / maxCol scans (:708-721) read back what this loop writes: the
        // first column c >= minCol with A3[c] or A2[c-1] defined, and the last column
        // c >= minCol - 1 with A3[c] or A2[c] defined.  Both are tracked here instead.
        int lastLive = (blo != U || up != U) ? lo3 : lo3 - 1;
        int firstLive = INT_MAX;
#pragma unroll 2
        for (int col = minCol; col < maxCol; ++col) {
            const int cur = XR(r2, col);
            const int dg = XR(r1, col - 1);
            const int sub = sc(XB(qres, col), XB(dres, k - col));
            int t = max(max(up, cur) + gap, dg + sub);
            const bool def = t >= thr;
            t = def ? t : U;
            XR(r3, col) = t;
            dbest = max(dbest, t);    // `undefined` never exceeds k * gap
            firstLive = min(firstLive, (def || up != U) ? col : INT_MAX);
            lastLive = (def || cur != U) ? col : lastLive;
            up = cur;
        }
        if (firstLive == INT_MAX) firstLive = (bhi != U || up != U) ? maxCol : maxCol + 1;
        best = max(best, dbest);
        minCol = firstLive;
        maxCol = lastLive + 2;
        // _calcExtendedLowerDiag / _calcExtendedUpperDiag (:517-537), the end clamps (:727-730)
        lowerDiag = min(lowerDiag, 2 * minCol - k);
        upperDiag = max(upperDiag, 2 * (maxCol - 1) - k - 2);
        minCol = max(minCol, k + 2 - rows);
        maxCol = min(maxCol, cols);
        if (minCol >= maxCol) {
            // position of the longest extension (:733-770)
            int lcol = hi3 - 1;
            int lrow = k - lcol;
            int ls = XR(r3, lcol);
            if (ls == U) {
                if (XR(r2, hi2 - 1) != U) {
                    lcol = hi2 - 1;
                    lrow = k - 1 - lcol;
                    ls = XR(r2, lcol);
                } else if (hi2 - lo2 + 1 > 2 && XR(r2, hi2 - 2) != U) {
                    lcol = hi2 - 2;
                    lrow = k - 1 - lcol;
                    ls = XR(r2, lcol);
                }
            }
            if (ls == U) {
                for (int c = lo1; c <= hi1; ++c) {
                    const int v = XR(r1, c);
                    if (v > ls) {
                        ls = v;
                        lcol = c;
                        lrow = k - 2 - lcol;
                    }
                }
            }
            finish(ls, ls != U, lrow, lcol);
        }
    }
#undef XR
#undef XB
    if (cells) atomicAdd(a.cells, (unsigned long long)cells);
}

// Writes the grown seeds and scores (_updateExtendedSeed, :539-579: left, then right, as
// extendSeed calls them).  Seeds without a finished result (invalid ones) stay unchanged.
__global__ void __launch_bounds__(kSeedBlock) k_apply_gapped(SeedArgs a)
{
    const int i = blockIdx.x * kSeedBlock + threadIdx.x;
    if (i >= a.num_seeds) return;
    const XResult r = a.results[i];
    if (!(r.flags & 4)) return;
    SeedDev s = a.seeds[i];
    if (r.flags & 1) {
        const int64_t bd = s.begin_h - s.begin_v;
        s.lower_diag = min(s.lower_diag, bd + r.l_lower);
        s.upper_diag = max(s.upper_diag, bd + r.l_upper);
        s.begin_h -= r.l_row;
        s.begin_v -= r.l_col;
    }
    if (r.flags & 2) {
        const int64_t ed = s.end_h - s.end_v;
        s.upper_diag = max(s.upper_diag, ed - r.r_lower);
        s.lower_diag = min(s.lower_diag, ed - r.r_upper);
        s.end_h += r.r_row;
        s.end_v += r.r_col;
    }
    a.seeds[i] = s;
    if (a.scores) {
        a.scores[2 * i] = r.l_score;
        a.scores[2 * i + 1] = r.r_score;
    }
}

}  // namespace gba
