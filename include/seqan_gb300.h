/*
 * seqan_gb300.h -- C-ABI of the GB300 batch pairwise-alignment engine.
 *
 * This is the drop-in boundary for SeqAn 2's batch alignment interface.  Every entry point
 * takes plain pointers and sizes; residues are the reference alphabets' ordValue codes
 * (Dna/Dna5: A=0 C=1 G=2 T=3 N=4; AminoAcid: the 27-letter order A B C D E F G H I J K L M
 * N O P Q R S T U V W Y Z X *).  One call aligns a whole batch on one GPU.
 *
 * Reference interfaces each entry point replaces (paths relative to the SeqAn 2 tree):
 *   gba_align_batch with GBA_OUT_SCORE, mode GBA_GLOBAL:
 *       globalAlignmentScore(ExecutionPolicy<Parallel,Vectorial>, StringSet, StringSet,
 *       Score, AlignConfig[, lower, upper])
 *       align_parallel/parallel_align_interface.h:330-340 -> align/global_alignment_unbanded.h:739-821,
 *       banded align/global_alignment_banded.h:558-652
 *   ... mode GBA_LOCAL: localAlignmentScore(...) parallel_align_interface.h:357-365 ->
 *       align/local_alignment_unbanded.h:554-572, banded align/local_alignment_banded.h:252
 *   ... with GBA_OUT_SEGMENTS: globalAlignment / localAlignment over StringSet<Gaps>
 *       parallel_align_interface.h:288-321 -> align/global_alignment_unbanded.h:831-888,
 *       align/global_alignment_banded.h:658-700, align/local_alignment_unbanded.h:367-399;
 *       segments are the reference's TraceSegment_ list (align/dp_trace_segment.h:60-100)
 *       that _adaptTraceSegmentsTo turns into Gaps (align/dp_traceback_adaptor.h:57-117).
 *   ... with GBA_OUT_CIGAR: getCigarString(cigar, gapsH, gapsV) bam_io/cigar.h:261-339.
 *   gba_batch.h_shared = 1: the one-vs-many overload (String vs StringSet)
 *       align/global_alignment_unbanded.h:766-821.
 *
 * Errors are status codes; nothing throws and nothing falls back to the CPU.
 */
#ifndef SEQAN_GB300_H_
#define SEQAN_GB300_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#if defined(__GNUC__)
#define GBA_API __attribute__((visibility("default")))
#else
#define GBA_API
#endif

/* Status codes returned by every entry point. */
enum {
    GBA_OK = 0,
    GBA_EINVAL = 1,        /* malformed arguments */
    GBA_ENOMEM = 2,        /* device or pinned allocation failed */
    GBA_EBUDGET = 3,       /* request exceeds the context's HBM budget */
    GBA_ECUDA = 4,         /* a CUDA call failed; see gba_last_error */
    GBA_ETIMEOUT = 5,      /* a bounded device wait or a host watchdog expired */
    GBA_EUNSUPPORTED = 6,  /* parameter combination not supported */
    GBA_ECAPACITY = 7,     /* an output buffer supplied by the caller is too small */
    GBA_EPARSE = 8         /* input text is not in the format (ParseError / UnexpectedEnd) */
};

/* Per-pair status flags (gba_result.pair_status). */
enum {
    GBA_PAIR_OK = 0,
    GBA_PAIR_INVALID = 1,   /* empty sequence or band outside the matrix: score = numeric min */
    GBA_PAIR_PROMOTED = 2,  /* 16-bit cells were requested but the pair may leave the exact
                               int16 range; it ran with 32-bit cells (exact result) */
    GBA_PAIR_FAILED = 3,    /* serving only: the request's batch failed (no result) */
    GBA_PAIR_SKIPPED = 4    /* gba_align_score_noalloc only: |H| above the call's max_h_len, not
                               computed (score = numeric min) */
};

/* GBA_ALIGN_EXTEND: the AlignExtend_ DP of extendAlignment's banded overloads
 * (align_extend/align_extend.h:137-206, align_extend/align_extend_base.h): a gap-initialised
 * first row and column, every cell tracked without a zero floor, traceback from the first maximum
 * to (0, 0) with the head gaps but no tail, and with GBA_FLAG_XDROP the X-drop terminator of
 * align_extend/dp_scout_xdrop.h (threshold gba_params.xdrop).  Banded only (band_on), 32-bit cells;
 * the band is valid when band_lower <= 0 <= band_upper (a free last row and column, not a free
 * first row or column), otherwise the pair is GBA_PAIR_INVALID with score INT32_MIN as the
 * reference returns.  gba_extend_alignments runs both sides of extendAlignment on it when its
 * params carry a band. */
enum { GBA_GLOBAL = 0, GBA_LOCAL = 1, GBA_ALIGN_EXTEND = 2 };
/* GBA_GAPS_AUTO picks affine iff gap_open != gap_extend, as the reference's
 * interfaces do (align/global_alignment_unbanded.h:801-810).  GBA_GAPS_DYNAMIC selects the
 * reference's DynamicGaps cells (align/dp_cell_dynamic.h, align/dp_formula_dynamic.h): one score and
 * two gap flags per cell, a gap extended when the neighbour's flag for its direction is set and
 * opened otherwise; unbanded global and local alignments (a band is GBA_EUNSUPPORTED). */
enum { GBA_GAPS_AUTO = 0, GBA_GAPS_LINEAR = 1, GBA_GAPS_AFFINE = 2, GBA_GAPS_DYNAMIC = 3 };
/* AlignConfig<TOP, LEFT, RIGHT, BOTTOM> (align/align_config.h:52-94). */
enum { GBA_FREE_TOP = 1, GBA_FREE_LEFT = 2, GBA_FREE_RIGHT = 4, GBA_FREE_BOTTOM = 8 };
/* Output selection bits. */
enum { GBA_OUT_SCORE = 1, GBA_OUT_END = 2, GBA_OUT_SEGMENTS = 4, GBA_OUT_CIGAR = 8 };
/* TraceSegment_ direction values (align/dp_profile.h:121-135). */
enum { GBA_SEG_DIAGONAL = 1, GBA_SEG_HORIZONTAL = 2, GBA_SEG_VERTICAL = 4 };

typedef struct gba_context gba_context;

typedef struct {
    int32_t device;            /* CUDA device ordinal */
    int64_t hbm_budget_bytes;  /* 0 = no budget; otherwise batches needing more fail with GBA_EBUDGET */
} gba_config;

typedef struct {
    int32_t mode;              /* GBA_GLOBAL / GBA_LOCAL / GBA_ALIGN_EXTEND */
    int32_t gap_model;         /* GBA_GAPS_* */
    int32_t free_ends;         /* GBA_FREE_* bits (global only; local treats all four as free) */
    int32_t band_on;           /* 1: DPBandConfig<BandOn>(band_lower, band_upper) */
    int32_t band_lower, band_upper;  /* diagonals, col - row convention (align/dp_band.h:111-161) */
    int32_t match, mismatch;   /* Score<T, Simple> (score/score_simple.h:54-98) */
    int32_t gap_open, gap_extend;  /* a gap of length k costs gap_open + (k-1) * gap_extend */
    const int32_t *matrix;     /* optional alphabet_size^2 substitution table (row = H code),
                                  e.g. the 27x27 Blosum62 of score/score_matrix_data.h */
    int32_t alphabet_size;     /* codes are < alphabet_size (<= 32 with a matrix); 0 = unknown */
    int32_t score_bits;        /* 16 or 32: the reference's TScoreValue width */
    int32_t outputs;           /* GBA_OUT_* bits */
    int32_t flags;             /* GBA_FLAG_* kernel selection (0 = automatic) */
    int32_t tile_variant;      /* packed kernel tiling: 0 = automatic (tuning table / autotune /
                                  default); v in 1..GBA_TILE_VARIANTS forces variant v - 1 */
    int32_t xdrop;             /* GBA_ALIGN_EXTEND with GBA_FLAG_XDROP: the X-drop threshold */
} gba_params;

/* Tiling variants of the packed kernel (rows per register strip x minimum resident blocks per
 * SM): 1 = 32 x 2, 2 = 32 x 3, 3 = 24 x 3, 4 = 24 x 4, 5 = 16 x 4. */
#define GBA_TILE_VARIANTS 5

/* Kernel selection flags (gba_params.flags); results are identical either way.
 * With equality scoring the engine uses its packed two-pairs-per-thread 16-bit kernel for global
 * score-only pairs when alphabet_size is between 1 and 8 (the caller's promise that every code is
 * below it, as the reference's alphabet types guarantee), the pair's values stay in the exact
 * int16 range and the batch holds at least 32768 pairs.  Other unbanded pairs with 16-bit cells in
 * the exact range, fewer than 1024 columns and at most 4096 rows, in batches of at least 4096
 * pairs, run the packed 16-bit warp kernel (two strips per lane, 4-bit trace; equality scoring
 * needs alphabet_size 1..8 there too); the remaining unbanded pairs run the 32-bit warp kernel,
 * banded pairs one thread per pair. */
enum {
    GBA_FLAG_GENERAL_KERNEL = 1,   /* force the one-pair-per-thread 32-bit kernel */
    GBA_FLAG_STRIP16 = 2,          /* packed kernel with 16-row strips instead of 32 */
    GBA_FLAG_PLAIN_BUCKETS = 4,    /* the plain GPU form (comparison baseline): the kernels the
                                      automatic routing picks, launched once per 8-residue
                                      bucket of max(|H|, |V|), input order inside a bucket, no
                                      split slots, default tiling, no graph; with
                                      GBA_FLAG_GENERAL_KERNEL the one-pair-per-thread kernel */
    GBA_FLAG_NO_GRAPH = 8,         /* launch kernels directly instead of replaying a CUDA graph */
    GBA_FLAG_AUTOTUNE = 16,        /* time the packed kernel's tiling variants on the first run
                                      of a plan and remember the fastest per batch shape */
    GBA_FLAG_PACKED = 32,          /* use the packed kernel for eligible pairs even in batches
                                      too small to fill the GPU with it */
    GBA_FLAG_PACKED_SPLIT = 64,    /* packed kernel: every pair runs as a split slot (one pair per
                                      thread, two strips at once) instead of only the longest */
    GBA_FLAG_PACKED_NO_SPLIT = 128,/* packed kernel: no split slots (two pairs per thread only) */
    GBA_FLAG_NO_WARP16 = 256,      /* pairs the packed 16-bit warp kernel would take run on the
                                      32-bit warp kernel instead */
    GBA_FLAG_WARP16 = 512,         /* packed 16-bit warp kernel for eligible pairs even in batches
                                      smaller than 4096 pairs */
    /* Not a kernel selection: GBA_ALIGN_EXTEND's X-drop terminator, threshold gba_params.xdrop. */
    GBA_FLAG_XDROP = 1024
};

/* A batch: concatenated residue codes with n+1 offsets for each side. */
typedef struct {
    int64_t num_pairs;
    const uint8_t *seq_h;
    const int64_t *off_h;      /* num_pairs + 1 entries (2 when h_shared) */
    const uint8_t *seq_v;
    const int64_t *off_v;      /* num_pairs + 1 entries */
    int32_t h_shared;          /* 1: every pair uses the single H sequence off_h[0]..off_h[1] */
    int32_t reserved;
} gba_batch;

typedef struct {
    uint32_t h_begin, v_begin, length, type;   /* TraceSegment_<unsigned, unsigned> */
} gba_segment;

/* Results.  Any pointer may be NULL when its output was not requested. */
typedef struct {
    int32_t *score;            /* [num_pairs] */
    int32_t *end_h, *end_v;    /* [num_pairs] best cell (column, row) */
    int32_t *begin_h, *begin_v;/* [num_pairs] alignment begin (GBA_OUT_SEGMENTS) */
    int32_t *pair_status;      /* [num_pairs] GBA_PAIR_* */
    /* Trace segments in the reference's order (traceback order, last segment = alignment
     * begin).  Pair k owns segments[segment_offsets[k] .. segment_offsets[k+1]). */
    gba_segment *segments;
    int64_t segment_capacity;
    int64_t *segment_offsets;  /* [num_pairs + 1] */
    /* CIGAR as BAM-style uint32 (length << 4 | op), op index into "MIDNSHP=X"; the
     * character string of getCigarString (bam_io/cigar.h:261-339), D runs >= 20 as N. */
    uint32_t *cigar;
    int64_t cigar_capacity;
    int64_t *cigar_offsets;    /* [num_pairs + 1] */
} gba_result;

/* Context: device, stream, cached device buffers, HBM budget. */
GBA_API int gba_create(gba_context **ctx, const gba_config *cfg);
GBA_API int gba_destroy(gba_context *ctx);
GBA_API const char *gba_status_string(int status);
/* Copies the last error message of this context (CUDA error text etc.). */
GBA_API int gba_last_error(gba_context *ctx, char *buf, size_t size);

/* Aligns a batch held in HOST memory and writes host results; blocks until done.
 * This is the call the reference-facing shim makes. */
GBA_API int gba_align_batch(gba_context *ctx, const gba_params *params, const gba_batch *batch,
                            gba_result *result);

/* --- Device-resident path (inputs already in HBM) ------------------------------------ */

typedef struct gba_plan gba_plan;

/* Builds a launch plan from HOST offsets (lengths, binning, scratch sizes) and uploads it.
 * The plan stays valid for any device batch with the same offsets. */
GBA_API int gba_plan_create(gba_context *ctx, const gba_params *params, const gba_batch *host_batch,
                            gba_plan **plan);
GBA_API int gba_plan_destroy(gba_context *ctx, gba_plan *plan);
/* Runs a plan on DEVICE inputs/outputs (pointers in dev_batch / dev_result are device
 * pointers; segment/cigar outputs are written into the plan's device buffers and can be
 * fetched with gba_plan_fetch).  Asynchronous on the context stream. */
GBA_API int gba_plan_execute(gba_context *ctx, gba_plan *plan, const gba_batch *dev_batch,
                             gba_result *dev_result);
/* Copies a plan's segment/CIGAR outputs to host buffers (synchronous). */
GBA_API int gba_plan_fetch(gba_context *ctx, gba_plan *plan, gba_result *host_result);

/* --- Memory, stream and timing helpers (so hosts need no other CUDA binding) ---------- */
GBA_API int gba_device_alloc(gba_context *ctx, void **ptr, size_t bytes);
GBA_API int gba_device_free(gba_context *ctx, void *ptr);
GBA_API int gba_host_alloc(gba_context *ctx, void **ptr, size_t bytes);   /* pinned */
GBA_API int gba_host_free(gba_context *ctx, void *ptr);
GBA_API int gba_copy_to_device(gba_context *ctx, void *dst, const void *src, size_t bytes);
GBA_API int gba_copy_to_host(gba_context *ctx, void *dst, const void *src, size_t bytes);
GBA_API int gba_synchronize(gba_context *ctx);
/* CUDA events on the context stream: time between the two marks in milliseconds. */
GBA_API int gba_timer_start(gba_context *ctx);
GBA_API int gba_timer_stop(gba_context *ctx, float *ms);

/* Statistics of the last batch: kernel time (CUDA events around the DP launch on the
 * context stream), launches, cells. */
typedef struct {
    float dp_kernel_ms;        /* DP kernel(s) */
    float traceback_kernel_ms; /* traceback + output kernels */
    int32_t kernel_launches;   /* kernels this library launched for the batch */
    int64_t cells;             /* algorithmic cells: sum m*n (in-band cells when banded) */
    int64_t trace_bytes;       /* trace matrix bytes written */
    int32_t tile_rows;         /* packed kernel: rows per register strip (0 = not used);
                                  gba_extend_alignments: rows per band (8 x lanes per task) */
    int32_t tile_min_blocks;   /* packed kernel: minimum resident blocks per SM */
    float host_plan_ms;        /* gba_align_batch: host planning time */
    float call_ms;             /* gba_align_batch: whole call, wall clock */
    int32_t dp_kernels;        /* GBA_KERNEL_* bits: the DP kernels the run launched */
    int32_t seed_ring;         /* gba_extend_seeds, GappedXDrop: shared-memory ring slots per seed
                                  (0: every seed ran on the global-memory fallback) */
    int64_t seed_fallbacks;    /* gba_extend_seeds: seeds re-run on the fallback kernel */
} gba_stats;

/* DP kernels (gba_stats.dp_kernels). */
enum {
    GBA_KERNEL_STRIP = 1,      /* one pair per thread, 16-row register strips, int32 */
    GBA_KERNEL_PACKED = 2,     /* two pairs per thread, int16x2 DPX */
    GBA_KERNEL_WARP = 4,       /* bands of 256 rows, one warp per band, anti-diagonal front */
    GBA_KERNEL_BANDED = 8,     /* banded DP, one pair per thread */
    GBA_KERNEL_WARP16 = 16,    /* bands of 64 strips, one warp per band, int16x2 DPX, 4-bit trace */
    GBA_KERNEL_DYNAMIC = 32    /* DynamicGaps cells, one pair per thread */
};
GBA_API int gba_get_stats(gba_context *ctx, gba_stats *stats);

/* Measures the device's 32-bit integer add/max rate (tera-ops per second) with a short
 * kernel.  No counterpart in the reference: it is the roofline denominator that the
 * benchmark reports the DP kernels against. */
GBA_API int gba_measure_int_peak(gba_context *ctx, double *tops);

/* --- Serving loop ---------------------------------------------------------------------
 * No counterpart in the reference, which only has the blocking batch call.  A server owns a
 * worker thread and `streams` batch slots, each with its own CUDA stream and device buffers
 * that stay allocated between batches.  gba_server_submit queues one pair (its codes are
 * copied); whenever a slot is free, the worker launches everything queued, in arrival order,
 * up to max_batch_pairs pairs and as long as the device bytes of all batches in flight stay
 * within hbm_budget_bytes, so requests that arrive while other batches run on the GPU are
 * admitted as slots and memory free up, and their work overlaps on the device.  Finished
 * batches are found by event query; gba_server_poll hands out their results.  Every request
 * runs the same kernels as gba_align_batch: its result does not depend on which other
 * requests share its batch.  All server calls are thread-safe. */
typedef struct gba_server gba_server;

typedef struct {
    int32_t device;
    int32_t streams;            /* batch slots in flight, 1..16 */
    int64_t max_batch_pairs;    /* cap on the pairs of one launched batch (>= 1) */
    int64_t hbm_budget_bytes;   /* admission bound on the device bytes of the batches in flight
                                   (0 = none); a request that alone exceeds it is refused */
} gba_server_config;

typedef struct {
    uint64_t tag;               /* the caller's tag from gba_server_submit */
    int32_t score, end_h, end_v;
    int32_t begin_h, begin_v;   /* with GBA_OUT_SEGMENTS */
    int32_t status;             /* GBA_PAIR_* */
    int32_t n_segments;         /* segments of this request in the poll's segment array */
    int64_t segment_offset;     /* first of them */
    double t_submit, t_done;    /* gba_clock_seconds() at submit / when its batch was found done */
} gba_request_result;

typedef struct {
    int64_t submitted, completed, pending;  /* pending: queued, not launched yet */
    int64_t batches;                        /* batches launched */
    int64_t cells;                          /* DP cells of launched batches */
    int64_t hbm_in_flight;                  /* device bytes of the batches in flight now */
    int64_t hbm_in_flight_peak;             /* largest value hbm_in_flight took */
} gba_server_stats;

/* params: the scoring scheme and outputs of every request (no CIGAR); copied. */
GBA_API int gba_server_create(gba_server **out, const gba_server_config *cfg, const gba_params *params);
/* Queues pair (h[0..m), v[0..n)).  GBA_EBUDGET when the pair alone needs more device bytes
 * than the budget. */
GBA_API int gba_server_submit(gba_server *srv, uint64_t tag, const uint8_t *h, int64_t m, const uint8_t *v,
                              int64_t n);
/* Moves up to max_results finished requests into results (completion order) and their
 * segments into segments[0..segment_capacity); *num_results / *num_segments say how many.
 * Stops early at a request whose segments no longer fit (GBA_ECAPACITY if even the first one
 * does not).  Does not wait. */
GBA_API int gba_server_poll(gba_server *srv, gba_request_result *results, int64_t max_results,
                            gba_segment *segments, int64_t segment_capacity, int64_t *num_results,
                            int64_t *num_segments);
GBA_API int gba_server_get_stats(gba_server *srv, gba_server_stats *stats);
/* Load replay (no counterpart in the reference): submits pair k of `requests` (host layout of
 * gba_batch, h_shared allowed) with tag first_tag + k at at_seconds[k] after the call starts,
 * waiting between submits on the calling thread; returns once all are submitted (the first
 * failing submit's status otherwise).  For driving the server with a recorded or synthetic
 * arrival process from native code. */
GBA_API int gba_server_submit_schedule(gba_server *srv, const gba_batch *requests, const double *at_seconds,
                                       uint64_t first_tag);
GBA_API int gba_server_last_error(gba_server *srv, char *buf, size_t size);
/* Stops the worker after the batches in flight finish; unpolled results are dropped. */
GBA_API int gba_server_destroy(gba_server *srv);
/* Monotonic clock in seconds (the clock of t_submit / t_done). */
GBA_API double gba_clock_seconds(void);

/* --- Allocation-free scores ------------------------------------------------------------
 * No counterpart in the reference.  For callers that cannot allocate device memory on the
 * call path: hosts whose device memory all comes from their own pool (a database or plugin
 * host that hands out buffers) and latency-bound request loops that keep cudaMalloc/cudaFree
 * -- which can synchronize the device and take unbounded time -- out of their requests.
 * The caller passes DEVICE pointers for inputs and outputs; the call needs no gba_context and
 * makes no allocation of any kind.  The DP's scratch is a static device array of
 * GBA_NOALLOC_SCRATCH_BYTES that every GPU loading the library holds until exit; one warp of
 * lanes needs 32 * (max_h_len + 1) * 8 bytes of it, and a max_h_len that does not fit is
 * refused with GBA_ECAPACITY.  Pairs longer than max_h_len are not computed and come back
 * with score numeric_limits<T>::min() and GBA_PAIR_SKIPPED; empty pairs get numeric min and
 * GBA_PAIR_INVALID as in gba_align_batch.  Scores and end positions only (no band, no
 * traceback); for every pair within max_h_len the score, end positions and status equal
 * gba_align_batch's.
 * Set-up: the first call on a device looks up the array's device address.  Under CUDA's lazy
 * module loading (the default) that is also when the array's memory is committed on the device,
 * and the first call with a given scoring shape (gap model, mode, table or not) loads that shape's
 * kernel code, so first calls may allocate and synchronize: make one call per shape at start-up
 * (or run with CUDA_MODULE_LOADING=EAGER), before any stream capture and before a host pool takes
 * the GPU's memory; repeated calls allocate nothing.  All
 * calls share the array: calls that overlap on the GPU race and must be serialized by the
 * caller.  An error already pending on the calling thread is left in place and reported as
 * GBA_ECUDA without a launch.  Asynchronous on `stream` (a cudaStream_t; NULL = legacy default
 * stream). */
#define GBA_NOALLOC_SCRATCH_BYTES (64u << 20)

typedef struct {
    int64_t num_pairs;
    const uint8_t *seq_h;      /* device: concatenated H codes */
    const int64_t *off_h;      /* device: num_pairs + 1 offsets */
    const uint8_t *seq_v;      /* device */
    const int64_t *off_v;      /* device */
    int32_t max_h_len;         /* caller's bound on every |H| in the batch */
    int32_t reserved;
} gba_noalloc_batch;

GBA_API int gba_align_score_noalloc(const gba_params *params, const gba_noalloc_batch *batch,
                                    int32_t *score, int32_t *end_h, int32_t *end_v,
                                    int32_t *pair_status, void *stream);

/* --- Seed extension ---------------------------------------------------------------------
 * extendSeed(seed, database, query, direction, MatchExtend) and
 * extendSeed(seed, database, query, direction, scoringScheme, scoreDropOff,
 *            UnGappedXDrop | GappedXDrop)
 * (seeds/seeds_extension.h:181-218, 283-360, 780-835) over a batch of Seed<Simple> seeds, one
 * call for the whole batch.  H is the database (horizontal) and V the query (vertical) side,
 * as in the reference.  Each seed grows in place exactly as the reference's call grows it:
 * begin/end positions in H and V and the lower/upper diagonals (H - V) its traces touched.
 * Scores are Score<int, Simple>(match, mismatch, gap) or an alphabet_size^2 matrix
 * (Score<int, ScoreMatrix<...>> with linear gap `gap`).  GappedXDrop requires gap < 0 (the
 * reference asserts gap open == extend < 0) and every substitution score >= gap: below that the
 * reference adds a substitution score to its `undefined` sentinel INT_MIN - gap and overflows
 * int, so such schemes are refused with GBA_EUNSUPPORTED.  Gapped segments are limited to
 * 2^29 residues (the reference computes 2 * max(rows, cols) in int). */
enum { GBA_MATCH_EXTEND = 0, GBA_UNGAPPED_XDROP = 1, GBA_GAPPED_XDROP = 2 };
/* ExtensionDirection (seeds/seeds_extension.h:123-129). */
enum { GBA_EXTEND_NONE = 0, GBA_EXTEND_LEFT = 1, GBA_EXTEND_RIGHT = 2, GBA_EXTEND_BOTH = 3 };

/* Seed<Simple, DefaultSeedConfig> (seeds/seeds_seed_simple.h:78-132): positions are size_t,
 * diagonals signed, diagonal = H position - V position. */
typedef struct {
    int64_t begin_h, begin_v, end_h, end_v;
    int64_t lower_diagonal, upper_diagonal;
} gba_seed;

typedef struct {
    int32_t method;            /* GBA_MATCH_EXTEND / GBA_UNGAPPED_XDROP / GBA_GAPPED_XDROP */
    int32_t direction;         /* GBA_EXTEND_* */
    int32_t score_drop_off;    /* X of the x-drop methods; |X| < 2^30 */
    int32_t match, mismatch;   /* Score<int, Simple> (ignored with a matrix) */
    int32_t gap;               /* linear gap score */
    const int32_t *matrix;     /* optional host alphabet_size^2 table, row = first argument of score() */
    int32_t alphabet_size;     /* 1..32 with a matrix */
    int32_t reserved;
} gba_extend_params;

/* Sequences and seeds.  Seed k lies on database seed_h[k] and query seed_v[k] (NULL: on
 * database k / query k). */
typedef struct {
    int64_t num_h;
    const uint8_t *seq_h;      /* concatenated database codes */
    const int64_t *off_h;      /* num_h + 1 offsets */
    int64_t num_v;
    const uint8_t *seq_v;      /* concatenated query codes */
    const int64_t *off_v;      /* num_v + 1 offsets */
    int64_t num_seeds;
    const int32_t *seed_h, *seed_v;
    int64_t max_v_len;         /* gba_extend_seeds_device: a bound on every query length */
} gba_seed_batch;

/* Extends the seeds of a HOST batch in place (blocking).  scores: NULL or 2 per seed, the
 * return values of the gapped left/right extensions (0 for an empty side, INT_MIN - gap when
 * no cell stayed within the drop-off).  A seed outside its sequences fails the call with
 * GBA_EINVAL, as does an empty UnGappedXDrop seed at the end of a sequence, whose left walk
 * the reference starts past the end. */
GBA_API int gba_extend_seeds(gba_context *ctx, const gba_extend_params *params, const gba_seed_batch *batch,
                             gba_seed *seeds, int32_t *scores);
/* The same on DEVICE pointers (batch arrays, seeds, scores; params->matrix stays a host
 * pointer), asynchronous on the context stream; invalid seeds are left unchanged and reported
 * by the next gba_synchronize as GBA_EINVAL. */
GBA_API int gba_extend_seeds_device(gba_context *ctx, const gba_extend_params *params,
                                    const gba_seed_batch *dev_batch, gba_seed *dev_seeds, int32_t *dev_scores);

/* --- Alignment extension ------------------------------------------------------------------
 * extendAlignment(align, [origScore,] hSeq, vSeq, positions, direction, [lowerDiag, upperDiag,]
 * [xDrop,] scoreScheme) (align_extend/align_extend.h:211-372, 494-620) over a batch; origScore and
 * the aligned part's own gaps only enter the returned score, which the caller forms (the Python
 * and C++ mirrors do).  For alignment k the
 * aligned part spans hSeq[begin_h, end_h) / vSeq[begin_v, end_v) (positions from
 * seeds[k]; the alignment itself is the caller's).  The left side runs the AlignExtend DP on the
 * reversed prefixes when direction has LEFT and both begins are > 0, the right side on the
 * suffixes when direction has RIGHT and both ends are inside their sequences: a gap-initialised
 * first row and column, every cell tracked without a zero floor, traceback from the first
 * maximum to the origin, and with xdrop_on the X-drop terminator of
 * align_extend/dp_scout_xdrop.h (a column whose maximum lies xdrop or more below the best score
 * ends the DP after the next inner-column check).  The reference's return value is
 * left_score + the aligned part's score + right_score. */
typedef struct {
    int32_t direction;         /* GBA_EXTEND_LEFT / GBA_EXTEND_RIGHT / GBA_EXTEND_BOTH */
    int32_t xdrop_on, xdrop;   /* the xDrop argument */
    int32_t match, mismatch;   /* Score<int, Simple> (ignored with a matrix) */
    int32_t gap_open, gap_extend;   /* Gotoh iff open != extend, as the reference picks */
    const int32_t *matrix;     /* optional host alphabet_size^2 table (row = H residue) */
    int32_t alphabet_size;     /* 1..32 with a matrix */
    int32_t band_on;           /* 1: the (lowerDiag, upperDiag) overloads: both sides run the banded
                                  AlignExtend_ DP (GBA_ALIGN_EXTEND) with this band */
    int32_t band_lower, band_upper;
} gba_extend_align_params;

typedef struct {
    int32_t *left_score, *right_score;   /* [num_seeds]; 0 for a side that was not extended */
    /* TraceSegment_ lists in traceback order (last segment = the side's alignment begin): the
     * left side's in prefix coordinates (after the reference's _reversePartialTrace,
     * align_extend/align_extend.h:91-109), the right side's in suffix coordinates.  Alignment
     * k's left side owns segments[segment_offsets[2k] .. [2k+1]), its right side
     * [segment_offsets[2k+1] .. [2k+2]). */
    gba_segment *segments;
    int64_t segment_capacity;
    int64_t *segment_offsets;  /* [2 * num_seeds + 1] */
} gba_extend_align_result;

GBA_API int gba_extend_alignments(gba_context *ctx, const gba_extend_align_params *params,
                                  const gba_seed_batch *batch, const gba_seed *seeds,
                                  gba_extend_align_result *result);

/* --- Suboptimal local alignments (Waterman-Eggert) --------------------------------------------
 * The reference's LocalAlignmentEnumerator<Score, Unbanded> driven by nextLocalAlignment until it
 * returns false or max_count alignments were taken (align/local_alignment_enumeration_unbanded.h,
 * align/local_alignment_waterman_eggert_impl.h), for every pair of a batch: linear gaps (gap =
 * the scheme's gap extension score), the score matrix filled from the sequence ends, each
 * alignment traced forward from the largest remaining score, its residue pairs forbidden and the
 * matrix declumped before the next.  Pair k's alignment i (i < count[k]) has score
 * score[k * max_count + i] (getScore), clipped source positions [begin_h, end_h) / [begin_v,
 * end_v), and its columns as runs in alignment order in segments[segment_offsets[k * max_count +
 * i] .. segment_offsets[k * max_count + i + 1]) ({h_begin, v_begin, length, type}: a run starts at
 * the next residue of each row; the two rows of an alignment whose first column is a gap start
 * at different columns, each at its first residue, as the reference's rows do).  status[k] =
 * GBA_ENUM_UNDEFINED_NEXT when the enumeration stopped because the reference's next step is
 * undefined (after an alignment whose first column is a gap, its declumping walk runs past the
 * rows' first positions). */
typedef struct {
    int32_t match, mismatch;   /* Score<int, Simple> (ignored with a matrix) */
    int32_t gap;               /* scoreGapExtend: every gap column costs this */
    int32_t cutoff;            /* the enumerator's cutoff: cells below it never become alignment ends */
    const int32_t *matrix;     /* optional host alphabet_size^2 table (row = H residue) */
    int32_t alphabet_size;     /* 1..32 with a matrix */
    int32_t max_count;         /* alignments per pair, 1..65536 */
} gba_enum_params;

enum { GBA_ENUM_DONE = 0, GBA_ENUM_UNDEFINED_NEXT = 1 };

typedef struct {
    int32_t *count, *status;                        /* [num_pairs] */
    int32_t *score, *begin_h, *end_h, *begin_v, *end_v;   /* [num_pairs * max_count] */
    gba_segment *segments;
    int64_t segment_capacity;
    int64_t *segment_offsets;                       /* [num_pairs * max_count + 1] */
} gba_enum_result;

GBA_API int gba_local_enumerate(gba_context *ctx, const gba_enum_params *params, const gba_batch *batch,
                                gba_enum_result *result);

/* The reference's LocalAlignmentEnumerator<Score, Banded>(score, lowerDiag, upperDiag, cutoff)
 * driven by nextLocalAlignment (align/local_alignment_enumeration_banded.h:56-121,
 * align/local_alignment_banded_waterman_eggert_impl.h): the matrix kept in band storage over the
 * diagonals lower_diag .. upper_diag (column - row), filled from the sequence begins, each
 * alignment traced backward from the largest remaining score, its diagonal cells forbidden and the
 * rows below re-filled while values change.  Same parameters and result layout as
 * gba_local_enumerate; status[k] = GBA_ENUM_UNDEFINED_NEXT where the reference's walk reads outside
 * its band storage or a character outside a sequence.  A band that does not cross the matrix
 * (lower_diag >= len(H) or upper_diag <= -len(V)) gives no alignment; the reference crashes there. */
GBA_API int gba_local_enumerate_banded(gba_context *ctx, const gba_enum_params *params, int32_t lower_diag,
                                       int32_t upper_diag, const gba_batch *batch, gba_enum_result *result);

/* --- Banded chain alignment ------------------------------------------------------------------
 * bandedChainAlignment(align, seedChain, scoreAnchor, scoreGap, AlignConfig, bandExtension)
 * (seeds/banded_chain_alignment.h:184-214) for every pair of a batch, each with its own seed
 * chain: the rectangle before the first anchor, a band of the anchor's diagonals widened by
 * bandExtension around each anchor and the rectangle to the next one, and the rectangle to the
 * matrix end, each grid started from the cells the previous grid's traceback reached; linear or
 * affine gaps (affine when either scheme's gap open differs from its gap extension).  Per pair:
 * the score (numeric_limits<int>::min() for an empty chain), the first trace of the reference's
 * trace set as TraceSegment_ runs in the reference's order (the rows _adaptTraceSegmentsTo builds
 * from them), and how many co-optimal traces the set held.  status[k]: GBA_CHAIN_NO_GLUE where
 * the reference throws std::logic_error (two grids' traces share no cell); GBA_CHAIN_UNDEFINED
 * where its behaviour is undefined (a grid past the sequences, an index past its vectors);
 * GBA_CHAIN_CAPACITY when more than max_traces co-optimal traces were open at once. */
typedef struct {
    int32_t match, mismatch, gap_extend, gap_open;   /* Score<int, Simple>(match, mismatch, ext, open) */
} gba_simple_score;

typedef struct {
    gba_simple_score anchor;   /* scores in the bands around the anchors */
    gba_simple_score gap;      /* scores in the rectangles between them */
    int32_t free_ends;         /* GBA_FREE_* (AlignConfig<TOP, LEFT, RIGHT, BOTTOM>) */
    int32_t band_extension;    /* >= 1; the reference's default is 15 */
    int32_t max_traces;        /* co-optimal traces kept per pair, 1..32; 0: 8, and the pairs that need
                                  more run again with 32 */
} gba_chain_params;

typedef struct {
    const int32_t *seeds;            /* host: 4 per seed (beginH, beginV, endH, endV of Seed<Simple>) */
    const int64_t *seed_offsets;     /* num_pairs + 1: pair k's chain is seeds [off[k], off[k+1]) */
} gba_chain_seeds;

enum { GBA_CHAIN_OK = 0, GBA_CHAIN_NO_GLUE = 1, GBA_CHAIN_UNDEFINED = 2, GBA_CHAIN_CAPACITY = 3 };

typedef struct {
    int32_t *score, *status, *num_traces;   /* [num_pairs] */
    gba_segment *segments;                  /* pair k: segments[segment_offsets[k] .. [k+1]) */
    int64_t segment_capacity;
    int64_t *segment_offsets;               /* [num_pairs + 1] */
} gba_chain_result;

GBA_API int gba_banded_chain(gba_context *ctx, const gba_chain_params *params, const gba_batch *batch,
                             const gba_chain_seeds *seeds, gba_chain_result *result);

/* --- Packed input ---------------------------------------------------------------------------
 * String<TValue, Packed<>> (sequence/string_packed.h) as the engine's input, uploaded as is: the
 * host string of a packed string is a 64-bit length word followed by data words, each holding
 * N = 64 / BitsPerValue values with the first one in the most significant used bits.  The words
 * cross to the device (4x fewer bytes than codes for Dna, 2.7x for Dna5) and are unpacked there. */
typedef struct {
    int64_t num;               /* packed strings */
    const uint64_t *words;     /* the strings' host words back to back (an empty string has none) */
    const int64_t *word_off;   /* num + 1 offsets into words */
    int32_t bits_per_value;    /* BitsPerValue<TValue>: 2 Dna, 3 Dna5, 5 AminoAcid */
    int32_t reserved;
} gba_packed_set;

/* gba_align_batch on packed sets: pair k is (h[k], v[k]), or (h[0], v[k]) with h_shared. */
GBA_API int gba_align_packed(gba_context *ctx, const gba_params *params, const gba_packed_set *h,
                             const gba_packed_set *v, int32_t h_shared, gba_result *result);

/* --- SAM output -----------------------------------------------------------------------------
 * The SAM lines of alignment records as the reference's SAM writer writes a BamAlignmentRecord
 * (bam_io/write_sam.h:126-217: QNAME, FLAG, RNAME or '*', POS + 1, MAPQ, CIGAR or '*', RNEXT as
 * '*', '=' or a name, PNEXT + 1, TLEN or '0', SEQ or '*', QUAL or '*', then the tags as
 * appendTagsBamToSam writes them: bam_io/bam_sam_conversion.h:250-360), formatted on the device.  Positions are 0-based with -1 for none, as in BamAlignmentRecord; the CIGAR is the
 * BAM-packed form of gba_result.cigar; SEQ is residue codes turned into seq_letters[code]. */
typedef struct {
    int64_t num;                               /* records */
    const char *qname;                         /* names back to back */
    const int64_t *qname_off;                  /* num + 1 */
    const uint16_t *flag;
    const int32_t *ref_id, *pos;               /* rID, beginPos */
    const uint8_t *mapq;
    const uint32_t *cigar;                     /* length << 4 | op index into "MIDNSHP=X" */
    const int64_t *cigar_off;                  /* num + 1 */
    const int32_t *next_ref_id, *next_pos, *tlen;
    const uint8_t *seq;                        /* residue codes */
    const int64_t *seq_off;                    /* num + 1 */
    const char *seq_letters;                   /* 32 letters, e.g. "ACGTN" padded */
    const char *qual;                          /* qualities back to back, or NULL: every QUAL '*' */
    const int64_t *qual_off;                   /* num + 1, or NULL */
    const char *contig_names;                  /* the context's contig names back to back */
    const int64_t *contig_off;                 /* num_contigs + 1 */
    int64_t num_contigs;
    /* BamAlignmentRecord.tags: each record's tags in BAM form (two name characters, a type
     * character, the value), back to back; NULL tags_off: no record has tags.  SAM writes them as
     * NAME:TYPE:VALUE separated by tabs (c, s, i, C, S, I as 'i'; Z and H up to their NUL; B arrays
     * as the element type and ","-prefixed values; float values (f, B:f) as printf "%g" of the
     * value, as the reference's appendNumber(float) writes them); malformed tags are GBA_EINVAL
     * there.  BAM appends the bytes as they are. */
    const char *tags;
    const int64_t *tags_off;                   /* num + 1, or NULL */
} gba_sam_records;

/* Writes the lines to out and their offsets to line_off[0..num] (line k is out[line_off[k] ..
 * line_off[k+1]), newline included); GBA_ECAPACITY (with line_off filled) if capacity is too
 * small. */
GBA_API int gba_format_sam(gba_context *ctx, const gba_sam_records *records, char *out, int64_t capacity,
                           int64_t *line_off);

/* --- FASTA / FASTQ input -------------------------------------------------------------------
 * Every record of a FASTA or FASTQ text, as the loop
 *     while (!atEnd(iter)) readRecord(id, seq, qual, iter, Fasta | Fastq);
 * reads them (seq_io/fasta_fastq.h:265-283 FASTA, :354-392 FASTQ) with seq a String<Dna>,
 * String<Dna5> or String<AminoAcid> (alphabet 4, 5, 27) and qual a CharString, into the layout
 * gba_align_batch takes: record k's residue codes are codes[seq_off[k], seq_off[k+1]), its id is
 * text[id_begin[k], id_end[k]) and its FASTQ qualities quals[seq_off[k], qual_end[k]) (FASTA:
 * qual_end[k] = seq_off[k]).  Whitespace inside a sequence is skipped; any other character
 * outside the alphabet (IsInAlphabet, stream/tokenization.h:51-63) is GBA_EPARSE with
 * error_offset at it, as the reference's ParseError; a non-empty text without a record start is
 * GBA_EPARSE with error_offset = length (UnexpectedEnd).  When a capacity is too small the call
 * returns GBA_ECAPACITY with num and residues set.  gba_read_fasta parses on the device;
 * gba_read_fastq parses on the host (ctx may be NULL), texts of 4 MB and more with the host's
 * threads: speculative record starts per slice, each confirmed by the previous slice's reading
 * ending on it, else one sequential reading (results are always the sequential ones). */
typedef struct {
    int64_t record_capacity;   /* entries of id_begin / id_end / qual_end (>= num) and seq_off (>= num + 1) */
    int64_t residue_capacity;  /* bytes of codes (and quals) */
    int64_t *id_begin, *id_end;
    int64_t *seq_off;
    int64_t *qual_end;         /* may be NULL */
    uint8_t *codes;
    char *quals;               /* FASTQ qualities; may be NULL */
    int64_t num;               /* out: records */
    int64_t residues;          /* out: residues of all records */
    int64_t error_offset;      /* out: text offset of a GBA_EPARSE, else -1 */
} gba_seq_records;

/* BAM records of the same fields: write(target, record, context, Bam()) for a BamAlignmentRecord
 * (bam_io/write_bam.h:100-271), the uncompressed record blocks (block_size, the
 * 32-byte core with bin = reg2bin(beginPos, beginPos + max(1, length in the reference)), name and
 * NUL, CIGAR words, Iupac sequence two codes per byte, qualities minus '!' or 0xFF, the tag
 * bytes), formatted on the device; rec_off[num + 1] gets each record's byte offset.  Names of more than 254 characters,
 * more than 65535 CIGAR operations and more qualities than residues are GBA_EINVAL (the core's
 * fields cannot hold them; the reference asserts on the last).  gba_bgzf_compress writes the blocks
 * as a BGZF file. */
GBA_API int gba_format_bam(gba_context *ctx, const gba_sam_records *records, char *out, int64_t capacity,
                           int64_t *rec_off);

/* BGZF compression of a byte stream (the reference's BgzfFile stream under BamFileOut,
 * stream/stream_compressor.h:60-130, 325-375): pages of 65,505 input bytes, each one gzip member
 * with the BGZF header ("BC" extra field = member size - 1), raw deflate data, CRC-32 and input
 * size, compressed on the device; with eof_marker the 28-byte empty member follows.  The member
 * partition, headers, CRC-32s and sizes are the reference's; the deflate data is this engine's
 * (greedy LZ77 with fixed Huffman codes, or a stored block), so each member inflates to the same
 * page while the compressed bytes differ from zlib's.  *out_len gets the size; GBA_ECAPACITY when
 * capacity is smaller. */
GBA_API int gba_bgzf_compress(gba_context *ctx, const uint8_t *data, int64_t length, int32_t eof_marker, uint8_t *out,
                              int64_t capacity, int64_t *out_len);

GBA_API int gba_read_fasta(gba_context *ctx, const char *text, int64_t length, int32_t alphabet,
                           gba_seq_records *records);
GBA_API int gba_read_fastq(gba_context *ctx, const char *text, int64_t length, int32_t alphabet,
                           gba_seq_records *records);

/* gba_align_batch on the records of two FASTA texts: pair k is (record k of text_h, record k of
 * text_v), or (the single record of text_h, record k of text_v) with h_shared.  Both texts are read
 * on the device as gba_read_fasta reads them and aligned from the codes left in HBM (only the record
 * offsets come back to the host, for the plan).  *num_pairs = the records of text_v; the result's
 * per-pair arrays hold pair_capacity entries (GBA_ECAPACITY when fewer). */
GBA_API int gba_align_fasta(gba_context *ctx, const gba_params *params, const char *text_h, int64_t len_h,
                            const char *text_v, int64_t len_v, int32_t alphabet, int32_t h_shared,
                            int64_t pair_capacity, int64_t *num_pairs, gba_result *result);

#ifdef __cplusplus
}
#endif
#endif
