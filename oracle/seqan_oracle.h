/*
 * seqan_oracle.h -- CPU restatement of SeqAn 2's pairwise DP (test infrastructure only).
 *
 * This header and seqan_oracle.c are the CHECKER for the GPU engine.  Only tests/,
 * __graft_entry__.smoke() and bench.py's CPU-baseline leg may load the oracle.  The
 * product path (seqan_gb300/) never links or calls it.
 *
 * Parity is pinned against the reference compiled from its own headers (oracle/ref/,
 * built into oracle/_ref/) and against golden fixtures generated from it
 * (tests/golden/).
 */
#ifndef SEQAN_ORACLE_H_
#define SEQAN_ORACLE_H_

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* AlignConfig<TOP, LEFT, RIGHT, BOTTOM> bits (align/align_config.h:52-94). */
enum {
    ORC_FREE_TOP = 1,     /* free first row    (DPFirstRow)    */
    ORC_FREE_LEFT = 2,    /* free first column (DPFirstColumn) */
    ORC_FREE_RIGHT = 4,   /* free last column  (DPLastColumn)  */
    ORC_FREE_BOTTOM = 8   /* free last row     (DPLastRow)     */
};

/* ORC_EXTEND: the DP of extendAlignment (align_extend/align_extend.h:115-206): AlignExtend_
 * profile (align_extend/align_extend_base.h), i.e. a gap-initialised first row and column, every
 * cell tracked without a zero floor, traceback to (0, 0) with no tail; unbanded, or banded
 * (the lowerDiag / upperDiag overloads) with the free last row and column of the profile. */
enum { ORC_GLOBAL = 0, ORC_LOCAL = 1, ORC_EXTEND = 2 };
enum { ORC_LINEAR = 0, ORC_AFFINE = 1, ORC_DYNAMIC = 2 };

/* TraceSegment_ direction values (align/dp_profile.h:121-135). */
enum { ORC_SEG_DIAGONAL = 1, ORC_SEG_HORIZONTAL = 2, ORC_SEG_VERTICAL = 4 };

typedef struct {
    int32_t mode;           /* ORC_GLOBAL / ORC_LOCAL / ORC_EXTEND */
    int32_t gap_model;      /* ORC_LINEAR / ORC_AFFINE / ORC_DYNAMIC (DPCell_<T, DynamicGaps>) */
    int32_t free_ends;      /* ORC_FREE_* bits, ignored for local (all free) */
    int32_t band_on;        /* 0 / 1 */
    int32_t band_lower;     /* lower diagonal, col - row convention */
    int32_t band_upper;
    int32_t match, mismatch, gap_open, gap_extend;
    const int32_t *matrix;  /* alphabet_size^2 substitution table (row = H code) or NULL */
    int32_t alphabet_size;
    int32_t score_bits;     /* 16 or 32: cell width; 16 wraps like SeqAn's int16 SIMD lanes */
    int32_t traceback;      /* 0 = score only, 1 = trace segments */
    int32_t xdrop_on;       /* ORC_EXTEND: the X-drop terminator (align_extend/dp_scout_xdrop.h) */
    int32_t xdrop;
    int32_t trace4;         /* 1: pass every trace value through the 4-bit code (orc_trace4_encode /
                               orc_trace4_decode) before the traceback, to check that 4 bits per
                               cell keep every traceback decision */
} orc_params;

/* The 4-bit trace code: bits 0-1 the source of S (0 none, 1 diagonal, 2 vertical = MAX_FROM_V,
 * 3 horizontal = MAX_FROM_H), bit 2 "E opened" (H_OPEN without H), bit 3 "F opened" (V_OPEN
 * without V).  Decoding gives back the reference's TraceBitMap_ byte of every inner cell; a cell
 * that lacks an open/extend pair (borders, band edges) decodes with "extend" for it. */
uint8_t orc_trace4_encode(uint8_t tv);
uint8_t orc_trace4_decode(uint8_t code, int32_t affine);

typedef struct {
    uint32_t h_begin, v_begin, length, type;  /* TraceSegment_<unsigned, unsigned> */
} orc_segment;

typedef struct {
    int32_t score;
    int32_t end_h, end_v;      /* coordinates of the best (traceback start) cell */
    int32_t begin_h, begin_v;  /* alignment begin (first segment in alignment order) */
    int32_t n_segments;        /* -1 if the segment buffer was too small */
    int32_t valid;             /* 0 if _isValidDPSettings failed (score = numeric min) */
} orc_result;

/* One pair.  segs may be NULL when traceback == 0. */
int orc_align_pair(const orc_params *p,
                   const uint8_t *h, int32_t m,
                   const uint8_t *v, int32_t n,
                   orc_result *out, orc_segment *segs, int32_t seg_cap);

/* A batch over concatenated code buffers (offsets have n_pairs + 1 entries).  Segments
 * of pair k go to segs[seg_off[k] .. seg_off[k+1]) where the caller sized each slot as
 * m + n + 4.  Runs with `threads` OpenMP threads (<= 0: all). */
int orc_align_batch(const orc_params *p, int64_t n_pairs,
                    const uint8_t *seq_h, const int64_t *off_h,
                    const uint8_t *seq_v, const int64_t *off_v,
                    orc_result *out, orc_segment *segs, const int64_t *seg_off,
                    int32_t threads);

/* ---- Seed extension (seeds/seeds_extension.h) ---------------------------------------
 * Seed<Simple>: positions in H (the "database") and V (the "query"), diagonals = H - V.
 * extendSeed(seed, database, query, direction, Score<int, Simple|ScoreMatrix>, scoreDropOff,
 * UnGappedXDrop | GappedXDrop) restated for int scores (TScoreValue = int, positions size_t,
 * diagonals signed).  The gapped form needs gap open == extend (linear) and, for defined
 * behaviour of the reference's int arithmetic, every substitution score >= the gap score. */
enum { ORC_EXTEND_LEFT = 1, ORC_EXTEND_RIGHT = 2, ORC_EXTEND_BOTH = 3 };
enum { ORC_MATCH_EXTEND = 0, ORC_XDROP_UNGAPPED = 1, ORC_XDROP_GAPPED = 2 };

typedef struct {
    int64_t begin_h, begin_v, end_h, end_v;
    int64_t lower_diag, upper_diag;
} orc_seed;

typedef struct {
    int32_t method;            /* ORC_MATCH_EXTEND | ORC_XDROP_* */
    int32_t direction;         /* ORC_EXTEND_* */
    int32_t match, mismatch;   /* Score<int, Simple> (ignored with a matrix) */
    int32_t gap;               /* linear gap score (open = extend) */
    int32_t xdrop;             /* scoreDropOff */
    const int32_t *matrix;     /* optional alphabet^2 table, row = first argument of score() */
    int32_t alphabet_size;
} orc_xdrop_params;

/* Extends one seed in place; the scores of the gapped extensions (left, right; 0 when that side
 * is empty, INT_MIN when nothing was defined) go to xscore[0..1] when non-NULL. */
int orc_extend_seed(const orc_xdrop_params *p, orc_seed *seed, const uint8_t *db, int64_t m,
                    const uint8_t *q, int64_t n, int32_t *xscore);

/* A batch of seeds over databases H and queries V given as concatenated codes + offsets; seed i
 * lies on H[seed_h[i]] and V[seed_v[i]] (NULL: index i).  xscores: NULL or 2 per seed.
 * threads <= 0: all. */
int orc_extend_seeds(const orc_xdrop_params *p, int64_t n_h, const uint8_t *seq_h, const int64_t *off_h,
                     int64_t n_v, const uint8_t *seq_v, const int64_t *off_v, int64_t n_seeds,
                     const int32_t *seed_h, const int32_t *seed_v, orc_seed *seeds, int32_t *xscores,
                     int32_t threads);

/* SAM lines of BamAlignmentRecord fields (bam_io/write_sam.h:126-217): record k's fields as in
 * the engine's gba_sam_records, its BAM tag bytes tags[toff[k], toff[k+1]) (toff NULL: none)
 * written as appendTagsBamToSam writes them.  Returns the text length (the text is written when it
 * fits cap), or -1 (also for malformed tags and float tag values).  threads <= 0: all. */
int64_t orc_write_sam(int64_t n, const char *qname, const int64_t *qoff, const uint16_t *flag, const int32_t *rid,
                      const int32_t *pos, const uint8_t *mapq, const uint32_t *cigar, const int64_t *coff,
                      const int32_t *rnext, const int32_t *pnext, const int32_t *tlen, const uint8_t *seq,
                      const int64_t *soff, const char *letters, const char *qual, const int64_t *quoff,
                      int64_t ncontigs, const char *cnames, const int64_t *cnoff, const char *tags,
                      const int64_t *toff, char *out, int64_t cap, int32_t threads);

/* BAM records of the same fields (bam_io/write_bam.h:100-271): the uncompressed record blocks,
 * each record's tag bytes at its end.  Returns the byte length (the bytes are written when they
 * fit cap), or -1. */
int64_t orc_write_bam(int64_t n, const char *qname, const int64_t *qoff, const uint16_t *flag, const int32_t *rid,
                      const int32_t *pos, const uint8_t *mapq, const uint32_t *cigar, const int64_t *coff,
                      const int32_t *rnext, const int32_t *pnext, const int32_t *tlen, const uint8_t *seq,
                      const int64_t *soff, const char *letters, const char *qual, const int64_t *quoff,
                      const char *tags, const int64_t *toff, char *out, int64_t cap, int32_t threads);

/* Records of FASTA (format 0) or FASTQ (format 1) text as the reference's readRecord loop reads
 * them (seq_io/fasta_fastq.h:265-283, :354-392), alphabet 4 Dna, 5 Dna5, 27 AminoAcid: record k's
 * id is text[id_begin[k], id_end[k]), its residues codes[seq_off[k], seq_off[k+1]), its qualities
 * quals[seq_off[k], qual_end[k]).  Returns 0, -1 on ParseError, -2 on UnexpectedEnd (err_off =
 * the text offset), -3 when rec_cap (>= num + 1) or res_cap is too small; *num and *residues are
 * the counts read.  Sequential, as the reference's reader is. */
int32_t orc_read_records(int32_t format, int32_t alphabet, const char *text, int64_t n, int64_t rec_cap,
                         int64_t *id_begin, int64_t *id_end, int64_t *seq_off, int64_t *qual_end,
                         int64_t res_cap, uint8_t *codes, char *quals, int64_t *num, int64_t *residues,
                         int64_t *err_off);

/* Waterman-Eggert suboptimal local alignments: the reference's LocalAlignmentEnumerator<Score,
 * Unbanded> (align/local_alignment_enumeration_unbanded.h) driving _smithWaterman /
 * _smithWatermanGetNext (align/local_alignment_waterman_eggert_impl.h).  Linear gaps (the
 * scheme's gap extension score), the matrix filled from the sequence ends, every cell with a value
 * of at least cutoff pushed on the reference's binary heap (misc/priority_type_heap.h), each
 * alignment traced forward from the heap's current maximum, and the cells of the last alignment
 * forbidden and their neighbourhood recomputed ("declumping") before the next.  Up to max_count
 * alignments: scores[k] (the enumerator's getScore), begins[2k] / ends[2k] the clipped source
 * begin / end in H, begins[2k+1] / ends[2k+1] in V, and the alignment columns as TraceSegment_-like
 * runs in alignment order: segs[seg_off[k] .. seg_off[k+1]) of {h_begin, v_begin, length, type}.
 * Returns the number of alignments (or -1 when seg_cap is too small).  *undefined_next is set
 * when the enumeration stopped because the reference's next step is undefined: after an
 * alignment whose first column is a gap its two rows start at different steps, the declumping
 * walk back over it (which stops only where both rows start) runs on into the rows' unaligned
 * prefixes, and when it passes their first position the reference's iterators leave their
 * arrays. */
typedef struct {
    int32_t match, mismatch, gap;   /* Score<int, Simple>; gap = scoreGapExtend */
    const int32_t *matrix;          /* alphabet_size^2 table (row = H residue) or NULL */
    int32_t alphabet_size;
    int32_t cutoff;
} orc_we_params;

int32_t orc_waterman_eggert(const orc_we_params *p, const uint8_t *h, int32_t m, const uint8_t *v, int32_t n,
                            int32_t max_count, int32_t *scores, int32_t *begins, int32_t *ends,
                            orc_segment *segs, int64_t seg_cap, int64_t *seg_off, int32_t *undefined_next);

/* The banded enumerator LocalAlignmentEnumerator<Score, Banded>(score, lower, upper, cutoff)
 * (align/local_alignment_enumeration_banded.h, align/local_alignment_banded_waterman_eggert_impl.h),
 * outputs as orc_waterman_eggert: per alignment the score, the clipped source positions of the two
 * rows and the runs over the union of the rows' clipped views. */
int32_t orc_waterman_eggert_banded(const orc_we_params *p, int32_t lower, int32_t upper, const uint8_t *h, int32_t m,
                                   const uint8_t *v, int32_t n, int32_t max_count, int32_t *scores, int32_t *begins,
                                   int32_t *ends, orc_segment *segs, int64_t seg_cap, int64_t *seg_off,
                                   int32_t *undefined_next);

/* orc_align_pair with CompleteTrace (ties keep the trace bits of every source, no start-cell
 * correction): the DP of a banded chain's grid that spans the whole matrix. */
int orc_align_pair_complete(const orc_params *p,
                            const uint8_t *h, int32_t m,
                            const uint8_t *v, int32_t n,
                            orc_result *out, orc_segment *segs, int32_t seg_cap);

/* Banded chain alignment (bandedChainAlignment, seeds/banded_chain_alignment.h:184-214;
 * banded_chain_oracle.c).  Two Score<int, Simple> schemes -- the anchors' and the
 * gaps' -- the AlignConfig free-end bits and the band extension k.  seeds: n_seeds x (beginH,
 * beginV, endH, endV) of Seed<Simple> in chain order.  Outputs: the score (numeric min for an
 * empty chain), the first trace of the reference's trace set as TraceSegment_ runs (type =
 * 1 diagonal, 2 horizontal, 4 vertical) in the reference's order, and the number of traces.
 * Returns 0; 1 where the reference throws (no glue point between two grids' traces); 2 where its
 * behaviour is undefined (a grid or an index past its sequences or vectors); -1 when the trace
 * does not fit seg_cap. */
typedef struct {
    int32_t match, mismatch, gap_extend, gap_open;
} orc_simple_score;

typedef struct {
    orc_simple_score anchor, gap;
    int32_t free_ends;        /* ORC_FREE_* */
    int32_t band_extension;   /* k >= 1 */
} orc_chain_params;

int32_t orc_banded_chain(const orc_chain_params *p, const uint8_t *h, int32_t m, const uint8_t *v, int32_t n,
                         int32_t n_seeds, const int32_t *seeds, int32_t *score, orc_segment *segs,
                         int32_t seg_cap, int32_t *n_segs, int32_t *n_traces);

#ifdef __cplusplus
}
#endif
#endif
