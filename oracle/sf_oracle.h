/*
 * CPU oracle for the spearfish alignment stage -- TEST INFRASTRUCTURE ONLY.
 *
 * A plain-C restatement of crates/map/src/align.rs (spearfish v0.3.2): Myers'
 * bit-parallel edit distance with Ukkonen's cutoff, the banded Gotoh pass
 * `run_core` over the scalar row kernel `row_scalar`, the banded local pass
 * `local_band_core`, the public entry points built on them, and the naive
 * definitions the reference's own tests compare against.  A traceback oracle
 * (full banded matrices, a stated tie order, CIGAR output) is added: the
 * reference computes no traceback, so CIGAR parity is unpinned and is checked
 * by re-scoring each CIGAR to the reference score and end cell.
 *
 * Only tests, the smoke check and the bench's CPU-baseline / reference arm may
 * load this library.  Nothing in the product path links or calls it.
 */
#ifndef SF_ORACLE_H
#define SF_ORACLE_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* align.rs:40-45 `Mode`. */
enum { OR_INFIX = 0, OR_PREFIX = 1, OR_GLOBAL = 2 };

/* align.rs:693 `NEG = i32::MIN / 4`. */
#define OR_NEG (INT32_MIN / 4)

/* `usize::MAX` stand-in: no band / no cut. */
#define OR_NOLIMIT ((uint64_t)UINT64_MAX)

/* align.rs:660-668 `Affine`. */
typedef struct {
    int32_t mat, mis, open, ext;
} or_affine_t;

/* align.rs:2111-2129 `Dp`, plus the DP_WORK counters of the pass. */
typedef struct {
    int32_t score;
    int32_t clip_best;
    int32_t cut_best;
    int32_t cut_score;
    uint64_t score_col;
    uint64_t clip_i, clip_j;
    uint64_t text_read;
    uint64_t last_row;
    uint64_t cells, rows;
} or_dp_t;

/* ---- Myers (align.rs:47-658) ------------------------------------------ */

/* `distance` (align.rs:88-168): the distance, or -1 for None. */
int64_t or_myers_distance(const uint8_t *p, uint64_t m, const uint8_t *t,
                          uint64_t n, int mode, uint32_t k);
/* `batch_lanes::<L>` (align.rs:557-653) over `count` texts in chunks of L. */
void or_myers_batch_lanes(const uint8_t *p, uint64_t m, const uint8_t *texts,
                          const uint64_t *offs, const uint64_t *lens,
                          uint64_t count, int lanes, int mode, uint32_t k,
                          int64_t *out);
/* The reference tests' `naive` (align.rs:2801-2827). */
uint32_t or_myers_naive(const uint8_t *p, uint64_t m, const uint8_t *t,
                        uint64_t n, int mode);

/* ---- Affine (align.rs:660-982, 2178-2666) ----------------------------- */

/* One pass of `run_core` (align.rs:2446-2666) with the scalar rows.
 * clip: 0 = None, else Some((xdrop, cell)). */
void or_affine_dp(const uint8_t *p, uint64_t m, const uint8_t *t, uint64_t n,
                  int mode, const or_affine_t *sc, uint64_t band, uint64_t geom,
                  int clip, int32_t xdrop, int cell, uint64_t cut,
                  or_dp_t *out);

int32_t or_affine(const uint8_t *p, uint64_t m, const uint8_t *t, uint64_t n,
                  int mode, const or_affine_t *sc, uint64_t band);
int32_t or_affine_extend(const uint8_t *p, uint64_t m, const uint8_t *t,
                         uint64_t n, const or_affine_t *sc, uint64_t band,
                         int32_t end_bonus, int32_t xdrop);
/* out4 = (score, pattern bases, text bases, text bases read). */
void or_affine_extend_window(const uint8_t *p, uint64_t m, const uint8_t *t,
                             uint64_t n, uint64_t window, const or_affine_t *sc,
                             uint64_t band, int32_t end_bonus, int32_t xdrop,
                             int64_t *out4);
/* Per text: (whole, cut, cols) as int64 triples. */
void or_affine_extend_sorted_cut_bonus(
    const uint8_t *p, uint64_t m, const uint8_t *texts, const uint64_t *offs,
    const uint64_t *lens, uint64_t count, const or_affine_t *sc, uint64_t band,
    int32_t end_bonus, int32_t xdrop, int diagonal, uint64_t window,
    uint64_t cut, int track_cut, int bonus_within_cut, int64_t *out3);
void or_affine_sorted(const uint8_t *p, uint64_t m, const uint8_t *texts,
                      const uint64_t *offs, const uint64_t *lens,
                      uint64_t count, int mode, const or_affine_t *sc,
                      uint64_t band, int32_t *out);
int32_t or_local_band_ends(const uint8_t *read, uint64_t m, const uint8_t *t,
                           uint64_t n, const or_affine_t *sc, int64_t dlo,
                           int64_t dhi, int32_t bonus0, int32_t bonus1);

/* Naive definitions from the reference tests (align.rs:2928-3014). */
int32_t or_naive_affine(const uint8_t *p, uint64_t m, const uint8_t *t,
                        uint64_t n, int mode, const or_affine_t *sc);
int32_t or_naive_extend(const uint8_t *p, uint64_t m, const uint8_t *t,
                        uint64_t n, const or_affine_t *sc);
int32_t or_naive_local(const uint8_t *p, uint64_t m, const uint8_t *t,
                       uint64_t n, const or_affine_t *sc, int32_t b0,
                       int32_t b1);
int32_t or_naive_local_band(const uint8_t *p, uint64_t m, const uint8_t *t,
                            uint64_t n, const or_affine_t *sc, int64_t dlo,
                            int64_t dhi, int32_t b0, int32_t b1);

/* ---- Traceback (new: no reference counterpart) ------------------------ */

/* CIGAR ops, BAM numbering. */
enum { OR_OP_M = 0, OR_OP_I = 1, OR_OP_D = 2, OR_OP_S = 4 };

/* Traceback kinds: which end cell the path starts from. */
enum {
    OR_TB_AFFINE = 0,  /* `affine` in a mode: (m, score_col) */
    OR_TB_EXTEND = 1   /* `affine_extend_window`: clip cell or (m, score_col) */
};

/* Result of a traceback.  `cigar` holds (len << 4 | op) words in forward
 * order.  status: 0 ok, 1 unreachable end (no path), -1 capacity too small. */
typedef struct {
    int32_t score;      /* the entry point's score */
    int32_t status;
    uint64_t end_i, end_j;      /* end cell (pattern, text) */
    uint64_t text_start;        /* text column the path leaves row 0 at */
    uint64_t n_ops;
} or_tb_t;

void or_affine_traceback(const uint8_t *p, uint64_t m, const uint8_t *t,
                         uint64_t n, int kind, int mode, const or_affine_t *sc,
                         uint64_t band, uint64_t window, int32_t end_bonus,
                         int32_t xdrop, uint32_t *cigar, uint64_t cap,
                         or_tb_t *out);

/* Score of a CIGAR over pattern/text (soft clips score 0, gap runs
 * -(open + ext * len), M columns +mat / -mis). */
int64_t or_cigar_score(const uint8_t *p, uint64_t m, const uint8_t *t,
                       uint64_t n, const uint32_t *cigar, uint64_t n_ops,
                       uint64_t text_start, const or_affine_t *sc,
                       uint64_t *p_used, uint64_t *t_end);

/* ---- CPU baseline driver (multi-threaded, one pair per task) ----------- */

/* Which row kernel the passes use: 0 scalar rows, 1 the NEON rows of
 * align.rs:2016-2085 (aarch64 only; scalar elsewhere).  Returns the level
 * actually used. */
int or_set_level(int level);
int or_get_level(void);

/* Extension jobs (kind 2): the window x + pad + x / pad_div (pad_div 0: no
 * term) for a read end of x bases, X-drop and end bonus. */
typedef struct {
    uint64_t pad, pad_div;
    int32_t xdrop, end_bonus;
} or_extend_opts_t;

/* Jobs: Myers distance per pair (kind 0; cap kv[q] when kv is not NULL, else
 * k), `affine` per pair (kind 1) or `affine_extend_window` per pair (kind 2,
 * whole score).  Sequences are byte codes; pair q is p[poff[q]..+plen[q]] vs
 * t[toff[q]..+tlen[q]]; its band is bv[q] when bv is not NULL, else band.
 * out: int64 per pair; cells_out (may be NULL): each pair's cells.  Returns
 * the summed DP_WORK cells (affine) or m*n cells (Myers). */
uint64_t or_run_pairs(int kind, int threads, const uint8_t *pseq,
                      const uint64_t *poff, const uint64_t *plen,
                      const uint8_t *tseq, const uint64_t *toff,
                      const uint64_t *tlen, uint64_t count, int mode,
                      uint32_t k, const uint32_t *kv, const or_affine_t *sc,
                      uint64_t band, const uint64_t *bv,
                      const or_extend_opts_t *ext, int64_t *out,
                      uint64_t *cells_out);

/* CIGAR checks of a batch on `threads` workers: pair q's ops
 * ops[cig_off[q]..+n_ops[q]] are re-scored from text base text_start[q]
 * (or_cigar_score).  code[q]: 0 the path consumes the whole pattern, ends at
 * text_end[q] and scores score[q]; 1 another score; 2 the pattern is not
 * consumed exactly; 3 another text end; 4 an op leaves the sequences or is
 * unknown.  Returns the number of pairs whose code is not 0. */
uint64_t or_check_cigars(int threads, const uint8_t *pseq, const uint64_t *poff,
                         const uint64_t *plen, const uint8_t *tseq,
                         const uint64_t *toff, const uint64_t *tlen,
                         uint64_t count, const uint32_t *ops,
                         const uint64_t *cig_off, const uint32_t *n_ops,
                         const uint64_t *text_start, const uint64_t *text_end,
                         const int32_t *score, const or_affine_t *sc,
                         int32_t *code);

#ifdef __cplusplus
}
#endif
#endif
