/*
 * sf_align.h -- C ABI of the GB300 (sm_103a) alignment stage for spearfish.
 *
 * Drop-in for the alignment entry points of spearfish's `map::align`
 * (crates/map/src/align.rs, v0.3.2).  Each function below names the
 * reference item it replaces.  All computation runs on the GPU; there is no
 * CPU fallback: without a usable CUDA device every call fails with
 * SF_ERR_CUDA.
 *
 * Conventions
 *  - Sequences are byte codes, one base per byte, exactly as the reference's
 *    `&[u8]` inputs: 0..3 = A, C, G, T.  Myers and the affine passes use
 *    `code & 3` (align.rs:78,120,2557); the local band's read may hold codes
 *    of 4 or more, which match nothing (align.rs:731-734).
 *  - `usize::MAX` arguments (no band, no cut) are SF_NOLIMIT.
 *  - Myers' `Option<u32>` is a uint32_t with SF_NONE for `None`.
 *  - Scores that the reference reports as unreachable are SF_NEG
 *    (align.rs:693, `i32::MIN / 4`).
 *  - Every function returns SF_OK (0) or a negative SF_ERR_* code;
 *    sf_last_error() gives a message for the calling thread.
 *  - Threading: any thread may call any function.  The one-call entry points
 *    use a per-thread context (its own CUDA stream and buffers) on the
 *    current device, as the reference keeps per-thread DP buffers
 *    (align.rs:2167-2171).  Explicit contexts (sf_context_*) are for the
 *    batched and serving forms; one context must not be used by two threads
 *    at once.  Large batches are prepared on a pool of up to seven host
 *    threads, started once per process.
 *
 * Environment (read when a plan is built; results never depend on them)
 *  - SF_AFFINE16=0: every affine pass on the 32-bit rows (no packed 16-bit
 *    rows).
 *  - SF_AFFINE16_LANES=16: 16-bit passes on half warps by default (the
 *    autotuner chooses per length bucket either way).
 *  - SF_SORTED_CHAINS=1: the sorted entry points run the passes that can
 *    share rows as chains (below, at sf_affine_sorted).
 *  - SF_BATCH_SEGMENTS=0: sf_batch_run builds every batch as one plan (no
 *    segments, below).
 */
#ifndef SF_ALIGN_H
#define SF_ALIGN_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define SF_OK 0
#define SF_ERR_INVALID (-1)  /* bad argument */
#define SF_ERR_CUDA (-2)     /* no device / CUDA runtime error */
#define SF_ERR_NOMEM (-3)    /* device or pinned allocation failed */
#define SF_ERR_TOO_LONG (-4) /* a sequence exceeds the supported length */
#define SF_ERR_TIMEOUT (-5)  /* a bounded wait ran out */
#define SF_ERR_CAPACITY (-6) /* an output buffer is too small */
#define SF_ERR_BUSY (-7)     /* serving: no slot or memory free */

#define SF_NONE UINT32_MAX
#define SF_NOLIMIT UINT64_MAX
#define SF_NEG (INT32_MIN / 4)

/* Longest pattern (read segment) the Myers kernels take, in bases. */
#define SF_MYERS_MAX_PATTERN 32768u

/* align.rs:40-45 `Mode`. */
typedef enum { SF_INFIX = 0, SF_PREFIX = 1, SF_GLOBAL = 2 } sf_mode;

/* align.rs:660-668 `Affine`: +mat per match, -mis per mismatch,
 * -(open + ext * l) per gap of length l. */
typedef struct {
    int32_t mat, mis, open, ext;
} sf_affine_t;

/* align.rs:678-690 `Affine::ONT`, `Affine::HIFI`. */
#define SF_AFFINE_ONT ((sf_affine_t){2, 4, 4, 2})
#define SF_AFFINE_HIFI ((sf_affine_t){1, 4, 6, 2})

/* ---- errors and devices ------------------------------------------------ */

const char *sf_last_error(void);
/* Library and kernel build identification (static string). */
const char *sf_version(void);
/* Selects the device the calling thread's one-call context uses
 * (default: the CUDA current device when the thread first calls in). */
int sf_set_device(int device);

/* ---- drop-in entry points (map::align) ---------------------------------- */

/* align.rs:88-91 `distance` (and `distance_with`, align.rs:93-168). */
int sf_distance(const uint8_t *pattern, uint64_t m, const uint8_t *text,
                uint64_t n, int mode, uint32_t k, uint32_t *out);

/* align.rs:174-200 `batch_distances`: one pattern, `count` texts, one k.
 * texts[q] points at lens[q] codes. */
int sf_batch_distances(const uint8_t *pattern, uint64_t m,
                       const uint8_t *const *texts, const uint64_t *lens,
                       uint64_t count, int mode, uint32_t k, uint32_t *out);

/* align.rs:655-658 `infix_distance`. */
int sf_infix_distance(const uint8_t *pattern, uint64_t m, const uint8_t *text,
                      uint64_t n, uint32_t *out);

/* align.rs:699-701 `affine`. band = SF_NOLIMIT for the exact score. */
int sf_affine(const uint8_t *pattern, uint64_t m, const uint8_t *text,
              uint64_t n, int mode, const sf_affine_t *sc, uint64_t band,
              int32_t *out);

/* align.rs:710-729 `affine_extend`. xdrop = INT32_MAX for none. */
int sf_affine_extend(const uint8_t *pattern, uint64_t m, const uint8_t *text,
                     uint64_t n, const sf_affine_t *sc, uint64_t band,
                     int32_t end_bonus, int32_t xdrop, int32_t *out);

/* align.rs:951-982 `affine_extend_window` result: (score, pattern bases,
 * text bases, text bases read). */
typedef struct {
    int32_t score;
    int32_t pad_;
    uint64_t pattern_bases;
    uint64_t text_bases;
    uint64_t text_read;
} sf_extend_t;

int sf_affine_extend_window(const uint8_t *pattern, uint64_t m,
                            const uint8_t *text, uint64_t n, uint64_t window,
                            const sf_affine_t *sc, uint64_t band,
                            int32_t end_bonus, int32_t xdrop, sf_extend_t *out);

/* align.rs:854-861 `affine_sorted`: results equal one `affine` per text.
 * The sorted entry points (this, the two below and sf_sorted_batch) count
 * DP work as align.rs:2210-2315 `affine_dp_sorted` does with its row sharing:
 * a text's pass counts only the rows after those it shares with the previous
 * text (same band shape, rows reading only the common prefix), and nothing
 * when it takes the previous result.  On the GPU every pass runs separately
 * by default; SF_SORTED_CHAINS=1 in the environment runs the passes that can
 * share rows as chains that resume from row snapshots (same results). */
int sf_affine_sorted(const uint8_t *pattern, uint64_t m,
                     const uint8_t *const *texts, const uint64_t *lens,
                     uint64_t count, int mode, const sf_affine_t *sc,
                     uint64_t band, int32_t *out);

/* align.rs:863-901 `affine_extend_sorted_cut` result per text:
 * (whole text, text cut at `cut`, text bases covered). */
typedef struct {
    int32_t whole;
    int32_t cut;
    uint64_t cols;
} sf_cut_t;

/* align.rs:880-901 `affine_extend_sorted_cut`. */
int sf_affine_extend_sorted_cut(const uint8_t *pattern, uint64_t m,
                                const uint8_t *const *texts,
                                const uint64_t *lens, uint64_t count,
                                const sf_affine_t *sc, uint64_t band,
                                int32_t end_bonus, int32_t xdrop, int diagonal,
                                uint64_t window, uint64_t cut, sf_cut_t *out);

/* align.rs:903-949 `affine_extend_sorted_cut_bonus`. */
int sf_affine_extend_sorted_cut_bonus(
    const uint8_t *pattern, uint64_t m, const uint8_t *const *texts,
    const uint64_t *lens, uint64_t count, const sf_affine_t *sc, uint64_t band,
    int32_t end_bonus, int32_t xdrop, int diagonal, uint64_t window,
    uint64_t cut, int track_cut, int bonus_within_cut, sf_cut_t *out);

/* align.rs:731-737 `local_band`. */
int sf_local_band(const uint8_t *read, uint64_t m, const uint8_t *text,
                  uint64_t n, const sf_affine_t *sc, int64_t dlo, int64_t dhi,
                  int32_t end_bonus, int32_t *out);

/* align.rs:741-760 `local_band_ends`. */
int sf_local_band_ends(const uint8_t *read, uint64_t m, const uint8_t *text,
                       uint64_t n, const sf_affine_t *sc, int64_t dlo,
                       int64_t dhi, int32_t bonus_start, int32_t bonus_end,
                       int32_t *out);

/* align.rs:2172-2176 `dp_work`: banded-affine cells and rows computed by the
 * calling thread's passes so far (counted always; the reference counts them
 * only with SPEARFISH_STATS). */
void sf_dp_work(uint64_t *cells, uint64_t *rows);

/* ---- traceback / CIGAR (new: the reference has no traceback) ------------
 * ops are BAM-style words (len << 4 | op), op 0 = M, 1 = I (pattern base
 * against no text base), 2 = D (text base against no pattern base),
 * 4 = S (pattern bases past the extension's end cell).  Tie order: H from
 * H' (diagonal or vertical) before E; diagonal before vertical; gap opening
 * before extending.  The CIGAR re-scores to `score` (minus the end bonus
 * where `score` includes it). */
typedef struct {
    int32_t score;    /* the entry point's score */
    int32_t status;   /* 0 ok, 1 no path (unreachable end), -1 capacity */
    uint64_t pattern_end; /* pattern bases the path covers (ends there) */
    uint64_t text_start;  /* text column the path starts at (Infix) */
    uint64_t text_end;    /* text column the path ends at */
    uint64_t n_ops;
} sf_cigar_t;

/* `affine` with the path of its best cell. */
int sf_affine_cigar(const uint8_t *pattern, uint64_t m, const uint8_t *text,
                    uint64_t n, int mode, const sf_affine_t *sc, uint64_t band,
                    uint32_t *ops, uint64_t cap, sf_cigar_t *out);

/* `affine_extend_window` with the path of the extension. */
int sf_affine_extend_window_cigar(const uint8_t *pattern, uint64_t m,
                                  const uint8_t *text, uint64_t n,
                                  uint64_t window, const sf_affine_t *sc,
                                  uint64_t band, int32_t end_bonus,
                                  int32_t xdrop, uint32_t *ops, uint64_t cap,
                                  sf_cigar_t *out);

/* ---- batched form --------------------------------------------------------
 * Thousands of (pattern, text) jobs of uneven length in one length-bucketed,
 * persistent launch per bucket, captured in a CUDA graph.  Sequences live in
 * one caller pool of byte codes; each job names its pattern and text by byte
 * offset and length. */

typedef struct sf_context sf_context;

int sf_context_create(int device, sf_context **out);
void sf_context_destroy(sf_context *ctx);

enum {
    SF_JOB_MYERS = 0,         /* `distance` in `mode` with threshold k */
    SF_JOB_AFFINE = 1,        /* `affine` in `mode` (score, optional CIGAR) */
    SF_JOB_EXTEND_WINDOW = 2, /* `affine_extend_window` (optional CIGAR) */
    SF_JOB_LOCAL = 3          /* `local_band_ends` */
};

typedef struct {
    uint64_t p_off; /* pattern: byte offset in the pool */
    uint64_t t_off; /* text: byte offset in the pool */
    uint32_t m, n;  /* lengths */
    uint8_t kind;   /* SF_JOB_* */
    uint8_t mode;   /* sf_mode (Myers, affine) */
    uint8_t want_cigar;
    uint8_t text_src; /* SF_TEXT_POOL: t_off is a byte offset in the pool;
                         SF_TEXT_STORE(_REV): t_off is a base position in the
                         context's transcript store (sf_context_use_store), the
                         window read forwards (backwards) */
    uint32_t k;      /* Myers threshold (SF_NONE: none) */
    uint64_t band;   /* affine band (SF_NOLIMIT: none) */
    uint64_t window; /* extend window */
    int64_t dlo, dhi; /* local band diagonals */
    int32_t end_bonus, end_bonus2; /* extend bonus; local (start, end) */
    int32_t xdrop;
    uint32_t sc_index; /* index into the batch's scoring table */
} sf_job_t;

typedef struct {
    int32_t score;      /* affine / extend / local score */
    uint32_t distance;  /* Myers: SF_NONE for None */
    uint64_t pattern_end, text_start, text_end, text_read;
    uint64_t cells;     /* DP cells computed (GCUPS numerator) */
    uint64_t cigar_off; /* first op of this job's CIGAR in the op pool */
    uint32_t n_ops;
    int32_t status;     /* 0 ok; 1 no path; negative SF_ERR_* */
} sf_result_t;

/* A batch prepared once and run many times: descriptors, bucketing and
 * device buffers are built at creation; sf_plan_execute launches the bucket
 * kernels (captured into a CUDA graph on first use) on inputs already
 * resident in HBM. */
typedef struct sf_plan sf_plan;

int sf_plan_create(sf_context *ctx, const sf_job_t *jobs, uint64_t count,
                   const sf_affine_t *scores, uint32_t n_scores,
                   uint64_t pool_bytes, sf_plan **out);
void sf_plan_destroy(sf_plan *plan);
/* Host pool -> device, copied on the plan's stream straight from `pool`.  From
 * pinned memory the copy is asynchronous: keep the pool unchanged until the
 * plan's stream has passed it (sf_plan_sync, sf_plan_download).  From pageable
 * memory the call returns once the bytes are staged. */
int sf_plan_upload(sf_plan *plan, const uint8_t *pool);
/* Run every job on the resident inputs (asynchronous). */
int sf_plan_execute(sf_plan *plan);
/* Results (and compacted CIGAR ops) -> host; waits for the plan's stream.
 * ops may be NULL when no job wants a CIGAR. */
int sf_plan_download(sf_plan *plan, sf_result_t *results, uint32_t *ops,
                     uint64_t ops_cap, uint64_t *ops_used);
/* Blocks until the plan's work is done. */
int sf_plan_sync(sf_plan *plan);
/* The plan's CUDA stream (cudaStream_t) for event timing. */
void *sf_plan_stream(sf_plan *plan);
/* Kernel launches one execute issues (for launch accounting). */
uint64_t sf_plan_launches(const sf_plan *plan);
/* Description of the plan's buckets as a static-lifetime JSON string. */
const char *sf_plan_describe(sf_plan *plan);
/* Each job's bucket: buckets[q] = the index, in sf_plan_describe's list, of
 * the bucket whose kernel runs job q (SF_NONE for a job that a row-sharing
 * chain runs).  `count` >= the plan's jobs.  No reference counterpart: the
 * reference has no buckets; this lets a caller attribute work per kernel. */
int sf_plan_job_buckets(const sf_plan *plan, uint32_t *buckets, uint64_t count);

/* Runs one execute in order on the plan's stream with CUDA events between
 * its stages -- pack, each bucket (in sf_plan_describe's order; a bucket
 * that keeps CIGARs walks its paths too), then the CIGAR compaction -- and
 * returns each stage's ms. */
int sf_plan_profile(sf_plan *plan, float *ms, uint32_t cap,
                    uint32_t *n_stages);

/* Autotuner (no reference counterpart: the reference's CPU path has no kernel
 * classes to choose).  Groups the plan's jobs by their default kernel class
 * (their length bucket) and times each group alone, `reps` executes per
 * candidate, in the classes it may run in instead: Myers, every (blocks per
 * lane, lanes per pair) that covers the group's longest pattern -- how much of
 * a warp a pair takes; affine register rows, the next two row widths -- where
 * the bucket edges fall.  The fastest per group is kept in the plan's context
 * (later plans and sf_batch_run in that context use it) and the plan is rebuilt
 * with it, its pool uploaded again from `pool`.  `report` (may be NULL)
 * receives a JSON summary.  Results do not depend on the classes. */
int sf_plan_tune(sf_plan *plan, const uint8_t *pool, uint32_t reps, char *report,
                 uint64_t cap);
/* Drops a context's autotuner choices: later plans use the default classes. */
int sf_context_untune(sf_context *ctx);

/* One call on the context's reusable plan: descriptors, upload, execute,
 * download (buffers grow and are reused across calls).  A batch of at least
 * 8,192 jobs whose jobs are of similar work (none above 8x the mean) runs in
 * up to four segments of consecutive jobs, each its own plan: the host
 * prepares segment k + 1 while the device runs segment k.  Results, CIGAR
 * ops and their order (job order) are the same either way. */
int sf_batch_run(sf_context *ctx, const uint8_t *pool, uint64_t pool_bytes,
                 const sf_job_t *jobs, uint64_t count,
                 const sf_affine_t *scores, uint32_t n_scores,
                 sf_result_t *results, uint32_t *ops, uint64_t ops_cap,
                 uint64_t *ops_used);

/* ---- device-resident transcript store ------------------------------------
 * The index's transcripts packed once in HBM, 2 bits a base in its own bit
 * order (crates/index/src/lib.rs:47-153 `tx_seq`, 253-280: 32 bases per u64,
 * base p at bits 2*(p % 32) of word p / 32).  Jobs of a plan built in a context
 * that uses the store (sf_context_use_store) may name their text as a window
 * of it (text_src = SF_TEXT_STORE, t_off = the window's first base in the
 * store's concatenation, as `tx_range` numbers it; n = its length): the window
 * is sliced on the device, so a batch uploads only reads and descriptors.  The
 * store must outlive every plan execution that reads it. */
enum {
    SF_TEXT_POOL = 0,
    SF_TEXT_STORE = 1,
    SF_TEXT_STORE_REV = 2 /* the store window read backwards (a leftward extension's
                             flank, as the mapper reverses it: lib.rs:2024-2027) */
};
typedef struct sf_store sf_store;

/* A store of `count` transcripts given as byte codes (0..3), concatenated in
 * `codes`, lens[q] codes each, on the context's device. */
int sf_store_create(sf_context *ctx, const uint8_t *codes, const uint64_t *lens,
                    uint64_t count, sf_store **out);
/* A store from the index's packed words as they are (`tx_seq`, `bases` bases). */
int sf_store_create_packed(sf_context *ctx, const uint64_t *tx_seq, uint64_t bases,
                           sf_store **out);
void sf_store_destroy(sf_store *store);
/* Bases the store holds. */
uint64_t sf_store_bases(const sf_store *store);
/* Later plans of this context resolve SF_TEXT_STORE texts in `store` (NULL: none). */
int sf_context_use_store(sf_context *ctx, sf_store *store);

/* ---- tie-break batching (map/src/lib.rs) --------------------------------
 * The mapper's tie-break asks, per read, for the edit distance to each of its
 * candidate texts under a threshold that tightens as it goes
 * (lib.rs:851-911 `Mapper::banded`).  Here a whole read batch's distinct
 * (read, text) distances run as one Myers launch, and each read's threshold is
 * applied in text order on the host -- the same values, since a batch
 * distance is exact whenever it is within its threshold (align.rs:87-168). */

/* lib.rs:851-911 `Mapper::banded`: out[q] = the distance of `read` to
 * texts[q] in `mode`, or k + 1 when it exceeds k = (best so far + cap)
 * (saturating); with distinct = 0 a repeated text is computed once and its
 * first value re-capped at the current k. */
int sf_banded(const uint8_t *read, uint64_t m, const uint8_t *const *texts,
              const uint64_t *lens, uint64_t count, int mode, uint32_t cap,
              int distinct, uint32_t *out);

typedef struct {
    uint64_t off, len; /* codes in the pool */
} sf_span_t;

typedef struct {
    uint64_t p_off;    /* the read's codes in the pool */
    uint64_t first;    /* index of its first text in the text list */
    uint32_t m;        /* read length */
    uint32_t count;    /* its texts: text list [first, first + count) */
    uint32_t mode;     /* sf_mode */
    uint32_t cap;      /* `banded`'s cap */
    uint32_t distinct; /* `banded`'s distinct */
    uint32_t pad_;
} sf_banded_read_t;

/* `banded` for n_reads reads at once (their texts consecutive in `texts`):
 * out[q] for texts[q], as sf_banded would give read by read. */
int sf_banded_batch(sf_context *ctx, const uint8_t *pool, uint64_t pool_bytes,
                    const sf_banded_read_t *reads, uint64_t n_reads,
                    const sf_span_t *texts, uint64_t n_texts, uint32_t *out);

/* lib.rs:414-425 `Ends`: the span-end extensions' scoring, band, end bonus,
 * X-drop, and the transcript flank searched beyond the read flank's length,
 * pad + flank / pad_div. */
typedef struct {
    sf_affine_t sc;
    uint64_t band;
    int32_t end_bonus, xdrop;
    uint32_t pad, pad_div;
} sf_ends_t;

/* A hit whose span is extended over the read's flanks (the TxHit fields
 * `extend_ends` reads and writes): the read in the hit's orientation (codes
 * in the pool), its transcript (a range of the context's store) and the span's
 * read / transcript coordinates, updated in place. */
typedef struct {
    uint64_t read_off;   /* the read's codes in the pool */
    uint64_t tx_start;   /* the transcript's first base in the store */
    uint32_t read_len, tx_len;
    uint32_t qstart, qend, tstart, tend;
} sf_hit_t;

/* lib.rs:2020-2035 `extend_ends` (with 2046-2073 `right_reach` and 2100-2114
 * `extend_dp`) for n hits in one device batch: each span extended leftwards
 * over the read prefix and the transcript flank before it (both read
 * backwards, lib.rs:2024-2027) when qstart > 0 and tstart > 0, and rightwards
 * when the read and the transcript go on.  The flanks are read from the
 * context's store; the reference's per-read cache of extensions
 * (lib.rs:427-430) only avoids recomputing equal results. */
int sf_extend_ends_batch(sf_context *ctx, const uint8_t *pool, uint64_t pool_bytes,
                         const sf_ends_t *e, sf_hit_t *hits, uint64_t n);

/* The tie-break's sorted DP calls (lib.rs:1294-1884 `segmented`: a read
 * segment against the candidates' distinct texts in sorted order) for many
 * segments in one batch.  Each call is one of the two sorted entry points. */
enum {
    SF_SORTED_AFFINE = 0,    /* align.rs:854-861 `affine_sorted` in `mode` */
    SF_SORTED_EXTEND_CUT = 1 /* align.rs:903-949 `affine_extend_sorted_cut_bonus` */
};
typedef struct {
    uint64_t p_off;    /* the read segment's codes in the pool */
    uint64_t first;    /* its first text in the text list */
    uint64_t band;
    uint64_t window;   /* extend: the window the band is laid out for */
    uint64_t cut;      /* extend: the cut (SF_NOLIMIT: none) */
    uint32_t m, count; /* segment length; texts [first, first + count) */
    uint32_t kind;     /* SF_SORTED_* */
    uint32_t mode;     /* affine_sorted's mode */
    int32_t end_bonus, xdrop;
    uint32_t diagonal, track_cut, bonus_within_cut;
    uint32_t sc_index; /* into `scores` */
} sf_sorted_call_t;

/* out[q] for texts[q]: the entry point's (whole, cut, cols) triple; for
 * affine_sorted the score as (x, x, 0), as lib.rs:1442-1445 uses it.  Equal to
 * the one-call entry points text by text. */
int sf_sorted_batch(sf_context *ctx, const uint8_t *pool, uint64_t pool_bytes,
                    const sf_affine_t *scores, uint32_t n_scores,
                    const sf_sorted_call_t *calls, uint64_t n_calls,
                    const sf_span_t *texts, uint64_t n_texts, sf_cut_t *out);

/* ---- serving: continuous batching ---------------------------------------
 * Requests (the jobs of a read batch over a byte pool the caller keeps alive
 * until it waits for them) are admitted in arrival order as soon as a slot
 * is free and the device memory they need fits the HBM budget; requests on
 * different slots run on the device at the same time.  A request's results
 * are the same alone as in any mix. */
typedef struct sf_server sf_server;

typedef struct {
    int device;
    uint32_t slots;       /* requests on the device at once (0: 8) */
    uint64_t hbm_budget;  /* bytes the slots may hold (0: 90% of free memory) */
    const sf_affine_t *scores; /* scoring table for sc_index (NULL: ONT) */
    uint32_t n_scores;
    sf_store *store;      /* transcript store for SF_TEXT_STORE texts (may be NULL) */
} sf_server_opts;

typedef struct {
    double queue_ms;  /* submitted -> admitted to a slot */
    double run_ms;    /* admitted -> results on the host */
    double total_ms;  /* submitted -> results on the host */
    uint64_t cells;   /* DP cells of the request */
    uint32_t slot;
    int32_t status;
} sf_request_stats;

typedef struct {
    uint64_t submitted, completed, failed, cells;
    uint64_t hbm_budget, hbm_held;
    uint32_t slots, busy_slots, pending, pad_;
} sf_server_stats;

int sf_server_create(const sf_server_opts *opts, sf_server **out);
/* Stops the loop; requests not yet waited for are dropped. */
void sf_server_destroy(sf_server *srv);
int sf_server_submit(sf_server *srv, const uint8_t *pool, uint64_t pool_bytes,
                     const sf_job_t *jobs, uint64_t count, uint64_t *ticket);
/* Waits at most timeout_ms (SF_ERR_TIMEOUT; the request stays pending), then
 * copies the request's results and compacted CIGAR ops and releases it. */
int sf_server_wait(sf_server *srv, uint64_t ticket, int32_t timeout_ms,
                   sf_result_t *results, uint32_t *ops, uint64_t ops_cap,
                   uint64_t *ops_used, sf_request_stats *stats);
int sf_server_query(sf_server *srv, sf_server_stats *out);

/* ---- without device allocation ------------------------------------------
 * No counterpart in the reference: `affine` (align.rs:699-701) for callers
 * that must not allocate device memory -- a latency-bound serving path, where
 * cudaMalloc and cudaFree synchronize the device and stall every request in
 * flight, or an application that hands this library device memory from its
 * own pool and forbids any other device allocation.  Inputs (byte codes) and
 * the output score are the caller's device buffers; everything else lives in
 * one file-scope device array of SF_NOALLOC_SCRATCH bytes per GPU, which
 * every call shares and which keeps the last call's contents.  Work is queued
 * on `stream` (a cudaStream_t; NULL for the default stream) and the score is
 * in *d_score once the stream reaches it.  Pattern and text are limited to
 * SF_NOALLOC_MAX_LEN bases each (SF_ERR_TOO_LONG beyond).  Calls whose work
 * overlaps on one GPU race on the array: order them (one stream).  The first
 * call on a device looks the array up with that device current; make it
 * before any stream capture.  The address is kept for the process: after a
 * cudaDeviceReset of that device the library must be loaded afresh before
 * this entry point is called again.  A score-only pass has no failure outcome
 * on the device (an unreachable end is NEG, as `affine` returns), so every
 * error is reported by the return code.  Its cells and rows are not added to
 * sf_dp_work's counters: the call returns before the pass has run. */
#define SF_NOALLOC_SCRATCH (1u << 19)
#define SF_NOALLOC_MAX_LEN 16384u
int sf_affine_noalloc(const uint8_t *d_pattern, uint64_t m,
                      const uint8_t *d_text, uint64_t n, int mode,
                      const sf_affine_t *sc, uint64_t band, int32_t *d_score,
                      void *stream);

/* ---- diagnostics -------------------------------------------------------- */

/* Measured int32 throughput of `device` (tera-ops/s) on the DP kernels'
 * add-then-max instruction mix: the roofline of the integer-bound DP. */
int sf_int_peak(int device, double *tops, double *ms);

#ifdef __cplusplus
}
#endif
#endif
