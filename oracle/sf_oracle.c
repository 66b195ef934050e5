/*
 * CPU oracle for the spearfish alignment stage -- TEST INFRASTRUCTURE ONLY.
 * See sf_oracle.h.  Every function names the lines of
 * crates/map/src/align.rs (spearfish v0.3.2) it restates.  Integer semantics
 * follow the Rust code: i32 arithmetic on cell scores, saturating adds where
 * the reference saturates, usize saturating band geometry.
 */
#include "sf_oracle.h"

#include <pthread.h>
#include <stdatomic.h>
#include <stdlib.h>
#include <string.h>

#if defined(__aarch64__)
#include <arm_neon.h>
#endif

#define NEG OR_NEG
#define W 64

static inline int32_t max32(int32_t a, int32_t b) { return a > b ? a : b; }
static inline int32_t min32(int32_t a, int32_t b) { return a < b ? a : b; }
static inline uint64_t usat_add(uint64_t a, uint64_t b) {
    return a > UINT64_MAX - b ? UINT64_MAX : a + b;
}
static inline uint64_t usat_sub(uint64_t a, uint64_t b) { return a > b ? a - b : 0; }
static inline uint64_t umin(uint64_t a, uint64_t b) { return a < b ? a : b; }
static inline uint64_t umax(uint64_t a, uint64_t b) { return a > b ? a : b; }
static inline int32_t sat_add32(int32_t a, int32_t b) {
    int64_t s = (int64_t)a + b;
    return s > INT32_MAX ? INT32_MAX : s < INT32_MIN ? INT32_MIN : (int32_t)s;
}
static inline int32_t sat_sub32(int32_t a, int32_t b) {
    int64_t s = (int64_t)a - b;
    return s > INT32_MAX ? INT32_MAX : s < INT32_MIN ? INT32_MIN : (int32_t)s;
}
/* Rust i32 `+ - *` in release builds wrap; cell values here never reach the
 * edges, but the wrapping forms keep the restatement defined either way. */
static inline int32_t wadd(int32_t a, int32_t b) { return (int32_t)((uint32_t)a + (uint32_t)b); }
static inline int32_t wsub(int32_t a, int32_t b) { return (int32_t)((uint32_t)a - (uint32_t)b); }
static inline int32_t wmul(int32_t a, int32_t b) { return (int32_t)((uint32_t)a * (uint32_t)b); }

/* ======================================================================
 * Myers
 * ====================================================================== */

/* align.rs:50-66 `block`. */
static inline int32_t myers_block(uint64_t *pv, uint64_t *mv, uint64_t eq, int32_t hin,
                                  unsigned bit) {
    uint64_t neg = (uint64_t)(hin < 0), pos = (uint64_t)(hin > 0);
    uint64_t p = *pv, m = *mv;
    uint64_t xv = eq | m;
    eq |= neg;
    uint64_t xh = (((eq & p) + p) ^ p) | eq;
    uint64_t ph = m | ~(xh | p);
    uint64_t mh = p & xh;
    int32_t hout = (int32_t)((ph >> bit) & 1) - (int32_t)((mh >> bit) & 1);
    ph = (ph << 1) | pos;
    mh = (mh << 1) | neg;
    *pv = mh | ~(xv | ph);
    *mv = ph & xv;
    return hout;
}

/* align.rs:75-84 `Pattern::new`: peq[b*4 + c]. */
static uint64_t *myers_peq(const uint8_t *p, uint64_t m) {
    uint64_t blocks = (m + W - 1) / W;
    uint64_t *peq = calloc(blocks * 4 + 4, sizeof(uint64_t));
    for (uint64_t i = 0; i < m; i++) peq[(i / W) * 4 + (p[i] & 3)] |= 1ull << (i % W);
    return peq;
}

/* align.rs:93-168 `distance_with`. */
static int64_t myers_with(const uint64_t *peq, uint64_t m, const uint8_t *t, uint64_t n,
                          int mode, uint32_t k32) {
    if (m == 0) {
        uint32_t d = mode == OR_GLOBAL ? (uint32_t)n : 0;
        return d <= k32 ? (int64_t)d : -1;
    }
    uint64_t mn = m + n;
    int32_t k = (int32_t)((uint64_t)k32 < mn ? k32 : (uint32_t)mn);
    uint64_t blocks = (m + W - 1) / W;
    unsigned last_bit = (unsigned)((m - 1) % W);
#define ROWS(b) ((b) + 1 == blocks ? (int32_t)last_bit + 1 : W)
#define BIT(b) ((b) + 1 == blocks ? last_bit : (unsigned)(W - 1))
    int32_t top = mode == OR_INFIX ? 0 : 1;
    uint64_t *pv = malloc(blocks * sizeof(uint64_t));
    uint64_t *mv = malloc(blocks * sizeof(uint64_t));
    int32_t *score = malloc(blocks * sizeof(int32_t));
    for (uint64_t b = 0; b < blocks; b++) {
        pv[b] = ~0ull;
        mv[b] = 0;
        score[b] = (int32_t)(b * W) + ROWS(b);
    }
    uint64_t kb = ((uint64_t)k + 1 + W - 1) / W;
    int64_t last = (int64_t)umin(blocks, kb) - 1;
    int32_t best = ((uint64_t)(last + 1) == blocks && score[blocks - 1] <= k) ? score[blocks - 1]
                                                                               : INT32_MAX;
    int64_t result = -2;
    for (uint64_t j = 0; j < n; j++) {
        unsigned c = t[j] & 3;
        int32_t hin = top;
        for (int64_t b = 0; b <= last; b++) {
            hin = myers_block(&pv[b], &mv[b], peq[b * 4 + c], hin, BIT((uint64_t)b));
            score[b] += hin;
        }
        uint64_t lb = (uint64_t)last;
        if (lb + 1 < blocks && score[lb] - hin <= k &&
            ((peq[(lb + 1) * 4 + c] & 1) != 0 || hin < 0)) {
            uint64_t nb = lb + 1;
            pv[nb] = ~0ull;
            mv[nb] = 0;
            int32_t h = myers_block(&pv[nb], &mv[nb], peq[nb * 4 + c], hin, BIT(nb));
            score[nb] = score[lb] - hin + ROWS(nb) + h;
            last += 1;
        } else {
            while (last >= 0 && score[last] >= k + W) last -= 1;
            if (last < 0) {
                if (mode == OR_GLOBAL)
                    result = -1;
                else
                    result = best <= k ? best : -1;
                break;
            }
        }
        if ((uint64_t)(last + 1) == blocks) {
            int32_t s = score[blocks - 1];
            if (mode == OR_GLOBAL) {
                if (j + 1 == n) best = s;
            } else {
                best = min32(best, s);
            }
        } else if (mode == OR_GLOBAL && j + 1 == n) {
            best = INT32_MAX;
        }
    }
    if (result == -2) {
        if (mode == OR_GLOBAL && n == 0) best = (int32_t)m;
        result = best <= k ? best : -1;
    }
    free(pv);
    free(mv);
    free(score);
    return result;
#undef ROWS
#undef BIT
}

int64_t or_myers_distance(const uint8_t *p, uint64_t m, const uint8_t *t, uint64_t n,
                          int mode, uint32_t k) {
    uint64_t *peq = myers_peq(p, m);
    int64_t d = myers_with(peq, m, t, n, mode, k);
    free(peq);
    return d;
}

/* align.rs:557-653 `batch_lanes::<L>`: L texts in lockstep, the union band. */
static void myers_lanes(const uint64_t *peq, uint64_t m, const uint8_t *const *tx_ptr,
                        const uint64_t *lens, int L, int mode, uint32_t k32, int64_t *out) {
    uint64_t n_max = 0;
    for (int l = 0; l < L; l++) n_max = umax(n_max, lens[l]);
    int32_t kk = (int32_t)((uint64_t)k32 < m + n_max ? k32 : (uint32_t)(m + n_max));
    uint64_t blocks = (m + W - 1) / W;
    unsigned last_bit = (unsigned)((m - 1) % W);
#define ROWS(b) ((b) + 1 == blocks ? (int32_t)last_bit + 1 : W)
#define BIT(b) ((b) + 1 == blocks ? last_bit : (unsigned)(W - 1))
    uint64_t *pv = malloc(blocks * L * sizeof(uint64_t));
    uint64_t *mv = malloc(blocks * L * sizeof(uint64_t));
    int32_t *score = malloc(blocks * L * sizeof(int32_t));
    for (uint64_t b = 0; b < blocks; b++)
        for (int l = 0; l < L; l++) {
            pv[b * L + l] = ~0ull;
            mv[b * L + l] = 0;
            score[b * L + l] = (int32_t)(b * W) + ROWS(b);
        }
    int32_t kw = kk + W;
    int64_t last = (int64_t)umin(blocks, ((uint64_t)kk + 1 + W - 1) / W) - 1;
    int32_t best0 = ((uint64_t)(last + 1) == blocks && (int32_t)m <= kk) ? (int32_t)m : INT32_MAX;
    int32_t best[64], h[64], top[64];
    unsigned c[64];
    int live[64];
    for (int l = 0; l < L; l++) {
        if (mode == OR_GLOBAL)
            best[l] = lens[l] == 0 ? (int32_t)m : INT32_MAX;
        else
            best[l] = best0;
    }
    int32_t h0 = mode == OR_INFIX ? 0 : 1;
    for (uint64_t j = 0; j < n_max; j++) {
        for (int l = 0; l < L; l++) {
            c[l] = j < lens[l] ? (tx_ptr[l][j] & 3) : 0;
            live[l] = j < lens[l];
            h[l] = h0;
        }
        for (int64_t b = 0; b <= last; b++)
            for (int l = 0; l < L; l++) {
                h[l] = myers_block(&pv[b * L + l], &mv[b * L + l], peq[b * 4 + c[l]], h[l],
                                   BIT((uint64_t)b));
                score[b * L + l] += h[l];
            }
        uint64_t lb = (uint64_t)last;
        int added = 0;
        if (lb + 1 < blocks) {
            uint64_t nb = lb + 1;
            int want = 0;
            for (int l = 0; l < L; l++) {
                top[l] = score[lb * L + l] - h[l];
                if (live[l] && top[l] <= kk && ((peq[nb * 4 + c[l]] & 1) != 0 || h[l] < 0))
                    want = 1;
            }
            if (want) {
                for (int l = 0; l < L; l++) {
                    pv[nb * L + l] = ~0ull;
                    mv[nb * L + l] = 0;
                    int32_t hn = myers_block(&pv[nb * L + l], &mv[nb * L + l],
                                             peq[nb * 4 + c[l]], h[l], BIT(nb));
                    score[nb * L + l] = top[l] + ROWS(nb) + hn;
                }
                last += 1;
                added = 1;
            }
        }
        if (!added) {
            for (;;) {
                if (last < 0) break;
                int any = 0;
                for (int l = 0; l < L; l++)
                    if (live[l] && score[(uint64_t)last * L + l] < kw) any = 1;
                if (any) break;
                last -= 1;
            }
            if (last < 0) break;
        }
        if ((uint64_t)(last + 1) == blocks)
            for (int l = 0; l < L; l++) {
                int32_t s = score[(blocks - 1) * L + l];
                if (mode == OR_GLOBAL) {
                    if (j + 1 == lens[l]) best[l] = s;
                } else if (live[l]) {
                    best[l] = min32(best[l], s);
                }
            }
    }
    for (int l = 0; l < L; l++) {
        uint64_t mn = m + lens[l];
        int32_t kl = (int32_t)((uint64_t)k32 < mn ? k32 : (uint32_t)mn);
        out[l] = best[l] <= kl ? best[l] : -1;
    }
    free(pv);
    free(mv);
    free(score);
#undef ROWS
#undef BIT
}

void or_myers_batch_lanes(const uint8_t *p, uint64_t m, const uint8_t *texts,
                          const uint64_t *offs, const uint64_t *lens, uint64_t count,
                          int lanes, int mode, uint32_t k, int64_t *out) {
    uint64_t *peq = myers_peq(p, m);
    if (lanes < 1) lanes = 1;
    if (lanes > 64) lanes = 64;
    for (uint64_t q = 0; q < count; q += (uint64_t)lanes) {
        int L = (int)umin((uint64_t)lanes, count - q);
        if (m == 0) {
            for (int l = 0; l < L; l++) out[q + l] = myers_with(peq, 0, NULL, lens[q + l], mode, k);
            continue;
        }
        const uint8_t *ptrs[64];
        uint64_t ls[64];
        for (int l = 0; l < L; l++) {
            ptrs[l] = texts + offs[q + l];
            ls[l] = lens[q + l];
        }
        myers_lanes(peq, m, ptrs, ls, L, mode, k, out + q);
    }
    free(peq);
}

/* align.rs:2801-2827 `naive`. */
uint32_t or_myers_naive(const uint8_t *p, uint64_t m, const uint8_t *t, uint64_t n, int mode) {
    uint32_t *prev = malloc((m + 1) * sizeof(uint32_t));
    uint32_t *cur = malloc((m + 1) * sizeof(uint32_t));
    for (uint64_t i = 0; i <= m; i++) prev[i] = (uint32_t)i;
    uint32_t best = (mode == OR_GLOBAL && n > 0) ? UINT32_MAX : prev[m];
    for (uint64_t j = 1; j <= n; j++) {
        cur[0] = mode == OR_INFIX ? 0 : (uint32_t)j;
        for (uint64_t i = 1; i <= m; i++) {
            uint32_t sub = prev[i - 1] + (p[i - 1] != t[j - 1]);
            uint32_t v = sub;
            if (prev[i] + 1 < v) v = prev[i] + 1;
            if (cur[i - 1] + 1 < v) v = cur[i - 1] + 1;
            cur[i] = v;
        }
        if (mode == OR_GLOBAL) {
            if (j == n) best = cur[m];
        } else if (cur[m] < best) {
            best = cur[m];
        }
        uint32_t *tmp = prev;
        prev = cur;
        cur = tmp;
    }
    free(prev);
    free(cur);
    return best;
}

/* ======================================================================
 * Affine rows
 * ====================================================================== */

/* align.rs:988-995 `excl_prefix_max`. */
static inline void excl_prefix_max(int32_t *xs, uint64_t w, int32_t init) {
    int32_t g = init;
    for (uint64_t k = 0; k < w; k++) {
        int32_t next = max32(g, xs[k]);
        xs[k] = g;
        g = next;
    }
}

/* Optional per-cell record for the traceback oracle: x = H without
 * horizontal gaps, and E, for the w cells of a row. */
typedef struct {
    int32_t *x, *e;
} row_rec;

/* align.rs:1027-1072 `row_scalar`.  hprev: w + 1 cells, fu/tx: w cells,
 * nh/nf: w + 1 cells (the last is the NEG sentinel). */
static int32_t row_scalar(const int32_t *hprev, const int32_t *fu, const uint8_t *tx,
                          int32_t *nh, int32_t *nf, uint64_t w, uint8_t c, int32_t mat,
                          int32_t mis, int32_t go, int32_t ext, int32_t e, int32_t floor_,
                          int32_t *hp, int32_t *gs, row_rec *rec) {
    nh[w] = NEG;
    nf[w] = NEG;
    for (uint64_t k = 0; k < w; k++) {
        int32_t fj = max32(max32(wsub(hprev[k + 1], go), wsub(fu[k], ext)), NEG);
        int32_t s = c == (tx[k] & 3) ? mat : -mis;
        int32_t x = max32(max32(wadd(hprev[k], s), fj), floor_);
        hp[k] = x;
        gs[k] = wadd(wsub(x, go), wmul(ext, (int32_t)k + 1));
        nf[k] = fj;
    }
    excl_prefix_max(gs, w, e);
    int32_t m = NEG;
    for (uint64_t k = 0; k < w; k++) {
        int32_t ek = wsub(gs[k], wmul(ext, (int32_t)k));
        int32_t v = max32(hp[k], ek);
        nh[k] = v;
        m = max32(m, v);
        if (rec) {
            rec->x[k] = hp[k];
            rec->e[k] = ek;
        }
    }
    return m;
}

#if defined(__aarch64__)
/* align.rs:1101-1125 `cells_scalar`. */
static int32_t cells_scalar(const int32_t *hprev, const int32_t *fu, const uint8_t *tx,
                            int32_t *nh, int32_t *nf, uint64_t w, uint8_t c, int32_t mat,
                            int32_t mis, int32_t go, int32_t ext, int32_t floor_, uint64_t k0,
                            int32_t carry, int32_t m) {
    for (uint64_t k = k0; k < w; k++) {
        int32_t fj = max32(max32(wsub(hprev[k + 1], go), wsub(fu[k], ext)), NEG);
        int32_t s = c == (tx[k] & 3) ? mat : -mis;
        int32_t x = max32(max32(wadd(hprev[k], s), fj), floor_);
        int32_t v = max32(x, wsub(carry, wmul(ext, (int32_t)k)));
        carry = max32(carry, wadd(wsub(x, go), wmul(ext, (int32_t)k + 1)));
        nh[k] = v;
        nf[k] = fj;
        m = max32(m, v);
    }
    return m;
}

/* align.rs:2023-2085 `row_neon`: 4-lane blocks, the rest by cells_scalar. */
static int32_t row_neon(const int32_t *hprev, const int32_t *fu, const uint8_t *tx,
                        int32_t *nh, int32_t *nf, uint64_t w, uint8_t c, int32_t mat,
                        int32_t mis, int32_t go, int32_t ext, int32_t e, int32_t floor_) {
    nh[w] = NEG;
    nf[w] = NEG;
    int32x4_t neg = vdupq_n_s32(NEG), vfloor = vdupq_n_s32(floor_);
    int32x4_t vgo = vdupq_n_s32(go), vext = vdupq_n_s32(ext);
    int32x4_t vmat = vdupq_n_s32(mat), vmis = vdupq_n_s32(-mis);
    uint32x4_t vc = vdupq_n_u32(c), three = vdupq_n_u32(3);
    const int32_t lane[4] = {0, 1, 2, 3};
    int32x4_t ek = vmulq_s32(vld1q_s32(lane), vext);
    int32x4_t step = vdupq_n_s32(4 * ext);
    int32x4_t cv = vdupq_n_s32(e);
    int32x4_t mx = neg;
    uint64_t k = 0;
    while (k + 4 <= w) {
        int32x4_t hd = vld1q_s32(hprev + k), hu = vld1q_s32(hprev + k + 1);
        int32x4_t fv = vld1q_s32(fu + k);
        uint32_t t4;
        memcpy(&t4, tx + k, 4);
        uint32x4_t t = vmovl_u16(vget_low_u16(vmovl_u8(vreinterpret_u8_u32(vdup_n_u32(t4)))));
        t = vandq_u32(t, three);
        int32x4_t fj = vmaxq_s32(vmaxq_s32(vsubq_s32(hu, vgo), vsubq_s32(fv, vext)), neg);
        int32x4_t s = vbslq_s32(vceqq_u32(t, vc), vmat, vmis);
        int32x4_t x = vmaxq_s32(vmaxq_s32(vaddq_s32(hd, s), fj), vfloor);
        int32x4_t g = vaddq_s32(vsubq_s32(x, vgo), vaddq_s32(ek, vext));
        int32x4_t v = vmaxq_s32(g, vextq_s32(neg, g, 3));
        v = vmaxq_s32(v, vextq_s32(neg, v, 2));
        int32x4_t excl = vextq_s32(cv, vmaxq_s32(v, cv), 3);
        cv = vmaxq_s32(cv, vdupq_laneq_s32(v, 3));
        int32x4_t hv = vmaxq_s32(x, vsubq_s32(excl, ek));
        vst1q_s32(nh + k, hv);
        vst1q_s32(nf + k, fj);
        mx = vmaxq_s32(mx, hv);
        ek = vaddq_s32(ek, step);
        k += 4;
    }
    return cells_scalar(hprev, fu, tx, nh, nf, w, c, mat, mis, go, ext, floor_, k,
                        vgetq_lane_s32(cv, 0), vmaxvq_s32(mx));
}
#endif

static _Atomic int g_level = 0;

int or_set_level(int level) {
#if defined(__aarch64__)
    atomic_store(&g_level, level ? 1 : 0);
#else
    (void)level;
    atomic_store(&g_level, 0);
#endif
    return atomic_load(&g_level);
}

int or_get_level(void) { return atomic_load(&g_level); }

/* One row through the active row kernel (the traceback record forces the
 * scalar passes, which expose x and E). */
static inline int32_t row_any(const int32_t *hprev, const int32_t *fu, const uint8_t *tx,
                              int32_t *nh, int32_t *nf, uint64_t w, uint8_t c, int32_t mat,
                              int32_t mis, int32_t go, int32_t ext, int32_t e, int32_t floor_,
                              int32_t *hp, int32_t *gs, row_rec *rec, int level) {
#if defined(__aarch64__)
    if (level == 1 && !rec)
        return row_neon(hprev, fu, tx, nh, nf, w, c, mat, mis, go, ext, e, floor_);
#else
    (void)level;
#endif
    return row_scalar(hprev, fu, tx, nh, nf, w, c, mat, mis, go, ext, e, floor_, hp, gs, rec);
}

/* Per-thread DP rows (align.rs:2145-2171 `DpBuf`). */
typedef struct {
    int32_t *h, *f, *nh, *nf, *hp, *gs;
    uint64_t cap;
} dpbuf;

static __thread dpbuf tls_buf;

static void dpbuf_reserve(dpbuf *b, uint64_t need) {
    if (b->cap >= need) return;
    uint64_t cap = need + need / 2 + 64;
    int32_t **v[6] = {&b->h, &b->f, &b->nh, &b->nf, &b->hp, &b->gs};
    for (int i = 0; i < 6; i++) {
        free(*v[i]);
        *v[i] = malloc(cap * sizeof(int32_t));
    }
    b->cap = cap;
}

/* Traceback record of a whole pass: per row its band and cells. */
typedef struct {
    uint64_t rows_cap;
    uint64_t *lo, *hi;      /* per row */
    uint64_t *off;          /* per row: offset of its band cells in the arrays */
    int32_t *H, *X, *E, *F; /* band cells, row after row */
    uint64_t used, cap;
} pass_rec;

static void rec_row(pass_rec *r, uint64_t i, uint64_t lo, uint64_t hi) {
    r->lo[i] = lo;
    r->hi[i] = hi;
    r->off[i] = r->used;
    uint64_t w = hi + 1 - lo;
    if (r->used + w > r->cap) {
        uint64_t cap = (r->used + w) * 2 + 64;
        r->H = realloc(r->H, cap * sizeof(int32_t));
        r->X = realloc(r->X, cap * sizeof(int32_t));
        r->E = realloc(r->E, cap * sizeof(int32_t));
        r->F = realloc(r->F, cap * sizeof(int32_t));
        r->cap = cap;
    }
    r->used += w;
}

/* align.rs:2446-2666 `run_core` (resume-free: a pass from row 0; the sorted
 * entry points equal separate passes, align.rs:2210-2214 and the reference
 * test `sorted_batch_matches_single`). */
static void run_core(const uint8_t *p, uint64_t m, const uint8_t *t, uint64_t n, int mode,
                     const or_affine_t *sc, uint64_t band, uint64_t geom, int clip, int32_t xdrop,
                     int cell, uint64_t cut, or_dp_t *out, pass_rec *rec, int level) {
    int32_t clip_best = 0;
    uint64_t ci = 0, cj = 0;
    int32_t cut_best = 0;
    int32_t mat = sc->mat, mis = sc->mis, ext = sc->ext;
    int32_t go = sc->open + sc->ext;
    int full = mode == OR_INFIX || band == OR_NOLIMIT;
    uint64_t below = usat_add(band, usat_sub(m, geom));
    uint64_t above = usat_add(band, usat_sub(geom, m));
#define RANGE(i, LO, HI)                                  \
    do {                                                  \
        if (full) {                                       \
            LO = 0;                                       \
            HI = n;                                       \
        } else {                                          \
            LO = usat_sub((i), below);                    \
            HI = umin(usat_add((i), above), n);           \
        }                                                 \
    } while (0)
    dpbuf *b = &tls_buf;
    dpbuf_reserve(b, n + 2);
    int32_t *h = b->h, *f = b->f, *nh = b->nh, *nf = b->nf;
    /* Fresh rows: the reference never reads outside a row's band and its
     * sentinels (align.rs:2490-2494), so stale contents cannot matter. */
    for (uint64_t j = 0; j < n + 2; j++) h[j] = f[j] = nh[j] = nf[j] = NEG;
    uint64_t lo0, hi0;
    RANGE(0, lo0, hi0);
    for (uint64_t j = lo0; j <= hi0; j++)
        h[j] = (j == 0 || mode == OR_INFIX) ? 0 : -(sc->open + wmul(sc->ext, (int32_t)j));
    for (uint64_t j = lo0; j <= hi0; j++) f[j] = NEG;
    if (lo0 > 0) h[lo0 - 1] = f[lo0 - 1] = NEG;
    h[hi0 + 1] = f[hi0 + 1] = NEG;
    if (rec) {
        rec_row(rec, 0, lo0, hi0);
        for (uint64_t j = lo0; j <= hi0; j++) {
            uint64_t o = rec->off[0] + j - lo0;
            rec->H[o] = rec->X[o] = h[j];
            rec->E[o] = rec->F[o] = NEG;
        }
    }
    uint64_t plo = lo0, phi = hi0;
    uint64_t cells = 0, rows = 0;
    row_rec rr = {0, 0};
    for (uint64_t i = 1; i <= m; i++) {
        uint64_t lo, hi;
        RANGE(i, lo, hi);
        if (lo > hi) {
            *out = (or_dp_t){.score = NEG, .score_col = 0, .clip_best = clip_best, .clip_i = ci,
                             .clip_j = cj, .text_read = n, .last_row = i, .cut_best = cut_best,
                             .cut_score = NEG, .cells = cells, .rows = rows};
            return;
        }
        uint8_t c = p[i - 1] & 3;
        uint64_t start = lo;
        int32_t e = NEG, row_max = NEG;
        if (rec) {
            rec_row(rec, i, lo, hi);
            rr.x = rec->X + rec->off[i] + (lo == 0 ? 1 : 0);
            rr.e = rec->E + rec->off[i] + (lo == 0 ? 1 : 0);
        }
        if (lo == 0) {
            int32_t fj = max32(wsub(h[0], go), wsub(f[0], ext));
            nh[0] = fj;
            nf[0] = fj;
            e = wsub(fj, go);
            start = 1;
            row_max = fj;
            if (rec) {
                uint64_t o = rec->off[i];
                rec->X[o] = fj;
                rec->E[o] = NEG;
            }
        }
        cells += hi + 1 - lo;
        rows += 1;
        if (start <= hi) {
            int32_t mm = row_any(&h[start - 1], &f[start], &t[start - 1], &nh[start], &nf[start],
                                 hi - start + 1, c, mat, mis, go, ext, e, NEG, b->hp, b->gs,
                                 rec ? &rr : NULL, level);
            row_max = max32(row_max, mm);
        } else {
            nh[hi + 1] = NEG;
            nf[hi + 1] = NEG;
        }
        if (rec)
            for (uint64_t j = lo; j <= hi; j++) {
                uint64_t o = rec->off[i] + j - lo;
                rec->H[o] = nh[j];
                rec->F[o] = nf[j];
            }
        if (cut != OR_NOLIMIT && lo <= cut) {
            int32_t row;
            if (hi <= cut) {
                row = row_max;
            } else {
                row = NEG;
                for (uint64_t j = lo; j <= cut; j++) row = max32(row, nh[j]);
            }
            cut_best = max32(cut_best, row);
        }
        if (clip) {
            int32_t row = row_max;
            if (row > clip_best) {
                clip_best = row;
                if (cell) {
                    uint64_t j = lo;
                    while (nh[j] != row) j++;
                    ci = i;
                    cj = j;
                }
            }
            if (row < sat_sub32(clip_best, xdrop)) {
                *out = (or_dp_t){.score = NEG, .score_col = 0, .clip_best = clip_best,
                                 .clip_i = ci, .clip_j = cj, .text_read = hi, .last_row = i,
                                 .cut_best = cut_best, .cut_score = NEG, .cells = cells,
                                 .rows = rows};
                return;
            }
        }
        int32_t *tmp = h;
        h = nh;
        nh = tmp;
        tmp = f;
        f = nf;
        nf = tmp;
        plo = lo;
        phi = hi;
    }
    int32_t score;
    uint64_t score_col;
    if (mode == OR_GLOBAL) {
        score = h[n];
        score_col = n;
    } else {
        int32_t x = NEG;
        uint64_t pos = 0;
        int seen = 0;
        for (uint64_t j = plo; j <= phi; j++)
            if (!seen || h[j] > x) {
                x = h[j];
                pos = j - plo;
                seen = 1;
            }
        score = x;
        score_col = plo + pos;
    }
    int32_t cut_score = NEG;
    if (cut != OR_NOLIMIT && plo <= cut) {
        uint64_t e2 = umin(phi, cut);
        for (uint64_t j = plo; j <= e2; j++) cut_score = max32(cut_score, h[j]);
    }
    *out = (or_dp_t){.score = score, .score_col = score_col, .clip_best = clip_best,
                     .clip_i = ci, .clip_j = cj, .text_read = phi, .last_row = m,
                     .cut_best = cut_best, .cut_score = cut_score, .cells = cells, .rows = rows};
#undef RANGE
}

void or_affine_dp(const uint8_t *p, uint64_t m, const uint8_t *t, uint64_t n, int mode,
                  const or_affine_t *sc, uint64_t band, uint64_t geom, int clip, int32_t xdrop,
                  int cell, uint64_t cut, or_dp_t *out) {
    run_core(p, m, t, n, mode, sc, band, geom, clip, xdrop, cell, cut, out, NULL,
             atomic_load(&g_level));
}

/* align.rs:699-701 `affine`. */
int32_t or_affine(const uint8_t *p, uint64_t m, const uint8_t *t, uint64_t n, int mode,
                  const or_affine_t *sc, uint64_t band) {
    or_dp_t d;
    or_affine_dp(p, m, t, n, mode, sc, band, n, 0, 0, 0, OR_NOLIMIT, &d);
    return d.score;
}

/* align.rs:710-729 `affine_extend`. */
int32_t or_affine_extend(const uint8_t *p, uint64_t m, const uint8_t *t, uint64_t n,
                         const or_affine_t *sc, uint64_t band, int32_t end_bonus,
                         int32_t xdrop) {
    or_dp_t d;
    or_affine_dp(p, m, t, n, OR_PREFIX, sc, band, n, 1, xdrop, 0, OR_NOLIMIT, &d);
    return max32(d.clip_best, sat_add32(d.score, end_bonus));
}

/* align.rs:957-982 `affine_extend_window`. */
void or_affine_extend_window(const uint8_t *p, uint64_t m, const uint8_t *t, uint64_t n,
                             uint64_t window, const or_affine_t *sc, uint64_t band,
                             int32_t end_bonus, int32_t xdrop, int64_t *out4) {
    or_dp_t d;
    or_affine_dp(p, m, t, n, OR_PREFIX, sc, band, umax(window, n), 1, xdrop, 1, OR_NOLIMIT,
                 &d);
    int32_t whole = sat_add32(d.score, end_bonus);
    if (d.clip_best >= whole) {
        out4[0] = d.clip_best;
        out4[1] = (int64_t)d.clip_i;
        out4[2] = (int64_t)d.clip_j;
    } else {
        out4[0] = whole;
        out4[1] = (int64_t)m;
        out4[2] = (int64_t)d.score_col;
    }
    out4[3] = (int64_t)d.text_read;
}

/* align.rs:903-949 `affine_extend_sorted_cut_bonus`, one pass per text. */
void or_affine_extend_sorted_cut_bonus(const uint8_t *p, uint64_t m, const uint8_t *texts,
                                       const uint64_t *offs, const uint64_t *lens,
                                       uint64_t count, const or_affine_t *sc, uint64_t band,
                                       int32_t end_bonus, int32_t xdrop, int diagonal,
                                       uint64_t window, uint64_t cut, int track_cut,
                                       int bonus_within_cut, int64_t *out3) {
    for (uint64_t q = 0; q < count; q++) {
        uint64_t n = lens[q];
        uint64_t geom = diagonal ? umin(m, n) : umax(n, window);
        or_dp_t d;
        or_affine_dp(p, m, texts + offs[q], n, OR_PREFIX, sc, band, geom, 1, xdrop,
                     track_cut && cut != OR_NOLIMIT, cut, &d);
        int32_t end = (bonus_within_cut && cut != OR_NOLIMIT)
                          ? max32(d.score, sat_add32(d.cut_score, end_bonus))
                          : sat_add32(d.score, end_bonus);
        int32_t whole = max32(d.clip_best, end);
        uint64_t cols = d.clip_best >= end ? d.clip_j : d.score_col;
        int32_t cutv = cut == OR_NOLIMIT ? whole : max32(d.cut_best, sat_add32(d.cut_score, end_bonus));
        out3[3 * q] = whole;
        out3[3 * q + 1] = cutv;
        out3[3 * q + 2] = (int64_t)cols;
    }
}

/* align.rs:856-861 `affine_sorted`. */
void or_affine_sorted(const uint8_t *p, uint64_t m, const uint8_t *texts, const uint64_t *offs,
                      const uint64_t *lens, uint64_t count, int mode, const or_affine_t *sc,
                      uint64_t band, int32_t *out) {
    for (uint64_t q = 0; q < count; q++)
        out[q] = or_affine(p, m, texts + offs[q], lens[q], mode, sc, band);
}

/* align.rs:741-760, 783-852 `local_band_ends` / `local_band_core`. */
int32_t or_local_band_ends(const uint8_t *read, uint64_t m, const uint8_t *t, uint64_t n,
                           const or_affine_t *sc, int64_t dlo, int64_t dhi, int32_t bonus0,
                           int32_t bonus1) {
    if (m == 0 || dlo > dhi) return 0;
    int32_t go = sc->open + sc->ext, ext = sc->ext;
    uint64_t w = n + 2;
    int32_t *hp = malloc(w * sizeof(int32_t)), *fp = malloc(w * sizeof(int32_t));
    int32_t *h = malloc(w * sizeof(int32_t)), *f = malloc(w * sizeof(int32_t));
    int32_t *tmp1 = malloc(w * sizeof(int32_t)), *tmp2 = malloc(w * sizeof(int32_t));
    for (uint64_t j = 0; j < w; j++) hp[j] = fp[j] = h[j] = f[j] = NEG;
#define CLAMP(v, a, b) ((v) < (a) ? (a) : (v) > (b) ? (b) : (v))
#define RNG(i, LO, HI)                                                   \
    do {                                                                 \
        int64_t l_ = CLAMP((int64_t)(i) + dlo, 0, (int64_t)n + 1);       \
        int64_t h_ = CLAMP((int64_t)(i) + dhi + 1, 0, (int64_t)n + 1);   \
        LO = (uint64_t)l_;                                               \
        HI = (uint64_t)(h_ > l_ ? h_ : l_);                              \
    } while (0)
    uint64_t lo, hi;
    RNG(0, lo, hi);
    for (uint64_t j = lo; j < hi; j++) hp[j] = bonus0;
    int32_t best = 0;
    int level = atomic_load(&g_level);
    for (uint64_t i = 1; i <= m; i++) {
        RNG(i, lo, hi);
        int32_t floor_ = i < m ? 0 : NEG;
        uint64_t start = lo;
        int32_t e = NEG, rowmax = NEG;
        if (lo == 0 && hi > 0) {
            int32_t fj = max32(max32(wsub(hp[0], go), wsub(fp[0], ext)), NEG);
            int32_t v = max32(fj, floor_);
            h[0] = v;
            f[0] = fj;
            start = 1;
            e = wsub(v, go);
            rowmax = v;
        }
        if (start < hi) {
            int32_t r = row_any(&hp[start - 1], &fp[start], &t[start - 1], &h[start], &f[start],
                                hi - start, read[i - 1], sc->mat, sc->mis, go, ext, e, floor_,
                                tmp1, tmp2, NULL, level);
            rowmax = max32(rowmax, r);
        } else {
            h[hi] = NEG;
            f[hi] = NEG;
        }
        best = max32(best, rowmax);
        if (i == m) best = max32(best, sat_add32(rowmax, bonus1));
        int32_t *x = hp;
        hp = h;
        h = x;
        x = fp;
        fp = f;
        f = x;
    }
    free(hp);
    free(fp);
    free(h);
    free(f);
    free(tmp1);
    free(tmp2);
    return best;
#undef RNG
#undef CLAMP
}

/* ======================================================================
 * Naive definitions (reference tests)
 * ====================================================================== */

/* align.rs:2928-2959 `naive_affine`. */
int32_t or_naive_affine(const uint8_t *p, uint64_t m, const uint8_t *t, uint64_t n, int mode,
                        const or_affine_t *sc) {
    int32_t go = sc->open + sc->ext;
    uint64_t cols = n + 1;
    int32_t *h = malloc((m + 1) * cols * sizeof(int32_t));
    int32_t *e = malloc((m + 1) * cols * sizeof(int32_t));
    int32_t *f = malloc((m + 1) * cols * sizeof(int32_t));
    for (uint64_t x = 0; x < (m + 1) * cols; x++) h[x] = e[x] = f[x] = NEG;
#define A(v, i, j) v[(i) * cols + (j)]
    A(h, 0, 0) = 0;
    for (uint64_t j = 1; j <= n; j++) {
        A(h, 0, j) = mode == OR_INFIX ? 0 : -(sc->open + sc->ext * (int32_t)j);
        A(e, 0, j) = A(h, 0, j);
    }
    for (uint64_t i = 1; i <= m; i++) {
        A(h, i, 0) = -(sc->open + sc->ext * (int32_t)i);
        A(f, i, 0) = A(h, i, 0);
        for (uint64_t j = 1; j <= n; j++) {
            A(e, i, j) = max32(A(h, i, j - 1) - go, A(e, i, j - 1) - sc->ext);
            A(f, i, j) = max32(A(h, i - 1, j) - go, A(f, i - 1, j) - sc->ext);
            int32_t s = p[i - 1] == t[j - 1] ? sc->mat : -sc->mis;
            A(h, i, j) = max32(max32(A(h, i - 1, j - 1) + s, A(e, i, j)), A(f, i, j));
        }
    }
    int32_t r;
    if (mode == OR_GLOBAL) {
        r = A(h, m, n);
    } else {
        r = A(h, m, 0);
        for (uint64_t j = 1; j <= n; j++) r = max32(r, A(h, m, j));
    }
#undef A
    free(h);
    free(e);
    free(f);
    return r;
}

/* align.rs:2961-2967 `naive_extend`. */
int32_t or_naive_extend(const uint8_t *p, uint64_t m, const uint8_t *t, uint64_t n,
                        const or_affine_t *sc) {
    int32_t best = INT32_MIN;
    for (uint64_t i = 0; i <= m; i++)
        for (uint64_t j = 0; j <= n; j++)
            best = max32(best, or_naive_affine(p, i, t, j, OR_GLOBAL, sc));
    return best;
}

/* align.rs:2969-2985 `naive_local`. */
int32_t or_naive_local(const uint8_t *p, uint64_t m, const uint8_t *t, uint64_t n,
                       const or_affine_t *sc, int32_t b0, int32_t b1) {
    int32_t best = 0;
    for (uint64_t i0 = 0; i0 < m; i0++)
        for (uint64_t i1 = i0 + 1; i1 <= m; i1++) {
            int32_t ends = b0 * (i0 == 0) + b1 * (i1 == m);
            for (uint64_t j0 = 0; j0 <= n; j0++)
                for (uint64_t j1 = j0; j1 <= n; j1++) {
                    int32_t x = or_naive_affine(p + i0, i1 - i0, t + j0, j1 - j0, OR_GLOBAL, sc);
                    best = max32(best, x + ends);
                }
        }
    return best;
}

/* align.rs:2987-3014 `naive_local_band`. */
int32_t or_naive_local_band(const uint8_t *p, uint64_t m, const uint8_t *t, uint64_t n,
                            const or_affine_t *sc, int64_t dlo, int64_t dhi, int32_t b0,
                            int32_t b1) {
    int32_t go = sc->open + sc->ext;
    uint64_t cols = n + 1;
    int32_t *h = malloc((m + 1) * cols * sizeof(int32_t));
    int32_t *e = malloc((m + 1) * cols * sizeof(int32_t));
    int32_t *f = malloc((m + 1) * cols * sizeof(int32_t));
    for (uint64_t x = 0; x < (m + 1) * cols; x++) h[x] = e[x] = f[x] = NEG;
#define A(v, i, j) v[(i) * cols + (j)]
#define INSIDE(i, j) (((int64_t)(j) - (int64_t)(i)) >= dlo && ((int64_t)(j) - (int64_t)(i)) <= dhi)
    for (uint64_t j = 0; j <= n; j++)
        if (INSIDE(0, j)) A(h, 0, j) = b0;
    int32_t best = 0;
    for (uint64_t i = 1; i <= m; i++)
        for (uint64_t j = 0; j <= n; j++) {
            if (!INSIDE(i, j)) continue;
            A(f, i, j) = max32(A(h, i - 1, j) - go, A(f, i - 1, j) - sc->ext);
            int32_t x = A(f, i, j);
            if (j > 0) {
                A(e, i, j) = max32(A(h, i, j - 1) - go, A(e, i, j - 1) - sc->ext);
                int32_t s = p[i - 1] == t[j - 1] ? sc->mat : -sc->mis;
                x = max32(max32(x, A(e, i, j)), A(h, i - 1, j - 1) + s);
            }
            A(h, i, j) = i < m ? max32(x, 0) : x;
            best = max32(best, A(h, i, j) + (i == m ? b1 : 0));
        }
#undef A
#undef INSIDE
    free(h);
    free(e);
    free(f);
    return best;
}

/* ======================================================================
 * Traceback oracle (no reference counterpart)
 *
 * Records every row of the `run_core` pass and walks back from the end cell.
 * Tie order: H prefers H' (= max(diagonal, vertical)) over E; H' prefers the
 * diagonal over F; E and F prefer opening over extending.  With H' preferred,
 * every E-open lands on a cell whose H equals its H', so four bits per cell
 * (H source, E open, F open) determine the path.
 * ====================================================================== */

typedef struct {
    uint32_t *ops;
    uint64_t n, cap;
    int overflow;
} opbuf;

static void push_op(opbuf *b, int op, uint64_t len) {
    if (len == 0) return;
    if (b->n > 0 && (b->ops[b->n - 1] & 15) == (uint32_t)op) {
        b->ops[b->n - 1] += (uint32_t)(len << 4);
        return;
    }
    if (b->n == b->cap) {
        b->overflow = 1;
        return;
    }
    b->ops[b->n++] = (uint32_t)(len << 4) | (uint32_t)op;
}

static int in_band(const pass_rec *r, uint64_t i, uint64_t j) {
    return j >= r->lo[i] && j <= r->hi[i];
}
static int32_t at(const int32_t *v, const pass_rec *r, uint64_t i, uint64_t j) {
    return in_band(r, i, j) ? v[r->off[i] + j - r->lo[i]] : NEG;
}

void or_affine_traceback(const uint8_t *p, uint64_t m, const uint8_t *t, uint64_t n, int kind,
                         int mode, const or_affine_t *sc, uint64_t band, uint64_t window,
                         int32_t end_bonus, int32_t xdrop, uint32_t *cigar, uint64_t cap,
                         or_tb_t *out) {
    pass_rec rec = {0};
    rec.rows_cap = m + 1;
    rec.lo = malloc((m + 1) * sizeof(uint64_t));
    rec.hi = malloc((m + 1) * sizeof(uint64_t));
    rec.off = malloc((m + 1) * sizeof(uint64_t));
    or_dp_t d;
    uint64_t ei, ej, clip_tail = 0;
    int32_t score;
    memset(out, 0, sizeof(*out));
    if (kind == OR_TB_AFFINE) {
        run_core(p, m, t, n, mode, sc, band, n, 0, 0, 0, OR_NOLIMIT, &d, &rec, 0);
        score = d.score;
        ei = m;
        ej = d.score_col;
    } else {
        run_core(p, m, t, n, OR_PREFIX, sc, band, umax(window, n), 1, xdrop, 1, OR_NOLIMIT, &d,
                 &rec, 0);
        int32_t whole = sat_add32(d.score, end_bonus);
        mode = OR_PREFIX;
        if (d.clip_best >= whole) {
            score = d.clip_best;
            ei = d.clip_i;
            ej = d.clip_j;
            clip_tail = m - ei;
        } else {
            score = whole;
            ei = m;
            ej = d.score_col;
        }
    }
    out->score = score;
    out->end_i = ei;
    out->end_j = ej;
    /* An end cell whose score is NEG-derived has no path. */
    int32_t endh = ei == 0 ? at(rec.H, &rec, 0, ej) : at(rec.H, &rec, ei, ej);
    if (endh <= NEG / 2) {
        out->status = 1;
        goto done;
    }
    uint32_t *rev = malloc((m + n + 4) * sizeof(uint32_t));
    opbuf ob = {rev, 0, m + n + 4, 0};
    push_op(&ob, OR_OP_S, clip_tail);
    int32_t go = sc->open + sc->ext, ext = sc->ext;
    uint64_t i = ei, j = ej;
    int state = 0; /* 0 H, 1 E, 2 F */
    int bad = 0;
    for (;;) {
        if (state == 0) {
            if (i == 0) {
                if (mode == OR_INFIX) {
                    out->text_start = j;
                } else {
                    push_op(&ob, OR_OP_D, j);
                    out->text_start = 0;
                }
                break;
            }
            if (j == 0) {
                push_op(&ob, OR_OP_I, i);
                out->text_start = 0;
                break;
            }
            int32_t x = at(rec.X, &rec, i, j), e = at(rec.E, &rec, i, j);
            if (e > x) {
                state = 1;
                continue;
            }
            int32_t s = (p[i - 1] & 3) == (t[j - 1] & 3) ? sc->mat : -sc->mis;
            int32_t diag = wadd(at(rec.H, &rec, i - 1, j - 1), s);
            int32_t fv = at(rec.F, &rec, i, j);
            if (diag >= fv) {
                push_op(&ob, OR_OP_M, 1);
                i--;
                j--;
            } else {
                state = 2;
            }
        } else if (state == 1) {
            if (j == 0 || !in_band(&rec, i, j - 1)) {
                bad = 1;
                break;
            }
            push_op(&ob, OR_OP_D, 1);
            int32_t xo = at(rec.X, &rec, i, j - 1), eo = at(rec.E, &rec, i, j - 1);
            state = wsub(xo, go) >= wsub(eo, ext) ? 0 : 1;
            j--;
        } else {
            push_op(&ob, OR_OP_I, 1);
            int32_t hu = at(rec.H, &rec, i - 1, j), fu = at(rec.F, &rec, i - 1, j);
            state = wsub(hu, go) >= wsub(fu, ext) ? 0 : 2;
            i--;
        }
    }
    if (bad) {
        out->status = 1;
    } else if (ob.overflow || ob.n > cap) {
        out->status = -1;
        out->n_ops = ob.n;
    } else {
        for (uint64_t q = 0; q < ob.n; q++) cigar[q] = rev[ob.n - 1 - q];
        out->n_ops = ob.n;
    }
    free(rev);
done:
    free(rec.lo);
    free(rec.hi);
    free(rec.off);
    free(rec.H);
    free(rec.X);
    free(rec.E);
    free(rec.F);
}

int64_t or_cigar_score(const uint8_t *p, uint64_t m, const uint8_t *t, uint64_t n,
                       const uint32_t *cigar, uint64_t n_ops, uint64_t text_start,
                       const or_affine_t *sc, uint64_t *p_used, uint64_t *t_end) {
    int64_t s = 0;
    uint64_t i = 0, j = text_start;
    for (uint64_t q = 0; q < n_ops; q++) {
        uint32_t op = cigar[q] & 15, len = cigar[q] >> 4;
        if (op == OR_OP_M) {
            for (uint32_t x = 0; x < len; x++, i++, j++) {
                if (i >= m || j >= n) return INT64_MIN;
                s += (p[i] & 3) == (t[j] & 3) ? sc->mat : -sc->mis;
            }
        } else if (op == OR_OP_I) {
            s -= sc->open + (int64_t)sc->ext * len;
            i += len;
        } else if (op == OR_OP_D) {
            s -= sc->open + (int64_t)sc->ext * len;
            j += len;
        } else if (op == OR_OP_S) {
            i += len;
        } else {
            return INT64_MIN;
        }
    }
    if (p_used) *p_used = i;
    if (t_end) *t_end = j;
    return s;
}

/* ======================================================================
 * CPU baseline driver: all pairs over `threads` workers, one pair per task
 * (the reference maps one read per worker thread).
 * ====================================================================== */

typedef struct {
    int kind, mode;
    uint32_t k;
    const uint32_t *kv;
    const uint8_t *pseq, *tseq;
    const uint64_t *poff, *plen, *toff, *tlen;
    uint64_t count, band;
    const uint64_t *bv;
    const or_affine_t *sc;
    or_extend_opts_t ext;
    int64_t *out;
    uint64_t *cells_out;
    _Atomic uint64_t next;
    _Atomic uint64_t cells;
    int level;
} pair_job;

static void *pair_worker(void *arg) {
    pair_job *j = arg;
    uint64_t cells = 0;
    for (;;) {
        uint64_t q = atomic_fetch_add(&j->next, 1);
        if (q >= j->count) break;
        const uint8_t *p = j->pseq + j->poff[q], *t = j->tseq + j->toff[q];
        uint64_t m = j->plen[q], n = j->tlen[q];
        const uint64_t band = j->bv ? j->bv[q] : j->band;
        uint64_t c;
        if (j->kind == 0) {
            j->out[q] = or_myers_distance(p, m, t, n, j->mode, j->kv ? j->kv[q] : j->k);
            c = m * n;
        } else if (j->kind == 2) {
            /* align.rs:957-982 `affine_extend_window` with the mapper's window
             * x + pad + x / pad_div (map/src/lib.rs:2101). */
            const uint64_t w = m + j->ext.pad + (j->ext.pad_div ? m / j->ext.pad_div : 0);
            or_dp_t d;
            run_core(p, m, t, n, OR_PREFIX, j->sc, band, umax(w, n), 1, j->ext.xdrop, 1,
                     OR_NOLIMIT, &d, NULL, j->level);
            const int32_t whole = sat_add32(d.score, j->ext.end_bonus);
            j->out[q] = d.clip_best >= whole ? d.clip_best : whole;
            c = d.cells;
        } else {
            or_dp_t d;
            run_core(p, m, t, n, j->mode, j->sc, band, n, 0, 0, 0, OR_NOLIMIT, &d, NULL,
                     j->level);
            j->out[q] = d.score;
            c = d.cells;
        }
        if (j->cells_out) j->cells_out[q] = c;
        cells += c;
    }
    atomic_fetch_add(&j->cells, cells);
    return NULL;
}

static void run_workers(void *(*fn)(void *), void *arg, int threads) {
    if (threads < 1) threads = 1;
    if (threads > 512) threads = 512;
    pthread_t tid[512];
    for (int i = 1; i < threads; i++) pthread_create(&tid[i], NULL, fn, arg);
    fn(arg);
    for (int i = 1; i < threads; i++) pthread_join(tid[i], NULL);
}

uint64_t or_run_pairs(int kind, int threads, const uint8_t *pseq, const uint64_t *poff,
                      const uint64_t *plen, const uint8_t *tseq, const uint64_t *toff,
                      const uint64_t *tlen, uint64_t count, int mode, uint32_t k,
                      const uint32_t *kv, const or_affine_t *sc, uint64_t band,
                      const uint64_t *bv, const or_extend_opts_t *ext, int64_t *out,
                      uint64_t *cells_out) {
    pair_job job = {.kind = kind, .mode = mode, .k = k, .kv = kv, .pseq = pseq, .tseq = tseq,
                    .poff = poff, .plen = plen, .toff = toff, .tlen = tlen, .count = count,
                    .band = band, .bv = bv, .sc = sc, .out = out, .cells_out = cells_out,
                    .level = atomic_load(&g_level)};
    if (ext) job.ext = *ext;
    atomic_store(&job.next, 0);
    atomic_store(&job.cells, 0);
    run_workers(pair_worker, &job, threads);
    return atomic_load(&job.cells);
}

/* ======================================================================
 * CIGAR checks of a whole batch (test infrastructure): each pair's ops
 * re-scored with or_cigar_score, on `threads` workers.
 * ====================================================================== */

typedef struct {
    const uint8_t *pseq, *tseq;
    const uint64_t *poff, *plen, *toff, *tlen;
    const uint32_t *ops;
    const uint64_t *cig_off, *text_start, *text_end;
    const uint32_t *n_ops;
    const int32_t *score;
    const or_affine_t *sc;
    uint64_t count;
    int32_t *code;
    _Atomic uint64_t next, bad;
} cigar_job;

static void *cigar_worker(void *arg) {
    cigar_job *j = arg;
    uint64_t bad = 0;
    for (;;) {
        uint64_t q = atomic_fetch_add(&j->next, 1);
        if (q >= j->count) break;
        uint64_t pu = 0, te = 0;
        const int64_t s = or_cigar_score(j->pseq + j->poff[q], j->plen[q], j->tseq + j->toff[q],
                                         j->tlen[q], j->ops + j->cig_off[q], j->n_ops[q],
                                         j->text_start[q], j->sc, &pu, &te);
        int32_t c = 0;
        if (s == INT64_MIN) c = 4;
        else if (pu != j->plen[q]) c = 2;
        else if (te != j->text_end[q]) c = 3;
        else if (s != (int64_t)j->score[q]) c = 1;
        j->code[q] = c;
        bad += c != 0;
    }
    atomic_fetch_add(&j->bad, bad);
    return NULL;
}

uint64_t or_check_cigars(int threads, const uint8_t *pseq, const uint64_t *poff,
                         const uint64_t *plen, const uint8_t *tseq, const uint64_t *toff,
                         const uint64_t *tlen, uint64_t count, const uint32_t *ops,
                         const uint64_t *cig_off, const uint32_t *n_ops,
                         const uint64_t *text_start, const uint64_t *text_end,
                         const int32_t *score, const or_affine_t *sc, int32_t *code) {
    cigar_job job = {.pseq = pseq, .tseq = tseq, .poff = poff, .plen = plen, .toff = toff,
                     .tlen = tlen, .ops = ops, .cig_off = cig_off, .text_start = text_start,
                     .text_end = text_end, .n_ops = n_ops, .score = score, .sc = sc,
                     .count = count, .code = code};
    atomic_store(&job.next, 0);
    atomic_store(&job.bad, 0);
    run_workers(cigar_worker, &job, threads);
    return atomic_load(&job.bad);
}
