/*
 * ORACLE — test infrastructure only. Nothing in the product path links,
 * loads or calls this file; tests/, the smoke check and bench.py's CPU
 * baseline legs use it as the checker.
 *
 * A plain-C restatement of the scalar bit-parallel Levenshtein core of
 * karims/editdist-bench (bitlev's CPU path). Every rule below follows a
 * cited reference location (paths relative to the reference project):
 *
 *   column step (Myers 1999, Hyyro block form) ... csrc/myers.c:22-36
 *   Peq table load / clear ........................ csrc/myers.c:48-56
 *   exact prefix/suffix trimming .................. csrc/myers.c:80-87
 *   pair: trim, shorter string = pattern, empty ... csrc/myers.c:89-99
 *   max_dist k: gap exit + column exit, k+1 ....... csrc/myers.c:101-143
 *   cross: query = pattern, no trimming,
 *          empty query -> (k>=0 && n>k) ? k+1 : n . csrc/edpy.c:91-127
 *   dtype saturation (uint8/uint16) ............... bitlev/_common.py:25-29
 *
 * Besides the distance, the *_trace entry points record, per pair, the
 * work the reference rule performs: trimmed pattern length m', text length
 * n' and the number of text columns e processed before the exit rule fires
 * (0 for a length-gap exit or an empty pattern). These feed the integer-op
 * roofline count and the exit-column labels of the learned scheduler.
 *
 * Parity of this restatement is pinned against the reference's own C core
 * compiled from its sources (oracle/build_oracle.py, `build_ref`) and against the
 * reference's known answers (tests/golden/).
 */
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include <pthread.h>

typedef uint64_t w64;

/* One column of one 64-row block. `hin` in {-1,0,+1} enters at the block's
 * top row; the horizontal delta leaving row `outbit` is returned. */
static inline int orc_step(w64 *pv_io, w64 *mv_io, w64 eq, int hin, int outbit) {
    w64 pv = *pv_io, mv = *mv_io;
    const w64 neg = (w64)(hin < 0), pos = (w64)(hin > 0);
    const w64 xv = eq | mv;
    eq |= neg;                                     /* a -1 carry acts as a match */
    const w64 xh = (((eq & pv) + pv) ^ pv) | eq;
    w64 ph = mv | ~(xh | pv);
    w64 mh = pv & xh;
    const int hout = (int)((ph >> outbit) & 1u) - (int)((mh >> outbit) & 1u);
    ph = (ph << 1) | pos;
    mh = (mh << 1) | neg;
    *pv_io = mh | ~(xv | ph);
    *mv_io = ph & xv;
    return hout;
}

typedef struct {
    w64 *peq;      /* 256 rows x nw words, all zero between patterns */
    w64 *pv, *mv;  /* nw words each */
    int nw;
} orc_ws;

static int ws_open(orc_ws *ws, int64_t max_pattern) {
    int nw = (int)((max_pattern + 63) / 64);
    if (nw < 1) nw = 1;
    ws->nw = nw;
    ws->peq = (w64 *)calloc((size_t)256 * nw, sizeof(w64));
    ws->pv = (w64 *)malloc(sizeof(w64) * nw);
    ws->mv = (w64 *)malloc(sizeof(w64) * nw);
    if (!ws->peq || !ws->pv || !ws->mv) {
        free(ws->peq); free(ws->pv); free(ws->mv);
        return -1;
    }
    return 0;
}

static void ws_close(orc_ws *ws) { free(ws->peq); free(ws->pv); free(ws->mv); }

static void peq_set(orc_ws *ws, const uint8_t *p, int m) {
    for (int i = 0; i < m; i++) ws->peq[(size_t)p[i] * ws->nw + (i >> 6)] |= (w64)1 << (i & 63);
}

static void peq_clear(orc_ws *ws, const uint8_t *p, int m) {
    for (int i = 0; i < m; i++) ws->peq[(size_t)p[i] * ws->nw + (i >> 6)] = 0;
}

/* Distance of the loaded pattern (m >= 1) to text t; k < 0: exact. With
 * k >= 0 returns min(d, k+1) using the reference's two exact exits. *cols
 * receives the number of text columns processed. */
static int run_columns(orc_ws *ws, int m, const uint8_t *t, int n, int k, int *cols) {
    *cols = 0;
    if (k >= 0 && (n > m ? n - m : m - n) > k) return k + 1;
    const int words = (m + 63) >> 6, last = (m - 1) & 63;
    for (int w = 0; w < words; w++) { ws->pv[w] = ~(w64)0; ws->mv[w] = 0; }
    int score = m;
    for (int j = 0; j < n; j++) {
        const w64 *row = ws->peq + (size_t)t[j] * ws->nw;
        int h = 1;                                 /* the top DP row grows by 1 per column */
        for (int w = 0; w + 1 < words; w++) h = orc_step(&ws->pv[w], &ws->mv[w], row[w], h, 63);
        score += orc_step(&ws->pv[words - 1], &ws->mv[words - 1], row[words - 1], h, last);
        *cols = j + 1;
        if (k >= 0 && score - (n - 1 - j) > k) return k + 1;
    }
    return score;
}

static void trim_pair(const uint8_t **a, int *la, const uint8_t **b, int *lb) {
    const int lim = *la < *lb ? *la : *lb;
    int p = 0;
    while (p < lim && (*a)[p] == (*b)[p]) p++;
    int s = 0;
    while (s < lim - p && (*a)[*la - 1 - s] == (*b)[*lb - 1 - s]) s++;
    *a += p; *b += p;
    *la -= p + s; *lb -= p + s;
}

typedef struct { int m, n, cols; } orc_trace_t;

static int pair_one(orc_ws *ws, const uint8_t *a, int la, const uint8_t *b, int lb,
                    int trim, int k, orc_trace_t *tr) {
    if (trim) trim_pair(&a, &la, &b, &lb);
    if (la > lb) { const uint8_t *t = a; a = b; b = t; int x = la; la = lb; lb = x; }
    tr->m = la; tr->n = lb; tr->cols = 0;
    if (k >= 0 && lb - la > k) return k + 1;
    if (la == 0) return lb;
    peq_set(ws, a, la);
    int d = run_columns(ws, la, b, lb, k, &tr->cols);
    peq_clear(ws, a, la);
    return d;
}

static int64_t max_min_len(const int64_t *oa, const int64_t *ob, int64_t lo, int64_t hi) {
    int64_t mx = 0;
    for (int64_t i = lo; i < hi; i++) {
        int64_t x = oa[i + 1] - oa[i], y = ob[i + 1] - ob[i];
        int64_t m = x < y ? x : y;
        if (m > mx) mx = m;
    }
    return mx;
}

static int pairs_range(const uint8_t *ba, const int64_t *oa, const uint8_t *bb, const int64_t *ob,
                       int64_t lo, int64_t hi, int k, int trim, int32_t *out,
                       int32_t *m_out, int32_t *n_out, int32_t *cols_out) {
    orc_ws ws;
    if (ws_open(&ws, max_min_len(oa, ob, lo, hi))) return -1;
    for (int64_t i = lo; i < hi; i++) {
        orc_trace_t tr;
        out[i] = pair_one(&ws, ba + oa[i], (int)(oa[i + 1] - oa[i]), bb + ob[i],
                          (int)(ob[i + 1] - ob[i]), trim, k, &tr);
        if (m_out) m_out[i] = tr.m;
        if (n_out) n_out[i] = tr.n;
        if (cols_out) cols_out[i] = tr.cols;
    }
    ws_close(&ws);
    return 0;
}

/* out[i] = d(a_i, b_i), or min(d, k+1) for k >= 0. Returns 0, or -1 when a
 * workspace allocation fails. */
int orc_pairs(const uint8_t *ba, const int64_t *oa, const uint8_t *bb, const int64_t *ob,
              int64_t n, int32_t k, int32_t trim, int32_t *out) {
    return pairs_range(ba, oa, bb, ob, 0, n, k, trim, out, NULL, NULL, NULL);
}

/* orc_pairs plus the per-pair work record (m', n', columns processed). */
int orc_pairs_trace(const uint8_t *ba, const int64_t *oa, const uint8_t *bb, const int64_t *ob,
                    int64_t n, int32_t k, int32_t trim, int32_t *out,
                    int32_t *m_trim, int32_t *n_trim, int32_t *cols) {
    return pairs_range(ba, oa, bb, ob, 0, n, k, trim, out, m_trim, n_trim, cols);
}

static int cross_rows(const uint8_t *bq, const int64_t *oq, int64_t q0, int64_t q1,
                      const uint8_t *bc, const int64_t *oc, int64_t nc, int k, int32_t *out,
                      int32_t *cols_out) {
    int64_t mx = 0;
    for (int64_t i = q0; i < q1; i++) if (oq[i + 1] - oq[i] > mx) mx = oq[i + 1] - oq[i];
    orc_ws ws;
    if (ws_open(&ws, mx)) return -1;
    for (int64_t i = q0; i < q1; i++) {
        const uint8_t *q = bq + oq[i];
        const int m = (int)(oq[i + 1] - oq[i]);
        int32_t *row = out + i * nc;
        int32_t *crow = cols_out ? cols_out + i * nc : NULL;
        if (m == 0) {
            for (int64_t j = 0; j < nc; j++) {
                const int n = (int)(oc[j + 1] - oc[j]);
                row[j] = (k >= 0 && n > k) ? k + 1 : n;
                if (crow) crow[j] = 0;
            }
            continue;
        }
        peq_set(&ws, q, m);
        for (int64_t j = 0; j < nc; j++) {
            int c = 0;
            row[j] = run_columns(&ws, m, bc + oc[j], (int)(oc[j + 1] - oc[j]), k, &c);
            if (crow) crow[j] = c;
        }
        peq_clear(&ws, q, m);
    }
    ws_close(&ws);
    return 0;
}

/* Row-major nq x nc matrix out[i*nc + j] = d(q_i, c_j) (min(d, k+1) for k >= 0). */
int orc_cross(const uint8_t *bq, const int64_t *oq, int64_t nq, const uint8_t *bc,
              const int64_t *oc, int64_t nc, int32_t k, int32_t *out) {
    return cross_rows(bq, oq, 0, nq, bc, oc, nc, k, out, NULL);
}

/* orc_cross plus the number of text columns processed per (query, choice). */
int orc_cross_trace(const uint8_t *bq, const int64_t *oq, int64_t nq, const uint8_t *bc,
                    const int64_t *oc, int64_t nc, int32_t k, int32_t *out, int32_t *cols) {
    return cross_rows(bq, oq, 0, nq, bc, oc, nc, k, out, cols);
}

/* Saturating conversion of int32 results to uint16 / uint8 (dtype code 1 / 2). */
void orc_saturate(const int32_t *in, int64_t n, int32_t dtype, void *out) {
    if (dtype == 1) {
        uint16_t *o = (uint16_t *)out;
        for (int64_t i = 0; i < n; i++) o[i] = (uint16_t)(in[i] > 65535 ? 65535 : in[i]);
    } else if (dtype == 2) {
        uint8_t *o = (uint8_t *)out;
        for (int64_t i = 0; i < n; i++) o[i] = (uint8_t)(in[i] > 255 ? 255 : in[i]);
    } else {
        memcpy(out, in, sizeof(int32_t) * (size_t)n);
    }
}

/* ---- threaded drivers for the CPU baseline: contiguous pair ranges or
 *      query-row ranges, one per thread (the split the reference's own
 *      one-process-per-core plan uses). ---------------------------------- */
typedef struct {
    int kind;                 /* 0 pairs, 1 cross */
    const uint8_t *ba, *bb;
    const int64_t *oa, *ob;
    int64_t lo, hi, nc;
    int k, trim, rc;
    int32_t *out;
} orc_job;

static void *orc_worker(void *arg) {
    orc_job *j = (orc_job *)arg;
    if (j->kind == 0)
        j->rc = pairs_range(j->ba, j->oa, j->bb, j->ob, j->lo, j->hi, j->k, j->trim, j->out,
                            NULL, NULL, NULL);
    else
        j->rc = cross_rows(j->ba, j->oa, j->lo, j->hi, j->bb, j->ob, j->nc, j->k, j->out, NULL);
    return NULL;
}

static int run_jobs(orc_job *base, int64_t total, int threads) {
    if (threads < 1) threads = 1;
    if (threads > 1024) threads = 1024;
    if ((int64_t)threads > total) threads = total > 0 ? (int)total : 1;
    orc_job *jobs = (orc_job *)malloc(sizeof(orc_job) * threads);
    pthread_t *tid = (pthread_t *)malloc(sizeof(pthread_t) * threads);
    char *live = (char *)calloc((size_t)threads, 1);
    if (!jobs || !tid || !live) { free(jobs); free(tid); free(live); return -1; }
    int rc = 0;
    for (int t = 0; t < threads; t++) {
        jobs[t] = *base;
        jobs[t].lo = total * t / threads;
        jobs[t].hi = total * (t + 1) / threads;
        jobs[t].rc = 0;
        if (t == threads - 1 || pthread_create(&tid[t], NULL, orc_worker, &jobs[t]) != 0)
            orc_worker(&jobs[t]);               /* the calling thread takes the last range */
        else
            live[t] = 1;
    }
    for (int t = 0; t < threads; t++)
        if (live[t]) pthread_join(tid[t], NULL);
    for (int t = 0; t < threads; t++) if (jobs[t].rc) rc = jobs[t].rc;
    free(jobs); free(tid); free(live);
    return rc;
}

int orc_pairs_mt(const uint8_t *ba, const int64_t *oa, const uint8_t *bb, const int64_t *ob,
                 int64_t n, int32_t k, int32_t trim, int32_t *out, int32_t threads) {
    orc_job j = {0, ba, bb, oa, ob, 0, n, 0, k, trim, 0, out};
    return run_jobs(&j, n, threads);
}

int orc_cross_mt(const uint8_t *bq, const int64_t *oq, int64_t nq, const uint8_t *bc,
                 const int64_t *oc, int64_t nc, int32_t k, int32_t *out, int32_t threads) {
    orc_job j = {1, bq, bc, oq, oc, 0, nq, nc, k, 0, 0, out};
    return run_jobs(&j, nq, threads);
}
