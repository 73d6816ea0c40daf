/* gb_serve.c -- request server: factor and solve requests of different sizes
 * served by a pool of worker threads, each with its own cholmod_common and
 * therefore its own CUDA stream, so that requests admitted together run on
 * the device at the same time (gb300_server_* in include/cholmod_gb300.h).
 *
 *   - symbolic analyses are cached by the caller's pattern id: a factor
 *     request for a known pattern copies the cached symbolic factor
 *     (gb300_batch_analyze of one system) instead of analysing again;
 *   - factors stay resident on the device, keyed by the caller's factor id;
 *     a factor request for a resident factor refactorizes it in place (the
 *     plan and device buffers are reused);
 *   - admission: a factor request starts only when its device-memory
 *     estimate fits under the budget; idle resident factors without queued
 *     work are evicted least recently used first to make room.  A resident
 *     factor holds only what its solves use: the update blocks and operand
 *     images of a factorization are scratch of the worker's Common, and
 *     after each factorization the precision the solves do not read is
 *     dropped (gb300_trim_factor); each factor is charged its measured
 *     device bytes (gb300_factor_device_bytes), also after each solve;
 *   - an evicted factor keeps the host copy of its A (within a host budget,
 *     oldest dropped first): a later solve against it factorizes it again
 *     before solving (a readmission), a later factor request refactorizes
 *     it as usual;
 *   - requests of one factor run in arrival order and never concurrently;
 *     queued solve requests of one factor are coalesced into one refined
 *     solve with all their right-hand sides (up to max_rhs columns);
 *   - every solve is the FP32 factor + FP64 refinement to backward error
 *     1e-12 (FP64 fallback as in gb300_solve_refined).
 *
 * No counterpart in the reference library (CHOLMOD is a per-call library;
 * its Common is per-thread state, which is why each worker owns one).
 */
#include <math.h>
#include <pthread.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

#include "gb_internal.h"

enum { REQ_FACTOR = 0, REQ_SOLVE = 1 };

typedef struct gb_sreq {
    int64_t id, factor_id, pattern_id, n;
    int kind, nrhs, status, done, batch_cols, iters;
    cholmod_sparse *A;            /* factor: owned copy of A (lower, CSC) */
    int64_t *perm;                /* factor: owned copy or NULL */
    double *B, *X;                /* solve: owned n x nrhs */
    double arrival, start, finish, berr;
    struct gb_sreq *next_q, *prev_q;  /* pending queue (arrival order) */
    struct gb_sreq *next_f;       /* the pending requests of the same factor id */
    struct gb_sreq *next_h;       /* hash chain */
} gb_sreq;

/* the pending requests of one factor id, in arrival order */
typedef struct gb_sfq {
    int64_t fid;
    int count;
    gb_sreq *head, *tail;
    struct gb_sfq *next_h;
} gb_sfq;

typedef struct gb_sfactor {
    int64_t id, pattern_id, bytes;
    cholmod_factor *L;            /* NULL until its first factorization succeeds */
    cholmod_sparse *A;
    int busy;
    int evicted;                  /* device state released; A kept on the host */
    int64_t est;                  /* device bytes when last resident */
    double last_use;
    struct gb_sfactor *next, *next_h;
} gb_sfactor;

typedef struct gb_spattern {
    int64_t id;
    cholmod_factor *L;            /* symbolic; NULL while being analysed */
    int state;                    /* 0 new, 2 being analysed, 1 ready, -1 failed */
    struct gb_spattern *next, *next_h;
} gb_spattern;

#define GB_SHASH 65536

struct gb300_server {
    pthread_mutex_t mu;
    pthread_cond_t cv;            /* work, completion, pattern ready */
    gb_sreq *qhead, *qtail;
    gb_sreq *hash[GB_SHASH];
    gb_sfactor *factors, *fhash[GB_SHASH];
    gb_spattern *patterns, *phash[GB_SHASH];
    gb_sfq *qhash[GB_SHASH];
    int nslots, ncommons, max_rhs, stop;
    int64_t budget, in_use, evictions, coalesced, served, readmissions;
    int64_t host_budget, host_kept;   /* host bytes of the evicted factors' A */
    pthread_t *th;
    cholmod_common *commons;
};

double gb300_server_now(void)
{
    struct timespec ts;
    clock_gettime(CLOCK_MONOTONIC, &ts);
    return (double)ts.tv_sec + 1e-9 * (double)ts.tv_nsec;
}

static unsigned hslot(int64_t id) { return (unsigned)(((uint64_t)id * 0x9E3779B97F4A7C15ull) >> 48); }

static gb_sreq *req_find(gb300_server *S, int64_t id)
{
    for (gb_sreq *r = S->hash[hslot(id)]; r; r = r->next_h)
        if (r->id == id) return r;
    return NULL;
}

static gb_sfactor *factor_find(gb300_server *S, int64_t id)
{
    for (gb_sfactor *f = S->fhash[hslot(id)]; f; f = f->next_h)
        if (f->id == id) return f;
    return NULL;
}

static void factor_add(gb300_server *S, gb_sfactor *F)
{
    F->next = S->factors;
    S->factors = F;
    const unsigned h = hslot(F->id);
    F->next_h = S->fhash[h];
    S->fhash[h] = F;
}

static void pattern_add(gb300_server *S, gb_spattern *p)
{
    p->next = S->patterns;
    S->patterns = p;
    const unsigned h = hslot(p->id);
    p->next_h = S->phash[h];
    S->phash[h] = p;
}

/* the pending-request list of a factor id (created when create) */
static gb_sfq *fq_get(gb300_server *S, int64_t fid, int create)
{
    const unsigned h = hslot(fid);
    for (gb_sfq *q = S->qhash[h]; q; q = q->next_h)
        if (q->fid == fid) return q;
    if (!create) return NULL;
    gb_sfq *q = calloc(1, sizeof *q);
    if (!q) return NULL;
    q->fid = fid;
    q->next_h = S->qhash[h];
    S->qhash[h] = q;
    return q;
}

static gb_spattern *pattern_find(gb300_server *S, int64_t id)
{
    for (gb_spattern *p = S->phash[hslot(id)]; p; p = p->next_h)
        if (p->id == id) return p;
    return NULL;
}

static void req_free_payload(gb_sreq *r, cholmod_common *c)
{
    if (r->A) gb300_free_sparse(&r->A, c);
    free(r->perm);
    free(r->B);
    r->perm = NULL;
    r->B = NULL;
}

/* admission estimate of a factor's resident device bytes before it was
 * measured: FP32 factor and diagonal-block inverses (about 1.5 xsize
 * entries), the FP64 copy of A in both triangles with its maps (~60 bytes
 * per stored entry of the lower part) and the refinement vectors */
static int64_t estimate_bytes(const cholmod_factor *L, const cholmod_sparse *A)
{
    int64_t nz = A ? (int64_t)((const int64_t *)A->p)[A->ncol] : 0;
    if (!L) return 100 * nz;
    return (int64_t)(6.0 * (double)L->xsize) + 60 * nz + 256 * (int64_t)L->n;
}

static int64_t host_bytes(const cholmod_sparse *A)
{
    return A ? (int64_t)(24 * ((const int64_t *)A->p)[A->ncol] + 8 * (A->ncol + 1)) : 0;
}

static void factor_unlink_free(gb300_server *S, gb_sfactor *victim, cholmod_common *c)
{
    for (gb_sfactor **pp = &S->factors; *pp; pp = &(*pp)->next)
        if (*pp == victim) { *pp = victim->next; break; }
    for (gb_sfactor **pp = &S->fhash[hslot(victim->id)]; *pp; pp = &(*pp)->next_h)
        if (*pp == victim) { *pp = victim->next_h; break; }
    if (victim->L) {
        gb300_release_factor(victim->L, c);
        gb300_free_factor(&victim->L, c);
    }
    gb300_free_sparse(&victim->A, c);
    free(victim);
}

static int pending_for(gb300_server *S, int64_t factor_id)
{
    const gb_sfq *q = fq_get(S, factor_id, 0);
    return q && q->count > 0;
}

/* under S->mu: release the device state of idle factors (least recently
 * used first) until need bytes fit; returns whether they fit.  An evicted
 * factor keeps its A on the host while the host budget allows (the oldest
 * evicted factors are dropped whole beyond it). */
static int make_room(gb300_server *S, int64_t need, cholmod_common *c)
{
    while (S->in_use + need > S->budget) {
        gb_sfactor *victim = NULL;
        for (gb_sfactor *f = S->factors; f; f = f->next) {
            if (f->busy || f->evicted || pending_for(S, f->id)) continue;
            if (!victim || f->last_use < victim->last_use) victim = f;
        }
        if (!victim) return S->in_use + need <= S->budget || S->in_use == 0;
        S->in_use -= victim->bytes;
        S->evictions++;
        if (victim->L) {
            gb300_release_factor(victim->L, c);
            gb300_free_factor(&victim->L, c);
        }
        victim->est = victim->bytes;
        victim->bytes = 0;
        if (!victim->A) { factor_unlink_free(S, victim, c); continue; }
        victim->evicted = 1;
        S->host_kept += host_bytes(victim->A);
        while (S->host_kept > S->host_budget) {
            gb_sfactor *old = NULL;
            for (gb_sfactor *f = S->factors; f; f = f->next)
                if (f->evicted && !f->busy && !pending_for(S, f->id)
                    && (!old || f->last_use < old->last_use)) old = f;
            if (!old) break;
            S->host_kept -= host_bytes(old->A);
            factor_unlink_free(S, old, c);
        }
    }
    return 1;
}

/* under S->mu: bring an evicted factor back under the budget (its device
 * state is rebuilt by the worker that takes it) */
static int readmit(gb300_server *S, gb_sfactor *F, cholmod_common *c)
{
    int64_t need = F->est > 0 ? F->est : estimate_bytes(F->L ? F->L : NULL, F->A);
    if (!make_room(S, need, c)) return 0;
    S->host_kept -= host_bytes(F->A);
    F->evicted = 0;
    F->bytes = need;
    S->in_use += need;
    return 1;
}

/* under S->mu: take r off the pending queue and off its factor id's list,
 * whose first request it is */
static void unlink_req(gb300_server *S, gb_sreq *r)
{
    if (r->prev_q) r->prev_q->next_q = r->next_q; else S->qhead = r->next_q;
    if (r->next_q) r->next_q->prev_q = r->prev_q; else S->qtail = r->prev_q;
    r->next_q = r->prev_q = NULL;
    gb_sfq *q = fq_get(S, r->factor_id, 0);
    if (q && q->head == r) {
        q->head = r->next_f;
        if (!q->head) q->tail = NULL;
        q->count--;
    }
    r->next_f = NULL;
}

/* under S->mu: the next runnable request (and, for a solve, the queued
 * solves of the same factor coalesced behind it), unlinked from the queue.
 * Only the first pending request of a factor id can run (its id's list);
 * lookups of factors, patterns and lists are hashed, so one scan costs
 * O(1) per pending request.  A solve whose factor neither exists nor has
 * a factor request queued before it (never factored, or evicted and
 * dropped) fails here. */
static gb_sreq *take_work(gb300_server *S, gb_sreq **group, int *ngroup, cholmod_common *c)
{
    /* the smallest need that found no room in this scan: a larger one will
     * not find any either (nothing is freed during the scan) */
    int64_t no_room = INT64_MAX;
    for (gb_sreq *r = S->qhead, *nx; r; r = nx) {
        nx = r->next_q;
        /* an earlier queued request of the same factor goes first */
        const gb_sfq *fq = fq_get(S, r->factor_id, 0);
        if (fq && fq->head != r) continue;
        gb_sfactor *F = factor_find(S, r->factor_id);
        if (r->kind == REQ_SOLVE && (!F || (F->evicted && !F->A))) {
            unlink_req(S, r);
            r->status = CHOLMOD_INVALID;
            r->start = r->finish = gb300_server_now();
            r->done = 1;
            S->served++;
            req_free_payload(r, c);
            pthread_cond_broadcast(&S->cv);
            continue;
        }
        gb_spattern *pat = NULL;
        int64_t need = 0;
        int runnable = !(F && F->busy);
        if (runnable && F && F->evicted) {
            /* a request of an evicted factor: a factor request replaces its
             * A, a solve refactorizes the kept one */
            gb_spattern *fp = pattern_find(S, F->pattern_id);
            if (r->kind == REQ_SOLVE && !(fp && fp->state == 1)) runnable = 0;
            else if (F->est >= no_room) runnable = 0;
            else {
                runnable = readmit(S, F, c);
                if (!runnable) no_room = F->est;
            }
            if (runnable && r->kind == REQ_SOLVE) S->readmissions++;
        } else if (runnable && r->kind == REQ_FACTOR && !F) {
            pat = pattern_find(S, r->pattern_id);
            if (pat && pat->state == 2) runnable = 0;   /* being analysed by a worker */
            else {
                need = pat && pat->L ? estimate_bytes(pat->L, r->A)
                                     : (int64_t)40 * ((const int64_t *)r->A->p)[r->A->ncol];
                runnable = need < no_room && make_room(S, need, c);
                if (!runnable && need < no_room) no_room = need;
            }
        }
        if (!runnable) continue;
        gb_sreq *follow = r->next_f;
        unlink_req(S, r);
        *ngroup = 0;
        group[(*ngroup)++] = r;
        if (r->kind == REQ_SOLVE) {
            /* coalesce the queued solves of the same factor that follow, up
             * to a refactorization of it or max_rhs columns */
            int cols = r->nrhs;
            for (gb_sreq *q = follow, *qn; q; q = qn) {
                qn = q->next_f;
                if (q->kind != REQ_SOLVE || q->n != r->n || cols + q->nrhs > S->max_rhs
                    || *ngroup >= 64)
                    break;
                unlink_req(S, q);
                group[(*ngroup)++] = q;
                cols += q->nrhs;
            }
        } else if (!F) {
            /* reserve the factor (and a new pattern) under the lock, so that no
             * other worker takes a request of the same factor or analyses the
             * same pattern meanwhile */
            F = calloc(1, sizeof *F);
            if (!pat) {
                pat = calloc(1, sizeof *pat);
                if (pat) {
                    pat->id = r->pattern_id;
                    pat->state = 0;
                    pattern_add(S, pat);
                }
            }
            if (F) {
                F->id = r->factor_id;
                F->pattern_id = r->pattern_id;
                F->bytes = need;
                factor_add(S, F);
                S->in_use += need;
            }
        }
        if (F) F->busy = 1;
        return r;
    }
    return NULL;
}

/* the factor's measured device bytes replace its charge (after a
 * factorization, first without what only the factorization used) */
static void charge(gb300_server *S, gb_sfactor *F, cholmod_common *c, int trim)
{
    if (!F->L) return;
    if (trim) gb300_trim_factor(F->L, c);
    int64_t bytes = gb300_factor_device_bytes(F->L, c);
    if (bytes <= 0) return;
    pthread_mutex_lock(&S->mu);
    S->in_use += bytes - F->bytes;
    F->bytes = bytes;
    pthread_mutex_unlock(&S->mu);
}

static void run_factor(gb300_server *S, gb_sreq *r, cholmod_common *c)
{
    pthread_mutex_lock(&S->mu);
    gb_spattern *p = pattern_find(S, r->pattern_id);
    gb_sfactor *F = factor_find(S, r->factor_id);
    int analyse = p && p->state == 0 && !p->L;
    if (analyse) p->state = 2;        /* this worker analyses it */
    while (!analyse && p && p->state == 2) pthread_cond_wait(&S->cv, &S->mu);   /* another does */
    pthread_mutex_unlock(&S->mu);
    if (!p || !F) { r->status = CHOLMOD_OUT_OF_MEMORY; return; }
    if (F->pattern_id != r->pattern_id) { r->status = CHOLMOD_INVALID; return; }
    if (analyse) {
        /* first request of this pattern: the symbolic analysis, kept */
        cholmod_factor *Ls = r->perm ? gb300_analyze_perm(r->A, r->perm, c) : NULL;
        pthread_mutex_lock(&S->mu);
        p->L = Ls;
        p->state = Ls ? 1 : -1;
        pthread_cond_broadcast(&S->cv);
        pthread_mutex_unlock(&S->mu);
    }
    if (p->state != 1 || !p->L || p->L->n != r->A->nrow) { r->status = CHOLMOD_INVALID; return; }
    if (!F->L) {
        int32_t zero = 0;
        cholmod_factor *Lp = p->L;
        F->L = gb300_batch_analyze(1, &Lp, 1, &zero, c);      /* a copy of the pattern */
        if (!F->L) { r->status = CHOLMOD_OUT_OF_MEMORY; return; }
    }
    if (F->A) gb300_free_sparse(&F->A, c);
    F->A = r->A;                  /* the factor keeps A for its refined solves */
    r->A = NULL;
    int ok = gb300_factorize_mixed(F->A, F->L, c);
    r->status = ok ? c->status : (c->status ? c->status : CHOLMOD_GPU_PROBLEM);
    charge(S, F, c, 1);
}

/* a readmitted factor: its pattern copied again and its kept A factorized */
static int refactor_kept(gb300_server *S, gb_sfactor *F, cholmod_common *c)
{
    pthread_mutex_lock(&S->mu);
    gb_spattern *p = pattern_find(S, F->pattern_id);
    pthread_mutex_unlock(&S->mu);
    if (!p || p->state != 1 || !p->L || !F->A) return CHOLMOD_INVALID;
    cholmod_factor *Lp = p->L;
    int32_t zero = 0;
    F->L = gb300_batch_analyze(1, &Lp, 1, &zero, c);
    if (!F->L) return CHOLMOD_OUT_OF_MEMORY;
    int ok = gb300_factorize_mixed(F->A, F->L, c);
    int st = ok ? c->status : (c->status ? c->status : CHOLMOD_GPU_PROBLEM);
    charge(S, F, c, 1);
    return st;
}

static void run_solves(gb300_server *S, gb_sreq **g, int ng, cholmod_common *c)
{
    pthread_mutex_lock(&S->mu);
    gb_sfactor *F = factor_find(S, g[0]->factor_id);
    pthread_mutex_unlock(&S->mu);
    if (F && !F->L && F->A) {
        int st = refactor_kept(S, F, c);
        if (st != CHOLMOD_OK) {
            for (int k = 0; k < ng; k++) g[k]->status = st;
            return;
        }
    }
    if (!F || !F->L || !F->A) {
        for (int k = 0; k < ng; k++) g[k]->status = CHOLMOD_INVALID;
        return;
    }
    int64_t n = (int64_t)F->L->n;
    for (int k = 0; k < ng; k++)
        if (g[k]->n != n) {
            for (int q = 0; q < ng; q++) g[q]->status = CHOLMOD_INVALID;
            return;
        }
    int cols = 0;
    for (int k = 0; k < ng; k++) cols += g[k]->nrhs;
    cholmod_dense *B = gb300_allocate_dense(n, cols, n, CHOLMOD_REAL + CHOLMOD_DOUBLE, c);
    if (!B) { for (int k = 0; k < ng; k++) g[k]->status = CHOLMOD_OUT_OF_MEMORY; return; }
    double *bx = B->x;
    int col = 0;
    for (int k = 0; k < ng; k++) {
        memcpy(bx + (int64_t)col * n, g[k]->B, sizeof(double) * n * g[k]->nrhs);
        col += g[k]->nrhs;
    }
    double info[4] = {0, 0, 0, 0};
    cholmod_dense *X = gb300_solve_refined(F->A, F->L, B, 1e-12, info, c);
    int status = X ? c->status : (c->status ? c->status : CHOLMOD_GPU_PROBLEM);
    col = 0;
    for (int k = 0; k < ng; k++) {
        gb_sreq *r = g[k];
        r->status = status;
        r->berr = info[3];
        r->iters = (int)info[0];
        r->batch_cols = cols;
        if (X) {
            r->X = malloc(sizeof(double) * n * r->nrhs);
            if (r->X) memcpy(r->X, (double *)X->x + (int64_t)col * X->d, sizeof(double) * n * r->nrhs);
            else r->status = CHOLMOD_OUT_OF_MEMORY;
        }
        col += r->nrhs;
    }
    gb300_free_dense(&X, c);
    gb300_free_dense(&B, c);
    charge(S, F, c, 0);           /* the solves' work buffers */
}

typedef struct { gb300_server *S; int slot; } gb_warg;

static void *worker(void *arg)
{
    gb300_server *S = ((gb_warg *)arg)->S;
    cholmod_common *c = &S->commons[((gb_warg *)arg)->slot];
    free(arg);
    gb_sreq *group[64];
    int ng = 0;
    pthread_mutex_lock(&S->mu);
    for (;;) {
        gb_sreq *r = NULL;
        while (!S->stop && !(r = take_work(S, group, &ng, c))) pthread_cond_wait(&S->cv, &S->mu);
        if (!r) break;
        pthread_mutex_unlock(&S->mu);
        double t0 = gb300_server_now();
        for (int k = 0; k < ng; k++) group[k]->start = t0;
        if (r->kind == REQ_FACTOR) run_factor(S, r, c);
        else run_solves(S, group, ng, c);
        double t1 = gb300_server_now();
        pthread_mutex_lock(&S->mu);
        gb_sfactor *F = factor_find(S, r->factor_id);
        if (F) { F->busy = 0; F->last_use = t1; }
        for (int k = 0; k < ng; k++) {
            group[k]->finish = t1;
            group[k]->done = 1;
            req_free_payload(group[k], c);
        }
        S->served += ng;
        if (ng > 1) S->coalesced += ng - 1;
        pthread_cond_broadcast(&S->cv);
    }
    pthread_mutex_unlock(&S->mu);
    return NULL;
}

int gb300_server_set_option(gb300_server *S, int option, int64_t value)
{
    if (!S) return FALSE;
    int ok = TRUE;
    pthread_mutex_lock(&S->mu);
    for (int i = 0; i < S->ncommons; i++) ok &= gb300_set_option(&S->commons[i], option, value);
    pthread_mutex_unlock(&S->mu);
    return ok;
}

gb300_server *gb300_server_create(int nslots, int64_t budget_bytes, int max_rhs)
{
    if (nslots < 1 || nslots > 64 || budget_bytes <= 0 || max_rhs < 1) return NULL;
    gb300_server *S = calloc(1, sizeof *S);
    if (!S) return NULL;
    S->nslots = nslots;
    S->budget = budget_bytes;
    S->host_budget = (int64_t)32 << 30;
    S->max_rhs = max_rhs;
    S->th = calloc(nslots, sizeof(pthread_t));
    S->commons = calloc(nslots, sizeof(cholmod_common));
    if (!S->th || !S->commons) { free(S->th); free(S->commons); free(S); return NULL; }
    pthread_mutex_init(&S->mu, NULL);
    pthread_cond_init(&S->cv, NULL);
    int started = 0;
    for (int i = 0; i < nslots; i++) {
        gb300_start(&S->commons[i]);
        S->commons[i].print = 0;
        S->ncommons = i + 1;
        gb_warg *a = malloc(sizeof *a);
        if (!a) break;
        a->S = S;
        a->slot = i;
        if (pthread_create(&S->th[i], NULL, worker, a) != 0) { free(a); break; }
        started++;
    }
    S->nslots = started;
    if (started == 0) { gb300_server_destroy(S); return NULL; }
    return S;
}

static int submit(gb300_server *S, gb_sreq *r)
{
    pthread_mutex_lock(&S->mu);
    if (req_find(S, r->id)) { pthread_mutex_unlock(&S->mu); return CHOLMOD_INVALID; }
    gb_sfq *fq = fq_get(S, r->factor_id, 1);
    if (!fq) { pthread_mutex_unlock(&S->mu); return CHOLMOD_OUT_OF_MEMORY; }
    unsigned h = hslot(r->id);
    r->next_h = S->hash[h];
    S->hash[h] = r;
    r->prev_q = S->qtail;
    r->next_q = NULL;
    if (S->qtail) S->qtail->next_q = r; else S->qhead = r;
    S->qtail = r;
    r->next_f = NULL;
    if (fq->tail) fq->tail->next_f = r; else fq->head = r;
    fq->tail = r;
    fq->count++;
    pthread_cond_broadcast(&S->cv);
    pthread_mutex_unlock(&S->mu);
    return CHOLMOD_OK;
}

int gb300_server_factor(gb300_server *S, int64_t req, int64_t factor_id, int64_t pattern_id,
                        int64_t n, const int64_t *Ap, const int64_t *Ai, const double *Ax,
                        const int64_t *perm, double arrival)
{
    if (!S || n < 0 || !Ap || (n > 0 && (!Ai || !Ax))) return CHOLMOD_INVALID;
    gb_sreq *r = calloc(1, sizeof *r);
    if (!r) return CHOLMOD_OUT_OF_MEMORY;
    cholmod_common *c = &S->commons[0];
    int64_t nz = Ap[n];
    pthread_mutex_lock(&S->mu);       /* commons[0]'s allocator statistics */
    r->A = gb300_allocate_sparse(n, n, nz, 1, 1, -1, CHOLMOD_REAL, c);
    pthread_mutex_unlock(&S->mu);
    if (!r->A) { free(r); return CHOLMOD_OUT_OF_MEMORY; }
    memcpy(r->A->p, Ap, sizeof(int64_t) * (n + 1));
    memcpy(r->A->i, Ai, sizeof(int64_t) * nz);
    memcpy(r->A->x, Ax, sizeof(double) * nz);
    if (perm) {
        r->perm = malloc(sizeof(int64_t) * (n > 0 ? n : 1));
        if (!r->perm) { gb300_free_sparse(&r->A, c); free(r); return CHOLMOD_OUT_OF_MEMORY; }
        memcpy(r->perm, perm, sizeof(int64_t) * n);
    }
    r->id = req;
    r->n = n;
    r->kind = REQ_FACTOR;
    r->factor_id = factor_id;
    r->pattern_id = pattern_id;
    r->arrival = arrival;
    int st = submit(S, r);
    if (st != CHOLMOD_OK) { req_free_payload(r, c); free(r); }
    return st;
}

int gb300_server_solve(gb300_server *S, int64_t req, int64_t factor_id, int64_t n, int nrhs,
                       const double *B, double arrival)
{
    if (!S || n < 0 || nrhs < 1 || nrhs > S->max_rhs || !B) return CHOLMOD_INVALID;
    gb_sreq *r = calloc(1, sizeof *r);
    if (!r) return CHOLMOD_OUT_OF_MEMORY;
    r->B = malloc(sizeof(double) * (n > 0 ? n : 1) * nrhs);
    if (!r->B) { free(r); return CHOLMOD_OUT_OF_MEMORY; }
    memcpy(r->B, B, sizeof(double) * n * nrhs);
    r->id = req;
    r->n = n;
    r->kind = REQ_SOLVE;
    r->factor_id = factor_id;
    r->nrhs = nrhs;
    r->arrival = arrival;
    int st = submit(S, r);
    if (st != CHOLMOD_OK) { free(r->B); free(r); }
    return st;
}

int gb300_server_wait(gb300_server *S, int64_t req, double *X, int64_t ldx, double *out)
{
    if (!S) return CHOLMOD_INVALID;
    pthread_mutex_lock(&S->mu);
    gb_sreq *r = req_find(S, req);
    if (!r) { pthread_mutex_unlock(&S->mu); return CHOLMOD_INVALID; }
    while (!r->done) pthread_cond_wait(&S->cv, &S->mu);
    /* unlink from the hash: a request is waited for once */
    gb_sreq **pp = &S->hash[hslot(req)];
    while (*pp != r) pp = &(*pp)->next_h;
    *pp = r->next_h;
    pthread_mutex_unlock(&S->mu);
    int st = r->status;
    if (out) {
        out[0] = r->arrival; out[1] = r->start; out[2] = r->finish; out[3] = r->berr;
        out[4] = r->iters; out[5] = r->status; out[6] = r->batch_cols;
    }
    if (X && r->X && ldx >= r->n)
        for (int k = 0; k < r->nrhs; k++) memcpy(X + k * ldx, r->X + k * r->n, sizeof(double) * r->n);
    free(r->X);
    free(r);
    return st;
}

int gb300_server_stats(gb300_server *S, double *out, int nout)
{
    if (!S || !out) return FALSE;
    pthread_mutex_lock(&S->mu);
    int64_t nf = 0, np = 0;
    for (gb_sfactor *f = S->factors; f; f = f->next) nf++;
    for (gb_spattern *p = S->patterns; p; p = p->next) np++;
    int64_t ne = 0;
    for (gb_sfactor *f = S->factors; f; f = f->next) ne += f->evicted;
    double v[10] = {(double)S->in_use, (double)S->budget, (double)(nf - ne), (double)np,
                    (double)S->evictions, (double)S->coalesced, (double)S->served,
                    (double)S->readmissions, (double)ne, (double)S->host_kept};
    pthread_mutex_unlock(&S->mu);
    for (int i = 0; i < nout && i < 10; i++) out[i] = v[i];
    return TRUE;
}

int gb300_server_destroy(gb300_server *S)
{
    if (!S) return FALSE;
    pthread_mutex_lock(&S->mu);
    S->stop = 1;
    pthread_cond_broadcast(&S->cv);
    pthread_mutex_unlock(&S->mu);
    for (int i = 0; i < S->nslots; i++) pthread_join(S->th[i], NULL);
    cholmod_common *c = &S->commons[0];
    for (int h = 0; h < GB_SHASH; h++) {
        gb_sreq *r = S->hash[h];
        while (r) {
            gb_sreq *nx = r->next_h;
            req_free_payload(r, c);
            free(r->X);
            free(r);
            r = nx;
        }
    }
    while (S->factors) {
        gb_sfactor *f = S->factors;
        S->factors = f->next;
        gb300_release_factor(f->L, c);
        gb300_free_factor(&f->L, c);
        gb300_free_sparse(&f->A, c);
        free(f);
    }
    while (S->patterns) {
        gb_spattern *p = S->patterns;
        S->patterns = p->next;
        if (p->L) gb300_free_factor(&p->L, c);
        free(p);
    }
    for (int h = 0; h < GB_SHASH; h++) {
        gb_sfq *q = S->qhash[h];
        while (q) {
            gb_sfq *nx = q->next_h;
            free(q);
            q = nx;
        }
    }
    for (int i = 0; i < S->ncommons; i++) gb300_finish(&S->commons[i]);
    pthread_mutex_destroy(&S->mu);
    pthread_cond_destroy(&S->cv);
    free(S->th);
    free(S->commons);
    free(S);
    return TRUE;
}
