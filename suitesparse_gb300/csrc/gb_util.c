/* gb_util.c -- object bookkeeping, errors, options for libcholmod_gb300.
 *
 * Memory that this library hands to the caller (L->x, factor arrays, dense
 * and sparse objects) is allocated the way CHOLMOD allocates it, so that the
 * reference's cholmod_l_free_* can release it: through SuiteSparse_malloc /
 * SuiteSparse_free when the reference's SuiteSparse_config library is loaded
 * in the process (weak references), plain malloc/free otherwise, with
 * Common->malloc_count / memory_inuse / memory_usage maintained as in
 * CHOLMOD/Utility/t_cholmod_malloc.c:40-52.
 */
#include "gb_internal.h"
#include <pthread.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

extern void *SuiteSparse_malloc(size_t nitems, size_t size_of_item) __attribute__((weak));
extern void *SuiteSparse_free(void *p) __attribute__((weak));

void *gb_malloc(size_t n, size_t size, cholmod_common *Common)
{
    if (n == 0) n = 1;
    if (size == 0) size = 1;
    if (n > SIZE_MAX / size) {
        GB_ERROR(CHOLMOD_TOO_LARGE, "problem too large");
        return NULL;
    }
    void *p = SuiteSparse_malloc ? SuiteSparse_malloc(n, size) : malloc(n * size);
    if (!p) {
        GB_ERROR(CHOLMOD_OUT_OF_MEMORY, "out of memory");
        return NULL;
    }
    if (Common) {
        Common->memory_inuse += n * size;
        Common->memory_usage = GB_MAX(Common->memory_usage, Common->memory_inuse);
        Common->malloc_count++;
    }
    return p;
}

void *gb_calloc(size_t n, size_t size, cholmod_common *Common)
{
    void *p = gb_malloc(n, size, Common);
    if (p) memset(p, 0, GB_MAX(n, 1) * GB_MAX(size, 1));
    return p;
}

void *gb_free(size_t n, size_t size, void *p, cholmod_common *Common)
{
    if (p) {
        if (SuiteSparse_free) SuiteSparse_free(p); else free(p);
        if (Common) {
            if (n == 0) n = 1;
            if (size == 0) size = 1;
            Common->malloc_count--;
            Common->memory_inuse -= n * size;
        }
    }
    return NULL;
}

void gb_error(int status, const char *file, int line, const char *msg,
              cholmod_common *Common)
{
    if (!Common) return;
    Common->status = status;
    if (!Common->try_catch) {
        if (Common->print > 0 && status < 0)
            fprintf(stderr, "CHOLMOD(gb300) error: %s (status %d) %s:%d\n",
                    msg, status, file, line);
        if (Common->error_handler)
            Common->error_handler(status, file, line, msg);
    }
}

/* ---- per-Common context ---------------------------------------------------
 * cholmod_common is part of the ABI and cannot grow, so this library's state
 * (options, device context, statistics) lives in a side table keyed by the
 * Common pointer.  gb300_finish removes the entry.                          */

struct gb_ctx_entry {
    cholmod_common *key;
    gb_ctx *ctx;
    struct gb_ctx_entry *next;
};
static struct gb_ctx_entry *ctx_head = NULL;
static pthread_mutex_t ctx_lock = PTHREAD_MUTEX_INITIALIZER;

/* defined in gb_numeric.c */
extern gb_ctx *gb_ctx_new(void);
extern void gb_ctx_delete(gb_ctx *ctx);

gb_ctx *gb_ctx_get(cholmod_common *Common, int create)
{
    gb_ctx *ctx = NULL;
    pthread_mutex_lock(&ctx_lock);
    for (struct gb_ctx_entry *e = ctx_head; e; e = e->next)
        if (e->key == Common) { ctx = e->ctx; break; }
    if (!ctx && create) {
        struct gb_ctx_entry *e = malloc(sizeof *e);
        ctx = gb_ctx_new();
        if (e && ctx) {
            e->key = Common;
            e->ctx = ctx;
            e->next = ctx_head;
            ctx_head = e;
        } else {
            free(e);
            if (ctx) gb_ctx_delete(ctx);
            ctx = NULL;
        }
    }
    pthread_mutex_unlock(&ctx_lock);
    return ctx;
}

static void ctx_remove(cholmod_common *Common)
{
    gb_ctx *ctx = NULL;
    pthread_mutex_lock(&ctx_lock);
    for (struct gb_ctx_entry **pe = &ctx_head; *pe; pe = &(*pe)->next) {
        if ((*pe)->key == Common) {
            struct gb_ctx_entry *e = *pe;
            *pe = e->next;
            ctx = e->ctx;
            free(e);
            break;
        }
    }
    pthread_mutex_unlock(&ctx_lock);
    if (ctx) gb_ctx_delete(ctx);
}

int gb300_start(cholmod_common *Common)
{
    if (!Common) return FALSE;
    memset(Common, 0, sizeof(cholmod_common));
    /* parameter defaults, values of CHOLMOD/Utility/t_cholmod_defaults.c */
    Common->dbound = 0.0;
    Common->grow0 = 1.2;
    Common->grow1 = 1.2;
    Common->grow2 = 5;
    Common->maxrank = 8;
    Common->final_asis = TRUE;
    Common->final_super = TRUE;
    Common->final_ll = FALSE;
    Common->final_pack = TRUE;
    Common->final_monotonic = TRUE;
    Common->final_resymbol = FALSE;
    Common->supernodal = CHOLMOD_AUTO;
    Common->supernodal_switch = 40;
    Common->prefer_upper = TRUE;
    Common->quick_return_if_not_posdef = FALSE;
    Common->metis_nswitch = 3000;
    Common->metis_dswitch = 0.66;
    Common->nrelax[0] = 4;
    Common->nrelax[1] = 16;
    Common->nrelax[2] = 48;
    Common->zrelax[0] = 0.8;
    Common->zrelax[1] = 0.1;
    Common->zrelax[2] = 0.05;
    Common->print = 3;
    Common->selected = EMPTY;
    Common->postorder = TRUE;
    for (int i = 0; i <= CHOLMOD_MAXMETHODS; i++) {
        Common->method[i].ordering = CHOLMOD_AMD;
        Common->method[i].fl = EMPTY;
        Common->method[i].lnz = EMPTY;
        Common->method[i].prune_dense = 10.0;
        Common->method[i].prune_dense2 = -1;
        Common->method[i].aggressive = TRUE;
        Common->method[i].nd_small = 200;
        Common->method[i].nd_compress = TRUE;
        Common->method[i].nd_camd = 1;
        Common->method[i].nd_oksep = 1.0;
    }
    Common->useGPU = EMPTY;
    Common->maxGpuMemFraction = 0.0;
    Common->itype = CHOLMOD_LONG;
    Common->mark = EMPTY;
    Common->blas_ok = TRUE;
    Common->chunk = 128000;
    Common->nthreads_max = 1;
    Common->status = CHOLMOD_OK;
    return TRUE;
}

int gb300_finish(cholmod_common *Common)
{
    if (!Common) return FALSE;
    ctx_remove(Common);
    return TRUE;
}

/* ---- object helpers ------------------------------------------------------- */

static size_t xsize_of(int xdtype)
{
    int dtype = xdtype & 4;
    return dtype == CHOLMOD_SINGLE ? sizeof(float) : sizeof(double);
}

cholmod_sparse *gb300_allocate_sparse(size_t nrow, size_t ncol, size_t nzmax,
    int sorted, int packed, int stype, int xdtype, cholmod_common *Common)
{
    if (!Common) return NULL;
    Common->status = CHOLMOD_OK;
    int xtype = xdtype & 3;
    cholmod_sparse *A = gb_calloc(1, sizeof(cholmod_sparse), Common);
    if (!A) return NULL;
    A->nrow = nrow;
    A->ncol = ncol;
    A->nzmax = GB_MAX(nzmax, 1);
    A->stype = stype;
    A->itype = CHOLMOD_LONG;
    A->xtype = xtype;
    A->dtype = xdtype & 4;
    A->sorted = sorted;
    A->packed = packed;
    A->p = gb_calloc(ncol + 1, sizeof(Int), Common);
    A->i = gb_malloc(A->nzmax, sizeof(Int), Common);
    if (!packed) A->nz = gb_calloc(ncol, sizeof(Int), Common);
    /* complex: (re, im) pairs in x; zomplex: re in x, im in z */
    if (xtype != CHOLMOD_PATTERN)
        A->x = gb_malloc(A->nzmax, xsize_of(xdtype) * (xtype == CHOLMOD_COMPLEX ? 2 : 1), Common);
    if (xtype == CHOLMOD_ZOMPLEX) A->z = gb_malloc(A->nzmax, xsize_of(xdtype), Common);
    if (!A->p || !A->i || (!packed && !A->nz) || (xtype != CHOLMOD_PATTERN && !A->x)
        || (xtype == CHOLMOD_ZOMPLEX && !A->z)) {
        gb300_free_sparse(&A, Common);
        return NULL;
    }
    return A;
}

int gb300_free_sparse(cholmod_sparse **Ah, cholmod_common *Common)
{
    if (!Ah || !*Ah) return TRUE;
    cholmod_sparse *A = *Ah;
    size_t e = A->dtype == CHOLMOD_SINGLE ? sizeof(float) : sizeof(double);
    gb_free(A->ncol + 1, sizeof(Int), A->p, Common);
    gb_free(A->nzmax, sizeof(Int), A->i, Common);
    gb_free(A->ncol, sizeof(Int), A->nz, Common);
    gb_free(A->nzmax, e * (A->xtype == CHOLMOD_COMPLEX ? 2 : 1), A->x, Common);
    gb_free(A->nzmax, e, A->z, Common);
    gb_free(1, sizeof(cholmod_sparse), A, Common);
    *Ah = NULL;
    return TRUE;
}

cholmod_dense *gb300_allocate_dense(size_t nrow, size_t ncol, size_t d,
                                    int xdtype, cholmod_common *Common)
{
    if (!Common) return NULL;
    Common->status = CHOLMOD_OK;
    const int xtype = xdtype & 3;
    if (xtype == CHOLMOD_PATTERN) {
        GB_ERROR(CHOLMOD_INVALID, "a dense matrix has values");
        return NULL;
    }
    if (d < nrow) d = nrow;
    cholmod_dense *X = gb_calloc(1, sizeof(cholmod_dense), Common);
    if (!X) return NULL;
    X->nrow = nrow;
    X->ncol = ncol;
    X->d = d;
    X->nzmax = GB_MAX(d * ncol, 1);
    X->xtype = xtype;
    X->dtype = xdtype & 4;
    X->x = gb_calloc(X->nzmax, xsize_of(xdtype) * (xtype == CHOLMOD_COMPLEX ? 2 : 1), Common);
    if (xtype == CHOLMOD_ZOMPLEX) X->z = gb_calloc(X->nzmax, xsize_of(xdtype), Common);
    if (!X->x || (xtype == CHOLMOD_ZOMPLEX && !X->z)) { gb300_free_dense(&X, Common); return NULL; }
    return X;
}

int gb300_free_dense(cholmod_dense **Xh, cholmod_common *Common)
{
    if (!Xh || !*Xh) return TRUE;
    cholmod_dense *X = *Xh;
    size_t e = X->dtype == CHOLMOD_SINGLE ? sizeof(float) : sizeof(double);
    gb_free(X->nzmax, e * (X->xtype == CHOLMOD_COMPLEX ? 2 : 1), X->x, Common);
    gb_free(X->nzmax, e, X->z, Common);
    gb_free(1, sizeof(cholmod_dense), X, Common);
    *Xh = NULL;
    return TRUE;
}



int gb300_free_factor(cholmod_factor **Lh, cholmod_common *Common)
{
    if (!Lh || !*Lh) return TRUE;
    cholmod_factor *L = *Lh;
    gb_release_factor_state(L);
    size_t n = L->n, ns = L->nsuper;
    size_t e = L->dtype == CHOLMOD_SINGLE ? sizeof(float) : sizeof(double);
    gb_free(n, sizeof(Int), L->Perm, Common);
    gb_free(n, sizeof(Int), L->ColCount, Common);
    gb_free(n, sizeof(Int), L->IPerm, Common);
    gb_free(ns + 1, sizeof(Int), L->super, Common);
    gb_free(ns + 1, sizeof(Int), L->pi, Common);
    gb_free(ns + 1, sizeof(Int), L->px, Common);
    gb_free(L->ssize, sizeof(Int), L->s, Common);
    if (L->x) gb_free(L->xsize, e, L->x, Common);
    gb_free(1, sizeof(cholmod_factor), L, Common);
    *Lh = NULL;
    return TRUE;
}
