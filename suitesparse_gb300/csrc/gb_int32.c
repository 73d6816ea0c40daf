/* gb_int32.c -- the int32 entry points cholmod_super_numeric,
 * cholmod_super_lsolve and cholmod_super_ltsolve (cholmod.h:4016, 4037,
 * 4058; the reference builds the same source, Supernodal/
 * cholmod_super_numeric.c and cholmod_super_solve.c, with Int = int32).
 *
 * The GPU path works on int64 indices.  An int32 factor gets an int64
 * shadow: a cholmod_factor whose index arrays (Perm, ColCount, IPerm,
 * super, pi, px, s) are widened copies and whose values are the int32
 * factor's own x.  The shadow is kept per factor (keyed by its address) so
 * that the plan built for the pattern, keyed by the shadow, serves every
 * refactorization and solve; its arrays are refreshed from the int32
 * factor on each call (a changed pattern changes their contents, which the
 * plan's fingerprint detects).  An int32 sparse matrix is widened for the
 * call only; its values are not copied.  Results and status are those of
 * the int64 path.  gb300_release_factor(L) drops the shadow.
 */
#include "gb_internal.h"
#include <pthread.h>
#include <stdlib.h>
#include <string.h>

typedef struct gb_shadow {
    const cholmod_factor *L32;
    cholmod_factor F;                /* int64 shadow */
    size_t cap[7];                   /* entries allocated per index array */
    struct gb_shadow *next;
} gb_shadow;

static gb_shadow *shadow_head;
static pthread_mutex_t shadow_lock = PTHREAD_MUTEX_INITIALIZER;

/* dst (int64, resized to n entries) = src (int32); NULL src gives NULL */
static int widen(void **dst, size_t *cap, const void *src, size_t n)
{
    if (!src) {
        free(*dst);
        *dst = NULL;
        *cap = 0;
        return TRUE;
    }
    if (*cap < n || !*dst) {
        free(*dst);
        *dst = malloc(sizeof(int64_t) * (n ? n : 1));
        *cap = *dst ? n : 0;
        if (!*dst) return FALSE;
    }
    const int32_t *s = src;
    int64_t *d = *dst;
    for (size_t k = 0; k < n; k++) d[k] = s[k];
    return TRUE;
}

static void shadow_free(gb_shadow *h)
{
    gb_release_factor_state(&h->F);
    free(h->F.Perm); free(h->F.ColCount); free(h->F.IPerm);
    free(h->F.super); free(h->F.pi); free(h->F.px); free(h->F.s);
    free(h);
}

/* The shadow of L (created on first use), its index arrays refreshed and
 * its scalar fields and values pointer copied from L. */
static cholmod_factor *shadow_get(cholmod_factor *L)
{
    pthread_mutex_lock(&shadow_lock);
    gb_shadow *h = shadow_head;
    while (h && h->L32 != L) h = h->next;
    if (!h) {
        h = calloc(1, sizeof(gb_shadow));
        if (h) {
            h->L32 = L;
            h->next = shadow_head;
            shadow_head = h;
        }
    }
    pthread_mutex_unlock(&shadow_lock);
    if (!h) return NULL;
    cholmod_factor *F = &h->F;
    void *keep[7] = {F->Perm, F->ColCount, F->IPerm, F->super, F->pi, F->px, F->s};
    *F = *L;                                   /* sizes, flags, x, z */
    F->Perm = keep[0]; F->ColCount = keep[1]; F->IPerm = keep[2];
    F->super = keep[3]; F->pi = keep[4]; F->px = keep[5]; F->s = keep[6];
    F->itype = CHOLMOD_LONG;
    F->p = F->i = F->nz = F->next = F->prev = NULL;
    const size_t n = L->n, ns1 = L->nsuper + 1;
    int ok = widen(&F->Perm, &h->cap[0], L->Perm, n)
             && widen(&F->ColCount, &h->cap[1], L->ColCount, n)
             && widen(&F->IPerm, &h->cap[2], L->IPerm, n)
             && widen(&F->super, &h->cap[3], L->super, ns1)
             && widen(&F->pi, &h->cap[4], L->pi, ns1)
             && widen(&F->px, &h->cap[5], L->px, ns1)
             && widen(&F->s, &h->cap[6], L->s, L->ssize);
    return ok ? F : NULL;
}

/* after the int64 call: what it changed in the shadow goes back to L */
static void shadow_put(cholmod_factor *L, const cholmod_factor *F)
{
    L->x = F->x;
    L->z = F->z;
    L->xtype = F->xtype;
    L->dtype = F->dtype;
    L->is_ll = F->is_ll;
    L->minor = F->minor;
    L->xsize = F->xsize;
}

int gb_release_int32_shadow(const cholmod_factor *L)
{
    pthread_mutex_lock(&shadow_lock);
    gb_shadow **pp = &shadow_head;
    while (*pp && (*pp)->L32 != L) pp = &(*pp)->next;
    gb_shadow *h = *pp;
    if (h) *pp = h->next;
    pthread_mutex_unlock(&shadow_lock);
    if (!h) return FALSE;
    shadow_free(h);
    return TRUE;
}

/* an int64 view of an int32 sparse matrix: widened p, i, nz; shared x, z */
static cholmod_sparse *widen_sparse(const cholmod_sparse *A, cholmod_sparse *W)
{
    *W = *A;
    W->itype = CHOLMOD_LONG;
    W->p = W->i = W->nz = NULL;
    size_t c[3] = {0, 0, 0};
    const size_t nnz = A->packed ? (size_t)((const int32_t *)A->p)[A->ncol] : A->nzmax;
    if (!widen(&W->p, &c[0], A->p, A->ncol + 1) || !widen(&W->i, &c[1], A->i, nnz)
        || (!A->packed && !widen(&W->nz, &c[2], A->nz, A->ncol))) {
        free(W->p); free(W->i); free(W->nz);
        return NULL;
    }
    return W;
}

static void free_widened(cholmod_sparse *W)
{
    if (!W) return;
    free(W->p); free(W->i); free(W->nz);
}

int cholmod_super_numeric(cholmod_sparse *A, cholmod_sparse *F, double beta[2], cholmod_factor *L,
                          cholmod_common *Common)
{
    if (!Common) return FALSE;
    if (Common->itype != CHOLMOD_INT) {        /* as the reference's RETURN_IF_NULL_COMMON */
        Common->status = CHOLMOD_INVALID;
        return FALSE;
    }
    if (!A || !L) { GB_ERROR(CHOLMOD_INVALID, "argument missing"); return FALSE; }
    if (A->itype != CHOLMOD_INT || L->itype != CHOLMOD_INT || (F && F->itype != CHOLMOD_INT)) {
        GB_ERROR(CHOLMOD_INVALID, "int32 objects required");
        return FALSE;
    }
    cholmod_sparse A64, F64;
    cholmod_sparse *a = widen_sparse(A, &A64), *f = NULL;
    if (a && F) {
        f = widen_sparse(F, &F64);
        if (!f) { free_widened(a); a = NULL; }
    }
    cholmod_factor *S = a ? shadow_get(L) : NULL;
    if (!S) {
        free_widened(a);
        free_widened(f);
        GB_ERROR(CHOLMOD_OUT_OF_MEMORY, "out of memory");
        return FALSE;
    }
    gb_autotune_first(a, f, beta, S, Common);
    int ok = gb_super_numeric(a, f, beta, S, Common);
    shadow_put(L, S);
    free_widened(a);
    free_widened(f);
    return ok;
}

static int solve32(cholmod_factor *L, cholmod_dense *X, cholmod_dense *E, cholmod_common *Common,
                   int forward)
{
    if (!Common) return FALSE;
    if (Common->itype != CHOLMOD_INT) {
        Common->status = CHOLMOD_INVALID;
        return FALSE;
    }
    if (!L || !X || !E) { GB_ERROR(CHOLMOD_INVALID, "argument missing"); return FALSE; }
    if (L->itype != CHOLMOD_INT) { GB_ERROR(CHOLMOD_INVALID, "int32 factor required"); return FALSE; }
    cholmod_factor *S = shadow_get(L);
    if (!S) { GB_ERROR(CHOLMOD_OUT_OF_MEMORY, "out of memory"); return FALSE; }
    return gb_super_solve(S, X, E, Common, forward);
}

int cholmod_super_lsolve(cholmod_factor *L, cholmod_dense *X, cholmod_dense *E,
                         cholmod_common *Common)
{
    return solve32(L, X, E, Common, 1);
}

int cholmod_super_ltsolve(cholmod_factor *L, cholmod_dense *X, cholmod_dense *E,
                          cholmod_common *Common)
{
    return solve32(L, X, E, Common, 0);
}
