/* gb_complex.c -- complex supernodal LL': cholmod_l_super_numeric with A
 * complex or zomplex (L complex) and cholmod_l_super_lsolve / _ltsolve with
 * a complex L (the reference's cs/cd/zs/zd numeric workers,
 * Supernodal/t_cholmod_super_numeric_worker.c with L_ENTRY 2, and its
 * complex sweeps, Supernodal/t_cholmod_super_solve_worker.c).
 *
 * Formulation: the real embedding.  A Hermitian matrix H is the real
 * symmetric matrix R(H) of twice the order in which each entry h is the
 * 2 x 2 block [Re h, -Im h; Im h, Re h].  R is a *-homomorphism (R(GH) =
 * R(G) R(H), R(H^H) = R(H)'), so H = L L^H with a real positive diagonal
 * gives R(H) = R(L) R(L)', and R(L) is lower triangular with a positive
 * diagonal: it is the Cholesky factor of R(H).  Doubling every column and
 * row of L's supernodal pattern gives a supernodal pattern of R(H) (same
 * supernodes, same etree), so the library's real GPU factorization of R(H)
 * on it (one task-graph launch, tensor-core tiles in FP32) yields R(L) up to
 * rounding, and a gather kernel reads L from the first column of each
 * block.  The sweeps run on the embedding of L itself (scattered exactly
 * from L's values): a complex vector stored as (re, im) pairs -- CHOLMOD's
 * complex dense layout -- is the embedded real vector, and R(L) x = b,
 * R(L)' x = b are L x = b and L^H x = b.  The price is twice the arithmetic
 * of a native complex factorization (each block holds re and im twice).
 *
 * As the reference: the imaginary part of A's diagonal is ignored (LAPACK's
 * zpotrf reads the real part only); beta[0] is added to the real part of
 * the diagonal (the imaginary part of beta is not used, worker :509-517);
 * in the A F form the imaginary parts of the diagonal of A F are ignored;
 * the first failing column gives L->minor and the clean-up of the real
 * path (columns from the failing one on are zero).  The complex factor is
 * always copied back to L->x.
 */
#include "gb_plan.h"
#include <pthread.h>
#include <stdlib.h>
#include <string.h>

typedef struct gb_cx {
    const cholmod_factor *L;
    uint64_t key;                /* pattern hash of L when E was built */
    cholmod_factor E;            /* the embedding's supernodal symbolic factor */
    double xdummy[2];            /* E.x: E's values live on the device only */
    const void *src_x;           /* the L->x whose values the device embedding holds */
    int src_dtype;
    void *d_cx;                  /* device copy of L's complex values */
    size_t cx_cap;
    struct gb_cx *next;
} gb_cx;

static gb_cx *cx_head;
static pthread_mutex_t cx_lock = PTHREAD_MUTEX_INITIALIZER;

static void cx_free_symbolic(gb_cx *h)
{
    gb_release_factor_state(&h->E);
    free(h->E.Perm); free(h->E.ColCount); free(h->E.super);
    free(h->E.pi); free(h->E.px); free(h->E.s);
    memset(&h->E, 0, sizeof h->E);
    h->src_x = NULL;
}

int gb_release_complex_shadow(const cholmod_factor *L)
{
    pthread_mutex_lock(&cx_lock);
    gb_cx **pp = &cx_head;
    while (*pp && (*pp)->L != L) pp = &(*pp)->next;
    gb_cx *h = *pp;
    if (h) *pp = h->next;
    pthread_mutex_unlock(&cx_lock);
    if (!h) return FALSE;
    cx_free_symbolic(h);
    if (h->d_cx) cudaFree(h->d_cx);
    free(h);
    return TRUE;
}

/* E = the embedding of L's supernodal pattern: super, pi doubled, px times
 * four, each row r of s as rows 2r, 2r + 1 */
static int embed_symbolic(gb_cx *h, const cholmod_factor *L)
{
    cx_free_symbolic(h);
    const Int n = (Int)L->n, ns = (Int)L->nsuper;
    const Int *Sup = L->super, *Pi = L->pi, *Px = L->px, *Ls = L->s, *CC = L->ColCount;
    const Int ssz = Pi[ns];
    cholmod_factor *E = &h->E;
    E->super = malloc(sizeof(Int) * (ns + 1));
    E->pi = malloc(sizeof(Int) * (ns + 1));
    E->px = malloc(sizeof(Int) * (ns + 1));
    E->s = malloc(sizeof(Int) * GB_MAX(2 * ssz, 1));
    E->Perm = malloc(sizeof(Int) * GB_MAX(2 * n, 1));
    E->ColCount = malloc(sizeof(Int) * GB_MAX(2 * n, 1));
    if (!E->super || !E->pi || !E->px || !E->s || !E->Perm || !E->ColCount) {
        cx_free_symbolic(h);
        return FALSE;
    }
    Int *sup = E->super, *pi = E->pi, *px = E->px, *es = E->s, *perm = E->Perm, *cc = E->ColCount;
    for (Int s = 0; s <= ns; s++) {
        sup[s] = 2 * Sup[s];
        pi[s] = 2 * Pi[s];
        px[s] = 4 * Px[s];
    }
    for (Int q = 0; q < ssz; q++) {
        es[2 * q] = 2 * Ls[q];
        es[2 * q + 1] = 2 * Ls[q] + 1;
    }
    if (ssz == 0) es[0] = 0;
    for (Int k = 0; k < 2 * n; k++) perm[k] = k;
    for (Int k = 0; k < n; k++) {
        const Int c = CC ? CC[k] : 1;
        cc[2 * k] = 2 * c;
        cc[2 * k + 1] = 2 * c - 1;
    }
    E->n = (size_t)(2 * n);
    E->minor = E->n;
    E->nsuper = (size_t)ns;
    E->ssize = (size_t)GB_MAX(2 * ssz, 1);
    E->xsize = (size_t)GB_MAX(px[ns], 1);
    E->maxcsize = 4 * GB_MAX(L->maxcsize, 1);
    E->maxesize = 2 * GB_MAX(L->maxesize, 1);
    E->ordering = CHOLMOD_NATURAL;
    E->is_ll = TRUE;
    E->is_super = TRUE;
    E->is_monotonic = TRUE;
    E->itype = CHOLMOD_LONG;
    E->xtype = CHOLMOD_PATTERN;
    E->dtype = L->dtype;
    h->key = gb_pattern_hash(L);
    return TRUE;
}

/* the embedding of L, built when missing or when L's pattern changed */
static gb_cx *cx_get(const cholmod_factor *L, cholmod_common *Common)
{
    pthread_mutex_lock(&cx_lock);
    gb_cx *h = cx_head;
    while (h && h->L != L) h = h->next;
    if (!h) {
        h = calloc(1, sizeof(gb_cx));
        if (h) { h->L = L; h->next = cx_head; cx_head = h; }
    }
    pthread_mutex_unlock(&cx_lock);
    if (!h) { GB_ERROR(CHOLMOD_OUT_OF_MEMORY, "out of memory"); return NULL; }
    if (!h->E.super || h->key != gb_pattern_hash(L) || h->E.n != 2 * L->n
        || h->E.nsuper != L->nsuper) {
        if (!embed_symbolic(h, L)) { GB_ERROR(CHOLMOD_OUT_OF_MEMORY, "out of memory"); return NULL; }
    }
    return h;
}

/* the real embedding of a complex or zomplex sparse matrix: lower (stype <
 * 0; entries above the diagonal ignored, the imaginary part of the diagonal
 * dropped) or general (stype 0) */
static cholmod_sparse *embed_sparse(const cholmod_sparse *A, cholmod_common *Common)
{
    const Int nr = (Int)A->nrow, nc = (Int)A->ncol;
    const Int *Ap = A->p, *Ai = A->i, *Anz = A->nz;
    const int lower = A->stype < 0, zomplex = A->xtype == CHOLMOD_ZOMPLEX;
    const int single = A->dtype == CHOLMOD_SINGLE;
    Int nz = 0;
    for (Int j = 0; j < nc; j++) {
        const Int p0 = Ap[j], p1 = A->packed ? Ap[j + 1] : p0 + Anz[j];
        for (Int p = p0; p < p1; p++) {
            const Int i = Ai[p];
            if (lower && i < j) continue;
            nz += (lower && i == j) ? 2 : 4;
        }
    }
    cholmod_sparse *S = gb300_allocate_sparse(2 * nr, 2 * nc, GB_MAX(nz, 1), A->sorted, TRUE,
                                              A->stype, CHOLMOD_REAL + A->dtype, Common);
    if (!S) return NULL;
    Int *Sp = S->p, *Si = S->i;
    double *xd = S->x;
    float *xf = S->x;
    Int q = 0;
    for (Int j = 0; j < nc; j++) {
        const Int p0 = Ap[j], p1 = A->packed ? Ap[j + 1] : p0 + Anz[j];
        for (int half = 0; half < 2; half++) {
            const Int c = 2 * j + half;
            Sp[c] = q;
            for (Int p = p0; p < p1; p++) {
                const Int i = Ai[p];
                if (lower && i < j) continue;
                double re, im;
                if (single) {
                    const float *x = A->x, *z = A->z;
                    re = zomplex ? x[p] : x[2 * p];
                    im = zomplex ? z[p] : x[2 * p + 1];
                } else {
                    const double *x = A->x, *z = A->z;
                    re = zomplex ? x[p] : x[2 * p];
                    im = zomplex ? z[p] : x[2 * p + 1];
                }
                /* column 2j: (2i, re), (2i+1, im); column 2j+1: (2i, -im),
                 * (2i+1, re); of a diagonal entry of a lower matrix only
                 * its real part, once per column */
                Int r[2];
                double v[2];
                int m = 0;
                if (lower && i == j) {
                    r[0] = c; v[0] = re; m = 1;
                } else if (half == 0) {
                    r[0] = 2 * i; v[0] = re; r[1] = 2 * i + 1; v[1] = im; m = 2;
                } else {
                    r[0] = 2 * i; v[0] = -im; r[1] = 2 * i + 1; v[1] = re; m = 2;
                }
                for (int t = 0; t < m; t++, q++) {
                    Si[q] = r[t];
                    if (single) xf[q] = (float)v[t];
                    else xd[q] = v[t];
                }
            }
        }
    }
    Sp[2 * nc] = q;
    return S;
}

static size_t esize(int dtype) { return dtype == CHOLMOD_SINGLE ? sizeof(float) : sizeof(double); }

/* the device embedding of the plan holds R(L) for the complex values in
 * h->d_cx: scattered, marked current, its inverses to be formed again */
static int scatter_current(gb_cx *h, gb_plan *P, gb_ctx *ctx, int dtype, const void *src_x)
{
    const int d = dtype == CHOLMOD_SINGLE ? 1 : 0;
    if (gb_launch_cx_scatter((int64_t)P->nsuper, P->d_Super, P->d_Pi, P->d_Px, h->d_cx, P->d_Lx[d],
                             dtype == CHOLMOD_SINGLE ? 4 : 0, ctx->stream) != 0)
        return FALSE;
    P->dev_valid[d] = 1;
    P->dev_valid[1 - d] = 0;
    P->host_x[d] = h->E.x;
    P->linv_valid[d] = 0;
    h->src_x = src_x;
    h->src_dtype = dtype;
    return TRUE;
}

int gb_super_numeric_complex(cholmod_sparse *A, cholmod_sparse *F, double beta[2],
                             cholmod_factor *L, cholmod_common *Common)
{
    Common->status = CHOLMOD_OK;
    const int dtype = A->dtype;
    gb_cx *h = cx_get(L, Common);
    if (!h) return FALSE;
    h->E.dtype = dtype;
    h->E.x = h->xdummy;
    h->E.xtype = CHOLMOD_PATTERN;
    cholmod_sparse *Ae = embed_sparse(A, Common), *Fe = NULL;
    if (Ae && A->stype == 0) Fe = embed_sparse(F, Common);
    if (!Ae || (A->stype == 0 && !Fe)) {
        gb300_free_sparse(&Ae, Common);
        return FALSE;
    }
    gb_ctx *ctx = NULL;
    int32_t anyfail = 0;
    gb_plan *P = gb_numeric_core(Ae, Fe, beta ? beta[0] : 0.0, &h->E, dtype, A->stype == 0,
                                 &anyfail, &ctx, Common);
    gb300_free_sparse(&Ae, Common);
    if (Fe) gb300_free_sparse(&Fe, Common);
    if (!P) return FALSE;
    const size_t e = esize(dtype);
    const Int xs = GB_MAX((Int)L->xsize, 1);
    if (L->xtype == CHOLMOD_PATTERN) {
        L->x = gb_malloc(2 * xs, e, Common);
        if (!L->x) return FALSE;
        L->xtype = CHOLMOD_COMPLEX;
        L->dtype = dtype;
    }
    L->is_ll = TRUE;
    L->minor = L->n;
    /* the first failing column: the same clean-up as the real path */
    int64_t zero_from = xs;
    if (anyfail) {
        int32_t *fail = malloc(sizeof(int32_t) * (P->nsuper + 1));
        if (!fail || cudaMemcpy(fail, P->d_fail, sizeof(int32_t) * P->nsuper,
                                cudaMemcpyDeviceToHost) != cudaSuccess) {
            free(fail);
            GB_ERROR(CHOLMOD_GPU_PROBLEM, "CUDA error");
            return FALSE;
        }
        const Int *Super = L->super, *Pi = L->pi, *Px = L->px;
        for (Int s = 0; s < P->nsuper; s++) {
            if (fail[s] < 0) continue;
            const Int col = fail[s] / 2, info = col + 1, nsrow = Pi[s + 1] - Pi[s];
            const Int keep = (info == 1 || Common->quick_return_if_not_posdef) ? 0 : info - 1;
            zero_from = Px[s] + keep * nsrow;
            L->minor = (size_t)(Super[s] + col);
            break;
        }
        free(fail);
    }
    const int d = dtype == CHOLMOD_SINGLE ? 1 : 0;
    int ok = gb_dev_grow(&h->d_cx, &h->cx_cap, 2 * e * (size_t)xs)
             && gb_launch_cx_gather((int64_t)P->nsuper, P->d_Super, P->d_Pi, P->d_Px, P->d_Lx[d],
                                    h->d_cx, zero_from, dtype == CHOLMOD_SINGLE ? 4 : 0,
                                    ctx->stream) == 0
             && cudaMemcpyAsync(L->x, h->d_cx, 2 * e * (size_t)xs, cudaMemcpyDeviceToHost,
                                ctx->stream) == cudaSuccess
             && scatter_current(h, P, ctx, dtype, L->x)
             && cudaStreamSynchronize(ctx->stream) == cudaSuccess;
    if (!ok) {
        h->src_x = NULL;
        GB_ERROR(CHOLMOD_GPU_PROBLEM, "CUDA error in the complex factorization");
        return FALSE;
    }
    if (L->minor < L->n) GB_ERROR(CHOLMOD_NOT_POSDEF, "matrix not positive definite");
    return Common->status >= CHOLMOD_OK;
}

int gb_super_solve_complex(cholmod_factor *L, cholmod_dense *X, cholmod_dense *E,
                           cholmod_common *Common, int forward)
{
    /* the reference's checks (Supernodal/cholmod_super_solve.c:66-100) */
    if (!X || !E) { GB_ERROR(CHOLMOD_INVALID, "argument missing"); return FALSE; }
    if (X->xtype != CHOLMOD_COMPLEX || E->xtype != CHOLMOD_COMPLEX
        || L->dtype != X->dtype || L->dtype != E->dtype) {
        GB_ERROR(CHOLMOD_INVALID, "L, X and E must have the same xtype and dtype");
        return FALSE;
    }
    if (X->d < X->nrow || L->n != X->nrow) {
        GB_ERROR(CHOLMOD_INVALID, "X and L dimensions must match");
        return FALSE;
    }
    if (E->nzmax < X->ncol * L->maxesize) {
        GB_ERROR(CHOLMOD_INVALID, "workspace E not large enough");
        return FALSE;
    }
    if (!L->is_ll || !L->is_super) { GB_ERROR(CHOLMOD_INVALID, "L not supernodal"); return FALSE; }
    Common->status = CHOLMOD_OK;
    if (L->n == 0 || X->ncol == 0) return TRUE;
    if (!L->x) { GB_ERROR(CHOLMOD_INVALID, "L has no numerical values"); return FALSE; }
    gb_cx *h = cx_get(L, Common);
    if (!h) return FALSE;
    gb_ctx *ctx = gb_ctx_get(Common, 1);
    if (!ctx || !gb_ctx_ready(ctx)) { GB_ERROR(CHOLMOD_GPU_PROBLEM, "no CUDA device"); return FALSE; }
    const int dtype = L->dtype, d = dtype == CHOLMOD_SINGLE ? 1 : 0;
    h->E.dtype = dtype;
    h->E.x = h->xdummy;
    h->E.xtype = CHOLMOD_REAL;
    gb_plan *P = gb_plan_get(&h->E, Common, ctx, 1);
    if (!P) return FALSE;
    if (!(h->src_x == L->x && h->src_dtype == dtype && P->dev_valid[d] && P->host_x[d] == h->E.x)) {
        /* L's values (from this library or not) into the device embedding */
        const size_t e = esize(dtype), xs = (size_t)GB_MAX((Int)L->xsize, 1);
        int ok = (P->d_Lx[d] || cudaMalloc(&P->d_Lx[d], e * (size_t)GB_MAX(P->xsize, 1)) == cudaSuccess)
                 && gb_dev_grow(&h->d_cx, &h->cx_cap, 2 * e * xs)
                 && cudaMemcpyAsync(h->d_cx, L->x, 2 * e * xs, cudaMemcpyHostToDevice,
                                    ctx->stream) == cudaSuccess
                 && scatter_current(h, P, ctx, dtype, L->x);
        if (!ok) {
            cudaGetLastError();
            h->src_x = NULL;
            GB_ERROR(CHOLMOD_GPU_PROBLEM, "CUDA error uploading L");
            return FALSE;
        }
    }
    /* X and E as the real arrays they are: (re, im) pairs */
    cholmod_dense Xr = *X, Er = *E;
    Xr.nrow = 2 * X->nrow;
    Xr.d = 2 * X->d;
    Xr.nzmax = 2 * X->nzmax;
    Xr.xtype = CHOLMOD_REAL;
    Xr.z = NULL;
    Er.nrow = 2 * E->nrow;
    Er.d = 2 * E->d;
    Er.nzmax = 2 * E->nzmax;
    Er.xtype = CHOLMOD_REAL;
    Er.z = NULL;
    return gb_super_solve(&h->E, &Xr, &Er, Common, forward);
}
