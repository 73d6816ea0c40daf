/* gb_simplicial.c -- cholmod_l_rowfac on the GPU: the simplicial numeric
 * LL' or LDL' factorization that cholmod_l_factorize_p runs when the
 * analysis chose the simplicial method (CHOLMOD/Cholesky/
 * cholmod_factorize.c:285-400 calls cholmod_rowfac(S, F, beta, 0, n, L);
 * the reference computes L row by row, Cholesky/t_cholmod_rowfac_worker.c).
 *
 * Formulation.  The factor's pattern is exact (no explicit zeros), so it is
 * the pattern of a supernodal factor whose supernodes merge only columns
 * with nested patterns.  That supernodal shadow (built once per pattern of
 * S with the relaxation limits at zero, gb_analyze_perm) is factorized by
 * the library's GPU supernodal LL' (one persistent task-graph launch), and
 * a gather kernel writes each column of it into the caller's simplicial
 * layout: L(j,j) and the rows below for LL'; for LDL', D(j,j) = L(j,j)^2 and
 * L(i,j) / L(j,j), the unit lower factor.  Columns from the first failing
 * pivot on are zero and L->minor is that column, as the reference leaves
 * them (rowfac worker :410-433: D(k,k) = 0 and L(k,i) = 0 for i >= minor,
 * the factorization continuing).
 *
 * Layout: a symbolic L is converted as the reference's change_factor does
 * for rowfac (Utility/t_cholmod_change_factor.c, unpacked simplicial):
 * column j starts at the running sum of its allotted space, len =
 * ColCount[j] clamped to [1, n-j] and grown to grow1 len + grow2 (at most
 * n-j), the array ends with grow0 times that total (at most n(n+1)/2);
 * next/prev hold the column order 0..n-1 (head n+1, tail n).  After the
 * call Li and Lnz hold each column's exact rows (sorted, diagonal first).
 *
 * Scope on the GPU (otherwise CHOLMOD_INVALID, with a message): the
 * symmetric case (stype > 0: triu(S) in column form, as factorize_p
 * passes it), real double or single, the whole factorization (kstart = 0,
 * kend = n), no dbound / sbound.  LDL' is formed from LL', so a matrix
 * that is not positive definite stops at its first non-positive pivot
 * (the reference's LDL' goes on through negative pivots and stops only at
 * a zero one).
 */
#include "gb_plan.h"
#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>

typedef struct gb_simp {
    const cholmod_factor *L;
    uint64_t key;                     /* hash of the lower pattern it was built for */
    int64_t n;
    cholmod_common C;                 /* private: the shadow's allocations */
    cholmod_factor *FS;               /* exact-pattern supernodal shadow */
    int64_t *h_src, *h_len;           /* per column: start in FS's values, length */
    int64_t *d_src, *d_dst, *d_len;
    void *d_out;
    size_t out_cap;
    struct gb_simp *next;
} gb_simp;

static gb_simp *simp_head;
static pthread_mutex_t simp_lock = PTHREAD_MUTEX_INITIALIZER;

static uint64_t pattern_key(Int n, const Int *Sp, const Int *Si)
{
    uint64_t h = 1469598103934665603ull ^ (uint64_t)n;
    for (Int j = 0; j <= n; j++) h = (h ^ (uint64_t)Sp[j]) * 1099511628211ull;
    for (Int p = 0; p < Sp[n]; p++) h = (h ^ (uint64_t)Si[p]) * 1099511628211ull;
    return h;
}

static void simp_clear(gb_simp *h)
{
    if (h->FS) {
        gb_release_factor_state(h->FS);
        gb300_free_factor(&h->FS, &h->C);
    }
    free(h->h_src); free(h->h_len);
    h->h_src = h->h_len = NULL;
    if (h->d_src) cudaFree(h->d_src);
    if (h->d_dst) cudaFree(h->d_dst);
    if (h->d_len) cudaFree(h->d_len);
    if (h->d_out) cudaFree(h->d_out);
    h->d_src = h->d_dst = h->d_len = NULL;
    h->d_out = NULL;
    h->out_cap = 0;
}

int gb_release_simplicial_shadow(const cholmod_factor *L)
{
    pthread_mutex_lock(&simp_lock);
    gb_simp **pp = &simp_head;
    while (*pp && (*pp)->L != L) pp = &(*pp)->next;
    gb_simp *h = *pp;
    if (h) *pp = h->next;
    pthread_mutex_unlock(&simp_lock);
    if (!h) return FALSE;
    simp_clear(h);
    free(h);
    return TRUE;
}

/* S (lower, column form) = transpose of the upper-stored A (columns of A
 * are rows of S); entries below A's diagonal are ignored, as the reference
 * ignores them.  Values converted to double (dtype of the factor) stay in
 * A's precision: the result has A's dtype. */
static cholmod_sparse *upper_to_lower(cholmod_sparse *A, cholmod_common *Common)
{
    const Int n = (Int)A->nrow;
    const Int *Ap = A->p, *Ai = A->i, *Anz = A->nz;
    const size_t e = A->dtype == CHOLMOD_SINGLE ? sizeof(float) : sizeof(double);
    Int *cnt = calloc(n + 1, sizeof(Int));
    if (!cnt) { GB_ERROR(CHOLMOD_OUT_OF_MEMORY, "out of memory"); return NULL; }
    Int nz = 0;
    for (Int j = 0; j < n; j++) {
        Int p = Ap[j], pend = A->packed ? Ap[j + 1] : p + Anz[j];
        for (; p < pend; p++) {
            const Int i = Ai[p];
            if (i <= j) { cnt[i]++; nz++; }
        }
    }
    cholmod_sparse *S = gb300_allocate_sparse(n, n, nz, TRUE, TRUE, -1, CHOLMOD_REAL + A->dtype,
                                              Common);
    if (!S) { free(cnt); return NULL; }
    Int *Sp = S->p, *Si = S->i;
    Sp[0] = 0;
    for (Int i = 0; i < n; i++) Sp[i + 1] = Sp[i] + cnt[i];
    for (Int i = 0; i < n; i++) cnt[i] = Sp[i];
    /* columns of A in increasing order: each row list of S comes out sorted */
    for (Int j = 0; j < n; j++) {
        Int p = Ap[j], pend = A->packed ? Ap[j + 1] : p + Anz[j];
        for (; p < pend; p++) {
            const Int i = Ai[p];
            if (i > j) continue;
            const Int q = cnt[i]++;
            Si[q] = j;
            memcpy((char *)S->x + q * e, (const char *)A->x + p * e, e);
        }
    }
    free(cnt);
    /* an unsorted A leaves the rows of S unsorted: sort each column */
    if (!A->sorted) {
        for (Int c = 0; c < n; c++) {
            for (Int p = Sp[c] + 1; p < Sp[c + 1]; p++) {
                Int key = Si[p], q = p - 1;
                char v[8];
                memcpy(v, (char *)S->x + p * e, e);
                while (q >= Sp[c] && Si[q] > key) {
                    Si[q + 1] = Si[q];
                    memcpy((char *)S->x + (q + 1) * e, (char *)S->x + q * e, e);
                    q--;
                }
                Si[q + 1] = key;
                memcpy((char *)S->x + (q + 1) * e, v, e);
            }
        }
    }
    return S;
}

/* the shadow of L for the lower pattern of S, built when missing or stale */
static gb_simp *simp_get(cholmod_factor *L, cholmod_sparse *S, cholmod_common *Common)
{
    const Int n = (Int)S->nrow;
    const uint64_t key = pattern_key(n, S->p, S->i);
    pthread_mutex_lock(&simp_lock);
    gb_simp *h = simp_head;
    while (h && h->L != L) h = h->next;
    if (!h) {
        h = calloc(1, sizeof(gb_simp));
        if (h) { h->L = L; h->next = simp_head; simp_head = h; }
    }
    pthread_mutex_unlock(&simp_lock);
    if (!h) { GB_ERROR(CHOLMOD_OUT_OF_MEMORY, "out of memory"); return NULL; }
    if (h->FS && h->key == key && h->n == n) return h;
    simp_clear(h);
    /* supernodes of columns with nested patterns only: no relaxation */
    memcpy(&h->C, Common, sizeof(cholmod_common));
    for (int k = 0; k < 3; k++) { h->C.nrelax[k] = 0; h->C.zrelax[k] = 0.0; }
    h->C.status = CHOLMOD_OK;
    Int *ident = malloc(sizeof(Int) * (n + 1));
    if (!ident) { GB_ERROR(CHOLMOD_OUT_OF_MEMORY, "out of memory"); return NULL; }
    for (Int k = 0; k < n; k++) ident[k] = k;
    h->FS = gb_analyze_perm(S, ident, &h->C);
    free(ident);
    if (!h->FS) { GB_ERROR(CHOLMOD_OUT_OF_MEMORY, "symbolic analysis of the pattern failed"); return NULL; }
    h->key = key;
    h->n = n;
    const Int *Super = h->FS->super, *Pi = h->FS->pi, *Px = h->FS->px;
    h->h_src = malloc(sizeof(int64_t) * (n + 1));
    h->h_len = malloc(sizeof(int64_t) * (n + 1));
    if (!h->h_src || !h->h_len) { GB_ERROR(CHOLMOD_OUT_OF_MEMORY, "out of memory"); return NULL; }
    for (Int s = 0; s < (Int)h->FS->nsuper; s++) {
        const Int k1 = Super[s], nsrow = Pi[s + 1] - Pi[s];
        for (Int j = k1; j < Super[s + 1]; j++) {
            const Int c = j - k1;
            h->h_src[j] = Px[s] + c * nsrow + c;
            h->h_len[j] = nsrow - c;
        }
    }
    const size_t b = sizeof(int64_t) * (n + 1);
    if (cudaMalloc((void **)&h->d_src, b) != cudaSuccess || cudaMalloc((void **)&h->d_dst, b) != cudaSuccess
        || cudaMalloc((void **)&h->d_len, b) != cudaSuccess
        || cudaMemcpy(h->d_src, h->h_src, b, cudaMemcpyHostToDevice) != cudaSuccess
        || cudaMemcpy(h->d_len, h->h_len, b, cudaMemcpyHostToDevice) != cudaSuccess) {
        cudaGetLastError();
        GB_ERROR(CHOLMOD_GPU_PROBLEM, "device allocation failed");
        return NULL;
    }
    return h;
}

/* the space the reference's change_factor gives column j (grow_column) */
static Int grow_len(Int len, double grow1, double grow2, Int maxlen)
{
    double x = grow1 * (double)len + grow2;
    if (x > (double)maxlen) x = (double)maxlen;
    len = (Int)x;
    if (len < 1) len = 1;
    if (len > maxlen) len = maxlen;
    return len;
}

/* symbolic simplicial L -> numeric, unpacked with slack (see the top) */
static int alloc_simplicial(cholmod_factor *L, int dtype, cholmod_common *Common)
{
    const Int n = (Int)L->n;
    const Int *ColCount = L->ColCount;
    double grow0 = isnan(Common->grow0) ? 1 : Common->grow0;
    double grow1 = isnan(Common->grow1) ? 1 : Common->grow1;
    double grow2 = (double)Common->grow2;
    const int grow = (grow0 >= 1.0) && (grow1 >= 1.0) && (grow2 > 0);
    Int *Lp = L->p ? L->p : gb_malloc(n + 1, sizeof(Int), Common);
    Int *Lnz = L->nz ? L->nz : gb_malloc(n + 1, sizeof(Int), Common);
    Int *Lnext = L->next ? L->next : gb_malloc(n + 2, sizeof(Int), Common);
    Int *Lprev = L->prev ? L->prev : gb_malloc(n + 2, sizeof(Int), Common);
    L->p = Lp; L->nz = Lnz; L->next = Lnext; L->prev = Lprev;
    if (!Lp || !Lnz || !Lnext || !Lprev) return FALSE;
    Int lnz = 0;
    for (Int j = 0; j < n; j++) {
        Lp[j] = lnz;
        Lnz[j] = 1;
        Int len = ColCount ? ColCount[j] : 1;
        if (len < 1) len = 1;
        if (len > n - j) len = n - j;
        if (grow) len = grow_len(len, grow1, grow2, n - j);
        lnz += len;
    }
    Lp[n] = lnz;
    if (grow) {
        double x = (double)lnz * grow0, d = (double)n;
        d = (d * d + d) / 2;
        if (x > d) x = d;
        if ((Int)x > lnz) lnz = (Int)x;
    }
    if (lnz < 1) lnz = 1;
    const size_t e = dtype == CHOLMOD_SINGLE ? sizeof(float) : sizeof(double);
    L->i = gb_malloc(lnz, sizeof(Int), Common);
    L->x = gb_calloc(lnz, e, Common);
    if (!L->i || !L->x) return FALSE;
    L->nzmax = lnz;
    const Int head = n + 1, tail = n;
    Lnext[head] = 0; Lprev[head] = EMPTY;
    Lnext[tail] = EMPTY; Lprev[tail] = n - 1;
    for (Int j = 0; j < n; j++) { Lnext[j] = j + 1; Lprev[j] = j - 1; }
    if (n > 0) Lprev[0] = head;
    if (n == 0) { Lnext[head] = tail; Lprev[tail] = head; }
    L->is_monotonic = TRUE;
    L->xtype = CHOLMOD_REAL;
    L->dtype = dtype;
    L->minor = n;
    return TRUE;
}

int cholmod_l_rowfac(cholmod_sparse *A, cholmod_sparse *F, double beta[2], size_t kstart,
                     size_t kend, cholmod_factor *L, cholmod_common *Common)
{
    /* the reference's argument checks (cholmod_rowfac.c:675-721) */
    if (!Common) return FALSE;
    if (Common->itype != CHOLMOD_LONG) { Common->status = CHOLMOD_INVALID; return FALSE; }
    if (!A || !L) { GB_ERROR(CHOLMOD_INVALID, "argument missing"); return FALSE; }
    if (A->xtype < CHOLMOD_REAL || A->xtype > CHOLMOD_ZOMPLEX || !A->x
        || L->xtype < CHOLMOD_PATTERN || L->xtype > CHOLMOD_ZOMPLEX) {
        GB_ERROR(CHOLMOD_INVALID, "invalid xtype");
        return FALSE;
    }
    if (L->xtype != CHOLMOD_PATTERN && (A->xtype != L->xtype || A->dtype != L->dtype)) {
        GB_ERROR(CHOLMOD_INVALID, "xtype or dtype of A and L do not match");
        return FALSE;
    }
    if (L->is_super) { GB_ERROR(CHOLMOD_INVALID, "can only do simplicial factorization"); return FALSE; }
    if (A->stype == 0) {
        if (!F) { GB_ERROR(CHOLMOD_INVALID, "argument missing"); return FALSE; }
        if (A->xtype != F->xtype) { GB_ERROR(CHOLMOD_INVALID, "xtype of A and F do not match"); return FALSE; }
    }
    if (A->stype < 0) { GB_ERROR(CHOLMOD_INVALID, "symmetric lower not supported"); return FALSE; }
    if (kend > L->n) { GB_ERROR(CHOLMOD_INVALID, "kend invalid"); return FALSE; }
    if (A->nrow != L->n) { GB_ERROR(CHOLMOD_INVALID, "dimensions of A and L do not match"); return FALSE; }
    Common->status = CHOLMOD_OK;
    Common->rowfacfl = 0;
    /* what the GPU path covers */
    if (A->stype == 0) {
        GB_ERROR(CHOLMOD_INVALID, "the A*F' form of the simplicial factorization is not on the GPU path");
        return FALSE;
    }
    if (A->xtype != CHOLMOD_REAL) {
        GB_ERROR(CHOLMOD_INVALID, "complex simplicial factorization is not on the GPU path");
        return FALSE;
    }
    if (A->itype != CHOLMOD_LONG || L->itype != CHOLMOD_LONG) {
        GB_ERROR(CHOLMOD_INVALID, "int64 (cholmod_l_) objects required");
        return FALSE;
    }
    const Int n = (Int)L->n;
    if (!(kstart == 0 && kend == (size_t)n)) {
        GB_ERROR(CHOLMOD_INVALID, "only the whole simplicial factorization (kstart 0, kend n) is on the GPU path");
        return FALSE;
    }
    if (Common->dbound > 0 || Common->sbound > 0) {
        GB_ERROR(CHOLMOD_INVALID, "dbound / sbound are not on the GPU path");
        return FALSE;
    }
    const int dtype = A->dtype;
    if (L->xtype == CHOLMOD_PATTERN) {
        if (!alloc_simplicial(L, dtype, Common)) {
            GB_ERROR(CHOLMOD_OUT_OF_MEMORY, "out of memory");
            return FALSE;
        }
    }
    L->minor = n;
    if (n == 0) return TRUE;
    cholmod_sparse *S = upper_to_lower(A, Common);
    if (!S) return FALSE;
    gb_simp *h = simp_get(L, S, Common);
    if (!h) { gb300_free_sparse(&S, Common); return FALSE; }
    /* the exact pattern into L: rows of each column, diagonal first; the
     * space of every column must hold its count */
    Int *Lp = L->p, *Li = L->i, *Lnz = L->nz, *Lnext = L->next;
    const Int *Super = h->FS->super, *Pi = h->FS->pi, *Ls = h->FS->s;
    int fits = TRUE;
    for (Int s = 0; fits && s < (Int)h->FS->nsuper; s++) {
        for (Int j = Super[s]; j < Super[s + 1]; j++) {
            const Int c = j - Super[s], len = h->h_len[j];
            const Int end = (Lnext && Lnext[j] >= 0 && Lnext[j] <= n) ? Lp[Lnext[j]] : (Int)L->nzmax;
            if (Lp[j] + len > end || Lp[j] + len > (Int)L->nzmax) { fits = FALSE; break; }
            memcpy(Li + Lp[j], Ls + Pi[s] + c, sizeof(Int) * len);
            Lnz[j] = len;
        }
    }
    if (!fits) {
        gb300_free_sparse(&S, Common);
        GB_ERROR(CHOLMOD_INVALID, "the column space of L does not hold the factor's pattern");
        return FALSE;
    }
    int64_t minor = n;
    gb_plan *P = gb_factor_device_only(S, beta ? beta[0] : 0.0, h->FS, dtype, &minor, Common);
    gb300_free_sparse(&S, Common);
    if (!P) return FALSE;
    gb_ctx *ctx = gb_ctx_get(Common, 0);
    const size_t e = dtype == CHOLMOD_SINGLE ? sizeof(float) : sizeof(double);
    const size_t out = e * (size_t)L->nzmax;
    int ok = gb_dev_grow(&h->d_out, &h->out_cap, out)
             && cudaMemcpyAsync(h->d_dst, Lp, sizeof(int64_t) * n, cudaMemcpyHostToDevice, ctx->stream) == cudaSuccess
             && cudaMemsetAsync(h->d_out, 0, out, ctx->stream) == cudaSuccess
             && gb_launch_simplicial_gather(n, h->d_src, h->d_dst, h->d_len, minor, !L->is_ll,
                                            P->d_Lx[dtype == CHOLMOD_SINGLE ? 1 : 0], h->d_out,
                                            dtype == CHOLMOD_SINGLE ? 4 : 0, ctx->stream) == 0
             && cudaMemcpyAsync(L->x, h->d_out, out, cudaMemcpyDeviceToHost, ctx->stream) == cudaSuccess
             && cudaStreamSynchronize(ctx->stream) == cudaSuccess;
    if (!ok) { GB_ERROR(CHOLMOD_GPU_PROBLEM, "CUDA error in the simplicial factorization"); return FALSE; }
    /* the reference's flop count: sum over columns of (count^2 - 1), plus
     * one square root per column for LL' */
    double fl = 0;
    for (Int j = 0; j < n; j++) fl += (double)h->h_len[j] * (double)h->h_len[j] - 1.0;
    if (L->is_ll) fl += (double)n;
    Common->rowfacfl = fl;
    if (minor < n) {
        L->minor = (size_t)minor;
        GB_ERROR(CHOLMOD_NOT_POSDEF, "not positive definite");
    }
    return TRUE;
}
