/* oracle.c -- CPU restatement of CHOLMOD's supernodal numeric factorization
 * and supernodal triangular solves.
 *
 * TEST INFRASTRUCTURE: this is the checker the GPU library is compared with
 * (tests/, __graft_entry__.smoke, and the CPU-baseline leg of bench.py).  The
 * product never links, loads or calls it.
 *
 * Algorithm: the left-looking supernodal LL' of
 * CHOLMOD/Supernodal/t_cholmod_super_numeric_worker.c, step for step:
 *   :358-399   zero supernode s and build Map (row -> position in s)
 *   :419-520   copy column k of S (rows >= k, through Map) and add beta
 *   :537-551   save Lpos/Next of the pending descendants
 *   :686-703   rows of descendant d that touch s: pdi1..pdi2 (ndrow1), ndrow2
 *   :768-883   C1 = L1*L1' (syrk, lower), C2 = L2*L1' (gemm)
 *   :896-930   RelativeMap and Lx[psx + RM[j]*nsrow + RM[i]] -= C[i + ndrow2*j]
 *   :950-967   move d to the list of its next ancestor
 *   :1004-1058 potrf of the diagonal block
 *   :1084-1146 not positive definite: L->minor, zero the rest, repeat s
 *   :1152-1218 trsm L2 = S2 / L1'
 *   :1222-1235 link s into its parent's list
 * and the sweeps of CHOLMOD/Supernodal/t_cholmod_super_solve_worker.c
 * (forward :63-301, backward :358-578).
 *
 * The dense kernels are the external BLAS/LAPACK routines the reference
 * calls (dsyrk/dgemm/dtrsm/dpotrf and single-precision twins), reached
 * through function pointers that the caller may set to a Fortran-ABI BLAS
 * (the Python side passes the OpenBLAS bundled with scipy); without them,
 * plain loops written here are used (same mathematics, slower).
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

typedef int64_t Int;
typedef int blasint;

typedef void (*gemm_d)(const char *, const char *, const blasint *, const blasint *,
                       const blasint *, const double *, const double *, const blasint *,
                       const double *, const blasint *, const double *, double *,
                       const blasint *);
typedef void (*syrk_d)(const char *, const char *, const blasint *, const blasint *,
                       const double *, const double *, const blasint *, const double *,
                       double *, const blasint *);
typedef void (*trsm_d)(const char *, const char *, const char *, const char *,
                       const blasint *, const blasint *, const double *, const double *,
                       const blasint *, double *, const blasint *);
typedef void (*potrf_d)(const char *, const blasint *, double *, const blasint *, blasint *);
typedef void (*gemm_s)(const char *, const char *, const blasint *, const blasint *,
                       const blasint *, const float *, const float *, const blasint *,
                       const float *, const blasint *, const float *, float *,
                       const blasint *);
typedef void (*syrk_s)(const char *, const char *, const blasint *, const blasint *,
                       const float *, const float *, const blasint *, const float *,
                       float *, const blasint *);
typedef void (*trsm_s)(const char *, const char *, const char *, const char *,
                       const blasint *, const blasint *, const float *, const float *,
                       const blasint *, float *, const blasint *);
typedef void (*potrf_s)(const char *, const blasint *, float *, const blasint *, blasint *);

static gemm_d B_dgemm;
static syrk_d B_dsyrk;
static trsm_d B_dtrsm;
static potrf_d B_dpotrf;
static gemm_s B_sgemm;
static syrk_s B_ssyrk;
static trsm_s B_strsm;
static potrf_s B_spotrf;

/* Install (or with NULLs, remove) the external BLAS/LAPACK. */
void oracle_set_blas(void *dgemm, void *dsyrk, void *dtrsm, void *dpotrf,
                     void *sgemm, void *ssyrk, void *strsm, void *spotrf)
{
    B_dgemm = (gemm_d)dgemm;
    B_dsyrk = (syrk_d)dsyrk;
    B_dtrsm = (trsm_d)dtrsm;
    B_dpotrf = (potrf_d)dpotrf;
    B_sgemm = (gemm_s)sgemm;
    B_ssyrk = (syrk_s)ssyrk;
    B_strsm = (trsm_s)strsm;
    B_spotrf = (potrf_s)spotrf;
}

int oracle_has_blas(void) { return B_dgemm && B_dsyrk && B_dtrsm && B_dpotrf; }

/* Both precisions share one body, instantiated twice below. */
#define REAL double
#define SUF(name) name##_d
#define GEMM B_dgemm
#define SYRK B_dsyrk
#define TRSM B_dtrsm
#define POTRF B_dpotrf
#define SQRT sqrt
#include "oracle_body.h"
#undef REAL
#undef SUF
#undef GEMM
#undef SYRK
#undef TRSM
#undef POTRF
#undef SQRT

#define REAL float
#define SUF(name) name##_s
#define GEMM B_sgemm
#define SYRK B_ssyrk
#define TRSM B_strsm
#define POTRF B_spotrf
#define SQRT sqrtf
#include "oracle_body.h"

/* dtype 0 = double, 4 = single (CHOLMOD's dtype codes). */
int oracle_super_numeric(int dtype, Int n, Int nsuper, const Int *Super, const Int *Pi,
                         const Int *Px, const Int *Ls, const Int *Sp, const Int *Si,
                         const void *Sx, double beta, int quick_return, void *Lx,
                         Int *minor)
{
    if (dtype == 4)
        return numeric_s(n, nsuper, Super, Pi, Px, Ls, Sp, Si, Sx, beta, quick_return, Lx, minor);
    return numeric_d(n, nsuper, Super, Pi, Px, Ls, Sp, Si, Sx, beta, quick_return, Lx, minor);
}

/* forward (lower = 1: X = L\X) or backward (lower = 0: X = L'\X) sweep */
int oracle_super_solve(int dtype, int lower, Int n, Int nsuper, const Int *Super,
                       const Int *Pi, const Int *Px, const Int *Ls, const void *Lx,
                       Int nrhs, void *X, Int ldx)
{
    if (dtype == 4) return sweep_s(lower, n, nsuper, Super, Pi, Px, Ls, Lx, nrhs, X, ldx);
    return sweep_d(lower, n, nsuper, Super, Pi, Px, Ls, Lx, nrhs, X, ldx);
}

/* Row pattern of a supernodal factor from its column partition.
 *
 * Given S = tril(P A P') (sorted lower CSC, n columns) and the supernode
 * partition Super [nsuper+1] that the reference's analysis chose, the rows
 * of supernode s are its own columns k1..k2-1 followed by every row i >= k2
 * that is nonzero in some column of s of S or in the pattern of a child
 * supernode (the supernodal form of the column-pattern recurrence
 * struct(L(:,j)) = struct(S(j:n,j)) U struct(L(:,c)) \ {c} over the etree
 * children c of j), in ascending order, as cholmod_super_symbolic stores
 * L->s (CHOLMOD/Supernodal/cholmod_super_symbolic.c:760-900 build the same
 * sets by row subtrees).  Children precede their parent in the postordered
 * numbering.  Output: Pi [nsuper+1], Px [nsuper+1] and *Ls_out (malloc'd,
 * *ssize entries; free with oracle_free).  Returns 0, or -1 (bad input or
 * out of memory).  Test infrastructure: lets the reference arm of the
 * benchmark and the CPU checks rebuild the reference's symbolic factor from
 * a fixture of Super alone, without the product library. */
static int cmp_int(const void *a, const void *b)
{
    Int x = *(const Int *)a, y = *(const Int *)b;
    return x < y ? -1 : x > y;
}

int oracle_super_pattern(Int n, const Int *Sp, const Int *Si, Int nsuper, const Int *Super,
                         Int *Pi, Int *Px, Int **Ls_out, Int *ssize)
{
    *Ls_out = NULL;
    *ssize = 0;
    if (n < 0 || nsuper < 0 || Super[0] != 0 || Super[nsuper] != n) return -1;
    Int *smap = malloc(sizeof(Int) * (n + 1));
    Int *mark = malloc(sizeof(Int) * (n + 1));
    Int *head = malloc(sizeof(Int) * (nsuper + 1));   /* children lists */
    Int *next = malloc(sizeof(Int) * (nsuper + 1));
    Int cap = 4 * (n + 16), len = 0;
    Int *Ls = malloc(sizeof(Int) * cap);
    int ok = smap && mark && head && next && Ls;
    for (Int s = 0; ok && s < nsuper; s++) {
        if (Super[s + 1] <= Super[s]) { ok = 0; break; }
        for (Int j = Super[s]; j < Super[s + 1]; j++) smap[j] = s;
        head[s] = -1;
    }
    for (Int i = 0; ok && i < n; i++) mark[i] = -1;
    Pi[0] = 0;
    Px[0] = 0;
    for (Int s = 0; ok && s < nsuper; s++) {
        const Int k1 = Super[s], k2 = Super[s + 1];
        const Int p0 = len;
        /* worst case: every row of the matrix */
        if (cap - len < n) {
            cap = 2 * cap + n;
            Int *t = realloc(Ls, sizeof(Int) * cap);
            if (!t) { ok = 0; break; }
            Ls = t;
        }
        for (Int k = k1; k < k2; k++) { Ls[len++] = k; mark[k] = s; }
        for (Int k = k1; k < k2; k++)
            for (Int p = Sp[k]; p < Sp[k + 1]; p++) {
                const Int i = Si[p];
                if (i < k || i >= n) { if (i < k) continue; ok = 0; break; }
                if (mark[i] != s) { mark[i] = s; Ls[len++] = i; }
            }
        for (Int c = head[s]; ok && c >= 0; c = next[c]) {
            const Int nscol_c = Super[c + 1] - Super[c];
            for (Int p = Pi[c] + nscol_c; p < Pi[c + 1]; p++) {
                const Int i = Ls[p];
                if (i >= k2 && mark[i] != s) { mark[i] = s; Ls[len++] = i; }
            }
        }
        if (!ok) break;
        qsort(Ls + p0 + (k2 - k1), len - p0 - (k2 - k1), sizeof(Int), cmp_int);
        Pi[s + 1] = len;
        Px[s + 1] = Px[s] + (k2 - k1) * (len - p0);
        /* parent: the supernode of the first row below the diagonal block */
        if (len - p0 > k2 - k1) {
            const Int par = smap[Ls[p0 + (k2 - k1)]];
            next[s] = head[par];
            head[par] = s;
        }
    }
    free(smap); free(mark); free(head); free(next);
    if (!ok) { free(Ls); return -1; }
    *Ls_out = Ls;
    *ssize = len;
    return 0;
}

void oracle_free(void *p) { free(p); }
