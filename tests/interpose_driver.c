/* interpose_driver.c -- a program written against the reference CHOLMOD API
 * (cholmod.h of the reference), as an unmodified user of the library would
 * write it: analyze -> factorize -> solve of a 2D 5-point Laplacian with
 * the supernodal method forced, through the int64 API (cholmod_l_*) or, with
 * a second argument "32", the int32 API (cholmod_*); a third argument
 * "simplicial" selects the simplicial method (cholmod_l_rowfac).
 *
 * Test infrastructure (tests/test_interpose.py): linked against the
 * reference library built from its sources (oracle/_ref/libcholmod_ref.so),
 * either alone, or with libcholmod_gb300.so ahead of it on the link line, or
 * with libcholmod_gb300.so in LD_PRELOAD.  In the last two cases the
 * reference's factorize reaches cholmod_l_super_numeric (or
 * cholmod_super_numeric) through its PLT
 * (CHOLMOD/Cholesky/cholmod_factorize.c:260) and so calls the GPU
 * library's.  Prints one line of results. */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include "cholmod.h"

static int simplicial;     /* third argument "simplicial": the simplicial method */

/* the same program for both index widths: ITYPE_T, P (function prefix) */
#define DRIVER(NAME, ITYPE_T, P)                                                          \
static void NAME(int64_t m)                                                              \
{                                                                                         \
    const int64_t n = m * m;                                                             \
    cholmod_common c;                                                                     \
    P##start(&c);                                                                         \
    c.supernodal = simplicial ? CHOLMOD_SIMPLICIAL : CHOLMOD_SUPERNODAL;                   \
    c.print = 0;                                                                          \
    c.error_handler = NULL;                                                               \
    cholmod_sparse *A = P##allocate_sparse(n, n, 3 * n, 1, 1, -1, CHOLMOD_REAL, &c);      \
    ITYPE_T *Ap = A->p, *Ai = A->i, nz = 0;                                               \
    double *Ax = A->x;                                                                    \
    for (int64_t j = 0; j < n; j++) {           /* lower triangle, column j */            \
        Ap[j] = nz;                                                                       \
        Ai[nz] = (ITYPE_T)j; Ax[nz++] = 4.0 + 1e-3;                                       \
        if ((j % m) + 1 < m) { Ai[nz] = (ITYPE_T)(j + 1); Ax[nz++] = -1.0; }              \
        if (j + m < n) { Ai[nz] = (ITYPE_T)(j + m); Ax[nz++] = -1.0; }                    \
    }                                                                                     \
    Ap[n] = nz;                                                                           \
    cholmod_dense *B = P##ones(n, 1, CHOLMOD_REAL, &c);                                   \
    cholmod_factor *L = P##analyze(A, &c);                                                \
    int ok = L ? P##factorize(A, L, &c) : 0;                                              \
    int fstatus = c.status;                                                               \
    double resid = -1;                                                                    \
    if (ok && fstatus == CHOLMOD_OK) {                                                    \
        cholmod_dense *X = P##solve(CHOLMOD_A, L, B, &c);                                 \
        if (X) {                                                                          \
            double one[2] = {1, 0}, mone[2] = {-1, 0};                                    \
            cholmod_dense *R = P##copy_dense(B, &c);                                      \
            P##sdmult(A, 0, mone, one, X, R, &c);                                         \
            resid = P##norm_dense(R, 0, &c)                                               \
                    / (P##norm_sparse(A, 0, &c) * P##norm_dense(X, 0, &c) + 1.0);         \
            P##free_dense(&R, &c);                                                        \
            P##free_dense(&X, &c);                                                        \
        }                                                                                 \
    }                                                                                     \
    printf("factorize_ok %d status %d is_super %d minor %ld n %ld resid %.3e\n", ok,       \
           fstatus, L ? L->is_super : -1, L ? (long)L->minor : -1L, (long)n, resid);      \
    P##free_factor(&L, &c);                                                               \
    P##free_dense(&B, &c);                                                                \
    P##free_sparse(&A, &c);                                                               \
    P##finish(&c);                                                                        \
}

DRIVER(run64, int64_t, cholmod_l_)
DRIVER(run32, int32_t, cholmod_)

int main(int argc, char **argv)
{
    const int64_t m = argc > 1 ? atol(argv[1]) : 20;
    simplicial = argc > 3 && strcmp(argv[3], "simplicial") == 0;
    if (argc > 2 && strcmp(argv[2], "32") == 0) run32(m);
    else run64(m);
    return 0;
}
