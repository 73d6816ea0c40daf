/* interpose_driver.c -- a program written against the reference CHOLMOD API
 * (cholmod.h of the reference), as an unmodified user of the library would
 * write it: cholmod_l_analyze -> cholmod_l_factorize -> cholmod_l_solve of a
 * 2D 5-point Laplacian with the supernodal method forced.
 *
 * Test infrastructure (tests/test_interpose.py): linked against the
 * reference library built from its sources (oracle/_ref/libcholmod_ref.so),
 * either alone, or with libcholmod_gb300.so ahead of it on the link line, or
 * with libcholmod_gb300.so in LD_PRELOAD.  In the last two cases the
 * reference's cholmod_l_factorize reaches cholmod_l_super_numeric through its
 * PLT (CHOLMOD/Cholesky/cholmod_factorize.c:260) and so calls the GPU
 * library's.  Prints one line of results. */
#include <stdio.h>
#include <stdlib.h>
#include "cholmod.h"

int main(int argc, char **argv)
{
    const int64_t m = argc > 1 ? atol(argv[1]) : 20, n = m * m;
    cholmod_common c;
    cholmod_l_start(&c);
    c.supernodal = CHOLMOD_SUPERNODAL;
    c.print = 0;
    c.error_handler = NULL;
    cholmod_sparse *A = cholmod_l_allocate_sparse(n, n, 3 * n, 1, 1, -1, CHOLMOD_REAL, &c);
    int64_t *Ap = A->p, *Ai = A->i, nz = 0;
    double *Ax = A->x;
    for (int64_t j = 0; j < n; j++) {            /* lower triangle, column j */
        Ap[j] = nz;
        Ai[nz] = j; Ax[nz++] = 4.0 + 1e-3;
        if ((j % m) + 1 < m) { Ai[nz] = j + 1; Ax[nz++] = -1.0; }
        if (j + m < n) { Ai[nz] = j + m; Ax[nz++] = -1.0; }
    }
    Ap[n] = nz;
    cholmod_dense *B = cholmod_l_ones(n, 1, CHOLMOD_REAL, &c);
    cholmod_factor *L = cholmod_l_analyze(A, &c);
    int ok = L ? cholmod_l_factorize(A, L, &c) : 0;
    int fstatus = c.status;
    double resid = -1;
    if (ok && fstatus == CHOLMOD_OK) {
        cholmod_dense *X = cholmod_l_solve(CHOLMOD_A, L, B, &c);
        if (X) {
            /* r = b - A x, |r|_inf / (|A|_inf |x|_inf + |b|_inf) */
            double one[2] = {1, 0}, mone[2] = {-1, 0};
            cholmod_dense *R = cholmod_l_copy_dense(B, &c);
            cholmod_l_sdmult(A, 0, mone, one, X, R, &c);
            resid = cholmod_l_norm_dense(R, 0, &c)
                    / (cholmod_l_norm_sparse(A, 0, &c) * cholmod_l_norm_dense(X, 0, &c) + 1.0);
            cholmod_l_free_dense(&R, &c);
            cholmod_l_free_dense(&X, &c);
        }
    }
    printf("factorize_ok %d status %d is_super %d minor %ld n %ld resid %.3e\n", ok, fstatus,
           L ? L->is_super : -1, L ? (long)L->minor : -1L, (long)n, resid);
    cholmod_l_free_factor(&L, &c);
    cholmod_l_free_dense(&B, &c);
    cholmod_l_free_sparse(&A, &c);
    cholmod_l_finish(&c);
    return 0;
}
