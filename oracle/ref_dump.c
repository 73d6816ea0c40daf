// ref_dump: drive the reference CHOLMOD (built by oracle/build_ref.py) on a
// matrix stored as raw binary files and dump its analysis, factor and solve.
//
// Test infrastructure only.  It produces the golden fixtures that pin the C
// restatement in oracle/ and the GPU path; it is never part of the product.
//
// Calls, in the order of the reference's demo (CHOLMOD/Demo/cholmod_di_demo.c
// :292-415): cholmod_l_analyze[_p] -> cholmod_l_factorize -> cholmod_l_solve,
// with Common->supernodal = CHOLMOD_SUPERNODAL and one ordering method.
//
// usage: ref_dump DIR ORDERING DTYPE [TRIALS]
//   DIR      holds meta.txt ("n nnz nrhs"), Ap.bin (int64 n+1), Ai.bin (int64),
//            Ax.bin (double), B.bin (double n*nrhs, optional), and for
//            ORDERING=given, UserPerm.bin (int64 n).  A is the lower triangle
//            (stype -1), sorted columns.
//   ORDERING amd | metis | given | natural
//   DTYPE    d | s  (double or single factorization of the same values)
//   TRIALS   number of timed factorizations (median reported), default 1
// outputs in DIR: out_meta.txt, Perm.bin, ColCount.bin, Super.bin, Pi.bin,
//   Px.bin, Ls.bin (int64), Lx.bin (double, widened when DTYPE=s), X.bin.
// REF_COMPLEX=1: A is complex (Hermitian, lower), its imaginary parts in
//   Az.bin and B's in Bz.bin (double); L->x and X are written as (re, im)
//   pairs of doubles in Lx.bin and X.bin.

#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include "cholmod.h"

static void *read_file(const char *dir, const char *name, size_t *bytes)
{
    char path[4096];
    snprintf(path, sizeof path, "%s/%s", dir, name);
    FILE *f = fopen(path, "rb");
    if (!f) return NULL;
    fseek(f, 0, SEEK_END);
    long sz = ftell(f);
    fseek(f, 0, SEEK_SET);
    void *buf = malloc(sz > 0 ? sz : 1);
    if (fread(buf, 1, sz, f) != (size_t)sz) { fclose(f); free(buf); return NULL; }
    fclose(f);
    if (bytes) *bytes = sz;
    return buf;
}

static void write_file(const char *dir, const char *name, const void *p, size_t bytes)
{
    char path[4096];
    snprintf(path, sizeof path, "%s/%s", dir, name);
    FILE *f = fopen(path, "wb");
    if (!f) { perror(path); exit(2); }
    if (bytes) fwrite(p, 1, bytes, f);
    fclose(f);
}

static int cmp_double(const void *a, const void *b)
{
    double x = *(const double *)a, y = *(const double *)b;
    return (x > y) - (x < y);
}

int main(int argc, char **argv)
{
    if (argc < 4) {
        fprintf(stderr, "usage: ref_dump DIR amd|metis|given|natural d|s [TRIALS]\n");
        return 2;
    }
    const char *dir = argv[1];
    const char *ord = argv[2];
    int single = (argv[3][0] == 's');
    int trials = argc > 4 ? atoi(argv[4]) : 1;
    if (trials < 1) trials = 1;

    char path[4096];
    snprintf(path, sizeof path, "%s/meta.txt", dir);
    FILE *mf = fopen(path, "r");
    if (!mf) { perror(path); return 2; }
    long n, nnz, nrhs = 0, sncol = 0;
    if (fscanf(mf, "%ld %ld %ld %ld", &n, &nnz, &nrhs, &sncol) < 2) { fclose(mf); return 2; }
    fclose(mf);

    int64_t *Ap = read_file(dir, "Ap.bin", NULL);
    int64_t *Ai = read_file(dir, "Ai.bin", NULL);
    double *Ax = read_file(dir, "Ax.bin", NULL);
    double *Bx = nrhs > 0 ? read_file(dir, "B.bin", NULL) : NULL;
    int64_t *UserPerm = read_file(dir, "UserPerm.bin", NULL);
    if (!Ap || !Ai || !Ax) { fprintf(stderr, "missing matrix files\n"); return 2; }
    const char *cx_env = getenv("REF_COMPLEX");
    const int cx = cx_env && cx_env[0] == '1';
    double *Az = cx ? read_file(dir, "Az.bin", NULL) : NULL;
    double *Bz = cx && nrhs > 0 ? read_file(dir, "Bz.bin", NULL) : NULL;
    if (cx && (!Az || (nrhs > 0 && !Bz))) { fprintf(stderr, "missing imaginary parts\n"); return 2; }
    const int xt = cx ? CHOLMOD_COMPLEX : CHOLMOD_REAL, ne = cx ? 2 : 1;

    cholmod_common c;
    cholmod_l_start(&c);
    c.supernodal = CHOLMOD_SUPERNODAL;
    /* REF_SIMPLICIAL=ll|ldl: the simplicial factorization instead (final_ll
     * as given); L->p, L->i, L->x, L->nz are dumped */
    const char *simp = getenv("REF_SIMPLICIAL");
    if (simp && (!strcmp(simp, "ll") || !strcmp(simp, "ldl"))) {
        c.supernodal = CHOLMOD_SIMPLICIAL;
        c.final_ll = !strcmp(simp, "ll");
    }
    c.nmethods = 1;
    c.postorder = 1;
    if (!strcmp(ord, "amd")) c.method[0].ordering = CHOLMOD_AMD;
    else if (!strcmp(ord, "metis")) c.method[0].ordering = CHOLMOD_METIS;
    else if (!strcmp(ord, "given")) c.method[0].ordering = CHOLMOD_GIVEN;
    else c.method[0].ordering = CHOLMOD_NATURAL;

    int dt = single ? CHOLMOD_SINGLE : CHOLMOD_DOUBLE;
    cholmod_sparse *A = cholmod_l_allocate_sparse(n, n, nnz, 1, 1, -1, xt + dt, &c);
    memcpy(A->p, Ap, (n + 1) * sizeof(int64_t));
    memcpy(A->i, Ai, nnz * sizeof(int64_t));
    for (long p = 0; p < nnz; p++) {
        for (int k = 0; k < ne; k++) {
            double v = k ? Az[p] : Ax[p];
            if (single) ((float *)A->x)[ne * p + k] = (float)v;
            else ((double *)A->x)[ne * p + k] = v;
        }
    }

    double t0 = SuiteSparse_time();
    cholmod_factor *L = (!strcmp(ord, "given") && UserPerm)
        ? cholmod_l_analyze_p(A, UserPerm, NULL, 0, &c)
        : cholmod_l_analyze(A, &c);
    double t_analyze = SuiteSparse_time() - t0;
    if (!L) { fprintf(stderr, "analyze failed %d\n", c.status); return 3; }

    double *tf = malloc(trials * sizeof(double));
    int ok = 1;
    for (int t = 0; t < trials; t++) {
        t0 = SuiteSparse_time();
        ok = cholmod_l_factorize(A, L, &c);
        tf[t] = SuiteSparse_time() - t0;
    }
    qsort(tf, trials, sizeof(double), cmp_double);
    double t_factor = tf[trials / 2];
    int fstatus = c.status;

    double t_solve = 0, resid = -1;
    if (Bx && nrhs > 0 && L->is_super && L->minor == (size_t)n) {
        cholmod_dense *B = cholmod_l_allocate_dense(n, nrhs, n, xt + dt, &c);
        for (long p = 0; p < n * nrhs; p++) {
            for (int k = 0; k < ne; k++) {
                double v = k ? Bz[p] : Bx[p];
                if (single) ((float *)B->x)[ne * p + k] = (float)v;
                else ((double *)B->x)[ne * p + k] = v;
            }
        }
        t0 = SuiteSparse_time();
        cholmod_dense *X = cholmod_l_solve(CHOLMOD_A, L, B, &c);
        t_solve = SuiteSparse_time() - t0;
        double *xo = malloc(ne * n * nrhs * sizeof(double));
        for (long p = 0; p < ne * n * nrhs; p++)
            xo[p] = single ? ((float *)X->x)[p] : ((double *)X->x)[p];
        write_file(dir, "X.bin", xo, ne * n * nrhs * sizeof(double));
        // backward error |b-Ax|/(|A||x|+|b|), inf-norms, column 0 (demo :614-617)
        double one[2] = {1, 0}, m1[2] = {-1, 0};
        cholmod_dense *R = cholmod_l_copy_dense(B, &c);
        cholmod_l_sdmult(A, 0, m1, one, X, R, &c);
        double rn = cholmod_l_norm_dense(R, 0, &c);
        double an = cholmod_l_norm_sparse(A, 0, &c);
        double xn = cholmod_l_norm_dense(X, 0, &c);
        double bn = cholmod_l_norm_dense(B, 0, &c);
        resid = rn / (an * xn + bn);
        free(xo);
        cholmod_l_free_dense(&R, &c);
        cholmod_l_free_dense(&X, &c);
        cholmod_l_free_dense(&B, &c);
    }

    /* sparse right-hand side (SBp/SBi/SBx.bin, sncol columns, double):
     * cholmod_l_spsolve for every sys, X written as SX<sys>{p,i,x}.bin */
    long spnz[9] = {0};
    int64_t *SBp = sncol > 0 ? read_file(dir, "SBp.bin", NULL) : NULL;
    int64_t *SBi = SBp ? read_file(dir, "SBi.bin", NULL) : NULL;
    double *SBx = SBp ? read_file(dir, "SBx.bin", NULL) : NULL;
    if (SBp && !single && !cx && L->is_super && L->minor == (size_t)n) {
        long bnz = SBp[sncol];
        cholmod_sparse *SB = cholmod_l_allocate_sparse(n, sncol, bnz > 0 ? bnz : 1, 0, 1, 0,
                                                       CHOLMOD_REAL + CHOLMOD_DOUBLE, &c);
        memcpy(SB->p, SBp, (sncol + 1) * sizeof(int64_t));
        if (bnz > 0) {
            memcpy(SB->i, SBi, bnz * sizeof(int64_t));
            memcpy(SB->x, SBx, bnz * sizeof(double));
        }
        for (int sys = 0; sys <= 8; sys++) {
            cholmod_sparse *X = cholmod_l_spsolve(sys, L, SB, &c);
            if (!X) { spnz[sys] = -1; continue; }
            int64_t *xp = X->p;
            char name[64];
            snprintf(name, sizeof name, "SX%dp.bin", sys);
            write_file(dir, name, xp, (sncol + 1) * sizeof(int64_t));
            snprintf(name, sizeof name, "SX%di.bin", sys);
            write_file(dir, name, X->i, xp[sncol] * sizeof(int64_t));
            snprintf(name, sizeof name, "SX%dx.bin", sys);
            write_file(dir, name, X->x, xp[sncol] * sizeof(double));
            spnz[sys] = (long)X->nzmax;
            cholmod_l_free_sparse(&X, &c);
        }
        cholmod_l_free_sparse(&SB, &c);
    }
    free(SBp); free(SBi); free(SBx);

    if (!L->is_super && L->xtype != CHOLMOD_PATTERN) {
        int64_t *lp = L->p;
        write_file(dir, "Lp.bin", L->p, (n + 1) * sizeof(int64_t));
        write_file(dir, "Lnz.bin", L->nz, n * sizeof(int64_t));
        write_file(dir, "Li.bin", L->i, L->nzmax * sizeof(int64_t));
        double *lx = malloc(L->nzmax * sizeof(double));
        for (size_t p = 0; p < L->nzmax; p++)
            lx[p] = single ? ((float *)L->x)[p] : ((double *)L->x)[p];
        write_file(dir, "SLx.bin", lx, L->nzmax * sizeof(double));
        free(lx);
        (void)lp;
    }
    write_file(dir, "Perm.bin", L->Perm, n * sizeof(int64_t));
    write_file(dir, "ColCount.bin", L->ColCount, n * sizeof(int64_t));
    if (L->is_super) {
        write_file(dir, "Super.bin", L->super, (L->nsuper + 1) * sizeof(int64_t));
        write_file(dir, "Pi.bin", L->pi, (L->nsuper + 1) * sizeof(int64_t));
        write_file(dir, "Px.bin", L->px, (L->nsuper + 1) * sizeof(int64_t));
        write_file(dir, "Ls.bin", L->s, L->ssize * sizeof(int64_t));
        if (L->x) {
            const size_t nx = (L->xtype == CHOLMOD_COMPLEX ? 2 : 1) * L->xsize;
            double *lx = malloc(nx * sizeof(double));
            for (size_t p = 0; p < nx; p++)
                lx[p] = single ? ((float *)L->x)[p] : ((double *)L->x)[p];
            write_file(dir, "Lx.bin", lx, nx * sizeof(double));
            free(lx);
        }
    }
    /* the reference's rough reciprocal condition number of the factor
     * (cholmod_rcond: (min L(j,j) / max L(j,j))^2 for LL') */
    double rcond = ok ? cholmod_l_rcond(L, &c) : -1.0;
    snprintf(path, sizeof path, "%s/out_meta.txt", dir);
    FILE *of = fopen(path, "w");
    fprintf(of, "nzmax %zu\nis_ll %d\n", L->nzmax, L->is_ll);
    fprintf(of, "is_super %d\nnsuper %zu\nssize %zu\nxsize %zu\nmaxcsize %zu\n"
                "maxesize %zu\nfl %.17g\nlnz %.17g\nanz %.17g\nminor %zu\n"
                "status %d\nfactor_ok %d\nfactor_status %d\nordering %d\n"
                "t_analyze %.6f\nt_factor %.6f\nt_solve %.6f\nresid %.6e\n"
                "nthreads %d\nrcond %.17g\n"
                "spnzmax %ld,%ld,%ld,%ld,%ld,%ld,%ld,%ld,%ld\n",
            L->is_super, L->nsuper, L->ssize, L->xsize, L->maxcsize, L->maxesize,
            c.fl, c.lnz, c.anz, L->minor, c.status, ok, fstatus, L->ordering,
            t_analyze, t_factor, t_solve, resid, c.nthreads_max, rcond,
            spnz[0], spnz[1], spnz[2], spnz[3], spnz[4], spnz[5], spnz[6], spnz[7], spnz[8]);
    fclose(of);

    cholmod_l_free_factor(&L, &c);
    cholmod_l_free_sparse(&A, &c);
    cholmod_l_finish(&c);
    return 0;
}
