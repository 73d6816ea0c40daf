/* oracle_body.h -- precision-generic body of oracle.c (included twice with
 * REAL = double / float).  Test infrastructure only. */

/* ---- dense kernels: external BLAS when installed, else plain loops ---- */

/* C(0:n,0:n) lower = A A', A n-by-k (lda), C ldc */
static void SUF(syrk_ln)(Int n, Int k, const REAL *A, Int lda, REAL *C, Int ldc)
{
    if (SYRK) {
        blasint N = (blasint)n, K = (blasint)k, LDA = (blasint)lda, LDC = (blasint)ldc;
        REAL one = 1, zero = 0;
        SYRK("L", "N", &N, &K, &one, A, &LDA, &zero, C, &LDC);
        return;
    }
    for (Int j = 0; j < n; j++) {
        for (Int i = j; i < n; i++) C[i + j * ldc] = 0;
        for (Int p = 0; p < k; p++) {
            REAL b = A[j + p * lda];
            if (b == 0) continue;
            for (Int i = j; i < n; i++) C[i + j * ldc] += A[i + p * lda] * b;
        }
    }
}

/* C(0:m,0:n) = A B', A m-by-k (lda), B n-by-k (ldb) */
static void SUF(gemm_nt)(Int m, Int n, Int k, const REAL *A, Int lda, const REAL *B, Int ldb,
                         REAL *C, Int ldc)
{
    if (GEMM) {
        blasint M = (blasint)m, N = (blasint)n, K = (blasint)k;
        blasint LDA = (blasint)lda, LDB = (blasint)ldb, LDC = (blasint)ldc;
        REAL one = 1, zero = 0;
        GEMM("N", "C", &M, &N, &K, &one, A, &LDA, B, &LDB, &zero, C, &LDC);
        return;
    }
    for (Int j = 0; j < n; j++) {
        for (Int i = 0; i < m; i++) C[i + j * ldc] = 0;
        for (Int p = 0; p < k; p++) {
            REAL b = B[j + p * ldb];
            if (b == 0) continue;
            for (Int i = 0; i < m; i++) C[i + j * ldc] += A[i + p * lda] * b;
        }
    }
}

/* LL' of A(0:n,0:n) lower in place; returns LAPACK info (0 or 1-based column) */
static Int SUF(potrf_l)(Int n, REAL *A, Int lda)
{
    if (POTRF) {
        blasint N = (blasint)n, LDA = (blasint)lda, info = 0;
        if (n == 0) return 0;
        POTRF("L", &N, A, &LDA, &info);
        return info;
    }
    for (Int j = 0; j < n; j++) {
        REAL d = A[j + j * lda];
        for (Int p = 0; p < j; p++) d -= A[j + p * lda] * A[j + p * lda];
        if (!(d > 0)) return j + 1;
        d = SQRT(d);
        A[j + j * lda] = d;
        for (Int i = j + 1; i < n; i++) {
            REAL v = A[i + j * lda];
            for (Int p = 0; p < j; p++) v -= A[i + p * lda] * A[j + p * lda];
            A[i + j * lda] = v / d;
        }
    }
    return 0;
}

/* B(0:m,0:n) = B / L' with L n-by-n lower (right side, transposed) */
static void SUF(trsm_rlt)(Int m, Int n, const REAL *Lm, Int ldl, REAL *B, Int ldb)
{
    if (TRSM) {
        blasint M = (blasint)m, N = (blasint)n, LDL = (blasint)ldl, LDB = (blasint)ldb;
        REAL one = 1;
        if (m == 0 || n == 0) return;
        TRSM("R", "L", "C", "N", &M, &N, &one, Lm, &LDL, B, &LDB);
        return;
    }
    for (Int j = 0; j < n; j++) {
        for (Int p = 0; p < j; p++) {
            REAL l = Lm[j + p * ldl];
            if (l == 0) continue;
            for (Int i = 0; i < m; i++) B[i + j * ldb] -= B[i + p * ldb] * l;
        }
        REAL d = Lm[j + j * ldl];
        for (Int i = 0; i < m; i++) B[i + j * ldb] /= d;
    }
}

/* ---- left-looking supernodal numeric factorization ---- */

static int SUF(numeric)(Int n, Int nsuper, const Int *Super, const Int *Pi, const Int *Px,
                        const Int *Ls, const Int *Sp, const Int *Si, const void *Sxv,
                        double beta, int quick_return, void *Lxv, Int *minor)
{
    const REAL *Sx = Sxv;
    REAL *Lx = Lxv;
    Int maxc = 1;
    /* C workspace: largest ndrow2*ndrow1 over all (d, s) pairs */
    for (Int d = 0; d < nsuper; d++) {
        Int nsc = Super[d + 1] - Super[d];
        Int nsr = Pi[d + 1] - Pi[d];
        Int m = nsr - nsc;
        if (m * m > maxc) maxc = m * m;
    }
    Int *Map = malloc(sizeof(Int) * (n + 1));
    Int *SuperMap = malloc(sizeof(Int) * (n + 1));
    Int *RelMap = malloc(sizeof(Int) * (n + 1));
    Int *Head = malloc(sizeof(Int) * (nsuper + 1));
    Int *Next = malloc(sizeof(Int) * (nsuper + 1));
    Int *Lpos = malloc(sizeof(Int) * (nsuper + 1));
    Int *Next_save = malloc(sizeof(Int) * (nsuper + 1));
    Int *Lpos_save = malloc(sizeof(Int) * (nsuper + 1));
    REAL *C = malloc(sizeof(REAL) * maxc);
    if (!Map || !SuperMap || !RelMap || !Head || !Next || !Lpos || !Next_save || !Lpos_save || !C) {
        free(Map); free(SuperMap); free(RelMap); free(Head); free(Next); free(Lpos);
        free(Next_save); free(Lpos_save); free(C);
        return -2;
    }
    for (Int s = 0; s < nsuper; s++) {
        Head[s] = -1;
        for (Int k = Super[s]; k < Super[s + 1]; k++) SuperMap[k] = s;
    }
    for (Int i = 0; i < n; i++) Map[i] = -1;
    Int xsize = Px[nsuper];
    int repeat_supernode = 0;
    Int nscol_new = 0;
    int status = 0;
    *minor = n;

    for (Int s = 0; s < nsuper; s++) {
        Int k1 = Super[s], k2 = Super[s + 1], nscol = k2 - k1;
        Int psi = Pi[s], psx = Px[s], psend = Pi[s + 1], nsrow = psend - psi;
        for (Int p = psx; p < psx + nsrow * nscol; p++) Lx[p] = 0;
        for (Int k = 0; k < nsrow; k++) Map[Ls[psi + k]] = k;
        for (Int k = k1; k < k2; k++) {
            for (Int p = Sp[k]; p < Sp[k + 1]; p++) {
                Int i = Si[p];
                if (i >= k) {
                    Int imap = Map[i];
                    if (imap >= 0 && imap < nsrow)
                        Lx[imap + psx + (k - k1) * nsrow] = Sx[p];
                }
            }
        }
        if (beta != 0.0) {
            Int pk = psx;
            for (Int k = k1; k < k2; k++) { Lx[pk] += (REAL)beta; pk += nsrow + 1; }
        }
        if (!repeat_supernode) {
            for (Int d = Head[s]; d != -1; d = Next[d]) { Lpos_save[d] = Lpos[d]; Next_save[d] = Next[d]; }
        } else {
            for (Int d = Head[s]; d != -1; d = Next[d]) { Lpos[d] = Lpos_save[d]; Next[d] = Next_save[d]; }
        }
        Int dnext = Head[s];
        while (dnext != -1) {
            Int d = dnext;
            Int kd1 = Super[d], kd2 = Super[d + 1], ndcol = kd2 - kd1;
            Int pdi = Pi[d], pdx = Px[d], pdend = Pi[d + 1], ndrow = pdend - pdi;
            Int p = Lpos[d];
            Int pdi1 = pdi + p, pdx1 = pdx + p, pdi2;
            for (pdi2 = pdi1; pdi2 < pdend && Ls[pdi2] < k2; pdi2++) ;
            Int ndrow1 = pdi2 - pdi1, ndrow2 = pdend - pdi1, ndrow3 = ndrow2 - ndrow1;
            SUF(syrk_ln)(ndrow1, ndcol, Lx + pdx1, ndrow, C, ndrow2);
            if (ndrow3 > 0)
                SUF(gemm_nt)(ndrow3, ndrow1, ndcol, Lx + pdx1 + ndrow1, ndrow, Lx + pdx1,
                             ndrow, C + ndrow1, ndrow2);
            for (Int i = 0; i < ndrow2; i++) RelMap[i] = Map[Ls[pdi1 + i]];
            for (Int j = 0; j < ndrow1; j++) {
                Int px = psx + RelMap[j] * nsrow;
                for (Int i = j; i < ndrow2; i++) Lx[px + RelMap[i]] -= C[i + ndrow2 * j];
            }
            dnext = Next[d];
            if (!repeat_supernode) {
                Lpos[d] = pdi2 - pdi;
                if (Lpos[d] < ndrow) {
                    Int dancestor = SuperMap[Ls[pdi2]];
                    Next[d] = Head[dancestor];
                    Head[dancestor] = d;
                }
            }
        }
        Int nscol2 = repeat_supernode ? nscol_new : nscol;
        Int info = SUF(potrf_l)(nscol2, Lx + psx, nsrow);
        if (repeat_supernode) {
            info = 0;
            for (Int q = psx + nsrow * nscol_new; q < psx + nsrow * nscol; q++) Lx[q] = 0;
        }
        if (info != 0) {
            status = 1;                               /* CHOLMOD_NOT_POSDEF */
            *minor = k1 + info - 1;
            for (Int ss = s + 1; ss < nsuper; ss++) Head[ss] = -1;
            for (Int q = psx; q < xsize; q++) Lx[q] = 0;
            if (info == 1 || quick_return) { Head[s] = -1; break; }
            repeat_supernode = 1;
            s--;
            nscol_new = info - 1;
            continue;
        }
        Int nsrow2 = nsrow - nscol2;
        if (nsrow2 > 0) {
            SUF(trsm_rlt)(nsrow2, nscol2, Lx + psx, nsrow, Lx + psx + nscol2, nsrow);
            if (!repeat_supernode) {
                Lpos[s] = nscol;
                Int sparent = SuperMap[Ls[psi + nscol]];
                Next[s] = Head[sparent];
                Head[sparent] = s;
            }
        }
        Head[s] = -1;
        if (repeat_supernode) break;
    }
    free(Map); free(SuperMap); free(RelMap); free(Head); free(Next); free(Lpos);
    free(Next_save); free(Lpos_save); free(C);
    return status;
}

/* ---- supernodal sweeps (nrhs columns, X leading dimension ldx) ---- */

static int SUF(sweep)(int lower, Int n, Int nsuper, const Int *Super, const Int *Pi,
                      const Int *Px, const Int *Ls, const void *Lxv, Int nrhs, void *Xv,
                      Int ldx)
{
    const REAL *Lx = Lxv;
    REAL *X = Xv;
    (void)n;
    Int maxe = 1;
    for (Int s = 0; s < nsuper; s++) {
        Int e = (Pi[s + 1] - Pi[s]) - (Super[s + 1] - Super[s]);
        if (e > maxe) maxe = e;
    }
    REAL *E = malloc(sizeof(REAL) * maxe * (nrhs > 0 ? nrhs : 1));
    if (!E) return -2;
    for (Int t = 0; t < nsuper; t++) {
        Int s = lower ? t : nsuper - 1 - t;
        Int k1 = Super[s], nscol = Super[s + 1] - k1;
        Int psi = Pi[s], psx = Px[s], nsrow = Pi[s + 1] - psi, nsrow2 = nsrow - nscol;
        Int ps2 = psi + nscol;
        const REAL *L1 = Lx + psx, *L2 = Lx + psx + nscol;
        for (Int r = 0; r < nrhs; r++) {
            REAL *x1 = X + k1 + r * ldx, *xr = X + r * ldx, *e = E + r * nsrow2;
            for (Int ii = 0; ii < nsrow2; ii++) e[ii] = xr[Ls[ps2 + ii]];
            if (lower) {
                /* x1 = L1 \ x1 ; e -= L2 x1 ; scatter e */
                for (Int j = 0; j < nscol; j++) {
                    REAL v = x1[j] / L1[j + j * nsrow];
                    x1[j] = v;
                    for (Int i = j + 1; i < nscol; i++) x1[i] -= L1[i + j * nsrow] * v;
                    for (Int i = 0; i < nsrow2; i++) e[i] -= L2[i + j * nsrow] * v;
                }
                for (Int ii = 0; ii < nsrow2; ii++) xr[Ls[ps2 + ii]] = e[ii];
            } else {
                /* x1 -= L2' e ; x1 = L1' \ x1 */
                for (Int j = 0; j < nscol; j++) {
                    REAL acc = 0;
                    for (Int i = 0; i < nsrow2; i++) acc += L2[i + j * nsrow] * e[i];
                    x1[j] -= acc;
                }
                for (Int j = nscol - 1; j >= 0; j--) {
                    REAL v = x1[j];
                    for (Int i = j + 1; i < nscol; i++) v -= L1[i + j * nsrow] * x1[i];
                    x1[j] = v / L1[j + j * nsrow];
                }
            }
        }
    }
    free(E);
    return 0;
}
