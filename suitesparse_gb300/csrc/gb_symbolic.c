/* gb_symbolic.c -- supernodal symbolic analysis for a given permutation.
 *
 * Host-side analysis that feeds the GPU numeric factorization in programs
 * that do not link the reference CHOLMOD.  Given A (symmetric, lower stored)
 * and the final fill-reducing permutation Perm (the one cholmod_analyze
 * leaves in L->Perm, postorder already folded in), it produces the
 * supernodal symbolic factor cholmod_analyze would produce for that ordering:
 *
 *   - the elimination tree and column counts of L for PAP' (both are unique
 *     functions of the pattern; computed here with Liu's path-compressed
 *     etree and row-subtree traversal, so any correct method matches
 *     CHOLMOD/Cholesky/cholmod_etree.c and cholmod_rowcolcounts.c);
 *   - Common->fl = sum ColCount^2, Common->lnz = sum ColCount, Common->anz =
 *     n + strictly-lower entries (cholmod_rowcolcounts.c:420-445, 513-524);
 *   - fundamental supernodes, relaxed amalgamation, the row pattern L->s,
 *     L->pi, L->px, maxcsize and maxesize, following the steps of
 *     CHOLMOD/Supernodal/cholmod_super_symbolic.c:400-930 (the merge rule of
 *     the relaxed amalgamation is a heuristic whose every step must match
 *     for the supernode partition to be identical, so the same steps are
 *     taken here, in this file's own code).
 */
#include "gb_internal.h"
#include <math.h>
#include <stdlib.h>
#include <string.h>

/* ---- S = tril(A(p,p)) ------------------------------------------------------ */

cholmod_sparse *gb_permute_lower(cholmod_sparse *A, const Int *Perm,
                                 cholmod_common *Common)
{
    Int n = (Int)A->nrow;
    const Int *Ap = A->p, *Ai = A->i, *Anz = A->nz;
    int single = A->dtype == CHOLMOD_SINGLE;
    Int *Pinv = gb_malloc(n, sizeof(Int), Common);
    Int *cnt = gb_calloc(n + 1, sizeof(Int), Common);
    if (!Pinv || !cnt) {
        gb_free(n, sizeof(Int), Pinv, Common);
        gb_free(n + 1, sizeof(Int), cnt, Common);
        return NULL;
    }
    for (Int k = 0; k < n; k++) Pinv[Perm ? Perm[k] : k] = k;
    Int nz = 0;
    for (Int j = 0; j < n; j++) {
        Int p = Ap[j], pend = A->packed ? Ap[j + 1] : p + Anz[j];
        for (; p < pend; p++) {
            Int i = Ai[p];
            if (i < j) continue;           /* upper entries of stype<0 ignored */
            Int pi = Pinv[i], pj = Pinv[j];
            cnt[GB_MIN(pi, pj)]++;
            nz++;
        }
    }
    cholmod_sparse *S = gb300_allocate_sparse(n, n, nz, TRUE, TRUE, -1,
        CHOLMOD_REAL + A->dtype, Common);
    if (!S) {
        gb_free(n, sizeof(Int), Pinv, Common);
        gb_free(n + 1, sizeof(Int), cnt, Common);
        return NULL;
    }
    Int *Sp = S->p, *Si = S->i;
    Sp[0] = 0;
    for (Int k = 0; k < n; k++) Sp[k + 1] = Sp[k] + cnt[k];
    for (Int k = 0; k < n; k++) cnt[k] = Sp[k];
    /* Scatter column by column of A in increasing *new row* order is not
     * guaranteed; sort each column afterwards (insertion sort, columns are
     * short). */
    for (Int j = 0; j < n; j++) {
        Int p = Ap[j], pend = A->packed ? Ap[j + 1] : p + Anz[j];
        for (; p < pend; p++) {
            Int i = Ai[p];
            if (i < j) continue;
            Int pi = Pinv[i], pj = Pinv[j];
            Int c = GB_MIN(pi, pj), r = GB_MAX(pi, pj);
            Int q = cnt[c]++;
            Si[q] = r;
            if (single) ((float *)S->x)[q] = ((const float *)A->x)[p];
            else ((double *)S->x)[q] = ((const double *)A->x)[p];
        }
    }
    for (Int k = 0; k < n; k++) {
        for (Int q = Sp[k] + 1; q < Sp[k + 1]; q++) {
            Int r = Si[q];
            double vd = single ? 0 : ((double *)S->x)[q];
            float vf = single ? ((float *)S->x)[q] : 0;
            Int t = q - 1;
            while (t >= Sp[k] && Si[t] > r) {
                Si[t + 1] = Si[t];
                if (single) ((float *)S->x)[t + 1] = ((float *)S->x)[t];
                else ((double *)S->x)[t + 1] = ((double *)S->x)[t];
                t--;
            }
            Si[t + 1] = r;
            if (single) ((float *)S->x)[t + 1] = vf; else ((double *)S->x)[t + 1] = vd;
        }
    }
    gb_free(n, sizeof(Int), Pinv, Common);
    gb_free(n + 1, sizeof(Int), cnt, Common);
    return S;
}

/* ---- upper pattern (row form of the lower S) ------------------------------ */

static int upper_pattern(Int n, const Int *Sp, const Int *Si, Int **Up_out,
                         Int **Ui_out, cholmod_common *Common)
{
    Int nz = Sp[n];
    Int *Up = gb_calloc(n + 1, sizeof(Int), Common);
    Int *Ui = gb_malloc(GB_MAX(nz, 1), sizeof(Int), Common);
    if (!Up || !Ui) {
        gb_free(n + 1, sizeof(Int), Up, Common);
        gb_free(nz, sizeof(Int), Ui, Common);
        return FALSE;
    }
    for (Int p = 0; p < nz; p++) Up[Si[p] + 1]++;
    for (Int k = 0; k < n; k++) Up[k + 1] += Up[k];
    Int *w = gb_malloc(n, sizeof(Int), Common);
    if (!w) { gb_free(n + 1, sizeof(Int), Up, Common); gb_free(nz, sizeof(Int), Ui, Common); return FALSE; }
    memcpy(w, Up, n * sizeof(Int));
    for (Int j = 0; j < n; j++)                /* rows of column i come out sorted */
        for (Int p = Sp[j]; p < Sp[j + 1]; p++) Ui[w[Si[p]]++] = j;
    gb_free(n, sizeof(Int), w, Common);
    *Up_out = Up;
    *Ui_out = Ui;
    return TRUE;
}

/* ---- relaxed supernodal partition and pattern ----------------------------- */

static void subtree_rows(Int k, Int k1, const Int *Up, const Int *Ui,
                         const Int *SuperMap, const Int *Sparent, Int *Flag,
                         Int *Ls, Int *Lpi2)
{
    /* rows i < k1 of column k of the upper part: walk the supernodal etree
     * from SuperMap[i] until a supernode already holding row k */
    for (Int p = Up[k]; p < Up[k + 1]; p++) {
        Int i = Ui[p];
        if (i >= k1) break;                    /* Ui sorted within a column */
        for (Int si = SuperMap[i]; Flag[si] != k; si = Sparent[si]) {
            Ls[Lpi2[si]++] = k;
            Flag[si] = k;
        }
    }
}

/* Column counts of L (diagonal included) by the algorithm of Gilbert, Ng
 * and Peyton ("An efficient algorithm to compute row and column counts for
 * sparse Cholesky factorization", SIAM J. Matrix Anal. Appl. 15, 1994): row
 * i of L is the row subtree of the etree spanned by the columns j < i with
 * A(i,j) != 0; walking the columns in a postorder, j is a leaf of row
 * subtree i exactly when its first descendant comes after the first
 * descendant of row i's previous leaf, and every leaf after the first adds
 * the path from itself up to the least common ancestor with the previous
 * leaf, found by a disjoint-set forest with path compression.  The counts
 * are kept as differences (delta) and summed up the tree at the end.  The
 * reference obtains the same counts with cholmod_rowcolcounts
 * (CHOLMOD/Cholesky/cholmod_rowcolcounts.c).  O(nnz(A) alpha(n)) time,
 * instead of visiting every entry of L.  S = tril(PAP') by columns; W: 5 n. */
static void col_counts(Int n, const Int *Parent, const Int *Sp, const Int *Si, Int *ColCount,
                       Int *W)
{
    Int *post = W, *head = W + n, *next = W + 2 * n, *stack = W + 3 * n;
    /* a postorder of the etree (children visited in increasing order) */
    for (Int j = 0; j < n; j++) head[j] = EMPTY;
    for (Int j = n - 1; j >= 0; j--)
        if (Parent[j] != EMPTY) { next[j] = head[Parent[j]]; head[Parent[j]] = j; }
    Int k = 0;
    for (Int r = 0; r < n; r++) {
        if (Parent[r] != EMPTY) continue;
        Int top = 0;
        stack[0] = r;
        while (top >= 0) {
            Int p = stack[top], c = head[p];
            if (c == EMPTY) { top--; post[k++] = p; }
            else { head[p] = next[c]; stack[++top] = c; }
        }
    }
    /* head/next/stack are free now: first descendant, largest first
     * descendant of each row subtree's last leaf, previous leaf, ancestor */
    Int *first = W + n, *maxfirst = W + 2 * n, *prevleaf = W + 3 * n, *anc = W + 4 * n;
    Int *delta = ColCount;
    for (Int j = 0; j < n; j++) { first[j] = EMPTY; maxfirst[j] = EMPTY; prevleaf[j] = EMPTY; anc[j] = j; }
    for (Int q = 0; q < n; q++) {
        Int j = post[q];
        delta[j] = first[j] == EMPTY;            /* 1 for a leaf of the etree */
        for (; j != EMPTY && first[j] == EMPTY; j = Parent[j]) first[j] = q;
    }
    for (Int q = 0; q < n; q++) {
        Int j = post[q];
        if (Parent[j] != EMPTY) delta[Parent[j]]--;
        for (Int p = Sp[j]; p < Sp[j + 1]; p++) {
            Int i = Si[p];
            if (i <= j || first[j] <= maxfirst[i]) continue;   /* j: not a leaf of row i */
            maxfirst[i] = first[j];
            Int jprev = prevleaf[i];
            prevleaf[i] = j;
            delta[j]++;
            if (jprev == EMPTY) continue;                      /* row i's first leaf */
            Int r = jprev;                                     /* least common ancestor */
            while (r != anc[r]) r = anc[r];
            for (Int t = jprev; t != r;) { Int up = anc[t]; anc[t] = r; t = up; }
            delta[r]--;
        }
        if (Parent[j] != EMPTY) anc[j] = Parent[j];
    }
    for (Int q = 0; q < n; q++) {
        Int j = post[q];
        if (Parent[j] != EMPTY) ColCount[Parent[j]] += ColCount[j];
    }
}

cholmod_factor *gb_analyze_perm(cholmod_sparse *A, const Int *Perm,
                                cholmod_common *Common)
{
    Int n = (Int)A->nrow;
    cholmod_factor *L = NULL;
    cholmod_sparse *S = gb_permute_lower(A, Perm, Common);
    if (!S) return NULL;
    const Int *Sp = S->p, *Si = S->i;
    Int *Up = NULL, *Ui = NULL;
    Int *Parent = gb_malloc(n, sizeof(Int), Common);
    Int *ColCount = gb_calloc(n, sizeof(Int), Common);
    Int *W = gb_malloc(6 * (n + 1), sizeof(Int), Common);
    if (!Parent || !ColCount || !W || !upper_pattern(n, Sp, Si, &Up, &Ui, Common))
        goto fail;

    /* elimination tree (Liu), using W as the ancestor array */
    Int *Anc = W;
    for (Int k = 0; k < n; k++) {
        Parent[k] = EMPTY;
        Anc[k] = EMPTY;
        for (Int p = Up[k]; p < Up[k + 1]; p++) {
            Int i = Ui[p];
            while (i != EMPTY && i < k) {
                Int inext = Anc[i];
                Anc[i] = k;
                if (inext == EMPTY) Parent[i] = k;
                i = inext;
            }
        }
    }

    /* column counts (with the diagonal) from the row subtrees' leaves */
    col_counts(n, Parent, Sp, Si, ColCount, W);
    {
        double fl = 0, lnz = 0, anz = (double)n;
        for (Int j = 0; j < n; j++) {
            double ff = (double)ColCount[j];
            lnz += ff;
            fl += ff * ff;
        }
        for (Int j = 0; j < n; j++)
            for (Int p = Sp[j]; p < Sp[j + 1]; p++)
                if (Si[p] > j) anz++;
        Common->fl = fl;
        Common->lnz = lnz;
        Common->anz = anz;
    }

    /* fundamental supernodes: j joins j-1 when j is j-1's parent, its only
     * child, and column j-1's pattern is column j's plus the diagonal */
    Int *Wi = W, *Super = W + (n + 1), *SuperMap = W + 2 * (n + 1),
        *Sparent = W + 3 * (n + 1), *Snz = W + 4 * (n + 1), *Merged = W + 5 * (n + 1);
    for (Int j = 0; j < n; j++) Wi[j] = 0;
    for (Int j = 0; j < n; j++)
        if (Parent[j] != EMPTY) Wi[Parent[j]]++;
    Int nfsuper = (n == 0) ? 0 : 1;
    Super[0] = 0;
    for (Int j = 1; j < n; j++) {
        if (Parent[j - 1] != j || ColCount[j - 1] != ColCount[j] + 1 || Wi[j] > 1)
            Super[nfsuper++] = j;
    }
    Super[nfsuper] = n;
    Int *Nscol = Wi;
    for (Int s = 0; s < nfsuper; s++)
        for (Int k = Super[s]; k < Super[s + 1]; k++) SuperMap[k] = s;
    for (Int s = 0; s < nfsuper; s++) {
        Int par = Parent[Super[s + 1] - 1];
        Sparent[s] = (par == EMPTY) ? EMPTY : SuperMap[par];
    }

    /* relaxed amalgamation: from the last pair backwards, merge s into its
     * parent s+1 when few columns or few explicit zeros would result */
    Int *Zeros = SuperMap;      /* SuperMap is rebuilt below */
    for (Int s = 0; s < nfsuper; s++) {
        Merged[s] = EMPTY;
        Nscol[s] = Super[s + 1] - Super[s];
        Zeros[s] = 0;
        Snz[s] = ColCount[Super[s]];
    }
    double zr0 = isnan(Common->zrelax[0]) ? 0 : Common->zrelax[0];
    double zr1 = isnan(Common->zrelax[1]) ? 0 : Common->zrelax[1];
    double zr2 = isnan(Common->zrelax[2]) ? 0 : Common->zrelax[2];
    Int nr0 = (Int)Common->nrelax[0], nr1 = (Int)Common->nrelax[1],
        nr2 = (Int)Common->nrelax[2];
    for (Int s = nfsuper - 2; s >= 0; s--) {
        if (Sparent[s] == EMPTY) continue;
        Int ss;
        for (ss = Sparent[s]; Merged[ss] != EMPTY; ss = Merged[ss]) ;
        Int sparent = ss;
        for (ss = Sparent[s]; Merged[ss] != EMPTY;) {   /* path compression */
            Int snext = Merged[ss];
            Merged[ss] = sparent;
            ss = snext;
        }
        if (sparent != s + 1) continue;
        Int nscol0 = Nscol[s], nscol1 = Nscol[s + 1], ns = nscol0 + nscol1;
        Int totzeros = Zeros[s + 1];
        double lnz1 = (double)Snz[s + 1];
        int merge;
        if (ns <= nr0) {
            merge = TRUE;
        } else {
            double lnz0 = (double)Snz[s];
            double xnewzeros = nscol0 * (lnz1 + nscol0 - lnz0);
            Int newzeros = nscol0 * (Snz[s + 1] + nscol0 - Snz[s]);
            if (xnewzeros == 0) {
                merge = TRUE;
            } else {
                double xtotzeros = ((double)totzeros) + xnewzeros;
                double xns = (double)ns;
                double xtotsize = (xns * (xns + 1) / 2) + xns * (lnz1 - nscol1);
                double z = xtotzeros / xtotsize;
                totzeros += newzeros;
                merge = ((ns <= nr1 && z < zr0) || (ns <= nr2 && z < zr1) || (z < zr2))
                        && (xtotsize < ((double)INT64_MAX) / sizeof(double));
            }
        }
        if (merge) {
            Zeros[s] = totzeros;
            Merged[s + 1] = s;
            Snz[s] = nscol0 + Snz[s + 1];
            Nscol[s] += Nscol[s + 1];
        }
    }
    Int nsuper = 0;
    for (Int s = 0; s < nfsuper; s++) {
        if (Merged[s] == EMPTY) {
            Super[nsuper] = Super[s];
            Snz[nsuper] = Snz[s];
            nsuper++;
        }
    }
    Super[nsuper] = n;
    for (Int s = 0; s < nsuper; s++)
        for (Int k = Super[s]; k < Super[s + 1]; k++) SuperMap[k] = s;
    for (Int s = 0; s < nsuper; s++) {
        Int par = Parent[Super[s + 1] - 1];
        Sparent[s] = (par == EMPTY) ? EMPTY : SuperMap[par];
    }
    size_t ssize = 0, xsize = 0;
    for (Int s = 0; s < nsuper; s++) {
        size_t nscol = (size_t)(Super[s + 1] - Super[s]), nsrow = (size_t)Snz[s];
        ssize += nsrow;
        xsize += nscol * nsrow;
    }

    /* allocate the supernodal symbolic factor */
    L = gb_calloc(1, sizeof(cholmod_factor), Common);
    if (!L) goto fail;
    L->n = n;
    L->minor = n;
    L->nsuper = nsuper;
    L->ssize = GB_MAX(ssize, 1);
    L->xsize = GB_MAX(xsize, 1);
    L->ordering = CHOLMOD_GIVEN;
    L->is_ll = TRUE;
    L->is_super = TRUE;
    L->is_monotonic = TRUE;
    L->itype = CHOLMOD_LONG;
    L->xtype = CHOLMOD_PATTERN;
    L->dtype = CHOLMOD_DOUBLE;
    L->Perm = gb_malloc(n, sizeof(Int), Common);
    L->ColCount = gb_malloc(n, sizeof(Int), Common);
    L->super = gb_malloc(nsuper + 1, sizeof(Int), Common);
    L->pi = gb_malloc(nsuper + 1, sizeof(Int), Common);
    L->px = gb_malloc(nsuper + 1, sizeof(Int), Common);
    L->s = gb_malloc(L->ssize, sizeof(Int), Common);
    if (!L->Perm || !L->ColCount || !L->super || !L->pi || !L->px || !L->s) goto fail;
    Int *LPerm = L->Perm, *Lsuper = L->super, *Lpi = L->pi, *Lpx = L->px, *Ls = L->s;
    for (Int k = 0; k < n; k++) LPerm[k] = Perm ? Perm[k] : k;
    memcpy(L->ColCount, ColCount, n * sizeof(Int));
    for (Int s = 0; s <= nsuper; s++) Lsuper[s] = Super[s];
    Ls[0] = 0;
    Int p = 0;
    for (Int s = 0; s < nsuper; s++) { Lpi[s] = p; p += Snz[s]; }
    Lpi[nsuper] = p;
    p = 0;
    for (Int s = 0; s < nsuper; s++) {
        Lpx[s] = p;
        p += (Lsuper[s + 1] - Lsuper[s]) * Snz[s];
    }
    Lpx[nsuper] = p;

    /* row pattern of each relaxed supernode */
    Int *Lpi2 = Wi, *Flag = Merged;
    for (Int s = 0; s < nsuper; s++) { Lpi2[s] = Lpi[s]; Flag[s] = EMPTY; }
    for (Int s = 0; s < nsuper; s++) {
        Int k1 = Lsuper[s], k2 = Lsuper[s + 1];
        for (Int k = k1; k < k2; k++) Ls[Lpi2[s]++] = k;
        for (Int k = k1; k < k2; k++) {
            Flag[s] = k;
            subtree_rows(k, k1, Up, Ui, SuperMap, Sparent, Flag, Ls, Lpi2);
        }
    }

    /* largest update block (maxcsize) and largest off-diagonal row count
     * (maxesize), as cholmod_super_symbolic.c:889-928 defines them */
    {
        Int maxcsize = 1, maxesize = 1;
        for (Int d = 0; d < nsuper; d++) {
            Int nscol = Lsuper[d + 1] - Lsuper[d];
            Int q = Lpi[d] + nscol, plast = q, pend = Lpi[d + 1];
            maxesize = GB_MAX(maxesize, pend - q);
            Int slast = (q == pend) ? EMPTY : SuperMap[Ls[q]];
            for (; q <= pend; q++) {
                Int s2 = (q == pend) ? EMPTY : SuperMap[Ls[q]];
                if (s2 != slast) {
                    Int ndrow1 = q - plast, ndrow2 = pend - plast;
                    maxcsize = GB_MAX(maxcsize, ndrow2 * ndrow1);
                    plast = q;
                    slast = s2;
                }
            }
        }
        L->maxcsize = maxcsize;
        L->maxesize = maxesize;
    }

    gb_free(6 * (n + 1), sizeof(Int), W, Common);
    gb_free(n, sizeof(Int), Parent, Common);
    gb_free(n, sizeof(Int), ColCount, Common);
    gb_free(n + 1, sizeof(Int), Up, Common);
    gb_free(Sp[n], sizeof(Int), Ui, Common);
    gb300_free_sparse(&S, Common);
    Common->status = CHOLMOD_OK;
    return L;

fail:
    if (L) gb300_free_factor(&L, Common);
    gb_free(6 * (n + 1), sizeof(Int), W, Common);
    gb_free(n, sizeof(Int), Parent, Common);
    gb_free(n, sizeof(Int), ColCount, Common);
    if (Up) gb_free(n + 1, sizeof(Int), Up, Common);
    if (Ui) gb_free(Sp[n], sizeof(Int), Ui, Common);
    gb300_free_sparse(&S, Common);
    return NULL;
}

cholmod_factor *gb300_analyze_perm(cholmod_sparse *A, const int64_t *Perm,
                                   cholmod_common *Common)
{
    if (!Common) return NULL;
    Common->status = CHOLMOD_OK;
    if (!A) { GB_ERROR(CHOLMOD_INVALID, "argument missing"); return NULL; }
    if (A->nrow != A->ncol || A->stype >= 0 || A->itype != CHOLMOD_LONG) {
        GB_ERROR(CHOLMOD_INVALID, "A must be square, symmetric-lower, int64");
        return NULL;
    }
    Int n = (Int)A->nrow;
    if (Perm) {   /* Perm must be a permutation of 0..n-1 */
        char *seen = calloc(n > 0 ? n : 1, 1);
        if (!seen) { GB_ERROR(CHOLMOD_OUT_OF_MEMORY, "out of memory"); return NULL; }
        for (Int k = 0; k < n; k++) {
            Int j = Perm[k];
            if (j < 0 || j >= n || seen[j]) {
                free(seen);
                GB_ERROR(CHOLMOD_INVALID, "invalid permutation");
                return NULL;
            }
            seen[j] = 1;
        }
        free(seen);
    }
    return gb_analyze_perm(A, Perm, Common);
}

/* Symbolic factor of a batch of independent systems: the block-diagonal
 * matrix diag(A_0, A_1, ...) where system i has the pattern of Lpat[sys_pat[i]]
 * (each a supernodal symbolic factor from gb300_analyze_perm or
 * cholmod_analyze).  Supernodes never span two blocks (the etree of a
 * block-diagonal matrix is a forest and relaxed amalgamation only merges a
 * supernode with its parent), so the result is the concatenation of the
 * blocks' factors with their column, row-index and value offsets, and it
 * equals gb300_analyze_perm of the block-diagonal matrix with the
 * block-diagonal permutation.  No counterpart in the reference, which
 * factors one matrix per call. */
cholmod_factor *gb300_batch_analyze(int npat, cholmod_factor *const *Lpat, int64_t nsys,
                                    const int32_t *sys_pat, cholmod_common *Common)
{
    if (!Common) return NULL;
    Common->status = CHOLMOD_OK;
    if (npat < 1 || !Lpat || nsys < 1 || !sys_pat) {
        GB_ERROR(CHOLMOD_INVALID, "invalid batch description");
        return NULL;
    }
    for (int p = 0; p < npat; p++) {
        const cholmod_factor *F = Lpat[p];
        if (!F || !F->is_super || F->itype != CHOLMOD_LONG || !F->super || !F->pi || !F->px
            || !F->s || !F->Perm || !F->ColCount) {
            GB_ERROR(CHOLMOD_INVALID, "each pattern must be a supernodal symbolic factor");
            return NULL;
        }
    }
    Int n = 0, nsuper = 0, ssz = 0, xsz = 0, maxc = 1, maxe = 1;
    for (int64_t i = 0; i < nsys; i++) {
        if (sys_pat[i] < 0 || sys_pat[i] >= npat) {
            GB_ERROR(CHOLMOD_INVALID, "system pattern index out of range");
            return NULL;
        }
        const cholmod_factor *F = Lpat[sys_pat[i]];
        const Int *Fpi = F->pi, *Fpx = F->px;
        n += (Int)F->n;
        nsuper += (Int)F->nsuper;
        ssz += Fpi[F->nsuper];
        xsz += Fpx[F->nsuper];
        maxc = GB_MAX(maxc, (Int)F->maxcsize);
        maxe = GB_MAX(maxe, (Int)F->maxesize);
    }
    cholmod_factor *L = gb_calloc(1, sizeof(cholmod_factor), Common);
    if (!L) return NULL;
    L->n = n;
    L->minor = n;
    L->nsuper = nsuper;
    L->ssize = GB_MAX(ssz, 1);
    L->xsize = GB_MAX(xsz, 1);
    L->maxcsize = maxc;
    L->maxesize = maxe;
    L->ordering = CHOLMOD_GIVEN;
    L->is_ll = TRUE;
    L->is_super = TRUE;
    L->is_monotonic = TRUE;
    L->itype = CHOLMOD_LONG;
    L->xtype = CHOLMOD_PATTERN;
    L->dtype = CHOLMOD_DOUBLE;
    L->Perm = gb_malloc(GB_MAX(n, 1), sizeof(Int), Common);
    L->ColCount = gb_malloc(GB_MAX(n, 1), sizeof(Int), Common);
    L->super = gb_malloc(nsuper + 1, sizeof(Int), Common);
    L->pi = gb_malloc(nsuper + 1, sizeof(Int), Common);
    L->px = gb_malloc(nsuper + 1, sizeof(Int), Common);
    L->s = gb_malloc(L->ssize, sizeof(Int), Common);
    if (!L->Perm || !L->ColCount || !L->super || !L->pi || !L->px || !L->s) {
        gb300_free_factor(&L, Common);
        return NULL;
    }
    Int *Perm = L->Perm, *CC = L->ColCount, *Sup = L->super, *Pi = L->pi, *Px = L->px, *Ls = L->s;
    Int c0 = 0, s0 = 0, p0 = 0, x0 = 0;
    for (int64_t i = 0; i < nsys; i++) {
        const cholmod_factor *F = Lpat[sys_pat[i]];
        const Int fn = (Int)F->n, fns = (Int)F->nsuper;
        const Int *FPerm = F->Perm, *FCC = F->ColCount, *FSup = F->super, *FPi = F->pi,
                  *FPx = F->px, *FLs = F->s;
        for (Int k = 0; k < fn; k++) {
            Perm[c0 + k] = c0 + FPerm[k];
            CC[c0 + k] = FCC[k];
        }
        for (Int s = 0; s < fns; s++) {
            Sup[s0 + s] = c0 + FSup[s];
            Pi[s0 + s] = p0 + FPi[s];
            Px[s0 + s] = x0 + FPx[s];
        }
        for (Int q = 0; q < FPi[fns]; q++) Ls[p0 + q] = c0 + FLs[q];
        c0 += fn;
        s0 += fns;
        p0 += FPi[fns];
        x0 += FPx[fns];
    }
    Sup[nsuper] = n;
    Pi[nsuper] = p0;
    Px[nsuper] = x0;
    if (ssz == 0) Ls[0] = 0;
    return L;
}
