/* gb_aft.c -- the unsymmetric form of cholmod_l_super_numeric: factorize
 * beta I + A F (F = A' or A(:,f)'), whose column k the reference assembles
 * into the supernode as the sum over the entries F(j,k) of F(j,k) A(:,j),
 * rows i >= k (Supernodal/t_cholmod_super_numeric_worker.c:471-506, the
 * matrix cholmod_factorize_p passes for an unsymmetric A,
 * Cholesky/cholmod_factorize.c:240-248).
 *
 * Here the product's lower triangle C = tril(A F) is formed before the
 * factorization: the host computes its pattern (integer work, sorted rows)
 * and, for every entry of C, the list of products that make it, (position
 * in A, position in F) in the order the reference adds them (F's column k
 * entry by entry, then A's column j row by row); the device sums each
 * list (gb_launch_pair_sum) into the values of C, which then go through
 * the ordinary symmetric-lower path.  The sums start from zero and add in
 * the same order as the reference's L_MULTADD loop.
 */
#include "gb_internal.h"
#include <stdlib.h>
#include <string.h>

/* C = tril(A F) pattern (n x n, packed, sorted, stype -1, values zero) and
 * the pair lists: products of entry e are pairs[2q], pairs[2q+1] (positions
 * in A->x and F->x) for q in [pptr[e], pptr[e+1]).  NULL on failure. */
cholmod_sparse *gb_aft_pattern(cholmod_sparse *A, cholmod_sparse *F, int64_t **pptr_out,
                               int64_t **pairs_out, cholmod_common *Common)
{
    const Int n = (Int)A->nrow;
    const Int *Ap = A->p, *Ai = A->i, *Anz = A->nz;
    const Int *Fp = F->p, *Fi = F->i, *Fnz = F->nz;
    Int *mark = malloc(sizeof(Int) * (n + 1));
    Int *rows = malloc(sizeof(Int) * (n + 1));
    Int *cp = calloc(n + 1, sizeof(Int));
    int64_t *pcnt = NULL, *pptr = NULL, *pairs = NULL;
    Int *epos = malloc(sizeof(Int) * (n + 1));
    cholmod_sparse *C = NULL;
    if (!mark || !rows || !cp || !epos) goto fail;
    for (Int i = 0; i < n; i++) mark[i] = -1;
    /* pass 1: entries per column, products in total */
    int64_t npairs = 0;
    for (Int k = 0; k < n; k++) {
        Int pf = Fp[k], pfend = F->packed ? Fp[k + 1] : pf + Fnz[k];
        for (; pf < pfend; pf++) {
            const Int j = Fi[pf];
            Int p = Ap[j], pend = A->packed ? Ap[j + 1] : p + Anz[j];
            for (; p < pend; p++) {
                const Int i = Ai[p];
                if (i < k) continue;
                npairs++;
                if (mark[i] != k) { mark[i] = k; cp[k + 1]++; }
            }
        }
    }
    for (Int k = 0; k < n; k++) cp[k + 1] += cp[k];
    const Int nz = cp[n];
    C = gb300_allocate_sparse(n, n, nz, TRUE, TRUE, -1, CHOLMOD_REAL + A->dtype, Common);
    pcnt = calloc(nz + 1, sizeof(int64_t));
    pptr = malloc(sizeof(int64_t) * (nz + 1));
    pairs = malloc(sizeof(int64_t) * 2 * (npairs + 1));
    if (!C || !pcnt || !pptr || !pairs) goto fail;
    Int *Cp = C->p, *Ci = C->i;
    memcpy(Cp, cp, sizeof(Int) * (n + 1));
    memset(C->x, 0, (A->dtype == CHOLMOD_SINGLE ? sizeof(float) : sizeof(double)) * (nz ? nz : 1));
    for (Int i = 0; i < n; i++) mark[i] = -1;
    /* pass 2: each column's rows, sorted; products per entry */
    for (Int k = 0; k < n; k++) {
        Int nr = 0;
        Int pf = Fp[k], pfend = F->packed ? Fp[k + 1] : pf + Fnz[k];
        for (Int q = pf; q < pfend; q++) {
            const Int j = Fi[q];
            Int p = Ap[j], pend = A->packed ? Ap[j + 1] : p + Anz[j];
            for (; p < pend; p++) {
                const Int i = Ai[p];
                if (i >= k && mark[i] != k) { mark[i] = k; rows[nr++] = i; }
            }
        }
        /* insertion sort: columns of C are short */
        for (Int a = 1; a < nr; a++) {
            Int v = rows[a], b = a - 1;
            while (b >= 0 && rows[b] > v) { rows[b + 1] = rows[b]; b--; }
            rows[b + 1] = v;
        }
        for (Int a = 0; a < nr; a++) {
            Ci[Cp[k] + a] = rows[a];
            epos[rows[a]] = Cp[k] + a;
        }
        for (Int q = pf; q < pfend; q++) {
            const Int j = Fi[q];
            Int p = Ap[j], pend = A->packed ? Ap[j + 1] : p + Anz[j];
            for (; p < pend; p++)
                if (Ai[p] >= k) pcnt[epos[Ai[p]] + 1]++;
        }
    }
    pptr[0] = 0;
    for (Int e = 0; e < nz; e++) pptr[e + 1] = pptr[e] + pcnt[e + 1];
    for (Int e = 0; e < nz; e++) pcnt[e] = pptr[e];
    /* pass 3: the products, in the reference's order for each entry */
    for (Int k = 0; k < n; k++) {
        for (Int a = Cp[k]; a < Cp[k + 1]; a++) epos[Ci[a]] = a;
        Int pf = Fp[k], pfend = F->packed ? Fp[k + 1] : pf + Fnz[k];
        for (Int q = pf; q < pfend; q++) {
            const Int j = Fi[q];
            Int p = Ap[j], pend = A->packed ? Ap[j + 1] : p + Anz[j];
            for (; p < pend; p++) {
                if (Ai[p] < k) continue;
                const int64_t w = pcnt[epos[Ai[p]]]++;
                pairs[2 * w] = p;
                pairs[2 * w + 1] = q;
            }
        }
    }
    free(mark); free(rows); free(cp); free(epos); free(pcnt);
    *pptr_out = pptr;
    *pairs_out = pairs;
    return C;
fail:
    free(mark); free(rows); free(cp); free(epos); free(pcnt); free(pptr); free(pairs);
    if (C) gb300_free_sparse(&C, Common);
    GB_ERROR(CHOLMOD_OUT_OF_MEMORY, "out of memory");
    return NULL;
}
