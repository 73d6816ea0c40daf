/* gb_valmap.c -- device-side value permutation for refactorizations.
 *
 * gb300_factorize_mixed needs, from the caller's A (lower triangle, CSC),
 * the values of S = tril(P A P') in the factor's column order (assembly),
 * both triangles of A in compressed rows (residual of the refinement) and
 * the diagonal scaling D = diag(A)^-1/2.  The reference forms S on the host
 * (cholmod_factorize.c:220-250, transpose_sym).  Here the index maps from
 * A's value array to those arrays are built once per pattern, by running
 * the host permutation on a copy of A whose values are their own positions,
 * and every factorization uploads only A's values and gathers on the GPU.
 * The caller's pattern is compared with the one the maps were built for on
 * every call (a pattern change rebuilds them).
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include "gb_internal.h"
#include "gb_plan.h"

void gb_valmap_free(gb_plan *P)
{
    free(P->h_vm_Ap); free(P->h_vm_Ai); free(P->h_vm_Anz);
    free(P->h_vm_Sp); free(P->h_vm_Si);
    P->h_vm_Ap = P->h_vm_Ai = P->h_vm_Anz = P->h_vm_Sp = P->h_vm_Si = NULL;
    void *dev[] = {P->d_smap, P->d_rmap, P->d_dmap, P->d_Ax};
    for (size_t i = 0; i < sizeof dev / sizeof dev[0]; i++)
        if (dev[i]) cudaFree(dev[i]);
    P->d_smap = P->d_rmap = P->d_dmap = NULL;
    P->d_Ax = NULL;
    P->ax_cap = 0;
    P->vm_valid = 0;
    P->vm_bytes = 0;
}

/* length of A's value array that entries can occupy */
static Int value_extent(const cholmod_sparse *A)
{
    Int n = (Int)A->ncol;
    const Int *Ap = A->p, *Anz = A->nz;
    if (A->packed) return Ap[n];
    Int e = 0;
    for (Int j = 0; j < n; j++) e = GB_MAX(e, Ap[j] + Anz[j]);
    return e;
}

/* The part of the pattern check that costs nothing: maps built for this n
 * and packing, and a packed A with as many entries, so that the value copy
 * and the gathers stay inside A->x and the device arrays.  The comparison
 * of Ap and Ai (gb_valmap_verify) can then run while the factorization
 * does. */
static int same_shape(const gb_plan *P, const cholmod_sparse *A)
{
    Int n = (Int)A->ncol;
    return P->vm_valid && P->vm_n == n && P->vm_packed == A->packed && A->packed
           && ((const Int *)A->p)[n] == P->vm_xlen;
}

static int same_pattern(const gb_plan *P, const cholmod_sparse *A)
{
    Int n = (Int)A->ncol;
    if (!P->vm_valid || P->vm_n != n || P->vm_packed != A->packed) return 0;
    if (memcmp(P->h_vm_Ap, A->p, sizeof(Int) * (n + 1)) != 0) return 0;
    if (!A->packed && memcmp(P->h_vm_Anz, A->nz, sizeof(Int) * n) != 0) return 0;
    return memcmp(P->h_vm_Ai, A->i, sizeof(Int) * P->vm_xlen) == 0;
}

#define UPLOAD(dst, src, bytes)                                                         \
    (cudaMalloc((void **)&(dst), (bytes) ? (bytes) : 16) == cudaSuccess                 \
     && (!(bytes) || cudaMemcpy((dst), (src), (bytes), cudaMemcpyHostToDevice) == cudaSuccess))

/* Build the maps for A's pattern.  Returns FALSE (maps unusable, the caller
 * falls back to the host path) on allocation failure or when A holds
 * duplicate entries (the tags of S would be sums, not positions). */
static int build(gb_plan *P, cholmod_sparse *A, cholmod_common *Common)
{
    gb_valmap_free(P);
    Int n = (Int)A->ncol, xlen = value_extent(A);
    const Int *Ap = A->p, *Ai = A->i, *Anz = A->nz;
    cholmod_sparse *T = gb300_allocate_sparse(n, n, GB_MAX(xlen, 1), A->sorted, A->packed, A->stype,
                                              CHOLMOD_REAL, Common);
    if (!T) return FALSE;
    memcpy(T->p, Ap, sizeof(Int) * (n + 1));
    memcpy(T->i, Ai, sizeof(Int) * xlen);
    if (!A->packed) memcpy(T->nz, Anz, sizeof(Int) * n);
    double *tx = T->x;
    for (Int p = 0; p < xlen; p++) tx[p] = (double)p;
    cholmod_sparse *S = gb_permute_lower(T, P->L->Perm, Common);
    gb300_free_sparse(&T, Common);
    if (!S) return FALSE;
    Int snz = ((Int *)S->p)[n];
    int64_t *smap = malloc(sizeof(int64_t) * GB_MAX(snz, 1));
    int ok = smap != NULL;
    const double *sx = S->x;
    for (Int q = 0; ok && q < snz; q++) {
        double v = sx[q];
        if (!(v >= 0 && v < (double)xlen) || v != floor(v)) ok = 0;
        else smap[q] = (int64_t)v;
    }
    /* both triangles in compressed rows; dmap = position of each diagonal */
    Int *cnt = calloc(n + 1, sizeof(Int));
    int64_t *Rp = malloc(sizeof(int64_t) * (n + 1)), *dmap = malloc(sizeof(int64_t) * (n + 1));
    ok = ok && cnt && Rp && dmap;
    Int rnz = 0;
    for (Int j = 0; ok && j < n; j++) {
        Int p = Ap[j], pend = A->packed ? Ap[j + 1] : p + Anz[j];
        for (; p < pend; p++) {
            Int i = Ai[p];
            if (i < j) continue;
            cnt[i]++;
            rnz++;
            if (i != j) { cnt[j]++; rnz++; }
        }
    }
    int32_t *Rj = ok ? malloc(sizeof(int32_t) * GB_MAX(rnz, 1)) : NULL;
    int64_t *rmap = ok ? malloc(sizeof(int64_t) * GB_MAX(rnz, 1)) : NULL;
    ok = ok && Rj && rmap;
    if (ok) {
        Rp[0] = 0;
        for (Int i = 0; i < n; i++) Rp[i + 1] = Rp[i] + cnt[i];
        for (Int i = 0; i < n; i++) { cnt[i] = Rp[i]; dmap[i] = -1; }
        for (Int j = 0; j < n; j++) {
            Int p = Ap[j], pend = A->packed ? Ap[j + 1] : p + Anz[j];
            for (; p < pend; p++) {
                Int i = Ai[p];
                if (i < j) continue;
                Rj[cnt[i]] = (int32_t)j;
                rmap[cnt[i]++] = p;
                if (i != j) {
                    Rj[cnt[j]] = (int32_t)i;
                    rmap[cnt[j]++] = p;
                } else {
                    dmap[i] = p;
                }
            }
        }
    }
    /* upload the maps and the patterns of S and of the rows */
    ok = ok && gb_dev_grow((void **)&P->d_Rp, &P->rp_cap, sizeof(int64_t) * (n + 1))
         && gb_dev_grow((void **)&P->d_Rj, &P->rj_cap, sizeof(int32_t) * (rnz + 1))
         && gb_dev_grow((void **)&P->d_Rx, &P->rx_cap, sizeof(double) * (rnz + 1))
         && cudaMemcpy(P->d_Rp, Rp, sizeof(int64_t) * (n + 1), cudaMemcpyHostToDevice) == cudaSuccess
         && (!rnz || cudaMemcpy(P->d_Rj, Rj, sizeof(int32_t) * rnz, cudaMemcpyHostToDevice) == cudaSuccess)
         && UPLOAD(P->d_smap, smap, sizeof(int64_t) * snz)
         && UPLOAD(P->d_rmap, rmap, sizeof(int64_t) * rnz)
         && UPLOAD(P->d_dmap, dmap, sizeof(int64_t) * n);
    if (ok) P->vm_bytes = sizeof(int64_t) * (size_t)(snz + rnz + n);
    if (ok) {
        P->h_vm_Ap = malloc(sizeof(Int) * (n + 1));
        P->h_vm_Ai = malloc(sizeof(Int) * GB_MAX(xlen, 1));
        P->h_vm_Anz = A->packed ? NULL : malloc(sizeof(Int) * GB_MAX(n, 1));
        P->h_vm_Sp = malloc(sizeof(Int) * (n + 1));
        P->h_vm_Si = malloc(sizeof(Int) * GB_MAX(snz, 1));
        ok = P->h_vm_Ap && P->h_vm_Ai && (A->packed || P->h_vm_Anz) && P->h_vm_Sp && P->h_vm_Si;
    }
    if (ok) {
        memcpy(P->h_vm_Ap, Ap, sizeof(Int) * (n + 1));
        memcpy(P->h_vm_Ai, Ai, sizeof(Int) * xlen);
        if (!A->packed) memcpy(P->h_vm_Anz, Anz, sizeof(Int) * n);
        memcpy(P->h_vm_Sp, S->p, sizeof(Int) * (n + 1));
        memcpy(P->h_vm_Si, S->i, sizeof(Int) * snz);
        P->vm_n = n;
        P->vm_packed = A->packed;
        P->vm_xlen = xlen;
        P->vm_snz = snz;
        P->vm_rnz = rnz;
        P->vm_valid = 1;
        P->s_from_vm = 0;
    }
    free(smap); free(cnt); free(Rp); free(dmap); free(Rj); free(rmap);
    gb300_free_sparse(&S, Common);
    if (!ok) gb_valmap_free(P);
    return ok;
}

/* Device copies of S = tril(PAP') (FP64 values), of A's rows and of the
 * scaling for the mixed factorization, from A's values.  FALSE: use the
 * host path. */
int gb_valmap_verify(const gb_plan *P, const cholmod_sparse *A) { return same_pattern(P, A); }

int gb_valmap_apply(gb_plan *P, gb_ctx *ctx, cholmod_sparse *A, cholmod_common *Common,
                    int *deferred)
{
    if (A->xtype != CHOLMOD_REAL || A->dtype != CHOLMOD_DOUBLE || A->itype != CHOLMOD_LONG) return FALSE;
    if (deferred && same_shape(P, A)) {
        *deferred = 1;
    } else {
        if (deferred) *deferred = 0;
        if (!same_pattern(P, A) && !build(P, A, Common)) return FALSE;
    }
    cudaStream_t st = ctx->stream;
    Int n = P->vm_n;
    size_t cap = 0;
    int ok = gb_dev_grow((void **)&P->d_Ax, &P->ax_cap, sizeof(double) * GB_MAX(P->vm_xlen, 1))
             && gb_dev_grow((void **)&P->d_Sp, &P->sp_cap, sizeof(int64_t) * (n + 1))
             && gb_dev_grow((void **)&P->d_Si, &P->si_cap, sizeof(int64_t) * GB_MAX(P->vm_snz, 1))
             && gb_dev_grow(&P->d_Sx, &P->sx_cap, sizeof(double) * GB_MAX(P->vm_snz, 1));
    if (ok && !P->d_scale) ok = gb_dev_grow((void **)&P->d_scale, &cap, sizeof(double) * (n + 1));
    cap = 0;
    if (ok && !P->d_scale_perm) ok = gb_dev_grow((void **)&P->d_scale_perm, &cap, sizeof(double) * (n + 1));
    if (!ok) return FALSE;
    if (!P->s_from_vm) {
        /* another entry point uploaded its own S meanwhile */
        ok = cudaMemcpyAsync(P->d_Sp, P->h_vm_Sp, sizeof(int64_t) * (n + 1), cudaMemcpyHostToDevice, st) == cudaSuccess
             && (!P->vm_snz || cudaMemcpyAsync(P->d_Si, P->h_vm_Si, sizeof(int64_t) * P->vm_snz,
                                               cudaMemcpyHostToDevice, st) == cudaSuccess);
        if (!ok) return FALSE;
        P->s_from_vm = 1;
    }
    ok = (!P->vm_xlen || cudaMemcpyAsync(P->d_Ax, A->x, sizeof(double) * P->vm_xlen,
                                         cudaMemcpyHostToDevice, st) == cudaSuccess)
         && gb_launch_gather(P->vm_snz, P->d_smap, P->d_Ax, (double *)P->d_Sx, st) == 0
         && gb_launch_gather(P->vm_rnz, P->d_rmap, P->d_Ax, P->d_Rx, st) == 0
         && gb_launch_diag_scale(n, P->d_dmap, P->d_Ax, P->d_Perm, P->d_scale, P->d_scale_perm, st) == 0
         && gb_launch_anorm_seg(P->nchunk, P->d_chunk, P->nseg, P->d_Rp, P->d_Rx, P->d_anorm_seg, st) == 0
         && cudaMemcpyAsync(P->h_anorm_seg, P->d_anorm_seg, sizeof(double) * P->nseg,
                            cudaMemcpyDeviceToHost, st) == cudaSuccess;
    if (!ok) return FALSE;
    /* h_anorm_seg (pinned) is complete at the caller's next synchronization
     * of the stream; P->anorm is formed there (gb_valmap_anorm) */
    ctx->launches += 4;
    return TRUE;
}

void gb_valmap_anorm(gb_plan *P)
{
    P->anorm = 0;
    for (int64_t g = 0; g < P->nseg; g++) P->anorm = fmax(P->anorm, P->h_anorm_seg[g]);
}
