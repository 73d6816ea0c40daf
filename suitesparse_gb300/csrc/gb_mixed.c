/* gb_mixed.c -- FP32 supernodal factor + FP64 iterative refinement.
 *
 * gb300_factorize_mixed: S = tril(PAP') is uploaded in FP64; the assembly
 * kernel applies the symmetric diagonal scaling D A D (D = diag(A)^-1/2, so
 * every diagonal entry of the scaled matrix is 1) per supernode while it
 * rounds the values to FP32, and the FP32 factor stays on the GPU.  A pivot
 * L(k,k)^2 <= eps_single (relative to the unit diagonal of the scaled
 * matrix), or a failed FP32 factorization, switches to the FP64 factor.
 *
 * gb300_solve_refined: x_0 = 0, r_0 = b; repeat  d = D P' L^-T L^-1 P D r
 * (sweeps in FP32), x += d, r = b - A x (FP64 SpMV on the GPU, both
 * triangles of A resident), until every column's backward error
 * |r|_inf / (|A|_inf |x|_inf + |b|_inf) <= tol.  When the backward error has
 * not decreased for 2 consecutive steps, the matrix is refactored in FP64
 * and refinement continues with that factor.  The refinement scheme is the
 * one the reference's demo applies once (CHOLMOD/Demo/cholmod_di_demo.c
 * :627-663: r = b - A x with cholmod_sdmult, solve, x += dx), iterated here
 * with the stopping and fallback rules above.
 */
#include "gb_plan.h"
#include <math.h>
#include <stdlib.h>
#include <string.h>

#define GB_MAX_REFINE 30

enum { GB_REASON_NONE = GB300_REASON_NONE, GB_REASON_FP32_FAILED = GB300_REASON_FP32_FAILED,
       GB_REASON_SMALL_PIVOT = GB300_REASON_SMALL_PIVOT, GB_REASON_STALLED = GB300_REASON_STALLED };

/* Full (both triangles) compressed-row copy of the lower-stored A: row i of
 * the result is column i of the full symmetric matrix. */
static int upload_full_A(gb_plan *P, gb_ctx *ctx, cholmod_sparse *A, cholmod_common *Common)
{
    Int n = (Int)A->nrow;
    const Int *Ap = A->p, *Ai = A->i, *Anz = A->nz;
    const double *Ax = A->x;
    Int *cnt = calloc(n + 1, sizeof(Int));
    if (!cnt) { GB_ERROR(CHOLMOD_OUT_OF_MEMORY, "out of memory"); return FALSE; }
    Int nz = 0;
    for (Int j = 0; j < n; j++) {
        Int p = Ap[j], pend = A->packed ? Ap[j + 1] : p + Anz[j];
        for (; p < pend; p++) {
            Int i = Ai[p];
            if (i < j) continue;
            cnt[i]++;
            nz++;
            if (i != j) { cnt[j]++; nz++; }
        }
    }
    int64_t *Rp = malloc(sizeof(int64_t) * (n + 1));
    int32_t *Rj = malloc(sizeof(int32_t) * (nz + 1));
    double *Rx = malloc(sizeof(double) * (nz + 1));
    double *dorig = malloc(sizeof(double) * (n + 1));
    double *dperm = malloc(sizeof(double) * (n + 1));
    int ok = Rp && Rj && Rx && dorig && dperm;
    if (ok) {
        Rp[0] = 0;
        for (Int i = 0; i < n; i++) Rp[i + 1] = Rp[i] + cnt[i];
        for (Int i = 0; i < n; i++) { cnt[i] = Rp[i]; dorig[i] = 0; }
        double anorm = 0;
        for (Int j = 0; j < n; j++) {
            Int p = Ap[j], pend = A->packed ? Ap[j + 1] : p + Anz[j];
            for (; p < pend; p++) {
                Int i = Ai[p];
                if (i < j) continue;
                Rj[cnt[i]] = (int32_t)j;
                Rx[cnt[i]++] = Ax[p];
                if (i != j) {
                    Rj[cnt[j]] = (int32_t)i;
                    Rx[cnt[j]++] = Ax[p];
                } else {
                    dorig[i] = Ax[p];
                }
            }
        }
        (void)anorm;
        const Int *Perm = P->L->Perm;
        for (Int i = 0; i < n; i++) dorig[i] = dorig[i] > 0 ? 1.0 / sqrt(dorig[i]) : 1.0;
        for (Int k = 0; k < n; k++) dperm[k] = dorig[Perm[k]];
        cudaStream_t st = ctx->stream;
        ok = gb_dev_grow((void **)&P->d_Rp, &P->rp_cap, sizeof(int64_t) * (n + 1))
             && gb_dev_grow((void **)&P->d_Rj, &P->rj_cap, sizeof(int32_t) * (nz + 1))
             && gb_dev_grow((void **)&P->d_Rx, &P->rx_cap, sizeof(double) * (nz + 1));
        size_t cap = 0;
        if (ok && !P->d_scale) ok = gb_dev_grow((void **)&P->d_scale, &cap, sizeof(double) * (n + 1));
        cap = 0;
        if (ok && !P->d_scale_perm) ok = gb_dev_grow((void **)&P->d_scale_perm, &cap, sizeof(double) * (n + 1));
        if (ok && !P->d_red) { cap = 0; ok = gb_dev_grow((void **)&P->d_red, &cap, sizeof(double) * 64); }
        ok = ok && cudaMemcpyAsync(P->d_Rp, Rp, sizeof(int64_t) * (n + 1), cudaMemcpyHostToDevice, st) == cudaSuccess
             && cudaMemcpyAsync(P->d_Rj, Rj, sizeof(int32_t) * nz, cudaMemcpyHostToDevice, st) == cudaSuccess
             && cudaMemcpyAsync(P->d_Rx, Rx, sizeof(double) * nz, cudaMemcpyHostToDevice, st) == cudaSuccess
             && cudaMemcpyAsync(P->d_scale, dorig, sizeof(double) * n, cudaMemcpyHostToDevice, st) == cudaSuccess
             && cudaMemcpyAsync(P->d_scale_perm, dperm, sizeof(double) * n, cudaMemcpyHostToDevice, st) == cudaSuccess
             && gb_launch_anorm_seg(P->nchunk, P->d_chunk, P->nseg, P->d_Rp, P->d_Rx, P->d_anorm_seg, st) == 0
             && cudaMemcpyAsync(P->h_anorm_seg, P->d_anorm_seg, sizeof(double) * P->nseg,
                                cudaMemcpyDeviceToHost, st) == cudaSuccess
             && cudaStreamSynchronize(st) == cudaSuccess;
        P->anorm = 0;
        for (int64_t g = 0; ok && g < P->nseg; g++) P->anorm = fmax(P->anorm, P->h_anorm_seg[g]);
        if (!ok) GB_ERROR(CHOLMOD_GPU_PROBLEM, "CUDA error uploading A");
    } else {
        GB_ERROR(CHOLMOD_OUT_OF_MEMORY, "out of memory");
    }
    free(cnt); free(Rp); free(Rj); free(Rx); free(dorig); free(dperm);
    return ok;
}

static int factor_fp64(gb_plan *P, gb_ctx *ctx, int reason, cholmod_common *Common)
{
    if (!gb_ensure_numeric(P, CHOLMOD_DOUBLE)) {
        GB_ERROR(CHOLMOD_GPU_PROBLEM, "device allocation failed");
        return FALSE;
    }
    int32_t anyfail = 0;
    int32_t dagerr = 0;
    int ok = gb_run_factor(P, ctx, P->d_Sx, CHOLMOD_DOUBLE, CHOLMOD_DOUBLE, NULL, 0.0)
             && cudaMemcpyAsync(&anyfail, P->d_anyfail, sizeof(int32_t), cudaMemcpyDeviceToHost,
                                ctx->stream) == cudaSuccess
             && cudaMemcpyAsync(&dagerr, P->d_ticket + 3, sizeof(int32_t), cudaMemcpyDeviceToHost,
                                ctx->stream) == cudaSuccess
             && cudaStreamSynchronize(ctx->stream) == cudaSuccess && !dagerr;
    if (!ok) { GB_ERROR(CHOLMOD_GPU_PROBLEM, "CUDA error in the FP64 factorization"); return FALSE; }
    P->mixed = 2;
    P->mixed_reason = reason;
    P->dev_valid[0] = 0;                 /* not L->x's values */
    if (anyfail) {
        gb_fix_not_posdef(P, ctx, (cholmod_factor *)P->L, CHOLMOD_DOUBLE, Common);
        return TRUE;
    }
    return TRUE;
}

int gb300_factorize_mixed(cholmod_sparse *A, cholmod_factor *L, cholmod_common *Common)
{
    if (!Common) return FALSE;
    if (!A || !L) { GB_ERROR(CHOLMOD_INVALID, "argument missing"); return FALSE; }
    if (A->stype >= 0 || A->nrow != A->ncol || A->nrow != L->n || !L->Perm || !L->is_super
        || A->xtype != CHOLMOD_REAL || A->dtype != CHOLMOD_DOUBLE || A->itype != CHOLMOD_LONG) {
        GB_ERROR(CHOLMOD_INVALID, "A must be real double symmetric-lower matching supernodal L");
        return FALSE;
    }
    Common->status = CHOLMOD_OK;
    gb_ctx *ctx = gb_ctx_get(Common, 1);
    if (!ctx || !gb_ctx_ready(ctx)) { GB_ERROR(CHOLMOD_GPU_PROBLEM, "no CUDA device"); return FALSE; }
    gb_plan *P = gb_plan_get(L, Common, ctx, 1);
    if (!P) return FALSE;
    /* values of S = tril(PAP'), rows of A and the scaling: gathered on the
     * device through per-pattern maps, or formed on the host */
    int ok = TRUE;
    if (!P->d_red) {                     /* pivot check and reduction words */
        size_t cap = 0;
        ok = gb_dev_grow((void **)&P->d_red, &cap, sizeof(double) * 64);
    }
    if (!ok) {
        GB_ERROR(CHOLMOD_OUT_OF_MEMORY, "device allocation failed");
        return FALSE;
    }
    int deferred = 0, via_maps = 0;
    if (gb_valmap_apply(P, ctx, A, Common, &deferred)) {
        via_maps = 1;
        ok = gb_ensure_numeric(P, CHOLMOD_SINGLE);
    } else {
        cholmod_sparse *S = gb_permute_lower(A, L->Perm, Common);
        if (!S) return FALSE;
        ok = gb_upload_input(P, ctx, S, CHOLMOD_DOUBLE) && upload_full_A(P, ctx, A, Common)
             && gb_ensure_numeric(P, CHOLMOD_SINGLE);
        gb300_free_sparse(&S, Common);
    }
    if (!ok) {
        if (Common->status == CHOLMOD_OK) GB_ERROR(CHOLMOD_GPU_PROBLEM, "device allocation failed");
        return FALSE;
    }
    L->minor = L->n;
    int32_t anyfail = 0;
    double mm[2] = {0, 0};
    cudaStream_t st = ctx->stream;
    cudaEventRecord(ctx->ev0, st);
    ok = gb_run_factor(P, ctx, P->d_Sx, CHOLMOD_DOUBLE, CHOLMOD_SINGLE, P->d_scale_perm, 0.0)
         && gb_launch_diag_minmax((int)P->nsuper, P->d_Super, P->d_Pi, P->d_Px, P->d_Lx[1], 4,
                                  P->d_red, st) == 0;
    cudaEventRecord(ctx->ev1, st);
    /* A's pattern, compared while the device factorizes (the values went
     * through the maps of the pattern they were built for) */
    const int changed = ok && deferred && !gb_valmap_verify(P, A);
    int32_t dagerr = 0;
    ok = ok && cudaMemcpyAsync(&anyfail, P->d_anyfail, sizeof(int32_t), cudaMemcpyDeviceToHost, st) == cudaSuccess
         && cudaMemcpyAsync(mm, P->d_red, 2 * sizeof(double), cudaMemcpyDeviceToHost, st) == cudaSuccess
         && cudaMemcpyAsync(&dagerr, P->d_ticket + 3, sizeof(int32_t), cudaMemcpyDeviceToHost, st) == cudaSuccess
         && cudaStreamSynchronize(st) == cudaSuccess && !dagerr;
    if (!ok) { GB_ERROR(CHOLMOD_GPU_PROBLEM, "CUDA error in the FP32 factorization"); return FALSE; }
    if (changed) {
        /* the pattern differs from the maps': rebuild them and factorize
         * again (the comparison is not deferred the second time) */
        P->vm_valid = 0;
        return gb300_factorize_mixed(A, L, Common);
    }
    if (via_maps) gb_valmap_anorm(P);
    float ms = 0;
    cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1);
    ctx->stats[0] = ms;
    P->mixed = 1;
    P->mixed_reason = GB_REASON_NONE;
    P->dev_valid[1] = 0;                 /* the FP32 factor is of D A D, not of L->x */
    if (anyfail) return factor_fp64(P, ctx, GB_REASON_FP32_FAILED, Common);
    /* small pivot: min L(k,k)^2 <= 2^-pivot_log2 max L(k,k)^2 (by default
     * 2^-23, the single-precision epsilon) */
    if (mm[0] <= ldexp(mm[1], -ctx->pivot_log2)) return factor_fp64(P, ctx, GB_REASON_SMALL_PIVOT, Common);
    return TRUE;
}

/* The device work of one refinement step on the context's stream: the
 * correction x += D P' L^-T L^-1 P D r, the residual r = b - A x, and the
 * per-segment, per-column backward-error terms in d_bred. */
static int refine_step_launch(gb_plan *P, gb_ctx *ctx, int nrhs, int single)
{
    cudaStream_t st = ctx->stream;
    const Int n = P->n;
    const int ydt = single ? 4 : 0;
    const double *scale = single ? P->d_scale : NULL;
    /* a batch: the segments (independent systems) already at the tolerance
     * (P->d_segact 0) get a zero correction, and the single-launch sweeps
     * skip their tasks */
    const int mask = P->d_segact != NULL;
    int ok = !mask || gb_launch_zero_inactive(P->nchunk, P->d_chunk, P->d_segact, P->d_R, n, nrhs,
                                              st) == 0;
    P->sweep_act = mask ? P->d_segact : NULL;
    ok = ok && gb_launch_perm_in(n, nrhs, P->d_Perm, scale, P->d_R, 0, n, P->d_Y, ydt, n, st) == 0
         && gb_run_sweep(P, ctx, single ? CHOLMOD_SINGLE : CHOLMOD_DOUBLE, nrhs, P->d_Y, 1)
         && gb_run_sweep(P, ctx, single ? CHOLMOD_SINGLE : CHOLMOD_DOUBLE, nrhs, P->d_Y, 0);
    P->sweep_act = NULL;
    return ok && gb_launch_perm_out(n, nrhs, P->d_Perm, scale, P->d_Y, ydt, n, P->d_X, 0, n, 1, st) == 0
           && gb_launch_residual(n, nrhs, P->d_Rp, P->d_Rj, P->d_Rx, P->d_X, n, P->d_bx, n,
                                 P->d_R, n, st) == 0
           && gb_launch_colmax3_seg(P->nchunk, P->d_chunk, P->nseg, nrhs, P->d_R, n, P->d_X, n,
                                    P->d_bx, n, P->d_bred, st) == 0;
}

/* every segment to be refined (the first step, and after an FP64 refactor) */
static int segact_all(gb_plan *P, cudaStream_t st)
{
    if (!P->d_segact) return TRUE;
    memset(P->h_segact, 1, (size_t)P->nseg);
    return cudaMemcpyAsync(P->d_segact, P->h_segact, (size_t)P->nseg, cudaMemcpyHostToDevice, st)
           == cudaSuccess;
}

void gb_graph_free(gb_plan *P)
{
    if (P->g_exec) cudaGraphExecDestroy((cudaGraphExec_t)P->g_exec);
    P->g_exec = NULL;
}

/* the buffers a captured step reads and writes (a reallocation of any of
 * them invalidates the graph) */
static void graph_bufs(gb_plan *P, int single, const void **b)
{
    b[0] = P->d_Y; b[1] = P->d_R; b[2] = P->d_X; b[3] = P->d_bx; b[4] = P->d_bred;
    b[5] = P->d_U; b[6] = P->d_Lx[single ? 1 : 0]; b[7] = P->d_Linv[single ? 1 : 0];
    b[8] = P->d_sws;
}

/* One refinement step: from the plan's CUDA graph when it matches, else
 * captured into one (when allowed) and replayed, else launched directly. */
static int refine_step(gb_plan *P, gb_ctx *ctx, int nrhs, int single, int may_capture)
{
    cudaStream_t st = ctx->stream;
    if (!ctx->graph_mode || ctx->sweep_mode != 1 || ctx->trace_on)
        return refine_step_launch(P, ctx, nrhs, single);
    const void *b[9];
    graph_bufs(P, single, b);
    int match = P->g_exec && P->g_nrhs == nrhs && P->g_single == single
                && memcmp(b, P->g_bufs, sizeof b) == 0;
    if (!match) {
        if (!may_capture) return refine_step_launch(P, ctx, nrhs, single);
        gb_graph_free(P);
        cudaGraph_t g = NULL;
        cudaGraphExec_t ge = NULL;
        const int64_t l0 = ctx->launches;
        int ok = cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal) == cudaSuccess;
        if (ok) {
            int launched = refine_step_launch(P, ctx, nrhs, single);
            ok = cudaStreamEndCapture(st, &g) == cudaSuccess && launched && g
                 && cudaGraphInstantiate(&ge, g, 0) == cudaSuccess;
        }
        if (g) cudaGraphDestroy(g);
        if (!ok) {
            /* capture refused: clear the error, launch directly */
            if (ge) cudaGraphExecDestroy(ge);
            cudaGetLastError();
            return refine_step_launch(P, ctx, nrhs, single);
        }
        P->g_exec = ge;
        P->g_launches = ctx->launches - l0;
        ctx->launches = l0;
        P->g_nrhs = nrhs;
        P->g_single = single;
        memcpy(P->g_bufs, b, sizeof b);
    }
    ctx->launches += P->g_launches;
    return cudaGraphLaunch((cudaGraphExec_t)P->g_exec, st) == cudaSuccess;
}

/* The refined solve into X: a caller's X of the right shape (n x nrhs,
 * real double, d >= n) is written in place, else a new one is allocated;
 * on failure an X allocated here is freed and NULL returned. */
static cholmod_dense *solve_refined_into(cholmod_sparse *A, cholmod_factor *L, cholmod_dense *B,
                                         double tol, double *info, cholmod_dense *Xin,
                                         cholmod_common *Common)
{
    if (!Common) return NULL;
    if (!A || !L || !B) { GB_ERROR(CHOLMOD_INVALID, "argument missing"); return NULL; }
    if (B->nrow != L->n || B->xtype != CHOLMOD_REAL || B->dtype != CHOLMOD_DOUBLE
        || A->nrow != L->n) {
        GB_ERROR(CHOLMOD_INVALID, "B must be real double with n rows");
        return NULL;
    }
    Common->status = CHOLMOD_OK;
    gb_ctx *ctx = gb_ctx_get(Common, 1);
    if (!ctx || !gb_ctx_ready(ctx)) { GB_ERROR(CHOLMOD_GPU_PROBLEM, "no CUDA device"); return NULL; }
    gb_plan *P = gb_plan_get(L, Common, ctx, 0);
    if (!P || !P->mixed) {
        GB_ERROR(CHOLMOD_INVALID, "no mixed-precision factor: call gb300_factorize_mixed first");
        return NULL;
    }
    Int n = P->n;
    int nrhs = (int)B->ncol;
    cholmod_dense *X = Xin;
    if (!X) X = gb300_allocate_dense(n, nrhs, n, CHOLMOD_REAL + CHOLMOD_DOUBLE, Common);
    if (!X) return NULL;
    if (info) { info[0] = 0; info[1] = 0; info[2] = P->mixed == 2; info[3] = 0; }
    if (n == 0 || nrhs == 0) return X;
    cudaStream_t st = ctx->stream;
    size_t nb = sizeof(double) * n * nrhs;
    /* backward error per independent block (segment) and column */
    const int64_t nsg = P->nseg, nred = 3 * nsg * nrhs;
    double *hred = malloc(sizeof(double) * nred);
    double *best = malloc(sizeof(double) * nsg * nrhs);
    int ok = hred && best && gb_dev_grow((void **)&P->d_X, &P->x_cap, nb)
             && gb_dev_grow((void **)&P->d_R, &P->r_cap, nb)
             && gb_dev_grow((void **)&P->d_bx, &P->bx_cap, nb)
             && gb_dev_grow(&P->d_Y, &P->y_cap, nb)
             && gb_dev_grow((void **)&P->d_bred, &P->bred_cap, sizeof(double) * nred);
    ok = ok && cudaMemcpy2DAsync(P->d_bx, sizeof(double) * n, B->x, sizeof(double) * B->d,
                                 sizeof(double) * n, nrhs, cudaMemcpyHostToDevice, st) == cudaSuccess
         && cudaMemsetAsync(P->d_X, 0, nb, st) == cudaSuccess
         && cudaMemcpyAsync(P->d_R, P->d_bx, nb, cudaMemcpyDeviceToDevice, st) == cudaSuccess
         && segact_all(P, st);
    cudaEventRecord(ctx->ev0, st);
    int it = 0, stall = 0;
    int32_t serr = 0;
    double bmax_all = 0, berr_max = INFINITY;
    for (int64_t r = 0; r < nsg * nrhs && best; r++) best[r] = INFINITY;
    while (ok && it < GB_MAX_REFINE) {
        /* correction with the current factor, residual, backward-error
         * terms: the first step of a solve whose buffers are new runs
         * directly (buffers, inverses and launch settings exist after it),
         * later ones may be captured into the pattern's graph */
        int single = (P->mixed == 1);
        ok = refine_step(P, ctx, nrhs, single, it > 0 || P->g_exec != NULL)
             && cudaMemcpyAsync(hred, P->d_bred, sizeof(double) * nred, cudaMemcpyDeviceToHost, st) == cudaSuccess
             && cudaMemcpyAsync(&serr, P->d_err, sizeof(int32_t), cudaMemcpyDeviceToHost, st) == cudaSuccess
             && cudaStreamSynchronize(st) == cudaSuccess && !(ctx->sweep_mode == 1 && serr);
        ctx->launches += 5;
        if (!ok) break;
        it++;
        berr_max = 0;
        int improved = 0, b_bad = 0;
        if (P->h_segact) memset(P->h_segact, 0, (size_t)nsg);
        for (int64_t q = 0; q < nsg * nrhs; q++) {
            const double *h = hred + 3 * q;
            const double an = P->h_anorm_seg[q / nrhs];
            double den = an * h[1] + h[2];
            /* a NaN or infinity in r, x, b or A (the device maxima keep
             * NaN) makes the column's backward error NaN: not converged */
            double be = (isfinite(h[0]) && isfinite(h[1]) && isfinite(h[2]) && isfinite(an)
                         && isfinite(den)) ? (den > 0 ? h[0] / den : 0) : NAN;
            if (be < best[q]) { if (be < 0.5 * best[q]) improved = 1; best[q] = be; }
            if (!(be <= berr_max)) berr_max = be;       /* keeps NaN */
            if (P->h_segact && !(be <= tol)) P->h_segact[q / nrhs] = 1;
            if (!isfinite(h[2])) b_bad = 1;
            bmax_all = fmax(bmax_all, h[2]);
        }
        if (berr_max <= tol) break;
        /* a right-hand side that is not finite cannot be refined by any
         * factor: stop with its NaN backward error */
        if (b_bad) break;
        stall = improved ? 0 : stall + 1;
        if (stall >= 2) {
            if (P->mixed == 2) break;           /* FP64 factor cannot do better */
            ok = factor_fp64(P, ctx, GB_REASON_STALLED, Common) && segact_all(P, st);
            stall = 0;
            if (info) info[2] = 1;
        } else if (P->d_segact) {
            /* the next step refines only the segments above the tolerance */
            ok = cudaMemcpyAsync(P->d_segact, P->h_segact, (size_t)nsg, cudaMemcpyHostToDevice, st)
                 == cudaSuccess;
        }
    }
    cudaEventRecord(ctx->ev1, st);
    ok = ok && cudaMemcpy2DAsync(X->x, sizeof(double) * X->d, P->d_X, sizeof(double) * n,
                                 sizeof(double) * n, nrhs, cudaMemcpyDeviceToHost, st) == cudaSuccess
         && cudaStreamSynchronize(st) == cudaSuccess;
    free(hred);
    free(best);
    if (!ok) {
        if (X != Xin) gb300_free_dense(&X, Common);
        if (Common->status == CHOLMOD_OK) GB_ERROR(CHOLMOD_GPU_PROBLEM, "CUDA error in refinement");
        return NULL;
    }
    float ms = 0;
    cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1);
    ctx->stats[2] = ms;
    if (info) { info[0] = it; info[1] = berr_max; info[3] = berr_max; info[2] = P->mixed == 2; }
    if (!(berr_max <= tol))              /* NaN included */
        GB_ERROR(CHOLMOD_DSMALL, "refinement did not reach the requested tolerance");
    return X;
}

int gb300_mixed_reason(cholmod_factor *L, cholmod_common *Common)
{
    if (!Common || !L) return -1;
    gb_ctx *ctx = gb_ctx_get(Common, 0);
    if (!ctx) return -1;
    gb_plan *P = gb_plan_get(L, Common, ctx, 0);
    if (!P || !P->mixed) return -1;
    return P->mixed == 1 ? GB_REASON_NONE : P->mixed_reason;
}

cholmod_dense *gb300_solve_refined(cholmod_sparse *A, cholmod_factor *L, cholmod_dense *B,
                                   double tol, double *info, cholmod_common *Common)
{
    return solve_refined_into(A, L, B, tol, info, NULL, Common);
}

int gb300_solve_refined2(cholmod_sparse *A, cholmod_factor *L, cholmod_dense *B, double tol,
                         double *info, cholmod_dense **X_Handle, cholmod_common *Common)
{
    if (!Common) return FALSE;
    if (!X_Handle) { GB_ERROR(CHOLMOD_INVALID, "argument missing"); return FALSE; }
    cholmod_dense *X = *X_Handle;
    if (X && B && L
        && !(X->nrow == L->n && X->ncol == B->ncol && X->d >= X->nrow && X->xtype == CHOLMOD_REAL
             && X->dtype == CHOLMOD_DOUBLE && X->x)) {
        gb300_free_dense(X_Handle, Common);          /* wrong shape: replaced */
        X = NULL;
    }
    cholmod_dense *R = solve_refined_into(A, L, B, tol, info, X, Common);
    if (!R) return FALSE;
    *X_Handle = R;
    return TRUE;
}
