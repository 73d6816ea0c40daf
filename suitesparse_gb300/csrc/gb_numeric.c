/* gb_numeric.c -- host drivers of the GPU factorization and sweeps, and the
 * CHOLMOD entry points cholmod_l_super_numeric / _lsolve / _ltsolve.
 *
 * Device state is attached to a factor through a side table keyed by the
 * cholmod_factor pointer and validated by a fingerprint of its supernodal
 * pattern (cholmod_factor is ABI and cannot grow).  The plan of a pattern
 * (gb_plan.c) is built and uploaded once; every factorization then uploads
 * only the values of A, replays the level sequence on one stream, checks one
 * word for a failed pivot, and copies L->x back unless the caller keeps the
 * factor on the device.  There is no CPU fallback: any CUDA failure returns
 * FALSE with Common->status = CHOLMOD_GPU_PROBLEM.
 */
#include "gb_plan.h"
#include <cuda_runtime.h>
#include <math.h>
#include <pthread.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

gb_ctx *gb_ctx_new(void)
{
    gb_ctx *c = calloc(1, sizeof(gb_ctx));
    if (!c) return NULL;
    c->opt_keep = 0;
    c->opt_small = GB_SMALL_MAX;
    c->opt_subwork = GB_SUBTREE_WORK;
    c->opt_warprows = GB_WARP_ROWS;
    c->opt_updgroup = GB_UPD_GROUP;
    c->device = -1;
    c->sweep_mode = 1;
    c->factor_mode = 1;
    c->tc_mode = 1;
    c->pivot_log2 = 23;
    c->graph_mode = 1;
    c->sweep_streams = 2;
    return c;
}

void gb_ctx_delete(gb_ctx *c)
{
    if (!c) return;
    if (c->stream) cudaStreamDestroy(c->stream);
    if (c->ev0) cudaEventDestroy(c->ev0);
    if (c->ev1) cudaEventDestroy(c->ev1);
    for (int i = 0; i < c->npev; i++) cudaEventDestroy(c->pev[i]);
    for (int i = 0; i < GB_SWEEP_STREAMS - 1; i++) {
        if (c->side[i]) cudaStreamDestroy(c->side[i]);
        if (c->ev_join[i]) cudaEventDestroy(c->ev_join[i]);
    }
    if (c->ev_fork) cudaEventDestroy(c->ev_fork);
    for (int d = 0; d < 2; d++)
        if (c->d_cbs[d]) cudaFree(c->d_cbs[d]);
    if (c->d_imgs) cudaFree(c->d_imgs);
    if (c->d_trace) cudaFree(c->d_trace);
    if (c->d_ftrace) cudaFree(c->d_ftrace);
    free(c->pev);
    free(c);
}

int gb_ctx_ready(gb_ctx *c)
{
    if (c->stream) return TRUE;
    if (cudaGetDevice(&c->device) != cudaSuccess) return FALSE;
    if (cudaDeviceGetAttribute(&c->sms, cudaDevAttrMultiProcessorCount, c->device) != cudaSuccess)
        return FALSE;
    if (cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess) return FALSE;
    if (cudaEventCreate(&c->ev0) != cudaSuccess) return FALSE;
    if (cudaEventCreate(&c->ev1) != cudaSuccess) return FALSE;
    return TRUE;
}

int64_t gb_option(cholmod_common *Common, int option)
{
    gb_ctx *c = gb_ctx_get(Common, 0);
    if (option == GB300_OPT_KEEP_ON_DEVICE) return c ? c->opt_keep : 0;
    if (option == GB300_OPT_SMALL_COLS) return c ? c->opt_small : GB_SMALL_MAX;
    if (option == GB300_OPT_SUBTREE_WORK) return c ? (int64_t)c->opt_subwork : (int64_t)GB_SUBTREE_WORK;
    if (option == GB300_OPT_WARP_ROWS) return c ? c->opt_warprows : GB_WARP_ROWS;
    if (option == GB300_OPT_UPD_GROUP) return c ? c->opt_updgroup : GB_UPD_GROUP;
    if (option == GB300_OPT_AUTOTUNE) return c ? c->opt_autotune : 0;
    return 0;
}

int gb300_set_option(cholmod_common *Common, int option, int64_t value)
{
    if (!Common) return FALSE;
    gb_ctx *c = gb_ctx_get(Common, 1);
    if (!c) { GB_ERROR(CHOLMOD_OUT_OF_MEMORY, "out of memory"); return FALSE; }
    if (option == GB300_OPT_KEEP_ON_DEVICE) c->opt_keep = value ? 1 : 0;
    else if (option == GB300_OPT_SWEEP) c->sweep_mode = value ? 1 : 0;
    else if (option == GB300_OPT_FACTOR) c->factor_mode = value ? 1 : 0;
    else if (option == GB300_OPT_TENSOR) c->tc_mode = value ? 1 : 0;
    else if (option == GB300_OPT_GRAPH) c->graph_mode = value ? 1 : 0;
    else if (option == GB300_OPT_PIVOT_LOG2) c->pivot_log2 = (int)GB_MAX(0, GB_MIN(60, value));
    else if (option == GB300_OPT_SWEEP_STREAMS)
        c->sweep_streams = (int)GB_MAX(1, GB_MIN(GB_SWEEP_STREAMS, value));
    else if (option == GB300_OPT_TRACE) c->trace_on = value ? 1 : 0;
    else if (option == GB300_OPT_PROFILE) {
        c->prof = value ? 1 : 0;
        for (int k = 0; k < 16; k++) c->kind_ms[k] = c->kind_n[k] = 0;
    }
    else if (option == GB300_OPT_SMALL_COLS) c->opt_small = GB_MAX(1, GB_MIN(GB_SMALL_MAX, value));
    else if (option == GB300_OPT_SUBTREE_WORK) c->opt_subwork = value < 0 ? 0.0 : (double)value;
    else if (option == GB300_OPT_WARP_ROWS) c->opt_warprows = GB_MAX(0, GB_MIN(GB_WARP_ROWS, value));
    else if (option == GB300_OPT_UPD_GROUP) c->opt_updgroup = GB_MAX(1, GB_MIN(GB_UPD_GROUP, value));
    else if (option == GB300_OPT_AUTOTUNE) { c->opt_autotune = value ? 1 : 0; c->tuned = 0; }
    else { GB_ERROR(CHOLMOD_INVALID, "unknown option"); return FALSE; }
    return TRUE;
}

int gb300_get_stats(cholmod_common *Common, double *out, int nout)
{
    gb_ctx *c = gb_ctx_get(Common, 0);
    if (!c || !out) return FALSE;
    for (int i = 0; i < nout && i < 8; i++) out[i] = c->stats[i];
    if (nout > 5) out[5] = (double)c->launches;
    return TRUE;
}

int gb300_get_profile(cholmod_common *Common, double *ms, double *count, int nkinds)
{
    gb_ctx *c = gb_ctx_get(Common, 0);
    if (!c) return FALSE;
    for (int k = 0; k < nkinds && k < 16; k++) {
        if (ms) ms[k] = c->kind_ms[k];
        if (count) count[k] = c->kind_n[k];
    }
    return TRUE;
}

int gb300_get_trace(cholmod_common *Common, int forward, unsigned long long *out, int64_t nmax)
{
    gb_ctx *c = gb_ctx_get(Common, 0);
    if (!c || !c->d_trace || !out) return -1;
    int64_t nt = c->trace_n[forward ? 0 : 1];
    if (nt > nmax) nt = nmax;
    if (cudaMemcpy(out, c->d_trace + c->trace_off[forward ? 0 : 1],
                   3 * nt * sizeof(unsigned long long), cudaMemcpyDeviceToHost) != cudaSuccess)
        return -1;
    return (int)nt;
}

int gb300_get_factor_trace(cholmod_common *Common, unsigned long long *out, int64_t nmax)
{
    gb_ctx *c = gb_ctx_get(Common, 0);
    if (!c || !c->d_ftrace || !out) return -1;
    int64_t nt = c->ftrace_n < nmax ? c->ftrace_n : nmax;
    if (cudaMemcpy(out, c->d_ftrace, 3 * nt * sizeof(unsigned long long),
                   cudaMemcpyDeviceToHost) != cudaSuccess)
        return -1;
    return (int)nt;
}

int gb300_fma_peak(int dtype, double *tflops)
{
    cudaStream_t st;
    if (!tflops || cudaStreamCreate(&st) != cudaSuccess) return FALSE;
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const int iters = dtype == 4 ? 4096 : 512, blocks = sms * 8;
    float ms = 0;
    int ok = gb_launch_fma_peak(dtype, iters, blocks, &ms, st) == 0      /* warm-up */
             && gb_launch_fma_peak(dtype, iters, blocks, &ms, st) == 0;
    cudaStreamDestroy(st);
    if (!ok || ms <= 0) return FALSE;
    /* 256 threads x 8 chains x iters x 2 flops per block */
    *tflops = 2.0 * 8.0 * iters * 256.0 * blocks / (ms * 1e-3) / 1e12;
    return TRUE;
}

/* ---- factor side table --------------------------------------------------- */

static gb_plan *plan_head = NULL;
static pthread_mutex_t plan_lock = PTHREAD_MUTEX_INITIALIZER;

static int plan_matches(const gb_plan *P, const cholmod_factor *L)
{
    return P->L == L && P->super_ptr == L->super && P->s_ptr == L->s && P->pi_ptr == L->pi
           && P->n == (Int)L->n && P->nsuper == (Int)L->nsuper
           && P->ssize == (Int)L->ssize && P->xsize == (Int)L->xsize;
}

static void plan_unlink(gb_plan *P)
{
    for (gb_plan **pp = &plan_head; *pp; pp = &(*pp)->next)
        if (*pp == P) { *pp = P->next; break; }
}

int gb_release_factor_state(cholmod_factor *L)
{
    gb_release_complex_shadow(L);
    pthread_mutex_lock(&plan_lock);
    gb_plan *found = NULL;
    for (gb_plan *P = plan_head; P; P = P->next)
        if (P->L == L) { found = P; break; }
    if (found) plan_unlink(found);
    pthread_mutex_unlock(&plan_lock);
    if (found) {
        cudaDeviceSynchronize();
        gb_plan_free(found);
    }
    return TRUE;
}

int gb300_factor_info(cholmod_factor *L, cholmod_common *Common, double *out, int nout)
{
    if (!Common || !L || !out) return FALSE;
    gb_ctx *ctx = gb_ctx_get(Common, 1);
    if (!ctx || !gb_ctx_ready(ctx)) { GB_ERROR(CHOLMOD_GPU_PROBLEM, "no CUDA device"); return FALSE; }
    gb_plan *P = gb_plan_get(L, Common, ctx, 1);
    if (!P) return FALSE;
    double v[10] = {P->fl_dag, (double)P->nlevels, (double)P->fact_seq.n, (double)P->cb_total,
                    (double)P->gemm_t.n, (double)P->nsuper, (double)P->fwd_seq.n,
                    (double)P->bwd_seq.n, (double)P->cbv_total, (double)P->mixed};
    for (int i = 0; i < nout && i < 10; i++) out[i] = v[i];
    return TRUE;
}

int gb300_release_factor(cholmod_factor *L, cholmod_common *Common)
{
    (void)Common;
    if (!L) return FALSE;
    if (L->itype == CHOLMOD_INT) return gb_release_int32_shadow(L);
    if (!L->is_super) return gb_release_simplicial_shadow(L);
    return gb_release_factor_state(L);
}

/* Find (or build and upload) the plan of L.  A stale entry for the same
 * pointer with a different pattern is dropped. */
gb_plan *gb_plan_get(cholmod_factor *L, cholmod_common *Common, gb_ctx *ctx, int create)
{
    pthread_mutex_lock(&plan_lock);
    gb_plan *P = NULL;
    for (gb_plan *q = plan_head; q; q = q->next)
        if (q->L == L) { P = q; break; }
    if (P && (!plan_matches(P, L) || P->hash != gb_pattern_hash(L)
              || (create && (P->small_cols != ctx->opt_small || P->sub_work != ctx->opt_subwork
                             || P->warp_rows != ctx->opt_warprows
                             || P->upd_group != ctx->opt_updgroup)))) {
        plan_unlink(P);
        pthread_mutex_unlock(&plan_lock);
        cudaStreamSynchronize(ctx->stream);
        gb_plan_free(P);
        pthread_mutex_lock(&plan_lock);
        P = NULL;
    }
    pthread_mutex_unlock(&plan_lock);
    if (P || !create) return P;
    P = gb_plan_build(L, ctx->opt_small, ctx->opt_subwork, ctx->opt_warprows, ctx->opt_updgroup);
    if (!P) { GB_ERROR(CHOLMOD_OUT_OF_MEMORY, "plan construction failed"); return NULL; }
    if (!gb_plan_upload(P)) {
        gb_plan_free(P);
        GB_ERROR(CHOLMOD_GPU_PROBLEM, "device allocation of the plan failed");
        return NULL;
    }
    pthread_mutex_lock(&plan_lock);
    P->next = plan_head;
    plan_head = P;
    pthread_mutex_unlock(&plan_lock);
    return P;
}

int gb_dev_grow(void **p, size_t *cap, size_t bytes)
{
    if (bytes <= *cap && *p) return TRUE;
    if (*p) cudaFree(*p);
    *p = NULL;
    *cap = 0;
    if (cudaMalloc(p, bytes ? bytes : 16) != cudaSuccess) { *p = NULL; return FALSE; }
    *cap = bytes;
    return TRUE;
}

static int dt_index(int dtype) { return dtype == CHOLMOD_SINGLE ? 1 : 0; }
static size_t dt_size(int dtype) { return dtype == CHOLMOD_SINGLE ? sizeof(float) : sizeof(double); }

/* the device factor of one precision */
int gb_ensure_numeric(gb_plan *P, int dtype)
{
    int d = dt_index(dtype);
    size_t e = dt_size(dtype);
    if (!P->d_Lx[d] && cudaMalloc(&P->d_Lx[d], e * GB_MAX(P->xsize, 1)) != cudaSuccess) {
        P->d_Lx[d] = NULL;
        return FALSE;
    }
    return TRUE;
}

/* device bytes held by a plan: its structures, factors, update blocks,
 * inverses, operand images, value maps and the grown work buffers */
size_t gb_plan_device_bytes(const gb_plan *P)
{
    size_t b = P->struct_bytes + P->vm_bytes;
    for (int d = 0; d < 2; d++) {
        const size_t e = d ? sizeof(float) : sizeof(double);
        if (P->d_Lx[d]) b += e * (size_t)GB_MAX(P->xsize, 1);
        if (P->d_Linv[d]) b += e * (size_t)GB_MAX(P->linv_total, 1);
    }
    b += P->sx_cap + P->si_cap + P->sp_cap + P->y_cap + P->u_cap + P->b_cap + P->spw_cap
         + P->sws_cap + P->ax_cap + P->rp_cap + P->rj_cap + P->rx_cap + P->x_cap + P->r_cap
         + P->bx_cap + P->bred_cap;
    if (P->d_scale) b += sizeof(double) * (size_t)(P->n + 1);
    if (P->d_scale_perm) b += sizeof(double) * (size_t)(P->n + 1);
    return b;
}

int64_t gb300_factor_device_bytes(cholmod_factor *L, cholmod_common *Common)
{
    if (!Common || !L) return -1;
    gb_ctx *ctx = gb_ctx_get(Common, 0);
    gb_plan *P = ctx ? gb_plan_get(L, Common, ctx, 0) : NULL;
    return P ? (int64_t)gb_plan_device_bytes(P) : 0;
}

int64_t gb300_trim_factor(cholmod_factor *L, cholmod_common *Common)
{
    if (!Common || !L) return -1;
    gb_ctx *ctx = gb_ctx_get(Common, 0);
    gb_plan *P = ctx ? gb_plan_get(L, Common, ctx, 0) : NULL;
    if (!P) return 0;
    if (cudaStreamSynchronize(ctx->stream) != cudaSuccess) {
        GB_ERROR(CHOLMOD_GPU_PROBLEM, "CUDA error");
        return -1;
    }
    const size_t before = gb_plan_device_bytes(P);
    /* the precision the refined solves do not use */
    const int unused = P->mixed == 1 ? 0 : (P->mixed == 2 ? 1 : -1);
    if (unused >= 0 && (P->d_Lx[unused] || P->d_Linv[unused])) {
        /* a captured refinement step may name these buffers: capture again */
        gb_graph_free(P);
        if (P->d_Lx[unused]) cudaFree(P->d_Lx[unused]);
        if (P->d_Linv[unused]) cudaFree(P->d_Linv[unused]);
        P->d_Lx[unused] = P->d_Linv[unused] = NULL;
        P->dev_valid[unused] = 0;
        P->linv_valid[unused] = 0;
    }
    return (int64_t)(before - gb_plan_device_bytes(P));
}

#define CU(call) do { if ((call) != cudaSuccess) goto cuda_fail; } while (0)
#define LK(call) do { if ((call) != 0) goto cuda_fail; } while (0)

/* Replay the factorization sequence.  Sx has dtype a_dtype; the factor is
 * computed in l_dtype; scale (device, optional) applies D A D. */
int gb_run_factor(gb_plan *P, gb_ctx *ctx, const void *Sx, int a_dtype, int l_dtype,
                  const double *scale, double beta)
{
    cudaStream_t st = ctx->stream;
    int d = dt_index(l_dtype);
    int ldt = l_dtype == CHOLMOD_SINGLE ? 4 : 0;
    int adt = a_dtype == CHOLMOD_SINGLE ? 4 : 0;
    if (!gb_dev_grow(&ctx->d_cbs[d], &ctx->cbs_cap[d], dt_size(l_dtype) * GB_MAX(P->cb_total, 1)))
        return FALSE;
    void *Lx = P->d_Lx[d], *CB = ctx->d_cbs[d];
    const gb_launch_rec *seq = P->fact_seq.p;
    int launches = 0;
    if (!P->d_Linv[d] && cudaMalloc(&P->d_Linv[d], dt_size(l_dtype) * GB_MAX(P->linv_total, 1))
                             != cudaSuccess) {
        P->d_Linv[d] = NULL;
        return FALSE;
    }
    void *Linv = P->d_Linv[d];
    int prof = ctx->prof;
    if (prof && ctx->npev < (int)(2 * P->fact_seq.n)) {
        int need = (int)(2 * P->fact_seq.n);
        cudaEvent_t *ev = realloc(ctx->pev, sizeof(cudaEvent_t) * need);
        if (!ev) prof = 0;
        else {
            ctx->pev = ev;
            for (int i = ctx->npev; i < need; i++) CU(cudaEventCreate(&ctx->pev[i]));
            ctx->npev = need;
        }
    }
    CU(cudaMemsetAsync(P->d_fail, 0xFF, sizeof(int32_t) * (P->nsuper + 1), st));
    CU(cudaMemsetAsync(P->d_anyfail, 0, sizeof(int32_t), st));
    CU(cudaMemsetAsync(P->d_ticket + 3, 0, sizeof(int32_t), st));
    if (ctx->factor_mode == 1) {
        /* one persistent launch over the whole-factorization task graph */
        size_t N = P->fd_t.n, n0 = P->fd_q0.n, n1 = P->fd_q1.n;
        gb_fpat *hp = &P->h_fd_pat;
        hp->pp = P->ptrs;
        hp->tasks = P->d_fd_t;
        hp->succ_ptr = P->d_fd_sp;
        hp->succ = P->d_fd_succ;
        hp->Sp = P->d_Sp;
        hp->Si = P->d_Si;
        hp->sub_list = P->d_fd_sub;
        hp->sub_meta = P->d_fd_smeta;
        hp->warp_rows = (int32_t)P->warp_rows;
        hp->ntasks = (int32_t)N;
        if (prof) CU(cudaEventRecord(ctx->pev[0], st));
        CU(cudaMemcpyAsync(P->d_fd_pat, hp, sizeof *hp, cudaMemcpyHostToDevice, st));
        CU(cudaMemcpyAsync(P->d_fd_cnt, P->d_fd_nd, sizeof(int32_t) * N, cudaMemcpyDeviceToDevice, st));
        CU(cudaMemsetAsync(P->d_fd_q, 0xFF, sizeof(int32_t) * 2 * N, st));
        if (n0) CU(cudaMemcpyAsync(P->d_fd_q, P->d_fd_qi, sizeof(int32_t) * n0, cudaMemcpyDeviceToDevice, st));
        if (n1) CU(cudaMemcpyAsync(P->d_fd_q + N, P->d_fd_qi + n0, sizeof(int32_t) * n1, cudaMemcpyDeviceToDevice, st));
        CU(cudaMemcpyAsync(P->d_dag_ctrl, P->d_fd_ctrl0, sizeof(int32_t) * GB_DAG_NCTRL, cudaMemcpyDeviceToDevice, st));
        gb_fdag_args a;
        memset(&a, 0, sizeof a);
        a.pats = P->d_fd_pat;
        a.inst = P->d_fd_inst;
        a.inst_base = P->d_fd_ibase;
        a.ninst = 1;
        a.ntotal = (int64_t)N;
        a.cnt = P->d_fd_cnt;
        a.q0 = P->d_fd_q;
        a.q1 = P->d_fd_q + N;
        a.ctrl = P->d_dag_ctrl;
        a.err = P->d_ticket + 3;
        a.smflag = P->d_dag_smf;
        if (++P->dag_epoch <= 0) P->dag_epoch = 1;
        a.epoch = P->dag_epoch;
        a.Sx = Sx;
        a.a_dtype = adt;
        a.scale = scale;
        a.beta = beta;
        a.use_tc = ctx->tc_mode && l_dtype == CHOLMOD_SINGLE && P->img_total > 0;
        if (a.use_tc && !gb_dev_grow(&ctx->d_imgs, &ctx->imgs_cap,
                                     sizeof(float) * GB_IMG_FLOATS_HOST * (size_t)P->img_total)) {
            /* no room for the operand images: the CUDA cores take the tiles */
            cudaGetLastError();
            a.use_tc = 0;
        }
        a.img = a.use_tc ? (float *)ctx->d_imgs : NULL;
        a.npoll = P->fd_spread ? 0 : GB_DAG_POLLERS;
        if (ctx->trace_on) {
            size_t need = 3 * (N + 1) * sizeof(unsigned long long);
            if (gb_dev_grow((void **)&ctx->d_ftrace, &ctx->ftrace_cap, need)) {
                a.trace = ctx->d_ftrace;
                ctx->ftrace_n = (int64_t)N;
            }
        }
        int grid = GB_MAX(1, ctx->sms) * 2;   /* resident blocks per SM */
        LK(gb_launch_fdag(&a, Lx, CB, Linv, ldt, grid, st));
        if (prof) {
            CU(cudaEventRecord(ctx->pev[1], st));
            CU(cudaStreamSynchronize(st));
            float ms = 0;
            CU(cudaEventElapsedTime(&ms, ctx->pev[0], ctx->pev[1]));
            ctx->kind_ms[GB_K_FDAG] += ms;
            ctx->kind_n[GB_K_FDAG] += 1;
        }
        ctx->stats[4] = 1;
        ctx->launches += 1;
        P->linv_valid[d] = 1;
        return TRUE;
    }
    for (size_t i = 0; i < P->fact_seq.n; i++) {
        const gb_launch_rec *r = &seq[i];
        if (prof) CU(cudaEventRecord(ctx->pev[2 * i], st));
        switch (r->kind) {
        case GB_K_ASM:
            LK(gb_launch_assemble(&P->ptrs, P->d_asm + r->off, r->count, P->d_Sp, P->d_Si,
                                  Sx, adt, scale, beta, Lx, CB, ldt, st));
            break;
        case GB_K_SMALL:
            LK(gb_launch_factor_small(&P->ptrs, P->d_node + r->off, r->count, Lx, Linv, ldt, st));
            break;
        case GB_K_POTRF:
            LK(gb_launch_potrf_diag(&P->ptrs, P->d_potrf + r->off, r->count, Lx, Linv, ldt, st));
            break;
        case GB_K_TRSM:
            LK(gb_launch_trsm_rows(&P->ptrs, P->d_trsm + r->off, r->count, Lx, Linv, ldt, st));
            break;
        case GB_K_GEMM:
            LK(gb_launch_gemm(&P->ptrs, P->d_gemm + r->off, P->d_gemm_owner + r->off,
                              r->count, Lx, CB, ldt, st));
            break;
        case GB_K_DAG: {
            const gb_dag_level *lv = (const gb_dag_level *)P->dag_lv.p + r->off;
            size_t nt = (size_t)lv->ntasks;
            CU(cudaMemcpyAsync(P->d_dag_cnt, P->d_dag_nd + lv->task_off, sizeof(int32_t) * nt,
                               cudaMemcpyDeviceToDevice, st));
            CU(cudaMemsetAsync(P->d_dag_q, 0xFF, sizeof(int32_t) * 2 * nt, st));
            if (lv->n0)
                CU(cudaMemcpyAsync(P->d_dag_q, P->d_dag_q0i + lv->q0_off, sizeof(int32_t) * lv->n0,
                                   cudaMemcpyDeviceToDevice, st));
            if (lv->n1)
                CU(cudaMemcpyAsync(P->d_dag_q + nt, P->d_dag_q1i + lv->q1_off,
                                   sizeof(int32_t) * lv->n1, cudaMemcpyDeviceToDevice, st));
            CU(cudaMemcpyAsync(P->d_dag_ctrl, P->d_dag_ctrl0 + GB_DAG_NCTRL * r->off,
                               sizeof(int32_t) * GB_DAG_NCTRL, cudaMemcpyDeviceToDevice, st));
            gb_dag_args a;
            a.tasks = P->d_dag_t + lv->task_off;
            a.ntasks = (int)nt;
            a.succ_ptr = P->d_dag_sp + lv->sp_off;
            a.succ = P->d_dag_succ + lv->succ_off;
            a.cnt = P->d_dag_cnt;
            a.q0 = P->d_dag_q;
            a.q1 = P->d_dag_q + nt;
            a.ctrl = P->d_dag_ctrl;
            a.err = P->d_ticket + 3;
            a.trace = NULL;
            a.smflag = P->d_dag_smf;
            if (++P->dag_epoch <= 0) P->dag_epoch = 1;
            a.epoch = P->dag_epoch;
            if (ctx->trace_on) {
                /* factorization trace: all levels' tasks, 3 words each */
                size_t need = 3 * (P->dag_t.n + 1) * sizeof(unsigned long long);
                if (gb_dev_grow((void **)&ctx->d_ftrace, &ctx->ftrace_cap, need)) {
                    a.trace = ctx->d_ftrace + 3 * lv->task_off;
                    ctx->ftrace_n = (int64_t)P->dag_t.n;
                }
            }
            int grid = GB_MAX(1, ctx->sms) * 2;  /* resident blocks per SM */
            LK(gb_launch_dag(&P->ptrs, &a, Lx, CB, Linv, ldt, grid, st));
            break;
        }
        }
        if (prof) CU(cudaEventRecord(ctx->pev[2 * i + 1], st));
        launches++;
    }
    if (prof) {
        CU(cudaStreamSynchronize(st));
        for (size_t i = 0; i < P->fact_seq.n; i++) {
            float ms = 0;
            CU(cudaEventElapsedTime(&ms, ctx->pev[2 * i], ctx->pev[2 * i + 1]));
            int k = seq[i].kind & 15;
            ctx->kind_ms[k] += ms;
            ctx->kind_n[k] += 1;
        }
    }
    ctx->stats[4] = launches;
    ctx->launches += launches;
    /* every diagonal block's inverse was formed with its factorization */
    P->linv_valid[d] = 1;
    return TRUE;
cuda_fail:
    return FALSE;
}

/* inverses of the diagonal blocks of the device factor (for the sweeps) */
int gb_run_inverse(gb_plan *P, gb_ctx *ctx, int l_dtype)
{
    int d = dt_index(l_dtype);
    if (!P->d_Linv[d] && cudaMalloc(&P->d_Linv[d], dt_size(l_dtype) * GB_MAX(P->linv_total, 1))
                             != cudaSuccess) {
        P->d_Linv[d] = NULL;
        return FALSE;
    }
    if (gb_launch_diag_inverse(&P->ptrs, P->d_sd, (int)P->sd_t.n, P->d_blkoff, P->d_linvoff,
                               P->d_Lx[d], P->d_Linv[d], l_dtype == CHOLMOD_SINGLE ? 4 : 0,
                               ctx->stream) != 0)
        return FALSE;
    ctx->launches += 1;
    P->linv_valid[d] = 1;
    return TRUE;
}

/* error word of the single-launch sweeps (call after a synchronization) */
static int sweep_failed(gb_plan *P)
{
    int32_t e = 0;
    if (cudaMemcpy(&e, P->d_err, sizeof(int32_t), cudaMemcpyDeviceToHost) != cudaSuccess) return TRUE;
    return e != 0;
}

/* Replay one sweep on Y (device, n x nrhs, ld n) with the device factor. */
/* One single-launch sweep pass over nrhs <= GB_SWEEP_COLS columns on
 * stream st, with its own dependency words (xready, done, ticket[0..1]) and
 * update vectors U (cbv_total x nrhs): the leaf subtrees (one warp each,
 * before the other tasks forward, after them backward) and the
 * dependency-driven launch. */
static int sweep_pass(gb_plan *P, gb_ctx *ctx, int l_dtype, int nrhs, void *Y, int forward,
                      cudaStream_t st, int32_t *xready, int32_t *done, int32_t *ticket, void *U,
                      int allow_trace)
{
    int d = dt_index(l_dtype);
    int ldt = l_dtype == CHOLMOD_SINGLE ? 4 : 0;
    const void *Lx = P->d_Lx[d];
    gb_sweep1_args a;
    a.tasks = forward ? P->d_sf : P->d_sb;
    a.ntasks = (int)(forward ? P->sf_t.n : P->sb_t.n);
    a.gptr = forward ? P->d_gf : P->d_gb;
    a.cptr = P->d_sf_cptr;
    a.crange = P->d_sf_crange;
    a.ngroups = (int)(forward ? P->gf.n : P->gb.n) - 1;
    a.blkoff = P->d_blkoff;
    a.linvoff = P->d_linvoff;
    a.ntask_s = forward ? P->d_ntask_f : P->d_ntask_b;
    a.parent = P->d_parent;
    a.xready = xready;
    a.done = done;
    a.ticket = ticket;
    a.err = P->d_err;
    a.trace = NULL;
    a.act = P->sweep_act;
    a.sseg = P->d_sseg;
    a.bchunk_ptr = P->d_bchunk_ptr;
    a.bchunk = P->d_bchunk;
    if (allow_trace && ctx->trace_on) {
        size_t need = 3 * (size_t)(P->sf_t.n + P->sb_t.n + 2) * sizeof(unsigned long long);
        if (gb_dev_grow((void **)&ctx->d_trace, &ctx->trace_cap, need)) {
            int64_t off = forward ? 0 : 3 * (int64_t)(P->sf_t.n + 1);
            a.trace = ctx->d_trace + off;
            ctx->trace_off[forward ? 0 : 1] = off;
            ctx->trace_n[forward ? 0 : 1] = a.ntasks;
        }
    }
    if (cudaMemsetAsync(xready, 0, sizeof(int32_t) * (P->nblk_total + 1), st) != cudaSuccess
        || cudaMemsetAsync(done, 0, sizeof(int32_t) * (P->nsuper + 1), st) != cudaSuccess
        || cudaMemsetAsync(ticket, 0, sizeof(int32_t) * 2, st) != cudaSuccess)
        return FALSE;
    int grid = GB_MAX(1, ctx->sms) * 4;
    const int nleaf = (int)P->lf_t.n;
    const int lgrid = GB_MAX(1, ctx->sms) * 16;
    if (forward && nleaf > 0) {
        if (gb_launch_sweep_leaf(1, &P->ptrs, P->d_lf, nleaf, P->d_blkoff, P->d_linvoff,
                                 P->d_ntask_f, done, ticket + 1, Lx, P->d_Linv[d],
                                 ldt, nrhs, Y, P->n, U, lgrid, P->leaf_rows, P->sweep_act, P->d_sseg, st) != 0)
            return FALSE;
        ctx->launches += 1;
    }
    if (a.ntasks > 0) {
        if (gb_launch_sweep1(forward, &P->ptrs, &a, Lx, P->d_Linv[d], ldt, nrhs, Y, P->n,
                             U, grid, st) != 0)
            return FALSE;
        ctx->launches += 1;
    }
    if (!forward && nleaf > 0) {
        if (gb_launch_sweep_leaf(0, &P->ptrs, P->d_lf, nleaf, P->d_blkoff, P->d_linvoff,
                                 P->d_ntask_b, done, ticket + 1, Lx, P->d_Linv[d],
                                 ldt, nrhs, Y, P->n, U, lgrid, P->leaf_rows, P->sweep_act, P->d_sseg, st) != 0)
            return FALSE;
        ctx->launches += 1;
    }
    return TRUE;
}

/* side streams and fork/join events of the concurrent sweep passes */
static int sweep_streams(gb_ctx *ctx)
{
    if (ctx->side_ok) return ctx->side_ok > 0;
    ctx->side_ok = -1;
    if (cudaEventCreateWithFlags(&ctx->ev_fork, cudaEventDisableTiming) != cudaSuccess) return FALSE;
    for (int c = 0; c < GB_SWEEP_STREAMS - 1; c++)
        if (cudaStreamCreateWithFlags(&ctx->side[c], cudaStreamNonBlocking) != cudaSuccess
            || cudaEventCreateWithFlags(&ctx->ev_join[c], cudaEventDisableTiming) != cudaSuccess)
            return FALSE;
    ctx->side_ok = 1;
    return TRUE;
}

int gb_run_sweep(gb_plan *P, gb_ctx *ctx, int l_dtype, int nrhs, void *Y, int forward)
{
    cudaStream_t st = ctx->stream;
    int d = dt_index(l_dtype);
    int ldt = l_dtype == CHOLMOD_SINGLE ? 4 : 0;
    size_t e = dt_size(l_dtype);
    const void *Lx = P->d_Lx[d];
    if (ctx->sweep_mode == 1) {
        if (!P->linv_valid[d] && !gb_run_inverse(P, ctx, l_dtype)) return FALSE;
        /* the sweep's error word, shared by its passes */
        if (cudaMemsetAsync(P->d_err, 0, sizeof(int32_t), st) != cudaSuccess) return FALSE;
        const int npass = (nrhs + GB_SWEEP_COLS - 1) / GB_SWEEP_COLS;
        const int ns = GB_MIN(npass, ctx->sweep_streams);
        const size_t ureg = e * (size_t)GB_MAX(P->cbv_total, 1) * GB_SWEEP_COLS;
        const size_t words = (size_t)(P->nblk_total + 1) + (size_t)(P->nsuper + 1) + 4;
        if (ns > 1 && sweep_streams(ctx) && gb_dev_grow(&P->d_U, &P->u_cap, ureg * ns)
            && gb_dev_grow((void **)&P->d_sws, &P->sws_cap, sizeof(int32_t) * words * ns)) {
            /* passes of GB_SWEEP_COLS columns, up to GB_SWEEP_STREAMS of them
             * at once on their own streams, each with its own dependency
             * words and update vectors: the passes' dependency chains
             * through the top separators overlap instead of following one
             * another */
            int ok = cudaEventRecord(ctx->ev_fork, st) == cudaSuccess;
            for (int c = 1; c < ns; c++)
                ok = ok && cudaStreamWaitEvent(ctx->side[c - 1], ctx->ev_fork, 0) == cudaSuccess;
            for (int p = 0; ok && p < npass; p++) {
                const int c = p % ns;
                cudaStream_t sc = c ? ctx->side[c - 1] : st;
                int32_t *xr = P->d_sws + words * c;
                int32_t *dn = xr + P->nblk_total + 1;
                int32_t *tk = dn + P->nsuper + 1;
                ok = sweep_pass(P, ctx, l_dtype, GB_MIN(GB_SWEEP_COLS, nrhs - p * GB_SWEEP_COLS),
                                (char *)Y + e * (size_t)p * GB_SWEEP_COLS * (size_t)P->n, forward,
                                sc, xr, dn, tk, (char *)P->d_U + ureg * c, 0);
            }
            /* the side streams join the main stream whatever happened */
            for (int c = 1; c < ns; c++) {
                int j = cudaEventRecord(ctx->ev_join[c - 1], ctx->side[c - 1]) == cudaSuccess
                        && cudaStreamWaitEvent(st, ctx->ev_join[c - 1], 0) == cudaSuccess;
                ok = ok && j;
            }
            return ok;
        }
        /* one pass after the other on the main stream */
        const int w = GB_MIN(nrhs, GB_SWEEP_COLS);
        if (!gb_dev_grow(&P->d_U, &P->u_cap, e * GB_MAX(P->cbv_total, 1) * w)) return FALSE;
        for (int k0 = 0; k0 < nrhs; k0 += GB_SWEEP_COLS)
            if (!sweep_pass(P, ctx, l_dtype, GB_MIN(GB_SWEEP_COLS, nrhs - k0),
                            (char *)Y + e * (size_t)k0 * (size_t)P->n, forward, st, P->d_xready,
                            P->d_done, P->d_ticket, P->d_U, npass == 1))
                return FALSE;
        return TRUE;
    }
    if (!gb_dev_grow(&P->d_U, &P->u_cap, e * GB_MAX(P->cbv_total, 1) * nrhs)) return FALSE;
    gb_vec *seqv = forward ? &P->fwd_seq : &P->bwd_seq;
    const gb_launch_rec *seq = seqv->p;
    for (size_t i = 0; i < seqv->n; i++) {
        const gb_launch_rec *r = &seq[i];
        int rc = 0;
        switch (r->kind) {
        case GB_K_FWD_SMALL: rc = gb_launch_sweep_node(0, &P->ptrs, P->d_node + r->off, r->count, Lx, ldt, nrhs, Y, P->n, P->d_U, st); break;
        case GB_K_FWD_GATHER: rc = gb_launch_sweep_node(1, &P->ptrs, P->d_node + r->off, r->count, Lx, ldt, nrhs, Y, P->n, P->d_U, st); break;
        case GB_K_BWD_SMALL: rc = gb_launch_sweep_node(2, &P->ptrs, P->d_node + r->off, r->count, Lx, ldt, nrhs, Y, P->n, P->d_U, st); break;
        case GB_K_FWD_DIAG: rc = gb_launch_sweep_step(0, &P->ptrs, P->d_sweep + r->off, r->count, Lx, ldt, nrhs, Y, P->n, P->d_U, st); break;
        case GB_K_FWD_PANEL: rc = gb_launch_sweep_step(1, &P->ptrs, P->d_sweep + r->off, r->count, Lx, ldt, nrhs, Y, P->n, P->d_U, st); break;
        case GB_K_BWD_OFFDIAG: rc = gb_launch_sweep_step(2, &P->ptrs, P->d_sweep + r->off, r->count, Lx, ldt, nrhs, Y, P->n, P->d_U, st); break;
        case GB_K_BWD_DIAG: rc = gb_launch_sweep_step(3, &P->ptrs, P->d_sweep + r->off, r->count, Lx, ldt, nrhs, Y, P->n, P->d_U, st); break;
        case GB_K_BWD_PANEL: rc = gb_launch_sweep_step(4, &P->ptrs, P->d_sweep + r->off, r->count, Lx, ldt, nrhs, Y, P->n, P->d_U, st); break;
        }
        if (rc) return FALSE;
    }
    ctx->launches += (int64_t)seqv->n;
    return TRUE;
}

/* After a factorization with a failed pivot: reproduce the reference's
 * state (CHOLMOD/Supernodal/t_cholmod_super_numeric_worker.c:1084-1146):
 * s0 = first failing supernode in index order, L->minor = its first column
 * + failing local column; columns from the failing one (or all of s0 when
 * the first column failed or quick_return_if_not_posdef) and every later
 * supernode are zero.  Supernodes before s0 are neither descendants of a
 * failing supernode nor affected by one, so their values are final. */
int gb_fix_not_posdef(gb_plan *P, gb_ctx *ctx, cholmod_factor *L, int l_dtype,
                          cholmod_common *Common)
{
    int32_t *fail = malloc(sizeof(int32_t) * (P->nsuper + 1));
    if (!fail) { GB_ERROR(CHOLMOD_OUT_OF_MEMORY, "out of memory"); return FALSE; }
    if (cudaMemcpyAsync(fail, P->d_fail, sizeof(int32_t) * P->nsuper, cudaMemcpyDeviceToHost,
                        ctx->stream) != cudaSuccess
        || cudaStreamSynchronize(ctx->stream) != cudaSuccess) {
        free(fail);
        GB_ERROR(CHOLMOD_GPU_PROBLEM, "CUDA error");
        return FALSE;
    }
    Int s0 = -1;
    for (Int s = 0; s < P->nsuper; s++) if (fail[s] >= 0) { s0 = s; break; }
    if (s0 < 0) { free(fail); return TRUE; }
    const Int *Super = L->super, *Pi = L->pi, *Px = L->px;
    Int info = fail[s0] + 1;                         /* LAPACK-style, 1-based */
    free(fail);
    Int nsrow = Pi[s0 + 1] - Pi[s0];
    Int keep = (info == 1 || Common->quick_return_if_not_posdef) ? 0 : info - 1;
    int d = dt_index(l_dtype);
    if (gb_launch_zero_range(P->d_Lx[d], l_dtype == CHOLMOD_SINGLE ? 4 : 0,
                             Px[s0] + keep * nsrow, P->xsize, ctx->stream) != 0) {
        GB_ERROR(CHOLMOD_GPU_PROBLEM, "CUDA error");
        return FALSE;
    }
    L->minor = (size_t)(Super[s0] + info - 1);
    P->linv_valid[d] = 0;
    if (Common->status == CHOLMOD_OK) GB_ERROR(CHOLMOD_NOT_POSDEF, "matrix not positive definite");
    return TRUE;
}

/* Upload S = A (lower, packed, sorted or not) values and pattern. */
int gb_upload_input(gb_plan *P, gb_ctx *ctx, cholmod_sparse *A, int a_dtype)
{
    Int n = (Int)A->ncol;
    const Int *Ap = A->p;
    Int nz = Ap[n];
    size_t e = dt_size(a_dtype);
    P->s_from_vm = 0;           /* d_Sp/d_Si now hold this S's pattern */
    if (!gb_dev_grow((void **)&P->d_Sp, &P->sp_cap, sizeof(int64_t) * (n + 1))) return FALSE;
    if (!gb_dev_grow((void **)&P->d_Si, &P->si_cap, sizeof(int64_t) * GB_MAX(nz, 1))) return FALSE;
    if (!gb_dev_grow(&P->d_Sx, &P->sx_cap, e * GB_MAX(nz, 1))) return FALSE;
    cudaStream_t st = ctx->stream;
    if (cudaMemcpyAsync(P->d_Sp, A->p, sizeof(int64_t) * (n + 1), cudaMemcpyHostToDevice, st) != cudaSuccess) return FALSE;
    if (nz && cudaMemcpyAsync(P->d_Si, A->i, sizeof(int64_t) * nz, cudaMemcpyHostToDevice, st) != cudaSuccess) return FALSE;
    if (nz && cudaMemcpyAsync(P->d_Sx, A->x, e * nz, cudaMemcpyHostToDevice, st) != cudaSuccess) return FALSE;
    return TRUE;
}

/* ======================================================================== */

int cholmod_l_super_numeric(cholmod_sparse *A, cholmod_sparse *F, double beta[2],
                            cholmod_factor *L, cholmod_common *Common)
{
    if (!Common) return FALSE;
    if (Common->itype != CHOLMOD_LONG) {      /* as the reference's RETURN_IF_NULL_COMMON */
        Common->status = CHOLMOD_INVALID;
        return FALSE;
    }
    gb_autotune_first(A, F, beta, L, Common);
    return gb_super_numeric(A, F, beta, L, Common);
}

/* The body of cholmod_l_super_numeric on int64 objects (also reached from
 * the int32 entry point through int64 shadow objects, gb_int32.c). */
int gb_super_numeric(cholmod_sparse *A, cholmod_sparse *F, double beta[2],
                     cholmod_factor *L, cholmod_common *Common)
{
    if (!Common) return FALSE;
    if (!L || !A) { GB_ERROR(CHOLMOD_INVALID, "argument missing"); return FALSE; }
    if (A->xtype < CHOLMOD_REAL || A->xtype > CHOLMOD_ZOMPLEX || !A->x) {
        GB_ERROR(CHOLMOD_INVALID, "invalid xtype");
        return FALSE;
    }
    if (L->xtype < CHOLMOD_PATTERN || L->xtype > CHOLMOD_COMPLEX) {
        GB_ERROR(CHOLMOD_INVALID, "invalid xtype");
        return FALSE;
    }
    if (A->stype < 0) {
        if (A->nrow != A->ncol || A->nrow != L->n) {
            GB_ERROR(CHOLMOD_INVALID, "invalid dimensions");
            return FALSE;
        }
    } else if (A->stype == 0) {
        /* beta I + A F, F = A' or A(:,f)' (the reference's checks,
         * Supernodal/cholmod_super_numeric.c:135-156) */
        if (A->nrow != L->n) { GB_ERROR(CHOLMOD_INVALID, "invalid dimensions"); return FALSE; }
        if (!F) { GB_ERROR(CHOLMOD_INVALID, "argument missing"); return FALSE; }
        if (F->xtype < CHOLMOD_REAL || F->xtype > CHOLMOD_ZOMPLEX || !F->x) {
            GB_ERROR(CHOLMOD_INVALID, "invalid xtype");
            return FALSE;
        }
        if (A->nrow != F->ncol || A->ncol != F->nrow || F->stype != 0) {
            GB_ERROR(CHOLMOD_INVALID, "F invalid");
            return FALSE;
        }
        if (A->xtype != F->xtype || A->dtype != F->dtype) {
            GB_ERROR(CHOLMOD_INVALID, "A and F must have same xtype and dtype");
            return FALSE;
        }
        if (F->itype != CHOLMOD_LONG) {
            GB_ERROR(CHOLMOD_INVALID, "int64 (cholmod_l_) objects required");
            return FALSE;
        }
    } else {
        GB_ERROR(CHOLMOD_INVALID, "symmetric upper case not supported");
        return FALSE;
    }
    if (!L->is_super) { GB_ERROR(CHOLMOD_INVALID, "L not supernodal"); return FALSE; }
    if (L->xtype != CHOLMOD_PATTERN) {
        if (!(A->xtype == CHOLMOD_REAL && L->xtype == CHOLMOD_REAL)
            && !(A->xtype >= CHOLMOD_COMPLEX && L->xtype == CHOLMOD_COMPLEX)) {
            GB_ERROR(CHOLMOD_INVALID, "complex type mismatch");
            return FALSE;
        }
        if (A->dtype != L->dtype) {
            GB_ERROR(CHOLMOD_INVALID, "A and L must have the same dtype");
            return FALSE;
        }
    }
    if (A->itype != CHOLMOD_LONG || L->itype != CHOLMOD_LONG) {
        GB_ERROR(CHOLMOD_INVALID, "int64 (cholmod_l_) objects required");
        return FALSE;
    }
    if (A->xtype != CHOLMOD_REAL) return gb_super_numeric_complex(A, F, beta, L, Common);
    Common->status = CHOLMOD_OK;
    const int dtype = A->dtype;
    gb_ctx *ctx = NULL;
    int32_t anyfail = 0;
    gb_plan *P = gb_numeric_core(A, F, beta ? beta[0] : 0.0, L, dtype, 0, &anyfail, &ctx, Common);
    if (!P) return FALSE;
    if (L->xtype == CHOLMOD_PATTERN) {
        /* supernodal symbolic -> numeric: allocate L->x (change_factor) */
        L->x = gb_malloc(L->xsize, dt_size(dtype), Common);
        if (!L->x) return FALSE;
        L->dtype = dtype;
        L->xtype = CHOLMOD_REAL;
    }
    L->is_ll = TRUE;
    L->minor = L->n;
    if (anyfail && !gb_fix_not_posdef(P, ctx, L, dtype, Common)) return FALSE;
    int d = dt_index(dtype);
    P->dev_valid[d] = 1;
    P->dev_valid[1 - d] = 0;
    P->host_x[d] = L->x;
    if (!ctx->opt_keep) {
        if (cudaMemcpyAsync(L->x, P->d_Lx[d], dt_size(dtype) * L->xsize, cudaMemcpyDeviceToHost,
                            ctx->stream) != cudaSuccess
            || cudaStreamSynchronize(ctx->stream) != cudaSuccess) {
            GB_ERROR(CHOLMOD_GPU_PROBLEM, "CUDA error copying L");
            return FALSE;
        }
    } else {
        cudaStreamSynchronize(ctx->stream);
    }
    return Common->status >= CHOLMOD_OK;
}

/* The device factorization behind cholmod_l_super_numeric: the input (S
 * lower, or beta I + A F in the A F form, packed on the host when it is
 * not), uploaded and factorized into the device factor of FL's plan in
 * dtype.  cx_diag: in the A F form the entries (2k+1, 2k) of the product
 * stay zero (the imaginary parts of a complex diagonal, in the real
 * embedding of a complex matrix, which the reference's complex
 * factorization ignores).  *anyfail: a pivot was not positive.  Returns the
 * plan, or NULL with Common->status set; FL's host values are untouched. */
gb_plan *gb_numeric_core(cholmod_sparse *A, cholmod_sparse *F, double beta, cholmod_factor *FL,
                         int dtype, int cx_diag, int32_t *anyfail, gb_ctx **pctx,
                         cholmod_common *Common)
{
    cholmod_sparse *Apk = A;
    /* the A F form: C = tril(A F), pattern and product lists on the host,
     * values on the device after the upload (gb_aft.c) */
    int64_t *aft_ptr = NULL, *aft_pairs = NULL;
    if (A->stype == 0) {
        Apk = gb_aft_pattern(A, F, &aft_ptr, &aft_pairs, Common);
        if (!Apk) return NULL;
        if (cx_diag) {
            /* drop the products of the entries (2k+1, 2k) */
            const Int nc = (Int)Apk->ncol, *Cp = Apk->p, *Ci = Apk->i;
            int64_t w = 0, start = 0;
            for (Int c = 0; c < nc; c++) {
                for (Int e = Cp[c]; e < Cp[c + 1]; e++) {
                    const int64_t p0 = start, p1 = aft_ptr[e + 1];
                    start = p1;
                    aft_ptr[e] = w;
                    if (c % 2 == 0 && Ci[e] == c + 1) continue;
                    for (int64_t q = p0; q < p1; q++) {
                        aft_pairs[2 * w] = aft_pairs[2 * q];
                        aft_pairs[2 * w + 1] = aft_pairs[2 * q + 1];
                        w++;
                    }
                }
            }
            aft_ptr[Cp[nc]] = w;
        }
    } else if (!A->packed) {
        /* pack the columns (unpacked input) on the host */
        Int n = (Int)A->ncol, nz = 0;
        const Int *Ap = A->p, *Anz = A->nz;
        for (Int j = 0; j < n; j++) nz += Anz[j];
        Apk = gb300_allocate_sparse(A->nrow, n, nz, A->sorted, TRUE, A->stype,
                                    CHOLMOD_REAL + dtype, Common);
        if (!Apk) return NULL;
        Int *Bp = Apk->p, *Bi = Apk->i;
        size_t e = dt_size(dtype);
        Int q = 0;
        for (Int j = 0; j < n; j++) {
            Bp[j] = q;
            memcpy(Bi + q, (Int *)A->i + Ap[j], sizeof(Int) * Anz[j]);
            memcpy((char *)Apk->x + q * e, (char *)A->x + Ap[j] * e, e * Anz[j]);
            q += Anz[j];
        }
        Bp[n] = q;
    }
    gb_plan *P = NULL;
    gb_ctx *ctx = gb_ctx_get(Common, 1);
    if (!ctx || !gb_ctx_ready(ctx)) {
        GB_ERROR(CHOLMOD_GPU_PROBLEM, "no CUDA device");
        goto done;
    }
    *pctx = ctx;
    P = gb_plan_get(FL, Common, ctx, 1);
    if (!P) goto done;
    if (!gb_ensure_numeric(P, dtype) || !gb_upload_input(P, ctx, Apk, dtype)) {
        GB_ERROR(CHOLMOD_GPU_PROBLEM, "device allocation failed");
        P = NULL;
        goto done;
    }
    if (aft_ptr) {
        /* values of C = tril(A F): each entry's products summed on the device */
        const Int nent = ((const Int *)Apk->p)[Apk->ncol];
        const Int *Ap0 = A->p, *Fp0 = F->p;
        const Int anz = A->packed ? Ap0[A->ncol] : A->nzmax, fnz = F->packed ? Fp0[F->ncol] : F->nzmax;
        const size_t e = dt_size(dtype);
        void *dA = NULL, *dF = NULL;
        int64_t *dptr = NULL, *dpairs = NULL;
        int okp = cudaMalloc(&dA, e * GB_MAX(anz, 1)) == cudaSuccess
                  && cudaMalloc(&dF, e * GB_MAX(fnz, 1)) == cudaSuccess
                  && cudaMalloc((void **)&dptr, sizeof(int64_t) * (nent + 1)) == cudaSuccess
                  && cudaMalloc((void **)&dpairs, sizeof(int64_t) * 2 * GB_MAX(aft_ptr[nent], 1)) == cudaSuccess
                  && cudaMemcpyAsync(dA, A->x, e * anz, cudaMemcpyHostToDevice, ctx->stream) == cudaSuccess
                  && cudaMemcpyAsync(dF, F->x, e * fnz, cudaMemcpyHostToDevice, ctx->stream) == cudaSuccess
                  && cudaMemcpyAsync(dptr, aft_ptr, sizeof(int64_t) * (nent + 1), cudaMemcpyHostToDevice, ctx->stream) == cudaSuccess
                  && cudaMemcpyAsync(dpairs, aft_pairs, sizeof(int64_t) * 2 * aft_ptr[nent], cudaMemcpyHostToDevice, ctx->stream) == cudaSuccess
                  && gb_launch_pair_sum(nent, dptr, dpairs, dA, dF, P->d_Sx, dtype == CHOLMOD_SINGLE ? 4 : 0,
                                        ctx->stream) == 0
                  && cudaStreamSynchronize(ctx->stream) == cudaSuccess;
        if (dA) cudaFree(dA);
        if (dF) cudaFree(dF);
        if (dptr) cudaFree(dptr);
        if (dpairs) cudaFree(dpairs);
        if (!okp) {
            cudaGetLastError();
            GB_ERROR(CHOLMOD_GPU_PROBLEM, "CUDA error forming A*F'");
            P = NULL;
            goto done;
        }
    }
    {
        cudaEventRecord(ctx->ev0, ctx->stream);
        int ok = gb_run_factor(P, ctx, P->d_Sx, dtype, dtype, NULL, beta);
        cudaEventRecord(ctx->ev1, ctx->stream);
        int32_t dagerr = 0;
        *anyfail = 0;
        if (ok) ok = cudaMemcpyAsync(anyfail, P->d_anyfail, sizeof(int32_t), cudaMemcpyDeviceToHost, ctx->stream) == cudaSuccess
                     && cudaMemcpyAsync(&dagerr, P->d_ticket + 3, sizeof(int32_t), cudaMemcpyDeviceToHost, ctx->stream) == cudaSuccess
                     && cudaStreamSynchronize(ctx->stream) == cudaSuccess && !dagerr;
        if (!ok) {
            GB_ERROR(CHOLMOD_GPU_PROBLEM, "CUDA error in the factorization");
            P = NULL;
            goto done;
        }
        float ms = 0;
        cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1);
        ctx->stats[0] = ms;
    }
done:
    if (Apk != A) gb300_free_sparse(&Apk, Common);
    free(aft_ptr);
    free(aft_pairs);
    return P;
}

/* Factorize S (lower, in FS's column order, dtype; beta added to the
 * diagonal) into the device factor of the supernodal symbolic factor FS,
 * without the supernodal not-positive-definite clean-up and without host
 * values.  *minor = the first column whose pivot was not positive (FS->n
 * when none); every column before it is complete.  Returns the plan (its
 * d_Lx[dtype] holds the factor) or NULL with Common->status set. */
gb_plan *gb_factor_device_only(cholmod_sparse *S, double beta, cholmod_factor *FS, int dtype,
                               int64_t *minor, cholmod_common *Common)
{
    gb_ctx *ctx = gb_ctx_get(Common, 1);
    if (!ctx || !gb_ctx_ready(ctx)) { GB_ERROR(CHOLMOD_GPU_PROBLEM, "no CUDA device"); return NULL; }
    gb_plan *P = gb_plan_get(FS, Common, ctx, 1);
    if (!P) return NULL;
    if (!gb_ensure_numeric(P, dtype) || !gb_upload_input(P, ctx, S, dtype)) {
        GB_ERROR(CHOLMOD_GPU_PROBLEM, "device allocation failed");
        return NULL;
    }
    cudaEventRecord(ctx->ev0, ctx->stream);
    int ok = gb_run_factor(P, ctx, P->d_Sx, dtype, dtype, NULL, beta);
    cudaEventRecord(ctx->ev1, ctx->stream);
    int32_t anyfail = 0, dagerr = 0;
    if (ok) ok = cudaMemcpyAsync(&anyfail, P->d_anyfail, sizeof(int32_t), cudaMemcpyDeviceToHost, ctx->stream) == cudaSuccess
                 && cudaMemcpyAsync(&dagerr, P->d_ticket + 3, sizeof(int32_t), cudaMemcpyDeviceToHost, ctx->stream) == cudaSuccess
                 && cudaStreamSynchronize(ctx->stream) == cudaSuccess && !dagerr;
    if (!ok) { GB_ERROR(CHOLMOD_GPU_PROBLEM, "CUDA error in the factorization"); return NULL; }
    float ms = 0;
    cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1);
    ctx->stats[0] = ms;
    int d = dt_index(dtype);
    P->dev_valid[d] = 0;                 /* no host values mirror it */
    P->dev_valid[1 - d] = 0;
    *minor = (int64_t)FS->n;
    if (anyfail) {
        int32_t *fail = malloc(sizeof(int32_t) * (P->nsuper + 1));
        if (!fail || cudaMemcpy(fail, P->d_fail, sizeof(int32_t) * P->nsuper,
                                cudaMemcpyDeviceToHost) != cudaSuccess) {
            free(fail);
            GB_ERROR(CHOLMOD_GPU_PROBLEM, "CUDA error");
            return NULL;
        }
        const Int *Super = FS->super;
        for (Int s = 0; s < P->nsuper; s++)
            if (fail[s] >= 0) { *minor = Super[s] + fail[s]; break; }
        free(fail);
    }
    return P;
}

/* device factor of L in dtype, uploading L->x when this library did not
 * produce the current values */
static gb_plan *factor_on_device(cholmod_factor *L, gb_ctx *ctx, cholmod_common *Common)
{
    gb_plan *P = gb_plan_get(L, Common, ctx, 1);
    if (!P) return NULL;
    int d = dt_index(L->dtype);
    if (P->dev_valid[d] && P->host_x[d] == L->x) return P;
    if (!L->x) { GB_ERROR(CHOLMOD_INVALID, "L has no numerical values"); return NULL; }
    if (!gb_ensure_numeric(P, L->dtype)) { GB_ERROR(CHOLMOD_GPU_PROBLEM, "device allocation failed"); return NULL; }
    if (cudaMemcpyAsync(P->d_Lx[d], L->x, dt_size(L->dtype) * L->xsize, cudaMemcpyHostToDevice,
                        ctx->stream) != cudaSuccess) {
        GB_ERROR(CHOLMOD_GPU_PROBLEM, "CUDA error");
        return NULL;
    }
    P->dev_valid[d] = 1;
    P->host_x[d] = L->x;
    P->linv_valid[d] = 0;
    return P;
}

static int super_solve(cholmod_factor *L, cholmod_dense *X, cholmod_dense *E,
                       cholmod_common *Common, int forward)
{
    if (!Common) return FALSE;
    if (!L || !X || !E) { GB_ERROR(CHOLMOD_INVALID, "argument missing"); return FALSE; }
    if (L->xtype == CHOLMOD_COMPLEX) return gb_super_solve_complex(L, X, E, Common, forward);
    if (L->xtype != CHOLMOD_REAL || X->xtype != CHOLMOD_REAL || E->xtype != CHOLMOD_REAL) {
        GB_ERROR(CHOLMOD_INVALID, "real factor and matrices required");
        return FALSE;
    }
    if (L->dtype != X->dtype || L->dtype != E->dtype) {
        GB_ERROR(CHOLMOD_INVALID, "all xtypes and dtypes must match");
        return FALSE;
    }
    if (!L->is_ll) { GB_ERROR(CHOLMOD_INVALID, "L must be LL', not LDL'"); return FALSE; }
    if (!L->is_super) { GB_ERROR(CHOLMOD_INVALID, "L must be supernodal"); return FALSE; }
    if (X->nrow != L->n) { GB_ERROR(CHOLMOD_INVALID, "X and L dimensions must match"); return FALSE; }
    if (E->nzmax < X->ncol * L->maxesize) {
        GB_ERROR(CHOLMOD_INVALID, "workspace E not large enough");
        return FALSE;
    }
    Common->status = CHOLMOD_OK;
    if (L->n == 0 || X->ncol == 0) return TRUE;
    gb_ctx *ctx = gb_ctx_get(Common, 1);
    if (!ctx || !gb_ctx_ready(ctx)) { GB_ERROR(CHOLMOD_GPU_PROBLEM, "no CUDA device"); return FALSE; }
    gb_plan *P = factor_on_device(L, ctx, Common);
    if (!P) return FALSE;
    int nrhs = (int)X->ncol;
    size_t e = dt_size(L->dtype);
    Int n = P->n;
    if (!gb_dev_grow(&P->d_Y, &P->y_cap, e * n * nrhs)) { GB_ERROR(CHOLMOD_GPU_PROBLEM, "device allocation failed"); return FALSE; }
    cudaStream_t st = ctx->stream;
    int ok = cudaMemcpy2DAsync(P->d_Y, e * n, X->x, e * X->d, e * n, nrhs,
                               cudaMemcpyHostToDevice, st) == cudaSuccess;
    cudaEventRecord(ctx->ev0, st);
    ok = ok && gb_run_sweep(P, ctx, L->dtype, nrhs, P->d_Y, forward);
    cudaEventRecord(ctx->ev1, st);
    ok = ok && cudaMemcpy2DAsync(X->x, e * X->d, P->d_Y, e * n, e * n, nrhs,
                                 cudaMemcpyDeviceToHost, st) == cudaSuccess;
    ok = ok && cudaStreamSynchronize(st) == cudaSuccess;
    ok = ok && !(ctx->sweep_mode == 1 && sweep_failed(P));
    if (!ok) { GB_ERROR(CHOLMOD_GPU_PROBLEM, "CUDA error in the solve"); return FALSE; }
    float ms = 0;
    cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1);
    ctx->stats[1] = ms;
    return TRUE;
}

int gb_super_solve(cholmod_factor *L, cholmod_dense *X, cholmod_dense *E, cholmod_common *Common,
                   int forward)
{
    return super_solve(L, X, E, Common, forward);
}

int cholmod_l_super_lsolve(cholmod_factor *L, cholmod_dense *X, cholmod_dense *E,
                           cholmod_common *Common)
{
    if (Common && Common->itype != CHOLMOD_LONG) { Common->status = CHOLMOD_INVALID; return FALSE; }
    return super_solve(L, X, E, Common, 1);
}

int cholmod_l_super_ltsolve(cholmod_factor *L, cholmod_dense *X, cholmod_dense *E,
                            cholmod_common *Common)
{
    if (Common && Common->itype != CHOLMOD_LONG) { Common->status = CHOLMOD_INVALID; return FALSE; }
    return super_solve(L, X, E, Common, 0);
}

/* ---- gb300_factorize / gb300_solve ---------------------------------------- */

int gb300_factorize(cholmod_sparse *A, double beta[2], cholmod_factor *L,
                    cholmod_common *Common)
{
    if (!Common) return FALSE;
    if (!A || !L) { GB_ERROR(CHOLMOD_INVALID, "argument missing"); return FALSE; }
    if (A->stype >= 0 || A->nrow != A->ncol || A->nrow != L->n || !L->Perm) {
        GB_ERROR(CHOLMOD_INVALID, "A must be symmetric-lower and match L");
        return FALSE;
    }
    cholmod_sparse *S = gb_permute_lower(A, L->Perm, Common);
    if (!S) return FALSE;
    double zero[2] = {0, 0};
    int ok = cholmod_l_super_numeric(S, NULL, beta ? beta : zero, L, Common);
    gb300_free_sparse(&S, Common);
    return ok;
}

/* X = op(B) on the device for the sys values of cholmod_l_solve with a
 * supernodal LL' factor: the permutation only for sys = A, P, Pt and an
 * ordering other than natural (CHOLMOD/Cholesky/cholmod_solve.c:262-267);
 * sys = P is X = P*B and Pt is X = P'*B (:616-650); every other sys is
 * X = P'*(op(L) \ (P*B)) with lsolve for A, LDLt, LD, L and ltsolve for A,
 * LDLt, DLt, Lt (:689-722), D = I.  B and X share P->d_B (n x nrhs,
 * leading dimension n); P->d_Y is the workspace.  *swept = 1 when a sweep
 * ran. */
static int gb_solve_dev(int sys, cholmod_factor *L, gb_plan *P, gb_ctx *ctx, int nrhs,
                        int *swept)
{
    Int n = P->n;
    int dt = L->dtype == CHOLMOD_SINGLE ? 4 : 0;
    cudaStream_t st = ctx->stream;
    const int64_t *perm = L->ordering != CHOLMOD_NATURAL ? P->d_Perm : NULL;
    const int64_t *pin = (sys == CHOLMOD_A || sys == CHOLMOD_P) ? perm : NULL;
    const int64_t *pout = (sys == CHOLMOD_A || sys == CHOLMOD_Pt) ? perm : NULL;
    int fwd = sys == CHOLMOD_A || sys == CHOLMOD_LDLt || sys == CHOLMOD_LD || sys == CHOLMOD_L;
    int bwd = sys == CHOLMOD_A || sys == CHOLMOD_LDLt || sys == CHOLMOD_DLt || sys == CHOLMOD_Lt;
    *swept = fwd || bwd;
    int ok = gb_launch_perm_in(n, nrhs, pin, NULL, P->d_B, dt, n, P->d_Y, dt, n, st) == 0;
    ok = ok && (!fwd || gb_run_sweep(P, ctx, L->dtype, nrhs, P->d_Y, 1));
    ok = ok && (!bwd || gb_run_sweep(P, ctx, L->dtype, nrhs, P->d_Y, 0));
    ok = ok && gb_launch_perm_out(n, nrhs, pout, NULL, P->d_Y, dt, n, P->d_B, dt, n, 0, st) == 0;
    return ok;
}

cholmod_dense *gb300_solve(int sys, cholmod_factor *L, cholmod_dense *B,
                           cholmod_common *Common)
{
    if (!Common) return NULL;
    if (!L || !B) { GB_ERROR(CHOLMOD_INVALID, "argument missing"); return NULL; }
    if (sys < CHOLMOD_A || sys > CHOLMOD_Pt) { GB_ERROR(CHOLMOD_INVALID, "invalid system"); return NULL; }
    if (L->xtype != CHOLMOD_REAL || !L->is_super || B->xtype != CHOLMOD_REAL
        || B->nrow != L->n || B->dtype != L->dtype) {
        GB_ERROR(CHOLMOD_INVALID, "invalid L or B");
        return NULL;
    }
    Common->status = CHOLMOD_OK;
    gb_ctx *ctx = gb_ctx_get(Common, 1);
    if (!ctx || !gb_ctx_ready(ctx)) { GB_ERROR(CHOLMOD_GPU_PROBLEM, "no CUDA device"); return NULL; }
    gb_plan *P = factor_on_device(L, ctx, Common);
    if (!P) return NULL;
    int nrhs = (int)B->ncol;
    Int n = P->n;
    size_t e = dt_size(L->dtype);
    cholmod_dense *X = gb300_allocate_dense(n, nrhs, n, CHOLMOD_REAL + L->dtype, Common);
    if (!X) return NULL;
    if (n == 0 || nrhs == 0) return X;
    cudaStream_t st = ctx->stream;
    int swept = 0;
    int ok = gb_dev_grow(&P->d_Y, &P->y_cap, e * n * nrhs) && gb_dev_grow(&P->d_B, &P->b_cap, e * n * nrhs);
    ok = ok && cudaMemcpy2DAsync(P->d_B, e * n, B->x, e * B->d, e * n, nrhs,
                                 cudaMemcpyHostToDevice, st) == cudaSuccess;
    cudaEventRecord(ctx->ev0, st);
    ok = ok && gb_solve_dev(sys, L, P, ctx, nrhs, &swept);
    cudaEventRecord(ctx->ev1, st);
    ok = ok && cudaMemcpyAsync(X->x, P->d_B, e * n * nrhs, cudaMemcpyDeviceToHost, st) == cudaSuccess;
    ok = ok && cudaStreamSynchronize(st) == cudaSuccess;
    ok = ok && !(swept && ctx->sweep_mode == 1 && sweep_failed(P));
    if (!ok) {
        gb300_free_dense(&X, Common);
        GB_ERROR(CHOLMOD_GPU_PROBLEM, "CUDA error in the solve");
        return NULL;
    }
    float ms = 0;
    cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1);
    ctx->stats[1] = ms;
    return X;
}

/* ---- cholmod_l_spsolve ------------------------------------------------------ */

#define GB_SP_CHUNK 64                /* right-hand-side columns per device pass */

static size_t sp_align(size_t b) { return (b + 255) & ~(size_t)255; }

/* X = A\B (or the other sys) for a sparse B, returned sparse
 * (CHOLMOD/Cholesky/cholmod_spsolve.c:56-278): the same argument checks and
 * result, X(:,j) holding the entries of the dense solution that are not zero
 * (x != 0; NaN kept), rows ascending, X packed and sorted with nzmax = nnz(X)
 * (at least 1).  Where the reference solves 4 columns at a time through
 * cholmod_l_solve, this solves up to 64 per pass on the GPU: the host packs
 * the chunk of B (for a duplicated row index the last entry wins, as in the
 * reference's scatter), the device scatters it into a dense block, solves,
 * counts the nonzeros of every 4096-row segment of every column and compacts
 * them; only the counts and the compacted entries come back. */
cholmod_sparse *cholmod_l_spsolve(int sys, cholmod_factor *L, cholmod_sparse *B,
                                  cholmod_common *Common)
{
    if (!Common) return NULL;
    if (!L || !B) { GB_ERROR(CHOLMOD_INVALID, "argument missing"); return NULL; }
    if (L->xtype != CHOLMOD_REAL || B->xtype != CHOLMOD_REAL) {
        GB_ERROR(CHOLMOD_INVALID, "L and B must be real");
        return NULL;
    }
    if (L->n != B->nrow) { GB_ERROR(CHOLMOD_INVALID, "dimensions of L and B do not match"); return NULL; }
    if (B->stype) { GB_ERROR(CHOLMOD_INVALID, "B cannot be stored in symmetric mode"); return NULL; }
    if (L->dtype != B->dtype) { GB_ERROR(CHOLMOD_INVALID, "dtype of L and B must match"); return NULL; }
    if (sys < CHOLMOD_A || sys > CHOLMOD_Pt) { GB_ERROR(CHOLMOD_INVALID, "invalid system"); return NULL; }
    if (!L->is_super) { GB_ERROR(CHOLMOD_INVALID, "L must be supernodal"); return NULL; }
    Common->status = CHOLMOD_OK;
    const Int n = (Int)L->n, nrhs = (Int)B->ncol;
    const Int *Bp = B->p, *Bi = B->i, *Bnz = B->nz;
    const int packed = B->packed;
    const size_t e = dt_size(L->dtype);
    const int dt = L->dtype == CHOLMOD_SINGLE ? 4 : 0;
    for (Int j = 0; j < nrhs; j++) {
        Int p0 = Bp[j], p1 = packed ? Bp[j + 1] : p0 + Bnz[j];
        for (Int p = p0; p < p1; p++)
            if (Bi[p] < 0 || Bi[p] >= n) { GB_ERROR(CHOLMOD_INVALID, "B row index out of range"); return NULL; }
    }
    gb_ctx *ctx = gb_ctx_get(Common, 1);
    if (!ctx || !gb_ctx_ready(ctx)) { GB_ERROR(CHOLMOD_GPU_PROBLEM, "no CUDA device"); return NULL; }
    gb_plan *P = factor_on_device(L, ctx, Common);
    if (!P) return NULL;

    const Int ch = GB_MIN(GB_MAX(nrhs, 1), GB_SP_CHUNK);
    const int64_t nseg = gb_sp_nseg(n);
    /* host staging: packed chunk of B, counts/offsets, growable X entries */
    Int *cp = malloc(sizeof(Int) * (ch + 1)), *cnt = malloc(sizeof(Int) * (nseg * ch + 1));
    Int *mark = malloc(sizeof(Int) * (n + 1));
    Int *Xp = calloc(nrhs + 1, sizeof(Int));
    size_t bcap = 1024, xcap = 1024, xnz = 0;
    Int *ci = malloc(sizeof(Int) * bcap), *Xi = malloc(sizeof(Int) * xcap);
    char *cx = malloc(e * bcap), *Xx = malloc(e * xcap);
    int ok = cp && cnt && mark && Xp && ci && Xi && cx && Xx, oom = !ok;
    for (Int i = 0; ok && i < n; i++) mark[i] = -1;
    cudaStream_t st = ctx->stream;
    int swept = 0;
    double dev_ms = 0;                /* device time of the passes (events) */
    for (Int j0 = 0; ok && n > 0 && j0 < nrhs; j0 += ch) {
        const Int j1 = GB_MIN(nrhs, j0 + ch), w = j1 - j0;
        /* pack B(:, j0:j1-1), the last of duplicated rows kept */
        size_t bnz = 0;
        for (Int j = j0; j < j1; j++) bnz += (size_t)(packed ? Bp[j + 1] - Bp[j] : Bnz[j]);
        if (bnz > bcap) {
            bcap = bnz;
            Int *ni = realloc(ci, sizeof(Int) * bcap);
            char *nx = ni ? realloc(cx, e * bcap) : NULL;
            if (ni) ci = ni;
            if (nx) cx = nx;
            if (!ni || !nx) { ok = 0; oom = 1; break; }
        }
        size_t q = 0;
        for (Int j = j0; j < j1; j++) {
            cp[j - j0] = (Int)q;
            Int p0 = Bp[j], p1 = packed ? Bp[j + 1] : p0 + Bnz[j];
            for (Int p = p1 - 1; p >= p0; p--) {
                if (mark[Bi[p]] == j) continue;
                mark[Bi[p]] = j;
                ci[q] = Bi[p];
                memcpy(cx + e * q, (const char *)B->x + e * p, e);
                q++;
            }
        }
        cp[w] = (Int)q;
        /* device scratch: cp, ci, cx, counts/offsets, X rows, X values */
        size_t o_cp = 0, o_ci = o_cp + sp_align(sizeof(Int) * (w + 1));
        size_t o_cx = o_ci + sp_align(sizeof(Int) * GB_MAX(q, 1));
        size_t o_cn = o_cx + sp_align(e * GB_MAX(q, 1));
        size_t o_xi = o_cn + sp_align(sizeof(Int) * (nseg * w + 1));
        size_t o_xx = o_xi + sp_align(sizeof(Int) * n * w);
        size_t tot = o_xx + sp_align(e * n * w);
        ok = gb_dev_grow(&P->d_Y, &P->y_cap, e * n * w) && gb_dev_grow(&P->d_B, &P->b_cap, e * n * w)
             && gb_dev_grow(&P->d_spw, &P->spw_cap, tot);
        if (!ok) break;
        char *base = (char *)P->d_spw;
        Int *d_cp = (Int *)(base + o_cp), *d_ci = (Int *)(base + o_ci), *d_cn = (Int *)(base + o_cn);
        Int *d_xi = (Int *)(base + o_xi);
        void *d_cx = base + o_cx, *d_xx = base + o_xx;
        ok = cudaMemcpyAsync(d_cp, cp, sizeof(Int) * (w + 1), cudaMemcpyHostToDevice, st) == cudaSuccess
             && (q == 0 || (cudaMemcpyAsync(d_ci, ci, sizeof(Int) * q, cudaMemcpyHostToDevice, st) == cudaSuccess
                            && cudaMemcpyAsync(d_cx, cx, e * q, cudaMemcpyHostToDevice, st) == cudaSuccess))
             && cudaEventRecord(ctx->ev0, st) == cudaSuccess
             && cudaMemsetAsync(P->d_B, 0, e * n * w, st) == cudaSuccess
             && gb_launch_sp_scatter(n, w, d_cp, d_ci, d_cx, dt, P->d_B, n, st) == 0
             && gb_solve_dev(sys, L, P, ctx, (int)w, &swept)
             && gb_launch_sp_count(n, w, P->d_B, dt, n, d_cn, st) == 0
             && cudaEventRecord(ctx->ev1, st) == cudaSuccess
             && cudaMemcpyAsync(cnt, d_cn, sizeof(Int) * nseg * w, cudaMemcpyDeviceToHost, st) == cudaSuccess
             && cudaStreamSynchronize(st) == cudaSuccess
             && !(swept && ctx->sweep_mode == 1 && sweep_failed(P));
        if (!ok) break;
        float ms = 0;
        cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1);
        dev_ms += ms;
        /* offsets of every (column, segment) within the chunk, columns first */
        size_t c = 0;
        for (Int j = 0; j < w; j++) {
            Xp[j0 + j] = (Int)(xnz + c);
            for (int64_t s = 0; s < nseg; s++) {
                size_t k = (size_t)cnt[j * nseg + s];
                cnt[j * nseg + s] = (Int)c;
                c += k;
            }
        }
        if (xnz + c > xcap) {
            size_t ncap = GB_MAX(xnz + c, 2 * xcap);
            Int *ni = realloc(Xi, sizeof(Int) * ncap);
            char *nx = ni ? realloc(Xx, e * ncap) : NULL;
            if (ni) Xi = ni;
            if (nx) Xx = nx;
            if (!ni || !nx) { ok = 0; oom = 1; break; }
            xcap = ncap;
        }
        ok = c == 0
             || (cudaMemcpyAsync(d_cn, cnt, sizeof(Int) * nseg * w, cudaMemcpyHostToDevice, st) == cudaSuccess
                 && gb_launch_sp_compact(n, w, P->d_B, dt, n, d_cn, d_xi, d_xx, st) == 0
                 && cudaMemcpyAsync(Xi + xnz, d_xi, sizeof(Int) * c, cudaMemcpyDeviceToHost, st) == cudaSuccess
                 && cudaMemcpyAsync(Xx + e * xnz, d_xx, e * c, cudaMemcpyDeviceToHost, st) == cudaSuccess
                 && cudaStreamSynchronize(st) == cudaSuccess);
        xnz += c;
        ctx->launches += 4 + (c > 0);   /* scatter, two permutations, count, compact */
    }
    ctx->stats[1] = dev_ms;
    cholmod_sparse *X = NULL;
    if (ok) {
        Xp[nrhs] = (Int)xnz;
        X = gb300_allocate_sparse(n, nrhs, GB_MAX(xnz, 1), TRUE, TRUE, 0, CHOLMOD_REAL + L->dtype, Common);
        if (X) {
            memcpy(X->p, Xp, sizeof(Int) * (nrhs + 1));
            if (xnz) {
                memcpy(X->i, Xi, sizeof(Int) * xnz);
                memcpy(X->x, Xx, e * xnz);
            }
        }
    } else if (oom) {
        GB_ERROR(CHOLMOD_OUT_OF_MEMORY, "out of memory");
    } else {
        GB_ERROR(CHOLMOD_GPU_PROBLEM, "CUDA error in the sparse solve");
    }
    free(cp); free(cnt); free(mark); free(Xp); free(ci); free(Xi); free(cx); free(Xx);
    return X;
}

/* The factorization task graph of L's plan, 8 int32 per task (type, s, b,
 * r, c, priority, level, 0), for inspecting a factorization trace.  Returns
 * the number of tasks. */
/* The single-launch sweep's task list of L's plan in ticket order (the
 * order of gb300_get_trace): 5 int32 per task: s, kind (0 diagonal block,
 * 1 off-diagonal rows), idx, r0, nr.  Supernodes of leaf subtrees (swept
 * by one warp each in their own launch) have no tasks.  Returns the count. */
int gb300_plan_sweep_tasks(cholmod_factor *L, cholmod_common *Common, int forward, int32_t *out,
                           int64_t nmax)
{
    if (!Common || !L) return -1;
    gb_ctx *ctx = gb_ctx_get(Common, 1);
    if (!ctx || !gb_ctx_ready(ctx)) return -1;
    gb_plan *P = gb_plan_get(L, Common, ctx, 1);
    if (!P) return -1;
    const gb_vec *v = forward ? &P->sf_t : &P->sb_t;
    const gb_stask *t = v->p;
    for (int64_t i = 0; out && i < (int64_t)v->n && i < nmax; i++) {
        out[5 * i + 0] = t[i].s; out[5 * i + 1] = t[i].kind; out[5 * i + 2] = t[i].idx;
        out[5 * i + 3] = t[i].r0; out[5 * i + 4] = t[i].nr;
    }
    return (int)v->n;
}

int gb300_plan_tasks(cholmod_factor *L, cholmod_common *Common, int32_t *out, int64_t nmax)
{
    if (!Common || !L) return -1;
    gb_ctx *ctx = gb_ctx_get(Common, 1);
    if (!ctx || !gb_ctx_ready(ctx)) return -1;
    gb_plan *P = gb_plan_get(L, Common, ctx, 1);
    if (!P) return -1;
    if (ctx->factor_mode == 1) {
        /* the whole-factorization graph, local ids as in the trace */
        const gb_dtask *f = P->fd_t.p;
        int64_t nf = (int64_t)P->fd_t.n;
        for (int64_t i = 0; out && i < nf && i < nmax; i++) {
            out[8 * i + 0] = f[i].type; out[8 * i + 1] = f[i].s; out[8 * i + 2] = f[i].b;
            out[8 * i + 3] = f[i].r; out[8 * i + 4] = f[i].c; out[8 * i + 5] = f[i].prio;
            out[8 * i + 6] = 0; out[8 * i + 7] = 0;
        }
        return (int)nf;
    }
    const gb_dtask *t = P->dag_t.p;
    const gb_dag_level *lv = P->dag_lv.p;
    int64_t n = (int64_t)P->dag_t.n;
    if (out) {
        for (size_t l = 0; l < P->dag_lv.n; l++) {
            for (int32_t q = 0; q < lv[l].ntasks; q++) {
                int64_t i = lv[l].task_off + q;
                if (i >= nmax) break;
                out[8 * i + 0] = t[i].type; out[8 * i + 1] = t[i].s; out[8 * i + 2] = t[i].b;
                out[8 * i + 3] = t[i].r; out[8 * i + 4] = t[i].c; out[8 * i + 5] = t[i].prio;
                out[8 * i + 6] = (int32_t)l; out[8 * i + 7] = 0;
            }
        }
    }
    return (int)n;
}

/* Rough reciprocal condition number of a factor, as the reference defines
 * it (CHOLMOD/Cholesky/cholmod_rcond.c:51-110 and t_cholmod_rcond_worker.c):
 * (min L(j,j) / max L(j,j))^2 for LL' (for LDL', min |D(j,j)| / max
 * |D(j,j)|), 1 for n = 0, 0 when the factorization failed (L->minor < n) or
 * a diagonal entry is NaN, EMPTY for a missing argument.  A supernodal
 * factor whose current values live on the GPU (a factorization with
 * GB300_OPT_KEEP_ON_DEVICE) is reduced there; any other factor is read from
 * L->x on the host, in the reference's order. */
double cholmod_l_rcond(cholmod_factor *L, cholmod_common *Common)
{
    if (!Common) return EMPTY;
    if (!L) { GB_ERROR(CHOLMOD_INVALID, "argument missing"); return EMPTY; }
    if (L->xtype != CHOLMOD_REAL) { GB_ERROR(CHOLMOD_INVALID, "only real factors"); return EMPTY; }
    Common->status = CHOLMOD_OK;
    const Int n = (Int)L->n;
    if (n == 0) return 1;
    if ((Int)L->minor < n) return 0;
    double lmin = 0, lmax = 0;
    int single = L->dtype == CHOLMOD_SINGLE;
    if (L->is_super) {
        gb_ctx *ctx = gb_ctx_get(Common, 0);
        gb_plan *P = ctx ? gb_plan_get(L, Common, ctx, 0) : NULL;
        int d = dt_index(L->dtype);
        if (P && P->dev_valid[d] && P->host_x[d] == L->x && P->d_Lx[d]) {
            size_t cap = 0;
            double r[3];
            int ok = (P->d_red || gb_dev_grow((void **)&P->d_red, &cap, sizeof(double) * 64))
                     && gb_launch_diag_range((int)P->nsuper, P->d_Super, P->d_Pi, P->d_Px, P->d_Lx[d],
                                             single ? 4 : 0, P->d_red, ctx->stream) == 0
                     && cudaMemcpyAsync(r, P->d_red, sizeof r, cudaMemcpyDeviceToHost, ctx->stream) == cudaSuccess
                     && cudaStreamSynchronize(ctx->stream) == cudaSuccess;
            if (!ok) { GB_ERROR(CHOLMOD_GPU_PROBLEM, "CUDA error"); return EMPTY; }
            if (r[2] != 0) return 0;
            lmin = r[0];
            lmax = r[1];
        } else {
            if (!L->x) { GB_ERROR(CHOLMOD_INVALID, "L has no numerical values"); return EMPTY; }
            const Int *Super = L->super, *Pi = L->pi, *Px = L->px;
            for (Int s = 0; s < (Int)L->nsuper; s++) {
                const Int nscol = Super[s + 1] - Super[s], nsrow = Pi[s + 1] - Pi[s];
                for (Int j = 0; j < nscol; j++) {
                    const Int q = Px[s] + j + j * nsrow;
                    const double v = single ? (double)((const float *)L->x)[q] : ((const double *)L->x)[q];
                    if (v != v) return 0;
                    if (s == 0 && j == 0) { lmin = lmax = v; }
                    else if (v < lmin) lmin = v;
                    else if (v > lmax) lmax = v;
                }
            }
        }
    } else {
        /* simplicial factor (produced elsewhere): diagonal at L->x[Lp[j]] */
        const Int *Lp = L->p;
        if (!Lp || !L->x) { GB_ERROR(CHOLMOD_INVALID, "L has no numerical values"); return EMPTY; }
        for (Int j = 0; j < n; j++) {
            double v = single ? (double)((const float *)L->x)[Lp[j]] : ((const double *)L->x)[Lp[j]];
            if (!L->is_ll) v = fabs(v);
            if (v != v) return 0;
            if (j == 0) { lmin = lmax = v; }
            else if (v < lmin) lmin = v;
            else if (v > lmax) lmax = v;
        }
    }
    double rcond = lmin / lmax;
    if (L->is_ll) rcond = rcond * rcond;
    return rcond;
}
