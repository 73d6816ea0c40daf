/* gb_plan.h -- per-pattern GPU plan of the supernodal factorization/sweeps.
 *
 * Everything here depends only on the supernodal pattern (L->super, L->pi,
 * L->px, L->s) and is built once per pattern on the host, uploaded once, and
 * reused by every refactorization and solve with that pattern:
 *   - the supernodal etree (parent, children in increasing order, levels);
 *   - the relative map of each supernode's off-diagonal rows into its
 *     parent's row list (the scatter target of the extend-add);
 *   - offsets of every update block (m^2 entries) and update vector;
 *   - the task lists and the launch sequence of the factorization and of
 *     the two sweeps, level by level.
 */
#ifndef GB_PLAN_H
#define GB_PLAN_H

#include "gb_internal.h"
#include "gb_kernels.cuh"
#include <cuda_runtime.h>

typedef struct {
    const int64_t *Super, *Pi, *Px, *cboff, *cbvoff;
    const int32_t *Ls, *relmap, *child_ptr, *child_list;
    int32_t *fail, *anyfail;
    const int32_t *blkoff;
    const int64_t *linvoff;
    const int64_t *imgbase;          /* first tensor-core operand image of s, -1 if none */
} gb_pattern_ptrs;

enum {
    GB_K_ASM = 1, GB_K_SMALL, GB_K_POTRF, GB_K_TRSM, GB_K_GEMM, GB_K_DAG,
    GB_K_FWD_SMALL, GB_K_FWD_GATHER, GB_K_FWD_DIAG, GB_K_FWD_PANEL,
    GB_K_BWD_SMALL, GB_K_BWD_OFFDIAG, GB_K_BWD_DIAG, GB_K_BWD_PANEL, GB_K_FDAG
};

typedef struct { int32_t kind, count; int64_t off; } gb_launch_rec;

/* one level's task graph inside the plan's concatenated arrays */
typedef struct {
    int64_t task_off, sp_off, succ_off, q0_off, q1_off;
    int32_t ntasks, n0, n1, total0, total1, pad;
} gb_dag_level;

/* arguments of the task-graph executor (device pointers of one level) */
typedef struct {
    const gb_dtask *tasks;
    int ntasks;
    const int32_t *succ_ptr, *succ;
    int32_t *cnt, *q0, *q1, *ctrl;
    int32_t *err;            /* persistent error word of the factorization */
    unsigned long long *trace;
    int32_t *smflag;         /* [GB_DAG_NSMF] launch epoch of the SM's poller */
    int32_t epoch;           /* distinct per launch, nonzero */
} gb_dag_args;

/* Whole-factorization task graph (one persistent launch for every level):
 * a pattern's local task list and successor CSR, and instances of it (one
 * per independent system of a batch; a single matrix is one instance), each
 * with its own value offsets, failure flags and global task-id base. */
typedef struct {
    gb_pattern_ptrs pp;              /* device pattern arrays */
    const gb_dtask *tasks;           /* local tasks */
    const int32_t *succ_ptr, *succ;  /* local successor CSR */
    const int64_t *Sp, *Si;          /* S = tril(PAP') column pointers/indices */
    const int32_t *sub_list;         /* supernodes of the SUBTREE tasks, wave by wave */
    const int32_t *sub_meta;         /* [3 per sub_list entry] at a wave's first entry:
                                      * ends of its fronts of <= 32 rows, of <= warp_rows
                                      * rows, and of the wave (relative to the task's
                                      * first entry) */
    int32_t ntasks, warp_rows;       /* fronts with at most warp_rows rows: one warp */
} gb_fpat;

typedef struct {
    int32_t pat, pad;
    int64_t base;                    /* global id of local task 0 */
    int64_t lx, cb, linv, sx, scale; /* element offsets into the value buffers */
    int32_t *fail, *anyfail;         /* [nsuper], [1] of this instance */
} gb_finst;

typedef struct {
    const gb_fpat *pats;             /* device */
    const gb_finst *inst;            /* device */
    const int64_t *inst_base;        /* device [ninst], ascending */
    int32_t ninst;
    int64_t ntotal;                  /* tasks over all instances */
    int32_t *cnt, *q0, *q1, *ctrl, *err, *smflag;
    int32_t epoch;
    unsigned long long *trace;
    const void *Sx;                  /* values of S (dtype a_dtype) */
    int a_dtype;                     /* 0 double, 4 single */
    const double *scale;             /* optional D A D scaling */
    double beta;
    int use_tc;                      /* FP32 tile products on the tensor cores */
    float *img;                      /* their operand images (GB_IMG_FLOATS each) */
    int npoll;                       /* blocks that serve only the critical queue (0: every
                                      * block serves it while it waits for bulk work) */
} gb_fdag_args;

/* right-hand-side columns per single-launch sweep pass, and passes that run
 * at once on their own streams */
#define GB_SWEEP_COLS 16
#define GB_SWEEP_STREAMS 4
#define GB_LEAF_MEMBERS 256        /* supernodes of a sweep leaf subtree */
#define GB_LEAF_ROWS 128           /* rows of a front in a sweep leaf subtree (one
                                    * diagonal block: at most 64 columns) */

/* a chunk of rows of one segment, for segmented reductions */
typedef struct { int64_t lo, hi; int32_t seg, pad; } gb_seg_chunk;
#define GB_SEG_CHUNK 4096

/* arguments of the single-launch sweeps (device pointers) */
typedef struct {
    const gb_stask *tasks;
    int ntasks;
    const int32_t *gptr;        /* [ngroups+1]: tickets name groups of consecutive tasks */
    int ngroups;
    const int32_t *blkoff;
    const int64_t *linvoff;
    const int32_t *ntask_s;
    const int32_t *parent;
    int32_t *xready, *done, *ticket, *err;
    unsigned long long *trace;
    const int32_t *cptr;        /* forward: [ntasks+1] start of each task's child ranges */
    const int32_t *crange;      /* forward: per task and child (child_list order) the
                                 * child's update-vector rows [a, b) in the task's rows */
    const int32_t *bchunk_ptr, *bchunk; /* backward: the block each row chunk waits for */
    const unsigned char *act;   /* optional [nseg]: 0 = skip the segment's tasks */
    const int32_t *sseg;        /* [nsuper] segment of each supernode (with act) */
} gb_sweep1_args;

/* growable host array */
typedef struct { void *p; size_t n, cap, esz; } gb_vec;

typedef struct gb_plan {
    /* identity of the pattern this plan was built for */
    const cholmod_factor *L;
    const void *super_ptr, *s_ptr, *pi_ptr;
    Int n, nsuper, ssize, xsize;
    Int small_cols;                   /* widest supernode factored whole by one block */
    double sub_work;                  /* work limit of a SUBTREE task (0: none) */
    Int warp_rows;                    /* fronts this tall or less run on one warp (0: none) */
    Int upd_group;                    /* panels whose trailing updates run at once (1..GB_UPD_GROUP) */
    uint64_t hash;

    /* host arrays derived from the pattern (kept for the plan's lifetime) */
    int32_t *h_child_ptr, *h_child_list, *h_relmap;
    int64_t *h_cboff, *h_cbvoff;

    int nlevels;
    int64_t cb_total, cbv_total;      /* entries of all update blocks/vectors */
    double fl_gemm;                   /* algorithmic flops of the tile updates */
    double fl_dag;                    /* algorithmic flops of the task graphs */

    /* host task arrays and launch sequences */
    gb_vec asm_t, node_t, potrf_t, trsm_t, gemm_t, gemm_owner, sweep_t;
    gb_vec fact_seq, fwd_seq, bwd_seq;

    /* device copies */
    int64_t *d_Super, *d_Pi, *d_Px, *d_cboff, *d_cbvoff, *d_Perm;
    int32_t *d_Ls, *d_relmap, *d_child_ptr, *d_child_list, *d_fail, *d_anyfail;
    gb_asm_task *d_asm;
    gb_node_task *d_node;
    gb_potrf_task *d_potrf;
    gb_trsm_task *d_trsm;
    gb_gemm_task *d_gemm;
    int32_t *d_gemm_owner;
    gb_sweep_task *d_sweep;
    gb_pattern_ptrs ptrs;

    /* per-level task graphs of the factorization */
    gb_vec dag_t, dag_sp, dag_succ, dag_nd, dag_q0, dag_q1, dag_lv;
    int32_t dag_max;
    gb_dtask *d_dag_t;
    int32_t *d_dag_sp, *d_dag_succ, *d_dag_nd, *d_dag_q0i, *d_dag_q1i, *d_dag_ctrl0;
    int32_t *d_dag_cnt, *d_dag_q, *d_dag_ctrl, *d_dag_smf;
    int32_t dag_epoch;

    /* whole-factorization task graph (local ids: level-graph tasks, then
     * assembly chunks, small supernodes, and two joins per supernode) */
    gb_vec fd_t, fd_sp, fd_succ, fd_nd, fd_q0, fd_q1, fd_sub, fd_smeta;
    int32_t fd_total0, fd_total1;
    int fd_spread;                   /* no elimination tree holds 5 % of the work (a batch):
                                      * no dedicated pollers (gb_fdag_args.npoll = 0) */
    gb_dtask *d_fd_t;
    int32_t *d_fd_sp, *d_fd_succ, *d_fd_nd, *d_fd_qi, *d_fd_ctrl0;
    int32_t *d_fd_cnt, *d_fd_q, *d_fd_sub, *d_fd_smeta;
    gb_fpat h_fd_pat;                 /* host copy, refreshed per factorization */
    gb_fpat *d_fd_pat;
    gb_finst *d_fd_inst;
    int64_t *d_fd_ibase;

    /* single-launch sweeps: tasks, diagonal-block inverses, flags */
    gb_vec sf_t, sb_t, sd_t;          /* forward, backward, diagonal-block tasks */
    gb_vec lf_t;                      /* leaf subtrees of the sweeps: (first, root) */
    int leaf_rows;                    /* most rows of a front in a leaf subtree */
    int32_t *d_lf;
    gb_vec sf_cptr, sf_crange;        /* forward tasks' child row ranges (gb_sweep1_args) */
    int32_t *d_sf_cptr, *d_sf_crange;
    int64_t nblk_total, linv_total;
    gb_stask *d_sf, *d_sb, *d_sd;
    gb_vec gf, gb;                    /* sweep task groups (forward, backward) */
    int32_t *d_gf, *d_gb;
    int32_t *d_blkoff, *d_ntask_f, *d_ntask_b, *d_parent;
    int32_t *h_bchunk_ptr, *h_bchunk, *d_bchunk_ptr, *d_bchunk; /* backward sweep: per supernode
                                      * and 64-row chunk below its diagonal, the block of the
                                      * chunk's first row */
    int64_t *d_linvoff;
    int32_t *d_xready, *d_done, *d_ticket, *d_err;
    int32_t *h_blkoff, *h_ntask_f, *h_ntask_b, *h_parent;
    int64_t *h_linvoff;
    void *d_Linv[2];
    int linv_valid[2];

    /* split operand images of the tensor-core tile products (FP32): per
     * supernode with tile tasks, one per panel b and 64-row block r >= b
     * (written by the panel solves, read by bulk copies) */
    int64_t *h_imgbase, *d_imgbase;
    int64_t img_total;                /* images (GB_IMG_FLOATS floats each) */

    /* numeric buffers, [0] double, [1] single */
    void *d_Lx[2];
    int dev_valid[2];                 /* device factor holds the last result */
    const void *host_x[2];            /* L->x that the device factor mirrors */

    /* inputs and sweep workspace */
    int64_t *d_Sp, *d_Si;
    void *d_Sx;
    size_t struct_bytes;               /* device bytes of the uploaded plan structures */
    size_t vm_bytes;                   /* device bytes of the value maps */
    size_t sx_cap, si_cap, sp_cap;
    void *d_Y, *d_U, *d_B;
    size_t y_cap, u_cap, b_cap;
    void *d_spw;                      /* cholmod_l_spsolve: B chunk, counts, X chunk */
    size_t spw_cap;
    int32_t *d_sws;                   /* dependency words of concurrent sweep passes */
    size_t sws_cap;

    /* full (both triangles) FP64 copy of A for residuals, plus scaling */
    int64_t *d_Rp;
    int32_t *d_Rj;
    /* value maps of the caller's A (gb_valmap.c) */
    int vm_valid, vm_packed, s_from_vm;
    int64_t vm_n, vm_xlen, vm_snz, vm_rnz;
    int64_t *h_vm_Ap, *h_vm_Ai, *h_vm_Anz, *h_vm_Sp, *h_vm_Si;
    int64_t *d_smap, *d_rmap, *d_dmap;
    double *d_Ax;
    size_t ax_cap;
    double *d_Rx, *d_scale, *d_scale_perm, *d_X, *d_R, *d_bx, *d_red;
    size_t rp_cap, rj_cap, rx_cap, x_cap, r_cap, bx_cap;
    uint64_t a_hash;
    int mixed;                        /* 0 none, 1 FP32 factor, 2 FP64 factor */
    int mixed_reason;                 /* why the FP64 factor was used */
    double anorm;                     /* |A|_inf of the refined system */
    /* independent blocks of A (trees of the supernodal etree) when each is a
     * contiguous range of original rows; else one segment of all rows.  The
     * refinement measures the backward error per segment and column. */
    int64_t nseg, nchunk;
    int64_t *h_seg;                   /* [nseg+1] row ranges */
    gb_seg_chunk *h_chunk;            /* row chunks of at most GB_SEG_CHUNK rows */
    gb_seg_chunk *d_chunk;
    double *h_anorm_seg, *d_anorm_seg, *d_bred;
    int32_t *h_sseg, *d_sseg;         /* nseg > 1: [nsuper] segment of each supernode */
    unsigned char *h_segact, *d_segact; /* [nseg] refinement: segment not yet converged */
    const unsigned char *sweep_act;   /* set during refinement steps: sweeps skip the
                                       * segments it marks 0 */
    int anorm_pinned;                 /* h_anorm_seg from cudaMallocHost */
    size_t bred_cap;
    /* CUDA graph of one refinement step (gb_mixed.c), per pattern: valid
     * for the right-hand-side count, factor precision and buffers it was
     * captured with */
    void *g_exec;
    int g_nrhs, g_single;
    int64_t g_launches;               /* kernel launches one replay makes */
    const void *g_bufs[9];

    struct gb_plan *next;             /* side-table chaining */
} gb_plan;

#ifdef __cplusplus
extern "C" {
#endif

/* per-Common library state (defined here for the drivers in gb_numeric.c
 * and gb_mixed.c) */
struct gb_ctx {
    cudaStream_t stream;
    int device;
    int64_t opt_keep, opt_small;
    double opt_subwork;                /* SUBTREE task work limit for new plans */
    int64_t opt_warprows;              /* one-warp front height limit for new plans */
    int64_t opt_updgroup;              /* grouped trailing updates of new plans */
    /* scratch of a factorization, grown as needed and reused by every
     * factor this Common factorizes (resident factors do not hold it):
     * update blocks per precision and the tensor-core operand images */
    void *d_cbs[2];
    size_t cbs_cap[2];
    void *d_imgs;
    size_t imgs_cap;
    int opt_autotune;                  /* 1 = the first super_numeric tunes the plan options */
    int tuned;                         /* the automatic tuning ran on this Common */
    double stats[8];
    int64_t launches;            /* kernel launches issued since creation */
    cudaEvent_t ev0, ev1;
    /* optional per-launch timing of the factorization (gb300_set_option
     * GB300_OPT_PROFILE): events around every launch, summed per kind */
    int prof;
    int sweep_mode;              /* 1 = single-launch sweeps (default), 0 = per level */
    int factor_mode;             /* 1 = one whole-factorization launch (default), 0 = per level */
    int tc_mode;                 /* 1 = FP32 tile products on the tensor cores (default) */
    int pivot_log2;              /* small-pivot threshold of the FP32 factor: 2^-pivot_log2 */
    int trace_on;                /* record per-task times of the sweeps */
    int graph_mode;              /* 1 = refinement steps replayed from a CUDA graph (default) */
    int sweep_streams;           /* passes of 16 columns run at once (1..GB_SWEEP_STREAMS) */
    unsigned long long *d_trace; /* device trace buffer (3 x tasks) */
    size_t trace_cap;
    int64_t trace_n[2];          /* tasks traced by the last forward/backward sweep */
    int64_t trace_off[2];
    unsigned long long *d_ftrace;  /* factorization task trace */
    size_t ftrace_cap;
    int64_t ftrace_n;
    int sms;
    cudaEvent_t *pev;
    int npev;
    /* concurrent sweep passes (more than GB_SWEEP_COLS right-hand sides):
     * side streams, fork and join events; side_ok 1 ready, -1 failed */
    cudaStream_t side[GB_SWEEP_STREAMS - 1];
    cudaEvent_t ev_fork, ev_join[GB_SWEEP_STREAMS - 1];
    int side_ok;
    double kind_ms[16], kind_n[16];
};

int gb_vec_push(gb_vec *v, const void *e);
void gb_vec_free(gb_vec *v);

/* Build the plan (host side) for a supernodal symbolic factor. */
/* Values of the caller's A to the device through the pattern's maps (built
 * on first use or pattern change; FALSE: use the host path).  With
 * deferred != NULL, a packed A of the maps' shape skips the comparison of
 * its pattern (*deferred = 1): the caller runs gb_valmap_verify while the
 * device works and redoes the work if it fails.  gb_valmap_anorm forms
 * P->anorm once the stream has been synchronized. */
int gb_valmap_apply(gb_plan *P, gb_ctx *ctx, cholmod_sparse *A, cholmod_common *Common,
                    int *deferred);
int gb_valmap_verify(const gb_plan *P, const cholmod_sparse *A);
void gb_valmap_anorm(gb_plan *P);
void gb_valmap_free(gb_plan *P);
void gb_graph_free(gb_plan *P);     /* gb_mixed.c */
gb_plan *gb_plan_build(const cholmod_factor *L, int64_t small_cols, double sub_work,
                       int64_t warp_rows, int64_t upd_group);
size_t gb_plan_device_bytes(const gb_plan *P);
/* Upload the pattern, task arrays and launch sequences. */
int gb_plan_upload(gb_plan *P);
void gb_plan_free(gb_plan *P);
uint64_t gb_pattern_hash(const cholmod_factor *L);

/* drivers shared by gb_numeric.c and gb_mixed.c */
int gb_ctx_ready(gb_ctx *c);
gb_plan *gb_plan_get(cholmod_factor *L, cholmod_common *Common, gb_ctx *ctx, int create);
int gb_dev_grow(void **p, size_t *cap, size_t bytes);
int gb_ensure_numeric(gb_plan *P, int dtype);
int gb_run_factor(gb_plan *P, gb_ctx *ctx, const void *Sx, int a_dtype, int l_dtype,
                  const double *scale, double beta);
int gb_run_sweep(gb_plan *P, gb_ctx *ctx, int l_dtype, int nrhs, void *Y, int forward);
int gb_run_inverse(gb_plan *P, gb_ctx *ctx, int l_dtype);
int gb_fix_not_posdef(gb_plan *P, gb_ctx *ctx, cholmod_factor *L, int l_dtype,
                      cholmod_common *Common);
int gb_upload_input(gb_plan *P, gb_ctx *ctx, cholmod_sparse *A, int a_dtype);

/* kernel launchers (gb_kernels.cu); dtype 0 = double, 4 = single; each
 * enqueues on st and returns the cudaError_t of the launch as int */
int gb_launch_assemble(const gb_pattern_ptrs *pp, const gb_asm_task *tasks, int ntasks,
                       const int64_t *Sp, const int64_t *Si, const void *Sx, int a_dtype,
                       const double *scale, double beta, void *Lx, void *CB, int l_dtype,
                       cudaStream_t st);
int gb_launch_factor_small(const gb_pattern_ptrs *pp, const gb_node_task *tasks, int ntasks,
                           void *Lx, void *Linv, int dtype, cudaStream_t st);
int gb_launch_potrf_diag(const gb_pattern_ptrs *pp, const gb_potrf_task *tasks, int ntasks,
                         void *Lx, void *Linv, int dtype, cudaStream_t st);
int gb_launch_trsm_rows(const gb_pattern_ptrs *pp, const gb_trsm_task *tasks, int ntasks,
                        void *Lx, const void *Linv, int dtype, cudaStream_t st);
int gb_launch_gemm(const gb_pattern_ptrs *pp, const gb_gemm_task *tasks, const int32_t *owner,
                   int ntasks, void *Lx, void *CB, int dtype, cudaStream_t st);
int gb_launch_sweep_node(int kind, const gb_pattern_ptrs *pp, const gb_node_task *tasks,
                         int ntasks, const void *Lx, int dtype, int nrhs, void *Y,
                         int64_t ldy, void *U, cudaStream_t st);
int gb_launch_sweep_step(int kind, const gb_pattern_ptrs *pp, const gb_sweep_task *tasks,
                         int ntasks, const void *Lx, int dtype, int nrhs, void *Y,
                         int64_t ldy, void *U, cudaStream_t st);
int gb_launch_perm_in(int64_t n, int nrhs, const int64_t *perm, const double *scale,
                      const void *B, int b_dtype, int64_t ldb, void *Y, int y_dtype,
                      int64_t ldy, cudaStream_t st);
int gb_launch_perm_out(int64_t n, int nrhs, const int64_t *perm, const double *scale,
                       const void *Y, int y_dtype, int64_t ldy, void *X, int x_dtype,
                       int64_t ldx, int add, cudaStream_t st);
int gb_launch_sp_scatter(int64_t n, int64_t ncol, const int64_t *Bp, const int64_t *Bi,
                         const void *Bx, int dtype, void *Y, int64_t ldy, cudaStream_t st);
int64_t gb_sp_nseg(int64_t n);
int gb_launch_sp_count(int64_t n, int64_t ncol, const void *X, int dtype, int64_t ldx,
                       int64_t *cnt, cudaStream_t st);
int gb_launch_sp_compact(int64_t n, int64_t ncol, const void *X, int dtype, int64_t ldx,
                         const int64_t *off, int64_t *Xi, void *Xx, cudaStream_t st);
int gb_launch_residual(int64_t n, int nrhs, const int64_t *Rp, const int32_t *Rj,
                       const double *Rx, const double *X, int64_t ldx, const double *B,
                       int64_t ldb, double *R, int64_t ldr, cudaStream_t st);
int gb_launch_colmax3(int64_t n, int nrhs, const double *R, int64_t ldr, const double *X,
                      int64_t ldx, const double *B, int64_t ldb, double *out, cudaStream_t st);
int gb_launch_anorm(int64_t n, const int64_t *Rp, const double *Rx, double *out, cudaStream_t st);
int gb_launch_gather(int64_t n, const int64_t *map, const double *src, double *dst, cudaStream_t st);
int gb_launch_diag_scale(int64_t n, const int64_t *dmap, const double *Ax, const int64_t *Perm,
                         double *scale, double *scale_perm, cudaStream_t st);
int gb_launch_anorm_seg(int64_t nchunk, const gb_seg_chunk *chunks, int64_t nseg, const int64_t *Rp,
                        const double *Rx, double *out, cudaStream_t st);
/* R(rows of the segments act marks 0, every column) = 0 */
int gb_launch_zero_inactive(int64_t nchunk, const gb_seg_chunk *chunks, const unsigned char *act,
                            double *R, int64_t ldr, int nrhs, cudaStream_t st);
int gb_launch_colmax3_seg(int64_t nchunk, const gb_seg_chunk *chunks, int64_t nseg, int nrhs,
                          const double *R, int64_t ldr, const double *X, int64_t ldx,
                          const double *B, int64_t ldb, double *out, cudaStream_t st);
int gb_launch_diag_range(int nsuper, const int64_t *Super, const int64_t *Pi,
                         const int64_t *Px, const void *Lx, int dtype, double *out,
                         cudaStream_t st);
int gb_launch_diag_minmax(int nsuper, const int64_t *Super, const int64_t *Pi,
                          const int64_t *Px, const void *Lx, int dtype, double *out,
                          cudaStream_t st);
int gb_launch_fma_peak(int dtype, int iters, int blocks, float *ms, cudaStream_t st);
int gb_launch_fdag(const gb_fdag_args *a, void *Lx, void *CB, void *Linv, int dtype, int grid,
                   cudaStream_t st);
int gb_launch_dag(const gb_pattern_ptrs *pp, const gb_dag_args *a, void *Lx, void *CB,
                  void *Linv, int dtype, int grid, cudaStream_t st);
int gb_launch_sweep1(int forward, const gb_pattern_ptrs *pp, const gb_sweep1_args *a,
                     const void *Lx, const void *Linv, int dtype, int nrhs, void *Y,
                     int64_t ldy, void *U, int grid, cudaStream_t st);
int gb_launch_sweep_leaf(int forward, const gb_pattern_ptrs *pp, const int32_t *leaf, int nleaf,
                         const int32_t *blkoff, const int64_t *linvoff, const int32_t *ntask_f,
                         int32_t *done, int32_t *ticket, const void *Lx, const void *Linv,
                         int dtype, int nrhs, void *Y, int64_t ldy, void *U, int grid, int lrows,
                         const unsigned char *act, const int32_t *sseg, cudaStream_t st);
int gb_launch_diag_inverse(const gb_pattern_ptrs *pp, const gb_stask *dtasks, int ndiag,
                           const int32_t *blkoff, const int64_t *linvoff, const void *Lx,
                           void *Linv, int dtype, cudaStream_t st);
int gb_launch_zero_range(void *x, int dtype, int64_t from, int64_t to, cudaStream_t st);
gb_plan *gb_factor_device_only(cholmod_sparse *S, double beta, cholmod_factor *FS, int dtype,
                               int64_t *minor, cholmod_common *Common);
int gb_launch_pair_sum(int64_t nent, const int64_t *pptr, const int64_t *pairs, const void *Ax,
                       const void *Fx, void *Cx, int dtype, cudaStream_t st);
int gb_launch_simplicial_gather(int64_t n, const int64_t *src, const int64_t *dst,
                                const int64_t *len, int64_t minor, int ldl, const void *Fx,
                                void *Lx, int dtype, cudaStream_t st);
int gb_launch_cx_gather(int64_t nsuper, const int64_t *Super_e, const int64_t *Pi_e,
                        const int64_t *Px_e, const void *E, void *Lx, int64_t zero_from, int dtype,
                        cudaStream_t st);
int gb_launch_cx_scatter(int64_t nsuper, const int64_t *Super_e, const int64_t *Pi_e,
                         const int64_t *Px_e, const void *Lx, void *E, int dtype, cudaStream_t st);
gb_plan *gb_numeric_core(cholmod_sparse *A, cholmod_sparse *F, double beta, cholmod_factor *FL,
                         int dtype, int cx_diag, int32_t *anyfail, gb_ctx **pctx,
                         cholmod_common *Common);

#ifdef __cplusplus
}
#endif

#endif
