/* cholmod_gb300.h -- GB300 (sm_103a) supernodal numeric Cholesky behind the
 * CHOLMOD C API.
 *
 * Two groups of declarations:
 *
 * 1. The CHOLMOD objects this library reads and writes (cholmod_common,
 *    cholmod_sparse, cholmod_factor, cholmod_dense) and the three CHOLMOD
 *    entry points it replaces.  The struct layouts must be byte-identical to
 *    CHOLMOD 5.3 built for int64 (cholmod_l_*) so that a program linked
 *    against the reference CHOLMOD can pass its own objects to this library:
 *    every member below has the type and position of the member of the same
 *    name in CHOLMOD/Include/cholmod.h (cholmod_common :501-999,
 *    cholmod_sparse :1168-1206, cholmod_factor :1539-1653, cholmod_dense
 *    :1802-1813), and tests/test_abi.py checks every offset against that
 *    header when the reference sources are present.  When this header and
 *    cholmod.h are both visible in one translation unit, include cholmod.h
 *    only (define CHOLMOD_GB300_USE_CHOLMOD_H before including this file).
 *
 * 2. gb300_* extensions: the host-side drivers a standalone program needs
 *    (symbolic analysis from a given permutation, the factorize/solve
 *    wrappers), the FP32-factor + FP64-refinement solver, and plain-pointer
 *    entry points for foreign-function callers.
 *
 * All functions are extern "C", take plain pointers and sizes, and report
 * errors the CHOLMOD way: TRUE/FALSE or NULL return, Common->status set,
 * Common->error_handler called unless Common->try_catch.
 */
#ifndef CHOLMOD_GB300_H
#define CHOLMOD_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#ifndef CHOLMOD_GB300_USE_CHOLMOD_H

/* ---- constants with the reference's values (cholmod.h) ---------------- */
#define CHOLMOD_PATTERN 0
#define CHOLMOD_REAL    1
#define CHOLMOD_COMPLEX 2
#define CHOLMOD_ZOMPLEX 3
#define CHOLMOD_DOUBLE  0
#define CHOLMOD_SINGLE  4
#define CHOLMOD_INT     0
#define CHOLMOD_LONG    2

#define CHOLMOD_OK            (0)
#define CHOLMOD_NOT_INSTALLED (-1)
#define CHOLMOD_OUT_OF_MEMORY (-2)
#define CHOLMOD_TOO_LARGE     (-3)
#define CHOLMOD_INVALID       (-4)
#define CHOLMOD_GPU_PROBLEM   (-5)
#define CHOLMOD_NOT_POSDEF    (1)
#define CHOLMOD_DSMALL        (2)

#define CHOLMOD_SIMPLICIAL 0
#define CHOLMOD_AUTO       1
#define CHOLMOD_SUPERNODAL 2

#define CHOLMOD_NATURAL     0
#define CHOLMOD_GIVEN       1
#define CHOLMOD_AMD         2
#define CHOLMOD_METIS       3
#define CHOLMOD_NESDIS      4
#define CHOLMOD_COLAMD      5
#define CHOLMOD_POSTORDERED 6
#define CHOLMOD_MAXMETHODS  9

#define CHOLMOD_A    0
#define CHOLMOD_LDLt 1
#define CHOLMOD_LD   2
#define CHOLMOD_DLt  3
#define CHOLMOD_L    4
#define CHOLMOD_Lt   5
#define CHOLMOD_D    6
#define CHOLMOD_P    7
#define CHOLMOD_Pt   8

#define CHOLMOD_HOST_SUPERNODE_BUFFERS 8

/* ---- cholmod_common: parameters, statistics, workspace ----------------- */
typedef struct cholmod_common_struct
{
    double dbound ;
    double grow0 ;
    double grow1 ;
    size_t grow2 ;
    size_t maxrank ;
    double supernodal_switch ;
    int supernodal ;
    int final_asis ;
    int final_super ;
    int final_ll ;
    int final_pack ;
    int final_monotonic ;
    int final_resymbol ;
    double zrelax [3] ;
    size_t nrelax [3] ;
    int prefer_zomplex ;
    int prefer_upper ;
    int quick_return_if_not_posdef ;
    int prefer_binary ;
    int print ;
    int precise ;
    int try_catch ;
    void (*error_handler) (int status, const char *file, int line,
        const char *message) ;
    int nmethods ;
    int current ;
    int selected ;
    struct cholmod_method_struct
    {
        double lnz ;
        double fl ;
        double prune_dense ;
        double prune_dense2 ;
        double nd_oksep ;
        double other_1 [4] ;
        size_t nd_small ;
        double other_2 [4] ;
        int aggressive ;
        int order_for_lu ;
        int nd_compress ;
        int nd_camd ;
        int nd_components ;
        int ordering ;
        size_t other_3 [4] ;
    } method [CHOLMOD_MAXMETHODS + 1] ;
    int postorder ;
    int default_nesdis ;
    double metis_memory ;
    double metis_dswitch ;
    size_t metis_nswitch ;
    size_t nrow ;
    int64_t mark ;
    size_t iworksize ;
    size_t xworkbytes ;
    void *Flag ;
    void *Head ;
    void *Xwork ;
    void *Iwork ;
    int itype ;
    int other_5 ;
    int no_workspace_reallocate ;
    int status ;
    double fl ;
    double lnz ;
    double anz ;
    double modfl ;
    size_t malloc_count ;
    size_t memory_usage ;
    size_t memory_inuse ;
    double nrealloc_col ;
    double nrealloc_factor ;
    double ndbounds_hit ;
    double rowfacfl ;
    double aatfl ;
    int called_nd ;
    int blas_ok ;
    double SPQR_grain ;
    double SPQR_small ;
    int SPQR_shrink ;
    int SPQR_nthreads ;
    double SPQR_flopcount ;
    double SPQR_analyze_time ;
    double SPQR_factorize_time ;
    double SPQR_solve_time ;
    double SPQR_flopcount_bound ;
    double SPQR_tol_used ;
    double SPQR_norm_E_fro ;
    int64_t SPQR_istat [8] ;
    double nsbounds_hit ;
    float sbound ;
    float other_6 ;
    int useGPU ;
    size_t maxGpuMemBytes ;
    double maxGpuMemFraction ;
    size_t gpuMemorySize ;
    double gpuKernelTime ;
    int64_t gpuFlops ;
    int gpuNumKernelLaunches ;
    void *cublasHandle ;
    void *gpuStream [CHOLMOD_HOST_SUPERNODE_BUFFERS] ;
    void *cublasEventPotrf [3] ;
    void *updateCKernelsComplete ;
    void *updateCBuffersFree [CHOLMOD_HOST_SUPERNODE_BUFFERS] ;
    void *dev_mempool ;
    size_t dev_mempool_size ;
    void *host_pinned_mempool ;
    size_t host_pinned_mempool_size ;
    size_t devBuffSize ;
    int    ibuffer ;
    double syrkStart ;
    double cholmod_cpu_gemm_time ;
    double cholmod_cpu_syrk_time ;
    double cholmod_cpu_trsm_time ;
    double cholmod_cpu_potrf_time ;
    double cholmod_gpu_gemm_time ;
    double cholmod_gpu_syrk_time ;
    double cholmod_gpu_trsm_time ;
    double cholmod_gpu_potrf_time ;
    double cholmod_assemble_time ;
    double cholmod_assemble_time2 ;
    size_t cholmod_cpu_gemm_calls ;
    size_t cholmod_cpu_syrk_calls ;
    size_t cholmod_cpu_trsm_calls ;
    size_t cholmod_cpu_potrf_calls ;
    size_t cholmod_gpu_gemm_calls ;
    size_t cholmod_gpu_syrk_calls ;
    size_t cholmod_gpu_trsm_calls ;
    size_t cholmod_gpu_potrf_calls ;
    double chunk ;
    int nthreads_max ;
} cholmod_common ;

/* ---- cholmod_sparse: compressed-column matrix -------------------------- */
typedef struct cholmod_sparse_struct
{
    size_t nrow ;
    size_t ncol ;
    size_t nzmax ;
    void *p ;       /* column pointers, size ncol+1 */
    void *i ;       /* row indices, size nzmax */
    void *nz ;      /* column counts if unpacked */
    void *x ;       /* values */
    void *z ;
    int stype ;     /* 0 unsymmetric, >0 upper stored, <0 lower stored */
    int itype ;
    int xtype ;
    int dtype ;
    int sorted ;
    int packed ;
} cholmod_sparse ;

/* ---- cholmod_factor: the supernodal layout consumed and produced ------- *
 * super[nsuper+1]: first column of each supernode; pi[nsuper+1]: start of
 * each supernode's row list in s; px[nsuper+1]: start of each supernode's
 * values in x; s[ssize]: row indices (the first nscol rows of supernode s are
 * its own columns super[s]..super[s+1]-1); x[xsize]: values, supernode s is
 * an nsrow-by-nscol column-major block with leading dimension nsrow.       */
typedef struct cholmod_factor_struct
{
    size_t n ;
    size_t minor ;
    void *Perm ;
    void *ColCount ;
    void *IPerm ;
    size_t nzmax ;
    void *p ;
    void *i ;
    void *x ;
    void *z ;
    void *nz ;
    void *next ;
    void *prev ;
    size_t nsuper ;
    size_t ssize ;
    size_t xsize ;
    size_t maxcsize ;
    size_t maxesize ;
    void *super ;
    void *pi ;
    void *px ;
    void *s ;
    int ordering ;
    int is_ll ;
    int is_super ;
    int is_monotonic ;
    int itype ;
    int xtype ;
    int dtype ;
    int useGPU ;
} cholmod_factor ;

/* ---- cholmod_dense: column-major dense matrix --------------------------- */
typedef struct cholmod_dense_struct
{
    size_t nrow ;
    size_t ncol ;
    size_t nzmax ;
    size_t d ;
    void *x ;
    void *z ;
    int xtype ;
    int dtype ;
} cholmod_dense ;

#endif /* CHOLMOD_GB300_USE_CHOLMOD_H */

/* ======================================================================== *
 * 1. Drop-in boundary: the CHOLMOD entry points this library replaces.     *
 * ======================================================================== */

/* Supernodal numeric LL' of A+beta*I (A = tril(PAP'), stype < 0) on the GPU.
 * Replaces CHOLMOD/Supernodal/cholmod_super_numeric.c:100-335 (declared at
 * CHOLMOD/Include/cholmod.h:4016-4027); called by cholmod_l_factorize_p at
 * CHOLMOD/Cholesky/cholmod_factorize.c:260.  Same contract: L symbolic or
 * numeric supernodal on input, numeric on output with L->x filled (unless
 * the factor is kept device-resident, see gb300_set_option), is_ll = TRUE,
 * L->minor = n on success.  Not positive definite: returns TRUE with
 * Common->status = CHOLMOD_NOT_POSDEF, L->minor = the failing column, that
 * supernode factorized only up to the failing column and all later
 * supernodes zero (quick_return_if_not_posdef: the failing supernode is
 * left zero).  Real double and real single are supported; complex/zomplex
 * input returns FALSE with CHOLMOD_INVALID.  The unsymmetric form (A with
 * stype 0, n x k, and F = A' or A(:,f)', k x n; the matrix
 * cholmod_factorize_p passes for an unsymmetric A) factorizes beta I + A F:
 * the pattern of tril(A F) and, per entry, its list of products are formed
 * on the host, the products summed on the device in the reference's order
 * (t_cholmod_super_numeric_worker.c:471-506), then the factorization runs
 * as for a symmetric-lower input. */
int cholmod_l_super_numeric (cholmod_sparse *A, cholmod_sparse *F,
    double beta [2], cholmod_factor *L, cholmod_common *Common) ;

/* Forward supernodal solve X = L\X on the GPU.  Replaces
 * CHOLMOD/Supernodal/cholmod_super_solve.c:52-139 (cholmod.h:4037); called by
 * cholmod_l_solve2 at CHOLMOD/Cholesky/cholmod_solve.c:698.  X is n-by-nrhs
 * with leading dimension X->d; E must be at least nrhs*L->maxesize entries
 * (checked as in the reference, not otherwise used). */
int cholmod_l_super_lsolve (cholmod_factor *L, cholmod_dense *X,
    cholmod_dense *E, cholmod_common *Common) ;

/* Backward supernodal solve X = L'\X on the GPU.  Replaces
 * CHOLMOD/Supernodal/cholmod_super_solve.c:153-240 (cholmod.h:4058); called
 * by cholmod_l_solve2 at CHOLMOD/Cholesky/cholmod_solve.c:699. */
int cholmod_l_super_ltsolve (cholmod_factor *L, cholmod_dense *X,
    cholmod_dense *E, cholmod_common *Common) ;

/* Simplicial numeric LL' or LDL' factorization on the GPU.  Replaces
 * CHOLMOD/Cholesky/cholmod_rowfac.c:588-604 (cholmod_l_rowfac); called by
 * cholmod_l_factorize_p for the simplicial method at
 * CHOLMOD/Cholesky/cholmod_factorize.c:393.  A is triu(S) in column form
 * (stype > 0), L a simplicial symbolic or numeric factor of the same
 * pattern.  The factor is computed by the GPU supernodal LL' on an
 * exact-pattern supernodal shadow of L (kept per factor) and written into
 * L's simplicial layout: a symbolic L gets the reference's unpacked layout
 * (Lp from ColCount with the grow0/grow1/grow2 slack, next/prev in column
 * order), Li/Lnz the exact rows, Lx L (LL') or D on the diagonal and the
 * unit factor below (LDL', L->is_ll = FALSE).  Not positive definite:
 * returns TRUE with CHOLMOD_NOT_POSDEF, L->minor the failing column, the
 * columns from it on zero, as the reference.  On the GPU path: stype > 0,
 * real double or single, kstart = 0 and kend = n, dbound = sbound = 0;
 * otherwise CHOLMOD_INVALID with a message.  LDL' is formed from LL', so an
 * indefinite matrix stops at its first non-positive pivot (the reference's
 * LDL' continues through negative pivots).  Sets Common->rowfacfl as the
 * reference counts it. */
int cholmod_l_rowfac (cholmod_sparse *A, cholmod_sparse *F, double beta [2],
    size_t kstart, size_t kend, cholmod_factor *L, cholmod_common *Common) ;

/* The int32 forms of the three entry points above, for programs of the
 * int32 CHOLMOD API (cholmod_start, cholmod_factorize, cholmod_solve):
 * cholmod_super_numeric (cholmod.h:4016), cholmod_super_lsolve (4037),
 * cholmod_super_ltsolve (4058); called by the int32 cholmod_factorize_p
 * (CHOLMOD/Cholesky/cholmod_factorize.c:260) and cholmod_solve2
 * (cholmod_solve.c:698-707).  Common->itype must be CHOLMOD_INT and A, F, L
 * int32 objects (otherwise CHOLMOD_INVALID, as in the reference).  The GPU
 * path runs on an int64 shadow of L's index arrays, kept per factor (its
 * device state stays attached between calls; gb300_release_factor(L) drops
 * it); L->x is L's own.  Results are those of the int64 entry points. */
int cholmod_super_numeric (cholmod_sparse *A, cholmod_sparse *F, double beta [2],
    cholmod_factor *L, cholmod_common *Common) ;
int cholmod_super_lsolve (cholmod_factor *L, cholmod_dense *X,
    cholmod_dense *E, cholmod_common *Common) ;
int cholmod_super_ltsolve (cholmod_factor *L, cholmod_dense *X,
    cholmod_dense *E, cholmod_common *Common) ;

/* Rough reciprocal condition number of a factor: (min L(j,j) / max
 * L(j,j))^2 for LL'; 1 for n = 0; 0 when the factorization failed
 * (L->minor < n) or a diagonal entry is NaN; EMPTY for a missing argument.
 * Replaces CHOLMOD/Cholesky/cholmod_rcond.c:51-110 (cholmod.h, cholmod_l_rcond);
 * a factor whose values live on the GPU (GB300_OPT_KEEP_ON_DEVICE) is
 * reduced there without a copy back. */
double cholmod_l_rcond (cholmod_factor *L, cholmod_common *Common) ;

/* Sparse right-hand side: X = A\B (or the system sys names, as in
 * cholmod_l_solve) for a sparse B, X returned sparse: the entries of the
 * dense solution that are not zero (NaN kept), rows ascending, packed and
 * sorted, nzmax = nnz(X) (at least 1); free with gb300_free_sparse.
 * Replaces CHOLMOD/Cholesky/cholmod_spsolve.c:56-278 (cholmod.h,
 * cholmod_l_spsolve), same argument checks (B unsymmetric, L->n ==
 * B->nrow, equal dtypes) and result.  L must be a real supernodal LL'
 * factor; B real, packed or not (for a row index given twice in a column
 * the last entry counts, as in the reference); a row index outside
 * [0, n) is CHOLMOD_INVALID.  Up to 64 columns per GPU pass, of which only
 * the nonzero entries are copied back. */
cholmod_sparse *cholmod_l_spsolve (int sys, cholmod_factor *L,
    cholmod_sparse *B, cholmod_common *Common) ;

/* ======================================================================== *
 * 2. gb300_* extensions.                                                    *
 * ======================================================================== */

/* Initialise a cholmod_common with CHOLMOD's default parameter values for
 * the fields this library reads (cholmod_l_start / cholmod_l_defaults,
 * CHOLMOD/Utility/t_cholmod_defaults.c:43-124).  For programs without the
 * reference library.  gb300_finish releases this library's device state
 * attached to Common. */
int gb300_start (cholmod_common *Common) ;
int gb300_finish (cholmod_common *Common) ;

/* Options (defaults in brackets):
 *  GB300_OPT_KEEP_ON_DEVICE [0]: 1 = do not copy L->x back to the host after
 *      the factorization; the factor stays resident on the GPU for solves.
 *  GB300_OPT_SMALL_COLS [64]: supernodes at most this wide are factorized by
 *      one thread block each; wider ones by the blocked multi-block path.
 *      A change applies from the next factorization (the plan is rebuilt).
 *  GB300_OPT_SUBTREE_WORK [4000000]: a subtree whose supernodes are all at
 *      most GB300_OPT_SMALL_COLS wide and whose estimated work (sum of
 *      nscol nsrow^2 + 1e4 per supernode) is at most this many flops is
 *      factorized whole by one thread block; 0 = never.  A change applies
 *      from the next factorization (the plan is rebuilt).
 *  GB300_OPT_WARP_ROWS [64]: in the one-launch factorization, a supernode
 *      factorized whole (a subtree member, or a small supernode on its own)
 *      whose front has at most this many rows (0-64) is assembled and
 *      factorized by one warp instead of a whole thread block; the subtree
 *      members run wave by wave (a wave: supernodes of equal height in the
 *      subtree), several one-warp fronts at once (eight of at most 32 rows,
 *      two of 33-64 rows).  The factor is the same bit for bit with every
 *      value.  0 = never (and no one-warp leaf subtrees in the sweeps).  A
 *      change applies from the next factorization (the plan is rebuilt).
 *  GB300_OPT_GRAPH [1]: 1 = gb300_solve_refined replays its refinement
 *      step (permutation, both sweeps, residual, backward error) from a
 *      CUDA graph captured once per pattern, right-hand-side count and
 *      factor precision (the first step of a solve with new buffers runs
 *      directly); 0 = every step launches its kernels one by one.
 *  GB300_OPT_SWEEP_STREAMS [2]: with more than 16 right-hand sides the
 *      sweeps run in passes of 16 columns; up to this many passes (1-4) run
 *      at once, each on its own stream with its own dependency words and
 *      update vectors.  The result is the same bit for bit with every value.
 *  GB300_OPT_PIVOT_LOG2 [23]: gb300_factorize_mixed switches to the FP64
 *      factor when the smallest pivot of the FP32 factor satisfies
 *      min L(k,k)^2 <= 2^-value * max L(k,k)^2 (23: the single-precision
 *      epsilon; 0 makes every FP32 factor take the FP64 path).
 *  GB300_OPT_PROFILE [0]: 1 = time every kernel launch of the factorization
 *      with CUDA events (summed per kernel kind, see gb300_get_profile); also
 *      clears the accumulated profile.
 *  GB300_OPT_SWEEP [1]: 1 = each sweep is one dependency-driven launch over
 *      all supernodes (diagonal blocks applied through their inverses);
 *      0 = one launch per etree level and block step.
 *  GB300_OPT_TRACE [0]: 1 = the single-launch sweeps record, per task, the
 *      global-timer values when it started, when its dependencies were met
 *      and when it finished (gb300_get_trace).
 *  GB300_OPT_FACTOR [1]: 1 = the numeric factorization is one persistent
 *      launch over a task graph of the whole etree (assembly chunks, small
 *      supernodes, tiles of the wide supernodes, update blocks; a supernode
 *      starts when its children's update blocks are done); 0 = one launch
 *      of each kind per etree level, levels in sequence.
 *  GB300_OPT_TENSOR [1]: 1 = in the FP32 factorization the tile and
 *      update-block products of the supernodes wider than the small
 *      cutoff run on the tensor cores (tcgen05 kind::tf32; the panel solves
 *      write each 64 x 64 block of L split into TF32 hi and FP32 lo parts,
 *      the products stage these by bulk asynchronous copies and form all
 *      four hi/lo products, draining the accumulator into FP32 sums every
 *      64 of K); 0 = FP32 multiply-adds on the CUDA cores.  The operand
 *      images take twice the FP32 factor's memory; when they cannot be
 *      allocated the CUDA cores take the products.
 *  GB300_OPT_UPD_GROUP [4]: in a supernode wider than the small cutoff the
 *      trailing updates of this many 64-column panels (1-4) run as one tile
 *      product of depth 64 x value; the updates within a group stay one
 *      panel deep (the diagonal chain waits on them).  A change applies
 *      from the next factorization (the plan is rebuilt).
 *  GB300_OPT_AUTOTUNE [0]: 1 = the first cholmod_l_super_numeric (or
 *      cholmod_super_numeric) on this Common runs gb300_autotune's default
 *      candidates on its own input (one timed factorization each after a
 *      warm-up), leaves the fastest set on the Common, then factorizes; a
 *      program that only calls the CHOLMOD API gets tuned plan options this
 *      way.  Setting the option again arms another tuning. */
#define GB300_OPT_KEEP_ON_DEVICE 1
#define GB300_OPT_SMALL_COLS     2
#define GB300_OPT_PROFILE        3
#define GB300_OPT_SWEEP          4
#define GB300_OPT_TRACE          5
#define GB300_OPT_FACTOR         6
#define GB300_OPT_TENSOR         7
#define GB300_OPT_SUBTREE_WORK   8
#define GB300_OPT_WARP_ROWS      9
#define GB300_OPT_GRAPH          10
#define GB300_OPT_SWEEP_STREAMS  11
#define GB300_OPT_PIVOT_LOG2     12
#define GB300_OPT_UPD_GROUP      13
#define GB300_OPT_AUTOTUNE       14
int gb300_set_option (cholmod_common *Common, int option, int64_t value) ;
/* The current value of an option with a numeric setting (SMALL_COLS,
 * SUBTREE_WORK, WARP_ROWS, UPD_GROUP, KEEP_ON_DEVICE, AUTOTUNE), the
 * default when none was set; 0 for the others. */
int64_t gb300_get_option (cholmod_common *Common, int option) ;

/* Autotuner of the plan options (small cutoff, subtree work limit, update
 * group).  cand: ncand rows of 3 values (GB300_OPT_SMALL_COLS,
 * GB300_OPT_SUBTREE_WORK, GB300_OPT_UPD_GROUP), or NULL for the default
 * list (gb300_autotune_candidates).  Each candidate is set on Common, one
 * factorization builds its plan, then reps (1-15) factorizations are timed
 * (the library's device time of the factorization launch, as
 * gb300_get_stats()[0]) and their median goes to ms[i] (ms may be NULL).
 * mixed: 1 = gb300_factorize_mixed, 0 = gb300_factorize of A (FP64).
 * Returns the index of the fastest candidate and leaves it set on Common;
 * -1 when a factorization failed (the options are then restored; Common->
 * status tells why).  L holds the last candidate's factor afterwards:
 * factorize again for the tuned one. */
int gb300_autotune (cholmod_sparse *A, cholmod_factor *L, int mixed, int reps,
    const int64_t *cand, int ncand, double *ms, cholmod_common *Common) ;
/* The default candidates: writes up to ncand rows of 3 values into cand
 * (may be NULL) and returns how many there are. */
int gb300_autotune_candidates (int64_t *cand, int ncand) ;
/* gb300_autotune with the timing supplied by the caller: timer(Common, ud)
 * performs one run under the options currently set on Common and returns
 * its milliseconds (negative: failed). */
typedef double (*gb300_tune_timer) (cholmod_common *Common, void *ud) ;
int gb300_autotune_with (const int64_t *cand, int ncand, int reps, double *ms,
    gb300_tune_timer timer, void *ud, cholmod_common *Common) ;

/* Supernodal symbolic analysis of A (stype < 0, lower) with a given final
 * (already postordered) permutation Perm: elimination tree, column counts,
 * fundamental supernodes, relaxed amalgamation and the row pattern L->s,
 * following CHOLMOD/Supernodal/cholmod_super_symbolic.c:147-938 with the
 * nrelax/zrelax parameters of Common.  Produces the factor cholmod_analyze
 * returns when its selected ordering ends in Perm (the weighted postorder of
 * cholmod_analyze.c:828-880 is already applied to Perm).  Sets Common->fl,
 * Common->lnz, Common->anz as cholmod_rowcolcounts does.  NULL on error. */
cholmod_factor *gb300_analyze_perm (cholmod_sparse *A, const int64_t *Perm,
    cholmod_common *Common) ;

/* S = tril(A(p,p)) then cholmod_l_super_numeric: the supernodal branch of
 * cholmod_l_factorize_p (CHOLMOD/Cholesky/cholmod_factorize.c:172-283) for a
 * symmetric-lower A.  beta may be NULL (zero). */
int gb300_factorize (cholmod_sparse *A, double beta [2], cholmod_factor *L,
    cholmod_common *Common) ;

/* X = A\B through L: Y = P*B, cholmod_l_super_lsolve, cholmod_l_super_ltsolve,
 * X = P'*Y (the supernodal branch of cholmod_l_solve2,
 * CHOLMOD/Cholesky/cholmod_solve.c:656-724).  The other sys values as
 * there: P*B and P'*B for CHOLMOD_P / CHOLMOD_Pt; the lower sweep alone
 * for CHOLMOD_L / CHOLMOD_LD, the upper alone for CHOLMOD_Lt / CHOLMOD_DLt,
 * both for CHOLMOD_LDLt, none for CHOLMOD_D, all of these without the
 * permutation (the reference applies L->Perm only for A, P and Pt,
 * cholmod_solve.c:262-267).
 * Returns a new dense X (free with gb300_free_dense) or NULL. */
cholmod_dense *gb300_solve (int sys, cholmod_factor *L, cholmod_dense *B,
    cholmod_common *Common) ;

/* FP32 factor + FP64 iterative refinement.  gb300_factorize_mixed computes an
 * FP32 supernodal factor of D*A*D (D = diag(A)^-1/2, symmetric diagonal
 * scaling applied per supernode during assembly) and keeps it on the GPU;
 * L->x is not written.  gb300_solve_refined solves A X = B in FP64 to the
 * backward error tol (|b-Ax|_inf / (|A|_inf |x|_inf + |b|_inf) per column)
 * with the residual SpMV and the update in FP64 on the GPU; when refinement
 * stalls (no residual reduction in 2 steps, or a pivot <= eps*max diagonal
 * in the FP32 factor) it refactors in FP64 and finishes with that factor.
 * info (optional, 4 doubles): [0] iterations, [1] final backward error,
 * [2] 1 if the FP64 fallback ran, [3] max backward error over columns.
 * A NaN or infinity in the residual, x, b or A makes a column's backward
 * error NaN, which never meets tol: refinement goes on to the FP64
 * fallback (or stops at once when b itself is not finite) and the call
 * ends with Common->status = CHOLMOD_DSMALL and info[1] = NaN. */
int gb300_factorize_mixed (cholmod_sparse *A, cholmod_factor *L,
    cholmod_common *Common) ;
cholmod_dense *gb300_solve_refined (cholmod_sparse *A, cholmod_factor *L,
    cholmod_dense *B, double tol, double *info, cholmod_common *Common) ;

/* Why the mixed factor of L is in FP64: 0 = it is not (the FP32 factor is
 * in use), 1 = the FP32 factorization failed (a pivot was not positive),
 * 2 = an FP32 pivot was small (GB300_OPT_PIVOT_LOG2), 3 = refinement
 * stalled (the backward error did not halve in 2 steps).  -1 when L has no
 * mixed factor. */
#define GB300_REASON_NONE        0
#define GB300_REASON_FP32_FAILED 1
#define GB300_REASON_SMALL_PIVOT 2
#define GB300_REASON_STALLED     3
int gb300_mixed_reason (cholmod_factor *L, cholmod_common *Common) ;

/* gb300_solve_refined writing into *X_Handle, as cholmod_l_solve2 reuses
 * its X (CHOLMOD/Cholesky/cholmod_solve.c:298, ensure_dense): an X of n
 * rows, B->ncol columns, d >= n, real double, is overwritten in place (it
 * may be page-locked by the caller, so that the result's copy back is a
 * plain DMA); any other X is freed and replaced, a NULL one allocated.
 * Returns TRUE, or FALSE with Common->status set. */
int gb300_solve_refined2 (cholmod_sparse *A, cholmod_factor *L, cholmod_dense *B,
    double tol, double *info, cholmod_dense **X_Handle, cholmod_common *Common) ;

/* Release the GPU state attached to L (device factor, plans, graphs).  The
 * plan of a factor is found again by the factor's address, sizes, pattern
 * array addresses and a fingerprint of sampled pattern entries; a caller
 * that rewrites L's pattern arrays in place calls this first. */
int gb300_release_factor (cholmod_factor *L, cholmod_common *Common) ;
/* Device bytes held by L's device state on Common's device (0 when it has
 * none): plan structures, factors, diagonal-block inverses, value maps and
 * work buffers.  The update blocks and tensor-core operand images of a
 * factorization are scratch of the Common, grown to the largest pattern it
 * factorized and shared by all its factors; gb300_finish frees them. */
int64_t gb300_factor_device_bytes (cholmod_factor *L, cholmod_common *Common) ;
/* After gb300_factorize_mixed: frees the factor of the precision the
 * refined solves do not read (the FP64 one when the FP32 factor is used,
 * else the FP32 one); a later factorization allocates it again.  Returns
 * the bytes freed. */
int64_t gb300_trim_factor (cholmod_factor *L, cholmod_common *Common) ;

/* Object helpers for programs without the reference library.  Memory comes
 * from malloc and is counted in Common->malloc_count / memory_inuse the way
 * CHOLMOD counts it, so CHOLMOD's own cholmod_l_free_* can free it too.
 * xdtype = xtype + dtype: real, complex ((re, im) pairs in x) or zomplex
 * (re in x, im in z); pattern for a sparse matrix only. */
cholmod_sparse *gb300_allocate_sparse (size_t nrow, size_t ncol, size_t nzmax,
    int sorted, int packed, int stype, int xdtype, cholmod_common *Common) ;
cholmod_dense *gb300_allocate_dense (size_t nrow, size_t ncol, size_t d,
    int xdtype, cholmod_common *Common) ;
int gb300_free_sparse (cholmod_sparse **A, cholmod_common *Common) ;
int gb300_free_dense (cholmod_dense **X, cholmod_common *Common) ;
int gb300_free_factor (cholmod_factor **L, cholmod_common *Common) ;

/* Layout of the CHOLMOD objects as compiled into this library: object 0 =
 * cholmod_common, 1 = cholmod_sparse, 2 = cholmod_factor, 3 = cholmod_dense.
 * gb300_abi_offset returns offsetof(object, field) or -1 for an unknown
 * field; gb300_abi_sizeof returns sizeof(object). */
long gb300_abi_offset (int object, const char *field) ;
long gb300_abi_sizeof (int object) ;

/* Per-kernel-kind totals of the profiled factorizations: ms[k] and count[k]
 * for kind k = 1 assembly, 2 small-supernode factor, 6 task graph of the
 * level (wide panels and update blocks). */
int gb300_get_profile (cholmod_common *Common, double *ms, double *count, int nkinds) ;

/* Per-task times (ns, device global timer) of the last traced forward
 * (forward = 1) or backward sweep: out[3t..3t+2] = start, dependencies met,
 * end of task t, tasks in ticket order.  Returns the number of tasks. */
int gb300_get_trace (cholmod_common *Common, int forward, unsigned long long *out,
    int64_t nmax) ;

/* Per-task trace of the last traced factorization's task graphs (all
 * levels, plan order): out[3t..3t+2] = claimed, finished (ns), block
 * (with the one-launch factorization: the SM id in the high 32 bits, the
 * block index in the low 32). */
int gb300_get_factor_trace (cholmod_common *Common, unsigned long long *out,
    int64_t nmax) ;

/* The factorization task graph of L's plan, 8 int32 per task: type, s, b,
 * r, c, priority, level, 0 (task types as in the trace).  With the one-launch
 * factorization (GB300_OPT_FACTOR = 1) the whole graph in the trace's order
 * (level 0); otherwise the per-level graphs.  Returns the count. */
int gb300_plan_tasks (cholmod_factor *L, cholmod_common *Common, int32_t *out, int64_t nmax) ;

/* The single-launch sweep's tasks (forward = 1 or backward) of L's plan in
 * ticket order, the order of gb300_get_trace: 5 int32 per task: s, kind
 * (0 diagonal block, 1 off-diagonal rows), idx, r0, nr.  Supernodes of the
 * sweeps' leaf subtrees have none.  Returns the count. */
int gb300_plan_sweep_tasks (cholmod_factor *L, cholmod_common *Common, int forward,
    int32_t *out, int64_t nmax) ;

/* Facts of the GPU plan of L (built if needed): [0] algorithmic flops of the
 * task graphs (wide panels' LL', solves and updates, and every update block), [1] etree levels, [2] launches per factorization, [3]
 * update-block entries, [4] tile-update tasks, [5] supernodes, [6] launches
 * per forward sweep, [7] per backward sweep, [8] update-vector entries,
 * [9] mixed state (0 none, 1 FP32 factor, 2 FP64 factor). */
int gb300_factor_info (cholmod_factor *L, cholmod_common *Common, double *out, int nout) ;

/* Measured multiply-add throughput of the current GPU's FP64 (dtype 0) or
 * FP32 (dtype 4) pipes, TFLOP/s (a register-resident FMA-chain probe). */
int gb300_fma_peak (int dtype, double *tflops) ;

/* Last device-side timings of this library for Common (milliseconds, CUDA
 * events on the library's stream): [0] factor, [1] last solve sweep pair
 * (for cholmod_l_spsolve: its passes' scatter, solve and count, summed),
 * [2] refined solve total, [3] assembly, [4] kernel launches of the last
 * factorization (count), [5] kernel launches issued through Common so far. */
int gb300_get_stats (cholmod_common *Common, double *out, int nout) ;

/* Batches of independent systems (no counterpart in the reference, which
 * factors one matrix per call).  gb300_batch_analyze returns the supernodal
 * symbolic factor of the block-diagonal matrix diag(A_0, ..., A_{nsys-1}),
 * system i having the pattern whose symbolic factor is Lpat[sys_pat[i]]; it
 * equals gb300_analyze_perm of that block-diagonal matrix with the
 * block-diagonal permutation, built by concatenation (no analysis is
 * repeated).  Factorize and solve the batch through the ordinary entry points
 * with the block-diagonal A (the systems' lower triangles placed on the
 * diagonal): the factorization is one persistent launch over the whole
 * forest, and gb300_solve_refined measures the backward error of each system
 * separately.  Free the result with gb300_free_factor. */
cholmod_factor *gb300_batch_analyze (int npat, cholmod_factor *const *Lpat,
    int64_t nsys, const int32_t *sys_pat, cholmod_common *Common) ;

/* Request server (no counterpart in the reference, a per-call library).
 * nslots worker threads, each with its own cholmod_common and CUDA stream,
 * take factor and solve requests as they arrive; requests that are admitted
 * together run on the GPU at the same time.  Symbolic analyses are cached by
 * the caller's pattern id (analysed once, with perm, on first sight);
 * factors stay resident on the device keyed by the caller's factor id (a
 * factor request for a resident factor refactorizes it in place); a factor
 * request is admitted when its device-memory estimate (from nnz(L)) fits
 * under budget_bytes, evicting idle factors least recently used first;
 * after each factorization a factor keeps only what its solves use
 * (gb300_trim_factor; update blocks and operand images are per-worker
 * scratch) and is charged its measured device bytes
 * (gb300_factor_device_bytes), also after each refined solve; an evicted
 * factor keeps the copy of its A on the host (up to 32 GB of evicted A's,
 * the oldest dropped first), so that a later solve against it factorizes
 * it again first (a readmission) instead of failing;
 * requests of one factor run in order, and queued solves of one factor are
 * coalesced into one refined solve of up to max_rhs columns.  Every solve is
 * the FP32 factor + FP64 refinement to backward error 1e-12.  A, perm and B
 * are copied at submission.  arrival is a gb300_server_now() time stamp.
 * gb300_server_wait blocks until request req is done, copies a solve's X
 * (n x nrhs, leading dimension ldx) and fills out[7]: arrival, start,
 * finish (seconds, gb300_server_now clock), backward error, refinement
 * iterations, status, columns of the coalesced solve.  Returns the
 * request's CHOLMOD status.  gb300_server_stats: [0] resident bytes, [1]
 * budget, [2] resident factors, [3] cached patterns, [4] evictions, [5]
 * solves merged into another, [6] requests served, [7] readmissions, [8]
 * evicted factors whose A is kept, [9] host bytes of those A's. */
typedef struct gb300_server gb300_server ;
gb300_server *gb300_server_create (int nslots, int64_t budget_bytes, int max_rhs) ;
int gb300_server_factor (gb300_server *S, int64_t req, int64_t factor_id,
    int64_t pattern_id, int64_t n, const int64_t *Ap, const int64_t *Ai,
    const double *Ax, const int64_t *perm, double arrival) ;
int gb300_server_solve (gb300_server *S, int64_t req, int64_t factor_id, int64_t n,
    int nrhs, const double *B, double arrival) ;
int gb300_server_wait (gb300_server *S, int64_t req, double *X, int64_t ldx, double *out) ;
int gb300_server_stats (gb300_server *S, double *out, int nout) ;
/* gb300_set_option on every worker's Common (before requests are
 * submitted); e.g. GB300_OPT_PIVOT_LOG2 = 0 makes every factorization take
 * the FP64 factor (the plain FP64 form of the stream).  TRUE when every
 * worker accepted it. */
int gb300_server_set_option (gb300_server *S, int option, int64_t value) ;
int gb300_server_destroy (gb300_server *S) ;
double gb300_server_now (void) ;

/* Failure-detection check (no counterpart in the reference): runs the
 * library's bounded device-side wait on a flag that nothing sets, giving up
 * after polls polls (each about 100 ns), the way every wait of the sweeps
 * and task graphs gives up.  out[0] = 1 if the wait succeeded (it cannot),
 * out[1] = the error word it set.  Returns TRUE when the kernel ran and the
 * CUDA context is still usable afterwards. */
int gb300_wait_probe (int64_t polls, int32_t *out) ;

/* Backward error of solutions that are already in device memory, with no
 * allocation of any kind (no counterpart in the reference library).  For
 * callers that must not allocate while they run: a serving loop with a
 * fixed memory footprint that cannot afford the implicit synchronization of
 * cudaMalloc/cudaFree, or an application that hands this library memory it
 * has already reserved.  Everything is caller-owned device memory:
 *   A:    n x n symmetric, BOTH triangles in compressed-column form
 *         (Ap [n+1], Ai [nnz] int64, Ax [nnz] double); by symmetry column i
 *         serves as row i of the residual;
 *   X, B: n x nrhs, column-major, leading dimensions ldx, ldb >= n;
 *   berr: nrhs doubles, receives |b - A x|_inf / (|A|_inf |x|_inf + |b|_inf)
 *         per column -- the measure gb300_solve_refined reports in info; a
 *         NaN or infinite entry in that column of x or b, or in A, gives
 *         NaN, so a non-finite solution never passes a tolerance test.
 * The work is queued on stream (a cudaStream_t, NULL for the default
 * stream) and the call returns without waiting.  The reduction scratch is a
 * fixed device array inside this library, sized for GB300_BERR_MAX_RHS
 * columns; it must be all zero when a call starts, which holds because it is
 * zero at load and every call zeroes it before it finishes.  Consequently
 * calls on one device must not overlap: issue them on one stream (or
 * otherwise order them); two calls in flight at once on the same device race
 * on the scratch.  The first call on each device looks up the scratch
 * address (cudaGetSymbolAddress, with that device current); make that first
 * call before any stream capture.  Returns 0, or GB300_NOALLOC_INVALID (bad
 * pointer, size or leading dimension), GB300_NOALLOC_TOO_LARGE (nrhs >
 * GB300_BERR_MAX_RHS; nothing is queued), GB300_NOALLOC_CUDA (CUDA error). */
#define GB300_BERR_MAX_RHS 64
#define GB300_NOALLOC_INVALID   (-1)
#define GB300_NOALLOC_TOO_LARGE (-2)
#define GB300_NOALLOC_CUDA      (-3)
int gb300_backward_error_noalloc (int64_t n, const int64_t *Ap, const int64_t *Ai,
    const double *Ax, int nrhs, const double *X, int64_t ldx, const double *B,
    int64_t ldb, double *berr, void *stream) ;

#ifdef __cplusplus
}
#endif

#endif /* CHOLMOD_GB300_H */
