/* gb_kernels.cuh -- task descriptors shared by the host plan builder (C) and
 * the CUDA kernels.  Plain structs of fixed-width integers so that the host
 * C code can fill arrays of them and upload them once per pattern. */
#ifndef GB_KERNELS_CUH
#define GB_KERNELS_CUH

#include <stdint.h>

/* Assembly of target front columns [t0, t1) of supernode s: zero them, add
 * the entries of A that fall there, then extend-add every child's update
 * block.  A front has nsrow columns: the first nscol are the L panel (in
 * L->x), the rest are the update block of s. */
typedef struct { int32_t s, t0, t1, pad; } gb_asm_task;

/* Factorize the diagonal nb-by-nb block at (c0, c0) of supernode s's panel
 * (dense LL'); nb <= GB_NB. */
typedef struct { int32_t s, c0, nb, pad; } gb_potrf_task;

/* Triangular solve X * L11' = B for panel rows [r0, r0+nr) of supernode s,
 * where L11 is the diagonal block at (c0, c0) of size nb.  nr <= GB_TRSM_ROWS */
typedef struct { int32_t s, c0, nb, r0, nr, pad0, pad1, pad2; } gb_trsm_task;

/* One output tile: C[0:m,0:n] -= A[0:m,0:k] * B[0:n,0:k]'  (m, n <= GB_TILE).
 * a, b index the factor values; c indexes the factor values or (flag
 * GB_GEMM_C_IN_CB) the update-block buffer.  GB_GEMM_LOWER: store only
 * entries with row >= col + diag_off (tiles crossing the diagonal). */
typedef struct {
    int64_t a, b, c;
    int32_t lda, ldb, ldc, m, n, k, flags, diag_off;
} gb_gemm_task;

#define GB_GEMM_C_IN_CB 1
#define GB_GEMM_LOWER   2

/* Supernodes handled whole by one thread block in the solve sweeps. */
typedef struct { int32_t s, pad; } gb_node_task;

/* Blocked triangular solve step of a wide supernode: block [c0, c0+nb). */
typedef struct { int32_t s, c0, nb, r0, nr, pad0, pad1, pad2; } gb_sweep_task;

/* Task of the single-launch sweeps: kind 0 = diagonal block idx of s (rows
 * r0..r0+nr of the supernode, r0 = 64*idx), kind 1 = off-diagonal rows
 * [r0, r0+nr) (r0 >= nscol) producing the update vector. */
typedef struct { int32_t s, kind, idx, r0, nr, pad0, pad1, pad2; } gb_stask;

/* Task of the per-level device task graph of the wide supernodes (64-grid
 * tiles of the panel of s; c0 = 64 b):
 *   POTRF (s, b)       LL' + inverse of the diagonal block of column block b
 *   TRSM  (s, b, r)    panel rows of row tile r below that block
 *   UPD   (s, b, r, c) tile (r, c) of the panel -= L(r, blks b..b+nbk-1)
 *                      L(c, blks b..b+nbk-1)' (nbk panels at once, k up
 *                      to 64 nbk)
 *   CB    (s, r, c)    update-block tile (r, c) -= L21(r) L21(c)', k = nscol
 * prio 0 = the tasks near the diagonal that the next steps wait on
 * (POTRF; TRSM of row tiles <= b+3; UPD of tiles r <= b+3, c <= b+2, and
 * the grouped updates of the next group's first column), 1 = bulk. */
typedef struct { int32_t type, s, b, r, c, prio, nbk, pad1; } gb_dtask;
/* panels whose trailing updates are applied at once (GB_DT_UPD nbk) */
#define GB_UPD_GROUP 4
#define GB_DT_POTRF 1
#define GB_DT_TRSM  2
#define GB_DT_UPD   3
#define GB_DT_CB    4
/* tasks of the whole-factorization graph (gb_plan.c):
 *   ASM   (s, b = t0, r = t1)  assembly of front columns [t0, t1) of s
 *   SMALL (s)                  whole supernode at most GB_SMALL_MAX wide
 *   JOIN  (s)                  no work: fan-in of a supernode's assembly
 *                              chunks, or of its children's update blocks
 *                              (also marks tasks folded into a NODE task) */
#define GB_DT_ASM   5
#define GB_DT_SMALL 6
#define GB_DT_JOIN  7
/*   NODE  (s)                  a small supernode whole: assembly, LL' and
 *                              every update-block tile, in one task */
#define GB_DT_NODE  8
/*   SUBTREE (s, b = offset, r = count)  a whole subtree of small supernodes
 *                              (list entries [b, b + r) of the pattern's
 *                              subtree list, children first), each as NODE,
 *                              in one task: no queue traffic inside it */
#define GB_DT_SUBTREE 9
/* DIAG (s, b, r, nbk): the diagonal chain of panel b >= 1 of a wide
 * supernode as one task: the panel solve of row block b by panel b - 1,
 * the update of tile (b, b) by panels r .. r + nbk - 1 (the last update of
 * that tile), then POTRF of panel b */
#define GB_DT_DIAG 10
#define GB_SUBTREE_WORK 4.0e6       /* work estimate per subtree task (flops) */
#define GB_NODE_MAX_ROWS 256        /* small supernodes fused into NODE tasks */
#define GB_WARP_ROWS 64             /* fronts at most this tall: one warp each */

/* control words of one task-graph launch: [0] head0 [1] tail0 [2] head1
 * [3] tail1 [4] blocks started [5] error [6] total0 [7] total1 [8] blocks
 * that left a poller's SM */
#define GB_DAG_NCTRL 16
#define GB_DAG_NSMF 1024    /* per-SM poller marks (indexed by %smid) */
#define GB_DAG_POLLERS 16   /* blocks that serve only the critical-path queue */

#define GB_NB 64            /* block size of the blocked paths */
/* floats of one tensor-core operand image (a 64-row block of a 64-column
 * panel, split into TF32 hi and FP32 lo parts): GB_IMG_FLOATS on the device */
#define GB_IMG_FLOATS_HOST 8192
#define GB_TILE 64          /* output tile edge of the update kernel */
#define GB_TRSM_ROWS 64     /* rows per triangular-solve task */
#define GB_SMALL_MAX 64     /* widest supernode factored by one block */

#endif
