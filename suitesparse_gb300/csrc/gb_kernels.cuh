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

#define GB_NB 64            /* block size of the blocked paths */
#define GB_TILE 64          /* output tile edge of the update kernel */
#define GB_TRSM_ROWS 128    /* rows per triangular-solve task */
#define GB_SMALL_MAX 64     /* widest supernode factored by one block */

#endif
