// gb_k_blocked.cu -- blocked path of wide supernodes: LL' of one diagonal
// block, triangular solve of the panel rows below it.
#include "gb_k_common.cuh"

// blocked path: LL' of the diagonal block at (c0, c0) of a wide supernode
template <typename T>
__global__ void __launch_bounds__(256)
k_potrf_diag(gb_dev_pattern P, const gb_potrf_task *__restrict__ tasks, T *Lx)
{
    __shared__ T A[GB_NB][GB_NB + 1];
    __shared__ int sfail;
    const gb_potrf_task tk = tasks[blockIdx.x];
    const int s = tk.s;
    if (P.fail[s] >= 0) return;
    const int nsrow = (int)(P.Pi[s + 1] - P.Pi[s]);
    T *blk = Lx + P.Px[s] + tk.c0 + (int64_t)tk.c0 * nsrow;
    const int nb = tk.nb;
    for (int idx = threadIdx.x; idx < nb * nb; idx += blockDim.x) {
        const int i = idx % nb, j = idx / nb;
        A[i][j] = (i >= j) ? blk[i + (int64_t)j * nsrow] : (T)0;
    }
    __syncthreads();
    const int fail = block_potrf<T, GB_NB>(A, nb, &sfail);
    for (int idx = threadIdx.x; idx < nb * nb; idx += blockDim.x) {
        const int i = idx % nb, j = idx / nb;
        if (i >= j) blk[i + (int64_t)j * nsrow] = A[i][j];
    }
    if (fail >= 0 && threadIdx.x == 0) {
        P.fail[s] = tk.c0 + fail;
        atomicExch(P.anyfail, 1);
    }
}

// blocked path: rows [r0, r0+nr) of the panel against the block at c0.  A
// block that failed in k_potrf_diag of this step still solves its leading
// (fail - c0) columns, which stay valid.
template <typename T>
__global__ void __launch_bounds__(GB_TRSM_ROWS)
k_trsm_rows(gb_dev_pattern P, const gb_trsm_task *__restrict__ tasks, T *Lx)
{
    __shared__ T A[GB_NB][GB_NB + 1];
    const gb_trsm_task tk = tasks[blockIdx.x];
    const int s = tk.s;
    const int f = P.fail[s];
    if (f >= 0 && f < tk.c0) return;
    const int ncols = (f >= 0) ? f - tk.c0 : tk.nb;
    const int nsrow = (int)(P.Pi[s + 1] - P.Pi[s]);
    T *panel = Lx + P.Px[s];
    const T *blk = panel + tk.c0 + (int64_t)tk.c0 * nsrow;
    const int nb = tk.nb;
    for (int idx = threadIdx.x; idx < nb * nb; idx += blockDim.x) {
        const int i = idx % nb, j = idx / nb;
        A[i][j] = (i >= j) ? blk[i + (int64_t)j * nsrow] : (T)0;
    }
    __syncthreads();
    rows_trsm<T, GB_NB>(panel, nsrow, tk.c0, A, ncols, tk.r0, tk.r0 + tk.nr);
}


extern "C" {

int gb_launch_potrf_diag(const gb_pattern_ptrs *pp, const gb_potrf_task *tasks, int ntasks,
                         void *Lx, int dtype, cudaStream_t st)
{
    if (ntasks <= 0) return 0;
    gb_dev_pattern P = gb_to_dev(pp);
    if (dtype == 0) k_potrf_diag<double><<<ntasks, 256, 0, st>>>(P, tasks, (double *)Lx);
    else k_potrf_diag<float><<<ntasks, 256, 0, st>>>(P, tasks, (float *)Lx);
    return (int)cudaGetLastError();
}

int gb_launch_trsm_rows(const gb_pattern_ptrs *pp, const gb_trsm_task *tasks, int ntasks,
                        void *Lx, int dtype, cudaStream_t st)
{
    if (ntasks <= 0) return 0;
    gb_dev_pattern P = gb_to_dev(pp);
    if (dtype == 0) k_trsm_rows<double><<<ntasks, GB_TRSM_ROWS, 0, st>>>(P, tasks, (double *)Lx);
    else k_trsm_rows<float><<<ntasks, GB_TRSM_ROWS, 0, st>>>(P, tasks, (float *)Lx);
    return (int)cudaGetLastError();
}


}  // extern "C"
