// gb_k_small.cu -- one thread block factors a supernode at most GB_SMALL_MAX
// wide: dense LL' of the diagonal block in shared memory, then the panel
// triangular solve (reference: dpotrf :1004-1058 and dtrsm :1152-1218 of
// t_cholmod_super_numeric_worker.c).
#include "gb_k_common.cuh"

template <typename T>
__global__ void __launch_bounds__(256)
k_factor_small(gb_dev_pattern P, const gb_node_task *__restrict__ tasks, T *Lx)
{
    __shared__ T A[GB_SMALL_MAX][GB_SMALL_MAX + 1];
    __shared__ int sfail;
    const int s = tasks[blockIdx.x].s;
    const int64_t k1 = P.Super[s];
    const int nscol = (int)(P.Super[s + 1] - k1);
    const int nsrow = (int)(P.Pi[s + 1] - P.Pi[s]);
    T *panel = Lx + P.Px[s];
    for (int idx = threadIdx.x; idx < nscol * nscol; idx += blockDim.x) {
        const int i = idx % nscol, j = idx / nscol;
        A[i][j] = (i >= j) ? panel[i + (int64_t)j * nsrow] : (T)0;
    }
    __syncthreads();
    const int fail = block_potrf<T, GB_SMALL_MAX>(A, nscol, &sfail);
    for (int idx = threadIdx.x; idx < nscol * nscol; idx += blockDim.x) {
        const int i = idx % nscol, j = idx / nscol;
        if (i >= j) panel[i + (int64_t)j * nsrow] = A[i][j];
    }
    if (fail >= 0 && threadIdx.x == 0) {
        P.fail[s] = fail;
        atomicExch(P.anyfail, 1);
    }
    __syncthreads();
    const int ncols = fail >= 0 ? fail : nscol;
    rows_trsm<T, GB_SMALL_MAX>(panel, nsrow, 0, A, ncols, nscol, nsrow);
}


extern "C" {

int gb_launch_factor_small(const gb_pattern_ptrs *pp, const gb_node_task *tasks, int ntasks,
                           void *Lx, int dtype, cudaStream_t st)
{
    if (ntasks <= 0) return 0;
    gb_dev_pattern P = gb_to_dev(pp);
    if (dtype == 0) k_factor_small<double><<<ntasks, 256, 0, st>>>(P, tasks, (double *)Lx);
    else k_factor_small<float><<<ntasks, 256, 0, st>>>(P, tasks, (float *)Lx);
    return (int)cudaGetLastError();
}


}  // extern "C"
