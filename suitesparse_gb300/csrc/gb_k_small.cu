// gb_k_small.cu -- one thread block factors a supernode at most GB_SMALL_MAX
// wide: left-looking LL' of the diagonal block in shared memory, its inverse
// (kept for the sweeps), then the panel rows below as 64-row products with
// that inverse (reference: dpotrf :1004-1058 and dtrsm :1152-1218 of
// t_cholmod_super_numeric_worker.c).
#include "gb_k_common.cuh"

#define NB GB_SMALL_MAX
#define LDT (NB + 1)

template <typename T>
__host__ __device__ constexpr size_t small_smem() { return sizeof(T) * (3 * NB * LDT); }

template <typename T>
__global__ void __launch_bounds__(256)
k_factor_small(gb_dev_pattern P, const gb_node_task *__restrict__ tasks, T *Lx, T *Linv)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    T (*A)[LDT] = (T (*)[LDT])smem_raw;          // diagonal block, row-major rows
    T *X = (T *)smem_raw + NB * LDT;              // inverse, column j at X + j*LDT
    T *Bt = X + NB * LDT;                         // panel chunk, Bt[k*LDT + r]
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
    const int fail = potrf_ll<T, NB>(A, nscol, &sfail);
    __syncthreads();
    for (int idx = threadIdx.x; idx < nscol * nscol; idx += blockDim.x) {
        const int i = idx % nscol, j = idx / nscol;
        if (i >= j) panel[i + (int64_t)j * nsrow] = A[i][j];
    }
    if (fail >= 0 && threadIdx.x == 0) {
        P.fail[s] = fail;
        atomicExch(P.anyfail, 1);
    }
    const int ncols = fail >= 0 ? fail : nscol;
    tri_inverse<T, NB>(A, nscol, X, LDT);
    __syncthreads();
    // inverse for the sweeps (column-major, leading dimension nscol)
    T *out = Linv + P.linvoff[P.blkoff[s]];
    for (int idx = threadIdx.x; idx < nscol * nscol; idx += blockDim.x) {
        const int i = idx % nscol, j = idx / nscol;
        out[i + (int64_t)j * nscol] = X[j * LDT + i];
    }
    // Lt[k*LDT + c] = Linv(c, k): transpose X in place into A's storage
    T *Lt = (T *)A;
    __syncthreads();
    for (int idx = threadIdx.x; idx < NB * NB; idx += blockDim.x) {
        const int c = idx % NB, k = idx / NB;
        Lt[k * LDT + c] = (c < nscol && k < nscol) ? X[k * LDT + c] : (T)0;
    }
    __syncthreads();
    for (int r0 = nscol; r0 < nsrow; r0 += NB) {
        const int nr = min(NB, nsrow - r0);
        for (int idx = threadIdx.x; idx < NB * NB; idx += blockDim.x) {
            const int r = idx % NB, k = idx / NB;
            Bt[k * LDT + r] = (r < nr && k < nscol) ? panel[r0 + r + (int64_t)k * nsrow] : (T)0;
        }
        __syncthreads();
        trsm_tile<T>(Bt, Lt, LDT, nr, nscol, ncols, panel + r0, nsrow);
        __syncthreads();
    }
}

extern "C" {

int gb_launch_factor_small(const gb_pattern_ptrs *pp, const gb_node_task *tasks, int ntasks,
                           void *Lx, void *Linv, int dtype, cudaStream_t st)
{
    if (ntasks <= 0) return 0;
    gb_dev_pattern P = gb_to_dev(pp);
    static int configured = 0;
    if (!configured) {
        cudaFuncSetAttribute(k_factor_small<double>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)small_smem<double>());
        cudaFuncSetAttribute(k_factor_small<float>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)small_smem<float>());
        configured = 1;
    }
    if (dtype == 0) k_factor_small<double><<<ntasks, 256, small_smem<double>(), st>>>(P, tasks, (double *)Lx, (double *)Linv);
    else k_factor_small<float><<<ntasks, 256, small_smem<float>(), st>>>(P, tasks, (float *)Lx, (float *)Linv);
    return (int)cudaGetLastError();
}

}  // extern "C"
