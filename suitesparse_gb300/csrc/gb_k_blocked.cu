// gb_k_blocked.cu -- blocked path of wide supernodes: LL' of one 64-column
// diagonal block plus its inverse (kept for the sweeps), and the panel rows
// below it as 64x64 products with that inverse.
#include "gb_k_common.cuh"

#define NB GB_NB
#define LDT (NB + 1)

template <typename T>
__global__ void __launch_bounds__(256)
k_potrf_diag(gb_dev_pattern P, const gb_potrf_task *__restrict__ tasks, T *Lx, T *Linv)
{
    __shared__ T A[NB][LDT];
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
    const int fail = potrf_ll<T, NB>(A, nb, &sfail);
    __syncthreads();
    for (int idx = threadIdx.x; idx < nb * nb; idx += blockDim.x) {
        const int i = idx % nb, j = idx / nb;
        if (i >= j) blk[i + (int64_t)j * nsrow] = A[i][j];
    }
    if (fail >= 0 && threadIdx.x == 0) {
        P.fail[s] = tk.c0 + fail;
        atomicExch(P.anyfail, 1);
    }
    tri_inverse<T, NB>(A, nb, Linv + P.linvoff[P.blkoff[s] + tk.c0 / NB], nb);
}

template <typename T>
__host__ __device__ constexpr size_t trsm_smem() { return sizeof(T) * (2 * NB * LDT); }

// rows [r0, r0+nr) of the panel: X = B * Linv_bb' for the block at c0.  A
// block that failed in k_potrf_diag of this step still solves its leading
// (fail - c0) columns, which stay valid.
template <typename T>
__global__ void __launch_bounds__(256)
k_trsm_rows(gb_dev_pattern P, const gb_trsm_task *__restrict__ tasks, T *Lx, const T *Linv)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    T *Bt = (T *)smem_raw, *Lt = Bt + NB * LDT;
    const gb_trsm_task tk = tasks[blockIdx.x];
    const int s = tk.s;
    const int f = P.fail[s];
    if (f >= 0 && f < tk.c0) return;
    const int ncols = (f >= 0) ? f - tk.c0 : tk.nb;
    const int nsrow = (int)(P.Pi[s + 1] - P.Pi[s]);
    T *panel = Lx + P.Px[s];
    const int nb = tk.nb, nr = tk.nr;
    const T *li = Linv + P.linvoff[P.blkoff[s] + tk.c0 / NB];   // column-major, ld nb
    for (int idx = threadIdx.x; idx < NB * NB; idx += blockDim.x) {
        const int c = idx % NB, k = idx / NB;
        Lt[k * LDT + c] = (c < nb && k < nb) ? li[c + (int64_t)k * nb] : (T)0;
        Bt[k * LDT + c] = (c < nr && k < nb) ? panel[tk.r0 + c + (int64_t)(tk.c0 + k) * nsrow] : (T)0;
    }
    __syncthreads();
    trsm_tile<T>(Bt, Lt, LDT, nr, nb, ncols, panel + tk.r0 + (int64_t)tk.c0 * nsrow, nsrow);
}

extern "C" {

int gb_launch_potrf_diag(const gb_pattern_ptrs *pp, const gb_potrf_task *tasks, int ntasks,
                         void *Lx, void *Linv, int dtype, cudaStream_t st)
{
    if (ntasks <= 0) return 0;
    gb_dev_pattern P = gb_to_dev(pp);
    if (dtype == 0) k_potrf_diag<double><<<ntasks, 64, 0, st>>>(P, tasks, (double *)Lx, (double *)Linv);
    else k_potrf_diag<float><<<ntasks, 64, 0, st>>>(P, tasks, (float *)Lx, (float *)Linv);
    return (int)cudaGetLastError();
}

int gb_launch_trsm_rows(const gb_pattern_ptrs *pp, const gb_trsm_task *tasks, int ntasks,
                        void *Lx, const void *Linv, int dtype, cudaStream_t st)
{
    if (ntasks <= 0) return 0;
    gb_dev_pattern P = gb_to_dev(pp);
    static int configured = 0;
    if (!configured) {
        cudaFuncSetAttribute(k_trsm_rows<double>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)trsm_smem<double>());
        cudaFuncSetAttribute(k_trsm_rows<float>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)trsm_smem<float>());
        configured = 1;
    }
    if (dtype == 0) k_trsm_rows<double><<<ntasks, 256, trsm_smem<double>(), st>>>(P, tasks, (double *)Lx, (const double *)Linv);
    else k_trsm_rows<float><<<ntasks, 256, trsm_smem<float>(), st>>>(P, tasks, (float *)Lx, (const float *)Linv);
    return (int)cudaGetLastError();
}

}  // extern "C"
