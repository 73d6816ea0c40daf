// gb_k_small.cu -- one thread block factors a supernode at most GB_SMALL_MAX
// wide: left-looking LL' of the diagonal block in shared memory, its inverse
// (kept for the sweeps), then the panel rows below as 64-row products with
// that inverse (reference: dpotrf :1004-1058 and dtrsm :1152-1218 of
// t_cholmod_super_numeric_worker.c).
#include "gb_k_bodies.cuh"

template <typename T>
__global__ void __launch_bounds__(256)
k_factor_small(gb_dev_pattern P, const gb_node_task *__restrict__ tasks, T *Lx, T *Linv)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ int sfail;
    factor_small_body<T>(P, tasks[blockIdx.x].s, Lx, Linv, smem_raw, &sfail);
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
