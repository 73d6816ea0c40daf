// gb_k_assemble.cu -- front assembly: zero, scatter A, extend-add of the
// children's update blocks through the relative map (owner-computes,
// children in a fixed order; reference: t_cholmod_super_numeric_worker.c
// :419-520 for A and :896-930 for the relative-map scatter).
#include "gb_k_bodies.cuh"

template <typename TA, typename TL>
__global__ void __launch_bounds__(256)
k_assemble(gb_dev_pattern P, const gb_asm_task *__restrict__ tasks,
           const int64_t *__restrict__ Sp, const int64_t *__restrict__ Si,
           const TA *__restrict__ Sx, const double *__restrict__ scale,
           double beta, TL *Lx, TL *CB)
{
    assemble_body<TA, TL>(P, tasks[blockIdx.x], Sp, Si, Sx, scale, beta, Lx, CB);
}

extern "C" {

// a_dtype: dtype of Sx; l_dtype: dtype of Lx/CB
int gb_launch_assemble(const gb_pattern_ptrs *pp, const gb_asm_task *tasks, int ntasks,
                       const int64_t *Sp, const int64_t *Si, const void *Sx, int a_dtype,
                       const double *scale, double beta, void *Lx, void *CB, int l_dtype,
                       cudaStream_t st)
{
    if (ntasks <= 0) return 0;
    gb_dev_pattern P = gb_to_dev(pp);
    if (a_dtype == 0 && l_dtype == 0)
        k_assemble<double, double><<<ntasks, 256, 0, st>>>(P, tasks, Sp, Si, (const double *)Sx, scale, beta, (double *)Lx, (double *)CB);
    else if (a_dtype == 0 && l_dtype == 4)
        k_assemble<double, float><<<ntasks, 256, 0, st>>>(P, tasks, Sp, Si, (const double *)Sx, scale, beta, (float *)Lx, (float *)CB);
    else
        k_assemble<float, float><<<ntasks, 256, 0, st>>>(P, tasks, Sp, Si, (const float *)Sx, scale, beta, (float *)Lx, (float *)CB);
    return (int)cudaGetLastError();
}


}  // extern "C"
