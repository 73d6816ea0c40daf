// gb_k_gemm.cu -- tile update C -= A B' of the supernodal factorization:
// the update blocks CB_s -= L21 L21' (reference: dsyrk/dgemm of
// t_cholmod_super_numeric_worker.c:768-883) and the trailing updates of the
// blocked path.
#include "gb_k_common.cuh"

// ---------------------------------------------------------------------------
// tile update C -= A B' (SIMT, 64x64 tile, 16-deep k slices in shared memory)
// ---------------------------------------------------------------------------

template <typename T>
__global__ void __launch_bounds__(256)
k_gemm_nt(gb_dev_pattern P, const gb_gemm_task *__restrict__ tasks,
          const int32_t *__restrict__ task_owner, T *Lx, T *CB)
{
    constexpr int BK = 16;
    __shared__ T As[BK][GB_TILE + 4];
    __shared__ T Bs[BK][GB_TILE + 4];
    const gb_gemm_task tk = tasks[blockIdx.x];
    if (task_owner && P.fail[task_owner[blockIdx.x]] >= 0) return;
    const T *A = Lx + tk.a;
    const T *B = Lx + tk.b;
    T *C = ((tk.flags & GB_GEMM_C_IN_CB) ? CB : Lx) + tk.c;
    const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
    T acc[4][4];
#pragma unroll
    for (int i = 0; i < 4; i++)
#pragma unroll
        for (int j = 0; j < 4; j++) acc[i][j] = (T)0;

    for (int k0 = 0; k0 < tk.k; k0 += BK) {
        // 64 x 16 slices of A and B: element (i, kk) at [i + kk*ld]
        for (int idx = threadIdx.x; idx < GB_TILE * BK; idx += 256) {
            const int i = idx & (GB_TILE - 1), kk = idx >> 6;
            const int kg = k0 + kk;
            As[kk][i] = (i < tk.m && kg < tk.k) ? A[i + (int64_t)kg * tk.lda] : (T)0;
            Bs[kk][i] = (i < tk.n && kg < tk.k) ? B[i + (int64_t)kg * tk.ldb] : (T)0;
        }
        __syncthreads();
#pragma unroll
        for (int kk = 0; kk < BK; kk++) {
            T a[4], b[4];
#pragma unroll
            for (int i = 0; i < 4; i++) a[i] = As[kk][ty + 16 * i];
#pragma unroll
            for (int j = 0; j < 4; j++) b[j] = Bs[kk][tx + 16 * j];
#pragma unroll
            for (int i = 0; i < 4; i++)
#pragma unroll
                for (int j = 0; j < 4; j++) acc[i][j] += a[i] * b[j];
        }
        __syncthreads();
    }
    const bool lower = (tk.flags & GB_GEMM_LOWER) != 0;
#pragma unroll
    for (int i = 0; i < 4; i++) {
        const int r = ty + 16 * i;
        if (r >= tk.m) continue;
#pragma unroll
        for (int j = 0; j < 4; j++) {
            const int c = tx + 16 * j;
            if (c >= tk.n) continue;
            if (lower && r - c < tk.diag_off) continue;
            C[r + (int64_t)c * tk.ldc] -= acc[i][j];
        }
    }
}


extern "C" {

int gb_launch_gemm(const gb_pattern_ptrs *pp, const gb_gemm_task *tasks, const int32_t *owner,
                   int ntasks, void *Lx, void *CB, int dtype, cudaStream_t st)
{
    if (ntasks <= 0) return 0;
    gb_dev_pattern P = gb_to_dev(pp);
    if (dtype == 0) k_gemm_nt<double><<<ntasks, 256, 0, st>>>(P, tasks, owner, (double *)Lx, (double *)CB);
    else k_gemm_nt<float><<<ntasks, 256, 0, st>>>(P, tasks, owner, (float *)Lx, (float *)CB);
    return (int)cudaGetLastError();
}


}  // extern "C"
