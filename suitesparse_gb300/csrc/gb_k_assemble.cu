// gb_k_assemble.cu -- front assembly: zero, scatter A, extend-add of the
// children's update blocks through the relative map (owner-computes,
// children in a fixed order; reference: t_cholmod_super_numeric_worker.c
// :419-520 for A and :896-930 for the relative-map scatter).
#include "gb_k_common.cuh"

// ---------------------------------------------------------------------------
// assembly: zero + scatter A + extend-add of the children's update blocks
// ---------------------------------------------------------------------------

template <typename TA, typename TL>
__global__ void __launch_bounds__(256)
k_assemble(gb_dev_pattern P, const gb_asm_task *__restrict__ tasks,
           const int64_t *__restrict__ Sp, const int64_t *__restrict__ Si,
           const TA *__restrict__ Sx, const double *__restrict__ scale,
           double beta, TL *Lx, TL *CB)
{
    const gb_asm_task tk = tasks[blockIdx.x];
    const int s = tk.s;
    const int64_t k1 = P.Super[s];
    const int nscol = (int)(P.Super[s + 1] - k1);
    const int64_t psi = P.Pi[s];
    const int nsrow = (int)(P.Pi[s + 1] - psi);
    const int m = nsrow - nscol;
    TL *panel = Lx + P.Px[s];
    TL *cb = CB + P.cboff[s];
    const int32_t *ls = P.Ls + psi;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int nwarps = blockDim.x >> 5;

    // 1. zero the target columns (whole panel column; lower part of CB column)
    for (int t = tk.t0 + warp; t < tk.t1; t += nwarps) {
        if (t < nscol) {
            TL *col = panel + (int64_t)t * nsrow;
            for (int i = lane; i < nsrow; i += 32) col[i] = (TL)0;
        } else {
            const int tc = t - nscol;
            TL *col = cb + (int64_t)tc * m;
            for (int i = tc + lane; i < m; i += 32) col[i] = (TL)0;
        }
    }
    __syncthreads();

    // 2. entries of A (lower part, rows >= column) of the panel columns
    const int tend = min(tk.t1, nscol);
    for (int t = tk.t0 + warp; t < tend; t += nwarps) {
        const int64_t k = k1 + t;
        TL *col = panel + (int64_t)t * nsrow;
        const double sk = scale ? scale[k] : 1.0;
        for (int64_t p = Sp[k] + lane; p < Sp[k + 1]; p += 32) {
            const int64_t i = Si[p];
            if (i < k) continue;
            const int pos = lower_bound_i32(ls, t, nsrow, i);
            if (pos < nsrow && (int64_t)ls[pos] == i) {
                double v = (double)Sx[p];
                if (i == k) v += beta;
                if (scale) v = v * (scale[i] * sk);
                col[pos] = (TL)v;
            }
        }
    }
    // beta on diagonal entries that A does not store
    __syncthreads();
    if (beta != 0.0) {
        for (int t = tk.t0 + threadIdx.x; t < tend; t += blockDim.x) {
            const int64_t k = k1 + t;
            bool has = false;
            for (int64_t p = Sp[k]; p < Sp[k + 1]; p++)
                if (Si[p] == k) { has = true; break; }
            if (!has) {
                double v = beta;
                if (scale) v *= scale[k] * scale[k];
                panel[t + (int64_t)t * nsrow] += (TL)v;
            }
        }
    }
    __syncthreads();

    // 3. extend-add of each child's update block, children in a fixed order
    const int cbeg = P.child_ptr[s], cend = P.child_ptr[s + 1];
    for (int ci = cbeg; ci < cend; ci++) {
        const int c = P.child_list[ci];
        const int64_t kc1 = P.Super[c];
        const int ncc = (int)(P.Super[c + 1] - kc1);
        const int64_t pic = P.Pi[c];
        const int mc = (int)(P.Pi[c + 1] - pic) - ncc;
        const int32_t *rm = P.relmap + pic + ncc;
        const TL *cbc = CB + P.cboff[c];
        const int j0 = lower_bound_i32(rm, 0, mc, tk.t0);
        const int j1 = lower_bound_i32(rm, j0, mc, tk.t1);
        for (int j = j0 + warp; j < j1; j += nwarps) {
            const int t = rm[j];
            const TL *src = cbc + (int64_t)j * mc;
            if (t < nscol) {
                TL *dst = panel + (int64_t)t * nsrow;
                for (int i = j + lane; i < mc; i += 32) dst[rm[i]] += src[i];
            } else {
                TL *dst = cb + (int64_t)(t - nscol) * m - nscol;
                for (int i = j + lane; i < mc; i += 32) dst[rm[i]] += src[i];
            }
        }
        __syncthreads();
    }
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
