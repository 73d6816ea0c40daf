// gb_k_sweep.cu -- supernodal forward / backward sweeps, level by level
// (reference: t_cholmod_super_solve_worker.c forward :63-301, backward
// :358-578).
#include "gb_k_common.cuh"

// ---------------------------------------------------------------------------
// supernodal sweeps.  Y is n x nrhs (leading dimension ldy) in the permuted
// order; U holds the update vectors (m_s x nrhs, leading dimension m_s, at
// cbvoff[s]*nrhs).
// ---------------------------------------------------------------------------

#define GB_RC 32   /* right-hand-side columns per pass in shared memory */

// zero U_s and gather the children's update vectors into Y (rows of s's
// columns) and U_s (the other rows).  Called with the whole block.
template <typename T>
__device__ void fwd_gather(const gb_dev_pattern &P, int s, int nrhs, T *Y, int64_t ldy, T *U)
{
    const int64_t k1 = P.Super[s];
    const int nscol = (int)(P.Super[s + 1] - k1);
    const int m = (int)(P.Pi[s + 1] - P.Pi[s]) - nscol;
    T *us = U + P.cbvoff[s] * nrhs;
    for (int idx = threadIdx.x; idx < m * nrhs; idx += blockDim.x) us[idx] = (T)0;
    __syncthreads();
    for (int ci = P.child_ptr[s]; ci < P.child_ptr[s + 1]; ci++) {
        const int c = P.child_list[ci];
        const int ncc = (int)(P.Super[c + 1] - P.Super[c]);
        const int64_t pic = P.Pi[c];
        const int mc = (int)(P.Pi[c + 1] - pic) - ncc;
        const int32_t *rm = P.relmap + pic + ncc;
        const T *uc = U + P.cbvoff[c] * nrhs;
        for (int idx = threadIdx.x; idx < mc * nrhs; idx += blockDim.x) {
            const int i = idx % mc, r = idx / mc;
            const int t = rm[i];
            const T v = uc[i + (int64_t)r * mc];
            if (t < nscol) Y[k1 + t + r * ldy] -= v;
            else us[(t - nscol) + (int64_t)r * m] += v;
        }
        __syncthreads();
    }
}

template <typename T>
__global__ void __launch_bounds__(256)
k_fwd_small(gb_dev_pattern P, const gb_node_task *__restrict__ tasks, const T *Lx,
            int nrhs, T *Y, int64_t ldy, T *U)
{
    __shared__ T X[GB_SMALL_MAX][GB_RC + 1];
    const int s = tasks[blockIdx.x].s;
    fwd_gather<T>(P, s, nrhs, Y, ldy, U);
    const int64_t k1 = P.Super[s];
    const int nscol = (int)(P.Super[s + 1] - k1);
    const int nsrow = (int)(P.Pi[s + 1] - P.Pi[s]);
    const int m = nsrow - nscol;
    const T *panel = Lx + P.Px[s];
    T *us = U + P.cbvoff[s] * nrhs;
    for (int rc = 0; rc < nrhs; rc += GB_RC) {
        const int nr = min(GB_RC, nrhs - rc);
        for (int idx = threadIdx.x; idx < nscol * nr; idx += blockDim.x) {
            const int j = idx % nscol, r = idx / nscol;
            X[j][r] = Y[k1 + j + (int64_t)(rc + r) * ldy];
        }
        __syncthreads();
        for (int j = 0; j < nscol; j++) {
            const T d = panel[j + (int64_t)j * nsrow];
            for (int r = threadIdx.x; r < nr; r += blockDim.x) X[j][r] /= d;
            __syncthreads();
            const int nt = nscol - j - 1;
            for (int idx = threadIdx.x; idx < nt * nr; idx += blockDim.x) {
                const int i = j + 1 + idx % nt, r = idx / nt;
                X[i][r] -= panel[i + (int64_t)j * nsrow] * X[j][r];
            }
            __syncthreads();
        }
        for (int idx = threadIdx.x; idx < nscol * nr; idx += blockDim.x) {
            const int j = idx % nscol, r = idx / nscol;
            Y[k1 + j + (int64_t)(rc + r) * ldy] = X[j][r];
        }
        for (int idx = threadIdx.x; idx < m * nr; idx += blockDim.x) {
            const int i = idx % m, r = idx / m;
            const T *row = panel + nscol + i;
            T acc = (T)0;
            for (int j = 0; j < nscol; j++) acc += row[(int64_t)j * nsrow] * X[j][r];
            us[i + (int64_t)(rc + r) * m] += acc;
        }
        __syncthreads();
    }
}

template <typename T>
__global__ void __launch_bounds__(256)
k_fwd_gather(gb_dev_pattern P, const gb_node_task *__restrict__ tasks, int nrhs,
             T *Y, int64_t ldy, T *U)
{
    fwd_gather<T>(P, tasks[blockIdx.x].s, nrhs, Y, ldy, U);
}

// wide supernode, forward step: solve the diagonal block [c0, c0+nb)
template <typename T>
__global__ void __launch_bounds__(256)
k_fwd_diag(gb_dev_pattern P, const gb_sweep_task *__restrict__ tasks, const T *Lx,
           int nrhs, T *Y, int64_t ldy)
{
    __shared__ T X[GB_NB][GB_RC + 1];
    const gb_sweep_task tk = tasks[blockIdx.x];
    const int s = tk.s;
    const int64_t k1 = P.Super[s];
    const int nsrow = (int)(P.Pi[s + 1] - P.Pi[s]);
    const T *blk = Lx + P.Px[s] + tk.c0 + (int64_t)tk.c0 * nsrow;
    const int nb = tk.nb;
    for (int rc = 0; rc < nrhs; rc += GB_RC) {
        const int nr = min(GB_RC, nrhs - rc);
        for (int idx = threadIdx.x; idx < nb * nr; idx += blockDim.x) {
            const int j = idx % nb, r = idx / nb;
            X[j][r] = Y[k1 + tk.c0 + j + (int64_t)(rc + r) * ldy];
        }
        __syncthreads();
        for (int j = 0; j < nb; j++) {
            const T d = blk[j + (int64_t)j * nsrow];
            for (int r = threadIdx.x; r < nr; r += blockDim.x) X[j][r] /= d;
            __syncthreads();
            const int nt = nb - j - 1;
            for (int idx = threadIdx.x; idx < nt * nr; idx += blockDim.x) {
                const int i = j + 1 + idx % nt, r = idx / nt;
                X[i][r] -= blk[i + (int64_t)j * nsrow] * X[j][r];
            }
            __syncthreads();
        }
        for (int idx = threadIdx.x; idx < nb * nr; idx += blockDim.x) {
            const int j = idx % nb, r = idx / nb;
            Y[k1 + tk.c0 + j + (int64_t)(rc + r) * ldy] = X[j][r];
        }
        __syncthreads();
    }
}

// wide supernode, forward step: rows [r0, r0+nr) below the block get
// Y -= L(rows, blk) x(blk) (rows of s's own columns) or U += ... (other rows)
template <typename T>
__global__ void __launch_bounds__(256)
k_fwd_panel(gb_dev_pattern P, const gb_sweep_task *__restrict__ tasks, const T *Lx,
            int nrhs, T *Y, int64_t ldy, T *U)
{
    __shared__ T X[GB_NB][GB_RC + 1];
    const gb_sweep_task tk = tasks[blockIdx.x];
    const int s = tk.s;
    const int64_t k1 = P.Super[s];
    const int nscol = (int)(P.Super[s + 1] - k1);
    const int nsrow = (int)(P.Pi[s + 1] - P.Pi[s]);
    const int m = nsrow - nscol;
    const T *panel = Lx + P.Px[s];
    T *us = U + P.cbvoff[s] * nrhs;
    const int nb = tk.nb;
    for (int rc = 0; rc < nrhs; rc += GB_RC) {
        const int nr = min(GB_RC, nrhs - rc);
        __syncthreads();
        for (int idx = threadIdx.x; idx < nb * nr; idx += blockDim.x) {
            const int j = idx % nb, r = idx / nb;
            X[j][r] = Y[k1 + tk.c0 + j + (int64_t)(rc + r) * ldy];
        }
        __syncthreads();
        for (int idx = threadIdx.x; idx < tk.nr * nr; idx += blockDim.x) {
            const int i = tk.r0 + idx % tk.nr, r = idx / tk.nr;
            const T *row = panel + i + (int64_t)tk.c0 * nsrow;
            T acc = (T)0;
            for (int j = 0; j < nb; j++) acc += row[(int64_t)j * nsrow] * X[j][r];
            if (i < nscol) Y[k1 + i + (int64_t)(rc + r) * ldy] -= acc;
            else us[(i - nscol) + (int64_t)(rc + r) * m] += acc;
        }
    }
}

// backward sweep, narrow supernode: x1 -= L21' Y(rows); x1 = L11' \ x1
template <typename T>
__global__ void __launch_bounds__(256)
k_bwd_small(gb_dev_pattern P, const gb_node_task *__restrict__ tasks, const T *Lx,
            int nrhs, T *Y, int64_t ldy)
{
    __shared__ T X[GB_SMALL_MAX][GB_RC + 1];
    const int s = tasks[blockIdx.x].s;
    const int64_t k1 = P.Super[s];
    const int nscol = (int)(P.Super[s + 1] - k1);
    const int64_t psi = P.Pi[s];
    const int nsrow = (int)(P.Pi[s + 1] - psi);
    const int m = nsrow - nscol;
    const T *panel = Lx + P.Px[s];
    const int32_t *rows = P.Ls + psi + nscol;
    for (int rc = 0; rc < nrhs; rc += GB_RC) {
        const int nr = min(GB_RC, nrhs - rc);
        for (int idx = threadIdx.x; idx < nscol * nr; idx += blockDim.x) {
            const int j = idx % nscol, r = idx / nscol;
            const T *col = panel + nscol + (int64_t)j * nsrow;
            const T *y = Y + (int64_t)(rc + r) * ldy;
            T acc = (T)0;
            for (int i = 0; i < m; i++) acc += col[i] * y[rows[i]];
            X[j][r] = y[k1 + j] - acc;
        }
        __syncthreads();
        for (int j = nscol - 1; j >= 0; j--) {
            const T d = panel[j + (int64_t)j * nsrow];
            for (int r = threadIdx.x; r < nr; r += blockDim.x) X[j][r] /= d;
            __syncthreads();
            for (int idx = threadIdx.x; idx < j * nr; idx += blockDim.x) {
                const int i = idx % j, r = idx / j;
                X[i][r] -= panel[j + (int64_t)i * nsrow] * X[j][r];
            }
            __syncthreads();
        }
        for (int idx = threadIdx.x; idx < nscol * nr; idx += blockDim.x) {
            const int j = idx % nscol, r = idx / nscol;
            Y[k1 + j + (int64_t)(rc + r) * ldy] = X[j][r];
        }
        __syncthreads();
    }
}

// backward sweep, wide supernode, first phase: columns [r0, r0+nr) of s
// (r0/nr reused as a column range) get x(j) -= L21(:, j)' Y(rows)
template <typename T>
__global__ void __launch_bounds__(256)
k_bwd_offdiag(gb_dev_pattern P, const gb_sweep_task *__restrict__ tasks, const T *Lx,
              int nrhs, T *Y, int64_t ldy)
{
    const gb_sweep_task tk = tasks[blockIdx.x];
    const int s = tk.s;
    const int64_t k1 = P.Super[s];
    const int nscol = (int)(P.Super[s + 1] - k1);
    const int64_t psi = P.Pi[s];
    const int nsrow = (int)(P.Pi[s + 1] - psi);
    const int m = nsrow - nscol;
    const T *panel = Lx + P.Px[s];
    const int32_t *rows = P.Ls + psi + nscol;
    for (int idx = threadIdx.x; idx < tk.nr * nrhs; idx += blockDim.x) {
        const int j = tk.r0 + idx % tk.nr, r = idx / tk.nr;
        const T *col = panel + nscol + (int64_t)j * nsrow;
        T *y = Y + (int64_t)r * ldy;
        T acc = (T)0;
        for (int i = 0; i < m; i++) acc += col[i] * y[rows[i]];
        y[k1 + j] -= acc;
    }
}

// backward sweep, wide supernode, diagonal block [c0, c0+nb): x = L_bb' \ x
template <typename T>
__global__ void __launch_bounds__(256)
k_bwd_diag(gb_dev_pattern P, const gb_sweep_task *__restrict__ tasks, const T *Lx,
           int nrhs, T *Y, int64_t ldy)
{
    __shared__ T X[GB_NB][GB_RC + 1];
    const gb_sweep_task tk = tasks[blockIdx.x];
    const int s = tk.s;
    const int64_t k1 = P.Super[s];
    const int nsrow = (int)(P.Pi[s + 1] - P.Pi[s]);
    const T *blk = Lx + P.Px[s] + tk.c0 + (int64_t)tk.c0 * nsrow;
    const int nb = tk.nb;
    for (int rc = 0; rc < nrhs; rc += GB_RC) {
        const int nr = min(GB_RC, nrhs - rc);
        for (int idx = threadIdx.x; idx < nb * nr; idx += blockDim.x) {
            const int j = idx % nb, r = idx / nb;
            X[j][r] = Y[k1 + tk.c0 + j + (int64_t)(rc + r) * ldy];
        }
        __syncthreads();
        for (int j = nb - 1; j >= 0; j--) {
            const T d = blk[j + (int64_t)j * nsrow];
            for (int r = threadIdx.x; r < nr; r += blockDim.x) X[j][r] /= d;
            __syncthreads();
            for (int idx = threadIdx.x; idx < j * nr; idx += blockDim.x) {
                const int i = idx % j, r = idx / j;
                X[i][r] -= blk[j + (int64_t)i * nsrow] * X[j][r];
            }
            __syncthreads();
        }
        for (int idx = threadIdx.x; idx < nb * nr; idx += blockDim.x) {
            const int j = idx % nb, r = idx / nb;
            Y[k1 + tk.c0 + j + (int64_t)(rc + r) * ldy] = X[j][r];
        }
        __syncthreads();
    }
}

// backward sweep, wide supernode: columns [r0, r0+nr) left of block c0 get
// x(j) -= L(blk, j)' x(blk)
template <typename T>
__global__ void __launch_bounds__(256)
k_bwd_panel(gb_dev_pattern P, const gb_sweep_task *__restrict__ tasks, const T *Lx,
            int nrhs, T *Y, int64_t ldy)
{
    const gb_sweep_task tk = tasks[blockIdx.x];
    const int s = tk.s;
    const int64_t k1 = P.Super[s];
    const int nsrow = (int)(P.Pi[s + 1] - P.Pi[s]);
    const T *panel = Lx + P.Px[s];
    for (int idx = threadIdx.x; idx < tk.nr * nrhs; idx += blockDim.x) {
        const int j = tk.r0 + idx % tk.nr, r = idx / tk.nr;
        const T *col = panel + tk.c0 + (int64_t)j * nsrow;
        T *y = Y + (int64_t)r * ldy + k1;
        T acc = (T)0;
        for (int i = 0; i < tk.nb; i++) acc += col[i] * y[tk.c0 + i];
        y[j] -= acc;
    }
}


extern "C" {

// kind: 0 fwd_small, 1 fwd_gather, 2 bwd_small (node tasks)
int gb_launch_sweep_node(int kind, const gb_pattern_ptrs *pp, const gb_node_task *tasks,
                         int ntasks, const void *Lx, int dtype, int nrhs, void *Y,
                         int64_t ldy, void *U, cudaStream_t st)
{
    if (ntasks <= 0) return 0;
    gb_dev_pattern P = gb_to_dev(pp);
    if (dtype == 0) {
        if (kind == 0) k_fwd_small<double><<<ntasks, 256, 0, st>>>(P, tasks, (const double *)Lx, nrhs, (double *)Y, ldy, (double *)U);
        else if (kind == 1) k_fwd_gather<double><<<ntasks, 256, 0, st>>>(P, tasks, nrhs, (double *)Y, ldy, (double *)U);
        else k_bwd_small<double><<<ntasks, 256, 0, st>>>(P, tasks, (const double *)Lx, nrhs, (double *)Y, ldy);
    } else {
        if (kind == 0) k_fwd_small<float><<<ntasks, 256, 0, st>>>(P, tasks, (const float *)Lx, nrhs, (float *)Y, ldy, (float *)U);
        else if (kind == 1) k_fwd_gather<float><<<ntasks, 256, 0, st>>>(P, tasks, nrhs, (float *)Y, ldy, (float *)U);
        else k_bwd_small<float><<<ntasks, 256, 0, st>>>(P, tasks, (const float *)Lx, nrhs, (float *)Y, ldy);
    }
    return (int)cudaGetLastError();
}

// kind: 0 fwd_diag, 1 fwd_panel, 2 bwd_offdiag, 3 bwd_diag, 4 bwd_panel
int gb_launch_sweep_step(int kind, const gb_pattern_ptrs *pp, const gb_sweep_task *tasks,
                         int ntasks, const void *Lx, int dtype, int nrhs, void *Y,
                         int64_t ldy, void *U, cudaStream_t st)
{
    if (ntasks <= 0) return 0;
    gb_dev_pattern P = gb_to_dev(pp);
#define GB_SWEEP(T)                                                                          \
    switch (kind) {                                                                          \
    case 0: k_fwd_diag<T><<<ntasks, 256, 0, st>>>(P, tasks, (const T *)Lx, nrhs, (T *)Y, ldy); break; \
    case 1: k_fwd_panel<T><<<ntasks, 256, 0, st>>>(P, tasks, (const T *)Lx, nrhs, (T *)Y, ldy, (T *)U); break; \
    case 2: k_bwd_offdiag<T><<<ntasks, 256, 0, st>>>(P, tasks, (const T *)Lx, nrhs, (T *)Y, ldy); break; \
    case 3: k_bwd_diag<T><<<ntasks, 256, 0, st>>>(P, tasks, (const T *)Lx, nrhs, (T *)Y, ldy); break; \
    default: k_bwd_panel<T><<<ntasks, 256, 0, st>>>(P, tasks, (const T *)Lx, nrhs, (T *)Y, ldy); break; \
    }
    if (dtype == 0) { GB_SWEEP(double) } else { GB_SWEEP(float) }
#undef GB_SWEEP
    return (int)cudaGetLastError();
}


}  // extern "C"
