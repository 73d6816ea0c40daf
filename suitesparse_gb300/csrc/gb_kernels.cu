// gb_kernels.cu -- sm_103a kernels of the supernodal numeric factorization
// and the supernodal triangular sweeps.
//
// Formulation: multifrontal, level-scheduled over the supernodal elimination
// tree.  Every supernode s owns a front of nsrow x nsrow entries: its first
// nscol columns are the L panel, stored in place in the CHOLMOD layout
// (L->x + L->px[s], column-major, leading dimension nsrow), and the trailing
// (nsrow-nscol)^2 lower triangle is its update block, kept in a device
// buffer (CB, leading dimension nsrow-nscol).  Supernodes of one etree level
// are independent, so each kernel below processes a whole level per launch:
//
//   k_assemble     zero the front, scatter the entries of A, extend-add the
//                  children's update blocks through the relative map (child
//                  row -> parent row position; rows are sorted, so the map is
//                  monotone).  Owner-computes, children summed in a fixed
//                  order: no float atomics, results independent of timing.
//   k_factor_small diagonal-block LL' plus panel triangular solve of a
//                  supernode at most GB_SMALL_MAX wide, one block each.
//   k_potrf_diag / k_trsm_rows / k_gemm_nt
//                  the blocked path for wider supernodes (diagonal block LL',
//                  panel triangular solve, trailing update), and the update
//                  block product CB -= L21 L21' (the dense contraction).
//
// The sweeps (forward L y = b, backward L' x = y) follow the same levels; the
// forward sweep carries, per supernode, the vector L21 x1 of contributions to
// its ancestors' rows (the update vector) and its parent gathers them, so
// again no two blocks write the same entry.
//
// Correspondence with the reference (CHOLMOD/Supernodal/
// t_cholmod_super_numeric_worker.c): assembly of A :419-520, descendant
// update + relative-map scatter :686-930, dpotrf :1004-1058, dtrsm
// :1152-1218, not-positive-definite handling :1084-1146; sweeps:
// t_cholmod_super_solve_worker.c:63-301 (forward) and :358-578 (backward).

#include <cuda_runtime.h>
#include <stdint.h>
#include "gb_plan.h"

struct gb_dev_pattern {
    const int64_t *Super, *Pi, *Px, *cboff, *cbvoff;
    const int32_t *Ls, *relmap, *child_ptr, *child_list;
    int32_t *fail;       // [nsuper] first failing local column, -1 if none
    int32_t *anyfail;    // [1] set to 1 when any supernode failed
};

__device__ __forceinline__ int lower_bound_i32(const int32_t *a, int lo, int hi, int64_t key)
{
    while (lo < hi) {
        int mid = (lo + hi) >> 1;
        if ((int64_t)a[mid] < key) lo = mid + 1; else hi = mid;
    }
    return lo;
}

template <typename T> __device__ __forceinline__ T gb_sqrt(T x);
template <> __device__ __forceinline__ double gb_sqrt<double>(double x) { return sqrt(x); }
template <> __device__ __forceinline__ float gb_sqrt<float>(float x) { return sqrtf(x); }

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

// ---------------------------------------------------------------------------
// dense LL' of an nb x nb block held in shared memory (right-looking).
// Returns the first failing local column, or -1.  Only A[i][j], i >= j, used.
// ---------------------------------------------------------------------------

template <typename T, int NB>
__device__ int block_potrf(T (*A)[NB + 1], int nb, int *sfail)
{
    if (threadIdx.x == 0) *sfail = -1;
    __syncthreads();
    for (int j = 0; j < nb; j++) {
        if (threadIdx.x == 0) {
            T d = A[j][j];
            if (!(d > (T)0)) *sfail = j;
            else A[j][j] = gb_sqrt<T>(d);
        }
        __syncthreads();
        if (*sfail >= 0) break;
        const T d = A[j][j];
        for (int i = j + 1 + threadIdx.x; i < nb; i += blockDim.x) A[i][j] /= d;
        __syncthreads();
        const int nt = nb - j - 1;
        for (int idx = threadIdx.x; idx < nt * nt; idx += blockDim.x) {
            const int ii = j + 1 + idx % nt, kk = j + 1 + idx / nt;
            if (ii >= kk) A[ii][kk] -= A[ii][j] * A[kk][j];
        }
        __syncthreads();
    }
    __syncthreads();
    return *sfail;
}

// rows r of a panel (leading dimension ld): X * L' = B for the nb columns
// starting at column c0, L = the factored block in shared memory; only the
// first ncols columns are solved (ncols < nb after a failed pivot).
template <typename T, int NB>
__device__ void rows_trsm(T *panel, int ld, int c0, T (*A)[NB + 1], int ncols,
                          int r_begin, int r_end)
{
    for (int r = r_begin + threadIdx.x; r < r_end; r += blockDim.x) {
        T *row = panel + r + (int64_t)c0 * ld;
        T x[NB];
#pragma unroll
        for (int j = 0; j < NB; j++) {
            if (j < ncols) {
                T v = row[(int64_t)j * ld];
#pragma unroll
                for (int k = 0; k < NB; k++)
                    if (k < j) v -= x[k] * A[j][k];
                x[j] = v / A[j][j];
                row[(int64_t)j * ld] = x[j];
            }
        }
    }
}

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

// ---------------------------------------------------------------------------
// permutations, scaling, residual (FP64) and norms
// ---------------------------------------------------------------------------

// Y(k, r) = scale(k-th permuted) * B(perm[k], r), converting type
template <typename TB, typename TY>
__global__ void k_perm_in(int64_t n, int nrhs, const int64_t *__restrict__ perm,
                          const double *__restrict__ scale, const TB *__restrict__ B,
                          int64_t ldb, TY *Y, int64_t ldy)
{
    const int64_t total = n * nrhs;
    for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < total;
         idx += (int64_t)gridDim.x * blockDim.x) {
        const int64_t k = idx % n, r = idx / n;
        const int64_t i = perm ? perm[k] : k;
        double v = (double)B[i + r * ldb];
        if (scale) v *= scale[i];
        Y[k + r * ldy] = (TY)v;
    }
}

// X(perm[k], r) = scale(perm[k]) * Y(k, r)  [op 0: assign, op 1: add]
template <typename TY, typename TX>
__global__ void k_perm_out(int64_t n, int nrhs, const int64_t *__restrict__ perm,
                           const double *__restrict__ scale, const TY *__restrict__ Y,
                           int64_t ldy, TX *X, int64_t ldx, int add)
{
    const int64_t total = n * nrhs;
    for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < total;
         idx += (int64_t)gridDim.x * blockDim.x) {
        const int64_t k = idx % n, r = idx / n;
        const int64_t i = perm ? perm[k] : k;
        double v = (double)Y[k + r * ldy];
        if (scale) v *= scale[i];
        if (add) X[i + r * ldx] += (TX)v;
        else X[i + r * ldx] = (TX)v;
    }
}

// R = B - A X with A in full compressed-row form (both triangles), FP64,
// one warp per row, fixed summation order; also |A|_inf row sums (once).
__global__ void k_residual(int64_t n, int nrhs, const int64_t *__restrict__ Rp,
                           const int32_t *__restrict__ Rj, const double *__restrict__ Rx,
                           const double *__restrict__ X, int64_t ldx,
                           const double *__restrict__ B, int64_t ldb,
                           double *R, int64_t ldr)
{
    const int lane = threadIdx.x & 31;
    const int64_t warp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t w = warp; w < n * nrhs; w += nwarps) {
        const int64_t i = w % n, r = w / n;
        const double *x = X + r * ldx;
        double acc = 0.0;
        for (int64_t p = Rp[i] + lane; p < Rp[i + 1]; p += 32) acc += Rx[p] * x[Rj[p]];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
        if (lane == 0) R[i + r * ldr] = B[i + r * ldb] - acc;
    }
}

// per column r: out[3r] = max|R|, out[3r+1] = max|X|, out[3r+2] = max|B|;
// one block per column, fixed reduction tree.
__global__ void k_colmax3(int64_t n, const double *__restrict__ R, int64_t ldr,
                          const double *__restrict__ X, int64_t ldx,
                          const double *__restrict__ B, int64_t ldb, double *out)
{
    __shared__ double sm[3][256];
    const int r = blockIdx.x;
    double a = 0, b = 0, c = 0;
    for (int64_t i = threadIdx.x; i < n; i += blockDim.x) {
        a = fmax(a, fabs(R[i + r * ldr]));
        b = fmax(b, fabs(X[i + r * ldx]));
        c = fmax(c, fabs(B[i + r * ldb]));
    }
    sm[0][threadIdx.x] = a;
    sm[1][threadIdx.x] = b;
    sm[2][threadIdx.x] = c;
    __syncthreads();
    for (int o = blockDim.x / 2; o > 0; o >>= 1) {
        if (threadIdx.x < o)
            for (int q = 0; q < 3; q++)
                sm[q][threadIdx.x] = fmax(sm[q][threadIdx.x], sm[q][threadIdx.x + o]);
        __syncthreads();
    }
    if (threadIdx.x == 0)
        for (int q = 0; q < 3; q++) out[3 * r + q] = sm[q][0];
}

// max over rows of sum |A(i,:)| (for the backward error denominator)
__global__ void k_anorm_inf(int64_t n, const int64_t *__restrict__ Rp,
                            const double *__restrict__ Rx, double *out)
{
    __shared__ double sm[256];
    double best = 0;
    for (int64_t i = threadIdx.x; i < n; i += blockDim.x) {
        double acc = 0;
        for (int64_t p = Rp[i]; p < Rp[i + 1]; p++) acc += fabs(Rx[p]);
        best = fmax(best, acc);
    }
    sm[threadIdx.x] = best;
    __syncthreads();
    for (int o = blockDim.x / 2; o > 0; o >>= 1) {
        if (threadIdx.x < o) sm[threadIdx.x] = fmax(sm[threadIdx.x], sm[threadIdx.x + o]);
        __syncthreads();
    }
    if (threadIdx.x == 0) *out = sm[0];
}

// zero factor entries [from, to) (not-positive-definite clean-up)
template <typename T>
__global__ void k_zero_range(T *x, int64_t from, int64_t to)
{
    for (int64_t i = from + blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < to;
         i += (int64_t)gridDim.x * blockDim.x)
        x[i] = (T)0;
}

// ---------------------------------------------------------------------------
// extern "C" launchers (plain pointers; dtype 0 = double, 4 = single)
// ---------------------------------------------------------------------------

extern "C" {


static gb_dev_pattern to_dev(const gb_pattern_ptrs *p)
{
    gb_dev_pattern d;
    d.Super = p->Super; d.Pi = p->Pi; d.Px = p->Px; d.cboff = p->cboff;
    d.cbvoff = p->cbvoff; d.Ls = p->Ls; d.relmap = p->relmap;
    d.child_ptr = p->child_ptr; d.child_list = p->child_list;
    d.fail = p->fail; d.anyfail = p->anyfail;
    return d;
}

// a_dtype: dtype of Sx; l_dtype: dtype of Lx/CB
int gb_launch_assemble(const gb_pattern_ptrs *pp, const gb_asm_task *tasks, int ntasks,
                       const int64_t *Sp, const int64_t *Si, const void *Sx, int a_dtype,
                       const double *scale, double beta, void *Lx, void *CB, int l_dtype,
                       cudaStream_t st)
{
    if (ntasks <= 0) return 0;
    gb_dev_pattern P = to_dev(pp);
    if (a_dtype == 0 && l_dtype == 0)
        k_assemble<double, double><<<ntasks, 256, 0, st>>>(P, tasks, Sp, Si, (const double *)Sx, scale, beta, (double *)Lx, (double *)CB);
    else if (a_dtype == 0 && l_dtype == 4)
        k_assemble<double, float><<<ntasks, 256, 0, st>>>(P, tasks, Sp, Si, (const double *)Sx, scale, beta, (float *)Lx, (float *)CB);
    else
        k_assemble<float, float><<<ntasks, 256, 0, st>>>(P, tasks, Sp, Si, (const float *)Sx, scale, beta, (float *)Lx, (float *)CB);
    return (int)cudaGetLastError();
}

int gb_launch_factor_small(const gb_pattern_ptrs *pp, const gb_node_task *tasks, int ntasks,
                           void *Lx, int dtype, cudaStream_t st)
{
    if (ntasks <= 0) return 0;
    gb_dev_pattern P = to_dev(pp);
    if (dtype == 0) k_factor_small<double><<<ntasks, 256, 0, st>>>(P, tasks, (double *)Lx);
    else k_factor_small<float><<<ntasks, 256, 0, st>>>(P, tasks, (float *)Lx);
    return (int)cudaGetLastError();
}

int gb_launch_potrf_diag(const gb_pattern_ptrs *pp, const gb_potrf_task *tasks, int ntasks,
                         void *Lx, int dtype, cudaStream_t st)
{
    if (ntasks <= 0) return 0;
    gb_dev_pattern P = to_dev(pp);
    if (dtype == 0) k_potrf_diag<double><<<ntasks, 256, 0, st>>>(P, tasks, (double *)Lx);
    else k_potrf_diag<float><<<ntasks, 256, 0, st>>>(P, tasks, (float *)Lx);
    return (int)cudaGetLastError();
}

int gb_launch_trsm_rows(const gb_pattern_ptrs *pp, const gb_trsm_task *tasks, int ntasks,
                        void *Lx, int dtype, cudaStream_t st)
{
    if (ntasks <= 0) return 0;
    gb_dev_pattern P = to_dev(pp);
    if (dtype == 0) k_trsm_rows<double><<<ntasks, GB_TRSM_ROWS, 0, st>>>(P, tasks, (double *)Lx);
    else k_trsm_rows<float><<<ntasks, GB_TRSM_ROWS, 0, st>>>(P, tasks, (float *)Lx);
    return (int)cudaGetLastError();
}

int gb_launch_gemm(const gb_pattern_ptrs *pp, const gb_gemm_task *tasks, const int32_t *owner,
                   int ntasks, void *Lx, void *CB, int dtype, cudaStream_t st)
{
    if (ntasks <= 0) return 0;
    gb_dev_pattern P = to_dev(pp);
    if (dtype == 0) k_gemm_nt<double><<<ntasks, 256, 0, st>>>(P, tasks, owner, (double *)Lx, (double *)CB);
    else k_gemm_nt<float><<<ntasks, 256, 0, st>>>(P, tasks, owner, (float *)Lx, (float *)CB);
    return (int)cudaGetLastError();
}

// kind: 0 fwd_small, 1 fwd_gather, 2 bwd_small (node tasks)
int gb_launch_sweep_node(int kind, const gb_pattern_ptrs *pp, const gb_node_task *tasks,
                         int ntasks, const void *Lx, int dtype, int nrhs, void *Y,
                         int64_t ldy, void *U, cudaStream_t st)
{
    if (ntasks <= 0) return 0;
    gb_dev_pattern P = to_dev(pp);
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
    gb_dev_pattern P = to_dev(pp);
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

static int grid_for(int64_t work)
{
    int64_t g = (work + 255) / 256;
    if (g < 1) g = 1;
    if (g > 152 * 16) g = 152 * 16;
    return (int)g;
}

// b_dtype/y_dtype: 0 double, 4 single
int gb_launch_perm_in(int64_t n, int nrhs, const int64_t *perm, const double *scale,
                      const void *B, int b_dtype, int64_t ldb, void *Y, int y_dtype,
                      int64_t ldy, cudaStream_t st)
{
    int g = grid_for(n * nrhs);
    if (b_dtype == 0 && y_dtype == 0)
        k_perm_in<double, double><<<g, 256, 0, st>>>(n, nrhs, perm, scale, (const double *)B, ldb, (double *)Y, ldy);
    else if (b_dtype == 0 && y_dtype == 4)
        k_perm_in<double, float><<<g, 256, 0, st>>>(n, nrhs, perm, scale, (const double *)B, ldb, (float *)Y, ldy);
    else if (b_dtype == 4 && y_dtype == 4)
        k_perm_in<float, float><<<g, 256, 0, st>>>(n, nrhs, perm, scale, (const float *)B, ldb, (float *)Y, ldy);
    else
        k_perm_in<float, double><<<g, 256, 0, st>>>(n, nrhs, perm, scale, (const float *)B, ldb, (double *)Y, ldy);
    return (int)cudaGetLastError();
}

int gb_launch_perm_out(int64_t n, int nrhs, const int64_t *perm, const double *scale,
                       const void *Y, int y_dtype, int64_t ldy, void *X, int x_dtype,
                       int64_t ldx, int add, cudaStream_t st)
{
    int g = grid_for(n * nrhs);
    if (y_dtype == 0 && x_dtype == 0)
        k_perm_out<double, double><<<g, 256, 0, st>>>(n, nrhs, perm, scale, (const double *)Y, ldy, (double *)X, ldx, add);
    else if (y_dtype == 4 && x_dtype == 0)
        k_perm_out<float, double><<<g, 256, 0, st>>>(n, nrhs, perm, scale, (const float *)Y, ldy, (double *)X, ldx, add);
    else if (y_dtype == 4 && x_dtype == 4)
        k_perm_out<float, float><<<g, 256, 0, st>>>(n, nrhs, perm, scale, (const float *)Y, ldy, (float *)X, ldx, add);
    else
        k_perm_out<double, float><<<g, 256, 0, st>>>(n, nrhs, perm, scale, (const double *)Y, ldy, (float *)X, ldx, add);
    return (int)cudaGetLastError();
}

int gb_launch_residual(int64_t n, int nrhs, const int64_t *Rp, const int32_t *Rj,
                       const double *Rx, const double *X, int64_t ldx, const double *B,
                       int64_t ldb, double *R, int64_t ldr, cudaStream_t st)
{
    int64_t warps = n * nrhs;
    int g = grid_for(warps * 32);
    k_residual<<<g, 256, 0, st>>>(n, nrhs, Rp, Rj, Rx, X, ldx, B, ldb, R, ldr);
    return (int)cudaGetLastError();
}

int gb_launch_colmax3(int64_t n, int nrhs, const double *R, int64_t ldr, const double *X,
                      int64_t ldx, const double *B, int64_t ldb, double *out, cudaStream_t st)
{
    k_colmax3<<<nrhs, 256, 0, st>>>(n, R, ldr, X, ldx, B, ldb, out);
    return (int)cudaGetLastError();
}

int gb_launch_anorm(int64_t n, const int64_t *Rp, const double *Rx, double *out, cudaStream_t st)
{
    k_anorm_inf<<<1, 256, 0, st>>>(n, Rp, Rx, out);
    return (int)cudaGetLastError();
}

int gb_launch_zero_range(void *x, int dtype, int64_t from, int64_t to, cudaStream_t st)
{
    if (to <= from) return 0;
    int g = grid_for(to - from);
    if (dtype == 0) k_zero_range<double><<<g, 256, 0, st>>>((double *)x, from, to);
    else k_zero_range<float><<<g, 256, 0, st>>>((float *)x, from, to);
    return (int)cudaGetLastError();
}

}  // extern "C"
