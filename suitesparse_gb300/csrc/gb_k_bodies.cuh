// gb_k_bodies.cuh -- the work of one assembly task and of one small-supernode
// factorization as device functions, run by their own kernels (one task per
// thread block) and by the whole-factorization task-graph executor.
#ifndef GB_K_BODIES_CUH
#define GB_K_BODIES_CUH

#include "gb_k_common.cuh"

// ---------------------------------------------------------------------------
// assembly of front columns [tk.t0, tk.t1) of supernode tk.s: zero + scatter
// A + extend-add of the children's update blocks (reference:
// t_cholmod_super_numeric_worker.c :419-520 for A, :896-930 for the
// relative-map scatter)
// ---------------------------------------------------------------------------

template <typename TA, typename TL>
__device__ void assemble_body(const gb_dev_pattern &P, const gb_asm_task tk,
                              const int64_t *__restrict__ Sp, const int64_t *__restrict__ Si,
                              const TA *__restrict__ Sx, const double *__restrict__ scale,
                              double beta, TL *Lx, TL *CB)
{
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
// a supernode at most GB_SMALL_MAX wide, whole: LL' of the diagonal block,
// its inverse (kept for the sweeps), the panel rows below as 64-row products
// with that inverse (reference: dpotrf :1004-1058, dtrsm :1152-1218).
// smem_raw: 3 * GB_SMALL_MAX * (GB_SMALL_MAX + 1) entries of T.
// ---------------------------------------------------------------------------

#define NB GB_SMALL_MAX
#define LDT (NB + 1)

template <typename T>
__host__ __device__ constexpr size_t small_smem() { return sizeof(T) * (3 * NB * LDT); }

template <typename T>
__device__ void factor_small_body(const gb_dev_pattern &P, int s, T *Lx, T *Linv,
                                  unsigned char *smem_raw, int *sfail_)
{
    T (*A)[LDT] = (T (*)[LDT])smem_raw;          // diagonal block, row-major rows
    T *X = (T *)smem_raw + NB * LDT;              // inverse, column j at X + j*LDT
    T *Bt = X + NB * LDT;                         // panel chunk, Bt[k*LDT + r]
    int &sfail = *sfail_;
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

#undef NB
#undef LDT

#endif
