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

// dst[rm[i]] += src[i] for i = i0, i0 + 32, ... < mc (one lane's share of a
// column; rm is injective, so each target takes one addition): eight rows
// at a time with every load issued before the adds, so that a long column
// costs few memory round trips
template <typename TL>
__device__ __forceinline__ void scatter_add_col(TL *__restrict__ dst, const TL *__restrict__ src,
                                                const int32_t *__restrict__ rm, int i0, int mc)
{
    int i = i0;
    for (; i + 7 * 32 < mc; i += 8 * 32) {
        int r[8];
        TL v[8], d[8];
#pragma unroll
        for (int u = 0; u < 8; u++) r[u] = rm[i + 32 * u];
#pragma unroll
        for (int u = 0; u < 8; u++) v[u] = src[i + 32 * u];
#pragma unroll
        for (int u = 0; u < 8; u++) d[u] = dst[r[u]];
#pragma unroll
        for (int u = 0; u < 8; u++) dst[r[u]] = d[u] + v[u];
    }
    for (; i < mc; i += 32) dst[rm[i]] += src[i];
}

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
            TL *dst = t < nscol ? panel + (int64_t)t * nsrow : cb + (int64_t)(t - nscol) * m - nscol;
            scatter_add_col<TL>(dst, src, rm, j + lane, mc);
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

// ---------------------------------------------------------------------------
// a front of at most MAXR (32 or 64) rows, whole, on one warp (rows r = lane,
// lane + 32): its assembly, LL' of the diagonal block, the block's inverse
// (kept for the sweeps), the panel rows below as products with that inverse,
// and the update block.  The front stays in the warp's shared region;
// nothing waits on another warp.  Every value is formed by the same
// operations in the same order as the block path (assemble_body,
// factor_small_body and the update-block tile), so the factor is the same
// bit for bit on either path:
//  * the diagonal block is factorized right-looking, which subtracts the
//    products L(i,k) L(j,k) from A(i,j) in the order k = 0, 1, ... exactly as
//    the block path's left-looking loop does;
//  * the inverse is the block path's column-by-column substitution;
//  * L21(r,c) = sum_k A21(r,k) Linv(c,k) summed from zero in k order;
//  * the update block is C - (sum_k L21(i,k) L21(j,k)), summed from zero.
// The reference forms the same quantities with dpotrf / dtrsm / dsyrk
// (t_cholmod_super_numeric_worker.c :1004-1058, :1152-1218, :640-720).
// ---------------------------------------------------------------------------

// bytes of one warp's shared region for fronts of at most MAXR rows
template <int MAXR, typename T>
__host__ __device__ constexpr size_t warp_front_smem()
{
    return sizeof(T) * (MAXR * (MAXR + 1) + MAXR) + sizeof(int) * (2 * MAXR + 2);
}

template <int MAXR, typename TA, typename T>
__device__ __noinline__ void warp_front(const gb_dev_pattern &P, int s, const int64_t *__restrict__ Sp,
                                        const int64_t *__restrict__ Si, const TA *__restrict__ Sx,
                                        const double *__restrict__ scale, double beta, T *Lx, T *CB,
                                        T *Linv, unsigned char *wsm)
{
    static_assert(MAXR == 32 || MAXR == 64, "fronts of 32 or 64 rows");
    constexpr int LD = MAXR + 1;
    constexpr unsigned FULL = 0xffffffffu;
    T *F = (T *)wsm;                       // front, column-major: F[j*LD + i]
    T *xd = F + MAXR * LD;                 // diagonal of the block inverse
    int *rows = (int *)(xd + MAXR);        // front row -> row of L
    int *spc = rows + MAXR;                // A's column starts, relative to Sp[k1]
    const int lane = threadIdx.x & 31;
    const int64_t k1 = P.Super[s];
    const int nscol = (int)(P.Super[s + 1] - k1);
    const int64_t psi = P.Pi[s];
    const int nsrow = (int)(P.Pi[s + 1] - psi);
    const int m = nsrow - nscol;
    T *panel = Lx + P.Px[s];

    // 1. zero the front; row indices; A's column starts
    for (int j = 0; j < nsrow; j++)
#pragma unroll
        for (int h = 0; h < MAXR; h += 32) F[j * LD + lane + h] = (T)0;
#pragma unroll
    for (int h = 0; h < MAXR; h += 32)
        rows[lane + h] = lane + h < nsrow ? P.Ls[psi + lane + h] : 0x7fffffff;
    const int64_t p0 = Sp[k1];
    for (int t = lane; t <= nscol; t += 32) spc[t] = (int)(Sp[k1 + t] - p0);
    __syncwarp();

    // 2. entries of A in the panel columns (rows at or below the diagonal)
    const int ne = spc[nscol];
    for (int q = lane; q < ne; q += 32) {
        int lo = 0, hi = nscol - 1;            // column: last t with spc[t] <= q
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (spc[mid] <= q) lo = mid; else hi = mid - 1;
        }
        const int t = lo;
        const int64_t k = k1 + t;
        const int64_t i = Si[p0 + q];
        if (i < k) continue;
        int a = t, b = nsrow;                  // front row of i
        while (a < b) {
            const int mid = (a + b) >> 1;
            if ((int64_t)rows[mid] < i) a = mid + 1; else b = mid;
        }
        if (a < nsrow && (int64_t)rows[a] == i) {
            double v = (double)Sx[p0 + q];
            if (i == k) v += beta;
            if (scale) v = v * (scale[i] * scale[k]);
            F[t * LD + a] = (T)v;
        }
    }
    __syncwarp();
    if (beta != 0.0) {                         // beta on diagonals A does not store
        for (int t = lane; t < nscol; t += 32) {
            const int64_t k = k1 + t;
            bool has = false;
            for (int q = spc[t]; q < spc[t + 1]; q++)
                if (Si[p0 + q] == k) { has = true; break; }
            if (!has) {
                double v = beta;
                if (scale) v *= scale[k] * scale[k];
                F[t * LD + t] += (T)v;
            }
        }
        __syncwarp();
    }

    // 3. extend-add of each child's update block, children in a fixed order
    // (loads of 8 columns issued before their adds; lane holds child rows
    // lane and lane + 32)
    for (int ci = P.child_ptr[s]; ci < P.child_ptr[s + 1]; ci++) {
        const int c = P.child_list[ci];
        const int ncc = (int)(P.Super[c + 1] - P.Super[c]);
        const int64_t pic = P.Pi[c];
        const int mc = (int)(P.Pi[c + 1] - pic) - ncc;
        const int32_t *rm = P.relmap + pic + ncc;
        const T *cbc = CB + P.cboff[c];
        int ri[MAXR / 32];
#pragma unroll
        for (int h = 0; h < MAXR / 32; h++) ri[h] = lane + 32 * h < mc ? rm[lane + 32 * h] : 0;
        for (int j0 = 0; j0 < mc; j0 += 8) {
            T v[MAXR / 32][8];
#pragma unroll
            for (int h = 0; h < MAXR / 32; h++)
#pragma unroll
                for (int u = 0; u < 8; u++) {
                    const int j = j0 + u, i = lane + 32 * h;
                    v[h][u] = (j < mc && i >= j && i < mc) ? cbc[i + (int64_t)j * mc] : (T)0;
                }
#pragma unroll
            for (int u = 0; u < 8; u++) {
                const int j = j0 + u;
                int rj = __shfl_sync(FULL, ri[0], j & 31);
                if (MAXR == 64) {
                    const int rj2 = __shfl_sync(FULL, ri[MAXR / 32 - 1], j & 31);
                    if (j >= 32) rj = rj2;
                }
#pragma unroll
                for (int h = 0; h < MAXR / 32; h++) {
                    const int i = lane + 32 * h;
                    if (j < mc && i >= j && i < mc) F[rj * LD + ri[h]] += v[h][u];
                }
            }
        }
        __syncwarp();
    }

    // 4. LL' of the diagonal block (rows and columns below nscol)
    int fail = -1;
    for (int k = 0; k < nscol; k++) {
        const T d = F[k * LD + k];
        if (!(d > (T)0)) { fail = k; break; }
        const T lkk = gb_sqrt<T>(d);
        __syncwarp();
#pragma unroll
        for (int h = 0; h < MAXR; h += 32) {
            const int r = lane + h;
            if (r == k) F[k * LD + k] = lkk;
            else if (r > k && r < nscol) F[k * LD + r] = F[k * LD + r] / lkk;
        }
        __syncwarp();
#pragma unroll
        for (int h = 0; h < MAXR; h += 32) {
            const int r = lane + h;
            if (r > k && r < nscol) {
                const T lik = F[k * LD + r];
                for (int j = k + 1; j <= r; j++) F[j * LD + r] -= lik * F[k * LD + j];
            }
        }
        __syncwarp();
    }

    // 5. X = inverse of the diagonal block, column j by the lane j mod 32:
    // X(j,j) in xd[j], X(i,j) for i > j in the block's upper triangle at
    // F[i*LD + j]
#pragma unroll
    for (int h = 0; h < MAXR; h += 32) {
        const int j = lane + h;
        if (j < nscol) {
            const T xjj = (T)1 / F[j * LD + j];
            xd[j] = xjj;
            for (int i = j + 1; i < nscol; i++) {
                T acc = (T)0;
                for (int k = j; k < i; k++) acc += F[k * LD + i] * (k == j ? xjj : F[k * LD + j]);
                F[i * LD + j] = -acc / F[i * LD + i];
            }
        }
    }
    __syncwarp();
    {
        T *out = Linv + P.linvoff[P.blkoff[s]];   // column-major, ld nscol
        for (int j = 0; j < nscol; j++)
            for (int r = lane; r < nscol; r += 32)
                out[r + (int64_t)j * nscol] = r < j ? (T)0 : (r == j ? xd[j] : F[r * LD + j]);
    }

    // 6. panel rows below: L21(r,c) = sum_{k<=c} A21(r,k) X(c,k), in place
    // from the last column, four columns at a time (A21(r,k), k <= c, is
    // still unchanged until the group's stores); each sum is formed from
    // zero in k order, the four and the lane's rows side by side
    const int ncols = fail >= 0 ? fail : nscol;
    for (int c0 = ncols - 1; c0 >= 0; c0 -= 4) {
        T acc[MAXR / 32][4];
#pragma unroll
        for (int h = 0; h < MAXR / 32; h++)
#pragma unroll
            for (int u = 0; u < 4; u++) acc[h][u] = (T)0;
        for (int k = 0; k <= c0; k++) {
            T a[MAXR / 32];
#pragma unroll
            for (int h = 0; h < MAXR / 32; h++) a[h] = F[k * LD + lane + 32 * h];
#pragma unroll
            for (int u = 0; u < 4; u++) {
                const int c = c0 - u;
                if (c >= 0 && k <= c) {
                    const T x = k == c ? xd[c] : F[c * LD + k];
#pragma unroll
                    for (int h = 0; h < MAXR / 32; h++) acc[h][u] += a[h] * x;
                }
            }
        }
#pragma unroll
        for (int h = 0; h < MAXR / 32; h++) {
            const int r = lane + 32 * h;
            if (r >= nscol && r < nsrow) {
#pragma unroll
                for (int u = 0; u < 4; u++)
                    if (c0 - u >= 0) F[(c0 - u) * LD + r] = acc[h][u];
            }
        }
    }
    __syncwarp();

    // 7. the panel (zero above the diagonal) and the update block
    for (int t = 0; t < nscol; t++)
        for (int r = lane; r < nsrow; r += 32)
            panel[r + (int64_t)t * nsrow] = r < t ? (T)0 : F[t * LD + r];
    // update block C - L21 L21', four columns at a time; each sum formed
    // from zero in k order
    T *cb = CB + P.cboff[s];
    for (int j0 = nscol; j0 < nsrow; j0 += 4) {
        T acc[MAXR / 32][4];
#pragma unroll
        for (int h = 0; h < MAXR / 32; h++)
#pragma unroll
            for (int u = 0; u < 4; u++) acc[h][u] = (T)0;
        if (fail < 0) {
            for (int k = 0; k < nscol; k++) {
                T a[MAXR / 32], b[4];
#pragma unroll
                for (int h = 0; h < MAXR / 32; h++) a[h] = F[k * LD + lane + 32 * h];
#pragma unroll
                for (int u = 0; u < 4; u++) b[u] = F[k * LD + min(j0 + u, MAXR)];
#pragma unroll
                for (int h = 0; h < MAXR / 32; h++)
#pragma unroll
                    for (int u = 0; u < 4; u++) acc[h][u] += a[h] * b[u];
            }
        }
#pragma unroll
        for (int h = 0; h < MAXR / 32; h++) {
            const int r = lane + 32 * h;
#pragma unroll
            for (int u = 0; u < 4; u++) {
                const int j = j0 + u;
                if (j < nsrow && r >= j && r < nsrow)
                    cb[(r - nscol) + (int64_t)(j - nscol) * m] = F[j * LD + r] - acc[h][u];
            }
        }
    }
    if (fail >= 0 && lane == 0) {
        P.fail[s] = fail;
        atomicExch(P.anyfail, 1);
    }
}

#endif
