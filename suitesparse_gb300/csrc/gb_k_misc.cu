// gb_k_misc.cu -- permutation with scaling, FP64 residual r = b - A x,
// norms for the backward error, diagonal extremes of the factor, clearing.
#include "gb_k_common.cuh"

// ---------------------------------------------------------------------------
// permutations, scaling, residual (FP64) and norms
// ---------------------------------------------------------------------------

// Y(k, r) = scale(k-th permuted) * B(perm[k], r), converting type
template <typename TB, typename TY>
__global__ void k_perm_in(int64_t n, int nrhs, const int64_t *__restrict__ perm,
                          const double *__restrict__ scale, const TB *__restrict__ B,
                          int64_t ldb, TY *Y, int64_t ldy)
{
    // one thread per row k, every column (the index and scale read once)
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n;
         k += (int64_t)gridDim.x * blockDim.x) {
        const int64_t i = perm ? perm[k] : k;
        const double sc = scale ? scale[i] : 1.0;
        for (int r = 0; r < nrhs; r++) {
            double v = (double)B[i + r * ldb];
            if (scale) v *= sc;
            Y[k + r * ldy] = (TY)v;
        }
    }
}

// X(perm[k], r) = scale(perm[k]) * Y(k, r)  [op 0: assign, op 1: add]
template <typename TY, typename TX>
__global__ void k_perm_out(int64_t n, int nrhs, const int64_t *__restrict__ perm,
                           const double *__restrict__ scale, const TY *__restrict__ Y,
                           int64_t ldy, TX *X, int64_t ldx, int add)
{
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n;
         k += (int64_t)gridDim.x * blockDim.x) {
        const int64_t i = perm ? perm[k] : k;
        const double sc = scale ? scale[i] : 1.0;
        for (int r = 0; r < nrhs; r++) {
            double v = (double)Y[k + r * ldy];
            if (scale) v *= sc;
            if (add) X[i + r * ldx] += (TX)v;
            else X[i + r * ldx] = (TX)v;
        }
    }
}

// R = B - A X with A in full compressed-row form (both triangles), FP64:
// one thread per row, up to four columns of X per pass so that each entry
// of A is read once per four right-hand sides; every sum runs over the row
// in order (a fixed order, the same for any number of columns).
__global__ void k_residual(int64_t n, int nrhs, const int64_t *__restrict__ Rp,
                           const int32_t *__restrict__ Rj, const double *__restrict__ Rx,
                           const double *__restrict__ X, int64_t ldx,
                           const double *__restrict__ B, int64_t ldb,
                           double *R, int64_t ldr)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x) {
        const int64_t p0 = Rp[i], p1 = Rp[i + 1];
        for (int r0 = 0; r0 < nrhs; r0 += 4) {
            const int nk = min(4, nrhs - r0);
            const double *x = X + r0 * ldx;
            double acc[4] = {0.0, 0.0, 0.0, 0.0};
            for (int64_t p = p0; p < p1; p++) {
                const double a = Rx[p];
                const int64_t j = Rj[p];
#pragma unroll
                for (int u = 0; u < 4; u++)
                    if (u < nk) acc[u] += a * x[j + u * ldx];
            }
#pragma unroll
            for (int u = 0; u < 4; u++)
                if (u < nk) R[i + (r0 + u) * ldr] = B[i + (r0 + u) * ldb] - acc[u];
        }
    }
}

// out[0] = min over the diagonal of L of L(k,k)^2, out[1] = max.  Grid-wide:
// per-block reduction, then 64-bit atomics on the bit patterns (the values
// are >= 0, for which IEEE order equals unsigned integer order).
__global__ void k_minmax_init(double *out)
{
    out[0] = __longlong_as_double(0x7FF0000000000000LL);   // +inf
    out[1] = 0.0;
}

template <typename T>
__global__ void k_diag_minmax(int nsuper, const int64_t *__restrict__ Super,
                              const int64_t *__restrict__ Pi, const int64_t *__restrict__ Px,
                              const T *__restrict__ Lx, double *out)
{
    __shared__ double smin[256], smax[256];
    double lo = __longlong_as_double(0x7FF0000000000000LL), hi = 0.0;
    const int lane = threadIdx.x & 31;
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int nwarps = (gridDim.x * blockDim.x) >> 5;
    for (int s = warp; s < nsuper; s += nwarps) {          // one warp per supernode
        const int nscol = (int)(Super[s + 1] - Super[s]);
        const int64_t nsrow = Pi[s + 1] - Pi[s];
        const T *panel = Lx + Px[s];
        for (int j = lane; j < nscol; j += 32) {
            const double d = (double)panel[j + j * nsrow];
            if (d != d) lo = 0.0;                       // NaN pivot: as small as can be
            else { lo = fmin(lo, d * d); hi = fmax(hi, d * d); }
        }
    }
    smin[threadIdx.x] = lo;
    smax[threadIdx.x] = hi;
    __syncthreads();
    for (int o = blockDim.x / 2; o > 0; o >>= 1) {
        if (threadIdx.x < o) {
            smin[threadIdx.x] = fmin(smin[threadIdx.x], smin[threadIdx.x + o]);
            smax[threadIdx.x] = fmax(smax[threadIdx.x], smax[threadIdx.x + o]);
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        atomicMin((unsigned long long *)&out[0], (unsigned long long)__double_as_longlong(smin[0]));
        atomicMax((unsigned long long *)&out[1], (unsigned long long)__double_as_longlong(smax[0]));
    }
}

// range of the factor's diagonal L(j,j) over every supernode: out[0] = min,
// out[1] = max (bit patterns of the positive values, 64-bit atomics),
// out[2] = nonzero when an entry is NaN.  out[0], out[1] start at +inf, 0.
template <typename T>
__global__ void k_diag_range(int nsuper, const int64_t *__restrict__ Super,
                             const int64_t *__restrict__ Pi, const int64_t *__restrict__ Px,
                             const T *__restrict__ Lx, double *out)
{
    __shared__ double smin[256], smax[256];
    __shared__ int snan;
    if (threadIdx.x == 0) snan = 0;
    __syncthreads();
    double lo = __longlong_as_double(0x7FF0000000000000LL), hi = 0.0;
    const int lane = threadIdx.x & 31;
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int nwarps = (gridDim.x * blockDim.x) >> 5;
    for (int s = warp; s < nsuper; s += nwarps) {          // one warp per supernode
        const int nscol = (int)(Super[s + 1] - Super[s]);
        const int64_t nsrow = Pi[s + 1] - Pi[s];
        const T *panel = Lx + Px[s];
        for (int j = lane; j < nscol; j += 32) {
            const double d = (double)panel[j + j * nsrow];
            if (d != d) snan = 1;
            else { lo = fmin(lo, d); hi = fmax(hi, d); }
        }
    }
    smin[threadIdx.x] = lo;
    smax[threadIdx.x] = hi;
    __syncthreads();
    for (int o = blockDim.x / 2; o > 0; o >>= 1) {
        if (threadIdx.x < o) {
            smin[threadIdx.x] = fmin(smin[threadIdx.x], smin[threadIdx.x + o]);
            smax[threadIdx.x] = fmax(smax[threadIdx.x], smax[threadIdx.x + o]);
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        atomicMin((unsigned long long *)&out[0], (unsigned long long)__double_as_longlong(smin[0]));
        atomicMax((unsigned long long *)&out[1], (unsigned long long)__double_as_longlong(smax[0]));
        if (snan) out[2] = 1.0;
    }
}

// per column r: out[3r] = max|R|, out[3r+1] = max|X|, out[3r+2] = max|B|
// (out zeroed first); grid-wide, 64-bit atomics on the bit patterns of the
// nonnegative maxima.  A NaN anywhere makes its maximum NaN (gb_maxnan,
// gb_maxbits), so a non-finite solution can never pass the test.
__global__ void k_colmax3(int64_t n, const double *__restrict__ R, int64_t ldr,
                          const double *__restrict__ X, int64_t ldx,
                          const double *__restrict__ B, int64_t ldb, double *out)
{
    __shared__ double sm[3][256];
    const int r = blockIdx.y;
    double a = 0, b = 0, c = 0;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x) {
        a = gb_maxnan(a, fabs(R[i + r * ldr]));
        b = gb_maxnan(b, fabs(X[i + r * ldx]));
        c = gb_maxnan(c, fabs(B[i + r * ldb]));
    }
    sm[0][threadIdx.x] = a;
    sm[1][threadIdx.x] = b;
    sm[2][threadIdx.x] = c;
    __syncthreads();
    for (int o = blockDim.x / 2; o > 0; o >>= 1) {
        if (threadIdx.x < o)
            for (int q = 0; q < 3; q++)
                sm[q][threadIdx.x] = gb_maxnan(sm[q][threadIdx.x], sm[q][threadIdx.x + o]);
        __syncthreads();
    }
    if (threadIdx.x == 0)
        for (int q = 0; q < 3; q++)
            atomicMax((unsigned long long *)&out[3 * r + q], gb_maxbits(sm[q][0]));
}

// max over rows of sum |A(i,:)| (for the backward error denominator)
__global__ void k_anorm_inf(int64_t n, const int64_t *__restrict__ Rp,
                            const double *__restrict__ Rx, double *out)
{
    __shared__ double sm[256];
    double best = 0;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x) {
        double acc = 0;
        for (int64_t p = Rp[i]; p < Rp[i + 1]; p++) acc += fabs(Rx[p]);
        best = gb_maxnan(best, acc);
    }
    sm[threadIdx.x] = best;
    __syncthreads();
    for (int o = blockDim.x / 2; o > 0; o >>= 1) {
        if (threadIdx.x < o) sm[threadIdx.x] = gb_maxnan(sm[threadIdx.x], sm[threadIdx.x + o]);
        __syncthreads();
    }
    if (threadIdx.x == 0)
        atomicMax((unsigned long long *)out, gb_maxbits(sm[0]));
}

// Segmented forms (one segment per independent block of A): block
// (chunk, r) reduces rows [lo, hi) of one segment, then 64-bit atomic max
// into that segment's slot (out zeroed first).  colmax: out[3 (seg nrhs + r)
// + q] for q = max|R|, max|X|, max|B|; anorm: out[seg] = max row sum |A|.
__global__ void k_colmax3_seg(const gb_seg_chunk *__restrict__ chunks, int nrhs,
                              const double *__restrict__ R, int64_t ldr,
                              const double *__restrict__ X, int64_t ldx,
                              const double *__restrict__ B, int64_t ldb, double *out)
{
    __shared__ double sm[3][256];
    const gb_seg_chunk ch = chunks[blockIdx.x];
    const int r = blockIdx.y;
    double a = 0, b = 0, c = 0;
    for (int64_t i = ch.lo + threadIdx.x; i < ch.hi; i += blockDim.x) {
        a = gb_maxnan(a, fabs(R[i + r * ldr]));
        b = gb_maxnan(b, fabs(X[i + r * ldx]));
        c = gb_maxnan(c, fabs(B[i + r * ldb]));
    }
    sm[0][threadIdx.x] = a;
    sm[1][threadIdx.x] = b;
    sm[2][threadIdx.x] = c;
    __syncthreads();
    for (int o = blockDim.x / 2; o > 0; o >>= 1) {
        if (threadIdx.x < o)
            for (int q = 0; q < 3; q++)
                sm[q][threadIdx.x] = gb_maxnan(sm[q][threadIdx.x], sm[q][threadIdx.x + o]);
        __syncthreads();
    }
    if (threadIdx.x == 0)
        for (int q = 0; q < 3; q++)
            atomicMax((unsigned long long *)&out[3 * ((int64_t)ch.seg * nrhs + r) + q],
                      gb_maxbits(sm[q][0]));
}

__global__ void k_anorm_seg(const gb_seg_chunk *__restrict__ chunks, const int64_t *__restrict__ Rp,
                            const double *__restrict__ Rx, double *out)
{
    __shared__ double sm[256];
    const gb_seg_chunk ch = chunks[blockIdx.x];
    double best = 0;
    for (int64_t i = ch.lo + threadIdx.x; i < ch.hi; i += blockDim.x) {
        double acc = 0;
        for (int64_t p = Rp[i]; p < Rp[i + 1]; p++) acc += fabs(Rx[p]);
        best = gb_maxnan(best, acc);
    }
    sm[threadIdx.x] = best;
    __syncthreads();
    for (int o = blockDim.x / 2; o > 0; o >>= 1) {
        if (threadIdx.x < o) sm[threadIdx.x] = gb_maxnan(sm[threadIdx.x], sm[threadIdx.x + o]);
        __syncthreads();
    }
    if (threadIdx.x == 0)
        atomicMax((unsigned long long *)&out[ch.seg], gb_maxbits(sm[0]));
}

// R(rows of the chunk, every column) = 0 when the chunk's segment is marked
// converged (act[seg] == 0): its correction is then zero
__global__ void k_zero_inactive(const gb_seg_chunk *__restrict__ chunks, const unsigned char *__restrict__ act,
                                double *R, int64_t ldr, int nrhs)
{
    const gb_seg_chunk ch = chunks[blockIdx.x];
    if (act[ch.seg]) return;
    for (int r = 0; r < nrhs; r++)
        for (int64_t i = ch.lo + threadIdx.x; i < ch.hi; i += blockDim.x) R[i + r * ldr] = 0.0;
}

// dst[q] = src[map[q]] (device-side value permutation)
__global__ void k_gather(int64_t n, const int64_t *__restrict__ map, const double *__restrict__ src,
                         double *__restrict__ dst)
{
    for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < n;
         q += (int64_t)gridDim.x * blockDim.x)
        dst[q] = src[map[q]];
}

// scale[i] = A(i,i)^-1/2 (1 when not positive or absent), scale_perm[k] =
// scale[Perm[k]]: the diagonal scaling D of the mixed factorization
__global__ void k_diag_scale(int64_t n, const int64_t *__restrict__ dmap, const double *__restrict__ Ax,
                             double *__restrict__ scale)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x) {
        const double d = dmap[i] >= 0 ? Ax[dmap[i]] : 0.0;
        scale[i] = d > 0 ? 1.0 / sqrt(d) : 1.0;
    }
}

__global__ void k_permute_vec(int64_t n, const int64_t *__restrict__ Perm, const double *__restrict__ v,
                              double *__restrict__ out)
{
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n;
         k += (int64_t)gridDim.x * blockDim.x)
        out[k] = v[Perm[k]];
}

// Simplicial layout of a factor computed on a supernodal pattern without
// explicit zeros: column j of L is the contiguous run Fx[src[j] ..
// src[j] + len[j]) (the supernode's column from its diagonal down), written
// to Lx[dst[j] ..].  ldl: D(j,j) = L(j,j)^2 on the diagonal and L(i,j) /
// L(j,j) below (the unit lower factor of L D L').  Columns j >= minor are
// zero (the factorization broke down at column minor).  One warp per column.
template <typename T>
__global__ void k_simplicial_gather(int64_t n, const int64_t *__restrict__ src,
                                    const int64_t *__restrict__ dst, const int64_t *__restrict__ len,
                                    int64_t minor, int ldl, const T *__restrict__ Fx, T *__restrict__ Lx)
{
    const int lane = threadIdx.x & 31;
    for (int64_t j = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5; j < n;
         j += ((int64_t)gridDim.x * blockDim.x) >> 5) {
        const int64_t s0 = src[j], d0 = dst[j], m = len[j];
        const bool zero = j >= minor;
        const T d = zero ? (T)0 : Fx[s0];
        for (int64_t t = lane; t < m; t += 32) {
            T v = zero ? (T)0 : Fx[s0 + t];
            if (ldl && !zero) v = (t == 0) ? d * d : v / d;
            Lx[d0 + t] = v;
        }
    }
}

// values of C = tril(A F): entry e = sum over its products q of
// Ax[pairs[2q]] Fx[pairs[2q+1]], from zero, in list order (the reference's
// order of multiply-adds)
template <typename T>
__global__ void k_pair_sum(int64_t nent, const int64_t *__restrict__ pptr,
                           const int64_t *__restrict__ pairs, const T *__restrict__ Ax,
                           const T *__restrict__ Fx, T *__restrict__ Cx)
{
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < nent;
         e += (int64_t)gridDim.x * blockDim.x) {
        T acc = (T)0;
        for (int64_t q = pptr[e]; q < pptr[e + 1]; q++) acc += Ax[pairs[2 * q]] * Fx[pairs[2 * q + 1]];
        Cx[e] = acc;
    }
}

// A complex supernodal factor and its real embedding: each complex entry
// l = re + i im is the 2 x 2 block [re -im; im re], so that supernode s of
// the embedding has twice the columns and rows of the complex supernode and
// starts at 4 px[s] (its index arrays are those of the embedding: Super_e,
// Pi_e, Px_e).  Complex entry (i, c) of s is at px[s] + c nsrow + i (pairs
// of reals); its block starts at row 2i of column 2c of the embedding.
// Gather: the first column of each block (re, im), the imaginary part of a
// diagonal entry zero, and every complex entry from zero_from on zero.
template <typename T>
__global__ void k_cx_gather(int64_t nsuper, const int64_t *__restrict__ Super_e,
                            const int64_t *__restrict__ Pi_e, const int64_t *__restrict__ Px_e,
                            const T *__restrict__ E, T *__restrict__ Lx, int64_t zero_from)
{
    for (int64_t s = blockIdx.x; s < nsuper; s += gridDim.x) {
        const int64_t nscol = (Super_e[s + 1] - Super_e[s]) / 2, nsrow = (Pi_e[s + 1] - Pi_e[s]) / 2;
        const int64_t pe = Px_e[s], pc = pe / 4, cnt = nscol * nsrow;
        for (int64_t t = threadIdx.x; t < cnt; t += blockDim.x) {
            const int64_t c = t / nsrow, i = t - c * nsrow, q = pc + t;
            T re = (T)0, im = (T)0;
            if (q < zero_from) {
                const int64_t src = pe + 2 * c * (2 * nsrow) + 2 * i;
                re = E[src];
                im = i == c ? (T)0 : E[src + 1];
            }
            Lx[2 * q] = re;
            Lx[2 * q + 1] = im;
        }
    }
}

// Scatter: the whole 2 x 2 block of every complex entry (a diagonal entry
// taken as real, so that the embedding stays lower triangular).
template <typename T>
__global__ void k_cx_scatter(int64_t nsuper, const int64_t *__restrict__ Super_e,
                             const int64_t *__restrict__ Pi_e, const int64_t *__restrict__ Px_e,
                             const T *__restrict__ Lx, T *__restrict__ E)
{
    for (int64_t s = blockIdx.x; s < nsuper; s += gridDim.x) {
        const int64_t nscol = (Super_e[s + 1] - Super_e[s]) / 2, nsrow = (Pi_e[s + 1] - Pi_e[s]) / 2;
        const int64_t pe = Px_e[s], pc = pe / 4, cnt = nscol * nsrow, lde = 2 * nsrow;
        for (int64_t t = threadIdx.x; t < cnt; t += blockDim.x) {
            const int64_t c = t / nsrow, i = t - c * nsrow, q = pc + t;
            const T re = Lx[2 * q], im = i == c ? (T)0 : Lx[2 * q + 1];
            const int64_t b0 = pe + 2 * c * lde + 2 * i, b1 = b0 + lde;
            E[b0] = re;
            E[b0 + 1] = im;
            E[b1] = -im;
            E[b1 + 1] = re;
        }
    }
}

// zero factor entries [from, to) (not-positive-definite clean-up)
template <typename T>
__global__ void k_zero_range(T *x, int64_t from, int64_t to)
{
    for (int64_t i = from + blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < to;
         i += (int64_t)gridDim.x * blockDim.x)
        x[i] = (T)0;
}


// FMA throughput probe: 8 independent multiply-add chains per thread.
template <typename T>
__global__ void __launch_bounds__(256) k_fma_peak(int iters, T seed, T *out)
{
    T a[8];
#pragma unroll
    for (int c = 0; c < 8; c++) a[c] = seed + (T)(threadIdx.x + c);
    const T m = (T)0.999999, b = (T)1e-7;
    for (int i = 0; i < iters; i++) {
#pragma unroll
        for (int c = 0; c < 8; c++) a[c] = a[c] * m + b;
    }
    T s = 0;
#pragma unroll
    for (int c = 0; c < 8; c++) s += a[c];
    if (s == (T)-12345.0) out[0] = s;     // keeps the chains live
}

// ---------------------------------------------------------------------------
// sparse right-hand sides and sparse solutions (cholmod_l_spsolve)
// ---------------------------------------------------------------------------

// Y(Bi[p], j) = Bx[p] for the packed columns 0 <= j < ncol of a chunk of B
// (Bp relative to the chunk); Y is zero on entry and the host has removed
// duplicate row indices, so no two lanes write one entry.  One warp per
// column; rows outside [0, n) are skipped.
template <typename T>
__global__ void k_sp_scatter(int64_t n, int64_t ncol, const int64_t *__restrict__ Bp,
                             const int64_t *__restrict__ Bi, const T *__restrict__ Bx, T *Y,
                             int64_t ldy)
{
    const int lane = threadIdx.x & 31;
    const int64_t warp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t j = warp; j < ncol; j += nwarps) {
        T *y = Y + j * ldy;
        for (int64_t p = Bp[j] + lane; p < Bp[j + 1]; p += 32) {
            const int64_t i = Bi[p];
            if (i >= 0 && i < n) y[i] = Bx[p];
        }
    }
}

// cnt[j * nseg + s] = number of entries x != 0 (a NaN counts) in rows
// s*GB_SP_SEG .. (s+1)*GB_SP_SEG-1 of column j of X.  Block (s, j), 256
// threads.
#define GB_SP_SEG 4096
template <typename T>
__global__ void __launch_bounds__(256) k_sp_count(int64_t n, int64_t nseg,
                                                  const T *__restrict__ X, int64_t ldx,
                                                  int64_t *cnt)
{
    __shared__ int w[8];
    const int64_t s = blockIdx.x, j = blockIdx.y;
    const int64_t r0 = s * GB_SP_SEG, r1 = r0 + GB_SP_SEG < n ? r0 + GB_SP_SEG : n;
    const T *x = X + j * ldx;
    int c = 0;
    for (int64_t i = r0 + threadIdx.x; i < r1; i += 256) c += x[i] != (T)0;
    c = __reduce_add_sync(0xffffffffu, c);
    if ((threadIdx.x & 31) == 0) w[threadIdx.x >> 5] = c;
    __syncthreads();
    if (threadIdx.x == 0) {
        int t = 0;
        for (int k = 0; k < 8; k++) t += w[k];
        cnt[j * nseg + s] = t;
    }
}

// The nonzero entries of segment s of column j of X, rows ascending, to
// Xi/Xx starting at off[j * nseg + s].  Block (s, j), 256 threads: per tile
// of 256 rows a ballot per warp and a prefix over the 8 warp counts.
template <typename T>
__global__ void __launch_bounds__(256) k_sp_compact(int64_t n, int64_t nseg,
                                                    const T *__restrict__ X, int64_t ldx,
                                                    const int64_t *__restrict__ off,
                                                    int64_t *Xi, T *Xx)
{
    __shared__ int w[8];
    const int64_t s = blockIdx.x, j = blockIdx.y;
    const int64_t r0 = s * GB_SP_SEG, r1 = r0 + GB_SP_SEG < n ? r0 + GB_SP_SEG : n;
    const T *x = X + j * ldx;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    int64_t base = off[j * nseg + s];
    for (int64_t t0 = r0; t0 < r1; t0 += 256) {
        const int64_t i = t0 + threadIdx.x;
        const T v = i < r1 ? x[i] : (T)0;
        const bool nz = i < r1 && v != (T)0;
        const unsigned b = __ballot_sync(0xffffffffu, nz);
        if (lane == 0) w[wid] = __popc(b);
        __syncthreads();
        int before = 0, total = 0;
        for (int k = 0; k < 8; k++) {
            const int c = w[k];
            before += k < wid ? c : 0;
            total += c;
        }
        if (nz) {
            const int64_t q = base + before + __popc(b & ((1u << lane) - 1u));
            Xi[q] = i;
            Xx[q] = v;
        }
        base += total;
        __syncthreads();
    }
}

extern "C" {

int gb_launch_fma_peak(int dtype, int iters, int blocks, float *ms, cudaStream_t st)
{
    cudaEvent_t e0, e1;
    void *out = NULL;
    if (cudaMalloc(&out, 16) != cudaSuccess) return 1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    cudaEventRecord(e0, st);
    if (dtype == 0) k_fma_peak<double><<<blocks, 256, 0, st>>>(iters, 1.0, (double *)out);
    else k_fma_peak<float><<<blocks, 256, 0, st>>>(iters, 1.0f, (float *)out);
    cudaEventRecord(e1, st);
    cudaEventSynchronize(e1);
    cudaEventElapsedTime(ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(out);
    return (int)cudaGetLastError();
}


// b_dtype/y_dtype: 0 double, 4 single
int gb_launch_perm_in(int64_t n, int nrhs, const int64_t *perm, const double *scale,
                      const void *B, int b_dtype, int64_t ldb, void *Y, int y_dtype,
                      int64_t ldy, cudaStream_t st)
{
    int g = gb_grid_for(n);
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
    int g = gb_grid_for(n);
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

// dtype: 0 double, 4 single
int gb_launch_sp_scatter(int64_t n, int64_t ncol, const int64_t *Bp, const int64_t *Bi,
                         const void *Bx, int dtype, void *Y, int64_t ldy, cudaStream_t st)
{
    int g = gb_grid_for(ncol * 32);
    if (dtype == 4) k_sp_scatter<float><<<g, 256, 0, st>>>(n, ncol, Bp, Bi, (const float *)Bx, (float *)Y, ldy);
    else k_sp_scatter<double><<<g, 256, 0, st>>>(n, ncol, Bp, Bi, (const double *)Bx, (double *)Y, ldy);
    return (int)cudaGetLastError();
}

int64_t gb_sp_nseg(int64_t n) { return (n + GB_SP_SEG - 1) / GB_SP_SEG; }

int gb_launch_sp_count(int64_t n, int64_t ncol, const void *X, int dtype, int64_t ldx,
                       int64_t *cnt, cudaStream_t st)
{
    const int64_t nseg = gb_sp_nseg(n);
    if (nseg == 0 || ncol == 0) return 0;
    if (nseg > 0x7fffffff || ncol > 65535) return (int)cudaErrorInvalidValue;
    dim3 g((unsigned)nseg, (unsigned)ncol);
    if (dtype == 4) k_sp_count<float><<<g, 256, 0, st>>>(n, nseg, (const float *)X, ldx, cnt);
    else k_sp_count<double><<<g, 256, 0, st>>>(n, nseg, (const double *)X, ldx, cnt);
    return (int)cudaGetLastError();
}

int gb_launch_sp_compact(int64_t n, int64_t ncol, const void *X, int dtype, int64_t ldx,
                         const int64_t *off, int64_t *Xi, void *Xx, cudaStream_t st)
{
    const int64_t nseg = gb_sp_nseg(n);
    if (nseg == 0 || ncol == 0) return 0;
    if (nseg > 0x7fffffff || ncol > 65535) return (int)cudaErrorInvalidValue;
    dim3 g((unsigned)nseg, (unsigned)ncol);
    if (dtype == 4) k_sp_compact<float><<<g, 256, 0, st>>>(n, nseg, (const float *)X, ldx, off, Xi, (float *)Xx);
    else k_sp_compact<double><<<g, 256, 0, st>>>(n, nseg, (const double *)X, ldx, off, Xi, (double *)Xx);
    return (int)cudaGetLastError();
}

int gb_launch_residual(int64_t n, int nrhs, const int64_t *Rp, const int32_t *Rj,
                       const double *Rx, const double *X, int64_t ldx, const double *B,
                       int64_t ldb, double *R, int64_t ldr, cudaStream_t st)
{
    int g = gb_grid_for(n);
    k_residual<<<g, 256, 0, st>>>(n, nrhs, Rp, Rj, Rx, X, ldx, B, ldb, R, ldr);
    return (int)cudaGetLastError();
}

int gb_launch_diag_minmax(int nsuper, const int64_t *Super, const int64_t *Pi,
                          const int64_t *Px, const void *Lx, int dtype, double *out,
                          cudaStream_t st)
{
    if (!out || !Lx) return (int)cudaErrorInvalidValue;
    k_minmax_init<<<1, 1, 0, st>>>(out);
    const int g = gb_grid_for(nsuper);
    if (dtype == 0) k_diag_minmax<double><<<g, 256, 0, st>>>(nsuper, Super, Pi, Px, (const double *)Lx, out);
    else k_diag_minmax<float><<<g, 256, 0, st>>>(nsuper, Super, Pi, Px, (const float *)Lx, out);
    return (int)cudaGetLastError();
}

int gb_launch_diag_range(int nsuper, const int64_t *Super, const int64_t *Pi,
                         const int64_t *Px, const void *Lx, int dtype, double *out,
                         cudaStream_t st)
{
    if (!out || !Lx || nsuper <= 0) return (int)cudaErrorInvalidValue;
    k_minmax_init<<<1, 1, 0, st>>>(out);
    if (cudaMemsetAsync(out + 2, 0, sizeof(double), st) != cudaSuccess) return 1;
    const int g = gb_grid_for(nsuper);
    if (dtype == 0) k_diag_range<double><<<g, 256, 0, st>>>(nsuper, Super, Pi, Px, (const double *)Lx, out);
    else k_diag_range<float><<<g, 256, 0, st>>>(nsuper, Super, Pi, Px, (const float *)Lx, out);
    return (int)cudaGetLastError();
}

int gb_launch_colmax3(int64_t n, int nrhs, const double *R, int64_t ldr, const double *X,
                      int64_t ldx, const double *B, int64_t ldb, double *out, cudaStream_t st)
{
    if (!out || !R || !X || !B) return (int)cudaErrorInvalidValue;
    if (cudaMemsetAsync(out, 0, sizeof(double) * 3 * nrhs, st) != cudaSuccess) return 1;
    int gx = (int)((n + 255) / 256);
    if (gx > 304) gx = 304;
    if (gx < 1) gx = 1;
    dim3 grid(gx, nrhs);
    k_colmax3<<<grid, 256, 0, st>>>(n, R, ldr, X, ldx, B, ldb, out);
    return (int)cudaGetLastError();
}

int gb_launch_anorm(int64_t n, const int64_t *Rp, const double *Rx, double *out, cudaStream_t st)
{
    if (cudaMemsetAsync(out, 0, sizeof(double), st) != cudaSuccess) return 1;
    k_anorm_inf<<<gb_grid_for(n), 256, 0, st>>>(n, Rp, Rx, out);
    return (int)cudaGetLastError();
}

int gb_launch_colmax3_seg(int64_t nchunk, const gb_seg_chunk *chunks, int64_t nseg, int nrhs,
                          const double *R, int64_t ldr, const double *X, int64_t ldx,
                          const double *B, int64_t ldb, double *out, cudaStream_t st)
{
    if (!out || !chunks || !R || !X || !B) return (int)cudaErrorInvalidValue;
    if (cudaMemsetAsync(out, 0, sizeof(double) * 3 * nseg * nrhs, st) != cudaSuccess) return 1;
    if (nchunk <= 0 || nrhs <= 0) return 0;
    dim3 grid((unsigned)nchunk, (unsigned)nrhs);
    k_colmax3_seg<<<grid, 256, 0, st>>>(chunks, nrhs, R, ldr, X, ldx, B, ldb, out);
    return (int)cudaGetLastError();
}

int gb_launch_zero_inactive(int64_t nchunk, const gb_seg_chunk *chunks, const unsigned char *act,
                            double *R, int64_t ldr, int nrhs, cudaStream_t st)
{
    if (nchunk <= 0 || nrhs <= 0) return 0;
    if (!chunks || !act || !R) return (int)cudaErrorInvalidValue;
    k_zero_inactive<<<(unsigned)nchunk, 256, 0, st>>>(chunks, act, R, ldr, nrhs);
    return (int)cudaGetLastError();
}

int gb_launch_anorm_seg(int64_t nchunk, const gb_seg_chunk *chunks, int64_t nseg, const int64_t *Rp,
                        const double *Rx, double *out, cudaStream_t st)
{
    if (!out || !chunks || !Rp || !Rx) return (int)cudaErrorInvalidValue;
    if (cudaMemsetAsync(out, 0, sizeof(double) * nseg, st) != cudaSuccess) return 1;
    if (nchunk <= 0) return 0;
    k_anorm_seg<<<(unsigned)nchunk, 256, 0, st>>>(chunks, Rp, Rx, out);
    return (int)cudaGetLastError();
}

int gb_launch_gather(int64_t n, const int64_t *map, const double *src, double *dst, cudaStream_t st)
{
    if (n <= 0) return 0;
    if (!map || !src || !dst) return (int)cudaErrorInvalidValue;
    k_gather<<<gb_grid_for(n), 256, 0, st>>>(n, map, src, dst);
    return (int)cudaGetLastError();
}

int gb_launch_diag_scale(int64_t n, const int64_t *dmap, const double *Ax, const int64_t *Perm,
                         double *scale, double *scale_perm, cudaStream_t st)
{
    if (n <= 0) return 0;
    if (!dmap || !Ax || !Perm || !scale || !scale_perm) return (int)cudaErrorInvalidValue;
    k_diag_scale<<<gb_grid_for(n), 256, 0, st>>>(n, dmap, Ax, scale);
    k_permute_vec<<<gb_grid_for(n), 256, 0, st>>>(n, Perm, scale, scale_perm);
    return (int)cudaGetLastError();
}

int gb_launch_simplicial_gather(int64_t n, const int64_t *src, const int64_t *dst,
                                const int64_t *len, int64_t minor, int ldl, const void *Fx,
                                void *Lx, int dtype, cudaStream_t st)
{
    if (n <= 0) return 0;
    int g = gb_grid_for(32 * n);
    if (dtype == 0)
        k_simplicial_gather<double><<<g, 256, 0, st>>>(n, src, dst, len, minor, ldl,
                                                        (const double *)Fx, (double *)Lx);
    else
        k_simplicial_gather<float><<<g, 256, 0, st>>>(n, src, dst, len, minor, ldl,
                                                       (const float *)Fx, (float *)Lx);
    return (int)cudaGetLastError();
}

int gb_launch_pair_sum(int64_t nent, const int64_t *pptr, const int64_t *pairs, const void *Ax,
                       const void *Fx, void *Cx, int dtype, cudaStream_t st)
{
    if (nent <= 0) return 0;
    int g = gb_grid_for(nent);
    if (dtype == 0)
        k_pair_sum<double><<<g, 256, 0, st>>>(nent, pptr, pairs, (const double *)Ax,
                                              (const double *)Fx, (double *)Cx);
    else
        k_pair_sum<float><<<g, 256, 0, st>>>(nent, pptr, pairs, (const float *)Ax,
                                             (const float *)Fx, (float *)Cx);
    return (int)cudaGetLastError();
}

int gb_launch_cx_gather(int64_t nsuper, const int64_t *Super_e, const int64_t *Pi_e,
                        const int64_t *Px_e, const void *E, void *Lx, int64_t zero_from, int dtype,
                        cudaStream_t st)
{
    if (nsuper <= 0) return 0;
    const int g = (int)(nsuper < 65535 ? nsuper : 65535);
    if (dtype == 0)
        k_cx_gather<double><<<g, 256, 0, st>>>(nsuper, Super_e, Pi_e, Px_e, (const double *)E,
                                               (double *)Lx, zero_from);
    else
        k_cx_gather<float><<<g, 256, 0, st>>>(nsuper, Super_e, Pi_e, Px_e, (const float *)E,
                                              (float *)Lx, zero_from);
    return (int)cudaGetLastError();
}

int gb_launch_cx_scatter(int64_t nsuper, const int64_t *Super_e, const int64_t *Pi_e,
                         const int64_t *Px_e, const void *Lx, void *E, int dtype, cudaStream_t st)
{
    if (nsuper <= 0) return 0;
    const int g = (int)(nsuper < 65535 ? nsuper : 65535);
    if (dtype == 0)
        k_cx_scatter<double><<<g, 256, 0, st>>>(nsuper, Super_e, Pi_e, Px_e, (const double *)Lx,
                                                (double *)E);
    else
        k_cx_scatter<float><<<g, 256, 0, st>>>(nsuper, Super_e, Pi_e, Px_e, (const float *)Lx,
                                               (float *)E);
    return (int)cudaGetLastError();
}

int gb_launch_zero_range(void *x, int dtype, int64_t from, int64_t to, cudaStream_t st)
{
    if (to <= from) return 0;
    int g = gb_grid_for(to - from);
    if (dtype == 0) k_zero_range<double><<<g, 256, 0, st>>>((double *)x, from, to);
    else k_zero_range<float><<<g, 256, 0, st>>>((float *)x, from, to);
    return (int)cudaGetLastError();
}


}  // extern "C"
