// gb_k_common.cuh -- device helpers shared by the kernel translation units
// (gb_k_*.cu): the pattern view passed to every kernel, searches, and the
// in-shared-memory dense LL' / triangular-solve building blocks.
#ifndef GB_K_COMMON_CUH
#define GB_K_COMMON_CUH

#include <cuda_runtime.h>
#include <stdint.h>
#include "gb_plan.h"

struct gb_dev_pattern {
    const int64_t *Super, *Pi, *Px, *cboff, *cbvoff;
    const int32_t *Ls, *relmap, *child_ptr, *child_list;
    const int32_t *blkoff;     // first 64-column diagonal block id of s
    const int64_t *linvoff;    // offset of each diagonal block's inverse
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

// Maximum that keeps NaN: fmax(a, NaN) returns a, which would let a
// solution holding NaN pass a backward-error test.  Operands are >= 0 or
// NaN.
__device__ __forceinline__ double gb_maxnan(double a, double b)
{
    return (b > a || b != b) ? b : a;
}

// Bit pattern for the 64-bit atomicMax of a maximum that is >= 0 or NaN:
// any NaN becomes the positive quiet NaN, which orders above +inf as an
// unsigned integer, so it survives every later atomicMax.
__device__ __forceinline__ unsigned long long gb_maxbits(double v)
{
    return v != v ? 0x7FF8000000000000ull : (unsigned long long)__double_as_longlong(v);
}

template <typename T> __device__ __forceinline__ T gb_sqrt(T x);
template <> __device__ __forceinline__ double gb_sqrt<double>(double x) { return sqrt(x); }
template <> __device__ __forceinline__ float gb_sqrt<float>(float x) { return sqrtf(x); }

// ---------------------------------------------------------------------------
// dense building blocks on one nb x nb block in shared memory (nb <= 64)
// ---------------------------------------------------------------------------

// Left-looking LL' of the lower block A (leading dimension NB+1): thread i
// owns row i; at column j it forms A(i,j) - sum_{k<j} L(i,k) L(j,k), thread j
// takes the square root, then rows below divide.  Two barriers per column.
// Returns the first column whose pivot is not positive (columns before it
// are final), or -1.
template <typename T, int NB>
__device__ int potrf_ll(T (*A)[NB + 1], int nb, int *sfail)
{
    const int i = threadIdx.x;
    if (i == 0) *sfail = -1;
    __syncthreads();
    for (int j = 0; j < nb; j++) {
        T sij = (T)0;
        if (i >= j && i < nb) {
            T acc = A[i][j];
            for (int k = 0; k < j; k++) acc -= A[i][k] * A[j][k];
            sij = acc;
            if (i == j) {
                if (!(acc > (T)0)) *sfail = j;
                else A[j][j] = gb_sqrt<T>(acc);
            }
        }
        __syncthreads();
        if (*sfail >= 0) return *sfail;
        if (i > j && i < nb) A[i][j] = sij / A[j][j];
        __syncthreads();
    }
    return -1;
}

// X = L^-1 of the factored lower block A: thread j forms column j by forward
// substitution into out + j*ldo (column-major X, zeros above the diagonal).
template <typename T, int NB>
__device__ void tri_inverse(const T (*A)[NB + 1], int nb, T *out, int ldo)
{
    const int j = threadIdx.x;
    if (j < nb) {
        T *x = out + (int64_t)j * ldo;
        for (int i = 0; i < j; i++) x[i] = (T)0;
        x[j] = (T)1 / A[j][j];
        for (int i = j + 1; i < nb; i++) {
            T acc = (T)0;
            for (int k = j; k < i; k++) acc += A[i][k] * x[k];
            x[i] = -acc / A[i][i];
        }
    }
}

// Panel triangular solve as a product with the block inverse:
// X(nr x nc) = B * Linv', with Bt[k*ldt + r] = B(r, k) and
// Lt[k*ldt + c] = Linv(c, k) in shared memory (256 threads, 4x4 each);
// only columns c < ncols are written to dst (column-major, ld).
template <typename T>
__device__ void trsm_tile(const T *Bt, const T *Lt, int ldt, int nr, int nc, int ncols,
                          T *dst, int64_t ld)
{
    const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
    T acc[4][4];
#pragma unroll
    for (int a = 0; a < 4; a++)
#pragma unroll
        for (int b = 0; b < 4; b++) acc[a][b] = (T)0;
    for (int k = 0; k < nc; k++) {
        T x[4], y[4];
#pragma unroll
        for (int a = 0; a < 4; a++) x[a] = Bt[k * ldt + ty + 16 * a];
#pragma unroll
        for (int b = 0; b < 4; b++) y[b] = Lt[k * ldt + tx + 16 * b];
#pragma unroll
        for (int a = 0; a < 4; a++)
#pragma unroll
            for (int b = 0; b < 4; b++) acc[a][b] += x[a] * y[b];
    }
#pragma unroll
    for (int a = 0; a < 4; a++) {
        const int r = ty + 16 * a;
#pragma unroll
        for (int b = 0; b < 4; b++) {
            const int cc = tx + 16 * b;
            if (r < nr && cc < ncols) dst[r + (int64_t)cc * ld] = acc[a][b];
        }
    }
}

// LL' of a 64 x 64 (nb <= 64) lower block in shared memory A (leading
// dimension 65) with 256 threads, blocked by 16 columns: warp 0 factors the
// 16 x 16 diagonal block in registers (lane = row, columns exchanged by
// shuffles), the rows below solve against it in registers, and the trailing
// lower part takes the rank-16 update.  Returns the first column whose
// pivot is not positive (earlier columns are final), or -1.
template <typename T>
__device__ int potrf64(T (*A)[65], int nb, int *sfail)
{
    const int tid = threadIdx.x;
    if (tid == 0) *sfail = -1;
    __syncthreads();
    for (int p0 = 0; p0 < nb; p0 += 16) {
        const int pw = min(16, nb - p0);
        if (tid < 32) {
            const int i = tid;
            T row[16];
#pragma unroll
            for (int k = 0; k < 16; k++) row[k] = (i < pw && k <= i) ? A[p0 + i][p0 + k] : (T)0;
            int bad = -1;
#pragma unroll
            for (int j = 0; j < 16; j++) {
                if (j < pw && bad < 0) {
                    const T d = __shfl_sync(0xffffffffu, row[j], j);
                    if (!(d > (T)0)) {
                        bad = j;
                    } else {
                        const T sd = gb_sqrt<T>(d);
                        if (i == j) row[j] = sd;
                        else if (i > j) row[j] /= sd;
#pragma unroll
                        for (int k = j + 1; k < 16; k++) {
                            const T lkj = __shfl_sync(0xffffffffu, row[j], k);
                            if (i >= k && k < pw) row[k] -= row[j] * lkj;
                        }
                    }
                }
            }
            if (i < pw) {
#pragma unroll
                for (int k = 0; k < 16; k++)
                    if (k <= i) A[p0 + i][p0 + k] = row[k];
            }
            if (i == 0 && bad >= 0) *sfail = p0 + bad;
        }
        __syncthreads();
        if (*sfail >= 0) return *sfail;
        // rows below the diagonal block: forward substitution in registers
        for (int r = p0 + pw + tid; r < nb; r += blockDim.x) {
            T x[16];
#pragma unroll
            for (int k = 0; k < 16; k++) x[k] = (k < pw) ? A[r][p0 + k] : (T)0;
#pragma unroll
            for (int j = 0; j < 16; j++) {
                if (j < pw) {
                    T v = x[j];
#pragma unroll
                    for (int k = 0; k < j; k++) v -= x[k] * A[p0 + j][p0 + k];
                    x[j] = v / A[p0 + j][p0 + j];
                }
            }
#pragma unroll
            for (int k = 0; k < 16; k++)
                if (k < pw) A[r][p0 + k] = x[k];
        }
        __syncthreads();
        // trailing lower part: rank-pw update, one (row, 8-column group) each
        const int t0 = p0 + pw, nt = nb - t0;
        const int ngroups = (nt + 7) / 8;
        for (int w = tid; w < nt * ngroups; w += blockDim.x) {
            const int r = t0 + w / ngroups, cb = t0 + 8 * (w % ngroups);
            if (cb > r) continue;
            T a[16];
#pragma unroll
            for (int k = 0; k < 16; k++) a[k] = (k < pw) ? A[r][p0 + k] : (T)0;
            for (int cc = cb; cc < cb + 8 && cc <= r; cc++) {
                T acc = A[r][cc];
#pragma unroll
                for (int k = 0; k < 16; k++) acc -= a[k] * A[cc][p0 + k];
                A[r][cc] = acc;
            }
        }
        __syncthreads();
    }
    return -1;
}

// X = L^-1 of the factored lower block A (leading dimension 65), formed in
// shared memory X (column j at X + j*65 by thread j < nb, four partial sums
// per entry) and then stored to out (column-major, leading dimension nb).
template <typename T>
__device__ void tri_inverse64(const T (*A)[65], int nb, T *X, T *out)
{
    const int j = threadIdx.x;
    if (j < nb) {
        T *x = X + j * 65;
        for (int i = 0; i < j; i++) x[i] = (T)0;
        x[j] = (T)1 / A[j][j];
        for (int i = j + 1; i < nb; i++) {
            T a0 = (T)0, a1 = (T)0, a2 = (T)0, a3 = (T)0;
            int k = j;
            for (; k + 3 < i; k += 4) {
                a0 += A[i][k] * x[k];
                a1 += A[i][k + 1] * x[k + 1];
                a2 += A[i][k + 2] * x[k + 2];
                a3 += A[i][k + 3] * x[k + 3];
            }
            for (; k < i; k++) a0 += A[i][k] * x[k];
            x[i] = -((a0 + a1) + (a2 + a3)) / A[i][i];
        }
    }
    __syncthreads();
    for (int idx = threadIdx.x; idx < nb * nb; idx += blockDim.x) {
        const int i = idx % nb, jj = idx / nb;
        out[i + (int64_t)jj * nb] = X[jj * 65 + i];
    }
}

// C(m x n) -= A(m x 64) B(n x 64)' with both operands staged whole in
// shared memory (As[k*65 + i], Bs[k*65 + i]); 256 threads, 4x4 each; store
// only r - c >= diag_off when lower.  k <= 64.
template <typename T>
__device__ void gemm_tile_k64(const T *A, int64_t lda, const T *B, int64_t ldb, T *C, int64_t ldc,
                              int m, int n, int k, bool lower, int diag_off, T *As, T *Bs)
{
    for (int idx = threadIdx.x; idx < 64 * 64; idx += 256) {
        const int i = idx & 63, kk = idx >> 6;
        As[kk * 65 + i] = (i < m && kk < k) ? A[i + (int64_t)kk * lda] : (T)0;
        Bs[kk * 65 + i] = (i < n && kk < k) ? B[i + (int64_t)kk * ldb] : (T)0;
    }
    __syncthreads();
    const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
    T acc[4][4];
#pragma unroll
    for (int i = 0; i < 4; i++)
#pragma unroll
        for (int j = 0; j < 4; j++) acc[i][j] = (T)0;
#pragma unroll 8
    for (int kk = 0; kk < k; kk++) {
        T a[4], b[4];
#pragma unroll
        for (int i = 0; i < 4; i++) a[i] = As[kk * 65 + ty + 16 * i];
#pragma unroll
        for (int j = 0; j < 4; j++) b[j] = Bs[kk * 65 + tx + 16 * j];
#pragma unroll
        for (int i = 0; i < 4; i++)
#pragma unroll
            for (int j = 0; j < 4; j++) acc[i][j] += a[i] * b[j];
    }
#pragma unroll
    for (int i = 0; i < 4; i++) {
        const int r = ty + 16 * i;
        if (r >= m) continue;
#pragma unroll
        for (int j = 0; j < 4; j++) {
            const int cc = tx + 16 * j;
            if (cc >= n) continue;
            if (lower && r - cc < diag_off) continue;
            C[r + (int64_t)cc * ldc] -= acc[i][j];
        }
    }
}

template <typename T> __device__ __forceinline__ T gb_rsqrt(T x);
template <> __device__ __forceinline__ double gb_rsqrt<double>(double x) { return rsqrt(x); }
template <> __device__ __forceinline__ float gb_rsqrt<float>(float x) { return rsqrtf(x); }

// One warp, lane i = row i of a 16 x 16 lower block held in registers
// (row[k] = A(i, k), k <= i; rows >= pw are zero): LL' in place, pivots by
// reciprocal square root (L(j,j) = d rsqrt(d), column j scaled by rsqrt(d)).
// rinv receives 1 / L(i,i) in lane i.  Returns the first column whose pivot
// is not positive (the same in every lane), or -1.
template <typename T>
__device__ __forceinline__ int warp_potrf16(T (&row)[16], T &rinv, int pw)
{
    const int i = threadIdx.x & 31;
    int bad = -1;
#pragma unroll
    for (int j = 0; j < 16; j++) {
        if (j < pw && bad < 0) {
            const T d = __shfl_sync(0xffffffffu, row[j], j);
            if (!(d > (T)0)) {
                bad = j;
            } else {
                const T r = gb_rsqrt<T>(d);
                if (i == j) { row[j] = d * r; rinv = r; }
                else if (i > j) row[j] *= r;
#pragma unroll
                for (int k = j + 1; k < 16; k++) {
                    const T lkj = __shfl_sync(0xffffffffu, row[j], k);
                    if (i >= k && k < pw) row[k] -= row[j] * lkj;
                }
            }
        }
    }
    return bad;
}

// One warp: lane c (< pv) forms column c of the inverse of the 16 x 16
// lower factor stored in A[p1.., p1..] (leading pv x pv block; zero
// elsewhere): x[r] = -(1 / L(r,r)) sum_{k<r} L(r, k) x[k] for r > c, with
// the factor read from shared memory (the same address in every lane) and
// 1 / L(r,r) taken from lane r's rinv.
template <typename T>
__device__ __forceinline__ void warp_trinv16(T (*A)[65], int p1, T rinv, T (&x)[16], int pv)
{
    const int c = threadIdx.x & 31;
    T rv[16];
#pragma unroll
    for (int r = 0; r < 16; r++) rv[r] = __shfl_sync(0xffffffffu, rinv, r);
#pragma unroll
    for (int r = 0; r < 16; r++) {
        T v = (T)0;
#pragma unroll
        for (int k = 0; k < r; k++) v += A[p1 + r][p1 + k] * x[k];
        x[r] = (r < pv && r >= c) ? ((r == c) ? rv[r] : -rv[r] * v) : (T)0;
    }
}

// Warp 0: diagonal 16 x 16 block of panel p1 (width pw1): take the rank-pwp
// update from the previous panel p0 (if p0 >= 0), factor, invert, store L
// into A and the inverse into X; on a non-positive pivot write its column
// to *sfail.
template <typename T>
__device__ __forceinline__ void diag_block16(T (*A)[65], T *X, int p1, int pw1, int p0, int pwp, int *sfail)
{
    const int i = threadIdx.x & 31;
    T row[16];
#pragma unroll
    for (int k = 0; k < 16; k++) row[k] = (i < pw1 && k <= i) ? A[p1 + i][p1 + k] : (T)0;
    if (p0 >= 0) {
        T a[16];
#pragma unroll
        for (int q = 0; q < 16; q++) a[q] = (i < pw1 && q < pwp) ? A[p1 + i][p0 + q] : (T)0;
#pragma unroll
        for (int k = 0; k < 16; k++) {
            if (k < pw1) {
                T s = (T)0;
#pragma unroll
                for (int q = 0; q < 16; q++) s += a[q] * A[p1 + k][p0 + q];
                if (k <= i) row[k] -= s;
            }
        }
    }
    T rinv = (T)0, x[16];
    const int bad = warp_potrf16<T>(row, rinv, pw1);
    const int pv = bad >= 0 ? bad : pw1;
    if (i < pw1) {
#pragma unroll
        for (int k = 0; k < 16; k++)
            if (k <= i) A[p1 + i][p1 + k] = row[k];
    }
    __syncwarp();
    warp_trinv16<T>(A, p1, rinv, x, pv);
    if (i < pv) {
#pragma unroll
        for (int r = 0; r < 16; r++)
            if (r >= i) X[(p1 + i) * 65 + p1 + r] = x[r];
    }
    if (bad >= 0 && i == 0) *sfail = p1 + bad;
}

// LL' and inverse of a 64 x 64 (nb <= 64) lower block in shared memory with
// 256 threads.  A (leading dimension 65) is overwritten by L; X receives
// L^-1 (X[c*65 + r] = Linv(r, c), zeros above the diagonal); Tm is scratch
// of 3*256 entries.  In 16-column panels: warp 0 factors and inverts the
// panel's diagonal block in registers; the rows below become A * inv(D)'
// (a half warp per row, operands by shuffle); then warp 0 applies the
// panel's update to the next diagonal block and factors it while the other
// warps update the rest of the trailing lower part.  The off-diagonal
// 16 x 16 blocks of the inverse follow in three waves, X_ij = -X_ii
// sum_{k=j}^{i-1} L_ik X_kj.  Returns the first column whose pivot is not
// positive, or -1; on failure the columns before it (of L and of the
// inverse) are final.
template <typename T>
__device__ int potrf_inv64(T (*A)[65], T *X, T *Tm, int nb, int *sfail)
{
    const int tid = threadIdx.x, warp = tid >> 5;
    for (int idx = tid; idx < 64 * 65; idx += blockDim.x) X[idx] = (T)0;
    if (tid == 0) *sfail = -1;
    __syncthreads();
    if (warp == 0) diag_block16<T>(A, X, 0, min(16, nb), -1, 0, sfail);
    __syncthreads();
    int nv = nb;
    for (int p0 = 0; p0 < nb; p0 += 16) {
        const int pw = min(16, nb - p0);
        const int f = *sfail;
        const int pv = (f >= 0) ? f - p0 : pw;
        // rows below the diagonal block: L(r, panel) = A(r, panel) inv(D)'
        const int rb = p0 + pw, nrows = nb - rb;
        for (int base = 0; base < nrows; base += 16) {
            const int rr = base + (tid >> 4), cc = tid & 15;
            const bool ok = rr < nrows;
            const T a = (ok && cc < pw) ? A[rb + rr][p0 + cc] : (T)0;
            T acc = (T)0;
#pragma unroll
            for (int q = 0; q < 16; q++) acc += __shfl_sync(0xffffffffu, a, q, 16) * X[(p0 + q) * 65 + p0 + cc];
            if (ok && cc < pv) A[rb + rr][p0 + cc] = acc;
        }
        if (f >= 0) { nv = f; break; }
        __syncthreads();
        if (rb < nb) {
            const int pw1 = min(16, nb - rb);
            if (warp == 0) {
                diag_block16<T>(A, X, rb, pw1, p0, pw, sfail);
            } else {
                // rows below the next diagonal block, columns rb..r
                const int t0 = rb + pw1, nt = nb - t0, ng = (nb - rb + 7) / 8;
                for (int w = tid - 32; w < nt * ng; w += blockDim.x - 32) {
                    const int r = t0 + w / ng, cb = rb + 8 * (w % ng);
                    if (cb > r) continue;
                    T a[16];
#pragma unroll
                    for (int q = 0; q < 16; q++) a[q] = (q < pw) ? A[r][p0 + q] : (T)0;
                    const int ce = min(cb + 8, r + 1);
                    for (int cc = cb; cc < ce; cc++) {
                        T s = (T)0;
#pragma unroll
                        for (int q = 0; q < 16; q++) s += a[q] * A[cc][p0 + q];
                        A[r][cc] -= s;
                    }
                }
            }
        }
        __syncthreads();
    }
    __syncthreads();
    // off-diagonal 16 x 16 blocks of the inverse, by distance d = i - j
    const int nbk = (nv + 15) / 16;
    for (int d = 1; d < nbk; d++) {
        const int nblk = nbk - d;          // blocks (j + d, j), j = 0..nblk-1
        for (int e = tid; e < nblk * 256; e += blockDim.x) {
            const int j = e / 256, rc = e % 256, r = rc / 16, cc = rc % 16, i = j + d;
            T acc = (T)0;
            for (int k = j; k < i; k++) {
#pragma unroll
                for (int q = 0; q < 16; q++)
                    acc += A[16 * i + r][16 * k + q] * X[(16 * j + cc) * 65 + 16 * k + q];
            }
            Tm[e] = acc;
        }
        __syncthreads();
        for (int e = tid; e < nblk * 256; e += blockDim.x) {
            const int j = e / 256, rc = e % 256, r = rc / 16, cc = rc % 16, i = j + d;
            T acc = (T)0;
#pragma unroll
            for (int q = 0; q < 16; q++)
                acc += X[(16 * i + q) * 65 + 16 * i + r] * Tm[j * 256 + q * 16 + cc];
            X[(16 * j + cc) * 65 + 16 * i + r] = -acc;
        }
        __syncthreads();
    }
    return nv < nb ? nv : -1;
}

// One 64 x 64 output tile of C -= A B' (SIMT): A is m x k (lda), B is n x k
// (ldb), both column-major; 16-deep k slices staged in As/Bs (each
// 16 x (64+4)); store only r - c >= diag_off when lower.  256 threads, 4x4.
template <typename T>
__device__ void gemm_tile_nt(const T *A, int64_t lda, const T *B, int64_t ldb, T *C, int64_t ldc,
                             int m, int n, int k, bool lower, int diag_off, T *As, T *Bs)
{
    constexpr int BK = 16, LDS = 68;
    const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
    T acc[4][4];
#pragma unroll
    for (int i = 0; i < 4; i++)
#pragma unroll
        for (int j = 0; j < 4; j++) acc[i][j] = (T)0;
    for (int k0 = 0; k0 < k; k0 += BK) {
        for (int idx = threadIdx.x; idx < 64 * BK; idx += 256) {
            const int i = idx & 63, kk = idx >> 6;
            const int kg = k0 + kk;
            As[kk * LDS + i] = (i < m && kg < k) ? A[i + (int64_t)kg * lda] : (T)0;
            Bs[kk * LDS + i] = (i < n && kg < k) ? B[i + (int64_t)kg * ldb] : (T)0;
        }
        __syncthreads();
#pragma unroll
        for (int kk = 0; kk < BK; kk++) {
            T a[4], b[4];
#pragma unroll
            for (int i = 0; i < 4; i++) a[i] = As[kk * LDS + ty + 16 * i];
#pragma unroll
            for (int j = 0; j < 4; j++) b[j] = Bs[kk * LDS + tx + 16 * j];
#pragma unroll
            for (int i = 0; i < 4; i++)
#pragma unroll
                for (int j = 0; j < 4; j++) acc[i][j] += a[i] * b[j];
        }
        __syncthreads();
    }
#pragma unroll
    for (int i = 0; i < 4; i++) {
        const int r = ty + 16 * i;
        if (r >= m) continue;
#pragma unroll
        for (int j = 0; j < 4; j++) {
            const int c = tx + 16 * j;
            if (c >= n) continue;
            if (lower && r - c < diag_off) continue;
            C[r + (int64_t)c * ldc] -= acc[i][j];
        }
    }
}

// FP32 tile update C[0:m, 0:n] -= A[0:m, 0:k] B[0:n, 0:k]' (m, n <= 64;
// column-major operands; lower: update only entries with row - col >=
// diag_off) with 256 threads.  Thread (tx, ty) = (tid % 16, tid / 16) owns
// rows 4tx..4tx+3 and columns 4ty..4ty+3; its C entries are read into
// registers before the k loop so their latency overlaps the first operand
// loads, and the products are summed from zero and subtracted once at the
// end (subtracting each product from C in turn loses accuracy in the
// Schur complement).  Operands move through shared memory in k chunks of 32
// (k-major, 68-float rows so a thread reads its 4 rows or columns as one
// float4), two stages: the next chunk is loaded into registers while the
// current one is multiplied.  S needs 2 x 2 x 32 x 68 floats.
__device__ __forceinline__ void gemm_tile_f32(const float *A, int64_t lda, const float *B, int64_t ldb,
                                              float *C, int64_t ldc, int m, int n, int k, bool lower,
                                              int diag_off, float *S)
{
    constexpr int BK = 32, LDS = 68, STAGE = 2 * BK * LDS;
    const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;
    float acc[4][4], cv[4][4];
#pragma unroll
    for (int j = 0; j < 4; j++) {
        const int cc = 4 * ty + j;
#pragma unroll
        for (int i = 0; i < 4; i++) {
            const int r = 4 * tx + i;
            cv[i][j] = (r < m && cc < n) ? C[r + (int64_t)cc * ldc] : 0.0f;
            acc[i][j] = 0.0f;
        }
    }
    // loader mapping: element q of this thread is row (tid & 63), k offset
    // (tid >> 6) + 4q of the chunk
    const int li = tid & 63, lk = tid >> 6;
    float ra[8], rb[8];
    auto load = [&](int k0) {
#pragma unroll
        for (int q = 0; q < 8; q++) {
            const int kg = k0 + lk + 4 * q;
            ra[q] = (li < m && kg < k) ? A[li + (int64_t)kg * lda] : 0.0f;
            rb[q] = (li < n && kg < k) ? B[li + (int64_t)kg * ldb] : 0.0f;
        }
    };
    auto store = [&](int st) {
        float *As = S + st * STAGE, *Bs = As + BK * LDS;
#pragma unroll
        for (int q = 0; q < 8; q++) {
            As[(lk + 4 * q) * LDS + li] = ra[q];
            Bs[(lk + 4 * q) * LDS + li] = rb[q];
        }
    };
    const int nch = (k + BK - 1) / BK;
    if (nch > 0) {
        load(0);
        store(0);
    }
    __syncthreads();
    for (int ch = 0; ch < nch; ch++) {
        const int st = ch & 1;
        if (ch + 1 < nch) load((ch + 1) * BK);
        const float *As = S + st * STAGE, *Bs = As + BK * LDS;
#pragma unroll 8
        for (int kk = 0; kk < BK; kk++) {
            const float4 a = *reinterpret_cast<const float4 *>(As + kk * LDS + 4 * tx);
            const float4 b = *reinterpret_cast<const float4 *>(Bs + kk * LDS + 4 * ty);
            const float av[4] = {a.x, a.y, a.z, a.w}, bv[4] = {b.x, b.y, b.z, b.w};
#pragma unroll
            for (int i = 0; i < 4; i++)
#pragma unroll
                for (int j = 0; j < 4; j++) acc[i][j] = fmaf(av[i], bv[j], acc[i][j]);
        }
        if (ch + 1 < nch) store(st ^ 1);
        __syncthreads();
    }
#pragma unroll
    for (int j = 0; j < 4; j++) {
        const int cc = 4 * ty + j;
#pragma unroll
        for (int i = 0; i < 4; i++) {
            const int r = 4 * tx + i;
            if (r < m && cc < n && !(lower && r - cc < diag_off)) C[r + (int64_t)cc * ldc] = cv[i][j] - acc[i][j];
        }
    }
}

// ---------------------------------------------------------------------------
// tensor-core tile update (tcgen05, kind::tf32, accumulator in TMEM)
// ---------------------------------------------------------------------------

#define GB_TC_SPIN (1 << 22)

// per block: TMEM accumulator (64 columns), the mbarrier the MMAs commit to,
// and its phase; ok = 0 after a wait gave up
struct gb_tc_ctx {
    uint32_t taddr;    // TMEM: two accumulators of 128 columns
    uint32_t mbar;     // two mbarriers (one per operand stage) at mbar, mbar + 8
    uint32_t phase;    // phase bit of each stage's mbarrier
    int ok;
};

#define GB_TC_COLS 256          // TMEM columns per block
#define GB_TC_SMEM (2 * 32768)  // two operand stages of 32 KB
#define GB_TC_MIN_K 128         // depth from which a tile runs on the tensor cores

__device__ __forceinline__ uint32_t gb_su32(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

// shared-memory matrix descriptor: K-major, no swizzle; core matrices of 8
// rows x 16 bytes, lbo = byte distance of core matrices adjacent along K,
// sbo = along M/N; bit 46 = descriptor version of tcgen05
__device__ __forceinline__ uint64_t gb_tc_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo)
{
    return (uint64_t)((saddr >> 4) & 0x3FFFu) | ((uint64_t)((lbo >> 4) & 0x3FFFu) << 16)
           | ((uint64_t)((sbo >> 4) & 0x3FFFu) << 32) | ((uint64_t)1 << 46);
}

__device__ __forceinline__ float gb_tf32_rna(float x)
{
    uint32_t r;
    asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
    return __uint_as_float(r);
}

// element (m, k) of a K-major tile with a K chunk of 32 (4-byte elements):
// lbo = 128 bytes, sbo = 1024 bytes
__device__ __forceinline__ uint32_t gb_tc_off(int m, int k)
{
    return (uint32_t)((m >> 3) * 1024 + (k >> 2) * 128 + (m & 7) * 16 + (k & 3) * 4);
}

__device__ __forceinline__ bool gb_mbar_wait(uint32_t mbar, uint32_t phase)
{
    for (int it = 0; it < GB_TC_SPIN; it++) {
        uint32_t done;
        asm volatile("{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
                     " selp.u32 %0, 1, 0, p;\n}" : "=r"(done) : "r"(mbar), "r"(phase) : "memory");
        if (done) return true;
    }
    return false;
}

// 32 lanes x 16 columns of 32-bit accumulator (warp w: TMEM lanes 32 w ..)
__device__ __forceinline__ void gb_tmem_ld16(uint32_t (&r)[16], uint32_t taddr)
{
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x16.b32 "
                 "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]),
                   "=r"(r[6]), "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]),
                   "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
                 : "r"(taddr) : "memory");
}

__device__ __forceinline__ void gb_tc_mma(uint32_t taddr, uint64_t a, uint64_t b, uint32_t idesc,
                                          uint32_t accumulate)
{
    asm volatile("{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
                 " tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n}"
                 :: "r"(taddr), "l"(a), "l"(b), "r"(idesc), "r"(accumulate) : "memory");
}

// One K chunk (32) of both operands into a stage: A' = [A_hi; A_lo] (128
// rows) and B' = [B_hi; B_lo] (128 rows), x_hi = x rounded to TF32, x_lo =
// x - x_hi, in the canonical K-major no-swizzle layout (gb_tc_off).  Element
// q of a thread: core matrix cm = 8 warp + q (rows 8 (cm & 7).., k 4 (cm >> 3)..),
// row 8 (cm & 7) + lane / 4, k 4 (cm >> 3) + lane % 4: a warp's store fills
// one 128-byte core matrix (no bank conflicts), its load reads 8 rows x 4
// columns (four 32-byte sectors).
__device__ __forceinline__ void gb_tc_stage(unsigned char *stage, int lane, int warp, const float (&xa)[8],
                                            const float (&xb)[8])
{
    unsigned char *Ap = stage, *Bp = stage + 16384;
#pragma unroll
    for (int q = 0; q < 8; q++) {
        const int cm = warp * 8 + q;
        const uint32_t off = (uint32_t)((cm & 7) * 1024 + (cm >> 3) * 128 + lane * 4);
        const float ah = gb_tf32_rna(xa[q]), bh = gb_tf32_rna(xb[q]);
        *(float *)(Ap + off) = ah;
        *(float *)(Ap + off + 8192) = xa[q] - ah;
        *(float *)(Bp + off) = bh;
        *(float *)(Bp + off + 8192) = xb[q] - bh;
    }
}

// C[0:m, 0:n] -= A[0:m, 0:k] B[0:n, 0:k]' (m, n <= 64, column-major; lower:
// only entries with row - col >= diag_off) on the tensor cores with 256
// threads.  FP32 operands are split x = hi + lo (hi = x rounded to TF32) and
// packed as A' = [A_hi; A_lo], B' = [B_hi; B_lo]; one MMA of
// tcgen05.mma.cta_group::1.kind::tf32, M = 128, N = 128, per K step of 8
// yields all four products hi*hi, hi*lo, lo*hi, lo*lo in the four quarters
// of the accumulator.  Consecutive K chunks of 32 alternate between two
// accumulators (TMEM columns 0-127 and 128-255), which halves the error of
// the tensor core's FP32 accumulation; the epilogue adds the quarters and
// the two accumulators in FP32 (max error near that of a sequential FP32
// sum: 3.7e-5 vs 2.7e-5 for 64 x 64 x 2048 of values in [-0.5, 0.5]).
// Pipeline: two operand stages in shared memory (GB_TC_SMEM), each with an
// mbarrier the MMAs commit to; the loads of chunk c + 2 are in flight while
// chunk c's MMAs run and chunk c + 1 is staged.  Every wait is bounded;
// returns false when one gave up (tc.ok = 0).
static __device__ __noinline__ bool gemm_tile_tc(const float *A, int64_t lda, const float *B, int64_t ldb,
                                                 float *C, int64_t ldc, int m, int n, int k, bool lower,
                                                 int diag_off, unsigned char *smem, gb_tc_ctx &tc)
{
    if (k <= 0) return true;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const uint32_t idesc = (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(128 >> 3) << 17)
                           | ((uint32_t)(128 >> 4) << 24);
    auto load = [&](float (&xa)[8], float (&xb)[8], int k0) {
#pragma unroll
        for (int q = 0; q < 8; q++) {
            const int cm = warp * 8 + q;
            const int r = (cm & 7) * 8 + (lane >> 2), kg = k0 + (cm >> 3) * 4 + (lane & 3);
            xa[q] = (r < m && kg < k) ? A[r + (int64_t)kg * lda] : 0.0f;
            xb[q] = (r < n && kg < k) ? B[r + (int64_t)kg * ldb] : 0.0f;
        }
    };
    const int nch = (k + 31) / 32;
    bool ok = true;
    auto step = [&](int c, const float (&xa)[8], const float (&xb)[8]) {
        const int st = c & 1;
        unsigned char *stage = smem + st * 32768;
        if (c >= 2) {
            // the MMAs of chunk c - 2 read this stage
            if (!gb_mbar_wait(tc.mbar + 8 * st, (tc.phase >> st) & 1u)) ok = false;
            tc.phase ^= 1u << st;
        }
        gb_tc_stage(stage, lane, warp, xa, xb);
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        __syncthreads();
        if (tid == 0) {
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            const uint32_t a0 = gb_su32(stage), b0 = gb_su32(stage + 16384);
#pragma unroll
            for (int j = 0; j < 4; j++)
                gb_tc_mma(tc.taddr + (uint32_t)(st * 128), gb_tc_desc(a0 + j * 256, 128, 1024),
                          gb_tc_desc(b0 + j * 256, 128, 1024), idesc, (c > 1 || j > 0) ? 1u : 0u);
            asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];"
                         :: "r"(tc.mbar + 8 * st) : "memory");
        }
    };
    float pa[2][8], pb[2][8];
#pragma unroll
    for (int u = 0; u < 2; u++)
        if (u < nch) load(pa[u], pb[u], u * 32);
    int issued = 0;
    for (int c = 0; c < nch && ok; c += 2) {
#pragma unroll
        for (int u = 0; u < 2; u++) {
            if (c + u < nch) {
                step(c + u, pa[u], pb[u]);
                issued = c + u + 1;
                if (c + u + 2 < nch) load(pa[u], pb[u], (c + u + 2) * 32);
            }
        }
        ok = __syncthreads_and(ok);
    }
    // the chunks whose MMAs were not waited for yet
    for (int c = issued >= 2 ? issued - 2 : 0; c < issued; c++) {
        const int st = c & 1;
        if (!gb_mbar_wait(tc.mbar + 8 * st, (tc.phase >> st) & 1u)) ok = false;
        tc.phase ^= 1u << st;
    }
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    if (!__syncthreads_and(ok)) {
        tc.ok = 0;
        return false;
    }
    // epilogue: warps 0-1 hold the rows of A_hi (TMEM lanes 0-63), warps 2-3
    // those of A_lo (lanes 64-127); columns j and 64 + j of an accumulator
    // are the products with B_hi and B_lo.  Each sums its quarters into a
    // 64 x 64 shared tile (T1: hi rows, T2: lo rows); then all threads
    // update C.
    float *T1 = (float *)smem, *T2 = T1 + 64 * 65;
    const bool two = nch > 1;
    if (warp < 4) {
        const int r = (warp & 1) * 32 + lane;
        float *T = warp < 2 ? T1 : T2;
        for (int c0 = 0; c0 < 64; c0 += 16) {
            uint32_t x[16], y[16];
            const uint32_t a = tc.taddr + ((uint32_t)(warp * 32) << 16) + (uint32_t)c0;
            gb_tmem_ld16(x, a);
            gb_tmem_ld16(y, a + 64u);
            asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
            float v[16];
#pragma unroll
            for (int q = 0; q < 16; q++) v[q] = __uint_as_float(x[q]) + __uint_as_float(y[q]);
            if (two) {
                gb_tmem_ld16(x, a + 128u);
                gb_tmem_ld16(y, a + 192u);
                asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
                for (int q = 0; q < 16; q++) v[q] += __uint_as_float(x[q]) + __uint_as_float(y[q]);
            }
#pragma unroll
            for (int q = 0; q < 16; q++) T[(c0 + q) * 65 + r] = v[q];
        }
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    for (int idx = tid; idx < 64 * 64; idx += blockDim.x) {
        const int r = idx & 63, col = idx >> 6;
        if (r < m && col < n && !(lower && r - col < diag_off))
            C[r + (int64_t)col * ldc] -= T1[col * 65 + r] + T2[col * 65 + r];
    }
    // the next task reuses shared memory and the accumulators
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    return true;
}

static inline __host__ __device__ gb_dev_pattern gb_to_dev(const gb_pattern_ptrs *p)
{
    gb_dev_pattern d;
    d.Super = p->Super; d.Pi = p->Pi; d.Px = p->Px; d.cboff = p->cboff;
    d.cbvoff = p->cbvoff; d.Ls = p->Ls; d.relmap = p->relmap;
    d.child_ptr = p->child_ptr; d.child_list = p->child_list;
    d.fail = p->fail; d.anyfail = p->anyfail;
    d.blkoff = p->blkoff; d.linvoff = p->linvoff;
    return d;
}

static inline int gb_grid_for(int64_t work)
{
    int64_t g = (work + 255) / 256;
    if (g < 1) g = 1;
    if (g > 152 * 16) g = 152 * 16;
    return (int)g;
}

#endif
