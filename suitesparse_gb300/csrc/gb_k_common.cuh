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
    const int64_t *imgbase;    // first operand image of s (tensor-core tiles), -1 if none
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

__device__ __forceinline__ void gb_img_store(const float (&acc)[4][4], int nr, int ncols, int m0,
                                             float *S, float *Imgdst);

// Panel triangular solve as a product with the block inverse:
// X(nr x nc) = B * Linv', with Bt[k*ldt + r] = B(r, k) and
// Lt[k*ldt + c] = Linv(c, k) in shared memory (256 threads, 4x4 each);
// only columns c < ncols are written to dst (column-major, ld).  FP32 with
// img: the block is also written as the split operand image of the
// tensor-core tile products (rows from m0; Bt and Lt, contiguous, serve as
// its 32 KB of staging space once the product is formed).
template <typename T>
__device__ void trsm_tile(const T *Bt, const T *Lt, int ldt, int nr, int nc, int ncols,
                          T *dst, int64_t ld, float *img = nullptr, int m0 = 0)
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
    if constexpr (sizeof(T) == 4) {
        if (img) {
            __syncthreads();
            gb_img_store(acc, nr, ncols, m0, (float *)Bt, img);
        }
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

// One warp, lane i = row i of the lower n x n (n <= 32) block held in
// registers (row[k] = A(i, k) for k <= i, zero elsewhere and in rows >= n):
// LL' in place, left-looking by columns.  Column j: every lane forms
// A(i, j) - sum_{k<j} L(i, k) L(j, k) from its own row (registers) and row
// j of L read from shared memory (S[j][k], the same address on every lane:
// a broadcast), subtracting the terms in the order k = 0, 1, ... (the
// products the right-looking form subtracts, in the same order, so the
// factor is the same bit for bit); lane j's value is the pivot d, passed
// through shared memory; L(j,j) = d rsqrt(d), the column scaled by
// rsqrt(d), and every lane stores its L(i, j) into S[i][j].  Only two warp
// barriers and no shuffles per column: the loads of a column's dot
// products are independent and overlap (3.3 us for 32 columns against
// 11.4 us for the right-looking form with a shuffle per update, measured
// alone on a GB300).  From the first pivot that is not positive on, the
// columns are formed from a unit pivot (finite, never read).  rinv
// receives 1 / L(i,i) in lane i (0 from the failing column on).  S: 32 x
// 33 and Pv: 2 entries of shared memory.  Returns the first column whose
// pivot is not positive (earlier columns are final), or -1.
template <typename T>
__device__ __forceinline__ int warp_chol32(T (&row)[32], T &rinv, int n, T (*S)[33], T *Pv)
{
    const int i = threadIdx.x & 31;
    int bad = n;
    rinv = (T)0;
#pragma unroll
    for (int j = 0; j < 32; j++) {
        T acc = row[j];
#pragma unroll
        for (int k = 0; k < j; k++) acc = acc - row[k] * S[j][k];
        if (i == j) Pv[j & 1] = acc;
        __syncwarp();
        const T d = Pv[j & 1];
        if (j < n && !(d > (T)0) && bad == n) bad = j;
        const T dd = j < bad ? d : (T)1;
        const T r = gb_rsqrt<T>(dd);
        const T lj = i == j ? dd * r : (i > j ? acc * r : row[j]);
        row[j] = lj;
        if (i == j) rinv = j < bad ? r : (T)0;
        S[i][j] = lj;
        __syncwarp();
    }
    return bad < n ? bad : -1;
}

// One warp: X = L^-1 of the lower n x n factor stored at A[o + i][o + k]
// (shared memory, leading dimension 65), lane j forming column j in
// registers: X(j, j) = 1 / L(j, j) (rinv of lane j), then row by row
// X(i, j) = -(1 / L(i, i)) sum_{m = j}^{i-1} L(i, m) X(m, j), the factor read
// by broadcast (every lane the same address).  Column j goes to
// X[(o + j) 65 + o + i] (rows i < j zero; rows >= n zero).
template <typename T>
__device__ __forceinline__ void warp_inv32(const T (*A)[65], int o, T rinv, int n, T *X)
{
    const int j = threadIdx.x & 31;
    T x[32];
#pragma unroll
    for (int i = 0; i < 32; i++) {
        const T ri = __shfl_sync(0xffffffffu, rinv, i);
        T v0 = (T)0, v1 = (T)0;
#pragma unroll
        for (int m = 0; m + 1 < i; m += 2) {
            v0 += A[o + i][o + m] * x[m];
            v1 += A[o + i][o + m + 1] * x[m + 1];
        }
        if (i & 1) v0 += A[o + i][o + i - 1] * x[i - 1];
        x[i] = (i >= n) ? (T)0 : (i == j ? ri : (i > j ? -ri * (v0 + v1) : (T)0));
    }
#pragma unroll
    for (int i = 0; i < 32; i++) X[(o + j) * 65 + o + i] = x[i];
}

// One copy each of the unrolled 32 x 32 routines, called for both
// diagonal sub-blocks of a 64 x 64 block: the executor runs them cold (one
// diagonal step between many other tasks), and fetching a second inlined
// copy of ~1,100 instructions cost more than the call.  chol32_block loads
// lane i's row of the block at A[o + i][o + k] (k <= i, rows < n) into
// registers, factors it (warp_chol32, S and Pv its scratch), stores it back
// and leaves 1 / L(i,i) in rinv[i]; inv32_block forms the inverse from the
// factor and rinv (warp_inv32).
template <typename T>
__device__ __noinline__ int chol32_block(T (*A)[65], int o, int n, T *rinv, T (*S)[33], T *Pv)
{
    const int lane = threadIdx.x & 31;
    T row[32], r;
#pragma unroll
    for (int k = 0; k < 32; k++) row[k] = (lane < n && k <= lane) ? A[o + lane][o + k] : (T)0;
    const int bad = warp_chol32<T>(row, r, n, S, Pv);
    if (lane < n) {
#pragma unroll
        for (int k = 0; k < 32; k++)
            if (k <= lane) A[o + lane][o + k] = row[k];
    }
    rinv[lane] = r;
    return bad;
}

template <typename T>
__device__ __noinline__ void inv32_block(const T (*A)[65], int o, const T *rinv, int n, T *X)
{
    warp_inv32<T>(A, o, rinv[threadIdx.x & 31], n, X);
}

// LL' and inverse of a 64 x 64 (nb <= 64) lower block in shared memory with
// 256 threads, in 2 x 2 blocks of 32: A = [A11; A21 A22] (leading dimension
// 65) is overwritten by L; X receives L^-1 (X[c*65 + r] = Linv(r, c), zeros
// above the diagonal); Tm is scratch of 32 x 33 + 66 entries.
//   L11 = chol(A11)                          (warp 0, registers)
//   X11 = L11^-1                             (warp 1, meanwhile:)
//   L21 = A21 L11^-T by substitution         (warp 2)
//   S = A22 - L21 L21', L22 = chol(S), X22 = L22^-1   (warps 0, 2-7; warp 0)
//   X21 = -X22 (L21 X11)                     (all threads, two products)
// The inverse of the first diagonal block is off the dependency chain: the
// warps that form L21, S and L22 synchronize on a named barrier of their
// own (224 threads) while warp 1 inverts.  Returns the first column whose
// pivot is not positive, or -1; on failure the columns before it (of L,
// its rows below included, and of the inverse) are final.
template <typename T>
__device__ int potrf_inv64(T (*A)[65], T *X, T *Tm, int nb, int *sfail)
{
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int n1 = min(32, nb), n2 = nb - n1;
    T *rinv11 = Tm + 32 * 33, *rinv22 = rinv11 + 32, *Pv = rinv22 + 32;
    for (int idx = tid; idx < 64 * 65; idx += blockDim.x) X[idx] = (T)0;
    if (tid == 0) *sfail = -1;
    __syncthreads();
    if (warp == 0) {
        const int bad = chol32_block<T>(A, 0, n1, rinv11, (T (*)[33])Tm, Pv);
        if (lane == 0 && bad >= 0) *sfail = bad;
    }
    __syncthreads();
    const int f1 = *sfail, v1 = f1 >= 0 ? f1 : n1;
    if (warp == 1) {
        inv32_block<T>(A, 0, rinv11, v1, X);
    } else if (n2 > 0) {
        // warps 0 and 2-7 (224 threads, named barrier 1)
        const int t7 = warp == 0 ? lane : tid - 32;
        if (warp == 2 && lane < n2) {
            // row 32 + lane of L21: L11 L21(i, :)' = A21(i, :)', columns < v1
            T a[32];
#pragma unroll
            for (int k = 0; k < 32; k++) a[k] = A[32 + lane][k];
#pragma unroll
            for (int c = 0; c < 32; c++) {
                if (c < v1) {
                    const T x = a[c] * rinv11[c];
                    a[c] = x;
#pragma unroll
                    for (int k = c + 1; k < 32; k++) a[k] -= x * A[k][c];
                }
            }
#pragma unroll
            for (int k = 0; k < 32; k++)
                if (k < v1) A[32 + lane][k] = a[k];
        }
        asm volatile("bar.sync 1, 224;" ::: "memory");
        if (f1 < 0) {
            // S = A22 - L21 L21' (lower)
            for (int o = t7; o < n2 * n2; o += 224) {
                const int i = o / n2, j = o - i * n2;
                if (j > i) continue;
                T a0 = (T)0, a1 = (T)0;
#pragma unroll
                for (int k = 0; k < 32; k += 2) {
                    a0 += A[32 + i][k] * A[32 + j][k];
                    a1 += A[32 + i][k + 1] * A[32 + j][k + 1];
                }
                A[32 + i][32 + j] -= a0 + a1;
            }
            asm volatile("bar.sync 1, 224;" ::: "memory");
            if (warp == 0) {
                const int bad = chol32_block<T>(A, 32, n2, rinv22, (T (*)[33])Tm, Pv);
                __syncwarp();
                inv32_block<T>(A, 32, rinv22, bad >= 0 ? bad : n2, X);
                if (lane == 0 && bad >= 0) *sfail = 32 + bad;
            }
        }
    }
    __syncthreads();
    if (f1 >= 0 || n2 <= 0) return f1;
    // T = L21 X11: T(i, c) = sum_k L21(i, k) X11(k, c) (X11 zero above its
    // diagonal; rows i >= n2 of T zero)
    for (int o = tid; o < 32 * 32; o += blockDim.x) {
        const int i = o >> 5, c = o & 31;
        T a0 = (T)0, a1 = (T)0;
        if (i < n2) {
#pragma unroll
            for (int k = 0; k < 32; k += 2) {
                a0 += A[32 + i][k] * X[c * 65 + k];
                a1 += A[32 + i][k + 1] * X[c * 65 + k + 1];
            }
        }
        Tm[i * 33 + c] = a0 + a1;
    }
    __syncthreads();
    // X21(i, c) = -sum_k X22(i, k) T(k, c) (X22 zero above its diagonal)
    for (int o = tid; o < n2 * 32; o += blockDim.x) {
        const int i = o >> 5, c = o & 31;
        T a0 = (T)0, a1 = (T)0;
#pragma unroll
        for (int k = 0; k < 32; k += 2) {
            a0 += X[(32 + k) * 65 + 32 + i] * Tm[k * 33 + c];
            a1 += X[(32 + k + 1) * 65 + 32 + i] * Tm[(k + 1) * 33 + c];
        }
        X[c * 65 + 32 + i] = -(a0 + a1);
    }
    __syncthreads();
    return *sfail;
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
// tensor-core tile products (tcgen05, kind::tf32, accumulators in TMEM) with
// operands staged by bulk asynchronous copies from split panel images
// ---------------------------------------------------------------------------

#define GB_TC_SPIN (1 << 22)

// TMEM columns per block: two accumulators of 128 columns (the executor's
// shared memory keeps at most 2 blocks per SM: 512 of 512 columns)
#define GB_TC_COLS 256
// operand stages in shared memory, 32 KB each (A' and B' of one K chunk)
#define GB_IMG_NS 3
#define GB_TC_SMEM (GB_IMG_NS * 32768)
// K chunks (32 deep) accumulated in one TMEM accumulator before it is
// drained into FP32 registers: 2 (8 MMA steps) keeps the factor's error
// near that of FP32 sums on the CUDA cores (1.37e-7 vs 1.24e-7 relative to
// the FP64 factor on a 40^3 Laplacian; with 8 chunks 1.67e-7, and the
// 64^3 case's refinement sometimes needed a third step)
#define GB_IMG_GROUP 2
// one image: a 64-row block of one 64-column panel, split x = hi + lo
// (hi = x rounded to TF32), as two K chunks of 32, each [hi rows 0-63;
// lo rows 64-127] x 32 in the canonical K-major no-swizzle layout of
// gb_img_off: 2 x 16 KB
#define GB_IMG_FLOATS GB_IMG_FLOATS_HOST

// per block: TMEM accumulators, mbarriers and their phases; ok = 0 after a
// wait gave up.  Barriers (8 bytes each from mbar): full[s] = s (operand
// stage s landed), empty[s] = GB_IMG_NS + s (the MMAs reading stage s are
// done), accd = 2 GB_IMG_NS (an accumulator's MMAs are done).  phase bit i
// is the parity of barrier i's next completion.
struct gb_tc_ctx {
    uint32_t taddr;
    uint32_t mbar;
    uint32_t phase;
    int ok;
};
#define GB_TC_NBAR (2 * GB_IMG_NS + 1)

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

// byte offset of element (m, k) (m < 128: rows 64-127 are the lo parts;
// k < 64) in an image: chunk k / 32 of 16 KB, then core matrices of 8 rows
// x 4 k (lbo = 128 bytes along K, sbo = 1024 bytes along M)
__device__ __forceinline__ uint32_t gb_img_off(int m, int k)
{
    return (uint32_t)((k >> 5) * 16384 + (m >> 3) * 1024 + ((k & 31) >> 2) * 128 + (m & 7) * 16
                      + (k & 3) * 4);
}

// image of 64-row block r of panel b of a supernode whose images start at
// image ibase, with R row blocks (only blocks r >= b are stored)
__device__ __forceinline__ const float *gb_img_ptr(const float *Img, int64_t ibase, int R, int b, int r)
{
    return Img + ((int64_t)ibase + (int64_t)b * R - ((int64_t)b * (b - 1)) / 2 + (r - b))
                 * (int64_t)GB_IMG_FLOATS;
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

// thread: wait for barrier i's next completion (bounded), track its parity
__device__ __forceinline__ bool gb_tc_wait(gb_tc_ctx &tc, int i)
{
    const bool ok = gb_mbar_wait(tc.mbar + 8u * (uint32_t)i, (tc.phase >> i) & 1u);
    tc.phase ^= 1u << i;
    return ok;
}

// 32 lanes x 16 columns of 32-bit accumulator (warp w: TMEM lanes 32 (w % 4) ..)
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

// Write the 64 x 64 panel block held by a trsm_tile thread layout (acc
// rows ty + 16 a, columns tx + 16 b; rows rr >= nr or columns >= ncols are
// zero) as an image at Imgdst: image row m0 + rr (rows 0..m0-1 zero), split
// into TF32 hi and FP32 lo parts.  Staged through S (32 KB of shared
// memory, free when called) so that the global stores are whole 16-byte
// vectors; all 256 threads.  The image is read later by the bulk-copy
// (async) proxy of another block, hence the proxy fence after the stores.
__device__ __forceinline__ void gb_img_store(const float (&acc)[4][4], int nr, int ncols, int m0,
                                             float *S, float *Imgdst)
{
    const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
    unsigned char *Sb = (unsigned char *)S;
#pragma unroll
    for (int a = 0; a < 4; a++) {
        const int rr = ty + 16 * a, m = m0 + rr;
        if (m >= 64) continue;
#pragma unroll
        for (int b = 0; b < 4; b++) {
            const int k = tx + 16 * b;
            const float v = (rr < nr && k < ncols) ? acc[a][b] : 0.0f;
            const float h = gb_tf32_rna(v);
            const uint32_t off = gb_img_off(m, k);
            *(float *)(Sb + off) = h;
            *(float *)(Sb + off + 8192) = v - h;
        }
    }
    for (int idx = threadIdx.x; idx < m0 * 64; idx += blockDim.x) {
        const uint32_t off = gb_img_off(idx >> 6, idx & 63);
        *(float *)(Sb + off) = 0.0f;
        *(float *)(Sb + off + 8192) = 0.0f;
    }
    __syncthreads();
    const float4 *src = (const float4 *)S;
    float4 *dst = (float4 *)Imgdst;
    for (int q = threadIdx.x; q < GB_IMG_FLOATS / 4; q += blockDim.x) dst[q] = src[q];
    asm volatile("fence.proxy.async.global;" ::: "memory");
    __syncthreads();
}

// C[i, j] -= sum over K chunks c = 0..nch-1 of A(i, k) B(j, k) for the 64 x
// 64 output of rows i in [i0, i1), columns j in [j0, j1) (lower: only i >=
// j), C[c_off + i + j ldc] in global memory.  Chunk c is K chunk c & 1 of
// panel b0 + c / 2; A's operand is the image of row block ra, B's of row
// block rb (gb_img_ptr).  One MMA of tcgen05.mma.cta_group::1.kind::tf32,
// M = 128, N = 128, per K step of 8 multiplies A' = [A_hi; A_lo] by B' =
// [B_hi; B_lo]: the four quarters of the accumulator hold hi*hi, hi*lo,
// lo*hi, lo*lo.  Thread 0 issues the bulk copies of each chunk's two
// images into one of GB_IMG_NS stages (mbarrier with transaction count)
// and the MMAs (committed to the stage's empty barrier), GB_IMG_NS - 1
// chunks ahead.  Every GB_IMG_GROUP chunks the accumulator alternates, and
// the one just finished is drained by all threads into FP32 registers (sums
// over at most 64 of K, then summed with round-to-nearest adds: the tensor
// core's FP32 accumulation truncates, and its error would otherwise grow
// linearly with K).  The epilogue adds the hi and lo rows' sums
// through shared memory and updates C, whose values were loaded while the
// operands were in flight.  Every wait is bounded; returns false when one
// gave up (tc.ok = 0), after waiting (bounded) for the copies and MMAs in
// flight.
static __device__ __noinline__ bool gemm_img_tc(const float *Img, int64_t ibase, int R, int ra, int rb,
                                                int b0, int nch, float *C, int64_t c_off, int64_t ldc,
                                                int i0, int i1, int j0, int j1, bool lower,
                                                unsigned char *smem, gb_tc_ctx &tc)
{
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const uint32_t idesc = (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(128 >> 3) << 17)
                           | ((uint32_t)(128 >> 4) << 24);
    const int NS = GB_IMG_NS;
    bool ok = true;
    auto issue = [&](int c) {
        const int st = c % NS, b = b0 + (c >> 1), h = c & 1;
        const float *pa = gb_img_ptr(Img, ibase, R, b, ra) + h * 4096;
        const float *pb = gb_img_ptr(Img, ibase, R, b, rb) + h * 4096;
        const uint32_t fb = tc.mbar + 8u * (uint32_t)st;
        const uint32_t dst = gb_su32(smem + st * 32768);
        asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;"
                     :: "r"(fb), "r"(32768) : "memory");
        asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
                     :: "r"(dst), "l"(pa), "r"(16384), "r"(fb) : "memory");
        asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
                     :: "r"(dst + 16384u), "l"(pb), "r"(16384), "r"(fb) : "memory");
    };
    // the images were written by other blocks through the generic proxy
    // (ordered by the executor's release/acquire); make them visible to the
    // async proxy before the copies
    int issued = 0, nmma = 0;     // thread 0: chunks loaded, chunks multiplied
    if (tid == 0) {
        asm volatile("fence.proxy.async.global;" ::: "memory");
        for (; issued < nch && issued < NS; issued++) issue(issued);
    }
    // C's values, in flight with the operands
    float cval[16];
#pragma unroll
    for (int q = 0; q < 16; q++) {
        const int idx = tid + 256 * q, i = idx & 63, j = idx >> 6;
        const bool in = i >= i0 && i < i1 && j >= j0 && j < j1 && !(lower && i < j);
        cval[q] = in ? C[c_off + i + (int64_t)j * ldc] : 0.0f;
    }
    float sum[32];
#pragma unroll
    for (int q = 0; q < 32; q++) sum[q] = 0.0f;
    // drain accumulator sel: this thread's TMEM lane 32 (warp % 4) + lane,
    // output columns 32 (warp / 4) .. + 31 (products with B_hi at those
    // columns, with B_lo at 64 + those columns)
    auto drain = [&](int sel) {
        const uint32_t base = tc.taddr + ((uint32_t)(32 * (warp & 3)) << 16)
                              + (uint32_t)(sel * 128 + 32 * (warp >> 2));
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
#pragma unroll
        for (int hf = 0; hf < 2; hf++) {
            uint32_t x[16], y[16];
            gb_tmem_ld16(x, base + 16u * hf);
            gb_tmem_ld16(y, base + 64u + 16u * hf);
            asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
            for (int q = 0; q < 16; q++) sum[16 * hf + q] += __uint_as_float(x[q]) + __uint_as_float(y[q]);
        }
        asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    };
    for (int c = 0; c < nch; c++) {
        const int g = c / GB_IMG_GROUP, gs = g * GB_IMG_GROUP;
        if (tid == 0 && ok) {
            const int st = c % NS;
            if (!gb_tc_wait(tc, st)) ok = false;
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            const uint32_t a0 = gb_su32(smem + st * 32768), bb0 = a0 + 16384u;
            const uint32_t acc = tc.taddr + (uint32_t)((g & 1) * 128);
#pragma unroll
            for (int j = 0; j < 4; j++)
                gb_tc_mma(acc, gb_tc_desc(a0 + j * 256, 128, 1024), gb_tc_desc(bb0 + j * 256, 128, 1024),
                          idesc, (c > gs || j > 0) ? 1u : 0u);
            asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];"
                         :: "r"(tc.mbar + 8u * (uint32_t)(NS + st)) : "memory");
            nmma = c + 1;
            // the group's last chunk, with more groups to come: signal the
            // accumulator's completion for its drain
            if (c == gs + GB_IMG_GROUP - 1 && c + 1 < nch)
                asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];"
                             :: "r"(tc.mbar + 8u * (uint32_t)(2 * NS)) : "memory");
            // refill the stage of chunk c - 1 (its MMAs are done or nearly)
            if (c >= 1 && issued < nch) {
                if (!gb_tc_wait(tc, NS + (c - 1) % NS)) ok = false;
                issue(issued++);
            }
        }
        // a new group's first MMAs are issued: drain the previous group's
        // accumulator meanwhile
        if (c == gs && c > 0) {
            if (!gb_tc_wait(tc, 2 * NS)) ok = false;
            if (ok) drain((g - 1) & 1);
            ok = __syncthreads_and(ok);
        }
    }
    // the MMAs whose stages were not refilled: their completion also
    // covers every earlier MMA
    if (tid == 0 && ok) {
        const int first = issued - NS > 0 ? issued - NS : 0;
        for (int c = first; c < issued; c++)
            if (!gb_tc_wait(tc, NS + c % NS)) ok = false;
    }
    ok = __syncthreads_and(ok);
    if (!ok) {
        // a wait gave up: before the block moves on (and releases its
        // TMEM), wait once more, bounded, for the copies no MMA consumed
        // and for every MMA issued (one more commit covers them all)
        if (tid == 0) {
            for (int c = nmma; c < issued; c++) gb_mbar_wait(tc.mbar + 8u * (uint32_t)(c % NS), 0u),
                                                 gb_mbar_wait(tc.mbar + 8u * (uint32_t)(c % NS), 1u);
            asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];"
                         :: "r"(tc.mbar + 8u * (uint32_t)(2 * NS)) : "memory");
            gb_mbar_wait(tc.mbar + 8u * (uint32_t)(2 * NS), 0u);
            gb_mbar_wait(tc.mbar + 8u * (uint32_t)(2 * NS), 1u);
        }
        __syncthreads();
        tc.ok = 0;
        return false;
    }
    if (nch > 0) drain(((nch - 1) / GB_IMG_GROUP) & 1);
    // hi rows (TMEM lanes 0-63) and lo rows (64-127) of each output row
    float *T = (float *)smem;
    __syncthreads();
    {
        const int row = 32 * (warp & 3) + lane, col = 32 * (warp >> 2);
#pragma unroll
        for (int q = 0; q < 32; q++) T[row * 65 + col + q] = sum[q];
    }
    __syncthreads();
#pragma unroll
    for (int q = 0; q < 16; q++) {
        const int idx = tid + 256 * q, i = idx & 63, j = idx >> 6;
        if (i >= i0 && i < i1 && j >= j0 && j < j1 && !(lower && i < j))
            C[c_off + i + (int64_t)j * ldc] = cval[q] - (T[i * 65 + j] + T[(64 + i) * 65 + j]);
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
    d.imgbase = p->imgbase;
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
