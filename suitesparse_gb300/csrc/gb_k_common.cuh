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

static inline gb_dev_pattern gb_to_dev(const gb_pattern_ptrs *p)
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
