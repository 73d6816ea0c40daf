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


static inline gb_dev_pattern gb_to_dev(const gb_pattern_ptrs *p)
{
    gb_dev_pattern d;
    d.Super = p->Super; d.Pi = p->Pi; d.Px = p->Px; d.cboff = p->cboff;
    d.cbvoff = p->cbvoff; d.Ls = p->Ls; d.relmap = p->relmap;
    d.child_ptr = p->child_ptr; d.child_list = p->child_list;
    d.fail = p->fail; d.anyfail = p->anyfail;
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
