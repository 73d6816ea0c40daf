// gb_k_noalloc.cu -- backward error of device-resident solutions without
// any allocation: the residual, column maxima and |A|_inf of the refined
// solve's convergence test, fused into one kernel whose reduction scratch is
// a file-scope device array (gb300_backward_error_noalloc in
// include/cholmod_gb300.h).

#include <cuda_runtime.h>
#include <stdint.h>
#include "cholmod_gb300.h"

// Reduction scratch: per column the bit patterns of max|b - A x|, max|x|,
// max|b| (nonnegative doubles, for which IEEE order equals unsigned
// order; a NaN is stored as the positive quiet NaN, above +inf), the bit
// pattern of |A|_inf, and the count of finished blocks.
// All zero when a call starts: zero at module load, and the last block of
// every call zeroes what the call used.
struct gb_berr_scratch {
    unsigned long long colmax[3 * GB300_BERR_MAX_RHS];
    unsigned long long anorm;
    unsigned int done;
    unsigned int pad;
};

static __device__ __align__(256) gb_berr_scratch gb_berr_scr;

// Maximum that keeps NaN (fmax(a, NaN) returns a); operands are >= 0 or NaN.
__device__ __forceinline__ double maxnan(double a, double b) { return (b > a || b != b) ? b : a; }

// Bit pattern for atomicMax: a NaN becomes the positive quiet NaN, which
// orders above +inf as an unsigned integer and so survives the reduction.
__device__ __forceinline__ unsigned long long maxbits(double v)
{
    return v != v ? 0x7FF8000000000000ull : (unsigned long long)__double_as_longlong(v);
}

// Block (bx, r): rows bx, bx + gridDim.x, ... of column r.  A holds both
// triangles in compressed-column form; by symmetry column i is row i, so
// r_i = b_i - sum_p Ax[p] x[Ai[p]] in stored order and the row sums of |A|
// are column sums.
__global__ void __launch_bounds__(256)
k_berr_noalloc(int64_t n, const int64_t *__restrict__ Ap, const int64_t *__restrict__ Ai,
               const double *__restrict__ Ax, int nrhs, const double *__restrict__ X,
               int64_t ldx, const double *__restrict__ B, int64_t ldb, double *berr,
               gb_berr_scratch *S)
{
    __shared__ double sm[4][256];
    __shared__ int last;
    const int r = blockIdx.y;
    const double *x = X + r * ldx, *b = B + r * ldb;
    double mr = 0, mx = 0, mb = 0, an = 0;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x) {
        double acc = 0, rs = 0;
        for (int64_t p = Ap[i]; p < Ap[i + 1]; p++) {
            acc += Ax[p] * x[Ai[p]];
            rs += fabs(Ax[p]);
        }
        mr = maxnan(mr, fabs(b[i] - acc));
        mx = maxnan(mx, fabs(x[i]));
        mb = maxnan(mb, fabs(b[i]));
        an = maxnan(an, rs);
    }
    sm[0][threadIdx.x] = mr;
    sm[1][threadIdx.x] = mx;
    sm[2][threadIdx.x] = mb;
    sm[3][threadIdx.x] = an;
    __syncthreads();
    for (int o = blockDim.x / 2; o > 0; o >>= 1) {
        if (threadIdx.x < o)
            for (int q = 0; q < 4; q++) sm[q][threadIdx.x] = maxnan(sm[q][threadIdx.x], sm[q][threadIdx.x + o]);
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        for (int q = 0; q < 3; q++)
            atomicMax(&S->colmax[3 * r + q], maxbits(sm[q][0]));
        if (r == 0) atomicMax(&S->anorm, maxbits(sm[3][0]));
        __threadfence();
        const unsigned int total = gridDim.x * gridDim.y;
        last = atomicAdd(&S->done, 1u) == total - 1;
    }
    __syncthreads();
    if (!last) return;
    // the last block: every other block's maxima are in place
    __threadfence();
    volatile unsigned long long *cm = S->colmax;
    const double anorm = __longlong_as_double((long long)*(volatile unsigned long long *)&S->anorm);
    for (int c = threadIdx.x; c < nrhs; c += blockDim.x) {
        const double rmax = __longlong_as_double((long long)cm[3 * c]);
        const double xmax = __longlong_as_double((long long)cm[3 * c + 1]);
        const double bmax = __longlong_as_double((long long)cm[3 * c + 2]);
        const double den = anorm * xmax + bmax;
        // a NaN or infinite term (in x, b or A) gives NaN: never converged
        const bool finite = isfinite(rmax) && isfinite(xmax) && isfinite(bmax) && isfinite(anorm)
                            && isfinite(den);
        berr[c] = !finite ? __longlong_as_double(0x7FF8000000000000ll) : den > 0 ? rmax / den : 0.0;
    }
    __syncthreads();
    for (int q = threadIdx.x; q < 3 * nrhs; q += blockDim.x) S->colmax[q] = 0ull;
    if (threadIdx.x == 0) {
        S->anorm = 0ull;
        S->done = 0u;
    }
}

#define GB_NOALLOC_MAX_DEVICES 64

static gb_berr_scratch *gb_berr_ptr[GB_NOALLOC_MAX_DEVICES];

extern "C" {

int gb300_backward_error_noalloc(int64_t n, const int64_t *Ap, const int64_t *Ai, const double *Ax,
                                 int nrhs, const double *X, int64_t ldx, const double *B,
                                 int64_t ldb, double *berr, void *stream)
{
    if (n < 0 || nrhs < 0) return GB300_NOALLOC_INVALID;
    if (nrhs > GB300_BERR_MAX_RHS) return GB300_NOALLOC_TOO_LARGE;
    if (nrhs == 0) return 0;
    if (!Ap || !X || !B || !berr || ldx < n || ldb < n) return GB300_NOALLOC_INVALID;
    if (n > 0 && (!Ai || !Ax)) return GB300_NOALLOC_INVALID;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= GB_NOALLOC_MAX_DEVICES)
        return GB300_NOALLOC_CUDA;
    gb_berr_scratch *S = __atomic_load_n(&gb_berr_ptr[dev], __ATOMIC_ACQUIRE);
    if (!S) {
        // once per device, with that device current
        void *p = NULL;
        if (cudaGetSymbolAddress(&p, gb_berr_scr) != cudaSuccess || !p) return GB300_NOALLOC_CUDA;
        S = (gb_berr_scratch *)p;
        __atomic_store_n(&gb_berr_ptr[dev], S, __ATOMIC_RELEASE);
    }
    int64_t gx = (n + 255) / 256;
    if (gx > 152) gx = 152;
    if (gx < 1) gx = 1;
    dim3 grid((unsigned)gx, (unsigned)nrhs);
    k_berr_noalloc<<<grid, 256, 0, (cudaStream_t)stream>>>(n, Ap, Ai, Ax, nrhs, X, ldx, B, ldb,
                                                           berr, S);
    return cudaGetLastError() == cudaSuccess ? 0 : GB300_NOALLOC_CUDA;
}

}  // extern "C"
