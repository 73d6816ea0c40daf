// gb_k_sweep1.cu -- single-launch supernodal sweeps.
//
// Each sweep (forward L y = b, backward L' x = y) is one kernel launch whose
// thread blocks take tasks in a fixed topological order through an atomic
// ticket and wait, with bounded spins, for the tasks they depend on.  Tasks
// are ordered by etree level (ascending for the forward sweep, descending
// for the backward sweep), so that independent branches interleave:
//
//   forward  per supernode s: its 64-row diagonal blocks in order, then its
//            off-diagonal row blocks.  A diagonal block waits for s's
//            children (their update vectors) and, one at a time, for the
//            earlier diagonal blocks of s:  x_i = Linv_ii (b_i - children -
//            sum_{j<i} L_ij x_j).  An off-diagonal row block takes the
//            diagonal blocks of s one at a time as they become final and
//            writes its rows of the update vector u_s = (children's
//            contributions) + L21 x1, which s's parent gathers
//            (owner-computes, children in a fixed order).
//   backward per supernode s, diagonal blocks last to first: wait for the
//            parent supernode (whose completion implies all ancestors'),
//            x_i = Linv_ii' (y_i - L21(:,i)' x(rows of s) - sum_{j>i} L_ji' x_j).
//
// Latency: the 64x64 tile of L needed after a wait is loaded into registers
// before the wait and parked in shared memory after it, so a dependency step
// costs one flag round trip plus shared-memory arithmetic.  Products reduce
// over 4 lanes with shuffles (no padded right-hand sides: the FP64 pipe of
// this GPU issues under 2 multiply-adds per clock per SM).
//
// A ticket names a group of consecutive tasks (runs of leaf-level tasks, 8
// per ticket; other tasks alone), run in order by the block that took it.  A
// task only waits for tasks listed before it, which belong to its own group
// (already done) or to groups taken by blocks already running, so the sweep
// cannot deadlock.  Every wait gives up
// after GB_SPIN_LIMIT polls, sets the error word and returns; every other
// waiter then returns at once.  Linv holds the inverse of every diagonal
// block (k_diag_inverse, after the factorization).
//
// Correspondence with the reference: CHOLMOD/Supernodal/
// t_cholmod_super_solve_worker.c (dtrsv/dtrsm + dgemv/dgemm per supernode,
// forward :63-301, backward :358-578).

#include "gb_k_common.cuh"

#define SR 64          // rows of a diagonal block / row block
#define TLD 65         // padded leading dimension of a shared tile
#define RCH 16         // right-hand-side columns per pass
#define GB_SPIN_LIMIT (1 << 22)

__device__ __forceinline__ int ld_acquire(const int32_t *p)
{
    int v;
    asm volatile("ld.acquire.gpu.global.b32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

__device__ __forceinline__ void st_release(int32_t *p, int v)
{
    asm volatile("st.release.gpu.global.b32 [%0], %1;" :: "l"(p), "r"(v) : "memory");
}

__device__ __forceinline__ void red_release_add(int32_t *p, int v)
{
    asm volatile("red.release.gpu.global.add.s32 [%0], %1;" :: "l"(p), "r"(v) : "memory");
}

__device__ __forceinline__ unsigned long long gtimer()
{
    unsigned long long t;
    asm volatile("mov.u64 %0, %globaltimer;" : "=l"(t));
    return t;
}

// thread 0 only: wait until *flag >= target; false on timeout / abort
__device__ bool wait_ge_n(const int32_t *flag, int target, int32_t *err, long long limit)
{
    if (ld_acquire(flag) >= target) return true;
    for (long long it = 0; it < limit; it++) {
        __nanosleep(32);
        if (ld_acquire(flag) >= target) return true;
        if ((it & 15) == 15 && ld_acquire(err)) return false;   // another waiter gave up
    }
    atomicExch(err, 1);
    return false;
}

__device__ bool wait_ge(const int32_t *flag, int target, int32_t *err)
{
    return wait_ge_n(flag, target, err, GB_SPIN_LIMIT);
}

// the bounded wait on a flag that nothing sets: it gives up after limit
// polls, sets the error word and returns (out[0] = whether the wait
// succeeded, out[1] = the error word)
__global__ void k_wait_probe(const int32_t *flag, int32_t *err, long long limit, int32_t *out)
{
    if (threadIdx.x == 0 && blockIdx.x == 0) {
        const bool ok = wait_ge_n(flag, 1, err, limit);
        out[0] = ok ? 1 : 0;
        out[1] = ld_acquire(err);
    }
}

// ---- 64x64 tiles: registers -> shared memory ------------------------------

// element (rr, cc) of the nr x nc region at base (leading dimension ld);
// thread t holds elements t + 256 q, q = 0..15 (coalesced along rr)
template <typename T>
__device__ __forceinline__ void tile_fetch(T (&reg)[16], const T *base, int64_t ld, int nr, int nc)
{
#pragma unroll
    for (int q = 0; q < 16; q++) {
        const int idx = threadIdx.x + q * 256;
        const int rr = idx & 63, cc = idx >> 6;
        reg[q] = (rr < nr && cc < nc) ? base[rr + (int64_t)cc * ld] : (T)0;
    }
}

// tile[cc * TLD + rr] = element (rr, cc)
template <typename T>
__device__ __forceinline__ void tile_park(T *tile, const T (&reg)[16])
{
#pragma unroll
    for (int q = 0; q < 16; q++) {
        const int idx = threadIdx.x + q * 256;
        tile[(idx >> 6) * TLD + (idx & 63)] = reg[q];
    }
}

// ys[r][k] += sign * sum_c op(tile)(r, c) xs[c][k],  op = identity (trans=0:
// element (r, c) = tile[c*TLD + r]) or transpose (trans=1: tile[r*TLD + c]).
// Thread layout: row r = 8*warp + lane/4, lanes lane%4 split c; 2 shuffles.
template <typename T, int NK>
__device__ __forceinline__ void tile_gemv_k(const T *tile, int trans, int nr, int nc,
                                            const T *xs, T *ys, int nk, T sign)
{
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int r = warp * 8 + (lane >> 2), q = lane & 3;
    for (int k0 = 0; k0 < nk; k0 += NK) {
        T acc[NK];
#pragma unroll
        for (int kk = 0; kk < NK; kk++) acc[kk] = (T)0;
        if (r < nr) {
            for (int c = q; c < nc; c += 4) {
                const T l = trans ? tile[r * TLD + c] : tile[c * TLD + r];
#pragma unroll
                for (int kk = 0; kk < NK; kk++) acc[kk] += l * xs[c * RCH + k0 + kk];
            }
        }
#pragma unroll
        for (int kk = 0; kk < NK; kk++) {
            T v = acc[kk];
            v += __shfl_xor_sync(0xffffffffu, v, 1);
            v += __shfl_xor_sync(0xffffffffu, v, 2);
            if (q == 0 && r < nr && k0 + kk < nk) ys[r * RCH + k0 + kk] += sign * v;
        }
    }
}

template <typename T>
__device__ void tile_gemv(const T *tile, int trans, int nr, int nc, const T *xs, T *ys,
                          int nk, T sign)
{
    if (nk == 1) tile_gemv_k<T, 1>(tile, trans, nr, nc, xs, ys, nk, sign);
    else if (nk <= 2) tile_gemv_k<T, 2>(tile, trans, nr, nc, xs, ys, nk, sign);
    else if (nk <= 4) tile_gemv_k<T, 4>(tile, trans, nr, nc, xs, ys, nk, sign);
    else tile_gemv_k<T, 8>(tile, trans, nr, nc, xs, ys, nk, sign);
    __syncthreads();
}

struct gb_sweep_state {
    const gb_stask *tasks;
    int ntasks;
    const int32_t *gptr;       // tickets name groups: tasks [gptr[g], gptr[g+1])
    int ngroups;
    const int32_t *blkoff;     // first global diagonal-block id of s
    const int64_t *linvoff;    // offset of each diagonal block's inverse
    const int32_t *ntask_s;    // tasks of supernode s in this sweep
    const int32_t *parent;     // supernodal etree parent (-1 root)
    int32_t *xready, *done, *ticket, *err;
    unsigned long long *trace; // optional: per task [start, dependencies met, end] (ns)
    const int32_t *cptr;       // forward: child row ranges of each task (gb_plan.c)
    const int32_t *crange;
    const int32_t *bchunk_ptr; // backward: per supernode and 64-row chunk of its rows
    const int32_t *bchunk;     // below the diagonal block, the block of the chunk's first row
    const unsigned char *act;  // optional: act[sseg[s]] == 0 skips supernode s's tasks
    const int32_t *sseg;       // (independent systems already converged: no task of
                               // another segment waits for them)
};

// dynamic shared memory: tile A, tile B (64 x TLD each), xs, ys (64 x RCH)
template <typename T>
__host__ __device__ constexpr size_t sweep_smem() { return sizeof(T) * (2 * SR * TLD + 2 * SR * RCH); }

template <typename T>
__global__ void __launch_bounds__(256, 3)
k_fwd_sweep(gb_dev_pattern P, gb_sweep_state S, const T *Lx, const T *Linv, int nrhs,
            T *Y, int64_t ldy, T *U)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    T *tA = (T *)smem_raw, *tB = tA + SR * TLD, *xs = tB + SR * TLD, *ys = xs + SR * RCH;
    __shared__ int sg, abort_;
    // children of the task's supernode, 32 at a time: update-vector rows
    // [a, b) that fall in the task's rows, their count mc, the offsets of
    // their relative map and update vector
    __shared__ int c_a[32], c_b[32], c_mc[32];
    __shared__ int64_t c_rm[32], c_u[32];
    T reg[16];
    for (;;) {
        if (threadIdx.x == 0) { sg = atomicAdd(S.ticket, 1); abort_ = 0; }
        __syncthreads();
        const int g = sg;
        if (g >= S.ngroups) return;
        const int tend = S.gptr[g + 1];
        for (int t = S.gptr[g]; t < tend; t++) {
        const gb_stask tk = S.tasks[t];
        if (S.act && !S.act[S.sseg[tk.s]]) continue;
        if (S.trace && threadIdx.x == 0) S.trace[3 * (size_t)t] = gtimer();
        const int s = tk.s;
        const int64_t k1 = P.Super[s];
        const int nscol = (int)(P.Super[s + 1] - k1);
        const int64_t psi = P.Pi[s];
        const int nsrow = (int)(P.Pi[s + 1] - psi);
        const int m = nsrow - nscol;
        const T *panel = Lx + P.Px[s];
        T *us = U + P.cbvoff[s] * nrhs;
        const int r0 = tk.r0, nr = tk.nr;
        const int nblk = (nscol + SR - 1) / SR;
        // the diagonal block's inverse depends on nothing: parked in tB
        // before any wait, off the dependency chain
        if (tk.kind == 0) {
            tile_fetch(reg, Linv + S.linvoff[S.blkoff[s] + tk.idx], nr, nr, nr);
            tile_park(tB, reg);
        }
        // first L tile this task needs, fetched before any wait
        if (tk.kind == 0 && tk.idx > 0) tile_fetch(reg, panel + r0, nsrow, nr, SR);
        else if (tk.kind == 1) tile_fetch(reg, panel + r0, nsrow, nr, min(SR, nscol));
        const int cb0 = P.child_ptr[s], nch = P.child_ptr[s + 1] - cb0;
        const int32_t *cr = S.crange + 2 * (int64_t)S.cptr[t];
        // the children's update vectors: warp 0 waits for up to 32 children
        // at once, one lane each
        if (threadIdx.x < 32) {
            bool ok = true;
            for (int j = (int)threadIdx.x; j < nch && ok; j += 32) {
                const int c = P.child_list[cb0 + j];
                ok = wait_ge(S.done + c, S.ntask_s[c], S.err);
            }
            if (__any_sync(0xffffffffu, !ok) && threadIdx.x == 0) abort_ = 1;
        }
        __syncthreads();
        if (abort_) return;
        if (S.trace && threadIdx.x == 0) S.trace[3 * (size_t)t + 1] = gtimer();
        for (int k0 = 0; k0 < nrhs; k0 += RCH) {
            const int nk = min(RCH, nrhs - k0);
            if (k0 > 0) {
                if (tk.kind == 0 && tk.idx > 0) tile_fetch(reg, panel + r0, nsrow, nr, SR);
                else if (tk.kind == 1) tile_fetch(reg, panel + r0, nsrow, nr, min(SR, nscol));
            }
            // start value: b (diagonal rows) or 0 (update-vector rows)
            for (int idx = threadIdx.x; idx < SR * RCH; idx += blockDim.x) {
                const int r = idx / RCH, k = idx % RCH;
                T v = (T)0;
                if (tk.kind == 0 && r < nr && k < nk) v = Y[k1 + r0 + r + (int64_t)(k0 + k) * ldy];
                ys[idx] = v;
            }
            __syncthreads();
            // gather the children's update vectors at rows [r0, r0+nr)
            const T gsign = tk.kind == 0 ? (T)-1 : (T)1;
            for (int j0 = 0; j0 < nch; j0 += 32) {
                // offsets of the next 32 children, fetched by warp 0's
                // lanes together
                if (threadIdx.x < 32 && j0 + (int)threadIdx.x < nch) {
                    const int j = j0 + (int)threadIdx.x;
                    const int c = P.child_list[cb0 + j];
                    const int ncc = (int)(P.Super[c + 1] - P.Super[c]);
                    const int64_t pic = P.Pi[c];
                    c_mc[threadIdx.x] = (int)(P.Pi[c + 1] - pic) - ncc;
                    c_rm[threadIdx.x] = pic + ncc;
                    c_u[threadIdx.x] = P.cbvoff[c] * nrhs;
                    c_a[threadIdx.x] = cr[2 * j];
                    c_b[threadIdx.x] = cr[2 * j + 1];
                }
                __syncthreads();
                const int nj = min(32, nch - j0);
                for (int jj = 0; jj < nj; jj++) {
                    const int a = c_a[jj], b = c_b[jj], mc = c_mc[jj];
                    const int32_t *rm = P.relmap + c_rm[jj];
                    const T *uc = U + c_u[jj];
                    for (int idx = threadIdx.x; idx < (b - a) * nk; idx += blockDim.x) {
                        const int i = a + idx % (b - a), k = idx / (b - a);
                        ys[(rm[i] - r0) * RCH + k] += gsign * uc[i + (int64_t)(k0 + k) * mc];
                    }
                    __syncthreads();
                }
            }
            if (tk.kind == 0) {
                const int i = tk.idx;
                for (int j = 0; j < i; j++) {
                    if (k0 == 0 && threadIdx.x == 0) {
                        if (!wait_ge(S.xready + S.blkoff[s] + j, 1, S.err)) abort_ = 1;
                    }
                    tile_park(tA, reg);
                    __syncthreads();
                    if (abort_) return;
                    for (int idx = threadIdx.x; idx < SR * RCH; idx += blockDim.x) {
                        const int c = idx / RCH, k = idx % RCH;
                        const int nc = min(SR, nscol - j * SR);
                        xs[idx] = (c < nc && k < nk) ? Y[k1 + j * SR + c + (int64_t)(k0 + k) * ldy] : (T)0;
                    }
                    __syncthreads();
                    if (j + 1 < i) tile_fetch(reg, panel + r0 + (int64_t)((j + 1) * SR) * nsrow, nsrow, nr, SR);
                    tile_gemv<T>(tA, 0, nr, min(SR, nscol - j * SR), xs, ys, nk, (T)-1);
                }
                // x_i = Linv_ii ys (Linv_ii parked in tB at the start)
                for (int idx = threadIdx.x; idx < SR * RCH; idx += blockDim.x) {
                    xs[idx] = ys[idx];
                    ys[idx] = (T)0;
                }
                __syncthreads();
                tile_gemv<T>(tB, 0, nr, nr, xs, ys, nk, (T)1);
                for (int idx = threadIdx.x; idx < nr * nk; idx += blockDim.x) {
                    const int r = idx % nr, k = idx / nr;
                    Y[k1 + r0 + r + (int64_t)(k0 + k) * ldy] = ys[r * RCH + k];
                }
                __syncthreads();
            } else {
                // update-vector rows: ys += L(rows, 0:nscol) x1, taking each
                // 64-column block of x1 as soon as it is final
                for (int j = 0; j < nblk; j++) {
                    const int nc = min(SR, nscol - j * SR);
                    if (k0 == 0 && threadIdx.x == 0) {
                        if (!wait_ge(S.xready + S.blkoff[s] + j, 1, S.err)) abort_ = 1;
                    }
                    tile_park(tA, reg);
                    __syncthreads();
                    if (abort_) return;
                    for (int idx = threadIdx.x; idx < SR * RCH; idx += blockDim.x) {
                        const int c = idx / RCH, k = idx % RCH;
                        xs[idx] = (c < nc && k < nk) ? Y[k1 + j * SR + c + (int64_t)(k0 + k) * ldy] : (T)0;
                    }
                    __syncthreads();
                    if (j + 1 < nblk)
                        tile_fetch(reg, panel + r0 + (int64_t)((j + 1) * SR) * nsrow, nsrow, nr,
                                   min(SR, nscol - (j + 1) * SR));
                    tile_gemv<T>(tA, 0, nr, nc, xs, ys, nk, (T)1);
                }
                for (int idx = threadIdx.x; idx < nr * nk; idx += blockDim.x) {
                    const int r = idx % nr, k = idx / nr;
                    us[(r0 - nscol) + r + (int64_t)(k0 + k) * m] = ys[r * RCH + k];
                }
                __syncthreads();
            }
        }
        if (threadIdx.x == 0) {
            // release stores after the block barrier: the block's writes of
            // x and u are visible to whoever acquires either word
            if (tk.kind == 0) st_release(S.xready + S.blkoff[s] + tk.idx, 1);
            red_release_add(S.done + s, 1);
            if (S.trace) S.trace[3 * (size_t)t + 2] = gtimer();
        }
        __syncthreads();
        }
    }
}

template <typename T>
__global__ void __launch_bounds__(256, 2)
k_bwd_sweep(gb_dev_pattern P, gb_sweep_state S, const T *Lx, const T *Linv, int nrhs,
            T *Y, int64_t ldy)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    T *tA = (T *)smem_raw, *tB = tA + SR * TLD, *xs = tB + SR * TLD, *ys = xs + SR * RCH;
    __shared__ int sg, abort_;
    T reg[16];
    for (;;) {
        if (threadIdx.x == 0) { sg = atomicAdd(S.ticket, 1); abort_ = 0; }
        __syncthreads();
        const int g = sg;
        if (g >= S.ngroups) return;
        const int tend = S.gptr[g + 1];
        for (int t = S.gptr[g]; t < tend; t++) {
        const gb_stask tk = S.tasks[t];
        if (S.act && !S.act[S.sseg[tk.s]]) continue;
        if (S.trace && threadIdx.x == 0) S.trace[3 * (size_t)t] = gtimer();
        const int s = tk.s;
        const int64_t k1 = P.Super[s];
        const int nscol = (int)(P.Super[s + 1] - k1);
        const int64_t psi = P.Pi[s];
        const int nsrow = (int)(P.Pi[s + 1] - psi);
        const int m = nsrow - nscol;
        const T *panel = Lx + P.Px[s];
        const int32_t *rows = P.Ls + psi + nscol;
        const int i = tk.idx, r0 = tk.r0, nr = tk.nr;
        const int nblk = (nscol + SR - 1) / SR;
        const int nch = (m + SR - 1) / SR;
        const int32_t *cblk = S.bchunk + S.bchunk_ptr[s];
        // the diagonal block's inverse, parked in tB before any wait
        tile_fetch(reg, Linv + S.linvoff[S.blkoff[s] + i], nr, nr, nr);
        tile_park(tB, reg);
        // the last L21 tile: rows of the farthest ancestors, final first
        if (m > 0)
            tile_fetch(reg, panel + nscol + (int64_t)(nch - 1) * SR + (int64_t)r0 * nsrow, nsrow,
                       m - (nch - 1) * SR, nr);
        __syncthreads();
        if (S.trace && threadIdx.x == 0) S.trace[3 * (size_t)t + 1] = gtimer();
        for (int k0 = 0; k0 < nrhs; k0 += RCH) {
            const int nk = min(RCH, nrhs - k0);
            if (k0 > 0 && m > 0)
                tile_fetch(reg, panel + nscol + (int64_t)(nch - 1) * SR + (int64_t)r0 * nsrow, nsrow,
                           m - (nch - 1) * SR, nr);
            for (int idx = threadIdx.x; idx < SR * RCH; idx += blockDim.x) {
                const int r = idx / RCH, k = idx % RCH;
                ys[idx] = (r < nr && k < nk) ? Y[k1 + r0 + r + (int64_t)(k0 + k) * ldy] : (T)0;
            }
            // ys -= L21(:, blk i)' x(rows of s), 64 rows at a time from the
            // last.  A chunk waits only for the diagonal block holding its
            // first row: the chunk's other rows lie in later blocks of that
            // supernode (final before it) or in its ancestors' blocks (rows
            // of its own below its diagonal, final before any of its
            // blocks), so the chunks of far ancestors are used while the
            // nearer ones are still being solved.  The next L tile is loaded
            // while a chunk is used; the chunk's x (xv: this thread's 4 of
            // the 64 x 16 entries, a gather through the row indices) after
            // its wait.
            T xv[4];
            for (int qc = nch - 1; qc >= 0; qc--) {
                const int q0 = qc * SR, nq = min(SR, m - q0);
                if (k0 == 0 && threadIdx.x == 0 && !wait_ge(S.xready + cblk[qc], 1, S.err)) abort_ = 1;
                __syncthreads();
                if (abort_) return;
#pragma unroll
                for (int u = 0; u < 4; u++) {
                    const int idx = threadIdx.x + 256 * u, c = idx / RCH, k = idx % RCH;
                    xv[u] = (q0 + c < m && k < nk) ? Y[rows[q0 + c] + (int64_t)(k0 + k) * ldy] : (T)0;
                }
                tile_park(tA, reg);
#pragma unroll
                for (int u = 0; u < 4; u++) xs[threadIdx.x + 256 * u] = xv[u];
                __syncthreads();
                if (qc > 0) tile_fetch(reg, panel + nscol + q0 - SR + (int64_t)r0 * nsrow, nsrow, SR, nr);
                tile_gemv<T>(tA, 1, nr, nq, xs, ys, nk, (T)-1);
            }
            // later diagonal blocks of s: ys -= L(blk j, blk i)' x_j
            if (nblk - 1 > i)
                tile_fetch(reg, panel + (nblk - 1) * SR + (int64_t)r0 * nsrow, nsrow,
                           min(SR, nscol - (nblk - 1) * SR), nr);
            __syncthreads();
            for (int j = nblk - 1; j > i; j--) {
                const int nc = min(SR, nscol - j * SR);
                if (k0 == 0 && threadIdx.x == 0) {
                    if (!wait_ge(S.xready + S.blkoff[s] + j, 1, S.err)) abort_ = 1;
                }
                tile_park(tA, reg);
                __syncthreads();
                if (abort_) return;
                for (int idx = threadIdx.x; idx < SR * RCH; idx += blockDim.x) {
                    const int c = idx / RCH, k = idx % RCH;
                    xs[idx] = (c < nc && k < nk) ? Y[k1 + j * SR + c + (int64_t)(k0 + k) * ldy] : (T)0;
                }
                __syncthreads();
                if (j - 1 > i)
                    tile_fetch(reg, panel + (j - 1) * SR + (int64_t)r0 * nsrow, nsrow, SR, nr);
                tile_gemv<T>(tA, 1, nr, nc, xs, ys, nk, (T)-1);
            }
            // x_i = Linv_ii' ys (Linv_ii parked in tB at the start)
            for (int idx = threadIdx.x; idx < SR * RCH; idx += blockDim.x) {
                xs[idx] = ys[idx];
                ys[idx] = (T)0;
            }
            __syncthreads();
            tile_gemv<T>(tB, 1, nr, nr, xs, ys, nk, (T)1);
            for (int idx = threadIdx.x; idx < nr * nk; idx += blockDim.x) {
                const int r = idx % nr, k = idx / nr;
                Y[k1 + r0 + r + (int64_t)(k0 + k) * ldy] = ys[r * RCH + k];
            }
            __syncthreads();
        }
        if (threadIdx.x == 0) {
            st_release(S.xready + S.blkoff[s] + i, 1);
            red_release_add(S.done + s, 1);
            if (S.trace) S.trace[3 * (size_t)t + 2] = gtimer();
        }
        __syncthreads();
        }
    }
}

// ---- leaf subtrees: one warp each ------------------------------------------
// A leaf subtree (supernodes s0..root, contiguous in postorder, every front
// at most GB_LEAF_ROWS rows and one diagonal block) is swept by one warp,
// rows r = lane, lane + 32, ..., the front staged in shared memory, with no
// waits: the forward sweep runs these before its other tasks (they depend on
// nothing), the backward sweep after them (they depend only on their
// ancestors' x, final by then).  Per supernode, forward:
//   y1 = b1 - (children's update-vector rows in the diagonal block),
//   x1 = Linv y1,  u = (children's rows below the diagonal block) + L21 x1;
// backward: y1 = x1 - L21' x(rows below), x1 = Linv' y1.  Children's update
// vectors are gathered in a fixed order (owner-computes); their offsets are
// fetched by the lanes together, one child per lane.  A warp takes its next
// subtree from a ticket.  Right-hand sides in chunks of LF_RC.

#define LF_RC 8                  // right-hand sides per chunk
#define LF_LD 9                  // staging row length (LF_RC + 1)
#define LF_WARPS 4               // warps per block

__device__ __forceinline__ int leaf_next(int32_t *ticket)
{
    int L = 0;
    if ((threadIdx.x & 31) == 0) L = atomicAdd(ticket, 1);
    return __shfl_sync(0xffffffffu, L, 0);
}

template <typename T>
__global__ void __launch_bounds__(32 * LF_WARPS, 8)
k_fwd_leaf(gb_dev_pattern P, const int32_t *__restrict__ leaf, int nleaf,
           const int32_t *__restrict__ blkoff, const int64_t *__restrict__ linvoff,
           const int32_t *__restrict__ ntask_f, int32_t *done, int32_t *ticket, const T *Lx,
           const T *Linv, int nrhs, T *Y, int64_t ldy, T *U, const unsigned char *act,
           const int32_t *sseg, int lrows)
{
    constexpr unsigned FULL = 0xffffffffu;
    extern __shared__ __align__(16) unsigned char lf_smem[];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    T *ys = (T *)lf_smem + (size_t)(2 * warp) * lrows * LF_LD, *xs = ys + (size_t)lrows * LF_LD;
    for (int L = leaf_next(ticket); L < nleaf; L = leaf_next(ticket)) {
        const int s0 = leaf[2 * L], root = leaf[2 * L + 1];
        if (act && !act[sseg[s0]]) continue;   // a converged system's subtree
        for (int s = s0; s <= root; s++) {
            const int64_t k1 = P.Super[s];
            const int nscol = (int)(P.Super[s + 1] - k1);
            const int nsrow = (int)(P.Pi[s + 1] - P.Pi[s]);
            const int m = nsrow - nscol;
            const T *panel = Lx + P.Px[s];
            const T *li = Linv + linvoff[blkoff[s]];
            T *us = U + P.cbvoff[s] * nrhs;
            const int cb = P.child_ptr[s], nch = P.child_ptr[s + 1] - cb;
            for (int k0 = 0; k0 < nrhs; k0 += LF_RC) {
                const int nk = min(LF_RC, nrhs - k0);
                for (int r = lane; r < nsrow; r += 32)
                    for (int k = 0; k < nk; k++)
                        ys[r * LF_LD + k] = r < nscol ? Y[k1 + r + (int64_t)(k0 + k) * ldy] : (T)0;
                __syncwarp();
                for (int j0 = 0; j0 < nch; j0 += 32) {
                    int mc = 0;
                    int64_t roff = 0, uoff = 0;
                    if (j0 + lane < nch) {
                        const int c = P.child_list[cb + j0 + lane];
                        const int ncc = (int)(P.Super[c + 1] - P.Super[c]);
                        const int64_t pic = P.Pi[c];
                        mc = (int)(P.Pi[c + 1] - pic) - ncc;
                        roff = pic + ncc;
                        uoff = P.cbvoff[c] * nrhs;
                    }
                    const int nj = min(32, nch - j0);
                    for (int j = 0; j < nj; j++) {
                        const int mcj = __shfl_sync(FULL, mc, j);
                        const int64_t rj = __shfl_sync(FULL, roff, j);
                        const int64_t uj = __shfl_sync(FULL, uoff, j);
                        for (int i = lane; i < mcj; i += 32) {
                            const int t = P.relmap[rj + i];
                            const T sg = t < nscol ? (T)-1 : (T)1;
                            for (int k = 0; k < nk; k++)
                                ys[t * LF_LD + k] += sg * U[uj + i + (int64_t)(k0 + k) * mcj];
                        }
                        __syncwarp();
                    }
                }
                for (int r = lane; r < nscol; r += 32) {
                    T x[LF_RC];
#pragma unroll
                    for (int k = 0; k < LF_RC; k++) x[k] = (T)0;
                    for (int c0 = 0; c0 <= r; c0 += 8) {
                        T lv[8];                  // eight loads in flight
#pragma unroll
                        for (int u = 0; u < 8; u++) lv[u] = c0 + u <= r ? li[r + (c0 + u) * nscol] : (T)0;
#pragma unroll
                        for (int u = 0; u < 8; u++)
                            if (c0 + u <= r)
#pragma unroll
                                for (int k = 0; k < LF_RC; k++) x[k] += lv[u] * ys[(c0 + u) * LF_LD + k];
                    }
#pragma unroll
                    for (int k = 0; k < LF_RC; k++)
                        if (k < nk) {
                            Y[k1 + r + (int64_t)(k0 + k) * ldy] = x[k];
                            xs[r * LF_LD + k] = x[k];
                        }
                }
                __syncwarp();
                for (int r = nscol + lane; r < nsrow; r += 32) {
                    T u[LF_RC];
#pragma unroll
                    for (int k = 0; k < LF_RC; k++) u[k] = ys[r * LF_LD + k];
                    for (int c0 = 0; c0 < nscol; c0 += 8) {
                        T lv[8];
#pragma unroll
                        for (int q = 0; q < 8; q++) lv[q] = c0 + q < nscol ? panel[r + (int64_t)(c0 + q) * nsrow] : (T)0;
#pragma unroll
                        for (int q = 0; q < 8; q++)
                            if (c0 + q < nscol)
#pragma unroll
                                for (int k = 0; k < LF_RC; k++) u[k] += lv[q] * xs[(c0 + q) * LF_LD + k];
                    }
#pragma unroll
                    for (int k = 0; k < LF_RC; k++)
                        if (k < nk) us[(r - nscol) + (int64_t)(k0 + k) * m] = u[k];
                }
                __syncwarp();
            }
        }
        if (lane == 0) done[root] = ntask_f[root];
    }
}

template <typename T>
__global__ void __launch_bounds__(32 * LF_WARPS, 8)
k_bwd_leaf(gb_dev_pattern P, const int32_t *__restrict__ leaf, int nleaf,
           const int32_t *__restrict__ blkoff, const int64_t *__restrict__ linvoff,
           int32_t *ticket, const T *Lx, const T *Linv, int nrhs, T *Y, int64_t ldy,
           const unsigned char *act, const int32_t *sseg, int lrows)
{
    extern __shared__ __align__(16) unsigned char lf_smem[];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    T *ys = (T *)lf_smem + (size_t)(2 * warp) * lrows * LF_LD, *xs = ys + (size_t)lrows * LF_LD;
    for (int L = leaf_next(ticket); L < nleaf; L = leaf_next(ticket)) {
        const int s0 = leaf[2 * L], root = leaf[2 * L + 1];
        if (act && !act[sseg[s0]]) continue;   // a converged system's subtree
        for (int s = root; s >= s0; s--) {
            const int64_t k1 = P.Super[s];
            const int nscol = (int)(P.Super[s + 1] - k1);
            const int64_t psi = P.Pi[s];
            const int nsrow = (int)(P.Pi[s + 1] - psi);
            const int m = nsrow - nscol;
            const T *panel = Lx + P.Px[s];
            const T *li = Linv + linvoff[blkoff[s]];
            for (int k0 = 0; k0 < nrhs; k0 += LF_RC) {
                const int nk = min(LF_RC, nrhs - k0);
                for (int q = lane; q < m; q += 32) {
                    const int64_t g = P.Ls[psi + nscol + q];
#pragma unroll
                    for (int k = 0; k < LF_RC; k++)
                        xs[q * LF_LD + k] = k < nk ? Y[g + (int64_t)(k0 + k) * ldy] : (T)0;
                }
                __syncwarp();
                for (int r = lane; r < nscol; r += 32) {
                    T y[LF_RC];
#pragma unroll
                    for (int k = 0; k < LF_RC; k++) y[k] = k < nk ? Y[k1 + r + (int64_t)(k0 + k) * ldy] : (T)0;
                    for (int q0 = 0; q0 < m; q0 += 8) {
                        T lv[8];
#pragma unroll
                        for (int u = 0; u < 8; u++) lv[u] = q0 + u < m ? panel[nscol + q0 + u + (int64_t)r * nsrow] : (T)0;
#pragma unroll
                        for (int u = 0; u < 8; u++)
                            if (q0 + u < m)
#pragma unroll
                                for (int k = 0; k < LF_RC; k++) y[k] -= lv[u] * xs[(q0 + u) * LF_LD + k];
                    }
#pragma unroll
                    for (int k = 0; k < LF_RC; k++) ys[r * LF_LD + k] = y[k];
                }
                __syncwarp();
                for (int r = lane; r < nscol; r += 32) {
                    T x[LF_RC];
#pragma unroll
                    for (int k = 0; k < LF_RC; k++) x[k] = (T)0;
                    for (int c0 = r; c0 < nscol; c0 += 8) {
                        T lv[8];
#pragma unroll
                        for (int u = 0; u < 8; u++) lv[u] = c0 + u < nscol ? li[c0 + u + r * nscol] : (T)0;
#pragma unroll
                        for (int u = 0; u < 8; u++)
                            if (c0 + u < nscol)
#pragma unroll
                                for (int k = 0; k < LF_RC; k++) x[k] += lv[u] * ys[(c0 + u) * LF_LD + k];
                    }
#pragma unroll
                    for (int k = 0; k < LF_RC; k++)
                        if (k < nk) Y[k1 + r + (int64_t)(k0 + k) * ldy] = x[k];
                }
                __syncwarp();
            }
        }
    }
}

// inverse of every diagonal block (lower triangular, nb <= 64), one block
// each: thread j computes column j of X = L^-1 by forward substitution,
// writing it straight to the output (its own earlier entries are re-read).
template <typename T>
__global__ void __launch_bounds__(SR)
k_diag_inverse(gb_dev_pattern P, const gb_stask *__restrict__ dtasks, const int32_t *blkoff,
               const int64_t *linvoff, const T *Lx, T *Linv)
{
    __shared__ T A[SR][SR + 1];
    const gb_stask tk = dtasks[blockIdx.x];
    const int s = tk.s;
    const int nsrow = (int)(P.Pi[s + 1] - P.Pi[s]);
    const int nb = tk.nr, r0 = tk.r0;
    const T *blk = Lx + P.Px[s] + r0 + (int64_t)r0 * nsrow;
    for (int idx = threadIdx.x; idx < nb * nb; idx += blockDim.x) {
        const int i = idx % nb, j = idx / nb;
        A[i][j] = (i >= j) ? blk[i + (int64_t)j * nsrow] : (T)0;
    }
    __syncthreads();
    T *out = Linv + linvoff[blkoff[s] + tk.idx];
    const int j = threadIdx.x;
    if (j < nb) {
        T *x = out + (int64_t)j * nb;
        for (int i = 0; i < j; i++) x[i] = (T)0;
        x[j] = (T)1 / A[j][j];
        for (int i = j + 1; i < nb; i++) {
            T acc = (T)0;
            for (int k = j; k < i; k++) acc += A[i][k] * x[k];
            x[i] = -acc / A[i][i];
        }
    }
}

extern "C" {

int gb_launch_sweep1(int forward, const gb_pattern_ptrs *pp, const gb_sweep1_args *a,
                     const void *Lx, const void *Linv, int dtype, int nrhs, void *Y,
                     int64_t ldy, void *U, int grid, cudaStream_t st)
{
    if (a->ntasks <= 0) return 0;
    gb_dev_pattern P = gb_to_dev(pp);
    gb_sweep_state S;
    S.tasks = a->tasks; S.ntasks = a->ntasks; S.blkoff = a->blkoff; S.linvoff = a->linvoff;
    S.ntask_s = a->ntask_s; S.parent = a->parent; S.xready = a->xready; S.done = a->done;
    S.ticket = a->ticket; S.err = a->err; S.trace = a->trace;
    S.gptr = a->gptr; S.ngroups = a->ngroups;
    S.cptr = a->cptr; S.crange = a->crange;
    S.act = a->act; S.sseg = a->sseg;
    S.bchunk_ptr = a->bchunk_ptr; S.bchunk = a->bchunk;
    if (!forward && (!S.bchunk_ptr || !S.bchunk)) return (int)cudaErrorInvalidValue;
    if (forward && (!S.cptr || !S.crange)) return (int)cudaErrorInvalidValue;
    if (S.act && !S.sseg) return (int)cudaErrorInvalidValue;
    if (grid > a->ngroups) grid = a->ngroups;
    static int configured = 0;
    if (!configured) {
        cudaFuncSetAttribute(k_fwd_sweep<double>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sweep_smem<double>());
        cudaFuncSetAttribute(k_bwd_sweep<double>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sweep_smem<double>());
        cudaFuncSetAttribute(k_fwd_sweep<float>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sweep_smem<float>());
        cudaFuncSetAttribute(k_bwd_sweep<float>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sweep_smem<float>());
        configured = 1;
    }
    if (dtype == 0) {
        const size_t sm = sweep_smem<double>();
        if (forward) k_fwd_sweep<double><<<grid, 256, sm, st>>>(P, S, (const double *)Lx, (const double *)Linv, nrhs, (double *)Y, ldy, (double *)U);
        else k_bwd_sweep<double><<<grid, 256, sm, st>>>(P, S, (const double *)Lx, (const double *)Linv, nrhs, (double *)Y, ldy);
    } else {
        const size_t sm = sweep_smem<float>();
        if (forward) k_fwd_sweep<float><<<grid, 256, sm, st>>>(P, S, (const float *)Lx, (const float *)Linv, nrhs, (float *)Y, ldy, (float *)U);
        else k_bwd_sweep<float><<<grid, 256, sm, st>>>(P, S, (const float *)Lx, (const float *)Linv, nrhs, (float *)Y, ldy);
    }
    return (int)cudaGetLastError();
}

int gb_launch_sweep_leaf(int forward, const gb_pattern_ptrs *pp, const int32_t *leaf, int nleaf,
                         const int32_t *blkoff, const int64_t *linvoff, const int32_t *ntask_f,
                         int32_t *done, int32_t *ticket, const void *Lx, const void *Linv,
                         int dtype, int nrhs, void *Y, int64_t ldy, void *U, int grid, int lrows,
                         const unsigned char *act, const int32_t *sseg, cudaStream_t st)
{
    // staging of each warp's front (ys, xs: lrows x LF_LD each)
    if (lrows < 1 || lrows > GB_LEAF_ROWS) return (int)cudaErrorInvalidValue;
    static int configured = 0;
    if (!configured) {
        const int mx = (int)(LF_WARPS * 2 * GB_LEAF_ROWS * LF_LD * sizeof(double));
        cudaFuncSetAttribute(k_fwd_leaf<double>, cudaFuncAttributeMaxDynamicSharedMemorySize, mx);
        cudaFuncSetAttribute(k_bwd_leaf<double>, cudaFuncAttributeMaxDynamicSharedMemorySize, mx);
        cudaFuncSetAttribute(k_fwd_leaf<float>, cudaFuncAttributeMaxDynamicSharedMemorySize, mx / 2);
        cudaFuncSetAttribute(k_bwd_leaf<float>, cudaFuncAttributeMaxDynamicSharedMemorySize, mx / 2);
        configured = 1;
    }
    const size_t lsm = (size_t)LF_WARPS * 2 * lrows * LF_LD * (dtype == 0 ? sizeof(double) : sizeof(float));
    if (act && !sseg) return (int)cudaErrorInvalidValue;
    if (nleaf <= 0) return 0;
    if (!leaf || !blkoff || !linvoff || !done || !ticket || !Lx || !Linv || !Y
        || (forward && (!ntask_f || !U)))
        return (int)cudaErrorInvalidValue;
    gb_dev_pattern P = gb_to_dev(pp);
    const int need = (nleaf + LF_WARPS - 1) / LF_WARPS;
    if (grid > need) grid = need;
    if (grid < 1) grid = 1;
    if (dtype == 0) {
        if (forward)
            k_fwd_leaf<double><<<grid, 32 * LF_WARPS, lsm, st>>>(P, leaf, nleaf, blkoff, linvoff, ntask_f, done, ticket,
                                                               (const double *)Lx, (const double *)Linv, nrhs, (double *)Y, ldy, (double *)U,
                                                               act, sseg, lrows);
        else
            k_bwd_leaf<double><<<grid, 32 * LF_WARPS, lsm, st>>>(P, leaf, nleaf, blkoff, linvoff, ticket,
                                                               (const double *)Lx, (const double *)Linv, nrhs, (double *)Y, ldy,
                                                               act, sseg, lrows);
    } else {
        if (forward)
            k_fwd_leaf<float><<<grid, 32 * LF_WARPS, lsm, st>>>(P, leaf, nleaf, blkoff, linvoff, ntask_f, done, ticket,
                                                              (const float *)Lx, (const float *)Linv, nrhs, (float *)Y, ldy, (float *)U,
                                                              act, sseg, lrows);
        else
            k_bwd_leaf<float><<<grid, 32 * LF_WARPS, lsm, st>>>(P, leaf, nleaf, blkoff, linvoff, ticket,
                                                              (const float *)Lx, (const float *)Linv, nrhs, (float *)Y, ldy,
                                                              act, sseg, lrows);
    }
    return (int)cudaGetLastError();
}

int gb300_wait_probe(int64_t polls, int32_t *out)
{
    if (!out || polls < 0 || polls > (1ll << 30)) return 0;
    int32_t *d = NULL;
    if (cudaMalloc((void **)&d, 4 * sizeof(int32_t)) != cudaSuccess) return 0;
    int ok = cudaMemset(d, 0, 4 * sizeof(int32_t)) == cudaSuccess;
    if (ok) {
        k_wait_probe<<<1, 32>>>(d, d + 1, (long long)polls, d + 2);
        ok = cudaGetLastError() == cudaSuccess && cudaDeviceSynchronize() == cudaSuccess
             && cudaMemcpy(out, d + 2, 2 * sizeof(int32_t), cudaMemcpyDeviceToHost) == cudaSuccess;
    }
    cudaFree(d);
    return ok;
}

int gb_launch_diag_inverse(const gb_pattern_ptrs *pp, const gb_stask *dtasks, int ndiag,
                           const int32_t *blkoff, const int64_t *linvoff, const void *Lx,
                           void *Linv, int dtype, cudaStream_t st)
{
    if (ndiag <= 0) return 0;
    gb_dev_pattern P = gb_to_dev(pp);
    if (dtype == 0) k_diag_inverse<double><<<ndiag, SR, 0, st>>>(P, dtasks, blkoff, linvoff, (const double *)Lx, (double *)Linv);
    else k_diag_inverse<float><<<ndiag, SR, 0, st>>>(P, dtasks, blkoff, linvoff, (const float *)Lx, (float *)Linv);
    return (int)cudaGetLastError();
}

}  // extern "C"
