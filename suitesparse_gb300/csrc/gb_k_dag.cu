// gb_k_dag.cu -- device task-graph executor for the wide supernodes of one
// etree level (and the update blocks of every supernode of the level).
//
// The task graph is static per symbolic pattern (built on the host,
// gb_plan.c): 64-grid tile tasks of a right-looking blocked LL' of each wide
// panel (diagonal LL' + inverse, panel solve, trailing update) and the
// update-block products.  One persistent launch executes it: thread 0 of a
// block pops a ready task (critical-path queue first), the block runs it,
// then thread 0 decrements the dependency counters of its successors and
// pushes each one that reaches zero onto the queue of its priority.  Blocks
// never wait for an unfinished task: a task is popped only when ready, so
// the executor cannot deadlock.  Popping from empty queues spins with a
// bound (GB_DAG_SPIN), after which the error word is set and every block
// returns.
//
// Reference (the same arithmetic, per supernode, on the CPU):
// CHOLMOD/Supernodal/t_cholmod_super_numeric_worker.c dpotrf :1004-1058,
// dtrsm :1152-1218, the dsyrk/dgemm update matrices :768-883.

#include "gb_k_bodies.cuh"

#define GB_DAG_SPIN (1 << 24)

// ready queues and control words of one executor launch
struct gb_dq {
    int32_t *q0, *q1;        // ready queues: slot = task id, -1 not yet written
    int32_t *ctrl;           // GB_DAG_NCTRL control words (gb_kernels.cuh)
    int32_t *err;            // error word kept across launches
    int32_t *smflag;         // per SM: epoch of the launch whose poller runs there
    int32_t epoch;
    int32_t npoll;           // blocks that serve only the critical queue
};

struct gb_dag_dev {
    gb_dq Q;
    const gb_dtask *tasks;
    int ntasks;
    const int32_t *succ_ptr, *succ;
    int32_t *cnt;            // live dependency counters
    unsigned long long *trace; // optional: per task [claimed, finished, block] (ns)
};

__device__ __forceinline__ unsigned long long dag_timer()
{
    unsigned long long t;
    asm volatile("mov.u64 %0, %globaltimer;" : "=l"(t));
    return t;
}

__device__ __forceinline__ int dag_ld_acquire(const int32_t *p)
{
    int v;
    asm volatile("ld.acquire.gpu.global.b32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

__device__ __forceinline__ void dag_st_release(int32_t *p, int v)
{
    asm volatile("st.release.gpu.global.b32 [%0], %1;" :: "l"(p), "r"(v) : "memory");
}

__device__ __forceinline__ int dag_add_acq_rel(int32_t *p, int v)
{
    int old;
    asm volatile("atom.acq_rel.gpu.global.add.s32 %0, [%1], %2;" : "=r"(old) : "l"(p), "r"(v) : "memory");
    return old;
}

// thread 0: claim slot h of a queue (the pusher reserved it with tail and
// writes it right away, or will once the task is ready)
__device__ int dag_take(const gb_dq &D, const int32_t *slots, int h)
{
    for (int k = 0; k < GB_DAG_SPIN; k++) {
        const int v = dag_ld_acquire(slots + h);
        if (v >= 0) return v;
        if (dag_ld_acquire(D.ctrl + 5)) return -2;
        __nanosleep(k < 64 ? 32 : 256);
    }
    atomicExch(D.ctrl + 5, 1);
    atomicExch(D.err, 1);
    return -2;
}

// Thread 0: the next task id, -1 when its queue is exhausted, -2 on error.
// The first D.npoll blocks to start serve the critical-path queue:
// they claim a slot only when it is already reserved (compare-and-swap on
// the head, no waiting for future tasks).  All other blocks claim bulk-queue
// slots in order with atomicAdd and wait for their slot to be filled.
// Deadlock-free: slots are reserved in order, so a block waiting on a bulk
// slot waits either for a slot being written or for a task not yet ready,
// and every ready task is either in a claimed slot (its block runs it) or
// is a critical task a poller can claim; pollers never wait.
__device__ int dag_pop(const gb_dq &D, int poller)
{
    int32_t *ctrl = D.ctrl;
    if (!poller) {
        const int h = atomicAdd(ctrl + 2, 1);
        if (h >= ctrl[7]) return -1;
        return dag_take(D, D.q1, h);
    }
    for (int it = 0; it < GB_DAG_SPIN; it++) {
        if (dag_ld_acquire(ctrl + 5)) return -2;
        // the critical total shrinks when a block keeps a critical task it
        // made ready (k_fdag) instead of queueing it
        const int total0 = dag_ld_acquire(ctrl + 6);
        int h0 = dag_ld_acquire(ctrl + 0);
        if (h0 < total0 && h0 < dag_ld_acquire(ctrl + 1)) {
            if (atomicCAS(ctrl + 0, h0, h0 + 1) == h0) return dag_take(D, D.q0, h0);
            continue;
        }
        if (h0 >= total0) return -1;
        __nanosleep(64);
    }
    atomicExch(ctrl + 5, 1);
    atomicExch(D.err, 1);
    return -2;
}

// Thread 0 of a bulk block when no block is a dedicated poller
// (D.npoll = 0): like dag_pop for a bulk block, but while its bulk slot is
// empty the block takes any ready critical task instead, keeping the slot's
// ticket (*ticket, -1 for none) for its next call.  Deadlock-free as
// dag_pop: a ready critical task is taken by any waiting bulk block, and a
// block whose bulk queue is exhausted serves the critical queue.
__device__ int dag_pop_bulk(const gb_dq &D, int *ticket)
{
    int32_t *ctrl = D.ctrl;
    if (*ticket < 0) {
        const int h = atomicAdd(ctrl + 2, 1);
        if (h >= ctrl[7]) return -1;
        *ticket = h;
    }
    for (int k = 0; k < GB_DAG_SPIN; k++) {
        const int v = dag_ld_acquire(D.q1 + *ticket);
        if (v >= 0) {
            *ticket = -1;
            return v;
        }
        if (dag_ld_acquire(ctrl + 5)) return -2;
        const int h0 = dag_ld_acquire(ctrl + 0);
        if (h0 < dag_ld_acquire(ctrl + 6) && h0 < dag_ld_acquire(ctrl + 1)
            && atomicCAS(ctrl + 0, h0, h0 + 1) == h0)
            return dag_take(D, D.q0, h0);
        __nanosleep(k < 64 ? 32 : 256);
    }
    atomicExch(ctrl + 5, 1);
    atomicExch(D.err, 1);
    return -2;
}

// warp 0: queue task v (its last dependency just finished) on the queue of
// its priority
__device__ __forceinline__ void dag_push(const gb_dq &D, int v, int prio)
{
    const int q = prio ? 1 : 0;
    const int slot = atomicAdd(D.ctrl + 2 * q + 1, 1);
    dag_st_release((q ? D.q1 : D.q0) + slot, v);
}

// warp 0, after the block finished task id (and a block barrier): release
// the block's writes, then decrement the successors' dependency counters,
// one successor per lane (critical successors come first in the list), and
// queue those that became ready
__device__ void dag_complete(const gb_dag_dev &D, int id)
{
    __threadfence();
    const int e0 = D.succ_ptr[id], e1 = D.succ_ptr[id + 1];
    for (int e = e0 + (int)(threadIdx.x & 31); e < e1; e += 32) {
        const int v = D.succ[e];
        if (dag_add_acq_rel(D.cnt + v, -1) == 1) dag_push(D.Q, v, D.tasks[v].prio);
    }
}

// thread 0 at the start of an executor block: 1 = poller, 0 = bulk block,
// 2 = leave.  The first D.npoll blocks to start serve the critical queue
// and mark their SM.  The critical path is a chain of latency-bound tasks,
// so a bulk block that finds itself on a marked SM leaves (at most 2 npoll
// of them, and only in a large grid, so that plenty of bulk blocks remain).
__device__ int dag_role(const gb_dq &D)
{
    int role = atomicAdd(D.ctrl + 4, 1) < D.npoll;
    unsigned smid;
    asm volatile("mov.u32 %0, %%smid;" : "=r"(smid));
    smid %= GB_DAG_NSMF;
    if (role) {
        atomicExch(D.smflag + smid, D.epoch);
    } else if (D.npoll > 0 && gridDim.x >= 4 * D.npoll && dag_ld_acquire(D.smflag + smid) == D.epoch
               && atomicAdd(D.ctrl + 8, 1) < 2 * D.npoll) {
        role = 2;
    }
    return role;
}

template <typename T>
__host__ __device__ constexpr size_t dag_smem()
{
    // diagonal block (64 x 65) + two operand tiles (64 x 65) for the panel
    // solve; the tile update uses 2 x 16 x 68 of the same space
    return sizeof(T) * (3 * 64 * 65);
}

// The POTRF and TRSM tile tasks, each with a register allocation of its own
// (their tile loads hold 16-32 registers per thread; inlined, they would
// push the tile products of the executor loop into spills).
template <typename T>
static __device__ __noinline__ void potrf_task(const gb_dev_pattern &P, const gb_dtask &tk, T *panel,
                                               int nscol, int nsrow, int f, T *Linv,
                                               unsigned char *smem_raw, int &sfail)
{
    T (*A)[65] = (T (*)[65])smem_raw;
    T *S1 = (T *)smem_raw + 64 * 65, *S2 = S1 + 64 * 65;
    const int s = tk.s;
    const int c0 = 64 * tk.b, nb = min(64, nscol - c0);
    if (f < 0) {
        T *blk = panel + c0 + (int64_t)c0 * nsrow;
        // every load of the tile in flight before the shared stores
        // (256 threads, 16 elements each)
        T v[16];
#pragma unroll
        for (int q = 0; q < 16; q++) {
            const int idx = threadIdx.x + 256 * q, i = idx & 63, j = idx >> 6;
            v[q] = (i < nb && j < nb && i >= j) ? blk[i + (int64_t)j * nsrow] : (T)0;
        }
#pragma unroll
        for (int q = 0; q < 16; q++) {
            const int idx = threadIdx.x + 256 * q;
            A[idx & 63][idx >> 6] = v[q];
        }
        __syncthreads();
        const int fl = potrf_inv64<T>(A, S1, S2, nb, &sfail);
        __syncthreads();
        for (int idx = threadIdx.x; idx < nb * nb; idx += blockDim.x) {
            const int i = idx % nb, j = idx / nb;
            if (i >= j) blk[i + (int64_t)j * nsrow] = A[i][j];
        }
        if (fl >= 0 && threadIdx.x == 0) {
            P.fail[s] = c0 + fl;
            atomicExch(P.anyfail, 1);
        }
        T *li = Linv + P.linvoff[P.blkoff[s] + tk.b];
        for (int idx = threadIdx.x; idx < nb * nb; idx += blockDim.x) {
            const int i = idx % nb, j = idx / nb;
            li[i + (int64_t)j * nb] = S1[j * 65 + i];
        }
    }
}

template <typename T>
static __device__ __noinline__ void trsm_task(const gb_dev_pattern &P, const gb_dtask &tk, T *panel,
                                              int nscol, int nsrow, int f, const T *Linv,
                                              unsigned char *smem_raw, float *Img)
{
    T *S1 = (T *)smem_raw + 64 * 65, *S2 = S1 + 64 * 65;
    const int s = tk.s;
    const int c0 = 64 * tk.b, nb = min(64, nscol - c0);
    if (!(f >= 0 && f < c0)) {
        const int ncols = (f >= 0) ? f - c0 : nb;
        const int r0 = max(64 * tk.r, c0 + nb), r1 = min(64 * tk.r + 64, nsrow);
        const int nr = r1 - r0;
        const T *li = Linv + P.linvoff[P.blkoff[s] + tk.b];
        // both tiles' loads in flight before the shared stores
        T v[16], w[16];
#pragma unroll
        for (int q = 0; q < 16; q++) {
            const int idx = threadIdx.x + 256 * q, cc = idx & 63, k = idx >> 6;
            v[q] = (cc < nb && k < nb) ? li[cc + (int64_t)k * nb] : (T)0;
            w[q] = (cc < nr && k < nb) ? panel[r0 + cc + (int64_t)(c0 + k) * nsrow] : (T)0;
        }
#pragma unroll
        for (int q = 0; q < 16; q++) {
            const int idx = threadIdx.x + 256 * q, cc = idx & 63, k = idx >> 6;
            S2[k * 65 + cc] = v[q];
            S1[k * 65 + cc] = w[q];
        }
        __syncthreads();
        // FP32 on the tensor cores: the block is also the operand image of
        // the tile products that read it (UPD, CB)
        float *img = nullptr;
        if (Img && P.imgbase[s] >= 0)
            img = (float *)gb_img_ptr(Img, P.imgbase[s], (nsrow + 63) / 64, tk.b, tk.r);
        trsm_tile<T>(S1, S2, 65, nr, nb, ncols, panel + r0 + (int64_t)c0 * nsrow, nsrow, img,
                     r0 - 64 * tk.r);
    }
}

// The diagonal step's last update of tile (b, b) and its LL' and inverse in
// one pass: C = A(b, b) - sum over the panels p of the update (tk.r ..
// tk.r + tk.nbk - 1) of L(b, p) L(b, p)', formed on the CUDA cores (each
// thread 4 x 4 entries of the tile, one 64-column panel staged in shared
// memory at a time) straight into the shared tile that potrf_inv64
// factors, so the tile makes no round trip through global memory between
// the update and the factorization.  The products are summed from zero and
// subtracted from A(b, b) once (subtracting each product in turn loses
// accuracy in the pivots).  The tile is the whole 64-row row block
// b: when panel b is narrower than 64, its rows below the diagonal block
// (read later by that row block's panel solve) are updated too and stored
// back.  Stores L(b, b) and its inverse as potrf_task does.  Skipped for a
// supernode that already failed.
template <typename T>
static __device__ __noinline__ void diag_update_potrf(const gb_dev_pattern &P, const gb_dtask &tk, T *Lx,
                                                      T *Linv, unsigned char *smem_raw, int &sfail)
{
    T (*A)[65] = (T (*)[65])smem_raw;
    T *S1 = (T *)smem_raw + 64 * 65, *S2 = S1 + 64 * 65;
    const int s = tk.s, b = tk.b;
    const int nscol = (int)(P.Super[s + 1] - P.Super[s]);
    const int nsrow = (int)(P.Pi[s + 1] - P.Pi[s]);
    if (P.fail[s] >= 0) return;
    T *panel = Lx + P.Px[s];
    const int c0 = 64 * b, nb = min(64, nscol - c0), mr = min(64, nsrow - c0);
    const int p0 = tk.r, nbk = max(1, tk.nbk);
    T *blk = panel + c0 + (int64_t)c0 * nsrow;
    const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
    T acc[4][4], cv[4][4];
#pragma unroll
    for (int a = 0; a < 4; a++)
#pragma unroll
        for (int q = 0; q < 4; q++) {
            const int i = ty + 16 * a, j = tx + 16 * q;
            cv[a][q] = (i < mr && j < nb && i >= j) ? blk[i + (int64_t)j * nsrow] : (T)0;
            acc[a][q] = (T)0;
        }
    for (int p = p0; p < p0 + nbk; p++) {
        const int kc = min(64, nscol - 64 * p);
        // S1[k * 65 + i] = L(c0 + i, 64 p + k); every load in flight first
        T v[16];
#pragma unroll
        for (int q = 0; q < 16; q++) {
            const int idx = threadIdx.x + 256 * q, i = idx & 63, k = idx >> 6;
            v[q] = (i < mr && k < kc) ? panel[c0 + i + (int64_t)(64 * p + k) * nsrow] : (T)0;
        }
#pragma unroll
        for (int q = 0; q < 16; q++) {
            const int idx = threadIdx.x + 256 * q;
            S1[(idx >> 6) * 65 + (idx & 63)] = v[q];
        }
        __syncthreads();
        for (int k = 0; k < kc; k++) {
            T x[4], y[4];
#pragma unroll
            for (int a = 0; a < 4; a++) x[a] = S1[k * 65 + ty + 16 * a];
#pragma unroll
            for (int q = 0; q < 4; q++) y[q] = S1[k * 65 + tx + 16 * q];
#pragma unroll
            for (int a = 0; a < 4; a++)
#pragma unroll
                for (int q = 0; q < 4; q++) acc[a][q] += x[a] * y[q];
        }
        __syncthreads();
    }
#pragma unroll
    for (int a = 0; a < 4; a++)
#pragma unroll
        for (int q = 0; q < 4; q++) acc[a][q] = cv[a][q] - acc[a][q];
#pragma unroll
    for (int a = 0; a < 4; a++)
#pragma unroll
        for (int q = 0; q < 4; q++) {
            const int i = ty + 16 * a, j = tx + 16 * q;
            A[i][j] = (i < nb && j < nb && i >= j) ? acc[a][q] : (T)0;
            if (i >= nb && i < mr && j < nb) blk[i + (int64_t)j * nsrow] = acc[a][q];
        }
    __syncthreads();
    const int fl = potrf_inv64<T>(A, S1, S2, nb, &sfail);
    __syncthreads();
    for (int idx = threadIdx.x; idx < nb * nb; idx += blockDim.x) {
        const int i = idx % nb, j = idx / nb;
        if (i >= j) blk[i + (int64_t)j * nsrow] = A[i][j];
    }
    if (fl >= 0 && threadIdx.x == 0) {
        P.fail[s] = c0 + fl;
        atomicExch(P.anyfail, 1);
    }
    T *li = Linv + P.linvoff[P.blkoff[s] + b];
    for (int idx = threadIdx.x; idx < nb * nb; idx += blockDim.x) {
        const int i = idx % nb, j = idx / nb;
        li[i + (int64_t)j * nb] = S1[j * 65 + i];
    }
}

// The work of one tile task (POTRF, TRSM, UPD or CB) of supernode tk.s.
// smem_raw: dag_smem<T>() bytes (GB_TC_SMEM with tc).  With tc and Img
// (FP32 on the tensor cores), TRSM also writes the split operand images and
// UPD / CB tiles read them (gemm_img_tc).  CB tiles with tk.b = 1 lie on the
// 64-row grid of the supernode's rows (tile (r, c): rows [max(64 r, nscol),
// min(64 r + 64, nsrow)) and likewise the columns, in update-block
// coordinates minus nscol), those with tk.b = 0 on the grid of the update
// block itself.
template <typename T>
__device__ void tile_body(const gb_dev_pattern &P, const gb_dtask &tk, T *Lx, T *CB, T *Linv,
                          unsigned char *smem_raw, int &sfail, gb_tc_ctx *tc, float *Img)
{
    T (*A)[65] = (T (*)[65])smem_raw;
    T *S1 = (T *)smem_raw + 64 * 65, *S2 = S1 + 64 * 65;
    const int s = tk.s;
    const int nscol = (int)(P.Super[s + 1] - P.Super[s]);
    const int nsrow = (int)(P.Pi[s + 1] - P.Pi[s]);
    T *panel = Lx + P.Px[s];
    const int f = P.fail[s];
    const bool img = tc && Img && P.imgbase[s] >= 0;
    if (tk.type == GB_DT_POTRF) {
        potrf_task<T>(P, tk, panel, nscol, nsrow, f, Linv, smem_raw, sfail);
    } else if (tk.type == GB_DT_TRSM) {
        trsm_task<T>(P, tk, panel, nscol, nsrow, f, Linv, smem_raw, img ? Img : nullptr);
    } else if (tk.type == GB_DT_UPD) {
        if (f < 0) {
            // panels b .. b + nbk - 1 at once: k = their columns
            const int nbk = max(1, tk.nbk);
            const int c0 = 64 * tk.b, kk = min(64 * (tk.b + nbk), nscol) - c0;
            const int cs = 64 * tk.c, ce = min(cs + 64, nscol);
            const int rs = max(64 * tk.r, cs), re = min(64 * tk.r + 64, nsrow);
            if constexpr (sizeof(T) == 4) {
                if (img) {
                    // rows 64 r.. of the images of row blocks r and c of
                    // those panels (rs = 64 r: r >= c); the last panel's
                    // second K chunk is empty when it is at most 32 wide
                    const int nb_last = kk - 64 * (nbk - 1);
                    gemm_img_tc(Img, P.imgbase[s], (nsrow + 63) / 64, tk.r, tk.c, tk.b,
                                2 * nbk - (nb_last > 32 ? 0 : 1), (float *)Lx,
                                P.Px[s] + rs + (int64_t)cs * nsrow, nsrow,
                                0, re - rs, 0, ce - cs, tk.r == tk.c, smem_raw, *tc);
                    return;
                }
                gemm_tile_f32(panel + rs + (int64_t)c0 * nsrow, nsrow,
                              panel + cs + (int64_t)c0 * nsrow, nsrow,
                              panel + rs + (int64_t)cs * nsrow, nsrow,
                              re - rs, ce - cs, kk, tk.r == tk.c, cs - rs, (float *)smem_raw);
            }
            else if (kk <= 64)
                gemm_tile_k64<T>(panel + rs + (int64_t)c0 * nsrow, nsrow,
                                 panel + cs + (int64_t)c0 * nsrow, nsrow,
                                 panel + rs + (int64_t)cs * nsrow, nsrow,
                                 re - rs, ce - cs, kk, tk.r == tk.c, cs - rs, S1, S2);
            else
                gemm_tile_nt<T>(panel + rs + (int64_t)c0 * nsrow, nsrow,
                                panel + cs + (int64_t)c0 * nsrow, nsrow,
                                panel + rs + (int64_t)cs * nsrow, nsrow,
                                re - rs, ce - cs, kk, tk.r == tk.c, cs - rs, S1, S2);
        }
    } else {  // GB_DT_CB
        if (f < 0) {
            const int m = nsrow - nscol;
            int I = 64 * tk.r, J = 64 * tk.c, mt = min(64, m - I), nt = min(64, m - J);
            if (tk.b == 1) {
                // 64-row grid of the supernode's rows
                const int ri = max(64 * tk.r, nscol), ci = max(64 * tk.c, nscol);
                mt = min(64 * tk.r + 64, nsrow) - ri;
                nt = min(64 * tk.c + 64, nsrow) - ci;
                I = ri - nscol;
                J = ci - nscol;
                if constexpr (sizeof(T) == 4) {
                    if (img) {
                        // output (i, j) = rows 64 r + i, 64 c + j of the
                        // images; those below nscol are skipped
                        const int i0 = ri - 64 * tk.r, j0 = ci - 64 * tk.c;
                        const int nb_last = nscol - 64 * ((nscol - 1) / 64);
                        const int nch = 2 * ((nscol + 63) / 64) - (nb_last > 32 ? 0 : 1);
                        gemm_img_tc(Img, P.imgbase[s], (nsrow + 63) / 64, tk.r, tk.c, 0, nch,
                                    (float *)CB, P.cboff[s] + (int64_t)(I - i0) + (int64_t)(J - j0) * m,
                                    m, i0, i0 + mt, j0, j0 + nt, tk.r == tk.c, smem_raw, *tc);
                        return;
                    }
                }
            }
            if constexpr (sizeof(T) == 4)
                gemm_tile_f32(panel + nscol + I, nsrow, panel + nscol + J, nsrow,
                              CB + P.cboff[s] + I + (int64_t)J * m, m,
                              mt, nt, nscol, tk.r == tk.c, 0, (float *)smem_raw);
            else
                gemm_tile_nt<T>(panel + nscol + I, nsrow, panel + nscol + J, nsrow,
                                CB + P.cboff[s] + I + (int64_t)J * m, m,
                                mt, nt, nscol, tk.r == tk.c, 0, S1, S2);
        }
    }
}

// The work of one task of the tile graph: POTRF, TRSM, UPD or CB as
// above, or DIAG (s, b, r, nbk), the diagonal chain of panel b as one task:
// the panel solve of row block b by panel b - 1, the update of tile (b, b)
// by panels r .. r + nbk - 1, then POTRF of panel b, in that order on this
// block (each step reads what the previous one wrote, after a barrier; the
// operand images written by the solve are fenced for the bulk copies).
template <typename T>
__device__ void dag_tile_task(const gb_dev_pattern &P, const gb_dtask &tk, T *Lx, T *CB, T *Linv,
                              unsigned char *smem_raw, int &sfail, gb_tc_ctx *tc = nullptr,
                              float *Img = nullptr)
{
    if (tk.type != GB_DT_DIAG) {
        tile_body<T>(P, tk, Lx, CB, Linv, smem_raw, sfail, tc, Img);
        return;
    }
    const gb_dtask t1 = {GB_DT_TRSM, tk.s, tk.b - 1, tk.b, 0, 0, 0, 0};
    tile_body<T>(P, t1, Lx, CB, Linv, smem_raw, sfail, tc, Img);
    __syncthreads();
    if (tc && !tc->ok) return;
    diag_update_potrf<T>(P, tk, Lx, Linv, smem_raw, sfail);
}

template <typename T>
__global__ void __launch_bounds__(256, 2)
k_dag(gb_dev_pattern P, gb_dag_dev D, T *Lx, T *CB, T *Linv)
{
    extern __shared__ __align__(1024) unsigned char smem_raw[];
    __shared__ int sid, sfail, spoll;
    if (threadIdx.x == 0) spoll = dag_role(D.Q);
    __syncthreads();
    if (spoll == 2) return;
    const int poller = spoll;
    for (;;) {
        if (threadIdx.x == 0) sid = dag_pop(D.Q, poller);
        __syncthreads();
        const int id = sid;
        if (id < 0) return;
        if (D.trace && threadIdx.x == 0) {
            D.trace[3 * (size_t)id] = dag_timer();
            D.trace[3 * (size_t)id + 2] = blockIdx.x;
        }
        const gb_dtask tk = D.tasks[id];
        dag_tile_task<T>(P, tk, Lx, CB, Linv, smem_raw, sfail);
        __syncthreads();
        if (threadIdx.x < 32) {
            if (D.trace && threadIdx.x == 0) D.trace[3 * (size_t)id + 1] = dag_timer();
            dag_complete(D, id);
        }
    }
}

// ---------------------------------------------------------------------------
// whole-factorization executor: every level's tile tasks, the assembly
// chunks and the small supernodes of one or more instances of a pattern in
// one persistent launch (graph built by gb_plan.c: fdag_build)
// ---------------------------------------------------------------------------

struct gb_fdag_dev {
    gb_dq Q;
    int use_tc;              // FP32 tile products on the tensor cores
    float *img;              // their split operand images (gb_img_ptr)
    const gb_fpat *pats;
    const gb_finst *inst;
    const int64_t *ibase;
    int ninst;
    int32_t *cnt;
    unsigned long long *trace;
    const void *Sx;
    int a_dtype;
    const double *scale;
    double beta;
};

// thread 0: the instance that owns global task id (ibase ascending)
__device__ __forceinline__ int fdag_instance(const gb_fdag_dev &D, int id)
{
    int lo = 0, hi = D.ninst - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (D.ibase[mid] <= id) lo = mid; else hi = mid - 1;
    }
    return lo;
}

// One-warp fronts of a subtree wave: fdag_nw64 warps own a region for
// fronts of up to 64 rows.  FP32: the other warps own regions for fronts of
// up to 32 rows and both kinds run in one phase (fdag_merged); FP64: the
// 32-row fronts (every warp) and the 64-row fronts run in two phases over
// the same space.
template <typename T>
__host__ __device__ constexpr int fdag_nw64()
{
    return sizeof(T) == 4 ? 6 : 3;
}

template <typename T>
__host__ __device__ constexpr bool fdag_merged()
{
    return sizeof(T) == 4;
}

template <typename T>
__host__ __device__ constexpr size_t fdag_front_smem()
{
    return fdag_merged<T>()
        ? fdag_nw64<T>() * warp_front_smem<64, T>() + (8 - fdag_nw64<T>()) * warp_front_smem<32, T>()
        : (fdag_nw64<T>() * warp_front_smem<64, T>() > 8 * warp_front_smem<32, T>()
               ? fdag_nw64<T>() * warp_front_smem<64, T>() : 8 * warp_front_smem<32, T>());
}

// dynamic shared memory of the executor: the tile tasks' space, the fronts'
// regions and (FP32) the operand stages of gemm_img_tc
template <typename T>
__host__ __device__ constexpr size_t fdag_smem()
{
    return (sizeof(T) == 4 && (size_t)GB_TC_SMEM > fdag_front_smem<T>() && (size_t)GB_TC_SMEM > dag_smem<T>())
        ? (size_t)GB_TC_SMEM
        : (fdag_front_smem<T>() > dag_smem<T>() ? fdag_front_smem<T>() : dag_smem<T>());
}

// two blocks share an SM (228 KB, 1 KB reserved per block, the kernel's
// static shared variables under 1 KB); with the tensor cores more than a
// third of the SM's shared memory, so that no third block (2 x GB_TC_COLS
// TMEM columns each) is resident
static_assert(2 * (fdag_smem<float>() + 2048) <= 228 * 1024
              && 2 * (fdag_smem<double>() + 2048) <= 228 * 1024, "executor: two blocks per SM");
static_assert(3 * fdag_smem<float>() > 228 * 1024, "tensor-core executor: at most two blocks per SM");

// All threads of the block, after a barrier that follows the work whose
// results the successors read: release the block's writes, decrement the
// dependency counters of successors succ[ea, eb) of the task (one round of
// atomics for up to blockDim.x successors) and queue those that became
// ready.  A join (no work, never queued) releases its own successors here.
// keep: a critical successor that becomes ready may be kept in *snext for
// this block to run next (a poller, at the end of its task); otherwise
// every ready successor is queued.  Ends with a barrier (snext, set by any
// thread, is read by thread 0).
__device__ void fdag_release(const gb_fdag_dev &D, const gb_fpat &PP, const gb_finst &I, int ea,
                             int eb, bool keep, int *snext)
{
    // the successor lists and the successors' type and priority are plan
    // data, never written by the launch: a thread's first successor is
    // read before the fence, so those loads overlap the fence instead of
    // adding two round trips after it
    const int e0 = ea + (int)threadIdx.x;
    int v0 = -1, ty0 = 0, pr0 = 0;
    if (e0 < eb) {
        v0 = PP.succ[e0];
        ty0 = PP.tasks[v0].type;
        pr0 = PP.tasks[v0].prio;
        __threadfence();
    }
    for (int e = e0; e < eb; e += (int)blockDim.x) {
        const bool first = e == e0;
        const int v = first ? v0 : PP.succ[e];
        const int g = (int)(I.base + v);
        if (dag_add_acq_rel(D.cnt + g, -1) != 1) continue;
        if ((first ? ty0 : PP.tasks[v].type) != GB_DT_JOIN) {
            const int prio = first ? pr0 : PP.tasks[v].prio;
            if (prio == 0 && keep && atomicCAS(snext, -1, g) == -1) {
                atomicSub(D.Q.ctrl + 6, 1);     // kept: one less to queue
                continue;
            }
            dag_push(D.Q, g, prio);
            continue;
        }
        for (int f = PP.succ_ptr[v]; f < PP.succ_ptr[v + 1]; f++) {
            const int w = PP.succ[f];
            const int gw = (int)(I.base + w);
            if (dag_add_acq_rel(D.cnt + gw, -1) != 1) continue;
            const int pw = PP.tasks[w].prio;
            if (pw == 0 && keep && atomicCAS(snext, -1, gw) == -1) {
                atomicSub(D.Q.ctrl + 6, 1);     // kept: one less to queue
                continue;
            }
            dag_push(D.Q, gw, pw);
        }
    }
    __syncthreads();
}

// one front of at most MAXR rows on the calling warp, A's values in the
// launch's precision
template <int MAXR, typename T>
__device__ __forceinline__ void fdag_warp_front(const gb_fdag_dev &D, const gb_finst &I, const gb_fpat &PP,
                                                const gb_dev_pattern &P, int s, const double *scale, T *Lx,
                                                T *CB, T *Linv, unsigned char *wsm)
{
    if (D.a_dtype == 0)
        warp_front<MAXR, double, T>(P, s, PP.Sp, PP.Si, (const double *)D.Sx + I.sx, scale, D.beta, Lx,
                                    CB, Linv, wsm);
    else
        warp_front<MAXR, float, T>(P, s, PP.Sp, PP.Si, (const float *)D.Sx + I.sx, scale, D.beta, Lx, CB,
                                   Linv, wsm);
}

template <typename T, bool TC>
__global__ void __launch_bounds__(256, 2)
k_fdag(gb_fdag_dev D, T *LxB, T *CBB, T *LinvB)
{
    extern __shared__ __align__(1024) unsigned char smem_raw[];
    __shared__ int sid, sinst, sfail, spoll, snext;
    __shared__ int sclaim[4];          // claim counters of subtree waves (two pairs)
    __shared__ int sticket;            // bulk slot held while serving critical tasks (npoll = 0)
    __shared__ __align__(8) uint64_t mbar[GB_TC_NBAR];
    __shared__ uint32_t tmem_base;
    if (threadIdx.x == 0) {
        spoll = dag_role(D.Q);
        snext = -1;
        sticket = -1;
    }
    __syncthreads();
    if (spoll == 2) return;
    // spoll: 1 = poller (a bulk block becomes one when the bulk queue is
    // exhausted, and serves the critical queue until it drains)
    // FP32: tile products on the tensor cores; two TMEM accumulators of 128
    // columns for the block's lifetime (GB_TC_COLS; the launch's shared
    // memory keeps at most 2 blocks per SM: 512 of 512 columns)
    gb_tc_ctx tcx = {0u, 0u, 0u, 1};
    gb_tc_ctx *tc = nullptr;
    if constexpr (TC && sizeof(T) == 4) {
        {
            if (threadIdx.x == 0) {
                for (int i = 0; i < GB_TC_NBAR; i++)
                    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" :: "r"(gb_su32(&mbar[i])), "r"(1));
                asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
            }
            if (threadIdx.x < 32) {
                asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;"
                             :: "r"(gb_su32(&tmem_base)), "r"(GB_TC_COLS));
                asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
            }
            asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
            __syncthreads();
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            tcx.taddr = tmem_base;
            tcx.mbar = gb_su32(&mbar[0]);
            tc = &tcx;
        }
    }
    for (;;) {
        if (threadIdx.x == 0) {
            // a critical task this block (a poller) made ready runs here
            // next, without a trip through the queue
            if (snext >= 0) {
                sid = snext;
                snext = -1;
            } else {
                sid = spoll || D.Q.npoll ? dag_pop(D.Q, spoll) : dag_pop_bulk(D.Q, &sticket);
                if (sid == -1 && !spoll) {
                    spoll = 1;
                    sid = dag_pop(D.Q, 1);
                }
            }
            if (sid >= 0) sinst = fdag_instance(D, sid);
        }
        __syncthreads();
        const int id = sid;
        if (id < 0) break;
        if (D.trace && threadIdx.x == 0) {
            unsigned smid;
            asm volatile("mov.u32 %0, %%smid;" : "=r"(smid));
            D.trace[3 * (size_t)id] = dag_timer();
            D.trace[3 * (size_t)id + 2] = ((unsigned long long)smid << 32) | blockIdx.x;
        }
        const gb_finst I = D.inst[sinst];
        const gb_fpat &PP = D.pats[I.pat];
        const int local = (int)(id - I.base);
        const gb_dtask tk = PP.tasks[local];
        gb_dev_pattern P = gb_to_dev(&PP.pp);
        P.fail = I.fail;
        P.anyfail = I.anyfail;
        T *Lx = LxB + I.lx, *CB = CBB + I.cb, *Linv = LinvB + I.linv;
        if (tk.type == GB_DT_ASM) {
            const gb_asm_task a = {tk.s, tk.b, tk.r, 0};
            const double *scale = D.scale ? D.scale + I.scale : nullptr;
            if (D.a_dtype == 0)
                assemble_body<double, T>(P, a, PP.Sp, PP.Si, (const double *)D.Sx + I.sx, scale,
                                         D.beta, Lx, CB);
            else
                assemble_body<float, T>(P, a, PP.Sp, PP.Si, (const float *)D.Sx + I.sx, scale,
                                        D.beta, Lx, CB);
        } else if (tk.type == GB_DT_SMALL) {
            factor_small_body<T>(P, tk.s, Lx, Linv, smem_raw, &sfail);
        } else if (tk.type == GB_DT_NODE || tk.type == GB_DT_SUBTREE) {
            // a small supernode whole (NODE), or every supernode of a subtree
            // wave by wave, children in earlier waves (SUBTREE).  A front of
            // at most warp_rows rows runs on one warp (a wave's such fronts
            // side by side, a warp each); any other runs on the whole block:
            // assembly, LL', then every update-block tile.  A
            // parent reads its children's update blocks, written by this
            // block, after a barrier.
            const double *scale = D.scale ? D.scale + I.scale : nullptr;
            const int warp = threadIdx.x >> 5;
            const bool node = tk.type == GB_DT_NODE;
            // a wave [q, w3): fronts of at most 32 rows [q, w1) and of at most
            // warp_rows rows [w1, w2), one warp each; others [w2, w3).  FP32:
            // one phase in which warps 0 .. NW64-1 take the 64-row fronts and
            // then, like every other warp, the 32-row ones, each warp claiming
            // the next front of a list; FP64: the 32-row fronts (eight at a
            // time), a barrier, the 64-row fronts (NW64 at a time).
            constexpr int NW64 = fdag_nw64<T>();
            constexpr size_t WF64 = warp_front_smem<64, T>(), WF32 = warp_front_smem<32, T>();
            int q = 0, w1 = 0, w2 = 0, w3 = 1, wave = 0;
            if (node) {
                const int nr = (int)(P.Pi[tk.s + 1] - P.Pi[tk.s]);
                w1 = nr <= min(PP.warp_rows, 32) ? 1 : 0;
                w2 = nr <= PP.warp_rows ? 1 : 0;
            }
            if constexpr (fdag_merged<T>()) {
                if (threadIdx.x == 0) sclaim[0] = sclaim[1] = 0;
                __syncthreads();
            }
            while (q < (node ? 1 : tk.r)) {
                if (!node) {
                    w1 = PP.sub_meta[3 * (tk.b + q)];
                    w2 = PP.sub_meta[3 * (tk.b + q) + 1];
                    w3 = PP.sub_meta[3 * (tk.b + q) + 2];
                    if (w3 <= q || w3 > tk.r || w1 < q || w1 > w2 || w2 > w3) {
                        if (threadIdx.x == 0) atomicExch(D.Q.err, 1);
                        break;
                    }
                }
                if constexpr (fdag_merged<T>()) {
                    // claim counters of this wave: sclaim[2 (wave & 1) ..];
                    // thread 0 clears the next wave's pair, which no warp
                    // touches before this wave's barrier (a wave always has
                    // one: the phase's, or the block fronts')
                    int *c64 = sclaim + 2 * (wave & 1), *c32 = c64 + 1;
                    if (threadIdx.x == 0) {
                        sclaim[2 * ((wave + 1) & 1)] = 0;
                        sclaim[2 * ((wave + 1) & 1) + 1] = 0;
                    }
                    const int lane = threadIdx.x & 31;
                    unsigned char *wsm = warp < NW64 ? smem_raw + (size_t)warp * WF64
                                                     : smem_raw + NW64 * WF64 + (size_t)(warp - NW64) * WF32;
                    if (warp < NW64 && w2 > w1) {
                        for (;;) {
                            int i = 0;
                            if (lane == 0) i = atomicAdd(c64, 1);
                            i = w1 + __shfl_sync(0xffffffffu, i, 0);
                            if (i >= w2) break;
                            fdag_warp_front<64, T>(D, I, PP, P, node ? tk.s : PP.sub_list[tk.b + i], scale,
                                                   Lx, CB, Linv, wsm);
                        }
                    }
                    if (w1 > q) {
                        for (;;) {
                            int i = 0;
                            if (lane == 0) i = atomicAdd(c32, 1);
                            i = q + __shfl_sync(0xffffffffu, i, 0);
                            if (i >= w1) break;
                            fdag_warp_front<32, T>(D, I, PP, P, node ? tk.s : PP.sub_list[tk.b + i], scale,
                                                   Lx, CB, Linv, wsm);
                        }
                    }
                    if (w2 > q) __syncthreads();
                } else {
                    for (int i = q + warp; i < w1; i += 8)
                        fdag_warp_front<32, T>(D, I, PP, P, node ? tk.s : PP.sub_list[tk.b + i], scale, Lx,
                                               CB, Linv, smem_raw + (size_t)warp * WF32);
                    if (w1 > q) __syncthreads();
                    if (warp < NW64) {
                        for (int i = w1 + warp; i < w2; i += NW64)
                            fdag_warp_front<64, T>(D, I, PP, P, node ? tk.s : PP.sub_list[tk.b + i], scale,
                                                   Lx, CB, Linv, smem_raw + (size_t)warp * WF64);
                    }
                    if (w2 > w1) __syncthreads();
                }
                for (int i = w2; i < w3; i++) {
                    const int s = node ? tk.s : PP.sub_list[tk.b + i];
                    const int nscol = (int)(P.Super[s + 1] - P.Super[s]);
                    const int nsrow = (int)(P.Pi[s + 1] - P.Pi[s]);
                    const int m = nsrow - nscol;
                    {
                        // every column at once (each entry still set from A,
                        // then added to by the children in their order)
                        const gb_asm_task a = {s, 0, nsrow, 0};
                        if (D.a_dtype == 0)
                            assemble_body<double, T>(P, a, PP.Sp, PP.Si, (const double *)D.Sx + I.sx,
                                                     scale, D.beta, Lx, CB);
                        else
                            assemble_body<float, T>(P, a, PP.Sp, PP.Si, (const float *)D.Sx + I.sx,
                                                    scale, D.beta, Lx, CB);
                        __syncthreads();
                    }
                    factor_small_body<T>(P, s, Lx, Linv, smem_raw, &sfail);
                    __syncthreads();
                    for (int J = 0; J < m; J += 64)
                        for (int I0 = J; I0 < m; I0 += 64) {
                            const gb_dtask ct = {GB_DT_CB, s, 0, I0 / 64, J / 64, 1, 0, 0};
                            dag_tile_task<T>(P, ct, Lx, CB, Linv, smem_raw, sfail);
                            __syncthreads();
                        }
                }
                q = w3;
                wave++;
            }
        } else {
            if (tk.type == GB_DT_DIAG) {
                // the diagonal chain of panel tk.b: the panel solve of row
                // block b, then the updates that read it may start (early
                // successors) while this block updates tile (b, b) and
                // factors panel b
                const gb_dtask t1 = {GB_DT_TRSM, tk.s, tk.b - 1, tk.b, 0, 0, 0, 0};
                tile_body<T>(P, t1, Lx, CB, Linv, smem_raw, sfail, TC ? tc : nullptr,
                             TC ? D.img : nullptr);
                __syncthreads();
                fdag_release(D, PP, I, PP.succ_ptr[local], PP.succ_ptr[local] + tk.pad1, false,
                             &snext);
                if (!TC || !tc || tcx.ok) diag_update_potrf<T>(P, tk, Lx, Linv, smem_raw, sfail);
            } else {
                dag_tile_task<T>(P, tk, Lx, CB, Linv, smem_raw, sfail, TC ? tc : nullptr,
                                 TC ? D.img : nullptr);
            }
            if (TC && tc && !tcx.ok) {
                // a tensor-core wait gave up: stop the executor (every block
                // returns on the error word)
                if (threadIdx.x == 0) {
                    atomicExch(D.Q.ctrl + 5, 1);
                    atomicExch(D.Q.err, 1);
                }
                break;
            }
        }
        __syncthreads();
        // the successors not released early (a DIAG task released its
        // first tk.pad1 after its panel solve)
        if (D.trace && threadIdx.x == 0) D.trace[3 * (size_t)id + 1] = dag_timer();
        fdag_release(D, PP, I, PP.succ_ptr[local] + (tk.type == GB_DT_DIAG ? tk.pad1 : 0),
                     PP.succ_ptr[local + 1], spoll != 0, &snext);
    }
    if (TC && tc) {
        // (a tile product whose wait gave up has already waited, bounded,
        // for its copies and MMAs in flight)
        asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
        __syncthreads();
        if (threadIdx.x < 32)
            asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" :: "r"(tcx.taddr), "r"(GB_TC_COLS));
    }
}

extern "C" {

int gb_launch_fdag(const gb_fdag_args *a, void *Lx, void *CB, void *Linv, int dtype, int grid,
                   cudaStream_t st)
{
    if (a->ntotal <= 0) return 0;
    gb_fdag_dev D;
    D.Q.q0 = a->q0; D.Q.q1 = a->q1; D.Q.ctrl = a->ctrl; D.Q.err = a->err;
    D.Q.smflag = a->smflag; D.Q.epoch = a->epoch; D.Q.npoll = a->npoll;
    D.pats = a->pats; D.inst = a->inst; D.ibase = a->inst_base; D.ninst = a->ninst;
    D.cnt = a->cnt; D.trace = a->trace;
    D.Sx = a->Sx; D.a_dtype = a->a_dtype; D.scale = a->scale; D.beta = a->beta;
    D.use_tc = a->use_tc && a->img;
    D.img = a->img;
    static int configured = 0;
    if (!configured) {
        cudaFuncSetAttribute(k_fdag<double, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)fdag_smem<double>());
        cudaFuncSetAttribute(k_fdag<float, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)fdag_smem<float>());
        cudaFuncSetAttribute(k_fdag<float, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)fdag_smem<float>());
        // the whole shared-memory carveout, so that two blocks fit an SM
        cudaFuncSetAttribute(k_fdag<double, false>, cudaFuncAttributePreferredSharedMemoryCarveout,
                             (int)cudaSharedmemCarveoutMaxShared);
        cudaFuncSetAttribute(k_fdag<float, false>, cudaFuncAttributePreferredSharedMemoryCarveout,
                             (int)cudaSharedmemCarveoutMaxShared);
        cudaFuncSetAttribute(k_fdag<float, true>, cudaFuncAttributePreferredSharedMemoryCarveout,
                             (int)cudaSharedmemCarveoutMaxShared);
        configured = 1;
    }
    if (grid > a->ntotal + GB_DAG_POLLERS) grid = (int)(a->ntotal + GB_DAG_POLLERS);
    if (grid < GB_DAG_POLLERS + 1) grid = GB_DAG_POLLERS + 1;
    if (dtype == 0)
        k_fdag<double, false><<<grid, 256, fdag_smem<double>(), st>>>(D, (double *)Lx, (double *)CB, (double *)Linv);
    else if (D.use_tc)
        k_fdag<float, true><<<grid, 256, fdag_smem<float>(), st>>>(D, (float *)Lx, (float *)CB, (float *)Linv);
    else
        k_fdag<float, false><<<grid, 256, fdag_smem<float>(), st>>>(D, (float *)Lx, (float *)CB, (float *)Linv);
    return (int)cudaGetLastError();
}

int gb_launch_dag(const gb_pattern_ptrs *pp, const gb_dag_args *a, void *Lx, void *CB,
                  void *Linv, int dtype, int grid, cudaStream_t st)
{
    if (a->ntasks <= 0) return 0;
    gb_dev_pattern P = gb_to_dev(pp);
    gb_dag_dev D;
    D.tasks = a->tasks; D.ntasks = a->ntasks; D.succ_ptr = a->succ_ptr; D.succ = a->succ;
    D.cnt = a->cnt; D.trace = a->trace;
    D.Q.q0 = a->q0; D.Q.q1 = a->q1; D.Q.ctrl = a->ctrl; D.Q.err = a->err;
    D.Q.smflag = a->smflag; D.Q.epoch = a->epoch; D.Q.npoll = GB_DAG_POLLERS;
    static int configured = 0;
    if (!configured) {
        cudaFuncSetAttribute(k_dag<double>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)dag_smem<double>());
        cudaFuncSetAttribute(k_dag<float>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)dag_smem<float>());
        configured = 1;
    }
    /* the first GB_DAG_POLLERS blocks serve only the critical queue: keep
     * at least one bulk block, and no more bulk blocks than tasks */
    if (grid > a->ntasks + GB_DAG_POLLERS) grid = a->ntasks + GB_DAG_POLLERS;
    if (grid < GB_DAG_POLLERS + 1) grid = GB_DAG_POLLERS + 1;
    if (dtype == 0) k_dag<double><<<grid, 256, dag_smem<double>(), st>>>(P, D, (double *)Lx, (double *)CB, (double *)Linv);
    else k_dag<float><<<grid, 256, dag_smem<float>(), st>>>(P, D, (float *)Lx, (float *)CB, (float *)Linv);
    return (int)cudaGetLastError();
}

}  // extern "C"
