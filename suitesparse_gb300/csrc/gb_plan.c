/* gb_plan.c -- host construction of the per-pattern GPU plan (see gb_plan.h).
 *
 * Level schedule: level(s) = 0 for a leaf of the supernodal etree, else
 * 1 + max level of its children; all supernodes of one level are
 * independent.  Per level the factorization issues
 *     ASM   (assembly + extend-add of every supernode of the level)
 *     SMALL (one block per supernode at most small_cols wide)
 *     per block column b of the wide supernodes: POTRF, TRSM, GEMM (trailing)
 *     GEMM  (update blocks CB_s -= L21 L21' of every supernode of the level)
 * and the sweeps issue the matching node / block-step launches.
 */
#include "gb_plan.h"
#include <stdlib.h>
#include <string.h>

int gb_vec_push(gb_vec *v, const void *e)
{
    if (v->n == v->cap) {
        size_t cap = v->cap ? 2 * v->cap : 64;
        void *p = realloc(v->p, cap * v->esz);
        if (!p) return FALSE;
        v->p = p;
        v->cap = cap;
    }
    memcpy((char *)v->p + v->n * v->esz, e, v->esz);
    v->n++;
    return TRUE;
}

void gb_vec_free(gb_vec *v)
{
    free(v->p);
    v->p = NULL;
    v->n = v->cap = 0;
}

static void vec_init(gb_vec *v, size_t esz) { memset(v, 0, sizeof *v); v->esz = esz; }

static uint64_t mix64(uint64_t h, uint64_t x)
{
    h ^= x + 0x9E3779B97F4A7C15ull + (h << 6) + (h >> 2);
    h *= 0xBF58476D1CE4E5B9ull;
    return h ^ (h >> 31);
}

/* fingerprint of the supernodal pattern: all of super/pi, every 16th row
 * index of s, and the sizes */
uint64_t gb_pattern_hash(const cholmod_factor *L)
{
    uint64_t h = mix64(0, L->n);
    h = mix64(h, L->nsuper);
    h = mix64(h, L->ssize);
    h = mix64(h, L->xsize);
    const Int *Super = L->super, *Pi = L->pi, *Ls = L->s;
    for (size_t s = 0; s <= L->nsuper; s++) h = mix64(mix64(h, Super[s]), Pi[s]);
    size_t ns = (size_t)Pi[L->nsuper];
    for (size_t p = 0; p < ns; p += 16) h = mix64(h, Ls[p]);
    if (ns) h = mix64(h, Ls[ns - 1]);
    return h;
}

/* flops of a tile update that land in stored entries (2 per multiply-add) */
static double gemm_flops(const gb_gemm_task *g)
{
    double cnt = 0;
    if (g->flags & GB_GEMM_LOWER) {
        for (int c = 0; c < g->n; c++) {
            int r0 = c + g->diag_off;          /* first stored row of column c */
            if (r0 < 0) r0 = 0;
            if (r0 < g->m) cnt += g->m - r0;
        }
    } else {
        cnt = (double)g->m * g->n;
    }
    return 2.0 * cnt * g->k;
}

static int push_launch(gb_vec *seq, int kind, size_t count, size_t off)
{
    if (count == 0) return TRUE;
    gb_launch_rec r;
    r.kind = kind;
    r.count = (int32_t)count;
    r.off = (int64_t)off;
    return gb_vec_push(seq, &r);
}

gb_plan *gb_plan_build(const cholmod_factor *L, int64_t small_cols)
{
    if (small_cols < 1) small_cols = 1;
    if (small_cols > GB_SMALL_MAX) small_cols = GB_SMALL_MAX;
    Int n = (Int)L->n, nsuper = (Int)L->nsuper;
    const Int *Super = L->super, *Pi = L->pi, *Px = L->px, *Ls = L->s;
    if (n >= INT32_MAX || (Int)L->ssize >= INT32_MAX) return NULL;

    gb_plan *P = calloc(1, sizeof(gb_plan));
    if (!P) return NULL;
    P->L = L;
    P->super_ptr = L->super;
    P->s_ptr = L->s;
    P->pi_ptr = L->pi;
    P->n = n;
    P->nsuper = nsuper;
    P->ssize = (Int)L->ssize;
    P->xsize = (Int)L->xsize;
    P->hash = gb_pattern_hash(L);
    vec_init(&P->asm_t, sizeof(gb_asm_task));
    vec_init(&P->node_t, sizeof(gb_node_task));
    vec_init(&P->potrf_t, sizeof(gb_potrf_task));
    vec_init(&P->trsm_t, sizeof(gb_trsm_task));
    vec_init(&P->gemm_t, sizeof(gb_gemm_task));
    vec_init(&P->gemm_owner, sizeof(int32_t));
    vec_init(&P->sweep_t, sizeof(gb_sweep_task));
    vec_init(&P->fact_seq, sizeof(gb_launch_rec));
    vec_init(&P->fwd_seq, sizeof(gb_launch_rec));
    vec_init(&P->bwd_seq, sizeof(gb_launch_rec));

    Int *SuperMap = malloc(sizeof(Int) * (n + 1));
    Int *parent = malloc(sizeof(Int) * (nsuper + 1));
    Int *level = malloc(sizeof(Int) * (nsuper + 1));
    int32_t *child_ptr = calloc(nsuper + 2, sizeof(int32_t));
    int32_t *child_list = malloc(sizeof(int32_t) * (nsuper + 1));
    int32_t *relmap = malloc(sizeof(int32_t) * (L->ssize + 1));
    Int *Map = malloc(sizeof(Int) * (n + 1));
    int64_t *cboff = malloc(sizeof(int64_t) * (nsuper + 1));
    int64_t *cbvoff = malloc(sizeof(int64_t) * (nsuper + 1));
    Int *lev_ptr = NULL, *lev_list = NULL;
    int ok = SuperMap && parent && level && child_ptr && child_list && relmap && Map
             && cboff && cbvoff;
    if (!ok) goto fail;

    for (Int s = 0; s < nsuper; s++)
        for (Int k = Super[s]; k < Super[s + 1]; k++) SuperMap[k] = s;
    for (Int s = 0; s < nsuper; s++) {
        Int nscol = Super[s + 1] - Super[s], nsrow = Pi[s + 1] - Pi[s];
        parent[s] = (nsrow > nscol) ? SuperMap[Ls[Pi[s] + nscol]] : EMPTY;
        if (parent[s] != EMPTY) child_ptr[parent[s] + 1]++;
    }
    for (Int s = 0; s < nsuper; s++) child_ptr[s + 1] += child_ptr[s];
    {
        int32_t *w = malloc(sizeof(int32_t) * (nsuper + 1));
        if (!w) goto fail;
        memcpy(w, child_ptr, sizeof(int32_t) * (nsuper + 1));
        for (Int s = 0; s < nsuper; s++)       /* children in increasing order */
            if (parent[s] != EMPTY) child_list[w[parent[s]]++] = (int32_t)s;
        free(w);
    }

    /* levels (children have smaller indices: one ascending pass) */
    int nlevels = 0;
    for (Int s = 0; s < nsuper; s++) {
        Int lv = 0;
        for (int32_t q = child_ptr[s]; q < child_ptr[s + 1]; q++)
            lv = GB_MAX(lv, level[child_list[q]] + 1);
        level[s] = lv;
        nlevels = (int)GB_MAX(nlevels, lv + 1);
    }
    P->nlevels = nlevels;
    lev_ptr = calloc(nlevels + 2, sizeof(Int));
    lev_list = malloc(sizeof(Int) * (nsuper + 1));
    if (!lev_ptr || !lev_list) goto fail;
    for (Int s = 0; s < nsuper; s++) lev_ptr[level[s] + 1]++;
    for (int l = 0; l < nlevels; l++) lev_ptr[l + 1] += lev_ptr[l];
    {
        Int *w = malloc(sizeof(Int) * (nlevels + 1));
        if (!w) goto fail;
        memcpy(w, lev_ptr, sizeof(Int) * (nlevels + 1));
        for (Int s = 0; s < nsuper; s++) lev_list[w[level[s]]++] = s;
        free(w);
    }

    /* relative map of each child's off-diagonal rows into its parent */
    for (Int i = 0; i < n; i++) Map[i] = EMPTY;
    for (Int i = 0; i < (Int)L->ssize; i++) relmap[i] = -1;
    for (Int p = 0; p < nsuper; p++) {
        for (Int q = Pi[p]; q < Pi[p + 1]; q++) Map[Ls[q]] = q - Pi[p];
        for (int32_t cq = child_ptr[p]; cq < child_ptr[p + 1]; cq++) {
            Int c = child_list[cq];
            Int ncc = Super[c + 1] - Super[c];
            for (Int q = Pi[c] + ncc; q < Pi[c + 1]; q++) relmap[q] = (int32_t)Map[Ls[q]];
        }
    }

    /* update block / vector offsets */
    int64_t cbt = 0, cbvt = 0;
    for (Int s = 0; s < nsuper; s++) {
        int64_t m = (Pi[s + 1] - Pi[s]) - (Super[s + 1] - Super[s]);
        cboff[s] = cbt;
        cbvoff[s] = cbvt;
        cbt += m * m;
        cbvt += m;
    }
    cboff[nsuper] = cbt;
    cbvoff[nsuper] = cbvt;
    P->cb_total = cbt;
    P->cbv_total = cbvt;

    /* ---- factorization sequence ---- */
    const int T = GB_TILE, NB = GB_NB;
    for (int l = 0; l < nlevels && ok; l++) {
        size_t a0 = P->asm_t.n;
        int maxsteps = 0;
        for (Int q = lev_ptr[l]; q < lev_ptr[l + 1]; q++) {
            Int s = lev_list[q];
            Int nsrow = Pi[s + 1] - Pi[s];
            /* assembly tasks: chunks of 64 front columns */
            for (Int t0 = 0; t0 < nsrow; t0 += 64) {
                gb_asm_task a = {(int32_t)s, (int32_t)t0, (int32_t)GB_MIN(t0 + 64, nsrow), 0};
                ok &= gb_vec_push(&P->asm_t, &a);
            }
            Int nscol = Super[s + 1] - Super[s];
            if (nscol > small_cols) maxsteps = (int)GB_MAX(maxsteps, (nscol + NB - 1) / NB);
        }
        ok &= push_launch(&P->fact_seq, GB_K_ASM, P->asm_t.n - a0, a0);
        size_t n0 = P->node_t.n;
        for (Int q = lev_ptr[l]; q < lev_ptr[l + 1]; q++) {
            Int s = lev_list[q];
            if (Super[s + 1] - Super[s] <= small_cols) {
                gb_node_task t = {(int32_t)s, 0};
                ok &= gb_vec_push(&P->node_t, &t);
            }
        }
        ok &= push_launch(&P->fact_seq, GB_K_SMALL, P->node_t.n - n0, n0);
        for (int b = 0; b < maxsteps && ok; b++) {
            size_t p0 = P->potrf_t.n, r0 = P->trsm_t.n, g0 = P->gemm_t.n;
            for (Int q = lev_ptr[l]; q < lev_ptr[l + 1]; q++) {
                Int s = lev_list[q];
                Int nscol = Super[s + 1] - Super[s], nsrow = Pi[s + 1] - Pi[s];
                if (nscol <= small_cols) continue;
                Int c0 = (Int)b * NB;
                if (c0 >= nscol) continue;
                Int nb = GB_MIN(NB, nscol - c0);
                gb_potrf_task pt = {(int32_t)s, (int32_t)c0, (int32_t)nb, 0};
                ok &= gb_vec_push(&P->potrf_t, &pt);
                for (Int r = c0 + nb; r < nsrow; r += GB_TRSM_ROWS) {
                    gb_trsm_task tt = {(int32_t)s, (int32_t)c0, (int32_t)nb, (int32_t)r,
                                       (int32_t)GB_MIN(GB_TRSM_ROWS, nsrow - r), 0, 0, 0};
                    ok &= gb_vec_push(&P->trsm_t, &tt);
                }
            }
            ok &= push_launch(&P->fact_seq, GB_K_POTRF, P->potrf_t.n - p0, p0);
            ok &= push_launch(&P->fact_seq, GB_K_TRSM, P->trsm_t.n - r0, r0);
            for (Int q = lev_ptr[l]; q < lev_ptr[l + 1]; q++) {
                Int s = lev_list[q];
                Int nscol = Super[s + 1] - Super[s], nsrow = Pi[s + 1] - Pi[s];
                if (nscol <= small_cols) continue;
                Int c0 = (Int)b * NB;
                if (c0 >= nscol) continue;
                Int nb = GB_MIN(NB, nscol - c0);
                Int t0 = c0 + nb;   /* trailing columns [t0, nscol), rows [t0, nsrow) */
                for (Int cs = t0; cs < nscol; cs += T) {
                    Int nc = GB_MIN(T, nscol - cs);
                    for (Int rs = cs; rs < nsrow; rs += T) {
                        /* rows of this tile that can be >= its columns */
                        Int nr = GB_MIN(T, nsrow - rs);
                        gb_gemm_task g;
                        memset(&g, 0, sizeof g);
                        g.a = Px[s] + rs + c0 * nsrow;
                        g.b = Px[s] + cs + c0 * nsrow;
                        g.c = Px[s] + rs + cs * nsrow;
                        g.lda = g.ldb = g.ldc = (int32_t)nsrow;
                        g.m = (int32_t)nr;
                        g.n = (int32_t)nc;
                        g.k = (int32_t)nb;
                        if (rs < cs + nc - 1) {        /* crosses the diagonal */
                            g.flags = GB_GEMM_LOWER;
                            g.diag_off = (int32_t)(cs - rs);
                        }
                        int32_t own = (int32_t)s;
                        ok &= gb_vec_push(&P->gemm_t, &g);
                        ok &= gb_vec_push(&P->gemm_owner, &own);
                        P->fl_gemm += gemm_flops(&g);
                    }
                }
            }
            ok &= push_launch(&P->fact_seq, GB_K_GEMM, P->gemm_t.n - g0, g0);
        }
        /* update blocks of the level */
        size_t g0 = P->gemm_t.n;
        for (Int q = lev_ptr[l]; q < lev_ptr[l + 1]; q++) {
            Int s = lev_list[q];
            Int nscol = Super[s + 1] - Super[s], nsrow = Pi[s + 1] - Pi[s];
            Int m = nsrow - nscol;
            for (Int J = 0; J < m; J += T) {
                for (Int I = J; I < m; I += T) {
                    gb_gemm_task g;
                    memset(&g, 0, sizeof g);
                    g.a = Px[s] + nscol + I;
                    g.b = Px[s] + nscol + J;
                    g.c = cboff[s] + I + J * m;
                    g.lda = g.ldb = (int32_t)nsrow;
                    g.ldc = (int32_t)m;
                    g.m = (int32_t)GB_MIN(T, m - I);
                    g.n = (int32_t)GB_MIN(T, m - J);
                    g.k = (int32_t)nscol;
                    g.flags = GB_GEMM_C_IN_CB | (I == J ? GB_GEMM_LOWER : 0);
                    g.diag_off = 0;
                    int32_t own = (int32_t)s;
                    ok &= gb_vec_push(&P->gemm_t, &g);
                    ok &= gb_vec_push(&P->gemm_owner, &own);
                    P->fl_gemm += gemm_flops(&g);
                }
            }
        }
        ok &= push_launch(&P->fact_seq, GB_K_GEMM, P->gemm_t.n - g0, g0);
    }

    /* ---- forward sweep sequence ---- */
    for (int l = 0; l < nlevels && ok; l++) {
        size_t n0 = P->node_t.n;
        int maxsteps = 0;
        for (Int q = lev_ptr[l]; q < lev_ptr[l + 1]; q++) {
            Int s = lev_list[q];
            Int nscol = Super[s + 1] - Super[s];
            if (nscol <= small_cols) {
                gb_node_task t = {(int32_t)s, 0};
                ok &= gb_vec_push(&P->node_t, &t);
            } else {
                maxsteps = (int)GB_MAX(maxsteps, (nscol + NB - 1) / NB);
            }
        }
        ok &= push_launch(&P->fwd_seq, GB_K_FWD_SMALL, P->node_t.n - n0, n0);
        n0 = P->node_t.n;
        for (Int q = lev_ptr[l]; q < lev_ptr[l + 1]; q++) {
            Int s = lev_list[q];
            if (Super[s + 1] - Super[s] > small_cols) {
                gb_node_task t = {(int32_t)s, 0};
                ok &= gb_vec_push(&P->node_t, &t);
            }
        }
        ok &= push_launch(&P->fwd_seq, GB_K_FWD_GATHER, P->node_t.n - n0, n0);
        for (int b = 0; b < maxsteps && ok; b++) {
            size_t d0 = P->sweep_t.n;
            for (Int q = lev_ptr[l]; q < lev_ptr[l + 1]; q++) {
                Int s = lev_list[q];
                Int nscol = Super[s + 1] - Super[s];
                Int c0 = (Int)b * NB;
                if (nscol <= small_cols || c0 >= nscol) continue;
                gb_sweep_task t = {(int32_t)s, (int32_t)c0, (int32_t)GB_MIN(NB, nscol - c0), 0, 0, 0, 0, 0};
                ok &= gb_vec_push(&P->sweep_t, &t);
            }
            ok &= push_launch(&P->fwd_seq, GB_K_FWD_DIAG, P->sweep_t.n - d0, d0);
            d0 = P->sweep_t.n;
            for (Int q = lev_ptr[l]; q < lev_ptr[l + 1]; q++) {
                Int s = lev_list[q];
                Int nscol = Super[s + 1] - Super[s], nsrow = Pi[s + 1] - Pi[s];
                Int c0 = (Int)b * NB;
                if (nscol <= small_cols || c0 >= nscol) continue;
                Int nb = GB_MIN(NB, nscol - c0);
                for (Int r = c0 + nb; r < nsrow; r += 128) {
                    gb_sweep_task t = {(int32_t)s, (int32_t)c0, (int32_t)nb, (int32_t)r,
                                       (int32_t)GB_MIN(128, nsrow - r), 0, 0, 0};
                    ok &= gb_vec_push(&P->sweep_t, &t);
                }
            }
            ok &= push_launch(&P->fwd_seq, GB_K_FWD_PANEL, P->sweep_t.n - d0, d0);
        }
    }

    /* ---- backward sweep sequence ---- */
    for (int l = nlevels - 1; l >= 0 && ok; l--) {
        size_t n0 = P->node_t.n;
        int maxsteps = 0;
        for (Int q = lev_ptr[l]; q < lev_ptr[l + 1]; q++) {
            Int s = lev_list[q];
            Int nscol = Super[s + 1] - Super[s];
            if (nscol <= small_cols) {
                gb_node_task t = {(int32_t)s, 0};
                ok &= gb_vec_push(&P->node_t, &t);
            } else {
                maxsteps = (int)GB_MAX(maxsteps, (nscol + NB - 1) / NB);
            }
        }
        ok &= push_launch(&P->bwd_seq, GB_K_BWD_SMALL, P->node_t.n - n0, n0);
        size_t d0 = P->sweep_t.n;
        for (Int q = lev_ptr[l]; q < lev_ptr[l + 1]; q++) {
            Int s = lev_list[q];
            Int nscol = Super[s + 1] - Super[s], nsrow = Pi[s + 1] - Pi[s];
            if (nscol <= small_cols || nsrow == nscol) continue;
            for (Int j = 0; j < nscol; j += 32) {
                gb_sweep_task t = {(int32_t)s, 0, 0, (int32_t)j, (int32_t)GB_MIN(32, nscol - j), 0, 0, 0};
                ok &= gb_vec_push(&P->sweep_t, &t);
            }
        }
        ok &= push_launch(&P->bwd_seq, GB_K_BWD_OFFDIAG, P->sweep_t.n - d0, d0);
        for (int b = maxsteps - 1; b >= 0 && ok; b--) {
            d0 = P->sweep_t.n;
            for (Int q = lev_ptr[l]; q < lev_ptr[l + 1]; q++) {
                Int s = lev_list[q];
                Int nscol = Super[s + 1] - Super[s];
                if (nscol <= small_cols) continue;
                Int nblk = (nscol + NB - 1) / NB;
                /* align each supernode's last block with the last step */
                Int bb = b - (maxsteps - nblk);
                if (bb < 0) continue;
                Int c0 = bb * NB;
                gb_sweep_task t = {(int32_t)s, (int32_t)c0, (int32_t)GB_MIN(NB, nscol - c0), 0, 0, 0, 0, 0};
                ok &= gb_vec_push(&P->sweep_t, &t);
            }
            ok &= push_launch(&P->bwd_seq, GB_K_BWD_DIAG, P->sweep_t.n - d0, d0);
            d0 = P->sweep_t.n;
            for (Int q = lev_ptr[l]; q < lev_ptr[l + 1]; q++) {
                Int s = lev_list[q];
                Int nscol = Super[s + 1] - Super[s];
                if (nscol <= small_cols) continue;
                Int nblk = (nscol + NB - 1) / NB;
                Int bb = b - (maxsteps - nblk);
                if (bb <= 0) continue;
                Int c0 = bb * NB;
                for (Int j = 0; j < c0; j += 32) {
                    gb_sweep_task t = {(int32_t)s, (int32_t)c0, (int32_t)GB_MIN(NB, nscol - c0),
                                       (int32_t)j, (int32_t)GB_MIN(32, c0 - j), 0, 0, 0};
                    ok &= gb_vec_push(&P->sweep_t, &t);
                }
            }
            ok &= push_launch(&P->bwd_seq, GB_K_BWD_PANEL, P->sweep_t.n - d0, d0);
        }
    }
    if (!ok) goto fail;

    P->h_child_ptr = child_ptr;
    P->h_child_list = child_list;
    P->h_relmap = relmap;
    P->h_cboff = cboff;
    P->h_cbvoff = cbvoff;
    free(SuperMap); free(parent); free(level); free(Map); free(lev_ptr); free(lev_list);
    return P;

fail:
    free(SuperMap); free(parent); free(level); free(Map); free(lev_ptr); free(lev_list);
    P->h_child_ptr = child_ptr;
    P->h_child_list = child_list;
    P->h_relmap = relmap;
    P->h_cboff = cboff;
    P->h_cbvoff = cbvoff;
    gb_plan_free(P);
    return NULL;
}

#define UP(dst, src, bytes)                                                    \
    do {                                                                       \
        size_t b_ = (bytes) ? (bytes) : 16;                                    \
        if (cudaMalloc((void **)&(dst), b_) != cudaSuccess) goto fail;         \
        if ((bytes) && cudaMemcpy((dst), (src), (bytes), cudaMemcpyHostToDevice) != cudaSuccess) goto fail; \
    } while (0)

int gb_plan_upload(gb_plan *P)
{
    const cholmod_factor *L = P->L;
    int32_t *child_ptr = P->h_child_ptr, *child_list = P->h_child_list, *relmap = P->h_relmap;
    int64_t *cboff = P->h_cboff, *cbvoff = P->h_cbvoff;
    Int ns = P->nsuper, n = P->n, ssz = P->ssize;
    int32_t *Ls32 = malloc(sizeof(int32_t) * (ssz + 1));
    int ok = FALSE;
    if (!Ls32) goto fail;
    const Int *Ls = L->s;
    for (Int i = 0; i < ssz; i++) Ls32[i] = (int32_t)Ls[i];
    UP(P->d_Super, L->super, sizeof(int64_t) * (ns + 1));
    UP(P->d_Pi, L->pi, sizeof(int64_t) * (ns + 1));
    UP(P->d_Px, L->px, sizeof(int64_t) * (ns + 1));
    UP(P->d_cboff, cboff, sizeof(int64_t) * (ns + 1));
    UP(P->d_cbvoff, cbvoff, sizeof(int64_t) * (ns + 1));
    UP(P->d_Perm, L->Perm, sizeof(int64_t) * n);
    UP(P->d_Ls, Ls32, sizeof(int32_t) * ssz);
    UP(P->d_relmap, relmap, sizeof(int32_t) * ssz);
    UP(P->d_child_ptr, child_ptr, sizeof(int32_t) * (ns + 1));
    UP(P->d_child_list, child_list, sizeof(int32_t) * ns);
    if (cudaMalloc((void **)&P->d_fail, sizeof(int32_t) * (ns + 1)) != cudaSuccess) goto fail;
    if (cudaMalloc((void **)&P->d_anyfail, sizeof(int32_t) * 4) != cudaSuccess) goto fail;
    UP(P->d_asm, P->asm_t.p, P->asm_t.n * P->asm_t.esz);
    UP(P->d_node, P->node_t.p, P->node_t.n * P->node_t.esz);
    UP(P->d_potrf, P->potrf_t.p, P->potrf_t.n * P->potrf_t.esz);
    UP(P->d_trsm, P->trsm_t.p, P->trsm_t.n * P->trsm_t.esz);
    UP(P->d_gemm, P->gemm_t.p, P->gemm_t.n * P->gemm_t.esz);
    UP(P->d_gemm_owner, P->gemm_owner.p, P->gemm_owner.n * P->gemm_owner.esz);
    UP(P->d_sweep, P->sweep_t.p, P->sweep_t.n * P->sweep_t.esz);
    P->ptrs.Super = P->d_Super;
    P->ptrs.Pi = P->d_Pi;
    P->ptrs.Px = P->d_Px;
    P->ptrs.cboff = P->d_cboff;
    P->ptrs.cbvoff = P->d_cbvoff;
    P->ptrs.Ls = P->d_Ls;
    P->ptrs.relmap = P->d_relmap;
    P->ptrs.child_ptr = P->d_child_ptr;
    P->ptrs.child_list = P->d_child_list;
    P->ptrs.fail = P->d_fail;
    P->ptrs.anyfail = P->d_anyfail;
    ok = TRUE;
fail:
    free(Ls32);
    return ok;
}

void gb_plan_free(gb_plan *P)
{
    if (!P) return;
    free(P->h_child_ptr); free(P->h_child_list); free(P->h_relmap);
    free(P->h_cboff); free(P->h_cbvoff);
    void *dev[] = {P->d_Super, P->d_Pi, P->d_Px, P->d_cboff, P->d_cbvoff, P->d_Perm,
                   P->d_Ls, P->d_relmap, P->d_child_ptr, P->d_child_list, P->d_fail,
                   P->d_anyfail, P->d_asm, P->d_node, P->d_potrf, P->d_trsm, P->d_gemm,
                   P->d_gemm_owner, P->d_sweep, P->d_Lx[0], P->d_Lx[1], P->d_CB[0],
                   P->d_CB[1], P->d_Sp, P->d_Si, P->d_Sx, P->d_Y, P->d_U, P->d_B,
                   P->d_Rp, P->d_Rj, P->d_Rx, P->d_scale, P->d_scale_perm, P->d_X, P->d_R,
                   P->d_bx, P->d_red};
    for (size_t i = 0; i < sizeof dev / sizeof dev[0]; i++)
        if (dev[i]) cudaFree(dev[i]);
    gb_vec_free(&P->asm_t); gb_vec_free(&P->node_t); gb_vec_free(&P->potrf_t);
    gb_vec_free(&P->trsm_t); gb_vec_free(&P->gemm_t); gb_vec_free(&P->gemm_owner);
    gb_vec_free(&P->sweep_t); gb_vec_free(&P->fact_seq); gb_vec_free(&P->fwd_seq);
    gb_vec_free(&P->bwd_seq);
    free(P);
}
