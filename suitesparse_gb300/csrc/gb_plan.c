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

/* A fingerprint of L's supernodal pattern, checked on every use of the plan
 * (with the sizes and array addresses): the sizes, every supernode's
 * boundaries and row count at up to 4096 evenly spaced supernodes, and up to
 * 4096 evenly spaced row indices, so that its cost does not grow with the
 * factor (a batch of 4096 systems has 1.7M supernodes).  A caller that
 * rewrites L's pattern arrays in place must release the factor's GPU state
 * (gb300_release_factor) first. */
uint64_t gb_pattern_hash(const cholmod_factor *L)
{
    uint64_t h = mix64(0, L->n);
    h = mix64(h, L->nsuper);
    h = mix64(h, L->ssize);
    h = mix64(h, L->xsize);
    const Int *Super = L->super, *Pi = L->pi, *Ls = L->s;
    const size_t ss = L->nsuper / 4096 + 1;
    for (size_t s = 0; s <= L->nsuper; s += ss) h = mix64(mix64(h, Super[s]), Pi[s]);
    h = mix64(mix64(h, Super[L->nsuper]), Pi[L->nsuper]);
    size_t ns = (size_t)Pi[L->nsuper];
    const size_t sp = ns / 4096 + 1;
    for (size_t p = 0; p < ns; p += sp) h = mix64(h, Ls[p]);
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

/* Whole-factorization task graph from the per-level graphs: local ids
 * [0, ndag) are the level-graph tasks (same order), then the assembly
 * chunks, the small supernodes, JA(s) (s assembled) and JK(s) (the update
 * blocks of all children of s are complete).  Edges: the level graphs' own;
 * ASM(s, *) -> JA(s) -> SMALL(s) or POTRF(s, block 0); SMALL(s) -> CB(s, *);
 * CB(c, *) -> JK(parent c) -> ASM(parent c, *) (a leaf's JK has no edges).
 * Joins carry no work and are never queued.  Every task of s follows
 * JA(s), so the front is assembled before any tile task touches it, and the
 * parent's assembly follows every update-block tile of every child. */
static void gb_order_succ(const gb_dtask *tasks, int32_t early, int32_t *succ, int32_t lo,
                          int32_t hi, int32_t *tmp);

typedef struct { double w; int32_t id; } gb_ready_est;

/* descending work, then ascending task id (a deterministic order) */
static int ready_est_cmp(const void *a, const void *b)
{
    const gb_ready_est *x = a, *y = b;
    if (x->w != y->w) return x->w > y->w ? -1 : 1;
    return (x->id > y->id) - (x->id < y->id);
}

static int fdag_build(gb_plan *P)
{
    const int64_t ns = P->nsuper;
    const size_t ndag = P->dag_t.n, nasm = P->asm_t.n;
    const gb_dtask *dt = P->dag_t.p;
    const gb_asm_task *at = P->asm_t.p;
    const gb_node_task *nt = P->node_t.p;
    const gb_launch_rec *seq = P->fact_seq.p;
    size_t nsmall = 0;
    for (size_t i = 0; i < P->fact_seq.n; i++)
        if (seq[i].kind == GB_K_SMALL) nsmall += (size_t)seq[i].count;
    const size_t A0 = ndag, S0 = A0 + nasm, JA0 = S0 + nsmall, JK0 = JA0 + (size_t)ns;
    const size_t SB0 = JK0 + (size_t)ns;
    const int64_t *Pi = P->L->pi, *Sup = P->L->super;
    int ok = 1;
    /* Subtrees of small supernodes run whole as one SUBTREE task: every
     * supernode of the subtree at most small_cols wide and the estimated
     * work (nscol nsrow^2 per supernode plus a fixed cost) at most
     * GB_SUBTREE_WORK; the largest such subtrees are taken.  Their members'
     * own tasks stay in the list as inert joins without edges. */
    int32_t *sub_root = malloc(sizeof(int32_t) * (ns + 1));
    double *work = calloc(ns + 1, sizeof(double));
    char *elig = malloc(ns + 1);
    size_t nsub = 0;
    if (!sub_root || !work || !elig) ok = 0;
    for (int64_t s = 0; ok && s < ns; s++) elig[s] = 1;
    for (int64_t s = 0; ok && s < ns; s++) {          /* children before parents */
        double nscol = (double)(Sup[s + 1] - Sup[s]), nsrow = (double)(Pi[s + 1] - Pi[s]);
        work[s] += nscol * nsrow * nsrow + 1.0e4;
        if (Sup[s + 1] - Sup[s] > P->small_cols) elig[s] = 0;
        int32_t par = P->h_parent[s];
        if (par >= 0) {
            work[par] += work[s];
            if (!elig[s]) elig[par] = 0;
        }
    }
    /* work of each elimination tree (at its root): a forest in which no
     * tree holds 5 % of the work (a batch of independent systems) has no
     * long critical chain to keep blocks waiting for */
    {
        double wtot = 0, wmax = 0;
        for (int64_t s = 0; ok && s < ns; s++)
            if (P->h_parent[s] < 0) {
                wtot += work[s];
                if (work[s] > wmax) wmax = work[s];
            }
        P->fd_spread = ok && wmax < 0.05 * wtot;
    }
#define SUB_OK(s) (elig[s] && work[s] <= P->sub_work)
    for (int64_t s = ns - 1; ok && s >= 0; s--) {      /* parents before children */
        int32_t par = P->h_parent[s];
        if (SUB_OK(s) && !(par >= 0 && SUB_OK(par))) { sub_root[s] = (int32_t)s; nsub++; }
        else sub_root[s] = (par >= 0 && SUB_OK(s)) ? sub_root[par] : -1;
    }
#undef SUB_OK
    int32_t *sub_off = ok ? calloc(ns + 2, sizeof(int32_t)) : NULL;
    if (!sub_off) ok = 0;
    for (int64_t s = 0; ok && s < ns; s++)
        if (sub_root[s] >= 0) sub_off[sub_root[s] + 1]++;
    for (int64_t s = 0; ok && s < ns; s++) sub_off[s + 1] += sub_off[s];
    if (ok) {
        /* members wave by wave: wave h holds the members of height h in the
         * subtree (leaves 0), so every member's children are in earlier
         * waves; within a wave the fronts of at most 32 rows come first
         * (one warp each, eight at a time), then those of at most warp_rows
         * rows (one warp each, 64-row regions), then the others (the whole
         * block each), each group in ascending order.  key = 3 height +
         * group. */
        int32_t *fill = malloc(sizeof(int32_t) * (ns + 1)), *lst = malloc(sizeof(int32_t) * (ns + 1));
        int32_t *key = malloc(sizeof(int32_t) * (ns + 1)), *meta = calloc(3 * (size_t)ns + 3, sizeof(int32_t));
        if (!fill || !lst || !key || !meta) ok = 0;
        for (int64_t s = 0; ok && s < ns; s++) key[s] = 0;
        for (int64_t s = 0; ok && s < ns; s++) {       /* children before parents */
            if (sub_root[s] < 0) continue;
            int32_t par = P->h_parent[s];
            if (par >= 0 && sub_root[par] == sub_root[s] && key[par] < key[s] + 3)
                key[par] = key[s] + 3;
        }
        const Int tiny = GB_MIN(P->warp_rows, 32);
        for (int64_t s = 0; ok && s < ns; s++) {
            if (sub_root[s] < 0) continue;
            const Int nr = Pi[s + 1] - Pi[s];
            key[s] += nr <= tiny ? 0 : (nr <= P->warp_rows ? 1 : 2);
        }
        /* counting sort of each subtree's members by key (stable) */
        int32_t maxkey = 0;
        for (int64_t s = 0; ok && s < ns; s++)
            if (sub_root[s] >= 0 && key[s] > maxkey) maxkey = key[s];
        int32_t *kcnt = ok ? calloc((size_t)maxkey + 4, sizeof(int32_t)) : NULL;
        if (!kcnt) ok = 0;
        for (int64_t s = 0; ok && s < ns; s++) fill[s] = 0;
        for (int64_t s = 0; ok && s < ns; s++)          /* members in ascending order */
            if (sub_root[s] >= 0) lst[sub_off[sub_root[s]] + fill[sub_root[s]]++] = (int32_t)s;
        for (int64_t r = 0; ok && r < ns; r++) {
            if (sub_root[r] != r) continue;
            const int32_t b = sub_off[r], e = sub_off[r + 1];
            int32_t kmax = 0;
            for (int32_t q = b; q < e; q++) if (key[lst[q]] > kmax) kmax = key[lst[q]];
            const int32_t kend = 3 * (kmax / 3) + 3;      /* keys 0 .. kend-1 */
            for (int32_t k = 0; k <= kend; k++) kcnt[k] = 0;
            for (int32_t q = b; q < e; q++) kcnt[key[lst[q]] + 1]++;
            for (int32_t k = 0; k < kend; k++) kcnt[k + 1] += kcnt[k];
            /* wave starts: per wave (keys 3h, 3h+1, 3h+2) the ends of its
             * three groups, relative to b */
            for (int32_t h = 0; 3 * h < kend; h++) {
                const int32_t w0 = kcnt[3 * h], w1 = kcnt[3 * h + 1], w2 = kcnt[3 * h + 2],
                              w3 = kcnt[3 * h + 3];
                if (w3 > w0) {
                    meta[3 * (size_t)(b + w0)] = w1;
                    meta[3 * (size_t)(b + w0) + 1] = w2;
                    meta[3 * (size_t)(b + w0) + 2] = w3;
                }
            }
            for (int32_t q = b; q < e; q++) {
                const int32_t s = lst[q];
                fill[s] = b + kcnt[key[s]]++;
            }
        }
        for (int64_t s = 0; ok && s < ns; s++)
            if (sub_root[s] >= 0) key[fill[s]] = (int32_t)s;
        for (int64_t q = 0; ok && q < sub_off[ns]; q++) {
            ok &= gb_vec_push(&P->fd_sub, &key[q]);
            for (int u = 0; u < 3; u++) ok &= gb_vec_push(&P->fd_smeta, &meta[3 * q + u]);
        }
        free(kcnt);
        free(fill);
        free(lst);
        free(key);
        free(meta);
    }
#define MEMBER(s) (sub_root[s] >= 0)
    const size_t N = SB0 + nsub;
    if (N >= (size_t)1 << 30) ok = 0;
    int32_t *potrf0 = malloc(sizeof(int32_t) * (ns + 1));
    int32_t *small_id = malloc(sizeof(int32_t) * (ns + 1));
    int32_t *cbp = calloc(ns + 2, sizeof(int32_t));
    int32_t *cbl = malloc(sizeof(int32_t) * (ndag + 1));
    int32_t *deg = NULL, *nd = NULL, *pos = NULL, *succ = NULL, *tmp = NULL;
    gb_vec E;
    vec_init(&E, 2 * sizeof(int32_t));
    if (!potrf0 || !small_id || !cbp || !cbl) ok = 0;
    for (int64_t s = 0; ok && s < ns; s++) potrf0[s] = small_id[s] = -1;
    /* small supernodes with few rows run whole as one NODE task: their
     * assembly chunks and update-block tiles stay in the list as inert
     * joins without edges */
#define FUSED(s) (MEMBER(s) || (Sup[(s) + 1] - Sup[s] <= P->small_cols && Pi[(s) + 1] - Pi[s] <= GB_NODE_MAX_ROWS))
    /* tasks */
    for (size_t i = 0; ok && i < ndag; i++) {
        gb_dtask t = dt[i];
        if (t.type == GB_DT_POTRF && t.b == 0) potrf0[t.s] = (int32_t)i;
        if (t.type == GB_DT_CB) {
            if (FUSED(t.s)) t.type = GB_DT_JOIN;
            else cbp[t.s + 2]++;
        }
        ok &= gb_vec_push(&P->fd_t, &t);
    }
    for (size_t i = 0; ok && i < nasm; i++) {
        gb_dtask t = {FUSED(at[i].s) ? GB_DT_JOIN : GB_DT_ASM, at[i].s, at[i].t0, at[i].t1, 0, 1, 0, 0};
        ok &= gb_vec_push(&P->fd_t, &t);
    }
    {
        size_t k = 0;
        for (size_t i = 0; ok && i < P->fact_seq.n; i++) {
            if (seq[i].kind != GB_K_SMALL) continue;
            for (int32_t q = 0; ok && q < seq[i].count; q++) {
                int32_t s = nt[seq[i].off + q].s;
                gb_dtask t = {MEMBER(s) ? GB_DT_JOIN : FUSED(s) ? GB_DT_NODE : GB_DT_SMALL, s, 0, 0, 0, 1, 0, 0};
                small_id[s] = (int32_t)(S0 + k++);
                ok &= gb_vec_push(&P->fd_t, &t);
            }
        }
    }
    for (int w = 0; w < 2 && ok; w++)
        for (int64_t s = 0; ok && s < ns; s++) {
            gb_dtask t = {GB_DT_JOIN, (int32_t)s, w, 0, 0, 0, 0, 0};
            ok &= gb_vec_push(&P->fd_t, &t);
        }
    int32_t *sub_id = ok ? malloc(sizeof(int32_t) * (ns + 1)) : NULL;
    if (!sub_id) ok = 0;
    for (int64_t s = 0, k = 0; ok && s < ns; s++) {
        sub_id[s] = -1;
        if (sub_root[s] != s) continue;
        gb_dtask t = {GB_DT_SUBTREE, (int32_t)s, sub_off[s], sub_off[s + 1] - sub_off[s], 0, 1, 0, 0};
        sub_id[s] = (int32_t)(SB0 + k++);
        ok &= gb_vec_push(&P->fd_t, &t);
    }
    /* update-block tiles of each supernode (CSR by supernode) */
    for (int64_t s = 0; ok && s < ns; s++) cbp[s + 2] += cbp[s + 1];
    for (size_t i = 0; ok && i < ndag; i++)
        if (dt[i].type == GB_DT_CB && !FUSED(dt[i].s)) cbl[cbp[dt[i].s + 1]++] = (int32_t)i;
    /* edges */
    const gb_dag_level *lv = P->dag_lv.p;
    const int32_t *lsp = P->dag_sp.p, *lsucc = P->dag_succ.p;
    for (size_t l = 0; ok && l < P->dag_lv.n; l++) {
        for (int32_t t = 0; ok && t < lv[l].ntasks; t++) {
            int32_t e0 = lsp[lv[l].sp_off + t], e1 = lsp[lv[l].sp_off + t + 1];
            for (int32_t e = e0; ok && e < e1; e++) {
                int32_t ed[2] = {(int32_t)(lv[l].task_off + t),
                                 (int32_t)(lv[l].task_off + lsucc[lv[l].succ_off + e])};
                ok &= gb_vec_push(&E, ed);
            }
        }
    }
    for (size_t i = 0; ok && i < nasm; i++) {
        int32_t a = (int32_t)(A0 + i), s = at[i].s;
        if (FUSED(s)) continue;
        int32_t e1[2] = {a, (int32_t)(JA0 + s)}, e2[2] = {(int32_t)(JK0 + s), a};
        ok &= gb_vec_push(&E, e1);
        if (P->h_child_ptr[s + 1] > P->h_child_ptr[s]) ok &= gb_vec_push(&E, e2);
    }
    for (int64_t s = 0; ok && s < ns; s++) {
        int32_t ja = (int32_t)(JA0 + s);
        if (MEMBER(s)) {
            /* SUBTREE(root) -> JK(parent of the root) */
            int32_t par = P->h_parent[s];
            if (sub_root[s] == s && par >= 0) {
                int32_t e[2] = {sub_id[s], (int32_t)(JK0 + par)};
                ok &= gb_vec_push(&E, e);
            }
            continue;
        }
        if (FUSED(s)) {
            /* JK(s) -> NODE(s) -> JK(parent) */
            if (small_id[s] < 0) { ok = 0; break; }
            if (P->h_child_ptr[s + 1] > P->h_child_ptr[s]) {
                int32_t e[2] = {(int32_t)(JK0 + s), small_id[s]};
                ok &= gb_vec_push(&E, e);
            }
            int32_t par = P->h_parent[s];
            if (par >= 0) {
                int32_t e[2] = {small_id[s], (int32_t)(JK0 + par)};
                ok &= gb_vec_push(&E, e);
            }
            continue;
        }
        if (small_id[s] >= 0) {
            int32_t e[2] = {ja, small_id[s]};
            ok &= gb_vec_push(&E, e);
            for (int32_t q = cbp[s]; ok && q < cbp[s + 1]; q++) {
                int32_t e2[2] = {small_id[s], cbl[q]};
                ok &= gb_vec_push(&E, e2);
            }
        } else if (potrf0[s] >= 0) {
            int32_t e[2] = {ja, potrf0[s]};
            ok &= gb_vec_push(&E, e);
        } else {
            ok = 0;                       /* every supernode has one of them */
        }
        int32_t par = P->h_parent[s];
        if (par >= 0)
            for (int32_t q = cbp[s]; ok && q < cbp[s + 1]; q++) {
                int32_t e[2] = {cbl[q], (int32_t)(JK0 + par)};
                ok &= gb_vec_push(&E, e);
            }
    }
    /* CSR, critical successors first; in-degrees; initial ready lists */
    if (ok) {
        deg = calloc(N + 1, sizeof(int32_t));
        nd = calloc(N + 1, sizeof(int32_t));
        pos = malloc(sizeof(int32_t) * (N + 1));
        succ = malloc(sizeof(int32_t) * (E.n + 1));
        tmp = malloc(sizeof(int32_t) * (E.n + 1));
        if (!deg || !nd || !pos || !succ || !tmp) ok = 0;
    }
    if (ok) {
        const int32_t *ed = E.p;
        const gb_dtask *ft = P->fd_t.p;
        for (size_t q = 0; q < E.n; q++) { deg[ed[2 * q] + 1]++; nd[ed[2 * q + 1]]++; }
        for (size_t t = 0; t < N; t++) deg[t + 1] += deg[t];
        memcpy(pos, deg, sizeof(int32_t) * (N + 1));
        for (size_t q = 0; q < E.n; q++) succ[pos[ed[2 * q]]++] = ed[2 * q + 1];
        for (size_t t = 0; t < N; t++)
            gb_order_succ(ft, ft[t].type == GB_DT_DIAG ? ft[t].pad1 : 0, succ, deg[t], deg[t + 1],
                          tmp);
        for (size_t t = 0; ok && t <= N; t++) ok &= gb_vec_push(&P->fd_sp, &deg[t]);
        for (size_t q = 0; ok && q < E.n; q++) ok &= gb_vec_push(&P->fd_succ, &succ[q]);
        /* joins are never queued: the block that finishes a join's last
         * predecessor releases its successors itself */
        P->fd_total0 = P->fd_total1 = 0;
        for (size_t t = 0; ok && t < N; t++) {
            int32_t id = (int32_t)t;
            ok &= gb_vec_push(&P->fd_nd, &nd[t]);
            if (ft[t].type == GB_DT_JOIN) {
                if (nd[t] == 0 && deg[t + 1] > deg[t]) ok = 0;   /* never released */
                continue;
            }
            if (ft[t].prio == 0) P->fd_total0++; else P->fd_total1++;
            if (nd[t] == 0) ok &= gb_vec_push(ft[t].prio == 0 ? &P->fd_q0 : &P->fd_q1, &id);
        }
        /* the bulk tasks ready at the start, largest estimated work first:
         * a launch whose leaves are large subtrees (a batch of systems) does
         * not end waiting on one that started last */
        if (ok && P->fd_q1.n > 1) {
            const size_t nq = P->fd_q1.n;
            int32_t *qv = P->fd_q1.p;
            gb_ready_est *ev = malloc(sizeof(gb_ready_est) * nq);
            if (!ev) ok = 0;
            for (size_t q = 0; ok && q < nq; q++) {
                const gb_dtask *ti = &ft[qv[q]];
                const int64_t sq = ti->s;
                const double nc = (double)(Sup[sq + 1] - Sup[sq]), nr = (double)(Pi[sq + 1] - Pi[sq]);
                double w = 0;
                if (ti->type == GB_DT_SUBTREE) w = work[sq];
                else if (ti->type == GB_DT_NODE || ti->type == GB_DT_SMALL) w = nc * nr * nr;
                else if (ti->type == GB_DT_ASM) w = nr * (double)(ti->r - ti->b);
                ev[q].w = w;
                ev[q].id = qv[q];
            }
            if (ok) {
                qsort(ev, nq, sizeof(gb_ready_est), ready_est_cmp);
                for (size_t q = 0; q < nq; q++) qv[q] = ev[q].id;
            }
            free(ev);
        }
    }
#undef FUSED
#undef MEMBER
    free(sub_root); free(work); free(elig); free(sub_off); free(sub_id);
    free(potrf0); free(small_id); free(cbp); free(cbl);
    free(deg); free(nd); free(pos); free(succ); free(tmp);
    gb_vec_free(&E);
    return ok;
}

/* Independent blocks: the trees of the supernodal etree.  With Perm, the
 * rows of each tree in the original order; if every tree is one contiguous
 * range of original rows (a batch of systems placed on the diagonal, or an
 * irreducible matrix), those ranges are the segments, else one segment. */
static int segments_build(gb_plan *P)
{
    const Int n = P->n, ns = P->nsuper;
    const Int *Super = P->L->super, *Perm = P->L->Perm;
    int32_t *root = malloc(sizeof(int32_t) * (ns + 1));
    int32_t *comp = malloc(sizeof(int32_t) * (n + 1));
    int ok = root && comp;
    /* parents come after children in supernode order */
    for (Int s = ns - 1; ok && s >= 0; s--) {
        int32_t par = P->h_parent[s];
        root[s] = par < 0 ? (int32_t)s : root[par];
    }
    for (Int s = 0; ok && s < ns; s++)
        for (Int k = Super[s]; k < Super[s + 1]; k++) comp[Perm ? Perm[k] : k] = root[s];
    Int runs = 0, ntrees = 0;
    for (Int s = 0; ok && s < ns; s++) ntrees += P->h_parent[s] < 0;
    for (Int i = 0; ok && i < n; i++) runs += (i == 0 || comp[i] != comp[i - 1]);
    int contiguous = ok && runs == ntrees;
    P->nseg = contiguous ? GB_MAX(runs, 1) : 1;
    P->h_seg = malloc(sizeof(int64_t) * (P->nseg + 1));
    if (!P->h_seg) ok = 0;
    if (ok) {
        if (contiguous && n > 0) {
            Int q = 0;
            for (Int i = 0; i < n; i++)
                if (i == 0 || comp[i] != comp[i - 1]) P->h_seg[q++] = i;
        } else {
            P->h_seg[0] = 0;
        }
        P->h_seg[P->nseg] = n;
        P->nchunk = 0;
        for (int64_t g = 0; g < P->nseg; g++) {
            int64_t len = P->h_seg[g + 1] - P->h_seg[g];
            P->nchunk += GB_MAX(1, (len + GB_SEG_CHUNK - 1) / GB_SEG_CHUNK);
        }
        P->h_chunk = malloc(sizeof(gb_seg_chunk) * P->nchunk);
        if (!P->h_chunk) ok = 0;
    }
    if (ok) {
        int64_t q = 0;
        for (int64_t g = 0; g < P->nseg; g++) {
            int64_t lo = P->h_seg[g], hi = P->h_seg[g + 1];
            do {
                gb_seg_chunk ch = {lo, GB_MIN(hi, lo + GB_SEG_CHUNK), (int32_t)g, 0};
                P->h_chunk[q++] = ch;
                lo += GB_SEG_CHUNK;
            } while (lo < hi);
        }
        /* the segment of each supernode (its first column's row of A), for
         * refinement steps that skip converged segments */
        if (P->nseg > 1) {
            P->h_sseg = malloc(sizeof(int32_t) * (ns + 1));
            P->h_segact = malloc((size_t)P->nseg);
            if (!P->h_sseg || !P->h_segact) ok = 0;
            for (Int s = 0; ok && s < ns; s++) {
                const Int i = Perm ? Perm[Super[s]] : Super[s];
                int64_t lo = 0, hi = P->nseg - 1;          /* last g with h_seg[g] <= i */
                while (lo < hi) {
                    const int64_t mid = (lo + hi + 1) / 2;
                    if (P->h_seg[mid] <= i) lo = mid; else hi = mid - 1;
                }
                P->h_sseg[s] = (int32_t)lo;
            }
        }
        /* pinned, so that its copy from the device does not wait for the
         * stream (plain memory when no device is present) */
        if (cudaMallocHost((void **)&P->h_anorm_seg, sizeof(double) * P->nseg) == cudaSuccess) {
            P->anorm_pinned = 1;
            memset(P->h_anorm_seg, 0, sizeof(double) * P->nseg);
        } else {
            cudaGetLastError();
            P->h_anorm_seg = calloc(P->nseg, sizeof(double));
        }
        if (!P->h_anorm_seg) ok = 0;
    }
    free(root);
    free(comp);
    return ok;
}

static int cmp_edge3(const void *a, const void *b)
{
    const int32_t *x = a, *y = b;
    for (int k = 0; k < 3; k++)
        if (x[k] != y[k]) return x[k] < y[k] ? -1 : 1;
    return 0;
}

/* Order the successors succ[lo, hi) of a task critical (prio 0) first;
 * a DIAG task's first `early` successors stay ahead of the others (its
 * executor releases them when its panel solve is done). */
static void gb_order_succ(const gb_dtask *tasks, int32_t early, int32_t *succ, int32_t lo,
                          int32_t hi, int32_t *tmp)
{
    const int32_t mid = lo + early < hi ? lo + early : hi;
    int32_t w = lo;
    for (int part = 0; part < 2; part++) {
        const int32_t a = part ? mid : lo, b = part ? hi : mid;
        for (int pass = 0; pass < 2; pass++)
            for (int32_t e = a; e < b; e++)
                if ((tasks[succ[e]].prio == 0) == (pass == 0)) tmp[w++] = succ[e];
    }
    memcpy(succ + lo, tmp + lo, sizeof(int32_t) * (size_t)(hi - lo));
}

/* Contract each chain (panel solve T of row block b by panel b - 1, the
 * update U of tile (b, b) that follows it, LL' P of panel b) of the level's
 * task graph into one DIAG task in P's place, which one block runs as the
 * three steps in order: the diagonal chain of a wide supernode then costs
 * one task hand-over per panel instead of three.  Edges into or out of T
 * and U move to the DIAG task (edges between the three vanish), T and U
 * leave the task list, and the local task ids are renumbered.  The
 * successors that only T had (the updates that read the block T solves)
 * are the DIAG task's "early" successors, listed first and counted in its
 * pad1: the executor releases them as soon as the solve is done, so that
 * they run beside the rest of the chain as they did beside U and P.  No
 * cycle arises: every path out of T or U that leaves the triple reaches
 * tasks of later panels only, and P's only predecessor is U. */
static int contract_diag(gb_plan *P, size_t t0g, gb_vec *edges, gb_vec *fuse)
{
    const int32_t ntl = (int32_t)(P->dag_t.n - t0g);
    gb_dtask *dt = (gb_dtask *)P->dag_t.p + t0g;
    int32_t *rep = malloc(sizeof(int32_t) * (ntl + 1));
    int32_t *nid = malloc(sizeof(int32_t) * (ntl + 1));
    unsigned char *isT = calloc(ntl + 1, 1);
    int32_t *E3 = malloc(sizeof(int32_t) * 3 * (edges->n + 1));
    if (!rep || !nid || !isT || !E3) { free(rep); free(nid); free(isT); free(E3); return 0; }
    for (int32_t t = 0; t < ntl; t++) rep[t] = t;
    const int32_t *F = fuse->p;
    for (size_t q = 0; q < fuse->n; q++) {
        const int32_t T = F[3 * q], U = F[3 * q + 1], Pt = F[3 * q + 2];
        rep[T] = rep[U] = Pt;
        isT[T] = 1;
        /* DIAG (s, b): b = P's panel; r, nbk = U's first panel and count */
        dt[Pt].type = GB_DT_DIAG;
        dt[Pt].r = dt[U].b;
        dt[Pt].nbk = GB_MAX(1, dt[U].nbk);
        dt[Pt].prio = 0;
        dt[Pt].pad1 = 0;
    }
    /* edges through rep, without self-loops; late = 0 for an edge out of a
     * T (an early successor unless another edge makes it wait) */
    const int32_t *E = edges->p;
    size_t w = 0;
    for (size_t q = 0; q < edges->n; q++) {
        const int32_t a = rep[E[2 * q]], b = rep[E[2 * q + 1]];
        if (a == b) continue;
        E3[3 * w] = a;
        E3[3 * w + 1] = b;
        E3[3 * w + 2] = isT[E[2 * q]] ? 0 : 1;
        w++;
    }
    /* duplicates: one edge, late if any copy is */
    qsort(E3, w, 3 * sizeof(int32_t), cmp_edge3);
    size_t u = 0;
    for (size_t q = 0; q < w; q++) {
        if (u && E3[3 * (u - 1)] == E3[3 * q] && E3[3 * (u - 1) + 1] == E3[3 * q + 1]) {
            E3[3 * (u - 1) + 2] |= E3[3 * q + 2];
            continue;
        }
        memmove(E3 + 3 * u, E3 + 3 * q, 3 * sizeof(int32_t));
        u++;
    }
    /* per source: early edges first (only DIAG sources have any) */
    for (size_t q = 0; q < u; q++) {
        const int32_t tmp = E3[3 * q + 1];
        E3[3 * q + 1] = E3[3 * q + 2];
        E3[3 * q + 2] = tmp;
    }
    qsort(E3, u, 3 * sizeof(int32_t), cmp_edge3);
    for (size_t q = 0; q < u; q++)
        if (E3[3 * q + 1] == 0 && dt[E3[3 * q]].type == GB_DT_DIAG) dt[E3[3 * q]].pad1++;
    /* drop the contracted tasks, renumber the rest */
    int32_t k = 0;
    for (int32_t t = 0; t < ntl; t++) {
        if (rep[t] != t) { nid[t] = -1; continue; }
        nid[t] = k;
        dt[k++] = dt[t];
    }
    P->dag_t.n = t0g + (size_t)k;
    int32_t *Eo = edges->p;
    for (size_t q = 0; q < u; q++) {
        Eo[2 * q] = nid[E3[3 * q]];
        Eo[2 * q + 1] = nid[E3[3 * q + 2]];
    }
    edges->n = u;
    free(rep);
    free(nid);
    free(isT);
    free(E3);
    return 1;
}

gb_plan *gb_plan_build(const cholmod_factor *L, int64_t small_cols, double sub_work,
                       int64_t warp_rows, int64_t upd_group)
{
    if (small_cols < 1) small_cols = 1;
    if (small_cols > GB_SMALL_MAX) small_cols = GB_SMALL_MAX;
    Int n = (Int)L->n, nsuper = (Int)L->nsuper;
    const Int *Super = L->super, *Pi = L->pi, *Px = L->px, *Ls = L->s;
    if (n >= INT32_MAX || (Int)L->ssize >= INT32_MAX) return NULL;

    gb_plan *P = calloc(1, sizeof(gb_plan));
    if (!P) return NULL;
    P->L = L;
    P->small_cols = small_cols;
    P->sub_work = sub_work;
    P->warp_rows = warp_rows < 0 ? 0 : (warp_rows > GB_WARP_ROWS ? GB_WARP_ROWS : warp_rows);
    P->upd_group = upd_group < 1 ? 1 : (upd_group > GB_UPD_GROUP ? GB_UPD_GROUP : upd_group);
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
    vec_init(&P->sf_t, sizeof(gb_stask));
    vec_init(&P->gf, sizeof(int32_t));
    vec_init(&P->gb, sizeof(int32_t));
    vec_init(&P->sb_t, sizeof(gb_stask));
    vec_init(&P->sd_t, sizeof(gb_stask));
    vec_init(&P->lf_t, 2 * sizeof(int32_t));
    vec_init(&P->sf_cptr, sizeof(int32_t));
    vec_init(&P->sf_crange, sizeof(int32_t));
    vec_init(&P->fact_seq, sizeof(gb_launch_rec));
    vec_init(&P->dag_t, sizeof(gb_dtask));
    vec_init(&P->dag_sp, sizeof(int32_t));
    vec_init(&P->dag_succ, sizeof(int32_t));
    vec_init(&P->dag_nd, sizeof(int32_t));
    vec_init(&P->dag_q0, sizeof(int32_t));
    vec_init(&P->dag_q1, sizeof(int32_t));
    vec_init(&P->dag_lv, sizeof(gb_dag_level));
    vec_init(&P->fd_t, sizeof(gb_dtask));
    vec_init(&P->fd_sp, sizeof(int32_t));
    vec_init(&P->fd_succ, sizeof(int32_t));
    vec_init(&P->fd_nd, sizeof(int32_t));
    vec_init(&P->fd_q0, sizeof(int32_t));
    vec_init(&P->fd_q1, sizeof(int32_t));
    vec_init(&P->fd_sub, sizeof(int32_t));
    vec_init(&P->fd_smeta, sizeof(int32_t));
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

    /* ---- factorization sequence: per level ASM, SMALL, DAG ---- */
    const int NB = GB_NB;
    gb_vec edges, fuse;
    vec_init(&edges, 2 * sizeof(int32_t));
    vec_init(&fuse, 3 * sizeof(int32_t));
    for (int l = 0; l < nlevels && ok; l++) {
        size_t a0 = P->asm_t.n;
        for (Int q = lev_ptr[l]; q < lev_ptr[l + 1]; q++) {
            Int s = lev_list[q];
            Int nsrow = Pi[s + 1] - Pi[s];
            /* assembly tasks: chunks of 64 front columns */
            for (Int t0 = 0; t0 < nsrow; t0 += 64) {
                gb_asm_task a = {(int32_t)s, (int32_t)t0, (int32_t)GB_MIN(t0 + 64, nsrow), 0};
                ok &= gb_vec_push(&P->asm_t, &a);
            }
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

        /* task graph of the level: tiles of the wide panels + update blocks */
        int32_t base = 0;
        size_t t0g = P->dag_t.n;
        edges.n = 0;
        fuse.n = 0;
        for (Int q = lev_ptr[l]; q < lev_ptr[l + 1] && ok; q++) {
            Int s = lev_list[q];
            Int nscol = Super[s + 1] - Super[s], nsrow = Pi[s + 1] - Pi[s];
            Int m = nsrow - nscol;
            Int Cp = (nscol + NB - 1) / NB, R = (nsrow + NB - 1) / NB;
            int32_t *Pid = NULL, *Tid = NULL, *Uid = NULL, *Aid = NULL;
            if (nscol > small_cols) {
                /* Blocked right-looking LL' in 64-column panels, grouped by
                 * G = upd_group panels: a tile (r, c) takes the update of
                 * each earlier panel of c's own group separately (UPD with
                 * one panel: the lookahead that the next diagonal steps
                 * wait on) and the updates of each earlier group at once
                 * (UPD with G panels, k up to 64 G), so that the bulk of
                 * the trailing update runs as deeper, fewer tile products.
                 * Updates of one tile run in panel order. */
                const Int G = P->upd_group, Q = (Cp + G - 1) / G;
                Pid = malloc(sizeof(int32_t) * Cp);
                Tid = malloc(sizeof(int32_t) * Cp * R);
                Uid = malloc(sizeof(int32_t) * Cp * R * Cp);
                Aid = malloc(sizeof(int32_t) * Q * R * Cp);
                if (!Pid || !Tid || !Uid || !Aid) {
                    free(Pid); free(Tid); free(Uid); free(Aid);
                    ok = 0;
                    break;
                }
                for (Int b = 0; b < Cp; b++) {
                    Int c0 = b * NB, nb = GB_MIN(NB, nscol - c0);
                    gb_dtask pt = {GB_DT_POTRF, (int32_t)s, (int32_t)b, 0, 0, 0, 0, 0};
                    Pid[b] = base + (int32_t)(P->dag_t.n - t0g);
                    ok &= gb_vec_push(&P->dag_t, &pt);
                    for (Int r = 0; r < R; r++) {
                        Tid[b * R + r] = -1;
                        if (r < b) continue;
                        Int r0 = GB_MAX(NB * r, c0 + nb), r1 = GB_MIN(NB * r + NB, nsrow);
                        if (r1 <= r0) continue;
                        gb_dtask tt = {GB_DT_TRSM, (int32_t)s, (int32_t)b, (int32_t)r, 0,
                                       r <= b + 3 ? 0 : 1, 0, 0};
                        Tid[b * R + r] = base + (int32_t)(P->dag_t.n - t0g);
                        ok &= gb_vec_push(&P->dag_t, &tt);
                    }
                    /* single-panel updates of the tiles in b's own group */
                    for (Int cc = 0; cc < Cp; cc++) {
                        for (Int r = 0; r < R; r++) {
                            Uid[(b * R + r) * Cp + cc] = -1;
                            if (cc <= b || r < cc || cc / G != b / G) continue;
                            gb_dtask ut = {GB_DT_UPD, (int32_t)s, (int32_t)b, (int32_t)r, (int32_t)cc,
                                           (cc <= b + 2 && r <= b + 3) ? 0 : 1, 1, 0};
                            Uid[(b * R + r) * Cp + cc] = base + (int32_t)(P->dag_t.n - t0g);
                            ok &= gb_vec_push(&P->dag_t, &ut);
                        }
                    }
                    /* after the group's last panel: its update of every tile
                     * right of the group */
                    if (b % G == G - 1 || b == Cp - 1) {
                        const Int q = b / G, bq = q * G;
                        for (Int cc = 0; cc < Cp; cc++) {
                            for (Int r = 0; r < R; r++) {
                                Aid[(q * R + r) * Cp + cc] = -1;
                                if (cc < G * (q + 1) || r < cc) continue;
                                gb_dtask at = {GB_DT_UPD, (int32_t)s, (int32_t)bq, (int32_t)r, (int32_t)cc,
                                               (cc == G * (q + 1) && r <= cc + 3) ? 0 : 1,
                                               (int32_t)(b + 1 - bq), 0};
                                Aid[(q * R + r) * Cp + cc] = base + (int32_t)(P->dag_t.n - t0g);
                                ok &= gb_vec_push(&P->dag_t, &at);
                            }
                        }
                    }
                }
                /* the last update task of tile (r, c), r >= c, or -1 */
#define LASTU(r, c) (((c) % G) ? Uid[(((c) - 1) * R + (r)) * Cp + (c)]             \
                     : ((c) > 0 ? Aid[(((c) / G - 1) * R + (r)) * Cp + (c)] : -1))
                /* edges of the blocked right-looking factorization */
                for (Int b = 0; b < Cp && ok; b++) {
                    int32_t e[2];
                    if (LASTU(b, b) >= 0) {
                        e[0] = LASTU(b, b); e[1] = Pid[b];
                        ok &= gb_vec_push(&edges, e);
                    }
                    for (Int r = b; r < R; r++) {
                        int32_t t = Tid[b * R + r];
                        if (t < 0) continue;
                        e[0] = Pid[b]; e[1] = t;
                        ok &= gb_vec_push(&edges, e);
                        if (LASTU(r, b) >= 0) {
                            e[0] = LASTU(r, b); e[1] = t;
                            ok &= gb_vec_push(&edges, e);
                        }
                    }
                    for (Int cc = b + 1; cc < Cp; cc++) {
                        if (cc / G != b / G) continue;
                        for (Int r = cc; r < R; r++) {
                            int32_t u = Uid[(b * R + r) * Cp + cc];
                            e[1] = u;
                            e[0] = Tid[b * R + r]; ok &= gb_vec_push(&edges, e);
                            if (r != cc) { e[0] = Tid[b * R + cc]; ok &= gb_vec_push(&edges, e); }
                            /* the previous update of the tile: this group's
                             * previous panel, or the previous group at once */
                            int32_t pv = (b % G) ? Uid[((b - 1) * R + r) * Cp + cc]
                                         : (b > 0 ? Aid[((b / G - 1) * R + r) * Cp + cc] : -1);
                            if (pv >= 0) { e[0] = pv; ok &= gb_vec_push(&edges, e); }
                        }
                    }
                    if (b % G == G - 1 || b == Cp - 1) {
                        /* the group's panel solves of rows r and cc: the last
                         * panel's (each earlier one precedes it through the
                         * tile (r, b) updates) */
                        const Int q = b / G;
                        for (Int cc = G * (q + 1); cc < Cp; cc++) {
                            for (Int r = cc; r < R; r++) {
                                int32_t u = Aid[(q * R + r) * Cp + cc];
                                e[1] = u;
                                e[0] = Tid[b * R + r]; ok &= gb_vec_push(&edges, e);
                                if (r != cc) { e[0] = Tid[b * R + cc]; ok &= gb_vec_push(&edges, e); }
                                if (q > 0) {
                                    e[0] = Aid[((q - 1) * R + r) * Cp + cc];
                                    ok &= gb_vec_push(&edges, e);
                                }
                            }
                        }
                    }
                }
                /* the diagonal chain: panel solve of row block b by panel
                 * b - 1, the update of tile (b, b) that follows it, LL' of
                 * panel b -- contracted into one DIAG task below */
                for (Int b = 1; b < Cp && ok; b++) {
                    int32_t tri[3] = {Tid[(b - 1) * R + b], LASTU(b, b), Pid[b]};
                    if (tri[0] < 0 || tri[1] < 0) continue;
                    ok &= gb_vec_push(&fuse, tri);
                }
#undef LASTU
            }
            if (Pid) {
                /* algorithmic flops of the panel tasks (2 per multiply-add) */
                for (Int b = 0; b < Cp; b++) {
                    double nb = (double)GB_MIN(NB, nscol - b * NB);
                    P->fl_dag += nb * nb * nb / 3.0;                         /* LL' */
                    P->fl_dag += (double)(nsrow - b * NB - nb) * nb * nb;    /* solve */
                    double w = (double)(nscol - b * NB - nb);                /* trailing cols */
                    double h = (double)(nsrow - b * NB - nb);                /* trailing rows */
                    P->fl_dag += (w * h - w * (w - 1) / 2.0) * 2.0 * nb;     /* lower update */
                }
            }
            {
                double mm = (double)m;
                P->fl_dag += mm * (mm + 1) / 2.0 * 2.0 * (double)nscol;     /* update block */
            }
            /* update-block tiles (k = nscol).  A supernode with panel tasks
             * tiles its update block on the 64-row grid of its own rows
             * (tk.b = 1), so that a tile's operand rows are exactly the
             * row blocks the panel solves produce (and write as the
             * tensor-core operand images); tile (r, c) needs the last
             * panel's solves of row blocks r and c. */
            if (Pid && m > 0) {
                const Int lastb = Cp - 1;
                for (Int cc = nscol / NB; cc < R && ok; cc++) {
                    for (Int r = cc; r < R && ok; r++) {
                        gb_dtask ct = {GB_DT_CB, (int32_t)s, 1, (int32_t)r, (int32_t)cc, 1, 0, 0};
                        int32_t cid = base + (int32_t)(P->dag_t.n - t0g);
                        ok &= gb_vec_push(&P->dag_t, &ct);
                        int32_t t1 = Tid[lastb * R + r], t2 = Tid[lastb * R + cc];
                        if (t1 < 0 || t2 < 0) { ok = 0; break; }
                        int32_t e[2] = {t1, cid};
                        ok &= gb_vec_push(&edges, e);
                        if (t2 != t1) { e[0] = t2; ok &= gb_vec_push(&edges, e); }
                    }
                }
            }
            /* a narrow supernode (factored whole by one SMALL task, which
             * precedes these tiles through its join): the update block's
             * own 64-grid */
            for (Int J = 0; !Pid && J < m && ok; J += NB) {
                for (Int I = J; I < m; I += NB) {
                    gb_dtask ct = {GB_DT_CB, (int32_t)s, 0, (int32_t)(I / NB), (int32_t)(J / NB), 1, 0, 0};
                    ok &= gb_vec_push(&P->dag_t, &ct);
                }
            }
            free(Pid); free(Tid); free(Uid); free(Aid);
        }
        if (!ok) break;
        if (fuse.n) ok = contract_diag(P, t0g, &edges, &fuse);
        if (!ok) break;
        /* CSR of successors, dependency counts, initial ready lists */
        int32_t ntl = (int32_t)(P->dag_t.n - t0g);
        gb_dag_level lv;
        memset(&lv, 0, sizeof lv);
        lv.task_off = (int64_t)t0g;
        lv.ntasks = ntl;
        lv.sp_off = (int64_t)P->dag_sp.n;
        lv.succ_off = (int64_t)P->dag_succ.n;
        lv.q0_off = (int64_t)P->dag_q0.n;
        lv.q1_off = (int64_t)P->dag_q1.n;
        if (ntl > 0) {
            int32_t *deg = calloc(ntl + 1, sizeof(int32_t));
            int32_t *nd = calloc(ntl + 1, sizeof(int32_t));
            int32_t *pos = malloc(sizeof(int32_t) * (ntl + 1));
            int32_t *succ = malloc(sizeof(int32_t) * (edges.n + 1));
            if (!deg || !nd || !pos || !succ) ok = 0;
            const int32_t *E = edges.p;
            for (size_t q2 = 0; ok && q2 < edges.n; q2++) { deg[E[2 * q2] + 1]++; nd[E[2 * q2 + 1]]++; }
            for (int32_t t = 0; ok && t < ntl; t++) deg[t + 1] += deg[t];
            if (ok) memcpy(pos, deg, sizeof(int32_t) * (ntl + 1));
            for (size_t q2 = 0; ok && q2 < edges.n; q2++) succ[pos[E[2 * q2]]++] = E[2 * q2 + 1];
            const gb_dtask *dt = (const gb_dtask *)P->dag_t.p + t0g;
            /* critical successors first: a finished task notifies its
             * successors 32 at a time, in list order */
            int32_t *tmp = ok ? malloc(sizeof(int32_t) * (edges.n + 1)) : NULL;
            if (!tmp) ok = 0;
            for (int32_t t = 0; ok && t < ntl; t++)
                gb_order_succ(dt, dt[t].type == GB_DT_DIAG ? dt[t].pad1 : 0, succ, deg[t],
                              deg[t + 1], tmp);
            free(tmp);
            for (int32_t t = 0; ok && t <= ntl; t++) ok &= gb_vec_push(&P->dag_sp, &deg[t]);
            for (size_t q2 = 0; ok && q2 < edges.n; q2++) ok &= gb_vec_push(&P->dag_succ, &succ[q2]);
            for (int32_t t = 0; ok && t < ntl; t++) {
                if (dt[t].prio == 0) lv.total0++; else lv.total1++;
                ok &= gb_vec_push(&P->dag_nd, &nd[t]);
                if (nd[t] == 0) {
                    if (dt[t].prio == 0) { ok &= gb_vec_push(&P->dag_q0, &t); lv.n0++; }
                    else { ok &= gb_vec_push(&P->dag_q1, &t); lv.n1++; }
                }
            }
            free(deg); free(nd); free(pos); free(succ);
            P->dag_max = GB_MAX(P->dag_max, ntl);
        }
        int32_t li = (int32_t)P->dag_lv.n;
        ok &= gb_vec_push(&P->dag_lv, &lv);
        if (ntl > 0) {
            gb_launch_rec r;
            r.kind = GB_K_DAG;
            r.count = ntl;
            r.off = li;
            ok &= gb_vec_push(&P->fact_seq, &r);
        }
    }
    gb_vec_free(&edges);
    gb_vec_free(&fuse);

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
    /* ---- single-launch sweep tasks (postorder = topological order) ---- */
    P->h_blkoff = malloc(sizeof(int32_t) * (nsuper + 1));
    P->h_ntask_f = malloc(sizeof(int32_t) * (nsuper + 1));
    P->h_ntask_b = malloc(sizeof(int32_t) * (nsuper + 1));
    P->h_parent = malloc(sizeof(int32_t) * (nsuper + 1));
    if (!P->h_blkoff || !P->h_ntask_f || !P->h_ntask_b || !P->h_parent) ok = 0;
    int64_t nblk_total = 0;
    for (Int s = 0; s < nsuper && ok; s++) {
        Int nscol = Super[s + 1] - Super[s], nsrow = Pi[s + 1] - Pi[s];
        Int nblk = (nscol + 63) / 64, m = nsrow - nscol;
        P->h_blkoff[s] = (int32_t)nblk_total;
        P->h_parent[s] = (int32_t)parent[s];
        nblk_total += nblk;
        P->h_ntask_b[s] = (int32_t)nblk;
        P->h_ntask_f[s] = (int32_t)(nblk + (m + 63) / 64);
        for (Int i = 0; i < nblk; i++) {     /* diagonal blocks in global block order */
            gb_stask t = {(int32_t)s, 0, (int32_t)i, (int32_t)(i * 64),
                          (int32_t)GB_MIN(64, nscol - i * 64), 0, 0, 0};
            ok &= gb_vec_push(&P->sd_t, &t);
        }
    }
    /* backward sweep: per supernode, the global diagonal block holding the
     * first row of each 64-row chunk of its rows below the diagonal block
     * (the chunk's x is final when that block is) */
    P->h_bchunk_ptr = ok ? malloc(sizeof(int32_t) * (nsuper + 1)) : NULL;
    if (!P->h_bchunk_ptr) ok = 0;
    int64_t nbchunk = 0;
    for (Int s = 0; s < nsuper && ok; s++) {
        P->h_bchunk_ptr[s] = (int32_t)nbchunk;
        nbchunk += (Pi[s + 1] - Pi[s] - (Super[s + 1] - Super[s]) + 63) / 64;
    }
    if (ok) P->h_bchunk_ptr[nsuper] = (int32_t)nbchunk;
    P->h_bchunk = ok ? malloc(sizeof(int32_t) * (nbchunk + 1)) : NULL;
    if (!P->h_bchunk || nbchunk >= INT32_MAX) ok = 0;
    for (Int s = 0; s < nsuper && ok; s++) {
        Int nscol = Super[s + 1] - Super[s], m = Pi[s + 1] - Pi[s] - nscol;
        for (Int q = 0; q < (m + 63) / 64; q++) {
            const Int g = Ls[Pi[s] + nscol + 64 * q], a = SuperMap[g];
            P->h_bchunk[P->h_bchunk_ptr[s] + q] = P->h_blkoff[a] + (int32_t)((g - Super[a]) / 64);
        }
    }
    /* leaf subtrees of the sweeps: maximal subtrees whose fronts all have at
     * most GB_LEAF_ROWS rows and one diagonal block (at most 64 columns), at
     * most leaf_cap supernodes each (below; none
     * when the one-warp fronts are off, warp_rows = 0).  One warp
     * sweeps a whole one (children first forward, parents first backward) in
     * a launch of its own, before the forward sweep's other tasks (a leaf
     * subtree depends on nothing) and after the backward sweep's (it depends
     * only on its ancestors).  In postorder a subtree is the index range
     * [root - size + 1, root]; its supernodes have no tasks in the lists. */
    int32_t *lcnt = calloc(nsuper + 1, sizeof(int32_t));
    char *lel = malloc(nsuper + 1), *lmem = calloc(nsuper + 1, 1);
    if (!lcnt || !lel || !lmem) ok = 0;
    for (Int s = 0; s < nsuper && ok; s++)
        lel[s] = P->warp_rows > 0 && Pi[s + 1] - Pi[s] <= GB_LEAF_ROWS && Super[s + 1] - Super[s] <= 64;
    for (Int s = 0; s < nsuper && ok; s++) {          /* children before parents */
        lcnt[s] += 1;
        if (parent[s] != EMPTY) {
            lcnt[parent[s]] += lcnt[s];
            if (!lel[s]) lel[parent[s]] = 0;
        }
    }
    /* members per leaf subtree: up to GB_LEAF_MEMBERS in a large forest (a
     * batch: many subtrees side by side, throughput), fewer in a small one
     * (one warp sweeps a subtree serially: its length is the leaf phase's
     * latency when there are few of them) */
    const Int leaf_cap = GB_MAX(16, GB_MIN(GB_LEAF_MEMBERS, nsuper / 1024));
#define LEAF_OK(s) (lel[s] && lcnt[s] <= leaf_cap)
    for (Int s = 0; s < nsuper && ok; s++) {
        if (!LEAF_OK(s) || (parent[s] != EMPTY && LEAF_OK(parent[s]))) continue;
        Int s0 = s - lcnt[s] + 1;
        int contiguous = s0 >= 0;
        for (Int q = s0; contiguous && q < s; q++)
            contiguous = parent[q] > q && parent[q] <= s;
        if (!contiguous) continue;
        int32_t pr[2] = {(int32_t)s0, (int32_t)s};
        ok &= gb_vec_push(&P->lf_t, pr);
        for (Int q = s0; q <= s; q++) {
            lmem[q] = 1;
            P->leaf_rows = (int)GB_MAX(P->leaf_rows, Pi[q + 1] - Pi[q]);
        }
    }
#undef LEAF_OK
    /* forward: levels ascending; backward: levels descending, so that a task
     * only depends on tasks listed before it and branches interleave */
    for (int l = 0; l < nlevels && ok; l++) {
        for (Int q = lev_ptr[l]; q < lev_ptr[l + 1]; q++) {
            Int s = lev_list[q];
            if (lmem[s]) continue;
            Int nscol = Super[s + 1] - Super[s], nsrow = Pi[s + 1] - Pi[s];
            Int nblk = (nscol + 63) / 64;
            for (Int i = 0; i < nblk; i++) {
                gb_stask t = {(int32_t)s, 0, (int32_t)i, (int32_t)(i * 64),
                              (int32_t)GB_MIN(64, nscol - i * 64), 0, 0, 0};
                ok &= gb_vec_push(&P->sf_t, &t);
            }
            for (Int r = nscol; r < nsrow; r += 64) {
                gb_stask t = {(int32_t)s, 1, 0, (int32_t)r, (int32_t)GB_MIN(64, nsrow - r), 0, 0, 0};
                ok &= gb_vec_push(&P->sf_t, &t);
            }
        }
    }
    for (int l = nlevels - 1; l >= 0 && ok; l--) {
        for (Int q = lev_ptr[l + 1] - 1; q >= lev_ptr[l]; q--) {
            Int s = lev_list[q];
            if (lmem[s]) continue;
            Int nscol = Super[s + 1] - Super[s];
            Int nblk = (nscol + 63) / 64;
            for (Int i = nblk - 1; i >= 0; i--) {
                gb_stask t = {(int32_t)s, 0, (int32_t)i, (int32_t)(i * 64),
                              (int32_t)GB_MIN(64, nscol - i * 64), 0, 0, 0};
                ok &= gb_vec_push(&P->sb_t, &t);
            }
        }
    }
    /* ticket groups: runs of tasks of leaf-level supernodes (levels 0-1, at
     * most 64 columns and 64 rows), 8 per ticket, so that the tens of
     * thousands of tiny tasks do not serialise on the ticket counter; every
     * other task is a group of its own.  A block runs its group in order, and
     * a task still depends only on tasks listed before it. */
    for (int w = 0; w < 2 && ok; w++) {
        gb_vec *tv = w ? &P->sb_t : &P->sf_t, *gv = w ? &P->gb : &P->gf;
        const gb_stask *tt = tv->p;
        int32_t start = 0;
        ok &= gb_vec_push(gv, &start);
        size_t q = 0;
        while (ok && q < tv->n) {
            size_t e = q + 1;
            Int s = tt[q].s;
            int small = level[s] <= 1 && Super[s + 1] - Super[s] <= 64 && Pi[s + 1] - Pi[s] <= 64;
            if (small)
                while (e < tv->n && e - q < 8) {
                    Int s2 = tt[e].s;
                    if (!(level[s2] <= 1 && Super[s2 + 1] - Super[s2] <= 64 && Pi[s2 + 1] - Pi[s2] <= 64)) break;
                    e++;
                }
            int32_t end = (int32_t)e;
            ok &= gb_vec_push(gv, &end);
            q = e;
        }
    }
    /* forward tasks: each child's update-vector rows that fall in the
     * task's rows [r0, r0 + nr) (the relative map is increasing), so the
     * sweep reads a range instead of searching the map on the device */
    {
        const gb_stask *tt = P->sf_t.p;
        int32_t cnt = 0;
        ok &= gb_vec_push(&P->sf_cptr, &cnt);
        for (size_t q = 0; ok && q < P->sf_t.n; q++) {
            const Int s0 = tt[q].s, r0 = tt[q].r0, r1 = tt[q].r0 + tt[q].nr;
            for (int32_t ci = child_ptr[s0]; ok && ci < child_ptr[s0 + 1]; ci++) {
                const Int c = child_list[ci], ncc = Super[c + 1] - Super[c];
                const int32_t *rm = relmap + Pi[c] + ncc;
                const Int mc = Pi[c + 1] - Pi[c] - ncc;
                Int lo = 0, hi = mc;
                while (lo < hi) { Int mid = (lo + hi) / 2; if (rm[mid] < r0) lo = mid + 1; else hi = mid; }
                const Int a = lo;
                hi = mc;
                while (lo < hi) { Int mid = (lo + hi) / 2; if (rm[mid] < r1) lo = mid + 1; else hi = mid; }
                int32_t ab[2] = {(int32_t)a, (int32_t)lo};
                ok &= gb_vec_push(&P->sf_crange, &ab[0]) && gb_vec_push(&P->sf_crange, &ab[1]);
                cnt++;
            }
            ok &= gb_vec_push(&P->sf_cptr, &cnt);
        }
    }
    free(lcnt); free(lel); free(lmem);
    P->nblk_total = nblk_total;
    P->h_linvoff = malloc(sizeof(int64_t) * (nblk_total + 1));
    if (!P->h_linvoff) ok = 0;
    if (ok) {
        int64_t off = 0;
        const gb_stask *sd = P->sd_t.p;
        for (size_t q = 0; q < P->sd_t.n; q++) {
            P->h_linvoff[q] = off;               /* sd_t is in global block order */
            off += (int64_t)sd[q].nr * sd[q].nr;
        }
        P->h_linvoff[nblk_total] = off;
        P->linv_total = off;
    }
    /* tensor-core operand images: a supernode with panel tasks (wider than
     * small_cols) has one per panel b < Cp and row block b <= r < R */
    P->h_imgbase = malloc(sizeof(int64_t) * (P->nsuper + 1));
    if (!P->h_imgbase) ok = 0;
    if (ok) {
        int64_t tot = 0;
        for (Int s = 0; s < P->nsuper; s++) {
            const Int nscol = Super[s + 1] - Super[s], nsrow = Pi[s + 1] - Pi[s];
            P->h_imgbase[s] = -1;
            if (nscol <= small_cols) continue;
            const int64_t Cp = (nscol + GB_NB - 1) / GB_NB, R = (nsrow + GB_NB - 1) / GB_NB;
            P->h_imgbase[s] = tot;
            tot += Cp * R - Cp * (Cp - 1) / 2;
        }
        P->h_imgbase[P->nsuper] = tot;
        P->img_total = tot;
    }
    if (!ok) goto fail;

    P->h_child_ptr = child_ptr;
    P->h_child_list = child_list;
    P->h_relmap = relmap;
    P->h_cboff = cboff;
    P->h_cbvoff = cbvoff;
    free(SuperMap); free(parent); free(level); free(Map); free(lev_ptr); free(lev_list);
    if (!fdag_build(P) || !segments_build(P)) { gb_plan_free(P); return NULL; }
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
        P->struct_bytes += b_;                                                 \
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
    UP(P->d_dag_t, P->dag_t.p, P->dag_t.n * P->dag_t.esz);
    UP(P->d_dag_sp, P->dag_sp.p, P->dag_sp.n * P->dag_sp.esz);
    UP(P->d_dag_succ, P->dag_succ.p, P->dag_succ.n * P->dag_succ.esz);
    UP(P->d_dag_nd, P->dag_nd.p, P->dag_nd.n * P->dag_nd.esz);
    UP(P->d_dag_q0i, P->dag_q0.p, P->dag_q0.n * P->dag_q0.esz);
    UP(P->d_dag_q1i, P->dag_q1.p, P->dag_q1.n * P->dag_q1.esz);
    {
        size_t nl = P->dag_lv.n;
        int32_t *ctrl0 = calloc(GB_DAG_NCTRL * (nl + 1), sizeof(int32_t));
        if (!ctrl0) goto fail;
        const gb_dag_level *lv = P->dag_lv.p;
        for (size_t i = 0; i < nl; i++) {
            ctrl0[GB_DAG_NCTRL * i + 1] = lv[i].n0;
            ctrl0[GB_DAG_NCTRL * i + 3] = lv[i].n1;
            ctrl0[GB_DAG_NCTRL * i + 6] = lv[i].total0;
            ctrl0[GB_DAG_NCTRL * i + 7] = lv[i].total1;
        }
        int okc = cudaMalloc((void **)&P->d_dag_ctrl0, sizeof(int32_t) * GB_DAG_NCTRL * (nl + 1)) == cudaSuccess
                  && cudaMemcpy(P->d_dag_ctrl0, ctrl0, sizeof(int32_t) * GB_DAG_NCTRL * (nl + 1), cudaMemcpyHostToDevice) == cudaSuccess;
        free(ctrl0);
        if (!okc) goto fail;
    }
    {
        size_t mx = (size_t)GB_MAX(P->dag_max, 1);
        if (cudaMalloc((void **)&P->d_dag_cnt, sizeof(int32_t) * mx) != cudaSuccess) goto fail;
        if (cudaMalloc((void **)&P->d_dag_q, sizeof(int32_t) * 2 * mx) != cudaSuccess) goto fail;
        P->struct_bytes += sizeof(int32_t) * 3 * mx;
        if (cudaMalloc((void **)&P->d_dag_ctrl, sizeof(int32_t) * GB_DAG_NCTRL) != cudaSuccess) goto fail;
        if (cudaMalloc((void **)&P->d_dag_smf, sizeof(int32_t) * GB_DAG_NSMF) != cudaSuccess) goto fail;
        if (cudaMemset(P->d_dag_smf, 0, sizeof(int32_t) * GB_DAG_NSMF) != cudaSuccess) goto fail;
    }
    UP(P->d_sf, P->sf_t.p, P->sf_t.n * P->sf_t.esz);
    UP(P->d_gf, P->gf.p, P->gf.n * P->gf.esz);
    UP(P->d_gb, P->gb.p, P->gb.n * P->gb.esz);
    UP(P->d_sb, P->sb_t.p, P->sb_t.n * P->sb_t.esz);
    UP(P->d_lf, P->lf_t.p, P->lf_t.n * P->lf_t.esz);
    UP(P->d_sf_cptr, P->sf_cptr.p, P->sf_cptr.n * P->sf_cptr.esz);
    UP(P->d_sf_crange, P->sf_crange.p, P->sf_crange.n * P->sf_crange.esz);
    UP(P->d_sd, P->sd_t.p, P->sd_t.n * P->sd_t.esz);
    UP(P->d_blkoff, P->h_blkoff, sizeof(int32_t) * (ns + 1));
    UP(P->d_ntask_f, P->h_ntask_f, sizeof(int32_t) * (ns + 1));
    UP(P->d_ntask_b, P->h_ntask_b, sizeof(int32_t) * (ns + 1));
    UP(P->d_bchunk_ptr, P->h_bchunk_ptr, sizeof(int32_t) * (ns + 1));
    UP(P->d_bchunk, P->h_bchunk, sizeof(int32_t) * (size_t)P->h_bchunk_ptr[ns]);
    UP(P->d_parent, P->h_parent, sizeof(int32_t) * (ns + 1));
    UP(P->d_linvoff, P->h_linvoff, sizeof(int64_t) * (P->nblk_total + 1));
    UP(P->d_imgbase, P->h_imgbase, sizeof(int64_t) * (ns + 1));
    if (cudaMalloc((void **)&P->d_xready, sizeof(int32_t) * (P->nblk_total + 1)) != cudaSuccess) goto fail;
    if (cudaMalloc((void **)&P->d_done, sizeof(int32_t) * (ns + 1)) != cudaSuccess) goto fail;
    P->struct_bytes += sizeof(int32_t) * (P->nblk_total + ns + 2);
    if (cudaMalloc((void **)&P->d_ticket, sizeof(int32_t) * 4) != cudaSuccess) goto fail;
    P->d_err = P->d_ticket + 2;
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
    P->ptrs.blkoff = P->d_blkoff;
    P->ptrs.linvoff = P->d_linvoff;
    P->ptrs.imgbase = P->d_imgbase;
    UP(P->d_chunk, P->h_chunk, sizeof(gb_seg_chunk) * P->nchunk);
    if (P->h_sseg) {
        UP(P->d_sseg, P->h_sseg, sizeof(int32_t) * P->nsuper);
        if (cudaMalloc((void **)&P->d_segact, (size_t)P->nseg + 16) != cudaSuccess) goto fail;
        P->struct_bytes += (size_t)P->nseg + 16;
    }
    if (cudaMalloc((void **)&P->d_anorm_seg, sizeof(double) * (P->nseg + 1)) != cudaSuccess) goto fail;
    /* whole-factorization task graph, one instance */
    UP(P->d_fd_t, P->fd_t.p, P->fd_t.n * P->fd_t.esz);
    UP(P->d_fd_sp, P->fd_sp.p, P->fd_sp.n * P->fd_sp.esz);
    UP(P->d_fd_succ, P->fd_succ.p, P->fd_succ.n * P->fd_succ.esz);
    UP(P->d_fd_nd, P->fd_nd.p, P->fd_nd.n * P->fd_nd.esz);
    UP(P->d_fd_sub, P->fd_sub.p, P->fd_sub.n * P->fd_sub.esz);
    UP(P->d_fd_smeta, P->fd_smeta.p, P->fd_smeta.n * P->fd_smeta.esz);
    {
        size_t n0 = P->fd_q0.n, n1 = P->fd_q1.n, N = P->fd_t.n;
        int32_t *qi = malloc(sizeof(int32_t) * (n0 + n1 + 1));
        if (!qi) goto fail;
        if (n0) memcpy(qi, P->fd_q0.p, sizeof(int32_t) * n0);
        if (n1) memcpy(qi + n0, P->fd_q1.p, sizeof(int32_t) * n1);
        int okq = cudaMalloc((void **)&P->d_fd_qi, sizeof(int32_t) * (n0 + n1 + 1)) == cudaSuccess
                  && cudaMemcpy(P->d_fd_qi, qi, sizeof(int32_t) * (n0 + n1), cudaMemcpyHostToDevice) == cudaSuccess;
        free(qi);
        if (!okq) goto fail;
        int32_t ctrl0[GB_DAG_NCTRL];
        memset(ctrl0, 0, sizeof ctrl0);
        ctrl0[1] = (int32_t)n0;
        ctrl0[3] = (int32_t)n1;
        ctrl0[6] = P->fd_total0;
        ctrl0[7] = P->fd_total1;
        UP(P->d_fd_ctrl0, ctrl0, sizeof ctrl0);
        if (cudaMalloc((void **)&P->d_fd_cnt, sizeof(int32_t) * (N + 1)) != cudaSuccess) goto fail;
        if (cudaMalloc((void **)&P->d_fd_q, sizeof(int32_t) * 2 * (N + 1)) != cudaSuccess) goto fail;
        P->struct_bytes += sizeof(int32_t) * (n0 + n1 + 3 * (N + 1));
        gb_finst inst;
        memset(&inst, 0, sizeof inst);
        inst.fail = P->d_fail;
        inst.anyfail = P->d_anyfail;
        UP(P->d_fd_inst, &inst, sizeof inst);
        int64_t ib = 0;
        UP(P->d_fd_ibase, &ib, sizeof ib);
        if (cudaMalloc((void **)&P->d_fd_pat, sizeof(gb_fpat)) != cudaSuccess) goto fail;
        memset(&P->h_fd_pat, 0, sizeof P->h_fd_pat);
    }
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
    free(P->h_blkoff); free(P->h_ntask_f); free(P->h_ntask_b); free(P->h_parent);
    free(P->h_bchunk_ptr); free(P->h_bchunk);
    free(P->h_linvoff);
    free(P->h_imgbase);
    gb_vec_free(&P->sf_t); gb_vec_free(&P->sb_t); gb_vec_free(&P->sd_t);
    gb_vec_free(&P->lf_t);
    gb_vec_free(&P->sf_cptr); gb_vec_free(&P->sf_crange);
    gb_vec_free(&P->gf); gb_vec_free(&P->gb);
    gb_vec_free(&P->dag_t); gb_vec_free(&P->dag_sp); gb_vec_free(&P->dag_succ);
    gb_vec_free(&P->dag_nd); gb_vec_free(&P->dag_q0); gb_vec_free(&P->dag_q1);
    gb_vec_free(&P->dag_lv);
    gb_valmap_free(P);
    gb_graph_free(P);
    free(P->h_seg); free(P->h_chunk); free(P->h_sseg); free(P->h_segact);
    if (P->anorm_pinned) cudaFreeHost(P->h_anorm_seg);
    else free(P->h_anorm_seg);
    gb_vec_free(&P->fd_t); gb_vec_free(&P->fd_sp); gb_vec_free(&P->fd_succ);
    gb_vec_free(&P->fd_nd); gb_vec_free(&P->fd_q0); gb_vec_free(&P->fd_q1);
    gb_vec_free(&P->fd_sub);
    gb_vec_free(&P->fd_smeta);
    void *dev[] = {P->d_Super, P->d_Pi, P->d_Px, P->d_cboff, P->d_cbvoff, P->d_Perm,
                   P->d_Ls, P->d_relmap, P->d_child_ptr, P->d_child_list, P->d_fail,
                   P->d_anyfail, P->d_asm, P->d_node, P->d_potrf, P->d_trsm, P->d_gemm,
                   P->d_gemm_owner, P->d_sweep, P->d_Lx[0], P->d_Lx[1],
                   P->d_Sp, P->d_Si, P->d_Sx, P->d_Y, P->d_U, P->d_B, P->d_spw, P->d_sws,
                   P->d_Rp, P->d_Rj, P->d_Rx, P->d_scale, P->d_scale_perm, P->d_X, P->d_R,
                   P->d_bx, P->d_red, P->d_sf, P->d_sb, P->d_sd, P->d_lf, P->d_sf_cptr, P->d_sf_crange, P->d_blkoff, P->d_ntask_f,
                   P->d_ntask_b, P->d_parent, P->d_bchunk_ptr, P->d_bchunk, P->d_linvoff, P->d_xready, P->d_done,
                   P->d_ticket, P->d_Linv[0], P->d_Linv[1], P->d_dag_t, P->d_dag_sp,
                   P->d_dag_succ, P->d_dag_nd, P->d_dag_q0i, P->d_dag_q1i, P->d_dag_ctrl0,
                   P->d_dag_cnt, P->d_dag_q, P->d_dag_ctrl, P->d_dag_smf, P->d_fd_t,
                   P->d_fd_sp, P->d_fd_succ, P->d_fd_nd, P->d_fd_qi, P->d_fd_ctrl0,
                   P->d_fd_cnt, P->d_fd_q, P->d_fd_pat, P->d_fd_inst, P->d_fd_ibase, P->d_fd_sub,
                   P->d_fd_smeta, P->d_imgbase,
                   P->d_chunk, P->d_anorm_seg, P->d_bred, P->d_gf, P->d_gb, P->d_sseg,
                   P->d_segact};
    for (size_t i = 0; i < sizeof dev / sizeof dev[0]; i++)
        if (dev[i]) cudaFree(dev[i]);
    gb_vec_free(&P->asm_t); gb_vec_free(&P->node_t); gb_vec_free(&P->potrf_t);
    gb_vec_free(&P->trsm_t); gb_vec_free(&P->gemm_t); gb_vec_free(&P->gemm_owner);
    gb_vec_free(&P->sweep_t); gb_vec_free(&P->fact_seq); gb_vec_free(&P->fwd_seq);
    gb_vec_free(&P->bwd_seq);
    free(P);
}
