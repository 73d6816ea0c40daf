/* Host check of the factorization's tile task graph (gb_plan.c), compiled
 * by tests/test_plan_dag.py with the library's host sources.
 *
 * For every update group 1..4: the task graph of every level is acyclic,
 * and executing the tile tasks of every wide supernode (POTRF, TRSM, UPD,
 * DIAG, CB on its own 64-row grid) in random topological orders of that
 * graph on a dense SPD front gives the front's blocked Cholesky: L and the
 * Schur complement of the update block, to rounding.  A DIAG task runs in
 * two parts with its early successors released in between, as on the GPU.
 * A missing dependency lets some order read a tile before its last update,
 * which shows as an error far above rounding.
 *
 * usage: plan_dag_check Ap.bin Ai.bin perm.bin  (int64 arrays of the lower
 * pattern of A and a postordered fill-reducing permutation) */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "gb_plan.h"

/* host sources only: what the planner links against but never calls here */
void gb_valmap_free(gb_plan *P) { (void)P; }
void gb_graph_free(gb_plan *P) { (void)P; }
gb_ctx *gb_ctx_new(void) { return NULL; }
void gb_ctx_delete(gb_ctx *c) { (void)c; }
int gb_release_factor_state(cholmod_factor *L) { (void)L; return 1; }

static void *read_all(const char *f, size_t *count)
{
    FILE *fp = fopen(f, "rb");
    if (!fp) return NULL;
    fseek(fp, 0, SEEK_END);
    long sz = ftell(fp);
    fseek(fp, 0, SEEK_SET);
    void *b = malloc(sz > 0 ? sz : 8);
    size_t got = fread(b, 1, sz, fp);
    fclose(fp);
    *count = got / 8;
    return b;
}

static uint64_t rng = 88172645463325252ull;
static uint64_t next_rand(void)
{
    rng ^= rng << 13;
    rng ^= rng >> 7;
    rng ^= rng << 17;
    return rng;
}

#define F_(i, j) F[(i) + (size_t)(j) * ld]

static void chol_block(double *F, int ld, int c0, int nb)
{
    for (int j = c0; j < c0 + nb; j++) {
        double d = F_(j, j);
        for (int k = c0; k < j; k++) d -= F_(j, k) * F_(j, k);
        d = sqrt(d);
        F_(j, j) = d;
        for (int i = j + 1; i < c0 + nb; i++) {
            double v = F_(i, j);
            for (int k = c0; k < j; k++) v -= F_(i, k) * F_(j, k);
            F_(i, j) = v / d;
        }
    }
}

static void solve_rows(double *F, int ld, int r0, int r1, int c0, int nb)
{
    for (int i = r0; i < r1; i++)
        for (int j = c0; j < c0 + nb; j++) {
            double v = F_(i, j);
            for (int k = c0; k < j; k++) v -= F_(i, k) * F_(j, k);
            F_(i, j) = v / F_(j, j);
        }
}

static void update(double *F, int ld, int r0, int r1, int q0, int q1, int k0, int k1, int lower)
{
    for (int j = q0; j < q1; j++)
        for (int i = r0; i < r1; i++) {
            if (lower && i < j) continue;
            double v = 0;
            for (int k = k0; k < k1; k++) v += F_(i, k) * F_(j, k);
            F_(i, j) -= v;
        }
}

static int imin(int a, int b) { return a < b ? a : b; }
static int imax(int a, int b) { return a > b ? a : b; }

/* the arithmetic of one task on the dense front of its supernode */
static void run_task(const gb_dtask *t, double **front, const int64_t *Super, const int64_t *Pi)
{
    const int s = t->s, nscol = (int)(Super[s + 1] - Super[s]), nsrow = (int)(Pi[s + 1] - Pi[s]);
    double *F = front[s];
    const int ld = nsrow;
    if (!F) return;
    if (t->type == GB_DT_POTRF) {
        const int c0 = 64 * t->b;
        chol_block(F, ld, c0, imin(64, nscol - c0));
    } else if (t->type == GB_DT_TRSM) {
        const int c0 = 64 * t->b, nb = imin(64, nscol - c0);
        solve_rows(F, ld, imax(64 * t->r, c0 + nb), imin(64 * t->r + 64, nsrow), c0, nb);
    } else if (t->type == GB_DT_UPD) {
        const int nbk = imax(1, t->nbk), cs = 64 * t->c;
        update(F, ld, imax(64 * t->r, cs), imin(64 * t->r + 64, nsrow), cs, imin(cs + 64, nscol),
               64 * t->b, imin(64 * (t->b + nbk), nscol), t->r == t->c);
    } else if (t->type == GB_DT_DIAG) {
        const gb_dtask a = {GB_DT_TRSM, t->s, t->b - 1, t->b, 0, 0, 0, 0};
        const gb_dtask b = {GB_DT_UPD, t->s, t->r, t->b, t->b, 0, t->nbk, 0};
        const gb_dtask c = {GB_DT_POTRF, t->s, t->b, 0, 0, 0, 0, 0};
        run_task(&a, front, Super, Pi);
        run_task(&b, front, Super, Pi);
        run_task(&c, front, Super, Pi);
    } else if (t->type == GB_DT_CB && t->b == 1) {
        update(F, ld, imax(64 * t->r, nscol), imin(64 * t->r + 64, nsrow), imax(64 * t->c, nscol),
               imin(64 * t->c + 64, nsrow), 0, nscol, t->r == t->c);
    }
}

int main(int argc, char **argv)
{
    if (argc < 4) return 2;
    size_t np, ni, nperm;
    int64_t *Ap = read_all(argv[1], &np), *Ai = read_all(argv[2], &ni), *perm = read_all(argv[3], &nperm);
    if (!Ap || !Ai || !perm) return 2;
    const int64_t n = (int64_t)nperm;
    cholmod_common c;
    memset(&c, 0, sizeof c);
    gb300_start(&c);
    cholmod_sparse *A = gb300_allocate_sparse(n, n, ni, 1, 1, -1, CHOLMOD_REAL, &c);
    memcpy(A->p, Ap, 8 * np);
    memcpy(A->i, Ai, 8 * ni);
    for (size_t q = 0; q < ni; q++) ((double *)A->x)[q] = 1.0;
    cholmod_factor *L = gb300_analyze_perm(A, perm, &c);
    if (!L) { printf("analysis failed\n"); return 2; }
    const int64_t *Super = L->super, *Pi = L->pi;
    const int ns = (int)L->nsuper;
    int bad = 0;
    for (int G = 1; G <= 4; G++) {
        gb_plan *P = gb_plan_build(L, 64, 16e6, 64, G);
        if (!P) { printf("plan failed\n"); return 2; }
        const gb_dtask *dt = P->dag_t.p;
        const gb_dag_level *lv = P->dag_lv.p;
        const int32_t *sp = P->dag_sp.p, *succ = P->dag_succ.p;
        long ndiag = 0, ntask = 0;
        for (size_t l = 0; l < P->dag_lv.n; l++) {
            const int nt = lv[l].ntasks;
            if (!nt) continue;
            const gb_dtask *t = dt + lv[l].task_off;
            const int32_t *lsp = sp + lv[l].sp_off, *ls = succ + lv[l].succ_off;
            ntask += nt;
            for (int k = 0; k < nt; k++) ndiag += t[k].type == GB_DT_DIAG;
            for (int trial = 0; trial < 3; trial++) {
                double **front = calloc(ns, sizeof(double *)), **ref = calloc(ns, sizeof(double *));
                for (int k = 0; k < nt; k++) {
                    const int s = t[k].s;
                    if (front[s] || !(t[k].type == GB_DT_POTRF || t[k].type == GB_DT_DIAG)) continue;
                    const int m = (int)(Pi[s + 1] - Pi[s]), nscol = (int)(Super[s + 1] - Super[s]);
                    double *F = front[s] = calloc((size_t)m * m, sizeof(double));
                    const int ld = m;
                    for (int j = 0; j < m; j++)
                        for (int i = j; i < m; i++)
                            F_(i, j) = i == j ? m + 1.0 : ((double)(next_rand() % 1000) / 1000.0 - 0.5) / m;
                    ref[s] = malloc((size_t)m * m * sizeof(double));
                    memcpy(ref[s], F, (size_t)m * m * sizeof(double));
                    for (int c0 = 0; c0 < nscol; c0 += 64) {
                        const int nb = imin(64, nscol - c0);
                        chol_block(ref[s], m, c0, nb);
                        solve_rows(ref[s], m, c0 + nb, m, c0, nb);
                        update(ref[s], m, c0 + nb, m, c0 + nb, m, c0, c0 + nb, 1);
                    }
                }
                /* a DIAG task runs in two parts, as the executor runs it:
                 * its panel solve, then (after its early successors were
                 * released, so that they may run first) the update of the
                 * diagonal tile and the LL'; ready entries >= nt are the
                 * second parts of DIAG tasks k - nt */
                int *cnt = calloc(nt, sizeof(int)), *ready = malloc(sizeof(int) * 2 * nt), nr = 0, done = 0;
                for (int k = 0; k < nt; k++)
                    for (int e = lsp[k]; e < lsp[k + 1]; e++) cnt[ls[e]]++;
                for (int k = 0; k < nt; k++)
                    if (!cnt[k]) ready[nr++] = k;
                while (nr) {
                    const int pick = (int)(next_rand() % (uint64_t)nr), k = ready[pick];
                    ready[pick] = ready[--nr];
                    int e0 = 0, e1 = 0;
                    if (k < nt && t[k].type == GB_DT_DIAG) {
                        const gb_dtask a = {GB_DT_TRSM, t[k].s, t[k].b - 1, t[k].b, 0, 0, 0, 0};
                        run_task(&a, front, Super, Pi);
                        e0 = lsp[k];
                        e1 = lsp[k] + t[k].pad1;
                        ready[nr++] = nt + k;
                    } else if (k >= nt) {
                        const int d = k - nt;
                        const gb_dtask b = {GB_DT_UPD, t[d].s, t[d].r, t[d].b, t[d].b, 0, t[d].nbk, 0};
                        const gb_dtask c = {GB_DT_POTRF, t[d].s, t[d].b, 0, 0, 0, 0, 0};
                        run_task(&b, front, Super, Pi);
                        run_task(&c, front, Super, Pi);
                        e0 = lsp[d] + t[d].pad1;
                        e1 = lsp[d + 1];
                        done++;
                    } else {
                        run_task(&t[k], front, Super, Pi);
                        e0 = lsp[k];
                        e1 = lsp[k + 1];
                        done++;
                    }
                    for (int e = e0; e < e1; e++)
                        if (--cnt[ls[e]] == 0) ready[nr++] = ls[e];
                }
                if (done != nt) {
                    printf("group %d level %zu: cycle (%d of %d tasks ran)\n", G, l, done, nt);
                    bad = 1;
                }
                for (int s = 0; s < ns; s++) {
                    if (!front[s]) continue;
                    const int m = (int)(Pi[s + 1] - Pi[s]);
                    double e = 0, nrm = 0;
                    for (size_t q = 0; q < (size_t)m * m; q++) {
                        const double d = front[s][q] - ref[s][q];
                        e += d * d;
                        nrm += ref[s][q] * ref[s][q];
                    }
                    if (!(sqrt(e / nrm) <= 1e-13)) {
                        printf("group %d supernode %d (%d rows): relative error %.3e\n", G, s, m, sqrt(e / nrm));
                        bad = 1;
                    }
                    free(front[s]);
                    free(ref[s]);
                }
                free(front); free(ref); free(cnt); free(ready);
            }
        }
        printf("group %d: %ld tile tasks, %ld DIAG\n", G, ntask, ndiag);
        gb_plan_free(P);
    }
    printf(bad ? "FAIL\n" : "OK\n");
    return bad;
}
