/* Autotuner of the factorization's plan options.
 *
 * Three options shape the task graph of a pattern: the small/large
 * supernode cutoff (GB300_OPT_SMALL_COLS: supernodes at most this wide are
 * factorized whole by one thread block, wider ones by 64 x 64 tile tasks),
 * the subtree work limit (GB300_OPT_SUBTREE_WORK: subtrees of small
 * supernodes up to this estimated work run as one task) and the depth of
 * the wide supernodes' trailing tile products (GB300_OPT_UPD_GROUP: the
 * updates of g panels run as one 64 x 64 x 64 g product).  The best values
 * depend on the pattern: a batch of small grids wants large subtrees, a 3D
 * separator tree wants more parallel tasks, a wide supernode deep products.
 *
 * gb300_autotune times the factorization of one matrix under each
 * candidate (the device time of the library's own CUDA events around the
 * factorization launch, median of a few repetitions after a warm-up that
 * builds the candidate's plan), leaves the fastest candidate set on the
 * cholmod_common and returns its index.  With GB300_OPT_AUTOTUNE set, the
 * first cholmod_l_super_numeric of a Common runs the same tuning on its own
 * input before it factorizes, so that a program that only calls the
 * CHOLMOD API gets tuned options. */
#include <stdlib.h>
#include <string.h>

#include "cholmod_gb300.h"
#include "gb_internal.h"
#include "gb_plan.h"

#define NOPT 3
static const int tune_opts[NOPT] = {GB300_OPT_SMALL_COLS, GB300_OPT_SUBTREE_WORK,
                                    GB300_OPT_UPD_GROUP};

/* (small cutoff, subtree work limit, update group) */
static const int64_t default_cand[][NOPT] = {
    {64, 4000000, 4}, {64, 16000000, 4}, {64, 1000000, 4}, {64, 0, 4},
    {32, 4000000, 4}, {16, 4000000, 4}, {64, 16000000, 2}, {64, 16000000, 1},
};
#define NDEFAULT ((int)(sizeof default_cand / sizeof default_cand[0]))

int gb300_autotune_candidates(int64_t *cand, int ncand)
{
    for (int i = 0; cand && i < ncand && i < NDEFAULT; i++)
        for (int k = 0; k < NOPT; k++) cand[NOPT * i + k] = default_cand[i][k];
    return NDEFAULT;
}

int64_t gb300_get_option(cholmod_common *Common, int option)
{
    return Common ? gb_option(Common, option) : 0;
}

typedef struct {
    cholmod_sparse *A, *F;
    double *beta;
    cholmod_factor *L;
    int mixed;            /* 0 FP64 factor of A, 1 mixed form, 2 super_numeric of (A, F, beta) */
} tune_case;

/* one factorization of the case; its device time from the library's events */
static double tune_timer(cholmod_common *Common, void *ud)
{
    tune_case *t = ud;
    int ok;
    if (t->mixed == 2) ok = gb_super_numeric(t->A, t->F, t->beta, t->L, Common);
    else if (t->mixed) ok = gb300_factorize_mixed(t->A, t->L, Common);
    else ok = gb300_factorize(t->A, NULL, t->L, Common);
    if (!ok) return -1.0;
    double st[8];
    gb300_get_stats(Common, st, 8);
    return st[0];
}

static int cmp_double(const void *a, const void *b)
{
    double x = *(const double *)a, y = *(const double *)b;
    return (x > y) - (x < y);
}

int gb300_autotune_with(const int64_t *cand, int ncand, int reps, double *ms,
                        gb300_tune_timer timer, void *ud, cholmod_common *Common)
{
    if (!Common) return -1;
    if (!cand) { cand = &default_cand[0][0]; ncand = NDEFAULT; }
    if (ncand < 1 || !timer) { GB_ERROR(CHOLMOD_INVALID, "no candidates"); return -1; }
    if (reps < 1) reps = 1;
    if (reps > 15) reps = 15;
    int64_t keep[NOPT];
    for (int k = 0; k < NOPT; k++) keep[k] = gb_option(Common, tune_opts[k]);
    int best = -1;
    double best_ms = 0, t[15];
    for (int i = 0; i < ncand; i++) {
        for (int k = 0; k < NOPT; k++) gb300_set_option(Common, tune_opts[k], cand[NOPT * i + k]);
        if (timer(Common, ud) < 0) { best = -1; break; }    /* warm-up: builds the plan */
        int r = 0;
        for (; r < reps; r++) {
            t[r] = timer(Common, ud);
            if (t[r] < 0) break;
        }
        if (r < reps) { best = -1; break; }
        qsort(t, reps, sizeof(double), cmp_double);
        double med = reps % 2 ? t[reps / 2] : 0.5 * (t[reps / 2 - 1] + t[reps / 2]);
        if (ms) ms[i] = med;
        if (best < 0 || med < best_ms) { best = i; best_ms = med; }
    }
    if (best < 0) {
        /* a failed factorization ends the tuning; the options are restored */
        for (int k = 0; k < NOPT; k++) gb300_set_option(Common, tune_opts[k], keep[k]);
        return -1;
    }
    for (int k = 0; k < NOPT; k++) gb300_set_option(Common, tune_opts[k], cand[NOPT * best + k]);
    return best;
}

int gb300_autotune(cholmod_sparse *A, cholmod_factor *L, int mixed, int reps,
                   const int64_t *cand, int ncand, double *ms, cholmod_common *Common)
{
    if (!Common) return -1;
    if (!A || !L) { GB_ERROR(CHOLMOD_INVALID, "argument missing"); return -1; }
    tune_case tc = {A, NULL, NULL, L, mixed ? 1 : 0};
    return gb300_autotune_with(cand, ncand, reps, ms, tune_timer, &tc, Common);
}

/* GB300_OPT_AUTOTUNE: tune on the first super_numeric call of the Common
 * (S, F, beta as that call got them; the call itself then factorizes with
 * the chosen options). */
void gb_autotune_first(cholmod_sparse *A, cholmod_sparse *F, double beta[2],
                       cholmod_factor *L, cholmod_common *Common)
{
    gb_ctx *ctx = gb_ctx_get(Common, 0);
    if (!ctx || !ctx->opt_autotune || ctx->tuned) return;
    ctx->tuned = 1;
    tune_case tc = {A, F, beta, L, 2};
    int status = Common->status;
    gb300_autotune_with(NULL, 0, 1, NULL, tune_timer, &tc, Common);
    Common->status = status;
}
