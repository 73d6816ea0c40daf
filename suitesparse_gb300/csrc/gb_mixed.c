/* gb_mixed.c -- FP32 factor + FP64 iterative refinement (filled in below). */
#include "gb_plan.h"

int gb300_factorize_mixed(cholmod_sparse *A, cholmod_factor *L, cholmod_common *Common)
{
    (void)A; (void)L;
    if (!Common) return FALSE;
    GB_ERROR(CHOLMOD_NOT_INSTALLED, "mixed precision path not built");
    return FALSE;
}

cholmod_dense *gb300_solve_refined(cholmod_sparse *A, cholmod_factor *L, cholmod_dense *B,
                                   double tol, double *info, cholmod_common *Common)
{
    (void)A; (void)L; (void)B; (void)tol; (void)info;
    if (!Common) return NULL;
    GB_ERROR(CHOLMOD_NOT_INSTALLED, "mixed precision path not built");
    return NULL;
}
