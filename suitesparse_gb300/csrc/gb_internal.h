/* gb_internal.h -- shared declarations of the host side of libcholmod_gb300.
 *
 * The host side is C: object bookkeeping (gb_util.c), the supernodal
 * symbolic analysis (gb_symbolic.c), the per-pattern GPU plan (gb_plan.c)
 * and the drivers of the numeric factorization and solves (gb_numeric.c).
 * Kernels live in gb_kernels.cu and are reached through the launchers
 * declared at the end of this file (plain pointers, extern "C").
 */
#ifndef GB_INTERNAL_H
#define GB_INTERNAL_H

#include "cholmod_gb300.h"
#include <stdint.h>
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef int64_t Int;
#define EMPTY (-1)
#ifndef TRUE
#define TRUE 1
#define FALSE 0
#endif
#define GB_MAX(a, b) ((a) > (b) ? (a) : (b))
#define GB_MIN(a, b) ((a) < (b) ? (a) : (b))

/* ---- gb_util.c ---------------------------------------------------------- */
void *gb_malloc(size_t n, size_t size, cholmod_common *Common);
void *gb_calloc(size_t n, size_t size, cholmod_common *Common);
void *gb_free(size_t n, size_t size, void *p, cholmod_common *Common);
/* CHOLMOD-style error report: sets Common->status, calls the handler. */
void gb_error(int status, const char *file, int line, const char *msg,
              cholmod_common *Common);
#define GB_ERROR(status, msg) gb_error(status, __FILE__, __LINE__, msg, Common)

/* Per-Common library state (options, device context, statistics). */
typedef struct gb_ctx gb_ctx;
gb_ctx *gb_ctx_get(cholmod_common *Common, int create);
int64_t gb_option(cholmod_common *Common, int option);
void gb_autotune_first(cholmod_sparse *A, cholmod_sparse *F, double beta[2],
                       cholmod_factor *L, cholmod_common *Common);

/* ---- gb_symbolic.c ------------------------------------------------------- */
/* Supernodal symbolic analysis of the lower-stored A permuted by Perm. */
cholmod_factor *gb_analyze_perm(cholmod_sparse *A, const Int *Perm,
                                cholmod_common *Common);
/* S = tril(A(p,p)) in sorted CSC (double values); caller frees with gb_free. */
cholmod_sparse *gb_permute_lower(cholmod_sparse *A, const Int *Perm,
                                 cholmod_common *Common);

/* ---- gb_numeric.c: the bodies of the int64 entry points ------------------ */
int gb_super_numeric(cholmod_sparse *A, cholmod_sparse *F, double beta[2], cholmod_factor *L,
                     cholmod_common *Common);
int gb_super_solve(cholmod_factor *L, cholmod_dense *X, cholmod_dense *E, cholmod_common *Common,
                   int forward);

/* drop the device state (plan, device factor) attached to L */
int gb_release_factor_state(cholmod_factor *L);

/* ---- gb_int32.c ---------------------------------------------------------- */
/* drop the int64 shadow (and its device state) of an int32 factor */
int gb_release_int32_shadow(const cholmod_factor *L);
/* ---- gb_aft.c ------------------------------------------------------------ */
cholmod_sparse *gb_aft_pattern(cholmod_sparse *A, cholmod_sparse *F, int64_t **pptr_out,
                               int64_t **pairs_out, cholmod_common *Common);

/* ---- gb_simplicial.c ----------------------------------------------------- */
int gb_release_simplicial_shadow(const cholmod_factor *L);

/* ---- gb_complex.c -------------------------------------------------------- */
/* complex (or zomplex input) supernodal LL' and sweeps through the real
 * embedding of the factor */
int gb_super_numeric_complex(cholmod_sparse *A, cholmod_sparse *F, double beta[2],
                             cholmod_factor *L, cholmod_common *Common);
int gb_super_solve_complex(cholmod_factor *L, cholmod_dense *X, cholmod_dense *E,
                           cholmod_common *Common, int forward);
int gb_release_complex_shadow(const cholmod_factor *L);

/* ---- kernel launchers (gb_kernels.cu) ------------------------------------ */
/* Every launcher enqueues on `stream` and returns a cudaError_t as int. */

#ifdef __cplusplus
}
#endif

#endif
