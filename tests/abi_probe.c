/* Prints offsetof / sizeof of the CHOLMOD objects as the reference's own
 * cholmod.h lays them out (compiled by tests/test_abi.py against the
 * reference include directory, when present). */
#include <stdio.h>
#include <stddef.h>
#include "cholmod.h"
#include "gb_abi_fields.h"

#define P(T, f) printf("%s %s %ld\n", #T, #f, (long)offsetof(T, f));

int main(void)
{
#define X(f) P(cholmod_common, f)
    GB_ABI_COMMON_FIELDS(X)
#undef X
#define X(f) P(cholmod_sparse, f)
    GB_ABI_SPARSE_FIELDS(X)
#undef X
#define X(f) P(cholmod_factor, f)
    GB_ABI_FACTOR_FIELDS(X)
#undef X
#define X(f) P(cholmod_dense, f)
    GB_ABI_DENSE_FIELDS(X)
#undef X
    printf("sizeof cholmod_common %ld\n", (long)sizeof(cholmod_common));
    printf("sizeof cholmod_sparse %ld\n", (long)sizeof(cholmod_sparse));
    printf("sizeof cholmod_factor %ld\n", (long)sizeof(cholmod_factor));
    printf("sizeof cholmod_dense %ld\n", (long)sizeof(cholmod_dense));
    return 0;
}
