/* gb_abi.c -- layout of the CHOLMOD objects as this library compiles them.
 *
 * gb300_abi_offset(object, field) returns offsetof(object, field) (or -1),
 * gb300_abi_sizeof(object) returns sizeof(object); object 0 = cholmod_common,
 * 1 = cholmod_sparse, 2 = cholmod_factor, 3 = cholmod_dense.  Used by the
 * Python bindings to address fields of cholmod_common, and by the ABI test
 * that compares every offset with the reference's cholmod.h.
 */
#include "gb_internal.h"
#include "gb_abi_fields.h"
#include <string.h>

#define GB_OFF(T, f) if (!strcmp(field, #f)) return (long)offsetof(T, f);

long gb300_abi_offset(int object, const char *field)
{
    if (!field) return -1;
    switch (object) {
    case 0:
#define X(f) GB_OFF(cholmod_common, f)
        GB_ABI_COMMON_FIELDS(X)
#undef X
        break;
    case 1:
#define X(f) GB_OFF(cholmod_sparse, f)
        GB_ABI_SPARSE_FIELDS(X)
#undef X
        break;
    case 2:
#define X(f) GB_OFF(cholmod_factor, f)
        GB_ABI_FACTOR_FIELDS(X)
#undef X
        break;
    case 3:
#define X(f) GB_OFF(cholmod_dense, f)
        GB_ABI_DENSE_FIELDS(X)
#undef X
        break;
    }
    return -1;
}

long gb300_abi_sizeof(int object)
{
    switch (object) {
    case 0: return (long)sizeof(cholmod_common);
    case 1: return (long)sizeof(cholmod_sparse);
    case 2: return (long)sizeof(cholmod_factor);
    case 3: return (long)sizeof(cholmod_dense);
    }
    return -1;
}
