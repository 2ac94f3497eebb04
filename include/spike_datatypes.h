/*
 * spike_datatypes.h -- scalar and status types of the SPIKE C API.
 *
 * Mirrors the types the reference exposes in OpenMP/spike_datatypes.h:86-107
 * (integer_t = int, Error_t = int, SPIKE_SUCCESS = 0, SPIKE_ERROR = 1) so that
 * code compiled against the reference headers links against this library
 * unchanged.  The reference picks its scalar type at compile time with
 * -D_DATATYPE_{S,D,C,Z}_; here the four typed entry points of
 * spike_interfaces.h carry the type instead, so no macro is needed.
 *
 * SPIKE_SUCCESS / SPIKE_ERROR are exported both as the const objects the
 * reference declares (OpenMP/spike_datatypes.h:103-104, defined in
 * OpenMP/spike_datatypes.c:43-44) and as enum-free macros of the same value
 * for callers that want a constant expression.
 */
#ifndef SPIKE_GB300_DATATYPES_H
#define SPIKE_GB300_DATATYPES_H

#include <stdint.h>
#include <stdlib.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef int      integer_t;
typedef int      Error_t;
typedef int      Bool_t;
typedef double   spike_timer_t;
typedef uint64_t uLong_t;

/* Exported objects with the reference's names and values. */
extern const Error_t SPIKE_SUCCESS;
extern const Error_t SPIKE_ERROR;

#define SPIKE_SUCCESS_VALUE 0
#define SPIKE_ERROR_VALUE   1

#ifdef __cplusplus
}
#endif

#endif /* SPIKE_GB300_DATATYPES_H */
