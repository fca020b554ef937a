/*
 * coupe.h — the C ABI of libcoupe_gpu.so for recursive coordinate and
 * inertial bisection.
 *
 * The enums, the data-set constructors and coupe_rcb / coupe_rib keep the
 * names, numeric values and signatures of coupe's own C header
 * (coupe-ffi/include/coupe.h), so that a program built against coupe's
 * libcoupe.so for these entry points links and runs against this library
 * unchanged.  Only the geometric bisection entry points are provided; the
 * other algorithms of coupe (Hilbert, greedy, Karmarkar-Karp,
 * Fiduccia-Mattheyses, adjacency structures) are not part of this library.
 */
#ifndef COUPE_H
#define COUPE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Error codes.  Values follow coupe-ffi/include/coupe.h:16-57 and
 * coupe-ffi/src/lib.rs:35-46. */
enum coupe_err {
	COUPE_ERR_OK,            /* success */
	COUPE_ERR_ALLOC,         /* host or device allocation failed */
	COUPE_ERR_CRASH,         /* internal error (a CUDA call failed, a device check tripped) */
	COUPE_ERR_BAD_DIMENSION, /* dimension is not 2 or 3 */
	COUPE_ERR_BAD_TYPE,      /* unsupported element type or value */
	COUPE_ERR_BIPART_ONLY,   /* kept for ABI compatibility; never returned here */
	COUPE_ERR_LEN_MISMATCH,  /* points and weights differ in length */
	COUPE_ERR_NOT_FOUND,     /* never returned by rcb/rib; multi_jagged: no partition scheme */
	COUPE_ERR_NEG_VALUES,    /* never returned by rcb/rib; multi_jagged: a negative weight */
};

/* Static, NUL-terminated message for an error code.
 * Replaces coupe_strerror (coupe-ffi/src/lib.rs:69-110). */
const char *coupe_strerror(enum coupe_err err);

/* Element types of a data set.  Values follow coupe-ffi/include/coupe.h:86-93
 * and coupe-ffi/src/data.rs:11-17. */
enum coupe_type {
	COUPE_INT,    /* int (32-bit, sums wrap at 32 bits) */
	COUPE_INT64,  /* int64_t (sums wrap at 64 bits) */
	COUPE_DOUBLE, /* double */
};

/* An opaque data set: an array, a repeated constant or a callback. */
typedef struct coupe_data coupe_data;

/* Frees a data set (NULL is allowed); never frees the memory it refers to.
 * Replaces coupe_data_free (coupe-ffi/src/lib.rs:112-120). */
void coupe_data_free(coupe_data *data);

/* A data set over `len` contiguous elements of `type` at `data` (for points:
 * `len` points of `dimension` doubles each, whatever `type` says, as in
 * coupe).  The array must outlive the data set.  Returns NULL on allocation
 * failure.  Replaces coupe_data_array (coupe-ffi/src/lib.rs:122-129). */
coupe_data *coupe_data_array(uintptr_t len, enum coupe_type type, const void *data);

/* A data set repeating `*value` `len` times.  Replaces coupe_data_constant
 * (coupe-ffi/src/lib.rs:131-138). */
coupe_data *coupe_data_constant(uintptr_t len, enum coupe_type type, const void *value);

/* A data set whose element i is `*i_th(context, i)`.  The callback may be
 * called in any order, more than once per index, and from several threads.
 * Replaces coupe_data_fn (coupe-ffi/src/lib.rs:140-157). */
coupe_data *coupe_data_fn(const void *context, uintptr_t len, enum coupe_type type,
		const void *(*i_th)(const void *, uintptr_t));

/* Recursive coordinate bisection into at most 2^iter_count parts.
 * `partition` receives one part id per point (ids start at zero).
 * Errors: COUPE_ERR_LEN_MISMATCH when the data sets differ in length (checked
 * first), COUPE_ERR_BAD_DIMENSION unless dimension is 2 or 3.  With integer
 * weights the ids are identical to coupe::Rcb's.
 * Replaces coupe_rcb (coupe-ffi/src/lib.rs:272-304,
 * coupe-ffi/include/coupe.h:278-280). */
enum coupe_err coupe_rcb(uintptr_t *partition, uintptr_t dimension,
		const coupe_data *points, const coupe_data *weights,
		uintptr_t iter_count, double tolerance);

/* Recursive inertial bisection: the points are first expressed in a basis
 * whose first axis is their principal inertia axis, then bisected as
 * coupe_rcb does.  Replaces coupe_rib (coupe-ffi/src/lib.rs:332-364,
 * coupe-ffi/include/coupe.h:294-296). */
enum coupe_err coupe_rib(uintptr_t *partition, uintptr_t dimension,
		const coupe_data *points, const coupe_data *weights,
		uintptr_t iter_count, double tolerance);

#ifdef __cplusplus
}
#endif

#endif /* COUPE_H */
