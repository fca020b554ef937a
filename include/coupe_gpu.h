/*
 * coupe_gpu.h — entry points of libcoupe_gpu.so beyond coupe's own ABI.
 *
 * coupe.h covers the drop-in calls.  The functions here add what a GPU
 * caller needs and the reference has no counterpart for: device-resident
 * inputs, the choice of key precision, run statistics and the detailed
 * message of the last error on the calling thread.
 */
#ifndef COUPE_GPU_H
#define COUPE_GPU_H

#include <stdint.h>
#include "coupe.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Key precision of the split search.
 * COUPE_GPU_REF32: coupe's arithmetic — f32 keys, f32 cuts, f32 distances
 *   (coupe/src/algorithms/recursive_bisection.rs:472-555, 604-616, 674-679).
 *   Part ids equal coupe::Rcb's for integer weights.  Default of coupe_rcb.
 * COUPE_GPU_F64: the same algorithm with f64 keys, cuts and split positions.
 * COUPE_GPU_F32KEY_F64BAND: f32 keys streamed, with every comparison whose
 *   f32 key cannot decide it re-checked in f64; the result equals
 *   COUPE_GPU_F64's. */
enum coupe_gpu_mode {
	COUPE_GPU_REF32 = 0,
	COUPE_GPU_F64 = 1,
	COUPE_GPU_F32KEY_F64BAND = 2,
};

/* Statistics of the last run on the calling thread. */
struct coupe_gpu_stats {
	uint64_t points;          /* N */
	uint64_t levels;          /* tree levels processed */
	uint64_t splits;          /* non-empty segments split */
	uint64_t split_steps;     /* bisection steps, summed over splits */
	uint64_t max_split_steps; /* most steps of one split */
	uint64_t hist_passes;     /* histogram passes launched */
	uint64_t hist_points;     /* points read by histogram passes */
	uint64_t band_points;     /* f64 coordinates read by histogram passes (band mode) */
	uint64_t kernel_launches; /* kernels launched by the run */
	uint64_t algo_bytes;      /* algorithmic HBM bytes of the run */
	double root_weight_sum;   /* total weight as f64 */
	double device_ms;         /* device time of the run (CUDA events) */
	int fixed_scale;          /* s of the 128-bit fixed-point weight sums */
	int mode;                 /* enum coupe_gpu_mode used */
	uint64_t weight_rechecks; /* f64 weights: decisions replayed with exact bins */
	/* Bound on |root_weight_sum - the exact sum of the weights|: f64
	 * weights are quantised to multiples of 2^-fixed_scale (at most half a
	 * quantum each) and the exact fixed-point total is rounded once to f64;
	 * 0 for integer weights (exact, wrapping sums). */
	double weight_sum_error_bound;
	uint64_t host_syncs;      /* host synchronisations of the level loop */
};

/* coupe_rcb with an explicit precision mode. */
enum coupe_err coupe_gpu_rcb(uintptr_t *partition, uintptr_t dimension,
		const coupe_data *points, const coupe_data *weights,
		uintptr_t iter_count, double tolerance, int mode);

/* coupe_rib with an explicit precision mode. */
enum coupe_err coupe_gpu_rib(uintptr_t *partition, uintptr_t dimension,
		const coupe_data *points, const coupe_data *weights,
		uintptr_t iter_count, double tolerance, int mode);

/* Rcb on device-resident inputs: `d_points` holds n points of `dimension`
 * doubles (AoS, 8-byte aligned), `d_weights` n elements of `weight_type`,
 * `d_partition` receives n part ids.  `stream` is a cudaStream_t (NULL: the
 * library's own stream); the call returns after the work on it completed.
 * `matrix` (host, dimension x dimension, row-major) may be NULL; when given,
 * every point p is replaced by matrix * p before the bisection, which is how
 * Rib applies its basis change. */
enum coupe_err coupe_gpu_rcb_device(uint64_t *d_partition, uint64_t n, uint64_t dimension,
		const double *d_points, enum coupe_type weight_type, const void *d_weights,
		uint64_t iter_count, double tolerance, int mode, const double *matrix,
		void *stream);

/* Batched Rcb on device-resident inputs: `nsets` independent point sets of
 * one dimension partitioned in one run (no counterpart in the reference; the
 * same result as one coupe_gpu_rcb_device call per set).  Set k is points
 * [set_offsets[k], set_offsets[k + 1]) of `d_points` / `d_weights` /
 * `d_partition` and is split into at most 2^iter_counts[k] parts; its ids
 * start at 0 like a run of that set alone.  `set_offsets` (nsets + 1
 * entries, starting at 0, non-decreasing) and `iter_counts` (nsets entries)
 * are host arrays.  Empty sets are allowed; a set with iter_count 0 gets id
 * 0 everywhere.  Limits: 2^32 - 1 points in all, at most 63 levels, and at
 * most 2^22 splits over all sets (else COUPE_ERR_ALLOC).  Returns after the
 * work on `stream` completed. */
enum coupe_err coupe_gpu_rcb_batched(uint64_t *d_partition, uint64_t nsets,
		const uint64_t *set_offsets, uint64_t dimension, const double *d_points,
		enum coupe_type weight_type, const void *d_weights,
		const uint32_t *iter_counts, double tolerance, int mode, void *stream);

/* Flag OR'ed into the mode of coupe_gpu_rib / coupe_gpu_rib_device (no
 * counterpart in the reference): the Rib inertia matrix weighs each point by
 * its weight — centroid sum(w p) / sum(w), M = sum(w (p - c)(p - c)^T).
 * coupe's inertia_matrix is unweighted (coupe/src/geometry.rs:273-284) and
 * stays the default.  The weights must have a positive finite sum, else
 * COUPE_ERR_BAD_TYPE. */
#define COUPE_GPU_WEIGHTED_INERTIA 0x100

/* Rib on device-resident inputs (see coupe_gpu_rcb_device). */
enum coupe_err coupe_gpu_rib_device(uint64_t *d_partition, uint64_t n, uint64_t dimension,
		const double *d_points, enum coupe_type weight_type, const void *d_weights,
		uint64_t iter_count, double tolerance, int mode, void *stream);

/* The Rib basis change of n device-resident points: writes obb_to_aabb
 * (host, dimension x dimension, row-major), the inverse of the Householder
 * reflection that maps the first axis onto the principal inertia axis
 * (coupe/src/geometry.rs:210-228, 273-319). */
enum coupe_err coupe_gpu_rib_matrix(uint64_t n, uint64_t dimension, const double *d_points,
		double *obb_to_aabb, void *stream);

/* The same with the weighted inertia matrix of COUPE_GPU_WEIGHTED_INERTIA
 * (no counterpart in the reference): `d_weights` holds n device-resident
 * elements of `weight_type`. */
enum coupe_err coupe_gpu_rib_matrix_weighted(uint64_t n, uint64_t dimension, const double *d_points,
		enum coupe_type weight_type, const void *d_weights, double *obb_to_aabb, void *stream);

/* The engine's f64 -> f32 key conversion (coupe's `point[coord] as f32`,
 * coupe/src/algorithms/recursive_bisection.rs:677) applied to n device
 * values, so that callers can check it against IEEE round-to-nearest-even.
 * The engine computes it with integer instructions. */
enum coupe_err coupe_gpu_f64_to_f32(const double *d_in, float *d_out, uint64_t n, void *stream);

/* Load of each part of a partition: loads[p] is the sum of the weights of
 * the points i with partition[i] == p, for p < num_parts
 * (coupe::imbalance::compute_parts_load, coupe/src/imbalance.rs:14-39).
 * `loads` (host) receives num_parts elements of the weights' type: c_int
 * and int64 loads wrap around like coupe's release build; double loads are
 * the exact sums (128-bit fixed point) rounded once.  Errors:
 * COUPE_ERR_BAD_TYPE for a part id >= num_parts (coupe panics) or a
 * non-finite double weight. */
enum coupe_err coupe_gpu_parts_load(const uintptr_t *partition, uintptr_t num_parts,
		const coupe_data *weights, void *loads);

/* coupe::imbalance::imbalance (coupe/src/imbalance.rs:41-77): the largest
 * (load - ideal) / ideal over the parts, ideal = total weight / num_parts;
 * 0 when num_parts is 0 or the ideal load is 0.  `partition` holds
 * weights->len part ids.  Errors as coupe_gpu_parts_load. */
enum coupe_err coupe_gpu_imbalance(uintptr_t num_parts, const uintptr_t *partition,
		const coupe_data *weights, double *imbalance);

/* Rcb on a cartesian grid (coupe::Grid::rcb, coupe/src/cartesian/mod.rs:
 * 130-179, cartesian/rcb.rs:52-281): `size` holds `dimension` (2 or 3) cell
 * counts; cell (x, y[, z]) is weight and partition entry
 * x + size[0] * (y + size[1] * z).  Splits start on axis 1 and cycle; each
 * is coupe's weighted median of the slab weights, which replays rayon's
 * fold_chunks with `threads` workers: pass the size of the rayon pool whose
 * result is to be reproduced (>= 2; with one worker coupe's search never
 * ends, and COUPE_ERR_BAD_TYPE is returned).  Ids are in
 * [0, 2^iter_count).  Integer weights wrap like coupe's release build; the
 * total of double weights is their exact sum rounded once (coupe's rayon
 * sum has no fixed order).  Errors: COUPE_ERR_BAD_DIMENSION for a dimension
 * other than 2 or 3 or a zero size, COUPE_ERR_LEN_MISMATCH unless the
 * weights hold one value per cell, COUPE_ERR_BAD_TYPE for a non-finite
 * double weight. */
enum coupe_err coupe_gpu_grid_rcb(uintptr_t *partition, uintptr_t dimension, const uintptr_t *size,
		const coupe_data *weights, uintptr_t iter_count, uintptr_t threads);
enum coupe_err coupe_gpu_grid_rcb_device(uint64_t *d_partition, uint64_t dimension, const uint64_t *size,
		enum coupe_type weight_type, const void *d_weights, uint64_t iter_count, uint64_t threads,
		void *stream);

/* coupe's axis_sort (coupe/src/algorithms/recursive_bisection.rs:815-827,
 * the sort MultiJagged applies per iteration): d_permutation gets 0..n-1
 * ordered by coordinate `coord` of the n device points (n x dimension
 * doubles).  coupe's sort is unstable; this one keeps equal coordinates in
 * index order (-0.0 sorts before +0.0), so results equal coupe's wherever
 * the coordinates are distinct.  dimension 1..64 and coord < dimension, else
 * COUPE_ERR_BAD_DIMENSION.  Returns after the work on `stream` completed. */
enum coupe_err coupe_gpu_axis_sort_device(uint64_t *d_permutation, uint64_t n, uint64_t dimension,
		const double *d_points, uint64_t coord, void *stream);

/* MultiJagged (coupe::MultiJagged, coupe/src/algorithms/multi_jagged.rs:
 * 150-295, 368-385; coupe-ffi has no binding for it): part_count parts in at
 * most max_iter iterations following coupe's partition scheme; iteration k
 * sorts every part along axis k % dimension and cuts it at the running
 * weights total * modifier, a cut moving past every point whose running
 * weight is within 4 ulps of the threshold.  Part ids are numbered as coupe
 * numbers them with one rayon worker (depth first).  Running weights are the
 * exact sums of the sorted weights rounded once (coupe's are sequential f64
 * sums of rayon chunks), so a cut can differ from coupe's only where these
 * differ in the last bits.  Weights: double, finite and non-negative
 * (COUPE_ERR_BAD_TYPE, COUPE_ERR_NEG_VALUES; coupe does not check).
 * Errors: COUPE_ERR_LEN_MISMATCH, COUPE_ERR_BAD_DIMENSION (dimension 1..64),
 * COUPE_ERR_BAD_TYPE for part_count 0, COUPE_ERR_NOT_FOUND when no scheme of
 * part_count parts in max_iter iterations exists (coupe panics),
 * COUPE_ERR_ALLOC for n >= 2^32 or part_count > 2^24. */
enum coupe_err coupe_gpu_multi_jagged(uintptr_t *partition, uintptr_t dimension, const coupe_data *points,
		const coupe_data *weights, uintptr_t part_count, uintptr_t max_iter);
enum coupe_err coupe_gpu_multi_jagged_device(uint64_t *d_partition, uint64_t n, uint64_t dimension,
		const double *d_points, const double *d_weights, uint64_t part_count, uint64_t max_iter,
		void *stream);

/* Barycentres of one block of mesh elements with the same node count
 * (mesh-part's points, tools/lib/lib.rs:511-539): element e's point is the
 * sum of the coordinates of its nodes d_nodes[e * nodes_per_element + j]
 * (0-based, in that order, from 0.0) divided by nodes_per_element.
 * Device arrays: d_coords (n_nodes x dimension doubles), d_nodes
 * (n_elements x nodes_per_element), d_out (n_elements x dimension).
 * dimension 2 or 3 (else COUPE_ERR_BAD_DIMENSION); nodes_per_element 2, 3,
 * 4 or 8 (else COUPE_ERR_BAD_TYPE); a node index >= n_nodes returns
 * COUPE_ERR_BAD_TYPE (coupe panics).  Returns after the work on `stream`
 * completed. */
enum coupe_err coupe_gpu_barycentres(uint64_t dimension, uint64_t n_nodes, const double *d_coords,
		uint64_t n_elements, uint64_t nodes_per_element, const uint64_t *d_nodes, double *d_out,
		void *stream);

/* Device-resident forms: n part ids in `d_partition`, n weights of
 * `weight_type` in `d_weights`; `loads` and `imbalance` are host memory.
 * Return after the work on `stream` completed. */
enum coupe_err coupe_gpu_parts_load_device(const uint64_t *d_partition, uint64_t n,
		enum coupe_type weight_type, const void *d_weights, uint64_t num_parts, void *loads,
		void *stream);
enum coupe_err coupe_gpu_imbalance_device(uint64_t num_parts, const uint64_t *d_partition,
		uint64_t n, enum coupe_type weight_type, const void *d_weights, double *imbalance,
		void *stream);

/* Stable split of one part of device-resident points by a cut, allocating
 * nothing.  No counterpart in the reference: coupe moves the points of a part
 * with an in-place, unstable partition inside Rcb
 * (coupe/src/algorithms/recursive_bisection.rs:122-181) and has no
 * allocation-free call.
 *
 * Meant for callers that must not allocate device memory once they are
 * running.  Examples: a mesh or particle code that works within a fixed
 * device-memory budget, or one that keeps its own kernels running on other
 * streams while it partitions.  cudaMalloc and cudaFree can synchronise the
 * whole device, and an allocation can fail once the budget is taken.  This
 * call uses no cudaMalloc/cudaFree, no pinned host memory and no library
 * allocator, and creates no stream or event.  Its only scratch is an
 * 8256-byte static device array inside the library.
 *
 * Moves the n points of `d_points` (AoS, `dimension` = 2 or 3 doubles each,
 * 8-byte aligned) and their n weights (`weight_type`) to `d_out_points` and
 * `d_out_weights`.  First come, in input order, the points with
 * point[coord] < cut (an IEEE comparison: a NaN coordinate or a NaN cut goes
 * right, -0 equals +0); then, in input order, all others.  *n_left (host
 * memory) receives the number of the former.  The outputs must not overlap
 * the inputs.  `stream` is a cudaStream_t (NULL: the default stream); the
 * call returns after its work on it completed.
 *
 * Limits: n <= 2^32 - 1; a larger n returns COUPE_ERR_ALLOC before touching
 * any memory.  The scratch holds 1024 per-chunk counts; chunks grow with n, so
 * no call needs more.  Each call clears the scratch words that must start at
 * zero before its kernels run.
 *
 * All calls on one device share the scratch.  Calls that overlap in time on
 * one device (from several threads, or on several streams) race and give
 * wrong results; serialise them.
 *
 * The first call on each device (with that device current) does a one-time
 * set-up: it looks up the scratch's device address with
 * cudaGetSymbolAddress and sets the kernels' shared-memory limit.  Every call
 * reads its result back and synchronises its stream, so no call can be made
 * while the stream is being captured.  The set-up is kept for the life of
 * the process: after cudaDeviceReset on a device, this entry point must not
 * be called on that device again.  A launch error left pending by the
 * caller's own earlier work is reported as such (COUPE_ERR_CRASH) before any
 * kernel of this call is launched. */
enum coupe_err coupe_gpu_split_noalloc(uint64_t n, uint64_t dimension,
		const double *d_points, enum coupe_type weight_type, const void *d_weights,
		uint64_t coord, double cut, double *d_out_points, void *d_out_weights,
		uint64_t *n_left, void *stream);

/* Copies the statistics of the calling thread's last run. */
void coupe_gpu_last_stats(struct coupe_gpu_stats *out);

/* Detailed message of the calling thread's last error ("" if none). */
const char *coupe_gpu_last_error(void);

/* Per-launch profiler of the calling device: enable != 0 turns it on, 0
 * off; both reset the totals.  When on, every kernel launch is bracketed by
 * CUDA events on its stream (small overhead). */
int coupe_gpu_profile(int enable);

/* Copies per-kernel totals since the last coupe_gpu_profile call: launches,
 * algorithmic bytes and milliseconds, for up to `capacity` kernel kinds.
 * Returns the number of kinds. */
int coupe_gpu_profile_read(uint64_t *counts, uint64_t *bytes, double *ms, int capacity);

/* Name of kernel kind `id` (as reported by coupe_gpu_profile_read). */
const char *coupe_gpu_kernel_name(int id);

/* Process-wide scheduling knobs; none of them changes a result.
 *   "force_index_path"        1: carry each point's input index through every
 *                             reorder instead of tracing the recorded splits
 *   "max_nbk"                 bisection steps per histogram pass (1..10)
 *   "reorder_chunks_per_cta"  work chunks per resident CTA in the reorder
 *   "hist_ctas_per_sm"        histogram CTAs per SM (0: as many as fit)
 *   "hist_waves"              histogram grid in this many waves of resident
 *                             CTAs (1..16; default 1)
 *   "exact_f64_hist"          1: bin f64 weights as exact fixed-point sums in
 *                             every pass (by default the bins hold truncated
 *                             sums and a decision they cannot settle is
 *                             replayed from exact bins)
 *   "reorder_kernel"          0 (default): per level, the bulk-copy reorder,
 *                             or for segments below 8192 points on average
 *                             the double-buffered one; 1 or 2 force either
 *   "autotune_cache"          1 (default): coupe_gpu_autotune returns the
 *                             schedule kept for a workload class tuned before
 *                             without timing again; 0: always time
 *   "sync_levels"             1: the host waits for each tree level before
 *                             queuing the next (by default a run is queued
 *                             whole and waited for once; a split needing more
 *                             than two histogram passes makes the host finish
 *                             from that level on level by level)
 * and two failure-handling knobs:
 *   "lookback_spin_limit"     polls of a reorder chunk's wait for its
 *                             predecessor's prefix before the run fails with
 *                             COUPE_ERR_CRASH (default 2^22; 0 makes every
 *                             unfinished predecessor a failure)
 *   "workspace_limit_mb"      cap on the engine's device workspace in MiB (0:
 *                             none); a run needing more fails with
 *                             COUPE_ERR_ALLOC before allocating
 * Returns COUPE_ERR_OK, or COUPE_ERR_BAD_TYPE for an unknown name. */
int coupe_gpu_set_option(const char *name, int64_t value);

/* Current value of a knob, or -1 for an unknown name. */
int64_t coupe_gpu_get_option(const char *name);

/* The schedule coupe_gpu_autotune chose. */
struct coupe_gpu_tuning {
	int max_nbk;
	int hist_ctas_per_sm;
	int reorder_chunks_per_cta;
	int hist_waves;   /* histogram grid: waves of resident CTAs */
	double device_ms; /* median device time of the chosen schedule */
};

/* Autotuner (no counterpart in the reference): runs the batched call of
 * coupe_gpu_rcb_batched (same arguments; nsets = 1 for one set) under each
 * candidate schedule of the knobs above, `repeats` timed runs each after one
 * warm-up, and keeps the fastest process-wide (the ids are the same under
 * every schedule).  `best` (may be NULL) receives the choice; d_partition
 * holds the ids of the last run.  60 candidates (bisection steps per pass
 * 6-10, histogram CTAs per SM 0/3/2, reorder chunks per CTA 1/2, one or two
 * waves of histogram CTAs): budget about 60 * (repeats + 1) runs of the
 * workload.  The choice is kept per
 * workload class (points and sets rounded down to powers of two, dimension,
 * weight type, mode, deepest iteration count): a later call for the same
 * class applies the kept schedule at once, runs nothing and leaves
 * d_partition untouched (option autotune_cache).  When the environment
 * variable COUPE_GPU_TUNE_CACHE names a file, the choices are also read from
 * it and appended to it, so that they outlive the process. */
enum coupe_err coupe_gpu_autotune(uint64_t *d_partition, uint64_t nsets,
		const uint64_t *set_offsets, uint64_t dimension, const double *d_points,
		enum coupe_type weight_type, const void *d_weights,
		const uint32_t *iter_counts, double tolerance, int mode, void *stream,
		int repeats, struct coupe_gpu_tuning *best);

/* Library version string. */
const char *coupe_gpu_version(void);

#ifdef __cplusplus
}
#endif

#endif /* COUPE_GPU_H */
