// Host-side interface between the C ABI (ffi.cpp) and the CUDA engine.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <mutex>
#include <string>
#include <vector>

#include "../../include/coupe_gpu.h"

namespace cg {

// One Rcb run on device-resident data.
struct RunArgs {
    uint64_t n = 0;
    int dim = 0;
    const double *d_points = nullptr;  // n * dim doubles, AoS
    int wtype = 0;                     // enum coupe_type
    const void *d_weights = nullptr;   // n elements of wtype
    uint64_t *d_part = nullptr;        // n part ids (output)
    uint64_t iter_count = 0;
    double tolerance = 0.0;
    int mode = COUPE_GPU_REF32;
    bool has_matrix = false;
    double matrix[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};  // row-major dim x dim
    cudaStream_t stream = nullptr;
    // several independent point sets (nsets > 1): set k is items
    // [set_off[k], set_off[k + 1]) with iter_count set_iters[k]; host arrays.
    // iter_count is then unused.
    uint64_t nsets = 1;
    const uint64_t *set_off = nullptr;
    const uint32_t *set_iters = nullptr;
    // host calls: the weights are still uploading until this event (the
    // weight kernels wait for it; the key conversion does not)
    cudaEvent_t weights_ready = nullptr;
    // host calls with a pinned id buffer: its device-mapped address; the
    // traversal then writes the ids there directly and sets *ids_on_host
    uint64_t *ids_host = nullptr;
    bool *ids_on_host = nullptr;
};

// Process-wide tuning knobs (coupe_gpu_set_option).  They change how the
// work is scheduled, never the result.
struct Tuning {
    int force_index_path = 0;        // 1: carry input indices through every reorder
    int max_nbk = 10;                // bisection steps per histogram pass (2^max_nbk bins)
    int reorder_chunks_per_cta = 1;  // reorder chunks per resident CTA
    int hist_ctas_per_sm = 0;        // histogram CTAs per SM (0: as many as fit)
    int hist_waves = 1;              // histogram grid: this many waves of resident CTAs
    int exact_f64_hist = 0;          // 1: f64 weights always binned exactly
    int reorder_kernel = 0;          // 0: by segment size; 1: k_reorder (bulk copies); 2: k_reorder_small
    // Failure handling (not scheduling): polls of a reorder chunk's bounded
    // look-back wait before it gives up with an error, and a cap on the
    // engine workspace in MiB (0: none; a run needing more fails with
    // COUPE_ERR_ALLOC before allocating, as an out-of-memory device would).
    int lookback_spin_limit = 1 << 22;
    int workspace_limit_mb = 0;
    // 1: wait for every level's decisions before queuing the next (the host
    // synchronises once per level); 0: queue the whole run and synchronise
    // once, finishing level by level only after a split needed a third pass.
    // The ids are the same.
    int sync_levels = 0;
    // 1: coupe_gpu_autotune returns the schedule kept for a workload class
    // tuned before (in this process, or in the COUPE_GPU_TUNE_CACHE file)
    int autotune_cache = 1;
};
Tuning &tuning();

// Largest number of recorded splits for which part ids come from a
// traversal (k_traverse) rather than from indices carried through reorders.
constexpr uint64_t TRAV_MAX_ENTRIES = 1ull << 22;

// Kernel kinds timed by the optional per-launch profiler.
enum KernelId {
    KID_CONVERT, KID_WABS, KID_WSUM, KID_ROOT, KID_HIST, KID_DECIDE, KID_CHILDREN, KID_REORDER,
    KID_ASSIGN, KID_FILL, KID_MOMENTS, KID_LOADS, KID_BARY, KID_GRID, KID_COUNT
};
const char *kernel_name(int id);

// Per-launch CUDA-event profiler: when on, every launch of a run is bracketed
// by two events on its stream; after the run's final synchronisation the
// elapsed times and the launch's algorithmic bytes are accumulated per kind.
struct Profiler {
    bool on = false;
    struct Rec {
        int id;
        uint64_t bytes;
        cudaEvent_t a, b;
    };
    std::vector<Rec> recs;
    std::vector<cudaEvent_t> pool;
    uint64_t count[KID_COUNT] = {};
    uint64_t bytes[KID_COUNT] = {};
    double ms[KID_COUNT] = {};
    cudaEvent_t take();
    void begin(int id, uint64_t bytes, cudaStream_t s);
    void end(cudaStream_t s);
    void resolve();  // call after the stream synchronised
    void reset();
};

// Per-device state: a stream, a grow-only workspace and pinned scalars.
// Runs on one device are serialised by `mu`.
struct DevCtx {
    int dev = -1;
    int sms = 0;
    cudaStream_t stream = nullptr;
    cudaStream_t stream2 = nullptr;  // host calls: the weight upload
    cudaEvent_t ev_pts = nullptr, ev_w = nullptr;
    void *ws = nullptr;
    size_t ws_cap = 0;
    void *h_pinned = nullptr;  // pinned host scratch for scalar read-backs
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    Profiler prof;
    std::mutex mu;
};

// Returns the calling thread's current device context (created on first use).
DevCtx *device_ctx(std::string *err);

// Ensures the workspace holds at least `bytes`; returns a coupe_err.
int ensure_workspace(DevCtx &C, size_t bytes, std::string *err);

// Runs Rcb (the basis change of RunArgs applied first when has_matrix).
int run_rcb(DevCtx &C, const RunArgs &a, coupe_gpu_stats *st, std::string *err);

// The Rib basis change (obb_to_aabb) of n device-resident points.
int rib_matrix(DevCtx &C, uint64_t n, int dim, const double *d_points, cudaStream_t stream, double *out,
               std::string *err, int wtype = -1, const void *d_weights = nullptr);

// Loads of parts 0..P-1 of a device-resident partition (coupe's
// compute_parts_load), written to the host array `loads` (P elements of the
// weights' type); COUPE_ERR_BAD_TYPE for a part id >= P or a non-finite
// f64 weight.
int parts_load(DevCtx &C, const uint64_t *d_part, uint64_t n, int wtype, const void *d_w, uint64_t P,
               cudaStream_t stream, void *loads, std::string *err);

// coupe's imbalance from the loads of P parts (host arithmetic).
double imbalance_of_loads(int wtype, const void *loads, uint64_t P);

// coupe's Grid::rcb on a device-resident grid of `dim` sizes (cells
// x + size[0] * (y + size[1] * z)); the weighted median replays `threads`
// rayon workers (>= 2).
int grid_rcb(DevCtx &C, int dim, const uint64_t *size, int wtype, const void *d_w, uint64_t iters, uint64_t threads,
             uint64_t *d_part, cudaStream_t stream, std::string *err);

// Barycentres of n_el elements of k nodes each (device node lists, 0-based)
// over n_nodes device coordinates of `dim` doubles; d_out gets n_el x dim.
int barycentres(DevCtx &C, int dim, const double *d_coords, uint64_t n_nodes, uint64_t k, const uint64_t *d_nodes,
                uint64_t n_el, double *d_out, cudaStream_t stream, std::string *err);

// The engine's per-point f64 -> f32 key conversion over n device values.
int f64_to_f32(DevCtx &C, const double *d_in, float *d_out, uint64_t n, cudaStream_t stream, std::string *err);

// coupe's axis_sort of the identity permutation of n device points of `dim`
// doubles along `coord` (recursive_bisection.rs:815-827): d_perm gets the
// point indices in ascending coordinate order, ties in index order.
int axis_sort(DevCtx &C, uint64_t n, int dim, const double *d_points, int coord, uint64_t *d_perm,
              cudaStream_t stream, std::string *err);

// coupe's MultiJagged (multi_jagged.rs:150-295) of n device points with f64
// weights into part_count parts in at most max_iter iterations.
int multi_jagged(DevCtx &C, uint64_t n, int dim, const double *d_points, const double *d_weights,
                 uint64_t part_count, uint64_t max_iter, uint64_t *d_part, cudaStream_t stream, std::string *err);

// Per-mode entry points, instantiated in separate translation units.
int run_rcb_ref32(DevCtx &C, const RunArgs &a, coupe_gpu_stats *st, std::string *err);
int run_rcb_f64(DevCtx &C, const RunArgs &a, coupe_gpu_stats *st, std::string *err);
int run_rcb_band(DevCtx &C, const RunArgs &a, coupe_gpu_stats *st, std::string *err);

// Maps a CUDA error to a coupe_err and records a message.
int cuda_fail(cudaError_t e, const char *what, std::string *err);

}  // namespace cg
