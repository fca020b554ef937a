// The C ABI of libcoupe_gpu.so (include/coupe.h, include/coupe_gpu.h).
//
// Semantics follow coupe-ffi (coupe-ffi/src/lib.rs, coupe-ffi/src/data.rs):
// data sets are arrays, constants or callbacks; points are always read as
// `dimension` doubles per item whatever the data set's type; the length
// mismatch is reported before a bad dimension; an empty input succeeds and
// leaves `partition` untouched.  Host inputs are gathered into pinned staging
// memory, copied to the device, partitioned there, and the ids copied back.
#include <cuda_runtime.h>

#include <cstdio>
#include <cstdlib>
#include <algorithm>
#include <cstring>
#include <map>
#include <mutex>
#include <new>
#include <string>
#include <vector>

#include "../../include/coupe.h"
#include "../../include/coupe_gpu.h"
#include "engine.h"
#include "split_noalloc.h"

struct coupe_data {
    int kind;  // 0 array, 1 constant, 2 callback
    uintptr_t len;
    int type;
    const void *ptr;  // array base or constant value
    const void *ctx;
    const void *(*i_th)(const void *, uintptr_t);
};

namespace {

thread_local std::string t_err;
thread_local coupe_gpu_stats t_stats;

size_t type_size(int t) { return t == COUPE_INT ? 4 : 8; }

coupe_data *new_data(int kind, uintptr_t len, int type, const void *ptr, const void *ctx,
                     const void *(*f)(const void *, uintptr_t)) {
    coupe_data *d = new (std::nothrow) coupe_data;
    if (!d) return nullptr;
    d->kind = kind;
    d->len = len;
    d->type = type;
    d->ptr = ptr;
    d->ctx = ctx;
    d->i_th = f;
    return d;
}

// Copies element i (elem bytes) of a data set to dst.
inline void fetch(const coupe_data *d, uintptr_t i, size_t elem, void *dst) {
    switch (d->kind) {
    case 0:
        std::memcpy(dst, (const char *)d->ptr + i * elem, elem);
        break;
    case 1:
        std::memcpy(dst, d->ptr, elem);
        break;
    default:
        std::memcpy(dst, d->i_th(d->ctx, i), elem);
        break;
    }
}

// Pinned staging buffers reused across calls on this thread.
struct Staging {
    void *p = nullptr;
    size_t cap = 0;
    ~Staging() {
        if (p) cudaFreeHost(p);
    }
    void *get(size_t bytes) {
        if (bytes <= cap) return p;
        if (p) cudaFreeHost(p);
        p = nullptr;
        cap = 0;
        if (cudaMallocHost(&p, bytes) != cudaSuccess) {
            cudaGetLastError();
            return nullptr;
        }
        cap = bytes;
        return p;
    }
};

// Device buffers for host calls, reused across calls on this thread.
struct DevBuf {
    void *p = nullptr;
    size_t cap = 0;
    int dev = -1;
    void *get(size_t bytes, int device) {
        if (bytes <= cap && device == dev) return p;
        if (p) cudaFree(p);
        p = nullptr;
        cap = 0;
        if (cudaMalloc(&p, bytes) != cudaSuccess) {
            cudaGetLastError();
            return nullptr;
        }
        cap = bytes;
        dev = device;
        return p;
    }
};

thread_local DevBuf t_dev;

// Is [p, p+bytes) pinned (page-locked or registered) host memory?
bool is_pinned(const void *p) {
    cudaPointerAttributes at;
    if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return at.type == cudaMemoryTypeHost;
}

// Host-side call: validate like coupe-ffi, stage, run on the device, copy back.
coupe_err host_call(bool rib, uintptr_t *partition, uintptr_t dimension, const coupe_data *points,
                    const coupe_data *weights, uintptr_t iter_count, double tolerance, int mode) {
    t_err.clear();
    std::memset(&t_stats, 0, sizeof(t_stats));
    const bool winert = rib && (mode & COUPE_GPU_WEIGHTED_INERTIA) != 0;
    mode &= ~COUPE_GPU_WEIGHTED_INERTIA;
    t_stats.mode = mode;
    if (!points || !weights) {
        t_err = "NULL data set";
        return COUPE_ERR_CRASH;
    }
    const uintptr_t n = points->len;
    if (n != weights->len) return COUPE_ERR_LEN_MISMATCH;  // coupe-ffi/src/lib.rs:285-288
    if (dimension != 2 && dimension != 3) return COUPE_ERR_BAD_DIMENSION;  // :297-301
    if (weights->type < COUPE_INT || weights->type > COUPE_DOUBLE) {
        t_err = "unknown weight type";
        return COUPE_ERR_BAD_TYPE;
    }
    if (n == 0) return COUPE_ERR_OK;  // recursive_bisection.rs:685-688
    if (!partition) {
        t_err = "NULL partition";
        return COUPE_ERR_CRASH;
    }
    std::string err;
    cg::DevCtx *C = cg::device_ctx(&err);
    if (!C) {
        t_err = err;
        return COUPE_ERR_CRASH;
    }
    const size_t pbytes = (size_t)n * dimension * sizeof(double);
    const size_t wsz = type_size(weights->type);
    const size_t wbytes = (size_t)n * wsz;
    const size_t obytes = (size_t)n * sizeof(uint64_t);
    std::lock_guard<std::mutex> lock(C->mu);
    cudaStream_t s = C->stream;
    char *dbuf = (char *)t_dev.get(pbytes + wbytes + obytes + 512, C->dev);
    if (!dbuf) {
        t_err = "device allocation of the input copy failed";
        return COUPE_ERR_ALLOC;
    }
    double *d_pts = (double *)dbuf;
    char *d_w = dbuf + ((pbytes + 255) & ~(size_t)255);
    uint64_t *d_part = (uint64_t *)(d_w + ((wbytes + 255) & ~(size_t)255));
    cudaError_t e;
    // points: arrays are copied as they are; constants and callbacks are
    // gathered into pinned staging first (coupe-ffi/src/data.rs:156-165).
    static thread_local Staging st_p, st_w;
    const void *src_p = points->ptr;
    if (points->kind != 0) {
        double *h = (double *)st_p.get(pbytes);
        if (!h) return COUPE_ERR_ALLOC;
        for (uintptr_t i = 0; i < n; ++i) fetch(points, i, dimension * sizeof(double), h + i * dimension);
        src_p = h;
    }
    const void *src_w = weights->ptr;
    if (weights->kind != 0) {
        char *h = (char *)st_w.get(wbytes);
        if (!h) return COUPE_ERR_ALLOC;
        for (uintptr_t i = 0; i < n; ++i) fetch(weights, i, wsz, h + i * wsz);
        src_w = h;
    }
    // The points go first; the weights follow on a second stream, so that
    // the key conversion runs while they upload (the weight kernels wait for
    // them).
    if ((e = cudaMemcpyAsync(d_pts, src_p, pbytes, cudaMemcpyHostToDevice, s)) != cudaSuccess ||
        (e = cudaEventRecord(C->ev_pts, s)) != cudaSuccess ||
        (e = cudaStreamWaitEvent(C->stream2, C->ev_pts, 0)) != cudaSuccess ||
        (e = cudaMemcpyAsync(d_w, src_w, wbytes, cudaMemcpyHostToDevice, C->stream2)) != cudaSuccess ||
        (e = cudaEventRecord(C->ev_w, C->stream2)) != cudaSuccess) {
        cudaStreamSynchronize(C->stream2);
        int rc = cg::cuda_fail(e, "host to device copy", &t_err);
        return (coupe_err)rc;
    }
    cg::RunArgs a;
    a.n = n;
    a.dim = (int)dimension;
    a.d_points = d_pts;
    a.wtype = weights->type;
    a.d_weights = d_w;
    a.d_part = d_part;
    a.iter_count = iter_count;
    a.tolerance = tolerance;
    a.mode = mode;
    a.stream = s;
    a.weights_ready = C->ev_w;
    // a pinned id buffer: the ids are written into it by the last kernel
    static_assert(sizeof(uintptr_t) == sizeof(uint64_t), "64-bit uintptr_t expected");
    bool ids_on_host = false;
    void *mapped = nullptr;
    if (is_pinned(partition) && cudaHostGetDevicePointer(&mapped, partition, 0) == cudaSuccess && mapped) {
        a.ids_host = (uint64_t *)mapped;
        a.ids_on_host = &ids_on_host;
    } else {
        cudaGetLastError();
    }
    int rc = COUPE_ERR_OK;
    if (rib) {
        double M[9];
        if (winert) cudaStreamWaitEvent(s, C->ev_w, 0);  // the weights' upload
        rc = winert ? cg::rib_matrix(*C, n, (int)dimension, d_pts, s, M, &err, weights->type, d_w)
                    : cg::rib_matrix(*C, n, (int)dimension, d_pts, s, M, &err);
        if (rc == COUPE_ERR_OK) {
            a.has_matrix = true;
            std::memcpy(a.matrix, M, sizeof(M));
        }
    }
    if (rc == COUPE_ERR_OK) rc = cg::run_rcb(*C, a, &t_stats, &err);
    cudaStreamSynchronize(C->stream2);  // the weight upload has ended (it has on success)
    if (rc != COUPE_ERR_OK) {
        t_err = err;
        return (coupe_err)rc;
    }
    if (!ids_on_host && (e = cudaMemcpyAsync(partition, d_part, obytes, cudaMemcpyDeviceToHost, s)) != cudaSuccess)
        return (coupe_err)cg::cuda_fail(e, "device to host copy", &t_err);
    if ((e = cudaStreamSynchronize(s)) != cudaSuccess)
        return (coupe_err)cg::cuda_fail(e, "device to host copy", &t_err);
    return COUPE_ERR_OK;
}

coupe_err device_call(bool rib, uint64_t *d_partition, uint64_t n, uint64_t dimension, const double *d_points,
                      coupe_type wtype, const void *d_weights, uint64_t iter_count, double tolerance, int mode,
                      const double *matrix, void *stream) {
    t_err.clear();
    std::memset(&t_stats, 0, sizeof(t_stats));
    const bool winert = rib && (mode & COUPE_GPU_WEIGHTED_INERTIA) != 0;
    mode &= ~COUPE_GPU_WEIGHTED_INERTIA;
    t_stats.mode = mode;
    if (dimension != 2 && dimension != 3) return COUPE_ERR_BAD_DIMENSION;
    if (wtype < COUPE_INT || wtype > COUPE_DOUBLE) {
        t_err = "unknown weight type";
        return COUPE_ERR_BAD_TYPE;
    }
    if (n == 0) return COUPE_ERR_OK;
    std::string err;
    cg::DevCtx *C = cg::device_ctx(&err);
    if (!C) {
        t_err = err;
        return COUPE_ERR_CRASH;
    }
    std::lock_guard<std::mutex> lock(C->mu);
    cg::RunArgs a;
    a.n = n;
    a.dim = (int)dimension;
    a.d_points = d_points;
    a.wtype = wtype;
    a.d_weights = d_weights;
    a.d_part = d_partition;
    a.iter_count = iter_count;
    a.tolerance = tolerance;
    a.mode = mode;
    a.stream = (cudaStream_t)stream;
    int rc = COUPE_ERR_OK;
    if (rib) {
        double M[9];
        rc = winert ? cg::rib_matrix(*C, n, (int)dimension, d_points, a.stream, M, &err, wtype, d_weights)
                    : cg::rib_matrix(*C, n, (int)dimension, d_points, a.stream, M, &err);
        if (rc == COUPE_ERR_OK) {
            a.has_matrix = true;
            std::memcpy(a.matrix, M, sizeof(M));
        }
    } else if (matrix) {
        a.has_matrix = true;
        std::memcpy(a.matrix, matrix, sizeof(double) * dimension * dimension);
    }
    if (rc == COUPE_ERR_OK) rc = cg::run_rcb(*C, a, &t_stats, &err);
    if (rc != COUPE_ERR_OK) t_err = err;
    return (coupe_err)rc;
}

}  // namespace

extern "C" {

const char *coupe_strerror(enum coupe_err err) {
    switch (err) {
    case COUPE_ERR_OK: return "success";
    case COUPE_ERR_ALLOC: return "allocation failed";
    case COUPE_ERR_CRASH: return "coupe encountered a bug and crashed";
    case COUPE_ERR_BAD_DIMENSION: return "this algorithm does not support the given mesh dimension";
    case COUPE_ERR_BAD_TYPE: return "this algorithm does not support the given type";
    case COUPE_ERR_BIPART_ONLY: return "this algorithm does not support k-way partitioning";
    case COUPE_ERR_LEN_MISMATCH: return "input iters (e.g. weights and points) don't have the same length";
    case COUPE_ERR_NOT_FOUND: return "no partition has been found for the given constraints";
    case COUPE_ERR_NEG_VALUES: return "this algorithm does not support negative values";
    }
    return "unknown error";
}

void coupe_data_free(coupe_data *data) { delete data; }

coupe_data *coupe_data_array(uintptr_t len, enum coupe_type type, const void *data) {
    return new_data(0, len, type, data, nullptr, nullptr);
}

coupe_data *coupe_data_constant(uintptr_t len, enum coupe_type type, const void *value) {
    return new_data(1, len, type, value, nullptr, nullptr);
}

coupe_data *coupe_data_fn(const void *context, uintptr_t len, enum coupe_type type,
                          const void *(*i_th)(const void *, uintptr_t)) {
    return new_data(2, len, type, nullptr, context, i_th);
}

enum coupe_err coupe_rcb(uintptr_t *partition, uintptr_t dimension, const coupe_data *points,
                         const coupe_data *weights, uintptr_t iter_count, double tolerance) {
    return host_call(false, partition, dimension, points, weights, iter_count, tolerance, COUPE_GPU_REF32);
}

enum coupe_err coupe_rib(uintptr_t *partition, uintptr_t dimension, const coupe_data *points,
                         const coupe_data *weights, uintptr_t iter_count, double tolerance) {
    return host_call(true, partition, dimension, points, weights, iter_count, tolerance, COUPE_GPU_REF32);
}

enum coupe_err coupe_gpu_rcb(uintptr_t *partition, uintptr_t dimension, const coupe_data *points,
                             const coupe_data *weights, uintptr_t iter_count, double tolerance, int mode) {
    return host_call(false, partition, dimension, points, weights, iter_count, tolerance, mode);
}

enum coupe_err coupe_gpu_rib(uintptr_t *partition, uintptr_t dimension, const coupe_data *points,
                             const coupe_data *weights, uintptr_t iter_count, double tolerance, int mode) {
    return host_call(true, partition, dimension, points, weights, iter_count, tolerance, mode);
}

enum coupe_err coupe_gpu_rcb_device(uint64_t *d_partition, uint64_t n, uint64_t dimension, const double *d_points,
                                    enum coupe_type weight_type, const void *d_weights, uint64_t iter_count,
                                    double tolerance, int mode, const double *matrix, void *stream) {
    return device_call(false, d_partition, n, dimension, d_points, weight_type, d_weights, iter_count, tolerance, mode,
                       matrix, stream);
}

enum coupe_err coupe_gpu_rib_device(uint64_t *d_partition, uint64_t n, uint64_t dimension, const double *d_points,
                                    enum coupe_type weight_type, const void *d_weights, uint64_t iter_count,
                                    double tolerance, int mode, void *stream) {
    return device_call(true, d_partition, n, dimension, d_points, weight_type, d_weights, iter_count, tolerance, mode,
                       nullptr, stream);
}

enum coupe_err coupe_gpu_rcb_batched(uint64_t *d_partition, uint64_t nsets, const uint64_t *set_offsets,
                                     uint64_t dimension, const double *d_points, enum coupe_type weight_type,
                                     const void *d_weights, const uint32_t *iter_counts, double tolerance, int mode,
                                     void *stream) {
    t_err.clear();
    std::memset(&t_stats, 0, sizeof(t_stats));
    t_stats.mode = mode;
    if (dimension != 2 && dimension != 3) return COUPE_ERR_BAD_DIMENSION;
    if (weight_type < COUPE_INT || weight_type > COUPE_DOUBLE) {
        t_err = "unknown weight type";
        return COUPE_ERR_BAD_TYPE;
    }
    if (nsets == 0) return COUPE_ERR_OK;
    if (!set_offsets || !iter_counts) {
        t_err = "set offsets and iteration counts are required";
        return COUPE_ERR_LEN_MISMATCH;
    }
    if (nsets >= (1ull << 31)) {
        t_err = "more than 2^31 - 1 sets";
        return COUPE_ERR_ALLOC;
    }
    if (set_offsets[0] != 0) {
        t_err = "set offsets must start at 0";
        return COUPE_ERR_LEN_MISMATCH;
    }
    for (uint64_t k = 0; k < nsets; ++k)
        if (set_offsets[k + 1] < set_offsets[k]) {
            t_err = "set offsets must not decrease";
            return COUPE_ERR_LEN_MISMATCH;
        }
    const uint64_t n = set_offsets[nsets];
    if (n == 0) return COUPE_ERR_OK;
    if (nsets == 1)
        return device_call(false, d_partition, n, dimension, d_points, weight_type, d_weights, iter_counts[0],
                           tolerance, mode, nullptr, stream);
    std::string err;
    cg::DevCtx *C = cg::device_ctx(&err);
    if (!C) {
        t_err = err;
        return COUPE_ERR_CRASH;
    }
    std::lock_guard<std::mutex> lock(C->mu);
    cg::RunArgs a;
    a.n = n;
    a.dim = (int)dimension;
    a.d_points = d_points;
    a.wtype = weight_type;
    a.d_weights = d_weights;
    a.d_part = d_partition;
    a.tolerance = tolerance;
    a.mode = mode;
    a.stream = (cudaStream_t)stream;
    a.nsets = nsets;
    a.set_off = set_offsets;
    a.set_iters = iter_counts;
    int rc = cg::run_rcb(*C, a, &t_stats, &err);
    if (rc != COUPE_ERR_OK) t_err = err;
    return (coupe_err)rc;
}

enum coupe_err coupe_gpu_rib_matrix(uint64_t n, uint64_t dimension, const double *d_points, double *obb_to_aabb,
                                    void *stream) {
    t_err.clear();
    if (dimension != 2 && dimension != 3) return COUPE_ERR_BAD_DIMENSION;
    if (n == 0) {
        t_err = "no points";
        return COUPE_ERR_CRASH;
    }
    std::string err;
    cg::DevCtx *C = cg::device_ctx(&err);
    if (!C) {
        t_err = err;
        return COUPE_ERR_CRASH;
    }
    std::lock_guard<std::mutex> lock(C->mu);
    int rc = cg::rib_matrix(*C, n, (int)dimension, d_points, (cudaStream_t)stream, obb_to_aabb, &err);
    if (rc != COUPE_ERR_OK) t_err = err;
    return (coupe_err)rc;
}

enum coupe_err coupe_gpu_rib_matrix_weighted(uint64_t n, uint64_t dimension, const double *d_points,
                                             enum coupe_type weight_type, const void *d_weights, double *obb_to_aabb,
                                             void *stream) {
    t_err.clear();
    if (dimension != 2 && dimension != 3) return COUPE_ERR_BAD_DIMENSION;
    if (weight_type < COUPE_INT || weight_type > COUPE_DOUBLE) {
        t_err = "unknown weight type";
        return COUPE_ERR_BAD_TYPE;
    }
    if (n == 0 || !d_weights) {
        t_err = "no points";
        return COUPE_ERR_CRASH;
    }
    std::string err;
    cg::DevCtx *C = cg::device_ctx(&err);
    if (!C) {
        t_err = err;
        return COUPE_ERR_CRASH;
    }
    std::lock_guard<std::mutex> lock(C->mu);
    int rc = cg::rib_matrix(*C, n, (int)dimension, d_points, (cudaStream_t)stream, obb_to_aabb, &err, weight_type,
                            d_weights);
    if (rc != COUPE_ERR_OK) t_err = err;
    return (coupe_err)rc;
}

enum coupe_err coupe_gpu_f64_to_f32(const double *d_in, float *d_out, uint64_t n, void *stream) {
    t_err.clear();
    std::string err;
    cg::DevCtx *C = cg::device_ctx(&err);
    if (!C) {
        t_err = err;
        return COUPE_ERR_CRASH;
    }
    std::lock_guard<std::mutex> lock(C->mu);
    int rc = cg::f64_to_f32(*C, d_in, d_out, n, (cudaStream_t)stream, &err);
    if (rc != COUPE_ERR_OK) t_err = err;
    return (coupe_err)rc;
}

// Loads (and, with `imbalance`, coupe's imbalance of them) of n device part
// ids and weights; the caller holds C.mu.
static coupe_err loads_locked(cg::DevCtx &C, const uint64_t *d_part, uint64_t n, int wtype, const void *d_w,
                              uint64_t num_parts, void *loads, double *imbalance, cudaStream_t s) {
    if (imbalance && num_parts == 0) {  // imbalance.rs:52-55, before any load is computed
        *imbalance = 0.0;
        return COUPE_ERR_OK;
    }
    std::vector<uint64_t> tmp;  // 8-byte slots hold any weight type
    if (imbalance) {
        tmp.resize(num_parts);
        loads = tmp.data();
    }
    std::string err;
    const int rc = cg::parts_load(C, d_part, n, wtype, d_w, num_parts, s, loads, &err);
    if (rc != COUPE_ERR_OK) {
        t_err = err;
        return (coupe_err)rc;
    }
    if (imbalance) *imbalance = cg::imbalance_of_loads(wtype, loads, num_parts);
    return COUPE_ERR_OK;
}

static coupe_err device_loads(const uint64_t *d_partition, uint64_t n, enum coupe_type weight_type,
                              const void *d_weights, uint64_t num_parts, void *loads, double *imbalance,
                              void *stream) {
    t_err.clear();
    if (imbalance && num_parts == 0) {  // imbalance.rs:52-55, before anything else
        *imbalance = 0.0;
        return COUPE_ERR_OK;
    }
    if (weight_type < COUPE_INT || weight_type > COUPE_DOUBLE) {
        t_err = "unknown weight type";
        return COUPE_ERR_BAD_TYPE;
    }
    if (!imbalance && num_parts > 0 && !loads) {
        t_err = "NULL loads";
        return COUPE_ERR_CRASH;
    }
    if (n > 0 && (!d_partition || !d_weights)) {
        t_err = "NULL partition or weights";
        return COUPE_ERR_CRASH;
    }
    std::string err;
    cg::DevCtx *C = cg::device_ctx(&err);
    if (!C) {
        t_err = err;
        return COUPE_ERR_CRASH;
    }
    std::lock_guard<std::mutex> lock(C->mu);
    return loads_locked(*C, d_partition, n, weight_type, d_weights, num_parts, loads, imbalance,
                        stream ? (cudaStream_t)stream : C->stream);
}

enum coupe_err coupe_gpu_parts_load_device(const uint64_t *d_partition, uint64_t n, enum coupe_type weight_type,
                                           const void *d_weights, uint64_t num_parts, void *loads, void *stream) {
    return device_loads(d_partition, n, weight_type, d_weights, num_parts, loads, nullptr, stream);
}

enum coupe_err coupe_gpu_imbalance_device(uint64_t num_parts, const uint64_t *d_partition, uint64_t n,
                                          enum coupe_type weight_type, const void *d_weights, double *imbalance,
                                          void *stream) {
    if (!imbalance) {
        t_err = "NULL imbalance";
        return COUPE_ERR_CRASH;
    }
    return device_loads(d_partition, n, weight_type, d_weights, num_parts, nullptr, imbalance, stream);
}

// Host forms: the part ids and the weights (gathered like host_call's) are
// copied to the device, then the loads are computed there.
static coupe_err host_loads(uintptr_t num_parts, const uintptr_t *partition, const coupe_data *weights, void *loads,
                            double *imbalance) {
    t_err.clear();
    if (!weights) {
        t_err = "NULL data set";
        return COUPE_ERR_CRASH;
    }
    if (weights->type < COUPE_INT || weights->type > COUPE_DOUBLE) {
        t_err = "unknown weight type";
        return COUPE_ERR_BAD_TYPE;
    }
    if (imbalance && num_parts == 0) {
        *imbalance = 0.0;
        return COUPE_ERR_OK;
    }
    if (!imbalance && num_parts > 0 && !loads) {
        t_err = "NULL loads";
        return COUPE_ERR_CRASH;
    }
    const uintptr_t n = weights->len;
    if (n > 0 && !partition) {
        t_err = "NULL partition";
        return COUPE_ERR_CRASH;
    }
    std::string err;
    cg::DevCtx *C = cg::device_ctx(&err);
    if (!C) {
        t_err = err;
        return COUPE_ERR_CRASH;
    }
    const size_t wsz = type_size(weights->type);
    const size_t pbytes = (size_t)n * sizeof(uint64_t), wbytes = (size_t)n * wsz;
    std::lock_guard<std::mutex> lock(C->mu);
    char *dbuf = (char *)t_dev.get(pbytes + wbytes + 512, C->dev);
    if (!dbuf) {
        t_err = "device allocation of the input copy failed";
        return COUPE_ERR_ALLOC;
    }
    uint64_t *d_part = (uint64_t *)dbuf;
    char *d_w = dbuf + ((pbytes + 255) & ~(size_t)255);
    static thread_local Staging st_w;
    const void *src_w = weights->ptr;
    if (weights->kind != 0 && n > 0) {
        char *h = (char *)st_w.get(wbytes);
        if (!h) return COUPE_ERR_ALLOC;
        for (uintptr_t i = 0; i < n; ++i) fetch(weights, i, wsz, h + i * wsz);
        src_w = h;
    }
    cudaStream_t s = C->stream;
    cudaError_t e;
    if (n > 0 && ((e = cudaMemcpyAsync(d_part, partition, pbytes, cudaMemcpyHostToDevice, s)) != cudaSuccess ||
                  (e = cudaMemcpyAsync(d_w, src_w, wbytes, cudaMemcpyHostToDevice, s)) != cudaSuccess))
        return (coupe_err)cg::cuda_fail(e, "host to device copy", &t_err);
    return loads_locked(*C, d_part, n, weights->type, d_w, num_parts, loads, imbalance, s);
}

// Argument checks of Grid::rcb shared by both entry points.
static coupe_err grid_checks(uint64_t dimension, const uint64_t *size, uint64_t n_weights, uint64_t threads,
                             uint64_t *cells) {
    if (dimension != 2 && dimension != 3) return COUPE_ERR_BAD_DIMENSION;
    if (!size) {
        t_err = "NULL size";
        return COUPE_ERR_CRASH;
    }
    uint64_t n = 1;
    for (uint64_t d = 0; d < dimension; ++d) {
        if (size[d] == 0) return COUPE_ERR_BAD_DIMENSION;  // coupe's sizes are NonZeroUsize
        if (n > UINT64_MAX / size[d]) {
            t_err = "grid too large";
            return COUPE_ERR_ALLOC;
        }
        n *= size[d];
    }
    if (n_weights != n) return COUPE_ERR_LEN_MISMATCH;
    if (threads < 2) {
        t_err = "threads must be at least 2 (coupe's median search does not end with one worker)";
        return COUPE_ERR_BAD_TYPE;
    }
    *cells = n;
    return COUPE_ERR_OK;
}

enum coupe_err coupe_gpu_grid_rcb_device(uint64_t *d_partition, uint64_t dimension, const uint64_t *size,
                                         enum coupe_type weight_type, const void *d_weights, uint64_t iter_count,
                                         uint64_t threads, void *stream) {
    t_err.clear();
    if (weight_type < COUPE_INT || weight_type > COUPE_DOUBLE) {
        t_err = "unknown weight type";
        return COUPE_ERR_BAD_TYPE;
    }
    uint64_t n = 0, nw = 1;
    if (size && (dimension == 2 || dimension == 3))
        for (uint64_t d = 0; d < dimension; ++d) nw *= size[d];
    const coupe_err c = grid_checks(dimension, size, nw, threads, &n);
    if (c != COUPE_ERR_OK) return c;
    if (!d_partition || !d_weights) {
        t_err = "NULL partition or weights";
        return COUPE_ERR_CRASH;
    }
    std::string err;
    cg::DevCtx *C = cg::device_ctx(&err);
    if (!C) {
        t_err = err;
        return COUPE_ERR_CRASH;
    }
    std::lock_guard<std::mutex> lock(C->mu);
    const int rc = cg::grid_rcb(*C, (int)dimension, size, weight_type, d_weights, iter_count, threads, d_partition,
                                (cudaStream_t)stream, &err);
    if (rc != COUPE_ERR_OK) t_err = err;
    return (coupe_err)rc;
}

enum coupe_err coupe_gpu_grid_rcb(uintptr_t *partition, uintptr_t dimension, const uintptr_t *size,
                                  const coupe_data *weights, uintptr_t iter_count, uintptr_t threads) {
    t_err.clear();
    if (!weights) {
        t_err = "NULL data set";
        return COUPE_ERR_CRASH;
    }
    if (weights->type < COUPE_INT || weights->type > COUPE_DOUBLE) {
        t_err = "unknown weight type";
        return COUPE_ERR_BAD_TYPE;
    }
    static_assert(sizeof(uintptr_t) == sizeof(uint64_t), "64-bit uintptr_t expected");
    uint64_t n = 0;
    const coupe_err c = grid_checks(dimension, (const uint64_t *)size, weights->len, threads, &n);
    if (c != COUPE_ERR_OK) return c;
    if (!partition) {
        t_err = "NULL partition";
        return COUPE_ERR_CRASH;
    }
    std::string err;
    cg::DevCtx *C = cg::device_ctx(&err);
    if (!C) {
        t_err = err;
        return COUPE_ERR_CRASH;
    }
    const size_t wsz = type_size(weights->type), wbytes = (size_t)n * wsz, obytes = (size_t)n * 8;
    std::lock_guard<std::mutex> lock(C->mu);
    char *dbuf = (char *)t_dev.get(wbytes + obytes + 512, C->dev);
    if (!dbuf) {
        t_err = "device allocation of the input copy failed";
        return COUPE_ERR_ALLOC;
    }
    char *d_w = dbuf;
    uint64_t *d_part = (uint64_t *)(dbuf + ((wbytes + 255) & ~(size_t)255));
    static thread_local Staging st_w;
    const void *src_w = weights->ptr;
    if (weights->kind != 0) {
        char *h = (char *)st_w.get(wbytes);
        if (!h) return COUPE_ERR_ALLOC;
        for (uintptr_t i = 0; i < n; ++i) fetch(weights, i, wsz, h + i * wsz);
        src_w = h;
    }
    cudaStream_t s = C->stream;
    cudaError_t e;
    if ((e = cudaMemcpyAsync(d_w, src_w, wbytes, cudaMemcpyHostToDevice, s)) != cudaSuccess)
        return (coupe_err)cg::cuda_fail(e, "host to device copy", &t_err);
    const int rc = cg::grid_rcb(*C, (int)dimension, (const uint64_t *)size, weights->type, d_w, iter_count, threads,
                                d_part, s, &err);
    if (rc != COUPE_ERR_OK) {
        t_err = err;
        return (coupe_err)rc;
    }
    if ((e = cudaMemcpyAsync(partition, d_part, obytes, cudaMemcpyDeviceToHost, s)) != cudaSuccess ||
        (e = cudaStreamSynchronize(s)) != cudaSuccess)
        return (coupe_err)cg::cuda_fail(e, "device to host copy", &t_err);
    return COUPE_ERR_OK;
}

enum coupe_err coupe_gpu_axis_sort_device(uint64_t *d_permutation, uint64_t n, uint64_t dimension,
                                         const double *d_points, uint64_t coord, void *stream) {
    t_err.clear();
    if (dimension == 0 || dimension > 64 || coord >= dimension) return COUPE_ERR_BAD_DIMENSION;
    if (n == 0) return COUPE_ERR_OK;
    if (!d_permutation || !d_points) {
        t_err = "NULL permutation or points";
        return COUPE_ERR_CRASH;
    }
    std::string err;
    cg::DevCtx *C = cg::device_ctx(&err);
    if (!C) {
        t_err = err;
        return COUPE_ERR_CRASH;
    }
    std::lock_guard<std::mutex> lock(C->mu);
    const int rc = cg::axis_sort(*C, n, (int)dimension, d_points, (int)coord, d_permutation, (cudaStream_t)stream,
                                 &err);
    if (rc != COUPE_ERR_OK) t_err = err;
    return (coupe_err)rc;
}

enum coupe_err coupe_gpu_multi_jagged_device(uint64_t *d_partition, uint64_t n, uint64_t dimension,
                                             const double *d_points, const double *d_weights, uint64_t part_count,
                                             uint64_t max_iter, void *stream) {
    t_err.clear();
    if (dimension == 0 || dimension > 64) return COUPE_ERR_BAD_DIMENSION;
    if (n == 0) return COUPE_ERR_OK;
    if (!d_partition || !d_points || !d_weights) {
        t_err = "NULL partition, points or weights";
        return COUPE_ERR_CRASH;
    }
    std::string err;
    cg::DevCtx *C = cg::device_ctx(&err);
    if (!C) {
        t_err = err;
        return COUPE_ERR_CRASH;
    }
    std::lock_guard<std::mutex> lock(C->mu);
    const int rc = cg::multi_jagged(*C, n, (int)dimension, d_points, d_weights, part_count, max_iter, d_partition,
                                    (cudaStream_t)stream, &err);
    if (rc != COUPE_ERR_OK) t_err = err;
    return (coupe_err)rc;
}

enum coupe_err coupe_gpu_multi_jagged(uintptr_t *partition, uintptr_t dimension, const coupe_data *points,
                                      const coupe_data *weights, uintptr_t part_count, uintptr_t max_iter) {
    t_err.clear();
    if (!points || !weights) {
        t_err = "NULL data set";
        return COUPE_ERR_CRASH;
    }
    const uintptr_t n = points->len;
    if (n != weights->len) return COUPE_ERR_LEN_MISMATCH;
    if (dimension == 0 || dimension > 64) return COUPE_ERR_BAD_DIMENSION;
    if (weights->type != COUPE_DOUBLE) {
        t_err = "MultiJagged takes double weights";
        return COUPE_ERR_BAD_TYPE;
    }
    if (n == 0) return COUPE_ERR_OK;
    if (!partition) {
        t_err = "NULL partition";
        return COUPE_ERR_CRASH;
    }
    std::string err;
    cg::DevCtx *C = cg::device_ctx(&err);
    if (!C) {
        t_err = err;
        return COUPE_ERR_CRASH;
    }
    const size_t pbytes = (size_t)n * dimension * sizeof(double), wbytes = (size_t)n * 8, obytes = (size_t)n * 8;
    std::lock_guard<std::mutex> lock(C->mu);
    char *dbuf = (char *)t_dev.get(pbytes + wbytes + obytes + 512, C->dev);
    if (!dbuf) {
        t_err = "device allocation of the input copy failed";
        return COUPE_ERR_ALLOC;
    }
    double *d_pts = (double *)dbuf;
    double *d_w = (double *)(dbuf + ((pbytes + 255) & ~(size_t)255));
    uint64_t *d_part = (uint64_t *)((char *)d_w + ((wbytes + 255) & ~(size_t)255));
    static thread_local Staging st_p, st_w;
    const void *src_p = points->ptr;
    if (points->kind != 0) {
        double *h = (double *)st_p.get(pbytes);
        if (!h) return COUPE_ERR_ALLOC;
        for (uintptr_t i = 0; i < n; ++i) fetch(points, i, dimension * sizeof(double), h + i * dimension);
        src_p = h;
    }
    const void *src_w = weights->ptr;
    if (weights->kind != 0) {
        char *h = (char *)st_w.get(wbytes);
        if (!h) return COUPE_ERR_ALLOC;
        for (uintptr_t i = 0; i < n; ++i) fetch(weights, i, 8, h + i * 8);
        src_w = h;
    }
    cudaStream_t s = C->stream;
    cudaError_t e;
    if ((e = cudaMemcpyAsync(d_pts, src_p, pbytes, cudaMemcpyHostToDevice, s)) != cudaSuccess ||
        (e = cudaMemcpyAsync(d_w, src_w, wbytes, cudaMemcpyHostToDevice, s)) != cudaSuccess)
        return (coupe_err)cg::cuda_fail(e, "host to device copy", &t_err);
    const int rc = cg::multi_jagged(*C, n, (int)dimension, d_pts, d_w, part_count, max_iter, d_part, s, &err);
    if (rc != COUPE_ERR_OK) {
        cudaStreamSynchronize(s);
        t_err = err;
        return (coupe_err)rc;
    }
    if ((e = cudaMemcpyAsync(partition, d_part, obytes, cudaMemcpyDeviceToHost, s)) != cudaSuccess ||
        (e = cudaStreamSynchronize(s)) != cudaSuccess)
        return (coupe_err)cg::cuda_fail(e, "device to host copy", &t_err);
    return COUPE_ERR_OK;
}

enum coupe_err coupe_gpu_barycentres(uint64_t dimension, uint64_t n_nodes, const double *d_coords,
                                     uint64_t n_elements, uint64_t nodes_per_element, const uint64_t *d_nodes,
                                     double *d_out, void *stream) {
    t_err.clear();
    if (dimension != 2 && dimension != 3) return COUPE_ERR_BAD_DIMENSION;
    if (nodes_per_element != 2 && nodes_per_element != 3 && nodes_per_element != 4 && nodes_per_element != 8) {
        t_err = "elements of 2, 3, 4 or 8 nodes";
        return COUPE_ERR_BAD_TYPE;
    }
    if (n_elements == 0) return COUPE_ERR_OK;
    if (!d_coords || !d_nodes || !d_out) {
        t_err = "NULL array";
        return COUPE_ERR_CRASH;
    }
    std::string err;
    cg::DevCtx *C = cg::device_ctx(&err);
    if (!C) {
        t_err = err;
        return COUPE_ERR_CRASH;
    }
    std::lock_guard<std::mutex> lock(C->mu);
    const int rc = cg::barycentres(*C, (int)dimension, d_coords, n_nodes, nodes_per_element, d_nodes, n_elements,
                                   d_out, (cudaStream_t)stream, &err);
    if (rc != COUPE_ERR_OK) t_err = err;
    return (coupe_err)rc;
}

enum coupe_err coupe_gpu_parts_load(const uintptr_t *partition, uintptr_t num_parts, const coupe_data *weights,
                                    void *loads) {
    return host_loads(num_parts, partition, weights, loads, nullptr);
}

enum coupe_err coupe_gpu_imbalance(uintptr_t num_parts, const uintptr_t *partition, const coupe_data *weights,
                                   double *imbalance) {
    if (!imbalance) {
        t_err = "NULL imbalance";
        return COUPE_ERR_CRASH;
    }
    return host_loads(num_parts, partition, weights, nullptr, imbalance);
}

void coupe_gpu_last_stats(struct coupe_gpu_stats *out) {
    if (out) *out = t_stats;
}

enum coupe_err coupe_gpu_split_noalloc(uint64_t n, uint64_t dimension, const double *d_points,
                                       enum coupe_type weight_type, const void *d_weights, uint64_t coord, double cut,
                                       double *d_out_points, void *d_out_weights, uint64_t *n_left, void *stream) {
    t_err.clear();
    const char *msg = "";
    const int rc = cg::split_noalloc(n, dimension, d_points, weight_type, d_weights, coord, cut, d_out_points,
                                     d_out_weights, n_left, stream, &msg);
    if (rc != COUPE_ERR_OK) t_err = msg;  // host memory, error path only
    return (coupe_err)rc;
}

const char *coupe_gpu_last_error(void) { return t_err.c_str(); }

const char *coupe_gpu_version(void) { return "coupe-gpu 0.1.0 (sm_103a)"; }

int coupe_gpu_profile(int enable) {
    std::string err;
    cg::DevCtx *C = cg::device_ctx(&err);
    if (!C) return COUPE_ERR_CRASH;
    std::lock_guard<std::mutex> lock(C->mu);
    C->prof.on = enable != 0;
    C->prof.reset();
    return COUPE_ERR_OK;
}

int coupe_gpu_profile_read(uint64_t *counts, uint64_t *bytes, double *ms, int capacity) {
    std::string err;
    cg::DevCtx *C = cg::device_ctx(&err);
    if (!C) return 0;
    std::lock_guard<std::mutex> lock(C->mu);
    int n = capacity < cg::KID_COUNT ? capacity : cg::KID_COUNT;
    for (int i = 0; i < n; ++i) {
        if (counts) counts[i] = C->prof.count[i];
        if (bytes) bytes[i] = C->prof.bytes[i];
        if (ms) ms[i] = C->prof.ms[i];
    }
    return cg::KID_COUNT;
}

const char *coupe_gpu_kernel_name(int id) { return cg::kernel_name(id); }

static int *option_slot(const char *name) {
    if (!name) return nullptr;
    cg::Tuning &t = cg::tuning();
    if (!std::strcmp(name, "force_index_path")) return &t.force_index_path;
    if (!std::strcmp(name, "max_nbk")) return &t.max_nbk;
    if (!std::strcmp(name, "reorder_chunks_per_cta")) return &t.reorder_chunks_per_cta;
    if (!std::strcmp(name, "hist_ctas_per_sm")) return &t.hist_ctas_per_sm;
    if (!std::strcmp(name, "hist_waves")) return &t.hist_waves;
    if (!std::strcmp(name, "exact_f64_hist")) return &t.exact_f64_hist;
    if (!std::strcmp(name, "reorder_kernel")) return &t.reorder_kernel;
    if (!std::strcmp(name, "lookback_spin_limit")) return &t.lookback_spin_limit;
    if (!std::strcmp(name, "workspace_limit_mb")) return &t.workspace_limit_mb;
    if (!std::strcmp(name, "sync_levels")) return &t.sync_levels;
    if (!std::strcmp(name, "autotune_cache")) return &t.autotune_cache;
    return nullptr;
}

int coupe_gpu_set_option(const char *name, int64_t value) {
    int *p = option_slot(name);
    if (!p) return COUPE_ERR_BAD_TYPE;
    *p = (int)value;
    return COUPE_ERR_OK;
}

int64_t coupe_gpu_get_option(const char *name) {
    int *p = option_slot(name);
    return p ? *p : -1;
}

}  // extern "C"

namespace {

// The autotuner's choices by workload class: the number of points and of sets
// (powers of two), the dimension, weight type, precision mode and deepest
// iteration count.  Kept for the process and, when the environment variable
// COUPE_GPU_TUNE_CACHE names a file, in that file (one line per class,
// appended when a class is first tuned, read at the first lookup).
struct TuneEntry {
    int max_nbk, hist_ctas_per_sm, reorder_chunks_per_cta, hist_waves;
    double ms;
};
std::mutex g_tune_mu;
std::map<std::string, TuneEntry> g_tune;
bool g_tune_loaded = false;

int log2_floor(uint64_t v) {
    int l = 0;
    while (v > 1) {
        v >>= 1;
        ++l;
    }
    return l;
}

std::string tune_key(uint64_t n, uint64_t nsets, uint64_t dim, int wtype, int mode, uint32_t iters) {
    char b[96];
    snprintf(b, sizeof(b), "n2^%d/sets2^%d/d%llu/w%d/m%d/it%u", log2_floor(n), log2_floor(nsets),
             (unsigned long long)dim, wtype, mode, iters);
    return b;
}

void tune_load_locked() {
    if (g_tune_loaded) return;
    g_tune_loaded = true;
    const char *path = std::getenv("COUPE_GPU_TUNE_CACHE");
    if (!path || !*path) return;
    FILE *f = std::fopen(path, "r");
    if (!f) return;
    char key[128];
    TuneEntry e;
    while (std::fscanf(f, "%127s %d %d %d %d %lf", key, &e.max_nbk, &e.hist_ctas_per_sm, &e.reorder_chunks_per_cta,
                       &e.hist_waves, &e.ms) == 6)
        g_tune[key] = e;
    std::fclose(f);
}

void tune_store_locked(const std::string &key, const TuneEntry &e) {
    g_tune[key] = e;
    const char *path = std::getenv("COUPE_GPU_TUNE_CACHE");
    if (!path || !*path) return;
    FILE *f = std::fopen(path, "a");
    if (!f) return;
    std::fprintf(f, "%s %d %d %d %d %.6f\n", key.c_str(), e.max_nbk, e.hist_ctas_per_sm, e.reorder_chunks_per_cta,
                 e.hist_waves, e.ms);
    std::fclose(f);
}

}  // namespace

extern "C" {

enum coupe_err coupe_gpu_autotune(uint64_t *d_partition, uint64_t nsets, const uint64_t *set_offsets,
                                  uint64_t dimension, const double *d_points, enum coupe_type weight_type,
                                  const void *d_weights, const uint32_t *iter_counts, double tolerance, int mode,
                                  void *stream, int repeats, struct coupe_gpu_tuning *best) {
    // Candidate schedules: bisection steps per histogram pass, histogram CTAs
    // per SM and waves of them, and reorder chunks per CTA.  None changes the
    // ids, so the fastest (median device time of `repeats` runs) is kept.
    cg::Tuning &t = cg::tuning();
    const cg::Tuning keep = t;
    const int reps = repeats < 1 ? 1 : (repeats > 15 ? 15 : repeats);
    // a workload class tuned before: its schedule, without timing
    uint32_t it_max = 0;
    for (uint64_t k = 0; k < nsets && iter_counts; ++k) it_max = std::max(it_max, iter_counts[k]);
    const uint64_t npts = nsets && set_offsets ? set_offsets[nsets] : 0;
    const std::string key = tune_key(npts, nsets, dimension, (int)weight_type, mode, it_max);
    if (cg::tuning().autotune_cache) {
        std::lock_guard<std::mutex> lock(g_tune_mu);
        tune_load_locked();
        auto hit = g_tune.find(key);
        if (hit != g_tune.end()) {
            t.max_nbk = hit->second.max_nbk;
            t.hist_ctas_per_sm = hit->second.hist_ctas_per_sm;
            t.reorder_chunks_per_cta = hit->second.reorder_chunks_per_cta;
            t.hist_waves = hit->second.hist_waves;
            if (best) {
                best->max_nbk = t.max_nbk;
                best->hist_ctas_per_sm = t.hist_ctas_per_sm;
                best->reorder_chunks_per_cta = t.reorder_chunks_per_cta;
                best->hist_waves = t.hist_waves;
                best->device_ms = hit->second.ms;
            }
            return COUPE_ERR_OK;
        }
    }
    double best_ms = 1e300;
    cg::Tuning best_t = keep;
    for (int nbk : {10, 9, 8, 7, 6})
        for (int hc : {0, 3, 2})
            for (int rc : {1, 2})
                for (int hw : {1, 2}) {
                t = keep;
                t.max_nbk = nbk;
                t.hist_ctas_per_sm = hc;
                t.reorder_chunks_per_cta = rc;
                t.hist_waves = hw;
                std::vector<double> ms;
                for (int r = 0; r < reps + 1; ++r) {
                    const coupe_err rc_ = coupe_gpu_rcb_batched(d_partition, nsets, set_offsets, dimension, d_points,
                                                                weight_type, d_weights, iter_counts, tolerance, mode,
                                                                stream);
                    if (rc_ != COUPE_ERR_OK) {
                        t = keep;
                        return rc_;
                    }
                    if (r > 0) ms.push_back(t_stats.device_ms);  // the first run warms up
                }
                std::sort(ms.begin(), ms.end());
                const double med = ms[ms.size() / 2];
                if (med < best_ms) {
                    best_ms = med;
                    best_t = t;
                }
            }
    t = best_t;
    if (cg::tuning().autotune_cache) {
        std::lock_guard<std::mutex> lock(g_tune_mu);
        tune_store_locked(key, TuneEntry{best_t.max_nbk, best_t.hist_ctas_per_sm, best_t.reorder_chunks_per_cta,
                                         best_t.hist_waves, best_ms});
    }
    if (best) {
        best->max_nbk = best_t.max_nbk;
        best->hist_ctas_per_sm = best_t.hist_ctas_per_sm;
        best->reorder_chunks_per_cta = best_t.reorder_chunks_per_cta;
        best->hist_waves = best_t.hist_waves;
        best->device_ms = best_ms;
    }
    return COUPE_ERR_OK;
}

}  // extern "C"
