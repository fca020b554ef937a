// Device contexts, workspace management, mode dispatch and the Rib basis
// change (OrientedBoundingBox::from_points, coupe/src/geometry.rs:210-228).
#include <cmath>
#include <cstring>
#include <map>
#include <memory>
#include <mutex>

#include "engine.h"
#include "kernels.cuh"

namespace cg {

Tuning &tuning() {
    static Tuning t;
    return t;
}

const char *kernel_name(int id) {
    // KID_ASSIGN: the kernel writing the part ids (a traversal, or k_assign)
    static const char *names[KID_COUNT] = {"k_convert", "k_wabs_max", "k_wsum", "k_root", "k_hist", "k_decide",
                                           "k_children", "k_reorder", "k_ids", "k_fill_u64", "k_moments",
                                           "k_part_loads", "k_barycentres", "k_grid"};
    return id >= 0 && id < KID_COUNT ? names[id] : "?";
}

cudaEvent_t Profiler::take() {
    if (!pool.empty()) {
        cudaEvent_t e = pool.back();
        pool.pop_back();
        return e;
    }
    cudaEvent_t e = nullptr;
    if (cudaEventCreate(&e) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    return e;
}

void Profiler::begin(int id, uint64_t nbytes, cudaStream_t s) {
    if (!on) return;
    Rec r;
    r.id = id;
    r.bytes = nbytes;
    r.a = take();
    r.b = take();
    if (!r.a || !r.b) return;
    cudaEventRecord(r.a, s);
    recs.push_back(r);
}

void Profiler::end(cudaStream_t s) {
    if (!on || recs.empty()) return;
    cudaEventRecord(recs.back().b, s);
}

void Profiler::resolve() {
    for (const Rec &r : recs) {
        float ms_ = 0.f;
        if (cudaEventElapsedTime(&ms_, r.a, r.b) == cudaSuccess) {
            count[r.id] += 1;
            bytes[r.id] += r.bytes;
            ms[r.id] += ms_;
        } else {
            cudaGetLastError();
        }
        pool.push_back(r.a);
        pool.push_back(r.b);
    }
    recs.clear();
}

void Profiler::reset() {
    for (int i = 0; i < KID_COUNT; ++i) {
        count[i] = 0;
        bytes[i] = 0;
        ms[i] = 0.0;
    }
}

int cuda_fail(cudaError_t e, const char *what, std::string *err) {
    if (err) *err = std::string(what) + ": " + cudaGetErrorString(e);
    cudaGetLastError();  // clear a sticky launch error of this thread
    return e == cudaErrorMemoryAllocation ? COUPE_ERR_ALLOC : COUPE_ERR_CRASH;
}

static std::mutex g_ctx_mu;
static std::map<int, std::unique_ptr<DevCtx>> g_ctx;

DevCtx *device_ctx(std::string *err) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) {
        cuda_fail(e, "cudaGetDevice", err);
        return nullptr;
    }
    std::lock_guard<std::mutex> g(g_ctx_mu);
    auto it = g_ctx.find(dev);
    if (it != g_ctx.end()) return it->second.get();
    std::unique_ptr<DevCtx> c(new DevCtx());
    c->dev = dev;
    if ((e = cudaDeviceGetAttribute(&c->sms, cudaDevAttrMultiProcessorCount, dev)) != cudaSuccess ||
        (e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking)) != cudaSuccess ||
        (e = cudaStreamCreateWithFlags(&c->stream2, cudaStreamNonBlocking)) != cudaSuccess ||
        (e = cudaEventCreateWithFlags(&c->ev_pts, cudaEventDisableTiming)) != cudaSuccess ||
        (e = cudaEventCreateWithFlags(&c->ev_w, cudaEventDisableTiming)) != cudaSuccess ||
        (e = cudaMallocHost(&c->h_pinned, 4096)) != cudaSuccess ||
        (e = cudaEventCreate(&c->ev0)) != cudaSuccess || (e = cudaEventCreate(&c->ev1)) != cudaSuccess) {
        cuda_fail(e, "device context", err);
        return nullptr;
    }
    DevCtx *r = c.get();
    g_ctx[dev] = std::move(c);
    return r;
}

int ensure_workspace(DevCtx &C, size_t bytes, std::string *err) {
    const int lim = tuning().workspace_limit_mb;
    if (lim > 0 && bytes > ((size_t)lim << 20)) {
        *err = "workspace of " + std::to_string(bytes) + " bytes exceeds the limit of " + std::to_string(lim) +
               " MiB (option workspace_limit_mb)";
        return COUPE_ERR_ALLOC;
    }
    if (bytes <= C.ws_cap) return COUPE_ERR_OK;
    if (C.ws) {
        cudaStreamSynchronize(C.stream);
        cudaFree(C.ws);
        C.ws = nullptr;
        C.ws_cap = 0;
    }
    size_t cap = bytes + bytes / 8;
    cudaError_t e = cudaMalloc(&C.ws, cap);
    if (e != cudaSuccess) return cuda_fail(e, "cudaMalloc workspace", err);
    C.ws_cap = cap;
    return COUPE_ERR_OK;
}

static __global__ void k_f64_to_f32(const double *__restrict__ in, float *__restrict__ out, uint64_t n) {
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x)
        out[i] = KeyF32::from_f64_bits(f64_bits(in[i]));
}

int f64_to_f32(DevCtx &C, const double *d_in, float *d_out, uint64_t n, cudaStream_t stream, std::string *err) {
    cudaStream_t s = stream ? stream : C.stream;
    if (n == 0) return COUPE_ERR_OK;
    const unsigned grid = (unsigned)std::min<uint64_t>((n + 255) / 256, (uint64_t)C.sms * 8);
    k_f64_to_f32<<<grid, 256, 0, s>>>(d_in, d_out, n);
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    return e == cudaSuccess ? COUPE_ERR_OK : cuda_fail(e, "k_f64_to_f32", err);
}

int run_rcb(DevCtx &C, const RunArgs &a, coupe_gpu_stats *st, std::string *err) {
    st->mode = a.mode;
    switch (a.mode) {
    case COUPE_GPU_REF32:
        return run_rcb_ref32(C, a, st, err);
    case COUPE_GPU_F64:
        return run_rcb_f64(C, a, st, err);
    case COUPE_GPU_F32KEY_F64BAND:
        return run_rcb_band(C, a, st, err);
    default:
        if (err) *err = "precision mode not available in this build";
        return COUPE_ERR_BAD_TYPE;
    }
}

// ---------------------------------------------------------------------------
// Rib basis change.  inertia_matrix (geometry.rs:273-284) is unweighted: the
// centroid c = sum(p)/n, then M = sum((p-c)(p-c)^T).  One pass computes it:
// with s = the first point, W = sum(w), S1 = sum(w (p - s)) and the upper
// triangle of S2 = sum(w (p - s)(p - s)^T); then c = s + S1 / W and
// M = S2 - S1 S1^T / W (w = 1 for coupe's matrix; the point weights for the
// opt-in weighted inertia).  The shift keeps the subtraction well
// conditioned.  Sums are reduced in a fixed order (fixed grid, fixed tree in
// each block, blocks summed in index order on the host), so the result does
// not change from run to run.  GB300 runs f64 arithmetic at a small fraction
// of its integer rate and this pass is bound by it: the upper triangle halves
// the products, and the one pass reads the points once.
// ---------------------------------------------------------------------------
constexpr int RIB_GRID = 1024;

template <int D>
__host__ __device__ constexpr int moment_terms() {
    return 1 + D + D * (D + 1) / 2;  // W, S1, upper triangle of S2
}

template <int D, class WS>
__global__ void __launch_bounds__(BLOCK) k_moments(const double *__restrict__ pts, uint64_t n,
                                                   const WS *__restrict__ w, double *partial) {
    constexpr int K = moment_terms<D>();
    __shared__ double sh[K][NWARPS];
    double acc[K];
#pragma unroll
    for (int k = 0; k < K; ++k) acc[k] = 0.0;
    double sft[D];
#pragma unroll
    for (int d = 0; d < D; ++d) sft[d] = pts[d];
    for (uint64_t i = (uint64_t)blockIdx.x * BLOCK + threadIdx.x; i < n; i += (uint64_t)gridDim.x * BLOCK) {
        double o[D], wo[D];
#pragma unroll
        for (int d = 0; d < D; ++d) o[d] = __dsub_rn(pts[i * D + d], sft[d]);
        if (w) {
            const double wi = (double)w[i];
            acc[0] = __dadd_rn(acc[0], wi);
#pragma unroll
            for (int d = 0; d < D; ++d) wo[d] = __dmul_rn(wi, o[d]);
        } else {
#pragma unroll
            for (int d = 0; d < D; ++d) wo[d] = o[d];
        }
#pragma unroll
        for (int d = 0; d < D; ++d) acc[1 + d] = __dadd_rn(acc[1 + d], wo[d]);
        int k = 1 + D;
#pragma unroll
        for (int a = 0; a < D; ++a)
#pragma unroll
            for (int b2 = a; b2 < D; ++b2, ++k) acc[k] = __dadd_rn(acc[k], __dmul_rn(wo[a], o[b2]));
    }
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int k = 0; k < K; ++k) {
        double v = acc[k];
        for (int off = 16; off > 0; off >>= 1) v = __dadd_rn(v, __shfl_down_sync(0xffffffffu, v, off));
        if (lane == 0) sh[k][warp] = v;
    }
    __syncthreads();
    if (threadIdx.x < K) {
        double v = 0.0;
        for (int w2 = 0; w2 < NWARPS; ++w2) v = __dadd_rn(v, sh[threadIdx.x][w2]);
        partial[blockIdx.x * K + threadIdx.x] = v;
    }
}

// ---------------------------------------------------------------------------
// The unweighted sums (coupe's matrix) without f64 arithmetic per point:
// each coordinate is split into an f32 pair (hi = RN32(x), lo = RN32(x - hi),
// hi + lo within 2^-48 |x|) by integer instructions, and the offsets, their
// products and the per-thread sums are pair arithmetic (error-free sums and
// fused-multiply-add products; Dekker 1971, Shewchuk 1997), good to about
// 2^-44 relative.  GB300's FP64 pipe runs at 1/64 of the f32 rate, and the f64
// version of this pass was bound by it.  A point with a coordinate outside
// [2^-50, 2^50] in magnitude (zeros excepted) is added in f64 instead.  The
// per-thread sums then join the same fixed-order f64 reduction.  (F2 and
// its helpers are in common.cuh.)
// ---------------------------------------------------------------------------
template <int D>
__global__ void __launch_bounds__(BLOCK) k_moments_f2(const double *__restrict__ pts, uint64_t n, double *partial) {
    constexpr int K = moment_terms<D>();
    __shared__ double sh[K][NWARPS];
    F2 acc[K];
    double slow[K];  // points outside the pairs' range
#pragma unroll
    for (int k = 0; k < K; ++k) {
        acc[k] = {0.0f, 0.0f};
        slow[k] = 0.0;
    }
    double sft[D];
    F2 sft2[D];
    bool sft_ok = true;
#pragma unroll
    for (int d = 0; d < D; ++d) {
        sft[d] = pts[d];
        sft_ok = f2_split(sft[d], sft2[d]) && sft_ok;
    }
    for (uint64_t i = (uint64_t)blockIdx.x * BLOCK + threadIdx.x; i < n; i += (uint64_t)gridDim.x * BLOCK) {
        double p[D];
        F2 o[D];
        bool ok = sft_ok;
#pragma unroll
        for (int d = 0; d < D; ++d) {
            p[d] = pts[i * D + d];
            F2 q;
            ok = f2_split(p[d], q) && ok;
            o[d] = f2_sub(q, sft2[d]);
        }
        if (ok) {
#pragma unroll
            for (int d = 0; d < D; ++d) f2_add(acc[1 + d], o[d]);
            int k = 1 + D;
#pragma unroll
            for (int a = 0; a < D; ++a)
#pragma unroll
                for (int b2 = a; b2 < D; ++b2, ++k) f2_add(acc[k], f2_mul(o[a], o[b2]));
        } else {
            double od[D];
#pragma unroll
            for (int d = 0; d < D; ++d) {
                od[d] = __dsub_rn(p[d], sft[d]);
                slow[1 + d] = __dadd_rn(slow[1 + d], od[d]);
            }
            int k = 1 + D;
#pragma unroll
            for (int a = 0; a < D; ++a)
#pragma unroll
                for (int b2 = a; b2 < D; ++b2, ++k) slow[k] = __dadd_rn(slow[k], __dmul_rn(od[a], od[b2]));
        }
    }
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int k = 0; k < K; ++k) {
        double v = __dadd_rn(__dadd_rn((double)acc[k].h, (double)acc[k].l), slow[k]);
        for (int off = 16; off > 0; off >>= 1) v = __dadd_rn(v, __shfl_down_sync(0xffffffffu, v, off));
        if (lane == 0) sh[k][warp] = v;
    }
    __syncthreads();
    if (threadIdx.x < K) {
        double v = 0.0;
        for (int w2 = 0; w2 < NWARPS; ++w2) v = __dadd_rn(v, sh[threadIdx.x][w2]);
        partial[blockIdx.x * K + threadIdx.x] = v;
    }
}

// Symmetric eigenvectors by cyclic Jacobi rotations (Golub & Van Loan,
// Matrix Computations, section 8.5), columns of v.
static void sym_eigen(const double *a_in, int n, double *ev, double *v) {
    double a[9];
    std::memcpy(a, a_in, sizeof(double) * n * n);
    for (int i = 0; i < n * n; ++i) v[i] = 0.0;
    for (int i = 0; i < n; ++i) v[i * n + i] = 1.0;
    for (int sweep = 0; sweep < 100; ++sweep) {
        double off = 0.0, diag = 0.0;
        for (int p = 0; p < n; ++p) {
            diag += a[p * n + p] * a[p * n + p];
            for (int q = p + 1; q < n; ++q) off += a[p * n + q] * a[p * n + q];
        }
        if (off == 0.0 || off <= 1e-300 * diag) break;
        for (int p = 0; p < n - 1; ++p)
            for (int q = p + 1; q < n; ++q) {
                const double apq = a[p * n + q];
                if (apq == 0.0) continue;
                const double tau = (a[q * n + q] - a[p * n + p]) / (2.0 * apq);
                const double t = (tau >= 0.0 ? 1.0 : -1.0) / (std::fabs(tau) + std::sqrt(1.0 + tau * tau));
                const double c = 1.0 / std::sqrt(1.0 + t * t), s = t * c;
                for (int k = 0; k < n; ++k) {  // A <- A J
                    const double x = a[k * n + p], y = a[k * n + q];
                    a[k * n + p] = c * x - s * y;
                    a[k * n + q] = s * x + c * y;
                }
                for (int k = 0; k < n; ++k) {  // A <- J^T A
                    const double x = a[p * n + k], y = a[q * n + k];
                    a[p * n + k] = c * x - s * y;
                    a[q * n + k] = s * x + c * y;
                }
                for (int k = 0; k < n; ++k) {  // V <- V J
                    const double x = v[k * n + p], y = v[k * n + q];
                    v[k * n + p] = c * x - s * y;
                    v[k * n + q] = s * x + c * y;
                }
            }
    }
    for (int i = 0; i < n; ++i) ev[i] = a[i * n + i];
}

// approx 0.5's default ulps comparison: |a-b| <= f64::EPSILON, else same sign
// and at most 4 representable values apart.
static bool ulps_close(double a, double b) {
    if (std::fabs(a - b) <= 2.220446049250313e-16) return true;
    if (std::signbit(a) != std::signbit(b)) return false;
    int64_t x, y;
    std::memcpy(&x, &a, 8);
    std::memcpy(&y, &b, 8);
    return (x > y ? x - y : y - x) <= 4;
}

// householder_reflection (geometry.rs:305-319) then its inverse (:219).
static bool obb_matrix(const double *inertia, int D, double *out) {
    double ev[3], V[9], v[3];
    sym_eigen(inertia, D, ev, V);
    int best = 0;
    for (int i = 1; i < D; ++i)
        if (ev[i] > ev[best]) best = i;
    for (int i = 0; i < D; ++i) v[i] = V[i * D + best];
    double nn = 0.0;
    for (int i = 0; i < D; ++i) nn += v[i] * v[i];
    const double nrm = std::sqrt(nn);
    double H[9];
    for (int i = 0; i < D * D; ++i) H[i] = 0.0;
    for (int i = 0; i < D; ++i) H[i * D + i] = 1.0;
    bool parallel = true;
    for (int i = 0; i < D; ++i) parallel = parallel && ulps_close(v[i] / nrm, i == 0 ? 1.0 : 0.0);
    if (!parallel) {
        const double sign = v[0] > 0.0 ? -1.0 : 1.0;
        double w[3];
        for (int i = 0; i < D; ++i) w[i] = v[i] + (i == 0 ? sign * nrm : 0.0);
        double wtw = 0.0;
        for (int i = 0; i < D; ++i) wtw += w[i] * w[i];
        for (int i = 0; i < D; ++i)
            for (int j = 0; j < D; ++j) H[i * D + j] -= 2.0 * w[i] * w[j] / wtw;
    }
    // inverse by the adjugate
    if (D == 2) {
        const double det = H[0] * H[3] - H[1] * H[2];
        if (det == 0.0) return false;
        out[0] = H[3] / det;
        out[1] = -H[1] / det;
        out[2] = -H[2] / det;
        out[3] = H[0] / det;
        return true;
    }
    double cof[9];
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) {
            const int r0 = (i + 1) % 3, r1 = (i + 2) % 3, c0 = (j + 1) % 3, c1 = (j + 2) % 3;
            cof[i * 3 + j] = H[r0 * 3 + c0] * H[r1 * 3 + c1] - H[r0 * 3 + c1] * H[r1 * 3 + c0];
        }
    const double det = H[0] * cof[0] + H[1] * cof[1] + H[2] * cof[2];
    if (det == 0.0) return false;
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) out[i * 3 + j] = cof[j * 3 + i] / det;
    return true;
}

template <int D, class WS>
static int launch_moments(const double *d_points, uint64_t n, const WS *d_w, double *d_part, cudaStream_t s,
                          std::string *err) {
    k_moments<D, WS><<<RIB_GRID, BLOCK, 0, s>>>(d_points, n, d_w, d_part);
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? (int)COUPE_ERR_OK : cuda_fail(e, "k_moments", err);
}

int rib_matrix(DevCtx &C, uint64_t n, int dim, const double *d_points, cudaStream_t stream, double *out,
               std::string *err, int wtype, const void *d_weights) {
    cudaStream_t s = stream ? stream : C.stream;
    const int K = dim == 2 ? moment_terms<2>() : moment_terms<3>();
    const size_t part_bytes = (size_t)RIB_GRID * K * sizeof(double);
    int rc = ensure_workspace(C, part_bytes, err);
    if (rc != COUPE_ERR_OK) return rc;
    double *d_part = (double *)C.ws;
    std::unique_ptr<double[]> h(new double[RIB_GRID * K]);
    const bool weighted = d_weights != nullptr;
    if (!weighted) {
        if (dim == 2)
            k_moments_f2<2><<<RIB_GRID, BLOCK, 0, s>>>(d_points, n, d_part);
        else
            k_moments_f2<3><<<RIB_GRID, BLOCK, 0, s>>>(d_points, n, d_part);
        const cudaError_t le = cudaGetLastError();
        rc = le == cudaSuccess ? (int)COUPE_ERR_OK : cuda_fail(le, "k_moments_f2", err);
    } else if (wtype == COUPE_INT) {
        rc = dim == 2 ? launch_moments<2>(d_points, n, (const int32_t *)d_weights, d_part, s, err)
                      : launch_moments<3>(d_points, n, (const int32_t *)d_weights, d_part, s, err);
    } else if (wtype == COUPE_INT64) {
        rc = dim == 2 ? launch_moments<2>(d_points, n, (const int64_t *)d_weights, d_part, s, err)
                      : launch_moments<3>(d_points, n, (const int64_t *)d_weights, d_part, s, err);
    } else {
        rc = dim == 2 ? launch_moments<2>(d_points, n, (const double *)d_weights, d_part, s, err)
                      : launch_moments<3>(d_points, n, (const double *)d_weights, d_part, s, err);
    }
    if (rc != COUPE_ERR_OK) return rc;
    cudaError_t e;
    if ((e = cudaMemcpyAsync(h.get(), d_part, part_bytes, cudaMemcpyDeviceToHost, s)) != cudaSuccess ||
        (e = cudaStreamSynchronize(s)) != cudaSuccess)
        return cuda_fail(e, "inertia", err);
    double t[10] = {0, 0, 0, 0, 0, 0, 0, 0, 0, 0};
    for (int b = 0; b < RIB_GRID; ++b)
        for (int k = 0; k < K; ++k) t[k] += h[b * K + k];
    const double W = weighted ? t[0] : (double)n;
    if (!(W > 0.0) || !std::isfinite(W)) {
        if (err) *err = "weighted inertia needs a positive finite weight sum";
        return COUPE_ERR_BAD_TYPE;
    }
    double m[9];
    int k = 1 + dim;
    for (int a = 0; a < dim; ++a)
        for (int b = a; b < dim; ++b, ++k) {
            const double v = t[k] - t[1 + a] * t[1 + b] / W;
            m[a * dim + b] = m[b * dim + a] = v;
        }
    if (!obb_matrix(m, dim, out)) {
        if (err) *err = "singular basis change";
        return COUPE_ERR_CRASH;
    }
    return COUPE_ERR_OK;
}

}  // namespace cg
