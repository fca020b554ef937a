// Part loads and imbalance of a partition, on the device: coupe's
// compute_parts_load and imbalance (coupe/src/imbalance.rs:14-77), the
// check that follows a partition (arc_swap.rs:447, tools/num-part/main.rs:250).
//
// One kernel streams the part ids (8 B) and weights (4 or 8 B) of every
// point once and adds each weight to its part's load: per CTA in shared
// memory when the loads fit (up to PRIV_MAX_BYTES), then one global atomic
// per non-zero load; else straight into global memory.  Consecutive points
// of a mesh often share a part, so a warp whose 32 points all have one part
// adds their sum once (32 lanes adding to one word are 32 serialised
// updates).  The last, O(parts), step runs on the host in the reference's
// order.
//
// Weights: i32 and i64 loads are sums with wrap-around, as coupe's release
// build computes them; f64 loads are the 128-bit fixed-point sums of
// common.cuh read back to f64 (one rounding; coupe's own f64 sums depend on
// rayon's split order).  A part id >= num_parts is an error (coupe indexes
// its load vector with it and panics).
#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>
#include <cstring>
#include <string>
#include <vector>

#include "engine.h"
#include "kernels.cuh"

namespace cg {

namespace {

constexpr uint32_t LOADS_BAD_ID = 1, LOADS_NONFINITE = 2;
constexpr size_t PRIV_MAX_BYTES = 96 * 1024;

struct LoadsScratch {
    unsigned long long amax_bits;  // largest |w| of f64 weights, as bits
    unsigned long long first_bad;  // smallest index of an out-of-range id
    uint32_t flags;
    uint32_t pad;
};

__global__ void __launch_bounds__(BLOCK) k_loads_wmax(const double *__restrict__ w, uint64_t n, LoadsScratch *sc) {
    uint64_t m = 0;
    for (uint64_t i = (uint64_t)blockIdx.x * BLOCK + threadIdx.x; i < n; i += (uint64_t)gridDim.x * BLOCK) {
        const uint64_t b = (uint64_t)__double_as_longlong(w[i]) & 0x7fffffffffffffffull;
        m = b > m ? b : m;
    }
    m = warp_max_u64(m);
    if ((threadIdx.x & 31) == 0) {
        atomicMax(&sc->amax_bits, (unsigned long long)m);
        if (m >= 0x7ff0000000000000ull) atomicOr(&sc->flags, LOADS_NONFINITE);
    }
}

// A weight as L 64-bit addends of its part's load.
__device__ __forceinline__ void load_limbs(int32_t w, int, uint64_t *q) { q[0] = (uint64_t)(int64_t)w; }
__device__ __forceinline__ void load_limbs(int64_t w, int, uint64_t *q) { q[0] = (uint64_t)w; }
__device__ __forceinline__ void load_limbs(double w, int fs, uint64_t *q) {
    const unsigned __int128 v = fixed_q_bits(w, fs);
    q[0] = (uint32_t)v;
    q[1] = (uint32_t)(v >> 32);
    q[2] = (uint32_t)(v >> 64);
    q[3] = (uint32_t)(v >> 96);
}

template <class W, int L>
__global__ void __launch_bounds__(BLOCK) k_part_loads(const uint64_t *__restrict__ part, const W *__restrict__ w,
                                                      uint64_t n, uint64_t P, int priv,
                                                      unsigned long long *__restrict__ acc, LoadsScratch *sc) {
    extern __shared__ unsigned long long sacc[];
    if (L > 1 && (sc->flags & LOADS_NONFINITE)) return;  // the call fails; nothing to add
    const int fs = L > 1 ? fixed_scale_from_max(__longlong_as_double((long long)sc->amax_bits), n) : 0;
    if (priv) {
        for (uint64_t j = threadIdx.x; j < P * L; j += BLOCK) sacc[j] = 0;
        __syncthreads();
    }
    unsigned long long *dst = priv ? sacc : acc;
    const int lane = threadIdx.x & 31;
    const uint64_t warps = (uint64_t)gridDim.x * NWARPS;
    // every lane of a warp runs every iteration (full-mask votes below)
    for (uint64_t base = ((uint64_t)blockIdx.x * NWARPS + (threadIdx.x >> 5)) * 32; base < n; base += warps * 32) {
        const uint64_t i = base + lane;
        uint64_t p = ~0ull, q[L];
#pragma unroll
        for (int l = 0; l < L; ++l) q[l] = 0;
        if (i < n) {
            p = part[i];
            if (p >= P) {
                atomicOr(&sc->flags, LOADS_BAD_ID);
                atomicMin(&sc->first_bad, (unsigned long long)i);
                p = ~0ull;
            } else {
                load_limbs(w[i], fs, q);
            }
        }
        const uint64_t p0 = __shfl_sync(0xffffffffu, p, 0);
        if (__all_sync(0xffffffffu, p == p0)) {
            if (p0 != ~0ull) {
#pragma unroll
                for (int l = 0; l < L; ++l) {
                    const uint64_t s = warp_sum_u64(q[l]);
                    if (lane == 0 && s) atomicAdd(&dst[p0 * L + l], (unsigned long long)s);
                }
            }
        } else if (p != ~0ull) {
#pragma unroll
            for (int l = 0; l < L; ++l)
                if (q[l]) atomicAdd(&dst[p * L + l], (unsigned long long)q[l]);
        }
    }
    if (priv) {
        __syncthreads();
        for (uint64_t j = threadIdx.x; j < P * L; j += BLOCK)
            if (sacc[j]) atomicAdd(&acc[j], sacc[j]);
    }
}

template <class W, int L>
int launch_loads(DevCtx &C, const uint64_t *d_part, const W *d_w, uint64_t n, uint64_t P, cudaStream_t s,
                 unsigned long long *acc, LoadsScratch *sc, std::string *err) {
    const size_t smem = (size_t)P * L * sizeof(unsigned long long);
    const int priv = smem <= PRIV_MAX_BYTES ? 1 : 0;
    const size_t dyn = priv ? smem : 0;
    const void *fn = (const void *)k_part_loads<W, L>;
    cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)PRIV_MAX_BYTES);
    if (e != cudaSuccess) return cuda_fail(e, "k_part_loads attribute", err);
    int per = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, fn, BLOCK, dyn) != cudaSuccess || per < 1) per = 1;
    // one resident wave: each CTA clears and flushes its loads once
    const uint64_t want = (n + BLOCK - 1) / BLOCK;
    const unsigned grid = (unsigned)std::max<uint64_t>(1, std::min<uint64_t>(want, (uint64_t)per * C.sms));
    C.prof.begin(KID_LOADS, n * (8 + sizeof(W)), s);
    k_part_loads<W, L><<<grid, BLOCK, dyn, s>>>(d_part, d_w, n, P, priv, acc, sc);
    if ((e = cudaGetLastError()) != cudaSuccess) return cuda_fail(e, "k_part_loads", err);
    C.prof.end(s);
    return COUPE_ERR_OK;
}

}  // namespace

int parts_load(DevCtx &C, const uint64_t *d_part, uint64_t n, int wtype, const void *d_w, uint64_t P,
               cudaStream_t stream, void *loads, std::string *err) {
    cudaStream_t s = stream ? stream : C.stream;
    const int L = wtype == COUPE_DOUBLE ? 4 : 1;
    if (P == 0 && n == 0) return COUPE_ERR_OK;
    if (P == 0 || P > (1ull << 40)) {
        if (err) *err = P == 0 ? "a part id is out of range (no parts)" : "too many parts";
        return P == 0 ? COUPE_ERR_BAD_TYPE : COUPE_ERR_ALLOC;
    }
    const size_t acc_bytes = (size_t)P * L * sizeof(unsigned long long);
    int rc = ensure_workspace(C, acc_bytes + 256, err);
    if (rc != COUPE_ERR_OK) return rc;
    LoadsScratch *sc = (LoadsScratch *)C.ws;
    unsigned long long *acc = (unsigned long long *)((char *)C.ws + 256);
    LoadsScratch init{};
    init.first_bad = ~0ull;
    cudaError_t e;
    if ((e = cudaMemcpyAsync(sc, &init, sizeof(init), cudaMemcpyHostToDevice, s)) != cudaSuccess ||
        (e = cudaMemsetAsync(acc, 0, acc_bytes, s)) != cudaSuccess)
        return cuda_fail(e, "loads set-up", err);
    if (n > 0) {
        if (wtype == COUPE_DOUBLE) {
            const unsigned g = (unsigned)std::max<uint64_t>(1, std::min<uint64_t>((n + BLOCK - 1) / BLOCK,
                                                                                   (uint64_t)C.sms * 4));
            C.prof.begin(KID_WABS, n * 8, s);
            k_loads_wmax<<<g, BLOCK, 0, s>>>((const double *)d_w, n, sc);
            if ((e = cudaGetLastError()) != cudaSuccess) return cuda_fail(e, "k_loads_wmax", err);
            C.prof.end(s);
            rc = launch_loads<double, 4>(C, d_part, (const double *)d_w, n, P, s, acc, sc, err);
        } else if (wtype == COUPE_INT64) {
            rc = launch_loads<int64_t, 1>(C, d_part, (const int64_t *)d_w, n, P, s, acc, sc, err);
        } else {
            rc = launch_loads<int32_t, 1>(C, d_part, (const int32_t *)d_w, n, P, s, acc, sc, err);
        }
        if (rc != COUPE_ERR_OK) return rc;
    }
    std::vector<unsigned long long> h(P * L);
    LoadsScratch hs;
    if ((e = cudaMemcpyAsync(&hs, sc, sizeof(hs), cudaMemcpyDeviceToHost, s)) != cudaSuccess ||
        (e = cudaMemcpyAsync(h.data(), acc, acc_bytes, cudaMemcpyDeviceToHost, s)) != cudaSuccess ||
        (e = cudaStreamSynchronize(s)) != cudaSuccess)
        return cuda_fail(e, "loads read-back", err);
    C.prof.resolve();
    if (hs.flags & LOADS_NONFINITE) {
        if (err) *err = "non-finite weight";
        return COUPE_ERR_BAD_TYPE;
    }
    if (hs.flags & LOADS_BAD_ID) {
        if (err) *err = "part id out of range at index " + std::to_string(hs.first_bad);
        return COUPE_ERR_BAD_TYPE;
    }
    if (wtype == COUPE_DOUBLE) {
        double amax;
        std::memcpy(&amax, &hs.amax_bits, sizeof(amax));
        const int fs = n ? fixed_scale_from_max(amax, n) : 0;
        double *out = (double *)loads;
        for (uint64_t p = 0; p < P; ++p) {
            const unsigned __int128 q = (unsigned __int128)h[p * 4] + ((unsigned __int128)h[p * 4 + 1] << 32) +
                                        ((unsigned __int128)h[p * 4 + 2] << 64) +
                                        ((unsigned __int128)h[p * 4 + 3] << 96);
            out[p] = fixed_to_f64(q, fs);
        }
    } else if (wtype == COUPE_INT64) {
        int64_t *out = (int64_t *)loads;
        for (uint64_t p = 0; p < P; ++p) out[p] = (int64_t)h[p];
    } else {
        int32_t *out = (int32_t *)loads;
        for (uint64_t p = 0; p < P; ++p) out[p] = (int32_t)(uint32_t)h[p];
    }
    return COUPE_ERR_OK;
}

// imbalance (coupe/src/imbalance.rs:41-77) from the loads: the total in the
// weights' own arithmetic, the ideal load total / num_parts, and the largest
// (load - ideal) / ideal; 0 when there are no parts or the ideal load is 0.
double imbalance_of_loads(int wtype, const void *loads, uint64_t P) {
    if (P == 0) return 0.0;
    std::vector<double> lf(P);
    double total;
    if (wtype == COUPE_DOUBLE) {
        const double *l = (const double *)loads;
        double t = 0.0;
        for (uint64_t p = 0; p < P; ++p) t += l[p];
        total = t;
        for (uint64_t p = 0; p < P; ++p) lf[p] = l[p];
    } else if (wtype == COUPE_INT64) {
        const int64_t *l = (const int64_t *)loads;
        uint64_t t = 0;
        for (uint64_t p = 0; p < P; ++p) t += (uint64_t)l[p];
        total = (double)(int64_t)t;
        for (uint64_t p = 0; p < P; ++p) lf[p] = (double)l[p];
    } else {
        const int32_t *l = (const int32_t *)loads;
        uint32_t t = 0;
        for (uint64_t p = 0; p < P; ++p) t += (uint32_t)l[p];
        total = (double)(int32_t)t;
        for (uint64_t p = 0; p < P; ++p) lf[p] = (double)l[p];
    }
    const double ideal = total / (double)P;
    if (ideal == 0.0) return 0.0;
    double mx = (lf[0] - ideal) / ideal;
    for (uint64_t p = 1; p < P; ++p) {
        const double v = (lf[p] - ideal) / ideal;
        if (!(v < mx)) mx = v;
    }
    return mx;
}

}  // namespace cg
