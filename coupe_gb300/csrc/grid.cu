// Rcb on a cartesian grid (coupe::Grid::rcb, coupe/src/cartesian/mod.rs:130-179,
// cartesian/rcb.rs:52-281).  The split tree is built level by level:
//   k_grid_slab_add   integer weights (order-free wrapping sums): one
//                     coalesced pass over every cell, which finds its
//                     subgrid by walking the tree built so far and adds its
//                     weight to its slab (warp-aggregated atomics);
//   k_grid_axis_sums  f64 weights: for every subgrid of the level, the weight
//                     of each slab across the split axis, one thread per
//                     slab, summed in coupe's order (so f64 sums round alike);
//   host              the weighted median of those slab weights, replaying
//                     rayon's fold_chunks with `threads` workers
//                     (cartesian/rcb.rs:53-101), and the two halves;
//   k_grid_assign     once the tree is known, each cell walks it from the
//                     root (first split on axis 1, then cycling) and gets
//                     2 id + side per split (IterationResult::part_of).
// Integer totals wrap like coupe's release build.  The root's f64 total is
// the 128-bit fixed-point sum rounded once (coupe's rayon sum has no fixed
// order); every other weight follows coupe's arithmetic.
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

constexpr double GRID_TOLERANCE = 0.01;  // cartesian/rcb.rs:45

struct GridSub {
    uint64_t off[3], size[3];
    uint64_t base;  // first output slot of this subgrid's slabs
    int coord;
    int pad;
};

// Weight sums in W's own arithmetic: i32 and i64 wrap, f64 rounds.
template <class W>
struct GAcc;
template <>
struct GAcc<int32_t> {
    typedef uint32_t A;
    __device__ static A add(A a, int32_t w) { return a + (uint32_t)w; }
};
template <>
struct GAcc<int64_t> {
    typedef uint64_t A;
    __device__ static A add(A a, int64_t w) { return a + (uint64_t)w; }
};
template <>
struct GAcc<double> {
    typedef double A;
    __device__ static A add(A a, double w) { return __dadd_rn(a, w); }
};

template <class W, int D>
__global__ void __launch_bounds__(BLOCK) k_grid_axis_sums(const W *__restrict__ w, uint64_t gw, uint64_t gh,
                                                          const GridSub *__restrict__ subs, uint32_t nsubs,
                                                          uint64_t total, typename GAcc<W>::A *__restrict__ out) {
    typedef typename GAcc<W>::A A;
    for (uint64_t t = (uint64_t)blockIdx.x * BLOCK + threadIdx.x; t < total; t += (uint64_t)gridDim.x * BLOCK) {
        uint32_t lo = 0, hi = nsubs;  // the last subgrid with base <= t
        while (hi - lo > 1) {
            const uint32_t m = (lo + hi) >> 1;
            if (subs[m].base <= t)
                lo = m;
            else
                hi = m;
        }
        const GridSub g = subs[lo];
        const uint64_t p = g.off[g.coord] + (t - g.base);
        A acc = A(0);
        // one row of the slab, cnt cells `stride` apart, added in order; the
        // loads of eight cells are issued before their adds
        auto row = [&](uint64_t base, uint64_t stride, uint64_t cnt) {
            uint64_t j = 0;
            for (; j + 8 <= cnt; j += 8) {
                W v[8];
#pragma unroll
                for (int u = 0; u < 8; ++u) v[u] = w[base + (j + u) * stride];
#pragma unroll
                for (int u = 0; u < 8; ++u) acc = GAcc<W>::add(acc, v[u]);
            }
            for (; j < cnt; ++j) acc = GAcc<W>::add(acc, w[base + j * stride]);
        };
        if (D == 2) {
            if (g.coord == 0)
                row(p + gw * g.off[1], gw, g.size[1]);  // y
            else
                row(g.off[0] + gw * p, 1, g.size[0]);  // x
        } else if (g.coord == 0) {  // y outer, z inner
            for (uint64_t y = g.off[1]; y < g.off[1] + g.size[1]; ++y) row(p + gw * (y + gh * g.off[2]), gw * gh, g.size[2]);
        } else if (g.coord == 1) {  // z outer, x inner
            for (uint64_t z = g.off[2]; z < g.off[2] + g.size[2]; ++z) row(g.off[0] + gw * (p + gh * z), 1, g.size[0]);
        } else {  // x outer, y inner
            for (uint64_t x = g.off[0]; x < g.off[0] + g.size[0]; ++x) row(x + gw * (g.off[1] + gh * p), gw, g.size[1]);
        }
        out[t] = acc;
    }
}

// Integer weights: the weight of every slab of the level's subgrids in one
// pass over the cells in memory order.  A cell walks the split tree from the
// root (first split on axis 1, then cycling) to its leaf; sub[leaf] is its
// subgrid at this level (-1: a finished one) and the slot is the subgrid's
// base plus the cell's position along the split axis.  The sums wrap like
// coupe's release build and do not depend on the order of the adds.  Along
// axis 1 or 2 a warp's 32 consecutive cells usually share one slot: then one
// lane adds their sum.
__device__ __forceinline__ void atomic_add_wrap(uint32_t *p, uint32_t v) { atomicAdd(p, v); }
__device__ __forceinline__ void atomic_add_wrap(uint64_t *p, uint64_t v) {
    atomicAdd((unsigned long long *)p, (unsigned long long)v);
}

template <class W, int D>
__global__ void __launch_bounds__(BLOCK) k_grid_slab_add(const W *__restrict__ w, uint64_t gw, uint64_t gh, uint64_t n,
                                                         const int64_t *__restrict__ pos,
                                                         const uint32_t *__restrict__ child,
                                                         const int32_t *__restrict__ sub,
                                                         const GridSub *__restrict__ subs,
                                                         typename GAcc<W>::A *__restrict__ out) {
    typedef typename GAcc<W>::A A;
    const uint64_t stride = (uint64_t)gridDim.x * BLOCK;
    // every lane of a warp runs the same number of iterations (the warp sums below)
    const uint64_t iters = (n + stride - 1) / stride;
    uint64_t i = (uint64_t)blockIdx.x * BLOCK + threadIdx.x;
    for (uint64_t it = 0; it < iters; ++it, i += stride) {
        uint64_t slot = ~0ull;
        A v = A(0);
        if (i < n) {
            uint64_t c[3];
            c[0] = i % gw;
            c[1] = D == 2 ? i / gw : (i / gw) % gh;
            c[2] = D == 3 ? i / gw / gh : 0;
            uint32_t node = 0;
            int coord = 1;
            int64_t at = pos[0];
            while (at >= 0) {
                node = child[node] + (c[coord] >= (uint64_t)at ? 1u : 0u);
                at = pos[node];
                coord = coord + 1 == D ? 0 : coord + 1;
            }
            const int32_t k = sub[node];
            if (k >= 0) {
                const GridSub &g = subs[k];
                slot = g.base + (c[g.coord] - g.off[g.coord]);
                v = (A)w[i];
            }
        }
        const uint64_t s0 = __shfl_sync(0xffffffffu, slot, 0);
        if (__all_sync(0xffffffffu, slot == s0)) {
            // one slot for the warp: its sum, added once
            A t = v;
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
            if ((threadIdx.x & 31) == 0 && s0 != ~0ull) atomic_add_wrap(&out[s0], t);
        } else if (slot != ~0ull) {
            atomic_add_wrap(&out[slot], v);
        }
    }
}

// Total weight: integers wrap (a u64 sum truncated to W), f64 weights as
// fixed-point limbs after their largest magnitude.
template <class W>
__global__ void __launch_bounds__(BLOCK) k_grid_total(const W *__restrict__ w, uint64_t n, int fs,
                                                      unsigned long long *acc) {
    uint64_t s[4] = {0, 0, 0, 0};
    for (uint64_t i = (uint64_t)blockIdx.x * BLOCK + threadIdx.x; i < n; i += (uint64_t)gridDim.x * BLOCK) {
        if constexpr (sizeof(W) == 8 && W(0.5) != W(0)) {
            const unsigned __int128 q = fixed_q_bits((double)w[i], fs);
            s[0] += (uint32_t)q;
            s[1] += (uint32_t)(q >> 32);
            s[2] += (uint32_t)(q >> 64);
            s[3] += (uint32_t)(q >> 96);
        } else {
            s[0] += (uint64_t)(int64_t)w[i];
        }
    }
#pragma unroll
    for (int l = 0; l < 4; ++l) {
        const uint64_t v = warp_sum_u64(s[l]);
        if ((threadIdx.x & 31) == 0 && v) atomicAdd(&acc[l], (unsigned long long)v);
    }
}

__global__ void __launch_bounds__(BLOCK) k_grid_wmax(const double *__restrict__ w, uint64_t n,
                                                     unsigned long long *out) {
    uint64_t m = 0;
    for (uint64_t i = (uint64_t)blockIdx.x * BLOCK + threadIdx.x; i < n; i += (uint64_t)gridDim.x * BLOCK) {
        const uint64_t b = (uint64_t)__double_as_longlong(w[i]) & 0x7fffffffffffffffull;
        m = b > m ? b : m;
    }
    m = warp_max_u64(m);
    if ((threadIdx.x & 31) == 0) atomicMax(out, (unsigned long long)m);
}

// pos[node] < 0: a whole subgrid; else the split position, children at
// child[node] (left) and child[node] + 1 (right).
template <int D>
__global__ void __launch_bounds__(BLOCK) k_grid_assign(const int64_t *__restrict__ pos,
                                                       const uint32_t *__restrict__ child, uint64_t gw, uint64_t gh,
                                                       uint64_t n, uint64_t *__restrict__ part) {
    for (uint64_t i = (uint64_t)blockIdx.x * BLOCK + threadIdx.x; i < n; i += (uint64_t)gridDim.x * BLOCK) {
        uint64_t c[3];
        c[0] = i % gw;
        c[1] = D == 2 ? i / gw : (i / gw) % gh;
        c[2] = D == 3 ? i / gw / gh : 0;
        uint64_t id = 0;
        uint32_t node = 0;
        int coord = 1;
        int64_t at = pos[0];
        while (at >= 0) {
            const bool right = c[coord] >= (uint64_t)at;
            id = 2 * id + (right ? 1 : 0);
            node = child[node] + (right ? 1u : 0u);
            at = pos[node];
            coord = coord + 1 == D ? 0 : coord + 1;
        }
        part[i] = id;
    }
}

// The host's W for one type: values, wrapping arithmetic, f64 -> W `as`.
template <class W>
struct HW;
template <>
struct HW<int32_t> {
    typedef int32_t V;
    static V add(V a, V b) { return (V)(uint32_t)((uint32_t)a + (uint32_t)b); }
    static V sub(V a, V b) { return (V)(uint32_t)((uint32_t)a - (uint32_t)b); }
    static V from_acc(uint64_t a) { return (V)(uint32_t)a; }
    static V from_f64(double x) {
        if (x != x) return 0;
        if (x >= 2147483647.0) return 2147483647;
        if (x <= -2147483648.0) return (V)0x80000000u;
        return (V)x;
    }
};
template <>
struct HW<int64_t> {
    typedef int64_t V;
    static V add(V a, V b) { return (V)((uint64_t)a + (uint64_t)b); }
    static V sub(V a, V b) { return (V)((uint64_t)a - (uint64_t)b); }
    static V from_acc(uint64_t a) { return (V)a; }
    static V from_f64(double x) {
        if (x != x) return 0;
        if (x >= 9223372036854775807.0) return INT64_MAX;
        if (x <= -9223372036854775808.0) return INT64_MIN;
        return (V)x;
    }
};
template <>
struct HW<double> {
    typedef double V;
    static V add(V a, V b) { return a + b; }
    static V sub(V a, V b) { return a - b; }
    static V from_f64(double x) { return x; }
};

// weighted_median (cartesian/rcb.rs:53-101) over n slab weights.
template <class W>
void weighted_median(const W *w, uint64_t n, W total, uint64_t threads, uint64_t *position, W *left_out) {
    const double ideal = (double)total / 2.0;
    const W min_part = HW<W>::from_f64(ideal * (1.0 - GRID_TOLERANCE));
    const W max_part = HW<W>::from_f64(ideal * (1.0 + GRID_TOLERANCE));
    uint64_t lo = 0, hi = n;
    W left = W(0);
    for (;;) {
        const uint64_t cs = std::max<uint64_t>(1, (hi - lo) / threads);
        const uint64_t lo0 = lo, hi0 = hi;
        const W left0 = left;
        W prefix = W(0);
        for (uint64_t start = lo0; start < hi0; start += cs) {
            const W pcw = HW<W>::add(left0, prefix);
            W csum = W(0);
            for (uint64_t j = start; j < std::min(start + cs, hi0); ++j) csum = HW<W>::add(csum, w[j]);
            prefix = HW<W>::add(prefix, csum);
            if (pcw < min_part) {
                lo = start;
                left = pcw;
            } else if (max_part < pcw) {
                hi = start;
                break;
            } else {
                *position = start;
                *left_out = pcw;
                return;
            }
        }
        if (lo + 1 >= hi) {
            *position = lo;
            *left_out = left;
            return;
        }
    }
}

struct GNode {
    uint64_t off[3], size[3];
    uint32_t index;  // in the tree arrays
    int coord;
    uint64_t iters;  // levels left
    double wf;       // total weight (f64), or
    int64_t wi;      // total weight (integers)
};

template <class W, int D>
int grid_run(DevCtx &C, const uint64_t *size, const W *d_w, uint64_t iters, uint64_t threads, uint64_t *d_part,
             cudaStream_t s, std::string *err) {
    typedef typename GAcc<W>::A A;
    constexpr bool F = sizeof(W) == 8 && W(0.5) != W(0);
    const uint64_t gw = size[0], gh = size[1];
    uint64_t n = 1;
    for (int d = 0; d < D; ++d) n *= size[d];
    cudaError_t e;
    int rc;
    const unsigned gs = (unsigned)std::max<uint64_t>(1, std::min<uint64_t>((n + BLOCK - 1) / BLOCK,
                                                                            (uint64_t)C.sms * 8));
    // the total weight
    if ((rc = ensure_workspace(C, 64, err)) != COUPE_ERR_OK) return rc;
    unsigned long long *tacc = (unsigned long long *)C.ws;
    if ((e = cudaMemsetAsync(tacc, 0, 64, s)) != cudaSuccess) return cuda_fail(e, "grid set-up", err);
    int fs = 0;
    unsigned long long h[5] = {0, 0, 0, 0, 0};
    if (F) {
        k_grid_wmax<<<gs, BLOCK, 0, s>>>((const double *)d_w, n, tacc + 4);
        if ((e = cudaGetLastError()) != cudaSuccess) return cuda_fail(e, "k_grid_wmax", err);
        if ((e = cudaMemcpyAsync(&h[4], tacc + 4, 8, cudaMemcpyDeviceToHost, s)) != cudaSuccess ||
            (e = cudaStreamSynchronize(s)) != cudaSuccess)
            return cuda_fail(e, "grid weights", err);
        if (h[4] >= 0x7ff0000000000000ull) {
            if (err) *err = "non-finite weight";
            return COUPE_ERR_BAD_TYPE;
        }
        double amax;
        std::memcpy(&amax, &h[4], 8);
        fs = fixed_scale_from_max(amax, n);
    }
    C.prof.begin(KID_GRID, n * sizeof(W), s);
    k_grid_total<W><<<gs, BLOCK, 0, s>>>(d_w, n, fs, tacc);
    if ((e = cudaGetLastError()) != cudaSuccess) return cuda_fail(e, "k_grid_total", err);
    C.prof.end(s);
    if ((e = cudaMemcpyAsync(h, tacc, 32, cudaMemcpyDeviceToHost, s)) != cudaSuccess ||
        (e = cudaStreamSynchronize(s)) != cudaSuccess)
        return cuda_fail(e, "grid total", err);
    GNode root{};
    for (int d = 0; d < 3; ++d) root.size[d] = d < D ? size[d] : 1;
    root.index = 0;
    root.coord = 1;
    root.iters = iters;
    if constexpr (F) {
        const unsigned __int128 q = (unsigned __int128)h[0] + ((unsigned __int128)h[1] << 32) +
                                    ((unsigned __int128)h[2] << 64) + ((unsigned __int128)h[3] << 96);
        root.wf = fixed_to_f64(q, fs);
    } else {
        root.wi = (int64_t)HW<W>::from_acc(h[0]);
    }
    std::vector<int64_t> tpos(1, -1);
    std::vector<uint32_t> tchild(1, 0);
    std::vector<GNode> level(1, root), next;
    std::vector<GridSub> subs;
    std::vector<A> sums;
    while (!level.empty()) {
        subs.clear();
        next.clear();
        uint64_t slots = 0;
        for (const GNode &g : level) {
            if (g.size[g.coord] == 0 || g.iters == 0) continue;  // a whole subgrid (cartesian/rcb.rs:114-116)
            GridSub sb{};
            for (int d = 0; d < 3; ++d) {
                sb.off[d] = g.off[d];
                sb.size[d] = g.size[d];
            }
            sb.coord = g.coord;
            sb.base = slots;
            slots += g.size[g.coord];
            subs.push_back(sb);
        }
        if (subs.empty()) break;
        if (tpos.size() + 2 * subs.size() > 0xffffffffull) {
            if (err) *err = "too many splits";
            return COUPE_ERR_ALLOC;
        }
        // workspace: the level's subgrids, its slab sums and (integer
        // weights) the tree so far with each leaf's subgrid
        const size_t tab = subs.size() * sizeof(GridSub), tab_al = (tab + 255) & ~(size_t)255;
        const size_t nb = tpos.size(), o_pos = tab_al + ((slots * sizeof(A) + 255) & ~(size_t)255),
                     o_child = o_pos + ((nb * 8 + 255) & ~(size_t)255),
                     o_sub = o_child + ((nb * 4 + 255) & ~(size_t)255), need = (F ? o_pos : o_sub + nb * 4) + 256;
        if ((rc = ensure_workspace(C, need, err)) != COUPE_ERR_OK) return rc;
        GridSub *d_subs = (GridSub *)C.ws;
        A *d_sums = (A *)((char *)C.ws + tab_al);
        sums.resize(slots);
        const unsigned ga = (unsigned)std::max<uint64_t>(1, std::min<uint64_t>((slots + BLOCK - 1) / BLOCK,
                                                                                (uint64_t)C.sms * 8));
        if ((e = cudaMemcpyAsync(d_subs, subs.data(), tab, cudaMemcpyHostToDevice, s)) != cudaSuccess)
            return cuda_fail(e, "grid table", err);
        if constexpr (F) {
            C.prof.begin(KID_GRID, n * sizeof(W), s);
            k_grid_axis_sums<W, D><<<ga, BLOCK, 0, s>>>(d_w, gw, gh, d_subs, (uint32_t)subs.size(), slots, d_sums);
            if ((e = cudaGetLastError()) != cudaSuccess) return cuda_fail(e, "k_grid_axis_sums", err);
            C.prof.end(s);
        } else {
            // the tree so far and each leaf's subgrid of this level
            std::vector<int32_t> tsub(tpos.size(), -1);
            {
                size_t kk = 0;
                for (const GNode &g : level)
                    if (!(g.size[g.coord] == 0 || g.iters == 0)) tsub[g.index] = (int32_t)kk++;
            }
            int64_t *d_tpos = (int64_t *)((char *)C.ws + o_pos);
            uint32_t *d_tchild = (uint32_t *)((char *)C.ws + o_child);
            int32_t *d_tsub = (int32_t *)((char *)C.ws + o_sub);
            if ((e = cudaMemcpyAsync(d_tpos, tpos.data(), nb * 8, cudaMemcpyHostToDevice, s)) != cudaSuccess ||
                (e = cudaMemcpyAsync(d_tchild, tchild.data(), nb * 4, cudaMemcpyHostToDevice, s)) != cudaSuccess ||
                (e = cudaMemcpyAsync(d_tsub, tsub.data(), nb * 4, cudaMemcpyHostToDevice, s)) != cudaSuccess ||
                (e = cudaMemsetAsync(d_sums, 0, slots * sizeof(A), s)) != cudaSuccess)
                return cuda_fail(e, "grid level", err);
            C.prof.begin(KID_GRID, n * sizeof(W), s);
            k_grid_slab_add<W, D><<<gs, BLOCK, 0, s>>>(d_w, gw, gh, n, d_tpos, d_tchild, d_tsub, d_subs, d_sums);
            if ((e = cudaGetLastError()) != cudaSuccess) return cuda_fail(e, "k_grid_slab_add", err);
            C.prof.end(s);
            // the host vectors above are read by the copies before they return
            if ((e = cudaStreamSynchronize(s)) != cudaSuccess) return cuda_fail(e, "grid level", err);
        }
        if ((e = cudaMemcpyAsync(sums.data(), d_sums, slots * sizeof(A), cudaMemcpyDeviceToHost, s)) !=
                cudaSuccess ||
            (e = cudaStreamSynchronize(s)) != cudaSuccess)
            return cuda_fail(e, "grid slab weights", err);
        size_t k = 0;
        for (const GNode &g : level) {
            if (g.size[g.coord] == 0 || g.iters == 0) continue;
            const GridSub &sb = subs[k++];
            const uint64_t len = g.size[g.coord];
            std::vector<W> aw(len);
            for (uint64_t j = 0; j < len; ++j) {
                if constexpr (F)
                    aw[j] = sums[sb.base + j];
                else
                    aw[j] = HW<W>::from_acc((uint64_t)sums[sb.base + j]);
            }
            W total;
            if constexpr (F)
                total = g.wf;
            else
                total = (W)g.wi;
            uint64_t position = 0;
            W left = W(0);
            weighted_median<W>(aw.data(), len, total, threads, &position, &left);
            const uint64_t at = position + g.off[g.coord];
            const W right = HW<W>::sub(total, left);
            tpos[g.index] = (int64_t)at;
            tchild[g.index] = (uint32_t)tpos.size();
            GNode lo = g, hi = g;
            lo.size[g.coord] = at - g.off[g.coord];
            hi.size[g.coord] -= at - g.off[g.coord];
            hi.off[g.coord] = at;
            lo.coord = hi.coord = (g.coord + 1) % D;
            lo.iters = hi.iters = g.iters - 1;
            lo.index = (uint32_t)tpos.size();
            hi.index = lo.index + 1;
            if constexpr (F) {
                lo.wf = (double)left;
                hi.wf = (double)right;
            } else {
                lo.wi = (int64_t)left;
                hi.wi = (int64_t)right;
            }
            tpos.push_back(-1);
            tpos.push_back(-1);
            tchild.push_back(0);
            tchild.push_back(0);
            next.push_back(lo);
            next.push_back(hi);
        }
        level.swap(next);
    }
    // the ids
    const size_t pb = tpos.size() * sizeof(int64_t), pb_al = (pb + 255) & ~(size_t)255;
    if ((rc = ensure_workspace(C, pb_al + tchild.size() * sizeof(uint32_t) + 256, err)) != COUPE_ERR_OK) return rc;
    int64_t *d_pos = (int64_t *)C.ws;
    uint32_t *d_child = (uint32_t *)((char *)C.ws + pb_al);
    if ((e = cudaMemcpyAsync(d_pos, tpos.data(), pb, cudaMemcpyHostToDevice, s)) != cudaSuccess ||
        (e = cudaMemcpyAsync(d_child, tchild.data(), tchild.size() * sizeof(uint32_t), cudaMemcpyHostToDevice, s)) !=
            cudaSuccess)
        return cuda_fail(e, "grid tree", err);
    C.prof.begin(KID_GRID, n * 8, s);
    k_grid_assign<D><<<gs, BLOCK, 0, s>>>(d_pos, d_child, gw, gh, n, d_part);
    if ((e = cudaGetLastError()) != cudaSuccess) return cuda_fail(e, "k_grid_assign", err);
    C.prof.end(s);
    if ((e = cudaStreamSynchronize(s)) != cudaSuccess) return cuda_fail(e, "grid ids", err);
    C.prof.resolve();
    return COUPE_ERR_OK;
}

}  // namespace

int grid_rcb(DevCtx &C, int dim, const uint64_t *size, int wtype, const void *d_w, uint64_t iters, uint64_t threads,
             uint64_t *d_part, cudaStream_t stream, std::string *err) {
    cudaStream_t s = stream ? stream : C.stream;
    if (wtype == COUPE_DOUBLE)
        return dim == 2 ? grid_run<double, 2>(C, size, (const double *)d_w, iters, threads, d_part, s, err)
                        : grid_run<double, 3>(C, size, (const double *)d_w, iters, threads, d_part, s, err);
    if (wtype == COUPE_INT64)
        return dim == 2 ? grid_run<int64_t, 2>(C, size, (const int64_t *)d_w, iters, threads, d_part, s, err)
                        : grid_run<int64_t, 3>(C, size, (const int64_t *)d_w, iters, threads, d_part, s, err);
    return dim == 2 ? grid_run<int32_t, 2>(C, size, (const int32_t *)d_w, iters, threads, d_part, s, err)
                    : grid_run<int32_t, 3>(C, size, (const int32_t *)d_w, iters, threads, d_part, s, err);
}

}  // namespace cg
