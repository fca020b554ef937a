// coupe's axis_sort and MultiJagged on the GPU
// (coupe/src/algorithms/recursive_bisection.rs:815-827,
// coupe/src/algorithms/multi_jagged.rs:75-295).
//
// MultiJagged splits every part of an iteration into num_splits + 1 parts
// of given weight shares (its partition scheme) along one axis, cycling the
// axis per iteration.  A level of the scheme is processed at once:
//   k_mj_keys        each position's segment and the ordered f64 code of its
//                    point's coordinate on the level's axis;
//   radix sorts      by coordinate, then (stably) by segment: every segment
//                    sorted along the axis, in place (axis_sort);
//   k_mj_limbs       each position's weight as 128-bit fixed point in four
//                    32-bit limbs, and inclusive scans of the limbs: exact
//                    prefix sums of the weights in sorted order;
//   k_mj_positions   one thread per segment: the thresholds (running sums of
//                    total * modifier, in f64 as coupe computes them) and,
//                    per threshold, the first position whose running weight
//                    exceeds it and is not within 4 ulps of it
//                    (compute_split_positions, multi_jagged.rs:222-295),
//                    by binary search over the exact prefix sums;
//   k_mj_leaf_ids    the part id of every position of a finished part.
// The host walks the scheme: it knows each segment's modifiers and splits the
// segments at the returned positions (split_at_mut_many, :297-318).
//
// The sorts use CUB's radix sort (the CUDA toolkit's C++ template library,
// compiled into this file); this row is off the Rcb path.
#include <cuda_runtime.h>
#include <stdint.h>

#include <cub/cub.cuh>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <memory>
#include <string>
#include <vector>

#include "engine.h"
#include "kernels.cuh"

namespace cg {

namespace {

// partition_scheme (multi_jagged.rs:75-103)
struct MjScheme {
    uint64_t num_splits = 0;
    std::vector<double> modifiers;
    std::vector<MjScheme> next;
    uint64_t leaf_id = 0;  // part id of a leaf (num_splits == 0), in the order coupe's recursion assigns them
};

// compute_modifiers (multi_jagged.rs:138-149)
std::vector<double> mj_modifiers(uint64_t num_regular_parts, uint64_t num_fat_parts, uint64_t num_regular_subparts,
                                 uint64_t num_fat_subparts) {
    const uint64_t num_subparts = num_regular_parts * num_regular_subparts + num_fat_parts * num_fat_subparts;
    std::vector<double> m;
    for (uint64_t i = 0; i < num_fat_parts; ++i) m.push_back((double)num_fat_subparts / (double)num_subparts);
    for (uint64_t i = 0; i < num_regular_parts; ++i) m.push_back((double)num_regular_subparts / (double)num_subparts);
    return m;
}

bool mj_scheme(uint64_t num_parts, uint64_t max_iter, MjScheme &out, int depth, std::string *err) {
    // (num_parts as f32).powf(1. / max_iter as f32).ceil() as usize
    const float root_f = std::ceil(std::pow((float)num_parts, 1.0f / (float)max_iter));
    // a node that splits has at least two children, so no scheme of fewer
    // than 2^64 parts is deeper than 64 splitting levels
    if (!(root_f >= 1.0f) || !(root_f < 4294967296.0f) || depth > 64) {
        *err = "no partition scheme for " + std::to_string(num_parts) + " parts in " + std::to_string(max_iter) +
               " iterations";
        return false;
    }
    const uint64_t approx_root = (uint64_t)root_f;
    const uint64_t rem = num_parts % approx_root, quotient = num_parts / approx_root;
    out.num_splits = approx_root - 1;
    out.modifiers = mj_modifiers(approx_root - rem, rem, quotient, quotient + 1);
    // a node that does not split is a part; coupe still builds the children
    // of such a node, but never visits them (multi_jagged.rs:191, :207)
    if (out.num_splits == 0) return true;
    if (max_iter == 0) {
        *err = "no partition scheme for " + std::to_string(num_parts) + " parts in 0 iterations";
        return false;
    }
    out.next.resize(approx_root);
    for (uint64_t i = 0; i < approx_root; ++i)
        if (!mj_scheme(i < rem ? quotient + 1 : quotient, max_iter - 1, out.next[i], depth + 1, err)) return false;
    return true;
}

// Leaves numbered as multi_jagged_recurse meets them with one worker:
// depth first, children in order (its part_id counter, :193-213).
void mj_number_leaves(MjScheme &s, uint64_t &next_id) {
    if (s.num_splits == 0) {
        s.leaf_id = next_id++;
        return;
    }
    for (MjScheme &c : s.next) mj_number_leaves(c, next_id);
}

struct MjSeg {
    uint64_t off, len;
    const MjScheme *sch;
    bool done;  // a finished part: its ids are written, its range stays in place
};

__global__ void k_mj_iota(uint64_t *v, uint64_t n) {
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x)
        v[i] = i;
}

// Position i holds item v[i] & 0xffffffff.  Writes the ordered code of the
// item's coordinate on `coord` and tags the item with its position's
// segment (segments tile [0, n) in order): v[i] = segment << 32 | item.
__global__ void k_mj_keys(const double *__restrict__ pts, int D, int coord, uint64_t *__restrict__ v, uint64_t n,
                          const uint64_t *__restrict__ seg_off, uint32_t S, uint64_t *__restrict__ key) {
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
        uint32_t lo = 0, hi = S;  // the last segment starting at or before i
        while (hi - lo > 1) {
            const uint32_t m = (lo + hi) >> 1;
            if (seg_off[m] <= i)
                lo = m;
            else
                hi = m;
        }
        const uint64_t item = v[i] & 0xffffffffull;
        v[i] = ((uint64_t)lo << 32) | item;
        key[i] = KeyF64::from_f64(pts[item * D + coord]);
    }
}

// 128-bit fixed-point weight of each position's item, in four 32-bit limbs
__global__ void k_mj_limbs(const double *__restrict__ w, const uint64_t *__restrict__ v, uint64_t n, int fs,
                           uint64_t *__restrict__ l0, uint64_t *__restrict__ l1, uint64_t *__restrict__ l2,
                           uint64_t *__restrict__ l3) {
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
        const unsigned __int128 q = fixed_q_bits(w[v[i] & 0xffffffffull], fs);
        l0[i] = (uint32_t)q;
        l1[i] = (uint32_t)(q >> 32);
        l2[i] = (uint32_t)(q >> 64);
        l3[i] = (uint32_t)(q >> 96);
    }
}

struct MjLimbs {
    const uint64_t *l[4];
};

__device__ __forceinline__ unsigned __int128 mj_prefix(const MjLimbs &P, uint64_t i) {
    return (unsigned __int128)P.l[0][i] + ((unsigned __int128)P.l[1][i] << 32) +
           ((unsigned __int128)P.l[2][i] << 64) + ((unsigned __int128)P.l[3][i] << 96);
}

// approx 0.5's default ulps comparison of f64 (|a-b| <= EPSILON, else same
// sign and at most 4 representable values apart), as coupe's
// compute_split_positions uses it (multi_jagged.rs:283-286)
__device__ __forceinline__ bool mj_ulps_eq(double a, double b) {
    if (fabs(a - b) <= 2.220446049250313e-16) return true;
    if (signbit(a) != signbit(b)) return false;
    const long long x = __double_as_longlong(a), y = __double_as_longlong(b);
    return (x > y ? x - y : y - x) <= 4;
}

// one thread per segment that splits: its thresholds and split positions
__global__ void k_mj_positions(MjLimbs P, const uint64_t *__restrict__ seg_off, const uint64_t *__restrict__ seg_len,
                               const uint32_t *__restrict__ mod_off, const uint32_t *__restrict__ nsplit,
                               const double *__restrict__ mods, uint32_t S, int fs, uint64_t *__restrict__ pos_out) {
    const uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= S || nsplit[s] == 0) return;
    const uint64_t off = seg_off[s], len = seg_len[s];
    const unsigned __int128 base = off ? mj_prefix(P, off - 1) : 0;
    auto cum = [&](uint64_t j) {  // weight of positions off .. off + j, exact, rounded once
        return fixed_to_f64(mj_prefix(P, off + j) - base, fs);
    };
    const double total = len ? cum(len - 1) : 0.0;
    double consumed = 0.0;
    for (uint32_t k = 0; k < nsplit[s]; ++k) {
        consumed += total * mods[mod_off[s] + k];
        const double T = consumed;
        // first j with cum(j) > T and not within 4 ulps of T; the running
        // weights do not decrease, so the others form a prefix
        uint64_t lo = 0, hi = len;
        while (lo < hi) {
            const uint64_t m = (lo + hi) >> 1;
            const double c = cum(m);
            if (c < T || mj_ulps_eq(T, c))
                lo = m + 1;
            else
                hi = m;
        }
        pos_out[mod_off[s] + k] = lo;
    }
}

// part ids of the positions of finished parts (one CTA per part)
__global__ void k_mj_leaf_ids(const uint64_t *__restrict__ v, const uint64_t *__restrict__ leaf_off,
                              const uint64_t *__restrict__ leaf_len, const uint64_t *__restrict__ leaf_id,
                              uint64_t *__restrict__ part) {
    const uint64_t off = leaf_off[blockIdx.x], len = leaf_len[blockIdx.x], id = leaf_id[blockIdx.x];
    for (uint64_t j = threadIdx.x; j < len; j += blockDim.x) part[v[off + j] & 0xffffffffull] = id;
}

// the items of positions in order (axis_sort's permutation)
__global__ void k_mj_items(const uint64_t *__restrict__ v, uint64_t n, uint64_t *__restrict__ out) {
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x)
        out[i] = v[i] & 0xffffffffull;
}

__global__ void k_mj_check_w(const double *__restrict__ w, uint64_t n, unsigned long long *amax_bits, int *neg) {
    unsigned long long m = 0;
    int ng = 0;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
        const unsigned long long b = (unsigned long long)__double_as_longlong(w[i]) & 0x7fffffffffffffffull;
        m = b > m ? b : m;
        ng |= w[i] < 0.0 ? 1 : 0;
    }
    atomicMax(amax_bits, m);
    if (ng) atomicOr(neg, 1);
}

#define MJ_CK(call)                                               \
    do {                                                          \
        cudaError_t e_ = (call);                                  \
        if (e_ != cudaSuccess) return cuda_fail(e_, #call, err);  \
    } while (0)

size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

}  // namespace

// Sorts the positions of every segment along `coord` (two stable radix
// sorts: by coordinate, then by segment).  v: segment-tagged items.
static int mj_sort(DevCtx &C, const double *d_points, int dim, int coord, uint64_t *v, uint64_t *v_alt, uint64_t *key,
                   uint64_t *key_alt, uint64_t n, const uint64_t *d_seg_off, uint32_t S, void *tmp, size_t tmp_bytes,
                   cudaStream_t s, std::string *err) {
    const unsigned grid = (unsigned)std::max<uint64_t>(1, std::min<uint64_t>((n + 255) / 256, (uint64_t)C.sms * 8));
    k_mj_keys<<<grid, 256, 0, s>>>(d_points, dim, coord, v, n, d_seg_off, S, key);
    MJ_CK(cudaGetLastError());
    size_t tb = tmp_bytes;
    MJ_CK(cub::DeviceRadixSort::SortPairs(tmp, tb, key, key_alt, v, v_alt, (int64_t)n, 0, 64, s));
    int sb = 0;
    while ((1ull << sb) < S) ++sb;
    if (sb == 0) {
        MJ_CK(cudaMemcpyAsync(v, v_alt, n * 8, cudaMemcpyDeviceToDevice, s));
    } else {
        tb = tmp_bytes;
        MJ_CK(cub::DeviceRadixSort::SortKeys(tmp, tb, v_alt, v, (int64_t)n, 32, 32 + sb, s));
    }
    return COUPE_ERR_OK;
}

struct MjWork {
    uint64_t *v, *v_alt, *key, *key_alt, *L[4], *t_off, *t_len, *t_pos, *t_lid;
    uint32_t *t_moff, *t_nsplit;
    double *t_mods;
    unsigned long long *d_amax;
    int *d_neg;
    void *tmp;
    size_t tmp_bytes;
};

static int mj_workspace(DevCtx &C, uint64_t n, uint64_t segcap, uint64_t modcap, cudaStream_t s, MjWork &W,
                        std::string *err) {
    size_t sort_tmp = 0, scan_tmp = 0;
    MJ_CK(cub::DeviceRadixSort::SortPairs(nullptr, sort_tmp, (const uint64_t *)nullptr, (uint64_t *)nullptr,
                                          (const uint64_t *)nullptr, (uint64_t *)nullptr, (int64_t)n, 0, 64, s));
    MJ_CK(cub::DeviceScan::InclusiveSum(nullptr, scan_tmp, (const uint64_t *)nullptr, (uint64_t *)nullptr, (int64_t)n,
                                        s));
    W.tmp_bytes = std::max(sort_tmp, scan_tmp);
    size_t bytes = 0;
    auto take = [&](size_t b) {
        const size_t o = bytes;
        bytes += align256(b);
        return o;
    };
    const size_t o_v = take(n * 8), o_va = take(n * 8), o_k = take(n * 8), o_ka = take(n * 8), o_l = take(4 * n * 8),
                 o_tab = take(segcap * 8 * 4 + segcap * 4 * 2), o_mods = take(modcap * 8 + modcap * 8),
                 o_tmp = take(W.tmp_bytes), o_sc = take(64);
    const int rc = ensure_workspace(C, bytes, err);
    if (rc != COUPE_ERR_OK) return rc;
    char *ws = (char *)C.ws;
    W.v = (uint64_t *)(ws + o_v);
    W.v_alt = (uint64_t *)(ws + o_va);
    W.key = (uint64_t *)(ws + o_k);
    W.key_alt = (uint64_t *)(ws + o_ka);
    for (int l = 0; l < 4; ++l) W.L[l] = (uint64_t *)(ws + o_l) + (size_t)l * n;
    W.t_off = (uint64_t *)(ws + o_tab);
    W.t_len = W.t_off + segcap;
    W.t_lid = W.t_len + segcap;
    W.t_pos = (uint64_t *)(ws + o_mods);
    W.t_mods = (double *)(W.t_pos + modcap);
    W.t_moff = (uint32_t *)(W.t_lid + segcap);
    W.t_nsplit = W.t_moff + segcap;
    W.tmp = ws + o_tmp;
    W.d_amax = (unsigned long long *)(ws + o_sc);
    W.d_neg = (int *)(W.d_amax + 1);
    return COUPE_ERR_OK;
}

int axis_sort(DevCtx &C, uint64_t n, int dim, const double *d_points, int coord, uint64_t *d_perm,
              cudaStream_t stream, std::string *err) {
    cudaStream_t s = stream ? stream : C.stream;
    if (n == 0) return COUPE_ERR_OK;
    if (n > 0xffffffffull) {
        *err = "more than 2^32 - 1 points";
        return COUPE_ERR_ALLOC;
    }
    MjWork W;
    int rc = mj_workspace(C, n, 2, 1, s, W, err);
    if (rc != COUPE_ERR_OK) return rc;
    const unsigned grid = (unsigned)std::max<uint64_t>(1, std::min<uint64_t>((n + 255) / 256, (uint64_t)C.sms * 8));
    k_mj_iota<<<grid, 256, 0, s>>>(W.v, n);
    MJ_CK(cudaMemsetAsync(W.t_off, 0, 8, s));
    rc = mj_sort(C, d_points, dim, coord, W.v, W.v_alt, W.key, W.key_alt, n, W.t_off, 1, W.tmp, W.tmp_bytes, s, err);
    if (rc != COUPE_ERR_OK) return rc;
    k_mj_items<<<grid, 256, 0, s>>>(W.v, n, d_perm);
    MJ_CK(cudaGetLastError());
    MJ_CK(cudaStreamSynchronize(s));
    return COUPE_ERR_OK;
}

int multi_jagged(DevCtx &C, uint64_t n, int dim, const double *d_points, const double *d_weights,
                 uint64_t part_count, uint64_t max_iter, uint64_t *d_part, cudaStream_t stream, std::string *err) {
    cudaStream_t s = stream ? stream : C.stream;
    if (part_count == 0) {
        *err = "part_count must be positive";
        return COUPE_ERR_BAD_TYPE;
    }
    if (part_count > (1ull << 24)) {
        *err = "part_count above 2^24";
        return COUPE_ERR_ALLOC;
    }
    if (n == 0) return COUPE_ERR_OK;
    if (n > 0xffffffffull) {
        *err = "more than 2^32 - 1 points";
        return COUPE_ERR_ALLOC;
    }
    MjScheme root;
    if (!mj_scheme(part_count, max_iter, root, 0, err)) return COUPE_ERR_NOT_FOUND;
    uint64_t nid = 0;
    mj_number_leaves(root, nid);
    // a level holds the finished parts (at most part_count) and the level's
    // splitting nodes (each has two parts or more below it: at most
    // part_count / 2), whose split positions number at most part_count
    const uint64_t segcap = 2 * part_count + 2, modcap = 2 * part_count + 2;
    MjWork W;
    int rc = mj_workspace(C, n, segcap, modcap, s, W, err);
    if (rc != COUPE_ERR_OK) return rc;
    const unsigned grid = (unsigned)std::max<uint64_t>(1, std::min<uint64_t>((n + 255) / 256, (uint64_t)C.sms * 8));

    // weights: finite and non-negative (running weights must not decrease);
    // the fixed-point scale of the largest
    MJ_CK(cudaMemsetAsync(W.d_amax, 0, 16, s));
    k_mj_check_w<<<grid, 256, 0, s>>>(d_weights, n, W.d_amax, W.d_neg);
    MJ_CK(cudaGetLastError());
    unsigned long long h_sc[2] = {0, 0};
    MJ_CK(cudaMemcpyAsync(h_sc, W.d_amax, 16, cudaMemcpyDeviceToHost, s));
    MJ_CK(cudaStreamSynchronize(s));
    double amax;
    std::memcpy(&amax, &h_sc[0], 8);
    if ((int)h_sc[1] & 1) {
        *err = "negative weights";
        return COUPE_ERR_NEG_VALUES;
    }
    if (!std::isfinite(amax)) {
        *err = "f64 weights must be finite";
        return COUPE_ERR_BAD_TYPE;
    }
    const int fs = fixed_scale_from_max(amax, n);

    k_mj_iota<<<grid, 256, 0, s>>>(W.v, n);
    MJ_CK(cudaGetLastError());
    std::vector<MjSeg> segs{{0, n, &root, false}};
    std::vector<uint64_t> h_off, h_len, h_lid, h_pos;
    std::vector<uint32_t> h_moff, h_nsplit;
    std::vector<double> h_mods;
    for (int level = 0;; ++level) {
        // finished parts: their ids (multi_jagged_recurse's leaves, :207-213)
        if (segs.size() > segcap) {
            *err = "internal: more segments than the table holds";
            return COUPE_ERR_CRASH;
        }
        h_off.clear();
        h_len.clear();
        h_lid.clear();
        for (MjSeg &g : segs)
            if (!g.done && g.sch->num_splits == 0) {
                g.done = true;
                if (!g.len) continue;
                h_off.push_back(g.off);
                h_len.push_back(g.len);
                h_lid.push_back(g.sch->leaf_id);
            }
        if (!h_off.empty()) {
            const size_t nl = h_off.size();
            MJ_CK(cudaMemcpyAsync(W.t_off, h_off.data(), nl * 8, cudaMemcpyHostToDevice, s));
            MJ_CK(cudaMemcpyAsync(W.t_len, h_len.data(), nl * 8, cudaMemcpyHostToDevice, s));
            MJ_CK(cudaMemcpyAsync(W.t_lid, h_lid.data(), nl * 8, cudaMemcpyHostToDevice, s));
            k_mj_leaf_ids<<<(unsigned)nl, 256, 0, s>>>(W.v, W.t_off, W.t_len, W.t_lid, d_part);
            MJ_CK(cudaGetLastError());
            MJ_CK(cudaStreamSynchronize(s));  // the host arrays are reused below
        }
        bool any = false;
        for (const MjSeg &g : segs) any = any || !g.done;
        if (!any) break;
        const uint32_t S = (uint32_t)segs.size();
        // every segment sorted along the level's axis (axis_sort, :192)
        h_off.clear();
        h_len.clear();
        h_moff.clear();
        h_nsplit.clear();
        h_mods.clear();
        for (const MjSeg &g : segs) {
            h_off.push_back(g.off);
            h_len.push_back(g.len);
            h_moff.push_back((uint32_t)h_mods.size());
            const uint32_t k = g.done ? 0u : (uint32_t)g.sch->num_splits;
            h_nsplit.push_back(k);
            for (uint32_t j = 0; j < k; ++j) h_mods.push_back(g.sch->modifiers[j]);
        }
        if (h_mods.size() > modcap) {
            *err = "internal: more split positions than the table holds";
            return COUPE_ERR_CRASH;
        }
        MJ_CK(cudaMemcpyAsync(W.t_off, h_off.data(), S * 8, cudaMemcpyHostToDevice, s));
        MJ_CK(cudaMemcpyAsync(W.t_len, h_len.data(), S * 8, cudaMemcpyHostToDevice, s));
        MJ_CK(cudaMemcpyAsync(W.t_moff, h_moff.data(), S * 4, cudaMemcpyHostToDevice, s));
        MJ_CK(cudaMemcpyAsync(W.t_nsplit, h_nsplit.data(), S * 4, cudaMemcpyHostToDevice, s));
        if (!h_mods.empty())
            MJ_CK(cudaMemcpyAsync(W.t_mods, h_mods.data(), h_mods.size() * 8, cudaMemcpyHostToDevice, s));
        rc = mj_sort(C, d_points, dim, level % dim, W.v, W.v_alt, W.key, W.key_alt, n, W.t_off, S, W.tmp,
                     W.tmp_bytes, s, err);
        if (rc != COUPE_ERR_OK) return rc;
        // exact running weights in sorted order, then the split positions
        // (compute_split_positions, :222-295)
        k_mj_limbs<<<grid, 256, 0, s>>>(d_weights, W.v, n, fs, W.L[0], W.L[1], W.L[2], W.L[3]);
        MJ_CK(cudaGetLastError());
        for (int l = 0; l < 4; ++l) {
            size_t tb = W.tmp_bytes;
            MJ_CK(cub::DeviceScan::InclusiveSum(W.tmp, tb, W.L[l], W.L[l], (int64_t)n, s));
        }
        MjLimbs P;
        for (int l = 0; l < 4; ++l) P.l[l] = W.L[l];
        k_mj_positions<<<(S + 127) / 128, 128, 0, s>>>(P, W.t_off, W.t_len, W.t_moff, W.t_nsplit, W.t_mods, S, fs,
                                                      W.t_pos);
        MJ_CK(cudaGetLastError());
        h_pos.assign(h_mods.size(), 0);
        if (!h_pos.empty())
            MJ_CK(cudaMemcpyAsync(h_pos.data(), W.t_pos, h_pos.size() * 8, cudaMemcpyDeviceToHost, s));
        MJ_CK(cudaStreamSynchronize(s));
        // the next level's segments: each split part's sub-ranges
        // (split_at_mut_many, :297-318) with the scheme's children; finished
        // parts keep their ranges
        std::vector<MjSeg> next;
        for (uint32_t i = 0; i < S; ++i) {
            const MjSeg &g = segs[i];
            if (g.done) {
                next.push_back(g);
                continue;
            }
            uint64_t prev = 0;
            for (uint32_t k = 0; k <= h_nsplit[i]; ++k) {
                const uint64_t p = k < h_nsplit[i] ? std::min<uint64_t>(std::max<uint64_t>(h_pos[h_moff[i] + k], prev),
                                                                        g.len)
                                                   : g.len;
                next.push_back(MjSeg{g.off + prev, p - prev, &g.sch->next[k], false});
                prev = p;
            }
        }
        // finished parts were merged back in range order: keep them (they
        // stay in place through the sorts); drop the done ones only when all
        // are done
        segs.swap(next);
    }
    return COUPE_ERR_OK;
}

}  // namespace cg
