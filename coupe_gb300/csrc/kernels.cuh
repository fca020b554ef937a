// CUDA kernels of the GB300 Rcb/Rib engine (sm_103a).
//
// A tree level is a list of segments (contiguous ranges of the reordered
// point arrays).  Per level:
//   k_hist    streams the keys and weights of the segments still searching
//             and bins them, per segment, on the 2^nbk - 1 candidate cuts
//             that the next nbk bisection steps of coupe's split loop can
//             visit (recursive_bisection.rs:471-572): count, weight and
//             smallest key per bin.
//   k_decide  replays up to nbk steps of that loop exactly from the bins
//             (one warp per segment) and either finishes the split or sets
//             up the next interval.
//   k_reorder once every split of the level is final, moves each segment's
//             items into [left | right] children (stable), replacing
//             reorder_split (recursive_bisection.rs:122-181, 437-453).
//   k_assign  on the last level writes the part ids directly.
// All device-side waits are bounded and report through RunScalars::err.
#pragma once

#include "common.cuh"

namespace cg {

constexpr int BLOCK = 256;
constexpr int NWARPS = BLOCK / 32;
constexpr int MAX_NBK = 10;
constexpr int MAX_NB = 1 << MAX_NBK;
#ifndef CG_HIST_ITEMS
#define CG_HIST_ITEMS 8
#endif
#ifndef CG_HIST_MINB
#define CG_HIST_MINB 4
#endif
constexpr int HIST_ITEMS = CG_HIST_ITEMS;    // items per thread per hist iteration (4-byte keys and weights)
constexpr int HIST_MINB = CG_HIST_MINB;      // histogram CTAs per SM the register budget is sized for
constexpr int CONV_TILE = 2 * BLOCK;          // points per k_convert tile
constexpr int R_ITEMS = 8;                   // items per thread per reorder tile
constexpr int R_TILE = BLOCK * R_ITEMS;      // 2048
constexpr uint64_t LB_AGG = 1ull << 62;      // look-back: aggregate published
constexpr uint64_t LB_INCL = 2ull << 62;     // look-back: inclusive prefix published
constexpr uint64_t LB_VALUE = (1ull << 62) - 1;
constexpr int PACK_WBITS_IN = 20;            // packed histograms take weights below 2^20

// ---------------------------------------------------------------------------
// Small reductions
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint64_t warp_min_u64(uint64_t v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        uint64_t w = __shfl_xor_sync(0xffffffffu, v, o);
        v = w < v ? w : v;
    }
    return v;
}
__device__ __forceinline__ uint64_t warp_max_u64(uint64_t v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        uint64_t w = __shfl_xor_sync(0xffffffffu, v, o);
        v = w > v ? w : v;
    }
    return v;
}
__device__ __forceinline__ uint64_t warp_sum_u64(uint64_t v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}
__device__ __forceinline__ uint32_t warp_min_u32(uint32_t v) { return __reduce_min_sync(0xffffffffu, v); }

template <class O>
__device__ __forceinline__ O warp_min_ord(O v);
template <>
__device__ __forceinline__ uint32_t warp_min_ord<uint32_t>(uint32_t v) {
    return warp_min_u32(v);
}
template <>
__device__ __forceinline__ uint64_t warp_min_ord<uint64_t>(uint64_t v) {
    return warp_min_u64(v);
}

// Exclusive scan of one u64 per thread over the block; returns the prefix
// and writes the block total.  `sh` holds NWARPS + 1 words.
// Inclusive prefix sum over the lanes of a warp.
__device__ __forceinline__ uint64_t warp_incl_scan_u64(uint64_t v) {
    const int lane = threadIdx.x & 31;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint64_t u = __shfl_up_sync(0xffffffffu, v, o);
        if (lane >= o) v += u;
    }
    return v;
}
// Minimum over lanes [lane, 31] of a warp.
template <class O>
__device__ __forceinline__ O warp_suffix_min(O v) {
    const int lane = threadIdx.x & 31;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const O u = __shfl_down_sync(0xffffffffu, v, o);
        if (lane + o < 32 && u < v) v = u;
    }
    return v;
}

__device__ __forceinline__ uint64_t block_exscan_u64(uint64_t v, uint64_t *sh, uint64_t &total) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint64_t inc = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        uint64_t u = __shfl_up_sync(0xffffffffu, inc, o);
        if (lane >= o) inc += u;
    }
    if (lane == 31) sh[warp] = inc;
    __syncthreads();
    if (warp == 0) {
        uint64_t t = lane < (int)(blockDim.x >> 5) ? sh[lane] : 0;
        uint64_t ti = t;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            uint64_t u = __shfl_up_sync(0xffffffffu, ti, o);
            if (lane >= o) ti += u;
        }
        if (lane < (int)(blockDim.x >> 5)) sh[lane] = ti - t;
        if (lane == 31) sh[32] = ti;
    }
    __syncthreads();
    uint64_t r = sh[warp] + inc - v;
    total = sh[32];
    __syncthreads();
    return r;
}

// Largest k with P[k] <= x, for P non-decreasing of length len (P[0] <= x).
__device__ __forceinline__ uint32_t upper_index(const uint64_t *P, uint32_t len, uint64_t x) {
    uint32_t lo = 0, hi = len;  // invariant: P[lo] <= x, answer in [lo, hi)
    while (hi - lo > 1) {
        uint32_t m = (lo + hi) >> 1;
        if (P[m] <= x)
            lo = m;
        else
            hi = m;
    }
    return lo;
}

template <class KT>
__device__ __forceinline__ uint32_t seg_index_of(const Seg<KT> *segs, uint32_t S, uint64_t x) {
    uint32_t lo = 0, hi = S;
    while (hi - lo > 1) {
        uint32_t m = (lo + hi) >> 1;
        if (segs[m].off <= x)
            lo = m;
        else
            hi = m;
    }
    return lo;
}
// The same by position in the level's list of items (Seg::voff).
template <class KT>
__device__ __forceinline__ uint32_t seg_index_of_v(const Seg<KT> *segs, uint32_t S, uint64_t x) {
    uint32_t lo = 0, hi = S;
    while (hi - lo > 1) {
        uint32_t m = (lo + hi) >> 1;
        if (segs[m].voff <= x)
            lo = m;
        else
            hi = m;
    }
    return lo;
}

// The set of input item i, remembered across calls: a thread walking items in
// increasing order searches the set table only when it leaves the last set.
struct SetCursor {
    uint32_t s = ~0u;
    uint64_t beg = 1, end = 0;
    // true when i is in another set than the previous item
    __device__ __forceinline__ bool move(const SetTab &T, uint64_t i) {
        if (i >= beg && i < end) return false;
        s = upper_index(T.off, T.count + 1, i);  // the last set starting at or before i
        beg = T.off[s];
        end = T.off[s + 1];
        return true;
    }
};

// Items [c0, c1) of n for CTA b of g when a CTA walks one contiguous range
// (tiles of `tile` items), so that its items span few sets.
struct CtaRange {
    uint64_t t0, t1;  // tiles
};
__device__ __forceinline__ CtaRange cta_tiles(uint64_t ntiles, uint32_t b, uint32_t g) {
    return CtaRange{ntiles * b / g, ntiles * (b + 1) / g};
}

// run_halted read once per CTA (thread 0, then a barrier), so that every
// thread of the CTA takes the same branch around the barriers that follow.
__device__ __forceinline__ bool cta_halted(const RunScalars *rs) {
    __shared__ int s_halt;
    if (threadIdx.x == 0) s_halt = run_halted(rs) ? 1 : 0;
    __syncthreads();
    return s_halt != 0;
}

__device__ __forceinline__ void atomic_max_ord(uint32_t *p, uint32_t v) { atomicMax(p, v); }

// 64-bit add to shared memory from 32-bit atomics: sm_103 has no 64-bit
// shared-memory add instruction (it becomes a compare-and-swap loop), while
// 32-bit shared atomics are native.  The low word's old value tells whether
// the add carried into the high word; once every add has landed the two words
// hold the exact sum (mod 2^64).
__device__ __forceinline__ void shared_add_u64(uint64_t *p, uint64_t v) {
    uint32_t *w = (uint32_t *)p;
    const uint32_t lo = (uint32_t)v;
    uint32_t hi = (uint32_t)(v >> 32);
    if (lo) {
        const uint32_t old = atomicAdd(&w[0], lo);
        hi += (uint32_t)(old + lo) < old ? 1u : 0u;
    }
    if (hi) atomicAdd(&w[1], hi);
}
__device__ __forceinline__ void atomic_max_ord(uint64_t *p, uint64_t v) {
    atomicMax((unsigned long long *)p, (unsigned long long)v);
}

// Asynchronous global -> shared copies (cp.async); each thread copies its own
// elements, so a tile arrives while the previous one is processed.  4- and
// 8-byte copies also fill L1 (.ca); 16-byte copies go through L2 only (.cg).
template <int BYTES>
__device__ __forceinline__ void cp_async(void *smem, const void *gmem) {
    static_assert(BYTES == 4 || BYTES == 8 || BYTES == 16, "cp.async copies 4, 8 or 16 bytes");
    const uint32_t s = (uint32_t)__cvta_generic_to_shared(smem);
    if (BYTES == 4)
        asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(s), "l"(gmem) : "memory");
    else if (BYTES == 8)
        asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(s), "l"(gmem) : "memory");
    else
        asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(s), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() {
    asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory");
}

// Bulk copies between global and shared memory (the copy engine behind TMA,
// one-dimensional form: no tensor map).  A load is issued by one thread and
// completes on an mbarrier that counts its bytes; a store reads shared
// memory asynchronously, tracked by bulk groups.  Addresses and sizes are
// multiples of 16 bytes.  Shared memory written by threads must be fenced
// into the async proxy before a bulk store reads it, and shared memory read
// by threads before a bulk load overwrites it.
__device__ __forceinline__ uint32_t smem_addr(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }
__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t arrivals) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" ::"r"(smem_addr(bar)), "r"(arrivals) : "memory");
}
__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t *bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(smem_addr(bar)), "r"(bytes)
                 : "memory");
}
// true once the phase with parity `phase` has completed (the call itself
// may suspend the thread for a short, bounded time)
__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, uint32_t phase) {
    uint32_t ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(ok)
        : "r"(smem_addr(bar)), "r"(phase)
        : "memory");
    return ok != 0;
}
// waits at most `limit` polls; false when the phase did not complete
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t *bar, uint32_t phase, uint32_t limit) {
    for (uint32_t i = 0; i <= limit; ++i)
        if (mbar_try_wait(bar, phase)) return true;
    return false;
}
__device__ __forceinline__ void bulk_load(void *dst_smem, const void *src, uint32_t bytes, uint64_t *bar) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];\n" ::"r"(
                     smem_addr(dst_smem)),
                 "l"(src), "r"(bytes), "r"(smem_addr(bar))
                 : "memory");
}
__device__ __forceinline__ void bulk_store(void *dst, const void *src_smem, uint32_t bytes) {
    asm volatile("cp.async.bulk.global.shared::cta.bulk_group [%0], [%1], %2;\n" ::"l"(dst), "r"(smem_addr(src_smem)),
                 "r"(bytes)
                 : "memory");
}
__device__ __forceinline__ void bulk_commit() { asm volatile("cp.async.bulk.commit_group;\n" ::: "memory"); }
// the committed bulk stores have read their shared memory
__device__ __forceinline__ void bulk_wait_read_all() { asm volatile("cp.async.bulk.wait_group.read 0;\n" ::: "memory"); }
// the committed bulk stores have completed
__device__ __forceinline__ void bulk_wait_all() { asm volatile("cp.async.bulk.wait_group 0;\n" ::: "memory"); }
__device__ __forceinline__ void fence_proxy_async_smem() { asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory"); }
__device__ __forceinline__ void fence_mbar_init() { asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory"); }

struct Mat {
    double m[9];
    int on;
};

// Where the band form reads an item's f64 coordinate: the input points (AoS)
// and the basis change k_convert applied to them (rows padded to 3 columns,
// so that a row is chosen with constant indices, not a runtime one).
struct BandSrc {
    const double *pts;
    double m[3][3];
    int on;
    int D;
    unsigned long long *count;  // coordinates read by histogram passes (the run's band_points)
};
inline BandSrc make_band_src(const double *pts, const Mat &M, int D, unsigned long long *count) {
    BandSrc b;
    b.pts = pts;
    b.count = count;
    b.on = M.on;
    b.D = D;
    for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c) b.m[r][c] = (r < D && c < D) ? M.m[r * D + c] : 0.0;
    return b;
}
enum : uint32_t { X_NONE = 0u, X_PENDING = 1u };

// Ordered f64 code of coordinate `coord` of input point `orig`, computed as
// k_convert computes it (the same products and sums, in the same order).
__device__ __forceinline__ uint64_t band_code(const BandSrc &bs, uint64_t orig, int coord) {
    const double *p = bs.pts + orig * (uint64_t)bs.D;
    double x;
    if (bs.on) {
        const double m0 = coord == 0 ? bs.m[0][0] : (coord == 1 ? bs.m[1][0] : bs.m[2][0]);
        const double m1 = coord == 0 ? bs.m[0][1] : (coord == 1 ? bs.m[1][1] : bs.m[2][1]);
        x = __dadd_rn(__dmul_rn(m0, p[0]), __dmul_rn(m1, p[1]));
        if (bs.D == 3) {
            const double m2 = coord == 0 ? bs.m[0][2] : (coord == 1 ? bs.m[1][2] : bs.m[2][2]);
            x = __dadd_rn(x, __dmul_rn(m2, p[2]));
        }
    } else {
        x = p[coord];
    }
    return KeyF64::from_f64(x);
}
// The same, out of line: for the rare band items of hot loops, so that the
// loops stay small (fewer branches and instruction-cache misses).
static __device__ __noinline__ uint64_t band_code_cold(const BandSrc *bs, uint64_t orig, int coord) {
    return band_code(*bs, orig, coord);
}
// Inline for Rcb (a load), out of line for Rib's basis change (its nine
// coefficients would otherwise hold registers across the caller's loop).
__device__ __forceinline__ uint64_t band_code_lean(const BandSrc &bs, uint64_t orig, int coord) {
    if (!bs.on) return KeyF64::from_f64(bs.pts[orig * (uint64_t)bs.D + coord]);
    return band_code_cold(&bs, orig, coord);
}

// ---------------------------------------------------------------------------
// k_convert: AoS f64 points -> D SoA key arrays (coupe's `point[coord] as
// f32`, recursive_bisection.rs:674-679), optionally after the Rib basis change
// p' = M p accumulated column by column (geometry.rs:203-205), and the f64
// bounding box (BoundingBox::from_points, geometry.rs:33-78: NaN never
// updates, the fold starts at f64::MAX / f64::MIN), per point set.  F2K:
// the instance for a basis change with f32 keys and one point set, which
// evaluates it in f32 pairs (point_f2); the others keep their registers.
// ---------------------------------------------------------------------------
template <int D, class KT, bool F2K = false>
__global__ void __launch_bounds__(BLOCK) k_convert(const double *__restrict__ pts, uint64_t n, Mat M,
                                                   typename KT::T *__restrict__ k0,
                                                   typename KT::T *__restrict__ k1,
                                                   typename KT::T *__restrict__ k2, RunScalars *rs, SetTab sets) {
    typedef typename KT::T K;
    __shared__ uint64_t red[2 * 3][NWARPS];
    uint64_t mn[3], mx[3];
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        mn[d] = ord_f64(1.7976931348623157e308);
        mx[d] = ord_f64(-1.7976931348623157e308);
    }
    K *outs[3] = {k0, k1, k2};
    // The basis change with f32 keys (one point set): f32-pair arithmetic
    // decides most points (point_f2), given the matrix entries as pairs.  A
    // point whose f64 value was computed bounds the block's box: s_fmn holds
    // the least f32 above such a value (as an ordered code), s_fmx the
    // greatest below; a point strictly between them cannot be an extreme
    // (those values are input points'), so its exact value is not needed.
    // One box per block, seeded across the whole input, leaves few points to
    // the f64 chain even for inputs in a drifting order (a mesh in index
    // order).
    __shared__ uint32_t s_fmn[3], s_fmx[3];
    F2 m2[D * D];
    bool mfast = false;
    if constexpr (F2K && sizeof(K) == 4) {
        if (M.on && sets.count <= 1) {
            mfast = true;
#pragma unroll
            for (int i = 0; i < D * D; ++i) mfast = f2_split(M.m[i], m2[i]) && mfast;
        }
    }
    // Several sets: each CTA converts one contiguous range of tiles and each
    // thread sends its box to the set table whenever its items enter another
    // set (a few times per thread).
    const bool multi = sets.count > 1;
    SetCursor cur;
    auto flush = [&]() {
        if (cur.s == ~0u) return;
#pragma unroll
        for (int d = 0; d < D; ++d) {
            atomicMin((unsigned long long *)&sets.bmin[cur.s * 3 + d], (unsigned long long)mn[d]);
            atomicMax((unsigned long long *)&sets.bmax[cur.s * 3 + d], (unsigned long long)mx[d]);
            mn[d] = ord_f64(1.7976931348623157e308);
            mx[d] = ord_f64(-1.7976931348623157e308);
        }
    };
    // q receives the raw bits of the (mapped) coordinates; without a basis
    // change nothing here executes an f64 instruction
    auto point = [&](const double *p, uint64_t *q) {
        if (M.on) {
#pragma unroll
            for (int r = 0; r < D; ++r) {
                double acc = __dmul_rn(M.m[r * D + 0], p[0]);
#pragma unroll
                for (int c = 1; c < D; ++c) acc = __dadd_rn(acc, __dmul_rn(M.m[r * D + c], p[c]));
                q[r] = f64_bits(acc);
            }
        } else {
#pragma unroll
            for (int d = 0; d < D; ++d) q[d] = f64_bits(p[d]);
        }
#pragma unroll
        for (int d = 0; d < D; ++d)
            if ((q[d] & 0x7fffffffffffffffull) <= 0x7ff0000000000000ull) {  // not NaN
                const uint64_t o = (q[d] & 0x8000000000000000ull) ? ~q[d] : (q[d] | 0x8000000000000000ull);
                mn[d] = o < mn[d] ? o : mn[d];
                mx[d] = o > mx[d] ? o : mx[d];
            }
    };
    // One point of a basis change with f32 keys, without f64 instructions:
    // y_r = coupe's chain ((m_r0 p0 + m_r1 p1) + m_r2 p2) in f64 is estimated
    // by an f32 pair Y_r within e_r = 2^-39 sum_c |m_rc p_c| (the pair products
    // and sums are good to about 2^-44 of that sum, the chain's own roundings
    // to 5 2^-53 of it, and the f32 sum of the magnitudes to 2^-22).  The
    // key RN32(y_r) is Y_r's high part when [Y_r - e_r, Y_r + e_r] holds no
    // f32 rounding boundary, and the point cannot move the box when its
    // bounds lie strictly inside (mnf, mxf).  false: take the f64 chain.
    auto point_f2 = [&](const double *p, K *kk) -> bool {
        F2 pp[D];
#pragma unroll
        for (int c = 0; c < D; ++c)
            if (!f2_split(p[c], pp[c])) return false;
        F2 y[D];
        float e[D];
#pragma unroll
        for (int r = 0; r < D; ++r) {
            F2 acc = f2_mul(m2[r * D], pp[0]);
            float sabs = fabsf(m2[r * D].h * pp[0].h);
#pragma unroll
            for (int c = 1; c < D; ++c) {
                f2_add(acc, f2_mul(m2[r * D + c], pp[c]));
                sabs += fabsf(m2[r * D + c].h * pp[c].h);
            }
            y[r] = acc;
            e[r] = sabs * 0x1p-39f;
        }
#pragma unroll
        for (int r = 0; r < D; ++r) {
            const uint32_t hb = __float_as_uint(y[r].h);
            const uint32_t ex = (hb >> 23) & 0xffu;
            if (ex < 25u || ex > 253u) return false;  // zero, tiny or near the f32 range's end
            const float u = __uint_as_float((ex - 23u) << 23);              // ulp(|Y_r.h|)
            const float up = 0.5f * u;                                       // half the gap away from zero
            const float down = (hb & 0x7fffffu) ? 0.5f * u : 0.25f * u;     // half the gap towards zero
            const float away = (hb >> 31) ? -y[r].l : y[r].l;               // Y_r - Y_r.h, away from zero
            if (!(away + e[r] < up && e[r] - away < down)) return false;
            kk[r] = y[r].h;
        }
#pragma unroll
        for (int r = 0; r < D; ++r) {
            const float slack = fabsf(y[r].l) + e[r] + fabsf(y[r].h) * 0x1p-22f;
            const float mnf = unord_f32(*(volatile uint32_t *)&s_fmn[r]);
            const float mxf = unord_f32(*(volatile uint32_t *)&s_fmx[r]);
            if (!(y[r].h - slack > mnf) || !(y[r].h + slack < mxf)) return false;
        }
        return true;
    };
    // after the f64 chain: the point's value bounds the block's box
    auto certify = [&](const uint64_t *q) {
#pragma unroll
        for (int d = 0; d < D; ++d) {
            if ((q[d] & 0x7fffffffffffffffull) > 0x7ff0000000000000ull) continue;  // NaN: not in the box
            const float f = f32_from_bits(f64bits_to_f32bits(q[d]));
            if (!isfinite(f)) continue;
            atomicMin(&s_fmn[d], ord_f32(f32_step(f, 1)));   // above the value
            atomicMax(&s_fmx[d], ord_f32(f32_step(f, -1)));  // below it
        }
    };
    // F2K: the points that need the f64 chain wait in a per-warp queue (their
    // coordinates and output position) and are evaluated 32 at a time, one
    // per lane, so that the FP64 pipe runs whole warps instead of one lane
    __shared__ double s_qp[F2K ? NWARPS : 1][F2K ? 64 : 1][3];
    __shared__ uint64_t s_qi[F2K ? NWARPS : 1][F2K ? 64 : 1];
    uint32_t qn = 0;  // entries in this warp's queue (the same in every lane)
    auto drain = [&](uint32_t cnt) {  // the first cnt <= 32 entries; every lane calls it
        const int ql = threadIdx.x & 31, qw = threadIdx.x >> 5;
        __syncwarp();
        if ((uint32_t)ql < cnt) {
            uint64_t q[D];
            point(&s_qp[qw][ql][0], q);
            const uint64_t i = s_qi[qw][ql];
#pragma unroll
            for (int d = 0; d < D; ++d) outs[d][i] = KT::from_f64_bits(q[d]);
            certify(q);
        }
        __syncwarp();
        qn -= cnt;  // the rest (fewer than 32) moves to the front
        double v[D];
        uint64_t vi = 0;
        if ((uint32_t)ql < qn) {
#pragma unroll
            for (int d = 0; d < D; ++d) v[d] = s_qp[qw][cnt + ql][d];
            vi = s_qi[qw][cnt + ql];
        }
        __syncwarp();
        if ((uint32_t)ql < qn) {
#pragma unroll
            for (int d = 0; d < D; ++d) s_qp[qw][ql][d] = v[d];
            s_qi[qw][ql] = vi;
        }
        __syncwarp();
    };
    if (F2K && mfast && n > 0) {
        // the box starts from one exact point per thread, drawn across the
        // whole input (an odd-multiplier hash of the thread's index), so its
        // extremes start near the input's
        if (threadIdx.x < 3) {
            s_fmn[threadIdx.x] = ord_f32(INFINITY);
            s_fmx[threadIdx.x] = ord_f32(-INFINITY);
        }
        __syncthreads();
        const uint64_t g = (uint64_t)blockIdx.x * BLOCK + threadIdx.x;
        uint64_t q[D];
        point(pts + ((g * 0x9E3779B97F4A7C15ull) % n) * D, q);
        certify(q);
        __syncthreads();
    }
    // Tiles of CONV_TILE points move to shared memory by asynchronous copies
    // (the next tile lands while this one is converted): consecutive threads
    // copy consecutive 16-byte pieces of the AoS input, so the loads are
    // coalesced; each thread then converts whole points from shared memory
    // and the SoA key stores are coalesced too.
    __shared__ __align__(16) double tile[2][CONV_TILE * D];
    const bool al16 = ((uintptr_t)pts & 15) == 0;
    const uint64_t ntiles = (n + CONV_TILE - 1) / CONV_TILE;
    auto prefetch = [&](uint64_t t, int buf) {
        const uint64_t p0 = t * CONV_TILE;
        const uint32_t nd = (uint32_t)(min((uint64_t)CONV_TILE, n - p0) * D);  // doubles in the tile
        const double *src = pts + p0 * D;
        if (al16) {
            // the tile starts on a 16-byte boundary (CONV_TILE * D * 8 is a multiple of 16)
            for (uint32_t q = threadIdx.x; q < nd / 2; q += BLOCK) cp_async<16>(&tile[buf][2 * q], src + 2 * q);
            if ((nd & 1) && threadIdx.x == 0) cp_async<8>(&tile[buf][nd - 1], src + nd - 1);
        } else {
            for (uint32_t q = threadIdx.x; q < nd; q += BLOCK) cp_async<8>(&tile[buf][q], src + q);
        }
        cp_async_commit();
    };
    int buf = 0;
    uint64_t t_first = blockIdx.x, t_end = ntiles, t_step = gridDim.x;
    if (multi) {
        const CtaRange r = cta_tiles(ntiles, blockIdx.x, gridDim.x);
        t_first = r.t0;
        t_end = r.t1;
        t_step = 1;
    }
    if (t_first < t_end) prefetch(t_first, 0);
    for (uint64_t t = t_first; t < t_end; t += t_step) {
        const uint64_t tn = t + t_step;
        if (tn < t_end) {
            prefetch(tn, buf ^ 1);
            cp_async_wait<1>();
        } else {
            cp_async_wait<0>();
        }
        __syncthreads();
        const uint64_t p0 = t * CONV_TILE;
        const uint32_t np = (uint32_t)min((uint64_t)CONV_TILE, n - p0);
#pragma unroll
        for (int r = 0; r < CONV_TILE / BLOCK; ++r) {
            const uint32_t j = r * BLOCK + threadIdx.x;
            bool queue = false;  // F2K: this lane's point waits for the f64 chain
            if (j < np) {
                if (multi && (p0 + j < cur.beg || p0 + j >= cur.end)) {
                    flush();
                    cur.move(sets, p0 + j);
                }
                bool done = false;
                if constexpr (F2K && sizeof(K) == 4) {
                    if (mfast) {
                        K kk[D];
                        if (point_f2(&tile[buf][j * D], kk)) {
#pragma unroll
                            for (int d = 0; d < D; ++d) outs[d][p0 + j] = kk[d];
                        } else {
                            queue = true;
                        }
                        done = true;
                    }
                }
                if (!done) {
                    uint64_t q[D];
                    point(&tile[buf][j * D], q);
#pragma unroll
                    for (int d = 0; d < D; ++d) outs[d][p0 + j] = KT::from_f64_bits(q[d]);
                }
            }
            if (F2K && mfast) {
                const int ql = threadIdx.x & 31, qw = threadIdx.x >> 5;
                const uint32_t m = __ballot_sync(0xffffffffu, queue);
                if (queue) {
                    const uint32_t at = qn + __popc(m & ((1u << ql) - 1));
#pragma unroll
                    for (int d = 0; d < D; ++d) s_qp[qw][at][d] = tile[buf][j * D + d];
                    s_qi[qw][at] = p0 + j;
                }
                qn += __popc(m);
                if (qn >= 32) drain(32);
            }
        }
        __syncthreads();  // the buffer is free for the tile after next
        buf ^= 1;
    }
    if (F2K && mfast && qn) drain(qn);
    if (multi) {
        flush();
        return;
    }
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int d = 0; d < D; ++d) {
        const uint64_t a = warp_min_u64(mn[d]), b = warp_max_u64(mx[d]);
        if (lane == 0) {
            red[2 * d][warp] = a;
            red[2 * d + 1][warp] = b;
        }
    }
    __syncthreads();
    if (threadIdx.x < 2 * D) {
        const int d = threadIdx.x >> 1;
        const bool is_max = threadIdx.x & 1;
        uint64_t v = red[threadIdx.x][0];
        for (int w = 1; w < NWARPS; ++w) {
            const uint64_t u = red[threadIdx.x][w];
            v = is_max ? (u > v ? u : v) : (u < v ? u : v);
        }
        if (is_max)
            atomicMax((unsigned long long *)&rs->bbox_max_ord[d], (unsigned long long)v);
        else
            atomicMin((unsigned long long *)&rs->bbox_min_ord[d], (unsigned long long)v);
    }
}

// Largest |w| of f64 weights as raw bits (non-finite values sort above).
static __global__ void __launch_bounds__(BLOCK) k_wabs_max(const double *__restrict__ w, uint64_t n, RunScalars *rs,
                                                          SetTab sets) {
    uint64_t m = 0;
    if (sets.count > 1) {
        // one contiguous range per CTA; a thread's maximum goes to its set
        // whenever its items enter another set
        const CtaRange r = cta_tiles((n + BLOCK - 1) / BLOCK, blockIdx.x, gridDim.x);
        SetCursor cur;
        for (uint64_t i = r.t0 * BLOCK + threadIdx.x; i < min(n, r.t1 * BLOCK); i += BLOCK) {
            if (i < cur.beg || i >= cur.end) {
                if (cur.s != ~0u) atomicMax((unsigned long long *)&sets.wabs[cur.s], (unsigned long long)m);
                m = 0;
                cur.move(sets, i);
            }
            const uint64_t b = (uint64_t)__double_as_longlong(w[i]) & 0x7fffffffffffffffull;
            m = b > m ? b : m;
        }
        if (cur.s != ~0u) atomicMax((unsigned long long *)&sets.wabs[cur.s], (unsigned long long)m);
        return;
    }
    for (uint64_t i = (uint64_t)blockIdx.x * BLOCK + threadIdx.x; i < n; i += (uint64_t)gridDim.x * BLOCK) {
        uint64_t b = (uint64_t)__double_as_longlong(w[i]) & 0x7fffffffffffffffull;
        m = b > m ? b : m;
    }
    m = warp_max_u64(m);
    if ((threadIdx.x & 31) == 0) atomicMax((unsigned long long *)&rs->wabs_max_bits, (unsigned long long)m);
}

// Shift of the approximate binned weights of a set of n items: its
// fixed-point weights are below 2^(126 - ceil(log2 n)), so q >> shift < 2^25.
__device__ __forceinline__ int approx_shift(uint64_t n) { return 101 - ceil_log2_u64(n); }

// Several sets, f64 weights: each set's fixed-point scale (from its own
// largest |w| and size, as a run of that set alone chooses it).
static __global__ void k_set_fs(SetTab sets, RunScalars *rs) {
    const uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= sets.count) return;
    const uint64_t b = sets.wabs[s], n = sets.off[s + 1] - sets.off[s];
    if (b >= 0x7ff0000000000000ull) atomicOr(&rs->err, ERR_NONFINITE_WEIGHT);
    sets.fs[s] = fixed_scale_from_max(__longlong_as_double((long long)b), n);
    sets.qb[s] = approx_shift(n);
}

__device__ __forceinline__ int run_fscale(const RunScalars *rs, uint64_t n) {
    return fixed_scale_from_max(__longlong_as_double((long long)rs->wabs_max_bits), n);
}

// Total weight (recursive_bisection.rs:684), order independent.
template <class WT>
__global__ void __launch_bounds__(BLOCK) k_wsum(const typename WT::S *__restrict__ w, uint64_t n, RunScalars *rs,
                                                uint16_t *__restrict__ c16, SetTab sets) {
    const bool multi = sets.count > 1;
    int fs = WT::LIMBS > 1 && !multi ? run_fscale(rs, n) : 0;
    uint64_t acc[WT::LIMBS];
#pragma unroll
    for (int l = 0; l < WT::LIMBS; ++l) acc[l] = 0;
    bool wide = WT::LIMBS > 1, not16 = false, neg = false;
    // several sets: one contiguous range per CTA; a thread's sum goes to its
    // set whenever its items enter another set
    uint64_t i0 = (uint64_t)blockIdx.x * BLOCK + threadIdx.x, i1 = n, step = (uint64_t)gridDim.x * BLOCK;
    if (multi) {
        const CtaRange r = cta_tiles((n + BLOCK - 1) / BLOCK, blockIdx.x, gridDim.x);
        i0 = r.t0 * BLOCK + threadIdx.x;
        i1 = min(n, r.t1 * BLOCK);
        step = BLOCK;
    }
    SetCursor cur;
    auto flush = [&]() {
        if (cur.s == ~0u) return;
#pragma unroll
        for (int l = 0; l < WT::LIMBS; ++l) {
            if (acc[l]) atomicAdd((unsigned long long *)&sets.wsum[cur.s * 4 + l], (unsigned long long)acc[l]);
            acc[l] = 0;
        }
    };
    for (uint64_t i = i0; i < i1; i += step) {
        if (multi && (i < cur.beg || i >= cur.end)) {
            flush();
            cur.move(sets, i);
            if (WT::LIMBS > 1) fs = sets.fs[cur.s];
        }
        const typename WT::S wi = w[i];
        uint64_t q[WT::LIMBS];
        WT::limbs(wi, fs, q);
#pragma unroll
        for (int l = 0; l < WT::LIMBS; ++l) acc[l] += q[l];
        if constexpr (WT::LIMBS > 1) {
            neg |= wi < 0;
        } else {
            wide |= !(wi >= 0 && wi < (1 << PACK_WBITS_IN));
            if (c16) {
                // the 16-bit copy of the level loop, used when no weight fails
                c16[i] = (uint16_t)wi;
                not16 |= !(wi >= 0 && wi < 65536);
            }
        }
    }
    if (__any_sync(0xffffffffu, not16) && (threadIdx.x & 31) == 0) atomicOr(&rs->narrow16, 1u);
    if (__any_sync(0xffffffffu, wide) && (threadIdx.x & 31) == 0) atomicOr(&rs->wide, 1u);
    if (__any_sync(0xffffffffu, neg) && (threadIdx.x & 31) == 0) atomicOr(&rs->fneg, 1u);
    if (multi) {
        flush();
        return;
    }
#pragma unroll
    for (int l = 0; l < WT::LIMBS; ++l) {
        uint64_t v = warp_sum_u64(acc[l]);
        if ((threadIdx.x & 31) == 0 && v) atomicAdd((unsigned long long *)&rs->wsum_limbs[l], (unsigned long long)v);
    }
}

// A root segment: items [off, off + n), its weight sum and its f64 box
// (rcb_recurse's first call, recursive_bisection.rs:696).
template <class KT, class WT>
__device__ Seg<KT> root_seg(uint64_t off, uint64_t voff, uint64_t n, uint32_t set, const uint64_t *limbs, int fs,
                            const uint64_t *bmin, const uint64_t *bmax, int D) {
    Seg<KT> s;
    s.off = off;
    s.voff = voff;
    s.heap = 0;
    s.sum = WT::bits(WT::value(limbs, fs));
    s.prev = ~0ull;
    s.wl = 0;
    s.n = (uint32_t)n;
    s.nleft = 0;
    s.state = SEG_ACTIVE;
    s.steps = 0;
    s.child = 0;
    s.xstate = 0;
    s.xkey = 0;
    s.set = set;
    s.sumx = SUMX_NONE;
    s.exactw = 0;
    s.wlx = 0;
    s.pad2 = 0;
    for (int l = 0; l < 4; ++l) s.xq[l] = 0;
    s.xcut = 0;
    s.xmin = ~0ull;
    for (int d = 0; d < 3; ++d) {
        double a = d < D ? unord_f64(bmin[d]) : 0.0;
        double b = d < D ? unord_f64(bmax[d]) : 0.0;
        s.bmin[d] = KT::cut_from_f64(a);
        s.bmax[d] = KT::cut_from_f64(b);
    }
    s.lo = s.bmin[0];
    s.hi = s.bmax[0];
    s.pivot = 0;
    s.split_pos = 0;
    return s;
}

// Root segment of a one-set run.
template <class KT, class WT>
__global__ void k_root(Seg<KT> *segs, uint32_t *list, uint64_t *P, uint64_t n, int D, RunScalars *rs, int approx,
                       uint64_t *lvl) {
    lvl[0] = 1;  // level 0: one segment of n items
    lvl[1] = n;
    const int fs = WT::LIMBS > 1 ? run_fscale(rs, n) : 0;
    rs->fscale = fs;
    rs->qb = approx_shift(n);
    // approximate bins need non-negative fixed-point weights
    rs->fapprox = WT::LIMBS > 1 && approx && rs->fneg == 0;
    if (WT::LIMBS > 1 && rs->wabs_max_bits >= 0x7ff0000000000000ull) rs->err |= ERR_NONFINITE_WEIGHT;
    segs[0] = root_seg<KT, WT>(0, 0, n, 0, rs->wsum_limbs, fs, rs->bbox_min_ord, rs->bbox_max_ord, D);
    list[0] = 0;
    P[0] = 0;
    P[1] = n;
}

// Root segments of several sets: root r belongs to set roots[r] and starts at
// P[r] in the level's list of items (P written by the host).
template <class KT, class WT>
__global__ void k_roots(Seg<KT> *segs, uint32_t *list, const uint64_t *P, const uint32_t *roots, uint32_t nroots,
                        int D, SetTab sets, RunScalars *rs, int approx, uint64_t *lvl) {
    const uint32_t r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r == 0) {
        rs->fapprox = WT::LIMBS > 1 && approx && rs->fneg == 0;
        lvl[0] = nroots;  // level 0: the root segments and their items
        lvl[1] = P[nroots];
    }
    if (r >= nroots) return;
    const uint32_t st = roots[r];
    const int fs = WT::LIMBS > 1 ? sets.fs[st] : 0;
    segs[r] = root_seg<KT, WT>(sets.off[st], P[r], sets.off[st + 1] - sets.off[st], st, &sets.wsum[st * 4], fs,
                               &sets.bmin[st * 3], &sets.bmax[st * 3], D);
    list[r] = r;
}

// Initial values of the set table's accumulators.
static __global__ void k_sets_init(SetTab sets) {
    const uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= sets.count) return;
    for (int d = 0; d < 3; ++d) {
        sets.bmin[s * 3 + d] = ord_f64(1.7976931348623157e308);
        sets.bmax[s * 3 + d] = ord_f64(-1.7976931348623157e308);
    }
    for (int l = 0; l < 4; ++l) sets.wsum[s * 4 + l] = 0;
    sets.wabs[s] = 0;
    sets.fs[s] = 0;
    sets.qb[s] = 0;
    sets.minheap[s] = ~0ull;
}

// ---------------------------------------------------------------------------
// Candidate cuts of a segment.  The 2^nbk - 1 cuts that coupe's loop can
// compute in its next nbk steps from the interval [lo, hi]
// (recursive_bisection.rs:472, 564-571) form a binary tree whose in-order
// sequence is non-decreasing: heap node (depth d, position p) has in-order
// rank (2p+1) 2^(nbk-1-d) - 1.  A key's bin is the number of cuts c with
// !(key < c), i.e. the leaf reached by descending the tree with
// `key < c ? left : right`; bins are in key order.
// ---------------------------------------------------------------------------
template <class KT, bool WARP = false>
__device__ __forceinline__ void build_sorted_cuts(typename KT::C lo, typename KT::C hi, int nbk,
                                                  typename KT::C *cuts, float4 *cbb = nullptr) {
    typedef typename KT::C K;
    // One depth of the tree at a time: node (d, p) at in-order rank
    // r = (2p + 1) h - 1, h = 2^(nbk-1-d), is the midpoint of the cuts at ranks
    // r - h and r + h (or lo / hi beyond the ends), which are exactly the
    // ancestors coupe's loop would have reached it from; one midpoint per cut
    // (f64 midpoints are costly on GB300).  Contains barriers: every thread of
    // the block (or with WARP, of the warp) calls it.
    const int nb = 1 << nbk;
    const int tr = WARP ? (threadIdx.x & 31) : threadIdx.x, TS = WARP ? 32 : blockDim.x;
    for (int d = 0; d < nbk; ++d) {
        const int h = 1 << (nbk - 1 - d);
        for (int p = tr; p < (1 << d); p += TS) {
            const int r = (2 * p + 1) * h - 1;
            const K a = r - h < 0 ? lo : cuts[r - h];
            const K b = r + h >= nb - 1 ? hi : cuts[r + h];
            cuts[r] = KT::cmid(a, b);
            if constexpr (KT::BAND) {
                // the band form also needs each cut's f32 bounds (bin r's
                // upper edge and band)
                const CutBounds cb = band_bounds(cuts[r]);
                cbb[r].y = cb.hi;
                cbb[r].z = cb.lo;
                cbb[r].w = 1.f;
            }
        }
        if (WARP)
            __syncwarp();
        else
            __syncthreads();
    }
    if constexpr (KT::BAND) {
        // bin b's record: (upper bound of cut b-1, upper bound of cut b,
        // lower bound of cut b, 1 when cut b exists); one 16-byte load
        // checks a guessed bin
        for (int b = tr; b < nb; b += TS) {
            cbb[b].x = b > 0 ? cbb[b - 1].y : -INFINITY;
            if (b == nb - 1) {
                cbb[b].y = INFINITY;
                cbb[b].z = INFINITY;
                cbb[b].w = 0.f;
            }
        }
        if (WARP)
            __syncwarp();
        else
            __syncthreads();
    }
}

// Grid position of a key in the interval [lo, hi] of nb bins:
// f = (approx(k) - l) sc + s with l = approx_cut(lo), sc = nb / RN32(hi - lo)
// (within 2^-23 of nb / (hi - lo): two f32 roundings) and the shift
// s = RN32(l - lo) sc, which corrects for l != lo (f64 interval ends; it is
// below the margin's ulp term, so its own rounding is negligible); i.e.
// (approx(k) - lo) nb / (hi - lo) up to roundings.  No f64 division.
struct GridMap {
    float l, sc, s;
    bool ok;  // finite, non-empty interval of normal f32 width
};
template <class KT>
__device__ __forceinline__ GridMap grid_map(typename KT::C lo, typename KT::C hi, int nb) {
    GridMap g;
    g.l = KT::approx_cut(lo);
    float w;
    if constexpr (sizeof(typename KT::C) == 4) {
        w = hi - lo;  // f32 interval ends: l == lo
        g.s = 0.0f;
        g.sc = (float)nb / w;
    } else {
        const double lod = KT::cval(lo), hid = KT::cval(hi);
        w = (float)(hid - lod);
        g.sc = (float)nb / w;
        g.s = (float)((double)g.l - lod) * g.sc;
    }
    g.ok = w >= 1.17549435e-38f && isfinite(g.l) && isfinite(g.sc) && isfinite(g.s);  // false for NaN
    return g;
}

// Bin lookup: an arithmetic first guess (cuts are close to an even grid),
// corrected against the exact sorted cuts (the guess, or its neighbour when
// it is one bin off); a binary search when the interval is degenerate or not
// finite, or the guess is further off.
struct BinGuess {
    float lo, scale, shift;
    int fast;
};

__device__ __forceinline__ BinGuess bin_guess(const GridMap &m) {
    BinGuess g;
    g.lo = m.l;
    g.scale = m.sc;
    g.shift = m.s;
    g.fast = m.ok;
    return g;
}

template <class KT>
__device__ __forceinline__ int bin_sorted(typename KT::T key, const typename KT::T *cuts, int nb, const BinGuess &g) {
    if (g.fast) {
        float f = fmaf(KT::approx(key) - g.lo, g.scale, g.shift);
        f = fminf(fmaxf(f, 0.0f), (float)(nb - 1));
        int b = __float2int_rz(f);
        if (b > 0 && KT::lt(key, cuts[b - 1]))
            --b;
        else if (b < nb - 1 && !KT::lt(key, cuts[b]))
            ++b;
        // the guess, if its two cuts confirm it; else the binary search
        // (cuts crowded at the precision of the keys make the guess far off)
        if ((b == 0 || !KT::lt(key, cuts[b - 1])) && (b == nb - 1 || KT::lt(key, cuts[b]))) return b;
    }
    int l = 0, r = nb - 1;
    while (l < r) {
        const int m = (l + r) >> 1;
        if (KT::lt(key, cuts[m]))
            r = m;
        else
            l = m + 1;
    }
    return l;
}

// Band form: the bin of a key (the number of cuts c with x >= c).  Cuts whose
// upper bound lies below the key are certainly passed; if the next cut's
// lower bound does not exceed the key, the f64 code decides from there.
template <class KT>
__device__ __forceinline__ int bin_band(float k, const uint64_t *cuts, const float4 *cbb, int nb,
                                        const BinGuess &g, bool &in_band) {
    int b = -1;
    float4 q;
    if (g.fast) {
        float f = fmaf(k - g.lo, g.scale, g.shift);
        f = fminf(fmaxf(f, 0.0f), (float)(nb - 1));
        b = __float2int_rz(f);
        q = cbb[b];
        // one step to the neighbour when the guess is one bin off
        if (b > 0 && !(k > q.x)) {
            --b;
            q = cbb[b];
        } else if (b < nb - 1 && k > q.y) {
            ++b;
            q = cbb[b];
        }
        // the guess stands if the bounds of its two cuts confirm it
        if (!((b == 0 || k > q.x) && (b == nb - 1 || !(k > q.y)))) b = -1;
    }
    if (b < 0) {
        // binary search: the first bin whose upper cut bound is >= k (a
        // narrow interval crowds many cuts into one f32 value)
        int l = 0, r = nb - 1;
        while (l < r) {
            const int m = (l + r) >> 1;
            if (k > cbb[m].y)
                l = m + 1;
            else
                r = m;
        }
        b = l;
        q = cbb[b];
    }
    in_band = q.w != 0.f && !(k < q.z);  // cut b's band: finish with bin_band_exact
    return b;
}
// The bin from cut b on, from the f64 code: the first cut above c, by binary
// search (a narrow interval can hold hundreds of cuts within one f32 band).
__device__ __forceinline__ int bin_band_exact(int b, uint64_t c, const uint64_t *cuts, int nb) {
    // usually cut b or b + 1 is the first above c (the key lies in one
    // cut's band); crowded cuts take the binary search
    if (b >= nb - 1 || KeyF64::lt(c, cuts[b])) return b;
    if (b + 1 >= nb - 1 || KeyF64::lt(c, cuts[b + 1])) return b + 1;
    b += 2;
    int r = nb - 1;  // answer in [b, r]
    while (b < r) {
        const int m = (b + r) >> 1;
        if (KeyF64::lt(c, cuts[m]))
            r = m;
        else
            b = m + 1;
    }
    return b;
}

// ---------------------------------------------------------------------------
// Bins without looking at the cuts.  A key's grid position
// f = (approx(k) - l) sc + s (grid_map) is (approx(k) - lo) nb / (hi - lo) to
// within E = (nb + 1) 2^-21 for keys inside the interval (the roundings of
// approx(k) - l and of the fused multiply-add, 2^-24 each, and sc's 2^-23, of
// values below nb + 1, with room to spare).  Every cut c_r lies within `dev` of its grid
// point lo + (r+1)(hi - lo)/nb, and the key within `dk` of the value whose
// bin is wanted (ulps of M = max(|lo|, |hi|)):
//   KeyF32: dev = nbk/2 (each of the at most nbk f32 midpoints on a cut's
//           path adds at most half an ulp), dk = 0;
//   KeyF64: f64 midpoints are exact to far below an f32 ulp (dev ~ 0), and
//           approx(k) truncates the key to f32: dk = 1;
//   KeyBand: dev ~ 0; a key in a cut's band [RD32(c), RU32(c)] lies within
//           one ulp of the cut, and x within half an ulp of its key: 1.
// So when the fraction of f is more than m = 1.01 sc (dev + dk) ulp + E
// (+ 2^-20 for the rounding of m) away from both bin edges, floor(f) is the
// key's bin and, in the band form, the key is outside every cut's band; the
// other keys take the exact search.  Intervals where m would exceed 1/4
// (narrow intervals far from zero, or ranges near the limits of f32) use the
// exact search for every key (m = 2 never passes the test).
// ---------------------------------------------------------------------------
struct FastBin {
    float l, sc, s, m, m1;  // m1 = 1 - m
};
template <class KT>
__device__ __forceinline__ FastBin fast_bin(const GridMap &g, typename KT::C hi, int nbk) {
    FastBin r;
    const float nb = (float)(1 << nbk);
    r.l = g.l;
    r.sc = g.sc;
    r.s = g.s;
    r.m = 2.0f;
    r.m1 = -1.0f;
    const float M = fmaxf(fabsf(g.l), fabsf(KT::approx_cut(hi)));
    if (!g.ok || !(M > 1e-30f) || !(M < 1e37f)) return r;
    const float ulps = (!KT::BAND && sizeof(typename KT::T) == 4) ? 0.5f * (float)nbk : 1.0f;
    const float u = M * 1.1920929e-7f + 1.4012985e-45f;  // >= ulp(M)
    const float m = 1.01f * ulps * u * g.sc + (nb + 1.0f) * 4.7683716e-7f + 9.5367432e-7f;
    if (m < 0.25f) {
        r.m = m;
        r.m1 = 1.0f - m;
    }
    return r;
}

// Keys that are certainly below every cut (bin 0) or at or above every cut
// (the last bin): every cut lies in [lo, hi].  In the band form, by the f32
// bounds of the f64 interval ends.
template <class KT>
struct EdgeTest {
    typename KT::T lo, hi;
    __device__ __forceinline__ bool below(typename KT::T k) const {
        if constexpr (KT::BAND)
            return k < lo;
        else
            return KT::lt(k, lo);
    }
    __device__ __forceinline__ bool above(typename KT::T k) const {
        if constexpr (KT::BAND)
            return k > hi;
        else
            return !KT::lt(k, hi);
    }
};
template <class KT>
__device__ __forceinline__ EdgeTest<KT> edge_test(typename KT::C lo, typename KT::C hi) {
    EdgeTest<KT> e;
    const typename KT::A M = fmax(fabs(KT::cval(lo)), fabs(KT::cval(hi)));
    if (!isfinite(M + M)) {
        // a midpoint may overflow to an infinite cut outside [lo, hi]: no
        // shortcut (below: nothing is under -inf; above: only +inf, which
        // is at or above every cut anyway; the band form: nothing above +inf)
        if constexpr (KT::BAND) {
            e.lo = -INFINITY;
            e.hi = INFINITY;
        } else {
            e.lo = KT::cut_from_f64(-INFINITY);
            e.hi = KT::cut_from_f64(INFINITY);
        }
        return e;
    }
    if constexpr (KT::BAND) {
        e.lo = band_bounds(lo).lo;  // k < RD32(lo) proves x < lo
        e.hi = band_bounds(hi).hi;  // k > RU32(hi) proves x > hi
    } else {
        e.lo = lo;
        e.hi = hi;
    }
    return e;
}

// Global histogram slots: [segment][bin]; inv stores ~ord(key) so that an
// all-zero slot means "no key" and atomicMax of ~ord is a min of keys.
template <class KT, class WT>
struct Hist {
    uint32_t *cnt;
    uint64_t *w;  // [seg][bin][LIMBS]
    typename KT::Ord *inv;
};

// Packed shared-memory accumulator for integer weights in [0, 2^20): one
// 64-bit atomic adds (1 << 44) + w, so count and weight share a word; a
// window of fewer than 2^20 items can neither overflow the 20-bit count nor
// carry out of the 44-bit weight sum.
constexpr int PACK_SHIFT = 44;
constexpr uint64_t PACK_WMASK = (1ull << PACK_SHIFT) - 1;
constexpr uint64_t PACK_WINDOW = 1ull << 19;

// Most bins per segment a histogram pass keeps in shared memory: four
// 64-bit limbs per bin for f64 weights allow fewer.
template <class WT>
__host__ __device__ constexpr int hist_max_nbk() {
    return WT::LIMBS > 1 ? 9 : MAX_NBK;
}

// ---------------------------------------------------------------------------
// k_hist: one static chunk of the active items per CTA; per segment piece a
// shared-memory histogram flushed to the segment's global bins.
// ---------------------------------------------------------------------------
template <class KT, class WT>
__global__ void __launch_bounds__(BLOCK, WT::LIMBS > 1 ? 3 : HIST_MINB) k_hist(const Seg<KT> *__restrict__ segs, const uint32_t *__restrict__ list,
                                                const uint64_t *__restrict__ P, uint32_t nlist,
                                                const typename KT::T *__restrict__ keys,
                                                const typename WT::S *__restrict__ wts, Hist<KT, WT> H, int nbk,
                                                uint64_t n_total, const RunScalars *rs, const uint64_t *nlist_ptr,
                                                const uint32_t *__restrict__ isrc, BandSrc bs, int coord,
                                                Seg<KT> *segs_w, const int32_t *__restrict__ set_fs,
                                                const int32_t *__restrict__ set_qb) {
    typedef typename KT::T K;
    typedef typename KT::C CK;
    typedef typename KT::Ord O;
    constexpr int L = WT::LIMBS;
    constexpr int HNB = 1 << hist_max_nbk<WT>();
    constexpr int BNB = KT::BAND ? HNB : 1;
    // items per thread per iteration: fewer with 8-byte keys or weights
    // (registers)
    constexpr int HI = (sizeof(K) == 4 && sizeof(typename WT::S) <= 4 && L == 1) ? HIST_ITEMS : HIST_ITEMS / 2;
    // 16-bit weights: a bin is a 32-bit count and a 32-bit weight sum, each
    // added by one native shared atomic, over windows of at most 2^15 items
    // (sums below 2^31); other weights add 64-bit words from 32-bit atomics
    constexpr bool C16 = sizeof(typename WT::S) == 2;
    constexpr uint64_t WINDOW = C16 ? (1ull << 15) : PACK_WINDOW;
    __shared__ CK cuts[HNB];
    __shared__ float4 cbb[BNB];  // band form: f32 bounds of each bin (see build_sorted_cuts)
    __shared__ uint64_t sw[HNB * L];  // packed count|weight (L == 1 and !wide), else weight limbs
    uint32_t *const sw32 = (uint32_t *)sw;  // 16-bit weights: 32-bit weight sums (counts in scnt)
    __shared__ uint32_t scnt[HNB];
    __shared__ O sinv[HNB];
    // each warp's queue of items that need the exact search over the cuts
    // (band form: or their f64 coordinate), as offsets in the piece, drained
    // 32 at a time, one item per lane, so that their dependent loads overlap
    // instead of stalling every iteration
    __shared__ uint32_t s_q[NWARPS][64];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int NB = 1 << nbk;
    int fs = L > 1 ? rs->fscale : 0;  // several sets: each set's own (set_fs)
    int qb = L > 1 ? rs->qb : 0;      // several sets: each set's own (set_qb)
    const bool packed_all = L == 1 && rs->wide == 0;
    const bool fapprox = L > 1 && rs->fapprox != 0;
    if (cta_halted(rs)) return;
    // the list's length from the device (a speculative pass: the list the
    // last scan left; a queued level: its segment count)
    if (nlist_ptr) nlist = (uint32_t)*nlist_ptr;
    const uint64_t T = P[nlist];
    const uint64_t c0 = T * blockIdx.x / gridDim.x, c1 = T * (blockIdx.x + 1) / gridDim.x;
    if (c0 >= c1) return;
    uint32_t k = upper_index(P, nlist + 1, c0);
    uint64_t pos = c0;
    int cur_s = -1;
    // Small segments (at most SMALL_SEG items, at most SNB bins), whole in
    // this CTA's range, are binned one per warp, up to NWARPS at once, each
    // warp on its own slice of the shared arrays with warp barriers only
    // (the CTA path below costs a dozen block barriers per piece).  One item
    // per lane per step; a band item's f64 coordinate is read in place.
    constexpr int SNB = HNB / NWARPS;
    constexpr uint64_t SMALL_SEG = 4096;
    auto small_seg = [&](const uint32_t kk) {
        const uint32_t s = list[kk];
        const Seg<KT> &sg = segs[s];
        const int sfs = L > 1 ? (set_fs ? set_fs[sg.set] : rs->fscale) : 0;
        const int sqb = L > 1 && set_fs ? set_qb[sg.set] : (L > 1 ? rs->qb : 0);
        const bool apx = fapprox && sg.exactw == 0;
        const bool spk = packed_all || apx;
        const bool accx = L > 1 && sg.sumx != SUMX_NONE;
        CK *const wc = cuts + warp * SNB;
        float4 *const wcb = cbb + (KT::BAND ? warp * SNB : 0);
        uint64_t *const wsw = sw + warp * SNB * L;
        uint32_t *const wcnt = scnt + warp * SNB;
        O *const winv = sinv + warp * SNB;
        const CK lo = sg.lo, hi = sg.hi;
        build_sorted_cuts<KT, true>(lo, hi, nbk, wc, wcb);
        for (int i = lane; i < NB; i += 32) {
            wcnt[i] = 0;
            winv[i] = 0;
#pragma unroll
            for (int l = 0; l < L; ++l) wsw[i * L + l] = 0;
        }
        __syncwarp();
        const BinGuess g = bin_guess(grid_map<KT>(lo, hi, NB));
        uint64_t xacc[L];
#pragma unroll
        for (int l = 0; l < L; ++l) xacc[l] = 0;
        uint64_t xm = ~0ull;
        uint32_t nband = 0;
        const uint64_t a = sg.off, b = a + P[kk + 1] - P[kk];
        for (uint64_t e = a + lane; e < b; e += 32) {
            const K kv = keys[e];
            uint64_t q[L];
            if constexpr (L > 1) {
                const unsigned __int128 qq = fixed_q_bits((double)wts[e], sfs);
                if (accx) {
                    xacc[0] += (uint32_t)qq;
                    xacc[1] += (uint32_t)(qq >> 32);
                    xacc[2] += (uint32_t)(qq >> 64);
                    xacc[3] += (uint32_t)(qq >> 96);
                }
                if (apx) {
                    q[0] = (uint64_t)(qq >> sqb);
#pragma unroll
                    for (int l = 1; l < L; ++l) q[l] = 0;
                } else {
                    q[0] = (uint32_t)qq;
                    q[1] = (uint32_t)(qq >> 32);
                    q[2] = (uint32_t)(qq >> 64);
                    q[3] = (uint32_t)(qq >> 96);
                }
            } else {
                WT::limbs(wts[e], sfs, q);
            }
            if (KT::isnan(kv)) continue;  // not binned; its weight is in the sum
            int bin;
            if constexpr (KT::BAND) {
                bool in_band;
                bin = bin_band<KT>(kv, wc, wcb, NB, g, in_band);
                const bool pend = sg.xstate == X_PENDING && KT::ord(kv) == sg.xkey;
                if (in_band || pend) {
                    // the key's bin is a lower bound; the f64 coordinate decides
                    const uint64_t c = band_code(bs, isrc ? isrc[e] : e, coord);
                    ++nband;
                    if (pend && !KeyF64::lt(c, sg.xcut)) xm = c < xm ? c : xm;
                    bin = bin_band_exact(bin, c, wc, NB);
                }
            } else {
                bin = bin_sorted<KT>(kv, wc, NB, g);
            }
            if (C16) {
                atomicAdd(&wcnt[bin], 1u);
                atomicAdd(&((uint32_t *)wsw)[bin], (uint32_t)q[0]);
            } else if (spk) {
                shared_add_u64(&wsw[bin], (1ull << PACK_SHIFT) | q[0]);
            } else {
                atomicAdd(&wcnt[bin], 1u);
#pragma unroll
                for (int l = 0; l < L; ++l)
                    if (q[l]) shared_add_u64(&wsw[bin * L + l], q[l]);
            }
            const O v = (O)~KT::ord(kv);
            if (v > winv[bin]) atomic_max_ord(&winv[bin], v);
        }
        if constexpr (L > 1) {
            if (accx) {
#pragma unroll
                for (int l = 0; l < L; ++l) {
                    const uint64_t v = warp_sum_u64(xacc[l]);
                    if (lane == 0 && v) atomicAdd((unsigned long long *)&segs_w[s].xq[l], (unsigned long long)v);
                }
            }
        }
        if constexpr (KT::BAND) {
            const uint64_t xw = warp_min_u64(xm);
            const uint64_t nw = warp_sum_u64(nband);
            if (lane == 0) {
                if (xw != ~0ull) atomicMin((unsigned long long *)&segs_w[s].xmin, (unsigned long long)xw);
                if (nw) atomicAdd(bs.count, (unsigned long long)nw);
            }
        }
        __syncwarp();
        for (int i = lane; i < NB; i += 32) {
            uint32_t c;
            uint64_t wl[L];
            if (C16) {
                c = wcnt[i];
                wl[0] = ((uint32_t *)wsw)[i];
            } else if (spk) {
                c = (uint32_t)(wsw[i] >> PACK_SHIFT);
                wl[0] = wsw[i] & PACK_WMASK;
#pragma unroll
                for (int l = 1; l < L; ++l) wl[l] = 0;
            } else {
                c = wcnt[i];
#pragma unroll
                for (int l = 0; l < L; ++l) wl[l] = wsw[i * L + l];
            }
            if (c) {
                const size_t gi = (size_t)s * NB + i;
                atomicAdd(&H.cnt[gi], c);
#pragma unroll
                for (int l = 0; l < L; ++l)
                    if (wl[l]) atomicAdd((unsigned long long *)&H.w[gi * L + l], (unsigned long long)wl[l]);
                atomic_max_ord(&H.inv[gi], winv[i]);
            }
        }
    };
    while (pos < c1) {
        // whole small segments from pos on: one per warp
        uint32_t m = 0;
        if (NB <= SNB) {
            while (m < NWARPS && k + m < nlist) {
                const uint64_t p0 = P[k + m], p1 = P[k + m + 1];
                if ((m == 0 && p0 != pos) || p1 > c1 || p1 - p0 > SMALL_SEG) break;
                ++m;
            }
        }
        if (m > 0) {
            __syncthreads();  // the shared arrays' previous users are done
            if (warp < (int)m) small_seg(k + warp);
            __syncthreads();
            pos = P[k + m];
            k += m;
            cur_s = -1;
            continue;
        }
        const uint32_t s = list[k];
        const uint64_t pe = min(min(c1, P[k + 1]), pos + WINDOW);
        const Seg<KT> &sg = segs[s];
        if (L > 1 && set_fs) {
            fs = set_fs[sg.set];
            qb = set_qb[sg.set];
        }
        // f64 weights: unless this segment's decisions asked for exact bins,
        // a bin holds the count and the sum of floor(q / 2^qb) of its items
        // (q: an item's fixed-point weight, below 2^(126 - ceil(log2 n)), so
        // floor(q / 2^qb) < 2^25 and 2^19 of them fit the packed 44 bits);
        // the decisions bound the exact sums from these.  The level's first
        // pass also sums the segment's exact q (every item, NaN keys too):
        // the segment's weight sum when it is a left child.
        const bool apx = fapprox && sg.exactw == 0;
        const bool packed = packed_all || apx;
        const bool accx = L > 1 && sg.sumx != SUMX_NONE;
        uint64_t xacc[L];
#pragma unroll
        for (int l = 0; l < L; ++l) xacc[l] = 0;
        auto item_q = [&](typename WT::S w, uint64_t *q) {
            if constexpr (L > 1) {
                const unsigned __int128 qq = fixed_q_bits((double)w, fs);
                if (accx) {
                    xacc[0] += (uint32_t)qq;
                    xacc[1] += (uint32_t)(qq >> 32);
                    xacc[2] += (uint32_t)(qq >> 64);
                    xacc[3] += (uint32_t)(qq >> 96);
                }
                if (apx) {
                    q[0] = (uint64_t)(qq >> qb);
#pragma unroll
                    for (int l = 1; l < L; ++l) q[l] = 0;
                } else {
                    q[0] = (uint32_t)qq;
                    q[1] = (uint32_t)(qq >> 32);
                    q[2] = (uint32_t)(qq >> 64);
                    q[3] = (uint32_t)(qq >> 96);
                }
            } else {
                WT::limbs(w, fs, q);
            }
        };
        const uint64_t a = sg.off + (pos - P[k]), b = a + (pe - pos);
        const CK lo = sg.lo, hi = sg.hi;
        __syncthreads();
        if ((int)s != cur_s) build_sorted_cuts<KT>(lo, hi, nbk, cuts, cbb);
        cur_s = (int)s;
        for (int i = threadIdx.x; i < NB; i += BLOCK) {
            scnt[i] = 0;
            sinv[i] = 0;
#pragma unroll
            for (int l = 0; l < L; ++l) sw[i * L + l] = 0;
        }
        __syncthreads();
        const GridMap gm = grid_map<KT>(lo, hi, NB);
        const BinGuess g = bin_guess(gm);
        const FastBin fb = fast_bin<KT>(gm, hi, nbk);
        const EdgeTest<KT> et = edge_test<KT>(lo, hi);
        bool xpend = false;  // band form: a decision waits for an exact minimum
        uint32_t xkey = 0;
        uint64_t xcut = 0;
        uint64_t xm = ~0ull;  // band form: this thread's part of that minimum
        uint32_t nband = 0;   // band form: f64 coordinates this thread read
        uint32_t qn = 0;      // entries in this warp's queue of exact-search items (same in every lane)
        if constexpr (KT::BAND) {
            xpend = sg.xstate == X_PENDING;
            xkey = sg.xkey;
            xcut = sg.xcut;
        }
        // The first and last bins take every key below the first cut and at
        // or above the last one.  Once the interval has narrowed, most keys
        // are there, so their sums stay in registers instead of atomics.
        uint32_t out_c[2] = {0, 0};
        uint64_t out_w[2][L];
        O out_inv[2] = {0, 0};
#pragma unroll
        for (int l = 0; l < L; ++l) out_w[0][l] = out_w[1][l] = 0;
        // adds a key of bin `bin` (weight limbs q, inverted key v)
        auto add_bin = [&](int bin, const uint64_t *q, O v) {
            if (bin == 0 || bin == NB - 1) {
                // constant indices only: keeps the sums in registers
                if (bin == 0) {
                    out_c[0] += 1;
#pragma unroll
                    for (int l = 0; l < L; ++l) out_w[0][l] += q[l];
                    out_inv[0] = v > out_inv[0] ? v : out_inv[0];
                } else {
                    out_c[1] += 1;
#pragma unroll
                    for (int l = 0; l < L; ++l) out_w[1][l] += q[l];
                    out_inv[1] = v > out_inv[1] ? v : out_inv[1];
                }
                return;
            }
            if (C16) {
                atomicAdd(&scnt[bin], 1u);
                atomicAdd(&sw32[bin], (uint32_t)q[0]);
            } else if (packed) {
                shared_add_u64(&sw[bin], (1ull << PACK_SHIFT) | q[0]);
            } else {
                atomicAdd(&scnt[bin], 1u);
#pragma unroll
                for (int l = 0; l < L; ++l)
                    if (q[l]) shared_add_u64(&sw[bin * L + l], q[l]);
            }
            if (v > sinv[bin]) atomic_max_ord(&sinv[bin], v);
        };
        // one queued item: the exact search over the cuts (and in the band
        // form, the f64 coordinate when the key is in a cut's band or is the
        // key a decision waits for)
        auto slow_item = [&](uint64_t e) {
            const K kk = keys[e];
            uint64_t q[L];
            item_q(wts[e], q);
            int bin;
            if constexpr (KT::BAND) {
                bool in_band;
                bin = bin_band<KT>(kk, cuts, cbb, NB, g, in_band);
                const bool pend = xpend && KT::ord(kk) == xkey;
                if (in_band || pend) {
                    const uint64_t c = band_code(bs, isrc ? isrc[e] : e, coord);
                    ++nband;
                    if (pend && !KeyF64::lt(c, xcut)) xm = c < xm ? c : xm;
                    bin = bin_band_exact(bin, c, cuts, NB);
                }
            } else {
                bin = bin_sorted<KT>(kk, cuts, NB, g);
            }
            add_bin(bin, q, (O)~KT::ord(kk));
        };
        // Passes after the first of a level search a narrowed interval: most
        // keys then fall outside it, into the first and last bins, whose sums
        // stay in registers (atomics on two words would serialise).  A
        // level's first pass spans the whole interval and adds those two
        // bins like any other.
        const bool ER = sg.steps != 0;    // edge bins in registers (uniform)
        const bool PD = KT::BAND && xpend;  // a decision waits for a key's exact minimum (uniform)
        {
            for (uint64_t base = a; base < b; base += (uint64_t)BLOCK * HI) {
                // items of this iteration: 32-bit offsets from base below lim
                const uint32_t lim = (uint32_t)min((uint64_t)BLOCK * HI, b - base);
                const K *kb = keys + base;
                const typename WT::S *wb = wts + base;
                K kv[HI];
                typename WT::S wv[HI];
#pragma unroll
                for (int i = 0; i < HI; ++i) {
                    const uint32_t li = i * BLOCK + threadIdx.x;
                    if (li < lim) {
                        kv[i] = kb[li];
                        wv[i] = wb[li];
                    }
                }
                // Bins from the grid position (fast_bin); the few items whose
                // position is too close to a bin edge take the exact search in
                // place.  Band-form items in a cut's band (and items whose key
                // a decision waits for) are only marked here and resolved from
                // the warp's queue, 32 at a time, so that their dependent f64
                // loads overlap.
                uint32_t slow = 0;
                int bins[HI];     // bin of an item to add by atomics (-1: none)
                uint32_t qlo[HI];  // f64 weights in packed bins: the truncated fixed-point weight
#pragma unroll
                for (int i = 0; i < HI; ++i) {
                    const uint32_t li = i * BLOCK + threadIdx.x;
                    const bool valid = li < lim;
                    const bool nan = KT::isnan(kv[i]);
                    if (L > 1 && accx && valid && nan) {
                        uint64_t q[L];
                        item_q(wv[i], q);  // a NaN key is not binned; its weight is in the sum
                    }
                    const bool binned = valid && !nan;
                    const bool below = et.below(kv[i]), above = !below && et.above(kv[i]);
                    const float f = fmaf(KT::approx(kv[i]) - fb.l, fb.sc, fb.s);
                    const int bg = __float2int_rz(f);
                    const float fr = f - (float)bg;
                    const bool fast = (uint32_t)bg < (uint32_t)NB && fr > fb.m && fr < fb.m1;
                    int bin = below ? 0 : (above ? NB - 1 : bg);
                    bool sl = false;  // queued for its f64 coordinate (band form)
                    if (binned && !below && !above && !fast) {
                        // rare: the exact search over the cuts, in place (the
                        // neighbouring cuts, else a binary search)
                        if constexpr (KT::BAND) {
                            bool in_band;
                            bin = bin_band<KT>(kv[i], cuts, cbb, NB, g, in_band);
                            sl = in_band;
                        } else if (fb.m < 1.0f) {
                            // the grid position is within m/2 of the key's
                            // and every cut within m/2 of its grid point
                            // (m < 1/4): the bin is bg - 1, bg or bg + 1
                            const int b0 = min(max(bg, 0), NB - 1);
                            bin = b0;
                            if (b0 > 0 && KT::lt(kv[i], cuts[b0 - 1]))
                                bin = b0 - 1;
                            else if (b0 < NB - 1 && !KT::lt(kv[i], cuts[b0]))
                                bin = b0 + 1;
                        } else {
                            bin = bin_sorted<KT>(kv[i], cuts, NB, BinGuess{0.f, 0.f, 0.f, 0});
                        }
                    }
                    if (PD) sl = sl || (binned && KT::ord(kv[i]) == xkey);
                    slow |= (uint32_t)sl << i;
                    const bool take = binned && !sl;
                    const bool edge = ER && take && (bin == 0 || bin == NB - 1);
                    bins[i] = take && !edge ? bin : -1;
                    qlo[i] = 0;
                    if constexpr (L == 1) {
                        if (ER) {
                            uint64_t q[1];
                            WT::limbs(wv[i], fs, q);
                            const O v = (O)~KT::ord(kv[i]);
                            const bool e0 = edge && bin == 0, e1 = edge && bin != 0;
                            out_c[0] += e0 ? 1u : 0u;
                            out_w[0][0] += e0 ? q[0] : 0ull;
                            out_inv[0] = e0 && v > out_inv[0] ? v : out_inv[0];
                            out_c[1] += e1 ? 1u : 0u;
                            out_w[1][0] += e1 ? q[0] : 0ull;
                            out_inv[1] = e1 && v > out_inv[1] ? v : out_inv[1];
                        }
                    } else if (take) {
                        uint64_t q[L];
                        item_q(wv[i], q);
                        qlo[i] = (uint32_t)q[0];
                        if (edge) add_bin(bin, q, (O)~KT::ord(kv[i]));
                    }
                }
                // the bins' current minima first (independent loads in flight
                // together), then the adds; a minimum read before another
                // thread lowered it only costs an extra atomic
                O old[HI];
#pragma unroll
                for (int i = 0; i < HI; ++i) old[i] = bins[i] >= 0 ? sinv[bins[i]] : (O)~(O)0;
#pragma unroll
                for (int i = 0; i < HI; ++i) {
                    const int bin = bins[i];
                    if (bin < 0) continue;
                    if (C16) {
                        atomicAdd(&scnt[bin], 1u);
                        atomicAdd(&sw32[bin], (uint32_t)wv[i]);
                    } else if (packed) {
                        uint64_t w0;
                        if constexpr (L == 1) {
                            uint64_t q[1];
                            WT::limbs(wv[i], fs, q);
                            w0 = q[0];
                        } else {
                            w0 = qlo[i];
                        }
                        shared_add_u64(&sw[bin], (1ull << PACK_SHIFT) | w0);
                    } else {
                        uint64_t q[L];
                        if constexpr (L == 1) {
                            WT::limbs(wv[i], fs, q);
                        } else {
                            const unsigned __int128 qq = fixed_q_bits((double)wv[i], fs);
                            q[0] = (uint32_t)qq;
                            q[1] = (uint32_t)(qq >> 32);
                            q[2] = (uint32_t)(qq >> 64);
                            q[3] = (uint32_t)(qq >> 96);
                        }
                        atomicAdd(&scnt[bin], 1u);
#pragma unroll
                        for (int l = 0; l < L; ++l)
                            if (q[l]) shared_add_u64(&sw[bin * L + l], q[l]);
                    }
                    const O v = (O)~KT::ord(kv[i]);
                    if (v > old[i]) atomic_max_ord(&sinv[bin], v);
                }
                // queue the marked items; every 32 of them are searched, one
                // per lane, and on the last iteration the queue's rest (a
                // single call site keeps the search's registers out of the
                // loop above)
                const bool fin = base + (uint64_t)BLOCK * HI >= b;
                // the item slots in which some lane marked an item (usually
                // one or two); then a last round that flushes the rest
                const uint32_t anyb = KT::BAND || PD ? __reduce_or_sync(0xffffffffu, slow) : 0u;
                if (anyb != 0 || (fin && qn)) {
                    uint32_t mm = anyb;
#pragma unroll 1
                    for (;;) {
                        const bool last = mm == 0;
                        const int i = last ? HI : __ffs(mm) - 1;
                        mm &= mm - 1;
                        const bool bit = !last && ((slow >> i) & 1u);
                        const uint32_t m = __ballot_sync(0xffffffffu, bit);
                        if (bit)
                            s_q[warp][qn + __popc(m & ((1u << lane) - 1))] =
                                (uint32_t)(base - a) + i * BLOCK + threadIdx.x;
                        qn += __popc(m);
                        if (qn >= 32 || (last && fin && qn)) {
                            const uint32_t cnt = qn < 32 ? qn : 32u;
                            __syncwarp();
                            if (lane < cnt) slow_item(a + s_q[warp][lane]);
                            // keep the rest (fewer than 32) at the front
                            qn -= cnt;
                            const uint32_t v = lane < qn ? s_q[warp][32 + lane] : 0u;
                            __syncwarp();
                            if (lane < qn) s_q[warp][lane] = v;
                        }
                        __syncwarp();
                        if (last) break;
                    }
                }
            }
        }
        if constexpr (L > 1) {
            if (accx) {
#pragma unroll
                for (int l = 0; l < L; ++l) {
                    const uint64_t v = warp_sum_u64(xacc[l]);
                    if ((threadIdx.x & 31) == 0 && v) atomicAdd((unsigned long long *)&segs_w[s].xq[l], (unsigned long long)v);
                }
            }
        }
        if constexpr (KT::BAND) {
            // one global update per warp and piece: a plane of equal
            // coordinates can put millions of items in one band
            const uint64_t xw = warp_min_u64(xm);
            const uint64_t nw = warp_sum_u64(nband);
            if ((threadIdx.x & 31) == 0) {
                if (xw != ~0ull) atomicMin((unsigned long long *)&segs_w[s].xmin, (unsigned long long)xw);
                if (nw) atomicAdd(bs.count, (unsigned long long)nw);
            }
        }
        // fold the out-of-interval sums into the edge bins (one lane per warp)
#pragma unroll
        for (int side = 0; side < 2; ++side) {
            const uint64_t c = warp_sum_u64(out_c[side]);
            uint64_t wsum[L];
#pragma unroll
            for (int l = 0; l < L; ++l) wsum[l] = warp_sum_u64(out_w[side][l]);
            const O inv = (O)~warp_min_ord<O>((O)~out_inv[side]);
            if ((threadIdx.x & 31) == 0 && c) {
                const int bin = side == 0 ? 0 : NB - 1;
                if (C16) {
                    atomicAdd(&scnt[bin], (uint32_t)c);
                    atomicAdd(&sw32[bin], (uint32_t)wsum[0]);
                } else if (packed) {
                    shared_add_u64(&sw[bin], (c << PACK_SHIFT) | wsum[0]);
                } else {
                    atomicAdd(&scnt[bin], (uint32_t)c);
#pragma unroll
                    for (int l = 0; l < L; ++l)
                        if (wsum[l]) shared_add_u64(&sw[bin * L + l], wsum[l]);
                }
                atomic_max_ord(&sinv[bin], inv);
            }
        }
        __syncthreads();
        for (int i = threadIdx.x; i < NB; i += BLOCK) {
            uint32_t c;
            uint64_t wl[L];
            if (C16) {
                c = scnt[i];
                wl[0] = sw32[i];
            } else if (packed) {
                c = (uint32_t)(sw[i] >> PACK_SHIFT);
                wl[0] = sw[i] & PACK_WMASK;
#pragma unroll
                for (int l = 1; l < L; ++l) wl[l] = 0;
            } else {
                c = scnt[i];
#pragma unroll
                for (int l = 0; l < L; ++l) wl[l] = sw[i * L + l];
            }
            if (c) {
                const size_t gi = (size_t)s * NB + i;
                atomicAdd(&H.cnt[gi], c);
#pragma unroll
                for (int l = 0; l < L; ++l)
                    if (wl[l]) atomicAdd((unsigned long long *)&H.w[gi * L + l], (unsigned long long)wl[l]);
                atomic_max_ord(&H.inv[gi], sinv[i]);
            }
        }
        pos = pe;
        if (pos == P[k + 1]) ++k;
    }
}

// Builds the next level's segments from the finished splits: left child
// (heap 2h+1, sum = weight_left, bbox max[coord] = split_pos) and right child
// (2h+2, sum - weight_left, bbox min[coord] = split_pos), empty children
// dropped (recursive_bisection.rs:586-588, 606-641).  Run by one CTA (the
// k_children kernel, or the last CTA of a decide launch) or, for wide
// levels, by a grid in three phases.  Also records the smallest heap id
// among the children (the id offset, :698-702).
enum : int { CHILD_ALL = 0, CHILD_COUNT = 1, CHILD_SCAN = 2, CHILD_WRITE = 3 };
constexpr uint32_t CHILD_GRID_MIN = 2048;  // segments from which a level uses the grid form

template <class KT, class WT>
__device__ __forceinline__ void children_body(Seg<KT> *segs, uint32_t S, int coord, int D, int write,
                                              uint32_t level, Seg<KT> *next, uint32_t *next_list, uint64_t *next_P,
                                              Trav<KT> *trav, RunScalars *rs, const SetTab &sets, int phase,
                                              uint64_t *blk, const uint64_t *S_ptr, uint64_t *lvl) {
    typedef typename KT::T K;
    __shared__ uint64_t sh[33];
    // launched right after a speculative pass: nothing to do while a segment
    // of the level is still searching (the host runs more passes, then this)
    if (cta_halted(rs) || rs->nactive != 0) return;
    if (S_ptr) S = (uint32_t)*S_ptr;  // the level's segment count from the device
    const bool multi = sets.count > 1;
    uint64_t outc = 0, outv = 0;
    uint64_t hmin = ~0ull;
    const int nc = (coord + 1) % D;
    // CHILD_ALL: one CTA walks every segment.  Levels with many segments use
    // a grid of CTAs, one per 1024 segments, in three launches:
    // CHILD_COUNT (each CTA's children and items into blk), CHILD_SCAN (one
    // CTA: blk becomes exclusive offsets) and CHILD_WRITE.
    uint32_t first = 0, stop = S;
    if (phase == CHILD_COUNT || phase == CHILD_WRITE) {
        first = blockIdx.x * blockDim.x;
        stop = min(S, first + blockDim.x);
        if (phase == CHILD_WRITE) {
            outc = blk[2 * blockIdx.x];
            outv = blk[2 * blockIdx.x + 1];
        }
    }
    if (phase == CHILD_SCAN) {
        const uint32_t nb = (S + 1023) / 1024;
        for (uint32_t b0 = 0; b0 < nb; b0 += blockDim.x) {
            const uint32_t b = b0 + threadIdx.x;
            const uint64_t c = b < nb ? blk[2 * b] : 0, v = b < nb ? blk[2 * b + 1] : 0;
            uint64_t tc, tv;
            const uint64_t ci = block_exscan_u64(c, sh, tc);
            const uint64_t vi = block_exscan_u64(v, sh, tv);
            if (b < nb) {
                blk[2 * b] = outc + ci;
                blk[2 * b + 1] = outv + vi;
            }
            outc += tc;
            outv += tv;
        }
        if (threadIdx.x == 0) {
            rs->nsegs_next = outc;
            rs->items_next = outv;
            if (lvl) {
                lvl[2 * (level + 1)] = outc;  // the next level's counts
                lvl[2 * (level + 1) + 1] = outv;
            }
            if (write) next_P[outc] = outv;
        }
        return;
    }
    for (uint32_t base = first; base < stop; base += blockDim.x) {
        const uint32_t s = base + threadIdx.x;
        Seg<KT> sg;
        uint32_t nl = 0, nr = 0;
        bool leaves = !write;  // the children are parts: no segments for them
        if (s < S) {
            sg = segs[s];
            nl = sg.nleft;
            if (nl > sg.n) {  // inconsistent split: report, and keep sizes in range
                atomicOr(&rs->err, ERR_COUNT_MISMATCH);
                nl = sg.n;
            }
            nr = sg.n - nl;
            if (multi && sets.iters[sg.set] <= level + 1) leaves = true;  // the set's last level
        }
        uint64_t tc, tv;
        const uint64_t ci = block_exscan_u64(leaves ? 0 : (nl > 0) + (nr > 0), sh, tc);
        const uint64_t vi = block_exscan_u64(leaves ? 0 : (uint64_t)nl + nr, sh, tv);
        if (phase == CHILD_COUNT) {
            if (threadIdx.x == 0) {
                blk[2 * blockIdx.x] = tc;
                blk[2 * blockIdx.x + 1] = tv;
            }
            return;
        }
        if (s < stop) {
            const uint64_t hl = 2 * sg.heap + 1, hr = 2 * sg.heap + 2;
            if (leaves) {
                uint64_t h = ~0ull;
                if (nl > 0) h = hl;
                if (nr > 0) h = hr < h ? hr : h;
                if (multi)
                    atomicMin((unsigned long long *)&sets.minheap[sg.set], (unsigned long long)h);
                else
                    hmin = h < hmin ? h : hmin;
            }
            if (trav) {
                Trav<KT> t;
                t.pivot = sg.pivot;
                t.flags = (sg.state == SEG_ALLLEFT ? TRAV_ALLLEFT : 0u) | (nl > 0 ? TRAV_HAS_LEFT : 0u);
                t.next = leaves ? sg.heap : outc + ci;
                t.blo = t.bhi = 0.f;
                if constexpr (KT::BAND) {
                    const CutBounds cb = band_bounds(sg.pivot);
                    t.blo = cb.lo;
                    t.bhi = cb.hi;
                }
                trav[s] = t;
            }
            if (!leaves) {
                segs[s].child = (uint32_t)(outc + ci);
                uint64_t c = outc + ci;
                const typename WT::V sum = WT::from_bits(sg.sum), wl = WT::from_bits(sg.wl);
                for (int side = 0; side < 2; ++side) {
                    const uint32_t cn = side == 0 ? nl : nr;
                    if (!cn) continue;
                    Seg<KT> ch;
                    ch.off = side == 0 ? sg.off : sg.off + nl;
                    ch.voff = outv + vi + (side == 0 ? 0 : nl);
                    ch.heap = side == 0 ? hl : hr;
                    if (sg.wlx) {
                        ch.sum = WT::bits(side == 0 ? wl : WT::sub(sum, wl));
                        ch.sumx = SUMX_NONE;
                    } else {
                        // weight_left known only within bounds: the next
                        // level's first pass sums the left child's items
                        ch.sum = side == 0 ? 0 : sg.sum;
                        ch.sumx = side == 0 ? SUMX_OWN : (nl > 0 ? SUMX_RIGHT : SUMX_NONE);
                    }
                    ch.exactw = 0;
                    ch.wlx = 0;
                    ch.pad2 = 0;
#pragma unroll
                    for (int l = 0; l < 4; ++l) ch.xq[l] = 0;
                    ch.prev = ~0ull;
                    ch.wl = 0;
                    ch.n = cn;
                    ch.nleft = 0;
                    ch.state = SEG_ACTIVE;
                    ch.steps = 0;
                    ch.child = 0;
                    ch.xstate = 0;
                    ch.xkey = 0;
                    ch.set = sg.set;
                    ch.xcut = 0;
                    ch.xmin = ~0ull;
                    for (int d = 0; d < 3; ++d) {
                        ch.bmin[d] = sg.bmin[d];
                        ch.bmax[d] = sg.bmax[d];
                    }
                    if (side == 0)
                        ch.bmax[coord] = sg.split_pos;
                    else
                        ch.bmin[coord] = sg.split_pos;
                    ch.lo = ch.bmin[nc];
                    ch.hi = ch.bmax[nc];
                    ch.pivot = 0;
                    ch.split_pos = 0;
                    next[c] = ch;
                    next_list[c] = (uint32_t)c;
                    next_P[c] = ch.voff;
                    ++c;
                }
            }
        }
        outc += tc;
        outv += tv;
    }
    hmin = warp_min_u64(hmin);
    if (!multi && (threadIdx.x & 31) == 0 && hmin != ~0ull)
        atomicMin((unsigned long long *)&rs->min_heap, (unsigned long long)hmin);
    if (phase == CHILD_ALL && threadIdx.x == 0) {
        rs->nsegs_next = outc;
        rs->items_next = outv;
        if (lvl) {
            lvl[2 * (level + 1)] = outc;  // the next level's counts
            lvl[2 * (level + 1) + 1] = outv;
        }
        if (write) next_P[outc] = outv;
    }
}

template <class KT, class WT>
__global__ void __launch_bounds__(1024) k_children(Seg<KT> *segs, uint32_t S, int coord, int D, int write,
                                                   uint32_t level, Seg<KT> *next, uint32_t *next_list,
                                                   uint64_t *next_P, Trav<KT> *trav, RunScalars *rs, SetTab sets,
                                                   int phase, uint64_t *blk, const uint64_t *S_ptr, uint64_t *lvl) {
    children_body<KT, WT>(segs, S, coord, D, write, level, next, next_list, next_P, trav, rs, sets, phase, blk,
                          S_ptr, lvl);
}

// The next level's segments built by the last CTA of a decide launch (levels
// below CHILD_GRID_MIN segments, after the speculative pass).
template <class KT>
struct ChildArgs {
    int on;
    uint32_t stall_level;  // nonzero: halt the queued run with this value if splits still search
    const uint64_t *S_ptr;  // the level's segment count on the device (NULL: S)
    uint64_t *lvl;          // per-level segment and item counts (the children write the next level's)
    uint32_t S;
    int coord, D, write;
    uint32_t level;
    Seg<KT> *next;
    uint32_t *next_list;
    uint64_t *next_P;
    Trav<KT> *trav;
    SetTab sets;
};

// Compacts the listed segments still searching into list2 with the exclusive
// prefix P2 of their sizes.  One CTA.
template <class KT>
__device__ __forceinline__ void scan_list_block(const Seg<KT> *__restrict__ segs, const uint32_t *__restrict__ list,
                                                const uint32_t *__restrict__ flags, uint32_t nlist, uint32_t *list2,
                                                uint64_t *P2, RunScalars *rs) {
    __shared__ uint64_t sh[33];
    uint64_t outc = 0, run = 0;
    for (uint32_t base = 0; base < nlist; base += blockDim.x) {
        const uint32_t k = base + threadIdx.x;
        const bool keep = k < nlist && flags[k];
        const uint32_t s = keep ? list[k] : 0;
        const uint64_t sz = keep ? segs[s].n : 0;
        uint64_t tc, tp;
        const uint64_t ci = block_exscan_u64(keep ? 1 : 0, sh, tc);
        const uint64_t pi = block_exscan_u64(sz, sh, tp);
        if (keep) {
            list2[outc + ci] = s;
            P2[outc + ci] = run + pi;
        }
        outc += tc;
        run += tp;
    }
    if (threadIdx.x == 0) {
        P2[outc] = run;
        rs->nactive = outc;
        rs->total_active = run;
        rs->pass_points += run;  // read by the pass that follows
    }
}

// ---------------------------------------------------------------------------
// k_decide: replays coupe's split loop (recursive_bisection.rs:470-572) for
// up to nbk steps per segment from its bins.  One warp per listed segment;
// every lane computes the same decisions.  The FP64 pipe bounds a decision
// step on this GPU, so the two f64 tests of a step are first settled in f32
// or integer arithmetic with a proven error bound (ImbalanceTest, band_far);
// only values within that bound of the threshold take the f64 expressions.
// ---------------------------------------------------------------------------

// coupe's imbalance test |(w - ideal) / ideal| <= tol, evaluated in f64
// (recursive_bisection.rs:547-551).  With f32 values wf = RN32(w),
// idf = RN32(ideal) (normal) and rinv = RN32(1 / |idf|), the f32 quotient
// q = RN32(|RN32(wf - idf)| rinv) lies within 2^-22 ((|w| + |ideal|) /
// |ideal| + q) of |w - ideal| / |ideal| (three roundings of 2^-24 on each
// term, the conversions of w and ideal included), and coupe's f64 quotient
// within 2^-51 of the same; so e = 2^-21 ((|wf| + |idf|) rinv + q) bounds
// their distance with room for the rounding of e and of q +- e.  q + e at or
// below RD32(tol) proves the test true, q - e above RU32(tol) proves it
// false; anything else (and every non-finite or extreme case) takes the
// f64 division.
struct ImbalanceTest {
    double ideal, tol;
    float idf, rinv, tlo, thi;
    bool fast;
};
__device__ __forceinline__ ImbalanceTest imbalance_test(double ideal, double tol) {
    ImbalanceTest t;
    t.ideal = ideal;
    t.tol = tol;
    t.idf = (float)ideal;
    const float a = fabsf(t.idf);
    t.rinv = 1.0f / a;
    t.tlo = __double2float_rd(tol);
    t.thi = __double2float_ru(tol);
    t.fast = a >= 0x1p-100f && a <= 0x1p100f;  // false for NaN
    return t;
}
template <class WT>
__device__ __forceinline__ bool imbalance_within(const ImbalanceTest &t, typename WT::V w) {
    if (t.fast) {
        const float wf = (float)w;
        const float q = fabsf(wf - t.idf) * t.rinv;
        const float e = 0x1p-21f * ((fabsf(wf) + fabsf(t.idf)) * t.rinv + q);
        const float up = q + e, dn = q - e;
        if (up <= t.tlo && up <= 0x1p127f) return true;  // (inf and NaN fail)
        if (dn > t.thi) return false;
    }
    return fabs((WT::f64(w) - t.ideal) / t.ideal) <= t.tol;
}

// Band form: true when hi <= t + d certainly fails for every distance d the
// f64 step could compute from the smallest right key k (its items' x lie in
// [t, max(next32(k), RU32(t))] =: [t, M]).  t + RN(x - t) rounds to at most
// M + 2^-51 A with A = max(|M|, |RD32(t)|) >= |x|, |t|, so RD32(hi) above
// RU32(M + 2^-50 A) proves hi > t + d.  Integer and f32 instructions only.
__device__ __forceinline__ bool band_far(float k, uint64_t t, uint64_t hi) {
    const CutBounds tb = band_bounds(t), hb = band_bounds(hi);
    const float nk = f32_step(k, 1);
    const float M = fmaxf(nk, tb.hi);
    const float A = fmaxf(fabsf(M), fabsf(tb.lo));
    if (!isfinite(k) || !isfinite(nk) || !isfinite(tb.lo) || !isfinite(M) || !isfinite(A)) return false;
    return hb.lo > __fadd_ru(M, __fmul_ru(A, 0x1p-50f));
}
template <class KT, class WT>
__device__ __forceinline__ void decide_one(Seg<KT> *segs, const uint32_t *__restrict__ list, const uint32_t k,
                                           Hist<KT, WT> H, int nbk, double tol, uint32_t *flags, RunScalars *rs,
                                           const int32_t *__restrict__ set_fs, const int32_t *__restrict__ set_qb) {
    typedef typename KT::C K;  // cuts and interval bounds
    typedef typename KT::Ord O;
    typedef typename WT::V V;
    constexpr int L = WT::LIMBS;
    // band form: empty bins hold no key at all (not +inf, a possible key)
    constexpr O NONE = KT::BAND ? (O)~(O)0 : KT::ORD_INF;
    const int lane = threadIdx.x & 31;
    const uint32_t s = list[k];
    Seg<KT> sg = segs[s];
    const int NB = 1 << nbk;
    // Lane l owns the block of BS consecutive bins starting at l*BS.  Steps
    // whose halves span whole blocks use the block totals; once a half is
    // narrower than a block, the one block left is spread over the lanes.
    const int BS = NB >= 32 ? NB / 32 : 1;
    const int fs = L > 1 ? (set_fs ? set_fs[sg.set] : rs->fscale) : 0;
    const int qb = L > 1 ? (set_qb ? set_qb[sg.set] : rs->qb) : 0;
    // f64 weights: bins of truncated weights (k_hist) unless exact ones were asked for
    const bool apx = L > 1 && rs->fapprox != 0 && sg.exactw == 0;
    const size_t g0 = (size_t)s * NB;
    auto load_bin = [&](int b, uint64_t &c, uint64_t *w, O &m) {
        const size_t g = g0 + b;
        c = H.cnt[g];
#pragma unroll
        for (int l = 0; l < L; ++l) w[l] = H.w[g * L + l];
        const O o = (O)~H.inv[g];
        m = KT::BAND ? o : (o > KT::ORD_INF ? KT::ORD_INF : o);
    };
    uint64_t Tc = 0, Tw[L];
    O Tm = NONE;
#pragma unroll
    for (int l = 0; l < L; ++l) Tw[l] = 0;
    if (lane * BS < NB) {
        int j = 0;
        {
            // eight bins per step in 16-byte loads, all in flight together
            // (a lane's block of bins is contiguous and 16-byte aligned)
            constexpr int MV = 8 * sizeof(O) / 16;  // 16-byte vectors of minima per step
            for (; j + 8 <= BS; j += 8) {
                const size_t g = g0 + lane * BS + j;
                uint4 c4[2], m4[MV];
                ulonglong2 w2[4 * L];
#pragma unroll
                for (int q = 0; q < 2; ++q) c4[q] = *(const uint4 *)&H.cnt[g + 4 * q];
#pragma unroll
                for (int q = 0; q < MV; ++q) m4[q] = *(const uint4 *)((const char *)&H.inv[g] + 16 * q);
#pragma unroll
                for (int q = 0; q < 4 * L; ++q) w2[q] = *(const ulonglong2 *)&H.w[g * L + 2 * q];
#pragma unroll
                for (int q = 0; q < 2; ++q) Tc += (uint64_t)c4[q].x + c4[q].y + c4[q].z + c4[q].w;
                const O *mo = (const O *)m4;
#pragma unroll
                for (int r = 0; r < 8; ++r) {
                    O o = (O)~mo[r];  // empty bins hold 0: ~0
                    if (!KT::BAND) o = o > KT::ORD_INF ? KT::ORD_INF : o;
                    Tm = o < Tm ? o : Tm;
                }
#pragma unroll
                for (int q = 0; q < 4 * L; ++q) {
                    // element 2q + h of the step is limb (2q + h) % L of a bin
                    Tw[(2 * q) % L] += w2[q].x;
                    Tw[(2 * q + 1) % L] += w2[q].y;
                }
            }
        }
        // four bins per step, their loads in flight together
        for (; j + 4 <= BS; j += 4) {
            uint64_t c[4], w[4][L];
            O m[4];
#pragma unroll
            for (int i = 0; i < 4; ++i) load_bin(lane * BS + j + i, c[i], w[i], m[i]);
#pragma unroll
            for (int i = 0; i < 4; ++i) {
                Tc += c[i];
#pragma unroll
                for (int l = 0; l < L; ++l) Tw[l] += w[i][l];
                Tm = m[i] < Tm ? m[i] : Tm;
            }
        }
        for (; j < BS; ++j) {
            uint64_t c, w[L];
            O m;
            load_bin(lane * BS + j, c, w, m);
            Tc += c;
#pragma unroll
            for (int l = 0; l < L; ++l) Tw[l] += w[l];
            Tm = m < Tm ? m : Tm;
        }
    }
    // Each step needs only the bins below the cut (count and weight left:
    // a prefix sum) and the smallest key at or above it (a suffix minimum),
    // so both are scanned once over the lane blocks and each step reads them
    // with one shuffle.
    uint64_t Ic = warp_incl_scan_u64(Tc), Iw[L];
#pragma unroll
    for (int l = 0; l < L; ++l) Iw[l] = warp_incl_scan_u64(Tw[l]);
    const O Sm = warp_suffix_min<O>(Tm);
    // Every binned key belongs to this segment.  More counts than items means
    // corrupt bins: no split is taken from them (the host stops the run before
    // any later kernel could use sizes derived from them).
    if (__shfl_sync(0xffffffffu, Ic, 31) > sg.n) {
        if (lane == 0) {
            flags[k] = 0;
            if (atomicOr(&rs->err, ERR_COUNT_MISMATCH) == 0) {
                rs->diag[0] = s;
                rs->diag[1] = sg.n;
            }
        }
        return;
    }
    // Once half of the interval is narrower than a block, the one block left
    // (fine_base ...) is spread over the lanes, one bin each, and scanned the
    // same way, on top of the prefix below the block and the minimum above it.
    bool fine = false;
    int fine_base = 0;
    uint64_t IFc = 0, IFw[L], Bc = 0, Bw[L];
    O FSm = NONE, Am = NONE;
#pragma unroll
    for (int l = 0; l < L; ++l) IFw[l] = Bw[l] = 0;

    // the level's first decisions settle a child's sum from exact sums of
    // the first pass: coupe's weight_left for a left child, sum - weight_left
    // for a right one (recursive_bisection.rs:606-641)
    V sum = WT::from_bits(sg.sum);
    if constexpr (L > 1) {
        if (sg.sumx == SUMX_OWN)
            sum = WT::value(sg.xq, fs);
        else if (sg.sumx == SUMX_RIGHT)
            sum = WT::sub(sum, WT::value(segs[s - 1].xq, fs));
    }
    const double ideal = WT::f64(sum) / 2.0;
    const ImbalanceTest imt = imbalance_test(ideal, tol);
    K lo = sg.lo, hi = sg.hi;
    uint64_t prev = sg.prev;
    int lo_b = 0, hi_b = NB;
    bool flag_exact = false;  // band form: a test needs an exact minimum first
    bool flag_exactw = false;  // f64 weights: a test needs exact bins first
    K xcut = 0;
    O xkey = 0;
    uint32_t state = SEG_ACTIVE;
    uint32_t steps = 0;
    K pivot = 0, split_pos = 0;
    V wl_out = 0;
    bool wl_exact = true;
    uint64_t nleft = 0;
    for (int step = 0; step < nbk; ++step) {
        const int mid_b = (lo_b + hi_b) >> 1;
        if (!fine && mid_b - lo_b < BS) {
            fine = true;
            fine_base = lo_b - lo_b % BS;  // the block holding [lo_b, hi_b)
            const int f = fine_base / BS;
            uint64_t c = 0, w[L];
            O m = NONE;
#pragma unroll
            for (int l = 0; l < L; ++l) w[l] = 0;
            if (lane < BS) load_bin(fine_base + lane, c, w, m);
            IFc = warp_incl_scan_u64(c);
#pragma unroll
            for (int l = 0; l < L; ++l) IFw[l] = warp_incl_scan_u64(w[l]);
            FSm = warp_suffix_min<O>(m);
            // prefix below block f, minimum above it
            const uint64_t pc = __shfl_sync(0xffffffffu, Ic, f > 0 ? f - 1 : 0);
            Bc = f > 0 ? pc : 0;
#pragma unroll
            for (int l = 0; l < L; ++l) {
                const uint64_t pw = __shfl_sync(0xffffffffu, Iw[l], f > 0 ? f - 1 : 0);
                Bw[l] = f > 0 ? pw : 0;
            }
            const O am = __shfl_sync(0xffffffffu, Sm, f + 1 < 32 ? f + 1 : 31);
            Am = f + 1 < 32 ? am : NONE;
        }
        // count and weight of the bins below mid_b, smallest key at or above it
        uint64_t count, wacc[L];
        O kminO;
        if (!fine) {
            const int ml = mid_b / BS;  // a block boundary
            const uint64_t pc = __shfl_sync(0xffffffffu, Ic, ml > 0 ? ml - 1 : 0);
            count = ml > 0 ? pc : 0;
#pragma unroll
            for (int l = 0; l < L; ++l) {
                const uint64_t pw = __shfl_sync(0xffffffffu, Iw[l], ml > 0 ? ml - 1 : 0);
                wacc[l] = ml > 0 ? pw : 0;
            }
            const O sm = __shfl_sync(0xffffffffu, Sm, ml < 32 ? ml : 31);
            kminO = ml < 32 ? sm : NONE;
        } else {
            const int j = mid_b - fine_base;  // < BS
            const uint64_t pc = __shfl_sync(0xffffffffu, IFc, j > 0 ? j - 1 : 0);
            count = Bc + (j > 0 ? pc : 0);
#pragma unroll
            for (int l = 0; l < L; ++l) {
                const uint64_t pw = __shfl_sync(0xffffffffu, IFw[l], j > 0 ? j - 1 : 0);
                wacc[l] = Bw[l] + (j > 0 ? pw : 0);
            }
            const O sm = __shfl_sync(0xffffffffu, FSm, j);
            kminO = sm < Am ? sm : Am;
        }
        const K t = KT::cmid(lo, hi);
        const typename KT::A tv = KT::cval(t), hv = KT::cval(hi);
        // distance of the nearest item on the right (recursive_bisection.rs:487):
        // exact, or in the band form bounds [dl, dh] of it
        typename KT::A dl, dh;
        bool far = false;  // band form: hi <= t + d is certainly false (band_far)
        if constexpr (KT::BAND) {
            if (kminO == NONE) {
                dl = dh = KT::inf();
            } else if (band_far(KT::unord(kminO), t, hi)) {
                far = true;
                dl = dh = 0.0;  // finite; the near tests below are false
            } else {
                double xl, xh;
                band_interval(KT::unord(kminO), xl, xh);
                if (xl < tv) xl = tv;  // items right of t are >= t (the bins are exact)
                if (xh < xl) xh = xl;
                if (sg.xstate == X_PENDING && sg.xcut == t && sg.xkey == (uint32_t)kminO && sg.xmin != ~0ull)
                    xl = xh = KeyF64::val(sg.xmin);  // found by the pass that just ran
                dl = xl - tv;
                dh = xh - tv;
            }
        } else {
            dl = dh = KT::cval(KT::unord(kminO)) - tv;
        }
        ++steps;
        if (KT::BAND && !(dl < KT::inf()) != !(dh < KT::inf())) {
            flag_exact = true;  // is there an item right of t at all? (a +inf key)
        } else if (!(dl < KT::inf())) {
            // no item on the right of t (recursive_bisection.rs:522-545)
            if (prev == count) {
                state = SEG_ALLLEFT;
                split_pos = hi;
                wl_out = sum;
                nleft = sg.n;
                break;
            }
            hi = t;
            prev = count;
            hi_b = mid_b;
            continue;
        }
        if (flag_exact) {
            --steps;  // this step is replayed once the minimum is exact
            xcut = t;
            xkey = kminO;
            if (sg.xstate == X_PENDING && sg.xcut == t && sg.xkey == (uint32_t)kminO && lane == 0)
                atomicOr(&rs->err, ERR_COUNT_MISMATCH);  // its resolution found no item
            break;
        }
        // weight_left: exact, or with truncated bins the interval
        // [A 2^qb, A 2^qb + count (2^qb - 1)] of its fixed-point value
        V wl = WT::value(wacc, fs), wl_hi = wl;
        if constexpr (L > 1) {
            if (apx) {
                const unsigned __int128 ql = (unsigned __int128)wacc[0] << qb;
                wl = fixed_to_f64(ql, fs);
                wl_hi = fixed_to_f64(ql + (unsigned __int128)count * ((((unsigned __int128)1) << qb) - 1), fs);
            }
        }
        // recursive_bisection.rs:547-563.  imbalance <= tol holds on an
        // interval of weight_left values that contains sum/2 (f64 rounding is
        // monotone), so two ends that agree settle it, unless both fail on
        // either side of sum/2; `hi <= t + dist` is monotone in dist.
        // (the upper end only with truncated bins)
        const bool p_lo = imbalance_within<WT>(imt, wl);
        const bool p_hi = apx ? imbalance_within<WT>(imt, wl_hi) : p_lo;
        const bool spans = apx && ideal != 0.0 && WT::f64(wl) <= ideal && ideal <= WT::f64(wl_hi);
        const bool imb_yes = p_lo && p_hi, imb_no = !p_lo && !p_hi && !(spans && tol >= 0.0);
        const bool near_lo = !far && hv <= tv + dl, near_hi = !far && hv <= tv + dh;
        const bool stop = count == prev || near_lo || imb_yes;
        bool need_x = false, need_w = false;
        if (!stop) {
            need_x = near_hi;  // band form: only the exact minimum tells
            need_w = !imb_no;
            // coupe's update (:564-571) is monotone in weight_left
            if (apx && !need_x && !need_w && WT::less(wl, WT::sub(sum, wl)) != WT::less(wl_hi, WT::sub(sum, wl_hi)))
                need_w = true;
        }
        if (need_x || need_w) {
            --steps;  // this step is replayed once its inputs are exact
            if (need_x) {
                flag_exact = true;
                xcut = t;
                xkey = kminO;
                if (sg.xstate == X_PENDING && sg.xcut == t && sg.xkey == (uint32_t)kminO && lane == 0)
                    atomicOr(&rs->err, ERR_COUNT_MISMATCH);  // its resolution found no item
            }
            if (need_w) {
                flag_exactw = true;
                if (!apx && lane == 0) atomicOr(&rs->err, ERR_COUNT_MISMATCH);  // exact bins cannot be undecided
            }
            break;
        }
        if (stop) {
            state = SEG_DONE;
            // items with key < pivot go left; in the band form the cut itself
            // (no item lies in [t, min right), so x < t is the same set)
            if constexpr (KT::BAND)
                pivot = t;
            else
                pivot = KT::unord(kminO);
            split_pos = t;
            wl_out = wl;
            wl_exact = !apx;
            nleft = count;
            break;
        }
        prev = count;
        if (WT::less(wl, WT::sub(sum, wl))) {
            lo = t;
            lo_b = mid_b;
        } else {
            hi = t;
            hi_b = mid_b;
        }
    }
    const uint32_t total_steps = sg.steps + steps;
    if (state != SEG_ACTIVE) {
        if (lane == 0) {
            Seg<KT> &o = segs[s];
            o.state = state;
            o.pivot = pivot;
            o.split_pos = split_pos;
            o.wl = WT::bits(wl_out);
            o.wlx = wl_exact ? 1u : 0u;
            if (L > 1 && sg.sumx != SUMX_NONE) {
                o.sum = WT::bits(sum);
                o.sumx = SUMX_NONE;
            }
            o.nleft = (uint32_t)nleft;
            o.steps = total_steps;
            o.lo = lo;
            o.hi = hi;
            o.prev = prev;
            if (KT::BAND) o.xstate = X_NONE;
            flags[k] = 0;
            atomicAdd((unsigned long long *)&rs->steps_total, (unsigned long long)total_steps);
            atomicMax((unsigned long long *)&rs->steps_max, (unsigned long long)total_steps);
            atomicAdd((unsigned long long *)&rs->splits, 1ull);
        }
    } else {
        // keep searching: clear this segment's bins for the next pass
        for (int b = lane; b < NB; b += 32) {
            const size_t g = g0 + b;
            H.cnt[g] = 0;
#pragma unroll
            for (int l = 0; l < L; ++l) H.w[g * L + l] = 0;
            H.inv[g] = 0;
        }
        if (lane == 0) {
            Seg<KT> &o = segs[s];
            o.lo = lo;
            o.hi = hi;
            o.prev = prev;
            o.steps = total_steps;
            if (L > 1 && sg.sumx != SUMX_NONE) {
                o.sum = WT::bits(sum);
                o.sumx = SUMX_NONE;
            }
            if (flag_exactw) {
                o.exactw = 1;
                atomicAdd(&rs->nexactw, 1u);
            }
            if (KT::BAND && flag_exact) {
                o.xstate = X_PENDING;
                o.xcut = xcut;
                o.xkey = (uint32_t)xkey;
                o.xmin = ~0ull;
                atomicAdd(&rs->nexact, 1u);
            } else if (KT::BAND) {
                o.xstate = X_NONE;
            }
            flags[k] = 1;
        }
    }
}

// One warp per listed segment (decide_one), spc segments per CTA; then the last CTA to finish lists
// the segments still searching and the prefix of their sizes for the next
// pass (list2, P2, rs->nactive).
template <class KT, class WT>
__global__ void __launch_bounds__(BLOCK) k_decide(Seg<KT> *segs, const uint32_t *__restrict__ list, uint32_t nlist,
                                                  Hist<KT, WT> H, int nbk, double tol, uint32_t *flags,
                                                  RunScalars *rs, const uint64_t *nlist_ptr,
                                                  const int32_t *__restrict__ set_fs,
                                                  const int32_t *__restrict__ set_qb, uint32_t *list2, uint64_t *P2,
                                                  ChildArgs<KT> ca, uint32_t spc) {
    __shared__ uint32_t s_last;
    if (cta_halted(rs)) return;
    // the list's length from the device (the grid is an upper bound); every
    // CTA reads it before the last one's scan overwrites it
    if (nlist_ptr) nlist = (uint32_t)*nlist_ptr;
    // spc of the CTA's warps take a segment each (fewer than all when the
    // list is short: the segments' FP64 work then spreads over more SMs)
    const uint32_t w = threadIdx.x >> 5, k = blockIdx.x * spc + w;
    if (w < spc && k < nlist) decide_one<KT, WT>(segs, list, k, H, nbk, tol, flags, rs, set_fs, set_qb);
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) s_last = atomicAdd(&rs->decide_done, 1u) == gridDim.x - 1;
    __syncthreads();
    if (s_last) {
        __threadfence();
        scan_list_block<KT>(segs, list, flags, nlist, list2, P2, rs);
        if (threadIdx.x == 0) {
            rs->decide_done = 0;
            // a queued level's last queued pass: splits still searching halt
            // the queued kernels after it (the host runs more passes)
            if (ca.stall_level && rs->nactive != 0) rs->stall = ca.stall_level;
        }
        if (ca.on) {
            __syncthreads();  // the scan's count (rs->nactive) is read below
            children_body<KT, WT>(segs, ca.S, ca.coord, ca.D, ca.write, ca.level, ca.next, ca.next_list, ca.next_P,
                                  ca.trav, rs, ca.sets, CHILD_ALL, nullptr, ca.S_ptr, ca.lvl);
        }
    }
}



// ---------------------------------------------------------------------------
// k_reorder: stable two-way partition of every segment of the level, out of
// place, one dynamic chunk of the item range per CTA at a time.  A chunk
// learns how many left items of its first segment precede it by a decoupled
// look-back over the chunks before it (bounded wait).  The chunk is walked in
// tiles; a tile arrives in shared memory by bulk copies (one per array,
// issued by one thread, completing on an mbarrier).  Every thread scatters
// its items into an output stage, the tile's left run then its right run,
// each placed at the alignment phase of its destination; once the stage is
// complete the next tile's copies are issued, and each run leaves by one bulk
// store per array (its 16-byte-aligned middle) plus plain stores of its few
// unaligned end elements.  One input buffer and one stage per CTA keep the
// shared memory small enough for three or four CTAs per SM, which hide the
// copies' latency better than a second buffer in fewer CTAs (measured).
// ---------------------------------------------------------------------------
template <int D, class KT, class WT>
struct ReorderArgs {
    const Seg<KT> *segs;
    uint32_t S;
    uint64_t n;  // items of the level's segments (chunks index their list, Seg::voff)
    uint64_t chunk;
    uint64_t nchunks;
    int coord;
    const typename KT::T *ksrc[3];
    typename KT::T *kdst[3];
    const typename WT::S *wsrc;
    typename WT::S *wdst;
    const uint32_t *isrc;  // NULL: identity
    uint32_t *idst;
    int wsafe;     // 1: wsrc is an engine buffer (tiles copied in 16-byte chunks)
    uint64_t *lb;  // look-back words, one per chunk, zeroed
    RunScalars *rs;
    BandSrc bs;    // band form: the f64 coordinates (through isrc)
    uint32_t spin_limit;  // polls of a look-back wait before it fails (ERR_LOOKBACK_TIMEOUT)
    const uint64_t *S_ptr;  // the level's segment and item counts on the device (NULL: S, n)
    const uint64_t *n_ptr;
};

// Items per thread per tile: 8 (2048 per tile) when an item moves at most 18
// bytes (then three CTAs' tiles and stages fit an SM's shared memory), else
// 4; and the CTAs per SM the registers are bounded for: four with 4-byte
// keys and 4 items, else three.
template <int D, class KT, class WT, bool IDX>
__host__ __device__ constexpr int reorder_items() {
    return D * sizeof(typename KT::T) + sizeof(typename WT::S) + (IDX ? 4 : 0) <= 18 ? 8 : 4;
}
template <int D, class KT, class WT, bool IDX>
__host__ __device__ constexpr int reorder_min_ctas() {
    return reorder_items<D, KT, WT, IDX>() == 4 && sizeof(typename KT::T) == 4 ? 4 : 3;
}
__host__ __device__ constexpr size_t al16(size_t x) { return (x + 15) & ~(size_t)15; }

// Dynamic shared memory of the reorder, in 16-byte-aligned arrays:
//   the input tile: D key arrays, the weights and (IDX) the input indices;
//   array a holds the 16-byte chunks covering the tile from the
//   aligned address at or below it (element li at head + li, head = ts mod
//   16 / element size), so RT elements and 16 bytes;
//   one output stage with the same arrays of RT + 24 elements: the left run
//   starts at element (left destination mod 8) and the right run at the next
//   element after it with the right destination's phase mod 8.
template <int D, class KT, class WT, bool IDX>
struct ReorderSmem {
    static constexpr int RT = BLOCK * reorder_items<D, KT, WT, IDX>();
    static constexpr size_t KS = sizeof(typename KT::T), WSZ = sizeof(typename WT::S);
    static constexpr size_t in_key = al16(RT * KS + 16);
    static constexpr size_t in_w = al16(RT * WSZ + 16);
    static constexpr size_t in_idx = IDX ? al16(RT * 4 + 16) : 0;
    static constexpr size_t in_tile = D * in_key + in_w + in_idx;
    static constexpr int OE = RT + 24;
    static constexpr size_t out_key = al16(OE * KS);
    static constexpr size_t out_w = al16(OE * WSZ);
    static constexpr size_t out_idx = IDX ? al16(OE * 4) : 0;
    static constexpr size_t out_tile = D * out_key + out_w + out_idx;
    static constexpr size_t bytes = in_tile + out_tile;
};
template <int D, class KT, class WT>
__host__ __device__ constexpr size_t reorder_smem(bool with_index) {
    return with_index ? ReorderSmem<D, KT, WT, true>::bytes : ReorderSmem<D, KT, WT, false>::bytes;
}
// polls of an input tile's mbarrier before the reorder gives up (the copies
// of a tile take microseconds; this is a guard, not a schedule)
constexpr uint32_t MBAR_SPIN_LIMIT = 1u << 22;

template <class KT>
__device__ __forceinline__ bool goes_left(typename KT::T key, const Seg<KT> &sg) {
    return sg.state == SEG_ALLLEFT || KT::lt(key, sg.pivot);
}
// Band form: x < pivot (the split cut), from the key unless it lies in the
// cut's band; `code` then supplies the item's f64 code.
template <class KT, class CodeFn>
__device__ __forceinline__ bool goes_left_band(float key, const Seg<KT> &sg, const CutBounds &pb, CodeFn code) {
    if (sg.state == SEG_ALLLEFT) return true;
    const int sd = band_side(key, pb);
    return sd < 0 || (sd == 0 && KeyF64::lt(code(), sg.pivot));
}

// A tile of a chunk: items [ts, te) of segment kk.
struct TileRef {
    uint32_t kk;
    uint64_t ts, te;
    uint64_t pend;  // end of the tile's piece (its segment, cut at the chunk end)
    bool first;     // the tile starts its piece
    bool valid;
};

// One run of a tile (len elements from stage element S on) to dst[G ..), by
// the first warp: the 16-byte-aligned middle [j0, j1) by one bulk store (lane
// 0), the elements before and after it by plain stores (lanes 0-15 and
// 16-23).  S has the
// phase of G mod 8 elements, so the middle is aligned on both sides.  A run
// without a whole aligned 16-byte block is all head (j0 = j1 = len < 16).
template <class E>
__device__ __forceinline__ void put_run(E *dst, const E *stg, uint64_t G, uint32_t S, uint32_t len, uint32_t cap,
                                        uint32_t *err) {
    if (S + len > cap) {  // a run past the stage: write nothing
        if (threadIdx.x == 0) atomicOr(err, ERR_TILE_PERM);
        return;
    }
    constexpr uint64_t m = 16 / sizeof(E) - 1;
    const uint64_t a0 = (G + m) & ~m;    // first aligned element at or after G
    const uint64_t a1 = (G + len) & ~m;  // last aligned element at or before the end
    uint32_t j0 = len, j1 = len;
    if (a1 > a0) {
        j0 = (uint32_t)(a0 - G);  // <= m
        j1 = (uint32_t)(a1 - G);  // len - j1 <= m
    }
    if (threadIdx.x == 0 && j1 > j0) bulk_store(dst + G + j0, stg + S + j0, (j1 - j0) * (uint32_t)sizeof(E));
    const uint32_t t = threadIdx.x;
    if (t < j0)
        dst[G + t] = stg[S + t];
    else if (t >= 16 && t - 16 < len - j1)
        dst[G + j1 + (t - 16)] = stg[S + j1 + (t - 16)];
}

// The number of keys kc[la, le) that go left, by the whole CTA: side(k) is
// -1 (left), 1 (right) or 0 (undecided by the key: the band form's f64
// check), and exact(e) decides item e then.  16-byte loads, four in flight
// per thread (16 KB per CTA), after a scalar head up to the first 16-byte
// boundary; the count is on the chunk's look-back chain, so its loads are
// kept in flight together, and the rare exact checks (a call) run after the
// keys of an iteration are no longer needed.
template <class K, class SideFn, class ExactFn>
__device__ __forceinline__ uint64_t count_left_keys(const K *__restrict__ kc, uint64_t la, uint64_t le, SideFn side,
                                                    ExactFn exact) {
    constexpr uint64_t V = 16 / sizeof(K);  // keys per 16 bytes
    uint64_t cnt = 0;
    auto one = [&](K k, uint64_t e) {
        const int sd = side(k);
        cnt += sd < 0 ? 1u : (sd == 0 ? exact(e) : 0u);
    };
    uint64_t a = (la + V - 1) & ~(V - 1);
    if (a > le) a = le;
    for (uint64_t e = la + threadIdx.x; e < a; e += BLOCK) one(kc[e], e);
    const uint64_t nq = (le - a) / V;  // whole 16-byte groups
    const uint4 *q4 = (const uint4 *)(kc + a);
    uint64_t q = threadIdx.x;
    for (; q + 3 * BLOCK < nq; q += 4 * BLOCK) {
        uint4 v[4];
#pragma unroll
        for (int j = 0; j < 4; ++j) v[j] = q4[q + j * BLOCK];
        uint32_t und = 0;  // bit j * V + i: key i of load j is undecided
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const K *kk = (const K *)&v[j];
#pragma unroll
            for (int i = 0; i < (int)V; ++i) {
                const int sd = side(kk[i]);
                cnt += sd < 0 ? 1u : 0u;
                und |= (sd == 0 ? 1u : 0u) << (j * V + i);
            }
        }
        while (und) {
            const int b = __ffs(und) - 1;
            und &= und - 1;
            cnt += exact(a + (q + (b / V) * BLOCK) * V + (b % V));
        }
    }
    for (; q < nq; q += BLOCK) {
        const uint4 v = q4[q];
        const K *kk = (const K *)&v;
        const uint64_t e = a + q * V;
#pragma unroll
        for (int i = 0; i < (int)V; ++i) one(kk[i], e + i);
    }
    for (uint64_t e = a + nq * V + threadIdx.x; e < le; e += BLOCK) one(kc[e], e);
    return cnt;
}

// IDX: the reorder also carries input indices (isrc -> idst); a compile-time
// choice, so that reorders without indices spend no shared memory or
// registers on them.
template <int D, class KT, class WT, bool IDX>
__global__ void __launch_bounds__(BLOCK, (reorder_min_ctas<D, KT, WT, IDX>())) k_reorder(ReorderArgs<D, KT, WT> A) {
    typedef typename KT::T K;
    typedef typename WT::S WS;
    typedef ReorderSmem<D, KT, WT, IDX> SM;
    constexpr int RI = reorder_items<D, KT, WT, IDX>();
    constexpr uint32_t RT = SM::RT;
    extern __shared__ __align__(16) unsigned char dsm[];
    __shared__ __align__(8) uint64_t s_bar;
    __shared__ uint32_t s_cnt[RI * NWARPS];
    __shared__ uint64_t sh[33];
    __shared__ uint64_t s_ticket, s_prefix;
    __shared__ uint32_t s_fail;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const K *__restrict__ kc = A.coord == 0 ? A.ksrc[0] : (A.coord == 1 ? A.ksrc[1] : A.ksrc[2]);
    auto in_key = [&](int d) { return (K *)(dsm + d * SM::in_key); };
    WS *const in_w = (WS *)(dsm + D * SM::in_key);
    uint32_t *const in_idx = (uint32_t *)(dsm + D * SM::in_key + SM::in_w);
    unsigned char *const ob = dsm + SM::in_tile;
    auto out_key = [&](int d) { return (K *)(ob + d * SM::out_key); };
    WS *const out_w = (WS *)(ob + D * SM::out_key);
    uint32_t *const out_idx = (uint32_t *)(ob + D * SM::out_key + SM::out_w);
    constexpr uint64_t KMASK = 16 / sizeof(K) - 1, WMASK = 16 / sizeof(WS) - 1, IMASK = 3;
    // engine buffers are copied in bulk; the caller's weights (level 0) and
    // the identity indices of level 0 are read or made per item
    const bool w_bulk = A.wsafe != 0;
    const bool i_bulk = IDX && A.isrc != nullptr;

    if (cta_halted(A.rs)) return;
    if (threadIdx.x == 0) {
        mbar_init(&s_bar, 1);
        fence_mbar_init();
    }
    __syncthreads();
    uint32_t phase = 0;     // parity of the input tile's next mbarrier phase
    bool inflight = false;  // a tile load issued and not yet waited for (same in every thread)

    // thread 0: the bulk loads of tile t
    auto load_tile = [&](const TileRef &t) {
        const uint64_t k0 = t.ts & ~KMASK;
        const uint32_t kbytes = (uint32_t)(((t.te - k0) * sizeof(K) + 15) & ~15ull);
        uint32_t total = D * kbytes;
        uint64_t w0 = 0, i0 = 0;
        uint32_t wbytes = 0, ibytes = 0;
        if (w_bulk) {
            w0 = t.ts & ~WMASK;
            wbytes = (uint32_t)(((t.te - w0) * sizeof(WS) + 15) & ~15ull);
            total += wbytes;
        }
        if (i_bulk) {
            i0 = t.ts & ~IMASK;
            ibytes = (uint32_t)(((t.te - i0) * 4 + 15) & ~15ull);
            total += ibytes;
        }
        mbar_arrive_expect_tx(&s_bar, total);
#pragma unroll
        for (int d = 0; d < D; ++d) bulk_load(in_key(d), A.ksrc[d] + k0, kbytes, &s_bar);
        if (w_bulk) bulk_load(in_w, A.wsrc + w0, wbytes, &s_bar);
        if (i_bulk) bulk_load(in_idx, A.isrc + i0, ibytes, &s_bar);
    };
    // every thread: wait for the tile (bounded); false (in every thread)
    // when a wait ran out
    auto wait_tile = [&]() -> bool {
        const bool ok = mbar_wait_bounded(&s_bar, phase, MBAR_SPIN_LIMIT);
        const bool all = __syncthreads_and(ok) != 0;
        if (all) {
            phase ^= 1u;
            inflight = false;
        }
        return all;
    };
    // a wait ran out: record it, give the copies in flight one more bounded
    // wait, let the bulk stores finish, and leave
    auto give_up = [&]() {
        if (threadIdx.x == 0) {
            atomicOr(&A.rs->err, ERR_COPY_TIMEOUT);
            if (inflight) mbar_wait_bounded(&s_bar, phase, MBAR_SPIN_LIMIT);
            bulk_wait_all();
        }
        __syncthreads();
    };

    // the level's counts from the device when the host queued the level
    // without them (chunks of the host's size over the actual items); kept
    // in locals: writing to the parameter struct would copy it to local
    // memory
    const uint32_t A_S = A.S_ptr ? (uint32_t)*A.S_ptr : A.S;
    const uint64_t A_n = A.n_ptr ? *A.n_ptr : A.n;
    const uint64_t A_nchunks = A.n_ptr ? (A_n + A.chunk - 1) / A.chunk : A.nchunks;
    for (;;) {
        if (threadIdx.x == 0) s_ticket = atomicAdd((unsigned long long *)&A.rs->ticket, 1ull);
        __syncthreads();
        const uint64_t t = s_ticket;
        if (t >= A_nchunks) break;
        // [c0, c1): positions in the list of the level's items; a segment's
        // items are at off + (position - voff)
        const uint64_t c0 = t * A.chunk, c1 = min(A_n, c0 + A.chunk);
        const uint32_t kf = seg_index_of_v<KT>(A.segs, A_S, c0);
        const uint32_t kl = seg_index_of_v<KT>(A.segs, A_S, c1 - 1);
        auto piece_end = [&](const Seg<KT> &g) { return g.off + (min(c1, g.voff + g.n) - g.voff); };
        const Seg<KT> sf = A.segs[kf];
        TileRef cur;
        cur.kk = kf;
        cur.ts = sf.off + (c0 - sf.voff);
        cur.pend = piece_end(sf);
        cur.te = min(cur.ts + RT, cur.pend);
        cur.first = true;
        cur.valid = true;
        if (threadIdx.x == 0) load_tile(cur);  // overlaps the count below
        inflight = true;
        // count the left items of the last piece
        const Seg<KT> sl = A.segs[kl];
        const uint64_t la = sl.off + (max(c0, sl.voff) - sl.voff), le = sl.off + (c1 - sl.voff);
        uint64_t cnt = 0;
        {
            CutBounds spb = {0.f, 0.f};
            if constexpr (KT::BAND) spb = band_bounds(sl.pivot);
            auto side = [&](K k) -> int {
                if constexpr (KT::BAND)
                    return sl.state == SEG_ALLLEFT ? -1 : band_side(k, spb);
                else
                    return goes_left<KT>(k, sl) ? -1 : 1;
            };
            auto exact = [&](uint64_t e) -> uint32_t {
                return KeyF64::lt(band_code_cold(&A.bs, A.isrc ? A.isrc[e] : e, A.coord), sl.pivot) ? 1u : 0u;
            };
            cnt = count_left_keys<K>(kc, la, le, side, exact);
        }
        uint64_t agg;
        block_exscan_u64(cnt, sh, agg);
        if (threadIdx.x == 0) {
            const bool last_starts_here = sl.voff >= c0;
            s_fail = 0;
            if (last_starts_here) atomicExch((unsigned long long *)&A.lb[t], (unsigned long long)(LB_INCL | agg));
            else atomicExch((unsigned long long *)&A.lb[t], (unsigned long long)(LB_AGG | agg));
            uint64_t prefix = 0;
            if (sf.voff < c0) {
                // look back: chunk t-1 ends inside segment kf
                int64_t j = (int64_t)t - 1;
                for (;;) {
                    uint64_t v;
                    uint32_t spins = 0;
                    while ((v = *((volatile uint64_t *)&A.lb[j])) == 0) {
                        if (++spins > A.spin_limit) break;
                        __nanosleep(64);
                    }
                    if (v == 0) {
                        atomicOr(&A.rs->err, ERR_LOOKBACK_TIMEOUT);
                        s_fail = 1;
                        break;
                    }
                    prefix += v & LB_VALUE;
                    if ((v & ~LB_VALUE) == LB_INCL) break;
                    if (--j < 0) {
                        atomicOr(&A.rs->err, ERR_LOOKBACK_TIMEOUT);
                        s_fail = 1;
                        break;
                    }
                }
                if (!last_starts_here)
                    atomicExch((unsigned long long *)&A.lb[t], (unsigned long long)(LB_INCL | ((prefix + agg) & LB_VALUE)));
            }
            s_prefix = prefix;
        }
        __syncthreads();
        if (s_fail) {
            // the chunk writes nothing; its tile must land before the buffer is reused
            if (!wait_tile()) {
                give_up();
                return;
            }
            continue;
        }
        const uint64_t prefix_first = s_prefix;
        // the current piece's segment, as scalars (kept in registers rather
        // than re-read from the segment table)
        uint64_t p_off = 0, p_nleft = 0;
        uint32_t p_state = 0;
        typename KT::C p_pivot = 0;
        CutBounds pb = {0.f, 0.f};  // band form: bounds of p_pivot
        uint64_t running = 0, seg_end = 0, left_end = 0;
        while (cur.valid) {
            // the next tile of the chunk (it may start the next segment); the
            // segment table is read once per piece, here
            TileRef nxt;
            nxt.valid = false;
            if (cur.te < cur.pend) {
                nxt.kk = cur.kk;
                nxt.ts = cur.te;
                nxt.pend = cur.pend;
                nxt.first = false;
                nxt.valid = true;
            } else if (cur.kk < kl) {
                nxt.kk = cur.kk + 1;
                const Seg<KT> &g = A.segs[nxt.kk];
                nxt.ts = g.off;
                nxt.pend = piece_end(g);
                nxt.first = true;
                nxt.valid = true;
            }
            if (nxt.valid) nxt.te = min(nxt.ts + RT, nxt.pend);
            if (!wait_tile()) {
                give_up();
                return;
            }
            if (cur.first) {
                const Seg<KT> &g = A.segs[cur.kk];
                p_off = g.off;
                p_nleft = g.nleft;
                p_state = g.state;
                p_pivot = g.pivot;
                if constexpr (KT::BAND) pb = band_bounds(p_pivot);
                running = cur.kk == kf ? prefix_first : 0;
                seg_end = p_off + g.n;
                left_end = p_off + p_nleft;
            }
            const uint32_t tcount = (uint32_t)(cur.te - cur.ts);
            const uint32_t kh = (uint32_t)(cur.ts & KMASK);
            const uint32_t wh = (uint32_t)(cur.ts & WMASK);
            const uint32_t ih = (uint32_t)(cur.ts & IMASK);
            const K *tkc = in_key(A.coord) + kh;
            // input index of the tile's item li (level 0: the identity)
            auto orig_of = [&](uint32_t li) -> uint32_t { return i_bulk ? in_idx[ih + li] : (uint32_t)(cur.ts + li); };
            bool fl[RI];
            uint32_t bal[RI];
#pragma unroll
            for (int i = 0; i < RI; ++i) {
                const uint32_t li = i * BLOCK + threadIdx.x;
                if constexpr (KT::BAND)
                    fl[i] = li < tcount &&
                            (p_state == SEG_ALLLEFT || band_side(tkc[li], pb) < 0 ||
                             (band_side(tkc[li], pb) == 0 &&
                              KeyF64::lt(band_code_cold(&A.bs, orig_of(li), A.coord), p_pivot)));
                else
                    fl[i] = li < tcount && (p_state == SEG_ALLLEFT || KT::lt(tkc[li], p_pivot));
                bal[i] = __ballot_sync(0xffffffffu, fl[i]);
                if (lane == 0) s_cnt[i * NWARPS + warp] = __popc(bal[i]);
            }
            __syncthreads();
            if (warp == 0) {
                // exclusive scan of RI * NWARPS counts in (row, warp) order
                constexpr int PER = (RI * NWARPS + 31) / 32;
                uint32_t v[PER], tot = 0;
#pragma unroll
                for (int j = 0; j < PER; ++j) {
                    const int idx = lane * PER + j;
                    v[j] = idx < RI * NWARPS ? s_cnt[idx] : 0;
                    tot += v[j];
                }
                uint32_t inc = tot;
#pragma unroll
                for (int o = 1; o < 32; o <<= 1) {
                    uint32_t u = __shfl_up_sync(0xffffffffu, inc, o);
                    if (lane >= o) inc += u;
                }
                uint32_t run = inc - tot;
#pragma unroll
                for (int j = 0; j < PER; ++j) {
                    const int idx = lane * PER + j;
                    if (idx < RI * NWARPS) s_cnt[idx] = run;
                    run += v[j];
                }
                if (lane == 31) sh[0] = inc;
                if (lane == 0) bulk_wait_read_all();  // the last tile's bulk stores have read the stage
            }
            __syncthreads();
            const uint32_t tile_left = (uint32_t)sh[0];
            // both runs are checked against the segment once per tile
            const uint64_t left_base = p_off + running;
            const uint64_t right_base = p_off + p_nleft + (cur.ts - p_off - running);
            const bool runs_ok = tile_left <= tcount && left_base + tile_left <= left_end && right_base >= left_end &&
                                 right_base + (tcount - tile_left) <= seg_end;
            if (!runs_ok && threadIdx.x == 0) atomicOr(&A.rs->err, ERR_SCATTER_BOUNDS);
            // stage elements of the two runs
            const uint32_t SL = (uint32_t)(left_base & 7);
            const uint32_t SR = ((SL + tile_left + 7) & ~7u) + (uint32_t)(right_base & 7);
            if (runs_ok) {
                const K *ik[D];
                K *ok[D];
#pragma unroll
                for (int d = 0; d < D; ++d) {
                    ik[d] = in_key(d) + kh;
                    ok[d] = out_key(d);
                }
                const WS *iw = w_bulk ? in_w + wh : A.wsrc + cur.ts;  // the caller's weights: read in place
                const uint32_t *ii = in_idx + ih;
                const uint32_t lmask = (1u << lane) - 1;
#pragma unroll
                for (int i = 0; i < RI; ++i) {
                    const uint32_t li = i * BLOCK + threadIdx.x;
                    if (li >= tcount) continue;
                    const uint32_t before = s_cnt[i * NWARPS + warp] + __popc(bal[i] & lmask);
                    // a rank outside its run would write past the stage: skip it
                    if (fl[i] ? before >= tile_left : li - before >= tcount - tile_left) {
                        atomicOr(&A.rs->err, ERR_TILE_PERM);
                        continue;
                    }
                    const uint32_t pos = fl[i] ? SL + before : SR + (li - before);
#pragma unroll
                    for (int d = 0; d < D; ++d) ok[d][pos] = ik[d][li];
                    out_w[pos] = iw[li];
                    if constexpr (IDX) out_idx[pos] = i_bulk ? ii[li] : (uint32_t)(cur.ts + li);
                }
            }
            fence_proxy_async_smem();  // the stage's writes (and the tile's reads), before the bulk copies
            __syncthreads();           // the stage is complete and the input tile free
            if (nxt.valid) {
                if (threadIdx.x == 0) load_tile(nxt);
                inflight = true;
            }
            if (runs_ok && warp == 0) {
                const uint32_t nr = tcount - tile_left;
#pragma unroll
                for (int d = 0; d < D; ++d) {
                    put_run<K>(A.kdst[d], out_key(d), left_base, SL, tile_left, SM::OE, &A.rs->err);
                    put_run<K>(A.kdst[d], out_key(d), right_base, SR, nr, SM::OE, &A.rs->err);
                }
                put_run<WS>(A.wdst, out_w, left_base, SL, tile_left, SM::OE, &A.rs->err);
                put_run<WS>(A.wdst, out_w, right_base, SR, nr, SM::OE, &A.rs->err);
                if constexpr (IDX) {
                    put_run<uint32_t>(A.idst, out_idx, left_base, SL, tile_left, SM::OE, &A.rs->err);
                    put_run<uint32_t>(A.idst, out_idx, right_base, SR, nr, SM::OE, &A.rs->err);
                }
                if (threadIdx.x == 0) bulk_commit();
            }
            running += tile_left;
            cur = nxt;
        }
    }
    if (threadIdx.x == 0) bulk_wait_all();
}

// ---------------------------------------------------------------------------
// k_reorder_small: the same partition for levels whose segments are smaller
// than a few tiles (the batched form's deep levels).  A piece of such a
// segment is one short tile, and k_reorder's single input buffer would wait
// for every tile's copies in turn; here two tile buffers are filled by
// per-thread asynchronous copies (cp.async), so the next piece's tile lands
// while the current one is partitioned.  The tile is permuted in shared
// memory (a 16-bit slot -> item table) and leaves as two coalesced runs.
// ---------------------------------------------------------------------------
// One tile in shared memory: D key arrays and a weight array, each with 16
// bytes of slack.  Arrays in engine buffers (keys, and weights after level 0)
// arrive as the 16-byte chunks covering the tile, starting at the aligned
// address at or below it; element li of the tile is then at li + head, head =
// ts mod (16 / element size).  Carried input indices are not double
// buffered: each thread loads its own items' indices into registers when the
// tile starts (overlapping the partition work) and parks them in one shared
// array for the output loop.
template <int D, class KT>
__host__ __device__ constexpr size_t small_reorder_key_stride() {
    return (size_t)R_TILE * sizeof(typename KT::T) + 16;
}
template <int D, class KT, class WT>
__host__ __device__ constexpr size_t small_reorder_tile_bytes() {
    return D * small_reorder_key_stride<D, KT>() + (size_t)R_TILE * sizeof(typename WT::S) + 16;
}

// Dynamic shared memory of the reorder: two tiles (asynchronous double
// buffering), the tile's inverse permutation and, when indices are carried,
// the tile's indices.
template <int D, class KT, class WT>
__host__ __device__ constexpr size_t small_reorder_smem(bool with_index) {
    return 2 * small_reorder_tile_bytes<D, KT, WT>() + (size_t)R_TILE * sizeof(uint16_t) +
           (with_index ? (size_t)R_TILE * sizeof(uint32_t) : 0);
}

// IDX: the reorder also carries input indices (isrc -> idst); a compile-time
// choice, so that reorders without indices spend no registers on them.  With
// 4-byte keys three CTAs fit an SM's shared memory; the bound keeps the
// registers within that too.
template <int D, class KT, class WT, bool IDX>
__global__ void __launch_bounds__(BLOCK, sizeof(typename KT::T) == 4 ? 3 : 2) k_reorder_small(ReorderArgs<D, KT, WT> A) {
    typedef typename KT::T K;
    typedef typename WT::S WS;
    extern __shared__ __align__(16) unsigned char dsm[];
    constexpr bool with_index = IDX;
    const size_t tile_bytes = small_reorder_tile_bytes<D, KT, WT>();
    uint16_t *perm = (uint16_t *)(dsm + 2 * tile_bytes);  // tile slot -> item of the tile
    uint32_t *s_idx = (uint32_t *)(perm + R_TILE);          // carried indices of the tile (item order)
    __shared__ uint32_t s_cnt[R_ITEMS * NWARPS];
    __shared__ uint64_t sh[33];
    __shared__ uint64_t s_ticket, s_prefix;
    __shared__ uint32_t s_fail;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const K *__restrict__ kc = A.coord == 0 ? A.ksrc[0] : (A.coord == 1 ? A.ksrc[1] : A.ksrc[2]);

    constexpr uint64_t KMASK = 16 / sizeof(K) - 1, WMASK = 16 / sizeof(WS) - 1;
    auto tile_keys = [&](int buf, int d) {
        return (K *)(dsm + buf * tile_bytes + (size_t)d * small_reorder_key_stride<D, KT>());
    };
    auto tile_w = [&](int buf) { return (WS *)(dsm + buf * tile_bytes + (size_t)D * small_reorder_key_stride<D, KT>()); };
    // input index of the item at position e of the level (identity on level 0)
    auto orig = [&](uint64_t e) { return A.isrc ? (uint64_t)A.isrc[e] : e; };
    // carried indices of this thread's items of a tile (loaded one tile ahead)
    auto load_ix = [&](const TileRef &t, uint32_t *ix) {
        const uint32_t cnt = (uint32_t)(t.te - t.ts);
#pragma unroll
        for (int i = 0; i < R_ITEMS; ++i) {
            const uint32_t li = i * BLOCK + threadIdx.x;
            ix[i] = li < cnt ? (uint32_t)orig(t.ts + li) : 0u;
        }
    };
    // the tile's keys and weights (element li at head + li)
    auto key_head = [&](uint64_t ts) { return (uint32_t)(ts & KMASK); };
    auto w_head = [&](uint64_t ts) { return A.wsafe ? (uint32_t)(ts & WMASK) : 0u; };
    auto tile_wt = [&](int buf, uint64_t ts) { return tile_w(buf) + w_head(ts); };
    auto prefetch = [&](const TileRef &t, int buf) {
        const uint32_t cnt = (uint32_t)(t.te - t.ts);
        {
            // keys: the 16-byte chunks covering [ts, te) (engine buffers, 256-byte
            // aligned, with slack after them, so the chunks stay readable)
            const uint64_t k0 = t.ts & ~KMASK;
            const uint32_t nq = (uint32_t)(((t.te - k0) * sizeof(K) + 15) >> 4);
#pragma unroll
            for (int d = 0; d < D; ++d) {
                const uint4 *src = (const uint4 *)(A.ksrc[d] + k0);
                uint4 *dst = (uint4 *)tile_keys(buf, d);
                for (uint32_t q = threadIdx.x; q < nq; q += BLOCK) cp_async<16>(dst + q, src + q);
            }
        }
        if (A.wsafe) {
            const uint64_t w0 = t.ts & ~WMASK;
            const uint32_t nq = (uint32_t)(((t.te - w0) * sizeof(WS) + 15) >> 4);
            const uint4 *src = (const uint4 *)(A.wsrc + w0);
            uint4 *dst = (uint4 *)tile_w(buf);
            for (uint32_t q = threadIdx.x; q < nq; q += BLOCK) cp_async<16>(dst + q, src + q);
        } else if constexpr (sizeof(WS) == 2) {
            // a caller's 16-bit array does not occur (16-bit weights are the
            // engine's own copy); kept element-wise for completeness
            for (uint32_t li = threadIdx.x; li < cnt; li += BLOCK) tile_w(buf)[li] = A.wsrc[t.ts + li];
        } else {
#pragma unroll
            for (int i = 0; i < R_ITEMS; ++i) {
                const uint32_t li = i * BLOCK + threadIdx.x;
                if (li < cnt) cp_async<sizeof(WS)>(tile_w(buf) + li, A.wsrc + t.ts + li);
            }
        }
        cp_async_commit();
    };

    if (cta_halted(A.rs)) return;
    // the level's counts from the device when the host queued the level
    // without them (chunks of the host's size over the actual items); kept
    // in locals: writing to the parameter struct would copy it to local
    // memory
    const uint32_t A_S = A.S_ptr ? (uint32_t)*A.S_ptr : A.S;
    const uint64_t A_n = A.n_ptr ? *A.n_ptr : A.n;
    const uint64_t A_nchunks = A.n_ptr ? (A_n + A.chunk - 1) / A.chunk : A.nchunks;
    for (;;) {
        if (threadIdx.x == 0) s_ticket = atomicAdd((unsigned long long *)&A.rs->ticket, 1ull);
        __syncthreads();
        const uint64_t t = s_ticket;
        if (t >= A_nchunks) break;
        // [c0, c1): positions in the list of the level's items; a segment's
        // items are at off + (position - voff)
        const uint64_t c0 = t * A.chunk, c1 = min(A_n, c0 + A.chunk);
        const uint32_t kf = seg_index_of_v<KT>(A.segs, A_S, c0);
        const uint32_t kl = seg_index_of_v<KT>(A.segs, A_S, c1 - 1);
        auto piece_end = [&](const Seg<KT> &g) { return g.off + (min(c1, g.voff + g.n) - g.voff); };
        const Seg<KT> sf = A.segs[kf];
        TileRef cur;
        cur.kk = kf;
        cur.ts = sf.off + (c0 - sf.voff);
        cur.pend = piece_end(sf);
        cur.te = min(cur.ts + R_TILE, cur.pend);
        cur.first = true;
        cur.valid = true;
        prefetch(cur, 0);  // overlaps the count below
        uint32_t ixn[R_ITEMS];  // indices of the next tile to process
        if (with_index) load_ix(cur, ixn);
        // count the left items of the last piece
        const Seg<KT> sl = A.segs[kl];
        const uint64_t la = sl.off + (max(c0, sl.voff) - sl.voff), le = sl.off + (c1 - sl.voff);
        uint64_t cnt = 0;
        {
            CutBounds spb = {0.f, 0.f};
            if constexpr (KT::BAND) spb = band_bounds(sl.pivot);
            auto side = [&](K k) -> int {
                if constexpr (KT::BAND)
                    return sl.state == SEG_ALLLEFT ? -1 : band_side(k, spb);
                else
                    return goes_left<KT>(k, sl) ? -1 : 1;
            };
            auto exact = [&](uint64_t e) -> uint32_t {
                return KeyF64::lt(band_code_cold(&A.bs, A.isrc ? A.isrc[e] : e, A.coord), sl.pivot) ? 1u : 0u;
            };
            cnt = count_left_keys<K>(kc, la, le, side, exact);
        }
        uint64_t agg;
        block_exscan_u64(cnt, sh, agg);
        if (threadIdx.x == 0) {
            const bool last_starts_here = sl.voff >= c0;
            s_fail = 0;
            if (last_starts_here) atomicExch((unsigned long long *)&A.lb[t], (unsigned long long)(LB_INCL | agg));
            else atomicExch((unsigned long long *)&A.lb[t], (unsigned long long)(LB_AGG | agg));
            uint64_t prefix = 0;
            if (sf.voff < c0) {
                // look back: chunk t-1 ends inside segment kf
                int64_t j = (int64_t)t - 1;
                for (;;) {
                    uint64_t v;
                    uint32_t spins = 0;
                    while ((v = *((volatile uint64_t *)&A.lb[j])) == 0) {
                        if (++spins > A.spin_limit) break;
                        __nanosleep(64);
                    }
                    if (v == 0) {
                        atomicOr(&A.rs->err, ERR_LOOKBACK_TIMEOUT);
                        s_fail = 1;
                        break;
                    }
                    prefix += v & LB_VALUE;
                    if ((v & ~LB_VALUE) == LB_INCL) break;
                    if (--j < 0) {
                        atomicOr(&A.rs->err, ERR_LOOKBACK_TIMEOUT);
                        s_fail = 1;
                        break;
                    }
                }
                if (!last_starts_here)
                    atomicExch((unsigned long long *)&A.lb[t], (unsigned long long)(LB_INCL | ((prefix + agg) & LB_VALUE)));
            }
            s_prefix = prefix;
        }
        __syncthreads();
        if (s_fail) {
            cp_async_wait<0>();  // the prefetched tile must land before the buffer is reused
            __syncthreads();
            continue;
        }
        const uint64_t prefix_first = s_prefix;
        // the current piece's segment, as scalars (kept in registers rather
        // than re-read from the segment table)
        uint64_t p_off = 0, p_nleft = 0;
        uint32_t p_state = 0;
        typename KT::C p_pivot = 0;
        CutBounds pb = {0.f, 0.f};  // band form: bounds of p_pivot
        uint64_t running = 0, seg_end = 0, left_end = 0;
        int tile_no = 0;
        while (cur.valid) {
            // the next tile of the chunk (it may start the next segment); the
            // segment table is read once per piece, here
            TileRef nxt;
            nxt.valid = false;
            if (cur.te < cur.pend) {
                nxt.kk = cur.kk;
                nxt.ts = cur.te;
                nxt.pend = cur.pend;
                nxt.first = false;
                nxt.valid = true;
            } else if (cur.kk < kl) {
                nxt.kk = cur.kk + 1;
                const Seg<KT> &g = A.segs[nxt.kk];
                nxt.ts = g.off;
                nxt.pend = piece_end(g);
                nxt.first = true;
                nxt.valid = true;
            }
            if (nxt.valid) {
                nxt.te = min(nxt.ts + R_TILE, nxt.pend);
                prefetch(nxt, (tile_no + 1) & 1);
                cp_async_wait<1>();
            } else {
                cp_async_wait<0>();
            }
            __syncthreads();  // this tile's copies are visible to every thread
            const int buf = tile_no & 1;
            if (cur.first) {
                const Seg<KT> &g = A.segs[cur.kk];
                p_off = g.off;
                p_nleft = g.nleft;
                p_state = g.state;
                p_pivot = g.pivot;
                if constexpr (KT::BAND) pb = band_bounds(p_pivot);
                running = cur.kk == kf ? prefix_first : 0;
                seg_end = p_off + g.n;
                left_end = p_off + p_nleft;
            }
            const uint32_t tcount = (uint32_t)(cur.te - cur.ts);
            const uint32_t kh = key_head(cur.ts);
            const K *tkc = tile_keys(buf, A.coord) + kh;
            const WS *tw = tile_wt(buf, cur.ts);
            uint32_t ix[R_ITEMS];  // carried indices of this thread's items
            if (with_index) {
#pragma unroll
                for (int i = 0; i < R_ITEMS; ++i) ix[i] = ixn[i];
                if (nxt.valid) load_ix(nxt, ixn);
            }
            bool fl[R_ITEMS];
            uint32_t bal[R_ITEMS];
#pragma unroll
            for (int i = 0; i < R_ITEMS; ++i) {
                const uint32_t li = i * BLOCK + threadIdx.x;
                if constexpr (KT::BAND)
                    fl[i] = li < tcount &&
                            (p_state == SEG_ALLLEFT || band_side(tkc[li], pb) < 0 ||
                             (band_side(tkc[li], pb) == 0 && KeyF64::lt(band_code_cold(&A.bs, ix[i], A.coord), p_pivot)));
                else
                    fl[i] = li < tcount && (p_state == SEG_ALLLEFT || KT::lt(tkc[li], p_pivot));
                bal[i] = __ballot_sync(0xffffffffu, fl[i]);
                if (lane == 0) s_cnt[i * NWARPS + warp] = __popc(bal[i]);
            }
            __syncthreads();
            if (warp == 0) {
                // exclusive scan of R_ITEMS * NWARPS counts in (row, warp) order
                constexpr int PER = (R_ITEMS * NWARPS + 31) / 32;
                uint32_t v[PER], tot = 0;
#pragma unroll
                for (int j = 0; j < PER; ++j) {
                    const int idx = lane * PER + j;
                    v[j] = idx < R_ITEMS * NWARPS ? s_cnt[idx] : 0;
                    tot += v[j];
                }
                uint32_t inc = tot;
#pragma unroll
                for (int o = 1; o < 32; o <<= 1) {
                    uint32_t u = __shfl_up_sync(0xffffffffu, inc, o);
                    if (lane >= o) inc += u;
                }
                uint32_t run = inc - tot;
#pragma unroll
                for (int j = 0; j < PER; ++j) {
                    const int idx = lane * PER + j;
                    if (idx < R_ITEMS * NWARPS) s_cnt[idx] = run;
                    run += v[j];
                }
                if (lane == 31) sh[0] = inc;
            }
            __syncthreads();
            const uint32_t tile_left = (uint32_t)sh[0];
#pragma unroll
            for (int i = 0; i < R_ITEMS; ++i) {
                const uint32_t li = i * BLOCK + threadIdx.x;
                if (li < tcount) {
                    const uint32_t before = s_cnt[i * NWARPS + warp] + __popc(bal[i] & ((1u << lane) - 1));
                    const uint32_t slot = fl[i] ? before : tile_left + (li - before);
                    if (slot < tcount)
                        perm[slot] = (uint16_t)li;
                    else
                        atomicOr(&A.rs->err, ERR_TILE_PERM);
                    if (with_index) s_idx[li] = ix[i];
                }
            }
            __syncthreads();
            // write the left run and the right run, coalesced (both runs are
            // checked against the segment once per tile)
            const uint64_t left_base = p_off + running;
            const uint64_t right_base = p_off + p_nleft + (cur.ts - p_off - running);
            const bool runs_ok = left_base + tile_left <= left_end && right_base >= left_end &&
                                 right_base + (tcount - tile_left) <= seg_end;
            if (!runs_ok && threadIdx.x == 0) atomicOr(&A.rs->err, ERR_SCATTER_BOUNDS);
            for (uint32_t k = threadIdx.x; runs_ok && k < tcount; k += BLOCK) {
                const uint32_t src = perm[k];
                const uint64_t d = k < tile_left ? left_base + k : right_base + (k - tile_left);
                if (src >= tcount) {
                    atomicOr(&A.rs->err, ERR_TILE_PERM);
                    continue;
                }
#pragma unroll
                for (int dd = 0; dd < D; ++dd) A.kdst[dd][d] = tile_keys(buf, dd)[kh + src];
                A.wdst[d] = tw[src];
                if (with_index) A.idst[d] = s_idx[src];
            }
            running += tile_left;
            __syncthreads();  // the buffer and perm are free again
            cur = nxt;
            ++tile_no;
        }
    }
}

// ---------------------------------------------------------------------------
// k_traverse: part ids in input order without carrying item indices through
// the reorders: each item walks the recorded splits from the root with its
// own keys (the copy of the level-0 keys), taking the side the reorder gave
// it, and gets its leaf's heap id minus the smallest heap id
// (recursive_bisection.rs:589-601, 698-702).  Coalesced reads and writes.
// ---------------------------------------------------------------------------
constexpr int TRAV_SMEM_BYTES = 40 * 1024;

template <int D, class KT>
__global__ void __launch_bounds__(BLOCK) k_traverse(const Trav<KT> *__restrict__ trav, uint64_t trav_total,
                                                    LevelOffsets lv, int levels, const typename KT::T *__restrict__ k0,
                                                    const typename KT::T *__restrict__ k1,
                                                    const typename KT::T *__restrict__ k2, uint64_t n,
                                                    uint64_t *__restrict__ part, const RunScalars *rs, BandSrc bs) {
    typedef typename KT::T K;
    constexpr int CAP = TRAV_SMEM_BYTES / sizeof(Trav<KT>);
    if (cta_halted(rs)) return;
    __shared__ Trav<KT> st[CAP];
    const uint64_t cached = trav_total < (uint64_t)CAP ? trav_total : (uint64_t)CAP;
    for (uint64_t j = threadIdx.x; j < cached; j += BLOCK) st[j] = trav[j];
    __syncthreads();
    const uint64_t hmin = rs->min_heap;
    for (uint64_t i = (uint64_t)blockIdx.x * BLOCK + threadIdx.x; i < n; i += (uint64_t)gridDim.x * BLOCK) {
        K key[3];
        key[0] = k0[i];
        key[1] = k1[i];
        if (D == 3) key[2] = k2[i];
        uint64_t seg = 0, id = 0;
        int c = 0;
        for (int L = 0; L < levels; ++L) {
            const uint64_t j = lv.off[L] + seg;
            const Trav<KT> t = j < cached ? st[j] : trav[j];
            const K kc = c == 0 ? key[0] : (c == 1 ? key[1] : key[D - 1]);
            bool left = (t.flags & TRAV_ALLLEFT) != 0;
            if constexpr (KT::BAND) {
                if (!left) {
                    const int sd = band_side(kc, CutBounds{t.blo, t.bhi});
                    left = sd < 0 || (sd == 0 && KeyF64::lt(band_code(bs, i, c == 0 ? 0 : (c == 1 ? 1 : D - 1)), t.pivot));
                }
            } else {
                left = left || KT::lt(kc, t.pivot);
            }
            if (L + 1 < levels)
                seg = t.next + (left ? 0 : ((t.flags & TRAV_HAS_LEFT) ? 1 : 0));
            else
                id = (left ? 2 * t.next + 1 : 2 * t.next + 2) - hmin;
            c = c + 1 == D ? 0 : c + 1;
        }
        part[i] = id;
    }
}

// ---------------------------------------------------------------------------
// k_traverse_smem: k_traverse for a table that fits in shared memory (the
// usual case: 1023 splits for 1024 parts), REF32 and F64 forms (the band
// form has k_traverse_band).  The table is staged as arrays:
// pivots, one 32-bit word per split (index of the first child in the next
// level | all-left flag << 30 | has-left flag << 31) and the heap ids of the
// last level.  Each thread walks TRAV_ILP items at once so that their
// dependent shared-memory lookups overlap.
// ---------------------------------------------------------------------------
constexpr int TRAV_ILP = 4;
constexpr size_t TRAV_SMEM_MAX = 96 * 1024;
constexpr uint32_t TRAV_NX_ALLLEFT = 1u << 30, TRAV_NX_HASLEFT = 1u << 31, TRAV_NX_INDEX = (1u << 30) - 1;

template <class KT>
__host__ __device__ constexpr size_t trav_smem_bytes(uint64_t total, uint64_t n_last) {
    return n_last * sizeof(uint64_t) +
           total * (sizeof(typename KT::C) + sizeof(uint32_t) + (KT::BAND ? 2 * sizeof(float) : 0));
}

template <int D, class KT>
__global__ void __launch_bounds__(BLOCK) k_traverse_smem(const Trav<KT> *__restrict__ trav, uint32_t total,
                                                         LevelOffsets lv, int levels,
                                                         const typename KT::T *__restrict__ k0,
                                                         const typename KT::T *__restrict__ k1,
                                                         const typename KT::T *__restrict__ k2, uint64_t n,
                                                         uint64_t *__restrict__ part, const RunScalars *rs,
                                                         BandSrc bs) {
    typedef typename KT::T K;
    typedef typename KT::C CK;
    if (cta_halted(rs)) return;
    extern __shared__ __align__(16) unsigned char dsm[];
    __shared__ uint32_t s_off[MAX_TRAV_LEVELS];
    const uint32_t off_last = (uint32_t)lv.off[levels - 1];
    uint64_t *s_heap = (uint64_t *)dsm;                       // [total - off_last]
    CK *s_piv = (CK *)(s_heap + (total - off_last));          // [total]
    float2 *s_bnd = (float2 *)(s_piv + total);                // band form: [total] (RD32, RU32)
    uint32_t *s_nx = (uint32_t *)(s_bnd + (KT::BAND ? total : 0));  // [total]
    for (uint32_t j = threadIdx.x; j < total; j += BLOCK) {
        const Trav<KT> t = trav[j];
        const uint32_t fl = ((t.flags & TRAV_ALLLEFT) ? TRAV_NX_ALLLEFT : 0u) | ((t.flags & TRAV_HAS_LEFT) ? TRAV_NX_HASLEFT : 0u);
        s_piv[j] = t.pivot;
        if constexpr (KT::BAND) s_bnd[j] = make_float2(t.blo, t.bhi);
        if (j < off_last) {
            s_nx[j] = fl | ((uint32_t)t.next & TRAV_NX_INDEX);
        } else {
            s_nx[j] = fl;
            s_heap[j - off_last] = t.next;
        }
    }
    for (int L = threadIdx.x; L < levels; L += BLOCK) s_off[L] = (uint32_t)lv.off[L];
    __syncthreads();
    const uint64_t hmin = rs->min_heap;
    const uint64_t step = (uint64_t)gridDim.x * BLOCK * TRAV_ILP;
    for (uint64_t base = (uint64_t)blockIdx.x * BLOCK * TRAV_ILP + threadIdx.x; base < n; base += step) {
        K key[TRAV_ILP][D];
        uint32_t seg[TRAV_ILP];
#pragma unroll
        for (int k = 0; k < TRAV_ILP; ++k) {
            const uint64_t i = base + (uint64_t)k * BLOCK;
            seg[k] = 0;
            if (i < n) {
                key[k][0] = k0[i];
                key[k][1] = k1[i];
                if (D == 3) key[k][D - 1] = k2[i];
            } else {
#pragma unroll
                for (int d = 0; d < D; ++d) key[k][d] = K();
            }
        }
        int c = 0;
        for (int L = 0; L + 1 < levels; ++L) {
            const uint32_t o = s_off[L];
#pragma unroll
            for (int k = 0; k < TRAV_ILP; ++k) {
                const uint32_t e = o + seg[k];
                const uint32_t x = s_nx[e];
                const K kc = c == 0 ? key[k][0] : (c == 1 ? key[k][1] : key[k][D - 1]);
                bool left = (x & TRAV_NX_ALLLEFT) != 0;
                if constexpr (KT::BAND) {
                    if (!left) {
                        const float2 bd = s_bnd[e];
                        const int sd = band_side(kc, CutBounds{bd.x, bd.y});
                        const uint64_t i = base + (uint64_t)k * BLOCK;
                        left = sd < 0 || (sd == 0 && i < n && KeyF64::lt(band_code(bs, i, c), s_piv[e]));
                    }
                } else {
                    left = left || KT::lt(kc, s_piv[e]);
                }
                seg[k] = (x & TRAV_NX_INDEX) + ((!left && (x & TRAV_NX_HASLEFT)) ? 1u : 0u);
            }
            c = c + 1 == D ? 0 : c + 1;
        }
#pragma unroll
        for (int k = 0; k < TRAV_ILP; ++k) {
            const uint64_t i = base + (uint64_t)k * BLOCK;
            const uint32_t e = off_last + seg[k];
            const K kc = c == 0 ? key[k][0] : (c == 1 ? key[k][1] : key[k][D - 1]);
            bool left = (s_nx[e] & TRAV_NX_ALLLEFT) != 0;
            if constexpr (KT::BAND) {
                if (!left) {
                    const float2 bd = s_bnd[e];
                    const int sd = band_side(kc, CutBounds{bd.x, bd.y});
                    left = sd < 0 || (sd == 0 && i < n && KeyF64::lt(band_code(bs, i, c), s_piv[e]));
                }
            } else {
                left = left || KT::lt(kc, s_piv[e]);
            }
            if (i < n) part[i] = 2 * s_heap[seg[k]] + (left ? 1 : 2) - hmin;
        }
    }
}

// ---------------------------------------------------------------------------
// k_traverse_sets: k_traverse for several sets.  An item starts at its set's
// root segment and walks its set's own number of levels; its id is relative
// to the smallest heap id of its set.  Items of a set with iter_count 0 get
// id 0.  Each CTA walks one contiguous range of items (few sets, so their
// splits stay in L1), TRAV_ILP items per thread at once.
// ---------------------------------------------------------------------------
// k_traverse_band: the band form's k_traverse_smem.  One 16-byte record per
// split holds what the walk reads at every level: the split's f32 bounds
// RD32(pivot) <= RU32(pivot) and the word of k_traverse_smem.  The records of
// a thread's TRAV_ILP items are loaded before any compare, and a key between
// the bounds (rare) reads its f64 coordinate and the split's f64 pivot from
// the global table after the others are compared.  The next items' keys load
// during each walk.
// ---------------------------------------------------------------------------
struct __align__(16) BandNode {
    float lo, hi;
    uint32_t nx, pad;
};

__host__ __device__ constexpr size_t trav_band_smem_bytes(uint64_t total, uint64_t n_last) {
    return total * sizeof(BandNode) + n_last * sizeof(uint64_t);
}

template <int D>
__global__ void __launch_bounds__(BLOCK) k_traverse_band(const Trav<KeyBand> *__restrict__ trav, uint32_t total,
                                                         LevelOffsets lv, int levels, const float *__restrict__ k0,
                                                         const float *__restrict__ k1, const float *__restrict__ k2,
                                                         uint64_t n, uint64_t *__restrict__ part,
                                                         const RunScalars *rs, BandSrc bs) {
    extern __shared__ __align__(16) unsigned char dsm[];
    __shared__ uint32_t s_off[MAX_TRAV_LEVELS];
    if (cta_halted(rs)) return;
    const uint32_t off_last = (uint32_t)lv.off[levels - 1];
    BandNode *s_node = (BandNode *)dsm;                   // [total]
    uint64_t *s_heap = (uint64_t *)(s_node + total);      // [total - off_last]
    for (uint32_t j = threadIdx.x; j < total; j += BLOCK) {
        const Trav<KeyBand> t = trav[j];
        BandNode nd;
        nd.lo = t.blo;
        nd.hi = t.bhi;
        nd.nx = ((t.flags & TRAV_ALLLEFT) ? TRAV_NX_ALLLEFT : 0u) | ((t.flags & TRAV_HAS_LEFT) ? TRAV_NX_HASLEFT : 0u);
        if (j < off_last) nd.nx |= (uint32_t)t.next & TRAV_NX_INDEX;
        nd.pad = 0;
        s_node[j] = nd;
        if (j >= off_last) s_heap[j - off_last] = t.next;
    }
    for (int L = threadIdx.x; L < levels; L += BLOCK) s_off[L] = (uint32_t)lv.off[L];
    __syncthreads();
    const uint64_t hmin = rs->min_heap;
    const uint64_t step = (uint64_t)gridDim.x * BLOCK * TRAV_ILP;
    auto load_keys = [&](uint64_t b0, float (*kk)[D]) {
#pragma unroll
        for (int k = 0; k < TRAV_ILP; ++k) {
            const uint64_t i = b0 + (uint64_t)k * BLOCK;
            if (i < n) {
                kk[k][0] = k0[i];
                kk[k][1] = k1[i];
                if (D == 3) kk[k][D - 1] = k2[i];
            } else {
#pragma unroll
                for (int d = 0; d < D; ++d) kk[k][d] = 0.0f;
            }
        }
    };
    float key[TRAV_ILP][D];
    uint64_t base = (uint64_t)blockIdx.x * BLOCK * TRAV_ILP + threadIdx.x;
    load_keys(base, key);
    for (; base < n; base += step) {
        float nxt[TRAV_ILP][D];
        load_keys(base + step, nxt);
        uint32_t seg[TRAV_ILP];
#pragma unroll
        for (int k = 0; k < TRAV_ILP; ++k) seg[k] = 0;
        // -1 left, 1 right (band_side; the f64 coordinate decides in the band)
        auto sides = [&](const BandNode *nd, uint32_t o, int c, int *sd) {
            bool band = false;
#pragma unroll
            for (int k = 0; k < TRAV_ILP; ++k) {
                const float kc = c == 0 ? key[k][0] : (c == 1 ? key[k][1] : key[k][D - 1]);
                sd[k] = (nd[k].nx & TRAV_NX_ALLLEFT) ? -1 : band_side(kc, CutBounds{nd[k].lo, nd[k].hi});
                band |= sd[k] == 0;
            }
            if (band) {
#pragma unroll 1
                for (int k = 0; k < TRAV_ILP; ++k) {
                    if (sd[k] != 0) continue;
                    const uint64_t i = base + (uint64_t)k * BLOCK;
                    sd[k] = (i < n && KeyF64::lt(band_code(bs, i, c), trav[o + seg[k]].pivot)) ? -1 : 1;
                }
            }
        };
        int c = 0;
        for (int L = 0; L + 1 < levels; ++L) {
            const uint32_t o = s_off[L];
            BandNode nd[TRAV_ILP];
#pragma unroll
            for (int k = 0; k < TRAV_ILP; ++k) nd[k] = s_node[o + seg[k]];
            int sd[TRAV_ILP];
            sides(nd, o, c, sd);
#pragma unroll
            for (int k = 0; k < TRAV_ILP; ++k)
                seg[k] = (nd[k].nx & TRAV_NX_INDEX) + ((sd[k] > 0 && (nd[k].nx & TRAV_NX_HASLEFT)) ? 1u : 0u);
            c = c + 1 == D ? 0 : c + 1;
        }
        BandNode nd[TRAV_ILP];
        uint64_t h[TRAV_ILP];
#pragma unroll
        for (int k = 0; k < TRAV_ILP; ++k) {
            nd[k] = s_node[off_last + seg[k]];
            h[k] = s_heap[seg[k]];
        }
        int sd[TRAV_ILP];
        sides(nd, off_last, c, sd);
#pragma unroll
        for (int k = 0; k < TRAV_ILP; ++k) {
            const uint64_t i = base + (uint64_t)k * BLOCK;
            if (i < n) part[i] = 2 * h[k] + (sd[k] < 0 ? 1 : 2) - hmin;
        }
#pragma unroll
        for (int k = 0; k < TRAV_ILP; ++k)
#pragma unroll
            for (int d = 0; d < D; ++d) key[k][d] = nxt[k][d];
    }
}

// ---------------------------------------------------------------------------
template <int D, class KT>
__global__ void __launch_bounds__(BLOCK) k_traverse_sets(const Trav<KT> *__restrict__ trav, LevelOffsets lv,
                                                         const typename KT::T *__restrict__ k0,
                                                         const typename KT::T *__restrict__ k1,
                                                         const typename KT::T *__restrict__ k2, uint64_t n,
                                                         uint64_t *__restrict__ part, SetTab sets, BandSrc bs,
                                                         const RunScalars *rs) {
    typedef typename KT::T K;
    constexpr uint64_t TILE = (uint64_t)BLOCK * TRAV_ILP;
    if (cta_halted(rs)) return;
    const CtaRange r = cta_tiles((n + TILE - 1) / TILE, blockIdx.x, gridDim.x);
    SetCursor cur;
    for (uint64_t t = r.t0; t < r.t1; ++t) {
        K key[TRAV_ILP][D];
        uint64_t seg[TRAV_ILP], hmin[TRAV_ILP];
        uint32_t depth[TRAV_ILP];
        uint32_t maxd = 0;
#pragma unroll
        for (int k = 0; k < TRAV_ILP; ++k) {
            const uint64_t i = t * TILE + (uint64_t)k * BLOCK + threadIdx.x;
            depth[k] = 0;
            seg[k] = 0;
            hmin[k] = 0;
#pragma unroll
            for (int d = 0; d < D; ++d) key[k][d] = K();
            if (i < n) {
                cur.move(sets, i);
                const uint32_t root = sets.root[cur.s];
                if (root != ~0u) {
                    depth[k] = sets.iters[cur.s];
                    seg[k] = root;
                    hmin[k] = sets.minheap[cur.s];
                }
                key[k][0] = k0[i];
                key[k][1] = k1[i];
                if (D == 3) key[k][D - 1] = k2[i];
                maxd = depth[k] > maxd ? depth[k] : maxd;
            }
        }
        uint64_t id[TRAV_ILP] = {};
        int c = 0;
        for (uint32_t L = 0; L < maxd; ++L) {
#pragma unroll
            for (int k = 0; k < TRAV_ILP; ++k) {
                if (L >= depth[k]) continue;
                const uint64_t i = t * TILE + (uint64_t)k * BLOCK + threadIdx.x;
                const Trav<KT> tr = trav[lv.off[L] + seg[k]];
                const K kc = c == 0 ? key[k][0] : (c == 1 ? key[k][1] : key[k][D - 1]);
                bool left = (tr.flags & TRAV_ALLLEFT) != 0;
                if constexpr (KT::BAND) {
                    if (!left) {
                        const int sd = band_side(kc, CutBounds{tr.blo, tr.bhi});
                        left = sd < 0 || (sd == 0 && KeyF64::lt(band_code(bs, i, c), tr.pivot));
                    }
                } else {
                    left = left || KT::lt(kc, tr.pivot);
                }
                if (L + 1 < depth[k])
                    seg[k] = tr.next + ((!left && (tr.flags & TRAV_HAS_LEFT)) ? 1 : 0);
                else
                    id[k] = 2 * tr.next + (left ? 1 : 2) - hmin[k];
            }
            c = c + 1 == D ? 0 : c + 1;
        }
#pragma unroll
        for (int k = 0; k < TRAV_ILP; ++k) {
            const uint64_t i = t * TILE + (uint64_t)k * BLOCK + threadIdx.x;
            if (i < n) part[i] = id[k];
        }
    }
}

// ---------------------------------------------------------------------------
// k_assign: last level — part id of every item = heap id of its leaf minus
// the smallest heap id (recursive_bisection.rs:589-601, 698-702).
// ---------------------------------------------------------------------------
template <class KT>
__global__ void __launch_bounds__(BLOCK) k_assign(const Seg<KT> *__restrict__ segs, uint32_t S, uint64_t n,
                                                  const typename KT::T *__restrict__ kc, const uint32_t *__restrict__ isrc,
                                                  uint64_t *__restrict__ part, RunScalars *rs, BandSrc bs, int coord,
                                                  const uint64_t *S_ptr) {
    if (cta_halted(rs)) return;
    if (S_ptr) S = (uint32_t)*S_ptr;
    const uint64_t c0 = n * blockIdx.x / gridDim.x, c1 = n * (blockIdx.x + 1) / gridDim.x;
    if (c0 >= c1) return;
    const uint64_t hmin = rs->min_heap;
    uint32_t k = seg_index_of<KT>(segs, S, c0);
    uint64_t pos = c0;
    while (pos < c1) {
        const Seg<KT> sg = segs[k];
        const uint64_t pe = min(c1, sg.off + sg.n);
        const uint64_t hl = 2 * sg.heap + 1 - hmin, hr = 2 * sg.heap + 2 - hmin;
        CutBounds pb = {0.f, 0.f};
        if constexpr (KT::BAND) pb = band_bounds(sg.pivot);
        for (uint64_t e = pos + threadIdx.x; e < pe; e += BLOCK) {
            bool left;
            if constexpr (KT::BAND)
                left = goes_left_band<KT>(kc[e], sg, pb, [&]() { return band_code(bs, isrc ? isrc[e] : e, coord); });
            else
                left = goes_left<KT>(kc[e], sg);
            const uint64_t id = left ? hl : hr;
            const uint64_t dst = isrc ? isrc[e] : e;
            if (dst < n)
                part[dst] = id;
            else
                atomicOr(&rs->err, ERR_SCATTER_BOUNDS);
        }
        pos = pe;
        ++k;
    }
}

static __global__ void k_fill_u64(uint64_t *p, uint64_t n, uint64_t v) {
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) p[i] = v;
}

}  // namespace cg
