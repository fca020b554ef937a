// TEST INFRASTRUCTURE ONLY — the oracle.
//
// A CPU restatement of coupe's recursive coordinate bisection (Rcb) and
// recursive inertial bisection (Rib).  Only tests/, __graft_entry__.smoke()
// and bench.py's CPU-baseline leg load this library, and only to check or to
// time against; the product (libcoupe_gpu.so) never links or calls it.
//
// Every function names the reference lines it restates (paths are relative to
// the coupe repository):
//   coupe/src/algorithms/recursive_bisection.rs  (rcb, rcb_recurse,
//       par_rcb_split, reorder_split_scalar, rib)
//   coupe/src/geometry.rs  (BoundingBox::from_points, inertia_matrix,
//       inertia_vector, householder_reflection, OrientedBoundingBox)
//   coupe-ffi/src/lib.rs, coupe-ffi/src/data.rs  (ABI semantics)
//
// Parity pin: the known answers of the reference's own tests (doctests of Rcb
// and Rib, test_rcb_basic, test_par_rcb_split, test_reorder_split_scalar, the
// geometry tests and the coupe-ffi rcb.c example) are checked against this
// file by tests/test_oracle_golden.py.
//
// Third-party arithmetic that the reference takes from dependencies absent
// here is restated from the published algorithms:
//   nalgebra 0.34.1 SymmetricEigen  -> cyclic Jacobi rotations (Golub & Van
//       Loan, "Matrix Computations", 4th ed., section 8.5)
//   nalgebra 0.34.1 try_inverse     -> adjugate / determinant (2x2, 3x3)
//   approx 0.5.1 Ulps::eq           -> |a-b| <= EPSILON, else same sign and
//       at most 4 units in the last place apart
//   rayon 1.11.0 fold/reduce/join   -> sequential folds (deterministic) or
//       OpenMP tasks and chunked folds (the timed CPU baseline)
//
// Build: oracle/Makefile (g++ -O2 -fopenmp -ffp-contract=off).  FP
// contraction must stay off: the reference does separate multiplies and adds.

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <limits>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

typedef __int128 i128;
typedef unsigned __int128 u128;

extern "C" {

// Weight kinds, numbered like coupe.h's enum coupe_type.
enum { OR_INT = 0, OR_INT64 = 1, OR_DOUBLE = 2 };
// Key precision: REF32 restates the reference (f32 keys and cuts); F64 is the
// same algorithm with every f32 replaced by f64.
enum { OR_REF32 = 0, OR_F64 = 1 };
// Mode flag: partition on `key < pivot` with NaN keys always on the right
// (the GPU engine's rule) instead of coupe's Hoare scans, which leave a
// NaN-keyed item on either side depending on its position in the segment.
enum { OR_NAN_RIGHT = 0x100 };
// How f64 weights are summed: sequentially left to right, or in the 128-bit
// fixed-point scheme (order independent, see fixed_q / fixed_to_f64).
enum { OR_FSUM_SEQ = 0, OR_FSUM_FIXED = 1 };

struct oracle_stats {
    uint64_t splits;       // par_rcb_split calls on non-empty segments
    uint64_t iterations;   // loop iterations summed over all splits
    uint64_t max_iterations;
    uint64_t pivot_ties;   // splits whose fold pivot differs from the min right key
    uint64_t active_points;  // sum over iterations of the segment size
    double root_sum;       // weight sum as f64
    int fixed_scale;       // s of the fixed-point scheme (f64 weights)
    int pad;
};

}  // extern "C"

namespace {

// ---------------------------------------------------------------------------
// 128-bit fixed-point sums of f64 weights (order independent).
// q(w) = round_half_even(w * 2^s) as a signed 128-bit integer, where
// s = 126 - e - ceil(log2(n)) and 2^(e-1) <= max|w| < 2^e, so any sum of at
// most n terms stays below 2^126 in magnitude.
// ---------------------------------------------------------------------------
static int ceil_log2(uint64_t n) {
    int l = 0;
    while (l < 63 && (uint64_t(1) << l) < n) ++l;
    return l;
}

static int fixed_scale_of(const double *w, size_t n) {
    double a = 0.0;
    for (size_t i = 0; i < n; ++i) {
        double v = std::fabs(w[i]);
        if (v > a) a = v;
    }
    if (a == 0.0) return 0;
    int e;
    std::frexp(a, &e);
    return 126 - e - ceil_log2(n);
}

static i128 fixed_q(double w, int s) {
    if (w == 0.0) return 0;
    int ex;
    double f = std::frexp(std::fabs(w), &ex);
    uint64_t m = (uint64_t)std::ldexp(f, 53);  // exact, in [2^52, 2^53)
    int x = ex - 53 + s;                        // |w| 2^s = m 2^x
    u128 q;
    if (x >= 0) {
        q = (u128)m << x;
    } else {
        int r = -x;
        if (r >= 54) {
            q = 0;
        } else {
            uint64_t qi = m >> r;
            uint64_t rem = m & ((uint64_t(1) << r) - 1);
            uint64_t half = uint64_t(1) << (r - 1);
            if (rem > half || (rem == half && (qi & 1))) ++qi;
            q = qi;
        }
    }
    return w < 0 ? -(i128)q : (i128)q;
}

static double fixed_to_f64(i128 Q, int s) {
    if (Q == 0) return 0.0;
    bool neg = Q < 0;
    u128 a = neg ? (u128)(-Q) : (u128)Q;
    int hb = 127;
    while (!((a >> hb) & 1)) --hb;
    uint64_t m;
    int x = 0;
    if (hb <= 52) {
        m = (uint64_t)a;
    } else {
        int sh = hb - 52;
        m = (uint64_t)(a >> sh);
        u128 rem = a & (((u128)1 << sh) - 1);
        u128 half = (u128)1 << (sh - 1);
        if (rem > half || (rem == half && (m & 1))) ++m;
        if (m == (uint64_t(1) << 53)) {
            m >>= 1;
            ++sh;
        }
        x = sh;
    }
    double r = std::ldexp((double)m, x - s);
    return neg ? -r : r;
}

// ---------------------------------------------------------------------------
// Weight arithmetic (RcbWeight, recursive_bisection.rs:708-722).  Integer
// weights wrap like release-built Rust; c_int wraps at 32 bits.
// ---------------------------------------------------------------------------
struct WI32 {
    typedef int32_t S;  // stored
    typedef int32_t V;  // value
    typedef uint32_t A; // accumulator
    static A zero() { return 0; }
    static A add(A a, S w, int) { return a + (uint32_t)w; }
    static A merge(A a, A b) { return a + b; }
    static V fin(A a, int) { return (int32_t)a; }
    static V sub(V a, V b) { return (int32_t)((uint32_t)a - (uint32_t)b); }
    static bool less(V a, V b) { return a < b; }
    static double f64(V v) { return (double)v; }
};
struct WI64 {
    typedef int64_t S;
    typedef int64_t V;
    typedef uint64_t A;
    static A zero() { return 0; }
    static A add(A a, S w, int) { return a + (uint64_t)w; }
    static A merge(A a, A b) { return a + b; }
    static V fin(A a, int) { return (int64_t)a; }
    static V sub(V a, V b) { return (int64_t)((uint64_t)a - (uint64_t)b); }
    static bool less(V a, V b) { return a < b; }
    static double f64(V v) { return (double)v; }
};
struct WF64Seq {
    typedef double S;
    typedef double V;
    typedef double A;
    static A zero() { return 0.0; }
    static A add(A a, S w, int) { return a + w; }
    static A merge(A a, A b) { return a + b; }
    static V fin(A a, int) { return a; }
    static V sub(V a, V b) { return a - b; }
    static bool less(V a, V b) { return a < b; }
    static double f64(V v) { return v; }
};
struct WF64Fixed {
    typedef double S;
    typedef double V;
    typedef i128 A;
    static A zero() { return 0; }
    static A add(A a, S w, int s) { return a + fixed_q(w, s); }
    static A merge(A a, A b) { return a + b; }
    static V fin(A a, int s) { return fixed_to_f64(a, s); }
    static V sub(V a, V b) { return a - b; }
    static bool less(V a, V b) { return a < b; }
    static double f64(V v) { return v; }
};

// Items (recursive_bisection.rs:105-109): D key slices, weights and the
// original index of each item (the reference moves &AtomicUsize pointers).
template <class K, class WT>
struct Items {
    K *keys[3];
    typename WT::S *w;
    uint64_t *idx;
    size_t n;
    Items sub(size_t off, size_t len) const {
        Items r = *this;
        for (int d = 0; d < 3; ++d) r.keys[d] = keys[d] ? keys[d] + off : nullptr;
        r.w = w + off;
        r.idx = idx + off;
        r.n = len;
        return r;
    }
};

// Where recurse records each split's position by heap id (oracle_record_splits;
// the test of float-weight parity traces mismatching ids to these).
static double *g_split_buf = nullptr;
static uint64_t g_split_cap = 0;

struct Ctx {
    int dim;
    double tol;
    int fscale;
    bool parallel;
    size_t min_len;  // rayon with_min_len(4096)
    bool nan_right;
    uint64_t *part;
    oracle_stats st;
};

template <class K, class WT>
static void swap_items(Items<K, WT> &it, int dim, size_t a, size_t b) {
    for (int d = 0; d < dim; ++d) std::swap(it.keys[d][a], it.keys[d][b]);
    std::swap(it.w[a], it.w[b]);
    std::swap(it.idx[a], it.idx[b]);
}

// reorder_split_scalar (recursive_bisection.rs:122-181): move the pivot to
// slot 0, Hoare-partition the rest on `key < pivot`, swap the pivot back to
// the boundary.  Returns the size of the left part.
template <class K, class WT>
static size_t reorder_split(Items<K, WT> &it, int dim, size_t pivot, int coord) {
    swap_items(it, dim, 0, pivot);
    const K pv = it.keys[coord][0];
    // the partition runs on the items 1..n (split_at_mut(1))
    size_t l = 0, r = it.n - 1;
    K *c = it.keys[coord] + 1;
    for (;;) {
        while (l < r && c[l] < pv) ++l;
        while (l < r && pv <= c[r - 1]) --r;
        if (r <= l) break;
        --r;
        swap_items(it, dim, 1 + l, 1 + r);
        ++l;
    }
    swap_items(it, dim, 0, l);
    return l;
}

// Stable two-way partition on `key < pivot value` (NaN keys go right).
template <class K, class WT>
static size_t stable_split(Items<K, WT> &it, int dim, size_t pivot, int coord) {
    const K pv = it.keys[coord][pivot];
    std::vector<size_t> order;
    order.reserve(it.n);
    for (size_t i = 0; i < it.n; ++i)
        if (it.keys[coord][i] < pv) order.push_back(i);
    const size_t nl = order.size();
    for (size_t i = 0; i < it.n; ++i)
        if (!(it.keys[coord][i] < pv)) order.push_back(i);
    for (int d = 0; d < dim; ++d) {
        std::vector<K> tmp(it.n);
        for (size_t i = 0; i < it.n; ++i) tmp[i] = it.keys[d][order[i]];
        std::copy(tmp.begin(), tmp.end(), it.keys[d]);
    }
    std::vector<typename WT::S> tw(it.n);
    std::vector<uint64_t> ti(it.n);
    for (size_t i = 0; i < it.n; ++i) {
        tw[i] = it.w[order[i]];
        ti[i] = it.idx[order[i]];
    }
    std::copy(tw.begin(), tw.end(), it.w);
    std::copy(ti.begin(), ti.end(), it.idx);
    return nl;
}

template <class K, class WT>
struct FoldAcc {
    size_t count;
    typename WT::A wl;
    bool found;
    size_t nidx;
    K nd;
};

// The fold of par_rcb_split (recursive_bisection.rs:478-503) over [lo, hi).
template <class K, class WT>
static FoldAcc<K, WT> fold_range(const K *key, const typename WT::S *w, size_t lo, size_t hi, K t,
                                 int fs) {
    FoldAcc<K, WT> a;
    a.count = 0;
    a.wl = WT::zero();
    a.found = false;
    a.nidx = 0;
    a.nd = std::numeric_limits<K>::infinity();
    for (size_t i = lo; i < hi; ++i) {
        K d = key[i] - t;
        if (d < (K)0) {
            a.count += 1;
            a.wl = WT::add(a.wl, w[i], fs);
        } else if (d < a.nd) {
            a.nd = d;
            a.nidx = i;
            a.found = true;
        }
    }
    return a;
}

// The reduce of par_rcb_split (recursive_bisection.rs:504-520): on equal
// distances the right operand wins.
template <class K, class WT>
static FoldAcc<K, WT> reduce2(const FoldAcc<K, WT> &x, const FoldAcc<K, WT> &y) {
    FoldAcc<K, WT> r;
    r.count = x.count + y.count;
    r.wl = WT::merge(x.wl, y.wl);
    if (x.nd < y.nd) {
        r.nd = x.nd;
        r.nidx = x.nidx;
        r.found = x.found;
    } else {
        r.nd = y.nd;
        r.nidx = y.nidx;
        r.found = y.found;
    }
    return r;
}

template <class K, class WT>
static FoldAcc<K, WT> fold_all(Ctx &cx, const K *key, const typename WT::S *w, size_t n, K t) {
    if (!cx.parallel || n < 2 * cx.min_len) return fold_range<K, WT>(key, w, 0, n, t, cx.fscale);
    size_t chunks = n / cx.min_len;
    if (chunks > 1024) chunks = 1024;
    std::vector<FoldAcc<K, WT>> partv(chunks);
    FoldAcc<K, WT> *part = partv.data();
    const size_t per = (n + chunks - 1) / chunks;
    const int fs = cx.fscale;
#pragma omp taskloop grainsize(1)
    for (size_t c = 0; c < chunks; ++c) {
        size_t lo = c * per, hi = std::min(n, lo + per);
        part[c] = fold_range<K, WT>(key, w, lo, hi, t, fs);
    }
    FoldAcc<K, WT> r = part[0];
    for (size_t c = 1; c < chunks; ++c) r = reduce2<K, WT>(r, part[c]);
    return r;
}

template <class K, class WT>
struct SplitOut {
    size_t nleft;
    typename WT::V wl;
    K split_pos;
};

// par_rcb_split (recursive_bisection.rs:456-573).
template <class K, class WT>
static SplitOut<K, WT> split(Ctx &cx, Items<K, WT> &it, int coord, K mn, K mx, typename WT::V sum) {
    size_t prev = SIZE_MAX;
    uint64_t iters = 0, active = 0;
    SplitOut<K, WT> o;
    for (;;) {
        ++iters;
        active += it.n;
        const K t = (mn + mx) / (K)2;
        FoldAcc<K, WT> a = fold_all<K, WT>(cx, it.keys[coord], it.w, it.n, t);
        if (!a.found) {
            if (prev == a.count) {
                o.nleft = it.n;
                o.wl = sum;
                o.split_pos = mx;
                break;
            }
            mx = t;
            prev = a.count;
            continue;
        }
        const typename WT::V wl = WT::fin(a.wl, cx.fscale);
        const double ideal = WT::f64(sum) / 2.0;
        const double imb = std::fabs((WT::f64(wl) - ideal) / ideal);
        if (a.count == prev || mx <= t + a.nd || imb <= cx.tol) {
            if (!cx.parallel) {
                // The GPU takes the smallest key >= t as the pivot; the fold
                // may pick another key at the same rounded distance.
                K kmin = std::numeric_limits<K>::infinity();
                for (size_t i = 0; i < it.n; ++i) {
                    K k = it.keys[coord][i];
                    if (k >= t && k < kmin) kmin = k;
                }
                if (!(it.keys[coord][a.nidx] == kmin)) cx.st.pivot_ties += 1;
            }
            o.nleft = cx.nan_right ? stable_split(it, cx.dim, a.nidx, coord)
                                   : reorder_split(it, cx.dim, a.nidx, coord);
            o.wl = wl;
            o.split_pos = t;
            break;
        }
        prev = a.count;
        const typename WT::V wr = WT::sub(sum, wl);
        if (WT::less(wl, wr))
            mn = t;
        else
            mx = t;
    }
    if (!cx.parallel) {
        cx.st.splits += 1;
        cx.st.iterations += iters;
        cx.st.active_points += active;
        cx.st.max_iterations = std::max<uint64_t>(cx.st.max_iterations, iters);
    }
    return o;
}

// rcb_recurse (recursive_bisection.rs:575-642).  The bounding box is kept in
// f64 and cast to K at use, as the reference does (`bb.p_min[coord] as f32`,
// `split_pos as f64`).
template <class K, class WT>
static void recurse(Ctx &cx, Items<K, WT> it, size_t iter_count, uint64_t iter_id, int coord,
                    typename WT::V sum, const double *bmin, const double *bmax) {
    if (it.n == 0) return;
    if (iter_count == 0) {
        uint64_t *part = cx.part;
        const uint64_t *idx = it.idx;
        const size_t n = it.n;
        if (cx.parallel && n >= 2 * cx.min_len) {
#pragma omp taskloop grainsize(4096)
            for (size_t i = 0; i < n; ++i) part[idx[i]] = iter_id;
        } else {
            for (size_t i = 0; i < n; ++i) part[idx[i]] = iter_id;
        }
        return;
    }
    const K mn = (K)bmin[coord];
    const K mx = (K)bmax[coord];
    SplitOut<K, WT> s = split<K, WT>(cx, it, coord, mn, mx, sum);
    if (g_split_buf && iter_id < g_split_cap) g_split_buf[iter_id] = (double)s.split_pos;
    double lmin[3], lmax[3], rmin[3], rmax[3];
    for (int d = 0; d < 3; ++d) {
        lmin[d] = rmin[d] = bmin[d];
        lmax[d] = rmax[d] = bmax[d];
    }
    lmax[coord] = (double)s.split_pos;
    rmin[coord] = (double)s.split_pos;
    Items<K, WT> L = it.sub(0, s.nleft);
    Items<K, WT> R = it.sub(s.nleft, it.n - s.nleft);
    const int nc = (coord + 1) % cx.dim;
    const typename WT::V rs = WT::sub(sum, s.wl);
    if (cx.parallel && it.n >= cx.min_len) {
#pragma omp task default(shared) firstprivate(L, lmin, lmax, nc, iter_count, iter_id, s)
        recurse<K, WT>(cx, L, iter_count - 1, 2 * iter_id + 1, nc, s.wl, lmin, lmax);
        recurse<K, WT>(cx, R, iter_count - 1, 2 * iter_id + 2, nc, rs, rmin, rmax);
#pragma omp taskwait
    } else {
        recurse<K, WT>(cx, L, iter_count - 1, 2 * iter_id + 1, nc, s.wl, lmin, lmax);
        recurse<K, WT>(cx, R, iter_count - 1, 2 * iter_id + 2, nc, rs, rmin, rmax);
    }
}

// BoundingBox::from_points (geometry.rs:33-78): f64 fold starting from
// (f64::MAX, f64::MIN) with `val < min` / `max < val`; NaN never updates.
static void bbox_f64(const double *pts, size_t n, int dim, double *bmin, double *bmax) {
    for (int d = 0; d < dim; ++d) {
        bmin[d] = std::numeric_limits<double>::max();
        bmax[d] = -std::numeric_limits<double>::max();
    }
    for (size_t i = 0; i < n; ++i)
        for (int d = 0; d < dim; ++d) {
            double v = pts[i * dim + d];
            if (v < bmin[d]) bmin[d] = v;
            if (bmax[d] < v) bmax[d] = v;
        }
}

// rcb (recursive_bisection.rs:644-705) on AoS f64 points.
template <class K, class WT>
static int rcb_typed(Ctx &cx, uint64_t *part, size_t n, const double *pts, const typename WT::S *w_in,
                     size_t iter_count) {
    if (n == 0) return 0;
    const int dim = cx.dim;
    std::vector<K> keyv[3];
    for (int d = 0; d < dim; ++d) keyv[d].resize(n);
    std::vector<typename WT::S> wv(w_in, w_in + n);
    std::vector<uint64_t> idxv(n);
    K *keys[3] = {nullptr, nullptr, nullptr};
    for (int d = 0; d < dim; ++d) keys[d] = keyv[d].data();
    uint64_t *idx = idxv.data();
    typename WT::S *w = wv.data();
    // coords[d] = points.map(|p| p[d] as f32)  (:674-679), the weight sum
    // (:684) and BoundingBox::from_points (:685), in chunks.
    const size_t chunk = 65536;
    const size_t nch = (n + chunk - 1) / chunk;
    std::vector<typename WT::A> accv(nch);
    std::vector<double> bbv(nch * 6);
    typename WT::A *accs = accv.data();
    double *bbs = bbv.data();
    const int fs = cx.fscale;
    auto body = [&](size_t c) {
        size_t lo = c * chunk, hi = std::min(n, lo + chunk);
        typename WT::A a = WT::zero();
        for (size_t i = lo; i < hi; ++i) {
            for (int d = 0; d < dim; ++d) keys[d][i] = (K)pts[i * dim + d];
            idx[i] = i;
            a = WT::add(a, w[i], fs);
        }
        accs[c] = a;
        bbox_f64(pts + lo * dim, hi - lo, dim, bbs + c * 6, bbs + c * 6 + 3);
    };
    if (cx.parallel) {
#pragma omp taskloop grainsize(1)
        for (size_t c = 0; c < nch; ++c) body(c);
    } else {
        for (size_t c = 0; c < nch; ++c) body(c);
    }
    typename WT::A acc = WT::zero();
    if (cx.parallel) {
        for (size_t c = 0; c < nch; ++c) acc = WT::merge(acc, accs[c]);
    } else {
        for (size_t i = 0; i < n; ++i) acc = WT::add(acc, w[i], fs);  // left to right
    }
    const typename WT::V sum = WT::fin(acc, cx.fscale);
    cx.st.root_sum = WT::f64(sum);
    double bmin[3] = {0, 0, 0}, bmax[3] = {0, 0, 0};
    for (int d = 0; d < dim; ++d) {
        bmin[d] = bbs[d];
        bmax[d] = bbs[3 + d];
        // reduce_with(min, max) over the chunk folds (geometry.rs:60-75)
        for (size_t c = 1; c < nch; ++c) {
            bmin[d] = std::fmin(bmin[d], bbs[c * 6 + d]);
            bmax[d] = std::fmax(bmax[d], bbs[c * 6 + 3 + d]);
        }
    }
    Items<K, WT> it;
    for (int d = 0; d < 3; ++d) it.keys[d] = keys[d];
    it.w = w;
    it.idx = idx;
    it.n = n;
    cx.part = part;
    recurse<K, WT>(cx, it, iter_count, 0, 0, sum, bmin, bmax);
    // part_ids -= min(part_ids)  (:698-702)
    uint64_t mn = part[0];
    for (size_t i = 1; i < n; ++i) mn = std::min(mn, part[i]);
    for (size_t i = 0; i < n; ++i) part[i] -= mn;
    return 0;
}

template <class K>
static int rcb_dispatch(Ctx &cx, uint64_t *part, size_t n, const double *pts, int wtype, const void *w,
                        size_t iter_count, int fsum) {
    switch (wtype) {
    case OR_INT:
        return rcb_typed<K, WI32>(cx, part, n, pts, (const int32_t *)w, iter_count);
    case OR_INT64:
        return rcb_typed<K, WI64>(cx, part, n, pts, (const int64_t *)w, iter_count);
    case OR_DOUBLE:
        cx.fscale = fixed_scale_of((const double *)w, n);
        cx.st.fixed_scale = cx.fscale;
        if (fsum == OR_FSUM_FIXED) return rcb_typed<K, WF64Fixed>(cx, part, n, pts, (const double *)w, iter_count);
        return rcb_typed<K, WF64Seq>(cx, part, n, pts, (const double *)w, iter_count);
    }
    return -1;
}

static int rcb_entry(uint64_t *part, size_t n, int dim, const double *pts, int wtype, const void *w,
                     size_t iter_count, double tol, int mode, int fsum, int threads, oracle_stats *st) {
    if (dim != 2 && dim != 3) return -1;
    Ctx cx;
    std::memset(&cx, 0, sizeof(cx));
    cx.dim = dim;
    cx.tol = tol;
    cx.min_len = 4096;
    cx.parallel = threads != 1;
    cx.nan_right = (mode & OR_NAN_RIGHT) != 0;
    mode &= 0xff;
    int rc = 0;
    if (!cx.parallel) {
        rc = mode == OR_F64 ? rcb_dispatch<double>(cx, part, n, pts, wtype, w, iter_count, fsum)
                            : rcb_dispatch<float>(cx, part, n, pts, wtype, w, iter_count, fsum);
    } else {
#ifdef _OPENMP
        int nt = threads > 0 ? threads : omp_get_max_threads();
#pragma omp parallel num_threads(nt)
#pragma omp single
#endif
        rc = mode == OR_F64 ? rcb_dispatch<double>(cx, part, n, pts, wtype, w, iter_count, fsum)
                            : rcb_dispatch<float>(cx, part, n, pts, wtype, w, iter_count, fsum);
    }
    if (st) *st = cx.st;
    return rc;
}

// ---------------------------------------------------------------------------
// Rib geometry (geometry.rs:203-319).
// ---------------------------------------------------------------------------

// inertia_matrix (geometry.rs:273-284): unweighted centroid, then
// sum of (p - c)(p - c)^T; both sums sequential.
static void inertia_matrix(const double *pts, size_t n, int dim, double *m /* dim*dim row-major */) {
    double c[3] = {0, 0, 0};
    for (size_t i = 0; i < n; ++i)
        for (int d = 0; d < dim; ++d) c[d] += pts[i * dim + d];
    for (int d = 0; d < dim; ++d) c[d] = c[d] / (double)n;
    for (int k = 0; k < dim * dim; ++k) m[k] = 0.0;
    for (size_t i = 0; i < n; ++i) {
        double o[3];
        for (int d = 0; d < dim; ++d) o[d] = pts[i * dim + d] - c[d];
        for (int a = 0; a < dim; ++a)
            for (int b = 0; b < dim; ++b) m[a * dim + b] += o[a] * o[b];
    }
}

// Symmetric eigen-decomposition by cyclic Jacobi rotations (Golub & Van
// Loan 8.5).  v receives the eigenvectors as columns.
static void jacobi_eigen(const double *a_in, int n, double *evals, double *v) {
    double a[9];
    for (int k = 0; k < n * n; ++k) a[k] = a_in[k];
    for (int i = 0; i < n; ++i)
        for (int j = 0; j < n; ++j) v[i * n + j] = i == j ? 1.0 : 0.0;
    for (int sweep = 0; sweep < 64; ++sweep) {
        double off = 0.0;
        for (int p = 0; p < n; ++p)
            for (int q = p + 1; q < n; ++q) off += a[p * n + q] * a[p * n + q];
        if (off == 0.0) break;
        for (int p = 0; p < n; ++p)
            for (int q = p + 1; q < n; ++q) {
                double apq = a[p * n + q];
                if (apq == 0.0) continue;
                double app = a[p * n + p], aqq = a[q * n + q];
                double theta = (aqq - app) / (2.0 * apq);
                double t = (theta >= 0 ? 1.0 : -1.0) / (std::fabs(theta) + std::sqrt(theta * theta + 1.0));
                double c = 1.0 / std::sqrt(t * t + 1.0), s = t * c;
                for (int k = 0; k < n; ++k) {
                    double akp = a[k * n + p], akq = a[k * n + q];
                    a[k * n + p] = c * akp - s * akq;
                    a[k * n + q] = s * akp + c * akq;
                }
                for (int k = 0; k < n; ++k) {
                    double apk = a[p * n + k], aqk = a[q * n + k];
                    a[p * n + k] = c * apk - s * aqk;
                    a[q * n + k] = s * apk + c * aqk;
                }
                for (int k = 0; k < n; ++k) {
                    double vkp = v[k * n + p], vkq = v[k * n + q];
                    v[k * n + p] = c * vkp - s * vkq;
                    v[k * n + q] = s * vkp + c * vkq;
                }
            }
    }
    for (int i = 0; i < n; ++i) evals[i] = a[i * n + i];
}

// inertia_vector (geometry.rs:286-303): eigenvector of the largest eigenvalue.
static void inertia_vector(const double *m, int dim, double *vec) {
    double ev[3], v[9];
    jacobi_eigen(m, dim, ev, v);
    int best = 0;
    for (int i = 1; i < dim; ++i)
        if (ev[i] > ev[best]) best = i;
    for (int i = 0; i < dim; ++i) vec[i] = v[i * dim + best];
}

// approx 0.5 Ulps::default().eq for one f64.
static bool ulps_eq(double a, double b) {
    if (std::fabs(a - b) <= std::numeric_limits<double>::epsilon()) return true;
    if (std::signbit(a) != std::signbit(b)) return false;
    int64_t ia, ib;
    std::memcpy(&ia, &a, 8);
    std::memcpy(&ib, &b, 8);
    int64_t d = ia > ib ? ia - ib : ib - ia;
    return d <= 4;
}

// householder_reflection (geometry.rs:305-319).
static void householder(const double *el, int dim, double *h) {
    double nrm2 = 0.0;
    for (int d = 0; d < dim; ++d) nrm2 += el[d] * el[d];
    const double nrm = std::sqrt(nrm2);
    bool par = true;
    for (int d = 0; d < dim; ++d)
        if (!ulps_eq(el[d] / nrm, d == 0 ? 1.0 : 0.0)) par = false;
    for (int i = 0; i < dim; ++i)
        for (int j = 0; j < dim; ++j) h[i * dim + j] = i == j ? 1.0 : 0.0;
    if (par) return;
    const double sign = el[0] > 0.0 ? -1.0 : 1.0;
    double w[16];  // dim <= 16 (the reference's own test uses 6)
    for (int d = 0; d < dim; ++d) w[d] = el[d] + (d == 0 ? sign * nrm : 0.0);
    double wtw = 0.0;
    for (int d = 0; d < dim; ++d) wtw += w[d] * w[d];
    for (int i = 0; i < dim; ++i)
        for (int j = 0; j < dim; ++j) h[i * dim + j] -= 2.0 * w[i] * w[j] / wtw;
}

// try_inverse (geometry.rs:219) by adjugate / determinant.
static bool inverse(const double *m, int dim, double *r) {
    if (dim == 2) {
        double det = m[0] * m[3] - m[1] * m[2];
        if (det == 0.0) return false;
        r[0] = m[3] / det;
        r[1] = -m[1] / det;
        r[2] = -m[2] / det;
        r[3] = m[0] / det;
        return true;
    }
    double c00 = m[4] * m[8] - m[5] * m[7];
    double c01 = m[5] * m[6] - m[3] * m[8];
    double c02 = m[3] * m[7] - m[4] * m[6];
    double det = m[0] * c00 + m[1] * c01 + m[2] * c02;
    if (det == 0.0) return false;
    r[0] = c00 / det;
    r[1] = (m[2] * m[7] - m[1] * m[8]) / det;
    r[2] = (m[1] * m[5] - m[2] * m[4]) / det;
    r[3] = c01 / det;
    r[4] = (m[0] * m[8] - m[2] * m[6]) / det;
    r[5] = (m[2] * m[3] - m[0] * m[5]) / det;
    r[6] = c02 / det;
    r[7] = (m[1] * m[6] - m[0] * m[7]) / det;
    r[8] = (m[0] * m[4] - m[1] * m[3]) / det;
    return true;
}

// obb_to_aabb * p (geometry.rs:203-205), accumulated column by column:
// r = M[:,0] p0; r += M[:,1] p1; ...
static void map_points(const double *pts, size_t n, int dim, const double *M, double *out) {
    for (size_t i = 0; i < n; ++i) {
        const double *p = pts + i * dim;
        for (int r = 0; r < dim; ++r) {
            double acc = M[r * dim + 0] * p[0];
            for (int c = 1; c < dim; ++c) acc = acc + M[r * dim + c] * p[c];
            out[i * dim + r] = acc;
        }
    }
}

}  // namespace

extern "C" {

// Rcb on AoS f64 points.  threads == 1: sequential and deterministic;
// otherwise OpenMP fork-join (0 = all threads).  Returns 0, or -1 for a bad
// dimension / weight type.
int oracle_rcb(uint64_t *part, uint64_t n, int dim, const double *pts, int wtype, const void *w,
               uint64_t iter_count, double tol, int mode, int fsum, int threads, oracle_stats *st) {
    return rcb_entry(part, n, dim, pts, wtype, w, iter_count, tol, mode, fsum, threads, st);
}

// The next oracle_rcb / oracle_rib call writes the position of the split of
// tree node h (heap numbering, root 0) to buf[h] for h < cap (nodes it does
// not split keep their value); buf == NULL stops recording.
void oracle_record_splits(double *buf, uint64_t cap) {
    g_split_buf = buf;
    g_split_cap = buf ? cap : 0;
}

// The weighted variant of the basis change (the GPU library's opt-in, no
// counterpart in coupe): centroid sum(w p) / sum(w), then sum(w (p-c)(p-c)^T),
// both sequential, then the same eigenvector, Householder and inverse.
int oracle_rib_matrix_weighted(uint64_t n, int dim, const double *pts, const double *w, double *obb_to_aabb) {
    if (dim != 2 && dim != 3) return -1;
    double c[3] = {0, 0, 0}, W = 0.0, m[9], v[3], h[9];
    for (size_t i = 0; i < n; ++i) {
        W += w[i];
        for (int d = 0; d < dim; ++d) c[d] += w[i] * pts[i * dim + d];
    }
    if (!(W > 0.0)) return -3;
    for (int d = 0; d < dim; ++d) c[d] = c[d] / W;
    for (int k = 0; k < dim * dim; ++k) m[k] = 0.0;
    for (size_t i = 0; i < n; ++i) {
        double o[3];
        for (int d = 0; d < dim; ++d) o[d] = pts[i * dim + d] - c[d];
        for (int a = 0; a < dim; ++a)
            for (int b = 0; b < dim; ++b) m[a * dim + b] += w[i] * o[a] * o[b];
    }
    inertia_vector(m, dim, v);
    householder(v, dim, h);
    if (!inverse(h, dim, obb_to_aabb)) return -2;
    return 0;
}

// The Rib basis change (OrientedBoundingBox::from_points, geometry.rs:210-228):
// writes obb_to_aabb (row-major dim x dim).
int oracle_rib_matrix(uint64_t n, int dim, const double *pts, double *obb_to_aabb) {
    if (dim != 2 && dim != 3) return -1;
    double m[9], v[3], h[9];
    inertia_matrix(pts, n, dim, m);
    inertia_vector(m, dim, v);
    householder(v, dim, h);
    if (!inverse(h, dim, obb_to_aabb)) return -2;
    return 0;
}

// rib (recursive_bisection.rs:829-851) with a given basis change: Rcb on the
// mapped points.  matrix == NULL computes it with oracle_rib_matrix.
int oracle_rib(uint64_t *part, uint64_t n, int dim, const double *pts, int wtype, const void *w,
               uint64_t iter_count, double tol, int mode, int fsum, int threads, const double *matrix,
               oracle_stats *st) {
    if (dim != 2 && dim != 3) return -1;
    if (n == 0) return 0;
    double M[9];
    if (matrix) {
        std::memcpy(M, matrix, sizeof(double) * dim * dim);
    } else {
        int rc = oracle_rib_matrix(n, dim, pts, M);
        if (rc) return rc;
    }
    std::vector<double> mapped(n * dim);
    map_points(pts, n, dim, M, mapped.data());
    return rcb_entry(part, n, dim, mapped.data(), wtype, w, iter_count, tol, mode, fsum, threads, st);
}

void oracle_map_points(const double *pts, uint64_t n, int dim, const double *M, double *out) {
    map_points(pts, n, dim, M, out);
}

void oracle_bbox(const double *pts, uint64_t n, int dim, double *bmin, double *bmax) {
    bbox_f64(pts, n, dim, bmin, bmax);
}

void oracle_inertia_matrix(const double *pts, uint64_t n, int dim, double *m) { inertia_matrix(pts, n, dim, m); }

void oracle_inertia_vector(const double *m, int dim, double *vec) { inertia_vector(m, dim, vec); }

void oracle_householder(const double *el, int dim, double *h) { householder(el, dim, h); }

int oracle_fixed_scale(const double *w, uint64_t n) { return fixed_scale_of(w, n); }

// Fixed-point sum of w[0..n) at scale s, converted back to f64.
double oracle_fixed_sum(const double *w, uint64_t n, int s) {
    i128 a = 0;
    for (uint64_t i = 0; i < n; ++i) a += fixed_q(w[i], s);
    return fixed_to_f64(a, s);
}

// One par_rcb_split on a 1-D f32 key array with u32 weights, as the
// reference's test_par_rcb_split drives it (recursive_bisection.rs:1041-1075):
// reorders keys/weights in place and returns the left size, weight_left and
// split_pos.
uint64_t oracle_split_f32_u32(float *keys, uint32_t *w, uint64_t n, double tol, float mn, float mx,
                              uint32_t *weight_left, float *split_pos) {
    // u32 weights behave like wrapping i32 for sums of this size; keep the
    // u32 compare of the reference by running the split on unsigned values.
    struct WU32 {
        typedef uint32_t S;
        typedef uint32_t V;
        typedef uint32_t A;
        static A zero() { return 0; }
        static A add(A a, S x, int) { return a + x; }
        static A merge(A a, A b) { return a + b; }
        static V fin(A a, int) { return a; }
        static V sub(V a, V b) { return a - b; }
        static bool less(V a, V b) { return a < b; }
        static double f64(V v) { return (double)v; }
    };
    std::vector<uint64_t> idx(n);
    for (uint64_t i = 0; i < n; ++i) idx[i] = i;
    Items<float, WU32> it;
    it.keys[0] = keys;
    it.keys[1] = it.keys[2] = nullptr;
    it.w = w;
    it.idx = idx.data();
    it.n = n;
    Ctx cx;
    std::memset(&cx, 0, sizeof(cx));
    cx.dim = 1;
    cx.tol = tol;
    cx.min_len = 4096;
    uint32_t sum = 0;
    for (uint64_t i = 0; i < n; ++i) sum += w[i];
    SplitOut<float, WU32> s = split<float, WU32>(cx, it, 0, mn, mx, sum);
    *weight_left = s.wl;
    *split_pos = s.split_pos;
    return s.nleft;
}

// reorder_split_scalar on a 1-D f32 array around keys[pivot]
// (recursive_bisection.rs:122-181); returns the left size.
uint64_t oracle_reorder_split_f32(float *keys, uint64_t n, uint64_t pivot) {
    std::vector<int32_t> w(n, 1);
    std::vector<uint64_t> idx(n);
    for (uint64_t i = 0; i < n; ++i) idx[i] = i;
    Items<float, WI32> it;
    it.keys[0] = keys;
    it.keys[1] = it.keys[2] = nullptr;
    it.w = w.data();
    it.idx = idx.data();
    it.n = n;
    return reorder_split(it, 1, pivot, 0);
}

}  // extern "C"
