// Shared device/host definitions of the GB300 Rcb/Rib engine: key and weight
// arithmetic, the 128-bit fixed-point weight sums, ordered encodings for
// atomic min/max, and the per-segment record of a tree level.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <cmath>
#include <cstring>

#define CG_HD __host__ __device__ __forceinline__

namespace cg {

// ---------------------------------------------------------------------------
// Ordered unsigned encodings: a < b (IEEE, non-NaN) iff enc(a) < enc(b).
// -0.0 encodes just below +0.0.
// ---------------------------------------------------------------------------
CG_HD uint32_t ord_f32(float f) {
#ifdef __CUDA_ARCH__
    uint32_t b = __float_as_uint(f);
#else
    uint32_t b;
    memcpy(&b, &f, 4);
#endif
    return (b & 0x80000000u) ? ~b : (b | 0x80000000u);
}
CG_HD float unord_f32(uint32_t u) {
    uint32_t b = (u & 0x80000000u) ? (u & 0x7fffffffu) : ~u;
#ifdef __CUDA_ARCH__
    return __uint_as_float(b);
#else
    float f;
    memcpy(&f, &b, 4);
    return f;
#endif
}
CG_HD uint64_t ord_f64(double f) {
#ifdef __CUDA_ARCH__
    uint64_t b = (uint64_t)__double_as_longlong(f);
#else
    uint64_t b;
    memcpy(&b, &f, 8);
#endif
    return (b & 0x8000000000000000ull) ? ~b : (b | 0x8000000000000000ull);
}
CG_HD double unord_f64(uint64_t u) {
    uint64_t b = (u & 0x8000000000000000ull) ? (u & 0x7fffffffffffffffull) : ~u;
#ifdef __CUDA_ARCH__
    return __longlong_as_double((long long)b);
#else
    double f;
    memcpy(&f, &b, 8);
    return f;
#endif
}

// ---------------------------------------------------------------------------
// f64 -> f32 round-to-nearest-even from the IEEE-754 binary64/binary32
// definitions, in integer instructions only.  GB300 executes f64 instructions
// (including the f64 -> f32 conversion) at a small fraction of its integer
// rate, so per-point conversions are done this way.  NaN gives a quiet NaN.
// ---------------------------------------------------------------------------
CG_HD uint32_t f64bits_to_f32bits(uint64_t b) {
    const uint32_t sign = (uint32_t)(b >> 32) & 0x80000000u;
    const uint64_t x = b & 0x7fffffffffffffffull;
    if (x - (897ull << 52) < (254ull << 52)) {
        // f32 exponent 1..254 before rounding: rebias the exponent field and
        // round the 52-bit fraction to 23 bits, to nearest even; a carry out
        // of the fraction moves to the next binade (254 -> 255 is +inf)
        const uint64_t t = x - (896ull << 52);
        return sign | (uint32_t)((t + 0x0fffffffull + ((t >> 29) & 1)) >> 29);
    }
    const int e = (int)((b >> 52) & 0x7ff);
    const uint64_t m = b & 0x000fffffffffffffull;
    if (e == 0x7ff) return sign | (m ? 0x7fc00000u : 0x7f800000u);
    if (e == 0) return sign;  // f64 subnormals are far below half the least f32 subnormal
    const uint64_t M = m | (1ull << 52);  // value = M * 2^(e - 1075)
    const int E = e - 896;                // biased f32 exponent
    if (E >= 1) {
        uint64_t r = M >> 29;
        const uint64_t rem = M & ((1ull << 29) - 1), half = 1ull << 28;
        if (rem > half || (rem == half && (r & 1))) ++r;
        // r in [2^23, 2^24]; a carry to 2^24 bumps the exponent (also to inf)
        const uint64_t bits = ((uint64_t)E << 23) + (r - (1ull << 23));
        return bits >= 0x7f800000ull ? (sign | 0x7f800000u) : (sign | (uint32_t)bits);
    }
    // subnormal (or zero) f32: r = M * 2^(e - 926)
    const int sh = 926 - e;  // >= 30
    if (sh >= 64) return sign;
    uint64_t r = M >> sh;
    const uint64_t rem = M & ((1ull << sh) - 1), half = 1ull << (sh - 1);
    if (rem > half || (rem == half && (r & 1))) ++r;
    return sign | (uint32_t)r;  // r == 2^23 is the least normal, as encoded
}
// f32 -> f64 widening of a normal float or a zero in integer instructions
// (exact: rebias the exponent, extend the fraction); false for subnormals,
// infinities and NaN, which the caller widens with the f64 unit.
CG_HD bool f32bits_to_f64bits(uint32_t u, uint64_t &out) {
    const uint32_t e = (u >> 23) & 0xffu;
    const uint64_t sgn = (uint64_t)(u & 0x80000000u) << 32;
    if (e == 0) {
        if (u & 0x7fffffu) return false;
        out = sgn;
        return true;
    }
    if (e == 255) return false;
    out = sgn | ((uint64_t)(e + 896u) << 52) | ((uint64_t)(u & 0x7fffffu) << 29);
    return true;
}

CG_HD uint64_t f64_bits(double v) {
#ifdef __CUDA_ARCH__
    return (uint64_t)__double_as_longlong(v);
#else
    uint64_t b;
    memcpy(&b, &v, 8);
    return b;
#endif
}
CG_HD float f32_from_bits(uint32_t b) {
#ifdef __CUDA_ARCH__
    return __uint_as_float(b);
#else
    float f;
    memcpy(&f, &b, 4);
    return f;
#endif
}

// ---------------------------------------------------------------------------
// Key precision.  A key type has a stored form T, an arithmetic form A, and
// the per-point operations lt (IEEE `<`), isnan and approx (a float near the
// value, for bin guesses).  Arithmetic (cuts, distances) only happens per
// segment, on A.
//   KeyF32: coupe's arithmetic — f32 keys, `(min + max) / 2.0` in f32, f32
//           distances (recursive_bisection.rs:472-553, 674-679).
//   KeyF64: the same algorithm in f64.  Keys are stored in the order-
//           preserving u64 encoding, so that per-point comparisons are
//           integer comparisons; -0.0 is stored as +0.0 and every NaN as
//           the largest code, which keeps IEEE `<` semantics.
// ---------------------------------------------------------------------------
struct KeyF32 {
    typedef float T;
    typedef float C;  // cuts, interval bounds, pivots and boxes
    typedef float A;
    typedef uint32_t Ord;
    static constexpr bool BAND = false;
    static constexpr Ord ORD_INF = 0xff800000u;  // ord_f32(+inf)
    CG_HD static Ord ord(T k) { return ord_f32(k); }
    CG_HD static T unord(Ord u) { return unord_f32(u); }
    CG_HD static T from_f64(double v) { return (float)v; }
    CG_HD static T from_f64_bits(uint64_t b) { return f32_from_bits(f64bits_to_f32bits(b)); }
    CG_HD static A val(T k) { return k; }
    CG_HD static A inf() { return unord_f32(ORD_INF); }
    CG_HD static bool lt(T a, T b) { return a < b; }
    CG_HD static bool isnan(T k) { return !(k == k); }
    CG_HD static float approx(T k) { return k; }
    // recursive_bisection.rs:472 — (min + max) / 2.0 in f32
    CG_HD static T mid(T a, T b) { return (a + b) / 2.0f; }
    CG_HD static C cut_from_f64(double v) { return (float)v; }
    CG_HD static float approx_cut(C c) { return c; }
    CG_HD static C cmid(C a, C b) { return mid(a, b); }
    CG_HD static A cval(C c) { return c; }
};
struct KeyF64 {
    typedef uint64_t T;
    typedef uint64_t C;
    typedef double A;
    typedef uint64_t Ord;
    static constexpr bool BAND = false;
    static constexpr Ord ORD_INF = 0xfff0000000000000ull;  // code of +inf
    static constexpr T NAN_CODE = ~0ull;
    CG_HD static T enc_bits(uint64_t b) {
        if ((b & 0x7fffffffffffffffull) > 0x7ff0000000000000ull) return NAN_CODE;
        if (b == 0x8000000000000000ull) b = 0;  // -0.0 compares equal to +0.0
        return (b & 0x8000000000000000ull) ? ~b : (b | 0x8000000000000000ull);
    }
    CG_HD static Ord ord(T k) { return k; }
    CG_HD static T unord(Ord u) { return u; }
    CG_HD static T from_f64(double v) { return enc_bits(f64_bits(v)); }
    CG_HD static T from_f64_bits(uint64_t b) { return enc_bits(b); }
    CG_HD static A val(T k) { return k > ORD_INF ? unord_f64(0xfff8000000000000ull) : unord_f64(k); }
    CG_HD static A inf() { return unord_f64(ORD_INF); }
    CG_HD static bool isnan(T k) { return k > ORD_INF; }
    CG_HD static bool lt(T a, T b) { return a < b && b <= ORD_INF; }
    CG_HD static float approx(T k) {
        // a float near the value, by truncating the f64 fields (integers only)
        const uint64_t b = (k & 0x8000000000000000ull) ? (k & 0x7fffffffffffffffull) : ~k;
        const uint32_t s = (uint32_t)(b >> 32) & 0x80000000u;
        const int e = (int)((b >> 52) & 0x7ff) - 896;
        if (e <= 0) return f32_from_bits(s);
        if (e >= 255) return f32_from_bits(s | 0x7f800000u);
        return f32_from_bits(s | ((uint32_t)e << 23) | (uint32_t)((b >> 29) & 0x7fffffu));
    }
    // (a + b) / 2 in f64: the sum by the f64 unit, the halving of a normal
    // sum (exact) by decrementing its exponent field; zeros, subnormals,
    // the smallest normals, infinities and NaN by the f64 division
    CG_HD static T mid(T a, T b) {
        const double s = val(a) + val(b);
        const uint64_t sb = f64_bits(s);
        const uint64_t ex = (sb >> 52) & 0x7ffu;
        if (ex > 1 && ex < 0x7ffu) return enc_bits(sb - (1ull << 52));
        return from_f64(s / 2.0);
    }
    CG_HD static C cut_from_f64(double v) { return from_f64(v); }
    CG_HD static float approx_cut(C c) { return approx(c); }
    CG_HD static C cmid(C a, C b) { return mid(a, b); }
    CG_HD static A cval(C c) { return val(c); }
};

// Band form (COUPE_GPU_F32KEY_F64BAND): the f32 keys k = RN32(x) of the REF32
// form are streamed, while cuts, interval bounds, split positions and boxes
// are KeyF64 codes with KeyF64's f64 arithmetic, so every decision is the
// F64 form's.  For an f64 cut c, k < RD32(c) implies x < c and k > RU32(c)
// implies x >= c; only k in [RD32(c), RU32(c)] needs the f64 coordinate,
// which is then read from the input (the band).  The per-bin minimum is kept
// on keys; the exact f64 minimum is fetched only when a stop test needs it.
// Deliberately no lt / mid / val: keys and cuts never meet without the band.
struct KeyBand {
    typedef float T;
    typedef uint64_t C;
    typedef double A;
    typedef uint32_t Ord;
    static constexpr bool BAND = true;
    static constexpr Ord ORD_INF = 0xff800000u;  // ord_f32(+inf)
    CG_HD static Ord ord(T k) { return ord_f32(k); }
    CG_HD static T unord(Ord u) { return unord_f32(u); }
    CG_HD static T from_f64_bits(uint64_t b) { return KeyF32::from_f64_bits(b); }
    CG_HD static bool isnan(T k) { return !(k == k); }
    CG_HD static float approx(T k) { return k; }
    CG_HD static A inf() { return KeyF64::inf(); }
    CG_HD static C cut_from_f64(double v) { return KeyF64::from_f64(v); }
    CG_HD static float approx_cut(C c) { return KeyF64::approx(c); }
    CG_HD static C cmid(C a, C b) { return KeyF64::mid(a, b); }
    CG_HD static A cval(C c) { return KeyF64::val(c); }
    CG_HD static bool clt(C a, C b) { return KeyF64::lt(a, b); }
};

// f32 bounds of an f64 cut code: RD32(c) and RU32(c) (equal when c is an f32).
struct CutBounds {
    float lo, hi;
};
CG_HD float f32_step(float f, int dir) {  // the neighbouring float (ordered codes are consecutive)
    return unord_f32(ord_f32(f) + (uint32_t)dir);
}
CG_HD CutBounds band_bounds(uint64_t code) {
    const double c = KeyF64::val(code);
    const uint32_t rb = f64bits_to_f32bits(f64_bits(c));
    const float r = f32_from_bits(rb);  // RN32(c)
    // the sign of (double)r - c: from the ordered codes when r widens in
    // integers and c is not NaN (codes order as the values do, -0 as +0),
    // else by the f64 unit (NaN compares neither equal nor less)
    int cmp;
    uint64_t rdb;
    if (code <= KeyF64::ORD_INF && f32bits_to_f64bits(rb, rdb)) {
        const uint64_t rc = KeyF64::enc_bits(rdb);
        cmp = rc == code ? 0 : (rc < code ? -1 : 1);
    } else {
        const double rd = (double)r;
        cmp = rd == c ? 0 : (rd < c ? -1 : 1);
    }
    CutBounds b;
    if (cmp == 0) {
        b.lo = b.hi = r;
    } else if (cmp < 0) {
        b.lo = r;
        b.hi = f32_step(r, 1);
    } else {
        b.lo = f32_step(r, -1);
        b.hi = r;
    }
    return b;
}
// -1: the key proves x < c; +1: it proves x >= c; 0: the band (NaN keys too)
CG_HD int band_side(float k, const CutBounds &b) { return k < b.lo ? -1 : (k > b.hi ? 1 : 0); }
// Closed f64 interval holding every x with RN32(x) == k (k not NaN): the
// midpoints to the neighbouring floats, or beyond the largest float for +-inf.
CG_HD void band_interval(float k, double &xl, double &xh) {
    const uint32_t o = ord_f32(k);
    const double inf = KeyF64::val(KeyF64::ORD_INF);
    if (o >= 0xff800000u) {  // +inf
        xl = (double)unord_f32(o - 1);
        xh = inf;
    } else if (o <= 0x007fffffu) {  // -inf
        xl = -inf;
        xh = (double)unord_f32(o + 1);
    } else {
        const double kd = (double)k;
        xl = (kd + (double)unord_f32(o - 1)) / 2.0;
        xh = (kd + (double)unord_f32(o + 1)) / 2.0;
    }
}

// ---------------------------------------------------------------------------
// 128-bit fixed-point sums of f64 weights.  For n weights whose largest
// magnitude A satisfies 2^(e-1) <= A < 2^e, the scale is
// s = 126 - e - ceil(log2 n); each weight becomes q = round_half_even(w 2^s)
// as a two's-complement 128-bit integer, so that any sum of at most n terms
// stays below 2^126 in magnitude and integer addition makes every sum
// independent of its order.  A sum Q is read back as an f64 by rounding |Q|
// to 53 significant bits (half to even) and scaling by 2^-s.
// ---------------------------------------------------------------------------
CG_HD int ceil_log2_u64(uint64_t n) {
    int l = 0;
    while (l < 63 && (1ull << l) < n) ++l;
    return l;
}

CG_HD int fixed_scale_from_max(double amax, uint64_t n) {
    if (!(amax > 0.0)) return 0;
    int e;
    frexp(amax, &e);
    return 126 - e - ceil_log2_u64(n);
}

// q(w) from the binary64 fields (integer instructions only: it runs per item).
CG_HD unsigned __int128 fixed_q_bits(double w, int s) {
    uint64_t bits;
#ifdef __CUDA_ARCH__
    bits = (uint64_t)__double_as_longlong(w);
#else
    memcpy(&bits, &w, 8);
#endif
    const int be = (int)((bits >> 52) & 0x7ff);
    const uint64_t frac = bits & 0x000fffffffffffffull;
    if (be == 0 && frac == 0) return 0;
    // |w| 2^s = m 2^x with m < 2^53
    const uint64_t m = be ? (frac | (1ull << 52)) : frac;
    const int x = (be ? be - 1075 : -1074) + s;
    const bool neg = (bits >> 63) != 0;
    unsigned __int128 q;
    if (x >= 0) {
        q = (unsigned __int128)m << x;
    } else {
        int r = -x;
        if (r >= 54) {
            q = 0;
        } else {
            uint64_t qi = m >> r;
            uint64_t rem = m & ((1ull << r) - 1);
            uint64_t half = 1ull << (r - 1);
            if (rem > half || (rem == half && (qi & 1))) ++qi;
            q = qi;
        }
    }
    return neg ? (unsigned __int128)0 - q : q;
}

CG_HD int clz128(unsigned __int128 a) {
    uint64_t hi = (uint64_t)(a >> 64), lo = (uint64_t)a;
#ifdef __CUDA_ARCH__
    return hi ? __clzll((long long)hi) : 64 + __clzll((long long)lo);
#else
    return hi ? __builtin_clzll(hi) : (lo ? 64 + __builtin_clzll(lo) : 128);
#endif
}

CG_HD double fixed_to_f64(unsigned __int128 Qbits, int s) {
    if (Qbits == 0) return 0.0;
    bool neg = (Qbits >> 127) != 0;
    unsigned __int128 a = neg ? (unsigned __int128)0 - Qbits : Qbits;
    int hb = 127 - clz128(a);
    uint64_t m;
    int x = 0;
    if (hb <= 52) {
        m = (uint64_t)a;
    } else {
        int sh = hb - 52;
        m = (uint64_t)(a >> sh);
        unsigned __int128 rem = a & (((unsigned __int128)1 << sh) - 1);
        unsigned __int128 half = (unsigned __int128)1 << (sh - 1);
        if (rem > half || (rem == half && (m & 1))) ++m;
        if (m == (1ull << 53)) {
            m >>= 1;
            ++sh;
        }
        x = sh;
    }
    // |value| = m 2^(x - s) with m < 2^53: a normal result is assembled
    // from its fields (no FP64 instruction), the rest by ldexp
    const int hm = 63 - (hb <= 52 ? clz128((unsigned __int128)m) - 64 : 11);  // top bit of m
    const int e = x - s + hm;                                                    // unbiased exponent
    if (e >= -1022 && e <= 1023) {
        const uint64_t mn = m << (52 - hm);  // in [2^52, 2^53), exact
        const uint64_t b = ((uint64_t)(e + 1023) << 52) | (mn & 0x000fffffffffffffull) | (neg ? 1ull << 63 : 0);
#ifdef __CUDA_ARCH__
        return __longlong_as_double((long long)b);
#else
        double r;
        memcpy(&r, &b, 8);
        return r;
#endif
    }
    double r = ldexp((double)m, x - s);
    return neg ? -r : r;
}

// ---------------------------------------------------------------------------
// Weight arithmetic (coupe's RcbWeight, recursive_bisection.rs:708-722, with
// release-build wrapping for integers).  Sums are accumulated in LIMBS
// unsigned 64-bit words so that atomics can add them in any order:
//   int32:  one word, the low 32 bits are the wrapped i32 sum;
//   int64:  one word, the wrapped i64 sum;
//   double: four words holding 32-bit chunks of the 128-bit fixed-point q,
//           recombined with carries (exact while fewer than 2^32 terms).
// V values travel through the segment table as 64 raw bits.
// ---------------------------------------------------------------------------
struct WtI32 {
    typedef int32_t S;
    typedef int32_t V;
    static constexpr int LIMBS = 1;
    static constexpr int CODE = 0;  // COUPE_INT
    CG_HD static void limbs(S w, int, uint64_t *l) { l[0] = (uint32_t)w; }
    CG_HD static V value(const uint64_t *l, int) { return (int32_t)(uint32_t)l[0]; }
    CG_HD static V sub(V a, V b) { return (int32_t)((uint32_t)a - (uint32_t)b); }
    CG_HD static bool less(V a, V b) { return a < b; }
    CG_HD static double f64(V v) { return (double)v; }
    CG_HD static uint64_t bits(V v) { return (uint64_t)(uint32_t)v; }
    CG_HD static V from_bits(uint64_t b) { return (int32_t)(uint32_t)b; }
};
struct WtI64 {
    typedef int64_t S;
    typedef int64_t V;
    static constexpr int LIMBS = 1;
    static constexpr int CODE = 1;  // COUPE_INT64
    CG_HD static void limbs(S w, int, uint64_t *l) { l[0] = (uint64_t)w; }
    CG_HD static V value(const uint64_t *l, int) { return (int64_t)l[0]; }
    CG_HD static V sub(V a, V b) { return (int64_t)((uint64_t)a - (uint64_t)b); }
    CG_HD static bool less(V a, V b) { return a < b; }
    CG_HD static double f64(V v) { return (double)v; }
    CG_HD static uint64_t bits(V v) { return (uint64_t)v; }
    CG_HD static V from_bits(uint64_t b) { return (int64_t)b; }
};
// Integer weights that all lie in [0, 2^16), stored in 16 bits for the level
// loop (less traffic per item); sums and values follow Base (WtI32: wrapped
// i32 sums, WtI64: i64 sums), so results are those of Base.
template <class Base>
struct WtC16 {
    typedef uint16_t S;
    typedef typename Base::V V;
    static constexpr int LIMBS = 1;
    static constexpr int CODE = Base::CODE;
    CG_HD static void limbs(S w, int, uint64_t *l) { l[0] = w; }
    CG_HD static V value(const uint64_t *l, int s) { return Base::value(l, s); }
    CG_HD static V sub(V a, V b) { return Base::sub(a, b); }
    CG_HD static bool less(V a, V b) { return Base::less(a, b); }
    CG_HD static double f64(V v) { return Base::f64(v); }
    CG_HD static uint64_t bits(V v) { return Base::bits(v); }
    CG_HD static V from_bits(uint64_t b) { return Base::from_bits(b); }
};
struct WtF64 {
    typedef double S;
    typedef double V;
    static constexpr int LIMBS = 4;
    static constexpr int CODE = 2;  // COUPE_DOUBLE
    CG_HD static void limbs(S w, int s, uint64_t *l) {
        unsigned __int128 q = fixed_q_bits(w, s);
        l[0] = (uint32_t)q;
        l[1] = (uint32_t)(q >> 32);
        l[2] = (uint32_t)(q >> 64);
        l[3] = (uint32_t)(q >> 96);
    }
    CG_HD static unsigned __int128 combine(const uint64_t *l) {
        return (unsigned __int128)l[0] + ((unsigned __int128)l[1] << 32) + ((unsigned __int128)l[2] << 64) +
               ((unsigned __int128)l[3] << 96);
    }
    CG_HD static V value(const uint64_t *l, int s) { return fixed_to_f64(combine(l), s); }
    CG_HD static V sub(V a, V b) { return a - b; }
    CG_HD static bool less(V a, V b) { return a < b; }
    CG_HD static double f64(V v) { return v; }
    CG_HD static uint64_t bits(V v) {
#ifdef __CUDA_ARCH__
        return (uint64_t)__double_as_longlong(v);
#else
        uint64_t b;
        memcpy(&b, &v, 8);
        return b;
#endif
    }
    CG_HD static V from_bits(uint64_t b) {
#ifdef __CUDA_ARCH__
        return __longlong_as_double((long long)b);
#else
        double v;
        memcpy(&v, &b, 8);
        return v;
#endif
    }
};

// ---------------------------------------------------------------------------
// One segment of a tree level (a contiguous range of the reordered arrays).
// ---------------------------------------------------------------------------
enum : uint32_t { SEG_ACTIVE = 0, SEG_DONE = 1, SEG_ALLLEFT = 2 };

template <class KT>
struct Seg {
    typedef typename KT::C K;
    uint64_t off;    // first item
    uint64_t voff;   // first item in the level's list of items still being split (off, when none has left)
    uint64_t heap;   // heap id: children of h are 2h+1 and 2h+2 (wrapping)
    uint64_t sum;    // weight sum (V bits)
    uint64_t prev;   // prev_count_left of the split loop (UINT64_MAX first)
    uint64_t wl;     // result: weight_left (V bits)
    uint32_t n;      // items
    uint32_t nleft;  // result: items sent left
    uint32_t state;  // SEG_*
    uint32_t steps;  // bisection steps taken so far
    uint32_t child;  // index of the first non-empty child in the next level
    uint32_t xstate; // band form: X_PENDING when xmin holds an exact minimum
    uint32_t xkey;   // band form: the f32 key (ordered) whose exact minimum xmin is
    uint32_t set;    // point set of the run the segment belongs to
    // f64 weights binned approximately (see k_hist): the exact sums come
    // from xq, the segment's own fixed-point sum (chunks of 32 bits, summed
    // by the level's first pass)
    uint32_t sumx;    // SUMX_*: how the first decide pass of the level sets `sum`
    uint32_t exactw;  // 1: the next passes bin exact fixed-point weights
    uint32_t wlx;     // 1: wl is exact (set with a split)
    uint32_t pad2;
    uint64_t xq[4];
    uint64_t xcut;   // band form: ... among the items at or right of this cut
    uint64_t xmin;   // band form: that minimum (f64 ordered code)
    K lo, hi;        // current search interval on this level's axis
    K pivot;         // result: items with key < pivot go left
    K split_pos;     // result: the cut position
    K bmin[3], bmax[3];
};

enum : uint32_t {
    SUMX_NONE = 0,   // sum is exact
    SUMX_OWN = 1,    // sum = the items' own fixed-point sum (a left child)
    SUMX_RIGHT = 2,  // sum = parent sum - left sibling's (segment index - 1) own sum
};

// One finished split as the final traversal needs it: items with
// (flags & TRAV_ALLLEFT) or key < pivot went to the left child.  `next` is
// the index of the first child in the next level's segment list, or on the
// last level the split segment's heap id.
enum : uint32_t { TRAV_ALLLEFT = 1u, TRAV_HAS_LEFT = 2u };

template <class KT>
struct Trav {
    typename KT::C pivot;
    uint32_t flags;
    uint64_t next;
    float blo, bhi;  // band form: RD32 / RU32 of the pivot
};

constexpr int MAX_TRAV_LEVELS = 63;
struct LevelOffsets {
    uint64_t off[MAX_TRAV_LEVELS];
};

// The point sets of a run: independent Rcb problems over consecutive item
// ranges of the input, each with its own iteration count.  One set: its
// totals live in RunScalars and these arrays are not read.
struct SetTab {
    uint32_t count;
    const uint64_t *off;    // [count + 1] first item of each set, input order
    const uint32_t *iters;  // [count] the set's iter_count
    const uint32_t *root;   // [count] index of the set's root segment on level 0 (~0u: none)
    uint64_t *bmin, *bmax;  // [count * 3] bounding box, ordered f64 codes
    uint64_t *wsum;         // [count * 4] weight sum limbs
    uint64_t *wabs;         // [count] largest |w| as raw f64 bits (f64 weights)
    int32_t *fs;            // [count] fixed-point scale (f64 weights)
    int32_t *qb;            // [count] shift of the approximate binned weights (f64 weights)
    uint64_t *minheap;      // [count] smallest heap id among the set's parts
};

// Error bits raised by kernels (read by the host after each synchronisation).
enum : uint32_t {
    ERR_LOOKBACK_TIMEOUT = 1u,
    ERR_SCATTER_BOUNDS = 2u,
    ERR_NONFINITE_WEIGHT = 4u,
    ERR_COUNT_MISMATCH = 8u,
    ERR_TILE_PERM = 16u,  // a reorder tile's permutation left its range
    ERR_COPY_TIMEOUT = 32u,  // a bulk copy into shared memory did not complete within its bounded wait
};

// Device-side scalars of one run.
struct RunScalars {
    uint64_t bbox_min_ord[3];
    uint64_t bbox_max_ord[3];
    uint64_t wabs_max_bits;   // largest |w| as raw f64 bits (f64 weights)
    uint64_t wsum_limbs[4];   // total weight
    uint64_t nactive;         // segments still searching after a decide pass
    uint64_t total_active;    // items in those segments
    uint64_t nsegs_next;      // non-empty children of the level
    uint64_t min_heap;        // smallest heap id of the last level
    uint64_t ticket;          // dynamic chunk counter of the reorder
    uint64_t steps_total;     // bisection steps summed over finished splits
    uint64_t steps_max;
    uint64_t splits;
    uint32_t err;
    int32_t fscale;
    uint32_t wide;      // nonzero: some weight is not an integer in [0, 2^20)
    uint32_t narrow16;  // nonzero: some integer weight is not in [0, 2^16)
    uint64_t diag[4];      // details of the first failed device check
    uint64_t pass_points;  // points read by refinement passes (sum over scans)
    uint32_t nexact;       // band form: decisions that waited for an exact minimum
    uint32_t pad2;
    unsigned long long band_points;  // band form: f64 coordinates read
    uint64_t items_next;             // items of the next level's segments
    uint32_t fneg;                   // f64 weights: some weight is negative
    int32_t qb;                      // f64 weights, one set: shift of the approximate binned weights
    uint32_t fapprox;                // f64 weights: bins hold approximate weights (see k_hist)
    uint32_t nexactw;                // decisions that needed exact f64 weight sums
    uint32_t decide_done;            // CTAs of the running k_decide that finished (reset by the last)
    uint32_t stall;                  // queued run: level + 1 whose splits need more passes than queued
};

// A queued kernel has nothing to do after a device check failed or a split
// needed more passes than were queued (the host finishes the run).
__host__ __device__ __forceinline__ bool run_halted(const RunScalars *rs) { return (rs->err | rs->stall) != 0; }

// ---------------------------------------------------------------------------
// f32 pairs: a value as hi + lo (|lo| <= ulp(hi)/2), with error-free sums
// and fused-multiply-add products (Dekker 1971, Shewchuk 1997); about 44
// significant bits at f32 speed.  GB300's FP64 pipe runs at 1/64 of the f32
// rate, so per-point f64 arithmetic is replaced by these where the result
// needs only a bounded error (or a bound decides it exactly).  They rely on
// f32 operations rounding to nearest one at a time (no contraction: the
// library is built with -fmad=false).
// ---------------------------------------------------------------------------
struct F2 {
    float h, l;
};
__device__ __forceinline__ F2 f2_two_sum(float a, float b) {
    const float s = a + b, v = s - a;
    return {s, (a - (s - v)) + (b - v)};
}
__device__ __forceinline__ F2 f2_fast(float a, float b) {  // |a| >= |b| or a == 0
    const float s = a + b;
    return {s, b - (s - a)};
}
__device__ __forceinline__ F2 f2_sub(F2 a, F2 b) {
    const F2 s = f2_two_sum(a.h, -b.h);
    return f2_fast(s.h, s.l + (a.l - b.l));
}
__device__ __forceinline__ F2 f2_mul(F2 a, F2 b) {
    const float p = a.h * b.h;
    float e = fmaf(a.h, b.h, -p);
    e = fmaf(a.h, b.l, e);
    e = fmaf(a.l, b.h, e);
    return f2_fast(p, e);
}
__device__ __forceinline__ void f2_add(F2 &acc, F2 x) {
    const F2 s = f2_two_sum(acc.h, x.h);
    acc = f2_fast(s.h, s.l + (acc.l + x.l));
}
// x as an f32 pair; false when |x| lies outside [2^-50, 2^50] (zeros pass)
__device__ __forceinline__ bool f2_split(double x, F2 &r) {
    const uint64_t b = (uint64_t)__double_as_longlong(x);
    const int e = (int)((b >> 52) & 0x7ff);
    if ((b << 1) == 0) {
        r = {0.0f, 0.0f};
        return true;
    }
    if (e < 1023 - 50 || e > 1023 + 50) return false;
    const uint64_t M = (b & 0x000fffffffffffffull) | (1ull << 52);  // |x| = M 2^(e - 1075)
    const uint64_t H = (M + 0x0fffffffull + ((M >> 29) & 1)) >> 29;  // RN(M / 2^29), at most 2^24
    const int32_t R = (int32_t)((int64_t)M - (int64_t)(H << 29));    // |R| <= 2^28
    const float sh = __uint_as_float((uint32_t)(e - 1046 + 127) << 23);  // 2^(e - 1046)
    const float sl = __uint_as_float((uint32_t)(e - 1075 + 127) << 23);  // 2^(e - 1075)
    float h = (float)(uint32_t)H * sh, l = (float)R * sl;  // exact scalings; (float)R rounds to nearest
    if (b >> 63) {
        h = -h;
        l = -l;
    }
    r = {h, l};
    return true;
}

}  // namespace cg
