// ffloat.cuh -- float-float ("double-float") arithmetic for FP64-accurate work off GB300's FP64
// pipe, which issues 2 lanes per clock per SM against 128 for FP32.
//
// A value is an unevaluated sum hi + lo of two floats (48 significant bits).  The operations
// follow the published error-free transformations: Knuth's two-sum, the FMA two-product, and
// the compensated dot product of Ogita, Rump and Oishi (2005) for sums of products; the
// reciprocal is one Newton step from the FP32 reciprocal.  Conversions from and to FP64 work on
// the bit patterns (integer pipe), for values in the normal float range.
#pragma once
#include <cstdint>

namespace lmtg {
namespace ff {

struct f2 {
    float h, l;
};

// s + e = a + b exactly
__device__ __forceinline__ void two_sum(float a, float b, float &s, float &e) {
    s = a + b;
    const float bb = s - a;
    e = (a - (s - bb)) + (b - bb);
}

// s + e = a + b exactly when |a| >= |b| (or a == 0)
__device__ __forceinline__ void fast_two_sum(float a, float b, float &s, float &e) {
    s = a + b;
    e = b - (s - a);
}

__device__ __forceinline__ f2 renorm(float s, float e) {
    f2 r;
    fast_two_sum(s, e, r.h, r.l);
    return r;
}

__device__ __forceinline__ f2 neg(f2 a) { return {-a.h, -a.l}; }

__device__ __forceinline__ f2 mul(f2 a, f2 b) {
    const float p = a.h * b.h;
    float e = fmaf(a.h, b.h, -p);
    e = fmaf(a.h, b.l, e);
    e = fmaf(a.l, b.h, e);
    return renorm(p, e);
}

// accurate sum (both parts' errors kept)
__device__ __forceinline__ f2 add(f2 a, f2 b) {
    float s, e, t, f;
    two_sum(a.h, b.h, s, e);
    two_sum(a.l, b.l, t, f);
    e += t;
    fast_two_sum(s, e, s, e);
    e += f;
    return renorm(s, e);
}

// 1 / a: the FP32 reciprocal refined by one Newton step, r = r0 + r0 (1 - a r0)
__device__ __forceinline__ f2 recip(f2 a) {
    const float r0 = 1.0f / a.h;
    const f2 e = add({1.0f, 0.0f}, neg(mul(a, {r0, 0.0f})));
    return renorm(r0, r0 * e.h);
}

// compensated sum of products: add(a, b) accumulates a * b, get() the rounded float-float total
struct Dot {
    float s = 0.f, c = 0.f;
    __device__ __forceinline__ void add(f2 a, f2 b) {
        const float p = a.h * b.h;
        float pl = fmaf(a.h, b.h, -p);
        pl = fmaf(a.h, b.l, pl);
        pl = fmaf(a.l, b.h, pl);
        float e;
        two_sum(s, p, s, e);
        c += e + pl;
    }
    __device__ __forceinline__ f2 get() const { return renorm(s, c); }
};

// d = hi + lo: hi the leading 24 significant bits (truncated), lo the next 29 rounded to float;
// zeros and values below 2^-126 give zeros (lo is dropped below 2^-74); inf, nan and values
// beyond the float range go through the conversion instruction (inf or nan)
__device__ __forceinline__ f2 split(double d) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(d);
    const unsigned top = (unsigned)(b >> 32), sign = top & 0x80000000u;
    const int ef = (int)((top >> 20) & 0x7ffu);
    const int eh = ef - 896;  // float exponent field of hi
    if (eh <= 0) return {__uint_as_float(sign), 0.f};
    if (eh >= 255) return {(float)d, 0.f};
    const float hi = __uint_as_float(sign | ((unsigned)eh << 23) | ((unsigned)(b >> 29) & 0x7fffffu));
    const unsigned rem = (unsigned)b & 0x1fffffffu;
    const int el = ef - 948;  // float exponent field of 2^(ef - 1075), the remainder's unit
    const float lo = (el > 0 && rem)
                         ? __uint_as_float(sign | __float_as_uint(__uint2float_rn(rem) * __uint_as_float((unsigned)el << 23)))
                         : 0.f;
    return {hi, lo};
}

// hi + lo (normalised, |lo| <= ulp(hi) / 2) to FP64, within two units of the last FP64 place
// (lo's bits below it are truncated); hi a normal float, zero (subnormals read as zero), inf
// or nan
__device__ __forceinline__ double to_double(f2 a) {
    const unsigned hb = __float_as_uint(a.h), lb = __float_as_uint(a.l);
    const int eh = (int)((hb >> 23) & 0xffu);
    if (eh == 0) return __longlong_as_double((long long)((unsigned long long)(hb & 0x80000000u) << 32));
    if (eh == 255) return (double)a.h;  // inf, nan
    // hi's significand in units of its FP64 last place 2^(eh - 127 - 52)
    const long long mh = (long long)(((unsigned long long)((hb & 0x7fffffu) | 0x800000u)) << 29);
    long long S = (hb >> 31) ? -mh : mh;
    const int el = (int)((lb >> 23) & 0xffu);
    if (el != 0) {
        const long long ml = (long long)((lb & 0x7fffffu) | 0x800000u);  // lo = ml 2^(el - 150)
        const int sh = el - eh + 29;                                        // <= 5 when normalised
        const long long L = sh >= 0 ? (ml << sh) : (sh > -40 ? (ml >> -sh) : 0ll);
        S += (lb >> 31) ? -L : L;
    }
    const unsigned long long sign = S < 0 ? (1ull << 63) : 0ull;
    unsigned long long M = S < 0 ? (unsigned long long)(-S) : (unsigned long long)S;
    long long E = eh - 127 + 1023;
    if (M >= (1ull << 53)) {
        M >>= 1;
        ++E;
    } else if (M < (1ull << 52)) {
        M <<= 1;
        --E;
    }
    return __longlong_as_double((long long)(sign | ((unsigned long long)E << 52) | (M & ((1ull << 52) - 1))));
}

}  // namespace ff
}  // namespace lmtg
