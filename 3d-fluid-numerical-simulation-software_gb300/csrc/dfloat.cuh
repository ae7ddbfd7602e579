// Double-float arithmetic: a value held as the unevaluated sum hi + lo of two FP32 numbers with
// |lo| <= ulp(hi) / 2, about 47 significant bits, computed on the FP32 pipe.
//
// Why: GB300 executes an FP64 instruction (add, multiply, FMA or conversion) in about 70 cycles of
// one SM sub-partition, whatever the number of active lanes, and FP32 instructions at one per
// cycle. Where an FP64 kernel is bound by the latency of a short dependent chain on few warps (the
// LU-SGS hyperplane sweep), the same chain in double-float is several times shorter.
//
// The algorithms are the published error-free transformations and double-word operations:
//   TwoSum (Knuth, The Art of Computer Programming vol. 2, 4.2.2) and Fast2Sum (Dekker, "A
//   floating-point technique for extending the available precision", Numer. Math. 18, 1971);
//   TwoProd by a fused multiply-add; the double-word sum, product and product by a single word of
//   Joldes, Muller and Popescu, "Tight and rigorous error bounds for basic building blocks of
//   double-word arithmetic", ACM TOMS 44(2), 2017 (their AccurateDWPlusDW, DWTimesDW3 and
//   DWTimesFP3, relative errors below 3u^2, 4u^2 and 2u^2 with u = 2^-24);
//   the reciprocal and the square root by one Newton-Raphson (Heron) step in double-word
//   arithmetic from an FP32 seed that is itself refined to about 2^-24.
// Every FP32 operation is written with an explicitly rounded intrinsic, so that the compiler
// neither contracts a product and a sum into an FMA nor reassociates: the transformations are only
// error-free as written.
//
// Conversions from and to FP64 use integer operations only (an FP64 conversion instruction costs
// as much as an FP64 FMA): the 52-bit fraction of a double is cut into its top 23 bits (hi) and the
// next 23 bits, rounded (lo); the sum of a pair is assembled as a 53-bit integer significand.
// Values below 2^-126 in magnitude become zero and the low word of values below 2^-80 is dropped;
// infinities and NaNs pass through (the flow variables, geometry and fluxes of the solver lie far
// inside these bounds; a non-finite value stays non-finite so the solver's checks still see it).
#pragma once
#include <cuda_runtime.h>

namespace gbt {

struct dfloat {
    float hi, lo;
};

__device__ __forceinline__ dfloat df_make(float hi, float lo) { dfloat r; r.hi = hi; r.lo = lo; return r; }

// s + e = a + b exactly (any magnitudes)
__device__ __forceinline__ void two_sum(float a, float b, float &s, float &e)
{
    s = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}
// s + e = a + b exactly, given |a| >= |b| (or a = 0)
__device__ __forceinline__ void fast_two_sum(float a, float b, float &s, float &e)
{
    s = __fadd_rn(a, b);
    e = __fsub_rn(b, __fsub_rn(s, a));
}
__device__ __forceinline__ dfloat df_norm(float a, float b)
{
    dfloat r;
    fast_two_sum(a, b, r.hi, r.lo);
    return r;
}

__device__ __forceinline__ dfloat df_from(float x) { return df_make(x, 0.f); }

__device__ __forceinline__ dfloat df_from(double x)
{
    const unsigned long long b = (unsigned long long)__double_as_longlong(x);
    const unsigned hw = (unsigned)(b >> 32), lw = (unsigned)b;
    const unsigned sign = hw & 0x80000000u;
    const int e = (int)((hw >> 20) & 0x7ffu);                 // biased FP64 exponent
    dfloat r;
    if (e >= 897 && e <= 1150) {                              // 2^-126 <= |x| < 2^128
        const unsigned fh = ((hw & 0xfffffu) << 3) | (lw >> 29);          // fraction bits 51..29
        const float hi = __uint_as_float(sign | ((unsigned)(e - 896) << 23) | fh);
        float lo = 0.f;
        if (e >= 943) {                                       // |x| >= 2^-80: the low word is normal
            // fraction bits 28..0 rounded to 23 bits (m <= 2^23), as an FP32 integer (exact by the
            // 2^23 bias), times 2^(E - 46) with E the unbiased exponent, with the sign of x
            const unsigned m = ((lw & 0x1fffffffu) + 32u) >> 6;
            const float fm = __fsub_rn(__uint_as_float(0x4B000000u + m), 8388608.0f);
            lo = __fmul_rn(fm, __uint_as_float(sign | ((unsigned)(e - 942) << 23)));
        }
        r = df_norm(hi, lo);                                  // hi was truncated: round the pair
    } else if (e < 897) {
        r = df_make(__uint_as_float(sign), 0.f);
    } else {
        r = df_make(__double2float_rn(x), 0.f);               // infinities, NaN, |x| >= 2^128
    }
    return r;
}

// hi + lo rounded to FP64 (the low word's bits beyond the FP64 significand truncated: within one
// FP64 unit in the last place, far below the pair's own precision)
__device__ __forceinline__ double df_to_double(dfloat a)
{
    const unsigned hb = __float_as_uint(a.hi), lb = __float_as_uint(a.lo);
    const int eh = (int)((hb >> 23) & 0xffu), el = (int)((lb >> 23) & 0xffu);
    if (eh == 0) return __longlong_as_double((long long)((unsigned long long)(hb & 0x80000000u) << 32));   // +-0
    if (eh == 255) return (double)a.hi;                       // infinity or NaN (FP64 conversion, rare path)
    // hi's significand at bit 52 of a 53-bit integer, in units of 2^(eh - 127 - 52)
    unsigned long long S = (unsigned long long)((hb & 0x7fffffu) | 0x800000u) << 29;
    int E = eh + 896;                                         // biased FP64 exponent of hi
    if (el != 0) {
        const unsigned long long ml = (unsigned long long)((lb & 0x7fffffu) | 0x800000u);
        const int sh = el - eh + 29;                          // the low word's units relative to hi's
        unsigned long long L = 0;
        if (sh >= 0) L = ml << sh;                            // |lo| <= ulp_f32(hi) / 2 gives sh <= 5
        else if (sh > -25) L = (ml + (1ull << (-sh - 1))) >> (-sh);
        if ((hb ^ lb) & 0x80000000u) {
            S -= L;
            if (S < (1ull << 52)) { S <<= 1; E -= 1; }        // hi a power of two and lo of the other sign
        } else {
            S += L;                                           // stays below 2^53
        }
    }
    const unsigned long long bits = ((unsigned long long)(hb & 0x80000000u) << 32) |
                                    ((unsigned long long)E << 52) | (S & ((1ull << 52) - 1));
    return __longlong_as_double((long long)bits);
}

__device__ __forceinline__ dfloat operator-(dfloat a) { return df_make(-a.hi, -a.lo); }

// AccurateDWPlusDW
__device__ __forceinline__ dfloat operator+(dfloat x, dfloat y)
{
    float sh, sl, th, tl, vh, vl;
    two_sum(x.hi, y.hi, sh, sl);
    two_sum(x.lo, y.lo, th, tl);
    const float c = __fadd_rn(sl, th);
    fast_two_sum(sh, c, vh, vl);
    const float w = __fadd_rn(tl, vl);
    return df_norm(vh, w);
}
__device__ __forceinline__ dfloat operator-(dfloat x, dfloat y) { return x + (-y); }

// DWPlusFP
__device__ __forceinline__ dfloat operator+(dfloat x, float y)
{
    float sh, sl;
    two_sum(x.hi, y, sh, sl);
    const float v = __fadd_rn(x.lo, sl);
    return df_norm(sh, v);
}

// DWTimesDW3
__device__ __forceinline__ dfloat operator*(dfloat x, dfloat y)
{
    const float ch = __fmul_rn(x.hi, y.hi);
    const float cl1 = __fmaf_rn(x.hi, y.hi, -ch);
    const float tl0 = __fmul_rn(x.lo, y.lo);
    const float tl1 = __fmaf_rn(x.hi, y.lo, tl0);
    const float cl2 = __fmaf_rn(x.lo, y.hi, tl1);
    const float cl3 = __fadd_rn(cl1, cl2);
    return df_norm(ch, cl3);
}

// DWTimesFP3
__device__ __forceinline__ dfloat operator*(dfloat x, float y)
{
    const float ch = __fmul_rn(x.hi, y);
    const float cl1 = __fmaf_rn(x.hi, y, -ch);
    const float cl3 = __fmaf_rn(x.lo, y, cl1);
    return df_norm(ch, cl3);
}

// a power of two times a pair: exact
__device__ __forceinline__ dfloat df_scale(dfloat x, float p2) { return df_make(__fmul_rn(x.hi, p2), __fmul_rn(x.lo, p2)); }

// 1 / y: FP32 seed (hardware approximation plus one FP32 Newton step, about 2^-24 relative to
// 1 / y.hi), then one Newton step r (1 + e), e = 1 - y r, with e formed from the exact product
// y.hi r (TwoProd) and y.lo r: relative error about 2^-47
__device__ __forceinline__ dfloat df_rcp(dfloat y)
{
    float r;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(y.hi));
    r = __fmaf_rn(r, __fmaf_rn(-y.hi, r, 1.0f), r);
    const float ph = __fmul_rn(y.hi, r);
    float pl = __fmaf_rn(y.hi, r, -ph);
    pl = __fmaf_rn(y.lo, r, pl);
    const float e = __fsub_rn(__fsub_rn(1.0f, ph), pl);       // 1 - ph is exact (ph within 2^-22 of 1)
    return df_norm(r, __fmul_rn(r, e));
}
__device__ __forceinline__ dfloat operator/(dfloat x, dfloat y) { return x * df_rcp(y); }

// sqrt(x), x > 0: s0 the correctly rounded FP32 root of x.hi, then one Heron step
// s = s0 + (x - s0^2) / (2 s0) with x - s0^2 from the exact square (TwoProd): relative error about
// 2^-47. sqrt(0) = 0.
__device__ __forceinline__ dfloat df_sqrt(dfloat x)
{
    if (!(x.hi > 0.f)) return df_make(__fsqrt_rn(x.hi), 0.f);
    const float s0 = __fsqrt_rn(x.hi);
    float r;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(s0));
    const float ph = __fmul_rn(s0, s0);
    const float pl = __fmaf_rn(s0, s0, -ph);
    const float d = __fadd_rn(__fsub_rn(__fsub_rn(x.hi, ph), pl), x.lo);   // x.hi - ph is exact
    return df_norm(s0, __fmul_rn(d, __fmul_rn(0.5f, r)));
}

__device__ __forceinline__ bool operator<(dfloat a, dfloat b) { return a.hi < b.hi || (a.hi == b.hi && a.lo < b.lo); }
__device__ __forceinline__ bool operator>(dfloat a, dfloat b) { return b < a; }
__device__ __forceinline__ bool operator<=(dfloat a, dfloat b) { return !(b < a); }
__device__ __forceinline__ bool operator>=(dfloat a, dfloat b) { return !(a < b); }

// Conversions between FP32 and FP64 by integer operations, giving the same bits as the conversion
// instructions (which run on the FP64 pipe): f32_to_f64 is exact; f64_to_f32_rn rounds to nearest,
// ties to even. The rare operands outside the plain cases (FP32 subnormals, results in the FP32
// subnormal range, infinities, NaN) take the conversion instruction.
__device__ __forceinline__ double f32_to_f64(float f)
{
    const unsigned u = __float_as_uint(f);
    const unsigned e = (u >> 23) & 0xffu;
    const unsigned long long sign = (unsigned long long)(u & 0x80000000u) << 32;
    const unsigned long long frac = (unsigned long long)(u & 0x7fffffu) << 29;
    if (e == 0 && (u & 0x7fffffu) == 0) return __longlong_as_double((long long)sign);   // +-0
    if (e == 0 || e == 255) return (double)f;
    return __longlong_as_double((long long)(sign | ((unsigned long long)(e + 896) << 52) | frac));
}
__device__ __forceinline__ float f64_to_f32_rn(double x)
{
    const unsigned long long b = (unsigned long long)__double_as_longlong(x);
    const unsigned hw = (unsigned)(b >> 32), lw = (unsigned)b;
    const unsigned sign = hw & 0x80000000u;
    const int e = (int)((hw >> 20) & 0x7ffu);
    if (e >= 897 && e <= 1150) {                              // normal FP32 range (overflow rounds to inf)
        unsigned f = sign | ((unsigned)(e - 896) << 23) | ((hw & 0xfffffu) << 3) | (lw >> 29);
        const unsigned rest = lw & 0x1fffffffu, half = 0x10000000u;
        if (rest > half || (rest == half && (f & 1u))) f += 1u;   // a carry moves into the exponent
        return __uint_as_float(f);
    }
    if (e <= 872) return __uint_as_float(sign);               // |x| < 2^-150: rounds to +-0
    return __double2float_rn(x);
}

// pairs stored in place of FP64 values (8 bytes each, same alignment)
__device__ __forceinline__ dfloat df_load(const double *p)
{
    const float2 v = *reinterpret_cast<const float2 *>(p);
    return df_make(v.x, v.y);
}
__device__ __forceinline__ void df_store(double *p, dfloat a) { *reinterpret_cast<float2 *>(p) = make_float2(a.hi, a.lo); }

}  // namespace gbt
