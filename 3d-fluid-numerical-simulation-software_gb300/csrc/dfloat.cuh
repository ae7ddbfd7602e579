// FP64 values split into pairs of FP32 numbers (hi + lo, |lo| <= ulp(hi) / 2, about 47 significant
// bits) and conversions between FP32 and FP64, all by integer and FP32 operations.
//
// Why: GB300 executes an FP64 instruction (add, multiply, FMA, or an FP32 <-> FP64 conversion) in
// about 70 cycles of one SM sub-partition, whatever the number of active lanes; integer and FP32
// instructions issue every cycle. The mixed form converts between its FP64 conserved variables and
// its FP32 working values in every cell of several kernels, and its residual norm forms a relative
// change of FP64 values per cell; done with these helpers they take no FP64-pipe instruction.
//
// The split of a double cuts its 52-bit fraction into the top 23 bits (hi) and the next 23 bits,
// rounded (lo), and renormalises the pair by Fast2Sum (Dekker, "A floating-point technique for
// extending the available precision", Numer. Math. 18, 1971). Values below 2^-126 in magnitude
// become zero and the low word of values below 2^-80 is dropped; infinities and NaNs pass through.
// The FP32 <-> FP64 conversions give the bits of the conversion instructions (round to nearest,
// ties to even); their rare operands outside the plain cases take the instruction itself.
#pragma once
#include <cuda_runtime.h>

namespace gbt {

struct dfloat {
    float hi, lo;
};

__device__ __forceinline__ dfloat df_make(float hi, float lo) { dfloat r; r.hi = hi; r.lo = lo; return r; }

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

}  // namespace gbt
