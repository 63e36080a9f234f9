// hos_f32x2.cuh -- two FP32 lanes in one register pair, computed with Blackwell's paired FP32
// instructions (fma / add / mul / sub .f32x2): one issue slot performs the operation on both
// lanes.  The FP32 face kernels are issue bound, so the hot arithmetic (the GKS flux of two
// Gauss points, the linear reconstruction of two variables) runs on F2 values.
//
// Every lane rounds as the scalar FP32 operation of that lane.  A product is kept unevaluated
// (P2) until it meets an addition, so a * b + c becomes one fused multiply-add as in the
// contracted scalar code; a product used on its own is rounded by a paired multiply.  The paired
// instructions take no negated operands (a negated pair costs two scalar instructions), so a
// difference with a product is a paired multiply and a paired subtraction, and -x is 0 - x.
// Transcendental functions, square roots and divisions run per lane with the scalar FP32
// routines.
#pragma once
#include <cuda_runtime.h>

namespace hos {

struct F2 {
    float2 v;
    F2() = default;
    __device__ __forceinline__ F2(float2 a) : v(a) {}
    __device__ __forceinline__ F2(float a, float b) : v(make_float2(a, b)) {}
    // broadcasts: T(c) of the templated math gives the same constant in both lanes
    __device__ __forceinline__ explicit F2(double a) : v(make_float2((float)a, (float)a)) {}
    __device__ __forceinline__ explicit F2(float a) : v(make_float2(a, a)) {}
    __device__ __forceinline__ explicit F2(int a) : v(make_float2((float)a, (float)a)) {}
};

namespace f2op {
__device__ __forceinline__ F2 fma(F2 a, F2 b, F2 c) { return F2(__ffma2_rn(a.v, b.v, c.v)); }
__device__ __forceinline__ F2 add(F2 a, F2 b) { return F2(__fadd2_rn(a.v, b.v)); }
__device__ __forceinline__ F2 mul(F2 a, F2 b) { return F2(__fmul2_rn(a.v, b.v)); }
__device__ __forceinline__ F2 sub(F2 a, F2 b) {
    unsigned long long d;
    asm("sub.rn.ftz.f32x2 %0, %1, %2;"
        : "=l"(d)
        : "l"(*reinterpret_cast<const unsigned long long*>(&a.v)), "l"(*reinterpret_cast<const unsigned long long*>(&b.v)));
    return F2(*reinterpret_cast<const float2*>(&d));
}
}  // namespace f2op

// an unevaluated product a * b
struct P2 {
    F2 a, b;
    __device__ __forceinline__ operator F2() const { return f2op::mul(a, b); }
};

__device__ __forceinline__ F2 operator-(F2 a) { return f2op::sub(F2(0.0f), a); }
__device__ __forceinline__ F2 operator-(P2 p) { return -F2(p); }

__device__ __forceinline__ P2 operator*(F2 a, F2 b) { return P2{a, b}; }
__device__ __forceinline__ P2 operator*(P2 p, F2 b) { return P2{F2(p), b}; }
__device__ __forceinline__ P2 operator*(F2 a, P2 q) { return P2{a, F2(q)}; }
__device__ __forceinline__ P2 operator*(P2 p, P2 q) { return P2{F2(p), F2(q)}; }

__device__ __forceinline__ F2 operator+(F2 a, F2 b) { return f2op::add(a, b); }
__device__ __forceinline__ F2 operator+(P2 p, F2 c) { return f2op::fma(p.a, p.b, c); }
__device__ __forceinline__ F2 operator+(F2 c, P2 p) { return f2op::fma(p.a, p.b, c); }
__device__ __forceinline__ F2 operator+(P2 p, P2 q) { return f2op::fma(p.a, p.b, F2(q)); }

__device__ __forceinline__ F2 operator-(F2 a, F2 b) { return f2op::sub(a, b); }
__device__ __forceinline__ F2 operator-(P2 p, F2 c) { return f2op::sub(F2(p), c); }
__device__ __forceinline__ F2 operator-(F2 c, P2 p) { return f2op::sub(c, F2(p)); }
__device__ __forceinline__ F2 operator-(P2 p, P2 q) { return f2op::sub(F2(p), F2(q)); }

__device__ __forceinline__ F2 operator/(F2 a, F2 b) { return F2(a.v.x / b.v.x, a.v.y / b.v.y); }
__device__ __forceinline__ F2 operator/(P2 p, F2 b) { return F2(p) / b; }
__device__ __forceinline__ F2 operator/(F2 a, P2 q) { return a / F2(q); }
__device__ __forceinline__ F2 operator/(P2 p, P2 q) { return F2(p) / F2(q); }

__device__ __forceinline__ F2& operator+=(F2& a, F2 b) { return a = a + b; }
__device__ __forceinline__ F2& operator+=(F2& a, P2 p) { return a = a + p; }
__device__ __forceinline__ F2& operator-=(F2& a, F2 b) { return a = a - b; }
__device__ __forceinline__ F2& operator*=(F2& a, F2 b) { return a = F2(a * b); }

// per-lane functions (the global FP32 / FP64 overloads stay visible beside them)
using ::sqrt;
__device__ __forceinline__ F2 sqrt(F2 a) { return F2(sqrtf(a.v.x), sqrtf(a.v.y)); }

// exp and erfc of the GKS flux.  FP64 keeps the library functions.  The FP32 forms avoid the
// conversion instructions of the library's expf / erfcf, which GB300 executes on its narrow FP64
// pipe: exp is the hardware base-2 exponential (__expf; error 2 + 1.2 |x| ulp, where the flux
// takes exp of arguments of a few tens at most, giving absolute errors far below the FP32
// rounding of the terms they multiply), and erfc is the Chebyshev-fitted form of Press et al.,
// Numerical Recipes in C, 2nd ed., section 6.2 (erfcc, fractional error below 1.2e-7):
//   erfc(z) = t exp(-z^2 + P(t)),  t = 1 / (1 + z / 2),  z >= 0,  erfc(-z) = 2 - erfc(z).
__device__ __forceinline__ double fexp(double x) { return exp(x); }
__device__ __forceinline__ float fexp(float x) { return __expf(x); }
__device__ __forceinline__ F2 fexp(F2 a) { return F2(__expf(a.v.x), __expf(a.v.y)); }
// P(t) of the fitted form, Horner from the highest coefficient
template <class T>
__device__ __forceinline__ T erfc_poly(T t) {
    T p = T(0.17087277) * t + T(-0.82215223);
    p = p * t + T(1.48851587);
    p = p * t + T(-1.13520398);
    p = p * t + T(0.27886807);
    p = p * t + T(-0.18628806);
    p = p * t + T(0.09678418);
    p = p * t + T(0.37409196);
    p = p * t + T(1.00002368);
    return p * t + T(-1.26551223);
}
__device__ __forceinline__ double ferfc(double x) { return erfc(x); }
__device__ __forceinline__ float ferfc(float x) {
    const float z = fabsf(x), t = 1.0f / (1.0f + 0.5f * z);
    const float r = t * __expf(erfc_poly(t) - z * z);
    return x >= 0.0f ? r : 2.0f - r;
}
__device__ __forceinline__ F2 ferfc(F2 a) {
    const F2 z(fabsf(a.v.x), fabsf(a.v.y));
    const F2 t(1.0f / (1.0f + 0.5f * z.v.x), 1.0f / (1.0f + 0.5f * z.v.y));
    const F2 q = erfc_poly(t) - z * z;
    const F2 r = t * F2(__expf(q.v.x), __expf(q.v.y));
    return F2(a.v.x >= 0.0f ? r.v.x : 2.0f - r.v.x, a.v.y >= 0.0f ? r.v.y : 2.0f - r.v.y);
}
__device__ __forceinline__ F2 fabsT(F2 a) { return F2(fabsf(a.v.x), fabsf(a.v.y)); }
__device__ __forceinline__ F2 fminT(F2 a, F2 b) { return F2(fminf(a.v.x, b.v.x), fminf(a.v.y, b.v.y)); }
__device__ __forceinline__ F2 fmaxT(F2 a, F2 b) { return F2(fmaxf(a.v.x, b.v.x), fmaxf(a.v.y, b.v.y)); }

// FP32 -> FP64 conversion on the integer pipes, for the FP32 kernels' FP64 stage combination
// (there the FP64 pipe, which also runs the conversion instruction, is the bound): exact for
// every normal FP32 value and zero; FP32 subnormals read as signed zero (the FP32 kernels flush
// them); infinities and NaNs keep their class and payload.
__device__ __forceinline__ double f32_to_f64(float x) {
    const unsigned u = __float_as_uint(x), m = u & 0x7fffffffu;
    unsigned hi = (m >> 3) + 0x38000000u;                  // exponent bias 127 -> 1023
    if (m >= 0x7f800000u) hi = (m >> 3) | 0x7ff00000u;     // infinity, NaN
    unsigned lo = u << 29;
    if (m < 0x00800000u) hi = lo = 0u;                     // zero, subnormal
    return __hiloint2double((int)(hi | (u & 0x80000000u)), (int)lo);
}

// FP64 -> FP32 rounding to nearest, ties to even, on the integer pipes (the bit pattern's high
// and low words in, the FP32 bit pattern out), for kernels whose bound is the FP64 pipe, which
// also runs the conversion instruction: IEEE rounding with FP32 subnormal results flushed to
// signed zero, as the -ftz build's float(x) gives for every result in FP32's normal range and
// for zero and infinity; NaNs give the canonical NaN.  The double's exponent field sits in bits
// 30..20 of hi: rebiased from 1023 to 127 (896 << 20 = 0x38000000) and shifted left by 3
// together with the top 3 bits of lo, it lands in the float's place beside 20 + 3 significand
// bits; the 29 dropped bits round, and a carry out of the significand moves into the exponent
// (up to infinity) by itself.
__host__ __device__ __forceinline__ unsigned f64_bits_to_f32_bits(unsigned hi, unsigned lo) {
    const unsigned s = hi & 0x80000000u, a = hi & 0x7fffffffu;
    if (a - 0x38100000u < 0x0fe00000u) {   // exponent field 897..1150: a normal FP32 before rounding
        const unsigned f = ((a - 0x38000000u) << 3) | (lo >> 29);
        const unsigned up = (lo & 0x1fffffffu) + ((lo >> 29) & 1u) > 0x10000000u;
        return s | (f + up);
    }
    // below 2^-126: zero, unless it rounds up to 2^-126 (from 2^-126 - 2^-150 on, ties to even)
    if (a < 0x38100000u) return a == 0x380fffffu && lo >= 0xe0000000u ? s | 0x00800000u : s;
    if (a > 0x7ff00000u || (a == 0x7ff00000u && lo != 0u)) return 0x7fffffffu;   // NaN
    return s | 0x7f800000u;                                                  // 2^128 and above
}
__device__ __forceinline__ float f64_to_f32(double x) {
    return __uint_as_float(f64_bits_to_f32_bits((unsigned)__double2hiint(x), (unsigned)__double2loint(x)));
}

// the sum of the two lanes
__device__ __forceinline__ float hsum(F2 a) { return a.v.x + a.v.y; }

// the scalar type of a compute type: the uniform parameters of the templated math
template <class T> struct ScalarOf { using type = T; };
template <> struct ScalarOf<F2> { using type = float; };

}  // namespace hos
