// ckt_divide.cuh -- correctly rounded fp32 quotients by a loop-invariant
// divisor without the divide routine.
//
// Every quotient of the reference's wire recurrence has a divisor that does
// not change inside the inner loop: dt, the wire's resistance R and its
// capacitance C (apps/circuit/circuit_gpu.cu:119-128, circuit.cc:391-400).
// EXACT mode must round each of them exactly as IEEE a / b does, because the
// recurrence's gain L/(dt R) >> 1 magnifies any one-ulp difference at every
// step.  Two constructions give RN(a / b) for a precomputed divisor:
//
//  * Division by dt = (float)1e-6, one multiply and one FMA:
//        q = RN(a*zh + RN(a*zl)),  zh = RN(1/dt) = 1e6,  zl = RN(1/dt - zh).
//    a*(zh + zl) is a/dt to about 2^-47 relative, so q can differ from
//    RN(a/dt) only where a/dt lies within that distance of a rounding
//    boundary; which dividends do is a property of the divisor (Brisebarre,
//    Muller and Raina, "Accelerating correctly rounded floating-point
//    division when the divisor is known in advance", IEEE Trans. Computers
//    53(8), 2004).  For this divisor every one of the 2^32 float dividends
//    was compared with IEEE division (tests/test_divide.py on the CPU,
//    tests/test_gpu_divide.py against __fdiv_rn on the GPU): q equals
//    RN(a/dt) for all of them, zeros, infinities and NaN included, except 98
//    dividends below 2^-124 in magnitude, where a*zl underflows.  Dividends
//    below kDtTiny therefore leave the fast path.
//
//  * Any other divisor b (per wire, or a dt other than (float)1e-6), three
//    FMAs and a multiply with y = RN(1/b), yl = RN(1/b - y), nb = -b:
//        q0 = RN(a*y + RN(a*yl))   within 1 ulp of a/b (error ~2^-46 a/b
//                                  plus half an ulp)
//        r  = RN(a + nb*q0)        exact, because q0 is within 1 ulp
//        q  = RN(q0 + r*y)         = RN(a/b) by Markstein's theorem
//    (P. W. Markstein, "Computation of elementary functions on the IBM RISC
//    System/6000 processor", IBM J. Res. Dev. 34(1), 1990; J.-M. Muller et
//    al., Handbook of Floating-Point Arithmetic, Birkhauser, the chapter on
//    FMA-based division).  The theorem needs every intermediate to stay
//    clear of overflow and of underflow: with |b| in [2^bmin, 2^bmax] and
//    |a| in [lo, hi] below, |a/b| lies in [2^-70, 2^120], the remainder's
//    quantum 2^(eb+eq-46) is at least 2^-147 (so r is representable), and
//    RN(a*yl)'s absolute error is far below an ulp of the quotient.
//    Dividends outside [lo, hi] -- zero, tiny, huge, infinite -- take
//    wide_quot below; NaN dividends stay on the fast path, where every
//    operation returns NaN as IEEE division does.
//
//  * Dividends outside [lo, hi] (wide_quot): scaling by a power of two
//    commutes with rounding while the scaled values stay normal, so
//    RN(a/b) = RN((a s)/b) / s.  A huge |a| in (hi, 2^128) is scaled by
//    2^-64 into (2^26, 2^64), inside both guarded ranges; the quotient is
//    normal, and when RN(a/b) overflows the scaled quotient is at least
//    2^64 (2^128 - 2^103, the overflow threshold, scaled to the midpoint
//    2^64 - 2^39, rounds up to the even 2^64), so multiplying back gives
//    the same infinity.  A tiny nonzero |a| below lo, subnormals included,
//    is scaled by 2^110 into [2^-39, 2^60), inside both ranges; multiplying
//    back is exact while RN(a/b) is normal, which |a| >= 2^-125 |b|
//    guarantees.  Zeros and infinities are a times RN(1/b), exact for them.
//    Dividends whose quotient may be subnormal (subnormal_quot) are left to
//    the divide routine.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

namespace ckt {

// dt = (float)1e-6 (DELTAT, apps/circuit/circuit.h:44) and its split
// reciprocal.
constexpr uint32_t kDtBits = 0x358637bdu;
constexpr uint32_t kDtZhBits = 0x49742400u;  // RN(1/dt) = 1e6
constexpr uint32_t kDtZlBits = 0x3b257666u;  // RN(1/dt - 1e6) = 2.5247573e-3
// The split-reciprocal quotient by dt is exact for |a| >= kDtTiny.
constexpr float kDtTiny = 0x1p-118f;

// Eligible divisors and guarded dividend ranges of the corrected quotient.
// R: |b| in [2^-8, 2^8], |a| in [2^-50, 2^100];
// C and a general dt: |b| in [2^-30, 2^30], |a| in [2^-40, 2^90].
// wide_quot is exact for every dividend but those subnormal_quot flags.
constexpr float kRMin = 0x1p-8f, kRMax = 0x1p8f, kRLo = 0x1p-50f, kRHi = 0x1p100f;
constexpr float kCMin = 0x1p-30f, kCMax = 0x1p30f, kCLo = 0x1p-40f, kCHi = 0x1p90f;

__device__ __forceinline__ float dt_zh() { return __int_as_float((int)kDtZhBits); }
__device__ __forceinline__ float dt_zl() { return __int_as_float((int)kDtZlBits); }

// a / (float)1e-6 for |a| >= kDtTiny, zeros, infinities and NaN.
__device__ __forceinline__ float dt_quot(float a) {
  return __fmaf_rn(a, dt_zh(), __fmul_rn(a, dt_zl()));
}
__device__ __forceinline__ float2 dt_quot2(float2 a) {
  const float zh = dt_zh(), zl = dt_zl();
  return __ffma2_rn(a, make_float2(zh, zh), __fmul2_rn(a, make_float2(zl, zl)));
}

// Per-divisor constants of the corrected quotient.
struct Recip {
  float nb, y, yl;
};
__device__ __forceinline__ Recip make_recip(float b) {
  Recip r;
  r.nb = -b;
  r.y = __frcp_rn(b);
  // 1 - b*y is exact for a correctly rounded reciprocal, so yl = RN(1/b - y)
  r.yl = __fdiv_rn(__fmaf_rn(-b, r.y, 1.0f), b);
  return r;
}

__device__ __forceinline__ bool divisor_ok(float b, float bmin, float bmax) {
  const float m = fabsf(b);
  return m >= bmin && m <= bmax;  // false for NaN
}

// True when the corrected quotient may not equal RN(a/b): |a| outside
// [lo, hi].  False for NaN.
__device__ __forceinline__ bool outside(float a, float lo, float hi) {
  const float m = fabsf(a);
  return (m < lo) | (m > hi);
}

__device__ __forceinline__ float recip_quot(float a, const Recip &k) {
  const float q0 = __fmaf_rn(a, k.y, __fmul_rn(a, k.yl));
  const float r = __fmaf_rn(q0, k.nb, a);
  return __fmaf_rn(r, k.y, q0);
}

// Two divisions at once (paired FP32 instructions); each lane rounds exactly
// as recip_quot.
struct Recip2 {
  float2 nb, y, yl;
};
__device__ __forceinline__ Recip2 make_recip2(float bx, float by) {
  const Recip a = make_recip(bx), b = make_recip(by);
  Recip2 r;
  r.nb = make_float2(a.nb, b.nb);
  r.y = make_float2(a.y, b.y);
  r.yl = make_float2(a.yl, b.yl);
  return r;
}
__device__ __forceinline__ float2 recip_quot2(float2 a, const Recip2 &k) {
  const float2 q0 = __ffma2_rn(a, k.y, __fmul2_rn(a, k.yl));
  const float2 r = __ffma2_rn(q0, k.nb, a);
  return __ffma2_rn(r, k.y, q0);
}

// True for a nonzero |a| below tiny (NaN: false).
__device__ __forceinline__ bool tiny_nonzero(float a, float tiny) {
  const float m = fabsf(a);
  return (m < tiny) & (m != 0.0f);
}

// True when RN(a/b) may be subnormal: a nonzero |a| below 2^-125 |b|
// (m * 2^125 is exact for the magnitudes compared; NaN: false).
__device__ __forceinline__ bool subnormal_quot(float a, const Recip &k) {
  const float m = fabsf(a);
  return (m != 0.0f) & (__fmul_rn(m, 0x1p125f) < fabsf(k.nb));
}
__device__ __forceinline__ bool subnormal_quot2(float2 a, const Recip2 &k) {
  const float2 m = __fmul2_rn(make_float2(fabsf(a.x), fabsf(a.y)), make_float2(0x1p125f, 0x1p125f));
  return ((a.x != 0.0f) & (m.x < fabsf(k.nb.x))) | ((a.y != 0.0f) & (m.y < fabsf(k.nb.y)));
}

// RN(a/b) for any a that subnormal_quot does not flag: the corrected
// quotient of a scaled into [lo, hi] (see above).
__device__ __forceinline__ float wide_quot(float a, const Recip &k, float lo, float hi) {
  const float m = fabsf(a);
  const float s = m > hi ? 0x1p-64f : (m < lo ? 0x1p110f : 1.0f);
  const float u = m > hi ? 0x1p64f : (m < lo ? 0x1p-110f : 1.0f);
  const float q = __fmul_rn(recip_quot(__fmul_rn(a, s), k), u);
  return (m == 0.0f || m == __int_as_float(0x7f800000)) ? __fmul_rn(a, k.y) : q;
}
__device__ __forceinline__ float2 wide_quot2(float2 a, const Recip2 &k, float lo, float hi) {
  const float mx = fabsf(a.x), my = fabsf(a.y);
  const float2 s = make_float2(mx > hi ? 0x1p-64f : (mx < lo ? 0x1p110f : 1.0f),
                               my > hi ? 0x1p-64f : (my < lo ? 0x1p110f : 1.0f));
  const float2 u = make_float2(mx > hi ? 0x1p64f : (mx < lo ? 0x1p-110f : 1.0f),
                               my > hi ? 0x1p64f : (my < lo ? 0x1p-110f : 1.0f));
  float2 q = __fmul2_rn(recip_quot2(__fmul2_rn(a, s), k), u);
  const float2 z = __fmul2_rn(a, k.y);
  const float inf = __int_as_float(0x7f800000);
  if (mx == 0.0f || mx == inf) q.x = z.x;
  if (my == 0.0f || my == inf) q.y = z.y;
  return q;
}

// RN(a/b) for any a and an eligible b: the corrected quotient inside the
// guarded range, the divide routine outside it.
__device__ __forceinline__ float quot_guarded(float a, float b, const Recip &k, float lo,
                                              float hi) {
  return outside(a, lo, hi) ? __fdiv_rn(a, b) : recip_quot(a, k);
}

}  // namespace ckt
