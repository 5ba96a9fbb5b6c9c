// ckt_kernels.cuh -- sm_103a kernels of the circuit hot path.
//
// Arithmetic follows the reference task bodies operation by operation
// (apps/circuit/circuit_gpu.cu:114-129, 281-283, 330-345; the CPU tasks at
// apps/circuit/circuit.cc:386-401, 430-431, 1300-1302).  Every operation of
// the EXACT paths uses an explicitly rounded intrinsic so that no multiply
// is ever contracted into an add: results are bit-identical to the
// reference's IEEE fp32 arithmetic.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

#include "ckt.h"
#include "ckt_divide.cuh"

namespace ckt {

// ---------------------------------------------------------------------------
// calc_new_currents: one thread per wire.  The 10 segment currents and 11
// node/segment voltages of a wire live in registers across the whole inner
// time-step loop; wire fields are structure-of-arrays so a warp's loads and
// stores of any one field are one contiguous 128-byte line.
// ---------------------------------------------------------------------------
// Correctly rounded a / b.  A NaN dividend gives the quiet NaN every GPU
// arithmetic instruction returns for NaN operands (0x7fffffff, the same bits
// __fdiv_rn produces) without entering the divide routine's special-case
// path; once the recurrence has overflowed, every dividend is NaN.
__device__ __forceinline__ float div_rn(float a, float b) {
  return (a != a) ? __int_as_float(0x7fffffff) : __fdiv_rn(a, b);
}

// EXACT with the divide routine, one wire per thread:
// ((dv) - (L*(i-I0))/dt) / R and V0 + (dt*(i_k - i_k+1))/C, each operation
// rounded exactly as the reference's fp32 source.  CKT_MODE_EXACT_DIVIDE, and
// the wires of CKT_MODE_EXACT whose divisors lie outside the range of the
// corrected quotients (DualExact below).
struct DivideStep {
  float L, R, C, dt;
  __device__ __forceinline__ DivideStep(float l, float r, float c, float d) : L(l), R(r), C(c), dt(d) {}
  __device__ __forceinline__ void step(float (&ni)[10], float (&nv)[11], const float (&I0)[10],
                                       const float (&V0)[9]) const {
#pragma unroll
    for (int k = 0; k < 10; k++) {
      const float dv = __fsub_rn(nv[k + 1], nv[k]);
      const float q = div_rn(__fmul_rn(L, __fsub_rn(ni[k], I0[k])), dt);
      ni[k] = div_rn(__fsub_rn(dv, q), R);
    }
#pragma unroll
    for (int k = 0; k < 9; k++)
      nv[k + 1] = __fadd_rn(V0[k], div_rn(__fmul_rn(dt, __fsub_rn(ni[k], ni[k + 1])), C));
  }
};

// FAST: the three divisors are loop-invariant, so their quotients are
// computed once per wire (correctly rounded) and every inner-loop divide
// becomes a multiply.  The step works on j_k = i_k * R, the current before
// its 1/R scale, and carries d_k = i_k - I0_k from step to step:
//   j_k   <- (v_k+1 - v_k) + (-L/dt) * d_k
//   v_k+1 <- ((dt/C)(1/R)) * (j_k - j_k+1) + V0_k
//   d_k   <- (1/R) j_k - I0_k           (every step but the last)
//   i_k   <- (1/R) j_k                  (after the last step)
// starting from d_k = I0_k - I0_k.  3 FP32 operations per current and 2
// per voltage: 48 per wire-step, against the reference expression's 96
// counted flops.  Within 1e-5 relative of EXACT in the finite regime, with
// EXACT's NaN/Inf classes at the configured steps.
constexpr int kModeFastScalar = CKT_MODE_FAST_SCALAR;

struct FastConsts {
  float nLdt, rR, dtC, dtCrR;
  __device__ __forceinline__ FastConsts(float l, float r, float c, float d) {
    nLdt = -__fdiv_rn(l, d);
    rR = __fdiv_rn(1.0f, r);
    dtC = __fdiv_rn(d, c);
    dtCrR = __fmul_rn(dtC, rR);
  }
};

// Scalar form of the paired steppers below (bit-identical to them).
// LAST: write the currents i_k into di instead of the next d_k.
struct FastStep {
  FastConsts k;
  __device__ __forceinline__ FastStep(float l, float r, float c, float d) : k(l, r, c, d) {}
  template <bool LAST>
  __device__ __forceinline__ void step(float (&di)[10], float (&nv)[11], const float (&I0)[10],
                                       const float (&V0)[9]) const {
    float j[10];
#pragma unroll
    for (int q = 0; q < 10; q++) j[q] = __fmaf_rn(k.nLdt, di[q], __fsub_rn(nv[q + 1], nv[q]));
#pragma unroll
    for (int q = 0; q < 9; q++) nv[q + 1] = __fmaf_rn(k.dtCrR, __fsub_rn(j[q], j[q + 1]), V0[q]);
#pragma unroll
    for (int q = 0; q < 10; q++) di[q] = LAST ? __fmul_rn(k.rR, j[q]) : __fmaf_rn(k.rR, j[q], -I0[q]);
  }
};

// FAST, packed: the same operations, two at a time with Blackwell's paired
// FP32 instructions (add/mul/fma .f32x2).  Segment k is paired with k+5:
// currents (d_p, d_p+5) for p < 5 and voltages (v_q, v_q+5) for q <= 5, so
// every current operation and all voltages but v5 are one paired
// instruction for two segments.  A difference a - b is fma(b, -1, a):
// exact product, one rounding -- the same bits as the subtraction.  Each
// component is rounded exactly as in the scalar step: bit-identical to it.
struct PackedFast {
  float2 nLdt, rR, dtCrR, neg1;
  float dtCrR1;
  __device__ __forceinline__ PackedFast(float l, float r, float c, float d) {
    const FastConsts k(l, r, c, d);
    nLdt = make_float2(k.nLdt, k.nLdt);
    rR = make_float2(k.rR, k.rR);
    dtCrR = make_float2(k.dtCrR, k.dtCrR);
    neg1 = make_float2(-1.0f, -1.0f);
    dtCrR1 = k.dtCrR;
  }
  // dp[p] = (d_p, d_p+5); nI0[p] = (-I0_p, -I0_p+5); vp[q] = (v_q, v_q+5);
  // V0p[j] = (V0_j, V0_j+5) for j < 4; V04 = V0_4.
  template <bool LAST>
  __device__ __forceinline__ void step(float2 (&dp)[5], float2 (&vp)[6], const float2 (&nI0)[5],
                                       const float2 (&V0p)[4], float V04) const {
    float2 jp[5];
#pragma unroll
    for (int p = 0; p < 5; p++) jp[p] = __ffma2_rn(nLdt, dp[p], __ffma2_rn(vp[p], neg1, vp[p + 1]));
#pragma unroll
    for (int q = 1; q < 5; q++)
      vp[q] = __ffma2_rn(dtCrR, __ffma2_rn(jp[q], neg1, jp[q - 1]), V0p[q - 1]);
    const float v5 = __fmaf_rn(dtCrR1, __fmaf_rn(jp[0].y, -1.0f, jp[4].x), V04);
    vp[0].y = v5;
    vp[5].x = v5;
#pragma unroll
    for (int p = 0; p < 5; p++) dp[p] = LAST ? __fmul2_rn(rR, jp[p]) : __ffma2_rn(rR, jp[p], nI0[p]);
  }
};

// FAST, two wires per thread: wire a's segment k and wire b's segment k
// share every paired instruction, so all 48 operations of a wire-step pair
// up with no cross-lane moves (24 instructions per wire-step).  Each lane is
// rounded exactly as the scalar step: bit-identical to it.
struct DualFast {
  float2 nLdt, rR, dtCrR, neg1;
  __device__ __forceinline__ DualFast(float2 l, float2 r, float2 c, float d) {
    const FastConsts ka(l.x, r.x, c.x, d), kb(l.y, r.y, c.y, d);
    nLdt = make_float2(ka.nLdt, kb.nLdt);
    rR = make_float2(ka.rR, kb.rR);
    dtCrR = make_float2(ka.dtCrR, kb.dtCrR);
    neg1 = make_float2(-1.0f, -1.0f);
  }
  // d[k] = (d_k of a, d_k of b), nv[k] likewise; nI0 = -I0; V0 = wire voltages.
  template <bool LAST>
  __device__ __forceinline__ void step(float2 (&d)[10], float2 (&nv)[11], const float2 (&nI0)[10],
                                       const float2 (&V0)[9]) const {
    float2 j[10];
#pragma unroll
    for (int k = 0; k < 10; k++) j[k] = __ffma2_rn(nLdt, d[k], __ffma2_rn(nv[k], neg1, nv[k + 1]));
#pragma unroll
    for (int k = 0; k < 9; k++)
      nv[k + 1] = __ffma2_rn(dtCrR, __ffma2_rn(j[k + 1], neg1, j[k]), V0[k]);
#pragma unroll
    for (int k = 0; k < 10; k++) d[k] = LAST ? __fmul2_rn(rR, j[k]) : __ffma2_rn(rR, j[k], nI0[k]);
  }
};

// EXACT, two wires per thread: the reference's operations in the reference's
// order, each rounded as IEEE fp32 rounds it, with the 29 divisions of a
// wire-step done as correctly rounded quotients by precomputed reciprocals
// (ckt_divide.cuh) instead of the divide routine.  Wire a's and wire b's
// operation k share one paired instruction.  A step runs in two phases:
//   currents:  a1_k = L (i_k - I0_k),  a2_k = (v_k+1 - v_k) - a1_k / dt,
//              i_k <- a2_k / R
//   voltages:  a3_k = dt (i_k - i_k+1), v_k+1 <- V0_k + a3_k / C
// Each phase first forms all of its dividends, then takes the corrected
// quotients when every dividend of the thread's two wires lies in the
// guarded range, and wide_quot otherwise (zero dividends, as in a loop's
// first step, large ones and infinities while the recurrence overflows),
// the divide routine only for dividends too tiny for wide_quot.  Every
// branch rounds every quotient to the same float, so the bits never depend
// on which one ran.  DTF: dt is (float)1e-6 and its quotients use the
// split reciprocal (2 operations); otherwise they are corrected quotients too.
template <bool DTF>
struct DualExact {
  float2 L, dt2, neg1;
  Recip2 kR, kC, kdt;
  float dt;
  __device__ __forceinline__ DualExact(float2 l, float2 r, float2 c, float d) {
    L = l;
    dt = d;
    dt2 = make_float2(d, d);
    neg1 = make_float2(-1.0f, -1.0f);
    kR = make_recip2(r.x, r.y);
    kC = make_recip2(c.x, c.y);
    if (!DTF) kdt = make_recip2(d, d);
  }
  // Both wires' divisors lie in the range the corrected quotients need.
  static __device__ __forceinline__ bool eligible(float2 r, float2 c, float d) {
    return divisor_ok(r.x, kRMin, kRMax) && divisor_ok(r.y, kRMin, kRMax) &&
           divisor_ok(c.x, kCMin, kCMax) && divisor_ok(c.y, kCMin, kCMax) &&
           (DTF || divisor_ok(d, kCMin, kCMax));
  }
  __device__ __forceinline__ float2 dt_div(float2 a) const {
    if (DTF) return dt_quot2(a);
    return recip_quot2(a, kdt);
  }
  // With DTF no dividend of dt needs a guard of its own: the split quotient
  // is exact unless |a1| < 2^-118, and then |a1/dt| < 2^-98, far below half
  // an ulp of any dv with |dv - a1/dt| >= 2^-50 (the guard on a2), so
  // a2 = RN(dv - a1/dt) = dv either way; when a2's guard fails, the divide
  // routine recomputes the quotient from a1.
  __device__ __forceinline__ bool dt_outside(float a) const {
    if (DTF) return false;
    return outside(a, kCLo, kCHi);
  }
  // ni: currents i_k; nv: voltages v_0..v_10 (v_0, v_10 the node voltages);
  // nI0 = -I0; V0 = the wire's voltages at the start of the loop.
  __device__ __forceinline__ void step(float2 (&ni)[10], float2 (&nv)[11],
                                       const float2 (&nI0)[10], const float2 (&V0)[9]) const {
    float2 a1[10], a2[10];
    bool bad = false;
#pragma unroll
    for (int k = 0; k < 10; k++) {
      a1[k] = __fmul2_rn(L, __fadd2_rn(ni[k], nI0[k]));
      const float2 dv = __ffma2_rn(nv[k], neg1, nv[k + 1]);
      a2[k] = __ffma2_rn(dt_div(a1[k]), neg1, dv);
      bad |= dt_outside(a1[k].x) | dt_outside(a1[k].y) | outside(a2[k].x, kRLo, kRHi) |
             outside(a2[k].y, kRLo, kRHi);
    }
    // A phase that leaves the corrected quotient (zeros, huge values and
    // infinities as a loop's state starts or blows up) takes wide_quot, and
    // the divide routine only for the rare dividends wide_quot does not
    // cover: with DTF a dt dividend below kDtTiny (whose split quotient may
    // be off), an R or C dividend whose quotient may be subnormal; without
    // DTF, phase 1 always.
    bool wide = false;  // phase 1 left the corrected quotient
    if (!bad) {
#pragma unroll
      for (int k = 0; k < 10; k++) ni[k] = recip_quot2(a2[k], kR);
    } else {
      bool rare = !DTF;
      if (DTF) {
#pragma unroll
        for (int k = 0; k < 10; k++)
          rare |= tiny_nonzero(a1[k].x, kDtTiny) | tiny_nonzero(a1[k].y, kDtTiny) |
                  subnormal_quot2(a2[k], kR);
      }
      if (!rare) {
#pragma unroll
        for (int k = 0; k < 10; k++) ni[k] = wide_quot2(a2[k], kR, kRLo, kRHi);
      } else {
        const float2 R = make_float2(-kR.nb.x, -kR.nb.y);
#pragma unroll
        for (int k = 0; k < 10; k++) {
          const float dx = __fsub_rn(nv[k + 1].x, nv[k].x), dy = __fsub_rn(nv[k + 1].y, nv[k].y);
          ni[k] = make_float2(__fdiv_rn(__fsub_rn(dx, __fdiv_rn(a1[k].x, dt)), R.x),
                              __fdiv_rn(__fsub_rn(dy, __fdiv_rn(a1[k].y, dt)), R.y));
        }
      }
      wide = true;
    }
    // With DTF, currents from corrected quotients are at most 2^100 / 2^-8
    // in magnitude, so |a3| <= dt 2^109 < 2^90: only the lower bound needs a
    // check.  Currents from a phase 1 that left them may be anything.
    float2 a3[9];
    bad = false;
#pragma unroll
    for (int k = 0; k < 9; k++) {
      a3[k] = __fmul2_rn(dt2, __ffma2_rn(ni[k + 1], neg1, ni[k]));
      bad |= (fabsf(a3[k].x) < kCLo) | (fabsf(a3[k].y) < kCLo);
    }
    if (!DTF || wide) {
#pragma unroll
      for (int k = 0; k < 9; k++) bad |= (fabsf(a3[k].x) > kCHi) | (fabsf(a3[k].y) > kCHi);
    }
    if (!bad) {
#pragma unroll
      for (int k = 0; k < 9; k++) nv[k + 1] = __fadd2_rn(V0[k], recip_quot2(a3[k], kC));
    } else {
      bool rare = false;
#pragma unroll
      for (int k = 0; k < 9; k++)
        rare |= subnormal_quot2(a3[k], kC);
      if (!rare) {
#pragma unroll
        for (int k = 0; k < 9; k++) nv[k + 1] = __fadd2_rn(V0[k], wide_quot2(a3[k], kC, kCLo, kCHi));
      } else {
        const float2 C = make_float2(-kC.nb.x, -kC.nb.y);
#pragma unroll
        for (int k = 0; k < 9; k++)
          nv[k + 1] = make_float2(__fadd_rn(V0[k].x, __fdiv_rn(a3[k].x, C.x)),
                                  __fadd_rn(V0[k].y, __fdiv_rn(a3[k].y, C.y)));
      }
    }
  }
  // step() for a state whose 10 currents and 9 wire voltages are all NaN,
  // in both wires.  Such a state stays NaN -- every new current and voltage
  // depends on a NaN of the previous step -- so every dividend is NaN, every
  // guard of step() lets it pass and step() takes exactly these operations:
  // the same arithmetic without the compares and the branches.
  __device__ __forceinline__ void step_all_nan(float2 (&ni)[10], float2 (&nv)[11],
                                               const float2 (&nI0)[10],
                                               const float2 (&V0)[9]) const {
    float2 a2[10];
#pragma unroll
    for (int k = 0; k < 10; k++) {
      const float2 a1 = __fmul2_rn(L, __fadd2_rn(ni[k], nI0[k]));
      a2[k] = __ffma2_rn(dt_div(a1), neg1, __ffma2_rn(nv[k], neg1, nv[k + 1]));
    }
#pragma unroll
    for (int k = 0; k < 10; k++) ni[k] = recip_quot2(a2[k], kR);
    float2 a3[9];
#pragma unroll
    for (int k = 0; k < 9; k++) a3[k] = __fmul2_rn(dt2, __ffma2_rn(ni[k + 1], neg1, ni[k]));
#pragma unroll
    for (int k = 0; k < 9; k++) nv[k + 1] = __fadd2_rn(V0[k], recip_quot2(a3[k], kC));
  }
  static __device__ __forceinline__ bool first_nan(const float2 (&ni)[10]) {
    return ni[0].x != ni[0].x;
  }
  static __device__ __forceinline__ bool all_nan(const float2 (&ni)[10], const float2 (&nv)[11]) {
    bool nan = true;
#pragma unroll
    for (int k = 0; k < 10; k++) nan &= (ni[k].x != ni[k].x) & (ni[k].y != ni[k].y);
#pragma unroll
    for (int k = 1; k < 10; k++) nan &= (nv[k].x != nv[k].x) & (nv[k].y != nv[k].y);
    return nan;
  }
};

// The inner loop of DualExact: step() in blocks of kNanCheckSteps; at each
// block boundary, once the states of all the warp's wires have become all
// NaN (as the reference's recurrence does within ~10-30 steps at the
// benchmark's inductances, and stays), the remaining steps run with
// step_all_nan -- every operation of every step still computed, the same
// bits.
constexpr int kNanCheckSteps = 16;
template <typename Stepper, typename F>
__device__ __forceinline__ void exact_steps(const Stepper &pk, int steps, F (&ni)[10], F (&nv)[11],
                                            const F (&nI0)[10], const F (&V0)[9]) {
  int j = 0;
#pragma unroll 1
  while (j < steps) {
    // The full test only once the first current is NaN (one compare on a
    // finite state); the switch only when every thread of the warp can take
    // it, so that a warp never runs the two loops one after the other.
    const bool mine = Stepper::first_nan(ni) && Stepper::all_nan(ni, nv);
    if (__all_sync(__activemask(), mine)) break;
    const int n = min(kNanCheckSteps, steps - j);
#pragma unroll 1
    for (int i = 0; i < n; i++) pk.step(ni, nv, nI0, V0);
    j += n;
  }
#pragma unroll 1
  for (; j < steps; j++) pk.step_all_nan(ni, nv, nI0, V0);
}

// EXACT, one wire per thread: DualExact's arithmetic and guards on scalar
// instructions (the batched kernel's one-wire tiles).  Bit-identical to it.
template <bool DTF>
struct SoloExact {
  float L, dt;
  Recip kR, kC, kdt;
  __device__ __forceinline__ SoloExact(float l, float r, float c, float d) {
    L = l;
    dt = d;
    kR = make_recip(r);
    kC = make_recip(c);
    if (!DTF) kdt = make_recip(d);
  }
  static __device__ __forceinline__ bool eligible(float r, float c, float d) {
    return divisor_ok(r, kRMin, kRMax) && divisor_ok(c, kCMin, kCMax) &&
           (DTF || divisor_ok(d, kCMin, kCMax));
  }
  __device__ __forceinline__ void step(float (&ni)[10], float (&nv)[11], const float (&I0)[10],
                                       const float (&V0)[9]) const {
    float a1[10], a2[10];
    bool bad = false;
#pragma unroll
    for (int k = 0; k < 10; k++) {
      a1[k] = __fmul_rn(L, __fsub_rn(ni[k], I0[k]));
      const float q1 = DTF ? dt_quot(a1[k]) : recip_quot(a1[k], kdt);
      a2[k] = __fsub_rn(__fsub_rn(nv[k + 1], nv[k]), q1);
      if (!DTF) bad |= outside(a1[k], kCLo, kCHi);
      bad |= outside(a2[k], kRLo, kRHi);
    }
    // Leaving the corrected quotient as DualExact::step does.
    bool wide = false;
    if (!bad) {
#pragma unroll
      for (int k = 0; k < 10; k++) ni[k] = recip_quot(a2[k], kR);
    } else {
      bool rare = !DTF;
      if (DTF) {
#pragma unroll
        for (int k = 0; k < 10; k++)
          rare |= tiny_nonzero(a1[k], kDtTiny) | subnormal_quot(a2[k], kR);
      }
      if (!rare) {
#pragma unroll
        for (int k = 0; k < 10; k++) ni[k] = wide_quot(a2[k], kR, kRLo, kRHi);
      } else {
        const float R = -kR.nb;
#pragma unroll
        for (int k = 0; k < 10; k++)
          ni[k] = __fdiv_rn(__fsub_rn(__fsub_rn(nv[k + 1], nv[k]), __fdiv_rn(a1[k], dt)), R);
      }
      wide = true;
    }
    float a3[9];
    bad = false;
#pragma unroll
    for (int k = 0; k < 9; k++) {
      a3[k] = __fmul_rn(dt, __fsub_rn(ni[k], ni[k + 1]));
      bad |= fabsf(a3[k]) < kCLo;
    }
    if (!DTF || wide) {
#pragma unroll
      for (int k = 0; k < 9; k++) bad |= fabsf(a3[k]) > kCHi;
    }
    if (!bad) {
#pragma unroll
      for (int k = 0; k < 9; k++) nv[k + 1] = __fadd_rn(V0[k], recip_quot(a3[k], kC));
    } else {
      bool rare = false;
#pragma unroll
      for (int k = 0; k < 9; k++) rare |= subnormal_quot(a3[k], kC);
      if (!rare) {
#pragma unroll
        for (int k = 0; k < 9; k++) nv[k + 1] = __fadd_rn(V0[k], wide_quot(a3[k], kC, kCLo, kCHi));
      } else {
        const float C = -kC.nb;
#pragma unroll
        for (int k = 0; k < 9; k++) nv[k + 1] = __fadd_rn(V0[k], __fdiv_rn(a3[k], C));
      }
    }
  }
  // step() for a state whose 10 currents and 9 wire voltages are all NaN:
  // the same operations without the compares and the branches (see
  // DualExact::step_all_nan).
  __device__ __forceinline__ void step_all_nan(float (&ni)[10], float (&nv)[11],
                                               const float (&I0)[10],
                                               const float (&V0)[9]) const {
    float a2[10];
#pragma unroll
    for (int k = 0; k < 10; k++) {
      const float a1 = __fmul_rn(L, __fsub_rn(ni[k], I0[k]));
      const float q1 = DTF ? dt_quot(a1) : recip_quot(a1, kdt);
      a2[k] = __fsub_rn(__fsub_rn(nv[k + 1], nv[k]), q1);
    }
#pragma unroll
    for (int k = 0; k < 10; k++) ni[k] = recip_quot(a2[k], kR);
    float a3[9];
#pragma unroll
    for (int k = 0; k < 9; k++) a3[k] = __fmul_rn(dt, __fsub_rn(ni[k], ni[k + 1]));
#pragma unroll
    for (int k = 0; k < 9; k++) nv[k + 1] = __fadd_rn(V0[k], recip_quot(a3[k], kC));
  }
  static __device__ __forceinline__ bool first_nan(const float (&ni)[10]) { return ni[0] != ni[0]; }
  static __device__ __forceinline__ bool all_nan(const float (&ni)[10], const float (&nv)[11]) {
    bool nan = true;
#pragma unroll
    for (int k = 0; k < 10; k++) nan &= ni[k] != ni[k];
#pragma unroll
    for (int k = 1; k < 10; k++) nan &= nv[k] != nv[k];
    return nan;
  }
};

__device__ __forceinline__ const float *pick_instance(uint8_t loc, const float *pvt,
                                                      const float *shr, const float *ghost) {
  // get_node (apps/circuit/circuit_gpu.cu:40-59) without its assert: a
  // location outside {0,1,2} reads the ghost instance; ckt_sanity_check_wires
  // and ckt_graph_create reject such wires.
  return loc == CKT_PRIVATE_PTR ? pvt : (loc == CKT_SHARED_PTR ? shr : ghost);
}

// Device views of the wire region and of the node voltages CNC reads.
struct WireArrays {
  const uint32_t *in_ptr, *out_ptr;
  const uint8_t *in_loc, *out_loc;
  const float *L, *R, *C;
  float *cur, *vol;
  int64_t S;  // segment stride
};
struct NodeVolts {
  const float *pvt, *shr, *ghost;
};

// One wire's whole inner loop: load, S steps in registers, store.
template <int MODE, int INIT>
__device__ __forceinline__ void cnc_wire(int64_t w, const WireArrays &a, const NodeVolts &nv_in,
                                         int steps, float dt, float *i0_out = nullptr,
                                         float *i9_out = nullptr) {
  const int64_t S = a.S;
  float I0[10], V0[9], ni[10], nv[11];
#pragma unroll
  for (int k = 0; k < 10; k++) I0[k] = a.cur[k * S + w];
#pragma unroll
  for (int k = 0; k < 9; k++) V0[k] = a.vol[k * S + w];
  const uint32_t in = a.in_ptr[w], out = a.out_ptr[w];
  const float v_out = pick_instance(a.out_loc[w], nv_in.pvt, nv_in.shr, nv_in.ghost)[out];
#pragma unroll
  for (int k = 0; k < 10; k++) ni[k] = I0[k];
  if (INIT == CKT_INIT_KERNEL) {
    nv[0] = pick_instance(a.in_loc[w], nv_in.pvt, nv_in.shr, nv_in.ghost)[in];
#pragma unroll
    for (int k = 0; k < 9; k++) nv[k + 1] = V0[k];
  } else {
#pragma unroll
    for (int k = 0; k < 9; k++) nv[k] = V0[k];
    nv[9] = 0.0f;
  }
  nv[10] = v_out;

  if constexpr (MODE == CKT_MODE_FAST) {
    const PackedFast pk(a.L[w], a.R[w], a.C[w], dt);
    float2 dp[5], nI0[5], vp[6], V0p[4];
#pragma unroll
    for (int p = 0; p < 5; p++) {
      nI0[p] = make_float2(-I0[p], -I0[p + 5]);
      dp[p] = __fadd2_rn(make_float2(I0[p], I0[p + 5]), nI0[p]);
    }
#pragma unroll
    for (int q = 0; q < 6; q++) vp[q] = make_float2(nv[q], nv[q + 5]);
#pragma unroll
    for (int q = 0; q < 4; q++) V0p[q] = make_float2(V0[q], V0[q + 5]);
    if (steps > 0) {
      int j = 1;
#pragma unroll 1
      for (; j + 4 <= steps; j += 4) {
        pk.step<false>(dp, vp, nI0, V0p, V0[4]);
        pk.step<false>(dp, vp, nI0, V0p, V0[4]);
        pk.step<false>(dp, vp, nI0, V0p, V0[4]);
        pk.step<false>(dp, vp, nI0, V0p, V0[4]);
      }
#pragma unroll 1
      for (; j < steps; j++) pk.step<false>(dp, vp, nI0, V0p, V0[4]);
      pk.step<true>(dp, vp, nI0, V0p, V0[4]);
#pragma unroll
      for (int p = 0; p < 5; p++) {
        ni[p] = dp[p].x;
        ni[p + 5] = dp[p].y;
      }
#pragma unroll
      for (int q = 0; q < 6; q++) {
        nv[q] = vp[q].x;
        nv[q + 5] = vp[q].y;
      }
    }
  } else if constexpr (MODE == kModeFastScalar) {
    const FastStep fs(a.L[w], a.R[w], a.C[w], dt);
    if (steps > 0) {
      float d[10];
#pragma unroll
      for (int k = 0; k < 10; k++) d[k] = __fsub_rn(I0[k], I0[k]);
      int j = 1;
#pragma unroll 1
      for (; j + 2 <= steps; j += 2) {
        fs.step<false>(d, nv, I0, V0);
        fs.step<false>(d, nv, I0, V0);
      }
      if (j < steps) fs.step<false>(d, nv, I0, V0);
      fs.step<true>(d, nv, I0, V0);
#pragma unroll
      for (int k = 0; k < 10; k++) ni[k] = d[k];
    }
  } else if (MODE == CKT_MODE_EXACT && __float_as_uint(dt) == kDtBits &&
             SoloExact<true>::eligible(a.R[w], a.C[w], dt)) {
    const SoloExact<true> ws(a.L[w], a.R[w], a.C[w], dt);
    exact_steps(ws, steps, ni, nv, I0, V0);
  } else if (MODE == CKT_MODE_EXACT && __float_as_uint(dt) != kDtBits &&
             SoloExact<false>::eligible(a.R[w], a.C[w], dt)) {
    const SoloExact<false> ws(a.L[w], a.R[w], a.C[w], dt);
    exact_steps(ws, steps, ni, nv, I0, V0);
  } else {
    static_assert(MODE == CKT_MODE_EXACT || MODE == CKT_MODE_EXACT_DIVIDE, "unknown mode");
    const DivideStep ws(a.L[w], a.R[w], a.C[w], dt);
    int j = 0;
#pragma unroll 1
    for (; j + 2 <= steps; j += 2) {
      ws.step(ni, nv, I0, V0);
      ws.step(ni, nv, I0, V0);
    }
    if (j < steps) ws.step(ni, nv, I0, V0);
  }

#pragma unroll
  for (int k = 0; k < 10; k++) a.cur[k * S + w] = ni[k];
#pragma unroll
  for (int k = 0; k < 9; k++) a.vol[k * S + w] = nv[k + 1];
  if (i0_out) *i0_out = ni[0];
  if (i9_out) *i9_out = ni[9];
}

// Two wires per thread (FAST: DualFast, EXACT: DualExact): thread t of a
// block handles wires base + t and base + t + 256, so each field's loads and
// stores stay one contiguous line per warp.  Without a partner wire the
// thread runs its wire in both lanes and stores one.
template <int MODE, int INIT>
__device__ __forceinline__ void cnc_wire_pair(int64_t wa, int64_t wb, bool has_b,
                                              const WireArrays &a, const NodeVolts &nvin,
                                              int steps, float dt, float2 *i0_out = nullptr,
                                              float2 *i9_out = nullptr) {
  static_assert(MODE == CKT_MODE_FAST || MODE == CKT_MODE_EXACT, "paired modes: FAST, EXACT");
  const int64_t S = a.S;
  const float2 L2 = make_float2(a.L[wa], a.L[wb]), R2 = make_float2(a.R[wa], a.R[wb]),
               C2 = make_float2(a.C[wa], a.C[wb]);
  const bool dt_fixed = __float_as_uint(dt) == kDtBits;
  if (MODE == CKT_MODE_EXACT &&
      !(dt_fixed ? DualExact<true>::eligible(R2, C2, dt) : DualExact<false>::eligible(R2, C2, dt))) {
    // a divisor outside the corrected quotients' range: the divide routine
    float ia0, ia9, ib0, ib9;
    cnc_wire<CKT_MODE_EXACT_DIVIDE, INIT>(wa, a, nvin, steps, dt, &ia0, &ia9);
    ib0 = ia0;
    ib9 = ia9;
    if (has_b) cnc_wire<CKT_MODE_EXACT_DIVIDE, INIT>(wb, a, nvin, steps, dt, &ib0, &ib9);
    if (i0_out) *i0_out = make_float2(ia0, ib0);
    if (i9_out) *i9_out = make_float2(ia9, ib9);
    return;
  }
  // FAST: ni holds d_k = i_k - I0_k during the loop, then the currents;
  // EXACT: ni holds the currents throughout.
  float2 ni[10], nI0[10], nv[11], V0[9];
#pragma unroll
  for (int k = 0; k < 10; k++) {
    const float x = a.cur[k * S + wa], y = a.cur[k * S + wb];
    nI0[k] = make_float2(-x, -y);
    ni[k] = MODE == CKT_MODE_FAST ? __fadd2_rn(make_float2(x, y), nI0[k]) : make_float2(x, y);
  }
#pragma unroll
  for (int k = 0; k < 9; k++) V0[k] = make_float2(a.vol[k * S + wa], a.vol[k * S + wb]);
  const float out_a = pick_instance(a.out_loc[wa], nvin.pvt, nvin.shr, nvin.ghost)[a.out_ptr[wa]];
  const float out_b = pick_instance(a.out_loc[wb], nvin.pvt, nvin.shr, nvin.ghost)[a.out_ptr[wb]];
  if (INIT == CKT_INIT_KERNEL) {
    nv[0] = make_float2(pick_instance(a.in_loc[wa], nvin.pvt, nvin.shr, nvin.ghost)[a.in_ptr[wa]],
                        pick_instance(a.in_loc[wb], nvin.pvt, nvin.shr, nvin.ghost)[a.in_ptr[wb]]);
#pragma unroll
    for (int k = 0; k < 9; k++) nv[k + 1] = V0[k];
  } else {
#pragma unroll
    for (int k = 0; k < 9; k++) nv[k] = V0[k];
    nv[9] = make_float2(0.0f, 0.0f);
  }
  nv[10] = make_float2(out_a, out_b);
  if constexpr (MODE == CKT_MODE_FAST) {
    const DualFast pk(L2, R2, C2, dt);
    if (steps > 0) {
      int j = 1;
#pragma unroll 1
      for (; j + 2 <= steps; j += 2) {
        pk.step<false>(ni, nv, nI0, V0);
        pk.step<false>(ni, nv, nI0, V0);
      }
      if (j < steps) pk.step<false>(ni, nv, nI0, V0);
      pk.step<true>(ni, nv, nI0, V0);
    } else {
#pragma unroll
      for (int k = 0; k < 10; k++) ni[k] = make_float2(-nI0[k].x, -nI0[k].y);  // no step: I0
    }
  } else if (dt_fixed) {
    const DualExact<true> pk(L2, R2, C2, dt);
    exact_steps(pk, steps, ni, nv, nI0, V0);
  } else {
    const DualExact<false> pk(L2, R2, C2, dt);
    exact_steps(pk, steps, ni, nv, nI0, V0);
  }
#pragma unroll
  for (int k = 0; k < 10; k++) a.cur[k * S + wa] = ni[k].x;
#pragma unroll
  for (int k = 0; k < 9; k++) a.vol[k * S + wa] = nv[k + 1].x;
  if (has_b) {
#pragma unroll
    for (int k = 0; k < 10; k++) a.cur[k * S + wb] = ni[k].y;
#pragma unroll
    for (int k = 0; k < 9; k++) a.vol[k * S + wb] = nv[k + 1].y;
  }
  if (i0_out) *i0_out = ni[0];
  if (i9_out) *i9_out = ni[9];
}

constexpr int kPairBlock = 256;  // threads; a block covers 2 * kPairBlock wires

template <int MODE, int INIT>
__global__ void __launch_bounds__(kPairBlock, 2)
    cnc_pair_kernel(uint32_t first_wire, uint32_t num_wires, WireArrays a, NodeVolts v, int steps,
                    float dt) {
  const uint32_t ta = blockIdx.x * (2 * kPairBlock) + threadIdx.x, tb = ta + kPairBlock;
  if (ta >= num_wires) return;
  const bool has_b = tb < num_wires;
  cnc_wire_pair<MODE, INIT>((int64_t)first_wire + ta, (int64_t)first_wire + (has_b ? tb : ta),
                            has_b, a, v, steps, dt);
}

template <int MODE, int INIT>
__global__ void __launch_bounds__(256)
    cnc_kernel(uint32_t first_wire, uint32_t num_wires, WireArrays a, NodeVolts v, int steps,
               float dt) {
  const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= num_wires) return;
  cnc_wire<MODE, INIT>((int64_t)first_wire + t, a, v, steps, dt);
}

// ---------------------------------------------------------------------------
// distribute_charge.  The reference adds -dt*I[0] to the in-node and
// +dt*I[9] to the out-node of every wire with atomicAdd (unordered).  Here
// each node GATHERS its contributions from a static CSR whose order is the
// reference CPU runtime's: wire order within a piece, private nodes updated
// in place, shared/ghost contributions folded per piece (identity 0) and the
// folds applied in ascending piece order.
// ---------------------------------------------------------------------------
__device__ __forceinline__ float contribution(uint32_t wire, uint32_t end,
                                              const float *__restrict__ I0,
                                              const float *__restrict__ I9, float dt) {
  // -dt * current[0] (in end) and dt * current[9] (out end),
  // apps/circuit/circuit.cc:430-431.
  return end ? __fmul_rn(dt, I9[wire]) : __fmul_rn(-dt, I0[wire]);
}

// Whole circuit, canonical order.  A block owns BLOCK consecutive nodes,
// whose contributions are one contiguous span of the CSR.  The block first
// stages the span in shared memory -- coalesced entry loads and independent
// current gathers, so every thread has many loads in flight -- then each
// thread sums its own node's run sequentially, in the reference order.
// COHERENT loads bypass L1: used when the currents were written by other
// blocks of the same (persistent) launch.
constexpr uint32_t kDcChunk = 4096;

template <bool COHERENT>
__device__ __forceinline__ float ld_f32(const float *p) {
  return COHERENT ? __ldcg(p) : *p;
}

// Returns the thread's node's new charge; STORE = false leaves charge[]
// unwritten for a caller that consumes the value itself.
template <uint32_t BLOCK, bool COHERENT, bool STORE = true>
__device__ __forceinline__ float dc_block(uint32_t x0, uint32_t xe,
                                         const uint32_t *__restrict__ off,
                                         const uint32_t *__restrict__ ent,
                                         const float *__restrict__ I0,
                                         const float *__restrict__ I9,
                                         float *__restrict__ charge, float dt, float *sval,
                                         uint32_t *smask) {
  const uint32_t x = x0 + threadIdx.x;
  const uint32_t lo = off[x0] & 0x7fffffffu, hi = off[xe] & 0x7fffffffu;
  uint32_t b = 0, e = 0;
  bool priv = true;
  float acc = 0.0f, fold = 0.0f;
  if (x < xe) {
    const uint32_t o0 = off[x], o1 = off[x + 1];
    priv = (o0 & 0x80000000u) != 0;
    b = o0 & 0x7fffffffu;
    e = o1 & 0x7fffffffu;
    acc = charge[x];
  }
  for (uint32_t c0 = lo; c0 < hi; c0 += kDcChunk) {
    const uint32_t cn = min(kDcChunk, hi - c0);
    // Stage in batches of kDcBatch entries per thread: all entry loads of a
    // batch first, then all of its current gathers, so every thread keeps
    // kDcBatch independent loads in flight at each of the two levels.
    constexpr uint32_t kDcBatch = 8;
    for (uint32_t j0 = 0; j0 < cn; j0 += kDcBatch * BLOCK) {
      uint32_t u[kDcBatch];
#pragma unroll
      for (uint32_t r = 0; r < kDcBatch; r++) {
        const uint32_t j = j0 + r * BLOCK + threadIdx.x;
        u[r] = j < cn ? ent[c0 + j] : 0u;
      }
      float v[kDcBatch];
#pragma unroll
      for (uint32_t r = 0; r < kDcBatch; r++) {
        const uint32_t w = u[r] >> 2;
        v[r] = (u[r] & 2u) ? ld_f32<COHERENT>(I9 + w) : ld_f32<COHERENT>(I0 + w);
      }
#pragma unroll
      for (uint32_t r = 0; r < kDcBatch; r++) {
        const uint32_t j = j0 + r * BLOCK + threadIdx.x;
        // group-start flags of the warp's 32 consecutive entries, one word
        const uint32_t m = __ballot_sync(0xffffffffu, (u[r] & 1u) != 0u);
        if (j < cn) {
          sval[j] = (u[r] & 2u) ? __fmul_rn(dt, v[r]) : __fmul_rn(-dt, v[r]);
          if ((threadIdx.x & 31u) == 0u) smask[j >> 5] = m;
        }
      }
    }
    __syncthreads();
    const uint32_t i0 = max(b, c0), i1 = min(e, c0 + cn);
    if (priv) {
      for (uint32_t i = i0; i < i1; i++) acc = __fadd_rn(acc, sval[i - c0]);
    } else {
      for (uint32_t i = i0; i < i1; i++) {
        if (((smask[(i - c0) >> 5] >> ((i - c0) & 31u)) & 1u) && i != b) {
          acc = __fadd_rn(acc, fold);
          fold = 0.0f;
        }
        fold = __fadd_rn(fold, sval[i - c0]);
      }
    }
    __syncthreads();
  }
  if (x < xe) {
    if (!priv && e > b) acc = __fadd_rn(acc, fold);
    if (STORE) charge[x] = acc;
  }
  return acc;
}

// The simple schedule: one thread per node walks its own run with dependent
// loads (no staging).  Same order, same bits.
template <bool COHERENT>
__device__ __forceinline__ void dc_node(uint32_t x, const uint32_t *__restrict__ off,
                                        const uint32_t *__restrict__ ent,
                                        const float *__restrict__ I0,
                                        const float *__restrict__ I9,
                                        float *__restrict__ charge, float dt) {
  const uint32_t o0 = off[x], o1 = off[x + 1];
  const uint32_t b = o0 & 0x7fffffffu, e = o1 & 0x7fffffffu;
  float acc = charge[x];
  if (o0 & 0x80000000u) {
    for (uint32_t i = b; i < e; i++) {
      const uint32_t u = ent[i], w = u >> 2;
      acc = __fadd_rn(acc, (u & 2u) ? __fmul_rn(dt, ld_f32<COHERENT>(I9 + w))
                                    : __fmul_rn(-dt, ld_f32<COHERENT>(I0 + w)));
    }
  } else {
    float fold = 0.0f;
    for (uint32_t i = b; i < e; i++) {
      const uint32_t u = ent[i], w = u >> 2;
      if ((u & 1u) && i != b) {
        acc = __fadd_rn(acc, fold);
        fold = 0.0f;
      }
      fold = __fadd_rn(fold, (u & 2u) ? __fmul_rn(dt, ld_f32<COHERENT>(I9 + w))
                                      : __fmul_rn(-dt, ld_f32<COHERENT>(I0 + w)));
    }
    if (e > b) acc = __fadd_rn(acc, fold);
  }
  charge[x] = acc;
}

constexpr uint32_t kDcBlock = 256;

static __global__ void __launch_bounds__(kDcBlock)
    dc_all_kernel(uint32_t node_begin, uint32_t node_end, const uint32_t *__restrict__ off,
                  const uint32_t *__restrict__ ent, const float *__restrict__ I0,
                  const float *__restrict__ I9, float *__restrict__ charge, float dt) {
  __shared__ float sval[kDcChunk];
  __shared__ uint32_t smask[kDcChunk / 32];
  const uint32_t x0 = node_begin + blockIdx.x * kDcBlock;
  dc_block<kDcBlock, false>(x0, min(node_end, x0 + kDcBlock), off, ent, I0, I9, charge, dt, sval,
                            smask);
}

// One piece: one thread per node the piece touches; private nodes are
// updated in place, shared/ghost nodes fold into the given instances.
static __global__ void __launch_bounds__(256)
    dc_piece_kernel(uint32_t t0, uint32_t nt, const uint32_t *__restrict__ touch_node,
                    const uint8_t *__restrict__ touch_loc, const uint32_t *__restrict__ touch_off,
                    const uint32_t *__restrict__ pent, const float *__restrict__ I0,
                    const float *__restrict__ I9, float *charge, float *shr_fold,
                    float *ghost_fold, float dt) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nt) return;
  const uint32_t t = t0 + i;
  const uint32_t x = touch_node[t];
  const uint8_t loc = touch_loc[t];
  float *tgt = loc == CKT_PRIVATE_PTR ? charge : (loc == CKT_SHARED_PTR ? shr_fold : ghost_fold);
  float acc = tgt[x];
  for (uint32_t e = touch_off[t]; e < touch_off[t + 1]; e++) {
    const uint32_t u = pent[e];
    acc = __fadd_rn(acc, contribution(u >> 1, u & 1u, I0, I9, dt));
  }
  tgt[x] = acc;
}

// One piece without the contribution graph (distribute_charge_kernel,
// apps/circuit/circuit_gpu.cu:245-286): one thread per wire adds -dt*I[0]
// to its in-node and dt*I[9] to its out-node with atomic adds -- private
// nodes into pvt's charge, shared and ghost nodes into their fold instances
// (reduce_local, circuit_gpu.cu:219-243).  Lanes of a warp whose wire ends
// land on the same node of the same instance first combine their
// contributions: __match_any_sync groups them, and the group's first lane
// adds the group's sum, in lane order, with one atomic.  The order of the
// additions at a node is unspecified, as with the reference's atomicAdd.
__device__ __forceinline__ void warp_aggregated_add(float *target, float v, uint64_t key,
                                                    float *sbuf) {
  const uint32_t lane = threadIdx.x & 31u;
  const uint32_t peers = __match_any_sync(__activemask(), key);
  if (peers == (1u << lane)) {
    atomicAdd(target, v);
    return;
  }
  sbuf[lane] = v;
  __syncwarp(peers);
  if (lane == (uint32_t)(__ffs(peers) - 1)) {
    float sum = sbuf[lane];
    for (uint32_t m = peers & (peers - 1); m; m &= m - 1) sum = __fadd_rn(sum, sbuf[__ffs(m) - 1]);
    atomicAdd(target, sum);
  }
  __syncwarp(peers);  // sbuf is reused by the wire's other end
}

static __global__ void __launch_bounds__(256)
    dc_atomic_kernel(uint32_t first_wire, uint32_t num_wires, const uint32_t *__restrict__ in_ptr,
                     const uint32_t *__restrict__ out_ptr, const uint8_t *__restrict__ in_loc,
                     const uint8_t *__restrict__ out_loc, const float *__restrict__ I0,
                     const float *__restrict__ I9, float *pvt_charge, float *shr_fold,
                     float *ghost_fold, float dt) {
  __shared__ float sbuf[256];
  const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= num_wires) return;
  const uint32_t w = first_wire + t;
  float *warp_buf = sbuf + (threadIdx.x & ~31u);
  const uint32_t a = in_ptr[w], b = out_ptr[w];
  const uint8_t la = in_loc[w], lb = out_loc[w];
  const float ca = __fmul_rn(-dt, I0[w]), cb = __fmul_rn(dt, I9[w]);
  float *ta = la == CKT_PRIVATE_PTR ? pvt_charge : (la == CKT_SHARED_PTR ? shr_fold : ghost_fold);
  float *tb = lb == CKT_PRIVATE_PTR ? pvt_charge : (lb == CKT_SHARED_PTR ? shr_fold : ghost_fold);
  warp_aggregated_add(ta + a, ca, ((uint64_t)(la > 2 ? 2 : la) << 32) | a, warp_buf);
  warp_aggregated_add(tb + b, cb, ((uint64_t)(lb > 2 ? 2 : lb) << 32) | b, warp_buf);
}

// Application of one piece's reduction instances.
static __global__ void __launch_bounds__(256)
    apply_fold_kernel(uint32_t t0, uint32_t nt, const uint32_t *__restrict__ touch_node,
                      const uint8_t *__restrict__ touch_loc, float *shr_fold, float *ghost_fold,
                      float *charge) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nt) return;
  const uint32_t t = t0 + i;
  const uint8_t loc = touch_loc[t];
  if (loc == CKT_PRIVATE_PTR) return;
  const uint32_t x = touch_node[t];
  float *fold = loc == CKT_SHARED_PTR ? shr_fold : ghost_fold;
  charge[x] = __fadd_rn(charge[x], fold[x]);
  fold[x] = 0.0f;
}

// ---------------------------------------------------------------------------
// update_voltages: v += q/C; v *= (1 - leak); q = 0
// (apps/circuit/circuit_gpu.cu:330-335, circuit.cc:1300-1302).
// ---------------------------------------------------------------------------
__device__ __forceinline__ float uv_one(float v, float q, float c, float l) {
  return __fmul_rn(__fadd_rn(v, __fdiv_rn(q, c)), __fsub_rn(1.0f, l));
}

// Whole node range, four nodes per thread with 16-byte loads and stores.
static __global__ void __launch_bounds__(256)
    uv_all_vec4_kernel(uint32_t n4, float4 *__restrict__ q, float4 *__restrict__ v,
                       const float4 *__restrict__ c, const float4 *__restrict__ l) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n4) return;
  const float4 qq = q[i], vv = v[i], cc = c[i], ll = l[i];
  float4 r;
  r.x = uv_one(vv.x, qq.x, cc.x, ll.x);
  r.y = uv_one(vv.y, qq.y, cc.y, ll.y);
  r.z = uv_one(vv.z, qq.z, cc.z, ll.z);
  r.w = uv_one(vv.w, qq.w, cc.w, ll.w);
  v[i] = r;
  q[i] = make_float4(0.f, 0.f, 0.f, 0.f);
}

static __global__ void __launch_bounds__(256)
    uv_all_scalar_kernel(uint32_t first, uint32_t n, float *__restrict__ q, float *__restrict__ v,
                         const float *__restrict__ c, const float *__restrict__ l) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const uint32_t x = first + i;
  v[x] = uv_one(v[x], q[x], c[x], l[x]);
  q[x] = 0.0f;
}

// One piece, instance chosen by the locator (circuit_gpu.cu:321-346).
static __global__ void __launch_bounds__(256)
    uv_piece_kernel(uint32_t first, uint32_t n, const int32_t *__restrict__ locator,
                    ckt_nodes pvt, ckt_nodes shr) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const uint32_t x = first + i;
  const ckt_nodes &s = locator[x] ? pvt : shr;
  s.voltage[x] = uv_one(s.voltage[x], s.charge[x], s.capacitance[x], s.leakage[x]);
  s.charge[x] = 0.0f;
}

// distribute_charge + update_voltages in one node pass (the fused loop): the
// staged gather of dc_block, and each node's final charge goes straight into
// the voltage update instead of through memory.  Same order, same bits as
// dc_all_kernel followed by the update_voltages kernels.
static __global__ void __launch_bounds__(kDcBlock)
    dcuv_kernel(uint32_t N, const uint32_t *__restrict__ off, const uint32_t *__restrict__ ent,
                const float *__restrict__ I0, const float *__restrict__ I9,
                float *__restrict__ charge, float *__restrict__ voltage,
                const float *__restrict__ cap, const float *__restrict__ leak, float dt) {
  __shared__ float sval[kDcChunk];
  __shared__ uint32_t smask[kDcChunk / 32];
  const uint32_t x0 = blockIdx.x * kDcBlock;
  const uint32_t xe = min(N, x0 + kDcBlock);
  const uint32_t x = x0 + threadIdx.x;
  float v = 0.0f, c = 1.0f, l = 0.0f;
  if (x < xe) {  // independent of the gather: in flight while it runs
    v = voltage[x];
    c = cap[x];
    l = leak[x];
  }
  const float q = dc_block<kDcBlock, false, false>(x0, xe, off, ent, I0, I9, charge, dt, sval,
                                                  smask);
  if (x < xe) {
    voltage[x] = uv_one(v, q, c, l);
    charge[x] = 0.0f;
  }
}

// ---------------------------------------------------------------------------
// Wire validation (sanity_check_positions, circuit_gpu.cu:151-184, with an
// error word instead of assert).  Records the smallest failing wire index.
// ---------------------------------------------------------------------------
static __global__ void __launch_bounds__(256)
    sanity_kernel(ckt_piece piece, const uint32_t *__restrict__ in_ptr,
                  const uint32_t *__restrict__ out_ptr, const uint8_t *__restrict__ in_loc,
                  const uint8_t *__restrict__ out_loc, uint32_t num_nodes_total,
                  unsigned long long *first_bad) {
  const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= piece.num_wires) return;
  const uint32_t w = piece.first_wire + t;
  const uint32_t a = in_ptr[w], b = out_ptr[w];
  const uint8_t la = in_loc[w], lb = out_loc[w];
  const uint32_t lo = piece.first_node, hi = piece.first_node + piece.num_nodes;
  bool ok = la <= CKT_SHARED_PTR && lb <= CKT_GHOST_PTR;  // in-node is never a ghost
  ok = ok && a >= lo && a < hi;
  ok = ok && b < num_nodes_total;
  if (ok) {
    const bool b_inside = b >= lo && b < hi;
    ok = (lb == CKT_GHOST_PTR) ? !b_inside : b_inside;
  }
  if (!ok) atomicMin(first_bad, (unsigned long long)w);
}

}  // namespace ckt
