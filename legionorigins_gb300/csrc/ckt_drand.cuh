// ckt_drand.cuh -- the generator's drand48 expressions evaluated exactly in
// integer arithmetic where that is possible.
//
// load_circuit (apps/circuit/circuit.cc:1121-1186) turns each 48-bit LCG state
// x into u = x * 2^-48 (drand48) and evaluates a few double expressions.
// Several of them are exact rationals over 2^48 before their final rounding,
// and the others round a product of x by an integer to 53 bits; both can be
// computed with integer instructions, which matters on GPUs whose FP64 rate
// is a small fraction of the FP32 rate.  Each helper states the expression it
// reproduces and why the result is bit-identical.  The host build of this
// header (plain C++) lets the CPU check every helper against the double
// arithmetic it replaces.
#pragma once

#include <cstdint>
#include <cstring>

#if defined(__CUDACC__)
#define CKT_HD __host__ __device__ __forceinline__
#else
#define CKT_HD inline
#endif

namespace ckt {
namespace drand {

CKT_HD int msb64(uint64_t v) {  // index of the highest set bit, v != 0
#if defined(__CUDA_ARCH__)
  return 63 - __clzll((long long)v);
#else
  return 63 - __builtin_clzll(v);
#endif
}

CKT_HD uint64_t mulhi64(uint64_t a, uint64_t b) {
#if defined(__CUDA_ARCH__)
  return __umul64hi(a, b);
#else
  return (uint64_t)(((unsigned __int128)a * b) >> 64);
#endif
}

// drand48's value u = x * 2^-48 (x < 2^48), assembled from its bits: exact.
CKT_HD double value(uint64_t x) {
  if (x == 0) return 0.0;
  const int m = msb64(x);  // <= 47
  const uint64_t bits = ((uint64_t)(m - 48 + 1023) << 52) | ((x << (52 - m)) & ((1ull << 52) - 1));
  double d;
  memcpy(&d, &bits, sizeof(d));
  return d;
}

// Rounds the integer q = hi * 2^64 + lo (< 2^80) to 53 significant bits, to
// nearest with ties to even, as the double product x * n does, and returns
// floor(result / 2^48).
CKT_HD uint64_t rn53_shr48(uint64_t hi, uint64_t lo) {
  if (hi == 0 && lo == 0) return 0;
  const int m = hi ? 64 + msb64(hi) : msb64(lo);
  if (m <= 52) return lo >> 48;  // exact (hi is 0)
  const int shift = m - 52;       // 1 .. 27
  uint64_t r = (lo >> shift) | (hi << (64 - shift));
  const uint64_t rem = lo & ((1ull << shift) - 1), half = 1ull << (shift - 1);
  if (rem > half || (rem == half && (r & 1u))) r++;
  return r >> (48 - shift);
}

// (int)(drand48() * n): u * n rounded to a double, truncated (n < 2^31).
CKT_HD uint32_t trunc_mul(uint64_t x, uint32_t n) {
  return (uint32_t)rn53_shr48(mulhi64(x, n), x * (uint64_t)n);
}

// Threshold of the in-piece test: ceil(pct * 2^48), 0 when pct <= 0.
inline uint64_t pct_threshold(double pct) {
  const double t = pct * 281474976710656.0;  // * 2^48, exact
  if (!(t > 0)) return 0;
  if (t >= 9223372036854775808.0) return ~0ull;
  const uint64_t f = (uint64_t)t;
  return ((double)f == t) ? f : f + 1;
}

// 100 * drand48() < pct: 100 * u rounded to a double (100 x < 2^55 keeps its
// top 53 bits), compared with pct; as integers, RN53(100 x) < pct * 2^48.
CKT_HD bool pct_below(uint64_t x, uint64_t threshold) {
  const uint64_t p = 100 * x;
  uint64_t r = p;
  if (p >> 53) {
    const int shift = msb64(p) - 52;  // 1 or 2
    r = p >> shift;
    const uint64_t rem = p & ((1ull << shift) - 1), half = 1ull << (shift - 1);
    if (rem > half || (rem == half && (r & 1u))) r++;
    r <<= shift;
  }
  return r < threshold;
}

CKT_HD float u64_to_float(uint64_t v) {
#if defined(__CUDA_ARCH__)
  return __ull2float_rn(v);
#else
  return (float)v;
#endif
}

CKT_HD float i64_to_float(int64_t v) {
#if defined(__CUDA_ARCH__)
  return __ll2float_rn(v);
#else
  return (float)v;
#endif
}

constexpr float kTwoM48 = 3.5527136788005009e-15f;  // 2^-48, exact

// (float)(drand48() * 10 + 1) = (10 x + 2^48) / 2^48 exactly (< 2^52), so the
// only rounding is the float conversion.
CKT_HD float resistance(uint64_t x) {
  return u64_to_float(10 * x + (1ull << 48)) * kTwoM48;
}

// (float)(2 * drand48() - 1) = (2 x - 2^48) / 2^48 exactly.
CKT_HD float node_voltage(uint64_t x) {
  return i64_to_float((int64_t)(2 * x) - (int64_t)(1ull << 48)) * kTwoM48;
}

// (float)(drand48() + 1) = (x + 2^48) / 2^48 exactly.
CKT_HD float node_capacitance(uint64_t x) {
  return u64_to_float(x + (1ull << 48)) * kTwoM48;
}

}  // namespace drand
}  // namespace ckt
