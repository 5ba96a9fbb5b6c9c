// ckt_divcheck.cu -- GPU checks of EXACT mode's quotients (ckt_divide.cuh)
// against the divide routine.  Verification tooling: built into
// libckt_tools.so, never into the product library.
#include <algorithm>

#include "ckt_divide.cuh"
#include "ckt_internal.h"
#include "ckt_tools.h"

namespace ckt {

__device__ __forceinline__ bool same_float(float a, float b) {
  return (a != a && b != b) || __float_as_uint(a) == __float_as_uint(b);
}

__device__ __forceinline__ void warp_add(unsigned long long *dst, uint32_t v) {
  v = __reduce_add_sync(0xffffffffu, v);
  if ((threadIdx.x & 31u) == 0u && v) atomicAdd(dst, (unsigned long long)v);
}

// Every dividend bit pattern in [begin, begin + count); the grid covers it
// with a grid-stride loop whose trip count is uniform across the warp.
__global__ void __launch_bounds__(256)
    dt_quotient_check_kernel(uint64_t begin, uint64_t count, unsigned long long *counts) {
  const float dt = __uint_as_float(kDtBits);
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  const uint64_t rounds = (count + stride - 1) / stride;
  const uint64_t t = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  uint32_t bad_trusted = 0, bad_other = 0;
  for (uint64_t r = 0; r < rounds; r++) {
    const uint64_t i = r * stride + t;
    if (i < count) {
      const float a = __uint_as_float((uint32_t)(begin + i));
      if (!same_float(dt_quot(a), __fdiv_rn(a, dt))) {
        if (!(fabsf(a) < kDtTiny) || a == 0.0f) bad_trusted++;
        else bad_other++;
      }
    }
  }
  warp_add(counts + 0, bad_trusted);
  warp_add(counts + 1, bad_other);
}

__device__ __forceinline__ uint64_t mix64(uint64_t x) {  // SplitMix64 finaliser
  x ^= x >> 30;
  x *= 0xbf58476d1ce4e5b9ull;
  x ^= x >> 27;
  x *= 0x94d049bb133111ebull;
  return x ^ (x >> 31);
}

// A float of random sign, mantissa and binary exponent in [e0, e1].
__device__ __forceinline__ float rand_float(uint64_t h, int e0, int e1) {
  const uint32_t span = (uint32_t)(e1 - e0 + 1);
  const int e = e0 + (int)((uint32_t)(h >> 32) % span);
  const uint32_t bits = (uint32_t)((e + 127) << 23) | ((uint32_t)h & 0x7fffffu) |
                        ((uint32_t)(h >> 23) & 0x80000000u);
  return __uint_as_float(bits);
}

// Any dividend: special values, the guard's edges, or random bit patterns.
__device__ __forceinline__ float rand_dividend(uint64_t h, float lo, float hi) {
  const uint32_t sel = (uint32_t)(h >> 56);
  const uint32_t sign = (uint32_t)(h >> 55) & 1u ? 0x80000000u : 0u;
  const float s = sign ? -1.0f : 1.0f;
  switch (sel & 15u) {
    case 0: {
      const float sp[8] = {0.0f, __uint_as_float(0x7f800000u), __uint_as_float(0x7fc00000u),
                           __uint_as_float(1u), __uint_as_float(0x007fffffu),
                           __uint_as_float(0x7f7fffffu), lo, hi};
      return s * sp[(sel >> 4) & 7u];
    }
    case 1:  // just inside or outside the guarded range
      return s * __uint_as_float(__float_as_uint((sel & 16u) ? lo : hi) + (uint32_t)(h & 7u) - 3u);
    case 2:
    case 3:
    case 4:
    case 5:  // any bit pattern: subnormals, NaN payloads, infinities included
      return __uint_as_float((uint32_t)h ^ (uint32_t)(h >> 32));
    default:  // normal floats over the whole exponent range
      return rand_float(h, -126, 127);
  }
}

__global__ void __launch_bounds__(256)
    recip_quotient_check_kernel(uint64_t seed, uint64_t count, int32_t divisor, int32_t near_ties,
                                unsigned long long *counts) {
  const int e0 = divisor == 0 ? -8 : -30, e1 = -e0 - 1;  // kRMin..kRMax, kCMin..kCMax
  const float lo = divisor == 0 ? kRLo : kCLo, hi = divisor == 0 ? kRHi : kCHi;
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  const uint64_t rounds = (count + stride - 1) / stride;
  const uint64_t t = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  uint32_t bad = 0, fast = 0, drawn = 0;
  for (uint64_t r = 0; r < rounds; r++) {
    const uint64_t i = r * stride + t;
    if (i >= count) continue;
    const uint64_t h1 = mix64(seed * 0x9e3779b97f4a7c15ull + 2 * i + 1);
    const uint64_t h2 = mix64(h1 ^ 0x632be59bd9b4e019ull);
    const float b = rand_float(h1, e0, e1);  // the divisor, inside the eligible range
    float a;
    if (near_ties) {
      // a = RN(b * m) with m a midpoint between two floats of the quotient's
      // range: a/b then lies within about an ulp of a rounding boundary.
      const float q = rand_float(h2, -60, 90);
      const double m = (double)q + 0.5 * ((double)__uint_as_float(__float_as_uint(fabsf(q)) + 1u) -
                                          (double)fabsf(q)) * (q < 0.0f ? -1.0 : 1.0);
      a = __double2float_rn((double)b * m);
      a = __uint_as_float(__float_as_uint(a) + (uint32_t)(h2 >> 61) - 3u);  // and its neighbours
    } else {
      a = rand_dividend(h2, lo, hi);
    }
    const Recip k = make_recip(b);
    const float got = quot_guarded(a, b, k, lo, hi);
    bad += !same_float(got, __fdiv_rn(a, b));
    fast += !outside(a, lo, hi);
    drawn++;
  }
  warp_add(counts + 0, bad);
  warp_add(counts + 1, fast);
  warp_add(counts + 2, drawn);
}

// wide_quot, the quotient of EXACT mode's phases that leave the guarded
// range, against the divide routine: dividends of every class -- huge up to
// FLT_MAX, tiny down to the smallest subnormal, the guarded range, zeros,
// infinities, NaN, quotients within an ulp of a rounding boundary or of the
// overflow threshold -- except those whose quotient may be subnormal
// (subnormal_quot), which the steppers leave to the divide routine.
__global__ void __launch_bounds__(256)
    wide_quotient_check_kernel(uint64_t seed, uint64_t count, int32_t divisor,
                               unsigned long long *counts) {
  const int be0 = divisor == 0 ? -8 : -30, be1 = -be0 - 1;
  const float lo = divisor == 0 ? kRLo : kCLo, hi = divisor == 0 ? kRHi : kCHi;
  const int lo_e = divisor == 0 ? -50 : -40, hi_e = divisor == 0 ? 100 : 90;
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  const uint64_t rounds = (count + stride - 1) / stride;
  const uint64_t t = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  uint32_t bad = 0, out = 0, drawn = 0;
  for (uint64_t r = 0; r < rounds; r++) {
    const uint64_t i = r * stride + t;
    if (i >= count) continue;
    const uint64_t h1 = mix64(seed * 0x9e3779b97f4a7c15ull + 2 * i + 1);
    const uint64_t h2 = mix64(h1 ^ 0x632be59bd9b4e019ull);
    const float b = rand_float(h1, be0, be1);
    const float sgn = (h2 >> 20) & 1u ? -1.0f : 1.0f;
    const float fmax = __uint_as_float(0x7f7fffffu);
    float a;
    switch ((uint32_t)((h2 >> 56) % 8u)) {
      case 0:
        a = rand_float(h2, hi_e, 127);
        break;
      case 1: {
        const int e = -149 + (int)((uint32_t)(h2 >> 32) % (uint32_t)(lo_e + 149));
        a = sgn * ldexpf(1.0f + (float)(h2 & 0x7fffffu) * 0x1p-23f, e);
        break;
      }
      case 2: {
        const float sp[8] = {0.0f, __uint_as_float(0x7f800000u), __uint_as_float(0x7fc00000u),
                             fmax, lo, hi, __uint_as_float(__float_as_uint(hi) + 1u),
                             __uint_as_float(__float_as_uint(lo) - 1u)};
        a = sgn * sp[(h2 >> 8) & 7u];
        break;
      }
      case 3: {
        const double m = (double)fmax + 0x1p103 * ((double)((h2 >> 8) & 7u) - 3.5) / 2.0;
        a = sgn * __double2float_rn((double)b * m);
        a = __uint_as_float(__float_as_uint(a) + (uint32_t)((h2 >> 12) & 3u) - 1u);
        break;
      }
      case 4:
      case 5: {
        const float q = (h2 >> 9) & 1u ? rand_float(h2, 60, 126) : rand_float(h2, -125, -60);
        const double mid = (double)q + 0.5 * ((double)__uint_as_float(__float_as_uint(fabsf(q)) + 1u) -
                                              (double)fabsf(q)) * (q < 0.0f ? -1.0 : 1.0);
        a = __double2float_rn((double)b * mid);
        a = __uint_as_float(__float_as_uint(a) + (uint32_t)((h2 >> 12) & 7u) - 3u);
        break;
      }
      default:
        a = rand_float(h2, -126, 127);
        break;
    }
    const Recip k = make_recip(b);
    if (subnormal_quot(a, k)) continue;
    bad += !same_float(wide_quot(a, k, lo, hi), __fdiv_rn(a, b));
    out += outside(a, lo, hi);
    drawn++;
  }
  warp_add(counts + 0, bad);
  warp_add(counts + 1, out);
  warp_add(counts + 2, drawn);
}

}  // namespace ckt

using namespace ckt;

extern "C" int ckt_check_dt_quotient(uint64_t begin, uint64_t count, unsigned long long *counts,
                                     void *stream) {
  CKT_REQUIRE(counts != nullptr, "counts is NULL");
  CKT_REQUIRE(count <= (1ull << 32) && begin + count <= (1ull << 32),
              "dividend range [%llu, %llu) exceeds the 2^32 float bit patterns",
              (unsigned long long)begin, (unsigned long long)(begin + count));
  if (count == 0) return CKT_OK;
  int dev = 0, sms = 0;
  CKT_CUDA(cudaGetDevice(&dev));
  CKT_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  const uint64_t want = (count + 255) / 256;
  const unsigned grid = (unsigned)std::min<uint64_t>(want, (uint64_t)sms * 8);
  dt_quotient_check_kernel<<<grid, 256, 0, as_stream(stream)>>>(begin, count, counts);
  CKT_CHECK_LAUNCH();
  return CKT_OK;
}

extern "C" int ckt_check_recip_quotient(uint64_t seed, uint64_t count, int32_t divisor,
                                        int32_t near_ties, unsigned long long *counts,
                                        void *stream) {
  CKT_REQUIRE(counts != nullptr, "counts is NULL");
  CKT_REQUIRE(divisor == 0 || divisor == 1, "divisor must be 0 (R) or 1 (C, dt), got %d",
              divisor);
  if (count == 0) return CKT_OK;
  int dev = 0, sms = 0;
  CKT_CUDA(cudaGetDevice(&dev));
  CKT_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  const uint64_t want = (count + 255) / 256;
  const unsigned grid = (unsigned)std::min<uint64_t>(want, (uint64_t)sms * 8);
  recip_quotient_check_kernel<<<grid, 256, 0, as_stream(stream)>>>(seed, count, divisor,
                                                                   near_ties, counts);
  CKT_CHECK_LAUNCH();
  return CKT_OK;
}

extern "C" int ckt_check_wide_quotient(uint64_t seed, uint64_t count, int32_t divisor,
                                       unsigned long long *counts, void *stream) {
  CKT_REQUIRE(counts != nullptr, "counts is NULL");
  CKT_REQUIRE(divisor == 0 || divisor == 1, "divisor must be 0 (R) or 1 (C), got %d", divisor);
  if (count == 0) return CKT_OK;
  int dev = 0, sms = 0;
  CKT_CUDA(cudaGetDevice(&dev));
  CKT_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  const uint64_t want = (count + 255) / 256;
  const unsigned grid = (unsigned)std::min<uint64_t>(want, (uint64_t)sms * 8);
  wide_quotient_check_kernel<<<grid, 256, 0, as_stream(stream)>>>(seed, count, divisor, counts);
  CKT_CHECK_LAUNCH();
  return CKT_OK;
}
