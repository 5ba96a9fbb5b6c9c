// ckt_probe.cu -- FP32-pipe peak probe used as the roofline denominator of
// calc_new_currents (the measured-peak file holds HBM and tensor peaks only).
// Eight independent FMA chains per thread keep all four SM sub-partitions'
// FP32 pipes issuing every cycle.
#include "ckt_internal.h"
#include "ckt_tools.h"

namespace ckt {

__global__ void __launch_bounds__(256) fma_probe_kernel(int32_t iters, float *sink) {
  float a[8];
  const float m = 1.0f + 1e-7f * (threadIdx.x & 7), c = 1e-7f;
#pragma unroll
  for (int i = 0; i < 8; i++) a[i] = (float)(threadIdx.x + i);
#pragma unroll 1
  for (int32_t j = 0; j < iters; j++) {
#pragma unroll
    for (int r = 0; r < 16; r++) {
#pragma unroll
      for (int i = 0; i < 8; i++) a[i] = __fmaf_rn(a[i], m, c);
    }
  }
  float s = 0.f;
#pragma unroll
  for (int i = 0; i < 8; i++) s += a[i];
  if (s == 12345.678f) sink[0] = s;  // keeps the chains live
}

// Same work as paired FMAs: four independent f32x2 chains per thread.
__global__ void __launch_bounds__(256) fma2_probe_kernel(int32_t iters, float *sink) {
  float2 a[4];
  const float mm = 1.0f + 1e-7f * (threadIdx.x & 7);
  const float2 m = make_float2(mm, mm), c = make_float2(1e-7f, 1e-7f);
#pragma unroll
  for (int i = 0; i < 4; i++) a[i] = make_float2((float)(threadIdx.x + 2 * i), (float)(threadIdx.x + 2 * i + 1));
#pragma unroll 1
  for (int32_t j = 0; j < iters; j++) {
#pragma unroll
    for (int r = 0; r < 16; r++) {
#pragma unroll
      for (int i = 0; i < 4; i++) a[i] = __ffma2_rn(a[i], m, c);
    }
  }
  float s = 0.f;
#pragma unroll
  for (int i = 0; i < 4; i++) s += a[i].x + a[i].y;
  if (s == 12345.678f) sink[0] = s;
}

}  // namespace ckt

extern "C" int ckt_fp32_fma_probe(uint32_t blocks, int32_t iters, int32_t paired, float *sink,
                                  void *stream) {
  CKT_REQUIRE(blocks > 0 && iters > 0 && sink != nullptr, "bad probe arguments");
  if (paired)
    ckt::fma2_probe_kernel<<<blocks, 256, 0, ckt::as_stream(stream)>>>(iters, sink);
  else
    ckt::fma_probe_kernel<<<blocks, 256, 0, ckt::as_stream(stream)>>>(iters, sink);
  CKT_CHECK_LAUNCH();
  return CKT_OK;
}
