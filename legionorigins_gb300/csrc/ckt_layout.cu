// ckt_layout.cu -- conversion between the reference's array-of-structs
// instances (CircuitWire, 128 bytes; CircuitNode, 16 bytes;
// apps/circuit/circuit.h:35-54) and the structure-of-arrays views the kernels
// use.  A warp moves 32 wires: it reads their 4 KB of AoS as 16-byte vectors
// into shared memory (coalesced), then writes each SoA field as one
// contiguous 128-byte run (coalesced) -- and the reverse.  Pointers may be
// device memory or host memory mapped for the device (zero-copy).
#include "ckt_internal.h"

namespace ckt {
namespace {

// Word offsets inside CircuitWire (32 x 4-byte words).
enum : int {
  kIn = 0, kOut = 1, kInLoc = 2, kOutLoc = 3, kL = 4, kR = 5, kCur = 6, kC = 16, kVol = 17,
  kWireWords = 32
};

constexpr int kWarpsPerBlock = 8;

__global__ void __launch_bounds__(256)
    wires_from_aos_kernel(const uint4 *__restrict__ aos, int64_t W, uint32_t *in_ptr,
                          uint32_t *out_ptr, uint8_t *in_loc, uint8_t *out_loc, float *L,
                          float *R, float *C, float *cur, float *vol, int64_t S) {
  __shared__ uint32_t sm[kWarpsPerBlock][32 * (kWireWords + 1)];  // +1 word per wire: no bank conflicts
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int64_t w0 = ((int64_t)blockIdx.x * kWarpsPerBlock + warp) * 32;
  if (w0 >= W) return;
  const int nw = (int)(W - w0 < 32 ? W - w0 : 32);
  uint32_t *s = sm[warp];
  // 32 wires = 256 uint4; lane j loads vectors j, j+32, ..., j+224
  for (int v = lane; v < nw * 8; v += 32) {
    const uint4 q = aos[w0 * 8 + v];
    const int wire = v >> 3, word = (v & 7) * 4;
    uint32_t *d = s + wire * (kWireWords + 1) + word;
    d[0] = q.x; d[1] = q.y; d[2] = q.z; d[3] = q.w;
  }
  __syncwarp();
  if (lane < nw) {
    const uint32_t *f = s + lane * (kWireWords + 1);
    const int64_t w = w0 + lane;
    in_ptr[w] = f[kIn];
    out_ptr[w] = f[kOut];
    in_loc[w] = (uint8_t)f[kInLoc];
    out_loc[w] = (uint8_t)f[kOutLoc];
    L[w] = __uint_as_float(f[kL]);
    R[w] = __uint_as_float(f[kR]);
    C[w] = __uint_as_float(f[kC]);
#pragma unroll
    for (int k = 0; k < 10; k++) cur[k * S + w] = __uint_as_float(f[kCur + k]);
#pragma unroll
    for (int k = 0; k < 9; k++) vol[k * S + w] = __uint_as_float(f[kVol + k]);
  }
}

__global__ void __launch_bounds__(256)
    wires_to_aos_kernel(uint4 *__restrict__ aos, int64_t W, const uint32_t *in_ptr,
                        const uint32_t *out_ptr, const uint8_t *in_loc, const uint8_t *out_loc,
                        const float *L, const float *R, const float *C, const float *cur,
                        const float *vol, int64_t S) {
  __shared__ uint32_t sm[kWarpsPerBlock][32 * (kWireWords + 1)];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int64_t w0 = ((int64_t)blockIdx.x * kWarpsPerBlock + warp) * 32;
  if (w0 >= W) return;
  const int nw = (int)(W - w0 < 32 ? W - w0 : 32);
  uint32_t *s = sm[warp];
  if (lane < nw) {
    uint32_t *f = s + lane * (kWireWords + 1);
    const int64_t w = w0 + lane;
    f[kIn] = in_ptr[w];
    f[kOut] = out_ptr[w];
    f[kInLoc] = in_loc[w];
    f[kOutLoc] = out_loc[w];
    f[kL] = __float_as_uint(L[w]);
    f[kR] = __float_as_uint(R[w]);
    f[kC] = __float_as_uint(C[w]);
#pragma unroll
    for (int k = 0; k < 10; k++) f[kCur + k] = __float_as_uint(cur[k * S + w]);
#pragma unroll
    for (int k = 0; k < 9; k++) f[kVol + k] = __float_as_uint(vol[k * S + w]);
#pragma unroll
    for (int k = kVol + 9; k < kWireWords; k++) f[k] = 0u;  // the six pad words
  }
  __syncwarp();
  for (int v = lane; v < nw * 8; v += 32) {
    const int wire = v >> 3, word = (v & 7) * 4;
    const uint32_t *d = s + wire * (kWireWords + 1) + word;
    aos[w0 * 8 + v] = make_uint4(d[0], d[1], d[2], d[3]);
  }
}

// CircuitNode {charge, voltage, capacitance, leakage}: one float4 per node.
__global__ void __launch_bounds__(256)
    nodes_from_aos_kernel(const float4 *__restrict__ aos, int64_t N, float *charge,
                          float *voltage, float *cap, float *leak) {
  const int64_t x = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (x >= N) return;
  const float4 q = aos[x];
  charge[x] = q.x;
  voltage[x] = q.y;
  cap[x] = q.z;
  leak[x] = q.w;
}

__global__ void __launch_bounds__(256)
    nodes_to_aos_kernel(float4 *__restrict__ aos, int64_t N, const float *charge,
                        const float *voltage, const float *cap, const float *leak) {
  const int64_t x = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (x >= N) return;
  aos[x] = make_float4(charge[x], voltage[x], cap[x], leak[x]);
}

int check_aligned(const void *p, const char *what) {
  CKT_REQUIRE((reinterpret_cast<uintptr_t>(p) & 15u) == 0, "%s must be 16-byte aligned", what);
  return CKT_OK;
}

}  // namespace
}  // namespace ckt

using namespace ckt;

extern "C" {

int ckt_wires_from_aos(const void *aos, int64_t num_wires, ckt_wires soa, void *stream) {
  CKT_REQUIRE(num_wires >= 0, "num_wires must be >= 0");
  if (num_wires == 0) return CKT_OK;
  int rc;
  if ((rc = validate_wires(soa)) || (rc = check_aligned(aos, "the AoS wire array"))) return rc;
  CKT_REQUIRE(soa.seg_stride >= num_wires, "seg_stride %lld < %lld wires",
              (long long)soa.seg_stride, (long long)num_wires);
  const unsigned blocks = (unsigned)((num_wires + 32 * kWarpsPerBlock - 1) / (32 * kWarpsPerBlock));
  wires_from_aos_kernel<<<blocks, 256, 0, as_stream(stream)>>>(
      static_cast<const uint4 *>(aos), num_wires, const_cast<uint32_t *>(soa.in_ptr),
      const_cast<uint32_t *>(soa.out_ptr), const_cast<uint8_t *>(soa.in_loc),
      const_cast<uint8_t *>(soa.out_loc), const_cast<float *>(soa.inductance),
      const_cast<float *>(soa.resistance), const_cast<float *>(soa.capacitance), soa.current,
      soa.voltage, soa.seg_stride);
  CKT_CHECK_LAUNCH();
  return CKT_OK;
}

int ckt_wires_to_aos(ckt_wires soa, int64_t num_wires, void *aos, void *stream) {
  CKT_REQUIRE(num_wires >= 0, "num_wires must be >= 0");
  if (num_wires == 0) return CKT_OK;
  int rc;
  if ((rc = validate_wires(soa)) || (rc = check_aligned(aos, "the AoS wire array"))) return rc;
  CKT_REQUIRE(soa.seg_stride >= num_wires, "seg_stride %lld < %lld wires",
              (long long)soa.seg_stride, (long long)num_wires);
  const unsigned blocks = (unsigned)((num_wires + 32 * kWarpsPerBlock - 1) / (32 * kWarpsPerBlock));
  wires_to_aos_kernel<<<blocks, 256, 0, as_stream(stream)>>>(
      static_cast<uint4 *>(aos), num_wires, soa.in_ptr, soa.out_ptr, soa.in_loc, soa.out_loc,
      soa.inductance, soa.resistance, soa.capacitance, soa.current, soa.voltage, soa.seg_stride);
  CKT_CHECK_LAUNCH();
  return CKT_OK;
}

int ckt_nodes_from_aos(const void *aos, int64_t num_nodes, ckt_nodes soa, void *stream) {
  CKT_REQUIRE(num_nodes >= 0, "num_nodes must be >= 0");
  if (num_nodes == 0) return CKT_OK;
  int rc;
  if ((rc = validate_nodes(soa, "soa")) || (rc = check_aligned(aos, "the AoS node array"))) return rc;
  nodes_from_aos_kernel<<<grid_for(num_nodes), 256, 0, as_stream(stream)>>>(
      static_cast<const float4 *>(aos), num_nodes, soa.charge, soa.voltage,
      const_cast<float *>(soa.capacitance), const_cast<float *>(soa.leakage));
  CKT_CHECK_LAUNCH();
  return CKT_OK;
}

int ckt_nodes_to_aos(ckt_nodes soa, int64_t num_nodes, void *aos, void *stream) {
  CKT_REQUIRE(num_nodes >= 0, "num_nodes must be >= 0");
  if (num_nodes == 0) return CKT_OK;
  int rc;
  if ((rc = validate_nodes(soa, "soa")) || (rc = check_aligned(aos, "the AoS node array"))) return rc;
  nodes_to_aos_kernel<<<grid_for(num_nodes), 256, 0, as_stream(stream)>>>(
      static_cast<float4 *>(aos), num_nodes, soa.charge, soa.voltage, soa.capacitance,
      soa.leakage);
  CKT_CHECK_LAUNCH();
  return CKT_OK;
}

}  // extern "C"
