// ckt_internal.h -- shared helpers of the circuit library (not part of the ABI).
#pragma once

#include <cuda_runtime.h>
#include <nvtx3/nvToolsExt.h>

#include <cstdarg>
#include <cstdint>
#include <cstdio>
#include <string>
#include <vector>

#include "ckt.h"

namespace ckt {

// Records the failure message for ckt_last_error() and returns `status`.
int set_error(int status, const char *fmt, ...);

inline cudaStream_t as_stream(void *s) { return reinterpret_cast<cudaStream_t>(s); }

// A named NVTX range over one library call (host side), for nsys / ncu
// range filters; costs nothing without an attached tool.
struct NvtxRange {
  explicit NvtxRange(const char *name) { nvtxRangePushA(name); }
  ~NvtxRange() { nvtxRangePop(); }
  NvtxRange(const NvtxRange &) = delete;
  NvtxRange &operator=(const NvtxRange &) = delete;
};

#define CKT_CUDA(expr)                                                          \
  do {                                                                          \
    cudaError_t ckt_err_ = (expr);                                              \
    if (ckt_err_ != cudaSuccess)                                                \
      return ::ckt::set_error(CKT_ECUDA, "%s failed: %s (%s:%d)", #expr,        \
                              cudaGetErrorString(ckt_err_), __FILE__, __LINE__); \
  } while (0)

#define CKT_CHECK_LAUNCH()                                                      \
  do {                                                                          \
    cudaError_t ckt_err_ = cudaGetLastError();                                  \
    if (ckt_err_ != cudaSuccess)                                                \
      return ::ckt::set_error(CKT_ECUDA, "kernel launch failed: %s (%s:%d)",    \
                              cudaGetErrorString(ckt_err_), __FILE__, __LINE__); \
  } while (0)

#define CKT_REQUIRE(cond, ...)                                                  \
  do {                                                                          \
    if (!(cond)) return ::ckt::set_error(CKT_EINVAL, __VA_ARGS__);              \
  } while (0)

// Entry encodings of the contribution graph.
//   node CSR entry: (wire << 2) | (end << 1) | starts_new_piece_group
//   piece CSR entry: (wire << 1) | end          (end: 0 = in, 1 = out)
//   node offset word: offset | (node_is_private << 31)
constexpr uint32_t kPrivateBit = 0x80000000u;
constexpr uint32_t kOffsetMask = 0x7fffffffu;
constexpr int64_t kMaxWires = (int64_t)1 << 29;  // 2W entries and offsets fit 31 bits

inline unsigned grid_for(uint64_t n, unsigned block = 256) {
  return (unsigned)((n + block - 1) / block);
}

// Validates the wires against the pieces and builds the whole-circuit CSR
// (node offsets with the private bit, entries in reduction order).
// When slots is non-null it also receives, per wire, the CSR positions of
// its in-end and out-end ([2W]: in at 2w, out at 2w+1).
int build_node_csr(const ckt_piece *pieces, int32_t num_pieces, uint32_t num_nodes,
                   const uint32_t *in_ptr, const uint32_t *out_ptr, const uint8_t *in_loc,
                   const uint8_t *out_loc, std::vector<uint32_t> &off, std::vector<uint32_t> &ent,
                   int64_t *num_wires, std::vector<uint32_t> *slots = nullptr);

// calc_new_currents over wires [first, first + n) (any mode/initialisation).
int launch_cnc(uint32_t first, uint32_t n, const ckt_wires &w, const float *vp, const float *vs,
               const float *vg, const ckt_params *p, cudaStream_t s);

int validate_wires(const ckt_wires &w);
int validate_nodes(const ckt_nodes &n, const char *what);
int validate_params(const ckt_params *p);

}  // namespace ckt

// The graph object behind the opaque ckt_graph handle.
struct ckt_graph {
  int64_t W = 0, N = 0;
  int32_t P = 0;
  std::vector<ckt_piece> pieces;
  // Whole-circuit node CSR (device).
  uint32_t *node_off = nullptr;  // [N + 1]
  uint32_t *node_ent = nullptr;  // [2W]
  // Per-piece CSR over the nodes each piece touches (device), concatenated
  // in piece order; piece k owns touched slots [touch_first[k],
  // touch_first[k+1]).
  std::vector<int64_t> touch_first;  // host, [P + 1]
  uint32_t *touch_node = nullptr;    // [T]
  uint8_t *touch_loc = nullptr;      // [T]
  uint32_t *touch_off = nullptr;     // [T + 1] into piece_ent
  uint32_t *piece_ent = nullptr;     // [2W]
  // Two-pass distribute_charge: each wire end's CSR position, a bit per CSR
  // entry marking the start of a piece group, and the contribution buffer.
  uint32_t *slot_in = nullptr, *slot_out = nullptr;  // [W]
  uint32_t *gstart = nullptr;                        // [ceil(2W / 32)]
  float *contrib = nullptr;                          // [2W] scratch
  int64_t device_bytes = 0;
};
