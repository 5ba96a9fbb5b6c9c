// ckt_noalloc.cu -- the wire check for callers that cannot allocate memory.
//
// ckt_sanity_check_wires allocates an error word per call.  Some callers
// may not allocate device memory at all: a runtime that reserves the GPU's
// memory for its own pools when it starts (so nothing is left to allocate
// from inside a task), code that must not call cudaMalloc/cudaFree because
// they can synchronise the whole device, or a service held to a fixed
// memory budget.  This variant checks many pieces in one launch with its
// scratch -- each piece's descriptor and its smallest failing wire -- in a
// fixed array that exists on every GPU on which the library is loaded.
// Inputs and outputs move by strided copies directly between the caller's
// arrays and that array, so the call allocates nothing, on the host or the
// device.
#include <algorithm>
#include <climits>

#include "ckt_internal.h"

namespace ckt {
namespace {

// One piece's scratch: its descriptor and the smallest failing wire
// (ULLONG_MAX when none), 24 bytes.
struct NoAllocSlot {
  ckt_piece piece;
  unsigned long long first_bad;
};

// The scratch: CKT_NOALLOC_MAX_PIECES slots (96 KB), held by every GPU that
// loads the library until the process exits.  Every call uses it and leaves
// its contents behind.
static __device__ __align__(256) NoAllocSlot g_noalloc_scratch[CKT_NOALLOC_MAX_PIECES];

// The host-side name of the array is not a device address: look the
// address up, with the calling thread's device current.  Looked up on every
// call rather than cached, so a device reset or a re-created context between
// calls cannot leave a stale address behind (the lookup is cheap once the
// library's module is loaded on the device, which the first call does).
int scratch_for_current_device(NoAllocSlot **out) {
  void *p = nullptr;
  const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
  if (e != cudaSuccess || p == nullptr)
    return set_error(CKT_ECUDA, "cudaGetSymbolAddress of the wire-check scratch failed: %s",
                     cudaGetErrorString(e));
  *out = static_cast<NoAllocSlot *>(p);
  return CKT_OK;
}

// The wire checks of sanity_kernel (ckt_kernels.cuh), for piece blockIdx.y.
__global__ void __launch_bounds__(256)
    sanity_pieces_kernel(NoAllocSlot *slots, const uint32_t *__restrict__ in_ptr,
                         const uint32_t *__restrict__ out_ptr, const uint8_t *__restrict__ in_loc,
                         const uint8_t *__restrict__ out_loc, uint32_t num_nodes_total) {
  NoAllocSlot &slot = slots[blockIdx.y];
  const ckt_piece piece = slot.piece;
  const uint32_t lo = piece.first_node, hi = piece.first_node + piece.num_nodes;
  for (uint32_t t = blockIdx.x * blockDim.x + threadIdx.x; t < piece.num_wires;
       t += gridDim.x * blockDim.x) {
    const uint32_t w = piece.first_wire + t;
    const uint32_t a = in_ptr[w], b = out_ptr[w];
    const uint8_t la = in_loc[w], lb = out_loc[w];
    bool ok = la <= CKT_SHARED_PTR && lb <= CKT_GHOST_PTR;
    ok = ok && a >= lo && a < hi;
    ok = ok && b < num_nodes_total;
    if (ok) {
      const bool b_inside = b >= lo && b < hi;
      ok = (lb == CKT_GHOST_PTR) ? !b_inside : b_inside;
    }
    if (!ok) atomicMin(&slot.first_bad, (unsigned long long)w);
  }
}

}  // namespace
}  // namespace ckt

using namespace ckt;

extern "C" int ckt_sanity_check_pieces_noalloc(const ckt_piece *pieces, int32_t num_pieces,
                                               ckt_wires wires, uint32_t num_nodes_total,
                                               int64_t *first_bad, void *stream) {
  CKT_REQUIRE(num_pieces >= 0, "num_pieces must be >= 0 (got %d)", num_pieces);
  CKT_REQUIRE(num_pieces <= CKT_NOALLOC_MAX_PIECES,
              "num_pieces %d exceeds CKT_NOALLOC_MAX_PIECES (%d), the size of the "
              "allocation-free scratch",
              num_pieces, CKT_NOALLOC_MAX_PIECES);
  if (num_pieces == 0) return CKT_OK;
  CKT_REQUIRE(pieces != nullptr && first_bad != nullptr, "pieces or first_bad is NULL");
  uint32_t max_wires = 0;
  for (int32_t k = 0; k < num_pieces; k++) max_wires = std::max(max_wires, pieces[k].num_wires);
  if (max_wires > 0)
    CKT_REQUIRE(wires.in_ptr && wires.out_ptr && wires.in_loc && wires.out_loc,
                "wire pointer/location arrays are NULL");
  NoAllocSlot *slots = nullptr;
  int rc = scratch_for_current_device(&slots);
  if (rc) return rc;
  const cudaStream_t s = as_stream(stream);
  // Descriptors in, and every piece's result back to "none" (all ones):
  // the array still holds the previous call's values.
  CKT_CUDA(cudaMemcpy2DAsync(&slots[0].piece, sizeof(NoAllocSlot), pieces, sizeof(ckt_piece),
                             sizeof(ckt_piece), (size_t)num_pieces, cudaMemcpyHostToDevice, s));
  CKT_CUDA(cudaMemset2DAsync(&slots[0].first_bad, sizeof(NoAllocSlot), 0xff,
                             sizeof(unsigned long long), (size_t)num_pieces, s));
  if (max_wires > 0) {
    const unsigned gx = std::min<unsigned>(grid_for(max_wires), 1024u);
    sanity_pieces_kernel<<<dim3(gx, (unsigned)num_pieces), 256, 0, s>>>(
        slots, wires.in_ptr, wires.out_ptr, wires.in_loc, wires.out_loc, num_nodes_total);
    CKT_CHECK_LAUNCH();
  }
  // Each slot's first_bad straight into the caller's int64 array; all ones
  // reads as -1.
  CKT_CUDA(cudaMemcpy2DAsync(first_bad, sizeof(int64_t), &slots[0].first_bad, sizeof(NoAllocSlot),
                             sizeof(unsigned long long), (size_t)num_pieces,
                             cudaMemcpyDeviceToHost, s));
  CKT_CUDA(cudaStreamSynchronize(s));
  for (int32_t k = 0; k < num_pieces; k++)
    if (first_bad[k] >= 0)
      return set_error(CKT_EBOUNDS, "piece %d: wire %lld fails the pointer/location checks", k,
                       (long long)first_bad[k]);
  return CKT_OK;
}
