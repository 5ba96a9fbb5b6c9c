// ckt_internal.h -- shared helpers of the circuit library (not part of the ABI).
#pragma once

#include <cuda_runtime.h>
#include <nvtx3/nvToolsExt.h>

#include <cstdarg>
#include <cstdint>
#include <cstdio>
#include <mutex>
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

// Tiled distribute_charge (dc_tile_kernel).  Nodes are cut into tiles of at
// most kTileNodesMax consecutive nodes, wires into chunks of kChunkWires.  A
// tile's contributions are cut into steps, each covering an ascending range
// of wires: a stream step holds entries of one chunk, whose I[0]/I[9] slices
// the block copies into shared memory whole (a chunk with more entries than
// a step holds takes consecutive steps); a ghost step merges chunks with few
// of the tile's contributions, whose currents a packing kernel
// (ghost_pack_kernel) has first copied, in wire order, into the step's
// region of the graph's ghost buffer: the in-ends' I[0] values, padded to a
// multiple of 4, then the out-ends' I[9] values, padded likewise.  The block
// copies the two runs to the same places a stream step's slices go, so an
// entry's value sits at end * kChunkWires + index in either kind of step.
// Steps run in wire order and, inside a step, a node's contributions in
// wire order, so every node still adds its contributions in the CSR's order.
// Inside a step, entries are grouped by the consumer warp that owns their
// node (node within tile mod kTileWarps) and, inside a warp, dealt to its 32
// lanes as whole runs, longest first to the least-loaded lane.  A step's
// block is a header of kStepHeaderWords words -- 16-bit offsets: lane list
// l = 32 w + L starts at header[l] (l < kTileLanes), header[kTileLanes] =
// entries -- followed by the entries, padded to a multiple of 4.
//   step record: {first block word, block words, chunk or ghost descriptor,
//                 first ghost slot}
//   ghost descriptor: kGhostStep | in-end count << kGhostCountBits | out-end count
//   entry word: index (kChunkBits: wire within chunk, or position within
//               the step's in- or out-end run) | end | node within tile
//               (13 bits) | flush | head | private, from the low bit up
// flush: the entry starts a new piece group and is not the node's first;
// head: first entry of its node within the step.  Padding words are kTePad.
//   ghost list entry (ghost_pack_kernel): {slot, wire << 1 | end}, sorted by
//   (wire / kPackWires, slot); ghost_block[b] = first entry of source block
//   b (wires [b kPackWires, (b + 1) kPackWires)) | kPackHasIn | kPackHasOut.
constexpr uint32_t kTileNodesMax = 8192;
constexpr uint32_t kChunkBits = 12;
constexpr uint32_t kChunkWires = 1u << kChunkBits;
constexpr uint32_t kGhostStep = 0x80000000u, kGhostCountBits = 13,
                   kGhostCountMask = (1u << kGhostCountBits) - 1u;
constexpr uint32_t kPackWires = 4096, kPackHasIn = 1u << 30, kPackHasOut = 1u << 31,
                   kPackFirstMask = kPackHasIn - 1u;
constexpr uint32_t kTeEnd = 1u << kChunkBits, kTeNodeShift = kChunkBits + 1,
                   kTeFlush = 1u << (kTeNodeShift + 13), kTeHead = kTeFlush << 1,
                   kTePriv = kTeHead << 1, kTePad = 0xffffffffu;
constexpr uint32_t kStepEntriesMax = kChunkWires;  // padded entries of one step
static_assert(kTePriv < (1u << 31), "entry word fields overflow");
static_assert(kStepEntriesMax <= kGhostCountMask, "ghost counts overflow");
constexpr uint32_t kTileWarps = 31;                // consumer warps of a block
constexpr uint32_t kTileLanes = 32 * kTileWarps;   // consumer lanes
constexpr uint32_t kStepHeaderWords = ((kTileLanes + 1 + 1) / 2 + 3) / 4 * 4;

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
  // Each wire end's CSR position and a bit per CSR entry marking the start
  // of a piece group (the graph's exported form, ckt_graph_export).
  uint32_t *slot_in = nullptr, *slot_out = nullptr;  // [W]
  uint32_t *gstart = nullptr;                        // [ceil(2W / 32)]
  // Tiled distribute_charge plan (see kTileNodesMax): tile t runs steps
  // [tile_step[t], tile_step[t + 1]).
  uint32_t tile_nodes = 0, num_tiles = 0;
  int64_t tile_num_steps = 0, tile_stream_steps = 0;
  uint32_t *tile_step = nullptr;   // [num_tiles + 1]
  uint4 *tile_steps = nullptr;     // [steps]
  uint32_t *tile_ent = nullptr;    // entry words, every step's run 16-byte aligned
  // Ghost steps' currents: ghost_slots floats, filled before each pass by
  // ghost_pack_kernel from the ghost_n entries of ghost_list.
  // ghost_staged: the packing stages whole current slices (many ghost ends
  // per source block) rather than reading each current directly.
  float *ghost = nullptr;
  uint2 *ghost_list = nullptr;
  uint32_t *ghost_block = nullptr;  // [ghost_blocks + 1]
  int64_t ghost_slots = 0, ghost_n = 0;
  uint32_t ghost_blocks = 0;
  bool ghost_staged = false;
  // Passes on one graph share its ghost buffer: a pass launched on another
  // stream than the previous one first waits for the previous one's end
  // (ghost_done, recorded after every pass), in the order the calls are
  // made.
  mutable std::mutex ghost_mu;
  mutable cudaEvent_t ghost_done = nullptr;
  mutable cudaStream_t ghost_stream = nullptr;
  mutable bool ghost_used = false;
  uint32_t *tile_mask = nullptr;   // [num_tiles * kTileNodesMax / 32] bit: the node's
                                   // folds are added at the end (shared/ghost, touched)
  // [1] bit 0: a copy wait timed out.  Pinned host memory mapped for the
  // device: the kernel stores into tile_error, the host reads
  // tile_error_host without a copy, so every later call on the graph sees a
  // pass that has finished with its tile unwritten.
  uint32_t *tile_error = nullptr;
  volatile uint32_t *tile_error_host = nullptr;
  // Bound of the tiled pass's copy waits; a wait that runs out sets the
  // error word instead of hanging the block.
  uint64_t tile_timeout_ns = 2000000000ull;
  int64_t device_bytes = 0;
};
