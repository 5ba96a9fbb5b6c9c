// ckt_round.h -- pieces shared by the batched form and the serving loop:
// per-circuit contribution graphs, round work tables and the round launch.
#pragma once

#include <vector>

#include "ckt_batch_inst.cuh"
#include "ckt_internal.h"

namespace ckt {

// Host-side contribution graph of one circuit (circuit-local numbering):
// node CSR with the private bit, each wire end's CSR slot, and a bit per CSR
// entry marking the start of a piece group.
struct HostGraph {
  std::vector<uint32_t> off, ent, slot_in, slot_out, gstart;
};

// Builds the graph of a circuit generated with shape `p` (pieces of
// wires_per_piece wires and nodes_per_piece nodes, numbered piece-major).
int build_circuit_graph(const ckt_gen_params &p, const uint32_t *in_ptr, const uint32_t *out_ptr,
                        const uint8_t *in_loc, const uint8_t *out_loc, HostGraph &g);

inline size_t gstart_words(int64_t W) { return (size_t)((2 * W + 31) / 32); }

// Work table of one round over circuits[0..C): CNC tiles longest first
// (cost = steps x wires), then DC and UV tiles circuit by circuit in the
// order in which the circuits' last CNC tiles are handed out.  Fills each
// circuit's cnc_items / dc_items.
void build_round_table(std::vector<RoundCircuit> &circuits, const ckt_batch_config &cfg,
                       std::vector<BatchItem> &items);

// The kernel for (mode, launch shape), or null.
BatchKernelFn round_kernel_for(int mode, const ckt_batch_config &cfg);

// Resident blocks per SM of the round kernel for this shape (both modes).
int round_blocks_per_sm(const ckt_batch_config &cfg, int *out);

// One round: clears the sync words (ticket, error, done counters of C
// circuits) and launches the persistent kernel on `s`.
int launch_round(int mode, const ckt_batch_config &cfg, int grid, const BatchItem *items,
                 uint32_t num_items, const RoundCircuit *circ, uint32_t C, uint32_t *sync_mem,
                 uint64_t timeout_ns, cudaStream_t s);

int check_batch_config(const ckt_batch_config *c);

}  // namespace ckt
