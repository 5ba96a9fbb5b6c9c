// ckt_round.cu -- per-circuit graphs, round work tables and round launches.
#include <algorithm>
#include <numeric>

#include "ckt_batch_inst.cuh"
#include "ckt_round.h"

namespace ckt {

int build_circuit_graph(const ckt_gen_params &p, const uint32_t *in_ptr, const uint32_t *out_ptr,
                        const uint8_t *in_loc, const uint8_t *out_loc, HostGraph &g) {
  std::vector<ckt_piece> pieces(p.num_pieces);
  for (int32_t k = 0; k < p.num_pieces; k++)
    pieces[k] = {(uint32_t)((int64_t)k * p.wires_per_piece), (uint32_t)p.wires_per_piece,
                 (uint32_t)((int64_t)k * p.nodes_per_piece), (uint32_t)p.nodes_per_piece};
  const int64_t N = (int64_t)p.num_pieces * p.nodes_per_piece;
  std::vector<uint32_t> slots;
  int64_t W = 0;
  int rc = build_node_csr(pieces.data(), p.num_pieces, (uint32_t)N, in_ptr, out_ptr, in_loc,
                          out_loc, g.off, g.ent, &W, &slots);
  if (rc) return rc;
  g.slot_in.resize(W);
  g.slot_out.resize(W);
  for (int64_t w = 0; w < W; w++) {
    g.slot_in[w] = slots[2 * w];
    g.slot_out[w] = slots[2 * w + 1];
  }
  g.gstart.assign(gstart_words(W), 0u);
  for (int64_t i = 0; i < 2 * W; i++)
    if (g.ent[i] & 1u) g.gstart[i >> 5] |= 1u << (i & 31);
  return CKT_OK;
}

void build_round_table(std::vector<RoundCircuit> &circuits, const ckt_batch_config &cfg,
                       std::vector<BatchItem> &items) {
  struct Cnc {
    uint64_t cost;
    uint32_t circuit, begin, count;
  };
  const uint32_t C = (uint32_t)circuits.size();
  std::vector<Cnc> cnc;
  const uint32_t tile = (uint32_t)(cfg.block * cfg.wires_per_thread);
  for (uint32_t k = 0; k < C; k++) {
    RoundCircuit &rc = circuits[k];
    rc.cnc_items = rc.dc_items = 0;
    for (uint32_t t = 0; t < rc.W; t += tile) {
      const uint32_t n = std::min(tile, rc.W - t);
      cnc.push_back({(uint64_t)std::max(rc.steps, 1) * n, k, t, n});
      rc.cnc_items++;
    }
  }
  std::stable_sort(cnc.begin(), cnc.end(), [](const Cnc &x, const Cnc &y) { return x.cost > y.cost; });
  std::vector<int64_t> last(C, -1);
  items.clear();
  items.reserve(cnc.size() * 2 + 2 * C);
  for (size_t i = 0; i < cnc.size(); i++) {
    items.push_back({(kItemCnc << 30) | cnc[i].circuit, cnc[i].begin, cnc[i].count, 0});
    last[cnc[i].circuit] = (int64_t)i;
  }
  std::vector<uint32_t> order(C);
  std::iota(order.begin(), order.end(), 0u);
  std::stable_sort(order.begin(), order.end(), [&](uint32_t x, uint32_t y) { return last[x] < last[y]; });
  for (uint32_t kind = 1; kind <= 2; kind++) {
    const uint32_t t = kind == 1 ? (uint32_t)cfg.block : 4u * (uint32_t)cfg.block;
    for (uint32_t k : order) {
      RoundCircuit &rc = circuits[k];
      for (uint32_t x = 0; x < rc.N; x += t) {
        items.push_back({(kind << 30) | k, x, std::min(t, rc.N - x), 0});
        if (kind == 1) rc.dc_items++;
      }
    }
  }
}

BatchKernelFn round_kernel_for(int mode, const ckt_batch_config &c) {
  return mode == CKT_MODE_EXACT ? batch_kernel_exact(c.block, c.wires_per_thread, c.dc_schedule)
                                : batch_kernel_fast(c.block, c.wires_per_thread, c.dc_schedule);
}

int round_blocks_per_sm(const ckt_batch_config &c, int *out) {
  int a = 0, b = 0;
  CKT_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(
      &a, reinterpret_cast<const void *>(round_kernel_for(CKT_MODE_FAST, c)), c.block, 0));
  CKT_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(
      &b, reinterpret_cast<const void *>(round_kernel_for(CKT_MODE_EXACT, c)), c.block, 0));
  *out = std::max(1, std::min(a, b));
  return CKT_OK;
}

int launch_round(int mode, const ckt_batch_config &cfg, int grid, const BatchItem *items,
                 uint32_t num_items, const RoundCircuit *circ, uint32_t C, uint32_t *sync_mem,
                 uint64_t timeout_ns, cudaStream_t s) {
  CKT_CUDA(cudaMemsetAsync(sync_mem, 0, (2 + 2 * (size_t)C) * sizeof(uint32_t), s));
  BatchSync sync = {sync_mem, sync_mem + 1, sync_mem + 2, sync_mem + 2 + C};
  float dt = (float)1e-6;
  void *args[] = {&items, &num_items, &circ, &sync, &dt, &timeout_ns};
  BatchKernelFn fn = round_kernel_for(mode, cfg);
  CKT_REQUIRE(fn != nullptr, "no round kernel for this configuration");
  CKT_CUDA(cudaLaunchKernel(reinterpret_cast<const void *>(fn), dim3(grid), dim3(cfg.block), args,
                            0, s));
  return CKT_OK;
}

int check_batch_config(const ckt_batch_config *c) {
  CKT_REQUIRE(c != nullptr, "config is NULL");
  CKT_REQUIRE(c->block == 128 || c->block == 256, "block must be 128 or 256 (got %d)", c->block);
  CKT_REQUIRE(c->wires_per_thread == 1 || c->wires_per_thread == 2,
              "wires_per_thread must be 1 or 2 (got %d)", c->wires_per_thread);
  CKT_REQUIRE(c->dc_schedule >= 0 && c->dc_schedule <= 2, "dc_schedule must be 0, 1 or 2");
  return CKT_OK;
}

}  // namespace ckt
