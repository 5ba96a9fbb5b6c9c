// ckt_batch.cu -- batched form: many independent circuits of uneven sizes,
// one outer loop of all of them in one persistent launch captured in a CUDA
// graph, with the launch shape and reduction schedule picked by an autotuner.
//
// Layout: the circuits are concatenated into one "union" circuit -- wires
// back to back, node ranges padded to multiples of 4 (so float4 node loads
// stay aligned), node pointers rebased -- with one contribution CSR.  No
// wire crosses circuits, so every per-circuit computation is unchanged and
// a circuit's results are bit-identical alone or in any batch.
#include <algorithm>
#include <cstring>
#include <map>
#include <mutex>
#include <numeric>
#include <thread>

#include "ckt_batch_inst.cuh"
#include "ckt_gen.h"
#include "ckt_internal.h"

using namespace ckt;

struct ckt_batch {
  int32_t C = 0;
  std::vector<ckt_gen_params> shapes;
  std::vector<int32_t> steps;
  std::vector<int64_t> wire_base, node_base;  // [C + 1]
  int64_t W = 0, N = 0;
  double updates = 0;
  // device arrays (union numbering)
  uint32_t *in_ptr = nullptr, *out_ptr = nullptr;
  uint8_t *in_loc = nullptr, *out_loc = nullptr;
  float *L = nullptr, *R = nullptr, *Cw = nullptr;
  float *cur = nullptr, *vol = nullptr, *charge = nullptr, *nvolt = nullptr;
  float *cap = nullptr, *leak = nullptr;
  int32_t *locator = nullptr;
  uint32_t *off = nullptr, *ent = nullptr;
  float *snap = nullptr;  // initial cur, vol, charge, nvolt
  // work tables for the current launch shape
  ckt_batch_config cfg = {256, 1, 0, 0};
  bool tables_valid = false;
  BatchItem *items = nullptr;
  uint32_t num_items = 0;
  BatchCircuit *circ = nullptr;
  std::vector<BatchCircuit> h_circ;
  uint32_t *sync_mem = nullptr;  // ticket, error, done_cnc[C], done_dc[C]
  int grid = 0;
  // CUDA graphs, one per mode
  cudaStream_t cap_stream = nullptr;
  cudaGraphExec_t gexec[2] = {nullptr, nullptr};
  uint64_t timeout_ns = 2000000000ull;
  int64_t device_bytes = 0;
  int sm_count = 0;
  std::vector<void *> allocs;
};

namespace {

int dalloc(ckt_batch *b, void **p, size_t bytes) {
  bytes = std::max<size_t>(bytes, 16);
  CKT_CUDA(cudaMalloc(p, bytes));
  b->allocs.push_back(*p);
  b->device_bytes += (int64_t)bytes;
  return CKT_OK;
}

template <typename T>
int dalloc_t(ckt_batch *b, T **p, size_t count) {
  return dalloc(b, reinterpret_cast<void **>(p), count * sizeof(T));
}

void free_batch(ckt_batch *b) {
  if (!b) return;
  for (int m = 0; m < 2; m++)
    if (b->gexec[m]) cudaGraphExecDestroy(b->gexec[m]);
  if (b->cap_stream) cudaStreamDestroy(b->cap_stream);
  for (void *p : b->allocs) cudaFree(p);
  delete b;
}

BatchKernelFn kernel_for(int mode, const ckt_batch_config &c) {
  return mode == CKT_MODE_EXACT ? batch_kernel_exact(c.block, c.wires_per_thread, c.dc_schedule)
                                : batch_kernel_fast(c.block, c.wires_per_thread, c.dc_schedule);
}

int check_config(const ckt_batch_config *c) {
  CKT_REQUIRE(c != nullptr, "config is NULL");
  CKT_REQUIRE(c->block == 128 || c->block == 256, "block must be 128 or 256 (got %d)", c->block);
  CKT_REQUIRE(c->wires_per_thread == 1 || c->wires_per_thread == 2,
              "wires_per_thread must be 1 or 2 (got %d)", c->wires_per_thread);
  CKT_REQUIRE(c->dc_schedule == 0 || c->dc_schedule == 1, "dc_schedule must be 0 or 1");
  return CKT_OK;
}

void invalidate_graphs(ckt_batch *b) {
  for (int m = 0; m < 2; m++)
    if (b->gexec[m]) {
      cudaGraphExecDestroy(b->gexec[m]);
      b->gexec[m] = nullptr;
    }
}

// Work table in ticket order: CNC tiles longest first (cost = steps x wires),
// then DC tiles and UV tiles circuit by circuit in the order in which the
// circuits' last CNC tiles were handed out.
int build_tables(ckt_batch *b) {
  const ckt_batch_config &c = b->cfg;
  struct Cnc {
    uint64_t cost;
    uint32_t circuit, begin, count;
  };
  std::vector<Cnc> cnc;
  std::vector<BatchCircuit> circ(b->C);
  const uint32_t tile = (uint32_t)(c.block * c.wires_per_thread);
  for (int32_t k = 0; k < b->C; k++) {
    const int64_t w0 = b->wire_base[k], W = b->wire_base[k + 1] - w0;
    circ[k].steps = b->steps[k];
    for (int64_t t = 0; t < W; t += tile) {
      const uint32_t n = (uint32_t)std::min<int64_t>(tile, W - t);
      cnc.push_back({(uint64_t)std::max(b->steps[k], 1) * n, (uint32_t)k, (uint32_t)(w0 + t), n});
      circ[k].cnc_items++;
    }
  }
  std::stable_sort(cnc.begin(), cnc.end(), [](const Cnc &x, const Cnc &y) { return x.cost > y.cost; });
  std::vector<int64_t> last(b->C, -1);
  std::vector<BatchItem> items;
  items.reserve(cnc.size() * 2);
  for (size_t i = 0; i < cnc.size(); i++) {
    items.push_back({(kItemCnc << 30) | cnc[i].circuit, cnc[i].begin, cnc[i].count, 0});
    last[cnc[i].circuit] = (int64_t)i;
  }
  std::vector<int32_t> order(b->C);
  std::iota(order.begin(), order.end(), 0);
  std::stable_sort(order.begin(), order.end(), [&](int32_t x, int32_t y) { return last[x] < last[y]; });
  for (int kind = 1; kind <= 2; kind++) {
    const uint32_t t = kind == 1 ? (uint32_t)c.block : 4u * (uint32_t)c.block;
    for (int32_t k : order) {
      const int64_t x0 = b->node_base[k];
      const int64_t n = (int64_t)b->shapes[k].num_pieces * b->shapes[k].nodes_per_piece;
      for (int64_t x = 0; x < n; x += t) {
        items.push_back({((uint32_t)kind << 30) | (uint32_t)k, (uint32_t)(x0 + x),
                         (uint32_t)std::min<int64_t>(t, n - x), 0});
        if (kind == 1) circ[k].dc_items++;
      }
    }
  }
  b->h_circ = circ;
  b->num_items = (uint32_t)items.size();
  if (b->items) {
    cudaFree(b->items);
    b->allocs.erase(std::find(b->allocs.begin(), b->allocs.end(), (void *)b->items));
    b->items = nullptr;
  }
  int rc;
  if ((rc = dalloc_t(b, &b->items, items.size()))) return rc;
  CKT_CUDA(cudaMemcpy(b->items, items.data(), items.size() * sizeof(BatchItem),
                      cudaMemcpyHostToDevice));
  CKT_CUDA(cudaMemcpy(b->circ, circ.data(), circ.size() * sizeof(BatchCircuit),
                      cudaMemcpyHostToDevice));
  int per_sm = 0;
  CKT_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(
      &per_sm, reinterpret_cast<const void *>(kernel_for(CKT_MODE_FAST, c)), c.block, 0));
  int per_sm_exact = 0;
  CKT_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(
      &per_sm_exact, reinterpret_cast<const void *>(kernel_for(CKT_MODE_EXACT, c)), c.block, 0));
  per_sm = std::max(1, std::min(per_sm, per_sm_exact));
  b->cfg.blocks_per_sm = per_sm;
  b->grid = b->sm_count * per_sm;
  b->tables_valid = true;
  invalidate_graphs(b);
  return CKT_OK;
}

int launch(ckt_batch *b, int mode, cudaStream_t s) {
  if (!b->tables_valid) {
    int rc = build_tables(b);
    if (rc) return rc;
  }
  CKT_CUDA(cudaMemsetAsync(b->sync_mem, 0, (2 + 2 * (size_t)b->C) * sizeof(uint32_t), s));
  BatchSync sync = {b->sync_mem, b->sync_mem + 1, b->sync_mem + 2, b->sync_mem + 2 + b->C};
  WireArrays wa = {b->in_ptr, b->out_ptr, b->in_loc, b->out_loc, b->L, b->R, b->Cw,
                   b->cur,    b->vol,     b->W};
  BatchNodes nd = {b->charge, b->nvolt, b->cap, b->leak};
  const BatchItem *items = b->items;
  uint32_t n = b->num_items;
  const BatchCircuit *circ = b->circ;
  const uint32_t *off = b->off, *ent = b->ent;
  float dt = (float)1e-6;
  uint64_t to = b->timeout_ns;
  void *args[] = {&items, &n, &circ, &sync, &wa, &nd, &off, &ent, &dt, &to};
  BatchKernelFn fn = kernel_for(mode, b->cfg);
  CKT_REQUIRE(fn != nullptr, "no kernel for this configuration");
  CKT_CUDA(cudaLaunchKernel(reinterpret_cast<const void *>(fn), dim3(b->grid), dim3(b->cfg.block),
                            args, 0, s));
  return CKT_OK;
}

int ensure_graph(ckt_batch *b, int mode) {
  if (b->gexec[mode]) return CKT_OK;
  if (!b->tables_valid) {
    int rc = build_tables(b);
    if (rc) return rc;
  }
  if (!b->cap_stream) CKT_CUDA(cudaStreamCreateWithFlags(&b->cap_stream, cudaStreamNonBlocking));
  cudaGraph_t g = nullptr;
  CKT_CUDA(cudaStreamBeginCapture(b->cap_stream, cudaStreamCaptureModeThreadLocal));
  int rc = launch(b, mode, b->cap_stream);
  cudaError_t e = cudaStreamEndCapture(b->cap_stream, &g);
  if (rc) {
    if (g) cudaGraphDestroy(g);
    return rc;
  }
  if (e != cudaSuccess) return set_error(CKT_ECUDA, "graph capture failed: %s", cudaGetErrorString(e));
  e = cudaGraphInstantiate(&b->gexec[mode], g, 0);
  cudaGraphDestroy(g);
  if (e != cudaSuccess) return set_error(CKT_ECUDA, "graph instantiate failed: %s", cudaGetErrorString(e));
  return CKT_OK;
}

// Host union arrays for the wires' static fields and the nodes.
struct HostUnion {
  std::vector<uint32_t> in_ptr, out_ptr;
  std::vector<uint8_t> in_loc, out_loc;
  std::vector<float> L, R, C, charge, nvolt, cap, leak;
  std::vector<int32_t> locator;
  void resize(int64_t W, int64_t N) {
    in_ptr.assign(W, 0); out_ptr.assign(W, 0); in_loc.assign(W, 0); out_loc.assign(W, 0);
    L.assign(W, 0.f); R.assign(W, 1.f); C.assign(W, 1.f);
    charge.assign(N, 0.f); nvolt.assign(N, 0.f); cap.assign(N, 1.f); leak.assign(N, 0.f);
    locator.assign(N, 1);
  }
  ckt_host_circuit slice(int64_t w0, int64_t x0, float *cur_dummy) {
    ckt_host_circuit h;
    h.in_ptr = in_ptr.data() + w0; h.out_ptr = out_ptr.data() + w0;
    h.in_loc = in_loc.data() + w0; h.out_loc = out_loc.data() + w0;
    h.inductance = L.data() + w0; h.resistance = R.data() + w0; h.capacitance = C.data() + w0;
    h.current = cur_dummy; h.voltage = cur_dummy;
    h.charge = charge.data() + x0; h.node_voltage = nvolt.data() + x0;
    h.node_capacitance = cap.data() + x0; h.node_leakage = leak.data() + x0;
    h.locator = locator.data() + x0;
    return h;
  }
};

int layout(ckt_batch *b, int32_t num, const ckt_gen_params *shapes, const int32_t *steps) {
  CKT_REQUIRE(num >= 1 && shapes && steps, "need at least one circuit, shapes and steps");
  b->C = num;
  b->shapes.assign(shapes, shapes + num);
  b->steps.assign(steps, steps + num);
  b->wire_base.assign(num + 1, 0);
  b->node_base.assign(num + 1, 0);
  for (int32_t k = 0; k < num; k++) {
    const ckt_gen_params &p = shapes[k];
    CKT_REQUIRE(p.num_pieces >= 1 && p.nodes_per_piece >= 1 && p.wires_per_piece >= 0,
                "circuit %d has a bad shape", k);
    CKT_REQUIRE(steps[k] >= 0, "circuit %d has negative steps", k);
    const int64_t W = (int64_t)p.num_pieces * p.wires_per_piece;
    const int64_t N = (int64_t)p.num_pieces * p.nodes_per_piece;
    b->wire_base[k + 1] = b->wire_base[k] + W;
    b->node_base[k + 1] = b->node_base[k] + ((N + 3) & ~int64_t(3));
    b->updates += (double)W * CKT_SEGMENTS * steps[k];
  }
  b->W = b->wire_base[num];
  b->N = b->node_base[num];
  CKT_REQUIRE(b->W <= kMaxWires && b->N < 0x7fffffffLL, "batch too large (W=%lld N=%lld)",
              (long long)b->W, (long long)b->N);
  CKT_CUDA(cudaDeviceGetAttribute(&b->sm_count, cudaDevAttrMultiProcessorCount, 0));
  return CKT_OK;
}

// Builds the union CSR, allocates and uploads everything.  cur/vol may be
// null (zero state).
int finish(ckt_batch *b, HostUnion &h, const std::vector<float> *cur, const std::vector<float> *vol) {
  std::vector<ckt_piece> pieces;
  for (int32_t k = 0; k < b->C; k++) {
    const ckt_gen_params &p = b->shapes[k];
    for (int32_t n = 0; n < p.num_pieces; n++)
      pieces.push_back({(uint32_t)(b->wire_base[k] + (int64_t)n * p.wires_per_piece),
                        (uint32_t)p.wires_per_piece,
                        (uint32_t)(b->node_base[k] + (int64_t)n * p.nodes_per_piece),
                        (uint32_t)p.nodes_per_piece});
  }
  std::vector<uint32_t> off, ent;
  int rc = build_node_csr(pieces.data(), (int32_t)pieces.size(), (uint32_t)b->N, h.in_ptr.data(),
                          h.out_ptr.data(), h.in_loc.data(), h.out_loc.data(), off, ent, nullptr);
  if (rc) return rc;
  const int64_t W = b->W, N = b->N, C = b->C;
  if ((rc = dalloc_t(b, &b->in_ptr, W)) || (rc = dalloc_t(b, &b->out_ptr, W)) ||
      (rc = dalloc_t(b, &b->in_loc, W)) || (rc = dalloc_t(b, &b->out_loc, W)) ||
      (rc = dalloc_t(b, &b->L, W)) || (rc = dalloc_t(b, &b->R, W)) ||
      (rc = dalloc_t(b, &b->Cw, W)) || (rc = dalloc_t(b, &b->cur, 10 * W)) ||
      (rc = dalloc_t(b, &b->vol, 9 * W)) || (rc = dalloc_t(b, &b->charge, N)) ||
      (rc = dalloc_t(b, &b->nvolt, N)) || (rc = dalloc_t(b, &b->cap, N)) ||
      (rc = dalloc_t(b, &b->leak, N)) || (rc = dalloc_t(b, &b->locator, N)) ||
      (rc = dalloc_t(b, &b->off, N + 1)) || (rc = dalloc_t(b, &b->ent, 2 * W)) ||
      (rc = dalloc_t(b, &b->snap, 19 * W + 2 * N)) || (rc = dalloc_t(b, &b->circ, C)) ||
      (rc = dalloc_t(b, &b->sync_mem, 2 + 2 * C)))
    return rc == CKT_ECUDA ? CKT_ENOMEM : rc;
  auto up = [](void *d, const void *s, size_t bytes) {
    return bytes ? cudaMemcpy(d, s, bytes, cudaMemcpyHostToDevice) : cudaSuccess;
  };
  CKT_CUDA(up(b->in_ptr, h.in_ptr.data(), W * 4));
  CKT_CUDA(up(b->out_ptr, h.out_ptr.data(), W * 4));
  CKT_CUDA(up(b->in_loc, h.in_loc.data(), W));
  CKT_CUDA(up(b->out_loc, h.out_loc.data(), W));
  CKT_CUDA(up(b->L, h.L.data(), W * 4));
  CKT_CUDA(up(b->R, h.R.data(), W * 4));
  CKT_CUDA(up(b->Cw, h.C.data(), W * 4));
  CKT_CUDA(up(b->charge, h.charge.data(), N * 4));
  CKT_CUDA(up(b->nvolt, h.nvolt.data(), N * 4));
  CKT_CUDA(up(b->cap, h.cap.data(), N * 4));
  CKT_CUDA(up(b->leak, h.leak.data(), N * 4));
  CKT_CUDA(up(b->locator, h.locator.data(), N * 4));
  CKT_CUDA(up(b->off, off.data(), (N + 1) * 4));
  CKT_CUDA(up(b->ent, ent.data(), 2 * W * 4));
  if (cur) CKT_CUDA(up(b->cur, cur->data(), 10 * W * 4));
  else CKT_CUDA(cudaMemset(b->cur, 0, 10 * W * 4));
  if (vol) CKT_CUDA(up(b->vol, vol->data(), 9 * W * 4));
  else CKT_CUDA(cudaMemset(b->vol, 0, 9 * W * 4));
  CKT_CUDA(cudaMemcpy(b->snap, b->cur, 10 * W * 4, cudaMemcpyDeviceToDevice));
  CKT_CUDA(cudaMemcpy(b->snap + 10 * W, b->vol, 9 * W * 4, cudaMemcpyDeviceToDevice));
  CKT_CUDA(cudaMemcpy(b->snap + 19 * W, b->charge, N * 4, cudaMemcpyDeviceToDevice));
  CKT_CUDA(cudaMemcpy(b->snap + 19 * W + N, b->nvolt, N * 4, cudaMemcpyDeviceToDevice));
  return CKT_OK;
}

std::mutex g_tune_mu;
std::map<std::tuple<int, int, int, int>, ckt_batch_config> g_tune_cache;

}  // namespace

extern "C" {

int ckt_batch_create(int32_t num_circuits, const ckt_gen_params *shapes,
                     const ckt_host_circuit *circuits, const int32_t *steps, ckt_batch **out) {
  CKT_REQUIRE(out != nullptr && circuits != nullptr, "NULL argument");
  *out = nullptr;
  ckt_batch *b = new ckt_batch();
  int rc = layout(b, num_circuits, shapes, steps);
  if (rc) { free_batch(b); return rc; }
  HostUnion h;
  h.resize(b->W, b->N);
  std::vector<float> cur(10 * b->W), vol(9 * b->W);
  for (int32_t k = 0; k < num_circuits; k++) {
    const ckt_host_circuit &c = circuits[k];
    const int64_t w0 = b->wire_base[k], W = b->wire_base[k + 1] - w0, x0 = b->node_base[k];
    const int64_t N = (int64_t)shapes[k].num_pieces * shapes[k].nodes_per_piece;
    if (!(c.in_ptr && c.out_ptr && c.in_loc && c.out_loc && c.inductance && c.resistance &&
          c.capacitance && c.current && c.voltage && c.charge && c.node_voltage &&
          c.node_capacitance && c.node_leakage && c.locator)) {
      free_batch(b);
      return set_error(CKT_EINVAL, "circuit %d has NULL arrays", k);
    }
    for (int64_t w = 0; w < W; w++) {
      h.in_ptr[w0 + w] = c.in_ptr[w] + (uint32_t)x0;
      h.out_ptr[w0 + w] = c.out_ptr[w] + (uint32_t)x0;
    }
    memcpy(h.in_loc.data() + w0, c.in_loc, W);
    memcpy(h.out_loc.data() + w0, c.out_loc, W);
    memcpy(h.L.data() + w0, c.inductance, W * 4);
    memcpy(h.R.data() + w0, c.resistance, W * 4);
    memcpy(h.C.data() + w0, c.capacitance, W * 4);
    for (int s = 0; s < 10; s++) memcpy(cur.data() + s * b->W + w0, c.current + s * W, W * 4);
    for (int s = 0; s < 9; s++) memcpy(vol.data() + s * b->W + w0, c.voltage + s * W, W * 4);
    memcpy(h.charge.data() + x0, c.charge, N * 4);
    memcpy(h.nvolt.data() + x0, c.node_voltage, N * 4);
    memcpy(h.cap.data() + x0, c.node_capacitance, N * 4);
    memcpy(h.leak.data() + x0, c.node_leakage, N * 4);
    memcpy(h.locator.data() + x0, c.locator, N * 4);
  }
  if ((rc = finish(b, h, &cur, &vol))) { free_batch(b); return rc; }
  *out = b;
  return CKT_OK;
}

int ckt_batch_generate(int32_t num_circuits, const ckt_gen_params *shapes, const int32_t *steps,
                       int32_t host_threads, ckt_batch **out) {
  CKT_REQUIRE(out != nullptr, "out is NULL");
  *out = nullptr;
  ckt_batch *b = new ckt_batch();
  int rc = layout(b, num_circuits, shapes, steps);
  if (rc) { free_batch(b); return rc; }
  HostUnion h;
  h.resize(b->W, b->N);
  const int T = std::max(1, std::min<int>(host_threads > 0 ? host_threads : 1, num_circuits));
  std::vector<int> rcs(num_circuits, CKT_OK);
  std::vector<std::thread> pool;
  float dummy = 0.f;
  for (int t = 0; t < T; t++)
    pool.emplace_back([&, t]() {
      for (int32_t k = t; k < num_circuits; k += T) {
        ckt_host_circuit s = h.slice(b->wire_base[k], b->node_base[k], &dummy);
        rcs[k] = generate_into(&shapes[k], &s, (uint32_t)b->node_base[k]);
      }
    });
  for (auto &th : pool) th.join();
  for (int32_t k = 0; k < num_circuits; k++)
    if (rcs[k]) { free_batch(b); return set_error(rcs[k], "generating circuit %d failed", k); }
  if ((rc = finish(b, h, nullptr, nullptr))) { free_batch(b); return rc; }
  *out = b;
  return CKT_OK;
}

int ckt_batch_destroy(ckt_batch *b) {
  free_batch(b);
  return CKT_OK;
}

int ckt_batch_info(const ckt_batch *b, int64_t *num_wires, int64_t *num_nodes,
                   double *segment_updates_per_run, int64_t *device_bytes) {
  CKT_REQUIRE(b != nullptr, "batch is NULL");
  if (num_wires) *num_wires = b->W;
  if (num_nodes) *num_nodes = b->N;
  if (segment_updates_per_run) *segment_updates_per_run = b->updates;
  if (device_bytes) *device_bytes = b->device_bytes;
  return CKT_OK;
}

int ckt_batch_circuit_offsets(const ckt_batch *b, int32_t circuit, int64_t *first_wire,
                              int64_t *first_node) {
  CKT_REQUIRE(b != nullptr && circuit >= 0 && circuit < b->C, "bad batch or circuit index");
  if (first_wire) *first_wire = b->wire_base[circuit];
  if (first_node) *first_node = b->node_base[circuit];
  return CKT_OK;
}

int ckt_batch_set_config(ckt_batch *b, const ckt_batch_config *c) {
  CKT_REQUIRE(b != nullptr, "batch is NULL");
  int rc = check_config(c);
  if (rc) return rc;
  b->cfg = *c;
  b->cfg.blocks_per_sm = 0;
  return build_tables(b);
}

int ckt_batch_get_config(const ckt_batch *b, ckt_batch_config *c) {
  CKT_REQUIRE(b != nullptr && c != nullptr, "NULL argument");
  *c = b->cfg;
  return CKT_OK;
}

int ckt_batch_set_timeout(ckt_batch *b, uint64_t timeout_ns) {
  CKT_REQUIRE(b != nullptr && timeout_ns > 0, "bad arguments");
  b->timeout_ns = timeout_ns;
  invalidate_graphs(b);
  return CKT_OK;
}

int ckt_batch_reset_state(ckt_batch *b, void *stream) {
  CKT_REQUIRE(b != nullptr, "batch is NULL");
  const cudaStream_t s = as_stream(stream);
  const int64_t W = b->W, N = b->N;
  CKT_CUDA(cudaMemcpyAsync(b->cur, b->snap, 10 * W * 4, cudaMemcpyDeviceToDevice, s));
  CKT_CUDA(cudaMemcpyAsync(b->vol, b->snap + 10 * W, 9 * W * 4, cudaMemcpyDeviceToDevice, s));
  CKT_CUDA(cudaMemcpyAsync(b->charge, b->snap + 19 * W, N * 4, cudaMemcpyDeviceToDevice, s));
  CKT_CUDA(cudaMemcpyAsync(b->nvolt, b->snap + 19 * W + N, N * 4, cudaMemcpyDeviceToDevice, s));
  return CKT_OK;
}

int ckt_batch_run(ckt_batch *b, int32_t mode, void *stream) {
  CKT_REQUIRE(b != nullptr, "batch is NULL");
  CKT_REQUIRE(mode == CKT_MODE_EXACT || mode == CKT_MODE_FAST, "unknown mode %d", mode);
  int rc = ensure_graph(b, mode);
  if (rc) return rc;
  CKT_CUDA(cudaGraphLaunch(b->gexec[mode], as_stream(stream)));
  return CKT_OK;
}

int ckt_batch_run_direct(ckt_batch *b, int32_t mode, void *stream) {
  CKT_REQUIRE(b != nullptr, "batch is NULL");
  CKT_REQUIRE(mode == CKT_MODE_EXACT || mode == CKT_MODE_FAST, "unknown mode %d", mode);
  return launch(b, mode, as_stream(stream));
}

int ckt_batch_check(ckt_batch *b, void *stream) {
  CKT_REQUIRE(b != nullptr, "batch is NULL");
  const cudaStream_t s = as_stream(stream);
  uint32_t err = 0;
  CKT_CUDA(cudaMemcpyAsync(&err, b->sync_mem + 1, 4, cudaMemcpyDeviceToHost, s));
  CKT_CUDA(cudaStreamSynchronize(s));
  if (err) return set_error(CKT_ETIMEOUT, "a persistent-kernel wait timed out (error word %u)", err);
  return CKT_OK;
}

int ckt_batch_run_sequential(ckt_batch *b, int32_t mode, void *stream) {
  CKT_REQUIRE(b != nullptr, "batch is NULL");
  const cudaStream_t s = as_stream(stream);
  ckt_wires w = {b->in_ptr, b->out_ptr, b->in_loc, b->out_loc, b->L, b->R, b->Cw,
                 b->cur,    b->vol,     b->W};
  const float *I0 = b->cur, *I9 = b->cur + 9 * b->W;
  for (int32_t k = 0; k < b->C; k++) {
    const ckt_gen_params &p = b->shapes[k];
    const int64_t w0 = b->wire_base[k], W = b->wire_base[k + 1] - w0, x0 = b->node_base[k];
    const int64_t N = (int64_t)p.num_pieces * p.nodes_per_piece;
    ckt_params prm = {b->steps[k], (float)1e-6, mode, CKT_INIT_KERNEL};
    int rc = launch_cnc((uint32_t)w0, (uint32_t)W, w, b->nvolt, b->nvolt, b->nvolt, &prm, s);
    if (rc) return rc;
    dc_all_kernel<<<grid_for(N, kDcBlock), kDcBlock, 0, s>>>((uint32_t)x0, (uint32_t)(x0 + N),
                                                           b->off, b->ent, I0, I9, b->charge,
                                                           prm.dt);
    CKT_CHECK_LAUNCH();
    const int64_t n4 = N / 4;
    if (n4)
      uv_all_vec4_kernel<<<grid_for(n4), 256, 0, s>>>(
          (uint32_t)n4, reinterpret_cast<float4 *>(b->charge + x0),
          reinterpret_cast<float4 *>(b->nvolt + x0), reinterpret_cast<const float4 *>(b->cap + x0),
          reinterpret_cast<const float4 *>(b->leak + x0));
    if (N > 4 * n4)
      uv_all_scalar_kernel<<<1, 256, 0, s>>>((uint32_t)(x0 + 4 * n4), (uint32_t)(N - 4 * n4),
                                             b->charge, b->nvolt, b->cap, b->leak);
    CKT_CHECK_LAUNCH();
  }
  return CKT_OK;
}

int ckt_batch_autotune(ckt_batch *b, int32_t mode, void *stream, ckt_batch_config *chosen) {
  CKT_REQUIRE(b != nullptr, "batch is NULL");
  CKT_REQUIRE(mode == CKT_MODE_EXACT || mode == CKT_MODE_FAST, "unknown mode %d", mode);
  const cudaStream_t s = as_stream(stream);
  int maxs = 0;
  for (int32_t x : b->steps) maxs = std::max(maxs, x);
  int lw = 0;
  while (((int64_t)1 << lw) < std::max<int64_t>(b->W, 1)) lw++;
  int lc = 0;
  while ((1 << lc) < b->C) lc++;
  const auto key = std::make_tuple(mode, lw, lc, maxs / 128);
  {
    std::lock_guard<std::mutex> g(g_tune_mu);
    auto it = g_tune_cache.find(key);
    if (it != g_tune_cache.end()) {
      int rc = ckt_batch_set_config(b, &it->second);
      if (rc == CKT_OK && chosen) *chosen = b->cfg;
      return rc;
    }
  }
  cudaEvent_t e0, e1;
  CKT_CUDA(cudaEventCreate(&e0));
  CKT_CUDA(cudaEventCreate(&e1));
  float best = 1e30f;
  ckt_batch_config best_cfg = b->cfg;
  int rc = CKT_OK;
  for (int block : {128, 256})
    for (int wpt : {1, 2})
      for (int dcs : {0, 1}) {
        ckt_batch_config c = {block, wpt, dcs, 0};
        if ((rc = ckt_batch_set_config(b, &c))) goto done;
        if ((rc = ckt_batch_reset_state(b, stream)) || (rc = launch(b, mode, s))) goto done;
        if ((rc = ckt_batch_check(b, stream))) goto done;
        if ((rc = ckt_batch_reset_state(b, stream))) goto done;
        cudaEventRecord(e0, s);
        if ((rc = launch(b, mode, s))) goto done;
        cudaEventRecord(e1, s);
        if ((rc = ckt_batch_check(b, stream))) goto done;
        float ms = 0.f;
        cudaEventElapsedTime(&ms, e0, e1);
        if (ms < best) {
          best = ms;
          best_cfg = b->cfg;
        }
      }
  rc = ckt_batch_set_config(b, &best_cfg);
  if (rc == CKT_OK) rc = ckt_batch_reset_state(b, stream);
  if (rc == CKT_OK) {
    std::lock_guard<std::mutex> g(g_tune_mu);
    g_tune_cache[key] = b->cfg;
  }
done:
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (rc == CKT_OK && chosen) *chosen = b->cfg;
  return rc;
}

int ckt_batch_read_state(ckt_batch *b, int32_t circuit, float *current, float *voltage,
                         float *charge, float *node_voltage, void *stream) {
  CKT_REQUIRE(b != nullptr && circuit >= 0 && circuit < b->C, "bad batch or circuit index");
  const cudaStream_t s = as_stream(stream);
  const int64_t w0 = b->wire_base[circuit], W = b->wire_base[circuit + 1] - w0;
  const int64_t x0 = b->node_base[circuit];
  const int64_t N = (int64_t)b->shapes[circuit].num_pieces * b->shapes[circuit].nodes_per_piece;
  if (current && W > 0)
    CKT_CUDA(cudaMemcpy2DAsync(current, W * 4, b->cur + w0, b->W * 4, W * 4, 10,
                               cudaMemcpyDeviceToHost, s));
  if (voltage && W > 0)
    CKT_CUDA(cudaMemcpy2DAsync(voltage, W * 4, b->vol + w0, b->W * 4, W * 4, 9,
                               cudaMemcpyDeviceToHost, s));
  if (charge) CKT_CUDA(cudaMemcpyAsync(charge, b->charge + x0, N * 4, cudaMemcpyDeviceToHost, s));
  if (node_voltage)
    CKT_CUDA(cudaMemcpyAsync(node_voltage, b->nvolt + x0, N * 4, cudaMemcpyDeviceToHost, s));
  CKT_CUDA(cudaStreamSynchronize(s));
  return CKT_OK;
}

int ckt_batch_upload_state(ckt_batch *b, const float *current, const float *voltage,
                           const float *charge, const float *node_voltage, void *stream) {
  CKT_REQUIRE(b != nullptr && current && voltage && charge && node_voltage, "NULL argument");
  const cudaStream_t s = as_stream(stream);
  CKT_CUDA(cudaMemcpyAsync(b->cur, current, 10 * b->W * 4, cudaMemcpyHostToDevice, s));
  CKT_CUDA(cudaMemcpyAsync(b->vol, voltage, 9 * b->W * 4, cudaMemcpyHostToDevice, s));
  CKT_CUDA(cudaMemcpyAsync(b->charge, charge, b->N * 4, cudaMemcpyHostToDevice, s));
  CKT_CUDA(cudaMemcpyAsync(b->nvolt, node_voltage, b->N * 4, cudaMemcpyHostToDevice, s));
  return CKT_OK;
}

int ckt_batch_download_state(ckt_batch *b, float *current, float *voltage, float *charge,
                             float *node_voltage, void *stream) {
  CKT_REQUIRE(b != nullptr && current && voltage && charge && node_voltage, "NULL argument");
  const cudaStream_t s = as_stream(stream);
  CKT_CUDA(cudaMemcpyAsync(current, b->cur, 10 * b->W * 4, cudaMemcpyDeviceToHost, s));
  CKT_CUDA(cudaMemcpyAsync(voltage, b->vol, 9 * b->W * 4, cudaMemcpyDeviceToHost, s));
  CKT_CUDA(cudaMemcpyAsync(charge, b->charge, b->N * 4, cudaMemcpyDeviceToHost, s));
  CKT_CUDA(cudaMemcpyAsync(node_voltage, b->nvolt, b->N * 4, cudaMemcpyDeviceToHost, s));
  return CKT_OK;
}

int ckt_batch_inject_stall(ckt_batch *b, int32_t circuit, int32_t enable) {
  CKT_REQUIRE(b != nullptr && circuit >= 0 && circuit < b->C, "bad batch or circuit index");
  if (!b->tables_valid) {
    int rc = build_tables(b);
    if (rc) return rc;
  }
  BatchCircuit c = b->h_circ[circuit];
  if (enable) c.cnc_items += 1;  // a CNC tile that no item will ever complete
  CKT_CUDA(cudaMemcpy(b->circ + circuit, &c, sizeof(c), cudaMemcpyHostToDevice));
  return CKT_OK;
}

}  // extern "C"
