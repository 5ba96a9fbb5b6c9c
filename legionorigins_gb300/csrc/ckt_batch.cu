// ckt_batch.cu -- batched form: many independent circuits of uneven sizes,
// one outer loop of all of them in one persistent launch replayed from a
// CUDA graph, with the launch shape and reduction schedule picked by an
// autotuner.
//
// Layout: each circuit keeps its own numbering; its arrays are blocks of
// batch-wide, field-major arrays (all circuits' currents in one array, all
// in-pointers in another, ...), so the state of the whole batch moves with
// one copy per field.  Node blocks start at multiples of 4 nodes so float4
// node loads stay aligned.  No wire crosses circuits: a circuit's results are
// bit-identical alone or in any batch.
#include <algorithm>
#include <cstring>
#include <functional>
#include <map>
#include <mutex>
#include <thread>
#include <tuple>

#include "ckt_gen.h"
#include "ckt_round.h"

using namespace ckt;

struct ckt_batch {
  int32_t C = 0;
  std::vector<ckt_gen_params> shapes;
  std::vector<int32_t> steps;
  // per-circuit offsets into the field arrays, [C + 1]
  std::vector<int64_t> wbase, nbase, obase, gbase;
  int64_t W = 0, N = 0, O = 0, G = 0;
  double updates = 0;
  // device field arrays
  uint32_t *in_ptr = nullptr, *out_ptr = nullptr, *slot_in = nullptr, *slot_out = nullptr;
  uint8_t *in_loc = nullptr, *out_loc = nullptr;
  float *L = nullptr, *R = nullptr, *Cw = nullptr;
  float *cur = nullptr, *vol = nullptr, *contrib = nullptr;
  uint32_t *ent = nullptr, *off = nullptr, *gstart = nullptr;
  float *charge = nullptr, *nvolt = nullptr, *cap = nullptr, *leak = nullptr;
  int32_t *locator = nullptr;
  float *snap = nullptr;  // initial cur, vol, charge, nvolt
  // round launch state
  std::vector<RoundCircuit> h_circ;
  RoundCircuit *d_circ = nullptr;
  BatchItem *d_items = nullptr;
  uint32_t num_items = 0;
  uint32_t *sync_mem = nullptr;
  ckt_batch_config cfg = {256, 1, 2, 0};
  bool tables_valid = false;
  int grid = 0;
  cudaStream_t cap_stream = nullptr;
  cudaGraphExec_t gexec[2] = {nullptr, nullptr};
  uint64_t timeout_ns = 2000000000ull;
  int64_t device_bytes = 0;
  int sm_count = 0;
  std::vector<void *> allocs;
};

namespace {

template <typename T>
int dalloc(ckt_batch *b, T **p, size_t count) {
  const size_t bytes = std::max<size_t>(count * sizeof(T), 256);
  cudaError_t e = cudaMalloc(reinterpret_cast<void **>(p), bytes);
  if (e != cudaSuccess)
    return set_error(CKT_ENOMEM, "cudaMalloc of %zu bytes failed: %s", bytes, cudaGetErrorString(e));
  b->allocs.push_back(*p);
  b->device_bytes += (int64_t)bytes;
  return CKT_OK;
}

void free_batch(ckt_batch *b) {
  if (!b) return;
  for (int m = 0; m < 2; m++)
    if (b->gexec[m]) cudaGraphExecDestroy(b->gexec[m]);
  if (b->cap_stream) cudaStreamDestroy(b->cap_stream);
  for (void *p : b->allocs) cudaFree(p);
  delete b;
}

void invalidate_graphs(ckt_batch *b) {
  for (int m = 0; m < 2; m++)
    if (b->gexec[m]) {
      cudaGraphExecDestroy(b->gexec[m]);
      b->gexec[m] = nullptr;
    }
}

int64_t wires_of(const ckt_gen_params &p) { return (int64_t)p.num_pieces * p.wires_per_piece; }
int64_t nodes_of(const ckt_gen_params &p) { return (int64_t)p.num_pieces * p.nodes_per_piece; }

int layout(ckt_batch *b, int32_t num, const ckt_gen_params *shapes, const int32_t *steps) {
  CKT_REQUIRE(num >= 1 && shapes && steps, "need at least one circuit, shapes and steps");
  b->C = num;
  b->shapes.assign(shapes, shapes + num);
  b->steps.assign(steps, steps + num);
  b->wbase.assign(num + 1, 0);
  b->nbase.assign(num + 1, 0);
  b->obase.assign(num + 1, 0);
  b->gbase.assign(num + 1, 0);
  for (int32_t k = 0; k < num; k++) {
    const ckt_gen_params &p = shapes[k];
    CKT_REQUIRE(p.num_pieces >= 1 && p.nodes_per_piece >= 1 && p.wires_per_piece >= 0,
                "circuit %d has a bad shape", k);
    CKT_REQUIRE(steps[k] >= 0, "circuit %d has negative steps", k);
    const int64_t W = wires_of(p), N = nodes_of(p);
    CKT_REQUIRE(W <= kMaxWires && N < 0x7fffffffLL, "circuit %d too large", k);
    b->wbase[k + 1] = b->wbase[k] + W;
    b->nbase[k + 1] = b->nbase[k] + ((N + 3) & ~int64_t(3));
    b->obase[k + 1] = b->obase[k] + N + 1;
    b->gbase[k + 1] = b->gbase[k] + (int64_t)gstart_words(W);
    b->updates += (double)W * CKT_SEGMENTS * steps[k];
  }
  b->W = b->wbase[num];
  b->N = b->nbase[num];
  b->O = b->obase[num];
  b->G = b->gbase[num];
  CKT_CUDA(cudaDeviceGetAttribute(&b->sm_count, cudaDevAttrMultiProcessorCount, 0));
  return CKT_OK;
}

// Host copies of the field arrays.
struct HostFields {
  std::vector<uint32_t> in_ptr, out_ptr, slot_in, slot_out, ent, off, gstart;
  std::vector<uint8_t> in_loc, out_loc;
  std::vector<float> L, R, C, charge, nvolt, cap, leak;
  std::vector<int32_t> locator;
  explicit HostFields(const ckt_batch *b) {
    in_ptr.assign(b->W, 0); out_ptr.assign(b->W, 0);
    slot_in.assign(b->W, 0); slot_out.assign(b->W, 0);
    in_loc.assign(b->W, 0); out_loc.assign(b->W, 0);
    L.assign(b->W, 0.f); R.assign(b->W, 1.f); C.assign(b->W, 1.f);
    ent.assign(2 * b->W, 0); off.assign(b->O, 0); gstart.assign(b->G, 0);
    charge.assign(b->N, 0.f); nvolt.assign(b->N, 0.f); cap.assign(b->N, 1.f);
    leak.assign(b->N, 0.f); locator.assign(b->N, 1);
  }
  ckt_host_circuit slice(const ckt_batch *b, int32_t k, float *unused) {
    const int64_t w0 = b->wbase[k], x0 = b->nbase[k];
    ckt_host_circuit h;
    h.in_ptr = in_ptr.data() + w0; h.out_ptr = out_ptr.data() + w0;
    h.in_loc = in_loc.data() + w0; h.out_loc = out_loc.data() + w0;
    h.inductance = L.data() + w0; h.resistance = R.data() + w0; h.capacitance = C.data() + w0;
    h.current = unused; h.voltage = unused;
    h.charge = charge.data() + x0; h.node_voltage = nvolt.data() + x0;
    h.node_capacitance = cap.data() + x0; h.node_leakage = leak.data() + x0;
    h.locator = locator.data() + x0;
    return h;
  }
};

// Builds circuit k's graph from its slice and stores it in the field arrays.
int store_graph(const ckt_batch *b, HostFields &h, int32_t k) {
  HostGraph g;
  const int64_t w0 = b->wbase[k];
  int rc = build_circuit_graph(b->shapes[k], h.in_ptr.data() + w0, h.out_ptr.data() + w0,
                               h.in_loc.data() + w0, h.out_loc.data() + w0, g);
  if (rc) return rc;
  std::copy(g.ent.begin(), g.ent.end(), h.ent.begin() + 2 * w0);
  std::copy(g.slot_in.begin(), g.slot_in.end(), h.slot_in.begin() + w0);
  std::copy(g.slot_out.begin(), g.slot_out.end(), h.slot_out.begin() + w0);
  std::copy(g.off.begin(), g.off.end(), h.off.begin() + b->obase[k]);
  std::copy(g.gstart.begin(), g.gstart.end(), h.gstart.begin() + b->gbase[k]);
  return CKT_OK;
}

int run_parallel(int32_t n, int threads, const std::function<int(int32_t)> &fn) {
  const int T = std::max(1, std::min<int>(threads, n));
  std::vector<int> rcs(n, CKT_OK);
  std::vector<std::string> errs(n);
  std::vector<std::thread> pool;
  for (int t = 0; t < T; t++)
    pool.emplace_back([&, t]() {
      for (int32_t k = t; k < n; k += T) {
        rcs[k] = fn(k);
        if (rcs[k]) errs[k] = ckt_last_error();
      }
    });
  for (auto &th : pool) th.join();
  for (int32_t k = 0; k < n; k++)
    if (rcs[k]) return set_error(rcs[k], "circuit %d: %s", k, errs[k].c_str());
  return CKT_OK;
}

int upload_all(ckt_batch *b, HostFields &h, const float *cur, const float *vol) {
  const int64_t W = b->W, N = b->N;
  int rc;
  if ((rc = dalloc(b, &b->in_ptr, W)) || (rc = dalloc(b, &b->out_ptr, W)) ||
      (rc = dalloc(b, &b->slot_in, W)) || (rc = dalloc(b, &b->slot_out, W)) ||
      (rc = dalloc(b, &b->in_loc, W)) || (rc = dalloc(b, &b->out_loc, W)) ||
      (rc = dalloc(b, &b->L, W)) || (rc = dalloc(b, &b->R, W)) || (rc = dalloc(b, &b->Cw, W)) ||
      (rc = dalloc(b, &b->cur, 10 * W)) || (rc = dalloc(b, &b->vol, 9 * W)) ||
      (rc = dalloc(b, &b->contrib, 2 * W)) || (rc = dalloc(b, &b->ent, 2 * W)) ||
      (rc = dalloc(b, &b->off, b->O)) || (rc = dalloc(b, &b->gstart, b->G)) ||
      (rc = dalloc(b, &b->charge, N)) || (rc = dalloc(b, &b->nvolt, N)) ||
      (rc = dalloc(b, &b->cap, N)) || (rc = dalloc(b, &b->leak, N)) ||
      (rc = dalloc(b, &b->locator, N)) || (rc = dalloc(b, &b->snap, 19 * W + 2 * N)) ||
      (rc = dalloc(b, &b->d_circ, b->C)) || (rc = dalloc(b, &b->sync_mem, 2 + 2 * b->C)))
    return rc;
  auto up = [](void *d, const void *s, size_t bytes) {
    return bytes ? cudaMemcpy(d, s, bytes, cudaMemcpyHostToDevice) : cudaSuccess;
  };
  CKT_CUDA(up(b->in_ptr, h.in_ptr.data(), W * 4));
  CKT_CUDA(up(b->out_ptr, h.out_ptr.data(), W * 4));
  CKT_CUDA(up(b->slot_in, h.slot_in.data(), W * 4));
  CKT_CUDA(up(b->slot_out, h.slot_out.data(), W * 4));
  CKT_CUDA(up(b->in_loc, h.in_loc.data(), W));
  CKT_CUDA(up(b->out_loc, h.out_loc.data(), W));
  CKT_CUDA(up(b->L, h.L.data(), W * 4));
  CKT_CUDA(up(b->R, h.R.data(), W * 4));
  CKT_CUDA(up(b->Cw, h.C.data(), W * 4));
  CKT_CUDA(up(b->ent, h.ent.data(), 2 * W * 4));
  CKT_CUDA(up(b->off, h.off.data(), b->O * 4));
  CKT_CUDA(up(b->gstart, h.gstart.data(), b->G * 4));
  CKT_CUDA(up(b->charge, h.charge.data(), N * 4));
  CKT_CUDA(up(b->nvolt, h.nvolt.data(), N * 4));
  CKT_CUDA(up(b->cap, h.cap.data(), N * 4));
  CKT_CUDA(up(b->leak, h.leak.data(), N * 4));
  CKT_CUDA(up(b->locator, h.locator.data(), N * 4));
  if (cur) CKT_CUDA(up(b->cur, cur, 10 * W * 4));
  else CKT_CUDA(cudaMemset(b->cur, 0, 10 * W * 4));
  if (vol) CKT_CUDA(up(b->vol, vol, 9 * W * 4));
  else CKT_CUDA(cudaMemset(b->vol, 0, 9 * W * 4));
  CKT_CUDA(cudaMemcpy(b->snap, b->cur, 10 * W * 4, cudaMemcpyDeviceToDevice));
  CKT_CUDA(cudaMemcpy(b->snap + 10 * W, b->vol, 9 * W * 4, cudaMemcpyDeviceToDevice));
  CKT_CUDA(cudaMemcpy(b->snap + 19 * W, b->charge, N * 4, cudaMemcpyDeviceToDevice));
  CKT_CUDA(cudaMemcpy(b->snap + 19 * W + N, b->nvolt, N * 4, cudaMemcpyDeviceToDevice));
  // descriptors
  b->h_circ.resize(b->C);
  for (int32_t k = 0; k < b->C; k++) {
    RoundCircuit &rc = b->h_circ[k];
    memset(&rc, 0, sizeof(rc));
    const int64_t w0 = b->wbase[k], x0 = b->nbase[k];
    rc.in_ptr = b->in_ptr + w0; rc.out_ptr = b->out_ptr + w0;
    rc.in_loc = b->in_loc + w0; rc.out_loc = b->out_loc + w0;
    rc.L = b->L + w0; rc.R = b->R + w0; rc.C = b->Cw + w0;
    rc.cur = b->cur + 10 * w0; rc.vol = b->vol + 9 * w0;
    rc.charge = b->charge + x0; rc.nvolt = b->nvolt + x0;
    rc.cap = b->cap + x0; rc.leak = b->leak + x0;
    rc.off = b->off + b->obase[k]; rc.ent = b->ent + 2 * w0;
    rc.slot_in = b->slot_in + w0; rc.slot_out = b->slot_out + w0;
    rc.gstart = b->gstart + b->gbase[k]; rc.contrib = b->contrib + 2 * w0;
    rc.W = (uint32_t)wires_of(b->shapes[k]);
    rc.N = (uint32_t)nodes_of(b->shapes[k]);
    rc.steps = b->steps[k];
  }
  return CKT_OK;
}

int build_tables(ckt_batch *b) {
  std::vector<BatchItem> items;
  build_round_table(b->h_circ, b->cfg, items);
  b->num_items = (uint32_t)items.size();
  if (b->d_items) {
    cudaFree(b->d_items);
    b->allocs.erase(std::find(b->allocs.begin(), b->allocs.end(), (void *)b->d_items));
    b->d_items = nullptr;
  }
  int rc;
  if ((rc = dalloc(b, &b->d_items, std::max<size_t>(items.size(), 1)))) return rc;
  if (!items.empty())
    CKT_CUDA(cudaMemcpy(b->d_items, items.data(), items.size() * sizeof(BatchItem),
                        cudaMemcpyHostToDevice));
  CKT_CUDA(cudaMemcpy(b->d_circ, b->h_circ.data(), b->h_circ.size() * sizeof(RoundCircuit),
                      cudaMemcpyHostToDevice));
  int per_sm = 1;
  if ((rc = round_blocks_per_sm(b->cfg, &per_sm))) return rc;
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
  return launch_round(mode, b->cfg, b->grid, b->d_items, b->num_items, b->d_circ, (uint32_t)b->C,
                      b->sync_mem, b->timeout_ns, s);
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

int check_mode(int32_t mode) {
  CKT_REQUIRE(mode == CKT_MODE_EXACT || mode == CKT_MODE_FAST, "unknown mode %d", mode);
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
  HostFields h(b);
  std::vector<float> cur(10 * b->W), vol(9 * b->W);
  for (int32_t k = 0; k < num_circuits; k++) {
    const ckt_host_circuit &c = circuits[k];
    const int64_t w0 = b->wbase[k], W = b->wbase[k + 1] - w0, x0 = b->nbase[k];
    const int64_t N = nodes_of(shapes[k]);
    if (!(c.in_ptr && c.out_ptr && c.in_loc && c.out_loc && c.inductance && c.resistance &&
          c.capacitance && c.current && c.voltage && c.charge && c.node_voltage &&
          c.node_capacitance && c.node_leakage && c.locator)) {
      free_batch(b);
      return set_error(CKT_EINVAL, "circuit %d has NULL arrays", k);
    }
    memcpy(h.in_ptr.data() + w0, c.in_ptr, W * 4);
    memcpy(h.out_ptr.data() + w0, c.out_ptr, W * 4);
    memcpy(h.in_loc.data() + w0, c.in_loc, W);
    memcpy(h.out_loc.data() + w0, c.out_loc, W);
    memcpy(h.L.data() + w0, c.inductance, W * 4);
    memcpy(h.R.data() + w0, c.resistance, W * 4);
    memcpy(h.C.data() + w0, c.capacitance, W * 4);
    memcpy(cur.data() + 10 * w0, c.current, 10 * W * 4);
    memcpy(vol.data() + 9 * w0, c.voltage, 9 * W * 4);
    memcpy(h.charge.data() + x0, c.charge, N * 4);
    memcpy(h.nvolt.data() + x0, c.node_voltage, N * 4);
    memcpy(h.cap.data() + x0, c.node_capacitance, N * 4);
    memcpy(h.leak.data() + x0, c.node_leakage, N * 4);
    memcpy(h.locator.data() + x0, c.locator, N * 4);
  }
  rc = run_parallel(num_circuits, (int)std::thread::hardware_concurrency(),
                    [&](int32_t k) { return store_graph(b, h, k); });
  if (!rc) rc = upload_all(b, h, cur.data(), vol.data());
  if (rc) { free_batch(b); return rc; }
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
  HostFields h(b);
  float unused = 0.f;
  rc = run_parallel(num_circuits, host_threads > 0 ? host_threads : 1, [&](int32_t k) {
    ckt_host_circuit s = h.slice(b, k, &unused);
    int r = generate_into(&b->shapes[k], &s, 0);
    return r ? r : store_graph(b, h, k);
  });
  if (!rc) rc = upload_all(b, h, nullptr, nullptr);
  if (rc) { free_batch(b); return rc; }
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
  if (first_wire) *first_wire = b->wbase[circuit];
  if (first_node) *first_node = b->nbase[circuit];
  return CKT_OK;
}

int ckt_batch_set_config(ckt_batch *b, const ckt_batch_config *c) {
  CKT_REQUIRE(b != nullptr, "batch is NULL");
  int rc = check_batch_config(c);
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
  NvtxRange range("ckt_batch_run");
  CKT_REQUIRE(b != nullptr, "batch is NULL");
  int rc = check_mode(mode);
  if (rc || (rc = ensure_graph(b, mode))) return rc;
  CKT_CUDA(cudaGraphLaunch(b->gexec[mode], as_stream(stream)));
  return CKT_OK;
}

int ckt_batch_run_direct(ckt_batch *b, int32_t mode, void *stream) {
  CKT_REQUIRE(b != nullptr, "batch is NULL");
  int rc = check_mode(mode);
  if (rc) return rc;
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

int ckt_batch_run_sequential(ckt_batch *b, int32_t mode, int32_t per_piece, void *stream) {
  CKT_REQUIRE(b != nullptr, "batch is NULL");
  int rc = check_mode(mode);
  if (rc) return rc;
  const cudaStream_t s = as_stream(stream);
  for (int32_t k = 0; k < b->C; k++) {
    const RoundCircuit &c = b->h_circ[k];
    const ckt_gen_params &p = b->shapes[k];
    ckt_wires w = {c.in_ptr, c.out_ptr, c.in_loc, c.out_loc, c.L, c.R, c.C, c.cur, c.vol,
                   (int64_t)std::max<uint32_t>(c.W, 1)};
    ckt_params prm = {c.steps, (float)1e-6, mode, CKT_INIT_KERNEL};
    if (per_piece) {
      for (int32_t n = 0; n < p.num_pieces; n++) {
        if ((rc = launch_cnc((uint32_t)((int64_t)n * p.wires_per_piece), (uint32_t)p.wires_per_piece,
                             w, c.nvolt, c.nvolt, c.nvolt, &prm, s)))
          return rc;
        CKT_CUDA(cudaStreamSynchronize(s));
      }
    } else if ((rc = launch_cnc(0, c.W, w, c.nvolt, c.nvolt, c.nvolt, &prm, s))) {
      return rc;
    }
    if (c.W > 0 && c.N > 0) {  // the plain path's distribute_charge
      dc_all_kernel<<<grid_for(c.N, kDcBlock), kDcBlock, 0, s>>>(
          0u, c.N, c.off, c.ent, c.cur, c.cur + 9 * (size_t)c.W, c.charge, prm.dt);
      CKT_CHECK_LAUNCH();
    }
    if (per_piece) {
      CKT_CUDA(cudaStreamSynchronize(s));
      for (int32_t n = 0; n < p.num_pieces; n++) {
        uv_all_scalar_kernel<<<grid_for(p.nodes_per_piece), 256, 0, s>>>(
            (uint32_t)((int64_t)n * p.nodes_per_piece), (uint32_t)p.nodes_per_piece, c.charge,
            c.nvolt, c.cap, c.leak);
        CKT_CHECK_LAUNCH();
        CKT_CUDA(cudaStreamSynchronize(s));
      }
    } else {
      const uint32_t n4 = c.N / 4;
      if (n4)
        uv_all_vec4_kernel<<<grid_for(n4), 256, 0, s>>>(
            n4, reinterpret_cast<float4 *>(c.charge), reinterpret_cast<float4 *>(c.nvolt),
            reinterpret_cast<const float4 *>(c.cap), reinterpret_cast<const float4 *>(c.leak));
      if (c.N > 4 * n4)
        uv_all_scalar_kernel<<<1, 256, 0, s>>>(4 * n4, c.N - 4 * n4, c.charge, c.nvolt, c.cap,
                                               c.leak);
      CKT_CHECK_LAUNCH();
    }
  }
  return CKT_OK;
}

int ckt_batch_autotune(ckt_batch *b, int32_t mode, void *stream, ckt_batch_config *chosen) {
  NvtxRange range("ckt_batch_autotune");
  CKT_REQUIRE(b != nullptr, "batch is NULL");
  int rc = check_mode(mode);
  if (rc) return rc;
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
      rc = ckt_batch_set_config(b, &it->second);
      if (rc == CKT_OK && chosen) *chosen = b->cfg;
      return rc;
    }
  }
  cudaEvent_t e0, e1;
  CKT_CUDA(cudaEventCreate(&e0));
  CKT_CUDA(cudaEventCreate(&e1));
  float best = 1e30f;
  ckt_batch_config best_cfg = b->cfg;
  for (int block : {128, 256})
    for (int wpt : {1, 2})
      for (int dcs : {0, 1, 2}) {
        if (rc) break;
        ckt_batch_config c = {block, wpt, dcs, 0};
        if ((rc = ckt_batch_set_config(b, &c)) || (rc = ckt_batch_reset_state(b, stream)) ||
            (rc = launch(b, mode, s)) || (rc = ckt_batch_check(b, stream)) ||
            (rc = ckt_batch_reset_state(b, stream)))
          break;
        cudaEventRecord(e0, s);
        if ((rc = launch(b, mode, s))) break;
        cudaEventRecord(e1, s);
        if ((rc = ckt_batch_check(b, stream))) break;
        float ms = 0.f;
        cudaEventElapsedTime(&ms, e0, e1);
        if (ms < best) {
          best = ms;
          best_cfg = b->cfg;
        }
      }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (rc) return rc;
  if ((rc = ckt_batch_set_config(b, &best_cfg)) || (rc = ckt_batch_reset_state(b, stream)))
    return rc;
  {
    std::lock_guard<std::mutex> g(g_tune_mu);
    g_tune_cache[key] = b->cfg;
  }
  if (chosen) *chosen = b->cfg;
  return CKT_OK;
}

int ckt_batch_read_state(ckt_batch *b, int32_t circuit, float *current, float *voltage,
                         float *charge, float *node_voltage, void *stream) {
  CKT_REQUIRE(b != nullptr && circuit >= 0 && circuit < b->C, "bad batch or circuit index");
  const cudaStream_t s = as_stream(stream);
  const RoundCircuit &c = b->h_circ[circuit];
  if (current && c.W)
    CKT_CUDA(cudaMemcpyAsync(current, c.cur, 10 * (size_t)c.W * 4, cudaMemcpyDeviceToHost, s));
  if (voltage && c.W)
    CKT_CUDA(cudaMemcpyAsync(voltage, c.vol, 9 * (size_t)c.W * 4, cudaMemcpyDeviceToHost, s));
  if (charge) CKT_CUDA(cudaMemcpyAsync(charge, c.charge, (size_t)c.N * 4, cudaMemcpyDeviceToHost, s));
  if (node_voltage)
    CKT_CUDA(cudaMemcpyAsync(node_voltage, c.nvolt, (size_t)c.N * 4, cudaMemcpyDeviceToHost, s));
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
  RoundCircuit c = b->h_circ[circuit];
  if (enable) c.cnc_items += 1;  // a CNC tile that no item will ever complete
  CKT_CUDA(cudaMemcpy(b->d_circ + circuit, &c, sizeof(c), cudaMemcpyHostToDevice));
  return CKT_OK;
}

}  // extern "C"
