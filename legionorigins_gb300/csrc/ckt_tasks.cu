// ckt_tasks.cu -- C-ABI entry points of the three leaf tasks (per piece and
// index-space), fold application and wire validation.
#include <climits>
#include <cstring>

#include "ckt_dctile.cuh"
#include "ckt_internal.h"
#include "ckt_kernels.cuh"

namespace ckt {

static thread_local std::string g_last_error;

int set_error(int status, const char *fmt, ...) {
  char buf[1024];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  g_last_error = buf;
  return status;
}

int validate_wires(const ckt_wires &w) {
  CKT_REQUIRE(w.in_ptr && w.out_ptr && w.in_loc && w.out_loc, "wire pointer/location arrays are NULL");
  CKT_REQUIRE(w.inductance && w.resistance && w.capacitance, "wire L/R/C arrays are NULL");
  CKT_REQUIRE(w.current && w.voltage, "wire current/voltage arrays are NULL");
  CKT_REQUIRE(w.seg_stride > 0, "wire seg_stride must be positive (got %lld)", (long long)w.seg_stride);
  return CKT_OK;
}

int validate_nodes(const ckt_nodes &n, const char *what) {
  CKT_REQUIRE(n.charge && n.voltage && n.capacitance && n.leakage, "%s node instance has NULL arrays",
              what);
  return CKT_OK;
}

int validate_params(const ckt_params *p) {
  CKT_REQUIRE(p != nullptr, "params is NULL");
  CKT_REQUIRE(p->steps >= 0, "steps must be >= 0 (got %d)", p->steps);
  CKT_REQUIRE(p->mode == CKT_MODE_EXACT || p->mode == CKT_MODE_FAST ||
                  p->mode == CKT_MODE_FAST_SCALAR || p->mode == CKT_MODE_EXACT_DIVIDE,
              "unknown mode %d", p->mode);
  CKT_REQUIRE(p->init == CKT_INIT_KERNEL || p->init == CKT_INIT_CPU_TASK, "unknown init %d", p->init);
  return CKT_OK;
}

WireArrays wire_arrays(const ckt_wires &w) {
  WireArrays a;
  a.in_ptr = w.in_ptr;
  a.out_ptr = w.out_ptr;
  a.in_loc = w.in_loc;
  a.out_loc = w.out_loc;
  a.L = w.inductance;
  a.R = w.resistance;
  a.C = w.capacitance;
  a.cur = w.current;
  a.vol = w.voltage;
  a.S = w.seg_stride;
  return a;
}

// SMs of the calling thread's current device (looked up once per device).
static int device_sms() {
  static thread_local int dev_cached = -1, sms = 0;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return 0;
  if (dev != dev_cached) {
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) sms = 0;
    dev_cached = dev;
  }
  return sms;
}

template <int M, int I>
static void launch_cnc_t(uint32_t first, uint32_t n, const ckt_wires &w, const float *vp,
                         const float *vs, const float *vg, const ckt_params *p, cudaStream_t s) {
  const WireArrays a = wire_arrays(w);
  const NodeVolts v = {vp, vs, vg};
  // EXACT with at most three warps per SM scheduler: one wire per thread in
  // one-warp blocks, spread over every SM, runs each step several times
  // faster than the paired kernel on the few SMs its blocks would occupy
  // (same bits: the scalar and paired steppers round every operation alike).
  const int sms = M == CKT_MODE_EXACT ? device_sms() : 0;
  if (M == CKT_MODE_EXACT && sms > 0 && n <= 384u * (uint32_t)sms) {
    cnc_kernel<M, I><<<grid_for(n, 32), 32, 0, s>>>(first, n, a, v, p->steps, p->dt);
    return;
  }
  if constexpr (M == CKT_MODE_FAST || M == CKT_MODE_EXACT)  // two wires per thread, paired
    cnc_pair_kernel<M, I><<<grid_for(n, 2 * kPairBlock), kPairBlock, 0, s>>>(first, n, a, v,
                                                                             p->steps, p->dt);
  else
    cnc_kernel<M, I><<<grid_for(n), 256, 0, s>>>(first, n, a, v, p->steps, p->dt);
}

int launch_cnc(uint32_t first, uint32_t n, const ckt_wires &w, const float *vp,
                      const float *vs, const float *vg, const ckt_params *p, cudaStream_t s) {
  if (n == 0) return CKT_OK;
  CKT_REQUIRE((int64_t)first + n <= w.seg_stride,
              "wire range [%u, %llu) exceeds seg_stride %lld", first,
              (unsigned long long)first + n, (long long)w.seg_stride);
  if (p->mode == CKT_MODE_EXACT) {
    if (p->init == CKT_INIT_KERNEL) launch_cnc_t<CKT_MODE_EXACT, CKT_INIT_KERNEL>(first, n, w, vp, vs, vg, p, s);
    else launch_cnc_t<CKT_MODE_EXACT, CKT_INIT_CPU_TASK>(first, n, w, vp, vs, vg, p, s);
  } else if (p->mode == CKT_MODE_FAST) {
    if (p->init == CKT_INIT_KERNEL) launch_cnc_t<CKT_MODE_FAST, CKT_INIT_KERNEL>(first, n, w, vp, vs, vg, p, s);
    else launch_cnc_t<CKT_MODE_FAST, CKT_INIT_CPU_TASK>(first, n, w, vp, vs, vg, p, s);
  } else if (p->mode == CKT_MODE_FAST_SCALAR) {
    if (p->init == CKT_INIT_KERNEL) launch_cnc_t<kModeFastScalar, CKT_INIT_KERNEL>(first, n, w, vp, vs, vg, p, s);
    else launch_cnc_t<kModeFastScalar, CKT_INIT_CPU_TASK>(first, n, w, vp, vs, vg, p, s);
  } else {
    if (p->init == CKT_INIT_KERNEL) launch_cnc_t<CKT_MODE_EXACT_DIVIDE, CKT_INIT_KERNEL>(first, n, w, vp, vs, vg, p, s);
    else launch_cnc_t<CKT_MODE_EXACT_DIVIDE, CKT_INIT_CPU_TASK>(first, n, w, vp, vs, vg, p, s);
  }
  CKT_CHECK_LAUNCH();
  return CKT_OK;
}

static int check_graph_wires(const ckt_graph *g, const ckt_wires &w) {
  CKT_REQUIRE(g != nullptr, "graph is NULL");
  CKT_REQUIRE(w.seg_stride >= g->W, "wires.seg_stride %lld is smaller than the graph's %lld wires",
              (long long)w.seg_stride, (long long)g->W);
  return CKT_OK;
}

// The tiled node pass needs 16-byte aligned current slices that may be read
// up to a multiple of 4 wires: current 16-byte aligned, seg_stride a
// multiple of 4 (then seg_stride >= W rounds W up).
static bool tile_plan_usable(const ckt_graph *g, const ckt_wires &w) {
  return g->num_tiles > 0 && (reinterpret_cast<uintptr_t>(w.current) & 15u) == 0 &&
         (w.seg_stride & 3) == 0;
}


template <bool UV>
static int launch_dc_tile(const ckt_graph *g, const ckt_wires &w, const ckt_nodes &n, float dt,
                          cudaStream_t s) {
  static thread_local int configured_device = -1;
  int dev = 0;
  CKT_CUDA(cudaGetDevice(&dev));
  if (configured_device != dev) {
    const int most = (int)dc_tile_smem_bytes(kTileNodesMax);
    CKT_CUDA(cudaFuncSetAttribute(dc_tile_kernel<true>,
                                  cudaFuncAttributeMaxDynamicSharedMemorySize, most));
    CKT_CUDA(cudaFuncSetAttribute(dc_tile_kernel<false>,
                                  cudaFuncAttributeMaxDynamicSharedMemorySize, most));
    configured_device = dev;
  }
  DcTileArgs a;
  a.tile_step = g->tile_step;
  a.steps = g->tile_steps;
  a.ent = g->tile_ent;
  a.ghost = g->ghost;
  a.mask = g->tile_mask;
  a.I0 = w.current;
  a.I9 = w.current + 9 * w.seg_stride;
  a.charge = n.charge;
  a.voltage = n.voltage;
  a.cap = n.capacitance;
  a.leak = n.leakage;
  a.error = g->tile_error;
  a.timeout_ns = g->tile_timeout_ns;
  a.N = (uint32_t)g->N;
  a.W = (uint32_t)g->W;
  a.tile_nodes = g->tile_nodes;
  a.node_copy = ((reinterpret_cast<uintptr_t>(n.voltage) | reinterpret_cast<uintptr_t>(n.capacitance) |
                  reinterpret_cast<uintptr_t>(n.leakage)) & 15u) == 0;
  a.dt = dt;
  // The ghost buffer is the graph's: passes on other streams are ordered
  // behind the previous pass (not inside a stream capture, where the
  // captured work is ordered by whoever launches the graph).
  std::lock_guard<std::mutex> lock(g->ghost_mu);
  cudaStreamCaptureStatus capture = cudaStreamCaptureStatusNone;
  if (cudaStreamIsCapturing(s, &capture) != cudaSuccess) {
    (void)cudaGetLastError();
    capture = cudaStreamCaptureStatusActive;
  }
  const bool order = g->ghost_n > 0 && capture == cudaStreamCaptureStatusNone;
  if (order && g->ghost_used && g->ghost_stream != s)
    CKT_CUDA(cudaStreamWaitEvent(s, g->ghost_done, 0));
  // The tile pass may start while the packing runs (programmatic dependent
  // launch): its stream steps need only calc_new_currents' results, which
  // were complete before the packing began; its copy lane waits for the
  // packing before the first ghost step.
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(g->num_tiles);
  cfg.blockDim = dim3(kTileBlock);
  cfg.dynamicSmemBytes = dc_tile_smem_bytes(g->tile_nodes);
  cfg.stream = s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  if (g->ghost_n > 0) {
    const uint32_t n = (uint32_t)g->ghost_n;
    if (g->ghost_staged) {
      ghost_pack_kernel<true><<<g->ghost_blocks, kPackBlock, 0, s>>>(
          g->ghost_list, g->ghost_block, n, (uint32_t)g->W, a.I0, a.I9, g->ghost);
    } else {
      const uint32_t per_block = kPackBlock * kPackPer;
      ghost_pack_kernel<false><<<(n + per_block - 1) / per_block, kPackBlock, 0, s>>>(
          g->ghost_list, g->ghost_block, n, (uint32_t)g->W, a.I0, a.I9, g->ghost);
    }
    CKT_CHECK_LAUNCH();
    cfg.attrs = attr;
    cfg.numAttrs = 1;
  }
  CKT_CUDA(cudaLaunchKernelEx(&cfg, dc_tile_kernel<UV>, a));
  if (order) {
    CKT_CUDA(cudaEventRecord(g->ghost_done, s));
    g->ghost_stream = s;
    g->ghost_used = true;
  }
  return CKT_OK;
}

// A tiled node pass that ran out of a copy wait left its tile's results
// unwritten and set the graph's host-visible error word; every later
// index-space call on the graph reports it until ckt_graph_check (or
// ckt_graph_tile_info) clears it.
static int check_tile_error(const ckt_graph *g) {
  if (g->tile_error_host && *g->tile_error_host)
    return set_error(CKT_ETIMEOUT,
                     "an earlier tiled node pass on this graph ran out of a copy wait and left "
                     "a tile unwritten (ckt_graph_check clears the report)");
  return CKT_OK;
}

// Completion wait of the blocking task forms.
static int wait_stream(void *stream, const char *task) {
  const cudaError_t e = cudaStreamSynchronize(as_stream(stream));
  if (e != cudaSuccess)
    return set_error(CKT_ECUDA, "%s failed on the device: %s", task, cudaGetErrorString(e));
  return CKT_OK;
}

}  // namespace ckt

using namespace ckt;

extern "C" {

int ckt_abi_version(void) { return CKT_ABI_VERSION; }

const char *ckt_last_error(void) { return g_last_error.c_str(); }

const char *ckt_status_string(int status) {
  switch (status) {
    case CKT_OK: return "ok";
    case CKT_EINVAL: return "invalid argument";
    case CKT_ECUDA: return "CUDA error";
    case CKT_EBOUNDS: return "pointer or location out of bounds";
    case CKT_ETIMEOUT: return "bounded device wait timed out";
    case CKT_ENOMEM: return "out of memory or over budget";
    case CKT_EBUSY: return "busy";
    case CKT_ECANCELLED: return "cancelled";
    default: return "unknown status";
  }
}

void ckt_default_params(ckt_params *out) {
  if (!out) return;
  out->steps = 10000;
  out->dt = (float)1e-6;
  out->mode = CKT_MODE_EXACT;
  out->init = CKT_INIT_KERNEL;
}

int ckt_calc_new_currents(const ckt_piece *piece, ckt_wires wires, ckt_nodes pvt, ckt_nodes shr,
                          ckt_nodes ghost, const ckt_params *prm, void *stream) {
  CKT_REQUIRE(piece != nullptr, "piece is NULL");
  int rc;
  if ((rc = validate_params(prm))) return rc;
  if (piece->num_wires == 0) return CKT_OK;
  if ((rc = validate_wires(wires))) return rc;
  CKT_REQUIRE(pvt.voltage && shr.voltage && ghost.voltage, "node voltage arrays are NULL");
  return launch_cnc(piece->first_wire, piece->num_wires, wires, pvt.voltage, shr.voltage,
                    ghost.voltage, prm, as_stream(stream));
}

int ckt_calc_new_currents_all(const ckt_graph *graph, ckt_wires wires, ckt_nodes nodes,
                              const ckt_params *prm, void *stream) {
  int rc;
  CKT_REQUIRE(graph != nullptr, "graph is NULL");
  if ((rc = validate_params(prm))) return rc;
  if (graph->W == 0) return CKT_OK;
  if ((rc = validate_wires(wires)) || (rc = check_graph_wires(graph, wires))) return rc;
  CKT_REQUIRE(nodes.voltage != nullptr, "node voltage array is NULL");
  return launch_cnc(0, (uint32_t)graph->W, wires, nodes.voltage, nodes.voltage, nodes.voltage, prm,
                    as_stream(stream));
}

int ckt_distribute_charge(const ckt_graph *graph, int32_t piece_index, ckt_wires wires,
                          ckt_nodes pvt, float *shr_fold, float *ghost_fold,
                          const ckt_params *prm, void *stream) {
  int rc;
  CKT_REQUIRE(graph != nullptr, "graph is NULL");
  if ((rc = validate_params(prm))) return rc;
  CKT_REQUIRE(piece_index >= 0 && piece_index < graph->P, "piece_index %d out of range [0, %d)",
              piece_index, graph->P);
  if (graph->pieces[piece_index].num_wires == 0) return CKT_OK;
  if ((rc = validate_wires(wires)) || (rc = check_graph_wires(graph, wires))) return rc;
  CKT_REQUIRE(pvt.charge != nullptr, "pvt.charge is NULL");
  const int64_t t0 = graph->touch_first[piece_index], t1 = graph->touch_first[piece_index + 1];
  if (t1 == t0) return CKT_OK;
  CKT_REQUIRE(shr_fold != nullptr && ghost_fold != nullptr, "fold instances are NULL");
  const float *I0 = wires.current, *I9 = wires.current + 9 * wires.seg_stride;
  dc_piece_kernel<<<grid_for(t1 - t0), 256, 0, as_stream(stream)>>>(
      (uint32_t)t0, (uint32_t)(t1 - t0), graph->touch_node, graph->touch_loc, graph->touch_off,
      graph->piece_ent, I0, I9, pvt.charge, shr_fold, ghost_fold, prm->dt);
  CKT_CHECK_LAUNCH();
  return CKT_OK;
}

int ckt_distribute_charge_atomic(const ckt_piece *piece, ckt_wires wires, ckt_nodes pvt,
                                 float *shr_fold, float *ghost_fold, const ckt_params *prm,
                                 void *stream) {
  CKT_REQUIRE(piece != nullptr, "piece is NULL");
  int rc;
  if ((rc = validate_params(prm))) return rc;
  if (piece->num_wires == 0) return CKT_OK;
  CKT_REQUIRE(wires.in_ptr && wires.out_ptr && wires.in_loc && wires.out_loc,
              "wire pointer/location arrays are NULL");
  CKT_REQUIRE(wires.current != nullptr && wires.seg_stride > 0,
              "wire currents are NULL or seg_stride is not positive");
  CKT_REQUIRE((int64_t)piece->first_wire + piece->num_wires <= wires.seg_stride,
              "wire range [%u, %llu) exceeds seg_stride %lld", piece->first_wire,
              (unsigned long long)piece->first_wire + piece->num_wires,
              (long long)wires.seg_stride);
  CKT_REQUIRE(pvt.charge != nullptr && shr_fold != nullptr && ghost_fold != nullptr,
              "pvt.charge or a fold instance is NULL");
  const float *I0 = wires.current, *I9 = wires.current + 9 * wires.seg_stride;
  dc_atomic_kernel<<<grid_for(piece->num_wires), 256, 0, as_stream(stream)>>>(
      piece->first_wire, piece->num_wires, wires.in_ptr, wires.out_ptr, wires.in_loc,
      wires.out_loc, I0, I9, pvt.charge, shr_fold, ghost_fold, prm->dt);
  CKT_CHECK_LAUNCH();
  return CKT_OK;
}

int ckt_distribute_charge_atomic_sync(const ckt_piece *piece, ckt_wires wires, ckt_nodes pvt,
                                      float *shr_fold, float *ghost_fold, const ckt_params *prm,
                                      void *stream) {
  const int rc =
      ckt_distribute_charge_atomic(piece, wires, pvt, shr_fold, ghost_fold, prm, stream);
  return rc ? rc : wait_stream(stream, "distribute_charge");
}

int ckt_apply_fold(const ckt_graph *graph, int32_t piece_index, float *shr_fold, float *ghost_fold,
                   float *charge, void *stream) {
  CKT_REQUIRE(graph != nullptr, "graph is NULL");
  CKT_REQUIRE(piece_index >= 0 && piece_index < graph->P, "piece_index %d out of range [0, %d)",
              piece_index, graph->P);
  CKT_REQUIRE(shr_fold && ghost_fold && charge, "NULL fold or charge array");
  const int64_t t0 = graph->touch_first[piece_index], t1 = graph->touch_first[piece_index + 1];
  if (t1 == t0) return CKT_OK;
  apply_fold_kernel<<<grid_for(t1 - t0), 256, 0, as_stream(stream)>>>(
      (uint32_t)t0, (uint32_t)(t1 - t0), graph->touch_node, graph->touch_loc, shr_fold, ghost_fold,
      charge);
  CKT_CHECK_LAUNCH();
  return CKT_OK;
}

int ckt_distribute_charge_all(const ckt_graph *graph, ckt_wires wires, ckt_nodes nodes,
                              const ckt_params *prm, void *stream) {
  int rc;
  CKT_REQUIRE(graph != nullptr, "graph is NULL");
  if ((rc = validate_params(prm))) return rc;
  if ((rc = check_tile_error(graph))) return rc;
  if (graph->N == 0 || graph->W == 0) return CKT_OK;  // no wire deposits anything
  if ((rc = validate_wires(wires)) || (rc = check_graph_wires(graph, wires))) return rc;
  CKT_REQUIRE(nodes.charge != nullptr, "nodes.charge is NULL");
  if (tile_plan_usable(graph, wires))
    return launch_dc_tile<false>(graph, wires, nodes, prm->dt, as_stream(stream));
  // The staged gather: measured faster than scattering the contributions
  // into CSR order and summing them contiguously, whose random 4-byte writes
  // cost as much as the gathers they replace.
  const float *I0 = wires.current, *I9 = wires.current + 9 * wires.seg_stride;
  dc_all_kernel<<<grid_for(graph->N, kDcBlock), kDcBlock, 0, as_stream(stream)>>>(
      0u, (uint32_t)graph->N, graph->node_off, graph->node_ent, I0, I9, nodes.charge, prm->dt);
  CKT_CHECK_LAUNCH();
  return CKT_OK;
}

int ckt_update_voltages(const ckt_piece *piece, ckt_nodes pvt, ckt_nodes shr,
                        const int32_t *locator, void *stream) {
  CKT_REQUIRE(piece != nullptr, "piece is NULL");
  int rc;
  if ((rc = validate_nodes(pvt, "pvt")) || (rc = validate_nodes(shr, "shr"))) return rc;
  CKT_REQUIRE(locator != nullptr, "locator is NULL");
  if (piece->num_nodes == 0) return CKT_OK;
  uv_piece_kernel<<<grid_for(piece->num_nodes), 256, 0, as_stream(stream)>>>(
      piece->first_node, piece->num_nodes, locator, pvt, shr);
  CKT_CHECK_LAUNCH();
  return CKT_OK;
}

int ckt_update_voltages_all(const ckt_graph *graph, ckt_nodes nodes, void *stream) {
  CKT_REQUIRE(graph != nullptr, "graph is NULL");
  int rc;
  if ((rc = validate_nodes(nodes, "nodes"))) return rc;
  const uint64_t N = (uint64_t)graph->N;
  if (N == 0) return CKT_OK;
  const cudaStream_t s = as_stream(stream);
  const bool aligned = ((reinterpret_cast<uintptr_t>(nodes.charge) |
                         reinterpret_cast<uintptr_t>(nodes.voltage) |
                         reinterpret_cast<uintptr_t>(nodes.capacitance) |
                         reinterpret_cast<uintptr_t>(nodes.leakage)) &
                        15u) == 0;
  uint64_t done = 0;
  if (aligned && N >= 4) {
    const uint64_t n4 = N / 4;
    uv_all_vec4_kernel<<<grid_for(n4), 256, 0, s>>>(
        (uint32_t)n4, reinterpret_cast<float4 *>(nodes.charge),
        reinterpret_cast<float4 *>(nodes.voltage),
        reinterpret_cast<const float4 *>(nodes.capacitance),
        reinterpret_cast<const float4 *>(nodes.leakage));
    CKT_CHECK_LAUNCH();
    done = n4 * 4;
  }
  if (done < N) {
    uv_all_scalar_kernel<<<grid_for(N - done), 256, 0, s>>>(
        (uint32_t)done, (uint32_t)(N - done), nodes.charge, nodes.voltage, nodes.capacitance,
        nodes.leakage);
    CKT_CHECK_LAUNCH();
  }
  return CKT_OK;
}

int ckt_calc_new_currents_sync(const ckt_piece *piece, ckt_wires wires, ckt_nodes pvt,
                               ckt_nodes shr, ckt_nodes ghost, const ckt_params *prm,
                               void *stream) {
  const int rc = ckt_calc_new_currents(piece, wires, pvt, shr, ghost, prm, stream);
  return rc ? rc : wait_stream(stream, "calc_new_currents");
}

int ckt_distribute_charge_sync(const ckt_graph *graph, int32_t piece_index, ckt_wires wires,
                               ckt_nodes pvt, float *shr_fold, float *ghost_fold,
                               const ckt_params *prm, void *stream) {
  const int rc =
      ckt_distribute_charge(graph, piece_index, wires, pvt, shr_fold, ghost_fold, prm, stream);
  return rc ? rc : wait_stream(stream, "distribute_charge");
}

int ckt_update_voltages_sync(const ckt_piece *piece, ckt_nodes pvt, ckt_nodes shr,
                             const int32_t *locator, void *stream) {
  const int rc = ckt_update_voltages(piece, pvt, shr, locator, stream);
  return rc ? rc : wait_stream(stream, "update_voltages");
}

int ckt_distribute_update_all(const ckt_graph *graph, ckt_wires wires, ckt_nodes nodes,
                              const ckt_params *prm, void *stream) {
  int rc;
  CKT_REQUIRE(graph != nullptr, "graph is NULL");
  if ((rc = validate_params(prm)) || (rc = validate_nodes(nodes, "nodes"))) return rc;
  if ((rc = check_tile_error(graph))) return rc;
  if (graph->N == 0) return CKT_OK;
  if (graph->W == 0) return ckt_update_voltages_all(graph, nodes, stream);
  if ((rc = validate_wires(wires)) || (rc = check_graph_wires(graph, wires))) return rc;
  if (tile_plan_usable(graph, wires))
    return launch_dc_tile<true>(graph, wires, nodes, prm->dt, as_stream(stream));
  const float *I0 = wires.current, *I9 = wires.current + 9 * wires.seg_stride;
  dcuv_kernel<<<grid_for(graph->N, kDcBlock), kDcBlock, 0, as_stream(stream)>>>(
      (uint32_t)graph->N, graph->node_off, graph->node_ent, I0, I9, nodes.charge, nodes.voltage,
      nodes.capacitance, nodes.leakage, prm->dt);
  CKT_CHECK_LAUNCH();
  return CKT_OK;
}

int ckt_run_loops_all(const ckt_graph *graph, ckt_wires wires, ckt_nodes nodes,
                      const ckt_params *prm, int32_t loops, void *stream) {
  NvtxRange range("ckt_run_loops_all");
  int rc;
  CKT_REQUIRE(graph != nullptr, "graph is NULL");
  if ((rc = validate_params(prm)) || (rc = validate_nodes(nodes, "nodes"))) return rc;
  CKT_REQUIRE(loops >= 0, "loops must be >= 0 (got %d)", loops);
  if ((rc = check_tile_error(graph))) return rc;
  for (int32_t l = 0; l < loops; l++) {
    if ((rc = ckt_calc_new_currents_all(graph, wires, nodes, prm, stream)) ||
        (rc = ckt_distribute_update_all(graph, wires, nodes, prm, stream)))
      return rc;
  }
  return CKT_OK;
}

int ckt_distribute_charge_all_sync(const ckt_graph *graph, ckt_wires wires, ckt_nodes nodes,
                                   const ckt_params *prm, void *stream) {
  const int rc = ckt_distribute_charge_all(graph, wires, nodes, prm, stream);
  return rc ? rc : ckt_graph_check(graph, stream);
}

int ckt_distribute_update_all_sync(const ckt_graph *graph, ckt_wires wires, ckt_nodes nodes,
                                   const ckt_params *prm, void *stream) {
  const int rc = ckt_distribute_update_all(graph, wires, nodes, prm, stream);
  return rc ? rc : ckt_graph_check(graph, stream);
}

int ckt_run_loops_all_sync(const ckt_graph *graph, ckt_wires wires, ckt_nodes nodes,
                           const ckt_params *prm, int32_t loops, void *stream) {
  const int rc = ckt_run_loops_all(graph, wires, nodes, prm, loops, stream);
  return rc ? rc : ckt_graph_check(graph, stream);
}

int ckt_sanity_check_wires(const ckt_piece *piece, ckt_wires wires, uint32_t num_nodes_total,
                           int64_t *first_bad, void *stream) {
  CKT_REQUIRE(piece != nullptr, "piece is NULL");
  CKT_REQUIRE(wires.in_ptr && wires.out_ptr && wires.in_loc && wires.out_loc,
              "wire pointer/location arrays are NULL");
  if (first_bad) *first_bad = -1;
  if (piece->num_wires == 0) return CKT_OK;
  const cudaStream_t s = as_stream(stream);
  unsigned long long *d_bad = nullptr;
  CKT_CUDA(cudaMallocAsync(&d_bad, sizeof(unsigned long long), s));
  const unsigned long long none = ULLONG_MAX;
  unsigned long long h_bad = none;
  int rc = CKT_OK;
  cudaError_t e = cudaMemcpyAsync(d_bad, &none, sizeof(none), cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess) {
    sanity_kernel<<<grid_for(piece->num_wires), 256, 0, s>>>(*piece, wires.in_ptr, wires.out_ptr,
                                                              wires.in_loc, wires.out_loc,
                                                              num_nodes_total, d_bad);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaMemcpyAsync(&h_bad, d_bad, sizeof(h_bad), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  cudaFreeAsync(d_bad, s);
  if (e != cudaSuccess) return set_error(CKT_ECUDA, "sanity check failed: %s", cudaGetErrorString(e));
  if (h_bad != none) {
    if (first_bad) *first_bad = (int64_t)h_bad;
    rc = set_error(CKT_EBOUNDS, "wire %llu fails the pointer/location checks", h_bad);
  }
  return rc;
}

}  // extern "C"
