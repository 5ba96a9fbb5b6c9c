// ckt_graph.cpp -- builds the static contribution graph of a circuit on the
// host and uploads it.
//
// The graph fixes the order in which distribute_charge's contributions are
// summed so that the GPU reproduces one legal schedule of the reference's
// reduction bit for bit:
//   * private nodes (apps/circuit/circuit.cc:184-196: READ_WRITE, EXCLUSIVE)
//     receive their contributions in place, in wire order (reduce() on a
//     normal instance is apply<true>, runtime/lowlevel.h:484-489);
//   * shared and ghost nodes (REDUCE, SIMULTANEOUS) receive, per piece, the
//     fold of that piece's contributions in wire order starting from the
//     identity 0.0f (runtime/lowlevel.h:478-483, circuit.cc:30); the runtime
//     then applies each piece's fold instance to the node
//     (runtime/lowlevel_dma.cc:323-355); pieces are applied in ascending
//     order here.
#include <algorithm>
#include <cstring>
#include <thread>
#include <utility>

#include "ckt_internal.h"

namespace ckt {

template <typename T>
static int upload(T **dst, const std::vector<T> &src, int64_t *bytes) {
  const size_t n = std::max<size_t>(src.size(), 1);
  CKT_CUDA(cudaMalloc(reinterpret_cast<void **>(dst), n * sizeof(T)));
  *bytes += (int64_t)(n * sizeof(T));
  if (!src.empty())
    CKT_CUDA(cudaMemcpy(*dst, src.data(), src.size() * sizeof(T), cudaMemcpyHostToDevice));
  return CKT_OK;
}

static void free_graph(ckt_graph *g) {
  if (!g) return;
  cudaFree(g->node_off);
  cudaFree(g->node_ent);
  cudaFree(g->touch_node);
  cudaFree(g->touch_loc);
  cudaFree(g->touch_off);
  cudaFree(g->piece_ent);
  cudaFree(g->slot_in);
  cudaFree(g->slot_out);
  cudaFree(g->gstart);
  cudaFree(g->tile_step);
  cudaFree(g->tile_steps);
  cudaFree(g->tile_ent);
  cudaFree(g->tile_mask);
  cudaFree(g->ghost);
  cudaFree(g->ghost_list);
  cudaFree(g->ghost_block);
  if (g->ghost_done) cudaEventDestroy(g->ghost_done);
  if (g->tile_error_host) cudaFreeHost(const_cast<uint32_t *>(g->tile_error_host));
  delete g;
}

}  // namespace ckt

using namespace ckt;

namespace ckt {

int build_node_csr(const ckt_piece *pieces, int32_t num_pieces, uint32_t num_nodes,
                   const uint32_t *in_ptr, const uint32_t *out_ptr, const uint8_t *in_loc,
                   const uint8_t *out_loc, std::vector<uint32_t> &off, std::vector<uint32_t> &ent,
                   int64_t *num_wires, std::vector<uint32_t> *slots) {
  CKT_REQUIRE(num_pieces >= 1 && pieces != nullptr, "need at least one piece");
  // Pieces tile [0, W) in order; node ranges lie inside [0, N) and are disjoint.
  int64_t W = 0;
  std::vector<int32_t> node_owner(num_nodes, -1);
  for (int32_t k = 0; k < num_pieces; k++) {
    const ckt_piece &p = pieces[k];
    CKT_REQUIRE(p.first_wire == (uint64_t)W, "piece %d starts at wire %u, expected %lld", k,
                p.first_wire, (long long)W);
    W += p.num_wires;
    CKT_REQUIRE((uint64_t)p.first_node + p.num_nodes <= num_nodes,
                "piece %d node range [%u, %llu) exceeds %u nodes", k, p.first_node,
                (unsigned long long)p.first_node + p.num_nodes, num_nodes);
    for (uint32_t i = 0; i < p.num_nodes; i++) {
      CKT_REQUIRE(node_owner[p.first_node + i] < 0, "node %u belongs to pieces %d and %d",
                  p.first_node + i, node_owner[p.first_node + i], k);
      node_owner[p.first_node + i] = k;
    }
  }
  CKT_REQUIRE(W <= kMaxWires, "%lld wires exceed the limit %lld", (long long)W,
              (long long)kMaxWires);
  CKT_REQUIRE(W == 0 || (in_ptr && out_ptr && in_loc && out_loc), "wire arrays are NULL");
  const int64_t N = num_nodes;

  // Validate every endpoint (sanity_check_positions, circuit_gpu.cu:151-184)
  // and that no node is used both as private and as shared/ghost.
  std::vector<uint8_t> kind(N, 0);  // 0 unused, 1 private, 2 shared/ghost
  for (int32_t k = 0; k < num_pieces; k++) {
    const ckt_piece &p = pieces[k];
    for (int64_t w = p.first_wire; w < (int64_t)p.first_wire + p.num_wires; w++) {
      const uint32_t xs[2] = {in_ptr[w], out_ptr[w]};
      const uint8_t ls[2] = {in_loc[w], out_loc[w]};
      for (int e = 0; e < 2; e++) {
        const uint32_t x = xs[e];
        if ((int64_t)x >= N || ls[e] > CKT_GHOST_PTR)
          return set_error(CKT_EBOUNDS, "wire %lld: %s pointer %u / location %u out of range",
                           (long long)w, e ? "out" : "in", x, ls[e]);
        const bool inside = node_owner[x] == k;
        const bool ok = (e == 0) ? (inside && ls[e] != CKT_GHOST_PTR)
                                 : (inside ? ls[e] != CKT_GHOST_PTR : ls[e] == CKT_GHOST_PTR);
        if (!ok)
          return set_error(CKT_EBOUNDS, "wire %lld: %s pointer %u inconsistent with location %u",
                           (long long)w, e ? "out" : "in", x, ls[e]);
        const uint8_t kd = ls[e] == CKT_PRIVATE_PTR ? 1 : 2;
        if (kind[x] && kind[x] != kd)
          return set_error(CKT_EBOUNDS,
                           "wire %lld: node %u is referenced both as private and as shared",
                           (long long)w, x);
        kind[x] = kd;
      }
    }
  }

  // Whole-circuit CSR: counting sort of the 2W endpoints by node; filling in
  // wire order keeps (wire, end) order inside each node.
  off.assign(N + 1, 0);
  ent.assign(2 * W, 0);
  for (int64_t w = 0; w < W; w++) {
    off[in_ptr[w] + 1]++;
    off[out_ptr[w] + 1]++;
  }
  for (int64_t x = 0; x < N; x++) off[x + 1] += off[x];
  {
    std::vector<uint32_t> fill(off.begin(), off.end() - 1);
    std::vector<int32_t> last_piece(N, -1);
    if (slots) slots->assign(2 * W, 0);
    for (int32_t k = 0; k < num_pieces; k++) {
      const ckt_piece &p = pieces[k];
      for (int64_t w = p.first_wire; w < (int64_t)p.first_wire + p.num_wires; w++) {
        const uint32_t xs[2] = {in_ptr[w], out_ptr[w]};
        for (uint32_t e = 0; e < 2; e++) {
          const uint32_t x = xs[e];
          const uint32_t start = last_piece[x] != k ? 1u : 0u;
          last_piece[x] = k;
          if (slots) (*slots)[2 * w + e] = fill[x];
          ent[fill[x]++] = ((uint32_t)w << 2) | (e << 1) | start;
        }
      }
    }
  }
  for (int64_t x = 0; x < N; x++)
    if (kind[x] != 2) off[x] |= kPrivateBit;
  if (num_wires) *num_wires = W;
  return CKT_OK;
}

// Tiled distribute_charge plan of one node tile (encoding in ckt_internal.h).
namespace {

struct TilePlan {
  std::vector<uint4> steps;  // entry and ghost-slot offsets local to the tile
  std::vector<uint32_t> ent;
  std::vector<uint32_t> gsrc;  // per ghost slot: wire << 1 | end, or kTePad
};

// A chunk with at least this many of the tile's contributions is copied
// whole (32 KB of I[0]/I[9]); the contributions of sparser chunks go
// through the ghost buffer (a list entry, a current read in wire order, a
// scattered store and a copy: about 20 bytes and one store request each).
constexpr uint32_t kDenseMin = kChunkWires / 8;

void plan_tile(const uint32_t *off, const uint32_t *ent, uint32_t x0, uint32_t xe,
               TilePlan &tp, std::vector<uint64_t> &keys, std::vector<uint64_t> &sparse) {
  // Key (chunk, node within tile, CSR position): sorted, each node's
  // contributions stay in CSR (= wire) order inside every chunk.
  const uint32_t lo = off[x0] & kOffsetMask;
  keys.clear();
  for (uint32_t x = x0; x < xe; x++) {
    const uint32_t b = off[x] & kOffsetMask, e = off[x + 1] & kOffsetMask;
    for (uint32_t i = b; i < e; i++)
      keys.push_back(((uint64_t)((ent[i] >> 2) / kChunkWires) << 45) |
                     ((uint64_t)(x - x0) << 32) | (i - lo));
  }
  std::sort(keys.begin(), keys.end());

  auto word = [&](uint64_t key, bool head) -> uint32_t {
    const uint32_t xl = (uint32_t)(key >> 32) & (kTileNodesMax - 1);
    const uint32_t i = lo + (uint32_t)key, x = x0 + xl;
    const uint32_t u = ent[i], w = u >> 2;
    const bool priv = (off[x] & kPrivateBit) != 0;
    const bool flush = !priv && (u & 1u) && i != (off[x] & kOffsetMask);
    return (w % kChunkWires) | ((u & 2u) ? kTeEnd : 0u) | (xl << kTeNodeShift) |
           (flush ? kTeFlush : 0u) | (head ? kTeHead : 0u) | (priv ? kTePriv : 0u);
  };
  // Emits [a, b) of `v` (sorted by node, then CSR position) as one step, or
  // as several when it holds more entries than a step's buffer (a node's
  // entries cut between two steps continue in the later one).  Inside a
  // step, a node's entries form one run, summed by one lane of the warp that
  // owns the node; each warp deals its runs, longest first, to whichever of
  // its 32 lanes has the fewest entries so far, so that its lanes finish
  // together.
  std::vector<std::pair<uint32_t, uint32_t>> runs;  // (length, first index)
  std::vector<uint32_t> order;
  std::vector<std::pair<uint32_t, uint32_t>> wruns[kTileWarps];
  std::vector<uint32_t> lane_runs[32];
  std::vector<uint32_t> gidx, gin, gout;
  auto emit = [&](const std::vector<uint64_t> &v, size_t a, size_t b, bool ghost,
                  uint32_t chunk) {
    runs.clear();
    for (size_t j = a; j < b;) {
      const uint64_t node = v[j] >> 32;
      size_t e = j + 1;
      while (e < b && (v[e] >> 32) == node) e++;
      runs.emplace_back((uint32_t)(e - j), (uint32_t)j);
      j = e;
    }
    std::stable_sort(runs.begin(), runs.end(),
                     [](const auto &x, const auto &y) { return x.first > y.first; });
    order.clear();
    for (const auto &r : runs)
      for (uint32_t j = r.second; j < r.second + r.first; j++) order.push_back(j);
    auto node_of = [&](uint32_t j) { return (uint32_t)(v[j] >> 32) & (kTileNodesMax - 1); };
    constexpr size_t kMax = kStepEntriesMax - 4;
    for (size_t c0 = 0; c0 < order.size(); c0 += kMax) {
      const size_t c1 = std::min(order.size(), c0 + kMax);
      // A ghost step's values: its in-ends' and out-ends' currents, each run
      // in wire order; an entry's index is its place in its end's run.
      uint32_t desc = chunk, g0 = 0;
      if (ghost) {
        gin.clear();
        gout.clear();
        for (size_t q = c0; q < c1; q++) {
          const uint32_t u = ent[lo + (uint32_t)v[order[q]]];
          ((u & 2u) ? gout : gin).push_back(u >> 2);
        }
        std::sort(gin.begin(), gin.end());
        std::sort(gout.begin(), gout.end());
        gidx.resize(c1 - c0);
        for (size_t q = c0; q < c1; q++) {
          const uint32_t u = ent[lo + (uint32_t)v[order[q]]];
          const auto &run = (u & 2u) ? gout : gin;
          gidx[q - c0] =
              (uint32_t)(std::lower_bound(run.begin(), run.end(), u >> 2) - run.begin());
        }
        g0 = (uint32_t)tp.gsrc.size();
        for (uint32_t e = 0; e < 2; e++) {
          const auto &run = e ? gout : gin;
          for (uint32_t w : run) tp.gsrc.push_back((w << 1) | e);
          while (tp.gsrc.size() % 4) tp.gsrc.push_back(kTePad);
        }
        desc = kGhostStep | ((uint32_t)gin.size() << kGhostCountBits) | (uint32_t)gout.size();
      }
      // The step's runs (pieces of `order` with one node), by owning warp.
      for (auto &wr : wruns) wr.clear();
      for (size_t q = c0; q < c1;) {
        size_t e = q + 1;
        while (e < c1 && node_of(order[e]) == node_of(order[q])) e++;
        wruns[node_of(order[q]) % kTileWarps].emplace_back((uint32_t)(e - q), (uint32_t)q);
        q = e;
      }
      const uint32_t b0 = (uint32_t)tp.ent.size();
      for (uint32_t h = 0; h < kStepHeaderWords; h++) tp.ent.push_back(0u);
      std::vector<uint16_t> hdr(2 * kStepHeaderWords, 0);
      uint32_t n = 0;
      for (uint32_t w = 0; w < kTileWarps; w++) {
        auto &wr = wruns[w];
        std::stable_sort(wr.begin(), wr.end(),
                         [](const auto &x, const auto &y) { return x.first > y.first; });
        uint32_t load[32] = {};
        for (auto &lr : lane_runs) lr.clear();
        for (uint32_t r = 0; r < (uint32_t)wr.size(); r++) {
          uint32_t best = 0;
          for (uint32_t L = 1; L < 32; L++)
            if (load[L] < load[best]) best = L;
          load[best] += wr[r].first;
          lane_runs[best].push_back(r);
        }
        for (uint32_t L = 0; L < 32; L++) {
          hdr[32 * w + L] = (uint16_t)n;
          for (uint32_t r : lane_runs[L])
            for (uint32_t k = 0; k < wr[r].first; k++) {
              const size_t q = wr[r].second + k;
              uint32_t wd = word(v[order[q]], k == 0);
              if (ghost) wd = (wd & ~(kChunkWires - 1)) | gidx[q - c0];
              tp.ent.push_back(wd);
              n++;
            }
        }
      }
      hdr[kTileLanes] = (uint16_t)n;
      for (uint32_t h = 0; h < kStepHeaderWords; h++)
        tp.ent[b0 + h] = (uint32_t)hdr[2 * h] | ((uint32_t)hdr[2 * h + 1] << 16);
      while ((tp.ent.size() - b0) % 4) tp.ent.push_back(kTePad);  // 16-byte blocks for the bulk copies
      tp.steps.push_back(make_uint4(b0, (uint32_t)tp.ent.size() - b0, desc, g0));
    }
  };
  auto flush_sparse = [&]() {
    if (sparse.empty()) return;
    // One wire range: order by (node, CSR position) only.
    for (uint64_t &k : sparse) k &= (1ull << 45) - 1;
    std::sort(sparse.begin(), sparse.end());
    emit(sparse, 0, sparse.size(), true, 0u);
    sparse.clear();
  };
  sparse.clear();
  for (size_t a = 0; a < keys.size();) {
    const uint64_t chunk = keys[a] >> 45;
    size_t b = a;
    while (b < keys.size() && (keys[b] >> 45) == chunk) b++;
    if (b - a >= kDenseMin) {
      flush_sparse();
      emit(keys, a, b, false, (uint32_t)chunk);
    } else {
      sparse.insert(sparse.end(), keys.begin() + a, keys.begin() + b);
    }
    a = b;
  }
  flush_sparse();
}

}  // namespace

// The whole-circuit tiled distribute_charge plan, on the host.
struct HostTilePlan {
  uint32_t T = 0;                   // tiles
  std::vector<uint32_t> tile_step;  // [T + 1]
  std::vector<uint4> steps;
  std::vector<uint32_t> ent;
  std::vector<uint2> glist;         // packing list {slot, wire << 1 | end}
  std::vector<uint32_t> gblock;     // [nblocks + 1]
  std::vector<uint32_t> mask;       // [T * kTileNodesMax / 32]
  int64_t gslots = 0;
  uint32_t nblocks = 0;
  bool staged = false;
};

// Plans every tile (in parallel), concatenates the tiles' steps, entries and
// ghost runs, and builds the packing list and the per-tile fold masks.
static int make_tile_plan(uint32_t N, int64_t W, const std::vector<uint32_t> &off,
                          const std::vector<uint32_t> &ent, uint32_t tile_nodes,
                          HostTilePlan &hp) {
  const uint32_t T = (N + tile_nodes - 1) / tile_nodes;
  std::vector<TilePlan> plans(T);
  const int nthr = (int)std::max(1u, std::min(std::thread::hardware_concurrency(), 64u));
  std::vector<std::thread> pool;
  for (int r = 0; r < nthr; r++)
    pool.emplace_back([&, r]() {
      std::vector<uint64_t> keys, sparse;
      for (uint32_t t = (uint32_t)r; t < T; t += (uint32_t)nthr)
        plan_tile(off.data(), ent.data(), t * tile_nodes, std::min(N, (t + 1) * tile_nodes),
                  plans[t], keys, sparse);
    });
  for (auto &th : pool) th.join();
  hp.T = T;
  hp.tile_step.assign(T + 1, 0);
  hp.steps.clear();
  hp.ent.clear();
  hp.glist.clear();
  hp.gslots = 0;
  for (uint32_t t = 0; t < T; t++) {
    hp.tile_step[t] = (uint32_t)hp.steps.size();
    const uint32_t eb = (uint32_t)hp.ent.size(), gb = (uint32_t)hp.gslots;
    for (uint4 s : plans[t].steps) hp.steps.push_back(make_uint4(s.x + eb, s.y, s.z, s.w + gb));
    hp.ent.insert(hp.ent.end(), plans[t].ent.begin(), plans[t].ent.end());
    for (size_t k = 0; k < plans[t].gsrc.size(); k++)
      if (plans[t].gsrc[k] != kTePad)
        hp.glist.push_back(make_uint2(gb + (uint32_t)k, plans[t].gsrc[k]));
    hp.gslots += (int64_t)plans[t].gsrc.size();
    if (hp.ent.size() > 0xffffffffull || hp.gslots > 0x7fffffffll)
      return set_error(CKT_EINVAL, "tiled plan too large for 32-bit offsets");
    std::vector<uint4>().swap(plans[t].steps);
    std::vector<uint32_t>().swap(plans[t].ent);
    std::vector<uint32_t>().swap(plans[t].gsrc);
  }
  hp.tile_step[T] = (uint32_t)hp.steps.size();
  // Packing order: by source block of kPackWires wires, then by slot, so
  // that a block's stores into one step's run are consecutive.
  std::sort(hp.glist.begin(), hp.glist.end(), [](const uint2 &x, const uint2 &y) {
    const uint32_t bx = (x.y >> 1) / kPackWires, by = (y.y >> 1) / kPackWires;
    return bx != by ? bx < by : x.x < y.x;
  });
  hp.nblocks = (uint32_t)((W + kPackWires - 1) / kPackWires);
  if (hp.glist.size() > kPackFirstMask)
    return set_error(CKT_EINVAL, "too many ghost contributions for the packing list");
  hp.gblock.assign(hp.nblocks + 1, 0u);
  for (size_t k = hp.glist.size(); k-- > 0;) {
    const uint32_t b = (hp.glist[k].y >> 1) / kPackWires;
    hp.gblock[b] = (hp.gblock[b] & ~kPackFirstMask) | (uint32_t)k |
                   ((hp.glist[k].y & 1u) ? kPackHasOut : kPackHasIn);
  }
  hp.gblock[hp.nblocks] = (uint32_t)hp.glist.size();
  for (uint32_t b = hp.nblocks; b-- > 0;)  // blocks without entries start where the next one does
    if ((hp.gblock[b] & (kPackHasIn | kPackHasOut)) == 0u)
      hp.gblock[b] = hp.gblock[b + 1] & kPackFirstMask;
  // Staged packing once the ghost ends average kPackWires / 8 per source
  // block: below that, reading whole slices costs more than the scattered
  // stores it saves.
  hp.staged = (int64_t)hp.glist.size() * 8 >= (int64_t)hp.nblocks * kPackWires;
  // Per tile, the nodes whose folds are added when the tile finishes: not
  // private and touched by at least one wire.
  hp.mask.assign((size_t)T * (kTileNodesMax / 32), 0u);
  for (uint32_t x = 0; x < N; x++)
    if (!(off[x] & kPrivateBit) && (off[x + 1] & kOffsetMask) > (off[x] & kOffsetMask)) {
      const uint32_t t = x / tile_nodes, i = x % tile_nodes;
      hp.mask[(size_t)t * (kTileNodesMax / 32) + i / 32] |= 1u << (i % 32);
    }
  return CKT_OK;
}

// Builds and uploads the tiled distribute_charge plan.
static int build_tile_plan(ckt_graph *g, const std::vector<uint32_t> &off,
                           const std::vector<uint32_t> &ent, uint32_t tile_nodes) {
  // Tile bases and node counts stay 32-bit in the kernel.
  if (g->N > 0x7fffffff || g->W == 0) return CKT_OK;
  HostTilePlan hp;
  int rc;
  if ((rc = make_tile_plan((uint32_t)g->N, g->W, off, ent, tile_nodes, hp))) return rc;
  if ((rc = upload(&g->tile_step, hp.tile_step, &g->device_bytes)) ||
      (rc = upload(&g->tile_steps, hp.steps, &g->device_bytes)) ||
      (rc = upload(&g->tile_ent, hp.ent, &g->device_bytes)) ||
      (rc = upload(&g->tile_mask, hp.mask, &g->device_bytes)) ||
      (rc = upload(&g->ghost_list, hp.glist, &g->device_bytes)) ||
      (rc = upload(&g->ghost_block, hp.gblock, &g->device_bytes)))
    return rc;
  g->ghost_blocks = hp.nblocks;
  g->ghost_staged = hp.staged;
  CKT_CUDA(cudaMalloc(reinterpret_cast<void **>(&g->ghost),
                      (size_t)std::max<int64_t>(hp.gslots, 4) * sizeof(float)));
  g->device_bytes += std::max<int64_t>(hp.gslots, 4) * (int64_t)sizeof(float);
  g->ghost_slots = hp.gslots;
  g->ghost_n = (int64_t)hp.glist.size();
  CKT_CUDA(cudaEventCreateWithFlags(&g->ghost_done, cudaEventDisableTiming));
  void *word = nullptr;
  CKT_CUDA(cudaHostAlloc(&word, sizeof(uint32_t), cudaHostAllocMapped));
  g->tile_error_host = static_cast<volatile uint32_t *>(word);
  *g->tile_error_host = 0u;
  CKT_CUDA(cudaHostGetDevicePointer(reinterpret_cast<void **>(&g->tile_error), word, 0));
  g->tile_nodes = tile_nodes;
  g->num_tiles = hp.T;
  g->tile_num_steps = (int64_t)hp.steps.size();
  g->tile_stream_steps = 0;
  for (const uint4 &s : hp.steps) g->tile_stream_steps += (s.z & kGhostStep) == 0u;
  return CKT_OK;
}

}  // namespace ckt

extern "C" {

int ckt_graph_create(const ckt_piece *pieces, int32_t num_pieces, uint32_t num_nodes,
                     const uint32_t *in_ptr, const uint32_t *out_ptr, const uint8_t *in_loc,
                     const uint8_t *out_loc, ckt_graph **out) {
  CKT_REQUIRE(out != nullptr, "out is NULL");
  *out = nullptr;
  std::vector<uint32_t> off, ent, slots;
  int64_t W = 0;
  int rc = build_node_csr(pieces, num_pieces, num_nodes, in_ptr, out_ptr, in_loc, out_loc, off,
                          ent, &W, &slots);
  if (rc) return rc;
  std::vector<uint32_t> slot_in(W), slot_out(W), gstart((2 * W + 31) / 32, 0u);
  for (int64_t w = 0; w < W; w++) {
    slot_in[w] = slots[2 * w];
    slot_out[w] = slots[2 * w + 1];
  }
  for (int64_t i = 0; i < 2 * W; i++)
    if (ent[i] & 1u) gstart[i >> 5] |= 1u << (i & 31);

  ckt_graph *g = new ckt_graph();
  g->W = W;
  g->N = num_nodes;
  g->P = num_pieces;
  g->pieces.assign(pieces, pieces + num_pieces);

  // Per-piece CSR over touched nodes, nodes ascending, wire order inside.
  std::vector<uint32_t> touch_node, touch_off, pent;
  std::vector<uint8_t> touch_loc;
  g->touch_first.assign(num_pieces + 1, 0);
  pent.reserve(2 * W);
  std::vector<uint64_t> keys;
  for (int32_t k = 0; k < num_pieces; k++) {
    const ckt_piece &p = pieces[k];
    g->touch_first[k] = (int64_t)touch_node.size();
    keys.clear();
    for (uint32_t i = 0; i < p.num_wires; i++) {
      const int64_t w = (int64_t)p.first_wire + i;
      keys.push_back(((uint64_t)in_ptr[w] << 32) | (2u * i));
      keys.push_back(((uint64_t)out_ptr[w] << 32) | (2u * i + 1));
    }
    std::sort(keys.begin(), keys.end());
    for (size_t j = 0; j < keys.size(); j++) {
      const uint32_t x = (uint32_t)(keys[j] >> 32);
      const uint32_t local = (uint32_t)keys[j];
      const uint32_t w = p.first_wire + (local >> 1), e = local & 1u;
      if (j == 0 || (uint32_t)(keys[j - 1] >> 32) != x) {
        touch_node.push_back(x);
        touch_loc.push_back(e ? out_loc[w] : in_loc[w]);
        touch_off.push_back((uint32_t)pent.size());
      }
      pent.push_back((w << 1) | e);
    }
  }
  g->touch_first[num_pieces] = (int64_t)touch_node.size();
  touch_off.push_back((uint32_t)pent.size());

  if ((rc = upload(&g->node_off, off, &g->device_bytes)) ||
      (rc = upload(&g->node_ent, ent, &g->device_bytes)) ||
      (rc = upload(&g->touch_node, touch_node, &g->device_bytes)) ||
      (rc = upload(&g->touch_loc, touch_loc, &g->device_bytes)) ||
      (rc = upload(&g->touch_off, touch_off, &g->device_bytes)) ||
      (rc = upload(&g->piece_ent, pent, &g->device_bytes)) ||
      (rc = upload(&g->slot_in, slot_in, &g->device_bytes)) ||
      (rc = upload(&g->slot_out, slot_out, &g->device_bytes)) ||
      (rc = upload(&g->gstart, gstart, &g->device_bytes)) ||
      (rc = build_tile_plan(g, off, ent, kTileNodesMax))) {
    free_graph(g);
    return rc;
  }
  *out = g;
  return CKT_OK;
}

int ckt_graph_destroy(ckt_graph *graph) {
  free_graph(graph);
  return CKT_OK;
}

int ckt_graph_export(const ckt_graph *g, uint32_t *off, uint32_t *ent, uint32_t *slot_in,
                     uint32_t *slot_out, uint32_t *gstart) {
  CKT_REQUIRE(g != nullptr, "graph is NULL");
  const int64_t W = g->W, N = g->N;
  if (off) CKT_CUDA(cudaMemcpy(off, g->node_off, (N + 1) * 4, cudaMemcpyDeviceToHost));
  if (W > 0) {
    if (ent) CKT_CUDA(cudaMemcpy(ent, g->node_ent, 2 * W * 4, cudaMemcpyDeviceToHost));
    if (slot_in) CKT_CUDA(cudaMemcpy(slot_in, g->slot_in, W * 4, cudaMemcpyDeviceToHost));
    if (slot_out) CKT_CUDA(cudaMemcpy(slot_out, g->slot_out, W * 4, cudaMemcpyDeviceToHost));
    if (gstart)
      CKT_CUDA(cudaMemcpy(gstart, g->gstart, ((2 * W + 31) / 32) * 4, cudaMemcpyDeviceToHost));
  }
  return CKT_OK;
}

int ckt_graph_info(const ckt_graph *g, int64_t *num_wires, int64_t *num_nodes,
                   int32_t *num_pieces, int64_t *device_bytes) {
  CKT_REQUIRE(g != nullptr, "graph is NULL");
  if (num_wires) *num_wires = g->W;
  if (num_nodes) *num_nodes = g->N;
  if (num_pieces) *num_pieces = g->P;
  if (device_bytes) *device_bytes = g->device_bytes;
  return CKT_OK;
}

int ckt_graph_tile_info(const ckt_graph *g, int32_t *tiles, int64_t *steps,
                        int64_t *stream_steps, uint32_t *error_word) {
  CKT_REQUIRE(g != nullptr, "graph is NULL");
  if (tiles) *tiles = (int32_t)g->num_tiles;
  if (steps) *steps = g->tile_num_steps;
  if (stream_steps) *stream_steps = g->tile_stream_steps;
  if (error_word) {
    *error_word = 0;
    if (g->tile_error_host) {
      // every stream's passes first: the word is then final
      CKT_CUDA(cudaDeviceSynchronize());
      *error_word = *g->tile_error_host;
      *g->tile_error_host = 0u;
    }
  }
  return CKT_OK;
}

int ckt_graph_check(const ckt_graph *g, void *stream) {
  CKT_REQUIRE(g != nullptr, "graph is NULL");
  const cudaError_t e = cudaStreamSynchronize(as_stream(stream));
  if (e != cudaSuccess)
    return set_error(CKT_ECUDA, "waiting for the graph's passes failed: %s", cudaGetErrorString(e));
  if (g->tile_error_host && *g->tile_error_host) {
    *g->tile_error_host = 0u;
    return set_error(CKT_ETIMEOUT,
                     "a tiled node pass's copy wait ran out (bound %llu ns): a tile's charges "
                     "and voltages were left unwritten",
                     (unsigned long long)g->tile_timeout_ns);
  }
  return CKT_OK;
}

int ckt_graph_set_tile_timeout(ckt_graph *g, uint64_t timeout_ns) {
  CKT_REQUIRE(g != nullptr, "graph is NULL");
  g->tile_timeout_ns = timeout_ns ? timeout_ns : 2000000000ull;
  return CKT_OK;
}

}  // extern "C"
