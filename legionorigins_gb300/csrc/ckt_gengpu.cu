// ckt_gengpu.cu -- the circuit generator on the device: the same random
// stream, graph and initial values as ckt_generate (load_circuit,
// apps/circuit/circuit.cc:1071-1288), bit for bit, plus the contribution
// graph of the index-space distribute_charge.
//
// drand48 is a 48-bit linear congruential generator, so the state after d
// draws is A_d*x + C_d (mod 2^48) and any position of the stream can be
// reached in log2(d) steps.  Nodes draw 3 values each; a wire draws 6 values
// (in-piece) or 7 (cross-piece), and which one depends on its own 5th draw,
// so wire start positions are a chain through the stream.  The chain is
// decoded in parallel by speculation: the stream is cut into chunks of
// kChunk draws, each chunk is decoded from all 7 possible entry phases (a
// wire starts at most 6 draws past a chunk boundary), the chunks' phase maps
// are composed to fix every chunk's true entry phase and first wire index,
// and every chunk then emits its wires.  Node pointers, locations and the
// graph follow in data-parallel kernels; per-node contribution lists are
// sorted by (wire, end) so the graph is identical to the host-built one.
#include <algorithm>
#include <mutex>
#include <vector>

#include "ckt_drand.cuh"
#include "ckt_internal.h"

namespace ckt {
namespace {

constexpr uint64_t kA = 0x5DEECE66Dull, kC = 0xBull, kMask = 0xffffffffffffull;
constexpr int kChunk = 256;       // draws per chunk
constexpr int kMapBlock = 256;    // chunks per block of the map composition
constexpr int kTopTile = 1024;    // blocks per shared-memory tile of the top-level walk

struct Jump {
  uint64_t a[48], c[48];  // state after 2^i draws: a[i]*x + c[i]
};

__constant__ Jump g_jump;

Jump make_jump() {
  Jump j;
  uint64_t a = kA, c = kC;
  for (int i = 0; i < 48; i++) {
    j.a[i] = a;
    j.c[i] = c;
    // (a, c) composed with itself: x -> a(ax + c) + c
    c = (a * c + c) & kMask;
    a = (a * a) & kMask;
  }
  return j;
}

// State after k draws, k < kChunk: a[k]*x + c[k], for jumps from a chunk's
// start to a wire inside it (lanes index it independently, so it lives in
// global memory, not the constant bank).
__device__ uint64_t g_near_a[kChunk], g_near_c[kChunk];

// The jump tables never change: they are copied to each device once.  (A
// per-call copy from pageable memory would wait for the stream's earlier
// work.)
constexpr int kMaxDevices = 64;

int ensure_jump_table() {
  static std::mutex mu;
  static bool loaded[kMaxDevices] = {};
  int dev = 0;
  CKT_CUDA(cudaGetDevice(&dev));
  CKT_REQUIRE(dev >= 0 && dev < kMaxDevices, "device %d out of range", dev);
  std::lock_guard<std::mutex> lk(mu);
  if (!loaded[dev]) {
    const Jump jump = make_jump();
    CKT_CUDA(cudaMemcpyToSymbol(g_jump, &jump, sizeof(Jump)));
    std::vector<uint64_t> na(kChunk), nc(kChunk);
    uint64_t a = 1, c = 0;
    for (int k = 0; k < kChunk; k++) {
      na[k] = a;
      nc[k] = c;
      c = (kA * c + kC) & kMask;  // one more draw: x -> A x + C
      a = (kA * a) & kMask;
    }
    CKT_CUDA(cudaMemcpyToSymbol(g_near_a, na.data(), kChunk * sizeof(uint64_t)));
    CKT_CUDA(cudaMemcpyToSymbol(g_near_c, nc.data(), kChunk * sizeof(uint64_t)));
    loaded[dev] = true;
  }
  return CKT_OK;
}

__device__ __forceinline__ uint64_t skip(uint64_t x, uint64_t d) {
  for (int i = 0; d; i++, d >>= 1)
    if (d & 1) x = (g_jump.a[i] * x + g_jump.c[i]) & kMask;
  return x;
}

// Advances the generator state by one draw and returns it (the draw's value
// is x * 2^-48; the drand helpers evaluate the expressions on x).
__device__ __forceinline__ uint64_t next(uint64_t &x) {
  x = (kA * x + kC) & kMask;
  return x;
}

// random_element of the piece's node set (its reversed order, see
// ckt_gen.cpp): first + npp - 1 - (int)(drand48() * npp).
__device__ __forceinline__ uint32_t pick(uint64_t x, uint32_t piece, uint32_t npp) {
  return piece * npp + npp - 1 - drand::trunc_mul(x, npp);
}

struct GenArgs {
  int32_t P, npp, wpp;
  double L_off, L_scale;
  uint64_t pct_thr;  // drand::pct_threshold(pct)
  uint64_t seed_state;
  int64_t W, N;
};

// The wire leaves its piece: !(100 * drand48() < pct) with more than one piece.
__device__ __forceinline__ bool crosses(const GenArgs &g, uint64_t x5) {
  return g.P > 1 && !drand::pct_below(x5, g.pct_thr);
}

// Node values: draws 3x, 3x+1, 3x+2 (circuit.cc:1121-1125).
__global__ void gen_nodes_kernel(GenArgs g, float *charge, float *nvolt, float *cap, float *leak,
                                 int32_t *locator) {
  const int64_t x0 = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) * 16;
  if (x0 >= g.N) return;
  uint64_t x = skip(g.seed_state, 3 * (uint64_t)x0);
  const int64_t x1 = min(g.N, x0 + 16);
  for (int64_t n = x0; n < x1; n++) {
    charge[n] = 0.f;
    nvolt[n] = drand::node_voltage(next(x));
    cap[n] = drand::node_capacitance(next(x));
    leak[n] = __double2float_rn(__dmul_rn((double)0.1f, drand::value(next(x))));
    locator[n] = 1;
  }
}

// Per chunk and entry phase q: where the chain leaves the chunk (0..6 past
// its end) and how many wires start inside it.  Only a wire's 5th draw (the
// in-piece test) matters here, so the state advances for every draw and is
// converted to a double only where some phase needs that test.
constexpr int kChunkWords = (kChunk + 4 + 31) / 32;  // in-piece test bits of a chunk's draws
constexpr int kMapsBlock = 128;

__global__ void __launch_bounds__(kMapsBlock)
    chunk_maps_kernel(GenArgs g, int64_t base, int64_t nchunks, uint8_t *exit_phase,
                      uint32_t *count) {
  __shared__ uint32_t sbits[kChunkWords][kMapsBlock];
  const int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= nchunks) return;
  // 1. the cross-piece test of every draw of the chunk, as bits (the same
  //    work on every lane)
  uint64_t x = skip(g.seed_state, (uint64_t)(base + c * kChunk));
#pragma unroll
  for (int wd = 0; wd < kChunkWords; wd++) {
    uint32_t bits = 0;
    for (int k = 0; k < 32; k++) bits |= (crosses(g, next(x)) ? 1u : 0u) << k;
    sbits[wd][threadIdx.x] = bits;
  }
  // 2. each entry phase hops wire to wire: 6 draws, or 7 when the wire's
  //    5th draw says it leaves its piece
#pragma unroll
  for (int q = 0; q < 7; q++) {
    uint32_t s = (uint32_t)q, n = 0;
    while (s < (uint32_t)kChunk) {
      const uint32_t t = s + 4;
      s += 6u + ((sbits[t >> 5][threadIdx.x] >> (t & 31u)) & 1u);
      n++;
    }
    exit_phase[c * 7 + q] = (uint8_t)(s - (uint32_t)kChunk);
    count[c * 7 + q] = n;
  }
}

// The chunk maps of kMapBlock consecutive chunks composed in shared memory:
// for every phase q the block might be entered with, each chunk's entry
// phase and the wires before it inside the block, and the block's own map.
__global__ void __launch_bounds__(128)
    map_block_kernel(int64_t nchunks, const uint8_t *__restrict__ exit_phase,
                     const uint32_t *__restrict__ count, uint8_t *rel_phase, uint32_t *rel_base,
                     uint8_t *bexit, uint32_t *bcount) {
  __shared__ uint8_t se[kMapBlock * 7];
  __shared__ uint32_t sc[kMapBlock * 7];
  const int64_t c0 = (int64_t)blockIdx.x * kMapBlock;
  const int n = (int)min((int64_t)kMapBlock, nchunks - c0);
  for (int i = threadIdx.x; i < n * 7; i += blockDim.x) {
    se[i] = exit_phase[c0 * 7 + i];
    sc[i] = count[c0 * 7 + i];
  }
  __syncthreads();
  if (threadIdx.x < 7) {
    const int q = threadIdx.x;
    int ph = q;
    uint32_t tot = 0;
    for (int k = 0; k < n; k++) {
      rel_phase[(c0 + k) * 7 + q] = (uint8_t)ph;
      rel_base[(c0 + k) * 7 + q] = tot;
      tot += sc[k * 7 + ph];
      ph = se[k * 7 + ph];
    }
    bexit[blockIdx.x * 7 + q] = (uint8_t)ph;
    bcount[blockIdx.x * 7 + q] = tot;
  }
}

// The chain through the blocks from phase 0 (the first wire starts at the
// first wire draw): every block's entry phase and first wire.  One block;
// the maps pass through shared memory a tile at a time, so the walk's
// dependent steps are shared-memory reads.
__global__ void __launch_bounds__(256)
    map_top_kernel(int64_t nblocks, const uint8_t *__restrict__ bexit,
                   const uint32_t *__restrict__ bcount, uint8_t *bphase, uint64_t *bbase) {
  __shared__ uint8_t se[kTopTile * 7];
  __shared__ uint32_t sc[kTopTile * 7];
  int ph = 0;
  uint64_t tot = 0;
  for (int64_t b0 = 0; b0 < nblocks; b0 += kTopTile) {
    const int n = (int)min((int64_t)kTopTile, nblocks - b0);
    __syncthreads();
    for (int i = threadIdx.x; i < n * 7; i += blockDim.x) {
      se[i] = bexit[b0 * 7 + i];
      sc[i] = bcount[b0 * 7 + i];
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      for (int k = 0; k < n; k++) {
        bphase[b0 + k] = (uint8_t)ph;
        bbase[b0 + k] = tot;
        tot += sc[k * 7 + ph];
        ph = se[k * 7 + ph];
      }
    }
  }
}

// Every chunk walks its wires from its entry phase and records where each
// starts in the draw stream (relative to the first wire draw).
__global__ void wire_starts_kernel(GenArgs g, int64_t base, int64_t nchunks,
                                   const uint8_t *__restrict__ rel_phase,
                                   const uint32_t *__restrict__ rel_base,
                                   const uint8_t *__restrict__ bphase,
                                   const uint64_t *__restrict__ bbase, uint32_t *starts,
                                   uint64_t *chunk_state) {
  const int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= nchunks) return;
  const int64_t b = c / kMapBlock;
  const int qb = bphase[b];  // the block's entry phase selects the chunk's entry
  int64_t w = (int64_t)bbase[b] + rel_base[c * 7 + qb];
  if (w >= g.W) return;
  const int64_t p0 = base + c * kChunk;
  uint32_t sr = rel_phase[c * 7 + qb];  // relative to p0
  uint64_t x = skip(g.seed_state, (uint64_t)p0);
  chunk_state[c] = x;
  uint32_t t = 0;
  while (sr < (uint32_t)kChunk && w < g.W) {
    starts[w] = (uint32_t)(c * kChunk + sr);
    while (t <= sr + 4) {  // advance to the wire's in-piece draw
      next(x);
      t++;
    }
    sr += crosses(g, x) ? 7u : 6u;
    w++;
  }
}

// One thread per wire (circuit.cc:1158-1186): jump to its first draw, draw
// R, L, C, the in-node, the in-piece test and the out-node, and store every
// field coalesced.
__global__ void gen_wires_kernel(GenArgs g, const uint32_t *__restrict__ starts,
                                 const uint64_t *__restrict__ chunk_state, uint32_t *in_ptr,
                                 uint32_t *out_ptr, float *L, float *R, float *C,
                                 int32_t *locator) {
  const int64_t w = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (w >= g.W) return;
  const uint32_t st = starts[w], k = st % (uint32_t)kChunk;
  uint64_t x = (__ldg(g_near_a + k) * chunk_state[st / (uint32_t)kChunk] + __ldg(g_near_c + k)) &
               kMask;
  const uint64_t xR = next(x), xL = next(x), xC = next(x), xIn = next(x), xPct = next(x);
  const uint32_t n = (uint32_t)(w / g.wpp);
  R[w] = drand::resistance(xR);
  L[w] = __double2float_rn(__dadd_rn(__dmul_rn(drand::value(xL), g.L_scale), g.L_off));
  C[w] = __double2float_rn(__dmul_rn(drand::value(xC), 0.1));
  in_ptr[w] = pick(xIn, n, (uint32_t)g.npp);
  if (!crosses(g, xPct)) {
    out_ptr[w] = pick(next(x), n, (uint32_t)g.npp);
  } else {
    int nn = (int)drand::trunc_mul(next(x), (uint32_t)(g.P - 1));
    if (nn >= (int)n) nn++;
    const uint32_t o = pick(next(x), (uint32_t)nn, (uint32_t)g.npp);
    out_ptr[w] = o;
    locator[o] = 0;
  }
}

// Locations (circuit.cc:1228-1244) and node degrees.
__global__ void gen_locs_kernel(GenArgs g, const uint32_t *in_ptr, const uint32_t *out_ptr,
                                const int32_t *locator, uint8_t *in_loc, uint8_t *out_loc,
                                uint32_t *deg) {
  const int64_t w = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (w >= g.W) return;
  const uint32_t n = (uint32_t)(w / g.wpp), a = in_ptr[w], b = out_ptr[w];
  in_loc[w] = locator[a] ? CKT_PRIVATE_PTR : CKT_SHARED_PTR;
  out_loc[w] = (b / (uint32_t)g.npp != n) ? CKT_GHOST_PTR
                                          : (locator[b] ? CKT_PRIVATE_PTR : CKT_SHARED_PTR);
  atomicAdd(deg + a, 1u);
  atomicAdd(deg + b, 1u);
}

// Exclusive scan of deg[0..n) into off[0..n] (off[n] = total), three passes.
constexpr int kScanBlock = 1024, kScanItems = 4;

__global__ void scan_blocks_kernel(const uint32_t *in, int64_t n, uint32_t *out, uint32_t *sums) {
  __shared__ uint32_t warp_tot[32];
  const int64_t i0 = ((int64_t)blockIdx.x * kScanBlock + threadIdx.x) * kScanItems;
  uint32_t v[kScanItems], t = 0;
#pragma unroll
  for (int k = 0; k < kScanItems; k++) {
    v[k] = (i0 + k < n) ? in[i0 + k] : 0u;
    t += v[k];
  }
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  uint32_t incl = t;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t y = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= o) incl += y;
  }
  if (lane == 31) warp_tot[wid] = incl;
  __syncthreads();
  if (wid == 0) {
    uint32_t w = warp_tot[lane], wi = w;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t y = __shfl_up_sync(0xffffffffu, wi, o);
      if (lane >= o) wi += y;
    }
    warp_tot[lane] = wi - w;  // exclusive prefix of warp totals
    if (lane == 31) sums[blockIdx.x] = wi;
  }
  __syncthreads();
  uint32_t run = warp_tot[wid] + incl - t;
#pragma unroll
  for (int k = 0; k < kScanItems; k++) {
    if (i0 + k < n) out[i0 + k] = run;
    run += v[k];
  }
}

__global__ void scan_sums_kernel(uint32_t *sums, int64_t nblocks, uint32_t *total) {
  uint32_t run = 0;
  for (int64_t b = 0; b < nblocks; b++) {
    const uint32_t v = sums[b];
    sums[b] = run;
    run += v;
  }
  *total = run;
}

__global__ void scan_add_kernel(uint32_t *out, int64_t n, const uint32_t *sums) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] += sums[i / ((int64_t)kScanBlock * kScanItems)];
}

__global__ void csr_fill_kernel(int64_t W, const uint32_t *in_ptr, const uint32_t *out_ptr,
                                uint32_t *cursor, uint32_t *tmp) {
  const int64_t w = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (w >= W) return;
  tmp[atomicAdd(cursor + in_ptr[w], 1u)] = (uint32_t)(w << 1);
  tmp[atomicAdd(cursor + out_ptr[w], 1u)] = (uint32_t)(w << 1) | 1u;
}

// Per node: sort its contributions by (wire, end), then write the entries
// with their piece-group flags, the wire ends' slots and the flag bits, and
// mark private nodes in the offsets.  A warp takes 32 consecutive nodes: their
// runs are one contiguous span, staged in shared memory (coalesced in and
// out), sorted there a node per lane; a span larger than the stage is sorted
// in place in tmp instead.
constexpr uint32_t kFinishSpan = 512;  // entries per warp staged in shared memory

__global__ void __launch_bounds__(256)
    csr_finish_kernel(GenArgs g, uint32_t *off, const int32_t *locator, uint32_t *tmp,
                      uint32_t *ent, uint32_t *slot_in, uint32_t *slot_out, uint32_t *gstart) {
  __shared__ uint32_t sbuf[8][kFinishSpan];
  const uint32_t lane = threadIdx.x & 31u, wp = threadIdx.x >> 5;
  const int64_t x0 = ((int64_t)blockIdx.x * 8 + wp) * 32;
  if (x0 >= g.N) return;
  const int64_t xe = min(g.N, x0 + 32), x = x0 + lane;
  const uint32_t lo = off[x0] & kOffsetMask, hi = off[xe] & kOffsetMask;
  const uint32_t span = hi - lo;
  const bool staged = span <= kFinishSpan;
  uint32_t *buf = sbuf[wp];
  if (staged)
    for (uint32_t j = lane; j < span; j += 32) buf[j] = tmp[lo + j];
  __syncwarp();
  if (x < xe) {
    const uint32_t b = off[x] & kOffsetMask, e = off[x + 1] & kOffsetMask;
    uint32_t *run = staged ? buf : tmp;    // entry i lives at run[i - rb]
    const uint32_t rb = staged ? lo : 0u;
    for (uint32_t i = b + 1; i < e; i++) {
      const uint32_t v = run[i - rb];
      uint32_t j = i;
      while (j > b && run[j - 1 - rb] > v) {
        run[j - rb] = run[j - 1 - rb];
        j--;
      }
      run[j - rb] = v;
    }
    int64_t last_piece = -1;
    for (uint32_t i = b; i < e; i++) {
      const uint32_t v = run[i - rb], w = v >> 1, end = v & 1u;
      const int64_t piece = w / g.wpp;
      const uint32_t start = piece != last_piece ? 1u : 0u;
      last_piece = piece;
      const uint32_t val = (w << 2) | (end << 1) | start;
      if (staged) {
        buf[i - lo] = val;
      } else {
        ent[i] = val;
        if (start) atomicOr(gstart + (i >> 5), 1u << (i & 31));
      }
      if (end) slot_out[w] = i;
      else slot_in[w] = i;
    }
    if (locator[x]) atomicOr(off + x, kPrivateBit);
  }
  __syncwarp();
  if (staged) {
    for (uint32_t j0 = 0; j0 < span; j0 += 32) {
      const uint32_t j = j0 + lane;
      const uint32_t val = j < span ? buf[j] : 0u;
      if (j < span) ent[lo + j] = val;
      // the group-start bits of these 32 entries, into their one or two words
      const uint32_t m = __ballot_sync(0xffffffffu, (val & 1u) != 0u);
      if (lane == 0 && m) {
        const uint32_t i0 = lo + j0, sh = i0 & 31u, wd = i0 >> 5;
        atomicOr(gstart + wd, m << sh);
        if (sh && (m >> (32 - sh))) atomicOr(gstart + wd + 1, m >> (32 - sh));
      }
    }
  }
}

}  // namespace
}  // namespace ckt

using namespace ckt;

extern "C" int ckt_generate_device(const ckt_gen_params *p, ckt_device_circuit *o, void *stream) {
  NvtxRange range("ckt_generate_device");
  CKT_REQUIRE(p != nullptr && o != nullptr, "NULL argument");
  const int32_t P = p->num_pieces, npp = p->nodes_per_piece, wpp = p->wires_per_piece;
  CKT_REQUIRE(P >= 1 && npp >= 1 && wpp >= 0, "bad shape P=%d npp=%d wpp=%d", P, npp, wpp);
  const int64_t N = (int64_t)P * npp, W = (int64_t)P * wpp;
  CKT_REQUIRE(N < 0x7fffffffLL && W <= kMaxWires, "circuit too large (N=%lld W=%lld)",
              (long long)N, (long long)W);
  CKT_REQUIRE(o->charge && o->node_voltage && o->node_capacitance && o->node_leakage &&
                  o->locator && o->off,
              "node arrays are NULL");
  CKT_REQUIRE(W == 0 || (o->in_ptr && o->out_ptr && o->in_loc && o->out_loc && o->inductance &&
                         o->resistance && o->capacitance && o->current && o->voltage && o->ent &&
                         o->slot_in && o->slot_out && o->gstart),
              "wire arrays are NULL");
  const cudaStream_t s = as_stream(stream);
  int jr = ensure_jump_table();
  if (jr) return jr;
  GenArgs g;
  g.P = P; g.npp = npp; g.wpp = wpp;
  g.pct_thr = drand::pct_threshold(p->pct_wire_in_piece);
  g.L_off = p->L_offset; g.L_scale = p->L_scale;
  g.seed_state = (((uint64_t)p->random_seed & 0xffffffffull) << 16) | 0x330Eull;
  g.W = W; g.N = N;

  gen_nodes_kernel<<<grid_for((N + 15) / 16), 256, 0, s>>>(g, o->charge, o->node_voltage,
                                                          o->node_capacitance, o->node_leakage,
                                                          o->locator);
  CKT_CHECK_LAUNCH();
  CKT_CUDA(cudaMemsetAsync(o->off, 0, (N + 1) * 4, s));
  if (W == 0) {
    // No contributions: only the private-node flags of the offsets remain
    // (every node is private); the entry arrays are never touched.
    csr_finish_kernel<<<grid_for(N), 256, 0, s>>>(g, o->off, o->locator, nullptr, nullptr,
                                                  nullptr, nullptr, nullptr);
    CKT_CHECK_LAUNCH();
    return CKT_OK;
  }

  // Scratch: chunk maps and their composition, degree cursors, unsorted
  // contributions.
  const int64_t base = 3 * N;
  const int64_t nchunks = (7 * W + 8 + kChunk - 1) / kChunk;
  const int64_t nblocks = (nchunks + kMapBlock - 1) / kMapBlock;
  const int64_t scan_blocks = (N + kScanBlock * kScanItems - 1) / (kScanBlock * kScanItems);
  const size_t sz_exit = nchunks * 7, sz_cnt = nchunks * 7 * 4, sz_rph = nchunks * 7,
               sz_rb = nchunks * 7 * 4, sz_bexit = nblocks * 7, sz_bcnt = nblocks * 7 * 4,
               sz_bph = nblocks, sz_bb = nblocks * 8, sz_deg = (N + 1) * 4,
               sz_sums = (scan_blocks + 1) * 4, sz_tmp = 2 * W * 4, sz_starts = W * 4,
               sz_cstate = nchunks * 8;
  auto al = [](size_t b) { return (b + 255) & ~size_t(255); };
  const size_t total = al(sz_exit) + al(sz_cnt) + al(sz_rph) + al(sz_rb) + al(sz_bexit) +
                       al(sz_bcnt) + al(sz_bph) + al(sz_bb) + al(sz_deg) + al(sz_sums) +
                       al(sz_tmp) + al(sz_starts) + al(sz_cstate);
  char *scratch = nullptr;
  CKT_CUDA(cudaMallocAsync(reinterpret_cast<void **>(&scratch), total, s));
  char *q = scratch;
  auto take = [&q, &al](size_t b) {
    char *r = q;
    q += al(b);
    return r;
  };
  uint8_t *exit_phase = (uint8_t *)take(sz_exit);
  uint32_t *count = (uint32_t *)take(sz_cnt);
  uint8_t *rel_phase = (uint8_t *)take(sz_rph);
  uint32_t *rel_base = (uint32_t *)take(sz_rb);
  uint8_t *bexit = (uint8_t *)take(sz_bexit);
  uint32_t *bcount = (uint32_t *)take(sz_bcnt);
  uint8_t *bphase = (uint8_t *)take(sz_bph);
  uint64_t *bbase = (uint64_t *)take(sz_bb);
  uint32_t *deg = (uint32_t *)take(sz_deg);
  uint32_t *sums = (uint32_t *)take(sz_sums);
  uint32_t *tmp = (uint32_t *)take(sz_tmp);
  uint32_t *starts = (uint32_t *)take(sz_starts);
  uint64_t *chunk_state = (uint64_t *)take(sz_cstate);
  int rc = CKT_OK;
  auto ok = [&rc](cudaError_t e) {
    if (rc == CKT_OK && e != cudaSuccess)
      rc = set_error(CKT_ECUDA, "device generator: %s", cudaGetErrorString(e));
  };

  chunk_maps_kernel<<<grid_for(nchunks, kMapsBlock), kMapsBlock, 0, s>>>(g, base, nchunks,
                                                                          exit_phase, count);
  ok(cudaGetLastError());
  map_block_kernel<<<(unsigned)nblocks, 128, 0, s>>>(nchunks, exit_phase, count, rel_phase,
                                                      rel_base, bexit, bcount);
  ok(cudaGetLastError());
  map_top_kernel<<<1, 256, 0, s>>>(nblocks, bexit, bcount, bphase, bbase);
  ok(cudaGetLastError());
  wire_starts_kernel<<<grid_for(nchunks, 128), 128, 0, s>>>(
      g, base, nchunks, rel_phase, rel_base, bphase, bbase, starts, chunk_state);
  ok(cudaGetLastError());
  gen_wires_kernel<<<grid_for(W), 256, 0, s>>>(g, starts, chunk_state, o->in_ptr, o->out_ptr,
                                               o->inductance, o->resistance, o->capacitance,
                                               o->locator);
  ok(cudaGetLastError());
  ok(cudaMemsetAsync(deg, 0, sz_deg, s));
  gen_locs_kernel<<<grid_for(W), 256, 0, s>>>(g, o->in_ptr, o->out_ptr, o->locator, o->in_loc,
                                              o->out_loc, deg);
  ok(cudaGetLastError());
  scan_blocks_kernel<<<(unsigned)scan_blocks, kScanBlock, 0, s>>>(deg, N, o->off, sums);
  ok(cudaGetLastError());
  scan_sums_kernel<<<1, 1, 0, s>>>(sums, scan_blocks, o->off + N);
  ok(cudaGetLastError());
  scan_add_kernel<<<grid_for(N), 256, 0, s>>>(o->off, N, sums);
  ok(cudaGetLastError());
  ok(cudaMemcpyAsync(deg, o->off, N * 4, cudaMemcpyDeviceToDevice, s));  // fill cursors
  csr_fill_kernel<<<grid_for(W), 256, 0, s>>>(W, o->in_ptr, o->out_ptr, deg, tmp);
  ok(cudaGetLastError());
  ok(cudaMemsetAsync(o->gstart, 0, ((2 * W + 31) / 32) * 4, s));
  csr_finish_kernel<<<grid_for(N), 256, 0, s>>>(g, o->off, o->locator, tmp, o->ent, o->slot_in,
                                                o->slot_out, o->gstart);
  ok(cudaGetLastError());
  ok(cudaMemsetAsync(o->current, 0, 10 * W * 4, s));
  ok(cudaMemsetAsync(o->voltage, 0, 9 * W * 4, s));
  cudaFreeAsync(scratch, s);
  return rc;
}
