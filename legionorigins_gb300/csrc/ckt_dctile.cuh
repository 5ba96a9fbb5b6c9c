// ckt_dctile.cuh -- distribute_charge (and the fused node pass) over node
// tiles, with the currents streamed into shared memory by bulk copies.
//
// The gather form (dc_block) reads I[0][w] / I[9][w] once per contribution
// at a random wire: every read moves a 32-byte L2 sector for 4 useful bytes,
// and the sector rate, not DRAM, bounds it.  Here a block owns a tile of
// consecutive nodes and keeps their running sums in shared memory.  The
// tile's contributions are grouped by 4096-wire chunk (the plan built with
// the graph, encoding in ckt_internal.h): for a chunk holding many of them,
// one lane of a copy warp moves the chunk's I[0] and I[9] slices and the
// step's entry block into a three-stage shared-memory ring with cp.async.bulk
// (completion on the stage's mbarrier).  The few contributions of sparse
// chunks -- in the benchmark circuits, the wires that end in another piece
// -- are packed first by ghost_pack_kernel, which reads their currents in
// wire order and stores each into its step's run of the graph's ghost
// buffer; the copy warp moves those runs like a chunk's slices.  (Gathering
// them inside the tile pass read one random 32-byte sector per value, mostly
// from DRAM, since the streamed chunks keep evicting the currents from L2.)
// 31 consumer warps own disjoint node sets, so they walk the steps without
// block barriers and hand each stage back through a second mbarrier; each
// lane sums its own list of whole node runs, balanced within the warp.  Each
// node still adds its contributions in CSR order -- private nodes in place,
// shared and ghost nodes through per-piece folds flushed at group starts --
// so the bits equal dc_block's.
#pragma once

#include "ckt_internal.h"
#include "ckt_kernels.cuh"

namespace ckt {

__device__ __forceinline__ uint32_t smem_addr(const void *p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count)
               : "memory");
}

__device__ __forceinline__ void mbar_init_fence() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t *bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)),
               "r"(bytes)
               : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(smem_addr(bar)), "r"(parity)
      : "memory");
  return ok != 0u;
}

// try_wait with a suspend-time hint: the thread sleeps until the phase
// completes or about hint_ns pass, instead of spinning on the barrier.
__device__ __forceinline__ bool mbar_try_wait_sleep(uint64_t *bar, uint32_t parity,
                                                    uint32_t hint_ns) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(smem_addr(bar)), "r"(parity), "r"(hint_ns)
      : "memory");
  return ok != 0u;
}

// Orders this thread's earlier shared-memory accesses (generic proxy) before
// its later bulk copies (async proxy) into the same buffers.
__device__ __forceinline__ void fence_proxy_async_smem() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

// 1-D bulk copy global -> shared; `bytes` and both addresses 16-byte aligned.
__device__ __forceinline__ void bulk_g2s(void *dst, const void *src, uint32_t bytes,
                                         uint64_t *bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::
          "r"(smem_addr(dst)),
      "l"(src), "r"(bytes), "r"(smem_addr(bar))
      : "memory");
}

__device__ __forceinline__ uint64_t dct_now_ns() {
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// Waits for phase `parity` of `bar` to complete, for at most timeout_ns.
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t *bar, uint32_t parity,
                                                  uint64_t timeout_ns) {
  if (mbar_try_wait(bar, parity)) return true;
  const uint64_t t0 = dct_now_ns();
  for (;;) {
    for (int k = 0; k < 64; k++)
      if (mbar_try_wait(bar, parity)) return true;
    if (dct_now_ns() - t0 > timeout_ns) return false;
  }
}

constexpr uint32_t kTileBlock = 32 * (kTileWarps + 1);  // consumer warps + one copy warp
constexpr uint32_t kTileStages = 3;
// Shared memory of one stage: I[0] and I[9] slices of a chunk (a ghost
// step's in-end and out-end runs in their place), then the step's block
// (header + entries).
constexpr uint32_t kStageVals = 2 * kChunkWires;
constexpr uint32_t kStageBlockWords = kStepHeaderWords + kStepEntriesMax;
constexpr uint32_t kStageBytes = (kStageVals + kStageBlockWords) * 4;

struct DcTileArgs {
  const uint32_t *tile_step;
  const uint4 *steps;
  const uint32_t *ent;
  const float *ghost;  // ghost steps' values, packed by ghost_pack_kernel
  const uint32_t *mask;  // per tile: nodes whose folds are added at the end
  const float *I0, *I9;  // 16-byte aligned; slices may be read up to a multiple of 4 wires
  float *charge, *voltage;
  const float *cap, *leak;
  uint32_t *error;
  uint64_t timeout_ns;
  uint32_t N, W, tile_nodes;
  uint32_t node_copy;  // voltage, cap, leak 16-byte aligned: staged by bulk copies
  float dt;
};

constexpr uint32_t kMaskWords = kTileNodesMax / 32;
// The last pass reads the tile's voltage, capacitance and leakage from two
// stages freed by the last steps: stage A holds voltage, then the first
// kLeakSplit leakages; stage B holds capacitance, then the rest.
constexpr uint32_t kLeakSplit = kStageBytes / 4 - kTileNodesMax;
static_assert(kLeakSplit % 4 == 0 && kLeakSplit <= kTileNodesMax &&
                  kTileNodesMax + (kTileNodesMax - kLeakSplit) <= kStageBytes / 4,
              "node data does not fit two stages");

__host__ __device__ constexpr uint32_t dc_tile_smem_bytes(uint32_t tile_nodes) {
  return 2 * tile_nodes * 4 + kMaskWords * 4 + kTileStages * kStageBytes +
         (2 * kTileStages + 2) * 8 + 16;
}

// Bounded wait that also gives up once another thread has raised `abort`.
__device__ __forceinline__ bool mbar_wait_abortable(uint64_t *bar, uint32_t parity,
                                                    const volatile uint32_t *abort,
                                                    uint64_t timeout_ns) {
  if (mbar_try_wait(bar, parity)) return true;
  const uint64_t t0 = dct_now_ns();
  for (;;) {
    if (mbar_try_wait_sleep(bar, parity, 20000u)) return true;
    if (*abort != 0u || dct_now_ns() - t0 > timeout_ns) return false;
  }
}

__device__ __forceinline__ void mbar_arrive(uint64_t *bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_addr(bar)) : "memory");
}

// One lane sums its list of node runs in a step: entries [b, e) of the
// step's block, runs back to back, each opened by a head entry; an entry's
// current is svals[end * kChunkWires + index].
__device__ __forceinline__ void dc_tile_lane_walk(const uint32_t *sent, const float *svals,
                                                  uint32_t b, uint32_t e, float2 *ssum,
                                                  float dt) {
  uint32_t node = 0xffffffffu;
  float acc = 0.0f, fold = 0.0f;
  for (uint32_t p = b; p < e; p++) {
    const uint32_t u = sent[p];
    const uint32_t end = (u & kTeEnd) ? 1u : 0u;
    const float v = svals[end * kChunkWires + (u & (kChunkWires - 1))];
    if (u & kTeHead) {
      if (node != 0xffffffffu) ssum[node] = make_float2(acc, fold);
      node = (u >> kTeNodeShift) & (kTileNodesMax - 1);
      const float2 t = ssum[node];
      acc = t.x;
      fold = t.y;
    }
    const float c = end ? __fmul_rn(dt, v) : __fmul_rn(-dt, v);
    if (u & kTePriv) {
      acc = __fadd_rn(acc, c);
    } else {
      if (u & kTeFlush) {
        acc = __fadd_rn(acc, fold);
        fold = 0.0f;
      }
      fold = __fadd_rn(fold, c);
    }
  }
  if (node != 0xffffffffu) ssum[node] = make_float2(acc, fold);
}

// Programmatic dependent launch: the tile pass is launched to start while
// ghost_pack_kernel still runs, and its copy lane waits for the packing's
// end (and the visibility of its stores) before the first ghost step's copy.
__device__ __forceinline__ void grid_dependents_launch() {
  asm volatile("griddepcontrol.launch_dependents;" :::);
}
__device__ __forceinline__ void grid_dependency_wait() {
  asm volatile("griddepcontrol.wait;" ::: "memory");
}
__device__ __forceinline__ void fence_proxy_async_global() {
  asm volatile("fence.proxy.async.global;" ::: "memory");
}

// Fills the ghost buffer: ghost[slot] = I[end][wire] for each list entry.
// The list is sorted by source block of kPackWires wires, then by slot.
//  * Many ghost ends (STAGED): a block takes one source block: it loads the
//    block's I[0] and/or I[9] slices into shared memory with coalesced
//    loads, then stores the block's entries from there, so that the stores
//    into one step's run go out together.  Its first kPackPer entries per
//    thread are loaded before the slices, so that the two loads overlap.
//  * Few ghost ends (whole slices would be mostly unused): a thread takes
//    kPackPer entries spread over the list and reads each current directly,
//    all its loads in flight together.
// Either way the tile pass may already be running (programmatic dependent
// launch); it waits for this grid before its first ghost step's copy.
constexpr uint32_t kPackBlock = 512, kPackPer = 4;
template <bool STAGED>
__global__ void __launch_bounds__(kPackBlock, 3) ghost_pack_kernel(const uint2 *__restrict__ list,
                                                                   const uint32_t *__restrict__ blk,
                                                                   uint32_t n, uint32_t W,
                                                                   const float *__restrict__ I0,
                                                                   const float *__restrict__ I9,
                                                                   float *__restrict__ ghost) {
  __shared__ float4 sv[STAGED ? 2 * kPackWires / 4 : 1];
  grid_dependents_launch();
  uint32_t first, last, stride, w0 = 0, d = 0;
  if (STAGED) {
    d = blk[blockIdx.x];
    first = (d & kPackFirstMask) + threadIdx.x;
    last = blk[blockIdx.x + 1] & kPackFirstMask;
    if (first - threadIdx.x == last) return;
    stride = kPackBlock;
    w0 = blockIdx.x * kPackWires;
  } else {
    first = blockIdx.x * kPackBlock + threadIdx.x;
    last = n;
    stride = gridDim.x * kPackBlock;
  }
  uint2 e[kPackPer];
#pragma unroll
  for (uint32_t j = 0; j < kPackPer; j++) {
    const uint32_t k = first + j * stride;
    e[j] = k < last ? list[k] : make_uint2(0xffffffffu, 0u);
  }
  if (STAGED) {
    const uint32_t nw4 = (min(kPackWires, W - w0) + 3u) / 4u;  // arrays extend to a multiple of 4
    const float4 *src0 = reinterpret_cast<const float4 *>(I0 + w0);
    const float4 *src1 = reinterpret_cast<const float4 *>(I9 + w0);
    for (uint32_t i = threadIdx.x; i < nw4; i += kPackBlock) {
      if (d & kPackHasIn) sv[i] = __ldcs(src0 + i);
      if (d & kPackHasOut) sv[kPackWires / 4 + i] = __ldcs(src1 + i);
    }
    __syncthreads();
    const float *sf = reinterpret_cast<const float *>(sv);
#pragma unroll
    for (uint32_t j = 0; j < kPackPer; j++)
      if (e[j].x != 0xffffffffu)
        ghost[e[j].x] = sf[(e[j].y & 1u) * kPackWires + (e[j].y >> 1) - w0];
    for (uint32_t k = first + kPackPer * stride; k < last; k += stride) {
      const uint2 f = list[k];
      ghost[f.x] = sf[(f.y & 1u) * kPackWires + (f.y >> 1) - w0];
    }
  } else {
    float v[kPackPer];
#pragma unroll
    for (uint32_t j = 0; j < kPackPer; j++)
      if (e[j].x != 0xffffffffu) v[j] = (e[j].y & 1u) ? I9[e[j].y >> 1] : I0[e[j].y >> 1];
#pragma unroll
    for (uint32_t j = 0; j < kPackPer; j++)
      if (e[j].x != 0xffffffffu) ghost[e[j].x] = v[j];
  }
}

// One block per node tile: warp kTileWarps (lane 0) copies the steps' data
// into a ring of kTileStages stages; consumer warp w sums the runs of the
// tile's nodes n with n mod kTileWarps == w, so no two warps touch a node
// and the warps run through the steps independently, each handing its stage
// back through the stage's `empty` barrier.  UV = true also applies
// update_voltages to the tile's nodes (the fused node pass: charge ends at
// zero).
template <bool UV>
__global__ void __launch_bounds__(kTileBlock, 1) dc_tile_kernel(DcTileArgs a) {
  extern __shared__ __align__(128) unsigned char dct_smem[];
  const uint32_t TN = a.tile_nodes;
  float2 *ssum = reinterpret_cast<float2 *>(dct_smem);  // per node: running sum, fold
  uint32_t *smask = reinterpret_cast<uint32_t *>(ssum + TN);
  unsigned char *stage0 = dct_smem + 2 * TN * 4 + kMaskWords * 4;
  uint64_t *full = reinterpret_cast<uint64_t *>(stage0 + kTileStages * kStageBytes);
  uint64_t *empty = full + kTileStages;
  uint64_t *maskbar = empty + kTileStages, *nodebar = maskbar + 1;
  volatile uint32_t *abort = reinterpret_cast<volatile uint32_t *>(nodebar + 1);
  auto vals_of = [&](uint32_t slot) {
    return reinterpret_cast<float *>(stage0 + slot * kStageBytes);
  };
  auto block_of = [&](uint32_t slot) {
    return reinterpret_cast<uint32_t *>(stage0 + slot * kStageBytes + kStageVals * 4);
  };

  const uint32_t t = blockIdx.x;
  const uint32_t x0 = t * TN, xe = min(a.N, x0 + TN), nn = xe - x0;
  const uint32_t s0 = a.tile_step[t], s1 = a.tile_step[t + 1];
  const uint32_t warp = threadIdx.x >> 5, lane = threadIdx.x & 31u;

  if (threadIdx.x == 0) {
    for (uint32_t k = 0; k < kTileStages; k++) {
      mbar_init(full + k, 1);
      mbar_init(empty + k, kTileWarps);
    }
    mbar_init(maskbar, 1);
    mbar_init(nodebar, 1);
    *abort = 0u;
    mbar_init_fence();
  }
  __syncthreads();

  // Copy warp: the copies of step s into its stage (after the stage's
  // previous contents have been handed back).
  uint32_t issued = 0;
  bool packed = false;  // the ghost buffer is known to be filled
  auto issue = [&](uint32_t s) -> bool {
    const uint32_t n = s - s0, slot = n % kTileStages;
    if (n >= kTileStages &&
        !mbar_wait_abortable(empty + slot, ((n / kTileStages) - 1) & 1u, abort, a.timeout_ns))
      return false;
    const uint4 st = a.steps[s];
    if ((st.z & kGhostStep) != 0u && !packed) {
      grid_dependency_wait();
      fence_proxy_async_global();
      packed = true;
    }
    // in-end and out-end values: [0, n0) and [kChunkWires, kChunkWires + n1)
    const float *src0, *src1;
    uint32_t n0, n1;
    if ((st.z & kGhostStep) == 0u) {
      n0 = n1 = (min(kChunkWires, a.W - st.z * kChunkWires) + 3u) & ~3u;
      src0 = a.I0 + st.z * kChunkWires;
      src1 = a.I9 + st.z * kChunkWires;
    } else {
      n0 = (((st.z >> kGhostCountBits) & kGhostCountMask) + 3u) & ~3u;
      n1 = ((st.z & kGhostCountMask) + 3u) & ~3u;
      src0 = a.ghost + st.w;
      src1 = src0 + n0;
    }
    uint64_t *bar = full + slot;
    fence_proxy_async_smem();
    mbar_expect_tx(bar, (st.y + n0 + n1) * 4);
    if (n0) bulk_g2s(vals_of(slot), src0, n0 * 4, bar);
    if (n1) bulk_g2s(vals_of(slot) + kChunkWires, src1, n1 * 4, bar);
    bulk_g2s(block_of(slot), a.ent + st.x, st.y * 4, bar);
    issued = max(issued, n + 1);
    return true;
  };
  const bool producer = warp == kTileWarps && lane == 0;
  uint32_t s_next = s0;
  if (producer) {  // the fold mask and the first stages load while the accumulators fill
    fence_proxy_async_smem();
    mbar_expect_tx(maskbar, kMaskWords * 4);
    bulk_g2s(smask, a.mask + (size_t)t * kMaskWords, kMaskWords * 4, maskbar);
    // The first stages' copies; a ghost step among them waits for the
    // packing, after the barrier below (each of these stages is used for the
    // first time, so the others go ahead out of order).
    for (; s_next < min(s1, s0 + kTileStages); s_next++)
      if ((a.steps[s_next].z & kGhostStep) == 0u) issue(s_next);
  }
  // Node data staged for the last pass: elements [0, nn4) of each array.
  const uint32_t nn4 = nn & ~3u, nsteps = s1 - s0;
  const bool stage_nodes = UV && a.node_copy && nn4 > 0 && nsteps >= 1;
  uint32_t slot_a = 0, slot_b = 0;
  if (stage_nodes) {  // the two stages not holding the last step
    slot_a = (nsteps - 1 + 1) % kTileStages;
    slot_b = (nsteps - 1 + 2) % kTileStages;
  }
  {
    constexpr uint32_t kPer = kTileNodesMax / kTileBlock;
    float q[kPer];
#pragma unroll
    for (uint32_t r = 0; r < kPer; r++) {
      const uint32_t i = threadIdx.x + r * kTileBlock;
      q[r] = i < nn ? a.charge[x0 + i] : 0.0f;
    }
#pragma unroll
    for (uint32_t r = 0; r < kPer; r++) {
      const uint32_t i = threadIdx.x + r * kTileBlock;
      if (i < nn) {
        ssum[i] = make_float2(q[r], 0.0f);
      }
    }
  }
  __syncthreads();

  bool node_issued = false;
  if (warp == kTileWarps) {
    if (producer) {
      for (uint32_t s = s0; s < min(s1, s0 + kTileStages); s++)
        if ((a.steps[s].z & kGhostStep) != 0u) issue(s);  // never waits: a first use
      for (; s_next < s1; s_next++)
        if (!issue(s_next)) {
          *abort = 1u;
          break;
        }
      if (stage_nodes && *abort == 0u) {
        // Stages A and B last held steps nsteps - 3 and nsteps - 2 (when the
        // tile has them): wait until the consumers hand them back.
        bool ok = true;
        for (uint32_t back = 3; back >= 2 && ok; back--) {
          if (nsteps < back) continue;
          const uint32_t n = nsteps - back;
          ok = mbar_wait_abortable(empty + n % kTileStages, (n / kTileStages) & 1u, abort,
                                   a.timeout_ns);
        }
        if (!ok) {
          *abort = 1u;
        } else {
          float *sa = vals_of(slot_a), *sb = vals_of(slot_b);
          const uint32_t la = min(nn4, kLeakSplit), lb = nn4 - la;
          fence_proxy_async_smem();
          mbar_expect_tx(nodebar, (3 * nn4) * 4);
          bulk_g2s(sa, a.voltage + x0, nn4 * 4, nodebar);
          bulk_g2s(sb, a.cap + x0, nn4 * 4, nodebar);
          bulk_g2s(sa + kTileNodesMax, a.leak + x0, la * 4, nodebar);
          if (lb) bulk_g2s(sb + kTileNodesMax, a.leak + x0 + la, lb * 4, nodebar);
          node_issued = true;
        }
      }
    }
  } else {
    for (uint32_t s = s0; s < s1; s++) {
      const uint32_t n = s - s0, slot = n % kTileStages;
      if (!mbar_wait_abortable(full + slot, (n / kTileStages) & 1u, abort, a.timeout_ns)) {
        *abort = 1u;
        break;
      }
      const uint32_t *blk = block_of(slot);
      const uint16_t *hdr = reinterpret_cast<const uint16_t *>(blk);
      const uint32_t last = hdr[kTileLanes];
      const uint32_t l = threadIdx.x;  // consumer lane list (warp * 32 + lane)
      const uint32_t b = hdr[l], e = l + 1 < kTileLanes ? hdr[l + 1] : last;
      dc_tile_lane_walk(blk + kStepHeaderWords, vals_of(slot), b, e, ssum, a.dt);
      __syncwarp();
      if (lane == 0) mbar_arrive(empty + slot);
    }
  }
  __syncthreads();

  const bool mask_ok = mbar_wait_bounded(maskbar, 0u, a.timeout_ns);
  const bool nodes_ok = !stage_nodes || mbar_wait_bounded(nodebar, 0u, a.timeout_ns);
  if (__syncthreads_or(*abort != 0u || !mask_ok || !nodes_ok)) {
    // A wait ran out: report it, let every copy still in flight land (with
    // a bound of its own, whatever the waits' limit was), and leave the
    // tile's results unwritten.
    if (producer) {
      constexpr uint64_t kDrainNs = 1000000000ull;
      *reinterpret_cast<volatile uint32_t *>(a.error) = 1u;  // host-mapped word
      __threadfence_system();
      mbar_wait_bounded(maskbar, 0u, kDrainNs);
      for (uint32_t n = issued > kTileStages ? issued - kTileStages : 0; n < issued; n++)
        mbar_wait_bounded(full + n % kTileStages, (n / kTileStages) & 1u, kDrainNs);
      if (node_issued) mbar_wait_bounded(nodebar, 0u, kDrainNs);
    }
    return;
  }

  const float *sv = vals_of(slot_a), *sc = vals_of(slot_b);
  constexpr uint32_t kPer = kTileNodesMax / kTileBlock;
#pragma unroll 4
  for (uint32_t r = 0; r < kPer; r++) {
    const uint32_t i = threadIdx.x + r * kTileBlock, x = x0 + i;
    if (i >= nn) break;
    const float2 t = ssum[i];
    float q = t.x;
    if ((smask[i >> 5] >> (i & 31u)) & 1u) q = __fadd_rn(q, t.y);
    if (UV) {
      float v, cap, leak;
      if (stage_nodes && i < nn4) {
        v = sv[i];
        cap = sc[i];
        leak = i < kLeakSplit ? sv[kTileNodesMax + i] : sc[kTileNodesMax + i - kLeakSplit];
      } else {
        v = a.voltage[x];
        cap = a.cap[x];
        leak = a.leak[x];
      }
      a.voltage[x] = uv_one(v, q, cap, leak);
      a.charge[x] = 0.0f;
    } else {
      a.charge[x] = q;
    }
  }
}

}  // namespace ckt
