// ckt_dctile.cuh -- distribute_charge (and the fused node pass) over node
// tiles, with the currents streamed into shared memory by bulk copies.
//
// The gather form (dc_block) reads I[0][w] / I[9][w] once per contribution
// at a random wire: every read moves a 32-byte L2 sector for 4 useful bytes,
// and the sector rate, not DRAM, bounds it.  Here a block owns a tile of
// consecutive nodes and keeps their running sums in shared memory.  The
// tile's contributions are grouped by 2048-wire chunk (the plan built with
// the graph, encoding in ckt_internal.h): for a chunk holding many of them,
// one thread copies the chunk's I[0] and I[9] slices and the step's entry
// words into shared memory with cp.async.bulk (completion on an mbarrier),
// several steps ahead of the threads summing; the few contributions of
// sparse chunks are gathered directly.  Each node still adds its
// contributions in CSR order -- private nodes in place, shared and ghost
// nodes through per-piece folds flushed at group starts -- so the bits
// equal dc_block's.
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

constexpr uint32_t kTileBlock = 1024;
constexpr uint32_t kTileStages = 6;
// Shared memory of one stage: I[0] and I[9] slices of a chunk, then the
// step's entry words.
constexpr uint32_t kStageVals = 2 * kChunkWires;
constexpr uint32_t kStageBytes = (kStageVals + kStepEntriesMax) * 4;

struct DcTileArgs {
  const uint32_t *tile_step;
  const uint4 *steps;
  const uint32_t *ent, *gw;
  const uint32_t *off;
  const float *I0, *I9;  // 16-byte aligned; slices may be read up to a multiple of 4 wires
  float *charge, *voltage;
  const float *cap, *leak;
  uint32_t *error;
  uint64_t timeout_ns;
  uint32_t N, W, tile_nodes;
  float dt;
};

__host__ __device__ constexpr uint32_t dc_tile_smem_bytes(uint32_t tile_nodes) {
  return 2 * tile_nodes * 4 + kTileStages * kStageBytes + kTileStages * 8;
}

// Block-wide: sums the step's node runs.  Entries and stream values are in
// shared memory; for a gather step value k is sval[k].  Each thread takes
// kWalkRows entries per pass; a row whose entry heads a run carries that
// run to its end, one entry per round, so the rows' shared-memory loads
// overlap instead of forming one dependent chain per thread.
constexpr uint32_t kWalkRows = 2;

__device__ __forceinline__ void dc_tile_walk(const uint32_t *sent, const float *sval,
                                             uint32_t cnt, bool stream, float *sacc,
                                             float *sfold, float dt) {
  for (uint32_t j0 = 0; j0 < cnt; j0 += kWalkRows * kTileBlock) {
    uint32_t u[kWalkRows], k[kWalkRows], node[kWalkRows];
    float acc[kWalkRows], fold[kWalkRows];
    bool head[kWalkRows], live[kWalkRows];
    bool any = false;
#pragma unroll
    for (uint32_t r = 0; r < kWalkRows; r++) {
      k[r] = j0 + r * kTileBlock + threadIdx.x;
      u[r] = k[r] < cnt ? sent[k[r]] : kTePad;
      head[r] = (u[r] & kTeHead) && u[r] != kTePad;
      live[r] = head[r];
      node[r] = (u[r] >> kTeNodeShift) & (kTileNodesMax - 1);
      acc[r] = 0.0f;
      fold[r] = 0.0f;
      if (head[r]) {
        acc[r] = sacc[node[r]];
        fold[r] = sfold[node[r]];
      }
      any |= head[r];
    }
    while (any) {
      any = false;
#pragma unroll
      for (uint32_t r = 0; r < kWalkRows; r++) {
        if (!live[r]) continue;
        const uint32_t end = (u[r] >> 11) & 1u;
        const float v =
            stream ? sval[end * kChunkWires + (u[r] & (kChunkWires - 1))] : sval[k[r]];
        const float c = end ? __fmul_rn(dt, v) : __fmul_rn(-dt, v);
        if (u[r] & kTePriv) {
          acc[r] = __fadd_rn(acc[r], c);
        } else {
          if (u[r] & kTeFlush) {
            acc[r] = __fadd_rn(acc[r], fold[r]);
            fold[r] = 0.0f;
          }
          fold[r] = __fadd_rn(fold[r], c);
        }
        if (++k[r] < cnt) {
          u[r] = sent[k[r]];
          live[r] = !(u[r] & kTeHead);  // the next node's run, or padding
        } else {
          live[r] = false;
        }
        any |= live[r];
      }
    }
#pragma unroll
    for (uint32_t r = 0; r < kWalkRows; r++)
      if (head[r]) {
        sacc[node[r]] = acc[r];
        sfold[node[r]] = fold[r];
      }
  }
}

// One block per node tile.  UV = true also applies update_voltages to the
// tile's nodes (the fused node pass: charge ends at zero).
template <bool UV>
__global__ void __launch_bounds__(kTileBlock, 1) dc_tile_kernel(DcTileArgs a) {
  extern __shared__ __align__(128) unsigned char dct_smem[];
  const uint32_t TN = a.tile_nodes;
  float *sacc = reinterpret_cast<float *>(dct_smem);
  float *sfold = sacc + TN;
  unsigned char *stage0 = dct_smem + 2 * TN * 4;
  uint64_t *bar = reinterpret_cast<uint64_t *>(stage0 + kTileStages * kStageBytes);
  auto sval_of = [&](uint32_t slot) {
    return reinterpret_cast<float *>(stage0 + slot * kStageBytes);
  };
  auto sent_of = [&](uint32_t slot) {
    return reinterpret_cast<uint32_t *>(stage0 + slot * kStageBytes + kStageVals * 4);
  };

  const uint32_t t = blockIdx.x;
  const uint32_t x0 = t * TN, xe = min(a.N, x0 + TN), nn = xe - x0;
  const uint32_t s0 = a.tile_step[t], s1 = a.tile_step[t + 1];

  if (threadIdx.x == 0) {
    for (uint32_t k = 0; k < kTileStages; k++) mbar_init(bar + k, 1);
    mbar_init_fence();
  }
  for (uint32_t i = threadIdx.x; i < nn; i += kTileBlock) {
    sacc[i] = a.charge[x0 + i];
    sfold[i] = 0.0f;
  }
  __syncthreads();

  // Thread 0 issues the copies of stream step s (record st) into slot
  // (s - s0) % stages.
  auto issue = [&](uint32_t s, const uint4 &st) {
    if (st.z == kGatherStep) return;
    const uint32_t slot = (s - s0) % kTileStages;
    const uint32_t w0 = st.z * kChunkWires;
    const uint32_t nw = (min(kChunkWires, a.W - w0) + 3u) & ~3u;
    uint64_t *b = bar + slot;
    fence_proxy_async_smem();
    mbar_expect_tx(b, 2 * nw * 4 + st.y * 4);
    bulk_g2s(sval_of(slot), a.I0 + w0, nw * 4, b);
    bulk_g2s(sval_of(slot) + kChunkWires, a.I9 + w0, nw * 4, b);
    bulk_g2s(sent_of(slot), a.ent + st.x, st.y * 4, b);
  };
  if (threadIdx.x == 0)
    for (uint32_t s = s0; s < min(s1, s0 + kTileStages); s++) issue(s, a.steps[s]);

  // Step records are loaded one step ahead (and, by thread 0, the record of
  // the step it issues next), so no global load latency sits between steps.
  uint32_t parity = 0;  // bit k: phase parity of slot k's next completion
  bool failed = false;
  uint4 st_next = s0 < s1 ? a.steps[s0] : make_uint4(0u, 0u, 0u, 0u);
  for (uint32_t s = s0; s < s1; s++) {
    const uint4 st = st_next;
    if (s + 1 < s1) st_next = a.steps[s + 1];
    uint4 st_issue = make_uint4(0u, 0u, kGatherStep, 0u);
    if (threadIdx.x == 0 && s + kTileStages < s1) st_issue = a.steps[s + kTileStages];
    const uint32_t slot = (s - s0) % kTileStages;
    const bool stream = st.z != kGatherStep;
    uint32_t *sent = sent_of(slot);
    float *sval = sval_of(slot);
    bool ok = true;
    if (stream) {
      ok = mbar_wait_bounded(bar + slot, (parity >> slot) & 1u, a.timeout_ns);
      if (ok) parity ^= 1u << slot;
    } else {
      // Gather step: entry words and currents staged by all threads, with
      // several independent loads in flight per thread.
      constexpr uint32_t kBatch = kStepEntriesMax / kTileBlock;
      for (uint32_t j0 = 0; j0 < st.y; j0 += kBatch * kTileBlock) {
        uint32_t u[kBatch], w[kBatch];
#pragma unroll
        for (uint32_t r = 0; r < kBatch; r++) {
          const uint32_t j = j0 + r * kTileBlock + threadIdx.x;
          u[r] = j < st.y ? a.ent[st.x + j] : kTePad;
          w[r] = j < st.y ? a.gw[st.w + j] : 0u;
        }
#pragma unroll
        for (uint32_t r = 0; r < kBatch; r++) {
          const uint32_t j = j0 + r * kTileBlock + threadIdx.x;
          if (j < st.y) {
            float v = 0.0f;
            if (u[r] != kTePad) v = (u[r] & kTeEnd) ? a.I9[w[r]] : a.I0[w[r]];
            sent[j] = u[r];
            sval[j] = v;
          }
        }
      }
      __syncthreads();
    }
    if (ok) dc_tile_walk(sent, sval, st.y, stream, sacc, sfold, a.dt);
    if (__syncthreads_or(!ok)) {
      failed = true;
      break;
    }
    if (threadIdx.x == 0 && s + kTileStages < s1) issue(s + kTileStages, st_issue);
  }

  if (failed) {
    // A copy never completed: report it, let the copies still in flight
    // land (bounded), and leave the tile's charges unwritten.
    if (threadIdx.x == 0) {
      atomicOr(a.error, 1u);
      for (uint32_t k = 0; k < kTileStages; k++)
        mbar_wait_bounded(bar + k, (parity >> k) & 1u, a.timeout_ns);
    }
    return;
  }

  for (uint32_t i = threadIdx.x; i < nn; i += kTileBlock) {
    const uint32_t x = x0 + i;
    const uint32_t o0 = a.off[x], o1 = a.off[x + 1];
    float q = sacc[i];
    if (!(o0 & kPrivateBit) && (o1 & kOffsetMask) > (o0 & kOffsetMask))
      q = __fadd_rn(q, sfold[i]);
    if (UV) {
      a.voltage[x] = uv_one(a.voltage[x], q, a.cap[x], a.leak[x]);
      a.charge[x] = 0.0f;
    } else {
      a.charge[x] = q;
    }
  }
}

}  // namespace ckt
