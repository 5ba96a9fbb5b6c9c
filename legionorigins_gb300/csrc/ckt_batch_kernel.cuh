// ckt_batch_kernel.cuh -- the persistent batched kernel: one launch runs one
// outer loop (calc_new_currents, distribute_charge, update_voltages) of every
// circuit of a batch of independent circuits of uneven sizes.
//
// Work is a table of items in ticket order: every CNC tile of every circuit
// (longest first), then the DC tiles, then the UV tiles.  Resident blocks
// take tickets from one atomic counter.  A DC tile of circuit c waits until
// all of c's CNC tiles are done, a UV tile until c's DC tiles are done; since
// every item a block waits for has a smaller ticket, it is already held by a
// running block and the wait ends.  Waits are bounded (%globaltimer): on
// timeout the block raises the batch's error word and every block returns at
// its next item; the host reads the word as CKT_ETIMEOUT.
#pragma once

#include "ckt_kernels.cuh"

namespace ckt {

enum : uint32_t { kItemCnc = 0u, kItemDc = 1u, kItemUv = 2u };

struct BatchItem {
  uint32_t kind_circuit;  // kind << 30 | circuit
  uint32_t begin;         // first wire (CNC) or node (DC, UV), union numbering
  uint32_t count;
  uint32_t pad;
};

struct BatchCircuit {
  int32_t steps;
  uint32_t cnc_items;
  uint32_t dc_items;
  uint32_t pad;
};

struct BatchNodes {
  float *charge, *voltage;
  const float *cap, *leak;
};

struct BatchSync {
  uint32_t *ticket;    // [1]
  uint32_t *error;     // [1]  bit 0: a wait timed out
  uint32_t *done_cnc;  // [circuits]
  uint32_t *done_dc;   // [circuits]
};

__device__ __forceinline__ uint64_t global_ns() {
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

__device__ __forceinline__ uint32_t ld_acquire(const uint32_t *p) {
  uint32_t v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

__device__ __forceinline__ uint32_t ld_relaxed(const uint32_t *p) {
  uint32_t v;
  asm volatile("ld.relaxed.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

// Bounded wait for *counter >= target.  Returns false on timeout or when
// another block has raised the error word.
__device__ __forceinline__ bool wait_count(const uint32_t *counter, uint32_t target,
                                           uint32_t *error, uint64_t timeout_ns) {
  if (ld_acquire(counter) >= target) return true;
  const uint64_t t0 = global_ns();
  while (true) {
    __nanosleep(128);
    if (ld_acquire(counter) >= target) return true;
    if (ld_relaxed(error) != 0u) return false;
    if (global_ns() - t0 > timeout_ns) {
      atomicOr(error, 1u);
      return false;
    }
  }
}

// UV over nodes [x0, x0 + n): float4 where aligned, scalar tail.  COHERENT:
// charge was written by other blocks of this launch.
template <uint32_t BLOCK>
__device__ __forceinline__ void uv_tile(uint32_t x0, uint32_t n, const BatchNodes &nd) {
  uint32_t done = 0;
  if ((x0 & 3u) == 0u) {
    const uint32_t n4 = n >> 2;
    float4 *q4 = reinterpret_cast<float4 *>(nd.charge + x0);
    float4 *v4 = reinterpret_cast<float4 *>(nd.voltage + x0);
    const float4 *c4 = reinterpret_cast<const float4 *>(nd.cap + x0);
    const float4 *l4 = reinterpret_cast<const float4 *>(nd.leak + x0);
    for (uint32_t i = threadIdx.x; i < n4; i += BLOCK) {
      const float4 qq = __ldcg(q4 + i), vv = __ldcg(v4 + i), cc = c4[i], ll = l4[i];
      float4 r;
      r.x = uv_one(vv.x, qq.x, cc.x, ll.x);
      r.y = uv_one(vv.y, qq.y, cc.y, ll.y);
      r.z = uv_one(vv.z, qq.z, cc.z, ll.z);
      r.w = uv_one(vv.w, qq.w, cc.w, ll.w);
      v4[i] = r;
      q4[i] = make_float4(0.f, 0.f, 0.f, 0.f);
    }
    done = n4 << 2;
  }
  for (uint32_t i = done + threadIdx.x; i < n; i += BLOCK) {
    const uint32_t x = x0 + i;
    nd.voltage[x] = uv_one(__ldcg(nd.voltage + x), __ldcg(nd.charge + x), nd.cap[x], nd.leak[x]);
    nd.charge[x] = 0.0f;
  }
}

// DCS: 0 = staged block gather, 1 = one thread per node.
template <uint32_t BLOCK, int WPT, int DCS, int MODE>
__global__ void __launch_bounds__(BLOCK, 768 / BLOCK)
    batch_kernel(const BatchItem *__restrict__ items, uint32_t num_items,
                 const BatchCircuit *__restrict__ circ, BatchSync sync, WireArrays wa,
                 BatchNodes nd, const uint32_t *__restrict__ off,
                 const uint32_t *__restrict__ ent, float dt, uint64_t timeout_ns) {
  __shared__ uint32_t s_item, s_go;
  __shared__ float sval[DCS == 0 ? kDcChunk : 1];
  __shared__ uint8_t sflag[DCS == 0 ? kDcChunk : 1];
  const float *I0 = wa.cur, *I9 = wa.cur + 9 * wa.S;
  const NodeVolts volts = {nd.voltage, nd.voltage, nd.voltage};
  while (true) {
    if (threadIdx.x == 0) {
      uint32_t it = atomicAdd(sync.ticket, 1u);
      uint32_t go = (it < num_items && ld_relaxed(sync.error) == 0u) ? 1u : 0u;
      if (go) {
        const BatchItem item = items[it];
        const uint32_t kind = item.kind_circuit >> 30, c = item.kind_circuit & 0x3fffffffu;
        if (kind == kItemDc)
          go = wait_count(sync.done_cnc + c, circ[c].cnc_items, sync.error, timeout_ns);
        else if (kind == kItemUv)
          go = wait_count(sync.done_dc + c, circ[c].dc_items, sync.error, timeout_ns);
      }
      s_item = it;
      s_go = go;
    }
    __syncthreads();
    const uint32_t it = s_item;
    const bool go = s_go != 0u;
    __syncthreads();
    if (!go) return;
    const BatchItem item = items[it];
    const uint32_t kind = item.kind_circuit >> 30, c = item.kind_circuit & 0x3fffffffu;
    if (kind == kItemCnc) {
      const int steps = circ[c].steps;
#pragma unroll 1
      for (int r = 0; r < WPT; r++) {
        const uint32_t t = (uint32_t)r * BLOCK + threadIdx.x;
        if (t < item.count)
          cnc_wire<MODE, CKT_INIT_KERNEL>((int64_t)item.begin + t, wa, volts, steps, dt);
      }
    } else if (kind == kItemDc) {
      if (DCS == 0) {
        dc_block<BLOCK, true>(item.begin, item.begin + item.count, off, ent, I0, I9, nd.charge,
                              dt, sval, sflag);
      } else {
        if (threadIdx.x < item.count)
          dc_node<true>(item.begin + threadIdx.x, off, ent, I0, I9, nd.charge, dt);
      }
    } else {
      uv_tile<BLOCK>(item.begin, item.count, nd);
    }
    __syncthreads();
    if (threadIdx.x == 0 && kind != kItemUv) {
      __threadfence();
      atomicAdd(kind == kItemCnc ? sync.done_cnc + c : sync.done_dc + c, 1u);
    }
  }
}

}  // namespace ckt
