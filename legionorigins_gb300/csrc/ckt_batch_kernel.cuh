// ckt_batch_kernel.cuh -- the persistent "round" kernel: one launch runs one
// outer loop (calc_new_currents, distribute_charge, update_voltages) of every
// circuit in a set of independent circuits of uneven sizes.  Used by the
// batched form (a fixed set) and the serving loop (the set of requests
// resident in a round).
//
// Each circuit is described by a RoundCircuit: its own arrays with local
// wire and node numbering.  Work is a table of items in ticket order: every
// CNC tile of every circuit (longest first), then the DC tiles, then the UV
// tiles.  Resident blocks take tickets from one atomic counter.  A DC tile of
// circuit c waits until all of c's CNC tiles are done, a UV tile until c's
// DC tiles are done; since every item a block waits for has a smaller
// ticket, it is already held by a running block and the wait ends.  Waits
// are bounded (%globaltimer): on timeout the block raises the launch's error
// word and every block returns at its next item; the host reads the word as
// CKT_ETIMEOUT.
#pragma once

#include "ckt_kernels.cuh"

namespace ckt {

enum : uint32_t { kItemCnc = 0u, kItemDc = 1u, kItemUv = 2u };

struct BatchItem {
  uint32_t kind_circuit;  // kind << 30 | circuit index in the launch
  uint32_t begin;         // first wire (CNC) or node (DC, UV), circuit-local
  uint32_t count;
  uint32_t pad;
};

// One circuit of a round launch.  All pointers are device pointers with
// circuit-local indexing (segment stride W).
struct RoundCircuit {
  const uint32_t *in_ptr, *out_ptr;
  const uint8_t *in_loc, *out_loc;
  const float *L, *R, *C;
  float *cur, *vol;
  float *charge, *nvolt;
  const float *cap, *leak;
  const uint32_t *off, *ent;                    // node CSR
  const uint32_t *slot_in, *slot_out, *gstart;  // two-pass / fused distribute_charge
  float *contrib;
  uint32_t W, N;
  int32_t steps;
  uint32_t cnc_items, dc_items;
  uint32_t pad[3];
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

// UV over local nodes [x0, x0 + n): float4 where aligned, scalar tail.
// charge was written by other blocks of this launch: L1-bypassing loads.
template <uint32_t BLOCK>
__device__ __forceinline__ void uv_tile(const RoundCircuit &rc, uint32_t x0, uint32_t n) {
  uint32_t done = 0;
  const bool aligned = ((x0 & 3u) == 0u) &&
                       (((reinterpret_cast<uintptr_t>(rc.charge) |
                          reinterpret_cast<uintptr_t>(rc.nvolt) |
                          reinterpret_cast<uintptr_t>(rc.cap) |
                          reinterpret_cast<uintptr_t>(rc.leak)) & 15u) == 0u);
  if (aligned) {
    const uint32_t n4 = n >> 2;
    float4 *q4 = reinterpret_cast<float4 *>(rc.charge + x0);
    float4 *v4 = reinterpret_cast<float4 *>(rc.nvolt + x0);
    const float4 *c4 = reinterpret_cast<const float4 *>(rc.cap + x0);
    const float4 *l4 = reinterpret_cast<const float4 *>(rc.leak + x0);
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
    rc.nvolt[x] = uv_one(__ldcg(rc.nvolt + x), __ldcg(rc.charge + x), rc.cap[x], rc.leak[x]);
    rc.charge[x] = 0.0f;
  }
}

// DC over local nodes [x0, xe) from the contribution buffer the CNC tiles
// filled (DC schedule 2).  Same order as dc_block.
template <uint32_t BLOCK>
__device__ __forceinline__ void dc_contrib_block(const RoundCircuit &rc, uint32_t x0, uint32_t xe,
                                                 float *sval) {
  const uint32_t x = x0 + threadIdx.x;
  const uint32_t lo = rc.off[x0] & 0x7fffffffu, hi = rc.off[xe] & 0x7fffffffu;
  uint32_t b = 0, e = 0;
  bool priv = true;
  float acc = 0.0f, fold = 0.0f;
  if (x < xe) {
    const uint32_t o0 = rc.off[x], o1 = rc.off[x + 1];
    priv = (o0 & 0x80000000u) != 0;
    b = o0 & 0x7fffffffu;
    e = o1 & 0x7fffffffu;
    acc = rc.charge[x];
  }
  for (uint32_t c0 = lo; c0 < hi; c0 += kDcChunk) {
    const uint32_t cn = min(kDcChunk, hi - c0);
#pragma unroll 4
    for (uint32_t j = threadIdx.x; j < cn; j += BLOCK) sval[j] = __ldcg(rc.contrib + c0 + j);
    __syncthreads();
    const uint32_t i0 = max(b, c0), i1 = min(e, c0 + cn);
    if (priv) {
      for (uint32_t i = i0; i < i1; i++) acc = __fadd_rn(acc, sval[i - c0]);
    } else {
      for (uint32_t i = i0; i < i1; i++) {
        if (i != b && ((rc.gstart[i >> 5] >> (i & 31u)) & 1u)) {
          acc = __fadd_rn(acc, fold);
          fold = 0.0f;
        }
        fold = __fadd_rn(fold, sval[i - c0]);
      }
    }
    __syncthreads();
  }
  if (x < xe) {
    if (!priv && e > b) acc = __fadd_rn(acc, fold);
    rc.charge[x] = acc;
  }
}

// DCS: 0 = staged block gather, 1 = one thread per node, 2 = contributions
// scattered by the CNC tiles then summed contiguously.
// Tiles of two wires per thread run both wires in one paired stepper
// (cnc_wire_pair), which needs more registers: two blocks of 256 per SM.
template <uint32_t BLOCK, int WPT, int DCS, int MODE>
__global__ void __launch_bounds__(BLOCK, (WPT == 2 ? 512 : 768) / BLOCK)
    round_kernel(const BatchItem *__restrict__ items, uint32_t num_items,
                 const RoundCircuit *__restrict__ circ, BatchSync sync, float dt,
                 uint64_t timeout_ns) {
  __shared__ uint32_t s_item, s_go;
  __shared__ float sval[DCS == 1 ? 1 : kDcChunk];
  __shared__ uint32_t smask[DCS == 0 ? kDcChunk / 32 : 1];
  while (true) {
    if (threadIdx.x == 0) {
      const uint32_t it = atomicAdd(sync.ticket, 1u);
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
    const RoundCircuit &rc = circ[c];
    if (kind == kItemCnc) {
      const WireArrays wa = {rc.in_ptr, rc.out_ptr, rc.in_loc, rc.out_loc, rc.L,
                             rc.R,      rc.C,       rc.cur,    rc.vol,     (int64_t)rc.W};
      const NodeVolts volts = {rc.nvolt, rc.nvolt, rc.nvolt};
      if constexpr (WPT == 2) {
        const uint32_t ta = threadIdx.x, tb = ta + BLOCK;
        if (ta < item.count) {
          const bool has_b = tb < item.count;
          const uint32_t w = item.begin + ta, wb = item.begin + (has_b ? tb : ta);
          float2 i0, i9;
          cnc_wire_pair<MODE, CKT_INIT_KERNEL>((int64_t)w, (int64_t)wb, has_b, wa, volts,
                                               rc.steps, dt, &i0, &i9);
          if (DCS == 2) {
            rc.contrib[rc.slot_in[w]] = __fmul_rn(-dt, i0.x);
            rc.contrib[rc.slot_out[w]] = __fmul_rn(dt, i9.x);
            if (has_b) {
              rc.contrib[rc.slot_in[wb]] = __fmul_rn(-dt, i0.y);
              rc.contrib[rc.slot_out[wb]] = __fmul_rn(dt, i9.y);
            }
          }
        }
      } else {
#pragma unroll 1
        for (int r = 0; r < WPT; r++) {
          const uint32_t t = (uint32_t)r * BLOCK + threadIdx.x;
          if (t < item.count) {
            const uint32_t w = item.begin + t;
            float i0, i9;
            cnc_wire<MODE, CKT_INIT_KERNEL>((int64_t)w, wa, volts, rc.steps, dt, &i0, &i9);
            if (DCS == 2) {
              rc.contrib[rc.slot_in[w]] = __fmul_rn(-dt, i0);
              rc.contrib[rc.slot_out[w]] = __fmul_rn(dt, i9);
            }
          }
        }
      }
    } else if (kind == kItemDc) {
      if (DCS == 0) {
        dc_block<BLOCK, true>(item.begin, item.begin + item.count, rc.off, rc.ent, rc.cur,
                              rc.cur + 9 * (size_t)rc.W, rc.charge, dt, sval, smask);
      } else if (DCS == 1) {
        if (threadIdx.x < item.count)
          dc_node<true>(item.begin + threadIdx.x, rc.off, rc.ent, rc.cur,
                        rc.cur + 9 * (size_t)rc.W, rc.charge, dt);
      } else {
        dc_contrib_block<BLOCK>(rc, item.begin, item.begin + item.count, sval);
      }
    } else {
      uv_tile<BLOCK>(rc, item.begin, item.count);
    }
    __syncthreads();
    if (threadIdx.x == 0 && kind != kItemUv) {
      __threadfence();
      atomicAdd(kind == kItemCnc ? sync.done_cnc + c : sync.done_dc + c, 1u);
    }
  }
}

}  // namespace ckt
