// ckt_batch_inst.cuh -- instantiation and launch helpers of the persistent
// batched kernel for one arithmetic mode (included by one .cu per mode so the
// instances compile in parallel).
#pragma once

#include "ckt_batch_kernel.cuh"

namespace ckt {

struct BatchLaunch {
  const BatchItem *items;
  uint32_t num_items;
  const BatchCircuit *circ;
  BatchSync sync;
  WireArrays wa;
  BatchNodes nd;
  const uint32_t *off, *ent;
  float dt;
  uint64_t timeout_ns;
};

using BatchKernelFn = void (*)(const BatchItem *, uint32_t, const BatchCircuit *, BatchSync,
                               WireArrays, BatchNodes, const uint32_t *, const uint32_t *, float,
                               uint64_t);

// Returns the kernel for (block, wires per thread, DC schedule), or null.
BatchKernelFn batch_kernel_exact(int block, int wpt, int dcs);
BatchKernelFn batch_kernel_fast(int block, int wpt, int dcs);

#define CKT_BATCH_TABLE(MODE)                                                    \
  switch (block * 100 + wpt * 10 + dcs) {                                        \
    case 12810: return batch_kernel<128, 1, 0, MODE>;                            \
    case 12811: return batch_kernel<128, 1, 1, MODE>;                            \
    case 12820: return batch_kernel<128, 2, 0, MODE>;                            \
    case 12821: return batch_kernel<128, 2, 1, MODE>;                            \
    case 25610: return batch_kernel<256, 1, 0, MODE>;                            \
    case 25611: return batch_kernel<256, 1, 1, MODE>;                            \
    case 25620: return batch_kernel<256, 2, 0, MODE>;                            \
    case 25621: return batch_kernel<256, 2, 1, MODE>;                            \
    default: return nullptr;                                                     \
  }

}  // namespace ckt
