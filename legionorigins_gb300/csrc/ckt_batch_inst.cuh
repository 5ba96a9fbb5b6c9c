// ckt_batch_inst.cuh -- instantiation and launch helpers of the persistent
// batched kernel for one arithmetic mode (included by one .cu per mode so the
// instances compile in parallel).
#pragma once

#include "ckt_batch_kernel.cuh"

namespace ckt {

using BatchKernelFn = void (*)(const BatchItem *, uint32_t, const RoundCircuit *, BatchSync, float,
                               uint64_t);

// Returns the kernel for (block, wires per thread, DC schedule), or null.
BatchKernelFn batch_kernel_exact(int block, int wpt, int dcs);
BatchKernelFn batch_kernel_fast(int block, int wpt, int dcs);

#define CKT_BATCH_TABLE(MODE)                                                    \
  switch (block * 100 + wpt * 10 + dcs) {                                        \
    case 12810: return round_kernel<128, 1, 0, MODE>;                            \
    case 12811: return round_kernel<128, 1, 1, MODE>;                            \
    case 12812: return round_kernel<128, 1, 2, MODE>;                            \
    case 12820: return round_kernel<128, 2, 0, MODE>;                            \
    case 12821: return round_kernel<128, 2, 1, MODE>;                            \
    case 12822: return round_kernel<128, 2, 2, MODE>;                            \
    case 25610: return round_kernel<256, 1, 0, MODE>;                            \
    case 25611: return round_kernel<256, 1, 1, MODE>;                            \
    case 25612: return round_kernel<256, 1, 2, MODE>;                            \
    case 25620: return round_kernel<256, 2, 0, MODE>;                            \
    case 25621: return round_kernel<256, 2, 1, MODE>;                            \
    case 25622: return round_kernel<256, 2, 2, MODE>;                            \
    default: return nullptr;                                                     \
  }

}  // namespace ckt
