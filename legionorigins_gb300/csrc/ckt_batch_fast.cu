// ckt_batch_fast.cu -- persistent batched kernels, FAST arithmetic.
#include "ckt_batch_inst.cuh"

namespace ckt {
BatchKernelFn batch_kernel_fast(int block, int wpt, int dcs) { CKT_BATCH_TABLE(CKT_MODE_FAST) }
}  // namespace ckt
