// ckt_batch_exact.cu -- persistent batched kernels, EXACT arithmetic.
#include "ckt_batch_inst.cuh"

namespace ckt {
BatchKernelFn batch_kernel_exact(int block, int wpt, int dcs) { CKT_BATCH_TABLE(CKT_MODE_EXACT) }
}  // namespace ckt
