// ckt_reduce.cu -- GPU form of LegionOrigins' reduction microbenchmark
// (benchmarks/reductions/reducetest.cc): a histogram whose elements are
// produced by the benchmark's own 48-bit-LCG hash, reduced into the target
// under four schedules that map the benchmark's cases onto the GPU's memory
// levels (global atomics, block-private folds in shared memory or L2,
// owner-local copies in shared memory, reduction lists in L2).
//
// Keys are recomputed from the element index wherever a schedule needs them
// (the benchmark's tasks do the same), so the schedules differ only in where
// the reductions land and how they reach the target.
#include <algorithm>

#include "ckt_internal.h"

namespace ckt {
namespace {

struct HistArgs {
  uint32_t base;       // 32-bit index of the first element: first_batch * batch_size
  uint32_t buckets;
  uint64_t total;      // elements
  uint32_t seed1, seed2;
  uint64_t mod_magic;  // remainder constant for `buckets` (see hist_key)
};

// Key of element e: myrand(start + i) % buckets (reducetest.cc:323-333,
// 341-344), with start + i = base + e in 32-bit unsigned arithmetic.  The
// remainder uses Lemire, Kaser and Kurz's direct computation ("Faster
// Remainder by Direct Computation", 2019): for 32-bit a and d >= 1 with
// M = floor((2^64 - 1) / d) + 1 (mod 2^64), a % d = high64((M * a mod 2^64) * d).
__device__ __forceinline__ uint32_t hist_key(const HistArgs &a, uint64_t e) {
  const uint32_t ival = a.base + (uint32_t)e;
  uint64_t r = ival;
#pragma unroll
  for (int j = 0; j < 16; j++) {
    r = (0x5DEECE66Dull * r + 0xBull) & 0xFFFFFFFFFFFFull;
    r ^= ((ival >> j) & 1u) ? a.seed1 : a.seed2;
  }
  return (uint32_t)__umul64hi(a.mod_magic * (uint32_t)r, (uint64_t)a.buckets);
}

__device__ __forceinline__ uint64_t gtid() {
  return (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
}
__device__ __forceinline__ uint64_t gstride() { return (uint64_t)gridDim.x * blockDim.x; }

// --- single: every reduction straight into the target ----------------------
__global__ void __launch_bounds__(256) single_kernel(HistArgs a, uint32_t *hist) {
  for (uint64_t e = gtid(); e < a.total; e += gstride()) atomicAdd(hist + hist_key(a, e), 1u);
}

// --- fold: block-private fold instance, then applied -----------------------
constexpr int kFoldBlock = 1024;

__global__ void __launch_bounds__(kFoldBlock) fold_smem_kernel(HistArgs a, uint32_t *hist) {
  extern __shared__ uint32_t fold[];
  for (uint32_t b = threadIdx.x; b < a.buckets; b += blockDim.x) fold[b] = 0u;  // identity
  __syncthreads();
  for (uint64_t e = gtid(); e < a.total; e += gstride()) atomicAdd(fold + hist_key(a, e), 1u);
  __syncthreads();
  for (uint32_t b = threadIdx.x; b < a.buckets; b += blockDim.x) {
    const uint32_t v = fold[b];
    if (v) atomicAdd(hist + b, v);
  }
}

// Fold copies in global memory (sized to stay in L2): block k uses copy
// k % copies.
__global__ void __launch_bounds__(256)
    fold_global_kernel(HistArgs a, uint32_t *folds, uint32_t copies) {
  uint32_t *fold = folds + (size_t)(blockIdx.x % copies) * a.buckets;
  for (uint64_t e = gtid(); e < a.total; e += gstride()) atomicAdd(fold + hist_key(a, e), 1u);
}

__global__ void __launch_bounds__(256)
    fold_apply_kernel(const uint32_t *folds, uint32_t copies, uint32_t buckets, uint32_t *hist) {
  for (uint64_t b = gtid(); b < buckets; b += gstride()) {
    uint32_t s = 0;
    for (uint32_t f = 0; f < copies; f++) s += __ldcs(folds + (size_t)f * buckets + b);
    if (s) hist[b] += s;
  }
}

// --- list: (pointer, value) entries, then applied ---------------------------
__global__ void __launch_bounds__(256) list_fill_kernel(HistArgs a, uint2 *entries) {
  for (uint64_t e = gtid(); e < a.total; e += gstride())
    entries[e] = make_uint2(hist_key(a, e), 1u);
}

__global__ void __launch_bounds__(256)
    list_apply_kernel(const uint2 *entries, uint64_t n, uint32_t *hist) {
  for (uint64_t i = gtid(); i < n; i += gstride()) {
    const uint2 en = __ldcs(entries + i);
    atomicAdd(hist + en.x, en.y);
  }
}

// --- localize: reductions routed to the owner of their bucket range ---------
constexpr uint32_t kMaxRanges = 4096;
constexpr int kMaxRangeShift = 14;          // 16384 buckets (64 KB) per owner
constexpr size_t kLocAux = 64 * 1024;       // count, base, fill arrays
constexpr int kScatterBlock = 256, kScatterItems = 16;
constexpr int kScatterChunk = kScatterBlock * kScatterItems;
constexpr int kScanBlock = 1024;

// Keys of the round's elements, and the number falling in each range.
__global__ void __launch_bounds__(256)
    loc_key_kernel(HistArgs a, int shift, uint32_t ranges, uint32_t *keys, uint32_t *count) {
  extern __shared__ uint32_t cnt[];
  for (uint32_t s = threadIdx.x; s < ranges; s += blockDim.x) cnt[s] = 0u;
  __syncthreads();
  for (uint64_t e = gtid(); e < a.total; e += gstride()) {
    const uint32_t k = hist_key(a, e);
    keys[e] = k;
    atomicAdd(cnt + (k >> shift), 1u);
  }
  __syncthreads();
  for (uint32_t s = threadIdx.x; s < ranges; s += blockDim.x)
    if (cnt[s]) atomicAdd(count + s, cnt[s]);
}

// Exclusive scan of the per-range counts: base[s] (base[ranges] = total) and
// the scatter cursors fill[s] = base[s].
__global__ void __launch_bounds__(kScanBlock)
    loc_scan_kernel(const uint32_t *count, uint32_t ranges, uint32_t *base, uint32_t *fill) {
  __shared__ uint32_t warp_sum[kScanBlock / 32];
  constexpr uint32_t kPer = kMaxRanges / kScanBlock;  // 4 ranges per thread
  const uint32_t t = threadIdx.x, lane = t & 31, warp = t >> 5;
  uint32_t v[kPer], local = 0;
#pragma unroll
  for (uint32_t j = 0; j < kPer; j++) {
    const uint32_t s = t * kPer + j;
    v[j] = s < ranges ? count[s] : 0u;
    local += v[j];
  }
  uint32_t incl = local;  // inclusive scan of the per-thread sums
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t y = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= (uint32_t)o) incl += y;
  }
  if (lane == 31) warp_sum[warp] = incl;
  __syncthreads();
  if (warp == 0) {
    uint32_t w = warp_sum[lane];
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t y = __shfl_up_sync(0xffffffffu, w, o);
      if (lane >= (uint32_t)o) w += y;
    }
    warp_sum[lane] = w;  // inclusive over warps
  }
  __syncthreads();
  uint32_t run = incl - local + (warp ? warp_sum[warp - 1] : 0u);
#pragma unroll
  for (uint32_t j = 0; j < kPer; j++) {
    const uint32_t s = t * kPer + j;
    if (s < ranges) {
      base[s] = run;
      fill[s] = run;
    }
    run += v[j];
  }
  if (t == kScanBlock - 1) base[ranges] = warp_sum[31];
}

// Moves every key to its range's segment of `sorted` (order inside a segment
// is immaterial: the owners add integers).
__global__ void __launch_bounds__(kScatterBlock)
    loc_scatter_kernel(const uint32_t *keys, uint64_t n, int shift, uint32_t ranges,
                       uint32_t *fill, uint32_t *sorted) {
  extern __shared__ uint32_t sm[];
  uint32_t *cnt = sm, *seg = sm + ranges;
  for (uint32_t s = threadIdx.x; s < ranges; s += blockDim.x) cnt[s] = 0u;
  __syncthreads();
  for (uint64_t c0 = (uint64_t)blockIdx.x * kScatterChunk; c0 < n;
       c0 += (uint64_t)gridDim.x * kScatterChunk) {
    uint32_t k[kScatterItems], r[kScatterItems];
#pragma unroll
    for (int j = 0; j < kScatterItems; j++) {
      const uint64_t i = c0 + (uint64_t)j * kScatterBlock + threadIdx.x;
      if (i < n) {
        k[j] = keys[i];
        r[j] = atomicAdd(cnt + (k[j] >> shift), 1u);
      }
    }
    __syncthreads();
    for (uint32_t s = threadIdx.x; s < ranges; s += blockDim.x) {
      const uint32_t c = cnt[s];
      if (c) {
        seg[s] = atomicAdd(fill + s, c);
        cnt[s] = 0u;
      }
    }
    __syncthreads();
#pragma unroll
    for (int j = 0; j < kScatterItems; j++) {
      const uint64_t i = c0 + (uint64_t)j * kScatterBlock + threadIdx.x;
      if (i < n) sorted[seg[k[j] >> shift] + r[j]] = k[j];
    }
    __syncthreads();
  }
}

// One block per range: copy the target's range into shared memory (the
// local instance), apply the range's reductions there, copy it back.  The
// block is the range's only writer, so neither copy needs atomics.
__global__ void __launch_bounds__(256)
    loc_owner_kernel(const uint32_t *sorted, const uint32_t *base, int shift, uint32_t buckets,
                     uint32_t *hist) {
  extern __shared__ uint32_t local[];
  const uint32_t s = blockIdx.x, lo = s << shift;
  const uint32_t nb = min(1u << shift, buckets - lo);
  for (uint32_t j = threadIdx.x; j < nb; j += blockDim.x) local[j] = hist[lo + j];
  __syncthreads();
  const uint32_t end = base[s + 1];
  for (uint32_t i = base[s] + threadIdx.x; i < end; i += blockDim.x)
    atomicAdd(local + (sorted[i] - lo), 1u);
  __syncthreads();
  for (uint32_t j = threadIdx.x; j < nb; j += blockDim.x) hist[lo + j] = local[j];
}

// --- host side ---------------------------------------------------------------
struct Plan {
  uint64_t total = 0, min_bytes = 0, good_bytes = 0;
  bool smem_fold = false;
  int shift = 0;        // localize: log2 of the buckets per range
  uint32_t ranges = 0;  // localize: number of ranges
};

int sm_count(int *out) {
  int dev = 0;
  CKT_CUDA(cudaGetDevice(&dev));
  CKT_CUDA(cudaDeviceGetAttribute(out, cudaDevAttrMultiProcessorCount, dev));
  return CKT_OK;
}

constexpr uint64_t kL2Budget = 32ull << 20;  // scratch worth keeping in L2 per round

int make_plan(const ckt_hist_params *p, int32_t schedule, Plan *pl) {
  CKT_REQUIRE(p != nullptr, "params is NULL");
  CKT_REQUIRE(p->buckets >= 1 && p->buckets <= (1u << 30), "buckets must be in [1, 2^30] (got %u)",
              p->buckets);
  CKT_REQUIRE(schedule >= CKT_RED_SINGLE && schedule <= CKT_RED_LIST, "unknown schedule %d",
              schedule);
  pl->total = (uint64_t)p->batch_size * p->num_batches;
  const uint64_t hist_bytes = 4ull * p->buckets;
  switch (schedule) {
    case CKT_RED_SINGLE:
      break;
    case CKT_RED_FOLD:
      pl->smem_fold = p->buckets <= CKT_HIST_SMEM_FOLD_BUCKETS;
      if (!pl->smem_fold) {
        const uint64_t copies = std::max<uint64_t>(1, std::min<uint64_t>(8, kL2Budget / hist_bytes));
        pl->min_bytes = hist_bytes;
        pl->good_bytes = copies * hist_bytes;
      }
      break;
    case CKT_RED_LOCALIZE: {
      CKT_REQUIRE(p->buckets <= CKT_HIST_LOCALIZE_MAX_BUCKETS,
                  "localize supports at most %u buckets (got %u)",
                  (unsigned)CKT_HIST_LOCALIZE_MAX_BUCKETS, p->buckets);
      int smc = 0, rc;
      if ((rc = sm_count(&smc))) return rc;
      // ranges of a power-of-two size: about two owners per SM, at most
      // 16384 buckets (64 KB of shared memory) each
      const uint64_t want = std::max<uint64_t>(1, (p->buckets + 2ull * smc - 1) / (2ull * smc));
      int shift = 0;
      while ((1ull << shift) < want && shift < kMaxRangeShift) shift++;
      while (((uint64_t)p->buckets + (1ull << shift) - 1) >> shift > kMaxRanges) shift++;
      pl->shift = shift;
      pl->ranges = (uint32_t)(((uint64_t)p->buckets + (1ull << shift) - 1) >> shift);
      pl->min_bytes = kLocAux + 8ull * kScatterChunk;
      pl->good_bytes = kLocAux + 8ull * std::min<uint64_t>(pl->total, kL2Budget / 4);
      break;
    }
    case CKT_RED_LIST:
      pl->min_bytes = 8ull * p->batch_size;
      pl->good_bytes =
          8ull * p->batch_size *
          std::max<uint64_t>(1, std::min<uint64_t>(p->num_batches,
                                                   (2 * kL2Budget) / std::max<uint64_t>(1, 8ull * p->batch_size)));
      break;
  }
  pl->good_bytes = std::max(pl->good_bytes, pl->min_bytes);
  return CKT_OK;
}

unsigned grid_persistent(int smc, uint64_t work_items, int block, int per_sm) {
  const uint64_t need = (work_items + block - 1) / block;
  const uint64_t cap = (uint64_t)smc * per_sm;
  return (unsigned)std::max<uint64_t>(1, std::min(need, cap));
}

}  // namespace
}  // namespace ckt

using namespace ckt;

extern "C" {

void ckt_hist_default_params(ckt_hist_params *out) {
  if (!out) return;
  out->buckets = 1048576;
  out->batch_size = 1048576;
  out->num_batches = 1024;
  out->first_batch = 0;
  out->seed1 = 12345;
  out->seed2 = 54321;
}

int ckt_hist_scratch_bytes(const ckt_hist_params *p, int32_t schedule, uint64_t *min_bytes,
                           uint64_t *good_bytes) {
  Plan pl;
  int rc;
  if ((rc = make_plan(p, schedule, &pl))) return rc;
  if (min_bytes) *min_bytes = pl.min_bytes;
  if (good_bytes) *good_bytes = pl.good_bytes;
  return CKT_OK;
}

int ckt_hist_run(const ckt_hist_params *p, int32_t schedule, uint32_t *hist, void *scratch,
                 uint64_t scratch_bytes, void *stream) {
  NvtxRange range("ckt_hist_run");
  Plan pl;
  int rc;
  if ((rc = make_plan(p, schedule, &pl))) return rc;
  CKT_REQUIRE(hist != nullptr, "hist is NULL");
  if (pl.total == 0) return CKT_OK;
  if (pl.min_bytes) {
    CKT_REQUIRE(scratch != nullptr, "schedule %d needs scratch memory", schedule);
    CKT_REQUIRE((reinterpret_cast<uintptr_t>(scratch) & 15u) == 0,
                "scratch must be 16-byte aligned");
    CKT_REQUIRE(scratch_bytes >= pl.min_bytes,
                "scratch of %llu bytes is below schedule %d's minimum of %llu",
                (unsigned long long)scratch_bytes, schedule, (unsigned long long)pl.min_bytes);
  }
  int smc = 0;
  if ((rc = sm_count(&smc))) return rc;
  const cudaStream_t s = as_stream(stream);
  HistArgs a;
  a.base = p->first_batch * p->batch_size;  // 32-bit unsigned, as the benchmark's start
  a.buckets = p->buckets;
  a.total = pl.total;
  a.seed1 = p->seed1;
  a.seed2 = p->seed2;
  a.mod_magic = UINT64_MAX / p->buckets + 1;

  switch (schedule) {
    case CKT_RED_SINGLE: {
      single_kernel<<<grid_persistent(smc, a.total, 256, 8), 256, 0, s>>>(a, hist);
      CKT_CHECK_LAUNCH();
      break;
    }
    case CKT_RED_FOLD: {
      if (pl.smem_fold) {
        const size_t smem = 4ull * p->buckets;
        CKT_CUDA(cudaFuncSetAttribute(fold_smem_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      (int)(4 * CKT_HIST_SMEM_FOLD_BUCKETS)));
        int per_sm = 0;
        CKT_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fold_smem_kernel,
                                                               kFoldBlock, smem));
        fold_smem_kernel<<<grid_persistent(smc, a.total, kFoldBlock, std::max(per_sm, 1)),
                           kFoldBlock, smem, s>>>(a, hist);
        CKT_CHECK_LAUNCH();
      } else {
        const uint64_t hist_bytes = 4ull * p->buckets;
        const uint32_t copies = (uint32_t)std::min<uint64_t>(8, scratch_bytes / hist_bytes);
        uint32_t *folds = static_cast<uint32_t *>(scratch);
        CKT_CUDA(cudaMemsetAsync(folds, 0, copies * hist_bytes, s));  // identity
        fold_global_kernel<<<grid_persistent(smc, a.total, 256, 8), 256, 0, s>>>(a, folds, copies);
        CKT_CHECK_LAUNCH();
        fold_apply_kernel<<<grid_persistent(smc, p->buckets, 256, 8), 256, 0, s>>>(
            folds, copies, p->buckets, hist);
        CKT_CHECK_LAUNCH();
      }
      break;
    }
    case CKT_RED_LIST: {
      // rounds of whole batches: each batch's list is complete before it is
      // applied, as the benchmark's copy_to applies a finished list
      const uint64_t per_round =
          std::max<uint64_t>(1, std::min<uint64_t>(p->num_batches,
                                                   scratch_bytes / (8ull * p->batch_size)));
      uint2 *entries = static_cast<uint2 *>(scratch);
      for (uint64_t b = 0; b < p->num_batches; b += per_round) {
        const uint64_t nb = std::min<uint64_t>(per_round, p->num_batches - b);
        HistArgs r = a;
        r.base = a.base + (uint32_t)(b * p->batch_size);
        r.total = nb * p->batch_size;
        list_fill_kernel<<<grid_persistent(smc, r.total, 256, 8), 256, 0, s>>>(r, entries);
        CKT_CHECK_LAUNCH();
        list_apply_kernel<<<grid_persistent(smc, r.total, 256, 8), 256, 0, s>>>(entries, r.total,
                                                                              hist);
        CKT_CHECK_LAUNCH();
      }
      break;
    }
    case CKT_RED_LOCALIZE: {
      char *base_ptr = static_cast<char *>(scratch);
      uint32_t *count = reinterpret_cast<uint32_t *>(base_ptr);
      uint32_t *seg_base = count + kMaxRanges;
      uint32_t *fill = seg_base + kMaxRanges + 64;
      const uint64_t cap = ((scratch_bytes - kLocAux) / 8) & ~uint64_t(3);
      const uint64_t per_round = std::min<uint64_t>(cap, std::min<uint64_t>(a.total, 1ull << 31));
      uint32_t *keys = reinterpret_cast<uint32_t *>(base_ptr + kLocAux);
      uint32_t *sorted = keys + per_round;
      const size_t owner_smem = 4ull << pl.shift;
      CKT_CUDA(cudaFuncSetAttribute(loc_owner_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    (int)(4u << kMaxRangeShift)));
      for (uint64_t e0 = 0; e0 < a.total; e0 += per_round) {
        HistArgs r = a;
        r.base = a.base + (uint32_t)e0;
        r.total = std::min<uint64_t>(per_round, a.total - e0);
        CKT_CUDA(cudaMemsetAsync(count, 0, 4ull * pl.ranges, s));
        loc_key_kernel<<<grid_persistent(smc, r.total, 256, 8), 256, 4ull * pl.ranges, s>>>(
            r, pl.shift, pl.ranges, keys, count);
        CKT_CHECK_LAUNCH();
        loc_scan_kernel<<<1, kScanBlock, 0, s>>>(count, pl.ranges, seg_base, fill);
        CKT_CHECK_LAUNCH();
        loc_scatter_kernel<<<grid_persistent(smc, r.total, kScatterChunk, 4), kScatterBlock,
                             8ull * pl.ranges, s>>>(keys, r.total, pl.shift, pl.ranges, fill,
                                                    sorted);
        CKT_CHECK_LAUNCH();
        loc_owner_kernel<<<pl.ranges, 256, owner_smem, s>>>(sorted, seg_base, pl.shift,
                                                            p->buckets, hist);
        CKT_CHECK_LAUNCH();
      }
      break;
    }
  }
  return CKT_OK;
}

}  // extern "C"
