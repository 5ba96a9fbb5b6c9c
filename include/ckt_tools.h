/*
 * ckt_tools.h -- measurement and verification helpers of the circuit
 * library, built into their own shared library (libckt_tools.so) beside the
 * product library libckt.so.  No counterpart in the reference.  Same
 * conventions as ckt.h: plain pointers, a ckt_status return, streams passed
 * as void * (NULL: the legacy default stream), device pointers where noted.
 */
#ifndef CKT_TOOLS_H
#define CKT_TOOLS_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* FP32 FMA throughput probe: launches `blocks` x 256 threads, each
 * performing iters*16*8 independent fused multiply-adds (2 flops each) -- as
 * single FMAs, or with `paired` != 0 as paired (f32x2) FMAs doing two each;
 * time it on `stream` to get the device's FP32-pipe peak, the roofline
 * denominator of calc_new_currents.  `sink` is a device float it may write. */
int ckt_fp32_fma_probe(uint32_t blocks, int32_t iters, int32_t paired, float *sink, void *stream);

/* The split-reciprocal quotient by dt = (float)1e-6 that EXACT mode's
 * calc_new_currents uses, against the divide routine (__fdiv_rn), for every
 * float dividend whose bit pattern lies in [begin, begin + count) (count up
 * to 2^32).  Adds to counts[0] the mismatches among the dividends the kernel
 * uses it for (magnitude >= 2^-118, zeros, infinities, NaN) and to counts[1]
 * those among the rest; equal means equal bits or both NaN.  `counts` is
 * device memory (2 x uint64), asynchronous on `stream`. */
int ckt_check_dt_quotient(uint64_t begin, uint64_t count, unsigned long long *counts,
                          void *stream);

/* The corrected quotient by a per-wire divisor (RN(1/b) and RN(1/b - RN(1/b))
 * with one correction step) with its guard, as EXACT mode uses it, against
 * __fdiv_rn on `count` pseudo-random (a, b) pairs drawn from `seed`.
 * divisor 0: b in the resistance range the kernel accepts ([2^-8, 2^8] in
 * magnitude), 1: the capacitance and general-dt range ([2^-30, 2^30]).
 * Dividends: any float (random exponents, signs, zeros, subnormals,
 * infinities, NaN, the guard's edges) or, with near_ties != 0, values whose
 * quotient lies within a few ulps of a rounding boundary of the inner range.
 * Adds to counts[0] the mismatches, to counts[1] the pairs that took the
 * corrected quotient, to counts[2] the pairs drawn (device memory, 3 x
 * uint64; asynchronous on `stream`). */
int ckt_check_recip_quotient(uint64_t seed, uint64_t count, int32_t divisor, int32_t near_ties,
                             unsigned long long *counts, void *stream);

/* The quotient EXACT mode takes for the dividends outside that range
 * (scaled by a power of two into it; zeros and infinities times the
 * reciprocal) against __fdiv_rn on `count` pseudo-random pairs: dividends
 * huge up to FLT_MAX, tiny down to the smallest subnormal (but not so tiny
 * that the quotient may be subnormal: |a| >= 2^-125 |b|), in range, zero,
 * infinite, NaN, or with a quotient within an ulp of a rounding boundary or
 * of overflowing.  Adds to counts[0] the mismatches,
 * to counts[1] the pairs outside the guarded range, to counts[2] the pairs
 * drawn. */
int ckt_check_wide_quotient(uint64_t seed, uint64_t count, int32_t divisor,
                            unsigned long long *counts, void *stream);

#ifdef __cplusplus
}
#endif
#endif /* CKT_TOOLS_H */
