/*
 * ckt_oracle.h -- CPU oracle for the circuit simulator's per-loop hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This is a plain-C restatement of the reference
 * circuit application (LegionOrigins apps/circuit) used to CHECK the CUDA
 * library: only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline
 * leg may load it.  The product library never links or calls it.
 *
 * Parity pin: the generator and the three CPU leaf tasks are checked
 * bit-for-bit against the reference's own apps/circuit/circuit.cc compiled
 * through oracle/refshim (a minimal Legion-API shim); see oracle/Makefile
 * and tests/golden/make_golden.py.
 *
 * What each function restates (reference file:line):
 *   ocl_generate        apps/circuit/circuit.cc:1071-1288 (load_circuit),
 *                       :1042-1049 (random_element), :1051-1069 (find_location)
 *   ocl_cnc_f32/_f64    apps/circuit/circuit_gpu.cu:61-149 (canonical init) and
 *                       apps/circuit/circuit.cc:352-413 (quirk init)
 *   ocl_dc_f32/_f64     apps/circuit/circuit.cc:415-443, :98-116, :18-68 with the
 *                       reduction-instance fold/apply order of
 *                       runtime/lowlevel.h:475-492 (pieces applied ascending)
 *   ocl_uv_f32/_f64     apps/circuit/circuit.cc:445-460, :1290-1307
 *   ocl_split_quotient_check, ocl_wide_quotient_check
 *                       the division by dt of apps/circuit/circuit.cc:391-393
 *                       as the GPU's EXACT mode forms it (split reciprocal),
 *                       against IEEE division, over ranges of dividends
 *   ocl_baseline_run    the shared-low-level CPU execution of the same three
 *                       tasks: one pthread per core, piece p on thread p mod T
 *                       (apps/circuit/circuit.cc:623-635), barriers between
 *                       index launches, 128-byte wires copied by value
 *                       (runtime/shared_lowlevel.cc:2812-2829).
 */
#ifndef CKT_ORACLE_H
#define CKT_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define OCL_SEGMENTS 10

enum { OCL_PRIVATE = 0, OCL_SHARED = 1, OCL_GHOST = 2 };

typedef struct {
  int32_t num_pieces;
  int32_t nodes_per_piece;
  int32_t wires_per_piece;
  int32_t pad0;
  double pct_wire_in_piece; /* compared as (100*drand48()) < pct */
  int64_t random_seed;
  double L_offset;          /* reference: 0.1  (circuit.cc:1163)  */
  double L_scale;           /* reference: 0.01 (circuit.cc:1163)  */
} ocl_params;

/* Generator.  Arrays are caller-allocated: W = P*wpp wires, N = P*npp nodes.
 * Wires and nodes are numbered piece-major as the reference allocates them. */
int ocl_generate(const ocl_params *p,
                 uint32_t *in_ptr, uint32_t *out_ptr,
                 uint8_t *in_loc, uint8_t *out_loc,
                 float *wire_L, float *wire_R, float *wire_C,
                 float *node_charge, float *node_voltage,
                 float *node_cap, float *node_leak,
                 int32_t *locator);

/* calc_new_currents over wires [w_begin, w_end).  current is segment-major
 * [10][stride], voltage [9][stride].  quirk=1 reproduces the CPU task's
 * initialisation (new_v[i]=V0[i] for i<9, new_v[9]:=0), quirk=0 the GPU
 * kernel's (new_v[0]=V(in), new_v[i+1]=V0[i]). */
void ocl_cnc_f32(int64_t w_begin, int64_t w_end, int64_t stride,
                 const uint32_t *in_ptr, const uint32_t *out_ptr,
                 const float *L, const float *R, const float *C,
                 float *current, float *voltage,
                 const float *node_voltage, int32_t steps, int32_t quirk);
void ocl_cnc_f64(int64_t w_begin, int64_t w_end, int64_t stride,
                 const uint32_t *in_ptr, const uint32_t *out_ptr,
                 const double *L, const double *R, const double *C,
                 double *current, double *voltage,
                 const double *node_voltage, int32_t steps, int32_t quirk);

/* distribute_charge for pieces 0..P-1 (piece k = wires
 * [first_wire[k], first_wire[k]+num_wires[k])).  Private endpoints are
 * applied to charge in wire order; shared/ghost endpoints fold into a
 * per-piece buffer (identity 0) that is applied after the piece, pieces
 * ascending.  scratch must hold N floats and be zero on entry (left zero). */
void ocl_dc_f32(int32_t P, const int64_t *first_wire, const int64_t *num_wires,
                int64_t stride, const uint32_t *in_ptr, const uint32_t *out_ptr,
                const uint8_t *in_loc, const uint8_t *out_loc,
                const float *current, float *node_charge, int64_t N,
                float *scratch);
void ocl_dc_f64(int32_t P, const int64_t *first_wire, const int64_t *num_wires,
                int64_t stride, const uint32_t *in_ptr, const uint32_t *out_ptr,
                const uint8_t *in_loc, const uint8_t *out_loc,
                const double *current, double *node_charge, int64_t N,
                double *scratch);

/* update_voltages over nodes [n_begin, n_end). */
void ocl_uv_f32(int64_t n_begin, int64_t n_end, float *charge, float *voltage,
                const float *cap, const float *leak);
void ocl_uv_f64(int64_t n_begin, int64_t n_end, double *charge, double *voltage,
                const double *cap, const double *leak);

/* Whole simulation in fp32 or fp64 on SoA state (serial, canonical order). */
void ocl_simulate_f32(const ocl_params *p, int32_t loops, int32_t steps, int32_t quirk,
                      const uint32_t *in_ptr, const uint32_t *out_ptr,
                      const uint8_t *in_loc, const uint8_t *out_loc,
                      const float *L, const float *R, const float *C,
                      float *current, float *voltage,
                      float *node_charge, float *node_voltage,
                      const float *node_cap, const float *node_leak);
void ocl_simulate_f64(const ocl_params *p, int32_t loops, int32_t steps, int32_t quirk,
                      const uint32_t *in_ptr, const uint32_t *out_ptr,
                      const uint8_t *in_loc, const uint8_t *out_loc,
                      const double *L, const double *R, const double *C,
                      double *current, double *voltage,
                      double *node_charge, double *node_voltage,
                      const double *node_cap, const double *node_leak);

/* Multithreaded CPU baseline in the reference's CPU execution style.
 * Runs `loops` outer loops of the three tasks over pieces [0, piece_limit)
 * with `threads` pthreads (piece p on thread p % threads) and returns the
 * elapsed seconds of the main loop only (packing to the 128-byte AoS wire
 * layout and back is outside the timed region).  State arrays are SoA as in
 * ocl_simulate_f32 and are updated in place.  Returns a negative value on
 * error. */
double ocl_baseline_run(const ocl_params *p, int32_t loops, int32_t steps,
                        int32_t threads, int32_t piece_limit, int32_t quirk,
                        const uint32_t *in_ptr, const uint32_t *out_ptr,
                        const uint8_t *in_loc, const uint8_t *out_loc,
                        const float *L, const float *R, const float *C,
                        float *current, float *voltage,
                        float *node_charge, float *node_voltage,
                        const float *node_cap, const float *node_leak);

/* ---- Reduction microbenchmark (benchmarks/reductions/reducetest.cc) ---- */

/* myrand (reducetest.cc:323-333): 16 rounds of the 48-bit LCG
 * r <- (0x5DEECE66D r + 0xB) mod 2^48, each followed by r ^= seed1 when bit
 * j of ival is set, else seed2; the low 32 bits of r. */
uint32_t ocl_hist_rand(uint64_t ival, uint32_t seed1, uint32_t seed2);

/* The histogram every reducetest case adds into its master instance: for
 * batches b = first_batch .. first_batch+num_batches-1 and i < batch_size,
 * hist[myrand(start + i) % buckets] += 1, with start = b * batch_size and
 * start + i both 32-bit unsigned as in the benchmark (reducetest.cc:174,
 * 341-347).  Adds into hist (it is not cleared). */
void ocl_histogram(uint32_t buckets, uint32_t batch_size, uint32_t num_batches,
                   uint32_t first_batch, uint32_t seed1, uint32_t seed2, uint32_t *hist);

/* The same histogram on `threads` pthreads in the benchmark's fastest CPU
 * schedule (redfold, reducetest.cc:378-400): batch b runs on thread
 * b % threads, which reduces into its own fold instance (identity 0) and
 * applies it to hist under a mutex when it is done.  Returns the elapsed
 * seconds, or a negative value on error. */
double ocl_histogram_threads(uint32_t buckets, uint32_t batch_size, uint32_t num_batches,
                             uint32_t first_batch, uint32_t seed1, uint32_t seed2,
                             int32_t threads, uint32_t *hist);

void ocl_split_quotient_check(uint64_t lo, uint64_t hi, float dt, float zh, float zl, float tiny,
                              uint64_t *bad_trusted, uint64_t *bad_other);

/* EXACT mode's quotient by R or C for dividends outside the corrected
 * quotient's guarded range, against IEEE division, on random pairs of every
 * dividend class (see the definition). */
void ocl_wide_quotient_check(uint64_t seed, uint64_t n, int divisor, uint64_t *bad,
                             uint64_t *outside, uint64_t *drawn);

#ifdef __cplusplus
}
#endif
#endif
