/*
 * ckt.h -- C ABI of the GB300-native circuit hot path.
 *
 * Drop-in CUDA variants of the three leaf tasks of LegionOrigins' circuit
 * simulator (apps/circuit), for sm_103a.  Plain pointers and sizes only: no
 * CUDA, torch or C++ types cross this boundary (streams are passed as
 * `void *` holding a cudaStream_t; NULL means the legacy default stream).
 *
 * Data contract (apps/circuit/circuit.h:13-76):
 *   - node and wire "pointers" are 32-bit absolute indices into their
 *     regions (runtime/common.h:11-52, apps/circuit/circuit.h:46-47);
 *   - a piece owns the contiguous wire range [first_wire, first_wire +
 *     num_wires) and node range [first_node, first_node + num_nodes)
 *     (apps/circuit/circuit.cc:1270-1280);
 *   - region instances are structure-of-arrays views indexed by absolute
 *     index, the role GPU_Accessor's array_base plays in the reference
 *     (runtime/lowlevel.h:749-833); per-segment wire arrays are
 *     segment-major with a caller-given stride;
 *   - each wire has CKT_SEGMENTS = 10 segments (circuit.h:42).
 *
 * Every entry point returns a ckt_status; none asserts, traps or exits.
 * ckt_last_error() describes the last failure on the calling thread.
 */
#ifndef CKT_H
#define CKT_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define CKT_SEGMENTS 10
#define CKT_ABI_VERSION 1

typedef enum {
  CKT_OK = 0,
  CKT_EINVAL = 1,    /* bad argument */
  CKT_ECUDA = 2,     /* a CUDA call failed */
  CKT_EBOUNDS = 3,   /* a pointer or location failed validation */
  CKT_ETIMEOUT = 4,  /* a bounded device wait ran out */
  CKT_ENOMEM = 5,    /* allocation refused (budget or device) */
  CKT_EBUSY = 6,     /* no free slot / queue full */
  CKT_ECANCELLED = 7 /* request cancelled */
} ckt_status;

/* PointerLocation (apps/circuit/circuit.h:12-16). */
typedef enum { CKT_PRIVATE_PTR = 0, CKT_SHARED_PTR = 1, CKT_GHOST_PTR = 2 } ckt_pointer_location;

/* Arithmetic of calc_new_currents. */
typedef enum {
  /* IEEE fp32 exactly as the reference writes it (correctly rounded
   * divides, no contraction): bit-identical to the reference CPU task.  Its
   * divisors (dt, R, C) are loop-invariant, so each wire carries their
   * reciprocals and every quotient is formed from them and corrected to the
   * IEEE quotient (Markstein's theorem); dividends where that construction
   * is not proven exact, and wires whose divisors lie outside its range, use
   * the divide routine.  Two wires per thread, paired FP32 instructions. */
  CKT_MODE_EXACT = 0,
  /* Loop-invariant quotients L/dt, 1/R and dt/C hoisted out of the inner
   * loop, each current carried before its 1/R scale, fused multiply-adds:
   * 48 FP32 operations per wire-step, within 1e-5 relative of EXACT in the
   * finite regime and with its NaN/Inf classes.  Issued as paired FP32
   * instructions (two wires per instruction in the per-piece and
   * index-space kernels, two segments in the batched kernel). */
  CKT_MODE_FAST = 1,
  /* FAST arithmetic issued one operation per instruction: bit-identical to
   * CKT_MODE_FAST (kept to check the paired forms and to measure them). */
  CKT_MODE_FAST_SCALAR = 2,
  /* CKT_MODE_EXACT with every quotient from the divide routine, one wire
   * per thread: the same bits (kept to check CKT_MODE_EXACT and to measure
   * it against). */
  CKT_MODE_EXACT_DIVIDE = 3
} ckt_mode;

/* Wire initialisation of calc_new_currents. */
typedef enum {
  /* GPU task semantics (apps/circuit/circuit_gpu.cu:107-112): new_v[0] =
   * in-node voltage, new_v[i+1] = wire.voltage[i]. */
  CKT_INIT_KERNEL = 0,
  /* CPU task semantics (apps/circuit/circuit.cc:380-384): new_v[i] =
   * wire.voltage[i] for i < 9, new_v[9] read before written (defined here
   * as 0), in-node voltage unused. */
  CKT_INIT_CPU_TASK = 1
} ckt_init;

/* CircuitPiece (apps/circuit/circuit.h:62-69) minus its region handles. */
typedef struct {
  uint32_t first_wire;
  uint32_t num_wires;
  uint32_t first_node;
  uint32_t num_nodes;
} ckt_piece;

/* Wire region instance (CircuitWire, apps/circuit/circuit.h:46-54), SoA.
 * current[k*seg_stride + w] is segment k of wire w (k < 10); voltage has 9
 * segments.  All pointers are device pointers. */
typedef struct {
  const uint32_t *in_ptr;
  const uint32_t *out_ptr;
  const uint8_t *in_loc;
  const uint8_t *out_loc;
  const float *inductance;
  const float *resistance;
  const float *capacitance;
  float *current;
  float *voltage;
  int64_t seg_stride;
} ckt_wires;

/* Node region instance (CircuitNode, apps/circuit/circuit.h:35-40), SoA,
 * absolute node index.  Device pointers. */
typedef struct {
  float *charge;
  float *voltage;
  const float *capacitance;
  const float *leakage;
} ckt_nodes;

typedef struct {
  int32_t steps; /* inner steps (STEPS, circuit.h:43; a runtime value here) */
  float dt;      /* DELTAT (circuit.h:44) = (float)1e-6 */
  int32_t mode;  /* ckt_mode */
  int32_t init;  /* ckt_init */
} ckt_params;

/* Static contribution graph of one circuit: for every node, the wire ends
 * that deposit charge on it, in the reference's reduction order.  Built once
 * from the wire endpoints (the role the runtime's region tree and reduction
 * instances play in the reference). */
typedef struct ckt_graph ckt_graph;

/* ------------------------------------------------------------------------
 * Library
 * ---------------------------------------------------------------------- */
int ckt_abi_version(void);
const char *ckt_last_error(void);
const char *ckt_status_string(int status);
/* Default parameters: steps 10000, dt (float)1e-6, EXACT, KERNEL init. */
void ckt_default_params(ckt_params *out);

/* ------------------------------------------------------------------------
 * The three leaf tasks, per piece (drop-in for the reference's GPU task
 * bodies).  Asynchronous on `stream`.
 * ---------------------------------------------------------------------- */

/* Replaces calc_new_currents_gpu (apps/circuit/circuit.h:83-88,
 * apps/circuit/circuit_gpu.cu:186-205).  Reads in/out node voltages from
 * pvt, shr or ghost by the wire's location (circuit_gpu.cu:40-59); writes
 * current[10] and voltage[9] of every wire of the piece. */
int ckt_calc_new_currents(const ckt_piece *piece, ckt_wires wires, ckt_nodes pvt,
                          ckt_nodes shr, ckt_nodes ghost, const ckt_params *prm,
                          void *stream);

/* Replaces distribute_charge_gpu (apps/circuit/circuit.h:90-95,
 * apps/circuit/circuit_gpu.cu:245-304).  Deposits -dt*I[0] on the in-node
 * and +dt*I[9] on the out-node of each wire of piece `piece_index` of
 * `graph`: private nodes' charge is updated in place in wire order
 * (apply<true>); shared and ghost nodes fold into `shr_fold` / `ghost_fold`
 * (float per absolute node index, the reduction instances of
 * runtime/lowlevel.h:835-881) in wire order.  Deterministic: no atomics.
 * Like the reference's per-task reduction instances, the folds must hold
 * the identity (0) for every node this piece touches: give each piece its
 * own fold buffers, or apply this piece's folds with ckt_apply_fold (which
 * resets them) before the next piece deposits into the same buffers. */
int ckt_distribute_charge(const ckt_graph *graph, int32_t piece_index, ckt_wires wires,
                          ckt_nodes pvt, float *shr_fold, float *ghost_fold,
                          const ckt_params *prm, void *stream);

/* Replaces distribute_charge_gpu (apps/circuit/circuit.h:90-95,
 * apps/circuit/circuit_gpu.cu:219-304) with the reference's own arguments:
 * the piece and its instances, no contribution graph.  Each wire of the
 * piece adds -dt*I[0] to its in-node and +dt*I[9] to its out-node with
 * atomic adds: private nodes' charge in `pvt` directly (apply), shared and
 * ghost nodes into `shr_fold` / `ghost_fold` (fold; float per absolute node
 * index, holding the identity 0 on entry as a fresh reduction instance
 * does).  Lanes of a warp whose ends land on the same node combine their
 * contributions first, so a heavily shared node takes one atomic per warp.
 * Like the reference's atomicAdd, the order of the additions at a node is
 * unspecified: sums may differ in the last bits from run to run and from the
 * deterministic ckt_distribute_charge.  Wires must pass
 * ckt_sanity_check_wires (locations in {0,1,2}, pointers inside their
 * instances); nothing else is checked on the device. */
int ckt_distribute_charge_atomic(const ckt_piece *piece, ckt_wires wires, ckt_nodes pvt,
                                 float *shr_fold, float *ghost_fold, const ckt_params *prm,
                                 void *stream);

/* The runtime's application of piece `piece_index`'s reduction instances
 * (runtime/lowlevel_dma.cc:323-355): charge[x] += fold[x] for every shared
 * or ghost node the piece touched, then fold[x] = 0.  Call pieces in
 * ascending order to reproduce the reference's canonical reduction. */
int ckt_apply_fold(const ckt_graph *graph, int32_t piece_index, float *shr_fold,
                   float *ghost_fold, float *charge, void *stream);

/* Replaces update_voltages_gpu (apps/circuit/circuit.h:97-101,
 * apps/circuit/circuit_gpu.cu:306-368): for every node of the piece,
 * choose pvt or shr by locator[x] (1 private, 0 shared), then
 * v += q/C; v *= (1 - leak); q = 0. */
int ckt_update_voltages(const ckt_piece *piece, ckt_nodes pvt, ckt_nodes shr,
                        const int32_t *locator, void *stream);

/* Blocking forms of the three tasks, with the reference's synchronous
 * semantics: its GPU task bodies return only after cudaDeviceSynchronize
 * (apps/circuit/circuit_gpu.cu:204, 303, 367).  Each launches exactly like
 * its asynchronous form, then waits for `stream` and returns CKT_ECUDA when
 * the launch or the work on the device failed. */
int ckt_calc_new_currents_sync(const ckt_piece *piece, ckt_wires wires, ckt_nodes pvt,
                               ckt_nodes shr, ckt_nodes ghost, const ckt_params *prm,
                               void *stream);
int ckt_distribute_charge_sync(const ckt_graph *graph, int32_t piece_index, ckt_wires wires,
                               ckt_nodes pvt, float *shr_fold, float *ghost_fold,
                               const ckt_params *prm, void *stream);
int ckt_update_voltages_sync(const ckt_piece *piece, ckt_nodes pvt, ckt_nodes shr,
                             const int32_t *locator, void *stream);
int ckt_distribute_charge_atomic_sync(const ckt_piece *piece, ckt_wires wires, ckt_nodes pvt,
                                      float *shr_fold, float *ghost_fold, const ckt_params *prm,
                                      void *stream);

/* Replaces sanity_check_wires_gpu (apps/circuit/circuit.h:103-104,
 * apps/circuit/circuit_gpu.cu:151-217) without its asserts: validates every
 * wire of the piece (locations in range, in-node inside the piece,
 * private/shared out-node inside the piece, ghost out-node outside it and
 * below num_nodes_total).  Synchronises `stream`; returns CKT_EBOUNDS and
 * stores the first bad wire in *first_bad (or -1) when a check fails. */
int ckt_sanity_check_wires(const ckt_piece *piece, ckt_wires wires, uint32_t num_nodes_total,
                           int64_t *first_bad, void *stream);

/* Allocation-free wire check.  No counterpart in the reference.
 * Checks pieces[0..num_pieces) in one launch, giving for each piece what
 * ckt_sanity_check_wires gives for it (first_bad[k]: smallest failing wire
 * of piece k, or -1), but allocates nothing -- neither device nor host
 * memory.  For callers that cannot allocate: a runtime that reserves the
 * GPU's memory for its own pools at start-up, code that must not call
 * cudaMalloc/cudaFree because they can synchronise the device, a process
 * held to a fixed memory budget.  Its scratch is one fixed array of
 * CKT_NOALLOC_MAX_PIECES slots (24 bytes each, 96 KB) that every GPU loading
 * the library holds until the process exits.
 *  - num_pieces above CKT_NOALLOC_MAX_PIECES is rejected with CKT_EINVAL.
 *  - Every call looks up the array's device address on the calling
 *    thread's current device; the first call on a device also loads the
 *    library's module there, so make it before any stream capture.
 *  - Every call uses the same array and leaves its contents behind (each
 *    call re-initialises what it reads).  Calls that overlap on the GPU --
 *    other streams, other host threads -- race on it: serialise them.
 *  - Synchronises `stream`; returns CKT_EBOUNDS when any piece fails. */
#define CKT_NOALLOC_MAX_PIECES 4096
int ckt_sanity_check_pieces_noalloc(const ckt_piece *pieces, int32_t num_pieces, ckt_wires wires,
                                    uint32_t num_nodes_total, int64_t *first_bad, void *stream);

/* ------------------------------------------------------------------------
 * Index-space launches: one launch per task over all pieces of a circuit
 * (the three execute_index_space calls of apps/circuit/circuit.cc:250-298),
 * bit-identical to running the per-piece calls in piece order followed by
 * ckt_apply_fold in piece order.
 * ---------------------------------------------------------------------- */
int ckt_calc_new_currents_all(const ckt_graph *graph, ckt_wires wires, ckt_nodes nodes,
                              const ckt_params *prm, void *stream);
/* ckt_distribute_charge_all and ckt_distribute_update_all launch two
 * kernels: one packs the currents of the graph's sparse contributions (in
 * the benchmark circuits, wires ending in another piece) into a buffer the
 * graph owns, and the tiled pass reads them from there.  Calls on one graph
 * may come from several streams and host threads: each pass made on another
 * stream than the previous pass on the graph first waits for that pass, in
 * the order the calls are made.  Inside a stream capture the calls add no
 * such wait, and the captured graph must not overlap other passes on the same
 * ckt_graph. */
int ckt_distribute_charge_all(const ckt_graph *graph, ckt_wires wires, ckt_nodes nodes,
                              const ckt_params *prm, void *stream);
int ckt_update_voltages_all(const ckt_graph *graph, ckt_nodes nodes, void *stream);

/* distribute_charge and update_voltages over all pieces fused into one node
 * pass (no counterpart in the reference, whose tasks meet only through
 * region instances): each node gathers its contributions as
 * ckt_distribute_charge_all does and feeds the sum straight into the
 * voltage update.  Bit-identical to ckt_distribute_charge_all followed by
 * ckt_update_voltages_all.  ckt_run_loops_all runs `loops` outer loops of
 * region_main (apps/circuit/circuit.cc:232-307) as ckt_calc_new_currents_all
 * plus this pass: two launches per loop instead of three. */
int ckt_distribute_update_all(const ckt_graph *graph, ckt_wires wires, ckt_nodes nodes,
                              const ckt_params *prm, void *stream);
int ckt_run_loops_all(const ckt_graph *graph, ckt_wires wires, ckt_nodes nodes,
                      const ckt_params *prm, int32_t loops, void *stream);

/* Failure of the tiled node pass.  ckt_distribute_charge_all and
 * ckt_distribute_update_all (and ckt_run_loops_all through them) use a tiled
 * pass whose copy waits are bounded (ckt_graph_set_tile_timeout).  A wait
 * that runs out leaves its tile's charges and voltages unwritten and sets the
 * graph's error word, which lives in host memory mapped for the device:
 *  - the asynchronous calls cannot know yet whether the pass they launch will
 *    fail; every later index-space call on the graph returns CKT_ETIMEOUT
 *    once a finished pass has set the word;
 *  - ckt_graph_check synchronises `stream`, then returns CKT_ETIMEOUT and
 *    clears the word if any pass on the graph set it (CKT_OK otherwise);
 *  - the _sync forms below run the asynchronous call, then ckt_graph_check.
 * The reference's tasks never fail silently either: their CUDA errors assert
 * (apps/circuit/circuit_gpu.cu:7-15). */
int ckt_graph_check(const ckt_graph *graph, void *stream);
int ckt_distribute_charge_all_sync(const ckt_graph *graph, ckt_wires wires, ckt_nodes nodes,
                                   const ckt_params *prm, void *stream);
int ckt_distribute_update_all_sync(const ckt_graph *graph, ckt_wires wires, ckt_nodes nodes,
                                   const ckt_params *prm, void *stream);
int ckt_run_loops_all_sync(const ckt_graph *graph, ckt_wires wires, ckt_nodes nodes,
                           const ckt_params *prm, int32_t loops, void *stream);

/* ------------------------------------------------------------------------
 * Reference-instance interop: conversion between the reference's
 * array-of-structs instances -- CircuitWire (128 bytes: in_ptr, out_ptr,
 * in_loc, out_loc as 4-byte ints, inductance, resistance, current[10],
 * capacitance, voltage[9], 6 pad floats) and CircuitNode (16 bytes: charge,
 * voltage, capacitance, leakage), apps/circuit/circuit.h:35-54 -- and the
 * structure-of-arrays views.  The AoS pointer may be device memory or host
 * memory mapped for the device (zero-copy instances, the placement of
 * apps/circuit/circuit.cc:903-914); it must be 16-byte aligned.  Pad floats
 * are written as zero.  Asynchronous on `stream`.
 * ---------------------------------------------------------------------- */
int ckt_wires_from_aos(const void *aos, int64_t num_wires, ckt_wires soa, void *stream);
int ckt_wires_to_aos(ckt_wires soa, int64_t num_wires, void *aos, void *stream);
int ckt_nodes_from_aos(const void *aos, int64_t num_nodes, ckt_nodes soa, void *stream);
int ckt_nodes_to_aos(ckt_nodes soa, int64_t num_nodes, void *aos, void *stream);

/* ------------------------------------------------------------------------
 * Contribution graph
 * ---------------------------------------------------------------------- */

/* Builds the graph from HOST copies of the wire endpoints.  pieces[] must
 * tile [0, W) with ascending first_wire; num_nodes is the node region size.
 * Validates every pointer and location (CKT_EBOUNDS names the first bad
 * wire in ckt_last_error()).  Allocates device memory. */
int ckt_graph_create(const ckt_piece *pieces, int32_t num_pieces, uint32_t num_nodes,
                     const uint32_t *in_ptr, const uint32_t *out_ptr, const uint8_t *in_loc,
                     const uint8_t *out_loc, ckt_graph **out);
int ckt_graph_destroy(ckt_graph *graph);
/* Sizes: wires, nodes, pieces, and device bytes held. */
int ckt_graph_info(const ckt_graph *graph, int64_t *num_wires, int64_t *num_nodes,
                   int32_t *num_pieces, int64_t *device_bytes);
/* The node-tile plan of the index-space distribute_charge and fused node
 * pass (used when wires.current is 16-byte aligned and seg_stride is a
 * multiple of 4): tiles, steps, steps whose current slices are copied whole,
 * and the error word (bit 0: a copy wait ran out and a tile's results were
 * left unwritten; reading it waits for the whole device and clears it).  No
 * counterpart in the reference. */
int ckt_graph_tile_info(const ckt_graph *graph, int32_t *tiles, int64_t *steps,
                        int64_t *stream_steps, uint32_t *error_word);
/* Bound of the tiled pass's waits on its copies, in ns (0: the default, 2 s).
 * No counterpart in the reference. */
int ckt_graph_set_tile_timeout(ckt_graph *graph, uint64_t timeout_ns);

/* ------------------------------------------------------------------------
 * Generator: restatement of load_circuit (apps/circuit/circuit.cc:1071-1288)
 * producing the same drand48 stream, graph and initial values.
 * ---------------------------------------------------------------------- */
typedef struct {
  int32_t num_pieces;      /* -p   */
  int32_t nodes_per_piece; /* -npp */
  int32_t wires_per_piece; /* -wpp */
  int32_t reserved;
  double pct_wire_in_piece; /* -pct, compared as (100*drand48()) < pct */
  int64_t random_seed;      /* -s   */
  double L_offset;          /* inductance = drand48()*L_scale + L_offset; */
  double L_scale;           /* the reference hard-codes 0.01 and 0.1     */
} ckt_gen_params;

/* Host structure-of-arrays circuit (caller-allocated; W = P*wpp, N = P*npp).
 * current is [10][W], voltage [9][W]. */
typedef struct {
  uint32_t *in_ptr, *out_ptr;
  uint8_t *in_loc, *out_loc;
  float *inductance, *resistance, *capacitance;
  float *current, *voltage;
  float *charge, *node_voltage, *node_capacitance, *node_leakage;
  int32_t *locator;
} ckt_host_circuit;

int ckt_generate(const ckt_gen_params *p, ckt_host_circuit *out);

/* Device-resident circuit with its contribution graph (all device
 * pointers, caller-allocated): wire arrays [W] (current [10][W], voltage
 * [9][W], ent [2W], gstart [ceil(2W/32)]), node arrays [N], off [N + 1]. */
typedef struct {
  uint32_t *in_ptr, *out_ptr;
  uint8_t *in_loc, *out_loc;
  float *inductance, *resistance, *capacitance;
  float *current, *voltage;
  float *charge, *node_voltage, *node_capacitance, *node_leakage;
  int32_t *locator;
  uint32_t *off;       /* node CSR offsets; bit 31 = private node */
  uint32_t *ent;       /* (wire << 2) | (end << 1) | starts-new-piece-group */
  uint32_t *slot_in;   /* CSR position of each wire's in-end */
  uint32_t *slot_out;  /* CSR position of each wire's out-end */
  uint32_t *gstart;    /* bit i = entry i starts a piece group */
} ckt_device_circuit;

/* The generator on the GPU: the same drand48 stream, graph and initial
 * values as ckt_generate, bit for bit, written straight into device memory,
 * and the contribution graph built there too (identical to the one
 * ckt_graph_create builds from the same wires).  Asynchronous on `stream`;
 * uses stream-ordered scratch memory. */
int ckt_generate_device(const ckt_gen_params *p, ckt_device_circuit *out, void *stream);

/* Copies a graph's whole-circuit CSR to host arrays (off [N + 1], ent [2W],
 * slot_in [W], slot_out [W], gstart [ceil(2W/32)]); NULL skips a field. */
int ckt_graph_export(const ckt_graph *graph, uint32_t *off, uint32_t *ent, uint32_t *slot_in,
                     uint32_t *slot_out, uint32_t *gstart);


/* ------------------------------------------------------------------------
 * Batched form: many independent circuits of uneven sizes.  One call of
 * ckt_batch_run advances EVERY circuit by one outer loop (calc_new_currents
 * with the circuit's own inner-step count, then distribute_charge, then
 * update_voltages) in ONE persistent kernel launch, replayed from a CUDA
 * graph.  Circuits are independent, so each one's results are bit-identical
 * to running it alone with the index-space calls.  No counterpart in the
 * reference, which runs one circuit per process.
 * ---------------------------------------------------------------------- */
typedef struct ckt_batch ckt_batch;

/* Launch shape of the persistent kernel; chosen by ckt_batch_autotune. */
typedef struct {
  int32_t block;            /* threads per block: 128 or 256 */
  int32_t wires_per_thread; /* calc_new_currents wires per thread per tile: 1 or 2 */
  int32_t dc_schedule;      /* distribute_charge: 0 staged block gather, 1 thread per node,
                               2 contributions scattered by the calc_new_currents tiles, then
                               summed contiguously */
  int32_t blocks_per_sm;    /* output: resident blocks per SM of the persistent grid */
} ckt_batch_config;

/* From host circuits (each sized by its shape; node pointers local to the
 * circuit).  steps[i] is circuit i's inner-step count. */
int ckt_batch_create(int32_t num_circuits, const ckt_gen_params *shapes,
                     const ckt_host_circuit *circuits, const int32_t *steps, ckt_batch **out);
/* Same, generating every circuit with the reference generator (in parallel
 * on `host_threads` threads). */
int ckt_batch_generate(int32_t num_circuits, const ckt_gen_params *shapes, const int32_t *steps,
                       int32_t host_threads, ckt_batch **out);
int ckt_batch_destroy(ckt_batch *batch);
/* Union sizes, wire-segment updates per run (sum of W x 10 x steps) and
 * device bytes held. */
int ckt_batch_info(const ckt_batch *batch, int64_t *num_wires, int64_t *num_nodes,
                   double *segment_updates_per_run, int64_t *device_bytes);
int ckt_batch_circuit_offsets(const ckt_batch *batch, int32_t circuit, int64_t *first_wire,
                              int64_t *first_node);
int ckt_batch_set_config(ckt_batch *batch, const ckt_batch_config *config);
int ckt_batch_get_config(const ckt_batch *batch, ckt_batch_config *config);
/* Times every launch shape on this batch (running it; the state is reset
 * afterwards), keeps the fastest and caches it per shape bucket. */
int ckt_batch_autotune(ckt_batch *batch, int32_t mode, void *stream, ckt_batch_config *chosen);
/* One outer loop of every circuit: one persistent launch through a CUDA
 * graph (captured on first use per mode). */
int ckt_batch_run(ckt_batch *batch, int32_t mode, void *stream);
/* Same launch without the graph. */
int ckt_batch_run_direct(ckt_batch *batch, int32_t mode, void *stream);
/* The plain path on the same batch, circuit after circuit (the comparison
 * point of the batched form): per_piece = 0, one launch per task per circuit
 * (index-space calls); per_piece = 1, calc_new_currents and update_voltages
 * launched piece by piece with a stream synchronisation after each launch,
 * as the reference's GPU task wrappers do (circuit_gpu.cu:204,367). */
int ckt_batch_run_sequential(ckt_batch *batch, int32_t mode, int32_t per_piece, void *stream);
/* Synchronises `stream` and reads the persistent kernel's error word:
 * CKT_ETIMEOUT if a bounded wait ran out. */
int ckt_batch_check(ckt_batch *batch, void *stream);
/* Bound of every device-side wait (default 2 s). */
int ckt_batch_set_timeout(ckt_batch *batch, uint64_t timeout_ns);
/* Restores the state the batch was created with. */
int ckt_batch_reset_state(ckt_batch *batch, void *stream);
/* Circuit `circuit`'s state to host arrays ([10][W_i], [9][W_i], [N_i],
 * [N_i]); NULL skips a field.  Synchronous. */
int ckt_batch_read_state(ckt_batch *batch, int32_t circuit, float *current, float *voltage,
                         float *charge, float *node_voltage, void *stream);
/* The whole batch's state from / to host memory, asynchronous on `stream`
 * (pinned host memory gives full copy speed).  Layout: circuit blocks back
 * to back in circuit order -- current[10 * W_total] holds circuit i's
 * [10][W_i] block at 10 * first_wire(i), voltage likewise with 9, charge and
 * node_voltage [N_total] hold circuit i's nodes at first_node(i) (node
 * blocks padded to multiples of 4); see ckt_batch_circuit_offsets. */
int ckt_batch_upload_state(ckt_batch *batch, const float *current, const float *voltage,
                           const float *charge, const float *node_voltage, void *stream);
int ckt_batch_download_state(ckt_batch *batch, float *current, float *voltage, float *charge,
                             float *node_voltage, void *stream);
/* Fault injection for tests: makes circuit `circuit`'s distribute_charge
 * tiles wait for a calc_new_currents tile that does not exist, so the wait
 * runs out (enable = 0 restores the table). */
int ckt_batch_inject_stall(ckt_batch *batch, int32_t circuit, int32_t enable);

/* ------------------------------------------------------------------------
 * Serving loop: circuit-solve requests arrive over time; each is built,
 * admitted when a slot and the HBM budget allow, kept resident on the
 * device, and advanced one outer loop per "round" -- one persistent launch
 * over every resident circuit -- until its loops are done (continuous
 * batching: requests join and leave between rounds; uploads and downloads
 * overlap the rounds).  Results are bit-identical to running the request
 * alone.  No counterpart in the reference.
 * ---------------------------------------------------------------------- */
typedef struct ckt_server ckt_server;

typedef struct {
  uint64_t hbm_budget_bytes; /* admission budget for resident circuits */
  int32_t max_circuits;      /* resident circuit slots */
  int32_t prep_threads;      /* host threads building requests' circuits */
  int32_t mode;              /* CKT_MODE_EXACT or CKT_MODE_FAST */
  int32_t keep_results;      /* keep final state for ckt_server_take_result */
  uint64_t round_timeout_ns; /* bound of the round kernel's device waits */
  ckt_batch_config launch;   /* round kernel launch shape */
  int32_t device_generate;   /* 1: build circuits with ckt_generate_device on the GPU;
                                0: on the host (prep_threads) and upload them */
  int32_t reserved;
} ckt_server_config;

/* One request: a circuit from the reference generator (shape and seed),
 * `steps` inner steps, `loops` outer loops. */
typedef struct {
  uint64_t request_id;
  ckt_gen_params shape;
  int32_t steps;
  int32_t loops;
} ckt_request;

/* Times are seconds on the server's clock (ckt_server_clock). */
typedef struct {
  uint64_t request_id;
  int32_t status; /* CKT_OK, CKT_ENOMEM (larger than the budget),
                     CKT_ECANCELLED, CKT_ETIMEOUT, CKT_EBOUNDS, ... */
  int32_t loops;  /* loops completed */
  double submit_s, admit_s, start_s, finish_s;
  int64_t wires, nodes;
  double segment_updates; /* wires x 10 x steps x loops completed */
} ckt_completion;

typedef struct {
  int64_t submitted, completed, rounds, resident_peak;
  uint64_t bytes_in_use, bytes_peak;
  double busy_s, clock_s;
} ckt_server_stats;

/* 80 GB budget, 4096 slots, one prep thread per host core, EXACT, results
 * not kept, 5 s round timeout, launch {128, 2, 0}, device generation. */
void ckt_server_default_config(ckt_server_config *config);
int ckt_server_create(const ckt_server_config *config, ckt_server **out);
/* Non-blocking; the id must be unused among the server's open requests. */
int ckt_server_submit(ckt_server *server, const ckt_request *request);
int ckt_server_cancel(ckt_server *server, uint64_t request_id);
/* Up to `capacity` finished requests, oldest first; non-blocking. */
int ckt_server_poll(ckt_server *server, ckt_completion *out, int32_t capacity, int32_t *count);
/* Blocks until every submitted request has finished (CKT_ETIMEOUT after
 * timeout_s). */
int ckt_server_wait(ckt_server *server, double timeout_s);
/* With keep_results: copies a finished request's final state ([10][W],
 * [9][W], [N], [N]) and forgets it. */
int ckt_server_take_result(ckt_server *server, uint64_t request_id, float *current,
                           float *voltage, float *charge, float *node_voltage);
int ckt_server_get_stats(ckt_server *server, ckt_server_stats *out);
double ckt_server_clock(const ckt_server *server);
/* Stops the threads, abandons open requests and frees everything. */
int ckt_server_destroy(ckt_server *server);

/* ------------------------------------------------------------------------
 * Reduction microbenchmark: the GPU form of benchmarks/reductions/
 * reducetest.cc.  A histogram of `buckets` unsigned counters receives one
 * +1 reduction per element; element i of batch b has key
 * myrand(start + i) % buckets with start = b * batch_size (32-bit unsigned
 * arithmetic, reducetest.cc:174, 323-347).  The schedules are the
 * benchmark's cases mapped onto the GPU's memory levels; every schedule adds
 * the same counts (integer addition: the order does not matter).
 * ---------------------------------------------------------------------- */
typedef enum {
  /* original / redsingle (reducetest.cc:335-348, 428-452): every element
   * reduces straight into the target instance -- one global atomic add. */
  CKT_RED_SINGLE = 0,
  /* redfold (:378-400): a fold instance per thread block, initialised to the
   * identity, receives the block's reductions and is then applied to the
   * target.  The fold lives in shared memory when buckets <=
   * CKT_HIST_SMEM_FOLD_BUCKETS, otherwise in a few L2-resident copies in the
   * scratch buffer. */
  CKT_RED_FOLD = 1,
  /* localize (:351-375): the owner of a range of buckets copies that range
   * of the target into its shared memory, applies every reduction that falls
   * in it without global atomics, and copies it back; the reductions are
   * first routed to their owners (keyed, counted, scattered by range). */
  CKT_RED_LOCALIZE = 2,
  /* redlist (:403-425): each batch appends (pointer, value) entries to a
   * reduction list in the scratch buffer; the lists are then applied to the
   * target. */
  CKT_RED_LIST = 3
} ckt_red_schedule;

#define CKT_HIST_SMEM_FOLD_BUCKETS 51200     /* 200 KB of 32-bit counters */
#define CKT_HIST_LOCALIZE_MAX_BUCKETS 67108864 /* 4096 ranges x 16384 buckets */

typedef struct {
  uint32_t buckets;     /* -buckets (default 1048576); >= 1 */
  uint32_t batch_size;  /* -bsize (default 1048576) */
  uint32_t num_batches; /* -batches (default 1024) */
  uint32_t first_batch; /* index of the first batch (0 in the benchmark) */
  uint32_t seed1;       /* 12345 (reducetest.cc:208) */
  uint32_t seed2;       /* 54321 (reducetest.cc:209) */
} ckt_hist_params;

/* The benchmark's defaults (reducetest.cc:205-209). */
void ckt_hist_default_params(ckt_hist_params *out);
/* Scratch bytes a schedule needs: *min_bytes at least (0 when it needs
 * none), *good_bytes for full speed (L2-sized rounds). */
int ckt_hist_scratch_bytes(const ckt_hist_params *p, int32_t schedule, uint64_t *min_bytes,
                           uint64_t *good_bytes);
/* Adds every batch's counts into hist[0..buckets) (device memory; its
 * contents are kept, like the benchmark's master instance).  `scratch` is
 * device memory of `scratch_bytes` >= the schedule's minimum, 16-byte
 * aligned, owned by the caller, free for the call's duration; its contents
 * need no initialisation and are left undefined.  Asynchronous on
 * `stream`. */
int ckt_hist_run(const ckt_hist_params *p, int32_t schedule, uint32_t *hist, void *scratch,
                 uint64_t scratch_bytes, void *stream);

#ifdef __cplusplus
}
#endif
#endif /* CKT_H */
