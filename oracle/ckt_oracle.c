/*
 * ckt_oracle.c -- CPU oracle for the circuit hot path (TEST INFRASTRUCTURE).
 *
 * Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg load
 * this file's library; the CUDA product never does.  Every function cites the
 * reference code it restates (paths relative to the LegionOrigins tree).
 *
 * Build with -ffp-contract=off: the reference's arithmetic has no fused
 * multiply-adds, and the generator's `drand48()*a + b` expressions must not
 * be contracted either (x86-64 compilers cannot contract them; aarch64 GCC
 * would by default).
 */
#define _DEFAULT_SOURCE
#define _XOPEN_SOURCE 700
#include "ckt_oracle.h"

#include <float.h>
#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

/* DELTAT is the double literal 1e-6 stored into `float dt`
 * (apps/circuit/circuit.h:44, circuit.cc:375, circuit_gpu.cu:104). */
#define OCL_DT_F ((float)1e-6)
#define OCL_DT_D ((double)(float)1e-6)

/* ------------------------------------------------------------------------ */
/* Generator: apps/circuit/circuit.cc:1071-1288                              */
/* ------------------------------------------------------------------------ */

/* random_element (circuit.cc:1042-1049) walks a std::set<utptr_t>.  utptr_t's
 * operator< is reversed (runtime/common.h:80: `ptr.value < this->value`), so
 * the set iterates in DESCENDING pointer order and index k selects the k-th
 * largest pointer.  The set is always the full node range of one piece
 * (nodes leave private_node_map only in the second pass, circuit.cc:1198). */
static uint32_t pick_node(int64_t first_node, int32_t npp)
{
  int k = (int)(drand48() * (double)(size_t)npp);
  return (uint32_t)(first_node + (int64_t)npp - 1 - k);
}

int ocl_generate(const ocl_params *p,
                 uint32_t *in_ptr, uint32_t *out_ptr,
                 uint8_t *in_loc, uint8_t *out_loc,
                 float *wire_L, float *wire_R, float *wire_C,
                 float *node_charge, float *node_voltage,
                 float *node_cap, float *node_leak,
                 int32_t *locator)
{
  const int32_t P = p->num_pieces, npp = p->nodes_per_piece, wpp = p->wires_per_piece;
  if (P < 1 || npp < 1 || wpp < 0) return -1;
  const int64_t N = (int64_t)P * npp, W = (int64_t)P * wpp;

  srand48((long)p->random_seed);                                  /* :1098 */

  /* Nodes, piece-major (:1108-1135). */
  for (int64_t x = 0; x < N; x++) {
    node_charge[x] = 0.f;
    node_voltage[x] = (float)(2 * drand48() - 1);
    node_cap[x] = (float)(drand48() + 1);
    node_leak[x] = (float)(0.1f * drand48());
    locator[x] = 1;
  }

  /* Wires, piece-major (:1140-1193). */
  for (int32_t n = 0; n < P; n++) {
    for (int32_t i = 0; i < wpp; i++) {
      const int64_t w = (int64_t)n * wpp + i;
      wire_R[w] = (float)(drand48() * 10 + 1);
      wire_L[w] = (float)(drand48() * p->L_scale + p->L_offset);
      wire_C[w] = (float)(drand48() * 0.1);
      in_ptr[w] = pick_node((int64_t)n * npp, npp);
      const int in_piece = (100 * drand48()) < p->pct_wire_in_piece;
      if (in_piece || P == 1) {
        /* P == 1: the reference's cross-piece branch would index piece 1,
         * which does not exist; every wire is kept in-piece instead and the
         * pct draw above is still consumed. */
        out_ptr[w] = pick_node((int64_t)n * npp, npp);
      } else {
        int nn = (int)(drand48() * (P - 1));
        if (nn >= n) nn++;
        out_ptr[w] = pick_node((int64_t)nn * npp, npp);
        locator[out_ptr[w]] = 0;                                   /* shared */
      }
    }
  }

  /* Locations (:1228-1244 with find_location :1051-1069). */
  for (int32_t n = 0; n < P; n++) {
    for (int32_t i = 0; i < wpp; i++) {
      const int64_t w = (int64_t)n * wpp + i;
      const uint32_t a = in_ptr[w], b = out_ptr[w];
      in_loc[w] = locator[a] ? OCL_PRIVATE : OCL_SHARED;
      if ((int64_t)(b / (uint32_t)npp) != n) out_loc[w] = OCL_GHOST;
      else out_loc[w] = locator[b] ? OCL_PRIVATE : OCL_SHARED;
    }
  }
  (void)W;
  return 0;
}

/* ------------------------------------------------------------------------ */
/* calc_new_currents: circuit_gpu.cu:61-149 / circuit.cc:352-413            */
/* ------------------------------------------------------------------------ */

#define CNC_BODY(T, DT)                                                        \
  for (int64_t w = w_begin; w < w_end; w++) {                                  \
    const T l = L[w], r = R[w], c = C[w];                                      \
    T I0[10], V0[9], ni[10], nv[11];                                           \
    for (int k = 0; k < 10; k++) I0[k] = current[k * stride + w];             \
    for (int k = 0; k < 9; k++) V0[k] = voltage[k * stride + w];               \
    for (int k = 0; k < 10; k++) ni[k] = I0[k];                                \
    if (quirk) {                                                               \
      for (int k = 0; k < 9; k++) nv[k] = V0[k];                               \
      nv[9] = 0;                                                               \
    } else {                                                                   \
      nv[0] = node_voltage[in_ptr[w]];                                         \
      for (int k = 0; k < 9; k++) nv[k + 1] = V0[k];                           \
    }                                                                          \
    nv[10] = node_voltage[out_ptr[w]];                                         \
    for (int32_t j = 0; j < steps; j++) {                                      \
      for (int k = 0; k < 10; k++)                                             \
        ni[k] = ((nv[k + 1] - nv[k]) - (l * (ni[k] - I0[k]) / DT)) / r;        \
      for (int k = 0; k < 9; k++)                                              \
        nv[k + 1] = V0[k] + DT * (ni[k] - ni[k + 1]) / c;                      \
    }                                                                          \
    for (int k = 0; k < 10; k++) current[k * stride + w] = ni[k];              \
    for (int k = 0; k < 9; k++) voltage[k * stride + w] = nv[k + 1];           \
  }

void ocl_cnc_f32(int64_t w_begin, int64_t w_end, int64_t stride,
                 const uint32_t *in_ptr, const uint32_t *out_ptr,
                 const float *L, const float *R, const float *C,
                 float *current, float *voltage,
                 const float *node_voltage, int32_t steps, int32_t quirk)
{
  const float dt = OCL_DT_F;
  CNC_BODY(float, dt)
}

void ocl_cnc_f64(int64_t w_begin, int64_t w_end, int64_t stride,
                 const uint32_t *in_ptr, const uint32_t *out_ptr,
                 const double *L, const double *R, const double *C,
                 double *current, double *voltage,
                 const double *node_voltage, int32_t steps, int32_t quirk)
{
  const double dt = OCL_DT_D;
  CNC_BODY(double, dt)
}

/* ------------------------------------------------------------------------ */
/* distribute_charge: circuit.cc:415-443, reduce_node :98-116,               */
/* AccumulateCharge :18-68, AccessorGeneric::reduce runtime/lowlevel.h:475  */
/* ------------------------------------------------------------------------ */

#define DC_BODY(T, DT)                                                         \
  int32_t *mark = (int32_t *)calloc((size_t)(N > 0 ? N : 1), sizeof(int32_t)); \
  int64_t *touched = NULL;                                                     \
  int64_t cap_t = 0;                                                           \
  for (int32_t k = 0; k < P; k++) {                                            \
    int64_t nt = 0;                                                            \
    if (cap_t < 2 * num_wires[k]) {                                            \
      cap_t = 2 * num_wires[k];                                                \
      touched = (int64_t *)realloc(touched, (size_t)(cap_t > 0 ? cap_t : 1) *  \
                                                sizeof(int64_t));              \
    }                                                                          \
    for (int64_t w = first_wire[k]; w < first_wire[k] + num_wires[k]; w++) {   \
      const T cin = -DT * current[0 * stride + w];                             \
      const T cout = DT * current[9 * stride + w];                             \
      const uint32_t xs[2] = {in_ptr[w], out_ptr[w]};                          \
      const uint8_t ls[2] = {in_loc[w], out_loc[w]};                           \
      const T cs[2] = {cin, cout};                                             \
      for (int e = 0; e < 2; e++) {                                            \
        const uint32_t x = xs[e];                                              \
        if (ls[e] == OCL_PRIVATE) {                                            \
          node_charge[x] = node_charge[x] + cs[e]; /* apply<true> */           \
        } else {                                                               \
          if (mark[x] != k + 1) { mark[x] = k + 1; touched[nt++] = x; }        \
          scratch[x] = scratch[x] + cs[e]; /* fold<true> */                    \
        }                                                                      \
      }                                                                        \
    }                                                                          \
    for (int64_t t = 0; t < nt; t++) {                                         \
      const int64_t x = touched[t];                                            \
      node_charge[x] = node_charge[x] + scratch[x]; /* apply fold instance */  \
      scratch[x] = 0;                                                          \
    }                                                                          \
  }                                                                            \
  free(touched);                                                               \
  free(mark);

void ocl_dc_f32(int32_t P, const int64_t *first_wire, const int64_t *num_wires,
                int64_t stride, const uint32_t *in_ptr, const uint32_t *out_ptr,
                const uint8_t *in_loc, const uint8_t *out_loc,
                const float *current, float *node_charge, int64_t N,
                float *scratch)
{
  const float dt = OCL_DT_F;
  DC_BODY(float, dt)
}

void ocl_dc_f64(int32_t P, const int64_t *first_wire, const int64_t *num_wires,
                int64_t stride, const uint32_t *in_ptr, const uint32_t *out_ptr,
                const uint8_t *in_loc, const uint8_t *out_loc,
                const double *current, double *node_charge, int64_t N,
                double *scratch)
{
  const double dt = OCL_DT_D;
  DC_BODY(double, dt)
}

/* ------------------------------------------------------------------------ */
/* update_voltages: circuit.cc:445-460, update_region_voltages :1290-1307    */
/* ------------------------------------------------------------------------ */

void ocl_uv_f32(int64_t n_begin, int64_t n_end, float *charge, float *voltage,
                const float *cap, const float *leak)
{
  for (int64_t x = n_begin; x < n_end; x++) {
    float v = voltage[x];
    v += charge[x] / cap[x];
    v *= (1.f - leak[x]);
    voltage[x] = v;
    charge[x] = 0.f;
  }
}

void ocl_uv_f64(int64_t n_begin, int64_t n_end, double *charge, double *voltage,
                const double *cap, const double *leak)
{
  for (int64_t x = n_begin; x < n_end; x++) {
    double v = voltage[x];
    v += charge[x] / cap[x];
    v *= (1.0 - leak[x]);
    voltage[x] = v;
    charge[x] = 0.0;
  }
}

/* ------------------------------------------------------------------------ */
/* Whole simulation, serial (region_main loop, circuit.cc:232-307)          */
/* ------------------------------------------------------------------------ */

#define SIM_BODY(T, CNC, DC, UV)                                               \
  const int32_t P = p->num_pieces;                                             \
  const int64_t W = (int64_t)P * p->wires_per_piece;                           \
  const int64_t N = (int64_t)P * p->nodes_per_piece;                           \
  int64_t *fw = (int64_t *)malloc(sizeof(int64_t) * (size_t)P);                \
  int64_t *nw = (int64_t *)malloc(sizeof(int64_t) * (size_t)P);                \
  T *scratch = (T *)calloc((size_t)(N > 0 ? N : 1), sizeof(T));                \
  for (int32_t k = 0; k < P; k++) {                                            \
    fw[k] = (int64_t)k * p->wires_per_piece;                                   \
    nw[k] = p->wires_per_piece;                                                \
  }                                                                            \
  for (int32_t l = 0; l < loops; l++) {                                        \
    CNC(0, W, W, in_ptr, out_ptr, L, R, C, current, voltage, node_voltage,     \
        steps, quirk);                                                         \
    DC(P, fw, nw, W, in_ptr, out_ptr, in_loc, out_loc, current, node_charge,   \
       N, scratch);                                                            \
    UV(0, N, node_charge, node_voltage, node_cap, node_leak);                  \
  }                                                                            \
  free(scratch);                                                               \
  free(nw);                                                                    \
  free(fw);

void ocl_simulate_f32(const ocl_params *p, int32_t loops, int32_t steps, int32_t quirk,
                      const uint32_t *in_ptr, const uint32_t *out_ptr,
                      const uint8_t *in_loc, const uint8_t *out_loc,
                      const float *L, const float *R, const float *C,
                      float *current, float *voltage,
                      float *node_charge, float *node_voltage,
                      const float *node_cap, const float *node_leak)
{
  SIM_BODY(float, ocl_cnc_f32, ocl_dc_f32, ocl_uv_f32)
}

void ocl_simulate_f64(const ocl_params *p, int32_t loops, int32_t steps, int32_t quirk,
                      const uint32_t *in_ptr, const uint32_t *out_ptr,
                      const uint8_t *in_loc, const uint8_t *out_loc,
                      const double *L, const double *R, const double *C,
                      double *current, double *voltage,
                      double *node_charge, double *node_voltage,
                      const double *node_cap, const double *node_leak)
{
  SIM_BODY(double, ocl_cnc_f64, ocl_dc_f64, ocl_uv_f64)
}

/* ------------------------------------------------------------------------ */
/* Multithreaded CPU baseline in the shared-low-level execution style        */
/* ------------------------------------------------------------------------ */

/* CircuitWire (apps/circuit/circuit.h:46-54): 128 bytes. */
typedef struct {
  uint32_t in_ptr, out_ptr;
  int32_t in_loc, out_loc;
  float inductance, resistance;
  float current[10];
  float capacitance;
  float voltage[9];
  float pad[6];
} bl_wire;

/* CircuitNode (apps/circuit/circuit.h:35-40): 16 bytes. */
typedef struct {
  float charge, voltage, capacitance, leakage;
} bl_node;

typedef struct {
  int32_t P, npp, wpp, threads, piece_limit, loops, steps, quirk;
  bl_wire *wires;
  bl_node *nodes;
  /* Reduction instances: per piece, a compact fold buffer over the
   * shared/ghost nodes its wires touch; each wire endpoint knows its slot. */
  int64_t *fold_first;   /* [P+1] slot ranges per piece */
  float *fold;           /* [total slots] */
  uint32_t *slot_in, *slot_out; /* [W] */
  /* Apply order: per owner piece, shared nodes with their (piece, slot)
   * contributions sorted by piece ascending. */
  int64_t *app_first;    /* [P+1] into app_node list */
  uint32_t *app_node;    /* shared nodes, grouped by owner piece */
  int64_t *app_cfirst;   /* [num app nodes + 1] into app_slot */
  int64_t *app_slot;     /* global fold slot, piece-ascending per node */
  pthread_barrier_t bar;
} bl_state;

typedef struct {
  bl_state *s;
  int32_t tid;
} bl_arg;

static inline void bl_read(const void *base, int64_t idx, size_t sz, void *dst)
{
  /* AccessorGeneric::get_untyped: memcpy at base + index*elmt_size. */
  memcpy(dst, (const char *)base + idx * (int64_t)sz, sz);
}
static inline void bl_write(void *base, int64_t idx, size_t sz, const void *src)
{
  memcpy((char *)base + idx * (int64_t)sz, src, sz);
}

static void bl_cnc_piece(bl_state *s, int32_t n)
{
  const float dt = OCL_DT_F;
  for (int64_t w = (int64_t)n * s->wpp; w < (int64_t)(n + 1) * s->wpp; w++) {
    bl_wire wire;
    bl_node in_node, out_node;
    bl_read(s->wires, w, sizeof(bl_wire), &wire);
    bl_read(s->nodes, wire.in_ptr, sizeof(bl_node), &in_node);
    bl_read(s->nodes, wire.out_ptr, sizeof(bl_node), &out_node);
    float nv[11], ni[10];
    for (int k = 0; k < 10; k++) ni[k] = wire.current[k];
    if (s->quirk) {
      for (int k = 0; k < 9; k++) nv[k] = wire.voltage[k];
      nv[9] = 0.f;
    } else {
      nv[0] = in_node.voltage;
      for (int k = 0; k < 9; k++) nv[k + 1] = wire.voltage[k];
    }
    nv[10] = out_node.voltage;
    for (int32_t j = 0; j < s->steps; j++) {
      for (int k = 0; k < 10; k++)
        ni[k] = ((nv[k + 1] - nv[k]) -
                 (wire.inductance * (ni[k] - wire.current[k]) / dt)) / wire.resistance;
      for (int k = 0; k < 9; k++)
        nv[k + 1] = wire.voltage[k] + dt * (ni[k] - ni[k + 1]) / wire.capacitance;
    }
    for (int k = 0; k < 10; k++) wire.current[k] = ni[k];
    for (int k = 0; k < 9; k++) wire.voltage[k] = nv[k + 1];
    bl_write(s->wires, w, sizeof(bl_wire), &wire);
  }
}

static void bl_dc_piece(bl_state *s, int32_t n)
{
  const float dt = 1e-6;
  for (int64_t w = (int64_t)n * s->wpp; w < (int64_t)(n + 1) * s->wpp; w++) {
    bl_wire wire;
    bl_read(s->wires, w, sizeof(bl_wire), &wire);
    const float cs[2] = {-dt * wire.current[0], dt * wire.current[9]};
    const uint32_t xs[2] = {wire.in_ptr, wire.out_ptr};
    const int32_t ls[2] = {wire.in_loc, wire.out_loc};
    const uint32_t sl[2] = {s->slot_in[w], s->slot_out[w]};
    for (int e = 0; e < 2; e++) {
      if (ls[e] == OCL_PRIVATE) {
        bl_node node;
        bl_read(s->nodes, xs[e], sizeof(bl_node), &node);
        node.charge += cs[e];
        bl_write(s->nodes, xs[e], sizeof(bl_node), &node);
      } else {
        s->fold[sl[e]] += cs[e];
      }
    }
  }
}

static void bl_apply_owner(bl_state *s, int32_t n)
{
  for (int64_t a = s->app_first[n]; a < s->app_first[n + 1]; a++) {
    bl_node node;
    bl_read(s->nodes, s->app_node[a], sizeof(bl_node), &node);
    for (int64_t c = s->app_cfirst[a]; c < s->app_cfirst[a + 1]; c++) {
      node.charge += s->fold[s->app_slot[c]];
      s->fold[s->app_slot[c]] = 0.f;
    }
    bl_write(s->nodes, s->app_node[a], sizeof(bl_node), &node);
  }
}

static void bl_uv_piece(bl_state *s, int32_t n)
{
  for (int64_t x = (int64_t)n * s->npp; x < (int64_t)(n + 1) * s->npp; x++) {
    bl_node node;
    bl_read(s->nodes, x, sizeof(bl_node), &node);
    node.voltage += node.charge / node.capacitance;
    node.voltage *= (1.f - node.leakage);
    node.charge = 0.f;
    bl_write(s->nodes, x, sizeof(bl_node), &node);
  }
}

static void *bl_worker(void *argp)
{
  bl_arg *a = (bl_arg *)argp;
  bl_state *s = a->s;
  const int32_t T = s->threads, t = a->tid;
  pthread_barrier_wait(&s->bar); /* start */
  for (int32_t l = 0; l < s->loops; l++) {
    for (int32_t n = t; n < s->piece_limit; n += T) bl_cnc_piece(s, n);
    pthread_barrier_wait(&s->bar);
    for (int32_t n = t; n < s->piece_limit; n += T) bl_dc_piece(s, n);
    pthread_barrier_wait(&s->bar);
    for (int32_t n = t; n < s->P; n += T) bl_apply_owner(s, n);
    pthread_barrier_wait(&s->bar);
    for (int32_t n = t; n < s->piece_limit; n += T) bl_uv_piece(s, n);
    pthread_barrier_wait(&s->bar);
  }
  return NULL;
}

static int cmp_i64_pair(const void *a, const void *b)
{
  const int64_t *x = (const int64_t *)a, *y = (const int64_t *)b;
  if (x[0] != y[0]) return x[0] < y[0] ? -1 : 1;
  if (x[1] != y[1]) return x[1] < y[1] ? -1 : 1;
  return 0;
}

double ocl_baseline_run(const ocl_params *p, int32_t loops, int32_t steps,
                        int32_t threads, int32_t piece_limit, int32_t quirk,
                        const uint32_t *in_ptr, const uint32_t *out_ptr,
                        const uint8_t *in_loc, const uint8_t *out_loc,
                        const float *L, const float *R, const float *C,
                        float *current, float *voltage,
                        float *node_charge, float *node_voltage,
                        const float *node_cap, const float *node_leak)
{
  bl_state s;
  memset(&s, 0, sizeof(s));
  s.P = p->num_pieces; s.npp = p->nodes_per_piece; s.wpp = p->wires_per_piece;
  s.threads = threads < 1 ? 1 : threads;
  s.piece_limit = (piece_limit < 1 || piece_limit > s.P) ? s.P : piece_limit;
  s.loops = loops; s.steps = steps; s.quirk = quirk;
  const int64_t W = (int64_t)s.P * s.wpp, N = (int64_t)s.P * s.npp;

  s.wires = (bl_wire *)aligned_alloc(128, (size_t)(W > 0 ? W : 1) * sizeof(bl_wire));
  s.nodes = (bl_node *)aligned_alloc(64, (size_t)(N > 0 ? N : 1) * sizeof(bl_node));
  s.slot_in = (uint32_t *)malloc((size_t)(W > 0 ? W : 1) * sizeof(uint32_t));
  s.slot_out = (uint32_t *)malloc((size_t)(W > 0 ? W : 1) * sizeof(uint32_t));
  s.fold_first = (int64_t *)calloc((size_t)s.P + 1, sizeof(int64_t));
  s.app_first = (int64_t *)calloc((size_t)s.P + 1, sizeof(int64_t));
  if (!s.wires || !s.nodes || !s.slot_in || !s.slot_out || !s.fold_first || !s.app_first)
    return -1.0;

  /* Pack SoA -> reference AoS layout (untimed). */
  for (int64_t w = 0; w < W; w++) {
    bl_wire *x = &s.wires[w];
    memset(x, 0, sizeof(*x));
    x->in_ptr = in_ptr[w]; x->out_ptr = out_ptr[w];
    x->in_loc = in_loc[w]; x->out_loc = out_loc[w];
    x->inductance = L[w]; x->resistance = R[w]; x->capacitance = C[w];
    for (int k = 0; k < 10; k++) x->current[k] = current[k * W + w];
    for (int k = 0; k < 9; k++) x->voltage[k] = voltage[k * W + w];
  }
  for (int64_t x = 0; x < N; x++) {
    s.nodes[x].charge = node_charge[x]; s.nodes[x].voltage = node_voltage[x];
    s.nodes[x].capacitance = node_cap[x]; s.nodes[x].leakage = node_leak[x];
  }

  /* Reduction-instance metadata (the runtime's instance creation; untimed):
   * slot = position of the node in the piece's sorted shared/ghost set. */
  int64_t *pairs = (int64_t *)malloc(sizeof(int64_t) * 2 * (size_t)(2 * (W > 0 ? W : 1)));
  int64_t total_slots = 0;
  int64_t *node_slot = (int64_t *)malloc(sizeof(int64_t) * (size_t)(N > 0 ? N : 1));
  int32_t *node_mark = (int32_t *)calloc((size_t)(N > 0 ? N : 1), sizeof(int32_t));
  /* (owner piece, node, piece, slot) contributions for the apply order. */
  int64_t *contrib = (int64_t *)malloc(sizeof(int64_t) * 3 * (size_t)(2 * (W > 0 ? W : 1)));
  int64_t ncontrib = 0;
  for (int32_t n = 0; n < s.P; n++) {
    s.fold_first[n] = total_slots;
    int64_t np = 0;
    for (int64_t w = (int64_t)n * s.wpp; w < (int64_t)(n + 1) * s.wpp; w++) {
      if (in_loc[w] != OCL_PRIVATE) { pairs[2 * np] = in_ptr[w]; pairs[2 * np + 1] = 0; np++; }
      if (out_loc[w] != OCL_PRIVATE) { pairs[2 * np] = out_ptr[w]; pairs[2 * np + 1] = 0; np++; }
    }
    qsort(pairs, (size_t)np, 2 * sizeof(int64_t), cmp_i64_pair);
    for (int64_t i = 0; i < np; i++) {
      if (i > 0 && pairs[2 * i] == pairs[2 * (i - 1)]) continue;
      const int64_t x = pairs[2 * i];
      node_slot[x] = total_slots;
      node_mark[x] = n + 1;
      contrib[3 * ncontrib] = x / s.npp;          /* owner piece */
      contrib[3 * ncontrib + 1] = x;              /* node */
      contrib[3 * ncontrib + 2] = total_slots;    /* slot (piece-ascending) */
      ncontrib++;
      total_slots++;
    }
    for (int64_t w = (int64_t)n * s.wpp; w < (int64_t)(n + 1) * s.wpp; w++) {
      s.slot_in[w] = in_loc[w] != OCL_PRIVATE ? (uint32_t)node_slot[in_ptr[w]] : 0u;
      s.slot_out[w] = out_loc[w] != OCL_PRIVATE ? (uint32_t)node_slot[out_ptr[w]] : 0u;
    }
  }
  s.fold_first[s.P] = total_slots;
  s.fold = (float *)calloc((size_t)(total_slots > 0 ? total_slots : 1), sizeof(float));
  /* Group contributions by (owner, node), slots already piece-ascending
   * because slots were handed out piece by piece. */
  qsort(contrib, (size_t)ncontrib, 3 * sizeof(int64_t), cmp_i64_pair);
  s.app_node = (uint32_t *)malloc(sizeof(uint32_t) * (size_t)(ncontrib > 0 ? ncontrib : 1));
  s.app_cfirst = (int64_t *)malloc(sizeof(int64_t) * (size_t)(ncontrib + 1));
  s.app_slot = (int64_t *)malloc(sizeof(int64_t) * (size_t)(ncontrib > 0 ? ncontrib : 1));
  int64_t napp = 0;
  for (int64_t i = 0; i < ncontrib; i++) {
    /* qsort on (owner, node) then slot: comparator looks at the first two
     * fields only, so sort the slot within equal (owner, node) runs below. */
    if (i == 0 || contrib[3 * i + 1] != contrib[3 * (i - 1) + 1]) {
      s.app_node[napp] = (uint32_t)contrib[3 * i + 1];
      s.app_cfirst[napp] = i;
      napp++;
    }
    s.app_slot[i] = contrib[3 * i + 2];
  }
  s.app_cfirst[napp] = ncontrib;
  for (int64_t a = 0; a < napp; a++) { /* insertion sort of slots (short runs) */
    for (int64_t i = s.app_cfirst[a] + 1; i < s.app_cfirst[a + 1]; i++) {
      int64_t v = s.app_slot[i], j = i - 1;
      while (j >= s.app_cfirst[a] && s.app_slot[j] > v) { s.app_slot[j + 1] = s.app_slot[j]; j--; }
      s.app_slot[j + 1] = v;
    }
  }
  {
    int64_t a = 0;
    for (int32_t n = 0; n <= s.P; n++) {
      while (a < napp && (int64_t)(s.app_node[a] / (uint32_t)s.npp) < n) a++;
      s.app_first[n] = a;
    }
  }
  /* Folds from pieces outside the sample must not be applied: they stay 0. */
  free(pairs); free(node_slot); free(node_mark); free(contrib);

  pthread_barrier_init(&s.bar, NULL, (unsigned)s.threads + 1);
  pthread_t *th = (pthread_t *)malloc(sizeof(pthread_t) * (size_t)s.threads);
  bl_arg *args = (bl_arg *)malloc(sizeof(bl_arg) * (size_t)s.threads);
  for (int32_t t = 0; t < s.threads; t++) {
    args[t].s = &s; args[t].tid = t;
    pthread_create(&th[t], NULL, bl_worker, &args[t]);
  }
  struct timespec t0, t1;
  clock_gettime(CLOCK_MONOTONIC, &t0);
  pthread_barrier_wait(&s.bar); /* release workers */
  for (int32_t l = 0; l < s.loops; l++)
    for (int ph = 0; ph < 4; ph++) pthread_barrier_wait(&s.bar);
  clock_gettime(CLOCK_MONOTONIC, &t1);
  for (int32_t t = 0; t < s.threads; t++) pthread_join(th[t], NULL);
  pthread_barrier_destroy(&s.bar);
  const double elapsed = (double)(t1.tv_sec - t0.tv_sec) + 1e-9 * (double)(t1.tv_nsec - t0.tv_nsec);

  /* Unpack (untimed). */
  for (int64_t w = 0; w < W; w++) {
    for (int k = 0; k < 10; k++) current[k * W + w] = s.wires[w].current[k];
    for (int k = 0; k < 9; k++) voltage[k * W + w] = s.wires[w].voltage[k];
  }
  for (int64_t x = 0; x < N; x++) {
    node_charge[x] = s.nodes[x].charge;
    node_voltage[x] = s.nodes[x].voltage;
  }
  free(th); free(args);
  free(s.wires); free(s.nodes); free(s.slot_in); free(s.slot_out);
  free(s.fold_first); free(s.fold); free(s.app_first); free(s.app_node);
  free(s.app_cfirst); free(s.app_slot);
  return elapsed;
}

/* ------------------------------------------------------------------------
 * Reduction microbenchmark (benchmarks/reductions/reducetest.cc)
 * ---------------------------------------------------------------------- */

uint32_t ocl_hist_rand(uint64_t ival, uint32_t seed1, uint32_t seed2)
{
  /* reducetest.cc:323-333 */
  uint64_t r = ival;
  for (int j = 0; j < 16; j++) {
    r = (0x5DEECE66DULL * r + 0xBULL) & 0xFFFFFFFFFFFFULL;
    r ^= ((ival >> j) & 1u) ? seed1 : seed2;
  }
  return (uint32_t)r;
}

static void hist_batches(uint32_t buckets, uint32_t batch_size, uint64_t b0, uint64_t b1,
                         uint32_t step, uint32_t seed1, uint32_t seed2, uint32_t *hist)
{
  /* reducetest.cc:174 (start = i * count, 32-bit unsigned) and :341-347 (the
   * task loop) */
  for (uint64_t b = b0; b < b1; b += step) {
    const uint32_t start = (uint32_t)(b * batch_size);
    for (uint32_t i = 0; i < batch_size; i++)
      hist[ocl_hist_rand((uint32_t)(start + i), seed1, seed2) % buckets] += 1u;
  }
}

void ocl_histogram(uint32_t buckets, uint32_t batch_size, uint32_t num_batches,
                   uint32_t first_batch, uint32_t seed1, uint32_t seed2, uint32_t *hist)
{
  hist_batches(buckets, batch_size, first_batch, (uint64_t)first_batch + num_batches, 1, seed1,
               seed2, hist);
}

typedef struct {
  uint32_t buckets, batch_size, step, seed1, seed2;
  uint64_t b0, b1;
  uint32_t *hist;
  pthread_mutex_t *mu;
  int failed;
} hist_job;

static void *hist_worker(void *argp)
{
  hist_job *j = (hist_job *)argp;
  uint32_t *fold = (uint32_t *)calloc(j->buckets, sizeof(uint32_t)); /* identity 0 */
  if (!fold) {
    j->failed = 1;
    return NULL;
  }
  hist_batches(j->buckets, j->batch_size, j->b0, j->b1, j->step, j->seed1, j->seed2, fold);
  pthread_mutex_lock(j->mu);
  for (uint32_t k = 0; k < j->buckets; k++) j->hist[k] += fold[k];
  pthread_mutex_unlock(j->mu);
  free(fold);
  return NULL;
}

double ocl_histogram_threads(uint32_t buckets, uint32_t batch_size, uint32_t num_batches,
                             uint32_t first_batch, uint32_t seed1, uint32_t seed2,
                             int32_t threads, uint32_t *hist)
{
  if (buckets == 0 || threads < 1 || !hist) return -1.0;
  if ((uint32_t)threads > num_batches && num_batches > 0) threads = (int32_t)num_batches;
  pthread_mutex_t mu = PTHREAD_MUTEX_INITIALIZER;
  hist_job *jobs = (hist_job *)calloc((size_t)threads, sizeof(hist_job));
  pthread_t *tid = (pthread_t *)calloc((size_t)threads, sizeof(pthread_t));
  if (!jobs || !tid) {
    free(jobs);
    free(tid);
    return -1.0;
  }
  struct timespec t0, t1;
  clock_gettime(CLOCK_MONOTONIC, &t0);
  int started = 0, failed = 0;
  for (int32_t t = 0; t < threads; t++) {
    hist_job *j = &jobs[t];
    j->buckets = buckets;
    j->batch_size = batch_size;
    j->b0 = (uint64_t)first_batch + (uint32_t)t;
    j->b1 = (uint64_t)first_batch + num_batches;
    j->step = (uint32_t)threads;
    j->seed1 = seed1;
    j->seed2 = seed2;
    j->hist = hist;
    j->mu = &mu;
    if (pthread_create(&tid[t], NULL, hist_worker, j) != 0) {
      failed = 1;
      break;
    }
    started++;
  }
  for (int t = 0; t < started; t++) {
    pthread_join(tid[t], NULL);
    failed |= jobs[t].failed;
  }
  clock_gettime(CLOCK_MONOTONIC, &t1);
  free(jobs);
  free(tid);
  if (failed) return -1.0;
  return (double)(t1.tv_sec - t0.tv_sec) + 1e-9 * (double)(t1.tv_nsec - t0.tv_nsec);
}

/* The division by dt of calc_new_currents, L*(new_i - I0)/dt
 * (apps/circuit/circuit.cc:391-393, circuit_gpu.cu:119-122), as the GPU's
 * EXACT mode evaluates it: fmaf(a, zh, a*zl) with zh + zl a split
 * reciprocal of dt.  Compares it with the IEEE quotient a/dt for every float
 * dividend whose bit pattern lies in [lo, hi) and counts the mismatches among
 * dividends of magnitude >= tiny (plus zeros, infinities, NaN: trusted) and
 * among the others; equal means equal bits, or both NaN. */
void ocl_split_quotient_check(uint64_t lo, uint64_t hi, float dt, float zh, float zl, float tiny,
                              uint64_t *bad_trusted, uint64_t *bad_other)
{
  uint64_t bt = 0, bo = 0;
  for (uint64_t i = lo; i < hi; i++) {
    const uint32_t u = (uint32_t)i;
    float a;
    memcpy(&a, &u, sizeof a);
    const float q = fmaf(a, zh, a * zl);
    const float r = a / dt;
    uint32_t uq, ur;
    memcpy(&uq, &q, sizeof uq);
    memcpy(&ur, &r, sizeof ur);
    if ((isnan(q) && isnan(r)) || uq == ur) continue;
    if (!(fabsf(a) < tiny) || a == 0.0f) bt++;
    else bo++;
  }
  *bad_trusted = bt;
  *bad_other = bo;
}

/* The R and C quotients of calc_new_currents (apps/circuit/circuit.cc:
 * 394-400, circuit_gpu.cu:123-128) as the GPU's EXACT mode evaluates a
 * dividend outside the corrected quotient's guarded range [lo, hi]: scaled
 * by 2^-64 (above hi) or 2^110 (below lo) into it, divided by the corrected
 * quotient (q0 = fmaf(a, y, a*yl), r = fmaf(q0, -b, a), q = fmaf(r, y, q0)
 * with y = RN(1/b), yl = RN(1/b - y)), and scaled back; zeros and
 * infinities as a*y.  Draws `n` (dividend, divisor) pairs from seed --
 * divisors in [2^-8, 2^8) (divisor 0, R) or [2^-30, 2^30) (1, C), dividends
 * from every class: huge up to FLT_MAX, tiny down to the smallest
 * subnormal, the guarded range, zeros, infinities, NaN, and values whose
 * quotient lies within an ulp of a rounding boundary or of the overflow
 * threshold -- and counts the pairs whose result differs from the IEEE
 * quotient a/b (`bad`; equal means equal bits, or both NaN), the pairs taken
 * outside [lo, hi] (`outside`) and all pairs drawn.  Pairs whose quotient
 * may be subnormal (a nonzero |a| below 2^-125 |b|) are not drawn: the GPU
 * leaves them to its divide routine. */
static uint64_t wq_mix(uint64_t x)
{
  x ^= x >> 30;
  x *= 0xbf58476d1ce4e5b9ull;
  x ^= x >> 27;
  x *= 0x94d049bb133111ebull;
  return x ^ (x >> 31);
}

static float wq_bits(uint32_t u)
{
  float f;
  memcpy(&f, &u, sizeof f);
  return f;
}

static uint32_t wq_u(float f)
{
  uint32_t u;
  memcpy(&u, &f, sizeof u);
  return u;
}

/* A float of random sign and mantissa with binary exponent in [e0, e1]. */
static float wq_rand(uint64_t h, int e0, int e1)
{
  const int e = e0 + (int)((uint32_t)(h >> 32) % (uint32_t)(e1 - e0 + 1));
  return wq_bits((uint32_t)((e + 127) << 23) | ((uint32_t)h & 0x7fffffu) |
                 ((uint32_t)(h >> 23) & 0x80000000u));
}

static float wq_recip_quot(float a, float y, float yl, float nb)
{
  const float q0 = fmaf(a, y, a * yl);
  const float r = fmaf(q0, nb, a);
  return fmaf(r, y, q0);
}

static float wq_wide_quot(float a, float y, float yl, float nb, float lo, float hi)
{
  const float m = fabsf(a);
  const float s = m > hi ? 0x1p-64f : (m < lo ? 0x1p110f : 1.0f);
  const float u = m > hi ? 0x1p64f : (m < lo ? 0x1p-110f : 1.0f);
  const float q = wq_recip_quot(a * s, y, yl, nb) * u;
  return (m == 0.0f || isinf(m)) ? a * y : q;
}

void ocl_wide_quotient_check(uint64_t seed, uint64_t n, int divisor, uint64_t *bad,
                             uint64_t *outside, uint64_t *drawn)
{
  const int be0 = divisor == 0 ? -8 : -30, be1 = -be0 - 1;
  const float lo = divisor == 0 ? 0x1p-50f : 0x1p-40f, hi = divisor == 0 ? 0x1p100f : 0x1p90f;
  const int lo_e = divisor == 0 ? -50 : -40, hi_e = divisor == 0 ? 100 : 90;
  uint64_t nbad = 0, nout = 0, nd = 0;
  for (uint64_t i = 0; i < n; i++) {
    const uint64_t h1 = wq_mix(seed * 0x9e3779b97f4a7c15ull + 2 * i + 1);
    const uint64_t h2 = wq_mix(h1 ^ 0x632be59bd9b4e019ull);
    const float b = wq_rand(h1, be0, be1);
    const float sgn = (h2 >> 20) & 1u ? -1.0f : 1.0f;
    float a;
    switch ((h2 >> 56) % 8u) {
      case 0:  /* huge */
        a = wq_rand(h2, hi_e, 127);
        break;
      case 1: {  /* tiny, subnormals included */
        const int e = -149 + (int)((uint32_t)(h2 >> 32) % (uint32_t)(lo_e + 149));
        a = sgn * ldexpf(1.0f + (float)(h2 & 0x7fffffu) * 0x1p-23f, e);
        break;
      }
      case 2: {  /* special values and the range edges */
        const float sp[8] = {0.0f, INFINITY, NAN, FLT_MAX, lo, hi, wq_bits(wq_u(hi) + 1u),
                             wq_bits(wq_u(lo) - 1u)};
        a = sgn * sp[(h2 >> 8) & 7u];
        break;
      }
      case 3: {  /* a/b within about an ulp of overflowing */
        const double m = (double)FLT_MAX + ldexp(1.0, 103) * ((double)((h2 >> 8) & 7u) - 3.5) / 2.0;
        a = sgn * (float)((double)b * m);
        a = wq_bits(wq_u(a) + (uint32_t)((h2 >> 12) & 3u) - 1u);
        break;
      }
      case 4:
      case 5: {  /* a/b within about an ulp of a rounding boundary, huge or tiny */
        const float q = (h2 >> 9) & 1u ? wq_rand(h2, 60, 126) : wq_rand(h2, -125, -60);
        const double mid = (double)q + 0.5 * ((double)wq_bits(wq_u(fabsf(q)) + 1u) - (double)fabsf(q)) *
                                           (q < 0.0f ? -1.0 : 1.0);
        a = (float)((double)b * mid);
        a = wq_bits(wq_u(a) + (uint32_t)((h2 >> 12) & 7u) - 3u);
        break;
      }
      default:  /* any exponent */
        a = wq_rand(h2, -126, 127);
        break;
    }
    if (a != 0.0f && fabsf(a) * 0x1p125f < fabsf(b)) continue;
    nd++;
    const float y = 1.0f / b, yl = fmaf(-b, y, 1.0f) / b;
    const float got = wq_wide_quot(a, y, yl, -b, lo, hi), want = a / b;
    nout += !(fabsf(a) >= lo && fabsf(a) <= hi);
    if (!((isnan(got) && isnan(want)) || wq_u(got) == wq_u(want))) nbad++;
  }
  *bad = nbad;
  *outside = nout;
  *drawn = nd;
}
