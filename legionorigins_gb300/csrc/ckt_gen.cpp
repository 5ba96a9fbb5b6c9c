// ckt_gen.cpp -- host circuit generator: the reference's load_circuit
// (apps/circuit/circuit.cc:1071-1288) restated in O(1) per random draw.
//
// It consumes the same srand48/drand48 stream in the same order, so it
// yields the same graph and initial values bit for bit:
//   nodes, piece-major:  voltage = 2*drand48()-1, capacitance = drand48()+1,
//                        leakage = 0.1f*drand48(), charge = 0   (:1121-1125)
//   wires, piece-major:  R = drand48()*10+1, L = drand48()*L_scale+L_offset,
//                        C = drand48()*0.1                       (:1162-1164)
//                        in  = random_element(piece n's nodes)   (:1166)
//                        if 100*drand48() < pct: out = random_element(piece n)
//                        else nn = int(drand48()*(P-1)), nn += (nn >= n),
//                             out = random_element(piece nn), out is shared
//   random_element (:1042-1049) walks a std::set<utptr_t>, whose
//   operator< is reversed (runtime/common.h:80), so index k is the k-th
//   LARGEST pointer: first_node + npp - 1 - k.
//   locations (:1228-1244): PRIVATE / SHARED for nodes of the wire's own
//   piece by the locator, GHOST for nodes of another piece.
// The arithmetic is double, rounded to float on store; this file is built
// with -ffp-contract=off so `drand48()*a + b` is never fused.
// With one piece the reference's cross-piece branch would index a piece that
// does not exist; here every wire stays in-piece (the pct draw is still
// consumed).
#include <cstdlib>

#include "ckt_internal.h"

extern "C" int ckt_generate(const ckt_gen_params *p, ckt_host_circuit *o) {
  CKT_REQUIRE(p != nullptr && o != nullptr, "NULL argument");
  const int32_t P = p->num_pieces, npp = p->nodes_per_piece, wpp = p->wires_per_piece;
  CKT_REQUIRE(P >= 1 && npp >= 1 && wpp >= 0, "bad shape P=%d npp=%d wpp=%d", P, npp, wpp);
  const int64_t N = (int64_t)P * npp, W = (int64_t)P * wpp;
  CKT_REQUIRE(N <= 0xffffffffLL && W <= ckt::kMaxWires, "circuit too large (N=%lld W=%lld)",
              (long long)N, (long long)W);
  CKT_REQUIRE(o->in_ptr && o->out_ptr && o->in_loc && o->out_loc && o->inductance &&
                  o->resistance && o->capacitance && o->current && o->voltage && o->charge &&
                  o->node_voltage && o->node_capacitance && o->node_leakage && o->locator,
              "host circuit has NULL arrays");

  srand48((long)p->random_seed);
  for (int64_t x = 0; x < N; x++) {
    o->charge[x] = 0.f;
    o->node_voltage[x] = (float)(2 * drand48() - 1);
    o->node_capacitance[x] = (float)(drand48() + 1);
    o->node_leakage[x] = (float)(0.1f * drand48());
    o->locator[x] = 1;
  }
  auto pick = [npp](int64_t piece) -> uint32_t {
    const int k = (int)(drand48() * (double)(size_t)npp);
    return (uint32_t)(piece * npp + npp - 1 - k);
  };
  for (int32_t n = 0; n < P; n++) {
    for (int32_t i = 0; i < wpp; i++) {
      const int64_t w = (int64_t)n * wpp + i;
      o->resistance[w] = (float)(drand48() * 10 + 1);
      o->inductance[w] = (float)(drand48() * p->L_scale + p->L_offset);
      o->capacitance[w] = (float)(drand48() * 0.1);
      o->in_ptr[w] = pick(n);
      const bool in_piece = (100 * drand48()) < p->pct_wire_in_piece;
      if (in_piece || P == 1) {
        o->out_ptr[w] = pick(n);
      } else {
        int nn = (int)(drand48() * (P - 1));
        if (nn >= n) nn++;
        o->out_ptr[w] = pick(nn);
        o->locator[o->out_ptr[w]] = 0;
      }
    }
  }
  for (int32_t n = 0; n < P; n++) {
    for (int32_t i = 0; i < wpp; i++) {
      const int64_t w = (int64_t)n * wpp + i;
      const uint32_t a = o->in_ptr[w], b = o->out_ptr[w];
      o->in_loc[w] = o->locator[a] ? CKT_PRIVATE_PTR : CKT_SHARED_PTR;
      o->out_loc[w] = ((int64_t)(b / (uint32_t)npp) != n)
                          ? CKT_GHOST_PTR
                          : (o->locator[b] ? CKT_PRIVATE_PTR : CKT_SHARED_PTR);
    }
  }
  for (int64_t k = 0; k < 10 * W; k++) o->current[k] = 0.f;
  for (int64_t k = 0; k < 9 * W; k++) o->voltage[k] = 0.f;
  return CKT_OK;
}
