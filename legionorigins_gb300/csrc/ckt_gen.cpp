// ckt_gen.cpp -- host circuit generator: the reference's load_circuit
// (apps/circuit/circuit.cc:1071-1288) restated in O(1) per random draw.
//
// It consumes the same random stream in the same order as the reference, so
// it yields the same graph and initial values bit for bit:
//   nodes, piece-major:  voltage = 2*u-1, capacitance = u+1,
//                        leakage = 0.1f*u, charge = 0            (:1121-1125)
//   wires, piece-major:  R = u*10+1, L = u*L_scale+L_offset, C = u*0.1
//                                                                 (:1162-1164)
//                        in  = random_element(piece n's nodes)   (:1166)
//                        if 100*u < pct: out = random_element(piece n)
//                        else nn = int(u*(P-1)), nn += (nn >= n),
//                             out = random_element(piece nn), out is shared
//   random_element (:1042-1049) walks a std::set<utptr_t>, whose
//   operator< is reversed (runtime/common.h:80), so index k is the k-th
//   LARGEST pointer: first_node + npp - 1 - k.
//   locations (:1228-1244): PRIVATE / SHARED for nodes of the wire's own
//   piece by the locator, GHOST for nodes of another piece.
// u is drand48(): the POSIX 48-bit linear congruential generator
// x' = (0x5DEECE66D x + 0xB) mod 2^48 seeded by srand48(s) as
// x = (s mod 2^32) << 16 | 0x330E, returning x'/2^48.  It is implemented
// here with explicit state (Lcg48) so that circuits can be generated
// concurrently; the values are exactly libc's.
// The arithmetic is double, rounded to float on store; this file is built
// with -ffp-contract=off so `u*a + b` is never fused.
// With one piece the reference's cross-piece branch would index a piece that
// does not exist; here every wire stays in-piece (the pct draw is still
// consumed).
#include <cmath>

#include "ckt_gen.h"
#include "ckt_internal.h"

namespace ckt {

int generate_into(const ckt_gen_params *p, const ckt_host_circuit *o, uint32_t node_base) {
  CKT_REQUIRE(p != nullptr && o != nullptr, "NULL argument");
  const int32_t P = p->num_pieces, npp = p->nodes_per_piece, wpp = p->wires_per_piece;
  CKT_REQUIRE(P >= 1 && npp >= 1 && wpp >= 0, "bad shape P=%d npp=%d wpp=%d", P, npp, wpp);
  const int64_t N = (int64_t)P * npp, W = (int64_t)P * wpp;
  CKT_REQUIRE(N + node_base <= 0xffffffffLL && W <= kMaxWires,
              "circuit too large (N=%lld W=%lld)", (long long)N, (long long)W);
  CKT_REQUIRE(o->in_ptr && o->out_ptr && o->in_loc && o->out_loc && o->inductance &&
                  o->resistance && o->capacitance && o->current && o->voltage && o->charge &&
                  o->node_voltage && o->node_capacitance && o->node_leakage && o->locator,
              "host circuit has NULL arrays");

  Lcg48 rng((int64_t)p->random_seed);
  for (int64_t x = 0; x < N; x++) {
    o->charge[x] = 0.f;
    o->node_voltage[x] = (float)(2 * rng.next() - 1);
    o->node_capacitance[x] = (float)(rng.next() + 1);
    o->node_leakage[x] = (float)(0.1f * rng.next());
    o->locator[x] = 1;
  }
  auto pick = [npp, &rng](int64_t piece) -> uint32_t {
    const int k = (int)(rng.next() * (double)(size_t)npp);
    return (uint32_t)(piece * npp + npp - 1 - k);
  };
  for (int32_t n = 0; n < P; n++) {
    for (int32_t i = 0; i < wpp; i++) {
      const int64_t w = (int64_t)n * wpp + i;
      o->resistance[w] = (float)(rng.next() * 10 + 1);
      o->inductance[w] = (float)(rng.next() * p->L_scale + p->L_offset);
      o->capacitance[w] = (float)(rng.next() * 0.1);
      o->in_ptr[w] = pick(n);
      const bool in_piece = (100 * rng.next()) < p->pct_wire_in_piece;
      if (in_piece || P == 1) {
        o->out_ptr[w] = pick(n);
      } else {
        int nn = (int)(rng.next() * (P - 1));
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
  if (node_base)
    for (int64_t w = 0; w < W; w++) {
      o->in_ptr[w] += node_base;
      o->out_ptr[w] += node_base;
    }
  return CKT_OK;
}

}  // namespace ckt

extern "C" int ckt_generate(const ckt_gen_params *p, ckt_host_circuit *o) {
  int rc = ckt::generate_into(p, o, 0);
  if (rc) return rc;
  const int64_t W = (int64_t)p->num_pieces * p->wires_per_piece;
  for (int64_t k = 0; k < 10 * W; k++) o->current[k] = 0.f;
  for (int64_t k = 0; k < 9 * W; k++) o->voltage[k] = 0.f;
  return CKT_OK;
}
