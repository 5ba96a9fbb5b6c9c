// ckt_gen.h -- generator internals shared by the plain and batched paths.
#pragma once

#include <cstdint>

#include "ckt.h"

namespace ckt {

// drand48's 48-bit LCG with explicit state (values identical to libc's
// srand48/drand48: POSIX fixes the multiplier, increment and seeding).
struct Lcg48 {
  uint64_t x;
  explicit Lcg48(int64_t seed) : x((((uint64_t)seed & 0xffffffffull) << 16) | 0x330Eull) {}
  double next() {
    x = (0x5DEECE66Dull * x + 0xBull) & 0xffffffffffffull;
    return (double)x * 0x1p-48;  // exact: 48 bits fit a double's mantissa
  }
};

// Fills the graph, locations and initial node values of one circuit (not
// its zero wire state); node pointers are offset by node_base.
int generate_into(const ckt_gen_params *p, const ckt_host_circuit *o, uint32_t node_base);

}  // namespace ckt
