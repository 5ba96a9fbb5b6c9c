"""The GPU generator's integer forms of load_circuit's drand48 expressions
(legionorigins_gb300/csrc/ckt_drand.cuh) against the double arithmetic they
replace, on the CPU: the header compiles as plain C++ and every helper must
give the same bits for random states, edge states and constructed rounding
ties."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "legionorigins_gb300", "csrc", "ckt_drand.cuh")

SOURCE = r'''
#include <cmath>
#include <cstdio>
#include <random>
#include "ckt_drand.cuh"
using namespace ckt::drand;
static uint64_t inv_mod_pow2(uint64_t a, int k) {
  uint64_t x = 1;
  for (int i = 0; i < 7; i++) x = x * (2 - a * x);
  return x & ((1ull << k) - 1);
}
int main() {
  std::mt19937_64 rng(12345);
  long bad = 0, n = 0;
  const uint64_t M48 = (1ull << 48) - 1;
  const uint64_t edge[] = {0, 1, 2, 3, M48, M48 - 1, 1ull << 47, (1ull << 47) - 1, (1ull << 47) + 1,
                           1ull << 24, (1ull << 24) + 1, 123456789};
  const uint32_t ns[] = {1, 2, 3, 7, 31, 32, 33, 64, 777, 4096, 16384, 65536, 1u << 24,
                         (1u << 30) + 3, 2147483647u};
  const double pcts[] = {0, 0.5, 50, 80, 83.25, 95, 99.999, 100, 100.5, -1};
  for (int i = 0; i < 300000; i++) {
    const uint64_t x = i < 12 ? edge[i] : (rng() & M48);
    const double u = (double)x * 0x1p-48;
    n++;
    bad += value(x) != u;
    bad += resistance(x) != (float)(u * 10 + 1);
    bad += node_voltage(x) != (float)(2 * u - 1);
    bad += node_capacitance(x) != (float)(u + 1);
    const uint32_t m = (i & 1) ? ns[i % 15] : (uint32_t)(rng() % 2147483647u) + 1;
    bad += trunc_mul(x, m) != (uint32_t)(int)(u * m);
    const double pct = (i % 3) ? pcts[i % 10] : 100 * u;  // also exactly at the boundary
    bad += pct_below(x, pct_threshold(pct)) != (100 * u < pct);
  }
  for (int i = 0; i < 300000; i++) {  // products whose dropped bits are exactly one half
    const uint32_t m = (uint32_t)((rng() % 2147483640u) + 3) | 1u;
    const int shift = 1 + (int)(rng() % 27);
    const uint64_t mask = (1ull << shift) - 1;
    const uint64_t low = ((1ull << (shift - 1)) * inv_mod_pow2(m, shift)) & mask;
    const uint64_t x = ((rng() & M48) & ~mask) | low;
    const double u = (double)x * 0x1p-48;
    n++;
    bad += trunc_mul(x, m) != (uint32_t)(int)(u * m);
  }
  printf("checked %ld bad %ld\n", n, bad);
  return bad != 0;
}
'''


@pytest.mark.skipif(shutil.which("g++") is None, reason="g++ not available")
def test_integer_drand_helpers_match_double_arithmetic(tmp_path):
    src = tmp_path / "check.cc"
    src.write_text(SOURCE)
    exe = tmp_path / "check"
    subprocess.run(["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-I",
                    os.path.dirname(HEADER), "-o", str(exe), str(src)], check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True)
    assert out.returncode == 0 and "bad 0" in out.stdout, out.stdout + out.stderr
