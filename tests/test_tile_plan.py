"""The node-tile plan of the tiled distribute_charge pass, on the CPU.

The plan builder (legionorigins_gb300/csrc/ckt_graph.cpp) is compiled with
g++ into a small checker that builds random graphs through build_node_csr,
plans every tile, and replays the GPU kernel's walk over the plan exactly
(stream steps read the chunk's staged currents, ghost steps the runs of
in-end and out-end currents the packing kernel stores for them, checked to
be each the step's wires in order; every consumer lane sums its list of
whole node runs,
private nodes in place, shared/ghost nodes through folds flushed at group
starts).  The result must equal, bit for bit, the sequential sum in CSR
order that the gather form computes; the plan's layout invariants (16-byte
blocks, step sizes, node ownership by warp, one run per node per step,
lists opening with a head) are checked on the way.  The whole-circuit plan
is then replayed as the library uploads it: its packing list (each ghost
slot once, sorted by source block and slot, with consistent block offsets
and end flags) fills a ghost buffer whose padding stays NaN, every tile
walks the concatenated steps from there, and the sums must match again.
"""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CSRC = os.path.join(ROOT, "legionorigins_gb300", "csrc")
INCLUDE = os.path.join(ROOT, "include")
CUDA = os.environ.get("CUDA_HOME", "/usr/local/cuda")

SOURCE = r'''
#include "ckt_graph.cpp"
#include <cstring>
#include <random>
namespace ckt {
int set_error(int status, const char *, ...) { return status; }
}
using namespace ckt;
static float fmul(float a, float b) { volatile float r = a * b; return r; }
static float fadd(float a, float b) { volatile float r = a + b; return r; }
#define FAIL(...) do { printf(__VA_ARGS__); printf("\n"); return 1; } while (0)

static int run(int P, int npp, int wpp, int nshared, double pct, uint64_t seed) {
  std::mt19937_64 rng(seed);
  const int W = P * wpp, N = P * npp;
  std::vector<ckt_piece> pieces(P);
  for (int k = 0; k < P; k++)
    pieces[k] = {(uint32_t)(k * wpp), (uint32_t)wpp, (uint32_t)(k * npp), (uint32_t)npp};
  std::vector<uint32_t> in(W), out(W);
  std::vector<uint8_t> il(W), ol(W);
  auto loc_of = [&](uint32_t x, int k) -> uint8_t {
    if ((int)(x / npp) != k) return CKT_GHOST_PTR;
    return (int)(x % npp) < nshared ? CKT_SHARED_PTR : CKT_PRIVATE_PTR;
  };
  for (int k = 0; k < P; k++)
    for (int i = 0; i < wpp; i++) {
      const int w = k * wpp + i;
      in[w] = k * npp + rng() % npp;
      il[w] = loc_of(in[w], k);
      if ((rng() % 1000000) / 1e4 < pct || P == 1 || nshared == 0) {
        out[w] = k * npp + rng() % npp;
      } else {
        int q = rng() % P;
        if (q == k) q = (q + 1) % P;
        out[w] = q * npp + rng() % nshared;
      }
      ol[w] = loc_of(out[w], k);
    }
  std::vector<uint32_t> off, ent;
  int64_t Wn = 0;
  if (build_node_csr(pieces.data(), P, N, in.data(), out.data(), il.data(), ol.data(), off, ent,
                     &Wn, nullptr))
    FAIL("graph rejected");
  std::vector<float> I0(W), I9(W), q0(N);
  std::uniform_real_distribution<float> U(-1, 1);
  for (int w = 0; w < W; w++) {
    I0[w] = U(rng) * (rng() % 7 == 0 ? 1e6f : 1.f);
    I9[w] = rng() % 50 == 0 ? -0.0f : U(rng);
  }
  for (int x = 0; x < N; x++) q0[x] = rng() % 3 == 0 ? -0.0f : U(rng);
  const float dt = 1e-6f;
  auto val = [&](uint32_t u) {
    return (u & 2u) ? fmul(dt, I9[u >> 2]) : fmul(-dt, I0[u >> 2]);
  };
  std::vector<float> ref(N), got(N);
  for (int x = 0; x < N; x++) {  // the gather form: CSR order
    const uint32_t b = off[x] & kOffsetMask, e = off[x + 1] & kOffsetMask;
    float acc = q0[x];
    if (off[x] & kPrivateBit) {
      for (uint32_t i = b; i < e; i++) acc = fadd(acc, val(ent[i]));
    } else {
      float fold = 0.f;
      for (uint32_t i = b; i < e; i++) {
        if ((ent[i] & 1u) && i != b) { acc = fadd(acc, fold); fold = 0.f; }
        fold = fadd(fold, val(ent[i]));
      }
      if (e > b) acc = fadd(acc, fold);
    }
    ref[x] = acc;
  }
  const uint32_t TN = kTileNodesMax, T = (N + TN - 1) / TN;
  for (uint32_t t = 0; t < T; t++) {
    TilePlan tp;
    std::vector<uint64_t> keys, sparse;
    const uint32_t x0 = t * TN, xe = std::min<uint32_t>(N, x0 + TN), nn = xe - x0;
    plan_tile(off.data(), ent.data(), x0, xe, tp, keys, sparse);
    std::vector<float> sacc(q0.begin() + x0, q0.begin() + xe), sfold(nn, 0.f);
    if (tp.ent.size() % 4 || tp.gsrc.size() % 4) FAIL("tile arrays not in 16-byte units");
    for (const uint4 &st : tp.steps) {
      if (st.x % 4 || st.y % 4 || st.w % 4) FAIL("step block not 16-byte aligned");
      if (st.y < kStepHeaderWords || st.y > kStepHeaderWords + kStepEntriesMax)
        FAIL("step block size %u", st.y);
      const bool stream = (st.z & kGhostStep) == 0u;
      const uint16_t *hdr = reinterpret_cast<const uint16_t *>(tp.ent.data() + st.x);
      const uint32_t total = hdr[kTileLanes];
      if (total > st.y - kStepHeaderWords) FAIL("entry count");
      const uint32_t *sent = tp.ent.data() + st.x + kStepHeaderWords;
      std::vector<float> sval(2 * kChunkWires, 0.f);
      uint32_t nrun[2] = {kChunkWires, kChunkWires};
      if (stream) {
        for (uint32_t i = 0; i < kChunkWires && st.z * kChunkWires + i < (uint32_t)W; i++) {
          sval[i] = I0[st.z * kChunkWires + i];
          sval[kChunkWires + i] = I9[st.z * kChunkWires + i];
        }
      } else {
        nrun[0] = (st.z >> kGhostCountBits) & kGhostCountMask;
        nrun[1] = st.z & kGhostCountMask;
        if (nrun[0] + nrun[1] != total) FAIL("ghost values %u + %u for %u entries", nrun[0], nrun[1], total);
        uint32_t g = st.w;
        for (uint32_t e = 0; e < 2; e++) {
          const uint32_t np = (nrun[e] + 3u) & ~3u;
          if (g + np > tp.gsrc.size()) FAIL("ghost run out of bounds");
          for (uint32_t i = 0; i < np; i++) {
            const uint32_t src = tp.gsrc[g + i];
            if (i >= nrun[e]) {
              if (src != kTePad) FAIL("ghost padding");
              continue;
            }
            if (src == kTePad || (src & 1u) != e) FAIL("ghost slot end");
            if (i > 0 && src <= tp.gsrc[g + i - 1]) FAIL("ghost run not in wire order");
            sval[e * kChunkWires + i] = e ? I9[src >> 1] : I0[src >> 1];
          }
          g += np;
        }
      }
      std::vector<int> seen(nn, 0);
      for (uint32_t l = 0; l < kTileLanes; l++) {
        const uint32_t b = hdr[l], e = l + 1 < kTileLanes ? hdr[l + 1] : total;
        if (b > e || e > total) FAIL("lane list bounds");
        uint32_t node = 0xffffffffu;
        float acc = 0.f, fold = 0.f;
        for (uint32_t p = b; p < e; p++) {
          const uint32_t u = sent[p], end = (u & kTeEnd) ? 1u : 0u;
          if ((u & (kChunkWires - 1)) >= nrun[end]) FAIL("ghost index out of its run");
          const float v = sval[end * kChunkWires + (u & (kChunkWires - 1))];
          const uint32_t x = (u >> kTeNodeShift) & (kTileNodesMax - 1);
          if (u & kTeHead) {
            if (node != 0xffffffffu) { sacc[node] = acc; sfold[node] = fold; }
            if (x >= nn || x % kTileWarps != l / 32) FAIL("node %u in lane %u", x, l);
            if (seen[x]++) FAIL("node %u has two runs in a step", x);
            node = x;
            acc = sacc[node];
            fold = sfold[node];
          } else if (p == b || x != node) {
            FAIL("run does not open with its head");
          }
          const float c = end ? fmul(dt, v) : fmul(-dt, v);
          if (u & kTePriv) {
            acc = fadd(acc, c);
          } else {
            if (u & kTeFlush) { acc = fadd(acc, fold); fold = 0.f; }
            fold = fadd(fold, c);
          }
        }
        if (node != 0xffffffffu) { sacc[node] = acc; sfold[node] = fold; }
      }
    }
    for (uint32_t i = 0; i < nn; i++) {
      const uint32_t x = x0 + i;
      float q = sacc[i];
      if (!(off[x] & kPrivateBit) && (off[x + 1] & kOffsetMask) > (off[x] & kOffsetMask))
        q = fadd(q, sfold[i]);
      got[x] = q;
    }
  }
  for (int x = 0; x < N; x++)
    if (memcmp(&got[x], &ref[x], 4)) FAIL("node %d: %a against %a", x, got[x], ref[x]);

  // The whole-circuit plan as the library uploads it: the packing list
  // fills the ghost buffer (padding slots stay NaN and must never be read),
  // and every tile replays from the concatenated steps and entries.
  HostTilePlan hp;
  if (make_tile_plan((uint32_t)N, W, off, ent, TN, hp)) FAIL("make_tile_plan failed");
  if (hp.T != T || hp.tile_step.size() != T + 1 || hp.tile_step[T] != hp.steps.size())
    FAIL("tile step table");
  std::vector<float> ghost((size_t)hp.gslots, NAN);
  std::vector<int> filled((size_t)hp.gslots, 0);
  for (size_t k = 0; k < hp.glist.size(); k++) {
    const uint2 g = hp.glist[k];
    if (g.x >= (uint64_t)hp.gslots || filled[g.x]++) FAIL("ghost slot %u twice or out of range", g.x);
    if ((g.y >> 1) >= (uint32_t)W) FAIL("ghost source wire out of range");
    if (k > 0) {
      const uint2 p = hp.glist[k - 1];
      const uint32_t bp = (p.y >> 1) / kPackWires, bk = (g.y >> 1) / kPackWires;
      if (bp > bk || (bp == bk && p.x >= g.x)) FAIL("packing list not sorted by (block, slot)");
    }
    ghost[g.x] = (g.y & 1u) ? I9[g.y >> 1] : I0[g.y >> 1];
  }
  if (hp.gblock.size() != hp.nblocks + 1 || hp.gblock[hp.nblocks] != hp.glist.size())
    FAIL("packing block table size");
  for (uint32_t b = 0; b < hp.nblocks; b++) {
    const uint32_t f = hp.gblock[b] & kPackFirstMask, l = hp.gblock[b + 1] & kPackFirstMask;
    if (f > l) FAIL("packing block %u runs backwards", b);
    bool in = false, out = false;
    for (uint32_t k = f; k < l; k++) {
      if ((hp.glist[k].y >> 1) / kPackWires != b) FAIL("entry %u outside its block %u", k, b);
      ((hp.glist[k].y & 1u) ? out : in) = true;
    }
    if (in != ((hp.gblock[b] & kPackHasIn) != 0) || out != ((hp.gblock[b] & kPackHasOut) != 0))
      FAIL("packing block %u flags", b);
  }
  for (uint32_t t = 0; t < T; t++) {
    const uint32_t x0 = t * TN, xe = std::min<uint32_t>(N, x0 + TN), nn = xe - x0;
    std::vector<float> sacc(q0.begin() + x0, q0.begin() + xe), sfold(nn, 0.f);
    for (uint32_t si = hp.tile_step[t]; si < hp.tile_step[t + 1]; si++) {
      const uint4 st = hp.steps[si];
      const uint16_t *hdr = reinterpret_cast<const uint16_t *>(hp.ent.data() + st.x);
      const uint32_t total = hdr[kTileLanes];
      const uint32_t *sent = hp.ent.data() + st.x + kStepHeaderWords;
      std::vector<float> sval(2 * kChunkWires, NAN);
      if ((st.z & kGhostStep) == 0u) {
        for (uint32_t i = 0; i < kChunkWires && st.z * kChunkWires + i < (uint32_t)W; i++) {
          sval[i] = I0[st.z * kChunkWires + i];
          sval[kChunkWires + i] = I9[st.z * kChunkWires + i];
        }
      } else {
        const uint32_t n0 = (((st.z >> kGhostCountBits) & kGhostCountMask) + 3u) & ~3u;
        const uint32_t n1 = ((st.z & kGhostCountMask) + 3u) & ~3u;
        if (st.w % 4 || st.w + n0 + n1 > hp.gslots) FAIL("ghost run of a step out of range");
        for (uint32_t i = 0; i < n0; i++) sval[i] = ghost[st.w + i];
        for (uint32_t i = 0; i < n1; i++) sval[kChunkWires + i] = ghost[st.w + n0 + i];
      }
      for (uint32_t l = 0; l < kTileLanes; l++) {
        const uint32_t b = hdr[l], e = l + 1 < kTileLanes ? hdr[l + 1] : total;
        uint32_t node = 0xffffffffu;
        float acc = 0.f, fold = 0.f;
        for (uint32_t p = b; p < e; p++) {
          const uint32_t u = sent[p], end = (u & kTeEnd) ? 1u : 0u;
          const float v = sval[end * kChunkWires + (u & (kChunkWires - 1))];
          if (std::isnan(v)) FAIL("tile %u read an unfilled value", t);
          if (u & kTeHead) {
            if (node != 0xffffffffu) { sacc[node] = acc; sfold[node] = fold; }
            node = (u >> kTeNodeShift) & (kTileNodesMax - 1);
            acc = sacc[node];
            fold = sfold[node];
          }
          const float c = end ? fmul(dt, v) : fmul(-dt, v);
          if (u & kTePriv) {
            acc = fadd(acc, c);
          } else {
            if (u & kTeFlush) { acc = fadd(acc, fold); fold = 0.f; }
            fold = fadd(fold, c);
          }
        }
        if (node != 0xffffffffu) { sacc[node] = acc; sfold[node] = fold; }
      }
    }
    for (uint32_t i = 0; i < nn; i++) {
      const uint32_t x = x0 + i;
      float q = sacc[i];
      if ((hp.mask[(size_t)t * (kTileNodesMax / 32) + i / 32] >> (i % 32)) & 1u) q = fadd(q, sfold[i]);
      if (memcmp(&q, &ref[x], 4)) FAIL("whole plan, node %u: %a against %a", x, q, ref[x]);
    }
  }
  printf("ghost %zu %d ", hp.glist.size(), hp.staged ? 1 : 0);
  return 0;
}

int main() {
  struct { int P, npp, wpp, ns; double pct; } cases[] = {
      {16, 2048, 8192, 256, 95},    // dense chunks, ghost contributions packed
      {4, 8192, 16384, 4096, 50},   // heavy cross-piece reduction
      {8, 1000, 4003, 100, 80},     // ragged wire count, tiles spanning pieces
      {3, 5, 7, 2, 50},             // tiny
      {1, 9000, 36000, 0, 100},     // one piece, a last tile of 808 nodes
      {5, 20000, 3, 100, 0},        // nearly no wires, all cross
      {7, 3, 3000, 3, 60},          // hub nodes: runs longer than a step
      {1, 1, 8192, 0, 100},         // one node: 16384 entries
      {16, 8192, 8192, 4096, 50},   // half the wires cross: staged packing
  };
  int rc = 0;
  for (int i = 0; i < 9; i++) {
    const int r = run(cases[i].P, cases[i].npp, cases[i].wpp, cases[i].ns, cases[i].pct, 11 + i);
    printf("case %d: %s\n", i, r ? "FAILED" : "ok");
    rc |= r;
  }
  return rc;
}
'''


@pytest.mark.skipif(shutil.which("g++") is None, reason="g++ not available")
def test_tile_plan_replays_to_the_gather_bits(tmp_path):
    src = tmp_path / "tile_plan_check.cc"
    src.write_text(SOURCE)
    exe = tmp_path / "tile_plan_check"
    lib = os.path.join(CUDA, "lib64")
    subprocess.run(["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-I", INCLUDE, "-I", CSRC,
                    "-I", os.path.join(CUDA, "include"), "-o", str(exe), str(src), "-L", lib,
                    "-lcudart", "-lpthread", f"-Wl,-rpath,{lib}"], check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True, timeout=300)
    assert out.returncode == 0, out.stdout + out.stderr
    assert out.stdout.count(": ok") == 9, out.stdout
    # both packing forms and plans without ghost steps are among the cases
    ghosts = [tuple(map(int, line.split("ghost ")[1].split()[:2]))
              for line in out.stdout.splitlines() if "ghost " in line]
    assert any(n > 0 and staged for n, staged in ghosts), out.stdout
    assert any(n > 0 and not staged for n, staged in ghosts), out.stdout
    assert any(n == 0 for n, _ in ghosts), out.stdout
