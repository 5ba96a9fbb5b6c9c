"""The oracle against the REFERENCE ITSELF (CPU only).

tests/golden/*.npz were produced by the reference's own apps/circuit/circuit.cc
(compiled unmodified through oracle/refshim, see tests/golden/make_golden.py):
its generator, its CPU leaf tasks (CPU-task initialisation, STEPS = 10000)
and its loop.  The oracle must reproduce them bit for bit.  When the
reference tree is present, a few more shapes are checked against the live
binary.
"""
import glob
import os

import numpy as np
import pytest

from conftest import GOLDEN, load_npz, same_bits

GEN_FIELDS = ["in_ptr", "out_ptr", "in_loc", "out_loc", "L", "R", "C", "current", "voltage",
              "charge", "node_voltage", "cap", "leak", "locator"]
STATE = ["current", "voltage", "charge", "node_voltage"]


def _params(O, arr):
    P, npp, wpp, pct, seed = (int(x) for x in arr)
    return O.GenParams(P, npp, wpp, pct, seed)


@pytest.mark.parametrize("path", sorted(glob.glob(os.path.join(GOLDEN, "gen_*.npz"))),
                         ids=lambda p: os.path.basename(p))
def test_generator_matches_reference(oracle, path):
    g = load_npz(os.path.basename(path))
    c = oracle.generate(_params(oracle, g["params"]))
    for k in GEN_FIELDS:
        assert same_bits(getattr(c, k), g[k]), k


@pytest.mark.parametrize("path", sorted(glob.glob(os.path.join(GOLDEN, "sim_*.npz"))),
                         ids=lambda p: os.path.basename(p))
def test_tasks_match_reference(oracle, path):
    g = load_npz(os.path.basename(path))
    p = _params(oracle, g["params"])
    c = oracle.generate(p)
    for k in GEN_FIELDS:
        setattr(c, k, np.ascontiguousarray(g["start_" + k]))
    oracle.simulate(c, int(g["loops"]), int(g["steps"]), quirk=True)
    for k in STATE:
        assert same_bits(getattr(c, k), g[k]), k
    if os.path.basename(path).startswith("sim_conv"):
        # the finite-regime fixtures really are finite
        for k in STATE:
            assert np.isfinite(g[k]).all(), k


def test_graph_invariants(oracle):
    """Generator invariants (load_circuit, circuit.cc:1140-1244)."""
    for args in [(4, 256, 1024, 95, 12345), (8, 64, 256, 50, 42), (6, 16, 64, 0, 11)]:
        p = oracle.GenParams(*args)
        c = oracle.generate(p)
        piece = np.arange(p.W) // p.wires_per_piece
        assert ((c.in_ptr // p.nodes_per_piece) == piece).all()  # in-node in own piece
        own = (c.out_ptr // p.nodes_per_piece) == piece
        assert (c.out_loc[~own] == oracle.GHOST).all()
        assert (c.out_loc[own] != oracle.GHOST).all()
        shared = np.zeros(p.N, bool)
        shared[c.out_ptr[~own]] = True
        assert np.array_equal(c.locator == 0, shared)            # shared iff a ghost target
        assert np.array_equal(c.in_loc == oracle.SHARED, shared[c.in_ptr])
        assert np.array_equal(c.out_loc[own] == oracle.SHARED, shared[c.out_ptr[own]])
        assert (c.in_loc != oracle.GHOST).all()


def test_generator_single_piece(oracle):
    """P = 1: the reference's cross-piece branch is undefined (it indexes
    piece 1); the oracle keeps every wire in-piece and consumes the pct draw."""
    c = oracle.generate(oracle.GenParams(1, 7, 50, 50.0, 3))
    assert (c.out_loc != oracle.GHOST).all() and (c.locator == 1).all()


def test_fp32_fp64_agree_in_finite_regime(oracle):
    p = oracle.GenParams(4, 256, 1024, 95, 12345, L_offset=0.001)
    c32 = oracle.generate(p)
    c64 = c32.astype(np.float64)
    oracle.simulate(c32, 2, 4)
    oracle.simulate(c64, 2, 4)
    for k in STATE:
        a, b = getattr(c32, k).astype(np.float64), getattr(c64, k)
        assert np.isfinite(a).all() and np.isfinite(b).all()
        err = np.abs(a - b) / np.maximum(np.abs(b), 1e-3)
        assert err.max() < 1e-3, (k, err.max())


@pytest.mark.parametrize("quirk", [False, True])
def test_cpu_baseline_matches_serial_oracle(oracle, quirk):
    p = oracle.GenParams(8, 32, 128, 60, 5, L_offset=0.001)
    a = oracle.generate(p)
    b = a.copy()
    oracle.simulate(a, 3, 5, quirk=quirk)
    t = oracle.baseline_run(b, 3, 5, threads=3, quirk=quirk)
    assert t >= 0
    for k in STATE:
        assert same_bits(getattr(a, k), getattr(b, k)), k


@pytest.mark.skipif(not os.path.isdir("/root/reference/apps/circuit"),
                    reason="reference tree not present (only in the development container)")
@pytest.mark.parametrize("args,loops", [((5, 12, 40, 75, 2024), 2), ((7, 3, 11, 30, 77), 1)])
def test_live_reference(oracle, tmp_path, args, loops):
    oracle.build_ref()
    p = oracle.GenParams(*args)
    init, final = oracle.run_reference(p, loops, str(tmp_path))
    c = oracle.generate(p)
    for k in GEN_FIELDS:
        assert same_bits(getattr(c, k), getattr(init, k)), k
    oracle.simulate(c, loops, 10000, quirk=True)
    for k in STATE:
        assert same_bits(getattr(c, k), getattr(final, k)), k


# -- reduction microbenchmark (benchmarks/reductions/reducetest.cc) ---------------

@pytest.mark.parametrize("path", sorted(glob.glob(os.path.join(GOLDEN, "hist_*.npz"))),
                         ids=lambda p: os.path.basename(p))
def test_histogram_matches_reference(oracle, path):
    """The reference's master histogram after its three default cases is
    three times the oracle's histogram, bucket for bucket."""
    g = load_npz(os.path.basename(path))
    buckets, batches, bsize = (int(x) for x in g["params"])
    h = oracle.histogram(buckets, bsize, batches)
    assert h.sum() == batches * bsize
    assert np.array_equal(g["master"], (h.astype(np.uint64) * int(g["cases"])).astype(np.uint32))


def test_histogram_threads_equals_serial(oracle):
    h = oracle.histogram(4099, 3000, 13)
    for threads in (1, 2, 5, 16):
        got, secs = oracle.histogram_threads(4099, 3000, 13, threads)
        assert np.array_equal(got, h) and secs >= 0


def test_histogram_first_batch_wraps_32_bits(oracle):
    """Element indices are 32-bit unsigned like the benchmark's start + i:
    batch 2**12 of 2**20 elements starts again at index 0."""
    bs = 1 << 12
    a = oracle.histogram(977, bs, 1, first_batch=(1 << 20))
    b = oracle.histogram(977, bs, 1, first_batch=0)
    assert np.array_equal(a, b)
    # a batch straddling 2**32 equals its two halves
    first = (1 << 32) // bs - 1
    c = oracle.histogram(977, bs, 2, first_batch=first)
    d = oracle.histogram(977, bs, 1, first_batch=first) + oracle.histogram(977, bs, 1)
    assert np.array_equal(c, d)


def test_hist_rand_known_values(oracle):
    """myrand restated independently in Python (reducetest.cc:323-333)."""
    def myrand(ival, s1, s2):
        r = ival
        for j in range(16):
            r = (0x5DEECE66D * r + 0xB) & 0xFFFFFFFFFFFF
            r ^= s1 if (ival >> j) & 1 else s2
        return r & 0xFFFFFFFF

    for ival in (0, 1, 2, 12345, 0xFFFF, 0x10000, 0xFFFFFFFF, 0x12345678):
        assert oracle.lib().ocl_hist_rand(ival, 12345, 54321) == myrand(ival, 12345, 54321)


@pytest.mark.skipif(not os.path.isdir("/root/reference/benchmarks/reductions"),
                    reason="reference tree absent")
def test_histogram_live_reference(oracle, tmp_path):
    oracle.build_ref()
    for buckets, batches, bsize in [(3, 4, 1001), (100003, 2, 20000)]:
        m = oracle.run_reducetest(buckets, batches, bsize, str(tmp_path / f"{buckets}"))
        h = oracle.histogram(buckets, bsize, batches)
        assert np.array_equal(m, (3 * h.astype(np.uint64)).astype(np.uint32))
