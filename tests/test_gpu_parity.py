"""Parity of the CUDA path with the oracle and with the reference itself.

Every kernel runs through the C ABI (include/ckt.h).  Bars:
  * EXACT mode: bit-identical to the fp32 oracle (every NaN equal to every
    NaN), and through CPU-task initialisation bit-identical to the
    reference's own CPU tasks (tests/golden/sim_*.npz);
  * FAST mode: |gpu - oracle| <= 1e-5 * max(|oracle|, 1e-6) per finite
    element in the finite regime, identical NaN/Inf classes at the
    configured step counts; max and RMS error against the fp64 oracle are
    reported.
"""
import os

import numpy as np
import pytest

from conftest import GOLDEN, load_npz, rel_err, same_bits

pytestmark = pytest.mark.gpu

STATE = ["current", "voltage", "charge", "node_voltage"]
FIELDS = ["in_ptr", "out_ptr", "in_loc", "out_loc", "L", "R", "C", "current", "voltage",
          "charge", "node_voltage", "cap", "leak", "locator"]
FAST_RTOL = 1e-5
FAST_TINY = 1e-6


def host_dict(c):
    return {k: np.ascontiguousarray(getattr(c, k)) for k in FIELDS}


def device(cuda, c):
    from legionorigins_gb300 import circuit as C

    p = c.params
    return C.DeviceCircuit(host_dict(c), C.Shape(p.num_pieces, p.nodes_per_piece,
                                                 p.wires_per_piece))


def run_gpu(cuda, dc, loops, steps, mode, init=0, per_piece=False, blocking=False):
    from legionorigins_gb300 import circuit as C

    prm = C.params(steps, mode, init)
    for _ in range(loops):
        if per_piece:
            dc.loop_per_piece(prm, blocking=blocking)
        else:
            dc.loop_index_space(prm)
    cuda.cuda.synchronize()
    return dc.to_host()


def cnc_only(cuda, dc, steps, mode, init=0):
    import ctypes

    from legionorigins_gb300 import circuit as C
    from legionorigins_gb300 import check, lib

    prm = C.params(steps, mode, init)
    check(lib().ckt_calc_new_currents_all(dc.graph.handle, dc.wires(), dc.nodes(),
                                          ctypes.byref(prm), None))
    cuda.cuda.synchronize()
    return dc.to_host()


SHAPES = {
    "cfg0": (4, 256, 1024, 95, 12345),
    "ragged": (3, 5, 7, 50, 7),
    "one_node_per_piece": (2, 1, 3, 0, 1),
    "all_cross": (6, 16, 64, 0, 11),
    "all_in_piece": (5, 33, 100, 100, 5),
    "single_piece": (1, 7, 50, 50, 3),
    "heavy_reduction": (16, 64, 256, 50, 42),
}


@pytest.mark.parametrize("steps", [1, 2, 4, 6, 1000])
def test_cnc_exact_bit_exact(cuda, oracle, steps):
    c = oracle.generate(oracle.GenParams(4, 256, 1024, 95, 12345, L_offset=0.001))
    # nonzero wire state so every term of the recurrence is exercised
    rng = np.random.default_rng(steps)
    c.current[:] = rng.uniform(-1, 1, c.current.shape).astype(np.float32)
    c.voltage[:] = rng.uniform(-1, 1, c.voltage.shape).astype(np.float32)
    dc = device(cuda, c)
    got = cnc_only(cuda, dc, steps, mode=0)
    oracle.calc_new_currents(c, steps)
    for k in ("current", "voltage"):
        assert same_bits(got[k], getattr(c, k)), k


@pytest.mark.parametrize("name", sorted(n for n in os.listdir(GOLDEN) if n.startswith("sim_")))
def test_gpu_matches_reference_cpu_tasks(cuda, oracle, name):
    """GPU (CPU-task initialisation, EXACT) against the reference's own
    circuit.cc output: bit for bit."""
    g = load_npz(name)
    P, npp, wpp, pct, seed = (int(x) for x in g["params"])
    c = oracle.generate(oracle.GenParams(P, npp, wpp, pct, seed))
    for k in FIELDS:
        setattr(c, k, np.ascontiguousarray(g["start_" + k]))
    dc = device(cuda, c)
    got = run_gpu(cuda, dc, int(g["loops"]), int(g["steps"]), mode=0, init=1)
    for k in STATE:
        assert same_bits(got[k], g[k]), k


@pytest.mark.parametrize("shape", sorted(SHAPES))
@pytest.mark.parametrize("steps,loops", [(1, 1), (4, 2), (6, 5), (1000, 2)])
def test_full_loop_exact(cuda, oracle, shape, steps, loops):
    c = oracle.generate(oracle.GenParams(*SHAPES[shape], L_offset=0.001))
    dc = device(cuda, c)
    got = run_gpu(cuda, dc, loops, steps, mode=0)
    oracle.simulate(c, loops, steps)
    for k in STATE:
        assert same_bits(got[k], getattr(c, k)), (shape, k)


@pytest.mark.parametrize("shape", ["cfg0", "heavy_reduction", "all_cross", "one_node_per_piece"])
def test_per_piece_calls_equal_index_space(cuda, oracle, shape):
    """The reference-shaped per-piece calls (CNC, DC into fold instances,
    fold application in piece order, UV by locator) and the fused
    index-space launches give identical bits."""
    c = oracle.generate(oracle.GenParams(*SHAPES[shape], L_offset=0.001))
    a = run_gpu(cuda, device(cuda, c), 3, 4, mode=0, per_piece=True)
    b = run_gpu(cuda, device(cuda, c), 3, 4, mode=0, per_piece=False)
    for k in STATE:
        assert np.array_equal(a[k].view(np.uint32), b[k].view(np.uint32)), k
    oracle.simulate(c, 3, 4)
    for k in STATE:
        assert same_bits(a[k], getattr(c, k)), k


@pytest.mark.parametrize("shape", [(2, 1, 5000, 50, 3), (3, 2, 9000, 0, 4), (1, 1, 3000, 95, 5)],
                         ids=lambda s: "x".join(str(v) for v in s))
def test_hub_nodes_exact(cuda, oracle, shape):
    """One or two nodes per piece and thousands of wires: a node's run spans
    several staging chunks of distribute_charge (more than 4096 entries)."""
    c = oracle.generate(oracle.GenParams(*shape, L_offset=0.001))
    a = run_gpu(cuda, device(cuda, c), 2, 2, mode=0)
    b = run_gpu(cuda, device(cuda, c), 2, 2, mode=0, per_piece=True)
    d = device(cuda, c)
    from legionorigins_gb300 import circuit as C
    d.run_loops(C.params(2, 0), 2)
    cuda.cuda.synchronize()
    f = d.to_host()
    oracle.simulate(c, 2, 2)
    for k in STATE:
        for got in (a, b, f):
            assert same_bits(got[k], getattr(c, k)), k


@pytest.mark.parametrize("P", [1, 2, 4])
@pytest.mark.parametrize("npp", [1, 2, 3])
@pytest.mark.parametrize("wpp", [1, 3, 8])
def test_small_shapes_exact(cuda, oracle, P, npp, wpp):
    """Every small shape: one piece, one node per piece (each in-piece wire
    has in == out), ragged wire counts; index-space and per-piece calls."""
    c = oracle.generate(oracle.GenParams(P, npp, wpp, 50, 7 * P + npp + wpp, L_offset=0.001))
    a = run_gpu(cuda, device(cuda, c), 2, 2, mode=0)
    b = run_gpu(cuda, device(cuda, c), 2, 2, mode=0, per_piece=True)
    oracle.simulate(c, 2, 2)
    for k in STATE:
        assert same_bits(a[k], getattr(c, k)), k
        assert same_bits(b[k], getattr(c, k)), k


@pytest.mark.parametrize("shape", sorted(SHAPES))
@pytest.mark.parametrize("mode,init", [(0, 0), (1, 0), (2, 0), (0, 1)])
def test_fused_loops_equal_index_space(cuda, oracle, shape, mode, init):
    """ckt_run_loops_all (contributions scattered by calc_new_currents, one
    node pass for distribute_charge + update_voltages) gives the bits of the
    three index-space launches per loop."""
    from legionorigins_gb300 import circuit as C

    c = oracle.generate(oracle.GenParams(*SHAPES[shape], L_offset=0.001))
    a_dev, b_dev = device(cuda, c), device(cuda, c)
    prm = C.params(3, mode, init)
    a_dev.run_loops(prm, 4)
    for _ in range(4):
        b_dev.loop_index_space(prm)
    cuda.cuda.synchronize()
    a, b = a_dev.to_host(), b_dev.to_host()
    for k in STATE:
        assert np.array_equal(a[k].view(np.uint32), b[k].view(np.uint32)), (shape, k)
    if mode == 0 and init == 0:
        oracle.simulate(c, 4, 3)
        for k in STATE:
            assert same_bits(a[k], getattr(c, k)), (shape, k)


def test_fused_loops_without_wires(cuda, oracle):
    """No wires: every loop is the voltage update alone."""
    from legionorigins_gb300 import circuit as C

    c = oracle.generate(oracle.GenParams(3, 4, 0, 95, 1, L_offset=0.001))
    c.charge[:] = np.linspace(-1, 1, c.charge.size, dtype=np.float32)
    dev = device(cuda, c)
    dev.run_loops(C.params(5, 0), 2)
    cuda.cuda.synchronize()
    got = dev.to_host()
    oracle.simulate(c, 2, 5)
    for k in STATE:
        assert same_bits(got[k], getattr(c, k)), k


@pytest.mark.parametrize("mode", [0, 1])
def test_blocking_task_forms_equal_async(cuda, oracle, mode):
    """ckt_*_sync (a device wait after every task, like the reference's GPU
    task bodies) gives the same bits as the asynchronous calls."""
    c = oracle.generate(oracle.GenParams(*SHAPES["heavy_reduction"], L_offset=0.001))
    a = run_gpu(cuda, device(cuda, c), 2, 3, mode=mode, per_piece=True, blocking=True)
    b = run_gpu(cuda, device(cuda, c), 2, 3, mode=mode, per_piece=True)
    for k in STATE:
        assert np.array_equal(a[k].view(np.uint32), b[k].view(np.uint32)), k


def test_blocking_form_reports_bad_arguments(cuda):
    import ctypes

    from legionorigins_gb300 import CktError, Nodes, Piece, check, lib

    piece = Piece(0, 4, 0, 4)
    rc = lib().ckt_update_voltages_sync(ctypes.byref(piece), Nodes(), Nodes(), None, None)
    with pytest.raises(CktError):
        check(rc)


@pytest.mark.parametrize("steps,loops", [(1, 1), (2, 1), (3, 2), (4, 2), (6, 1)])
def test_fast_mode_within_tolerance(cuda, oracle, steps, loops):
    c = oracle.generate(oracle.GenParams(4, 256, 1024, 95, 12345, L_offset=0.001))
    c64 = c.astype(np.float64)
    got = run_gpu(cuda, device(cuda, c), loops, steps, mode=1)
    oracle.simulate(c, loops, steps)
    oracle.simulate(c64, loops, steps)
    for k in STATE:
        ref = getattr(c, k)
        assert np.isfinite(ref).all(), "case left the finite regime"
        assert np.array_equal(np.isfinite(got[k]), np.isfinite(ref)), k
        r = np.abs(got[k].astype(np.float64) - ref) / np.maximum(np.abs(ref), FAST_TINY)
        assert r.max() <= FAST_RTOL, (k, r.max())
        e64 = rel_err(got[k], getattr(c64, k), FAST_TINY)
        print(f"fast S={steps} Lp={loops} {k}: max rel vs fp32 oracle {r.max():.2e}, "
              f"vs fp64 max {e64.max():.2e} rms {np.sqrt((e64 ** 2).mean()):.2e}")


@pytest.mark.parametrize("steps,loops", [(1, 1), (3, 2), (1000, 2)])
@pytest.mark.parametrize("init", [0, 1])
def test_paired_fast_equals_scalar_fast(cuda, oracle, steps, loops, init):
    """The paired-instruction FAST step rounds every segment exactly as the
    one-at-a-time FAST step: identical bits."""
    c = oracle.generate(oracle.GenParams(4, 256, 1024, 95, 12345, L_offset=0.001))
    rng = np.random.default_rng(7)
    c.current[:] = rng.uniform(-1, 1, c.current.shape).astype(np.float32)
    c.voltage[:] = rng.uniform(-1, 1, c.voltage.shape).astype(np.float32)
    a = run_gpu(cuda, device(cuda, c), loops, steps, mode=1, init=init)
    b = run_gpu(cuda, device(cuda, c), loops, steps, mode=2, init=init)
    for k in STATE:
        assert np.array_equal(a[k].view(np.uint32), b[k].view(np.uint32)), k


def test_fast_mode_classes_at_configured_steps(cuda, oracle):
    c = oracle.generate(oracle.GenParams(4, 256, 1024, 95, 12345, L_offset=0.001))
    got = run_gpu(cuda, device(cuda, c), 5, 1000, mode=1)
    oracle.simulate(c, 5, 1000)
    for k in STATE:
        ref = getattr(c, k)
        for cls in (np.isnan, np.isposinf, np.isneginf):
            assert np.array_equal(cls(got[k]), cls(ref)), (k, cls.__name__)
        fin = np.isfinite(ref)
        if fin.any():
            r = np.abs(got[k][fin].astype(np.float64) - ref[fin]) / np.maximum(np.abs(ref[fin]), FAST_TINY)
            assert r.max() <= FAST_RTOL, k


def test_sanity_check_flags_a_corrupted_wire(cuda, oracle):
    import ctypes

    from legionorigins_gb300 import lib

    c = oracle.generate(oracle.GenParams(4, 16, 64, 80, 3))
    dc = device(cuda, c)
    dc.sanity_check()  # clean circuit passes
    dc.t["in_ptr"][70] = 5  # wire 70 is in piece 1 (nodes 16..31): in-node now outside it
    bad = ctypes.c_int64()
    rc = lib().ckt_sanity_check_wires(ctypes.byref(dc.pieces[1]), dc.wires(), dc.shape.N,
                                      ctypes.byref(bad), None)
    assert rc == 3 and bad.value == 70


def test_empty_pieces(cuda, oracle):
    c = oracle.generate(oracle.GenParams(3, 4, 0, 95, 1))
    got = run_gpu(cuda, device(cuda, c), 2, 10, mode=0)
    oracle.simulate(c, 2, 10)
    for k in STATE:
        assert same_bits(got[k], getattr(c, k)), k


@pytest.mark.slow
def test_config1_full_size_one_loop(cuda, oracle):
    """64 pieces x 16384 nodes x 65536 wires, S = 1000, EXACT.  CNC is
    checked on a slice of wires (each wire is independent given the node
    voltages), DC and UV on the whole circuit from the GPU's own currents;
    a second run must give identical bits (determinism)."""
    p = oracle.GenParams(64, 16384, 65536, 95, 12345, L_offset=0.001)
    c = oracle.generate(p)
    dc = device(cuda, c)
    import ctypes

    from legionorigins_gb300 import check, lib
    from legionorigins_gb300 import circuit as C

    prm = C.params(1000, 0)
    L, g, w, n = lib(), dc.graph.handle, dc.wires(), dc.nodes()
    check(L.ckt_calc_new_currents_all(g, w, n, ctypes.byref(prm), None))
    cuda.cuda.synchronize()
    after_cnc = dc.to_host()
    sl = slice(0, 20000)
    ref = c.copy()
    oracle.calc_new_currents(ref, 1000, w_begin=0, w_end=20000)
    for k in ("current", "voltage"):
        assert same_bits(after_cnc[k][:, sl], getattr(ref, k)[:, sl]), k
    check(L.ckt_distribute_charge_all(g, w, n, ctypes.byref(prm), None))
    check(L.ckt_update_voltages_all(g, n, None))
    cuda.cuda.synchronize()
    got = dc.to_host()
    c.current[:], c.voltage[:] = after_cnc["current"], after_cnc["voltage"]
    oracle.distribute_charge(c)
    oracle.update_voltages(c)
    for k in ("charge", "node_voltage"):
        assert same_bits(got[k], getattr(c, k)), k
    dc2 = device(cuda, oracle.generate(p))
    got2 = run_gpu(cuda, dc2, 1, 1000, mode=0)
    for k in STATE:
        assert np.array_equal(got[k].view(np.uint32), got2[k].view(np.uint32)), k


@pytest.mark.slow
def test_config2_heavy_reduction_full_size(cuda, oracle):
    """128 pieces x 8192 nodes x 32768 wires, 50% in-piece: half of the
    scatters land on shared/ghost nodes.  Whole-circuit bit parity in the
    finite regime (S = 2, two loops)."""
    p = oracle.GenParams(128, 8192, 32768, 50, 12345, L_offset=0.001)
    c = oracle.generate(p)
    got = run_gpu(cuda, device(cuda, c), 2, 2, mode=0)
    oracle.simulate(c, 2, 2)
    for k in STATE:
        assert same_bits(got[k], getattr(c, k)), k
    assert (c.locator == 0).mean() > 0.3


@pytest.mark.parametrize("shape", ["heavy_reduction", "cfg0", "all_cross"])
def test_separate_region_instances(cuda, oracle, shape):
    """The reference hands each task distinct region instances: private
    nodes, the piece's own shared nodes, the piece's ghost nodes (absolute
    indexing, only the instance's own nodes valid).  Here every instance holds
    NaN outside its nodes, so a wire end read from the wrong instance, or a
    charge applied to the wrong one, poisons the result.  The per-piece calls
    on separate instances give the bits of the index-space launches."""
    import ctypes

    from legionorigins_gb300 import Nodes, check, lib
    from legionorigins_gb300 import circuit as C

    torch = cuda
    P, npp, wpp, pct, seed = SHAPES[shape]
    N = P * npp
    c = oracle.generate(oracle.GenParams(P, npp, wpp, pct, seed, L_offset=0.001))
    ref, sep = device(cuda, c), device(cuda, c)
    prm = C.params(3, 0)
    L = lib()
    priv = c.locator == 1

    def masked(vals, mask):
        a = np.full(N, np.nan, np.float32)
        a[mask] = vals[mask]
        return torch.from_numpy(a).cuda()

    pq, pv, pc, pl = (masked(x, priv) for x in (c.charge, c.node_voltage, c.cap, c.leak))
    sq, sv, sc, sl = (masked(x, ~priv) for x in (c.charge, c.node_voltage, c.cap, c.leak))
    pvt = Nodes(pq.data_ptr(), pv.data_ptr(), pc.data_ptr(), pl.data_ptr())
    shr = Nodes(sq.data_ptr(), sv.data_ptr(), sc.data_ptr(), sl.data_ptr())
    locator = torch.from_numpy(c.locator).cuda()
    g, w = sep.graph.handle, sep.wires()
    sf, gf = sep.shr_fold.data_ptr(), sep.ghost_fold.data_ptr()
    for _ in range(2):
        ref.loop_index_space(prm)
        # calc_new_currents: the piece's own shared voltages and its ghost
        # voltages as two more instances, from the shared instance's values
        shv = sv.cpu().numpy()
        keep = []
        for k in range(P):
            own = np.zeros(N, bool)
            own[k * npp:(k + 1) * npp] = True
            own &= ~priv
            ws = slice(k * wpp, (k + 1) * wpp)
            ghost = np.zeros(N, bool)
            ghost[c.out_ptr[ws][c.out_loc[ws] == 2]] = True
            ov, gv = masked(shv, own), masked(shv, ghost)
            keep += [ov, gv]
            check(L.ckt_calc_new_currents(ctypes.byref(sep.pieces[k]), w, pvt,
                                          Nodes(0, ov.data_ptr(), 0, 0),
                                          Nodes(0, gv.data_ptr(), 0, 0), ctypes.byref(prm), None))
        # distribute_charge: private nodes in place, shared/ghost folds applied
        # to the shared instance, piece by piece
        for k in range(P):
            check(L.ckt_distribute_charge(g, k, w, pvt, sf, gf, ctypes.byref(prm), None))
            check(L.ckt_apply_fold(g, k, sf, gf, sq.data_ptr(), None))
        for k in range(P):
            check(L.ckt_update_voltages(ctypes.byref(sep.pieces[k]), pvt, shr,
                                        locator.data_ptr(), None))
        torch.cuda.synchronize()
    a = ref.to_host()
    b = sep.to_host()
    for k in ("current", "voltage"):
        assert np.array_equal(a[k].view(np.uint32), b[k].view(np.uint32)), k
    got_v = np.where(priv, pv.cpu().numpy(), sv.cpu().numpy())
    got_q = np.where(priv, pq.cpu().numpy(), sq.cpu().numpy())
    assert np.array_equal(got_v.view(np.uint32), a["node_voltage"].view(np.uint32))
    assert np.array_equal(got_q.view(np.uint32), a["charge"].view(np.uint32))
