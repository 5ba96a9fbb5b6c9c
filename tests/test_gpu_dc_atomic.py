"""The graph-free distribute_charge (ckt_distribute_charge_atomic): the
reference's distribute_charge_gpu arguments -- a piece and its instances,
no contribution graph -- with warp-aggregated atomic adds
(apps/circuit/circuit_gpu.cu:219-304).

Its additions at a node come in an unspecified order, as the reference's
atomicAdd's do, so it is checked against the oracle's canonical order with
the error bound of fp32 summation in any order: per node with n terms,
|gpu - oracle| <= 2 n 2^-24 sum |terms| (each of the two sums is within
(n - 1) 2^-24 sum |terms| of the exact one); and, for nodes of at most 32
terms whose sum does not cancel (|oracle| >= 0.1 sum |terms|), within 1e-5
relative.  At the configured inner steps,
where most values are NaN or infinite, the NaN/+-Inf/finite classes must
match exactly.  Every piece runs as the reference's task does: fresh
(zero) fold instances, private charges updated in place, then the folds
applied to the shared instance, piece by piece.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

FIELDS = ["in_ptr", "out_ptr", "in_loc", "out_loc", "L", "R", "C", "current", "voltage",
          "charge", "node_voltage", "cap", "leak", "locator"]
SHAPES = {
    "cfg0": (4, 256, 1024, 95, 12345),
    "heavy_reduction": (16, 64, 256, 50, 42),
    "all_cross": (6, 16, 64, 0, 11),
    "hub": (2, 1, 5000, 50, 3),           # every wire end on one of two nodes: big warp groups
    "one_piece": (1, 7, 50, 50, 3),
}


def run_atomic(cuda, c, steps, blocking=False):
    """calc_new_currents (EXACT, index space), then distribute_charge piece
    by piece through the graph-free entry point; returns (charge after the
    folds are applied, the currents it used)."""
    from legionorigins_gb300 import Nodes, check, lib
    from legionorigins_gb300 import circuit as C

    p = c.params
    dc = C.DeviceCircuit({k: np.ascontiguousarray(getattr(c, k)) for k in FIELDS},
                         C.Shape(p.num_pieces, p.nodes_per_piece, p.wires_per_piece))
    prm = C.params(steps, 0)
    L, w = lib(), dc.wires()
    check(L.ckt_calc_new_currents_all(dc.graph.handle, w, dc.nodes(), ctypes.byref(prm), None))
    N = p.num_pieces * p.nodes_per_piece
    shr, ghost = (cuda.zeros(N, dtype=cuda.float32, device="cuda") for _ in range(2))
    charge = dc.t["charge"]
    pvt = Nodes(charge.data_ptr(), dc.t["node_voltage"].data_ptr(), dc.t["cap"].data_ptr(),
                dc.t["leak"].data_ptr())
    fn = L.ckt_distribute_charge_atomic_sync if blocking else L.ckt_distribute_charge_atomic
    for k in range(p.num_pieces):
        shr.zero_()
        ghost.zero_()
        check(fn(ctypes.byref(dc.pieces[k]), w, pvt, shr.data_ptr(), ghost.data_ptr(),
                 ctypes.byref(prm), None))
        touched = (shr != 0) | (ghost != 0) | cuda.isnan(shr) | cuda.isnan(ghost)
        charge[touched] = (charge + shr + ghost)[touched]
    cuda.cuda.synchronize()
    out = dc.to_host()
    dc.close()
    return out["charge"], out["current"]


def abs_sum(c, current):
    """Per node: sum |terms| (its starting charge and every contribution) and
    the number of terms."""
    dt = np.float32(1e-6)
    a = np.abs(np.float64(dt) * current[0].astype(np.float64))
    b = np.abs(np.float64(dt) * current[9].astype(np.float64))
    N = c.params.num_pieces * c.params.nodes_per_piece
    s = (np.bincount(c.in_ptr, a, N) + np.bincount(c.out_ptr, b, N)
         + np.abs(c.charge.astype(np.float64)))
    n = np.bincount(c.in_ptr, None, N) + np.bincount(c.out_ptr, None, N) + 1
    return s, n


U = 2.0 ** -24


@pytest.mark.parametrize("shape", sorted(SHAPES))
@pytest.mark.parametrize("blocking", [False, True])
def test_atomic_distribute_charge_finite_regime(cuda, oracle, shape, blocking):
    c = oracle.generate(oracle.GenParams(*SHAPES[shape], L_offset=0.001))
    rng = np.random.default_rng(5)
    c.charge[:] = rng.uniform(-1e-6, 1e-6, c.charge.shape).astype(np.float32)
    got, cur = run_atomic(cuda, c, 3, blocking)
    ref = c.copy()
    oracle.calc_new_currents(ref, 3)
    assert np.array_equal(cur.view(np.uint32), ref.current.view(np.uint32))
    s_abs, n = abs_sum(c, ref.current)
    oracle.distribute_charge(ref)
    r = ref.charge.astype(np.float64)
    g = got.astype(np.float64)
    assert np.isfinite(r).all() and np.isfinite(g).all()
    err = np.abs(g - r)
    bound = 2 * n * U * s_abs
    assert (err <= bound + 1e-30).all(), float((err / np.maximum(bound, 1e-30)).max())
    well = (np.abs(r) >= 0.1 * s_abs) & (n <= 32)
    rel = err[well] / np.maximum(np.abs(r[well]), 1e-30)
    assert rel.max(initial=0.0) <= 1e-5, rel.max()
    print(f"{shape}: max |err| / sum|contrib| {float((err / np.maximum(s_abs, 1e-30)).max()):.2e}, "
          f"max rel (no cancellation) {rel.max(initial=0.0):.2e}, "
          f"bit-equal nodes {np.mean(got.view(np.uint32) == ref.charge.view(np.uint32)):.3f}")


@pytest.mark.parametrize("shape", ["cfg0", "heavy_reduction"])
def test_atomic_distribute_charge_classes_at_configured_steps(cuda, oracle, shape):
    c = oracle.generate(oracle.GenParams(*SHAPES[shape], L_offset=0.001))
    got, cur = run_atomic(cuda, c, 1000)
    ref = c.copy()
    ref.current[:] = cur
    oracle.distribute_charge(ref)
    for cls in (np.isnan, np.isposinf, np.isneginf):
        assert np.array_equal(cls(got), cls(ref.charge)), cls.__name__
    fin = np.isfinite(ref.charge)
    if fin.any():
        s_abs, n = abs_sum(c, cur)
        err = np.abs(got[fin].astype(np.float64) - ref.charge[fin])
        assert (err <= 2 * n[fin] * U * s_abs[fin] + 1e-30).all()


def test_atomic_distribute_charge_rejects_bad_arguments(cuda, ckt):
    from legionorigins_gb300 import Nodes, Piece, Wires, lib
    from legionorigins_gb300 import circuit as C

    L = lib()
    prm = C.params(1, 0)
    rc = L.ckt_distribute_charge_atomic(ctypes.byref(Piece(0, 4, 0, 4)), Wires(), Nodes(), None,
                                        None, ctypes.byref(prm), None)
    assert rc == 1
    assert L.ckt_distribute_charge_atomic(None, Wires(), Nodes(), None, None, ctypes.byref(prm),
                                          None) == 1
