"""The tiled node pass (distribute_charge over node tiles, currents copied
into shared memory chunk by chunk) against the per-node gather form.

The index-space distribute_charge and the fused node pass take the tiled
form when the current array is 16-byte aligned and its segment stride is a
multiple of 4, and the gather form otherwise.  Both must give the same bits
as each other and as the oracle, on shapes with dense chunks, sparse chunks
(packed into the graph's ghost buffer first), hub nodes whose runs cross
many chunks, tiles that straddle pieces, and heavy cross-piece reduction.
"""
import ctypes

import numpy as np
import pytest

from conftest import same_bits

pytestmark = pytest.mark.gpu

STATE = ["current", "voltage", "charge", "node_voltage"]
FIELDS = ["in_ptr", "out_ptr", "in_loc", "out_loc", "L", "R", "C", "current", "voltage",
          "charge", "node_voltage", "cap", "leak", "locator"]

SHAPES = {
    "cfg0": (4, 256, 1024, 95, 12345),
    "heavy_reduction": (16, 64, 256, 50, 42),
    "all_cross": (6, 16, 64, 0, 11),
    "hub": (7, 3, 3000, 60, 8),
    "many_pieces_per_tile": (40, 300, 1200, 95, 3),
    "tile_per_piece": (3, 8192, 2048, 90, 5),
    "tiles_straddle_pieces": (2, 20000, 80000, 97, 9),
    "last_tile_one_node": (1, 8193, 32772, 100, 13),
    "one_hub_node": (1, 1, 8192, 100, 3),           # 16384 entries of one node, several steps
    "ragged_wire_count": (3, 50, 333, 80, 17),      # W = 999: the last chunk copy is rounded up
}


class Strided:
    """A device circuit whose current/voltage segments sit `stride` floats
    apart (stride >= W); the gap holds NaN."""

    def __init__(self, cuda, c, stride):
        from legionorigins_gb300 import circuit as C

        p = c.params
        host = {k: np.ascontiguousarray(getattr(c, k)) for k in FIELDS}
        self.dc = C.DeviceCircuit(host, C.Shape(p.num_pieces, p.nodes_per_piece,
                                                p.wires_per_piece))
        self.W, self.stride = self.dc.shape.W, stride
        t = self.dc.t
        for k, segs in (("current", 10), ("voltage", 9)):
            buf = cuda.full((segs, stride), float("nan"), dtype=cuda.float32, device="cuda")
            buf[:, :self.W] = t[k].view(segs, self.W)
            t[k] = buf

    def wires(self):
        from legionorigins_gb300 import Wires

        t = self.dc.t
        return Wires(t["in_ptr"].data_ptr(), t["out_ptr"].data_ptr(), t["in_loc"].data_ptr(),
                     t["out_loc"].data_ptr(), t["L"].data_ptr(), t["R"].data_ptr(),
                     t["C"].data_ptr(), t["current"].data_ptr(), t["voltage"].data_ptr(),
                     self.stride)

    def loops(self, prm, n, fused):
        from legionorigins_gb300 import check, lib

        L, g, w, nd = lib(), self.dc.graph.handle, self.wires(), self.dc.nodes()
        for _ in range(n):
            check(L.ckt_calc_new_currents_all(g, w, nd, ctypes.byref(prm), None))
            if fused:
                check(L.ckt_distribute_update_all(g, w, nd, ctypes.byref(prm), None))
            else:
                check(L.ckt_distribute_charge_all(g, w, nd, ctypes.byref(prm), None))
                check(L.ckt_update_voltages_all(g, nd, None))

    def state(self, cuda):
        cuda.cuda.synchronize()
        t = self.dc.t
        out = {k: t[k][:, :self.W].contiguous().cpu().numpy() for k in ("current", "voltage")}
        out.update({k: t[k].cpu().numpy() for k in ("charge", "node_voltage")})
        return out


def tile_info(dc):
    from legionorigins_gb300 import check, lib

    tiles, steps, stream = ctypes.c_int32(), ctypes.c_int64(), ctypes.c_int64()
    err = ctypes.c_uint32()
    check(lib().ckt_graph_tile_info(dc.graph.handle, ctypes.byref(tiles), ctypes.byref(steps),
                                    ctypes.byref(stream), ctypes.byref(err)))
    return tiles.value, steps.value, stream.value, err.value


@pytest.mark.parametrize("shape", sorted(SHAPES))
@pytest.mark.parametrize("fused", [False, True], ids=["three_launch", "fused"])
def test_tiled_equals_gather_and_oracle(cuda, oracle, shape, fused):
    from legionorigins_gb300 import circuit as C

    c = oracle.generate(oracle.GenParams(*SHAPES[shape], L_offset=0.001))
    W = c.params.num_pieces * c.params.wires_per_piece
    pad = (-W) % 4
    tiled = Strided(cuda, c, W + pad + 4)   # a multiple of 4: the tiled form
    gather = Strided(cuda, c, W + pad + 6)  # 2 mod 4: the gather form
    prm = C.params(2, 0)
    tiled.loops(prm, 3, fused)
    gather.loops(prm, 3, fused)
    a, b = tiled.state(cuda), gather.state(cuda)
    for k in STATE:
        assert np.array_equal(a[k].view(np.uint32), b[k].view(np.uint32)), (shape, k)
    oracle.simulate(c, 3, 2)
    for k in STATE:
        assert same_bits(a[k], getattr(c, k)), (shape, k)
    tiles, steps, stream, err = tile_info(tiled.dc)
    assert tiles == -(-c.params.num_pieces * c.params.nodes_per_piece // 8192)
    assert steps >= stream >= 0 and err == 0


def test_plan_has_stream_and_ghost_steps(cuda, oracle):
    """Config-1 pieces (16384 nodes, 65536 wires each): each half-piece tile
    copies every chunk of its own piece (a chunk with more of the tile's
    entries than a step holds takes two steps) and takes its contributions
    from other pieces' wires through ghost steps."""
    c = oracle.generate(oracle.GenParams(4, 16384, 65536, 95, 12345, L_offset=0.001))
    dc = Strided(cuda, c, 4 * 65536).dc
    tiles, steps, stream, err = tile_info(dc)
    assert tiles == 8
    assert 8 * 8 <= stream <= 8 * 64  # chunks of 1024 to 8192 wires
    assert steps > stream
    assert err == 0


def test_nan_currents_propagate_identically(cuda, oracle):
    """The divergent regime (S = 1000): NaN and +-Inf currents flow through
    both forms to the same bits."""
    from legionorigins_gb300 import circuit as C

    c = oracle.generate(oracle.GenParams(*SHAPES["cfg0"], L_offset=0.001))
    W = c.params.num_pieces * c.params.wires_per_piece
    tiled, gather = Strided(cuda, c, W), Strided(cuda, c, W + 2)
    prm = C.params(1000, 0)
    tiled.loops(prm, 2, True)
    gather.loops(prm, 2, True)
    a, b = tiled.state(cuda), gather.state(cuda)
    for k in STATE:
        assert np.array_equal(a[k].view(np.uint32), b[k].view(np.uint32)), k
    assert np.isnan(a["node_voltage"]).any()


@pytest.mark.parametrize("shape", ["cfg0", "hub", "tiles_straddle_pieces"])
def test_unaligned_node_arrays(cuda, oracle, shape):
    """Node arrays that start 4 bytes past a 16-byte boundary: the fused pass
    reads voltage, capacitance and leakage from global memory instead of
    staging them by bulk copies; same bits as the aligned arrays."""
    from legionorigins_gb300 import Nodes, check, lib
    from legionorigins_gb300 import circuit as C

    c = oracle.generate(oracle.GenParams(*SHAPES[shape], L_offset=0.001))
    W = c.params.num_pieces * c.params.wires_per_piece
    stride = W + (-W) % 4 + 4
    a, b = Strided(cuda, c, stride), Strided(cuda, c, stride)
    N = c.params.num_pieces * c.params.nodes_per_piece
    off = {}
    for k, src in (("charge", "charge"), ("node_voltage", "node_voltage"), ("cap", "cap"),
                   ("leak", "leak")):
        buf = cuda.zeros(N + 1, dtype=cuda.float32, device="cuda")
        buf[1:] = b.dc.t[src]
        off[k] = buf
    nodes_b = Nodes(off["charge"].data_ptr() + 4, off["node_voltage"].data_ptr() + 4,
                    off["cap"].data_ptr() + 4, off["leak"].data_ptr() + 4)
    prm = C.params(2, 0)
    L = lib()
    for _ in range(3):
        check(L.ckt_calc_new_currents_all(a.dc.graph.handle, a.wires(), a.dc.nodes(),
                                          ctypes.byref(prm), None))
        check(L.ckt_distribute_update_all(a.dc.graph.handle, a.wires(), a.dc.nodes(),
                                          ctypes.byref(prm), None))
        check(L.ckt_calc_new_currents_all(b.dc.graph.handle, b.wires(), nodes_b,
                                          ctypes.byref(prm), None))
        check(L.ckt_distribute_update_all(b.dc.graph.handle, b.wires(), nodes_b,
                                          ctypes.byref(prm), None))
    cuda.cuda.synchronize()
    got_a = a.state(cuda)
    for k, name in (("charge", "charge"), ("node_voltage", "node_voltage")):
        got_b = off[k][1:].cpu().numpy()
        assert np.array_equal(got_a[name].view(np.uint32), got_b.view(np.uint32)), (shape, k)
    for k in ("current", "voltage"):
        got_b = b.state(cuda)[k]
        assert np.array_equal(got_a[k].view(np.uint32), got_b.view(np.uint32)), (shape, k)
    assert tile_info(b.dc)[3] == 0


@pytest.mark.parametrize("fused", [False, True], ids=["charge", "fused"])
def test_one_graph_shared_by_two_streams(cuda, oracle, fused):
    """Two circuits of one topology, with different states, run on two
    streams through the same graph, their calls interleaved: the passes
    share the graph's ghost buffer, so the library orders each pass behind
    the previous one, and each circuit gets the bits it gets alone."""
    from legionorigins_gb300 import check, lib
    from legionorigins_gb300 import circuit as C

    c = oracle.generate(oracle.GenParams(8, 16384, 65536, 50, 21, L_offset=0.001))
    W = c.params.num_pieces * c.params.wires_per_piece
    stride = W + (-W) % 4 + 4
    runs = [Strided(cuda, c, stride) for _ in range(4)]  # a, b shared; a, b alone
    rng = np.random.default_rng(5)
    bstate = {k: rng.uniform(-1, 1, getattr(c, k).shape).astype(np.float32)
              for k in ("current", "voltage")}
    for r in (runs[1], runs[3]):
        for k, v in bstate.items():
            r.dc.t[k][:, :W] = cuda.from_numpy(v).cuda()
    prm = C.params(1, 0)
    L, g = lib(), runs[0].dc.graph.handle
    s1, s2 = cuda.cuda.Stream(), cuda.cuda.Stream()
    cuda.cuda.synchronize()

    def step(r, graph, stream):
        w, n = r.wires(), r.dc.nodes()
        check(L.ckt_calc_new_currents_all(graph, w, n, ctypes.byref(prm), stream))
        if fused:
            check(L.ckt_distribute_update_all(graph, w, n, ctypes.byref(prm), stream))
        else:
            check(L.ckt_distribute_charge_all(graph, w, n, ctypes.byref(prm), stream))

    for _ in range(3):
        step(runs[0], g, s1.cuda_stream)
        step(runs[1], g, s2.cuda_stream)
    for r in runs[2:]:
        for _ in range(3):
            step(r, r.dc.graph.handle, None)
    cuda.cuda.synchronize()
    for shared, alone in ((runs[0], runs[2]), (runs[1], runs[3])):
        a, b = shared.state(cuda), alone.state(cuda)
        for k in STATE:
            assert np.array_equal(a[k].view(np.uint32), b[k].view(np.uint32)), k
    assert tile_info(runs[0].dc)[3] == 0


def test_copy_wait_that_runs_out_reports_and_recovers(cuda, oracle):
    """Waits bounded at 1 ns run out before the copies land: the pass sets
    the graph's error word (read and cleared through ckt_graph_tile_info),
    lets its copies land and returns; with the default bound the next pass
    over the same circuit gives the gather form's bits."""
    from legionorigins_gb300 import check, lib
    from legionorigins_gb300 import circuit as C

    c = oracle.generate(oracle.GenParams(*SHAPES["tiles_straddle_pieces"], L_offset=0.001))
    W = c.params.num_pieces * c.params.wires_per_piece
    stride = W + (-W) % 4 + 4
    tiled, gather = Strided(cuda, c, stride), Strided(cuda, c, stride + 2)
    prm = C.params(2, 0)
    L, g = lib(), tiled.dc.graph.handle
    check(L.ckt_graph_set_tile_timeout(g, 1))
    check(L.ckt_distribute_charge_all(g, tiled.wires(), tiled.dc.nodes(), ctypes.byref(prm), None))
    cuda.cuda.synchronize()
    assert tile_info(tiled.dc)[3] == 1
    assert tile_info(tiled.dc)[3] == 0  # cleared by the read
    check(L.ckt_graph_set_tile_timeout(g, 0))
    for d in (tiled, gather):
        for k in ("charge", "node_voltage"):
            d.dc.t[k].copy_(cuda.from_numpy(np.ascontiguousarray(getattr(c, k))))
    tiled.loops(prm, 2, True)
    gather.loops(prm, 2, True)
    a, b = tiled.state(cuda), gather.state(cuda)
    for k in STATE:
        assert np.array_equal(a[k].view(np.uint32), b[k].view(np.uint32)), k
    assert tile_info(tiled.dc)[3] == 0


def test_run_out_wait_is_reported_by_the_loop_calls(cuda, oracle):
    """The loop calls do not return CKT_OK over a tile left unwritten:
    ckt_run_loops_all_sync returns CKT_ETIMEOUT; after ckt_run_loops_all,
    ckt_graph_check returns it, and until then every later index-space call
    on the graph does; once checked, the same circuit runs again with the
    oracle's bits."""
    from legionorigins_gb300 import lib
    from legionorigins_gb300 import circuit as C

    ETIMEOUT = 4
    c = oracle.generate(oracle.GenParams(*SHAPES["tiles_straddle_pieces"], L_offset=0.001))
    dc = C.DeviceCircuit({k: np.ascontiguousarray(getattr(c, k)) for k in FIELDS},
                         C.Shape(c.params.num_pieces, c.params.nodes_per_piece,
                                 c.params.wires_per_piece))
    assert tile_info(dc)[0] > 0
    prm = C.params(2, 0)
    L, g, w, n = lib(), dc.graph.handle, dc.wires(), dc.nodes()
    assert L.ckt_graph_set_tile_timeout(g, 1) == 0
    assert L.ckt_run_loops_all_sync(g, w, n, ctypes.byref(prm), 2, None) == ETIMEOUT
    assert b"copy wait" in L.ckt_last_error()
    assert L.ckt_graph_check(g, None) == 0  # the sync form already cleared it
    assert L.ckt_run_loops_all(g, w, n, ctypes.byref(prm), 1, None) == 0  # launched
    cuda.cuda.synchronize()
    # a finished pass left a tile unwritten: later calls refuse to continue
    assert L.ckt_distribute_update_all(g, w, n, ctypes.byref(prm), None) == ETIMEOUT
    assert L.ckt_distribute_charge_all(g, w, n, ctypes.byref(prm), None) == ETIMEOUT
    assert L.ckt_run_loops_all(g, w, n, ctypes.byref(prm), 1, None) == ETIMEOUT
    assert L.ckt_graph_check(g, None) == ETIMEOUT
    assert L.ckt_graph_check(g, None) == 0
    assert L.ckt_distribute_charge_all_sync(g, w, n, ctypes.byref(prm), None) == ETIMEOUT
    assert L.ckt_distribute_update_all_sync(g, w, n, ctypes.byref(prm), None) == ETIMEOUT
    assert L.ckt_graph_set_tile_timeout(g, 0) == 0
    dc.load_state({k: np.ascontiguousarray(getattr(c, k)) for k in STATE})
    dc.run_loops(prm, 2, blocking=True)
    got = dc.to_host()
    oracle.simulate(c, 2, 2)
    for k in STATE:
        assert same_bits(got[k], getattr(c, k)), k
