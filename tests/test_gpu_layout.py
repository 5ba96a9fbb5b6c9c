"""AoS <-> SoA interop with the reference's CircuitWire / CircuitNode
instances (apps/circuit/circuit.h:35-54): round trips are exact, and a
circuit loaded from AoS instances simulates to the same bits."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

STATE = ["current", "voltage", "charge", "node_voltage"]


def test_aos_round_trip_and_simulation(cuda, oracle):
    import ctypes

    from legionorigins_gb300 import check, lib
    from legionorigins_gb300 import circuit as C

    torch = cuda
    p = oracle.GenParams(5, 37, 333, 80, 9, L_offset=0.001)   # W not a multiple of 32
    c = oracle.generate(p)
    rng = np.random.default_rng(3)
    c.current[:] = rng.standard_normal(c.current.shape).astype(np.float32)
    c.voltage[:] = rng.standard_normal(c.voltage.shape).astype(np.float32)
    nodes_aos, wires_aos = oracle.circuit_to_aos(c)
    d_wires = torch.from_numpy(wires_aos.view(np.uint8).copy()).cuda()
    d_nodes = torch.from_numpy(nodes_aos.view(np.uint8).copy()).cuda()
    host = {k: np.zeros_like(getattr(c, k)) for k in ("in_ptr", "out_ptr", "in_loc", "out_loc",
                                                       "L", "R", "C", "current", "voltage",
                                                       "charge", "node_voltage", "cap", "leak")}
    host["locator"] = c.locator.copy()
    # the graph needs real endpoints: build the device circuit from the oracle's,
    # then overwrite every wire/node field from the AoS instances
    dc = C.DeviceCircuit({k: getattr(c, k) for k in host}, C.Shape(p.num_pieces,
                         p.nodes_per_piece, p.wires_per_piece))
    for k in ("current", "voltage", "L", "R", "C", "charge", "node_voltage", "cap", "leak"):
        dc.t[k].zero_()
    check(lib().ckt_wires_from_aos(d_wires.data_ptr(), p.W, dc.wires(), None))
    check(lib().ckt_nodes_from_aos(d_nodes.data_ptr(), p.N, dc.nodes(), None))
    torch.cuda.synchronize()
    for k in ("in_ptr", "out_ptr", "in_loc", "out_loc", "L", "R", "C", "current", "voltage"):
        assert np.array_equal(dc.t[k].cpu().numpy(), getattr(c, k)), k
    for k, f in (("charge", "charge"), ("node_voltage", "node_voltage"), ("cap", "cap"),
                 ("leak", "leak")):
        assert np.array_equal(dc.t[k].cpu().numpy(), getattr(c, f)), k
    # back to AoS: identical bytes (pad words are zero in both)
    out_w = torch.zeros_like(d_wires)
    out_n = torch.zeros_like(d_nodes)
    check(lib().ckt_wires_to_aos(dc.wires(), p.W, out_w.data_ptr(), None))
    check(lib().ckt_nodes_to_aos(dc.nodes(), p.N, out_n.data_ptr(), None))
    torch.cuda.synchronize()
    assert np.array_equal(out_w.cpu().numpy(), wires_aos.view(np.uint8))
    assert np.array_equal(out_n.cpu().numpy(), nodes_aos.view(np.uint8))
    # simulate from the AoS-loaded state: same bits as the oracle
    prm = C.params(3, 0)
    dc.loop_index_space(prm)
    dc.loop_index_space(prm)
    torch.cuda.synchronize()
    got = dc.to_host()
    oracle.simulate(c, 2, 3)
    for k in STATE:
        a, b = got[k], getattr(c, k)
        na, nb = np.isnan(a), np.isnan(b)
        assert np.array_equal(na, nb) and np.array_equal(a[~na].view(np.uint32),
                                                         b[~nb].view(np.uint32)), k
