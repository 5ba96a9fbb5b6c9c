"""The generator on the GPU (ckt_generate_device) against the host generator
(ckt_generate) and the host graph builder (ckt_graph_create): every array and
the whole contribution graph bit for bit."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SHAPES = [
    (4, 256, 1024, 95.0, 12345),   # the plain CPU-runnable configuration
    (1, 7, 50, 50.0, 3),           # one piece: no cross-piece wires
    (3, 5, 7, 50.0, 7),            # ragged
    (2, 1, 3, 0.0, 1),             # one node per piece, every wire crosses
    (6, 16, 64, 0.0, 11),
    (5, 33, 100, 100.0, 5),        # every wire in-piece
    (3, 4, 0, 95.0, 1),            # no wires
    (16, 4096, 16384, 95.0, 42),   # many chunks of the draw stream
    (32, 777, 3001, 83.25, 77),    # real-valued pct, odd sizes
    (2, 1, 5000, 50.0, 3),         # hub nodes: a warp's span exceeds the sort stage
    (1, 3, 20000, 95.0, 9),        # one piece, three nodes
]


def device_generate(torch, shape):
    from legionorigins_gb300 import DeviceCircuitArrays, GenParams, check, lib

    P, npp, wpp, pct, seed = shape
    W, N = P * wpp, P * npp
    d = {
        "in_ptr": torch.empty(W, dtype=torch.int32), "out_ptr": torch.empty(W, dtype=torch.int32),
        "in_loc": torch.empty(W, dtype=torch.uint8), "out_loc": torch.empty(W, dtype=torch.uint8),
        "inductance": torch.empty(W), "resistance": torch.empty(W), "capacitance": torch.empty(W),
        "current": torch.full((10, W), 7.0), "voltage": torch.full((9, W), 7.0),
        "charge": torch.empty(N), "node_voltage": torch.empty(N), "node_capacitance": torch.empty(N),
        "node_leakage": torch.empty(N), "locator": torch.empty(N, dtype=torch.int32),
        "off": torch.empty(N + 1, dtype=torch.int32), "ent": torch.empty(2 * W, dtype=torch.int32),
        "slot_in": torch.empty(W, dtype=torch.int32), "slot_out": torch.empty(W, dtype=torch.int32),
        "gstart": torch.empty((2 * W + 31) // 32, dtype=torch.int32),
    }
    d = {k: v.cuda() for k, v in d.items()}
    arr = DeviceCircuitArrays(*[d[k].data_ptr() if d[k].numel() else None
                                for k, _ in DeviceCircuitArrays._fields_])
    gp = GenParams(P, npp, wpp, 0, pct, seed, 0.001, 0.01)
    check(lib().ckt_generate_device(ctypes.byref(gp), ctypes.byref(arr), None))
    torch.cuda.synchronize()
    return {k: v.cpu().numpy() for k, v in d.items()}


@pytest.mark.parametrize("shape", SHAPES, ids=lambda s: "x".join(str(v) for v in s))
def test_device_generator_matches_host(cuda, shape):
    from legionorigins_gb300 import check, lib
    from legionorigins_gb300 import circuit as C

    P, npp, wpp, pct, seed = shape
    W, N = P * wpp, P * npp
    dev = device_generate(cuda, shape)
    h = C.generate(P, npp, wpp, pct, seed, 0.001, 0.01)
    pairs = [("in_ptr", "in_ptr"), ("out_ptr", "out_ptr"), ("in_loc", "in_loc"),
             ("out_loc", "out_loc"), ("inductance", "L"), ("resistance", "R"),
             ("capacitance", "C"), ("charge", "charge"), ("node_voltage", "node_voltage"),
             ("node_capacitance", "cap"), ("node_leakage", "leak"), ("locator", "locator"),
             ("current", "current"), ("voltage", "voltage")]
    for dk, hk in pairs:
        a = dev[dk].view(np.uint8).reshape(-1)
        b = np.ascontiguousarray(h[hk]).view(np.uint8).reshape(-1)
        assert np.array_equal(a, b), dk
    g = C.Graph(C.Shape(P, npp, wpp).pieces(), N, h["in_ptr"], h["out_ptr"], h["in_loc"],
                h["out_loc"])
    ref = {"off": np.empty(N + 1, np.uint32), "ent": np.empty(2 * W, np.uint32),
           "slot_in": np.empty(W, np.uint32), "slot_out": np.empty(W, np.uint32),
           "gstart": np.empty((2 * W + 31) // 32, np.uint32)}
    check(lib().ckt_graph_export(g.handle, *[ref[k].ctypes.data for k in
                                            ("off", "ent", "slot_in", "slot_out", "gstart")]))
    for k, v in ref.items():
        assert np.array_equal(dev[k].view(np.uint32), v), k
    g.close()
