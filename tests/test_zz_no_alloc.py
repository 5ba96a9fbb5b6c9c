"""The allocation-free wire check (ckt_sanity_check_pieces_noalloc).

It exists for callers that may not allocate device memory -- a runtime that
has reserved the GPU's memory for its own pools, code that must not
synchronise the device through cudaMalloc/cudaFree, a process held to a fixed
memory budget.  Its scratch is a fixed array shared by every call, so the
test makes two calls in a row (the second must not see the first's
leftovers) and compares each with the allocating per-piece entry point,
ckt_sanity_check_wires.  This file is named to be collected last.
"""
import ctypes

import numpy as np
import pytest

FIELDS = ["in_ptr", "out_ptr", "in_loc", "out_loc", "L", "R", "C", "current", "voltage",
          "charge", "node_voltage", "cap", "leak", "locator"]


def _device_circuit(oracle):
    from legionorigins_gb300 import circuit as C

    p = oracle.GenParams(12, 40, 300, 80, 21)
    c = oracle.generate(p)
    host = {k: np.ascontiguousarray(getattr(c, k)) for k in FIELDS}
    return C.DeviceCircuit(host, C.Shape(p.num_pieces, p.nodes_per_piece, p.wires_per_piece))


def _noalloc(ckt, dc):
    n = len(dc.pieces)
    out = (ctypes.c_int64 * n)()
    rc = ckt.lib().ckt_sanity_check_pieces_noalloc(dc.pieces, n, dc.wires(), dc.shape.N, out,
                                                  None)
    return rc, list(out)


def _per_piece(ckt, dc):
    out, rcs = [], []
    for k in range(len(dc.pieces)):
        bad = ctypes.c_int64()
        rcs.append(ckt.lib().ckt_sanity_check_wires(ctypes.byref(dc.pieces[k]), dc.wires(),
                                                    dc.shape.N, ctypes.byref(bad), None))
        out.append(bad.value)
    return (3 if 3 in rcs else 0), out


@pytest.mark.gpu
def test_noalloc_check_matches_the_allocating_check_twice_in_a_row(cuda, oracle, ckt):
    dc = _device_circuit(oracle)
    # First call: a circuit with bad wires in three pieces.
    dc.t["in_ptr"][305] = 0          # piece 1's wire 5: in-node in piece 0
    dc.t["out_ptr"][910] = 10_000    # piece 3: out-node beyond the node region
    dc.t["out_loc"][2999] = 7        # piece 9: location out of range
    dc.t["out_ptr"][2950] = 361      # piece 9, earlier wire: in-piece node marked ...
    dc.t["out_loc"][2950] = 2        # ... as a ghost
    cuda.cuda.synchronize()
    rc_a, a = _noalloc(ckt, dc)
    rc_b, b = _per_piece(ckt, dc)
    assert rc_a == rc_b == 3
    assert a == b
    assert a[1] == 305 and a[3] == 910 and a[9] == 2950
    assert sum(x >= 0 for x in a) == 3
    # Second call, on a clean circuit: the scratch still holds the first
    # call's results and must not leak into this one.
    clean = _device_circuit(oracle)
    rc_a, a = _noalloc(ckt, clean)
    rc_b, b = _per_piece(ckt, clean)
    assert rc_a == rc_b == 0
    assert a == b == [-1] * len(clean.pieces)


def test_noalloc_check_rejects_too_many_pieces(ckt):
    from legionorigins_gb300 import Piece, Wires

    n = 4097
    pieces = (Piece * n)()
    out = (ctypes.c_int64 * n)()
    rc = ckt.lib().ckt_sanity_check_pieces_noalloc(pieces, n, Wires(), 1, out, None)
    assert rc == 1
    assert b"CKT_NOALLOC_MAX_PIECES" in ckt.lib().ckt_last_error()
