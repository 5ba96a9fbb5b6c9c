"""Host-side checks of the C-ABI library that need no GPU: it loads, it
exports every entry point include/ckt.h declares, its generator matches the
oracle, and its argument validation fails cleanly before any CUDA call."""
import ctypes
import os
import re

import numpy as np
import pytest

from conftest import ROOT

HEADERS = [os.path.join(ROOT, "include", f) for f in sorted(os.listdir(os.path.join(ROOT, "include")))
           if f.endswith(".h")]


def declared_symbols(headers=None):
    names = set()
    for h in headers or HEADERS:
        text = open(h).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        for m in re.finditer(r"^\s*(?:const\s+)?[A-Za-z_][\w\s\*]*?\b(ckt_\w+)\s*\(", text, re.M):
            names.add(m.group(1))
    return sorted(names)


def test_every_header_is_checked():
    assert sorted(os.path.basename(h) for h in HEADERS) == ["ckt.h", "ckt_tools.h"]


def test_library_exports_every_declared_symbol(ckt):
    names = declared_symbols([os.path.join(ROOT, "include", "ckt.h")])
    assert len(names) >= 15
    L = ckt.lib()
    missing = [n for n in names if not hasattr(L, n)]
    assert not missing, missing
    # ... and the Python binding types every one of them
    assert set(names) <= set(ckt.SIGNATURES), set(names) - set(ckt.SIGNATURES)


def test_tools_library_exports_every_declared_symbol(ckt):
    """The measurement and verification helpers live in their own library,
    not in the product's."""
    names = declared_symbols([os.path.join(ROOT, "include", "ckt_tools.h")])
    assert "ckt_fp32_fma_probe" in names and "ckt_check_dt_quotient" in names
    T = ckt.tools()
    missing = [n for n in names if not hasattr(T, n)]
    assert not missing, missing
    assert set(names) == set(ckt.TOOLS_SIGNATURES)
    product = ckt.lib()
    assert not any(hasattr(product, n) for n in names)


def test_abi_version_and_strings(ckt):
    L = ckt.lib()
    assert L.ckt_abi_version() == 1
    assert L.ckt_status_string(0) == b"ok"
    p = ckt.Params()
    L.ckt_default_params(ctypes.byref(p))
    assert p.steps == 10000 and p.mode == ckt.MODE_EXACT and p.init == ckt.INIT_KERNEL
    assert np.float32(p.dt) == np.float32(1e-6)


@pytest.mark.parametrize("args", [(4, 256, 1024, 95, 12345), (3, 5, 7, 50, 7), (1, 4, 9, 50, 3),
                                  (8, 64, 256, 50, 42), (2, 1, 3, 0, 1), (5, 33, 100, 100, 5)])
def test_product_generator_matches_oracle(ckt, oracle, args):
    from legionorigins_gb300 import circuit as C

    h = C.generate(*args)
    o = oracle.generate(oracle.GenParams(*args))
    for k, v in h.items():
        assert np.array_equal(v, getattr(o, k)), k


def test_product_generator_baseline_inductance(ckt, oracle):
    from legionorigins_gb300 import circuit as C

    h = C.generate(4, 16, 64, 95, 9, L_offset=0.001, L_scale=0.01)
    o = oracle.generate(oracle.GenParams(4, 16, 64, 95, 9, L_offset=0.001, L_scale=0.01))
    assert np.array_equal(h["L"], o.L)
    assert (h["L"] >= 0.001).all() and (h["L"] < 0.011).all()


def _graph_create(ckt, pieces, N, in_ptr, out_ptr, in_loc, out_loc):
    from legionorigins_gb300.circuit import _vp

    arrs = [np.ascontiguousarray(a) for a in (in_ptr, out_ptr, in_loc, out_loc)]
    h = ctypes.c_void_p()
    rc = ckt.lib().ckt_graph_create(pieces, len(pieces), N, *[_vp(a) for a in arrs],
                                    ctypes.byref(h))
    return rc, ckt.lib().ckt_last_error().decode()


def test_graph_rejects_bad_wires_before_touching_the_gpu(ckt):
    from legionorigins_gb300 import circuit as C

    shape = C.Shape(2, 4, 3)
    h = C.generate(2, 4, 3, 50.0, 1)
    pieces = shape.pieces()
    cases = []
    a = dict(h); a["in_ptr"] = h["in_ptr"].copy(); a["in_ptr"][1] = 7       # in-node in another piece
    cases.append((a, "inconsistent"))
    a = dict(h); a["out_ptr"] = h["out_ptr"].copy(); a["out_ptr"][0] = 99    # beyond the node region
    cases.append((a, "out of range"))
    a = dict(h); a["out_loc"] = h["out_loc"].copy(); a["out_loc"][2] = 5     # bad location value
    cases.append((a, "out of range"))
    for a, msg in cases:
        rc, err = _graph_create(ckt, pieces, shape.N, a["in_ptr"], a["out_ptr"], a["in_loc"],
                                a["out_loc"])
        assert rc == 3 and msg in err, (rc, err)   # CKT_EBOUNDS


def test_graph_rejects_bad_piece_tiling(ckt):
    from legionorigins_gb300 import Piece

    z = np.zeros(4, np.uint32)
    pieces = (Piece * 2)(Piece(0, 2, 0, 2), Piece(3, 2, 2, 2))  # gap at wire 2
    rc, err = _graph_create(ckt, pieces, 4, z, z, z.astype(np.uint8), z.astype(np.uint8))
    assert rc == 1 and "starts at wire" in err
    pieces = (Piece * 2)(Piece(0, 2, 0, 3), Piece(2, 2, 2, 2))  # node 2 in both pieces
    rc, err = _graph_create(ckt, pieces, 4, z, z, z.astype(np.uint8), z.astype(np.uint8))
    assert rc == 1 and "belongs to pieces" in err


def test_entry_points_validate_arguments(ckt):
    L = ckt.lib()
    prm = ckt.default_params(steps=1)
    assert L.ckt_calc_new_currents(None, ckt.Wires(), ckt.Nodes(), ckt.Nodes(), ckt.Nodes(),
                                   ctypes.byref(prm), None) == 1
    piece = ckt.Piece(0, 4, 0, 4)
    assert L.ckt_calc_new_currents(ctypes.byref(piece), ckt.Wires(), ckt.Nodes(), ckt.Nodes(),
                                   ckt.Nodes(), ctypes.byref(prm), None) == 1
    assert b"NULL" in L.ckt_last_error()
    bad = ckt.Params(1, ckt.DT, 7, 0)
    w = ckt.Wires(*([8] * 9), 4)
    n = ckt.Nodes(8, 8, 8, 8)
    assert L.ckt_calc_new_currents(ctypes.byref(piece), w, n, n, n, ctypes.byref(bad), None) == 1
    assert b"mode" in L.ckt_last_error()
    assert L.ckt_distribute_charge_all(None, w, n, ctypes.byref(prm), None) == 1
    assert L.ckt_update_voltages_all(None, n, None) == 1
    assert L.ckt_apply_fold(None, 0, None, None, None, None) == 1
    assert L.ckt_graph_tile_info(None, None, None, None, None) == 1
    assert L.ckt_graph_set_tile_timeout(None, 1) == 1
    assert b"graph is NULL" in L.ckt_last_error()


def test_hist_entry_points_validate_arguments(ckt):
    """The reduction microbenchmark's checks run before any CUDA call."""
    from legionorigins_gb300 import reductions as R

    L = ckt.lib()
    d = ckt.HistParams()
    L.ckt_hist_default_params(ctypes.byref(d))
    assert (d.buckets, d.batch_size, d.num_batches, d.seed1, d.seed2) == (
        1048576, 1048576, 1024, 12345, 54321)
    assert (d.buckets, d.batch_size, d.num_batches) == tuple(
        getattr(R.params(), k) for k in ("buckets", "batch_size", "num_batches"))
    bad = R.params(buckets=0)
    assert L.ckt_hist_run(ctypes.byref(bad), 0, 8, None, 0, None) == 1
    assert b"buckets" in L.ckt_last_error()
    p = R.params(buckets=16, batch_size=4, num_batches=2)
    assert L.ckt_hist_run(ctypes.byref(p), 9, 8, None, 0, None) == 1
    assert b"schedule" in L.ckt_last_error()
    assert L.ckt_hist_run(ctypes.byref(p), 0, None, None, 0, None) == 1
    big = R.params(buckets=(1 << 26) + 1, batch_size=4, num_batches=1)
    assert L.ckt_hist_run(ctypes.byref(big), ckt.RED_LOCALIZE, 8, None, 0, None) == 1
    assert b"localize" in L.ckt_last_error()
    lo, hi = ctypes.c_uint64(), ctypes.c_uint64()
    assert L.ckt_hist_scratch_bytes(ctypes.byref(p), ckt.RED_SINGLE, ctypes.byref(lo),
                                    ctypes.byref(hi)) == 0 and lo.value == hi.value == 0
    assert L.ckt_hist_scratch_bytes(ctypes.byref(p), ckt.RED_LIST, ctypes.byref(lo),
                                    ctypes.byref(hi)) == 0 and lo.value == 32 and hi.value >= 32
    wide = R.params(buckets=1 << 20, batch_size=4, num_batches=1)
    assert L.ckt_hist_scratch_bytes(ctypes.byref(wide), ckt.RED_FOLD, ctypes.byref(lo),
                                    ctypes.byref(hi)) == 0 and lo.value == 4 << 20
    # too little scratch for a list: rejected before anything runs
    assert L.ckt_hist_run(ctypes.byref(p), ckt.RED_LIST, 8, 16, 8, None) == 1
    assert b"minimum" in L.ckt_last_error()
