"""Host-side driver of the circuit hot path: generate a circuit, place its
regions in HBM, and run the reference's loop (apps/circuit/circuit.cc:232-307)
through the C ABI.

Arrays use these names throughout (numpy on the host, torch on the device):
  wires: in_ptr, out_ptr (u32), in_loc, out_loc (u8), L, R, C (f32),
         current [10, W], voltage [9, W] (f32, segment-major)
  nodes: charge, node_voltage, cap, leak (f32), locator (i32)
torch is used only to own device memory and streams.
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass

import numpy as np

from . import (DT, INIT_KERNEL, MODE_EXACT, SEGMENTS, GenParams, HostCircuit, Nodes, Params,
               Piece, Wires, check, lib)

WIRE_FIELDS = ("in_ptr", "out_ptr", "in_loc", "out_loc", "L", "R", "C", "current", "voltage")
NODE_FIELDS = ("charge", "node_voltage", "cap", "leak", "locator")
STATE_FIELDS = ("current", "voltage", "charge", "node_voltage")


@dataclass
class Shape:
    num_pieces: int
    nodes_per_piece: int
    wires_per_piece: int

    @property
    def W(self) -> int:
        return self.num_pieces * self.wires_per_piece

    @property
    def N(self) -> int:
        return self.num_pieces * self.nodes_per_piece

    def pieces(self) -> "ctypes.Array[Piece]":
        arr = (Piece * self.num_pieces)()
        for k in range(self.num_pieces):
            arr[k] = Piece(k * self.wires_per_piece, self.wires_per_piece,
                           k * self.nodes_per_piece, self.nodes_per_piece)
        return arr


def _vp(a: np.ndarray) -> int:
    assert a.flags["C_CONTIGUOUS"], "arrays must be contiguous"
    return a.ctypes.data


def generate(num_pieces: int, nodes_per_piece: int, wires_per_piece: int,
             pct_wire_in_piece: float = 95.0, random_seed: int = 12345,
             L_offset: float = 0.1, L_scale: float = 0.01) -> dict:
    """load_circuit (apps/circuit/circuit.cc:1071-1288) through ckt_generate."""
    P, npp, wpp = num_pieces, nodes_per_piece, wires_per_piece
    W, N = P * wpp, P * npp
    h = {
        "in_ptr": np.empty(W, np.uint32), "out_ptr": np.empty(W, np.uint32),
        "in_loc": np.empty(W, np.uint8), "out_loc": np.empty(W, np.uint8),
        "L": np.empty(W, np.float32), "R": np.empty(W, np.float32), "C": np.empty(W, np.float32),
        "current": np.empty((SEGMENTS, W), np.float32),
        "voltage": np.empty((SEGMENTS - 1, W), np.float32),
        "charge": np.empty(N, np.float32), "node_voltage": np.empty(N, np.float32),
        "cap": np.empty(N, np.float32), "leak": np.empty(N, np.float32),
        "locator": np.empty(N, np.int32),
    }
    hc = HostCircuit(*[_vp(h[k]) for k in ("in_ptr", "out_ptr", "in_loc", "out_loc", "L", "R",
                                           "C", "current", "voltage", "charge", "node_voltage",
                                           "cap", "leak", "locator")])
    gp = GenParams(P, npp, wpp, 0, float(pct_wire_in_piece), int(random_seed), float(L_offset),
                   float(L_scale))
    check(lib().ckt_generate(ctypes.byref(gp), ctypes.byref(hc)))
    return h


class Graph:
    """Owns a ckt_graph built from host wire endpoints."""

    def __init__(self, pieces, num_nodes: int, in_ptr, out_ptr, in_loc, out_loc):
        self.handle = ctypes.c_void_p()
        arrs = [np.ascontiguousarray(a) for a in (in_ptr, out_ptr, in_loc, out_loc)]
        check(lib().ckt_graph_create(pieces, len(pieces), int(num_nodes),
                                     *[_vp(a) for a in arrs], ctypes.byref(self.handle)))
        self.pieces = pieces

    def info(self):
        w, n, b = ctypes.c_int64(), ctypes.c_int64(), ctypes.c_int64()
        p = ctypes.c_int32()
        check(lib().ckt_graph_info(self.handle, ctypes.byref(w), ctypes.byref(n), ctypes.byref(p),
                                   ctypes.byref(b)))
        return {"wires": w.value, "nodes": n.value, "pieces": p.value, "device_bytes": b.value}

    def close(self):
        if self.handle:
            lib().ckt_graph_destroy(self.handle)
            self.handle = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class DeviceCircuit:
    """A circuit resident in HBM (structure-of-arrays torch tensors) plus its
    contribution graph.  All task calls are asynchronous on `stream`."""

    def __init__(self, host: dict, shape: Shape, device: str = "cuda", pieces=None):
        import torch

        self.torch = torch
        self.shape = shape
        self.pieces = pieces if pieces is not None else shape.pieces()
        self.t = {k: torch.from_numpy(np.ascontiguousarray(v)).to(device) for k, v in host.items()}
        self.graph = Graph(self.pieces, shape.N, host["in_ptr"], host["out_ptr"], host["in_loc"],
                           host["out_loc"])
        # Reduction instances for the per-piece drop-in path (float per node).
        self.shr_fold = torch.zeros(shape.N, dtype=torch.float32, device=device)
        self.ghost_fold = torch.zeros(shape.N, dtype=torch.float32, device=device)

    # -- views ----------------------------------------------------------------
    def wires(self) -> Wires:
        t = self.t
        return Wires(t["in_ptr"].data_ptr(), t["out_ptr"].data_ptr(), t["in_loc"].data_ptr(),
                     t["out_loc"].data_ptr(), t["L"].data_ptr(), t["R"].data_ptr(),
                     t["C"].data_ptr(), t["current"].data_ptr(), t["voltage"].data_ptr(),
                     self.shape.W)

    def nodes(self) -> Nodes:
        t = self.t
        return Nodes(t["charge"].data_ptr(), t["node_voltage"].data_ptr(), t["cap"].data_ptr(),
                     t["leak"].data_ptr())

    # -- state ----------------------------------------------------------------
    def load_state(self, host: dict) -> None:
        for k in STATE_FIELDS:
            self.t[k].copy_(self.torch.from_numpy(np.ascontiguousarray(host[k])))

    def to_host(self, fields=STATE_FIELDS) -> dict:
        return {k: self.t[k].cpu().numpy() for k in fields}

    # -- the reference loop ---------------------------------------------------
    def loop_index_space(self, prm: Params, stream: int = 0) -> None:
        """One outer loop as three index-space launches."""
        L, g, w, n = lib(), self.graph.handle, self.wires(), self.nodes()
        check(L.ckt_calc_new_currents_all(g, w, n, ctypes.byref(prm), stream))
        check(L.ckt_distribute_charge_all(g, w, n, ctypes.byref(prm), stream))
        check(L.ckt_update_voltages_all(g, n, stream))

    def run_loops(self, prm: Params, loops: int, stream: int = 0, blocking: bool = False) -> None:
        """`loops` outer loops with distribute_charge and update_voltages
        fused into one node pass (two launches per loop); bit-identical to
        `loops` calls of loop_index_space.  blocking: wait for the stream and
        raise if a tiled node pass ran out of a copy wait (ckt_run_loops_all_sync)."""
        fn = lib().ckt_run_loops_all_sync if blocking else lib().ckt_run_loops_all
        check(fn(self.graph.handle, self.wires(), self.nodes(), ctypes.byref(prm), loops, stream))

    def check(self, stream: int = 0) -> None:
        """Waits for `stream` and raises CktError (CKT_ETIMEOUT) if a tiled
        node pass on this circuit's graph left a tile unwritten."""
        check(lib().ckt_graph_check(self.graph.handle, stream))

    def loop_per_piece(self, prm: Params, stream: int = 0, blocking: bool = False) -> None:
        """One outer loop as the reference's per-piece task calls: CNC for
        every piece; DC for every piece, each followed by the application of
        that piece's reduction instances (the runtime applies a point's
        instances once the point finishes, points in ascending order; the
        two fold buffers are reused, and ckt_apply_fold returns them to the
        identity); UV for every piece.  `blocking` uses the *_sync forms,
        which wait for the device after every task like the reference's GPU
        task bodies."""
        L, g, w, n = lib(), self.graph.handle, self.wires(), self.nodes()
        cnc = L.ckt_calc_new_currents_sync if blocking else L.ckt_calc_new_currents
        dc = L.ckt_distribute_charge_sync if blocking else L.ckt_distribute_charge
        uv = L.ckt_update_voltages_sync if blocking else L.ckt_update_voltages
        locator = self.t["locator"].data_ptr()
        for k in range(len(self.pieces)):
            check(cnc(ctypes.byref(self.pieces[k]), w, n, n, n, ctypes.byref(prm), stream))
        sf, gf = self.shr_fold.data_ptr(), self.ghost_fold.data_ptr()
        for k in range(len(self.pieces)):
            check(dc(g, k, w, n, sf, gf, ctypes.byref(prm), stream))
            check(L.ckt_apply_fold(g, k, sf, gf, n.charge, stream))
        for k in range(len(self.pieces)):
            check(uv(ctypes.byref(self.pieces[k]), n, n, locator, stream))

    def sanity_check(self, stream: int = 0) -> None:
        bad = ctypes.c_int64()
        for k in range(len(self.pieces)):
            check(lib().ckt_sanity_check_wires(ctypes.byref(self.pieces[k]), self.wires(),
                                               self.shape.N, ctypes.byref(bad), stream))

    def close(self) -> None:
        self.graph.close()


def params(steps: int, mode: int = MODE_EXACT, init: int = INIT_KERNEL) -> Params:
    return Params(int(steps), DT, int(mode), int(init))
