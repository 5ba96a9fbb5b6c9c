"""Batched form: many independent circuits advanced together by one
persistent kernel launch per outer loop (include/ckt.h, ckt_batch_*)."""
from __future__ import annotations

import ctypes
import os

import numpy as np

from . import BatchConfig, GenParams, HostCircuit, check, lib
from .workloads import CircuitSpec


def _gp(s: CircuitSpec) -> GenParams:
    return GenParams(s.num_pieces, s.nodes_per_piece, s.wires_per_piece, 0,
                     float(s.pct_wire_in_piece), int(s.random_seed), float(s.L_offset),
                     float(s.L_scale))


class Batch:
    """A batch of circuits resident in HBM.

    host_circuits: optional list of dicts (legionorigins_gb300.circuit field
    names, circuit-local node pointers); without it every circuit is
    generated by the reference generator from its spec."""

    def __init__(self, specs: list[CircuitSpec], host_circuits=None, threads: int = 0):
        self.specs = list(specs)
        n = len(self.specs)
        shapes = (GenParams * n)(*[_gp(s) for s in self.specs])
        steps = (ctypes.c_int32 * n)(*[s.steps for s in self.specs])
        self.handle = ctypes.c_void_p()
        if host_circuits is None:
            threads = threads or os.cpu_count() or 1
            check(lib().ckt_batch_generate(n, shapes, steps, threads, ctypes.byref(self.handle)))
        else:
            self._keep = [{k: np.ascontiguousarray(v) for k, v in h.items()} for h in host_circuits]
            hcs = (HostCircuit * n)(*[HostCircuit(*[h[k].ctypes.data for k in (
                "in_ptr", "out_ptr", "in_loc", "out_loc", "L", "R", "C", "current", "voltage",
                "charge", "node_voltage", "cap", "leak", "locator")]) for h in self._keep])
            check(lib().ckt_batch_create(n, shapes, hcs, steps, ctypes.byref(self.handle)))

    def info(self) -> dict:
        w, n, b = ctypes.c_int64(), ctypes.c_int64(), ctypes.c_int64()
        u = ctypes.c_double()
        check(lib().ckt_batch_info(self.handle, ctypes.byref(w), ctypes.byref(n), ctypes.byref(u),
                                   ctypes.byref(b)))
        return {"wires": w.value, "nodes": n.value, "segment_updates_per_run": u.value,
                "device_bytes": b.value}

    def config(self) -> dict:
        c = BatchConfig()
        check(lib().ckt_batch_get_config(self.handle, ctypes.byref(c)))
        return {"block": c.block, "wires_per_thread": c.wires_per_thread,
                "dc_schedule": c.dc_schedule, "blocks_per_sm": c.blocks_per_sm}

    def set_config(self, block: int, wires_per_thread: int, dc_schedule: int) -> None:
        c = BatchConfig(block, wires_per_thread, dc_schedule, 0)
        check(lib().ckt_batch_set_config(self.handle, ctypes.byref(c)))

    def autotune(self, mode: int, stream: int = 0) -> dict:
        c = BatchConfig()
        check(lib().ckt_batch_autotune(self.handle, mode, stream, ctypes.byref(c)))
        return self.config()

    def run(self, mode: int, stream: int = 0) -> None:
        check(lib().ckt_batch_run(self.handle, mode, stream))

    def run_direct(self, mode: int, stream: int = 0) -> None:
        check(lib().ckt_batch_run_direct(self.handle, mode, stream))

    def run_sequential(self, mode: int, stream: int = 0, per_piece: bool = False) -> None:
        check(lib().ckt_batch_run_sequential(self.handle, mode, int(per_piece), stream))

    def check(self, stream: int = 0) -> int:
        """0, or the ckt_status of the last run (e.g. 4 = a wait timed out)."""
        return lib().ckt_batch_check(self.handle, stream)

    def set_timeout(self, ns: int) -> None:
        check(lib().ckt_batch_set_timeout(self.handle, int(ns)))

    def inject_stall(self, circuit: int, enable: bool = True) -> None:
        check(lib().ckt_batch_inject_stall(self.handle, circuit, int(enable)))

    def reset_state(self, stream: int = 0) -> None:
        check(lib().ckt_batch_reset_state(self.handle, stream))

    def read(self, circuit: int, stream: int = 0) -> dict:
        s = self.specs[circuit]
        W, N = s.wires, s.nodes
        out = {"current": np.empty((10, W), np.float32), "voltage": np.empty((9, W), np.float32),
               "charge": np.empty(N, np.float32), "node_voltage": np.empty(N, np.float32)}
        check(lib().ckt_batch_read_state(self.handle, circuit, out["current"].ctypes.data,
                                         out["voltage"].ctypes.data, out["charge"].ctypes.data,
                                         out["node_voltage"].ctypes.data, stream))
        return out

    def close(self) -> None:
        if self.handle:
            lib().ckt_batch_destroy(self.handle)
            self.handle = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
