"""Serving loop: circuit-solve requests admitted under an HBM budget, kept
resident, advanced together one outer loop per persistent launch
(include/ckt.h, ckt_server_*)."""
from __future__ import annotations

import ctypes

import numpy as np

from . import Completion, Request, ServerConfig, ServerStats, check, lib
from .batch import _gp
from .workloads import CircuitSpec


class Server:
    def __init__(self, mode: int = 0, hbm_budget_bytes: int = 80 << 30, max_circuits: int = 4096,
                 prep_threads: int = 0, keep_results: bool = False, launch=None,
                 round_timeout_ns: int = 0, device_generate: bool = True):
        cfg = ServerConfig()
        lib().ckt_server_default_config(ctypes.byref(cfg))
        cfg.mode = mode
        cfg.hbm_budget_bytes = int(hbm_budget_bytes)
        cfg.max_circuits = max_circuits
        if prep_threads:
            cfg.prep_threads = prep_threads
        cfg.keep_results = int(keep_results)
        cfg.device_generate = int(device_generate)
        if round_timeout_ns:
            cfg.round_timeout_ns = round_timeout_ns
        if launch is not None:
            cfg.launch.block, cfg.launch.wires_per_thread, cfg.launch.dc_schedule = launch
        self.handle = ctypes.c_void_p()
        check(lib().ckt_server_create(ctypes.byref(cfg), ctypes.byref(self.handle)))
        self.specs: dict[int, CircuitSpec] = {}

    def submit(self, request_id: int, spec: CircuitSpec) -> None:
        r = Request(request_id, _gp(spec), spec.steps, spec.loops)
        check(lib().ckt_server_submit(self.handle, ctypes.byref(r)))
        self.specs[request_id] = spec

    def cancel(self, request_id: int) -> None:
        check(lib().ckt_server_cancel(self.handle, request_id))

    def poll(self, capacity: int = 4096) -> list[dict]:
        buf = (Completion * capacity)()
        n = ctypes.c_int32()
        check(lib().ckt_server_poll(self.handle, buf, capacity, ctypes.byref(n)))
        return [{k: getattr(buf[i], k) for k, _ in Completion._fields_} for i in range(n.value)]

    def wait(self, timeout_s: float) -> int:
        return lib().ckt_server_wait(self.handle, float(timeout_s))

    def take_result(self, request_id: int) -> dict:
        s = self.specs[request_id]
        W, N = s.wires, s.nodes
        out = {"current": np.empty((10, W), np.float32), "voltage": np.empty((9, W), np.float32),
               "charge": np.empty(N, np.float32), "node_voltage": np.empty(N, np.float32)}
        check(lib().ckt_server_take_result(self.handle, request_id, out["current"].ctypes.data,
                                           out["voltage"].ctypes.data, out["charge"].ctypes.data,
                                           out["node_voltage"].ctypes.data))
        return out

    def stats(self) -> dict:
        st = ServerStats()
        check(lib().ckt_server_get_stats(self.handle, ctypes.byref(st)))
        return {k: getattr(st, k) for k, _ in ServerStats._fields_}

    def clock(self) -> float:
        return lib().ckt_server_clock(self.handle)

    def close(self) -> None:
        if self.handle:
            lib().ckt_server_destroy(self.handle)
            self.handle = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
