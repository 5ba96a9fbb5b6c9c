"""GB300-native circuit hot path (calc_new_currents / distribute_charge /
update_voltages of LegionOrigins' circuit simulator) behind a C ABI.

The compute lives in legionorigins_gb300/_build/libckt.so (CUDA for sm_103a
plus host C++), built by legionorigins_gb300.build.build().  This module
is the ctypes binding of include/ckt.h.  There is no CPU fallback: if the
library is missing, every entry point raises.
"""
from __future__ import annotations

import ctypes
import os

from . import build as _build

__all__ = ["lib", "CktError", "Piece", "Wires", "Nodes", "Params", "GenParams", "HostCircuit",
           "MODE_EXACT", "MODE_FAST", "INIT_KERNEL", "INIT_CPU_TASK", "check"]

LIB_PATH = _build.LIB

MODE_EXACT, MODE_FAST, MODE_FAST_SCALAR, MODE_EXACT_DIVIDE = 0, 1, 2, 3
INIT_KERNEL, INIT_CPU_TASK = 0, 1
PRIVATE_PTR, SHARED_PTR, GHOST_PTR = 0, 1, 2
SEGMENTS = 10
DT = float.fromhex("0x1.0c6f7ap-20")  # (float)1e-6


class CktError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"ckt status {status}: {msg}")
        self.status = status


class Piece(ctypes.Structure):
    _fields_ = [("first_wire", ctypes.c_uint32), ("num_wires", ctypes.c_uint32),
                ("first_node", ctypes.c_uint32), ("num_nodes", ctypes.c_uint32)]


class Wires(ctypes.Structure):
    _fields_ = [(n, ctypes.c_void_p) for n in ("in_ptr", "out_ptr", "in_loc", "out_loc",
                                              "inductance", "resistance", "capacitance",
                                              "current", "voltage")] + [
        ("seg_stride", ctypes.c_int64)]


class Nodes(ctypes.Structure):
    _fields_ = [(n, ctypes.c_void_p) for n in ("charge", "voltage", "capacitance", "leakage")]


class Params(ctypes.Structure):
    _fields_ = [("steps", ctypes.c_int32), ("dt", ctypes.c_float), ("mode", ctypes.c_int32),
                ("init", ctypes.c_int32)]


class GenParams(ctypes.Structure):
    _fields_ = [("num_pieces", ctypes.c_int32), ("nodes_per_piece", ctypes.c_int32),
                ("wires_per_piece", ctypes.c_int32), ("reserved", ctypes.c_int32),
                ("pct_wire_in_piece", ctypes.c_double), ("random_seed", ctypes.c_int64),
                ("L_offset", ctypes.c_double), ("L_scale", ctypes.c_double)]


class HostCircuit(ctypes.Structure):
    _fields_ = [(n, ctypes.c_void_p) for n in (
        "in_ptr", "out_ptr", "in_loc", "out_loc", "inductance", "resistance", "capacitance",
        "current", "voltage", "charge", "node_voltage", "node_capacitance", "node_leakage",
        "locator")]


class BatchConfig(ctypes.Structure):
    _fields_ = [("block", ctypes.c_int32), ("wires_per_thread", ctypes.c_int32),
                ("dc_schedule", ctypes.c_int32), ("blocks_per_sm", ctypes.c_int32)]


class ServerConfig(ctypes.Structure):
    _fields_ = [("hbm_budget_bytes", ctypes.c_uint64), ("max_circuits", ctypes.c_int32),
                ("prep_threads", ctypes.c_int32), ("mode", ctypes.c_int32),
                ("keep_results", ctypes.c_int32), ("round_timeout_ns", ctypes.c_uint64),
                ("launch", BatchConfig), ("device_generate", ctypes.c_int32),
                ("reserved", ctypes.c_int32)]


class Request(ctypes.Structure):
    _fields_ = [("request_id", ctypes.c_uint64), ("shape", GenParams), ("steps", ctypes.c_int32),
                ("loops", ctypes.c_int32)]


class Completion(ctypes.Structure):
    _fields_ = [("request_id", ctypes.c_uint64), ("status", ctypes.c_int32),
                ("loops", ctypes.c_int32), ("submit_s", ctypes.c_double),
                ("admit_s", ctypes.c_double), ("start_s", ctypes.c_double),
                ("finish_s", ctypes.c_double), ("wires", ctypes.c_int64),
                ("nodes", ctypes.c_int64), ("segment_updates", ctypes.c_double)]


class ServerStats(ctypes.Structure):
    _fields_ = [("submitted", ctypes.c_int64), ("completed", ctypes.c_int64),
                ("rounds", ctypes.c_int64), ("resident_peak", ctypes.c_int64),
                ("bytes_in_use", ctypes.c_uint64), ("bytes_peak", ctypes.c_uint64),
                ("busy_s", ctypes.c_double), ("clock_s", ctypes.c_double)]


class DeviceCircuitArrays(ctypes.Structure):
    _fields_ = [(n, ctypes.c_void_p) for n in (
        "in_ptr", "out_ptr", "in_loc", "out_loc", "inductance", "resistance", "capacitance",
        "current", "voltage", "charge", "node_voltage", "node_capacitance", "node_leakage",
        "locator", "off", "ent", "slot_in", "slot_out", "gstart")]


class HistParams(ctypes.Structure):
    _fields_ = [(n, ctypes.c_uint32) for n in (
        "buckets", "batch_size", "num_batches", "first_batch", "seed1", "seed2")]


RED_SINGLE, RED_FOLD, RED_LOCALIZE, RED_LIST = 0, 1, 2, 3


# (name, restype, argtypes) of every exported symbol declared in include/ckt.h
_P = ctypes.c_void_p
_I32, _I64, _U32 = ctypes.c_int32, ctypes.c_int64, ctypes.c_uint32
SIGNATURES = {
    "ckt_abi_version": (ctypes.c_int, []),
    "ckt_last_error": (ctypes.c_char_p, []),
    "ckt_status_string": (ctypes.c_char_p, [ctypes.c_int]),
    "ckt_default_params": (None, [ctypes.POINTER(Params)]),
    "ckt_calc_new_currents": (ctypes.c_int, [ctypes.POINTER(Piece), Wires, Nodes, Nodes, Nodes,
                                             ctypes.POINTER(Params), _P]),
    "ckt_distribute_charge": (ctypes.c_int, [_P, _I32, Wires, Nodes, _P, _P,
                                             ctypes.POINTER(Params), _P]),
    "ckt_apply_fold": (ctypes.c_int, [_P, _I32, _P, _P, _P, _P]),
    "ckt_distribute_charge_atomic": (ctypes.c_int, [ctypes.POINTER(Piece), Wires, Nodes, _P, _P,
                                                    ctypes.POINTER(Params), _P]),
    "ckt_distribute_charge_atomic_sync": (ctypes.c_int, [ctypes.POINTER(Piece), Wires, Nodes,
                                                         _P, _P, ctypes.POINTER(Params), _P]),
    "ckt_update_voltages": (ctypes.c_int, [ctypes.POINTER(Piece), Nodes, Nodes, _P, _P]),
    "ckt_calc_new_currents_sync": (ctypes.c_int, [ctypes.POINTER(Piece), Wires, Nodes, Nodes,
                                                  Nodes, ctypes.POINTER(Params), _P]),
    "ckt_distribute_charge_sync": (ctypes.c_int, [_P, _I32, Wires, Nodes, _P, _P,
                                                  ctypes.POINTER(Params), _P]),
    "ckt_update_voltages_sync": (ctypes.c_int, [ctypes.POINTER(Piece), Nodes, Nodes, _P, _P]),
    "ckt_sanity_check_wires": (ctypes.c_int, [ctypes.POINTER(Piece), Wires, _U32,
                                              ctypes.POINTER(_I64), _P]),
    "ckt_calc_new_currents_all": (ctypes.c_int, [_P, Wires, Nodes, ctypes.POINTER(Params), _P]),
    "ckt_distribute_charge_all": (ctypes.c_int, [_P, Wires, Nodes, ctypes.POINTER(Params), _P]),
    "ckt_update_voltages_all": (ctypes.c_int, [_P, Nodes, _P]),
    "ckt_run_loops_all": (ctypes.c_int, [_P, Wires, Nodes, ctypes.POINTER(Params), _I32, _P]),
    "ckt_distribute_update_all": (ctypes.c_int, [_P, Wires, Nodes, ctypes.POINTER(Params), _P]),
    "ckt_graph_check": (ctypes.c_int, [_P, _P]),
    "ckt_distribute_charge_all_sync": (ctypes.c_int, [_P, Wires, Nodes, ctypes.POINTER(Params),
                                                      _P]),
    "ckt_distribute_update_all_sync": (ctypes.c_int, [_P, Wires, Nodes, ctypes.POINTER(Params),
                                                      _P]),
    "ckt_run_loops_all_sync": (ctypes.c_int, [_P, Wires, Nodes, ctypes.POINTER(Params), _I32,
                                              _P]),
    "ckt_graph_create": (ctypes.c_int, [ctypes.POINTER(Piece), _I32, _U32, _P, _P, _P, _P,
                                        ctypes.POINTER(_P)]),
    "ckt_graph_destroy": (ctypes.c_int, [_P]),
    "ckt_graph_info": (ctypes.c_int, [_P, ctypes.POINTER(_I64), ctypes.POINTER(_I64),
                                      ctypes.POINTER(_I32), ctypes.POINTER(_I64)]),
    "ckt_graph_tile_info": (ctypes.c_int, [_P, ctypes.POINTER(ctypes.c_int32),
                                           ctypes.POINTER(_I64), ctypes.POINTER(_I64),
                                           ctypes.POINTER(ctypes.c_uint32)]),
    "ckt_graph_set_tile_timeout": (ctypes.c_int, [_P, ctypes.c_uint64]),
    "ckt_generate": (ctypes.c_int, [ctypes.POINTER(GenParams), ctypes.POINTER(HostCircuit)]),
    "ckt_hist_default_params": (None, [ctypes.POINTER(HistParams)]),
    "ckt_hist_scratch_bytes": (ctypes.c_int, [ctypes.POINTER(HistParams), _I32,
                                              ctypes.POINTER(ctypes.c_uint64),
                                              ctypes.POINTER(ctypes.c_uint64)]),
    "ckt_hist_run": (ctypes.c_int, [ctypes.POINTER(HistParams), _I32, _P, _P, ctypes.c_uint64,
                                    _P]),
    "ckt_sanity_check_pieces_noalloc": (ctypes.c_int, [ctypes.POINTER(Piece), _I32, Wires, _U32,
                                                       ctypes.POINTER(_I64), _P]),
    "ckt_batch_create": (ctypes.c_int, [_I32, ctypes.POINTER(GenParams),
                                        ctypes.POINTER(HostCircuit), ctypes.POINTER(_I32),
                                        ctypes.POINTER(_P)]),
    "ckt_batch_generate": (ctypes.c_int, [_I32, ctypes.POINTER(GenParams), ctypes.POINTER(_I32),
                                          _I32, ctypes.POINTER(_P)]),
    "ckt_batch_destroy": (ctypes.c_int, [_P]),
    "ckt_batch_info": (ctypes.c_int, [_P, ctypes.POINTER(_I64), ctypes.POINTER(_I64),
                                      ctypes.POINTER(ctypes.c_double), ctypes.POINTER(_I64)]),
    "ckt_batch_circuit_offsets": (ctypes.c_int, [_P, _I32, ctypes.POINTER(_I64),
                                                 ctypes.POINTER(_I64)]),
    "ckt_batch_set_config": (ctypes.c_int, [_P, ctypes.POINTER(BatchConfig)]),
    "ckt_batch_get_config": (ctypes.c_int, [_P, ctypes.POINTER(BatchConfig)]),
    "ckt_batch_autotune": (ctypes.c_int, [_P, _I32, _P, ctypes.POINTER(BatchConfig)]),
    "ckt_batch_run": (ctypes.c_int, [_P, _I32, _P]),
    "ckt_batch_run_direct": (ctypes.c_int, [_P, _I32, _P]),
    "ckt_batch_run_sequential": (ctypes.c_int, [_P, _I32, _I32, _P]),
    "ckt_batch_check": (ctypes.c_int, [_P, _P]),
    "ckt_batch_set_timeout": (ctypes.c_int, [_P, ctypes.c_uint64]),
    "ckt_batch_reset_state": (ctypes.c_int, [_P, _P]),
    "ckt_batch_read_state": (ctypes.c_int, [_P, _I32, _P, _P, _P, _P, _P]),
    "ckt_batch_upload_state": (ctypes.c_int, [_P, _P, _P, _P, _P, _P]),
    "ckt_batch_download_state": (ctypes.c_int, [_P, _P, _P, _P, _P, _P]),
    "ckt_batch_inject_stall": (ctypes.c_int, [_P, _I32, _I32]),
    "ckt_generate_device": (ctypes.c_int, [ctypes.POINTER(GenParams),
                                           ctypes.POINTER(DeviceCircuitArrays), _P]),
    "ckt_graph_export": (ctypes.c_int, [_P, _P, _P, _P, _P, _P]),
    "ckt_wires_from_aos": (ctypes.c_int, [_P, _I64, Wires, _P]),
    "ckt_wires_to_aos": (ctypes.c_int, [Wires, _I64, _P, _P]),
    "ckt_nodes_from_aos": (ctypes.c_int, [_P, _I64, Nodes, _P]),
    "ckt_nodes_to_aos": (ctypes.c_int, [Nodes, _I64, _P, _P]),
    "ckt_server_default_config": (None, [ctypes.POINTER(ServerConfig)]),
    "ckt_server_create": (ctypes.c_int, [ctypes.POINTER(ServerConfig), ctypes.POINTER(_P)]),
    "ckt_server_submit": (ctypes.c_int, [_P, ctypes.POINTER(Request)]),
    "ckt_server_cancel": (ctypes.c_int, [_P, ctypes.c_uint64]),
    "ckt_server_poll": (ctypes.c_int, [_P, ctypes.POINTER(Completion), _I32,
                                       ctypes.POINTER(_I32)]),
    "ckt_server_wait": (ctypes.c_int, [_P, ctypes.c_double]),
    "ckt_server_take_result": (ctypes.c_int, [_P, ctypes.c_uint64, _P, _P, _P, _P]),
    "ckt_server_get_stats": (ctypes.c_int, [_P, ctypes.POINTER(ServerStats)]),
    "ckt_server_clock": (ctypes.c_double, [_P]),
    "ckt_server_destroy": (ctypes.c_int, [_P]),
}

# ... and of include/ckt_tools.h (libckt_tools.so: measurement and
# verification helpers, not the product library)
TOOLS_SIGNATURES = {
    "ckt_fp32_fma_probe": (ctypes.c_int, [_U32, _I32, _I32, _P, _P]),
    "ckt_check_dt_quotient": (ctypes.c_int, [ctypes.c_uint64, ctypes.c_uint64, _P, _P]),
    "ckt_check_recip_quotient": (ctypes.c_int, [ctypes.c_uint64, ctypes.c_uint64, _I32, _I32, _P,
                                                _P]),
    "ckt_check_wide_quotient": (ctypes.c_int, [ctypes.c_uint64, ctypes.c_uint64, _I32, _P, _P]),
}

_lib = None
_tools = None


def tools() -> ctypes.CDLL:
    """Load libckt_tools.so (the FP32 probe and the quotient checks)."""
    global _tools
    if _tools is None:
        lib()
        if not os.path.exists(_build.TOOLS_LIB):
            raise RuntimeError(f"{_build.TOOLS_LIB} is not built; run legionorigins_gb300.build.build()")
        T = ctypes.CDLL(_build.TOOLS_LIB)
        for name, (res, args) in TOOLS_SIGNATURES.items():
            fn = getattr(T, name)
            fn.restype = res
            fn.argtypes = args
        _tools = T
    return _tools


def lib(build_if_missing: bool = False) -> ctypes.CDLL:
    """Load libckt.so.  Raises if it has not been built (no fallback)."""
    global _lib
    if _lib is not None:
        return _lib
    if build_if_missing:
        _build.build()
    if not os.path.exists(LIB_PATH):
        raise RuntimeError(f"{LIB_PATH} is not built; run legionorigins_gb300.build.build()")
    L = ctypes.CDLL(LIB_PATH)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args
    _lib = L
    return L


def check(status: int) -> None:
    if status != 0:
        msg = lib().ckt_last_error().decode(errors="replace")
        raise CktError(status, msg)


def default_params(steps: int = 10000, mode: int = MODE_EXACT, init: int = INIT_KERNEL) -> Params:
    p = Params()
    lib().ckt_default_params(ctypes.byref(p))
    p.steps, p.mode, p.init = steps, mode, init
    return p
