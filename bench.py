"""Benchmark of the circuit hot path on GB300.

Default workload (one GPU): the plain circuit at scale -- 64 pieces x 16384
nodes x 65536 wires per piece (4,194,304 wires), 95% of wires in-piece, 10
segments per wire, dt = 1e-6, 1000 inner steps, 10 outer loops, fp32, inputs
from the reference generator's distributions with seed 12345 (inductance
U[0.001, 0.011)).

One STEP is one whole simulation of that workload, as the reference times it
(apps/circuit/circuit.cc:164-167, 311-312): the circuit state is reset to its
generated values, then 10 outer loops of calc_new_currents (all pieces),
distribute_charge (all pieces), update_voltages (all pieces) run.  The
metric is wire-segment updates per second = wires x 10 segments x 1000
inner steps x 10 loops / time.  The working set (411 MB of wire state) is
larger than L2.

  value  device-resident: state reset by a device copy, then per loop the
         library's two launches (calc_new_currents, then one node pass for
         distribute_charge + update_voltages; bit-identical to the three task
         launches), on one stream
  e2e    through ckt_run_loops_all with host buffers: every step copies the
         circuit from pinned host memory to the device, runs the 10 loops and
         copies the resulting state back; with two device copies of the
         circuit, a step's copies overlap its neighbours' loops
  index_space_tasks  the same steps through the three separate index-space
         task launches per loop (the drop-in boundary), with their kernels

`--impl reference` times the reference's CPU implementation of the same three
tasks (its shared-low-level execution style: one thread per core, piece p on
thread p mod T, barriers between launches, 128-byte wires copied by value) on
the host cores, restated in oracle/ckt_oracle.c because the reference's own
circuit.cc cannot be built against the runtime it ships with.

Usage: python bench.py [--gpus N] [--steps K] [--warmup W] [--mode fast|exact]
                       [--impl ours|reference]
Multi-GPU (torchrun): every rank simulates its own replica of the circuit
(the path needs no exchange between replicas); value sums all ranks' updates
over the slowest rank's time.
"""
from __future__ import annotations

import argparse
import ctypes
import json
import math
import os
import statistics
import subprocess
import sys
import time

import numpy as np

# More hardware work queues than the default 8, so that the separate copy and
# compute streams of the end-to-end pipelines do not share one queue and
# wait on each other's unrelated work (set before the CUDA context exists).
os.environ.setdefault("CUDA_DEVICE_MAX_CONNECTIONS", "32")

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "wire-segment updates/s at 1 GB300 (plain vs batched/served); p50/p99 solve latency"
UNIT = "wire-segment updates/s"
SHAPE = dict(num_pieces=64, nodes_per_piece=16384, wires_per_piece=65536)
PCT, SEED, INNER_STEPS, OUTER_LOOPS = 95.0, 12345, 1000, 10
L_OFFSET, L_SCALE = 0.001, 0.01
FLOPS_PER_WIRE_STEP = 96  # the reference's own count (apps/circuit/circuit.cc:324)
# FP32-pipe operations calc_new_currents issues per wire-step in its common
# path: EXACT 67 plain operations + 10 split-reciprocal quotients by dt (2
# each) + 19 corrected quotients by R and C (4 each); FAST 48.
FP32_OPS_PER_WIRE_STEP = {0: 163, 1: 48}
CNC_TRAFFIC_PER_WIRE = (103.879424e6 + 21.284608e6) / 1048576  # measured DRAM bytes per wire


def workload_config(mode: str, pieces: int = SHAPE["num_pieces"]) -> dict:
    if INNER_STEPS != 1000:
        return {"workload": "PROFILING CASE, not the configured workload: the heavy-reduction "
                            "circuit (128 x 8192 x 32768, 50% in-piece, S=500 x 10 loops)",
                "mode": mode}
    if pieces != SHAPE["num_pieces"]:
        return {"workload": f"PROFILING CASE, not the configured workload: {pieces} pieces x "
                            f"16384 nodes x 65536 wires/piece, S=1000 x 10 loops", "mode": mode}
    return {
        "workload": "plain circuit at scale: 64 pieces x 16384 nodes x 65536 wires/piece "
                    "(4,194,304 wires), 95% in-piece, 10 segments, S=1000 inner steps x "
                    "10 outer loops per step, seed 12345",
        "pieces": SHAPE["num_pieces"], "nodes_per_piece": SHAPE["nodes_per_piece"],
        "wires_per_piece": SHAPE["wires_per_piece"], "inner_steps": INNER_STEPS,
        "outer_loops_per_step": OUTER_LOOPS, "mode": mode,
        "l2": "inputs larger than L2 (411 MB of wire state per step)",
    }


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


class Clocks:
    """nvidia-smi sampled every 200 ms during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.path = os.path.join("/tmp", f"ckt_clocks_{os.getpid()}.csv")

    def __enter__(self):
        try:
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.Q}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=self.f, stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
            self.f.close()

    def summary(self) -> dict:
        if self.proc is None or not os.path.exists(self.path):
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        rows = []
        for line in open(self.path):
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                rows.append((float(parts[1]), float(parts[2]), parts[5:9]))
            except ValueError:
                continue
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for _, _, r in rows for i, v in enumerate(r) if v == "Active"})
        loaded = [r[0] for r in rows]
        return {"sm_mhz": statistics.median(loaded), "sm_max_mhz": max(r[1] for r in rows),
                "samples": len(rows), "reasons": reasons}


def measured_peaks() -> dict:
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        try:
            return json.load(open(p))
        except ValueError:
            pass
    return {}


def cpu_threads() -> int:
    try:
        return len(os.sched_getaffinity(0))
    except AttributeError:
        return os.cpu_count() or 1


def reference_sample(threads: int, target_s: float):
    """A bounded sample of the workload for the CPU implementation: one
    outer loop of S=1000 over the first `pieces` pieces (whole pieces, one
    or more per thread), sized to about `target_s` seconds."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import ckt_oracle as O

    O.build()
    p = O.GenParams(SHAPE["num_pieces"], SHAPE["nodes_per_piece"], SHAPE["wires_per_piece"],
                    PCT, SEED, L_offset=L_OFFSET, L_scale=L_SCALE)
    base = O.generate(p)
    # calibrate on one piece per thread at 100 inner steps
    pieces = min(threads, p.num_pieces)
    c = base.copy()
    t = O.baseline_run(c, 1, 100, threads, pieces)
    per_piece_step = t / 100.0 / math.ceil(pieces / threads)
    rounds = max(1, min(p.num_pieces // threads if threads <= p.num_pieces else 1,
                        int(target_s / max(per_piece_step * INNER_STEPS, 1e-9))))
    pieces = min(p.num_pieces, threads * rounds)
    return O, p, base, pieces


def port_vs_reference() -> dict | None:
    """The reference's own circuit.cc (compiled unmodified through the shim,
    -O3 as its runtime.mk builds, single-threaded) timed on this host beside
    the C restatement on one thread on the same circuit and steps: shows
    that the restatement the CPU baseline runs is as fast as the
    reference's own code.  None when the reference binary is not built."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import ckt_oracle as O

    if not os.path.exists(O.REF_BIN):
        return None
    p = O.GenParams(2, 1024, 4096, PCT, SEED, L_offset=0.1, L_scale=0.01)
    try:
        tr = min(O.time_reference(p, 1) for _ in range(2))
    except (OSError, RuntimeError, subprocess.CalledProcessError) as e:
        return {"unavailable": f"the reference binary did not run: {e}"}
    tp = min(O.baseline_run(O.generate(p), 1, 10000, 1, 2) for _ in range(2))
    return {"circuit": "2 pieces x 1024 nodes x 4096 wires/piece, 95% in-piece, the reference's "
                       "own inductance range, 1 loop of its STEPS = 10000 inner steps",
            "reference_s": tr, "port_s": tp, "port_over_reference_rate": tr / tp,
            "note": "apps/circuit/circuit.cc's own main loop (its ELAPSED TIME), built "
                    "unmodified through oracle/refshim at -O3, single-threaded; the port "
                    "(oracle/ckt_oracle.c) on one thread"}


def run_reference_arm(args) -> None:
    ws, rank, _ = dist_env()
    if rank != 0:
        return
    if args.workload == "reductions":
        cpu = None
        vals = []
        for _ in range(args.steps):
            cpu = red_cpu_baseline(args)
            vals.append(cpu["value"])
        value = statistics.median(vals)
        cpu["value"] = value
        print(json.dumps({
            "impl": "reference", "metric": RED_METRIC, "value": value, "unit": "reductions/s",
            "n_gpus": ws, "steps": args.steps, "warmup": args.warmup, "ms_per_step": None,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u32",
            "data": "synthetic (the benchmark's own hash of the element index)",
            "config": {"workload": "reducetest dense: 262144 buckets, batches of 4194304, "
                                   "redfold on the host cores"},
            "cpu_baseline": cpu,
            "e2e": {"value": value, "unit": "reductions/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}), flush=True)
        return
    threads = cpu_threads()
    O, p, base, pieces = reference_sample(threads, args.cpu_sample_s)
    updates = pieces * p.wires_per_piece * 10 * INNER_STEPS
    for _ in range(args.warmup):
        O.baseline_run(base.copy(), 1, INNER_STEPS, threads, pieces)
    times = []
    for _ in range(args.steps):
        c = base.copy()
        times.append(O.baseline_run(c, 1, INNER_STEPS, threads, pieces))
    total = sum(times)
    value = updates * args.steps / total
    sample = (f"1 outer loop x {INNER_STEPS} inner steps over {pieces} of "
              f"{p.num_pieces} pieces ({pieces * p.wires_per_piece} wires) per step")
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * total / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (reference generator, seed 12345)",
        "config": workload_config("reference CPU tasks (IEEE fp32)"),
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
                         "sample": sample,
                         "port_vs_reference_single_thread": port_vs_reference()},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def same_bits(a, b) -> bool:
    """Bit equality where every NaN equals every NaN (NaN payloads differ
    between the host ISA and the GPU)."""
    na, nb = np.isnan(a), np.isnan(b)
    return bool(np.array_equal(na, nb) and
                np.array_equal(a[~na].view(np.uint32), b[~nb].view(np.uint32)))


def accuracy_check(torch, G, C, mode, shape_args, configured_steps) -> dict:
    """The arithmetic this run times, against the oracle (the checker, on the
    host) on the timed workload's own circuit.
      finite regime: the whole circuit, 4 inner steps x 2 loops, every value
        finite: bit equality with the fp32 oracle (the reference's
        arithmetic), per-element relative error against it and against the
        fp64 oracle;
      configured steps: one loop at the configured inner steps (the
        recurrence overflows to NaN): calc_new_currents on the first piece's
        wires (each wire is independent given the node voltages),
        distribute_charge + update_voltages on the whole circuit from the
        GPU's currents; bit equality and NaN/+-Inf/finite class agreement."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import ckt_oracle as O

    O.build()
    P, npp, wpp, pct = shape_args
    gp = O.GenParams(P, npp, wpp, pct, SEED, L_offset=L_OFFSET, L_scale=L_SCALE)
    base = O.generate(gp)
    fields = ("in_ptr", "out_ptr", "in_loc", "out_loc", "L", "R", "C", "current", "voltage",
              "charge", "node_voltage", "cap", "leak", "locator")
    state = ("current", "voltage", "charge", "node_voltage")
    shape = C.Shape(P, npp, wpp)

    def device():
        return C.DeviceCircuit({k: np.ascontiguousarray(getattr(base, k)) for k in fields}, shape)

    def rel(a, b):
        a, b = a.astype(np.float64).ravel(), b.astype(np.float64).ravel()
        f = np.isfinite(a) & np.isfinite(b)
        return np.abs(a[f] - b[f]) / np.maximum(np.abs(b[f]), 1e-6)

    def cls(a):
        return np.where(np.isnan(a), 0, np.where(np.isposinf(a), 1, np.where(np.isneginf(a), 2, 3)))

    dc = device()
    dc.run_loops(C.params(4, mode), 2, blocking=True)
    got = dc.to_host()
    dc.close()
    ref32 = base.copy()
    O.simulate(ref32, 2, 4)
    ref64 = base.astype(np.float64)
    O.simulate(ref64, 2, 4)
    r32 = np.concatenate([rel(got[k], getattr(ref32, k)) for k in state])
    r64 = np.concatenate([rel(got[k], getattr(ref64, k)) for k in state])
    rr = np.concatenate([rel(getattr(ref32, k), getattr(ref64, k)) for k in state])
    finite = {
        "circuit": f"{P} x {npp} x {wpp}, {pct:g}% in-piece (the timed circuit, whole)",
        "inner_steps": 4, "loops": 2,
        "all_finite": bool(all(np.isfinite(getattr(ref32, k)).all() for k in state)),
        "bit_identical_to_fp32_reference": all(same_bits(got[k], getattr(ref32, k))
                                               for k in state),
        "max_rel_err_vs_fp32_reference": float(r32.max()),
        "elements_over_1e-5_vs_fp32_reference": int((r32 > 1e-5).sum()),
        "elements": int(r32.size),
        "max_rel_err_vs_fp64": float(r64.max()),
        "rms_rel_err_vs_fp64": float(np.sqrt(np.mean(r64 ** 2))),
        "fp32_reference_vs_fp64": {"max_rel_err": float(rr.max()),
                                   "rms_rel_err": float(np.sqrt(np.mean(rr ** 2)))},
    }
    dc = device()
    L = G.lib()
    prm = C.params(configured_steps, mode)
    G.check(L.ckt_calc_new_currents_all(dc.graph.handle, dc.wires(), dc.nodes(),
                                        ctypes.byref(prm), None))
    torch.cuda.synchronize()
    after_cnc = dc.to_host()
    G.check(L.ckt_distribute_update_all_sync(dc.graph.handle, dc.wires(), dc.nodes(),
                                             ctypes.byref(prm), None))
    after = dc.to_host()
    dc.close()
    ref = base.copy()
    O.calc_new_currents(ref, configured_steps, w_begin=0, w_end=wpp)
    c2 = base.copy()
    c2.current[:], c2.voltage[:] = after_cnc["current"], after_cnc["voltage"]
    O.distribute_charge(c2)
    O.update_voltages(c2)
    pairs = [(after_cnc[k][:, :wpp], getattr(ref, k)[:, :wpp]) for k in ("current", "voltage")]
    pairs += [(after[k], getattr(c2, k)) for k in ("charge", "node_voltage")]
    n_el = sum(a.size for a, _ in pairs)
    configured = {
        "inner_steps": configured_steps, "loops": 1,
        "checked": f"calc_new_currents on wires [0, {wpp}) (piece 0); distribute_charge + "
                   "update_voltages on every node",
        "bit_identical_to_fp32_reference": all(same_bits(a, b) for a, b in pairs),
        "class_match_vs_fp32_reference": sum(int((cls(a) == cls(b)).sum()) for a, b in pairs) / n_el,
        "elements": n_el,
        "finite_elements": int(sum(np.isfinite(a).sum() for a, _ in pairs)),
    }
    return {"finite_regime": finite, "configured_steps": configured}


def batch_accuracy_check(torch, mode, specs) -> dict:
    """The same statement for the batched kernel (which the serving rounds
    run too): the first 8 circuits of the workload's mix, each with 4 inner
    steps, 2 loops, against the fp64 oracle; and the first 4 at their own
    inner-step counts, 1 loop, NaN/+-Inf/finite classes against the fp32
    oracle."""
    from dataclasses import replace

    from legionorigins_gb300.batch import Batch

    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import ckt_oracle as O

    O.build()
    state = ("current", "voltage", "charge", "node_voltage")

    def oracle_circuit(sp):
        return O.generate(O.GenParams(*sp.gen_args()[:5], L_offset=sp.L_offset,
                                      L_scale=sp.L_scale))

    def cls(a):
        return np.where(np.isnan(a), 0, np.where(np.isposinf(a), 1, np.where(np.isneginf(a), 2, 3)))

    def rel_err(a, b):
        a, b = a.astype(np.float64), b.astype(np.float64)
        return (np.abs(a - b) / np.maximum(np.abs(b), 1e-6)).ravel()

    finite = [replace(sp, steps=4) for sp in specs[:8]]
    b = Batch(finite)
    b.run(mode)
    b.run(mode)
    torch.cuda.synchronize()
    def norm_err(a, b):  # per field: ||a - b|| / ||b|| over the finite elements of b
        a, b = a.astype(np.float64).ravel(), b.astype(np.float64).ravel()
        f = np.isfinite(b) & np.isfinite(a)
        return float(np.linalg.norm(a[f] - b[f]) / max(np.linalg.norm(b[f]), 1e-30))

    rels, rels32, refs, norm32 = [], [], [], 0.0
    for i, sp in enumerate(finite):
        got = b.read(i)
        ref64 = oracle_circuit(sp).astype(np.float64)
        O.simulate(ref64, 2, sp.steps)
        ref32 = oracle_circuit(sp)
        O.simulate(ref32, 2, sp.steps)
        for k in state:
            rels.append(rel_err(got[k], getattr(ref64, k)))
            rels32.append(rel_err(got[k], getattr(ref32, k)))
            refs.append(rel_err(getattr(ref32, k), getattr(ref64, k)))
            norm32 = max(norm32, norm_err(got[k], getattr(ref32, k)))
    b.close()
    rel, rel32, refrel = np.concatenate(rels), np.concatenate(rels32), np.concatenate(refs)
    configured = list(specs[:4])
    b = Batch(configured)
    b.run(mode)
    torch.cuda.synchronize()
    same = total = 0
    for i, sp in enumerate(configured):
        got = b.read(i)
        ref = oracle_circuit(sp)
        O.simulate(ref, 1, sp.steps)
        same += sum(int((cls(got[k]) == cls(getattr(ref, k))).sum()) for k in state)
        total += sum(got[k].size for k in state)
    b.close()
    return {"finite_regime": {"circuits": "the first 8 of the mix, 4 inner steps", "loops": 2,
                              "max_rel_err_vs_fp64": float(rel.max()),
                              "rms_rel_err_vs_fp64": float(np.sqrt(np.mean(rel ** 2))),
                              "max_rel_err_vs_fp32_reference": float(rel32.max()),
                              "max_normwise_err_vs_fp32_reference": norm32,
                              "fp32_reference_vs_fp64": {
                                  "max_rel_err": float(refrel.max()),
                                  "rms_rel_err": float(np.sqrt(np.mean(refrel ** 2))),
                                  "note": "the reference's own fp32 arithmetic (the oracle "
                                          "restating it bit for bit) against fp64: the stiff "
                                          "recurrence amplifies fp32 rounding"}},
            "configured_steps": {"circuits": "the first 4 of the mix at their inner steps",
                                 "loops": 1, "class_match_vs_fp32_oracle": same / total,
                                 "elements": total}}


def fp32_peak(torch, G, stream) -> dict:
    """Measured FP32 FMA throughput (FLOP/s) of this GPU, best of 5, with
    single and with paired (f32x2) FMAs; the roofline uses the larger."""
    sm = torch.cuda.get_device_properties(0).multi_processor_count
    sink = torch.zeros(1, device="cuda")
    blocks, iters = sm * 8, 2048
    flops = blocks * 256 * iters * 16 * 8 * 2
    out = {}
    s0, s1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    for paired in (0, 1):
        best = 0.0
        for i in range(6):
            s0.record(stream)
            G.check(G.tools().ckt_fp32_fma_probe(blocks, iters, paired, sink.data_ptr(),
                                               stream.cuda_stream))
            s1.record(stream)
            s1.synchronize()
            if i:
                best = max(best, flops / (s0.elapsed_time(s1) * 1e-3))
        out["paired" if paired else "single"] = best
    out["peak"] = max(out["single"], out["paired"])
    return out


def plain_measure(torch, G, C, host, shape, mode, inner, loops, steps, warmup, local,
                  peak32=None, hbm=None, count_nonfinite=False) -> dict:
    """Device-resident timing of one plain workload: a step resets the state
    by a device copy and runs `loops` outer loops of the library's loop
    (calc_new_currents, then the fused node pass); then the three separate
    task launches per loop, for the node kernels' own times.  CUDA events on
    the launching stream; the tiled pass's error word is checked after every
    timed section."""
    L = G.lib()
    dc = C.DeviceCircuit(host, shape, device=f"cuda:{local}")
    stream = torch.cuda.Stream()
    sp = stream.cuda_stream
    prm = C.params(inner, mode)
    pristine = {k: dc.t[k].clone() for k in C.STATE_FIELDS}
    g, w, n = dc.graph.handle, dc.wires(), dc.nodes()
    E = lambda: torch.cuda.Event(enable_timing=True)  # noqa: E731
    ev = {"cnc": [], "dcuv": [], "dc": [], "uv": []}
    calls = {"fused": (("cnc", lambda: L.ckt_calc_new_currents_all(g, w, n, ctypes.byref(prm), sp)),
                       ("dcuv", lambda: L.ckt_distribute_update_all(g, w, n, ctypes.byref(prm),
                                                                    sp))),
             "tasks": (("cnc", lambda: L.ckt_calc_new_currents_all(g, w, n, ctypes.byref(prm), sp)),
                       ("dc", lambda: L.ckt_distribute_charge_all(g, w, n, ctypes.byref(prm), sp)),
                       ("uv", lambda: L.ckt_update_voltages_all(g, n, sp)))}

    def step(form, record):
        with torch.cuda.stream(stream):
            for k in C.STATE_FIELDS:
                dc.t[k].copy_(pristine[k], non_blocking=True)
        for _ in range(loops):
            for name, fn in calls[form]:
                if record and not (form == "tasks" and name == "cnc"):
                    a, b = E(), E()
                    a.record(stream)
                    G.check(fn())
                    b.record(stream)
                    ev[name].append((a, b))
                else:
                    G.check(fn())

    for _ in range(warmup):
        step("fused", False)
    torch.cuda.synchronize()
    t0, t1 = E(), E()
    t0.record(stream)
    for _ in range(steps):
        step("fused", True)
    t1.record(stream)
    torch.cuda.synchronize()
    G.check(L.ckt_graph_check(g, sp))
    elapsed = t0.elapsed_time(t1) * 1e-3
    nonfinite = None
    if count_nonfinite:  # the state one step leaves: how much of it is NaN or infinite
        torch.cuda.synchronize()
        bad = sum(int((~torch.isfinite(dc.t[k])).sum()) for k in C.STATE_FIELDS)
        nonfinite = bad / sum(dc.t[k].numel() for k in C.STATE_FIELDS)
    step("tasks", False)
    for _ in range(max(1, min(steps, 2))):
        step("tasks", True)
    torch.cuda.synchronize()
    G.check(L.ckt_graph_check(g, sp))
    dc.close()
    ms = {k: 1e3 * statistics.mean(a.elapsed_time(b) * 1e-3 for a, b in v) for k, v in ev.items()}
    W, N = shape.W, shape.N
    byts = {"dcuv": 16 * W + 24 * N, "dc": 16 * W + 8 * N, "uv": 24 * N}
    kern = {"calc_new_currents": {"ms": ms["cnc"]}}
    if peak32:
        kern["calc_new_currents"]["frac_fp32_peak"] = (FLOPS_PER_WIRE_STEP * W * inner /
                                                       (ms["cnc"] * 1e-3) / peak32)
    for name, key in (("distribute_update", "dcuv"), ("distribute_charge", "dc"),
                      ("update_voltages", "uv")):
        kern[name] = {"ms": ms[key], "algo_bytes": byts[key],
                      "gbs": byts[key] / (ms[key] * 1e-3) / 1e9}
        if hbm:
            kern[name]["frac_hbm"] = kern[name]["gbs"] / hbm
    updates = W * 10 * inner * loops * steps
    out = {"value": updates / elapsed, "unit": UNIT, "ms_per_step": 1e3 * elapsed / steps,
           "steps": steps, "kernels": kern}
    if count_nonfinite:
        out["nonfinite_fraction_after_step"] = nonfinite
    return out


def main() -> None:
    global INNER_STEPS
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--mode", choices=["fast", "exact"], default="exact",
                    help="exact: the reference's fp32 arithmetic bit for bit (the headline); "
                         "fast: reassociated FMA arithmetic, reported beside it")
    ap.add_argument("--no-extras", action="store_true",
                    help="plain workload: skip the config-0/config-2, finite-regime, FAST, "
                         "batched and served sub-measurements")
    ap.add_argument("--extra-serve-rates", default="120,260",
                    help="plain workload: offered request rates (requests/s) of the served "
                         "sub-measurement")
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--cpu-sample-s", type=float, default=3.0,
                    help="target seconds of CPU work per sampled step of the CPU baseline")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--workload", choices=["plain", "batched", "serve", "reductions",
                                           "generate", "layout"],
                    default="plain",
                    help="plain: 64x16384x65536 circuit (default); batched: 256 mixed circuits; "
                         "serve: Poisson request stream; reductions: the reduction "
                         "microbenchmark (reducetest) under each schedule; generate: building "
                         "the config-1 circuit on the GPU vs the host; layout: AoS <-> SoA")
    ap.add_argument("--rates", default="100,200,400,600,800",
                    help="serve: offered request rates (requests/s) to sweep")
    ap.add_argument("--serve-seconds", type=float, default=6.0,
                    help="serve: seconds of arrivals per rate")
    ap.add_argument("--serve-plain-sample", type=int, default=48,
                    help="serve: requests of the stream also timed through the plain path")
    ap.add_argument("--serve-launch", default="",
                    help="serve: round launch shape block,wires_per_thread,dc_schedule "
                         "(default: the library's)")
    ap.add_argument("--plain-config", type=int, choices=[1, 2], default=1,
                    help="profiling only: 2 times the heavy-reduction circuit (128 x 8192 x "
                         "32768, 50%% in-piece, S=500) as the plain workload instead of config 1")
    ap.add_argument("--pieces", type=int, default=SHAPE["num_pieces"],
                    help="profiling only: simulate the first P pieces' shape (P x 16384 x 65536)")
    ap.add_argument("--batch-launch", default="",
                    help="batched, profiling only: launch shape block,wires_per_thread,dc_schedule "
                         "instead of the autotuner's choice")
    ap.add_argument("--circuits", type=int, default=256,
                    help="batched: number of circuits of the mix (256 for the benchmark; fewer "
                         "only to profile)")
    args = ap.parse_args()
    if args.warmup < 3:
        ap.error("--warmup must be >= 3")
    if args.impl == "reference":
        run_reference_arm(args)
        return

    import torch

    import legionorigins_gb300 as G
    from legionorigins_gb300 import build as B
    from legionorigins_gb300 import circuit as C

    ws, rank, local = dist_env()
    if not torch.cuda.is_available():
        raise SystemExit("bench.py needs a CUDA device")
    torch.cuda.set_device(local)
    dist = None
    if ws > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    B.build()
    L = G.lib()
    mode = G.MODE_FAST if args.mode == "fast" else G.MODE_EXACT

    if args.workload == "batched":
        run_batched(args, torch, G, ws, rank, local, dist, mode)
        return
    if args.workload == "serve":
        run_serve(args, torch, G, ws, rank, local, dist, mode)
        return
    if args.workload == "reductions":
        run_reductions(args, torch, G, ws, rank, local, dist)
        return
    if args.workload == "generate":
        run_generate(args, torch, G, ws, rank, local, dist)
        return
    if args.workload == "layout":
        run_layout(args, torch, G, ws, rank, local, dist)
        return

    # CPU baseline first (rank 0, N=1 only), before any GPU work is queued.
    cpu_baseline = None
    if rank == 0 and ws == 1 and not args.no_cpu_baseline:
        threads = cpu_threads()
        O, p, base, pieces = reference_sample(threads, args.cpu_sample_s)
        t = O.baseline_run(base.copy(), 1, INNER_STEPS, threads, pieces)
        cpu_baseline = {
            "value": pieces * p.wires_per_piece * 10 * INNER_STEPS / t, "unit": UNIT,
            "cores": threads, "kind": "port",
            "sample": f"1 outer loop x {INNER_STEPS} inner steps over {pieces} of {p.num_pieces} "
                      f"pieces ({pieces * p.wires_per_piece} wires), reference CPU tasks "
                      f"restated in C (oracle/ckt_oracle.c, -O3), {threads} threads",
            "port_vs_reference_single_thread": port_vs_reference(),
        }

    # Accuracy of the arithmetic this run uses, stated with the number (the
    # oracle as the checker, on the host): the library's loop on the timed
    # circuit itself against the fp32 and fp64 oracles.
    accuracy = None
    if rank == 0 and ws == 1 and not args.no_cpu_baseline:
        accuracy = accuracy_check(torch, G, C, mode, (SHAPE["num_pieces"], SHAPE["nodes_per_piece"],
                                                      SHAPE["wires_per_piece"], PCT), INNER_STEPS)

    if args.plain_config == 2:  # profiling: the heavy-reduction circuit as the plain workload
        INNER_STEPS = 500
        shape = C.Shape(128, 8192, 32768)
        host = C.generate(128, 8192, 32768, 50.0, SEED, L_OFFSET, L_SCALE)
    else:
        shape = C.Shape(args.pieces, SHAPE["nodes_per_piece"], SHAPE["wires_per_piece"])
        host = C.generate(shape.num_pieces, shape.nodes_per_piece, shape.wires_per_piece, PCT,
                          SEED + 0, L_OFFSET, L_SCALE)
    dc = C.DeviceCircuit(host, shape, device=f"cuda:{local}")
    stream = torch.cuda.Stream()
    sp = stream.cuda_stream
    prm = C.params(INNER_STEPS, mode)
    pristine = {k: dc.t[k].clone() for k in C.STATE_FIELDS}
    g, w, n = dc.graph.handle, dc.wires(), dc.nodes()
    graph_bytes = dc.graph.info()["device_bytes"]
    tiles = ctypes.c_int32()
    G.check(L.ckt_graph_tile_info(g, ctypes.byref(tiles), None, None, None))
    node_pass = ("tiled (dc_tile_kernel)" if tiles.value > 0 and w.current % 16 == 0
                 and w.seg_stride % 4 == 0 else "gather (dc_all_kernel / dcuv_kernel)")
    E = lambda: torch.cuda.Event(enable_timing=True)  # noqa: E731

    def reset():
        with torch.cuda.stream(stream):
            for k in C.STATE_FIELDS:
                dc.t[k].copy_(pristine[k], non_blocking=True)

    # The library's loop: calc_new_currents, then one node pass for
    # distribute_charge + update_voltages (ckt_run_loops_all, bit-identical
    # to the three task launches).  The three separate index-space launches
    # -- the drop-in boundary -- are timed after it.
    fused = (("cnc", lambda: L.ckt_calc_new_currents_all(g, w, n, ctypes.byref(prm), sp)),
             ("dcuv", lambda: L.ckt_distribute_update_all(g, w, n, ctypes.byref(prm), sp)))
    tasks = (("cnc", lambda: L.ckt_calc_new_currents_all(g, w, n, ctypes.byref(prm), sp)),
             ("dc", lambda: L.ckt_distribute_charge_all(g, w, n, ctypes.byref(prm), sp)),
             ("uv", lambda: L.ckt_update_voltages_all(g, n, sp)))
    kernel_events = {"cnc": [], "dcuv": [], "dc": [], "uv": []}

    def loop(record: bool, calls=fused):
        for name, fn in calls:
            if record:
                a, b = E(), E()
                a.record(stream)
                G.check(fn())
                b.record(stream)
                kernel_events[name].append((a, b))
            else:
                G.check(fn())

    def step(record: bool, calls=fused):
        reset()
        for _ in range(OUTER_LOOPS):
            loop(record, calls)

    def barrier():
        if dist is not None:
            dist.barrier()

    torch.cuda.synchronize()
    for _ in range(args.warmup):
        step(False)
    torch.cuda.synchronize()
    barrier()
    t0, t1 = E(), E()
    with Clocks(local) as clk:
        torch.cuda.synchronize()
        t0.record(stream)
        for _ in range(args.steps):
            step(True)
        t1.record(stream)
        torch.cuda.synchronize()
    G.check(L.ckt_graph_check(g, sp))  # no tiled pass left a tile unwritten
    barrier()
    from legionorigins_gb300 import replicas

    updates_per_step = shape.W * 10 * INNER_STEPS * OUTER_LOOPS
    total, elapsed, _ = replicas.aggregate(updates_per_step * args.steps,
                                           t0.elapsed_time(t1) * 1e-3, device="cuda")
    value = total / elapsed
    launches = sum(len(v) for v in kernel_events.values())
    kt = {k: [a.elapsed_time(b) * 1e-3 for a, b in v] for k, v in kernel_events.items()}

    # The drop-in boundary: the three index-space task launches per loop.
    cnc_fused = kernel_events["cnc"]
    kernel_events["cnc"] = []
    task_steps = max(3, min(args.steps, 5))
    for _ in range(args.warmup):
        step(False, tasks)
    torch.cuda.synchronize()
    u0, u1 = E(), E()
    u0.record(stream)
    for _ in range(task_steps):
        step(True, tasks)
    u1.record(stream)
    torch.cuda.synchronize()
    G.check(L.ckt_graph_check(g, sp))
    tasks_value = updates_per_step * task_steps / (u0.elapsed_time(u1) * 1e-3)
    kt_tasks = {k: [a.elapsed_time(b) * 1e-3 for a, b in kernel_events[k]]
                for k in ("cnc", "dc", "uv")}
    kernel_events["cnc"] = cnc_fused

    # Roofline of the dominant kernel (calc_new_currents, FP32-pipe bound).
    probe = fp32_peak(torch, G, stream)
    peak32 = probe["peak"]
    cnc_s = statistics.mean(kt["cnc"])
    cnc_flops = FLOPS_PER_WIRE_STEP * shape.W * INNER_STEPS
    peaks = measured_peaks()
    hbm = peaks.get("hbm_gbs")
    hbm_src = "measured (MEASURED_PEAKS.json)" if hbm else "fallback 6800 GB/s"
    hbm = hbm or 6800.0
    dc_bytes = 16 * shape.W + 8 * shape.N
    uv_bytes = 24 * shape.N
    # fused node pass: the two tasks' bytes (16 W + 8 N and 24 N) less the
    # charge written by one and read by the other (8 N)
    dcuv_bytes = 16 * shape.W + 24 * shape.N
    dc_s, uv_s = statistics.mean(kt_tasks["dc"]), statistics.mean(kt_tasks["uv"])
    dcuv_s = statistics.mean(kt["dcuv"])
    roofline = {
        "kernel": "calc_new_currents", "bound": "fp32", "unit": "TFLOP/s",
        "achieved": cnc_flops / cnc_s / 1e12, "peak": peak32 / 1e12,
        "frac": cnc_flops / cnc_s / peak32,
        "peak_source": "measured FP32 FMA throughput on this GPU (ckt_fp32_fma_probe, max of "
                       f"single {probe['single'] / 1e12:.1f} and paired f32x2 "
                       f"{probe['paired'] / 1e12:.1f} TFLOP/s)",
        "algorithmic": f"{FLOPS_PER_WIRE_STEP} flops per wire-step x {shape.W} wires x "
                       f"{INNER_STEPS} steps per launch",
        # ncu dram__bytes_read.sum + dram__bytes_write.sum of one launch over
        # 1,048,576 wires (103.9 + 21.3 MB), scaled by the wires: the traffic
        # is per wire (96 B read, up to 76 B written) and the same in every
        # mode, which load and store the same fields
        "traffic": CNC_TRAFFIC_PER_WIRE * shape.W,
        "traffic_unit": "bytes per launch",
        # The reference counts a division as one flop; a correctly rounded
        # fp32 quotient costs more than one FP32-pipe operation.  The issued
        # operations per wire-step give the pipe's own utilisation.
        "issued_fp32_ops_per_wire_step": FP32_OPS_PER_WIRE_STEP[mode],
        "pipe_frac": (FP32_OPS_PER_WIRE_STEP[mode] * shape.W * INNER_STEPS / cnc_s) /
                     (peak32 / 2),
    }
    # A device-to-device copy that moves the same bytes (half read, half
    # written), timed where the node pass runs -- right after
    # calc_new_currents, with its dirty lines in L2: what a memory-bound pass
    # of that size reaches on this GPU, fixed launch and ramp costs included.
    def same_bytes_copy(nbytes: int) -> float:
        src = torch.ones(nbytes // 2, dtype=torch.uint8, device=f"cuda:{local}")
        dst = torch.empty_like(src)
        ts = []
        for _ in range(3):
            with torch.cuda.stream(stream):
                G.check(L.ckt_calc_new_currents_all(g, w, n, ctypes.byref(prm), sp))
                a, b = E(), E()
                a.record(stream)
                dst.copy_(src)
                b.record(stream)
            torch.cuda.synchronize()
            ts.append(a.elapsed_time(b) * 1e-3)
        reset()
        torch.cuda.synchronize()
        return statistics.median(ts)

    copy_s = {k: same_bytes_copy(b) for k, b in
              (("dcuv", 16 * shape.W + 24 * shape.N), ("dc", 16 * shape.W + 8 * shape.N),
               ("uv", 24 * shape.N))}
    cnc_task_s = statistics.mean(kt_tasks["cnc"])
    kernels = {
        "calc_new_currents": {"ms": 1e3 * cnc_s, "tflops": cnc_flops / cnc_s / 1e12,
                              "frac_fp32_peak": cnc_flops / cnc_s / peak32},
        "distribute_update": {"ms": 1e3 * dcuv_s, "algo_bytes": dcuv_bytes,
                              "gbs": dcuv_bytes / dcuv_s / 1e9,
                              "frac_hbm": dcuv_bytes / dcuv_s / 1e9 / hbm,
                              "same_bytes_copy_ms": 1e3 * copy_s["dcuv"],
                              "frac_of_same_bytes_copy": copy_s["dcuv"] / dcuv_s,
                              "form": node_pass,
                              "note": "distribute_charge + update_voltages in one node pass"},
        "hbm_peak_gbs": hbm, "hbm_peak_source": hbm_src,
    }
    index_space_tasks = {
        "value": tasks_value, "unit": UNIT, "steps": task_steps,
        "note": "the three index-space task launches per loop (ckt_calc_new_currents_all, "
                "ckt_distribute_charge_all, ckt_update_voltages_all)",
        "calc_new_currents": {"ms": 1e3 * cnc_task_s,
                              "frac_fp32_peak": cnc_flops / cnc_task_s / peak32},
        "distribute_charge": {"ms": 1e3 * dc_s, "algo_bytes": dc_bytes,
                              "gbs": dc_bytes / dc_s / 1e9, "frac_hbm": dc_bytes / dc_s / 1e9 / hbm,
                              "same_bytes_copy_ms": 1e3 * copy_s["dc"],
                              "frac_of_same_bytes_copy": copy_s["dc"] / dc_s},
        "update_voltages": {"ms": 1e3 * uv_s, "algo_bytes": uv_bytes,
                            "gbs": uv_bytes / uv_s / 1e9, "frac_hbm": uv_bytes / uv_s / 1e9 / hbm,
                            "same_bytes_copy_ms": 1e3 * copy_s["uv"],
                            "frac_of_same_bytes_copy": copy_s["uv"] / uv_s},
    }

    # End to end through the same C-ABI calls with host buffers.
    h2d_keys = ("in_ptr", "out_ptr", "in_loc", "out_loc", "L", "R", "C", "current", "voltage",
                "charge", "node_voltage", "cap", "leak", "locator")
    pinned = {k: torch.from_numpy(np.ascontiguousarray(host[k])).pin_memory() for k in h2d_keys}
    out_pinned = {k: torch.empty_like(pinned[k]).pin_memory() for k in C.STATE_FIELDS}
    h2d = sum(v.numel() * v.element_size() for v in pinned.values())
    d2h = sum(v.numel() * v.element_size() for v in out_pinned.values())

    # Two device copies of the circuit, so that one step's upload and the
    # previous step's download overlap a step's loops: uploads on one copy
    # stream, downloads on another (the two directions use separate copy
    # engines), the loops on the compute stream.  Every step still copies
    # its whole circuit in and its state out.
    dc2 = C.DeviceCircuit(host, shape, device=f"cuda:{local}")
    bufs = [(dc, g, w, n), (dc2, dc2.graph.handle, dc2.wires(), dc2.nodes())]
    outs = [out_pinned, {k: torch.empty_like(v).pin_memory() for k, v in out_pinned.items()}]
    up, down = torch.cuda.Stream(), torch.cuda.Stream()
    freed = [None, None]  # event: buffer's last download done

    def e2e_step(i):
        b, gb, wb, nb = bufs[i % 2]
        with torch.cuda.stream(up):
            if freed[i % 2] is not None:
                up.wait_event(freed[i % 2])
            for k in h2d_keys:
                b.t[k].copy_(pinned[k], non_blocking=True)
            loaded = torch.cuda.Event()
            loaded.record(up)
        stream.wait_event(loaded)
        G.check(L.ckt_run_loops_all(gb, wb, nb, ctypes.byref(prm), OUTER_LOOPS, sp))
        done = torch.cuda.Event()
        done.record(stream)
        with torch.cuda.stream(down):
            down.wait_event(done)
            for k in C.STATE_FIELDS:
                outs[i % 2][k].copy_(b.t[k], non_blocking=True)
            freed[i % 2] = torch.cuda.Event()
            freed[i % 2].record(down)

    for i in range(args.warmup):
        e2e_step(i)
    torch.cuda.synchronize()
    barrier()
    e0, e1 = E(), E()
    w0 = time.perf_counter()
    e0.record(stream)
    up.wait_event(e0)
    for i in range(args.steps):
        e2e_step(args.warmup + i)
    stream.wait_stream(down)
    e1.record(stream)
    torch.cuda.synchronize()
    wall = time.perf_counter() - w0
    for b_ in bufs:
        G.check(L.ckt_graph_check(b_[1], sp))
    barrier()
    e2e_total, e2e_s, _ = replicas.aggregate(updates_per_step * args.steps,
                                             max(e0.elapsed_time(e1) * 1e-3, wall), device="cuda")
    e2e = {"value": e2e_total / e2e_s, "unit": UNIT,
           "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
           "note": "ckt_run_loops_all on host buffers: every step uploads the whole circuit from "
                   "pinned memory and downloads its state; two device copies let one step's "
                   "copies overlap the neighbouring step's loops.  The contribution graph and "
                   "node-tile plan (graph_device_bytes) are built once and stay resident, as "
                   "the reference's ELAPSED excludes load_circuit (circuit.cc:164-167)"}

    # The other configurations and forms, one GPU: heavy reduction (config
    # 2), the CPU-runnable shape (config 0), EXACT on a finite-regime state of
    # the config-1 circuit, FAST mode on config 1 with its error against the
    # reference's arithmetic, the batched mix (config 3) and the served
    # request stream (config 4).
    extras = {}
    if ws == 1 and not args.no_extras:
        peak32 = fp32_peak(torch, G, stream)["peak"]
        hbm_gbs = measured_peaks().get("hbm_gbs") or 6800.0
        s2 = C.Shape(128, 8192, 32768)
        h2 = C.generate(128, 8192, 32768, 50.0, SEED, L_OFFSET, L_SCALE)
        extras["config2"] = {
            "workload": "heavy reduction: 128 pieces x 8192 nodes x 32768 wires/piece "
                        "(4,194,304 wires), 50% in-piece, S=500 x 10 loops per step, seed 12345",
            **plain_measure(torch, G, C, h2, s2, mode, 500, 10, 3, 3, local, peak32, hbm_gbs),
            "accuracy": (accuracy_check(torch, G, C, mode, (128, 8192, 32768, 50.0), 500)
                         if not args.no_cpu_baseline else None)}
        del h2
        s0 = C.Shape(4, 256, 1024)
        h0 = C.generate(4, 256, 1024, PCT, SEED, L_OFFSET, L_SCALE)
        extras["config0"] = {
            "workload": "CPU-runnable shape: 4 pieces x 256 nodes x 1024 wires/piece, 95% "
                        "in-piece, S=1000 x 5 loops per step (4,096 wires: 8 blocks, the GPU "
                        "mostly idle)",
            **plain_measure(torch, G, C, h0, s0, mode, 1000, 5, 5, 3, local, peak32, hbm_gbs)}
        conv = {k: v.copy() for k, v in host.items()}
        rng = np.random.default_rng(1)
        conv["L"][:] = rng.uniform(1e-7, 9e-7, conv["L"].shape).astype(np.float32)
        for k, shp in (("current", conv["current"].shape), ("voltage", conv["voltage"].shape),
                       ("node_voltage", conv["node_voltage"].shape)):
            conv[k][:] = rng.uniform(-1, 1, shp).astype(np.float32)
        extras["finite_regime"] = {
            "workload": "the config-1 circuit with a convergent state (inductance U[1e-7, 9e-7), "
                        "currents and voltages U[-1, 1)), ONE outer loop of 1000 inner steps "
                        "per step: the recurrence contracts on all but a few wires (those "
                        "with the smallest capacitances), so nearly every operand is finite; "
                        "over further loops their NaN spreads through the node voltages",
            **plain_measure(torch, G, C, conv, shape, mode, INNER_STEPS, 1, 5, 3, local,
                            peak32, hbm_gbs, count_nonfinite=True)}
        del conv
        other = G.MODE_FAST if mode == G.MODE_EXACT else G.MODE_EXACT
        extras["fast_mode" if other == G.MODE_FAST else "exact_mode"] = {
            "mode": "fast" if other == G.MODE_FAST else "exact",
            **plain_measure(torch, G, C, host, shape, other, INNER_STEPS, OUTER_LOOPS, 3, 3, local,
                            peak32, hbm_gbs),
            "accuracy": (accuracy_check(torch, G, C, other, (SHAPE["num_pieces"],
                                                             SHAPE["nodes_per_piece"],
                                                             SHAPE["wires_per_piece"], PCT),
                                        INNER_STEPS)
                         if not args.no_cpu_baseline else None),
            "note": "FAST hoists L/dt, 1/R and dt/C and uses fused multiply-adds: not the "
                    "reference's rounding, so the stiff recurrence (gain L/(dt R) >> 1) "
                    "magnifies its one-ulp differences; see its accuracy block"}
        bres = batched_result(args, torch, G, ws, local, None, mode, 3, 3, piece_sync=False,
                              accuracy=not args.no_cpu_baseline)
        extras["batched"] = {k: bres[k] for k in ("value", "unit", "ms_per_step", "config",
                                                  "plain_sequential", "roofline", "accuracy",
                                                  "e2e", "clocks", "index_space_frac_fp32_peak")}
        sres = serve_result(args, torch, G, ws, local, mode,
                            [float(x) for x in args.extra_serve_rates.split(",") if x], 3.0, 12, 3,
                            accuracy=not args.no_cpu_baseline)
        extras["served"] = {k: sres[k] for k in ("value", "unit", "config", "latency_ms",
                                                 "latency_at_offered_rps",
                                                 "throughput_at_that_rate",
                                                 "capacity_offered_rps", "sweep",
                                                 "plain_sequential", "accuracy", "clocks")}

    if rank == 0:
        # the reference app's own report (apps/circuit/circuit.cc:314-333), per
        # simulation of OUTER_LOOPS loops, on stderr beside the JSON line
        sim_time = elapsed / args.steps
        ops = (shape.W * (10 * 6 + 9 * 4) * INNER_STEPS + shape.W * 4 + shape.N * 4) * OUTER_LOOPS
        print(f"ELAPSED TIME = {sim_time:7.3f} s", file=sys.stderr)
        print(f"GFLOPS = {1e-9 * ops / sim_time:7.3f} GFLOPS", file=sys.stderr)
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * elapsed / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (reference generator distributions, seed 12345)",
            "config": {**workload_config(args.mode, shape.num_pieces),
                       "graph_device_bytes": graph_bytes},
            "roofline": roofline,
            "cpu_baseline": cpu_baseline, "e2e": e2e, "gpu_launches": launches,
            "clocks": clk.summary(), "kernels": kernels, "index_space_tasks": index_space_tasks,
            "accuracy": accuracy,
            "replicas": "one independent circuit per GPU" if ws > 1 else None,
            **extras,
        }
        print(json.dumps(line), flush=True)
    if dist is not None:
        dist.destroy_process_group()


def run_batched(args, torch, G, ws, rank, local, dist, mode) -> None:
    line = batched_result(args, torch, G, ws, local, dist, mode, args.steps, args.warmup,
                          piece_sync=True, accuracy=ws == 1 and not args.no_cpu_baseline)
    if rank == 0:
        print(json.dumps(line), flush=True)
    if dist is not None:
        dist.destroy_process_group()


def batched_result(args, torch, G, ws, local, dist, mode, steps, warmup, piece_sync=True,
                   accuracy=True) -> dict:
    """Batched mixed sizes: 256 independent circuits (pieces U{1..32}, nodes
    per piece log-uniform [256, 16384], 4 wires per node, in-piece fraction
    U[0.8, 0.98], inner steps U{100..1000}, seeds 0..255, one outer loop).
    One step = reset the batch's state, then one persistent launch (CUDA
    graph replay) that runs every circuit's loop.  The plain path on the same
    circuits (circuit after circuit, three launches each) is timed beside it;
    piece_sync adds the reference-shaped per-piece synchronous calls."""
    from legionorigins_gb300.batch import Batch
    from legionorigins_gb300.workloads import mixed_batch

    specs = mixed_batch(args.circuits)
    t_build = time.perf_counter()
    b = Batch(specs, threads=cpu_threads())
    t_build = time.perf_counter() - t_build
    info = b.info()
    stream = torch.cuda.Stream()
    sp = stream.cuda_stream
    if getattr(args, "batch_launch", ""):
        b.set_config(*(int(x) for x in args.batch_launch.split(",")))
        cfg = b.config()
    else:
        cfg = b.autotune(mode, sp)
    updates = info["segment_updates_per_run"]
    E = lambda: torch.cuda.Event(enable_timing=True)  # noqa: E731

    def timed(fn, steps):
        events = []
        for _ in range(steps):
            G.check(G.lib().ckt_batch_reset_state(b.handle, sp))
            a, z = E(), E()
            a.record(stream)
            fn()
            z.record(stream)
            events.append((a, z))
        return events

    for _ in range(warmup):
        b.reset_state(sp)
        b.run(mode, sp)
    assert b.check(sp) == 0
    torch.cuda.synchronize()
    if dist is not None:
        dist.barrier()
    t0, t1 = E(), E()
    with Clocks(local) as clk:
        t0.record(stream)
        ev = timed(lambda: b.run(mode, sp), steps)
        t1.record(stream)
        torch.cuda.synchronize()
    if b.check(sp) != 0:
        raise SystemExit("persistent kernel reported a timeout")
    from legionorigins_gb300 import replicas

    if dist is not None:
        dist.barrier()
    total, elapsed, _ = replicas.aggregate(updates * steps, t0.elapsed_time(t1) * 1e-3,
                                           device="cuda")
    kern = [a.elapsed_time(z) * 1e-3 for a, z in ev]
    value = total / elapsed

    # The plain path on the same 256 circuits: circuit after circuit with
    # index-space launches, and piece by piece with a synchronisation after
    # every launch (the reference's task granularity).  Wall-clock timed.
    def plain(per_piece):
        b.reset_state(sp)
        b.run_sequential(mode, sp, per_piece)
        torch.cuda.synchronize()
        steps_ = max(1, min(steps, 3))
        w0 = time.perf_counter()
        for _ in range(steps_):
            G.check(G.lib().ckt_batch_reset_state(b.handle, sp))
            b.run_sequential(mode, sp, per_piece)
        torch.cuda.synchronize()
        return updates * steps_ / (time.perf_counter() - w0)

    seq = plain(False)
    seq_piece = plain(True) if piece_sync else None
    pieces_total = sum(s.num_pieces for s in specs)

    # End to end: every step copies the batch's state in from pinned host
    # memory, runs, and copies it back (topology and constants stay
    # resident).  Three instances of the batch let a step's upload and the
    # earlier steps' downloads (separate streams: separate copy engines)
    # overlap the launches: an instance is refilled only once its download
    # of three steps before has finished, so a slow host link delays no
    # launch as long as one upload plus one download fits in two launches.
    W, N = info["wires"], info["nodes"]
    hin = [torch.zeros(n, dtype=torch.float32).pin_memory() for n in (10 * W, 9 * W, N, N)]
    G.check(G.lib().ckt_batch_reset_state(b.handle, sp))
    G.check(G.lib().ckt_batch_download_state(b.handle, *[t.data_ptr() for t in hin], sp))
    n_inst = 3
    houts = [[torch.empty_like(t).pin_memory() for t in hin] for _ in range(n_inst)]
    torch.cuda.synchronize()
    h2d = sum(t.numel() * 4 for t in hin)
    extra = [Batch(specs, threads=cpu_threads()) for _ in range(n_inst - 1)]
    for bx in extra:
        bx.set_config(cfg["block"], cfg["wires_per_thread"], cfg["dc_schedule"])
    pair = [b] + extra
    up, down = torch.cuda.Stream(), torch.cuda.Stream()
    freed = [None] * n_inst

    def e2e_step(i):
        k = i % n_inst
        bb = pair[k]
        ev = [E() for _ in range(6)]  # upload, run, download: start and end
        with torch.cuda.stream(up):
            if freed[k] is not None:
                up.wait_event(freed[k])
            ev[0].record(up)
            G.check(G.lib().ckt_batch_upload_state(bb.handle, *[t.data_ptr() for t in hin],
                                                   up.cuda_stream))
            ev[1].record(up)
        stream.wait_event(ev[1])
        ev[2].record(stream)
        bb.run(mode, sp)
        ev[3].record(stream)
        with torch.cuda.stream(down):
            down.wait_event(ev[3])
            ev[4].record(down)
            G.check(G.lib().ckt_batch_download_state(
                bb.handle, *[t.data_ptr() for t in houts[k]], down.cuda_stream))
            ev[5].record(down)
            freed[k] = ev[5]
        e2e_events.append(ev)

    e2e_events = []
    e2e_warm = max(warmup, n_inst)  # every instance runs (and builds its graph) once
    for i in range(e2e_warm):
        e2e_step(i)
    torch.cuda.synchronize()
    e2e_events.clear()
    e0, e1 = E(), E()
    w0 = time.perf_counter()
    e0.record(stream)
    up.wait_event(e0)
    for i in range(steps):
        e2e_step(e2e_warm + i)
    stream.wait_stream(down)
    e1.record(stream)
    torch.cuda.synchronize()
    e2e_s = max(e0.elapsed_time(e1) * 1e-3, time.perf_counter() - w0)
    for bx in extra:
        bx.close()
    e2e_parts = {name: statistics.median(ev[2 * j].elapsed_time(ev[2 * j + 1])
                                         for ev in e2e_events)
                 for j, name in enumerate(("upload_ms", "run_ms", "download_ms"))}
    e2e_parts["step_ms"] = 1e3 * e2e_s / max(1, steps)
    e2e_parts["upload_gbs"] = h2d / e2e_parts["upload_ms"] / 1e6
    # when each of the first timed steps' copies and launch ran (ms from the
    # start of the timed region): shows where the pipeline waits
    e2e_parts["timeline_ms"] = [[round(e0.elapsed_time(x), 1) for x in ev]
                                for ev in e2e_events[:4]]

    probe = fp32_peak(torch, G, stream)
    flops = sum(FLOPS_PER_WIRE_STEP * s.wires * s.steps for s in specs)
    k_mean = statistics.mean(kern)
    if True:
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": steps,
            "warmup": warmup, "ms_per_step": 1e3 * elapsed / steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (reference generator distributions, seeds 0..255)",
            "config": {
                "workload": f"batched mixed sizes: {len(specs)} independent circuits, pieces U{{1..32}}, "
                            "nodes/piece log-uniform [256,16384], 4 wires/node, in-piece "
                            "U[0.8,0.98], inner steps U{100..1000}, 1 outer loop; one "
                            "persistent launch per step (CUDA graph)",
                "mode": args.mode, "circuits": len(specs), "wires": sum(s.wires for s in specs),
                "segment_updates_per_step": updates, "launch_shape": cfg,
                "l2": f"inputs larger than L2 ({19 * W * 4 / 1e9:.1f} GB of wire state)",
                "host_build_s": t_build,
            },
            "plain_sequential": {
                "index_space_per_circuit": {"value": seq, "unit": UNIT,
                                            "speedup_batched_over_it": value / seq,
                                            "launches_per_step": 4 * len(specs)},
                "per_piece_synchronous": {"value": seq_piece, "unit": UNIT,
                                          "speedup_batched_over_it": value / seq_piece,
                                          "launches_per_step": 2 * pieces_total + 2 * len(specs)}
                if seq_piece else None,
                "ceiling_note": "the plain kernel already runs near the FP32 pipe's limit, so "
                                "batching can only remove the plain path's idle time between "
                                "and within per-circuit launches: its ceiling over the "
                                "index-space path is (plain kernel's fraction of peak) / "
                                "(index-space path's fraction of peak)",
            },
            "roofline": {"kernel": "batch_kernel (persistent: calc_new_currents + "
                                   "distribute_charge + update_voltages)",
                         "bound": "fp32", "unit": "TFLOP/s", "achieved": flops / k_mean / 1e12,
                         "peak": probe["peak"] / 1e12, "frac": flops / k_mean / probe["peak"],
                         "traffic": None},
            "cpu_baseline": None,
            "accuracy": batch_accuracy_check(torch, mode, specs) if accuracy else None,
            "e2e": {"value": ws * updates * steps / e2e_s, "unit": UNIT,
                    "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": h2d,
                    "parts_median": e2e_parts,
                    "note": "circuit state in and out every step (topology resident); three "
                            "batch instances let a step's copies overlap its neighbours' "
                            "launches"},
            "gpu_launches": steps, "clocks": clk.summary(),
        }
    b.close()
    line["index_space_frac_fp32_peak"] = (flops / (updates / seq) / probe["peak"]
                                          if seq else None)
    return line


# Reduction microbenchmark (benchmarks/reductions/reducetest.cc): the
# configurations of the reference's published plot (asplos_plot.py:13-25),
# with 128 batches -- the benchmark's 8 batches per node at 16 nodes, its
# largest run -- and its published 16-node rates in M reductions/s.
RED_CONFIGS = {
    # name: (buckets, batch size, batches)
    "dense": (262144, 4194304, 128),
    "default": (1048576, 1048576, 128),
    "sparse": (4194304, 65536, 128),
    "any": (65536, 65536, 128),
}
RED_PUBLISHED_16_NODES = {  # asplos_plot.py:14-25, last column (16 nodes)
    ("dense", "redfold"): 1346.854, ("dense", "localize"): 13.435,
    ("dense", "redlist"): 168.342, ("sparse", "redfold"): 95.344,
    ("sparse", "localize"): 7.168, ("sparse", "redlist"): 109.948,
    ("any", "redsingle"): 1.624, ("any", "original"): 0.096,
}
RED_HEADLINE = ("dense", "redfold")
RED_METRIC = "histogram reductions/s (reducetest: dense 262144 buckets x 128 batches of 4194304)"


def red_launches(p, case: str, scratch: int) -> int:
    """Kernels one ckt_hist_run launches (mirrors ckt_reduce.cu's rounds)."""
    from legionorigins_gb300 import reductions as R

    total = p.batch_size * p.num_batches
    sched = R.CASES[case]
    if total == 0:
        return 0
    if sched == 0:
        return 1
    if sched == 1:
        return 1 if p.buckets <= 51200 else 2
    if sched == 3:
        per = max(1, min(p.num_batches, scratch // (8 * p.batch_size)))
        return 2 * -(-p.num_batches // per)
    per = min(((scratch - 65536) // 8) & ~3, total, 1 << 31)
    return 4 * -(-total // per)


def run_reductions(args, torch, G, ws, rank, local, dist) -> None:
    """Histogram reductions under each schedule (ckt_hist_run), timed with
    CUDA events per case, L2 flushed between timed runs (the histograms fit
    in L2; the inputs are hashed element indices, not arrays)."""
    from legionorigins_gb300 import reductions as R

    stream = torch.cuda.Stream()
    sp = stream.cuda_stream
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
    cases = ["redfold", "localize", "redlist", "redsingle"]
    sweep, launches, e2e = [], 0, None
    with Clocks(local) as clk:
        for name, (buckets, bsize, batches) in RED_CONFIGS.items():
            p = R.params(buckets, bsize, batches)
            h = R.Histogram(p, cases=cases)
            total = bsize * batches
            for case in cases:
                sched = R.CASES[case]
                with torch.cuda.stream(stream):
                    for _ in range(args.warmup):
                        h.run(sched, sp)
                    times = []
                    for _ in range(args.steps):
                        flush.fill_(1)
                        e0 = torch.cuda.Event(enable_timing=True)
                        e1 = torch.cuda.Event(enable_timing=True)
                        e0.record(stream)
                        h.run(sched, sp)
                        e1.record(stream)
                        e1.synchronize()
                        times.append(e0.elapsed_time(e1) * 1e-3)
                launches += args.steps * red_launches(p, case, h.scratch.numel())
                sec = statistics.median(times)
                pub = RED_PUBLISHED_16_NODES.get((name, case))
                sweep.append({"config": name, "buckets": buckets, "batch_size": bsize,
                              "batches": batches, "case": case, "seconds_median": sec,
                              "reductions_per_s": total / sec,
                              "reference_16_nodes_per_s": pub * 1e6 if pub else None})
            if name == RED_HEADLINE[0]:
                # end to end: the target histogram comes from pinned host
                # memory and goes back to it around every run
                host = torch.zeros(buckets, dtype=torch.int32).pin_memory()
                back = torch.empty_like(host).pin_memory()
                sched = R.CASES[RED_HEADLINE[1]]
                tt = []
                with torch.cuda.stream(stream):
                    for i in range(args.warmup + args.steps):
                        flush.fill_(1)
                        e0 = torch.cuda.Event(enable_timing=True)
                        e1 = torch.cuda.Event(enable_timing=True)
                        e0.record(stream)
                        h.hist.copy_(host, non_blocking=True)
                        h.run(sched, sp)
                        back.copy_(h.hist, non_blocking=True)
                        e1.record(stream)
                        e1.synchronize()
                        if i >= args.warmup:
                            tt.append(e0.elapsed_time(e1) * 1e-3)
                launches += args.steps * red_launches(p, RED_HEADLINE[1], h.scratch.numel())
                e2e = {"value": total / statistics.median(tt), "unit": "reductions/s",
                       "h2d_bytes_per_step": 4 * buckets, "d2h_bytes_per_step": 4 * buckets}
            del h
    head = next(r for r in sweep if (r["config"], r["case"]) == RED_HEADLINE)
    cpu = None
    if rank == 0 and ws == 1 and not args.no_cpu_baseline:
        cpu = red_cpu_baseline(args)
    if rank == 0:
        buckets, bsize, batches = RED_CONFIGS[RED_HEADLINE[0]]
        line = {
            "metric": RED_METRIC, "value": head["reductions_per_s"], "unit": "reductions/s",
            "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": 1e3 * head["seconds_median"], "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "u32",
            "data": "synthetic (the benchmark's own hash of the element index, seeds 12345/54321)",
            "config": {"workload": "reducetest dense: 262144 buckets, 128 batches x 4194304, "
                                   "redfold schedule; sweep over the plot's configurations",
                       "buckets": buckets, "batch_size": bsize, "batches": batches,
                       "l2": "flushed (256 MB write) before every timed run"},
            "sweep": sweep, "cpu_baseline": cpu, "e2e": e2e, "gpu_launches": launches,
            "clocks": clk.summary(),
            "reference_published": "benchmarks/reductions/asplos_plot.py:14-25 (Keeneland, "
                                   "16 nodes), per sweep row",
        }
        print(json.dumps(line), flush=True)
    if dist is not None:
        dist.destroy_process_group()


def red_cpu_baseline(args) -> dict:
    """The oracle's histogram on every host core in the benchmark's fastest
    CPU schedule (redfold), on a bounded sample of the dense configuration."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import ckt_oracle as O

    O.build()
    threads = cpu_threads()
    buckets, bsize, batches = RED_CONFIGS[RED_HEADLINE[0]]
    _, t = O.histogram_threads(buckets, bsize // 16, threads, threads)  # calibrate
    per_batch = t  # one round of `threads` batches of bsize/16
    n = max(threads, min(batches, int(args.cpu_sample_s / max(per_batch * 16, 1e-9)) * threads))
    _, secs = O.histogram_threads(buckets, bsize, n, threads)
    return {"value": n * bsize / secs, "unit": "reductions/s", "cores": threads, "kind": "port",
            "sample": f"{n} of {batches} batches of {bsize} ({buckets} buckets), "
                      f"oracle/ckt_oracle.c redfold on {threads} threads"}


def run_generate(args, torch, G, ws, rank, local, dist) -> None:
    """Building one config-1 circuit (64 x 16384 x 65536, 4,194,304 wires):
    the reference generator and graph on the host (ckt_generate +
    ckt_graph_create, which a host-built request pays before upload) against
    ckt_generate_device, which leaves the same arrays and graph on the GPU."""
    from legionorigins_gb300 import DeviceCircuitArrays, GenParams
    from legionorigins_gb300 import circuit as C

    P, npp, wpp = SHAPE["num_pieces"], SHAPE["nodes_per_piece"], SHAPE["wires_per_piece"]
    W, N = P * wpp, P * npp
    t = time.perf_counter()
    host = C.generate(P, npp, wpp, PCT, SEED, L_OFFSET, L_SCALE)
    t_gen = time.perf_counter() - t
    t = time.perf_counter()
    g = C.Graph(C.Shape(P, npp, wpp).pieces(), N, host["in_ptr"], host["out_ptr"], host["in_loc"],
                host["out_loc"])
    t_graph = time.perf_counter() - t
    g.close()
    dev = {
        "in_ptr": (W, torch.int32), "out_ptr": (W, torch.int32), "in_loc": (W, torch.uint8),
        "out_loc": (W, torch.uint8), "inductance": (W, torch.float32),
        "resistance": (W, torch.float32), "capacitance": (W, torch.float32),
        "current": (10 * W, torch.float32), "voltage": (9 * W, torch.float32),
        "charge": (N, torch.float32), "node_voltage": (N, torch.float32),
        "node_capacitance": (N, torch.float32), "node_leakage": (N, torch.float32),
        "locator": (N, torch.int32), "off": (N + 1, torch.int32), "ent": (2 * W, torch.int32),
        "slot_in": (W, torch.int32), "slot_out": (W, torch.int32),
        "gstart": ((2 * W + 31) // 32, torch.int32)}
    d = {k: torch.empty(n, dtype=t_, device="cuda") for k, (n, t_) in dev.items()}
    arr = DeviceCircuitArrays(*[d[k].data_ptr() for k, _ in DeviceCircuitArrays._fields_])
    gp = GenParams(P, npp, wpp, 0, PCT, SEED, L_OFFSET, L_SCALE)
    stream = torch.cuda.Stream()
    sp = stream.cuda_stream
    for _ in range(args.warmup):
        G.check(G.lib().ckt_generate_device(ctypes.byref(gp), ctypes.byref(arr), sp))
    torch.cuda.synchronize()
    ts = []
    with Clocks(local) as clk:
        for _ in range(args.steps):
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            G.check(G.lib().ckt_generate_device(ctypes.byref(gp), ctypes.byref(arr), sp))
            b.record(stream)
            b.synchronize()
            ts.append(a.elapsed_time(b) * 1e-3)
    same = all(np.array_equal(d[k].cpu().numpy().view(host[h].dtype), host[h])
               for k, h in (("in_ptr", "in_ptr"), ("out_ptr", "out_ptr"), ("inductance", "L")))
    dev_s = statistics.median(ts)
    if rank == 0:
        print(json.dumps({
            "metric": "circuit build time, 4,194,304-wire config-1 circuit with its graph",
            "value": 1e3 * dev_s, "unit": "ms", "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * dev_s, "higher_is_better": False,
            "scaling": "weak", "vs_baseline": None, "dtype": "u32/f32",
            "data": "synthetic (the reference generator, seed 12345)",
            "config": {"workload": "ckt_generate_device: generator + node CSR on the GPU",
                       "wires": W, "nodes": N},
            "host_ms": {"generate": 1e3 * t_gen, "graph": 1e3 * t_graph,
                        "threads": "library default"},
            "speedup_over_host": (t_gen + t_graph) / dev_s, "matches_host_sample": same,
            "gpu_launches": None, "clocks": clk.summary()}), flush=True)


def run_layout(args, torch, G, ws, rank, local, dist) -> None:
    """AoS <-> SoA conversion of a config-1 circuit's wires (4,194,304 x 128-byte
    CircuitWire): from device memory, and from pinned host memory mapped for
    the device (zero-copy over NVLink-C2C)."""
    from legionorigins_gb300 import circuit as C

    P, npp, wpp = SHAPE["num_pieces"], SHAPE["nodes_per_piece"], SHAPE["wires_per_piece"]
    shape = C.Shape(P, npp, wpp)
    host = C.generate(P, npp, wpp, PCT, SEED, L_OFFSET, L_SCALE)
    dc = C.DeviceCircuit(host, shape, device="cuda")
    W = shape.W
    aos_dev = torch.zeros(128 * W, dtype=torch.uint8, device="cuda")
    aos_host = torch.zeros(128 * W, dtype=torch.uint8).pin_memory()
    stream = torch.cuda.Stream()
    sp = stream.cuda_stream
    soa_bytes = 98 * W  # in/out 8, locations 2, L/R/C 12, current 40, voltage 36
    L = G.lib()
    cases = {
        "to_aos_device": lambda: L.ckt_wires_to_aos(dc.wires(), W, aos_dev.data_ptr(), sp),
        "from_aos_device": lambda: L.ckt_wires_from_aos(aos_dev.data_ptr(), W, dc.wires(), sp),
        "to_aos_host_mapped": lambda: L.ckt_wires_to_aos(dc.wires(), W, aos_host.data_ptr(), sp),
        "from_aos_host_mapped": lambda: L.ckt_wires_from_aos(aos_host.data_ptr(), W, dc.wires(),
                                                             sp),
    }
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
    out = {}
    peaks = measured_peaks()
    hbm = peaks.get("hbm_gbs") or 6800.0
    with Clocks(local) as clk:
        for name, fn in cases.items():
            with torch.cuda.stream(stream):
                for _ in range(args.warmup):
                    G.check(fn())
                ts = []
                for _ in range(args.steps):
                    flush.fill_(1)
                    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                    a.record(stream)
                    G.check(fn())
                    b.record(stream)
                    b.synchronize()
                    ts.append(a.elapsed_time(b) * 1e-3)
            sec = statistics.median(ts)
            out[name] = {"ms": 1e3 * sec, "gbs": (128 * W + soa_bytes) / sec / 1e9,
                         "frac_hbm": (128 * W + soa_bytes) / sec / 1e9 / hbm}
    torch.cuda.synchronize()
    if rank == 0:
        head = out["from_aos_device"]
        print(json.dumps({
            "metric": "AoS -> SoA wire conversion bandwidth, 4,194,304 CircuitWire (128 B)",
            "value": head["gbs"], "unit": "GB/s", "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": head["ms"], "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "u32/f32",
            "data": "synthetic (the reference generator, seed 12345)",
            "config": {"workload": "ckt_wires_from_aos / ckt_wires_to_aos on the config-1 wires",
                       "bytes_per_call": 128 * W + soa_bytes,
                       "l2": "flushed (256 MB write) before every timed call"},
            "cases": out, "hbm_peak_gbs": hbm, "gpu_launches": 4 * args.steps,
            "clocks": clk.summary()}), flush=True)


def run_serve(args, torch, G, ws, rank, local, dist, mode) -> None:
    rates = [float(x) for x in args.rates.split(",") if x]
    line = serve_result(args, torch, G, ws, local, mode, rates, args.serve_seconds,
                        args.serve_plain_sample, args.warmup,
                        accuracy=ws == 1 and not args.no_cpu_baseline)
    if rank == 0:
        print(json.dumps(line), flush=True)
    if dist is not None:
        dist.destroy_process_group()


def serve_result(args, torch, G, ws, local, mode, rates, seconds, plain_sample, warmup,
                 accuracy=True) -> dict:
    """Serving loop: circuit-solve requests arrive as a Poisson stream at each
    offered rate; per request, total wires log-uniform in [1e3, 4e6], 4 wires
    per node, 8..64 pieces, 95% in-piece, inner steps U{100..1000}, 1..5 outer
    loops, seed = request id; admission under an 80 GB HBM budget.  Reports
    throughput (wire-segment updates of completed requests over the span from
    first arrival to last completion) and p50/p99 latency (completion minus
    arrival) per rate."""
    import random

    from legionorigins_gb300.serve import Server
    from legionorigins_gb300.workloads import serve_request

    sweep = []
    next_id = 0
    warm = Server(mode=mode, prep_threads=cpu_threads())
    for i in range(warmup):
        warm.submit(i, serve_request(10_000_000 + i))
    warm.wait(120.0)
    warm.close()
    clk_all = []
    for rate in rates:
        launch = tuple(int(x) for x in args.serve_launch.split(",")) if args.serve_launch else None
        srv = Server(mode=mode, prep_threads=cpu_threads(), hbm_budget_bytes=80 << 30,
                     launch=launch)
        rng = random.Random(int(rate * 1000) + 7)
        t = 0.0
        arrivals = []
        while t < seconds:
            t += rng.expovariate(rate)
            arrivals.append(t)
        with Clocks(local) as clk:
            t0 = time.perf_counter()
            base = srv.clock()
            for a in arrivals:
                d = a - (time.perf_counter() - t0)
                if d > 0:
                    time.sleep(d)
                srv.submit(next_id, serve_request(next_id))
                next_id += 1
            rc = srv.wait(600.0)
        clk_all.append(clk.summary())
        done = srv.poll(len(arrivals) + 16)
        st = srv.stats()
        srv.close()
        ok = [c for c in done if c["status"] == 0]
        lat = sorted(c["finish_s"] - c["submit_s"] for c in ok)
        span = max(c["finish_s"] for c in ok) - min(c["submit_s"] for c in ok) if ok else 0.0
        upd = sum(c["segment_updates"] for c in ok)
        pct = lambda q: lat[min(len(lat) - 1, int(q * len(lat)))] if lat else None  # noqa: E731
        sweep.append({
            "offered_rps": rate, "submitted": len(arrivals), "completed_ok": len(ok),
            "failed": len(done) - len(ok), "wait_rc": rc,
            "throughput": upd / span if span > 0 else 0.0,
            "completed_rps": len(ok) / span if span > 0 else 0.0,
            "latency_ms": {"p50": 1e3 * pct(0.50), "p99": 1e3 * pct(0.99),
                           "max": 1e3 * lat[-1]} if lat else None,
            "queue_to_start_ms_p50": 1e3 * sorted(c["start_s"] - c["submit_s"] for c in ok)[len(ok) // 2] if ok else None,
            "rounds": st["rounds"], "resident_peak": st["resident_peak"],
            "hbm_peak_gb": st["bytes_peak"] / 1e9, "gpu_busy_s": st["busy_s"],
        })
    # The same request stream through the plain path, one request at a time
    # (circuit already resident, only its loops timed): index-space launches,
    # and the reference's per-piece task calls with a device wait after each.
    from legionorigins_gb300 import circuit as C

    plain = {"index_space": [0, 0.0], "per_piece_blocking": [0, 0.0]}
    stream = torch.cuda.Stream()
    sp = stream.cuda_stream
    for rid in range(plain_sample):
        spec = serve_request(rid)
        host = C.generate(*spec.gen_args())
        shape = C.Shape(spec.num_pieces, spec.nodes_per_piece, spec.wires_per_piece)
        dc = C.DeviceCircuit(host, shape)
        prm = C.params(spec.steps, mode)
        torch.cuda.synchronize()
        for name, acc in plain.items():
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            for _ in range(spec.loops):
                if name == "index_space":
                    dc.loop_index_space(prm, sp)
                else:
                    dc.loop_per_piece(prm, sp, blocking=True)
            b.record(stream)
            b.synchronize()
            acc[0] += spec.segment_updates  # wires x 10 x steps x loops
            acc[1] += a.elapsed_time(b) * 1e-3
        dc.close()
        del dc
    plain_rates = {k: (v[0] / v[1] if v[1] > 0 else None) for k, v in plain.items()}
    best = max(sweep, key=lambda r: r["throughput"])
    # latency is quoted at the highest offered rate the server keeps up with
    # (completes >= 95% of the offered rate); above it queueing dominates
    kept = [r for r in sweep if r["completed_rps"] >= 0.95 * r["offered_rps"]]
    quiet = max(kept, key=lambda r: r["offered_rps"]) if kept else min(sweep, key=lambda r: r["offered_rps"])
    if True:
        line = {
            "metric": METRIC, "value": best["throughput"], "unit": UNIT, "n_gpus": ws,
            "steps": len(rates), "warmup": warmup,
            "ms_per_step": None, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32",
            "data": "synthetic request stream (reference generator, seed = request id)",
            "config": {
                "workload": "serving loop: Poisson arrivals, total wires log-uniform [1e3,4e6], "
                            "4 wires/node, 8..64 pieces, 95% in-piece, inner steps U{100..1000}, "
                            "outer loops U{1..5}, 80 GB HBM admission budget, continuous "
                            "batching (one persistent launch per round)",
                "mode": args.mode, "seconds_of_arrivals_per_rate": seconds,
                "rates_rps": rates, "launch": args.serve_launch or "library default",
            },
            "latency_ms": quiet["latency_ms"], "latency_at_offered_rps": quiet["offered_rps"],
            "throughput_at_that_rate": quiet["throughput"],
            # the rounds run the batched kernel: its accuracy on the stream's
            # first requests of at most 300,000 wires
            "accuracy": (batch_accuracy_check(
                torch, mode, [r for r in (serve_request(i) for i in range(200))
                              if r.wires <= 300_000][:8]) if accuracy else None),
            "capacity_offered_rps": best["offered_rps"], "sweep": sweep,
            "plain_sequential": {
                "requests": plain_sample,
                **{k: {"value": v, "unit": UNIT,
                       "served_over_it": (best["throughput"] / v) if v else None}
                   for k, v in plain_rates.items()},
                "note": "requests 0..n-1 of the stream, one at a time, circuit resident, "
                        "only their loops timed (device events): the plain path's best case",
            },
            "e2e": {"value": best["throughput"], "unit": UNIT, "h2d_bytes_per_step": None,
                    "d2h_bytes_per_step": None,
                    "note": "serving is end to end by construction: each request is submitted "
                            "from the host, its circuit is built on the GPU (or on the host and "
                            "uploaded), and its final state is read back to host memory"},
            "clocks": clk_all[-1] if clk_all else None,
        }
    return line


if __name__ == "__main__":
    main()
