"""numpy front end for the C oracle (oracle/ckt_oracle.c) and the reference
pin binary (oracle/_ref/circuit_ref).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and
bench.py's CPU-baseline leg, never by the product package.

The oracle restates the reference circuit application's generator and leaf
tasks (LegionOrigins apps/circuit/circuit.cc:352-460, 1071-1307 and
apps/circuit/circuit_gpu.cu:61-149) and the reduction microbenchmark's
histogram (benchmarks/reductions/reducetest.cc:174, 323-347); ckt_oracle.h
lists the file:line each function follows.  Its parity is pinned by
tests/test_oracle_pin.py against the reference's own circuit.cc and
reducetest.cc, compiled through oracle/refshim and oracle/refshim_lowlevel.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
from dataclasses import dataclass, field

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libckt_oracle.so")
REF_BIN = os.path.join(HERE, "_ref", "circuit_ref")
REDUCE_REF_BIN = os.path.join(HERE, "_ref", "reducetest_ref")
SEGMENTS = 10
PRIVATE, SHARED, GHOST = 0, 1, 2


class _Params(ctypes.Structure):
    _fields_ = [
        ("num_pieces", ctypes.c_int32),
        ("nodes_per_piece", ctypes.c_int32),
        ("wires_per_piece", ctypes.c_int32),
        ("pad0", ctypes.c_int32),
        ("pct_wire_in_piece", ctypes.c_double),
        ("random_seed", ctypes.c_int64),
        ("L_offset", ctypes.c_double),
        ("L_scale", ctypes.c_double),
    ]


def build(force: bool = False) -> str:
    """Compile the oracle library with its Makefile (gcc, seconds)."""
    if force or not os.path.exists(LIB_PATH) or (
        os.path.getmtime(LIB_PATH) < os.path.getmtime(os.path.join(HERE, "ckt_oracle.c"))
    ):
        subprocess.run(["make", "-s", "-C", HERE, "_build/libckt_oracle.so"], check=True)
    return LIB_PATH


STAGED_REFERENCE = os.path.join(os.path.dirname(HERE), "baseline", "_ref", "LegionOrigins")


def build_ref(reference: str | None = None) -> str | None:
    """Compile the reference's circuit.cc (and reducetest.cc) through the
    shim: from the reference tree when it is present (and stage the files
    those builds read into the git-ignored baseline/_ref/LegionOrigins), else
    from that staged copy; None when neither exists."""
    if reference and os.path.isdir(os.path.join(reference, "apps", "circuit")):
        subprocess.run(["make", "-s", "-C", HERE, "stage", f"REFERENCE={reference}",
                        f"STAGE={STAGED_REFERENCE}"], check=True)
    elif os.path.isdir(os.path.join(STAGED_REFERENCE, "apps", "circuit")):
        reference = STAGED_REFERENCE
    else:
        return None
    subprocess.run(["make", "-s", "-C", HERE, "ref", f"REFERENCE={reference}"], check=True)
    return REF_BIN


def time_reference(p: "GenParams", loops: int = 1) -> float:
    """ELAPSED TIME of the reference's own circuit.cc main loop
    (apps/circuit/circuit.cc:311-318: `loops` outer loops of STEPS = 10000
    inner steps, its CPU tasks, single-threaded through the shim), seconds."""
    if not os.path.exists(REF_BIN):
        raise FileNotFoundError(REF_BIN)
    if p.L_offset != 0.1 or p.L_scale != 0.01:
        raise ValueError("the reference hard-codes L = drand48()*0.01 + 0.1")
    args = [REF_BIN, "-l", str(loops), "-p", str(p.num_pieces), "-npp", str(p.nodes_per_piece),
            "-wpp", str(p.wires_per_piece), "-pct", str(int(p.pct_wire_in_piece)),
            "-s", str(p.random_seed)]
    out = subprocess.run(args, check=True, capture_output=True, text=True).stdout
    for line in out.splitlines():
        if line.startswith("ELAPSED TIME"):
            return float(line.split("=")[1].split()[0])
    raise RuntimeError("the reference printed no ELAPSED TIME")


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(LIB_PATH)
        P = ctypes.c_void_p
        L.ocl_generate.argtypes = [ctypes.POINTER(_Params)] + [P] * 12
        L.ocl_generate.restype = ctypes.c_int
        i64, i32 = ctypes.c_int64, ctypes.c_int32
        L.ocl_cnc_f32.argtypes = [i64, i64, i64, P, P, P, P, P, P, P, P, i32, i32]
        L.ocl_cnc_f64.argtypes = [i64, i64, i64, P, P, P, P, P, P, P, P, i32, i32]
        L.ocl_dc_f32.argtypes = [i32, P, P, i64, P, P, P, P, P, P, i64, P]
        L.ocl_dc_f64.argtypes = [i32, P, P, i64, P, P, P, P, P, P, i64, P]
        L.ocl_uv_f32.argtypes = [i64, i64, P, P, P, P]
        L.ocl_uv_f64.argtypes = [i64, i64, P, P, P, P]
        L.ocl_simulate_f32.argtypes = [ctypes.POINTER(_Params), i32, i32, i32] + [P] * 13
        L.ocl_simulate_f64.argtypes = [ctypes.POINTER(_Params), i32, i32, i32] + [P] * 13
        L.ocl_baseline_run.argtypes = [ctypes.POINTER(_Params), i32, i32, i32, i32, i32] + [P] * 13
        L.ocl_baseline_run.restype = ctypes.c_double
        u32, u64 = ctypes.c_uint32, ctypes.c_uint64
        L.ocl_hist_rand.argtypes = [u64, u32, u32]
        L.ocl_hist_rand.restype = u32
        L.ocl_histogram.argtypes = [u32] * 6 + [P]
        L.ocl_histogram.restype = None
        L.ocl_histogram_threads.argtypes = [u32] * 6 + [i32, P]
        L.ocl_histogram_threads.restype = ctypes.c_double
        f32 = ctypes.c_float
        L.ocl_split_quotient_check.argtypes = [u64, u64, f32, f32, f32, f32, P, P]
        L.ocl_split_quotient_check.restype = None
        L.ocl_wide_quotient_check.argtypes = [u64, u64, i32, P, P, P]
        L.ocl_wide_quotient_check.restype = None
        _lib = L
    return _lib


def _p(a: np.ndarray):
    assert a.flags["C_CONTIGUOUS"]
    return a.ctypes.data_as(ctypes.c_void_p)


@dataclass
class GenParams:
    """Generator parameters (the reference CLI's -p -npp -wpp -pct -s plus the
    inductance range, which the reference hard-codes at circuit.cc:1163)."""

    num_pieces: int
    nodes_per_piece: int
    wires_per_piece: int
    pct_wire_in_piece: float = 95.0
    random_seed: int = 12345
    L_offset: float = 0.1
    L_scale: float = 0.01

    @property
    def W(self) -> int:
        return self.num_pieces * self.wires_per_piece

    @property
    def N(self) -> int:
        return self.num_pieces * self.nodes_per_piece

    def c(self) -> _Params:
        return _Params(self.num_pieces, self.nodes_per_piece, self.wires_per_piece, 0,
                       float(self.pct_wire_in_piece), int(self.random_seed),
                       float(self.L_offset), float(self.L_scale))


@dataclass
class Circuit:
    """A circuit in structure-of-arrays form.  current is [10, W] and voltage
    [9, W] (segment-major); node arrays are [N]."""

    params: GenParams
    in_ptr: np.ndarray
    out_ptr: np.ndarray
    in_loc: np.ndarray
    out_loc: np.ndarray
    L: np.ndarray
    R: np.ndarray
    C: np.ndarray
    current: np.ndarray
    voltage: np.ndarray
    charge: np.ndarray
    node_voltage: np.ndarray
    cap: np.ndarray
    leak: np.ndarray
    locator: np.ndarray
    extra: dict = field(default_factory=dict)

    def copy(self) -> "Circuit":
        kw = {k: (v.copy() if isinstance(v, np.ndarray) else v) for k, v in self.__dict__.items()}
        return Circuit(**kw)

    def astype(self, dt) -> "Circuit":
        c = self.copy()
        for k in ("L", "R", "C", "current", "voltage", "charge", "node_voltage", "cap", "leak"):
            setattr(c, k, np.ascontiguousarray(getattr(c, k).astype(dt)))
        return c


def generate(p: GenParams) -> Circuit:
    W, N = p.W, p.N
    c = Circuit(
        params=p,
        in_ptr=np.zeros(W, np.uint32), out_ptr=np.zeros(W, np.uint32),
        in_loc=np.zeros(W, np.uint8), out_loc=np.zeros(W, np.uint8),
        L=np.zeros(W, np.float32), R=np.zeros(W, np.float32), C=np.zeros(W, np.float32),
        current=np.zeros((SEGMENTS, W), np.float32),
        voltage=np.zeros((SEGMENTS - 1, W), np.float32),
        charge=np.zeros(N, np.float32), node_voltage=np.zeros(N, np.float32),
        cap=np.zeros(N, np.float32), leak=np.zeros(N, np.float32),
        locator=np.zeros(N, np.int32),
    )
    pc = p.c()
    rc = lib().ocl_generate(ctypes.byref(pc), _p(c.in_ptr), _p(c.out_ptr), _p(c.in_loc),
                            _p(c.out_loc), _p(c.L), _p(c.R), _p(c.C), _p(c.charge),
                            _p(c.node_voltage), _p(c.cap), _p(c.leak), _p(c.locator))
    if rc != 0:
        raise ValueError(f"ocl_generate failed ({rc})")
    return c


def _fn(name: str, dtype):
    return getattr(lib(), name + ("_f64" if np.dtype(dtype) == np.float64 else "_f32"))


def calc_new_currents(c: Circuit, steps: int, quirk: bool = False,
                      w_begin: int = 0, w_end: int | None = None) -> None:
    W = c.params.W
    w_end = W if w_end is None else w_end
    _fn("ocl_cnc", c.L.dtype)(w_begin, w_end, W, _p(c.in_ptr), _p(c.out_ptr), _p(c.L), _p(c.R),
                              _p(c.C), _p(c.current), _p(c.voltage), _p(c.node_voltage),
                              int(steps), int(quirk))


def distribute_charge(c: Circuit) -> None:
    p = c.params
    fw = np.arange(p.num_pieces, dtype=np.int64) * p.wires_per_piece
    nw = np.full(p.num_pieces, p.wires_per_piece, np.int64)
    scratch = np.zeros(p.N, c.charge.dtype)
    _fn("ocl_dc", c.charge.dtype)(p.num_pieces, _p(fw), _p(nw), p.W, _p(c.in_ptr),
                                  _p(c.out_ptr), _p(c.in_loc), _p(c.out_loc), _p(c.current),
                                  _p(c.charge), p.N, _p(scratch))


def update_voltages(c: Circuit) -> None:
    _fn("ocl_uv", c.charge.dtype)(0, c.params.N, _p(c.charge), _p(c.node_voltage), _p(c.cap),
                                  _p(c.leak))


def simulate(c: Circuit, loops: int, steps: int, quirk: bool = False) -> None:
    pc = c.params.c()
    _fn("ocl_simulate", c.L.dtype)(ctypes.byref(pc), int(loops), int(steps), int(quirk),
                                   _p(c.in_ptr), _p(c.out_ptr), _p(c.in_loc), _p(c.out_loc),
                                   _p(c.L), _p(c.R), _p(c.C), _p(c.current), _p(c.voltage),
                                   _p(c.charge), _p(c.node_voltage), _p(c.cap), _p(c.leak))


def baseline_run(c: Circuit, loops: int, steps: int, threads: int, piece_limit: int = 0,
                 quirk: bool = False) -> float:
    """Multithreaded CPU baseline (fp32, in place).  Returns main-loop seconds."""
    pc = c.params.c()
    t = lib().ocl_baseline_run(ctypes.byref(pc), int(loops), int(steps), int(threads),
                               int(piece_limit), int(quirk), _p(c.in_ptr), _p(c.out_ptr),
                               _p(c.in_loc), _p(c.out_loc), _p(c.L), _p(c.R), _p(c.C),
                               _p(c.current), _p(c.voltage), _p(c.charge), _p(c.node_voltage),
                               _p(c.cap), _p(c.leak))
    if t < 0:
        raise MemoryError("ocl_baseline_run failed")
    return t


# --------------------------------------------------------------------------
# Reference pin: the reference's circuit.cc run through oracle/refshim
# --------------------------------------------------------------------------

# apps/circuit/circuit.h:35-54 in numpy form.
NODE_DTYPE = np.dtype([("charge", "<f4"), ("voltage", "<f4"), ("capacitance", "<f4"),
                       ("leakage", "<f4")])
WIRE_DTYPE = np.dtype([("in_ptr", "<u4"), ("out_ptr", "<u4"), ("in_loc", "<i4"),
                       ("out_loc", "<i4"), ("inductance", "<f4"), ("resistance", "<f4"),
                       ("current", "<f4", (10,)), ("capacitance", "<f4"),
                       ("voltage", "<f4", (9,)), ("pad", "<f4", (6,))])
assert NODE_DTYPE.itemsize == 16 and WIRE_DTYPE.itemsize == 128


def circuit_from_aos(p: GenParams, nodes: np.ndarray, wires: np.ndarray,
                     locator: np.ndarray) -> Circuit:
    return Circuit(
        params=p,
        in_ptr=np.ascontiguousarray(wires["in_ptr"]), out_ptr=np.ascontiguousarray(wires["out_ptr"]),
        in_loc=np.ascontiguousarray(wires["in_loc"].astype(np.uint8)),
        out_loc=np.ascontiguousarray(wires["out_loc"].astype(np.uint8)),
        L=np.ascontiguousarray(wires["inductance"]), R=np.ascontiguousarray(wires["resistance"]),
        C=np.ascontiguousarray(wires["capacitance"]),
        current=np.ascontiguousarray(wires["current"].T),
        voltage=np.ascontiguousarray(wires["voltage"].T),
        charge=np.ascontiguousarray(nodes["charge"]),
        node_voltage=np.ascontiguousarray(nodes["voltage"]),
        cap=np.ascontiguousarray(nodes["capacitance"]), leak=np.ascontiguousarray(nodes["leakage"]),
        locator=np.ascontiguousarray(locator.astype(np.int32)),
    )


def circuit_to_aos(c: Circuit):
    nodes = np.zeros(c.params.N, NODE_DTYPE)
    nodes["charge"], nodes["voltage"] = c.charge, c.node_voltage
    nodes["capacitance"], nodes["leakage"] = c.cap, c.leak
    wires = np.zeros(c.params.W, WIRE_DTYPE)
    wires["in_ptr"], wires["out_ptr"] = c.in_ptr, c.out_ptr
    wires["in_loc"], wires["out_loc"] = c.in_loc, c.out_loc
    wires["inductance"], wires["resistance"], wires["capacitance"] = c.L, c.R, c.C
    wires["current"], wires["voltage"] = c.current.T, c.voltage.T
    return nodes, wires


def run_reference(p: GenParams, loops: int, workdir: str, override: Circuit | None = None):
    """Run the reference's circuit.cc (inner steps fixed at its STEPS=10000)
    and return (initial circuit, final circuit) as the reference produced
    them.  `override` replaces the wire and node state after load_circuit
    (the graph must be the generator's own)."""
    if not os.path.exists(REF_BIN):
        raise FileNotFoundError(REF_BIN)
    os.makedirs(workdir, exist_ok=True)
    pre = os.path.join(workdir, "ref")
    env = dict(os.environ, CKT_REFSHIM_DUMP=pre)
    if override is not None:
        nodes, wires = circuit_to_aos(override)
        nodes.tofile(pre + ".ovr.r0.bin")
        wires.tofile(pre + ".ovr.r1.bin")
        env["CKT_REFSHIM_OVERRIDE"] = pre + ".ovr"
    if p.L_offset != 0.1 or p.L_scale != 0.01:
        raise ValueError("the reference hard-codes L = drand48()*0.01 + 0.1")
    args = [REF_BIN, "-l", str(loops), "-p", str(p.num_pieces), "-npp", str(p.nodes_per_piece),
            "-wpp", str(p.wires_per_piece), "-pct", str(int(p.pct_wire_in_piece)),
            "-s", str(p.random_seed)]
    subprocess.run(args, check=True, env=env, stdout=subprocess.DEVNULL)
    out = []
    for stage in ("init", "final"):
        nodes = np.fromfile(f"{pre}.{stage}.r0.bin", NODE_DTYPE)
        wires = np.fromfile(f"{pre}.{stage}.r1.bin", WIRE_DTYPE)
        loc = np.fromfile(f"{pre}.{stage}.r2.bin", "<i4")
        out.append(circuit_from_aos(p, nodes, wires, loc))
    return out[0], out[1]


# -- reduction microbenchmark (benchmarks/reductions/reducetest.cc) ------------
HIST_SEEDS = (12345, 54321)  # reducetest.cc:208-209


def histogram(buckets: int, batch_size: int, num_batches: int, first_batch: int = 0,
              seed1: int = HIST_SEEDS[0], seed2: int = HIST_SEEDS[1]) -> np.ndarray:
    """The histogram one reducetest case adds into its master instance."""
    h = np.zeros(buckets, np.uint32)
    lib().ocl_histogram(buckets, batch_size, num_batches, first_batch, seed1, seed2, _p(h))
    return h


def histogram_threads(buckets: int, batch_size: int, num_batches: int, threads: int,
                      first_batch: int = 0, seed1: int = HIST_SEEDS[0],
                      seed2: int = HIST_SEEDS[1]):
    """(histogram, seconds) on `threads` CPU threads in the redfold schedule."""
    h = np.zeros(buckets, np.uint32)
    secs = lib().ocl_histogram_threads(buckets, batch_size, num_batches, first_batch, seed1,
                                       seed2, threads, _p(h))
    if secs < 0:
        raise RuntimeError("ocl_histogram_threads failed")
    return h, secs


def run_reducetest(buckets: int, num_batches: int, batch_size: int, workdir: str) -> np.ndarray:
    """Run the reference's reducetest.cc (its default cases redfold, localize
    and redlist, all adding into one master instance) and return the master
    histogram it leaves behind."""
    if not os.path.exists(REDUCE_REF_BIN):
        raise FileNotFoundError(REDUCE_REF_BIN)
    os.makedirs(workdir, exist_ok=True)
    path = os.path.join(workdir, "master.bin")
    env = dict(os.environ, CKT_REFSHIM_DUMP=path)
    args = [REDUCE_REF_BIN, "-buckets", str(buckets), "-batches", str(num_batches),
            "-bsize", str(batch_size)]
    subprocess.run(args, check=True, env=env, stdout=subprocess.DEVNULL)
    return np.fromfile(path, "<u4")


def split_quotient_check(lo: int, hi: int, dt: float, zh: float, zl: float, tiny: float):
    """Mismatch counts (trusted, other) of fmaf(a, zh, a*zl) against a/dt over
    the float dividends with bit patterns in [lo, hi); see
    ocl_split_quotient_check."""
    bt, bo = ctypes.c_uint64(), ctypes.c_uint64()
    lib().ocl_split_quotient_check(lo, hi, dt, zh, zl, tiny, ctypes.byref(bt), ctypes.byref(bo))
    return bt.value, bo.value


def wide_quotient_check(seed: int, n: int, divisor: int):
    """(bad, outside, drawn) of EXACT mode's quotient by R (divisor 0) or C
    (1) outside the guarded range against IEEE division; see
    ocl_wide_quotient_check."""
    bad, out, drawn = ctypes.c_uint64(), ctypes.c_uint64(), ctypes.c_uint64()
    lib().ocl_wide_quotient_check(seed, n, divisor, ctypes.byref(bad), ctypes.byref(out),
                                  ctypes.byref(drawn))
    return bad.value, out.value, drawn.value
