"""Generate the golden fixtures in this folder from the REFERENCE ITSELF.

The reference circuit application (LegionOrigins apps/circuit/circuit.cc)
is compiled unmodified through oracle/refshim (a single-threaded stand-in for
the early Legion API it was written against) and run with its own main():
its own load_circuit generator, its own CPU leaf tasks and its own loop.
Its region contents are dumped after load_circuit and after the last loop.

Fixtures:
  gen_<name>.npz   generator output (graph, locations, initial values)
  sim_<name>.npz   final state after `loops` outer loops of the reference's
                   CPU tasks (inner steps = the reference's STEPS = 10000, CPU
                   task initialisation).  "div" cases use the generated values
                   (the recurrence overflows to NaN); "conv" cases replace the
                   wire/node state after load_circuit with a seeded
                   convergent state (inductance 1e-7..9e-7, random currents
                   and voltages) so every value stays finite and the
                   arithmetic is pinned bit for bit.

  hist_<name>.npz  the master histogram the reference's reduction
                   microbenchmark (benchmarks/reductions/reducetest.cc,
                   compiled unmodified through oracle/refshim_lowlevel)
                   leaves after its default cases redfold, localize and
                   redlist, each of which adds the full histogram into it.

Run in a tree where the reference is present:
    python tests/golden/make_golden.py [--reference /path/to/LegionOrigins]
                                       [--only circuit|hist]
"""
from __future__ import annotations

import argparse
import os
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "..", "..", "oracle"))
import ckt_oracle as O  # noqa: E402

GEN_CASES = {
    # name: (pieces, nodes/piece, wires/piece, pct, seed)
    "cfg0": (4, 256, 1024, 95, 12345),       # the plain CPU-runnable shape
    "p4n8w16": (4, 8, 16, 80, 12345),
    "p3n5w7": (3, 5, 7, 50, 7),
    "p2n1w3": (2, 1, 3, 0, 1),               # one node per piece: in == out
    "p8n64w256pct50": (8, 64, 256, 50, 42),  # heavy cross-piece traffic
    "p5n33w100pct100": (5, 33, 100, 100, 5),  # every wire in-piece
    "p6n16w64pct0": (6, 16, 64, 0, 11),      # every wire crosses pieces
}

SIM_CASES = {
    # name: (gen case params, loops, convergent override seed or None)
    "div_p4n16w64": ((4, 16, 64, 70, 99), 2, None),
    "div_p3n5w7": ((3, 5, 7, 50, 7), 1, None),
    "conv_p4n16w64": ((4, 16, 64, 70, 99), 2, 1),
    "conv_p8n32w128pct50": ((8, 32, 128, 50, 3), 3, 2),
    "conv_p2n1w3": ((2, 1, 3, 0, 1), 2, 3),
    "conv_p6n16w64pct0": ((6, 16, 64, 0, 11), 1, 4),
}

HIST_CASES = {
    # name: (buckets, batches, batch size)
    "b1000_n8_s5000": (1000, 8, 5000),
    "b1_n2_s100": (1, 2, 100),                     # one bucket takes everything
    "b65537_n5_s7777": (65537, 5, 7777),           # ragged sizes
    "b4096_n3_s65536": (4096, 3, 65536),
    "b1048576_n4_s65536": (1048576, 4, 65536),     # the benchmark's bucket count
    "b7_n3_s0": (7, 3, 0),                         # empty batches
}
HIST_CASES_RUN = 3  # redfold, localize, redlist (reducetest.cc:259-261)

FIELDS = ["in_ptr", "out_ptr", "in_loc", "out_loc", "L", "R", "C", "current", "voltage",
          "charge", "node_voltage", "cap", "leak", "locator"]


def convergent_state(c: O.Circuit, seed: int) -> O.Circuit:
    """Seeded finite-regime state: gain L/(dt*R) < 1 keeps the recurrence
    contracting over the reference's 10000 inner steps."""
    rng = np.random.default_rng(seed)
    o = c.copy()
    o.L[:] = rng.uniform(1e-7, 9e-7, o.L.shape).astype(np.float32)
    o.current[:] = rng.uniform(-1, 1, o.current.shape).astype(np.float32)
    o.voltage[:] = rng.uniform(-1, 1, o.voltage.shape).astype(np.float32)
    o.node_voltage[:] = rng.uniform(-1, 1, o.node_voltage.shape).astype(np.float32)
    return o


def save(path: str, c: O.Circuit, **extra) -> None:
    arrays = {k: getattr(c, k) for k in FIELDS}
    arrays.update(extra)
    np.savez_compressed(path, **arrays)


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", default="/root/reference")
    ap.add_argument("--only", choices=["circuit", "hist"], default=None)
    args = ap.parse_args()
    if O.build_ref(args.reference) is None:
        sys.exit(f"reference tree not found at {args.reference}")
    work = tempfile.mkdtemp(prefix="ckt_golden_")
    if args.only != "circuit":
        for name, (buckets, batches, bsize) in HIST_CASES.items():
            master = O.run_reducetest(buckets, batches, bsize, os.path.join(work, name))
            np.savez_compressed(os.path.join(HERE, f"hist_{name}.npz"), master=master,
                                params=np.array([buckets, batches, bsize], np.int64),
                                cases=np.array(HIST_CASES_RUN))
            print("wrote", f"hist_{name}.npz")
    if args.only == "hist":
        return
    for name, (P, npp, wpp, pct, seed) in GEN_CASES.items():
        p = O.GenParams(P, npp, wpp, pct, seed)
        init, _ = O.run_reference(p, 1, os.path.join(work, name))
        save(os.path.join(HERE, f"gen_{name}.npz"), init,
             params=np.array([P, npp, wpp, pct, seed], np.int64))
        print("wrote", f"gen_{name}.npz")
    for name, ((P, npp, wpp, pct, seed), loops, ovr) in SIM_CASES.items():
        p = O.GenParams(P, npp, wpp, pct, seed)
        override = None
        if ovr is not None:
            override = convergent_state(O.generate(p), ovr)
        init, final = O.run_reference(p, loops, os.path.join(work, name), override=override)
        start = override if override is not None else init
        extra = {f"start_{k}": getattr(start, k) for k in FIELDS}
        save(os.path.join(HERE, f"sim_{name}.npz"), final,
             params=np.array([P, npp, wpp, pct, seed], np.int64),
             loops=np.array(loops), steps=np.array(10000), **extra)
        print("wrote", f"sim_{name}.npz")


if __name__ == "__main__":
    main()
