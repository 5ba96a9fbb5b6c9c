"""The reduction microbenchmark (LegionOrigins benchmarks/reductions/
reducetest.cc) on the GPU.

The benchmark histograms `num_batches` batches of `batch_size` hashed
elements into `buckets` unsigned counters under several reduction
schedules and prints ELAPSED(<case>) for each (reducetest.cc:152-200).
Here each case is one ckt_hist_run call (include/ckt.h) with the schedule
the case maps to:

    original, redsingle -> CKT_RED_SINGLE   (direct reductions)
    redfold             -> CKT_RED_FOLD     (fold instance, then applied)
    localize            -> CKT_RED_LOCALIZE (owner-local copy, then written back)
    redlist             -> CKT_RED_LIST     (reduction list, then applied)

Like the benchmark, every case adds into the same target histogram.
"""
from __future__ import annotations

import ctypes

from . import RED_FOLD, RED_LIST, RED_LOCALIZE, RED_SINGLE, HistParams, check, lib

CASES = {
    "original": RED_SINGLE,
    "redfold": RED_FOLD,
    "localize": RED_LOCALIZE,
    "redlist": RED_LIST,
    "redsingle": RED_SINGLE,
}
# the cases the benchmark runs without -doslow (reducetest.cc:257-263)
DEFAULT_CASES = ("redfold", "localize", "redlist")


def params(buckets: int = 1048576, batch_size: int = 1048576, num_batches: int = 1024,
           first_batch: int = 0, seed1: int = 12345, seed2: int = 54321) -> HistParams:
    """The benchmark's arguments; defaults are its own (reducetest.cc:205-209)."""
    return HistParams(buckets, batch_size, num_batches, first_batch, seed1, seed2)


def scratch_bytes(p: HistParams, schedule: int) -> tuple[int, int]:
    """(minimum, full-speed) scratch bytes for a schedule."""
    lo, hi = ctypes.c_uint64(), ctypes.c_uint64()
    check(lib().ckt_hist_scratch_bytes(ctypes.byref(p), schedule, ctypes.byref(lo),
                                       ctypes.byref(hi)))
    return lo.value, hi.value


class Histogram:
    """A device histogram (the benchmark's master instance) and the scratch
    the schedules need, allocated once through torch."""

    def __init__(self, p: HistParams, cases=DEFAULT_CASES, device: str = "cuda"):
        import torch

        self.torch, self.p = torch, p
        self.hist = torch.zeros(p.buckets, dtype=torch.int32, device=device)
        need = max([scratch_bytes(p, CASES[c])[1] for c in cases] + [16])
        self.scratch = torch.empty(need, dtype=torch.uint8, device=device)

    def run(self, schedule: int, stream: int = 0) -> None:
        check(lib().ckt_hist_run(ctypes.byref(self.p), schedule, self.hist.data_ptr(),
                                 self.scratch.data_ptr(), self.scratch.numel(), stream))

    def run_case(self, name: str, verbose: bool = True) -> float:
        """One benchmark case, timed with CUDA events on the current stream;
        prints ELAPSED(name) = seconds like the benchmark."""
        torch = self.torch
        s = torch.cuda.current_stream()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record(s)
        self.run(CASES[name], s.cuda_stream)
        e1.record(s)
        e1.synchronize()
        secs = e0.elapsed_time(e1) * 1e-3
        if verbose:
            print(f"ELAPSED({name}) = {secs:f}")
        return secs

    def counts(self):
        """The histogram as uint32 on the host."""
        import numpy as np

        return self.hist.cpu().numpy().view(np.uint32)
