"""The reduction microbenchmark (benchmarks/reductions/reducetest.cc) on the
GPU, through ckt_hist_run: every schedule's histogram equals the oracle's
bucket for bucket, and the benchmark's default case sequence reproduces the
reference's own master histogram (tests/golden/hist_*.npz)."""
import ctypes
import glob
import os

import numpy as np
import pytest

from conftest import GOLDEN, load_npz

pytestmark = pytest.mark.gpu

SCHEDULES = {"single": 0, "fold": 1, "localize": 2, "list": 3}


def run(cuda, p, schedules, start=None, scratch=None):
    from legionorigins_gb300 import check, lib
    from legionorigins_gb300 import reductions as R

    torch = cuda
    h = torch.zeros(p.buckets, dtype=torch.int32, device="cuda")
    if start is not None:
        h.copy_(torch.from_numpy(start.view(np.int32)))
    for s in schedules:
        lo, hi = R.scratch_bytes(p, s)
        n = hi if scratch is None else max(lo, scratch)
        buf = torch.empty(max(n, 16), dtype=torch.uint8, device="cuda")
        check(lib().ckt_hist_run(ctypes.byref(p), s, h.data_ptr(), buf.data_ptr(), n, None))
    torch.cuda.synchronize()
    return h.cpu().numpy().view(np.uint32)


@pytest.mark.parametrize("path", sorted(glob.glob(os.path.join(GOLDEN, "hist_*.npz"))),
                         ids=lambda p: os.path.basename(p))
def test_default_cases_match_reference_master(cuda, path):
    """redfold, localize, redlist into one master instance, as the
    benchmark runs them: the reference's master histogram, exactly."""
    from legionorigins_gb300 import reductions as R

    g = load_npz(os.path.basename(path))
    buckets, batches, bsize = (int(x) for x in g["params"])
    p = R.params(buckets, bsize, batches)
    got = run(cuda, p, [SCHEDULES["fold"], SCHEDULES["localize"], SCHEDULES["list"]])
    assert np.array_equal(got, g["master"])


SHAPES = [
    # buckets, batch size, batches, first batch
    (1, 1000, 3, 0),            # one bucket: every reduction collides
    (3, 4097, 2, 0),
    (1000, 5000, 8, 0),
    (51200, 20000, 3, 0),       # largest shared-memory fold
    (51201, 20000, 3, 0),       # smallest L2 fold
    (65537, 7777, 5, 0),
    (1048576, 65536, 4, 0),
    (4194304, 100000, 2, 0),
    (977, 4096, 2, (1 << 20) - 1),  # element indices wrap at 2^32
]


@pytest.mark.parametrize("schedule", sorted(SCHEDULES))
@pytest.mark.parametrize("shape", SHAPES, ids=lambda s: "x".join(str(v) for v in s))
def test_schedule_matches_oracle(cuda, oracle, schedule, shape):
    from legionorigins_gb300 import reductions as R

    buckets, bsize, batches, first = shape
    p = R.params(buckets, bsize, batches, first)
    want = oracle.histogram(buckets, bsize, batches, first_batch=first)
    rng = np.random.default_rng(buckets)
    start = rng.integers(0, 1 << 32, buckets, dtype=np.uint64).astype(np.uint32)
    got = run(cuda, p, [SCHEDULES[schedule]], start=start)
    assert np.array_equal(got, start + want)  # the target keeps its contents (mod 2^32)


@pytest.mark.parametrize("schedule", ["fold", "localize", "list"])
def test_minimum_scratch_many_rounds(cuda, oracle, schedule):
    """The smallest scratch each schedule accepts: one batch per list round,
    4096 elements per localize round, one L2 fold copy."""
    from legionorigins_gb300 import reductions as R

    p = R.params(70001, 3001, 7)
    want = oracle.histogram(70001, 3001, 7)
    got = run(cuda, p, [SCHEDULES[schedule]], scratch=0)
    assert np.array_equal(got, want)


def test_localize_largest_bucket_count(cuda, oracle):
    from legionorigins_gb300 import reductions as R

    b = 1 << 26
    p = R.params(b, 50000, 2)
    got = run(cuda, p, [SCHEDULES["localize"]])
    assert np.array_equal(got, oracle.histogram(b, 50000, 2))


def test_empty_batches_leave_target_unchanged(cuda):
    from legionorigins_gb300 import reductions as R

    start = np.arange(17, dtype=np.uint32)
    for p in (R.params(17, 0, 5), R.params(17, 5, 0)):
        got = run(cuda, p, list(SCHEDULES.values()), start=start)
        assert np.array_equal(got, start)


def test_run_case_prints_elapsed(cuda, oracle, capsys):
    from legionorigins_gb300 import reductions as R

    p = R.params(4096, 10000, 4)
    h = R.Histogram(p, cases=R.DEFAULT_CASES)
    for name in R.DEFAULT_CASES:
        assert h.run_case(name) >= 0
    assert np.array_equal(h.counts(), 3 * oracle.histogram(4096, 10000, 4))
    out = capsys.readouterr().out
    assert "ELAPSED(redfold)" in out and "ELAPSED(redlist)" in out
