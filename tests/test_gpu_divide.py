"""EXACT mode's quotients against the GPU's divide routine (__fdiv_rn).

calc_new_currents divides by dt, R and C (apps/circuit/circuit_gpu.cu:
119-128).  EXACT mode forms those quotients from precomputed reciprocals:
the split reciprocal of dt = (float)1e-6 for dividends of magnitude
>= 2^-118, and a once-corrected quotient (Markstein's theorem) for R and C
inside a guarded dividend range, the divide routine elsewhere.  These tests
compare the constructions with __fdiv_rn through libckt_tools.so:
every float dividend for dt (2^32 of them), and billions of random and
near-tie (a, b) pairs for the per-wire divisors.
"""
import ctypes

import pytest

pytestmark = pytest.mark.gpu


def counts(cuda, n):
    return cuda.zeros(n, dtype=cuda.int64, device="cuda")


def test_dt_quotient_every_float(cuda, ckt):
    c = counts(cuda, 2)
    T = ckt.tools()
    for half in range(2):  # the 2^32 dividends in two launches
        ckt.check(T.ckt_check_dt_quotient(half << 31, 1 << 31, c.data_ptr(), None))
    cuda.cuda.synchronize()
    trusted, other = c.tolist()
    assert trusted == 0
    assert other == 98  # below 2^-124, as the CPU sweep finds (tests/test_divide.py)


@pytest.mark.parametrize("divisor", [0, 1], ids=["R", "C"])
@pytest.mark.parametrize("near_ties", [0, 1], ids=["any", "near_ties"])
def test_corrected_quotient_random_pairs(cuda, ckt, divisor, near_ties):
    c = counts(cuda, 3)
    n = 1 << 31
    ckt.check(ckt.tools().ckt_check_recip_quotient(1234 + divisor + 2 * near_ties, n, divisor,
                                                   near_ties, c.data_ptr(), None))
    cuda.cuda.synchronize()
    bad, fast, drawn = c.tolist()
    print(f"divisor {'RC'[divisor]} near_ties {near_ties}: {drawn} pairs, "
          f"{fast} on the corrected quotient, {bad} mismatches")
    assert drawn == n
    assert bad == 0
    assert fast > n // 4  # most pairs exercise the corrected quotient itself


@pytest.mark.parametrize("divisor", [0, 1], ids=["R", "C"])
def test_wide_quotient_random_pairs(cuda, ckt, divisor):
    """The quotient of the phases that leave the guarded range (the state's
    zeros at the start of a loop, huge values and infinities as it blows
    up): every class of dividend, those whose quotient may be subnormal
    excepted, equals __fdiv_rn."""
    c = counts(cuda, 3)
    n = 1 << 30
    ckt.check(ckt.tools().ckt_check_wide_quotient(4321 + divisor, n, divisor, c.data_ptr(), None))
    cuda.cuda.synchronize()
    bad, outside, drawn = c.tolist()
    print(f"divisor {'RC'[divisor]}: {drawn} pairs, {outside} outside the guarded range, "
          f"{bad} mismatches")
    assert bad == 0
    assert drawn > n // 2 and outside > drawn // 2
