"""The division by dt of EXACT mode, checked on the CPU.

calc_new_currents divides L*(i - I0) by dt = (float)1e-6 ten times per
wire-step (apps/circuit/circuit.cc:391-393, circuit_gpu.cu:119-122).  The
GPU's EXACT mode forms that quotient as fma(a, zh, a*zl), zh = RN(1/dt),
zl = RN(1/dt - zh), and uses it only for dividends of magnitude >= 2^-118
(smaller ones, zero included, take the divide routine).  Here the C
library's fmaf evaluates the same expression for every one of the 2^32
float dividends and compares it with IEEE division a/dt: no mismatch is
allowed among the dividends the kernel trusts it for.  The GPU test
(tests/test_gpu_divide.py) repeats the sweep against __fdiv_rn.
"""
import concurrent.futures as cf
import os

import numpy as np

DT_BITS, ZH_BITS, ZL_BITS = 0x358637BD, 0x49742400, 0x3B257666
TINY = 2.0 ** -118


def f32(bits):
    return float(np.array([bits], np.uint32).view(np.float32)[0])


def test_split_reciprocal_constants():
    """zh and zl are the round-to-nearest split of 1/dt."""
    from fractions import Fraction

    dt, zh, zl = f32(DT_BITS), f32(ZH_BITS), f32(ZL_BITS)
    assert np.float32(1e-6) == np.float32(dt)
    inv = 1 / Fraction(dt)

    def rn32(x):
        f = np.float32(float(x))
        cands = [np.nextafter(f, np.float32(-np.inf)), f, np.nextafter(f, np.float32(np.inf))]
        return float(min(cands, key=lambda c: abs(Fraction(float(c)) - x)))

    assert zh == rn32(inv) == 1e6
    assert zl == rn32(inv - Fraction(zh))
    assert zl > 0  # a*zl keeps the sign of a: signed zeros and infinities stay exact


def test_split_quotient_equals_ieee_division_for_every_float(oracle):
    dt, zh, zl = f32(DT_BITS), f32(ZH_BITS), f32(ZL_BITS)
    chunks = 256
    step = (1 << 32) // chunks
    threads = max(1, min(16, os.cpu_count() or 1))
    with cf.ThreadPoolExecutor(threads) as ex:
        res = list(ex.map(lambda c: oracle.split_quotient_check(c * step, (c + 1) * step, dt, zh,
                                                                zl, TINY), range(chunks)))
    trusted = sum(r[0] for r in res)
    other = sum(r[1] for r in res)
    assert trusted == 0
    # below 2^-124 the product a*zl underflows and some quotients are off
    assert other == 98, other


def test_wide_quotient_equals_ieee_division(oracle):
    """EXACT mode's quotient by R and C for dividends outside the corrected
    quotient's guarded range -- scaled by a power of two into it, zeros and
    infinities as a times RN(1/b) -- restated in C with fmaf: equal to IEEE
    a/b on every pair drawn (huge, tiny down to the smallest subnormal as
    long as the quotient stays normal, zeros, infinities, NaN, near rounding
    boundaries and near overflow).  The GPU
    test (tests/test_gpu_divide.py) repeats it against __fdiv_rn."""
    for divisor in (0, 1):
        bad, outside, drawn = oracle.wide_quotient_check(11 + divisor, 1 << 22, divisor)
        assert bad == 0, (divisor, bad)
        assert drawn > 3 << 20 and outside > drawn // 2
