"""EXACT mode (corrected quotients by precomputed reciprocals, two wires per
thread) against the divide-routine form CKT_MODE_EXACT_DIVIDE and the fp32
oracle: identical bits on every state, including the ones that leave the
corrected quotients' range -- zeros, subnormals, huge and infinite values,
NaN, signed zeros -- and divisors outside it (R or C zero, tiny, huge,
negative, NaN), which take the divide routine.
"""
import numpy as np
import pytest

from conftest import same_bits

pytestmark = pytest.mark.gpu

STATE = ["current", "voltage", "charge", "node_voltage"]
FIELDS = ["in_ptr", "out_ptr", "in_loc", "out_loc", "L", "R", "C", "current", "voltage",
          "charge", "node_voltage", "cap", "leak", "locator"]
EXACT, FAST, EXACT_DIVIDE = 0, 1, 3


def device(c):
    from legionorigins_gb300 import circuit as C

    p = c.params
    host = {k: np.ascontiguousarray(getattr(c, k)) for k in FIELDS}
    return C.DeviceCircuit(host, C.Shape(p.num_pieces, p.nodes_per_piece, p.wires_per_piece))


def cnc(cuda, dc, steps, mode, init=0):
    import ctypes

    from legionorigins_gb300 import check, lib
    from legionorigins_gb300 import circuit as C

    prm = C.params(steps, mode, init)
    check(lib().ckt_calc_new_currents_all(dc.graph.handle, dc.wires(), dc.nodes(),
                                          ctypes.byref(prm), None))
    cuda.cuda.synchronize()
    return dc.to_host()


def wide(rng, shape):
    """Values over many binades with both signs."""
    mag = np.exp2(rng.uniform(-30, 30, shape))
    return (mag * rng.choice([-1.0, 1.0], shape)).astype(np.float32)


def sprinkle(rng, a, frac=0.01):
    """Replaces a fraction of the elements with edge values."""
    edge = np.array([0.0, -0.0, np.inf, -np.inf, np.nan, 1e-45, -1e-45, 1e-40, 3e38, -3e38,
                     2.0 ** -60, 2.0 ** 95, 2.0 ** -118, 2.0 ** 101], np.float32)
    m = rng.random(a.shape) < frac
    a[m] = rng.choice(edge, m.sum())
    return a


@pytest.mark.parametrize("steps", [1, 2, 3, 7, 64, 1000])
@pytest.mark.parametrize("init", [0, 1])
def test_exact_equals_divide_routine_on_wide_states(cuda, oracle, steps, init):
    c = oracle.generate(oracle.GenParams(8, 512, 2048, 80, 77, L_offset=0.001))
    rng = np.random.default_rng(steps * 2 + init)
    c.current[:] = sprinkle(rng, wide(rng, c.current.shape))
    c.voltage[:] = sprinkle(rng, wide(rng, c.voltage.shape))
    c.node_voltage[:] = sprinkle(rng, wide(rng, c.node_voltage.shape))
    a = cnc(cuda, device(c), steps, EXACT, init)
    b = cnc(cuda, device(c), steps, EXACT_DIVIDE, init)
    for k in ("current", "voltage"):
        assert same_bits(a[k], b[k]), k
    if steps <= 64:
        oracle.calc_new_currents(c, steps, quirk=bool(init))
        for k in ("current", "voltage"):
            assert same_bits(a[k], getattr(c, k)), k


def test_exact_divisors_outside_the_corrected_range(cuda, oracle):
    """Wires whose R or C is zero, subnormal, huge, negative or NaN run on the
    divide routine; their partners and neighbours are unaffected."""
    c = oracle.generate(oracle.GenParams(4, 256, 1024, 95, 5, L_offset=0.001))
    rng = np.random.default_rng(3)
    c.current[:] = rng.uniform(-1, 1, c.current.shape).astype(np.float32)
    c.voltage[:] = rng.uniform(-1, 1, c.voltage.shape).astype(np.float32)
    odd = np.array([0.0, 1e-40, 2.0 ** -31, 2.0 ** 31, 3e38, -2.5, -1e-3, np.nan, np.inf], np.float32)
    for field in ("R", "C"):
        arr = getattr(c, field)
        idx = rng.choice(arr.size, 200, replace=False)
        arr[idx] = rng.choice(odd, idx.size)
    for steps in (1, 4, 100):
        a = cnc(cuda, device(c), steps, EXACT)
        b = cnc(cuda, device(c), steps, EXACT_DIVIDE)
        for k in ("current", "voltage"):
            assert same_bits(a[k], b[k]), (steps, k)


def test_exact_general_dt(cuda, oracle):
    """A dt other than (float)1e-6 divides through the corrected quotient
    (or, outside its range, the divide routine) and gives the oracle's bits."""
    import ctypes

    from legionorigins_gb300 import check, lib
    from legionorigins_gb300 import circuit as C

    c = oracle.generate(oracle.GenParams(4, 64, 256, 90, 9, L_offset=0.001))
    rng = np.random.default_rng(11)
    c.current[:] = rng.uniform(-1, 1, c.current.shape).astype(np.float32)
    c.voltage[:] = rng.uniform(-1, 1, c.voltage.shape).astype(np.float32)
    for dt in (2.5e-7, 1e-3, 0.75, 2.0 ** -40):
        outs = []
        for mode in (EXACT, EXACT_DIVIDE):
            dc = device(c)
            prm = C.params(5, mode)
            prm.dt = dt
            check(lib().ckt_calc_new_currents_all(dc.graph.handle, dc.wires(), dc.nodes(),
                                                  ctypes.byref(prm), None))
            cuda.cuda.synchronize()
            outs.append(dc.to_host())
        for k in ("current", "voltage"):
            assert same_bits(outs[0][k], outs[1][k]), (dt, k)


@pytest.mark.slow
@pytest.mark.parametrize("cfg", ["config1", "config2"])
def test_full_size_finite_regime_exact(cuda, oracle, cfg):
    """Config 1 (64 x 16384 x 65536, 95% in-piece) and config 2 (128 x 8192
    x 32768, 50% in-piece) at full size, 4 inner steps x 2 loops (finite
    values throughout): the library's loop in EXACT mode equals the fp32
    oracle bit for bit on every wire and node.  FAST mode on the same
    circuits is reported per element against the fp32 oracle and against
    the fp64 oracle."""
    shape = (64, 16384, 65536, 95) if cfg == "config1" else (128, 8192, 32768, 50)
    p = oracle.GenParams(*shape, 12345, L_offset=0.001)
    c = oracle.generate(p)
    from legionorigins_gb300 import circuit as C

    got = {}
    for mode in (EXACT, FAST):
        dc = device(c)
        dc.run_loops(C.params(4, mode), 2)
        cuda.cuda.synchronize()
        got[mode] = dc.to_host()
        dc.close()
    c64 = c.astype(np.float64)
    oracle.simulate(c, 2, 4)
    oracle.simulate(c64, 2, 4)
    for k in STATE:
        ref = getattr(c, k)
        assert np.isfinite(ref).all(), k
        assert same_bits(got[EXACT][k], ref), k
        r64 = np.abs(got[EXACT][k].astype(np.float64) - getattr(c64, k)) / np.maximum(
            np.abs(getattr(c64, k)), 1e-30)
        f = got[FAST][k].astype(np.float64)
        rf = np.abs(f - ref) / np.maximum(np.abs(ref), 1e-6)
        print(f"{cfg} {k}: EXACT vs fp64 max {r64.max():.2e} rms {np.sqrt((r64 ** 2).mean()):.2e}; "
              f"FAST vs fp32 reference max {rf.max():.2e} (elements over 1e-5: "
              f"{int((rf > 1e-5).sum())} of {rf.size})")


@pytest.mark.parametrize("steps", [16, 17, 100])
def test_exact_all_nan_wires_beside_finite_ones(cuda, oracle, steps):
    """Wires whose whole state is NaN drop the quotient guards (no dividend
    can then leave NaN); their neighbours in the same warps keep them.  Both
    end with the divide-routine form's bits and the oracle's."""
    c = oracle.generate(oracle.GenParams(4, 256, 1024, 95, 21, L_offset=0.001))
    rng = np.random.default_rng(steps)
    c.current[:] = rng.uniform(-1, 1, c.current.shape).astype(np.float32)
    c.voltage[:] = rng.uniform(-1, 1, c.voltage.shape).astype(np.float32)
    nan_wires = rng.random(c.current.shape[1]) < 0.5
    c.current[:, nan_wires] = np.nan
    c.voltage[:, nan_wires] = np.nan
    a = cnc(cuda, device(c), steps, EXACT)
    b = cnc(cuda, device(c), steps, EXACT_DIVIDE)
    for k in ("current", "voltage"):
        assert same_bits(a[k], b[k]), k
        assert np.isnan(a[k][:, nan_wires]).all(), k
    oracle.calc_new_currents(c, steps)
    for k in ("current", "voltage"):
        assert same_bits(a[k], getattr(c, k)), k
