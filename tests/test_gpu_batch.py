"""The batched form: one persistent launch advances many circuits of uneven
sizes; every circuit must come out bit-identical to running it alone."""
import numpy as np
import pytest

from conftest import same_bits

pytestmark = pytest.mark.gpu

STATE = ["current", "voltage", "charge", "node_voltage"]
FIELDS = ["in_ptr", "out_ptr", "in_loc", "out_loc", "L", "R", "C", "current", "voltage",
          "charge", "node_voltage", "cap", "leak", "locator"]


def small_specs():
    from legionorigins_gb300.workloads import CircuitSpec

    return [
        CircuitSpec(4, 64, 256, 90.0, 1, 6),
        CircuitSpec(1, 7, 50, 50.0, 3, 5),        # one piece
        CircuitSpec(3, 5, 7, 50.0, 7, 4),         # ragged
        CircuitSpec(2, 1, 3, 0.0, 11, 6),         # one node per piece, all cross
        CircuitSpec(6, 40, 100, 83.5, 12, 2),     # real-valued pct
        CircuitSpec(5, 33, 0, 95.0, 13, 3),       # no wires at all
        CircuitSpec(16, 128, 512, 50.0, 14, 1),   # heavy reduction
        CircuitSpec(2, 1, 5000, 50.0, 15, 2),     # hub nodes: runs over several staging chunks
    ]


def oracle_run(oracle, spec, loops, quirk=False):
    p = oracle.GenParams(*spec.gen_args()[:5], L_offset=spec.L_offset, L_scale=spec.L_scale)
    c = oracle.generate(p)
    oracle.simulate(c, loops, spec.steps, quirk=quirk)
    return c


@pytest.fixture(scope="module")
def specs():
    return small_specs()


@pytest.mark.parametrize("mode", [0, 1])
def test_batched_matches_circuits_run_alone(cuda, oracle, specs, mode):
    from legionorigins_gb300 import circuit as C
    from legionorigins_gb300.batch import Batch

    b = Batch(specs)
    for _ in range(2):
        b.run(mode)
    assert b.check() == 0
    for i, s in enumerate(specs):
        got = b.read(i)
        if mode == 0:
            ref = oracle_run(oracle, s, 2)
            for k in STATE:
                assert same_bits(got[k], getattr(ref, k)), (i, k)
        else:  # FAST: bit-identical to the plain FAST path on the circuit alone
            h = C.generate(*s.gen_args())
            dc = C.DeviceCircuit(h, C.Shape(s.num_pieces, s.nodes_per_piece, s.wires_per_piece))
            prm = C.params(s.steps, 1)
            dc.loop_index_space(prm)
            dc.loop_index_space(prm)
            cuda.cuda.synchronize()
            alone = dc.to_host()
            for k in STATE:
                assert np.array_equal(got[k].view(np.uint32), alone[k].view(np.uint32)), (i, k)
    b.close()


def test_every_launch_shape_and_the_sequential_path_agree(cuda, specs):
    from legionorigins_gb300.batch import Batch

    b = Batch(specs)
    results = []
    for block in (128, 256):
        for wpt in (1, 2):
            for dcs in (0, 1, 2):
                b.set_config(block, wpt, dcs)
                b.reset_state()
                b.run(0)
                assert b.check() == 0
                results.append([b.read(i) for i in range(len(specs))])
    for per_piece in (False, True):
        b.reset_state()
        b.run_sequential(0, per_piece=per_piece)
        cuda.cuda.synchronize()
        results.append([b.read(i) for i in range(len(specs))])
    for r in results[1:]:
        for i in range(len(specs)):
            for k in STATE:
                assert np.array_equal(r[i][k].view(np.uint32), results[0][i][k].view(np.uint32))
    b.close()


def test_autotune_picks_a_valid_shape_and_keeps_results(cuda, oracle, specs):
    from legionorigins_gb300.batch import Batch

    b = Batch(specs)
    cfg = b.autotune(0)
    assert cfg["block"] in (128, 256) and cfg["wires_per_thread"] in (1, 2)
    assert cfg["blocks_per_sm"] >= 1
    b.run(0)
    assert b.check() == 0
    for i, s in enumerate(specs):
        ref = oracle_run(oracle, s, 1)
        got = b.read(i)
        for k in STATE:
            assert same_bits(got[k], getattr(ref, k)), (i, k)
    b.close()


def test_same_result_alone_and_in_the_mix(cuda, specs):
    from legionorigins_gb300.batch import Batch
    from legionorigins_gb300.workloads import mixed_batch

    mix = mixed_batch(12)
    mix = [s for s in mix if s.wires < 300_000][:6]
    target = specs[0]
    alone = Batch([target])
    alone.run(1)
    a = alone.read(0)
    together = Batch(mix[:3] + [target] + mix[3:])
    together.autotune(1)
    together.run(1)
    assert together.check() == 0
    b = together.read(3)
    for k in STATE:
        assert np.array_equal(a[k].view(np.uint32), b[k].view(np.uint32)), k


def test_bounded_wait_times_out_cleanly(cuda, specs):
    """A distribute_charge tile made to wait for a calc_new_currents tile
    that does not exist: the bounded wait runs out, the kernel reports
    CKT_ETIMEOUT, and the context stays usable."""
    from legionorigins_gb300.batch import Batch

    b = Batch(specs)
    b.set_timeout(50_000_000)  # 50 ms
    b.inject_stall(2, True)
    b.run_direct(0)
    assert b.check() == 4
    b.inject_stall(2, False)
    b.reset_state()
    b.run(0)
    assert b.check() == 0
    b.close()
