"""The serving loop: requests arrive while others are on the GPU, are admitted
under an HBM budget, share rounds, and each result is bit-identical to the
request run alone."""
import time

import numpy as np
import pytest

from conftest import same_bits

pytestmark = pytest.mark.gpu

STATE = ["current", "voltage", "charge", "node_voltage"]


def spec(P, npp, wpp, seed, steps, loops, pct=95.0):
    from legionorigins_gb300.workloads import CircuitSpec

    return CircuitSpec(P, npp, wpp, pct, seed, steps, loops)


def alone(cuda, s, mode):
    from legionorigins_gb300 import circuit as C

    h = C.generate(*s.gen_args())
    dc = C.DeviceCircuit(h, C.Shape(s.num_pieces, s.nodes_per_piece, s.wires_per_piece))
    prm = C.params(s.steps, mode)
    for _ in range(s.loops):
        dc.loop_index_space(prm)
    cuda.cuda.synchronize()
    return dc.to_host()


@pytest.mark.parametrize("device_generate", [True, False])
@pytest.mark.parametrize("mode", [0, 1], ids=["exact", "fast"])
def test_each_result_is_the_same_alone_and_in_the_mix(cuda, device_generate, mode):
    from legionorigins_gb300.serve import Server

    mix = [spec(8, 64, 256, 101, 40, 3), spec(12, 30, 120, 102, 25, 1),
           spec(20, 256, 1024, 103, 60, 2), spec(9, 5, 20, 104, 33, 5),
           spec(64, 128, 512, 105, 10, 4), spec(16, 1000, 4000, 106, 15, 2)]
    srv = Server(mode=mode, keep_results=True, prep_threads=4, device_generate=device_generate)
    # staggered arrivals: later requests arrive while earlier ones run
    for i, s in enumerate(mix):
        srv.submit(i, s)
        time.sleep(0.002 * (i % 3))
    assert srv.wait(120.0) == 0
    done = {c["request_id"]: c for c in srv.poll()}
    assert sorted(done) == list(range(len(mix)))
    assert all(c["status"] == 0 and c["loops"] == mix[c["request_id"]].loops for c in done.values())
    st = srv.stats()
    assert st["rounds"] >= max(s.loops for s in mix)
    for i, s in enumerate(mix):
        got = srv.take_result(i)
        ref = alone(cuda, s, mode)
        for k in STATE:
            assert np.array_equal(got[k].view(np.uint32), ref[k].view(np.uint32)), (i, k)
    srv.close()


def test_exact_mode_served_matches_oracle(cuda, oracle):
    from legionorigins_gb300.serve import Server

    reqs = [spec(4, 16, 64, 7, 6, 2), spec(3, 5, 7, 8, 4, 3, pct=50.0)]
    srv = Server(mode=0, keep_results=True, prep_threads=2)
    for i, s in enumerate(reqs):
        srv.submit(i, s)
    assert srv.wait(60.0) == 0
    for i, s in enumerate(reqs):
        got = srv.take_result(i)
        c = oracle.generate(oracle.GenParams(*s.gen_args()[:5], L_offset=s.L_offset,
                                             L_scale=s.L_scale))
        oracle.simulate(c, s.loops, s.steps)
        for k in STATE:
            assert same_bits(got[k], getattr(c, k)), (i, k)
    srv.close()


def test_admission_respects_the_hbm_budget(cuda):
    from legionorigins_gb300.serve import Server

    s = spec(16, 256, 1024, 11, 50, 2)
    one = 16 * 1024 * 130 + 16 * 256 * 30  # a little more than one circuit's device bytes
    srv = Server(mode=1, hbm_budget_bytes=int(one * 1.3), keep_results=False, prep_threads=2)
    for i in range(5):
        srv.submit(i, spec(16, 256, 1024, 20 + i, 50, 2))
    srv.submit(99, spec(64, 4096, 16384, 5, 10, 1))  # larger than the whole budget
    assert srv.wait(120.0) == 0
    done = {c["request_id"]: c for c in srv.poll()}
    assert all(done[i]["status"] == 0 for i in range(5))
    assert done[99]["status"] == 5  # CKT_ENOMEM
    st = srv.stats()
    assert st["resident_peak"] == 1
    assert st["bytes_peak"] <= int(one * 1.3)
    srv.close()


def test_cancel_and_bad_requests(cuda):
    from legionorigins_gb300 import CktError
    from legionorigins_gb300.serve import Server

    srv = Server(mode=1, keep_results=False, prep_threads=1, max_circuits=1)
    for i in range(4):
        srv.submit(i, spec(32, 2048, 8192, 30 + i, 1000, 5))
    srv.cancel(3)
    with pytest.raises(CktError):
        srv.submit(10, spec(0, 4, 4, 1, 1, 1))   # no pieces
    with pytest.raises(CktError):
        srv.submit(2, spec(2, 4, 4, 1, 1, 1))    # id still open (queued behind 0 and 1)
    assert srv.wait(300.0) == 0
    done = {c["request_id"]: c for c in srv.poll()}
    assert done[3]["status"] == 7  # CKT_ECANCELLED
    assert all(done[i]["status"] == 0 for i in range(3))
    srv.close()


def test_destroy_with_open_requests_is_clean(cuda):
    from legionorigins_gb300.serve import Server

    srv = Server(mode=1, prep_threads=2)
    for i in range(8):
        srv.submit(i, spec(32, 1024, 4096, 40 + i, 1000, 5))
    time.sleep(0.05)
    srv.close()
    # the device is still usable afterwards
    srv2 = Server(mode=1, keep_results=True, prep_threads=1)
    srv2.submit(0, spec(2, 8, 32, 1, 5, 1))
    assert srv2.wait(60.0) == 0
    srv2.close()
