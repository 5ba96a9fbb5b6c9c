"""Workload definitions of the batched and served forms (CPU only)."""
from legionorigins_gb300.workloads import SplitMix64, mixed_batch, serve_request


def test_splitmix64_known_values():
    # splitmix64 seeded with 0: first outputs of the published generator
    r = SplitMix64(0)
    assert r.next() == 0xE220A8397B1DCDAF
    assert r.next() == 0x6E789E6AA1B965F4


def test_mixed_batch_shapes_are_the_configured_distribution():
    from legionorigins_gb300.workloads import mixed_batch

    m = mixed_batch(256)
    assert len(m) == 256 and [s.random_seed for s in m] == list(range(256))
    assert all(1 <= s.num_pieces <= 32 for s in m)
    assert all(256 <= s.nodes_per_piece <= 16384 and s.wires_per_piece == 4 * s.nodes_per_piece
               for s in m)
    assert all(80.0 <= s.pct_wire_in_piece <= 98.0 for s in m)
    assert all(100 <= s.steps <= 1000 for s in m)
    assert len({s.num_pieces for s in m}) > 20


def test_serve_requests_are_the_configured_distribution():
    reqs = [serve_request(i) for i in range(2000)]
    assert all(8 <= r.num_pieces <= 64 for r in reqs)
    assert all(1e3 / 64 <= r.wires <= 4e6 + 64 for r in reqs)
    assert all(100 <= r.steps <= 1000 and 1 <= r.loops <= 5 for r in reqs)
    assert all(r.pct_wire_in_piece == 95.0 for r in reqs)
    assert all(r.nodes_per_piece * 4 >= r.wires_per_piece for r in reqs)
    small = sum(r.wires < 1e4 for r in reqs) / len(reqs)
    assert 0.15 < small < 0.45   # log-uniform: ~29% below 1e4
