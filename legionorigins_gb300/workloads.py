"""Synthetic workload definitions for the batched and served forms.

Shapes are drawn with splitmix64 (a published 64-bit mixing generator:
x += 0x9E3779B97F4A7C15; z = x; z = (z ^ z>>30) * 0xBF58476D1CE4E5B9;
z = (z ^ z>>27) * 0x94D049BB133111EB; return z ^ z>>31), one stream per
circuit or request, so every shape is reproducible on any machine.  Each
circuit's graph and values then come from the reference generator seeded
with the circuit's own seed.  Inductance is U[0.001, 0.011) as in the
benchmark configurations.
"""
from __future__ import annotations

import math
from dataclasses import dataclass

MASK = (1 << 64) - 1
L_OFFSET, L_SCALE = 0.001, 0.01


class SplitMix64:
    def __init__(self, seed: int):
        self.x = seed & MASK

    def next(self) -> int:
        self.x = (self.x + 0x9E3779B97F4A7C15) & MASK
        z = self.x
        z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & MASK
        z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & MASK
        return z ^ (z >> 31)

    def uniform(self) -> float:
        return (self.next() >> 11) * 2.0 ** -53


@dataclass
class CircuitSpec:
    num_pieces: int
    nodes_per_piece: int
    wires_per_piece: int
    pct_wire_in_piece: float
    random_seed: int
    steps: int
    loops: int = 1
    L_offset: float = L_OFFSET
    L_scale: float = L_SCALE

    @property
    def wires(self) -> int:
        return self.num_pieces * self.wires_per_piece

    @property
    def nodes(self) -> int:
        return self.num_pieces * self.nodes_per_piece

    @property
    def segment_updates(self) -> int:
        return self.wires * 10 * self.steps * self.loops

    def gen_args(self):
        return (self.num_pieces, self.nodes_per_piece, self.wires_per_piece,
                self.pct_wire_in_piece, self.random_seed, self.L_offset, self.L_scale)


def mixed_batch(n: int = 256, first_seed: int = 0) -> list[CircuitSpec]:
    """Batched mixed sizes: per circuit, pieces uniform in {1..32}, nodes
    per piece log-uniform in [256, 16384], 4 wires per node, in-piece
    fraction U[0.8, 0.98], inner steps uniform in {100..1000}, one outer
    loop, reference-generator seed = circuit index."""
    out = []
    for c in range(first_seed, first_seed + n):
        r = SplitMix64(0xC1C0 ^ (c * 0x100000001B3))
        P = 1 + r.next() % 32
        npp = int(round(math.exp(math.log(256) + r.uniform() * math.log(16384 / 256))))
        pct = 100.0 * (0.8 + 0.18 * r.uniform())
        S = 100 + r.next() % 901
        out.append(CircuitSpec(P, npp, 4 * npp, pct, c, S, 1))
    return out


def serve_request(req_id: int, stream_seed: int = 0) -> CircuitSpec:
    """One circuit-solve request: total wires log-uniform in [1e3, 4e6],
    4 wires per node, 8..64 pieces, 95% in-piece, inner steps uniform in
    {100..1000}, 1..5 outer loops, reference-generator seed = request id."""
    r = SplitMix64((stream_seed * 0x9E3779B1 + req_id * 0x85EBCA77 + 0x5E5E) & MASK)
    W = math.exp(math.log(1e3) + r.uniform() * math.log(4e6 / 1e3))
    P = 8 + r.next() % 57
    wpp = max(1, math.ceil(W / P))
    npp = max(1, math.ceil(wpp / 4))
    S = 100 + r.next() % 901
    Lp = 1 + r.next() % 5
    return CircuitSpec(P, npp, wpp, 95.0, req_id, S, Lp)
