"""Seeded many-graph workloads for the batched solve and the serving loop.

The graph mix: n log-uniform in [2^8, 2^20], average degree uniform in
[4, 32], families alternating G(n, m) and 2-D random geometric graphs,
weights uniform in [1, 254], one seed per graph.  Graphs are generated on
the device by the library's own generators (kamsta_gen_gnm_dev,
kamsta_gen_rgg2d_dev), which are bit-identical to the oracle's CPU ones.
"""
from __future__ import annotations

import math
from dataclasses import dataclass

import numpy as np


@dataclass
class GraphSpec:
    family: str      # "gnm" | "rgg2d"
    n: int
    avg_degree: float
    seed: int

    def gnm_m(self) -> int:
        return min(self.n * (self.n - 1) // 2, int(self.n * self.avg_degree / 2))

    def rgg_radius(self) -> float:
        return math.sqrt(self.avg_degree / (math.pi * self.n))


def mixed_specs(count: int, seed: int, log_n_lo: float = 8.0, log_n_hi: float = 20.0,
                deg_lo: float = 4.0, deg_hi: float = 32.0) -> list[GraphSpec]:
    rng = np.random.default_rng(seed)
    out = []
    for i in range(count):
        n = int(round(2.0 ** rng.uniform(log_n_lo, log_n_hi)))
        deg = float(rng.uniform(deg_lo, deg_hi))
        out.append(GraphSpec("gnm" if i % 2 == 0 else "rgg2d", n, deg, seed * 1_000_003 + i))
    return out


def materialize(ctx, specs: list[GraphSpec], stream: int = 0):
    """Generate every graph on the device.  Returns (edges, out, entries)
    lists: one int32 (m, 3) edge tensor per graph, one (n, 3) output tensor,
    and the directed entry counts."""
    import torch
    edges, outs, counts = [], [], []
    for s in specs:
        if s.family == "gnm":
            m = s.gnm_m()
            d = torch.empty((max(2 * m, 1), 3), dtype=torch.int32, device="cuda")
            md = ctx.gen_gnm_dev(s.n, m, s.seed, 254, d.data_ptr(), stream=stream)
        else:
            r = s.rgg_radius()
            md = ctx.gen_rgg2d_dev(s.n, r, s.seed, 254, stream=stream)
            d = torch.empty((max(md, 1), 3), dtype=torch.int32, device="cuda")
            ctx.gen_rgg2d_dev(s.n, r, s.seed, 254, d.data_ptr(), md, stream=stream)
        edges.append(d)
        outs.append(torch.empty((max(s.n, 1), 3), dtype=torch.int32, device="cuda"))
        counts.append(md)
    return edges, outs, counts


def descs_for(K, specs, edges, outs, counts):
    arr = (K.GraphDesc * len(specs))()
    for i, s in enumerate(specs):
        arr[i].edges = edges[i].data_ptr()
        arr[i].m_directed = counts[i]
        arr[i].n = s.n
        arr[i].out = outs[i].data_ptr()
    return arr


def percentiles(values_ms, qs=(50, 99, 99.9)) -> dict:
    a = np.sort(np.asarray(values_ms, dtype=np.float64))
    if len(a) == 0:
        return {f"p{q}_ms": None for q in qs}
    return {f"p{q}_ms".replace(".", "_"): float(np.percentile(a, q)) for q in qs}
