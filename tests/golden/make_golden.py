"""Writes tests/golden/*.json -- known-answer fixtures for the MSF path.

The reference (KaMSTa) ships no golden vectors: its only test
(tests/test_sets.sh) compares the MSF weight against a sequential Kruskal.
These fixtures pin the oracle instead:

* tiny_graphs.json: hand-built graphs whose minimum spanning forest under
  the (w, min(u,v), max(u,v)) order was worked out by hand (listed below);
  this script asserts that an independent pure-Python Kruskal agrees before
  writing them.
* gnm_summaries.json: seeded G(n,m) graphs from the oracle generator with
  the SHA-256 of their directed edge list and of their forest, the forest
  weight and size -- pins the generator and the oracle's Kruskal together.

Run: python tests/golden/make_golden.py
"""
import hashlib
import json
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
from tests import _oracle as O  # noqa: E402

W32 = 0xFFFFFFFF
# (name, n, undirected edges (u, v, w), hand-derived forest as (min, max, w))
TINY = [
    ("triangle_equal", 3, [(0, 1, 5), (0, 2, 5), (1, 2, 5)], [(0, 1, 5), (0, 2, 5)]),
    ("path_decreasing", 4, [(0, 1, 3), (1, 2, 2), (2, 3, 1)], [(0, 1, 3), (1, 2, 2), (2, 3, 1)]),
    ("square_diag_equal", 4, [(0, 1, 1), (1, 2, 1), (2, 3, 1), (0, 3, 1), (0, 2, 1)],
     [(0, 1, 1), (0, 2, 1), (0, 3, 1)]),
    ("two_components_isolated", 6, [(0, 1, 4), (1, 2, 2), (0, 2, 3), (3, 4, 7)],
     [(0, 2, 3), (1, 2, 2), (3, 4, 7)]),
    ("star_hub", 7, [(0, 1, 9), (0, 2, 8), (0, 3, 7), (0, 4, 6), (0, 5, 5), (0, 6, 4),
                     (1, 2, 10), (2, 3, 10), (3, 4, 10), (4, 5, 10), (5, 6, 10), (1, 6, 10)],
     [(0, 1, 9), (0, 2, 8), (0, 3, 7), (0, 4, 6), (0, 5, 5), (0, 6, 4)]),
    ("no_edges", 3, [], []),
    ("single_edge", 2, [(0, 1, 254)], [(0, 1, 254)]),
    ("cycle4_equal", 4, [(0, 1, 1), (1, 2, 1), (2, 3, 1), (0, 3, 1)],
     [(0, 1, 1), (0, 3, 1), (1, 2, 1)]),
    ("extreme_weights", 3, [(0, 1, W32), (1, 2, 0), (0, 2, W32)], [(0, 1, W32), (1, 2, 0)]),
    ("path_increasing_long", 9, [(i, i + 1, i + 1) for i in range(8)] + [(0, 8, 100)],
     [(i, i + 1, i + 1) for i in range(8)]),
    ("complete5_ties", 5, [(u, v, 1 + ((u + v) % 2)) for u in range(5) for v in range(u + 1, 5)],
     [(0, 1, 2), (0, 2, 1), (0, 4, 1), (1, 3, 1)]),
    ("heavy_hub_light_ring", 5, [(0, 1, 50), (0, 2, 50), (0, 3, 50), (0, 4, 50),
                                 (1, 2, 1), (2, 3, 2), (3, 4, 3)],
     [(0, 1, 50), (1, 2, 1), (2, 3, 2), (3, 4, 3)]),
]

GNM = [(16, 40, 1), (1000, 3000, 2), (1 << 10, 1 << 13, 3), (1 << 12, 1 << 15, 4),
       (1 << 14, 1 << 17, 5), (1 << 16, 1 << 20, 6)]


def sha(a) -> str:
    return hashlib.sha256(a.tobytes()).hexdigest()


def main():
    tiny = []
    for name, n, und, forest in TINY:
        e = O.symmetric_from_undirected(und)
        py = sorted((min(u, v), max(u, v), w) for u, v, w in O.py_kruskal(e, n))
        assert py == sorted(forest), (name, py, forest)
        tiny.append({"name": name, "n": n, "edges": [list(t) for t in und],
                     "forest": [list(t) for t in sorted(forest)],
                     "weight": sum(w for _, _, w in forest)})
    with open(os.path.join(HERE, "tiny_graphs.json"), "w") as f:
        json.dump(tiny, f, indent=1)
    gnm = []
    for n, m, seed in GNM:
        e = O.gen_gnm(n, m, seed)
        mst, w = O.kruskal(e, n)
        gnm.append({"n": n, "m": m, "seed": seed, "max_weight": 254,
                    "edges_sha256": sha(e), "forest_sha256": sha(O.canon_keys(mst)),
                    "forest_size": int(len(mst)), "forest_weight": w})
    with open(os.path.join(HERE, "gnm_summaries.json"), "w") as f:
        json.dump(gnm, f, indent=1)
    print(f"wrote {len(tiny)} tiny graphs, {len(gnm)} G(n,m) summaries")


if __name__ == "__main__":
    main()
