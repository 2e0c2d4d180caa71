/*
 * oracle.h -- CPU test infrastructure for the GB300 MSF solver.
 *
 * THIS IS THE ORACLE, NOT THE PRODUCT.  Only tests/, __graft_entry__.smoke()
 * and bench.py's CPU-baseline / reference arm may load it.  The product path
 * (kamsta_gb300, libkamsta_gpu.so) never links or calls anything here.
 *
 * Contents:
 *   oracle_kruskal          -- known-answer MSF: Kruskal under the
 *                              (w, src, dst) order over the both-directions
 *                              input, restating the reference checker
 *                              include/algorithms/base_case_mst_algos.hpp:91-112
 *                              with union-find include/datastructures/union_find.hpp:9-32.
 *   oracle_boruvka_filter   -- OpenMP restatement of the reference's
 *                              single-rank local filter-Boruvka
 *                              (local_mst_respecting_cut_edges.hpp:101-302 and
 *                              the mst_utils_*.hpp round primitives); the timed
 *                              "reference CPU" baseline (kind "port").
 *   oracle_gen_gnm          -- seeded G(n,m) generator; bit-identical to the
 *                              device generator kamsta_gen_gnm_dev.
 *   oracle_gen_rgg2d        -- seeded 2-D random geometric graph; bit-identical
 *                              to kamsta_gen_rgg2d_dev.
 *   oracle_gen_rhg          -- seeded threshold random hyperbolic graph;
 *                              bit-identical to kamsta_gen_rhg_dev.
 *   oracle_gen_grid         -- 2-D / 3-D lattice (gen_grid_rmat.cpp);
 *                              bit-identical to kamsta_gen_grid_dev.
 *   oracle_gen_rgg3d        -- seeded 3-D random geometric graph;
 *                              bit-identical to kamsta_gen_rgg3d_dev.
 *   oracle_gen_rmat         -- seeded R-MAT graph; bit-identical to
 *                              kamsta_gen_rmat_dev.
 *
 * Parity status: the reference ships no golden vectors (its only test,
 * tests/test_sets.sh, checks the MSF weight against this same Kruskal).
 * Kruskal is pinned by hand-checked tiny graphs in tests/golden/.
 */
#ifndef KAMSTA_ORACLE_H
#define KAMSTA_ORACLE_H
#include <stdint.h>

#include "../include/kamsta_gpu.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Kruskal MSF.  out: capacity >= n entries.  Returns 0 on success. */
int oracle_kruskal(const kamsta_wedge* edges, uint64_t m_directed, uint32_t n,
                   kamsta_wedge* out, uint64_t* out_count,
                   uint64_t* total_weight);

/* Restated reference local filter-Boruvka on `threads` OpenMP threads
 * (0 = all).  out: capacity >= n entries.  Per-phase counters go to
 * rounds_out (may be NULL). */
int oracle_boruvka_filter(const kamsta_wedge* edges, uint64_t m_directed,
                          uint32_t n, int threads, kamsta_wedge* out,
                          uint64_t* out_count, uint64_t* total_weight,
                          uint32_t* rounds_out);

/* Seeded G(n,m): the first m distinct unordered pairs {u != v} of the
 * candidate stream, weights uniform in [1, max_weight], both directions,
 * sorted by (src, dst).  out: capacity 2*m.  Returns 0, or 1 if m exceeds
 * n(n-1)/2. */
int oracle_gen_gnm(uint32_t n, uint64_t m, uint64_t seed, uint32_t max_weight,
                   kamsta_wedge* out, uint64_t* m_directed_out);

/* Seeded 2-D random geometric graph (unit square, integer coordinates,
 * radius in [0, 1]; `distance` a weight rule as in kamsta_gen_rgg2d_dev);
 * definition in oracle.cpp, bit-identical to the device generator
 * kamsta_gen_rgg2d_dev.  *m_directed_out receives the number of
 * directed entries; returns 0, 2 if it exceeds `capacity` (nothing written),
 * 1 on bad arguments. */
int oracle_gen_rgg2d(uint32_t n, double radius, uint64_t seed, uint32_t max_weight,
                     uint32_t distance, kamsta_wedge* out, uint64_t capacity,
                     uint64_t* m_directed_out);

/* Seeded threshold random hyperbolic graph (power-law exponent gamma > 2,
 * target average degree); definition in oracle.cpp, bit-identical to the
 * device generator kamsta_gen_rhg_dev on the same machine.  Same return
 * convention as oracle_gen_rgg2d. */
int oracle_gen_rhg(uint32_t n, double gamma, double avg_degree, uint64_t seed,
                   uint32_t max_weight, kamsta_wedge* out, uint64_t capacity,
                   uint64_t* m_directed_out);

/* Lattice X x Y x Z (Z = 1: 2-D), +-1 steps along each axis, wrapping when
 * `periodic`, each edge kept with probability p.  Return convention as
 * oracle_gen_rgg2d. */
int oracle_gen_grid(uint32_t x, uint32_t y, uint32_t z, double p, int periodic, uint64_t seed,
                    uint32_t max_weight, kamsta_wedge* out, uint64_t capacity,
                    uint64_t* m_directed_out);

/* Seeded 3-D random geometric graph in the unit cube.  Return convention as
 * oracle_gen_rgg2d. */
int oracle_gen_rgg3d(uint32_t n, double radius, uint64_t seed, uint32_t max_weight,
                     uint32_t distance, kamsta_wedge* out, uint64_t capacity,
                     uint64_t* m_directed_out);

/* Seeded R-MAT graph on 2^log_n vertices from `samples` samples with
 * quadrant probabilities a, b, c (d = 1 - a - b - c).  Return convention as
 * oracle_gen_rgg2d. */
int oracle_gen_rmat(uint32_t log_n, uint64_t samples, double a, double b, double c,
                    uint64_t seed, uint32_t max_weight, kamsta_wedge* out, uint64_t capacity,
                    uint64_t* m_directed_out);

/* Number of OpenMP threads the oracle uses when threads == 0. */
int oracle_max_threads(void);

#ifdef __cplusplus
}
#endif
#endif
