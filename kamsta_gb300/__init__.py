"""kamsta_gb300 -- minimum spanning forests on one NVIDIA GB300.

Python mirror of KaMSTa's algorithm API (hybridMST namespace):

    boruvka(input_edges, config)         hybrid_boruvka.hpp:263-301
    filter_boruvka(input_edges, config)  hybrid_boruvka_edgefilter.hpp:420-462
    AlgorithmConfig / LocalPreprocessing / Compression
                                         algorithm_configurations.hpp:6-34

`input_edges` holds directed entries sorted by (src, dst) with both
directions of every edge (the reference's WEdgeList contract).  The result
is the minimum spanning forest under the (w, min, max) order as a WEDGE
array of (min, max, w) entries.  All compute runs in libkamsta_gpu.so on the
GPU; a missing library or a failing call raises, nothing falls back to CPU.
"""
from __future__ import annotations

import ctypes as C
import enum
from dataclasses import dataclass

import numpy as np

from . import _native
from ._native import (FLAG_DEDUPE_ALWAYS, FLAG_DEDUPE_NEVER, FLAG_SORT_OUTPUT, FLAG_TRACE,
                      FLAG_VALIDATE, WEDGE, WEDGE64, KamstaError, Stats, check, lib)

__all__ = ["LocalPreprocessing", "Compression", "AlgorithmConfig", "boruvka", "filter_boruvka",
           "boruvka_wedge64", "Context", "WEDGE", "WEDGE64", "KamstaError", "Stats",
           "as_wedges", "mst_weight", "version"]


class LocalPreprocessing(enum.IntEnum):
    NO_PREPROCESSING = 0
    MODIFIED_BORUVKA = 1
    REDUCE_EDGES_THEN_BORUVKA = 2


class Compression(enum.IntEnum):
    NO_COMPRESSION = 0
    SEVEN_BIT_DIFF_ENCODING = 1


@dataclass
class AlgorithmConfig:
    """AlgorithmConfig (algorithm_configurations.hpp:27-34) plus GPU knobs."""
    local_preprocessing: LocalPreprocessing = LocalPreprocessing.NO_PREPROCESSING
    compression: Compression = Compression.NO_COMPRESSION
    filter_threshold: int = 4
    validate: bool = False
    sort_output: bool = False
    dedupe: str = "auto"        # "auto" | "never" | "always"
    dedupe_ratio: int = 0
    trace: bool = False
    seed: int | None = None

    def to_c(self) -> _native.Cfg:
        c = _native.default_cfg()
        c.local_preprocessing = int(self.local_preprocessing)
        c.compression = int(self.compression)
        c.filter_threshold = int(self.filter_threshold)
        flags = 0
        if self.validate:
            flags |= FLAG_VALIDATE
        if self.sort_output:
            flags |= FLAG_SORT_OUTPUT
        if self.trace:
            flags |= FLAG_TRACE
        if self.dedupe == "never":
            flags |= FLAG_DEDUPE_NEVER
        elif self.dedupe == "always":
            flags |= FLAG_DEDUPE_ALWAYS
        c.flags = flags
        c.dedupe_ratio = int(self.dedupe_ratio)
        if self.seed is not None:
            c.seed = int(self.seed)
        return c


def version() -> str:
    return lib().kamsta_version().decode()


def as_wedges(edges) -> np.ndarray:
    """View/convert edges as a contiguous WEDGE array ((m,3) uint32 accepted)."""
    a = np.asarray(edges)
    if a.dtype == WEDGE:
        return np.ascontiguousarray(a)
    if a.ndim == 2 and a.shape[1] == 3:
        return np.ascontiguousarray(a.astype(np.uint32)).view(WEDGE).reshape(-1)
    if a.dtype.names and {"src", "dst", "w"} <= set(a.dtype.names):
        out = np.empty(len(a), WEDGE)
        out["src"], out["dst"], out["w"] = a["src"], a["dst"], a["w"]
        return out
    raise TypeError("edges must be a WEDGE array or an (m, 3) integer array")


def mst_weight(mst: np.ndarray) -> int:
    return int(mst["w"].astype(np.uint64).sum())


def _infer_n(e: np.ndarray) -> int:
    if len(e) == 0:
        return 0
    return int(max(int(e["src"].max()), int(e["dst"].max()))) + 1


def _solve(fn, input_edges, config, n, stats):
    e = as_wedges(input_edges)
    if n is None:
        n = _infer_n(e)
    cfg = (config or AlgorithmConfig()).to_c()
    out = np.empty(max(int(n), 1), WEDGE)
    cnt = C.c_uint64(0)
    st = Stats()
    check(fn(e.ctypes.data_as(C.c_void_p), len(e), int(n), C.byref(cfg),
             out.ctypes.data_as(C.c_void_p), C.byref(cnt), C.byref(st)))
    if stats is not None:
        stats.update(st.as_dict())
    return out[: cnt.value].copy()


def boruvka(input_edges, config: AlgorithmConfig | None = None, n: int | None = None,
            stats: dict | None = None) -> np.ndarray:
    """hybridMST::boruvka on the GPU (host buffers in, host buffers out)."""
    return _solve(lib().kamsta_mst_boruvka, input_edges, config, n, stats)


def filter_boruvka(input_edges, config: AlgorithmConfig | None = None, n: int | None = None,
                   stats: dict | None = None) -> np.ndarray:
    """hybridMST::filter_boruvka on the GPU (host buffers in, host buffers out)."""
    return _solve(lib().kamsta_mst_filter_boruvka, input_edges, config, n, stats)


def boruvka_wedge64(input_edges: np.ndarray, config: AlgorithmConfig | None = None,
                    n: int | None = None, stats: dict | None = None) -> np.ndarray:
    """boruvka over the reference's 24-byte WEdge layout."""
    e = np.ascontiguousarray(input_edges, dtype=WEDGE64)
    if n is None:
        n = int(max(e["src"].max(), e["dst"].max())) + 1 if len(e) else 0
    cfg = (config or AlgorithmConfig()).to_c()
    out = np.empty(max(int(n), 1), WEDGE64)
    cnt = C.c_uint64(0)
    st = Stats()
    check(lib().kamsta_mst_boruvka_wedge64(e.ctypes.data_as(C.c_void_p), len(e), int(n),
                                           C.byref(cfg), out.ctypes.data_as(C.c_void_p),
                                           C.byref(cnt), C.byref(st)))
    if stats is not None:
        stats.update(st.as_dict())
    return out[: cnt.value].copy()


class Context:
    """A solver context on one device: scratch pool + stream (kamsta_ctx).

    Device entry points take raw device pointers (e.g. torch tensor
    data_ptr()) and an optional cudaStream_t handle as an int.
    """

    def __init__(self, device: int = 0):
        h = C.c_void_p()
        check(lib().kamsta_ctx_create(int(device), C.byref(h)))
        self._h = h
        self.device = device

    @property
    def handle(self):
        return self._h

    def close(self):
        if self._h:
            lib().kamsta_ctx_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def pool_bytes(self) -> int:
        return int(lib().kamsta_ctx_pool_bytes(self._h))

    def trim(self):
        check(lib().kamsta_ctx_trim(self._h))

    def _dev(self, fn, d_edges: int, m: int, n: int, d_out: int, config, stream, stats):
        cfg = (config or AlgorithmConfig()).to_c()
        cnt = C.c_uint64(0)
        st = Stats()
        check(fn(self._h, C.c_void_p(d_edges), int(m), int(n), C.byref(cfg), C.c_void_p(d_out),
                 C.byref(cnt), C.byref(st), C.c_void_p(stream or 0)))
        if stats is not None:
            stats.update(st.as_dict())
        return int(cnt.value)

    def boruvka_dev(self, d_edges: int, m: int, n: int, d_out: int, config=None, stream=0,
                    stats: dict | None = None) -> int:
        """kamsta_mst_boruvka_dev; returns the number of forest edges."""
        return self._dev(lib().kamsta_mst_boruvka_dev, d_edges, m, n, d_out, config, stream, stats)

    def filter_boruvka_dev(self, d_edges: int, m: int, n: int, d_out: int, config=None,
                           stream=0, stats: dict | None = None) -> int:
        return self._dev(lib().kamsta_mst_filter_boruvka_dev, d_edges, m, n, d_out, config,
                         stream, stats)

    def gen_gnm_dev(self, n: int, m: int, seed: int, max_weight: int, d_out: int,
                    stream=0) -> int:
        """Device G(n,m) generator; d_out needs 2*m entries.  Returns 2*m."""
        cnt = C.c_uint64(0)
        check(lib().kamsta_gen_gnm_dev(self._h, int(n), int(m), int(seed), int(max_weight),
                                       C.c_void_p(d_out), C.byref(cnt), C.c_void_p(stream or 0)))
        return int(cnt.value)
