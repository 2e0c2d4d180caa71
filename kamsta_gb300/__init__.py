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
import os
from dataclasses import dataclass

import numpy as np

from . import _native
from ._native import (FLAG_DEDUPE_ALWAYS, FLAG_DEDUPE_NEVER, FLAG_FILTER, FLAG_SORT_OUTPUT,
                      FLAG_TRACE, FLAG_VALIDATE, WEDGE, WEDGE64, BatchStats, GraphDesc,
                      KamstaError, Stats, check, lib)

__all__ = ["LocalPreprocessing", "Compression", "AlgorithmConfig", "boruvka", "filter_boruvka",
           "boruvka_wedge64", "Context", "WEDGE", "WEDGE64", "KamstaError", "Stats",
           "as_wedges", "mst_weight", "version", "batch", "GraphDesc", "BatchStats", "Server", "Compressed",
           "boruvka_7bit"]


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
    filter: bool = False        # batch / serving: filter_boruvka instead of boruvka
    items_per_thread: int = 0   # first-pass tile: 6, 8 or 12 entries per thread (0 = 6)
    seg_items_per_thread: int = 0  # list-pass tile: 2, 4 or 8 records per thread (0 = 2)

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
        if self.filter:
            flags |= FLAG_FILTER
        if self.dedupe == "never":
            flags |= FLAG_DEDUPE_NEVER
        elif self.dedupe == "always":
            flags |= FLAG_DEDUPE_ALWAYS
        c.flags = flags
        c.dedupe_ratio = int(self.dedupe_ratio)
        c.items_per_thread = int(self.items_per_thread)
        c.seg_items_per_thread = int(self.seg_items_per_thread)
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


def mtx_header(path) -> tuple[int, int, int]:
    """(rows, cols, stored entries) of a MatrixMarket coordinate file (host
    only, kamsta_mtx_header)."""
    r, c, e = C.c_uint64(0), C.c_uint64(0), C.c_uint64(0)
    check(lib().kamsta_mtx_header(os.fsencode(path), C.byref(r), C.byref(c), C.byref(e)))
    return int(r.value), int(c.value), int(e.value)


class Compressed:
    """A 7-bit varint difference-encoded edge list (kamsta_cgraph) in host
    memory: per chunk a raw first edge and a byte offset, then varint(src -
    prev_src), varint(dst), varint(w) per edge (the reference's
    SEVEN_BIT_DIFF_ENCODING container)."""

    def __init__(self, edges, n: int, chunk_edges: int = 2048, pinned: bool = False):
        """pinned: the compressed bytes go to page-locked host memory (torch),
        so that their copy to the device runs at the host link's rate."""
        e = as_wedges(edges)
        self.m, self.n, self.chunk_edges = len(e), int(n), int(chunk_edges)
        self.num_chunks = (self.m + self.chunk_edges - 1) // self.chunk_edges
        self.offset = np.zeros(self.num_chunks + 1, np.uint64)
        self.first = np.empty(max(self.num_chunks, 1), WEDGE)
        nb = C.c_uint64(0)
        L = lib()
        ep = e.ctypes.data if len(e) else None
        check(L.kamsta_encode_7bit(ep, self.m, self.chunk_edges, self.offset.ctypes.data, None,
                                   None, 0, C.byref(nb)))
        if pinned:
            import torch
            self._pin = torch.empty(max(nb.value, 1), dtype=torch.uint8, pin_memory=True)
            self.data = self._pin.numpy()
        else:
            self.data = np.empty(max(nb.value, 1), np.uint8)
        check(L.kamsta_encode_7bit(ep, self.m, self.chunk_edges, self.offset.ctypes.data,
                                   self.first.ctypes.data, self.data.ctypes.data, nb.value,
                                   C.byref(nb)))
        self.data_bytes = int(nb.value)

    def c_struct(self, offset_ptr=None, first_ptr=None, data_ptr=None) -> _native.CGraph:
        return _native.CGraph(self.m, self.n, self.chunk_edges, self.num_chunks,
                              self.data_bytes,
                              offset_ptr if offset_ptr is not None else self.offset.ctypes.data,
                              first_ptr if first_ptr is not None else self.first.ctypes.data,
                              data_ptr if data_ptr is not None else self.data.ctypes.data)

    def total_bytes(self) -> int:
        return self.data_bytes + 8 * (self.num_chunks + 1) + 12 * self.num_chunks


def boruvka_7bit(cg: "Compressed", config: AlgorithmConfig | None = None,
                 stats: dict | None = None) -> np.ndarray:
    """kamsta_mst_boruvka_7bit: solve from compressed host memory."""
    g = cg.c_struct()
    cfg = (config or AlgorithmConfig()).to_c()
    out = np.empty(max(cg.n, 1), WEDGE)
    cnt = C.c_uint64(0)
    st = Stats()
    check(lib().kamsta_mst_boruvka_7bit(C.byref(g), C.byref(cfg), out.ctypes.data_as(C.c_void_p),
                                        C.byref(cnt), C.byref(st)))
    if stats is not None:
        stats.update(st.as_dict())
    return out[: cnt.value].copy()


def batch(graphs, config: AlgorithmConfig | None = None, budget_bytes: int = 0,
          stats: dict | None = None, context: "Context | None" = None):
    """kamsta_mst_batch over host arrays: `graphs` is a list of (edges, n).

    Returns one (status, forest) pair per graph; each forest is sorted by
    (src, dst) and equals boruvka() on that graph alone.
    """
    es = [as_wedges(e) for e, _ in graphs]
    outs = [np.empty(max(int(n), 1), WEDGE) for _, n in graphs]
    descs = (GraphDesc * max(len(graphs), 1))()
    for i, ((_, n), e, o) in enumerate(zip(graphs, es, outs)):
        descs[i].edges = e.ctypes.data if len(e) else None
        descs[i].m_directed = len(e)
        descs[i].n = int(n)
        descs[i].out = o.ctypes.data
    cfg = (config or AlgorithmConfig()).to_c()
    st = BatchStats()
    h = context.handle if context is not None else None
    check(lib().kamsta_mst_batch(h, descs, len(graphs), C.byref(cfg), int(budget_bytes),
                                 C.byref(st)))
    if stats is not None:
        stats.update(st.as_dict())
    return [(int(descs[i].status), outs[i][: descs[i].out_count].copy())
            for i in range(len(graphs))]


class Server:
    """Continuous-batching MST request loop on one device (kamsta_server).

    submit() takes device pointers (edges already written); poll() returns
    finished jobs as dicts with ticket, tag, status, out_count, total_weight,
    batch_size and the submit / start / finish times in microseconds.
    """

    def __init__(self, device: int = 0, budget_bytes: int = 0, max_batch: int = 0,
                 workers: int = 2, config: AlgorithmConfig | None = None,
                 tuning: dict | None = None):
        c = _native.ServerCfg()
        check(lib().kamsta_server_cfg_default(C.byref(c)))
        if budget_bytes:
            c.budget_bytes = int(budget_bytes)
        if max_batch:
            c.max_batch = int(max_batch)
        c.workers = int(workers)
        c.solver = (config or AlgorithmConfig()).to_c()
        if tuning:
            c.small_threads = int(tuning.get("small_threads", 0))
            c.small_max_n = int(tuning.get("small_max_n", 0))
        h = C.c_void_p()
        check(lib().kamsta_server_create(int(device), C.byref(c), C.byref(h)))
        self._h = h
        self._buf = (_native.Completion * 4096)()

    def submit(self, d_edges: int, m_directed: int, n: int, d_out: int, tag: int = 0) -> int:
        r = _native.Request(C.c_void_p(d_edges or None), int(m_directed), int(n), 0,
                            C.c_void_p(d_out or None), int(tag))
        t = C.c_uint64(0)
        check(lib().kamsta_server_submit(self._h, C.byref(r), C.byref(t)))
        return int(t.value)

    def poll(self, timeout_us: int = 0) -> list:
        cnt = C.c_uint32(0)
        s = lib().kamsta_server_poll(self._h, self._buf, len(self._buf), C.byref(cnt),
                                     int(timeout_us))
        if s == _native.E_NOTREADY:
            return []
        check(s)
        return [{"ticket": c.ticket, "tag": c.user_tag, "status": c.status,
                 "batch_size": c.batch_size, "out_count": c.out_count,
                 "total_weight": c.total_weight, "submit_us": c.submit_us,
                 "start_us": c.start_us, "finish_us": c.finish_us}
                for c in self._buf[: cnt.value]]

    def cancel(self, ticket: int) -> bool:
        """Withdraw a queued job (it completes with E_CANCELLED); False if it
        is already in a wave or finished."""
        s = lib().kamsta_server_cancel(self._h, int(ticket))
        if s == _native.E_NOTREADY:
            return False
        check(s)
        return True

    def stats(self) -> dict:
        q, f, b, w = C.c_uint64(), C.c_uint64(), C.c_uint64(), C.c_uint64()
        check(lib().kamsta_server_stats(self._h, C.byref(q), C.byref(f), C.byref(b), C.byref(w)))
        return {"queued": q.value, "in_flight": f.value, "bytes_in_use": b.value,
                "waves": w.value}

    def memory(self) -> dict:
        """Per-worker device-memory limit and the largest amount any worker's
        context held during a wave so far."""
        lim, peak = C.c_uint64(), C.c_uint64()
        check(lib().kamsta_server_memory(self._h, C.byref(lim), C.byref(peak)))
        return {"worker_limit": lim.value, "peak_worker_bytes": peak.value}

    def close(self):
        if self._h:
            check(lib().kamsta_server_destroy(self._h))
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


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

    def set_memory_limit(self, nbytes: int) -> None:
        """Cap the device bytes this context may have in use (0 = no cap);
        a call over the cap raises E_OOM and the context stays usable."""
        check(lib().kamsta_ctx_set_memory_limit(self._h, int(nbytes)))

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

    def batch_dev(self, descs, config=None, budget_bytes: int = 0, stream=0,
                  stats: dict | None = None):
        """kamsta_mst_batch_dev over a ctypes GraphDesc array (device pointers)."""
        cfg = (config or AlgorithmConfig()).to_c()
        st = BatchStats()
        check(lib().kamsta_mst_batch_dev(self._h, descs, len(descs), C.byref(cfg),
                                         int(budget_bytes), C.byref(st), C.c_void_p(stream or 0)))
        if stats is not None:
            stats.update(st.as_dict())
        return descs

    def gen_gnm_dev(self, n: int, m: int, seed: int, max_weight: int, d_out: int,
                    stream=0) -> int:
        """Device G(n,m) generator; d_out needs 2*m entries.  Returns 2*m."""
        cnt = C.c_uint64(0)
        check(lib().kamsta_gen_gnm_dev(self._h, int(n), int(m), int(seed), int(max_weight),
                                       C.c_void_p(d_out), C.byref(cnt), C.c_void_p(stream or 0)))
        return int(cnt.value)

    def gen_rgg2d_dev(self, n: int, radius: float, seed: int, max_weight: int, d_out: int = 0,
                      capacity: int = 0, stream=0, distance: int = 0) -> int:
        """Device 2-D random geometric graph.  With d_out == 0 it only counts;
        returns the number of directed entries.  distance: 0 random weights,
        1 Euclidean, 2 squared Euclidean (KAMSTA_DISTANCE_*)."""
        cnt = C.c_uint64(0)
        check(lib().kamsta_gen_rgg2d_dev(self._h, int(n), float(radius), int(seed),
                                         int(max_weight), int(distance), C.c_void_p(d_out or 0),
                                         int(capacity), C.byref(cnt), C.c_void_p(stream or 0)))
        return int(cnt.value)

    def gen_rhg_dev(self, n: int, gamma: float, avg_degree: float, seed: int, max_weight: int,
                    d_out: int = 0, capacity: int = 0, stream=0) -> int:
        """Device threshold random hyperbolic graph.  With d_out == 0 it only
        counts; returns the number of directed entries."""
        cnt = C.c_uint64(0)
        check(lib().kamsta_gen_rhg_dev(self._h, int(n), float(gamma), float(avg_degree),
                                       int(seed), int(max_weight), C.c_void_p(d_out or 0),
                                       int(capacity), C.byref(cnt), C.c_void_p(stream or 0)))
        return int(cnt.value)

    def gen_grid_dev(self, x: int, y: int, z: int = 1, p: float = 1.0, periodic: bool = True,
                     seed: int = 1, max_weight: int = 254, d_out: int = 0, capacity: int = 0,
                     stream=0) -> int:
        """Device lattice x * y * z (z = 1: the 2-D grid), +-1 steps along
        each axis, wrapping when `periodic`, each edge kept with probability
        p.  With d_out == 0 it only counts; returns the directed entries."""
        cnt = C.c_uint64(0)
        check(lib().kamsta_gen_grid_dev(self._h, int(x), int(y), int(z), float(p), int(periodic),
                                        int(seed), int(max_weight), C.c_void_p(d_out or 0),
                                        int(capacity), C.byref(cnt), C.c_void_p(stream or 0)))
        return int(cnt.value)

    def gen_rgg3d_dev(self, n: int, radius: float, seed: int, max_weight: int = 254,
                      d_out: int = 0, capacity: int = 0, stream=0, distance: int = 0) -> int:
        """Device 3-D random geometric graph in the unit cube.  With
        d_out == 0 it only counts; returns the directed entries.  distance
        as in gen_rgg2d_dev."""
        cnt = C.c_uint64(0)
        check(lib().kamsta_gen_rgg3d_dev(self._h, int(n), float(radius), int(seed),
                                         int(max_weight), int(distance), C.c_void_p(d_out or 0),
                                         int(capacity), C.byref(cnt), C.c_void_p(stream or 0)))
        return int(cnt.value)

    def gen_rmat_dev(self, log_n: int, samples: int, seed: int, a: float = 0.57,
                     b: float = 0.19, c: float = 0.19, max_weight: int = 254, d_out: int = 0,
                     capacity: int = 0, stream=0) -> int:
        """Device R-MAT graph on 2^log_n vertices from `samples` samples.
        With d_out == 0 it only counts; returns the directed entries."""
        cnt = C.c_uint64(0)
        check(lib().kamsta_gen_rmat_dev(self._h, int(log_n), int(samples), float(a), float(b),
                                        float(c), int(seed), int(max_weight),
                                        C.c_void_p(d_out or 0), int(capacity), C.byref(cnt),
                                        C.c_void_p(stream or 0)))
        return int(cnt.value)

    def load_mtx_dev(self, path, seed: int = 1, max_weight: int = 254, stream=0):
        """A MatrixMarket coordinate file as solver input on the device (the
        reference's unweighted input; hash weights in [1, max_weight]).
        Returns (edges tensor (m, 3) int32 on cuda, m_directed, n)."""
        import torch
        _, _, entries = mtx_header(path)
        cap = max(2 * entries, 1)
        d = torch.empty((cap, 3), dtype=torch.int32, device="cuda")
        m, n = C.c_uint64(0), C.c_uint32(0)
        check(lib().kamsta_load_mtx_dev(self._h, os.fsencode(path), int(seed), int(max_weight),
                                        C.c_void_p(d.data_ptr()), cap, C.byref(m), C.byref(n),
                                        C.c_void_p(stream or 0)))
        return d[: m.value], int(m.value), int(n.value)

    def load_wedge9_dev(self, paths, symmetrize: bool = True, stream=0):
        """Stream the reference's 9-byte binary edge files to the device.
        Returns (edges tensor (m, 3) int32 on cuda, m_directed, n)."""
        import torch
        if isinstance(paths, (str, bytes)):
            paths = [paths]
        arr = (C.c_char_p * len(paths))(*[p.encode() if isinstance(p, str) else p
                                          for p in paths])
        flags = _native.LOAD_SYMMETRIZE if symmetrize else 0
        cap = C.c_uint64(0)
        check(lib().kamsta_wedge9_capacity(arr, len(paths), flags, C.byref(cap)))
        out = torch.empty((max(cap.value, 1), 3), dtype=torch.int32, device="cuda")
        m, n = C.c_uint64(0), C.c_uint32(0)
        check(lib().kamsta_load_wedge9_dev(self._h, arr, len(paths), flags,
                                           C.c_void_p(out.data_ptr()), cap.value, C.byref(m),
                                           C.byref(n), C.c_void_p(stream or 0)))
        return out[: m.value], int(m.value), int(n.value)

    def _cgraph_dev(self, cg: "Compressed"):
        import torch
        off = torch.from_numpy(cg.offset.view(np.int64)).cuda()
        first = torch.from_numpy(cg.first.view(np.uint32).view(np.int32).copy()).cuda()
        data = torch.from_numpy(cg.data.view(np.int8).copy()).cuda()
        torch.cuda.synchronize()
        return (off, first, data), cg.c_struct(off.data_ptr(), first.data_ptr(), data.data_ptr())

    def decode_7bit_dev(self, cg: "Compressed", d_out: int, stream=0):
        """Decode a compressed graph (copied to the device first) into d_out."""
        keep, g = self._cgraph_dev(cg)
        check(lib().kamsta_decode_7bit_dev(self._h, C.byref(g), C.c_void_p(d_out),
                                           C.c_void_p(stream or 0)))
        return keep

    def boruvka_7bit_dev(self, g, d_out: int, config=None, stream=0,
                         stats: dict | None = None) -> int:
        """kamsta_mst_boruvka_7bit_dev; g is a CGraph of device pointers."""
        cfg = (config or AlgorithmConfig()).to_c()
        cnt = C.c_uint64(0)
        st = Stats()
        check(lib().kamsta_mst_boruvka_7bit_dev(self._h, C.byref(g), C.byref(cfg),
                                                C.c_void_p(d_out), C.byref(cnt), C.byref(st),
                                                C.c_void_p(stream or 0)))
        if stats is not None:
            stats.update(st.as_dict())
        return int(cnt.value)

    def batch_autotune(self, descs, config=None, stream=0) -> dict:
        """kamsta_batch_autotune on a sample of graphs (GraphDesc array)."""
        cfg = (config or AlgorithmConfig()).to_c()
        t = _native.Tuning()
        check(lib().kamsta_batch_autotune(self._h, descs, len(descs), C.byref(cfg), C.byref(t),
                                          C.c_void_p(stream or 0)))
        return t.as_dict()

    def autotune_tiles(self, d_edges: int, m: int, n: int, d_out: int, config=None,
                       stream=0) -> dict:
        """kamsta_autotune_tiles: times every tile pair on this input and
        keeps the fastest in the context (used when the config leaves the
        tiles at 0)."""
        cfg = (config or AlgorithmConfig()).to_c()
        t = _native.TileTuning()
        check(lib().kamsta_autotune_tiles(self._h, C.c_void_p(d_edges), int(m), int(n),
                                          C.byref(cfg), C.c_void_p(d_out), C.byref(t),
                                          C.c_void_p(stream or 0)))
        return t.as_dict()

    def set_tiles(self, items_per_thread: int = 0, seg_items_per_thread: int = 0):
        check(lib().kamsta_ctx_set_tiles(self._h, int(items_per_thread),
                                         int(seg_items_per_thread)))

    def set_tuning(self, small_threads: int = 0, small_max_n: int = 0):
        t = _native.Tuning()
        t.small_threads, t.small_max_n = int(small_threads), int(small_max_n)
        check(lib().kamsta_ctx_set_tuning(self._h, C.byref(t)))
