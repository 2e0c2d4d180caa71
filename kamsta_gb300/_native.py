"""ctypes binding of libkamsta_gpu.so (the C ABI in include/kamsta_gpu.h).

The library is loaded from the package directory only.  There is no CPU
fallback: if the library is missing or a call fails, an exception is raised.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libkamsta_gpu.so")

# status codes (kamsta_gpu.h)
(OK, E_INPUT, E_OOM, E_CUDA, E_NOCONVERGE, E_UNSUPPORTED, E_BUDGET, E_NOTREADY,
 E_CANCELLED) = range(9)
STATUS_NAMES = {0: "OK", 1: "E_INPUT", 2: "E_OOM", 3: "E_CUDA", 4: "E_NOCONVERGE",
                5: "E_UNSUPPORTED", 6: "E_BUDGET", 7: "E_NOTREADY", 8: "E_CANCELLED"}

FLAG_VALIDATE = 0x1
FLAG_SORT_OUTPUT = 0x2
FLAG_DEDUPE_NEVER = 0x4
FLAG_DEDUPE_ALWAYS = 0x8
FLAG_TRACE = 0x10
FLAG_FILTER = 0x20
DISTANCE_RANDOM, DISTANCE_EUCLIDEAN, DISTANCE_SQUARED_EUCLIDEAN = 0, 1, 2
LOAD_SYMMETRIZE = 0x1
TRACE_MAX = 128
PHASES = ["plan", "first_pass", "round_edges", "round_verts", "class_pass", "finalize", "emit",
          "dedupe"]

# numpy views of the edge layouts
WEDGE = np.dtype([("src", "<u4"), ("dst", "<u4"), ("w", "<u4")])          # kamsta_wedge
WEDGE64 = np.dtype([("src", "<u8"), ("dst", "<u8"), ("w", "<u4"), ("pad_", "<u4")])


class KamstaError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__(f"{STATUS_NAMES.get(status, status)}: {message}")
        self.status = status


class Cfg(C.Structure):
    _fields_ = [("local_preprocessing", C.c_int32), ("compression", C.c_int32),
                ("filter_threshold", C.c_uint64), ("flags", C.c_uint32),
                ("dedupe_ratio", C.c_uint32), ("seed", C.c_uint64),
                ("seg_items_per_thread", C.c_uint32), ("items_per_thread", C.c_uint32)]


class Stats(C.Structure):
    _fields_ = [("num_mst_edges", C.c_uint64), ("total_weight", C.c_uint64),
                ("rounds", C.c_uint32), ("levels", C.c_uint32),
                ("dedupe_passes", C.c_uint32), ("gpu_launches", C.c_uint32),
                ("device_ms", C.c_double), ("alg_bytes", C.c_uint64),
                ("trace_len", C.c_uint32), ("row_scans", C.c_uint32),
                ("trace_m", C.c_uint64 * TRACE_MAX), ("trace_n", C.c_uint64 * TRACE_MAX),
                ("phase_ms", C.c_double * len(PHASES)), ("phase_bytes", C.c_uint64 * len(PHASES)),
                ("phase_launches", C.c_uint32 * len(PHASES))]

    def as_dict(self) -> dict:
        skip = ("trace_m", "trace_n", "phase_ms", "phase_bytes", "phase_launches")
        d = {k: getattr(self, k) for k, _ in self._fields_ if k not in skip}
        d["trace"] = [(int(self.trace_m[i]), int(self.trace_n[i])) for i in range(self.trace_len)]
        d["phases"] = {name: {"ms": float(self.phase_ms[i]), "bytes": int(self.phase_bytes[i]),
                              "launches": int(self.phase_launches[i])}
                       for i, name in enumerate(PHASES)}
        return d


class GraphDesc(C.Structure):
    _fields_ = [("edges", C.c_void_p), ("m_directed", C.c_uint64), ("n", C.c_uint32),
                ("status", C.c_int32), ("out", C.c_void_p), ("out_count", C.c_uint64),
                ("total_weight", C.c_uint64)]


class BatchStats(C.Structure):
    _fields_ = [("graphs", C.c_uint32), ("waves", C.c_uint32), ("gpu_launches", C.c_uint32),
                ("pad_", C.c_uint32), ("entries", C.c_uint64), ("vertices", C.c_uint64),
                ("forest_edges", C.c_uint64), ("device_ms", C.c_double),
                ("solve_ms", C.c_double)]

    def as_dict(self) -> dict:
        return {k: getattr(self, k) for k, _ in self._fields_ if k != "pad_"}


class ServerCfg(C.Structure):
    _fields_ = [("budget_bytes", C.c_uint64), ("max_batch", C.c_uint32),
                ("workers", C.c_uint32), ("solver", Cfg), ("small_threads", C.c_uint32),
                ("small_max_n", C.c_uint32)]


class Request(C.Structure):
    _fields_ = [("d_edges", C.c_void_p), ("m_directed", C.c_uint64), ("n", C.c_uint32),
                ("pad_", C.c_uint32), ("d_out", C.c_void_p), ("user_tag", C.c_uint64)]


class Completion(C.Structure):
    _fields_ = [("ticket", C.c_uint64), ("user_tag", C.c_uint64), ("status", C.c_int32),
                ("batch_size", C.c_uint32), ("out_count", C.c_uint64),
                ("total_weight", C.c_uint64), ("submit_us", C.c_double),
                ("start_us", C.c_double), ("finish_us", C.c_double)]


class CGraph(C.Structure):
    _fields_ = [("m_directed", C.c_uint64), ("n", C.c_uint32), ("chunk_edges", C.c_uint32),
                ("num_chunks", C.c_uint64), ("data_bytes", C.c_uint64),
                ("chunk_offset", C.c_void_p), ("chunk_first", C.c_void_p), ("data", C.c_void_p)]


class Tuning(C.Structure):
    _fields_ = [("small_threads", C.c_uint32), ("small_max_n", C.c_uint32),
                ("threads_ms", C.c_double * 3), ("cutoff_ms", C.c_double * 4)]

    def as_dict(self) -> dict:
        return {"small_threads": self.small_threads, "small_max_n": self.small_max_n,
                "threads_ms": dict(zip((256, 512, 1024), list(self.threads_ms))),
                "cutoff_ms": dict(zip((4096, 8192, 16384, 32768), list(self.cutoff_ms)))}


class TileTuning(C.Structure):
    _fields_ = [("items_per_thread", C.c_uint32), ("seg_items_per_thread", C.c_uint32),
                ("ms", C.c_double * 6)]
    PAIRS = ("6x2", "8x2", "12x2", "6x4", "8x4", "12x4")

    def as_dict(self) -> dict:
        return {"items_per_thread": self.items_per_thread,
                "seg_items_per_thread": self.seg_items_per_thread,
                "ms": dict(zip(self.PAIRS, list(self.ms)))}


_lib = None

# Every symbol declared in include/kamsta_gpu.h, with its ctypes signature.
P = C.c_void_p
U32, U64, I32 = C.c_uint32, C.c_uint64, C.c_int
SIGNATURES = {
    "kamsta_cfg_default": (I32, [C.POINTER(Cfg)]),
    "kamsta_version": (C.c_char_p, []),
    "kamsta_last_error": (C.c_char_p, []),
    "kamsta_ctx_create": (I32, [C.c_int, C.POINTER(P)]),
    "kamsta_ctx_destroy": (I32, [P]),
    "kamsta_ctx_trim": (I32, [P]),
    "kamsta_ctx_pool_bytes": (U64, [P]),
    "kamsta_ctx_set_memory_limit": (I32, [P, U64]),
    "kamsta_mst_boruvka": (I32, [P, U64, U32, C.POINTER(Cfg), P, C.POINTER(U64), C.POINTER(Stats)]),
    "kamsta_mst_filter_boruvka": (I32, [P, U64, U32, C.POINTER(Cfg), P, C.POINTER(U64),
                                        C.POINTER(Stats)]),
    "kamsta_mst_boruvka_wedge64": (I32, [P, U64, U64, C.POINTER(Cfg), P, C.POINTER(U64),
                                         C.POINTER(Stats)]),
    "kamsta_mst_boruvka_dev": (I32, [P, P, U64, U32, C.POINTER(Cfg), P, C.POINTER(U64),
                                     C.POINTER(Stats), P]),
    "kamsta_mst_filter_boruvka_dev": (I32, [P, P, U64, U32, C.POINTER(Cfg), P, C.POINTER(U64),
                                            C.POINTER(Stats), P]),
    "kamsta_server_cfg_default": (I32, [C.POINTER(ServerCfg)]),
    "kamsta_server_create": (I32, [C.c_int, C.POINTER(ServerCfg), C.POINTER(P)]),
    "kamsta_server_submit": (I32, [P, C.POINTER(Request), C.POINTER(U64)]),
    "kamsta_server_poll": (I32, [P, C.POINTER(Completion), U32, C.POINTER(U32), U32]),
    "kamsta_server_cancel": (I32, [P, U64]),
    "kamsta_server_stats": (I32, [P, C.POINTER(U64), C.POINTER(U64), C.POINTER(U64),
                                  C.POINTER(U64)]),
    "kamsta_server_memory": (I32, [P, C.POINTER(U64), C.POINTER(U64)]),
    "kamsta_server_destroy": (I32, [P]),
    "kamsta_encode_7bit": (I32, [P, U64, U32, P, P, P, U64, C.POINTER(U64)]),
    "kamsta_decode_7bit_dev": (I32, [P, C.POINTER(CGraph), P, P]),
    "kamsta_mst_boruvka_7bit_dev": (I32, [P, C.POINTER(CGraph), C.POINTER(Cfg), P,
                                          C.POINTER(U64), C.POINTER(Stats), P]),
    "kamsta_mst_boruvka_7bit": (I32, [C.POINTER(CGraph), C.POINTER(Cfg), P, C.POINTER(U64),
                                      C.POINTER(Stats)]),
    "kamsta_wedge9_capacity": (I32, [C.POINTER(C.c_char_p), U32, U32, C.POINTER(U64)]),
    "kamsta_load_wedge9_dev": (I32, [P, C.POINTER(C.c_char_p), U32, U32, P, U64,
                                     C.POINTER(U64), C.POINTER(U32), P]),
    "kamsta_mtx_header": (I32, [C.c_char_p, C.POINTER(U64), C.POINTER(U64), C.POINTER(U64)]),
    "kamsta_load_mtx_dev": (I32, [P, C.c_char_p, U64, U32, P, U64, C.POINTER(U64),
                                  C.POINTER(U32), P]),
    "kamsta_gen_gnm_dev": (I32, [P, U32, U64, U64, U32, P, C.POINTER(U64), P]),
    "kamsta_gen_rgg2d_dev": (I32, [P, U32, C.c_double, U64, U32, U32, P, U64, C.POINTER(U64),
                                   P]),
    "kamsta_gen_rhg_dev": (I32, [P, U32, C.c_double, C.c_double, U64, U32, P, U64,
                                 C.POINTER(U64), P]),
    "kamsta_gen_grid_dev": (I32, [P, U32, U32, U32, C.c_double, C.c_int, U64, U32, P, U64,
                                  C.POINTER(U64), P]),
    "kamsta_gen_rgg3d_dev": (I32, [P, U32, C.c_double, U64, U32, U32, P, U64, C.POINTER(U64),
                                   P]),
    "kamsta_gen_rmat_dev": (I32, [P, U32, U64, C.c_double, C.c_double, C.c_double, U64, U32, P,
                                  U64, C.POINTER(U64), P]),
    "kamsta_mst_boruvka_noalloc": (I32, [P, U64, U32, P, C.POINTER(U64), C.POINTER(U64), P]),
    "kamsta_mst_batch_dev": (I32, [P, C.POINTER(GraphDesc), U32, C.POINTER(Cfg), U64,
                                   C.POINTER(BatchStats), P]),
    "kamsta_batch_autotune": (I32, [P, C.POINTER(GraphDesc), U32, C.POINTER(Cfg),
                                    C.POINTER(Tuning), P]),
    "kamsta_ctx_set_tuning": (I32, [P, C.POINTER(Tuning)]),
    "kamsta_autotune_tiles": (I32, [P, P, U64, U32, P, P, C.POINTER(TileTuning), P]),
    "kamsta_ctx_set_tiles": (I32, [P, U32, U32]),
    "kamsta_mst_batch": (I32, [P, C.POINTER(GraphDesc), U32, C.POINTER(Cfg), U64,
                               C.POINTER(BatchStats)]),
}


def lib():
    """Load libkamsta_gpu.so (raises if it has not been built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError(f"{LIB_PATH} is missing: run kamsta_gb300.build.build() first")
        L = C.CDLL(LIB_PATH)
        for name, (res, args) in SIGNATURES.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def check(status: int) -> None:
    if status != OK:
        msg = lib().kamsta_last_error()
        raise KamstaError(status, msg.decode() if msg else "")


def default_cfg() -> Cfg:
    c = Cfg()
    check(lib().kamsta_cfg_default(C.byref(c)))
    return c
