"""CPU tests of the C ABI boundary: the library loads, exports every symbol
declared in include/kamsta_gpu.h, and the ctypes mirror matches the C
layouts.  No compute call is made (no GPU here)."""
import ctypes as C
import os
import re
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "kamsta_gpu.h")


def declared_symbols():
    src = open(HEADER).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(kamsta_[a-z0-9_]+)\s*\(", src)))


def test_header_declares_entry_points():
    syms = declared_symbols()
    for s in ("kamsta_mst_boruvka", "kamsta_mst_filter_boruvka", "kamsta_mst_boruvka_dev",
              "kamsta_mst_filter_boruvka_dev", "kamsta_ctx_create", "kamsta_last_error"):
        assert s in syms


def test_library_exports_every_declared_symbol(kamsta):
    from kamsta_gb300 import _native
    L = C.CDLL(_native.LIB_PATH)
    missing = [s for s in declared_symbols() if not hasattr(L, s)]
    assert not missing, missing
    # and the ctypes signature table covers them all
    assert set(declared_symbols()) <= set(_native.SIGNATURES)


def test_struct_layouts_match_header(kamsta, tmp_path):
    from kamsta_gb300 import _native
    prog = tmp_path / "sz.c"
    prog.write_text('#include <stdio.h>\n#include <stddef.h>\n#include "kamsta_gpu.h"\n'
                    'int main(){printf("%zu %zu %zu %zu %zu %zu\\n", sizeof(kamsta_cfg),'
                    'sizeof(kamsta_stats), sizeof(kamsta_wedge), sizeof(kamsta_wedge64),'
                    'offsetof(kamsta_stats, trace_m), offsetof(kamsta_cfg, seed));}\n')
    exe = tmp_path / "sz"
    subprocess.run(["gcc", "-I", os.path.join(ROOT, "include"), str(prog), "-o", str(exe)],
                   check=True)
    got = [int(x) for x in subprocess.run([str(exe)], capture_output=True, text=True,
                                          check=True).stdout.split()]
    assert got == [C.sizeof(_native.Cfg), C.sizeof(_native.Stats), _native.WEDGE.itemsize,
                   _native.WEDGE64.itemsize, _native.Stats.trace_m.offset,
                   _native.Cfg.seed.offset]


def test_cfg_default_mirrors_reference_algorithm_config(kamsta):
    """AlgorithmConfig defaults (algorithm_configurations.hpp:31-33)."""
    c = kamsta._native.default_cfg()
    assert c.local_preprocessing == kamsta.LocalPreprocessing.NO_PREPROCESSING
    assert c.compression == kamsta.Compression.NO_COMPRESSION
    assert c.filter_threshold == 4


def test_config_flags_roundtrip(kamsta):
    cfg = kamsta.AlgorithmConfig(local_preprocessing=kamsta.LocalPreprocessing.MODIFIED_BORUVKA,
                                 validate=True, sort_output=True, dedupe="never", trace=True)
    c = cfg.to_c()
    assert c.local_preprocessing == 1
    assert c.flags == (kamsta.FLAG_VALIDATE | kamsta.FLAG_SORT_OUTPUT |
                       kamsta.FLAG_DEDUPE_NEVER | kamsta.FLAG_TRACE)


def test_as_wedges_conversions(kamsta):
    a = np.array([[0, 1, 5], [1, 0, 5]], dtype=np.int64)
    w = kamsta.as_wedges(a)
    assert w.dtype == kamsta.WEDGE and list(w["w"]) == [5, 5]
    with pytest.raises(TypeError):
        kamsta.as_wedges(np.zeros((3, 2)))


def test_version_string(kamsta):
    assert "sm_103a" in kamsta.version()
