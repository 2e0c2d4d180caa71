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
                    'int main(){printf("%zu %zu %zu %zu %zu %zu %zu %zu %zu %zu %zu %zu %zu %zu\\n", sizeof(kamsta_cfg),'
                    'sizeof(kamsta_stats), sizeof(kamsta_wedge), sizeof(kamsta_wedge64),'
                    'offsetof(kamsta_stats, trace_m), offsetof(kamsta_cfg, seed),'
                    'sizeof(kamsta_graph_desc), offsetof(kamsta_graph_desc, out),'
                    'sizeof(kamsta_batch_stats), sizeof(kamsta_server_cfg), sizeof(kamsta_request),'
                    'sizeof(kamsta_completion), sizeof(kamsta_cgraph), sizeof(kamsta_tuning));}\n')
    exe = tmp_path / "sz"
    subprocess.run(["gcc", "-I", os.path.join(ROOT, "include"), str(prog), "-o", str(exe)],
                   check=True)
    got = [int(x) for x in subprocess.run([str(exe)], capture_output=True, text=True,
                                          check=True).stdout.split()]
    assert got == [C.sizeof(_native.Cfg), C.sizeof(_native.Stats), _native.WEDGE.itemsize,
                   _native.WEDGE64.itemsize, _native.Stats.trace_m.offset,
                   _native.Cfg.seed.offset, C.sizeof(_native.GraphDesc),
                   _native.GraphDesc.out.offset, C.sizeof(_native.BatchStats),
                   C.sizeof(_native.ServerCfg), C.sizeof(_native.Request),
                   C.sizeof(_native.Completion), C.sizeof(_native.CGraph),
                   C.sizeof(_native.Tuning)]


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


def test_cpp_adapter_compiles_against_reference_shapes(kamsta, tmp_path):
    """include/kamsta_gpu.hpp accepts WEdge/AlgorithmConfig-shaped types
    (definitions.hpp:66-84, algorithm_configurations.hpp:27-34) and links
    against the library (no GPU call is made)."""
    prog = tmp_path / "adapter.cpp"
    prog.write_text(r'''
#include <cstdint>
#include <cstdio>
#include <vector>
#include "kamsta_gpu.hpp"
enum class LocalPreprocessing { NO_PREPROCESSING = 0, MODIFIED_BORUVKA = 1 };
enum class Compression { NO_COMPRESSION = 0 };
struct AlgorithmConfig {
  LocalPreprocessing local_preprocessing = LocalPreprocessing::MODIFIED_BORUVKA;
  Compression compression = Compression::NO_COMPRESSION;
  std::size_t filter_threshold = 4;
};
struct WEdge {
  uint64_t src_, dst_; uint32_t weight_;
  WEdge(uint64_t s, uint64_t d, uint32_t w) : src_(s), dst_(d), weight_(w) {}
  uint64_t get_src() const { return src_; }
  uint64_t get_dst() const { return dst_; }
  uint32_t get_weight() const { return weight_; }
};
int main(int argc, char**) {
  AlgorithmConfig cfg;
  kamsta_cfg k = kamsta_gpu::to_cfg(cfg);
  std::printf("%d %d %llu\n", k.local_preprocessing, k.compression,
              (unsigned long long)k.filter_threshold);
  if (argc > 5) {  // never taken: instantiate the solve paths
    std::vector<WEdge> e{{0, 1, 3}, {1, 0, 3}};
    auto a = kamsta_gpu::boruvka(e, cfg);
    auto b = kamsta_gpu::filter_boruvka(e, cfg);
    return static_cast<int>(a.size() + b.size());
  }
  return 0;
}
''')
    exe = tmp_path / "adapter"
    libdir = os.path.join(ROOT, "kamsta_gb300")
    subprocess.run(["g++", "-std=c++17", "-I", os.path.join(ROOT, "include"), str(prog),
                    "-L", libdir, "-lkamsta_gpu", f"-Wl,-rpath,{libdir}", "-o", str(exe)],
                   check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split()
    assert out == ["1", "0", "4"]


def test_status_codes_and_flags_match_header(kamsta):
    """Every KAMSTA_E_* / KAMSTA_FLAG_* value in the header equals the
    ctypes mirror's constant of the same name."""
    from kamsta_gb300 import _native
    src = open(HEADER).read()
    defs = dict((k, int(v, 0)) for k, v in
                re.findall(r"#define\s+KAMSTA_((?:E|FLAG)_[A-Z0-9_]+)\s+(0x[0-9a-fA-F]+|\d+)", src))
    assert "E_CANCELLED" in defs and "FLAG_VALIDATE" in defs
    for name, value in defs.items():
        assert getattr(_native, name) == value, name
        if name.startswith("E_"):
            assert _native.STATUS_NAMES[value] == name
