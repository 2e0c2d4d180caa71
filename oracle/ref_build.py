"""Build recipe for the oracle's reference build (test infrastructure).

Compiles KaMSTa's own single-rank hot path -- its headers, unchanged, driven
by oracle/ref_driver.cpp -- into oracle/_ref/libkamsta_ref.so with g++ and
OpenMP.  The MPI / parlay / KaGen-interface / IPS4o names the headers use come
from oracle/ref_shim/ (the submodules that would provide them are empty).

Two steps, so that the build also works where the reference's source tree is
not mounted:
  1. amalgamate: oracle/ref_driver.cpp with every #include that resolves
     inside the reference tree (include/, external/) expanded in place, once
     per header; system and shim includes stay #include lines.  The result,
     oracle/_ref/ref_amalgam.cpp, is a build product (git-ignored, like the
     .so) and is written only where the reference tree exists;
  2. compile oracle/_ref/ref_amalgam.cpp -I oracle/ref_shim.
Nothing here is part of the product library.
"""
import os
import re
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT_DIR = os.path.join(HERE, "_ref")
AMALGAM = os.path.join(OUT_DIR, "ref_amalgam.cpp")
LIB = os.path.join(OUT_DIR, "libkamsta_ref.so")
SHIM = os.path.join(HERE, "ref_shim")
DRIVER = os.path.join(HERE, "ref_driver.cpp")
REF_ROOT = os.environ.get("KAMSTA_REFERENCE_ROOT", "/root/reference")
_INC = re.compile(r'^\s*#\s*include\s*([<"])([^>"]+)[>"]')


def _ref_dirs():
    return [os.path.join(REF_ROOT, "include"), os.path.join(REF_ROOT, "external")]


def _resolve(name, quote, cur_dir):
    """Path of a header inside the reference tree, or None (system / shim)."""
    cands = ([cur_dir] if quote == '"' and cur_dir else []) + _ref_dirs()
    for d in cands:
        p = os.path.normpath(os.path.join(d, name))
        if p.startswith(os.path.normpath(REF_ROOT) + os.sep) and os.path.isfile(p):
            return p
    return None


def amalgamate() -> str:
    seen = set()
    out = []

    def emit(path, is_ref):
        cur_dir = os.path.dirname(path)
        rel = os.path.relpath(path, REF_ROOT) if is_ref else os.path.basename(path)
        out.append(f'#line 1 "{rel}"\n')
        with open(path, encoding="utf-8") as f:
            for lineno, line in enumerate(f, 1):
                if is_ref and re.match(r"^\s*#\s*pragma\s+once", line):
                    out.append("\n")
                    continue
                m = _INC.match(line)
                if m:
                    p = _resolve(m.group(2), m.group(1), cur_dir)
                    if p is not None:
                        if p not in seen:
                            seen.add(p)
                            emit(p, True)
                            out.append(f'#line {lineno + 1} "{rel}"\n')
                        else:
                            out.append("\n")
                        continue
                out.append(line)

    emit(DRIVER, False)
    os.makedirs(OUT_DIR, exist_ok=True)
    tmp = AMALGAM + ".tmp"
    with open(tmp, "w", encoding="utf-8") as f:
        f.write("// Generated by oracle/ref_build.py from the reference's sources and\n"
                "// oracle/ref_driver.cpp.  Build product; not tracked.\n")
        f.writelines(out)
    os.replace(tmp, AMALGAM)
    return AMALGAM


def available() -> bool:
    return os.path.isdir(os.path.join(REF_ROOT, "include")) or os.path.isfile(AMALGAM)


def build(force: bool = False, verbose: bool = False) -> str:
    """Returns the path of libkamsta_ref.so; raises FileNotFoundError when
    neither the reference tree nor a carried amalgam is present."""
    have_ref = os.path.isdir(os.path.join(REF_ROOT, "include"))
    if have_ref:
        deps = [DRIVER] + [os.path.join(r, f) for r, _, fs in os.walk(SHIM) for f in fs]
        if force or not os.path.exists(AMALGAM) or any(
                os.path.getmtime(d) > os.path.getmtime(AMALGAM) for d in deps):
            amalgamate()
    elif not os.path.isfile(AMALGAM):
        raise FileNotFoundError("reference build: neither the reference tree nor "
                                "oracle/_ref/ref_amalgam.cpp is present")
    shim_files = [os.path.join(r, f) for r, _, fs in os.walk(SHIM) for f in fs]
    if not force and os.path.exists(LIB):
        t = os.path.getmtime(LIB)
        if all(os.path.getmtime(d) <= t for d in [AMALGAM] + shim_files):
            return LIB
    # the reference's own build defines NDEBUG USE_ASSERTIONS and
    # PARLAY_OPENMP at -O3 (CMakeLists.txt:41-43); -march=native and -mcx16
    # are left out so that the same recipe builds on x86-64 and aarch64
    cmd = ["g++", "-O3", "-std=c++17", "-fopenmp", "-fPIC", "-shared", "-DNDEBUG",
           "-DUSE_ASSERTIONS", "-DPARLAY_OPENMP", "-w", "-I", SHIM, "-o", LIB + ".tmp", AMALGAM]
    if verbose:
        print(" ".join(cmd), file=sys.stderr)
    subprocess.run(cmd, check=True)
    os.replace(LIB + ".tmp", LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
