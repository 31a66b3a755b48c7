"""Build recipe for libkf (the CUDA path tracer) and the CPU oracle.

Everything is compiled in-tree, without cmake:
  kuafu_gb300/libkf.so     nvcc, sm_103a only, one object per translation unit (parallel)
  oracle/liboracle.so      g++ -O2 -ffp-contract=off (test infrastructure)
  kuafu_gb300/_build/      object files

Usage: python -m kuafu_gb300.build [--verbose] [--ptxas]
"""
from __future__ import annotations

import argparse
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
BUILD = PKG / "_build"
LIB = PKG / "libkf.so"
ORACLE_DIR = ROOT / "oracle"
ORACLE_LIB = ORACLE_DIR / "liboracle.so"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]

# Translation units and their extra flags. The path-tracing kernels keep
# -fmad=false so every float expression rounds as written (bit parity with the
# oracle); the tensor-core kernels are free to contract.
SOURCES = [
    ("kf_api.cu", ["-fmad=false"]),
    ("kf_scene.cu", ["-fmad=false"]),
    ("kf_render.cu", ["-fmad=false"]),
    ("kf_bvh.cu", ["-fmad=false"]),
    ("kf_wavefront.cu", ["-fmad=false"]),
    ("kf_conv.cu", []),
    ("kf_denoise.cu", []),
    ("kf_autotune.cu", []),
    ("kf_mesh.cpp", []),
    ("kf_obj.cpp", []),
]


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found: libkf needs the CUDA toolkit (there is no CPU fallback)")


def _run(cmd: list[str], verbose: bool) -> str:
    if verbose:
        print(" ".join(cmd), flush=True)
    p = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if p.returncode != 0:
        raise RuntimeError(f"command failed ({p.returncode}): {' '.join(cmd)}\n{p.stdout}")
    return p.stdout


def _stale(target: Path, deps: list[Path]) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps if d.exists())


def build_libkf(verbose: bool = False, ptxas: bool = False, force: bool = False) -> Path:
    nvcc = _nvcc()
    BUILD.mkdir(exist_ok=True)
    headers = list(CSRC.glob("*.h")) + list(CSRC.glob("*.cuh")) + list((ROOT / "include").glob("*.h"))
    objs = []
    jobs = []
    for name, extra in SOURCES:
        src = CSRC / name
        obj = BUILD / (name + ".o")
        objs.append(obj)
        if force or ptxas or _stale(obj, [src] + headers):
            cmd = [nvcc, *ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-ffp-contract=off",
                   "-Xcompiler", "-fvisibility=hidden", "-I", str(ROOT / "include"), *extra, "-c", str(src),
                   "-o", str(obj)]
            if name.endswith(".cpp"):
                cmd[1:1] = ["-x", "cu"]
            if ptxas and name.endswith(".cu"):
                cmd += ["-Xptxas", "-v"]
            jobs.append(cmd)
    if jobs:
        with cf.ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
            outs = list(ex.map(lambda c: _run(c, verbose), jobs))
        if ptxas:
            for o in outs:
                print(o)
    if jobs or not LIB.exists():
        _run([nvcc, *ARCH, "-shared", "-o", str(LIB), *map(str, objs), "-lcudart"], verbose)
    return LIB


EXAMPLE_SRC = ROOT / "examples" / "cornell_facade.cpp"
EXAMPLE_BIN = BUILD / "cornell_facade"


def build_example(verbose: bool = False, force: bool = False) -> Path:
    """The C++ facade example (include/kuafu_gb300/kuafu.hpp over libkf)."""
    BUILD.mkdir(exist_ok=True)
    deps = [EXAMPLE_SRC, ROOT / "include" / "kuafu_gb300" / "kuafu.hpp", ROOT / "include" / "kf.h", LIB]
    if force or _stale(EXAMPLE_BIN, deps):
        cxx = os.environ.get("CXX", "g++")
        _run([cxx, "-std=c++17", "-O2", "-I", str(ROOT / "include"), "-o", str(EXAMPLE_BIN), str(EXAMPLE_SRC),
              "-L", str(PKG), "-lkf", f"-Wl,-rpath,{PKG}"], verbose)
    return EXAMPLE_BIN


def build_oracle(verbose: bool = False, force: bool = False) -> Path:
    src = ORACLE_DIR / "kf_oracle.cpp"
    deps = [src, ORACLE_DIR / "kf_oracle.h", ROOT / "include" / "kf_types.h"]
    if force or _stale(ORACLE_LIB, deps):
        cxx = os.environ.get("CXX", "g++")
        _run([cxx, "-std=c++17", "-O2", "-ffp-contract=off", "-fPIC", "-shared", "-pthread", "-o", str(ORACLE_LIB),
              str(src)], verbose)
    return ORACLE_LIB


def main(argv=None) -> int:
    ap = argparse.ArgumentParser(description=__doc__)
    ap.add_argument("--verbose", action="store_true")
    ap.add_argument("--ptxas", action="store_true", help="print register / spill reports")
    ap.add_argument("--force", action="store_true")
    a = ap.parse_args(argv)
    build_oracle(a.verbose, a.force)
    build_libkf(a.verbose, a.ptxas, a.force)
    build_example(a.verbose, a.force)
    print(f"built {LIB}, {ORACLE_LIB} and {EXAMPLE_BIN}")
    return 0


if __name__ == "__main__":
    sys.exit(main())
