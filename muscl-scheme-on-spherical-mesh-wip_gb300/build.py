"""Builds the in-tree shared libraries of the GB300 MUSCL step.

* ``lib/libsplash_gb300.so`` — the product: host C++ (mesh, geometry,
  C ABI) + CUDA kernels for sm_103a.
* ``oracle/liboracle.so`` — the CPU restatement used as test oracle.
* ``oracle/_ref/ref_runner`` — the reference solver itself, compiled from
  its own sources when the reference checkout is present (fixture
  generation only).

Compilation runs the translation units in parallel; there is no cmake.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
REPO = PKG.parent
CSRC = PKG / "csrc"
LIBDIR = PKG / "lib"
OBJDIR = PKG / "_build"
INCLUDE = REPO / "include"
ORACLE = REPO / "oracle"
LIBNAME = "libsplash_gb300.so"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
CXXFLAGS = ["-std=c++17", "-O3", "-fPIC", "-fopenmp", "-ffp-contract=off", "-Wall",
            "-Wno-unknown-pragmas", "-fvisibility=hidden", "-fvisibility-inlines-hidden"]
# per-.cu extra flags: the FP64 path must not fuse multiply-adds (reference
# operand order); the mixed path may.
CU_FLAGS = {
    "step_fp64.cu": ["-fmad=false"],
    "adjoint.cu": ["-fmad=false"],
    "diagnostics.cu": ["-fmad=false"],
    "cfl_noalloc.cu": ["-fmad=false"],
    "step_mixed.cu": ["-fmad=true", "-prec-div=false", "-prec-sqrt=false", "-ftz=true"],
}


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found: the CUDA 13 toolkit is required to build splash_gb300")


def _cuda_home() -> Path:
    return Path(_nvcc()).resolve().parent.parent


def _run(cmd: list[str]) -> None:
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError("build step failed:\n" + " ".join(cmd) + "\n" + res.stdout + res.stderr)


def _newer(src: Path, dst: Path, deps: list[Path]) -> bool:
    if not dst.exists():
        return True
    t = dst.stat().st_mtime
    return any(p.stat().st_mtime > t for p in [src, *deps] if p.exists())


def build_library(verbose: bool = False, force: bool = False) -> Path:
    """Compiles lib/libsplash_gb300.so (sm_103a) and returns its path."""
    OBJDIR.mkdir(exist_ok=True)
    LIBDIR.mkdir(exist_ok=True)
    nvcc = _nvcc()
    cuda_inc = _cuda_home() / "include"
    headers = list(CSRC.glob("*.hpp")) + list(CSRC.glob("*.cuh")) + list(INCLUDE.glob("*.h"))
    jobs = []
    objs = []
    for src in sorted(CSRC.glob("*.cpp")):
        obj = OBJDIR / (src.stem + ".o")
        objs.append(obj)
        if force or _newer(src, obj, headers):
            jobs.append(["g++", *CXXFLAGS, f"-I{INCLUDE}", f"-I{CSRC}", f"-I{cuda_inc}",
                         "-c", str(src), "-o", str(obj)])
    for src in sorted(CSRC.glob("*.cu")):
        obj = OBJDIR / (src.stem + ".cu.o")
        objs.append(obj)
        if force or _newer(src, obj, headers):
            jobs.append([nvcc, *ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
                         "-Xcompiler", "-fvisibility=hidden",
                         *CU_FLAGS.get(src.name, []), f"-I{INCLUDE}", f"-I{CSRC}",
                         "-c", str(src), "-o", str(obj)])
    with cf.ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 4))) as ex:
        for cmd, fut in [(c, ex.submit(_run, c)) for c in jobs]:
            if verbose:
                print(" ".join(cmd), file=sys.stderr)
            fut.result()
    lib = LIBDIR / LIBNAME
    if force or jobs or not lib.exists():
        _run([nvcc, *ARCH, "-shared", "-o", str(lib), *map(str, objs),
              "-Xcompiler", "-fopenmp", "-lgomp"])
    return lib


def build_oracle(verbose: bool = False, force: bool = False) -> Path:
    """Compiles the CPU oracle oracle/liboracle.so (test infrastructure)."""
    src = ORACLE / "splash_oracle.cpp"
    out = ORACLE / "liboracle.so"
    if force or _newer(src, out, []):
        cmd = ["g++", "-std=c++17", "-O3", "-fPIC", "-fopenmp", "-ffp-contract=off", "-shared",
               str(src), "-o", str(out)]
        if verbose:
            print(" ".join(cmd), file=sys.stderr)
        _run(cmd)
    return out


def build_reference_runner(ref_root: str | Path | None = None, verbose: bool = False) -> Path | None:
    """Compiles the reference solver (oracle/_ref/ref_runner) from the
    reference checkout at ref_root (or $SPLASH_REFERENCE); returns None when
    neither names a checkout (fixture generation only: the tests use the
    committed fixtures)."""
    root = ref_root or os.environ.get("SPLASH_REFERENCE")
    if not root:
        return None
    ref = Path(root)
    if not (ref / "src" / "MUSCL_base" / "MUSCL_base.hpp").exists():
        return None
    cmd = ["make", "-s", "-C", str(ORACLE / "ref"), f"REF={ref}", f"-j{os.cpu_count() or 4}"]
    if verbose:
        print(" ".join(cmd), file=sys.stderr)
    _run(cmd)
    return ORACLE / "_ref" / "ref_runner"


if __name__ == "__main__":
    v = "-v" in sys.argv
    f = "--force" in sys.argv
    print(build_library(verbose=v, force=f))
    print(build_oracle(verbose=v, force=f))
    print(build_reference_runner(os.environ.get("SPLASH_REFERENCE"), verbose=v))
