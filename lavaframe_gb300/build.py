"""Builds the native libraries in-tree.

  lavaframe_gb300/liblfcore.so   product: host scene layer + CUDA kernels (sm_103a) + C ABI
  oracle/liblfo.so               CPU oracle (test infrastructure only)
  oracle/_ref/*                  reference code compiled from a local reference checkout
                                 (only when one is available; never shipped)

Host C++ is compiled with -ffp-contract=off and device code with --fmad=false: the BVH
build and the path-tracing arithmetic must not be contracted into fused multiply-adds,
otherwise results stop being bit-identical between the CPU oracle and the GPU.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parent.parent
PKG = ROOT / "lavaframe_gb300"
CSRC = PKG / "csrc"
BUILD = PKG / "_build"
LIB = PKG / "liblfcore.so"
ORACLE = ROOT / "oracle"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
CXXFLAGS = ["-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-fno-fast-math", "-Wall", "-Wno-unused-function"]
NVCCFLAGS = ARCH + ["-O3", "--fmad=false", "-prec-div=true", "-prec-sqrt=true", "-ftz=false", "-lineinfo",
                    "-std=c++17", "-Xcompiler", "-fPIC,-ffp-contract=off"]


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found")


def _newest(paths) -> float:
    return max((p.stat().st_mtime for p in paths if p.exists()), default=0.0)


def _run(cmd, verbose):
    if verbose:
        print(" ".join(str(c) for c in cmd), flush=True)
    r = subprocess.run([str(c) for c in cmd], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"command failed ({r.returncode}): {' '.join(str(c) for c in cmd)}\n{r.stdout}\n{r.stderr}")
    return r


def _compile_all(jobs, verbose):
    with cf.ThreadPoolExecutor(max_workers=max(2, os.cpu_count() or 2)) as ex:
        futs = [ex.submit(_run, j, verbose) for j in jobs]
        for f in futs:
            f.result()


def build_core(verbose: bool = False, force: bool = False) -> Path:
    BUILD.mkdir(exist_ok=True)
    headers = list(CSRC.rglob("*.h")) + list(CSRC.rglob("*.cuh")) + list((ROOT / "include").glob("*.h"))
    hstamp = _newest(headers)
    nvcc = _nvcc()
    objs, jobs = [], []
    for src in sorted((CSRC / "host").glob("*.cpp")):
        obj = BUILD / (src.stem + ".o")
        objs.append(obj)
        if force or not obj.exists() or obj.stat().st_mtime < max(src.stat().st_mtime, hstamp):
            jobs.append(["g++", *CXXFLAGS, "-I", ROOT / "include", "-c", src, "-o", obj])
    for src in sorted((CSRC / "device").glob("*.cu")):
        obj = BUILD / (src.stem + ".cu.o")
        objs.append(obj)
        if force or not obj.exists() or obj.stat().st_mtime < max(src.stat().st_mtime, hstamp):
            jobs.append([nvcc, *NVCCFLAGS, "-I", ROOT / "include", "-c", src, "-o", obj])
    _compile_all(jobs, verbose)
    if force or jobs or not LIB.exists() or LIB.stat().st_mtime < _newest(objs):
        tmp = LIB.with_suffix(".so.tmp")
        _run([nvcc, *ARCH, "-shared", "-o", tmp, *objs, "-lpthread"], verbose)
        os.replace(tmp, LIB)
    return LIB


def build_oracle(verbose: bool = False, force: bool = False) -> Path:
    out = ORACLE / "liblfo.so"
    srcs = sorted(ORACLE.glob("lfo*.cpp"))
    deps = srcs + list(ORACLE.glob("*.h")) + [CSRC / "lf_contract.h", CSRC / "lf_vec.h"]
    if force or not out.exists() or out.stat().st_mtime < _newest(deps):
        tmp = out.with_suffix(".so.tmp")
        _run(["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-ffp-contract=off", "-fno-fast-math", "-pthread",
              "-I", CSRC, "-o", tmp, *srcs], verbose)
        os.replace(tmp, out)
    return out


def build_reference(verbose: bool = False, force: bool = False):
    """Compiles the reference's own host code and shaders into oracle/_ref when a reference
    checkout is available (LAVAFRAME_REFERENCE, else a `reference` directory beside the repository)."""
    script = ORACLE / "build_ref.py"
    if not script.exists():
        return None
    r = subprocess.run([sys.executable, str(script)] + (["--force"] if force else []), capture_output=True, text=True)
    if verbose:
        print(r.stdout, r.stderr)
    if r.returncode != 0:
        raise RuntimeError(f"reference build failed:\n{r.stdout}\n{r.stderr}")
    return ORACLE / "_ref"


def build_all(verbose: bool = False, force: bool = False):
    with cf.ThreadPoolExecutor(max_workers=3) as ex:
        f1 = ex.submit(build_core, verbose, force)
        f2 = ex.submit(build_oracle, verbose, force)
        f3 = ex.submit(build_reference, verbose, force)
        return f1.result(), f2.result(), f3.result()


if __name__ == "__main__":
    print(build_all(verbose="-v" in sys.argv, force="--force" in sys.argv))
