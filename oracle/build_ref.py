"""Recipe: compile the reference's own code into oracle/_ref/ (test infrastructure).

Two artefacts, both built straight from the reference checkout (read-only, never copied
into the repository):
  libref_host.so    the reference host scene code - Loader, Scene, Mesh (tinyobjloader),
                    Camera, HDRLoader and the vendored RadeonRays BVH build/flatten - plus
                    oracle/ref_host_harness.cpp, a C-ABI wrapper of ours.
  libref_shader.so  the reference GLSL path tracer (shaders/renderer.glsl and
                    shaders/common/*.glsl) compiled as C++ through oracle/glsl_shim.h
                    (see oracle/ref_shader_gen.py), used to pin the CPU restatement.

Flags follow the reference's MSVC /fp:precise build: no floating-point contraction.
Without a reference checkout this recipe does nothing (exit 0): the GPU host never has one,
and nothing there needs these files.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
OUT = HERE / "_ref"
# the reference checkout: LAVAFRAME_REFERENCE, else a `reference` directory beside this repository
REF = Path(os.environ.get("LAVAFRAME_REFERENCE", HERE.parent.parent / "reference"))


def _run(cmd):
    r = subprocess.run([str(c) for c in cmd], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"failed: {' '.join(map(str, cmd))}\n{r.stdout}\n{r.stderr}")


def _stale(out: Path, deps) -> bool:
    if not out.exists():
        return True
    t = out.stat().st_mtime
    return any(Path(d).stat().st_mtime > t for d in deps if Path(d).exists())


def build_host(force=False) -> Path:
    lf = REF / "LavaFrame"
    rr = lf / "thirdparty" / "RadeonRays"
    srcs = [lf / f for f in ("Scene.cpp", "Mesh.cpp", "Loader.cpp", "Camera.cpp", "hdrloader.cpp", "Texture.cpp")]
    srcs += [rr / f for f in ("bbox.cpp", "bvh.cpp", "split_bvh.cpp", "bvh_translator.cpp")]
    srcs.append(HERE / "ref_host_harness.cpp")
    out = OUT / "libref_host.so"
    if not force and not _stale(out, srcs + [HERE / "ref_compat.h"]):
        return out
    inc = [lf, rr, lf / "thirdparty" / "gl3w", lf / "thirdparty" / "stb", lf / "thirdparty" / "imgui",
           lf / "thirdparty" / "imguizmo"]
    obj_dir = OUT / "obj"
    obj_dir.mkdir(parents=True, exist_ok=True)
    flags = ["-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-fno-fast-math", "-w", "-include",
             HERE / "ref_compat.h"] + [x for d in inc for x in ("-I", d)]
    objs = []
    jobs = []
    for s in srcs:
        o = obj_dir / (s.stem + ".o")
        objs.append(o)
        jobs.append(["g++", *flags, "-c", s, "-o", o])
    with cf.ThreadPoolExecutor(max_workers=os.cpu_count() or 4) as ex:
        list(ex.map(_run, jobs))
    _run(["g++", "-shared", "-o", out, *objs])
    return out


def build_shader(force=False):
    gen = HERE / "ref_shader_gen.py"
    if not gen.exists():
        return None
    r = subprocess.run([sys.executable, str(gen), "--out", str(OUT)] + (["--force"] if force else []),
                       capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"shader build failed:\n{r.stdout}\n{r.stderr}")
    return OUT / "libref_shader.so"


def main():
    force = "--force" in sys.argv
    if not (REF / "LavaFrame" / "Scene.cpp").exists():
        print("no reference checkout; skipping")
        return 0
    OUT.mkdir(exist_ok=True)
    with cf.ThreadPoolExecutor(max_workers=2) as ex:
        a = ex.submit(build_host, force)
        b = ex.submit(build_shader, force)
        print(a.result(), b.result())
    return 0


if __name__ == "__main__":
    sys.exit(main())
