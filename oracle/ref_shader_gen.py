"""Recipe (test infrastructure): compile the reference GLSL path tracer for the CPU.

Reads shaders/renderer.glsl from the reference checkout, expands its `#include` lines the way
LavaFrame's ShaderInclude::load does (ShaderIncludes.h:83-135), and rewrites the few GLSL
constructs C++ spells differently - nothing else:
  - `#version` is dropped; `uniform`, top-level `in`/`out` qualifiers are dropped;
  - `inout T x` parameters become `T& x`, `in T x` parameters `T x`;
  - float literals get an `f` suffix (GLSL literals are single precision);
  - `mat3(m)` becomes `mat3_of(m)`, `.xyzw` of a fetched texel is dropped;
  - the local `State`/`LightSampleRec`/`BsdfSampleRec` records are value-initialised (the
    GLSL leaves them undefined; zero is the definition the oracle and the GPU path use).
Each combination of the preprocessor switches TiledRenderer injects (ENVMAP, LIGHTS, RR with
RR_DEPTH, CONSTANT_BG; TiledRenderer.cpp:78-91) becomes one C++ struct whose members are the
shader's uniforms and globals and whose member functions are the shader's functions.
shaders/postprocess.glsl, the display pass, goes through the same rewriting into one more
struct driven once per output pixel (refsh_postprocess). glsl_shim.h supplies the GLSL types
and built-ins. Output goes to oracle/_ref/ only.
"""
from __future__ import annotations

import argparse
import concurrent.futures as cf
import os
import re
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
# the reference checkout: LAVAFRAME_REFERENCE, else a `reference` directory beside this repository
REF = Path(os.environ.get("LAVAFRAME_REFERENCE", HERE.parent.parent / "reference"))
SHADERS = REF / "shaders"
CSRC = HERE.parent / "lavaframe_gb300" / "csrc"


def expand(path: Path, seen=None) -> str:
    out = []
    for line in path.read_text().splitlines():
        m = re.match(r"\s*#include\s+(\S+)", line)
        if m:
            out.append(expand(SHADERS / m.group(1)))
        else:
            out.append(line)
    return "\n".join(out)


FLOAT_LIT = re.compile(r"(?<![\w.])(\d+\.\d*(?:[eE][+-]?\d+)?|\.\d+(?:[eE][+-]?\d+)?)(?![\w.])")


def to_cpp(src: str) -> str:
    src = re.sub(r"^\s*#version.*$", "", src, flags=re.M)
    src = re.sub(r"\buniform\s+", "", src)
    src = re.sub(r"^\s*out\s+", "", src, flags=re.M)
    src = re.sub(r"^\s*in\s+", "", src, flags=re.M)
    src = re.sub(r"\binout\s+(\w+)\s+(\w+)", r"\1& \2", src)
    src = re.sub(r"([(,]\s*)in\s+(\w+)\s+(\w+)", r"\1\2 \3", src)
    src = FLOAT_LIT.sub(lambda m: m.group(1) + "f", src)
    src = re.sub(r"\bmat3\(", "mat3_of(", src)
    src = src.replace(".xyzw", "")
    src = re.sub(r"^(\s*)(State|LightSampleRec|BsdfSampleRec)\s+(\w+)\s*;", r"\1\2 \3{};", src, flags=re.M)
    return src


SWITCHES = ["ENVMAP", "LIGHTS", "RR", "CONSTANT_BG"]
DEFINED = ["PI", "TWO_PI", "INFINITY", "EPS", "QUAD_LIGHT", "SPHERE_LIGHT", "DISTANT_LIGHT", "RR_DEPTH"] + SWITCHES


def variant_source(body: str, mask: int) -> str:
    lines = ["#include \"glsl_shim.h\"", "#include \"ref_shader_harness.h\"", "#undef INFINITY", "namespace glsl {"]
    for bit, name in enumerate(SWITCHES):
        if mask & (1 << bit):
            lines.append(f"#define {name}")
    lines.append("#define RR_DEPTH rrDepthValue")
    lines.append(f"struct RefShader{mask} {{")
    lines.append("int rrDepthValue;")
    lines.append(body)
    lines.append("};")
    lines += [f"#undef {d}" for d in DEFINED]
    lines.append("}")
    lines.append(f'extern "C" int refsh_render_v{mask}(const lfo_view* v, const lfo_params* p, int first, int n, '
                 f'float* accum, float* paths, int threads) {{ return refsh::render<glsl::RefShader{mask}>(v, p, first, n, '
                 f'accum, paths, threads); }}')
    return "\n".join(lines) + "\n"


def dispatcher() -> str:
    decls = "\n".join(f'extern "C" int refsh_render_v{m}(const lfo_view*, const lfo_params*, int, int, float*, float*, int);'
                      for m in range(16))
    table = ", ".join(f"refsh_render_v{m}" for m in range(16))
    return f"""#include "ref_shader_harness.h"
{decls}
// Renders with the shader variant TiledRenderer would compile for these options.
extern "C" int refsh_render(const lfo_view* v, const lfo_params* p, int first, int n, float* accum, float* paths,
                            int threads)
{{
    typedef int (*Fn)(const lfo_view*, const lfo_params*, int, int, float*, float*, int);
    static const Fn table[16] = {{{table}}};
    int mask = 0;
    if (p->use_env_map && v->env_rgb && v->env_width > 0) mask |= 1;
    if (v->num_lights > 0) mask |= 2;
    if (p->enable_rr) mask |= 4;
    if (p->use_constant_bg) mask |= 8;
    return table[mask](v, p, first, n, accum, paths, threads);
}}
"""


def post_source(body: str) -> str:
    """postprocess.glsl as a struct whose members are its uniforms, its in/out variables and its
    functions, plus a driver that runs main() once per output pixel the way TiledRenderer's
    display pass does (TiledRenderer.cpp:540-552): TexCoords at the pixel centre, the
    accumulation texture (RGB32F, GL_LINEAR, GL_REPEAT) bound as pathTraceTexture."""
    return f"""#include "glsl_shim.h"
#include <cstdint>
namespace glsl {{
struct RefPost {{
{body}
}};
}}
struct PostIn
{{
    int32_t tonemap, use_ca, use_ca_distortion, use_vignette, preview;
    float ca_distance, ca_p1, ca_p2, ca_p3, vignette_intensity, vignette_power;
}};
// rgbf: W x H x 3 colour of the display pass, row 0 at the bottom.
extern "C" int refsh_postprocess(const float* accum_rgb, int W, int H, const PostIn* q, int samples, float* rgbf)
{{
    glsl::RefPost s{{}};
    s.pathTraceTexture.data = accum_rgb;
    s.pathTraceTexture.w = W;
    s.pathTraceTexture.h = H;
    s.pathTraceTexture.comps = 3;
    s.pathTraceTexture.linear = true;
    s.isInPreview = q->preview != 0;
    s.invSampleCounter = 1.0f / (float)samples;
    s.tonemapIndex = q->tonemap;
    s.useCA = q->use_ca != 0;
    s.useCADistortion = q->use_ca_distortion != 0;
    s.caDistance = q->ca_distance;
    s.caP1 = q->ca_p1;
    s.caP2 = q->ca_p2;
    s.caP3 = q->ca_p3;
    s.useVignette = q->use_vignette != 0;
    s.vignetteIntensity = q->vignette_intensity;
    s.vignettePower = q->vignette_power;
    for (int y = 0; y < H; ++y)
        for (int x = 0; x < W; ++x)
        {{
            s.TexCoords = glsl::vec2(((float)x + 0.5f) / (float)W, ((float)y + 0.5f) / (float)H);
            s.main();
            float* o = rgbf + ((size_t)y * W + x) * 3;
            o[0] = s.color.x;
            o[1] = s.color.y;
            o[2] = s.color.z;
        }}
    return 0;
}}
"""


def run(cmd):
    r = subprocess.run([str(c) for c in cmd], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"failed: {' '.join(map(str, cmd))}\n{r.stdout[-4000:]}\n{r.stderr[-8000:]}")


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--out", default=str(HERE / "_ref"))
    ap.add_argument("--force", action="store_true")
    args = ap.parse_args()
    out = Path(args.out)
    lib = out / "libref_shader.so"
    deps = [HERE / "glsl_shim.h", HERE / "ref_shader_harness.h", Path(__file__), CSRC / "lf_contract.h"]
    deps += list(SHADERS.rglob("*.glsl"))
    if lib.exists() and not args.force and all(d.stat().st_mtime <= lib.stat().st_mtime for d in deps):
        print(lib)
        return 0
    gen = out / "gen"
    gen.mkdir(parents=True, exist_ok=True)
    body = to_cpp(expand(SHADERS / "renderer.glsl"))
    (gen / "renderer_cpp.inc").write_text(body)
    srcs = []
    for m in range(16):
        p = gen / f"variant{m}.cpp"
        p.write_text(variant_source(body, m))
        srcs.append(p)
    d = gen / "dispatch.cpp"
    d.write_text(dispatcher())
    srcs.append(d)
    post = gen / "post.cpp"
    post.write_text(post_source(to_cpp((SHADERS / "postprocess.glsl").read_text())))
    srcs.append(post)
    flags = ["-O2", "-std=c++20", "-fPIC", "-ffp-contract=off", "-fno-fast-math", "-w", "-I", HERE, "-I", CSRC]
    objs = [gen / (s.stem + ".o") for s in srcs]
    with cf.ThreadPoolExecutor(max_workers=os.cpu_count() or 4) as ex:
        list(ex.map(run, [["g++", *flags, "-c", s, "-o", o] for s, o in zip(srcs, objs)]))
    run(["g++", "-shared", "-pthread", "-o", lib, *objs])
    print(lib)
    return 0


if __name__ == "__main__":
    sys.exit(main())
