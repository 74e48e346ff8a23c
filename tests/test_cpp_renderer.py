"""The C++ drop-in (include/lavaframe_gb300_renderer.hpp): a program written like LavaFrame's
Main.cpp loads a .scene file with LoadSceneFromFile, drives CudaRenderer with Update()/Render()
per tile and reads GetOutputBuffer / GetOutputBufferHDR. Its output must equal the C ABI's
frame rendered with the same tiles, RNG keying and display settings."""
import shutil
import subprocess

import numpy as np
import pytest

import lavaframe_gb300 as lf
from tests.conftest import ROOT

pytestmark = pytest.mark.gpu

SCENE = """
Camera
{
    position 0.5 0.5 -1.3
    lookAt 0.5 0.5 0.5
    fov 45
}

Renderer
{
    resolution 48 40
    maxDepth 4
    tileWidth 16
    tileHeight 20
    tonemapIndex 3
    useVignette 1
    vignetteIntensity 0.5
    vignettePower 2
}

light
{
    position 0.375 0.999 0.375
    emission 17 12 4
    v1 0.625 0.999 0.375
    v2 0.375 0.999 0.625
    type Quad
}

material white
{
    color 0.73 0.73 0.73
}

material red
{
    color 0.63 0.065 0.05
}

mesh
{
    file box.obj
    material white
}

mesh
{
    file wall.obj
    material red
}
"""

BOX = """v 0 0 0
v 1 0 0
v 1 0 1
v 0 0 1
v 0 1 0
v 1 1 0
v 1 1 1
v 0 1 1
vn 0 1 0
vn 0 -1 0
vn 0 0 -1
vn -1 0 0
f 1//1 2//1 3//1 4//1
f 5//2 8//2 7//2 6//2
f 4//3 3//3 7//3 8//3
f 2//4 6//4 7//4 3//4
"""

WALL = """v 0 0 0
v 0 0 1
v 0 1 1
v 0 1 0
vn 1 0 0
f 1//1 2//1 3//1 4//1
"""

PROGRAM = r"""
#include <cstdio>
#include <cstdlib>
#include "lavaframe_gb300_renderer.hpp"
#include "lf_scene.h"

int main(int argc, char** argv)
{
    LavaFrame::Scene scene;
    LavaFrame::RenderOptions options;
    if (!LavaFrame::LoadSceneFromFile(argv[1], &scene, options)) return 2;
    scene.renderOptions = options;
    LavaFrame::CudaRenderer<LavaFrame::Scene> renderer(&scene, 0);
    renderer.Init();
    const int passes = std::atoi(argv[2]);
    while (renderer.GetSampleCount() <= passes)
    {
        renderer.Update(0.016f);
        if (renderer.GetSampleCount() > passes) break;
        renderer.Render();
    }
    unsigned char* rgb = nullptr;
    float* hdr = nullptr;
    int w = 0, h = 0;
    renderer.GetOutputBuffer(&rgb, w, h);
    renderer.GetOutputBufferHDR(&hdr, w, h);
    FILE* f = std::fopen(argv[3], "wb");
    std::fwrite(&w, 4, 1, f);
    std::fwrite(&h, 4, 1, f);
    std::fwrite(&passes, 4, 1, f);
    const int samples = renderer.GetSampleCount();
    std::fwrite(&samples, 4, 1, f);
    std::fwrite(rgb, 1, (size_t)w * h * 3, f);
    std::fwrite(hdr, 4, (size_t)w * h * 3, f);
    std::fclose(f);
    delete[] rgb;
    delete[] hdr;
    renderer.Finish();
    return 0;
}
"""


def test_cpp_renderer_equals_the_c_abi(ctx, tmp_path):
    cxx = shutil.which("g++")
    if not cxx:
        pytest.skip("no C++ compiler")
    (tmp_path / "scene.lfs").write_text(SCENE)
    (tmp_path / "box.obj").write_text(BOX)
    (tmp_path / "wall.obj").write_text(WALL)
    (tmp_path / "main.cpp").write_text(PROGRAM)
    exe = tmp_path / "render"
    lib = ROOT / "lavaframe_gb300"
    subprocess.run([cxx, "-std=c++17", "-O2", "-I", str(ROOT / "include"), "-I",
                    str(ROOT / "lavaframe_gb300" / "csrc" / "host"), str(tmp_path / "main.cpp"), "-o", str(exe),
                    "-L", str(lib), "-llfcore", f"-Wl,-rpath,{lib}"], check=True)
    passes = 3
    subprocess.run([str(exe), str(tmp_path / "scene.lfs"), str(passes), str(tmp_path / "out.bin")], check=True,
                   timeout=120)
    raw = (tmp_path / "out.bin").read_bytes()
    w, h, _, samples = np.frombuffer(raw[:16], np.int32)
    rgb8 = np.frombuffer(raw[16:16 + w * h * 3], np.uint8).reshape(h, w, 3)
    hdr = np.frombuffer(raw[16 + w * h * 3:], np.float32).reshape(h, w, 3)

    # the same render through the C ABI: tiled frames keyed like TiledRenderer (frame_base 2)
    s = lf.HostScene()
    s.load_file(str(tmp_path / "scene.lfs"))
    p = s.render_params()
    assert (p.width, p.height) == (w, h)
    p.tile_width, p.tile_height = 16, 20     # the scene's tileWidth / tileHeight
    p.frame_base = 2
    ds = ctx.upload(s)
    f = lf.Frame(ctx, ds, p, lf.FRAME_TILED_FRAMES)
    f.render(0, passes)
    f.sync()
    acc = f.accum()
    pp = lf.PostParams.defaults(3)
    pp.use_vignette, pp.vignette_intensity, pp.vignette_power = 1, 0.5, 2.0
    ref8, _ = f.postprocess(int(samples), pp)
    f.close()
    ds.close()
    assert np.array_equal(hdr, acc * np.float32(1.0 / samples))
    assert np.array_equal(rgb8, ref8)
    assert rgb8.mean() > 5
