"""The C++ renderer as a drop-in for LavaFrame's own renderer pointer: a translation unit that
includes the reference's Scene.h and Renderer.h (from a reference checkout) and assigns
CudaRenderer<LavaFrame::Scene, LavaFrame::Renderer> to a LavaFrame::Renderer*, as InitRenderer
does (Main.cpp:88-96), must compile against the reference's headers unchanged. Skipped where
no reference checkout exists."""
import shutil
import subprocess

import pytest

from tests.conftest import REFERENCE, ROOT

SOURCE = r"""
#include "Scene.h"
#include "Renderer.h"
#include "lavaframe_gb300_renderer.hpp"

LavaFrame::Renderer* init_renderer(LavaFrame::Scene* scene)
{
    LavaFrame::Renderer* r = new LavaFrame::CudaRenderer<LavaFrame::Scene, LavaFrame::Renderer>(scene, 0);
    r->Init();
    r->Update(0.016f);
    r->Render();
    int w = 0, h = 0;
    unsigned char* ldr = nullptr;
    float* hdr = nullptr;
    r->GetOutputBuffer(&ldr, w, h);
    r->GetOutputBufferHDR(&hdr, w, h);
    (void)r->GetProgress();
    (void)r->GetSampleCount();
    (void)r->SetViewport(w, h);
    delete[] ldr;
    delete[] hdr;
    return r;
}
"""


def test_cuda_renderer_is_a_reference_renderer(tmp_path):
    lf_dir = REFERENCE / "LavaFrame"
    if not (lf_dir / "Renderer.h").exists():
        pytest.skip("no reference checkout on this host")
    if not shutil.which("g++"):
        pytest.skip("no C++ compiler")
    src = tmp_path / "dropin.cpp"
    src.write_text(SOURCE)
    inc = [lf_dir, lf_dir / "thirdparty" / "RadeonRays", lf_dir / "thirdparty" / "gl3w", lf_dir / "thirdparty" / "stb",
           lf_dir / "thirdparty" / "imgui", ROOT / "include"]
    cmd = ["g++", "-std=c++17", "-fsyntax-only", "-w"] + [x for d in inc for x in ("-I", str(d))] + [str(src)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-4000:]
