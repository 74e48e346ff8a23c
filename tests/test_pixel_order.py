"""The order in which a sample's paths visit a tile's pixels (lf_pixel.h `pixel_of`, used by the
engine's refill, the per-batch generate kernel and the per-path readback) must take every
pixel exactly once, for every tile shape, and group ids 32 at a time into 8 x 4 blocks where
whole blocks fit. The header is compiled for the host here and checked exhaustively."""
import shutil
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]

SRC = r"""
#include <cstdio>
#include <vector>
#include "lf_pixel.h"
int main()
{
    const int sizes[][2] = {{1, 1}, {7, 3}, {8, 4}, {9, 5}, {13, 1}, {1, 13}, {16, 8}, {31, 17},
                            {64, 36}, {80, 56}, {100, 7}, {6, 100}, {256, 256}, {1920, 1080}, {1280, 720}};
    for (auto& s : sizes)
    {
        const int w = s[0], h = s[1];
        std::vector<int> seen((size_t)w * h, 0);
        for (int lp = 0; lp < w * h; ++lp)
        {
            int x, y;
            lfd::pixel_of(lp, w, h, x, y);
            if (x < 0 || x >= w || y < 0 || y >= h) { std::printf("out %d %d %d\n", w, h, lp); return 1; }
            ++seen[(size_t)y * w + x];
            // inside the part whole blocks cover, ids 32k..32k+31 form one 8 x 4 block
            if (lp < (w & ~7) * (h & ~3))
            {
                int x0, y0;
                lfd::pixel_of(lp & ~31, w, h, x0, y0);
                if (x - x0 != (lp & 7) || y - y0 != ((lp & 31) >> 3)) { std::printf("block %d %d %d\n", w, h, lp); return 1; }
            }
        }
        for (int v : seen)
            if (v != 1) { std::printf("cover %d %d\n", w, h); return 1; }
    }
    std::printf("ok\n");
    return 0;
}
"""


@pytest.mark.skipif(shutil.which("g++") is None, reason="needs g++")
def test_pixel_order_is_a_blocked_permutation(tmp_path):
    src = tmp_path / "pixel_order.cpp"
    src.write_text(SRC)
    exe = tmp_path / "pixel_order"
    subprocess.run(["g++", "-std=c++17", "-O1", "-D__host__=", "-D__device__=",
                    "-I", str(ROOT / "lavaframe_gb300" / "csrc" / "device"), str(src), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True)
    assert out.returncode == 0 and out.stdout.strip() == "ok", out.stdout
