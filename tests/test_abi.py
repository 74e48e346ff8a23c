"""The C-ABI library loads and exports every entry point declared in include/*.h."""
import ctypes as C
import re

from tests.conftest import ROOT


def declared_symbols():
    names = []
    for h in sorted((ROOT / "include").glob("*.h")):
        text = h.read_text()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        names += re.findall(r"\b(lf_[a-z0-9_]+)\s*\(", text)
    return sorted(set(names))


def test_every_declared_symbol_is_exported():
    import lavaframe_gb300 as lf

    L = C.CDLL(str(lf.LIB_PATH))
    names = declared_symbols()
    assert len(names) > 40
    missing = [n for n in names if not hasattr(L, n)]
    assert not missing, missing


def test_python_binding_covers_the_header():
    import lavaframe_gb300 as lf

    assert set(declared_symbols()) == set(lf.exported_symbols())


def test_struct_layouts_match_header(tmp_path):
    """The ctypes mirrors of lf_scene_view / lf_render_params / lf_hit have the C layout."""
    import shutil
    import subprocess

    import pytest

    import lavaframe_gb300 as lf

    cc = shutil.which("gcc") or shutil.which("cc")
    if not cc:
        pytest.skip("no C compiler")
    src = tmp_path / "sz.c"
    src.write_text('#include <stdio.h>\n#include <stddef.h>\n#include "lavaframe_gb300.h"\n'
                   'int main(void){printf("%zu %zu %zu %zu %zu %zu %zu %zu %zu %zu\\n", sizeof(lf_scene_view),'
                   ' sizeof(lf_render_params), sizeof(lf_hit), offsetof(lf_render_params, seed),'
                   ' offsetof(lf_scene_view, env_width), sizeof(lf_server_config), sizeof(lf_job_info),'
                   ' sizeof(lf_server_stats), offsetof(lf_server_stats, scenes_resident), sizeof(lf_post_params));'
                   'return 0;}')
    exe = tmp_path / "sz"
    subprocess.run([cc, "-I", str(ROOT / "include"), str(src), "-o", str(exe)], check=True)
    got = [int(x) for x in subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split()]
    want = [C.sizeof(lf.SceneView), C.sizeof(lf.RenderParams), lf.HIT_DTYPE.itemsize,
            lf.RenderParams.seed.offset, lf.SceneView.env_width.offset, C.sizeof(lf.ServerConfig),
            C.sizeof(lf.JobInfo), C.sizeof(lf.ServerStats), lf.ServerStats.scenes_resident.offset,
            C.sizeof(lf.PostParams)]
    assert got == want
