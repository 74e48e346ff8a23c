"""Generates tests/golden/shader_paths.npz and tests/golden/scenes.json.

Every case (tests/golden/cases.py) is rebuilt with the reference's own host code (BVH build
and flatten, oracle/_ref/libref_host.so) and rendered with the reference's own GLSL shader
compiled for the CPU (oracle/_ref/libref_shader.so, see oracle/ref_shader_gen.py). The stored
per-path radiance pins the oracle and the CUDA path; the stored array digests pin the
product's host scene layer. tests/golden/postprocess.npz holds the reference's display pass
(postprocess.glsl, compiled the same way) of one accumulation buffer under every tone map, CA
and vignette setting of cases.post_settings(). Needs a reference checkout:

    python oracle/build_ref.py && python tests/golden/make_golden.py
"""
import ctypes as C
import json
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

from tests import refhost  # noqa: E402
from tests.golden import cases  # noqa: E402

REF = ROOT / "oracle" / "_ref"


def main():
    rh = refhost.RefHost(REF / "libref_host.so")
    sh = C.CDLL(str(REF / "libref_shader.so"))
    sh.refsh_render.argtypes = [C.c_void_p] * 2 + [C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_int]
    out = {}
    meta = {}
    import lavaframe_gb300 as lf

    for name, spp in cases.CASES.items():
        a, p, extras = cases.build(name)
        # rebuild the BVH arrays with the reference's own host code from the same meshes
        s = lf.HostScene()
        # mesh layout of the product scene (same generator, unmodified)
        if name.startswith("cornell"):
            s.gen_cornell(32 if name != "cornell_lights" else 24, 32 if name != "cornell_lights" else 24)
        elif name == "room":
            s.gen_room(300, 4)
        else:
            s.gen_icospheres(6, 3, 5, 64, 32)
        s.build()
        counts, inst_mesh, inst_mat = s.layout()
        r = rh.build(counts, a["vertices"], a["normals"], inst_mesh, a["transforms"], inst_mat, a["materials"])
        for k in ["nodes", "vert_indices", "vertices", "normals", "transforms"]:
            assert r[k].tobytes() == a[k].tobytes(), (name, k)
        ref_arrays = dict(a)
        ref_arrays.update({k: r[k] for k in ["nodes", "vert_indices", "vertices", "normals", "transforms"]})
        if "env_rgb" in a:
            marg, cond = rh.hdr_tables(a["env_rgb"])
            assert marg.tobytes() == a["env_marginal"].tobytes() and cond.tobytes() == a["env_conditional"].tobytes()
        view, keep = cases.make_view(ref_arrays, extras)
        H, W = p.height, p.width
        acc = np.zeros((H, W, 3), np.float32)
        paths = np.zeros((spp, H, W, 3), np.float32)
        sh.refsh_render(C.addressof(view), C.addressof(p), 0, spp, acc.ctypes.data, paths.ctypes.data, 0)
        out[name] = paths
        params = {f: (list(getattr(p, f)) if hasattr(getattr(p, f), "__len__") else getattr(p, f))
                  for f, _ in p._fields_}
        meta[name] = {"spp": spp, "width": W, "height": H, "params": params,
                      "digests": {k: cases.digest(ref_arrays[k]) for k in cases.KEYS},
                      "top_level_index": int(ref_arrays["top_level_index"]),
                      "mean_radiance": float(paths.mean())}
        print(name, paths.shape, float(paths.mean()))
    np.savez_compressed(ROOT / "tests" / "golden" / "shader_paths.npz", **out)
    # display pass: the reference's postprocess.glsl compiled for the CPU, per setting
    sh.refsh_postprocess.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_void_p, C.c_int, C.c_void_p]
    acc = cases.post_input()
    post = {"input": acc}
    for k, q in enumerate(cases.post_settings()):
        rgbf = np.zeros(acc.shape, np.float32)
        sh.refsh_postprocess(acc.ctypes.data, acc.shape[1], acc.shape[0], C.addressof(q), cases.POST_SAMPLES,
                             rgbf.ctypes.data)
        post[f"setting{k}"] = rgbf
    np.savez_compressed(ROOT / "tests" / "golden" / "postprocess.npz", **post)
    (ROOT / "tests" / "golden" / "scenes.json").write_text(json.dumps(meta, indent=1, sort_keys=True))


if __name__ == "__main__":
    main()
