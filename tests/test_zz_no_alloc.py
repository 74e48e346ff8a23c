"""lf_render_noalloc: rendering for callers that cannot allocate device memory while they
render (fixed-arena plugin hosts, allocation-free frame loops, CUDA graph recording).

The entry point keeps all wavefront state in a fixed device array of the library and
accumulates into a buffer the caller owns. Checked through the C ABI against the regular
lf_frame_render path on two calls in a row (the second continues the accumulation), with
the path-radiance tolerance the parity tests use.
"""
import ctypes as C

import numpy as np
import pytest

import lavaframe_gb300 as lf
from tests import scenes

pytestmark = pytest.mark.gpu

RTOL = 1e-4


def test_noalloc_render_matches_frame_render_on_two_calls(ctx):
    s = scenes.build("cornell")
    p = s.render_params()
    ds = ctx.upload(s)
    L = lf.lib()
    W, H = p.width, p.height

    f = lf.Frame(ctx, ds, p)
    f.render(0, 3)
    want1 = f.accum()
    f.render(3, 2)
    want2 = f.accum()
    f.close()

    d_acc = C.c_void_p()
    ctx._c(L.lf_device_alloc(ctx.h, W * H * 16, C.byref(d_acc)))
    zeros = np.zeros((H, W, 4), np.float32)
    ctx._c(L.lf_copy_to_device(ctx.h, d_acc, zeros.ctypes.data_as(C.c_void_p), zeros.nbytes))
    got = []
    for first, count in ((0, 3), (3, 2)):
        ctx._c(L.lf_render_noalloc(ds.h, C.byref(p), first, count, d_acc))
        out = np.empty((H, W, 4), np.float32)
        ctx._c(L.lf_copy_to_host(ctx.h, out.ctypes.data_as(C.c_void_p), d_acc, out.nbytes))
        got.append(out[..., :3].copy())
    ctx._c(L.lf_device_free(ctx.h, d_acc))

    for g, w in zip(got, (want1, want2)):
        np.testing.assert_allclose(g, w, rtol=RTOL, atol=1e-6)
    ds.close()


def test_noalloc_rejects_tiles_beyond_capacity(ctx):
    s = scenes.build("cornell")
    p = s.render_params()
    p.width, p.height = 512, 512          # 262144 pixels in one tile: above the capacity
    ds = ctx.upload(s)
    L = lf.lib()
    d_acc = C.c_void_p()
    ctx._c(L.lf_device_alloc(ctx.h, 512 * 512 * 16, C.byref(d_acc)))
    st = L.lf_render_noalloc(ds.h, C.byref(p), 0, 1, d_acc)
    assert st == 1 and "exceeds the fixed capacity" in ctx.error()
    p.tile_width, p.tile_height = 256, 256   # tiled, each tile fits
    ctx._c(L.lf_copy_to_device(ctx.h, d_acc, np.zeros(512 * 512 * 4, np.float32).ctypes.data_as(C.c_void_p),
                               512 * 512 * 16))
    ctx._c(L.lf_render_noalloc(ds.h, C.byref(p), 0, 1, d_acc))
    ctx._c(L.lf_device_free(ctx.h, d_acc))
    ds.close()
