"""lf_render_noalloc: rendering for callers that cannot allocate device memory while they
render - plugin hosts that give the renderer a fixed device arena and budget every byte
themselves, and frame loops that forbid allocation inside a frame (cudaMalloc/cudaFree can
stall the device and can fail once another allocator holds the memory).

The entry point keeps all wavefront state in a fixed device array of the library and
accumulates into a buffer the caller owns. Checked through the C ABI against the regular
lf_frame_render path on two calls in a row (the second continues the accumulation): the
accumulation buffers must be byte-identical, untiled and with tiles that do not divide the
frame. Kept in a file of its own that pytest collects last.
"""
import ctypes as C

import numpy as np
import pytest

import lavaframe_gb300 as lf
from tests import scenes

pytestmark = pytest.mark.gpu

CALLS = ((0, 3), (3, 2))   # (first sample, count) of the two calls in a row


def frame_render_sums(ctx, ds, p):
    f = lf.Frame(ctx, ds, p)
    want = []
    for first, count in CALLS:
        f.render(first, count)
        want.append(f.accum())
    f.close()
    return want


def noalloc_sums(ctx, ds, p):
    L = lf.lib()
    W, H = p.width, p.height
    d_acc = C.c_void_p()
    ctx._c(L.lf_device_alloc(ctx.h, W * H * 16, C.byref(d_acc)))
    zeros = np.zeros((H, W, 4), np.float32)
    ctx._c(L.lf_copy_to_device(ctx.h, d_acc, zeros.ctypes.data_as(C.c_void_p), zeros.nbytes))
    got = []
    for first, count in CALLS:
        ctx._c(L.lf_render_noalloc(ds.h, C.byref(p), first, count, d_acc))
        out = np.empty((H, W, 4), np.float32)
        ctx._c(L.lf_copy_to_host(ctx.h, out.ctypes.data_as(C.c_void_p), d_acc, out.nbytes))
        got.append(np.ascontiguousarray(out[..., :3]))
    ctx._c(L.lf_device_free(ctx.h, d_acc))
    return got


@pytest.mark.parametrize("size,tile", [(None, None), ((512, 512), (256, 256)), ((300, 200), (128, 96))])
def test_noalloc_render_equals_frame_render_on_two_calls(ctx, size, tile):
    s = scenes.build("cornell")
    p = s.render_params()
    if size:
        p.width, p.height = size
    if tile:
        p.tile_width, p.tile_height = tile
    ds = ctx.upload(s)
    want = frame_render_sums(ctx, ds, p)
    got = noalloc_sums(ctx, ds, p)
    ds.close()
    for k, (g, w) in enumerate(zip(got, want)):
        assert g.tobytes() == w.tobytes(), f"call {k}: {(g != w).any(-1).sum()} pixels differ"
    assert got[1].sum() > got[0].sum() > 0


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
    ctx._c(L.lf_device_free(ctx.h, d_acc))
    ds.close()
