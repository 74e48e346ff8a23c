"""Edge cases against the oracle, through the C ABI: empty and ragged ray batches, rays that
start outside the scene or point away from it, zero-length and negative segments, frames of
one pixel and ragged tiles, and the full 10.5M-triangle microbench scene checked through
size-independent properties (any-hit answers the closest-hit question exactly; an oracle spot
check; every hit lies within the segment), and host queries split into pieces whose copies
overlap tracing."""
import numpy as np
import pytest

import lavaframe_gb300 as lf
import oracle
from tests import scenes
from tests.test_gpu_parity import compare_hits, soup_rays

pytestmark = pytest.mark.gpu


def small_soup():
    return lf.HostScene().gen_soup(1 << 10, 10, 7).build()


@pytest.mark.parametrize("n", [0, 1, 31, 33, 4097])
def test_empty_and_ragged_batches(ctx, n):
    s = small_soup()
    ds = ctx.upload(s)
    rays = soup_rays(s, max(n, 1), seed=11)[:n]
    hits = ctx.trace_closest(ds, rays)
    occ = ctx.trace_any(ds, rays)
    assert len(hits) == n and len(occ) == n
    if n:
        ref, _ = oracle.trace_closest(s.view(), rays)
        assert compare_hits(hits, ref) == 0
        ref_occ, _ = oracle.trace_any(s.view(), rays)
        assert np.array_equal(occ, ref_occ)
    ds.close()


@pytest.mark.parametrize("chunks", [2, 3, 8])
def test_host_queries_in_pieces_match_whole(ctx, chunks):
    # pieces are sorted and traced on their own while the others are copied; every ray's
    # answer must be the one of the whole query (ragged sizes: the last piece takes the rest)
    s = small_soup()
    ds = ctx.upload(s)
    for n in (1, 1023, 3 * 4097 + 5):
        rays = soup_rays(s, n, seed=13)
        ctx.set_host_chunks(1)
        whole, whole_occ = ctx.trace_closest(ds, rays), ctx.trace_any(ds, rays)
        ctx.set_host_chunks(chunks)
        try:
            hits, occ = ctx.trace_closest(ds, rays), ctx.trace_any(ds, rays)
        finally:
            ctx.set_host_chunks(0)
        assert hits.tobytes() == whole.tobytes() and np.array_equal(occ, whole_occ)
        ref, _ = oracle.trace_closest(s.view(), rays)
        assert compare_hits(hits, ref) == 0
    ds.close()


def test_results_written_into_mapped_host_blocks(ctx):
    # an output range inside a block from lf_host_alloc is written by the kernels directly
    # (whole query or pieces); the answers equal those copied back into pageable memory
    import ctypes as C

    s = small_soup()
    ds = ctx.upload(s)
    n = 3 * 4097 + 5
    rays = soup_rays(s, n, seed=14)
    whole = ctx.trace_closest(ds, rays)
    whole_occ = ctx.trace_any(ds, rays)
    L = lf.lib()
    size = n * 16 + 64
    blk = C.c_void_p()
    ctx._c(L.lf_host_alloc(ctx.h, size, C.byref(blk)))
    fr = rays.ctypes.data_as(C.POINTER(C.c_float))
    try:
        for chunks in (1, 3):
            ctx.set_host_chunks(chunks)
            for off in (0, 48):
                C.memset(blk.value, 0xFF, size)
                ctx._c(L.lf_trace_closest(ctx.h, ds.h, fr, n, blk.value + off, 0))
                assert bytes((C.c_char * (n * 16)).from_address(blk.value + off)) == whole.tobytes()
            C.memset(blk.value, 0xFF, size)
            ctx._c(L.lf_trace_any(ctx.h, ds.h, fr, n, blk.value + 5, 0))
            got = np.frombuffer(bytes((C.c_char * n).from_address(blk.value + 5)), np.uint8)
            assert np.array_equal(got, whole_occ)
    finally:
        ctx.set_host_chunks(0)
        ctx._c(L.lf_host_free(ctx.h, blk))
    ds.close()


def edge_rays(s, n=4096, seed=12):
    """Four groups: origins outside the scene box heading away, origins outside heading in,
    segments of length zero / below zero / tiny, axis-aligned directions."""
    a = s.arrays()
    root = a["nodes"][a["top_level_index"]]
    lo, hi = root[0:3].astype(np.float32), root[3:6].astype(np.float32)
    rays = soup_rays(s, n, seed=seed)
    rng = np.random.default_rng(seed)
    k = n // 4
    centre = (lo + hi) * 0.5
    out = hi + np.float32(5.0) + rng.random((k, 3), dtype=np.float32) * 10
    away = out - centre
    rays[:k, 0:3] = out
    rays[:k, 4:7] = away / np.linalg.norm(away, axis=1, keepdims=True)
    rays[k:2 * k, 0:3] = out
    rays[k:2 * k, 4:7] = -rays[:k, 4:7]
    rays[2 * k:3 * k, 7] = rng.choice(np.array([0.0, -1.0, 1e-6, 1e-30], np.float32), k)
    axes = np.eye(3, dtype=np.float32)[rng.integers(0, 3, k)] * rng.choice(np.array([-1, 1], np.float32), (k, 1))
    rays[3 * k:4 * k, 4:7] = axes
    return rays


def test_rays_outside_the_scene_and_short_segments(ctx):
    s = small_soup()
    ds = ctx.upload(s)
    rays = edge_rays(s)
    hits = ctx.trace_closest(ds, rays)
    ref, _ = oracle.trace_closest(s.view(), rays)
    assert compare_hits(hits, ref) == 0
    occ = ctx.trace_any(ds, rays)
    ref_occ, _ = oracle.trace_any(s.view(), rays)
    assert np.array_equal(occ, ref_occ)
    k = len(rays) // 4
    assert (hits["prim"][:k] < 0).all()                  # heading away from the box
    assert (hits["prim"][2 * k:3 * k] < 0).all()         # segments of length <= 1e-6
    assert (hits["prim"][k:2 * k] >= 0).any()            # some heading in do hit
    ds.close()


@pytest.mark.parametrize("size,tile", [((1, 1), None), ((37, 23), (16, 10)), ((5, 64), (64, 64))])
def test_tiny_and_ragged_frames_match_oracle(ctx, size, tile):
    s = scenes.build("cornell")
    p = s.render_params()
    p.width, p.height = size
    if tile:
        p.tile_width, p.tile_height = tile
    ds = ctx.upload(s)
    f = lf.Frame(ctx, ds, p)
    f.render(0, 2)
    f.sync()
    dev = f.accum()
    ref, _, _ = oracle.render(s.view(), p, 0, 2, want_paths=False)
    assert dev.tobytes() == ref.tobytes()
    f.close()
    ds.close()


def test_full_microbench_scene_properties(ctx):
    s = lf.HostScene().gen_soup(1 << 20, 10, 1).build()   # the 10,485,760-triangle microbench scene
    ds = ctx.upload(s)
    rays = soup_rays(s, 1 << 22, seed=2)
    hits = ctx.trace_closest(ds, rays)
    occ = ctx.trace_any(ds, rays)
    found = hits["prim"] >= 0
    # the any-hit query answers the closest-hit query's question exactly (no lights here)
    assert np.array_equal(occ.astype(bool), found)
    # hits lie on the segment
    assert (hits["t"][found] >= 0).all() and (hits["t"][found] < rays[found, 7]).all()
    assert 0.5 < found.mean() < 1.0
    idx = np.random.default_rng(5).choice(len(rays), 2048, replace=False)
    ref, _ = oracle.trace_closest(s.view(), rays[idx])
    assert compare_hits(hits[idx], ref) == 0
    # the same query in four pieces, with copies overlapping the tracing
    ctx.set_host_chunks(4)
    try:
        assert ctx.trace_closest(ds, rays).tobytes() == hits.tobytes()
    finally:
        ctx.set_host_chunks(0)
    ds.close()
