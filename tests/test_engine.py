"""The multi-job engine (path regeneration in a fixed slot pool, graph-captured steps) against
the bounce-synchronous per-batch pipeline and the oracle, through the C ABI.

Every configuration must give the same per-path radiance bits, the same accumulation bits and
the same ray counts: the engine only changes which slot a path runs in and when.
"""
import numpy as np
import pytest

import lavaframe_gb300 as lf
import oracle
from tests import scenes

pytestmark = pytest.mark.gpu

DEFAULT_SLOTS = 1 << 24
DEFAULT_SHADE_CAP = 512


def icospheres():
    return lf.HostScene().gen_icospheres(6, 3, 5, 64, 32).build()


def render(ctx, s, spp, flags=0, size=None, tile=None, first=0, batch=0):
    p = s.render_params()
    if size:
        p.width, p.height = size
    if tile:
        p.tile_width, p.tile_height = tile
    ds = ctx.upload(s)
    f = lf.Frame(ctx, ds, p, flags)
    if batch:
        f.set_batch(batch)
    f.render(first, spp)
    f.sync()
    out = {"accum": f.accum(), "counters": f.counters()}
    if not tile:
        out["paths"] = f.paths(spp)
    f.close()
    ds.close()
    return out, p


def same_bits(a, b):
    return a.view(np.uint32).tobytes() == b.view(np.uint32).tobytes()


@pytest.mark.parametrize("name", ["cornell", "icospheres"])
@pytest.mark.parametrize("flags", [lf.FRAME_PER_BATCH, lf.FRAME_PER_BATCH | lf.FRAME_USE_GRAPH])
def test_engine_equals_per_batch_pipeline(ctx, name, flags):
    s = icospheres() if name == "icospheres" else scenes.build(name)
    size = (64, 36) if name == "icospheres" else None
    eng, _ = render(ctx, s, 3, size=size)
    ref, _ = render(ctx, s, 3, flags=flags, size=size)
    assert same_bits(eng["accum"], ref["accum"])
    assert same_bits(eng["paths"], ref["paths"])
    assert eng["counters"][1:] == ref["counters"][1:]   # extension rays, shadow rays, clamps


@pytest.mark.parametrize("slots", [1024, 1000])
def test_small_pool_regenerates_and_matches_oracle(ctx, slots):
    """1024 slots for 4608 paths: most slots run several paths; partial edge tiles. 1000 slots:
    a pool that the refill's 1024-slot scan steps do not divide."""
    s = icospheres()
    try:
        ctx.configure_engine(slots=slots)
        assert ctx.engine_info()["slots"] == slots
        got, p = render(ctx, s, 2, size=(64, 36), tile=(20, 12), first=1)
        ref_acc, _, ctr = oracle.render(s.view(), p, 1, 2, want_paths=False)
        assert same_bits(got["accum"], ref_acc)
        assert got["counters"][1] == ctr[1]
        got, p = render(ctx, s, 2, size=(64, 36))
        ref_acc, ref_paths, _ = oracle.render(s.view(), p, 0, 2, want_paths=True)
        assert same_bits(got["paths"], ref_paths)
        assert same_bits(got["accum"], ref_acc)
    finally:
        ctx.configure_engine(slots=DEFAULT_SLOTS, block_extend=0, block_shade=0, block_shadow=0,
                             shade_threads_per_sm=DEFAULT_SHADE_CAP)


@pytest.mark.parametrize("slots", [1024, 4096])
def test_sort_by_material_keeps_results(ctx, slots):
    """Shade taking the surface hits bucketed by material class (opaque, metal, transmissive,
    textured): per-path radiance, accumulation and ray counts unchanged. Pools smaller than the
    frame's paths keep the step kernels (not only the drain) running."""
    s = icospheres()
    classes = set()
    a = s.arrays()
    _, _, inst_mat = s.layout()
    for m in inst_mat:
        mp = a["materials"][m]
        classes.add(2 if mp[16] > 0 else 1 if mp[8] >= 0.5 else 0)
    assert len(classes) >= 2
    try:
        ctx.configure_engine(slots=slots)
        ctx.set_engine_sort(False)
        base, p = render(ctx, s, 3, size=(64, 36))
        ctx.set_engine_sort(True)
        got, _ = render(ctx, s, 3, size=(64, 36))
        ctx.set_engine_sort("auto")   # the default: sorted here, the scene mixes classes
        auto, _ = render(ctx, s, 3, size=(64, 36))
    finally:
        ctx.set_engine_sort("auto")
        ctx.configure_engine(slots=DEFAULT_SLOTS, block_extend=0, block_shade=0, block_shadow=0,
                             shade_threads_per_sm=DEFAULT_SHADE_CAP)
    for r in (got, auto):
        assert same_bits(r["paths"], base["paths"])
        assert same_bits(r["accum"], base["accum"])
        assert r["counters"][1:] == base["counters"][1:]
    ref_acc, _, _ = oracle.render(s.view(), p, 0, 3, want_paths=False)
    assert same_bits(got["accum"], ref_acc)


def test_depth_zero_job_is_black_and_matches_oracle(ctx):
    """A job of depth 0: its paths go from the refill straight to the done list and the finish
    kernel writes out zero radiance; no ray is traced. Small pools keep the step kernels running."""
    s = icospheres()
    try:
        ctx.configure_engine(slots=1024)
        p = s.render_params()
        p.width, p.height = 48, 27
        p.max_depth = 0
        ds = ctx.upload(s)
        f = lf.Frame(ctx, ds, p)
        f.render(0, 3)
        f.sync()
        acc, ctr = f.accum(), f.counters()
        f.close()
        ds.close()
    finally:
        ctx.configure_engine(slots=DEFAULT_SLOTS, block_extend=0, block_shade=0, block_shadow=0,
                             shade_threads_per_sm=DEFAULT_SHADE_CAP)
    ref_acc, _, ref_ctr = oracle.render(s.view(), p, 0, 3, want_paths=False)
    assert same_bits(acc, ref_acc)
    assert not acc.any()
    assert ctr[1] == 0 and ref_ctr[1] == 0


@pytest.mark.parametrize("drain", [0, 1 << 10, 1 << 24])
def test_drain_threshold_keeps_results(ctx, drain):
    """The run's switch to the one-kernel drain (never, late, or from the first step) changes
    only how the last paths are traced."""
    s = icospheres()
    try:
        ctx.configure_engine(slots=2048)
        base, p = render(ctx, s, 3, size=(64, 36))
        ctx.set_engine_drain(drain)
        got, _ = render(ctx, s, 3, size=(64, 36))
    finally:
        ctx.set_engine_drain(1 << 22)
        ctx.configure_engine(slots=DEFAULT_SLOTS, block_extend=0, block_shade=0, block_shadow=0,
                             shade_threads_per_sm=DEFAULT_SHADE_CAP)
    assert same_bits(got["paths"], base["paths"])
    assert same_bits(got["accum"], base["accum"])
    assert got["counters"][1:] == base["counters"][1:]


@pytest.mark.parametrize("blocks", [(64, 256, 96), (256, 64, 512)])
def test_engine_block_sizes_do_not_change_results(ctx, blocks):
    s = scenes.build("cornell")
    base, _ = render(ctx, s, 2)
    try:
        ctx.configure_engine(0, *blocks)
        got, _ = render(ctx, s, 2)
    finally:
        ctx.configure_engine(0, 0, 0, 0, DEFAULT_SHADE_CAP)
    assert same_bits(got["paths"], base["paths"])
    assert same_bits(got["accum"], base["accum"])


def test_passes_split_by_batch_size_accumulate_in_order(ctx):
    """Five samples in passes of two: three passes per tile, accumulated in sample order."""
    s = scenes.build("cornell")
    one, _ = render(ctx, s, 5)
    split, _ = render(ctx, s, 5, batch=2)
    assert same_bits(one["accum"], split["accum"])
    assert one["counters"][1:] == split["counters"][1:]


def test_frames_of_two_scenes_alternate(ctx):
    """Two frames on two scenes share the context's engine (job slots) without interference."""
    a, b = scenes.build("cornell"), icospheres()
    pa, pb = a.render_params(), b.render_params()
    pb.width, pb.height = 48, 27
    da, db = ctx.upload(a), ctx.upload(b)
    fa, fb = lf.Frame(ctx, da, pa), lf.Frame(ctx, db, pb)
    for k in range(2):
        fa.render(k, 1)
        fb.render(k, 1)
    fa.sync()
    ra, _, _ = oracle.render(a.view(), pa, 0, 2, want_paths=False)
    rb, _, _ = oracle.render(b.view(), pb, 0, 2, want_paths=False)
    assert same_bits(fa.accum(), ra)
    assert same_bits(fb.accum(), rb)
    for h in (fa, fb, da, db):
        h.close()


def test_autotuner_picks_a_setting_and_results_stay_exact(ctx, tmp_path):
    from lavaframe_gb300 import autotune

    s = scenes.build("cornell")
    base, p = render(ctx, s, 2)
    ds = ctx.upload(s)
    try:
        cache = tmp_path / "tune.json"
        r = autotune.tune(ctx, ds, p, spp=2, repeats=1, triangles=int(s.view().num_tris), cache=cache)
        assert set(r["config"]) == set(autotune.DEFAULT) and len(r["trials"]) >= 13 and not r["cached"]
        again = autotune.tune(ctx, ds, p, spp=2, repeats=1, triangles=int(s.view().num_tris), cache=cache)
        assert again["cached"] and again["config"] == r["config"]
        got, _ = render(ctx, s, 2)
    finally:
        ds.close()
        autotune.apply_default(ctx)
    assert same_bits(got["paths"], base["paths"])
