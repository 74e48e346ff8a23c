"""CUDA path vs the CPU oracle on the same seeded inputs, through the C ABI.

Bars: first-hit instance / packed-triangle ids and hit distances bit-exact; any-hit answers
identical; per-path radiance bit-exact (the arithmetic contract makes host and device run
the same IEEE operations), with the 1e-4 relative tolerance of the build plan as the
reported fallback bar; accumulation buffers identical.
"""
import json
import numpy as np
import pytest

import lavaframe_gb300 as lf
import oracle
from tests import scenes

pytestmark = pytest.mark.gpu

PATH_RTOL = 1e-4   # per-path radiance tolerance (relative)


def soup_rays(s, n, seed=2, tmax=1e6):
    a = s.arrays()
    root = a["nodes"][a["top_level_index"]]
    return lf.gen_rays(root[0:3], root[3:6], n, seed, tmax)


def compare_hits(dev, ref):
    same_t = dev["t"].view(np.uint32) == ref["t"].view(np.uint32)
    same = same_t & (dev["instance"] == ref["instance"]) & (dev["prim"] == ref["prim"]) & (dev["light"] == ref["light"])
    return int((~same).sum())


@pytest.mark.parametrize("wide", [True, False])
@pytest.mark.parametrize("culling", [True, False])
def test_closest_hit_ids_bit_exact_on_soup(ctx, culling, wide):
    s = lf.HostScene().gen_soup(1 << 14, 10, 1).build()
    ds = ctx.upload(s)
    ds.set_traversal(wide)
    if not culling:
        ds.set_culling(-1.0, 0.0)
    rays = soup_rays(s, 1 << 18)
    dev = ctx.trace_closest(ds, rays)
    ref, _ = oracle.trace_closest(s.view(), rays)
    mism = compare_hits(dev, ref)
    assert mism == 0, f"{mism} of {len(rays)} rays differ"
    assert (dev["prim"] >= 0).mean() > 0.05
    ds.close()


@pytest.mark.parametrize("flags", [lf.TRACE_SIMPLE, lf.TRACE_UNSORTED, 0])
def test_trace_variants_agree_with_oracle(ctx, flags):
    """Per-thread, persistent, and binned+persistent traversal give the same hits."""
    s = lf.HostScene().gen_soup(1 << 12, 10, 5).build()
    ds = ctx.upload(s)
    rays = soup_rays(s, 100003, seed=9)          # not a multiple of the warp size
    dev = ctx.trace_closest(ds, rays, flags=flags)
    ref, _ = oracle.trace_closest(s.view(), rays)
    assert compare_hits(dev, ref) == 0
    occ = ctx.trace_any(ds, rays, flags=flags)
    ref_occ, _ = oracle.trace_any(s.view(), rays)
    assert np.array_equal(occ, ref_occ)
    ds.close()


def test_any_hit_matches_on_soup(ctx):
    s = lf.HostScene().gen_soup(1 << 14, 10, 1).build()
    ds = ctx.upload(s)
    rays = soup_rays(s, 1 << 18, seed=3, tmax=30.0)
    dev = ctx.trace_any(ds, rays)
    ref, _ = oracle.trace_any(s.view(), rays)
    assert np.array_equal(dev, ref)
    assert 0.01 < dev.mean() < 0.99
    ds.close()


def test_traversal_counters_match_oracle_with_culling(ctx):
    s = lf.HostScene().gen_soup(1 << 12, 10, 1).build()
    ds = ctx.upload(s)
    rays = soup_rays(s, 1 << 15)
    ctx.trace_closest(ds, rays, flags=lf.TRACE_STATS)
    dstats = ctx.trace_stats()
    view = s.view()
    a = s.arrays()
    extent = float(np.abs(a["nodes"][:, :6]).max())
    cull_abs = 64 * float(np.spacing(np.float32(extent)))
    _, ostats = oracle.trace_closest(view, rays, cull_rel=1e-4, cull_abs=cull_abs)
    # inner-node visits and triangle tests: same visit order, same culling
    assert dstats[0] == int(ostats[0]) and dstats[1] == int(ostats[1])
    ds.close()


def axis_rays_on_planes():
    """Rays with zero direction components whose origins lie on box planes of the Cornell
    scene: the slab test meets 0 * inf there, so these take the exact (NaN-propagating) box
    test; the others check the fast one next to it."""
    coords = np.array([0.0, 0.05, 0.265, 0.5, 0.6, 0.999, 1.0], np.float32)
    dirs = [(1, 0, 0), (-1, 0, 0), (0, 1, 0), (0, -1, 0), (0, 0, 1), (0, 0, -1), (1, 1, 0), (0, -1, 1),
            (1, 0, -1), (0.3, 0.4, 0.5)]
    rays = []
    for x in coords:
        for y in coords:
            for z in coords:
                for d in dirs:
                    dv = np.array(d, np.float32)
                    dv = dv / np.float32(np.sqrt(np.float32((dv * dv).sum())))
                    rays.append([x, y, z, 0, dv[0], dv[1], dv[2], 1e6])
    return np.array(rays, np.float32)


def test_zero_direction_components_match_oracle(ctx):
    s = scenes.build("cornell")
    ds = ctx.upload(s)
    rays = axis_rays_on_planes()
    for flags in (0, lf.TRACE_SIMPLE):
        dev = ctx.trace_closest(ds, rays, flags=flags)
        ref, _ = oracle.trace_closest(s.view(), rays)
        assert compare_hits(dev, ref) == 0
        occ = ctx.trace_any(ds, rays, flags=flags)
        ref_occ, _ = oracle.trace_any(s.view(), rays)
        assert np.array_equal(occ, ref_occ)
    ds.close()


def test_closest_hit_with_lights_on_cornell(ctx):
    s = scenes.build("cornell")
    ds = ctx.upload(s)
    rng = np.random.default_rng(4)
    n = 1 << 16
    o = rng.uniform(0.05, 0.95, (n, 3)).astype(np.float32)
    d = rng.normal(size=(n, 3)).astype(np.float32)
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    rays = np.zeros((n, 8), np.float32)
    rays[:, 0:3] = o
    rays[:, 4:7] = d
    rays[:, 7] = 1e6
    dev = ctx.trace_closest(ds, rays, flags=lf.TRACE_LIGHTS)
    ref, _ = oracle.trace_closest(s.view(), rays, lights=True)
    assert compare_hits(dev, ref) == 0
    assert (dev["light"] >= 0).sum() > 0
    ds.close()


def render_both(ctx, s, spp, first=0, flags=0, tile=None, size=None):
    p = s.render_params()
    if size:
        p.width, p.height = size
    if tile:
        p.tile_width, p.tile_height = tile
    ds = ctx.upload(s)
    f = lf.Frame(ctx, ds, p, flags)
    f.render(first, spp)
    f.sync()
    dev_acc = f.accum()
    dev_paths = f.paths(spp) if not tile else None
    ref_acc, ref_paths, ctr = oracle.render(s.view(), p, first, spp, want_paths=not tile)
    counters = f.counters()
    f.close()
    ds.close()
    return dev_acc, dev_paths, ref_acc, ref_paths, counters, ctr


def assert_paths_match(dev_paths, ref_paths):
    exact = dev_paths.view(np.uint32) == ref_paths.view(np.uint32)
    frac_exact = exact.all(axis=-1).mean()
    rel = np.abs(dev_paths - ref_paths) / np.maximum(np.abs(ref_paths), 1e-6)
    rel = np.where(np.isfinite(ref_paths) & np.isfinite(dev_paths), rel, 0.0)
    assert frac_exact == 1.0 or rel.max() <= PATH_RTOL, (frac_exact, float(rel.max()))
    return frac_exact


@pytest.mark.parametrize("name,spp", [("cornell", 4), ("room", 2)])
def test_path_radiance_matches_oracle(ctx, name, spp):
    if name == "room":
        s = lf.HostScene().gen_room(300, 4).build()
        size = (64, 36)
    else:
        s = scenes.build(name)
        size = None
    dev_acc, dev_paths, ref_acc, ref_paths, counters, ctr = render_both(ctx, s, spp, size=size)
    frac = assert_paths_match(dev_paths, ref_paths)
    assert frac == 1.0
    assert dev_acc.tobytes() == ref_acc.tobytes()
    assert counters[1] == ctr[1]          # extension rays traced


def test_icospheres_env_transmission_match_oracle(ctx):
    s = lf.HostScene().gen_icospheres(6, 3, 5, 64, 32).build()
    p = s.render_params()
    p.width, p.height = 64, 36
    ds = ctx.upload(s)
    f = lf.Frame(ctx, ds, p)
    f.render(0, 2)
    f.sync()
    dev_paths = f.paths(2)
    ref_acc, ref_paths, _ = oracle.render(s.view(), p, 0, 2, want_paths=True)
    assert_paths_match(dev_paths, ref_paths)
    assert f.accum().tobytes() == ref_acc.tobytes()
    f.close()
    ds.close()


def test_tiled_render_matches_oracle(ctx):
    s = scenes.build("cornell")
    dev_acc, _, ref_acc, _, _, _ = render_both(ctx, s, 2, first=3, tile=(40, 24))
    assert dev_acc.tobytes() == ref_acc.tobytes()


def test_progressive_batches_equal_one_call(ctx):
    s = scenes.build("cornell")
    p = s.render_params()
    ds = ctx.upload(s)
    f1 = lf.Frame(ctx, ds, p, lf.FRAME_FP64_ACCUM)
    f1.render(0, 6)
    f2 = lf.Frame(ctx, ds, p)
    f2.set_batch(2)
    f2.render(0, 3)
    f2.render(3, 3)
    a1, a2 = f1.accum(), f2.accum()
    assert a1.tobytes() == a2.tobytes()
    np.testing.assert_allclose(f1.accum64(), a1, rtol=1e-5, atol=1e-5)
    for f in (f1, f2):
        f.close()
    ds.close()


def test_invalid_scene_view_is_rejected(ctx):
    s = scenes.build("cornell")
    v = s.view()
    v.top_level_index = v.num_nodes + 5
    import ctypes as C

    h = C.c_void_p()
    st = lf.lib().lf_scene_upload(ctx.h, C.byref(v), C.byref(h))
    assert st == 1 and not h


@pytest.mark.parametrize("name", ["cornell", "cornell_lights", "cornell_textures", "room", "icospheres",
                                  "icospheres_constbg_tiled", "icospheres_lens", "icospheres_absorb"])
def test_gpu_paths_equal_reference_shader(ctx, name):
    """Device paths against the reference GLSL shader compiled for the CPU (golden vectors)."""
    import json

    from tests.conftest import ROOT
    from tests.golden import cases

    gold = np.load(ROOT / "tests" / "golden" / "shader_paths.npz")[name]
    meta = json.loads((ROOT / "tests" / "golden" / "scenes.json").read_text())[name]
    a, _, extras = cases.build(name)
    for k in cases.KEYS:   # the scene generator is portable: same arrays on this host
        assert cases.digest(a[k]) == meta["digests"][k], k
    p = cases.stored_params(meta)
    view, keep = cases.make_view(a, extras)
    ds = lf.DeviceScene(ctx, view)
    f = lf.Frame(ctx, ds, p)
    spp = gold.shape[0]
    f.render(0, spp)
    f.sync()
    if p.tile_width:
        got = f.accum()[None]
        gold = gold.sum(axis=0, keepdims=True)
    else:
        got = f.paths(spp)
    same = np.all((got == gold) | (np.isnan(got) & np.isnan(gold)), axis=-1)
    f.close()
    ds.close()
    assert same.all(), f"{(~same).sum()} of {same.size} paths differ"


def tie_scene():
    """A 16 x 16 grid of squares in the plane z = 0.5, two triangles each, instanced twice with
    the same identity transform (a third instance is shifted): every hit has an exact twin in the
    other instance, and rays through grid lines hit two adjacent triangles at the same distance."""
    s = lf.HostScene()
    n = 16
    verts, norms = [], []
    for i in range(n):
        for j in range(n):
            x0, x1, y0, y1 = i / n, (i + 1) / n, j / n, (j + 1) / n
            for (a, b, c) in (((x0, y0), (x1, y0), (x1, y1)), ((x0, y0), (x1, y1), (x0, y1))):
                for p in (a, b, c):
                    verts.append([p[0], p[1], 0.5, 0.0])
                    norms.append([0.0, 0.0, 1.0, 0.0])
    mid = s.add_mesh(np.array(verts), np.array(norms))
    m28 = np.zeros(28, np.float32)
    m28[0:3] = 0.8
    m28[6] = 1.0          # roughness
    mat = s.add_material(m28)
    eye = np.eye(4, dtype=np.float32)
    s.add_instance(mid, eye.ravel(), mat)
    s.add_instance(mid, eye.ravel(), mat)
    shifted = eye.copy()
    shifted[3, 2] = 0.25
    s.add_instance(mid, shifted.ravel(), mat)
    s.set_camera([0.5, 0.5, 2.0], [0.5, 0.5, 0.0], 45.0)
    return s.build()


def test_equal_distance_hits_follow_the_reference_order(ctx):
    s = tie_scene()
    ds = ctx.upload(s)
    g = np.arange(0, 17) / 16.0
    pts = np.array([(x, y) for x in g for y in g] + [((i + 0.5) / 16, j / 16) for i in range(16) for j in range(17)] +
                   [((i + 0.3) / 16, (i + 0.3) / 16) for i in range(16)], np.float32)
    rays = []
    for (x, y) in pts:
        for dz, oz in ((-1.0, 2.0), (1.0, -1.0)):
            rays.append([x, y, oz, 0, 0, 0, dz, 1e6])
        d = np.array([0.3, -0.2, -1.0], np.float32)
        d /= np.float32(np.sqrt(np.float32((d * d).sum())))
        o = np.array([x, y, 0.5], np.float32) - d * np.float32(1.5)
        rays.append([o[0], o[1], o[2], 0, d[0], d[1], d[2], 1e6])
    rays = np.array(rays, np.float32)
    ref, _ = oracle.trace_closest(s.view(), rays)
    hit = ref["prim"] >= 0
    assert hit.mean() > 0.5
    for flags in (0, lf.TRACE_SIMPLE):
        dev = ctx.trace_closest(ds, rays, flags=flags)
        assert compare_hits(dev, ref) == 0
    ds.close()


def move_all(s, seed):
    """Moves every instance of a built host scene (new transforms, materials kept) and runs
    Scene::RebuildInstances."""
    from tests.test_scene_reference import moved_instances

    new_xf = moved_instances(s.arrays(), seed)
    _, _, inst_mat = s.layout()
    for i in range(len(new_xf)):
        s.set_instance(i, new_xf[i], int(inst_mat[i]))
    s.rebuild_instances()


def test_instance_update_ray_queries_match_oracle(ctx):
    """lf_scene_update_instances (Renderer::Update's partial re-upload, Renderer.cpp:190-205)
    after Scene::RebuildInstances: queries on the updated device scene equal the oracle on the
    moved scene, and equal a fresh upload of it."""
    s = lf.HostScene().gen_soup(1 << 12, 10, 3).build()
    ds = ctx.upload(s)
    rays = soup_rays(s, 1 << 16, seed=5)
    before = ctx.trace_closest(ds, rays)
    move_all(s, 9)
    ds.update_instances(s)
    dev = ctx.trace_closest(ds, rays)
    ref, _ = oracle.trace_closest(s.view(), rays)
    assert compare_hits(dev, ref) == 0
    assert compare_hits(before, ref) > 1000          # the move changed the answers
    occ = ctx.trace_any(ds, rays)
    ref_occ, _ = oracle.trace_any(s.view(), rays)
    assert np.array_equal(occ, ref_occ)
    fresh = ctx.upload(s)
    assert ctx.trace_closest(fresh, rays).tobytes() == dev.tobytes()
    fresh.close()
    ds.close()


def test_instance_update_render_matches_oracle(ctx):
    s = lf.HostScene().gen_icospheres(6, 3, 5, 64, 32).build()
    p = s.render_params()
    p.width, p.height = 64, 36
    ds = ctx.upload(s)
    f = lf.Frame(ctx, ds, p)
    f.render(0, 2)
    f.sync()
    before = f.paths(2)
    move_all(s, 4)
    ds.update_instances(s)
    f.reset()                       # the frame that rendered before the move continues
    f.render(0, 2)
    f.sync()
    ref_acc, ref_paths, _ = oracle.render(s.view(), p, 0, 2, want_paths=True)
    assert_paths_match(f.paths(2), ref_paths) == 1.0
    assert f.accum().tobytes() == ref_acc.tobytes()
    assert before.tobytes() != ref_paths.tobytes()
    f.close()
    ds.close()
