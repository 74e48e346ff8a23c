"""Host scene layer against the reference's own host code compiled from source
(Loader, Scene, Mesh/tinyobjloader, Camera, HDRLoader, RadeonRays BVH + BvhTranslator):
every flattened array must be byte-identical."""
import numpy as np
import pytest

import lavaframe_gb300 as lf
from tests import scenes
from tests.conftest import REFERENCE

KEYS = ["nodes", "vert_indices", "vertices", "normals", "transforms", "materials", "lights"]


def assert_same(ours, ref, keys=KEYS):
    for k in keys:
        assert ours[k].shape == ref[k].shape, k
        assert ours[k].tobytes() == ref[k].tobytes(), k
    assert ours["top_level_index"] == ref["top_level_index"]


@pytest.mark.parametrize("name", list(scenes.GENERATED))
def test_generated_scene_matches_reference_build(name, ref_host):
    s = scenes.build(name)
    a = s.arrays()
    counts, inst_mesh, inst_mat = s.layout()
    r = ref_host.build(counts, a["vertices"], a["normals"], inst_mesh, a["transforms"], inst_mat, a["materials"])
    assert_same(a, r, keys=["nodes", "vert_indices", "vertices", "normals", "transforms", "materials"])


def test_large_icosphere_mesh_matches_reference_build(ref_host):
    s = lf.HostScene().gen_icospheres(2, 6, 11, 16, 8).build()
    a = s.arrays()
    counts, inst_mesh, inst_mat = s.layout()
    r = ref_host.build(counts, a["vertices"], a["normals"], inst_mesh, a["transforms"], inst_mat, a["materials"])
    assert_same(a, r, keys=["nodes", "vert_indices", "vertices", "normals", "transforms"])


def cornell_fixture():
    p = REFERENCE / "build_include" / "assets" / "cornell_box.lfs"
    if not p.exists():
        pytest.skip("reference fixture not available on this host")
    return p


def test_cornell_fixture_loader_matches_reference(ref_host):
    path = cornell_fixture()
    r = ref_host.load(path)
    s = lf.HostScene().load_file(path)
    a = s.arrays()
    assert_same(a, r)
    assert a["nodes"].shape == (43, 9) and a["top_level_index"] == 29 and a["vert_indices"].shape[0] == 36
    p = s.render_params()
    cam = np.concatenate([p.cam_position, p.cam_right, p.cam_up, p.cam_forward,
                          [p.cam_fov, p.cam_focal_dist, p.cam_aperture]]).astype(np.float32)
    assert cam.tobytes() == r["camera"].tobytes()
    assert [p.width, p.height, p.max_depth, p.enable_rr, p.rr_depth] == list(r["options"])


def test_obj_reader_matches_tinyobj(ref_host):
    path = cornell_fixture().parent / "cornell_box" / "glass_sphere.obj"
    rv, rn = ref_host.load_obj(path)
    s = lf.HostScene()
    mid = lf.lib().lf_hscene_add_mesh_file(s.h, str(path).encode())
    assert mid == 0
    s.add_material(np.zeros(28, np.float32))
    s.add_instance(mid, np.eye(4, dtype=np.float32), 0)
    s.build()
    a = s.arrays()
    # vertex order inside the flat array is mesh order, identical to the reference mesh
    assert a["vertices"].tobytes() == rv.tobytes()
    assert a["normals"].tobytes() == rn.tobytes()


@pytest.mark.parametrize("kind", ["random", "sky"])
def test_env_tables_match_reference(kind, ref_host):
    if kind == "random":
        rgb = np.random.default_rng(5).gamma(0.5, 2.0, size=(32, 64, 3)).astype(np.float32)
    else:
        s = lf.HostScene().gen_icospheres(1, 1, 3, 128, 64).build()
        rgb = s.arrays()["env_rgb"]
    marg, cond = ref_host.hdr_tables(rgb)
    s = lf.HostScene()
    s.add_hdr(rgb)
    s.gen_cornell(8, 8)
    s.build()
    a = s.arrays()
    assert a["env_marginal"].tobytes() == marg.tobytes()
    assert a["env_conditional"].tobytes() == cond.tobytes()


@pytest.mark.parametrize("eye,at,fov", [((0.5, 0.5, -1.3), (0.5, 0.5, 0.5), 45.0), ((0, 20, 75), (0, 0, 0), 45.0),
                                        ((1.0, 1.7, 1.0), (9.0, 1.0, 6.0), 60.0), ((3, -2, 5), (-1, 4, 0.5), 33.0)])
def test_camera_matches_reference(eye, at, fov, ref_host):
    r = ref_host.camera(eye, at, fov)
    s = lf.HostScene()
    s.set_camera(eye, at, fov, 0.0, 0.1)
    s.gen_cornell(8, 8)
    s.set_camera(eye, at, fov, 0.0, 0.1)
    s.build()
    p = s.render_params()
    cam = np.concatenate([p.cam_position, p.cam_right, p.cam_up, p.cam_forward,
                          [p.cam_fov, p.cam_focal_dist, p.cam_aperture]]).astype(np.float32)
    assert cam.tobytes() == r.tobytes()


def moved_instances(a, seed):
    """New transforms (each instance shifted, every third also turned about its own z axis)
    and permuted materials for every instance of a built scene."""
    rng = np.random.default_rng(seed)
    xf = a["transforms"].reshape(-1, 4, 4).astype(np.float32).copy()
    ext = float(np.abs(a["nodes"][:, :6]).max())
    for i in range(len(xf)):
        xf[i, 3, :3] += rng.uniform(-0.1, 0.1, 3).astype(np.float32) * np.float32(ext)
        if i % 3 == 0:
            c, s_ = np.cos(0.4 + i), np.sin(0.4 + i)
            rot = np.array([[c, s_, 0], [-s_, c, 0], [0, 0, 1]], np.float32)
            xf[i, :3, :3] = (rot @ xf[i, :3, :3]).astype(np.float32)
    return xf.reshape(-1, 16)


@pytest.mark.parametrize("gen", ["soup", "icospheres"])
def test_instance_move_matches_reference_rebuild(gen, ref_host):
    """Scene::RebuildInstances after instances move (Scene.cpp:165-178, BvhTranslator::UpdateTLAS
    bvh_translator.cpp:125-131): the rebuilt TLAS part of the node array and the transforms must
    be byte-identical to the reference's."""
    s = scenes.build(gen)
    a = s.arrays()
    counts, inst_mesh, inst_mat = s.layout()
    new_xf = moved_instances(a, 7)
    n_mat = a["materials"].shape[0]
    new_mat = (np.asarray(inst_mat) + 1) % n_mat
    before, after = ref_host.build_and_move(counts, a["vertices"], a["normals"], inst_mesh, a["transforms"], inst_mat,
                                            a["materials"], new_xf, new_mat)
    assert_same(a, before, keys=["nodes", "transforms"])
    for i in range(len(new_mat)):
        s.set_instance(i, new_xf[i], int(new_mat[i]))
    s.rebuild_instances()
    b = s.arrays()
    assert b["nodes"].tobytes() != a["nodes"].tobytes()
    assert_same(b, after, keys=["nodes", "vert_indices", "vertices", "normals", "transforms", "materials"])
