"""Scenes of the golden-vector cases. Each case is built with the product's host API, then
optionally modified (extra light types, texture maps, render switches); `make_view` turns the
arrays into an lf_scene_view. tests/golden/make_golden.py renders the same cases with the
reference shader compiled for the CPU and the reference host BVH build."""
import ctypes as C
import hashlib

import numpy as np

import lavaframe_gb300 as lf

KEYS = ["nodes", "vert_indices", "vertices", "normals", "transforms", "materials", "lights"]


def digest(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def _textures():
    """Four 16x16 RGBA8 layers: albedo, metallic-roughness, normal map, emission map."""
    y, x = np.mgrid[0:16, 0:16]
    t = np.zeros((4, 16, 16, 4), np.uint8)
    t[0, ..., 0] = 40 + 12 * x
    t[0, ..., 1] = 40 + 12 * y
    t[0, ..., 2] = 200
    t[1, ..., 0] = (x * 16) % 256
    t[1, ..., 1] = 60 + 10 * y
    t[2, ..., 0] = 128 + 3 * (x - 8)
    t[2, ..., 1] = 128 + 3 * (y - 8)
    t[2, ..., 2] = 240
    t[3, ..., 0] = 255 * ((x + y) % 2)
    t[3, ..., 1] = 90
    t[3, ..., 2] = 30
    t[..., 3] = 255
    return t


def build(name):
    """Returns (arrays, params, extras) for a case."""
    s = lf.HostScene()
    if name in ("cornell", "cornell_lights", "cornell_textures"):
        s.gen_cornell(32 if name != "cornell_lights" else 24, 32 if name != "cornell_lights" else 24)
    elif name == "room":
        s.gen_room(300, 4)
    elif name in ("icospheres", "icospheres_constbg_tiled", "icospheres_lens", "icospheres_absorb"):
        s.gen_icospheres(6, 3, 5, 64, 32)
    else:
        raise KeyError(name)
    if name == "cornell_lights":
        # sphere light (type 1) and distant light (type 2) next to the quad light
        sph = np.array([0.25, 0.6, 0.6, 6, 5, 4, 0, 0, 0, 0, 0, 0, 0.08, 4 * np.pi * 0.08 * 0.08, 1], np.float32)
        dst = np.array([0.3, 1.0, -0.5, 0.5, 0.5, 0.6, 0, 0, 0, 0, 0, 0, 0, 0, 2], np.float32)
        s.add_light(sph)
        s.add_light(dst)
    s.build()
    a = s.arrays()
    p = s.render_params()
    extras = {}
    if name == "room":
        p.width, p.height = 48, 27
    if name == "icospheres":
        p.width, p.height = 48, 27
    if name == "icospheres_constbg_tiled":
        p.width, p.height = 32, 18
        p.use_constant_bg = 1
        p.bg_color[0], p.bg_color[1], p.bg_color[2] = 0.2, 0.3, 0.4
        p.tile_width, p.tile_height = 20, 12
    if name == "icospheres_lens":
        p.width, p.height = 32, 18
        p.cam_aperture = 0.3
        p.cam_focal_dist = 40.0
        p.hdr_multiplier = 2.0
        p.frame_base = 7
    if name == "icospheres_absorb":
        # transmissive, absorbing interiors (pathtrace.glsl:263-272): every material but the
        # first becomes a smooth dielectric whose extinction is reached at atDistance
        p.width, p.height = 48, 27
        m = a["materials"].copy()
        m[1:, 8] = 0.0                       # metallic
        m[1:, 9] = 0.05                      # roughness
        m[1:, 16] = 1.0                      # transmission (specTrans)
        m[1:, 17] = 1.5                      # ior
        m[1:, 18] = 0.6                      # atDistance
        m[1:, 20:23] = [0.3, 0.55, 0.85]     # extinction
        a["materials"] = m
    if name == "cornell_lights":
        p.enable_rr = 0
        p.max_depth = 5
    if name == "cornell_textures":
        m = a["materials"].copy()
        m[1, 24:28] = [0, 1, 2, -1]     # white walls: albedo, metallic-roughness, normal map
        m[2, 24:28] = [-1, -1, -1, 3]   # red wall: emission map
        a["materials"] = m
        extras["textures"] = _textures()
    return a, p, extras


def make_view(a, extras):
    """lf_scene_view over numpy arrays; the returned tuple keeps them alive."""
    keep = {k: np.ascontiguousarray(v) for k, v in a.items() if isinstance(v, np.ndarray)}
    keep.update({k: np.ascontiguousarray(v) for k, v in extras.items()})
    v = lf.SceneView()

    def fp(k):
        return keep[k].ctypes.data_as(C.POINTER(C.c_float))

    v.nodes = fp("nodes")
    v.num_nodes = len(keep["nodes"])
    v.top_level_index = int(a["top_level_index"])
    v.vert_indices = keep["vert_indices"].ctypes.data_as(C.POINTER(C.c_int32))
    v.num_tris = len(keep["vert_indices"])
    v.vertices_uvx = fp("vertices")
    v.normals_uvy = fp("normals")
    v.num_vertices = len(keep["vertices"])
    v.materials = fp("materials")
    v.num_materials = len(keep["materials"])
    v.transforms = fp("transforms")
    v.num_instances = len(keep["transforms"])
    if len(keep["lights"]):
        v.lights = fp("lights")
        v.num_lights = len(keep["lights"])
    if "env_rgb" in keep:
        v.env_rgb = fp("env_rgb")
        v.env_marginal = fp("env_marginal")
        v.env_conditional = fp("env_conditional")
        v.env_height, v.env_width = keep["env_rgb"].shape[:2]
    if "textures" in keep:
        t = keep["textures"]
        v.textures = t.ctypes.data_as(C.POINTER(C.c_uint8))
        v.num_textures, v.tex_height, v.tex_width = t.shape[:3]
    return v, keep


CASES = {
    # name: samples
    "cornell": 2,
    "cornell_lights": 2,
    "cornell_textures": 2,
    "room": 2,
    "icospheres": 2,
    "icospheres_constbg_tiled": 1,
    "icospheres_lens": 1,
    "icospheres_absorb": 2,
}


def post_settings():
    """Display-pass settings of the post-process golden vectors: every tone map with
    RenderOptions' defaults, then vignette, chromatic aberration (offset and distortion forms),
    both together, and the preview path."""
    out = []
    for t in range(7):
        out.append(lf.PostParams.defaults(t))
    p = lf.PostParams.defaults(2)
    p.use_vignette, p.vignette_intensity, p.vignette_power = 1, 0.7, 1.5
    out.append(p)
    p = lf.PostParams.defaults(3)
    p.use_ca, p.ca_distance = 1, 0.5
    out.append(p)
    p = lf.PostParams.defaults(1)
    p.use_ca, p.use_ca_distortion, p.ca_distance = 1, 1, 0.8
    out.append(p)
    p = lf.PostParams.defaults(6)
    p.use_ca, p.use_ca_distortion, p.ca_distance, p.ca_p1, p.ca_p2, p.ca_p3 = 1, 1, 0.6, 2.0, 1.5, 0.4
    p.use_vignette, p.vignette_intensity, p.vignette_power = 1, 0.5, 2.5
    out.append(p)
    p = lf.PostParams.defaults(4)
    p.use_ca, p.preview = 1, 1                     # preview ignores chromatic aberration
    out.append(p)
    return out


POST_SAMPLES = 16


def post_input():
    """Accumulated sum over POST_SAMPLES samples fed to the display pass (24 x 40 RGB)."""
    rng = np.random.default_rng(0)
    return (rng.gamma(1.5, 1.0, (24, 40, 3)) * POST_SAMPLES).astype(np.float32)


def stored_params(meta_case):
    """Render parameters exactly as the golden vectors were made (the camera basis comes from
    the host's double-precision libm, which may round differently on another host)."""
    p = lf.RenderParams()
    for f, _ in p._fields_:
        v = meta_case["params"][f]
        if isinstance(v, list):
            arr = getattr(p, f)
            for i, x in enumerate(v):
                arr[i] = x
        else:
            setattr(p, f, v)
    return p
