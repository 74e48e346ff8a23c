"""GB300 path-tracing core for LavaFrame: Python bindings of the C ABI.

The native library (liblfcore.so, built in-tree by `lavaframe_gb300.build`) holds the host
scene layer (LavaFrame::Scene, BVH build and flatten, loader) and the sm_103a CUDA kernels.
This module only marshals arguments through ctypes; there is no Python or CPU fallback for
any GPU operation: if the library or a GPU is missing, calls raise.
"""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

import numpy as np

_HERE = Path(__file__).resolve().parent
LIB_PATH = _HERE / "liblfcore.so"

LF_OK = 0
STATUS = {0: "LF_OK", 1: "LF_ERR_INVALID", 2: "LF_ERR_CUDA", 3: "LF_ERR_OOM", 4: "LF_ERR_DEVICE",
          5: "LF_ERR_TIMEOUT", 6: "LF_ERR_STATE", 7: "LF_ERR_IO", 8: "LF_ERR_BUDGET"}
TRACE_LIGHTS = 0x1
TRACE_STATS = 0x2
TRACE_UNSORTED = 0x4
TRACE_SIMPLE = 0x8
FRAME_FP64_ACCUM = 0x1
FRAME_USE_GRAPH = 0x2
FRAME_TILED_FRAMES = 0x4
FRAME_PER_BATCH = 0x8

# symbol -> (restype, argtypes); kept in the same order as include/lavaframe_gb300.h
_P = C.c_void_p
_F = C.POINTER(C.c_float)
_I = C.POINTER(C.c_int32)
_SIG = {
    "lf_hscene_create": (C.c_int, [C.POINTER(_P)]),
    "lf_hscene_destroy": (None, [_P]),
    "lf_hscene_last_error": (C.c_char_p, [_P]),
    "lf_hscene_load_file": (C.c_int, [_P, C.c_char_p]),
    "lf_hscene_add_mesh": (C.c_int32, [_P, _F, _F, C.c_int32]),
    "lf_hscene_add_mesh_file": (C.c_int32, [_P, C.c_char_p]),
    "lf_hscene_add_material": (C.c_int32, [_P, _F]),
    "lf_hscene_add_instance": (C.c_int32, [_P, C.c_int32, _F, C.c_int32]),
    "lf_hscene_add_light": (C.c_int32, [_P, _F]),
    "lf_hscene_set_camera": (C.c_int, [_P, _F, _F, C.c_float, C.c_float, C.c_float]),
    "lf_hscene_add_hdr_file": (C.c_int, [_P, C.c_char_p]),
    "lf_hscene_add_hdr": (C.c_int, [_P, _F, C.c_int32, C.c_int32]),
    "lf_hscene_build": (C.c_int, [_P, C.c_int32]),
    "lf_hscene_set_instance": (C.c_int, [_P, C.c_int32, _F, C.c_int32]),
    "lf_hscene_rebuild_instances": (C.c_int, [_P]),
    "lf_hscene_view": (C.c_int, [_P, _P]),
    "lf_hscene_counts": (C.c_int, [_P, _I]),
    "lf_hscene_layout": (C.c_int, [_P, _I, _I, _I]),
    "lf_hscene_render_params": (C.c_int, [_P, _P]),
    "lf_gen_cornell": (C.c_int, [_P, C.c_int32, C.c_int32]),
    "lf_gen_cornell_tess": (C.c_int, [_P, C.c_int32, C.c_int32, C.c_int32]),
    "lf_gen_soup": (C.c_int, [_P, C.c_int32, C.c_int32, C.c_uint64]),
    "lf_gen_icospheres": (C.c_int, [_P, C.c_int32, C.c_int32, C.c_uint64, C.c_int32, C.c_int32]),
    "lf_gen_room": (C.c_int, [_P, C.c_int32, C.c_uint64]),
    "lf_gen_rays": (C.c_int, [_F, _F, C.c_int64, C.c_uint64, C.c_float, _F]),
    "lf_ctx_create": (C.c_int, [C.c_int32, C.POINTER(_P)]),
    "lf_ctx_destroy": (None, [_P]),
    "lf_ctx_last_error": (C.c_char_p, [_P]),
    "lf_ctx_device_errors": (C.c_uint32, [_P]),
    "lf_ctx_sync": (C.c_int, [_P]),
    "lf_ctx_timer_start": (C.c_int, [_P]),
    "lf_ctx_timer_stop": (C.c_int, [_P, _F]),
    "lf_ctx_configure_engine": (C.c_int, [_P, C.c_int32, C.c_int32, C.c_int32, C.c_int32, C.c_int32]),
    "lf_ctx_set_host_chunks": (C.c_int, [_P, C.c_int32]),
    "lf_ctx_set_engine_sort": (C.c_int, [_P, C.c_int32]),
    "lf_ctx_set_engine_drain": (C.c_int, [_P, C.c_int64]),
    "lf_ctx_kernel_timer": (C.c_int, [_P, C.c_int32]),
    "lf_ctx_device_attrs": (C.c_int, [_P, C.POINTER(C.c_int32), C.POINTER(C.c_int32)]),
    "lf_ctx_kernel_timer_read": (C.c_int, [_P, C.POINTER(C.c_double), C.POINTER(C.c_int64)]),
    "lf_ctx_engine_info": (C.c_int, [_P, C.POINTER(C.c_int64), C.POINTER(C.c_int64)]),
    "lf_scene_upload": (C.c_int, [_P, _P, C.POINTER(_P)]),
    "lf_scene_update_instances": (C.c_int, [_P, _P]),
    "lf_scene_release": (C.c_int, [_P]),
    "lf_scene_set_culling": (C.c_int, [_P, C.c_float, C.c_float]),
    "lf_scene_set_traversal": (C.c_int, [_P, C.c_int32]),
    "lf_scene_device_bytes": (C.c_size_t, [_P]),
    "lf_trace_closest": (C.c_int, [_P, _P, _F, C.c_int64, _P, C.c_uint32]),
    "lf_trace_any": (C.c_int, [_P, _P, _F, C.c_int64, _P, C.c_uint32]),
    "lf_trace_closest_device": (C.c_int, [_P, _P, _P, C.c_int64, _P, C.c_uint32]),
    "lf_trace_any_device": (C.c_int, [_P, _P, _P, C.c_int64, _P, C.c_uint32]),
    "lf_trace_stats": (C.c_int, [_P, C.POINTER(C.c_uint64)]),
    "lf_host_alloc": (C.c_int, [_P, C.c_size_t, C.POINTER(_P)]),
    "lf_host_free": (C.c_int, [_P, _P]),
    "lf_device_alloc": (C.c_int, [_P, C.c_size_t, C.POINTER(_P)]),
    "lf_device_free": (C.c_int, [_P, _P]),
    "lf_copy_to_device": (C.c_int, [_P, _P, _P, C.c_size_t]),
    "lf_copy_to_host": (C.c_int, [_P, _P, _P, C.c_size_t]),
    "lf_frame_create": (C.c_int, [_P, _P, _P, C.c_uint32, C.POINTER(_P)]),
    "lf_frame_render": (C.c_int, [_P, C.c_int32, C.c_int32]),
    "lf_frame_render_tile": (C.c_int, [_P, C.c_int32, C.c_int32, C.c_int32]),
    "lf_frame_sync": (C.c_int, [_P]),
    "lf_frame_read_accum": (C.c_int, [_P, _F]),
    "lf_frame_read_accum64": (C.c_int, [_P, C.POINTER(C.c_double)]),
    "lf_frame_read_paths": (C.c_int, [_P, _F, C.c_int32]),
    "lf_frame_reset": (C.c_int, [_P]),
    "lf_frame_counters": (C.c_int, [_P, C.POINTER(C.c_uint64)]),
    "lf_frame_set_batch": (C.c_int, [_P, C.c_int32]),
    "lf_frame_release": (C.c_int, [_P]),
    "lf_render_noalloc": (C.c_int, [_P, _P, C.c_int32, C.c_int32, _P]),
    "lf_frame_postprocess": (C.c_int, [_P, _P, C.c_int32, _P, _F]),
    "lf_write_png": (C.c_int, [C.c_char_p, _P, C.c_int32, C.c_int32]),
    "lf_write_ppm": (C.c_int, [C.c_char_p, _P, C.c_int32, C.c_int32]),
    "lf_write_pfm": (C.c_int, [C.c_char_p, _F, C.c_int32, C.c_int32]),
    "lf_write_bmp": (C.c_int, [C.c_char_p, _P, C.c_int32, C.c_int32]),
    "lf_write_tga": (C.c_int, [C.c_char_p, _P, C.c_int32, C.c_int32]),
    "lf_write_exr": (C.c_int, [C.c_char_p, _F, C.c_int32, C.c_int32]),
    "lf_write_jpg": (C.c_int, [C.c_char_p, _P, C.c_int32, C.c_int32, C.c_int32]),
    "lf_write_exr_compressed": (C.c_int, [C.c_char_p, _F, C.c_int32, C.c_int32, C.c_int32]),
    "lf_server_create": (C.c_int, [_P, _P, C.POINTER(_P)]),
    "lf_server_add_scene": (C.c_int, [_P, _P, C.POINTER(C.c_int64)]),
    "lf_server_remove_scene": (C.c_int, [_P, C.c_int64]),
    "lf_server_submit": (C.c_int, [_P, C.c_int64, _P, C.c_int32, C.POINTER(C.c_int64)]),
    "lf_server_job_info": (C.c_int, [_P, C.c_int64, _P]),
    "lf_server_wait": (C.c_int, [_P, C.c_int64, C.c_int32]),
    "lf_server_read": (C.c_int, [_P, C.c_int64, _F]),
    "lf_server_release_job": (C.c_int, [_P, C.c_int64]),
    "lf_server_get_stats": (C.c_int, [_P, _P]),
    "lf_server_destroy": (C.c_int, [_P]),
    "lf_guide_create": (C.c_int, [_P, _F, _F, C.c_uint64, C.POINTER(_P)]),
    "lf_guide_release": (C.c_int, [_P]),
    "lf_guide_get_params": (C.c_int, [_P, _F, _F]),
    "lf_guide_set_params": (C.c_int, [_P, _F, _F]),
    "lf_guide_gradients": (C.c_int, [_P, _F, C.c_int32, _F, _F, _F]),
    "lf_guide_train": (C.c_int, [_P, _F, C.c_int32, C.c_float, _F]),
    "lf_guide_train_device": (C.c_int, [_P, _P, C.c_int32, C.c_float]),
    "lf_guide_eval": (C.c_int, [_P, _F, C.c_int32, _F, _F]),
    "lf_guide_set_tensor_path": (C.c_int, [_P, C.c_int32]),
    "lf_frame_set_guide": (C.c_int, [_P, _P, C.c_float, C.c_int32, C.c_float]),
    "lf_frame_guide_stats": (C.c_int, [_P, C.POINTER(C.c_uint64), C.POINTER(C.c_uint64)]),
}


class SceneView(C.Structure):
    _fields_ = [("nodes", _F), ("num_nodes", C.c_int32), ("top_level_index", C.c_int32),
                ("vert_indices", _I), ("num_tris", C.c_int32),
                ("vertices_uvx", _F), ("normals_uvy", _F), ("num_vertices", C.c_int32),
                ("materials", _F), ("num_materials", C.c_int32),
                ("transforms", _F), ("num_instances", C.c_int32),
                ("lights", _F), ("num_lights", C.c_int32),
                ("env_rgb", _F), ("env_marginal", _F), ("env_conditional", _F),
                ("env_width", C.c_int32), ("env_height", C.c_int32),
                ("textures", C.POINTER(C.c_uint8)), ("tex_width", C.c_int32), ("tex_height", C.c_int32),
                ("num_textures", C.c_int32)]


class RenderParams(C.Structure):
    _fields_ = [("width", C.c_int32), ("height", C.c_int32), ("max_depth", C.c_int32),
                ("enable_rr", C.c_int32), ("rr_depth", C.c_int32), ("use_env_map", C.c_int32),
                ("use_constant_bg", C.c_int32), ("bg_color", C.c_float * 3), ("hdr_multiplier", C.c_float),
                ("cam_position", C.c_float * 3), ("cam_right", C.c_float * 3), ("cam_up", C.c_float * 3),
                ("cam_forward", C.c_float * 3), ("cam_fov", C.c_float), ("cam_focal_dist", C.c_float),
                ("cam_aperture", C.c_float), ("seed", C.c_uint32), ("frame_base", C.c_int32),
                ("tile_width", C.c_int32), ("tile_height", C.c_int32)]


HIT_DTYPE = np.dtype([("t", "<f4"), ("instance", "<i4"), ("prim", "<i4"), ("light", "<i4")])

_lib = None


def lib():
    """Loads liblfcore.so (building it is `lavaframe_gb300.build.build_core`)."""
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            raise RuntimeError(f"{LIB_PATH} is missing; run lavaframe_gb300.build.build_core() first")
        L = C.CDLL(str(LIB_PATH))
        for name, (res, args) in _SIG.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def exported_symbols():
    return list(_SIG)


class LFError(RuntimeError):
    def __init__(self, status, msg=""):
        super().__init__(f"{STATUS.get(status, status)}: {msg}")
        self.status = status


def _fp(a):
    return a.ctypes.data_as(_F)


def _chk(st, msg_fn=lambda: ""):
    if st != LF_OK:
        raise LFError(st, msg_fn())


class HostScene:
    """LavaFrame::Scene through the C ABI (lf_hscene_*)."""

    def __init__(self):
        self.h = _P()
        _chk(lib().lf_hscene_create(C.byref(self.h)))

    def close(self):
        if self.h:
            lib().lf_hscene_destroy(self.h)
            self.h = _P()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def error(self):
        return lib().lf_hscene_last_error(self.h).decode()

    def _c(self, st):
        _chk(st, self.error)

    def load_file(self, path):
        self._c(lib().lf_hscene_load_file(self.h, str(path).encode()))
        return self

    def add_mesh(self, verts, normals):
        v = np.ascontiguousarray(verts, np.float32).reshape(-1, 4)
        n = np.ascontiguousarray(normals, np.float32).reshape(-1, 4)
        mid = lib().lf_hscene_add_mesh(self.h, _fp(v), _fp(n), len(v))
        if mid < 0:
            raise LFError(1, self.error())
        return mid

    def add_material(self, m28):
        m = np.ascontiguousarray(m28, np.float32).reshape(28)
        return lib().lf_hscene_add_material(self.h, _fp(m))

    def add_instance(self, mesh, xf16, material):
        x = np.ascontiguousarray(xf16, np.float32).reshape(16)
        return lib().lf_hscene_add_instance(self.h, mesh, _fp(x), material)

    def add_light(self, l15):
        l = np.ascontiguousarray(l15, np.float32).reshape(15)
        return lib().lf_hscene_add_light(self.h, _fp(l))

    def set_camera(self, eye, at, fov_deg, aperture=0.0, focal=1.0):
        e = np.asarray(eye, np.float32)
        a = np.asarray(at, np.float32)
        self._c(lib().lf_hscene_set_camera(self.h, _fp(e), _fp(a), fov_deg, aperture, focal))

    def add_hdr(self, rgb):
        rgb = np.ascontiguousarray(rgb, np.float32)
        h, w = rgb.shape[:2]
        self._c(lib().lf_hscene_add_hdr(self.h, _fp(rgb), w, h))

    def build(self, threads=0):
        self._c(lib().lf_hscene_build(self.h, threads))
        return self

    def set_instance(self, i, xf16, material):
        x = np.ascontiguousarray(xf16, np.float32).reshape(16)
        self._c(lib().lf_hscene_set_instance(self.h, i, _fp(x), material))

    def rebuild_instances(self):
        self._c(lib().lf_hscene_rebuild_instances(self.h))

    def view(self) -> SceneView:
        v = SceneView()
        self._c(lib().lf_hscene_view(self.h, C.byref(v)))
        return v

    def render_params(self) -> RenderParams:
        p = RenderParams()
        self._c(lib().lf_hscene_render_params(self.h, C.byref(p)))
        return p

    def arrays(self):
        """Copies of the flat scene arrays (reference layouts) as numpy arrays."""
        v = self.view()

        def grab(ptr, n, cols, dtype=np.float32):
            if not ptr or n == 0:
                return np.zeros((0, cols), dtype)
            return np.ctypeslib.as_array(ptr, shape=(n * cols,)).astype(dtype, copy=True).reshape(n, cols)

        out = {
            "nodes": grab(v.nodes, v.num_nodes, 9),
            "top_level_index": v.top_level_index,
            "vert_indices": grab(v.vert_indices, v.num_tris, 3, np.int32),
            "vertices": grab(v.vertices_uvx, v.num_vertices, 4),
            "normals": grab(v.normals_uvy, v.num_vertices, 4),
            "materials": grab(v.materials, v.num_materials, 28),
            "transforms": grab(v.transforms, v.num_instances, 16),
            "lights": grab(v.lights, v.num_lights, 15),
        }
        if v.env_width > 0:
            out["env_rgb"] = grab(v.env_rgb, v.env_width * v.env_height, 3).reshape(v.env_height, v.env_width, 3)
            out["env_marginal"] = grab(v.env_marginal, v.env_height, 2)
            out["env_conditional"] = grab(v.env_conditional, v.env_width * v.env_height, 2)
        return out

    def layout(self):
        """(mesh vertex counts, instance mesh ids, instance material ids) before flattening."""
        cnt = (C.c_int32 * 4)()
        self._c(lib().lf_hscene_counts(self.h, cnt))
        mc = np.zeros(cnt[0], np.int32)
        im = np.zeros(cnt[1], np.int32)
        imat = np.zeros(cnt[1], np.int32)
        self._c(lib().lf_hscene_layout(self.h, mc.ctypes.data_as(_I), im.ctypes.data_as(_I), imat.ctypes.data_as(_I)))
        return mc, im, imat

    # procedural workloads
    def gen_cornell(self, width=256, height=256, subdiv=1):
        """Procedural Cornell box; subdiv > 1 splits every face into subdiv^2 quads."""
        if subdiv == 1:
            self._c(lib().lf_gen_cornell(self.h, width, height))
        else:
            self._c(lib().lf_gen_cornell_tess(self.h, width, height, subdiv))
        return self

    def gen_soup(self, instances, tris_per_instance, seed=1):
        self._c(lib().lf_gen_soup(self.h, instances, tris_per_instance, seed))
        return self

    def gen_icospheres(self, instances=64, level=6, seed=3, env_w=1024, env_h=512):
        self._c(lib().lf_gen_icospheres(self.h, instances, level, seed, env_w, env_h))
        return self

    def gen_room(self, boxes, seed=4):
        self._c(lib().lf_gen_room(self.h, boxes, seed))
        return self


def gen_rays(lo, hi, n, seed=2, tmax=1.0e6):
    out = np.empty((n, 8), np.float32)
    lo = np.asarray(lo, np.float32)
    hi = np.asarray(hi, np.float32)
    _chk(lib().lf_gen_rays(_fp(lo), _fp(hi), n, seed, tmax, _fp(out)))
    return out


class Context:
    """One GPU, one stream (lf_ctx)."""

    def __init__(self, device=0):
        self.h = _P()
        _chk(lib().lf_ctx_create(device, C.byref(self.h)), lambda: "lf_ctx_create failed (no GPU?)")

    def error(self):
        return lib().lf_ctx_last_error(self.h).decode()

    def _c(self, st):
        _chk(st, self.error)

    def close(self):
        if self.h:
            lib().lf_ctx_destroy(self.h)
            self.h = _P()

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def sync(self):
        self._c(lib().lf_ctx_sync(self.h))

    def timer_start(self):
        self._c(lib().lf_ctx_timer_start(self.h))

    def timer_stop(self):
        ms = C.c_float()
        self._c(lib().lf_ctx_timer_stop(self.h, C.byref(ms)))
        return ms.value

    def device_errors(self):
        return lib().lf_ctx_device_errors(self.h)

    def configure_engine(self, slots=0, block_extend=0, block_shade=0, block_shadow=0, shade_threads_per_sm=0):
        """Pool size, kernel block sizes and shade register cap of the multi-job engine
        (0 = keep the pool / default)."""
        self._c(lib().lf_ctx_configure_engine(self.h, slots, block_extend, block_shade, block_shadow,
                                              shade_threads_per_sm))

    def device_attrs(self):
        """{"sm_count", "max_sm_mhz"} of the context's device."""
        n, mhz = C.c_int32(), C.c_int32()
        self._c(lib().lf_ctx_device_attrs(self.h, C.byref(n), C.byref(mhz)))
        return {"sm_count": n.value, "max_sm_mhz": mhz.value}

    def kernel_timer(self, on):
        """Times the traversal kernel of the device ray queries alone (CUDA events)."""
        self._c(lib().lf_ctx_kernel_timer(self.h, 1 if on else 0))

    def kernel_timer_read(self):
        """(summed milliseconds, launches) of the traversal kernels timed since the last read."""
        ms, n = C.c_double(), C.c_int64()
        self._c(lib().lf_ctx_kernel_timer_read(self.h, C.byref(ms), C.byref(n)))
        return ms.value, n.value

    def set_engine_drain(self, paths):
        """Paths in flight at which a frame run switches to the one-kernel drain (0 = never)."""
        self._c(lib().lf_ctx_set_engine_drain(self.h, int(paths)))

    def set_engine_sort(self, sort_by_material):
        """Engine sort-by-material: shade takes the paths that hit a surface grouped by the class
        of their material (results unchanged). True / 1 on, False / 0 off, "auto" / 2 (default)
        on for single-job renders of scenes with more than one material class."""
        mode = 2 if sort_by_material == "auto" else int(sort_by_material)
        self._c(lib().lf_ctx_set_engine_sort(self.h, mode))

    def set_host_chunks(self, chunks=0):
        """Pieces of host-buffer ray queries whose copies overlap tracing (0 = automatic)."""
        self._c(lib().lf_ctx_set_host_chunks(self.h, chunks))

    def engine_info(self):
        slots, nbytes = C.c_int64(), C.c_int64()
        self._c(lib().lf_ctx_engine_info(self.h, C.byref(slots), C.byref(nbytes)))
        return {"slots": slots.value, "device_bytes": nbytes.value}

    def upload(self, host_scene: HostScene) -> "DeviceScene":
        v = host_scene.view()
        return DeviceScene(self, v)

    def trace_closest(self, scene, rays, flags=0):
        rays = np.ascontiguousarray(rays, np.float32).reshape(-1, 8)
        hits = np.empty(len(rays), HIT_DTYPE)
        self._c(lib().lf_trace_closest(self.h, scene.h, _fp(rays), len(rays), hits.ctypes.data_as(_P), flags))
        return hits

    def trace_any(self, scene, rays, flags=0):
        rays = np.ascontiguousarray(rays, np.float32).reshape(-1, 8)
        occ = np.empty(len(rays), np.uint8)
        self._c(lib().lf_trace_any(self.h, scene.h, _fp(rays), len(rays), occ.ctypes.data_as(_P), flags))
        return occ

    def trace_stats(self):
        out = (C.c_uint64 * 3)()
        self._c(lib().lf_trace_stats(self.h, out))
        return list(out)


class DeviceScene:
    def __init__(self, ctx: Context, view: SceneView):
        self.ctx = ctx
        self.h = _P()
        ctx._c(lib().lf_scene_upload(ctx.h, C.byref(view), C.byref(self.h)))

    def set_traversal(self, wide):
        """1: 4-wide tree (default); 0: the reference's binary tree."""
        self.ctx._c(lib().lf_scene_set_traversal(self.h, 1 if wide else 0))

    def set_culling(self, rel, abs_margin=0.0):
        self.ctx._c(lib().lf_scene_set_culling(self.h, rel, abs_margin))

    def update_instances(self, host_scene: HostScene):
        v = host_scene.view()
        self.ctx._c(lib().lf_scene_update_instances(self.h, C.byref(v)))

    def device_bytes(self):
        return lib().lf_scene_device_bytes(self.h)

    def close(self):
        if self.h:
            lib().lf_scene_release(self.h)
            self.h = _P()


class PostParams(C.Structure):
    """lf_post_params: RenderOptions' display settings (tonemap 0..6, CA, vignette)."""
    _fields_ = [("tonemap", C.c_int32), ("use_ca", C.c_int32), ("use_ca_distortion", C.c_int32),
                ("use_vignette", C.c_int32), ("preview", C.c_int32), ("ca_distance", C.c_float),
                ("ca_p1", C.c_float), ("ca_p2", C.c_float), ("ca_p3", C.c_float),
                ("vignette_intensity", C.c_float), ("vignette_power", C.c_float)]

    @classmethod
    def defaults(cls, tonemap=2):
        """RenderOptions' defaults (Renderer.h:25-44)."""
        return cls(tonemap, 0, 0, 0, 0, 0.05, 5.0, -0.5, 0.5, 0.0, 1.0)


def write_image(path, img, jpg_quality=90, exr_compression=3):
    """PNG / BMP / TGA / JPEG / PPM from (H, W, 3) uint8, PFM / EXR from float32, chosen by the
    file extension (PNG otherwise); row 0 = bottom. EXR compression: 0 none, 1 RLE, 2 ZIPS,
    3 ZIP."""
    path = str(path)
    h, w = img.shape[:2]
    ext = path.rsplit(".", 1)[-1].lower()
    if ext in ("pfm", "exr"):
        a = np.ascontiguousarray(img, np.float32)
        if ext == "exr":
            _chk(lib().lf_write_exr_compressed(path.encode(), _fp(a), w, h, int(exr_compression)))
        else:
            _chk(lib().lf_write_pfm(path.encode(), _fp(a), w, h))
    else:
        a = np.ascontiguousarray(img, np.uint8)
        if ext in ("jpg", "jpeg"):
            _chk(lib().lf_write_jpg(path.encode(), a.ctypes.data_as(_P), w, h, int(jpg_quality)))
            return
        fn = {"ppm": lib().lf_write_ppm, "bmp": lib().lf_write_bmp, "tga": lib().lf_write_tga}.get(ext, lib().lf_write_png)
        _chk(fn(path.encode(), a.ctypes.data_as(_P), w, h))


class ServerConfig(C.Structure):
    _fields_ = [("memory_budget", C.c_uint64), ("paths_per_pass", C.c_int32), ("passes_per_job", C.c_int32)]


class JobInfo(C.Structure):
    _fields_ = [("state", C.c_int32), ("samples_done", C.c_int32), ("submit_ms", C.c_double),
                ("start_ms", C.c_double), ("finish_ms", C.c_double)]


class ServerStats(C.Structure):
    _fields_ = [("jobs_submitted", C.c_uint64), ("jobs_done", C.c_uint64), ("paths", C.c_uint64),
                ("ext_rays", C.c_uint64), ("shadow_rays", C.c_uint64), ("scene_uploads", C.c_uint64),
                ("scene_evictions", C.c_uint64), ("device_bytes", C.c_uint64), ("scenes_resident", C.c_int32),
                ("jobs_running", C.c_int32), ("jobs_queued", C.c_int32)]


JOB_QUEUED, JOB_RUNNING, JOB_DONE, JOB_FAILED = 0, 1, 2, 3


class Server:
    """Serving loop (lf_server): jobs of registered scenes, continuous batching on the GPU."""

    def __init__(self, ctx: Context, memory_budget=0, paths_per_pass=0, passes_per_job=0):
        self.ctx = ctx
        self.h = _P()
        self._scenes = {}   # id -> HostScene kept alive (the server re-uploads from its arrays)
        self._dims = {}
        cfg = ServerConfig(memory_budget, paths_per_pass, passes_per_job)
        ctx._c(lib().lf_server_create(ctx.h, C.byref(cfg), C.byref(self.h)))

    def add_scene(self, host_scene: "HostScene") -> int:
        v = host_scene.view()
        sid = C.c_int64()
        self.ctx._c(lib().lf_server_add_scene(self.h, C.byref(v), C.byref(sid)))
        self._scenes[sid.value] = host_scene
        return sid.value

    def remove_scene(self, sid):
        self.ctx._c(lib().lf_server_remove_scene(self.h, sid))
        self._scenes.pop(sid, None)

    def submit(self, sid, params: RenderParams, spp) -> int:
        jid = C.c_int64()
        self.ctx._c(lib().lf_server_submit(self.h, sid, C.byref(params), spp, C.byref(jid)))
        self._dims[jid.value] = (params.height, params.width)
        return jid.value

    def info(self, jid):
        out = JobInfo()
        self.ctx._c(lib().lf_server_job_info(self.h, jid, C.byref(out)))
        return {"state": out.state, "samples_done": out.samples_done, "submit_ms": out.submit_ms,
                "start_ms": out.start_ms, "finish_ms": out.finish_ms}

    def wait(self, jid, timeout_ms=-1):
        """True when done, False on timeout."""
        st = lib().lf_server_wait(self.h, jid, timeout_ms)
        if st == 5:
            return False
        self.ctx._c(st)
        return True

    def read(self, jid):
        h, w = self._dims[jid]
        out = np.empty((h, w, 3), np.float32)
        self.ctx._c(lib().lf_server_read(self.h, jid, _fp(out)))
        return out

    def release(self, jid):
        self.ctx._c(lib().lf_server_release_job(self.h, jid))
        self._dims.pop(jid, None)

    def stats(self):
        out = ServerStats()
        self.ctx._c(lib().lf_server_get_stats(self.h, C.byref(out)))
        return {k: getattr(out, k) for k, _ in out._fields_}

    def close(self):
        if self.h:
            lib().lf_server_destroy(self.h)
            self.h = _P()


GUIDE_WEIGHTS = 15360
GUIDE_GRID_PARAMS = 8 * 16384 * 4
GUIDE_SAMPLE_FLOATS = 16
GUIDE_MIX_FLOATS = 40


class Guide:
    """Learned path-guiding model (lf_guide): hash grid + MLP -> vMF mixture, trained on the GPU."""

    def __init__(self, ctx: Context, lo, hi, seed=0):
        self.ctx = ctx
        self.h = _P()
        lo = np.ascontiguousarray(lo, np.float32)
        hi = np.ascontiguousarray(hi, np.float32)
        ctx._c(lib().lf_guide_create(ctx.h, _fp(lo), _fp(hi), seed, C.byref(self.h)))

    def params(self):
        w = np.empty(GUIDE_WEIGHTS, np.float32)
        g = np.empty(GUIDE_GRID_PARAMS, np.float32)
        self.ctx._c(lib().lf_guide_get_params(self.h, _fp(w), _fp(g)))
        return w, g

    def set_params(self, w, g):
        w = np.ascontiguousarray(w, np.float32)
        g = np.ascontiguousarray(g, np.float32)
        self.ctx._c(lib().lf_guide_set_params(self.h, _fp(w), _fp(g)))

    def gradients(self, samples):
        samples = np.ascontiguousarray(samples, np.float32).reshape(-1, GUIDE_SAMPLE_FLOATS)
        dw = np.empty(GUIDE_WEIGHTS, np.float32)
        dg = np.empty(GUIDE_GRID_PARAMS, np.float32)
        loss = np.zeros(1, np.float32)
        self.ctx._c(lib().lf_guide_gradients(self.h, _fp(samples), len(samples), _fp(dw), _fp(dg), _fp(loss)))
        return float(loss[0]), dw, dg

    def train(self, samples, lr=1e-2):
        samples = np.ascontiguousarray(samples, np.float32).reshape(-1, GUIDE_SAMPLE_FLOATS)
        loss = np.zeros(1, np.float32)
        self.ctx._c(lib().lf_guide_train(self.h, _fp(samples), len(samples), lr, _fp(loss)))
        return float(loss[0])

    def set_tensor_path(self, tcgen05):
        """MLP inference on the tcgen05 tensor cores (True) or the warp-level mma.sync kernel."""
        self.ctx._c(lib().lf_guide_set_tensor_path(self.h, 1 if tcgen05 else 0))

    def eval(self, queries):
        q = np.ascontiguousarray(queries, np.float32).reshape(-1, GUIDE_SAMPLE_FLOATS)
        mix = np.empty((len(q), GUIDE_MIX_FLOATS), np.float32)
        pdf = np.empty(len(q), np.float32)
        self.ctx._c(lib().lf_guide_eval(self.h, _fp(q), len(q), _fp(mix), _fp(pdf)))
        return mix, pdf

    def close(self):
        if self.h:
            lib().lf_guide_release(self.h)
            self.h = _P()


class Frame:
    """Progressive render target (lf_frame)."""

    def __init__(self, ctx: Context, scene: DeviceScene, params: RenderParams, flags=0):
        self.ctx = ctx
        self.params = params
        self.h = _P()
        ctx._c(lib().lf_frame_create(ctx.h, scene.h, C.byref(params), flags, C.byref(self.h)))

    def render(self, first_sample, count):
        self.ctx._c(lib().lf_frame_render(self.h, first_sample, count))

    def sync(self):
        self.ctx._c(lib().lf_frame_sync(self.h))

    def accum(self):
        out = np.empty((self.params.height, self.params.width, 3), np.float32)
        self.ctx._c(lib().lf_frame_read_accum(self.h, _fp(out)))
        return out

    def accum64(self):
        out = np.empty((self.params.height, self.params.width, 3), np.float64)
        self.ctx._c(lib().lf_frame_read_accum64(self.h, out.ctypes.data_as(C.POINTER(C.c_double))))
        return out

    def paths(self, max_samples):
        out = np.empty((max_samples, self.params.height, self.params.width, 3), np.float32)
        self.ctx._c(lib().lf_frame_read_paths(self.h, _fp(out), max_samples))
        return out

    def reset(self):
        self.ctx._c(lib().lf_frame_reset(self.h))

    def counters(self):
        out = (C.c_uint64 * 4)()
        self.ctx._c(lib().lf_frame_counters(self.h, out))
        return list(out)

    def set_batch(self, spp):
        self.ctx._c(lib().lf_frame_set_batch(self.h, spp))

    def postprocess(self, samples, params=None):
        """Display pass: (rgb8, rgbf) of the accumulated sum over `samples`, row 0 = bottom."""
        params = params or PostParams.defaults()
        rgb8 = np.empty((self.params.height, self.params.width, 3), np.uint8)
        rgbf = np.empty((self.params.height, self.params.width, 3), np.float32)
        self.ctx._c(lib().lf_frame_postprocess(self.h, C.byref(params), samples, rgb8.ctypes.data_as(_P), _fp(rgbf)))
        return rgb8, rgbf

    def set_guide(self, guide, alpha=0.5, train_every=4, lr=1e-2):
        """Guided rendering with `guide` (None detaches); trains on every train_every-th sample."""
        self.ctx._c(lib().lf_frame_set_guide(self.h, guide.h if guide else None, alpha, train_every, lr))

    def guide_stats(self):
        steps, samples = C.c_uint64(), C.c_uint64()
        self.ctx._c(lib().lf_frame_guide_stats(self.h, C.byref(steps), C.byref(samples)))
        return {"adam_steps": steps.value, "training_samples": samples.value}

    def close(self):
        if self.h:
            lib().lf_frame_release(self.h)
            self.h = _P()
