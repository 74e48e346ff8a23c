"""ctypes wrapper of oracle/_ref/libref_host.so: the reference's host scene code plus a
harness (oracle/ref_host_harness.cpp). Used only by tests to pin the product's host layer."""
import ctypes as C

import numpy as np

ARRAYS = [("nodes", 9, np.float32), ("vert_indices", 3, np.int32), ("vertices", 4, np.float32),
          ("normals", 4, np.float32), ("transforms", 16, np.float32), ("materials", 28, np.float32),
          ("lights", 15, np.float32)]


class RefHost:
    def __init__(self, path):
        R = C.CDLL(str(path))
        P = C.c_void_p
        R.ref_scene_load.restype = P
        R.ref_scene_load.argtypes = [C.c_char_p]
        R.ref_scene_build.restype = P
        R.ref_scene_build.argtypes = [C.c_int, P, P, P, C.c_int, P, P, P, C.c_int, P]
        R.ref_scene_free.argtypes = [P]
        R.ref_scene_move_instances.argtypes = [P, C.c_int, P, P]
        R.ref_scene_array.restype = P
        R.ref_scene_array.argtypes = [P, C.c_int, C.POINTER(C.c_longlong)]
        R.ref_scene_top_level_index.argtypes = [P]
        R.ref_scene_camera.argtypes = [P, P, P]
        R.ref_camera.argtypes = [P, P, C.c_float, P]
        R.ref_hdr_tables.argtypes = [P, C.c_int, C.c_int, P, P]
        R.ref_load_obj.argtypes = [C.c_char_p, P, P, C.c_int]
        self.R = R

    def _arrays(self, h):
        out = {}
        for k, (name, cols, dt) in enumerate(ARRAYS):
            n = C.c_longlong()
            p = self.R.ref_scene_array(h, k, C.byref(n))
            if n.value == 0:
                out[name] = np.zeros((0, cols), dt)
                continue
            raw = np.ctypeslib.as_array(C.cast(p, C.POINTER(C.c_uint32)), shape=(n.value * cols,)).copy()
            out[name] = raw.view(dt).reshape(-1, cols)
        out["top_level_index"] = self.R.ref_scene_top_level_index(h)
        return out

    def load(self, path):
        h = self.R.ref_scene_load(str(path).encode())
        assert h, f"reference loader failed on {path}"
        out = self._arrays(h)
        cam = np.zeros(15, np.float32)
        opts = np.zeros(5, np.int32)
        self.R.ref_scene_camera(h, cam.ctypes.data, opts.ctypes.data)
        out["camera"] = cam
        out["options"] = opts
        self.R.ref_scene_free(h)
        return out

    def build(self, mesh_counts, vertices, normals, inst_mesh, transforms, inst_mat, materials):
        mc = np.ascontiguousarray(mesh_counts, np.int32)
        v = np.ascontiguousarray(vertices, np.float32)
        n = np.ascontiguousarray(normals, np.float32)
        im = np.ascontiguousarray(inst_mesh, np.int32)
        xf = np.ascontiguousarray(transforms, np.float32)
        imat = np.ascontiguousarray(inst_mat, np.int32)
        mats = np.ascontiguousarray(materials, np.float32)
        h = self.R.ref_scene_build(len(mc), mc.ctypes.data, v.ctypes.data, n.ctypes.data, len(im), im.ctypes.data,
                                   xf.ctypes.data, imat.ctypes.data, len(mats), mats.ctypes.data)
        out = self._arrays(h)
        self.R.ref_scene_free(h)
        return out

    def build_and_move(self, mesh_counts, vertices, normals, inst_mesh, transforms, inst_mat, materials, new_xf,
                       new_mat):
        """Arrays of the scene built with the reference's code, then after Scene::RebuildInstances
        with the instances' new transforms and materials."""
        mc = np.ascontiguousarray(mesh_counts, np.int32)
        v = np.ascontiguousarray(vertices, np.float32)
        n = np.ascontiguousarray(normals, np.float32)
        im = np.ascontiguousarray(inst_mesh, np.int32)
        xf = np.ascontiguousarray(transforms, np.float32)
        imat = np.ascontiguousarray(inst_mat, np.int32)
        mats = np.ascontiguousarray(materials, np.float32)
        h = self.R.ref_scene_build(len(mc), mc.ctypes.data, v.ctypes.data, n.ctypes.data, len(im), im.ctypes.data,
                                   xf.ctypes.data, imat.ctypes.data, len(mats), mats.ctypes.data)
        before = self._arrays(h)
        nx = np.ascontiguousarray(new_xf, np.float32)
        nm = np.ascontiguousarray(new_mat, np.int32)
        self.R.ref_scene_move_instances(h, len(nm), nx.ctypes.data, nm.ctypes.data)
        after = self._arrays(h)
        self.R.ref_scene_free(h)
        return before, after

    def camera(self, eye, at, fov):
        out = np.zeros(15, np.float32)
        e = np.asarray(eye, np.float32)
        a = np.asarray(at, np.float32)
        self.R.ref_camera(e.ctypes.data, a.ctypes.data, fov, out.ctypes.data)
        return out

    def hdr_tables(self, rgb):
        rgb = np.ascontiguousarray(rgb, np.float32)
        h, w = rgb.shape[:2]
        marg = np.zeros((h, 2), np.float32)
        cond = np.zeros((w * h, 2), np.float32)
        self.R.ref_hdr_tables(rgb.ctypes.data, w, h, marg.ctypes.data, cond.ctypes.data)
        return marg, cond

    def load_obj(self, path, cap=1 << 20):
        v = np.zeros((cap, 4), np.float32)
        n = np.zeros((cap, 4), np.float32)
        cnt = self.R.ref_load_obj(str(path).encode(), v.ctypes.data, n.ctypes.data, cap)
        assert cnt > 0
        return v[:cnt], n[:cnt]
