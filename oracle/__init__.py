"""CPU oracle (test infrastructure): ctypes wrapper of oracle/liblfo.so.

The oracle restates the reference GLSL path tracer in scalar C++ and runs it on the host
cores. Only tests, the smoke check and the bench's CPU-baseline leg use it, to check results;
the product path never imports it.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB = HERE / "liblfo.so"
_lib = None


def lib():
    global _lib
    if _lib is None:
        if not LIB.exists():
            raise RuntimeError(f"{LIB} missing; build with lavaframe_gb300.build.build_oracle()")
        L = C.CDLL(str(LIB))
        P = C.c_void_p
        L.lfo_trace_closest.argtypes = [P, P, C.c_int64, P, C.c_int32, C.c_float, C.c_float, C.c_int32, P, P]
        L.lfo_trace_any.argtypes = [P, P, C.c_int64, P, C.c_int32, C.c_float, C.c_float, C.c_int32, P]
        L.lfo_render.argtypes = [P, P, C.c_int32, C.c_int32, P, P, C.c_int32, C.c_int32, C.c_int32, C.c_float,
                                 C.c_float, P]
        L.lfo_math.argtypes = [C.c_int32, P, P, C.c_int64, P]
        L.lfo_rand_sequence.argtypes = [C.c_float, C.c_float, C.c_int32, C.c_uint32, C.c_int32, P]
        L.lfo_postprocess.argtypes = [P, C.c_int32, C.c_int32, P, C.c_int32, P, P]
        L.lfo_bsdf_fn.argtypes = [C.c_int32, P, P, C.c_int64, P]
        L.lfo_aabb.argtypes = [P, P, C.c_int64, P]
        L.lfo_disney_samples.argtypes = [P, C.c_float, P, C.c_int32, C.c_uint32, P]
        _lib = L
    return _lib


MATH_FN = {"sin": 0, "cos": 1, "tan": 2, "atan2": 3, "acos": 4, "exp": 5, "log": 6, "pow": 7}


def contract(fn, x, y=None):
    """Evaluates a function of the arithmetic contract on the host, element-wise."""
    x = np.ascontiguousarray(x, np.float32)
    yy = None if y is None else np.ascontiguousarray(y, np.float32)
    out = np.empty_like(x)
    lib().lfo_math(MATH_FN[fn], x.ctypes.data, None if yy is None else yy.ctypes.data, x.size, out.ctypes.data)
    return out


BSDF_FN = {"dielectric_fresnel": 0, "gtr2": 1, "smith_g_ggx": 2, "gtr1": 3, "schlick_fresnel": 4}


def bsdf_fn(fn, x, y=None):
    """Element-wise DielectricFresnel(x, eta=y), GTR2(NdotH=x, a=y), SmithG_GGX(NdotV=x, a=y),
    GTR1(NdotH=x, a=y) or SchlickFresnel(x) of the restated shader."""
    x = np.ascontiguousarray(x, np.float32)
    yy = None if y is None else np.ascontiguousarray(np.broadcast_to(y, x.shape), np.float32)
    out = np.empty_like(x)
    lib().lfo_bsdf_fn(BSDF_FN[fn], x.ctypes.data, None if yy is None else yy.ctypes.data, x.size, out.ctypes.data)
    return out


def aabb(box_min, box_max, origins, directions):
    """AABBIntersect of each ray against one box: entry distance, exit distance from inside,
    or -1 for a miss."""
    box = np.ascontiguousarray(np.concatenate([box_min, box_max]), np.float32)
    rays = np.ascontiguousarray(np.concatenate([origins, directions], axis=1), np.float32)
    out = np.empty(len(rays), np.float32)
    lib().lfo_aabb(box.ctypes.data, rays.ctypes.data, len(rays), out.ctypes.data)
    return out


MATERIAL_FIELDS = ["albedo_r", "albedo_g", "albedo_b", "specular", "emission_r", "emission_g", "emission_b",
                   "anisotropic", "metallic", "roughness", "subsurface", "specular_tint", "sheen", "sheen_tint",
                   "clearcoat", "clearcoat_roughness", "spec_trans", "ior", "at_distance", "extinction_r",
                   "extinction_g", "extinction_b", "tex0", "tex1", "tex2", "tex3"]


def disney_samples(material, eta, wo, n, seed=1):
    """n DisneySample draws at a surface with normal +z and DisneyEval at each sampled direction:
    an (n, 11) array of L xyz, sampled f xyz, sampled pdf, evaluated f xyz, evaluated pdf."""
    m = np.zeros(len(MATERIAL_FIELDS), np.float32)
    for k, v in material.items():
        m[MATERIAL_FIELDS.index(k)] = v
    wo = np.ascontiguousarray(wo, np.float32)
    out = np.empty((n, 11), np.float32)
    lib().lfo_disney_samples(m.ctypes.data, float(eta), wo.ctypes.data, n, seed, out.ctypes.data)
    return out


def rand_sequence(px, py, frame, n, seed=0):
    out = np.empty(n, np.float32)
    lib().lfo_rand_sequence(px, py, frame, seed, n, out.ctypes.data)
    return out


HIT_DTYPE = np.dtype([("t", "<f4"), ("instance", "<i4"), ("prim", "<i4"), ("light", "<i4")])


def trace_closest(view, rays, lights=False, cull_rel=-1.0, cull_abs=0.0, threads=0, want_ties=False):
    """Hits (t, instance, packed triangle, light) per ray; cull_rel < 0 = shader semantics.
    With want_ties, also a per-ray flag: 1 where the closest triangle hit has an
    equal-distance competitor (the answer then depends only on the visit order)."""
    rays = np.ascontiguousarray(rays, np.float32).reshape(-1, 8)
    hits = np.empty(len(rays), HIT_DTYPE)
    stats = np.zeros(5, np.uint64)
    ties = np.zeros(len(rays), np.uint8) if want_ties else None
    lib().lfo_trace_closest(C.addressof(view), rays.ctypes.data, len(rays), hits.ctypes.data, int(lights), cull_rel,
                            cull_abs, threads, stats.ctypes.data, ties.ctypes.data if want_ties else None)
    return (hits, stats, ties) if want_ties else (hits, stats)


def trace_any(view, rays, lights=False, cull_rel=-1.0, cull_abs=0.0, threads=0):
    rays = np.ascontiguousarray(rays, np.float32).reshape(-1, 8)
    occ = np.empty(len(rays), np.uint8)
    stats = np.zeros(5, np.uint64)
    lib().lfo_trace_any(C.addressof(view), rays.ctypes.data, len(rays), occ.ctypes.data, int(lights), cull_rel,
                        cull_abs, threads, stats.ctypes.data)
    return occ, stats


def render(view, params, first_sample, num_samples, accum=None, want_paths=False, row_stride=1, row_offset=0,
           threads=0, cull_rel=-1.0, cull_abs=0.0):
    """Accumulated radiance (H, W, 3) float32 over the samples, in sample order, plus the
    per-sample path radiance when asked for, and counters [paths, extension rays, node
    visits, light clamps]."""
    H, W = params.height, params.width
    if accum is None:
        accum = np.zeros((H, W, 3), np.float32)
    paths = np.zeros((num_samples, H, W, 3), np.float32) if want_paths else None
    ctr = np.zeros(4, np.uint64)
    lib().lfo_render(C.addressof(view), C.addressof(params), first_sample, num_samples, accum.ctypes.data,
                     paths.ctypes.data if paths is not None else None, row_stride, row_offset, threads, cull_rel,
                     cull_abs, ctr.ctypes.data)
    return accum, paths, ctr


def postprocess(accum_rgb, params, samples):
    """postprocess.glsl on a (H, W, 3) accumulated sum: returns (rgb8, rgbf), row 0 = bottom.
    `params` is a lavaframe_gb300.PostParams (same field layout as the oracle's)."""
    acc = np.ascontiguousarray(accum_rgb, np.float32)
    h, w = acc.shape[:2]
    rgb8 = np.empty((h, w, 3), np.uint8)
    rgbf = np.empty((h, w, 3), np.float32)
    lib().lfo_postprocess(acc.ctypes.data, w, h, C.addressof(params), samples, rgb8.ctypes.data, rgbf.ctypes.data)
    return rgb8, rgbf
