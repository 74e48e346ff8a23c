"""Known-answer tests of the oracle's restatement of the shader's BSDF and intersection
building blocks (disney.glsl, sampling.glsl, intersection.glsl): analytic values, the
normalisation of the microfacet distributions, the slab test's three outcomes, and the
consistency of DisneySample with DisneyEval for a single-lobe material."""
import numpy as np
import pytest

import oracle


@pytest.fixture(scope="module", autouse=True)
def built():
    from lavaframe_gb300 import build as b

    b.build_oracle()


def test_dielectric_fresnel_known_answers():
    etas = np.array([1 / 1.5, 1 / 1.33, 1.5, 2.0], np.float32)
    normal = oracle.bsdf_fn("dielectric_fresnel", np.ones_like(etas), etas)
    # normal incidence: ((1 - eta) / (1 + eta))^2
    np.testing.assert_allclose(normal, ((1 - etas) / (1 + etas)) ** 2, rtol=1e-5)
    # total internal reflection leaving the denser medium at grazing angles
    tir = oracle.bsdf_fn("dielectric_fresnel", np.array([0.05, 0.2], np.float32), np.float32(1.5))
    assert np.all(tir == 1.0)
    # between the two ends the reflectance rises towards grazing incidence
    cos = np.linspace(1.0, 0.01, 64, dtype=np.float32)
    f = oracle.bsdf_fn("dielectric_fresnel", cos, np.float32(1 / 1.5))
    assert np.all(np.diff(f) >= -1e-7) and f[-1] > 0.8


@pytest.mark.parametrize("a", [0.1, 0.3, 0.7, 1.0])
def test_gtr2_is_normalised(a):
    # integral over the hemisphere of D(h) cos(theta_h) d(omega) = 1
    th = (np.arange(200000, dtype=np.float64) + 0.5) * (np.pi / 2) / 200000
    d = oracle.bsdf_fn("gtr2", np.cos(th).astype(np.float32), np.float32(a)).astype(np.float64)
    integral = (d * np.cos(th) * np.sin(th)).sum() * (np.pi / 2 / 200000) * 2 * np.pi
    assert abs(integral - 1.0) < 2e-3, integral


@pytest.mark.parametrize("a", [0.1, 0.5])
def test_gtr1_is_normalised(a):
    th = (np.arange(200000, dtype=np.float64) + 0.5) * (np.pi / 2) / 200000
    d = oracle.bsdf_fn("gtr1", np.cos(th).astype(np.float32), np.float32(a)).astype(np.float64)
    integral = (d * np.cos(th) * np.sin(th)).sum() * (np.pi / 2 / 200000) * 2 * np.pi
    assert abs(integral - 1.0) < 2e-3, integral


def test_smith_and_schlick_known_answers():
    # the shader's G1 form 1 / (NdotV + sqrt(a^2 + NdotV^2 - a^2 NdotV^2)) is 1/2 at normal view
    g = oracle.bsdf_fn("smith_g_ggx", np.ones(3, np.float32), np.array([0.1, 0.5, 1.0], np.float32))
    np.testing.assert_allclose(g, 0.5, rtol=1e-6)
    s = oracle.bsdf_fn("schlick_fresnel", np.array([1.0, 0.0, 0.5], np.float32))
    np.testing.assert_allclose(s, [0.0, 1.0, 0.5 ** 5], rtol=1e-6)


def test_aabb_entry_exit_and_miss():
    o = np.array([[-1, 0.5, 0.5], [0.5, 0.5, 0.5], [-1, 2, 0.5], [2, 0.5, 0.5], [0.5, 0.5, -3]], np.float32)
    d = np.array([[1, 0, 0], [1, 0, 0], [1, 0, 0], [1, 0, 0], [0, 0, 1]], np.float32)
    t = oracle.aabb(np.zeros(3), np.ones(3), o, d)
    # entry from outside, exit from inside, miss beside, box behind the ray, entry along z
    np.testing.assert_array_equal(t, np.array([1.0, 0.5, -1.0, -1.0, 3.0], np.float32))


def test_disney_sample_matches_eval_for_a_single_lobe():
    # metallic, no clearcoat, no transmission: DisneySample picks the specular lobe only, so its
    # pdf and value must be DisneyEval's at the sampled direction (up to the half vector being
    # the sampled one in DisneySample and normalize(L + V) in DisneyEval)
    mat = {"albedo_r": 0.9, "albedo_g": 0.6, "albedo_b": 0.3, "metallic": 1.0, "roughness": 0.4, "ior": 1.5,
           "at_distance": 1.0}
    wo = np.array([0.3, 0.2, 0.0], np.float32)
    wo[2] = np.sqrt(1 - wo[0] ** 2 - wo[1] ** 2)
    s = oracle.disney_samples(mat, 1 / 1.5, wo, 4096, seed=3)
    up = (s[:, 2] > 0) & (s[:, 6] > 0)
    assert up.mean() > 0.8
    np.testing.assert_allclose(s[up, 6], s[up, 10], rtol=5e-3)
    np.testing.assert_allclose(s[up, 3:6], s[up, 7:10], rtol=5e-3, atol=1e-6)
    below = s[:, 2] <= 0
    assert np.all(s[below, 3:7] == 0)


def test_white_metal_furnace():
    # a white metal (Schlick reflectance 1) returns almost all energy when it is nearly a
    # mirror: the estimator f cos / pdf averages to ~1 at low roughness, never exceeds 1, and
    # falls as roughness grows (single-scattering microfacets lose the light that scatters twice)
    wo = np.array([0.0, 0.0, 1.0], np.float32)
    means = []
    for rough in (0.02, 0.3, 0.8):
        mat = {"albedo_r": 1.0, "albedo_g": 1.0, "albedo_b": 1.0, "metallic": 1.0, "roughness": rough, "ior": 1.5,
               "at_distance": 1.0}
        s = oracle.disney_samples(mat, 1 / 1.5, wo, 20000, seed=5)
        ok = s[:, 6] > 0
        w = np.where(ok, s[:, 3] * np.maximum(s[:, 2], 0) / np.where(ok, s[:, 6], 1), 0.0)
        means.append(float(w.mean()))
    assert 0.95 < means[0] < 1.02, means
    assert all(0.0 < m < 1.02 for m in means), means
    assert means[0] > means[1] > means[2], means
