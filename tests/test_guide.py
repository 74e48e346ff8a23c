"""Learned path guiding: the FP64 oracle against finite differences (CPU), and the GPU's FP16
tensor-core forward/backward against the oracle (gradient check), plus training progress."""
import numpy as np
import pytest

import lavaframe_gb300 as lf
from oracle import guide as G


def unit(a):
    return a / np.linalg.norm(a, axis=1, keepdims=True)


def random_batch(n, seed):
    rng = np.random.default_rng(seed)
    p = rng.uniform(0.02, 0.98, (n, 3))
    wo, nrm, wd = (unit(rng.normal(size=(n, 3))) for _ in range(3))
    w = rng.uniform(0.1, 2.0, n)
    return p, wo, nrm, wd, w


def records(p, wo, nrm, wd, w):
    rec = np.zeros((len(p), 16), np.float32)
    rec[:, 0:3], rec[:, 3:6], rec[:, 6:9], rec[:, 9:12], rec[:, 12] = p, wo, nrm, wd, w
    return rec


def test_oracle_gradients_match_finite_differences():
    grid, W = G.init_params(3)
    grid = [g * 1e3 for g in grid]
    p, wo, nrm, wd, w = random_batch(32, 1)
    _, dW, dg, _ = G.loss_and_grads(grid, W, p, wo, nrm, wd, w)
    eps = 1e-6
    for l, (i, j) in ((0, (5, 7)), (1, (0, 0)), (2, (17, 40)), (3, (39, 63))):
        Wp = [x.copy() for x in W]
        Wp[l][i, j] += eps
        Wm = [x.copy() for x in W]
        Wm[l][i, j] -= eps
        fd = (G.loss_and_grads(grid, Wp, p, wo, nrm, wd, w)[0] - G.loss_and_grads(grid, Wm, p, wo, nrm, wd, w)[0]) / (2 * eps)
        assert abs(fd - dW[l][i, j]) <= 1e-6 + 1e-4 * abs(fd)
    _, corners = G.encode(grid, p, wo, nrm)
    idx = corners[1][0][0, 5]
    gp = [x.copy() for x in grid]
    gp[1][idx, 2] += eps
    gm = [x.copy() for x in grid]
    gm[1][idx, 2] -= eps
    fd = (G.loss_and_grads(gp, W, p, wo, nrm, wd, w)[0] - G.loss_and_grads(gm, W, p, wo, nrm, wd, w)[0]) / (2 * eps)
    assert abs(fd - dg[1][idx, 2]) <= 1e-7 + 1e-4 * abs(fd)


def test_oracle_mixture_is_a_density():
    grid, W = G.init_params(5)
    rng = np.random.default_rng(2)
    out = rng.normal(size=(3, 48)) * 2.0
    # Monte Carlo over the sphere with uniform directions: E[pdf / (1 / 4pi)] = 1
    d = unit(rng.normal(size=(400000, 3)))
    for k in range(3):
        q = G.pdf(np.repeat(out[k:k + 1], len(d), axis=0), d)
        assert abs(q.mean() * 4 * np.pi - 1.0) < 0.03


def flat_params(grid, W):
    wflat = np.concatenate([W[0].ravel(), W[1].ravel(), W[2].ravel(), W[3].ravel()]).astype(np.float32)
    gflat = np.stack(grid).astype(np.float32).ravel()
    return wflat, gflat


@pytest.mark.gpu
@pytest.mark.parametrize("tensor", [False, True])
def test_device_gradients_match_fp64_oracle(ctx, tensor):
    """Loss, weight and grid gradients of the warp-level mma.sync kernel and of the tcgen05
    kernel (128-sample tiles; 1000 samples end on a partial tile) against the FP64 oracle."""
    grid, W = G.init_params(7)
    grid = [g * 2e3 for g in grid]             # grid features of order 0.1
    wflat, gflat = flat_params(grid, W)
    # the device computes with FP16 working copies: the oracle uses the same rounded values
    W16 = [G.f16(x) for x in W]
    grid16 = [G.f16(x) for x in grid]
    p, wo, nrm, wd, w = random_batch(1000, 3)
    gd = lf.Guide(ctx, [0, 0, 0], [1, 1, 1])
    try:
        gd.set_params(wflat, gflat)
        gd.set_tensor_path(tensor)
        loss, dw, dg = gd.gradients(records(p, wo, nrm, wd, w))
        assert ctx.device_errors() == 0
    finally:
        gd.close()
    ref_loss, ref_dW, ref_dg, _ = G.loss_and_grads(grid16, W16, p, wo, nrm, wd, w)
    assert abs(loss - ref_loss) <= 2e-3 * abs(ref_loss) + 1e-4
    offs = [0, 4096, 8192, 12288, 15360]
    for l in range(4):
        got = dw[offs[l]:offs[l + 1]].reshape(ref_dW[l].shape)
        rel = np.linalg.norm(got - ref_dW[l]) / np.linalg.norm(ref_dW[l])
        assert rel < 2e-2, (l, rel)
    ref_g = np.stack(ref_dg).ravel()
    rel = np.linalg.norm(dg - ref_g) / np.linalg.norm(ref_g)
    assert rel < 2e-2, rel


@pytest.mark.gpu
def test_device_pdf_matches_oracle(ctx):
    grid, W = G.init_params(9)
    grid = [g * 2e3 for g in grid]
    W = [x * 3.0 for x in W]                    # sharper lobes than at initialisation
    wflat, gflat = flat_params(grid, W)
    p, wo, nrm, wd, w = random_batch(512, 4)
    gd = lf.Guide(ctx, [0, 0, 0], [1, 1, 1])
    try:
        gd.set_params(wflat, gflat)
        gd.set_tensor_path(False)      # the warp-level kernel; tcgen05 has its own test below
        mix, pdf = gd.eval(records(p, wo, nrm, wd, w))
    finally:
        gd.close()
    x, _ = G.encode([G.f16(g) for g in grid], p, wo, nrm)
    _, out = G.forward([G.f16(m) for m in W], G.f16(x))
    ref = G.pdf(out, wd)
    np.testing.assert_allclose(pdf, ref, rtol=3e-2, atol=1e-4)
    assert np.all(np.diff(mix.reshape(-1, 8, 5)[:, :, 4], axis=1) >= 0)   # cumulative weights
    np.testing.assert_allclose(mix.reshape(-1, 8, 5)[:, -1, 4], 1.0)


@pytest.mark.gpu
@pytest.mark.parametrize("tensor", [False, True])
def test_training_fits_a_position_dependent_distribution(ctx, tensor):
    """Directions concentrated around an axis that depends on position: Adam on the GPU lowers
    the loss well below that of the initial (nearly uniform) mixture."""
    rng = np.random.default_rng(6)
    gd = lf.Guide(ctx, [0, 0, 0], [1, 1, 1], seed=1)
    gd.set_tensor_path(tensor)

    def batch(n):
        p = rng.uniform(0, 1, (n, 3))
        axis = unit(np.stack([np.cos(6 * p[:, 0]), np.sin(6 * p[:, 0]), 0.5 * np.ones(n)], 1))
        d = unit(axis + 0.15 * rng.normal(size=(n, 3)))
        wo = unit(rng.normal(size=(n, 3)))
        nrm = unit(rng.normal(size=(n, 3)))
        return records(p, wo, nrm, d, np.ones(n))

    try:
        first = gd.train(batch(16384), lr=1e-2)
        for _ in range(300):
            last = gd.train(batch(16384), lr=1e-2)
    finally:
        gd.close()
    # uniform density on the sphere: -log(1 / 4 pi) = 2.53
    assert first > 2.0
    assert last < first - 2.0, (first, last)


@pytest.mark.gpu
@pytest.mark.parametrize("n", [1000, 128 * 152 * 3 + 77])
def test_tcgen05_inference_matches_warp_mma_and_oracle(ctx, n):
    """MLP inference on the tcgen05 tensor cores (128-query tiles, TMEM accumulators) against
    the warp-level mma.sync kernel and the FP64 oracle on the same FP16 parameters; the second
    size runs several tiles per CTA and ends on a partial tile."""
    grid, W = G.init_params(11)
    grid = [g * 2e3 for g in grid]
    W = [x * 3.0 for x in W]
    wflat, gflat = flat_params(grid, W)
    p, wo, nrm, wd, w = random_batch(n, 5)
    rec = records(p, wo, nrm, wd, w)
    gd = lf.Guide(ctx, [0, 0, 0], [1, 1, 1])
    try:
        gd.set_params(wflat, gflat)
        gd.set_tensor_path(False)
        mix_w, pdf_w = gd.eval(rec)
        gd.set_tensor_path(True)
        mix_t, pdf_t = gd.eval(rec)
        assert ctx.device_errors() == 0
    finally:
        gd.close()
    np.testing.assert_allclose(mix_t, mix_w, rtol=1e-2, atol=1e-3)
    np.testing.assert_allclose(pdf_t, pdf_w, rtol=2e-2, atol=1e-4)
    close = np.isclose(mix_t, mix_w, rtol=1e-5, atol=1e-6).mean()
    assert close > 0.9, close     # most values agree to FP32 summation order
    m = min(n, 2000)
    x, _ = G.encode([G.f16(g) for g in grid], p[:m], wo[:m], nrm[:m])
    _, out = G.forward([G.f16(v) for v in W], G.f16(x))
    ref = G.pdf(out, wd[:m])
    # an FP16 rounding of a hidden activation can flip between the FP64 oracle and an FP32 sum
    # and move a sharp lobe's density by a few percent: bound almost all, and every one loosely
    rel = np.abs(pdf_t[:m] - ref) / (np.abs(ref) + 1e-4)
    assert (rel < 3e-2).mean() > 0.995, (rel < 3e-2).mean()
    assert rel.max() < 0.15, rel.max()
    rel_w = np.abs(pdf_w[:m] - ref) / (np.abs(ref) + 1e-4)
    assert np.median(rel) < 2 * np.median(rel_w) + 1e-6


@pytest.mark.gpu
@pytest.mark.parametrize("tensor", [False, True])
def test_sampling_mixture_means_are_unit_vectors(ctx, tensor):
    """Lobes whose raw mean vectors are near zero (an untrained or collapsing lobe) still sample
    unit directions: the mixture the guided shade draws from normalises every mean exactly, and
    its pdf is the oracle's sampling density."""
    grid, W = G.init_params(13)
    grid = [g * 2e3 for g in grid]
    W = [x.copy() for x in W]
    for i in range(8):
        W[3][5 * i:5 * i + 3] *= 1e-4          # mean rows of every lobe: |mu_raw| ~ 1e-5
    wflat, gflat = flat_params(grid, W)
    p, wo, nrm, wd, w = random_batch(700, 7)
    gd = lf.Guide(ctx, [0, 0, 0], [1, 1, 1])
    try:
        gd.set_params(wflat, gflat)
        gd.set_tensor_path(tensor)
        mix, pdf = gd.eval(records(p, wo, nrm, wd, w))
    finally:
        gd.close()
    mu = mix.reshape(-1, 8, 5)[:, :, 0:3]
    np.testing.assert_allclose(np.linalg.norm(mu, axis=-1), 1.0, atol=1e-5)
    x, _ = G.encode([G.f16(g) for g in grid], p, wo, nrm)
    _, out = G.forward([G.f16(v) for v in W], G.f16(x))
    ref = G.pdf(out, wd)
    rel = np.abs(pdf - ref) / (np.abs(ref) + 1e-4)
    assert (rel < 3e-2).mean() > 0.99, (rel < 3e-2).mean()
