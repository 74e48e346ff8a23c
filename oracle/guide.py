"""CPU oracle of the learned path-guiding model (test infrastructure, FP64 numpy).

The model (identical definition to the device kernels in lavaframe_gb300/csrc/device/lf_guide.cu):

  input (64)  = 8 hash-grid levels x 4 features of the shading position, normalised to the scene
                box (trilinear interpolation of the level's vertex table; dense index while the
                level's vertices fit the table, else the spatial hash x*1 ^ y*2654435761 ^
                z*805459861 mod T), followed by one-blob encodings (8 Gaussian bins, sigma 1/8)
                of theta/pi and phi/(2 pi) of the outgoing direction and of the shading normal;
  MLP         = 64 -> 64 -> 64 -> 64 -> 48, ReLU after the hidden layers, no biases;
  mixture     = 8 von Mises-Fisher lobes from outputs 0..39, per lobe (mu_raw xyz, kappa_raw,
                logit): mu = mu_raw / sqrt(|mu_raw|^2 + 1e-6), kappa = exp(clamp(kappa_raw, -3, 7)),
                weights = softmax(logits); pdf(w) = sum_i pi_i k_i / (2 pi (1 - exp(-2 k_i)))
                * exp(k_i (mu_i . w - 1)); the sampling mixture (`pdf`, what guided rendering
                draws from) normalises mu_i exactly, mu_raw / |mu_raw|, so that it is a density of
                unit directions; the loss keeps the regularised mean above;
  loss        = mean over samples of -weight * log(pdf(direction) + 1e-12): weighted maximum
                likelihood of directions sampled by the tracer, weighted by the luminance of the
                incident radiance they carried over the pdf they were sampled with (the KL
                objective of neural importance sampling, Mueller et al. 2019).

No reference counterpart: LavaFrame samples directions from the BSDF only. Only tests use this
module, to check the device gradients.
"""
from __future__ import annotations

import numpy as np

LEVELS = 8
FEATURES = 4
LOG2_T = 14
T = 1 << LOG2_T
BASE_RES = 16
MAX_RES = 512
BLOB_BINS = 8
BLOB_SIGMA = 1.0 / 8.0
LOBES = 8
HIDDEN = 64
OUT = 48
P1, P2, P3 = 1, 2654435761, 805459861


def level_resolutions():
    """Integer grid resolution per level (the device receives these integers)."""
    b = np.exp((np.log(MAX_RES) - np.log(BASE_RES)) / (LEVELS - 1))
    return [int(np.floor(BASE_RES * b ** l)) for l in range(LEVELS)]


def vertex_index(res, x, y, z):
    n = res + 1
    if n * n * n <= T:
        return (x + y * n + z * n * n).astype(np.int64)
    h = (x.astype(np.uint64) * np.uint64(P1)) ^ (y.astype(np.uint64) * np.uint64(P2)) ^ \
        (z.astype(np.uint64) * np.uint64(P3))
    return ((h & np.uint64(0xFFFFFFFF)) % np.uint64(T)).astype(np.int64)


def grid_corners(p01):
    """Per level: corner table indices (N, 8) and trilinear weights (N, 8)."""
    out = []
    for l, res in enumerate(level_resolutions()):
        pos = np.clip(p01, 0.0, 1.0) * res
        i0 = np.minimum(np.floor(pos).astype(np.int64), res - 1)
        fr = pos - i0
        idx = np.empty((len(p01), 8), np.int64)
        wts = np.empty((len(p01), 8), np.float64)
        for c in range(8):
            dx, dy, dz = c & 1, (c >> 1) & 1, (c >> 2) & 1
            idx[:, c] = vertex_index(res, i0[:, 0] + dx, i0[:, 1] + dy, i0[:, 2] + dz)
            wts[:, c] = (np.where(dx, fr[:, 0], 1 - fr[:, 0]) * np.where(dy, fr[:, 1], 1 - fr[:, 1]) *
                         np.where(dz, fr[:, 2], 1 - fr[:, 2]))
        out.append((idx, wts))
    return out


def sph01(d):
    """(theta/pi, phi/(2 pi)) of unit vectors, phi = atan2(y, x) + pi."""
    th = np.arccos(np.clip(d[:, 2], -1.0, 1.0)) / np.pi
    ph = (np.arctan2(d[:, 1], d[:, 0]) + np.pi) / (2 * np.pi)
    return th, ph


def one_blob(s):
    c = (np.arange(BLOB_BINS) + 0.5) / BLOB_BINS
    return np.exp(-0.5 * ((s[:, None] - c[None, :]) / BLOB_SIGMA) ** 2)


def encode(grid, p01, wo, n):
    """Input vectors (N, 64) and the corner data needed for the grid gradient."""
    corners = grid_corners(p01)
    feats = []
    for l, (idx, wts) in enumerate(corners):
        tab = grid[l][idx]                       # (N, 8, F)
        feats.append((tab * wts[:, :, None]).sum(axis=1))
    a, b = sph01(wo)
    c, d = sph01(n)
    x = np.concatenate(feats + [one_blob(a), one_blob(b), one_blob(c), one_blob(d)], axis=1)
    return x, corners


def forward(W, x):
    """Pre-activations and activations of the MLP; returns (hs, out) with hs[0] = x."""
    hs = [x]
    h = x
    for l in range(3):
        h = np.maximum(W[l] @ h.T, 0.0).T
        hs.append(h)
    out = (W[3] @ h.T).T
    return hs, out


def mixture(out):
    o = out[:, :40].reshape(-1, LOBES, 5)
    raw = o[:, :, 0:3]
    nrm = np.sqrt((raw * raw).sum(-1) + 1e-6)
    mu = raw / nrm[..., None]
    kr = o[:, :, 3]
    kap = np.exp(np.clip(kr, -3.0, 7.0))
    lg = o[:, :, 4]
    lg = lg - lg.max(axis=1, keepdims=True)
    e = np.exp(lg)
    pi = e / e.sum(axis=1, keepdims=True)
    return mu, kap, pi, raw, nrm, kr


def vmf(mu, kap, w):
    dot = (mu * w[:, None, :]).sum(-1)
    norm = kap / (2 * np.pi * (1 - np.exp(-2 * kap)))
    return norm * np.exp(kap * (dot - 1.0)), dot


def pdf(out, w):
    """Density of the sampling mixture: lobe means normalised exactly (zero raw vectors: +z)."""
    _, kap, pi, raw, *_ = mixture(out)
    ln = np.sqrt((raw * raw).sum(-1))
    unit = np.where(ln[..., None] > 1e-30, raw / np.maximum(ln, 1e-300)[..., None], np.array([0.0, 0.0, 1.0]))
    f, _ = vmf(unit, kap, w)
    return (pi * f).sum(1)


def loss_and_grads(grid, W, p01, wo, n, wdir, weight):
    """Loss (mean over samples) and its gradients w.r.t. the four weight matrices and the grid
    tables, in FP64."""
    N = len(p01)
    x, corners = encode(grid, p01, wo, n)
    hs, out = forward(W, x)
    mu, kap, pi, raw, nrm, kr = mixture(out)
    f, dot = vmf(mu, kap, wdir)
    q = (pi * f).sum(1)
    loss = float((-weight * np.log(q + 1e-12)).mean())
    # d loss_s / d q_s (mean over samples folded in)
    dq = -weight / (q + 1e-12) / N
    g_pi = dq[:, None] * f
    g_f = dq[:, None] * pi
    # softmax
    g_lg = pi * (g_pi - (pi * g_pi).sum(1, keepdims=True))
    # f = k/(2pi(1-e^{-2k})) exp(k(dot-1))
    e2 = np.exp(-2 * kap)
    dlogf_dk = 1.0 / kap - 2 * e2 / (1 - e2) + (dot - 1.0)
    g_k = g_f * f * dlogf_dk
    g_kr = g_k * kap * ((kr > -3.0) & (kr < 7.0))
    g_mu = (g_f * f * kap)[..., None] * wdir[:, None, :]
    # mu = raw / nrm
    g_raw = (g_mu - mu * (g_mu * mu).sum(-1, keepdims=True)) / nrm[..., None]
    d_out = np.zeros_like(out)
    d5 = d_out[:, :40].reshape(-1, LOBES, 5)
    d5[:, :, 0:3] = g_raw
    d5[:, :, 3] = g_kr
    d5[:, :, 4] = g_lg
    d_out[:, :40] = d5.reshape(-1, 40)
    # MLP backward
    dW = [None] * 4
    dW[3] = d_out.T @ hs[3]
    g = d_out @ W[3]
    for l in (2, 1, 0):
        g = g * (hs[l + 1] > 0)
        dW[l] = g.T @ hs[l]
        g = g @ W[l]
    dx = g
    dgrid = [np.zeros_like(t) for t in grid]
    for l, (idx, wts) in enumerate(corners):
        gl = dx[:, l * FEATURES:(l + 1) * FEATURES]
        for c in range(8):
            np.add.at(dgrid[l], idx[:, c], wts[:, c:c + 1] * gl)
    return loss, dW, dgrid, d_out


def init_params(seed=0):
    """Grid tables U(-1e-4, 1e-4), weights U(-s, s) with s = sqrt(6 / (fan_in + fan_out))."""
    rng = np.random.default_rng(seed)
    grid = [rng.uniform(-1e-4, 1e-4, (T, FEATURES)) for _ in range(LEVELS)]
    shapes = [(HIDDEN, 64), (HIDDEN, HIDDEN), (HIDDEN, HIDDEN), (OUT, HIDDEN)]
    W = [rng.uniform(-1, 1, s) * np.sqrt(6.0 / (s[0] + s[1])) for s in shapes]
    W[3][40:] = 0.0
    return grid, W


def f16(a):
    return np.asarray(a, np.float64).astype(np.float16).astype(np.float64)
