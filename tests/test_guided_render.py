"""Guided rendering (learned path guiding in the wavefront pipeline): the one-sample MIS
estimator must stay unbiased (same image mean as BSDF sampling), and a trained guide must
lower the error at equal samples on the occluded-light room, where BSDF sampling rarely finds
the doorway the light comes through."""
import numpy as np
import pytest

import lavaframe_gb300 as lf

pytestmark = pytest.mark.gpu


def room():
    s = lf.HostScene().gen_room(4000, 4).build()
    a = s.arrays()
    top = int(a["top_level_index"])
    return s, a["nodes"][top][0:3], a["nodes"][top][3:6]


def render(ctx, ds, p, first, spp, guide=None, train_every=2, batch=8):
    f = lf.Frame(ctx, ds, p, lf.FRAME_FP64_ACCUM)
    f.set_batch(batch)
    if guide is not None:
        f.set_guide(guide, 0.5, train_every, 1e-2)
    f.render(first, spp)
    f.sync()
    img = f.accum64() / spp
    stats = f.guide_stats()
    f.close()
    return img, stats


def test_guided_estimator_is_unbiased_and_trains(ctx):
    s, lo, hi = room()
    p = s.render_params()
    p.width, p.height = 96, 54
    ds = ctx.upload(s)
    g = lf.Guide(ctx, lo, hi, seed=2)
    try:
        plain, _ = render(ctx, ds, p, 0, 2048)
        guided, st = render(ctx, ds, p, 50000, 2048, guide=g)
    finally:
        g.close()
        ds.close()
    assert st["adam_steps"] > 50 and st["training_samples"] > 100000
    m_plain, m_guided = plain.mean(), guided.mean()
    assert abs(m_guided - m_plain) < 0.03 * m_plain, (m_plain, m_guided)
    # 6 x 4 blocks of 16 x 13.5 pixels: local means agree too
    bp = plain[:52, :96].reshape(4, 13, 6, 16, 3).mean(axis=(1, 3, 4))
    bg = guided[:52, :96].reshape(4, 13, 6, 16, 3).mean(axis=(1, 3, 4))
    assert np.all(np.abs(bg - bp) < 0.1 * bp + 0.01 * m_plain), (bp, bg)


def test_trained_guide_lowers_error_at_equal_samples(ctx):
    s, lo, hi = room()
    p = s.render_params()
    p.width, p.height = 96, 54
    ds = ctx.upload(s)
    g = lf.Guide(ctx, lo, hi, seed=3)
    try:
        ref, _ = render(ctx, ds, p, 0, 8192, batch=64)
        render(ctx, ds, p, 20000, 512, guide=g, train_every=1)            # training run
        guided, _ = render(ctx, ds, p, 40000, 64, guide=g, train_every=0)  # frozen guide
        plain, _ = render(ctx, ds, p, 40000, 64)
    finally:
        g.close()
        ds.close()
    e_plain = np.sqrt(((plain - ref) ** 2).mean())
    e_guided = np.sqrt(((guided - ref) ** 2).mean())
    assert e_guided < 0.85 * e_plain, (e_plain, e_guided)


@pytest.mark.parametrize("tensor", [False, True])
def test_online_training_helps_for_every_seed(ctx, tensor):
    """Online training as the guiding workload runs it (batches of 16 samples, Adam after every
    second batch, lr 1e-2), repeated over four guide seeds and sample streams: every run's
    guide must lower the error at equal samples, and the worst run is bounded. Inference on
    the warp-level kernel and on tcgen05."""
    s, lo, hi = room()
    p = s.render_params()
    p.width, p.height = 96, 54
    ds = ctx.upload(s)
    ratios = []
    try:
        ref, _ = render(ctx, ds, p, 0, 8192, batch=64)
        plain, _ = render(ctx, ds, p, 90000, 64)
        e_plain = np.sqrt(((plain - ref) ** 2).mean())
        for seed in range(1, 5):
            g = lf.Guide(ctx, lo, hi, seed=seed)
            g.set_tensor_path(tensor)
            try:
                _, st = render(ctx, ds, p, 20000 * seed, 384, guide=g, train_every=2, batch=16)
                guided, _ = render(ctx, ds, p, 90000, 64, guide=g, train_every=0)
            finally:
                g.close()
            assert st["adam_steps"] > 0
            ratios.append(float(np.sqrt(((guided - ref) ** 2).mean()) / e_plain))
    finally:
        ds.close()
    assert max(ratios) < 0.95, ratios
    assert np.mean(ratios) < 0.85, ratios
    assert ctx.device_errors() == 0
