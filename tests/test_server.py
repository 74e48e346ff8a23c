"""Serving loop (lf_server): continuous batching of jobs of different scenes, memory-budget
admission and LRU eviction. Each job's image must be the one lf_frame_render gives for the
same scene and parameters, bit for bit, whether it ran alone or among other jobs."""
import numpy as np
import pytest

import lavaframe_gb300 as lf
import oracle
from tests import scenes

pytestmark = pytest.mark.gpu


def frame_alone(ctx, s, p, spp):
    ds = ctx.upload(s)
    f = lf.Frame(ctx, ds, p)
    f.render(0, spp)
    f.sync()
    out = f.accum()
    f.close()
    ds.close()
    return out


def job_mix():
    cornell = scenes.build("cornell")
    ico = lf.HostScene().gen_icospheres(6, 3, 5, 64, 32).build()
    room = lf.HostScene().gen_room(300, 4).build()
    jobs = []
    for s, size, spp, depth in ((cornell, (64, 64), 5, 4), (ico, (48, 27), 3, 8), (room, (40, 24), 4, 6),
                                (cornell, (32, 48), 2, 3), (ico, (64, 36), 2, 5)):
        p = s.render_params()
        p.width, p.height = size
        p.max_depth = depth
        jobs.append((s, p, spp))
    return jobs


def test_single_job_equals_frame_and_oracle(ctx):
    s = scenes.build("cornell")
    p = s.render_params()
    p.width, p.height = 48, 48
    srv = lf.Server(ctx)
    try:
        sid = srv.add_scene(s)
        jid = srv.submit(sid, p, 3)
        assert srv.wait(jid, 60000)
        got = srv.read(jid)
        info = srv.info(jid)
        assert info["state"] == lf.JOB_DONE and info["samples_done"] == 3
        assert info["finish_ms"] >= info["start_ms"] >= info["submit_ms"]
        srv.release(jid)
    finally:
        srv.close()
    ref_acc, _, _ = oracle.render(s.view(), p, 0, 3, want_paths=False)
    assert got.tobytes() == ref_acc.tobytes()
    assert got.tobytes() == frame_alone(ctx, s, p, 3).tobytes()


@pytest.mark.parametrize("paths_per_pass", [0, 1500])
def test_jobs_in_a_mix_equal_jobs_alone(ctx, paths_per_pass):
    """Five jobs of three scenes submitted together; small passes force many interleaved
    passes per job in the same engine steps."""
    jobs = job_mix()
    srv = lf.Server(ctx, paths_per_pass=paths_per_pass, passes_per_job=3)
    try:
        ids = {}
        got = {}
        for k, (s, p, spp) in enumerate(jobs):
            sid = ids.setdefault(id(s), srv.add_scene(s))
            got[k] = srv.submit(sid, p, spp)
        for k, jid in got.items():
            assert srv.wait(jid, 120000)
            got[k] = srv.read(jid)
            srv.release(jid)
        st = srv.stats()
        assert st["jobs_done"] == len(jobs)
        assert st["paths"] == sum(p.width * p.height * spp for _, p, spp in jobs)
    finally:
        srv.close()
    for k, (s, p, spp) in enumerate(jobs):
        assert got[k].tobytes() == frame_alone(ctx, s, p, spp).tobytes(), k


def test_depth_zero_job_beside_regular_jobs(ctx):
    """Multi-job steps with a job of depth 0 among regular ones: its paths are written out by
    the finish kernel (black image) while the others' images stay those they have alone."""
    cornell = scenes.build("cornell")
    ico = lf.HostScene().gen_icospheres(6, 3, 5, 64, 32).build()
    zero = ico.render_params()
    zero.width, zero.height, zero.max_depth = 40, 24, 0
    reg = cornell.render_params()
    reg.width, reg.height = 48, 32
    reg2 = ico.render_params()
    reg2.width, reg2.height = 40, 24
    srv = lf.Server(ctx, paths_per_pass=1500, passes_per_job=2)
    try:
        sc, si = srv.add_scene(cornell), srv.add_scene(ico)
        jobs = [(srv.submit(si, zero, 3), ico, zero, 3), (srv.submit(sc, reg, 3), cornell, reg, 3),
                (srv.submit(si, reg2, 2), ico, reg2, 2)]
        got = []
        for jid, _, _, _ in jobs:
            assert srv.wait(jid, 60000)
            got.append(srv.read(jid))
            srv.release(jid)
    finally:
        srv.close()
    assert not got[0].any()
    for img, (_, s, p, spp) in zip(got[1:], jobs[1:]):
        assert img.tobytes() == frame_alone(ctx, s, p, spp).tobytes()


def test_budget_evicts_idle_scenes_least_recently_used(ctx):
    """A budget that holds the engine pool and one scene at a time: alternating scenes
    upload and evict, and every result stays exact."""
    a = lf.HostScene().gen_icospheres(4, 4, 7, 64, 32).build()
    b = lf.HostScene().gen_icospheres(4, 4, 8, 64, 32).build()
    pool = ctx_pool_bytes(ctx)
    ds = ctx.upload(a)
    scene_bytes = ds.device_bytes()
    ds.close()
    budget = pool + scene_bytes + scene_bytes // 2 + (64 << 10)
    srv = lf.Server(ctx, memory_budget=budget, paths_per_pass=4096, passes_per_job=1)
    try:
        sa, sb = srv.add_scene(a), srv.add_scene(b)
        results = []
        for k, sid in enumerate([sa, sb, sa, sb]):
            s = a if sid == sa else b
            p = s.render_params()
            p.width, p.height = 32, 18
            jid = srv.submit(sid, p, 2)
            assert srv.wait(jid, 60000)
            results.append((s, p, srv.read(jid)))
            srv.release(jid)
        st = srv.stats()
        assert st["scene_evictions"] >= 3 and st["scene_uploads"] >= 4
        assert st["device_bytes"] <= budget
    finally:
        srv.close()
    for s, p, img in results:
        assert img.tobytes() == frame_alone(ctx, s, p, 2).tobytes()


def test_job_larger_than_budget_is_refused(ctx):
    s = scenes.build("cornell")
    srv = lf.Server(ctx, memory_budget=ctx_pool_bytes(ctx) + (1 << 20))
    try:
        sid = srv.add_scene(s)
        p = s.render_params()
        p.width, p.height = 2048, 2048
        with pytest.raises(lf.LFError):
            srv.submit(sid, p, 64)
    finally:
        srv.close()


def ctx_pool_bytes(ctx):
    info = ctx.engine_info()
    if not info["slots"]:
        ctx.configure_engine(0)
        info = ctx.engine_info()
    return info["device_bytes"]


def test_wait_times_out_then_completes(ctx):
    s = lf.HostScene().gen_icospheres(13, 5, 3, 256, 128).build()
    p = s.render_params()
    p.width, p.height = 640, 360
    srv = lf.Server(ctx)
    try:
        sid = srv.add_scene(s)
        jid = srv.submit(sid, p, 64)
        assert not srv.wait(jid, 0)
        assert srv.wait(jid, 120000)
        assert srv.info(jid)["samples_done"] == 64
    finally:
        srv.close()


def test_unreleased_jobs_fail_the_next_job_instead_of_blocking(ctx):
    """A budget that holds one job: while a finished job's buffers are not released, a job that
    does not fit fails at once (nothing running would free memory) instead of waiting forever;
    after the release the next job runs."""
    s = lf.HostScene().gen_icospheres(4, 4, 7, 64, 32).build()
    pool = ctx_pool_bytes(ctx)
    ds = ctx.upload(s)
    scene_bytes = ds.device_bytes()
    ds.close()
    p = s.render_params()
    p.width, p.height = 32, 18
    pix = p.width * p.height
    need = pix * 16 + 2 * pix * 16              # accumulation + one pass of 2 samples
    srv = lf.Server(ctx, memory_budget=pool + scene_bytes + need + 1024, paths_per_pass=4096, passes_per_job=1)
    try:
        sid = srv.add_scene(s)
        j1 = srv.submit(sid, p, 2)
        assert srv.wait(j1, 60000)
        j2 = srv.submit(sid, p, 2)
        with pytest.raises(lf.LFError):
            srv.wait(j2, 60000)
        assert srv.info(j2)["state"] == lf.JOB_FAILED
        assert "not released" in ctx.error()
        img1 = srv.read(j1)
        srv.release(j1)
        srv.release(j2)
        j3 = srv.submit(sid, p, 2)
        assert srv.wait(j3, 60000)
        assert srv.read(j3).tobytes() == img1.tobytes()
        srv.release(j3)
    finally:
        srv.close()
