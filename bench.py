"""Benchmark of the GB300 path-tracing core.

Headline (the intersection microbench): closest-hit queries of 2^24 rays (origins uniform
in the scene box, directions uniform on the sphere, tmax = 1e6) against a 10,485,760-
triangle soup of 2^20 instances x 10 triangles built with the reference's BVH algorithm.
  value   Grays/s with rays and hits resident in HBM (CUDA events on the launching stream)
  e2e     the same through lf_trace_closest with page-locked host buffers: every step copies
          the rays in and the hits out
Roofline: the traversal kernel is bound by instruction issue under divergence, not by HBM
(its DRAM traffic is a few percent of peak), so `roofline` is its warp-instruction issue rate
(instructions per ray from the committed ncu summary x rays per second of the kernel alone,
timed with CUDA events around each launch) against 4 issue slots per SM per clock at the SM
clock sampled during the run; its DRAM bytes and their fraction of the measured HBM peak are
reported beside it.
Secondary numbers (reported under "extra"): progressive renders of the Cornell box
(256^2, 64 spp, depth 4; image RMSE against the 16k-spp FP64 oracle render), of the
13-icosphere ~1.06M-triangle scene and of the 64-icosphere 5.2M-triangle scene (1920x1080,
16 spp, depth 8) in Msamples/s and extension rays/s, guided vs plain time to the plain
1024-spp error on the occluded-light room at 1280x720, and the serving loop.

`--impl reference` times the CPU restatement of the reference traversal (the reference's
own GPU path is an OpenGL shader and cannot run here) on the host cores.
Multi-GPU: replicas only - every rank runs the full workload on its own GPU.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

import numpy as np  # noqa: E402


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--instances-log2", type=int, default=20)
    ap.add_argument("--rays-log2", type=int, default=24)
    ap.add_argument("--no-extras", action="store_true")
    ap.add_argument("--cpu-seconds", type=float, default=10.0, help="target length of the CPU baseline sample")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline (profiling runs)")
    ap.add_argument("--no-e2e", action="store_true", help="skip the host-buffer pass (profiling runs)")
    ap.add_argument("--host-chunks", type=int, default=0,
                    help="pieces of the host-buffer pass whose copies overlap tracing (0 = the library's choice)")
    ap.add_argument("--spp-batch", type=int, default=0, help="samples per wavefront batch of the render workloads")
    ap.add_argument("--frame-flags", type=int, default=0, help="lf_frame flags of the render workloads (8 = per-batch)")
    ap.add_argument("--engine-slots", type=int, default=0, help="path slots of the engine pool (0 = default)")
    ap.add_argument("--shade-cap", type=int, default=0, help="engine shade register cap, threads per SM (512/768/1024; 0 = 512)")
    ap.add_argument("--jobs", type=int, default=0, help="serving workload: number of jobs (0 = default)")
    ap.add_argument("--sort-by-material", type=int, default=-1, choices=[-1, 0, 1, 2],
                    help="render workloads: engine sort-by-material mode (0 off, 1 on, 2 auto; -1 the default)")
    ap.add_argument("--engine-drain", type=int, default=-1, help="render workloads: engine drain threshold (paths)")
    ap.add_argument("--autotune", action="store_true", help="render workloads: autotune the engine first")
    ap.add_argument("--traversal", default="wide", choices=["wide", "binary"], help="BVH traversal")
    ap.add_argument("--c4-size", default="1280x720", help="guiding workload resolution WxH")
    ap.add_argument("--render-size", default="", help="c1/c3 workloads: override the resolution WxH (profiling)")
    ap.add_argument("--c4-ref-spp", type=int, default=16384, help="guiding workload reference samples")
    ap.add_argument("--c4-alpha", type=float, default=0.5, help="guiding workload: mixture selection probability")
    ap.add_argument("--c4-every", type=int, default=2, help="guiding workload: train after every n-th batch")
    ap.add_argument("--c4-batch", type=int, default=16, help="guiding workload: samples per batch")
    ap.add_argument("--c4-lr", type=float, default=1e-2, help="guiding workload: Adam learning rate")
    ap.add_argument("--c4-tensor", type=int, default=-1,
                    help="guiding workload: MLP on mma.sync (0), tcgen05 (1) or both (-1)")
    ap.add_argument("--workload", default="microbench",
                    choices=["microbench", "c1", "c3", "c3full", "c4", "c4batches", "c5"],
                    help="microbench = headline; c1/c3/c3full = one render workload alone (profiling)")
    return ap.parse_args()


def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as td

        td.init_process_group("gloo", init_method="env://")
    return world, rank, local


def barrier(world):
    if world > 1:
        import torch.distributed as td

        td.barrier()


def max_over_ranks(world, x):
    if world == 1:
        return x
    import torch
    import torch.distributed as td

    t = torch.tensor([x], dtype=torch.float64)
    td.all_reduce(t, op=td.ReduceOp.MAX)
    return float(t.item())


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms during a region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except (FileNotFoundError, OSError):
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], 0.0, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = max(mx, float(f[2]))
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": mx, "reasons": sorted(reasons), "samples": len(sm)}


def measured_peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def build_soup(inst_log2):
    import lavaframe_gb300 as lf

    t = time.time()
    s = lf.HostScene().gen_soup(1 << inst_log2, 10, 1)
    t_gen = time.time() - t
    t = time.time()
    s.build()
    t_build = time.time() - t
    return s, t_gen, t_build


def soup_rays(s, n):
    import lavaframe_gb300 as lf

    a = s.view()
    nodes = np.ctypeslib.as_array(a.nodes, shape=(a.num_nodes * 9,)).reshape(-1, 9)
    root = nodes[a.top_level_index]
    return lf.gen_rays(root[0:3], root[3:6], n, 2), root


PROFILE_KEYS = ("warp_inst_per_ray", "lanes_per_inst", "dram_bytes_per_ray", "l2_bytes_per_ray")


def traversal_profile():
    """Per-ray counters of the traversal kernel from the committed ncu summaries (the
    full-scene capture first, then the reduced one): warp instructions, active lanes per
    instruction, DRAM and L2 bytes."""
    vals = {}
    for name in ("c2_trace_wide_full.md", "c2_trace_wide_small.md"):
        prof = ROOT / "profiles" / name
        if not prof.exists():
            continue
        for line in prof.read_text().splitlines():
            for key in PROFILE_KEYS:
                if line.startswith(key + ":") and key not in vals:
                    vals[key] = float(line.split(":")[1].split()[0])
                    vals[key + "_from"] = f"profiles/{name}"
    return vals


def algorithmic_bytes_per_ray(stats, nrays):
    """Reference data model: 32 B ray + 16 B hit, 36 B per node box tested (two per inner
    node visit), 60 B per triangle test (12 B indices + 3 x 16 B vertices), 64 B per
    instance entered (its transform)."""
    inner, tris, inst = float(stats[0]), float(stats[1]), float(stats[4])
    return 32.0 + 16.0 + (36.0 * 2.0 * inner + 60.0 * tris + 64.0 * inst) / nrays


def cpu_baseline(view, rays, target_s):
    """The oracle's ClosestHit with the shader's semantics (no distance culling: every box the
    reference's traversal would test is tested) on all host threads, over a leading sample of
    the rays sized to take about target_s seconds."""
    import oracle

    threads = os.cpu_count() or 1
    n = min(len(rays), 1 << 14)
    t = time.time()
    _, st = oracle.trace_closest(view, rays[:n], threads=threads)
    dt = max(time.time() - t, 1e-3)
    m = int(min(len(rays), max(n, n * target_s / dt)))
    m = max(n, (m // n) * n)
    t = time.time()
    _, st = oracle.trace_closest(view, rays[:m], threads=threads)
    dt = time.time() - t
    return m / dt / 1e9, threads, m, dt, st


def run_reference(args, world, rank):
    if rank != 0:
        return
    import lavaframe_gb300 as lf  # host scene layer only (BVH build), no GPU
    import oracle

    from lavaframe_gb300 import build as b
    b.build_core()
    b.build_oracle()
    # The scene and rays come from the product's host layer: the GPU host has no reference
    # checkout, and the layer's node arrays are byte-identical to the reference's own build.
    s, _, _ = build_soup(args.instances_log2)
    rays, root = soup_rays(s, 1 << args.rays_log2)
    view = s.view()
    threads = os.cpu_count() or 1
    # ClosestHit with the shader's semantics: no distance culling (closest_hit.glsl:69-201)
    n = min(len(rays), 1 << 14)
    t = time.time()
    oracle.trace_closest(view, rays[:n], threads=threads)
    per = (time.time() - t) / n
    sample = int(min(len(rays), max(n, 5.0 / max(per, 1e-9))))
    sample = max(n, (sample // n) * n)
    for i in range(args.warmup):
        oracle.trace_closest(view, rays[:n], threads=threads)
    times = []
    for i in range(args.steps):
        off = (i * sample) % max(1, len(rays) - sample + 1)
        t = time.time()
        oracle.trace_closest(view, rays[off:off + sample], threads=threads)
        times.append(time.time() - t)
    total = sum(times)
    v = sample * args.steps / total / 1e9
    line = {
        "impl": "reference", "metric": "closest-hit Grays/s (intersection microbench)", "value": v, "unit": "Grays/s",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup, "ms_per_step": total / args.steps * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": f"intersection microbench: {1 << args.instances_log2} instances x 10 triangles, "
                               f"2^{args.rays_log2} rays (each step a {sample}-ray sample)",
                   "parallelism": "host threads"},
        "cpu_baseline": {"value": v, "unit": "Grays/s", "cores": threads, "kind": "port",
                         "sample": f"{sample} rays per step of the 2^{args.rays_log2}-ray set"},
        "e2e": {"value": v, "unit": "Grays/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "note": "the reference traces in an OpenGL fragment shader that cannot run on this host; "
                "this arm times the scalar C++ restatement of its ClosestHit (shader semantics, no distance "
                "culling) on all host cores; scene and rays are built by the product's host layer, whose node "
                "arrays are byte-identical to the reference's build; each step is a sample of the 2^24 rays",
    }
    print(json.dumps(line), flush=True)


def c1_reference_image():
    """The Cornell box's 16,384-spp FP64-accumulated oracle render (a committed fixture made by
    tests/golden/make_c1_reference.py), or None."""
    path = ROOT / "tests" / "golden" / "c1_reference_16k.npz"
    if not path.exists():
        return None
    g = np.load(path)
    return g["mean"].astype(np.float64), int(g["spp"])


def render_extra(ctx, which, spp=None, spp_batch=0, flags=0, tune=False, wide=True, size=None, sort=None):
    """One render workload on the engine (or the per-batch pipeline with flags=8). sort: None
    keeps the engine's sort-by-material mode (default "auto": sorted when the scene mixes
    material classes), else the mode to render with (0 off, 1 on)."""
    import lavaframe_gb300 as lf

    if which == "c1":
        s = lf.HostScene().gen_cornell(256, 256).build()
        spp = spp or 64
    else:
        s = lf.HostScene().gen_icospheres(64 if which == "c3full" else 13, 6, 3, 1024, 512).build()
        spp = spp or 16
    p = s.render_params()
    if size:
        p.width, p.height = size
    ds = ctx.upload(s)
    ds.set_traversal(wide)
    tuned = None
    if tune:
        from lavaframe_gb300 import autotune

        tuned = autotune.tune(ctx, ds, p, spp=spp, triangles=int(s.view().num_tris))
    if sort is not None:
        ctx.set_engine_sort(sort)
    f = lf.Frame(ctx, ds, p, flags)
    if spp_batch:
        f.set_batch(spp_batch)
    f.render(0, 1)
    f.sync()
    runs = []
    for _ in range(2):   # two timed renders of the same samples; the faster one is reported
        f.reset()
        ctx.timer_start()
        f.render(0, spp)
        runs.append(ctx.timer_stop())
        f.sync()
    ms = min(runs)
    ctr = f.counters()
    out = {"Msamples_per_s": ctr[0] / (ms / 1e3) / 1e6, "ext_rays_per_s": ctr[1] / (ms / 1e3),
           "shadow_rays_per_s": ctr[2] / (ms / 1e3), "ms": ms, "ms_runs": runs, "spp": spp,
           "resolution": [p.width, p.height], "max_depth": p.max_depth,
           "triangles": int(s.view().num_tris), "extension_rays": int(ctr[1]),
           "sort_by_material": "auto" if sort is None else int(sort)}
    if which == "c1" and not size:
        ref = c1_reference_image()
        if ref is not None:
            img = f.accum().astype(np.float64) / spp
            out["rmse_vs_oracle_16k_fp64"] = float(np.sqrt(((img - ref[0]) ** 2).mean()))
            out["oracle_reference_spp"] = ref[1]
    if tuned:
        out["autotuned"] = {"config": tuned["config"], "trials": len(tuned["trials"])}
    f.close()
    if sort is not None:
        ctx.set_engine_sort("auto")
    ds.close()
    return out


SERVE_RESOLUTIONS = [(256, 256), (512, 512), (1024, 1024), (1920, 1080), (2048, 2048)]
SERVE_SIZES = [1e4, 1e5, 1e6, 5e6]   # triangles: the log-uniform range's ends and two points between


def serve_scene_pool():
    """Scenes the serving jobs draw from: each of the three generators (Cornell box with
    tessellated faces, icospheres with the HDR environment, occluded-light room) at about 10k,
    100k, 1M and 5M triangles. Built once on the host; the server uploads them on admission and
    evicts idle ones least recently used first."""
    import lavaframe_gb300 as lf

    pool = []
    for t in SERVE_SIZES:
        k = max(1, int(round((t / 34.0) ** 0.5)))                      # 34 k^2 triangles
        pool.append(("cornell", lf.HostScene().gen_cornell(256, 256, k).build()))
    for inst, level in ((2, 4), (5, 5), (13, 6), (64, 6)):            # 10k, 102k, 1.06M, 5.2M
        pool.append(("icospheres", lf.HostScene().gen_icospheres(inst, level, 3, 1024, 512).build()))
    for t in SERVE_SIZES:
        pool.append(("room", lf.HostScene().gen_room(int(t / 12), 4).build()))   # 12 triangles per box
    return pool


def serve_jobs(pool, n, seed=11, max_spp=256):
    """Job list: generator uniform over the three, size log-uniform in [1e4, 5e6] triangles
    (the pool scene of that generator nearest in log size), resolution, spp U{1..max_spp},
    depth U{4..10}, and an exponential arrival gap of mean 1 (scaled by the rate later)."""
    rng = np.random.default_rng(seed)
    jobs = []
    for _ in range(n):
        gen = ["cornell", "icospheres", "room"][rng.integers(3)]
        target = np.exp(rng.uniform(np.log(1e4), np.log(5e6)))
        cands = [(abs(np.log(max(1, int(sc.view().num_tris))) - np.log(target)), k) for k, (g, sc) in enumerate(pool)
                 if g == gen]
        scene = min(cands)[1]
        w, h = SERVE_RESOLUTIONS[rng.integers(len(SERVE_RESOLUTIONS))]
        jobs.append({"scene": scene, "width": w, "height": h, "spp": int(rng.integers(1, max_spp + 1)),
                     "depth": int(rng.integers(4, 11)), "gap": float(rng.exponential(1.0))})
    return jobs


def run_serving(ctx, n_jobs, max_spp=256, budget_gb=0.0, rate=20.0, low_load=0.5):
    """Serving loop workload. The same jobs run three ways: all submitted at once (batch-only
    throughput), arriving as a Poisson stream at `rate` jobs/s, and arriving at the rate that
    offers `low_load` of the batch throughput (so that latency is not queueing). A memory
    budget below the scenes' total (budget_gb above the engine pool) makes the server evict
    idle scenes under load."""
    import lavaframe_gb300 as lf
    from lavaframe_gb300 import autotune

    autotune.apply_default(ctx)   # creates the engine if needed, default setting
    pool = serve_scene_pool()
    jobs = serve_jobs(pool, n_jobs, max_spp=max_spp)
    samples = int(sum(j["width"] * j["height"] * j["spp"] for j in jobs))
    pool_bytes = ctx.engine_info()["device_bytes"]
    budget = int(pool_bytes + budget_gb * (1 << 30)) if budget_gb > 0 else 0

    def params(j):
        p = pool[j["scene"]][1].render_params()
        p.width, p.height, p.max_depth = j["width"], j["height"], j["depth"]
        return p

    def one_run(arrival_rate, limit_s=600.0):
        srv = lf.Server(ctx, memory_budget=budget)
        sids = [srv.add_scene(sc) for _, sc in pool]
        pending, infos = [], {}

        def reap():
            # a client reads and releases each job as it finishes, so finished jobs do not
            # hold budget that later jobs need
            for jid in list(pending):
                if srv.wait(jid, 0):
                    infos[jid] = srv.info(jid)
                    srv.release(jid)
                    pending.remove(jid)

        try:
            t0 = time.perf_counter()
            due = 0.0
            for j in jobs:
                if arrival_rate:
                    due += j["gap"] / arrival_rate
                    while due - (time.perf_counter() - t0) > 0:
                        reap()
                        time.sleep(min(0.002, max(0.0, due - (time.perf_counter() - t0))))
                pending.append(srv.submit(sids[j["scene"]], params(j), j["spp"]))
            while pending:
                reap()
                if time.perf_counter() - t0 > limit_s:
                    raise RuntimeError(f"serving run exceeded {limit_s} s with {len(pending)} jobs left")
                time.sleep(0.001)
            wall = time.perf_counter() - t0
            st = srv.stats()
        finally:
            srv.close()
        infos = list(infos.values())
        lat = np.array([i["finish_ms"] - i["submit_ms"] for i in infos])
        span = (max(i["finish_ms"] for i in infos) - min(i["submit_ms"] for i in infos)) / 1e3
        return {"arrival_rate_per_s": arrival_rate or None, "wall_s": wall, "makespan_s": span,
                "Msamples_per_s": samples / span / 1e6, "ext_rays_per_s": st["ext_rays"] / span,
                "p50_ms": float(np.percentile(lat, 50)), "p99_ms": float(np.percentile(lat, 99)),
                "max_ms": float(lat.max()), "scene_uploads": st["scene_uploads"],
                "scene_evictions": st["scene_evictions"]}

    batch = one_run(0.0)
    serve = one_run(rate)
    low_rate = low_load * n_jobs / batch["makespan_s"]
    low = one_run(low_rate)
    return {"jobs": n_jobs, "samples": samples, "max_spp": max_spp, "memory_budget_bytes": budget or None,
            "engine_pool_bytes": pool_bytes, "batch_only": batch, "serving": serve,
            "serving_over_batch": serve["Msamples_per_s"] / batch["Msamples_per_s"],
            "serving_low_load": dict(low, offered_load=low_load),
            "scenes": [{"generator": g, "triangles": int(sc.view().num_tris), "device_bytes": None}
                       for g, sc in pool]}


def run_guiding(ctx, width, height, ref_spp, plain_spp=1024, batch=16, every=2, max_factor=3.0, alpha=0.5, lr=1e-2,
                tensor=(0, 1), seeds=(1, 2)):
    """Time-to-error of learned path guiding on the occluded-light room (16.7k boxes, ~200k
    triangles, depth 10): the plain tracer's error after plain_spp samples, against an FP64
    reference of ref_spp samples, and the wall time the guided tracer (trained online, Adam
    every `every`-th batch of `batch` samples) needs to reach the same error - for each MLP
    path (0 warp-level mma.sync, 1 tcgen05) and guide seed; the reference and the plain render
    are made once."""
    import lavaframe_gb300 as lf

    s = lf.HostScene().gen_room(16700, 4).build()
    a = s.arrays()
    top = int(a["top_level_index"])
    lo, hi = a["nodes"][top][0:3], a["nodes"][top][3:6]
    p = s.render_params()
    p.width, p.height = width, height
    ds = ctx.upload(s)

    def frame():
        return lf.Frame(ctx, ds, p, lf.FRAME_FP64_ACCUM)

    f = frame()
    f.set_batch(16)
    t0 = time.perf_counter()
    f.render(0, ref_spp)
    f.sync()
    t_ref = time.perf_counter() - t0
    ref = f.accum64() / ref_spp
    f.close()

    def rmse(img):
        return float(np.sqrt(((img - ref) ** 2).mean()))

    f = frame()
    f.render(1 << 20, 8)
    f.sync()
    f.reset()
    t0 = time.perf_counter()
    f.render(1 << 20, plain_spp)
    f.sync()
    t_plain = time.perf_counter() - t0
    target = rmse(f.accum64() / plain_spp)
    f.close()

    runs = []
    for tc in tensor:
        for seed in seeds:
            g = lf.Guide(ctx, lo, hi, seed=seed)
            g.set_tensor_path(bool(tc))
            f = frame()
            f.set_batch(batch)
            f.set_guide(g, alpha, every, lr)
            spent, done, reached, last = 0.0, 0, False, None
            while spent < max_factor * t_plain:
                t0 = time.perf_counter()
                f.render((1 << 20) + done, batch)
                f.sync()
                spent += time.perf_counter() - t0
                done += batch
                if done % 16 == 0:
                    last = rmse(f.accum64() / done)
                    if last <= target:
                        reached = True
                        break
            st = f.guide_stats()
            f.close()
            g.close()
            runs.append({"mlp": "tcgen05" if tc else "mma.sync", "seed": seed, "reached": reached, "spp": done,
                         "seconds": spent, "rmse": last, "time_ratio": spent / t_plain if reached else None,
                         "ms_per_sample": spent / done * 1e3, "adam_steps": st["adam_steps"]})
    ds.close()
    ratios = [r["time_ratio"] for r in runs if r["time_ratio"] is not None]
    return {"resolution": [width, height], "triangles": int(s.view().num_tris), "max_depth": int(p.max_depth),
            "reference_spp": ref_spp, "reference_s": t_ref, "plain_spp": plain_spp, "plain_s": t_plain,
            "plain_ms_per_sample": t_plain / plain_spp * 1e3, "plain_rmse": target, "runs": runs,
            "time_ratio_best": min(ratios) if ratios else None,
            "time_ratio_median": float(np.median(ratios)) if ratios else None,
            "runs_reached": f"{len(ratios)} of {len(runs)}",
            "batch": batch, "train_every": every, "alpha": alpha, "lr": lr}


def guided_batches(ctx, width, height, batch=16, tensor=1):
    """Per-sample cost on the occluded-light room of the engine, of the per-batch pipeline and
    of guided batches (Adam after every second batch), each after its warm-up. One per-batch
    batch and two guided batches (one that trains, one that does not) run between
    cuProfilerStart and cuProfilerStop, so that `ncu --profile-from-start off` lists exactly
    their launches."""
    import ctypes

    import lavaframe_gb300 as lf

    s = lf.HostScene().gen_room(16700, 4).build()
    a = s.arrays()
    top = int(a["top_level_index"])
    lo, hi = a["nodes"][top][0:3], a["nodes"][top][3:6]
    p = s.render_params()
    p.width, p.height = width, height
    ds = ctx.upload(s)
    try:
        cu = ctypes.CDLL("libcuda.so.1")
    except OSError:
        cu = None

    def timed(f, first, n):
        f.sync()
        t = time.perf_counter()
        f.render(first, n)
        f.sync()
        return time.perf_counter() - t

    out = {"resolution": [width, height], "batch": batch}
    f = lf.Frame(ctx, ds, p, lf.FRAME_FP64_ACCUM)
    f.render(0, batch)
    out["engine_ms_per_spp"] = timed(f, batch, 4 * batch) / (4 * batch) * 1e3
    f.close()
    f = lf.Frame(ctx, ds, p, lf.FRAME_FP64_ACCUM | lf.FRAME_PER_BATCH)
    f.set_batch(batch)
    f.render(0, batch)
    out["per_batch_ms_per_spp"] = timed(f, batch, 4 * batch) / (4 * batch) * 1e3
    if cu:
        f.sync()
        cu.cuProfilerStart()
        f.render(5 * batch, batch)
        f.sync()
        cu.cuProfilerStop()
    f.close()
    g = lf.Guide(ctx, lo, hi, seed=1)
    g.set_tensor_path(bool(tensor))
    f = lf.Frame(ctx, ds, p, lf.FRAME_FP64_ACCUM)
    f.set_batch(batch)
    f.set_guide(g, 0.5, 2, 1e-2)
    for k in range(8):
        f.render(k * batch, batch)
    per = [timed(f, (8 + k) * batch, batch) / batch * 1e3 for k in range(8)]
    out["guided_ms_per_spp_batches"] = per
    out["guided_ms_per_spp"] = float(np.mean(per))
    if cu:
        f.sync()
        cu.cuProfilerStart()
        f.render(16 * batch, batch)
        f.render(17 * batch, batch)
        f.sync()
        cu.cuProfilerStop()
    f.close()
    g.close()
    ds.close()
    return out


def main():
    args = parse()
    world, rank, local = dist_setup()
    if args.impl == "reference":
        run_reference(args, world, rank)
        barrier(world)
        return

    import lavaframe_gb300 as lf
    from lavaframe_gb300 import build as b

    b.build_core()
    b.build_oracle()
    ctx = lf.Context(local)
    if args.engine_slots or args.shade_cap:
        ctx.configure_engine(slots=args.engine_slots, shade_threads_per_sm=args.shade_cap or 512)
    if args.engine_drain >= 0:
        ctx.set_engine_drain(args.engine_drain)
    if args.workload == "c4":
        cw, ch = (int(x) for x in args.c4_size.split("x"))
        paths = (0, 1) if args.c4_tensor < 0 else (args.c4_tensor,)
        r = run_guiding(ctx, cw, ch, args.c4_ref_spp, batch=args.c4_batch, every=args.c4_every, alpha=args.c4_alpha,
                        lr=args.c4_lr, tensor=paths)
        if rank == 0:
            print(json.dumps({"metric": "c4 guided / plain time to the plain 1024-spp error",
                              "value": r["time_ratio_median"],
                              "unit": "ratio", "higher_is_better": False, "detail": r}), flush=True)
        ctx.close()
        return
    if args.workload == "c4batches":
        cw, ch = (int(x) for x in args.c4_size.split("x"))
        r = guided_batches(ctx, cw, ch, tensor=max(args.c4_tensor, 0) if args.c4_tensor >= 0 else 1)
        if rank == 0:
            print(json.dumps({"metric": "c4 per-sample cost of plain and guided batches", "value": r["guided_ms_per_spp"],
                              "unit": "ms/spp", "higher_is_better": False, "detail": r}), flush=True)
        ctx.close()
        return
    if args.workload == "c5":
        r = run_serving(ctx, args.jobs or 48, budget_gb=3.0)
        if rank == 0:
            print(json.dumps({"metric": "c5 serving Msamples/s", "value": r["serving"]["Msamples_per_s"],
                              "unit": "Msamples/s", "detail": r}), flush=True)
        ctx.close()
        return
    if args.workload != "microbench":
        size = tuple(int(x) for x in args.render_size.split("x")) if args.render_size else None
        r = render_extra(ctx, args.workload, spp_batch=args.spp_batch, flags=args.frame_flags,
                         tune=args.autotune, wide=args.traversal == "wide", size=size, sort=None if args.sort_by_material < 0 else args.sort_by_material)
        if rank == 0:
            print(json.dumps({"metric": f"{args.workload} extension rays/s", "value": r["ext_rays_per_s"],
                              "unit": "rays/s", "detail": r}), flush=True)
        ctx.close()
        return
    s, t_gen, t_build = build_soup(args.instances_log2)
    nrays = 1 << args.rays_log2
    rays, root = soup_rays(s, nrays)
    ds = ctx.upload(s)
    ds.set_traversal(args.traversal == "wide")
    L = lf.lib()
    import ctypes as C

    # device-resident inputs
    d_rays, d_hits = C.c_void_p(), C.c_void_p()
    ctx._c(L.lf_device_alloc(ctx.h, rays.nbytes, C.byref(d_rays)))
    ctx._c(L.lf_device_alloc(ctx.h, nrays * 16, C.byref(d_hits)))
    ctx._c(L.lf_copy_to_device(ctx.h, d_rays, rays.ctypes.data_as(C.c_void_p), rays.nbytes))

    for _ in range(args.warmup):
        ctx._c(L.lf_trace_closest_device(ctx.h, ds.h, d_rays, nrays, d_hits, 0))
    ctx.sync()
    barrier(world)
    ctx.kernel_timer(True)        # event pair around each traversal kernel launch
    with ClockSampler(local) as clk:
        ctx.timer_start()
        for _ in range(args.steps):
            ctx._c(L.lf_trace_closest_device(ctx.h, ds.h, d_rays, nrays, d_hits, 0))
        ms = ctx.timer_stop()
        ctx.sync()
    kernel_ms, kernel_launches = ctx.kernel_timer_read()
    ctx.kernel_timer(False)
    barrier(world)
    ms = max_over_ranks(world, ms)
    value = world * nrays * args.steps / (ms / 1e3) / 1e9

    # end to end: page-locked host rays in, hits out, every step
    e2e_steps = 0 if args.no_e2e else args.steps
    h_rays, h_hits = C.c_void_p(), C.c_void_p()
    ctx._c(L.lf_host_alloc(ctx.h, rays.nbytes, C.byref(h_rays)))
    ctx._c(L.lf_host_alloc(ctx.h, nrays * 16, C.byref(h_hits)))
    C.memmove(h_rays, rays.ctypes.data, rays.nbytes)
    fr = C.cast(h_rays, C.POINTER(C.c_float))
    ctx.set_host_chunks(args.host_chunks)
    for _ in range(args.warmup if e2e_steps else 1):
        ctx._c(L.lf_trace_closest(ctx.h, ds.h, fr, nrays, h_hits, 0))
    barrier(world)
    t = time.perf_counter()
    for _ in range(e2e_steps):
        ctx._c(L.lf_trace_closest(ctx.h, ds.h, fr, nrays, h_hits, 0))
    e2e_s = time.perf_counter() - t
    barrier(world)
    e2e_s = max_over_ranks(world, e2e_s)
    e2e = world * nrays * e2e_steps / e2e_s / 1e9 if e2e_steps else None
    hits = np.frombuffer((C.c_char * (nrays * 16)).from_address(h_hits.value), dtype=lf.HIT_DTYPE).copy()

    # traversal counts for the algorithmic bytes (device counters, same visit order as the oracle)
    n_stats = min(nrays, 1 << 20)
    ctx.trace_closest(ds, rays[:n_stats], flags=lf.TRACE_STATS)
    dstats = ctx.trace_stats()
    extra = {}
    if rank == 0:
        import oracle

        cpu_v, cores, sample, cpu_dt, ostats = cpu_baseline(s.view(), rays, 0.0 if args.no_cpu else args.cpu_seconds)
        # spot check: the sampled rays agree with the oracle bit for bit
        ref_hits, _ = oracle.trace_closest(s.view(), rays[:4096])
        extra["parity_spot_check_4096_rays"] = bool(ref_hits.tobytes() == hits[:4096].tobytes())
        bpr = algorithmic_bytes_per_ray(ostats, sample)
        hbm_peak, peak_kind = measured_peaks()
        # the traversal kernel alone: CUDA events around each of its launches in the timed loop
        kernel_s = kernel_ms / 1e3 / max(1, kernel_launches)
        kernel_rays_per_s = nrays / kernel_s
        # issue roofline: 4 warp schedulers per SM, one instruction each per clock, at the median
        # SM clock sampled during the timed region; instructions per ray from the ncu summary
        attrs = ctx.device_attrs()
        clocks = clk.summary()
        sm_mhz = clocks.get("sm_mhz") or attrs["max_sm_mhz"]
        prof = traversal_profile()
        issue_peak = attrs["sm_count"] * 4 * sm_mhz * 1e6 / 1e9
        inst = prof.get("warp_inst_per_ray")
        achieved = inst * kernel_rays_per_s / 1e9 if inst else None
        traffic = prof["dram_bytes_per_ray"] * nrays if "dram_bytes_per_ray" in prof else None
        dram_gbs = traffic / kernel_s / 1e9 if traffic else None
        roofline = {
            "bound": "issue", "achieved": achieved, "peak": issue_peak, "unit": "Gwarp-instructions/s",
            "frac": achieved / issue_peak if achieved else None, "traffic": traffic,
            "peak_kind": f"{attrs['sm_count']} SMs x 4 schedulers x {sm_mhz:.0f} MHz (median SM clock sampled "
                         f"during the timed region)",
            "kernel": "trace_fetch_wide_kernel<false>", "kernel_ms_per_launch": kernel_s * 1e3,
            "kernel_launches": kernel_launches, "kernel_rays_per_s": kernel_rays_per_s,
            "warp_inst_per_ray": inst, "lanes_per_inst": prof.get("lanes_per_inst"),
            "simt_efficiency": prof["lanes_per_inst"] / 32.0 if "lanes_per_inst" in prof else None,
            "counters_from": prof.get("warp_inst_per_ray_from"),
            "dram_bytes_per_ray": prof.get("dram_bytes_per_ray"), "dram_GBps": dram_gbs,
            "dram_frac_of_hbm": dram_gbs / hbm_peak if dram_gbs else None,
            "l2_bytes_per_ray": prof.get("l2_bytes_per_ray"),
            "hbm_peak_GBps": hbm_peak, "hbm_peak_kind": peak_kind,
            "reference_model_bytes_per_ray": bpr,
            "note": "instruction issue is the bound (DRAM traffic is a few percent of HBM); the reference "
                    "data-model bytes (every binary node box, triangle and transform the reference shader would "
                    "fetch) are informational"}
        if not args.no_extras:
            from lavaframe_gb300 import autotune

            renders = (("c1", "c1", {}), ("c3_1m", "c3", {}), ("c3_1m_unsorted", "c3", {"sort": 0}),
                       ("c3_1m_per_batch", "c3", {"flags": 8}), ("c3_5m", "c3full", {}),
                       ("c3_1m_autotuned", "c3", {"tune": True}))
            for w, which, kw in renders:
                try:
                    extra[w] = render_extra(ctx, which, **kw)
                except Exception as e:  # reported, not fatal for the headline
                    extra[w] = {"error": str(e)}
                autotune.apply_default(ctx)   # the other workloads run on the default engine
            for w, fn in (("c4_guiding_1280x720", lambda: run_guiding(ctx, 1280, 720, args.c4_ref_spp)),
                          ("c5_serving_48_jobs", lambda: run_serving(ctx, 48, budget_gb=3.0))):
                try:
                    extra[w] = fn()
                except Exception as e:  # reported, not fatal for the headline
                    extra[w] = {"error": str(e)}
        extra.update({"scene_build_s": t_build, "scene_generate_s": t_gen, "hit_fraction": float((hits["prim"] >= 0).mean()),
                      "device_counters_per_ray": [x / n_stats for x in dstats],
                      "oracle_counters_per_ray": [float(x) / sample for x in ostats],
                      "algorithmic_bytes_per_ray": bpr, "scene_device_bytes": int(ds.device_bytes())})
        line = {
            "metric": "closest-hit Grays/s (intersection microbench)", "value": value, "unit": "Grays/s",
            "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": f"intersection microbench: {1 << args.instances_log2} instances x 10 triangles "
                                   f"({(1 << args.instances_log2) * 10} tris), 2^{args.rays_log2} rays, tmax 1e6",
                       "rays": nrays, "triangles": (1 << args.instances_log2) * 10,
                       "parallelism": "replicas" if world > 1 else "single GPU",
                       "l2": "inputs larger than L2 (rays 512 MiB + scene > 129 MB), no flush"},
            "e2e": {"value": e2e, "unit": "Grays/s", "h2d_bytes_per_step": int(rays.nbytes),
                    "d2h_bytes_per_step": int(nrays * 16)},
            "roofline": roofline,
            "cpu_baseline": {"value": cpu_v, "unit": "Grays/s", "cores": cores, "kind": "port",
                             "sample": f"{sample} of the 2^{args.rays_log2} rays, {cpu_dt:.1f} s"},
            "clocks": clocks,
            # per binned query: ray_keys, the three bin-scan kernels, ray_scatter, traversal
            "gpu_launches": args.steps * 6,
            "extra": extra,
        }
        print(json.dumps(line), flush=True)
    barrier(world)
    L.lf_host_free(ctx.h, h_rays)
    L.lf_host_free(ctx.h, h_hits)
    L.lf_device_free(ctx.h, d_rays)
    L.lf_device_free(ctx.h, d_hits)
    ds.close()
    ctx.close()


if __name__ == "__main__":
    main()
