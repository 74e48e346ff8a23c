"""Autotuner of the path engine (no reference counterpart).

Chooses the engine's pool size (paths in flight), the block sizes of its extend and shadow
kernels, the register cap of its shade kernel, whether shade takes the surface hits sorted
by material class, and the number of paths in flight at which a run switches to its one-kernel
drain, by timing short renders of the workload itself on the GPU, one knob at a
time (coordinate descent from the current setting). The
result is applied to the context and can be cached in a JSON file keyed by the workload
signature (resolution, samples, depth, triangles).
"""
from __future__ import annotations

import json
from pathlib import Path

CANDIDATES = {
    "slots": [1 << 21, 1 << 22, 1 << 23, 1 << 24],
    "shade_threads_per_sm": [0, 512, 768, 1024],
    "block_extend": [64, 128, 256],
    "block_shadow": [64, 128, 256],
    "sort_by_material": [0, 1],   # the default 2 sorts when the scene mixes material classes
    "drain_paths": [1 << 21, 1 << 22, 1 << 23],
}
DEFAULT = {"slots": 1 << 24, "shade_threads_per_sm": 512, "block_extend": 128, "block_shadow": 128,
           "sort_by_material": 2, "drain_paths": 1 << 22}
MARGIN = 0.02   # a setting replaces the current one only when it is this much faster (timing noise)


def _signature(params, spp, triangles):
    return f"{params.width}x{params.height}:spp{spp}:depth{params.max_depth}:tris{triangles}"


def _apply(ctx, cfg):
    ctx.configure_engine(slots=cfg["slots"], block_extend=cfg["block_extend"], block_shade=128,
                         block_shadow=cfg["block_shadow"], shade_threads_per_sm=cfg["shade_threads_per_sm"])
    ctx.set_engine_sort(cfg.get("sort_by_material", 2))
    ctx.set_engine_drain(cfg.get("drain_paths", 1 << 22))


def apply_default(ctx):
    """Puts the engine of `ctx` back on the default setting."""
    _apply(ctx, DEFAULT)


def _time_render(ctx, device_scene, params, spp, repeats):
    """Best device time (CUDA events on the context's stream) of `repeats` renders of `spp`
    samples, after a one-sample warm-up render."""
    import lavaframe_gb300 as lf

    f = lf.Frame(ctx, device_scene, params)
    try:
        f.render(0, 1)
        f.sync()
        best = float("inf")
        for r in range(repeats):
            f.reset()
            ctx.timer_start()
            f.render(1 + r * spp, spp)
            ms = ctx.timer_stop()
            f.sync()
            best = min(best, ms / 1e3)
    finally:
        f.close()
    return best


def tune(ctx, device_scene, params, spp=4, repeats=3, triangles=0, cache: str | Path | None = None):
    """Tunes the engine of `ctx` for rendering `spp` samples of `params` on `device_scene` and
    applies the best setting. Time it with the sample count the workload renders: the share of
    the drain at the end of a render depends on it. Returns {"config", "seconds", "trials",
    "cached"}."""
    key = _signature(params, spp, triangles)
    store = {}
    if cache is not None and Path(cache).exists():
        store = json.loads(Path(cache).read_text())
        if key in store:
            _apply(ctx, store[key]["config"])
            return dict(store[key], cached=True)
    cfg = dict(DEFAULT)
    _apply(ctx, cfg)
    best = _time_render(ctx, device_scene, params, spp, repeats)
    trials = [{"config": dict(cfg), "seconds": best}]
    for knob, values in CANDIDATES.items():
        for v in values:
            if v == cfg[knob]:
                continue
            trial = dict(cfg, **{knob: v})
            _apply(ctx, trial)
            t = _time_render(ctx, device_scene, params, spp, repeats)
            trials.append({"config": trial, "seconds": t})
            if t < best * (1.0 - MARGIN):
                best, cfg = t, trial
    _apply(ctx, cfg)
    result = {"config": cfg, "seconds": best, "trials": trials}
    if cache is not None:
        store[key] = {"config": cfg, "seconds": best}
        Path(cache).write_text(json.dumps(store, indent=1))
    return dict(result, cached=False)
