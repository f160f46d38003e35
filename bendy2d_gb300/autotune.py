"""Autotuner for the executor tunables (b2d_set_tuning / b2d_batch_set_tuning).

Coordinate descent from the defaults: for one tunable at a time, each
candidate value is timed on the real scene (CUDA events around `steps`
updates after warm-up) and the fastest kept.  Tunables:

  width_per_thread  group size T = pow2 >= (mean level width / this)
  t_max             largest group size
  max_groups        groups per CTA for T > 32 (1 spreads bodies over SMs)
  serial_width      schedule width below which a body runs serially
  resident          hold a body's whole schedule in shared memory when it fits
  stage_frac        serial bodies with chains >= this x the longest run alone,
                    links staged in shared memory
  bucket_factor     collision-grid buckets per world: pow2 >= this x particles
Results are cached in memory by a scene signature.
"""
from __future__ import annotations

import time
from typing import Callable, Optional

SPACE = {
    "width_per_thread": [0.25, 0.5, 1.0],
    "t_max": [128, 256, 512],
    "max_groups": [1, 2],
    "serial_width": [1.5, 2.0, 4.0],
    "resident": [0, 1],
    "stage_frac": [0.4, 0.67, 1.01],
    "bucket_factor": [1.0, 2.0, 4.0],
}
_CACHE: dict = {}


def signature(scenes) -> tuple:
    sc = scenes if isinstance(scenes, (list, tuple)) else [scenes]
    return (len(sc), sum(s.n_particles for s in sc), sum(len(s.la) for s in sc),
            sc[0].sub_steps, sc[0].link_iters, sc[0].collide, sc[0].mode)


def _time_config(make: Callable, cfg: dict, steps: int, warmup: int) -> float:
    import torch
    runner, dt = make()
    runner.set_tuning(**cfg)
    for _ in range(warmup):
        runner.update(dt)
    runner.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record()
    for _ in range(steps):
        runner.update(dt)
    runner.synchronize()
    e1.record()
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / steps
    runner.close()
    return ms


def autotune(scenes, steps: int = 5, warmup: int = 3, space: Optional[dict] = None,
             log: Optional[list] = None) -> dict:
    """Best tunables for a scene (Solver) or a list of scenes (Batch)."""
    key = signature(scenes)
    if key in _CACHE:
        return dict(_CACHE[key])
    from .api import Batch

    def make():
        if isinstance(scenes, (list, tuple)):
            b = Batch([s.to_solver() for s in scenes])
            return b, scenes[0].dt
        return scenes.to_solver(), scenes.dt

    space = space or SPACE
    best = {}
    best_ms = _time_config(make, best, steps, warmup)
    if log is not None:
        log.append(({}, best_ms))
    for name, values in space.items():
        for v in values:
            cfg = dict(best, **{name: v})
            ms = _time_config(make, cfg, steps, warmup)
            if log is not None:
                log.append((cfg, ms))
            if ms < best_ms * 0.98:
                best, best_ms = cfg, ms
    _CACHE[key] = dict(best)
    best["_ms_per_step"] = best_ms
    return best
