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
  collide_thread_min  particles in the collide pass from which it runs one
                    thread per particle instead of three lanes each
  grid_slot_max     collision particles up to which the grid is built by
                    slot inserts (above: a counting sort each sub-step)
The tuning only moves work between executors and launch shapes; results are
bit-identical whatever it picks.  Results are cached in memory by a scene
signature.
"""
from __future__ import annotations

from typing import Callable, Optional

SPACE = {
    "width_per_thread": [0.25, 0.5, 1.0],
    "t_max": [128, 256, 512],
    "max_groups": [1, 2],
    "serial_width": [1.5, 2.0, 4.0],
    "resident": [0, 1],
    "stage_frac": [0.4, 0.67, 1.01],
    "bucket_factor": [1.0, 2.0, 4.0],
    "collide_thread_min": [0, 131072, 1 << 30],
    "grid_slot_max": [0, 262144, 1 << 30],
}
# The planner's defaults for the tunables above (PlanTuning in
# csrc/engine.hpp); a candidate is always applied on top of these, so one
# runner can be re-tuned in place.
DEFAULTS = {
    "width_per_thread": 0.5,
    "t_max": 512,
    "max_groups": 15,
    "serial_width": 2.0,
    "resident": 1,
    "stage_frac": 1.01,
    "bucket_factor": 2.0,
    "collide_thread_min": 131072,
    "grid_slot_max": 262144,
}
# tunables that matter for batches of chain-like worlds (rings), where the
# serial executors carry the step
RING_SPACE = {
    "stage_frac": [0.4, 0.55, 0.67, 0.85, 1.01],
    "serial_width": [1.5, 2.0, 4.0],
}
_CACHE: dict = {}


def signature(scenes) -> tuple:
    sc = scenes if isinstance(scenes, (list, tuple)) else [scenes]
    return (len(sc), sum(s.n_particles for s in sc), sum(len(s.la) for s in sc),
            sc[0].sub_steps, sc[0].link_iters, sc[0].collide, sc[0].mode)


def event_timer(runner, dt: float, steps: int, warmup: int) -> float:
    """ms per update: `warmup` updates, then `steps` updates between CUDA
    events on the current stream (the runner synchronises first)."""
    import torch
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
    return e0.elapsed_time(e1) / steps


def tune_runner(runner, time_ms: Callable[[object], float], space: Optional[dict] = None,
                log: Optional[list] = None, keep: float = 0.98) -> dict:
    """Coordinate descent on one runner (a Solver or a Batch), re-tuned in
    place: every candidate is the best tuning so far with one tunable
    changed, on top of DEFAULTS.  time_ms(runner) times the current tuning
    (warm-up included).  Returns the best tuning with its time under
    "_ms_per_step" and leaves the runner tuned to it."""
    space = space or SPACE

    def apply(cfg: dict) -> None:
        runner.set_tuning(**{k: cfg.get(k, DEFAULTS[k]) for k in space})

    best: dict = {}
    apply(best)
    best_ms = time_ms(runner)
    if log is not None:
        log.append(({}, best_ms))
    for name, values in space.items():
        for v in values:
            if v == best.get(name, DEFAULTS[name]):
                continue
            cfg = dict(best, **{name: v})
            apply(cfg)
            ms = time_ms(runner)
            if log is not None:
                log.append((cfg, ms))
            if ms < best_ms * keep:
                best, best_ms = cfg, ms
    apply(best)
    out = dict(best)
    out["_ms_per_step"] = best_ms
    return out


def autotune(scenes, steps: int = 5, warmup: int = 3, space: Optional[dict] = None,
             log: Optional[list] = None) -> dict:
    """Best tunables for a scene (Solver) or a list of scenes (Batch)."""
    key = signature(scenes)
    if key in _CACHE:
        return dict(_CACHE[key])
    from .api import Batch
    if isinstance(scenes, (list, tuple)):
        runner, dt = Batch([s.to_solver() for s in scenes]), scenes[0].dt
    else:
        runner, dt = scenes.to_solver(), scenes.dt
    best = tune_runner(runner, lambda r: event_timer(r, dt, steps, warmup), space, log)
    runner.close()
    _CACHE[key] = {k: v for k, v in best.items() if not k.startswith("_")}
    return best
