"""Benchmark: particle-substeps/s of Solver::update on GB300.

Workload (N=1): the single large world of 64 cloth grids of 32x32
(65,536 particles, 249,984 links) in a 2000^2 box with initial velocities
N(0, 0.5), particle-particle / particle-circle / particle-polygon collisions
on (radius 0.5, cell 1.0), 16 circles, 8 convex polygons, 8 sub-steps, 4 link
iterations, reference-order link mode.  A step is one Solver::update(1/60).

  value    device time (CUDA events on the solver's stream), inputs resident,
           L2 flushed (256 MiB write) between timed steps
  e2e      the same step through the C ABI with the state uploaded from and
           downloaded to pinned host memory inside the timed region
  roofline dominant kernel: algorithmic bytes per launch / CUDA-event time
  cpu_baseline  the CPU oracle (port of the reference) on a bounded sample

--impl reference times the CPU port of the reference on the same workload.
Under torchrun (N>1) every rank runs its own replica (worlds are
independent; there is no collective on the data path): weak scaling.
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

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "particle-substeps/s"
WORKLOAD = "64 cloth grids 32x32 (65,536 particles, 249,984 links), collisions on, 8 sub-steps, 4 link iterations"


def _peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.idx = gpu_index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.idx}", f"--query-gpu={self.FIELDS}",
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
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx.append(float(f[2]))
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx),
                "reasons": sorted(reasons), "samples": len(sm)}


def build_scene(seed: int = 0):
    from bendy2d_gb300 import scenes
    return scenes.config2(seed=seed)


def config_dict(sc, world: int) -> dict:
    """The workload description both arms print (identical by design)."""
    return {"workload": WORKLOAD, "particles": sc.n_particles, "links": int(len(sc.la)),
            "sub_steps": sc.sub_steps, "link_iters": sc.link_iters,
            "mode": "reference-order", "collisions": "pp+pc+ppoly",
            "l2": "flushed (256 MiB write) between timed steps",
            "parallelism": f"replicas x{world}"}


def algorithmic_bytes(kernel: str, sc) -> float:
    """Algorithmic bytes of one launch of a kernel of the profile
    (kernel_byte_models); a whole-step executor launch (worlds without
    collisions) covers every sub-step: links and 32 B of bounds+integrate per
    particle each."""
    m = kernel_byte_models(sc)
    if kernel.startswith("exec_groups_full") or kernel == "exec_serial_full":
        return sc.sub_steps * (m["links"][0] + 32.0 * sc.n_particles)
    if kernel.startswith("exec_"):
        return m["links"][0]
    if kernel.startswith("rigid"):
        return m["rigid"][0]
    return m[kernel][0] if kernel in m else 0.0


def step_bytes_per_unit(sc) -> float:
    """Algorithmic HBM bytes of a whole update per particle-substep:
    bounds+integrate 32 B, plus per link and iteration 12 B (endpoints, rest)
    or 16 B (with a stiffness other than 1) and 32 B (read+write of both
    positions)."""
    n, l = sc.n_particles, len(sc.la)
    s = 16.0 if np.any(np.asarray(sc.stiff) != 1.0) else 12.0
    return 32.0 + sc.link_iters * (l / max(n, 1)) * (s + 32.0)


def step_roofline(value: float, bytes_per_unit: float) -> dict:
    """Whole-update roofline: algorithmic bytes x particle-substeps/s
    against the measured HBM copy bandwidth."""
    peak, kind = _peaks()
    gbs = value * bytes_per_unit / 1e9
    return {"bound": "hbm", "bytes_per_unit": bytes_per_unit, "achieved": gbs, "peak": peak,
            "unit": "GB/s", "frac": gbs / peak, "peak_source": kind}


def run_cpu_oracle(sc, budget_s: float, max_steps: int = 1000):
    from oracle import load_scene
    o = load_scene(sc)
    steps = 0
    t0 = time.perf_counter()
    while steps < max_steps:
        o.update(sc.dt)
        steps += 1
        if time.perf_counter() - t0 >= budget_s:
            break
    dt = time.perf_counter() - t0
    return sc.n_particles * sc.sub_steps * steps / dt, steps, dt


def run_batched_comparison(args, torch, flush, stream, world: int = 1, rank: int = 0):
    """Configuration 3: 4096 independent ring worlds (log-uniform 64..4096
    particles) stepped (a) batched: one launch sequence for all worlds, CUDA
    graph, with the default tunables and with the ones the autotuner picks
    on this batch; (b) plain: one world per launch, no graph; (c) the CPU
    port of the reference on a sample of worlds across all host cores.
    Under torchrun the worlds are sharded across ranks (sharding.shard,
    balanced by particle-substeps, no exchange): each rank steps its shard
    and the batched value is all worlds' particle-substeps over the slowest
    rank's step (legs (b) and (c) run at N = 1 only)."""
    import concurrent.futures as cf
    from bendy2d_gb300 import Batch, autotune, scenes
    from bendy2d_gb300.sharding import shard, world_cost
    from oracle import load_scene
    all_worlds = scenes.config3(seed=0, n_worlds=args.batched_worlds)
    units = sum(w.n_particles * w.sub_steps for w in all_worlds)
    worlds = all_worlds
    if world > 1:
        worlds = [all_worlds[i] for i in shard([world_cost(w) for w in all_worlds], world)[rank]]
    dt = worlds[0].dt
    out = {"workload": f"{len(all_worlds)} worlds of 1-8 hub-and-spoke rings, particles "
                       "log-uniform in [64, 4096], 2 circles + floor polygon each, 8 sub-steps, "
                       "1 link iteration (batched_i4: 4)", "worlds": len(all_worlds),
           "particles": int(sum(w.n_particles for w in all_worlds)),
           "ranks": world, "l2": "flushed (256 MiB write) between timed steps"}

    def timed_steps(batch, k):
        ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
              for _ in range(k)]
        torch.cuda.synchronize()
        with torch.cuda.stream(stream):
            for e0, e1 in ev:
                flush.zero_()
                e0.record(stream)
                batch.update(dt)
                e1.record(stream)
        batch.synchronize()
        torch.cuda.synchronize()
        return sum(a.elapsed_time(b) for a, b in ev) / k

    def slowest(ms):
        if world == 1:
            return ms
        t = torch.tensor([ms], device="cuda")
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        return float(t.item())

    b = Batch([w.to_solver() for w in worlds])
    b.set_stream(stream.cuda_stream)
    for _ in range(3):
        b.update(dt)
    ms = slowest(timed_steps(b, args.batched_steps))
    bpu = sum(step_bytes_per_unit(w) * w.n_particles for w in all_worlds) / \
        max(1, sum(w.n_particles for w in all_worlds))
    out["batched"] = {"value": units / (ms / 1e3), "ms_per_step": ms,
                      "launches_per_step": b.launch_count(),
                      "roofline": step_roofline(units / (ms / 1e3), bpu)}
    if world == 1 and not args.no_autotune:
        # the autotuner re-tunes the same batch in place (every candidate is
        # timed like the default, after a re-plan and warm-up)
        def time_ms(r):
            for _ in range(3):
                r.update(dt)
            return timed_steps(r, max(2, args.batched_steps // 2))
        log = []
        best = autotune.tune_runner(b, time_ms, autotune.RING_SPACE, log)
        for _ in range(3):
            b.update(dt)
        ms_t = timed_steps(b, args.batched_steps)
        out["batched_autotuned"] = {
            "value": units / (ms_t / 1e3), "ms_per_step": ms_t,
            "tuning": {k: v for k, v in best.items() if not k.startswith("_")},
            "candidates_timed": len(log), "space": autotune.RING_SPACE}
    b.close()
    if world > 1:
        return out
    # the same worlds with 4 link iterations (batched only)
    w4 = scenes.config3(seed=0, n_worlds=args.batched_worlds, link_iters=4)
    b4 = Batch([w.to_solver() for w in w4])
    b4.set_stream(stream.cuda_stream)
    for _ in range(3):
        b4.update(dt)
    ms4 = timed_steps(b4, args.batched_steps)
    bpu4 = sum(step_bytes_per_unit(w) * w.n_particles for w in w4) / \
        max(1, sum(w.n_particles for w in w4))
    out["batched_i4"] = {"value": units / (ms4 / 1e3), "ms_per_step": ms4,
                         "roofline": step_roofline(units / (ms4 / 1e3), bpu4)}
    b4.close()
    p = Batch([w.to_solver() for w in worlds])
    p.set_plain(True)
    p.set_stream(stream.cuda_stream)
    p.update(dt)
    ms = timed_steps(p, max(1, min(3, args.batched_steps)))
    out["plain"] = {"value": units / (ms / 1e3), "ms_per_step": ms,
                    "launches_per_step": p.launch_count()}
    p.close()
    out["batched_over_plain"] = out["batched"]["value"] / out["plain"]["value"]
    # CPU port of the reference, worlds spread over all host cores
    cores = os.cpu_count() or 1
    sample = worlds[:: max(1, len(worlds) // args.cpu_worlds)][: args.cpu_worlds]
    orcs = [load_scene(w) for w in sample]
    t0 = time.perf_counter()
    with cf.ThreadPoolExecutor(max_workers=cores) as ex:
        list(ex.map(lambda o: o.update(dt), orcs))
    el = time.perf_counter() - t0
    su = sum(w.n_particles * w.sub_steps for w in sample)
    out["cpu"] = {"value": su / el, "cores": cores, "kind": "port",
                  "sample": f"{len(sample)} of the worlds, one update each, worlds across "
                            f"{cores} threads"}
    return out


def link_residual(solver, sc) -> dict:
    """|len - rest| / rest over the particle links (float64 on the host):
    max, 99th percentile and median"""
    p, _ = solver.read_state()
    a, b = sc.la.astype(np.int64), sc.lb.astype(np.int64)
    d = np.linalg.norm(p[a].astype(np.float64) - p[b], axis=1)
    r = np.abs(d - sc.rest) / sc.rest
    return {"max": float(r.max()), "p99": float(np.percentile(r, 99)),
            "median": float(np.median(r))}


def energy(pos, prev, h: float, g) -> float:
    """Total energy per unit mass of the solver particles, in float64:
    sum of 1/2 |(pos - prev) / h|^2 (the Verlet velocity of
    src/particle.rs:20-25 over one sub-step) minus g . pos."""
    p = pos.astype(np.float64)
    v = (p - prev.astype(np.float64)) / h
    return float(0.5 * np.sum(v * v) - np.sum(p @ np.asarray(g, np.float64)))


def residual_of(pos, sc) -> np.ndarray:
    """|len - rest| / rest of every particle link (float64)"""
    a, b = sc.la.astype(np.int64), sc.lb.astype(np.int64)
    d = np.linalg.norm(pos[a].astype(np.float64) - pos[b], axis=1)
    return np.abs(d - sc.rest) / sc.rest


def run_config1_long(args, torch, stream) -> dict:
    """Configuration 1 over its full run (600 updates of the 32x32 cloth,
    reference semantics): the GPU against the CPU port of the reference, bit
    parity at the last step, and the long-run statistics (constraint residual
    and total-energy drift per step) in reference order and in the fast
    coloured order."""
    from bendy2d_gb300 import MODE_FAST, MODE_REFERENCE, scenes
    from oracle import load_scene
    steps = args.config1_steps
    out = {"workload": "32x32 cloth (1,024 particles, 3,906 links), 4 static circles, static "
                       f"floor polygon, 8 sub-steps, 4 link iterations, {steps} updates",
           "steps": steps}
    marks = sorted({1, 10, 100, steps // 2, steps} & set(range(1, steps + 1)))
    for name, mode in (("reference_order", MODE_REFERENCE), ("fast", MODE_FAST)):
        sc = scenes.config1(seed=0, steps=steps)
        sc.mode = mode
        h = sc.dt / sc.sub_steps
        # timed: every update back to back (the working set stays in L2)
        s = sc.to_solver()
        s.set_stream(stream.cuda_stream)
        for _ in range(3):
            s.update(sc.dt)
        s.synchronize()
        s.close()
        s = sc.to_solver()
        s.set_stream(stream.cuda_stream)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        with torch.cuda.stream(stream):
            e0.record(stream)
            for _ in range(steps):
                s.update(sc.dt)
            e1.record(stream)
        s.synchronize()
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1)
        final_timed = s.read_state()
        order = s.link_order() if mode == MODE_FAST else None
        s.close()
        # statistics: the same run again, state read back after every update
        s = sc.to_solver()
        e_start = energy(sc.pos, sc.prev, h, sc.gravity)
        en, rmax, rp99 = [], [], []
        for _ in range(steps):
            s.update(sc.dt)
            p, q = s.read_state()
            en.append(energy(p, q, h, sc.gravity))
            r = residual_of(p, sc)
            rmax.append(float(r.max()))
            rp99.append(float(np.percentile(r, 99)))
        same_runs = bool(np.array_equal(p.view(np.uint32), final_timed[0].view(np.uint32)))
        s.close()
        # the CPU port of the reference over the same run (fast mode: the
        # oracle replays the GPU's colour order)
        o = load_scene(sc, link_order=order)
        t0 = time.perf_counter()
        for _ in range(steps):
            o.update(sc.dt)
        el = time.perf_counter() - t0
        op, oq = o.particles()
        units = sc.n_particles * sc.sub_steps * steps
        en = np.asarray(en)
        scale = max(abs(e_start), 1e-30)
        out[name] = {
            "gpu": {"value": units / (ms / 1e3), "ms_per_step": ms / steps},
            "cpu": {"value": units / el, "ms_per_step": el / steps * 1e3, "cores": 1,
                    "kind": "port"},
            "bit_exact_vs_cpu_at_last_step": bool(
                np.array_equal(p.view(np.uint32), op.view(np.uint32)) and
                np.array_equal(q.view(np.uint32), oq.view(np.uint32))),
            "timed_and_statistics_runs_identical": same_runs,
            "residual": {"at_step": marks, "max": [rmax[k - 1] for k in marks],
                         "p99": [rp99[k - 1] for k in marks]},
            "energy": {"initial": e_start, "at_step": marks,
                       "value": [float(en[k - 1]) for k in marks],
                       "drift_rel_final": float((en[-1] - e_start) / scale),
                       "max_abs_dev_rel": float(np.max(np.abs(en - e_start)) / scale)},
        }
    return out


def run_config5(args, torch, flush, stream):
    """Configuration 5: 1024 cloth grids (1,048,576 particles, 3,999,744 links),
    20 sub-steps, 8 link iterations, particle collisions, 64 circles, 32
    polygons; fast coloured mode against reference order, with residuals."""
    from bendy2d_gb300 import MODE_FAST, MODE_REFERENCE, scenes
    out = {"workload": "1024 cloth grids 32x32 (1,048,576 particles, 3,999,744 links) in "
                       "4000^2, 20 sub-steps, 8 link iterations, particle collisions, 64 static "
                       "circles, 32 static polygons", "steps": args.config5_steps}
    for name, mode in (("fast", MODE_FAST), ("reference_order", MODE_REFERENCE)):
        sc = scenes.config5(seed=0, mode=mode)
        s = sc.to_solver()
        s.set_stream(stream.cuda_stream)
        s.update(sc.dt)
        s.synchronize()
        ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
              for _ in range(args.config5_steps)]
        torch.cuda.synchronize()
        with torch.cuda.stream(stream):
            for e0, e1 in ev:
                flush.zero_()
                e0.record(stream)
                s.update(sc.dt)
                e1.record(stream)
        s.synchronize()
        torch.cuda.synchronize()
        ms = sum(a.elapsed_time(b) for a, b in ev) / len(ev)
        v = sc.n_particles * sc.sub_steps / (ms / 1e3)
        res = {"value": v, "ms_per_step": ms,
               "residual_after": link_residual(s, sc),
               "levels_per_sub_step_per_body": s.plan_stats()["levels"] / 1024,
               "roofline": step_roofline(v, step_bytes_per_unit(sc)),
               "kernel_rooflines": config5_kernel_rooflines(s, sc, torch, flush, stream)}
        s.close()
        # statistics run: residual and energy after every update, and where
        # the worst links are
        s = sc.to_solver()
        h = sc.dt / sc.sub_steps
        e_start = energy(sc.pos, sc.prev, h, sc.gravity)
        rmax, rp99, en = [], [], []
        for _ in range(args.config5_steps):
            s.update(sc.dt)
            p, q = s.read_state()
            r = residual_of(p, sc)
            rmax.append(float(r.max()))
            rp99.append(float(np.percentile(r, 99)))
            en.append(energy(p, q, h, sc.gravity))
        s.close()
        inside, near_c = overlap_at_start(sc)
        a, b = sc.la.astype(np.int64), sc.lb.astype(np.int64)
        torn = r > 0.5
        ends = np.concatenate([a[torn], b[torn]])
        started = inside | near_c
        res["per_step"] = {"residual_max": rmax, "residual_p99": rp99, "energy": en,
                           "energy_initial": e_start,
                           "energy_drift_rel_final": (en[-1] - e_start) / max(abs(e_start), 1e-30)}
        torn_bodies = np.unique(ends // 1024)  # 1,024 particles per cloth body
        res["stretched_links"] = {
            "links_over_half_rest": int(torn.sum()),
            "bodies_with_such_links": int(len(torn_bodies)),
            "of_those_bodies_starting_with_a_particle_in_reach_of_a_polygon_or_circle": int(
                len(np.intersect1d(torn_bodies, np.unique(np.nonzero(started)[0] // 1024)))),
            "particles_starting_inside_or_within_reach_of_a_polygon": int(inside.sum()),
            "particles_starting_within_reach_of_a_circle": int(near_c.sum())}
        out[name] = res
    return out


def grid_buckets(sc) -> int:
    """Collision-grid buckets of one world: a power of two >= 2 x particles, >= 64."""
    n = max(2 * sc.n_particles, 64)
    return 1 << (n - 1).bit_length()


# the engine's default for the tunable grid_slot_max: collision grids of up
# to this many particles are built by slot inserts, larger ones by a sort
GRID_SLOT_MAX = 262144


def kernel_byte_models(sc, slotted=None) -> dict:
    """Algorithmic bytes per launch of every kernel of the sub-step pipeline,
    each array counted once (f32 state, u32 indices).  name -> (bytes, model).
    slotted: the collision grid is built by slot inserts, else by the
    counting sort (count, scan, scatter); None: the engine's default choice
    for this world's size."""
    if slotted is None:
        slotted = sc.n_particles <= GRID_SLOT_MAX
    n, l, I = sc.n_particles, len(sc.la), sc.link_iters
    nb = grid_buckets(sc)
    nv = sum(len(g["points"]) for g in sc.polygons)
    nc = len(sc.circles)
    stiff = np.any(np.asarray(sc.stiff) != 1.0)
    return {
        "links": (I * l * ((16.0 if stiff else 12.0) + 32.0),
                  "I x L x (12 B link record + 2 x (8 B read + 8 B write) of positions): "
                  "logical bytes of the link passes; the executor keeps a body in shared "
                  "memory through its passes, so DRAM sees only the body's load and store"),
        "grid_count": (24.0 * n, "per particle: read pos 8 B, bucket counter atomic 8 B, "
                                 "write (bucket, rank) 8 B"),
        "grid_scan": (16.0 * nb, "per bucket: read count 4 B, clear it 4 B, write range 8 B"),
        "grid_scatter": (40.0 * n, "per particle: read pos 8 B, (bucket, rank) 8 B, range 8 B, "
                                   "write sorted entry 16 B"),
        "grid_insert": (32.0 * n, "per particle: read pos 8 B, bucket cell word atomic 8 B, "
                                  "write its entry 16 B (a slot or an overflow entry)"),
        "collide_integrate": ((48.0 * n + 16.0 * nb,
                               "per particle: pos and prev read, pos and prev written (32 B), "
                               "its entry read (16 B); per bucket its cell word read once (8 B) "
                               "and the other parity's cleared (8 B); neighbour entries re-read "
                               "through L1/L2 are not counted again") if slotted else
                              (56.0 * n + 8.0 * nb,
                               "per particle: pos and prev read, pos and prev written (32 B), "
                               "its sorted entry read (16 B), its (bucket, rank) slot 8 B; per "
                               "bucket its range once (8 B); neighbour entries re-read through "
                               "L1/L2 are not counted again")),
        "rigid": (48.0 * (nc + nv), "per circle and polygon vertex: pos, prev, acc read and "
                                    "written"),
        "copy_back": (16.0 * n, "per particle: read pos from the second buffer, write it back"),
    }


def kernel_rooflines(prof: dict, sc, launches_per_step: dict) -> dict:
    """Per-kernel rooflines of one update from the CUDA-event profile (each
    launch timed alone, serially): achieved = algorithmic bytes per launch
    (kernel_byte_models) / mean launch time, against the measured HBM copy
    bandwidth.  The times of all kernels add up to the serial step time."""
    peak, kind = _peaks()
    models = kernel_byte_models(sc, slotted="grid_scan" not in prof)
    groups = {"links": [k for k in prof if k.startswith("exec_")],
              "rigid": [k for k in prof if k.startswith("rigid")]}
    for k in ("grid_insert", "grid_count", "grid_scan", "grid_scatter", "collide_integrate",
              "copy_back"):
        groups[k] = [k] if k in prof else []
    out = {}
    for g, names in groups.items():
        ms = sum(prof[k] for k in names)
        if ms <= 0.0:
            continue
        nl = launches_per_step.get(g, 1)
        nbytes, model = models[g]
        per_launch_ms = ms / nl
        gbs = nbytes / (per_launch_ms / 1e3) / 1e9
        out[g] = {"kernels": names, "ms_per_step": ms, "launches_per_step": nl,
                  "algorithmic_bytes_per_launch": nbytes, "byte_model": model,
                  "achieved": gbs, "peak": peak, "unit": "GB/s", "frac": gbs / peak,
                  "peak_source": kind}
    out["serial_sum_ms_per_step"] = sum(prof.values())
    return out


# Warp-instructions per link solve of the shared-memory link executor, from
# its ncu captures (instructions executed / link solves of the launch):
# configuration 5, 133.4 M / 32.0 M (profiles/config5_collide_and_links.md);
# configuration 2, 4.34 M / 1.0 M (profiles/exec_groups_links_config2.md).
LINK_WARP_INSTR = {"config5": 133.4e6 / (1024 * 3906 * 8), "config2": 4.3354e6 / (64 * 3906 * 4)}


def link_issue_bound(torch, ms_per_step: float, solves_per_step: float, per_solve: float) -> dict:
    """The link executor against the SMs' instruction-issue rate (one
    warp-instruction per cycle per sub-partition, four per SM, at the
    maximum SM clock): link solves x warp-instructions per solve / time."""
    props = torch.cuda.get_device_properties(0)
    mhz = 2070.0
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        mhz = float(json.loads(p.read_text()).get("sm_max_mhz", mhz))
    peak = props.multi_processor_count * 4 * mhz * 1e6
    achieved = solves_per_step * per_solve / (ms_per_step / 1e3)
    return {"bound": "issue", "warp_instructions_per_link_solve": per_solve,
            "achieved": achieved, "peak": peak, "unit": "warp-instructions/s",
            "frac": achieved / peak}


def config5_kernel_rooflines(s, sc, torch, flush, stream) -> dict:
    """Per-kernel rooflines of one configuration-5 update at this
    throughput-bound size (kernel_rooflines), with the link executor also
    against the instruction-issue rate, its real bound here."""
    with torch.cuda.stream(stream):
        flush.zero_()
    s.synchronize()
    s.set_profiling(True)
    s.update(sc.dt)
    prof = s.profile()
    s.set_profiling(False)
    S = sc.sub_steps
    out = kernel_rooflines(prof, sc, {"links": S, "grid_insert": S, "grid_count": S,
                                      "grid_scan": S, "grid_scatter": S,
                                      "collide_integrate": S, "rigid": S + 1, "copy_back": 1})
    if "links" in out:
        out["links"]["issue"] = link_issue_bound(
            torch, out["links"]["ms_per_step"], S * sc.link_iters * len(sc.la),
            LINK_WARP_INSTR["config5"])
    return out


def overlap_at_start(sc):
    """Solver particles that start inside a polygon (crossing number) or
    within particle radius of a polygon edge, and those within reach of a
    circle: the extension's one-way contacts push these out at the first
    sub-step, by up to a polygon's depth."""
    pos = sc.pos.astype(np.float64)
    near_p = np.zeros(len(pos), bool)
    for g in sc.polygons:
        v = np.asarray(g["points"], np.float64)
        ins = np.zeros(len(pos), bool)
        for e in range(len(v)):
            a, b = v[e], v[(e + 1) % len(v)]
            cross = (a[1] > pos[:, 1]) != (b[1] > pos[:, 1])
            dy = b[1] - a[1]
            t = (pos[:, 1] - a[1]) / (dy if dy != 0.0 else 1.0)
            ins ^= cross & (pos[:, 0] < a[0] + t * (b[0] - a[0]))
            ab = b - a
            u = np.clip(((pos - a) @ ab) / max(float(ab @ ab), 1e-30), 0.0, 1.0)
            near_p |= np.linalg.norm(pos - (a + u[:, None] * ab), axis=1) < sc.radius
        near_p |= ins
    near_c = np.zeros(len(pos), bool)
    for c in sc.circles:
        near_c |= np.linalg.norm(pos - np.asarray(c["pos"], np.float64), axis=1) < \
            float(c["radius"]) + sc.radius
    return near_p, near_c


def run_profile_config(args, torch) -> None:
    """One configuration alone, for profilers: --warmup updates, then
    --steps updates timed with CUDA events (L2 not flushed).  Launch order
    per update is fixed, so a profiler can skip a known number of launches."""
    from bendy2d_gb300 import Batch, MODE_FAST, scenes
    from bendy2d_gb300 import build as b
    b.build()
    torch.cuda.set_device(0)
    k = args.profile_config
    if args.profile_large:
        n = args.profile_large
        rng = np.random.default_rng(0)
        sc = scenes._assemble(f"cloth{n}", [scenes.grid_body(n, n, (10.0, 20.0), 1.0, 0.01, rng)],
                              bounds=(0.0, 0.0, 4.0 * n, 4.0 * n), sub_steps=8, link_iters=4)
        runner, dt, units = sc.to_solver(), sc.dt, sc.n_particles * sc.sub_steps
        k = f"large{n}"
    elif k == 1:
        sc = scenes.config1(seed=0)
        runner, dt, units = sc.to_solver(), sc.dt, sc.n_particles * sc.sub_steps
    elif k == 2:
        sc = build_scene(0)
        runner, dt, units = sc.to_solver(), sc.dt, sc.n_particles * sc.sub_steps
    elif k == 3:
        worlds = scenes.config3(seed=0, n_worlds=args.batched_worlds)
        runner, dt = Batch([w.to_solver() for w in worlds]), worlds[0].dt
        units = sum(w.n_particles * w.sub_steps for w in worlds)
    else:
        sc = scenes.config5(seed=0, mode=MODE_FAST)
        runner, dt, units = sc.to_solver(), sc.dt, sc.n_particles * sc.sub_steps
    if args.tuning:
        runner.set_tuning(**json.loads(args.tuning))
    for _ in range(args.warmup):
        runner.update(dt)
    runner.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record()
    for _ in range(args.steps):
        runner.update(dt)
    runner.synchronize()
    e1.record()
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / max(args.steps, 1)
    print(json.dumps({"profile_config": k, "steps": args.steps, "warmup": args.warmup,
                      "ms_per_step": ms, "value": units / (ms / 1e3), "unit": METRIC,
                      "launches_per_step": runner.launch_count()}))
    runner.close()


def dist_env():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=50)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--cpu-budget", type=float, default=15.0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--batched-worlds", type=int, default=4096)
    ap.add_argument("--batched-steps", type=int, default=10)
    ap.add_argument("--cpu-worlds", type=int, default=512)
    ap.add_argument("--no-batched", action="store_true")
    ap.add_argument("--no-autotune", action="store_true",
                    help="skip the autotuned configuration-3 batch")
    ap.add_argument("--serve-window", type=float, default=10.0,
                    help="arrival window of the stated 2,000 req/s rate (s)")
    ap.add_argument("--serve-drain", type=float, default=150.0,
                    help="longest wait for outstanding requests after a window (s)")
    ap.add_argument("--serve-max-resident", type=int, default=4_000_000,
                    help="residency limit of the server, solver particles (0: none); "
                         "larger ticks amortise each tick's host work (2 M: 3.31, 4 M: "
                         "3.49, 8 M: 3.60 G/s served at 2,000 req/s) and lengthen each "
                         "request's service time")
    ap.add_argument("--serve-low-rate", type=float, default=150.0,
                    help="arrival rate of the unsaturated serving run (req/s)")
    ap.add_argument("--serve-low-window", type=float, default=30.0)
    ap.add_argument("--config5-steps", type=int, default=5)
    ap.add_argument("--config1-steps", type=int, default=600)
    ap.add_argument("--no-config1", action="store_true")
    ap.add_argument("--no-config5", action="store_true")
    ap.add_argument("--no-serve", action="store_true")
    ap.add_argument("--profile-config", type=int, choices=[1, 2, 3, 5], default=0,
                    help="run only --warmup + --steps updates of one configuration (the "
                         "command the ncu summaries profile) and print its step time")
    ap.add_argument("--tuning", default="", metavar="JSON",
                    help="with --profile-config / --profile-large: executor tunables to set "
                         "first, as a JSON object (grid_slot_max 0: the sorted collision grid)")
    ap.add_argument("--profile-large", type=int, default=0, metavar="SIDE",
                    help="like --profile-config, for one SIDE x SIDE cloth without "
                         "collisions (8 sub-steps, 4 link passes): a body for the "
                         "large-body executor when it exceeds one CTA's shared memory")
    args = ap.parse_args()
    world, rank, local = dist_env()

    if args.impl == "reference":
        if rank != 0:
            return
        sc = build_scene()
        warm = max(args.warmup, 3)
        from oracle import load_scene
        o = load_scene(sc)
        for _ in range(warm):
            o.update(sc.dt)
        # bounded sample: at most --steps updates, and at most ~cpu-budget seconds
        t0 = time.perf_counter()
        k = 0
        while k < args.steps:
            o.update(sc.dt)
            k += 1
            if time.perf_counter() - t0 >= args.cpu_budget:
                break
        el = time.perf_counter() - t0
        v = sc.n_particles * sc.sub_steps * k / el
        print(json.dumps({
            "impl": "reference", "metric": METRIC, "value": v, "unit": METRIC,
            "n_gpus": args.gpus, "steps": k, "warmup": warm,
            "ms_per_step": el / k * 1e3, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded scene generator, bendy2d_gb300/scenes.py:config2)",
            "config": config_dict(sc, world),
            "cpu_baseline": {"value": v, "unit": METRIC, "cores": 1, "kind": "port",
                             "sample": f"{k} updates of the full workload (C port of the "
                                       "reference, single thread like Solver::update)"},
            "e2e": {"value": v, "unit": METRIC, "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0},
        }))
        return

    import torch
    if args.profile_config or args.profile_large:
        run_profile_config(args, torch)
        return
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    from bendy2d_gb300 import build as b
    b.build()
    sc = build_scene(seed=rank)
    stream = torch.cuda.Stream()
    s = sc.to_solver()
    s.set_stream(stream.cuda_stream)
    flush = torch.empty(256 * 1024 * 1024, dtype=torch.uint8, device="cuda")
    units = sc.n_particles * sc.sub_steps

    def barrier():
        if world > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()

    # warm-up (also builds the plan and captures the graph)
    for _ in range(max(args.warmup, 3)):
        s.update(sc.dt)
    s.synchronize()

    # ---- device-timed steps, state resident, L2 flushed between steps
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
          for _ in range(args.steps)]
    barrier()
    with ClockSampler(local) as clk:
        with torch.cuda.stream(stream):
            for e0, e1 in ev:
                flush.zero_()
                e0.record(stream)
                s.update(sc.dt)
                e1.record(stream)
        s.synchronize()
        barrier()
    ms = sum(e0.elapsed_time(e1) for e0, e1 in ev)
    ms_t = torch.tensor([ms], device="cuda")
    if world > 1:
        torch.distributed.all_reduce(ms_t, op=torch.distributed.ReduceOp.MAX)
    ms_max = float(ms_t.item())
    value = units * args.steps * world / (ms_max / 1e3)
    launches = s.launch_count() * args.steps

    # ---- end to end through the C ABI with pinned host buffers
    nbytes = s.state_bytes()
    h_in = torch.empty(nbytes, dtype=torch.uint8, pin_memory=True)
    h_out = torch.empty(nbytes, dtype=torch.uint8, pin_memory=True)
    s.state_download_async(h_in.data_ptr())
    s.synchronize()
    e2e_ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
              for _ in range(args.steps)]
    barrier()
    with torch.cuda.stream(stream):
        for e0, e1 in e2e_ev:
            flush.zero_()
            e0.record(stream)
            s.state_upload_async(h_in.data_ptr())
            s.update(sc.dt)
            s.state_download_async(h_out.data_ptr())
            e1.record(stream)
    s.synchronize()
    barrier()
    e2e_ms = sum(e0.elapsed_time(e1) for e0, e1 in e2e_ev)
    e2e_t = torch.tensor([e2e_ms], device="cuda")
    if world > 1:
        torch.distributed.all_reduce(e2e_t, op=torch.distributed.ReduceOp.MAX)
    e2e_value = units * args.steps * world / (float(e2e_t.item()) / 1e3)

    # ---- per-kernel times (CUDA events around each launch, same stream)
    s.set_profiling(True)
    prof_tot = {}
    nprof = max(3, min(args.steps, 10))
    for _ in range(nprof):
        with torch.cuda.stream(stream):
            flush.zero_()
        s.update(sc.dt)
        for k, v in s.profile().items():
            prof_tot[k] = prof_tot.get(k, 0.0) + v
    s.set_profiling(False)
    # launches of each kernel per step
    dom = max(prof_tot, key=prof_tot.get)

    def launches_per_step(name: str) -> int:
        if name.startswith("exec_") and "full" not in name:
            return sc.sub_steps  # one link-phase launch per sub-step
        if name in ("grid_insert", "grid_count", "grid_scan", "grid_scatter",
                    "collide_integrate"):
            return sc.sub_steps
        if name == "rigid_ext":
            return sc.sub_steps + 1  # phase A of sub-step 0, B+A between sub-steps, B last
        return 1

    nl = launches_per_step(dom)
    dom_ms = prof_tot[dom] / nprof / nl
    peak, peak_kind = _peaks()
    alg = algorithmic_bytes(dom, sc)
    achieved = alg / (dom_ms / 1e3) / 1e9
    traffic = None
    tf = ROOT / "profiles" / "traffic.json"
    if tf.exists():
        traffic = json.loads(tf.read_text()).get(dom)
    # the link executor is bound by its level chain, not by memory: levels per
    # launch (one body) and the time each level takes
    chain = None
    if dom.startswith("exec_groups"):
        st = s.plan_stats()
        lv = st["levels"] / max(1, st["group_bodies"])
        chain = {"levels_per_launch": lv, "ns_per_level": dom_ms * 1e6 / lv,
                 "issue": link_issue_bound(torch, dom_ms, sc.link_iters * len(sc.la),
                                           LINK_WARP_INSTR["config2"])}

    # every rank steps its shard of the configuration-3 worlds
    batched = None
    if not args.no_batched:
        batched = run_batched_comparison(args, torch, flush, stream, world, rank)

    if rank != 0:
        if world > 1:
            torch.distributed.destroy_process_group()
        return

    cpu = None
    if not args.no_cpu_baseline and world == 1:
        v, k, el = run_cpu_oracle(sc, args.cpu_budget)
        cpu = {"value": v, "unit": METRIC, "cores": 1, "kind": "port",
               "sample": f"{k} updates of the full workload in {el:.1f} s (C port of the "
                         "reference, single thread)"}

    config1 = None
    if not args.no_config1 and world == 1:
        config1 = run_config1_long(args, torch, stream)
    config5 = None
    if not args.no_config5 and world == 1:
        config5 = run_config5(args, torch, flush, stream)
    serving = serving_low = None
    if not args.no_serve and world == 1:
        from bendy2d_gb300.serving import request_pool, run_poisson
        req_workload = ("worlds of log-uniform [64, 16384] particles built like configuration 2 "
                        "(32-wide grids, particle collisions), steps uniform in [60, 600], "
                        "dt 1/60, 8 sub-steps, 4 link iterations, 40 GB budget")
        pool = request_pool(64, 0)
        # the stated rate offers ~15.5 G particle-substeps/s, several times what
        # one GPU serves: a bounded window measures the served capacity, and
        # its latencies measure the backlog
        serving = run_poisson(lam=2000.0, duration=args.serve_window, seed=0,
                              budget_bytes=40 << 30, drain_s=args.serve_drain,
                              scenes_pool=pool, max_resident_particles=args.serve_max_resident)
        serving["workload"] = "Poisson arrivals at 2000 req/s, " + req_workload
        # an arrival rate below the served capacity: latencies measure service
        serving_low = run_poisson(lam=args.serve_low_rate, duration=args.serve_low_window,
                                  seed=1, budget_bytes=40 << 30, drain_s=args.serve_drain,
                                  scenes_pool=pool, max_resident_particles=args.serve_max_resident)
        serving_low["workload"] = (f"Poisson arrivals at {args.serve_low_rate:g} req/s, "
                                   + req_workload)

    out = {
        "metric": METRIC, "value": value, "unit": METRIC, "n_gpus": world, "steps": args.steps,
        "warmup": max(args.warmup, 3), "ms_per_step": ms_max / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded scene generator, bendy2d_gb300/scenes.py:config2)",
        "config": config_dict(sc, world),
        "e2e": {"value": e2e_value, "unit": METRIC, "h2d_bytes_per_step": nbytes,
                "d2h_bytes_per_step": nbytes},
        "roofline": {"bound": "hbm", "kernel": dom, "achieved": achieved, "peak": peak,
                     "unit": "GB/s", "frac": achieved / peak, "peak_source": peak_kind,
                     "traffic": traffic, "algorithmic_bytes_per_launch": alg,
                     "launch_ms": dom_ms, "chain": chain},
        "kernel_ms_per_step": {k: v / nprof for k, v in sorted(prof_tot.items())},
        "kernel_rooflines": kernel_rooflines(
            {k: v / nprof for k, v in prof_tot.items()}, sc,
            {"links": sc.sub_steps, "grid_insert": sc.sub_steps, "grid_count": sc.sub_steps,
             "grid_scan": sc.sub_steps,
             "grid_scatter": sc.sub_steps, "collide_integrate": sc.sub_steps,
             "rigid": sc.sub_steps + 1, "copy_back": 1}),
        "gpu_launches": launches,
        "clocks": clk.summary(),
        "cpu_baseline": cpu,
        "batched_config3": batched,
        "serving_config4": serving,
        "serving_unsaturated": serving_low,
        "stress_config5": config5,
        "long_run_config1": config1,
    }
    print(json.dumps(out))
    if world > 1:
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
