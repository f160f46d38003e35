"""Serving: continuous batching of world-solve requests (Python side).

``Server`` wraps the native request loop (include/bendy2d.h, b2d_server_*):
requests are admitted under a device-memory budget, kept device-resident
across steps, and stepped together.  ``run_poisson`` drives it with seeded
Poisson arrivals of configuration-4 requests (a config-2-style world of
log-uniform [64, 16384] particles and a step count uniform in [60, 600]) and
reports latency percentiles beside throughput.
"""
from __future__ import annotations

import ctypes as C
import threading
import time
from typing import Optional

import numpy as np

from . import _native as N
from .api import Solver

QUEUED, RUNNING, DONE, FAILED, CANCELLED = 0, 1, 2, 3, 4


class Server:
    def __init__(self, budget_bytes: int):
        self._lib = N.load()
        h = C.c_void_p()
        N.check(self._lib.b2d_server_create(int(budget_bytes), C.byref(h)))
        self._h = h

    def start(self) -> None:
        N.check(self._lib.b2d_server_start(self._h))

    def stop(self) -> None:
        N.check(self._lib.b2d_server_stop(self._h))

    def close(self) -> None:
        if getattr(self, "_h", None):
            self._lib.b2d_server_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def submit(self, world: Solver, steps: int, dt: float) -> int:
        rid = C.c_uint64()
        N.check(self._lib.b2d_server_submit(self._h, world._h, steps, dt, C.byref(rid)))
        return rid.value

    def poll(self, rid: int) -> int:
        st = C.c_int()
        N.check(self._lib.b2d_server_poll(self._h, rid, C.byref(st)))
        return st.value

    def cancel(self, rid: int) -> None:
        """Drop a request: a queued one at once, a running one when the tick
        in flight ends; it is then listed by finished() as CANCELLED."""
        N.check(self._lib.b2d_server_cancel(self._h, rid))

    def set_max_resident_particles(self, n: int) -> None:
        """Admission keeps the resident solver particles at or below n (0: no
        limit); one request is always admitted onto an idle device."""
        N.check(self._lib.b2d_server_set_max_resident_particles(self._h, int(n)))

    def set_fault(self, kind: int, value: int) -> None:
        """Fault injection for tests (FAULT_* of _native), applied before the
        worker's next tick."""
        N.check(self._lib.b2d_server_set_fault(self._h, int(kind), int(value)))

    def finished(self, cap: int = 4096) -> list:
        buf = (C.c_uint64 * cap)()
        n = C.c_size_t()
        N.check(self._lib.b2d_server_finished(self._h, buf, cap, C.byref(n)))
        return [buf[i] for i in range(n.value)]

    def take(self, rid: int) -> tuple:
        """(solver holding the final world, latency s, queueing s)"""
        out = Solver()
        lat, q = C.c_double(), C.c_double()
        N.check(self._lib.b2d_server_take(self._h, rid, out._h, C.byref(lat), C.byref(q)))
        return out, lat.value, q.value

    def stats(self) -> dict:
        s = N.CServerStats()
        N.check(self._lib.b2d_server_get_stats(self._h, C.byref(s)))
        return {k: getattr(s, k) for k, _ in N.CServerStats._fields_}


def request_pool(n: int, seed: int, lo: int = 64, hi: int = 16384) -> list:
    """n request worlds with particle counts log-uniform in [lo, hi]."""
    from . import scenes
    rng = np.random.default_rng(seed)
    sizes = np.exp(rng.uniform(np.log(lo), np.log(hi), size=n)).astype(int)
    return [scenes.config4_request(rng, int(k)) for k in sizes]


def run_poisson(lam: float = 2000.0, duration: float = 60.0, seed: int = 0,
                budget_bytes: int = 40 << 30, pool: int = 64, steps_lo: int = 60,
                steps_hi: int = 600, drain_s: float = 30.0,
                scenes_pool: Optional[list] = None,
                max_resident_particles: int = 0) -> dict:
    """Seeded Poisson arrivals for `duration` seconds; waits up to `drain_s`
    afterwards for outstanding requests.  Latency = submit to completion.

    Reported beside the latency percentiles (over completed requests): the
    offered load (particle-substeps of every submitted request / arrival
    window), the served throughput (particle-substeps of completed requests /
    wall time from the first arrival to the last completion or the drain
    limit) and their ratio; a ratio well below 1 means the arrivals exceed
    the device's capacity and the latencies measure the backlog."""
    rng = np.random.default_rng(seed + 1)
    worlds = scenes_pool or request_pool(pool, seed)
    solvers = [w.to_solver() for w in worlds]
    gaps = rng.exponential(1.0 / lam, size=int(lam * duration * 1.5) + 16)
    times = np.cumsum(gaps)
    times = times[times < duration]
    picks = rng.integers(0, len(worlds), size=len(times))
    steps = rng.integers(steps_lo, steps_hi + 1, size=len(times))
    units_of = np.array([int(worlds[w].n_particles) * worlds[w].sub_steps for w in picks],
                        np.float64) * steps
    sv = Server(budget_bytes)
    if max_resident_particles:
        sv.set_max_resident_particles(max_resident_particles)
    sv.start()
    info = {}
    lock = threading.Lock()
    t0 = time.perf_counter()

    def submitter():
        for k, (t, w, st) in enumerate(zip(times, picks, steps)):
            delay = t0 + t - time.perf_counter()
            if delay > 0:
                time.sleep(delay)
            rid = sv.submit(solvers[w], int(st), worlds[w].dt)
            with lock:
                info[rid] = (k, float(units_of[k]))

    th = threading.Thread(target=submitter, daemon=True)
    th.start()
    lat, qt, done_units = [], [], 0.0
    deadline = t0 + duration + drain_s
    done = 0
    t_last = t0
    while True:
        for rid in sv.finished():
            s, l, q = sv.take(rid)
            lat.append(l)
            qt.append(q)
            with lock:
                done_units += info[rid][1]
            done += 1
            t_last = time.perf_counter()
            s.close()
        if not th.is_alive() and done >= len(times):
            break
        if time.perf_counter() > deadline:
            t_last = time.perf_counter()
            break
        time.sleep(0.002)
    wall = t_last - t0
    stats = sv.stats()
    sv.stop()
    sv.close()
    lat_ms = np.asarray(lat) * 1e3
    offered = float(units_of.sum()) / duration
    served = done_units / wall if wall > 0 else 0.0
    return {
        "arrival_rate_per_s": lam, "arrival_window_s": duration, "submitted": int(len(times)),
        "completed": done, "incomplete_at_drain_limit": int(len(times)) - done,
        "drain_limit_s": drain_s, "wall_s": wall,
        "max_resident_particles": int(max_resident_particles),
        "p50_latency_ms": float(np.percentile(lat_ms, 50)) if done else None,
        "p99_latency_ms": float(np.percentile(lat_ms, 99)) if done else None,
        "mean_queue_ms": float(np.mean(qt) * 1e3) if done else None,
        "offered_particle_substeps_per_s": offered,
        "served_particle_substeps_per_s": served,
        "served_over_offered": served / offered if offered > 0 else None,
        "stepped_particle_substeps_per_s": stats["particle_substeps"] / wall if wall > 0 else 0.0,
        "ticks": stats["ticks"], "budget_bytes": budget_bytes,
        "worker_s": {"admit": stats["admit_ns"] / 1e9, "step": stats["step_ns"] / 1e9,
                     "retire": stats["retire_ns"] / 1e9},
    }
