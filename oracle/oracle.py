"""ctypes wrapper of the C oracle (oracle/b2d_oracle.c).  Test infrastructure."""
from __future__ import annotations

import ctypes as C
from typing import Optional

import numpy as np

from . import build as _build

_lib = None
_F = C.POINTER(C.c_float)
_U = C.POINTER(C.c_uint64)


def _load():
    global _lib
    if _lib is None:
        lib = C.CDLL(str(_build.build()))
        P = C.c_void_p
        sig = {
            "orc_new": ([], P), "orc_free": ([P], None), "orc_clone": ([P], P),
            "orc_set_gravity": ([P, C.c_float, C.c_float], None),
            "orc_set_bounds": ([P, C.c_float, C.c_float, C.c_float, C.c_float], None),
            "orc_set_sub_steps": ([P, C.c_uint32], None),
            "orc_set_link_iters": ([P, C.c_uint32], None),
            "orc_set_collide": ([P, C.c_uint32, C.c_float, C.c_float], None),
            "orc_add_particles": ([P, C.c_size_t, _F, _F], None),
            "orc_add_particle_links": ([P, C.c_size_t, _U, _U, _F, _F], None),
            "orc_add_circle": ([P, _F, _F, _F, C.c_float, C.c_int], None),
            "orc_add_circle_link": ([P, C.c_uint64, C.c_uint64, C.c_float], None),
            "orc_add_polygon": ([P, C.c_size_t, _F, _F, _F, C.c_size_t, _U, _U, _F, C.c_int,
                                 C.c_float, C.c_float, C.c_float], None),
            "orc_add_polygon_circle": ([P, C.c_float, C.c_float, C.c_float, C.c_size_t,
                                        C.c_int], None),
            "orc_add_polygon_points": ([P, C.c_size_t, _F, C.c_int], None),
            "orc_update": ([P, C.c_float], C.c_int),
            "orc_particle_len": ([P], C.c_size_t), "orc_circle_len": ([P], C.c_size_t),
            "orc_polygon_len": ([P], C.c_size_t),
            "orc_polygon_vertex_len": ([P, C.c_size_t], C.c_size_t),
            "orc_polygon_link_len": ([P, C.c_size_t], C.c_size_t),
            "orc_read_particles": ([P, _F, _F], None),
            "orc_read_circles": ([P, _F, _F], None),
            "orc_read_polygon": ([P, C.c_size_t, _F, _F, _F], None),
            "orc_read_polygon_links": ([P, C.c_size_t, _U, _U, _F], None),
            "orc_link_residual": ([P], C.c_double),
        }
        for name, (args, res) in sig.items():
            fn = getattr(lib, name)
            fn.argtypes = args
            fn.restype = res
        _lib = lib
    return _lib


def _f(a):
    if a is None:
        return None
    return np.ascontiguousarray(a, dtype=np.float32).ctypes.data_as(_F)


class Oracle:
    """The reference's Solver, restated in C, driven with the same calls."""

    def __init__(self, _handle=None):
        self._lib = _load()
        self._h = _handle or self._lib.orc_new()
        self._keep = []

    def __del__(self):
        try:
            if self._h:
                self._lib.orc_free(self._h)
                self._h = None
        except Exception:
            pass

    def clone(self) -> "Oracle":
        return Oracle(self._lib.orc_clone(self._h))

    def set_gravity(self, x, y): self._lib.orc_set_gravity(self._h, x, y)
    def set_bounds(self, px, py, sx, sy): self._lib.orc_set_bounds(self._h, px, py, sx, sy)
    def set_sub_steps(self, n): self._lib.orc_set_sub_steps(self._h, n)
    def set_link_iters(self, n): self._lib.orc_set_link_iters(self._h, n)
    def set_collision(self, flags, r=0.5, cell=1.0): self._lib.orc_set_collide(self._h, flags, r, cell)

    def add_particles(self, pos, prev=None):
        pos = np.ascontiguousarray(pos, np.float32).reshape(-1, 2)
        prev = None if prev is None else np.ascontiguousarray(prev, np.float32).reshape(-1, 2)
        self._lib.orc_add_particles(self._h, len(pos), _f(pos), _f(prev))

    def add_particle_links(self, a, b, rest, stiff=None):
        a = np.ascontiguousarray(a, np.uint64)
        b = np.ascontiguousarray(b, np.uint64)
        rest = np.ascontiguousarray(rest, np.float32)
        st = None if stiff is None else np.ascontiguousarray(stiff, np.float32)
        self._lib.orc_add_particle_links(self._h, len(a), a.ctypes.data_as(_U),
                                         b.ctypes.data_as(_U), _f(rest), _f(st))

    def add_circle(self, pos, prev=None, acc=None, radius=1.0, is_static=False):
        self._lib.orc_add_circle(self._h, _f(np.asarray(pos, np.float32)),
                                 _f(None if prev is None else np.asarray(prev, np.float32)),
                                 _f(None if acc is None else np.asarray(acc, np.float32)),
                                 radius, int(is_static))

    def add_circle_link(self, a, b, rest): self._lib.orc_add_circle_link(self._h, a, b, rest)

    def add_polygon(self, pos, prev=None, acc=None, links=(), is_static=False,
                    center=(0.0, 0.0), scale=1.0):
        pos = np.ascontiguousarray(pos, np.float32).reshape(-1, 2)
        la = np.asarray([l[0] for l in links], np.uint64)
        lb = np.asarray([l[1] for l in links], np.uint64)
        lt = np.asarray([l[2] for l in links], np.float32)
        self._lib.orc_add_polygon(self._h, len(pos), _f(pos), _f(prev), _f(acc), len(la),
                                  la.ctypes.data_as(_U), lb.ctypes.data_as(_U), _f(lt),
                                  int(is_static), center[0], center[1], scale)

    def add_polygon_circle(self, radius, x, y, n, is_static):
        self._lib.orc_add_polygon_circle(self._h, radius, x, y, n, int(is_static))

    def add_polygon_points(self, pts, is_static):
        pts = np.ascontiguousarray(pts, np.float32).reshape(-1, 2)
        self._lib.orc_add_polygon_points(self._h, len(pts), _f(pts), int(is_static))

    def update(self, dt) -> int:
        return self._lib.orc_update(self._h, dt)

    def particles(self):
        n = self._lib.orc_particle_len(self._h)
        pos = np.empty((n, 2), np.float32)
        prev = np.empty((n, 2), np.float32)
        self._lib.orc_read_particles(self._h, _f_out(pos), _f_out(prev))
        return pos, prev

    def circles(self):
        n = self._lib.orc_circle_len(self._h)
        pos = np.empty((n, 2), np.float32)
        prev = np.empty((n, 2), np.float32)
        self._lib.orc_read_circles(self._h, _f_out(pos), _f_out(prev))
        return pos, prev

    def polygons(self):
        out = []
        for k in range(self._lib.orc_polygon_len(self._h)):
            n = self._lib.orc_polygon_vertex_len(self._h, k)
            pos = np.empty((n, 2), np.float32)
            prev = np.empty((n, 2), np.float32)
            ctr = np.empty(2, np.float32)
            self._lib.orc_read_polygon(self._h, k, _f_out(pos), _f_out(prev), _f_out(ctr))
            out.append((pos, prev, ctr))
        return out

    def polygon_links(self, k):
        n = self._lib.orc_polygon_link_len(self._h, k)
        a = np.empty(n, np.uint64)
        b = np.empty(n, np.uint64)
        t = np.empty(n, np.float32)
        self._lib.orc_read_polygon_links(self._h, k, a.ctypes.data_as(_U),
                                         b.ctypes.data_as(_U), _f_out(t))
        return a, b, t

    def link_residual(self) -> float:
        return self._lib.orc_link_residual(self._h)


def _f_out(a: np.ndarray):
    return a.ctypes.data_as(_F)


def load_scene(scene, link_order: Optional[np.ndarray] = None) -> Oracle:
    """Load a bendy2d_gb300.scenes.Scene into a fresh oracle.  link_order
    (fast mode) permutes the particle links into the order the GPU runs."""
    o = Oracle()
    o.set_gravity(*scene.gravity)
    o.set_bounds(*scene.bounds)
    o.set_sub_steps(scene.sub_steps)
    o.set_link_iters(scene.link_iters)
    o.set_collision(scene.collide, scene.radius, scene.cell)
    o.add_particles(scene.pos, scene.prev)
    la, lb, rest, stiff = scene.la, scene.lb, scene.rest, scene.stiff
    if link_order is not None:
        idx = np.asarray(link_order, np.int64)
        la, lb, rest, stiff = la[idx], lb[idx], rest[idx], stiff[idx]
    if len(la):
        o.add_particle_links(la, lb, rest, stiff)
    for c in scene.circles:
        o.add_circle(c["pos"], c["prev"], c["acc"], float(c["radius"]), c["static"])
    for a, b, r in scene.circle_links:
        o.add_circle_link(int(a), int(b), float(r))
    for g in scene.polygons:
        o.add_polygon_points(g["points"], g["static"])
    return o
