"""ctypes binding of the C ABI in include/bendy2d.h.

The library is built in-tree (bendy2d_gb300/_build/libbendy2d_gb300.so); there
is no CPU fallback, so a missing library is an import-time error.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

_LIB_PATH = Path(__file__).resolve().parent / "_build" / "libbendy2d_gb300.so"

B2D_OK = 0
FAULT_WAIT_TIMEOUT, FAULT_GRID_CAP, FAULT_ALLOC = 1, 2, 3
ERRORS = {
    1: "null argument", 2: "particle link index", 3: "circle link index",
    4: "polygon link index", 5: "bad argument", 6: "index out of range", 7: "CUDA error",
    8: "device error", 9: "over budget", 10: "buffer too small", 11: "bad state",
}


class B2DError(RuntimeError):
    def __init__(self, code: int, message: str):
        super().__init__(f"[{code}] {ERRORS.get(code, 'error')}: {message}")
        self.code = code


class Vec2(C.Structure):
    _fields_ = [("x", C.c_float), ("y", C.c_float)]


class CParticle(C.Structure):
    _fields_ = [("pos", Vec2), ("prev_pos", Vec2), ("acc", Vec2)]


class CLink(C.Structure):
    _fields_ = [("particle_a", C.c_uint64), ("particle_b", C.c_uint64),
                ("target_distance", C.c_float), ("stiffness", C.c_float)]


class CCircle(C.Structure):
    _fields_ = [("point", CParticle), ("radius", C.c_float), ("is_static", C.c_uint32)]


class CNoAllocParams(C.Structure):
    _fields_ = [("gravity_x", C.c_float), ("gravity_y", C.c_float),
                ("bounds_x", C.c_float), ("bounds_y", C.c_float),
                ("bounds_w", C.c_float), ("bounds_h", C.c_float), ("dt", C.c_float),
                ("sub_steps", C.c_uint32), ("particle_radius", C.c_float),
                ("grid_cell", C.c_float)]


class CServerStats(C.Structure):
    _fields_ = [(k, C.c_uint64) for k in ("submitted", "admitted", "completed", "failed",
                                          "queued", "active", "ticks", "particle_substeps",
                                          "resident_bytes", "admit_ns", "step_ns",
                                          "retire_ns", "cancelled", "resident_particles")]


class CPlanStats(C.Structure):
    _fields_ = [("bodies", C.c_uint32), ("group_bodies", C.c_uint32),
                ("serial_bodies", C.c_uint32), ("global_bodies", C.c_uint32),
                ("levels", C.c_uint64), ("ops", C.c_uint64), ("colours", C.c_uint32),
                ("device_bytes", C.c_uint64), ("large_bodies", C.c_uint32)]


_P = C.c_void_p
_F = C.POINTER(C.c_float)
_U64 = C.POINTER(C.c_uint64)
_SZ = C.POINTER(C.c_size_t)

# name -> argtypes (all return int)
SIGNATURES = {
    "b2d_solver_create": [C.POINTER(_P)],
    "b2d_solver_destroy": [_P],
    "b2d_solver_clone": [_P, C.POINTER(_P)],
    "b2d_set_gravity": [_P, C.c_float, C.c_float],
    "b2d_get_gravity": [_P, C.POINTER(Vec2)],
    "b2d_set_bounds": [_P, C.c_float, C.c_float, C.c_float, C.c_float],
    "b2d_get_bounds": [_P, C.POINTER(Vec2), C.POINTER(Vec2)],
    "b2d_set_bounds_active": [_P, C.c_int],
    "b2d_get_bounds_active": [_P, C.POINTER(C.c_int)],
    "b2d_add_particle": [_P, C.c_float, C.c_float],
    "b2d_add_circle": [_P, C.POINTER(CCircle)],
    "b2d_add_polygon": [_P, C.c_size_t, C.POINTER(CParticle), C.c_size_t, C.POINTER(CLink),
                        C.c_int, Vec2, C.c_float],
    "b2d_add_particle_link": [_P, C.c_uint64, C.c_uint64, C.c_float],
    "b2d_add_circle_link": [_P, C.c_uint64, C.c_uint64, C.c_float],
    "b2d_add_particle_prev": [_P, C.c_float, C.c_float, C.c_float, C.c_float],
    "b2d_add_particles": [_P, C.c_size_t, _F, _F],
    "b2d_add_particle_links": [_P, C.c_size_t, _U64, _U64, _F, _F],
    "b2d_add_polygon_circle": [_P, C.c_float, Vec2, C.c_size_t, C.c_int],
    "b2d_add_polygon_points": [_P, C.c_size_t, C.POINTER(Vec2), C.c_int],
    "b2d_set_sub_steps": [_P, C.c_uint32],
    "b2d_get_sub_steps": [_P, C.POINTER(C.c_uint32)],
    "b2d_set_link_iters": [_P, C.c_uint32],
    "b2d_set_mode": [_P, C.c_int],
    "b2d_set_collision": [_P, C.c_uint32, C.c_float, C.c_float],
    "b2d_set_circle_static": [_P, C.c_size_t, C.c_int],
    "b2d_set_tuning": [_P, C.c_char_p, C.c_double],
    "b2d_update": [_P, C.c_float],
    "b2d_set_fault": [_P, C.c_int, C.c_uint64],
    "b2d_get_particle_len": [_P, _SZ],
    "b2d_get_circles_len": [_P, _SZ],
    "b2d_get_polygons_len": [_P, _SZ],
    "b2d_get_particle_links_len": [_P, _SZ],
    "b2d_get_circle_links_len": [_P, _SZ],
    "b2d_get_particle_links": [_P, C.POINTER(CLink), C.c_size_t],
    "b2d_get_circle_links": [_P, C.POINTER(CLink), C.c_size_t],
    "b2d_get_particles": [_P, C.POINTER(CParticle), C.c_size_t],
    "b2d_get_circles": [_P, C.POINTER(CCircle), C.c_size_t],
    "b2d_get_particle": [_P, C.c_size_t, C.POINTER(CParticle)],
    "b2d_get_circle": [_P, C.c_size_t, C.POINTER(CCircle)],
    "b2d_get_polygon_info": [_P, C.c_size_t, _SZ, _SZ, C.POINTER(C.c_int), C.POINTER(Vec2),
                             _F],
    "b2d_get_polygon": [_P, C.c_size_t, C.POINTER(CParticle), C.c_size_t, C.POINTER(CLink),
                        C.c_size_t],
    "b2d_read_state": [_P, _F, _F],
    "b2d_write_state": [_P, _F, _F],
    "b2d_set_stream": [_P, _P],
    "b2d_synchronize": [_P],
    "b2d_set_graphs": [_P, C.c_int],
    "b2d_set_profiling": [_P, C.c_int],
    "b2d_get_profile": [_P, C.c_char_p, C.c_size_t, _F, C.c_size_t, _SZ],
    "b2d_get_launch_count": [_P, C.POINTER(C.c_uint32)],
    "b2d_state_bytes": [_P, _SZ],
    "b2d_state_upload_async": [_P, _P],
    "b2d_state_download_async": [_P, _P],
    "b2d_get_plan_stats": [_P, C.POINTER(CPlanStats)],
    "b2d_get_link_order": [_P, _U64, C.c_size_t],
    "b2d_collide_substeps_noalloc": [_P, _P, C.c_size_t, C.POINTER(CNoAllocParams), _P],
    "b2d_batch_create": [C.POINTER(_P)],
    "b2d_batch_destroy": [_P],
    "b2d_batch_add": [_P, _P],
    "b2d_batch_remove": [_P, _P],
    "b2d_batch_update": [_P, C.c_float],
    "b2d_batch_synchronize": [_P],
    "b2d_batch_set_stream": [_P, _P],
    "b2d_batch_set_profiling": [_P, C.c_int],
    "b2d_batch_get_profile": [_P, C.c_char_p, C.c_size_t, _F, C.c_size_t, _SZ],
    "b2d_batch_get_launch_count": [_P, C.POINTER(C.c_uint32)],
    "b2d_batch_set_plain": [_P, C.c_int],
    "b2d_batch_set_tuning": [_P, C.c_char_p, C.c_double],
    "b2d_server_create": [C.c_uint64, C.POINTER(_P)],
    "b2d_server_destroy": [_P],
    "b2d_server_start": [_P],
    "b2d_server_stop": [_P],
    "b2d_server_submit": [_P, _P, C.c_uint32, C.c_float, C.POINTER(C.c_uint64)],
    "b2d_server_poll": [_P, C.c_uint64, C.POINTER(C.c_int)],
    "b2d_server_cancel": [_P, C.c_uint64],
    "b2d_server_set_max_resident_particles": [_P, C.c_uint64],
    "b2d_server_set_fault": [_P, C.c_int, C.c_uint64],
    "b2d_server_take": [_P, C.c_uint64, _P, C.POINTER(C.c_double), C.POINTER(C.c_double)],
    "b2d_server_get_stats": [_P, C.POINTER(CServerStats)],
    "b2d_server_finished": [_P, C.POINTER(C.c_uint64), C.c_size_t, C.POINTER(C.c_size_t)],
}

_lib = None


def lib_path() -> Path:
    return _LIB_PATH


def load() -> C.CDLL:
    """Load the C-ABI library; raise if it has not been built."""
    global _lib
    if _lib is not None:
        return _lib
    if not _LIB_PATH.exists():
        raise ImportError(
            f"{_LIB_PATH} is missing: build it with `python -c \"import __graft_entry__ as g; "
            "g.build()\"` (bendy2d-gb300 has no CPU fallback)")
    lib = C.CDLL(str(_LIB_PATH))
    for name, args in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.argtypes = args
        fn.restype = C.c_int
    lib.b2d_last_error.restype = C.c_char_p
    lib.b2d_last_error.argtypes = []
    lib.b2d_version.restype = C.c_char_p
    lib.b2d_version.argtypes = []
    _lib = lib
    return lib


def check(code: int) -> None:
    if code != B2D_OK:
        msg = _lib.b2d_last_error().decode() if _lib is not None else ""
        raise B2DError(code, msg)
