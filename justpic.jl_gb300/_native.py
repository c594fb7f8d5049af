"""ctypes binding of libjustpic_gb300.so (include/justpic_gb300.h).

The library is loaded lazily on first use. There is no fallback: if the shared
library has not been built, every entry point raises ``NativeLibraryMissing``.
"""
from __future__ import annotations

import ctypes
import os
import threading

from . import native_build as _build

JP_OK = 0
JP_ERR_INVALID_ARGUMENT = -1
JP_ERR_CUDA = -2
JP_ERR_OUT_OF_MEMORY = -3
JP_ERR_BISECTION_LIMIT = -4
JP_ERR_NOT_BUILT = -5
JP_ERR_ADJOINT_WINDOW = -6

JP_WARN_FAR_MOVE = 0x2
JP_WARN_NO_NEIGHBOUR = 0x4

JP_EULER, JP_RUNGE_KUTTA2, JP_RUNGE_KUTTA4 = 0, 1, 2
JP_MAX_ARGS = 16


class JustPICError(RuntimeError):
    """A failing call of the native library (CUDA error, iteration cap, ...)."""

    def __init__(self, code: int, message: str):
        super().__init__(f"{message} (code {code})")
        self.code = code


class ArgumentError(ValueError):
    """Counterpart of Julia's ArgumentError raised by the reference."""


class NativeLibraryMissing(ImportError):
    pass


class GridDesc(ctypes.Structure):
    _fields_ = [
        ("ndim", ctypes.c_int32),
        ("uniform", ctypes.c_int32),
        ("xi_vel", (ctypes.POINTER(ctypes.c_double) * 3) * 3),
        ("n_vel", (ctypes.c_int64 * 3) * 3),
    ]


P3 = ctypes.c_void_p * 3

# (name, restype, argtypes) for every symbol of include/justpic_gb300.h
SIGNATURES = [
    ("jp_particles_create", ctypes.c_int,
     [ctypes.POINTER(ctypes.c_void_p), ctypes.POINTER(GridDesc), ctypes.c_int32, ctypes.c_int32, ctypes.c_int32,
      ctypes.c_uint64]),
    ("jp_particles_destroy", ctypes.c_int, [ctypes.c_void_p]),
    ("jp_particles_info", ctypes.c_int,
     [ctypes.c_void_p, ctypes.POINTER(ctypes.c_int32), ctypes.c_int64 * 3, ctypes.POINTER(ctypes.c_int32),
      ctypes.POINTER(ctypes.c_int32), ctypes.POINTER(ctypes.c_int32), ctypes.POINTER(ctypes.c_int64)]),
    ("jp_set_stream", ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p]),
    ("jp_set_synchronous", ctypes.c_int, [ctypes.c_void_p, ctypes.c_int32]),
    ("jp_synchronize", ctypes.c_int, [ctypes.c_void_p]),
    ("jp_get_warnings", ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ctypes.c_uint32), ctypes.c_int32]),
    ("jp_get_move_counts", ctypes.c_int, [ctypes.c_void_p, ctypes.c_uint64 * 3, ctypes.c_int32]),
    ("jp_grid2particle_n", ctypes.c_int,
     [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int32, P3, ctypes.c_void_p]),
    ("jp_particle2grid_n", ctypes.c_int,
     [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int32, P3, ctypes.c_void_p]),
    ("jp_get_rng_counter", ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ctypes.c_uint64)]),
    ("jp_set_rng_counter", ctypes.c_int, [ctypes.c_void_p, ctypes.c_uint64]),
    ("jp_last_error", ctypes.c_char_p, []),
    ("jp_init_particles", ctypes.c_int, [ctypes.c_void_p, P3, ctypes.c_void_p]),
    ("jp_advection", ctypes.c_int,
     [ctypes.c_void_p, ctypes.c_int32, ctypes.c_double, P3, ctypes.c_double, P3, ctypes.c_void_p]),
    ("jp_advection_linp", ctypes.c_int,
     [ctypes.c_void_p, ctypes.c_int32, ctypes.c_double, P3, ctypes.c_double, P3, ctypes.c_void_p]),
    ("jp_advection_mqs", ctypes.c_int,
     [ctypes.c_void_p, ctypes.c_int32, ctypes.c_double, P3, ctypes.c_double, P3, ctypes.c_void_p]),
    ("jp_move_particles", ctypes.c_int, [ctypes.c_void_p, P3, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int32]),
    ("jp_move_particles_noalloc", ctypes.c_int,
     [ctypes.c_void_p, P3, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int32]),
    ("jp_inject_particles", ctypes.c_int, [ctypes.c_void_p, P3, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int32]),
    ("jp_inject_particles_phase", ctypes.c_int,
     [ctypes.c_void_p, P3, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
      ctypes.c_int32]),
    ("jp_grid2particle", ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, P3, ctypes.c_void_p]),
    ("jp_particle2grid", ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, P3, ctypes.c_void_p]),
    # split-precision (FP32 cell offset) form
    ("jp_offsets_from_coords", ctypes.c_int, [ctypes.c_void_p, P3, ctypes.c_void_p, P3]),
    ("jp_coords_from_offsets", ctypes.c_int, [ctypes.c_void_p, P3, ctypes.c_void_p, P3]),
    ("jp_advection_f32", ctypes.c_int,
     [ctypes.c_void_p, ctypes.c_int32, ctypes.c_double, P3, ctypes.c_double, P3, ctypes.c_void_p]),
    ("jp_move_particles_f32", ctypes.c_int,
     [ctypes.c_void_p, P3, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int32]),
    ("jp_inject_particles_f32", ctypes.c_int,
     [ctypes.c_void_p, P3, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int32]),
    ("jp_grid2particle_f32", ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, P3, ctypes.c_void_p]),
    ("jp_particle2grid_f32", ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, P3, ctypes.c_void_p]),
    # transfers beside the hot path
    ("jp_grid2particle_flip", ctypes.c_int,
     [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_double, P3, ctypes.c_void_p]),
    ("jp_centroid2particle", ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, P3]),
    ("jp_phase_ratios", ctypes.c_int,
     [ctypes.c_void_p, ctypes.c_int32, ctypes.c_void_p, P3, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]),
    ("jp_phase_ratios_midpoints", ctypes.c_int, [ctypes.c_void_p, ctypes.c_int32, ctypes.c_void_p, P3, P3]),
    ("jp_particle2centroid", ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, P3]),
    ("jp_advection_record_bytes", ctypes.c_int, [ctypes.c_void_p, ctypes.c_int32, ctypes.POINTER(ctypes.c_uint64)]),
    ("jp_advection_record", ctypes.c_int,
     [ctypes.c_void_p, ctypes.c_int32, ctypes.c_double, P3, ctypes.c_double, P3, ctypes.c_void_p, ctypes.c_void_p]),
    ("jp_advection_vjp_recorded", ctypes.c_int,
     [ctypes.c_void_p, ctypes.c_int32, ctypes.c_double, ctypes.c_double, ctypes.c_void_p, ctypes.c_void_p, P3, P3]),
    ("jp_selftest_weight", ctypes.c_int,
     [ctypes.c_uint64, ctypes.c_int64, ctypes.POINTER(ctypes.c_int64), ctypes.POINTER(ctypes.c_uint64)]),
    ("jp_cellarray_permute", ctypes.c_int,
     [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64, ctypes.c_int32, ctypes.c_int32,
      ctypes.c_int32]),
    # adjoint (2D, FP64)
    ("jp_particle2grid_with_weights", ctypes.c_int,
     [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, P3, ctypes.c_void_p]),
    ("jp_move_permutation", ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p]),
    ("jp_permute_vjp", ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                      ctypes.c_int32]),
    ("jp_slot_ids", ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]),
    ("jp_inject_vjp", ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                     ctypes.c_int32, ctypes.c_int32]),
    ("jp_advection_vjp", ctypes.c_int,
     [ctypes.c_void_p, ctypes.c_int32, ctypes.c_double, P3, ctypes.c_double, P3, ctypes.c_void_p, P3, P3]),
    ("jp_particle2grid_vjp", ctypes.c_int,
     [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, P3, ctypes.c_void_p, ctypes.c_void_p,
      ctypes.c_void_p, ctypes.c_void_p]),
    ("jp_grid2particle_vjp", ctypes.c_int,
     [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, P3, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]),
    # adjoint of the split-precision form
    ("jp_slot_ids_i32", ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]),
    ("jp_inject_vjp_i32", ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                         ctypes.c_int32, ctypes.c_int32]),
    ("jp_advection_vjp_f32", ctypes.c_int,
     [ctypes.c_void_p, ctypes.c_int32, ctypes.c_double, P3, ctypes.c_double, P3, ctypes.c_void_p, P3, P3]),
    ("jp_particle2grid_f32_with_weights", ctypes.c_int,
     [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, P3, ctypes.c_void_p]),
    ("jp_particle2grid_vjp_f32", ctypes.c_int,
     [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, P3, ctypes.c_void_p, ctypes.c_void_p,
      ctypes.c_void_p, ctypes.c_void_p]),
]

_lib = None
_lock = threading.Lock()


def library_path() -> str:
    return _build.LIB


def load(build_if_missing: bool = False):
    """Load the shared library (building it first if asked and nvcc exists)."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        path = _build.LIB
        if build_if_missing and _build.is_stale():
            _build.build()
        if not os.path.exists(path):
            raise NativeLibraryMissing(
                f"{path} is not built; run `python -c \"import __graft_entry__ as g; g.build()\"` "
                "(the GB300 kernels have no CPU fallback)")
        lib = ctypes.CDLL(path)
        for name, res, args in SIGNATURES:
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _lib = lib
        return lib


def last_error() -> str:
    msg = load().jp_last_error()
    return msg.decode("utf-8", "replace") if msg else ""


def check(rc: int, what: str = "") -> None:
    if rc == JP_OK:
        return
    msg = last_error() or what
    if rc == JP_ERR_INVALID_ARGUMENT:
        raise ArgumentError(msg)
    raise JustPICError(rc, msg)
