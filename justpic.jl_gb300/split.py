"""Split-precision form: an int32 cell (the slot's cell) plus an FP32 offset
within it, on top of the same ``Particles`` container (geometry, index and
injection counter are shared with the FP64 form).

``xi = init_offsets(particles)`` converts the container's FP64 coordinates
into FP32 offsets in cell units; the ``*_f32_`` functions mirror the FP64 API
(``advection_f32_(particles, xi, method, V32, dt)`` etc.) with FP32 velocity,
particle and vertex fields. ``coords_from_offsets(particles, xi)`` returns
FP64 coordinates for output. Uniform (``LinRange``) grids and vector grids
with the standard staggering (cell midpoints plus one ghost node at each end
for the centred axes); the container decides at creation.
"""
from __future__ import annotations

import ctypes

import torch

from . import _native
from ._native import JP_MAX_ARGS, ArgumentError, P3
from .api import _bind_stream, _check_cellarray, _finish, _vertex_shape
from .integrators import AbstractAdvectionIntegrator
from .particles import CellArray, Particles


def _p3(arrs, N):
    return P3(*[a.data_ptr() for a in arrs], *([None] * (3 - N)))


def _check_xi(p: Particles, xi):
    xi = tuple(xi)
    if len(xi) != p.ndim:
        raise ArgumentError(f"xi must have {p.ndim} components")
    for d, a in enumerate(xi):
        _check_cellarray(p, a, f"xi[{d}]", torch.float32)
    return xi


def cell_array_f32(particles: Particles, fill=0.0) -> CellArray:
    data = torch.full((particles.max_xcell, int(torch.tensor(particles.ni).prod())), float(fill),
                      dtype=torch.float32, device="cuda")
    return CellArray(data, particles.ni)


def init_cell_arrays_f32(particles: Particles, n) -> tuple:
    """FP32 counterpart of ``init_cell_arrays``."""
    return tuple(cell_array_f32(particles, 0.0) for _ in range(int(n)))


def grid_field_f32(shape, fill=0.0) -> torch.Tensor:
    t = torch.full(tuple(reversed(shape)), float(fill), dtype=torch.float32, device="cuda")
    return t.permute(*reversed(range(t.dim())))


def init_offsets(particles: Particles) -> tuple:
    """FP32 offsets (cell units) of the container's live particles; NaN in empty slots."""
    xi = tuple(cell_array_f32(particles, float("nan")) for _ in range(particles.ndim))
    _bind_stream(particles)
    rc = _native.load().jp_offsets_from_coords(particles.handle, _p3(particles.coords, particles.ndim),
                                               particles.index.data_ptr(), _p3(xi, particles.ndim))
    _finish(particles, rc, "offsets_from_coords")
    return xi


def coords_from_offsets(particles: Particles, xi) -> tuple:
    """FP64 coordinates x = x_cell + xi * dx of the live particles (NaN elsewhere)."""
    xi = _check_xi(particles, xi)
    out = tuple(CellArray(torch.full_like(c.data, float("nan")), particles.ni) for c in particles.coords)
    _bind_stream(particles)
    rc = _native.load().jp_coords_from_offsets(particles.handle, _p3(xi, particles.ndim), particles.index.data_ptr(),
                                               _p3(out, particles.ndim))
    _finish(particles, rc, "coords_from_offsets")
    return out


def _args32(p, args):
    args = tuple(args) if args is not None else ()
    if len(args) > JP_MAX_ARGS:
        raise ArgumentError(f"at most {JP_MAX_ARGS} particle fields are supported")
    for k, a in enumerate(args):
        _check_cellarray(p, a, f"args[{k}]", torch.float32)
    arr = (ctypes.c_void_p * max(1, len(args)))(*[a.data_ptr() for a in args])
    return arr, len(args)


def _check_grid32(t, shape, what):
    if not isinstance(t, torch.Tensor) or t.dtype != torch.float32:
        raise ArgumentError(f"{what} must be a float32 CUDA tensor")
    if not t.is_cuda or tuple(t.shape) != tuple(shape):
        raise ArgumentError(f"{what} has shape {tuple(t.shape)}, expected {tuple(shape)}")
    strides = [1]
    for n in shape[:-1]:
        strides.append(strides[-1] * n)
    if tuple(t.stride()) != tuple(strides):
        raise ArgumentError(f"{what} must be column-major (Julia layout)")


def advection_f32_(particles: Particles, xi, method: AbstractAdvectionIntegrator, V, dt) -> None:
    """``advection!`` on FP32 offsets with FP32 staggered velocity components."""
    if not isinstance(method, AbstractAdvectionIntegrator):
        raise ArgumentError("method must be Euler(), RungeKutta2(α) or RungeKutta4()")
    xi = _check_xi(particles, xi)
    V = tuple(V)
    N = particles.ndim
    if len(V) != N:
        raise ArgumentError(f"V must have {N} components")
    for c in range(N):
        _check_grid32(V[c], tuple(len(x) for x in particles.xi_vel[c]), f"V[{c}]")
    _bind_stream(particles)
    rc = _native.load().jp_advection_f32(particles.handle, method.code, float(method.alpha), _p3(V, N), float(dt),
                                         _p3(xi, N), particles.index.data_ptr())
    _finish(particles, rc, "advection_f32!")


def move_particles_f32_(particles: Particles, xi, args=()) -> None:
    xi = _check_xi(particles, xi)
    arr, n = _args32(particles, args)
    _bind_stream(particles)
    rc = _native.load().jp_move_particles_f32(particles.handle, _p3(xi, particles.ndim), particles.index.data_ptr(),
                                              arr, n)
    _finish(particles, rc, "move_particles_f32!")


def inject_particles_f32_(particles: Particles, xi, args=()) -> None:
    xi = _check_xi(particles, xi)
    arr, n = _args32(particles, args)
    _bind_stream(particles)
    rc = _native.load().jp_inject_particles_f32(particles.handle, _p3(xi, particles.ndim),
                                                particles.index.data_ptr(), arr, n)
    _finish(particles, rc, "inject_particles_f32!")


def grid2particle_f32_(Fp: CellArray, F: torch.Tensor, particles: Particles, xi) -> None:
    xi = _check_xi(particles, xi)
    _check_cellarray(particles, Fp, "Fp", torch.float32)
    _check_grid32(F, _vertex_shape(particles), "F")
    _bind_stream(particles)
    rc = _native.load().jp_grid2particle_f32(particles.handle, Fp.data_ptr(), F.data_ptr(), _p3(xi, particles.ndim),
                                             particles.index.data_ptr())
    _finish(particles, rc, "grid2particle_f32!")


def particle2grid_f32_(F: torch.Tensor, Fp: CellArray, particles: Particles, xi) -> None:
    xi = _check_xi(particles, xi)
    _check_cellarray(particles, Fp, "Fp", torch.float32)
    _check_grid32(F, _vertex_shape(particles), "F")
    _bind_stream(particles)
    rc = _native.load().jp_particle2grid_f32(particles.handle, F.data_ptr(), Fp.data_ptr(), _p3(xi, particles.ndim),
                                             particles.index.data_ptr())
    _finish(particles, rc, "particle2grid_f32!")
