"""The hot-path functions of JustPIC.jl, one native call each.

Julia's in-place ``f!`` becomes ``f_`` here (PyTorch's in-place convention):

===========================  ==============================================================
Python                       reference
===========================  ==============================================================
``advection_``               ``advection!`` (src/Particles/Advection/advection.jl:21)
``advection_LinP_``          ``advection_LinP!`` (src/Particles/Advection/advection_LinP.jl:13)
``advection_MQS_``           ``advection_MQS!`` (src/Particles/Advection/advection_MQS.jl:16)
``move_particles_``          ``move_particles!`` (src/Particles/move_safe.jl:21)
``inject_particles_``        ``inject_particles!`` (src/Particles/injection.jl:19)
``inject_particles_phase_``  ``inject_particles_phase!`` (src/Particles/injection.jl:133)
``grid2particle_``           ``grid2particle!`` (src/Interpolations/grid_to_particle.jl:26)
``particle2grid_``           ``particle2grid!`` (src/Interpolations/particle_to_grid.jl:23)
===========================  ==============================================================

Calls are synchronous (like the reference's ``launch!``) unless
``set_synchronous(particles, False)`` was called; kernels run on PyTorch's
current CUDA stream.
"""
from __future__ import annotations

import ctypes
import warnings

import numpy as np
import torch

from . import _native
from ._native import JP_MAX_ARGS, JP_WARN_FAR_MOVE, JP_WARN_NO_NEIGHBOUR, ArgumentError, P3, check
from .integrators import AbstractAdvectionIntegrator
from .particles import CellArray, Particles


def _bind_stream(p: Particles) -> None:
    s = torch.cuda.current_stream()
    _native.load().jp_set_stream(p.handle, s.cuda_stream)


def _warn_bits(bits: int) -> None:
    if bits & JP_WARN_FAR_MOVE:
        warnings.warn("move_particles!: a particle moved more than one cell in one step and was dropped "
                      "(the reference's colour passes race in this case)", RuntimeWarning, stacklevel=3)
    if bits & JP_WARN_NO_NEIGHBOUR:
        warnings.warn("inject_particles!: an injected particle had no live neighbour; its fields were left "
                      "unchanged", RuntimeWarning, stacklevel=3)


def _finish(p: Particles, rc: int, what: str) -> None:
    check(rc, what)
    if p._synchronous:
        bits = ctypes.c_uint32(0)
        check(_native.load().jp_get_warnings(p.handle, ctypes.byref(bits), 1))
        if bits.value:
            _warn_bits(bits.value)


Particles._synchronous = True


def set_synchronous(p: Particles, synchronous: bool) -> None:
    """Toggle the per-call synchronisation (default on, as ``launch!``)."""
    check(_native.load().jp_set_synchronous(p.handle, 1 if synchronous else 0))
    p._synchronous = bool(synchronous)


def synchronize(p: Particles) -> None:
    """Wait for queued work and raise any device-side error."""
    check(_native.load().jp_synchronize(p.handle))
    bits = ctypes.c_uint32(0)
    check(_native.load().jp_get_warnings(p.handle, ctypes.byref(bits), 1))
    if bits.value:
        _warn_bits(bits.value)


def move_counts(p: Particles, clear: bool = False) -> dict:
    """Particles removed by move_particles! since the last clearing call: those
    that left the domain, those that moved more than one cell in a step
    (dropped), and those whose new cell had no free slot at or after the
    walk's starting point (dropped, as in src/Particles/move_safe.jl:113-114).
    Waits for the container's stream."""
    out = (ctypes.c_uint64 * 3)()
    check(_native.load().jp_get_move_counts(p.handle, out, 1 if clear else 0), "move_counts")
    return {"left_domain": int(out[0]), "moved_too_far": int(out[1]), "no_free_slot": int(out[2])}


def _coords(p: Particles) -> P3:
    return P3(*[c.data_ptr() for c in p.coords], *([None] * (3 - p.ndim)))


def _check_cellarray(p: Particles, A: CellArray, what: str, dtype=torch.float64) -> None:
    if not isinstance(A, CellArray):
        raise ArgumentError(f"{what} must be a CellArray")
    if A.data.dtype != dtype or not A.data.is_cuda:
        raise ArgumentError(f"{what} must hold {dtype} CUDA data")
    if A.ni != p.ni or A.ncap != p.max_xcell:
        raise ArgumentError(f"{what} does not have the particle layout {p.max_xcell} x {p.ni}")


def _check_grid(t: torch.Tensor, shape, what: str) -> None:
    if not isinstance(t, torch.Tensor) or not t.is_cuda or t.dtype != torch.float64:
        raise ArgumentError(f"{what} must be a float64 CUDA tensor")
    if tuple(t.shape) != tuple(shape):
        raise ArgumentError(f"{what} has shape {tuple(t.shape)}, expected {tuple(shape)}")
    expected = tuple(int(np.prod(shape[:d])) for d in range(len(shape)))
    if tuple(t.stride()) != expected:
        raise ArgumentError(f"{what} must be column-major (Julia layout); use TA(backend)(array)")


def _args(p: Particles, args):
    args = tuple(args) if args is not None else ()
    if len(args) > JP_MAX_ARGS:
        raise ArgumentError(f"at most {JP_MAX_ARGS} particle fields are supported")
    for k, a in enumerate(args):
        _check_cellarray(p, a, f"args[{k}]")
    arr = (ctypes.c_void_p * max(1, len(args)))(*[a.data_ptr() for a in args])
    return arr, len(args)


def _advect(particles: Particles, method, V, dt, entry: str, what: str) -> None:
    if not isinstance(method, AbstractAdvectionIntegrator):
        raise ArgumentError("method must be Euler(), RungeKutta2(α) or RungeKutta4()")
    N = particles.ndim
    V = tuple(V)
    if len(V) != N:
        raise ArgumentError(f"V must have {N} components")
    for c in range(N):
        _check_grid(V[c], tuple(len(x) for x in particles.xi_vel[c]), f"V[{c}]")
    _bind_stream(particles)
    vp = P3(*[v.data_ptr() for v in V], *([None] * (3 - N)))
    rc = getattr(_native.load(), entry)(particles.handle, method.code, float(method.alpha), vp, float(dt),
                                        _coords(particles), particles.index.data_ptr())
    _finish(particles, rc, what)


def advection_(particles: Particles, method: AbstractAdvectionIntegrator, V, dt) -> None:
    """``advection!(particles, method, V, dt)``: advect every live particle
    through the staggered velocity components ``V`` (one per axis)."""
    _advect(particles, method, V, dt, "jp_advection", "advection!")


def advection_LinP_(particles: Particles, method: AbstractAdvectionIntegrator, V, dt) -> None:
    """``advection_LinP!(particles, method, V, dt)``
    (src/Particles/Advection/advection_LinP.jl:13): as ``advection_`` with
    the LinP velocity interpolation."""
    _advect(particles, method, V, dt, "jp_advection_linp", "advection_LinP!")


def advection_MQS_(particles: Particles, method: AbstractAdvectionIntegrator, V, dt) -> None:
    """``advection_MQS!(particles, method, V, dt)``
    (src/Particles/Advection/advection_MQS.jl:16): as ``advection_`` with the
    MQS velocity interpolation."""
    _advect(particles, method, V, dt, "jp_advection_mqs", "advection_MQS!")


def move_particles_(particles: Particles, args=()) -> None:
    """``move_particles!(particles, args)``: relocate particles that left their
    cell, carrying the per-particle fields ``args``."""
    arr, n = _args(particles, args)
    _bind_stream(particles)
    rc = _native.load().jp_move_particles(particles.handle, _coords(particles), particles.index.data_ptr(), arr, n)
    _finish(particles, rc, "move_particles!")


def inject_particles_(particles: Particles, args=()) -> None:
    """``inject_particles!(particles, args)``: reseed under-populated cells."""
    arr, n = _args(particles, args)
    _bind_stream(particles)
    rc = _native.load().jp_inject_particles(particles.handle, _coords(particles), particles.index.data_ptr(),
                                            arr, n)
    _finish(particles, rc, "inject_particles!")


def inject_particles_phase_(particles: Particles, particles_phases: CellArray, args=(), fields=()) -> None:
    """``inject_particles_phase!(particles, particles_phases, args, fields, grid)``
    (src/Particles/injection.jl:133): reseed every under-populated quadrant;
    a new particle takes the phase of its nearest neighbour and ``args[k]``
    the clamped interpolation of grid field ``fields[k]`` (cell-centred when
    its shape is the cells', else on the vertices). The grid is the one the
    particles were made on."""
    _check_cellarray(particles, particles_phases, "particles_phases")
    arr, n = _args(particles, args)
    fields = tuple(fields) if fields is not None else ()
    if len(fields) != n:
        raise ArgumentError("args and fields must have the same length")
    centred = []
    for k, f in enumerate(fields):
        c = isinstance(f, torch.Tensor) and tuple(f.shape) == tuple(particles.ni)
        _check_grid(f, tuple(particles.ni) if c else _vertex_shape(particles), f"fields[{k}]")
        if c and min(particles.ni) < 2:
            raise ArgumentError(f"fields[{k}]: a cell-centred field needs at least 2 cells per axis")
        centred.append(1 if c else 0)
    fp = (ctypes.c_void_p * max(1, n))(*[f.data_ptr() for f in fields])
    cf = (ctypes.c_int32 * max(1, n))(*centred)
    _bind_stream(particles)
    rc = _native.load().jp_inject_particles_phase(particles.handle, _coords(particles), particles.index.data_ptr(),
                                                  particles_phases.data_ptr(), arr, fp, cf, n)
    _finish(particles, rc, "inject_particles_phase!")


def _vertex_shape(p: Particles):
    return tuple(n + 1 for n in p.ni)


def _field_lists(a, b, what):
    a, b = tuple(a), tuple(b)
    if len(a) != len(b) or not 1 <= len(a) <= _native.JP_MAX_ARGS:
        raise ArgumentError(f"{what}: the two tuples need the same length, 1 to {_native.JP_MAX_ARGS} fields")
    return a, b


def _ptr_array(xs):
    return (ctypes.c_void_p * len(xs))(*[x.data_ptr() for x in xs])


def grid2particle_(Fp, F, particles: Particles) -> None:
    """``grid2particle!(Fp, F, particles)``: vertex field -> particles. With
    tuples ``Fp`` and ``F`` the tuple form (grid_to_particle.jl:84-103): all
    fields in one call, live particles with a NaN coordinate skipped."""
    if isinstance(Fp, (tuple, list)):
        Fps, Fs = _field_lists(Fp, F, "grid2particle!")
        for k, (fp, f) in enumerate(zip(Fps, Fs)):
            _check_cellarray(particles, fp, f"Fp[{k}]")
            _check_grid(f, _vertex_shape(particles), f"F[{k}]")
        _bind_stream(particles)
        rc = _native.load().jp_grid2particle_n(particles.handle, _ptr_array(Fps), _ptr_array(Fs), len(Fs),
                                               _coords(particles), particles.index.data_ptr())
        _finish(particles, rc, "grid2particle!")
        return
    _check_cellarray(particles, Fp, "Fp")
    _check_grid(F, _vertex_shape(particles), "F")
    _bind_stream(particles)
    rc = _native.load().jp_grid2particle(particles.handle, Fp.data_ptr(), F.data_ptr(), _coords(particles),
                                         particles.index.data_ptr())
    _finish(particles, rc, "grid2particle!")


def particle2grid_(F, Fp, particles: Particles) -> None:
    """``particle2grid!(F, Fp, particles)``: particles -> vertex field. With
    tuples ``F`` and ``Fp`` the tuple form (particle_to_grid.jl:70-109,
    153-199): the weights are formed once for all fields."""
    if isinstance(F, (tuple, list)):
        Fs, Fps = _field_lists(F, Fp, "particle2grid!")
        for k, (f, fp) in enumerate(zip(Fs, Fps)):
            _check_cellarray(particles, fp, f"Fp[{k}]")
            _check_grid(f, _vertex_shape(particles), f"F[{k}]")
        _bind_stream(particles)
        rc = _native.load().jp_particle2grid_n(particles.handle, _ptr_array(Fs), _ptr_array(Fps), len(Fs),
                                               _coords(particles), particles.index.data_ptr())
        _finish(particles, rc, "particle2grid!")
        return
    _check_cellarray(particles, Fp, "Fp")
    _check_grid(F, _vertex_shape(particles), "F")
    _bind_stream(particles)
    rc = _native.load().jp_particle2grid(particles.handle, F.data_ptr(), Fp.data_ptr(), _coords(particles),
                                         particles.index.data_ptr())
    _finish(particles, rc, "particle2grid!")


# ---- transfers beside the hot path ------------------------------------------
def _centre_shape(p: Particles):
    return tuple(p.ni)


def grid2particle_flip_(Fp: CellArray, xvi, F: torch.Tensor, F0: torch.Tensor, particles: Particles,
                        alpha: float = 0.0) -> None:
    """``grid2particle_flip!(Fp, xvi, F, F0, particles; α)``
    (src/Interpolations/grid_to_particle.jl:125): PIC/FLIP blend of the vertex
    fields F (new) and F0 (old) into Fp. ``xvi`` must be the particles'
    vertex grid (or None for it)."""
    _check_cellarray(particles, Fp, "Fp")
    _check_grid(F, _vertex_shape(particles), "F")
    _check_grid(F0, _vertex_shape(particles), "F0")
    if xvi is not None:
        for d in range(particles.ndim):
            if not np.array_equal(np.asarray(xvi[d], dtype=np.float64), np.asarray(particles.xvi[d])):
                raise ArgumentError("grid2particle_flip!: xvi must be the particles' vertex grid")
    _bind_stream(particles)
    rc = _native.load().jp_grid2particle_flip(particles.handle, Fp.data_ptr(), F.data_ptr(), F0.data_ptr(),
                                              float(alpha), _coords(particles), particles.index.data_ptr())
    _finish(particles, rc, "grid2particle_flip!")


def centroid2particle_(Fp: CellArray, F: torch.Tensor, particles: Particles) -> None:
    """``centroid2particle!(Fp, F, particles)`` (src/Interpolations/centroid_to_particle.jl:13):
    cell-centred field F (one value per cell) to the particles."""
    _check_cellarray(particles, Fp, "Fp")
    _check_grid(F, _centre_shape(particles), "F")
    _bind_stream(particles)
    rc = _native.load().jp_centroid2particle(particles.handle, Fp.data_ptr(), F.data_ptr(), _coords(particles))
    _finish(particles, rc, "centroid2particle!")


def particle2centroid_(F: torch.Tensor, Fp: CellArray, particles: Particles) -> None:
    """``particle2centroid!(F, Fp, particles)`` (src/Interpolations/particle_to_grid_centroid.jl:10):
    particles to the cell centres."""
    _check_cellarray(particles, Fp, "Fp")
    _check_grid(F, _centre_shape(particles), "F")
    _bind_stream(particles)
    rc = _native.load().jp_particle2centroid(particles.handle, F.data_ptr(), Fp.data_ptr(), _coords(particles))
    _finish(particles, rc, "particle2centroid!")


# ---- phase ratios -------------------------------------------------------------
class PhaseRatios:
    """``PhaseRatios`` (src/PhaseRatios/PhaseRatios.jl:12-33, constructors.jl:18-57):
    ``center``, ``vertex``, ``Vx``, ``Vy`` (, ``Vz`` and the 3D edge
    midpoints ``yz``, ``xz``, ``xy``) are CUDA float64 tensors of shape
    (nphases, nodes) in the CellArray layout (phase k of node n at
    n + nodes * k), node index column-major over the location's grid."""

    MIDPOINTS = (("xy", (1, 1, 0)), ("yz", (0, 1, 1)), ("xz", (1, 0, 1)))

    def __init__(self, nphases: int, ni):
        ni = tuple(int(n) for n in ni)
        self.nphases = int(nphases)
        self.ni = ni

        def alloc(shape):
            return torch.zeros((self.nphases, int(np.prod(shape))), dtype=torch.float64, device="cuda")

        self.center = alloc(ni)
        self.vertex = alloc(tuple(n + 1 for n in ni))
        self.faces = tuple(alloc(tuple(n + (1 if e == d else 0) for e, n in enumerate(ni))) for d in range(len(ni)))
        self.Vx, self.Vy = self.faces[0], self.faces[1]
        self.Vz = self.faces[2] if len(ni) == 3 else None
        self.midpoints = None
        if len(ni) == 3:
            self.midpoints = tuple(alloc(tuple(n + o for n, o in zip(ni, off))) for _, off in self.MIDPOINTS)
            self.xy, self.yz, self.xz = self.midpoints


def update_phase_ratios_(phase_ratios: PhaseRatios, particles: Particles, phases: CellArray) -> None:
    """``update_phase_ratios!(phase_ratios, particles, phases)`` (src/PhaseRatios/utils.jl:3-40):
    the fraction of each phase (ids 1..nphases in the per-slot field
    ``phases``) at cell centres, vertices, faces and, in 3D, edge midpoints."""
    _check_cellarray(particles, phases, "phases")
    if phase_ratios.ni != particles.ni:
        raise ArgumentError("phase_ratios does not match the particles' grid")
    _bind_stream(particles)
    faces = P3(*[f.data_ptr() for f in phase_ratios.faces], *([None] * (3 - particles.ndim)))
    rc = _native.load().jp_phase_ratios(particles.handle, phase_ratios.nphases, phases.data_ptr(),
                                        _coords(particles), phase_ratios.center.data_ptr(),
                                        phase_ratios.vertex.data_ptr(), faces)
    if rc == 0 and particles.ndim == 3:
        mids = P3(*[m.data_ptr() for m in phase_ratios.midpoints])
        rc = _native.load().jp_phase_ratios_midpoints(particles.handle, phase_ratios.nphases, phases.data_ptr(),
                                                      _coords(particles), mids)
    _finish(particles, rc, "update_phase_ratios!")

