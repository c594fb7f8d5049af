"""Adjoint of the FP64 hot path: vector-Jacobian products of one
advection! step (2D), grid2particle! and particle2grid! (2D and 3D), replay of the relocation
done by move_particles!/inject_particles!, and a checkpointed reverse sweep
over a whole run.

The reference has no counterpart (ChainRulesCore is not among its
dependencies, Project.toml:6-16); this module is what a ChainRulesCore
``rrule`` of the Julia API would call, written as ``torch.autograd.Function``
objects on the Python side. Every product runs in the native library
(``jp_*_vjp``); transposes are gathers in a fixed order, so gradients are
reproducible run to run.

Relocation is not differentiated: the move's slot map and the injection's
source ids are recorded as integer data in the forward sweep and replayed.
Dropped particles pass no gradient back; injected particles copy the fields
of a neighbour (the gradient flows back to that neighbour) and their
positions depend on nothing.

Memory stays bounded by recomputation: a run of N steps keeps the particle
state (positions, occupancy, injection RNG counter) every ``k`` steps, and
the reverse sweep re-runs each segment of k steps forward, recording that
segment's positions and slot maps, before stepping back through it.
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass

import torch

from . import _native
from ._native import ArgumentError, P3, check
from .api import _bind_stream, _check_cellarray, _check_grid, _coords, _finish, _vertex_shape
from .api import advection_, inject_particles_, move_particles_
from .integrators import AbstractAdvectionIntegrator
from .particles import CellArray, Particles, grid_field


def _require_2d(p: Particles) -> None:
    if p.ndim != 2:
        raise ArgumentError("the adjoint is built for 2D particles")


def _ptrs(arrays):
    arrays = list(arrays)
    return (ctypes.c_void_p * max(1, len(arrays)))(*[a.data_ptr() for a in arrays])


def _p3(ts):
    ts = list(ts)
    return P3(*[t.data_ptr() for t in ts], *([None] * (3 - len(ts))))


def _like(p: Particles, fill=0.0) -> CellArray:
    return CellArray(torch.full(tuple(p.index.data.shape), float(fill), dtype=torch.float64, device="cuda"), p.ni)


# ------------------------------------------------------------ single products
def particle2grid_with_weights_(F: torch.Tensor, W: torch.Tensor, Fp: CellArray, particles: Particles) -> None:
    """particle2grid! that also writes the weight sum of every vertex to W."""
    _check_cellarray(particles, Fp, "Fp")
    _check_grid(F, _vertex_shape(particles), "F")
    _check_grid(W, _vertex_shape(particles), "W")
    _bind_stream(particles)
    rc = _native.load().jp_particle2grid_with_weights(particles.handle, F.data_ptr(), W.data_ptr(), Fp.data_ptr(),
                                                      _coords(particles), particles.index.data_ptr())
    _finish(particles, rc, "particle2grid!")


def particle2grid_vjp_(gFp: CellArray, gX, gF: torch.Tensor, F: torch.Tensor, W: torch.Tensor, Fp: CellArray,
                       particles: Particles, coords=None, index=None) -> None:
    """Adds dL/dFp to gFp and (if gX is not None) dL/dX to gX, from gF = dL/dF
    of ``particle2grid!(F, Fp, particles)`` (F, W: its outputs). 2D and 3D."""
    coords = coords if coords is not None else particles.coords
    index = index if index is not None else particles.index
    _bind_stream(particles)
    gx = _p3(gX) if gX is not None else None
    rc = _native.load().jp_particle2grid_vjp(particles.handle, F.data_ptr(), W.data_ptr(), Fp.data_ptr(),
                                             _p3(coords), index.data_ptr(), gF.data_ptr(), gFp.data_ptr(), gx)
    _finish(particles, rc, "particle2grid! adjoint")


def grid2particle_vjp_(gF, gX, gFp: CellArray, F, particles: Particles, coords=None, index=None) -> None:
    """Adds dL/dF to gF (if not None) and dL/dX to gX (if not None), from
    gFp = dL/dFp of ``grid2particle!(Fp, F, particles)``. 2D and 3D."""
    coords = coords if coords is not None else particles.coords
    index = index if index is not None else particles.index
    _bind_stream(particles)
    rc = _native.load().jp_grid2particle_vjp(particles.handle, F.data_ptr() if F is not None else None,
                                             gFp.data_ptr(), _p3(coords), index.data_ptr(),
                                             gF.data_ptr() if gF is not None else None,
                                             _p3(gX) if gX is not None else None)
    _finish(particles, rc, "grid2particle! adjoint")


def advection_vjp_(particles: Particles, method: AbstractAdvectionIntegrator, V, dt, coords, index, lam,
                   gV) -> None:
    """One ``advection!(particles, method, V, dt)`` step taken from ``coords``
    (positions before the step): ``lam`` (dL/dX after) becomes dL/dX before,
    and dL/dV is added to ``gV``."""
    _require_2d(particles)
    _bind_stream(particles)
    rc = _native.load().jp_advection_vjp(particles.handle, method.code, float(method.alpha), _p3(V), float(dt),
                                         _p3(coords), index.data_ptr(), _p3(lam), _p3(gV))
    _finish(particles, rc, "advection! adjoint")


def record_buffer(particles: Particles, method: AbstractAdvectionIntegrator) -> torch.Tensor:
    """Device buffer for one recorded advection step (jp_advection_record_bytes)."""
    n = ctypes.c_uint64(0)
    check(_native.load().jp_advection_record_bytes(particles.handle, method.code, ctypes.byref(n)))
    return torch.empty(int(n.value), dtype=torch.uint8, device="cuda")


def advection_record_(particles: Particles, method: AbstractAdvectionIntegrator, V, dt, rec: torch.Tensor) -> None:
    """``advection!`` (the same positions, bit for bit) that also records each
    live particle's velocity samples into ``rec`` for advection_vjp_recorded_."""
    _require_2d(particles)
    _bind_stream(particles)
    rc = _native.load().jp_advection_record(particles.handle, method.code, float(method.alpha), _p3(V), float(dt),
                                            _coords(particles), particles.index.data_ptr(), rec.data_ptr())
    _finish(particles, rc, "advection! (recorded)")


def advection_vjp_recorded_(particles: Particles, method: AbstractAdvectionIntegrator, dt, rec: torch.Tensor, index,
                            lam, gV) -> None:
    """advection_vjp_ of a recorded step: no replay of the stages. ``index``
    is the occupancy before the step."""
    _require_2d(particles)
    _bind_stream(particles)
    rc = _native.load().jp_advection_vjp_recorded(particles.handle, method.code, float(method.alpha), float(dt),
                                                  rec.data_ptr(), index.data_ptr(), _p3(lam), _p3(gV))
    _finish(particles, rc, "advection! adjoint (recorded)")


def move_permutation(particles: Particles) -> torch.Tensor:
    """Slot map of the last move_particles! call: dest[s, c] = linear slot now
    holding the particle that sat in slot (s, c) before it, or -1."""
    dest = torch.empty((particles.max_xcell, particles.index.data.shape[1]), dtype=torch.int32, device="cuda")
    _bind_stream(particles)
    _finish(particles, _native.load().jp_move_permutation(particles.handle, dest.data_ptr()), "move_permutation")
    return dest


def permute_vjp_(particles: Particles, dest: torch.Tensor, post, pre) -> None:
    """pre[k] = post[k] gathered through ``dest`` (0 where it is -1)."""
    post, pre = list(post), list(pre)
    _bind_stream(particles)
    rc = _native.load().jp_permute_vjp(particles.handle, dest.data_ptr(), _ptrs(post), _ptrs(pre), len(post))
    _finish(particles, rc, "move_particles! adjoint")


def slot_ids(particles: Particles, index=None) -> CellArray:
    """ids[s, c] = linear slot for live slots, -1 elsewhere (a particle field
    to pass through inject_particles!)."""
    index = index if index is not None else particles.index
    ids = CellArray(torch.empty(tuple(particles.index.data.shape), dtype=torch.float64, device="cuda"),
                    particles.ni)  # every slot is written
    _bind_stream(particles)
    _finish(particles, _native.load().jp_slot_ids(particles.handle, index.data_ptr(), ids.data_ptr()), "slot_ids")
    return ids


def inject_vjp_(particles: Particles, ids: CellArray, post, pre, copies) -> None:
    """Replay of an inject_particles! call traced with ``ids``. ``copies``:
    True/False for every array, or one flag per array (True for particle
    fields, whose values injected particles copied; False for positions).
    With ``pre`` the same arrays as ``post`` it works in place: the sources
    gather their copies' cotangents, the injected slots keep theirs (a
    following permute_vjp_ reads only the slots that existed before)."""
    _require_2d(particles)
    post, pre = list(post), list(pre)
    flags = [bool(copies)] * len(post) if isinstance(copies, bool) else [bool(c) for c in copies]
    mask = sum(1 << k for k, f in enumerate(flags) if f)
    _bind_stream(particles)
    rc = _native.load().jp_inject_vjp(particles.handle, ids.data_ptr(), _ptrs(post), _ptrs(pre), len(post), mask)
    _finish(particles, rc, "inject_particles! adjoint")


# ------------------------------------------------------------ whole runs
@dataclass
class _State:
    coords: tuple
    index: torch.Tensor
    rng: int


def _save(p: Particles) -> _State:
    return _State(tuple(c.data.clone() for c in p.coords), p.index.data.clone(), p.rng_counter)


def _restore(p: Particles, s: _State) -> None:
    for c, d in zip(p.coords, s.coords):
        c.data.copy_(d)
    p.index.data.copy_(s.index)
    p.rng_counter = s.rng


class _deferred:
    """Queue the library calls without a host synchronisation after each
    (errors surface at the synchronisation on exit)."""

    def __init__(self, p: Particles):
        self.p = p

    def __enter__(self):
        from .api import set_synchronous
        self.prev = self.p._synchronous
        set_synchronous(self.p, False)
        return self

    def __exit__(self, exc_type, exc, tb):
        from .api import set_synchronous, synchronize
        set_synchronous(self.p, self.prev)
        if exc_type is None:
            synchronize(self.p)
        return False


def _step(p: Particles, method, V, dt, fields, inject: bool) -> None:
    advection_(p, method, V, dt)
    move_particles_(p, fields)
    if inject:
        inject_particles_(p, fields)


def misfit(F: torch.Tensor, W: torch.Tensor, target: torch.Tensor):
    """0.5 * sum over vertices holding particles of (F - target)^2, and dL/dF."""
    r = torch.where(W > 0, F - target, torch.zeros_like(F))
    return 0.5 * float((r * r).sum()), r


def _recorded_step(p: Particles, method, V, dt, fields, inject: bool):
    """One step that also records what the reverse sweep needs: the velocity
    samples of its advection, the occupancy before it, the move's slot map and
    the injection's source ids."""
    idx = p.index.data.clone()
    X = record_buffer(p, method)
    advection_record_(p, method, V, dt, X)
    move_particles_(p, fields)
    dest = move_permutation(p)
    ids = None
    if inject:
        ids = slot_ids(p)
        inject_particles_(p, tuple(fields) + (ids,))
    return X, idx, dest, ids


def run_forward(particles: Particles, method, V, dt, nsteps: int, T: CellArray, inject: bool = True,
                checkpoint_every: int = 0, record_last_segment: bool = False, record_segments: int = None):
    """Run nsteps of advection!/move_particles!(/inject_particles!) carrying
    the particle field T, in place; returns the checkpoints taken every
    ``checkpoint_every`` steps (the state before steps 0, k, 2k, ...) and,
    with ``record_segments`` > 0 (``record_last_segment``: 1), the records of
    the steps of that many trailing segments, oldest first (the reverse sweep
    need not run those again)."""
    K = record_segments if record_segments is not None else (1 if record_last_segment else 0)
    cps, recs = [], []
    k = checkpoint_every
    first = first_recorded_step(nsteps, k, K)
    for n in range(nsteps):
        if k and n % k == 0:
            cps.append(_save(particles))
        if n >= first:
            recs.append(_recorded_step(particles, method, V, dt, (T,), inject))
        else:
            _step(particles, method, V, dt, (T,), inject)
    return (cps, recs) if K > 0 else cps


def first_recorded_step(nsteps: int, checkpoint_every: int, segments: int) -> int:
    """The first step whose record is kept when the records of the last
    ``segments`` segments of ``checkpoint_every`` steps are kept (the start of
    the segments-th segment from the end; nsteps when none are kept, 0 without
    checkpoints)."""
    if segments <= 0 or nsteps <= 0:
        return max(0, nsteps)
    if not checkpoint_every:
        return 0
    k = int(checkpoint_every)
    return max(0, ((nsteps - 1) // k - (segments - 1)) * k)


def record_step_bytes(particles: Particles, method) -> int:
    """Device bytes the reverse sweep keeps for one recorded step: the velocity
    samples, the occupancy before the step, the move's slot map and the
    injection's source ids."""
    n = ctypes.c_uint64(0)
    check(_native.load().jp_advection_record_bytes(particles.handle, method.code, ctypes.byref(n)))
    return int(n.value) + particles.index.data.numel() * (1 + 4 + 8)


def kept_segments(particles: Particles, method, nsteps: int, checkpoint_every: int,
                  budget_bytes: int = 64 << 30) -> int:
    """How many trailing segments' records fit in ``budget_bytes`` (and in half
    of the device memory free now): at least 1, at most all segments."""
    k = max(1, int(checkpoint_every))
    nseg = max(1, -(-nsteps // k))
    free = torch.cuda.mem_get_info()[0]
    cap = min(int(budget_bytes), free // 2)
    return int(max(1, min(nseg, cap // max(1, k * record_step_bytes(particles, method)))))


def reverse_sweep(particles: Particles, method, V, dt, nsteps: int, checkpoints, k: int, gX, gT: CellArray,
                  inject: bool = True, last_records=None):
    """Back-propagate dL/dX (gX) and dL/dT (gT) of the state after nsteps to
    the state before step 0, accumulating dL/dV (``last_records``: the records
    run_forward kept of the last steps, if any; the segments they cover are not
    run again). The particles are left in the state before step 0. Returns
    (gV, gX0, gT0)."""
    _require_2d(particles)
    gV = tuple(grid_field(tuple(v.shape), 0.0) for v in V)
    lam = [c.data.clone() for c in gX]
    gT = gT.data.clone()
    tmp_x = [torch.empty_like(lam[0]) for _ in range(2)]
    tmp_t = torch.empty_like(gT)
    nseg = len(checkpoints)
    first = nsteps - len(last_records) if last_records else nsteps  # the first step with a kept record
    for seg in reversed(range(nseg)):
        n0 = seg * k
        n1 = min(n0 + k, nsteps)
        if n0 >= first:
            recs = last_records[n0 - first:n1 - first]
        else:  # recompute the segment, recording positions and slot maps
            _restore(particles, checkpoints[seg])
            recs = [_recorded_step(particles, method, V, dt, (), inject) for _ in range(n0, n1)]
        for X, idx, dest, ids in reversed(recs):
            if ids is not None:  # in place: the sources gather their copies' field cotangents
                inject_vjp_(particles, ids, lam + [gT], lam + [gT], copies=(False, False, True))
            permute_vjp_(particles, dest, lam + [gT], tmp_x + [tmp_t])
            lam, tmp_x = tmp_x, lam
            gT, tmp_t = tmp_t, gT
            advection_vjp_recorded_(particles, method, dt, X, _Idx(idx), lam, gV)
    _restore(particles, checkpoints[0])
    ni = particles.ni
    return gV, tuple(CellArray(l, ni) for l in lam), CellArray(gT, ni)


class _Idx:
    """A recorded index tensor with the data_ptr() the C ABI wrappers use."""

    def __init__(self, t: torch.Tensor):
        self.t = t

    def data_ptr(self) -> int:
        return self.t.data_ptr()


def misfit_gradient(particles: Particles, method, V, dt, nsteps: int, T0: CellArray, target: torch.Tensor,
                    checkpoint_every: int = 10, inject: bool = True, record_segments: int = None):
    """Loss 0.5 ||particle2grid(T after nsteps) - target||^2 and its gradients
    with respect to the velocity grids V and the initial particle field T0.

    The forward run checkpoints the state every ``checkpoint_every`` steps; the
    records of the last ``record_segments`` segments (default: as many as
    kept_segments fits in its memory budget) stay in device memory, and the
    reverse sweep runs every other segment again from its checkpoint.
    The particles and T0 are not modified (the run works on copies). Returns
    (loss, gV, gT0)."""
    _require_2d(particles)
    if not isinstance(method, AbstractAdvectionIntegrator):
        raise ArgumentError("method must be Euler(), RungeKutta2(α) or RungeKutta4()")
    k = max(1, int(checkpoint_every))
    K = kept_segments(particles, method, nsteps, k) if record_segments is None else max(1, int(record_segments))
    start = _save(particles)
    T = CellArray(T0.data.clone(), T0.ni)
    try:
        with _deferred(particles):
            cps, last = run_forward(particles, method, V, dt, nsteps, T, inject, checkpoint_every=k,
                                    record_segments=K)
            if not cps:
                cps = [start]
            F = grid_field(_vertex_shape(particles), 0.0)
            W = grid_field(_vertex_shape(particles), 0.0)
            particle2grid_with_weights_(F, W, T, particles)
            loss, gF = misfit(F, W, target)
            gT = _like(particles)
            gX = tuple(_like(particles) for _ in range(particles.ndim))
            particle2grid_vjp_(gT, gX, _colmajor(gF), F, W, T, particles)
            gV, _, gT0 = reverse_sweep(particles, method, V, dt, nsteps, cps, k, gX, gT, inject,
                                       last_records=last)
    finally:
        _restore(particles, start)
    return loss, gV, gT0


def _colmajor(t: torch.Tensor) -> torch.Tensor:
    out = grid_field(tuple(t.shape), 0.0)
    out.copy_(t)
    return out


def forward_field(particles: Particles, method, V, dt, nsteps: int, T0: CellArray, inject: bool = True):
    """The gridded field F and vertex weights W after nsteps (particles and T0
    untouched)."""
    start = _save(particles)
    T = CellArray(T0.data.clone(), T0.ni)
    try:
        with _deferred(particles):
            run_forward(particles, method, V, dt, nsteps, T, inject)
            F = grid_field(_vertex_shape(particles), 0.0)
            W = grid_field(_vertex_shape(particles), 0.0)
            particle2grid_with_weights_(F, W, T, particles)
    finally:
        _restore(particles, start)
    return F, W


def misfit_value(particles: Particles, method, V, dt, nsteps: int, T0: CellArray, target: torch.Tensor,
                 inject: bool = True) -> float:
    """The loss of misfit_gradient alone (particles and T0 untouched)."""
    F, W = forward_field(particles, method, V, dt, nsteps, T0, inject)
    return misfit(F, W, target)[0]


def misfit_difference(Fp, Wp, Fm, Wm, target) -> float:
    """L(+) - L(-) of two runs, formed vertex by vertex before the sum (a
    central finite difference then keeps its round-off to the vertices the
    perturbation reached)."""
    rp = torch.where(Wp > 0, Fp - target, torch.zeros_like(Fp))
    rm = torch.where(Wm > 0, Fm - target, torch.zeros_like(Fm))
    return 0.5 * float(((rp - rm) * (rp + rm)).sum())


class PICMisfit(torch.autograd.Function):
    """loss = PICMisfit.apply(Vx, Vy, T0data, particles, method, dt, nsteps,
    target, checkpoint_every, inject): the misfit of misfit_gradient as an
    autograd node; backward returns dL/dVx, dL/dVy, dL/dT0 (the Julia
    counterpart is an rrule of the same run)."""

    @staticmethod
    def forward(ctx, Vx, Vy, T0data, particles, method, dt, nsteps, target, checkpoint_every=10, inject=True):
        V = (Vx.detach(), Vy.detach())
        T0 = CellArray(T0data.detach(), particles.ni)
        k = max(1, int(checkpoint_every))
        start = _save(particles)
        T = CellArray(T0.data.clone(), T0.ni)
        try:
            cps = run_forward(particles, method, V, dt, nsteps, T, inject, checkpoint_every=k) or [start]
            F = grid_field(_vertex_shape(particles), 0.0)
            W = grid_field(_vertex_shape(particles), 0.0)
            particle2grid_with_weights_(F, W, T, particles)
            loss, gF = misfit(F, W, target)
            ctx.saved = (particles, method, V, dt, nsteps, cps, k, inject, F, W, T, _colmajor(gF),
                         _save(particles))
        finally:
            _restore(particles, start)
        return torch.tensor(loss, dtype=torch.float64, device=Vx.device)

    @staticmethod
    def backward(ctx, gl):
        particles, method, V, dt, nsteps, cps, k, inject, F, W, T, gF, final = ctx.saved
        start = _save(particles)
        try:
            _restore(particles, final)
            gT = _like(particles)
            gX = tuple(_like(particles) for _ in range(particles.ndim))
            particle2grid_vjp_(gT, gX, gF, F, W, T, particles)
            gV, _, gT0 = reverse_sweep(particles, method, V, dt, nsteps, cps, k, gX, gT, inject)
        finally:
            _restore(particles, start)
        s = gl.to(torch.float64)
        return (gV[0] * s, gV[1] * s, gT0.data * s) + (None,) * 7


class Grid2Particle(torch.autograd.Function):
    """Fp = Grid2Particle.apply(F, particles): grid2particle! as an autograd
    node (positions fixed); backward is the transpose gather."""

    @staticmethod
    def forward(ctx, F, particles):
        from .api import grid2particle_
        Fp = _like(particles)
        Fc = _colmajor(F.detach())
        grid2particle_(Fp, Fc, particles)
        ctx.particles = particles
        ctx.shape = tuple(F.shape)
        return Fp.data

    @staticmethod
    def backward(ctx, gFp):
        p = ctx.particles
        gF = grid_field(ctx.shape, 0.0)
        grid2particle_vjp_(gF, None, CellArray(gFp.contiguous().to(torch.float64), p.ni), None, p)
        return gF, None


class Particle2Grid(torch.autograd.Function):
    """F = Particle2Grid.apply(Fp, particles): particle2grid! as an autograd
    node (positions fixed)."""

    @staticmethod
    def forward(ctx, Fp, particles):
        F = grid_field(_vertex_shape(particles), 0.0)
        W = grid_field(_vertex_shape(particles), 0.0)
        T = CellArray(Fp.detach().contiguous(), particles.ni)
        particle2grid_with_weights_(F, W, T, particles)
        ctx.saved = (particles, F, W, T)
        return F

    @staticmethod
    def backward(ctx, gF):
        p, F, W, T = ctx.saved
        gFp = _like(p)
        particle2grid_vjp_(gFp, None, _colmajor(gF), F, W, T, p)
        return gFp.data, None


class AdvectionStep(torch.autograd.Function):
    """(X', Y') = AdvectionStep.apply(Vx, Vy, X, Y, particles, method, dt):
    one advection! step out of place (X, Y: coordinate data of the
    particles' layout), differentiable in the velocities and the positions."""

    @staticmethod
    def forward(ctx, Vx, Vy, X, Y, particles, method, dt):
        _require_2d(particles)
        saved = tuple(c.data.clone() for c in particles.coords)
        try:
            particles.coords[0].data.copy_(X.detach())
            particles.coords[1].data.copy_(Y.detach())
            V = (_colmajor(Vx.detach()), _colmajor(Vy.detach()))
            advection_(particles, method, V, dt)
            out = tuple(c.data.clone() for c in particles.coords)
        finally:
            for c, d in zip(particles.coords, saved):
                c.data.copy_(d)
        ctx.saved = (particles, method, V, dt, X.detach().clone(), Y.detach().clone(),
                     particles.index.data.clone())
        return out

    @staticmethod
    def backward(ctx, gX, gY):
        p, method, V, dt, X, Y, idx = ctx.saved
        lam = [gX.contiguous().clone(), gY.contiguous().clone()]
        gV = tuple(grid_field(tuple(v.shape), 0.0) for v in V)
        advection_vjp_(p, method, V, dt, (X, Y), _Idx(idx), lam, gV)
        return gV[0], gV[1], lam[0], lam[1], None, None, None


# ---------------------------------------------- split-precision (FP32) form
def particle2grid_f32_with_weights_(F: torch.Tensor, W: torch.Tensor, Fp: CellArray, particles: Particles,
                                    xi) -> None:
    """particle2grid! of the FP32 form that also writes the FP64 weight sums W."""
    from .split import _check_xi, _p3 as _p3n
    xi = _check_xi(particles, xi)
    _bind_stream(particles)
    rc = _native.load().jp_particle2grid_f32_with_weights(particles.handle, F.data_ptr(), W.data_ptr(),
                                                          Fp.data_ptr(), _p3n(xi, particles.ndim),
                                                          particles.index.data_ptr())
    _finish(particles, rc, "particle2grid_f32!")


def particle2grid_vjp_f32_(gFp: CellArray, gxi, gF: torch.Tensor, F: torch.Tensor, W: torch.Tensor, Fp: CellArray,
                           particles: Particles, xi, index=None) -> None:
    """FP32 form: adds dL/dFp to gFp and (if gxi is not None) dL/d(offset) to gxi."""
    _require_2d(particles)
    index = index if index is not None else particles.index
    _bind_stream(particles)
    rc = _native.load().jp_particle2grid_vjp_f32(particles.handle, F.data_ptr(), W.data_ptr(), Fp.data_ptr(),
                                                 _p3(xi), index.data_ptr(), gF.data_ptr(), gFp.data_ptr(),
                                                 _p3(gxi) if gxi is not None else None)
    _finish(particles, rc, "particle2grid_f32! adjoint")


def advection_vjp_f32_(particles: Particles, method: AbstractAdvectionIntegrator, V, dt, xi, index, lam,
                       gV) -> None:
    """FP32 form: one advection_f32! step taken from offsets ``xi``; ``lam``
    (dL/d(offset) after, FP64) becomes dL/d(offset) before; dL/dV is added
    to ``gV`` (FP64)."""
    _require_2d(particles)
    _bind_stream(particles)
    rc = _native.load().jp_advection_vjp_f32(particles.handle, method.code, float(method.alpha), _p3(V), float(dt),
                                             _p3(xi), index.data_ptr(), _p3(lam), _p3(gV))
    _finish(particles, rc, "advection_f32! adjoint")


def slot_ids_i32(particles: Particles) -> torch.Tensor:
    """int32 ids (slot index or -1) to carry through inject_particles_f32! as
    an FP32 field (``ids.view(torch.float32)``; copied bit for bit)."""
    ids = torch.empty(tuple(particles.index.data.shape), dtype=torch.int32, device="cuda")
    _bind_stream(particles)
    _finish(particles, _native.load().jp_slot_ids_i32(particles.handle, particles.index.data_ptr(),
                                                      ids.data_ptr()), "slot_ids_i32")
    return ids


def inject_vjp_i32_(particles: Particles, ids: torch.Tensor, post, pre, copies) -> None:
    _require_2d(particles)
    post, pre = list(post), list(pre)
    flags = [bool(copies)] * len(post) if isinstance(copies, bool) else [bool(c) for c in copies]
    mask = sum(1 << k for k, f in enumerate(flags) if f)
    _bind_stream(particles)
    rc = _native.load().jp_inject_vjp_i32(particles.handle, ids.data_ptr(), _ptrs(post), _ptrs(pre), len(post),
                                          mask)
    _finish(particles, rc, "inject_particles_f32! adjoint")


@dataclass
class _StateF32:
    xi: tuple
    index: torch.Tensor
    rng: int


def _save_f32(p: Particles, xi) -> _StateF32:
    return _StateF32(tuple(x.data.clone() for x in xi), p.index.data.clone(), p.rng_counter)


def _restore_f32(p: Particles, xi, s: _StateF32) -> None:
    for x, d in zip(xi, s.xi):
        x.data.copy_(d)
    p.index.data.copy_(s.index)
    p.rng_counter = s.rng


def _recorded_step_f32(p: Particles, xi, method, V, dt, fields, inject: bool):
    from .split import advection_f32_, inject_particles_f32_, move_particles_f32_
    X = tuple(x.data.clone() for x in xi)
    idx = p.index.data.clone()
    advection_f32_(p, xi, method, V, dt)
    move_particles_f32_(p, xi, fields)
    dest = move_permutation(p)
    ids = None
    if inject:
        ids = slot_ids_i32(p)
        inject_particles_f32_(p, xi, tuple(fields) + (CellArray(ids.view(torch.float32), p.ni),))
    return X, idx, dest, ids


def kept_segments_f32(particles: Particles, nsteps: int, checkpoint_every: int, budget_bytes: int = 64 << 30) -> int:
    """kept_segments for misfit_gradient_f32, whose recorded step keeps the
    FP32 offsets, the occupancy, the slot map and the int32 source ids."""
    k = max(1, int(checkpoint_every))
    per_step = particles.index.data.numel() * (2 * 4 + 1 + 4 + 4)
    nseg = max(1, -(-nsteps // k))
    cap = min(int(budget_bytes), torch.cuda.mem_get_info()[0] // 2)
    return int(max(1, min(nseg, cap // max(1, k * per_step))))


def misfit_gradient_f32(particles: Particles, xi, method, V, dt, nsteps: int, T0: CellArray, target: torch.Tensor,
                        checkpoint_every: int = 10, inject: bool = True, record_segments: int = None):
    """The FP32 (split-precision) variant of misfit_gradient: the run uses the
    FP32 forward path (offsets ``xi``, FP32 velocities V and particle field
    T0, FP32 target); cotangents and the returned gradients are FP64. Records
    of the last ``record_segments`` segments are kept as in misfit_gradient.
    The particles, xi and T0 are not modified. Returns (loss, gV, gT0)."""
    from .split import advection_f32_, grid_field_f32, inject_particles_f32_, move_particles_f32_
    _require_2d(particles)
    k = max(1, int(checkpoint_every))
    K = kept_segments_f32(particles, nsteps, k) if record_segments is None else max(1, int(record_segments))
    start = _save_f32(particles, xi)
    T = CellArray(T0.data.clone(), T0.ni)
    shape = _vertex_shape(particles)
    try:
        with _deferred(particles):
            cps, last = [], []
            first = first_recorded_step(nsteps, k, K)
            for n in range(nsteps):
                if n % k == 0:
                    cps.append(_save_f32(particles, xi))
                if n >= first:
                    last.append(_recorded_step_f32(particles, xi, method, V, dt, (T,), inject))
                else:
                    advection_f32_(particles, xi, method, V, dt)
                    move_particles_f32_(particles, xi, (T,))
                    if inject:
                        inject_particles_f32_(particles, xi, (T,))
            if not cps:
                cps = [start]
            F = grid_field_f32(shape)
            W = grid_field(shape, 0.0)
            particle2grid_f32_with_weights_(F, W, T, particles, xi)
            F64 = F.double()
            loss, gF = misfit(F64, W, target.double())
            gT = _like(particles)
            gX = [_like(particles) for _ in range(2)]
            particle2grid_vjp_f32_(gT, gX, _colmajor(gF), F, W, T, particles, xi)
            gV = tuple(grid_field(tuple(v.shape), 0.0) for v in V)
            lam = [c.data.clone() for c in gX]
            gTd = gT.data.clone()
            tmp_x = [torch.empty_like(lam[0]) for _ in range(2)]
            tmp_t = torch.empty_like(gTd)
            nseg = len(cps)
            for seg in reversed(range(nseg)):
                n0 = seg * k
                n1 = min(n0 + k, nsteps)
                if last and n0 >= first:
                    recs = last[n0 - first:n1 - first]
                else:
                    _restore_f32(particles, xi, cps[seg])
                    recs = [_recorded_step_f32(particles, xi, method, V, dt, (), inject) for _ in range(n0, n1)]
                for X, idx, dest, ids in reversed(recs):
                    if ids is not None:  # in place, as in misfit_gradient's sweep
                        inject_vjp_i32_(particles, ids, lam + [gTd], lam + [gTd], copies=(False, False, True))
                    permute_vjp_(particles, dest, lam + [gTd], tmp_x + [tmp_t])
                    lam, tmp_x = tmp_x, lam
                    gTd, tmp_t = tmp_t, gTd
                    advection_vjp_f32_(particles, method, V, dt, X, _Idx(idx), lam, gV)
    finally:
        _restore_f32(particles, xi, start)
    return loss, gV, CellArray(gTd, particles.ni)


__all__ = ["particle2grid_with_weights_", "particle2grid_vjp_", "grid2particle_vjp_", "advection_vjp_",
           "move_permutation", "permute_vjp_", "slot_ids", "inject_vjp_", "run_forward", "reverse_sweep",
           "record_step_bytes", "kept_segments", "kept_segments_f32", "first_recorded_step",
           "misfit", "misfit_gradient", "misfit_value", "forward_field", "misfit_difference", "PICMisfit", "Grid2Particle", "Particle2Grid",
           "AdvectionStep", "particle2grid_f32_with_weights_", "particle2grid_vjp_f32_", "advection_vjp_f32_",
           "slot_ids_i32", "inject_vjp_i32_", "misfit_gradient_f32"]
