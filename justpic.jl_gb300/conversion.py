"""Host <-> device conversion and checkpoints.

``Array(x)`` copies a device container to the host in the reference's CPU
layout (src/CellArrays/conversion.jl:19-100): a per-slot array of the CPU
CellArray (blocklength 1) keeps the slots of a cell together, element
``(slot s, cell c)`` at ``s + max_xcell * c``; here that is a C-ordered numpy
array of shape ``(ncells, ncap)`` (the same bytes as Julia's
``(1, ncap, ncells)`` data array). ``TA(backend)(Float64, host)`` goes back
(ext/JustPICCUDAExt.jl:51-191). The permute runs on the GPU
(``jp_cellarray_permute``) around one device<->host copy per array.

``checkpointing_particles`` (src/IO/JLD2.jl:1-129) writes the same entries as
the reference's checkpoint (particles, phases, phase_ratios, chain, time,
timestep, particle_args, extra keywords) into an ``.npz`` archive, written
next to the destination and renamed into place; ``load_checkpoint`` reads it
back into host containers.
"""
from __future__ import annotations

import dataclasses
import json
import os
import tempfile

import numpy as np
import torch

from . import _native
from ._native import ArgumentError, check
from .particles import CUDABackend, CellArray, LinRange, Particles, _check_backend

_DTYPES = {"Float64": np.float64, "Float32": np.float32, np.float64: np.float64, np.float32: np.float32,
           float: np.float64, torch.float64: np.float64, torch.float32: np.float32}


def _np_dtype(T):
    if T is None:
        return None
    try:
        return _DTYPES[T]
    except (KeyError, TypeError):
        raise ArgumentError(f"unsupported element type {T!r}: use Float64 or Float32") from None


@dataclasses.dataclass
class HostCellArray:
    """A CPU CellArray: ``data[c, s]`` is component ``s`` of node ``c`` (the
    node index column-major over ``ni``)."""
    data: np.ndarray
    ni: tuple

    @property
    def ncap(self) -> int:
        return self.data.shape[1]


@dataclasses.dataclass
class HostParticles:
    """``Array(particles)``: the container's arrays on the host."""
    coords: tuple
    index: HostCellArray
    nxcell: int
    max_xcell: int
    min_xcell: int
    np: int
    xi_vel: tuple
    uniform: bool
    seed: int
    rng_counter: int

    @property
    def ni(self):
        return self.index.ni

    @property
    def ndim(self) -> int:
        return len(self.coords)


@dataclasses.dataclass
class HostPhaseRatios:
    """``Array(phase_ratios)``: one HostCellArray of nphases per location."""
    nphases: int
    ni: tuple
    fields: dict


def _permute(p: Particles, src: torch.Tensor, dst: torch.Tensor, nnodes: int, ncomp: int, to_cpu: bool) -> None:
    from .api import _bind_stream
    _bind_stream(p)
    check(_native.load().jp_cellarray_permute(p.handle, src.data_ptr(), dst.data_ptr(), int(nnodes), int(ncomp),
                                              src.element_size(), 1 if to_cpu else 0), "CellArray conversion")


def _to_host(p: Particles, t: torch.Tensor, nnodes: int, T=None) -> np.ndarray:
    """GPU-form tensor (ncomp, nnodes) -> host array (nnodes, ncomp) in CPU form."""
    ncomp = t.shape[0]
    out = torch.empty((nnodes, ncomp), dtype=t.dtype, device=t.device)
    _permute(p, t.contiguous(), out, nnodes, ncomp, True)
    a = out.cpu().numpy()
    dt = _np_dtype(T)
    return a.astype(dt) if dt is not None and a.dtype != np.uint8 else a


def _to_device(p: Particles, a: np.ndarray, dtype: torch.dtype) -> torch.Tensor:
    """Host array (nnodes, ncomp) in CPU form -> GPU-form tensor (ncomp, nnodes)."""
    nnodes, ncomp = a.shape
    src = torch.from_numpy(np.ascontiguousarray(a)).to(device="cuda", dtype=dtype)
    out = torch.empty((ncomp, nnodes), dtype=dtype, device="cuda")
    _permute(p, src, out, nnodes, ncomp, False)
    return out


def Array(*args):
    """``Array(x)`` / ``Array(T, x)`` for Particles, CellArray, PhaseRatios,
    tuples of those and grid tensors (-> Fortran-ordered numpy arrays). The
    CellArray and PhaseRatios forms need the particles for the GPU stream:
    ``Array(x, particles)`` / ``Array(T, x, particles)``."""
    from .api import PhaseRatios
    T = None
    if len(args) >= 2 and not isinstance(args[0], (Particles, CellArray, PhaseRatios, tuple, list, torch.Tensor)):
        T, args = args[0], args[1:]
    x = args[0]
    p = args[1] if len(args) > 1 else None
    if isinstance(x, Particles):
        nc = int(np.prod(x.ni))
        coords = tuple(HostCellArray(_to_host(x, c.data, nc, T), x.ni) for c in x.coords)
        index = HostCellArray(_to_host(x, x.index.data, nc).astype(bool), x.ni)
        return HostParticles(coords, index, x.nxcell, x.max_xcell, x.min_xcell, x.np,
                             tuple(tuple(np.asarray(v, dtype=np.float64).copy() for v in comp) for comp in x.xi_vel),
                             bool(x.uniform), int(x.seed), int(x.rng_counter))
    if isinstance(x, (tuple, list)):
        return tuple(Array(*(((T,) if T is not None else ()) + (e,) + ((p,) if p is not None else ()))) for e in x)
    if isinstance(x, CellArray):
        if p is None:
            raise ArgumentError("Array(cell_array, particles): the particles give the stream")
        return HostCellArray(_to_host(p, x.data, int(np.prod(x.ni)), T), x.ni)
    if isinstance(x, PhaseRatios):
        if p is None:
            raise ArgumentError("Array(phase_ratios, particles): the particles give the stream")
        fields = {}
        for name in _phase_locations(x):
            t = getattr(x, name)
            fields[name] = _to_host(p, t, t.shape[1], T)
        return HostPhaseRatios(x.nphases, tuple(x.ni), fields)
    if isinstance(x, torch.Tensor):
        a = x.detach().cpu().numpy()
        dt = _np_dtype(T)
        return np.asfortranarray(a.astype(dt) if dt is not None else a)
    return x


def _phase_locations(pr):
    names = ["center", "vertex", "Vx", "Vy"]
    if len(pr.ni) == 3:
        names += ["Vz", "xy", "yz", "xz"]
    return names


def to_device(T, x, particles: Particles | None = None):
    """``TA(backend)(T, x)`` for host containers: HostParticles -> Particles
    (a new native container on the same grids, its slots and injection
    counter restored), HostCellArray / HostPhaseRatios -> device forms (these
    need the particles for the stream)."""
    dt = _np_dtype(T) if T is not None else np.float64
    tdt = torch.float64 if dt == np.float64 else torch.float32
    if isinstance(x, HostParticles):
        from .particles import init_particles_empty
        xi_vel = x.xi_vel
        if x.uniform:
            xi_vel = tuple(tuple(LinRange(v[0], v[-1], len(v)) for v in comp) for comp in xi_vel)
        p = init_particles_empty(CUDABackend, x.nxcell, x.max_xcell, x.min_xcell, *xi_vel, seed=x.seed)
        for d in range(x.ndim):
            p.coords[d].data.copy_(_to_device(p, x.coords[d].data, torch.float64))
        p.index.data.copy_(_to_device(p, x.index.data.astype(np.uint8), torch.uint8))
        p.rng_counter = x.rng_counter
        return p
    if isinstance(x, (tuple, list)):
        return tuple(to_device(T, e, particles) for e in x)
    if isinstance(x, HostCellArray):
        if particles is None:
            raise ArgumentError("TA(backend)(T, cell_array, particles): the particles give the stream")
        return CellArray(_to_device(particles, x.data, tdt), x.ni)
    if isinstance(x, HostPhaseRatios):
        if particles is None:
            raise ArgumentError("TA(backend)(T, phase_ratios, particles): the particles give the stream")
        from .api import PhaseRatios
        pr = PhaseRatios(x.nphases, x.ni)
        for name, a in x.fields.items():
            getattr(pr, name).copy_(_to_device(particles, a, torch.float64))
        return pr
    raise ArgumentError(f"cannot convert {type(x).__name__} to the device")


# ------------------------------------------------------------- checkpoints
_FORMAT = "justpic-gb300-checkpoint-1"


def checkpoint_name(dst, me=None) -> str:
    """src/IO/JLD2.jl:3-6, with the archive suffix."""
    if me is None:
        return os.path.join(dst, "particles_checkpoint.npz")
    return os.path.join(dst, f"particles_checkpoint{int(me):04d}.npz")


def _flatten(prefix, x, out, meta):
    if x is None:
        meta[prefix] = None
    elif isinstance(x, HostParticles):
        meta[prefix] = {"type": "Particles", "nxcell": x.nxcell, "max_xcell": x.max_xcell, "min_xcell": x.min_xcell,
                        "np": x.np, "ni": list(x.ni), "uniform": x.uniform, "seed": x.seed,
                        "rng_counter": x.rng_counter, "ndim": x.ndim}
        for d, c in enumerate(x.coords):
            out[f"{prefix}/coords/{d}"] = c.data
        out[f"{prefix}/index"] = x.index.data
        for c, comp in enumerate(x.xi_vel):
            for d, v in enumerate(comp):
                out[f"{prefix}/xi_vel/{c}/{d}"] = np.asarray(v)
    elif isinstance(x, HostCellArray):
        meta[prefix] = {"type": "CellArray", "ni": list(x.ni)}
        out[prefix] = x.data
    elif isinstance(x, HostPhaseRatios):
        meta[prefix] = {"type": "PhaseRatios", "nphases": x.nphases, "ni": list(x.ni), "fields": list(x.fields)}
        for name, a in x.fields.items():
            out[f"{prefix}/{name}"] = a
    elif isinstance(x, (tuple, list)):
        meta[prefix] = {"type": "tuple", "n": len(x)}
        for k, e in enumerate(x):
            _flatten(f"{prefix}/{k}", e, out, meta)
    elif isinstance(x, np.ndarray):
        meta[prefix] = {"type": "array"}
        out[prefix] = x
    elif isinstance(x, (int, float, bool, str)):
        meta[prefix] = {"type": "scalar", "value": x}
    else:
        raise ArgumentError(f"checkpoint entry {prefix!r}: unsupported type {type(x).__name__}")


def _unflatten(prefix, arrays, meta):
    m = meta[prefix]
    if m is None:
        return None
    kind = m["type"]
    if kind == "Particles":
        ni = tuple(m["ni"])
        N = m["ndim"]
        coords = tuple(HostCellArray(arrays[f"{prefix}/coords/{d}"], ni) for d in range(N))
        index = HostCellArray(arrays[f"{prefix}/index"], ni)
        xi_vel = tuple(tuple(arrays[f"{prefix}/xi_vel/{c}/{d}"] for d in range(N)) for c in range(N))
        return HostParticles(coords, index, m["nxcell"], m["max_xcell"], m["min_xcell"], m["np"], xi_vel,
                             m["uniform"], m["seed"], m["rng_counter"])
    if kind == "CellArray":
        return HostCellArray(arrays[prefix], tuple(m["ni"]))
    if kind == "PhaseRatios":
        return HostPhaseRatios(m["nphases"], tuple(m["ni"]), {n: arrays[f"{prefix}/{n}"] for n in m["fields"]})
    if kind == "tuple":
        return tuple(_unflatten(f"{prefix}/{k}", arrays, meta) for k in range(m["n"]))
    if kind == "array":
        return arrays[prefix]
    return m["value"]


def _host(x, particles):
    if x is None or isinstance(x, (HostParticles, HostCellArray, HostPhaseRatios, np.ndarray, int, float, bool, str)):
        return x
    if isinstance(x, (tuple, list)):
        return tuple(_host(e, particles) for e in x)
    return Array(x, particles)


def checkpointing_particles(dst, particles, me=None, *, phases=None, phase_ratios=None, chain=None, t=None, dt=None,
                            particle_args=None, **kwargs) -> str:
    """``checkpointing_particles(dst, particles[, me]; phases, phase_ratios,
    chain, t, dt, particle_args, kwargs...)`` (src/IO/JLD2.jl:8-129): write
    the host copies of the given containers to ``dst``; returns the path."""
    if chain is not None:
        raise ArgumentError("marker chains are not part of this library")
    os.makedirs(dst, exist_ok=True)
    fname = checkpoint_name(dst, me)
    entries = {"particles": Array(particles), "phases": _host(phases, particles),
               "phase_ratios": _host(phase_ratios, particles), "chain": None, "time": t, "timestep": dt,
               "particle_args": _host(tuple(particle_args), particles) if particle_args is not None else None}
    for key, value in kwargs.items():
        if key in entries:
            raise ArgumentError(f"checkpoint keyword {key!r} is reserved")
        entries[key] = _host(value, particles)
    arrays, meta = {}, {}
    for key, value in entries.items():
        _flatten(key, value, arrays, meta)
    arrays["__meta__"] = np.frombuffer(json.dumps({"format": _FORMAT, "keys": list(entries), "entries": meta})
                                       .encode(), dtype=np.uint8)
    fd, tmp = tempfile.mkstemp(dir=dst, prefix=".particles_checkpoint", suffix=".npz")
    try:
        with os.fdopen(fd, "wb") as f:
            np.savez(f, **arrays)
        os.replace(tmp, fname)
    finally:
        if os.path.exists(tmp):
            os.unlink(tmp)
    return fname


def load_checkpoint(path) -> dict:
    """Read a checkpoint back into host containers, keyed like the
    reference's file (``data["particles"]``, ``data["phases"]``, ...); pass
    them to ``TA(backend)(Float64, ...)`` to continue on the GPU."""
    with np.load(path) as z:
        arrays = {k: z[k] for k in z.files}
    info = json.loads(arrays.pop("__meta__").tobytes().decode())
    if info.get("format") != _FORMAT:
        raise ArgumentError(f"{path}: not a checkpoint of this library")
    return {key: _unflatten(key, arrays, info["entries"]) for key in info["keys"]}


__all__ = ["Array", "HostCellArray", "HostParticles", "HostPhaseRatios", "checkpoint_name",
           "checkpointing_particles", "load_checkpoint", "to_device", "_check_backend"]
