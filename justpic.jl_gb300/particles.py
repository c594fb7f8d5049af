"""Particle containers: ``CellArray``, ``Particles``, ``init_particles`` and
``init_cell_arrays``, mirroring src/particles.jl, src/launch.jl:78-112 and
src/Particles/particles_utils.jl of JustPIC.jl.

Device memory comes from PyTorch (CUDA tensors); the compute is the native
library. Layout of every per-slot array is the reference's GPU CellArray
(blocklength 0, ext/JustPICCUDAExt.jl:29): ``data`` has shape
``(max_xcell, ncells)`` so that slot ``s`` of cell ``c`` sits at
``c + ncells * s`` with ``c`` the column-major (x fastest) linear cell index.
Grid fields are device tensors with the Julia shape (e.g. ``(nx+1, ny+1)``)
and column-major strides; ``TA(backend)(a)`` builds them from host arrays.
"""
from __future__ import annotations

import ctypes
import numbers

import numpy as np
import torch

from . import _native
from ._native import ArgumentError, GridDesc, check

DEFAULT_SEED = 0x4A50

CUDABackend = "CUDABackend"
_BACKENDS = ("CUDA", "CUDABackend", "GB300", "cuda")


def _check_backend(backend) -> None:
    if backend not in _BACKENDS:
        raise ArgumentError(
            f"backend {backend!r} is not supported: this library runs the GB300 CUDA kernels only")


class LinRange:
    """Julia's ``LinRange(start, stop, len)``: element j (0-based) is
    ``(1 - t) * start + t * stop`` with ``t = j / (len - 1)`` (Base.lerpi).
    Grids given as LinRange use the reference's range rules (one spacing per
    axis); plain arrays use the vector rules (per-interval spacing)."""

    def __init__(self, start, stop, length: int):
        self.start = float(start)
        self.stop = float(stop)
        self.length = int(length)
        j = np.arange(self.length, dtype=np.float64)
        t = j / float(self.length - 1) if self.length > 1 else np.zeros(1)
        self._values = (1.0 - t) * self.start + t * self.stop

    def __len__(self):
        return self.length

    def __getitem__(self, i):
        return self._values[i]

    def __array__(self, dtype=None, copy=None):
        return self._values.astype(dtype) if dtype is not None else self._values

    @property
    def values(self) -> np.ndarray:
        return self._values

    def __repr__(self):
        return f"LinRange({self.start}, {self.stop}, {self.length})"


def _host_vector(x) -> np.ndarray:
    if isinstance(x, LinRange):
        return x.values
    if isinstance(x, torch.Tensor):
        x = x.detach().cpu().numpy()
    return np.ascontiguousarray(np.asarray(x, dtype=np.float64))


class CellArray:
    """Fixed-capacity per-cell storage (CellArrays.jl ``CellArray`` with
    blocklength 0). ``data`` is a CUDA tensor of shape ``(ncap, ncells)``."""

    def __init__(self, data: torch.Tensor, ni):
        self.data = data
        self.ni = tuple(int(n) for n in ni)
        if data.dim() != 2 or data.shape[1] != int(np.prod(self.ni)) or not data.is_contiguous():
            raise ArgumentError("CellArray data must be a contiguous (ncap, ncells) tensor")

    @property
    def ncap(self) -> int:
        return self.data.shape[0]

    def size(self):
        return self.ni

    @property
    def shape(self):
        return self.ni

    def linear(self, *I) -> int:
        c, stride = 0, 1
        for i, n in zip(I, self.ni):
            c += int(i) * stride
            stride *= n
        return c

    def cell(self, *I) -> torch.Tensor:
        """All slots of cell I (0-based), i.e. Julia's ``A[I...]``."""
        return self.data[:, self.linear(*I)]

    def __getitem__(self, key):
        """``A[ip, i, j(, k)]`` (0-based): one slot, like ``CAI.@index A[ip, I...]``."""
        ip, *I = key
        return self.data[ip, self.linear(*I)]

    def numpy(self) -> np.ndarray:
        return self.data.detach().cpu().numpy()

    def data_ptr(self) -> int:
        return self.data.data_ptr()


def cell_array(backend, x, ncells, ni) -> CellArray:
    """``cell_array(backend, x, ncells, ni)`` (src/launch.jl:101-108)."""
    _check_backend(backend)
    ncap = int(np.prod(ncells))
    n = int(np.prod(ni))
    if isinstance(x, (bool, np.bool_)):
        data = torch.full((ncap, n), int(x), dtype=torch.uint8, device="cuda")
    else:
        data = torch.full((ncap, n), float(x), dtype=torch.float64, device="cuda")
    return CellArray(data, ni)


def TA(backend):
    """Array constructor of a backend (JustPIC ``TA``): host array (Julia shape,
    any order) -> CUDA float64 tensor with the same shape and column-major
    strides. ``TA(backend)(T, x[, particles])`` also takes the host containers
    of ``Array`` (particles, cell arrays, phase ratios; ext/JustPICCUDAExt.jl:51-191)."""
    _check_backend(backend)

    def convert(*args):
        if len(args) >= 2:
            T, x, rest = args[0], args[1], args[2:]
            from . import conversion
            if isinstance(x, (conversion.HostParticles, conversion.HostCellArray, conversion.HostPhaseRatios,
                              tuple, list)):
                return conversion.to_device(T, x, *rest)
            a = np.asarray(x, dtype=conversion._np_dtype(T))
        else:
            a = np.asarray(args[0], dtype=np.float64)
        rev = tuple(reversed(range(a.ndim)))
        return torch.from_numpy(np.ascontiguousarray(a.transpose(rev))).to("cuda").permute(*rev)

    return convert


def grid_field(shape, fill=0.0) -> torch.Tensor:
    """A column-major CUDA float64 tensor of Julia shape filled with ``fill``."""
    t = torch.full(tuple(reversed(shape)), float(fill), dtype=torch.float64, device="cuda")
    return t.permute(*reversed(range(t.dim())))


class Particles:
    """``Particles`` (src/particles.jl:17-46) backed by the native container."""

    def __init__(self, handle, coords, index, nxcell, max_xcell, min_xcell, np_, di, _di, xci, xvi, xi_vel,
                 uniform, seed):
        self._handle = handle
        self.backend = CUDABackend
        self.coords = coords
        self.index = index
        self.nxcell = nxcell
        self.max_xcell = max_xcell
        self.min_xcell = min_xcell
        self.np = np_
        self.di = di
        self._di = _di
        self.xci = xci
        self.xvi = xvi
        self.xi_vel = xi_vel
        self.uniform = uniform
        self.seed = seed

    @property
    def ndim(self) -> int:
        return len(self.coords)

    @property
    def ni(self):
        return self.index.ni

    @property
    def handle(self):
        return self._handle

    def __del__(self):
        h = getattr(self, "_handle", None)
        if h:
            try:
                _native.load().jp_particles_destroy(h)
            except Exception:
                pass
            self._handle = None

    # the injection RNG counter (number of inject calls so far)
    @property
    def rng_counter(self) -> int:
        v = ctypes.c_uint64(0)
        check(_native.load().jp_get_rng_counter(self._handle, ctypes.byref(v)))
        return v.value

    @rng_counter.setter
    def rng_counter(self, value: int) -> None:
        check(_native.load().jp_set_rng_counter(self._handle, int(value)))


def _center_coordinates(xi_vel, uniform=False):
    """center_coordinates (src/Particles/particles_utils.jl:55-69): the
    interior of the ghost-expanded centre grids. A range stays a range
    (Julia's LinRange[2:end-1] = LinRange(r[2], r[end-1], n - 2), elements
    recomputed from those end points); vectors are sliced."""
    src = [xi_vel[1][0], xi_vel[0][1]] + ([xi_vel[0][2]] if len(xi_vel) == 3 else [])
    out = []
    for v in src:
        v = np.asarray(v, dtype=np.float64)
        if uniform and len(v) > 3:
            out.append(LinRange(v[1], v[len(v) - 2], len(v) - 2).values)
        else:
            out.append(v[1:-1])
    return tuple(out)


def init_particles(backend, nxcell, max_xcell, min_xcell, *xi_vel, seed: int = DEFAULT_SEED) -> Particles:
    """``init_particles(backend, nxcell, max_xcell, min_xcell, xi_vel...)``
    (src/Particles/particles_utils.jl:30-166): random quadrant-stratified seeding.

    ``xi_vel`` are the staggered velocity grids, one tuple of axis vectors per
    velocity component. If every vector is a ``LinRange`` the range rules
    apply (a single spacing per axis), otherwise the vector rules.
    """
    p = init_particles_empty(backend, nxcell, max_xcell, min_xcell, *xi_vel, seed=seed)
    from .api import _bind_stream, _finish
    _bind_stream(p)
    ptrs = _native.P3(*[c.data_ptr() for c in p.coords], *([None] * (3 - p.ndim)))
    _finish(p, _native.load().jp_init_particles(p.handle, ptrs, p.index.data_ptr()), "init_particles")
    return p


def init_particles_empty(backend, nxcell, max_xcell, min_xcell, *xi_vel, seed: int = DEFAULT_SEED) -> Particles:
    """The container of ``init_particles`` with every slot empty (NaN
    coordinates, index false): the target of a restart."""
    _check_backend(backend)
    if len(xi_vel) == 1 and isinstance(xi_vel[0], tuple) and len(xi_vel[0]) in (2, 3) and \
            isinstance(xi_vel[0][0], tuple):
        xi_vel = xi_vel[0]
    if len(xi_vel) == 0:
        raise ArgumentError("The velocity grid cannot be empty")
    if not isinstance(nxcell, numbers.Number):
        raise ArgumentError("structured (NTuple) nxcell layouts are not supported by this backend")
    N = len(xi_vel)
    if N not in (2, 3) or any(len(comp) != N for comp in xi_vel):
        raise ArgumentError("xi_vel must hold N grids of N axes each, N = 2 or 3")
    uniform = all(isinstance(x, LinRange) for comp in xi_vel for x in comp)
    host = tuple(tuple(_host_vector(x) for x in comp) for comp in xi_vel)

    desc = GridDesc()
    desc.ndim = N
    desc.uniform = 1 if uniform else 0
    for c in range(N):
        for d in range(N):
            desc.xi_vel[c][d] = host[c][d].ctypes.data_as(ctypes.POINTER(ctypes.c_double))
            desc.n_vel[c][d] = len(host[c][d])
    lib = _native.load()
    handle = ctypes.c_void_p()
    check(lib.jp_particles_create(ctypes.byref(handle), ctypes.byref(desc), int(nxcell), int(max_xcell),
                                  int(min_xcell), int(seed) & 0xFFFFFFFFFFFFFFFF))
    ndim = ctypes.c_int32()
    nc = (ctypes.c_int64 * 3)()
    nx_r, mx_r, mn_r = ctypes.c_int32(), ctypes.c_int32(), ctypes.c_int32()
    np_ = ctypes.c_int64()
    check(lib.jp_particles_info(handle, ctypes.byref(ndim), nc, ctypes.byref(nx_r), ctypes.byref(mx_r),
                                ctypes.byref(mn_r), ctypes.byref(np_)))
    ni = tuple(int(nc[d]) for d in range(N))

    xvi = tuple(host[d][d] for d in range(N))
    xci = _center_coordinates(host, uniform)
    if uniform:
        if any(len(x) < 2 for x in xci):
            # the reference takes getindex(xci, 2) - first(xci) (particles_utils.jl:137), which
            # has no second centre on a single-cell axis of a range grid
            raise ArgumentError("range grids need at least 2 cells per axis (use vector grids for one cell)")
        dvert = tuple(x[1] - x[0] for x in xvi)
        dcent = tuple(x[1] - x[0] for x in xci)
        dvel = tuple(tuple(x[1] - x[0] for x in comp) for comp in host)
        inv = lambda v: 1.0 / v  # noqa: E731
    else:
        dvert = tuple(np.diff(x) for x in xvi)
        dcent = tuple(np.diff(x) for x in xci)
        dvel = tuple(tuple(np.diff(x) for x in comp) for comp in host)
        inv = lambda v: 1.0 / np.asarray(v)  # noqa: E731
    di = {"center": dcent, "vertex": dvert, "velocity": dvel}
    _di = {"center": tuple(inv(v) for v in dcent), "vertex": tuple(inv(v) for v in dvert),
           "velocity": tuple(tuple(inv(v) for v in comp) for comp in dvel)}

    coords = tuple(cell_array(backend, float("nan"), (mx_r.value,), ni) for _ in range(N))
    index = cell_array(backend, False, (mx_r.value,), ni)
    return Particles(handle, coords, index, nx_r.value, mx_r.value, mn_r.value, np_.value, di, _di, xci, xvi, host,
                     uniform, seed)


def init_cell_arrays(particles: Particles, n) -> tuple:
    """``init_cell_arrays(particles, Val(n))`` (particles_utils.jl:294-301):
    n zero-filled per-slot fields with the particle layout."""
    n = int(n)
    return tuple(cell_array(CUDABackend, 0.0, (particles.max_xcell,), particles.ni) for _ in range(n))
