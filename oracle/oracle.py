"""ctypes front end of the CPU oracle (jp_oracle.c).

TEST INFRASTRUCTURE ONLY: imported by tests/, ``__graft_entry__.smoke()`` and the
``cpu_baseline`` leg of bench.py to check (or time beside) the CUDA library. The
product package never imports it.

Arrays use the layouts of the reference's GPU path:
  * per-slot arrays: numpy ``(max_xcell, ncells)`` C-order, i.e. element
    ``[s, c]`` at ``c + ncells * s`` (CellArray blocklength 0,
    ext/JustPICCUDAExt.jl:29), cell index column-major (x fastest);
  * grid fields: numpy arrays in Fortran order with the Julia shape, e.g. a
    vertex field of an nx x ny grid has shape ``(nx + 1, ny + 1)``.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "libjp_oracle.so")

EULER, RK2, RK4 = 0, 1, 2
LINEAR, LINP, MQS = 0, 1, 2  # velocity interpolation of advection!, advection_LinP!, advection_MQS!
# 3D edge midpoints of update_phase_ratios! (src/PhaseRatios/midpoints.jl:214-224)
MIDPOINTS = (("xy", (1, 1, 0)), ("yz", (0, 1, 1)), ("xz", (1, 0, 1)))
ERR_BISECTION_LIMIT, ERR_FAR_MOVE, ERR_NO_NEIGHBOUR = 0x1, 0x2, 0x4

_dp = ctypes.POINTER(ctypes.c_double)


class _Grid(ctypes.Structure):
    _fields_ = [
        ("ndim", ctypes.c_int32),
        ("n", ctypes.c_int64 * 3),
        ("ncells", ctypes.c_int64),
        ("nxcell", ctypes.c_int32),
        ("max_xcell", ctypes.c_int32),
        ("min_xcell", ctypes.c_int32),
        ("np_quadrant", ctypes.c_int32),
        ("seed", ctypes.c_uint64),
        ("xv", _dp * 3),
        ("dxv", _dp * 3),
        ("xvel", (_dp * 3) * 3),
        ("dxvel", (_dp * 3) * 3),
        ("nvel", (ctypes.c_int64 * 3) * 3),
        ("xc", _dp * 3),
        ("dxc", _dp * 3),
    ]


def build(force: bool = False) -> str:
    """Compile the oracle shared library with its Makefile (gcc, OpenMP)."""
    srcs = [os.path.join(_HERE, f) for f in ("jp_oracle.c", "jp_oracle_jvp.c", "jp_oracle.h")]
    if force or not os.path.exists(_LIB_PATH) or \
            os.path.getmtime(_LIB_PATH) < max(os.path.getmtime(s) for s in srcs):
        subprocess.run(["make", "-s", "-C", _HERE, "-B" if force else "all"], check=True)
    return _LIB_PATH


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(_LIB_PATH)
        G = ctypes.POINTER(_Grid)
        P3 = ctypes.c_void_p * 3
        L.jpo_set_threads.argtypes = [ctypes.c_int]
        L.jpo_init_particles.argtypes = [G, P3, ctypes.c_void_p]
        L.jpo_advection.argtypes = [G, ctypes.c_int, ctypes.c_double, P3, ctypes.c_double, P3, ctypes.c_void_p]
        L.jpo_advection.restype = ctypes.c_int
        L.jpo_advection_interp.argtypes = [G, ctypes.c_int, ctypes.c_int, ctypes.c_double, P3, ctypes.c_double, P3,
                                           ctypes.c_void_p]
        L.jpo_advection_interp.restype = ctypes.c_int
        L.jpo_interp_velocity.argtypes = [G, ctypes.c_int, P3, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
        L.jpo_interp_velocity.restype = ctypes.c_int
        L.jpo_move_particles.argtypes = [G, P3, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int]
        L.jpo_move_particles.restype = ctypes.c_int
        L.jpo_inject_particles.argtypes = [G, P3, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, ctypes.c_uint32]
        L.jpo_inject_particles.restype = ctypes.c_int
        L.jpo_inject_particles_phase.argtypes = [G, P3, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                                 ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, ctypes.c_uint32]
        L.jpo_inject_particles_phase.restype = ctypes.c_int
        L.jpo_grid2particle.argtypes = [G, ctypes.c_void_p, ctypes.c_void_p, P3, ctypes.c_void_p]
        L.jpo_particle2grid.argtypes = [G, ctypes.c_void_p, ctypes.c_void_p, P3, ctypes.c_void_p]
        L.jpo_grid2particle_flip.argtypes = [G, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_double,
                                             P3, ctypes.c_void_p]
        L.jpo_particle2grid_n.argtypes = [G, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, P3, ctypes.c_void_p]
        L.jpo_grid2particle_n.argtypes = [G, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, P3, ctypes.c_void_p]
        L.jpo_centroid2particle.argtypes = [G, ctypes.c_void_p, ctypes.c_void_p, P3]
        L.jpo_particle2centroid.argtypes = [G, ctypes.c_void_p, ctypes.c_void_p, P3]
        L.jpo_phase_ratios_center.argtypes = [G, ctypes.c_int, ctypes.c_void_p, P3, ctypes.c_void_p]
        L.jpo_phase_ratios_vertex.argtypes = [G, ctypes.c_int, ctypes.c_void_p, P3, ctypes.c_void_p]
        L.jpo_phase_ratios_face.argtypes = [G, ctypes.c_int, ctypes.c_void_p, P3, ctypes.c_int, ctypes.c_void_p]
        L.jpo_phase_ratios_midpoint.argtypes = [G, ctypes.c_int, ctypes.c_void_p, P3, ctypes.c_int, ctypes.c_void_p]
        L.jpo_advection_jvp.argtypes = [G, ctypes.c_int, ctypes.c_double, P3, P3, ctypes.c_double, P3, P3,
                                        ctypes.c_void_p]
        L.jpo_advection_jvp.restype = ctypes.c_int
        L.jpo_particle2grid_jvp.argtypes = [G, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                            P3, P3, ctypes.c_void_p]
        L.jpo_first_stage.argtypes = [ctypes.c_int, ctypes.c_double, ctypes.c_double, ctypes.c_int,
                                      _dp, _dp, _dp]
        L.jpo_second_stage.argtypes = [ctypes.c_double, ctypes.c_double, ctypes.c_int, _dp, _dp, _dp, _dp]
        L.jpo_lerp.argtypes = [ctypes.c_int, _dp, _dp]
        L.jpo_lerp.restype = ctypes.c_double
        L.jpo_bisection.argtypes = [ctypes.c_double, _dp, ctypes.c_int64, ctypes.c_int64,
                                    ctypes.POINTER(ctypes.c_int)]
        L.jpo_bisection.restype = ctypes.c_int64
        L.jpo_rand.argtypes = [ctypes.c_uint64, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_uint64,
                               ctypes.c_uint32, ctypes.c_uint32]
        L.jpo_rand.restype = ctypes.c_double
        L.jpo_philox.argtypes = [ctypes.c_uint32 * 4, ctypes.c_uint32 * 2, ctypes.c_uint32 * 4]
        _lib = L
    return _lib


def set_threads(n: int) -> None:
    lib().jpo_set_threads(int(n))


def _ptr(a: np.ndarray):
    return a.ctypes.data_as(ctypes.c_void_p) if a is not None else None


def _dptr(a: np.ndarray):
    return a.ctypes.data_as(_dp)


def _centres(xi_vel, uniform: bool):
    """Particles.xci and di.center (src/Particles/particles_utils.jl:56-79,
    :108-140): the interior of the ghost-expanded centre grids
    xi_vel[1][0], xi_vel[0][1] (, xi_vel[0][2]). A range keeps being a range:
    Julia's LinRange[2:end-1] is LinRange(r[2], r[end-1], n - 2), whose
    elements are recomputed from those end points; its spacing is one number,
    element 2 minus element 1. Vectors are sliced; spacing = diff."""
    N = len(xi_vel)
    src = [xi_vel[1][0], xi_vel[0][1]] + ([xi_vel[0][2]] if N == 3 else [])
    xc, dxc = [], []
    for v in src:
        v = np.asarray(v, dtype=np.float64)
        n = len(v) - 2
        if uniform:
            j = np.arange(n, dtype=np.float64)
            t = j / float(n - 1) if n > 1 else np.zeros(1)
            x = (1.0 - t) * v[1] + t * v[n]
            d = np.full(max(n - 1, 1), x[1] - x[0] if n > 1 else 0.0)
        else:
            x = np.ascontiguousarray(v[1:-1])
            d = np.ascontiguousarray(np.diff(x)) if n > 1 else np.zeros(1)
        xc.append(np.ascontiguousarray(x))
        dxc.append(np.ascontiguousarray(d))
    return tuple(xc), tuple(dxc)


def _spacing(x: np.ndarray, uniform: bool) -> np.ndarray:
    """di of init_particles: scalar x[2]-x[1] for ranges (particles_utils.jl:137-139),
    diff(x) for vector grids (particles_utils.jl:76-79), stored per interval."""
    if uniform:
        return np.full(len(x) - 1, x[1] - x[0], dtype=np.float64)
    return np.ascontiguousarray(np.diff(x), dtype=np.float64)


class OracleParticles:
    """The geometry part of a ``Particles`` container (particles.jl:17-46) plus the
    per-slot arrays, all on the host."""

    def __init__(self, xi_vel, nxcell, max_xcell, min_xcell, uniform=True, seed=0x4A50):
        ndim = len(xi_vel)
        assert ndim in (2, 3)
        self.ndim = ndim
        self.xi_vel = tuple(tuple(np.ascontiguousarray(a, dtype=np.float64) for a in comp) for comp in xi_vel)
        self.xvi = tuple(self.xi_vel[d][d] for d in range(ndim))
        self.n = tuple(len(x) - 1 for x in self.xvi)
        self.ncells = int(np.prod(self.n))
        nq = 2 ** ndim
        self.np_quadrant = -(-int(nxcell) // nq)
        self.nxcell = self.np_quadrant * nq
        self.max_xcell = max(self.nxcell, int(max_xcell))
        self.min_xcell = int(min_xcell)
        self.seed = int(seed)
        self.uniform = bool(uniform)
        self.dxv = tuple(_spacing(x, uniform) for x in self.xvi)
        self.dxvel = tuple(tuple(_spacing(x, uniform) for x in comp) for comp in self.xi_vel)
        self.xc, self.dxc = _centres(self.xi_vel, uniform)
        g = _Grid()
        g.ndim = ndim
        for d in range(3):
            g.n[d] = self.n[d] if d < ndim else 1
        g.ncells = self.ncells
        g.nxcell, g.max_xcell, g.min_xcell = self.nxcell, self.max_xcell, self.min_xcell
        g.np_quadrant = self.np_quadrant
        g.seed = self.seed
        for d in range(ndim):
            g.xv[d] = _dptr(self.xvi[d])
            g.dxv[d] = _dptr(self.dxv[d])
            for c in range(ndim):
                g.xvel[c][d] = _dptr(self.xi_vel[c][d])
                g.dxvel[c][d] = _dptr(self.dxvel[c][d])
                g.nvel[c][d] = len(self.xi_vel[c][d])
            g.xc[d] = _dptr(self.xc[d])
            g.dxc[d] = _dptr(self.dxc[d])
        self._g = g
        shape = (self.max_xcell, self.ncells)
        self.coords = tuple(np.full(shape, np.nan) for _ in range(ndim))
        self.index = np.zeros(shape, dtype=np.uint8)
        self.inject_calls = 0

    # -- helpers ---------------------------------------------------------
    def _p3(self, arrs):
        P3 = ctypes.c_void_p * 3
        v = [None, None, None]
        for i, a in enumerate(arrs):
            assert a.flags.c_contiguous or a.flags.f_contiguous
            v[i] = a.ctypes.data
        return P3(*v)

    def _args(self, args):
        args = tuple(args)
        arr = (ctypes.c_void_p * max(1, len(args)))(*[a.ctypes.data for a in args])
        return arr, len(args)

    def cell_array(self, fill=0.0):
        return np.full((self.max_xcell, self.ncells), fill, dtype=np.float64)

    # -- the hot path ----------------------------------------------------
    def init_particles(self):
        lib().jpo_init_particles(ctypes.byref(self._g), self._p3(self.coords), _ptr(self.index))

    def advection(self, method, alpha, V, dt, interp=LINEAR):
        """advection! (interp LINEAR), advection_LinP! (LINP) or advection_MQS! (MQS)."""
        V = [np.asfortranarray(v, dtype=np.float64) for v in V]
        self._keep = V
        return lib().jpo_advection_interp(ctypes.byref(self._g), int(method), int(interp), float(alpha),
                                          self._p3(V), float(dt), self._p3(self.coords), _ptr(self.index))

    def interp_velocity(self, V, p, I, interp=LINEAR):
        """One velocity sample at point p, the bisection seeded by 0-based cell I."""
        V = [np.asfortranarray(v, dtype=np.float64) for v in V]
        pa = np.ascontiguousarray(p, dtype=np.float64)
        Ia = np.ascontiguousarray(I, dtype=np.int64)
        out = np.zeros(self.ndim)
        lib().jpo_interp_velocity(ctypes.byref(self._g), int(interp), self._p3(V), _ptr(pa), _ptr(Ia), _ptr(out))
        return out

    def move_particles(self, args=()):
        a, n = self._args(args)
        return lib().jpo_move_particles(ctypes.byref(self._g), self._p3(self.coords), _ptr(self.index), a, n)

    def inject_particles(self, args=()):
        a, n = self._args(args)
        err = lib().jpo_inject_particles(ctypes.byref(self._g), self._p3(self.coords), _ptr(self.index), a, n,
                                         self.inject_calls)
        self.inject_calls += 1
        return err

    def inject_particles_phase(self, phases, args=(), fields=()):
        """inject_particles_phase!(particles, phases, args, fields): a field of
        the cells' shape is cell-centred, one of the vertices' shape a vertex
        field. Shares the injection call counter with inject_particles."""
        args, fields = tuple(args), tuple(np.asfortranarray(f, dtype=np.float64) for f in fields)
        assert len(args) == len(fields)
        centred = (ctypes.c_int * max(1, len(args)))(*[int(tuple(f.shape) == tuple(self.n)) for f in fields])
        a, n = self._args(args)
        fp = (ctypes.c_void_p * max(1, len(fields)))(*[f.ctypes.data for f in fields])
        self._keep = fields
        err = lib().jpo_inject_particles_phase(ctypes.byref(self._g), self._p3(self.coords), _ptr(self.index),
                                               _ptr(phases), a, fp, centred, n, self.inject_calls)
        self.inject_calls += 1
        return err

    def grid2particle(self, Fp, F):
        F = np.asfortranarray(F, dtype=np.float64)
        lib().jpo_grid2particle(ctypes.byref(self._g), _ptr(Fp), _ptr(F), self._p3(self.coords), _ptr(self.index))

    def particle2grid(self, F, Fp):
        assert F.flags.f_contiguous and F.dtype == np.float64
        lib().jpo_particle2grid(ctypes.byref(self._g), _ptr(F), _ptr(Fp), self._p3(self.coords), _ptr(self.index))

    def particle2grid_n(self, Fs, Fps):
        """particle2grid!(F::NTuple, Fp::NTuple, particles) on lists of fields."""
        assert len(Fs) == len(Fps) and 1 <= len(Fs) <= 16
        for F in Fs:
            assert F.flags.f_contiguous and F.dtype == np.float64
        dst = (ctypes.c_void_p * len(Fs))(*[_ptr(F) for F in Fs])
        src = (ctypes.c_void_p * len(Fps))(*[_ptr(f) for f in Fps])
        lib().jpo_particle2grid_n(ctypes.byref(self._g), dst, src, len(Fs), self._p3(self.coords), _ptr(self.index))

    def grid2particle_n(self, Fps, Fs):
        """grid2particle!(Fp::NTuple, F::NTuple, particles) on lists of fields."""
        assert len(Fs) == len(Fps) and 1 <= len(Fs) <= 16
        Fs = [np.asfortranarray(F, dtype=np.float64) for F in Fs]
        dst = (ctypes.c_void_p * len(Fps))(*[_ptr(f) for f in Fps])
        src = (ctypes.c_void_p * len(Fs))(*[_ptr(F) for F in Fs])
        lib().jpo_grid2particle_n(ctypes.byref(self._g), dst, src, len(Fs), self._p3(self.coords), _ptr(self.index))

    # -- the adjacent transfers -------------------------------------------
    def grid2particle_flip(self, Fp, F, F0, alpha=0.0):
        F = np.asfortranarray(F, dtype=np.float64)
        F0 = np.asfortranarray(F0, dtype=np.float64)
        lib().jpo_grid2particle_flip(ctypes.byref(self._g), _ptr(Fp), _ptr(F), _ptr(F0), float(alpha),
                                     self._p3(self.coords), _ptr(self.index))

    def centroid2particle(self, Fp, F):
        F = np.asfortranarray(F, dtype=np.float64)
        lib().jpo_centroid2particle(ctypes.byref(self._g), _ptr(Fp), _ptr(F), self._p3(self.coords))

    def particle2centroid(self, F, Fp):
        assert F.flags.f_contiguous and F.dtype == np.float64
        lib().jpo_particle2centroid(ctypes.byref(self._g), _ptr(F), _ptr(Fp), self._p3(self.coords))

    # -- phase ratios (src/PhaseRatios/) ---------------------------------
    def phase_ratios(self, phases, nphases):
        """update_phase_ratios!: dict of arrays (nphases, nodes) for 'center',
        'vertex', the faces 'Vx', 'Vy' (, 'Vz') and in 3D the edge midpoints
        'xy', 'yz', 'xz'; node index column-major over the location's grid."""
        N = self.ndim
        G = ctypes.byref(self._g)
        c3 = self._p3(self.coords)
        out = {"center": np.zeros((nphases, self.ncells))}
        lib().jpo_phase_ratios_center(G, int(nphases), _ptr(phases), c3, _ptr(out["center"]))
        nv = int(np.prod([n + 1 for n in self.n]))
        out["vertex"] = np.zeros((nphases, nv))
        lib().jpo_phase_ratios_vertex(G, int(nphases), _ptr(phases), c3, _ptr(out["vertex"]))
        for d, name in enumerate(["Vx", "Vy", "Vz"][:N]):
            nf = int(np.prod([n + (1 if e == d else 0) for e, n in enumerate(self.n)]))
            out[name] = np.zeros((nphases, nf))
            lib().jpo_phase_ratios_face(G, int(nphases), _ptr(phases), c3, d, _ptr(out[name]))
        if N == 3:
            for which, (name, off) in enumerate(MIDPOINTS):
                nm = int(np.prod([n + o for n, o in zip(self.n, off)]))
                out[name] = np.zeros((nphases, nm))
                lib().jpo_phase_ratios_midpoint(G, int(nphases), _ptr(phases), c3, which, _ptr(out[name]))
        return out

    # -- forward-mode derivatives (dual numbers through the same code) ----
    def advection_jvp(self, method, alpha, V, dV, dt, dcoords):
        """advection! on (value, tangent) pairs: coords advance exactly as in
        ``advection``; ``dcoords`` (per-slot arrays) carry the tangent for a
        velocity tangent ``dV`` (grid fields like V, or None)."""
        V = [np.asfortranarray(v, dtype=np.float64) for v in V]
        dV = [np.asfortranarray(v, dtype=np.float64) for v in dV] if dV is not None else None
        self._keep = (V, dV)
        return lib().jpo_advection_jvp(ctypes.byref(self._g), int(method), float(alpha), self._p3(V),
                                       self._p3(dV if dV is not None else []), float(dt),
                                       self._p3(self.coords), self._p3(dcoords), _ptr(self.index))

    def particle2grid_jvp(self, F, dF, Fp, dFp, dcoords):
        """particle2grid! and its tangent dF for tangents dFp (or None) and dcoords."""
        assert F.flags.f_contiguous and dF.flags.f_contiguous
        lib().jpo_particle2grid_jvp(ctypes.byref(self._g), _ptr(F), _ptr(dF), _ptr(Fp), _ptr(dFp),
                                    self._p3(self.coords), self._p3(dcoords), _ptr(self.index))


# -- known-answer helpers (test/test_integrators.jl, test_interpolation_kernels.jl)
def first_stage(method, alpha, dt, v, p):
    v = np.asarray(v, dtype=np.float64)
    p = np.asarray(p, dtype=np.float64)
    out = np.empty_like(p)
    lib().jpo_first_stage(method, alpha, dt, len(p), _dptr(v), _dptr(p), _dptr(out))
    return tuple(out)


def second_stage(alpha, dt, v0, v1, p):
    v0, v1, p = (np.asarray(a, dtype=np.float64) for a in (v0, v1, p))
    out = np.empty_like(p)
    lib().jpo_second_stage(alpha, dt, len(p), _dptr(v0), _dptr(v1), _dptr(p), _dptr(out))
    return tuple(out)


def lerp(v, t):
    v = np.asarray(v, dtype=np.float64)
    t = np.asarray(t, dtype=np.float64)
    return lib().jpo_lerp(len(t), _dptr(v), _dptr(t))


def bisection(px, x, seed):
    x = np.ascontiguousarray(x, dtype=np.float64)
    err = ctypes.c_int(0)
    r = lib().jpo_bisection(float(px), _dptr(x), len(x), int(seed), ctypes.byref(err))
    return r, err.value


def rand(seed, stream, call, cell, slot, dim):
    return lib().jpo_rand(seed, stream, call, cell, slot, dim)


def philox4x32_10(ctr, key):
    c = (ctypes.c_uint32 * 4)(*ctr)
    k = (ctypes.c_uint32 * 2)(*key)
    o = (ctypes.c_uint32 * 4)()
    lib().jpo_philox(c, k, o)
    return tuple(o)
