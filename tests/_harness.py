"""Run one seeded setup through both the CPU oracle and the CUDA library.

The oracle (oracle/oracle.py) is the checker; the library is the thing under
test. Both receive the same grids, velocity fields and seed.
"""
from __future__ import annotations

import numpy as np

import justpic_gb300 as jp
from justpic_gb300 import workloads as W
from oracle import oracle as O

INTERPS = {  # advection!, advection_LinP!, advection_MQS!
    "linear": (O.LINEAR, jp.advection_),
    "linp": (O.LINP, jp.advection_LinP_),
    "mqs": (O.MQS, jp.advection_MQS_),
}
METHODS = {
    "euler": (O.EULER, jp.Euler(), 0.5),
    "rk2": (O.RK2, jp.RungeKutta2(), 0.5),
    "rk2_23": (O.RK2, jp.RungeKutta2(2 / 3), 2 / 3),
    "rk4": (O.RK4, jp.RungeKutta4(), 0.5),
}


def refined_axis(n, seed, stretch=0.35):
    """Strictly increasing non-uniform vertex vector on [0, 1] with n cells."""
    rng = np.random.default_rng(seed)
    w = 1.0 + stretch * rng.uniform(-1, 1, n)
    x = np.concatenate([[0.0], np.cumsum(w)])
    return x / x[-1]


def expand_vector(x):
    """expand_range for vectors (test/test_2D.jl:44-50)."""
    return np.concatenate([[x[0] - (x[1] - x[0])], x, [x[-1] + (x[-1] - x[-2])]])


def refined_grid(ni, seed=7):
    N = len(ni)
    xv = tuple(refined_axis(ni[d], seed + d) for d in range(N))
    xc = tuple(0.5 * (x[1:] + x[:-1]) for x in xv)
    grid_v = tuple(tuple(xv[d] if d == c else expand_vector(xc[d]) for d in range(N)) for c in range(N))
    dx = tuple(float(np.min(np.diff(x))) for x in xv)
    return {"ndim": N, "ni": tuple(ni), "xv": xv, "xc": xc, "dx": dx, "grid_v": grid_v}


class Pair:
    """Oracle and GPU containers seeded identically."""

    def __init__(self, g, nxcell, max_xcell, min_xcell, seed=0x4A50, nfields=0, uniform=None):
        uniform = all(isinstance(x, jp.LinRange) for comp in g["grid_v"] for x in comp) if uniform is None \
            else uniform
        self.g = g
        host_grids = tuple(tuple(np.asarray(x, dtype=np.float64) for x in comp) for comp in g["grid_v"])
        self.o = O.OracleParticles(host_grids, nxcell, max_xcell, min_xcell, uniform=uniform, seed=seed)
        self.o.init_particles()
        self.p = jp.init_particles(jp.CUDABackend, nxcell, max_xcell, min_xcell, *g["grid_v"], seed=seed)
        self.of = [self.o.cell_array() for _ in range(nfields)]
        self.pf = list(jp.init_cell_arrays(self.p, nfields))

    # -- mirrored operations -------------------------------------------
    def advection(self, method, V, dt, interp="linear"):
        om, pm, alpha = METHODS[method]
        oi, fn = INTERPS[interp]
        err = self.o.advection(om, alpha, V, dt, oi)
        fn(self.p, pm, tuple(jp.TA("CUDA")(v) for v in V), dt)
        return err

    def move(self):
        err = self.o.move_particles(self.of)
        jp.move_particles_(self.p, tuple(self.pf))
        return err

    def inject(self):
        err = self.o.inject_particles(self.of)
        jp.inject_particles_(self.p, tuple(self.pf))
        return err

    def g2p(self, k, F):
        self.o.grid2particle(self.of[k], F)
        jp.grid2particle_(self.pf[k], jp.TA("CUDA")(F), self.p)

    def p2g(self, k):
        shape = tuple(n + 1 for n in self.p.ni)
        Fo = np.asfortranarray(np.zeros(shape))
        self.o.particle2grid(Fo, self.of[k])
        Fg = jp.grid_field(shape)
        jp.particle2grid_(Fg, self.pf[k], self.p)
        return Fo, Fg.cpu().numpy()

    # -- comparisons ---------------------------------------------------
    def assert_same(self, what=""):
        idx_o = self.o.index
        idx_g = self.p.index.numpy()
        assert np.array_equal(idx_o, idx_g), f"{what}: index masks differ in {np.sum(idx_o != idx_g)} slots"
        for d in range(self.o.ndim):
            assert_bits_equal(self.o.coords[d], self.p.coords[d].numpy(), f"{what}: coords[{d}]")
        live = idx_o.astype(bool)
        for k in range(len(self.of)):
            assert_bits_equal(self.of[k][live], self.pf[k].numpy()[live], f"{what}: field[{k}] (live slots)")


def assert_bits_equal(a, b, what=""):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    same = (a.view(np.uint64) == b.view(np.uint64)) | (np.isnan(a) & np.isnan(b))
    if not np.all(same):
        bad = np.argwhere(~same)
        i = tuple(bad[0])
        raise AssertionError(f"{what}: {len(bad)} values differ, first at {i}: {a[i]!r} vs {b[i]!r}")


def membership(index, coords_list=None):
    """Occupancy count per cell (the bit-exact parity quantity)."""
    return np.asarray(index, dtype=np.int64).sum(axis=0)


__all__ = ["Pair", "METHODS", "W", "O", "jp", "assert_bits_equal", "refined_grid", "membership"]
