"""The oracle's LinP and MQS velocity interpolations (advection_LinP!,
advection_MQS!) against a plain-Python restatement written from the
reference's Julia source in its own 1-based form, bit for bit (muladd is
evaluated exactly with rationals, then rounded once, as an FMA does), plus the
known answers of the reference's refined-grid test (test/test_2D.jl:169-230):
the seed cell does not matter, and uniform grids reproduce linear fields."""
from fractions import Fraction

import numpy as np
import pytest

from oracle import oracle as O
from justpic_gb300 import workloads as W

from _harness import expand_vector


def fma(a, b, c):
    return float(Fraction(a) * Fraction(b) + Fraction(c))


def lerp1(t, v0, v1):  # src/Interpolations/ndlerp.jl:15
    return fma(t, v1, fma(-t, v0, v0))


def lerp(v, t):  # ndlerp.jl:11-14: x innermost
    if len(t) == 1:
        return lerp1(t[0], v[0], v[1])
    h = len(v) // 2
    return lerp1(t[-1], lerp(v[:h], t[:-1]), lerp(v[h:], t[:-1]))


def bisection(px, x, seed):  # src/Utils.jl:117-130, 1-based
    lo, hi = 1, len(x)
    while True:
        if x[seed - 1] <= px <= x[seed]:
            return seed
        if x[seed - 1] < px:
            lo = seed
            seed = (hi + seed) // 2
        else:
            hi = seed
            seed = (lo + seed) // 2


class Field:
    """F[i, j(, k)] with 1-based indices."""

    def __init__(self, F):
        self.F = np.asarray(F)
        self.size = self.F.shape

    def __getitem__(self, I):
        return float(self.F[tuple(i - 1 for i in I)])


def corner_values(F, idx):  # src/Advection/advection.jl:3-27
    if len(idx) == 2:
        i, j = idx
        return (F[i, j], F[i + 1, j], F[i, j + 1], F[i + 1, j + 1])
    i, j, k = idx
    return (F[i, j, k], F[i + 1, j, k], F[i, j + 1, k], F[i + 1, j + 1, k],
            F[i, j, k + 1], F[i + 1, j, k + 1], F[i, j + 1, k + 1], F[i + 1, j + 1, k + 1])


AUGMENT = {  # augment_offset (advection_LinP.jl:365-391): (offsetᵢ, offsetⱼ, offsetₖ)
    1: (((-1, 0, 1),) * 4, ((0, 0, 0), (1, 1, 1), (0, 0, 0), (1, 1, 1)), ((0, 0, 0), (0, 0, 0), (1, 1, 1), (1, 1, 1))),
    2: (((0, 0, 0), (1, 1, 1), (0, 0, 0), (1, 1, 1)), ((-1, 0, 1),) * 4, ((0, 0, 0), (0, 0, 0), (1, 1, 1), (1, 1, 1))),
    3: (((0, 0, 0), (0, 0, 0), (1, 1, 1), (1, 1, 1)), ((0, 0, 0), (1, 1, 1), (0, 0, 0), (1, 1, 1)), ((-1, 0, 1),) * 4),
}


def interpolate_V_to_P(F, xc, p, dx, comp, idx):  # advection_LinP.jl:207-330
    clamp = lambda a, n: min(max(a, 1), n)  # noqa: E731
    I = list(idx)
    I[comp - 1] += int(p[comp - 1] > xc[comp - 1] + dx[comp - 1] / 2)
    oi, oj, ok = AUGMENT[comp]
    if len(idx) == 2:
        nx, ny = F.size
        i, j = I
        vals = [[F[clamp(i + oi[r][s], nx), clamp(j + oj[r][s], ny)] for s in range(3)] for r in range(2)]
    else:
        nx, ny, nz = F.size
        i, j, k = I
        # rows 3 and 4 read offsetⱼ[1] and offsetⱼ[2], as the reference does
        ojr = (oj[0], oj[1], oj[0], oj[1])
        vals = [[F[clamp(i + oi[r][s], nx), clamp(j + ojr[r][s], ny), clamp(k + ok[r][s], nz)] for s in range(3)]
                for r in range(4)]
    av = []
    for row in vals:
        av += [(row[0] + row[1]) / 2, (row[2] + row[1]) / 2]
    if comp == 1:
        return tuple(av)
    order = (0, 2, 1, 3, 4, 6, 5, 7)[:len(av)]
    return tuple(av[o] for o in order)


def interp_linp(p, xi, dxi, F, comp, seed):  # advection_LinP.jl:112-140
    idx = tuple(bisection(p[d], xi[d], seed[d]) for d in range(len(p)))
    xc = tuple(float(xi[d][idx[d] - 1]) for d in range(len(p)))
    dx = tuple(float(dxi[d][idx[d] - 1]) for d in range(len(p)))
    tL = tuple((p[d] - xc[d]) * (1.0 / dx[d]) for d in range(len(p)))
    VL = lerp(corner_values(F, idx), tL)
    if not all(1 < idx[d] < F.size[d] - 1 for d in range(len(p))):
        return VL
    FP = interpolate_V_to_P(F, xc, p, dx, comp, idx)
    off = 1 - 2 * int(p[comp - 1] < xc[comp - 1] + dx[comp - 1] / 2)
    xP = list(xc)
    xP[comp - 1] = xc[comp - 1] + off * dx[comp - 1] / 2
    tP = tuple((p[d] - xP[d]) * (1.0 / dx[d]) for d in range(len(p)))
    VP = lerp(FP, tP)
    A = 2 / 3
    return A * VL + (1 - A) * VP


def mqs_pair(t, a, b, lo, hi):  # one `lerp + correction` of src/Interpolations/MQS.jl
    v0, v1, v2 = (lo, a, b) if t < 0.5 else (a, b, hi)
    corr = 0.5 * (t - 0.5) ** 2 * (fma(-2.0, v1, v0) + v2)
    return lerp1(t, a, b) + corr


def mqs(F, v, t, idx, comp):  # src/Interpolations/MQS.jl
    if len(idx) == 2:
        i, j = idx
        if comp == 1:
            r0 = mqs_pair(t[0], v[0], v[1], F[i - 1, j], F[i + 2, j])
            r1 = mqs_pair(t[0], v[2], v[3], F[i - 1, j + 1], F[i + 2, j + 1])
            return lerp1(t[1], r0, r1)
        r0 = mqs_pair(t[1], v[0], v[2], F[i, j - 1], F[i, j + 2])
        r1 = mqs_pair(t[1], v[1], v[3], F[i + 1, j - 1], F[i + 1, j + 2])
        return lerp1(t[0], r0, r1)
    i, j, k = idx
    if comp in (1, 2):  # MQS.jl:62-69: bottom and top both with layer k's stencil

        def four(w):
            if comp == 1:
                r0 = mqs_pair(t[0], w[0], w[1], F[i - 1, j, k], F[i + 2, j, k])
                r1 = mqs_pair(t[0], w[2], w[3], F[i - 1, j + 1, k], F[i + 2, j + 1, k])
                return lerp1(t[1], r0, r1)
            r0 = mqs_pair(t[1], w[0], w[2], F[i, j - 1, k], F[i, j + 2, k])
            r1 = mqs_pair(t[1], w[1], w[3], F[i + 1, j - 1, k], F[i + 1, j + 2, k])
            return lerp1(t[0], r0, r1)

        return lerp1(t[2], four(v[0:4]), four(v[4:8]))

    def fourz(w):  # MQS.jl:131-158 with (t1, t3)
        r0 = mqs_pair(t[0], w[0], w[1], F[i - 1, j, k], F[i + 2, j, k])
        r1 = mqs_pair(t[0], w[2], w[3], F[i - 1, j, k + 1], F[i + 2, j, k + 1])
        return lerp1(t[2], r0, r1)

    return lerp1(t[1], fourz((v[0], v[1], v[4], v[5])), fourz((v[2], v[3], v[6], v[7])))


def interp_mqs(p, xi, dxi, F, comp, seed):  # advection_MQS.jl:108-124
    idx = tuple(bisection(p[d], xi[d], seed[d]) for d in range(len(p)))
    xc = tuple(float(xi[d][idx[d] - 1]) for d in range(len(p)))
    dx = tuple(float(dxi[d][idx[d] - 1]) for d in range(len(p)))
    t = tuple((p[d] - xc[d]) * (1.0 / dx[d]) for d in range(len(p)))
    v = corner_values(F, idx)
    if all(1 < idx[d] < F.size[d] - 1 for d in range(len(p))):
        return mqs(F, v, t, idx, comp)
    return lerp(v, t)


def _oracle(g, uniform):
    grids = tuple(tuple(np.asarray(x, dtype=np.float64) for x in comp) for comp in g["grid_v"])
    P = O.OracleParticles(grids, 4 if g["ndim"] == 2 else 8, 8, 1, uniform=uniform)
    return P, grids


def _refined_2d():
    xv = np.array([0.0, 0.05, 0.12, 0.21, 0.32, 0.45, 0.6, 0.77, 0.91, 1.0])
    yv = np.array([0.0, 0.04, 0.1, 0.18, 0.29, 0.43, 0.58, 0.74, 0.89, 1.0])
    xc, yc = 0.5 * (xv[1:] + xv[:-1]), 0.5 * (yv[1:] + yv[:-1])
    return {"ndim": 2, "ni": (9, 9), "xv": (xv, yv), "grid_v": ((xv, expand_vector(yc)), (expand_vector(xc), yv))}


CASES = [("uniform2d", lambda: W.grid((7, 6)), True), ("refined2d", _refined_2d, False),
         ("uniform3d", lambda: W.grid((5, 6, 5)), True)]


@pytest.mark.parametrize("name,make,uniform", CASES)
@pytest.mark.parametrize("interp", [O.LINP, O.MQS])
def test_interpolation_matches_restatement(name, make, uniform, interp):
    g = make()
    N = g["ndim"]
    P, grids = _oracle(g, uniform)
    rng = np.random.default_rng(17)
    V = [np.asfortranarray(rng.standard_normal(tuple(len(x) for x in grids[c]))) for c in range(N)]
    xv = [np.asarray(x) for x in g["xv"]]
    fn = interp_linp if interp == O.LINP else interp_mqs
    for _ in range(150 if N == 2 else 60):
        p = tuple(float(rng.uniform(xv[d][0], xv[d][-1])) for d in range(N))
        seed0 = tuple(int(np.searchsorted(xv[d], p[d]) - 1) for d in range(N))  # the particle's cell, 0-based
        seed0 = tuple(min(max(s, 0), len(xv[d]) - 2) for d, s in enumerate(seed0))
        got = P.interp_velocity(V, p, seed0, interp)
        for c in range(N):
            xi = grids[c]
            dxi = [np.full(len(x) - 1, x[1] - x[0]) if uniform else np.diff(x) for x in xi]
            want = fn(p, xi, dxi, Field(V[c]), c + 1, tuple(s + 1 for s in seed0))
            assert got[c] == want or (np.isnan(got[c]) and np.isnan(want)), (name, c, p, got[c], want)


@pytest.mark.parametrize("interp", [O.LINP, O.MQS])
def test_refined_grid_linear_field_and_seed_independence(interp):
    """test/test_2D.jl:169-199: on the refined grid, p = (0.22, 0.48) seeded at
    cell (3, 3) or at its parent cell gives the same velocity; a constant
    field is reproduced to rounding, and on a uniform grid a linear one too
    (on a refined grid neither scheme is exact for linear fields: LinP's
    pressure points sit half the current interval from the node, not at the
    midpoints it averages, and MQS's curvature term assumes even spacing)."""
    xv = np.array([0.0, 0.1, 0.3, 0.6, 1.0])
    yv = np.linspace(0.0, 1.0, 5)
    xc, yc = 0.5 * (xv[1:] + xv[:-1]), 0.5 * (yv[1:] + yv[:-1])
    g = {"ndim": 2, "ni": (4, 4), "xv": (xv, yv), "grid_v": ((xv, expand_vector(yc)), (expand_vector(xc), yv))}
    P, grids = _oracle(g, False)
    Vx = W.on_grid(lambda x, y: 2.0 * x + y, grids[0])
    Vy = W.on_grid(lambda x, y: x - 3.0 * y, grids[1])
    p = (0.22, 0.48)
    seeded = P.interp_velocity((Vx, Vy), p, (2, 2), interp)
    parent = (int(np.searchsorted(xv, p[0]) - 1), int(np.searchsorted(yv, p[1]) - 1))
    corrected = P.interp_velocity((Vx, Vy), p, parent, interp)
    np.testing.assert_allclose(seeded, corrected, rtol=1e-14)
    const = (np.full_like(Vx, 0.08), np.full_like(Vy, 0.02))
    np.testing.assert_allclose(P.interp_velocity(const, p, (2, 2), interp), [0.08, 0.02], rtol=1e-15)
    gu = W.grid((8, 8))
    Pu, gr = _oracle(gu, True)
    Vxu = W.on_grid(lambda x, y: 2.0 * x + y, gr[0])
    Vyu = W.on_grid(lambda x, y: x - 3.0 * y, gr[1])
    rng = np.random.default_rng(3)
    for _ in range(50):
        q = tuple(float(v) for v in rng.uniform(0, 1, 2))
        cell = tuple(min(int(v * 8), 7) for v in q)
        np.testing.assert_allclose(Pu.interp_velocity((Vxu, Vyu), q, cell, interp),
                                   [2 * q[0] + q[1], q[0] - 3 * q[1]], rtol=1e-13, atol=1e-15)


def test_advection_linear_field_3d_linp():
    """In 3D, LinP reproduces linear fields in x and y, so one Euler step moves
    particles by dt * v(p) to rounding. Its z-component does not: the
    reference's augment_offset/swap_F for z put the y-shifted, z-averaged and
    x-shifted pressure values at the x, y and z corners of the lerp
    (advection_LinP.jl:257-330, 382-391), and 3D MQS corrects both layers
    with layer k's stencil (MQS.jl:62-76); the restatement test above pins
    both as the reference computes them."""
    g = W.grid((6, 5, 6))
    P, grids = _oracle(g, True)
    P.init_particles()
    V = [W.on_grid(lambda x, y, z, c=c: (c + 1.0) * x - 0.5 * y + (2.0 - c) * z, grids[c]) for c in range(3)]
    live = P.index.astype(bool)
    x0 = [P.coords[d].copy() for d in range(3)]
    dt = 1e-3
    assert P.advection(O.EULER, 0.5, V, dt, O.LINP) == 0
    for c in range(2):
        v = (c + 1.0) * x0[0] - 0.5 * x0[1] + (2.0 - c) * x0[2]
        np.testing.assert_allclose(P.coords[c][live], x0[c][live] + dt * v[live], rtol=0, atol=1e-15)
