"""The CPU oracle against the reference's own known-answer and tolerance tests
(test/test_integrators.jl, test/test_interpolation_kernels.jl, test/test_2D.jl,
test/test_3D.jl). These pin the restatement without running Julia."""
import numpy as np
import pytest

from oracle import oracle as O
from justpic_gb300 import workloads as W
import justpic_gb300 as jp


# --- test/test_integrators.jl ------------------------------------------------
def test_rk2_first_stage_exact_2d():
    assert O.first_stage(O.RK2, 0.5, 0.1, (3.0, 4.0), (1.0, 2.0)) == (1.15, 2.2)  # :17-18


def test_rk2_second_stage_2d():
    p1 = O.first_stage(O.RK2, 0.5, 0.1, (3.0, 4.0), (1.0, 2.0))
    np.testing.assert_allclose(O.second_stage(0.5, 0.1, (3.0, 4.0), (3.1, 4.1), p1), (1.46, 2.61))  # :19
    p1 = O.first_stage(O.RK2, 2 / 3, 0.1, (3.0, 4.0), (1.0, 2.0))
    np.testing.assert_allclose(p1, (1.2, 2.266666666))  # :23
    np.testing.assert_allclose(O.second_stage(2 / 3, 0.1, (3.0, 4.0), (3.1, 4.1), p1), (1.5075, 2.67416666))  # :24


def test_euler_first_stage_exact():
    assert O.first_stage(O.EULER, 0.5, 0.1, (3.0, 4.0), (1.0, 2.0)) == (1.3, 2.4)  # :39
    assert O.first_stage(O.EULER, 0.5, 0.1, (3.0, 4.0, 5.0), (1.0, 2.0, 3.0)) == (1.3, 2.4, 3.5)  # :78


def test_rk2_3d():
    p1 = O.first_stage(O.RK2, 0.5, 0.1, (3.0, 4.0, 5.0), (1.0, 2.0, 3.0))
    assert p1 == (1.15, 2.2, 3.25)  # :57
    np.testing.assert_allclose(O.second_stage(0.5, 0.1, (3.0, 4.0, 5.0), (3.1, 4.1, 5.1), p1), (1.46, 2.61, 3.76))
    p1 = O.first_stage(O.RK2, 2 / 3, 0.1, (3.0, 4.0, 5.0), (1.0, 2.0, 3.0))
    np.testing.assert_allclose(p1, (1.2, 2.266666666, 3.3333333333333335))  # :62
    np.testing.assert_allclose(O.second_stage(2 / 3, 0.1, (3.0, 4.0, 5.0), (3.1, 4.1, 5.1), p1),
                               (1.5075, 2.67416666, 3.8408333333333333))  # :63


def test_integrator_argument_errors():
    with pytest.raises(jp.ArgumentError):
        jp.RungeKutta2(1.1)
    with pytest.raises(jp.ArgumentError):
        jp.RungeKutta2(-0.1)
    assert jp.RungeKutta2().alpha == 0.5 and jp.RungeKutta2(2 / 3).alpha == 2 / 3
    assert isinstance(jp.Euler("potato"), jp.Euler)


# --- test/test_interpolation_kernels.jl:47-60 ----------------------------------
def test_lerp_exact():
    assert O.lerp((1.0, 2.0), (0.5,)) == 1.5
    assert O.lerp((1.0, 2.0, 1.0, 2.0), (0.5, 0.5)) == 1.5
    assert O.lerp((1.0, 2.0, 1.0, 2.0, 1.0, 2.0, 1.0, 2.0), (0.5, 0.5, 0.5)) == 1.5


# --- src/Utils.jl:108-130 bisection semantics -----------------------------------
def test_bisection_closed_interval_and_ties():
    x = np.linspace(0.0, 1.0, 11)
    rng = np.random.default_rng(1)
    for seed in range(10):
        for px in rng.uniform(0, 1, 50):
            s, err = O.bisection(px, x, seed)
            assert err == 0 and x[s] <= px <= x[s + 1]
    # a point on a node: the seed's own interval wins when it holds it
    assert O.bisection(x[4], x, 4)[0] == 4
    assert O.bisection(x[4], x, 3)[0] == 3


def test_cell_index_bounds_like_the_reference():
    """test/test_2D.jl:143-167: for points drawn in [0, 1] on range(0, 1, 11)
    and in [-1, 0] on range(-1, 0, 11), the cell found satisfies
    x[i] <= p < x[i + 1]; the same on a refined vector axis. The oracle's cell
    search (find_parent_cell_bisection, from any seed cell) is the one the
    kernels use."""
    rng = np.random.default_rng(5)
    axes = [np.linspace(0.0, 1.0, 11), np.linspace(-1.0, 0.0, 11),
            np.concatenate([[0.0], np.cumsum(1.0 + 0.35 * rng.uniform(-1, 1, 10))]) / 10.0]
    axes[2] = axes[2] / axes[2][-1]
    for x in axes:
        for px in rng.uniform(x[0], x[-1], 200):
            for seed in (0, 4, len(x) - 2):
                i, err = O.bisection(px, x, seed)
                assert err == 0 and x[i] <= px < x[i + 1], (px, i, seed)


def test_bisection_is_bounded():
    x = np.linspace(0.0, 1.0, 11)
    s, err = O.bisection(float("nan"), x, 3)
    assert err == O.ERR_BISECTION_LIMIT


# --- counter RNG (Philox4x32-10, published known answers) ---------------------
@pytest.mark.parametrize("ctr,key,out", [
    ((0, 0, 0, 0), (0, 0), (0x6627e8d5, 0xe169c58d, 0xbc57ac4c, 0x9b00dbd8)),
    ((0xffffffff,) * 4, (0xffffffff,) * 2, (0x408f276d, 0x41c83b0e, 0xa20bc7c6, 0x6d5451fd)),
    ((0x243f6a88, 0x85a308d3, 0x13198a2e, 0x03707344), (0xa4093822, 0x299f31d0),
     (0xd16cfe09, 0x94fdcceb, 0x5001e420, 0x24126ea1)),
])
def test_philox_known_answers(ctr, key, out):
    # known-answer vectors of the Philox4x32-10 publication (Random123 distribution)
    assert O.philox4x32_10(ctr, key) == out


def test_rng_uniform_range_and_determinism():
    vals = [O.rand(7, 1, 2, c, s, d) for c in range(5) for s in range(3) for d in range(2)]
    assert all(0.0 <= v < 1.0 for v in vals)
    assert vals == [O.rand(7, 1, 2, c, s, d) for c in range(5) for s in range(3) for d in range(2)]
    assert len(set(vals)) == len(vals)


# --- interpolation tests (test_interpolation_kernels.jl:62-116, :118-180) ------
def _oracle_particles(g, nxcell, max_xcell, min_xcell, seed=0x4A50):
    grids = tuple(tuple(np.asarray(x) for x in comp) for comp in g["grid_v"])
    P = O.OracleParticles(grids, nxcell, max_xcell, min_xcell, uniform=True, seed=seed)
    P.init_particles()
    return P


@pytest.mark.parametrize("ndim", [2, 3])
def test_g2p_linear_field_and_p2g_error(ndim):
    g = W.grid((4,) * ndim)
    P = _oracle_particles(g, 5 if ndim == 2 else 12, 5 if ndim == 2 else 12, 1)
    axis = ndim - 1
    T = W.linear_T(g, axis)
    pT = P.cell_array()
    P.grid2particle(pT, T)
    live = P.index.astype(bool)
    np.testing.assert_allclose(pT[live], P.coords[axis][live], rtol=1e-12)  # pT ≈ coords
    T2 = np.asfortranarray(np.zeros_like(T))
    P.particle2grid(T2, pT)
    assert np.linalg.norm(T2 - T) / T.size < 0.1


@pytest.mark.parametrize("ndim", [2, 3])
def test_flip_and_centroid_transfers_linear_fields(ndim):
    """test_interpolation_kernels.jl:96-115 (2D), :163-180 (3D): FLIP with
    T0 = T keeps the PIC values; a linear centroid field interpolates exactly
    (2D: checked on cell (2, 2), 3D: everywhere); particle2centroid! error
    below 0.1."""
    g = W.grid((4,) * ndim)
    P = _oracle_particles(g, 5 if ndim == 2 else 12, 5 if ndim == 2 else 12, 1)
    axis = ndim - 1
    T = W.linear_T(g, axis)
    pT = P.cell_array()
    P.grid2particle(pT, T)
    live = P.index.astype(bool)
    assert live.all()  # nxcell rounds up to max_xcell: every slot holds a particle
    P.grid2particle_flip(pT, T, T.copy(order="F"))
    np.testing.assert_allclose(pT, P.coords[axis], rtol=1e-12)
    Tc = W.on_grid(lambda *x: x[axis] + 0.0 * x[0], g["xc"])
    P.centroid2particle(pT, Tc)
    if ndim == 2:
        c = 1 + 4 * 1  # cell (2, 2) of the 1-based reference test
        np.testing.assert_allclose(pT[:, c], P.coords[axis][:, c], rtol=1e-12)
    else:
        np.testing.assert_allclose(pT, P.coords[axis], rtol=1e-12)
    Tc2 = np.asfortranarray(np.zeros_like(Tc))
    P.particle2centroid(Tc2, pT)
    assert np.linalg.norm(Tc2 - Tc) / Tc.size < 0.1


def test_flip_blend_arithmetic():
    """grid_to_particle.jl:163-168: Fp = muladd(F_pic, a, (Fp + F_pic - F0_pic) (1 - a))."""
    g = W.grid((3, 3))
    P = _oracle_particles(g, 4, 4, 1)
    T = W.linear_T(g, 0)
    T0 = np.asfortranarray(0.5 * T)
    pT = P.cell_array(0.25)
    P.grid2particle_flip(pT, T, T0, alpha=0.3)
    x = P.coords[0]
    pic, pic0 = x, 0.5 * x  # linear fields interpolate exactly (to rounding)
    np.testing.assert_allclose(pT, 0.3 * pic + (0.25 + pic - pic0) * 0.7, rtol=1e-12)


def test_init_particles_layout():
    g = W.grid((6, 5))
    P = _oracle_particles(g, 24, 48, 12)
    assert P.nxcell == 24 and P.max_xcell == 48 and P.np_quadrant == 6
    assert P.index[:24].all() and not P.index[24:].any()
    # quadrant-stratified: slot l of quadrant q lies in that quadrant
    xv, yv = (np.asarray(a) for a in g["xv"])
    for c in range(P.ncells):
        i, j = c % 6, c // 6
        for l in range(24):
            q = l // 6
            x, y = P.coords[0][l, c], P.coords[1][l, c]
            hx, hy = (xv[i + 1] - xv[i]) / 2, (yv[j + 1] - yv[j]) / 2
            x0, y0 = xv[i] + hx * (q & 1), yv[j] + hy * (q >> 1)
            assert x0 <= x <= x0 + hx and y0 <= y <= y0 + hy
    # nxcell is rounded up to a multiple of 2^N and max_xcell follows
    P2 = _oracle_particles(g, 25, 20, 10)
    assert P2.nxcell == 28 and P2.max_xcell == 28


# --- miniapps with their tolerances (test/test_2D.jl:482-653) -----------------
def _miniapp(g, V, T, dt, nsteps, alpha, nxcell=25, max_xcell=50, min_xcell=10, uniform=True):
    grids = tuple(tuple(np.asarray(x) for x in comp) for comp in g["grid_v"])
    P = O.OracleParticles(grids, nxcell, max_xcell, min_xcell, uniform=uniform)
    P.init_particles()
    pT = P.cell_array()
    T = np.asfortranarray(T.copy())
    P.grid2particle(pT, T)
    sumT = T.sum()
    for _ in range(nsteps):
        P.particle2grid(T, pT)
        P.advection(O.RK2, alpha, V, dt)
        P.move_particles((pT,))
        P.inject_particles((pT,))
        P.grid2particle(pT, T)
    return abs(sumT - T.sum()) / sumT


def test_advection_2d_miniapp():
    g = W.grid((64, 64))
    V = W.stream_velocity(g)
    err = _miniapp(g, V, W.linear_T(g, 1), W.cfl_dt(g, V, 0.5), 25, 2 / 3)
    assert err < 1e-2  # test_2D.jl:540-545


def test_advection_2d_refined_miniapp():
    from _harness import refined_grid
    xv = np.array([0.0, 0.05, 0.12, 0.21, 0.32, 0.45, 0.6, 0.77, 0.91, 1.0])
    yv = np.array([0.0, 0.04, 0.1, 0.18, 0.29, 0.43, 0.58, 0.74, 0.89, 1.0])
    from _harness import expand_vector
    xc, yc = 0.5 * (xv[1:] + xv[:-1]), 0.5 * (yv[1:] + yv[:-1])
    g = {"ndim": 2, "ni": (9, 9), "xv": (xv, yv), "grid_v": ((xv, expand_vector(yc)), (expand_vector(xc), yv)),
         "dx": (np.min(np.diff(xv)), np.min(np.diff(yv)))}
    V = W.stream_velocity(g)
    T = W.on_grid(lambda x, y: y + 0 * x, (xv, yv))
    err = _miniapp(g, V, T, W.cfl_dt(g, V, 0.5), 25, 2 / 3, uniform=False)
    assert err < 1e-1  # test_2D.jl:592-597
    assert refined_grid  # imported helper used by the GPU tests too


def _miniapp_3d_refined_grid():
    """The refined 9^3 grid of test/test_3D.jl:388-399 (cell midpoints, expand_range ghosts)."""
    from _harness import expand_vector
    xv = np.array([0.0, 0.04, 0.09, 0.16, 0.25, 0.37, 0.52, 0.68, 0.84, 1.0])
    yv = np.array([0.0, 0.05, 0.11, 0.2, 0.31, 0.44, 0.58, 0.73, 0.87, 1.0])
    zv = np.array([0.0, 0.03, 0.08, 0.15, 0.26, 0.4, 0.56, 0.72, 0.88, 1.0])
    xvi = (xv, yv, zv)
    ext = tuple(expand_vector(0.5 * (x[1:] + x[:-1])) for x in xvi)
    grid_v = tuple(tuple(xvi[d] if d == c else ext[d] for d in range(3)) for c in range(3))
    return {"ndim": 3, "ni": (9, 9, 9), "xv": xvi, "grid_v": grid_v,
            "dx": tuple(float(np.min(np.diff(x))) for x in xvi)}


def miniapp_3d_inputs(g):
    """test/test_3D.jl:357-368, 401-415: the x-z stream function velocity on the
    staggered grids, T = z on the vertices, dt = min(dx_min / max|V|) / 4."""
    V = W.stream_velocity_3d(g)
    T = W.on_grid(lambda x, y, z: z + 0 * x + 0 * y, g["xv"])
    dt = min(g["dx"][d] / float(np.max(np.abs(V[d]))) for d in range(3) if np.max(np.abs(V[d])) > 0) / 4
    return V, T, dt


def test_advection_3d_refined_miniapp():
    # test_3D.jl:387-432 and :445-453: 125/150/100 particles per cell (cells wider
    # than 64 slots), 5 cycles of particle2grid!, RK2 advection!, move_particles!,
    # inject_particles!, grid2particle!; relative change of sum(T) below 1e-1
    g = _miniapp_3d_refined_grid()
    V, T, dt = miniapp_3d_inputs(g)
    err = _miniapp(g, V, T, dt, 5, 0.5, nxcell=125, max_xcell=150, min_xcell=100, uniform=False)
    assert np.isfinite(err) and err < 1e-1


def test_rotating_circle_miniapp():
    # test_2D.jl:599-653 (rotation of a disc; 100 steps of dt = 200)
    n = 256
    g = W.grid((n - 1, n - 1))
    vi = lambda x: np.pi * 1e-5 * (x - 0.5)  # noqa: E731
    Vx = W.on_grid(lambda x, y: -vi(y) + 0 * x, g["grid_v"][0])
    Vy = W.on_grid(lambda x, y: vi(x) + 0 * y, g["grid_v"][1])
    dx = g["dx"][0]
    R = 6 * dx
    T = W.on_grid(lambda x, y: (((x - 0.25) ** 2 + (y - 0.25) ** 2) <= R ** 2) * 1.0, g["xv"])
    tmax = 1 / (np.pi * 1e-5 / (2 * np.pi)) / 10
    nsteps = int(tmax // 200) + 1
    err = _miniapp(g, (Vx, Vy), T, 200.0, nsteps, 0.5)
    assert err < 1e-1


# --- inject_particles_phase! (src/Particles/injection.jl:133-325) -------------
@pytest.mark.parametrize("ndim", [2, 3])
def test_inject_phase_checks_every_quadrant(ndim):
    """A cell whose last quadrant is empty: inject_particles! stops at the
    first (full) quadrant and leaves it, inject_particles_phase! refills it
    with new particles that take the nearest particle's phase and the
    interpolated grid fields."""
    ni = (4,) * ndim
    g = W.grid(ni)
    nxcell, mx, mn = (24, 48, 12) if ndim == 2 else (24, 48, 16)
    P1 = _oracle_particles(g, nxcell, mx, mn)
    P2 = _oracle_particles(g, nxcell, mx, mn)
    npq = P1.np_quadrant
    cell = (1,) * ndim
    c = sum(cell[d] * 4 ** d for d in range(ndim))
    last = (1 << ndim) - 1
    for P in (P1, P2):
        for l in range(last * npq, (last + 1) * npq):
            P.index[l, c] = 0
            for d in range(ndim):
                P.coords[d][l, c] = np.nan
    before = P1.index.copy()
    assert P1.inject_particles(()) == 0
    assert np.array_equal(P1.index, before)  # first quadrant full: nothing injected

    ids = P2.cell_array(np.nan)
    live0 = P2.index.astype(bool)
    ids[live0] = np.arange(live0.sum(), dtype=np.float64)  # unique phase id per particle
    pT, pS = P2.cell_array(), P2.cell_array()
    lin = lambda *x: sum((d + 1.0) * x[d] for d in range(ndim))  # noqa: E731
    Fv = W.on_grid(lin, g["xv"])
    Fc = W.on_grid(lin, g["xc"])
    assert P2.inject_particles_phase(ids, (pT, pS), (Fv, Fc)) == 0
    new = P2.index.astype(bool) & ~live0
    min_xq = -(-mn // (1 << ndim))
    assert new.sum() == min_xq and new[:, c].sum() == min_xq
    xv = [np.asarray(a) for a in g["xv"]]
    pts = np.stack([P2.coords[d] for d in range(ndim)], axis=-1)
    orig = pts[live0]
    for l in np.nonzero(new[:, c])[0]:
        p = pts[l, c]
        for d in range(ndim):  # inside the refilled (upper) quadrant
            mid = 0.5 * (xv[d][cell[d]] + xv[d][cell[d] + 1])
            assert mid < p[d] < xv[d][cell[d] + 1]
        src = np.argwhere(ids == ids[l, c])
        assert len(src) >= 1 and not np.isnan(ids[l, c])
        dsrc = min(np.sum((pts[i, j] - p) ** 2) for i, j in src if (i, j) != (l, c))
        assert dsrc <= np.min(np.sum((orig - p) ** 2, axis=-1))  # no original particle is nearer
        np.testing.assert_allclose(pT[l, c], lin(*p), rtol=1e-12)
        np.testing.assert_allclose(pS[l, c], lin(*p), rtol=1e-12)


def test_inject_phase_clamps_to_corner_extrema():
    """Interpolated values never leave the range of the cell's grid values
    (injection.jl:300-316): a centred field whose bracketing centres are
    clamped at the domain edge gives the extrapolation clipped to the corners."""
    g = W.grid((4, 4))
    P = _oracle_particles(g, 24, 48, 12)
    for l in range(24):  # empty cell (0, 0) entirely
        P.index[l, 0] = 0
        P.coords[0][l, 0] = P.coords[1][l, 0] = np.nan
    ids = P.cell_array(1.0)
    pS = P.cell_array()
    Fc = W.on_grid(lambda x, y: np.exp(3 * x) + y, g["xc"])
    assert P.inject_particles_phase(ids, (pS,), (Fc,)) == 0
    live = P.index.astype(bool)
    vals = pS[:, 0][live[:, 0]]
    corners = Fc[0:2, 0:2]
    assert len(vals) > 0
    assert vals.min() >= corners.min() and vals.max() <= corners.max()
    assert np.all(ids[:, 0][live[:, 0]] == 1.0)


def _midpoint_ratios_loops(P, phases, nph, off):
    """Plain-loop restatement of phase_ratios_midpoint! (src/PhaseRatios/midpoints.jl:128-212)
    in 1-based indices, for a cross-check of the oracle on a small grid."""
    n = P.n
    xc = [np.asarray(P.xc[d]) for d in range(3)]
    dx = [np.asarray(P.dxv[d]) for d in range(3)]
    Mn = tuple(n[d] + off[d] for d in range(3))
    out = np.zeros((nph,) + Mn)
    masks = ((1, 0, 0), (0, 1, 0), (0, 0, 1), (1, 1, 1))

    def gather(I, xm):
        w = np.zeros(nph)
        for mask in masks:
            J = tuple(min(I[d] + off[d] * mask[d], n[d]) for d in range(3))
            di = [dx[d][J[d] - 1] for d in range(3)]
            c = (J[0] - 1) + n[0] * ((J[1] - 1) + n[1] * (J[2] - 1))
            for s in range(P.max_xcell):
                p = [P.coords[d][s, c] for d in range(3)]
                if any(np.isnan(p)) or not all(abs(p[d] - xm[d]) <= di[d] / 2 for d in range(3)):
                    continue
                x = np.prod([1.0 - abs(xm[d] - p[d]) / di[d] for d in range(3)])
                if not np.isnan(phases[s, c]):
                    w[int(phases[s, c]) - 1] += x
        w = w / w.sum() if w.sum() != 0 else w * np.nan
        return np.where(np.isnan(w), 0.0, w)

    for k in range(1, n[2] + 1):
        for j in range(1, n[1] + 1):
            for i in range(1, n[0] + 1):
                I = (i, j, k)
                cc = [xc[d][I[d] - 1] for d in range(3)]
                di = [dx[d][I[d] - 1] for d in range(3)]
                out[(slice(None),) + tuple(I[d] + off[d] - 1 for d in range(3))] = \
                    gather(I, [cc[d] + di[d] * off[d] / 2 for d in range(3)])
                if any(off[d] * I[d] == 1 for d in range(3)):
                    b = [int(n[d] == off[d] * I[d]) for d in range(3)]
                    w = gather(I, [cc[d] + di[d] * off[d] * b[d] / 2 for d in range(3)])
                    for r in (0, 1):
                        out[(slice(None),) + tuple(I[d] - 1 + r * b[d] for d in range(3))] = w
    return out.reshape(nph, -1, order="F")


def test_phase_ratios_midpoints_against_loops():
    g = W.grid((3, 4, 3))
    P = _oracle_particles(g, 8, 16, 4)
    rng = np.random.default_rng(9)
    ph = np.where(P.index.astype(bool), rng.integers(1, 4, P.index.shape).astype(np.float64), np.nan)
    ref = P.phase_ratios(ph, 3)
    for name, off in O.MIDPOINTS:
        np.testing.assert_allclose(ref[name], _midpoint_ratios_loops(P, ph, 3, off), rtol=1e-13, atol=1e-15,
                                   err_msg=name)
        s = ref[name].sum(axis=0)
        assert np.all((np.abs(s - 1) < 1e-12) | (s == 0))


def test_oracle_tuple_forms_match_the_scalar_forms():
    """The oracle's tuple grid2particle! equals the scalar one field by field;
    its tuple particle2grid! equals the scalar one in 3D (both normalise by
    wF * inv(w)) and differs from the 2D scalar form (wF / w) by at most one
    rounding."""
    for ni in [(9, 7), (4, 5, 3)]:
        g = W.grid(ni)
        grids = tuple(tuple(np.asarray(x) for x in comp) for comp in g["grid_v"])
        o = O.OracleParticles(grids, 24, 48, 12, uniform=True)
        o.init_particles()
        Fs = [W.gaussian_T(g, center=(0.4,) * len(ni)), W.linear_T(g, 0)]
        tup = [o.cell_array() for _ in Fs]
        o.grid2particle_n(tup, Fs)
        live = o.index.astype(bool)
        for k, F in enumerate(Fs):
            one = o.cell_array()
            o.grid2particle(one, F)
            assert np.array_equal(one[live], tup[k][live])
        shape = tuple(n + 1 for n in ni)
        Gt = [np.asfortranarray(np.zeros(shape)) for _ in Fs]
        o.particle2grid_n(Gt, tup)
        for k in range(len(Fs)):
            Gs = np.asfortranarray(np.zeros(shape))
            o.particle2grid(Gs, tup[k])
            if len(ni) == 3:
                assert np.array_equal(Gs, Gt[k])
            else:
                assert np.all(np.abs(Gs - Gt[k]) <= np.spacing(np.abs(Gs)))


@pytest.mark.parametrize("ndim", [2, 3])
def test_particle2grid_jvp_matches_oracle_fd(ndim):
    """The oracle's dual-number particle2grid! (the checker of the grid transfers'
    adjoint) against central differences of its own forward: a random tangent of
    the field and of every coordinate, compared vertex by vertex."""
    g = W.grid((5, 4) if ndim == 2 else (4, 3, 3))
    P = _oracle_particles(g, 8, 16, 4)
    T = W.gaussian_T(g, width2=0.05)
    pT = P.cell_array()
    P.grid2particle(pT, T)
    live = P.index.astype(bool)
    rng = np.random.default_rng(3)
    dT = np.where(live, rng.standard_normal(live.shape), 0.0)
    dX = [np.where(live, rng.standard_normal(live.shape), 0.0) for _ in range(ndim)]
    shape = tuple(n + 1 for n in g["ni"])
    F = np.asfortranarray(np.zeros(shape))
    dF = np.asfortranarray(np.zeros(shape))
    P.particle2grid_jvp(F, dF, pT, dT, [np.ascontiguousarray(x) for x in dX])
    F0 = np.asfortranarray(np.zeros(shape))
    P.particle2grid(F0, pT)
    np.testing.assert_array_equal(F, F0)  # the dual run's values are the forward's
    x0 = [c.copy() for c in P.coords]
    h = 1e-6

    def forward(sign):
        for d in range(ndim):
            P.coords[d][...] = x0[d] + sign * h * dX[d]
        Fs = np.asfortranarray(np.zeros(shape))
        P.particle2grid(Fs, np.where(live, pT + sign * h * dT, pT))
        return Fs

    fd = (forward(1.0) - forward(-1.0)) / (2 * h)
    for d in range(ndim):
        P.coords[d][...] = x0[d]
    scale = np.max(np.abs(dF))
    np.testing.assert_allclose(dF, fd, rtol=1e-5, atol=1e-6 * scale)
