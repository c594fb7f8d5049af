"""GPU parity of the transfers beside the hot path (grid2particle_flip!,
centroid2particle!, particle2centroid!) against the CPU oracle, bit for bit,
on particles that have been advected, moved and re-injected."""
import numpy as np
import pytest
import torch

from _harness import Pair, W, assert_bits_equal, jp, refined_grid

pytestmark = pytest.mark.gpu


def _moved_pair(ni, refined):
    g = refined_grid(ni) if refined else W.grid(ni)
    pair = Pair(g, 24, 48, 12, nfields=1)
    V = W.stream_velocity(g) if len(ni) == 2 else W.stream_velocity_3d(g)
    pair.g2p(0, W.linear_T(g, 0))
    dt = W.cfl_dt(g, V)
    for _ in range(3):
        pair.advection("rk2", V, dt)
        pair.move()
        pair.inject()
    pair.assert_same("setup")
    return pair, g


CASES = [((16, 16), False), ((11, 9), True), ((6, 5, 7), False), ((5, 6, 4), True)]


@pytest.mark.parametrize("ni,refined", CASES)
@pytest.mark.parametrize("alpha", [0.0, 0.3])
def test_grid2particle_flip_bit_exact(ni, refined, alpha):
    pair, g = _moved_pair(ni, refined)
    rng = np.random.default_rng(3)
    shape = tuple(n + 1 for n in ni)
    F = np.asfortranarray(rng.standard_normal(shape))
    F0 = np.asfortranarray(rng.standard_normal(shape))
    pair.o.grid2particle_flip(pair.of[0], F, F0, alpha)
    jp.grid2particle_flip_(pair.pf[0], pair.p.xvi, jp.TA("CUDA")(F), jp.TA("CUDA")(F0), pair.p, alpha)
    pair.assert_same("grid2particle_flip!")


@pytest.mark.parametrize("ni,refined", CASES)
def test_centroid_transfers_bit_exact(ni, refined):
    pair, g = _moved_pair(ni, refined)
    rng = np.random.default_rng(4)
    Fc = np.asfortranarray(rng.standard_normal(tuple(ni)))
    pair.o.centroid2particle(pair.of[0], Fc)
    jp.centroid2particle_(pair.pf[0], jp.TA("CUDA")(Fc), pair.p)
    pair.assert_same("centroid2particle!")
    Fo = np.asfortranarray(np.zeros(tuple(ni)))
    pair.o.particle2centroid(Fo, pair.of[0])
    Fg = jp.grid_field(tuple(ni))
    jp.particle2centroid_(Fg, pair.pf[0], pair.p)
    assert_bits_equal(Fo, Fg.cpu().numpy(), "particle2centroid!")


def test_centroid_transfers_reject_single_cell_axes():
    # one cell along x: the centre grid has a single node, nothing to interpolate between
    xv, yv = np.array([0.0, 1.0]), np.linspace(0.0, 1.0, 5)
    xc, yc = np.array([0.5]), 0.5 * (yv[1:] + yv[:-1])

    def expand(x, d):
        return np.concatenate([[x[0] - d], x, [x[-1] + d]])

    grids = ((xv, expand(yc, 0.25)), (expand(xc, 1.0), yv))
    p = jp.init_particles(jp.CUDABackend, 4, 4, 1, *grids)
    (pT,) = jp.init_cell_arrays(p, 1)
    with pytest.raises(jp.ArgumentError):
        jp.centroid2particle_(pT, jp.grid_field((1, 4)), p)
    with pytest.raises(jp.ArgumentError):
        jp.particle2centroid_(jp.grid_field((1, 4)), pT, p)


@pytest.mark.parametrize("ni,refined", CASES)
@pytest.mark.parametrize("nphases", [2, 3])
def test_phase_ratios_bit_exact(ni, refined, nphases):
    pair, g = _moved_pair(ni, refined)
    live = pair.o.index.astype(bool)
    # phase ids from the particles' position: bands along the last axis, ids 1..nphases
    ph = np.floor(pair.o.coords[len(ni) - 1] * nphases) + 1.0
    ph = np.where(live, np.clip(ph, 1, nphases), np.nan)
    ref = pair.o.phase_ratios(ph, nphases)
    phases = jp.CellArray(torch.from_numpy(np.ascontiguousarray(ph)).cuda(), pair.p.ni)
    pr = jp.PhaseRatios(nphases, ni)
    jp.update_phase_ratios_(pr, pair.p, phases)
    assert_bits_equal(ref["center"], pr.center.cpu().numpy(), "center")
    assert_bits_equal(ref["vertex"], pr.vertex.cpu().numpy(), "vertex")
    for d, name in enumerate(["Vx", "Vy", "Vz"][:len(ni)]):
        assert_bits_equal(ref[name], pr.faces[d].cpu().numpy(), name)
    if len(ni) == 3:
        for name in ("xy", "yz", "xz"):
            assert_bits_equal(ref[name], getattr(pr, name).cpu().numpy(), name)
            s = getattr(pr, name).sum(dim=0).cpu().numpy()
            assert np.all((np.abs(s - 1.0) < 1e-12) | (s == 0.0)), name


def _set_field(pair, k, values):
    pair.of[k][...] = values
    pair.pf[k].data.copy_(torch.from_numpy(np.ascontiguousarray(values)))


def _inject_phase(pair, fields):
    err = pair.o.inject_particles_phase(pair.of[0], pair.of[1:], fields)
    jp.inject_particles_phase_(pair.p, pair.pf[0], tuple(pair.pf[1:]), tuple(jp.TA("CUDA")(f) for f in fields))
    return err


@pytest.mark.parametrize("ni,refined", CASES)
def test_inject_particles_phase_bit_exact(ni, refined):
    """inject_particles_phase! against the oracle: phases copied from the
    nearest particle, one vertex and one cell-centred field interpolated,
    every quadrant refilled; after advection and move_particles! carrying
    the phases."""
    g = refined_grid(ni) if refined else W.grid(ni)
    pair = Pair(g, 24, 48, 20, nfields=3)  # phases, vertex-interpolated, centre-interpolated
    _set_field(pair, 0, W.shear_phases(pair.o.coords, pair.o.index))
    V = W.stream_velocity(g) if len(ni) == 2 else W.stream_velocity_3d(g)
    rng = np.random.default_rng(6)
    Fv = np.asfortranarray(rng.standard_normal(tuple(n + 1 for n in ni)))
    Fc = np.asfortranarray(rng.standard_normal(tuple(ni)))
    dt = W.cfl_dt(g, V)
    injected = 0
    for step in range(3):
        pair.advection("rk2", V, dt)
        pair.move()
        before = int(pair.o.index.sum())
        _inject_phase(pair, (Fv, Fc))
        injected += int(pair.o.index.sum()) - before
        pair.assert_same(f"inject_particles_phase! step {step}")
    assert injected > 0


def test_pure_shear_phase_miniapp_bit_exact():
    """The phase miniapp (test/test_2D.jl:385-481) on 32^2 cells with 64
    slots per cell (the bit-mask kernels; the miniapp's own 80 slots are
    covered by the wide-cell tests), 10 steps of RK2 + move +
    inject_particles_phase! + update_phase_ratios!, against the oracle; the
    ratios sum to one."""
    g, V, dt = W.pure_shear((32, 32))
    pair = Pair(g, 60, 64, 50, nfields=1, uniform=True)
    _set_field(pair, 0, W.shear_phases(pair.o.coords, pair.o.index))
    pr = jp.PhaseRatios(2, g["ni"])
    for step in range(10):
        pair.advection("rk2", V, dt)
        pair.move()
        _inject_phase(pair, ())
        pair.assert_same(f"pure shear step {step}")
        ref = pair.o.phase_ratios(pair.of[0], 2)
        jp.update_phase_ratios_(pr, pair.p, pair.pf[0])
        assert_bits_equal(ref["center"], pr.center.cpu().numpy(), "center")
        assert_bits_equal(ref["vertex"], pr.vertex.cpu().numpy(), "vertex")
    for name, a in (("center", pr.center), ("vertex", pr.vertex), ("Vx", pr.Vx), ("Vy", pr.Vy)):
        s = a.sum(dim=0).cpu().numpy()
        np.testing.assert_allclose(s, 1.0, rtol=1e-12, err_msg=name)  # test_2D.jl:476-479


def test_pure_shear_phase_miniapp_full_size():
    """The same miniapp at its own size (128^2 cells, 60/80/50 particles per
    cell, 20 steps) on the GPU alone: every location keeps ratios summing to
    one."""
    g, V, dt = W.pure_shear((128, 128))
    p = jp.init_particles(jp.CUDABackend, 60, 80, 50, *g["grid_v"])
    (phases,) = jp.init_cell_arrays(p, 1)
    ph = W.shear_phases([c.numpy() for c in p.coords], p.index.numpy())
    phases.data.copy_(torch.from_numpy(np.ascontiguousarray(ph)))
    pr = jp.PhaseRatios(2, g["ni"])
    jp.update_phase_ratios_(pr, p, phases)
    Vd = tuple(jp.TA("CUDA")(v) for v in V)
    for _ in range(20):
        jp.advection_(p, jp.RungeKutta2(), Vd, dt)
        jp.move_particles_(p, (phases,))
        jp.inject_particles_phase_(p, phases, (), ())
        jp.update_phase_ratios_(pr, p, phases)
    for name, a in (("center", pr.center), ("vertex", pr.vertex), ("Vx", pr.Vx), ("Vy", pr.Vy)):
        s = a.sum(dim=0).cpu().numpy()
        np.testing.assert_allclose(s, 1.0, rtol=1e-12, err_msg=name)
    ph_now = phases.numpy()[p.index.numpy().astype(bool)]
    assert set(np.unique(ph_now)) <= {1.0, 2.0}
