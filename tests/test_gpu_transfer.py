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
