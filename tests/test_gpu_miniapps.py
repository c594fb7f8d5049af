"""The reference's 3D advection miniapps (test/test_3D.jl:335-469) on the GPU:
125 / 150 / 100 particles per cell (cells wider than 64 slots), five cycles of
particle2grid!, RK2 advection!, move_particles!, inject_particles! and
grid2particle! with T = z, acceptance as in the reference: the relative change
of sum(T) below 1e-1.

  * refined 9^3 grid: the CUDA library against the oracle bit for bit after
    every call (occupancy, coordinates, field on live slots, gridded field);
  * uniform 63^3 grid (31M particles): the library alone (the oracle would
    take minutes here), against the reference's tolerance."""
import numpy as np
import pytest

from _harness import Pair, W, assert_bits_equal, jp
from test_oracle_kat import _miniapp_3d_refined_grid, miniapp_3d_inputs

pytestmark = pytest.mark.gpu


def test_refined_3d_miniapp_matches_oracle():
    g = _miniapp_3d_refined_grid()
    V, T, dt = miniapp_3d_inputs(g)
    pr = Pair(g, 125, 150, 100, nfields=1, uniform=False)
    pr.g2p(0, T)
    pr.assert_same("grid2particle!")
    sumT = T.sum()
    for it in range(5):
        Fo, Fg = pr.p2g(0)
        assert_bits_equal(Fo, Fg, f"cycle {it}: particle2grid!")
        T = np.asfortranarray(Fo)
        pr.advection("rk2", V, dt)
        pr.assert_same(f"cycle {it}: advection!")
        pr.move()
        pr.assert_same(f"cycle {it}: move_particles!")
        pr.inject()
        pr.assert_same(f"cycle {it}: inject_particles!")
        pr.g2p(0, T)
        pr.assert_same(f"cycle {it}: grid2particle!")
    err = abs(sumT - T.sum()) / sumT
    assert np.isfinite(err) and err < 1e-1


def test_uniform_3d_miniapp_full_size():
    n = 64
    g = W.grid((n - 1,) * 3)
    V, T, dt = miniapp_3d_inputs(g)
    p = jp.init_particles(jp.CUDABackend, 125, 150, 100, *g["grid_v"])
    Vd = tuple(jp.TA("CUDA")(v) for v in V)
    Td = jp.TA("CUDA")(T)
    pT, = jp.init_cell_arrays(p, 1)
    jp.grid2particle_(pT, Td, p)
    sumT = float(Td.sum())
    for _ in range(5):
        jp.particle2grid_(Td, pT, p)
        jp.advection_(p, jp.RungeKutta2(), Vd, dt)
        jp.move_particles_(p, (pT,))
        jp.inject_particles_(p, (pT,))
        jp.grid2particle_(pT, Td, p)
    err = abs(sumT - float(Td.sum())) / sumT
    assert np.isfinite(err) and err < 1e-1, err
    assert jp.move_counts(p)["moved_too_far"] == 0
