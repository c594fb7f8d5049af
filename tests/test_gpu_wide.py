"""Cells of more than 64 slots (the reference's own miniapp capacities:
60/80/50 in the 2D phase miniapp, 125/150/100 in the 3D advection miniapps,
125/125/125 in the 3D phase-ratio test) against the oracle, bit for bit."""
import numpy as np
import pytest
import torch

from _harness import Pair, W, assert_bits_equal, jp, refined_grid

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("ni,refined,cap", [((12, 10), False, (100, 128, 80)), ((9, 11), True, (60, 80, 50)),
                                             ((5, 4, 6), False, (125, 150, 100))])
def test_wide_cells_hot_path_bit_exact(ni, refined, cap):
    g = refined_grid(ni) if refined else W.grid(ni)
    pair = Pair(g, *cap, nfields=1)
    assert pair.p.max_xcell == pair.o.max_xcell > 64
    pair.assert_same("init")
    V = W.stream_velocity(g) if len(ni) == 2 else W.stream_velocity_3d(g)
    pair.g2p(0, W.linear_T(g, 0))
    pair.assert_same("grid2particle!")
    dt = W.cfl_dt(g, V, 0.5)
    injected = 0
    for step, interp in enumerate(["linear", "linp", "mqs"]):
        pair.advection("rk2", V, dt, interp)
        pair.assert_same(f"advection {interp}")
        pair.move()
        pair.assert_same(f"move step {step}")
        before = int(pair.o.index.sum())
        pair.inject()
        injected += int(pair.o.index.sum()) - before
        pair.assert_same(f"inject step {step}")
    Fo, Fg = pair.p2g(0)
    assert_bits_equal(Fo, Fg, "particle2grid!")
    assert injected > 0
    F = np.asfortranarray(np.random.default_rng(2).standard_normal(tuple(n + 1 for n in ni)))
    pair.o.grid2particle_flip(pair.of[0], F, 0.5 * F, 0.3)
    jp.grid2particle_flip_(pair.pf[0], None, jp.TA("CUDA")(F), jp.TA("CUDA")(np.asfortranarray(0.5 * F)), pair.p, 0.3)
    pair.assert_same("grid2particle_flip!")
    Fc = np.asfortranarray(np.random.default_rng(3).standard_normal(tuple(ni)))
    pair.o.centroid2particle(pair.of[0], Fc)
    jp.centroid2particle_(pair.pf[0], jp.TA("CUDA")(Fc), pair.p)
    pair.assert_same("centroid2particle!")
    Fo = np.asfortranarray(np.zeros(tuple(ni)))
    pair.o.particle2centroid(Fo, pair.of[0])
    Fg = jp.grid_field(tuple(ni))
    jp.particle2centroid_(Fg, pair.pf[0], pair.p)
    assert_bits_equal(Fo, Fg.cpu().numpy(), "particle2centroid!")


def test_wide_cells_noalloc_move_matches():
    g = W.grid((10, 9))
    pair = Pair(g, 60, 80, 50, nfields=1)
    V = W.stream_velocity(g)
    pair.advection("rk2", V, W.cfl_dt(g, V, 0.5))
    pair.o.move_particles(pair.of)
    lib = jp._native.load()
    coords = jp._native.P3(*[c.data_ptr() for c in pair.p.coords], None)
    args = (jp._native.ctypes.c_void_p * 1)(pair.pf[0].data_ptr())
    assert lib.jp_move_particles_noalloc(pair.p.handle, coords, pair.p.index.data_ptr(), args, 1) == 0
    jp.synchronize(pair.p)
    pair.assert_same("move (no scratch)")


def test_pure_shear_phase_miniapp_reference_capacity():
    """test/test_2D.jl:385-481 with its own 60/80/50 particles per cell on
    32^2 cells, 8 steps against the oracle; ratios sum to one."""
    g, V, dt = W.pure_shear((32, 32))
    pair = Pair(g, 60, 80, 50, nfields=1, uniform=True)
    ph = W.shear_phases(pair.o.coords, pair.o.index)
    pair.of[0][...] = ph
    pair.pf[0].data.copy_(torch.from_numpy(np.ascontiguousarray(ph)))
    pr = jp.PhaseRatios(2, g["ni"])
    for step in range(8):
        pair.advection("rk2", V, dt)
        pair.move()
        pair.o.inject_particles_phase(pair.of[0], (), ())
        jp.inject_particles_phase_(pair.p, pair.pf[0], (), ())
        pair.assert_same(f"pure shear step {step}")
        ref = pair.o.phase_ratios(pair.of[0], 2)
        jp.update_phase_ratios_(pr, pair.p, pair.pf[0])
        for name in ("center", "vertex", "Vx", "Vy"):
            assert_bits_equal(ref[name], getattr(pr, name).cpu().numpy(), name)
    for name in ("center", "vertex", "Vx", "Vy"):
        np.testing.assert_allclose(getattr(pr, name).sum(dim=0).cpu().numpy(), 1.0, rtol=1e-12, err_msg=name)


def test_phase_ratios_3d_reference_test_size():
    """test/test_CellArrays.jl:137-186: 31^3 cells, 125/125/125 particles, 5
    random phase ids in every slot; every location's ratios sum to one."""
    g = W.grid((31, 31, 31))
    p = jp.init_particles(jp.CUDABackend, 125, 125, 125, *g["grid_v"])
    assert p.max_xcell == 128  # 125 rounded up to 16 per octant
    gen = torch.Generator(device="cuda").manual_seed(5)
    ph = torch.randint(1, 6, p.index.data.shape, generator=gen, device="cuda").double()
    pr = jp.PhaseRatios(5, p.ni)
    jp.update_phase_ratios_(pr, p, jp.CellArray(ph.contiguous(), p.ni))
    for name in ("center", "vertex", "Vx", "Vy", "Vz", "xy", "yz", "xz"):
        s = getattr(pr, name).sum(dim=0).cpu().numpy()
        np.testing.assert_allclose(s, 1.0, rtol=1e-12, err_msg=name)


def test_wide_cells_rejected_by_the_adjoint():
    """The adjoint keeps 64-bit slot masks; wider cells are refused at the boundary."""
    from justpic_gb300 import adjoint as A

    g = W.grid((8, 8))
    p = jp.init_particles(jp.CUDABackend, 60, 80, 50, *g["grid_v"])
    with pytest.raises(jp.ArgumentError):
        A.slot_ids(p)
