"""GPU parity: every hot-path call of the CUDA library against the CPU oracle
on the same seeded inputs, through the C ABI. Integer/index results must match
exactly; the FP64 results are compared bit for bit as well (the kernels keep
the oracle's operation order and its fma sites), which is stricter than the
1e-12 relative tolerance of the contract."""
import numpy as np
import pytest

from _harness import METHODS, Pair, W, assert_bits_equal, jp, refined_grid

pytestmark = pytest.mark.gpu



def _setup(ni, nxcell=24, max_xcell=48, min_xcell=12, nfields=1, refined=False, seed=0x4A50):
    g = refined_grid(ni) if refined else W.grid(ni)
    return Pair(g, nxcell, max_xcell, min_xcell, seed=seed, nfields=nfields), g


@pytest.mark.parametrize("ni", [(8, 8), (13, 7), (4, 5, 6)])
def test_init_particles_bit_exact(ni):
    pair, _ = _setup(ni)
    pair.assert_same("init")
    assert pair.p.nxcell == pair.o.nxcell and pair.p.max_xcell == pair.o.max_xcell


@pytest.mark.parametrize("method", list(METHODS))
@pytest.mark.parametrize("ni", [(16, 16), (9, 14), (6, 5, 7)])
def test_advection_bit_exact(method, ni):
    pair, g = _setup(ni)
    V = W.stream_velocity(g) if len(ni) == 2 else W.stream_velocity_3d(g)
    dt = W.cfl_dt(g, V, 0.5)
    assert pair.advection(method, V, dt) == 0
    pair.assert_same(f"advection {method}")


@pytest.mark.parametrize("interp", ["linp", "mqs"])
@pytest.mark.parametrize("method", ["euler", "rk2_23", "rk4"])
@pytest.mark.parametrize("ni,refined", [((16, 16), False), ((11, 9), True), ((6, 5, 7), False),
                                         ((5, 6, 4), True)])
def test_advection_linp_mqs_bit_exact(interp, method, ni, refined):
    """advection_LinP! / advection_MQS! against the oracle, then a full step
    (move_particles! + inject_particles!) so the next advection starts from
    relocated particles."""
    pair, g = _setup(ni, refined=refined)
    rng = np.random.default_rng(8)
    V = W.stream_velocity(g) if len(ni) == 2 else W.stream_velocity_3d(g)
    V = tuple(np.asfortranarray(v * (1.0 + 0.2 * rng.standard_normal(v.shape))) for v in V)
    dt = W.cfl_dt(g, V, 0.5)
    for step in range(2):
        assert pair.advection(method, V, dt, interp) == 0
        pair.assert_same(f"advection {interp} {method} step {step}")
        pair.move()
        pair.inject()
        pair.assert_same(f"move+inject after {interp} step {step}")


def test_advection_outside_limits_gives_inf():
    # a step far beyond the velocity grid sends particles to Inf (advection.jl:104-108)
    pair, g = _setup((8, 8))
    V = W.stream_velocity(g)
    pair.advection("rk2", V, 50 * W.cfl_dt(g, V))
    pair.assert_same("advection, huge dt")
    assert np.isinf(pair.p.coords[0].numpy()[pair.p.index.numpy().astype(bool)]).any()


@pytest.mark.parametrize("ni,refined", [((16, 16), False), ((11, 9), True), ((6, 6, 6), False),
                                         ((5, 7, 4), True)])
def test_move_particles_bit_exact(ni, refined):
    pair, g = _setup(ni, refined=refined)
    V = W.stream_velocity(g) if len(ni) == 2 else W.stream_velocity_3d(g)
    T = W.linear_T(g, 1)
    pair.g2p(0, T)
    dt = W.cfl_dt(g, V)
    for step in range(4):
        pair.advection("rk2", V, dt)
        assert pair.move() == 0
        pair.assert_same(f"move step {step}")


@pytest.mark.parametrize("ni", [(12, 10), (5, 6, 4)])
def test_move_after_scratch_grows_bit_exact(ni):
    """The colour passes are captured once per container into a CUDA graph over
    the container's move scratch; a move with more particle fields reallocates
    that scratch, and the passes must be captured again."""
    g = W.grid(ni)
    pair = Pair(g, 24, 48, 12, nfields=4)
    V = W.stream_velocity(g) if len(ni) == 2 else W.stream_velocity_3d(g)
    dt = W.cfl_dt(g, V)
    for k in range(4):
        pair.g2p(k, W.linear_T(g, k % len(ni)))
    for step, nf in enumerate([0, 1, 4, 1, 0]):  # no fields, then more (the scratch grows), then fewer
        pair.advection("rk2", V, dt)
        pair.o.move_particles(pair.of[:nf])
        jp.move_particles_(pair.p, tuple(pair.pf[:nf]))
        pair.assert_same(f"move step {step} with {nf} fields")


def test_move_full_cells_drop_like_reference():
    # tiny capacity: relocation overflows, the first-free-slot-after-starting_point
    # rule decides who is dropped (move_safe.jl:115-117)
    pair, g = _setup((10, 10), nxcell=8, max_xcell=9, min_xcell=2)
    V = W.stream_velocity(g)
    pair.g2p(0, W.linear_T(g, 0))
    dt = W.cfl_dt(g, V)
    full = 0
    for step in range(6):
        pair.advection("rk2_23", V, dt)
        before = int(pair.p.index.numpy().sum())
        jp.move_counts(pair.p, clear=True)
        pair.move()
        pair.assert_same(f"overflow move step {step}")
        counts = jp.move_counts(pair.p)
        # every particle the move removed is counted once
        assert before - int(pair.p.index.numpy().sum()) == sum(counts.values()), counts
        full += counts["no_free_slot"]
    assert pair.p.index.numpy().sum() < pair.o.ncells * pair.o.nxcell  # particles were dropped
    assert full > 0


@pytest.mark.parametrize("ni", [(16, 16), (7, 6, 5)])
def test_move_counts_name_every_removed_particle(ni):
    """A step of three CFL widths: some particles leave the domain, some move
    more than one cell; move_counts tells them apart like a host check of the
    positions does, and the move still matches the oracle."""
    pair, g = _setup(ni)
    N = len(ni)
    V = W.stream_velocity(g) if N == 2 else W.stream_velocity_3d(g)
    pair.advection("rk2", V, 3 * W.cfl_dt(g, V))
    idx = pair.p.index.numpy().astype(bool)
    X = [pair.p.coords[d].numpy() for d in range(N)]
    cells = np.arange(idx.shape[1])
    inside = np.ones_like(idx)
    far = np.zeros_like(idx)
    stride = 1
    for d in range(N):
        I = (cells // stride) % ni[d]
        stride *= ni[d]
        with np.errstate(invalid="ignore"):
            inside &= (X[d] > 0.0) & (X[d] < 1.0)
            T = np.floor(np.where(np.isfinite(X[d]), X[d], 0.0) * ni[d])
        far |= np.abs(T - I[None, :]) > 1
    jp.move_counts(pair.p, clear=True)
    with pytest.warns(RuntimeWarning):
        pair.move()
    pair.assert_same("move after a long step")
    counts = jp.move_counts(pair.p)
    assert counts["left_domain"] == int((idx & ~inside).sum())
    assert counts["moved_too_far"] == int((idx & inside & far).sum()) > 0


@pytest.mark.parametrize("ni", [(12, 12), (5, 6, 4)])
def test_inject_particles_bit_exact(ni):
    pair, g = _setup(ni, nxcell=8 if len(ni) == 2 else 8, max_xcell=24, min_xcell=8)
    T = W.gaussian_T(g)
    pair.g2p(0, T)
    # empty a block of cells on both sides identically, then reinject
    idx = pair.o.index
    rng = np.random.default_rng(3)
    kill = rng.random(idx.shape) < 0.6
    kill &= idx.astype(bool)
    import torch
    for d in range(pair.o.ndim):
        pair.o.coords[d][kill] = np.nan
        pair.p.coords[d].data[torch.from_numpy(kill).cuda()] = float("nan")
    pair.of[0][kill] = np.nan
    pair.pf[0].data[torch.from_numpy(kill).cuda()] = float("nan")
    idx[kill] = 0
    pair.p.index.data[torch.from_numpy(kill).cuda()] = 0
    pair.assert_same("before inject")
    pair.inject()
    pair.assert_same("inject")
    pair.inject()  # second call uses the next RNG counter
    pair.assert_same("inject twice")


@pytest.mark.parametrize("ni,min_xcell", [((6, 5), 200), ((4, 3, 3), 500)])
def test_inject_many_per_quadrant_bit_exact(ni, min_xcell):
    """A min_xcell above max_xcell (the reference does not bound it) makes the first
    quadrant take every free slot of a cell: more new particles than one batch of
    the warp's draws holds (16 in 2D, 10 in 3D)."""
    pair, g = _setup(ni, nxcell=4 if len(ni) == 2 else 8, max_xcell=64, min_xcell=min_xcell)
    pair.g2p(0, W.gaussian_T(g))
    pair.assert_same("before inject")
    pair.inject()
    pair.assert_same("inject")
    live = pair.o.index.astype(bool)
    assert live.sum(axis=0).min() == 64  # every free slot was filled
    pair.inject()
    pair.assert_same("inject twice")


@pytest.mark.parametrize("ni,refined", [((8, 8), False), ((10, 7), True), ((4, 4, 4), False), ((5, 3, 4), True)])
def test_grid2particle_bit_exact(ni, refined):
    pair, g = _setup(ni, refined=refined)
    T = W.gaussian_T(g)
    pair.g2p(0, T)
    pair.assert_same("g2p")


def test_grid2particle_linear_field_reproduces_coordinate():
    # test/test_interpolation_kernels.jl:86-94
    g = W.grid((4, 4))
    p = jp.init_particles(jp.CUDABackend, 5, 5, 1, *g["grid_v"])
    pT, = jp.init_cell_arrays(p, 1)
    jp.grid2particle_(pT, jp.TA("CUDA")(W.linear_T(g, 1)), p)
    live = p.index.numpy().astype(bool)
    np.testing.assert_allclose(pT.numpy()[live], p.coords[1].numpy()[live], rtol=1e-14, atol=1e-15)


@pytest.mark.parametrize("ni,refined", [((8, 8), False), ((10, 7), True), ((4, 4, 4), False), ((5, 3, 4), True)])
def test_particle2grid_bit_exact(ni, refined):
    pair, g = _setup(ni, refined=refined)
    pair.g2p(0, W.gaussian_T(g))
    Fo, Fg = pair.p2g(0)
    assert_bits_equal(Fo, Fg, "p2g")


def test_particle2grid_error_small():
    # test/test_interpolation_kernels.jl:100-105: norm(T2 - T)/length(T) < 0.1
    g = W.grid((4, 4))
    p = jp.init_particles(jp.CUDABackend, 5, 5, 1, *g["grid_v"])
    pT, = jp.init_cell_arrays(p, 1)
    T = W.linear_T(g, 1)
    jp.grid2particle_(pT, jp.TA("CUDA")(T), p)
    T2 = jp.grid_field(T.shape)
    jp.particle2grid_(T2, pT, p)
    assert np.linalg.norm(T2.cpu().numpy() - T) / T.size < 0.1


@pytest.mark.parametrize("ndim", [2, 3])
def test_miniapp_steps_bit_exact(ndim):
    """The reference's miniapp loop (test/test_2D.jl:516-524) for several steps."""
    ni = (24, 24) if ndim == 2 else (8, 8, 8)
    pair, g = _setup(ni, nxcell=25 if ndim == 2 else 24, max_xcell=50 if ndim == 2 else 48,
                     min_xcell=10 if ndim == 2 else 12)
    V = W.stream_velocity(g) if ndim == 2 else W.stream_velocity_3d(g)
    T = W.linear_T(g, 1)
    dt = W.cfl_dt(g, V, 0.5)
    pair.g2p(0, T)
    for it in range(10):
        Fo, Fg = pair.p2g(0)
        assert_bits_equal(Fo, Fg, f"p2g it {it}")
        pair.advection("rk2_23", V, dt)
        pair.move()
        pair.inject()
        pair.g2p(0, Fo)
        pair.assert_same(f"miniapp it {it}")


def test_advection_miniapp_conserves_like_reference():
    """advection_test_2D (test/test_2D.jl:482-538): relative drift of sum(T) < 1e-2."""
    g = W.grid((64, 64))
    p = jp.init_particles(jp.CUDABackend, 25, 50, 10, *g["grid_v"])
    pT, = jp.init_cell_arrays(p, 1)
    Vx, Vy = W.stream_velocity(g)
    V = (jp.TA("CUDA")(Vx), jp.TA("CUDA")(Vy))
    T = jp.TA("CUDA")(W.linear_T(g, 1))
    dt = W.cfl_dt(g, (Vx, Vy), 0.5)
    jp.grid2particle_(pT, T, p)
    sumT = float(T.sum())
    for _ in range(25):
        jp.particle2grid_(T, pT, p)
        jp.advection_(p, jp.RungeKutta2(2 / 3), V, dt)
        jp.move_particles_(p, (pT,))
        jp.inject_particles_(p, (pT,))
        jp.grid2particle_(pT, T, p)
    assert abs(sumT - float(T.sum())) / sumT < 1e-2


def test_bad_arguments_raise():
    g = W.grid((4, 4))
    p = jp.init_particles(jp.CUDABackend, 4, 8, 2, *g["grid_v"])
    with pytest.raises(jp.ArgumentError):
        jp.advection_(p, jp.RungeKutta2(), (jp.grid_field((3, 3)), jp.grid_field((3, 3))), 0.1)
    with pytest.raises(jp.ArgumentError):
        jp.grid2particle_(jp.init_cell_arrays(p, 1)[0], jp.grid_field((4, 4)), p)
