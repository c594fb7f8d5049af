"""Tuple forms of the grid transfers (particle2grid!(F::NTuple, Fp::NTuple,
particles), src/Interpolations/particle_to_grid.jl:70-109, 153-199;
grid2particle!(Fp::NTuple, F::NTuple, particles),
src/Interpolations/grid_to_particle.jl:84-103): the CUDA library's one-call
forms against the oracle's, bit for bit, for 1 to 5 fields (more than four
fields take several launches), on uniform and refined grids in 2D and 3D."""
import numpy as np
import pytest
import torch

from _harness import Pair, W, assert_bits_equal, jp, refined_grid

pytestmark = pytest.mark.gpu


def _fields(g, n):
    N = g["ndim"]
    out = []
    for k in range(n):
        c = tuple(0.3 + 0.1 * k + 0.05 * d for d in range(N))
        out.append(W.gaussian_T(g, center=c, width2=0.02 + 0.01 * k))
    return out


@pytest.mark.parametrize("nf", [1, 2, 3, 5])
@pytest.mark.parametrize("ni,refined", [((14, 11), False), ((9, 12), True), ((6, 5, 7), False), ((5, 4, 6), True)])
def test_tuple_transfers_bit_exact(ni, refined, nf):
    g = refined_grid(ni) if refined else W.grid(ni)
    pair = Pair(g, 24, 48, 12, nfields=nf)
    Fs = _fields(g, nf)
    # grid2particle!, tuple form
    pair.o.grid2particle_n(pair.of, Fs)
    jp.grid2particle_(tuple(pair.pf), tuple(jp.TA("CUDA")(F) for F in Fs), pair.p)
    pair.assert_same("grid2particle! tuple")
    # a step, so particle2grid! sees relocated particles
    V = W.stream_velocity(g) if len(ni) == 2 else W.stream_velocity_3d(g)
    pair.advection("rk2", V, W.cfl_dt(g, V, 0.5))
    pair.move()
    pair.assert_same("move")
    shape = tuple(n + 1 for n in ni)
    Fo = [np.asfortranarray(np.zeros(shape)) for _ in range(nf)]
    pair.o.particle2grid_n(Fo, pair.of)
    Fg = tuple(jp.grid_field(shape) for _ in range(nf))
    jp.particle2grid_(Fg, tuple(pair.pf), pair.p)
    for k in range(nf):
        assert_bits_equal(Fo[k], Fg[k].cpu().numpy(), f"particle2grid! tuple field {k}")


def test_tuple_forms_against_the_scalar_forms():
    """grid2particle!: each field of the tuple form equals the scalar form.
    particle2grid!: in 3D the normalisations agree (wF * inv(w)), so each
    field equals the scalar form; in 2D the scalar form divides (wF / w) and
    the tuple form multiplies by inv(w): at most one rounding apart."""
    for ni in [(12, 10), (5, 6, 4)]:
        g = W.grid(ni)
        p = jp.init_particles(jp.CUDABackend, 24, 48, 12, *g["grid_v"])
        Fs = [jp.TA("CUDA")(F) for F in _fields(g, 3)]
        tup = jp.init_cell_arrays(p, 3)
        one = jp.init_cell_arrays(p, 3)
        jp.grid2particle_(tuple(tup), tuple(Fs), p)
        for k in range(3):
            jp.grid2particle_(one[k], Fs[k], p)
            live = p.index.numpy().astype(bool)
            assert_bits_equal(tup[k].numpy()[live], one[k].numpy()[live], f"g2p field {k}")
        shape = tuple(n + 1 for n in ni)
        Gt = tuple(jp.grid_field(shape) for _ in range(3))
        jp.particle2grid_(Gt, tuple(tup), p)
        for k in range(3):
            Gs = jp.grid_field(shape)
            jp.particle2grid_(Gs, tup[k], p)
            a, b = Gt[k].cpu().numpy(), Gs.cpu().numpy()
            if len(ni) == 3:
                assert_bits_equal(a, b, f"p2g field {k}")
            else:
                assert np.all(np.abs(a - b) <= np.spacing(np.abs(b)))


def test_tuple_grid2particle_skips_nan_coordinates():
    g = W.grid((6, 6))
    pair = Pair(g, 8, 16, 2, nfields=2)
    live = pair.o.index.astype(bool)
    s, c = np.argwhere(live)[3]
    pair.o.coords[0][s, c] = np.nan
    pair.p.coords[0].data[s, c] = float("nan")
    for k in range(2):
        pair.of[k][:] = -1.0
        pair.pf[k].data.fill_(-1.0)
    Fs = _fields(g, 2)
    pair.o.grid2particle_n(pair.of, Fs)
    jp.grid2particle_(tuple(pair.pf), tuple(jp.TA("CUDA")(F) for F in Fs), pair.p)
    pair.assert_same("tuple grid2particle! with a NaN coordinate")
    assert pair.pf[0].numpy()[s, c] == -1.0 and pair.pf[1].numpy()[s, c] == -1.0


def test_tuple_forms_check_their_arguments():
    g = W.grid((4, 4))
    p = jp.init_particles(jp.CUDABackend, 8, 16, 2, *g["grid_v"])
    f = jp.init_cell_arrays(p, 2)
    F = jp.grid_field((5, 5))
    with pytest.raises(jp.ArgumentError):
        jp.particle2grid_((F,), tuple(f), p)
    with pytest.raises(jp.ArgumentError):
        jp.grid2particle_((), (), p)
    torch.cuda.synchronize()
