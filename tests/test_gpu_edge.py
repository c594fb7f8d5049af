"""Edge cases of the hot path against the oracle, bit for bit: an empty
container (injection with no neighbours anywhere), single-cell grids, the
maximum capacity of 1024 slots, particles sitting exactly on cell faces and
vertices (the bisection's ties), and live particles with NaN or infinite
coordinates."""
import warnings

import numpy as np
import pytest
import torch

from _harness import Pair, W, assert_bits_equal, jp

pytestmark = pytest.mark.gpu


def _grid(ni):
    """W.grid, with the ghost-node centre axes written as LinRange(-dx/2, 1 + dx/2, n + 2)
    (test/test_2D.jl:414) so that single-cell axes work too."""
    N = len(ni)
    xv = tuple(jp.LinRange(0.0, 1.0, n + 1) for n in ni)
    dx = tuple(1.0 / n for n in ni)
    xc = tuple(jp.LinRange(dx[d] / 2, 1.0 - dx[d] / 2, ni[d]) for d in range(N))
    ext = tuple(jp.LinRange(-dx[d] / 2, 1.0 + dx[d] / 2, ni[d] + 2) for d in range(N))
    grid_v = tuple(tuple(xv[d] if d == c else ext[d] for d in range(N)) for c in range(N))
    return {"ndim": N, "ni": tuple(ni), "xv": xv, "xc": xc, "dx": dx, "grid_v": grid_v}


def _set_state(pair, X, index):
    for d in range(len(X)):
        pair.o.coords[d][...] = X[d]
        pair.p.coords[d].data.copy_(torch.from_numpy(np.ascontiguousarray(X[d])))
    pair.o.index[...] = index
    pair.p.index.data.copy_(torch.from_numpy(np.ascontiguousarray(index.astype(np.uint8))))


def _step_all(pair, g, V, dt, steps=2):
    for step in range(steps):
        pair.advection("rk2", V, dt)
        pair.assert_same(f"advection {step}")
        pair.move()
        pair.assert_same(f"move {step}")
        with warnings.catch_warnings():
            warnings.simplefilter("ignore", RuntimeWarning)
            pair.inject()
        pair.assert_same(f"inject {step}")
    if pair.of:
        Fo, Fg = pair.p2g(0)
        assert_bits_equal(Fo, Fg, "particle2grid!")


@pytest.mark.parametrize("ni", [(6, 5), (3, 4, 3)])
def test_empty_container_is_reseeded_like_the_oracle(ni):
    g = W.grid(ni)
    pair = Pair(g, 24, 48, 12, nfields=1)
    shape = pair.o.index.shape
    _set_state(pair, [np.full(shape, np.nan) for _ in ni], np.zeros(shape, dtype=np.uint8))
    V = W.stream_velocity(g) if len(ni) == 2 else W.stream_velocity_3d(g)
    with warnings.catch_warnings():
        warnings.simplefilter("ignore", RuntimeWarning)  # injected particles find no neighbour to copy from
        pair.inject()
    pair.assert_same("inject into an empty container")
    assert pair.o.index.sum() > 0
    _step_all(pair, g, V, W.cfl_dt(g, V, 0.5))


@pytest.mark.parametrize("ni", [(1, 1), (1, 1, 1), (1, 3)])
def test_single_cell_axes(ni):
    """Vector grids (the reference's range grids have no centre spacing on a
    single-cell axis: getindex(xci, 2) fails, particles_utils.jl:137)."""
    g = _grid(ni)
    with pytest.raises(jp.ArgumentError):
        jp.init_particles(jp.CUDABackend, 8, 16, 4, *g["grid_v"])
    g["grid_v"] = tuple(tuple(np.asarray(x, dtype=np.float64) for x in comp) for comp in g["grid_v"])
    pair = Pair(g, 8, 16, 4, nfields=1)
    V = W.rotation_velocity(g) if len(ni) == 2 else W.stream_velocity_3d(g)
    pair.g2p(0, W.linear_T(g, 0))
    pair.assert_same("grid2particle!")
    _step_all(pair, g, V, 0.2 * W.cfl_dt(g, V), steps=3)


def test_maximum_capacity():
    g = W.grid((3, 2))
    pair = Pair(g, 1000, 1024, 900, nfields=1)
    assert pair.p.max_xcell == 1024
    pair.g2p(0, W.linear_T(g, 1))
    V = W.stream_velocity(g)
    _step_all(pair, g, V, 0.5 * W.cfl_dt(g, V))


@pytest.mark.parametrize("ni", [(8, 6), (4, 3, 5)])
def test_particles_on_faces_and_vertices(ni):
    """Positions exactly on vertex-grid lines: isincell (strict) calls them
    movers and the bisection's closed interval test meets ties."""
    g = W.grid(ni)
    pair = Pair(g, 8, 16, 4, nfields=1)
    rng = np.random.default_rng(21)
    X = [c.copy() for c in pair.o.coords]
    live = pair.o.index.astype(bool)
    for d in range(len(ni)):
        xv = np.asarray(g["xv"][d])
        snap = rng.random(X[d].shape) < 0.4
        k = rng.integers(0, len(xv), X[d].shape)
        X[d] = np.where(live & snap, xv[k], X[d])  # some on their own faces, some on far lines
    _set_state(pair, X, pair.o.index.copy())
    pair.g2p(0, W.linear_T(g, 0))
    pair.assert_same("grid2particle! on faces")
    V = W.stream_velocity(g) if len(ni) == 2 else W.stream_velocity_3d(g)
    Vz = tuple(np.asfortranarray(0.0 * v) for v in V)  # no motion: move sees the snapped positions
    pair.advection("euler", Vz, 1.0)
    pair.move()
    pair.assert_same("move from faces")
    _step_all(pair, g, V, 0.5 * W.cfl_dt(g, V))


@pytest.mark.parametrize("ni", [(8, 6), (4, 3, 5)])
def test_nan_and_infinite_positions(ni):
    g = W.grid(ni)
    pair = Pair(g, 12, 24, 6, nfields=1)
    X = [c.copy() for c in pair.o.coords]
    live = np.argwhere(pair.o.index.astype(bool))
    for n, (s, c) in enumerate(live[::7]):
        X[n % len(ni)][s, c] = [np.nan, np.inf, -np.inf][n % 3]
    _set_state(pair, X, pair.o.index.copy())
    V = W.stream_velocity(g) if len(ni) == 2 else W.stream_velocity_3d(g)
    pair.g2p(0, W.linear_T(g, 0))
    pair.assert_same("grid2particle! with NaN/Inf positions")
    Fo, Fg = pair.p2g(0)
    assert_bits_equal(Fo, Fg, "particle2grid! with NaN/Inf positions")
    _step_all(pair, g, V, 0.5 * W.cfl_dt(g, V))


@pytest.mark.parametrize("ni", [(8, 8), (4, 4, 3)])
def test_inject_nearest_ties_take_the_first_in_order(ni):
    """Exact distance ties in the nearest-neighbour search of inject_particles!
    (index_min_distance, injection.jl:330-393): in every other cell all 40 live
    particles share one position (so slots s and s + 32, which the search gives
    to the same lane, tie too) and carry distinct field values; the other cells
    are empty and inject. The field a new particle copies shows which of the
    tied particles won: the first in the reference's order, on both sides."""
    g = _grid(ni)
    N = len(ni)
    pair = Pair(g, 24, 48, 12, nfields=1)
    M, nc = pair.o.index.shape
    rng = np.random.default_rng(11)
    X = [np.full((M, nc), np.nan) for _ in range(N)]
    index = np.zeros((M, nc), dtype=np.uint8)
    for c in range(nc):
        I = np.unravel_index(c, ni, order="F")
        if sum(I) % 2:
            continue
        index[:40, c] = 1
        for d in range(N):
            X[d][:40, c] = (I[d] + rng.uniform(0.05, 0.95)) / ni[d]
    _set_state(pair, X, index)
    F = np.where(index.astype(bool), rng.random((M, nc)), np.nan)
    pair.of[0][...] = F
    pair.pf[0].data.copy_(torch.from_numpy(np.ascontiguousarray(F)))
    pair.assert_same("before inject")
    for call in range(2):
        pair.inject()
        pair.assert_same(f"inject {call}")
    assert pair.p.index.numpy().sum() > index.sum()  # the empty cells were reseeded
