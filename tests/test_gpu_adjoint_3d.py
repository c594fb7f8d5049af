"""Adjoint of the grid transfers in 3D (particle2grid! and grid2particle!) on
a uniform and a refined grid.

  * particle2grid!: against forward-mode derivatives (dual numbers) through
    the CPU oracle, whose forward is bit-identical to the library's
    (test_gpu_parity.py): single-slot tangents of the field and of each
    coordinate, and one random tangent of all of them, to 1e-9 relative
    (floor: 1e-9 of the largest gradient checked);
  * grid2particle!: linear in the field and in each coordinate along its
    axis, so central differences carry no truncation error: relative 1e-6
    of the difference, floor 1e-6 of the largest gradient checked
    (test_gpu_adjoint.py's rule); and the transpose identity.
"""
import numpy as np
import pytest
import torch

from _harness import Pair, W, assert_bits_equal, jp, refined_grid
from justpic_gb300 import adjoint as A
from test_gpu_adjoint import _close, _pick_nodes

pytestmark = pytest.mark.gpu

GRIDS = [pytest.param(False, id="uniform"), pytest.param(True, id="refined")]


def _setup(refined, ni=(7, 6, 5), seed=0x4A50):
    g = refined_grid(ni) if refined else W.grid(ni)
    p = jp.init_particles(jp.CUDABackend, 12, 24, 6, *g["grid_v"], seed=seed)
    return g, p


def _sample(p, rng, n=10):
    live = p.index.numpy().astype(bool)
    slots = np.argwhere(live)
    return live, slots[rng.choice(len(slots), n, replace=False)]


@pytest.mark.parametrize("refined", GRIDS)
def test_particle2grid_vjp_3d_matches_oracle_jvp(refined):
    g = refined_grid((7, 6, 5)) if refined else W.grid((7, 6, 5))
    pr = Pair(g, 12, 24, 6, nfields=1)
    T = W.gaussian_T(g, width2=0.05)
    pr.g2p(0, T)
    pr.assert_same("grid2particle!")
    p, o, Tp = pr.p, pr.o, pr.pf[0]
    shape = tuple(n + 1 for n in p.ni)
    rng = np.random.default_rng(5)
    cw = rng.standard_normal(shape)
    F = jp.grid_field(shape)
    Wt = jp.grid_field(shape)
    A.particle2grid_with_weights_(F, Wt, Tp, p)
    Fo, _ = pr.p2g(0)
    assert_bits_equal(Fo, F.cpu().numpy(), "particle2grid_with_weights")
    gTp = A._like(p)
    gX = tuple(A._like(p) for _ in range(3))
    A.particle2grid_vjp_(gTp, gX, jp.TA("CUDA")(cw), F, Wt, Tp, p)
    gT, gx = gTp.numpy(), [x.numpy() for x in gX]
    live = o.index.astype(bool)
    Tho = pr.of[0]

    def jvp(dT, dX):
        Fj = np.asfortranarray(np.zeros(shape))
        dF = np.asfortranarray(np.zeros(shape))
        o.particle2grid_jvp(Fj, dF, Tho, dT, [np.ascontiguousarray(x) for x in dX])
        return float(np.sum(cw * dF))

    zero = np.zeros(live.shape)
    slots = np.argwhere(live)
    sel = slots[rng.choice(len(slots), 8, replace=False)]
    adj, ref = [], []
    for s_, c in sel:
        e = np.zeros(live.shape)
        e[s_, c] = 1.0
        ref.append(jvp(e, [zero, zero, zero]))
        adj.append(gT[s_, c])
        for d in range(3):
            dX = [zero, zero, zero]
            dX[d] = e
            ref.append(jvp(zero, dX))
            adj.append(gx[d][s_, c])
    dT = np.where(live, rng.standard_normal(live.shape), 0.0)
    dX = [np.where(live, rng.standard_normal(live.shape), 0.0) for _ in range(3)]
    ref.append(jvp(dT, dX))
    adj.append(float(np.sum(gT[live] * dT[live]) + sum(np.sum(gx[d][live] * dX[d][live]) for d in range(3))))
    adj, ref = np.array(adj), np.array(ref)
    floor = np.max(np.abs(ref))
    assert np.all(np.abs(adj - ref) <= 1e-9 * np.maximum(np.abs(ref), floor)), (adj, ref)


@pytest.mark.parametrize("refined", GRIDS)
def test_grid2particle_vjp_3d_matches_fd(refined):
    g, p = _setup(refined)
    T = W.gaussian_T(g, width2=0.05)
    Td = jp.TA("CUDA")(T)
    (Tp,) = jp.init_cell_arrays(p, 1)
    rng = np.random.default_rng(6)
    live, sel = _sample(p, rng)
    cp = np.where(live, rng.standard_normal(live.shape), 0.0)

    def forward(F=Td):
        jp.grid2particle_(Tp, F, p)
        return Tp.numpy()

    gF = jp.grid_field(T.shape)
    gX = tuple(A._like(p) for _ in range(3))
    A.grid2particle_vjp_(gF, gX, jp.CellArray(torch.from_numpy(cp).cuda(), p.ni), Td, p)
    h = 1e-6
    adj, fd = [], []
    gFh = gF.cpu().numpy()
    for node in _pick_nodes(T.shape, 16, rng):
        Tpl, Tmi = T.copy(order="F"), T.copy(order="F")
        Tpl[node] += h
        Tmi[node] -= h
        fd.append(np.sum((forward(jp.TA("CUDA")(Tpl)) - forward(jp.TA("CUDA")(Tmi)))[live] * cp[live]) / (2 * h))
        adj.append(gFh[node])
    _close(adj, fd, "dL/dF through grid2particle! (3D)")
    hx = 1e-6
    for d in range(3):
        adj, fd = [], []
        for s, c in sel:
            x0 = float(p.coords[d].data[s, c])
            p.coords[d].data[s, c] = x0 + hx
            fp = forward()[s, c]
            p.coords[d].data[s, c] = x0 - hx
            fm = forward()[s, c]
            p.coords[d].data[s, c] = x0
            fd.append((fp - fm) * cp[s, c] / (2 * hx))
            adj.append(float(gX[d].data[s, c]))
        _close(adj, fd, f"dL/dX{'xyz'[d]} through grid2particle! (3D)")


def test_grid2particle_vjp_3d_is_the_transpose():
    """<gFp, G F> = <G^T gFp, F> for the linear map G = grid2particle! at fixed
    positions, on random F and gFp (the gather order makes both sides exact
    up to summation round-off)."""
    g, p = _setup(False, ni=(9, 8, 7))
    rng = np.random.default_rng(8)
    shape = tuple(n + 1 for n in p.ni)
    F = rng.standard_normal(shape)
    (Fp,) = jp.init_cell_arrays(p, 1)
    jp.grid2particle_(Fp, jp.TA("CUDA")(F), p)
    live = p.index.numpy().astype(bool)
    cp = np.where(live, rng.standard_normal(live.shape), 0.0)
    gF = jp.grid_field(shape)
    A.grid2particle_vjp_(gF, None, jp.CellArray(torch.from_numpy(cp).cuda(), p.ni), None, p)
    lhs = float(np.sum(Fp.numpy()[live] * cp[live]))
    rhs = float(np.sum(gF.cpu().numpy() * F))
    assert abs(lhs - rhs) <= 1e-11 * max(abs(lhs), 1.0), (lhs, rhs)


def test_autograd_transfers_3d():
    """Particle2Grid(Grid2Particle(F)) as autograd nodes in 3D: the gradient of
    sum(c * F') against finite differences on a few vertices."""
    g, p = _setup(False)
    rng = np.random.default_rng(9)
    shape = tuple(n + 1 for n in p.ni)
    F0 = torch.from_numpy(W.gaussian_T(g, width2=0.05).copy(order="F")).cuda()
    c = torch.from_numpy(rng.standard_normal(shape)).cuda()

    def field(F):
        return A.Particle2Grid.apply(A.Grid2Particle.apply(F, p), p)

    F = F0.clone().requires_grad_(True)
    (field(F) * c).sum().backward()
    grad = F.grad.cpu().numpy()
    h = 1e-6
    adj, fd = [], []
    for node in _pick_nodes(shape, 12, rng):
        Fpl, Fmi = F0.clone(), F0.clone()
        Fpl[node] += h
        Fmi[node] -= h
        with torch.no_grad():
            fd.append(float(((field(Fpl) - field(Fmi)) * c).sum()) / (2 * h))
        adj.append(grad[node])
    _close(adj, fd, "d sum(c * P2G(G2P(F))) / dF (3D)")
