"""Adjoint of the FP64 path (2D) against central finite differences of the
forward path and against forward-mode derivatives (dual numbers) through
the CPU oracle.

The forward path is bit-identical to the CPU oracle (test_gpu_parity.py), and
test_fd_is_oracle_fd checks that on the perturbed runs too, so every finite
difference below is also a finite difference through the oracle.

Tolerances: finite differences, relative 1e-6 of the difference with a floor
of 1e-6 of the largest checked gradient (nodes no particle reaches have a
zero gradient on both sides); differences are formed per particle / per
vertex before any reduction, so their round-off stays below it. Dual numbers
through the oracle carry no truncation or cancellation error, so the adjoint
must match them to 1e-9 relative (floor: 1e-9 of the largest gradient).
"""
import numpy as np
import pytest
import torch

from _harness import METHODS, O, Pair, W, jp
from justpic_gb300 import adjoint as A

pytestmark = pytest.mark.gpu

RTOL = 1e-6


def _close(adj, fd, what):
    adj, fd = np.asarray(adj, dtype=np.float64), np.asarray(fd, dtype=np.float64)
    scale = max(np.max(np.abs(fd)), 1e-300)
    err = np.abs(adj - fd)
    bad = err > RTOL * np.maximum(np.abs(fd), scale)
    assert not bad.any(), (f"{what}: {bad.sum()} of {len(fd)} differ; worst rel "
                           f"{np.max(err / np.maximum(np.abs(fd), scale)):.3e}\nadj={adj[bad][:4]}\nfd={fd[bad][:4]}")


def _setup(ni=(16, 16), nxcell=16, max_xcell=32, min_xcell=8, seed=0x4A50):
    g = W.grid(ni)
    p = jp.init_particles(jp.CUDABackend, nxcell, max_xcell, min_xcell, *g["grid_v"], seed=seed)
    Vh = W.perturbed_stream_velocity(g)
    return g, p, Vh


def _dev(Vh):
    return tuple(jp.TA("CUDA")(v) for v in Vh)


def _set_coords(p, X):
    for c, x in zip(p.coords, X):
        c.data.copy_(x)


def _pick_nodes(shape, n, rng):
    flat = rng.choice(int(np.prod(shape)), size=n, replace=False)
    return [np.unravel_index(f, shape, order="F") for f in flat]


# --------------------------------------------------------------- one step
@pytest.mark.parametrize("method", ["euler", "rk2", "rk2_23", "rk4"])
def test_advection_vjp_matches_fd(method):
    g, p, Vh = _setup()
    _, pm, _ = METHODS[method]
    V = _dev(Vh)
    dt = W.cfl_dt(g, Vh, 0.8)
    X0 = tuple(c.data.clone() for c in p.coords)
    live = p.index.data.bool()
    rng = np.random.default_rng(1)
    lam_np = [np.where(live.cpu().numpy(), rng.standard_normal(live.shape), 0.0) for _ in range(2)]

    def forward(Vd, X=X0):
        _set_coords(p, X)
        jp.advection_(p, pm, Vd, dt)
        return [c.data.cpu().numpy().copy() for c in p.coords]

    # A particle whose stage point leaves a velocity grid's limits is sent to Inf
    # (src/Particles/Advection/advection.jl:104-108) whatever the perturbation: it
    # carries no derivative and the adjoint gives it none. Such particles (and the
    # empty slots, NaN) are left out of the finite differences explicitly.
    base = forward(V)
    on_grid = live.cpu().numpy() & np.isfinite(base[0]) & np.isfinite(base[1])
    lam_np = [np.where(on_grid, l, 0.0) for l in lam_np]
    lam = [torch.from_numpy(l).cuda() for l in lam_np]
    gV = tuple(jp.grid_field(v.shape) for v in Vh)
    A.advection_vjp_(p, pm, V, dt, X0, A._Idx(p.index.data), lam, gV)
    h = 1e-6
    for c in range(2):
        adj, fd = [], []
        for node in _pick_nodes(Vh[c].shape, 16, rng):
            Vp = [v.copy(order="F") for v in Vh]
            Vm = [v.copy(order="F") for v in Vh]
            Vp[c][node] += h
            Vm[c][node] -= h
            xp, xm = forward(_dev(Vp)), forward(_dev(Vm))
            assert all(np.all(np.isfinite(x[d][on_grid])) for x in (xp, xm) for d in range(2))
            fd.append(sum(np.sum((xp[d][on_grid] - xm[d][on_grid]) * lam_np[d][on_grid]) for d in range(2)) / (2 * h))
            adj.append(gV[c].cpu().numpy()[node])
        _close(adj, fd, f"{method} dL/dV{'xy'[c]}")
    # positions
    hx = 1e-9
    slots = np.argwhere(on_grid)
    sel = slots[rng.choice(len(slots), 12, replace=False)]
    lam0 = [l.cpu().numpy() for l in lam]
    for d in range(2):
        adj, fd = [], []
        for s, cell in sel:
            Xp = [x.clone() for x in X0]
            Xm = [x.clone() for x in X0]
            Xp[d][s, cell] += hx
            Xm[d][s, cell] -= hx
            xp, xm = forward(V, Xp), forward(V, Xm)
            fd.append(sum((xp[e][s, cell] - xm[e][s, cell]) * lam_np[e][s, cell] for e in range(2)) / (2 * hx))
            adj.append(lam0[d][s, cell])
        _close(adj, fd, f"{method} dL/dX{'xy'[d]}")


def test_advection_vjp_window_error():
    # a dt far above the CFL limit puts stage points outside the gather window
    g, p, Vh = _setup((8, 8))
    V = _dev(Vh)
    dt = 2.5 * W.cfl_dt(g, Vh)
    lam = [torch.ones_like(c.data) for c in p.coords]
    gV = tuple(jp.grid_field(v.shape) for v in Vh)
    X0 = tuple(c.data.clone() for c in p.coords)
    with pytest.raises(jp.JustPICError, match="window"):
        A.advection_vjp_(p, jp.RungeKutta2(), V, dt, X0, A._Idx(p.index.data), lam, gV)


@pytest.mark.parametrize("method", ["euler", "rk2", "rk2_23", "rk4"])
@pytest.mark.parametrize("dt_factor", [0.5, 0.9])
def test_recorded_advection_and_vjp_match(method, dt_factor):
    """jp_advection_record moves particles exactly like advection! and its
    recorded VJP returns exactly what the replaying VJP returns."""
    _, pm, alpha = METHODS[method]
    g, p, Vh = _setup((12, 10))
    V = _dev(Vh)
    dt = dt_factor * W.cfl_dt(g, Vh)
    X0 = tuple(c.data.clone() for c in p.coords)
    idx0 = p.index.data.clone()
    jp.advection_(p, pm, V, dt)
    X1 = tuple(c.data.clone() for c in p.coords)
    _set_coords(p, X0)
    rec = A.record_buffer(p, pm)
    A.advection_record_(p, pm, V, dt, rec)
    for d in range(2):
        assert torch.equal(torch.nan_to_num(p.coords[d].data, nan=-7.0), torch.nan_to_num(X1[d], nan=-7.0))
    rng = np.random.default_rng(3)
    lam0 = [torch.from_numpy(rng.standard_normal(tuple(c.data.shape))).cuda() for c in p.coords]
    la = [l.clone() for l in lam0]
    lb = [l.clone() for l in lam0]
    ga = tuple(jp.grid_field(v.shape) for v in Vh)
    gb = tuple(jp.grid_field(v.shape) for v in Vh)
    A.advection_vjp_(p, pm, V, dt, X0, A._Idx(idx0), la, ga)
    A.advection_vjp_recorded_(p, pm, dt, rec, A._Idx(idx0), lb, gb)
    live = idx0.bool()
    for d in range(2):
        assert torch.equal(la[d][live], lb[d][live])
        assert torch.equal(ga[d], gb[d])


def test_recorded_advection_sends_far_particles_to_inf_like_advection():
    g, p, Vh = _setup((8, 8))
    V = _dev(Vh)
    X0 = tuple(c.data.clone() for c in p.coords)
    dt = 0.02 * W.cfl_dt(g, Vh)
    # particles placed outside the velocity grids get Inf velocities (advection.jl:104-108)
    bad = tuple(x.clone() for x in X0)
    bad[0][0, :8] = 5.0
    _set_coords(p, bad)
    jp.advection_(p, jp.RungeKutta2(), V, dt)
    X1 = tuple(c.data.clone() for c in p.coords)
    _set_coords(p, bad)
    A.advection_record_(p, jp.RungeKutta2(), V, dt, A.record_buffer(p, jp.RungeKutta2()))
    for d in range(2):
        assert torch.equal(torch.nan_to_num(p.coords[d].data, nan=-7.0), torch.nan_to_num(X1[d], nan=-7.0))
    assert torch.isinf(p.coords[0].data[0, :8]).all()


# ------------------------------------------------------ interpolations
def test_particle2grid_vjp_matches_fd():
    g, p, _ = _setup()
    T = W.gaussian_T(g)
    (Tp,) = jp.init_cell_arrays(p, 1)
    jp.grid2particle_(Tp, jp.TA("CUDA")(T), p)
    shape = tuple(n + 1 for n in p.ni)
    rng = np.random.default_rng(2)
    cw = rng.standard_normal(shape)

    def forward():
        F = jp.grid_field(shape)
        jp.particle2grid_(F, Tp, p)
        return F.cpu().numpy()

    F = jp.grid_field(shape)
    Wt = jp.grid_field(shape)
    A.particle2grid_with_weights_(F, Wt, Tp, p)
    assert np.array_equal(F.cpu().numpy(), forward())  # same kernel, same sums
    gTp = A._like(p)
    gX = tuple(A._like(p) for _ in range(2))
    A.particle2grid_vjp_(gTp, gX, jp.TA("CUDA")(cw), F, Wt, Tp, p)
    live = p.index.numpy().astype(bool)
    slots = np.argwhere(live)
    sel = slots[rng.choice(len(slots), 12, replace=False)]
    h = 1e-6
    adj, fd = [], []
    for s, c in sel:
        v0 = float(Tp.data[s, c])
        Tp.data[s, c] = v0 + h
        fp = forward()
        Tp.data[s, c] = v0 - h
        fm = forward()
        Tp.data[s, c] = v0
        fd.append(np.sum((fp - fm) * cw) / (2 * h))
        adj.append(float(gTp.data[s, c]))
    _close(adj, fd, "dL/dFp")
    hx = 1e-9
    for d in range(2):
        adj, fd = [], []
        for s, c in sel:
            x0 = float(p.coords[d].data[s, c])
            p.coords[d].data[s, c] = x0 + hx
            fp = forward()
            p.coords[d].data[s, c] = x0 - hx
            fm = forward()
            p.coords[d].data[s, c] = x0
            fd.append(np.sum((fp - fm) * cw) / (2 * hx))
            adj.append(float(gX[d].data[s, c]))
        _close(adj, fd, f"dL/dX{'xy'[d]} through particle2grid!")


def test_grid2particle_vjp_matches_fd():
    g, p, _ = _setup()
    T = W.gaussian_T(g)
    Td = jp.TA("CUDA")(T)
    (Tp,) = jp.init_cell_arrays(p, 1)
    live = p.index.numpy().astype(bool)
    rng = np.random.default_rng(3)
    cp = np.where(live, rng.standard_normal(live.shape), 0.0)

    def forward(F=Td):
        jp.grid2particle_(Tp, F, p)
        return Tp.numpy()

    gF = jp.grid_field(T.shape)
    gX = tuple(A._like(p) for _ in range(2))
    A.grid2particle_vjp_(gF, gX, jp.CellArray(torch.from_numpy(cp).cuda(), p.ni), Td, p)
    h = 1e-6
    adj, fd = [], []
    for node in _pick_nodes(T.shape, 16, rng):
        Tpl, Tmi = T.copy(order="F"), T.copy(order="F")
        Tpl[node] += h
        Tmi[node] -= h
        fd.append(np.sum((forward(jp.TA("CUDA")(Tpl)) - forward(jp.TA("CUDA")(Tmi)))[live] * cp[live]) / (2 * h))
        adj.append(gF.cpu().numpy()[node])
    _close(adj, fd, "dL/dF through grid2particle!")
    slots = np.argwhere(live)
    sel = slots[rng.choice(len(slots), 12, replace=False)]
    hx = 1e-9
    for d in range(2):
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
        _close(adj, fd, f"dL/dX{'xy'[d]} through grid2particle!")


# ------------------------------------------------------ relocation replay
def test_move_permutation_replays_the_move():
    g, p, Vh = _setup()
    V = _dev(Vh)
    dt = W.cfl_dt(g, Vh)
    jp.advection_(p, jp.RungeKutta2(), V, dt)
    Xa = [c.numpy().copy() for c in p.coords]
    live0 = p.index.numpy().astype(bool)
    jp.move_particles_(p, ())
    dest = A.move_permutation(p).cpu().numpy()
    live1 = p.index.numpy().astype(bool)
    assert np.all(dest[~live0] == -1)
    d = dest[live0]
    kept = d[d >= 0]
    assert len(np.unique(kept)) == len(kept), "two particles share a destination"
    assert len(kept) == live1.sum(), "every live slot after the move has exactly one origin"
    flat_live1 = live1.reshape(-1)
    assert flat_live1[kept].all()
    for k in range(2):
        post = p.coords[k].numpy().reshape(-1)
        assert np.array_equal(post[kept], Xa[k][live0][d >= 0]), "moved coordinates are copies"
    # the gather replay
    post = [torch.from_numpy(np.where(live1, np.random.default_rng(k).standard_normal(live1.shape), 0.0)).cuda()
            for k in range(2)]
    pre = [torch.empty_like(t) for t in post]
    A.permute_vjp_(p, torch.from_numpy(dest).cuda(), post, pre)
    for k in range(2):
        ref = np.where(dest >= 0, post[k].cpu().numpy().reshape(-1)[np.maximum(dest, 0)], 0.0)
        assert np.array_equal(pre[k].cpu().numpy(), ref)


def _depleted(seed=0x51):
    """A state whose cells are under-populated, so inject_particles! acts."""
    g, p, Vh = _setup((16, 16), nxcell=8, max_xcell=16, min_xcell=8, seed=seed)
    V = _dev(Vh)
    dt = W.cfl_dt(g, Vh)
    (T,) = jp.init_cell_arrays(p, 1)
    jp.grid2particle_(T, jp.TA("CUDA")(W.gaussian_T(g)), p)
    for _ in range(6):
        jp.advection_(p, jp.RungeKutta2(), V, dt)
        jp.move_particles_(p, (T,))
    return g, p, V, dt, T


def test_inject_ids_name_the_sources():
    g, p, V, dt, T = _depleted()
    live0 = p.index.numpy().astype(bool)
    ids = A.slot_ids(p)
    jp.inject_particles_(p, (T, ids))
    live1 = p.index.numpy().astype(bool)
    idn = ids.numpy()
    flat = np.arange(live0.size).reshape(live0.shape)
    assert np.all(idn[live0] == flat[live0])
    new = live1 & ~live0
    assert new.sum() > 0, "the setup must make inject_particles! add particles"
    src = idn[new].astype(np.int64)
    assert np.all(src >= 0) and np.all(live0.reshape(-1)[src]), "sources are particles that existed before"
    Tn = T.numpy()
    assert np.array_equal(Tn[new], Tn.reshape(-1)[src]), "injected fields are copies of their source"
    # replay: positions (no copies) and fields (copies)
    rng = np.random.default_rng(4)
    post = torch.from_numpy(np.where(live1, rng.standard_normal(live1.shape), 0.0)).cuda()
    pre_x, pre_t = torch.empty_like(post), torch.empty_like(post)
    A.inject_vjp_(p, ids, [post], [pre_x], copies=False)
    A.inject_vjp_(p, ids, [post], [pre_t], copies=True)
    both = [torch.empty_like(post), torch.empty_like(post)]
    A.inject_vjp_(p, ids, [post, post], both, copies=(False, True))  # one call, per-array flags
    assert torch.equal(both[0], pre_x) and torch.equal(both[1], pre_t)
    pn = post.cpu().numpy()
    ref_x = np.where(live0, pn, 0.0)
    assert np.array_equal(pre_x.cpu().numpy(), ref_x)
    ref_t = ref_x.reshape(-1).copy()
    np.add.at(ref_t, src, pn[new])
    np.testing.assert_allclose(pre_t.cpu().numpy().reshape(-1), ref_t, rtol=1e-14, atol=1e-300)
    # in place: the slots that existed before the injection get the same values as
    # out of place (bit for bit); the injected ones keep theirs
    inp = [post.clone(), post.clone()]
    A.inject_vjp_(p, ids, inp, inp, copies=(False, True))
    assert torch.equal(inp[0][torch.from_numpy(live0).cuda()], pre_x[torch.from_numpy(live0).cuda()])
    assert torch.equal(inp[1][torch.from_numpy(live0).cuda()], pre_t[torch.from_numpy(live0).cuda()])
    assert torch.equal(inp[1][torch.from_numpy(new).cuda()], post[torch.from_numpy(new).cuda()])
    with pytest.raises(jp.ArgumentError):
        A.inject_vjp_(p, ids, [post, post], [post, torch.empty_like(post)], copies=True)


# ------------------------------------------------------------ whole run
def _run_case(ni=(32, 32), nsteps=20, seed=0x4A50):
    g, p, Vh = _setup(ni, seed=seed)
    V = _dev(Vh)
    dt = W.cfl_dt(g, Vh)
    (T0,) = jp.init_cell_arrays(p, 1)
    jp.grid2particle_(T0, jp.TA("CUDA")(W.gaussian_T(g)), p)
    target = jp.TA("CUDA")(W.fourier_target(g))
    return g, p, Vh, V, dt, T0, target, nsteps


def _fields(p, method, V, dt, nsteps, T0):
    """Gridded T after nsteps and its weight mask, from a copy of the state."""
    start = A._save(p)
    T = jp.CellArray(T0.data.clone(), T0.ni)
    try:
        A.run_forward(p, method, V, dt, nsteps, T, True)
        shape = tuple(n + 1 for n in p.ni)
        F, Wt = jp.grid_field(shape), jp.grid_field(shape)
        A.particle2grid_with_weights_(F, Wt, T, p)
        return F.cpu().numpy(), Wt.cpu().numpy() > 0
    finally:
        A._restore(p, start)


def _dloss(fp, mp, fm, mm, target):
    # 0.5 sum (r+^2 - r-^2) formed per vertex
    rp = np.where(mp, fp - target, 0.0)
    rm = np.where(mm, fm - target, 0.0)
    return 0.5 * np.sum((rp - rm) * (rp + rm))


def test_misfit_gradient_matches_fd():
    g, p, Vh, V, dt, T0, target, nsteps = _run_case()
    method = jp.RungeKutta2()
    loss, gV, gT0 = A.misfit_gradient(p, method, V, dt, nsteps, T0, target, checkpoint_every=5)
    tgt = target.cpu().numpy()
    f0, m0 = _fields(p, method, V, dt, nsteps, T0)
    assert abs(loss - 0.5 * np.sum(np.where(m0, f0 - tgt, 0.0) ** 2)) <= 1e-12 * loss
    rng = np.random.default_rng(5)
    h = 1e-6
    for c in range(2):
        gc = gV[c].cpu().numpy()
        # half the nodes where the gradient is large, half anywhere
        big = np.argsort(-np.abs(gc.reshape(-1, order="F")))[:64]
        nodes = [np.unravel_index(f, gc.shape, order="F") for f in rng.choice(big, 6, replace=False)]
        nodes += _pick_nodes(gc.shape, 6, rng)
        adj, fd = [], []
        for node in nodes:
            Vp = [v.copy(order="F") for v in Vh]
            Vm = [v.copy(order="F") for v in Vh]
            Vp[c][node] += h
            Vm[c][node] -= h
            fp, mp = _fields(p, method, _dev(Vp), dt, nsteps, T0)
            fm, mm = _fields(p, method, _dev(Vm), dt, nsteps, T0)
            fd.append(_dloss(fp, mp, fm, mm, tgt) / (2 * h))
            adj.append(gc[node])
        _close(adj, fd, f"misfit dL/dV{'xy'[c]}")
    live = p.index.numpy().astype(bool)
    slots = np.argwhere(live)
    sel = slots[rng.choice(len(slots), 10, replace=False)]
    adj, fd = [], []
    for s, cc in sel:
        v0 = float(T0.data[s, cc])
        T0.data[s, cc] = v0 + h
        fp, mp = _fields(p, method, V, dt, nsteps, T0)
        T0.data[s, cc] = v0 - h
        fm, mm = _fields(p, method, V, dt, nsteps, T0)
        T0.data[s, cc] = v0
        fd.append(_dloss(fp, mp, fm, mm, tgt) / (2 * h))
        adj.append(float(gT0.data[s, cc]))
    _close(adj, fd, "misfit dL/dT0")


def test_misfit_gradient_is_reproducible_and_checkpoint_independent():
    g, p, Vh, V, dt, T0, target, nsteps = _run_case(ni=(24, 24), nsteps=12)
    method = jp.RungeKutta2()
    l1, gV1, gT1 = A.misfit_gradient(p, method, V, dt, nsteps, T0, target, checkpoint_every=4)
    l2, gV2, gT2 = A.misfit_gradient(p, method, V, dt, nsteps, T0, target, checkpoint_every=4)
    l3, gV3, gT3 = A.misfit_gradient(p, method, V, dt, nsteps, T0, target, checkpoint_every=5)
    assert l1 == l2 == l3
    for a, b, c in zip(gV1 + (gT1.data,), gV2 + (gT2.data,), gV3 + (gT3.data,)):
        assert torch.equal(a, b), "gradients differ between two identical runs"
        assert torch.equal(a, c), "gradients depend on the checkpoint spacing"
    # how many trailing segments keep their records (the others run again) changes nothing
    assert A.kept_segments(p, method, nsteps, 4) == 3  # all of them, at this size
    for K in (1, 2):
        lk, gVk, gTk = A.misfit_gradient(p, method, V, dt, nsteps, T0, target, checkpoint_every=4,
                                         record_segments=K)
        assert lk == l1
        for a, b in zip(gV1 + (gT1.data,), gVk + (gTk.data,)):
            assert torch.equal(a, b), f"gradients depend on the segments kept ({K})"


def test_pic_misfit_autograd():
    g, p, Vh, V, dt, T0, target, nsteps = _run_case(ni=(16, 16), nsteps=8)
    method = jp.RungeKutta2()
    Vx = V[0].clone().requires_grad_(True)
    Vy = V[1].clone().requires_grad_(True)
    T0d = T0.data.clone().requires_grad_(True)
    loss = A.PICMisfit.apply(Vx, Vy, T0d, p, method, dt, nsteps, target, 3, True)
    loss.backward()
    l_ref, gV, gT0 = A.misfit_gradient(p, method, V, dt, nsteps, T0, target, checkpoint_every=3)
    assert float(loss) == l_ref
    assert torch.equal(Vx.grad, gV[0]) and torch.equal(Vy.grad, gV[1])
    assert torch.equal(T0d.grad, gT0.data)


def test_fd_is_oracle_fd():
    # the perturbed forward runs used for finite differences match the oracle bit for bit
    g = W.grid((16, 16))
    Vh = W.perturbed_stream_velocity(g)
    Vh[0][5, 7] += 1e-6
    dt = W.cfl_dt(g, Vh)
    pair = Pair(g, 16, 32, 8, nfields=1)
    pair.g2p(0, W.gaussian_T(g))
    for _ in range(6):
        pair.advection("rk2", Vh, dt)
        pair.move()
        pair.inject()
    pair.assert_same("perturbed run")
    Fo, Fg = pair.p2g(0)
    assert np.array_equal(np.nan_to_num(Fo, nan=-7.0), np.nan_to_num(Fg, nan=-7.0))


# --------------------------------------------- forward mode through the oracle
def oracle_jvp_run(g, Vh, dV, dt, nsteps, T0_grid, target, dT0=None, method=O.RK2, alpha=0.5,
                   nxcell=16, max_xcell=32, min_xcell=8, seed=0x4A50):
    """dL along (dV, dT0) by dual numbers through the oracle: the tangents of
    positions and of T ride along as particle fields through move and inject
    (an injected particle copies T and its tangent; its position tangent is 0)."""
    o = O.OracleParticles(tuple(tuple(np.asarray(x, dtype=np.float64) for x in c) for c in g["grid_v"]),
                          nxcell, max_xcell, min_xcell, seed=seed)
    o.init_particles()
    T = o.cell_array()
    o.grid2particle(T, T0_grid)
    dT = o.cell_array() if dT0 is None else dT0.copy()
    dX = [o.cell_array() for _ in range(2)]
    for _ in range(nsteps):
        o.advection_jvp(method, alpha, Vh, dV, dt, dX)
        o.move_particles([T, dT, dX[0], dX[1]])
        before = o.index.copy()
        o.inject_particles([T, dT, dX[0], dX[1]])
        new = o.index.astype(bool) & ~before.astype(bool)
        for d in range(2):
            dX[d][new] = 0.0
    shape = tuple(n + 1 for n in o.n)
    F = np.asfortranarray(np.zeros(shape))
    dF = np.asfortranarray(np.zeros(shape))
    o.particle2grid_jvp(F, dF, T, dT, dX)
    ok = np.isfinite(F)
    return float(np.sum(np.where(ok, (F - target) * dF, 0.0))), o


@pytest.mark.parametrize("method,nsteps", [("rk2", 20), ("rk4", 10), ("euler", 10)])
def test_misfit_gradient_matches_oracle_jvp(method, nsteps):
    g, p, Vh, V, dt, T0, target, _ = _run_case(ni=(32, 32), nsteps=nsteps)
    om, pm, alpha = METHODS[method]
    loss, gV, gT0 = A.misfit_gradient(p, pm, V, dt, nsteps, T0, target, checkpoint_every=4)
    Tg = W.gaussian_T(g)
    tgt = target.cpu().numpy()
    rng = np.random.default_rng(6)
    gmax = max(float(v.abs().max()) for v in gV)
    adj, jvp = [], []
    for c in range(2):
        gc = gV[c].cpu().numpy()
        big = np.argsort(-np.abs(gc.reshape(-1, order="F")))[:32]
        nodes = [np.unravel_index(f, gc.shape, order="F") for f in rng.choice(big, 3, replace=False)]
        nodes += _pick_nodes(gc.shape, 2, rng)
        for node in nodes:
            dV = [np.zeros_like(v) for v in Vh]
            dV[c][node] = 1.0
            d, _ = oracle_jvp_run(g, Vh, dV, dt, nsteps, Tg, tgt, method=om, alpha=alpha)
            jvp.append(d)
            adj.append(gc[node])
    adj, jvp = np.array(adj), np.array(jvp)
    err = np.abs(adj - jvp)
    assert np.all(err <= 1e-9 * np.maximum(np.abs(jvp), gmax)), f"dL/dV vs oracle JVP: {adj} {jvp}"
    # initial particle field: dL/dT0 along single slots
    live = p.index.numpy().astype(bool)
    slots = np.argwhere(live)
    g0 = gT0.numpy()
    for s, cc in slots[rng.choice(len(slots), 4, replace=False)]:
        dT0 = np.zeros(live.shape)
        dT0[s, cc] = 1.0
        d, _ = oracle_jvp_run(g, Vh, None, dt, nsteps, Tg, tgt, dT0=dT0, method=om, alpha=alpha)
        assert abs(g0[s, cc] - d) <= 1e-10 * max(abs(d), float(np.max(np.abs(g0)))), (s, cc, g0[s, cc], d)


def test_c5_gradient_matches_oracle_jvp():
    """The C5 adjoint run at full size (512^2 cells, 16 particles per cell,
    RK2, 100 steps, checkpoints every 10) against dual numbers through the
    oracle on the velocity nodes of largest gradient (about a minute of host
    time per node)."""
    cfg = W.setup("C5")
    g, Vh, dt = cfg["grid"], cfg["V"], cfg["dt"]
    p = jp.init_particles(jp.CUDABackend, cfg["nxcell"], cfg["max_xcell"], cfg["min_xcell"], *g["grid_v"])
    (T0,) = jp.init_cell_arrays(p, 1)
    jp.grid2particle_(T0, jp.TA("CUDA")(cfg["T"]), p)
    target = jp.TA("CUDA")(cfg["T_target"])
    loss, gV, gT0 = A.misfit_gradient(p, jp.RungeKutta2(), _dev(Vh), dt, cfg["steps"], T0, target,
                                      checkpoint_every=cfg["checkpoint_every"])
    gmax = max(float(v.abs().max()) for v in gV)
    for c in range(2):
        gc = gV[c].cpu().numpy()
        node = np.unravel_index(int(np.argmax(np.abs(gc))), gc.shape)
        dV = [np.zeros_like(v) for v in Vh]
        dV[c][node] = 1.0
        d, _ = oracle_jvp_run(g, Vh, dV, dt, cfg["steps"], cfg["T"], cfg["T_target"], nxcell=cfg["nxcell"],
                              max_xcell=cfg["max_xcell"], min_xcell=cfg["min_xcell"])
        assert abs(gc[node] - d) <= 1e-9 * max(abs(d), gmax), (c, node, gc[node], d)


# ------------------------------------------- split-precision (FP32) variant
def _f32_case(ni=(32, 32), nsteps=20):
    g, p, Vh, V, dt, T0, target, _ = _run_case(ni=ni, nsteps=nsteps)
    xi = jp.init_offsets(p)
    V32 = tuple(v.float() for v in V)
    T0f = jp.CellArray(T0.data.float().contiguous(), p.ni)
    return g, p, V, V32, dt, T0, T0f, target, xi, nsteps


@pytest.mark.parametrize("method", ["rk2", "rk4"])
def test_f32_adjoint_agrees_with_fp64_adjoint(method):
    """The split-precision run follows the FP64 run to FP32 rounding (a few
    particles make other discrete choices), so its gradients must agree with
    the FP64 adjoint's to FP32-form accuracy."""
    g, p, V, V32, dt, T0, T0f, target, xi, nsteps = _f32_case()
    _, pm, _ = METHODS[method]
    l64, gV64, gT64 = A.misfit_gradient(p, pm, V, dt, nsteps, T0, target, checkpoint_every=5)
    l32, gV32, gT32 = A.misfit_gradient_f32(p, xi, pm, V32, dt, nsteps, T0f, target.float(), checkpoint_every=5)
    assert abs(l32 - l64) <= 2e-3 * l64
    for a, b in zip(gV32 + (gT32.data,), gV64 + (gT64.data,)):
        a, b = a.double().flatten(), b.double().flatten()
        rel = float((a - b).norm() / b.norm())
        cos = float((a @ b) / (a.norm() * b.norm()))
        assert rel < 2e-2 and cos > 0.999, (rel, cos)


def test_f32_adjoint_is_reproducible():
    g, p, V, V32, dt, T0, T0f, target, xi, nsteps = _f32_case(ni=(24, 24), nsteps=8)
    m = jp.RungeKutta2()
    r1 = A.misfit_gradient_f32(p, xi, m, V32, dt, nsteps, T0f, target.float(), checkpoint_every=3)
    r2 = A.misfit_gradient_f32(p, xi, m, V32, dt, nsteps, T0f, target.float(), checkpoint_every=4)
    assert r1[0] == r2[0]
    for a, b in zip(r1[1] + (r1[2].data,), r2[1] + (r2[2].data,)):
        assert torch.equal(a, b)
