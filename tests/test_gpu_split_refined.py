"""Split-precision form on grids whose spacing varies (the kernels read
per-cell width tables), against the FP64 form on the same seeded runs. The form
has no reference counterpart; its error is stated against the FP64 form.

Tolerances (written here, asserted below), in units of the grid's smallest
cell width h:
  * conversion round trip: 2^-23 of the local cell width;
  * one step (Euler, RK2, RK4): 2e-5 h;
  * 40 RK2 steps of advection + move (2D; 20 in 3D): 2e-4 h for every
    particle present in both runs (tracked by id), with at least 95% of the
    FP64 run's particles present in the split run;
  * grid2particle: 1e-6 of the field's range; particle2grid: 1e-5 of the range
    against the FP64 form, 1e-6 of the largest value against inverse-distance
    sums formed on the host in FP64 from the FP32 offsets and the per-cell
    widths;
  * injection: every cell's first quadrant holds min_xcell / 2^N particles.

Cells wider than 64 slots (uniform and refined) run the wide move and
injection kernels; they are held to the same bounds and to determinism.
"""
import numpy as np
import pytest
import torch

from _harness import W, jp, refined_grid

pytestmark = pytest.mark.gpu


def _ids(p):
    """Particle ids as one FP64 field and two exact FP32 fields (hi * 4096 + lo)."""
    live = p.index.data.bool()
    ids = torch.full(p.index.data.shape, float("nan"), dtype=torch.float64, device="cuda")
    ids[live] = torch.arange(int(live.sum()), device="cuda", dtype=torch.float64)
    hi = torch.floor(ids / 4096.0)
    lo = ids - hi * 4096.0
    return ids, hi.float(), lo.float()


def _pair(g, nxcell=24, max_xcell=48, min_xcell=12):
    a = jp.init_particles(jp.CUDABackend, nxcell, max_xcell, min_xcell, *g["grid_v"])
    b = jp.init_particles(jp.CUDABackend, nxcell, max_xcell, min_xcell, *g["grid_v"])
    return a, b


def _velocity(g):
    return W.stream_velocity(g) if g["ndim"] == 2 else W.cellular_velocity_3d(g)


def _local_width(g, p):
    """Per slot: the width of its cell along each axis (ncap, ncells, N)."""
    ni = g["ni"]
    N = len(ni)
    cells = np.arange(int(np.prod(ni)))
    out = []
    for d in range(N):
        I = (cells // int(np.prod(ni[:d]))) % ni[d]
        out.append(np.diff(np.asarray(g["xv"][d]))[I])
    return np.broadcast_to(np.stack(out, axis=1)[None], (p.index.data.shape[0], len(cells), N))


@pytest.mark.parametrize("ni", [(40, 30), (10, 9, 7)])
def test_offsets_round_trip_refined(ni):
    g = refined_grid(ni)
    a, _ = _pair(g)
    xi = jp.init_offsets(a)
    live = a.index.numpy().astype(bool)
    back = jp.coords_from_offsets(a, xi)
    h = _local_width(g, a)
    for d in range(len(ni)):
        x = xi[d].numpy()[live]
        assert np.all((x >= 0) & (x < 1))
        err = np.abs(back[d].numpy()[live] - a.coords[d].numpy()[live]) / h[..., d][live]
        assert err.max() <= 2.0 ** -23


@pytest.mark.parametrize("method", ["euler", "rk2", "rk4"])
@pytest.mark.parametrize("ni", [(48, 40), (12, 10, 8)])
def test_one_step_matches_fp64_refined(ni, method):
    g = refined_grid(ni)
    a, b = _pair(g)
    V = _velocity(g)
    dt = W.cfl_dt(g, V, 0.5)
    m = {"rk2": jp.RungeKutta2(), "rk4": jp.RungeKutta4(), "euler": jp.Euler()}[method]
    xi = jp.init_offsets(b)
    jp.advection_(a, m, tuple(jp.TA("CUDA")(v) for v in V), dt)
    jp.advection_f32_(b, xi, m, tuple(jp.TA("CUDA")(v).float() for v in V), dt)
    back = jp.coords_from_offsets(b, xi)
    live = a.index.numpy().astype(bool)
    # a stage point outside a velocity grid samples Inf in both forms (3D: the z
    # drift carries stage points through the top): the same particles go non-finite
    fa = np.all([np.isfinite(c.numpy()[live]) for c in a.coords], axis=0)
    fb = np.all([np.isfinite(c.numpy()[live]) for c in back], axis=0)
    assert np.array_equal(fa, fb), f"{method}: {int((fa != fb).sum())} particles finite in one form only"
    for d in range(len(ni)):
        err = np.abs(back[d].numpy()[live][fa] - a.coords[d].numpy()[live][fa]) / g["dx"][d]
        assert err.max() < 2e-5, f"{method}: axis {d} max error {err.max():.3g} smallest cell widths"


@pytest.mark.parametrize("ni,steps", [((64, 48), 40), ((14, 12, 10), 20)])
def test_many_steps_error_refined(ni, steps):
    g = refined_grid(ni)
    N = len(ni)
    a, b = _pair(g, min_xcell=0)
    V = _velocity(g)
    dt = W.cfl_dt(g, V, 0.5)
    Va = tuple(jp.TA("CUDA")(v) for v in V)
    Vb = tuple(jp.TA("CUDA")(v).float() for v in V)
    ida, _, _ = _ids(a)
    _, hib, lob = _ids(b)
    fa = jp.CellArray(ida, a.ni)
    fb = (jp.CellArray(hib.contiguous(), b.ni), jp.CellArray(lob.contiguous(), b.ni))
    xi = jp.init_offsets(b)
    jp.move_counts(a, clear=True)
    jp.move_counts(b, clear=True)
    for _ in range(steps):
        jp.advection_(a, jp.RungeKutta2(), Va, dt)
        jp.move_particles_(a, (fa,))
        jp.advection_f32_(b, xi, jp.RungeKutta2(), Vb, dt)
        jp.move_particles_f32_(b, xi, fb)
    live_a = a.index.numpy().astype(bool)
    ids_a = fa.numpy()[live_a].astype(np.int64)
    pa = np.stack([c.numpy()[live_a] for c in a.coords], axis=1)
    live_b = b.index.numpy().astype(bool)
    ids_b = fb[0].numpy()[live_b].astype(np.int64) * 4096 + fb[1].numpy()[live_b].astype(np.int64)
    back = jp.coords_from_offsets(b, xi)
    pb = np.stack([c.numpy()[live_b] for c in back], axis=1)
    common, ia, ib = np.intersect1d(ids_a, ids_b, return_indices=True)
    assert len(common) > 0.95 * len(ids_a)
    err = np.abs(pa[ia] - pb[ib]) / np.asarray(g["dx"])[None, :]
    assert err.max() < 2e-4, f"max error {err.max():.3g} smallest cell widths"
    for d in range(N):
        x = xi[d].numpy()[live_b]
        assert np.all((x >= 0) & (x < 1)), "offsets stay inside their cells after every move"
    cb = jp.move_counts(b)
    assert cb["moved_too_far"] == 0


@pytest.mark.parametrize("ni", [(30, 22), (9, 8, 7)])
def test_grid_transfers_refined(ni):
    g = refined_grid(ni)
    N = len(ni)
    a, b = _pair(g)
    T = W.gaussian_T(g, center=(0.5,) * N, width2=0.05)
    xi = jp.init_offsets(b)
    pa, = jp.init_cell_arrays(a, 1)
    pb, = jp.init_cell_arrays_f32(b, 1)
    jp.grid2particle_(pa, jp.TA("CUDA")(T), a)
    jp.grid2particle_f32_(pb, jp.TA("CUDA")(T).float(), b, xi)
    live = a.index.numpy().astype(bool)
    rng = T.max() - T.min()
    assert np.abs(pa.numpy()[live] - pb.numpy()[live]).max() < 1e-6 * rng
    Fa = jp.grid_field(T.shape)
    Fb = jp.grid_field_f32(T.shape)
    jp.particle2grid_(Fa, pa, a)
    jp.particle2grid_f32_(Fb, pb, b, xi)
    assert np.abs(Fa.cpu().numpy() - Fb.cpu().numpy()).max() < 1e-5 * rng
    # the same sums formed on the host in FP64 from the FP32 offsets and per-cell widths
    X = [xi[d].numpy().astype(np.float64) for d in range(N)]
    f = pb.numpy().astype(np.float64)
    h = _local_width(g, b).astype(np.float32)
    cells = np.arange(live.shape[1])
    I = [(cells // int(np.prod(ni[:k]))) % ni[k] for k in range(N)]
    W_ = np.zeros(T.shape)
    WF = np.zeros(T.shape)
    for corner in np.ndindex(*(2,) * N):
        d2 = sum(((corner[d] - X[d]) * h[..., d].astype(np.float64)) ** 2 for d in range(N))
        with np.errstate(divide="ignore", invalid="ignore"):
            w = np.where(live, 1.0 / d2, 0.0)
        v = tuple(np.broadcast_to(I[d] + corner[d], live.shape)[live] for d in range(N))
        np.add.at(W_, v, w[live])
        np.add.at(WF, v, (w * np.where(live, f, 0.0))[live])
    ref = WF / W_
    got = Fb.cpu().numpy().astype(np.float64)
    assert np.all(W_ > 0)
    assert np.max(np.abs(got - ref)) < 1e-6 * np.max(np.abs(ref))


@pytest.mark.parametrize("ni", [(16, 14), (6, 6, 5)])
def test_injection_refills_depleted_quadrants_refined(ni):
    g = refined_grid(ni)
    N = len(ni)
    _, b = _pair(g, nxcell=8 * (N - 1), max_xcell=24 * (N - 1), min_xcell=8)
    xi = jp.init_offsets(b)
    T, = jp.init_cell_arrays_f32(b, 1)
    T.data[b.index.data.bool()] = 1.0
    kill = (torch.rand(b.index.data.shape, device="cuda", generator=torch.Generator("cuda").manual_seed(5)) < 0.7)
    kill &= b.index.data.bool()
    b.index.data[kill] = 0
    for d in range(N):
        xi[d].data[kill] = float("nan")
    jp.inject_particles_f32_(b, xi, (T,))
    live = b.index.numpy().astype(bool)
    inq = live.copy()
    for d in range(N):
        x = xi[d].numpy()
        inq &= (x > 0) & (x < 0.5)
    min_q = (8 + (1 << N) - 1) >> N
    assert np.all(inq.sum(axis=0) >= min_q), "every cell's first quadrant holds at least min_xcell / 2^N particles"
    assert np.all(np.isfinite(T.numpy()[live]))
    # injected particles copy the field of a particle of the 3^N neighbourhood: all ones here
    assert np.all(T.numpy()[live] == 1.0)


@pytest.mark.parametrize("ni,refined", [((24, 20), False), ((20, 16), True), ((8, 7, 6), False), ((7, 6, 6), True)])
def test_wide_cells_against_fp64(ni, refined):
    """Cells of more than 64 slots (the reference's 3D miniapps use 125 / 150 /
    100): the split form's wide move and injection kernels, 10 cycles of
    advection + move + inject + grid2particle against the FP64 form; position
    error 2e-4 h by id, offsets inside their cells, particle counts within 1%,
    and the move and injection rules the same as the narrow kernels'
    (deterministic: two runs bit-identical)."""
    g = refined_grid(ni) if refined else W.grid(ni)
    N = len(ni)
    nxcell, max_xcell, min_xcell = (90, 120, 60) if N == 2 else (125, 150, 100)
    a, b = _pair(g, nxcell, max_xcell, min_xcell)
    c = jp.init_particles(jp.CUDABackend, nxcell, max_xcell, min_xcell, *g["grid_v"])
    V = _velocity(g)
    dt = W.cfl_dt(g, V, 0.5)
    Va = tuple(jp.TA("CUDA")(v) for v in V)
    Vb = tuple(jp.TA("CUDA")(v).float() for v in V)
    ida, _, _ = _ids(a)
    _, hib, lob = _ids(b)
    fa = jp.CellArray(ida, a.ni)
    fb = (jp.CellArray(hib.contiguous(), b.ni), jp.CellArray(lob.contiguous(), b.ni))
    fc = (jp.CellArray(hib.clone(), c.ni), jp.CellArray(lob.clone(), c.ni))
    xb, xc = jp.init_offsets(b), jp.init_offsets(c)
    for _ in range(10):
        jp.advection_(a, jp.RungeKutta2(), Va, dt)
        jp.move_particles_(a, (fa,))
        for p, x, f in ((b, xb, fb), (c, xc, fc)):
            jp.advection_f32_(p, x, jp.RungeKutta2(), Vb, dt)
            jp.move_particles_f32_(p, x, f)
    assert torch.equal(b.index.data, c.index.data)
    for d in range(N):
        assert torch.equal(xb[d].data.nan_to_num(-7.0), xc[d].data.nan_to_num(-7.0))
    live_a = a.index.numpy().astype(bool)
    ids_a = fa.numpy()[live_a].astype(np.int64)
    pa = np.stack([q.numpy()[live_a] for q in a.coords], axis=1)
    live_b = b.index.numpy().astype(bool)
    ids_b = fb[0].numpy()[live_b].astype(np.int64) * 4096 + fb[1].numpy()[live_b].astype(np.int64)
    back = jp.coords_from_offsets(b, xb)
    pb = np.stack([q.numpy()[live_b] for q in back], axis=1)
    assert abs(len(ids_b) - len(ids_a)) <= 0.01 * len(ids_a)
    common, ia, ib = np.intersect1d(ids_a, ids_b, return_indices=True)
    assert len(common) > 0.95 * len(ids_a)
    err = np.abs(pa[ia] - pb[ib]) / np.asarray(g["dx"])[None, :]
    assert err.max() < 2e-4, f"max error {err.max():.3g} smallest cell widths"
    for d in range(N):
        x = xb[d].numpy()[live_b]
        assert np.all((x >= 0) & (x < 1))
    # injection into depleted wide cells: the first quadrant refilled, fields copied from neighbours
    T, = jp.init_cell_arrays_f32(b, 1)
    T.data[b.index.data.bool()] = 1.0
    kill = (torch.rand(b.index.data.shape, device="cuda", generator=torch.Generator("cuda").manual_seed(3)) < 0.8)
    kill &= b.index.data.bool()
    b.index.data[kill] = 0
    for d in range(N):
        xb[d].data[kill] = float("nan")
    jp.inject_particles_f32_(b, xb, (T,))
    live = b.index.numpy().astype(bool)
    inq = live.copy()
    for d in range(N):
        x = xb[d].numpy()
        inq &= (x > 0) & (x < 0.5)
    min_q = (min_xcell + (1 << N) - 1) >> N
    assert np.all(inq.sum(axis=0) >= min_q)
    assert np.all(T.numpy()[live] == 1.0)
    # grid2particle / particle2grid over the wide slot rows against the FP64 form
    Tg = W.gaussian_T(g, center=(0.5,) * N, width2=0.05)
    pa2, = jp.init_cell_arrays(a, 1)
    jp.grid2particle_(pa2, jp.TA("CUDA")(Tg), a)
    xa = jp.init_offsets(a)
    pf, = jp.init_cell_arrays_f32(a, 1)
    jp.grid2particle_f32_(pf, jp.TA("CUDA")(Tg).float(), a, xa)
    la = a.index.numpy().astype(bool)
    rng = Tg.max() - Tg.min()
    assert np.abs(pa2.numpy()[la] - pf.numpy()[la]).max() < 1e-6 * rng
    Fa, Fb = jp.grid_field(Tg.shape), jp.grid_field_f32(Tg.shape)
    jp.particle2grid_(Fa, pa2, a)
    jp.particle2grid_f32_(Fb, pf, a, xa)
    assert np.abs(Fa.cpu().numpy() - Fb.cpu().numpy()).max() < 1e-5 * rng


def test_other_staggering_is_refused():
    """Centred nodes that are not the cell midpoints: the split form refuses the
    grid (the FP64 form takes it)."""
    ni = (12, 10)
    xv = tuple(np.linspace(0.0, 1.0, n + 1) ** 1.3 for n in ni)
    xc = tuple(0.3 * x[1:] + 0.7 * x[:-1] for x in xv)
    ext = tuple(np.concatenate([[x[0] - 0.05], x, [x[-1] + 0.05]]) for x in xc)
    grid_v = tuple(tuple(xv[d] if d == c else ext[d] for d in range(2)) for c in range(2))
    p = jp.init_particles(jp.CUDABackend, 8, 16, 4, *grid_v)
    with pytest.raises(jp.ArgumentError):
        jp.init_offsets(p)
