"""Split-precision form (int32 cell + FP32 offset) against the FP64 form on the
same seeded runs. The form has no reference counterpart; these tests pin its
conversions, its slot-allocation determinism and its error in cell widths.

Tolerances (written here, asserted below):
  * conversion round trip: 2^-23 cell widths (one FP32 ulp of an offset < 1);
  * one RK2 step: 1e-5 cell widths;
  * 60 RK2 steps of advection + move: 1e-4 cell widths for every particle
    present in both runs (tracked by id);
  * particle2grid: 1e-5 relative to the field's range against the FP64 form;
    1e-6 of the field's largest value against the same inverse-distance sums
    formed on the host in FP64 from the FP32 offsets (the kernel sums FP32
    weights in compensated pairs).
"""
import numpy as np
import pytest
import torch

from _harness import W, jp

pytestmark = pytest.mark.gpu

ULP_XI = 2.0 ** -23


def _ids(p):
    """Particle ids as one FP64 field and two exact FP32 fields (hi * 4096 + lo)."""
    live = p.index.data.bool()
    ids = torch.full(p.index.data.shape, float("nan"), dtype=torch.float64, device="cuda")
    ids[live] = torch.arange(int(live.sum()), device="cuda", dtype=torch.float64)
    hi = torch.floor(ids / 4096.0)
    lo = ids - hi * 4096.0
    return ids, hi.float(), lo.float()


def _positions_by_id(p, coords, id_field, live_only=True):
    live = p.index.numpy().astype(bool)
    ids = id_field[live].astype(np.int64)
    pos = np.stack([c.numpy()[live] for c in coords], axis=1)
    return ids, pos


def _pair(ni, nxcell=24, max_xcell=48, min_xcell=12):
    g = W.grid(ni)
    a = jp.init_particles(jp.CUDABackend, nxcell, max_xcell, min_xcell, *g["grid_v"])
    b = jp.init_particles(jp.CUDABackend, nxcell, max_xcell, min_xcell, *g["grid_v"])
    return g, a, b


def test_offsets_round_trip():
    g, a, _ = _pair((40, 30))
    xi = jp.init_offsets(a)
    live = a.index.numpy().astype(bool)
    for d in range(2):
        x = xi[d].numpy()[live]
        assert np.all((x >= 0) & (x < 1)), "offsets of freshly seeded particles lie in [0, 1)"
    back = jp.coords_from_offsets(a, xi)
    for d in range(2):
        err = np.abs(back[d].numpy()[live] - a.coords[d].numpy()[live]) / g["dx"][d]
        assert err.max() <= ULP_XI


@pytest.mark.parametrize("method", ["rk2", "rk4", "euler"])
def test_one_step_matches_fp64(method):
    g, a, b = _pair((48, 40))
    V = W.stream_velocity(g)
    dt = W.cfl_dt(g, V, 0.5)
    m = {"rk2": jp.RungeKutta2(), "rk4": jp.RungeKutta4(), "euler": jp.Euler()}[method]
    xi = jp.init_offsets(b)
    jp.advection_(a, m, tuple(jp.TA("CUDA")(v) for v in V), dt)
    jp.advection_f32_(b, xi, m, tuple(jp.TA("CUDA")(v).float() for v in V), dt)
    back = jp.coords_from_offsets(b, xi)
    live = a.index.numpy().astype(bool)
    for d in range(2):
        err = np.abs(back[d].numpy()[live] - a.coords[d].numpy()[live]) / g["dx"][d]
        assert err.max() < 1e-5, f"{method}: max error {err.max():.3g} cell widths"


def test_many_steps_error_in_cell_widths():
    g, a, b = _pair((64, 64), min_xcell=0)
    V = W.stream_velocity(g)
    dt = W.cfl_dt(g, V, 0.5)
    Va = tuple(jp.TA("CUDA")(v) for v in V)
    Vb = tuple(jp.TA("CUDA")(v).float() for v in V)
    ida, _, _ = _ids(a)
    _, hib, lob = _ids(b)
    fa = jp.CellArray(ida, a.ni)
    fb = (jp.CellArray(hib.contiguous(), b.ni), jp.CellArray(lob.contiguous(), b.ni))
    xi = jp.init_offsets(b)
    for _ in range(60):
        jp.advection_(a, jp.RungeKutta2(), Va, dt)
        jp.move_particles_(a, (fa,))
        jp.advection_f32_(b, xi, jp.RungeKutta2(), Vb, dt)
        jp.move_particles_f32_(b, xi, fb)
    ids_a, pa = _positions_by_id(a, a.coords, fa.numpy())
    live_b = b.index.numpy().astype(bool)
    ids_b = (fb[0].numpy()[live_b].astype(np.int64) * 4096 + fb[1].numpy()[live_b].astype(np.int64))
    back = jp.coords_from_offsets(b, xi)
    pb = np.stack([c.numpy()[live_b] for c in back], axis=1)
    common, ia, ib = np.intersect1d(ids_a, ids_b, return_indices=True)
    assert len(common) > 0.95 * len(ids_a)
    err = np.abs(pa[ia] - pb[ib]) / np.asarray(g["dx"])[None, :]
    assert err.max() < 1e-4, f"max error {err.max():.3g} cell widths"
    # offsets stay inside their cells after every move
    for d in range(2):
        x = xi[d].numpy()[live_b]
        assert np.all((x >= 0) & (x < 1))


def test_move_is_deterministic_and_conserves():
    g, a, b = _pair((32, 32))
    V = tuple(jp.TA("CUDA")(v).float() for v in W.stream_velocity(g))
    dt = W.cfl_dt(g, W.stream_velocity(g))
    xa, xb = jp.init_offsets(a), jp.init_offsets(b)
    n0 = int(a.index.data.sum())
    for _ in range(5):
        for p, x in ((a, xa), (b, xb)):
            jp.advection_f32_(p, x, jp.RungeKutta2(), V, dt)
            jp.move_particles_f32_(p, x)
    assert torch.equal(a.index.data, b.index.data)
    for d in range(2):
        assert torch.equal(xa[d].data.nan_to_num(-7.0), xb[d].data.nan_to_num(-7.0))
    assert int(a.index.data.sum()) <= n0


def test_grid_transfers_against_fp64():
    g, a, b = _pair((24, 20))
    T = W.gaussian_T(g, center=(0.5, 0.5), width2=0.05)
    xi = jp.init_offsets(b)
    pa, = jp.init_cell_arrays(a, 1)
    pb, = jp.init_cell_arrays_f32(b, 1)
    jp.grid2particle_(pa, jp.TA("CUDA")(T), a)
    jp.grid2particle_f32_(pb, jp.TA("CUDA")(T).float(), b, xi)
    live = a.index.numpy().astype(bool)
    assert np.abs(pa.numpy()[live] - pb.numpy()[live]).max() < 1e-6
    Fa = jp.grid_field(T.shape)
    Fb = jp.grid_field_f32(T.shape)
    jp.particle2grid_(Fa, pa, a)
    jp.particle2grid_f32_(Fb, pb, b, xi)
    rng = T.max() - T.min()
    assert np.abs(Fa.cpu().numpy() - Fb.cpu().numpy()).max() < 1e-5 * rng


def test_injection_refills_depleted_quadrants():
    g, _, b = _pair((16, 16), nxcell=8, max_xcell=24, min_xcell=8)
    xi = jp.init_offsets(b)
    T, = jp.init_cell_arrays_f32(b, 1)
    T.data[b.index.data.bool()] = 1.0
    kill = (torch.rand(b.index.data.shape, device="cuda", generator=torch.Generator("cuda").manual_seed(5)) < 0.7)
    kill &= b.index.data.bool()
    b.index.data[kill] = 0
    for d in range(2):
        xi[d].data[kill] = float("nan")
    jp.inject_particles_f32_(b, xi, (T,))
    live = b.index.numpy().astype(bool)
    x0, x1 = xi[0].numpy(), xi[1].numpy()
    inq = live & (x0 > 0) & (x0 < 0.5) & (x1 > 0) & (x1 < 0.5)
    assert np.all(inq.sum(axis=0) >= 2), "every cell's first quadrant holds at least min_xcell / 4 particles"
    assert np.all(np.isfinite(T.numpy()[live]))


@pytest.mark.parametrize("ni", [(37, 29), (9, 7, 6)])
def test_particle2grid_f32_against_host_sums(ni):
    """Every vertex: sum_p w_p F_p / sum_p w_p over the particles of its 2^N
    cells, w_p = 1 / |vertex - particle|^2 with the distance in physical units
    formed from the FP32 offsets, summed on the host in FP64."""
    g = W.grid(ni)
    N = len(ni)
    p = jp.init_particles(jp.CUDABackend, 24, 48, 12, *g["grid_v"])
    xi = jp.init_offsets(p)
    T = W.gaussian_T(g, center=(0.5,) * N, width2=0.05)
    pT, = jp.init_cell_arrays_f32(p, 1)
    jp.grid2particle_f32_(pT, jp.TA("CUDA")(T).float(), p, xi)
    F = jp.grid_field_f32(T.shape)
    jp.particle2grid_f32_(F, pT, p, xi)
    live = p.index.numpy().astype(bool)
    X = [xi[d].numpy().astype(np.float64) for d in range(N)]
    f = pT.numpy().astype(np.float64)
    dx = np.asarray(g["dx"])
    cells = np.arange(live.shape[1])
    I = [(cells // int(np.prod(ni[:d]))) % ni[d] for d in range(N)]
    W_ = np.zeros(T.shape)
    WF = np.zeros(T.shape)
    for corner in np.ndindex(*(2,) * N):
        d2 = sum(((corner[d] - X[d]) * np.float32(dx[d])) ** 2 for d in range(N))
        with np.errstate(divide="ignore", invalid="ignore"):
            w = np.where(live, 1.0 / d2, 0.0)
        v = tuple(np.broadcast_to(I[d] + corner[d], live.shape)[live] for d in range(N))
        np.add.at(W_, v, w[live])
        np.add.at(WF, v, (w * np.where(live, f, 0.0))[live])
    ref = WF / W_
    got = F.cpu().numpy().astype(np.float64)
    assert np.all(W_ > 0)
    assert np.max(np.abs(got - ref)) < 1e-6 * np.max(np.abs(ref))
