"""Host <-> device conversion (src/CellArrays/conversion.jl, ext/JustPICCUDAExt.jl:51-191)
and checkpoint restarts on the GPU: the CPU layout is the transpose of the
GPU layout bit for bit, conversions round-trip, and a run restarted from a
checkpoint continues exactly like the uninterrupted one (the injection
counter travels with the particles)."""
import numpy as np
import pytest
import torch

from _harness import W, assert_bits_equal, jp, refined_grid

pytestmark = pytest.mark.gpu


def _stepped(ni, refined=False, steps=2):
    g = refined_grid(ni) if refined else W.grid(ni)
    p = jp.init_particles(jp.CUDABackend, 24, 48, 12, *g["grid_v"])
    T, S = jp.init_cell_arrays(p, 2)
    Tv = W.linear_T(g, 0)
    jp.grid2particle_(T, jp.TA("CUDA")(Tv), p)
    jp.grid2particle_(S, jp.TA("CUDA")(W.linear_T(g, len(ni) - 1)), p)
    V = W.stream_velocity(g) if len(ni) == 2 else W.stream_velocity_3d(g)
    Vd = tuple(jp.TA("CUDA")(v) for v in V)
    dt = W.cfl_dt(g, V, 0.5)
    for _ in range(steps):
        jp.advection_(p, jp.RungeKutta2(), Vd, dt)
        jp.move_particles_(p, (T, S))
        jp.inject_particles_(p, (T, S))
    return p, (T, S), Vd, dt, g


@pytest.mark.parametrize("ni,refined", [((13, 7), False), ((11, 9), True), ((5, 6, 4), False)])
def test_array_is_the_cpu_layout(ni, refined):
    p, (T, S), _, _, _ = _stepped(ni, refined)
    h = jp.Array(p)
    for d in range(p.ndim):
        assert h.coords[d].data.shape == (int(np.prod(ni)), p.max_xcell)
        assert_bits_equal(h.coords[d].data, p.coords[d].data.cpu().numpy().T, f"coords[{d}]")
    np.testing.assert_array_equal(h.index.data, p.index.data.cpu().numpy().T.astype(bool))
    hT = jp.Array(T, p)
    assert_bits_equal(hT.data, T.data.cpu().numpy().T, "field")
    h32 = jp.Array("Float32", p)
    assert h32.coords[0].data.dtype == np.float32
    np.testing.assert_array_equal(h32.coords[0].data, h.coords[0].data.astype(np.float32))
    assert h.rng_counter == p.rng_counter == 2


@pytest.mark.parametrize("ni,refined", [((13, 7), False), ((11, 9), True), ((5, 6, 4), False)])
def test_round_trip_and_restart_continues_exactly(ni, refined, tmp_path):
    p, (T, S), Vd, dt, g = _stepped(ni, refined)
    path = jp.checkpointing_particles(str(tmp_path), p, particle_args=(T, S), t=0.5, dt=dt)
    data = jp.load_checkpoint(path)
    q = jp.TA("CUDA")("Float64", data["particles"])
    qT, qS = jp.TA("CUDA")("Float64", data["particle_args"], q)
    for d in range(p.ndim):
        assert_bits_equal(q.coords[d].data.cpu().numpy(), p.coords[d].data.cpu().numpy(), f"coords[{d}]")
    assert torch.equal(q.index.data, p.index.data)
    assert_bits_equal(qT.data.cpu().numpy(), T.data.cpu().numpy(), "T")
    assert q.rng_counter == p.rng_counter and data["time"] == 0.5
    for pp, (A, B) in ((p, (T, S)), (q, (qT, qS))):
        for _ in range(2):
            jp.advection_(pp, jp.RungeKutta2(), Vd, dt)
            jp.move_particles_(pp, (A, B))
            jp.inject_particles_(pp, (A, B))
    for d in range(p.ndim):
        assert_bits_equal(q.coords[d].data.cpu().numpy(), p.coords[d].data.cpu().numpy(), f"restart coords[{d}]")
    assert torch.equal(q.index.data, p.index.data)
    live = p.index.data.bool()
    assert_bits_equal(qS.data[live].cpu().numpy(), S.data[live].cpu().numpy(), "restart S")


def test_phase_ratios_round_trip():
    p, (T, S), _, _, g = _stepped((6, 5, 7))
    ph = torch.where(p.index.data.bool(), 1.0 + (p.coords[0].data > 0.5).double(), torch.nan)
    phases = jp.CellArray(ph.contiguous(), p.ni)
    pr = jp.PhaseRatios(2, p.ni)
    jp.update_phase_ratios_(pr, p, phases)
    h = jp.Array(pr, p)
    assert set(h.fields) == {"center", "vertex", "Vx", "Vy", "Vz", "xy", "yz", "xz"}
    assert_bits_equal(h.fields["xy"], pr.xy.cpu().numpy().T, "xy")
    back = jp.TA("CUDA")("Float64", h, p)
    for name in h.fields:
        assert torch.equal(getattr(back, name), getattr(pr, name)), name


def test_permute_full_size_round_trip():
    """The 1024^2-cell, 48-slot container (50M slots) through both directions."""
    g = W.grid((1024, 1024))
    p = jp.init_particles(jp.CUDABackend, 24, 48, 12, *g["grid_v"])
    h = jp.Array(p)
    assert h.coords[1].data.shape == (1024 * 1024, 48)
    np.testing.assert_array_equal(h.index.data[:, :24], True)
    np.testing.assert_array_equal(h.index.data[:, 24:], False)
    q = jp.TA("CUDA")("Float64", h)
    for d in range(2):
        assert torch.equal(torch.nan_to_num(q.coords[d].data, nan=-1.0), torch.nan_to_num(p.coords[d].data, nan=-1.0))
    assert torch.equal(q.index.data, p.index.data)
