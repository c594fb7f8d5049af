"""Checkpoint files (src/IO/JLD2.jl:1-129) on the host: the archive holds the
reference's entries and reads back exactly; names follow checkpoint_name."""
import os

import numpy as np
import pytest

import justpic_gb300 as jp
from justpic_gb300 import conversion as C


def _host_particles(ni=(5, 3), M=8, seed=0x4A50):
    rng = np.random.default_rng(1)
    nc = int(np.prod(ni))
    idx = rng.random((nc, M)) < 0.6
    coords = tuple(C.HostCellArray(np.where(idx, rng.random((nc, M)), np.nan), ni) for _ in ni)
    xi_vel = tuple(tuple(np.linspace(0, 1, n + (1 if d == c else 2)) for d, n in enumerate(ni)) for c in range(len(ni)))
    return C.HostParticles(coords, C.HostCellArray(idx, ni), 4, M, 2, nc * M, xi_vel, True, seed, 7)


def test_checkpoint_names():
    assert C.checkpoint_name("out").endswith(os.path.join("out", "particles_checkpoint.npz"))
    assert C.checkpoint_name("out", 3).endswith("particles_checkpoint0003.npz")  # lpad 4 (JLD2.jl:4-6)


def test_checkpoint_round_trip(tmp_path):
    hp = _host_particles()
    ph = C.HostCellArray(np.arange(15 * 8, dtype=np.float64).reshape(15, 8), (5, 3))
    pr = C.HostPhaseRatios(2, (5, 3), {"center": np.full((15, 2), 0.5), "vertex": np.full((24, 2), 0.25)})
    args = (C.HostCellArray(np.ones((15, 8)), (5, 3)), C.HostCellArray(np.zeros((15, 8)), (5, 3)))
    path = jp.checkpointing_particles(str(tmp_path), hp, 12, phases=ph, phase_ratios=pr, t=1.5, dt=0.25,
                                      particle_args=args, step=42, extra=np.arange(3))
    assert os.path.basename(path) == "particles_checkpoint0012.npz"
    assert sorted(os.listdir(tmp_path)) == ["particles_checkpoint0012.npz"]  # no temporary left behind
    data = jp.load_checkpoint(path)
    assert set(data) == {"particles", "phases", "phase_ratios", "chain", "time", "timestep", "particle_args",
                         "step", "extra"}
    q = data["particles"]
    for d in range(2):
        np.testing.assert_array_equal(q.coords[d].data, hp.coords[d].data)
    np.testing.assert_array_equal(q.index.data, hp.index.data)
    assert (q.nxcell, q.max_xcell, q.min_xcell, q.seed, q.rng_counter, q.uniform) == (4, 8, 2, 0x4A50, 7, True)
    for c in range(2):
        for d in range(2):
            np.testing.assert_array_equal(q.xi_vel[c][d], hp.xi_vel[c][d])
    np.testing.assert_array_equal(data["phases"].data, ph.data)
    np.testing.assert_array_equal(data["phase_ratios"].fields["vertex"], pr.fields["vertex"])
    assert data["time"] == 1.5 and data["timestep"] == 0.25 and data["chain"] is None and data["step"] == 42
    assert len(data["particle_args"]) == 2 and np.all(data["particle_args"][0].data == 1.0)
    np.testing.assert_array_equal(data["extra"], np.arange(3))


def test_checkpoint_rejects_marker_chains_and_reserved_keys(tmp_path):
    hp = _host_particles()
    with pytest.raises(jp.ArgumentError):
        jp.checkpointing_particles(str(tmp_path), hp, chain=object())
    with pytest.raises(jp.ArgumentError):
        jp.checkpointing_particles(str(tmp_path), hp, time=3.0)
