"""GPU parity at the benchmark configurations' own sizes: the CUDA library
against the CPU oracle on the same seeded inputs, step by step, comparing
occupancy masks, coordinates (all slots), the particle field (live slots) and
the gridded field bit for bit.

  * C1: 256^2 cells, 24/48/12 particles per cell, stream-function velocity,
    RK2, advection! + move_particles!, all 750 steps (compared every 250);
  * C2: 1024^2 cells, rigid rotation, the reference miniapp cycle
    (test/test_2D.jl:516-524: particle2grid!, advection!, move_particles!,
    inject_particles!, grid2particle!), 3 steps;
  * C3: 128^3 cells, cellular flow + z drift, particle2grid!, advection!,
    move_particles!, inject_particles! (trilinear), 2 steps.

The oracle uses every host core; these runs take tens of seconds each."""
import os

import numpy as np
import pytest

from _harness import O, W, assert_bits_equal, jp

pytestmark = pytest.mark.gpu


class FullPair:
    """One workload of justpic_gb300.workloads in the oracle and on the GPU."""

    def __init__(self, name):
        O.set_threads(os.cpu_count() or 1)
        self.cfg = cfg = W.setup(name)
        g = cfg["grid"]
        grids = tuple(tuple(np.asarray(x) for x in comp) for comp in g["grid_v"])
        self.o = O.OracleParticles(grids, cfg["nxcell"], cfg["max_xcell"], cfg["min_xcell"], uniform=True)
        self.o.init_particles()
        self.p = jp.init_particles(jp.CUDABackend, cfg["nxcell"], cfg["max_xcell"], cfg["min_xcell"],
                                   *g["grid_v"])
        self.nf = cfg["fields"]
        self.of = [self.o.cell_array() for _ in range(self.nf)]
        self.pf = list(jp.init_cell_arrays(self.p, self.nf))
        self.V = cfg["V"]
        self.Vd = tuple(jp.TA("CUDA")(v) for v in self.V)
        self.dt = cfg["dt"]
        self.Fo = np.asfortranarray(cfg["T"].copy())
        self.Fg = jp.TA("CUDA")(cfg["T"])
        jp.set_synchronous(self.p, False)
        if self.nf:
            self.o.grid2particle(self.of[0], self.Fo)
            jp.grid2particle_(self.pf[0], self.Fg, self.p)

    def step(self, ops):
        o, p = self.o, self.p
        for op in ops:
            if op == "particle2grid!":
                o.particle2grid(self.Fo, self.of[0])
                jp.particle2grid_(self.Fg, self.pf[0], p)
            elif op == "advection!":
                assert o.advection(O.RK2, 0.5, self.V, self.dt) == 0
                jp.advection_(p, jp.RungeKutta2(), self.Vd, self.dt)
            elif op == "move_particles!":
                assert o.move_particles(self.of) == 0
                jp.move_particles_(p, tuple(self.pf))
            elif op == "inject_particles!":
                assert o.inject_particles(self.of) == 0
                jp.inject_particles_(p, tuple(self.pf))
            elif op == "grid2particle!":
                o.grid2particle(self.of[0], self.Fo)
                jp.grid2particle_(self.pf[0], self.Fg, p)

    def assert_same(self, what):
        jp.synchronize(self.p)
        idx_o = self.o.index
        idx_g = self.p.index.numpy()
        assert np.array_equal(idx_o, idx_g), f"{what}: index masks differ in {np.sum(idx_o != idx_g)} slots"
        assert np.array_equal(idx_o.sum(axis=0), idx_g.astype(np.int64).sum(axis=0)), f"{what}: occupancy"
        for d in range(self.o.ndim):
            assert_bits_equal(self.o.coords[d], self.p.coords[d].numpy(), f"{what}: coords[{d}]")
        live = idx_o.astype(bool)
        for k in range(self.nf):
            assert_bits_equal(self.of[k][live], self.pf[k].numpy()[live], f"{what}: field[{k}] (live slots)")
        if self.nf:
            assert_bits_equal(self.Fo, self.Fg.cpu().numpy(), f"{what}: gridded field")


def test_c1_full_size_750_steps():
    fp = FullPair("C1")
    ops = ["advection!", "move_particles!"]
    live0 = int(fp.o.index.sum())
    for step in range(1, 751):
        fp.step(ops)
        if step % 250 == 0:
            fp.assert_same(f"C1 step {step}")
    counts = jp.move_counts(fp.p)
    assert counts["moved_too_far"] == 0, counts
    # C1 has no injection: every particle the run lost was removed by a move, and counted
    assert live0 - int(fp.o.index.sum()) == counts["left_domain"] + counts["no_free_slot"]


def test_c2_full_size_miniapp_cycle():
    fp = FullPair("C2")
    ops = ["particle2grid!", "advection!", "move_particles!", "inject_particles!", "grid2particle!"]
    for step in range(3):
        fp.step(ops)
        fp.assert_same(f"C2 step {step}")
    assert jp.move_counts(fp.p)["moved_too_far"] == 0


def test_c3_full_size_3d_cycle():
    fp = FullPair("C3")
    ops = ["particle2grid!", "advection!", "move_particles!", "inject_particles!"]
    for step in range(2):
        fp.step(ops)
        fp.assert_same(f"C3 step {step}")
    assert jp.move_counts(fp.p)["moved_too_far"] == 0
