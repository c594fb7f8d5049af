"""Golden vectors of the hot path, generated by the CPU oracle.

The reference (Julia) cannot run here and publishes no reference outputs, so
its own known-answer tests pin the oracle (tests/test_oracle_kat.py) and this
script freezes the oracle's results on a set of seeded runs: small 2D and 3D
grids (uniform and refined), every integrator, with a particle field, and the
C1 configuration (256^2 cells, 24/48/12 particles per cell) at full size for
a few steps. Every input is made of exact IEEE operations (LinRange grids,
polynomial velocity and field values, numpy's PCG64 stream for the refined
grids), so the vectors are the same on every machine.

What is stored (golden.json): per run, the live-particle count after every
step and SHA-256 digests of the final occupancy mask, the coordinates and the
particle field of the live slots (dead slots hashed as 0), the gridded field
(vertices without particles hashed as a fixed value), and of the transfers
beside the hot path applied to the final state (grid2particle_flip!,
centroid2particle!, particle2centroid!).

    python tests/golden/make_golden.py        # rewrite golden.json

tests/test_golden.py checks the oracle against the file; test_gpu_golden.py
checks the CUDA library against it.
"""
from __future__ import annotations

import hashlib
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

from justpic_gb300 import workloads as W  # noqa: E402
from justpic_gb300.particles import LinRange  # noqa: E402

GOLDEN = os.path.join(HERE, "golden.json")
SEED = 0x4A50
EMPTY_VERTEX = -12345.0

# name: (cells, nxcell, max_xcell, min_xcell, method, alpha, steps, refined)
CASES = {
    "2d_4x4_rk2": ((4, 4), 24, 48, 12, "rk2", 0.5, 6, False),
    "2d_8x8_euler": ((8, 8), 24, 48, 12, "euler", 0.5, 6, False),
    "2d_16x16_rk4": ((16, 16), 16, 32, 8, "rk4", 0.5, 6, False),
    "2d_13x7_rk2_alpha": ((13, 7), 24, 48, 12, "rk2", 2.0 / 3.0, 6, False),
    "2d_11x9_refined_rk2": ((11, 9), 24, 48, 12, "rk2", 0.5, 6, True),
    "3d_4x4x4_rk2": ((4, 4, 4), 24, 48, 12, "rk2", 0.5, 4, False),
    "3d_6x5x7_refined_rk4": ((6, 5, 7), 24, 48, 12, "rk4", 0.5, 4, True),
    "c1_256x256_rk2": ((256, 256), 24, 48, 12, "rk2", 0.5, 5, False),
}


def refined_vertices(n, seed, stretch=0.35):
    rng = np.random.default_rng(seed)
    w = 1.0 + stretch * rng.uniform(-1, 1, n)
    x = np.concatenate([[0.0], np.cumsum(w)])
    return x / x[-1]


def make_grid(ni, refined):
    N = len(ni)
    if not refined:
        return W.grid(ni)
    xv = tuple(refined_vertices(ni[d], 7 + d) for d in range(N))
    xc = tuple(0.5 * (x[1:] + x[:-1]) for x in xv)

    def expand(x):
        return np.concatenate([[x[0] - (x[1] - x[0])], x, [x[-1] + (x[-1] - x[-2])]])

    grid_v = tuple(tuple(xv[d] if d == c else expand(xc[d]) for d in range(N)) for c in range(N))
    return {"ndim": N, "ni": tuple(ni), "xv": xv, "xc": xc, "grid_v": grid_v}


def velocity(g):
    """Polynomial swirl (exact arithmetic): vx = 4 (y - 1/2) x (1 - x),
    vy = -4 (x - 1/2) y (1 - y) (3D: the same in x-y, vz = (z - 1/2) / 4)."""
    N = g["ndim"]
    if N == 2:
        vx = lambda x, y: 4.0 * (y - 0.5) * x * (1.0 - x)  # noqa: E731
        vy = lambda x, y: -4.0 * (x - 0.5) * y * (1.0 - y)  # noqa: E731
        return W.on_grid(vx, g["grid_v"][0]), W.on_grid(vy, g["grid_v"][1])
    vx = lambda x, y, z: 4.0 * (y - 0.5) * x * (1.0 - x)  # noqa: E731
    vy = lambda x, y, z: -4.0 * (x - 0.5) * y * (1.0 - y)  # noqa: E731
    vz = lambda x, y, z: 0.25 * (z - 0.5)  # noqa: E731
    gv = g["grid_v"]
    return W.on_grid(vx, gv[0]), W.on_grid(vy, gv[1]), W.on_grid(vz, gv[2])


def field(g):
    """Vertex field x + 2y (+ 3z)."""
    return W.on_grid(lambda *x: sum((d + 1.0) * x[d] for d in range(len(x))), g["xv"])


def dt_of(g, V):
    dx = min(float(np.min(np.diff(np.asarray(x)))) for x in g["xv"])
    vmax = max(float(np.max(np.abs(v))) for v in V)
    return 0.8 * dx / vmax


def digest(a) -> str:
    return hashlib.sha256(np.ascontiguousarray(a, dtype=np.float64).tobytes()).hexdigest()


def grid_digest(F):
    return digest(np.asfortranarray(np.where(np.isnan(F), EMPTY_VERTEX, F)).ravel(order="F"))


def summarise(index, coords, T, F, live_per_step, flip, c2p, p2c):
    live = np.asarray(index).astype(bool)
    return {
        "live_per_step": [int(v) for v in live_per_step],
        "index": hashlib.sha256(np.ascontiguousarray(live, dtype=np.uint8).tobytes()).hexdigest(),
        "coords": [digest(np.where(live, c, 0.0)) for c in coords],
        "field": digest(np.where(live, T, 0.0)),
        "grid_field": grid_digest(F),
        "grid2particle_flip": digest(np.where(live, flip, 0.0)),
        "centroid2particle": digest(np.where(live, c2p, 0.0)),
        "particle2centroid": grid_digest(p2c),
    }


def centre_field(g):
    """Cell-centred field x + 2y (+ 3z) on the cell centres."""
    return W.on_grid(lambda *x: sum((d + 1.0) * x[d] for d in range(len(x))), g["xc"])


def inputs(name):
    ni, nxcell, mx, mn, method, alpha, steps, refined = CASES[name]
    g = make_grid(ni, refined)
    V = velocity(g)
    return g, V, field(g), dt_of(g, V), (nxcell, mx, mn, method, alpha, steps)


def run_oracle(name):
    from oracle import oracle as O

    g, V, T0, dt, (nxcell, mx, mn, method, alpha, steps) = inputs(name)
    m = {"euler": O.EULER, "rk2": O.RK2, "rk4": O.RK4}[method]
    uniform = not CASES[name][7]
    o = O.OracleParticles(tuple(tuple(np.asarray(x, dtype=np.float64) for x in c) for c in g["grid_v"]),
                          nxcell, mx, mn, uniform=uniform, seed=SEED)
    o.init_particles()
    T = o.cell_array()
    o.grid2particle(T, T0)
    live = []
    for _ in range(steps):
        o.advection(m, alpha, V, dt)
        o.move_particles([T])
        o.inject_particles([T])
        live.append(int(o.index.sum()))
    F = np.asfortranarray(np.zeros(tuple(n + 1 for n in o.n)))
    o.particle2grid(F, T)
    flip = T.copy()
    o.grid2particle_flip(flip, T0, np.asfortranarray(0.5 * T0), 0.25)
    c2p = o.cell_array()
    o.centroid2particle(c2p, centre_field(g))
    p2c = np.asfortranarray(np.zeros(tuple(o.n)))
    o.particle2centroid(p2c, T)
    return summarise(o.index, o.coords, T, F, live, flip, c2p, p2c)


def run_gpu(name):
    import justpic_gb300 as jp

    g, V, T0, dt, (nxcell, mx, mn, method, alpha, steps) = inputs(name)
    pm = {"euler": jp.Euler(), "rk2": jp.RungeKutta2(alpha), "rk4": jp.RungeKutta4()}[method]
    grids = g["grid_v"]
    if CASES[name][7]:  # vector grids
        grids = tuple(tuple(np.asarray(x, dtype=np.float64) for x in c) for c in grids)
    p = jp.init_particles(jp.CUDABackend, nxcell, mx, mn, *grids, seed=SEED)
    (T,) = jp.init_cell_arrays(p, 1)
    jp.grid2particle_(T, jp.TA("CUDA")(T0), p)
    Vd = tuple(jp.TA("CUDA")(v) for v in V)
    live = []
    for _ in range(steps):
        jp.advection_(p, pm, Vd, dt)
        jp.move_particles_(p, (T,))
        jp.inject_particles_(p, (T,))
        live.append(int(p.index.data.sum()))
    F = jp.grid_field(tuple(n + 1 for n in p.ni))
    jp.particle2grid_(F, T, p)
    flip = jp.CellArray(T.data.clone(), p.ni)
    jp.grid2particle_flip_(flip, None, jp.TA("CUDA")(T0), jp.TA("CUDA")(np.asfortranarray(0.5 * T0)), p, 0.25)
    (c2p,) = jp.init_cell_arrays(p, 1)
    jp.centroid2particle_(c2p, jp.TA("CUDA")(centre_field(g)), p)
    p2c = jp.grid_field(tuple(p.ni))
    jp.particle2centroid_(p2c, T, p)
    return summarise(p.index.numpy(), [c.numpy() for c in p.coords], T.numpy(), F.cpu().numpy(), live,
                     flip.numpy(), c2p.numpy(), p2c.cpu().numpy())


def load():
    with open(GOLDEN) as f:
        return json.load(f)


def main():
    out = {"generator": "tests/golden/make_golden.py (CPU oracle, seed 0x4A50)", "cases": {}}
    for name in CASES:
        out["cases"][name] = run_oracle(name)
        print(name, out["cases"][name]["live_per_step"])
    with open(GOLDEN, "w") as f:
        json.dump(out, f, indent=1, sort_keys=True)
        f.write("\n")


if __name__ == "__main__":
    main()
