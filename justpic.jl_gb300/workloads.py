"""Synthetic inputs with the shapes of the benchmark configurations.

The reference publishes no dataset for this path; every workload is a seeded
analytic setup in the style of its miniapps (README.md:29-113,
test/test_2D.jl:482-653, test/test_3D.jl:335-469). Host-side numpy only: grids
are ``LinRange`` objects, grid fields Fortran-ordered arrays with the Julia
shape, so the same inputs feed the CUDA library and the CPU oracle.
"""
from __future__ import annotations

import numpy as np

from .particles import LinRange


def expand_range(x: LinRange) -> LinRange:
    """One extra node on each side (test/test_2D.jl:35-42)."""
    dx = x[1] - x[0]
    return LinRange(x[0] - dx, x[len(x) - 1] + dx, len(x) + 2)


def grid(ni, L=None):
    """Uniform grid of ``ni`` cells on [0, L] per axis with the staggered
    ghost-node velocity grids of the reference's miniapps."""
    N = len(ni)
    L = L or (1.0,) * N
    xv = tuple(LinRange(0.0, L[d], ni[d] + 1) for d in range(N))
    dx = tuple(xv[d][1] - xv[d][0] for d in range(N))
    xc = tuple(LinRange(0.0 + dx[d] / 2, L[d] - dx[d] / 2, ni[d]) for d in range(N))
    grid_v = tuple(tuple(xv[d] if d == c else expand_range(xc[d]) for d in range(N)) for c in range(N))
    return {"ndim": N, "ni": tuple(ni), "xv": xv, "xc": xc, "dx": dx, "grid_v": grid_v}


def on_grid(f, axes) -> np.ndarray:
    """Evaluate f on the tensor grid of ``axes`` (Julia comprehension order,
    x fastest), returned Fortran-ordered."""
    mesh = np.meshgrid(*[np.asarray(a) for a in axes], indexing="ij")
    return np.asfortranarray(f(*mesh).astype(np.float64))


def stream_velocity(g):
    """README.md:66-78: vx = 250 sin(pi x) cos(pi y), vy = -250 cos(pi x) sin(pi y)."""
    vx = lambda x, y: 250.0 * np.sin(np.pi * x) * np.cos(np.pi * y)  # noqa: E731
    vy = lambda x, y: -250.0 * np.cos(np.pi * x) * np.sin(np.pi * y)  # noqa: E731
    return on_grid(vx, g["grid_v"][0]), on_grid(vy, g["grid_v"][1])


def rotation_velocity(g):
    """Rigid rotation about (0.5, 0.5): vx = -(y - 0.5), vy = x - 0.5."""
    vx = lambda x, y: -(y - 0.5)  # noqa: E731
    vy = lambda x, y: x - 0.5  # noqa: E731
    return on_grid(vx, g["grid_v"][0]), on_grid(vy, g["grid_v"][1])


def cellular_velocity_3d(g, drift=0.1):
    """vx = sin(pi x)cos(pi y)cos(pi z), vy = -cos(pi x)sin(pi y)cos(pi z),
    vz = drift (uniform), on the staggered 3D grids."""
    vx = lambda x, y, z: np.sin(np.pi * x) * np.cos(np.pi * y) * np.cos(np.pi * z)  # noqa: E731
    vy = lambda x, y, z: -np.cos(np.pi * x) * np.sin(np.pi * y) * np.cos(np.pi * z)  # noqa: E731
    vz = lambda x, y, z: drift + 0.0 * x  # noqa: E731
    gv = g["grid_v"]
    return on_grid(vx, gv[0]), on_grid(vy, gv[1]), on_grid(vz, gv[2])


def stream_velocity_3d(g):
    """test/test_3D.jl:53-56: vx = 250 sin(pi x)cos(pi z), vy = 0, vz = -250 cos(pi x)sin(pi z)."""
    vx = lambda x, y, z: 250.0 * np.sin(np.pi * x) * np.cos(np.pi * z)  # noqa: E731
    vy = lambda x, y, z: 0.0 * x  # noqa: E731
    vz = lambda x, y, z: -250.0 * np.cos(np.pi * x) * np.sin(np.pi * z)  # noqa: E731
    gv = g["grid_v"]
    return on_grid(vx, gv[0]), on_grid(vy, gv[1]), on_grid(vz, gv[2])


def gaussian_T(g, center=None, width2=0.01):
    """Vertex field exp(-|x - center|^2 / width2)."""
    N = g["ndim"]
    center = center or ((0.5, 0.75) if N == 2 else (0.5, 0.5, 0.5))

    def f(*x):
        r2 = sum((x[d] - center[d]) ** 2 for d in range(N))
        return np.exp(-r2 / width2)

    return on_grid(f, g["xv"])


def linear_T(g, axis):
    """Vertex field equal to the coordinate along ``axis`` (test_interpolation_kernels.jl:81-83)."""
    return on_grid(lambda *x: x[axis] + 0.0 * x[0], g["xv"])


def cfl_dt(g, V, factor=1.0):
    """dt = min over axes of dx / max|V| (README.md:77), times ``factor``
    (axes whose velocity is zero everywhere do not limit dt)."""
    return factor * min(g["dx"][d] / float(np.max(np.abs(V[d]))) for d in range(g["ndim"])
                        if np.max(np.abs(V[d])) > 0)


# The benchmark configurations (sizes, particle counts, steps).
CONFIGS = {
    "C1": dict(ni=(256, 256), nxcell=24, max_xcell=48, min_xcell=12, method="RK2", steps=750,
               velocity="stream", fields=0,
               desc="2D RK2 advection, FP64, 256x256 cells, stream-function velocity, advection!+move_particles!"),
    "C2": dict(ni=(1024, 1024), nxcell=24, max_xcell=48, min_xcell=12, method="RK2", steps=500,
               velocity="rotation", fields=1,
               desc="2D temperature advection, FP64, 1024x1024 cells, rigid rotation, advection!+move_particles!"
                    "+inject_particles!+grid2particle!+particle2grid!"),
    "C4": dict(ni=(2048, 2048), nxcell=24, max_xcell=48, min_xcell=12, method="RK4", steps=750,
               velocity="stream", fields=1,
               desc="2D split-precision comparison, 2048x2048 cells, stream-function velocity, RK4, C2 step"),
    "C5": dict(ni=(512, 512), nxcell=16, max_xcell=32, min_xcell=8, method="RK2", steps=100,
               velocity="stream+noise", fields=1, checkpoint_every=10,
               desc="2D adjoint run, FP64, 512x512 cells, stream-function velocity plus N(0, (0.1*250)^2) node "
                    "noise, misfit 0.5||particle2grid(T) - T_target||^2, gradients w.r.t. Vx, Vy, T0"),
    "C3": dict(ni=(128, 128, 128), nxcell=24, max_xcell=48, min_xcell=12, method="RK2", steps=300,
               velocity="cellular3d", fields=1,
               desc="3D temperature advection, FP64, 128^3 cells, cellular flow + 0.1 z drift, advection!"
                    "+move_particles!+inject_particles!+particle2grid!"),
}


def pure_shear(ni=(128, 128), rate=-1.0):
    """The phase miniapp's pure-shear setup (test/test_2D.jl:385-433): unit
    square centred on the origin, ghost-node velocity grids
    LinRange(-L/2 - dx/2, L/2 + dx/2, n + 2), vx = x * rate, vy = -y * rate.
    Returns (grid, (Vx, Vy), dt) with dt = 0.25 * min(dx) / max|V|."""
    nx, ny = ni
    xv = (LinRange(-0.5, 0.5, nx + 1), LinRange(-0.5, 0.5, ny + 1))
    dx = (1.0 / nx, 1.0 / ny)
    xc = tuple(LinRange(-0.5 + dx[d] / 2, 0.5 - dx[d] / 2, ni[d]) for d in range(2))
    ext = tuple(LinRange(-0.5 - dx[d] / 2, 0.5 + dx[d] / 2, ni[d] + 2) for d in range(2))
    grid_v = ((xv[0], ext[1]), (ext[0], xv[1]))
    g = {"ndim": 2, "ni": tuple(ni), "xv": xv, "xc": xc, "dx": dx, "grid_v": grid_v}
    x = np.asarray(xv[0])
    y = np.asarray(xv[1])
    Vx = np.asfortranarray(np.repeat((x * rate)[:, None], ny + 2, axis=1))
    Vy = np.asfortranarray(np.repeat((-y * rate)[None, :], nx + 2, axis=0))
    dt = 0.25 * min(dx) / max(float(np.max(np.abs(Vx))), float(np.max(np.abs(Vy))))
    return g, (Vx, Vy), dt


def shear_phases(coords, index):
    """Phase 1 where x < y, else 2, on live slots (test/test_2D.jl:387-401);
    dead slots hold NaN."""
    x, y = (np.asarray(c) for c in coords[:2])
    return np.where(np.asarray(index).astype(bool), np.where(x < y, 1.0, 2.0), np.nan)


def perturbed_stream_velocity(g, sigma=0.1 * 250.0, seed=5):
    """The stream-function velocity plus i.i.d. N(0, sigma^2) noise on every
    staggered node (fixed over time)."""
    rng = np.random.default_rng(seed)
    return tuple(np.asfortranarray(v + sigma * rng.standard_normal(v.shape)) for v in stream_velocity(g))


def fourier_target(g, nmodes=16, kmax=4, seed=11):
    """A smooth random vertex field: the sum of ``nmodes`` Fourier modes with
    integer wavenumbers 0 <= kx, ky <= kmax, random phases and N(0, 1/4)
    amplitudes."""
    rng = np.random.default_rng(seed)
    kx = rng.integers(0, kmax + 1, nmodes)
    ky = rng.integers(0, kmax + 1, nmodes)
    ph = rng.uniform(0.0, 2.0 * np.pi, nmodes)
    amp = 0.5 * rng.standard_normal(nmodes)

    def f(x, y):
        out = np.zeros_like(x)
        for m in range(nmodes):
            out += amp[m] * np.cos(2.0 * np.pi * (kx[m] * x + ky[m] * y) + ph[m])
        return out

    return on_grid(f, g["xv"])


def setup(name: str, ni=None):
    """Grid, velocity, vertex temperature and dt of a configuration
    (``ni`` overrides the cell counts, e.g. for a small profiling case)."""
    cfg = dict(CONFIGS[name])
    if ni is not None:
        cfg["ni"] = tuple(ni)
    g = grid(cfg["ni"])
    if cfg["velocity"] == "stream":
        V = stream_velocity(g)
    elif cfg["velocity"] == "stream+noise":
        V = perturbed_stream_velocity(g)
        cfg["T_target"] = fourier_target(g)
    elif cfg["velocity"] == "rotation":
        V = rotation_velocity(g)
    else:
        V = cellular_velocity_3d(g)
    T = gaussian_T(g) if g["ndim"] == 2 else gaussian_T(g, width2=0.15 ** 2)
    dt = cfl_dt(g, V)
    cfg.update(grid=g, V=V, T=T, dt=dt)
    return cfg


__all__ = ["expand_range", "grid", "on_grid", "stream_velocity", "rotation_velocity", "cellular_velocity_3d",
           "stream_velocity_3d", "perturbed_stream_velocity", "fourier_target", "gaussian_T", "linear_T", "cfl_dt",
           "CONFIGS", "setup"]
