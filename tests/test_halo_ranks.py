"""update_cell_halo! (src/CellArrays/ImplicitGlobalGrid.jl:36-41) on two gloo
ranks on CPU: each rank holds a local slab of a global CellArray (overlap 2),
its halo planes are spoiled, and the exchange must bring back the global
values: the plane below from the neighbour below, the plane above from the
neighbour above, every slot of every array (coordinates, occupancy, field).
Cases: 2D split along x, 3D split along y, and a periodic axis with two
ranks. No GPU."""
import json
import os
import socket
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

RANK_SCRIPT = r"""
import json, os, sys
sys.path.insert(0, sys.argv[1])
import numpy as np, torch
import torch.distributed as dist
dist.init_process_group("gloo")
rank = dist.get_rank()
from justpic_gb300.particles import CellArray
from justpic_gb300.halo import CartesianGrid, update_cell_halo_

def slab(glob, ni_g, axis, lo, n):
    # the local cells lo .. lo+n-1 along axis (periodic wrap) of a global (ncap, ncells) array
    g = glob.reshape(glob.shape[0], *reversed(ni_g))  # (ncap, [z,] y, x)
    ax = g.ndim - 1 - axis
    idx = [(lo + k) % ni_g[axis] for k in range(n)]
    loc = np.take(g, idx, axis=ax)
    ni = list(ni_g); ni[axis] = n
    return np.ascontiguousarray(loc.reshape(glob.shape[0], -1)), tuple(ni)

results = {}
for name, ni_g, axis, period, dims in [("2d_x", (10, 7), 0, False, (2, 1)),
                                     ("3d_y", (5, 10, 4), 1, False, (1, 2, 1)),
                                     ("2d_x_periodic", (8, 5), 0, True, (2, 1))]:
    rng = np.random.default_rng(3)
    ncells = int(np.prod(ni_g))
    globs = [rng.standard_normal((6, ncells)), (rng.random((6, ncells)) < 0.5).astype(np.uint8),
             rng.standard_normal((6, ncells)).astype(np.float32)]
    ol = 2
    n = ni_g[axis] // 2 + ol // 2 if not period else ni_g[axis] // 2 + ol
    lo = rank * (ni_g[axis] // 2) - (0 if not period else ol // 2)
    if not period:
        lo = 0 if rank == 0 else ni_g[axis] - n
    locs = []
    for gl in globs:
        a, ni = slab(gl, ni_g, axis, lo, n)
        locs.append((a, ni))
    arrays = [CellArray(torch.from_numpy(a.copy()), ni) for a, ni in locs]
    # spoil the halo planes the exchange is to fill
    grid = CartesianGrid(dims=dims, periods=tuple(period if d == axis else False for d in range(3)),
                         overlaps=(ol, ol, ol))
    ncap = 6
    full = [a.data.clone() for a in arrays]
    lin = np.arange(int(np.prod(ni))).reshape(tuple(reversed(ni)))
    first = np.take(lin, [0], axis=lin.ndim - 1 - axis).ravel()
    last = np.take(lin, [n - 1], axis=lin.ndim - 1 - axis).ravel()
    spoil = []
    if grid.neighbour(rank, axis, -1) is not None:
        spoil.append(first)
    if grid.neighbour(rank, axis, +1) is not None:
        spoil.append(last)
    for a in arrays:
        for cells in spoil:
            a.data[:, torch.from_numpy(cells)] = 0
    update_cell_halo_(*arrays, grid=grid)
    results[name] = all(torch.equal(a.data, f) for a, f in zip(arrays, full)) and len(spoil) > 0
dist.barrier()
dist.destroy_process_group()
with open(sys.argv[2], "w") as f:
    json.dump(results, f)
"""


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_halo_exchange_two_gloo_ranks(tmp_path):
    pytest.importorskip("torch.distributed")
    port = _free_port()
    script = tmp_path / "rank.py"
    script.write_text(RANK_SCRIPT)
    procs = []
    for r in range(2):
        env = dict(os.environ, RANK=str(r), LOCAL_RANK=str(r), WORLD_SIZE="2", MASTER_ADDR="127.0.0.1",
                   MASTER_PORT=str(port), CUDA_VISIBLE_DEVICES="")
        procs.append(subprocess.Popen([sys.executable, str(script), ROOT, str(tmp_path / f"out{r}.json")],
                                      env=env, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True))
    logs = []
    for pr in procs:
        try:
            logs.append(pr.communicate(timeout=240)[0])
        except subprocess.TimeoutExpired:
            pr.kill()
            logs.append(pr.communicate()[0])
    for r, pr in enumerate(procs):
        assert pr.returncode == 0, f"rank {r} failed:\n{logs[r]}"
    for r in range(2):
        out = json.loads((tmp_path / f"out{r}.json").read_text())
        assert out == {"2d_x": True, "3d_y": True, "2d_x_periodic": True}, (r, out)


def test_plane_rule_single_process():
    """The planes chosen along an axis: plane ol to the rank below, plane
    n - ol + 1 to the rank above (1-based), received into the last / first
    plane; neighbours of a non-periodic edge are absent."""
    import torch

    from justpic_gb300.halo import CartesianGrid, _plane_cells

    g = CartesianGrid(dims=(3, 2), periods=(False, True), overlaps=(2, 2, 2))
    assert g.coords(4) == (1, 1) and g.rank_of((1, 1)) == 4
    assert g.neighbour(0, 0, -1) is None and g.neighbour(0, 0, +1) == 1
    assert g.neighbour(0, 1, -1) == 3 and g.neighbour(3, 1, +1) == 0
    cells = _plane_cells((4, 3), 0, 1)
    assert torch.equal(torch.sort(cells).values, torch.tensor([1, 5, 9]))
