"""Edge cases of the split-precision form (int32 cell + FP32 offset), which has
no oracle: the rules are stated in cell units and checked directly.

  * an offset exactly 1.0 on an axis belongs to the next cell, where it becomes
    0.0 exactly; 0.0 stays; 1.0 in the last cell of an axis leaves the domain;
  * NaN offsets of a live particle: the particle leaves (counted as such);
  * an offset two cells away: the particle is dropped and counted as moved too
    far (with a warning), never written into a cell it does not belong to;
  * an empty container: injection gives every cell's first quadrant min_xQ
    particles, identically in two containers seeded alike.
"""
import warnings

import numpy as np
import pytest
import torch

from _harness import W, jp

pytestmark = pytest.mark.gpu


def _container(ni=(8, 6), nxcell=8, max_xcell=24, min_xcell=4):
    g = W.grid(ni)
    p = jp.init_particles(jp.CUDABackend, nxcell, max_xcell, min_xcell, *g["grid_v"])
    return g, p, jp.init_offsets(p)


def _first_live(p):
    live = p.index.numpy().astype(bool)
    return live.argmax(axis=0)  # the first live slot of every cell


def test_offsets_on_faces():
    g, p, xi = _container()
    ni = p.ni
    nc = int(np.prod(ni))
    s = _first_live(p)
    cells = np.arange(nc)
    x = xi[0].data
    # the first live particle of every cell: x offset exactly 1.0 (right face), y untouched
    x[torch.from_numpy(s).cuda(), torch.from_numpy(cells).cuda()] = 1.0
    y_before = xi[1].numpy()[s, cells].copy()
    live0 = int(p.index.data.sum())
    jp.move_counts(p, clear=True)
    jp.move_particles_f32_(p, xi)
    counts = jp.move_counts(p)
    # the last column's particles left the domain, every other one is in the next cell at offset 0.0
    assert counts["left_domain"] == ni[1] and counts["moved_too_far"] == 0
    live = p.index.numpy().astype(bool)
    xa, ya = xi[0].numpy(), xi[1].numpy()
    found = 0
    for c in cells:
        i, j = c % ni[0], c // ni[0]
        if i == ni[0] - 1:
            continue
        dest = c + 1
        hit = live[:, dest] & (xa[:, dest] == 0.0) & (ya[:, dest] == y_before[c])
        found += int(hit.any())
    assert found == nc - ni[1]
    assert int(p.index.data.sum()) + counts["no_free_slot"] == live0 - ni[1]
    x_live = xa[live]
    assert np.all((x_live >= 0) & (x_live < 1))


def test_offset_zero_stays():
    g, p, xi = _container()
    s = _first_live(p)
    cells = np.arange(int(np.prod(p.ni)))
    xi[0].data[torch.from_numpy(s).cuda(), torch.from_numpy(cells).cuda()] = 0.0
    before = p.index.data.clone()
    jp.move_counts(p, clear=True)
    jp.move_particles_f32_(p, xi)
    assert torch.equal(before, p.index.data)
    assert sum(jp.move_counts(p).values()) == 0


def test_nan_offsets_leave():
    g, p, xi = _container()
    s = _first_live(p)
    cells = np.arange(int(np.prod(p.ni)))
    xi[1].data[torch.from_numpy(s).cuda(), torch.from_numpy(cells).cuda()] = float("nan")
    live0 = int(p.index.data.sum())
    jp.move_counts(p, clear=True)
    jp.move_particles_f32_(p, xi)
    counts = jp.move_counts(p)
    assert counts["left_domain"] == len(cells)
    assert int(p.index.data.sum()) == live0 - len(cells)
    live = p.index.numpy().astype(bool)
    for d in range(2):
        assert np.all(np.isfinite(xi[d].numpy()[live]))
        assert np.all(np.isnan(xi[d].numpy()[~live]))


def test_far_moves_are_dropped_and_counted():
    g, p, xi = _container(ni=(10, 8))
    s = _first_live(p)
    ni = p.ni
    # interior cells only: two cells to the right stays inside the grid
    cells = np.array([c for c in range(int(np.prod(ni))) if c % ni[0] < ni[0] - 2])
    xi[0].data[torch.from_numpy(s[cells]).cuda(), torch.from_numpy(cells).cuda()] = 2.5
    live0 = int(p.index.data.sum())
    jp.move_counts(p, clear=True)
    with warnings.catch_warnings(record=True) as w:
        warnings.simplefilter("always")
        jp.move_particles_f32_(p, xi)
    counts = jp.move_counts(p)
    assert counts["moved_too_far"] == len(cells) and counts["left_domain"] == 0
    assert int(p.index.data.sum()) == live0 - len(cells)
    assert any("more than one cell" in str(x.message) for x in w)
    live = p.index.numpy().astype(bool)
    assert np.all((xi[0].numpy()[live] >= 0) & (xi[0].numpy()[live] < 1))


def test_empty_container_is_reseeded():
    outs = []
    for _ in range(2):
        g, p, xi = _container(ni=(7, 5), nxcell=8, max_xcell=24, min_xcell=8)
        T, = jp.init_cell_arrays_f32(p, 1)
        p.index.data.zero_()
        for d in range(2):
            xi[d].data.fill_(float("nan"))
        with warnings.catch_warnings():
            warnings.simplefilter("ignore")  # the first particles of a cell have no neighbour to copy from
            jp.inject_particles_f32_(p, xi, (T,))
        live = p.index.numpy().astype(bool)
        x0, x1 = xi[0].numpy(), xi[1].numpy()
        inq = live & (x0 > 0) & (x0 < 0.5) & (x1 > 0) & (x1 < 0.5)
        assert np.all(inq.sum(axis=0) >= 2), "each cell's first quadrant holds min_xcell / 4 particles"
        assert np.all((x0[live] > 0) & (x0[live] < 1) & (x1[live] > 0) & (x1[live] < 1))
        outs.append((p.index.data.clone(), xi[0].data.clone(), xi[1].data.clone()))
    assert torch.equal(outs[0][0], outs[1][0])
    for d in (1, 2):
        assert torch.equal(outs[0][d].nan_to_num(-7.0), outs[1][d].nan_to_num(-7.0))
