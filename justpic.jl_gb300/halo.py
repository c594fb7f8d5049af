"""``update_cell_halo!`` (src/CellArrays/ImplicitGlobalGrid.jl:36-41): the halo
exchange of CellArrays between the ranks of a Cartesian process grid, the step
that the reference's MPI runs take before ``move_particles!``
(scripts/temperature_advection_MPI.jl:87-98) so that particles that crossed a
rank boundary are seen by the neighbouring rank.

The reference delegates each array to ``ImplicitGlobalGrid.update_halo!``
(ImplicitGlobalGrid.jl 0.16/0.17, a dependency not vendored with the
reference). Its published rule, with a halo one plane wide, restated here:
local arrays of neighbouring ranks overlap by ``ol`` planes along an axis; a
rank sends its plane ``ol`` (1-based) to the neighbour below, which writes it
into its last plane, and its plane ``n - ol + 1`` to the neighbour above, which
writes it into its first plane; axes are processed in order (x, then y, then
z) so that edge and corner halos arrive through the earlier exchanges; a
periodic axis wraps around; an axis with a single rank and no periodicity, or
with ``ol < 2``, exchanges nothing. A CellArray's planes are its cells with a
fixed index along the axis, every slot included.

This is host logic over ``torch.distributed`` point-to-point messages: with
the gloo backend on CPU tensors (how the tests run it, two ranks) or with NCCL
on device tensors. It launches no kernel of this library.
"""
from __future__ import annotations

from dataclasses import dataclass
from typing import Sequence

import torch

from ._native import ArgumentError
from .particles import CellArray


@dataclass(frozen=True)
class CartesianGrid:
    """The process grid of ``init_global_grid``: ``dims`` ranks per axis,
    ``periods`` per axis, ``overlaps`` (planes shared by neighbouring local
    arrays, per axis, in the arrays' own cell index space). Rank r sits at the
    coordinates of r in column-major order (x fastest)."""

    dims: Sequence[int]
    periods: Sequence[bool] = (False, False, False)
    overlaps: Sequence[int] = (2, 2, 2)

    def coords(self, rank: int):
        out, r = [], int(rank)
        for n in self.dims:
            out.append(r % n)
            r //= n
        return tuple(out)

    def rank_of(self, coords) -> int:
        r, stride = 0, 1
        for c, n in zip(coords, self.dims):
            r += c * stride
            stride *= n
        return r

    def neighbour(self, rank: int, axis: int, side: int):
        """The rank below (side -1) or above (+1) along ``axis``, or None."""
        c = list(self.coords(rank))
        c[axis] += side
        if not 0 <= c[axis] < self.dims[axis]:
            if not self.periods[axis]:
                return None
            c[axis] %= self.dims[axis]
        return self.rank_of(c)


def _plane_cells(ni, axis: int, k: int) -> torch.Tensor:
    """Linear cell indices (x fastest) of the cells with index k along
    ``axis``, in an order that depends only on the plane's shape (so that a
    sent plane lands cell for cell in the receiver's plane)."""
    grids = torch.meshgrid(*[torch.arange(n) for n in ni], indexing="ij")
    lin = torch.zeros_like(grids[0])
    stride = 1
    for d, n in enumerate(ni):
        lin = lin + grids[d] * stride
        stride *= n
    return lin[grids[axis] == k].contiguous()


def update_cell_halo_(*arrays: CellArray, grid: CartesianGrid, group=None) -> None:
    """``update_cell_halo!(x::CellArray...)``: exchange the halo planes of
    every array with the neighbouring ranks of ``grid`` (see the module
    docstring for the rule). Every rank of the process group calls it with
    arrays of the same shapes."""
    import torch.distributed as dist

    if not arrays:
        return
    ni = arrays[0].ni
    N = len(ni)
    if len(grid.dims) < N:
        raise ArgumentError("update_cell_halo!: the process grid has fewer axes than the arrays")
    for a in arrays:
        if not isinstance(a, CellArray) or a.ni != ni:
            raise ArgumentError("update_cell_halo!: every array must be a CellArray on the same cell grid")
    me = dist.get_rank(group)
    for axis in range(N):
        ol = int(grid.overlaps[axis])
        n = ni[axis]
        if ol < 2 or ol > n:
            continue
        below, above = grid.neighbour(me, axis, -1), grid.neighbour(me, axis, +1)
        if below is None and above is None:
            continue
        dev = arrays[0].data.device
        send_lo = _plane_cells(ni, axis, ol - 1).to(dev)  # plane ol (1-based), to the rank below
        send_hi = _plane_cells(ni, axis, n - ol).to(dev)  # plane n - ol + 1, to the rank above
        recv_hi = _plane_cells(ni, axis, n - 1).to(dev)   # the last plane, from the rank above
        recv_lo = _plane_cells(ni, axis, 0).to(dev)       # the first plane, from the rank below
        # tag 0: a plane sent to the rank below (it lands in that rank's last plane),
        # tag 1: a plane sent to the rank above (it lands in its first plane)
        for a in arrays:
            down = a.data.index_select(1, send_lo).contiguous() if below is not None else None
            up = a.data.index_select(1, send_hi).contiguous() if above is not None else None
            if below == me and above == me:  # one rank on a periodic axis: its own planes
                a.data[:, recv_hi] = down
                a.data[:, recv_lo] = up
                continue
            ops, bufs = [], {}
            if below is not None:
                ops.append(dist.P2POp(dist.isend, down, below, group, tag=0))
                bufs["lo"] = torch.empty((a.ncap, recv_lo.numel()), dtype=a.data.dtype, device=dev)
                ops.append(dist.P2POp(dist.irecv, bufs["lo"], below, group, tag=1))
            if above is not None:
                ops.append(dist.P2POp(dist.isend, up, above, group, tag=1))
                bufs["hi"] = torch.empty((a.ncap, recv_hi.numel()), dtype=a.data.dtype, device=dev)
                ops.append(dist.P2POp(dist.irecv, bufs["hi"], above, group, tag=0))
            for req in dist.batch_isend_irecv(ops):
                req.wait()
            if "lo" in bufs:
                a.data[:, recv_lo] = bufs["lo"]
            if "hi" in bufs:
                a.data[:, recv_hi] = bufs["hi"]


__all__ = ["CartesianGrid", "update_cell_halo_"]
