"""inject_particles! of the split-precision form, bit for bit against a host
restatement of its rules with an exhaustive nearest-neighbour search.

The form has no reference counterpart; its injection follows the FP64 form's
walk in cell units (colour passes over cells of equal index parity, quadrants
in order, a cell stops at its first quadrant holding min_xQ particles, new
particles in the free slots in order, each at quadrant corner + 1/2 (0.05 +
0.95 u) with u the FP32 Philox draw (seed, inject stream, call, cell, slot,
dim), the field copied from the first minimum of the FP32 squared physical
distance over the 3^N neighbour cells' particles in candidate order). The
kernel prunes that search (a neighbour is staged and scanned only when the
gap to its side of the cell can beat the best distance so far); this test
scans every candidate and must give the same slots, offsets and fields.

Arithmetic is restated in FP32 with IEEE rounding: numpy float32 for single
operations, and an exactly rounded fused multiply-add (the product is exact
in float64; a float64 sum that lands on a float32 rounding boundary is
resolved with exact rationals)."""
from fractions import Fraction

import numpy as np
import pytest
import torch

from _harness import O, W, jp, refined_grid

pytestmark = pytest.mark.gpu

F32 = np.float32


def _round_f32(q: Fraction) -> np.float32:
    f = F32(float(q))
    best = None
    for cand in (np.nextafter(f, F32(-np.inf)), f, np.nextafter(f, F32(np.inf))):
        err = abs(Fraction(float(cand)) - q)
        key = (err, int(np.array(cand, dtype=np.float32).view(np.uint32)) & 1)
        if best is None or key < best[0]:
            best = (key, cand)
    return F32(best[1])


def fmaf(a, b, c) -> np.float32:
    a, b, c = F32(a), F32(b), F32(c)
    d = float(a) * float(b) + float(c)  # a * b is exact in float64; one float64 rounding
    f = F32(d)
    # a float64 sum that sits exactly between two float32 values may hide the exact value's side
    lo, hi = np.nextafter(f, F32(-np.inf)), np.nextafter(f, F32(np.inf))
    if d == (float(f) + float(lo)) / 2 or d == (float(f) + float(hi)) / 2:
        return _round_f32(Fraction(float(a)) * Fraction(float(b)) + Fraction(float(c)))
    return f


def rand_f32(seed, call, cell, slot, dim) -> np.float32:
    ctr = (cell & 0xFFFFFFFF, (cell >> 32) & 0xFFFFFFFF, (slot & 0xFFFF) | ((dim & 0xFF) << 16) | (1 << 24), call)
    key = (seed & 0xFFFFFFFF, (seed >> 32) & 0xFFFFFFFF)
    out = O.philox4x32_10(ctr, key)
    return F32((out[0] >> 8) * 2.0 ** -24)


def host_inject(ni, index, xi, field, widths, uniform, min_xcell, seed, call):
    """index (M, ncells) bool, xi list of (M, ncells) float32, field (M, ncells) float32:
    modified in place. widths[d]: FP64 cell widths along axis d; on a uniform grid every
    cell takes the first width and the neighbour ratios are 1, as in the kernels."""
    N = len(ni)
    M, nc = index.shape
    NB = 3 ** N
    CENTER = NB // 2
    min_xq = (min_xcell + (1 << N) - 1) >> N

    def lin(I):
        return I[0] + ni[0] * (I[1] + (ni[1] * I[2] if N == 3 else 0))

    passes = [(p // 2, p % 2) for p in range(4)] if N == 2 else [(p // 4, (p // 2) % 2, p % 2) for p in range(8)]
    for par in passes:
        for c in range(nc):
            I = [c % ni[0], (c // ni[0]) % ni[1]] + ([c // (ni[0] * ni[1])] if N == 3 else [])
            if any(I[d] % 2 != par[d] for d in range(N)):
                continue
            if uniform:
                h = [F32(widths[d][0]) for d in range(N)]
                rl = rh = [F32(1)] * N
            else:
                h = [F32(widths[d][I[d]]) for d in range(N)]
                rl = [F32(widths[d][I[d] - 1] / widths[d][I[d]]) if I[d] > 0 else F32(1) for d in range(N)]
                rh = [F32(widths[d][I[d] + 1] / widths[d][I[d]]) if I[d] + 1 < ni[d] else F32(1)
                      for d in range(N)]
            for q in range(1 << N):
                qc = [F32(0.5) * F32((q >> d) & 1) for d in range(N)]
                count = sum(1 for s in range(M) if index[s, c] and
                            all(qc[d] < xi[d][s, c] < qc[d] + F32(0.5) for d in range(N)))
                if count >= min_xq:
                    break
                free = [s for s in range(M) if not index[s, c]]
                for i in free:
                    count += 1
                    pn = [qc[d] + F32(0.5) * fmaf(F32(0.95), rand_f32(seed, call, c, i, d), F32(0.05))
                          for d in range(N)]
                    for d in range(N):
                        xi[d][i, c] = pn[d]
                    index[i, c] = True
                    best, src = np.inf, None
                    for nb in range(NB):
                        off = [nb % 3 - 1, (nb // 3) % 3 - 1, nb // 9 - 1][:N]
                        J = [I[d] + off[d] for d in range(N)]
                        if any(J[d] < 0 or J[d] >= ni[d] for d in range(N)):
                            continue
                        cj = lin(J)
                        for s in range(M):
                            if not index[s, cj] or (nb == CENTER and s == i):
                                continue
                            ss = F32(0)
                            for d in range(N):
                                x = xi[d][s, cj]
                                r = (x - F32(1)) * rl[d] if off[d] < 0 else (fmaf(x, rh[d], F32(1)) if off[d] > 0 else x)
                                e = (F32(r) - pn[d]) * h[d]
                                ss = fmaf(e, e, ss)
                            if ss < best:
                                best, src = ss, (s, cj)
                    if src is not None:
                        field[i, c] = field[src]
                    if count >= min_xq:
                        break


CASES = [((12, 10), False, None), ((11, 9), True, None), ((6, 5, 4), False, None), ((5, 5, 4), True, None),
         # min_xcell above max_xcell: a quadrant fills every free slot, more new particles
         # than one batch of the warp's draws holds (16 in 2D, 10 in 3D)
         ((4, 3), False, (4, 64, 200)), ((3, 2, 2), True, (8, 64, 500))]


@pytest.mark.parametrize("ni,refined,caps", CASES)
def test_split_injection_matches_exhaustive_host_search(ni, refined, caps):
    g = refined_grid(ni) if refined else W.grid(ni)
    N = len(ni)
    nxcell, max_xcell, min_xcell = caps or ((16, 40, 12) if N == 2 else (16, 40, 16))
    p = jp.init_particles(jp.CUDABackend, nxcell, max_xcell, min_xcell, *g["grid_v"], seed=7)
    xi = jp.init_offsets(p)
    T, = jp.init_cell_arrays_f32(p, 1)
    live = p.index.data.bool()
    T.data[live] = torch.arange(int(live.sum()), device="cuda", dtype=torch.float32)
    # deplete: whole cells empty, others thinned, so that every search path is taken
    gen = torch.Generator("cuda").manual_seed(11)
    kill = (torch.rand(p.index.data.shape, device="cuda", generator=gen) < 0.6) & live
    kill[:, ::5] = live[:, ::5]
    p.index.data[kill] = 0
    for d in range(N):
        xi[d].data[kill] = float("nan")
    T.data[kill] = float("nan")
    index0 = p.index.numpy().astype(bool).copy()
    xi0 = [x.numpy().astype(np.float32).copy() for x in xi]
    f0 = T.numpy().astype(np.float32).copy()
    call = p.rng_counter
    jp.inject_particles_f32_(p, xi, (T,))
    widths = [np.diff(np.asarray(g["xv"][d], dtype=np.float64)) for d in range(N)]
    host_inject(ni, index0, xi0, f0, widths, not refined, min_xcell, p.seed, call)
    assert np.array_equal(index0, p.index.numpy().astype(bool))
    for d in range(N):
        a, b = xi0[d], xi[d].numpy().astype(np.float32)
        assert np.array_equal(np.isnan(a), np.isnan(b)) and np.array_equal(a[~np.isnan(a)], b[~np.isnan(b)]), d
    a, b = f0, T.numpy().astype(np.float32)
    assert np.array_equal(np.isnan(a), np.isnan(b)) and np.array_equal(a[~np.isnan(a)], b[~np.isnan(b)])
    assert int(index0.sum()) > int((~kill.cpu().numpy() & live.cpu().numpy()).sum())  # particles were injected
