"""jp_move_particles_noalloc: move_particles! for host programs that may not
call cudaMalloc once their time loop runs (device memory handed out up front by
their own pool, or no room for the synchronisation an allocation may cause).
The entry point takes its scratch from a fixed device array inside the library
instead of cudaMalloc, so it is checked here, through the C ABI, against the
ordinary jp_move_particles on identical inputs, for two calls in a row (the
second call reuses the array the first one left behind). This file is
collected last so that a run stopping at the first failure has already run
every other test; it also passes on its own in a fresh process."""
import ctypes

import numpy as np
import pytest

from _harness import W, assert_bits_equal, jp

pytestmark = pytest.mark.gpu


def _pair(ni, nxcell=24, max_xcell=48, min_xcell=12):
    g = W.grid(ni)
    a = jp.init_particles(jp.CUDABackend, nxcell, max_xcell, min_xcell, *g["grid_v"])
    b = jp.init_particles(jp.CUDABackend, nxcell, max_xcell, min_xcell, *g["grid_v"])
    fa, = jp.init_cell_arrays(a, 1)
    fb, = jp.init_cell_arrays(b, 1)
    T = jp.TA("CUDA")(W.gaussian_T(g) if len(ni) == 2 else W.gaussian_T(g, width2=0.15 ** 2))
    jp.grid2particle_(fa, T, a)
    jp.grid2particle_(fb, T, b)
    return g, a, b, fa, fb


def _noalloc_move(p, fields):
    lib = jp._native.load()
    coords = jp._native.P3(*[c.data_ptr() for c in p.coords], *([None] * (3 - p.ndim)))
    args = (ctypes.c_void_p * max(1, len(fields)))(*[f.data_ptr() for f in fields])
    return lib.jp_move_particles_noalloc(p.handle, coords, p.index.data_ptr(), args, len(fields))


@pytest.mark.parametrize("ni", [(60, 50), (14, 12, 10)])
def test_noalloc_move_matches_move_on_two_calls(ni):
    g, a, b, fa, fb = _pair(ni)
    V = W.stream_velocity(g) if len(ni) == 2 else W.cellular_velocity_3d(g)
    Vd = tuple(jp.TA("CUDA")(v) for v in V)
    dt = W.cfl_dt(g, V)
    for call in range(2):
        jp.advection_(a, jp.RungeKutta2(), Vd, dt)
        jp.advection_(b, jp.RungeKutta2(), Vd, dt)
        jp.move_particles_(a, (fa,))
        assert _noalloc_move(b, (fb,)) == 0, jp._native.last_error()
        # bit-exact, the tolerance of every other FP64 parity test in this suite
        assert np.array_equal(a.index.numpy(), b.index.numpy()), f"call {call}: index differs"
        for d in range(len(ni)):
            assert_bits_equal(a.coords[d].numpy(), b.coords[d].numpy(), f"call {call}: coords[{d}]")
        live = a.index.numpy().astype(bool)
        assert_bits_equal(fa.numpy()[live], fb.numpy()[live], f"call {call}: field")


def test_noalloc_rejects_a_grid_beyond_its_buffer():
    g = W.grid((512, 512))  # 262144 cells x 48 slots needs far more than the fixed buffer
    p = jp.init_particles(jp.CUDABackend, 24, 48, 12, *g["grid_v"])
    f, = jp.init_cell_arrays(p, 1)
    rc = _noalloc_move(p, (f,))
    assert rc == jp._native.JP_ERR_INVALID_ARGUMENT
    assert "fixed buffer" in jp._native.last_error()


def test_noalloc_move_is_not_replayed_by_move_permutation():
    """The call leaves the container's own move record alone, so a later
    jp_move_permutation must refuse instead of replaying an older move."""
    from justpic_gb300 import adjoint as A

    g, a, b, fa, fb = _pair((40, 36))
    V = W.stream_velocity(g)
    Vd = tuple(jp.TA("CUDA")(v) for v in V)
    dt = W.cfl_dt(g, V)
    jp.advection_(b, jp.RungeKutta2(), Vd, dt)
    jp.move_particles_(b, (fb,))  # an ordinary move: its record can be replayed
    A.move_permutation(b)
    jp.advection_(b, jp.RungeKutta2(), Vd, dt)
    assert _noalloc_move(b, (fb,)) == 0, jp._native.last_error()
    with pytest.raises(Exception, match="no record to replay"):
        A.move_permutation(b)


def test_noalloc_wide_cells_beyond_the_buffer_size():
    """Cells of more than 64 slots run the per-cell schedule, which uses no
    scratch: a grid whose masked scratch would exceed the buffer is accepted
    and moves exactly like jp_move_particles."""
    g = W.grid((128, 128))  # 16384 cells x 80 slots: ~48 MB if it needed the masked scratch
    a = jp.init_particles(jp.CUDABackend, 60, 80, 50, *g["grid_v"])
    b = jp.init_particles(jp.CUDABackend, 60, 80, 50, *g["grid_v"])
    assert a.max_xcell > 64
    V = W.stream_velocity(g)
    Vd = tuple(jp.TA("CUDA")(v) for v in V)
    dt = W.cfl_dt(g, V)
    jp.advection_(a, jp.RungeKutta2(), Vd, dt)
    jp.advection_(b, jp.RungeKutta2(), Vd, dt)
    jp.move_particles_(a, ())
    assert _noalloc_move(b, ()) == 0, jp._native.last_error()
    assert np.array_equal(a.index.numpy(), b.index.numpy())
    for d in range(2):
        assert_bits_equal(a.coords[d].numpy(), b.coords[d].numpy(), f"coords[{d}]")
