"""GB300-native particle-in-cell hot path of JustPIC.jl.

The Julia API of the reference, one function per exported hot-path symbol, on
top of the C ABI of ``libjustpic_gb300.so`` (``include/justpic_gb300.h``):

    particles = init_particles(CUDABackend, 24, 48, 12, grid_vx, grid_vy)
    pT, = init_cell_arrays(particles, 1)
    advection_(particles, RungeKutta2(), (Vx, Vy), dt)
    move_particles_(particles, (pT,))
    inject_particles_(particles, (pT,))
    grid2particle_(pT, T, particles)
    particle2grid_(T, pT, particles)

All compute runs in hand-written sm_103a CUDA kernels; there is no CPU path.
"""
from ._native import ArgumentError, JustPICError, NativeLibraryMissing  # noqa: F401
from .api import (  # noqa: F401
    advection_,
    advection_LinP_,
    advection_MQS_,
    centroid2particle_,
    grid2particle_,
    grid2particle_flip_,
    particle2centroid_,
    PhaseRatios,
    update_phase_ratios_,
    inject_particles_,
    inject_particles_phase_,
    move_counts,
    move_particles_,
    particle2grid_,
    set_synchronous,
    synchronize,
)
from .halo import CartesianGrid, update_cell_halo_  # noqa: F401
from .integrators import AbstractAdvectionIntegrator, Euler, RungeKutta2, RungeKutta4  # noqa: F401
from .particles import (  # noqa: F401
    DEFAULT_SEED,
    TA,
    CellArray,
    CUDABackend,
    LinRange,
    Particles,
    cell_array,
    grid_field,
    init_cell_arrays,
    init_particles,
)


def build(force: bool = False) -> str:
    """Compile libjustpic_gb300.so for sm_103a (nvcc) and return its path."""
    from . import native_build as _b
    return _b.build(force=force)

from .split import (  # noqa: F401,E402
    advection_f32_,
    cell_array_f32,
    coords_from_offsets,
    grid2particle_f32_,
    grid_field_f32,
    init_cell_arrays_f32,
    init_offsets,
    inject_particles_f32_,
    move_particles_f32_,
    particle2grid_f32_,
)
from .conversion import (  # noqa: F401,E402
    Array,
    HostCellArray,
    HostParticles,
    HostPhaseRatios,
    checkpoint_name,
    checkpointing_particles,
    load_checkpoint,
)
