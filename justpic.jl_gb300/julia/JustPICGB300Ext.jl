# JustPICGB300Ext: routes JustPIC's particle-in-cell hot path to the GB300
# library libjustpic_gb300.so through its C ABI (include/justpic_gb300.h).
#
# A package extension a JustPIC maintainer would add next to
# ext/JustPICCUDAExt.jl: particles built for the GB300Backend tag keep JustPIC's
# CUDA CellArray storage (blocklength 0: slot s of cell c at c + ncells * s),
# so every CellArray's data pointer goes to the library without a copy. The
# functions below are the reference's own (same names, argument order and
# meaning); each forwards to the C entry point that replaces it.
#
# This file has not been compiled: neither the build machine nor the GPU
# machines of this repository have a Julia toolchain. The Python host layer in
# justpic.jl_gb300/api.py binds the same symbols and is what the tests run.
module JustPICGB300Ext

using JustPIC, CUDA, CellArrays
import JustPIC: init_particles, advection!, advection_LinP!, advection_MQS!, move_particles!,
    inject_particles!, inject_particles_phase!, grid2particle!, particle2grid!, grid2particle_flip!,
    centroid2particle!, particle2centroid!, update_phase_ratios!

const lib = get(ENV, "JUSTPIC_GB300_LIB", "libjustpic_gb300.so")

# status codes (JP_OK / JP_ERR_INVALID_ARGUMENT / ...) and integrator codes
const JP_OK = Cint(0)
const JP_ERR_INVALID_ARGUMENT = Cint(-1)
const JP_EULER, JP_RUNGE_KUTTA2, JP_RUNGE_KUTTA4 = Int32(0), Int32(1), Int32(2)
const JP_WARN_FAR_MOVE, JP_WARN_NO_NEIGHBOUR = UInt32(0x2), UInt32(0x4)

struct GB300Backend end  # backend tag: Particles{GB300Backend, ...}

"""Owner of a `jp_particles*`: grid geometry, error word, scratch."""
mutable struct Handle
    ptr::Ptr{Cvoid}
end

struct GridDesc          # jp_grid_desc
    ndim::Int32
    uniform::Int32
    xi_vel::NTuple{9, Ptr{Float64}}  # [component][axis], row-major 3x3
    n_vel::NTuple{9, Int64}
end

last_error() = unsafe_string(ccall((:jp_last_error, lib), Cstring, ()))

function check(rc)
    rc == JP_OK && return nothing
    rc == JP_ERR_INVALID_ARGUMENT && throw(ArgumentError(last_error()))
    return error(last_error())
end

ptr(A::CellArray) = reinterpret(Ptr{Cvoid}, pointer(A.data))
ptr(A::CuArray) = reinterpret(Ptr{Cvoid}, pointer(A))
# the C ABI's `const double* const coords[3]` is a pointer to three pointers:
# a Vector (rooted by ccall for the call), NULL past the grid's dimension
ptrs3(t) = Ptr{Cvoid}[i <= length(t) ? ptr(t[i]) : C_NULL for i in 1:3]
ptrvec(t) = Ptr{Cvoid}[ptr(x) for x in t]

code(::Euler) = JP_EULER
code(::RungeKutta2) = JP_RUNGE_KUTTA2
code(::RungeKutta4) = JP_RUNGE_KUTTA4
alpha(m::RungeKutta2) = Float64(m.α)
alpha(::Any) = 0.5

# one handle per Particles container, released with it
const HANDLES = IdDict{Any, Handle}()
handle(p) = HANDLES[p]

function create_handle(xi_vel, nxcell, max_xcell, min_xcell, seed)
    N = length(xi_vel)
    host = [collect(Float64, xi_vel[c][d]) for c in 1:N, d in 1:N]
    uniform = all(x -> x isa AbstractRange, Iterators.flatten(xi_vel))
    xp = ntuple(9) do k
        c, d = (k - 1) ÷ 3 + 1, (k - 1) % 3 + 1
        c <= N && d <= N ? pointer(host[c, d]) : Ptr{Float64}(0)
    end
    nv = ntuple(9) do k
        c, d = (k - 1) ÷ 3 + 1, (k - 1) % 3 + 1
        c <= N && d <= N ? Int64(length(host[c, d])) : Int64(0)
    end
    desc = Ref(GridDesc(Int32(N), Int32(uniform), xp, nv))
    out = Ref{Ptr{Cvoid}}(C_NULL)
    GC.@preserve host check(ccall((:jp_particles_create, lib), Cint,
        (Ptr{Ptr{Cvoid}}, Ptr{GridDesc}, Int32, Int32, Int32, UInt64),
        out, desc, nxcell, max_xcell, min_xcell, seed))
    h = Handle(out[])
    finalizer(h -> ccall((:jp_particles_destroy, lib), Cint, (Ptr{Cvoid},), h.ptr), h)
    ccall((:jp_set_stream, lib), Cint, (Ptr{Cvoid}, Ptr{Cvoid}), h.ptr, CUDA.stream().handle)
    return h
end

# init_particles(GB300Backend, nxcell, max_xcell, min_xcell, xi_vel...)
# (src/Particles/particles_utils.jl:30-166): JustPIC's CUDA containers, seeded
# on the device by jp_init_particles with the counter-based RNG
function init_particles(::Type{GB300Backend}, nxcell, max_xcell, min_xcell, xi_vel...; seed = 0x4A50)
    q = init_particles(JustPIC.CUDABackend, nxcell, max_xcell, min_xcell, xi_vel...)
    # the same storage under the GB300 backend tag (src/particles.jl:29-43)
    p = Particles(GB300Backend, q.coords, q.index, q.nxcell, q.max_xcell, q.min_xcell, q.np, q.di, q._di,
                  q.xci, q.xvi, q.xi_vel)
    h = create_handle(xi_vel, nxcell, max_xcell, min_xcell, UInt64(seed))
    HANDLES[p] = h
    check(ccall((:jp_init_particles, lib), Cint, (Ptr{Cvoid}, Ptr{Ptr{Cvoid}}, Ptr{Cvoid}),
        h.ptr, ptrs3(p.coords), ptr(p.index)))
    return p
end

# every JustPIC function not routed here still runs its own CUDA kernels on the
# same storage (ka_backend follows the index array, src/launch.jl:24)
const GP = Particles{GB300Backend}

function warn_bits(p)
    bits = Ref{UInt32}(0)
    check(ccall((:jp_get_warnings, lib), Cint, (Ptr{Cvoid}, Ptr{UInt32}, Int32), handle(p).ptr, bits, 1))
    bits[] & JP_WARN_FAR_MOVE != 0 &&
        @warn "move_particles!: a particle moved more than one cell in one step and was dropped"
    bits[] & JP_WARN_NO_NEIGHBOUR != 0 &&
        @warn "inject_particles!: an injected particle had no live neighbour; its fields were left unchanged"
    return nothing
end

# ---- the hot path --------------------------------------------------------
for (f, sym) in ((:advection!, :jp_advection), (:advection_LinP!, :jp_advection_linp),
                 (:advection_MQS!, :jp_advection_mqs))
    @eval function $f(p::GP, method::JustPIC.AbstractAdvectionIntegrator, V, dt)
        check(ccall(($(QuoteNode(sym)), lib), Cint,
            (Ptr{Cvoid}, Int32, Float64, Ptr{Ptr{Cvoid}}, Float64, Ptr{Ptr{Cvoid}}, Ptr{Cvoid}),
            handle(p).ptr, code(method), alpha(method), ptrs3(V), Float64(dt), ptrs3(p.coords), ptr(p.index)))
    end
end

function move_particles!(p::GP, args)
    a = ptrvec(args)
    check(ccall((:jp_move_particles, lib), Cint,
        (Ptr{Cvoid}, Ptr{Ptr{Cvoid}}, Ptr{Cvoid}, Ptr{Ptr{Cvoid}}, Int32),
        handle(p).ptr, ptrs3(p.coords), ptr(p.index), a, length(a)))
    return warn_bits(p)
end

# move_particles! for host loops that may not allocate device memory once they
# run (jp_move_particles_noalloc: scratch from a fixed array in the library)
function move_particles_noalloc!(p::GP, args)
    a = ptrvec(args)
    check(ccall((:jp_move_particles_noalloc, lib), Cint,
        (Ptr{Cvoid}, Ptr{Ptr{Cvoid}}, Ptr{Cvoid}, Ptr{Ptr{Cvoid}}, Int32),
        handle(p).ptr, ptrs3(p.coords), ptr(p.index), a, length(a)))
    return warn_bits(p)
end

# calls are synchronous by default, as launch! is; turn that off to queue a
# time step and wait once (synchronize raises any device-side error)
synchronous!(p::GP, on::Bool) =
    check(ccall((:jp_set_synchronous, lib), Cint, (Ptr{Cvoid}, Int32), handle(p).ptr, Int32(on)))
synchronize(p::GP) = (check(ccall((:jp_synchronize, lib), Cint, (Ptr{Cvoid},), handle(p).ptr)); warn_bits(p))

function inject_particles!(p::GP, args)
    a = ptrvec(args)
    check(ccall((:jp_inject_particles, lib), Cint,
        (Ptr{Cvoid}, Ptr{Ptr{Cvoid}}, Ptr{Cvoid}, Ptr{Ptr{Cvoid}}, Int32),
        handle(p).ptr, ptrs3(p.coords), ptr(p.index), a, length(a)))
    return warn_bits(p)
end

grid2particle!(Fp, F, p::GP) =
    check(ccall((:jp_grid2particle, lib), Cint,
        (Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Ptr{Cvoid}}, Ptr{Cvoid}),
        handle(p).ptr, ptr(Fp), ptr(F), ptrs3(p.coords), ptr(p.index)))

particle2grid!(F, Fp, p::GP) =
    check(ccall((:jp_particle2grid, lib), Cint,
        (Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Ptr{Cvoid}}, Ptr{Cvoid}),
        handle(p).ptr, ptr(F), ptr(Fp), ptrs3(p.coords), ptr(p.index)))

# the tuple forms (grid_to_particle.jl:84-103, particle_to_grid.jl:70-109, 153-199)
grid2particle!(Fp::NTuple{N}, F::NTuple{N}, p::GP) where {N} =
    check(ccall((:jp_grid2particle_n, lib), Cint,
        (Ptr{Cvoid}, Ptr{Ptr{Cvoid}}, Ptr{Ptr{Cvoid}}, Int32, Ptr{Ptr{Cvoid}}, Ptr{Cvoid}),
        handle(p).ptr, ptrvec(Fp), ptrvec(F), Int32(N), ptrs3(p.coords), ptr(p.index)))

particle2grid!(F::NTuple{N}, Fp::NTuple{N}, p::GP) where {N} =
    check(ccall((:jp_particle2grid_n, lib), Cint,
        (Ptr{Cvoid}, Ptr{Ptr{Cvoid}}, Ptr{Ptr{Cvoid}}, Int32, Ptr{Ptr{Cvoid}}, Ptr{Cvoid}),
        handle(p).ptr, ptrvec(F), ptrvec(Fp), Int32(N), ptrs3(p.coords), ptr(p.index)))

"""Particles removed by move_particles! since the last call with clear:
(left_domain, moved_too_far, no_free_slot)."""
function move_counts(p::GP; clear = false)
    out = Ref{NTuple{3, UInt64}}((0, 0, 0))
    check(ccall((:jp_get_move_counts, lib), Cint, (Ptr{Cvoid}, Ptr{NTuple{3, UInt64}}, Int32),
        handle(p).ptr, out, Int32(clear)))
    return (left_domain = out[][1], moved_too_far = out[][2], no_free_slot = out[][3])
end

# ---- the rows beside the hot path ----------------------------------------
function inject_particles_phase!(p::GP, phases, args, fields)
    a, f = ptrvec(args), ptrvec(fields)
    centred = Int32[size(x) == size(p.index) for x in fields]  # cell-centred vs vertex fields
    check(ccall((:jp_inject_particles_phase, lib), Cint,
        (Ptr{Cvoid}, Ptr{Ptr{Cvoid}}, Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Ptr{Cvoid}}, Ptr{Ptr{Cvoid}},
         Ptr{Int32}, Int32),
        handle(p).ptr, ptrs3(p.coords), ptr(p.index), ptr(phases), a, f, centred, length(a)))
    return warn_bits(p)
end

# every location of PhaseRatios is a CellArray of nphases-vectors on its node
# grid (blocklength 0): its data pointer is passed as is
function update_phase_ratios!(pr::JustPIC.PhaseRatios, p::GP, xci, xvi, phases)
    n = Int32(JustPIC.numphases(pr))
    faces = length(p.coords) == 2 ? (ptr(pr.Vx), ptr(pr.Vy), C_NULL) : (ptr(pr.Vx), ptr(pr.Vy), ptr(pr.Vz))
    check(ccall((:jp_phase_ratios, lib), Cint,
        (Ptr{Cvoid}, Int32, Ptr{Cvoid}, Ptr{Ptr{Cvoid}}, Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Ptr{Cvoid}}),
        handle(p).ptr, n, ptr(phases), ptrs3(p.coords), ptr(pr.center), ptr(pr.vertex), faces))
    length(p.coords) == 3 && check(ccall((:jp_phase_ratios_midpoints, lib), Cint,
        (Ptr{Cvoid}, Int32, Ptr{Cvoid}, Ptr{Ptr{Cvoid}}, Ptr{Ptr{Cvoid}}),
        handle(p).ptr, n, ptr(phases), ptrs3(p.coords), (ptr(pr.xy), ptr(pr.yz), ptr(pr.xz))))
    return nothing
end

grid2particle_flip!(Fp, xvi, F, F0, p::GP; α = 0.0) =
    check(ccall((:jp_grid2particle_flip, lib), Cint,
        (Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Cvoid}, Float64, Ptr{Ptr{Cvoid}}, Ptr{Cvoid}),
        handle(p).ptr, ptr(Fp), ptr(F), ptr(F0), Float64(α), ptrs3(p.coords), ptr(p.index)))

centroid2particle!(Fp, xci, F, p::GP) =
    check(ccall((:jp_centroid2particle, lib), Cint,
        (Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Ptr{Cvoid}}),
        handle(p).ptr, ptr(Fp), ptr(F), ptrs3(p.coords)))

particle2centroid!(F, Fp, xci, p::GP) =
    check(ccall((:jp_particle2centroid, lib), Cint,
        (Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Ptr{Cvoid}}),
        handle(p).ptr, ptr(F), ptr(Fp), ptrs3(p.coords)))

# Array(CellArray) of a GPU CellArray: the (3, 2, 1) permute on the device,
# then one copy to the host (src/CellArrays/conversion.jl:36-41)
function to_cpu_layout(A::CellArray, p::GP)
    tmp = similar(A.data)
    check(ccall((:jp_cellarray_permute, lib), Cint,
        (Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Cvoid}, Int64, Int32, Int32, Int32),
        handle(p).ptr, ptr(A), pointer(tmp), Int64(length(A)), Int32(size(A.data, 2)),
        Int32(sizeof(eltype(A.data))), Int32(1)))
    return Array(tmp)  # the CPU CellArray's data, the slots of a cell together
end

# ---- split-precision form (no reference counterpart) ----------------------
# Float32 offsets xi[d] in [0, 1) in the CellArray layout; the cell of a slot
# is implicit. Uniform and vector grids with the standard staggering (cell
# midpoints plus one ghost node at each end along the centred axes).
offsets!(xi, p::GP) = check(ccall((:jp_offsets_from_coords, lib), Cint,
    (Ptr{Cvoid}, Ptr{Ptr{Cvoid}}, Ptr{Cvoid}, Ptr{Ptr{Cvoid}}),
    handle(p).ptr, ptrs3(p.coords), ptr(p.index), ptrs3(xi)))

coords!(p::GP, xi) = check(ccall((:jp_coords_from_offsets, lib), Cint,
    (Ptr{Cvoid}, Ptr{Ptr{Cvoid}}, Ptr{Cvoid}, Ptr{Ptr{Cvoid}}),
    handle(p).ptr, ptrs3(xi), ptr(p.index), ptrs3(p.coords)))

advection_f32!(p::GP, xi, method, V, dt) = check(ccall((:jp_advection_f32, lib), Cint,
    (Ptr{Cvoid}, Int32, Float64, Ptr{Ptr{Cvoid}}, Float64, Ptr{Ptr{Cvoid}}, Ptr{Cvoid}),
    handle(p).ptr, code(method), alpha(method), ptrs3(V), Float64(dt), ptrs3(xi), ptr(p.index)))

for (f, sym) in ((:move_particles_f32!, :jp_move_particles_f32), (:inject_particles_f32!, :jp_inject_particles_f32))
    @eval function $f(p::GP, xi, args)
        a = ptrvec(args)
        check(ccall(($(QuoteNode(sym)), lib), Cint,
            (Ptr{Cvoid}, Ptr{Ptr{Cvoid}}, Ptr{Cvoid}, Ptr{Ptr{Cvoid}}, Int32),
            handle(p).ptr, ptrs3(xi), ptr(p.index), a, length(a)))
        return warn_bits(p)
    end
end

grid2particle_f32!(Fp, F, p::GP, xi) = check(ccall((:jp_grid2particle_f32, lib), Cint,
    (Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Ptr{Cvoid}}, Ptr{Cvoid}),
    handle(p).ptr, ptr(Fp), ptr(F), ptrs3(xi), ptr(p.index)))

particle2grid_f32!(F, Fp, p::GP, xi) = check(ccall((:jp_particle2grid_f32, lib), Cint,
    (Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Ptr{Cvoid}}, Ptr{Cvoid}),
    handle(p).ptr, ptr(F), ptr(Fp), ptrs3(xi), ptr(p.index)))

end  # module
