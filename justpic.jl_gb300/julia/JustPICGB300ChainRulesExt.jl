# JustPICGB300ChainRulesExt: ChainRulesCore rrules for a run of the
# particle-in-cell loop with a particle2grid! misfit and for single calls
# (grid2particle!, particle2grid!, one advection! step), over the library's
# vector-Jacobian entry points (include/justpic_gb300.h, "adjoint"). No
# counterpart in the reference (ChainRulesCore is not one of its
# dependencies); it is the Julia form of the reverse sweep in
# justpic.jl_gb300/adjoint.py, which the tests check against central finite
# differences and against forward-mode derivatives through the oracle.
#
# misfit_run(p, method, V, T0, target, dt, n, k) advances the particles n steps
# (advection!, move_particles!, inject_particles! carrying the field T) and
# returns 0.5 * ||particle2grid(T) - target||^2 over the vertices that have
# particles. The rrule checkpoints the state every k steps; the pullback runs
# each segment again while recording (velocity samples, move permutations,
# injection sources) and steps back through it. Relocation is replayed as
# integer data and is not differentiated. 2D, FP64; a stage point more than
# one cell away from its particle's cell raises JP_ERR_ADJOINT_WINDOW.
#
# Never compiled here: there is no Julia toolchain on this repository's
# machines.
module JustPICGB300ChainRulesExt

using ChainRulesCore, CUDA, CellArrays, JustPIC
using ..JustPICGB300Ext: lib, check, handle, ptr, ptrs3, ptrvec, code, alpha, GP

# ---- state saved at a checkpoint: positions, occupancy, injection counter
function save_state(p::GP)
    c = Ref{UInt64}(0)
    check(ccall((:jp_get_rng_counter, lib), Cint, (Ptr{Cvoid}, Ptr{UInt64}), handle(p).ptr, c))
    return (map(x -> copy(x.data), p.coords), copy(p.index.data), c[])
end

function restore_state!(p::GP, st)
    coords, index, counter = st
    foreach((dst, src) -> copyto!(dst.data, src), p.coords, coords)
    copyto!(p.index.data, index)
    check(ccall((:jp_set_rng_counter, lib), Cint, (Ptr{Cvoid}, UInt64), handle(p).ptr, counter))
    return nothing
end

# ---- the entry points of the reverse sweep
record_bytes(p, method) = (n = Ref{UInt64}(0);
    check(ccall((:jp_advection_record_bytes, lib), Cint, (Ptr{Cvoid}, Int32, Ptr{UInt64}),
                handle(p).ptr, code(method), n)); n[])

advection_record!(p, method, V, dt, rec::CuArray{UInt8}) = check(ccall((:jp_advection_record, lib), Cint,
    (Ptr{Cvoid}, Int32, Float64, Ptr{Ptr{Cvoid}}, Float64, Ptr{Ptr{Cvoid}}, Ptr{Cvoid}, Ptr{Cvoid}),
    handle(p).ptr, code(method), alpha(method), ptrs3(V), Float64(dt), ptrs3(p.coords), ptr(p.index), pointer(rec)))

vjp_advection!(p, method, dt, rec, idx, lam, gV) = check(ccall((:jp_advection_vjp_recorded, lib), Cint,
    (Ptr{Cvoid}, Int32, Float64, Float64, Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Ptr{Cvoid}}, Ptr{Ptr{Cvoid}}),
    handle(p).ptr, code(method), alpha(method), Float64(dt), pointer(rec), pointer(idx), ptrs3(lam), ptrs3(gV)))

move_permutation!(dest::CuArray{Int32}, p) =
    check(ccall((:jp_move_permutation, lib), Cint, (Ptr{Cvoid}, Ptr{Cvoid}), handle(p).ptr, pointer(dest)))

slot_ids!(ids, p) = check(ccall((:jp_slot_ids, lib), Cint, (Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Cvoid}),
    handle(p).ptr, ptr(p.index), ptr(ids)))

permute_vjp!(p, dest, post, pre) = check(ccall((:jp_permute_vjp, lib), Cint,
    (Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Ptr{Cvoid}}, Ptr{Ptr{Cvoid}}, Int32),
    handle(p).ptr, pointer(dest), ptrvec(post), ptrvec(pre), length(post)))

inject_vjp!(p, ids, post, pre, copies) = check(ccall((:jp_inject_vjp, lib), Cint,
    (Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Ptr{Cvoid}}, Ptr{Ptr{Cvoid}}, Int32, Int32),
    handle(p).ptr, ptr(ids), ptrvec(post), ptrvec(pre), length(post), Int32(copies)))

function particle2grid_with_weights(T, p)
    F = CUDA.zeros(Float64, length.(p.xvi)...)
    W = similar(F)
    check(ccall((:jp_particle2grid_with_weights, lib), Cint,
        (Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Ptr{Cvoid}}, Ptr{Cvoid}),
        handle(p).ptr, ptr(F), ptr(W), ptr(T), ptrs3(p.coords), ptr(p.index)))
    return F, W
end

particle2grid_vjp!(gT, gX, gF, F, W, T, p) = check(ccall((:jp_particle2grid_vjp, lib), Cint,
    (Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Ptr{Cvoid}}, Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Cvoid},
     Ptr{Ptr{Cvoid}}),
    handle(p).ptr, ptr(F), ptr(W), ptr(T), ptrs3(p.coords), ptr(p.index), ptr(gF), ptr(gT), ptrs3(gX)))

# ---- the differentiated function and its rule
function misfit_run(p::GP, method, V, T0, target, dt, n, k)
    T = copy(T0)
    for _ in 1:n
        JustPIC.advection!(p, method, V, dt)
        JustPIC.move_particles!(p, (T,))
        JustPIC.inject_particles!(p, (T,))
    end
    F, W = particle2grid_with_weights(T, p)
    r = ifelse.(W .> 0, F .- target, 0.0)
    return sum(abs2, r) / 2
end

function ChainRulesCore.rrule(::typeof(misfit_run), p::GP, method, V, T0, target, dt, n, k)
    cps = []                               # the state every k steps
    T = copy(T0)
    for s in 0:(n - 1)
        s % k == 0 && push!(cps, (save_state(p), copy(T.data)))
        JustPIC.advection!(p, method, V, dt)
        JustPIC.move_particles!(p, (T,))
        JustPIC.inject_particles!(p, (T,))
    end
    F, W = particle2grid_with_weights(T, p)
    r = ifelse.(W .> 0, F .- target, 0.0)
    loss = sum(abs2, r) / 2
    final = save_state(p)
    function pullback(Δ)
        restore_state!(p, final)
        gT = zero(T)
        gX = map(zero, p.coords)
        particle2grid_vjp!(gT, gX, Δ .* r, F, W, T, p)
        gV = map(zero, V)
        tmpT, tmpX = zero(T), map(zero, p.coords)
        for seg in reverse(eachindex(cps))   # recompute a segment, then step back through it
            st, Tseg = cps[seg]
            restore_state!(p, st)
            copyto!(T.data, Tseg)
            steps = ((seg - 1) * k):(min(seg * k, n) - 1)
            recs = map(steps) do _
                idx = copy(p.index.data)
                rec = CuArray{UInt8}(undef, record_bytes(p, method))
                advection_record!(p, method, V, dt, rec)
                JustPIC.move_particles!(p, ())
                dest = similar(p.index.data, Int32)
                move_permutation!(dest, p)
                ids = similar(T)
                slot_ids!(ids, p)
                JustPIC.inject_particles!(p, (ids,))
                (rec, idx, dest, ids)
            end
            for (rec, idx, dest, ids) in reverse(recs)
                # injected copies return their field cotangent to their source (bit 2: the field)
                inject_vjp!(p, ids, (gX..., gT), (tmpX..., tmpT), 0b100)
                permute_vjp!(p, dest, (tmpX..., tmpT), (gX..., gT))
                vjp_advection!(p, method, dt, rec, idx, gX, gV)
            end
        end
        return (NoTangent(), NoTangent(), NoTangent(), gV, gT, NoTangent(), NoTangent(), NoTangent(),
                NoTangent())
    end
    return loss, pullback
end

# ---- per-call rules (the Julia form of Grid2Particle, Particle2Grid and
# AdvectionStep in justpic.jl_gb300/adjoint.py): functional forms on the raw
# arrays (a CellArray's data in its slot layout, grid fields, coordinates),
# positions fixed for the transfers. 2D and 3D for the transfers; the
# advection step is 2D like the rest of the adjoint.

# Fp (slot data) = grid2particle!(Fp, F, p) on a fresh array
function grid2particle_data(F::CuArray{Float64}, p::GP)
    Fp, = JustPIC.init_cell_arrays(p, Val(1))
    JustPIC.grid2particle!(Fp, F, p)
    return Fp.data
end

function ChainRulesCore.rrule(::typeof(grid2particle_data), F::CuArray{Float64}, p::GP)
    Fp = grid2particle_data(F, p)
    function pullback(ΔFp)
        gF = zero(F)
        g = CuArray{Float64}(unthunk(ΔFp))
        check(ccall((:jp_grid2particle_vjp, lib), Cint,
            (Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Ptr{Cvoid}}, Ptr{Cvoid}, Ptr{Cvoid},
             Ptr{Ptr{Cvoid}}),
            handle(p).ptr, ptr(F), ptr(g), ptrs3(p.coords), ptr(p.index), ptr(gF), C_NULL))
        return NoTangent(), gF, NoTangent()
    end
    return Fp, pullback
end

# F (vertex field) = particle2grid!(F, Fp, p) from slot data Fp
function particle2grid_data(Fp::CuArray{Float64}, p::GP)
    T, = JustPIC.init_cell_arrays(p, Val(1))
    copyto!(T.data, Fp)
    F, _ = particle2grid_with_weights(T, p)
    return F
end

function ChainRulesCore.rrule(::typeof(particle2grid_data), Fp::CuArray{Float64}, p::GP)
    T, = JustPIC.init_cell_arrays(p, Val(1))
    copyto!(T.data, Fp)
    F, W = particle2grid_with_weights(T, p)
    function pullback(ΔF)
        gT = zero(T)
        g = CuArray{Float64}(unthunk(ΔF))
        check(ccall((:jp_particle2grid_vjp, lib), Cint,
            (Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Ptr{Cvoid}}, Ptr{Cvoid}, Ptr{Cvoid},
             Ptr{Cvoid}, Ptr{Ptr{Cvoid}}),
            handle(p).ptr, ptr(F), ptr(W), ptr(T), ptrs3(p.coords), ptr(p.index), ptr(g), ptr(gT),
            C_NULL))
        return NoTangent(), gT.data, NoTangent()
    end
    return F, pullback
end

# X' = one advection! step of the positions X (a tuple of coordinate data
# arrays in the slot layout) through the velocity grids V; p supplies the grid
# and the occupancy, and its own coordinates are left as they were
function advection_step(X::Tuple, V::Tuple, p::GP, method, dt)
    saved = map(c -> copy(c.data), p.coords)
    foreach((c, x) -> copyto!(c.data, x), p.coords, X)
    JustPIC.advection!(p, method, V, dt)
    out = map(c -> copy(c.data), p.coords)
    foreach((c, x) -> copyto!(c.data, x), p.coords, saved)
    return out
end

function ChainRulesCore.rrule(::typeof(advection_step), X::Tuple, V::Tuple, p::GP, method, dt)
    out = advection_step(X, V, p, method, dt)
    X0 = map(copy, X)
    idx = copy(p.index.data)
    function pullback(ΔX)
        lam = map(d -> CuArray{Float64}(unthunk(d)), unthunk(ΔX))  # dL/dX' in, dL/dX out
        gV = map(zero, V)
        check(ccall((:jp_advection_vjp, lib), Cint,
            (Ptr{Cvoid}, Int32, Float64, Ptr{Ptr{Cvoid}}, Float64, Ptr{Ptr{Cvoid}}, Ptr{Cvoid},
             Ptr{Ptr{Cvoid}}, Ptr{Ptr{Cvoid}}),
            handle(p).ptr, code(method), alpha(method), ptrs3(V), Float64(dt), ptrs3(X0), ptr(idx),
            ptrs3(lam), ptrs3(gV)))
        return NoTangent(), Tuple(lam), Tuple(gV), NoTangent(), NoTangent(), NoTangent()
    end
    return out, pullback
end

end  # module
