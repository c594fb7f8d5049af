/*
 * justpic_gb300.h -- C ABI of the GB300-native JustPIC particle-in-cell hot path.
 *
 * One handle (`jp_particles`) carries the geometry part of JustPIC's
 * `Particles` struct (src/particles.jl:17-46): dimension, cell counts, the
 * vertex grid `xvi`, the staggered velocity grids `xi_vel`, their spacings and
 * `nxcell/max_xcell/min_xcell`. The per-slot data (coordinates, the occupancy
 * `index`, particle fields) stay owned by the caller as plain device pointers
 * laid out like the reference's GPU CellArrays (blocklength 0,
 * ext/JustPICCUDAExt.jl:29): slot s (0-based) of cell c (0-based, column-major,
 * x fastest) is element c + ncells * s. The index is one byte per slot
 * (Julia Bool). Grid fields (velocity components, vertex fields) are
 * column-major device arrays with x fastest.
 *
 * Every mutating entry point replaces one exported Julia function of the
 * reference and keeps its semantics: it works in place, returns JP_OK (0) or a
 * negative JP_ERR_* code (the Julia side turns it into an exception), and is
 * synchronous by default like the reference's `launch!` (src/launch.jl:65-69).
 * Kernels run on the stream given to jp_set_stream (default: the legacy
 * default stream). The handle is not thread-safe.
 *
 * Limits: ndim 2 or 3; 1 <= max_xcell <= JP_MAX_XCELL (cells above 64 slots
 * run the reference's own per-cell schedule for move_particles! and
 * inject_particles!, in both forms; the adjoint needs max_xcell <= 64); at
 * most JP_MAX_ARGS particle fields per call; grids strictly increasing.
 */
#ifndef JUSTPIC_GB300_H
#define JUSTPIC_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define JP_OK 0
#define JP_ERR_INVALID_ARGUMENT (-1) /* ArgumentError in the reference */
#define JP_ERR_CUDA (-2)             /* a CUDA runtime call failed */
#define JP_ERR_OUT_OF_MEMORY (-3)
#define JP_ERR_BISECTION_LIMIT (-4)  /* a cell search hit its iteration cap */
#define JP_ERR_NOT_BUILT (-5)
#define JP_ERR_ADJOINT_WINDOW (-6)   /* an adjoint gather met a particle outside its fixed window */

#define JP_MAX_ARGS 16
#define JP_MAX_XCELL 1024

/* warning bits (jp_get_warnings): conditions the reference does not report */
#define JP_WARN_FAR_MOVE 0x2     /* a particle moved more than one cell; it was dropped */
#define JP_WARN_NO_NEIGHBOUR 0x4 /* an injected particle had no live neighbour to copy fields from */

/* integrators, src/Advection/types.jl:17-49 */
#define JP_EULER 0
#define JP_RUNGE_KUTTA2 1
#define JP_RUNGE_KUTTA4 2

typedef struct jp_particles jp_particles;

/*
 * Grid description: the staggered velocity grids of init_particles
 * (src/Particles/particles_utils.jl:30-35). xi_vel[c][d] is the coordinate
 * vector (host memory) of velocity component c along axis d, of length
 * n_vel[c][d]. The vertex grid is xi_vel[d][d], so the cell count along d is
 * n_vel[d][d] - 1. `uniform` selects the spacing rule: 1 = range grids (one
 * spacing x[1] - x[0] per axis, particles_utils.jl:137-139), 0 = vector grids
 * (per-interval diff, particles_utils.jl:76-79).
 */
typedef struct jp_grid_desc {
    int32_t ndim;
    int32_t uniform;
    const double* xi_vel[3][3];
    int64_t n_vel[3][3];
} jp_grid_desc;

/*
 * Create a container. Replaces the geometry part of init_particles
 * (src/Particles/particles_utils.jl:48-106 and :108-166): nxcell is rounded up
 * to a multiple of 2^ndim and max_xcell raised to at least that. `seed` keys
 * the counter RNG used by jp_init_particles and jp_inject_particles.
 */
int jp_particles_create(jp_particles** out, const jp_grid_desc* grid, int32_t nxcell,
                        int32_t max_xcell, int32_t min_xcell, uint64_t seed);
int jp_particles_destroy(jp_particles* p);

/* Read back the derived sizes (the fields of Particles, src/particles.jl:17-29). */
int jp_particles_info(const jp_particles* p, int32_t* ndim, int64_t ncells[3], int32_t* nxcell,
                      int32_t* max_xcell, int32_t* min_xcell, int64_t* np);

int jp_set_stream(jp_particles* p, void* cuda_stream);
/* 1 (default): every call synchronizes and reports device-side errors, like
   launch! (src/launch.jl:65-69). 0: calls only enqueue; jp_synchronize reports. */
int jp_set_synchronous(jp_particles* p, int32_t synchronous);
int jp_synchronize(jp_particles* p);
/* Sticky warning bits (JP_WARN_*) since the last call with clear = 1. */
int jp_get_warnings(jp_particles* p, uint32_t* bits, int32_t clear);

/*
 * Particles removed by move_particles! calls since the last call with
 * clear = 1 (no reference counterpart; the reference removes them silently,
 * src/Particles/move_safe.jl:96-117): counts[0] left the domain, counts[1]
 * moved more than one cell in a step and were dropped, counts[2] found no free
 * slot at or after the walk's starting point in their new cell. Waits for the
 * container's stream.
 */
int jp_get_move_counts(jp_particles* p, uint64_t counts[3], int32_t clear);
/* Number of inject calls so far: the `call` word of the injection RNG counter. */
int jp_get_rng_counter(const jp_particles* p, uint64_t* counter);
int jp_set_rng_counter(jp_particles* p, uint64_t counter);
/* Message of the last failing call on this thread. */
const char* jp_last_error(void);

/*
 * Seed particles: fill_coords_index! (src/Particles/particles_utils.jl:168-194).
 * Writes every slot: np_quadrant random points per quadrant/octant in slots
 * 0..nxcell-1 (index 1), NaN and index 0 elsewhere.
 */
int jp_init_particles(jp_particles* p, double* const coords[3], uint8_t* index);

/*
 * advection! (src/Particles/Advection/advection.jl:35-62): advect every live
 * particle through the staggered velocity components V[0..ndim-1] (device,
 * sized n_vel[c][0] x n_vel[c][1] (x n_vel[c][2])). method = JP_EULER,
 * JP_RUNGE_KUTTA2 (alpha in (0, 1)) or JP_RUNGE_KUTTA4.
 */
int jp_advection(jp_particles* p, int32_t method, double alpha, const double* const V[3],
                 double dt, double* const coords[3], const uint8_t* index);

/*
 * advection_LinP! (src/Particles/Advection/advection_LinP.jl:27-62) and
 * advection_MQS! (src/Particles/Advection/advection_MQS.jl:30-66): as
 * jp_advection, with the LinP (2/3 N-linear + 1/3 pressure-point) or MQS
 * (quadratic-spline corrected) velocity interpolation wherever the parent
 * interval is at least one interval away from the component grid's edges
 * (N-linear elsewhere), as the reference does.
 */
int jp_advection_linp(jp_particles* p, int32_t method, double alpha, const double* const V[3],
                      double dt, double* const coords[3], const uint8_t* index);
int jp_advection_mqs(jp_particles* p, int32_t method, double alpha, const double* const V[3],
                     double dt, double* const coords[3], const uint8_t* index);

/*
 * move_particles! (src/Particles/move_safe.jl:21-125): relocate particles that
 * left their cell, carrying the nargs particle fields args[0..nargs-1]. Slot
 * allocation reproduces the reference's colour passes exactly. The first move
 * of a container allocates its scratch and captures the colour passes into a
 * CUDA graph on a private stream; later moves launch that graph on the
 * container's stream (a stream that is being captured by the caller gets the
 * plain launches instead; the scratch allocation itself is not allowed inside
 * a capture, so make the first move before capturing).
 */
int jp_move_particles(jp_particles* p, double* const coords[3], uint8_t* index,
                      double* const* args, int32_t nargs);

/*
 * move_particles! for callers that cannot allocate device memory. It has no
 * counterpart in the reference. Some host programs may not call cudaMalloc
 * once their time loop runs: an application whose device memory is all
 * handed out up front by its own pool or by a framework that owns the GPU, or
 * a loop that cannot absorb the device-wide synchronisation an allocation may
 * cause. jp_move_particles allocates its scratch on a container's first move,
 * so those callers use this entry point instead.
 *
 * Same arguments and results as jp_move_particles, but the scratch memory the
 * relocation needs (64-bit occupancy masks per cell, a code, an origin tag and
 * a shadow record per slot) comes from one fixed device array of
 * JP_NOALLOC_SCRATCH_BYTES that is part of the library: every GPU on which the
 * library is loaded holds it until the process exits. A container needing more
 * (88 bytes per cell in 2D, 40 in 3D, rounded up to a multiple of 256, plus (8*s+3) bytes
 * per slot with s = ndim+nargs, 4 when that is 3) is rejected with
 * JP_ERR_INVALID_ARGUMENT and a message naming the sizes; use
 * jp_move_particles there. Containers of more than 64 slots per cell need no
 * scratch (they run the per-cell schedule) and are never rejected for size.
 * The first call on a device looks up the array's device address (and may
 * load the library's device code), so make that first call before any stream
 * capture; the address is kept for the process and does not survive a
 * cudaDeviceReset, after which this entry point must not be used on that
 * device. All calls share the array and leave their contents in it; nothing
 * needs to start at zero. Calls whose kernels overlap on the GPU (e.g. on two
 * streams) race on the array. The call does not touch the container's own
 * move record, so a jp_move_permutation after it is refused.
 */
#define JP_NOALLOC_SCRATCH_BYTES (32u << 20)
int jp_move_particles_noalloc(jp_particles* p, double* const coords[3], uint8_t* index,
                              double* const* args, int32_t nargs);

/*
 * inject_particles! (src/Particles/injection.jl:19-131): reseed quadrants of
 * under-populated cells; new particles copy the fields of their nearest
 * neighbour.
 */
int jp_inject_particles(jp_particles* p, double* const coords[3], uint8_t* index,
                        double* const* args, int32_t nargs);

/*
 * inject_particles_phase! (src/Particles/injection.jl:133-325): as
 * jp_inject_particles, but every quadrant of a cell is checked, a new
 * particle takes the phase id (per-slot FP64 field `phases`) of its nearest
 * neighbour, and particle field args[k] takes the clamped N-linear
 * interpolation of grid field fields[k] at the new particle: cell-centred
 * (shape ni, column-major) when centred[k] != 0, else on the vertices (shape
 * ni + 1). Shares the injection call counter with jp_inject_particles.
 */
int jp_inject_particles_phase(jp_particles* p, double* const coords[3], uint8_t* index, double* phases,
                              double* const* args, const double* const* fields, const int32_t* centred,
                              int32_t nargs);

/* grid2particle! (src/Interpolations/grid_to_particle.jl:26-45): vertex field F
   (n0+1 x n1+1 (x n2+1)) to the live slots of Fp. */
int jp_grid2particle(jp_particles* p, double* Fp, const double* F, const double* const coords[3],
                     const uint8_t* index);

/* particle2grid! (src/Interpolations/particle_to_grid.jl:23-151): inverse
   squared distance average of Fp onto the vertex field F. */
int jp_particle2grid(jp_particles* p, double* F, const double* Fp, const double* const coords[3],
                     const uint8_t* index);

/*
 * The tuple forms, nfields (1 to JP_MAX_ARGS) fields in one call; the
 * coordinates and the weights are read and formed once for all fields.
 * jp_grid2particle_n: grid2particle!(Fp::NTuple, F::NTuple, particles)
 *   (src/Interpolations/grid_to_particle.jl:84-103): live particles with a NaN
 *   coordinate are skipped, as in the reference's tuple kernel.
 * jp_particle2grid_n: particle2grid!(F::NTuple, Fp::NTuple, particles)
 *   (src/Interpolations/particle_to_grid.jl:70-109 (2D), 153-199 (3D)): the
 *   scalar form's weights and order, one weighted sum per field, each
 *   normalised as wF * inv(w). (The reference's own tuple kernels stop for
 *   more than one field: the 2D one indexes a scalar accumulator with the
 *   field number, the 3D one reads an undefined slot variable; these are the
 *   sums both spell out.)
 */
int jp_grid2particle_n(jp_particles* p, double* const* Fp, const double* const* F, int32_t nfields,
                       const double* const coords[3], const uint8_t* index);
int jp_particle2grid_n(jp_particles* p, double* const* F, const double* const* Fp, int32_t nfields,
                       const double* const coords[3], const uint8_t* index);

/*
 * Transfers beside the hot path, on the same layout (FP64, 2D and 3D):
 * grid2particle_flip!(Fp, xvi, F, F0, particles; α)
 *   (src/Interpolations/grid_to_particle.jl:125-170) with xvi = the container's
 *   vertex grid: Fp = muladd(F_pic, α, (Fp + F_pic - F0_pic) (1 - α)) for every
 *   live slot, F and F0 vertex fields;
 * centroid2particle!(Fp, F, particles) (src/Interpolations/centroid_to_particle.jl:13-46):
 *   N-linear interpolation of the cell-centred field F (n0 x n1 (x n2)) to every
 *   slot with non-NaN coordinates;
 * particle2centroid!(F, Fp, particles) (src/Interpolations/particle_to_grid_centroid.jl:10-110):
 *   bilinear-weight average of each cell's particles at its centre.
 * The centroid transfers use the container's centre grids (Particles.xci,
 * di.center) and need the ghost-expanded centre grids of init_particles with
 * at least 2 cells per axis (JP_ERR_INVALID_ARGUMENT otherwise).
 */
int jp_grid2particle_flip(jp_particles* p, double* Fp, const double* F, const double* F0, double alpha,
                          const double* const coords[3], const uint8_t* index);

/*
 * update_phase_ratios!(phase_ratios, particles, phases) (src/PhaseRatios/utils.jl:3-40):
 * for phase ids 1..nphases (<= 16) in the per-slot field `phases`, the phase
 * fractions at the cell centres (center, n0 x n1 (x n2) nodes), the vertices
 * (vertex, (n0+1) x ...) and the faces (faces[d], n + e_d nodes: the
 * reference's Vx, Vy, Vz), each laid out out[k * nodes + node] like a
 * CellArray of nphases-vectors. NULL skips a location. Kernels:
 * centers.jl:3-30, vertices.jl:4-107, midpoints.jl:3-94.
 *
 * jp_phase_ratios_midpoints: the 3D edge midpoints (midpoints.jl:108-242),
 * mids[0] = xy (n + (1,1,0) nodes), mids[1] = yz (n + (0,1,1)), mids[2] = xz
 * (n + (1,0,1)); needs at least 2 cells per axis.
 */
int jp_phase_ratios(jp_particles* p, int32_t nphases, const double* phases, const double* const coords[3],
                    double* center, double* vertex, double* const faces[3]);
int jp_phase_ratios_midpoints(jp_particles* p, int32_t nphases, const double* phases,
                              const double* const coords[3], double* const mids[3]);
int jp_centroid2particle(jp_particles* p, double* Fp, const double* F, const double* const coords[3]);

/*
 * CellArray layout conversion (src/CellArrays/conversion.jl:36-41,
 * ext/JustPICCUDAExt.jl:178-191, the permutedims(data, (3, 2, 1)) between
 * the GPU and CPU CellArrays): component k of node c sits at c + nnodes * k
 * in the GPU form (blocklength 0) and at k + ncomp * c in the CPU form
 * (blocklength 1). to_cpu != 0 converts GPU form -> CPU form, else back.
 * src and dst are distinct device buffers of nnodes * ncomp elements of
 * elem_bytes (1, 2, 4 or 8) bytes; runs on the container's stream. Used for
 * Array(particles) / TA(backend)(Float64, data) and checkpoints.
 */
/*
 * Recorded adjoint steps (2D, FP64, max_xcell <= 64). jp_advection_record is
 * jp_advection (same positions, bit for bit) that also writes, into a device
 * buffer of jp_advection_record_bytes bytes, each live particle's velocity
 * samples (local coordinates, bilinear gradients, deposit window);
 * jp_advection_vjp_recorded is jp_advection_vjp for that step from the record
 * instead of a replay of the stages (index = the occupancy before the step;
 * gV is added to). A stage point more than one cell from its particle's cell
 * raises JP_ERR_ADJOINT_WINDOW at recording.
 */
int jp_advection_record_bytes(jp_particles* p, int32_t method, uint64_t* bytes);
int jp_advection_record(jp_particles* p, int32_t method, double alpha, const double* const V[3], double dt,
                        double* const coords[3], const uint8_t* index, void* rec);
int jp_advection_vjp_recorded(jp_particles* p, int32_t method, double alpha, double dt, const void* rec,
                              const uint8_t* index, double* const lam[3], double* const gV[3]);

/*
 * Diagnostic (no reference counterpart): checks the integer-pipe evaluation of
 * particle2grid!'s weight inv(sqrt(ss)^2) against CUDA's correctly rounded
 * double sqrt, multiply and reciprocal, bit for bit, on n seeded inputs drawn
 * from the whole double range (plus the edge families listed in
 * csrc/jp_particles.cu). Writes the number of mismatches and the bits of the
 * first mismatching input (0 if none). Synchronous; needs no container.
 */
int jp_selftest_weight(uint64_t seed, int64_t n, int64_t* mismatches, uint64_t* first_bad_input);

int jp_cellarray_permute(jp_particles* p, const void* src, void* dst, int64_t nnodes, int32_t ncomp,
                         int32_t elem_bytes, int32_t to_cpu);
int jp_particle2centroid(jp_particles* p, double* F, const double* Fp, const double* const coords[3]);

/*
 * Adjoint (vector-Jacobian products) of the FP64 path, 2D; the grid
 * transfers (jp_particle2grid_with_weights, jp_particle2grid_vjp,
 * jp_grid2particle_vjp) in 2D and 3D. max_xcell <= 64. No counterpart in
 * the reference: it is what a ChainRulesCore rrule of the
 * Julia API calls. Gradient arrays share the layout of the values they
 * belong to. Transposes are gathers with a fixed summation order: results are
 * reproducible run to run. Particle relocation is replayed as integer data
 * from the forward sweep and is not differentiated.
 *
 * jp_particle2grid_with_weights: particle2grid!, also writing the weight sum
 *   W of every vertex (needed by jp_particle2grid_vjp).
 * jp_move_permutation: right after jp_move_particles, dest[a] = slot that
 *   now holds the particle that sat in slot a before the move, or -1
 *   (empty slot, dropped particle). int32; needs < 2^31 slots.
 * jp_permute_vjp: pre[k][a] = post[k][dest[a]] (0 where dest is -1), k < n <= 8.
 * jp_slot_ids: ids[a] = a (as a double) for live slots, -1 elsewhere. Pass ids
 *   as an extra particle field to jp_inject_particles: afterwards an injected
 *   slot holds the id of the particle its fields were copied from.
 * jp_inject_vjp: with those ids, pre[k][a] = post[k][a] for slots that existed
 *   before the injection and 0 for injected ones; for the arrays k whose bit is
 *   set in `copies`, each existing slot also receives post[k] of the slots
 *   injected from it (set the bits of particle fields, not of positions).
 *   With pre[k] == post[k] for every array it works in place: only the sources
 *   receive their copies' cotangents and the injected slots keep their values,
 *   which a following jp_permute_vjp never reads.
 * jp_advection_vjp: one advection! step (same method, alpha, V, dt) taken
 *   from coords (the positions BEFORE the step): lam holds dL/dX after the step
 *   on entry and dL/dX before it on return; dL/dV is ADDED to gV. Fails with
 *   JP_ERR_ADJOINT_WINDOW if a stage point lies more than one cell from its
 *   particle's cell (dt above the CFL limit).
 * jp_particle2grid_vjp: from gF = dL/dF, ADDS dL/dFp to gFp and, when gX is
 *   not NULL, dL/dX to gX. F and W are the forward's outputs.
 * jp_grid2particle_vjp: from gFp = dL/dFp, ADDS dL/dF to gF (when not NULL)
 *   and dL/dX to gX (when not NULL; needs F).
 */
int jp_particle2grid_with_weights(jp_particles* p, double* F, double* W, const double* Fp,
                                  const double* const coords[3], const uint8_t* index);
int jp_move_permutation(jp_particles* p, int32_t* dest);
int jp_permute_vjp(jp_particles* p, const int32_t* dest, const double* const* post, double* const* pre,
                   int32_t n);
int jp_slot_ids(jp_particles* p, const uint8_t* index, double* ids);
int jp_inject_vjp(jp_particles* p, const double* ids, const double* const* post, double* const* pre, int32_t n,
                  int32_t copies);
int jp_advection_vjp(jp_particles* p, int32_t method, double alpha, const double* const V[3], double dt,
                     const double* const coords[3], const uint8_t* index, double* const lam[3],
                     double* const gV[3]);
int jp_particle2grid_vjp(jp_particles* p, const double* F, const double* W, const double* Fp,
                         const double* const coords[3], const uint8_t* index, const double* gF, double* gFp,
                         double* const gX[3]);
int jp_grid2particle_vjp(jp_particles* p, const double* F, const double* gFp, const double* const coords[3],
                         const uint8_t* index, double* gF, double* const gX[3]);

/*
 * Adjoint of the split-precision form (2D; uniform grids with the standard
 * staggering). Offsets, velocities and fields are the form's FP32 arrays;
 * cotangents are FP64: lam = dL/d(offset, cell units), gV and gF as above.
 * jp_advection_vjp_f32 replays jp_advection_f32's stages in FP32 and sweeps
 * back in FP64, with the FP64 entry's window rule and accumulation order.
 * jp_particle2grid_f32_with_weights writes the FP64 weight sum of each vertex.
 * Injection is traced with int32 ids (jp_slot_ids_i32) passed through
 * jp_inject_particles_f32 as an FP32 field (copied bit for bit) and replayed
 * by jp_inject_vjp_i32; the move's slot map is jp_move_permutation.
 */
int jp_slot_ids_i32(jp_particles* p, const uint8_t* index, int32_t* ids);
int jp_inject_vjp_i32(jp_particles* p, const int32_t* ids, const double* const* post, double* const* pre,
                      int32_t n, int32_t copies);
int jp_advection_vjp_f32(jp_particles* p, int32_t method, double alpha, const float* const V[3], double dt,
                         const float* const xi[3], const uint8_t* index, double* const lam[3],
                         double* const gV[3]);
int jp_particle2grid_f32_with_weights(jp_particles* p, float* F, double* W, const float* Fp,
                                      const float* const xi[3], const uint8_t* index);
int jp_particle2grid_vjp_f32(jp_particles* p, const float* F, const double* W, const float* Fp,
                             const float* const xi[3], const uint8_t* index, const double* gF, double* gFp,
                             double* const gxi[3]);

/*
 * Split-precision form (no reference counterpart; the scope of this library
 * asks for it beside the plain FP64 form). Each particle is the cell of its
 * slot (an implicit int32 index) plus an FP32 offset xi in [0, 1)^N in units
 * of the cell spacing, stored in the same blocklength-0 layout as the
 * coordinates (4 bytes per value). Velocity fields, particle fields and vertex
 * fields are FP32; FP64 is used for the weight sums of particle2grid. Grids:
 * uniform, or with spacing that varies (per-cell width tables built by
 * jp_particles_create), in both cases with the standard staggering of the
 * velocity components (the vertex grid along the component's axis; the cell
 * midpoints plus one ghost node at each end along the others); other grids get
 * JP_ERR_INVALID_ARGUMENT. Semantics in cell units: a particle belongs to its
 * cell when 0 <= xi < 1; move_particles sends it to cell + floor(xi) (the
 * offset scaled to the new cell's width where widths differ) with the same
 * colour-pass slot allocation as the FP64 form; the other rules follow the
 * FP64 form (see jp_f32.cu). Error against the FP64 form is measured by the
 * tests and the bench.
 */
int jp_offsets_from_coords(jp_particles* p, const double* const coords[3], const uint8_t* index,
                           float* const xi[3]);
int jp_coords_from_offsets(jp_particles* p, const float* const xi[3], const uint8_t* index,
                           double* const coords[3]);
int jp_advection_f32(jp_particles* p, int32_t method, double alpha, const float* const V[3], double dt,
                     float* const xi[3], const uint8_t* index);
int jp_move_particles_f32(jp_particles* p, float* const xi[3], uint8_t* index, float* const* args,
                          int32_t nargs);
int jp_inject_particles_f32(jp_particles* p, float* const xi[3], uint8_t* index, float* const* args,
                            int32_t nargs);
int jp_grid2particle_f32(jp_particles* p, float* Fp, const float* F, const float* const xi[3],
                         const uint8_t* index);
int jp_particle2grid_f32(jp_particles* p, float* F, const float* Fp, const float* const xi[3],
                         const uint8_t* index);

#ifdef __cplusplus
}
#endif
#endif /* JUSTPIC_GB300_H */
