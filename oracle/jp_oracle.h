/*
 * jp_oracle.h -- CPU restatement of JustPIC.jl's particle-in-cell hot path.
 *
 * TEST INFRASTRUCTURE ONLY. This is the correctness oracle that the CUDA
 * library is checked against (and the timed CPU baseline of bench.py). No
 * product code path links, loads or calls it.
 *
 * Data layout is the reference's GPU CellArray layout (blocklength 0,
 * ext/JustPICCUDAExt.jl:29): a per-slot quantity q of slot s (0-based) in cell c
 * (0-based, column-major, x fastest) lives at q[c + ncells * s]. Grid fields
 * (velocity components, vertex fields) are column-major with x fastest.
 *
 * Parity status: pinned against the reference's own known-answer tests
 * (test/test_integrators.jl, test/test_interpolation_kernels.jl,
 * test/test_2D.jl) that need no Julia; the reference itself (Julia) cannot run
 * in this container, so the slot-level semantics follow the cited source lines.
 */
#ifndef JP_ORACLE_H
#define JP_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct jpo_grid {
    int32_t ndim;            /* 2 or 3 */
    int64_t n[3];            /* cells per dimension */
    int64_t ncells;
    int32_t nxcell;          /* already rounded to a multiple of 2^ndim */
    int32_t max_xcell;
    int32_t min_xcell;
    int32_t np_quadrant;
    uint64_t seed;
    const double* xv[3];     /* vertex coordinates, length n[d] + 1 */
    const double* dxv[3];    /* vertex spacing per cell, length n[d] */
    const double* xvel[3][3];  /* velocity grid of component c along dim d */
    const double* dxvel[3][3]; /* its spacing per interval, length nvel - 1 */
    int64_t nvel[3][3];
    const double* xc[3];     /* cell centres (Particles.xci), length n[d] */
    const double* dxc[3];    /* their spacing (Particles.di.center) per interval, length n[d] - 1 */
} jpo_grid;

/* error bits returned by the mutating calls (0 = clean) */
#define JPO_ERR_BISECTION_LIMIT 0x1
#define JPO_ERR_FAR_MOVE 0x2
#define JPO_ERR_NO_NEIGHBOUR 0x4

#define JPO_EULER 0
#define JPO_RK2 1
#define JPO_RK4 2
#define JPO_INTERP_LINP 1
#define JPO_INTERP_MQS 2

void jpo_set_threads(int nthreads);

/* particle seeding: src/Particles/particles_utils.jl:168-194 */
void jpo_init_particles(const jpo_grid* g, double* const coords[3], uint8_t* index);

/* advection!: src/Particles/Advection/advection.jl:35-91 */
int jpo_advection(const jpo_grid* g, int method, double alpha, const double* const V[3],
                  double dt, double* const coords[3], const uint8_t* index);
int jpo_advection_interp(const jpo_grid* g, int method, int interp, double alpha, const double* const V[3],
                         double dt, double* const coords[3], const uint8_t* index);
int jpo_interp_velocity(const jpo_grid* g, int interp, const double* const V[3], const double* p,
                        const int64_t* I, double* v);

/* move_particles!: src/Particles/move_safe.jl:21-125 */
int jpo_move_particles(const jpo_grid* g, double* const coords[3], uint8_t* index,
                       double* const* args, int nargs);

/* inject_particles!: src/Particles/injection.jl:19-131 */
int jpo_inject_particles(const jpo_grid* g, double* const coords[3], uint8_t* index,
                         double* const* args, int nargs, uint32_t call);

/* inject_particles_phase!: src/Particles/injection.jl:137-325; fields[k] is
   cell-centred (n cells) when centred[k], a vertex field otherwise */
int jpo_inject_particles_phase(const jpo_grid* g, double* const coords[3], uint8_t* index, double* phases,
                               double* const* args, const double* const* fields, const int* centred, int nargs,
                               uint32_t call);

/* grid2particle!: src/Interpolations/grid_to_particle.jl:26-82 */
void jpo_grid2particle(const jpo_grid* g, double* Fp, const double* F,
                       const double* const coords[3], const uint8_t* index);

/* particle2grid!: src/Interpolations/particle_to_grid.jl:23-151 */
void jpo_particle2grid(const jpo_grid* g, double* F, const double* Fp,
                       const double* const coords[3], const uint8_t* index);

/* tuple forms (at most JPO_MAX_FIELDS fields): particle2grid!(F::NTuple, Fp::NTuple, particles),
   src/Interpolations/particle_to_grid.jl:70-109, 153-199; grid2particle!(Fp::NTuple, F::NTuple, particles),
   src/Interpolations/grid_to_particle.jl:84-103 */
#define JPO_MAX_FIELDS 16
void jpo_particle2grid_n(const jpo_grid* g, double* const* F, const double* const* Fp, int nf,
                         const double* const coords[3], const uint8_t* index);
void jpo_grid2particle_n(const jpo_grid* g, double* const* Fp, const double* const* F, int nf,
                         const double* const coords[3], const uint8_t* index);

/* grid2particle_flip!: src/Interpolations/grid_to_particle.jl:125-170 */
void jpo_grid2particle_flip(const jpo_grid* g, double* Fp, const double* F, const double* F0, double alpha,
                            const double* const coords[3], const uint8_t* index);

/* centroid2particle!: src/Interpolations/centroid_to_particle.jl:13-46; F is a cell-centred field
   (n[0] x n[1] (x n[2])) */
void jpo_centroid2particle(const jpo_grid* g, double* Fp, const double* F, const double* const coords[3]);

/* particle2centroid!: src/Interpolations/particle_to_grid_centroid.jl:10-45, :88-110 */
void jpo_particle2centroid(const jpo_grid* g, double* F, const double* Fp, const double* const coords[3]);

/* update_phase_ratios! pieces (src/PhaseRatios/): out[k * nodes + node] for
   phases 1..nph (at most 16); phases are the per-slot phase ids */
void jpo_phase_ratios_center(const jpo_grid* g, int nph, const double* phases, const double* const coords[3],
                             double* out);
void jpo_phase_ratios_vertex(const jpo_grid* g, int nph, const double* phases, const double* const coords[3],
                             double* out);
void jpo_phase_ratios_face(const jpo_grid* g, int nph, const double* phases, const double* const coords[3],
                           int dim, double* out);
void jpo_phase_ratios_midpoint(const jpo_grid* g, int nph, const double* phases, const double* const coords[3],
                               int which, double* out);

/* forward-mode derivatives (jp_oracle_jvp.c): the same calls on (value,
   tangent) pairs; dV / dFp may be NULL (zero tangent) */
int jpo_advection_jvp(const jpo_grid* g, int method, double alpha, const double* const V[3],
                      const double* const dV[3], double dt, double* const coords[3], double* const dcoords[3],
                      const uint8_t* index);
void jpo_particle2grid_jvp(const jpo_grid* g, double* F, double* dF, const double* Fp, const double* dFp,
                           const double* const coords[3], const double* const dcoords[3], const uint8_t* index);

/* known-answer helpers (test/test_integrators.jl, test_interpolation_kernels.jl) */
void jpo_first_stage(int method, double alpha, double dt, int n, const double* v,
                     const double* p, double* out);
void jpo_second_stage(double alpha, double dt, int n, const double* v0, const double* v1,
                      const double* p, double* out);
double jpo_lerp(int n, const double* v, const double* t);
int64_t jpo_bisection(double px, const double* x, int64_t len, int64_t seed, int* err);
void jpo_philox(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]);
double jpo_rand(uint64_t seed, uint32_t stream, uint32_t call, uint64_t cell, uint32_t slot,
                uint32_t dim);

#ifdef __cplusplus
}
#endif
#endif
