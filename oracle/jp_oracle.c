/*
 * jp_oracle.c -- FP64 CPU restatement of JustPIC.jl's particle-in-cell hot path.
 *
 * TEST INFRASTRUCTURE ONLY: the correctness oracle for the CUDA library and the
 * CPU baseline that bench.py times. Nothing in the product links or calls it.
 *
 * Every function follows the cited Julia lines of the reference (paths are
 * relative to the JustPIC.jl repository), keeping its operation order:
 *   - `muladd` / `@muladd` sites become C99 fma(); every other product and sum
 *     is rounded separately (compile with -ffp-contract=off);
 *   - @muladd of a product of more than two factors splits it as
 *     muladd(first factor, product of the rest, addend) (MuladdMacro 0.2);
 *   - colour passes, slot walks, the `starting_point` carry of
 *     move_particles! and the `break` of inject_particles! are kept;
 *   - the in-kernel rand() calls are replaced by the shared Philox4x32-10
 *     counter RNG of include/justpic_gb300_rng.h.
 * Two cases where the reference is undefined get a defined result that the
 * CUDA library shares: a particle that moved more than one cell in one step
 * (the reference's colour passes race) is dropped and JPO_ERR_FAR_MOVE is
 * raised; an injected particle with no live neighbour in its 3^N block (the
 * reference reads slot 0, out of bounds) keeps its field values and raises
 * JPO_ERR_NO_NEIGHBOUR.
 */
#include "jp_oracle.h"
#include "../include/justpic_gb300_rng.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

static int g_threads = 0;

void jpo_set_threads(int nthreads) { g_threads = nthreads; }

static int nthreads(void)
{
#ifdef _OPENMP
    return g_threads > 0 ? g_threads : omp_get_max_threads();
#else
    return 1;
#endif
}

#define JPO_BISECT_CAP 256

/* ---------------------------------------------------------------- helpers */

static inline void cell_coords(const jpo_grid* g, int64_t c, int64_t I[3])
{
    I[0] = c % g->n[0];
    I[1] = (c / g->n[0]) % g->n[1];
    I[2] = g->ndim == 3 ? c / (g->n[0] * g->n[1]) : 0;
}

static inline int64_t cell_linear(const jpo_grid* g, const int64_t I[3])
{
    return I[0] + g->n[0] * (I[1] + (g->ndim == 3 ? g->n[1] * I[2] : 0));
}

/* lerp(t, v0, v1) = muladd(t, v1, muladd(-t, v0, v0)): src/Interpolations/ndlerp.jl:15 */
static inline double lerp1(double t, double v0, double v1)
{
    return fma(t, v1, fma(-t, v0, v0));
}

/* recursive N-linear lerp, x first then y then z: src/Interpolations/ndlerp.jl:11-14 */
static inline double lerpN(int n, const double* v, const double* t)
{
    if (n == 1) return lerp1(t[0], v[0], v[1]);
    if (n == 2) return lerp1(t[1], lerp1(t[0], v[0], v[1]), lerp1(t[0], v[2], v[3]));
    return lerp1(t[2],
                 lerp1(t[1], lerp1(t[0], v[0], v[1]), lerp1(t[0], v[2], v[3])),
                 lerp1(t[1], lerp1(t[0], v[4], v[5]), lerp1(t[0], v[6], v[7])));
}

double jpo_lerp(int n, const double* v, const double* t) { return lerpN(n, v, t); }

/*
 * find_parent_cell_bisection (src/Utils.jl:117-130), 0-based: returns s with
 * x[s] <= px <= x[s+1], starting from `seed`, lo = 0, hi = len - 1. The
 * reference loop is unbounded; here it stops after JPO_BISECT_CAP steps.
 */
int64_t jpo_bisection(double px, const double* x, int64_t len, int64_t seed, int* err)
{
    int64_t lo = 0, hi = len - 1, s = seed;
    for (int it = 0; it < JPO_BISECT_CAP; ++it) {
        if (x[s] <= px && px <= x[s + 1]) return s;
        if (x[s] < px) {
            lo = s;
            s = (hi + s) / 2;
        } else {
            hi = s;
            s = (lo + s) / 2;
        }
    }
    *err |= JPO_ERR_BISECTION_LIMIT;
    return s;
}

/* isincell: xv < px < xv + dx on every axis, src/Particles/utils.jl:7-15 */
static inline int isincell(int n, const double* p, const double* corner, const double* dx)
{
    int in = 1;
    for (int d = 0; d < n; ++d) in &= (corner[d] < p[d]) & (p[d] < corner[d] + dx[d]);
    return in;
}

/* --------------------------------------------------------- init_particles */

void jpo_init_particles(const jpo_grid* g, double* const coords[3], uint8_t* index)
{
    const int N = g->ndim;
    const int64_t nc = g->ncells;
    const int M = g->max_xcell;
    const int NQ = 1 << N;
#pragma omp parallel for schedule(static) num_threads(nthreads())
    for (int64_t c = 0; c < nc; ++c) {
        int64_t I[3];
        cell_coords(g, c, I);
        double x0[3], dx[3];
        for (int d = 0; d < N; ++d) {
            x0[d] = g->xv[d][I[d]];
            dx[d] = g->dxv[d][I[d]];
        }
        for (int s = 0; s < M; ++s) {
            for (int d = 0; d < N; ++d) coords[d][c + nc * s] = NAN;
            index[c + nc * s] = 0;
        }
        /* fill_coords_index!: src/Particles/particles_utils.jl:168-194 */
        int l = 0;
        for (int iq = 0; iq < NQ; ++iq) {
            double xc[3];
            for (int d = 0; d < N; ++d) xc[d] = x0[d] + (dx[d] * (double)((iq >> d) & 1)) / 2.0;
            for (int q = 0; q < g->np_quadrant; ++q) {
                for (int d = 0; d < N; ++d) {
                    double r = jp_rand_uniform(g->seed, JP_RNG_STREAM_INIT, 0u, (uint64_t)c,
                                               (uint32_t)l, (uint32_t)d);
                    coords[d][c + nc * l] = xc[d] + (dx[d] / 2.0) * r;
                }
                index[c + nc * l] = 1;
                ++l;
            }
        }
    }
}

/* -------------------------------------------------------------- advection */

/*
 * interp_velocity2particle for one component (src/Particles/Advection/advection.jl:93-148,
 * src/Advection/advection.jl:3-47): Inf outside the component grid's limits,
 * else bisection seeded by the cell index, corner values and N-linear lerp.
 */
static double linp_value(const jpo_grid* g, int comp, const double* V, const double* p, const int64_t* idx,
                         const double* xc, const double* dx, double VL);
static double mqs_value(const jpo_grid* g, int comp, const double* V, const int64_t* idx, const double* v,
                        const double* t);

/* `interp`: the velocity interpolation of the advection call, 0 N-linear
   (advection!), JPO_INTERP_LINP (advection_LinP!) or JPO_INTERP_MQS
   (advection_MQS!) */
static double interp_component(const jpo_grid* g, int comp, const double* p, const int64_t* I,
                               const double* V, int* err, int interp)
{
    const int N = g->ndim;
    for (int d = 0; d < N; ++d) {
        const double* x = g->xvel[comp][d];
        const int64_t L = g->nvel[comp][d];
        if (!(x[0] <= p[d] && p[d] <= x[L - 1])) return INFINITY;
    }
    int64_t idx[3] = {0, 0, 0};
    double t[3], xcs[3], dxs[3];
    for (int d = 0; d < N; ++d) {
        const double* x = g->xvel[comp][d];
        idx[d] = jpo_bisection(p[d], x, g->nvel[comp][d], I[d], err);
        const double xc = x[idx[d]];
        const double dx = g->dxvel[comp][d][idx[d]];
        xcs[d] = xc;
        dxs[d] = dx;
        t[d] = (p[d] - xc) * (1.0 / dx);
    }
    const int64_t L0 = g->nvel[comp][0], L1 = g->nvel[comp][1];
    double v[8];
    if (N == 2) {
        const int64_t b = idx[0] + L0 * idx[1];
        v[0] = V[b];
        v[1] = V[b + 1];
        v[2] = V[b + L0];
        v[3] = V[b + L0 + 1];
    } else {
        const int64_t b = idx[0] + L0 * (idx[1] + L1 * idx[2]);
        const int64_t sz = L0 * L1;
        v[0] = V[b];
        v[1] = V[b + 1];
        v[2] = V[b + L0];
        v[3] = V[b + L0 + 1];
        v[4] = V[b + sz];
        v[5] = V[b + sz + 1];
        v[6] = V[b + sz + L0];
        v[7] = V[b + sz + L0 + 1];
    }
    const double VL = lerpN(N, v, t);
    if (interp == 0) return VL;
    /* away from the edges only: 1 < index < size - 1 (1-based) on every axis */
    for (int d = 0; d < N; ++d)
        if (!(idx[d] >= 1 && idx[d] <= g->nvel[comp][d] - 3)) return VL;
    if (interp == JPO_INTERP_LINP) return linp_value(g, comp, V, p, idx, xcs, dxs, VL);
    return mqs_value(g, comp, V, idx, v, t);
}

/* F(i, j[, k]) of a component grid, indices clamped to the grid */
static inline double vel_at(const jpo_grid* g, int comp, const double* V, int64_t i, int64_t j, int64_t k)
{
    const int64_t L0 = g->nvel[comp][0], L1 = g->nvel[comp][1], L2 = g->ndim == 3 ? g->nvel[comp][2] : 1;
    i = i < 0 ? 0 : (i > L0 - 1 ? L0 - 1 : i);
    j = j < 0 ? 0 : (j > L1 - 1 ? L1 - 1 : j);
    k = k < 0 ? 0 : (k > L2 - 1 ? L2 - 1 : k);
    return V[i + L0 * (j + L1 * k)];
}

/* LinP (src/Particles/Advection/advection_LinP.jl:92-391) for component
   `comp` at a cell away from the grid's edges: VL (the N-linear value) blended
   with the N-linear interpolation of velocities averaged to the pressure
   points, 2/3 VL + (1 - 2/3) VP, without fused operations. */
static double linp_value(const jpo_grid* g, int comp, const double* V, const double* p, const int64_t* idx,
                         const double* xc, const double* dx, double VL)
{
    const int N = g->ndim;
    int64_t b[3] = {idx[0], idx[1], N == 3 ? idx[2] : 0};
    /* offset_LinP: +1 past the middle of the interval along the component axis */
    b[comp] += p[comp] > xc[comp] + dx[comp] / 2.0 ? 1 : 0;
    /* rows of augment_offset (:352-391): the shifts of rows 2..4 */
    int64_t row[4][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
    const int r2 = comp == 1 ? 0 : 1; /* row 2 shifts x (y-component) or y */
    const int r3 = comp == 2 ? 0 : 2; /* row 3 shifts x (z-component) or z */
    row[1][r2] = 1;
    if (N == 3) { /* row 4 = the shifts of rows 2 and 3 together */
        row[2][r3] = 1;
        row[3][r2] = 1;
        row[3][r3] = 1;
    }
    const int nrows = N == 3 ? 4 : 2;
    double av[8];
    for (int r = 0; r < nrows; ++r) {
        double f[3];
        for (int s = -1; s <= 1; ++s) {
            int64_t q[3] = {b[0] + row[r][0], b[1] + row[r][1], b[2] + row[r][2]};
            q[comp] += s;
            f[s + 1] = vel_at(g, comp, V, q[0], q[1], q[2]);
        }
        av[2 * r] = (f[0] + f[1]) / 2.0;
        av[2 * r + 1] = (f[2] + f[1]) / 2.0;
    }
    double FP[8];
    if (comp == 0) {
        for (int k = 0; k < 2 * nrows; ++k) FP[k] = av[k];
    } else { /* swap_F: (1, 3, 2, 4, 5, 7, 6, 8) */
        static const int SW[8] = {0, 2, 1, 3, 4, 6, 5, 7};
        for (int k = 0; k < 2 * nrows; ++k) FP[k] = av[SW[k]];
    }
    /* correct_xci_to_pressure_point (:151-189) */
    double xP[3] = {xc[0], xc[1], N == 3 ? xc[2] : 0.0};
    const int off = 1 - 2 * (p[comp] < xc[comp] + dx[comp] / 2.0);
    xP[comp] = xc[comp] + ((double)off * dx[comp]) / 2.0;
    double tP[3];
    for (int d = 0; d < N; ++d) tP[d] = (p[d] - xP[d]) * (1.0 / dx[d]);
    const double VP = lerpN(N, FP, tP);
    const double A = 2.0 / 3.0;
    const double a = A * VL;
    const double bb = (1.0 - A) * VP;
    return a + bb;
}

/* half * (t - half)^2 * (muladd(-2, v1, v0) + v2) (src/Interpolations/MQS.jl) */
static inline double mqs_correction(double t, double v0, double v1, double v2)
{
    const double d = t - 0.5;
    const double q = 0.5 * (d * d);
    const double s = fma(-2.0, v1, v0) + v2;
    return q * s;
}

/* one MQS pair: lerp of (a, b) at t plus the curvature correction, with the
   stencil extended below (lo) or above (hi) */
static inline double mqs_edge(double t, double a, double b, double lo, double hi)
{
    const double l = lerp1(t, a, b);
    const double c = t < 0.5 ? mqs_correction(t, lo, a, b) : mqs_correction(t, a, b, hi);
    return l + c;
}

/* MQS (src/Interpolations/MQS.jl:1-131) for component `comp` at a cell away
   from the grid's edges; v are the corner values, t the normalised position. */
static double mqs_value(const jpo_grid* g, int comp, const double* V, const int64_t* idx, const double* v,
                        const double* t)
{
    const int64_t i = idx[0], j = idx[1];
    if (g->ndim == 2) {
        if (comp == 0) { /* MQS-x: corrections along x, then lerp along y */
            const double r0 = mqs_edge(t[0], v[0], v[1], vel_at(g, 0, V, i - 1, j, 0), vel_at(g, 0, V, i + 2, j, 0));
            const double r1 =
                mqs_edge(t[0], v[2], v[3], vel_at(g, 0, V, i - 1, j + 1, 0), vel_at(g, 0, V, i + 2, j + 1, 0));
            return lerp1(t[1], r0, r1);
        }
        const double r0 = mqs_edge(t[1], v[0], v[2], vel_at(g, 1, V, i, j - 1, 0), vel_at(g, 1, V, i, j + 2, 0));
        const double r1 =
            mqs_edge(t[1], v[1], v[3], vel_at(g, 1, V, i + 1, j - 1, 0), vel_at(g, 1, V, i + 1, j + 2, 0));
        return lerp1(t[0], r0, r1);
    }
    const int64_t k = idx[2];
    if (comp == 0 || comp == 1) { /* the 2D pair at layers k and k + 1, both with the stencil of layer k */
        double r[2];
        for (int h = 0; h < 2; ++h) {
            const double* w = v + 4 * h;
            double e0, e1;
            if (comp == 0) {
                e0 = mqs_edge(t[0], w[0], w[1], vel_at(g, 0, V, i - 1, j, k), vel_at(g, 0, V, i + 2, j, k));
                e1 = mqs_edge(t[0], w[2], w[3], vel_at(g, 0, V, i - 1, j + 1, k), vel_at(g, 0, V, i + 2, j + 1, k));
                r[h] = lerp1(t[1], e0, e1);
            } else {
                e0 = mqs_edge(t[1], w[0], w[2], vel_at(g, 1, V, i, j - 1, k), vel_at(g, 1, V, i, j + 2, k));
                e1 = mqs_edge(t[1], w[1], w[3], vel_at(g, 1, V, i + 1, j - 1, k), vel_at(g, 1, V, i + 1, j + 2, k));
                r[h] = lerp1(t[0], e0, e1);
            }
        }
        return lerp1(t[2], r[0], r[1]);
    }
    /* MQS-z: front (v1, v2, v5, v6) and back (v3, v4, v7, v8) with the stencil
       of row j, corrections along x, lerp along z, then along y */
    double r[2];
    for (int h = 0; h < 2; ++h) {
        const double w[4] = {v[2 * h], v[2 * h + 1], v[2 * h + 4], v[2 * h + 5]};
        const double e0 = mqs_edge(t[0], w[0], w[1], vel_at(g, 2, V, i - 1, j, k), vel_at(g, 2, V, i + 2, j, k));
        const double e1 =
            mqs_edge(t[0], w[2], w[3], vel_at(g, 2, V, i - 1, j, k + 1), vel_at(g, 2, V, i + 2, j, k + 1));
        r[h] = lerp1(t[2], e0, e1);
    }
    return lerp1(t[1], r[0], r[1]);
}

static void interp_velocity(const jpo_grid* g, const double* p, const int64_t* I,
                            const double* const V[3], double* v, int* err, int interp)
{
    for (int c = 0; c < g->ndim; ++c) v[c] = interp_component(g, c, p, I, V[c], err, interp);
}

/* one velocity sample (interp_velocity2particle[_LinP|_MQS]) at p, bisection
   seeded by the 0-based cell I */
int jpo_interp_velocity(const jpo_grid* g, int interp, const double* const V[3], const double* p,
                        const int64_t* I, double* v)
{
    int err = 0;
    interp_velocity(g, p, I, V, v, &err, interp);
    return err;
}

void jpo_first_stage(int method, double alpha, double dt, int n, const double* v,
                     const double* p, double* out)
{
    /* src/Advection/Euler.jl:1-6 and src/Advection/RK2.jl:7-20:
       muladd(sign, (alpha*dt)*v, p) with sign = 1 */
    for (int d = 0; d < n; ++d) {
        if (method == JPO_EULER)
            out[d] = fma(1.0, dt * v[d], p[d]);
        else
            out[d] = fma(1.0, (alpha * dt) * v[d], p[d]);
    }
}

void jpo_second_stage(double alpha, double dt, int n, const double* v0, const double* v1,
                      const double* p, double* out)
{
    /* src/Advection/RK2.jl:22-44 */
    if (alpha == 0.5) {
        for (int d = 0; d < n; ++d) out[d] = fma(1.0, dt * v1[d], p[d]);
    } else {
        const double ia = 1.0 / alpha;
        const double a = fma(-0.5, ia, 1.0);
        const double b = 0.5 * ia;
        for (int d = 0; d < n; ++d) {
            const double x = fma(a, v0[d], b * v1[d]);
            out[d] = fma(1.0, dt * x, p[d]);
        }
    }
}

static void advect_particle(const jpo_grid* g, int method, double alpha, const double* const V[3],
                            double dt, const int64_t* I, const double* p0, double* pout, int* err, int interp)
{
    const int N = g->ndim;
    if (method == JPO_RK2) {
        /* src/Particles/Advection/advection.jl:154-179 */
        double v0[3], v1[3], p1[3];
        interp_velocity(g, p0, I, V, v0, err, interp);
        jpo_first_stage(JPO_RK2, alpha, dt, N, v0, p0, p1);
        interp_velocity(g, p1, I, V, v1, err, interp);
        jpo_second_stage(alpha, dt, N, v0, v1, p0, pout);
    } else if (method == JPO_RK4) {
        /* src/Particles/Advection/advection.jl:261-279 (no muladd) */
        double k1[3], k2[3], k3[3], k4[3], q[3];
        interp_velocity(g, p0, I, V, k1, err, interp);
        for (int d = 0; d < N; ++d) q[d] = p0[d] + (dt * k1[d]) / 2.0;
        interp_velocity(g, q, I, V, k2, err, interp);
        for (int d = 0; d < N; ++d) q[d] = p0[d] + (dt * k2[d]) / 2.0;
        interp_velocity(g, q, I, V, k3, err, interp);
        for (int d = 0; d < N; ++d) q[d] = p0[d] + dt * k3[d];
        interp_velocity(g, q, I, V, k4, err, interp);
        for (int d = 0; d < N; ++d)
            pout[d] = p0[d] + (dt * (((k1[d] + 2.0 * k2[d]) + 2.0 * k3[d]) + k4[d])) / 6.0;
    } else {
        /* src/Particles/Advection/advection.jl:348-367 */
        double v0[3];
        interp_velocity(g, p0, I, V, v0, err, interp);
        jpo_first_stage(JPO_EULER, alpha, dt, N, v0, p0, pout);
    }
}

int jpo_advection(const jpo_grid* g, int method, double alpha, const double* const V[3],
                  double dt, double* const coords[3], const uint8_t* index)
{
    return jpo_advection_interp(g, method, 0, alpha, V, dt, coords, index);
}

/* advection! / advection_LinP! / advection_MQS!
   (src/Particles/Advection/advection.jl:21-91, advection_LinP.jl:27-90,
   advection_MQS.jl:30-94): the same integrators, with the velocity
   interpolation `interp` */
int jpo_advection_interp(const jpo_grid* g, int method, int interp, double alpha, const double* const V[3],
                         double dt, double* const coords[3], const uint8_t* index)
{
    const int N = g->ndim;
    const int64_t nc = g->ncells;
    const int M = g->max_xcell;
    int err = 0;
#pragma omp parallel for schedule(static) num_threads(nthreads()) reduction(| : err)
    for (int64_t c = 0; c < nc; ++c) {
        int64_t I[3];
        cell_coords(g, c, I);
        /* advection_kernel!: src/Particles/Advection/advection.jl:66-91 */
        for (int s = 0; s < M; ++s) {
            if (!index[c + nc * s]) continue;
            double p0[3], p[3];
            for (int d = 0; d < N; ++d) p0[d] = coords[d][c + nc * s];
            advect_particle(g, method, alpha, V, dt, I, p0, p, &err, interp);
            for (int d = 0; d < N; ++d) coords[d][c + nc * s] = p[d];
        }
    }
    return err;
}

/* -------------------------------------------------------- move_particles! */

static void move_cell(const jpo_grid* g, const int64_t* idx, double* const coords[3],
                      uint8_t* index, double* const* args, int nargs, const double* dom_lo,
                      const double* dom_hi, int* err)
{
    const int N = g->ndim;
    const int64_t nc = g->ncells;
    const int M = g->max_xcell;
    const int64_t c = cell_linear(g, idx);
    double corner[3], dx[3];
    for (int d = 0; d < N; ++d) {
        corner[d] = g->xv[d][idx[d]];
        dx[d] = g->dxv[d][idx[d]];
    }
    /* move_kernel!: src/Particles/move_safe.jl:72-125 */
    int sp = 0; /* starting_point */
    for (int ip = 0; ip < M; ++ip) {
        const int64_t a = c + nc * ip;
        if (!index[a]) continue;
        double p[3];
        for (int d = 0; d < N; ++d) p[d] = coords[d][a];
        if (isincell(N, p, corner, dx)) continue;
        /* indomain: strict, src/Particles/move_safe.jl:199-206 */
        int inside = 1;
        for (int d = 0; d < N; ++d) inside &= (dom_lo[d] < p[d]) & (p[d] < dom_hi[d]);
        if (!inside) {
            index[a] = 0;
            for (int d = 0; d < N; ++d) coords[d][a] = NAN;
            for (int k = 0; k < nargs; ++k) args[k][a] = NAN;
            continue;
        }
        int64_t T[3] = {0, 0, 0};
        int far = 0;
        for (int d = 0; d < N; ++d) {
            T[d] = jpo_bisection(p[d], g->xv[d], g->n[d] + 1, idx[d], err);
            if (T[d] - idx[d] > 1 || idx[d] - T[d] > 1) far = 1;
        }
        double cached[64];
        for (int k = 0; k < nargs; ++k) cached[k] = args[k][a];
        index[a] = 0;
        for (int d = 0; d < N; ++d) coords[d][a] = NAN;
        for (int k = 0; k < nargs; ++k) args[k][a] = NAN;
        if (far) {
            *err |= JPO_ERR_FAR_MOVE;
            continue;
        }
        const int64_t t = cell_linear(g, T);
        int free_idx = -1;
        for (int i = sp; i < M; ++i) { /* find_free_memory: move_safe.jl:192-197 */
            if (!index[t + nc * i]) {
                free_idx = i;
                break;
            }
        }
        if (free_idx < 0) continue;
        sp = free_idx;
        const int64_t b = t + nc * free_idx;
        index[b] = 1;
        for (int d = 0; d < N; ++d) coords[d][b] = p[d];
        for (int k = 0; k < nargs; ++k) args[k][b] = cached[k];
    }
}

int jpo_move_particles(const jpo_grid* g, double* const coords[3], uint8_t* index,
                       double* const* args, int nargs)
{
    const int N = g->ndim;
    int err = 0;
    double lo[3], hi[3];
    int64_t ncol[3] = {1, 1, 1};
    for (int d = 0; d < N; ++d) {
        /* domain_limits = extrema.(grid): src/Particles/move_safe.jl:27 */
        lo[d] = g->xv[d][0];
        hi[d] = g->xv[d][0];
        for (int64_t i = 0; i <= g->n[d]; ++i) {
            const double x = g->xv[d][i];
            if (x < lo[d]) lo[d] = x;
            if (x > hi[d]) hi[d] = x;
        }
        ncol[d] = (g->n[d] + 2) / 3;
    }
    const int npass = N == 2 ? 9 : 27;
    const int64_t ntot = ncol[0] * ncol[1] * ncol[2];
    for (int pass = 0; pass < npass; ++pass) {
        /* offsets loop: i outermost, last axis innermost (move_safe.jl:32,39) */
        int64_t off[3];
        if (N == 2) {
            off[0] = pass / 3;
            off[1] = pass % 3;
            off[2] = 0;
        } else {
            off[0] = pass / 9;
            off[1] = (pass / 3) % 3;
            off[2] = pass % 3;
        }
#pragma omp parallel for schedule(static) num_threads(nthreads()) reduction(| : err)
        for (int64_t w = 0; w < ntot; ++w) {
            int64_t J[3] = {w % ncol[0], (w / ncol[0]) % ncol[1], w / (ncol[0] * ncol[1])};
            int64_t idx[3] = {0, 0, 0};
            int ok = 1;
            for (int d = 0; d < N; ++d) {
                idx[d] = 3 * J[d] + off[d];
                if (idx[d] >= g->n[d]) ok = 0;
            }
            if (ok) move_cell(g, idx, coords, index, args, nargs, lo, hi, &err);
        }
    }
    return err;
}

/* ------------------------------------------------------ inject_particles! */

/* index_min_distance: src/Particles/injection.jl:330-393 */
static int nearest_particle(const jpo_grid* g, double* const coords[3], const uint8_t* index,
                            const double* pn, int cur_slot, const int64_t* I, int64_t* best_a)
{
    const int N = g->ndim;
    const int64_t nc = g->ncells;
    const int M = g->max_xcell;
    double dmin = INFINITY;
    int found = 0;
    const int kr = N == 3 ? 1 : 0;
    for (int64_t k = I[2] - kr; k <= I[2] + kr; ++k) {
        for (int64_t j = I[1] - 1; j <= I[1] + 1; ++j) {
            for (int64_t i = I[0] - 1; i <= I[0] + 1; ++i) {
                if (i < 0 || j < 0 || k < 0) continue;
                if (i >= g->n[0] || j >= g->n[1] || (N == 3 && k >= g->n[2])) continue;
                const int64_t J[3] = {i, j, k};
                const int64_t c = cell_linear(g, J);
                const int self = (i == I[0] && j == I[1] && k == I[2]);
                for (int ip = 0; ip < M; ++ip) {
                    if (self && ip == cur_slot) continue;
                    const int64_t a = c + nc * ip;
                    if (!index[a]) continue;
                    double s;
                    if (N == 2) {
                        const double px = coords[0][a], py = coords[1][a];
                        if (isnan(px) || isnan(py)) continue;
                        const double dxx = px - pn[0], dyy = py - pn[1];
                        s = dxx * dxx + dyy * dyy;
                    } else {
                        const double dxx = coords[0][a] - pn[0];
                        const double dyy = coords[1][a] - pn[1];
                        const double dzz = coords[2][a] - pn[2];
                        s = (dxx * dxx + dyy * dyy) + dzz * dzz;
                    }
                    const double dist = sqrt(s);
                    if (dist < dmin) {
                        dmin = dist;
                        *best_a = a;
                        found = 1;
                    }
                }
            }
        }
    }
    return found;
}

static void inject_cell(const jpo_grid* g, const int64_t* idx, double* const coords[3],
                        uint8_t* index, double* const* args, int nargs, uint32_t call, int* err)
{
    /* _inject_particles!: src/Particles/injection.jl:68-131 */
    const int N = g->ndim;
    const int64_t nc = g->ncells;
    const int M = g->max_xcell;
    const int NQ = 1 << N;
    const int64_t c = cell_linear(g, idx);
    double corner[3], dq[3];
    for (int d = 0; d < N; ++d) {
        corner[d] = g->xv[d][idx[d]];
        dq[d] = g->dxv[d][idx[d]] / 2.0;
    }
    const int min_xq = (g->min_xcell + NQ - 1) / NQ; /* cld(min_xcell, 2^N) */
    for (int q = 0; q < NQ; ++q) {
        double qc[3];
        for (int d = 0; d < N; ++d) qc[d] = corner[d] + dq[d] * (double)((q >> d) & 1);
        int count = 0;
        for (int i = 0; i < M; ++i) {
            const int64_t a = c + nc * i;
            if (!index[a]) continue;
            double p[3];
            for (int d = 0; d < N; ++d) p[d] = coords[d][a];
            if (isincell(N, p, qc, dq)) ++count;
        }
        if (count >= min_xq) break;
        for (int i = 0; i < M; ++i) {
            const int64_t a = c + nc * i;
            if (index[a]) continue;
            ++count;
            double pn[3];
            for (int d = 0; d < N; ++d) {
                /* new_particle: src/Particles/injection.jl:411-417 */
                const double r = jp_rand_uniform(g->seed, JP_RNG_STREAM_INJECT, call,
                                                 (uint64_t)c, (uint32_t)i, (uint32_t)d);
                pn[d] = qc[d] + dq[d] * fma(0.95, r, 0.05);
            }
            for (int d = 0; d < N; ++d) coords[d][a] = pn[d];
            index[a] = 1;
            int64_t src = 0;
            if (nearest_particle(g, coords, index, pn, i, idx, &src)) {
                for (int k = 0; k < nargs; ++k) args[k][a] = args[k][src];
            } else if (nargs > 0) {
                *err |= JPO_ERR_NO_NEIGHBOUR;
            }
            if (count >= min_xq) break;
        }
    }
}

/* Julia's min / max on floats: NaN wins, -0.0 is below +0.0 */
static inline double jl_min(double x, double y)
{
    return ((y < x) || (!!signbit(y) > !!signbit(x))) ? (isnan(x) ? x : y) : (isnan(y) ? y : x);
}

static inline double jl_max(double x, double y)
{
    return ((y > x) || (!!signbit(y) < !!signbit(x))) ? (isnan(x) ? x : y) : (isnan(y) ? y : x);
}

/* the field value given to an injected particle by inject_particles_phase!
   (src/Particles/injection.jl:300-318): the N-linear interpolation at p of a
   cell-centred field (the centre cell below p, clamped, centre spacing) or a
   vertex field (the particle's own cell), clamped to the extrema of the
   interpolation's corner values */
static double phase_field_value(const jpo_grid* g, const double* F, int centred, const double* pn, const int64_t* I,
                                const double* corner, const double* dq)
{
    const int N = g->ndim;
    int64_t J[3] = {0, 0, 0};
    double t[3];
    int64_t L0, L1;
    if (centred) {
        for (int d = 0; d < N; ++d) {
            const double xcen = corner[d] + dq[d];
            int64_t j = pn[d] < xcen ? I[d] - 1 : I[d];
            const int64_t hi = g->n[d] - 2;
            j = j < 0 ? 0 : (j > hi ? hi : j);
            J[d] = j;
            t[d] = (pn[d] - g->xc[d][j]) * (1.0 / g->dxc[d][j]);
        }
        L0 = g->n[0];
        L1 = g->n[1];
    } else {
        for (int d = 0; d < N; ++d) {
            J[d] = I[d];
            t[d] = (pn[d] - g->xv[d][I[d]]) * (1.0 / g->dxv[d][I[d]]);
        }
        L0 = g->n[0] + 1;
        L1 = g->n[1] + 1;
    }
    const int64_t b = J[0] + L0 * (J[1] + (N == 3 ? L1 * J[2] : 0));
    const int64_t sz = L0 * L1;
    const int64_t off[8] = {b, b + 1, b + L0, b + L0 + 1, b + sz, b + sz + 1, b + sz + L0, b + sz + L0 + 1};
    double v[8] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
    for (int k = 0; k < (1 << N); ++k) v[k] = F[off[k]];
    const double tmp = lerpN(N, v, t);
    double lo = v[0], hi = v[0];
    for (int k = 1; k < (1 << N); ++k) {
        hi = jl_max(v[k], hi);
        lo = jl_min(v[k], lo);
    }
    return tmp > hi ? hi : (tmp < lo ? lo : tmp);  /* clamp */
}

/* _inject_particles_phase! (src/Particles/injection.jl:232-325): as
   _inject_particles! but every quadrant is checked (`continue`, not `break`),
   the new particle copies the phase of its nearest neighbour, and each field
   in args takes the clamped interpolation of the matching grid field. */
static void inject_cell_phase(const jpo_grid* g, const int64_t* idx, double* const coords[3], uint8_t* index,
                              double* phases, double* const* args, const double* const* fields,
                              const int* centred, int nargs, uint32_t call, int* err)
{
    const int N = g->ndim;
    const int64_t nc = g->ncells;
    const int M = g->max_xcell;
    const int NQ = 1 << N;
    const int64_t c = cell_linear(g, idx);
    double corner[3], dq[3];
    for (int d = 0; d < N; ++d) {
        corner[d] = g->xv[d][idx[d]];
        dq[d] = g->dxv[d][idx[d]] / 2.0;
    }
    const int min_xq = (g->min_xcell + NQ - 1) / NQ;
    for (int q = 0; q < NQ; ++q) {
        double qc[3];
        for (int d = 0; d < N; ++d) qc[d] = corner[d] + dq[d] * (double)((q >> d) & 1);
        int count = 0;
        for (int i = 0; i < M; ++i) {
            const int64_t a = c + nc * i;
            if (!index[a]) continue;
            double p[3];
            for (int d = 0; d < N; ++d) p[d] = coords[d][a];
            if (isincell(N, p, qc, dq)) ++count;
        }
        if (count >= min_xq) continue;
        for (int i = 0; i < M; ++i) {
            const int64_t a = c + nc * i;
            if (index[a]) continue;
            ++count;
            double pn[3];
            for (int d = 0; d < N; ++d) {
                const double r = jp_rand_uniform(g->seed, JP_RNG_STREAM_INJECT, call, (uint64_t)c, (uint32_t)i,
                                                 (uint32_t)d);
                pn[d] = qc[d] + dq[d] * fma(0.95, r, 0.05);
            }
            int64_t src = 0;
            if (nearest_particle(g, coords, index, pn, i, idx, &src))
                phases[a] = phases[src];
            else
                *err |= JPO_ERR_NO_NEIGHBOUR;
            for (int d = 0; d < N; ++d) coords[d][a] = pn[d];
            index[a] = 1;
            for (int k = 0; k < nargs; ++k)
                args[k][a] = phase_field_value(g, fields[k], centred[k], pn, idx, corner, dq);
            if (count >= min_xq) break;
        }
    }
}

int jpo_inject_particles_phase(const jpo_grid* g, double* const coords[3], uint8_t* index, double* phases,
                               double* const* args, const double* const* fields, const int* centred, int nargs,
                               uint32_t call)
{
    const int N = g->ndim;
    int err = 0;
    int64_t ncol[3] = {1, 1, 1};
    for (int d = 0; d < N; ++d) ncol[d] = (g->n[d] + 1) / 2;
    const int npass = 1 << N;
    const int64_t ntot = ncol[0] * ncol[1] * ncol[2];
    for (int pass = 0; pass < npass; ++pass) {
        int64_t off[3];
        if (N == 2) {
            off[0] = pass / 2;
            off[1] = pass % 2;
            off[2] = 0;
        } else {
            off[0] = pass / 4;
            off[1] = (pass / 2) % 2;
            off[2] = pass % 2;
        }
#pragma omp parallel for schedule(static) num_threads(nthreads()) reduction(| : err)
        for (int64_t w = 0; w < ntot; ++w) {
            int64_t J[3] = {w % ncol[0], (w / ncol[0]) % ncol[1], w / (ncol[0] * ncol[1])};
            int64_t idx[3] = {0, 0, 0};
            int ok = 1;
            for (int d = 0; d < N; ++d) {
                idx[d] = 2 * J[d] + off[d];
                if (idx[d] >= g->n[d]) ok = 0;
            }
            if (ok) inject_cell_phase(g, idx, coords, index, phases, args, fields, centred, nargs, call, &err);
        }
    }
    return err;
}

int jpo_inject_particles(const jpo_grid* g, double* const coords[3], uint8_t* index,
                         double* const* args, int nargs, uint32_t call)
{
    const int N = g->ndim;
    int err = 0;
    int64_t ncol[3] = {1, 1, 1};
    for (int d = 0; d < N; ++d) ncol[d] = (g->n[d] + 1) / 2; /* ceil(n*0.5) */
    const int npass = 1 << N;
    const int64_t ntot = ncol[0] * ncol[1] * ncol[2];
    for (int pass = 0; pass < npass; ++pass) {
        /* offsets loop: i outermost, last axis innermost (injection.jl:31,38) */
        int64_t off[3];
        if (N == 2) {
            off[0] = pass / 2;
            off[1] = pass % 2;
            off[2] = 0;
        } else {
            off[0] = pass / 4;
            off[1] = (pass / 2) % 2;
            off[2] = pass % 2;
        }
#pragma omp parallel for schedule(static) num_threads(nthreads()) reduction(| : err)
        for (int64_t w = 0; w < ntot; ++w) {
            int64_t J[3] = {w % ncol[0], (w / ncol[0]) % ncol[1], w / (ncol[0] * ncol[1])};
            int64_t idx[3] = {0, 0, 0};
            int ok = 1;
            for (int d = 0; d < N; ++d) {
                idx[d] = 2 * J[d] + off[d];
                if (idx[d] >= g->n[d]) ok = 0;
            }
            if (ok) inject_cell(g, idx, coords, index, args, nargs, call, &err);
        }
    }
    return err;
}

/* ---------------------------------------------------------- grid2particle! */

void jpo_grid2particle(const jpo_grid* g, double* Fp, const double* F,
                       const double* const coords[3], const uint8_t* index)
{
    const int N = g->ndim;
    const int64_t nc = g->ncells;
    const int M = g->max_xcell;
    const int64_t V0 = g->n[0] + 1, V1 = g->n[1] + 1;
#pragma omp parallel for schedule(static) num_threads(nthreads())
    for (int64_t c = 0; c < nc; ++c) {
        int64_t I[3];
        cell_coords(g, c, I);
        /* _grid2particle_classic!: src/Interpolations/grid_to_particle.jl:64-82 */
        double x0[3], dx[3], v[8];
        for (int d = 0; d < N; ++d) {
            x0[d] = g->xv[d][I[d]];
            dx[d] = g->dxv[d][I[d]];
        }
        const int64_t b = I[0] + V0 * (I[1] + (N == 3 ? V1 * I[2] : 0));
        v[0] = F[b];
        v[1] = F[b + 1];
        v[2] = F[b + V0];
        v[3] = F[b + V0 + 1];
        if (N == 3) {
            const int64_t sz = V0 * V1;
            v[4] = F[b + sz];
            v[5] = F[b + sz + 1];
            v[6] = F[b + sz + V0];
            v[7] = F[b + sz + V0 + 1];
        }
        for (int s = 0; s < M; ++s) {
            const int64_t a = c + nc * s;
            if (!index[a]) continue;
            double t[3];
            for (int d = 0; d < N; ++d) t[d] = (coords[d][a] - x0[d]) * (1.0 / dx[d]);
            Fp[a] = lerpN(N, v, t);
        }
    }
}

/* ---------------------------------------------------- grid2particle_flip! */

/*
 * grid2particle_flip!(Fp, xvi, F, F0, particles; α) with xvi = the vertex grid
 * (src/Interpolations/grid_to_particle.jl:125-170): per live particle the PIC
 * values of F and F0 at its position, then the blend
 * muladd(F_pic, α, (Fp + (F_pic - F0_pic)) * (1 - α)). The spacing is
 * grid_size(xvi) (src/Interpolations/utils.jl:61-63): the smallest vertex
 * spacing of each axis, used for every cell.
 */
void jpo_grid2particle_flip(const jpo_grid* g, double* Fp, const double* F, const double* F0, double alpha,
                            const double* const coords[3], const uint8_t* index)
{
    const int N = g->ndim;
    const int64_t nc = g->ncells;
    const int M = g->max_xcell;
    const int64_t V0 = g->n[0] + 1, V1 = g->n[1] + 1;
    double di[3];
    for (int d = 0; d < N; ++d) {
        double m = g->xv[d][1] - g->xv[d][0];
        for (int64_t i = 1; i < g->n[d]; ++i) {
            const double s = g->xv[d][i + 1] - g->xv[d][i];
            m = s < m ? s : m;
        }
        di[d] = fabs(m);
    }
    const double beta = 1.0 - alpha;
#pragma omp parallel for schedule(static) num_threads(nthreads())
    for (int64_t c = 0; c < nc; ++c) {
        int64_t I[3];
        cell_coords(g, c, I);
        double x0[3], v[8], v0[8];
        for (int d = 0; d < N; ++d) x0[d] = g->xv[d][I[d]];
        const int64_t b = I[0] + V0 * (I[1] + (N == 3 ? V1 * I[2] : 0));
        const int64_t sz = V0 * V1;
        const int64_t off[8] = {b, b + 1, b + V0, b + V0 + 1, b + sz, b + sz + 1, b + sz + V0, b + sz + V0 + 1};
        for (int k = 0; k < (1 << N); ++k) {
            v[k] = F[off[k]];
            v0[k] = F0[off[k]];
        }
        for (int s = 0; s < M; ++s) {
            const int64_t a = c + nc * s;
            if (!index[a]) continue;
            double t[3];
            for (int d = 0; d < N; ++d) t[d] = (coords[d][a] - x0[d]) * (1.0 / di[d]);
            const double fpic = lerpN(N, v, t), f0pic = lerpN(N, v0, t);
            const double flip = Fp[a] + (fpic - f0pic);
            Fp[a] = fma(fpic, alpha, flip * beta);
        }
    }
}

/* ------------------------------------------------------- centroid2particle! */

/*
 * centroid2particle!(Fp, F, particles) (src/Interpolations/centroid_to_particle.jl:13-46):
 * every slot with non-NaN coordinates (the reference tests the coordinates,
 * not the index) takes the N-linear interpolation of the cell-centred field F
 * from the centre cell below it along each axis (its own cell's centre, or the
 * previous one if the particle lies below that centre), clamped to the
 * centre grid, with the centre spacing of Particles.di.center.
 */
void jpo_centroid2particle(const jpo_grid* g, double* Fp, const double* F, const double* const coords[3])
{
    const int N = g->ndim;
    const int64_t nc = g->ncells;
    const int M = g->max_xcell;
    const int64_t C0 = g->n[0], C1 = g->n[1];
#pragma omp parallel for schedule(static) num_threads(nthreads())
    for (int64_t c = 0; c < nc; ++c) {
        int64_t I[3];
        cell_coords(g, c, I);
        for (int s = 0; s < M; ++s) {
            const int64_t a = c + nc * s;
            double p[3];
            int nan = 0;
            for (int d = 0; d < N; ++d) {
                p[d] = coords[d][a];
                nan |= isnan(p[d]);
            }
            if (nan) continue;
            int64_t J[3] = {0, 0, 0};
            double t[3];
            for (int d = 0; d < N; ++d) {
                int64_t j = p[d] < g->xc[d][I[d]] ? I[d] - 1 : I[d];  /* shifted_index */
                const int64_t hi = g->n[d] - 2;                        /* clamp to 1..size(F)-1 (1-based) */
                j = j < 0 ? 0 : (j > hi ? hi : j);
                J[d] = j;
                t[d] = (p[d] - g->xc[d][j]) * (1.0 / g->dxc[d][j]);
            }
            const int64_t b = J[0] + C0 * (J[1] + (N == 3 ? C1 * J[2] : 0));
            const int64_t sz = C0 * C1;
            double v[8];
            const int64_t off[8] = {b, b + 1, b + C0, b + C0 + 1, b + sz, b + sz + 1, b + sz + C0, b + sz + C0 + 1};
            for (int k = 0; k < (1 << N); ++k) v[k] = F[off[k]];
            Fp[a] = lerpN(N, v, t);
        }
    }
}

/* ------------------------------------------------------- particle2centroid! */

/*
 * particle2centroid!(F, Fp, particles) (src/Interpolations/particle_to_grid_centroid.jl:10-45 2D,
 * :88-110 3D): per cell, the bilinear-weight average of its own particles'
 * values at the cell centre, weight prod_d muladd(-|xc_d - p_d|, inv(dx_d), 1)
 * (bilinear_weight, src/Interpolations/particle_to_grid.jl:210-222) with the
 * cell's vertex spacing. 2D skips slots with any NaN coordinate, 3D those
 * whose first coordinate is NaN; 2D divides, 3D multiplies by the inverse.
 */
void jpo_particle2centroid(const jpo_grid* g, double* F, const double* Fp, const double* const coords[3])
{
    const int N = g->ndim;
    const int64_t nc = g->ncells;
    const int M = g->max_xcell;
#pragma omp parallel for schedule(static) num_threads(nthreads())
    for (int64_t c = 0; c < nc; ++c) {
        int64_t I[3];
        cell_coords(g, c, I);
        double xcen[3], dx[3];
        for (int d = 0; d < N; ++d) {
            xcen[d] = g->xc[d][I[d]];
            dx[d] = g->dxv[d][I[d]];
        }
        double w = 0.0, wF = 0.0;
        for (int s = 0; s < M; ++s) {
            const int64_t a = c + nc * s;
            double p[3];
            int skip = 0;
            for (int d = 0; d < N; ++d) {
                p[d] = coords[d][a];
                if (N == 2 || d == 0) skip |= isnan(p[d]);
            }
            if (skip) continue;
            double wi = 1.0;
            for (int d = 0; d < N; ++d) wi *= fma(-fabs(xcen[d] - p[d]), 1.0 / dx[d], 1.0);
            w += wi;
            wF = fma(wi, Fp[a], wF);
        }
        F[c] = N == 2 ? wF / w : wF * (1.0 / w);
    }
}

/* ---------------------------------------------------------- phase ratios */

#define JPO_MAX_PHASES 16

/* bilinear_weight (src/PhaseRatios/utils.jl:64-74): prod_d muladd(-|a_d - b_d|, inv(di_d), 1) */
static inline double bilinear_weight(int N, const double* a, const double* b, const double* di)
{
    double val = 1.0;
    for (int d = 0; d < N; ++d) val *= fma(-fabs(a[d] - b[d]), 1.0 / di[d], 1.0);
    return val;
}

/* w .* inv(sum(w)) with sum a left fold over the phases */
static inline void normalise(int nph, double* w)
{
    double s = w[0];
    for (int k = 1; k < nph; ++k) s = s + w[k];
    const double is = 1.0 / s;
    for (int k = 0; k < nph; ++k) w[k] = w[k] * is;
}

/* w .+ x .* ntuple(j -> ph == j) (src/PhaseRatios/utils.jl:55-58): only the
   matching phase moves (the others add a signed zero) */
static inline void accumulate_weight(int nph, double* w, double x, double ph)
{
    for (int k = 0; k < nph; ++k)
        if (ph == (double)(k + 1)) w[k] = w[k] + x;
}

static inline void cell_spacing(const jpo_grid* g, const int64_t* J, double* di)
{
    for (int d = 0; d < g->ndim; ++d) di[d] = g->dxv[d][J[d]];
}

/* phase_ratios_center! (src/PhaseRatios/centers.jl:3-30, phase_ratio_weights
   utils.jl:44-61): the cell's own particles, weight at the cell centre with
   the cell's vertex spacing; slots skipped when their first coordinate is NaN. */
void jpo_phase_ratios_center(const jpo_grid* g, int nph, const double* phases, const double* const coords[3],
                             double* out)
{
    const int N = g->ndim;
    const int64_t nc = g->ncells;
    const int M = g->max_xcell;
#pragma omp parallel for schedule(static) num_threads(nthreads())
    for (int64_t c = 0; c < nc; ++c) {
        int64_t I[3];
        cell_coords(g, c, I);
        double xc[3], di[3], w[JPO_MAX_PHASES] = {0};
        for (int d = 0; d < N; ++d) xc[d] = g->xc[d][I[d]];
        cell_spacing(g, I, di);
        for (int s = 0; s < M; ++s) {
            const int64_t a = c + nc * s;
            double p[3] = {0.0, 0.0, 0.0};
            for (int d = 0; d < N; ++d) p[d] = coords[d][a];
            if (isnan(p[0])) continue;
            accumulate_weight(nph, w, bilinear_weight(N, xc, p, di), phases[a]);
        }
        normalise(nph, w);
        for (int k = 0; k < nph; ++k) out[c + nc * k] = w[k];
    }
}

/* phase_ratios_vertex! (src/PhaseRatios/vertices.jl:4-107): particles of the
   2^N cells around the vertex (offsets -1..0, the first axis outermost), those
   within half a cell of it on every axis, weight with each cell's spacing. */
void jpo_phase_ratios_vertex(const jpo_grid* g, int nph, const double* phases, const double* const coords[3],
                             double* out)
{
    const int N = g->ndim;
    const int64_t nc = g->ncells;
    const int M = g->max_xcell;
    const int64_t V0 = g->n[0] + 1, V1 = g->n[1] + 1, V2 = N == 3 ? g->n[2] + 1 : 1;
    const int64_t nv = V0 * V1 * V2;
#pragma omp parallel for schedule(static) num_threads(nthreads())
    for (int64_t v = 0; v < nv; ++v) {
        const int64_t I[3] = {v % V0, (v / V0) % V1, v / (V0 * V1)};
        double xv[3], w[JPO_MAX_PHASES] = {0};
        for (int d = 0; d < N; ++d) xv[d] = g->xv[d][I[d]];
        for (int oi = -1; oi <= 0; ++oi)
            for (int oj = -1; oj <= 0; ++oj)
                for (int ok = (N == 3 ? -1 : 0); ok <= 0; ++ok) {
                    const int64_t J[3] = {I[0] + oi, I[1] + oj, N == 3 ? I[2] + ok : 0};
                    if (J[0] < 0 || J[0] >= g->n[0] || J[1] < 0 || J[1] >= g->n[1]) continue;
                    if (N == 3 && (J[2] < 0 || J[2] >= g->n[2])) continue;
                    const int64_t c = J[0] + g->n[0] * (J[1] + g->n[1] * J[2]);
                    double di[3];
                    cell_spacing(g, J, di);
                    for (int s = 0; s < M; ++s) {
                        const int64_t a = c + nc * s;
                        double p[3];
                        int nan = 0, far = 0;
                        for (int d = 0; d < N; ++d) {
                            p[d] = coords[d][a];
                            nan |= isnan(p[d]);
                        }
                        if (nan) continue;
                        for (int d = 0; d < N && !far; ++d) far = fabs(p[d] - xv[d]) >= di[d] / 2.0;
                        if (far) continue;
                        accumulate_weight(nph, w, bilinear_weight(N, xv, p, di), phases[a]);
                    }
                }
        normalise(nph, w);
        for (int k = 0; k < nph; ++k) out[v + nv * k] = w[k];
    }
}

/* isinhalfcell (src/PhaseRatios/utils.jl:79): |p_d - x_d| <= di_d / 2 on every axis */
static inline int in_half_cell(int N, const double* p, const double* x, const double* di)
{
    int in = 1;
    for (int d = 0; d < N; ++d) in &= fabs(p[d] - x[d]) <= di[d] / 2.0;
    return in;
}

static void face_cell_particles(const jpo_grid* g, int nph, const double* phases, const double* const coords[3],
                                int64_t c, const double* x, const double* di, double* w)
{
    const int N = g->ndim;
    const int64_t nc = g->ncells;
    for (int s = 0; s < g->max_xcell; ++s) {
        const int64_t a = c + nc * s;
        double p[3];
        int nan = 0;
        for (int d = 0; d < N; ++d) {
            p[d] = coords[d][a];
            nan |= isnan(p[d]);
        }
        if (nan || !in_half_cell(N, p, x, di)) continue;
        accumulate_weight(nph, w, bilinear_weight(N, x, p, di), phases[a]);
    }
}

/* phase_ratios_face! (src/PhaseRatios/midpoints.jl:3-94) along axis `dim`: per
   cell I, the face I + e_dim gathers the particles of cells I and
   min(I + e_dim, n) (the last cell twice at the far boundary, as the reference
   does) within half a cell of the face; the first cell also writes face I
   (the near boundary), with the spacing the loop left behind. Faces without
   particles get 0. The output grid is n + e_dim. */
void jpo_phase_ratios_face(const jpo_grid* g, int nph, const double* phases, const double* const coords[3],
                           int dim, double* out)
{
    const int N = g->ndim;
    const int64_t nc = g->ncells;
    int64_t F[3] = {g->n[0], g->n[1], N == 3 ? g->n[2] : 1};
    F[dim] += 1;
    const int64_t nf = F[0] * F[1] * F[2];
#pragma omp parallel for schedule(static) num_threads(nthreads())
    for (int64_t c = 0; c < nc; ++c) {
        int64_t I[3];
        cell_coords(g, c, I);
        double di[3], xf[3], w[JPO_MAX_PHASES] = {0};
        cell_spacing(g, I, di);
        for (int d = 0; d < N; ++d) xf[d] = g->xc[d][I[d]] + (d == dim ? (di[d] * 1.0) / 2.0 : (di[d] * 0.0) / 2.0);
        double xcen[3];
        for (int d = 0; d < N; ++d) xcen[d] = g->xc[d][I[d]];
        for (int it = 0; it < 2; ++it) {
            int64_t J[3] = {I[0], I[1], I[2]};
            if (it == 1) J[dim] = J[dim] + 1 < g->n[dim] ? J[dim] + 1 : g->n[dim] - 1;
            cell_spacing(g, J, di);
            face_cell_particles(g, nph, phases, coords, J[0] + g->n[0] * (J[1] + g->n[1] * J[2]), xf, di, w);
        }
        normalise(nph, w);
        int64_t Fi[3] = {I[0], I[1], I[2]};
        Fi[dim] += 1;
        const int64_t fo = Fi[0] + F[0] * (Fi[1] + F[1] * Fi[2]);
        for (int k = 0; k < nph; ++k) out[fo + nf * k] = isnan(w[k]) ? 0.0 : w[k];
        if (I[dim] == 0) {
            double xb[3], wb[JPO_MAX_PHASES] = {0};
            for (int d = 0; d < N; ++d) xb[d] = xcen[d] - (d == dim ? (di[d] * 1.0) / 2.0 : (di[d] * 0.0) / 2.0);
            face_cell_particles(g, nph, phases, coords, c, xb, di, wb);
            normalise(nph, wb);
            const int64_t fb = I[0] + F[0] * (I[1] + F[1] * I[2]);
            for (int k = 0; k < nph; ++k) out[fb + nf * k] = isnan(wb[k]) ? 0.0 : wb[k];
        }
    }
}

/* phase_ratios_midpoint! (src/PhaseRatios/midpoints.jl:108-242), 3D: the
   edge midpoints `which` = 0 (xy, offsets (1,1,0)), 1 (yz, (0,1,1)), 2 (xz,
   (1,0,1)). Per cell I the midpoint I + offsets sits at the cell centre plus
   half the cell's spacing along the offset axes and gathers the cells
   min(I + offsets .* mask, n) for mask (1,0,0), (0,1,0), (0,0,1), (1,1,1) in
   that order (a clamped cell is visited again). A cell on a first boundary
   of an offset axis also writes midpoint I, and midpoint I + b where b marks
   the offset axes on which I is the last cell, both from the particles
   around the cell centre moved by half a spacing along b. Midpoints without
   particles get 0. Output shape: n + offsets. */
void jpo_phase_ratios_midpoint(const jpo_grid* g, int nph, const double* phases, const double* const coords[3],
                               int which, double* out)
{
    static const int OFF[3][3] = {{1, 1, 0}, {0, 1, 1}, {1, 0, 1}};
    static const int MASK[4][3] = {{1, 0, 0}, {0, 1, 0}, {0, 0, 1}, {1, 1, 1}};
    const int* off = OFF[which];
    const int64_t nc = g->ncells;
    const int64_t Mn[3] = {g->n[0] + off[0], g->n[1] + off[1], g->n[2] + off[2]};
    const int64_t nm = Mn[0] * Mn[1] * Mn[2];
#pragma omp parallel for schedule(static) num_threads(nthreads())
    for (int64_t c = 0; c < nc; ++c) {
        int64_t I[3];
        cell_coords(g, c, I);
        double xcen[3], di[3], xm[3], w[JPO_MAX_PHASES] = {0};
        cell_spacing(g, I, di);
        for (int d = 0; d < 3; ++d) {
            xcen[d] = g->xc[d][I[d]];
            xm[d] = xcen[d] + (di[d] * (double)off[d]) / 2.0;
        }
        for (int m = 0; m < 4; ++m) {
            int64_t J[3];
            for (int d = 0; d < 3; ++d) {
                const int64_t j = I[d] + off[d] * MASK[m][d];
                J[d] = j < g->n[d] - 1 ? j : g->n[d] - 1;
            }
            double dj[3];
            cell_spacing(g, J, dj);
            face_cell_particles(g, nph, phases, coords, J[0] + g->n[0] * (J[1] + g->n[1] * J[2]), xm, dj, w);
        }
        normalise(nph, w);
        const int64_t mo = (I[0] + off[0]) + Mn[0] * ((I[1] + off[1]) + Mn[1] * (I[2] + off[2]));
        for (int k = 0; k < nph; ++k) out[mo + nm * k] = isnan(w[k]) ? 0.0 : w[k];
        /* isboundary (utils.jl:86-91): the first cell along an offset axis */
        int first = 0, b[3];
        for (int d = 0; d < 3; ++d) {
            first |= off[d] && I[d] == 0;
            b[d] = off[d] && I[d] == g->n[d] - 1; /* lastboundary_offset, midpoints.jl:226-229 */
        }
        if (!first) continue;
        double xb[3], wb[JPO_MAX_PHASES] = {0};
        for (int d = 0; d < 3; ++d) xb[d] = xcen[d] - ((di[d] * (double)off[d]) * (double)(0 - b[d])) / 2.0;
        for (int m = 0; m < 4; ++m) {
            int64_t J[3];
            for (int d = 0; d < 3; ++d) {
                const int64_t j = I[d] + off[d] * MASK[m][d];
                J[d] = j < g->n[d] - 1 ? j : g->n[d] - 1;
            }
            double dj[3];
            cell_spacing(g, J, dj);
            face_cell_particles(g, nph, phases, coords, J[0] + g->n[0] * (J[1] + g->n[1] * J[2]), xb, dj, wb);
        }
        normalise(nph, wb);
        for (int r = 0; r < 2; ++r) {
            const int64_t K[3] = {I[0] + r * b[0], I[1] + r * b[1], I[2] + r * b[2]};
            const int64_t ko = K[0] + Mn[0] * (K[1] + Mn[1] * K[2]);
            for (int k = 0; k < nph; ++k) out[ko + nm * k] = isnan(wb[k]) ? 0.0 : wb[k];
        }
    }
}

/* ---------------------------------------------------------- particle2grid! */

void jpo_particle2grid(const jpo_grid* g, double* F, const double* Fp,
                       const double* const coords[3], const uint8_t* index)
{
    const int N = g->ndim;
    const int64_t nc = g->ncells;
    const int M = g->max_xcell;
    const int64_t V0 = g->n[0] + 1, V1 = g->n[1] + 1, V2 = N == 3 ? g->n[2] + 1 : 1;
    const int64_t nv = V0 * V1 * V2;
#pragma omp parallel for schedule(static) num_threads(nthreads())
    for (int64_t v = 0; v < nv; ++v) {
        const int64_t i = v % V0, j = (v / V0) % V1, k = v / (V0 * V1);
        const double xq = g->xv[0][i], yq = g->xv[1][j], zq = N == 3 ? g->xv[2][k] : 0.0;
        double w = 0.0, wF = 0.0;
        /* src/Interpolations/particle_to_grid.jl:37-68 (2D), :113-151 (3D) */
        const int kmin = N == 3 ? -1 : 0;
        for (int ko = kmin; ko <= 0; ++ko) {
            const int64_t kc = k + ko;
            if (N == 3 && !(0 <= kc && kc < g->n[2])) continue;
            for (int jo = -1; jo <= 0; ++jo) {
                const int64_t jc = j + jo;
                if (!(0 <= jc && jc < g->n[1])) continue;
                for (int io = -1; io <= 0; ++io) {
                    const int64_t ic = i + io;
                    if (!(0 <= ic && ic < g->n[0])) continue;
                    const int64_t c = ic + g->n[0] * (jc + g->n[1] * (N == 3 ? kc : 0));
                    for (int s = 0; s < M; ++s) {
                        const int64_t a = c + nc * s;
                        if (!index[a]) continue;
                        double ss;
                        const double ddx = xq - coords[0][a];
                        const double ddy = yq - coords[1][a];
                        if (N == 2) {
                            ss = ddx * ddx + ddy * ddy;
                        } else {
                            const double ddz = zq - coords[2][a];
                            ss = (ddx * ddx + ddy * ddy) + ddz * ddz;
                        }
                        const double dist = sqrt(ss);
                        const double wi = 1.0 / (dist * dist);
                        w += wi;
                        wF = fma(wi, Fp[a], wF);
                    }
                }
            }
        }
        F[v] = N == 2 ? wF / w : wF * (1.0 / w);
    }
}

/*
 * particle2grid! with a tuple of fields (src/Interpolations/particle_to_grid.jl:
 * 70-109 in 2D, 153-199 in 3D): the scalar form's cells, slots and weights
 * (inv(distance^2)), one weighted sum per field, ωxF[j] = muladd(ω_i, Fp[j],
 * ωxF[j]) in slot order, then F[j] = ωxF[j] * inv(ω) for every field (2D and
 * 3D alike). The reference's tuple kernels themselves stop on their first
 * particle for more than one field: the 2D one starts ωxF as one number and
 * indexes it with the field number (a bounds error from the second field on),
 * the 3D one reads Fp[j][i, ...] with `i` undefined in that scope (its slot
 * variable is `ip`). These sums are what both spell out: a separate
 * accumulator per field, starting at zero.
 */
void jpo_particle2grid_n(const jpo_grid* g, double* const* F, const double* const* Fp, int nf,
                         const double* const coords[3], const uint8_t* index)
{
    const int N = g->ndim;
    const int64_t nc = g->ncells;
    const int M = g->max_xcell;
    const int64_t V0 = g->n[0] + 1, V1 = g->n[1] + 1, V2 = N == 3 ? g->n[2] + 1 : 1;
    const int64_t nv = V0 * V1 * V2;
#pragma omp parallel for schedule(static) num_threads(nthreads())
    for (int64_t v = 0; v < nv; ++v) {
        const int64_t i = v % V0, j = (v / V0) % V1, k = v / (V0 * V1);
        const double xq = g->xv[0][i], yq = g->xv[1][j], zq = N == 3 ? g->xv[2][k] : 0.0;
        double w = 0.0, wF[JPO_MAX_FIELDS];
        for (int f = 0; f < nf; ++f) wF[f] = 0.0;
        const int kmin = N == 3 ? -1 : 0;
        for (int ko = kmin; ko <= 0; ++ko) {
            const int64_t kc = k + ko;
            if (N == 3 && !(0 <= kc && kc < g->n[2])) continue;
            for (int jo = -1; jo <= 0; ++jo) {
                const int64_t jc = j + jo;
                if (!(0 <= jc && jc < g->n[1])) continue;
                for (int io = -1; io <= 0; ++io) {
                    const int64_t ic = i + io;
                    if (!(0 <= ic && ic < g->n[0])) continue;
                    const int64_t c = ic + g->n[0] * (jc + g->n[1] * (N == 3 ? kc : 0));
                    for (int s = 0; s < M; ++s) {
                        const int64_t a = c + nc * s;
                        if (!index[a]) continue;
                        double ss;
                        const double ddx = xq - coords[0][a];
                        const double ddy = yq - coords[1][a];
                        if (N == 2) {
                            ss = ddx * ddx + ddy * ddy;
                        } else {
                            const double ddz = zq - coords[2][a];
                            ss = (ddx * ddx + ddy * ddy) + ddz * ddz;
                        }
                        const double dist = sqrt(ss);
                        const double wi = 1.0 / (dist * dist);
                        w += wi;
                        for (int f = 0; f < nf; ++f) wF[f] = fma(wi, Fp[f][a], wF[f]);
                    }
                }
            }
        }
        const double iw = 1.0 / w;
        for (int f = 0; f < nf; ++f) F[f][v] = wF[f] * iw;
    }
}

/*
 * grid2particle! with a tuple of fields (src/Interpolations/grid_to_particle.jl:
 * 84-103, through _grid2particle at :235-250): a live particle with a NaN
 * coordinate is skipped (any(isnan, pᵢ)); every other one gets, for each field,
 * the N-linear interpolation of that field's cell corners at
 * t = (p - x_corner) * inv(di).
 */
void jpo_grid2particle_n(const jpo_grid* g, double* const* Fp, const double* const* F, int nf,
                         const double* const coords[3], const uint8_t* index)
{
    const int N = g->ndim;
    const int64_t nc = g->ncells;
    const int M = g->max_xcell;
    const int64_t V0 = g->n[0] + 1, V1 = g->n[1] + 1;
#pragma omp parallel for schedule(static) num_threads(nthreads())
    for (int64_t c = 0; c < nc; ++c) {
        int64_t I[3];
        cell_coords(g, c, I);
        double x0[3], dx[3];
        for (int d = 0; d < N; ++d) {
            x0[d] = g->xv[d][I[d]];
            dx[d] = g->dxv[d][I[d]];
        }
        const int64_t b = I[0] + V0 * (I[1] + (N == 3 ? V1 * I[2] : 0));
        const int64_t sz = V0 * V1;
        for (int s = 0; s < M; ++s) {
            const int64_t a = c + nc * s;
            if (!index[a]) continue;
            int nan = 0;
            for (int d = 0; d < N; ++d) nan |= isnan(coords[d][a]);
            if (nan) continue;
            double t[3];
            for (int d = 0; d < N; ++d) t[d] = (coords[d][a] - x0[d]) * (1.0 / dx[d]);
            for (int f = 0; f < nf; ++f) {
                const double* Ff = F[f];
                double v[8];
                v[0] = Ff[b];
                v[1] = Ff[b + 1];
                v[2] = Ff[b + V0];
                v[3] = Ff[b + V0 + 1];
                if (N == 3) {
                    v[4] = Ff[b + sz];
                    v[5] = Ff[b + sz + 1];
                    v[6] = Ff[b + sz + V0];
                    v[7] = Ff[b + sz + V0 + 1];
                }
                Fp[f][a] = lerpN(N, v, t);
            }
        }
    }
}

double jpo_rand(uint64_t seed, uint32_t stream, uint32_t call, uint64_t cell, uint32_t slot,
                uint32_t dim)
{
    return jp_rand_uniform(seed, stream, call, cell, slot, dim);
}

void jpo_philox(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4])
{
    jp_philox4x32_10(ctr, key, out);
}
