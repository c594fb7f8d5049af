/*
 * jp_oracle_jvp.c -- forward-mode (dual-number) derivatives through the CPU
 * oracle: advection! and particle2grid! carried out on (value, tangent)
 * pairs.
 *
 * TEST INFRASTRUCTURE ONLY: it checks the hand-written adjoint of the CUDA
 * library (a vector-Jacobian product must equal the Jacobian-vector product in
 * every direction). The value parts repeat the operations of jp_oracle.c in
 * the same order, so they are bit-identical to the oracle's results and every
 * discrete choice (cell, slot, Inf outside the grid) is the oracle's; the
 * tangent parts are the exact first-order derivatives of those operations
 * (dual-number arithmetic). move_particles! and inject_particles! need no
 * derivative code: tangents travel with the particles as extra particle
 * fields.
 */
#include "jp_oracle.h"

#include <math.h>

typedef struct {
    double v, d;
} dual;

static inline dual dconst(double x) { return (dual){x, 0.0}; }
static inline dual dadd(dual a, dual b) { return (dual){a.v + b.v, a.d + b.d}; }
static inline dual dsub(dual a, dual b) { return (dual){a.v - b.v, a.d - b.d}; }
static inline dual dmul(dual a, dual b) { return (dual){a.v * b.v, a.d * b.v + a.v * b.d}; }
static inline dual dscale(double s, dual a) { return (dual){s * a.v, s * a.d}; }
static inline dual ddivc(dual a, double s) { return (dual){a.v / s, a.d / s}; }
static inline dual dfma(dual a, dual b, dual c) { return (dual){fma(a.v, b.v, c.v), a.d * b.v + a.v * b.d + c.d}; }
static inline dual dneg(dual a) { return (dual){-a.v, -a.d}; }

/* lerp(t, v0, v1) = muladd(t, v1, muladd(-t, v0, v0)) (src/Interpolations/ndlerp.jl:15) */
static inline dual dlerp1(dual t, dual v0, dual v1) { return dfma(t, v1, dfma(dneg(t), v0, v0)); }

static dual dlerpN(int n, const dual* v, const dual* t)
{
    if (n == 2) return dlerp1(t[1], dlerp1(t[0], v[0], v[1]), dlerp1(t[0], v[2], v[3]));
    return dlerp1(t[2], dlerp1(t[1], dlerp1(t[0], v[0], v[1]), dlerp1(t[0], v[2], v[3])),
                  dlerp1(t[1], dlerp1(t[0], v[4], v[5]), dlerp1(t[0], v[6], v[7])));
}

/* interp_component of jp_oracle.c on duals (src/Particles/Advection/advection.jl:93-148) */
static dual dinterp_component(const jpo_grid* g, int comp, const dual* p, const int64_t* I, const double* V,
                              const double* dV, int* err)
{
    const int N = g->ndim;
    for (int d = 0; d < N; ++d) {
        const double* x = g->xvel[comp][d];
        const int64_t L = g->nvel[comp][d];
        if (!(x[0] <= p[d].v && p[d].v <= x[L - 1])) return (dual){INFINITY, 0.0};
    }
    int64_t idx[3] = {0, 0, 0};
    dual t[3];
    for (int d = 0; d < N; ++d) {
        const double* x = g->xvel[comp][d];
        idx[d] = jpo_bisection(p[d].v, x, g->nvel[comp][d], I[d], err);
        const double xc = x[idx[d]];
        const double dx = g->dxvel[comp][d][idx[d]];
        t[d] = dmul(dsub(p[d], dconst(xc)), dconst(1.0 / dx));
    }
    const int64_t L0 = g->nvel[comp][0], L1 = g->nvel[comp][1];
    dual v[8];
    int64_t off[8];
    const int64_t b = N == 2 ? idx[0] + L0 * idx[1] : idx[0] + L0 * (idx[1] + L1 * idx[2]);
    const int64_t sz = L0 * L1;
    off[0] = b;
    off[1] = b + 1;
    off[2] = b + L0;
    off[3] = b + L0 + 1;
    off[4] = b + sz;
    off[5] = b + sz + 1;
    off[6] = b + sz + L0;
    off[7] = b + sz + L0 + 1;
    for (int k = 0; k < (1 << N); ++k) v[k] = (dual){V[off[k]], dV ? dV[off[k]] : 0.0};
    return dlerpN(N, v, t);
}

static void dinterp_velocity(const jpo_grid* g, const dual* p, const int64_t* I, const double* const V[3],
                             const double* const dV[3], dual* v, int* err)
{
    for (int c = 0; c < g->ndim; ++c) v[c] = dinterp_component(g, c, p, I, V[c], dV ? dV[c] : 0, err);
}

/* advect_particle of jp_oracle.c on duals (src/Particles/Advection/advection.jl:154-179,
   :261-279, :348-367; src/Advection/RK2.jl) */
static void dadvect_particle(const jpo_grid* g, int method, double alpha, const double* const V[3],
                             const double* const dV[3], double dt, const int64_t* I, const dual* p0, dual* pout,
                             int* err)
{
    const int N = g->ndim;
    if (method == JPO_RK2) {
        dual v0[3], v1[3], p1[3];
        dinterp_velocity(g, p0, I, V, dV, v0, err);
        for (int d = 0; d < N; ++d) p1[d] = dfma(dconst(1.0), dscale(alpha * dt, v0[d]), p0[d]);
        dinterp_velocity(g, p1, I, V, dV, v1, err);
        if (alpha == 0.5) {
            for (int d = 0; d < N; ++d) pout[d] = dfma(dconst(1.0), dscale(dt, v1[d]), p0[d]);
        } else {
            const double ia = 1.0 / alpha;
            const double a = fma(-0.5, ia, 1.0);
            const double b = 0.5 * ia;
            for (int d = 0; d < N; ++d) {
                const dual x = dfma(dconst(a), v0[d], dscale(b, v1[d]));
                pout[d] = dfma(dconst(1.0), dscale(dt, x), p0[d]);
            }
        }
    } else if (method == JPO_RK4) {
        dual k1[3], k2[3], k3[3], k4[3], q[3];
        dinterp_velocity(g, p0, I, V, dV, k1, err);
        for (int d = 0; d < N; ++d) q[d] = dadd(p0[d], ddivc(dscale(dt, k1[d]), 2.0));
        dinterp_velocity(g, q, I, V, dV, k2, err);
        for (int d = 0; d < N; ++d) q[d] = dadd(p0[d], ddivc(dscale(dt, k2[d]), 2.0));
        dinterp_velocity(g, q, I, V, dV, k3, err);
        for (int d = 0; d < N; ++d) q[d] = dadd(p0[d], dscale(dt, k3[d]));
        dinterp_velocity(g, q, I, V, dV, k4, err);
        for (int d = 0; d < N; ++d) {
            const dual s = dadd(dadd(dadd(k1[d], dscale(2.0, k2[d])), dscale(2.0, k3[d])), k4[d]);
            pout[d] = dadd(p0[d], ddivc(dscale(dt, s), 6.0));
        }
    } else {
        dual v0[3];
        dinterp_velocity(g, p0, I, V, dV, v0, err);
        for (int d = 0; d < N; ++d) pout[d] = dfma(dconst(1.0), dscale(dt, v0[d]), p0[d]);
    }
}

int jpo_advection_jvp(const jpo_grid* g, int method, double alpha, const double* const V[3],
                      const double* const dV[3], double dt, double* const coords[3], double* const dcoords[3],
                      const uint8_t* index)
{
    const int N = g->ndim;
    const int64_t nc = g->ncells;
    const int M = g->max_xcell;
    int err = 0;
#pragma omp parallel for schedule(static) reduction(| : err)
    for (int64_t c = 0; c < nc; ++c) {
        int64_t I[3];
        I[0] = c % g->n[0];
        I[1] = (c / g->n[0]) % g->n[1];
        I[2] = N == 3 ? c / (g->n[0] * g->n[1]) : 0;
        for (int s = 0; s < M; ++s) {
            const int64_t a = c + nc * s;
            if (!index[a]) continue;
            dual p0[3], p[3];
            for (int d = 0; d < N; ++d) p0[d] = (dual){coords[d][a], dcoords[d][a]};
            dadvect_particle(g, method, alpha, V, dV, dt, I, p0, p, &err);
            for (int d = 0; d < N; ++d) {
                coords[d][a] = p[d].v;
                dcoords[d][a] = isfinite(p[d].v) ? p[d].d : 0.0;  /* a particle sent to Inf is dropped */
            }
        }
    }
    return err;
}

/* jpo_particle2grid on duals (src/Interpolations/particle_to_grid.jl:37-68, :113-151) */
void jpo_particle2grid_jvp(const jpo_grid* g, double* F, double* dF, const double* Fp, const double* dFp,
                           const double* const coords[3], const double* const dcoords[3], const uint8_t* index)
{
    const int N = g->ndim;
    const int64_t nc = g->ncells;
    const int M = g->max_xcell;
    const int64_t V0 = g->n[0] + 1, V1 = g->n[1] + 1, V2 = N == 3 ? g->n[2] + 1 : 1;
    const int64_t nv = V0 * V1 * V2;
#pragma omp parallel for schedule(static)
    for (int64_t v = 0; v < nv; ++v) {
        const int64_t i = v % V0, j = (v / V0) % V1, k = v / (V0 * V1);
        const double xq = g->xv[0][i], yq = g->xv[1][j], zq = N == 3 ? g->xv[2][k] : 0.0;
        dual w = dconst(0.0), wF = dconst(0.0);
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
                        const dual ddx = dsub(dconst(xq), (dual){coords[0][a], dcoords[0][a]});
                        const dual ddy = dsub(dconst(yq), (dual){coords[1][a], dcoords[1][a]});
                        dual ss;
                        if (N == 2) {
                            ss = dadd(dmul(ddx, ddx), dmul(ddy, ddy));
                        } else {
                            const dual ddz = dsub(dconst(zq), (dual){coords[2][a], dcoords[2][a]});
                            ss = dadd(dadd(dmul(ddx, ddx), dmul(ddy, ddy)), dmul(ddz, ddz));
                        }
                        const double dist = sqrt(ss.v);
                        const dual ddist = {dist, ss.d / (2.0 * dist)};
                        const dual d2 = dmul(ddist, ddist);
                        const double wiv = 1.0 / d2.v;
                        const dual wi = {wiv, -d2.d * wiv * wiv};
                        w = dadd(w, wi);
                        wF = dfma(wi, (dual){Fp[a], dFp ? dFp[a] : 0.0}, wF);
                    }
                }
            }
        }
        dual f;
        if (N == 2) {
            f.v = wF.v / w.v;
            f.d = (wF.d - f.v * w.d) / w.v;
        } else {
            const double iw = 1.0 / w.v;
            f.v = wF.v * iw;
            f.d = (wF.d - f.v * w.d) * iw;
        }
        F[v] = f.v;
        dF[v] = f.d;
    }
}
