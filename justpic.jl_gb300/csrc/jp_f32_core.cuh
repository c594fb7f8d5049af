// jp_f32_core.cuh -- types and device helpers of the split-precision form
// (FP32 cell offsets) shared by its forward kernels (jp_f32.cu) and its
// adjoint (jp_adjoint.cu).
#pragma once

#include <math_constants.h>

#include <cmath>

#include "jp_internal.cuh"

namespace jp {

struct XiF {
    float* x[3];
};
struct CXiF {
    const float* x[3];
};
struct ArgsF {
    float* a[JP_MAX_ARGS];
    int n;
};
struct CVelF {
    const float* v[3];
};

// per-call constants of the FP32 form
struct F32Params {
    float dx[3];   // spacing per axis
    float w[3];    // dt / dx per axis (time step in cell units per unit velocity)
    float aw[3];   // alpha * dt / dx
    float ca, cb;  // RK2 blend for alpha != 1/2
    int half;
    int cells;     // spacing varies: per-cell tables (ax) and per-cell steps (dt, adt times 1/dx[i])
    double dt, adt;
    F32Axes ax;
};

__device__ __forceinline__ float lerpf1(float t, float v0, float v1) { return fmaf(t, v1, fmaf(-t, v0, v0)); }

template <int DIM>
__device__ __forceinline__ float lerpNf(const float* v, const float* t)
{
    if (DIM == 2) return lerpf1(t[1], lerpf1(t[0], v[0], v[1]), lerpf1(t[0], v[2], v[3]));
    return lerpf1(t[2], lerpf1(t[1], lerpf1(t[0], v[0], v[1]), lerpf1(t[0], v[2], v[3])),
                  lerpf1(t[1], lerpf1(t[0], v[4], v[5]), lerpf1(t[0], v[6], v[7])));
}

// Velocity component `comp` at cell I + offset xi.
template <int DIM>
__device__ __forceinline__ float velocity_f32(const DevGrid& g, int comp, const int* I, const float* xi,
                                              const float* __restrict__ V)
{
    int k[3];
    float t[3];
#pragma unroll
    for (int d = 0; d < DIM; ++d) {
        const float y = (d == comp) ? xi[d] : xi[d] + 0.5f;
        if (!(fabsf(y) < 1e6f)) return CUDART_INF_F;  // NaN, Inf or far outside
        const float fl = floorf(y);
        int kk = I[d] + (int)fl;
        float tt = y - fl;
        const int L = (int)g.nvel[comp][d];
        if (kk == L - 1 && tt == 0.0f) {  // exactly on the last node
            kk = L - 2;
            tt = 1.0f;
        }
        if (kk < 0 || kk > L - 2) return CUDART_INF_F;  // outside the grid's limits
        k[d] = kk;
        t[d] = tt;
    }
    const int64_t L0 = g.nvel[comp][0];
    float v[8];
    if (DIM == 2) {
        const float* b = V + k[0] + L0 * k[1];
        v[0] = __ldg(b);
        v[1] = __ldg(b + 1);
        v[2] = __ldg(b + L0);
        v[3] = __ldg(b + L0 + 1);
    } else {
        const int64_t L1 = g.nvel[comp][1];
        const int64_t sz = L0 * L1;
        const float* b = V + k[0] + L0 * (k[1] + L1 * (int64_t)k[2]);
        v[0] = __ldg(b);
        v[1] = __ldg(b + 1);
        v[2] = __ldg(b + L0);
        v[3] = __ldg(b + L0 + 1);
        v[4] = __ldg(b + sz);
        v[5] = __ldg(b + sz + 1);
        v[6] = __ldg(b + sz + L0);
        v[7] = __ldg(b + sz + L0 + 1);
    }
    return lerpNf<DIM>(v, t);
}

// The same samples on a grid whose spacing varies (per-cell tables): every
// component of the velocity at offset xi of cell I (xi in cell I's units, any
// value). Per axis the point is first carried into the cell that holds it (a
// walk of at most kWalkCells cells, never past the first or last cell), then
// component c takes, along its own axis, the vertex interval of that cell and,
// along the others, the interval of the centred nodes around the point: the
// cell's centre sits at offset 1/2, its neighbours' centres (or the ghost
// nodes at the ends) at the spacings of tables cl / cr. Outside a grid's
// limits (or for a point farther than the walk) the sample is Inf.
constexpr int kWalkCells = 8;

template <int DIM>
__device__ __forceinline__ void velocity_f32_cells(const DevGrid& g, const F32Axes& ax, const int* I,
                                                   const float* xi, const CVelF& V, float* out)
{
    int k[3];
    float u[3];
#pragma unroll
    for (int d = 0; d < DIM; ++d) {
        int kk = I[d];
        float uu = xi[d];
        const int n = (int)g.n[d];
        for (int it = 0; it < kWalkCells; ++it) {
            if (uu >= 1.0f && kk < n - 1) {
                uu = (uu - 1.0f) * __ldg(ax.tor[d] + kk);
                ++kk;
            } else if (uu < 0.0f && kk > 0) {
                uu = fmaf(uu, __ldg(ax.tol[d] + kk), 1.0f);
                --kk;
            } else {
                break;
            }
        }
        if ((uu >= 1.0f && kk < n - 1) || (uu < 0.0f && kk > 0)) uu = CUDART_NAN_F;  // farther than the walk
        k[d] = kk;
        u[d] = uu;
    }
#pragma unroll
    for (int c = 0; c < DIM; ++c) {
        int kn[3];
        float t[3];
        bool ok = true;
#pragma unroll
        for (int d = 0; d < DIM; ++d) {
            if (d == c) {  // vertex nodes: interval k, t = u
                kn[d] = k[d];
                t[d] = u[d];
            } else if (u[d] >= 0.5f) {  // centred nodes k+1 (the centre) and k+2
                kn[d] = k[d] + 1;
                t[d] = (u[d] - 0.5f) * __ldg(ax.cr[d] + k[d]);
            } else {  // centred nodes k and k+1 (the centre)
                kn[d] = k[d];
                t[d] = fmaf(u[d] - 0.5f, __ldg(ax.cl[d] + k[d]), 1.0f);
            }
            ok &= t[d] >= 0.0f && t[d] <= 1.0f;  // false for NaN
        }
        if (!ok) {
            out[c] = CUDART_INF_F;
            continue;
        }
        const float* Vc = V.v[c];
        const int64_t L0 = g.nvel[c][0];
        float v[8];
        if (DIM == 2) {
            const float* b = Vc + kn[0] + L0 * kn[1];
            v[0] = __ldg(b);
            v[1] = __ldg(b + 1);
            v[2] = __ldg(b + L0);
            v[3] = __ldg(b + L0 + 1);
        } else {
            const int64_t L1 = g.nvel[c][1];
            const int64_t sz = L0 * L1;
            const float* b = Vc + kn[0] + L0 * (kn[1] + L1 * (int64_t)kn[2]);
            v[0] = __ldg(b);
            v[1] = __ldg(b + 1);
            v[2] = __ldg(b + L0);
            v[3] = __ldg(b + L0 + 1);
            v[4] = __ldg(b + sz);
            v[5] = __ldg(b + sz + 1);
            v[6] = __ldg(b + sz + L0);
            v[7] = __ldg(b + sz + L0 + 1);
        }
        out[c] = lerpNf<DIM>(v, t);
    }
}

inline F32Params make_params(const jp_particles* P, double alpha, double dt)
{
    F32Params p{};
    for (int d = 0; d < 3; ++d) {
        const double dx = P->dx_host[d];
        p.dx[d] = (float)dx;
        p.w[d] = (float)(dt / dx);
        p.aw[d] = (float)(alpha * dt / dx);
    }
    const double ia = 1.0 / alpha;
    p.ca = (float)std::fma(-0.5, ia, 1.0);
    p.cb = (float)(0.5 * ia);
    p.half = alpha == 0.5;
    p.cells = P->f32_cells;
    p.dt = dt;
    p.adt = alpha * dt;
    p.ax = P->f32ax;
    return p;
}

// particle2grid! weight of the split form, 1 / distance^2 in FP32: the
// special-function unit's reciprocal (rcp.approx.f32, one instruction instead
// of the correctly rounded sequence; deterministic, its error of the order of
// the FP32 distance's own rounding). The forward sums and the adjoint use it
// alike.
__device__ __forceinline__ float p2g_weight_f32(float ss)
{
    float r;
    asm("rcp.approx.f32 %0, %1;" : "=f"(r) : "f"(ss));
    return r;
}

}  // namespace jp
