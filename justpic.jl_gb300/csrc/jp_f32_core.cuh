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
    int uniform;   // one spacing per axis: dx, w and aw above hold for every cell
    F32Axes ax;    // per-cell tables (any grid)
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
    p.uniform = P->g.uniform;
    p.ax = P->f32ax;
    return p;
}

}  // namespace jp
