// jp_particles.cu -- per-cell kernels: particle seeding, advection!,
// grid2particle! and particle2grid!.
//
// Layout: one thread per cell (or per vertex column for particle2grid!), a warp
// covers 32 consecutive cells along x, so every per-slot load and store of the
// blocklength-0 CellArray (element c + ncells*s) is one coalesced 256-byte
// (FP64) or 32-byte (index) transaction per warp.
#include <math_constants.h>

#include <cmath>

#include "jp_internal.cuh"
#include "jp_weight.cuh"

namespace jp {

struct CVel {
    const double* v[3];
};

// ------------------------------------------------------------- seeding
// fill_coords_index!: src/Particles/particles_utils.jl:168-194
template <int DIM>
__global__ void __launch_bounds__(kThreads) init_kernel(DevGrid g, Coords X, uint8_t* __restrict__ index)
{
    const int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= g.ncells) return;
    int64_t I[3];
    cell_coords(g, c, I);
    const int64_t nc = g.ncells;
    double x0[3], dx[3];
#pragma unroll
    for (int d = 0; d < DIM; ++d) {
        x0[d] = ldg(g.xv[d] + I[d]);
        dx[d] = ldg(g.dxv[d] + I[d]);
    }
    int l = 0;
    for (int iq = 0; iq < (1 << DIM); ++iq) {
        double xc[3];
#pragma unroll
        for (int d = 0; d < DIM; ++d) xc[d] = x0[d] + (dx[d] * (double)((iq >> d) & 1)) / 2.0;
        for (int q = 0; q < g.np_quadrant; ++q, ++l) {
#pragma unroll
            for (int d = 0; d < DIM; ++d) {
                const double r = jp_rand_uniform(g.seed, JP_RNG_STREAM_INIT, 0u, (uint64_t)c, (uint32_t)l,
                                                 (uint32_t)d);
                X.c[d][c + nc * l] = xc[d] + (dx[d] / 2.0) * r;
            }
            index[c + nc * l] = 1;
        }
    }
    for (; l < g.max_xcell; ++l) {
#pragma unroll
        for (int d = 0; d < DIM; ++d) X.c[d][c + nc * l] = CUDART_NAN;
        index[c + nc * l] = 0;
    }
}

// ----------------------------------------------------------- advection
// interp_velocity2particle for component `comp`
// (src/Particles/Advection/advection.jl:93-148, src/Advection/advection.jl:3-47).
// A point inside the seed interval [x[I], x[I+1]] is inside the grid's limits
// too, so the limits test (check_local_limits) only runs when that first
// bisection test fails; the result is the same for every input. The seed test
// itself compares integer keys (exact, see okey) and falls back to the FP64
// comparisons of the reference whenever it does not accept.
struct AdvParams {
    double adt;  // alpha * dt (first stage)
    double dt;
    double ca;   // RK2 with alpha != 1/2: 1 - 1/(2 alpha) and 1/(2 alpha)
    double cb;
    int half;    // alpha == 1/2
};

// Velocity interpolation of the advection call: N-linear (advection!), LinP
// (advection_LinP!) or MQS (advection_MQS!).
constexpr int kInterpLinear = 0;
constexpr int kInterpLinP = 1;
constexpr int kInterpMQS = 2;

// F(i, j[, k]) of a component grid, indices clamped to the grid
template <int DIM>
__device__ __forceinline__ double vel_at(const DevGrid& g, int comp, const double* __restrict__ V, int64_t i,
                                         int64_t j, int64_t k)
{
    const int64_t L0 = g.nvel[comp][0], L1 = g.nvel[comp][1], L2 = DIM == 3 ? g.nvel[comp][2] : 1;
    i = i < 0 ? 0 : (i > L0 - 1 ? L0 - 1 : i);
    j = j < 0 ? 0 : (j > L1 - 1 ? L1 - 1 : j);
    k = k < 0 ? 0 : (k > L2 - 1 ? L2 - 1 : k);
    return ldg(V + i + L0 * (j + L1 * k));
}

// LinP (src/Particles/Advection/advection_LinP.jl:112-391) away from the
// grid's edges: 2/3 of the N-linear value VL plus 1/3 of the N-linear
// interpolation of the velocities averaged to the pressure points
// (interpolate_V_to_P, its augment_offset rows and swap_F order included),
// each product and sum rounded on its own as the reference writes it.
template <int DIM>
__device__ double linp_value(const DevGrid& g, int comp, const double* __restrict__ V, const double* p,
                             const int64_t* idx, const double* xc, const double* dx, double VL)
{
    int64_t b[3] = {idx[0], idx[1], DIM == 3 ? idx[2] : 0};
    b[comp] += p[comp] > xc[comp] + dx[comp] / 2.0 ? 1 : 0;  // offset_LinP
    const int r2 = comp == 1 ? 0 : 1;  // row 2 shifts x (y-component) or y
    const int r3 = comp == 2 ? 0 : 2;  // row 3 shifts x (z-component) or z
    constexpr int NR = DIM == 3 ? 4 : 2;
    double av[8];
#pragma unroll
    for (int r = 0; r < NR; ++r) {
        int64_t q[3] = {b[0], b[1], b[2]};
        if (r == 1 || r == 3) q[r2] += 1;
        if (r >= 2) q[r3] += 1;
        double f[3];
#pragma unroll
        for (int s = 0; s < 3; ++s) {
            int64_t e[3] = {q[0], q[1], q[2]};
            e[comp] += s - 1;
            f[s] = vel_at<DIM>(g, comp, V, e[0], e[1], e[2]);
        }
        av[2 * r] = (f[0] + f[1]) / 2.0;
        av[2 * r + 1] = (f[2] + f[1]) / 2.0;
    }
    double FP[8];
    if (comp == 0) {
#pragma unroll
        for (int k = 0; k < 2 * NR; ++k) FP[k] = av[k];
    } else {  // swap_F: (1, 3, 2, 4, 5, 7, 6, 8)
#pragma unroll
        for (int k = 0; k < 2 * NR; ++k) FP[k] = av[(k & 4) | ((k & 1) << 1) | ((k & 2) >> 1)];
    }
    // correct_xci_to_pressure_point (advection_LinP.jl:151-189)
    double tP[3];
    const int off = 1 - 2 * (p[comp] < xc[comp] + dx[comp] / 2.0 ? 1 : 0);
#pragma unroll
    for (int d = 0; d < DIM; ++d) {
        const double xP = d == comp ? xc[d] + ((double)off * dx[d]) / 2.0 : xc[d];
        tP[d] = (p[d] - xP) * ldg(g.ixvel[comp][d] + idx[d]);
    }
    const double VP = lerpN<DIM>(FP, tP);
    constexpr double A = 2.0 / 3.0;
    constexpr double B = 1.0 - A;
    return __dadd_rn(__dmul_rn(A, VL), __dmul_rn(B, VP));
}

// lerp of (a, b) at t plus half * (t - half)^2 * (muladd(-2, v1, v0) + v2)
// with the stencil extended below (lo) or above (hi): one edge of MQS
// (src/Interpolations/MQS.jl), each operation rounded on its own.
__device__ __forceinline__ double mqs_edge(double t, double a, double b, double lo, double hi)
{
    const bool below = t < 0.5;
    const double v0 = below ? lo : a, v1 = below ? a : b, v2 = below ? b : hi;
    const double d = __dadd_rn(t, -0.5);
    const double corr = __dmul_rn(__dmul_rn(0.5, __dmul_rn(d, d)), __dadd_rn(fma(-2.0, v1, v0), v2));
    return __dadd_rn(lerp1(t, a, b), corr);
}

// MQS (src/Interpolations/MQS.jl:1-158) away from the grid's edges, v the
// corner values and t the normalised position. In 3D the layer k + 1 (x, y)
// and row j + 1 (z) corrections use the stencil of layer k / row j, as the
// reference does.
template <int DIM>
__device__ double mqs_value(const DevGrid& g, int comp, const double* __restrict__ V, const int64_t* idx,
                            const double* v, const double* t)
{
    const int64_t i = idx[0], j = idx[1], k = DIM == 3 ? idx[2] : 0;
    if (DIM == 2) {
        if (comp == 0) {
            const double r0 = mqs_edge(t[0], v[0], v[1], vel_at<2>(g, 0, V, i - 1, j, 0), vel_at<2>(g, 0, V, i + 2, j, 0));
            const double r1 =
                mqs_edge(t[0], v[2], v[3], vel_at<2>(g, 0, V, i - 1, j + 1, 0), vel_at<2>(g, 0, V, i + 2, j + 1, 0));
            return lerp1(t[1], r0, r1);
        }
        const double r0 = mqs_edge(t[1], v[0], v[2], vel_at<2>(g, 1, V, i, j - 1, 0), vel_at<2>(g, 1, V, i, j + 2, 0));
        const double r1 =
            mqs_edge(t[1], v[1], v[3], vel_at<2>(g, 1, V, i + 1, j - 1, 0), vel_at<2>(g, 1, V, i + 1, j + 2, 0));
        return lerp1(t[0], r0, r1);
    }
    double r[2];
    if (comp == 0) {
        const double lo0 = vel_at<3>(g, 0, V, i - 1, j, k), hi0 = vel_at<3>(g, 0, V, i + 2, j, k);
        const double lo1 = vel_at<3>(g, 0, V, i - 1, j + 1, k), hi1 = vel_at<3>(g, 0, V, i + 2, j + 1, k);
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            const double* w = v + 4 * h;
            r[h] = lerp1(t[1], mqs_edge(t[0], w[0], w[1], lo0, hi0), mqs_edge(t[0], w[2], w[3], lo1, hi1));
        }
        return lerp1(t[2], r[0], r[1]);
    }
    if (comp == 1) {
        const double lo0 = vel_at<3>(g, 1, V, i, j - 1, k), hi0 = vel_at<3>(g, 1, V, i, j + 2, k);
        const double lo1 = vel_at<3>(g, 1, V, i + 1, j - 1, k), hi1 = vel_at<3>(g, 1, V, i + 1, j + 2, k);
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            const double* w = v + 4 * h;
            r[h] = lerp1(t[0], mqs_edge(t[1], w[0], w[2], lo0, hi0), mqs_edge(t[1], w[1], w[3], lo1, hi1));
        }
        return lerp1(t[2], r[0], r[1]);
    }
    // MQS-z: front (v1, v2, v5, v6) and back (v3, v4, v7, v8), corrections along x
    const double lo0 = vel_at<3>(g, 2, V, i - 1, j, k), hi0 = vel_at<3>(g, 2, V, i + 2, j, k);
    const double lo1 = vel_at<3>(g, 2, V, i - 1, j, k + 1), hi1 = vel_at<3>(g, 2, V, i + 2, j, k + 1);
#pragma unroll
    for (int h = 0; h < 2; ++h)
        r[h] = lerp1(t[2], mqs_edge(t[0], v[2 * h], v[2 * h + 1], lo0, hi0),
                     mqs_edge(t[0], v[2 * h + 4], v[2 * h + 5], lo1, hi1));
    return lerp1(t[1], r[0], r[1]);
}

template <int DIM, int INTERP = kInterpLinear>
__device__ __forceinline__ double interp_component(const DevGrid& g, int comp, const double* p,
                                                   const long long* kp, bool pnan, const int* I,
                                                   const double* __restrict__ V, int* errs)
{
    int64_t idx[3];
    double xc[3];
#pragma unroll
    for (int d = 0; d < DIM; ++d) {
        const double* x = g.xvel[comp][d];
        const int J = I[d];
        const double a = ldg(x + J), b = ldg(x + J + 1);
        const long long ka = okey(a), kb = okey(b);
        if (!pnan && ka <= kp[d] && kp[d] <= kb) {  // the reference's first test (closed interval)
            idx[d] = J;
            xc[d] = a;
        } else if (!pnan && kb < kp[d] && J + 2 < g.nvel[comp][d] && kp[d] < okey(ldg(x + J + 2))) {
            // strictly inside the next interval: the only answer the bisection can give
            idx[d] = J + 1;
            xc[d] = b;
        } else if (!pnan && kp[d] < ka && J >= 1 && okey(ldg(x + J - 1)) < kp[d]) {
            idx[d] = J - 1;  // strictly inside the previous interval
            xc[d] = ldg(x + J - 1);
        } else {
#pragma unroll
            for (int e = 0; e < DIM; ++e)
                if (!(g.lim_lo[comp][e] <= p[e] && p[e] <= g.lim_hi[comp][e])) return CUDART_INF;
            idx[d] = find_cell(p[d], x, g.nvel[comp][d], I[d], errs);
            xc[d] = ldg(x + idx[d]);
        }
    }
    double t[3];
#pragma unroll
    for (int d = 0; d < DIM; ++d) t[d] = (p[d] - xc[d]) * ldg(g.ixvel[comp][d] + idx[d]);
    const int64_t L0 = g.nvel[comp][0];
    double v[8];
    if (DIM == 2) {
        const double* b = V + idx[0] + L0 * idx[1];
        v[0] = ldg(b);
        v[1] = ldg(b + 1);
        v[2] = ldg(b + L0);
        v[3] = ldg(b + L0 + 1);
    } else {
        const int64_t L1 = g.nvel[comp][1];
        const int64_t sz = L0 * L1;
        const double* b = V + idx[0] + L0 * (idx[1] + L1 * idx[2]);
        v[0] = ldg(b);
        v[1] = ldg(b + 1);
        v[2] = ldg(b + L0);
        v[3] = ldg(b + L0 + 1);
        v[4] = ldg(b + sz);
        v[5] = ldg(b + sz + 1);
        v[6] = ldg(b + sz + L0);
        v[7] = ldg(b + sz + L0 + 1);
    }
    const double VL = lerpN<DIM>(v, t);
    if (INTERP == kInterpLinear) return VL;
    // away from the edges only: 1 < index < size - 1 (1-based) on every axis
    bool inner = true;
#pragma unroll
    for (int d = 0; d < DIM; ++d) inner &= idx[d] >= 1 && idx[d] <= g.nvel[comp][d] - 3;
    if (!inner) return VL;
    if (INTERP == kInterpLinP) {
        double dx[3];
#pragma unroll
        for (int d = 0; d < DIM; ++d) dx[d] = ldg(g.dxvel[comp][d] + idx[d]);
        return linp_value<DIM>(g, comp, V, p, idx, xc, dx, VL);
    }
    return mqs_value<DIM>(g, comp, V, idx, v, t);
}

template <int DIM, int INTERP = kInterpLinear>
__device__ __forceinline__ void interp_velocity(const DevGrid& g, const CVel& V, const double* p, const int* I,
                                                double* v, int* errs)
{
    long long kp[3];
    bool pnan = false;
#pragma unroll
    for (int d = 0; d < DIM; ++d) {
        kp[d] = okey(p[d]);
        pnan |= is_nan_bits(p[d]);
    }
#pragma unroll
    for (int c = 0; c < DIM; ++c) v[c] = interp_component<DIM, INTERP>(g, c, p, kp, pnan, I, V.v[c], errs);
}

// advect_particle: RK2 src/Particles/Advection/advection.jl:154-179 with
// first/second_stage of src/Advection/RK2.jl (muladd(1, (alpha*dt)*v, p) etc.);
// RK4 :261-279; Euler :348-367.
template <int DIM, int METHOD, int INTERP = kInterpLinear>
__device__ __forceinline__ void advect_particle(const DevGrid& g, const CVel& V, const AdvParams& P,
                                                const int* I, const double* p0, double* p, int* errs)
{
    if (METHOD == JP_RUNGE_KUTTA2) {
        double v0[3], v1[3], p1[3];
        interp_velocity<DIM, INTERP>(g, V, p0, I, v0, errs);
#pragma unroll
        for (int d = 0; d < DIM; ++d) p1[d] = fma(1.0, P.adt * v0[d], p0[d]);
        interp_velocity<DIM, INTERP>(g, V, p1, I, v1, errs);
        if (P.half) {
#pragma unroll
            for (int d = 0; d < DIM; ++d) p[d] = fma(1.0, P.dt * v1[d], p0[d]);
        } else {
#pragma unroll
            for (int d = 0; d < DIM; ++d) p[d] = fma(1.0, P.dt * fma(P.ca, v0[d], P.cb * v1[d]), p0[d]);
        }
    } else if (METHOD == JP_RUNGE_KUTTA4) {
        double k1[3], k2[3], k3[3], k4[3], q[3];
        interp_velocity<DIM, INTERP>(g, V, p0, I, k1, errs);
#pragma unroll
        for (int d = 0; d < DIM; ++d) q[d] = p0[d] + (P.dt * k1[d]) * 0.5;  // x / 2 == x * 0.5 exactly
        interp_velocity<DIM, INTERP>(g, V, q, I, k2, errs);
#pragma unroll
        for (int d = 0; d < DIM; ++d) q[d] = p0[d] + (P.dt * k2[d]) * 0.5;
        interp_velocity<DIM, INTERP>(g, V, q, I, k3, errs);
#pragma unroll
        for (int d = 0; d < DIM; ++d) q[d] = p0[d] + P.dt * k3[d];
        interp_velocity<DIM, INTERP>(g, V, q, I, k4, errs);
#pragma unroll
        for (int d = 0; d < DIM; ++d)
            p[d] = p0[d] + __ddiv_rn(P.dt * (((k1[d] + 2.0 * k2[d]) + 2.0 * k3[d]) + k4[d]), 6.0);
    } else {
        double v0[3];
        interp_velocity<DIM, INTERP>(g, V, p0, I, v0, errs);
#pragma unroll
        for (int d = 0; d < DIM; ++d) p[d] = fma(1.0, P.dt * v0[d], p0[d]);
    }
}

// advection_kernel! (src/Particles/Advection/advection.jl:66-91): one warp per
// 32 consecutive cells, work spread over the warp's live slots.
template <int DIM, int METHOD, int INTERP>
__global__ void __launch_bounds__(32 * kWarpsPerBlock)
    advect_kernel(DevGrid g, CVel V, AdvParams P, Coords X, const uint8_t* __restrict__ index, int* d_err)
{
    __shared__ SlotList lists[kWarpsPerBlock];
    __shared__ int cellI[kWarpsPerBlock][32][3];
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int64_t c0 = ((int64_t)blockIdx.x * kWarpsPerBlock + w) * 32;
    if (c0 >= g.ncells) return;
    const int64_t nc = g.ncells;
    const int M = g.max_xcell;
    {
        int64_t I[3];
        cell_coords(g, min(c0 + lane, nc - 1), I);
#pragma unroll
        for (int d = 0; d < 3; ++d) cellI[w][lane][d] = (int)I[d];
    }
    int errs = 0;
    // slots in chunks of 64 (one chunk unless max_xcell > 64)
    for (int s0 = 0; s0 < M; s0 += 64) {
        const int Mc = min(64, M - s0);
        uint64_t mine;
        const int K = build_slot_list(lists[w], index + nc * s0, c0, nc, Mc, lane, &mine);
        for (int k = lane; k < K; k += 32) {
            int s, l;
            slot_item(lists[w], Mc, k, &s, &l);
            const int64_t a = c0 + l + nc * (s0 + s);
            int I[3] = {cellI[w][l][0], cellI[w][l][1], cellI[w][l][2]};
            double p0[3], p[3];
#pragma unroll
            for (int d = 0; d < DIM; ++d) p0[d] = X.c[d][a];
            advect_particle<DIM, METHOD, INTERP>(g, V, P, I, p0, p, &errs);
#pragma unroll
            for (int d = 0; d < DIM; ++d) X.c[d][a] = p[d];
        }
        __syncwarp();
    }
    raise_err(d_err, errs);
}

// ------------------------------------------------------- grid2particle!
// _grid2particle_classic! (src/Interpolations/grid_to_particle.jl:64-82): the
// corner values, lower-left vertex and inverse spacing of each of the warp's
// cells are staged once, then the warp's live slots are interpolated.
template <int DIM>
__global__ void __launch_bounds__(32 * kWarpsPerBlock)
    g2p_kernel(DevGrid g, double* __restrict__ Fp, const double* __restrict__ F, CCoords X,
               const uint8_t* __restrict__ index)
{
    __shared__ SlotList lists[kWarpsPerBlock];
    __shared__ double cellv[kWarpsPerBlock][32][(1 << DIM) + 2 * DIM];
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int64_t c0 = ((int64_t)blockIdx.x * kWarpsPerBlock + w) * 32;
    if (c0 >= g.ncells) return;
    const int64_t nc = g.ncells;
    const int M = g.max_xcell;
    {
        int64_t I[3];
        cell_coords(g, min(c0 + lane, nc - 1), I);
        const int64_t V0 = g.n[0] + 1, V1 = g.n[1] + 1;
        double* cv = cellv[w][lane];
        const double* b = F + I[0] + V0 * (I[1] + (DIM == 3 ? V1 * I[2] : 0));
        cv[0] = ldg(b);
        cv[1] = ldg(b + 1);
        cv[2] = ldg(b + V0);
        cv[3] = ldg(b + V0 + 1);
        if (DIM == 3) {
            const int64_t sz = V0 * V1;
            cv[4] = ldg(b + sz);
            cv[5] = ldg(b + sz + 1);
            cv[6] = ldg(b + sz + V0);
            cv[7] = ldg(b + sz + V0 + 1);
        }
#pragma unroll
        for (int d = 0; d < DIM; ++d) {
            cv[(1 << DIM) + d] = ldg(g.xv[d] + I[d]);
            cv[(1 << DIM) + DIM + d] = ldg(g.ixv[d] + I[d]);
        }
    }
    for (int s0 = 0; s0 < M; s0 += 64) {  // slots in chunks of 64
        const int Mc = min(64, M - s0);
        uint64_t mine;
        const int K = build_slot_list(lists[w], index + nc * s0, c0, nc, Mc, lane, &mine);
        for (int k = lane; k < K; k += 32) {
            int s, l;
            slot_item(lists[w], Mc, k, &s, &l);
            const int64_t a = c0 + l + nc * (s0 + s);
            const double* cv = cellv[w][l];
            double t[3];
#pragma unroll
            for (int d = 0; d < DIM; ++d) t[d] = (X.c[d][a] - cv[(1 << DIM) + d]) * cv[(1 << DIM) + DIM + d];
            Fp[a] = lerpN<DIM>(cv, t);
        }
        __syncwarp();
    }
}

constexpr int kFieldsPerLaunchG2P = 4;

// grid2particle! with a tuple of fields (src/Interpolations/grid_to_particle.jl:
// 84-103): a live particle with a NaN coordinate is skipped; every other one
// forms its normalised coordinates once and interpolates each field's corner
// values (loaded through the read-only cache: the warp's particles share the
// corners of its 32 cells).
struct G2PFields {
    const double* f[kFieldsPerLaunchG2P];
    double* fp[kFieldsPerLaunchG2P];
};

template <int DIM, int NF>
__global__ void __launch_bounds__(32 * kWarpsPerBlock)
    g2p_n_kernel(DevGrid g, G2PFields GF, CCoords X, const uint8_t* __restrict__ index)
{
    __shared__ SlotList lists[kWarpsPerBlock];
    __shared__ double cellx[kWarpsPerBlock][32][2 * DIM];
    __shared__ int64_t cellb[kWarpsPerBlock][32];
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int64_t c0 = ((int64_t)blockIdx.x * kWarpsPerBlock + w) * 32;
    if (c0 >= g.ncells) return;
    const int64_t nc = g.ncells;
    const int M = g.max_xcell;
    const int64_t V0 = g.n[0] + 1, V1 = g.n[1] + 1, SZ = V0 * V1;
    {
        int64_t I[3];
        cell_coords(g, min(c0 + lane, nc - 1), I);
        cellb[w][lane] = I[0] + V0 * (I[1] + (DIM == 3 ? V1 * I[2] : 0));
#pragma unroll
        for (int d = 0; d < DIM; ++d) {
            cellx[w][lane][d] = ldg(g.xv[d] + I[d]);
            cellx[w][lane][DIM + d] = ldg(g.ixv[d] + I[d]);
        }
    }
    for (int s0 = 0; s0 < M; s0 += 64) {  // slots in chunks of 64
        const int Mc = min(64, M - s0);
        uint64_t mine;
        const int K = build_slot_list(lists[w], index + nc * s0, c0, nc, Mc, lane, &mine);
        for (int k = lane; k < K; k += 32) {
            int s, l;
            slot_item(lists[w], Mc, k, &s, &l);
            const int64_t a = c0 + l + nc * (s0 + s);
            double t[3];
            bool nan = false;
#pragma unroll
            for (int d = 0; d < DIM; ++d) {
                const double x = X.c[d][a];
                nan |= is_nan_bits(x);
                t[d] = (x - cellx[w][l][d]) * cellx[w][l][DIM + d];
            }
            if (nan) continue;  // any(isnan, pᵢ) && continue
            const int64_t b = cellb[w][l];
#pragma unroll
            for (int f = 0; f < NF; ++f) {
                const double* F = GF.f[f];
                double v[8];
                v[0] = ldg(F + b);
                v[1] = ldg(F + b + 1);
                v[2] = ldg(F + b + V0);
                v[3] = ldg(F + b + V0 + 1);
                if (DIM == 3) {
                    v[4] = ldg(F + b + SZ);
                    v[5] = ldg(F + b + SZ + 1);
                    v[6] = ldg(F + b + SZ + V0);
                    v[7] = ldg(F + b + SZ + V0 + 1);
                }
                GF.fp[f][a] = lerpN<DIM>(v, t);
            }
        }
        __syncwarp();
    }
}

// ------------------------------------------------------- particle2grid!
// src/Interpolations/particle_to_grid.jl:37-68 (2D), :113-151 (3D).
// One thread per vertex column marching along the last axis over `chunk`
// vertex rows: the cells of row r are read once and feed both vertex r (its
// upper half of the stencil) and vertex r+1 (its lower half), so every vertex
// accumulates its cells in the reference's order (offsets of the last axis
// outermost, x innermost, slots in order) and the sums are bit-identical. Each
// cell is walked through its 64-bit live mask, so no lane spends FP64 issue
// slots on empty slots; the mask of the left neighbour cell comes from the
// neighbouring lane. The loop trip count is the same for every lane of a warp.
// Fields of a particle2grid! call: one for the scalar form, up to four per
// launch for the tuple form (particle_to_grid.jl:70-109, 153-199).
constexpr int kFieldsPerLaunch = 4;
struct P2GFields {
    const double* fp[kFieldsPerLaunch];
    double* f[kFieldsPerLaunch];
};

template <int DIM, int NF>
__device__ __forceinline__ void p2g_cell(int64_t c, uint64_t mask, int64_t nc, const double* q_cur,
                                         const double* q_nxt, bool do_cur, bool do_nxt, const P2GFields& PF,
                                         const CCoords& X, double& w_c, double* wF_c, double& w_n, double* wF_n)
{
    while (mask) {
        const int s = __ffsll((long long)mask) - 1;
        mask &= mask - 1;
        const int64_t a = c + nc * s;
        double p[3];
#pragma unroll
        for (int d = 0; d < DIM; ++d) p[d] = X.c[d][a];
        double f[NF];
#pragma unroll
        for (int k = 0; k < NF; ++k) f[k] = PF.fp[k][a];
        // the two vertices share the column (x in 2D, x and y in 3D): those terms of
        // distance(xv, p)^2 = ((x - px)^2 + (y - py)^2) [+ (z - pz)^2] are formed once
        const double dx = q_cur[0] - p[0];
        double shared, ec, en;
        if (DIM == 2) {
            shared = dx * dx;
            ec = q_cur[1] - p[1];
            en = q_nxt[1] - p[1];
        } else {
            const double dy = q_cur[1] - p[1];
            shared = dx * dx + dy * dy;
            ec = q_cur[2] - p[2];
            en = q_nxt[2] - p[2];
        }
        if (do_cur) {
            const double wi = inv_dist2(shared + ec * ec);  // inv(distance^2), particle_to_grid.jl:203-205
            w_c += wi;
#pragma unroll
            for (int k = 0; k < NF; ++k) wF_c[k] = fma(wi, f[k], wF_c[k]);
        }
        if (do_nxt) {
            const double wi = inv_dist2(shared + en * en);
            w_n += wi;
#pragma unroll
            for (int k = 0; k < NF; ++k) wF_n[k] = fma(wi, f[k], wF_n[k]);
        }
    }
}

// TUPLE: the tuple form's normalisation, F[k] = wF[k] * inv(w) for every field
// (particle_to_grid.jl:103-108, 193-198); otherwise the scalar form's wF / w in
// 2D (:67) and wF * inv(w) in 3D (:150).
template <int DIM, int NF, bool TUPLE>
__global__ void __launch_bounds__(kThreads)
    p2g_kernel(DevGrid g, P2GFields PF, CCoords X, const uint8_t* __restrict__ index, int chunk, int64_t nthreads,
               double* __restrict__ Wout)
{
    const int64_t V0 = g.n[0] + 1, V1 = g.n[1] + 1;
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int lane = threadIdx.x & 31;
    constexpr int LAST = DIM - 1;
    const int64_t nlast = g.n[LAST];  // cells along the marching axis
    const int64_t cols = DIM == 2 ? V0 : V0 * V1;
    const int64_t nc = g.ncells;
    const int M = g.max_xcell;
    const bool active = t < nthreads;
    const int64_t col = active ? t % cols : 0;
    const int64_t q = active ? t / cols : 0;
    const int64_t r0 = q * chunk;
    const int64_t r1 = active ? min(r0 + (int64_t)chunk, nlast + 1) : r0;
    const int64_t i = col % V0;
    const int64_t j = DIM == 3 ? col / V0 : 0;
    const bool has_i0 = i >= 1, has_i1 = i < g.n[0];          // cells i-1 and i exist
    const bool has_j0 = DIM == 2 || j >= 1, has_j1 = DIM == 2 || j < g.n[1];
    double q_cur[3] = {0.0, 0.0, 0.0}, q_nxt[3] = {0.0, 0.0, 0.0};
    q_cur[0] = q_nxt[0] = ldg(g.xv[0] + i);
    if (DIM == 3) q_cur[1] = q_nxt[1] = ldg(g.xv[1] + j);

    // cell index of (i + di, j + dj, r); valid only where the has_* flags say so
    auto cell = [&](int di, int dj, int64_t r) -> int64_t {
        return DIM == 2 ? (i + di) + g.n[0] * r : (i + di) + g.n[0] * ((j + dj) + g.n[1] * r);
    };
    // accumulate row r into (cur, nxt): cells in reference order
    auto row = [&](int64_t r, bool do_cur, bool do_nxt, double& w_c, double* wF_c, double& w_n, double* wF_n) {
        const bool rok = active && r >= 0 && r < nlast;
        // own cell (i, j, r) and its left neighbour (i-1, j, r) from the lane to the left
        const uint64_t m_own = (rok && has_i1 && has_j1) ? live_mask(index, cell(0, 0, r), nc, M) : 0;
        uint64_t m_left = __shfl_up_sync(0xffffffffu, m_own, 1);
        if (lane == 0 && rok && has_i0 && has_j1) m_left = live_mask(index, cell(-1, 0, r), nc, M);
        if (!(rok && has_i0 && has_j1)) m_left = 0;
        if (DIM == 3) {
            // row j-1 first (joffset = -1), then row j
            const uint64_t mb0 = (rok && has_i0 && has_j0) ? live_mask(index, cell(-1, -1, r), nc, M) : 0;
            const uint64_t mb1 = (rok && has_i1 && has_j0) ? live_mask(index, cell(0, -1, r), nc, M) : 0;
            if (mb0) p2g_cell<DIM, NF>(cell(-1, -1, r), mb0, nc, q_cur, q_nxt, do_cur, do_nxt, PF, X, w_c, wF_c, w_n, wF_n);
            if (mb1) p2g_cell<DIM, NF>(cell(0, -1, r), mb1, nc, q_cur, q_nxt, do_cur, do_nxt, PF, X, w_c, wF_c, w_n, wF_n);
        }
        if (m_left) p2g_cell<DIM, NF>(cell(-1, 0, r), m_left, nc, q_cur, q_nxt, do_cur, do_nxt, PF, X, w_c, wF_c, w_n, wF_n);
        if (m_own) p2g_cell<DIM, NF>(cell(0, 0, r), m_own, nc, q_cur, q_nxt, do_cur, do_nxt, PF, X, w_c, wF_c, w_n, wF_n);
    };

    double w_c = 0.0, w_n = 0.0, wF_c[NF], wF_n[NF];
#pragma unroll
    for (int k = 0; k < NF; ++k) wF_c[k] = wF_n[k] = 0.0;
    // prologue: row r0-1 is the lower half of vertex r0's stencil
    if (active && r0 >= 1) q_nxt[LAST] = ldg(g.xv[LAST] + r0);
    {
        double wd = 0.0, wFd[NF];
#pragma unroll
        for (int k = 0; k < NF; ++k) wFd[k] = 0.0;
        row(r0 - 1, false, true, wd, wFd, w_c, wF_c);
    }
    for (int k = 0; k < chunk; ++k) {
        const int64_t r = r0 + k;
        const bool vok = r < r1;  // vertex row r belongs to this thread
        const bool has_next = r + 1 < r1;
        if (vok) q_cur[LAST] = ldg(g.xv[LAST] + r);
        if (has_next) q_nxt[LAST] = ldg(g.xv[LAST] + r + 1);
        w_n = 0.0;
#pragma unroll
        for (int f = 0; f < NF; ++f) wF_n[f] = 0.0;
        row(vok ? r : -1, vok, has_next, w_c, wF_c, w_n, wF_n);
        if (vok) {
            const int64_t v = DIM == 2 ? i + V0 * r : i + V0 * (j + V1 * r);
            if (TUPLE || DIM == 3) {
                const double iw = __drcp_rn(w_c);
#pragma unroll
                for (int f = 0; f < NF; ++f) PF.f[f][v] = wF_c[f] * iw;
            } else {
                PF.f[0][v] = wF_c[0] / w_c;
            }
            if (Wout) Wout[v] = w_c;  // weight sums, kept for the adjoint
        }
        w_c = w_n;
#pragma unroll
        for (int f = 0; f < NF; ++f) wF_c[f] = wF_n[f];
    }
}

// particle2grid! for cells of more than 64 slots: one thread per vertex, the
// cells of its stencil and their slots in the reference's order (the same sums
// as p2g_kernel, without the per-cell bit masks).
template <int DIM, bool TUPLE>
__global__ void __launch_bounds__(kThreads)
    p2g_wide_kernel(DevGrid g, P2GFields PF, int nf, CCoords X, const uint8_t* __restrict__ index,
                    double* __restrict__ Wout)
{
    const int64_t V0 = g.n[0] + 1, V1 = g.n[1] + 1, V2 = DIM == 3 ? g.n[2] + 1 : 1;
    const int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= V0 * V1 * V2) return;
    const int64_t nc = g.ncells;
    const int64_t i = v % V0, j = (v / V0) % V1, k = v / (V0 * V1);
    double q[3];
    q[0] = ldg(g.xv[0] + i);
    q[1] = ldg(g.xv[1] + j);
    q[2] = DIM == 3 ? ldg(g.xv[2] + k) : 0.0;
    double w = 0.0, wF[kFieldsPerLaunch] = {0.0, 0.0, 0.0, 0.0};
    for (int ko = (DIM == 3 ? -1 : 0); ko <= 0; ++ko) {
        const int64_t kc = k + ko;
        if (DIM == 3 && !(0 <= kc && kc < g.n[2])) continue;
        for (int jo = -1; jo <= 0; ++jo) {
            const int64_t jc = j + jo;
            if (!(0 <= jc && jc < g.n[1])) continue;
            for (int io = -1; io <= 0; ++io) {
                const int64_t ic = i + io;
                if (!(0 <= ic && ic < g.n[0])) continue;
                const int64_t c = ic + g.n[0] * (jc + g.n[1] * (DIM == 3 ? kc : 0));
                for (int s = 0; s < g.max_xcell; ++s) {
                    const int64_t a = c + nc * s;
                    if (!index[a]) continue;
                    const double dx = q[0] - X.c[0][a], dy = q[1] - X.c[1][a];
                    double ss;
                    if (DIM == 2) {
                        ss = dx * dx + dy * dy;
                    } else {
                        const double dz = q[2] - X.c[2][a];
                        ss = (dx * dx + dy * dy) + dz * dz;
                    }
                    const double wi = inv_dist2(ss);
                    w += wi;
#pragma unroll
                    for (int f = 0; f < kFieldsPerLaunch; ++f)
                        if (f < nf) wF[f] = fma(wi, PF.fp[f][a], wF[f]);
                }
            }
        }
    }
    if (TUPLE || DIM == 3) {
        const double iw = __drcp_rn(w);
#pragma unroll
        for (int f = 0; f < kFieldsPerLaunch; ++f)
            if (f < nf) PF.f[f][v] = wF[f] * iw;
    } else {
        PF.f[0][v] = wF[0] / w;
    }
    if (Wout) Wout[v] = w;
}

// ------------------------------------------------ weight self-test
// inv_dist2 against CUDA's sqrt / multiply / reciprocal chain, bit for bit, on
// seeded inputs: the whole normal range, the edges where d^2 or its inverse
// leave it, squares of short doubles and their neighbours, sums of squares of
// cell-sized distances (the inputs particle2grid! sees), and special values.
__device__ __forceinline__ uint64_t mix64(uint64_t x)  // SplitMix64 finaliser
{
    x += 0x9E3779B97F4A7C15ull;
    x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
    x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
    return x ^ (x >> 31);
}

__global__ void weight_selftest_kernel(uint64_t seed, int64_t n, unsigned long long* bad,
                                       unsigned long long* first)
{
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const uint64_t h = mix64(seed ^ mix64((uint64_t)i)), h2 = mix64(h);
        const uint64_t frac = h & ((1ull << 52) - 1);
        double ss;
        switch ((int)(h2 % 6)) {
            case 0:  // any positive normal
                ss = __longlong_as_double((long long)((((h2 >> 8) % 2046 + 1) << 52) | frac));
                break;
            case 1: {  // exponents where d^2 or 1/d^2 approach the ends of the normal range
                const uint64_t e = (h2 >> 8) & 1 ? 1 + (h2 >> 9) % 560 : 1486 + (h2 >> 9) % 561;
                ss = __longlong_as_double((long long)((e << 52) | frac));
                break;
            }
            case 2: {  // squares of short doubles and their neighbours (exact and near-exact roots)
                const double k = (double)((h >> 30) | 1) * __longlong_as_double((long long)(((h2 >> 8) % 1200 + 420) << 52));
                const long long b = __double_as_longlong(__dmul_rn(k, k)) + (long long)((h2 >> 20) % 5) - 2;
                ss = __longlong_as_double(b);
                break;
            }
            case 3: {  // cell-sized distances
                const double x = (double)(h >> 11) * 0x1p-53 * 1e-3, y = (double)(h2 >> 11) * 0x1p-53 * 1e-3;
                ss = __dadd_rn(__dmul_rn(x, x), __dmul_rn(y, y));
                break;
            }
            case 4: {  // significands near 1 and 2 (reciprocal and rounding boundaries)
                const uint64_t f2 = (h2 >> 8) & 1 ? (h & 0xFFFF) : ((1ull << 52) - 1 - (h & 0xFFFF));
                ss = __longlong_as_double((long long)((((h2 >> 9) % 2046 + 1) << 52) | f2));
                break;
            }
            default: {  // zeros, subnormals, infinities, NaN, negatives, powers of two
                const int k = (int)((h2 >> 8) % 7);
                const double sp[7] = {0.0, -0.0, CUDART_INF, CUDART_NAN, -1.5, 0.0, 0.0};
                ss = k < 5 ? sp[k]
                           : (k == 5 ? __longlong_as_double((long long)frac)
                                     : __longlong_as_double((long long)(((h2 >> 9) % 2046 + 1) << 52)));
            }
        }
        const double a = inv_dist2(ss), b = weight_intrinsic(ss);
        const bool same = __double_as_longlong(a) == __double_as_longlong(b) || (isnan(a) && isnan(b));
        if (!same) {
            atomicAdd(bad, 1ull);
            atomicCAS(first, 0ull, (unsigned long long)__double_as_longlong(ss));
        }
    }
}

cudaError_t launch_weight_selftest(uint64_t seed, int64_t n, unsigned long long* d_bad, unsigned long long* d_first,
                                   cudaStream_t st)
{
    weight_selftest_kernel<<<152 * 8, 256, 0, st>>>(seed, n, d_bad, d_first);
    return cudaGetLastError();
}

// ------------------------------------------------------------ launchers
cudaError_t launch_init(jp_particles* P, double* const coords[3], uint8_t* index)
{
    Coords X{{coords[0], coords[1], P->g.ndim == 3 ? coords[2] : nullptr}};
    const unsigned nb = grid_blocks(P->g.ncells);
    if (P->g.ndim == 2)
        init_kernel<2><<<nb, kThreads, 0, P->stream>>>(P->g, X, index);
    else
        init_kernel<3><<<nb, kThreads, 0, P->stream>>>(P->g, X, index);
    return cudaGetLastError();
}

cudaError_t launch_advection(jp_particles* P, int method, double alpha, const double* const V[3], double dt,
                             double* const coords[3], const uint8_t* index)
{
    return launch_advection_interp(P, method, kInterpLinear, alpha, V, dt, coords, index);
}

cudaError_t launch_advection_interp(jp_particles* P, int method, int interp, double alpha, const double* const V[3],
                                    double dt, double* const coords[3], const uint8_t* index)
{
    const bool d3 = P->g.ndim == 3;
    Coords X{{coords[0], coords[1], d3 ? coords[2] : nullptr}};
    CVel Vv{{V[0], V[1], d3 ? V[2] : nullptr}};
    AdvParams ap;
    ap.adt = alpha * dt;
    ap.dt = dt;
    const double ia = 1.0 / alpha;  // second_stage, src/Advection/RK2.jl:38-41
    ap.ca = std::fma(-0.5, ia, 1.0);
    ap.cb = 0.5 * ia;
    ap.half = alpha == 0.5;
    const unsigned nb = grid_blocks(P->g.ncells, 32 * kWarpsPerBlock);
    const int nt = 32 * kWarpsPerBlock;
    cudaStream_t s = P->stream;
#define JP_ADV(D, M, IP) advect_kernel<D, M, IP><<<nb, nt, 0, s>>>(P->g, Vv, ap, X, index, P->d_err)
#define JP_ADV_M(D, IP)                                  \
    do {                                                 \
        if (method == JP_RUNGE_KUTTA2) JP_ADV(D, JP_RUNGE_KUTTA2, IP); \
        else if (method == JP_RUNGE_KUTTA4) JP_ADV(D, JP_RUNGE_KUTTA4, IP); \
        else JP_ADV(D, JP_EULER, IP);                    \
    } while (0)
#define JP_ADV_I(D)                                                  \
    do {                                                             \
        if (interp == kInterpLinP) JP_ADV_M(D, kInterpLinP);         \
        else if (interp == kInterpMQS) JP_ADV_M(D, kInterpMQS);      \
        else JP_ADV_M(D, kInterpLinear);                             \
    } while (0)
    if (!d3)
        JP_ADV_I(2);
    else
        JP_ADV_I(3);
#undef JP_ADV_I
#undef JP_ADV_M
#undef JP_ADV
    return cudaGetLastError();
}

cudaError_t launch_g2p(jp_particles* P, double* Fp, const double* F, const double* const coords[3],
                       const uint8_t* index)
{
    const bool d3 = P->g.ndim == 3;
    CCoords X{{coords[0], coords[1], d3 ? coords[2] : nullptr}};
    const unsigned nb = grid_blocks(P->g.ncells, 32 * kWarpsPerBlock);
    const int nt = 32 * kWarpsPerBlock;
    if (!d3)
        g2p_kernel<2><<<nb, nt, 0, P->stream>>>(P->g, Fp, F, X, index);
    else
        g2p_kernel<3><<<nb, nt, 0, P->stream>>>(P->g, Fp, F, X, index);
    return cudaGetLastError();
}

// particle2grid! of nf fields (nf > 1 or tuple: the tuple form), fields in
// launches of at most four; every launch forms the same weights in the same
// order, so the result does not depend on how the fields are grouped
// Launch shape of p2g_kernel: `chunk` vertex rows per thread along the last
// axis. Each thread also walks the cell row below its first vertex row, so
// short chunks repeat work, and the threads run in waves of what the GPU holds
// at once (SMs x resident blocks of this kernel x block size): a last wave
// filled only in part leaves SMs idle while it runs, and under about one and a
// half waves the SMs run short of warps to hide the loads' latency. The chunk
// is the one (3..16 rows) that minimises (chunk + 1/2) x the number of waves
// among those giving at least 1.5 waves, else 2 (small grids: as many threads
// as possible); on one GB300 this picks 4 rows at 1024^2 and 5 at 128^3, the
// fastest or within 3% of the fastest of a measured sweep over 2..16. Results
// do not depend on it: every vertex sums its cells in the same order whatever
// the chunk.
struct P2GShape {
    int chunk;
    int64_t threads;
    unsigned blocks;
};

template <int DIM, int NF, bool TUPLE>
static P2GShape p2g_shape(int64_t cols, int64_t rows)
{
    static const double resident = [] {  // threads of this kernel the GPU holds at once
        int dev = 0, sms = 0, bps = 0;
        if (cudaGetDevice(&dev) != cudaSuccess ||
            cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess ||
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, p2g_kernel<DIM, NF, TUPLE>, kThreads, 0) !=
                cudaSuccess ||
            sms <= 0 || bps <= 0) {
            cudaGetLastError();
            return 152.0 * 1024.0;
        }
        return (double)sms * bps * kThreads;
    }();
    int chunk = 2;
    double best = 0.0;
    for (int c = 3; c <= 16; ++c) {
        const double waves = (double)(cols * ((rows + c - 1) / c)) / resident;
        if (waves < 1.5) continue;
        const double cost = (c + 0.5) * std::ceil(waves);
        if (chunk == 2 || cost < best) {
            chunk = c;
            best = cost;
        }
    }
    const int64_t threads = cols * ((rows + chunk - 1) / chunk);
    return P2GShape{chunk, threads, grid_blocks(threads)};
}

static cudaError_t p2g_launch(jp_particles* P, double* const* F, const double* const* Fp, int nf, bool tuple,
                              const double* const coords[3], const uint8_t* index, double* W)
{
    const bool d3 = P->g.ndim == 3;
    CCoords X{{coords[0], coords[1], d3 ? coords[2] : nullptr}};
    const int64_t V0 = P->g.n[0] + 1, V1 = P->g.n[1] + 1;
    const int64_t cols = d3 ? V0 * V1 : V0;
    const int64_t rows = P->g.n[d3 ? 2 : 1] + 1;
    const unsigned nbw = grid_blocks(V0 * V1 * (d3 ? P->g.n[2] + 1 : 1));
    for (int f0 = 0; f0 < nf; f0 += kFieldsPerLaunch) {
        const int n = nf - f0 < kFieldsPerLaunch ? nf - f0 : kFieldsPerLaunch;
        P2GFields PF{};
        for (int k = 0; k < n; ++k) {
            PF.fp[k] = Fp[f0 + k];
            PF.f[k] = F[f0 + k];
        }
        double* Wk = f0 == 0 ? W : nullptr;
        cudaStream_t st = P->stream;
        if (P->g.max_xcell > 64) {
            if (!d3)
                tuple ? p2g_wide_kernel<2, true><<<nbw, kThreads, 0, st>>>(P->g, PF, n, X, index, Wk)
                      : p2g_wide_kernel<2, false><<<nbw, kThreads, 0, st>>>(P->g, PF, n, X, index, Wk);
            else
                p2g_wide_kernel<3, true><<<nbw, kThreads, 0, st>>>(P->g, PF, n, X, index, Wk);
            continue;
        }
#define JP_P2G(D, NF, T)                                                                                    \
    do {                                                                                                    \
        const P2GShape sh = p2g_shape<D, NF, T>(cols, rows);                                                \
        p2g_kernel<D, NF, T><<<sh.blocks, kThreads, 0, st>>>(P->g, PF, X, index, sh.chunk, sh.threads, Wk); \
    } while (0)
        if (!d3) {
            if (!tuple) JP_P2G(2, 1, false);
            else if (n == 1) JP_P2G(2, 1, true);
            else if (n == 2) JP_P2G(2, 2, true);
            else if (n == 3) JP_P2G(2, 3, true);
            else JP_P2G(2, 4, true);
        } else {
            if (n == 1) JP_P2G(3, 1, true);
            else if (n == 2) JP_P2G(3, 2, true);
            else if (n == 3) JP_P2G(3, 3, true);
            else JP_P2G(3, 4, true);
        }
#undef JP_P2G
    }
    return cudaGetLastError();
}

cudaError_t launch_p2g(jp_particles* P, double* F, const double* Fp, const double* const coords[3],
                       const uint8_t* index, double* W)
{
    return p2g_launch(P, &F, &Fp, 1, false, coords, index, W);
}

cudaError_t launch_g2p_n(jp_particles* P, double* const* Fp, const double* const* F, int nf,
                         const double* const coords[3], const uint8_t* index)
{
    const bool d3 = P->g.ndim == 3;
    CCoords X{{coords[0], coords[1], d3 ? coords[2] : nullptr}};
    const unsigned nb = grid_blocks(P->g.ncells, 32 * kWarpsPerBlock);
    const int nt = 32 * kWarpsPerBlock;
    for (int f0 = 0; f0 < nf; f0 += kFieldsPerLaunchG2P) {
        const int n = nf - f0 < kFieldsPerLaunchG2P ? nf - f0 : kFieldsPerLaunchG2P;
        G2PFields GF{};
        for (int k = 0; k < n; ++k) {
            GF.f[k] = F[f0 + k];
            GF.fp[k] = Fp[f0 + k];
        }
#define JP_G2P(D, NF) g2p_n_kernel<D, NF><<<nb, nt, 0, P->stream>>>(P->g, GF, X, index)
        if (!d3) {
            if (n == 1) JP_G2P(2, 1);
            else if (n == 2) JP_G2P(2, 2);
            else if (n == 3) JP_G2P(2, 3);
            else JP_G2P(2, 4);
        } else {
            if (n == 1) JP_G2P(3, 1);
            else if (n == 2) JP_G2P(3, 2);
            else if (n == 3) JP_G2P(3, 3);
            else JP_G2P(3, 4);
        }
#undef JP_G2P
    }
    return cudaGetLastError();
}

cudaError_t launch_p2g_n(jp_particles* P, double* const* F, const double* const* Fp, int nf,
                         const double* const coords[3], const uint8_t* index)
{
    return p2g_launch(P, F, Fp, nf, true, coords, index, nullptr);
}

}  // namespace jp
