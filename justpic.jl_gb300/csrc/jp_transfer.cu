// jp_transfer.cu -- the transfers beside the hot path that work on the same
// layout: grid2particle_flip! (PIC/FLIP blend), centroid2particle! and
// particle2centroid! (cell-centred fields), FP64, 2D and 3D.
//
// Each follows the reference's operation order (fma at its muladd sites), so
// the results are bit-identical to the CPU oracle; see the kernel comments for
// the reference lines.
#include <math_constants.h>

#include "jp_internal.cuh"

namespace jp {

// ---------------------------------------------------- grid2particle_flip!
// src/Interpolations/grid_to_particle.jl:125-170: for every live particle,
// F_pic and F0_pic at its position (one normalisation, the cell's corners of
// F and F0), then Fp = muladd(F_pic, a, (Fp + (F_pic - F0_pic)) * (1 - a)).
// The spacing is grid_size(xvi): the smallest vertex spacing of each axis.
template <int DIM>
__global__ void __launch_bounds__(32 * kWarpsPerBlock)
    g2p_flip_kernel(DevGrid g, double* __restrict__ Fp, const double* __restrict__ F, const double* __restrict__ F0,
                    double alpha, CCoords X, const uint8_t* __restrict__ index)
{
    constexpr int NV = 1 << DIM;
    __shared__ SlotList lists[kWarpsPerBlock];
    __shared__ double cellv[kWarpsPerBlock][32][2 * NV + DIM];
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int64_t c0 = ((int64_t)blockIdx.x * kWarpsPerBlock + w) * 32;
    if (c0 >= g.ncells) return;
    const int64_t nc = g.ncells;
    const int M = g.max_xcell;
    {
        int64_t I[3];
        cell_coords(g, min(c0 + lane, nc - 1), I);
        const int64_t V0 = g.n[0] + 1, V1 = g.n[1] + 1, sz = V0 * V1;
        const int64_t b = I[0] + V0 * (I[1] + (DIM == 3 ? V1 * I[2] : 0));
        const int64_t off[8] = {b, b + 1, b + V0, b + V0 + 1, b + sz, b + sz + 1, b + sz + V0, b + sz + V0 + 1};
        double* cv = cellv[w][lane];
#pragma unroll
        for (int k = 0; k < NV; ++k) {
            cv[k] = ldg(F + off[k]);
            cv[NV + k] = ldg(F0 + off[k]);
        }
#pragma unroll
        for (int d = 0; d < DIM; ++d) cv[2 * NV + d] = ldg(g.xv[d] + I[d]);
    }
    uint64_t mine;
    const int K = build_slot_list(lists[w], index, c0, nc, M, lane, &mine);
    const double beta = 1.0 - alpha;
    for (int k = lane; k < K; k += 32) {
        int s, l;
        slot_item(lists[w], M, k, &s, &l);
        const int64_t a = c0 + l + nc * s;
        const double* cv = cellv[w][l];
        double t[3];
#pragma unroll
        for (int d = 0; d < DIM; ++d) t[d] = (X.c[d][a] - cv[2 * NV + d]) * g.idmin[d];
        const double fpic = lerpN<DIM>(cv, t), f0pic = lerpN<DIM>(cv + NV, t);
        const double flip = Fp[a] + (fpic - f0pic);
        Fp[a] = fma(fpic, alpha, flip * beta);
    }
}

// ---------------------------------------------------- centroid2particle!
// Slot list of a warp's 32 cells built from the coordinates: the reference's
// centroid kernels take every slot whose coordinates are not NaN, whatever
// the index says.
template <int DIM>
__device__ __forceinline__ int build_coord_list(SlotList& Lst, const CCoords& X, int64_t c0, int64_t nc, int M,
                                                int lane)
{
    const bool valid = c0 + lane < nc;
    int K = 0;
#pragma unroll 4
    for (int s = 0; s < M; ++s) {
        bool live = valid;
        if (valid) {
#pragma unroll
            for (int d = 0; d < DIM; ++d) live = live & !is_nan_bits(X.c[d][c0 + lane + nc * s]);
        }
        const uint32_t m = __ballot_sync(0xffffffffu, live);
        if (lane == 0) {
            Lst.mask[s] = m;
            Lst.pre[s] = K;
        }
        K += __popc(m);
    }
    if (lane == 0) Lst.pre[M] = K;
    __syncwarp();
    return K;
}

// src/Interpolations/centroid_to_particle.jl:29-46: the centre cell below the
// particle along each axis (its own cell's centre, or the previous one when
// the particle lies below it: shifted_index), clamped to the centre grid, then
// the N-linear interpolation of the centred field F with the centre spacing.
template <int DIM>
__global__ void __launch_bounds__(32 * kWarpsPerBlock)
    c2p_kernel(DevGrid g, double* __restrict__ Fp, const double* __restrict__ F, CCoords X)
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
    const int K = build_coord_list<DIM>(lists[w], X, c0, nc, M, lane);
    const int64_t C0 = g.n[0], C1 = g.n[1], sz = C0 * C1;
    for (int k = lane; k < K; k += 32) {
        int s, l;
        slot_item(lists[w], M, k, &s, &l);
        const int64_t a = c0 + l + nc * s;
        int64_t J[3] = {0, 0, 0};
        double t[3];
#pragma unroll
        for (int d = 0; d < DIM; ++d) {
            const double p = X.c[d][a];
            const int I = cellI[w][l][d];
            int64_t j = p < ldg(g.xc[d] + I) ? I - 1 : I;
            const int64_t hi = g.n[d] - 2;
            j = j < 0 ? 0 : (j > hi ? hi : j);
            J[d] = j;
            t[d] = (p - ldg(g.xc[d] + j)) * ldg(g.ixc[d] + j);
        }
        const int64_t b = J[0] + C0 * (J[1] + (DIM == 3 ? C1 * J[2] : 0));
        double v[8];
        v[0] = ldg(F + b);
        v[1] = ldg(F + b + 1);
        v[2] = ldg(F + b + C0);
        v[3] = ldg(F + b + C0 + 1);
        if (DIM == 3) {
            v[4] = ldg(F + b + sz);
            v[5] = ldg(F + b + sz + 1);
            v[6] = ldg(F + b + sz + C0);
            v[7] = ldg(F + b + sz + C0 + 1);
        }
        Fp[a] = lerpN<DIM>(v, t);
    }
}

// ---------------------------------------------------- particle2centroid!
// src/Interpolations/particle_to_grid_centroid.jl:24-45 (2D), :88-110 (3D):
// one thread per cell over its slots in order; weight
// prod_d muladd(-|xc_d - p_d|, inv(dx_d), 1) (bilinear_weight,
// src/Interpolations/particle_to_grid.jl:210-222) with the cell's vertex
// spacing. 2D skips slots with any NaN coordinate and divides; 3D skips those
// whose first coordinate is NaN and multiplies by the inverse.
template <int DIM>
__global__ void __launch_bounds__(kThreads)
    p2c_kernel(DevGrid g, double* __restrict__ F, const double* __restrict__ Fp, CCoords X)
{
    const int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= g.ncells) return;
    const int64_t nc = g.ncells;
    int64_t I[3];
    cell_coords(g, c, I);
    double xcen[3], idx[3];
#pragma unroll
    for (int d = 0; d < DIM; ++d) {
        xcen[d] = ldg(g.xc[d] + I[d]);
        idx[d] = ldg(g.ixv[d] + I[d]);
    }
    double w = 0.0, wF = 0.0;
    for (int s = 0; s < g.max_xcell; ++s) {
        const int64_t a = c + nc * s;
        double p[3];
        bool skip = false;
#pragma unroll
        for (int d = 0; d < DIM; ++d) {
            p[d] = X.c[d][a];
            if (DIM == 2 || d == 0) skip |= is_nan_bits(p[d]);
        }
        if (skip) continue;
        double wi = 1.0;
#pragma unroll
        for (int d = 0; d < DIM; ++d) wi *= fma(-fabs(xcen[d] - p[d]), idx[d], 1.0);
        w += wi;
        wF = fma(wi, Fp[a], wF);
    }
    F[c] = DIM == 2 ? wF / w : wF * (1.0 / w);
}

// ------------------------------------------------------------ launchers
cudaError_t launch_g2p_flip(jp_particles* P, double* Fp, const double* F, const double* F0, double alpha,
                            const double* const coords[3], const uint8_t* index)
{
    const bool d3 = P->g.ndim == 3;
    CCoords X{{coords[0], coords[1], d3 ? coords[2] : nullptr}};
    const unsigned nb = grid_blocks(P->g.ncells, 32 * kWarpsPerBlock);
    const int nt = 32 * kWarpsPerBlock;
    if (d3)
        g2p_flip_kernel<3><<<nb, nt, 0, P->stream>>>(P->g, Fp, F, F0, alpha, X, index);
    else
        g2p_flip_kernel<2><<<nb, nt, 0, P->stream>>>(P->g, Fp, F, F0, alpha, X, index);
    return cudaGetLastError();
}

cudaError_t launch_c2p(jp_particles* P, double* Fp, const double* F, const double* const coords[3])
{
    const bool d3 = P->g.ndim == 3;
    CCoords X{{coords[0], coords[1], d3 ? coords[2] : nullptr}};
    const unsigned nb = grid_blocks(P->g.ncells, 32 * kWarpsPerBlock);
    const int nt = 32 * kWarpsPerBlock;
    if (d3)
        c2p_kernel<3><<<nb, nt, 0, P->stream>>>(P->g, Fp, F, X);
    else
        c2p_kernel<2><<<nb, nt, 0, P->stream>>>(P->g, Fp, F, X);
    return cudaGetLastError();
}

cudaError_t launch_p2c(jp_particles* P, double* F, const double* Fp, const double* const coords[3])
{
    const bool d3 = P->g.ndim == 3;
    CCoords X{{coords[0], coords[1], d3 ? coords[2] : nullptr}};
    const unsigned nb = grid_blocks(P->g.ncells);
    if (d3)
        p2c_kernel<3><<<nb, kThreads, 0, P->stream>>>(P->g, F, Fp, X);
    else
        p2c_kernel<2><<<nb, kThreads, 0, P->stream>>>(P->g, F, Fp, X);
    return cudaGetLastError();
}

}  // namespace jp
