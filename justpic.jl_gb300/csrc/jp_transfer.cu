// jp_transfer.cu -- the transfers beside the hot path that work on the same
// layout: grid2particle_flip! (PIC/FLIP blend), centroid2particle! and
// particle2centroid! (cell-centred fields), and the phase ratios of
// update_phase_ratios!, FP64, 2D and 3D.
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
    const double beta = 1.0 - alpha;
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
            for (int d = 0; d < DIM; ++d) t[d] = (X.c[d][a] - cv[2 * NV + d]) * g.idmin[d];
            const double fpic = lerpN<DIM>(cv, t), f0pic = lerpN<DIM>(cv + NV, t);
            const double flip = Fp[a] + (fpic - f0pic);
            Fp[a] = fma(fpic, alpha, flip * beta);
        }
        __syncwarp();
    }
}

// ---------------------------------------------------- centroid2particle!
// Slot list of a warp's 32 cells built from the coordinates: the reference's
// centroid kernels take every slot whose coordinates are not NaN, whatever
// the index says.
template <int DIM>
__device__ __forceinline__ int build_coord_list(SlotList& Lst, const CCoords& X, int64_t c0, int64_t nc, int s0,
                                                int M, int lane)
{
    const bool valid = c0 + lane < nc;
    int K = 0;
#pragma unroll 4
    for (int s = 0; s < M; ++s) {
        bool live = valid;
        if (valid) {
#pragma unroll
            for (int d = 0; d < DIM; ++d) live = live & !is_nan_bits(X.c[d][c0 + lane + nc * (s0 + s)]);
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
    const int64_t C0 = g.n[0], C1 = g.n[1], sz = C0 * C1;
    for (int s0 = 0; s0 < M; s0 += 64) {  // slots in chunks of 64
    const int Mc = min(64, M - s0);
    const int K = build_coord_list<DIM>(lists[w], X, c0, nc, s0, Mc, lane);
    for (int k = lane; k < K; k += 32) {
        int s, l;
        slot_item(lists[w], Mc, k, &s, &l);
        const int64_t a = c0 + l + nc * (s0 + s);
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
    __syncwarp();
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

// ---------------------------------------------------------- phase ratios
// update_phase_ratios! (src/PhaseRatios/): the fraction of each phase (ids
// 1..nph in a per-slot field) around cell centres, vertices and faces, as a
// bilinear-weight average of the nearby particles. One thread per output
// node, particles and phases in the reference's order, so the sums are
// bit-identical to the CPU oracle. Output: out[k * nodes + node].
constexpr int kMaxPhases = 16;

template <int DIM>
__device__ __forceinline__ double bilinear_weight(const double* a, const double* b, const double* idi)
{
    double val = 1.0;
#pragma unroll
    for (int d = 0; d < DIM; ++d) val *= fma(-fabs(a[d] - b[d]), idi[d], 1.0);
    return val;
}

__device__ __forceinline__ void accumulate_phase(double* w, int nph, double x, double ph)
{
    for (int k = 0; k < nph; ++k)
        if (ph == (double)(k + 1)) w[k] = w[k] + x;
}

__device__ __forceinline__ void store_normalised(double* w, int nph, double* out, int64_t node, int64_t nodes,
                                                 bool nan_to_zero)
{
    double s = w[0];
    for (int k = 1; k < nph; ++k) s = s + w[k];
    const double is = 1.0 / s;
    for (int k = 0; k < nph; ++k) {
        const double v = w[k] * is;
        out[node + nodes * k] = (nan_to_zero && isnan(v)) ? 0.0 : v;
    }
}

// src/PhaseRatios/centers.jl:3-30 with phase_ratio_weights (utils.jl:44-61):
// the cell's own slots whose first coordinate is not NaN.
template <int DIM>
__global__ void __launch_bounds__(kThreads)
    phase_center_kernel(DevGrid g, int nph, const double* __restrict__ phases, CCoords X, double* __restrict__ out)
{
    const int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= g.ncells) return;
    const int64_t nc = g.ncells;
    int64_t I[3];
    cell_coords(g, c, I);
    double xc[3], idi[3], w[kMaxPhases];
    for (int k = 0; k < kMaxPhases; ++k) w[k] = 0.0;
#pragma unroll
    for (int d = 0; d < DIM; ++d) {
        xc[d] = ldg(g.xc[d] + I[d]);
        idi[d] = ldg(g.ixv[d] + I[d]);
    }
    for (int s = 0; s < g.max_xcell; ++s) {
        const int64_t a = c + nc * s;
        double p[3];
#pragma unroll
        for (int d = 0; d < DIM; ++d) p[d] = X.c[d][a];
        if (is_nan_bits(p[0])) continue;
        accumulate_phase(w, nph, bilinear_weight<DIM>(xc, p, idi), phases[a]);
    }
    store_normalised(w, nph, out, c, nc, false);
}

// src/PhaseRatios/vertices.jl:14-107: the 2^N cells around the vertex (offsets
// -1..0, first axis outermost), particles within half a cell of it.
template <int DIM>
__global__ void __launch_bounds__(kThreads)
    phase_vertex_kernel(DevGrid g, int nph, const double* __restrict__ phases, CCoords X, double* __restrict__ out)
{
    const int64_t V0 = g.n[0] + 1, V1 = g.n[1] + 1, V2 = DIM == 3 ? g.n[2] + 1 : 1;
    const int64_t nv = V0 * V1 * V2;
    const int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= nv) return;
    const int64_t nc = g.ncells;
    const int64_t I[3] = {v % V0, (v / V0) % V1, v / (V0 * V1)};
    double xv[3], w[kMaxPhases];
    for (int k = 0; k < kMaxPhases; ++k) w[k] = 0.0;
#pragma unroll
    for (int d = 0; d < DIM; ++d) xv[d] = ldg(g.xv[d] + I[d]);
    for (int oi = -1; oi <= 0; ++oi)
        for (int oj = -1; oj <= 0; ++oj)
            for (int ok = (DIM == 3 ? -1 : 0); ok <= 0; ++ok) {
                const int64_t J[3] = {I[0] + oi, I[1] + oj, DIM == 3 ? I[2] + ok : 0};
                if (J[0] < 0 || J[0] >= g.n[0] || J[1] < 0 || J[1] >= g.n[1]) continue;
                if (DIM == 3 && (J[2] < 0 || J[2] >= g.n[2])) continue;
                const int64_t c = cell_linear<DIM>(g, J);
                double di[3], idi[3];
#pragma unroll
                for (int d = 0; d < DIM; ++d) {
                    di[d] = ldg(g.dxv[d] + J[d]);
                    idi[d] = ldg(g.ixv[d] + J[d]);
                }
                for (int s = 0; s < g.max_xcell; ++s) {
                    const int64_t a = c + nc * s;
                    double p[3];
                    bool nan = false, far = false;
#pragma unroll
                    for (int d = 0; d < DIM; ++d) {
                        p[d] = X.c[d][a];
                        nan |= is_nan_bits(p[d]);
                    }
                    if (nan) continue;
#pragma unroll
                    for (int d = 0; d < DIM; ++d) far |= fabs(p[d] - xv[d]) >= di[d] / 2.0;
                    if (far) continue;
                    accumulate_phase(w, nph, bilinear_weight<DIM>(xv, p, idi), phases[a]);
                }
            }
    store_normalised(w, nph, out, v, nv, false);
}

template <int DIM>
__device__ __forceinline__ void face_cell(const DevGrid& g, int nph, const double* __restrict__ phases,
                                          const CCoords& X, int64_t c, const double* xf, const double* di,
                                          const double* idi, double* w)
{
    const int64_t nc = g.ncells;
    for (int s = 0; s < g.max_xcell; ++s) {
        const int64_t a = c + nc * s;
        double p[3];
        bool nan = false, in = true;
#pragma unroll
        for (int d = 0; d < DIM; ++d) {
            p[d] = X.c[d][a];
            nan |= is_nan_bits(p[d]);
        }
        if (nan) continue;
#pragma unroll
        for (int d = 0; d < DIM; ++d) in &= fabs(p[d] - xf[d]) <= di[d] / 2.0;  // isinhalfcell, utils.jl:79
        if (!in) continue;
        accumulate_phase(w, nph, bilinear_weight<DIM>(xf, p, idi), phases[a]);
    }
}

// src/PhaseRatios/midpoints.jl:19-94 along axis `dim`, one thread per cell I:
// face I + e gathers cells I and min(I + e, n) (the last cell twice at the far
// boundary, as the reference does); the first cell also writes face I, with
// the spacing the loop left behind. Faces without particles get 0.
template <int DIM>
__global__ void __launch_bounds__(kThreads)
    phase_face_kernel(DevGrid g, int nph, const double* __restrict__ phases, CCoords X, int dim,
                      double* __restrict__ out)
{
    const int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= g.ncells) return;
    int64_t I[3];
    cell_coords(g, c, I);
    int64_t F[3] = {g.n[0], g.n[1], DIM == 3 ? g.n[2] : 1};
    F[dim] += 1;
    const int64_t nf = F[0] * F[1] * F[2];
    double xcen[3], xf[3], di[3], idi[3], w[kMaxPhases];
    for (int k = 0; k < kMaxPhases; ++k) w[k] = 0.0;
#pragma unroll
    for (int d = 0; d < DIM; ++d) {
        xcen[d] = ldg(g.xc[d] + I[d]);
        di[d] = ldg(g.dxv[d] + I[d]);
        xf[d] = xcen[d] + (d == dim ? (di[d] * 1.0) / 2.0 : (di[d] * 0.0) / 2.0);
    }
    for (int it = 0; it < 2; ++it) {
        int64_t J[3] = {I[0], I[1], I[2]};
        if (it == 1) J[dim] = J[dim] + 1 < g.n[dim] ? J[dim] + 1 : g.n[dim] - 1;
#pragma unroll
        for (int d = 0; d < DIM; ++d) {
            di[d] = ldg(g.dxv[d] + J[d]);
            idi[d] = ldg(g.ixv[d] + J[d]);
        }
        face_cell<DIM>(g, nph, phases, X, cell_linear<DIM>(g, J), xf, di, idi, w);
    }
    int64_t Fi[3] = {I[0], I[1], I[2]};
    Fi[dim] += 1;
    store_normalised(w, nph, out, Fi[0] + F[0] * (Fi[1] + F[1] * Fi[2]), nf, true);
    if (I[dim] == 0) {
        double xb[3], wb[kMaxPhases];
        for (int k = 0; k < kMaxPhases; ++k) wb[k] = 0.0;
#pragma unroll
        for (int d = 0; d < DIM; ++d) xb[d] = xcen[d] - (d == dim ? (di[d] * 1.0) / 2.0 : (di[d] * 0.0) / 2.0);
        face_cell<DIM>(g, nph, phases, X, c, xb, di, idi, wb);
        store_normalised(wb, nph, out, I[0] + F[0] * (I[1] + F[1] * I[2]), nf, true);
    }
}

// src/PhaseRatios/midpoints.jl:108-242 (3D edge midpoints), one thread per
// cell I, offsets e = (1,1,0) xy, (0,1,1) yz, (1,0,1) xz: midpoint I + e at
// the cell centre plus half the cell's spacing along e gathers the cells
// min(I + e .* mask, n) for mask (1,0,0), (0,1,0), (0,0,1), (1,1,1) (a clamped
// cell counts again). A cell first along an offset axis also writes midpoint
// I and I + b (b: the offset axes where I is the last cell) from the
// particles around the centre moved by half a spacing along b. Writes never
// overlap when every axis has two cells or more.
__constant__ int kMidOff[3][3] = {{1, 1, 0}, {0, 1, 1}, {1, 0, 1}};
__constant__ int kMidMask[4][3] = {{1, 0, 0}, {0, 1, 0}, {0, 0, 1}, {1, 1, 1}};

__device__ __forceinline__ void midpoint_gather(const DevGrid& g, int nph, const double* __restrict__ phases,
                                                const CCoords& X, const int64_t* I, const int* off,
                                                const double* xm, double* w)
{
    for (int m = 0; m < 4; ++m) {
        int64_t J[3];
        double di[3], idi[3];
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            const int64_t j = I[d] + off[d] * kMidMask[m][d];
            J[d] = j < g.n[d] - 1 ? j : g.n[d] - 1;
            di[d] = ldg(g.dxv[d] + J[d]);
            idi[d] = ldg(g.ixv[d] + J[d]);
        }
        face_cell<3>(g, nph, phases, X, cell_linear<3>(g, J), xm, di, idi, w);
    }
}

__global__ void __launch_bounds__(kThreads)
    phase_midpoint_kernel(DevGrid g, int nph, const double* __restrict__ phases, CCoords X, int which,
                          double* __restrict__ out)
{
    const int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= g.ncells) return;
    int off[3];
#pragma unroll
    for (int d = 0; d < 3; ++d) off[d] = kMidOff[which][d];
    int64_t I[3];
    cell_coords(g, c, I);
    const int64_t Mn[3] = {g.n[0] + off[0], g.n[1] + off[1], g.n[2] + off[2]};
    const int64_t nm = Mn[0] * Mn[1] * Mn[2];
    double xcen[3], di[3], xm[3], w[kMaxPhases];
    for (int k = 0; k < kMaxPhases; ++k) w[k] = 0.0;
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        xcen[d] = ldg(g.xc[d] + I[d]);
        di[d] = ldg(g.dxv[d] + I[d]);
        xm[d] = xcen[d] + (di[d] * (double)off[d]) / 2.0;
    }
    midpoint_gather(g, nph, phases, X, I, off, xm, w);
    store_normalised(w, nph, out, (I[0] + off[0]) + Mn[0] * ((I[1] + off[1]) + Mn[1] * (I[2] + off[2])), nm, true);
    bool first = false;
    int b[3];
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        first |= off[d] && I[d] == 0;
        b[d] = (off[d] && I[d] == g.n[d] - 1) ? 1 : 0;
    }
    if (!first) return;
    double xb[3];
    for (int k = 0; k < kMaxPhases; ++k) w[k] = 0.0;
#pragma unroll
    for (int d = 0; d < 3; ++d) xb[d] = xcen[d] - ((di[d] * (double)off[d]) * (double)(0 - b[d])) / 2.0;
    midpoint_gather(g, nph, phases, X, I, off, xb, w);
    store_normalised(w, nph, out, I[0] + Mn[0] * (I[1] + Mn[1] * I[2]), nm, true);
    if (b[0] | b[1] | b[2])
        store_normalised(w, nph, out, (I[0] + b[0]) + Mn[0] * ((I[1] + b[1]) + Mn[1] * (I[2] + b[2])), nm, true);
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

cudaError_t launch_phase_ratios(jp_particles* P, int nph, const double* phases, const double* const coords[3],
                                double* center, double* vertex, double* const faces[3])
{
    const bool d3 = P->g.ndim == 3;
    CCoords X{{coords[0], coords[1], d3 ? coords[2] : nullptr}};
    cudaStream_t st = P->stream;
    const unsigned nb = grid_blocks(P->g.ncells);
    const int64_t nv = (P->g.n[0] + 1) * (P->g.n[1] + 1) * (d3 ? P->g.n[2] + 1 : 1);
    if (d3) {
        if (center) phase_center_kernel<3><<<nb, kThreads, 0, st>>>(P->g, nph, phases, X, center);
        if (vertex) phase_vertex_kernel<3><<<grid_blocks(nv), kThreads, 0, st>>>(P->g, nph, phases, X, vertex);
        for (int d = 0; d < 3; ++d)
            if (faces && faces[d]) phase_face_kernel<3><<<nb, kThreads, 0, st>>>(P->g, nph, phases, X, d, faces[d]);
    } else {
        if (center) phase_center_kernel<2><<<nb, kThreads, 0, st>>>(P->g, nph, phases, X, center);
        if (vertex) phase_vertex_kernel<2><<<grid_blocks(nv), kThreads, 0, st>>>(P->g, nph, phases, X, vertex);
        for (int d = 0; d < 2; ++d)
            if (faces && faces[d]) phase_face_kernel<2><<<nb, kThreads, 0, st>>>(P->g, nph, phases, X, d, faces[d]);
    }
    return cudaGetLastError();
}

cudaError_t launch_phase_midpoints(jp_particles* P, int nph, const double* phases, const double* const coords[3],
                                   double* const mids[3])
{
    CCoords X{{coords[0], coords[1], coords[2]}};
    const unsigned nb = grid_blocks(P->g.ncells);
    for (int w = 0; w < 3; ++w)
        if (mids[w]) phase_midpoint_kernel<<<nb, kThreads, 0, P->stream>>>(P->g, nph, phases, X, w, mids[w]);
    return cudaGetLastError();
}

}  // namespace jp
