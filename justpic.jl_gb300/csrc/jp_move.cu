// jp_move.cu -- move_particles! and inject_particles!.
//
// move_particles! (src/Particles/move_safe.jl:21-125) is a sequential slot walk
// per source cell, run in 3^N colour passes; its slot allocation (first free
// slot at or after `starting_point`, which carries over between target cells)
// decides which particles survive a full cell. It is reproduced exactly in
// three stages:
//   1. classify (all cells, one coalesced pass): which live slots left their
//      cell, where they go (one of the 3^N neighbours, or out), and a copy of
//      the movers' coordinates and fields into a shadow array;
//   2. allocate (3^N colour launches): the reference's walk, replayed on
//      64-bit occupancy masks only (L2-resident), recording for every refilled
//      slot the origin of its particle;
//   3. apply (all cells): refilled slots gather their particle from the
//      shadow, vacated slots become NaN / false.
// No atomics are used on the data path and the result does not depend on
// scheduling.
//
// inject_particles! (src/Particles/injection.jl:19-131) only changes a cell
// whose first quadrant is under-populated (the `break` at injection.jl:100
// ends the walk otherwise), and that test depends on the cell alone. A
// coalesced flag pass finds those cells; the 2^N colour passes then run the
// reference's sequential walk for flagged cells only.
#include <math_constants.h>

#include "jp_internal.cuh"

namespace jp {

struct MoveView {
    uint64_t* L0;
    uint64_t* L;
    uint64_t* M;
    uint64_t* R;
    uint64_t* U;
    uint8_t* code;
    uint16_t* orig;
    double* shadow;
    int64_t nslots;
};

// -------------------------------------------------------------- classify
template <int DIM>
__global__ void __launch_bounds__(kThreads)
    move_classify(DevGrid g, Coords X, const uint8_t* __restrict__ index, Args A, MoveView S, int* d_err)
{
    const int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= g.ncells) return;
    int64_t I[3];
    cell_coords(g, c, I);
    const int64_t nc = g.ncells;
    double corner[3], dx[3];
#pragma unroll
    for (int d = 0; d < DIM; ++d) {
        corner[d] = ldg(g.xv[d] + I[d]);
        dx[d] = ldg(g.dxv[d] + I[d]);
    }
    uint64_t L = 0, Mv = 0;
    int errs = 0;
    for (int s = 0; s < g.max_xcell; ++s) {
        const int64_t a = c + nc * s;
        if (!index[a]) continue;
        const uint64_t bit = 1ull << s;
        L |= bit;
        double p[3];
#pragma unroll
        for (int d = 0; d < DIM; ++d) p[d] = X.c[d][a];
        if (isincell<DIM>(p, corner, dx)) continue;  // move_safe.jl:93
        Mv |= bit;
        bool inside = true;  // indomain, strict (move_safe.jl:199-206)
#pragma unroll
        for (int d = 0; d < DIM; ++d) inside = inside & (g.dom_lo[d] < p[d]) & (p[d] < g.dom_hi[d]);
        uint8_t code = kCodeExit;
        if (inside) {
            int off[3] = {0, 0, 0};
            double cT[3], dT[3];
            bool far = false;
#pragma unroll
            for (int d = 0; d < DIM; ++d) {
                const int64_t T = find_cell(p[d], g.xv[d], g.n[d] + 1, I[d], &errs);
                off[d] = (int)(T - I[d]);
                far |= (off[d] > 1) | (off[d] < -1);
                cT[d] = ldg(g.xv[d] + T);
                dT[d] = ldg(g.dxv[d] + T);
            }
            if (far) {
                errs |= kWarnFarMove;
            } else {
                code = (uint8_t)nb_code<DIM>(off);
                if (!isincell<DIM>(p, cT, dT)) code |= kCodeUnstable;
#pragma unroll
                for (int d = 0; d < DIM; ++d) S.shadow[d * S.nslots + a] = p[d];
                for (int k = 0; k < A.n; ++k) S.shadow[(DIM + k) * S.nslots + a] = A.a[k][a];
            }
        }
        S.code[a] = code;
    }
    S.L0[c] = L;
    S.L[c] = L;
    S.M[c] = Mv;
    S.R[c] = 0;
    S.U[c] = 0;
    raise_err(d_err, errs);
}

// -------------------------------------------------------------- allocate
// One colour pass of move_particles!: sources 3*J + o, neighbourhoods
// disjoint, so every mask touched here belongs to exactly one thread.
template <int DIM>
__global__ void __launch_bounds__(kThreads)
    move_allocate(DevGrid g, MoveView S, int o0, int o1, int o2, int64_t m0, int64_t m1, int64_t m2)
{
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= m0 * m1 * m2) return;
    int64_t idx[3];
    idx[0] = 3 * (t % m0) + o0;
    idx[1] = 3 * ((t / m0) % m1) + o1;
    idx[2] = DIM == 3 ? 3 * (t / (m0 * m1)) + o2 : 0;
#pragma unroll
    for (int d = 0; d < DIM; ++d)
        if (idx[d] >= g.n[d]) return;
    const int64_t nc = g.ncells;
    const int64_t sc = cell_linear<DIM>(g, idx);
    const uint64_t Mv = S.M[sc];
    uint64_t U = S.U[sc];
    if (Mv == 0 && U == 0) return;
    uint64_t L = S.L[sc], R = S.R[sc];
    const int nslot = g.max_xcell;
    const uint64_t valid = nslot == 64 ? ~0ull : ((1ull << nslot) - 1);
    int sp = 0;  // starting_point (move_safe.jl:83)
    int cur = 0;
    while (cur < nslot) {
        uint64_t cand = L & ((Mv & ~R) | (R & U)) & (~0ull << cur);
        if (!cand) break;
        const int s = __ffsll((long long)cand) - 1;
        cur = s + 1;
        const uint64_t bit = 1ull << s;
        int code;
        bool unstable;
        bool from_refill = (R & bit) != 0;
        uint16_t tag = 0;
        if (from_refill) {
            code = self_code<DIM>();
            unstable = true;
            tag = S.orig[sc + nc * s];
        } else {
            const uint8_t cb = S.code[sc + nc * s];
            if (cb == kCodeExit) {  // left the domain (or moved too far): cleared
                L &= ~bit;
                continue;
            }
            code = cb & 0x1F;
            unstable = (cb & kCodeUnstable) != 0;
        }
        // remove the particle from its slot (move_safe.jl:110-112)
        L &= ~bit;
        R &= ~bit;
        U &= ~bit;
        int off[3];
        nb_offset<DIM>(code, off);
        int64_t T[3] = {idx[0] + off[0], idx[1] + off[1], DIM == 3 ? idx[2] + off[2] : 0};
        const int64_t tc = cell_linear<DIM>(g, T);
        if (!from_refill) {
            const int back[3] = {-off[0], -off[1], -off[2]};
            tag = (uint16_t)(nb_code<DIM>(back) | (s << 5));
        }
        const bool same = tc == sc;
        uint64_t LT = same ? L : S.L[tc];
        // find_free_memory(starting_point, ...) (move_safe.jl:192-197)
        const uint64_t freem = ~LT & valid & (~0ull << sp);
        if (!freem) continue;  // dropped: no free slot at or after starting_point
        const int f = __ffsll((long long)freem) - 1;
        sp = f;
        const uint64_t fb = 1ull << f;
        uint64_t RT = same ? R : S.R[tc];
        uint64_t UT = same ? U : S.U[tc];
        LT |= fb;
        RT |= fb;
        UT = unstable ? (UT | fb) : (UT & ~fb);
        S.orig[tc + nc * f] = tag;
        if (same) {
            L = LT;
            R = RT;
            U = UT;
        } else {
            S.L[tc] = LT;
            S.R[tc] = RT;
            S.U[tc] = UT;
        }
    }
    S.L[sc] = L;
    S.R[sc] = R;
    S.U[sc] = U;
}

// ----------------------------------------------------------------- apply
template <int DIM>
__global__ void __launch_bounds__(kThreads)
    move_apply(DevGrid g, Coords X, uint8_t* __restrict__ index, Args A, MoveView S)
{
    const int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= g.ncells) return;
    const uint64_t L0 = S.L0[c], L = S.L[c], R = S.R[c];
    uint64_t changed = (L0 & ~L) | R;
    if (!changed) return;
    int64_t I[3];
    cell_coords(g, c, I);
    const int64_t nc = g.ncells;
    while (changed) {
        const int s = __ffsll((long long)changed) - 1;
        changed &= changed - 1;
        const int64_t a = c + nc * s;
        if ((R >> s) & 1) {
            const uint16_t tag = S.orig[a];
            int off[3];
            nb_offset<DIM>(tag & 0x1F, off);
            const int64_t J[3] = {I[0] + off[0], I[1] + off[1], DIM == 3 ? I[2] + off[2] : 0};
            const int64_t b = cell_linear<DIM>(g, J) + nc * (tag >> 5);
#pragma unroll
            for (int d = 0; d < DIM; ++d) X.c[d][a] = S.shadow[d * S.nslots + b];
            for (int k = 0; k < A.n; ++k) A.a[k][a] = S.shadow[(DIM + k) * S.nslots + b];
            index[a] = 1;
        } else {
#pragma unroll
            for (int d = 0; d < DIM; ++d) X.c[d][a] = CUDART_NAN;
            for (int k = 0; k < A.n; ++k) A.a[k][a] = CUDART_NAN;
            index[a] = 0;
        }
    }
}

// ------------------------------------------------------------- injection
// first quadrant occupancy test (injection.jl:81-100 for the first vertex)
template <int DIM>
__global__ void __launch_bounds__(kThreads)
    inject_flag(DevGrid g, CCoords X, const uint8_t* __restrict__ index, uint8_t* __restrict__ flag)
{
    const int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= g.ncells) return;
    int64_t I[3];
    cell_coords(g, c, I);
    const int64_t nc = g.ncells;
    double qc[3], dq[3];
#pragma unroll
    for (int d = 0; d < DIM; ++d) {
        qc[d] = ldg(g.xv[d] + I[d]);
        dq[d] = ldg(g.dxv[d] + I[d]) / 2.0;
    }
    const int min_xq = (g.min_xcell + (1 << DIM) - 1) >> DIM;
    int count = 0;
    for (int s = 0; s < g.max_xcell && count < min_xq; ++s) {
        const int64_t a = c + nc * s;
        if (!index[a]) continue;
        double p[3];
#pragma unroll
        for (int d = 0; d < DIM; ++d) p[d] = X.c[d][a];
        count += isincell<DIM>(p, qc, dq) ? 1 : 0;
    }
    flag[c] = count < min_xq ? 1 : 0;
}

// index_min_distance: src/Particles/injection.jl:330-393
template <int DIM>
__device__ bool nearest_particle(const DevGrid& g, const Coords& X, const uint8_t* __restrict__ index,
                                 const double* pn, int cur_slot, const int64_t* I, int64_t* best)
{
    const int64_t nc = g.ncells;
    double dmin = CUDART_INF;
    bool found = false;
    const int kr = DIM == 3 ? 1 : 0;
    for (int64_t k = I[2] - kr; k <= I[2] + kr; ++k) {
        for (int64_t j = I[1] - 1; j <= I[1] + 1; ++j) {
            for (int64_t i = I[0] - 1; i <= I[0] + 1; ++i) {
                if (i < 0 || j < 0 || k < 0) continue;
                if (i >= g.n[0] || j >= g.n[1] || (DIM == 3 && k >= g.n[2])) continue;
                const int64_t J[3] = {i, j, k};
                const int64_t cc = cell_linear<DIM>(g, J);
                const bool self = (i == I[0]) && (j == I[1]) && (k == I[2]);
                for (int ip = 0; ip < g.max_xcell; ++ip) {
                    if (self && ip == cur_slot) continue;
                    const int64_t a = cc + nc * ip;
                    if (!index[a]) continue;
                    double ss;
                    if (DIM == 2) {
                        const double px = X.c[0][a], py = X.c[1][a];
                        if (isnan(px) || isnan(py)) continue;
                        const double dxx = px - pn[0], dyy = py - pn[1];
                        ss = dxx * dxx + dyy * dyy;
                    } else {
                        const double dxx = X.c[0][a] - pn[0];
                        const double dyy = X.c[1][a] - pn[1];
                        const double dzz = X.c[2][a] - pn[2];
                        ss = (dxx * dxx + dyy * dyy) + dzz * dzz;
                    }
                    const double dist = sqrt(ss);
                    if (dist < dmin) {
                        dmin = dist;
                        *best = a;
                        found = true;
                    }
                }
            }
        }
    }
    return found;
}

// _inject_particles!: src/Particles/injection.jl:68-131, for flagged cells
template <int DIM>
__global__ void __launch_bounds__(kThreads)
    inject_pass(DevGrid g, Coords X, uint8_t* __restrict__ index, Args A, const uint8_t* __restrict__ flag,
                uint32_t call, int o0, int o1, int o2, int64_t m0, int64_t m1, int64_t m2, int* d_err)
{
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= m0 * m1 * m2) return;
    int64_t idx[3];
    idx[0] = 2 * (t % m0) + o0;
    idx[1] = 2 * ((t / m0) % m1) + o1;
    idx[2] = DIM == 3 ? 2 * (t / (m0 * m1)) + o2 : 0;
#pragma unroll
    for (int d = 0; d < DIM; ++d)
        if (idx[d] >= g.n[d]) return;
    const int64_t c = cell_linear<DIM>(g, idx);
    if (!flag[c]) return;
    const int64_t nc = g.ncells;
    double corner[3], dq[3];
#pragma unroll
    for (int d = 0; d < DIM; ++d) {
        corner[d] = ldg(g.xv[d] + idx[d]);
        dq[d] = ldg(g.dxv[d] + idx[d]) / 2.0;
    }
    const int min_xq = (g.min_xcell + (1 << DIM) - 1) >> DIM;
    int errs = 0;
    for (int q = 0; q < (1 << DIM); ++q) {
        double qc[3];
#pragma unroll
        for (int d = 0; d < DIM; ++d) qc[d] = corner[d] + dq[d] * (double)((q >> d) & 1);
        int count = 0;
        for (int i = 0; i < g.max_xcell; ++i) {
            const int64_t a = c + nc * i;
            if (!index[a]) continue;
            double p[3];
#pragma unroll
            for (int d = 0; d < DIM; ++d) p[d] = X.c[d][a];
            count += isincell<DIM>(p, qc, dq) ? 1 : 0;
        }
        if (count >= min_xq) break;
        for (int i = 0; i < g.max_xcell; ++i) {
            const int64_t a = c + nc * i;
            if (index[a]) continue;
            ++count;
            double pn[3];
#pragma unroll
            for (int d = 0; d < DIM; ++d) {
                const double r = jp_rand_uniform(g.seed, JP_RNG_STREAM_INJECT, call, (uint64_t)c, (uint32_t)i,
                                                 (uint32_t)d);
                pn[d] = qc[d] + dq[d] * fma(0.95, r, 0.05);  // new_particle, injection.jl:411-417
            }
#pragma unroll
            for (int d = 0; d < DIM; ++d) X.c[d][a] = pn[d];
            index[a] = 1;
            int64_t src = 0;
            if (nearest_particle<DIM>(g, X, index, pn, i, idx, &src)) {
                for (int k = 0; k < A.n; ++k) A.a[k][a] = A.a[k][src];
            } else if (A.n > 0) {
                errs |= kWarnNoNeighbour;
            }
            if (count >= min_xq) break;
        }
    }
    raise_err(d_err, errs);
}

// ------------------------------------------------------------ launchers
static cudaError_t ensure_move_scratch(jp_particles* P, int comps)
{
    MoveScratch& m = P->move;
    if (m.L0 && m.shadow_comps >= comps) return cudaSuccess;
    if (m.L0) {
        cudaError_t e = cudaStreamSynchronize(P->stream);
        if (e != cudaSuccess) return e;
        cudaFree(m.L0);
        m = MoveScratch();
    }
    const int64_t nc = P->g.ncells;
    const int64_t ns = nc * P->g.max_xcell;
    size_t bytes = 5 * nc * sizeof(uint64_t);  // masks first (8-byte aligned)
    const size_t off_shadow = bytes;
    bytes += (size_t)comps * ns * sizeof(double);
    const size_t off_orig = bytes;
    bytes += ns * sizeof(uint16_t);
    const size_t off_code = bytes;
    bytes += ns * sizeof(uint8_t);
    char* base = nullptr;
    cudaError_t e = cudaMalloc(&base, bytes);
    if (e != cudaSuccess) return e;
    m.L0 = (uint64_t*)base;
    m.L = m.L0 + nc;
    m.M = m.L + nc;
    m.R = m.M + nc;
    m.U = m.R + nc;
    m.shadow = (double*)(base + off_shadow);
    m.orig = (uint16_t*)(base + off_orig);
    m.code = (uint8_t*)(base + off_code);
    m.shadow_comps = comps;
    m.bytes = bytes;
    return cudaSuccess;
}

cudaError_t launch_move(jp_particles* P, double* const coords[3], uint8_t* index, double* const* args,
                        int nargs)
{
    const int N = P->g.ndim;
    cudaError_t e = ensure_move_scratch(P, N + nargs);
    if (e != cudaSuccess) return e;
    Coords X{{coords[0], coords[1], N == 3 ? coords[2] : nullptr}};
    Args A{};
    A.n = nargs;
    for (int k = 0; k < nargs; ++k) A.a[k] = args[k];
    const MoveScratch& m = P->move;
    MoveView S{m.L0, m.L, m.M, m.R, m.U, m.code, m.orig, m.shadow, P->g.ncells * P->g.max_xcell};
    cudaStream_t st = P->stream;
    const unsigned nb = grid_blocks(P->g.ncells);
    int64_t mc[3] = {1, 1, 1};
    for (int d = 0; d < N; ++d) mc[d] = (P->g.n[d] + 2) / 3;  // ceil(n/3)
    const unsigned nbp = grid_blocks(mc[0] * mc[1] * mc[2]);
    if (N == 2) {
        move_classify<2><<<nb, kThreads, 0, st>>>(P->g, X, index, A, S, P->d_err);
        for (int pass = 0; pass < 9; ++pass)  // offsetᵢ outer, offsetⱼ inner (move_safe.jl:32)
            move_allocate<2><<<nbp, kThreads, 0, st>>>(P->g, S, pass / 3, pass % 3, 0, mc[0], mc[1], 1);
        move_apply<2><<<nb, kThreads, 0, st>>>(P->g, X, index, A, S);
    } else {
        move_classify<3><<<nb, kThreads, 0, st>>>(P->g, X, index, A, S, P->d_err);
        for (int pass = 0; pass < 27; ++pass)  // i outer, k inner (move_safe.jl:39)
            move_allocate<3><<<nbp, kThreads, 0, st>>>(P->g, S, pass / 9, (pass / 3) % 3, pass % 3, mc[0], mc[1],
                                                       mc[2]);
        move_apply<3><<<nb, kThreads, 0, st>>>(P->g, X, index, A, S);
    }
    return cudaGetLastError();
}

cudaError_t launch_inject(jp_particles* P, double* const coords[3], uint8_t* index, double* const* args,
                          int nargs, uint32_t call)
{
    const int N = P->g.ndim;
    if (!P->inject.flag) {
        cudaError_t e = cudaMalloc(&P->inject.flag, P->g.ncells);
        if (e != cudaSuccess) return e;
    }
    Coords X{{coords[0], coords[1], N == 3 ? coords[2] : nullptr}};
    CCoords CX{{coords[0], coords[1], N == 3 ? coords[2] : nullptr}};
    Args A{};
    A.n = nargs;
    for (int k = 0; k < nargs; ++k) A.a[k] = args[k];
    cudaStream_t st = P->stream;
    const unsigned nb = grid_blocks(P->g.ncells);
    int64_t mc[3] = {1, 1, 1};
    for (int d = 0; d < N; ++d) mc[d] = (P->g.n[d] + 1) / 2;  // ceil(n/2)
    const unsigned nbp = grid_blocks(mc[0] * mc[1] * mc[2]);
    uint8_t* flag = P->inject.flag;
    if (N == 2) {
        inject_flag<2><<<nb, kThreads, 0, st>>>(P->g, CX, index, flag);
        for (int pass = 0; pass < 4; ++pass)
            inject_pass<2><<<nbp, kThreads, 0, st>>>(P->g, X, index, A, flag, call, pass / 2, pass % 2, 0, mc[0],
                                                     mc[1], 1, P->d_err);
    } else {
        inject_flag<3><<<nb, kThreads, 0, st>>>(P->g, CX, index, flag);
        for (int pass = 0; pass < 8; ++pass)
            inject_pass<3><<<nbp, kThreads, 0, st>>>(P->g, X, index, A, flag, call, pass / 4, (pass / 2) % 2,
                                                     pass % 2, mc[0], mc[1], mc[2], P->d_err);
    }
    return cudaGetLastError();
}

}  // namespace jp
