// jp_f32.cu -- the split-precision form of the hot path.
//
// Each particle is its slot's cell (an implicit int32 cell index: the
// CellArray slot belongs to one cell) plus an FP32 offset xi in [0, 1)^N in
// units of that cell's spacing, so round-off scales with the cell width and not
// with the domain. Velocities, interpolation weights and Runge-Kutta stages
// are FP32; FP64 is kept for the weight sums of particle2grid!. On a uniform
// grid every spacing is one number per axis; on a grid whose spacing varies
// the kernels read per-cell tables of widths and width ratios (F32Axes), and
// offsets carried across a face are converted to the new cell's units. The
// form has no reference counterpart: its error is stated against the FP64 form
// on the same seeded run.
//
// Semantics in cell units (FP64 form: the reference's rules):
//   * a particle belongs to its cell when 0 <= xi < 1 on every axis;
//   * velocity component c is sampled on its staggered grid: along its own
//     axis the nodes are the cell vertices (node k at k), along the others the
//     ghost-expanded centres (node k at k - 1/2; on a grid whose spacing
//     varies, the cell midpoints and the grid's own ghost nodes); outside a
//     grid's limits the sample is Inf, as in the reference;
//   * move_particles! sends a particle to cell + floor(xi) with
//     xi - floor(xi) (one FP32 operation, kept below 1; scaled to the new
//     cell's width where the spacing varies, and dropped as a move of more
//     than one cell if it then lies outside that cell), with the reference's
//     colour-pass slot allocation (shared allocate stage);
//   * inject_particles! follows the reference's quadrant walk; new offsets are
//     quadrant corner + 1/2 * (0.05 + 0.95 r) and the nearest neighbour is the
//     first minimum of the FP32 squared physical distance in k -> j -> i ->
//     slot order;
//   * particle2grid! weights are 1 / |vertex - particle|^2 in FP32, summed at
//     FP64 accuracy in the reference's order (compensated FP32 pairs within a
//     cell, FP64 across cells).
#include <math_constants.h>

#include <cmath>

#include "jp_f32_core.cuh"
#include "jp_internal.cuh"
#include "jp_move_core.cuh"

namespace jp {

// ------------------------------------------------------------ conversions
template <int DIM>
__global__ void __launch_bounds__(kThreads)
    to_offsets(DevGrid g, CCoords X, const uint8_t* __restrict__ index, XiF Xi)
{
    const int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= g.ncells) return;
    int64_t I[3];
    cell_coords(g, c, I);
    const int64_t nc = g.ncells;
    double x0[3], ix[3];
#pragma unroll
    for (int d = 0; d < DIM; ++d) {
        x0[d] = ldg(g.xv[d] + I[d]);
        ix[d] = ldg(g.ixv[d] + I[d]);
    }
    for (int s = 0; s < g.max_xcell; ++s) {
        const int64_t a = c + nc * s;
        const bool live = index[a] != 0;
#pragma unroll
        for (int d = 0; d < DIM; ++d) Xi.x[d][a] = live ? (float)((X.c[d][a] - x0[d]) * ix[d]) : CUDART_NAN_F;
    }
}

template <int DIM>
__global__ void __launch_bounds__(kThreads)
    to_coords(DevGrid g, CXiF Xi, const uint8_t* __restrict__ index, Coords X)
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
    for (int s = 0; s < g.max_xcell; ++s) {
        const int64_t a = c + nc * s;
        const bool live = index[a] != 0;
#pragma unroll
        for (int d = 0; d < DIM; ++d) X.c[d][a] = live ? fma((double)Xi.x[d][a], dx[d], x0[d]) : CUDART_NAN;
    }
}

// ------------------------------------------------------------- advection
// sample(x, v): every velocity component at offset x of the particle's cell;
// w / aw: dt / dx and alpha dt / dx of that cell per axis
template <int DIM, int METHOD, class Sample>
__device__ __forceinline__ void advect_f32(const F32Params& P, const float* w, const float* aw, const float* x0,
                                           float* x, Sample sample)
{
    float v0[3], v1[3], q[3];
    if (METHOD == JP_RUNGE_KUTTA2) {
        sample(x0, v0);
#pragma unroll
        for (int d = 0; d < DIM; ++d) q[d] = fmaf(aw[d], v0[d], x0[d]);
        sample(q, v1);
#pragma unroll
        for (int d = 0; d < DIM; ++d)
            x[d] = P.half ? fmaf(w[d], v1[d], x0[d]) : fmaf(w[d], fmaf(P.ca, v0[d], P.cb * v1[d]), x0[d]);
    } else if (METHOD == JP_RUNGE_KUTTA4) {
        float k1[3], k2[3], k3[3], k4[3];
        sample(x0, k1);
#pragma unroll
        for (int d = 0; d < DIM; ++d) q[d] = fmaf(0.5f * w[d], k1[d], x0[d]);
        sample(q, k2);
#pragma unroll
        for (int d = 0; d < DIM; ++d) q[d] = fmaf(0.5f * w[d], k2[d], x0[d]);
        sample(q, k3);
#pragma unroll
        for (int d = 0; d < DIM; ++d) q[d] = fmaf(w[d], k3[d], x0[d]);
        sample(q, k4);
#pragma unroll
        for (int d = 0; d < DIM; ++d)
            x[d] = fmaf(w[d] * (1.0f / 6.0f), (k1[d] + 2.0f * k2[d]) + (2.0f * k3[d] + k4[d]), x0[d]);
    } else {
        sample(x0, v0);
#pragma unroll
        for (int d = 0; d < DIM; ++d) x[d] = fmaf(w[d], v0[d], x0[d]);
    }
}

// A warp takes 32 consecutive cells and their live particles in slot-major
// order (full lanes whatever the occupancy). CELLS: the grid's spacing varies;
// each cell's steps are dt and alpha dt times the container's 1/dx[i] (one
// FP64 product per cell and axis), its samples walk the per-cell tables.
template <int DIM, int METHOD, bool CELLS, bool WIDE>
__global__ void __launch_bounds__(32 * kWarpsPerBlock)
    advect_f32_kernel(DevGrid g, CVelF V, F32Params P, XiF Xi, const uint8_t* __restrict__ index)
{
    __shared__ SlotList lists[kWarpsPerBlock];
    __shared__ int cellI[kWarpsPerBlock][32][3];
    __shared__ float cellW[CELLS ? kWarpsPerBlock : 1][32][2 * DIM];
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
        if (CELLS) {
#pragma unroll
            for (int d = 0; d < DIM; ++d) {
                const double ix = ldg(g.ixv[d] + I[d]);
                cellW[w][lane][d] = (float)(P.dt * ix);
                cellW[w][lane][DIM + d] = (float)(P.adt * ix);
            }
        }
    }
    for (int s0 = 0; s0 < (WIDE ? M : 1); s0 += 64) {  // WIDE: slots in chunks of 64 (max_xcell > 64)
        const int Mc = min(64, M - s0);
        uint64_t mine;
        const int K = build_slot_list(lists[w], index + nc * s0, c0, nc, Mc, lane, &mine);
        int row = 0;
        for (int k = lane; k < K; k += 32) {
            int s, l;
            slot_item_next(lists[w], Mc, k, &row, &s, &l);
            const int64_t a = c0 + l + nc * (s0 + s);
            const int I[3] = {cellI[w][l][0], cellI[w][l][1], cellI[w][l][2]};
            float x0[3], x[3];
#pragma unroll
            for (int d = 0; d < DIM; ++d) x0[d] = Xi.x[d][a];
            if (CELLS) {
                float wc[3], awc[3];
#pragma unroll
                for (int d = 0; d < DIM; ++d) {
                    wc[d] = cellW[w][l][d];
                    awc[d] = cellW[w][l][DIM + d];
                }
                advect_f32<DIM, METHOD>(P, wc, awc, x0, x,
                                        [&](const float* xi, float* v) { velocity_f32_cells<DIM>(g, P.ax, I, xi, V, v); });
            } else {
                advect_f32<DIM, METHOD>(P, P.w, P.aw, x0, x, [&](const float* xi, float* v) {
#pragma unroll
                    for (int c = 0; c < DIM; ++c) v[c] = velocity_f32<DIM>(g, c, I, xi, V.v[c]);
                });
            }
#pragma unroll
            for (int d = 0; d < DIM; ++d) Xi.x[d][a] = x[d];
        }
        if (WIDE) __syncwarp();  // the next chunk rebuilds the warp's list
    }
}

// ------------------------------------------------------------------- move
struct MoveViewF {
    MoveView m;
    float* shadow;  // interleaved records: DIM offsets, then the fields
};

// Destination of a particle at offset xi of cell I (xi outside [0, 1) on some
// axis): the neighbour offset per axis and the re-normalised offset in that
// cell, kept below 1. xi - floor(xi) is one correctly rounded FP32
// subtraction: for floor = 1 it is exact (Sterbenz), for floor = -1 the exact
// 1 + xi fits FP64 whenever it does not round to 1.0f in FP32 either, so this
// equals the FP64 difference rounded to FP32 without the FP64 pipe. CELLS:
// the grid's spacing varies; an offset carried into a neighbour is converted
// to that cell's units (tables tor / tol), and one that still lies outside
// the neighbour has moved more than one cell. inside: the destination is a
// cell of the grid (false for NaN / Inf offsets: left the domain); far: it is
// more than one cell away (the particle is dropped).
template <int DIM, bool CELLS>
__device__ __forceinline__ void offset_destination(const DevGrid& g, const F32Axes& ax, const int* I,
                                                   const float* xi, float* v, int* off, bool* inside, bool* far)
{
    bool in = true, fr = false;
#pragma unroll
    for (int d = 0; d < DIM; ++d) {
        off[d] = 0;
        if (!(fabsf(xi[d]) < 1e6f)) {  // NaN / Inf: left the domain
            in = false;
            continue;
        }
        const float fl = floorf(xi[d]);
        int o = (int)fl;
        float rr = xi[d] - fl;
        if (CELLS && o == 1) {  // (xi - 1) dx[i] / dx[i+1]
            rr = (xi[d] - 1.0f) * __ldg(ax.tor[d] + I[d]);
            if (!(rr < 1.0f)) o = 2;
        } else if (CELLS && o == -1) {  // 1 + xi dx[i] / dx[i-1]
            rr = fmaf(xi[d], __ldg(ax.tol[d] + I[d]), 1.0f);
            if (rr < 0.0f) o = -2;
        }
        const int T = I[d] + o;
        in &= T >= 0 && T < g.n[d];
        fr |= o > 1 || o < -1;
        off[d] = o;
        v[d] = rr < 1.0f ? rr : 0x1.fffffep-1f;
    }
    *inside = in;
    *far = fr;
}

// The FP64 classify's scheme (slot-major live particles over the lanes, loads
// of a batch in flight together, records written after a warp barrier at
// their cell's next record), four particles per lane in flight.
template <int DIM, bool CELLS>
__global__ void __launch_bounds__(32 * kWarpsPerBlock)
    move_classify_f32(DevGrid g, XiF Xi, const uint8_t* __restrict__ index, ArgsF A, MoveViewF S, F32Axes ax,
                      int* d_err)
{
    __shared__ SlotList lists[kWarpsPerBlock];
    __shared__ int cellI[kWarpsPerBlock][32][3];
    __shared__ unsigned long long movers[kWarpsPerBlock][32];
    constexpr int NT = DIM == 2 ? 9 : 1;  // 2D: movers bound for each of the 9 neighbours
    __shared__ unsigned long long tmask[kWarpsPerBlock][NT][32];
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
        movers[w][lane] = 0;
#pragma unroll
        for (int k = 0; k < NT; ++k) tmask[w][k][lane] = 0;
    }
    uint64_t L;
    const int K = build_slot_list(lists[w], index, c0, nc, M, lane, &L);
    const int comps = S.m.comps;
    const bool whole = comps == 4;
    int errs = 0, n_exit = 0, n_far = 0;
    // one live particle: its destination code (kCodeStay, kCodeExit or a neighbour
    // code) and, for a mover, its re-normalised offsets in v
    auto classify_one = [&](int s, int l, int64_t a, const float* xi, float* v) -> uint8_t {
        bool out = false;
#pragma unroll
        for (int d = 0; d < DIM; ++d) out |= !(xi[d] >= 0.0f && xi[d] < 1.0f);
        if (!out) return kCodeStay;
        const unsigned long long bit = 1ull << s;
        atomicOr(&movers[w][l], bit);
        int off[3];
        bool inside, far;
        const int I[3] = {cellI[w][l][0], cellI[w][l][1], cellI[w][l][2]};
        offset_destination<DIM, CELLS>(g, ax, I, xi, v, off, &inside, &far);
        uint8_t code = kCodeExit;
        if (!inside) {
            ++n_exit;
        } else if (far) {
            errs |= kWarnFarMove;
            ++n_far;
        } else {
            code = (uint8_t)nb_code<DIM>(off);
        }
        if (DIM == 2) {
            if (code != kCodeExit) atomicOr(&tmask[w][code][l], bit);
        } else {
            S.m.code[a] = code;
        }
        return code;
    };
    constexpr int B = 4;
    int row = 0;
    for (int k0 = lane; k0 < K; k0 += 32 * B) {
        int sl[B], ll[B];
        int64_t al[B];
        float xl[B][3], fl[B][4 - DIM], vl[B][4];
        bool has[B];
        uint8_t code[B];
#pragma unroll
        for (int u = 0; u < B; ++u) {
            const int k = k0 + 32 * u;
            has[u] = k < K;
            sl[u] = 0;
            ll[u] = 0;
            if (has[u]) slot_item_next(lists[w], M, k, &row, &sl[u], &ll[u]);
            al[u] = c0 + ll[u] + nc * sl[u];
#pragma unroll
            for (int d = 0; d < DIM; ++d) xl[u][d] = has[u] ? Xi.x[d][al[u]] : 0.0f;
#pragma unroll
            for (int j = 0; j < 4 - DIM; ++j) fl[u][j] = (has[u] && whole && j < A.n) ? A.a[j][al[u]] : 0.0f;
        }
#pragma unroll
        for (int u = 0; u < B; ++u) {
#pragma unroll
            for (int j = 0; j < 4; ++j) vl[u][j] = 0.0f;
            code[u] = has[u] ? classify_one(sl[u], ll[u], al[u], xl[u], vl[u]) : kCodeStay;
        }
        __syncwarp();  // every mover bit of this batch is set
#pragma unroll
        for (int u = 0; u < B; ++u) {
            if (code[u] == kCodeStay || code[u] == kCodeExit) continue;
            const int l = ll[u];
            const int r = __popcll(movers[w][l] & ((1ull << sl[u]) - 1));
            float* rp = S.shadow + S.m.record(c0 + l, r);
            if (whole) {
#pragma unroll
                for (int j = 0; j < 4 - DIM; ++j) vl[u][DIM + j] = fl[u][j];
                *reinterpret_cast<float4*>(rp) = make_float4(vl[u][0], vl[u][1], vl[u][2], vl[u][3]);
            } else if (comps == 2) {
                *reinterpret_cast<float2*>(rp) = make_float2(vl[u][0], vl[u][1]);
            } else {
#pragma unroll
                for (int d = 0; d < DIM; ++d) rp[d] = vl[u][d];
                for (int j = 0; j < A.n; ++j) rp[DIM + j] = A.a[j][al[u]];
            }
        }
    }
    __syncwarp();
    const int64_t c = c0 + lane;
    if (c < nc) {
        S.m.L(c) = L;
        S.m.R(c) = 0;
        S.m.U(c) = 0;
        S.m.L0(c) = L;
        S.m.M(c) = movers[w][lane];
        if (DIM == 2) {  // bit j of a mover's neighbour code in plane j
            uint64_t P[4] = {0, 0, 0, 0}, RT = 0;
#pragma unroll
            for (int k = 0; k < 9; ++k) {
                const uint64_t t = tmask[w][k][lane];
                RT |= t;
#pragma unroll
                for (int j = 0; j < 4; ++j)
                    if ((k >> j) & 1) P[j] |= t;
            }
#pragma unroll
            for (int j = 0; j < 4; ++j) S.m.P(c, j) = P[j];
            S.m.RT(c) = RT;
            S.m.UN(c) = 0;  // a renormalised offset lies inside its new cell
        }
    }
    add_move_counts(g.counts, n_exit, n_far, 0);
    raise_err(d_err, errs);
}

template <int DIM>
__global__ void __launch_bounds__(kThreads)
    move_apply_f32(DevGrid g, XiF Xi, uint8_t* __restrict__ index, ArgsF A, MoveViewF S)
{
    const int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t nc = g.ncells;
    const bool valid = c < nc;
    uint64_t L0 = 0, L = 0, R = 0;
    if (valid) {
        L0 = S.m.L0(c);
        L = S.m.L(c);
        R = S.m.R(c);
    }
    const uint64_t changed = (L0 & ~L) | R;
    const uint32_t hi_any = __reduce_max_sync(0xffffffffu, changed ? 64u - (uint32_t)__clzll((long long)changed) : 0u);
    if (hi_any == 0) return;
    int64_t I[3] = {0, 0, 0};
    if (valid) cell_coords(g, c, I);
    const int comps = S.m.comps;
    if (comps == 4 || comps == 2) {
        // eight slot rows per step, the warp still on the same row at a time (stores of
        // one row share sectors); the rows' origin tags, then their records, are
        // loaded together, so a step waits for two loads instead of two per row
        constexpr int B = 8;
        for (int s0 = 0; s0 < (int)hi_any; s0 += B) {
            bool ch[B], rf[B];
            uint16_t tag[B];
#pragma unroll
            for (int u = 0; u < B; ++u) {
                const int s = s0 + u;
                ch[u] = s < (int)hi_any && ((changed >> s) & 1);
                rf[u] = ch[u] && ((R >> s) & 1);
                tag[u] = rf[u] ? S.m.orig[c + nc * s] : (uint16_t)0;
            }
            float v[B][4];
#pragma unroll
            for (int u = 0; u < B; ++u) {
#pragma unroll
                for (int k = 0; k < 4; ++k) v[u][k] = CUDART_NAN_F;  // a vacated slot
                if (!rf[u]) continue;
                int off[3];
                nb_offset<DIM>(tag[u] & 0x1F, off);
                const int64_t J[3] = {I[0] + off[0], I[1] + off[1], DIM == 3 ? I[2] + off[2] : 0};
                const float* rec = S.shadow + S.m.record(cell_linear<DIM>(g, J), tag[u] >> 5);
                if (comps == 4) {
                    const float4 r4 = *reinterpret_cast<const float4*>(rec);
                    v[u][0] = r4.x;
                    v[u][1] = r4.y;
                    v[u][2] = r4.z;
                    v[u][3] = r4.w;
                } else {
                    const float2 r2 = *reinterpret_cast<const float2*>(rec);
                    v[u][0] = r2.x;
                    v[u][1] = r2.y;
                }
            }
#pragma unroll
            for (int u = 0; u < B; ++u) {
                if (!ch[u]) continue;
                const int64_t a = c + nc * (s0 + u);
#pragma unroll
                for (int d = 0; d < DIM; ++d) Xi.x[d][a] = v[u][d];
#pragma unroll
                for (int k = 0; k < 4 - DIM; ++k)
                    if (k < A.n) A.a[k][a] = v[u][DIM + k];
                index[a] = rf[u] ? 1 : 0;
            }
        }
        return;
    }
    for (int s = 0; s < (int)hi_any; ++s) {
        if (!((changed >> s) & 1)) continue;
        const int64_t a = c + nc * s;
        if ((R >> s) & 1) {
            const uint16_t tag = S.m.orig[a];
            int off[3];
            nb_offset<DIM>(tag & 0x1F, off);
            const int64_t J[3] = {I[0] + off[0], I[1] + off[1], DIM == 3 ? I[2] + off[2] : 0};
            const float* rec = S.shadow + S.m.record(cell_linear<DIM>(g, J), tag >> 5);
            if (comps == 4) {  // the whole 16-byte record in one load
                const float4 r4 = *reinterpret_cast<const float4*>(rec);
                const float v[4] = {r4.x, r4.y, r4.z, r4.w};
#pragma unroll
                for (int d = 0; d < DIM; ++d) Xi.x[d][a] = v[d];
#pragma unroll
                for (int k = 0; k < 4 - DIM; ++k)
                    if (k < A.n) A.a[k][a] = v[DIM + k];
            } else if (comps == 2) {
                const float2 r2 = *reinterpret_cast<const float2*>(rec);
                Xi.x[0][a] = r2.x;
                Xi.x[1][a] = r2.y;
            } else {
#pragma unroll
                for (int d = 0; d < DIM; ++d) Xi.x[d][a] = rec[d];
                for (int k = 0; k < A.n; ++k) A.a[k][a] = rec[DIM + k];
            }
            index[a] = 1;
        } else {
#pragma unroll
            for (int d = 0; d < DIM; ++d) Xi.x[d][a] = CUDART_NAN_F;
            for (int k = 0; k < A.n; ++k) A.a[k][a] = CUDART_NAN_F;
            index[a] = 0;
        }
    }
}

// ------------------------------------------------------------- injection
struct InjectListsF {
    int* counts;
    int* list;
    uint64_t* lm;  // occupancy mask per cell
    int64_t off[8];
};

template <int DIM>
__global__ void __launch_bounds__(kThreads)
    inject_flag_f32(DevGrid g, CXiF Xi, const uint8_t* __restrict__ index, InjectListsF Ls)
{
    const int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int lane = threadIdx.x & 31;
    bool flag = false;
    int col = 0;
    if (c < g.ncells) {
        int64_t I[3];
        cell_coords(g, c, I);
        col = (int)(I[0] & 1) + 2 * (int)(I[1] & 1) + (DIM == 3 ? 4 * (int)(I[2] & 1) : 0);
        const int64_t nc = g.ncells;
        const int min_xq = (g.min_xcell + (1 << DIM) - 1) >> DIM;
        // the cell's occupancy mask, kept for the passes' neighbourhood staging
        const uint64_t live = live_mask(index, c, nc, g.max_xcell);
        Ls.lm[c] = live;
        int count = 0;  // live particles in the first quadrant, counted until min_xq is reached
        constexpr int B = 8;  // slots per step, their loads in flight together (4: 3% slower at C3)
        for (uint64_t m = live; m && count < min_xq;) {
            float xs[B][DIM];
            bool lv[B];
#pragma unroll
            for (int u = 0; u < B; ++u) {
                lv[u] = m != 0;
                const int64_t a = c + nc * (lv[u] ? __ffsll((long long)m) - 1 : 0);
                m &= m - 1;
#pragma unroll
                for (int d = 0; d < DIM; ++d) xs[u][d] = lv[u] ? Xi.x[d][a] : 0.0f;
            }
#pragma unroll
            for (int u = 0; u < B; ++u) {
                bool in = lv[u];
#pragma unroll
                for (int d = 0; d < DIM; ++d) in = in && xs[u][d] > 0.0f && xs[u][d] < 0.5f;
                count += in ? 1 : 0;
            }
        }
        flag = count < min_xq;
    }
    const unsigned active = __ballot_sync(0xffffffffu, flag);
    if (flag) {
        const unsigned grp = __match_any_sync(active, col);
        const int leader = __ffs(grp) - 1;
        const int rank = __popc(grp & ((1u << lane) - 1u));
        int base = 0;
        if (lane == leader) base = atomicAdd(&Ls.counts[col], __popc(grp));
        base = __shfl_sync(grp, base, leader);
        Ls.list[Ls.off[col] + base + rank] = (int)c;
    }
}

template <int DIM>
__host__ __device__ __forceinline__ size_t hood_bytes_f32(int M)
{
    const int n = (DIM == 2 ? 9 : 27) * M;
    const size_t bytes = (size_t)n * (DIM * sizeof(float) + 1);
    return (bytes + 15) & ~(size_t)15;
}

// One flagged cell per warp. The cell's own particles are staged in shared
// memory (offsets in its units); a neighbour cell is staged only when a new
// particle's search needs it. The nearest neighbour of a new particle is the
// first minimum of the FP32 squared physical distance in candidate order
// (neighbour cells k -> j -> i, slots in order): the search scans the own
// cell, then every neighbour whose lower bound (the gap from the new particle
// to that neighbour's side of the cell, per axis, squared and summed, less a
// relative 2^-18 for the rounding of the candidates' own distances) does not
// exceed the best squared distance found there. A skipped neighbour holds no
// candidate at or below that distance, so the minimum and its tie order are
// those of the full scan.
template <int DIM>
__device__ void inject_cell_warp_f32(const DevGrid& g, const F32Params& P, const XiF& Xi,
                                     uint8_t* __restrict__ index, uint64_t* lm, const ArgsF& A, uint32_t call,
                                     int64_t c, float* const* r, uint8_t* live, int lane, int* errs)
{
    const unsigned full = 0xffffffffu;
    const int64_t nc = g.ncells;
    const int M = g.max_xcell;
    constexpr int NB = DIM == 2 ? 9 : 27;
    constexpr int CENTER = DIM == 2 ? 4 : 13;
    const int ncand = NB * M;
    int64_t I[3];
    cell_coords(g, c, I);
    // this cell's widths and its neighbours' widths in its units (1 on a uniform grid)
    float h[3], rl[3], rh[3];
#pragma unroll
    for (int d = 0; d < DIM; ++d) {
        h[d] = P.cells ? __ldg(P.ax.dxf[d] + I[d]) : P.dx[d];
        rl[d] = P.cells ? __ldg(P.ax.nbl[d] + I[d]) : 1.0f;
        rh[d] = P.cells ? __ldg(P.ax.nbr[d] + I[d]) : 1.0f;
    }
    // lane nb < NB: neighbour nb's cell and occupancy (the flag pass's per-cell masks)
    int64_t nbc = 0;
    uint64_t nbm = 0;
    int nbo[3] = {0, 0, 0};
    if (lane < NB) {
        nbo[0] = lane % 3 - 1;
        nbo[1] = (lane / 3) % 3 - 1;
        nbo[2] = DIM == 3 ? lane / 9 - 1 : 0;
        const int64_t J[3] = {I[0] + nbo[0], I[1] + nbo[1], DIM == 3 ? I[2] + nbo[2] : 0};
        const bool ok = J[0] >= 0 && J[1] >= 0 && J[0] < g.n[0] && J[1] < g.n[1] &&
                        (DIM == 2 || (J[2] >= 0 && J[2] < g.n[2]));
        if (ok) {
            nbc = cell_linear<DIM>(g, J);
            nbm = lm[nbc];
        }
    }
    // Stage the neighbours in `want` (a warp-uniform set): positions in this cell's
    // units, loads of a batch in flight together, rounds holding no wanted cell skipped.
    auto stage = [&](uint32_t want) {
        // loads per lane in flight: 2 in 2D (fewer registers, more resident warps: 0.51 -> 0.46 ms
        // at 1024^2), 8 in 3D (occupancy there is held by the shared-memory staging)
        constexpr int B = DIM == 2 ? 2 : 8;
        for (int bo = 0; bo < ncand; bo += 32 * B) {
            const int nlo = bo / M, nhi = min(NB - 1, (bo + 32 * B - 1) / M);
            if (!((want >> nlo) & (0xffffffffu >> (31 - (nhi - nlo))))) continue;
            float xs[B][DIM];
            bool lv[B], in[B];
#pragma unroll
            for (int u = 0; u < B; ++u) {
                const int o = bo + 32 * u + lane;
                const int nb = o / M, sl = o - nb * M;
                const uint64_t m = __shfl_sync(full, nbm, nb < NB ? nb : 0);
                const int64_t cc = __shfl_sync(full, nbc, nb < NB ? nb : 0);
                in[u] = o < ncand && ((want >> nb) & 1u);
                lv[u] = in[u] && ((m >> sl) & 1ull);
                if (lv[u]) {
#pragma unroll
                    for (int d = 0; d < DIM; ++d) xs[u][d] = Xi.x[d][cc + nc * sl];
                }
            }
#pragma unroll
            for (int u = 0; u < B; ++u) {
                if (!in[u]) continue;
                const int o = bo + 32 * u + lane;
                const int nb = o / M;
                const int off[3] = {nb % 3 - 1, (nb / 3) % 3 - 1, DIM == 3 ? nb / 9 - 1 : 0};
                if (lv[u]) {  // x of cell i-1 -> (x - 1) dx[i-1] / dx[i]; of cell i+1 -> 1 + x dx[i+1] / dx[i]
#pragma unroll
                    for (int d = 0; d < DIM; ++d)
                        r[d][o] = off[d] < 0 ? (xs[u][d] - 1.0f) * rl[d]
                                             : (off[d] > 0 ? fmaf(xs[u][d], rh[d], 1.0f) : xs[u][d]);
                }
                live[o] = lv[u] ? 1 : 0;
            }
        }
        __syncwarp();
    };
    // lexicographic (squared distance, candidate) minimum over the neighbours in `set`
    auto scan = [&](uint32_t set, const float* pn, int self, float& best, int& bo) {
        float lb = CUDART_INF_F;
        int lo = 0x7fffffff;
        for (uint32_t m = set; m; m &= m - 1) {
            const int nb = __ffs(m) - 1;
            for (int sl = lane; sl < M; sl += 32) {
                const int o = nb * M + sl;
                if (!live[o] || o == self) continue;
                float ss = 0.0f;
#pragma unroll
                for (int d = 0; d < DIM; ++d) {
                    const float e = (r[d][o] - pn[d]) * h[d];
                    ss = fmaf(e, e, ss);
                }
                if (ss < lb || (ss == lb && o < lo)) {  // NaN never wins
                    lb = ss;
                    lo = o;
                }
            }
        }
#pragma unroll
        for (int sh = 16; sh > 0; sh >>= 1) {
            const float ob = __shfl_xor_sync(full, lb, sh);
            const int oo = __shfl_xor_sync(full, lo, sh);
            if (ob < lb || (ob == lb && oo < lo)) {
                lb = ob;
                lo = oo;
            }
        }
        if (lb < best || (lb == best && lo < bo)) {
            best = lb;
            bo = lo;
        }
    };
    uint32_t staged = 1u << CENTER;
    stage(staged);
    const int min_xq = (g.min_xcell + (1 << DIM) - 1) >> DIM;
    const int base = CENTER * M;
    for (int q = 0; q < (1 << DIM); ++q) {
        float qc[3];
#pragma unroll
        for (int d = 0; d < DIM; ++d) qc[d] = 0.5f * (float)((q >> d) & 1);
        int cnt = 0;
        for (int s = lane; s < M; s += 32) {
            if (!live[base + s]) continue;
            bool in = true;
#pragma unroll
            for (int d = 0; d < DIM; ++d) in = in && r[d][base + s] > qc[d] && r[d][base + s] < qc[d] + 0.5f;
            cnt += in ? 1 : 0;
        }
        int count = __reduce_add_sync(full, cnt);
        if (count >= min_xq) break;
        const bool f0 = lane < M && !live[base + lane];
        const bool f1 = lane + 32 < M && !live[base + lane + 32];
        uint64_t freem = (uint64_t)__ballot_sync(full, f0) | ((uint64_t)__ballot_sync(full, f1) << 32);
        constexpr int SPB = 32 / DIM;  // new particles per batch of draws
        int k = 0;
        float ub = 0.0f;
        while (freem) {
            if (k % SPB == 0)
                ub = batch_draws<DIM, float>(freem, lane, [&](int slot, int d) {
                    return jp_rand_uniform_f32(g.seed, JP_RNG_STREAM_INJECT, call, (uint64_t)c, (uint32_t)slot,
                                               (uint32_t)d);
                });
            const int i = __ffsll((long long)freem) - 1;
            freem &= freem - 1;
            ++count;
            float pn[3];
#pragma unroll
            for (int d = 0; d < DIM; ++d) {
                const float u = __shfl_sync(full, ub, (k % SPB) * DIM + d);
                pn[d] = qc[d] + 0.5f * fmaf(0.95f, u, 0.05f);
            }
            ++k;
            const int64_t ai = c + nc * i;
            if (lane == 0) {
#pragma unroll
                for (int d = 0; d < DIM; ++d) {
                    Xi.x[d][ai] = pn[d];
                    r[d][base + i] = pn[d];
                }
                index[ai] = 1;
                live[base + i] = 1;
            }
            __syncwarp();
            float best = CUDART_INF_F;
            int bo = 0x7fffffff;
            scan(1u << CENTER, pn, base + i, best, bo);
            // the neighbours that may hold a candidate at or below the best so far: pn lies in
            // (0, 1) on every axis, so the gap to neighbour side -1 is pn, to side +1 is 1 - pn
            bool need = false;
            if (lane < NB && lane != CENTER && nbm != 0) {
                float lbd = 0.0f;
#pragma unroll
                for (int d = 0; d < DIM; ++d) {
                    const float gap = nbo[d] < 0 ? pn[d] : (nbo[d] > 0 ? 1.0f - pn[d] : 0.0f);
                    const float e = gap * h[d];
                    lbd = fmaf(e, e, lbd);
                }
                need = lbd * (1.0f - 0x1p-18f) <= best;
            }
            const uint32_t S = __ballot_sync(full, need);
            if (S & ~staged) {
                stage(S & ~staged);
                staged |= S;
            }
            scan(S, pn, base + i, best, bo);
            if (bo != 0x7fffffff) {
                const int nb = bo / M, sl = bo - nb * M;
                const int64_t J[3] = {I[0] + nb % 3 - 1, I[1] + (nb / 3) % 3 - 1, DIM == 3 ? I[2] + nb / 9 - 1 : 0};
                const int64_t src = cell_linear<DIM>(g, J) + nc * sl;
                for (int k = lane; k < A.n; k += 32) A.a[k][ai] = A.a[k][src];
            } else if (A.n > 0) {
                *errs |= kWarnNoNeighbour;
            }
            __syncwarp();
            if (count >= min_xq) break;
        }
    }
    // the cell's occupancy after its injections, for the later passes' staging
    __syncwarp();
    const bool o0 = lane < M && live[base + lane];
    const bool o1 = lane + 32 < M && live[base + lane + 32];
    const uint64_t own = (uint64_t)__ballot_sync(full, o0) | ((uint64_t)__ballot_sync(full, o1) << 32);
    if (lane == 0) lm[c] = own;
}

// A colour pass: warps take the colour's flagged cells in turn.
template <int DIM>
__device__ __forceinline__ void inject_pass_f32_body(const DevGrid& g, const F32Params& P, const XiF& Xi,
                                                     uint8_t* __restrict__ index, const ArgsF& A,
                                                     const InjectListsF& Ls, int col, uint32_t call, int* d_err)
{
    extern __shared__ __align__(16) unsigned char smem_f32[];
    const int lane = threadIdx.x & 31;
    const int wib = threadIdx.x >> 5;
    const int M = g.max_xcell;
    const int ncand = (DIM == 2 ? 9 : 27) * M;
    unsigned char* base = smem_f32 + (size_t)wib * hood_bytes_f32<DIM>(M);
    float* r[3];
#pragma unroll
    for (int d = 0; d < DIM; ++d) r[d] = (float*)base + (size_t)d * ncand;
    uint8_t* live = base + (size_t)DIM * ncand * sizeof(float);
    const int nwarps = (gridDim.x * blockDim.x) >> 5;
    const int gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int count = Ls.counts[col];
    int errs = 0;
    for (int k = gw; k < count; k += nwarps) {
        const int64_t c = Ls.list[Ls.off[col] + k];
        inject_cell_warp_f32<DIM>(g, P, Xi, index, Ls.lm, A, call, c, r, live, lane, &errs);
        __syncwarp();
    }
    raise_err(d_err, errs);
}

// 3D: three blocks of four warps per SM, held there by the shared-memory staging
template <int DIM>
__global__ void inject_pass_f32(DevGrid g, F32Params P, XiF Xi, uint8_t* __restrict__ index, ArgsF A,
                                InjectListsF Ls, int col, uint32_t call, int* d_err)
{
    inject_pass_f32_body<DIM>(g, P, Xi, index, A, Ls, col, call, d_err);
}

// 2D: six blocks of four warps per SM (80 registers, no spills; a sweep of 5..8 blocks
// at C2 gave 0.374, 0.364, 0.363, 0.364 ms per call)
template <>
__global__ void __launch_bounds__(128, 6)
    inject_pass_f32<2>(DevGrid g, F32Params P, XiF Xi, uint8_t* __restrict__ index, ArgsF A, InjectListsF Ls,
                       int col, uint32_t call, int* d_err)
{
    inject_pass_f32_body<2>(g, P, Xi, index, A, Ls, col, call, d_err);
}

// ------------------------------------------------------- grid2particle!
// One thread per cell (its corner values in registers), a warp on 32
// consecutive cells walking the slot rows up to its highest live slot, four
// rows in flight per lane: every load and store is a coalesced row access.
template <int DIM, bool WIDE>
__global__ void __launch_bounds__(kThreads)
    g2p_f32_kernel(DevGrid g, float* __restrict__ Fp, const float* __restrict__ F, CXiF Xi,
                   const uint8_t* __restrict__ index)
{
    const int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t nc = g.ncells;
    const bool valid = c < nc;
    const int M = g.max_xcell;
    float cv[1 << DIM];
    uint64_t L = 0;
    {
        int64_t I[3];
        cell_coords(g, valid ? c : nc - 1, I);
        const int64_t V0 = g.n[0] + 1, V1 = g.n[1] + 1;
        const float* b = F + I[0] + V0 * (I[1] + (DIM == 3 ? V1 * I[2] : 0));
        cv[0] = __ldg(b);
        cv[1] = __ldg(b + 1);
        cv[2] = __ldg(b + V0);
        cv[3] = __ldg(b + V0 + 1);
        if (DIM == 3) {
            const int64_t sz = V0 * V1;
            cv[4] = __ldg(b + sz);
            cv[5] = __ldg(b + sz + 1);
            cv[6] = __ldg(b + sz + V0);
            cv[7] = __ldg(b + sz + V0 + 1);
        }
    }
    for (int q0 = 0; q0 < (WIDE ? M : 1); q0 += 64) {  // WIDE: slots in chunks of 64 (max_xcell > 64)
        if (valid) L = live_mask(index + nc * q0, c, nc, min(64, M - q0));
        const int hi = (int)__reduce_max_sync(0xffffffffu, L ? 64u - (uint32_t)__clzll((long long)L) : 0u);
        constexpr int B = 4;
        for (int s0 = 0; s0 < hi; s0 += B) {
            float t[B][3];
            bool lv[B];
#pragma unroll
            for (int u = 0; u < B; ++u) {
                const int s = s0 + u;
                lv[u] = s < hi && ((L >> s) & 1);
#pragma unroll
                for (int d = 0; d < DIM; ++d) t[u][d] = lv[u] ? Xi.x[d][c + nc * (q0 + s)] : 0.0f;
            }
#pragma unroll
            for (int u = 0; u < B; ++u)
                if (lv[u]) Fp[c + nc * (q0 + s0 + u)] = lerpNf<DIM>(cv, t[u]);
        }
    }
}

// ------------------------------------------------------- particle2grid!
// The FP64 form's accumulation order (per vertex: cells with the offsets of
// the last axis outermost, x innermost, slots in order); weights in FP32, their sums (and the weighted field sums) at FP64 accuracy: within one
// cell the terms are summed as compensated FP32 pairs (error-free TwoSum and
// TwoProduct, Knuth / Dekker), and each cell's pair is added to the vertex's
// FP64 accumulators. For the <= 64 terms of a cell the pair keeps the sum to
// about 2^-42 relative, so the result matches FP64 summation to far below the
// FP32 weights' own rounding, at a few FP64 operations per cell instead of two
// per particle (GB300 issues FP64 at 1/64 of its FP32 rate).
struct CSum {
    float h = 0.0f, l = 0.0f;
};

// s += x with the rounding error kept in s.l (TwoSum; needs -fmad=false)
__device__ __forceinline__ void csum_add(CSum& s, float x)
{
    const float t = s.h + x;
    const float bp = t - s.h;
    const float err = (s.h - (t - bp)) + (x - bp);
    s.h = t;
    s.l += err;
}

// s += a * b, the product's rounding error (exact by fmaf) added to s.l
__device__ __forceinline__ void csum_add_prod(CSum& s, float a, float b)
{
    const float p = a * b;
    const float e = fmaf(a, b, -p);
    csum_add(s, p);
    s.l += e;
}

__device__ __forceinline__ double csum_value(const CSum& s) { return (double)s.h + (double)s.l; }

// Cell-centric form of the same sums: one lane per cell, a warp on 32
// consecutive cells of a cell row (lane 0 is the column to the left of the
// warp's vertex columns), marching up the rows of a band. The warp walks each
// cell row's slot rows up to its highest live slot (coalesced rows, four in
// flight per lane), so every particle is read once per band; per particle it
// forms the weights of the cell's 2^N corners and adds them to one compensated
// pair per corner, in slot order (the pair of a (vertex, cell)). A vertex then
// adds its cells' pairs in the reference's cell order in FP64: the lower
// corners of a cell row finish the vertex row below it, the upper corners
// start the row above. No cell is read again for each of its vertices.
__device__ __forceinline__ float p2g_w_f32(float qx, float e) { return p2g_weight_f32(fmaf(e, e, qx)); }

template <bool WIDE>
__global__ void __launch_bounds__(kThreads)
    p2g_f32_cells2d(DevGrid g, F32Params P, float* __restrict__ F, const float* __restrict__ Fp, CXiF Xi,
                    const uint8_t* __restrict__ index, int chunk, double* __restrict__ Wout)
{
    const unsigned full = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    const int64_t warp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int64_t n0 = g.n[0], n1 = g.n[1], V0 = n0 + 1, nc = g.ncells;
    const int64_t wcols = (V0 + 30) / 31;
    const int64_t band = warp / wcols, wc = warp - band * wcols;
    const int64_t r0 = band * chunk;
    if (r0 > n1) return;  // the whole warp
    const int64_t r1 = min(r0 + (int64_t)chunk, n1 + 1);  // vertex rows [r0, r1)
    const int64_t ci = wc * 31 + lane - 1;                 // this lane's cell column
    const bool col_ok = ci >= 0 && ci < n0;
    const bool out_ok = lane >= 1 && ci < V0;             // lanes 1..31 own vertex column ci
    const int M = g.max_xcell;
    const float dx = P.cells && col_ok ? __ldg(P.ax.dxf[0] + ci) : P.dx[0];
    double w_acc = 0.0, f_acc = 0.0;  // the vertex (ci, cr) being summed
    for (int64_t cr = r0 - 1; cr < r1; ++cr) {
        const bool cell_ok = col_ok && cr >= 0 && cr < n1;
        const float dy = P.cells && cr >= 0 && cr < n1 ? __ldg(P.ax.dxf[1] + cr) : P.dx[1];
        const int64_t c = cell_ok ? ci + n0 * cr : 0;
        // corners (0,0), (1,0), (0,1), (1,1) of the cell in cell units
        CSum w00, f00, w10, f10, w01, f01, w11, f11;
        for (int q0 = 0; q0 < (WIDE ? M : 1); q0 += 64) {  // WIDE: slots in chunks of 64 (max_xcell > 64)
            const uint64_t L = cell_ok ? live_mask(index + nc * q0, c, nc, min(64, M - q0)) : 0;
            const int hi = (int)__reduce_max_sync(full, L ? 64u - (uint32_t)__clzll((long long)L) : 0u);
            constexpr int B = 4;
            for (int s0 = 0; s0 < hi; s0 += B) {
                float x[B], y[B], f[B];
                bool lv[B];
#pragma unroll
                for (int u = 0; u < B; ++u) {
                    const int s = s0 + u;
                    lv[u] = s < hi && ((L >> s) & 1);
                    const int64_t a = c + nc * (q0 + s);
                    x[u] = lv[u] ? Xi.x[0][a] : 0.0f;
                    y[u] = lv[u] ? Xi.x[1][a] : 0.0f;
                    f[u] = lv[u] ? Fp[a] : 0.0f;
                }
#pragma unroll
                for (int u = 0; u < B; ++u) {
                    if (!lv[u]) continue;
                    // distance^2 = fmaf(ey, ey, ex * ex), e = (corner - xi) * dx per axis
                    const float ex0 = (0.0f - x[u]) * dx, ex1 = (1.0f - x[u]) * dx;
                    const float ey0 = (0.0f - y[u]) * dy, ey1 = (1.0f - y[u]) * dy;
                    const float qx0 = fmaf(ex0, ex0, 0.0f), qx1 = fmaf(ex1, ex1, 0.0f);
                    const float a00 = p2g_w_f32(qx0, ey0), a10 = p2g_w_f32(qx1, ey0);
                    const float a01 = p2g_w_f32(qx0, ey1), a11 = p2g_w_f32(qx1, ey1);
                    csum_add(w00, a00);
                    csum_add_prod(f00, a00, f[u]);
                    csum_add(w10, a10);
                    csum_add_prod(f10, a10, f[u]);
                    csum_add(w01, a01);
                    csum_add_prod(f01, a01, f[u]);
                    csum_add(w11, a11);
                    csum_add_prod(f11, a11, f[u]);
                }
            }
        }
        // vertex (ci, cr), the lower side of this cell row: its cells (ci-1, cr-1) and (ci, cr-1) are in
        // the accumulators; (ci-1, cr) [corner (1,0) of the lane to the left] and (ci, cr) [corner (0,0)] follow
        const double lw10 = __shfl_up_sync(full, csum_value(w10), 1), lf10 = __shfl_up_sync(full, csum_value(f10), 1);
        if (cr >= r0) {
            w_acc += lw10;
            f_acc += lf10;
            w_acc += csum_value(w00);
            f_acc += csum_value(f00);
            if (out_ok) {
                const int64_t v = ci + V0 * cr;
                F[v] = (float)(f_acc / w_acc);
                if (Wout) Wout[v] = w_acc;
            }
        }
        // vertex (ci, cr + 1), the upper side: (ci-1, cr) [corner (1,1) to the left], then (ci, cr) [corner (0,1)]
        const double lw11 = __shfl_up_sync(full, csum_value(w11), 1), lf11 = __shfl_up_sync(full, csum_value(f11), 1);
        w_acc = 0.0 + lw11;
        f_acc = 0.0 + lf11;
        w_acc += csum_value(w01);
        f_acc += csum_value(f01);
    }
}

// The 3D cell-centric sums: a block of 8 warps covers 8 consecutive cell rows
// along y (warp 0 the row below the block's vertex rows), each warp 32 cells
// along x (lane 0 the column to the left), marching up a band of z rows. Each
// lane forms its cell's 8 corner pairs per z row; a vertex adds, per z row in
// the reference's order, the pairs of its cells (i-1, j-1), (i, j-1) (from the
// warp below, through shared memory), (i-1, j) (the lane to the left) and
// (i, j) (its own): the lower corners finish the vertex row of this z row, the
// upper corners start the next one.
template <bool WIDE>
__global__ void __launch_bounds__(kThreads, 4)
    p2g_f32_cells3d(DevGrid g, F32Params P, float* __restrict__ F, const float* __restrict__ Fp, CXiF Xi,
                    const uint8_t* __restrict__ index, int band, double* __restrict__ Wout)
{
    // the corners (cx, 1, cz) of every lane's cell, as (w, wF): [warp][lane][cx][cz][2]
    __shared__ double up[kWarpsPerBlock][32][2][2][2];
    const unsigned full = 0xffffffffu;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int64_t n0 = g.n[0], n1 = g.n[1], n2 = g.n[2], V0 = n0 + 1, V1 = n1 + 1, nc = g.ncells;
    const int64_t wcols = (V0 + 30) / 31, jgroups = (V1 + 6) / 7;
    const int64_t b = blockIdx.x;
    const int64_t wc = b % wcols, jg = (b / wcols) % jgroups, kb = b / (wcols * jgroups);
    const int64_t r0 = kb * band;
    if (r0 > n2) return;  // the whole block
    const int64_t r1 = min(r0 + (int64_t)band, n2 + 1);  // vertex rows along z: [r0, r1)
    const int64_t ci = wc * 31 + lane - 1, cj = jg * 7 + w - 1;
    const bool colrow_ok = ci >= 0 && ci < n0 && cj >= 0 && cj < n1;
    const bool out_ok = lane >= 1 && w >= 1 && ci < V0 && cj < V1;  // vertex (ci, cj, .)
    const int M = g.max_xcell;
    const float dx = P.cells && ci >= 0 && ci < n0 ? __ldg(P.ax.dxf[0] + ci) : P.dx[0];
    const float dy = P.cells && cj >= 0 && cj < n1 ? __ldg(P.ax.dxf[1] + cj) : P.dx[1];
    double w_acc = 0.0, f_acc = 0.0;
    for (int64_t cr = r0 - 1; cr < r1; ++cr) {
        const bool cell_ok = colrow_ok && cr >= 0 && cr < n2;
        const float dz = P.cells && cr >= 0 && cr < n2 ? __ldg(P.ax.dxf[2] + cr) : P.dx[2];
        const int64_t c = cell_ok ? ci + n0 * (cj + n1 * cr) : 0;
        CSum cw[2][2][2], cf[2][2][2];  // [cx][cy][cz]
        for (int q0 = 0; q0 < (WIDE ? M : 1); q0 += 64) {  // WIDE: slots in chunks of 64 (max_xcell > 64)
            const uint64_t L = cell_ok ? live_mask(index + nc * q0, c, nc, min(64, M - q0)) : 0;
            const int hi = (int)__reduce_max_sync(full, L ? 64u - (uint32_t)__clzll((long long)L) : 0u);
            constexpr int B = 2;  // rows in flight per lane (2 measured 6% faster than 4 at 128^3)
            for (int s0 = 0; s0 < hi; s0 += B) {
                float x[B], y[B], z[B], f[B];
                bool lv[B];
#pragma unroll
                for (int u = 0; u < B; ++u) {
                    const int s = s0 + u;
                    lv[u] = s < hi && ((L >> s) & 1);
                    const int64_t a = c + nc * (q0 + s);
                    x[u] = lv[u] ? Xi.x[0][a] : 0.0f;
                    y[u] = lv[u] ? Xi.x[1][a] : 0.0f;
                    z[u] = lv[u] ? Xi.x[2][a] : 0.0f;
                    f[u] = lv[u] ? Fp[a] : 0.0f;
                }
#pragma unroll
                for (int u = 0; u < B; ++u) {
                    if (!lv[u]) continue;
                    float qx[2], ey[2], ez[2];
#pragma unroll
                    for (int k = 0; k < 2; ++k) {
                        const float ex = ((float)k - x[u]) * dx;
                        qx[k] = fmaf(ex, ex, 0.0f);
                        ey[k] = ((float)k - y[u]) * dy;
                        ez[k] = ((float)k - z[u]) * dz;
                    }
#pragma unroll
                    for (int kx = 0; kx < 2; ++kx)
#pragma unroll
                        for (int ky = 0; ky < 2; ++ky) {
                            const float qxy = fmaf(ey[ky], ey[ky], qx[kx]);
#pragma unroll
                            for (int kz = 0; kz < 2; ++kz) {
                                const float wi = p2g_weight_f32(fmaf(ez[kz], ez[kz], qxy));
                                csum_add(cw[kx][ky][kz], wi);
                                csum_add_prod(cf[kx][ky][kz], wi, f[u]);
                            }
                        }
                }
            }
        }
#pragma unroll
        for (int kx = 0; kx < 2; ++kx)
#pragma unroll
            for (int kz = 0; kz < 2; ++kz) {
                up[w][lane][kx][kz][0] = csum_value(cw[kx][1][kz]);
                up[w][lane][kx][kz][1] = csum_value(cf[kx][1][kz]);
            }
        __syncthreads();
        const int wb = w >= 1 ? w - 1 : 0, lb = lane >= 1 ? lane - 1 : 0;
#pragma unroll
        for (int kz = 0; kz < 2; ++kz) {
            // cells (i-1, j-1), (i, j-1), (i-1, j), (i, j) of this z row, lower (kz = 0) or upper (kz = 1) corners
            const double a_w = up[wb][lb][1][kz][0], a_f = up[wb][lb][1][kz][1];
            const double b_w = up[wb][lane][0][kz][0], b_f = up[wb][lane][0][kz][1];
            const double c_w = __shfl_up_sync(full, csum_value(cw[1][0][kz]), 1);
            const double c_f = __shfl_up_sync(full, csum_value(cf[1][0][kz]), 1);
            if (kz == 0) {
                if (cr >= r0) {
                    w_acc += a_w;
                    f_acc += a_f;
                    w_acc += b_w;
                    f_acc += b_f;
                    w_acc += c_w;
                    f_acc += c_f;
                    w_acc += csum_value(cw[0][0][0]);
                    f_acc += csum_value(cf[0][0][0]);
                    if (out_ok) {
                        const int64_t v = ci + V0 * (cj + V1 * cr);
                        F[v] = (float)(f_acc / w_acc);
                        if (Wout) Wout[v] = w_acc;
                    }
                }
            } else {
                w_acc = 0.0 + a_w;
                f_acc = 0.0 + a_f;
                w_acc += b_w;
                f_acc += b_f;
                w_acc += c_w;
                f_acc += c_f;
                w_acc += csum_value(cw[0][0][1]);
                f_acc += csum_value(cf[0][0][1]);
            }
        }
        __syncthreads();  // the next z row overwrites `up`
    }
}

// ------------------------------------------------- cells above 64 slots
// Containers with max_xcell > 64 do not fit the 64-bit slot masks of the
// move and injection kernels above. They run the colour passes directly, as
// the FP64 form does for such cells: move_particles! with one thread per cell
// walking its slots in order (the starting point of the free-slot search
// carried across the cell's movers), inject_particles! with one warp per cell
// (quadrant counts, free slots and the nearest-neighbour search shared by the
// warp). Same rules and results as the kernels above.
template <int DIM, bool CELLS>
__global__ void __launch_bounds__(kThreads)
    move_wide_f32(DevGrid g, XiF Xi, uint8_t* __restrict__ index, ArgsF A, F32Axes ax, int pass, int* d_err)
{
    int64_t ncol[3] = {1, 1, 1}, off[3] = {0, 0, 0};
#pragma unroll
    for (int d = 0; d < DIM; ++d) ncol[d] = (g.n[d] + 2) / 3;
    if (DIM == 2) {
        off[0] = pass / 3;
        off[1] = pass % 3;
    } else {
        off[0] = pass / 9;
        off[1] = (pass / 3) % 3;
        off[2] = pass % 3;
    }
    const int64_t w = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (w >= ncol[0] * ncol[1] * ncol[2]) return;
    const int64_t J[3] = {w % ncol[0], (w / ncol[0]) % ncol[1], w / (ncol[0] * ncol[1])};
    int I[3] = {0, 0, 0};
#pragma unroll
    for (int d = 0; d < DIM; ++d) {
        const int64_t i = 3 * J[d] + off[d];
        if (i >= g.n[d]) return;
        I[d] = (int)i;
    }
    const int64_t nc = g.ncells;
    const int M = g.max_xcell;
    const int64_t I64[3] = {I[0], I[1], I[2]};
    const int64_t c = cell_linear<DIM>(g, I64);
    int errs = 0, n_exit = 0, n_far = 0, n_full = 0;
    int sp = 0;  // starting point of the free-slot search
    for (int ip = 0; ip < M; ++ip) {
        const int64_t a = c + nc * ip;
        if (!index[a]) continue;
        float xi[3];
        bool out = false;
#pragma unroll
        for (int d = 0; d < DIM; ++d) {
            xi[d] = Xi.x[d][a];
            out |= !(xi[d] >= 0.0f && xi[d] < 1.0f);
        }
        if (!out) continue;
        float v[3];
        int o[3];
        bool inside, far;
        offset_destination<DIM, CELLS>(g, ax, I, xi, v, o, &inside, &far);
        float cached[JP_MAX_ARGS];
        for (int k = 0; k < A.n; ++k) cached[k] = A.a[k][a];
        index[a] = 0;
#pragma unroll
        for (int d = 0; d < DIM; ++d) Xi.x[d][a] = CUDART_NAN_F;
        for (int k = 0; k < A.n; ++k) A.a[k][a] = CUDART_NAN_F;
        if (!inside) {
            ++n_exit;
            continue;
        }
        if (far) {
            errs |= kWarnFarMove;
            ++n_far;
            continue;
        }
        const int64_t T[3] = {I[0] + o[0], I[1] + o[1], DIM == 3 ? I[2] + o[2] : 0};
        const int64_t tc = cell_linear<DIM>(g, T);
        int fr = -1;
        for (int i = sp; i < M; ++i)
            if (!index[tc + nc * i]) {
                fr = i;
                break;
            }
        if (fr < 0) {  // target cell full: dropped
            ++n_full;
            continue;
        }
        sp = fr;
        const int64_t b = tc + nc * fr;
        index[b] = 1;
#pragma unroll
        for (int d = 0; d < DIM; ++d) Xi.x[d][b] = v[d];
        for (int k = 0; k < A.n; ++k) A.a[k][b] = cached[k];
    }
    if ((n_exit | n_far | n_full) && g.counts) {
        if (n_exit) atomicAdd(g.counts + 0, (unsigned long long)n_exit);
        if (n_far) atomicAdd(g.counts + 1, (unsigned long long)n_far);
        if (n_full) atomicAdd(g.counts + 2, (unsigned long long)n_full);
    }
    raise_err(d_err, errs);
}

template <int DIM>
__global__ void __launch_bounds__(32 * kWarpsPerBlock)
    inject_wide_f32(DevGrid g, F32Params P, XiF Xi, uint8_t* __restrict__ index, ArgsF A, int pass, uint32_t call,
                    int* d_err)
{
    int64_t ncol[3] = {1, 1, 1}, off[3] = {0, 0, 0};
#pragma unroll
    for (int d = 0; d < DIM; ++d) ncol[d] = (g.n[d] + 1) / 2;
    if (DIM == 2) {
        off[0] = pass / 2;
        off[1] = pass % 2;
    } else {
        off[0] = pass / 4;
        off[1] = (pass / 2) % 2;
        off[2] = pass % 2;
    }
    const int lane = threadIdx.x & 31;
    const int64_t w = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (w >= ncol[0] * ncol[1] * ncol[2]) return;
    const int64_t J[3] = {w % ncol[0], (w / ncol[0]) % ncol[1], w / (ncol[0] * ncol[1])};
    int64_t I[3] = {0, 0, 0};
#pragma unroll
    for (int d = 0; d < DIM; ++d) {
        I[d] = 2 * J[d] + off[d];
        if (I[d] >= g.n[d]) return;  // the same for the whole warp
    }
    const int64_t nc = g.ncells;
    const int M = g.max_xcell;
    constexpr int NB = DIM == 2 ? 9 : 27;
    constexpr int CENTER = DIM == 2 ? 4 : 13;
    const int64_t c = cell_linear<DIM>(g, I);
    float h[3], rl[3], rh[3];
#pragma unroll
    for (int d = 0; d < DIM; ++d) {
        h[d] = P.cells ? __ldg(P.ax.dxf[d] + I[d]) : P.dx[d];
        rl[d] = P.cells ? __ldg(P.ax.nbl[d] + I[d]) : 1.0f;
        rh[d] = P.cells ? __ldg(P.ax.nbr[d] + I[d]) : 1.0f;
    }
    const int min_xq = (g.min_xcell + (1 << DIM) - 1) >> DIM;
    int errs = 0;
    for (int q = 0; q < (1 << DIM); ++q) {
        float qc[3];
#pragma unroll
        for (int d = 0; d < DIM; ++d) qc[d] = 0.5f * (float)((q >> d) & 1);
        int cnt = 0;
        for (int s = lane; s < M; s += 32) {
            const int64_t a = c + nc * s;
            if (!index[a]) continue;
            bool in = true;
#pragma unroll
            for (int d = 0; d < DIM; ++d) {
                const float x = Xi.x[d][a];
                in = in && x > qc[d] && x < qc[d] + 0.5f;
            }
            cnt += in ? 1 : 0;
        }
        int count = __reduce_add_sync(0xffffffffu, cnt);
        if (count >= min_xq) break;
        bool done = false;
        for (int base = 0; base < M && !done; base += 32) {
            const int s = base + lane;
            uint32_t freem = __ballot_sync(0xffffffffu, s < M && !index[c + nc * s]);
            while (freem) {
                const int i = base + __ffs(freem) - 1;
                freem &= freem - 1;
                ++count;
                float pn[3];
#pragma unroll
                for (int d = 0; d < DIM; ++d) {
                    const float u = jp_rand_uniform_f32(g.seed, JP_RNG_STREAM_INJECT, call, (uint64_t)c, (uint32_t)i,
                                                        (uint32_t)d);
                    pn[d] = qc[d] + 0.5f * fmaf(0.95f, u, 0.05f);
                }
                const int64_t ai = c + nc * i;
                if (lane == 0) {
#pragma unroll
                    for (int d = 0; d < DIM; ++d) Xi.x[d][ai] = pn[d];
                    index[ai] = 1;
                }
                __syncwarp();
                // nearest: first minimum of the FP32 squared physical distance in candidate order
                float best = CUDART_INF_F;
                int bo = 0x7fffffff;
                for (int o = lane; o < NB * M; o += 32) {
                    const int nb = o / M, sl = o - nb * M;
                    if (nb == CENTER && sl == i) continue;
                    const int ox[3] = {nb % 3 - 1, (nb / 3) % 3 - 1, DIM == 3 ? nb / 9 - 1 : 0};
                    const int64_t K[3] = {I[0] + ox[0], I[1] + ox[1], I[2] + ox[2]};
                    if (K[0] < 0 || K[1] < 0 || K[0] >= g.n[0] || K[1] >= g.n[1]) continue;
                    if (DIM == 3 && (K[2] < 0 || K[2] >= g.n[2])) continue;
                    const int64_t b = cell_linear<DIM>(g, K) + nc * sl;
                    if (!index[b]) continue;
                    float ss = 0.0f;
#pragma unroll
                    for (int d = 0; d < DIM; ++d) {
                        const float x = Xi.x[d][b];
                        const float r = ox[d] < 0 ? (x - 1.0f) * rl[d] : (ox[d] > 0 ? fmaf(x, rh[d], 1.0f) : x);
                        const float e = (r - pn[d]) * h[d];
                        ss = fmaf(e, e, ss);
                    }
                    if (ss < best) {  // NaN never wins
                        best = ss;
                        bo = o;
                    }
                }
#pragma unroll
                for (int sh = 16; sh > 0; sh >>= 1) {
                    const float ob = __shfl_xor_sync(0xffffffffu, best, sh);
                    const int oo = __shfl_xor_sync(0xffffffffu, bo, sh);
                    if (ob < best || (ob == best && oo < bo)) {
                        best = ob;
                        bo = oo;
                    }
                }
                if (bo != 0x7fffffff) {
                    const int nb = bo / M, sl = bo - nb * M;
                    const int64_t K[3] = {I[0] + nb % 3 - 1, I[1] + (nb / 3) % 3 - 1,
                                          DIM == 3 ? I[2] + nb / 9 - 1 : 0};
                    const int64_t src = cell_linear<DIM>(g, K) + nc * sl;
                    for (int k = lane; k < A.n; k += 32) A.a[k][ai] = A.a[k][src];
                } else if (A.n > 0) {
                    errs |= kWarnNoNeighbour;
                }
                __syncwarp();
                if (count >= min_xq) {
                    done = true;
                    break;
                }
            }
        }
    }
    raise_err(d_err, errs);
}

// ------------------------------------------------------------ launchers
cudaError_t launch_to_offsets(jp_particles* P, const double* const coords[3], const uint8_t* index,
                              float* const xi[3])
{
    const bool d3 = P->g.ndim == 3;
    CCoords X{{coords[0], coords[1], d3 ? coords[2] : nullptr}};
    XiF Xi{{xi[0], xi[1], d3 ? xi[2] : nullptr}};
    const unsigned nb = grid_blocks(P->g.ncells);
    if (!d3)
        to_offsets<2><<<nb, kThreads, 0, P->stream>>>(P->g, X, index, Xi);
    else
        to_offsets<3><<<nb, kThreads, 0, P->stream>>>(P->g, X, index, Xi);
    return cudaGetLastError();
}

cudaError_t launch_to_coords(jp_particles* P, const float* const xi[3], const uint8_t* index,
                             double* const coords[3])
{
    const bool d3 = P->g.ndim == 3;
    Coords X{{coords[0], coords[1], d3 ? coords[2] : nullptr}};
    CXiF Xi{{xi[0], xi[1], d3 ? xi[2] : nullptr}};
    const unsigned nb = grid_blocks(P->g.ncells);
    if (!d3)
        to_coords<2><<<nb, kThreads, 0, P->stream>>>(P->g, Xi, index, X);
    else
        to_coords<3><<<nb, kThreads, 0, P->stream>>>(P->g, Xi, index, X);
    return cudaGetLastError();
}

cudaError_t launch_advection_f32(jp_particles* P, int method, double alpha, const float* const V[3], double dt,
                                 float* const xi[3], const uint8_t* index)
{
    const bool d3 = P->g.ndim == 3;
    XiF Xi{{xi[0], xi[1], d3 ? xi[2] : nullptr}};
    CVelF Vv{{V[0], V[1], d3 ? V[2] : nullptr}};
    const F32Params prm = make_params(P, alpha, dt);
    const bool wide = P->g.max_xcell > 64;
    const unsigned nb = grid_blocks(P->g.ncells, 32 * kWarpsPerBlock);
    const int nt = 32 * kWarpsPerBlock;
    cudaStream_t s = P->stream;
#define JP_ADVF(D, M)                                                                              \
    (wide ? (prm.cells ? advect_f32_kernel<D, M, true, true><<<nb, nt, 0, s>>>(P->g, Vv, prm, Xi, index)   \
                       : advect_f32_kernel<D, M, false, true><<<nb, nt, 0, s>>>(P->g, Vv, prm, Xi, index)) \
          : (prm.cells ? advect_f32_kernel<D, M, true, false><<<nb, nt, 0, s>>>(P->g, Vv, prm, Xi, index)  \
                       : advect_f32_kernel<D, M, false, false><<<nb, nt, 0, s>>>(P->g, Vv, prm, Xi, index)))
    if (!d3) {
        if (method == JP_RUNGE_KUTTA2) JP_ADVF(2, JP_RUNGE_KUTTA2);
        else if (method == JP_RUNGE_KUTTA4) JP_ADVF(2, JP_RUNGE_KUTTA4);
        else JP_ADVF(2, JP_EULER);
    } else {
        if (method == JP_RUNGE_KUTTA2) JP_ADVF(3, JP_RUNGE_KUTTA2);
        else if (method == JP_RUNGE_KUTTA4) JP_ADVF(3, JP_RUNGE_KUTTA4);
        else JP_ADVF(3, JP_EULER);
    }
#undef JP_ADVF
    return cudaGetLastError();
}

static cudaError_t launch_move_wide_f32(jp_particles* P, float* const xi[3], uint8_t* index, float* const* args,
                                        int nargs)
{
    const int N = P->g.ndim;
    P->move.replayable = 0;  // this move leaves no record in the container's scratch
    XiF Xi{{xi[0], xi[1], N == 3 ? xi[2] : nullptr}};
    ArgsF A{};
    A.n = nargs;
    for (int k = 0; k < nargs; ++k) A.a[k] = args[k];
    int64_t cols = 1;
    for (int d = 0; d < N; ++d) cols *= (P->g.n[d] + 2) / 3;
    const unsigned nb = grid_blocks(cols);
    const F32Axes& ax = P->f32ax;
    const bool cells = P->f32_cells != 0;
    for (int pass = 0; pass < (N == 2 ? 9 : 27); ++pass) {
        if (N == 2) {
            if (cells)
                move_wide_f32<2, true><<<nb, kThreads, 0, P->stream>>>(P->g, Xi, index, A, ax, pass, P->d_err);
            else
                move_wide_f32<2, false><<<nb, kThreads, 0, P->stream>>>(P->g, Xi, index, A, ax, pass, P->d_err);
        } else {
            if (cells)
                move_wide_f32<3, true><<<nb, kThreads, 0, P->stream>>>(P->g, Xi, index, A, ax, pass, P->d_err);
            else
                move_wide_f32<3, false><<<nb, kThreads, 0, P->stream>>>(P->g, Xi, index, A, ax, pass, P->d_err);
        }
    }
    return cudaGetLastError();
}

cudaError_t launch_move_f32(jp_particles* P, float* const xi[3], uint8_t* index, float* const* args, int nargs)
{
    if (P->g.max_xcell > 64) return launch_move_wide_f32(P, xi, index, args, nargs);  // needs no scratch
    const int N = P->g.ndim;
    // FP32 records (4 bytes per value) fit in the scratch sized for FP64 records
    cudaError_t e = ensure_move_scratch(P, shadow_stride(N + nargs));
    if (e != cudaSuccess) return e;
    P->move.replayable = 1;
    XiF Xi{{xi[0], xi[1], N == 3 ? xi[2] : nullptr}};
    ArgsF A{};
    A.n = nargs;
    for (int k = 0; k < nargs; ++k) A.a[k] = args[k];
    const MoveScratch& m = P->move;
    MoveViewF S;
    S.m = MoveView{m.rec,    P->g.ncells, m.code, m.orig, m.shadow, P->g.ncells * P->g.max_xcell,
                   shadow_stride(N + nargs), P->g.max_xcell};  // 3 values padded to 4: 16-byte records
    S.shadow = (float*)m.shadow;
    cudaStream_t st = P->stream;
    const unsigned nb = grid_blocks(P->g.ncells);
    const unsigned nbw = grid_blocks(P->g.ncells, 32 * kWarpsPerBlock);
    const int ntw = 32 * kWarpsPerBlock;
    const F32Axes& ax = P->f32ax;
    if (N == 2) {
        if (P->f32_cells)
            move_classify_f32<2, true><<<nbw, ntw, 0, st>>>(P->g, Xi, index, A, S, ax, P->d_err);
        else
            move_classify_f32<2, false><<<nbw, ntw, 0, st>>>(P->g, Xi, index, A, S, ax, P->d_err);
        e = run_allocate_passes(P, S.m, st);
        if (e != cudaSuccess) return e;
        move_apply_f32<2><<<nb, kThreads, 0, st>>>(P->g, Xi, index, A, S);
    } else {
        if (P->f32_cells)
            move_classify_f32<3, true><<<nbw, ntw, 0, st>>>(P->g, Xi, index, A, S, ax, P->d_err);
        else
            move_classify_f32<3, false><<<nbw, ntw, 0, st>>>(P->g, Xi, index, A, S, ax, P->d_err);
        e = run_allocate_passes(P, S.m, st);
        if (e != cudaSuccess) return e;
        move_apply_f32<3><<<nb, kThreads, 0, st>>>(P->g, Xi, index, A, S);
    }
    return cudaGetLastError();
}

cudaError_t launch_inject_f32(jp_particles* P, float* const xi[3], uint8_t* index, float* const* args, int nargs,
                              uint32_t call)
{
    const int N = P->g.ndim;
    const int64_t nc = P->g.ncells;
    if (P->g.max_xcell > 64) {  // one warp per cell of each colour, no flag pass
        XiF Xi{{xi[0], xi[1], N == 3 ? xi[2] : nullptr}};
        ArgsF A{};
        A.n = nargs;
        for (int k = 0; k < nargs; ++k) A.a[k] = args[k];
        const F32Params prm = make_params(P, 0.5, 0.0);
        int64_t cols = 1;
        for (int d = 0; d < N; ++d) cols *= (P->g.n[d] + 1) / 2;
        const unsigned nb = grid_blocks(cols * 32, 32 * kWarpsPerBlock);
        for (int pass = 0; pass < (1 << N); ++pass) {
            if (N == 2)
                inject_wide_f32<2><<<nb, 32 * kWarpsPerBlock, 0, P->stream>>>(P->g, prm, Xi, index, A, pass, call,
                                                                              P->d_err);
            else
                inject_wide_f32<3><<<nb, 32 * kWarpsPerBlock, 0, P->stream>>>(P->g, prm, Xi, index, A, pass, call,
                                                                              P->d_err);
        }
        return cudaGetLastError();
    }
    {
        cudaError_t e = ensure_inject_scratch(P);
        if (e != cudaSuccess) return e;
    }
    InjectListsF Ls;
    Ls.counts = P->inject.counts;
    Ls.list = P->inject.list;
    Ls.lm = P->inject.lm;
    int64_t cnt[3][2];
    for (int d = 0; d < 3; ++d)
        for (int o = 0; o < 2; ++o) cnt[d][o] = d < N ? (P->g.n[d] - o + 1) / 2 : (o == 0 ? 1 : 0);
    int64_t off = 0;
    for (int col = 0; col < 8; ++col) {
        Ls.off[col] = off;
        off += cnt[0][col & 1] * cnt[1][(col >> 1) & 1] * cnt[2][(col >> 2) & 1];
    }
    cudaStream_t st = P->stream;
    cudaError_t e = cudaMemsetAsync(P->inject.counts, 0, 8 * sizeof(int), st);
    if (e != cudaSuccess) return e;
    XiF Xi{{xi[0], xi[1], N == 3 ? xi[2] : nullptr}};
    CXiF CX{{xi[0], xi[1], N == 3 ? xi[2] : nullptr}};
    ArgsF A{};
    A.n = nargs;
    for (int k = 0; k < nargs; ++k) A.a[k] = args[k];
    const F32Params prm = make_params(P, 0.5, 0.0);
    const unsigned nb = grid_blocks(nc);
    const int M = P->g.max_xcell;
    const int wpb = 4;
    const size_t smem = N == 2 ? wpb * hood_bytes_f32<2>(M) : wpb * hood_bytes_f32<3>(M);
    const unsigned nbp = (unsigned)(152 * 8);
    if (N == 2) {
        inject_flag_f32<2><<<nb, kThreads, 0, st>>>(P->g, CX, index, Ls);
        for (int pass = 0; pass < 4; ++pass) {
            const int col = (pass / 2) + 2 * (pass % 2);
            inject_pass_f32<2><<<nbp, 32 * wpb, smem, st>>>(P->g, prm, Xi, index, A, Ls, col, call, P->d_err);
        }
    } else {
        if (smem > 48 * 1024) {
            e = cudaFuncSetAttribute(inject_pass_f32<3>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
            if (e != cudaSuccess) return e;
        }
        inject_flag_f32<3><<<nb, kThreads, 0, st>>>(P->g, CX, index, Ls);
        for (int pass = 0; pass < 8; ++pass) {
            const int col = (pass / 4) + 2 * ((pass / 2) % 2) + 4 * (pass % 2);
            inject_pass_f32<3><<<nbp, 32 * wpb, smem, st>>>(P->g, prm, Xi, index, A, Ls, col, call, P->d_err);
        }
    }
    return cudaGetLastError();
}

cudaError_t launch_g2p_f32(jp_particles* P, float* Fp, const float* F, const float* const xi[3],
                           const uint8_t* index)
{
    const bool d3 = P->g.ndim == 3;
    CXiF Xi{{xi[0], xi[1], d3 ? xi[2] : nullptr}};
    const unsigned nb = grid_blocks(P->g.ncells);
    const bool wide = P->g.max_xcell > 64;
    if (!d3)
        wide ? g2p_f32_kernel<2, true><<<nb, kThreads, 0, P->stream>>>(P->g, Fp, F, Xi, index)
             : g2p_f32_kernel<2, false><<<nb, kThreads, 0, P->stream>>>(P->g, Fp, F, Xi, index);
    else
        wide ? g2p_f32_kernel<3, true><<<nb, kThreads, 0, P->stream>>>(P->g, Fp, F, Xi, index)
             : g2p_f32_kernel<3, false><<<nb, kThreads, 0, P->stream>>>(P->g, Fp, F, Xi, index);
    return cudaGetLastError();
}

cudaError_t launch_p2g_f32(jp_particles* P, float* F, const float* Fp, const float* const xi[3],
                           const uint8_t* index, double* W)
{
    const bool d3 = P->g.ndim == 3;
    CXiF Xi{{xi[0], xi[1], d3 ? xi[2] : nullptr}};
    const F32Params prm = make_params(P, 0.5, 0.0);
    const bool wide = P->g.max_xcell > 64;
    const int64_t V0 = P->g.n[0] + 1, V1 = P->g.n[1] + 1;
    const int64_t rows = P->g.n[d3 ? 2 : 1] + 1;
    if (!d3) {
        // cell-centric: warps of 31 vertex columns (+ one cell column to the left) over bands of
        // `band` vertex rows; bands as long as still leave about 4096 warps, 4 to 8 rows (a sweep
        // of 2..32 on one GB300: 8 the fastest at 1024^2, within 1% of the fastest at 2048^2)
        const int64_t wcols = (V0 + 30) / 31;
        int band = (int)((wcols * rows) / 4096);
        band = band < 4 ? 4 : (band > 8 ? 8 : band);
        const int64_t warps = wcols * ((rows + band - 1) / band);
        if (wide)
            p2g_f32_cells2d<true><<<grid_blocks(warps * 32), kThreads, 0, P->stream>>>(P->g, prm, F, Fp, Xi, index,
                                                                                       band, W);
        else
            p2g_f32_cells2d<false><<<grid_blocks(warps * 32), kThreads, 0, P->stream>>>(P->g, prm, F, Fp, Xi, index,
                                                                                        band, W);
    } else {
        // blocks of 31 x 7 vertex columns over bands of z rows, as long as still leave about 1024
        // blocks, 4 to 8 rows (8 the fastest of a sweep of 2..32 at 128^3)
        const int64_t wcols = (V0 + 30) / 31, jgroups = (V1 + 6) / 7;
        int band = (int)((wcols * jgroups * rows) / 1024);
        band = band < 4 ? 4 : (band > 8 ? 8 : band);
        const int64_t blocks = wcols * jgroups * ((rows + band - 1) / band);
        if (wide)
            p2g_f32_cells3d<true><<<(unsigned)blocks, kThreads, 0, P->stream>>>(P->g, prm, F, Fp, Xi, index, band, W);
        else
            p2g_f32_cells3d<false><<<(unsigned)blocks, kThreads, 0, P->stream>>>(P->g, prm, F, Fp, Xi, index, band, W);
    }
    return cudaGetLastError();
}

}  // namespace jp
