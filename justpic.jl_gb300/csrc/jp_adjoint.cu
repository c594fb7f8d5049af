// jp_adjoint.cu -- hand-written adjoint (vector-Jacobian products) of the
// FP64 hot path in 2D: one advection! step (Euler, RK2, RK4), particle2grid!,
// grid2particle!, and the replay of move_particles!'s and
// inject_particles!'s slot maps.
//
// None of this has a counterpart in the reference. Conventions:
//   * lam holds dL/d(position) per slot; gV dL/d(velocity node) per
//     component; gF dL/d(vertex field); gFp dL/d(particle field);
//   * relocation is integer data recorded in the forward sweep (the move's
//     destination map, the injection's source ids) and replayed by gathers;
//     it is not differentiated: dropped particles pass no gradient back, and
//     the positions of injected particles depend on nothing;
//   * every transpose is a gather with a fixed summation order, so results do
//     not depend on scheduling (no floating-point atomics).
//
// Transpose of the velocity sampling: a particle owned by cell I whose stage
// points stay within one cell of I deposits only on velocity nodes in a fixed
// window around I (4 x 5 nodes for Vx, 5 x 4 for Vy on the ghost-node grids).
// A replay kernel stages each particle's samples per slot; one thread per
// cell then accumulates its particles' deposits, in slot order, into the
// cell's 40 partial sums; one thread per velocity node adds the partial sums
// of the 20 owning cells whose windows contain it. A stage point outside the
// window is reported as JP_ERR_ADJOINT_WINDOW.
#include <cmath>

#include <math_constants.h>

#include "jp_f32_core.cuh"
#include "jp_internal.cuh"
#include "jp_move_core.cuh"
#include "jp_weight.cuh"

namespace jp {

constexpr int kWinParts = 40;    // 4*5 + 5*4 partial sums per owning cell
constexpr int kInjectReach = 4;  // 2D: four colour passes, each copy reaches one cell further

// node window of Vx (comp 0) / Vy (comp 1) around the owning cell
__host__ __device__ constexpr int win_nx(int comp) { return comp == 0 ? 4 : 5; }
__host__ __device__ constexpr int win_ny(int comp) { return comp == 0 ? 5 : 4; }

// ------------------------------------------------------- move permutation
// dest[a] = slot holding, after the last move, the particle that sat in slot a
// before it; -1 for empty slots and dropped particles.
__global__ void __launch_bounds__(kThreads) perm_init(DevGrid g, MoveView S, int32_t* __restrict__ dest)
{
    const int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= g.ncells) return;
    const int64_t nc = g.ncells;
    const uint64_t stay = S.L0(c) & S.L(c) & ~S.R(c);
    for (int s = 0; s < g.max_xcell; ++s) {
        const int64_t a = c + nc * s;
        dest[a] = ((stay >> s) & 1) ? (int32_t)a : -1;
    }
}

template <int DIM>
__global__ void __launch_bounds__(kThreads) perm_scatter(DevGrid g, MoveView S, int32_t* __restrict__ dest)
{
    const int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= g.ncells) return;
    const int64_t nc = g.ncells;
    uint64_t R = S.R(c);
    if (!R) return;
    int64_t I[3];
    cell_coords(g, c, I);
    while (R) {
        const int s = __ffsll((long long)R) - 1;
        R &= R - 1;
        const int64_t a = c + nc * s;
        const uint16_t tag = S.orig[a];  // source cell's neighbour code, the mover's rank there
        int off[3];
        nb_offset<DIM>(tag & 0x1F, off);
        const int64_t J[3] = {I[0] + off[0], I[1] + off[1], DIM == 3 ? I[2] + off[2] : 0};
        const int64_t src = cell_linear<DIM>(g, J);
        const int s_src = nth_set_bit64(S.M(src), tag >> 5);
        dest[src + nc * s_src] = (int32_t)a;  // each origin has one destination
    }
}

struct PermArrays {
    const double* post[8];
    double* pre[8];
    int n;
};

__global__ void __launch_bounds__(kThreads)
    permute_vjp_kernel(int64_t nslots, const int32_t* __restrict__ dest, PermArrays P)
{
    const int64_t a = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (a >= nslots) return;
    const int32_t d = dest[a];
    const bool ok = d >= 0 && d < nslots;
    for (int k = 0; k < P.n; ++k) P.pre[k][a] = ok ? P.post[k][d] : 0.0;
}

// ------------------------------------------------------------ injection

// Per cell: the slots whose id names another slot (particles injected by the
// traced call), after checking that each source lies within reach; and a flag
// on every cell holding a source (an order-free atomicOr), so the gather
// below only scans its window from those cells.
// ids: a slot's own index when it held a particle before the traced call, the
// index of the particle its fields were copied from when it was injected, a
// negative value otherwise; as doubles (FP64 fields) or as int32 (carried bit
// for bit through an FP32 field).
// Slot ids as doubles hold whole numbers below 2^53; they are built and read on
// the integer pipe (GB300's FP64 conversions run at the FP64 rate): the double
// of a >= 0 is exponent floor(log2 a) and the bits below the leading one.
__device__ __forceinline__ uint64_t id_bits(int64_t a)
{
    if (a == 0) return 0ull;
    const int e = 63 - __clzll(a);  // a < 2^53
    return ((uint64_t)(1023 + e) << 52) | (((uint64_t)a << (52 - e)) & ((1ull << 52) - 1));
}

// the whole number a double id holds, or -1 for anything else (negative, NaN, >= 2^53)
__device__ __forceinline__ int64_t id_value(double id)
{
    const uint64_t b = (uint64_t)__double_as_longlong(id);
    if (b == 0) return 0;
    const int E = (int)(b >> 52);  // sign bit included
    if (E < 1023 || E > 1023 + 52) return -1;
    const int e = E - 1023;
    const uint64_t m = (b & ((1ull << 52) - 1)) | (1ull << 52);
    if (m & ((1ull << (52 - e)) - 1)) return -1;  // not a whole number
    return (int64_t)(m >> (52 - e));
}

__device__ __forceinline__ bool id_other(double id, int64_t a)
{
    const int64_t v = id_value(id);
    return v >= 0 && v != a;
}
__device__ __forceinline__ bool id_other(int32_t id, int64_t a) { return id >= 0 && (int64_t)id != a; }
__device__ __forceinline__ bool id_self(double id, int64_t a) { return id_value(id) == a; }
__device__ __forceinline__ bool id_self(int32_t id, int64_t a) { return (int64_t)id == a; }
__device__ __forceinline__ int64_t id_slot(double id, int64_t ns)
{
    const int64_t v = id_value(id);
    return v >= 0 && v < ns ? v : ns;
}
__device__ __forceinline__ int64_t id_slot(int32_t id, int64_t ns) { return (int64_t)id < ns ? (int64_t)id : ns; }
__device__ __forceinline__ double id_make(int64_t a, double) { return __longlong_as_double((long long)id_bits(a)); }
__device__ __forceinline__ int32_t id_make(int64_t a, int32_t) { return (int32_t)a; }
__device__ __forceinline__ double id_none(double) { return -1.0; }
__device__ __forceinline__ int32_t id_none(int32_t) { return -1; }

template <typename IdT>
__global__ void __launch_bounds__(kThreads)
    slot_ids_kernel(int64_t nslots, const uint8_t* __restrict__ index, IdT* __restrict__ ids)
{
    const int64_t a = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (a >= nslots) return;
    ids[a] = index[a] ? id_make(a, IdT()) : id_none(IdT());
}


template <typename IdT>
__global__ void __launch_bounds__(kThreads)
    inject_mask_kernel(DevGrid g, const IdT* __restrict__ ids, uint64_t* __restrict__ inj,
                       unsigned* __restrict__ srcflag, int* d_err)
{
    const int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= g.ncells) return;
    const int64_t nc = g.ncells;
    const int64_t ns = nc * g.max_xcell;
    const int64_t cx = c % g.n[0], cy = c / g.n[0];
    uint64_t m = 0;
    int errs = 0;
    constexpr int U = 4;  // slots whose ids are loaded together (the loop is bound by load latency)
    for (int s0 = 0; s0 < g.max_xcell; s0 += U) {
        IdT idl[U];
#pragma unroll
        for (int u = 0; u < U; ++u) idl[u] = s0 + u < g.max_xcell ? ids[c + nc * (s0 + u)] : ids[c];
#pragma unroll
        for (int u = 0; u < U; ++u) {
            const int s = s0 + u;
            if (s >= g.max_xcell) break;
            const int64_t a = c + nc * s;
            const IdT id = idl[u];
            if (id_other(id, a)) {
                const int64_t src = id_slot(id, ns);
                const int64_t sc = src % nc;
                const int64_t sx = sc % g.n[0], sy = sc / g.n[0];
                if (src >= ns || sx < cx - kInjectReach || sx > cx + kInjectReach || sy < cy - kInjectReach ||
                    sy > cy + kInjectReach) {
                    errs |= kErrAdjointWindow;
                } else {
                    m |= 1ull << s;
                    atomicOr(srcflag + sc, 1u);
                }
            }
        }
    }
    inj[c] = m;
    raise_err(d_err, errs);
}

// Source cell c adds to pre[k][src] (arrays k in `copies`) post[k][b] of every
// slot b injected from one of its slots: cells of the window in order (y outer,
// x inner), slots ascending.
template <typename IdT>
__device__ __forceinline__ void gather_copies(const DevGrid& g, const IdT* __restrict__ ids,
                                              const uint64_t* __restrict__ inj, const PermArrays& P,
                                              unsigned copies, int64_t c)
{
    const int64_t nc = g.ncells;
    const int64_t ns = nc * g.max_xcell;
    const int64_t cx = c % g.n[0], cy = c / g.n[0];
    constexpr int RW = 2 * kInjectReach + 1;  // window width
    const int64_t x0 = cx - kInjectReach;
    for (int64_t y = max(cy - kInjectReach, (int64_t)0); y <= min(cy + kInjectReach, g.n[1] - 1); ++y) {
        // the injected-slot masks of one window row, loaded together
        uint64_t row[RW];
#pragma unroll
        for (int j = 0; j < RW; ++j) {
            const int64_t x = x0 + j;
            row[j] = (x >= 0 && x < g.n[0]) ? inj[x + g.n[0] * y] : 0ull;
        }
#pragma unroll
        for (int j = 0; j < RW; ++j) {
            const int64_t w = (x0 + j) + g.n[0] * y;
            uint64_t m = row[j];
            while (m) {
                const int s = __ffsll((long long)m) - 1;
                m &= m - 1;
                const int64_t b = w + nc * s;
                const int64_t src = id_slot(ids[b], ns);  // a slot index: inject_mask_kernel checked it
                if (src % nc != c) continue;
                for (int k = 0; k < P.n; ++k)
                    if ((copies >> k) & 1u) P.pre[k][src] += P.post[k][b];
            }
        }
    }
}

// pre[k][a] = post[k][a] for slots that existed before the injection (id ==
// own slot), 0 otherwise; for the arrays k in the `copies` bit mask, a
// pre-existing slot also collects post[k][b] of every slot b injected from it,
// cells of the window in order (y outer, x inner), slots ascending.
template <typename IdT>
__global__ void __launch_bounds__(kThreads)
    inject_vjp_kernel(DevGrid g, const IdT* __restrict__ ids, const uint64_t* __restrict__ inj,
                      const unsigned* __restrict__ srcflag, PermArrays P, unsigned copies)
{
    const int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= g.ncells) return;
    const int64_t nc = g.ncells;
    const int M = g.max_xcell;
    // U slots at a time: their ids, then per array their values, are loaded together
    // (the loop is bound by load latency, not by bandwidth)
    constexpr int U = 4;
    for (int s0 = 0; s0 < M; s0 += U) {
        bool kept[U];
#pragma unroll
        for (int u = 0; u < U; ++u) {
            const int64_t a = c + nc * (s0 + u);
            kept[u] = s0 + u < M && id_self(ids[s0 + u < M ? a : c], a);
        }
        for (int k = 0; k < P.n; ++k) {
            double v[U];
#pragma unroll
            for (int u = 0; u < U; ++u) v[u] = kept[u] ? P.post[k][c + nc * (s0 + u)] : 0.0;
#pragma unroll
            for (int u = 0; u < U; ++u)
                if (s0 + u < M) P.pre[k][c + nc * (s0 + u)] = v[u];
        }
    }
    if (!copies || !srcflag[c]) return;
    gather_copies(g, ids, inj, P, copies, c);
}

// The in-place form (pre == post): only the sources gather their copies'
// cotangents. The slots the injection filled keep their values: the move's
// transpose that follows reads only the slots that existed before the
// injection, and those are the ones this leaves as they were (plus the copies).
template <typename IdT>
__global__ void __launch_bounds__(kThreads)
    inject_vjp_inplace_kernel(DevGrid g, const IdT* __restrict__ ids, const uint64_t* __restrict__ inj,
                              const unsigned* __restrict__ srcflag, PermArrays P, unsigned copies)
{
    const int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= g.ncells || !srcflag[c]) return;
    gather_copies(g, ids, inj, P, copies, c);
}

// --------------------------------------------------------- advection step
// Value, gradient, grid cell and local coordinates of one velocity component
// at p, with the forward's cell selection (seed = the particle's cell; the
// limits test only when the seed interval does not hold p).
struct Samp {
    double v;
    double dv[2];
    int idx[2];
    double t[2];
    bool ok;
};

__device__ __forceinline__ Samp sample2(const DevGrid& g, int comp, const double* p, const int* I,
                                        const double* __restrict__ V, int* errs)
{
    Samp r;
    r.ok = true;
#pragma unroll
    for (int d = 0; d < 2; ++d) {
        const double* x = g.xvel[comp][d];
        const int J = I[d];
        const double a = ldg(x + J), b = ldg(x + J + 1);
        const long long kp = okey(p[d]), ka = okey(a), kb = okey(b);
        const bool pnan = is_nan_bits(p[d]);
        int64_t k;
        // the forward's cell selection (interp_component): the seed test, then the open
        // neighbouring intervals (the only answers the bisection can give there), on
        // integer keys (exact for non-NaN values, off the FP64 pipe)
        if (!pnan && ka <= kp && kp <= kb) {
            k = J;
        } else if (!pnan && kb < kp && J + 2 < g.nvel[comp][d] && kp < okey(ldg(x + J + 2))) {
            k = J + 1;
        } else if (!pnan && kp < ka && J >= 1 && okey(ldg(x + J - 1)) < kp) {
            k = J - 1;
        } else {
            if (!(g.lim_lo[comp][0] <= p[0] && p[0] <= g.lim_hi[comp][0] && g.lim_lo[comp][1] <= p[1] &&
                  p[1] <= g.lim_hi[comp][1])) {
                r.ok = false;
                return r;
            }
            k = find_cell(p[d], x, g.nvel[comp][d], J, errs);
        }
        r.idx[d] = (int)k;
        r.t[d] = (p[d] - ldg(x + k)) * ldg(g.ixvel[comp][d] + k);
    }
    const int64_t L0 = g.nvel[comp][0];
    const double* b = V + r.idx[0] + L0 * r.idx[1];
    const double v00 = ldg(b), v10 = ldg(b + 1), v01 = ldg(b + L0), v11 = ldg(b + L0 + 1);
    const double tx = r.t[0], ty = r.t[1];
    const double a0 = lerp1(tx, v00, v10), a1 = lerp1(tx, v01, v11);
    r.v = lerp1(ty, a0, a1);
    // gradient of the bilinear form: d/dtx = (1-ty)(v10-v00) + ty(v11-v01), d/dty = a1 - a0
    const double ax = v10 - v00, bx = v11 - v01;
    r.dv[0] = fma(ty, bx - ax, ax) * ldg(g.ixvel[comp][0] + r.idx[0]);
    r.dv[1] = (a1 - a0) * ldg(g.ixvel[comp][1] + r.idx[1]);
    return r;
}

struct AdjParams {
    double dt, adt;
    double ca, cb;  // RK2: X' = X + dt (ca V(X) + cb V(X + alpha dt V(X)))
    int method;
    int half;  // alpha == 1/2: the forward's X' = X + dt V(X1)
};

// J^T g for the two components sampled at one point
__device__ __forceinline__ void jt(const Samp* s, const double* g, double* out)
{
    out[0] = s[0].dv[0] * g[0] + s[1].dv[0] * g[1];
    out[1] = s[0].dv[1] * g[0] + s[1].dv[1] * g[1];
}

template <int METHOD>
constexpr int adj_stages()
{
    return METHOD == JP_RUNGE_KUTTA4 ? 4 : (METHOD == JP_RUNGE_KUTTA2 ? 2 : 1);
}

// Per-slot record of one velocity sample q (stage q/2, component q%2) of a
// particle, written by the replay kernel and read by the deposit kernel:
// local coordinates, cotangent and window position (one byte: ox | oy << 4,
// 0xFF when the sample deposits nothing).
struct Staging {
    double* t;     // [(q * 2 + d) * nslots + a]
    double* gk;    // [q * nslots + a]
    uint8_t* win;  // [q * nslots + a]
    int64_t nslots;
};

// Replay: a warp covers 32 consecutive cells and its lanes take their live
// particles in slot-major order (full lanes whatever the occupancy, and no
// shared memory beyond the slot list, so many warps hide the latency of the
// dependent velocity loads). Each particle's stages are replayed with the
// forward's cell selection, lam (dL/dX after the step) becomes dL/dX before
// it, and every velocity sample's deposit data is staged per slot.
template <int METHOD>
__global__ void __launch_bounds__(32 * kWarpsPerBlock, METHOD == JP_RUNGE_KUTTA4 ? 2 : 3)
    advect_vjp_kernel(DevGrid g, const double* __restrict__ V0, const double* __restrict__ V1, AdjParams P,
                      CCoords X, const uint8_t* __restrict__ index, Coords Lam, Staging stg, int* d_err)
{
    constexpr int NS = adj_stages<METHOD>();
    __shared__ SlotList lists[kWarpsPerBlock];
    __shared__ int cellI[kWarpsPerBlock][32][2];
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int64_t c0 = ((int64_t)blockIdx.x * kWarpsPerBlock + w) * 32;
    if (c0 >= g.ncells) return;
    const int64_t nc = g.ncells;
    const int M = g.max_xcell;
    {
        const int64_t c = min(c0 + lane, nc - 1);
        cellI[w][lane][0] = (int)(c % g.n[0]);
        cellI[w][lane][1] = (int)(c / g.n[0]);
    }
    uint64_t mine;
    const int K = build_slot_list(lists[w], index, c0, nc, M, lane, &mine);
    const double* Vc[2] = {V0, V1};
    const int64_t ns = stg.nslots;
    int errs = 0;
    for (int k = lane; k < K; k += 32) {
        int s, l;
        slot_item(lists[w], M, k, &s, &l);
        const int64_t a = c0 + l + nc * s;
        const int I[2] = {cellI[w][l][0], cellI[w][l][1]};
        const double p0[2] = {X.c[0][a], X.c[1][a]};
        const double lam[2] = {Lam.c[0][a], Lam.c[1][a]};
        // forward stages with the forward's arithmetic, keeping every sample
        Samp S[NS][2];
        bool ok = true;
#pragma unroll
        for (int q = 0; q < NS; ++q) {
            double x[2];
#pragma unroll
            for (int d = 0; d < 2; ++d) {
                if (q == 0)
                    x[d] = p0[d];
                else if (METHOD == JP_RUNGE_KUTTA2)
                    x[d] = fma(1.0, P.adt * S[0][d].v, p0[d]);
                else if (q < 3)
                    x[d] = p0[d] + (P.dt * S[q - 1][d].v) * 0.5;
                else
                    x[d] = p0[d] + P.dt * S[2][d].v;
            }
#pragma unroll
            for (int cc = 0; cc < 2; ++cc) {
                S[q][cc] = sample2(g, cc, x, I, Vc[cc], &errs);
                ok &= S[q][cc].ok;
            }
            if (!ok) break;
        }
        if (!ok) {  // the forward sent this particle to Inf; move_particles! dropped it
            Lam.c[0][a] = 0.0;
            Lam.c[1][a] = 0.0;
#pragma unroll
            for (int q = 0; q < 2 * NS; ++q) stg.win[q * ns + a] = 0xFF;
            continue;
        }
        // reverse sweep over the stages: gk[q] = dL/d(velocity sample of stage q)
        double gk[NS][2], l0[2] = {lam[0], lam[1]}, qb[2];
        if (METHOD == JP_RUNGE_KUTTA2) {
#pragma unroll
            for (int d = 0; d < 2; ++d) {
                gk[NS - 1][d] = P.dt * P.cb * lam[d];
                gk[0][d] = P.dt * P.ca * lam[d];
            }
            jt(S[NS - 1], gk[NS - 1], qb);  // x1 = p0 + alpha dt k0
#pragma unroll
            for (int d = 0; d < 2; ++d) {
                l0[d] += qb[d];
                gk[0][d] += P.adt * qb[d];
            }
        } else if (METHOD == JP_RUNGE_KUTTA4) {
            const double w6 = P.dt / 6.0;
#pragma unroll
            for (int d = 0; d < 2; ++d) {
                gk[0][d] = w6 * lam[d];
                gk[1][d] = 2.0 * w6 * lam[d];
                gk[2][d] = 2.0 * w6 * lam[d];
                gk[NS - 1][d] = w6 * lam[d];
            }
#pragma unroll
            for (int q = NS - 1; q >= 1; --q) {  // x3 = p0 + dt k2, x2 = p0 + dt/2 k1, x1 = p0 + dt/2 k0
                jt(S[q], gk[q], qb);
                const double h = q == 3 ? P.dt : 0.5 * P.dt;
#pragma unroll
                for (int d = 0; d < 2; ++d) {
                    l0[d] += qb[d];
                    gk[q - 1][d] += h * qb[d];
                }
            }
        } else {
#pragma unroll
            for (int d = 0; d < 2; ++d) gk[0][d] = P.dt * lam[d];
        }
        jt(S[0], gk[0], qb);  // the first stage samples at p0 itself
#pragma unroll
        for (int d = 0; d < 2; ++d) l0[d] += qb[d];
        Lam.c[0][a] = l0[0];
        Lam.c[1][a] = l0[1];
#pragma unroll
        for (int q = 0; q < NS; ++q)
#pragma unroll
            for (int cc = 0; cc < 2; ++cc) {
                const int j = 2 * q + cc;
                const int ox = S[q][cc].idx[0] - I[0] + 1, oy = S[q][cc].idx[1] - I[1] + 1;
                const bool in = ox >= 0 && ox <= win_nx(cc) - 2 && oy >= 0 && oy <= win_ny(cc) - 2;
                if (!in) errs |= kErrAdjointWindow;
                stg.win[j * ns + a] = in ? (uint8_t)(ox | (oy << 4)) : (uint8_t)0xFF;
                stg.t[(2 * j) * ns + a] = S[q][cc].t[0];
                stg.t[(2 * j + 1) * ns + a] = S[q][cc].t[1];
                stg.gk[j * ns + a] = gk[q][cc];
            }
    }
    raise_err(d_err, errs);
}

// ----------------------------------------- recorded stages (no replay)
// A step's record, written by the recording advection and read by the
// recorded VJP and the deposit: per slot and velocity sample j = 2 q + comp,
// the local coordinates t and the gradient dv of the bilinear sample, and the
// window byte (as in Staging; 0xFF: deposits nothing), then one byte per slot
// that is 0 when the forward sent the particle to Inf. Layout (ns slots, NQ
// samples): t[(2j + d) ns + a], dv[(2j + d) ns + a], win[j ns + a], okf[a].
struct Record {
    double* t;
    double* dv;
    uint8_t* win;
    uint8_t* okf;
    int64_t nslots;
};

template <int METHOD>
__host__ __device__ constexpr int rec_samples()
{
    return 2 * adj_stages<METHOD>();
}

__host__ __device__ inline size_t record_bytes(int64_t ns, int nq)
{
    return (size_t)ns * nq * (4 * sizeof(double) + 1) + (size_t)ns;
}

__host__ __device__ inline Record record_view(void* base, int64_t ns, int nq)
{
    Record r;
    r.t = (double*)base;
    r.dv = r.t + 2 * (size_t)nq * ns;
    r.win = (uint8_t*)(r.dv + 2 * (size_t)nq * ns);
    r.okf = r.win + (size_t)nq * ns;
    r.nslots = ns;
    return r;
}

// advection! (RK2, RK4, Euler; 2D FP64) that also records every velocity
// sample for the reverse sweep. The stages are the adjoint replay's (the
// forward's arithmetic and cell selection), so positions are those of
// advection!, bit for bit; a sample outside its grid's limits is Inf, as in the
// forward. A stage point outside the deposit window raises JP_ERR_ADJOINT_WINDOW.
template <int METHOD>
__global__ void __launch_bounds__(32 * kWarpsPerBlock, METHOD == JP_RUNGE_KUTTA4 ? 2 : 4)
    advect_record_kernel(DevGrid g, const double* __restrict__ V0, const double* __restrict__ V1, AdjParams P,
                         Coords X, const uint8_t* __restrict__ index, Record rec, int* d_err)
{
    constexpr int NS = adj_stages<METHOD>();
    __shared__ SlotList lists[kWarpsPerBlock];
    __shared__ int cellI[kWarpsPerBlock][32][2];
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int64_t c0 = ((int64_t)blockIdx.x * kWarpsPerBlock + w) * 32;
    if (c0 >= g.ncells) return;
    const int64_t nc = g.ncells;
    const int M = g.max_xcell;
    {
        const int64_t c = min(c0 + lane, nc - 1);
        cellI[w][lane][0] = (int)(c % g.n[0]);
        cellI[w][lane][1] = (int)(c / g.n[0]);
    }
    uint64_t mine;
    const int K = build_slot_list(lists[w], index, c0, nc, M, lane, &mine);
    const double* Vc[2] = {V0, V1};
    const int64_t ns = rec.nslots;
    int errs = 0;
    for (int k = lane; k < K; k += 32) {
        int s, l;
        slot_item(lists[w], M, k, &s, &l);
        const int64_t a = c0 + l + nc * s;
        const int I[2] = {cellI[w][l][0], cellI[w][l][1]};
        const double p0[2] = {X.c[0][a], X.c[1][a]};
        double v[NS][2];
        bool ok = true;
#pragma unroll
        for (int q = 0; q < NS; ++q) {
            double x[2];
#pragma unroll
            for (int d = 0; d < 2; ++d) {
                if (q == 0)
                    x[d] = p0[d];
                else if (METHOD == JP_RUNGE_KUTTA2)
                    x[d] = fma(1.0, P.adt * v[0][d], p0[d]);
                else if (q < 3)
                    x[d] = p0[d] + (P.dt * v[q - 1][d]) * 0.5;
                else
                    x[d] = p0[d] + P.dt * v[2][d];
            }
#pragma unroll
            for (int cc = 0; cc < 2; ++cc) {
                const Samp S = sample2(g, cc, x, I, Vc[cc], &errs);
                v[q][cc] = S.ok ? S.v : CUDART_INF;  // interp_velocity2particle outside the limits
                ok &= S.ok;
                // written as soon as sampled (fewer live registers); a particle the forward
                // sends to Inf gets its windows cleared below
                const int j = 2 * q + cc;
                uint8_t wv = 0xFF;
                if (S.ok) {
                    const int ox = S.idx[0] - I[0] + 1, oy = S.idx[1] - I[1] + 1;
                    const bool in = ox >= 0 && ox <= win_nx(cc) - 2 && oy >= 0 && oy <= win_ny(cc) - 2;
                    if (in) wv = (uint8_t)(ox | (oy << 4));
                    else errs |= kErrAdjointWindow;
                    rec.t[(2 * j) * ns + a] = S.t[0];
                    rec.t[(2 * j + 1) * ns + a] = S.t[1];
                    rec.dv[(2 * j) * ns + a] = S.dv[0];
                    rec.dv[(2 * j + 1) * ns + a] = S.dv[1];
                }
                rec.win[j * ns + a] = wv;
            }
        }
#pragma unroll
        for (int d = 0; d < 2; ++d) {  // the forward's update (advect_particle)
            double pd;
            if (METHOD == JP_RUNGE_KUTTA2)
                pd = P.half ? fma(1.0, P.dt * v[1][d], p0[d])
                            : fma(1.0, P.dt * fma(P.ca, v[0][d], P.cb * v[1][d]), p0[d]);
            else if (METHOD == JP_RUNGE_KUTTA4)
                pd = p0[d] + __ddiv_rn(P.dt * (((v[0][d] + 2.0 * v[1][d]) + 2.0 * v[2][d]) + v[3][d]), 6.0);
            else
                pd = fma(1.0, P.dt * v[0][d], p0[d]);
            X.c[d][a] = pd;
        }
        rec.okf[a] = ok ? 1 : 0;
        if (!ok)
#pragma unroll
            for (int j = 0; j < 2 * NS; ++j) rec.win[j * ns + a] = 0xFF;
    }
    raise_err(d_err, errs);
}

// The VJP of a recorded step: lam (dL/dX after the step) becomes dL/dX before
// it, and each sample's cotangent gk goes to the staging for the deposit
// (which reads t and the window byte from the record).
template <int METHOD>
__global__ void __launch_bounds__(32 * kWarpsPerBlock)
    advect_vjp_rec_kernel(DevGrid g, AdjParams P, const uint8_t* __restrict__ index, Record rec, Coords Lam,
                          double* __restrict__ gk_out)
{
    constexpr int NS = adj_stages<METHOD>();
    __shared__ SlotList lists[kWarpsPerBlock];
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int64_t c0 = ((int64_t)blockIdx.x * kWarpsPerBlock + w) * 32;
    if (c0 >= g.ncells) return;
    const int64_t nc = g.ncells;
    const int M = g.max_xcell;
    uint64_t mine;
    const int K = build_slot_list(lists[w], index, c0, nc, M, lane, &mine);
    const int64_t ns = rec.nslots;
    for (int k = lane; k < K; k += 32) {
        int s, l;
        slot_item(lists[w], M, k, &s, &l);
        const int64_t a = c0 + l + nc * s;
        if (!rec.okf[a]) {  // the forward sent this particle to Inf; move_particles! dropped it
            Lam.c[0][a] = 0.0;
            Lam.c[1][a] = 0.0;
            continue;
        }
        const double lam[2] = {Lam.c[0][a], Lam.c[1][a]};
        Samp S[NS][2];
#pragma unroll
        for (int q = 0; q < NS; ++q)
#pragma unroll
            for (int cc = 0; cc < 2; ++cc) {
                const int j = 2 * q + cc;
                S[q][cc].dv[0] = rec.dv[(2 * j) * ns + a];
                S[q][cc].dv[1] = rec.dv[(2 * j + 1) * ns + a];
            }
        double gk[NS][2], l0[2] = {lam[0], lam[1]}, qb[2];
        if (METHOD == JP_RUNGE_KUTTA2) {
#pragma unroll
            for (int d = 0; d < 2; ++d) {
                gk[NS - 1][d] = P.dt * P.cb * lam[d];
                gk[0][d] = P.dt * P.ca * lam[d];
            }
            jt(S[NS - 1], gk[NS - 1], qb);
#pragma unroll
            for (int d = 0; d < 2; ++d) {
                l0[d] += qb[d];
                gk[0][d] += P.adt * qb[d];
            }
        } else if (METHOD == JP_RUNGE_KUTTA4) {
            const double w6 = P.dt / 6.0;
#pragma unroll
            for (int d = 0; d < 2; ++d) {
                gk[0][d] = w6 * lam[d];
                gk[1][d] = 2.0 * w6 * lam[d];
                gk[2][d] = 2.0 * w6 * lam[d];
                gk[NS - 1][d] = w6 * lam[d];
            }
#pragma unroll
            for (int q = NS - 1; q >= 1; --q) {
                jt(S[q], gk[q], qb);
                const double h = q == 3 ? P.dt : 0.5 * P.dt;
#pragma unroll
                for (int d = 0; d < 2; ++d) {
                    l0[d] += qb[d];
                    gk[q - 1][d] += h * qb[d];
                }
            }
        } else {
#pragma unroll
            for (int d = 0; d < 2; ++d) gk[0][d] = P.dt * lam[d];
        }
        jt(S[0], gk[0], qb);
#pragma unroll
        for (int d = 0; d < 2; ++d) l0[d] += qb[d];
        Lam.c[0][a] = l0[0];
        Lam.c[1][a] = l0[1];
#pragma unroll
        for (int q = 0; q < NS; ++q)
#pragma unroll
            for (int cc = 0; cc < 2; ++cc) gk_out[(2 * q + cc) * ns + a] = gk[q][cc];
    }
}

constexpr int kDepThreads = 128;

// Deposit: one thread per owning cell adds its particles' staged samples, in
// slot order, to the cell's 40 window partial sums (shared memory), then
// writes them out for the node gather. The lanes of a warp walk the slots
// together (up to the highest live slot of the warp), so every load of the
// staged arrays is coalesced across the warp's 32 cells.
template <int NQ>
__global__ void __launch_bounds__(kDepThreads)
    deposit_kernel(DevGrid g, const uint8_t* __restrict__ index, Staging stg, double* __restrict__ parts)
{
    __shared__ double part[kWinParts][kDepThreads];
    const int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t nc = g.ncells;
    const bool valid = c < nc;
    const int64_t ns = stg.nslots;
    const int t = threadIdx.x;
    for (int k = 0; k < kWinParts; ++k) part[k][t] = 0.0;
    const uint64_t m = valid ? live_mask(index, c, nc, g.max_xcell) : 0;
    const uint32_t hi = __reduce_max_sync(0xffffffffu, m ? 64u - (uint32_t)__clzll((long long)m) : 0u);
    for (int s = 0; s < (int)hi; ++s) {
        if (!((m >> s) & 1)) continue;
        const int64_t a = c + nc * s;
#pragma unroll
        for (int q = 0; q < NQ; ++q) {
            const uint8_t wv = stg.win[q * ns + a];
            if (wv == 0xFF) continue;
            const int cc = q & 1;
            const int NX = win_nx(cc);
            const int b = (cc == 0 ? 0 : 20) + (wv & 0xF) + NX * (wv >> 4);
            const double tx = stg.t[(2 * q) * ns + a], ty = stg.t[(2 * q + 1) * ns + a];
            const double gq = stg.gk[q * ns + a];
            const double g0 = gq * (1.0 - ty), g1 = gq * ty;
            part[b][t] = fma(g0, 1.0 - tx, part[b][t]);
            part[b + 1][t] = fma(g0, tx, part[b + 1][t]);
            part[b + NX][t] = fma(g1, 1.0 - tx, part[b + NX][t]);
            part[b + NX + 1][t] = fma(g1, tx, part[b + NX + 1][t]);
        }
    }
    if (valid)
        for (int k = 0; k < kWinParts; ++k) parts[k * nc + c] = part[k][t];
}

// s += x with the rounding error kept in s.y (TwoSum; needs -fmad=false)
__device__ __forceinline__ void csum2_add(float2& s, float x)
{
    const float t = s.x + x;
    const float bp = t - s.x;
    const float err = (s.x - (t - bp)) + (x - bp);
    s.x = t;
    s.y += err;
}

// The deposit of the split-precision form: its staged coordinates are the
// forward's FP32 interpolation coordinates (t in FP32, exact) and its staged
// cotangents are rounded to FP32, so the bilinear terms are formed in FP32
// and summed per window part as compensated FP32 pairs, in the same slot
// order as deposit_kernel; each pair becomes one FP64 partial sum at the end.
// The FP64 pipe (1/64 of the FP32 rate, and idle for the lanes on empty
// slots) is left to the per-cell write-out.
template <int NQ>
__global__ void __launch_bounds__(kDepThreads)
    deposit_f32_kernel(DevGrid g, const uint8_t* __restrict__ index, Staging stg, double* __restrict__ parts)
{
    __shared__ float2 part[kWinParts][kDepThreads];
    const int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t nc = g.ncells;
    const bool valid = c < nc;
    const int64_t ns = stg.nslots;
    const int t = threadIdx.x;
    const float* tf = reinterpret_cast<const float*>(stg.t);
    const float* gkf = reinterpret_cast<const float*>(stg.gk);
    for (int k = 0; k < kWinParts; ++k) part[k][t] = make_float2(0.0f, 0.0f);
    const uint64_t m = valid ? live_mask(index, c, nc, g.max_xcell) : 0;
    const uint32_t hi = __reduce_max_sync(0xffffffffu, m ? 64u - (uint32_t)__clzll((long long)m) : 0u);
    for (int s = 0; s < (int)hi; ++s) {
        if (!((m >> s) & 1)) continue;
        const int64_t a = c + nc * s;
#pragma unroll
        for (int q = 0; q < NQ; ++q) {
            const uint8_t wv = stg.win[q * ns + a];
            if (wv == 0xFF) continue;
            const int cc = q & 1;
            const int NX = win_nx(cc);
            const int b = (cc == 0 ? 0 : 20) + (wv & 0xF) + NX * (wv >> 4);
            const float tx = tf[(2 * q) * ns + a], ty = tf[(2 * q + 1) * ns + a];
            const float gq = gkf[q * ns + a];
            const float g0 = gq * (1.0f - ty), g1 = gq * ty;
            csum2_add(part[b][t], g0 * (1.0f - tx));
            csum2_add(part[b + 1][t], g0 * tx);
            csum2_add(part[b + NX][t], g1 * (1.0f - tx));
            csum2_add(part[b + NX + 1][t], g1 * tx);
        }
    }
    if (valid)
        for (int k = 0; k < kWinParts; ++k) parts[k * nc + c] = (double)part[k][t].x + (double)part[k][t].y;
}

// ------------------------------------------- split-precision form (FP32)
// Velocity sample of the FP32 form (velocity_f32's cell and local
// coordinates, in cell units) with its gradient with respect to the offset.
struct SampF {
    float v;
    float dv[2];
    int idx[2];
    float t[2];
    bool ok;
};

__device__ __forceinline__ SampF sample2_f32(const DevGrid& g, int comp, const int* I, const float* xi,
                                             const float* __restrict__ V)
{
    SampF r;
    r.ok = true;
#pragma unroll
    for (int d = 0; d < 2; ++d) {
        const float y = (d == comp) ? xi[d] : xi[d] + 0.5f;
        if (!(fabsf(y) < 1e6f)) {
            r.ok = false;
            return r;
        }
        const float fl = floorf(y);
        int kk = I[d] + (int)fl;
        float tt = y - fl;
        const int L = (int)g.nvel[comp][d];
        if (kk == L - 1 && tt == 0.0f) {
            kk = L - 2;
            tt = 1.0f;
        }
        if (kk < 0 || kk > L - 2) {
            r.ok = false;
            return r;
        }
        r.idx[d] = kk;
        r.t[d] = tt;
    }
    const int64_t L0 = g.nvel[comp][0];
    const float* b = V + r.idx[0] + L0 * r.idx[1];
    const float v00 = __ldg(b), v10 = __ldg(b + 1), v01 = __ldg(b + L0), v11 = __ldg(b + L0 + 1);
    const float tx = r.t[0], ty = r.t[1];
    const float a0 = lerpf1(tx, v00, v10), a1 = lerpf1(tx, v01, v11);
    r.v = lerpf1(ty, a0, a1);
    const float ax = v10 - v00, bx = v11 - v01;
    r.dv[0] = fmaf(ty, bx - ax, ax);
    r.dv[1] = a1 - a0;
    return r;
}

__device__ __forceinline__ void jt_f(const SampF* s, const double* g, double* out)
{
    out[0] = (double)s[0].dv[0] * g[0] + (double)s[1].dv[0] * g[1];
    out[1] = (double)s[0].dv[1] * g[0] + (double)s[1].dv[1] * g[1];
}

// Replay kernel of the FP32 form: the stages of advect_f32 (offsets in cell
// units, FP32, the same operations), then the same reverse sweep as the FP64
// kernel with the per-axis step w = dt/dx, carried out in FP64; lam is
// dL/d(offset). The staged samples (FP32 coordinates and cotangents) feed
// deposit_f32_kernel and the same node gather.
template <int METHOD>
__global__ void __launch_bounds__(32 * kWarpsPerBlock, METHOD == JP_RUNGE_KUTTA4 ? 2 : 3)
    advect_vjp_f32_kernel(DevGrid g, const float* __restrict__ V0, const float* __restrict__ V1, F32Params P,
                          CXiF Xi, const uint8_t* __restrict__ index, Coords Lam, Staging stg, int* d_err)
{
    constexpr int NS = adj_stages<METHOD>();
    __shared__ SlotList lists[kWarpsPerBlock];
    __shared__ int cellI[kWarpsPerBlock][32][2];
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int64_t c0 = ((int64_t)blockIdx.x * kWarpsPerBlock + w) * 32;
    if (c0 >= g.ncells) return;
    const int64_t nc = g.ncells;
    const int M = g.max_xcell;
    {
        const int64_t c = min(c0 + lane, nc - 1);
        cellI[w][lane][0] = (int)(c % g.n[0]);
        cellI[w][lane][1] = (int)(c / g.n[0]);
    }
    uint64_t mine;
    const int K = build_slot_list(lists[w], index, c0, nc, M, lane, &mine);
    const float* Vc[2] = {V0, V1};
    const int64_t ns = stg.nslots;
    const double wd[2] = {(double)P.w[0], (double)P.w[1]}, awd[2] = {(double)P.aw[0], (double)P.aw[1]};
    float* tf = reinterpret_cast<float*>(stg.t);
    float* gkf = reinterpret_cast<float*>(stg.gk);
    int errs = 0;
    // the next particle's offsets and cotangents are loaded while this one is worked on
    auto fetch = [&](int kk, int64_t& a, int& l, float* x0, double* lam) {
        int s;
        slot_item(lists[w], M, kk, &s, &l);
        a = c0 + l + nc * s;
        x0[0] = Xi.x[0][a];
        x0[1] = Xi.x[1][a];
        lam[0] = Lam.c[0][a];
        lam[1] = Lam.c[1][a];
    };
    int64_t na = 0;
    int nl = 0;
    float nx0[2] = {0.0f, 0.0f};
    double nlam[2] = {0.0, 0.0};
    if (lane < K) fetch(lane, na, nl, nx0, nlam);
    for (int k = lane; k < K; k += 32) {
        const int64_t a = na;
        const int l = nl;
        const float x0[2] = {nx0[0], nx0[1]};
        const double lam[2] = {nlam[0], nlam[1]};
        if (k + 32 < K) fetch(k + 32, na, nl, nx0, nlam);
        const int I[2] = {cellI[w][l][0], cellI[w][l][1]};
        SampF S[NS][2];
        bool ok = true;
#pragma unroll
        for (int q = 0; q < NS; ++q) {
            float x[2];
#pragma unroll
            for (int d = 0; d < 2; ++d) {
                if (q == 0)
                    x[d] = x0[d];
                else if (METHOD == JP_RUNGE_KUTTA2)
                    x[d] = fmaf(P.aw[d], S[0][d].v, x0[d]);
                else if (q < 3)
                    x[d] = fmaf(0.5f * P.w[d], S[q - 1][d].v, x0[d]);
                else
                    x[d] = fmaf(P.w[d], S[2][d].v, x0[d]);
            }
#pragma unroll
            for (int cc = 0; cc < 2; ++cc) {
                S[q][cc] = sample2_f32(g, cc, I, x, Vc[cc]);
                ok &= S[q][cc].ok;
            }
            if (!ok) break;
        }
        if (!ok) {  // the forward sent this particle to Inf; move_particles! dropped it
            Lam.c[0][a] = 0.0;
            Lam.c[1][a] = 0.0;
#pragma unroll
            for (int q = 0; q < 2 * NS; ++q) stg.win[q * ns + a] = 0xFF;
            continue;
        }
        double gk[NS][2], l0[2] = {lam[0], lam[1]}, qb[2];
        if (METHOD == JP_RUNGE_KUTTA2) {
            const double A = P.half ? 0.0 : (double)P.ca, B = P.half ? 1.0 : (double)P.cb;
#pragma unroll
            for (int d = 0; d < 2; ++d) {
                gk[NS - 1][d] = wd[d] * B * lam[d];
                gk[0][d] = wd[d] * A * lam[d];
            }
            jt_f(S[NS - 1], gk[NS - 1], qb);  // x1 = x0 + aw v0
#pragma unroll
            for (int d = 0; d < 2; ++d) {
                l0[d] += qb[d];
                gk[0][d] += awd[d] * qb[d];
            }
        } else if (METHOD == JP_RUNGE_KUTTA4) {
#pragma unroll
            for (int d = 0; d < 2; ++d) {
                const double w6 = wd[d] / 6.0;
                gk[0][d] = w6 * lam[d];
                gk[1][d] = 2.0 * w6 * lam[d];
                gk[2][d] = 2.0 * w6 * lam[d];
                gk[NS - 1][d] = w6 * lam[d];
            }
#pragma unroll
            for (int q = NS - 1; q >= 1; --q) {
                jt_f(S[q], gk[q], qb);
#pragma unroll
                for (int d = 0; d < 2; ++d) {
                    l0[d] += qb[d];
                    gk[q - 1][d] += (q == 3 ? wd[d] : 0.5 * wd[d]) * qb[d];
                }
            }
        } else {
#pragma unroll
            for (int d = 0; d < 2; ++d) gk[0][d] = wd[d] * lam[d];
        }
        jt_f(S[0], gk[0], qb);
#pragma unroll
        for (int d = 0; d < 2; ++d) l0[d] += qb[d];
        Lam.c[0][a] = l0[0];
        Lam.c[1][a] = l0[1];
#pragma unroll
        for (int q = 0; q < NS; ++q)
#pragma unroll
            for (int cc = 0; cc < 2; ++cc) {
                const int j = 2 * q + cc;
                const int ox = S[q][cc].idx[0] - I[0] + 1, oy = S[q][cc].idx[1] - I[1] + 1;
                const bool in = ox >= 0 && ox <= win_nx(cc) - 2 && oy >= 0 && oy <= win_ny(cc) - 2;
                if (!in) errs |= kErrAdjointWindow;
                stg.win[j * ns + a] = in ? (uint8_t)(ox | (oy << 4)) : (uint8_t)0xFF;
                tf[(2 * j) * ns + a] = S[q][cc].t[0];  // FP32 staging (deposit_f32_kernel)
                tf[(2 * j + 1) * ns + a] = S[q][cc].t[1];
                gkf[j * ns + a] = (float)gk[q][cc];
            }
    }
    raise_err(d_err, errs);
}

// particle2grid! of the FP32 form, per particle: F_v = sum_i w_i f_i / W_v with
// w = 1 / ss, ss = sum_d ((k_d - xi_d) dx_d)^2 in FP32 (the forward's
// weights), so
//   dL/dFp_i  += sum_v gF_v w_i / W_v
//   dL/dxi_d  += sum_v gF_v (f_i - F_v) / W_v * 2 w_i^2 (k_d - xi_d) dx_d^2
__global__ void __launch_bounds__(32 * kWarpsPerBlock)
    p2g_vjp_f32_kernel(DevGrid g, F32Params P, const float* __restrict__ F, const double* __restrict__ W,
                       const float* __restrict__ Fp, CXiF Xi, const uint8_t* __restrict__ index,
                       const double* __restrict__ gF, double* __restrict__ gFp, Coords gX)
{
    __shared__ SlotList lists[kWarpsPerBlock];
    __shared__ int cellI[kWarpsPerBlock][32][2];
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int64_t c0 = ((int64_t)blockIdx.x * kWarpsPerBlock + w) * 32;
    if (c0 >= g.ncells) return;
    const int64_t nc = g.ncells;
    const int M = g.max_xcell;
    {
        const int64_t c = min(c0 + lane, nc - 1);
        cellI[w][lane][0] = (int)(c % g.n[0]);
        cellI[w][lane][1] = (int)(c / g.n[0]);
    }
    uint64_t mine;
    const int K = build_slot_list(lists[w], index, c0, nc, M, lane, &mine);
    const int64_t V0 = g.n[0] + 1;
    for (int k = lane; k < K; k += 32) {
        int s, l;
        slot_item(lists[w], M, k, &s, &l);
        const int64_t a = c0 + l + nc * s;
        const int I[2] = {cellI[w][l][0], cellI[w][l][1]};
        const float xi[2] = {Xi.x[0][a], Xi.x[1][a]};
        const double f = (double)Fp[a];
        double gf = 0.0, gx = 0.0, gy = 0.0;
        for (int kb = 0; kb < 2; ++kb)
            for (int ka = 0; ka < 2; ++ka) {
                const int64_t v = (I[0] + ka) + V0 * (I[1] + kb);
                const float ex = ((float)ka - xi[0]) * P.dx[0], ey = ((float)kb - xi[1]) * P.dx[1];
                float ss = 0.0f;
                ss = fmaf(ex, ex, ss);
                ss = fmaf(ey, ey, ss);
                const double wi = (double)p2g_weight_f32(ss);
                const double r = ldg(gF + v) / ldg(W + v);
                gf = fma(r, wi, gf);
                const double q = r * (f - (double)__ldg(F + v)) * 2.0 * wi * wi;
                gx = fma(q, (double)ex * (double)P.dx[0], gx);
                gy = fma(q, (double)ey * (double)P.dx[1], gy);
            }
        gFp[a] += gf;
        if (gX.c[0]) {
            gX.c[0][a] += gx;
            gX.c[1][a] += gy;
        }
    }
}

// dL/dV at every node of component `comp`: the partial sums of the owning
// cells whose window holds the node (cells y outer, x inner).
__global__ void __launch_bounds__(kThreads)
    vel_gather_kernel(DevGrid g, int comp, const double* __restrict__ parts, double* __restrict__ gV)
{
    const int64_t L0 = g.nvel[comp][0], L1 = g.nvel[comp][1];
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= L0 * L1) return;
    const int64_t i = t % L0, j = t / L0;
    const int NX = win_nx(comp), NY = win_ny(comp);
    const int64_t nc = g.ncells;
    double acc = 0.0;
    // owning cell (cx, cy) holds node (i, j) at window position (i - cx + 1, j - cy + 1)
    for (int64_t cy = max(j + 2 - NY, (int64_t)0); cy <= min(j + 1, g.n[1] - 1); ++cy)
        for (int64_t cx = max(i + 2 - NX, (int64_t)0); cx <= min(i + 1, g.n[0] - 1); ++cx) {
            const int k = (comp == 0 ? 0 : 20) + (int)(i - cx + 1) + NX * (int)(j - cy + 1);
            acc += parts[k * nc + cx + g.n[0] * cy];
        }
    gV[t] += acc;
}

// --------------------------------------------------------- particle2grid!
// per particle: F_v = sum_i w_vi Fp_i / W_v with w = 1 / |x_v - x_i|^2, so
//   dL/dFp_i += sum_v gF_v w_vi / W_v
//   dL/dx_i  += sum_v gF_v (Fp_i - F_v) / W_v * 2 (x_v - x_i) w_vi^2
__global__ void __launch_bounds__(32 * kWarpsPerBlock)
    p2g_vjp_kernel(DevGrid g, const double* __restrict__ F, const double* __restrict__ W,
                   const double* __restrict__ Fp, CCoords X, const uint8_t* __restrict__ index,
                   const double* __restrict__ gF, double* __restrict__ gFp, Coords gX)
{
    __shared__ SlotList lists[kWarpsPerBlock];
    __shared__ int cellI[kWarpsPerBlock][32][2];
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int64_t c0 = ((int64_t)blockIdx.x * kWarpsPerBlock + w) * 32;
    if (c0 >= g.ncells) return;
    const int64_t nc = g.ncells;
    const int M = g.max_xcell;
    {
        int64_t I[3];
        cell_coords(g, min(c0 + lane, nc - 1), I);
        cellI[w][lane][0] = (int)I[0];
        cellI[w][lane][1] = (int)I[1];
    }
    uint64_t mine;
    const int K = build_slot_list(lists[w], index, c0, nc, M, lane, &mine);
    const int64_t V0 = g.n[0] + 1;
    for (int k = lane; k < K; k += 32) {
        int s, l;
        slot_item(lists[w], M, k, &s, &l);
        const int64_t a = c0 + l + nc * s;
        const int I[2] = {cellI[w][l][0], cellI[w][l][1]};
        const double px = X.c[0][a], py = X.c[1][a], f = Fp[a];
        double gf = 0.0, gx = 0.0, gy = 0.0;
        for (int kb = 0; kb < 2; ++kb)
            for (int ka = 0; ka < 2; ++ka) {
                const int64_t v = (I[0] + ka) + V0 * (I[1] + kb);
                const double ex = ldg(g.xv[0] + I[0] + ka) - px, ey = ldg(g.xv[1] + I[1] + kb) - py;
                const double wi = inv_dist2(ex * ex + ey * ey);  // the forward weight, bit for bit
                const double r = ldg(gF + v) / ldg(W + v);
                gf = fma(r, wi, gf);
                const double q = r * (f - ldg(F + v)) * 2.0 * wi * wi;
                gx = fma(q, ex, gx);
                gy = fma(q, ey, gy);
            }
        gFp[a] += gf;
        if (gX.c[0]) {
            gX.c[0][a] += gx;
            gX.c[1][a] += gy;
        }
    }
}

// --------------------------------------------------------- grid2particle!
// dL/dF_v += sum over the particles of the (up to) four cells around v of
// gFp_i * (bilinear weight of v at x_i), cells y outer, x inner, slots ascending.
__global__ void __launch_bounds__(kThreads)
    g2p_vjp_kernel(DevGrid g, const double* __restrict__ gFp, CCoords X, const uint8_t* __restrict__ index,
                   double* __restrict__ gF)
{
    const int64_t V0 = g.n[0] + 1, V1 = g.n[1] + 1;
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= V0 * V1) return;
    const int64_t i = t % V0, j = t / V0;
    const int64_t nc = g.ncells;
    double acc = 0.0;
    for (int64_t cy = j - 1; cy <= j; ++cy) {
        if (cy < 0 || cy >= g.n[1]) continue;
        for (int64_t cx = i - 1; cx <= i; ++cx) {
            if (cx < 0 || cx >= g.n[0]) continue;
            const int64_t c = cx + g.n[0] * cy;
            const double x0 = ldg(g.xv[0] + cx), y0 = ldg(g.xv[1] + cy);
            const double ixx = ldg(g.ixv[0] + cx), iyy = ldg(g.ixv[1] + cy);
            uint64_t m = live_mask(index, c, nc, g.max_xcell);
            while (m) {
                const int s = __ffsll((long long)m) - 1;
                m &= m - 1;
                const int64_t a = c + nc * s;
                const double tx = (X.c[0][a] - x0) * ixx, ty = (X.c[1][a] - y0) * iyy;
                const double fx = cx == i ? 1.0 - tx : tx;
                const double fy = cy == j ? 1.0 - ty : ty;
                acc = fma(gFp[a], fx * fy, acc);
            }
        }
    }
    gF[t] += acc;
}

// dL/dx_i += gFp_i * grad(bilinear F)(x_i)
__global__ void __launch_bounds__(kThreads)
    g2p_vjp_pos_kernel(DevGrid g, const double* __restrict__ F, const double* __restrict__ gFp, CCoords X,
                       const uint8_t* __restrict__ index, Coords gX)
{
    const int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= g.ncells) return;
    const int64_t nc = g.ncells;
    const int64_t cx = c % g.n[0], cy = c / g.n[0];
    const int64_t V0 = g.n[0] + 1;
    const double* b = F + cx + V0 * cy;
    const double f00 = ldg(b), f10 = ldg(b + 1), f01 = ldg(b + V0), f11 = ldg(b + V0 + 1);
    const double x0 = ldg(g.xv[0] + cx), y0 = ldg(g.xv[1] + cy);
    const double ixx = ldg(g.ixv[0] + cx), iyy = ldg(g.ixv[1] + cy);
    uint64_t m = live_mask(index, c, nc, g.max_xcell);
    while (m) {
        const int s = __ffsll((long long)m) - 1;
        m &= m - 1;
        const int64_t a = c + nc * s;
        const double tx = (X.c[0][a] - x0) * ixx, ty = (X.c[1][a] - y0) * iyy;
        const double gp = gFp[a];
        gX.c[0][a] += gp * ((1.0 - ty) * (f10 - f00) + ty * (f11 - f01)) * ixx;
        gX.c[1][a] += gp * ((1.0 - tx) * (f01 - f00) + tx * (f11 - f10)) * iyy;
    }
}

// ----------------------------------------------- the transfers in 3D
// The same products over the 8 corners of a cell. The forward weight is
// inv((dx^2 + dy^2) + dz^2) with d = vertex - particle, as particle2grid! forms
// it in 3D; corners are taken x fastest, then y, then z.
__global__ void __launch_bounds__(32 * kWarpsPerBlock)
    p2g_vjp_kernel3(DevGrid g, const double* __restrict__ F, const double* __restrict__ W,
                    const double* __restrict__ Fp, CCoords X, const uint8_t* __restrict__ index,
                    const double* __restrict__ gF, double* __restrict__ gFp, Coords gX)
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
        for (int d = 0; d < 3; ++d) cellI[w][lane][d] = (int)I[d];
    }
    uint64_t mine;
    const int K = build_slot_list(lists[w], index, c0, nc, M, lane, &mine);
    const int64_t V0 = g.n[0] + 1, V1 = g.n[1] + 1;
    for (int k = lane; k < K; k += 32) {
        int s, l;
        slot_item(lists[w], M, k, &s, &l);
        const int64_t a = c0 + l + nc * s;
        const int I[3] = {cellI[w][l][0], cellI[w][l][1], cellI[w][l][2]};
        const double p[3] = {X.c[0][a], X.c[1][a], X.c[2][a]};
        const double f = Fp[a];
        double gf = 0.0, gx[3] = {0.0, 0.0, 0.0};
        for (int q = 0; q < 8; ++q) {
            const int o[3] = {q & 1, (q >> 1) & 1, q >> 2};
            const int64_t v = (I[0] + o[0]) + V0 * ((I[1] + o[1]) + V1 * (int64_t)(I[2] + o[2]));
            double e[3];
            for (int d = 0; d < 3; ++d) e[d] = ldg(g.xv[d] + I[d] + o[d]) - p[d];
            const double wi = inv_dist2((e[0] * e[0] + e[1] * e[1]) + e[2] * e[2]);
            const double r = ldg(gF + v) / ldg(W + v);
            gf = fma(r, wi, gf);
            const double qd = r * (f - ldg(F + v)) * 2.0 * wi * wi;
            for (int d = 0; d < 3; ++d) gx[d] = fma(qd, e[d], gx[d]);
        }
        gFp[a] += gf;
        if (gX.c[0])
            for (int d = 0; d < 3; ++d) gX.c[d][a] += gx[d];
    }
}

// dL/dF_v of grid2particle! in 3D: the (up to) eight cells around v, z outer,
// then y, then x, slots ascending; weight = product of the per-axis linear weights.
__global__ void __launch_bounds__(kThreads)
    g2p_vjp_kernel3(DevGrid g, const double* __restrict__ gFp, CCoords X, const uint8_t* __restrict__ index,
                    double* __restrict__ gF)
{
    const int64_t V0 = g.n[0] + 1, V1 = g.n[1] + 1, V2 = g.n[2] + 1;
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= V0 * V1 * V2) return;
    const int64_t i = t % V0, j = (t / V0) % V1, kz = t / (V0 * V1);
    const int64_t nc = g.ncells;
    double acc = 0.0;
    for (int64_t cz = kz - 1; cz <= kz; ++cz) {
        if (cz < 0 || cz >= g.n[2]) continue;
        for (int64_t cy = j - 1; cy <= j; ++cy) {
            if (cy < 0 || cy >= g.n[1]) continue;
            for (int64_t cx = i - 1; cx <= i; ++cx) {
                if (cx < 0 || cx >= g.n[0]) continue;
                const int64_t c = cx + g.n[0] * (cy + g.n[1] * cz);
                const double x0 = ldg(g.xv[0] + cx), y0 = ldg(g.xv[1] + cy), z0 = ldg(g.xv[2] + cz);
                const double ixx = ldg(g.ixv[0] + cx), iyy = ldg(g.ixv[1] + cy), izz = ldg(g.ixv[2] + cz);
                uint64_t m = live_mask(index, c, nc, g.max_xcell);
                while (m) {
                    const int s = __ffsll((long long)m) - 1;
                    m &= m - 1;
                    const int64_t a = c + nc * s;
                    const double tx = (X.c[0][a] - x0) * ixx, ty = (X.c[1][a] - y0) * iyy,
                                 tz = (X.c[2][a] - z0) * izz;
                    const double fx = cx == i ? 1.0 - tx : tx;
                    const double fy = cy == j ? 1.0 - ty : ty;
                    const double fz = cz == kz ? 1.0 - tz : tz;
                    acc = fma(gFp[a], fx * fy * fz, acc);
                }
            }
        }
    }
    gF[t] += acc;
}

// dL/dx_i += gFp_i * grad(trilinear F)(x_i): along axis d, the differences of
// the corner values across d weighted by the other two axes' linear weights.
__global__ void __launch_bounds__(kThreads)
    g2p_vjp_pos_kernel3(DevGrid g, const double* __restrict__ F, const double* __restrict__ gFp, CCoords X,
                        const uint8_t* __restrict__ index, Coords gX)
{
    const int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= g.ncells) return;
    const int64_t nc = g.ncells;
    int64_t I[3];
    cell_coords(g, c, I);
    const int64_t V0 = g.n[0] + 1, V1 = g.n[1] + 1;
    const double* b = F + I[0] + V0 * (I[1] + V1 * I[2]);
    double f[8];  // corner q = x + 2 y + 4 z
    for (int q = 0; q < 8; ++q) f[q] = ldg(b + (q & 1) + V0 * ((q >> 1) & 1) + V0 * V1 * (q >> 2));
    double x0[3], ix[3];
    for (int d = 0; d < 3; ++d) {
        x0[d] = ldg(g.xv[d] + I[d]);
        ix[d] = ldg(g.ixv[d] + I[d]);
    }
    uint64_t m = live_mask(index, c, nc, g.max_xcell);
    while (m) {
        const int s = __ffsll((long long)m) - 1;
        m &= m - 1;
        const int64_t a = c + nc * s;
        double t[3];
        for (int d = 0; d < 3; ++d) t[d] = (X.c[d][a] - x0[d]) * ix[d];
        const double gp = gFp[a];
        for (int d = 0; d < 3; ++d) {
            const int e1 = d == 0 ? 1 : 0, e2 = d == 2 ? 1 : 2;  // the other two axes
            double acc = 0.0;
            for (int q = 0; q < 8; ++q) {
                if (!((q >> d) & 1)) continue;
                const double w1 = (q >> e1) & 1 ? t[e1] : 1.0 - t[e1];
                const double w2 = (q >> e2) & 1 ? t[e2] : 1.0 - t[e2];
                acc = fma(f[q] - f[q - (1 << d)], w1 * w2, acc);
            }
            gX.c[d][a] += gp * acc * ix[d];
        }
    }
}

// ------------------------------------------------------------ launchers
// Adjoint scratch: the 40 window partial sums and the injected-slot mask per
// cell, then the per-slot staging of up to 8 velocity samples (RK4).
constexpr int kMaxSamples = 8;

static size_t adjoint_scratch_bytes(const DevGrid& g)
{
    const size_t nc = (size_t)g.ncells, ns = nc * (size_t)g.max_xcell;
    return nc * (kWinParts * sizeof(double) + sizeof(uint64_t)) +
           ns * kMaxSamples * (3 * sizeof(double) + sizeof(uint8_t)) + nc * sizeof(unsigned);
}

static cudaError_t ensure_adjoint_scratch(jp_particles* P)
{
    if (P->adj_rec) return cudaSuccess;
    return cudaMalloc(&P->adj_rec, adjoint_scratch_bytes(P->g));
}

static double* adj_parts(jp_particles* P) { return (double*)P->adj_rec; }
static uint64_t* adj_inj(jp_particles* P) { return (uint64_t*)((double*)P->adj_rec + kWinParts * P->g.ncells); }

static Staging adj_staging(jp_particles* P)
{
    const int64_t nc = P->g.ncells, ns = nc * P->g.max_xcell;
    Staging s;
    s.t = (double*)(adj_inj(P) + nc);
    s.gk = s.t + 2 * kMaxSamples * ns;
    s.win = (uint8_t*)(s.gk + kMaxSamples * ns);
    s.nslots = ns;
    return s;
}

static unsigned* adj_srcflag(jp_particles* P)
{
    const Staging s = adj_staging(P);
    return (unsigned*)(s.win + kMaxSamples * s.nslots);
}

cudaError_t launch_move_permutation(jp_particles* P, int32_t* dest)
{
    const MoveScratch& m = P->move;
    if (!m.rec) return cudaErrorInvalidValue;
    const unsigned nb = grid_blocks(P->g.ncells);
    MoveView S{m.rec, P->g.ncells, m.code, m.orig, m.shadow, P->g.ncells * P->g.max_xcell, 0, P->g.max_xcell};
    perm_init<<<nb, kThreads, 0, P->stream>>>(P->g, S, dest);
    if (P->g.ndim == 2)
        perm_scatter<2><<<nb, kThreads, 0, P->stream>>>(P->g, S, dest);
    else
        perm_scatter<3><<<nb, kThreads, 0, P->stream>>>(P->g, S, dest);
    return cudaGetLastError();
}

static PermArrays perm_arrays(const double* const* post, double* const* pre, int n)
{
    PermArrays A{};
    A.n = n;
    for (int k = 0; k < n; ++k) {
        A.post[k] = post[k];
        A.pre[k] = pre[k];
    }
    return A;
}

cudaError_t launch_permute_vjp(jp_particles* P, const int32_t* dest, const double* const* post, double* const* pre,
                               int n)
{
    const int64_t ns = P->g.ncells * P->g.max_xcell;
    permute_vjp_kernel<<<grid_blocks(ns), kThreads, 0, P->stream>>>(ns, dest, perm_arrays(post, pre, n));
    return cudaGetLastError();
}

template <typename IdT>
static cudaError_t slot_ids(jp_particles* P, const uint8_t* index, IdT* ids)
{
    const int64_t ns = P->g.ncells * P->g.max_xcell;
    slot_ids_kernel<IdT><<<grid_blocks(ns), kThreads, 0, P->stream>>>(ns, index, ids);
    return cudaGetLastError();
}

cudaError_t launch_slot_ids(jp_particles* P, const uint8_t* index, double* ids) { return slot_ids(P, index, ids); }
cudaError_t launch_slot_ids_i32(jp_particles* P, const uint8_t* index, int32_t* ids)
{
    return slot_ids(P, index, ids);
}

template <typename IdT>
static cudaError_t inject_vjp(jp_particles* P, const IdT* ids, const double* const* post, double* const* pre, int n,
                              unsigned copies)
{
    cudaError_t e = ensure_adjoint_scratch(P);
    if (e != cudaSuccess) return e;
    const unsigned nb = grid_blocks(P->g.ncells);
    const bool inplace = n > 0 && post[0] == pre[0];  // the C ABI checked that all or none alias
    if (copies) {
        e = cudaMemsetAsync(adj_srcflag(P), 0, (size_t)P->g.ncells * sizeof(unsigned), P->stream);
        if (e != cudaSuccess) return e;
        inject_mask_kernel<IdT><<<nb, kThreads, 0, P->stream>>>(P->g, ids, adj_inj(P), adj_srcflag(P), P->d_err);
    }
    if (inplace) {
        if (copies)
            inject_vjp_inplace_kernel<IdT><<<nb, kThreads, 0, P->stream>>>(P->g, ids, adj_inj(P), adj_srcflag(P),
                                                                           perm_arrays(post, pre, n), copies);
    } else {
        inject_vjp_kernel<IdT><<<nb, kThreads, 0, P->stream>>>(P->g, ids, adj_inj(P), adj_srcflag(P),
                                                               perm_arrays(post, pre, n), copies);
    }
    return cudaGetLastError();
}

cudaError_t launch_inject_vjp(jp_particles* P, const double* ids, const double* const* post, double* const* pre,
                              int n, unsigned copies)
{
    return inject_vjp(P, ids, post, pre, n, copies);
}
cudaError_t launch_inject_vjp_i32(jp_particles* P, const int32_t* ids, const double* const* post,
                                  double* const* pre, int n, unsigned copies)
{
    return inject_vjp(P, ids, post, pre, n, copies);
}

static AdjParams adj_params(int method, double alpha, double dt)
{
    AdjParams prm;
    prm.method = method;
    prm.dt = dt;
    prm.adt = alpha * dt;
    const double ia = 1.0 / alpha;  // the forward's coefficients (alpha == 1/2 takes the dt * V(X1) form)
    prm.ca = alpha == 0.5 ? 0.0 : std::fma(-0.5, ia, 1.0);
    prm.cb = alpha == 0.5 ? 1.0 : 0.5 * ia;
    prm.half = alpha == 0.5;
    return prm;
}

template <int METHOD>
static cudaError_t launch_advect_vjp(jp_particles* P, cudaStream_t st, const double* const V[3],
                                     const AdjParams& prm, const CCoords& X, const uint8_t* index, const Coords& L)
{
    const Staging stg = adj_staging(P);
    advect_vjp_kernel<METHOD><<<grid_blocks(P->g.ncells, 32 * kWarpsPerBlock), 32 * kWarpsPerBlock, 0, st>>>(
        P->g, V[0], V[1], prm, X, index, L, stg, P->d_err);
    deposit_kernel<2 * adj_stages<METHOD>()><<<grid_blocks(P->g.ncells, kDepThreads), kDepThreads, 0, st>>>(
        P->g, index, stg, adj_parts(P));
    return cudaGetLastError();
}

cudaError_t launch_advection_vjp(jp_particles* P, int method, double alpha, const double* const V[3], double dt,
                                 const double* const coords[3], const uint8_t* index, double* const lam[3],
                                 double* const gV[3])
{
    cudaError_t e = ensure_adjoint_scratch(P);
    if (e != cudaSuccess) return e;
    const AdjParams prm = adj_params(method, alpha, dt);
    CCoords X{{coords[0], coords[1], nullptr}};
    Coords L{{lam[0], lam[1], nullptr}};
    cudaStream_t st = P->stream;
    if (method == JP_RUNGE_KUTTA2)
        e = launch_advect_vjp<JP_RUNGE_KUTTA2>(P, st, V, prm, X, index, L);
    else if (method == JP_RUNGE_KUTTA4)
        e = launch_advect_vjp<JP_RUNGE_KUTTA4>(P, st, V, prm, X, index, L);
    else
        e = launch_advect_vjp<JP_EULER>(P, st, V, prm, X, index, L);
    if (e != cudaSuccess) return e;
    for (int c = 0; c < 2; ++c) {
        const int64_t nn = P->g.nvel[c][0] * P->g.nvel[c][1];
        vel_gather_kernel<<<grid_blocks(nn), kThreads, 0, st>>>(P->g, c, adj_parts(P), gV[c]);
    }
    return cudaGetLastError();
}

static int method_samples(int method)
{
    return method == JP_RUNGE_KUTTA4 ? 8 : (method == JP_RUNGE_KUTTA2 ? 4 : 2);
}

size_t advection_record_bytes(const jp_particles* P, int method)
{
    return record_bytes(P->g.ncells * P->g.max_xcell, method_samples(method));
}

cudaError_t launch_advection_record(jp_particles* P, int method, double alpha, const double* const V[3], double dt,
                                    double* const coords[3], const uint8_t* index, void* rec)
{
    const AdjParams prm = adj_params(method, alpha, dt);
    Coords X{{coords[0], coords[1], nullptr}};
    const int64_t ns = P->g.ncells * P->g.max_xcell;
    const Record r = record_view(rec, ns, method_samples(method));
    const unsigned nb = grid_blocks(P->g.ncells, 32 * kWarpsPerBlock);
    const int nt = 32 * kWarpsPerBlock;
    cudaStream_t st = P->stream;
    if (method == JP_RUNGE_KUTTA2)
        advect_record_kernel<JP_RUNGE_KUTTA2><<<nb, nt, 0, st>>>(P->g, V[0], V[1], prm, X, index, r, P->d_err);
    else if (method == JP_RUNGE_KUTTA4)
        advect_record_kernel<JP_RUNGE_KUTTA4><<<nb, nt, 0, st>>>(P->g, V[0], V[1], prm, X, index, r, P->d_err);
    else
        advect_record_kernel<JP_EULER><<<nb, nt, 0, st>>>(P->g, V[0], V[1], prm, X, index, r, P->d_err);
    return cudaGetLastError();
}

cudaError_t launch_advection_vjp_recorded(jp_particles* P, int method, double alpha, double dt, const void* rec,
                                          const uint8_t* index, double* const lam[3], double* const gV[3])
{
    cudaError_t e = ensure_adjoint_scratch(P);
    if (e != cudaSuccess) return e;
    const AdjParams prm = adj_params(method, alpha, dt);
    Coords L{{lam[0], lam[1], nullptr}};
    const int64_t ns = P->g.ncells * P->g.max_xcell;
    const int nq = method_samples(method);
    const Record r = record_view(const_cast<void*>(rec), ns, nq);
    Staging stg = adj_staging(P);
    stg.t = r.t;  // the deposit reads the recorded coordinates and windows
    stg.win = r.win;
    cudaStream_t st = P->stream;
    const unsigned nb = grid_blocks(P->g.ncells, 32 * kWarpsPerBlock);
    const unsigned nd = grid_blocks(P->g.ncells, kDepThreads);
    const int nt = 32 * kWarpsPerBlock;
    if (method == JP_RUNGE_KUTTA2) {
        advect_vjp_rec_kernel<JP_RUNGE_KUTTA2><<<nb, nt, 0, st>>>(P->g, prm, index, r, L, stg.gk);
        deposit_kernel<4><<<nd, kDepThreads, 0, st>>>(P->g, index, stg, adj_parts(P));
    } else if (method == JP_RUNGE_KUTTA4) {
        advect_vjp_rec_kernel<JP_RUNGE_KUTTA4><<<nb, nt, 0, st>>>(P->g, prm, index, r, L, stg.gk);
        deposit_kernel<8><<<nd, kDepThreads, 0, st>>>(P->g, index, stg, adj_parts(P));
    } else {
        advect_vjp_rec_kernel<JP_EULER><<<nb, nt, 0, st>>>(P->g, prm, index, r, L, stg.gk);
        deposit_kernel<2><<<nd, kDepThreads, 0, st>>>(P->g, index, stg, adj_parts(P));
    }
    for (int c = 0; c < 2; ++c) {
        const int64_t nn = P->g.nvel[c][0] * P->g.nvel[c][1];
        vel_gather_kernel<<<grid_blocks(nn), kThreads, 0, st>>>(P->g, c, adj_parts(P), gV[c]);
    }
    return cudaGetLastError();
}

cudaError_t launch_advection_vjp_f32(jp_particles* P, int method, double alpha, const float* const V[3], double dt,
                                     const float* const xi[3], const uint8_t* index, double* const lam[3],
                                     double* const gV[3])
{
    cudaError_t e = ensure_adjoint_scratch(P);
    if (e != cudaSuccess) return e;
    const F32Params prm = make_params(P, alpha, dt);
    CXiF X{{xi[0], xi[1], nullptr}};
    Coords L{{lam[0], lam[1], nullptr}};
    const Staging stg = adj_staging(P);
    cudaStream_t st = P->stream;
    const unsigned nb = grid_blocks(P->g.ncells, 32 * kWarpsPerBlock);
    const unsigned nd = grid_blocks(P->g.ncells, kDepThreads);
    const int nt = 32 * kWarpsPerBlock;
    if (method == JP_RUNGE_KUTTA2) {
        advect_vjp_f32_kernel<JP_RUNGE_KUTTA2><<<nb, nt, 0, st>>>(P->g, V[0], V[1], prm, X, index, L, stg, P->d_err);
        deposit_f32_kernel<4><<<nd, kDepThreads, 0, st>>>(P->g, index, stg, adj_parts(P));
    } else if (method == JP_RUNGE_KUTTA4) {
        advect_vjp_f32_kernel<JP_RUNGE_KUTTA4><<<nb, nt, 0, st>>>(P->g, V[0], V[1], prm, X, index, L, stg, P->d_err);
        deposit_f32_kernel<8><<<nd, kDepThreads, 0, st>>>(P->g, index, stg, adj_parts(P));
    } else {
        advect_vjp_f32_kernel<JP_EULER><<<nb, nt, 0, st>>>(P->g, V[0], V[1], prm, X, index, L, stg, P->d_err);
        deposit_f32_kernel<2><<<nd, kDepThreads, 0, st>>>(P->g, index, stg, adj_parts(P));
    }
    for (int c = 0; c < 2; ++c) {
        const int64_t nn = P->g.nvel[c][0] * P->g.nvel[c][1];
        vel_gather_kernel<<<grid_blocks(nn), kThreads, 0, st>>>(P->g, c, adj_parts(P), gV[c]);
    }
    return cudaGetLastError();
}

cudaError_t launch_p2g_vjp_f32(jp_particles* P, const float* F, const double* W, const float* Fp,
                               const float* const xi[3], const uint8_t* index, const double* gF, double* gFp,
                               double* const gxi[3])
{
    const F32Params prm = make_params(P, 0.5, 0.0);
    CXiF X{{xi[0], xi[1], nullptr}};
    Coords G{{gxi ? gxi[0] : nullptr, gxi ? gxi[1] : nullptr, nullptr}};
    p2g_vjp_f32_kernel<<<grid_blocks(P->g.ncells, 32 * kWarpsPerBlock), 32 * kWarpsPerBlock, 0, P->stream>>>(
        P->g, prm, F, W, Fp, X, index, gF, gFp, G);
    return cudaGetLastError();
}

cudaError_t launch_p2g_vjp(jp_particles* P, const double* F, const double* W, const double* Fp,
                           const double* const coords[3], const uint8_t* index, const double* gF, double* gFp,
                           double* const gX[3])
{
    const bool d3 = P->g.ndim == 3;
    CCoords X{{coords[0], coords[1], d3 ? coords[2] : nullptr}};
    Coords G{{gX ? gX[0] : nullptr, gX ? gX[1] : nullptr, gX && d3 ? gX[2] : nullptr}};
    const unsigned nb = grid_blocks(P->g.ncells, 32 * kWarpsPerBlock);
    if (d3)
        p2g_vjp_kernel3<<<nb, 32 * kWarpsPerBlock, 0, P->stream>>>(P->g, F, W, Fp, X, index, gF, gFp, G);
    else
        p2g_vjp_kernel<<<nb, 32 * kWarpsPerBlock, 0, P->stream>>>(P->g, F, W, Fp, X, index, gF, gFp, G);
    return cudaGetLastError();
}

cudaError_t launch_g2p_vjp(jp_particles* P, const double* F, const double* gFp, const double* const coords[3],
                           const uint8_t* index, double* gF, double* const gX[3])
{
    if (P->g.ndim == 3) {
        CCoords X{{coords[0], coords[1], coords[2]}};
        if (gF) {
            const int64_t nv = (P->g.n[0] + 1) * (P->g.n[1] + 1) * (P->g.n[2] + 1);
            g2p_vjp_kernel3<<<grid_blocks(nv), kThreads, 0, P->stream>>>(P->g, gFp, X, index, gF);
        }
        if (gX) {
            Coords G{{gX[0], gX[1], gX[2]}};
            g2p_vjp_pos_kernel3<<<grid_blocks(P->g.ncells), kThreads, 0, P->stream>>>(P->g, F, gFp, X, index, G);
        }
        return cudaGetLastError();
    }
    CCoords X{{coords[0], coords[1], nullptr}};
    if (gF) {
        const int64_t nv = (P->g.n[0] + 1) * (P->g.n[1] + 1);
        g2p_vjp_kernel<<<grid_blocks(nv), kThreads, 0, P->stream>>>(P->g, gFp, X, index, gF);
    }
    if (gX) {
        Coords G{{gX[0], gX[1], nullptr}};
        g2p_vjp_pos_kernel<<<grid_blocks(P->g.ncells), kThreads, 0, P->stream>>>(P->g, F, gFp, X, index, G);
    }
    return cudaGetLastError();
}

}  // namespace jp
