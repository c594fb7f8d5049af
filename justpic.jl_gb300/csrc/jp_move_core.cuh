// jp_move_core.cuh -- the slot-allocation stage of move_particles!, shared by
// the FP64 and the split-precision (FP32 cell offset) forms: it works on
// occupancy masks and destination codes only, whatever the particle data.
#pragma once

#include "jp_internal.cuh"

namespace jp {

constexpr int kAllocThreads = 64;  // small blocks spread the sparse colour passes over all SMs

// Per-cell 64-bit slot masks, one array of ncells words each (a warp's
// accesses to one mask are coalesced): the occupancy L, the refilled slots R,
// the refilled slots whose particle is not strictly inside U, the occupancy
// before the move L0 and the movers M; in 2D also the movers bound for each
// of the 9 neighbours and the movers not strictly inside their new cell.
constexpr int kRecWords2D = 15;
constexpr int kRecWords3D = 5;

struct MoveView {
    uint64_t* rec;  // the mask arrays, one after the other
    int64_t nc;     // cells (the length of each mask array)
    uint8_t* code;
    uint16_t* orig;
    double* shadow;
    int64_t nslots;
    int comps;  // stride of the shadow records: DIM coordinates, then the fields (records are interleaved)
    __device__ __forceinline__ uint64_t& L(int64_t c) const { return rec[c]; }
    __device__ __forceinline__ uint64_t& R(int64_t c) const { return rec[nc + c]; }
    __device__ __forceinline__ uint64_t& U(int64_t c) const { return rec[2 * nc + c]; }
    __device__ __forceinline__ uint64_t& L0(int64_t c) const { return rec[3 * nc + c]; }
    __device__ __forceinline__ uint64_t& M(int64_t c) const { return rec[4 * nc + c]; }
    // 2D: k < 9 movers bound for neighbour k, k = 9 movers not strictly inside their new cell
    __device__ __forceinline__ uint64_t& T(int64_t c, int k) const { return rec[(5 + k) * nc + c]; }
};

constexpr int kTargetMasks2D = 10;

// -------------------------------------------------------------- allocate
// One colour pass of move_particles!: sources 3*J + o, neighbourhoods
// disjoint, so every mask touched here belongs to exactly one thread. The
// destination codes and the masks of every neighbour the walk will touch are
// loaded up front (independent loads), the walk then runs on thread-local
// copies, and the touched masks are written back at the end.
template <int DIM>
__global__ void __launch_bounds__(kAllocThreads)
    move_allocate(DevGrid g, MoveView S, int o0, int o1, int o2, int64_t m0, int64_t m1, int64_t m2)
{
    constexpr int NB = DIM == 2 ? 9 : 27;
    constexpr int CENTER = DIM == 2 ? 4 : 13;
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
    const uint64_t Mv = S.M(sc);
    const uint64_t U0 = S.U(sc);
    if (Mv == 0 && U0 == 0) return;
    uint64_t nL[NB], nR[NB], nU[NB];
    uint8_t codes[64];
    nL[CENTER] = S.L(sc);
    nR[CENTER] = S.R(sc);
    nU[CENTER] = U0;
    uint32_t touched = 1u << CENTER;
    // codes of the original movers (slots not refilled by an earlier pass)
    uint64_t orig_movers = Mv & ~nR[CENTER];
    for (uint64_t m = orig_movers; m; m &= m - 1) {
        const int s = __ffsll((long long)m) - 1;
        const uint8_t cb = S.code[sc + nc * s];
        codes[s] = cb;
        if (cb != kCodeExit) touched |= 1u << (cb & 0x1F);
    }
    for (uint32_t m = touched & ~(1u << CENTER); m; m &= m - 1) {
        const int nb = __ffs(m) - 1;
        int off[3];
        nb_offset<DIM>(nb, off);
        const int64_t J[3] = {idx[0] + off[0], idx[1] + off[1], DIM == 3 ? idx[2] + off[2] : 0};
        const int64_t jc = cell_linear<DIM>(g, J);
        nL[nb] = S.L(jc);
        nR[nb] = S.R(jc);
        nU[nb] = S.U(jc);
    }
    const int nslot = g.max_xcell;
    const uint64_t valid = nslot == 64 ? ~0ull : ((1ull << nslot) - 1);
    int sp = 0;  // starting_point (move_safe.jl:83)
    int cur = 0;
    while (cur < nslot) {
        const uint64_t L = nL[CENTER], R = nR[CENTER], U = nU[CENTER];
        const uint64_t cand = L & ((Mv & ~R) | (R & U)) & (~0ull << cur);
        if (!cand) break;
        const int s = __ffsll((long long)cand) - 1;
        cur = s + 1;
        const uint64_t bit = 1ull << s;
        int code;
        bool unstable;
        const bool from_refill = (R & bit) != 0;
        uint16_t tag = 0;
        if (from_refill) {
            code = CENTER;
            unstable = true;
            tag = S.orig[sc + nc * s];
        } else {
            const uint8_t cb = codes[s];
            if (cb == kCodeExit) {  // left the domain (or moved too far): cleared
                nL[CENTER] = L & ~bit;
                continue;
            }
            code = cb & 0x1F;
            unstable = (cb & kCodeUnstable) != 0;
            int off[3];
            nb_offset<DIM>(code, off);
            const int back[3] = {-off[0], -off[1], -off[2]};
            tag = (uint16_t)(nb_code<DIM>(back) | (s << 5));
        }
        // remove the particle from its slot (move_safe.jl:110-112)
        nL[CENTER] = L & ~bit;
        nR[CENTER] = R & ~bit;
        nU[CENTER] = U & ~bit;
        // find_free_memory(starting_point, ...) (move_safe.jl:192-197)
        const uint64_t freem = ~nL[code] & valid & (~0ull << sp);
        if (!freem) continue;  // dropped: no free slot at or after starting_point
        const int f = __ffsll((long long)freem) - 1;
        sp = f;
        const uint64_t fb = 1ull << f;
        nL[code] |= fb;
        nR[code] |= fb;
        nU[code] = unstable ? (nU[code] | fb) : (nU[code] & ~fb);
        int off[3];
        nb_offset<DIM>(code, off);
        const int64_t T[3] = {idx[0] + off[0], idx[1] + off[1], DIM == 3 ? idx[2] + off[2] : 0};
        S.orig[cell_linear<DIM>(g, T) + nc * f] = tag;
    }
    for (uint32_t m = touched; m; m &= m - 1) {
        const int nb = __ffs(m) - 1;
        int off[3];
        nb_offset<DIM>(nb, off);
        const int64_t J[3] = {idx[0] + off[0], idx[1] + off[1], DIM == 3 ? idx[2] + off[2] : 0};
        const int64_t jc = cell_linear<DIM>(g, J);
        S.L(jc) = nL[nb];
        S.R(jc) = nR[nb];
        S.U(jc) = nU[nb];
    }
}

// The 2D colour pass with the whole walk in registers: the destinations come
// as nine per-target masks written by the classify stage (plus the mask of
// particles that are not strictly inside their new cell), the occupancy masks
// of the 3x3 neighbourhood are loaded once, and every update selects its
// target with unrolled predicated operations, so no thread-local array is
// indexed at run time. Same walk, same result as move_allocate<2>.
static __global__ void __launch_bounds__(kAllocThreads)
    move_allocate_2d(DevGrid g, MoveView S, int o0, int o1, int64_t m0, int64_t m1)
{
    constexpr int CENTER = 4;
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= m0 * m1) return;
    const int64_t ix = 3 * (t % m0) + o0, iy = 3 * (t / m0) + o1;
    if (ix >= g.n[0] || iy >= g.n[1]) return;
    const int64_t nc = g.ncells;
    const int64_t sc = ix + g.n[0] * iy;
    const uint64_t Mv = S.M(sc);
    const uint64_t U0 = S.U(sc);
    if (Mv == 0 && U0 == 0) return;
    uint64_t nL[9], nR[9], nU[9], tm[9];
#pragma unroll
    for (int k = 0; k < 9; ++k) {
        const int64_t jx = ix + k % 3 - 1, jy = iy + k / 3 - 1;
        const bool in = jx >= 0 && jy >= 0 && jx < g.n[0] && jy < g.n[1];
        const int64_t jc = jx + g.n[0] * jy;
        nL[k] = in ? S.L(jc) : 0;
        nR[k] = in ? S.R(jc) : 0;
        nU[k] = in ? S.U(jc) : 0;
        tm[k] = S.T(sc, k);
    }
    const uint64_t unst = S.T(sc, 9);
    const int nslot = g.max_xcell;
    const uint64_t valid = nslot == 64 ? ~0ull : ((1ull << nslot) - 1);
    uint32_t touched = 1u << CENTER;
    int sp = 0;  // starting_point (move_safe.jl:83)
    int cur = 0;
    while (cur < nslot) {
        const uint64_t L = nL[CENTER], R = nR[CENTER], U = nU[CENTER];
        const uint64_t cand = L & ((Mv & ~R) | (R & U)) & (~0ull << cur);
        if (!cand) break;
        const int s = __ffsll((long long)cand) - 1;
        cur = s + 1;
        const uint64_t bit = 1ull << s;
        int code = -1;
        bool unstable;
        uint16_t tag;
        if (R & bit) {  // refilled by an earlier pass and not strictly inside: walked again
            code = CENTER;
            unstable = true;
            tag = S.orig[sc + nc * s];
        } else {
#pragma unroll
            for (int k = 0; k < 9; ++k)
                if (tm[k] & bit) code = k;
            if (code < 0) {  // left the domain (or moved too far): cleared
                nL[CENTER] = L & ~bit;
                continue;
            }
            unstable = (unst & bit) != 0;
            const int back = (1 - (code % 3 - 1)) + 3 * (1 - (code / 3 - 1));
            tag = (uint16_t)(back | (s << 5));
        }
        // remove the particle from its slot (move_safe.jl:110-112)
        nL[CENTER] = L & ~bit;
        nR[CENTER] = R & ~bit;
        nU[CENTER] = U & ~bit;
        // find_free_memory(starting_point, ...) (move_safe.jl:192-197)
        uint64_t tL = 0;
#pragma unroll
        for (int k = 0; k < 9; ++k) tL = k == code ? nL[k] : tL;
        const uint64_t freem = ~tL & valid & (~0ull << sp);
        if (!freem) continue;  // dropped: no free slot at or after starting_point
        const int f = __ffsll((long long)freem) - 1;
        sp = f;
        const uint64_t fb = 1ull << f;
#pragma unroll
        for (int k = 0; k < 9; ++k)
            if (k == code) {
                nL[k] |= fb;
                nR[k] |= fb;
                nU[k] = unstable ? (nU[k] | fb) : (nU[k] & ~fb);
            }
        touched |= 1u << code;
        const int64_t tx = ix + code % 3 - 1, ty = iy + code / 3 - 1;
        S.orig[tx + g.n[0] * ty + nc * f] = tag;
    }
#pragma unroll
    for (int k = 0; k < 9; ++k)
        if ((touched >> k) & 1) {
            const int64_t jc = (ix + k % 3 - 1) + g.n[0] * (iy + k / 3 - 1);
            S.L(jc) = nL[k];
            S.R(jc) = nR[k];
            S.U(jc) = nU[k];
        }
}

}  // namespace jp
