// jp_move_core.cuh -- the slot-allocation stage of move_particles!, shared by
// the FP64 and the split-precision (FP32 cell offset) forms: it works on
// occupancy masks and destination codes only, whatever the particle data.
#pragma once

#include "jp_internal.cuh"

namespace jp {

constexpr int kAllocThreads = 64;  // small blocks spread the sparse colour passes over all SMs

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
    int comps;  // values per shadow record: DIM coordinates, then the fields (records are interleaved)
};

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
    const uint64_t Mv = S.M[sc];
    const uint64_t U0 = S.U[sc];
    if (Mv == 0 && U0 == 0) return;
    uint64_t nL[NB], nR[NB], nU[NB];
    uint8_t codes[64];
    nL[CENTER] = S.L[sc];
    nR[CENTER] = S.R[sc];
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
        nL[nb] = S.L[jc];
        nR[nb] = S.R[jc];
        nU[nb] = S.U[jc];
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
        S.L[jc] = nL[nb];
        S.R[jc] = nR[nb];
        S.U[jc] = nU[nb];
    }
}

}  // namespace jp
