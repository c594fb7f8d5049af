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
// before the move L0 and the movers M; in 2D also the movers' destinations as
// four bit planes of their neighbour code (bit j of the code of slot s is bit
// s of plane j), the movers that have a destination (the others leave the
// domain) and the movers not strictly inside their new cell.
constexpr int kRecWords2D = 11;
constexpr int kRecWords3D = 5;

// Shadow records: the movers of cell c, in slot order, are records
// c * max_xcell + 0, 1, 2, ... (the rank of a mover is the number of movers
// in lower slots of its cell), so a cell's movers sit together. An origin tag
// names a refilled slot's particle by the neighbour code of its source cell
// (bits 0..4) and its rank there (bits 5..10).
struct MoveView {
    uint64_t* rec;  // the mask arrays, one after the other
    int64_t nc;     // cells (the length of each mask array)
    uint8_t* code;
    uint16_t* orig;
    double* shadow;
    int64_t nslots;
    int comps;  // stride of the shadow records: DIM coordinates, then the fields (records are interleaved)
    int mx;     // max_xcell: records per cell
    __device__ __forceinline__ uint64_t& L(int64_t c) const { return rec[c]; }
    __device__ __forceinline__ uint64_t& R(int64_t c) const { return rec[nc + c]; }
    __device__ __forceinline__ uint64_t& U(int64_t c) const { return rec[2 * nc + c]; }
    __device__ __forceinline__ uint64_t& L0(int64_t c) const { return rec[3 * nc + c]; }
    __device__ __forceinline__ uint64_t& M(int64_t c) const { return rec[4 * nc + c]; }
    // 2D: bit plane j < 4 of the movers' neighbour codes, the routed movers, the unstable ones
    __device__ __forceinline__ uint64_t& P(int64_t c, int j) const { return rec[(5 + j) * nc + c]; }
    __device__ __forceinline__ uint64_t& RT(int64_t c) const { return rec[9 * nc + c]; }
    __device__ __forceinline__ uint64_t& UN(int64_t c) const { return rec[10 * nc + c]; }
    // first value of the record of rank r of cell c
    __device__ __forceinline__ int64_t record(int64_t c, int r) const { return (c * mx + r) * comps; }
};

__device__ __forceinline__ uint16_t make_tag(int code, int rank) { return (uint16_t)(code | (rank << 5)); }


// position of the n-th set bit (n from 0) of a 64-bit mask
__device__ __forceinline__ int nth_set_bit64(uint64_t m, int n)
{
    const uint32_t lo = (uint32_t)m;
    const int cl = __popc(lo);
    return n < cl ? nth_set_bit(lo, n) : 32 + nth_set_bit((uint32_t)(m >> 32), n - cl);
}

// Per-launch counts of the move, added to the container's counters: [0]
// particles that left the domain, [1] particles that moved more than one cell
// (dropped), [2] particles dropped because their new cell had no free slot at
// or after the walk's starting point.
__device__ __forceinline__ void add_move_counts(unsigned long long* counts, int n_exit, int n_far, int n_full)
{
    const unsigned full = 0xffffffffu;
    n_exit = __reduce_add_sync(full, n_exit);
    n_far = __reduce_add_sync(full, n_far);
    n_full = __reduce_add_sync(full, n_full);
    if ((threadIdx.x & 31) == 0 && counts) {
        if (n_exit) atomicAdd(counts + 0, (unsigned long long)n_exit);
        if (n_far) atomicAdd(counts + 1, (unsigned long long)n_far);
        if (n_full) atomicAdd(counts + 2, (unsigned long long)n_full);
    }
}

// One 32-byte shadow record (4 doubles) in a single 256-bit access: a gather
// of a record is one sector request instead of one per value. p must be
// 32-byte aligned (records start at a multiple of 32 bytes of a 256-byte
// aligned array).
__device__ __forceinline__ void load_rec4(const double* p, double v[4])
{
    asm volatile("ld.global.v4.f64 {%0, %1, %2, %3}, [%4];"
                 : "=d"(v[0]), "=d"(v[1]), "=d"(v[2]), "=d"(v[3])
                 : "l"(p));
}

__device__ __forceinline__ void store_rec4(double* p, const double v[4])
{
    asm volatile("st.global.v4.f64 [%0], {%1, %2, %3, %4};" ::"l"(p), "d"(v[0]), "d"(v[1]), "d"(v[2]), "d"(v[3])
                 : "memory");
}

// Byte offset of the shadow records in a move scratch block: after the mask
// arrays, rounded up to 256 bytes (records of 4 values are stored as 16- and
// 32-byte vectors, so they need at least that alignment).
inline size_t move_shadow_offset(const DevGrid& g)
{
    const size_t rs = g.ndim == 2 ? kRecWords2D : kRecWords3D;
    return (rs * (size_t)g.ncells * sizeof(uint64_t) + 255) & ~(size_t)255;
}

// -------------------------------------------------------------- allocate
// One colour pass of move_particles! in 3D: sources 3*J + o, neighbourhoods
// disjoint, so every mask touched here belongs to exactly one thread. The
// walk is the 2D pass's (below), on 27 neighbours:
//  * the destination codes of the source's original movers are read four
//    loads at a time and kept as five bit planes (bit j of slot s's code in
//    plane j), with the movers that leave and those not strictly inside their
//    new cell as two more masks: no per-slot table in local memory;
//  * the masks of the neighbours the walk may touch are loaded together and
//    kept in the thread's own column of shared memory (27 x 64 threads x 2
//    words: one indexed access per step, conflict-free);
//  * the slots still to visit are a mask; the centre cell's masks stay in
//    registers; a neighbour's R mask is formed at the write-back (a free slot
//    has its R and U bits clear, so R gains exactly the slots L gained) and
//    its U mask changes only for unstable insertions.
static __global__ void __launch_bounds__(kAllocThreads)
    move_allocate_3d(DevGrid g, MoveView S, int o0, int o1, int o2, int64_t m0, int64_t m1, int64_t m2)
{
    constexpr int NB = 27;
    constexpr int CENTER = 13;
    __shared__ uint64_t sL[NB][kAllocThreads], sU[NB][kAllocThreads];
    const int tid = threadIdx.x;
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + tid;
    if (t >= m0 * m1 * m2) return;
    int64_t idx[3];
    idx[0] = 3 * (t % m0) + o0;
    idx[1] = 3 * ((t / m0) % m1) + o1;
    idx[2] = 3 * (t / (m0 * m1)) + o2;
#pragma unroll
    for (int d = 0; d < 3; ++d)
        if (idx[d] >= g.n[d]) return;
    const int64_t nc = g.ncells;
    const int64_t sc = cell_linear<3>(g, idx);
    const uint64_t Mv = S.M(sc);
    const uint64_t U0 = S.U(sc);
    if (Mv == 0 && U0 == 0) return;
    uint64_t Lc = S.L(sc), Rc = S.R(sc), Uc = U0;
    // the original movers' codes (slots not refilled by an earlier pass)
    uint64_t P0 = 0, P1 = 0, P2 = 0, P3 = 0, P4 = 0, exits = 0, unst = 0;
    uint32_t touched = 0;  // neighbours (not the centre) the walk may change
    for (uint64_t m = Mv & ~Rc; m;) {
        int sl[4];
        uint8_t cb[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            sl[u] = m ? __ffsll((long long)m) - 1 : -1;
            m &= m - 1;
        }
#pragma unroll
        for (int u = 0; u < 4; ++u) cb[u] = sl[u] >= 0 ? S.code[sc + nc * sl[u]] : kCodeExit;
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            if (sl[u] < 0) continue;
            const uint64_t bit = 1ull << sl[u];
            if (cb[u] == kCodeExit) {
                exits |= bit;
                continue;
            }
            const int code = min((int)(cb[u] & 0x1F), NB - 1);
            if (code & 1) P0 |= bit;
            if (code & 2) P1 |= bit;
            if (code & 4) P2 |= bit;
            if (code & 8) P3 |= bit;
            if (code & 16) P4 |= bit;
            if (cb[u] & kCodeUnstable) unst |= bit;
            if (code != CENTER) touched |= 1u << code;
        }
    }
    const int64_t n0 = g.n[0], n01 = g.n[0] * g.n[1];
#pragma unroll
    for (int k = 0; k < NB; ++k) {
        if (k == CENTER || !((touched >> k) & 1u)) continue;
        const int64_t jc = sc + (k % 3 - 1) + n0 * ((k / 3) % 3 - 1) + n01 * (k / 9 - 1);
        sL[k][tid] = S.L(jc);
        sU[k][tid] = S.U(jc);
    }
    const int nslot = g.max_xcell;
    const uint64_t valid = nslot == 64 ? ~0ull : ((1ull << nslot) - 1);
    // the reference's candidates: live slots that are original movers, or refilled
    // by an earlier pass and not strictly inside; a particle put back into the
    // centre cell ahead of the walk is added
    uint64_t todo = Lc & ((Mv & ~Rc) | (Rc & Uc));
    uint64_t from_sp = valid;  // slots at or after starting_point (move_safe.jl:83)
    int n_full = 0;
    while (todo) {
        const uint64_t bit = todo & (0ull - todo);
        todo ^= bit;
        const int s = __ffsll((long long)bit) - 1;
        const bool refill = (Rc & bit) != 0;  // refilled by an earlier pass: walked again, into the centre
        if (!refill && (exits & bit)) {  // left the domain (or moved too far): cleared
            Lc &= ~bit;
            continue;
        }
        const int code = refill ? CENTER
                                : ((P0 & bit) ? 1 : 0) | ((P1 & bit) ? 2 : 0) | ((P2 & bit) ? 4 : 0) |
                                      ((P3 & bit) ? 8 : 0) | ((P4 & bit) ? 16 : 0);
        const bool unstable = refill || (unst & bit) != 0;
        const uint16_t tag = refill ? S.orig[sc + nc * s]
                                    : make_tag(NB - 1 - code, __popcll(Mv & (bit - 1)));  // the way back
        // remove the particle from its slot (move_safe.jl:110-112)
        Lc &= ~bit;
        Rc &= ~bit;
        Uc &= ~bit;
        // find_free_memory(starting_point, ...) (move_safe.jl:192-197)
        const uint64_t tL = code == CENTER ? Lc : sL[code][tid];
        const uint64_t freem = ~tL & from_sp;
        if (!freem) {  // dropped: no free slot at or after starting_point
            ++n_full;
            continue;
        }
        const uint64_t fb = freem & (0ull - freem);
        from_sp = valid & ~(fb - 1);
        if (code == CENTER) {
            Lc |= fb;
            Rc |= fb;
            if (unstable) {
                Uc |= fb;
                if (fb > bit) todo |= fb;  // ahead of the walk: visited again
            } else {
                Uc &= ~fb;
            }
        } else {
            sL[code][tid] = tL | fb;
            if (unstable) sU[code][tid] |= fb;
        }
        const int f = __ffsll((long long)fb) - 1;
        const int64_t tc = sc + (code % 3 - 1) + n0 * ((code / 3) % 3 - 1) + n01 * (code / 9 - 1);
        S.orig[tc + nc * f] = tag;
    }
    S.L(sc) = Lc;
    S.R(sc) = Rc;
    S.U(sc) = Uc;
    if (n_full && g.counts) atomicAdd(g.counts + 2, (unsigned long long)n_full);
    // a neighbour only gained slots in this walk: R = R before | the slots L gained
    // (its R and L in memory are still those before the walk: this thread alone writes them)
    for (uint32_t m = touched; m; m &= m - 1) {
        const int k = __ffs(m) - 1;
        const int64_t jc = sc + (k % 3 - 1) + n0 * ((k / 3) % 3 - 1) + n01 * (k / 9 - 1);
        const uint64_t Lf = sL[k][tid];
        S.R(jc) = S.R(jc) | (Lf & ~S.L(jc));
        S.L(jc) = Lf;
        S.U(jc) = sU[k][tid];
    }
}

// The 2D colour pass. A pass has one thread per source cell and few cells
// (n/3 x n/3 of them), so its time is the latency of one thread's walk, and
// the walk is written for a short dependency chain per step:
//  * the slots still to visit are a mask (the candidates of the reference's
//    slot loop; a particle put back into the centre cell ahead of the walk
//    is added to it), popped lowest bit first;
//  * the destination of a slot comes from the four bit planes of the
//    movers' neighbour codes written by the classify stage (no per-slot table);
//  * "first free slot at or after starting_point" is the lowest set bit of
//    the free mask under a running mask of the slots >= starting_point;
//  * the centre cell's masks stay in registers, the eight neighbours' sit in
//    the thread's own column of shared memory (one indexed access, no select
//    over the neighbours), all global loads are issued before the first
//    shared-memory store.
static __global__ void __launch_bounds__(kAllocThreads)
    move_allocate_2d(DevGrid g, MoveView S, int o0, int o1, int64_t m0, int64_t m1)
{
    constexpr int CENTER = 4;
    // [neighbour][thread]: a warp's 64-bit accesses are conflict-free whatever neighbour each lane picks.
    // A neighbour's R mask is not read during the walk: it is formed at the write-back (below).
    __shared__ uint64_t sL[9][kAllocThreads], sU[9][kAllocThreads];
    const int tid = threadIdx.x;
    const int64_t t = (int64_t)blockIdx.x * kAllocThreads + tid;
    if (t >= m0 * m1) return;
    int64_t qx, qy;
    if (m0 * m1 <= (int64_t)0xFFFFFFFF) {  // 32-bit division
        const uint32_t t32 = (uint32_t)t, w = (uint32_t)m0;
        const uint32_t y = t32 / w;
        qy = y;
        qx = t32 - y * w;
    } else {
        qy = t / m0;
        qx = t - qy * m0;
    }
    const int64_t ix = 3 * qx + o0, iy = 3 * qy + o1;
    const int64_t nx = g.n[0];
    if (ix >= nx || iy >= g.n[1]) return;
    const int64_t nc = g.ncells;
    const int64_t sc = ix + nx * iy;
    const uint64_t Mv = S.M(sc);
    const uint64_t U0 = S.U(sc);
    if (Mv == 0 && U0 == 0) return;
    uint64_t Lc = S.L(sc), Rc = S.R(sc), Uc = U0;
    uint64_t nl[9], nu[9];
#pragma unroll
    for (int k = 0; k < 9; ++k) {
        if (k == CENTER) continue;
        const int64_t jx = ix + k % 3 - 1, jy = iy + k / 3 - 1;
        const bool in = jx >= 0 && jy >= 0 && jx < nx && jy < g.n[1];
        const int64_t jc = jx + nx * jy;
        nl[k] = in ? S.L(jc) : 0;
        nu[k] = in ? S.U(jc) : 0;
    }
    // bit j of a slot's destination code in plane j; movers with no destination leave the domain
    const uint64_t P0 = S.P(sc, 0), P1 = S.P(sc, 1), P2 = S.P(sc, 2), P3 = S.P(sc, 3);
    const uint64_t routed = S.RT(sc), unst = S.UN(sc);
#pragma unroll
    for (int k = 0; k < 9; ++k) {
        if (k == CENTER) continue;
        sL[k][tid] = nl[k];
        sU[k][tid] = nu[k];
    }
    const uint64_t exits = Mv & ~routed;
    const int nslot = g.max_xcell;
    const uint64_t valid = nslot == 64 ? ~0ull : ((1ull << nslot) - 1);
    uint32_t touched = 0;  // neighbours (not the centre) whose masks changed
    // the reference's candidates: live slots that are original movers, or
    // refilled by an earlier pass and not strictly inside
    uint64_t todo = Lc & ((Mv & ~Rc) | (Rc & Uc));
    uint64_t from_sp = valid;  // slots at or after starting_point (move_safe.jl:83)
    int n_full = 0;
    while (todo) {
        const uint64_t bit = todo & (0ull - todo);
        todo ^= bit;
        const bool refill = (Rc & bit) != 0;  // refilled by an earlier pass: walked again, into the centre
        if (!refill && (exits & bit)) {  // left the domain (or moved too far): cleared
            Lc &= ~bit;
            continue;
        }
        // (a slot sits in one per-target mask; the clamp only keeps the shared-memory
        // index in range should the masks ever be inconsistent)
        const int code = refill ? CENTER
                                : min(((P0 & bit) ? 1 : 0) | ((P1 & bit) ? 2 : 0) | ((P2 & bit) ? 4 : 0) |
                                          ((P3 & bit) ? 8 : 0),
                                      8);
        const bool unstable = refill || (unst & bit) != 0;
        // remove the particle from its slot (move_safe.jl:110-112)
        Lc &= ~bit;
        Rc &= ~bit;
        Uc &= ~bit;
        // find_free_memory(starting_point, ...) (move_safe.jl:192-197)
        const uint64_t tL = code == CENTER ? Lc : sL[code][tid];
        const uint64_t freem = ~tL & from_sp;
        if (!freem) {  // dropped: no free slot at or after starting_point
            ++n_full;
            continue;
        }
        const uint64_t fb = freem & (0ull - freem);
        from_sp = valid & ~(fb - 1);
        if (code == CENTER) {
            Lc |= fb;
            Rc |= fb;
            if (unstable) {
                Uc |= fb;
                if (fb > bit) todo |= fb;  // ahead of the walk: visited again
            } else {
                Uc &= ~fb;
            }
        } else {
            // a free slot has its R and U bits clear (U within R within L): a stable
            // particle leaves U as it is, and R gains the slot at the write-back
            sL[code][tid] = tL | fb;
            if (unstable) sU[code][tid] |= fb;
            touched |= 1u << code;
        }
        const int s = __ffsll((long long)bit) - 1, f = __ffsll((long long)fb) - 1;
        uint16_t tag;
        if (refill)
            tag = S.orig[sc + nc * s];
        else
            tag = make_tag(8 - code, __popcll(Mv & (bit - 1)));  // 8 - code: the neighbour code of the way back
        const int dy = code / 3 - 1, dx = code - 3 * (dy + 1) - 1;
        S.orig[sc + dx + nx * dy + nc * f] = tag;
    }
    S.L(sc) = Lc;
    S.R(sc) = Rc;
    S.U(sc) = Uc;
    if (n_full && g.counts) atomicAdd(g.counts + 2, (unsigned long long)n_full);
    // a neighbour only gained slots in this walk: R = R before | the slots L gained
    // (its R and L in memory are still those before the walk: this thread alone writes them)
#pragma unroll
    for (int k = 0; k < 9; ++k) {
        if (k == CENTER || !((touched >> k) & 1u)) continue;
        const int64_t jc = sc + (k % 3 - 1) + nx * (k / 3 - 1);
        const uint64_t Lf = sL[k][tid];
        S.R(jc) = S.R(jc) | (Lf & ~nl[k]);
        S.L(jc) = Lf;
        S.U(jc) = sU[k][tid];
    }
}

}  // namespace jp
