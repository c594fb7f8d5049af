// jp_move.cu -- move_particles! and inject_particles!.
//
// move_particles! (src/Particles/move_safe.jl:21-125) is a sequential slot walk
// per source cell, run in 3^N colour passes; its slot allocation (first free
// slot at or after `starting_point`, which carries over between target cells)
// decides which particles survive a full cell. It is reproduced exactly in
// three stages:
//   1. classify (all cells, one pass over the live slots): which particles left
//      their cell, where they go (one of the 3^N neighbours, or out), and a
//      copy of the movers' coordinates and fields into a shadow array;
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
// ends the walk otherwise), and that test depends on the cell alone. A flag
// pass over all cells appends those cells to one work list per colour and
// records each cell's occupancy mask and particle bounding box; each of the
// 2^N colour passes then gives every listed cell a warp that keeps the cell's
// own particles in shared memory and runs the reference's sequential walk with
// warp-wide counts and an exact nearest-neighbour search that only visits the
// neighbour cells whose box can hold a nearer particle. Cells of one colour
// are independent, so the list order (set by atomics) does not change any
// result. Containers of more than 64 slots per cell use the reference's own
// per-cell schedule instead (bottom of this file).
#include <math_constants.h>

#include <climits>
#include <limits>
#include <mutex>

#include "jp_internal.cuh"
#include "jp_move_core.cuh"

namespace jp {

// find_parent_cell_bisection with integer-key comparisons (px not NaN):
// the local walk of find_cell, ties replayed by bisect_exact.
__device__ __forceinline__ int64_t find_cell_key(double px, long long kp, const double* x, int64_t len,
                                                 int64_t seed, int* errs)
{
    long long ka = okey(ldg(x + seed)), kb = okey(ldg(x + seed + 1));
    if (ka <= kp && kp <= kb) return seed;
    int64_t k = seed;
    if (kp < ka) {
#pragma unroll 1
        for (int it = 0; it < 4 && k > 0; ++it) {
            --k;
            kb = ka;
            ka = okey(ldg(x + k));
            if (ka <= kp && kp <= kb) return (kp == ka || kp == kb) ? bisect_exact(px, x, len, seed, errs) : k;
        }
    } else {
#pragma unroll 1
        for (int it = 0; it < 4 && k + 2 < len; ++it) {
            ++k;
            ka = kb;
            kb = okey(ldg(x + k + 1));
            if (ka <= kp && kp <= kb) return (kp == ka || kp == kb) ? bisect_exact(px, x, len, seed, errs) : k;
        }
    }
    return bisect_exact(px, x, len, seed, errs);
}

// -------------------------------------------------------------- classify
// A warp covers 32 consecutive cells and spreads their live particles over its
// lanes in slot-major order (full lanes whatever the occupancy), two particles
// per lane in flight: coordinates and fields are loaded together, then the
// particles are classified (their movers' bits go to per-target masks in
// shared memory, one atomic each), and after a warp barrier each routed
// mover writes its record to its cell's next records: its rank is the number of
// movers in lower slots of its cell, all of which lie in this or an earlier
// batch (slot-major order).
template <int DIM>
__global__ void __launch_bounds__(32 * kWarpsPerBlock)
    move_classify(DevGrid g, Coords X, const uint8_t* __restrict__ index, Args A, MoveView S, int* d_err)
{
    __shared__ SlotList lists[kWarpsPerBlock];
    __shared__ long long cellk[kWarpsPerBlock][32][2 * DIM];  // keys of corner and corner + dx
    __shared__ int cellI[kWarpsPerBlock][32][3];
    __shared__ unsigned long long movers[kWarpsPerBlock][32];
    constexpr int NT = DIM == 2 ? 10 : 1;  // 2D: movers bound for each of the 9 neighbours, unstable ones
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
        for (int d = 0; d < DIM; ++d) {
            const double lo = ldg(g.xv[d] + I[d]);
            cellk[w][lane][d] = okey(lo);
            cellk[w][lane][DIM + d] = okey(lo + ldg(g.dxv[d] + I[d]));  // xv + dx (isincell)
            cellI[w][lane][d] = (int)I[d];
        }
        movers[w][lane] = 0;
#pragma unroll
        for (int k = 0; k < NT; ++k) tmask[w][k][lane] = 0;
    }
    long long kdlo[3], kdhi[3];
#pragma unroll
    for (int d = 0; d < DIM; ++d) {
        kdlo[d] = okey(g.dom_lo[d]);
        kdhi[d] = okey(g.dom_hi[d]);
    }
    uint64_t L;
    const int K = build_slot_list(lists[w], index, c0, nc, M, lane, &L);
    int errs = 0, n_exit = 0, n_far = 0;
    const int comps = S.comps;
    const bool rec4 = comps == 4;
    // classify one live particle (coordinates p): its destination code, kCodeExit when it leaves
    auto classify_one = [&](int s, int l, int64_t a, const double* p) -> uint8_t {
        long long kp[3];
        bool pnan = false;
#pragma unroll
        for (int d = 0; d < DIM; ++d) {
            kp[d] = okey(p[d]);
            pnan |= is_nan_bits(p[d]);
        }
        bool in = !pnan;  // isincell, strict (src/Particles/utils.jl:7-15)
#pragma unroll
        for (int d = 0; d < DIM; ++d) in = in & (cellk[w][l][d] < kp[d]) & (kp[d] < cellk[w][l][DIM + d]);
        if (in) return kCodeStay;  // move_safe.jl:93
        const unsigned long long bit = 1ull << s;
        atomicOr(&movers[w][l], bit);
        bool inside = !pnan;  // indomain, strict (move_safe.jl:199-206)
#pragma unroll
        for (int d = 0; d < DIM; ++d) inside = inside & (kdlo[d] < kp[d]) & (kp[d] < kdhi[d]);
        uint8_t code = kCodeExit;
        if (inside) {
            int off[3] = {0, 0, 0};
            bool far = false, inT = true;
#pragma unroll
            for (int d = 0; d < DIM; ++d) {
                const int I = cellI[w][l][d];
                const int64_t T = find_cell_key(p[d], kp[d], g.xv[d], g.n[d] + 1, I, &errs);
                off[d] = (int)(T - I);
                far |= (off[d] > 1) | (off[d] < -1);
                const double lo = ldg(g.xv[d] + T);
                inT = inT & (okey(lo) < kp[d]) & (kp[d] < okey(lo + ldg(g.dxv[d] + T)));
            }
            if (far) {
                errs |= kWarnFarMove;
                ++n_far;
            } else {
                code = (uint8_t)nb_code<DIM>(off);
                if (!inT) code |= kCodeUnstable;
            }
        } else {
            ++n_exit;
        }
        if (DIM == 2) {
            if (code != kCodeExit) {
                atomicOr(&tmask[w][code & 0x1F][l], bit);
                if (code & kCodeUnstable) atomicOr(&tmask[w][9][l], bit);
            }
        } else {
            S.code[a] = code;
        }
        return code;
    };
    constexpr int B = 2;
    for (int k0 = lane; k0 < K; k0 += 32 * B) {
        int sl[B], ll[B];
        int64_t al[B];
        double pl[B][3], fl[B][4 - DIM];
        bool has[B];
        uint8_t code[B];
#pragma unroll
        for (int u = 0; u < B; ++u) {
            const int k = k0 + 32 * u;
            has[u] = k < K;
            sl[u] = 0;
            ll[u] = 0;
            if (has[u]) slot_item(lists[w], M, k, &sl[u], &ll[u]);
            al[u] = c0 + ll[u] + nc * sl[u];
#pragma unroll
            for (int d = 0; d < DIM; ++d) pl[u][d] = has[u] ? X.c[d][al[u]] : 0.0;
#pragma unroll
            for (int j = 0; j < 4 - DIM; ++j) fl[u][j] = (has[u] && rec4 && j < A.n) ? A.a[j][al[u]] : 0.0;
        }
#pragma unroll
        for (int u = 0; u < B; ++u) code[u] = has[u] ? classify_one(sl[u], ll[u], al[u], pl[u]) : kCodeStay;
        __syncwarp();  // every mover bit of this batch is set
#pragma unroll
        for (int u = 0; u < B; ++u) {
            if (code[u] == kCodeStay || code[u] == kCodeExit) continue;
            const int l = ll[u];
            const int r = __popcll(movers[w][l] & ((1ull << sl[u]) - 1));
            double* rp = S.shadow + S.record(c0 + l, r);
            if (rec4) {  // the whole record in one 32-byte store
                double v[4] = {0.0, 0.0, 0.0, 0.0};
#pragma unroll
                for (int d = 0; d < DIM; ++d) v[d] = pl[u][d];
#pragma unroll
                for (int j = 0; j < 4 - DIM; ++j) v[DIM + j] = fl[u][j];
                store_rec4(rp, v);
            } else if (comps == 2) {
                *reinterpret_cast<double2*>(rp) = make_double2(pl[u][0], pl[u][1]);
            } else {
#pragma unroll
                for (int d = 0; d < DIM; ++d) rp[d] = pl[u][d];
                for (int j = 0; j < A.n; ++j) rp[DIM + j] = A.a[j][al[u]];
            }
        }
    }
    __syncwarp();
    const int64_t c = c0 + lane;
    if (c < nc) {
        S.L(c) = L;
        S.R(c) = 0;
        S.U(c) = 0;
        S.L0(c) = L;
        S.M(c) = movers[w][lane];
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
            for (int j = 0; j < 4; ++j) S.P(c, j) = P[j];
            S.RT(c) = RT;
            S.UN(c) = tmask[w][9][lane];
        }
    }
    add_move_counts(g.counts, n_exit, n_far, 0);
    raise_err(d_err, errs);
}

// ----------------------------------------------------------------- apply
// Slot-major over a warp's 32 cells: at each slot the lanes whose slot changed
// store together, so every 32-byte sector is written in one go. A refilled
// slot gathers its record from the source cell named by its origin tag.
template <int DIM>
__global__ void __launch_bounds__(kThreads)
    move_apply(DevGrid g, Coords X, uint8_t* __restrict__ index, Args A, MoveView S)
{
    const int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t nc = g.ncells;
    const bool valid = c < nc;
    uint64_t L0 = 0, L = 0, R = 0;
    if (valid) {
        L0 = S.L0(c);
        L = S.L(c);
        R = S.R(c);
    }
    uint64_t changed = (L0 & ~L) | R;
    // slots past the highest changed slot of any lane need no visit
    const uint32_t hi_any = __reduce_max_sync(0xffffffffu, changed ? 64u - (uint32_t)__clzll((long long)changed) : 0u);
    if (hi_any == 0) return;
    int64_t I[3] = {0, 0, 0};
    if (valid) cell_coords(g, c, I);
    if (S.comps == 4 || S.comps == 2) {
        // four slot rows per step (eight hold 100 registers for the same time), the warp
        // still on the same row at a time (stores of one row share sectors); the rows'
        // origin tags, then their records, are loaded together, so a step waits for two
        // loads instead of two per row
        constexpr int B = 4;
        for (int s0 = 0; s0 < (int)hi_any; s0 += B) {
            bool ch[B], rf[B];
            uint16_t tag[B];
#pragma unroll
            for (int u = 0; u < B; ++u) {
                const int s = s0 + u;
                ch[u] = s < (int)hi_any && ((changed >> s) & 1);
                rf[u] = ch[u] && ((R >> s) & 1);
                tag[u] = rf[u] ? S.orig[c + nc * s] : (uint16_t)0;
            }
            double v[B][4];
#pragma unroll
            for (int u = 0; u < B; ++u) {
#pragma unroll
                for (int k = 0; k < 4; ++k) v[u][k] = CUDART_NAN;  // a vacated slot
                if (!rf[u]) continue;
                int off[3];
                nb_offset<DIM>(tag[u] & 0x1F, off);
                const int64_t J[3] = {I[0] + off[0], I[1] + off[1], DIM == 3 ? I[2] + off[2] : 0};
                const double* rec = S.shadow + S.record(cell_linear<DIM>(g, J), tag[u] >> 5);
                if (S.comps == 4) {
                    load_rec4(rec, v[u]);
                } else {
                    const double2 r2 = *reinterpret_cast<const double2*>(rec);
                    v[u][0] = r2.x;
                    v[u][1] = r2.y;
                }
            }
#pragma unroll
            for (int u = 0; u < B; ++u) {
                if (!ch[u]) continue;
                const int64_t a = c + nc * (s0 + u);
#pragma unroll
                for (int d = 0; d < DIM; ++d) X.c[d][a] = v[u][d];
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
            const uint16_t tag = S.orig[a];
            int off[3];
            nb_offset<DIM>(tag & 0x1F, off);
            const int64_t J[3] = {I[0] + off[0], I[1] + off[1], DIM == 3 ? I[2] + off[2] : 0};
            const double* rp = S.shadow + S.record(cell_linear<DIM>(g, J), tag >> 5);
            if (S.comps == 4) {  // the whole record in one 32-byte load
                double v[4];
                load_rec4(rp, v);
#pragma unroll
                for (int d = 0; d < DIM; ++d) X.c[d][a] = v[d];
#pragma unroll
                for (int k = 0; k < 4 - DIM; ++k)
                    if (k < A.n) A.a[k][a] = v[DIM + k];
            } else if (S.comps == 2) {
                const double2 v = *reinterpret_cast<const double2*>(rp);
                X.c[0][a] = v.x;
                X.c[1][a] = v.y;
            } else {
#pragma unroll
                for (int d = 0; d < DIM; ++d) X.c[d][a] = rp[d];
                for (int k = 0; k < A.n; ++k) A.a[k][a] = rp[DIM + k];
            }
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
struct InjectLists {
    int* counts;     // [8]
    int* list;       // ncells entries
    uint64_t* lm;    // occupancy mask per cell
    float* box;      // bounding box of each cell's live particles: lo[0..2], hi[0..2], rounded outwards
    int64_t off[8];  // start of each colour's region in `list`
};

template <int DIM>
__device__ __forceinline__ int colour_of(const int64_t* I)
{
    return (int)(I[0] & 1) + 2 * (int)(I[1] & 1) + (DIM == 3 ? 4 * (int)(I[2] & 1) : 0);
}

// Occupancy test of a cell before its pass: inject_particles! only works on a
// cell whose first quadrant is short (injection.jl:81-100 stops at the first
// quadrant that is not), inject_particles_phase! (PHASE) on a cell with any
// short quadrant (injection.jl:262-280). A cell's own slots change only in its
// own pass, so the test on the state before the colour passes is exact.
// Flagged cells are appended to their colour's list.
template <int DIM, bool PHASE>
__global__ void __launch_bounds__(kThreads)
    inject_flag(DevGrid g, CCoords X, const uint8_t* __restrict__ index, InjectLists Ls)
{
    const int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int lane = threadIdx.x & 31;
    const bool valid = c < g.ncells;
    const int64_t nc = g.ncells;
    int64_t I[3] = {0, 0, 0};
    cell_coords(g, valid ? c : 0, I);
    const int col = colour_of<DIM>(I);
    // quadrant bounds: lower half corner .. corner + dx/2, upper half corner + dx/2 .. + dx/2
    // (quadrant_corners, injection.jl:442-466; isincell strict)
    long long klo[2][3], khi[2][3];
#pragma unroll
    for (int d = 0; d < DIM; ++d) {
        const double lo = ldg(g.xv[d] + I[d]), h = ldg(g.dxv[d] + I[d]) / 2.0;
        klo[0][d] = okey(lo);
        khi[0][d] = okey(lo + h);
        klo[1][d] = okey(lo + h);
        khi[1][d] = okey((lo + h) + h);
    }
    // the cell's occupancy mask, kept for the passes
    const uint64_t live = valid ? live_mask(index, c, nc, g.max_xcell) : 0ull;
    if (valid) Ls.lm[c] = live;
    // one sweep over the slots, the same slot across the warp (coalesced): the bounding box
    // of the live particles on order-preserving integer keys (NaN coordinates never win a
    // search and are left out) and the quadrant counts
    long long blo[3] = {LLONG_MAX, LLONG_MAX, LLONG_MAX}, bhi[3] = {LLONG_MIN, LLONG_MIN, LLONG_MIN};
    int cq[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    const int smax = __reduce_max_sync(0xffffffffu, live ? 64 - __clzll((long long)live) : 0);
    constexpr int B = 4;  // slots per step, their loads in flight together
    for (int s0 = 0; s0 < smax; s0 += B) {
        double xs[B][DIM];
        bool lv[B];
#pragma unroll
        for (int u = 0; u < B; ++u) {
            const int s = s0 + u;
            lv[u] = s < smax && ((live >> s) & 1ull);
#pragma unroll
            for (int d = 0; d < DIM; ++d) xs[u][d] = lv[u] ? X.c[d][c + nc * s] : 0.0;
        }
#pragma unroll
        for (int u = 0; u < B; ++u) {
            if (!lv[u]) continue;
            unsigned in0 = 0, in1 = 0;
#pragma unroll
            for (int d = 0; d < DIM; ++d) {
                const double x = xs[u][d];
                const bool ok = !is_nan_bits(x);
                const long long k = okey(x);
                if (ok) {
                    blo[d] = min(blo[d], k);
                    bhi[d] = max(bhi[d], k);
                }
                in0 |= (unsigned)(ok & (klo[0][d] < k) & (k < khi[0][d])) << d;
                in1 |= (unsigned)(ok & (klo[1][d] < k) & (k < khi[1][d])) << d;
            }
            constexpr unsigned full = (1u << DIM) - 1u;
#pragma unroll
            for (int q = 0; q < (PHASE ? (1 << DIM) : 1); ++q)  // quadrant q: upper half where bit d of q is set
                cq[q] += (((in1 & (unsigned)q) | (in0 & ~(unsigned)q & full)) == full) ? 1 : 0;
        }
    }
    bool flag = false;
    if (valid) {
#pragma unroll
        for (int d = 0; d < DIM; ++d) {
            const bool any = blo[d] <= bhi[d];
            Ls.box[6 * c + d] = any ? __double2float_rd(okey_value(blo[d])) : CUDART_INF_F;
            Ls.box[6 * c + 3 + d] = any ? __double2float_ru(okey_value(bhi[d])) : -CUDART_INF_F;
        }
        const int min_xq = (g.min_xcell + (1 << DIM) - 1) >> DIM;
        // inject_particles! looks at a cell only while its first quadrant is short
        // (injection.jl:81-100), inject_particles_phase! at any short quadrant (:262-280)
#pragma unroll
        for (int q = 0; q < (PHASE ? (1 << DIM) : 1); ++q) flag |= cq[q] < min_xq;
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

__device__ __forceinline__ double warp_min(double v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = fmin(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}

// Grid fields that inject_particles_phase! interpolates onto new particles
// (one per particle field of Args), each cell-centred or on the vertices.
struct PhaseFields {
    const double* f[JP_MAX_ARGS];
    int centred[JP_MAX_ARGS];
    double* phases;  // per-slot phase ids, copied from the nearest neighbour
};

// Julia's min / max on floats: NaN wins, -0.0 is below +0.0
__device__ __forceinline__ double jl_min(double x, double y)
{
    return ((y < x) || (signbit(y) && !signbit(x))) ? (isnan(x) ? x : y) : (isnan(y) ? y : x);
}
__device__ __forceinline__ double jl_max(double x, double y)
{
    return ((y > x) || (!signbit(y) && signbit(x))) ? (isnan(x) ? x : y) : (isnan(y) ? y : x);
}

// src/Particles/injection.jl:300-318: the clamped N-linear interpolation of a
// cell-centred (centre cell below p, clamped; centre spacing) or vertex field
// (the particle's own cell) at the new particle.
template <int DIM>
__device__ double phase_field_value(const DevGrid& g, const double* __restrict__ F, bool centred, const double* pn,
                                    const int64_t* I, const double* corner, const double* dq)
{
    int64_t J[3] = {0, 0, 0};
    double t[3];
    int64_t L0, L1;
    if (centred) {
#pragma unroll
        for (int d = 0; d < DIM; ++d) {
            const double xcen = corner[d] + dq[d];
            int64_t j = pn[d] < xcen ? I[d] - 1 : I[d];
            const int64_t hi = g.n[d] - 2;
            j = j < 0 ? 0 : (j > hi ? hi : j);
            J[d] = j;
            t[d] = (pn[d] - ldg(g.xc[d] + j)) * ldg(g.ixc[d] + j);
        }
        L0 = g.n[0];
        L1 = g.n[1];
    } else {
#pragma unroll
        for (int d = 0; d < DIM; ++d) {
            J[d] = I[d];
            t[d] = (pn[d] - ldg(g.xv[d] + I[d])) * ldg(g.ixv[d] + I[d]);
        }
        L0 = g.n[0] + 1;
        L1 = g.n[1] + 1;
    }
    const int64_t b = J[0] + L0 * (J[1] + (DIM == 3 ? L1 * J[2] : 0));
    const int64_t sz = L0 * L1;
    const int64_t off[8] = {b, b + 1, b + L0, b + L0 + 1, b + sz, b + sz + 1, b + sz + L0, b + sz + L0 + 1};
    double v[8];
#pragma unroll
    for (int k = 0; k < (1 << DIM); ++k) v[k] = ldg(F + off[k]);
    const double tmp = lerpN<DIM>(v, t);
    double lo = v[0], hi = v[0];
#pragma unroll
    for (int k = 1; k < (1 << DIM); ++k) {
        hi = jl_max(v[k], hi);
        lo = jl_min(v[k], lo);
    }
    return tmp > hi ? hi : (tmp < lo ? lo : tmp);
}

// per-lane minimum of the squared distance: (ss1, the smallest order o with it)
// and the smallest squared distance above ss1
struct NearestTrack {
    double ss1, ss2;
    int o1;
    __device__ __forceinline__ NearestTrack()
        : ss1(std::numeric_limits<double>::infinity()), ss2(std::numeric_limits<double>::infinity()), o1(0x7fffffff)
    {
    }
    __device__ __forceinline__ void add(double ss, int o)
    {
        if (ss < ss1) {  // NaN never enters
            ss2 = ss1;
            ss1 = ss;
            o1 = o;
        } else if (ss == ss1) {
            o1 = min(o1, o);
        } else if (ss < ss2) {
            ss2 = ss;
        }
    }
};

// squared distance of the reference's distance() (sum of squares, x first)
template <int DIM>
__device__ __forceinline__ double own_ss(const double* own, int M, int s, const double* pn)
{
    double e[3];
#pragma unroll
    for (int d = 0; d < DIM; ++d) e[d] = own[d * M + s] - pn[d];
    return DIM == 2 ? e[0] * e[0] + e[1] * e[1] : (e[0] * e[0] + e[1] * e[1]) + e[2] * e[2];
}

template <int DIM>
__device__ __forceinline__ double glob_ss(const Coords& X, int64_t b, const double* pn)
{
    double e[3];
#pragma unroll
    for (int d = 0; d < DIM; ++d) e[d] = X.c[d][b] - pn[d];
    return DIM == 2 ? e[0] * e[0] + e[1] * e[1] : (e[0] * e[0] + e[1] * e[1]) + e[2] * e[2];
}

// ---- the integer screen of the nearest-neighbour search ----
// Coordinates become signed fixed-point integers in units of 2^(emax - 1075),
// emax one above the largest biased exponent of the domain bounds, by integer
// operations on their bits (truncated toward zero: the real value lies within
// one unit). Differences of two such integers are exact, so a squared distance
// is known within bounds from per-axis differences known within 2 units; the
// bounds are formed in FP32 with directed rounding. None of this touches the
// FP64 pipe, which is the scarce resource of the exact search.
constexpr long long kFixNone = LLONG_MIN;  // no fixed-point value (NaN, Inf, beyond the scale)

template <int DIM>
__device__ __forceinline__ int fix_emax(const DevGrid& g)
{
    int e = 0;
#pragma unroll
    for (int d = 0; d < DIM; ++d) {
        e = max(e, (int)((__double_as_longlong(g.dom_lo[d]) >> 52) & 0x7FF));
        e = max(e, (int)((__double_as_longlong(g.dom_hi[d]) >> 52) & 0x7FF));
    }
    return min(e + 1, 2046);
}

__device__ __forceinline__ long long fix_double(double x, int emax)
{
    const unsigned long long b = (unsigned long long)__double_as_longlong(x);
    const int e = (int)((b >> 52) & 0x7FF);
    if (e == 0x7FF || e > emax) return kFixNone;
    const unsigned long long m = (b & ((1ull << 52) - 1)) | (e ? (1ull << 52) : 0ull);
    const int sh = emax - (e ? e : 1);  // x = m 2^(max(e,1) - 1075)
    const unsigned long long v = sh >= 64 ? 0ull : (m >> sh);
    return (b >> 63) ? -(long long)v : (long long)v;
}

__device__ __forceinline__ long long fix_float(float x, int emax)
{
    const uint32_t b = __float_as_uint(x);
    const int e = (int)((b >> 23) & 0xFF);
    if (e == 0xFF) return kFixNone;
    const unsigned long long m = (b & 0x7FFFFFu) | (e ? 0x800000u : 0u);
    const int sh = (e ? e : 1) + 925 - emax;  // x = m 2^(max(e,1) - 150), unit 2^(emax - 1075)
    unsigned long long v;
    if (sh >= 0) {
        if (sh > 38) return kFixNone;  // |v| would reach 2^62
        v = m << sh;
    } else {
        v = -sh >= 64 ? 0ull : (m >> -sh);
    }
    return (b >> 31) ? -(long long)v : (long long)v;
}

// lo <= squared distance / unit^2 <= hi, for per-axis differences dx known within 2 units
template <int DIM>
__device__ __forceinline__ void ss_bounds(const long long* dx, float* lo, float* hi)
{
    float l = 0.0f, h = 0.0f;
#pragma unroll
    for (int d = 0; d < DIM; ++d) {
        const long long a = dx[d] < 0 ? -dx[d] : dx[d];
        const float al = __ll2float_rd(a > 2 ? a - 2 : 0);
        const float ah = __ll2float_ru(a + 2);
        l = __fmaf_rd(al, al, l);
        h = __fmaf_ru(ah, ah, h);
    }
    *lo = l;
    *hi = h;
}

// per lane: the smallest upper bound seen, and the candidate with the smallest
// lower bound (lo1, o1) with the next lower bound lo2
struct ScreenTrack {
    float hmin, lo1, lo2;
    int o1;
    __device__ __forceinline__ ScreenTrack()
        : hmin(std::numeric_limits<float>::infinity()), lo1(std::numeric_limits<float>::infinity()),
          lo2(std::numeric_limits<float>::infinity()), o1(-1)
    {
    }
    __device__ __forceinline__ void add(float lo, float hi, int o)
    {
        hmin = fminf(hmin, hi);
        if (lo < lo1) {
            lo2 = lo1;
            lo1 = lo;
            o1 = o;
        } else if (lo < lo2) {
            lo2 = lo;
        }
    }
};

// screen bounds of one candidate from its coordinates (a candidate without a
// fixed-point value is kept: lo 0, hi infinite)
template <int DIM>
__device__ __forceinline__ void screen_double(const double* q, const long long* pnI, int emax, float* lo, float* hi)
{
    long long dx[3];
    bool ok = true;
#pragma unroll
    for (int d = 0; d < DIM; ++d) {
        const long long v = fix_double(q[d], emax);
        ok &= v != kFixNone;
        dx[d] = v - pnI[d];
    }
    if (ok) {
        ss_bounds<DIM>(dx, lo, hi);
    } else {
        *lo = 0.0f;
        *hi = CUDART_INF_F;
    }
}

template <int DIM>
__device__ __forceinline__ void screen_fixed(const long long* ownI, int M, int s, const long long* pnI, float* lo,
                                             float* hi)
{
    long long dx[3];
    bool ok = true;
#pragma unroll
    for (int d = 0; d < DIM; ++d) {
        const long long v = ownI[d * M + s];
        ok &= v != kFixNone;
        dx[d] = v - pnI[d];
    }
    if (ok) {
        ss_bounds<DIM>(dx, lo, hi);
    } else {
        *lo = 0.0f;
        *hi = CUDART_INF_F;
    }
}

// minimum over the warp of non-negative doubles (or +Inf), on their bit patterns
__device__ __forceinline__ double warp_min_nonneg(double v)
{
    unsigned long long b = (unsigned long long)__double_as_longlong(v);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const unsigned long long w = __shfl_xor_sync(0xffffffffu, b, o);
        b = w < b ? w : b;
    }
    return __longlong_as_double((long long)b);
}

__device__ __forceinline__ float warp_min_nonneg(float v)
{
    return __uint_as_float(__reduce_min_sync(0xffffffffu, __float_as_uint(v)));
}

// One cell of _inject_particles! / _inject_particles_phase! per warp, with a
// pruned exact nearest-neighbour search. The cell's own particles sit in shared
// memory; for each new particle the warp first finds the nearest of them, then
// examines only the neighbour cells whose bounding box (from the flag pass,
// rounded outwards, widened by the new particles of earlier passes) can hold a
// particle at most that far: a skipped cell's particles are all farther, by a
// margin far above the rounding of the distances, so the minimum and its first
// occurrence in the reference's order (cells k, j, i, x fastest; slots in
// order; index_min_distance, injection.jl:330-393) are those of the full search.
template <int DIM, bool PHASE>
__device__ void inject_cell_pruned(const DevGrid& g, const Coords& X, uint8_t* __restrict__ index,
                                   const InjectLists& Ls, const Args& A, const PhaseFields& PF, uint32_t call,
                                   int64_t c, double* __restrict__ own, long long* __restrict__ ownI, int lane,
                                   int* errs)
{
    const int64_t nc = g.ncells;
    const int M = g.max_xcell;
    constexpr int NB = DIM == 2 ? 9 : 27;
    constexpr int CENTER = DIM == 2 ? 4 : 13;
    int64_t I[3];
    cell_coords(g, c, I);
    double corner[3], dq[3];
#pragma unroll
    for (int d = 0; d < DIM; ++d) {
        corner[d] = ldg(g.xv[d] + I[d]);
        dq[d] = ldg(g.dxv[d] + I[d]) / 2.0;
    }
    uint64_t ownm = Ls.lm[c];
    const int emax = fix_emax<DIM>(g);
    // the cell's own coordinates (own[d * M + s]) and their fixed-point values
    for (int s = lane; s < M; s += 32) {
        const bool lv = (ownm >> s) & 1ull;
#pragma unroll
        for (int d = 0; d < DIM; ++d) {
            const double x = lv ? X.c[d][c + nc * s] : CUDART_NAN;
            own[d * M + s] = x;
            ownI[d * M + s] = fix_double(x, emax);
        }
    }
    // lane nb < NB holds neighbour cell nb: its index, occupancy and box
    int64_t nbc = -1;
    uint64_t nbm = 0;
    float blo[3] = {0.f, 0.f, 0.f}, bhi[3] = {0.f, 0.f, 0.f};
    if (lane < NB && lane != CENTER) {
        const int64_t J[3] = {I[0] + lane % 3 - 1, I[1] + (lane / 3) % 3 - 1, DIM == 3 ? I[2] + lane / 9 - 1 : 0};
        const bool ok = J[0] >= 0 && J[1] >= 0 && J[0] < g.n[0] && J[1] < g.n[1] &&
                        (DIM == 2 || (J[2] >= 0 && J[2] < g.n[2]));
        if (ok) {
            nbc = cell_linear<DIM>(g, J);
            nbm = Ls.lm[nbc];
#pragma unroll
            for (int d = 0; d < DIM; ++d) {
                blo[d] = Ls.box[6 * nbc + d];
                bhi[d] = Ls.box[6 * nbc + 3 + d];
            }
        }
    }
    // the box in fixed point, widened by one unit each way (kFixNone: always examined)
    long long bloI[3] = {0, 0, 0}, bhiI[3] = {0, 0, 0};
    bool box_fixed = nbm != 0;
#pragma unroll
    for (int d = 0; d < DIM; ++d) {
        bloI[d] = fix_float(blo[d], emax);
        bhiI[d] = fix_float(bhi[d], emax);
        box_fixed &= bloI[d] != kFixNone && bhiI[d] != kFixNone;
    }
    // the own cell's box grows with its new particles (read by later passes)
    float olo = 0.f, ohi = 0.f;
    if (lane < DIM) {
        olo = Ls.box[6 * c + lane];
        ohi = Ls.box[6 * c + 3 + lane];
    }
    __syncwarp();
    const int min_xq = (g.min_xcell + (1 << DIM) - 1) >> DIM;
    for (int q = 0; q < (1 << DIM); ++q) {
        double qc[3];
        long long klo[3], khi[3];
#pragma unroll
        for (int d = 0; d < DIM; ++d) {
            qc[d] = corner[d] + dq[d] * (double)((q >> d) & 1);
            klo[d] = okey(qc[d]);
            khi[d] = okey(qc[d] + dq[d]);  // isincell(p, vertex, di_quadrant)
        }
        int cnt = 0;
        for (int s = lane; s < M; s += 32) {
            if (!((ownm >> s) & 1ull)) continue;
            bool in = true;
#pragma unroll
            for (int d = 0; d < DIM; ++d) {
                const double x = own[d * M + s];
                const long long k = okey(x);
                in = in & !is_nan_bits(x) & (klo[d] < k) & (k < khi[d]);
            }
            cnt += in ? 1 : 0;
        }
        int count = __reduce_add_sync(0xffffffffu, cnt);
        if (count >= min_xq) {
            if (PHASE) continue;  // inject_particles_phase! checks every quadrant (injection.jl:273)
            break;                // injection.jl:100
        }
        uint64_t freem = ~ownm & (M == 64 ? ~0ull : ((1ull << M) - 1));
        constexpr int SPB = 32 / DIM;  // new particles per batch of draws
        int k = 0;
        double ub = 0.0;
        while (freem) {
            if (k % SPB == 0)
                ub = batch_draws<DIM, double>(freem, lane, [&](int slot, int d) {
                    return jp_rand_uniform(g.seed, JP_RNG_STREAM_INJECT, call, (uint64_t)c, (uint32_t)slot,
                                           (uint32_t)d);
                });
            const int i = __ffsll((long long)freem) - 1;
            freem &= freem - 1;
            ++count;
            double pn[3];
#pragma unroll
            for (int d = 0; d < DIM; ++d) {
                const double r = __shfl_sync(0xffffffffu, ub, (k % SPB) * DIM + d);
                pn[d] = qc[d] + dq[d] * fma(0.95, r, 0.05);  // new_particle, injection.jl:411-417
            }
            ++k;
            const int64_t ai = c + nc * i;
            long long pnI[3] = {0, 0, 0};
            bool pn_fixed = true;
#pragma unroll
            for (int d = 0; d < DIM; ++d) {
                pnI[d] = fix_double(pn[d], emax);
                pn_fixed &= pnI[d] != kFixNone;
            }
            if (lane == 0) {
#pragma unroll
                for (int d = 0; d < DIM; ++d) {
                    X.c[d][ai] = pn[d];
                    own[d * M + i] = pn[d];
                    ownI[d * M + i] = pnI[d];
                }
                index[ai] = 1;
            }
            if (lane < DIM) {
                const double p = lane == 0 ? pn[0] : (lane == 1 ? pn[1] : pn[DIM - 1]);
                olo = fminf(olo, __double2float_rd(p));
                ohi = fmaxf(ohi, __double2float_ru(p));
            }
            ownm |= 1ull << i;
            __syncwarp();
            // The reference takes the first minimum of the rounded distance sqrt(ss) in its
            // order. (a) Screen: every candidate's squared distance is bounded on the
            // integer pipe; only candidates whose lower bound is within a relative 2^-20 of
            // the smallest upper bound can be the nearest (any other is farther by far more
            // than the rounding of the reference's distances), and those few are (b)
            // evaluated exactly in FP64. The exact search compares squared distances and
            // keeps, per lane, the smallest (ss1, first o) and the smallest larger ss2:
            // when no other candidate's squared distance lies within a relative 2^-50 of
            // the minimum, no other candidate can round to the same distance (a larger root
            // is ~2 ulps above) and the minimum's first occurrence is the answer; otherwise
            // (in practice never) the rounded distances are compared again. Without a
            // fixed-point value for the new particle every candidate is evaluated exactly.
            ScreenTrack st;
            // (a1) the own cell's particles
            for (int s = lane; s < M; s += 32)
                if (s != i && ((ownm >> s) & 1ull)) {
                    float lo, hi;
                    screen_fixed<DIM>(ownI, M, s, pnI, &lo, &hi);
                    st.add(lo, hi, CENTER * M + s);
                }
            const float h_own = pn_fixed ? warp_min_nonneg(st.hmin) : CUDART_INF_F;
            // (a2) neighbour cells whose box may hold a particle that close
            bool look = false;
            if (nbm != 0) {
                look = true;
                if (box_fixed && pn_fixed && h_own < CUDART_INF_F) {
                    float lb2 = 0.0f;  // lower bound of the squared distance to the box
#pragma unroll
                    for (int d = 0; d < DIM; ++d) {
                        const long long gap = max(0ll, max(bloI[d] - pnI[d] - 2, pnI[d] - bhiI[d] - 2));
                        const float gf = __ll2float_rd(gap);
                        lb2 = __fmaf_rd(gf, gf, lb2);
                    }
                    look = !(lb2 > __fmul_ru(h_own, 1.0f + 0x1p-20f));
                }
            }
            const uint32_t cells = __ballot_sync(0xffffffffu, look);
            for (uint32_t cl = cells; cl;) {
                const int nb = __ffs(cl) - 1;
                cl &= cl - 1;
                const uint64_t m = __shfl_sync(0xffffffffu, nbm, nb);
                const int64_t cc = __shfl_sync(0xffffffffu, nbc, nb);
                for (int s = lane; s < M; s += 32)
                    if ((m >> s) & 1ull) {
                        double q[3];
#pragma unroll
                        for (int d = 0; d < DIM; ++d) q[d] = X.c[d][cc + nc * s];
                        float lo, hi;
                        screen_double<DIM>(q, pnI, emax, &lo, &hi);
                        st.add(lo, hi, nb * M + s);
                    }
            }
            const float thr = pn_fixed ? __fmul_ru(warp_min_nonneg(st.hmin), 1.0f + 0x1p-20f) : CUDART_INF_F;
            // (b) exact squared distances of the candidates that pass the screen: each lane's
            // best one, and all of a lane's candidates when a second one passes too
            NearestTrack nt;
            {
                const int o = st.o1 >= 0 ? st.o1 : CENTER * M;
                const int nb1 = o / M, s1 = o - nb1 * M;
                const int64_t cc1 = __shfl_sync(0xffffffffu, nbc, nb1);
                if (st.o1 >= 0 && st.lo1 <= thr) {
                    if (nb1 == CENTER) {
                        nt.add(own_ss<DIM>(own, M, s1, pn), o);
                    } else {
                        nt.add(glob_ss<DIM>(X, cc1 + nc * s1, pn), o);
                    }
                }
            }
            const bool again = st.lo2 <= thr;
            if (__any_sync(0xffffffffu, again)) {
                NearestTrack nt2;
                for (int s = lane; s < M; s += 32)
                    if (again && s != i && ((ownm >> s) & 1ull)) {
                        float lo, hi;
                        screen_fixed<DIM>(ownI, M, s, pnI, &lo, &hi);
                        if (!pn_fixed || lo <= thr) nt2.add(own_ss<DIM>(own, M, s, pn), CENTER * M + s);
                    }
                for (uint32_t cl = cells; cl;) {
                    const int nb = __ffs(cl) - 1;
                    cl &= cl - 1;
                    const uint64_t m = __shfl_sync(0xffffffffu, nbm, nb);
                    const int64_t cc = __shfl_sync(0xffffffffu, nbc, nb);
                    for (int s = lane; s < M; s += 32)
                        if (again && ((m >> s) & 1ull)) {
                            double q[3];
#pragma unroll
                            for (int d = 0; d < DIM; ++d) q[d] = X.c[d][cc + nc * s];
                            float lo, hi;
                            screen_double<DIM>(q, pnI, emax, &lo, &hi);
                            if (!pn_fixed || lo <= thr) nt2.add(glob_ss<DIM>(X, cc + nc * s, pn), nb * M + s);
                        }
                }
                if (again) nt = nt2;
            }
            const double ss_min = warp_min_nonneg(nt.ss1);
            const double ss_next = warp_min_nonneg(nt.ss1 > ss_min ? nt.ss1 : nt.ss2);
            int win = __reduce_min_sync(0xffffffffu, (nt.ss1 == ss_min && ss_min < CUDART_INF) ? nt.o1 : 0x7fffffff);
            if (ss_min < CUDART_INF && ss_next <= ss_min * (1.0 + 0x1p-50)) {
                // near tie: first candidate in order whose rounded distance is the minimum
                const double dmin = __dsqrt_rn(ss_min);
                int lo = 0x7fffffff;
                for (int s = lane; s < M; s += 32)
                    if (s != i && ((ownm >> s) & 1ull) && __dsqrt_rn(own_ss<DIM>(own, M, s, pn)) == dmin)
                        lo = min(lo, CENTER * M + s);
                for (uint32_t cl = cells; cl;) {
                    const int nb = __ffs(cl) - 1;
                    cl &= cl - 1;
                    const uint64_t m = __shfl_sync(0xffffffffu, nbm, nb);
                    const int64_t cc = __shfl_sync(0xffffffffu, nbc, nb);
                    for (int s = lane; s < M; s += 32)
                        if (((m >> s) & 1ull) && __dsqrt_rn(glob_ss<DIM>(X, cc + nc * s, pn)) == dmin)
                            lo = min(lo, nb * M + s);
                }
                win = __reduce_min_sync(0xffffffffu, lo);
            }
            int64_t src = -1;
            if (win != 0x7fffffff) {
                const int nb = win / M, s = win - nb * M;
                const int64_t J[3] = {I[0] + nb % 3 - 1, I[1] + (nb / 3) % 3 - 1, DIM == 3 ? I[2] + nb / 9 - 1 : 0};
                src = cell_linear<DIM>(g, J) + nc * s;
            }
            if (PHASE) {
                if (src >= 0) {
                    if (lane == 0) PF.phases[ai] = PF.phases[src];
                } else {
                    *errs |= kWarnNoNeighbour;
                }
                for (int k = lane; k < A.n; k += 32)
                    A.a[k][ai] = phase_field_value<DIM>(g, PF.f[k], PF.centred[k] != 0, pn, I, corner, dq);
            } else if (src >= 0) {
                for (int k = lane; k < A.n; k += 32) A.a[k][ai] = A.a[k][src];
            } else if (A.n > 0) {
                *errs |= kWarnNoNeighbour;
            }
            __syncwarp();
            if (count >= min_xq) break;
        }
    }
    if (lane == 0) Ls.lm[c] = ownm;
    if (lane < DIM) {
        Ls.box[6 * c + lane] = olo;
        Ls.box[6 * c + 3 + lane] = ohi;
    }
}


// One colour pass: warps take the colour's listed cells in turn.
template <int DIM, bool PHASE>
__global__ void __launch_bounds__(256, 3)
    inject_pass(DevGrid g, Coords X, uint8_t* __restrict__ index, Args A, PhaseFields PF, InjectLists Ls,
                            int col, uint32_t call, int* d_err)
{
    extern __shared__ __align__(16) unsigned char smem_inject[];
    const int lane = threadIdx.x & 31;
    const int wib = threadIdx.x >> 5;
    const int M = g.max_xcell;
    double* own = (double*)smem_inject + (size_t)wib * DIM * M;
    long long* ownI = (long long*)((double*)smem_inject + (size_t)(blockDim.x >> 5) * DIM * M) + (size_t)wib * DIM * M;
    const int nwarps = (gridDim.x * blockDim.x) >> 5;
    const int gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int count = Ls.counts[col];
    int errs = 0;
    for (int k = gw; k < count; k += nwarps) {
        const int64_t c = Ls.list[Ls.off[col] + k];
        inject_cell_pruned<DIM, PHASE>(g, X, index, Ls, A, PF, call, c, own, ownI, lane, &errs);
        __syncwarp();
    }
    raise_err(d_err, errs);
}

// ------------------------------------------------- cells above 64 slots
// Containers with max_xcell > 64 do not fit the 64-bit slot masks of the
// kernels above. They run the reference's own schedule instead: the colour
// passes of move_particles! with one thread per cell walking its slots in
// order (move_safe.jl:64-125), and the colour passes of inject_particles! with
// one warp per cell (injection.jl:68-131, 232-325), the warp sharing the
// quadrant counts and the nearest-neighbour search. Same results, bit for bit.

// one cell of move_kernel! (src/Particles/move_safe.jl:72-125)
template <int DIM>
__global__ void __launch_bounds__(kThreads)
    move_wide_kernel(DevGrid g, Coords X, uint8_t* __restrict__ index, Args A, int pass, int* d_err)
{
    int64_t ncol[3] = {1, 1, 1}, off[3] = {0, 0, 0};
#pragma unroll
    for (int d = 0; d < DIM; ++d) ncol[d] = (g.n[d] + 2) / 3;
    if (DIM == 2) {  // offsets: i outermost, last axis innermost (move_safe.jl:32,39)
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
    int64_t I[3] = {0, 0, 0};
#pragma unroll
    for (int d = 0; d < DIM; ++d) {
        I[d] = 3 * J[d] + off[d];
        if (I[d] >= g.n[d]) return;
    }
    const int64_t nc = g.ncells;
    const int M = g.max_xcell;
    const int64_t c = cell_linear<DIM>(g, I);
    double corner[3], dx[3];
#pragma unroll
    for (int d = 0; d < DIM; ++d) {
        corner[d] = ldg(g.xv[d] + I[d]);
        dx[d] = ldg(g.dxv[d] + I[d]);
    }
    int errs = 0, n_exit = 0, n_far = 0, n_full = 0;
    int sp = 0;  // starting_point
    for (int ip = 0; ip < M; ++ip) {
        const int64_t a = c + nc * ip;
        if (!index[a]) continue;
        double p[3];
#pragma unroll
        for (int d = 0; d < DIM; ++d) p[d] = X.c[d][a];
        if (isincell<DIM>(p, corner, dx)) continue;
        bool inside = true;  // indomain, strict (move_safe.jl:199-206)
#pragma unroll
        for (int d = 0; d < DIM; ++d) inside &= (g.dom_lo[d] < p[d]) & (p[d] < g.dom_hi[d]);
        if (!inside) {
            index[a] = 0;
#pragma unroll
            for (int d = 0; d < DIM; ++d) X.c[d][a] = CUDART_NAN;
            for (int k = 0; k < A.n; ++k) A.a[k][a] = CUDART_NAN;
            ++n_exit;
            continue;
        }
        int64_t T[3] = {0, 0, 0};
        bool far = false;
#pragma unroll
        for (int d = 0; d < DIM; ++d) {
            T[d] = find_cell(p[d], g.xv[d], g.n[d] + 1, I[d], &errs);
            far |= T[d] - I[d] > 1 || I[d] - T[d] > 1;
        }
        double cached[JP_MAX_ARGS];
        for (int k = 0; k < A.n; ++k) cached[k] = A.a[k][a];
        index[a] = 0;
#pragma unroll
        for (int d = 0; d < DIM; ++d) X.c[d][a] = CUDART_NAN;
        for (int k = 0; k < A.n; ++k) A.a[k][a] = CUDART_NAN;
        if (far) {  // the reference's colour passes race here; the particle is dropped
            errs |= kWarnFarMove;
            ++n_far;
            continue;
        }
        const int64_t tc = cell_linear<DIM>(g, T);
        int fr = -1;
        for (int i = sp; i < M; ++i)  // find_free_memory (move_safe.jl:192-197)
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
        for (int d = 0; d < DIM; ++d) X.c[d][b] = p[d];
        for (int k = 0; k < A.n; ++k) A.a[k][b] = cached[k];
    }
    if ((n_exit | n_far | n_full) && g.counts) {
        if (n_exit) atomicAdd(g.counts + 0, (unsigned long long)n_exit);
        if (n_far) atomicAdd(g.counts + 1, (unsigned long long)n_far);
        if (n_full) atomicAdd(g.counts + 2, (unsigned long long)n_full);
    }
    raise_err(d_err, errs);
}

// one cell of _inject_particles! / _inject_particles_phase! per warp
template <int DIM, bool PHASE>
__global__ void __launch_bounds__(32 * kWarpsPerBlock)
    inject_wide_kernel(DevGrid g, Coords X, uint8_t* __restrict__ index, Args A, PhaseFields PF, int pass,
                       uint32_t call, int* d_err)
{
    int64_t ncol[3] = {1, 1, 1}, off[3] = {0, 0, 0};
#pragma unroll
    for (int d = 0; d < DIM; ++d) ncol[d] = (g.n[d] + 1) / 2;
    if (DIM == 2) {  // offsets: i outermost, last axis innermost (injection.jl:31,38)
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
    double corner[3], dq[3];
#pragma unroll
    for (int d = 0; d < DIM; ++d) {
        corner[d] = ldg(g.xv[d] + I[d]);
        dq[d] = ldg(g.dxv[d] + I[d]) / 2.0;
    }
    const int min_xq = (g.min_xcell + (1 << DIM) - 1) >> DIM;
    int errs = 0;
    for (int q = 0; q < (1 << DIM); ++q) {
        double qc[3];
#pragma unroll
        for (int d = 0; d < DIM; ++d) qc[d] = corner[d] + dq[d] * (double)((q >> d) & 1);
        int cnt = 0;
        for (int s = lane; s < M; s += 32) {
            const int64_t a = c + nc * s;
            if (!index[a]) continue;
            double p[3];
#pragma unroll
            for (int d = 0; d < DIM; ++d) p[d] = X.c[d][a];
            cnt += isincell<DIM>(p, qc, dq) ? 1 : 0;
        }
        int count = __reduce_add_sync(0xffffffffu, cnt);
        if (count >= min_xq) {
            if (PHASE) continue;  // every quadrant is checked (injection.jl:273)
            break;                // injection.jl:100
        }
        bool done = false;
        for (int base = 0; base < M && !done; base += 32) {
            const int s = base + lane;
            uint32_t freem = __ballot_sync(0xffffffffu, s < M && !index[c + nc * s]);
            while (freem) {
                const int i = base + __ffs(freem) - 1;
                freem &= freem - 1;
                ++count;
                double pn[3];
#pragma unroll
                for (int d = 0; d < DIM; ++d) {
                    const double r = jp_rand_uniform(g.seed, JP_RNG_STREAM_INJECT, call, (uint64_t)c, (uint32_t)i,
                                                     (uint32_t)d);
                    pn[d] = qc[d] + dq[d] * fma(0.95, r, 0.05);  // new_particle, injection.jl:411-417
                }
                const int64_t ai = c + nc * i;
                if (lane == 0) {
#pragma unroll
                    for (int d = 0; d < DIM; ++d) X.c[d][ai] = pn[d];
                    index[ai] = 1;
                }
                __syncwarp();
                // index_min_distance: neighbour cells k, j, i (x fastest), slots in order, strict <
                double lbest = CUDART_INF;
                int lo = 0x7fffffff;
                for (int o = lane; o < NB * M; o += 32) {
                    const int nb = o / M, sl = o - nb * M;
                    if (nb == CENTER && sl == i) continue;
                    const int64_t K[3] = {I[0] + nb % 3 - 1, I[1] + (nb / 3) % 3 - 1,
                                          DIM == 3 ? I[2] + nb / 9 - 1 : 0};
                    if (K[0] < 0 || K[1] < 0 || K[0] >= g.n[0] || K[1] >= g.n[1]) continue;
                    if (DIM == 3 && (K[2] < 0 || K[2] >= g.n[2])) continue;
                    const int64_t b = cell_linear<DIM>(g, K) + nc * sl;
                    if (!index[b]) continue;
                    double e[3];
#pragma unroll
                    for (int d = 0; d < DIM; ++d) e[d] = X.c[d][b] - pn[d];
                    const double ss = DIM == 2 ? e[0] * e[0] + e[1] * e[1] : (e[0] * e[0] + e[1] * e[1]) + e[2] * e[2];
                    const double dist = __dsqrt_rn(ss);
                    if (dist < lbest) {  // lane-strided order: the first of equal distances stays
                        lbest = dist;
                        lo = o;
                    }
                }
                const double best = warp_min(lbest);
                const int win = __reduce_min_sync(0xffffffffu, lbest == best && best < CUDART_INF ? lo : 0x7fffffff);
                int64_t src = -1;
                if (win != 0x7fffffff) {
                    const int nb = win / M, sl = win - nb * M;
                    const int64_t K[3] = {I[0] + nb % 3 - 1, I[1] + (nb / 3) % 3 - 1,
                                          DIM == 3 ? I[2] + nb / 9 - 1 : 0};
                    src = cell_linear<DIM>(g, K) + nc * sl;
                }
                if (PHASE) {
                    if (src >= 0) {
                        if (lane == 0) PF.phases[ai] = PF.phases[src];
                    } else {
                        errs |= kWarnNoNeighbour;
                    }
                    for (int k = lane; k < A.n; k += 32)
                        A.a[k][ai] = phase_field_value<DIM>(g, PF.f[k], PF.centred[k] != 0, pn, I, corner, dq);
                } else if (src >= 0) {
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
cudaError_t ensure_inject_scratch(jp_particles* P)
{
    if (P->inject.counts) return cudaSuccess;
    const int64_t nc = P->g.ncells;
    const size_t list_bytes = ((8 + (size_t)nc) * sizeof(int) + 7) & ~(size_t)7;
    const size_t lm_bytes = (size_t)nc * sizeof(uint64_t);
    char* base = nullptr;
    cudaError_t e = cudaMalloc(&base, list_bytes + lm_bytes + (size_t)nc * 6 * sizeof(float));
    if (e != cudaSuccess) return e;
    P->inject.counts = (int*)base;
    P->inject.list = P->inject.counts + 8;
    P->inject.lm = (uint64_t*)(base + list_bytes);
    P->inject.box = (float*)(base + list_bytes + lm_bytes);
    return cudaSuccess;
}

cudaError_t ensure_move_scratch(jp_particles* P, int comps)
{
    MoveScratch& m = P->move;
    if (m.rec && m.shadow_comps >= comps) return cudaSuccess;
    if (m.rec) {
        cudaError_t e = cudaStreamSynchronize(P->stream);
        if (e != cudaSuccess) return e;
        if (m.passes) cudaGraphExecDestroy(m.passes);
        cudaFree(m.rec);
        m = MoveScratch();
    }
    const int64_t nc = P->g.ncells;
    const int64_t ns = nc * P->g.max_xcell;
    size_t bytes = move_shadow_offset(P->g);  // mask arrays first
    const size_t off_shadow = bytes;
    bytes += (size_t)comps * ns * sizeof(double);
    const size_t off_orig = bytes;
    bytes += ns * sizeof(uint16_t);
    const size_t off_code = bytes;
    bytes += ns * sizeof(uint8_t);
    char* base = nullptr;
    cudaError_t e = cudaMalloc(&base, bytes);
    if (e != cudaSuccess) return e;
    m.rec = (uint64_t*)base;
    m.shadow = (double*)(base + off_shadow);
    m.orig = (uint16_t*)(base + off_orig);
    m.code = (uint8_t*)(base + off_code);
    m.shadow_comps = comps;
    m.bytes = bytes;
    return cudaSuccess;
}

static cudaError_t launch_move_wide(jp_particles* P, double* const coords[3], uint8_t* index,
                                    double* const* args, int nargs)
{
    const int N = P->g.ndim;
    Coords X{{coords[0], coords[1], N == 3 ? coords[2] : nullptr}};
    Args A{};
    A.n = nargs;
    for (int k = 0; k < nargs; ++k) A.a[k] = args[k];
    int64_t per = 1;
    for (int d = 0; d < N; ++d) per *= (P->g.n[d] + 2) / 3;
    const unsigned nb = grid_blocks(per);
    for (int pass = 0; pass < (N == 2 ? 9 : 27); ++pass) {
        if (N == 2)
            move_wide_kernel<2><<<nb, kThreads, 0, P->stream>>>(P->g, X, index, A, pass, P->d_err);
        else
            move_wide_kernel<3><<<nb, kThreads, 0, P->stream>>>(P->g, X, index, A, pass, P->d_err);
    }
    return cudaGetLastError();
}

cudaError_t launch_move(jp_particles* P, double* const coords[3], uint8_t* index, double* const* args,
                        int nargs)
{
    if (P->g.max_xcell > 64) return launch_move_wide(P, coords, index, args, nargs);
    const int N = P->g.ndim;
    cudaError_t e = ensure_move_scratch(P, shadow_stride(N + nargs));
    if (e != cudaSuccess) return e;
    P->move.replayable = 1;
    Coords X{{coords[0], coords[1], N == 3 ? coords[2] : nullptr}};
    Args A{};
    A.n = nargs;
    for (int k = 0; k < nargs; ++k) A.a[k] = args[k];
    const MoveScratch& m = P->move;
    MoveView S{m.rec,    P->g.ncells, m.code, m.orig, m.shadow, P->g.ncells * P->g.max_xcell, shadow_stride(N + nargs),
               P->g.max_xcell};
    cudaStream_t st = P->stream;
    const unsigned nb = grid_blocks(P->g.ncells);
    const unsigned nbw = grid_blocks(P->g.ncells, 32 * kWarpsPerBlock);
    const int ntw = 32 * kWarpsPerBlock;
    cudaError_t e2 = cudaSuccess;
    if (N == 2) {
        move_classify<2><<<nbw, ntw, 0, st>>>(P->g, X, index, A, S, P->d_err);
        e2 = run_allocate_passes(P, S, st);
        move_apply<2><<<nb, kThreads, 0, st>>>(P->g, X, index, A, S);
    } else {
        move_classify<3><<<nbw, ntw, 0, st>>>(P->g, X, index, A, S, P->d_err);
        e2 = run_allocate_passes(P, S, st);
        move_apply<3><<<nb, kThreads, 0, st>>>(P->g, X, index, A, S);
    }
    if (e2 != cudaSuccess) return e2;
    return cudaGetLastError();
}

// the 3^N colour passes of the allocate stage, in the reference's order
void launch_allocate_passes(const DevGrid& g, const MoveView& S, cudaStream_t st)
{
    int64_t mc[3] = {1, 1, 1};
    for (int d = 0; d < g.ndim; ++d) mc[d] = (g.n[d] + 2) / 3;  // ceil(n/3)
    const unsigned nbp = grid_blocks(mc[0] * mc[1] * mc[2], kAllocThreads);
    if (g.ndim == 2) {
        for (int pass = 0; pass < 9; ++pass)  // offsetᵢ outer, offsetⱼ inner (move_safe.jl:32)
            move_allocate_2d<<<nbp, kAllocThreads, 0, st>>>(g, S, pass / 3, pass % 3, mc[0], mc[1]);
    } else {
        for (int pass = 0; pass < 27; ++pass)  // i outer, k inner (move_safe.jl:39)
            move_allocate_3d<<<nbp, kAllocThreads, 0, st>>>(g, S, pass / 9, (pass / 3) % 3, pass % 3, mc[0],
                                                            mc[1], mc[2]);
    }
}

// The colour passes are 3^N short launches whose time is mostly one thread's
// walk, so the gaps between launches count. Their arguments never change for
// a container's scratch: the first move captures them on a private stream into
// a graph, later moves launch that graph on the caller's stream (one launch
// instead of 9 or 27). A stream that is itself being captured (a caller
// building its own graph) gets the plain launches; so does any failure to
// capture or instantiate.
cudaError_t run_allocate_passes(jp_particles* P, const MoveView& S, cudaStream_t st)
{
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    if (cudaStreamIsCapturing(st, &cs) != cudaSuccess || cs != cudaStreamCaptureStatusNone) {
        cudaGetLastError();
        launch_allocate_passes(P->g, S, st);
        return cudaGetLastError();
    }
    MoveScratch& m = P->move;
    if (m.passes && m.passes_key != (const void*)S.rec) {
        cudaGraphExecDestroy(m.passes);
        m.passes = nullptr;
    }
    if (!m.passes) {
        cudaStream_t cap = nullptr;
        cudaGraph_t graph = nullptr;
        cudaGraphExec_t exec = nullptr;
        bool ok = cudaStreamCreateWithFlags(&cap, cudaStreamNonBlocking) == cudaSuccess;
        if (ok) ok = cudaStreamBeginCapture(cap, cudaStreamCaptureModeThreadLocal) == cudaSuccess;
        if (ok) {
            launch_allocate_passes(P->g, S, cap);
            ok = cudaStreamEndCapture(cap, &graph) == cudaSuccess && graph;
        }
        if (ok) ok = cudaGraphInstantiate(&exec, graph, 0) == cudaSuccess;
        if (graph) cudaGraphDestroy(graph);
        if (cap) cudaStreamDestroy(cap);
        cudaGetLastError();
        if (!ok) {
            launch_allocate_passes(P->g, S, st);
            return cudaGetLastError();
        }
        m.passes = exec;
        m.passes_key = S.rec;
    }
    return cudaGraphLaunch(m.passes, st);
}

template <bool PHASE>
static cudaError_t inject_launch(jp_particles* P, double* const coords[3], uint8_t* index, double* const* args,
                                 int nargs, const PhaseFields& PF, uint32_t call);

cudaError_t launch_inject(jp_particles* P, double* const coords[3], uint8_t* index, double* const* args,
                          int nargs, uint32_t call)
{
    return inject_launch<false>(P, coords, index, args, nargs, PhaseFields{}, call);
}

cudaError_t launch_inject_phase(jp_particles* P, double* const coords[3], uint8_t* index, double* phases,
                                double* const* args, const double* const* fields, const int* centred, int nargs,
                                uint32_t call)
{
    PhaseFields PF{};
    PF.phases = phases;
    for (int k = 0; k < nargs; ++k) {
        PF.f[k] = fields[k];
        PF.centred[k] = centred[k];
    }
    return inject_launch<true>(P, coords, index, args, nargs, PF, call);
}

template <bool PHASE>
static cudaError_t inject_launch(jp_particles* P, double* const coords[3], uint8_t* index, double* const* args,
                                 int nargs, const PhaseFields& PF, uint32_t call)
{
    if (P->g.max_xcell > 64) {
        const int N = P->g.ndim;
        Coords X{{coords[0], coords[1], N == 3 ? coords[2] : nullptr}};
        Args A{};
        A.n = nargs;
        for (int k = 0; k < nargs; ++k) A.a[k] = args[k];
        int64_t per = 1;
        for (int d = 0; d < N; ++d) per *= (P->g.n[d] + 1) / 2;
        const unsigned nb = grid_blocks(per * 32, 32 * kWarpsPerBlock);
        for (int pass = 0; pass < (1 << N); ++pass) {
            if (N == 2)
                inject_wide_kernel<2, PHASE><<<nb, 32 * kWarpsPerBlock, 0, P->stream>>>(P->g, X, index, A, PF, pass,
                                                                                         call, P->d_err);
            else
                inject_wide_kernel<3, PHASE><<<nb, 32 * kWarpsPerBlock, 0, P->stream>>>(P->g, X, index, A, PF, pass,
                                                                                         call, P->d_err);
        }
        return cudaGetLastError();
    }
    const int N = P->g.ndim;
    const int64_t nc = P->g.ncells;
    cudaError_t e = ensure_inject_scratch(P);
    if (e != cudaSuccess) return e;
    InjectLists Ls;
    Ls.counts = P->inject.counts;
    Ls.list = P->inject.list;
    Ls.lm = P->inject.lm;
    Ls.box = P->inject.box;
    // colour regions: cells whose index parity along every axis is fixed
    int64_t cnt[3][2];
    for (int d = 0; d < 3; ++d)
        for (int o = 0; o < 2; ++o) cnt[d][o] = d < N ? (P->g.n[d] - o + 1) / 2 : (o == 0 ? 1 : 0);
    int64_t off = 0;
    for (int col = 0; col < 8; ++col) {
        Ls.off[col] = off;
        off += cnt[0][col & 1] * cnt[1][(col >> 1) & 1] * cnt[2][(col >> 2) & 1];
    }
    cudaStream_t st = P->stream;
    e = cudaMemsetAsync(P->inject.counts, 0, 8 * sizeof(int), st);
    if (e != cudaSuccess) return e;
    Coords X{{coords[0], coords[1], N == 3 ? coords[2] : nullptr}};
    CCoords CX{{coords[0], coords[1], N == 3 ? coords[2] : nullptr}};
    Args A{};
    A.n = nargs;
    for (int k = 0; k < nargs; ++k) A.a[k] = args[k];
    const unsigned nb = grid_blocks(nc);
    const int M = P->g.max_xcell;
    const int wpb = 8;  // warps per block of the pass kernels
    const size_t smem = (size_t)wpb * N * M * (sizeof(double) + sizeof(long long));  // coordinates + fixed point
    // enough warps to keep every SM busy; each strides over its colour's list
    const unsigned nbp = (unsigned)(152 * 8);
    if (N == 2) {
        if (smem > 48 * 1024) {
            e = cudaFuncSetAttribute(inject_pass<2, PHASE>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
            if (e != cudaSuccess) return e;
        }
        inject_flag<2, PHASE><<<nb, kThreads, 0, st>>>(P->g, CX, index, Ls);
        for (int pass = 0; pass < 4; ++pass) {  // offsetᵢ outer, offsetⱼ inner (injection.jl:31)
            const int col = (pass / 2) + 2 * (pass % 2);
            inject_pass<2, PHASE><<<nbp, 32 * wpb, smem, st>>>(P->g, X, index, A, PF, Ls, col, call, P->d_err);
        }
    } else {
        if (smem > 48 * 1024) {
            e = cudaFuncSetAttribute(inject_pass<3, PHASE>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
            if (e != cudaSuccess) return e;
        }
        inject_flag<3, PHASE><<<nb, kThreads, 0, st>>>(P->g, CX, index, Ls);
        for (int pass = 0; pass < 8; ++pass) {  // i outer, k inner (injection.jl:38)
            const int col = (pass / 4) + 2 * ((pass / 2) % 2) + 4 * (pass % 2);
            inject_pass<3, PHASE><<<nbp, 32 * wpb, smem, st>>>(P->g, X, index, A, PF, Ls, col, call, P->d_err);
        }
    }
    return cudaGetLastError();
}

// ------------------------------------------- move_particles! without allocating
// jp_move_particles_noalloc runs the same three stages as launch_move, but its
// scratch (occupancy masks, destination codes, origin tags, shadow records)
// lives in this fixed device array instead of memory obtained from cudaMalloc.
// The array is part of this library's device image: every GPU on which the
// library's kernels are loaded holds these bytes until the process exits. All
// calls share it and each call overwrites what the previous one left; nothing
// in it has to start at zero, because every stage writes each entry it later
// reads within the same call. Two calls whose kernels overlap on the GPU (for
// example on two streams) race on the array.
static_assert(kNoAllocScratchBytes == JP_NOALLOC_SCRATCH_BYTES, "fixed scratch size differs from the header");
static __device__ __align__(256) unsigned char g_move_scratch[kNoAllocScratchBytes];

namespace {
constexpr int kMaxDevices = 64;
std::mutex g_move_scratch_mutex;             // guards the table below (host threads may call concurrently)
void* g_move_scratch_addr[kMaxDevices] = {};  // device address of g_move_scratch, per device
}  // namespace

size_t move_scratch_bytes(const DevGrid& g, int comps)
{
    const size_t nc = (size_t)g.ncells;
    const size_t ns = nc * (size_t)g.max_xcell;
    return move_shadow_offset(g) + (size_t)comps * ns * sizeof(double) + ns * sizeof(uint16_t) + ns;
}

// Host code may not use g_move_scratch's name as a device address: it stands
// for a host-side shadow. The first call on each device (with that device
// current) asks the runtime for the real address and keeps it; this may load
// the library's device image, so that first call should happen before any
// stream capture. The table is filled under a mutex, so host threads calling
// at the same time get the same address. The address belongs to the device's
// current context: after cudaDeviceReset the library's device image is loaded
// again and may sit elsewhere, so a process that resets a device must not use
// this entry point on that device afterwards.
static cudaError_t move_scratch_address(void** out)
{
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= kMaxDevices) return cudaErrorInvalidDevice;
    std::lock_guard<std::mutex> lock(g_move_scratch_mutex);
    if (!g_move_scratch_addr[dev]) {
        void* p = nullptr;
        e = cudaGetSymbolAddress(&p, g_move_scratch);
        if (e != cudaSuccess) return e;
        g_move_scratch_addr[dev] = p;
    }
    *out = g_move_scratch_addr[dev];
    return cudaSuccess;
}

cudaError_t launch_move_noalloc(jp_particles* P, double* const coords[3], uint8_t* index, double* const* args,
                                int nargs)
{
    // this move leaves the container's own move record untouched: it no longer
    // describes the last move, so jp_move_permutation must not replay it
    P->move.replayable = 0;
    if (P->g.max_xcell > 64) return launch_move_wide(P, coords, index, args, nargs);  // needs no scratch
    const int N = P->g.ndim;
    void* scratch = nullptr;
    cudaError_t e = move_scratch_address(&scratch);
    if (e != cudaSuccess) return e;
    const int64_t nc = P->g.ncells;
    const int64_t ns = nc * P->g.max_xcell;
    char* base = (char*)scratch;
    MoveView S;
    S.rec = (uint64_t*)base;
    S.nc = nc;
    S.shadow = (double*)(base + move_shadow_offset(P->g));
    S.orig = (uint16_t*)((char*)S.shadow + (size_t)shadow_stride(N + nargs) * ns * sizeof(double));
    S.code = (uint8_t*)((char*)S.orig + ns * sizeof(uint16_t));
    S.nslots = ns;
    S.comps = shadow_stride(N + nargs);
    S.mx = P->g.max_xcell;
    Coords X{{coords[0], coords[1], N == 3 ? coords[2] : nullptr}};
    Args A{};
    A.n = nargs;
    for (int k = 0; k < nargs; ++k) A.a[k] = args[k];
    cudaStream_t st = P->stream;
    const unsigned nb = grid_blocks(nc);
    const unsigned nbw = grid_blocks(nc, 32 * kWarpsPerBlock);
    const int ntw = 32 * kWarpsPerBlock;
    if (N == 2) {
        move_classify<2><<<nbw, ntw, 0, st>>>(P->g, X, index, A, S, P->d_err);
        launch_allocate_passes(P->g, S, st);
        move_apply<2><<<nb, kThreads, 0, st>>>(P->g, X, index, A, S);
    } else {
        move_classify<3><<<nbw, ntw, 0, st>>>(P->g, X, index, A, S, P->d_err);
        launch_allocate_passes(P->g, S, st);
        move_apply<3><<<nb, kThreads, 0, st>>>(P->g, X, index, A, S);
    }
    return cudaGetLastError();
}

}  // namespace jp
