// jp_internal.cuh -- shared device helpers and the container state of the
// GB300 particle-in-cell library (all kernels compile for sm_103a with
// -fmad=false: every fused multiply-add below is an explicit fma()).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/justpic_gb300.h"
#include "../../include/justpic_gb300_rng.h"

namespace jp {

// device-side error / warning bits (one int word per container)
constexpr int kErrBisection = 0x1;
constexpr int kWarnFarMove = 0x2;
constexpr int kWarnNoNeighbour = 0x4;
constexpr int kErrAdjointWindow = 0x8;  // adjoint gather window exceeded

constexpr int kBisectCap = 256;
constexpr int kThreads = 256;

// move_particles! destination codes: neighbour code (0..3^N-1) in bits 0..4,
// bit 6 = the particle is not strictly inside its new cell (it will be
// re-examined as a mover when that cell is walked), 0x3F = leaves / dropped.
constexpr uint8_t kCodeExit = 0x3F;
constexpr uint8_t kCodeUnstable = 0x40;
constexpr uint8_t kCodeStay = 0x80;  // live slot that did not move (never read as a destination)

// Geometry of a container, passed to kernels by value.
struct DevGrid {
    int ndim;
    int max_xcell;
    int nxcell;
    int min_xcell;
    int np_quadrant;
    int uniform;
    int64_t n[3];
    int64_t ncells;
    uint64_t seed;
    const double* xv[3];        // vertex grid, n[d]+1
    const double* dxv[3];       // vertex spacing per cell, n[d]
    const double* ixv[3];       // 1/spacing per cell (the reference's inv(di), computed once)
    const double* xvel[3][3];   // velocity grid of component c along axis d
    const double* dxvel[3][3];  // its spacing per interval
    const double* ixvel[3][3];  // 1/spacing per interval
    int64_t nvel[3][3];
    double dom_lo[3], dom_hi[3];  // extrema of the vertex grid
    double lim_lo[3][3], lim_hi[3][3];  // first/last of every velocity grid
    const double* xc[3];   // cell centres (Particles.xci), n[d]
    const double* dxc[3];  // their spacing (di.center) per interval, n[d] - 1
    const double* ixc[3];  // 1/spacing
    double idmin[3];       // 1 / smallest vertex spacing per axis (grid_size, the FLIP transfer's di)
    // move_particles! counts since the last jp_get_move_counts with clear: particles that
    // left the domain, moved more than one cell (dropped), found no free slot (dropped)
    unsigned long long* counts;
};

// Per-cell spacing tables of the split-precision form on grids whose spacing
// varies (one array of n[d] entries per axis and table, built at container
// creation). Ratios past the ends of an axis are 1.
struct F32Axes {
    const float* dxf[3];  // cell widths dx[i]
    const float* nbl[3];  // dx[i-1] / dx[i]: a length in cell i-1's units -> cell i's
    const float* nbr[3];  // dx[i+1] / dx[i]
    const float* tol[3];  // dx[i] / dx[i-1]: a length in cell i's units -> cell i-1's
    const float* tor[3];  // dx[i] / dx[i+1]
    const float* cl[3];   // dx[i] / (distance from the centred node left of cell i's centre to that centre)
    const float* cr[3];   // dx[i] / (distance from cell i's centre to the centred node right of it)
};

// Scratch owned by a container for move_particles! (allocated on first use).
struct MoveScratch {
    uint64_t* rec = nullptr;  // the per-cell 64-bit slot mask arrays (layout: MoveView)
    uint8_t* code = nullptr;  // destination code per mover slot (3D)
    uint16_t* orig = nullptr; // origin tag per refilled slot
    double* shadow = nullptr; // movers' coordinates and fields, per component
    int shadow_comps = 0;
    size_t bytes = 0;
    // the masks and origin tags above describe the container's last move (set by
    // the moves that use this scratch, cleared by any move that does not), so
    // jp_move_permutation can rebuild that move's permutation from them
    int replayable = 0;
    // the colour passes of a move on this scratch, captured once as a CUDA graph
    // (their arguments depend only on the container and the scratch's address)
    cudaGraphExec_t passes = nullptr;
    const void* passes_key = nullptr;
};

struct InjectScratch {
    int* counts = nullptr;     // flagged cells per colour (8 counters), then the lists
    int* list = nullptr;       // flagged cells, one region per colour
    uint64_t* lm = nullptr;    // occupancy mask per cell (written by the flag pass)
    float* box = nullptr;      // bounding box of each cell's live particles (flag pass)
};

// counters, lists and masks of inject_particles! in one allocation
cudaError_t ensure_inject_scratch(jp_particles* P);

}  // namespace jp

struct jp_particles {
    jp::DevGrid g;
    double* dev_block = nullptr;  // all grid vectors in one allocation
    int* d_err = nullptr;         // device error/warning word
    int* h_err = nullptr;         // pinned mirror
    cudaStream_t stream = nullptr;
    int synchronous = 1;
    uint32_t warnings = 0;
    uint64_t inject_calls = 0;
    double dx_host[3] = {1.0, 1.0, 1.0};  // spacing per axis (uniform grids) for the split-precision form
    int staggered_std = 0;                // uniform grids with ghost nodes half a cell out (the fast split form)
    int f32_cells = 0;                    // the split-precision form runs on per-cell spacing tables
    float* f32_block = nullptr;           // those tables (F32Axes), one allocation
    jp::F32Axes f32ax{};
    int centres_ok = 0;                   // the centre grids have one node per cell and >= 2 nodes per axis
    jp::MoveScratch move;
    jp::InjectScratch inject;
    void* adj_rec = nullptr;  // adjoint records of the last advection VJP
};

namespace jp {

__device__ __forceinline__ void cell_coords(const DevGrid& g, int64_t c, int64_t I[3])
{
    I[0] = c % g.n[0];
    I[1] = (c / g.n[0]) % g.n[1];
    I[2] = g.ndim == 3 ? c / (g.n[0] * g.n[1]) : 0;
}

template <int DIM>
__device__ __forceinline__ int64_t cell_linear(const DevGrid& g, const int64_t I[3])
{
    if (DIM == 2) return I[0] + g.n[0] * I[1];
    return I[0] + g.n[0] * (I[1] + g.n[1] * I[2]);
}

__device__ __forceinline__ double ldg(const double* p) { return __ldg(p); }

// lerp(t, v0, v1) = muladd(t, v1, muladd(-t, v0, v0)) (src/Interpolations/ndlerp.jl:15)
__device__ __forceinline__ double lerp1(double t, double v0, double v1)
{
    return fma(t, v1, fma(-t, v0, v0));
}

template <int DIM>
__device__ __forceinline__ double lerpN(const double* v, const double* t)
{
    if (DIM == 2) return lerp1(t[1], lerp1(t[0], v[0], v[1]), lerp1(t[0], v[2], v[3]));
    return lerp1(t[2], lerp1(t[1], lerp1(t[0], v[0], v[1]), lerp1(t[0], v[2], v[3])),
                 lerp1(t[1], lerp1(t[0], v[4], v[5]), lerp1(t[0], v[6], v[7])));
}

// find_parent_cell_bisection (src/Utils.jl:117-130), 0-based, bounded.
// Result: s with x[s] <= px <= x[s+1]. When px lies strictly between two
// nodes that s is unique, so a short local walk from the seed finds it; only a
// px that sits exactly on a node (two valid answers) replays the reference's
// bisection step by step to get the same pick.
__device__ __forceinline__ int64_t bisect_exact(double px, const double* x, int64_t len,
                                                int64_t seed, int* errs)
{
    int64_t lo = 0, hi = len - 1, s = seed;
    for (int it = 0; it < kBisectCap; ++it) {
        const double a = ldg(x + s), b = ldg(x + s + 1);
        if (a <= px && px <= b) return s;
        if (a < px) {
            lo = s;
            s = (hi + s) / 2;
        } else {
            hi = s;
            s = (lo + s) / 2;
        }
    }
    *errs |= kErrBisection;
    return s;
}

__device__ __forceinline__ int64_t find_cell(double px, const double* x, int64_t len, int64_t seed,
                                             int* errs)
{
    double a = ldg(x + seed), b = ldg(x + seed + 1);
    if (a <= px && px <= b) return seed;  // the reference's first test
    int64_t k = seed;
    if (px < a) {
#pragma unroll 1
        for (int it = 0; it < 4 && k > 0; ++it) {
            --k;
            b = a;
            a = ldg(x + k);
            if (a <= px && px <= b) {
                if (px == a || px == b) return bisect_exact(px, x, len, seed, errs);
                return k;
            }
        }
    } else if (px > b) {
#pragma unroll 1
        for (int it = 0; it < 4 && k + 2 < len; ++it) {
            ++k;
            a = b;
            b = ldg(x + k + 1);
            if (a <= px && px <= b) {
                if (px == a || px == b) return bisect_exact(px, x, len, seed, errs);
                return k;
            }
        }
    }
    return bisect_exact(px, x, len, seed, errs);
}

template <int DIM>
__device__ __forceinline__ bool isincell(const double* p, const double* corner, const double* dx)
{
    bool in = true;
#pragma unroll
    for (int d = 0; d < DIM; ++d) in = in & (corner[d] < p[d]) & (p[d] < corner[d] + dx[d]);
    return in;
}

template <int DIM>
__host__ __device__ constexpr int self_code()
{
    return DIM == 2 ? 4 : 13;
}

template <int DIM>
__device__ __forceinline__ int nb_code(const int off[3])
{
    return DIM == 2 ? (off[0] + 1) + 3 * (off[1] + 1)
                    : (off[0] + 1) + 3 * (off[1] + 1) + 9 * (off[2] + 1);
}

template <int DIM>
__device__ __forceinline__ void nb_offset(int code, int off[3])
{
    off[0] = code % 3 - 1;
    off[1] = (code / 3) % 3 - 1;
    off[2] = DIM == 3 ? code / 9 - 1 : 0;
}

__device__ __forceinline__ void raise_err(int* d_err, int bits)
{
    if (bits) atomicOr(d_err, bits);
}

// ---- injection draws, a batch per warp ----------------------------------
// A cell's new particles take the free slots lowest first, each with DIM
// draws that depend only on (slot, axis). Instead of every lane drawing every
// value, lane l draws axis l % DIM of the (l / DIM)-th lowest slot of `free`
// (32 / DIM slots per batch; 0 for lanes past the batch or the free slots);
// new particle k of the batch reads its axis d from lane k * DIM + d.
template <int DIM, typename T, typename Draw>
__device__ __forceinline__ T batch_draws(uint64_t free, int lane, Draw draw)
{
    const int j = lane / DIM, d = lane - j * DIM;
    if (j >= 32 / DIM) return T(0);
    uint64_t m = free;
    for (int t = 0; t < j && m; ++t) m &= m - 1;
    return m ? draw(__ffsll((long long)m) - 1, d) : T(0);
}

// ---- exact IEEE comparisons on the integer pipe ------------------------
// GB300 issues FP64 instructions (compares included) at a small fraction of
// its integer rate, so range tests use an order-preserving integer key of
// the double: for non-NaN x, y,  x <= y  <=>  okey(x) <= okey(y)  and
// x < y  <=>  okey(x) < okey(y)  (-0.0 maps to the key of +0.0). A NaN
// compares false with everything, exactly like the FP64 comparison.
__device__ __forceinline__ long long okey(double x)
{
    long long b = __double_as_longlong(x);
    b = (b == (long long)0x8000000000000000ull) ? 0ll : b;
    return b ^ ((b >> 63) & 0x7fffffffffffffffll);
}

// the double of an integer key (inverse of okey; -0.0 comes back as +0.0)
__device__ __forceinline__ double okey_value(long long k)
{
    return __longlong_as_double(k ^ ((k >> 63) & 0x7fffffffffffffffll));
}

__device__ __forceinline__ bool is_nan_bits(double x)
{
    return (__double_as_longlong(x) & 0x7fffffffffffffffll) > 0x7ff0000000000000ll;
}

// ---- warp-level compaction of live slots -------------------------------
// A warp owns 32 consecutive cells. `mask[s]` holds, per slot s, the lanes
// whose cell has slot s live; `pre[s]` is the number of live slots before s.
// Live slot number k (slot-major order) belongs to slot s with
// pre[s] <= k < pre[s+1] and to the lane of the (k - pre[s])-th set bit of
// mask[s]. Work then runs with all 32 lanes busy instead of one lane per cell
// stepping through mostly empty slots.
struct SlotList {
    uint32_t mask[64];
    int pre[65];
};

__device__ __forceinline__ int nth_set_bit(uint32_t m, int n)
{
    int pos = 0, c;
    c = __popc(m & 0xFFFFu);
    if (n >= c) { n -= c; m >>= 16; pos += 16; }
    c = __popc(m & 0xFFu);
    if (n >= c) { n -= c; m >>= 8; pos += 8; }
    c = __popc(m & 0xFu);
    if (n >= c) { n -= c; m >>= 4; pos += 4; }
    c = __popc(m & 0x3u);
    if (n >= c) { n -= c; m >>= 2; pos += 2; }
    if (n >= (int)(m & 1u)) pos += 1;
    return pos;
}

// Builds the list for cells c0 .. c0+31 (lanes past ncells own no cell) and
// returns the number of live slots. Also returns the lane's own 64-bit live mask.
__device__ __forceinline__ int build_slot_list(SlotList& Lst, const uint8_t* __restrict__ index, int64_t c0,
                                               int64_t nc, int M, int lane, uint64_t* own_live)
{
    const bool valid = c0 + lane < nc;
    int K = 0;
    uint64_t mine = 0;
#pragma unroll 4
    for (int s = 0; s < M; ++s) {
        const bool live = valid && index[c0 + lane + nc * s] != 0;
        const uint32_t m = __ballot_sync(0xffffffffu, live);
        if (lane == 0) {
            Lst.mask[s] = m;
            Lst.pre[s] = K;
        }
        mine |= (uint64_t)live << s;
        K += __popc(m);
    }
    if (lane == 0) Lst.pre[M] = K;
    __syncwarp();
    *own_live = mine;
    return K;
}

__device__ __forceinline__ void slot_item(const SlotList& Lst, int M, int k, int* slot, int* lane)
{
    int lo = 0, hi = M;
    while (hi - lo > 1) {
        const int mid = (lo + hi) >> 1;
        if (Lst.pre[mid] <= k) lo = mid;
        else hi = mid;
    }
    *slot = lo;
    *lane = nth_set_bit(Lst.mask[lo], k - Lst.pre[lo]);
}

// slot_item for a lane whose items k only increase (k, k + 32, ...): the row
// of item k is searched forward from the row of the lane's previous item
// (*row, 0 before the first), a few rows back, instead of bisected over all
// rows. Same answer: the last row s with pre[s] <= k.
__device__ __forceinline__ void slot_item_next(const SlotList& Lst, int M, int k, int* row, int* slot, int* lane)
{
    int s = *row;
    while (s + 1 < M && Lst.pre[s + 1] <= k) ++s;
    *row = s;
    *slot = s;
    *lane = nth_set_bit(Lst.mask[s], k - Lst.pre[s]);
}

constexpr int kWarpsPerBlock = 8;

// 64-bit occupancy mask of cell c (bit s = slot s is live)
__device__ __forceinline__ uint64_t live_mask(const uint8_t* __restrict__ index, int64_t c, int64_t nc, int M)
{
    uint64_t m = 0;
#pragma unroll 8
    for (int s = 0; s < M; ++s) m |= (uint64_t)(index[c + nc * s] != 0) << s;
    return m;
}

inline unsigned grid_blocks(int64_t n, int threads = kThreads)
{
    return (unsigned)((n + threads - 1) / threads);
}

// launchers (one translation unit each)
cudaError_t launch_init(jp_particles* P, double* const coords[3], uint8_t* index);
cudaError_t launch_advection(jp_particles* P, int method, double alpha, const double* const V[3],
                             double dt, double* const coords[3], const uint8_t* index);
// interp: 0 N-linear (advection!), 1 LinP (advection_LinP!), 2 MQS (advection_MQS!)
cudaError_t launch_advection_interp(jp_particles* P, int method, int interp, double alpha, const double* const V[3],
                                    double dt, double* const coords[3], const uint8_t* index);
cudaError_t launch_move(jp_particles* P, double* const coords[3], uint8_t* index,
                        double* const* args, int nargs);
cudaError_t launch_inject(jp_particles* P, double* const coords[3], uint8_t* index,
                          double* const* args, int nargs, uint32_t call);
cudaError_t launch_inject_phase(jp_particles* P, double* const coords[3], uint8_t* index, double* phases,
                                double* const* args, const double* const* fields, const int* centred, int nargs,
                                uint32_t call);
cudaError_t launch_g2p(jp_particles* P, double* Fp, const double* F, const double* const coords[3],
                       const uint8_t* index);
// transfers beside the hot path (jp_transfer.cu)
cudaError_t launch_g2p_flip(jp_particles* P, double* Fp, const double* F, const double* F0, double alpha,
                            const double* const coords[3], const uint8_t* index);
cudaError_t launch_c2p(jp_particles* P, double* Fp, const double* F, const double* const coords[3]);
cudaError_t launch_p2c(jp_particles* P, double* F, const double* Fp, const double* const coords[3]);
cudaError_t launch_phase_ratios(jp_particles* P, int nph, const double* phases, const double* const coords[3],
                                double* center, double* vertex, double* const faces[3]);
cudaError_t launch_phase_midpoints(jp_particles* P, int nph, const double* phases, const double* const coords[3],
                                   double* const mids[3]);
// CellArray layout conversion, GPU form (node + nnodes * k) <-> CPU form (k + ncomp * node)
cudaError_t launch_cell_permute(jp_particles* P, const void* src, void* dst, int64_t nnodes, int ncomp,
                                int elem_bytes, bool to_cpu);
// inv_dist2 (particle2grid! weights) against CUDA's chain: mismatch count and first bad input
cudaError_t launch_weight_selftest(uint64_t seed, int64_t n, unsigned long long* d_bad, unsigned long long* d_first,
                                   cudaStream_t st);
// advection! that records its velocity samples, and the VJP of a recorded step (2D FP64)
size_t advection_record_bytes(const jp_particles* P, int method);
cudaError_t launch_advection_record(jp_particles* P, int method, double alpha, const double* const V[3], double dt,
                                    double* const coords[3], const uint8_t* index, void* rec);
cudaError_t launch_advection_vjp_recorded(jp_particles* P, int method, double alpha, double dt, const void* rec,
                                          const uint8_t* index, double* const lam[3], double* const gV[3]);
cudaError_t launch_p2g(jp_particles* P, double* F, const double* Fp, const double* const coords[3],
                       const uint8_t* index, double* W = nullptr);
// the tuple forms of particle2grid! and grid2particle! (nf fields)
cudaError_t launch_p2g_n(jp_particles* P, double* const* F, const double* const* Fp, int nf,
                         const double* const coords[3], const uint8_t* index);
cudaError_t launch_g2p_n(jp_particles* P, double* const* Fp, const double* const* F, int nf,
                         const double* const coords[3], const uint8_t* index);

// adjoint (jp_adjoint.cu), 2D
cudaError_t launch_move_permutation(jp_particles* P, int32_t* dest);
cudaError_t launch_permute_vjp(jp_particles* P, const int32_t* dest, const double* const* post, double* const* pre,
                               int n);
cudaError_t launch_slot_ids(jp_particles* P, const uint8_t* index, double* ids);
cudaError_t launch_inject_vjp(jp_particles* P, const double* ids, const double* const* post, double* const* pre,
                              int n, unsigned copies);
cudaError_t launch_advection_vjp(jp_particles* P, int method, double alpha, const double* const V[3], double dt,
                                 const double* const coords[3], const uint8_t* index, double* const lam[3],
                                 double* const gV[3]);
cudaError_t launch_p2g_vjp(jp_particles* P, const double* F, const double* W, const double* Fp,
                           const double* const coords[3], const uint8_t* index, const double* gF, double* gFp,
                           double* const gX[3]);
cudaError_t launch_g2p_vjp(jp_particles* P, const double* F, const double* gFp, const double* const coords[3],
                           const uint8_t* index, double* gF, double* const gX[3]);

// scratch of move_particles! owned by the container (allocated on first use)
cudaError_t ensure_move_scratch(jp_particles* P, int comps);
// stride of a shadow record of `comps` doubles: 3 (2D with one field) is padded
// to 4, so that every record is one aligned 32-byte sector for apply's gathers
inline int shadow_stride(int comps) { return comps == 3 ? 4 : comps; }
struct MoveView;
void launch_allocate_passes(const DevGrid& g, const MoveView& S, cudaStream_t st);
// the same passes of a move on the container's own scratch, replayed from a CUDA graph
cudaError_t run_allocate_passes(jp_particles* P, const MoveView& S, cudaStream_t st);

// split-precision form (jp_f32.cu)
cudaError_t launch_to_offsets(jp_particles* P, const double* const coords[3], const uint8_t* index,
                              float* const xi[3]);
cudaError_t launch_to_coords(jp_particles* P, const float* const xi[3], const uint8_t* index,
                             double* const coords[3]);
cudaError_t launch_advection_f32(jp_particles* P, int method, double alpha, const float* const V[3], double dt,
                                 float* const xi[3], const uint8_t* index);
cudaError_t launch_move_f32(jp_particles* P, float* const xi[3], uint8_t* index, float* const* args, int nargs);
cudaError_t launch_inject_f32(jp_particles* P, float* const xi[3], uint8_t* index, float* const* args, int nargs,
                              uint32_t call);
cudaError_t launch_g2p_f32(jp_particles* P, float* Fp, const float* F, const float* const xi[3],
                           const uint8_t* index);
cudaError_t launch_p2g_f32(jp_particles* P, float* F, const float* Fp, const float* const xi[3],
                           const uint8_t* index, double* W = nullptr);
// adjoint of the split-precision form (jp_adjoint.cu), 2D
cudaError_t launch_slot_ids_i32(jp_particles* P, const uint8_t* index, int32_t* ids);
cudaError_t launch_inject_vjp_i32(jp_particles* P, const int32_t* ids, const double* const* post,
                                  double* const* pre, int n, unsigned copies);
cudaError_t launch_advection_vjp_f32(jp_particles* P, int method, double alpha, const float* const V[3], double dt,
                                     const float* const xi[3], const uint8_t* index, double* const lam[3],
                                     double* const gV[3]);
cudaError_t launch_p2g_vjp_f32(jp_particles* P, const float* F, const double* W, const float* Fp,
                               const float* const xi[3], const uint8_t* index, const double* gF, double* gFp,
                               double* const gxi[3]);

// move_particles! with its scratch in a fixed device array (no allocation)
constexpr size_t kNoAllocScratchBytes = (size_t)32 << 20;
size_t move_scratch_bytes(const DevGrid& g, int comps);
cudaError_t launch_move_noalloc(jp_particles* P, double* const coords[3], uint8_t* index,
                                double* const* args, int nargs);

// argument blocks passed by value
struct Coords {
    double* c[3];
};
struct CCoords {
    const double* c[3];
};
struct Args {
    double* a[JP_MAX_ARGS];
    int n;
};

}  // namespace jp
