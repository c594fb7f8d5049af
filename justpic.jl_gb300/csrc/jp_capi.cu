// jp_capi.cu -- the extern "C" boundary: container life cycle, argument
// checks, error reporting and dispatch to the kernel launchers.
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "jp_internal.cuh"

namespace {

thread_local std::string g_last_error;

int fail(int code, const std::string& msg)
{
    g_last_error = msg;
    return code;
}

// the adjoint keeps 64-bit slot masks: cells of at most 64 slots
#define JP_REQUIRE_NARROW(P, what)                                                                        \
    do {                                                                                                  \
        if ((P) && (P)->g.max_xcell > 64)                                                                 \
            return fail(JP_ERR_INVALID_ARGUMENT, std::string(what) + ": needs max_xcell <= 64");         \
    } while (0)

int cuda_fail(cudaError_t e, const char* where)
{
    return fail(e == cudaErrorMemoryAllocation ? JP_ERR_OUT_OF_MEMORY : JP_ERR_CUDA,
                std::string(where) + ": " + cudaGetErrorString(e));
}

bool strictly_increasing(const double* x, int64_t n)
{
    for (int64_t i = 1; i < n; ++i)
        if (!(x[i] > x[i - 1])) return false;
    return true;
}

// After a launch: in synchronous mode wait, fold the device error word into a
// status code and the sticky warnings.
int finish(jp_particles* P, cudaError_t launch_err, const char* what)
{
    if (launch_err != cudaSuccess) return cuda_fail(launch_err, what);
    if (!P->synchronous) return JP_OK;
    return jp_synchronize(P);
}

bool check_coords(const jp_particles* P, const void* const* c)
{
    for (int d = 0; d < P->g.ndim; ++d)
        if (c == nullptr || c[d] == nullptr) return false;
    return true;
}

}  // namespace

extern "C" {

const char* jp_last_error(void) { return g_last_error.c_str(); }

int jp_particles_create(jp_particles** out, const jp_grid_desc* grid, int32_t nxcell,
                        int32_t max_xcell, int32_t min_xcell, uint64_t seed)
{
    if (!out || !grid) return fail(JP_ERR_INVALID_ARGUMENT, "null argument");
    *out = nullptr;
    const int N = grid->ndim;
    if (N != 2 && N != 3) return fail(JP_ERR_INVALID_ARGUMENT, "ndim must be 2 or 3");
    if (nxcell <= 0) return fail(JP_ERR_INVALID_ARGUMENT, "nxcell must be positive");
    for (int c = 0; c < N; ++c)
        for (int d = 0; d < N; ++d) {
            if (!grid->xi_vel[c][d] || grid->n_vel[c][d] < 2)
                return fail(JP_ERR_INVALID_ARGUMENT, "The velocity grid cannot be empty");
            if (!strictly_increasing(grid->xi_vel[c][d], grid->n_vel[c][d]))
                return fail(JP_ERR_INVALID_ARGUMENT, "velocity grids must be strictly increasing");
        }
    // particles_utils.jl:86-91: quadrant rounding of nxcell, max_xcell >= nxcell
    const int NQ = 1 << N;
    const int npq = (nxcell + NQ - 1) / NQ;
    const int nx_r = npq * NQ;
    const int mx = max_xcell > nx_r ? max_xcell : nx_r;
    if (mx > JP_MAX_XCELL) return fail(JP_ERR_INVALID_ARGUMENT, "max_xcell above JP_MAX_XCELL is not supported");

    auto* P = new jp_particles();
    jp::DevGrid& g = P->g;
    g.ndim = N;
    g.uniform = grid->uniform ? 1 : 0;
    g.np_quadrant = npq;
    g.nxcell = nx_r;
    g.max_xcell = mx;
    g.min_xcell = min_xcell;
    g.seed = seed;
    g.ncells = 1;
    for (int d = 0; d < 3; ++d) g.n[d] = 1;
    for (int d = 0; d < N; ++d) {
        g.n[d] = grid->n_vel[d][d] - 1;
        g.ncells *= g.n[d];
    }
    // host staging of every grid vector: coordinates, spacings (the
    // reference's di) and their inverses (its _di = inv.(di), computed once
    // here with the same IEEE division the kernels would use)
    std::vector<double> host;
    size_t off_xv[3], off_dxv[3], off_ixv[3], off_xvel[3][3], off_dxvel[3][3], off_ixvel[3][3];
    auto push = [&](const double* x, int64_t n) {
        size_t o = host.size();
        host.insert(host.end(), x, x + n);
        return o;
    };
    auto push_spacing = [&](const double* x, int64_t n, bool inverse) {
        size_t o = host.size();
        for (int64_t i = 0; i + 1 < n; ++i) {
            const double dx = grid->uniform ? x[1] - x[0] : x[i + 1] - x[i];
            host.push_back(inverse ? 1.0 / dx : dx);
        }
        return o;
    };
    for (int d = 0; d < N; ++d) {
        const double* x = grid->xi_vel[d][d];
        off_xv[d] = push(x, g.n[d] + 1);
        off_dxv[d] = push_spacing(x, g.n[d] + 1, false);
        off_ixv[d] = push_spacing(x, g.n[d] + 1, true);
        double lo = x[0], hi = x[0];
        for (int64_t i = 0; i <= g.n[d]; ++i) {
            lo = x[i] < lo ? x[i] : lo;
            hi = x[i] > hi ? x[i] : hi;
        }
        g.dom_lo[d] = lo;
        g.dom_hi[d] = hi;
        P->dx_host[d] = x[1] - x[0];
    }
    for (int c = 0; c < N; ++c)
        for (int d = 0; d < N; ++d) {
            const double* x = grid->xi_vel[c][d];
            const int64_t n = grid->n_vel[c][d];
            off_xvel[c][d] = push(x, n);
            off_dxvel[c][d] = push_spacing(x, n, false);
            off_ixvel[c][d] = push_spacing(x, n, true);
            g.nvel[c][d] = n;
            g.lim_lo[c][d] = x[0];  // inner_limits: first/last (src/Advection/advection.jl:73-81)
            g.lim_hi[c][d] = x[n - 1];
        }
    // Cell centres (Particles.xci) and their spacing (di.center): the interior
    // of the ghost-expanded centre grids (src/Particles/particles_utils.jl:56-79,
    // :108-140). A range stays a range: Julia's LinRange[2:end-1] is
    // LinRange(r[2], r[end-1], n - 2), whose elements are recomputed from those
    // end points ((1 - t) a + t b, t = k / (n - 1)); its spacing is element 2
    // minus element 1. Vector grids are sliced, spacing = diff.
    size_t off_xc[3], off_dxc[3], off_ixc[3];
    P->centres_ok = 1;
    for (int d = 0; d < N; ++d) {
        const double* v = d == 0 ? grid->xi_vel[1][0] : grid->xi_vel[0][d];
        const int64_t n = (d == 0 ? grid->n_vel[1][0] : grid->n_vel[0][d]) - 2;
        if (n != g.n[d] || n < 2) P->centres_ok = 0;
        const int64_t m = n < 1 ? 1 : n;
        std::vector<double> xc((size_t)m, 0.0), dxc((size_t)(m > 1 ? m - 1 : 1), 1.0), ixc(dxc.size(), 1.0);
        for (int64_t k = 0; k < n; ++k) {
            if (grid->uniform && n > 1) {
                const double tk = (double)k / (double)(n - 1);
                xc[k] = (1.0 - tk) * v[1] + tk * v[n];
            } else {
                xc[k] = v[k + 1];
            }
        }
        for (int64_t k = 0; k + 1 < n; ++k) {
            dxc[k] = grid->uniform ? xc[1] - xc[0] : xc[k + 1] - xc[k];
            ixc[k] = 1.0 / dxc[k];
        }
        off_xc[d] = push(xc.data(), (int64_t)xc.size());
        off_dxc[d] = push(dxc.data(), (int64_t)dxc.size());
        off_ixc[d] = push(ixc.data(), (int64_t)ixc.size());
        // grid_size(xvi) of grid2particle_flip!: the smallest vertex spacing (src/Interpolations/utils.jl:61-63)
        const double* x = grid->xi_vel[d][d];
        double dm = x[1] - x[0];
        for (int64_t i = 1; i < g.n[d]; ++i) dm = (x[i + 1] - x[i]) < dm ? (x[i + 1] - x[i]) : dm;
        g.idmin[d] = 1.0 / std::fabs(dm);
    }
    // The split-precision form samples velocities in cell units. Its fast path
    // takes uniform grids with the standard staggering: component c on the
    // vertices along axis c and on the ghost-expanded cell centres (vertex origin
    // - dx/2 + k*dx) along the others.
    P->staggered_std = grid->uniform ? 1 : 0;
    for (int c = 0; c < N && P->staggered_std; ++c)
        for (int d = 0; d < N && P->staggered_std; ++d) {
            const double* x = grid->xi_vel[c][d];
            const int64_t n = grid->n_vel[c][d];
            const double x0 = grid->xi_vel[d][d][0], dx = P->dx_host[d];
            const double shift = c == d ? 0.0 : -0.5;
            if (n != (c == d ? g.n[d] + 1 : g.n[d] + 2)) {
                P->staggered_std = 0;
                break;
            }
            for (int64_t k = 0; k < n; ++k)
                if (std::fabs(x[k] - (x0 + ((double)k + shift) * dx)) > 1e-9 * dx * (double)(n + 1)) {
                    P->staggered_std = 0;
                    break;
                }
        }
    // Otherwise (spacing that varies, or other ghost nodes) the form runs on per-cell
    // tables when the staggering is the standard one on that grid: component c on
    // the vertex grid along axis c; along the others the cell midpoints, with one
    // ghost node below the first vertex and one above the last, the same nodes for
    // every component.
    std::vector<float> ftab;
    size_t ftab_off[7][3] = {};
    P->f32_cells = 0;
    if (!P->staggered_std) {
        bool ok = true;
        for (int d = 0; d < N && ok; ++d) {
            const double* xv = grid->xi_vel[d][d];
            const int64_t n = g.n[d];
            const double* z0 = nullptr;
            for (int c = 0; c < N && ok; ++c) {
                if (c == d) continue;
                const double* z = grid->xi_vel[c][d];
                if (grid->n_vel[c][d] != n + 2 || !(z[0] < xv[0]) || !(z[n + 1] > xv[n])) {
                    ok = false;
                    break;
                }
                for (int64_t k = 0; k < n && ok; ++k) {
                    const double h = xv[k + 1] - xv[k];
                    ok = std::fabs(z[k + 1] - 0.5 * (xv[k] + xv[k + 1])) <= 1e-9 * h * (double)(n + 1);
                }
                if (ok && z0)
                    ok = std::fabs(z[0] - z0[0]) <= 1e-9 * (xv[1] - xv[0]) &&
                         std::fabs(z[n + 1] - z0[n + 1]) <= 1e-9 * (xv[n] - xv[n - 1]);
                if (!z0) z0 = z;
            }
            if (!ok || !z0) break;
            // tables of axis d: widths, neighbour ratios, centred-node spacings (from z0)
            std::vector<double> h((size_t)n);
            for (int64_t k = 0; k < n; ++k) h[k] = xv[k + 1] - xv[k];
            for (int t = 0; t < 7; ++t) {
                ftab_off[t][d] = ftab.size();
                for (int64_t k = 0; k < n; ++k) {
                    double v = 1.0;
                    switch (t) {
                        case 0: v = h[k]; break;
                        case 1: v = k > 0 ? h[k - 1] / h[k] : 1.0; break;
                        case 2: v = k + 1 < n ? h[k + 1] / h[k] : 1.0; break;
                        case 3: v = k > 0 ? h[k] / h[k - 1] : 1.0; break;
                        case 4: v = k + 1 < n ? h[k] / h[k + 1] : 1.0; break;
                        case 5: v = h[k] / (z0[k + 1] - z0[k]); break;
                        default: v = h[k] / (z0[k + 2] - z0[k + 1]); break;
                    }
                    ftab.push_back((float)v);
                }
            }
        }
        P->f32_cells = ok ? 1 : 0;
    }
    cudaError_t e = cudaMalloc(&P->dev_block, host.size() * sizeof(double));
    if (e == cudaSuccess)
        e = cudaMemcpy(P->dev_block, host.data(), host.size() * sizeof(double), cudaMemcpyHostToDevice);
    if (e == cudaSuccess && P->f32_cells) {
        e = cudaMalloc(&P->f32_block, ftab.size() * sizeof(float));
        if (e == cudaSuccess)
            e = cudaMemcpy(P->f32_block, ftab.data(), ftab.size() * sizeof(float), cudaMemcpyHostToDevice);
        if (e == cudaSuccess) {
            const float** tabs[7] = {P->f32ax.dxf, P->f32ax.nbl, P->f32ax.nbr, P->f32ax.tol,
                                     P->f32ax.tor, P->f32ax.cl,  P->f32ax.cr};
            for (int t = 0; t < 7; ++t)
                for (int d = 0; d < N; ++d) tabs[t][d] = P->f32_block + ftab_off[t][d];
        }
    }
    if (e == cudaSuccess) e = cudaMalloc(&P->d_err, sizeof(int));
    if (e == cudaSuccess) e = cudaMemset(P->d_err, 0, sizeof(int));
    if (e == cudaSuccess) e = cudaMalloc(&g.counts, 3 * sizeof(unsigned long long));
    if (e == cudaSuccess) e = cudaMemset(g.counts, 0, 3 * sizeof(unsigned long long));
    if (e == cudaSuccess) e = cudaMallocHost(&P->h_err, sizeof(int));
    if (e != cudaSuccess) {
        int rc = cuda_fail(e, "jp_particles_create");
        jp_particles_destroy(P);
        return rc;
    }
    for (int d = 0; d < N; ++d) {
        g.xc[d] = P->dev_block + off_xc[d];
        g.dxc[d] = P->dev_block + off_dxc[d];
        g.ixc[d] = P->dev_block + off_ixc[d];
        g.xv[d] = P->dev_block + off_xv[d];
        g.dxv[d] = P->dev_block + off_dxv[d];
        g.ixv[d] = P->dev_block + off_ixv[d];
        for (int c = 0; c < N; ++c) {
            g.xvel[c][d] = P->dev_block + off_xvel[c][d];
            g.dxvel[c][d] = P->dev_block + off_dxvel[c][d];
            g.ixvel[c][d] = P->dev_block + off_ixvel[c][d];
        }
    }
    *out = P;
    return JP_OK;
}

int jp_particles_destroy(jp_particles* P)
{
    if (!P) return JP_OK;
    cudaFree(P->dev_block);
    cudaFree(P->f32_block);
    cudaFree(P->d_err);
    cudaFree(P->g.counts);
    if (P->h_err) cudaFreeHost(P->h_err);
    if (P->move.passes) cudaGraphExecDestroy(P->move.passes);
    cudaFree(P->move.rec);  // one allocation holds all move scratch
    cudaFree(P->inject.counts);  // counters and lists share one allocation
    cudaFree(P->adj_rec);
    delete P;
    return JP_OK;
}

int jp_particles_info(const jp_particles* P, int32_t* ndim, int64_t ncells[3], int32_t* nxcell,
                      int32_t* max_xcell, int32_t* min_xcell, int64_t* np)
{
    if (!P) return fail(JP_ERR_INVALID_ARGUMENT, "null container");
    if (ndim) *ndim = P->g.ndim;
    if (ncells)
        for (int d = 0; d < 3; ++d) ncells[d] = P->g.n[d];
    if (nxcell) *nxcell = P->g.nxcell;
    if (max_xcell) *max_xcell = P->g.max_xcell;
    if (min_xcell) *min_xcell = P->g.min_xcell;
    if (np) *np = (int64_t)P->g.max_xcell * P->g.ncells;
    return JP_OK;
}

int jp_set_stream(jp_particles* P, void* s)
{
    if (!P) return fail(JP_ERR_INVALID_ARGUMENT, "null container");
    P->stream = (cudaStream_t)s;
    return JP_OK;
}

int jp_set_synchronous(jp_particles* P, int32_t sync)
{
    if (!P) return fail(JP_ERR_INVALID_ARGUMENT, "null container");
    P->synchronous = sync ? 1 : 0;
    return JP_OK;
}

int jp_synchronize(jp_particles* P)
{
    if (!P) return fail(JP_ERR_INVALID_ARGUMENT, "null container");
    cudaError_t e = cudaMemcpyAsync(P->h_err, P->d_err, sizeof(int), cudaMemcpyDeviceToHost, P->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(P->stream);
    if (e != cudaSuccess) return cuda_fail(e, "jp_synchronize");
    const int bits = *P->h_err;
    if (bits) {
        e = cudaMemsetAsync(P->d_err, 0, sizeof(int), P->stream);
        if (e != cudaSuccess) return cuda_fail(e, "jp_synchronize");
    }
    P->warnings |= (uint32_t)(bits & (jp::kWarnFarMove | jp::kWarnNoNeighbour));
    if (bits & jp::kErrBisection)
        return fail(JP_ERR_BISECTION_LIMIT, "cell search exceeded its iteration cap (NaN or out-of-grid position)");
    if (bits & jp::kErrAdjointWindow)
        return fail(JP_ERR_ADJOINT_WINDOW,
                    "adjoint: a stage point or an injection source lies outside the window the gather covers "
                    "(a step moved a particle more than one cell)");
    return JP_OK;
}

int jp_get_warnings(jp_particles* P, uint32_t* bits, int32_t clear)
{
    if (!P || !bits) return fail(JP_ERR_INVALID_ARGUMENT, "null argument");
    *bits = P->warnings;
    if (clear) P->warnings = 0;
    return JP_OK;
}

int jp_get_move_counts(jp_particles* P, uint64_t counts[3], int32_t clear)
{
    if (!P || !counts) return fail(JP_ERR_INVALID_ARGUMENT, "null argument");
    unsigned long long h[3] = {0, 0, 0};
    cudaError_t e = cudaMemcpyAsync(h, P->g.counts, sizeof(h), cudaMemcpyDeviceToHost, P->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(P->stream);
    if (e == cudaSuccess && clear) e = cudaMemsetAsync(P->g.counts, 0, sizeof(h), P->stream);
    if (e != cudaSuccess) return cuda_fail(e, "jp_get_move_counts");
    for (int k = 0; k < 3; ++k) counts[k] = h[k];
    return JP_OK;
}

int jp_get_rng_counter(const jp_particles* P, uint64_t* counter)
{
    if (!P || !counter) return fail(JP_ERR_INVALID_ARGUMENT, "null argument");
    *counter = P->inject_calls;
    return JP_OK;
}

int jp_set_rng_counter(jp_particles* P, uint64_t counter)
{
    if (!P) return fail(JP_ERR_INVALID_ARGUMENT, "null container");
    P->inject_calls = counter;
    return JP_OK;
}

int jp_init_particles(jp_particles* P, double* const coords[3], uint8_t* index)
{
    if (!P || !index || !check_coords(P, (const void* const*)coords))
        return fail(JP_ERR_INVALID_ARGUMENT, "jp_init_particles: null pointer");
    return finish(P, jp::launch_init(P, coords, index), "jp_init_particles");
}

static int advection_common(jp_particles* P, int32_t method, int interp, double alpha, const double* const V[3],
                            double dt, double* const coords[3], const uint8_t* index, const char* what)
{
    if (!P || !index || !check_coords(P, (const void* const*)coords) ||
        !check_coords(P, (const void* const*)V))
        return fail(JP_ERR_INVALID_ARGUMENT, std::string(what) + ": null pointer");
    if (method != JP_EULER && method != JP_RUNGE_KUTTA2 && method != JP_RUNGE_KUTTA4)
        return fail(JP_ERR_INVALID_ARGUMENT, std::string(what) + ": unknown integrator");
    if (method == JP_RUNGE_KUTTA2 && !(0.0 < alpha && alpha < 1.0))
        return fail(JP_ERR_INVALID_ARGUMENT, "Only 0 < α < 1 is supported");
    return finish(P, jp::launch_advection_interp(P, method, interp, alpha, V, dt, coords, index), what);
}

int jp_advection(jp_particles* P, int32_t method, double alpha, const double* const V[3], double dt,
                 double* const coords[3], const uint8_t* index)
{
    return advection_common(P, method, 0, alpha, V, dt, coords, index, "jp_advection");
}

int jp_advection_linp(jp_particles* P, int32_t method, double alpha, const double* const V[3], double dt,
                      double* const coords[3], const uint8_t* index)
{
    return advection_common(P, method, 1, alpha, V, dt, coords, index, "jp_advection_linp");
}

int jp_advection_mqs(jp_particles* P, int32_t method, double alpha, const double* const V[3], double dt,
                     double* const coords[3], const uint8_t* index)
{
    return advection_common(P, method, 2, alpha, V, dt, coords, index, "jp_advection_mqs");
}

int jp_move_particles(jp_particles* P, double* const coords[3], uint8_t* index, double* const* args,
                      int32_t nargs)
{
    if (!P || !index || !check_coords(P, (const void* const*)coords))
        return fail(JP_ERR_INVALID_ARGUMENT, "jp_move_particles: null pointer");
    if (nargs < 0 || nargs > JP_MAX_ARGS || (nargs > 0 && !args))
        return fail(JP_ERR_INVALID_ARGUMENT, "jp_move_particles: bad particle field list");
    for (int k = 0; k < nargs; ++k)
        if (!args[k]) return fail(JP_ERR_INVALID_ARGUMENT, "jp_move_particles: null field");
    return finish(P, jp::launch_move(P, coords, index, args, nargs), "jp_move_particles");
}

int jp_move_particles_noalloc(jp_particles* P, double* const coords[3], uint8_t* index, double* const* args,
                              int32_t nargs)
{
    if (!P || !index || !check_coords(P, (const void* const*)coords))
        return fail(JP_ERR_INVALID_ARGUMENT, "jp_move_particles_noalloc: null pointer");
    if (nargs < 0 || nargs > JP_MAX_ARGS || (nargs > 0 && !args))
        return fail(JP_ERR_INVALID_ARGUMENT, "jp_move_particles_noalloc: bad particle field list");
    for (int k = 0; k < nargs; ++k)
        if (!args[k]) return fail(JP_ERR_INVALID_ARGUMENT, "jp_move_particles_noalloc: null field");
    // cells of more than 64 slots run the per-cell schedule, which needs no scratch
    const size_t need =
        P->g.max_xcell > 64 ? 0 : jp::move_scratch_bytes(P->g, jp::shadow_stride(P->g.ndim + nargs));
    if (need > jp::kNoAllocScratchBytes)
        return fail(JP_ERR_INVALID_ARGUMENT,
                    "jp_move_particles_noalloc: this container needs " + std::to_string(need) +
                        " bytes of scratch but the fixed buffer holds " + std::to_string(jp::kNoAllocScratchBytes) +
                        " (JP_NOALLOC_SCRATCH_BYTES); use jp_move_particles for larger grids");
    return finish(P, jp::launch_move_noalloc(P, coords, index, args, nargs), "jp_move_particles_noalloc");
}

int jp_inject_particles(jp_particles* P, double* const coords[3], uint8_t* index, double* const* args,
                        int32_t nargs)
{
    if (!P || !index || !check_coords(P, (const void* const*)coords))
        return fail(JP_ERR_INVALID_ARGUMENT, "jp_inject_particles: null pointer");
    if (nargs < 0 || nargs > JP_MAX_ARGS || (nargs > 0 && !args))
        return fail(JP_ERR_INVALID_ARGUMENT, "jp_inject_particles: bad particle field list");
    for (int k = 0; k < nargs; ++k)
        if (!args[k]) return fail(JP_ERR_INVALID_ARGUMENT, "jp_inject_particles: null field");
    const uint32_t call = (uint32_t)P->inject_calls;
    P->inject_calls += 1;
    return finish(P, jp::launch_inject(P, coords, index, args, nargs, call), "jp_inject_particles");
}

int jp_inject_particles_phase(jp_particles* P, double* const coords[3], uint8_t* index, double* phases,
                              double* const* args, const double* const* fields, const int32_t* centred,
                              int32_t nargs)
{
    if (!P || !index || !phases || !check_coords(P, (const void* const*)coords))
        return fail(JP_ERR_INVALID_ARGUMENT, "jp_inject_particles_phase: null pointer");
    if (nargs < 0 || nargs > JP_MAX_ARGS || (nargs > 0 && (!args || !fields || !centred)))
        return fail(JP_ERR_INVALID_ARGUMENT, "jp_inject_particles_phase: bad field list");
    int cflags[JP_MAX_ARGS] = {0};
    for (int k = 0; k < nargs; ++k) {
        if (!args[k] || !fields[k]) return fail(JP_ERR_INVALID_ARGUMENT, "jp_inject_particles_phase: null field");
        cflags[k] = centred[k] != 0;
        // a centred field needs two centres per axis to interpolate between
        for (int d = 0; d < P->g.ndim && cflags[k]; ++d)
            if (P->g.n[d] < 2)
                return fail(JP_ERR_INVALID_ARGUMENT, "jp_inject_particles_phase: centred field on a 1-cell axis");
    }
    const uint32_t call = (uint32_t)P->inject_calls;
    P->inject_calls += 1;
    return finish(P, jp::launch_inject_phase(P, coords, index, phases, args, fields, cflags, nargs, call),
                  "jp_inject_particles_phase");
}

// ---- split-precision form ----------------------------------------------
static int check_f32(const jp_particles* P, const void* const* xi, const void* index, const char* what)
{
    if (!P || !index || !check_coords(P, xi)) return fail(JP_ERR_INVALID_ARGUMENT, std::string(what) + ": null pointer");
    if (!P->staggered_std && !P->f32_cells)
        return fail(JP_ERR_INVALID_ARGUMENT, std::string(what) +
                                                 ": the FP32 cell-offset form needs the standard staggering of the "
                                                 "velocity components (vertex grid along the component's axis, cell "
                                                 "midpoints plus one ghost node at each end along the others)");
    return JP_OK;
}

int jp_offsets_from_coords(jp_particles* P, const double* const coords[3], const uint8_t* index, float* const xi[3])
{
    int rc = check_f32(P, (const void* const*)xi, index, "jp_offsets_from_coords");
    if (rc) return rc;
    if (!check_coords(P, (const void* const*)coords))
        return fail(JP_ERR_INVALID_ARGUMENT, "jp_offsets_from_coords: null pointer");
    return finish(P, jp::launch_to_offsets(P, coords, index, xi), "jp_offsets_from_coords");
}

int jp_coords_from_offsets(jp_particles* P, const float* const xi[3], const uint8_t* index, double* const coords[3])
{
    int rc = check_f32(P, (const void* const*)xi, index, "jp_coords_from_offsets");
    if (rc) return rc;
    if (!check_coords(P, (const void* const*)coords))
        return fail(JP_ERR_INVALID_ARGUMENT, "jp_coords_from_offsets: null pointer");
    return finish(P, jp::launch_to_coords(P, xi, index, coords), "jp_coords_from_offsets");
}

int jp_advection_f32(jp_particles* P, int32_t method, double alpha, const float* const V[3], double dt,
                     float* const xi[3], const uint8_t* index)
{
    int rc = check_f32(P, (const void* const*)xi, index, "jp_advection_f32");
    if (rc) return rc;
    if (!check_coords(P, (const void* const*)V)) return fail(JP_ERR_INVALID_ARGUMENT, "jp_advection_f32: null velocity");
    if (method != JP_EULER && method != JP_RUNGE_KUTTA2 && method != JP_RUNGE_KUTTA4)
        return fail(JP_ERR_INVALID_ARGUMENT, "jp_advection_f32: unknown integrator");
    if (method == JP_RUNGE_KUTTA2 && !(0.0 < alpha && alpha < 1.0))
        return fail(JP_ERR_INVALID_ARGUMENT, "Only 0 < α < 1 is supported");
    return finish(P, jp::launch_advection_f32(P, method, alpha, V, dt, xi, index), "jp_advection_f32");
}

int jp_move_particles_f32(jp_particles* P, float* const xi[3], uint8_t* index, float* const* args, int32_t nargs)
{
    int rc = check_f32(P, (const void* const*)xi, index, "jp_move_particles_f32");
    if (rc) return rc;
    if (nargs < 0 || nargs > JP_MAX_ARGS || (nargs > 0 && !args))
        return fail(JP_ERR_INVALID_ARGUMENT, "jp_move_particles_f32: bad particle field list");
    for (int k = 0; k < nargs; ++k)
        if (!args[k]) return fail(JP_ERR_INVALID_ARGUMENT, "jp_move_particles_f32: null field");
    return finish(P, jp::launch_move_f32(P, xi, index, args, nargs), "jp_move_particles_f32");
}

int jp_inject_particles_f32(jp_particles* P, float* const xi[3], uint8_t* index, float* const* args, int32_t nargs)
{
    int rc = check_f32(P, (const void* const*)xi, index, "jp_inject_particles_f32");
    if (rc) return rc;
    if (nargs < 0 || nargs > JP_MAX_ARGS || (nargs > 0 && !args))
        return fail(JP_ERR_INVALID_ARGUMENT, "jp_inject_particles_f32: bad particle field list");
    for (int k = 0; k < nargs; ++k)
        if (!args[k]) return fail(JP_ERR_INVALID_ARGUMENT, "jp_inject_particles_f32: null field");
    const uint32_t call = (uint32_t)P->inject_calls;
    P->inject_calls += 1;
    return finish(P, jp::launch_inject_f32(P, xi, index, args, nargs, call), "jp_inject_particles_f32");
}

int jp_grid2particle_f32(jp_particles* P, float* Fp, const float* F, const float* const xi[3], const uint8_t* index)
{
    int rc = check_f32(P, (const void* const*)xi, index, "jp_grid2particle_f32");
    if (rc) return rc;
    if (!Fp || !F) return fail(JP_ERR_INVALID_ARGUMENT, "jp_grid2particle_f32: null field");
    return finish(P, jp::launch_g2p_f32(P, Fp, F, xi, index), "jp_grid2particle_f32");
}

int jp_particle2grid_f32(jp_particles* P, float* F, const float* Fp, const float* const xi[3], const uint8_t* index)
{
    int rc = check_f32(P, (const void* const*)xi, index, "jp_particle2grid_f32");
    if (rc) return rc;
    if (!Fp || !F) return fail(JP_ERR_INVALID_ARGUMENT, "jp_particle2grid_f32: null field");
    return finish(P, jp::launch_p2g_f32(P, F, Fp, xi, index), "jp_particle2grid_f32");
}

// ---- adjoint (FP64; the grid transfers in 2D and 3D, the rest in 2D) ----
static int check_adj(const jp_particles* P, const void* const* coords, const void* index, const char* what,
                     bool any_dim = false)
{
    if (!P || !index || !check_coords(P, coords))
        return fail(JP_ERR_INVALID_ARGUMENT, std::string(what) + ": null pointer");
    if (!any_dim && P->g.ndim != 2)
        return fail(JP_ERR_INVALID_ARGUMENT, std::string(what) + ": the adjoint is built for 2D");
    return JP_OK;
}

static bool slots_fit_int32(const jp_particles* P)
{
    return (double)P->g.ncells * P->g.max_xcell < 2147483647.0;
}

int jp_move_permutation(jp_particles* P, int32_t* dest)
{
    JP_REQUIRE_NARROW(P, "jp_move_permutation");
    if (!P || !dest) return fail(JP_ERR_INVALID_ARGUMENT, "jp_move_permutation: null pointer");
    if (!P->move.rec || !P->move.replayable)
        return fail(JP_ERR_INVALID_ARGUMENT,
                    "jp_move_permutation: the container's last move left no record to replay (no move yet, or it "
                    "was a jp_move_particles_noalloc call)");
    if (!slots_fit_int32(P)) return fail(JP_ERR_INVALID_ARGUMENT, "jp_move_permutation: more than 2^31 slots");
    return finish(P, jp::launch_move_permutation(P, dest), "jp_move_permutation");
}

int jp_permute_vjp(jp_particles* P, const int32_t* dest, const double* const* post, double* const* pre, int32_t n)
{
    JP_REQUIRE_NARROW(P, "jp_permute_vjp");
    if (!P || !dest || !post || !pre || n < 0 || n > 8)
        return fail(JP_ERR_INVALID_ARGUMENT, "jp_permute_vjp: bad arguments");
    for (int k = 0; k < n; ++k)
        if (!post[k] || !pre[k] || post[k] == pre[k])
            return fail(JP_ERR_INVALID_ARGUMENT, "jp_permute_vjp: null or aliased array");
    return finish(P, jp::launch_permute_vjp(P, dest, post, pre, n), "jp_permute_vjp");
}

int jp_slot_ids(jp_particles* P, const uint8_t* index, double* ids)
{
    JP_REQUIRE_NARROW(P, "jp_slot_ids");
    if (!P || !index || !ids) return fail(JP_ERR_INVALID_ARGUMENT, "jp_slot_ids: null pointer");
    return finish(P, jp::launch_slot_ids(P, index, ids), "jp_slot_ids");
}

int jp_inject_vjp(jp_particles* P, const double* ids, const double* const* post, double* const* pre, int32_t n,
                  int32_t copies)
{
    JP_REQUIRE_NARROW(P, "jp_inject_vjp");
    if (!P || !ids || !post || !pre || n < 0 || n > 8)
        return fail(JP_ERR_INVALID_ARGUMENT, "jp_inject_vjp: bad arguments");
    if (P->g.ndim != 2) return fail(JP_ERR_INVALID_ARGUMENT, "jp_inject_vjp: the adjoint is built for 2D");
    // in place (pre[k] == post[k] for every array) or out of place (no array aliased)
    for (int k = 0; k < n; ++k)
        if (!post[k] || !pre[k] || (post[k] == pre[k]) != (post[0] == pre[0]))
            return fail(JP_ERR_INVALID_ARGUMENT, "jp_inject_vjp: null array, or only some arrays aliased");
    return finish(P, jp::launch_inject_vjp(P, ids, post, pre, n, (unsigned)copies & ((1u << n) - 1u)),
                  "jp_inject_vjp");
}

int jp_advection_vjp(jp_particles* P, int32_t method, double alpha, const double* const V[3], double dt,
                     const double* const coords[3], const uint8_t* index, double* const lam[3], double* const gV[3])
{
    JP_REQUIRE_NARROW(P, "jp_advection_vjp");
    int rc = check_adj(P, (const void* const*)coords, index, "jp_advection_vjp");
    if (rc) return rc;
    if (!check_coords(P, (const void* const*)V) || !check_coords(P, (const void* const*)lam) ||
        !check_coords(P, (const void* const*)gV))
        return fail(JP_ERR_INVALID_ARGUMENT, "jp_advection_vjp: null pointer");
    if (method != JP_EULER && method != JP_RUNGE_KUTTA2 && method != JP_RUNGE_KUTTA4)
        return fail(JP_ERR_INVALID_ARGUMENT, "jp_advection_vjp: unknown integrator");
    if (method == JP_RUNGE_KUTTA2 && !(0.0 < alpha && alpha < 1.0))
        return fail(JP_ERR_INVALID_ARGUMENT, "Only 0 < α < 1 is supported");
    return finish(P, jp::launch_advection_vjp(P, method, alpha, V, dt, coords, index, lam, gV), "jp_advection_vjp");
}

int jp_particle2grid_with_weights(jp_particles* P, double* F, double* W, const double* Fp,
                                  const double* const coords[3], const uint8_t* index)
{
    if (!P || !Fp || !F || !W || !index || !check_coords(P, (const void* const*)coords))
        return fail(JP_ERR_INVALID_ARGUMENT, "jp_particle2grid_with_weights: null pointer");
    return finish(P, jp::launch_p2g(P, F, Fp, coords, index, W), "jp_particle2grid_with_weights");
}

int jp_particle2grid_vjp(jp_particles* P, const double* F, const double* W, const double* Fp,
                         const double* const coords[3], const uint8_t* index, const double* gF, double* gFp,
                         double* const gX[3])
{
    JP_REQUIRE_NARROW(P, "jp_particle2grid_vjp");
    int rc = check_adj(P, (const void* const*)coords, index, "jp_particle2grid_vjp", true);
    if (rc) return rc;
    if (!F || !W || !Fp || !gF || !gFp || (gX && !check_coords(P, (const void* const*)gX)))
        return fail(JP_ERR_INVALID_ARGUMENT, "jp_particle2grid_vjp: null pointer");
    return finish(P, jp::launch_p2g_vjp(P, F, W, Fp, coords, index, gF, gFp, gX), "jp_particle2grid_vjp");
}

int jp_grid2particle_vjp(jp_particles* P, const double* F, const double* gFp, const double* const coords[3],
                         const uint8_t* index, double* gF, double* const gX[3])
{
    JP_REQUIRE_NARROW(P, "jp_grid2particle_vjp");
    int rc = check_adj(P, (const void* const*)coords, index, "jp_grid2particle_vjp", true);
    if (rc) return rc;
    if (!gFp || (gX && (!F || !check_coords(P, (const void* const*)gX))))
        return fail(JP_ERR_INVALID_ARGUMENT, "jp_grid2particle_vjp: null pointer");
    return finish(P, jp::launch_g2p_vjp(P, F, gFp, coords, index, gF, gX), "jp_grid2particle_vjp");
}

int jp_grid2particle(jp_particles* P, double* Fp, const double* F, const double* const coords[3],
                     const uint8_t* index)
{
    if (!P || !Fp || !F || !index || !check_coords(P, (const void* const*)coords))
        return fail(JP_ERR_INVALID_ARGUMENT, "jp_grid2particle: null pointer");
    return finish(P, jp::launch_g2p(P, Fp, F, coords, index), "jp_grid2particle");
}

// ---- adjoint of the split-precision form (2D) ---------------------------
static int check_f32_adj(const jp_particles* P, const char* what)
{
    if (P->g.ndim != 2) return fail(JP_ERR_INVALID_ARGUMENT, std::string(what) + ": the adjoint is built for 2D");
    if (!P->g.uniform || !P->staggered_std)
        return fail(JP_ERR_INVALID_ARGUMENT, std::string(what) + ": the split-precision form needs uniform "
                                                                 "grids with the standard ghost-node staggering");
    return JP_OK;
}

int jp_slot_ids_i32(jp_particles* P, const uint8_t* index, int32_t* ids)
{
    JP_REQUIRE_NARROW(P, "jp_slot_ids_i32");
    if (!P || !index || !ids) return fail(JP_ERR_INVALID_ARGUMENT, "jp_slot_ids_i32: null pointer");
    if (!slots_fit_int32(P)) return fail(JP_ERR_INVALID_ARGUMENT, "jp_slot_ids_i32: more than 2^31 slots");
    return finish(P, jp::launch_slot_ids_i32(P, index, ids), "jp_slot_ids_i32");
}

int jp_inject_vjp_i32(jp_particles* P, const int32_t* ids, const double* const* post, double* const* pre,
                      int32_t n, int32_t copies)
{
    JP_REQUIRE_NARROW(P, "jp_inject_vjp_i32");
    if (!P || !ids || !post || !pre || n < 0 || n > 8)
        return fail(JP_ERR_INVALID_ARGUMENT, "jp_inject_vjp_i32: bad arguments");
    if (P->g.ndim != 2) return fail(JP_ERR_INVALID_ARGUMENT, "jp_inject_vjp_i32: the adjoint is built for 2D");
    // in place (pre[k] == post[k] for every array) or out of place (no array aliased)
    for (int k = 0; k < n; ++k)
        if (!post[k] || !pre[k] || (post[k] == pre[k]) != (post[0] == pre[0]))
            return fail(JP_ERR_INVALID_ARGUMENT, "jp_inject_vjp_i32: null array, or only some arrays aliased");
    return finish(P, jp::launch_inject_vjp_i32(P, ids, post, pre, n, (unsigned)copies & ((1u << n) - 1u)),
                  "jp_inject_vjp_i32");
}

int jp_advection_vjp_f32(jp_particles* P, int32_t method, double alpha, const float* const V[3], double dt,
                         const float* const xi[3], const uint8_t* index, double* const lam[3], double* const gV[3])
{
    JP_REQUIRE_NARROW(P, "jp_advection_vjp_f32");
    if (!P || !index || !check_coords(P, (const void* const*)xi) || !check_coords(P, (const void* const*)V) ||
        !check_coords(P, (const void* const*)lam) || !check_coords(P, (const void* const*)gV))
        return fail(JP_ERR_INVALID_ARGUMENT, "jp_advection_vjp_f32: null pointer");
    int rc = check_f32_adj(P, "jp_advection_vjp_f32");
    if (rc) return rc;
    if (method != JP_EULER && method != JP_RUNGE_KUTTA2 && method != JP_RUNGE_KUTTA4)
        return fail(JP_ERR_INVALID_ARGUMENT, "jp_advection_vjp_f32: unknown integrator");
    if (method == JP_RUNGE_KUTTA2 && !(0.0 < alpha && alpha < 1.0))
        return fail(JP_ERR_INVALID_ARGUMENT, "Only 0 < α < 1 is supported");
    return finish(P, jp::launch_advection_vjp_f32(P, method, alpha, V, dt, xi, index, lam, gV),
                  "jp_advection_vjp_f32");
}

int jp_particle2grid_f32_with_weights(jp_particles* P, float* F, double* W, const float* Fp, const float* const xi[3],
                                      const uint8_t* index)
{
    JP_REQUIRE_NARROW(P, "jp_particle2grid_f32_with_weights");
    if (!P || !F || !W || !Fp || !index || !check_coords(P, (const void* const*)xi))
        return fail(JP_ERR_INVALID_ARGUMENT, "jp_particle2grid_f32_with_weights: null pointer");
    if (!P->g.uniform || !P->staggered_std)
        return fail(JP_ERR_INVALID_ARGUMENT, "jp_particle2grid_f32_with_weights: the split-precision form needs "
                                             "uniform grids with the standard ghost-node staggering");
    return finish(P, jp::launch_p2g_f32(P, F, Fp, xi, index, W), "jp_particle2grid_f32_with_weights");
}

int jp_particle2grid_vjp_f32(jp_particles* P, const float* F, const double* W, const float* Fp,
                             const float* const xi[3], const uint8_t* index, const double* gF, double* gFp,
                             double* const gxi[3])
{
    JP_REQUIRE_NARROW(P, "jp_particle2grid_vjp_f32");
    if (!P || !F || !W || !Fp || !gF || !gFp || !index || !check_coords(P, (const void* const*)xi) ||
        (gxi && !check_coords(P, (const void* const*)gxi)))
        return fail(JP_ERR_INVALID_ARGUMENT, "jp_particle2grid_vjp_f32: null pointer");
    int rc = check_f32_adj(P, "jp_particle2grid_vjp_f32");
    if (rc) return rc;
    return finish(P, jp::launch_p2g_vjp_f32(P, F, W, Fp, xi, index, gF, gFp, gxi), "jp_particle2grid_vjp_f32");
}

int jp_phase_ratios(jp_particles* P, int32_t nphases, const double* phases, const double* const coords[3],
                    double* center, double* vertex, double* const faces[3])
{
    if (!P || !phases || !check_coords(P, (const void* const*)coords))
        return fail(JP_ERR_INVALID_ARGUMENT, "update_phase_ratios!: null pointer");
    if (nphases < 1 || nphases > 16)
        return fail(JP_ERR_INVALID_ARGUMENT, "update_phase_ratios!: 1 to 16 phases are supported");
    if (!P->centres_ok)
        return fail(JP_ERR_INVALID_ARGUMENT,
                    "update_phase_ratios!: needs ghost-expanded centre grids with at least 2 cells per axis");
    return finish(P, jp::launch_phase_ratios(P, nphases, phases, coords, center, vertex, faces),
                  "update_phase_ratios!");
}

int jp_phase_ratios_midpoints(jp_particles* P, int32_t nphases, const double* phases,
                              const double* const coords[3], double* const mids[3])
{
    if (!P || !phases || !mids || !check_coords(P, (const void* const*)coords))
        return fail(JP_ERR_INVALID_ARGUMENT, "update_phase_ratios!: null pointer");
    if (P->g.ndim != 3) return fail(JP_ERR_INVALID_ARGUMENT, "update_phase_ratios!: edge midpoints are 3D only");
    if (nphases < 1 || nphases > 16)
        return fail(JP_ERR_INVALID_ARGUMENT, "update_phase_ratios!: 1 to 16 phases are supported");
    if (!P->centres_ok)
        return fail(JP_ERR_INVALID_ARGUMENT,
                    "update_phase_ratios!: needs ghost-expanded centre grids with at least 2 cells per axis");
    return finish(P, jp::launch_phase_midpoints(P, nphases, phases, coords, mids), "update_phase_ratios!");
}

int jp_cellarray_permute(jp_particles* P, const void* src, void* dst, int64_t nnodes, int32_t ncomp,
                         int32_t elem_bytes, int32_t to_cpu)
{
    if (!P || !src || !dst) return fail(JP_ERR_INVALID_ARGUMENT, "jp_cellarray_permute: null pointer");
    if (nnodes < 0 || ncomp < 0) return fail(JP_ERR_INVALID_ARGUMENT, "jp_cellarray_permute: negative size");
    if (elem_bytes != 1 && elem_bytes != 2 && elem_bytes != 4 && elem_bytes != 8)
        return fail(JP_ERR_INVALID_ARGUMENT, "jp_cellarray_permute: elem_bytes must be 1, 2, 4 or 8");
    const uintptr_t a = (uintptr_t)src, b = (uintptr_t)dst;
    const uintptr_t n = (uintptr_t)nnodes * (uintptr_t)ncomp * (uintptr_t)elem_bytes;
    if (a % elem_bytes || b % elem_bytes)
        return fail(JP_ERR_INVALID_ARGUMENT, "jp_cellarray_permute: misaligned buffer");
    if (n && a < b + n && b < a + n) return fail(JP_ERR_INVALID_ARGUMENT, "jp_cellarray_permute: buffers overlap");
    return finish(P, jp::launch_cell_permute(P, src, dst, nnodes, ncomp, elem_bytes, to_cpu != 0),
                  "jp_cellarray_permute");
}

int jp_advection_record_bytes(jp_particles* P, int32_t method, uint64_t* bytes)
{
    if (!P || !bytes) return fail(JP_ERR_INVALID_ARGUMENT, "jp_advection_record_bytes: null pointer");
    JP_REQUIRE_NARROW(P, "jp_advection_record_bytes");
    if (P->g.ndim != 2) return fail(JP_ERR_INVALID_ARGUMENT, "jp_advection_record_bytes: the adjoint is 2D");
    *bytes = (uint64_t)jp::advection_record_bytes(P, method);
    return JP_OK;
}

int jp_advection_record(jp_particles* P, int32_t method, double alpha, const double* const V[3], double dt,
                        double* const coords[3], const uint8_t* index, void* rec)
{
    JP_REQUIRE_NARROW(P, "jp_advection_record");
    if (!P || !index || !rec || !check_coords(P, (const void* const*)coords) ||
        !check_coords(P, (const void* const*)V))
        return fail(JP_ERR_INVALID_ARGUMENT, "jp_advection_record: null pointer");
    if (P->g.ndim != 2) return fail(JP_ERR_INVALID_ARGUMENT, "jp_advection_record: the adjoint is 2D");
    if (method != JP_EULER && method != JP_RUNGE_KUTTA2 && method != JP_RUNGE_KUTTA4)
        return fail(JP_ERR_INVALID_ARGUMENT, "jp_advection_record: unknown integrator");
    if (method == JP_RUNGE_KUTTA2 && !(0.0 < alpha && alpha < 1.0))
        return fail(JP_ERR_INVALID_ARGUMENT, "Only 0 < α < 1 is supported");
    return finish(P, jp::launch_advection_record(P, method, alpha, V, dt, coords, index, rec), "jp_advection_record");
}

int jp_advection_vjp_recorded(jp_particles* P, int32_t method, double alpha, double dt, const void* rec,
                              const uint8_t* index, double* const lam[3], double* const gV[3])
{
    JP_REQUIRE_NARROW(P, "jp_advection_vjp_recorded");
    if (!P || !rec || !index || !lam || !gV || !lam[0] || !lam[1] || !gV[0] || !gV[1])
        return fail(JP_ERR_INVALID_ARGUMENT, "jp_advection_vjp_recorded: null pointer");
    if (P->g.ndim != 2) return fail(JP_ERR_INVALID_ARGUMENT, "jp_advection_vjp_recorded: the adjoint is 2D");
    if (method != JP_EULER && method != JP_RUNGE_KUTTA2 && method != JP_RUNGE_KUTTA4)
        return fail(JP_ERR_INVALID_ARGUMENT, "jp_advection_vjp_recorded: unknown integrator");
    return finish(P, jp::launch_advection_vjp_recorded(P, method, alpha, dt, rec, index, lam, gV),
                  "jp_advection_vjp_recorded");
}

int jp_selftest_weight(uint64_t seed, int64_t n, int64_t* mismatches, uint64_t* first_bad_input)
{
    if (!mismatches || n < 0) return fail(JP_ERR_INVALID_ARGUMENT, "jp_selftest_weight: bad arguments");
    unsigned long long* d = nullptr;
    cudaError_t e = cudaMalloc(&d, 2 * sizeof(unsigned long long));
    if (e != cudaSuccess) return cuda_fail(e, "jp_selftest_weight");
    unsigned long long h[2] = {0, 0};
    e = cudaMemset(d, 0, sizeof(h));
    if (e == cudaSuccess) e = jp::launch_weight_selftest(seed, n, d, d + 1, 0);
    if (e == cudaSuccess) e = cudaMemcpy(h, d, sizeof(h), cudaMemcpyDeviceToHost);
    cudaFree(d);
    if (e != cudaSuccess) return cuda_fail(e, "jp_selftest_weight");
    *mismatches = (int64_t)h[0];
    if (first_bad_input) *first_bad_input = h[1];
    return JP_OK;
}

int jp_grid2particle_flip(jp_particles* P, double* Fp, const double* F, const double* F0, double alpha,
                          const double* const coords[3], const uint8_t* index)
{
    if (!P || !Fp || !F || !F0 || !index || !check_coords(P, (const void* const*)coords))
        return fail(JP_ERR_INVALID_ARGUMENT, "grid2particle_flip!: null pointer");
    return finish(P, jp::launch_g2p_flip(P, Fp, F, F0, alpha, coords, index), "grid2particle_flip!");
}

int jp_centroid2particle(jp_particles* P, double* Fp, const double* F, const double* const coords[3])
{
    if (!P || !Fp || !F || !check_coords(P, (const void* const*)coords))
        return fail(JP_ERR_INVALID_ARGUMENT, "centroid2particle!: null pointer");
    if (!P->centres_ok)
        return fail(JP_ERR_INVALID_ARGUMENT,
                    "centroid2particle!: needs ghost-expanded centre grids with at least 2 cells per axis");
    return finish(P, jp::launch_c2p(P, Fp, F, coords), "centroid2particle!");
}

int jp_particle2centroid(jp_particles* P, double* F, const double* Fp, const double* const coords[3])
{
    if (!P || !Fp || !F || !check_coords(P, (const void* const*)coords))
        return fail(JP_ERR_INVALID_ARGUMENT, "particle2centroid!: null pointer");
    if (!P->centres_ok)
        return fail(JP_ERR_INVALID_ARGUMENT,
                    "particle2centroid!: needs ghost-expanded centre grids with at least 2 cells per axis");
    return finish(P, jp::launch_p2c(P, F, Fp, coords), "particle2centroid!");
}

int jp_particle2grid(jp_particles* P, double* F, const double* Fp, const double* const coords[3],
                     const uint8_t* index)
{
    if (!P || !Fp || !F || !index || !check_coords(P, (const void* const*)coords))
        return fail(JP_ERR_INVALID_ARGUMENT, "jp_particle2grid: null pointer");
    return finish(P, jp::launch_p2g(P, F, Fp, coords, index), "jp_particle2grid");
}

static int check_field_lists(const void* const* a, const void* const* b, int32_t nfields, const char* what)
{
    if (nfields < 1 || nfields > JP_MAX_ARGS || !a || !b)
        return fail(JP_ERR_INVALID_ARGUMENT, std::string(what) + ": bad field list (1 to JP_MAX_ARGS fields)");
    for (int k = 0; k < nfields; ++k)
        if (!a[k] || !b[k]) return fail(JP_ERR_INVALID_ARGUMENT, std::string(what) + ": null field");
    return JP_OK;
}

int jp_particle2grid_n(jp_particles* P, double* const* F, const double* const* Fp, int32_t nfields,
                       const double* const coords[3], const uint8_t* index)
{
    if (!P || !index || !check_coords(P, (const void* const*)coords))
        return fail(JP_ERR_INVALID_ARGUMENT, "jp_particle2grid_n: null pointer");
    int rc = check_field_lists((const void* const*)F, (const void* const*)Fp, nfields, "jp_particle2grid_n");
    if (rc) return rc;
    return finish(P, jp::launch_p2g_n(P, F, Fp, nfields, coords, index), "jp_particle2grid_n");
}

int jp_grid2particle_n(jp_particles* P, double* const* Fp, const double* const* F, int32_t nfields,
                       const double* const coords[3], const uint8_t* index)
{
    if (!P || !index || !check_coords(P, (const void* const*)coords))
        return fail(JP_ERR_INVALID_ARGUMENT, "jp_grid2particle_n: null pointer");
    int rc = check_field_lists((const void* const*)Fp, (const void* const*)F, nfields, "jp_grid2particle_n");
    if (rc) return rc;
    return finish(P, jp::launch_g2p_n(P, Fp, F, nfields, coords, index), "jp_grid2particle_n");
}

}  // extern "C"
