/*
 * justpic_gb300_rng.h -- counter-based random numbers for particle seeding and
 * reinjection.
 *
 * The reference draws `rand()` inside its kernels
 * (src/Particles/particles_utils.jl:189 for init_particles,
 *  src/Particles/injection.jl:414 for inject_particles!), which makes a run
 * impossible to reproduce bit for bit. This library replaces every such draw by
 * Philox4x32-10 (Salmon, Moraes, Dror, Shaw, "Parallel random numbers: as easy
 * as 1, 2, 3", SC'11) evaluated at a counter that names the draw:
 *
 *     counter = { cell (low 32 bits), cell (high 32 bits),
 *                 slot | dim << 16 | stream << 24, call }
 *     key     = { seed (low 32 bits), seed (high 32 bits) }
 *
 * stream 0 = init_particles (call 0), stream 1 = inject_particles! (call = the
 * number of earlier inject calls on the same container). `cell` is the 0-based
 * column-major linear cell index, `slot` the 0-based slot inside the cell and
 * `dim` the 0-based coordinate axis. The first two output words form a 64-bit
 * integer u; the double is (u >> 11) * 2^-53, uniform on [0, 1) like Julia's
 * rand(Float64).
 *
 * The header is plain C99 with optional CUDA qualifiers so that the device code
 * and any host consumer evaluate the identical function.
 */
#ifndef JUSTPIC_GB300_RNG_H
#define JUSTPIC_GB300_RNG_H

#include <stdint.h>

#if defined(__CUDACC__)
#define JP_RNG_QUAL static __host__ __device__ __forceinline__
#else
#define JP_RNG_QUAL static inline
#endif

#define JP_RNG_STREAM_INIT 0u
#define JP_RNG_STREAM_INJECT 1u

/* One Philox4x32 round constant set (published multipliers and Weyl increments). */
#define JP_PHILOX_M0 0xD2511F53u
#define JP_PHILOX_M1 0xCD9E8D57u
#define JP_PHILOX_W0 0x9E3779B9u
#define JP_PHILOX_W1 0xBB67AE85u

JP_RNG_QUAL void jp_mulhilo32(uint32_t a, uint32_t b, uint32_t* hi, uint32_t* lo)
{
    uint64_t p = (uint64_t)a * (uint64_t)b;
    *hi = (uint32_t)(p >> 32);
    *lo = (uint32_t)p;
}

/* Philox4x32 with 10 rounds: out = bijection(ctr) keyed by key. */
JP_RNG_QUAL void jp_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4])
{
    uint32_t c0 = ctr[0], c1 = ctr[1], c2 = ctr[2], c3 = ctr[3];
    uint32_t k0 = key[0], k1 = key[1];
    for (int r = 0; r < 10; ++r) {
        uint32_t hi0, lo0, hi1, lo1;
        jp_mulhilo32(JP_PHILOX_M0, c0, &hi0, &lo0);
        jp_mulhilo32(JP_PHILOX_M1, c2, &hi1, &lo1);
        uint32_t n0 = hi1 ^ c1 ^ k0;
        uint32_t n1 = lo1;
        uint32_t n2 = hi0 ^ c3 ^ k1;
        uint32_t n3 = lo0;
        c0 = n0; c1 = n1; c2 = n2; c3 = n3;
        k0 += JP_PHILOX_W0;
        k1 += JP_PHILOX_W1;
    }
    out[0] = c0; out[1] = c1; out[2] = c2; out[3] = c3;
}

/* Uniform double on [0, 1) for draw (stream, call, cell, slot, dim). */
JP_RNG_QUAL double jp_rand_uniform(uint64_t seed, uint32_t stream, uint32_t call,
                                   uint64_t cell, uint32_t slot, uint32_t dim)
{
    uint32_t ctr[4], key[2], out[4];
    ctr[0] = (uint32_t)cell;
    ctr[1] = (uint32_t)(cell >> 32);
    ctr[2] = (slot & 0xFFFFu) | ((dim & 0xFFu) << 16) | ((stream & 0xFFu) << 24);
    ctr[3] = call;
    key[0] = (uint32_t)seed;
    key[1] = (uint32_t)(seed >> 32);
    jp_philox4x32_10(ctr, key, out);
    uint64_t u = ((uint64_t)out[0] << 32) | (uint64_t)out[1];
    return (double)(u >> 11) * 0x1.0p-53;
}

/* The same draw as a float on [0, 1): the top 24 bits of that 64-bit integer. */
JP_RNG_QUAL float jp_rand_uniform_f32(uint64_t seed, uint32_t stream, uint32_t call,
                                      uint64_t cell, uint32_t slot, uint32_t dim)
{
    uint32_t ctr[4], key[2], out[4];
    ctr[0] = (uint32_t)cell;
    ctr[1] = (uint32_t)(cell >> 32);
    ctr[2] = (slot & 0xFFFFu) | ((dim & 0xFFu) << 16) | ((stream & 0xFFu) << 24);
    ctr[3] = call;
    key[0] = (uint32_t)seed;
    key[1] = (uint32_t)(seed >> 32);
    jp_philox4x32_10(ctr, key, out);
    return (float)(out[0] >> 8) * 0x1.0p-24f;
}

#endif /* JUSTPIC_GB300_RNG_H */
