// jp_weight.cuh -- the inverse-distance weight of particle2grid!,
// w = inv(distance^2) with distance = sqrt(ss) (src/Interpolations/particle_to_grid.jl:203-205),
// i.e. w = RN(1 / RN(RN(sqrt(ss))^2)) in IEEE double, without FP64 instructions.
//
// GB300 issues FP64 at 2 lanes per clock per SM, 64 times below its FP32 and
// integer rates, and CUDA's correctly rounded double sqrt and reciprocal cost
// most of particle2grid!'s FP64 issue slots. Here the three roundings are
// carried out on the 53-bit significands with 64/128-bit integer arithmetic:
//
//  * sqrt: for ss = m 2^t (t even after moving one bit into m), the root's
//    significand is RN(sqrt(N)) with N = m 2^52 < 2^106. q = floor(sqrt(N)) comes
//    from a float-float seed (~46 bits) and one Newton correction
//    q += (N - q^2)/(2q), the quotient taken in FP32 (it only has to be right
//    to a unit), then the exact remainder r = N - q^2 is brought into [0, 2q].
//    sqrt(N) is never a half-integer, so RN rounds up exactly when r > q.
//  * square: the 106-bit product of the root's significand with itself,
//    rounded to 53 bits, ties to even.
//  * reciprocal: for a significand M in [2^52, 2^53), floor(2^105 / M) the same
//    way (float-float seed, one Newton correction q += (2^105 - qM)/M, exact
//    remainder into [0, M)); 2^105 / M is never a half-integer, so RN rounds
//    up exactly when 2 r > M.
//
// This is textbook Newton-Raphson with an exact integer remainder test (e.g.
// J.-M. Muller et al., Handbook of Floating-Point Arithmetic, 2nd ed., ch. 4.7
// and 11, and the integer square root of Knuth, TAOCP vol. 2, 4.3.3). Inputs
// outside the range where every intermediate stays a normal double (ss zero,
// subnormal, Inf, NaN, or a result that would leave the normal range) and any
// remainder test that fails take CUDA's own __dsqrt_rn / __dmul_rn /
// __drcp_rn chain instead. jp_selftest_weight checks the two against each
// other bit for bit.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace jp {

struct U128 {
    uint64_t lo, hi;
};

__device__ __forceinline__ U128 mul_u64(uint64_t a, uint64_t b) { return {a * b, __umul64hi(a, b)}; }

// a positive normal float as an integer: x = mant << shift (shift >= 0 here)
__device__ __forceinline__ uint64_t float_to_scaled_u64(float x, int scale2)
{
    const uint32_t b = __float_as_uint(x);
    const uint64_t mant = (b & 0x7FFFFFu) | 0x800000u;
    const int shift = (int)((b >> 23) & 0xFFu) - 150 + scale2;  // x 2^scale2 = mant 2^shift
    return shift >= 0 ? mant << shift : mant >> (-shift);
}

// an int64 of magnitude < 2^62 as a float (relative error < 2^-23)
__device__ __forceinline__ float i64_to_float(int64_t v)
{
    return fmaf(__int2float_rn((int)(v >> 32)), 0x1p32f, __uint2float_rn((uint32_t)v));
}

// floor(sqrt(m 2^52)) for m in [2^52, 2^54), with r = m 2^52 - q^2 in [0, 2q]; false
// if the remainder could not be brought there. Seed: the float-float square
// root s + t of m (s = RN(sqrt(a)) for the top 24 bits a of m, its exact
// residual a - s^2 from one FMA), good to ~2^-46; then one Newton step on the
// 64-bit residual (|N - q^2| < 2^62 there, so its low 64 bits are exact).
__device__ __forceinline__ bool isqrt_sig(uint64_t m, uint64_t* q_out, uint64_t* r_out)
{
    const uint64_t Nlo = m << 52;  // N mod 2^64
    const float a = __uint2float_rn((uint32_t)(m >> 30)) * 0x1p30f;  // exact: top 24 bits of m
    const float b = __uint2float_rn((uint32_t)(m & ((1u << 30) - 1)));
    const float s = __fsqrt_rn(a);
    const float e = fmaf(-s, s, a);  // exact
    const float hs = 0.5f / s;
    const float t = (e + b) * hs;
    uint64_t q = float_to_scaled_u64(s, 26) + (int64_t)__float2int_rn(t * 0x1p26f);
    int64_t r = (int64_t)(Nlo - q * q);
    q += (int64_t)__float2int_rn(i64_to_float(r) * hs * 0x1p-26f);
    r = (int64_t)(Nlo - q * q);
#pragma unroll
    for (int k = 0; k < 2; ++k)
        if (r < 0) {  // q too large: N - (q-1)^2 = r + 2q - 1
            r += (int64_t)(2 * q - 1);
            q -= 1;
        }
#pragma unroll
    for (int k = 0; k < 2; ++k)
        if (r > (int64_t)(2 * q)) {  // q too small: N - (q+1)^2 = r - 2q - 1
            r -= (int64_t)(2 * q + 1);
            q += 1;
        }
    *q_out = q;
    *r_out = (uint64_t)r;
    return r >= 0 && r <= (int64_t)(2 * q);
}

// floor(2^105 / M) for M in [2^52, 2^53), with r = 2^105 - q M in [0, M); false
// if the remainder could not be brought there. Seed: the float-float
// reciprocal g + t (g = RN(1/A) for the top 24 bits A of M, its exact residual
// 1 - g A from one FMA), good to ~2^-46; then one Newton step on the 64-bit
// residual.
__device__ __forceinline__ bool irecip_sig(uint64_t M, uint64_t* q_out, uint64_t* r_out)
{
    const float A = __uint2float_rn((uint32_t)(M >> 29)) * 0x1p29f;  // exact: top 24 bits of M
    const float B = __uint2float_rn((uint32_t)(M & ((1u << 29) - 1)));
    const float g = __frcp_rn(A);
    const float e = fmaf(-g, A, 1.0f);  // exact
    const float t = g * fmaf(-g, B, e);
    uint64_t q = float_to_scaled_u64(g, 105) + (int64_t)__float2int_rn(t * 0x1p105f);
    int64_t r = (int64_t)(0 - q * M);  // 2^105 - q M mod 2^64
    q += (int64_t)__float2int_rn(i64_to_float(r) * g);
    r = (int64_t)(0 - q * M);
#pragma unroll
    for (int k = 0; k < 2; ++k)
        if (r < 0) {
            r += (int64_t)M;
            q -= 1;
        }
#pragma unroll
    for (int k = 0; k < 2; ++k)
        if (r >= (int64_t)M) {
            r -= (int64_t)M;
            q += 1;
        }
    *q_out = q;
    *r_out = (uint64_t)r;
    return r >= 0 && r < (int64_t)M;
}

// CUDA's chain, the reference arithmetic of inv(sqrt(ss)^2)
__device__ __forceinline__ double weight_intrinsic(double ss)
{
    const double d = __dsqrt_rn(ss);
    return __drcp_rn(__dmul_rn(d, d));
}

// RN(1 / RN(RN(sqrt(ss))^2)) on the integer pipe; CUDA's chain outside the normal range
__device__ __forceinline__ double inv_dist2(double ss)
{
    const uint64_t B = (uint64_t)__double_as_longlong(ss);
    const int E = (int)(B >> 52);  // sign bit included: negative values fail the range test
    if (E < 1 || E > 2046) return weight_intrinsic(ss);
    // ss = m 2^t, m in [2^52, 2^53); make t even
    uint64_t m = (B & ((1ull << 52) - 1)) | (1ull << 52);
    int t = E - 1075;
    if (t & 1) {
        m <<= 1;
        t -= 1;
    }
    uint64_t q, r;
    bool ok = isqrt_sig(m, &q, &r);
    // d = dm 2^de, dm in [2^52, 2^53]
    uint64_t dm = q + (r > q ? 1 : 0);
    int de = (t - 52) / 2;
    if (dm == (1ull << 53)) {
        dm = 1ull << 52;
        de += 1;
    }
    // d^2 rounded to 53 bits, ties to even
    const U128 P = mul_u64(dm, dm);  // in [2^104, 2^106)
    int s = (P.hi >> 41) ? 53 : 52;
    uint64_t m2 = (P.hi << (64 - s)) | (P.lo >> s);
    const uint64_t rest = P.lo & ((1ull << s) - 1), half = 1ull << (s - 1);
    m2 += (rest > half || (rest == half && (m2 & 1))) ? 1 : 0;
    if (m2 == (1ull << 53)) {
        m2 = 1ull << 52;
        s += 1;
    }
    const int e2 = 2 * de + s;  // d^2 = m2 2^e2
    // 1 / d^2 = (2^105 / m2) 2^(-105 - e2)
    uint64_t wq, wr;
    ok &= irecip_sig(m2, &wq, &wr);
    uint64_t wm = wq + (2 * wr > m2 ? 1 : 0);
    int we = -105 - e2;
    if (wm >= (1ull << 53)) {  // m2 = 2^52: the quotient is exactly 2^53
        wm >>= 1;
        we += 1;
    }
    const int bd2 = e2 + 1075, bw = we + 1075;  // biased exponents of d^2 and w
    if (!ok || bd2 < 1 || bd2 > 2046 || bw < 1 || bw > 2046) return weight_intrinsic(ss);
    return __longlong_as_double((long long)(((uint64_t)bw << 52) | (wm & ((1ull << 52) - 1))));
}

}  // namespace jp
