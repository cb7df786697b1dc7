// FP64 <-> FP32 conversions by integer operations (the mixed path's sweeps
// and Krylov basis).
//
// GB300 runs FP64 arithmetic and the FP64<->FP32 conversion instructions on
// its FP64 pipe, at about 1.6 operations per SM and clock (FP32: about 119),
// so kernels that convert doubles in their inner loops spend their time
// there. These conversions give the instruction's result bit for bit (round
// to nearest even) with integer operations; the rare inputs outside the
// float normal range take the instruction out of line.
#ifndef FCG_FP_BITS_CUH
#define FCG_FP_BITS_CUH

#include <cuda_runtime.h>
#include <stdint.h>

namespace fcg {
namespace {  // every translation unit its own copy

// float -> double (exact for every input: zeros, subnormals, infinities
// and NaNs included)
__device__ __forceinline__ double f2d_bits(float f) {
    const uint32_t u = __float_as_uint(f), e = (u >> 23) & 0xffu, m = u & 0x7fffffu;
    const uint64_t sign = (uint64_t)(u & 0x80000000u) << 32;
    uint64_t bits;
    if (e == 255u) {
        bits = sign | 0x7ff0000000000000ull | ((uint64_t)m << 29);
    } else if (e != 0u) {
        bits = sign | ((uint64_t)(e + 896u) << 52) | ((uint64_t)m << 29);
    } else if (m == 0u) {
        bits = sign;
    } else {  // subnormal: m * 2^-149 with its top bit at position p
        const int p = 31 - __clz(m);
        bits = sign | ((uint64_t)(p + 874) << 52) | (((uint64_t)m << (52 - p)) & 0xfffffffffffffull);
    }
    return __longlong_as_double((long long)bits);
}

// the conversion instruction, out of line: only rare inputs take it
__device__ __noinline__ float d2f_rare(double d) { return (float)d; }

// double -> float, round to nearest even: integer operations for results in
// the normal float range (and zero), the instruction for the rest
__device__ __forceinline__ float d2f_bits(double d) {
    const uint32_t hi = (uint32_t)__double2hiint(d), lo = (uint32_t)__double2loint(d);
    const uint32_t e = (hi >> 20) & 0x7ffu;
    if (((hi & 0x7fffffffu) | lo) == 0u) return __uint_as_float(hi & 0x80000000u);
    if (e < 897u || e > 1150u) return d2f_rare(d);
    const uint32_t m = ((hi & 0xfffffu) << 3) | (lo >> 29), rest = lo & 0x1fffffffu;
    uint32_t f = (hi & 0x80000000u) | ((e - 896u) << 23) | m;
    f += (rest > 0x10000000u || (rest == 0x10000000u && (m & 1u))) ? 1u : 0u;  // a carry rounds into the exponent
    return __uint_as_float(f);
}

// double -> unevaluated FP32 pair (x + y): x holds the leading 24
// significant bits of d (truncated), y the next 23 (truncated), so x + y is
// within 2^-46 of d, relative. Integer operations and one exact FP32
// subtraction (the next 23 bits placed under a power of two, minus that
// power) for |d| in [2^-103, 2^128); zero and FP64 subnormals give (0, 0);
// the rest converts out of line.
__device__ __noinline__ float2 d2pair_rare(double d) {
    const float h = __double2float_rz(d);
    return make_float2(h, __double2float_rn(d - (double)h));
}

__device__ __forceinline__ float2 d2pair_bits(double d) {
    const uint32_t hi = (uint32_t)__double2hiint(d), lo = (uint32_t)__double2loint(d);
    const uint32_t e = (hi >> 20) & 0x7ffu;
    if (e - 920u > 230u) return e == 0u ? make_float2(0.0f, 0.0f) : d2pair_rare(d);
    const uint32_t sign = hi & 0x80000000u, eb = (e - 896u) << 23;
    const uint32_t fh = sign | eb | ((hi & 0xfffffu) << 3) | (lo >> 29);
    const uint32_t base = sign | (eb - (23u << 23));
    const float y = __fsub_rn(__uint_as_float(base | ((lo >> 6) & 0x7fffffu)), __uint_as_float(base));
    return make_float2(__uint_as_float(fh), y);
}

// pair -> double: x + y rounded once
__device__ __forceinline__ double pair2d(float2 p) { return __dadd_rn(f2d_bits(p.x), f2d_bits(p.y)); }

}  // namespace
}  // namespace fcg

#endif
