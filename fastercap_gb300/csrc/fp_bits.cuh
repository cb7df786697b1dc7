// FP64 <-> FP32 conversions by integer operations (the mixed path's sweeps).
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

}  // namespace
}  // namespace fcg

#endif
