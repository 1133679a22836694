// exact.cuh — order-independent sums of non-negative doubles.
//
// Each addend is truncated to a multiple of 2^-64 and added into a 128-bit unsigned
// fixed-point accumulator (64 integer bits, 64 fraction bits). Integer addition is
// associative, so a sum is the same bits whatever the order of the addends, the grid, the
// threads or the reduction tree; the total converts back to the nearest double (ties to
// even). The truncation error is below n * 2^-64 for n addends, far under the rounding
// error of a sequential double sum of the same values. Used by the Longstaff-Schwartz
// regressions, whose exercise decisions must not depend on the launch shape.
#pragma once

#include <cstdint>
#include <cstring>
#include <cmath>

#ifdef __CUDACC__
#define FX_HD __host__ __device__ __forceinline__
#else
#define FX_HD inline
#endif

struct Fx128 {
    uint64_t lo, hi;
};

// largest addend accepted (2^36): with fewer than 2^27 addends the integer part stays
// below 2^63
constexpr double FX_MAX_ADDEND = 68719476736.0;

FX_HD void fx_add(Fx128& a, uint64_t lo, uint64_t hi)
{
    a.lo += lo;
    a.hi += hi + (a.lo < lo ? 1u : 0u);
}

FX_HD void fx_add(Fx128& a, const Fx128& b) { fx_add(a, b.lo, b.hi); }

FX_HD uint64_t fx_bits(double x)
{
#ifdef __CUDA_ARCH__
    return (uint64_t)__double_as_longlong(x);
#else
    uint64_t b;
    std::memcpy(&b, &x, sizeof b);
    return b;
#endif
}

// add x (0 <= x < 2^63, finite) truncated to a multiple of 2^-64
FX_HD void fx_add(Fx128& a, double x)
{
    const uint64_t b = fx_bits(x);
    const int ex = (int)(b >> 52) & 0x7ff;
    if (ex == 0) return; // zero or subnormal: below 2^-64
    const uint64_t mant = (b & 0xFFFFFFFFFFFFFull) | (1ull << 52);
    // x = mant * 2^(ex - 1075); in units of 2^-64 that is mant << (ex - 1011)
    const int sh = ex - 1011;
    uint64_t lo, hi;
    if (sh >= 64) {
        lo = 0;
        hi = mant << (sh - 64);
    } else if (sh > 0) {
        lo = mant << sh;
        hi = mant >> (64 - sh);
    } else if (sh > -53) {
        lo = mant >> (-sh);
        hi = 0;
    } else {
        return;
    }
    fx_add(a, lo, hi);
}

// add x when 0 <= x < FX_MAX_ADDEND, else set bad (negative, too large, inf or NaN):
// integer tests on the bit pattern only
FX_HD void fx_add_checked(Fx128& a, double x, bool& bad)
{
    const uint64_t b = fx_bits(x);
    if (b >= 0x4230000000000000ull) { // 2^36, or the sign bit set
        if ((b << 1) != 0) bad = true; // -0.0 adds nothing
        return;
    }
    fx_add(a, x);
}

FX_HD int fx_clz64(uint64_t v)
{
#ifdef __CUDA_ARCH__
    return __clzll((long long)v);
#else
    return v ? __builtin_clzll(v) : 64;
#endif
}

FX_HD double fx_u64_to_double(uint64_t v)
{
#ifdef __CUDA_ARCH__
    return __ull2double_rn(v);
#else
    return (double)v; // round to nearest under the default rounding mode
#endif
}

// d 2^k for d = 0 or d >= 1, -64 <= k <= 0: exact (the result is a normal double)
FX_HD double fx_scale(double d, int k)
{
#ifdef __CUDA_ARCH__
    const long long b = __double_as_longlong(d);
    return b == 0 ? 0.0 : __longlong_as_double(b + ((long long)k << 52));
#else
    return std::ldexp(d, k);
#endif
}

// the nearest double to the fixed-point value (hi * 2^64 + lo) * 2^-64
FX_HD double fx_to_double(const Fx128& a)
{
    if (a.hi == 0) return fx_scale(fx_u64_to_double(a.lo), -64);
    // keep the top 64 significant bits and fold the rest into a sticky bit, which sits
    // 11 bits below the double's rounding position: rounding the 64 bits then rounds the
    // 128-bit value correctly, ties included
    const int s = 64 - fx_clz64(a.hi); // right shift that leaves 64 bits, 1..64
    uint64_t top, rest;
    if (s == 64) {
        top = a.hi;
        rest = a.lo;
    } else {
        top = (a.hi << (64 - s)) | (a.lo >> s);
        rest = a.lo & ((1ull << s) - 1);
    }
    top |= rest ? 1u : 0u;
    return fx_scale(fx_u64_to_double(top), s - 64);
}
