// FP32 <-> FP64 conversions on the integer pipe.
//
// On GB300 a hardware F2F conversion between float and double issues on the
// FP64 unit, which runs at a small fraction of the FP32 rate; a memory-bound
// kernel that converts every element can end up FP64-bound.  These versions
// assemble the IEEE-754 bit patterns with integer operations instead:
//   f2d: exact for every finite float; subnormal floats become signed zero.
//   d2f: round-to-nearest-even for results in the normal float range;
//        |x| < 2^-126 becomes signed zero, |x| >= 2^128 becomes +-inf,
//        NaN stays NaN.
// Host versions (same arithmetic, memcpy bit casts) exist for the unit test.
#pragma once

#include <stdint.h>
#include <string.h>

#if defined(__CUDACC__)
#define AMPE_BC_HD __host__ __device__ __forceinline__
#else
#define AMPE_BC_HD inline
#endif

namespace ampe {

AMPE_BC_HD uint32_t bc_float_bits(float x)
{
#ifdef __CUDA_ARCH__
   return __float_as_uint(x);
#else
   uint32_t u;
   memcpy(&u, &x, 4);
   return u;
#endif
}

AMPE_BC_HD float bc_bits_float(uint32_t u)
{
#ifdef __CUDA_ARCH__
   return __uint_as_float(u);
#else
   float x;
   memcpy(&x, &u, 4);
   return x;
#endif
}

AMPE_BC_HD void bc_double_words(double x, uint32_t& hi, uint32_t& lo)
{
#ifdef __CUDA_ARCH__
   hi = (uint32_t)__double2hiint(x);
   lo = (uint32_t)__double2loint(x);
#else
   uint64_t u;
   memcpy(&u, &x, 8);
   hi = (uint32_t)(u >> 32);
   lo = (uint32_t)u;
#endif
}

AMPE_BC_HD double bc_words_double(uint32_t hi, uint32_t lo)
{
#ifdef __CUDA_ARCH__
   return __hiloint2double((int)hi, (int)lo);
#else
   const uint64_t u = ((uint64_t)hi << 32) | lo;
   double x;
   memcpy(&x, &u, 8);
   return x;
#endif
}

// float -> double
AMPE_BC_HD double f2d(float x)
{
   const uint32_t u = bc_float_bits(x);
   const uint32_t s = u & 0x80000000u;
   const uint32_t e = (u >> 23) & 0xffu;
   const uint32_t m = u & 0x7fffffu;
   if (e == 0) return bc_words_double(s, 0u);
   const uint32_t de = e == 0xffu ? 0x7ffu : e + 896u;  // rebias 127 -> 1023
   return bc_words_double(s | (de << 20) | (m >> 3), m << 29);
}

// double -> float, round to nearest even
AMPE_BC_HD float d2f(double x)
{
   uint32_t hi, lo;
   bc_double_words(x, hi, lo);
   const uint32_t s = hi & 0x80000000u;
   const uint32_t ah = hi & 0x7fffffffu;
   const int e = (int)(ah >> 20);
   if (e >= 1151) {  // |x| >= 2^128, inf or NaN
      if (e == 2047 && ((ah & 0xfffffu) | lo)) return bc_bits_float(s | 0x7fc00000u);
      return bc_bits_float(s | 0x7f800000u);
   }
   if (e < 897) return bc_bits_float(s);  // below the normal float range
   uint32_t f = ((uint32_t)(e - 896) << 23) | ((ah & 0xfffffu) << 3) | (lo >> 29);
   const uint32_t rem = lo & 0x1fffffffu;  // the 29 dropped bits
   if (rem > 0x10000000u || (rem == 0x10000000u && (f & 1u))) f += 1u;
   return bc_bits_float(s | f);
}

}  // namespace ampe
