// Division of 31-bit indices by an invariant divisor with one high multiply
// (Granlund & Montgomery, "Division by invariant integers using
// multiplication", PLDI 1994): with s = ceil(log2 d) and
// m = 2^32 (2^s - d) / d + 1, n / d = (umulhi(n, m) + n) >> s for n < 2^31.
// Plain C++ on the host (tested there), __umulhi on the device.
#pragma once

#if defined(__CUDACC__)
#define AMPE_FD_HD __host__ __device__ __forceinline__
#else
#define AMPE_FD_HD inline
#endif

namespace ampe {

struct FastDiv {
   unsigned d = 1, m = 1, s = 0;
   FastDiv() = default;
   explicit FastDiv(unsigned dd) : d(dd < 1 ? 1 : dd)
   {
      s = 0;
      while (s < 31 && (1u << s) < d) s++;
      const unsigned long long one = 1;
      m = (unsigned)(((one << 32) * ((one << s) - d)) / d + 1);
   }
   AMPE_FD_HD unsigned div(unsigned n) const
   {
#ifdef __CUDA_ARCH__
      const unsigned t = __umulhi(n, m);
#else
      const unsigned t = (unsigned)(((unsigned long long)n * m) >> 32);
#endif
      return (t + n) >> s;
   }
};

}  // namespace ampe
