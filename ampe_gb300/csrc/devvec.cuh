// Device vector kernels and deterministic reductions used by the stepper
// (the N_Vector operations of Sundials_SAMRAIVector.cc:106-205 and SAMRAI's
// RMS / WRMS norms).  Reductions are two-pass with a fixed block count and
// a fixed summation order, so repeated runs give bit-identical results.
#pragma once

#include "common.cuh"

namespace ampe {

// partial sums of the deterministic two-pass reductions: a fixed count (8
// per SM of a GB300), so that the summation order, and with it every
// reduced value, is the same on any device
constexpr int kRedBlocks = 1216;
constexpr int kRedThreads = 256;

template <class F>
__device__ __forceinline__ double block_sum(double v, double* sh)
{
   for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
   const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
   if (l == 0) sh[w] = v;
   __syncthreads();
   v = 0.0;
   if (w == 0) {
      v = l < (int)(blockDim.x >> 5) ? sh[l] : 0.0;
      for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
   }
   return v;
}

struct NoOp {};

// part[b] = sum over the block's grid-stride range of f(t)
template <class F>
__global__ void k_partial(long long n, F f, double* part)
{
   __shared__ double sh[32];
   double acc = 0.0;
#pragma unroll 4
   for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < n;
        t += (long long)gridDim.x * blockDim.x)
      acc += f(t);
   acc = block_sum<NoOp>(acc, sh);
   if (threadIdx.x == 0) part[blockIdx.x] = acc;
}

// as k_partial for FP32 terms: each thread sums its terms in FP32 with
// Kahan compensation (no FP64 instruction per element), the block and the
// finishing pass sum the per-thread results in FP64
template <class F>
__global__ void k_partial_f(long long n, F f, double* part)
{
   __shared__ double sh[32];
   float acc = 0.f, comp = 0.f;
#pragma unroll 4
   for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < n;
        t += (long long)gridDim.x * blockDim.x) {
      const float y = f(t) - comp;
      const float s = acc + y;
      comp = (s - acc) - y;
      acc = s;
   }
   const double a = block_sum<NoOp>((double)acc, sh);
   if (threadIdx.x == 0) part[blockIdx.x] = a;
}

static __global__ void k_finish(const double* part, int np, double* out, int slot)
{
   __shared__ double sh[32];
   double acc = 0.0;
   for (int t = threadIdx.x; t < np; t += blockDim.x) acc += part[t];
   acc = block_sum<NoOp>(acc, sh);
   if (threadIdx.x == 0) out[slot] = acc;
}

template <class F>
__global__ void k_map(long long n, F f)
{
   for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < n;
        t += (long long)gridDim.x * blockDim.x)
      f(t);
}

inline unsigned map_blocks(long long n)
{
   long long b = (n + 255) / 256;
   if (b > max_blocks()) b = max_blocks();
   return (unsigned)(b < 1 ? 1 : b);
}

template <class F>
inline int map(long long n, F f, cudaStream_t s)
{
   k_map<<<map_blocks(n), 256, 0, s>>>(n, f);
   return launch_status();
}

// Reduction helper owning the partials buffer and a pinned result slot.
struct Reducer {
   double* part = nullptr;  // device [kRedBlocks]
   double* dres = nullptr;  // device [16]
   double* hres = nullptr;  // pinned host [16]
   cudaStream_t s = nullptr;
   int init(cudaStream_t st)
   {
      s = st;
      if (cudaMalloc(&part, sizeof(double) * kRedBlocks) != cudaSuccess)
         return AMPE_ERR_CUDA;
      if (cudaMalloc(&dres, sizeof(double) * 16) != cudaSuccess)
         return AMPE_ERR_CUDA;
      if (cudaMallocHost(&hres, sizeof(double) * 16) != cudaSuccess)
         return AMPE_ERR_CUDA;
      return AMPE_OK;
   }
   void release()
   {
      if (part) cudaFree(part);
      if (dres) cudaFree(dres);
      if (hres) cudaFreeHost(hres);
      part = dres = hres = nullptr;
   }
   template <class F>
   void enqueue(long long n, F f, int slot)
   {
      long long nb = (n + kRedThreads - 1) / kRedThreads;
      int blocks = (int)(nb < kRedBlocks ? (nb < 1 ? 1 : nb) : kRedBlocks);
      k_partial<<<blocks, kRedThreads, 0, s>>>(n, f, part);
      k_finish<<<1, 1024, 0, s>>>(part, blocks, dres, slot);
      g_launches += 2;
   }
   // copy slots [0, nslots) to the host and wait
   const double* fetch(int nslots)
   {
      cudaMemcpyAsync(hres, dres, sizeof(double) * nslots,
                      cudaMemcpyDeviceToHost, s);
      cudaStreamSynchronize(s);
      return hres;
   }
   template <class F>
   double sum(long long n, F f)
   {
      enqueue(n, f, 0);
      return fetch(1)[0];
   }
   // sum of FP32 terms (k_partial_f), FP64 result
   template <class F>
   double sumf(long long n, F f)
   {
      long long nb = (n + kRedThreads - 1) / kRedThreads;
      int blocks = (int)(nb < kRedBlocks ? (nb < 1 ? 1 : nb) : kRedBlocks);
      k_partial_f<<<blocks, kRedThreads, 0, s>>>(n, f, part);
      k_finish<<<1, 1024, 0, s>>>(part, blocks, dres, 0);
      g_launches += 2;
      return fetch(1)[0];
   }
};

}  // namespace ampe
