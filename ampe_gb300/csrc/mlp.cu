// Surrogate MLP for the KKS initial guess: (phi, c, T) -> logit(cL), logit(cS)
// 3 -> 64 -> 64 -> 64 -> 2, SiLU, BF16 weights, FP32 accumulation.
//
// Inference (k_mlp_infer_tc) runs on the fifth-generation tensor cores:
// 128 cells per tile, tcgen05.mma (kind::f16, BF16 x BF16 -> FP32) issued by
// one thread from shared-memory operands in the canonical no-swizzle K-major
// layout, accumulators in tensor memory read back with tcgen05.ld; the bias
// + SiLU epilogue runs on packed bf16x2 and writes the next layer's operand.
// Training runs on the tensor cores too: k_mlp_train_tc does the forward and
// backward products of one 128-sample tile per CTA with BF16 operands and
// FP32 accumulators, k_mlp_reduce_adam sums the tiles' gradients and takes
// the FP32 Adam step of the master weights.
//
// Labels come from the FP64 KKS Newton (kks_newton), started from (c, c).
#include <cuda_bf16.h>

#include <cmath>
#include <cstring>
#include <vector>

#include "common.cuh"
#include "mlp.cuh"

namespace ampe {

// ---------------------------------------------------------------------------
// canonical no-swizzle K-major operand layout: core matrices of 8 rows x 16
// bytes (8 BF16 along K) stored contiguously; core (g, kc) at
// ((g * (Kt / 8)) + kc) * 128 bytes.  LBO (K direction) = 128 B,
// SBO (row-group direction) = Kt * 16 B.
// ---------------------------------------------------------------------------
__host__ __device__ inline int canon_off(int r, int k, int Kt)
{
   return (((r >> 3) * (Kt >> 3) + (k >> 3)) << 7) + ((r & 7) << 4) + ((k & 7) << 1);
}

// ---------------------------------------------------------------------------
// deterministic sample generator (counter-based hash)
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint32_t hash32(uint32_t x)
{
   x ^= x >> 16;
   x *= 0x7feb352dU;
   x ^= x >> 15;
   x *= 0x846ca68bU;
   x ^= x >> 16;
   return x;
}

__device__ __forceinline__ double u01(uint32_t seed, uint32_t i, uint32_t s)
{
   const uint32_t h = hash32(seed * 0x9e3779b9U ^ hash32(i * 3u + s));
   return ((double)h + 0.5) * (1.0 / 4294967296.0);
}

__device__ __forceinline__ void encode_inputs(const MlpNorm& nz, double phi,
                                              double c, double T, float* x)
{
   x[0] = (float)(2.0 * phi - 1.0);
   x[1] = (float)(2.0 * c - 1.0);
   x[2] = (float)((T - nz.t_mid) * nz.t_inv_half);
}

// the same encoding in FP32 for the inference kernels: no FP64 instruction
// per cell (the conversions of phi and c run on the integer pipe)
struct NormF {
   float t_mid, t_inv_half, T0, gdx;
   int mode;
};
__device__ __forceinline__ NormF norm_f(const MlpNorm& nz, const ampe_model_t& m)
{
   return NormF{(float)nz.t_mid, (float)nz.t_inv_half, (float)m.T0, (float)(m.gradT * m.dx[0]),
                m.temp_mode};
}
__device__ __forceinline__ void encode_inputs_f(const NormF& nf, const Grid& g,
                                                const double* tfield, double phi, double c,
                                                int i, int j, int k, float* x)
{
   float T = nf.T0;
   if (nf.mode == AMPE_TEMP_GRADIENT) {
      T = nf.T0 + nf.gdx * ((float)i + 0.5f);
   } else if (nf.mode == AMPE_TEMP_FIELD) {
      T = d2f(tfield[g.c(i, j, k)]);
   }
   x[0] = 2.f * d2f(phi) - 1.f;
   x[1] = 2.f * d2f(c) - 1.f;
   x[2] = (T - nf.t_mid) * nf.t_inv_half;
}

__device__ __forceinline__ float logit_clip(double c)
{
   double l = log(c / (1.0 - c));
   if (l > 14.0) l = 14.0;
   if (l < -14.0) l = -14.0;
   return (float)l;
}

// samples: x [n][4] (3 used), target [n][2] logits.  T uniform in [tlo, thi]
__global__ void k_gen_samples(ampe_model_t m, MlpNorm nz, uint32_t seed,
                              long long n, double tlo, double thi, double clo,
                              double chi, float* x, float* target,
                              unsigned long long* fails)
{
   unsigned long long nf = 0;
   for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < n;
        t += (long long)gridDim.x * blockDim.x) {
      const double phi = u01(seed, (uint32_t)t, 0);
      const double c = clo + (chi - clo) * u01(seed, (uint32_t)t, 1);
      const double T = tlo + (thi - tlo) * u01(seed, (uint32_t)t, 2);
      const ThermoCoef th = thermo_coef(m, T);
      const double h = interp_func(phi, m.conc_interp);
      double xs[2] = {c, c};
      if (kks_newton(th, h, c, xs, 100, 1e-12) < 0) {
         nf++;
         xs[0] = c;
         xs[1] = c;
      }
      float in[3];
      encode_inputs(nz, phi, c, T, in);
      x[4 * t + 0] = in[0];
      x[4 * t + 1] = in[1];
      x[4 * t + 2] = in[2];
      x[4 * t + 3] = 0.f;
      target[2 * t + 0] = logit_clip(xs[0]);
      target[2 * t + 1] = logit_clip(xs[1]);
   }
   if (fails && nf) atomicAdd(fails, nf);
}

// ---------------------------------------------------------------------------
// training kernels (FP32, weights rounded to BF16 in the forward pass)
// layer l: Z = X W^T + b, A = silu(Z) (last layer: identity)
// W stored row-major [out][in] FP32 (master copy)
// ---------------------------------------------------------------------------
__device__ __forceinline__ float bf16r(float w)
{
   return __bfloat162float(__float2bfloat16_rn(w));
}

__device__ __forceinline__ float silu(float z) { return z / (1.f + expf(-z)); }

__device__ __forceinline__ float dsilu(float z)
{
   const float s = 1.f / (1.f + expf(-z));
   return s * (1.f + z * (1.f - s));
}

// BF16 canonical copies for the tensor-core kernels: the forward operands
// W_l [out][in] (K = in) and, for the backward products dX = dZ W, W_l^T
// [in][out] (K = out) of layers 2-4
__global__ void k_pack_weights(const float* W1, const float* W2,
                               const float* W3, const float* W4,
                               __nv_bfloat16* p1, __nv_bfloat16* p2,
                               __nv_bfloat16* p3, __nv_bfloat16* p4,
                               __nv_bfloat16* p4t, __nv_bfloat16* p3t, __nv_bfloat16* p2t)
{
   const int t = blockIdx.x * blockDim.x + threadIdx.x;
   // W1: 64 x 16 (K padded from 3)
   if (t < 64 * 16) {
      const int r = t / 16, k = t % 16;
      const float v = k < 3 ? W1[r * 3 + k] : 0.f;
      p1[canon_off(r, k, 16) / 2] = __float2bfloat16_rn(v);
   }
   if (t < 64 * 64) {
      const int r = t / 64, k = t % 64;
      p2[canon_off(r, k, 64) / 2] = __float2bfloat16_rn(W2[t]);
      p3[canon_off(r, k, 64) / 2] = __float2bfloat16_rn(W3[t]);
   }
   // W4: 16 x 64 (N padded from 2)
   if (t < 16 * 64) {
      const int r = t / 64, k = t % 64;
      const float v = r < 2 ? W4[r * 64 + k] : 0.f;
      p4[canon_off(r, k, 64) / 2] = __float2bfloat16_rn(v);
   }
   // W4^T: 64 (in) x 16 (out padded from 2)
   if (t < 64 * 16) {
      const int r = t / 16, k = t % 16;
      const float v = k < 2 ? W4[k * 64 + r] : 0.f;
      p4t[canon_off(r, k, 16) / 2] = __float2bfloat16_rn(v);
   }
   // W3^T, W2^T: 64 (in) x 64 (out)
   if (t < 64 * 64) {
      const int r = t / 64, k = t % 64;
      p3t[canon_off(r, k, 64) / 2] = __float2bfloat16_rn(W3[k * 64 + r]);
      p2t[canon_off(r, k, 64) / 2] = __float2bfloat16_rn(W2[k * 64 + r]);
   }
}

// ---------------------------------------------------------------------------
// tensor-core inference
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint32_t smem_u32(const void* p)
{
   return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ uint64_t umma_desc(uint32_t saddr, uint32_t lbo,
                                              uint32_t sbo)
{
   uint64_t d = 0;
   d |= (uint64_t)((saddr >> 4) & 0x3FFF);
   d |= (uint64_t)((lbo >> 4) & 0x3FFF) << 16;
   d |= (uint64_t)((sbo >> 4) & 0x3FFF) << 32;
   d |= (uint64_t)1 << 46;  // descriptor version for tcgen05
   // base offset 0, absolute LBO mode 0, layout type 0 = no swizzle
   return d;
}

// BF16 x BF16 -> FP32, K-major A and B, M = 128
__host__ __device__ constexpr uint32_t umma_idesc(int n)
{
   return (1u << 4)            // D format FP32
          | (1u << 7)          // A format BF16
          | (1u << 10)         // B format BF16
          | ((uint32_t)(n >> 3) << 17) | ((uint32_t)(128 >> 4) << 24);
}

__device__ __forceinline__ void umma_f16(uint32_t tmem_d, uint64_t adesc,
                                         uint64_t bdesc, uint32_t idesc,
                                         uint32_t accumulate)
{
   asm volatile(
       "{\n\t.reg .pred p;\n\t"
       "setp.ne.b32 p, %4, 0;\n\t"
       "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(tmem_d),
       "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate));
}

__device__ __forceinline__ void umma_commit(uint32_t mbar)
{
   asm volatile(
       "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(mbar)
       : "memory");
}

__device__ __forceinline__ void mbar_init(uint32_t mbar, int count)
{
   asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(mbar), "r"(count));
}

// default bound of the mbarrier waits (try_wait polls)
constexpr int kWaitLimit = 1 << 22;

// bounded wait on an mbarrier phase; returns false after `limit` polls
__device__ __forceinline__ bool mbar_wait(uint32_t mbar, uint32_t parity, int limit)
{
   for (int it = 0; it < limit; it++) {
      uint32_t done;
      asm volatile(
          "{\n\t.reg .pred p;\n\t"
          "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
          "selp.u32 %0, 1, 0, p;\n\t}\n"
          : "=r"(done)
          : "r"(mbar), "r"(parity)
          : "memory");
      if (done) return true;
   }
   return false;
}

__device__ __forceinline__ void tc_fence_before()
{
   asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void tc_fence_after()
{
   asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void fence_async_smem()
{
   asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

#define TMEM_LD_X16(taddr, r)                                                     \
   asm volatile(                                                                 \
       "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11," \
       "%12,%13,%14,%15}, [%16];"                                                \
       : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]),  \
         "=r"(r[6]), "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]),           \
         "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])        \
       : "r"(taddr))

__device__ __forceinline__ void tmem_wait_ld()
{
   asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
}

__device__ __forceinline__ uint32_t silu_bf16x2(float a, float b)
{
   // silu(x) = x (1/2 + tanh(x/2)/2) on packed bf16x2
   __nv_bfloat162 x = __floats2bfloat162_rn(a, b);
   const __nv_bfloat162 half = __floats2bfloat162_rn(0.5f, 0.5f);
   __nv_bfloat162 h = __hmul2(x, half);
   uint32_t hu = *reinterpret_cast<uint32_t*>(&h), tu;
   asm("tanh.approx.bf16x2 %0, %1;" : "=r"(tu) : "r"(hu));
   __nv_bfloat162 t = *reinterpret_cast<__nv_bfloat162*>(&tu);
   __nv_bfloat162 s = __hfma2(t, half, half);
   __nv_bfloat162 y = __hmul2(x, s);
   return *reinterpret_cast<uint32_t*>(&y);
}

struct __align__(128) MlpSmem {
   __nv_bfloat16 w1[64 * 16];
   __nv_bfloat16 w2[64 * 64];
   __nv_bfloat16 w3[64 * 64];
   __nv_bfloat16 w4[16 * 64];
   __nv_bfloat16 x0[128 * 16];
   __nv_bfloat16 act[128 * 64];
   float b[3 * 64 + 2];
   unsigned long long mbar;
   uint32_t tmem;
};

constexpr int kMlpTmemCols = 64;

// one 64-column layer epilogue: bias + SiLU -> act (canonical, Kt = 64)
__device__ __forceinline__ void epilogue64(uint32_t taddr, const float* bias,
                                           __nv_bfloat16* act, int row)
{
#pragma unroll
   for (int q = 0; q < 4; q++) {
      uint32_t r[16];
      TMEM_LD_X16(taddr + 16 * q, r);
      tmem_wait_ld();
#pragma unroll
      for (int h = 0; h < 2; h++) {
         uint4 pk;
         const int base = 16 * q + 8 * h;
         pk.x = silu_bf16x2(__uint_as_float(r[8 * h + 0]) + bias[base + 0],
                            __uint_as_float(r[8 * h + 1]) + bias[base + 1]);
         pk.y = silu_bf16x2(__uint_as_float(r[8 * h + 2]) + bias[base + 2],
                            __uint_as_float(r[8 * h + 3]) + bias[base + 3]);
         pk.z = silu_bf16x2(__uint_as_float(r[8 * h + 4]) + bias[base + 4],
                            __uint_as_float(r[8 * h + 5]) + bias[base + 5]);
         pk.w = silu_bf16x2(__uint_as_float(r[8 * h + 6]) + bias[base + 6],
                            __uint_as_float(r[8 * h + 7]) + bias[base + 7]);
         *reinterpret_cast<uint4*>(reinterpret_cast<char*>(act) +
                                   canon_off(row, base, 64)) = pk;
      }
   }
}

// guess_l / guess_s for the interior cells of the grid (interior index t).
// wait_limit bounds every mbarrier wait; skip_issue (a test of that error
// path) makes the issuing thread commit nothing, so the first wait runs out
// with no MMA in flight, the error flag is set and the tensor memory freed.
__global__ void __launch_bounds__(128) k_mlp_infer_tc(
    ampe_model_t m, Grid g, MlpNorm nz, const __nv_bfloat16* wpk,
    const float* bias, const double* phi, const double* conc,
    const double* tfield, float* guess_l, float* guess_s, int* err, int wait_limit,
    int skip_issue)
{
   extern __shared__ __align__(1024) unsigned char smraw[];
   MlpSmem& S = *reinterpret_cast<MlpSmem*>(smraw);
   const int tid = threadIdx.x, warp = tid >> 5;
   // stage weights (BF16 canonical, packed back to back) and biases
   {
      const uint4* src = reinterpret_cast<const uint4*>(wpk);
      uint4* dst = reinterpret_cast<uint4*>(S.w1);
      const int n16 = (int)((sizeof(S.w1) + sizeof(S.w2) + sizeof(S.w3) + sizeof(S.w4)) / 16);
      for (int i = tid; i < n16; i += blockDim.x) dst[i] = src[i];
      for (int i = tid; i < 3 * 64 + 2; i += blockDim.x) S.b[i] = bias[i];
      // zero the padded K columns of x0 once (only k < 3 are rewritten)
      for (int i = tid; i < (int)(sizeof(S.x0) / 16); i += blockDim.x)
         reinterpret_cast<uint4*>(S.x0)[i] = make_uint4(0, 0, 0, 0);
   }
   const uint32_t mbar = smem_u32(&S.mbar);
   if (tid == 0) mbar_init(mbar, 1);
   if (warp == 0) {
      asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                       smem_u32(&S.tmem)),
                   "r"(kMlpTmemCols));
      asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
   }
   asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
   tc_fence_before();
   __syncthreads();
   tc_fence_after();
   const uint32_t tmem = S.tmem;
   const uint32_t t_row = tmem + ((uint32_t)(warp * 32) << 16);
   const uint32_t a0 = smem_u32(S.x0), aact = smem_u32(S.act);
   const uint32_t w1 = smem_u32(S.w1), w2 = smem_u32(S.w2), w3 = smem_u32(S.w3),
                  w4 = smem_u32(S.w4);
   uint32_t phase = 0;
   bool ok = true;
   const long long N = g.cells();
   const long long ntiles = (N + 127) / 128;
   const NormF nfl = norm_f(nz, m);
   for (long long tile = blockIdx.x; tile < ntiles && ok; tile += gridDim.x) {
      const long long row = tile * 128 + tid;
      const long long t = row < N ? row : -1;
      // ---- inputs ----
      float in[3] = {0.f, 0.f, 0.f};
      if (t >= 0) {
         int i, j, k;
         g.ijk(t, i, j, k);
         const long long c = g.c(i, j, k);
         encode_inputs_f(nfl, g, tfield, phi[c], conc[c], i, j, k, in);
      }
      {
         __nv_bfloat162 p01 = __floats2bfloat162_rn(in[0], in[1]);
         __nv_bfloat162 p2 = __floats2bfloat162_rn(in[2], 0.f);
         uint2 v;
         v.x = *reinterpret_cast<uint32_t*>(&p01);
         v.y = *reinterpret_cast<uint32_t*>(&p2);
         *reinterpret_cast<uint2*>(reinterpret_cast<char*>(S.x0) + canon_off(tid, 0, 16)) = v;
      }
      fence_async_smem();
      tc_fence_before();
      __syncthreads();
      // ---- layer 1: [128 x 16] x [64 x 16]^T ----
      if (tid == 0 && !skip_issue) {
         tc_fence_after();
         umma_f16(tmem, umma_desc(a0, 128, 256), umma_desc(w1, 128, 256), umma_idesc(64), 0);
         umma_commit(mbar);
      }
      ok = __syncthreads_and(mbar_wait(mbar, phase, wait_limit));
      if (!ok) break;
      phase ^= 1;
      tc_fence_after();
      epilogue64(t_row, S.b, S.act, tid);
      // ---- layers 2, 3: [128 x 64] x [64 x 64]^T ----
      for (int layer = 0; layer < 2 && ok; layer++) {
         fence_async_smem();
         tc_fence_before();
         __syncthreads();
         if (tid == 0 && !skip_issue) {
            tc_fence_after();
            const uint32_t wb = layer == 0 ? w2 : w3;
#pragma unroll
            for (int s = 0; s < 4; s++)
               umma_f16(tmem, umma_desc(aact + 256 * s, 128, 1024),
                        umma_desc(wb + 256 * s, 128, 1024), umma_idesc(64), s > 0);
            umma_commit(mbar);
         }
         ok = __syncthreads_and(mbar_wait(mbar, phase, wait_limit));
         if (!ok) break;
         phase ^= 1;
         tc_fence_after();
         // the layer's input buffer is free again: the MMAs have completed
         epilogue64(t_row, S.b + 64 * (layer + 1), S.act, tid);
      }
      if (!ok) break;
      // ---- layer 4: [128 x 64] x [16 x 64]^T (2 outputs used) ----
      fence_async_smem();
      tc_fence_before();
      __syncthreads();
      if (tid == 0 && !skip_issue) {
         tc_fence_after();
#pragma unroll
         for (int s = 0; s < 4; s++)
            umma_f16(tmem, umma_desc(aact + 256 * s, 128, 1024),
                     umma_desc(w4 + 256 * s, 128, 1024), umma_idesc(16), s > 0);
         umma_commit(mbar);
      }
      ok = __syncthreads_and(mbar_wait(mbar, phase, wait_limit));
      if (!ok) break;
      phase ^= 1;
      tc_fence_after();
      uint32_t r[16];
      TMEM_LD_X16(t_row, r);
      tmem_wait_ld();
      if (t >= 0) {
         const float y0 = __uint_as_float(r[0]) + S.b[192];
         const float y1 = __uint_as_float(r[1]) + S.b[193];
         guess_l[t] = 1.f / (1.f + __expf(-y0));
         guess_s[t] = 1.f / (1.f + __expf(-y1));
      }
      tc_fence_before();
      __syncthreads();  // TMEM and x0 reused by the next tile
   }
   if (!ok) {
      // a commit did not arrive in time: flag it, give the MMAs in flight
      // one more bounded wait, then release the tensor memory
      if (tid == 0 && err) atomicExch(err, 1);
      mbar_wait(mbar, phase, wait_limit);
   }
   tc_fence_before();
   __syncthreads();
   if (warp == 0) {
      tc_fence_after();
      asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem),
                   "r"(kMlpTmemCols));
   }
}

// ---------------------------------------------------------------------------
// tensor-core training step: forward and backward of one 128-sample tile per
// CTA on tcgen05 (BF16 operands, FP32 accumulators in tensor memory)
//
// Layer l: Z = X W^T + b, A = silu(Z) (identity for the last layer); loss
// 1/2 mean over samples of the squared logit errors.  Backward, per layer:
//   dW_l (| db_l) = dZ_l^T [X_l | 1]   M = 128 (out padded), N = in + ones
//                                     column (80, or 16 for layer 1),
//                                     K = 128 samples;
//   dX_{l-1} = dZ_l W_l                M = 128 samples, N = in, K = out;
//   dZ_{l-1} = dX_{l-1} silu'(Z_{l-1}) (silu' kept in FP32 in tensor memory).
// Every operand is stored K-major in the canonical no-swizzle layout, so the
// backward products read transposed copies written by the forward epilogue
// (X_l^T) and by the packing kernel (W_l^T).  Each CTA writes its tile's
// weight and bias gradients as one partial; k_mlp_reduce_adam sums the
// partials in a fixed order, so a training step is deterministic.
// ---------------------------------------------------------------------------
struct __align__(128) TrainSmem {
   // packed weights, in the order the packing kernel writes them
   __nv_bfloat16 w1[64 * 16];
   __nv_bfloat16 w2[64 * 64];
   __nv_bfloat16 w3[64 * 64];
   __nv_bfloat16 w4[16 * 64];
   __nv_bfloat16 w4t[64 * 16];  // [in][out padded to 16]
   __nv_bfloat16 w3t[64 * 64];  // [in][out]
   __nv_bfloat16 w2t[64 * 64];
   __nv_bfloat16 x0[128 * 16];    // inputs, K-major (K = 16: 3 used)
   __nv_bfloat16 act[128 * 64];   // A operand of the next forward layer
   __nv_bfloat16 x0t[16 * 128];   // [feature | ones | 0][sample]
   __nv_bfloat16 at[3][80 * 128]; // [feature 64 | ones | 0 x 15][sample]
   __nv_bfloat16 dzt[128 * 128];  // [out, rows >= out zero][sample]
   __nv_bfloat16 dzn[128 * 64];   // [sample][out] (K = 64, or 16 for layer 4)
   float b[3 * 64 + 2];
   float red[4];
   unsigned long long mbar;
   uint32_t tmem;
};

constexpr int kTrainTmemCols = 512;  // [0,64) Z / dX, [128,208) dW, [256,448) silu'

#define TMEM_ST_X16(taddr, r)                                                       \
   asm volatile(                                                                   \
       "tcgen05.st.sync.aligned.32x32b.x16.b32 [%0], {%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11," \
       "%12,%13,%14,%15,%16};" ::"r"(taddr),                                        \
       "r"(r[0]), "r"(r[1]), "r"(r[2]), "r"(r[3]), "r"(r[4]), "r"(r[5]), "r"(r[6]),  \
       "r"(r[7]), "r"(r[8]), "r"(r[9]), "r"(r[10]), "r"(r[11]), "r"(r[12]),         \
       "r"(r[13]), "r"(r[14]), "r"(r[15]))

__device__ __forceinline__ void tmem_wait_st()
{
   asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory");
}

__device__ __forceinline__ float silu_f(float z) { return z / (1.f + __expf(-z)); }
__device__ __forceinline__ float dsilu_f(float z)
{
   const float s = 1.f / (1.f + __expf(-z));
   return s * (1.f + z * (1.f - s));
}

__device__ __forceinline__ void st_bf16(__nv_bfloat16* base, int byte_off, float v)
{
   *reinterpret_cast<__nv_bfloat16*>(reinterpret_cast<char*>(base) + byte_off) =
       __float2bfloat16_rn(v);
}

// 8 consecutive K values of row `row` (K-major canonical, K-tile Kt) as bf16
__device__ __forceinline__ void st_bf16x8(__nv_bfloat16* base, int row, int k0, int Kt,
                                          const float* v)
{
   uint4 pk;
   __nv_bfloat162 p;
   p = __floats2bfloat162_rn(v[0], v[1]);
   pk.x = *reinterpret_cast<uint32_t*>(&p);
   p = __floats2bfloat162_rn(v[2], v[3]);
   pk.y = *reinterpret_cast<uint32_t*>(&p);
   p = __floats2bfloat162_rn(v[4], v[5]);
   pk.z = *reinterpret_cast<uint32_t*>(&p);
   p = __floats2bfloat162_rn(v[6], v[7]);
   pk.w = *reinterpret_cast<uint32_t*>(&p);
   *reinterpret_cast<uint4*>(reinterpret_cast<char*>(base) + canon_off(row, k0, Kt)) = pk;
}

// partial gradient of one CTA: [W0 b0 W1 b1 W2 b2 W3 b3] as in the master
// parameter vector; loss partial in part_loss[blockIdx.x]
__global__ void __launch_bounds__(128, 1) k_mlp_train_tc(
    const __nv_bfloat16* wpk, const float* bias, const float* x, const float* target, int B,
    float* partials, int npar, float* part_loss, int* err, int wait_limit, int skip_issue)
{
   extern __shared__ __align__(1024) unsigned char smraw[];
   TrainSmem& S = *reinterpret_cast<TrainSmem*>(smraw);
   const int tid = threadIdx.x, warp = tid >> 5;
   const int row = tid;
   const int s = blockIdx.x * 128 + row;
   const bool valid = s < B;
   const float invB = 1.f / (float)B;
   {
      const uint4* src = reinterpret_cast<const uint4*>(wpk);
      uint4* dst = reinterpret_cast<uint4*>(S.w1);
      const int n16 = (int)((sizeof(S.w1) + sizeof(S.w2) + sizeof(S.w3) + sizeof(S.w4) +
                             sizeof(S.w4t) + sizeof(S.w3t) + sizeof(S.w2t)) / 16);
      for (int i = tid; i < n16; i += blockDim.x) dst[i] = src[i];
      for (int i = tid; i < 3 * 64 + 2; i += blockDim.x) S.b[i] = bias[i];
      // zero x0, the transposed inputs and dZ^T (their padding stays zero)
      const uint4 z = make_uint4(0, 0, 0, 0);
      for (int i = tid; i < (int)(sizeof(S.x0) / 16); i += blockDim.x)
         reinterpret_cast<uint4*>(S.x0)[i] = z;
      for (int i = tid; i < (int)(sizeof(S.x0t) / 16); i += blockDim.x)
         reinterpret_cast<uint4*>(S.x0t)[i] = z;
      for (int i = tid; i < (int)(sizeof(S.at) / 16); i += blockDim.x)
         reinterpret_cast<uint4*>(&S.at[0][0])[i] = z;
      for (int i = tid; i < (int)(sizeof(S.dzt) / 16); i += blockDim.x)
         reinterpret_cast<uint4*>(S.dzt)[i] = z;
   }
   __syncthreads();
   // inputs (BF16) in both layouts, and the ones rows of the transposed
   // operands (bias gradients come out of the same products)
   float in[3] = {0.f, 0.f, 0.f};
   if (valid)
      for (int q = 0; q < 3; q++) in[q] = x[4 * (long long)s + q];
   for (int q = 0; q < 3; q++) {
      st_bf16(S.x0, canon_off(row, q, 16), in[q]);
      st_bf16(S.x0t, canon_off(q, row, 128), in[q]);
   }
   st_bf16(S.x0t, canon_off(3, row, 128), 1.f);
   for (int l = 0; l < 3; l++) st_bf16(S.at[l], canon_off(64, row, 128), 1.f);
   const uint32_t mbar = smem_u32(&S.mbar);
   if (tid == 0) mbar_init(mbar, 1);
   if (warp == 0) {
      asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                       smem_u32(&S.tmem)),
                   "r"(kTrainTmemCols));
      asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
   }
   asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
   fence_async_smem();
   tc_fence_before();
   __syncthreads();
   tc_fence_after();
   const uint32_t tmem = S.tmem;
   const uint32_t lane_off = (uint32_t)(warp * 32) << 16;
   const uint32_t t_acc = tmem + lane_off;           // Z / dX, columns [0, 64)
   const uint32_t t_dw = tmem + 128 + lane_off;      // dW, columns [128, 208)
   const uint32_t t_sd = tmem + 256 + lane_off;      // silu', columns [256, 448)
   const uint32_t ax0 = smem_u32(S.x0), aact = smem_u32(S.act);
   uint32_t phase = 0;
   bool ok = true;
   auto wait_mma = [&]() {
      ok = __syncthreads_and(mbar_wait(mbar, phase, wait_limit));
      phase ^= 1;
      tc_fence_after();
   };
   auto issue_begin = [&]() {
      fence_async_smem();
      tc_fence_before();
      __syncthreads();
   };
   // ---------------- forward ----------------
   issue_begin();
   if (tid == 0 && !skip_issue) {
      tc_fence_after();
      umma_f16(tmem, umma_desc(ax0, 128, 256), umma_desc(smem_u32(S.w1), 128, 256),
               umma_idesc(64), 0);
      umma_commit(mbar);
   }
   wait_mma();
   for (int l = 0; l < 3 && ok; l++) {
      // epilogue of layer l: Z + b, silu' to tensor memory, A in both layouts
#pragma unroll
      for (int q = 0; q < 4; q++) {
         uint32_t r[16];
         TMEM_LD_X16(t_acc + 16 * q, r);
         tmem_wait_ld();
         float a[16];
         uint32_t d[16];
#pragma unroll
         for (int j = 0; j < 16; j++) {
            const float z = __uint_as_float(r[j]) + S.b[64 * l + 16 * q + j];
            a[j] = silu_f(z);
            d[j] = __float_as_uint(dsilu_f(z));
         }
         TMEM_ST_X16(t_sd + 64 * l + 16 * q, d);
         st_bf16x8(S.act, row, 16 * q, 64, a);
         st_bf16x8(S.act, row, 16 * q + 8, 64, a + 8);
#pragma unroll
         for (int j = 0; j < 16; j++) st_bf16(S.at[l], canon_off(16 * q + j, row, 128), a[j]);
      }
      tmem_wait_st();
      issue_begin();
      if (tid == 0 && !skip_issue) {
         tc_fence_after();
         if (l < 2) {
            const uint32_t wb = smem_u32(l == 0 ? S.w2 : S.w3);
#pragma unroll
            for (int k = 0; k < 4; k++)
               umma_f16(tmem, umma_desc(aact + 256 * k, 128, 1024),
                        umma_desc(wb + 256 * k, 128, 1024), umma_idesc(64), k > 0);
         } else {
#pragma unroll
            for (int k = 0; k < 4; k++)
               umma_f16(tmem, umma_desc(aact + 256 * k, 128, 1024),
                        umma_desc(smem_u32(S.w4) + 256 * k, 128, 1024), umma_idesc(16), k > 0);
         }
         umma_commit(mbar);
      }
      wait_mma();
   }
   float lossv = 0.f;
   if (ok) {
      // ---------------- loss and dZ of the last layer ----------------
      uint32_t r[16];
      TMEM_LD_X16(t_acc, r);
      tmem_wait_ld();
      float dz[16];
#pragma unroll
      for (int j = 0; j < 16; j++) dz[j] = 0.f;
      if (valid) {
         for (int o = 0; o < 2; o++) {
            const float y = __uint_as_float(r[o]) + S.b[192 + o];
            const float e = y - target[2 * (long long)s + o];
            lossv += 0.5f * e * e;
            dz[o] = e * invB;
         }
      }
      st_bf16(S.dzt, canon_off(0, row, 128), dz[0]);
      st_bf16(S.dzt, canon_off(1, row, 128), dz[1]);
      st_bf16x8(S.dzn, row, 0, 16, dz);
      st_bf16x8(S.dzn, row, 8, 16, dz + 8);
   }
   // ---------------- backward, layers 4 .. 1 ----------------
   const int poff[4] = {0, 64 * 3 + 64, 64 * 3 + 64 + 64 * 64 + 64,
                        64 * 3 + 64 + 2 * (64 * 64 + 64)};
   float* part = partials + (size_t)blockIdx.x * npar;
   for (int l = 3; l >= 0 && ok; l--) {
      const int nout = l == 3 ? 2 : 64;
      const int nin = l == 0 ? 3 : 64;
      const int ndw = l == 0 ? 16 : 80;
      issue_begin();
      if (tid == 0 && !skip_issue) {
         tc_fence_after();
         const uint32_t bt = l == 0 ? smem_u32(S.x0t) : smem_u32(S.at[l - 1]);
         // dW_l | db_l = dZ^T [X | 1], K = 128 samples
#pragma unroll
         for (int k = 0; k < 8; k++)
            umma_f16(tmem + 128, umma_desc(smem_u32(S.dzt) + 256 * k, 128, 2048),
                     umma_desc(bt + 256 * k, 128, 2048), umma_idesc(ndw), k > 0);
         if (l > 0) {  // dX_{l-1} = dZ W
            if (l == 3) {
               umma_f16(tmem, umma_desc(smem_u32(S.dzn), 128, 256),
                        umma_desc(smem_u32(S.w4t), 128, 256), umma_idesc(64), 0);
            } else {
               const uint32_t wt = smem_u32(l == 2 ? S.w3t : S.w2t);
#pragma unroll
               for (int k = 0; k < 4; k++)
                  umma_f16(tmem, umma_desc(smem_u32(S.dzn) + 256 * k, 128, 1024),
                           umma_desc(wt + 256 * k, 128, 1024), umma_idesc(64), k > 0);
            }
         }
         umma_commit(mbar);
      }
      wait_mma();
      if (!ok) break;
      // weight and bias gradients of this tile: rows 0..nout-1 (warps 0, 1)
      if (warp < 2) {
         for (int q = 0; q < ndw / 16; q++) {
            uint32_t r[16];
            TMEM_LD_X16(t_dw + 16 * q, r);
            tmem_wait_ld();
            if (row < nout) {
#pragma unroll
               for (int j = 0; j < 16; j++) {
                  const int c = 16 * q + j;
                  const float v = __uint_as_float(r[j]);
                  if (c < nin)
                     part[poff[l] + row * nin + c] = v;
                  else if (c == (l == 0 ? 3 : 64))
                     part[poff[l] + nout * nin + row] = v;
               }
            }
         }
      }
      if (l == 0) break;
      // dZ_{l-1} = dX_{l-1} silu'(Z_{l-1}) for this row -> dZ^T and dZ
#pragma unroll
      for (int q = 0; q < 4; q++) {
         uint32_t r[16], d[16];
         TMEM_LD_X16(t_acc + 16 * q, r);
         TMEM_LD_X16(t_sd + 64 * (l - 1) + 16 * q, d);
         tmem_wait_ld();
         float dz[16];
#pragma unroll
         for (int j = 0; j < 16; j++)
            dz[j] = valid ? __uint_as_float(r[j]) * __uint_as_float(d[j]) : 0.f;
#pragma unroll
         for (int j = 0; j < 16; j++) st_bf16(S.dzt, canon_off(16 * q + j, row, 128), dz[j]);
         st_bf16x8(S.dzn, row, 16 * q, 64, dz);
         st_bf16x8(S.dzn, row, 16 * q + 8, 64, dz + 8);
      }
   }
   // loss partial: warp sums, then the four warps in order
   for (int o = 16; o > 0; o >>= 1) lossv += __shfl_xor_sync(0xffffffffu, lossv, o);
   if ((tid & 31) == 0) S.red[warp] = lossv;
   if (!ok) {
      if (tid == 0 && err) atomicExch(err, 1);
      mbar_wait(mbar, phase, wait_limit);
   }
   tc_fence_before();
   __syncthreads();
   if (tid == 0) part_loss[blockIdx.x] = ((S.red[0] + S.red[1]) + S.red[2]) + S.red[3];
   if (warp == 0) {
      tc_fence_after();
      asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem),
                   "r"(kTrainTmemCols));
   }
}

// gradient = sum of the CTA partials (fixed order), then one Adam update of
// the FP32 master weights (lr = 0: the sum only)
__global__ void k_mlp_reduce_adam(int n, int nparts, const float* partials, float* grads,
                                  float* w, float* m1, float* m2, float lr, float b1, float b2,
                                  float eps, float c1, float c2)
{
   const int t = blockIdx.x * blockDim.x + threadIdx.x;
   if (t >= n) return;
   float g = 0.f;
   for (int p = 0; p < nparts; p++) g += partials[(size_t)p * n + t];
   grads[t] = g;
   if (lr == 0.f) return;
   const float a = b1 * m1[t] + (1.f - b1) * g;
   const float v = b2 * m2[t] + (1.f - b2) * g * g;
   m1[t] = a;
   m2[t] = v;
   w[t] -= lr * (a / c1) / (sqrtf(v / c2) + eps);
}

// FP32 CUDA-core reference of the same inference (validation / fallback-free
// comparison in the tests): weights rounded to BF16, activations rounded to
// BF16 at layer boundaries, exact SiLU.
__global__ void k_mlp_infer_simt(ampe_model_t m, Grid g, MlpNorm nz,
                                 const float* W1, const float* W2,
                                 const float* W3, const float* W4,
                                 const float* bias, const double* phi,
                                 const double* conc, const double* tfield,
                                 float* guess_l, float* guess_s)
{
   const NormF nfl = norm_f(nz, m);
   for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
        t < g.cells(); t += (long long)gridDim.x * blockDim.x) {
      int i, j, k;
      g.ijk(t, i, j, k);
      const long long c = g.c(i, j, k);
      float x[64], y[64];
      encode_inputs_f(nfl, g, tfield, phi[c], conc[c], i, j, k, x);
      for (int q = 0; q < 3; q++) x[q] = bf16r(x[q]);
      for (int o = 0; o < 64; o++) {
         float a = bias[o];
         for (int q = 0; q < 3; q++) a += x[q] * bf16r(W1[o * 3 + q]);
         y[o] = bf16r(silu(a));
      }
      const float* Ws[2] = {W2, W3};
      for (int l = 0; l < 2; l++) {
         for (int o = 0; o < 64; o++) {
            float a = bias[64 * (l + 1) + o];
            for (int q = 0; q < 64; q++) a += y[q] * bf16r(Ws[l][o * 64 + q]);
            x[o] = bf16r(silu(a));
         }
         for (int o = 0; o < 64; o++) y[o] = x[o];
      }
      float out[2];
      for (int o = 0; o < 2; o++) {
         float a = bias[192 + o];
         for (int q = 0; q < 64; q++) a += y[q] * bf16r(W4[o * 64 + q]);
         out[o] = a;
      }
      guess_l[t] = 1.f / (1.f + expf(-out[0]));
      guess_s[t] = 1.f / (1.f + expf(-out[1]));
   }
}

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
static const int kLayerK[4] = {3, 64, 64, 64};
static const int kLayerN[4] = {64, 64, 64, 2};

static int wcount(int l) { return kLayerK[l] * kLayerN[l]; }

int Mlp::nparams() const
{
   int n = 0;
   for (int l = 0; l < 4; l++) n += wcount(l) + kLayerN[l];
   return n;
}

int Mlp::create(const ampe_model_t& model, int batch_max)
{
   m = model;
   batch = batch_max;
   const int np = nparams();
   size_t bytes_w = sizeof(float) * np;
   if (cudaMalloc(&params, bytes_w) || cudaMalloc(&grads, bytes_w) ||
       cudaMalloc(&m1, bytes_w) || cudaMalloc(&m2, bytes_w))
      return AMPE_ERR_CUDA;
   cudaMemset(m1, 0, bytes_w);
   cudaMemset(m2, 0, bytes_w);
   // forward operands W1..W4 and backward operands W4^T, W3^T, W2^T
   const size_t pk =
       sizeof(__nv_bfloat16) * (64 * 16 + 2 * 64 * 64 + 16 * 64 + 64 * 16 + 2 * 64 * 64);
   if (cudaMalloc(&packed, pk)) return AMPE_ERR_CUDA;
   // one gradient partial and one loss partial per 128-sample tile
   ntiles = (batch + 127) / 128;
   if (cudaMalloc(&partials, sizeof(float) * (size_t)ntiles * np) ||
       cudaMalloc(&losspart, sizeof(float) * (size_t)ntiles) || cudaMalloc(&err, sizeof(int)))
      return AMPE_ERR_CUDA;
   cudaMemset(err, 0, sizeof(int));
   return AMPE_OK;
}

void Mlp::release()
{
   void* ps[] = {params, grads, m1, m2, packed, partials, losspart, err, samples_x, samples_t};
   for (void* p : ps)
      if (p) cudaFree(p);
}

float* Mlp::W(int l) const
{
   size_t off = 0;
   for (int q = 0; q < l; q++) off += wcount(q) + kLayerN[q];
   return params + off;
}
float* Mlp::b(int l) const { return W(l) + wcount(l); }
float* Mlp::gW(int l) const { return grads + (W(l) - params); }
float* Mlp::gb(int l) const { return grads + (b(l) - params); }

// He-style init on the host (seeded), uploaded
int Mlp::init_weights(uint32_t seed)
{
   std::vector<float> h(nparams());
   uint64_t s = seed * 6364136223846793005ULL + 1442695040888963407ULL;
   auto rnd = [&]() {
      s = s * 6364136223846793005ULL + 1442695040888963407ULL;
      return ((s >> 11) * (1.0 / 9007199254740992.0)) * 2.0 - 1.0;
   };
   size_t off = 0;
   for (int l = 0; l < 4; l++) {
      const float sc = (float)std::sqrt(3.0 / kLayerK[l]);
      for (int q = 0; q < wcount(l); q++) h[off++] = sc * (float)rnd();
      for (int q = 0; q < kLayerN[l]; q++) h[off++] = 0.f;
   }
   return cudaMemcpy(params, h.data(), sizeof(float) * h.size(), cudaMemcpyHostToDevice)
              ? AMPE_ERR_CUDA
              : AMPE_OK;
}

int Mlp::pack(cudaStream_t s)
{
   __nv_bfloat16* p1 = (__nv_bfloat16*)packed;
   __nv_bfloat16* p2 = p1 + 64 * 16;
   __nv_bfloat16* p3 = p2 + 64 * 64;
   __nv_bfloat16* p4 = p3 + 64 * 64;
   __nv_bfloat16* p4t = p4 + 16 * 64;
   __nv_bfloat16* p3t = p4t + 64 * 16;
   __nv_bfloat16* p2t = p3t + 64 * 64;
   k_pack_weights<<<16, 256, 0, s>>>(W(0), W(1), W(2), W(3), p1, p2, p3, p4, p4t, p3t, p2t);
   // contiguous biases for the inference and training kernels
   if (!bias_cat) cudaMalloc(&bias_cat, sizeof(float) * (3 * 64 + 2));
   for (int l = 0; l < 4; l++)
      cudaMemcpyAsync(bias_cat + 64 * l, b(l), sizeof(float) * kLayerN[l],
                      cudaMemcpyDeviceToDevice, s);
   return launch_status();
}

// one training step on samples x[B][4], target[B][2]: forward and backward
// on the tensor cores (one CTA per 128 samples), the partials summed into
// grads and, when lr > 0, one Adam update and the repacked operands
int Mlp::step_tc(const float* x, const float* target, int B, float lr, cudaStream_t s,
                 float* loss_out)
{
   if (B < 1 || B > batch) return AMPE_ERR_INVALID;
   const int nt = (B + 127) / 128;
   const int smem = (int)sizeof(TrainSmem) + 1024;
   static std::atomic<unsigned long long> attr{0};
   if (first_on_device(attr))
      cudaFuncSetAttribute(k_mlp_train_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
   const int np = nparams();
   k_mlp_train_tc<<<nt, 128, smem, s>>>((const __nv_bfloat16*)packed, bias_cat, x, target, B,
                                        partials, np, losspart, err, wait_limit, skip_issue);
   int rc = launch_status();
   if (rc) return rc;
   float c1 = 1.f, c2 = 1.f;
   const float b1 = 0.9f, b2 = 0.999f;
   if (lr > 0.f) {
      step++;
      c1 = 1.f - std::pow(b1, (float)step);
      c2 = 1.f - std::pow(b2, (float)step);
   }
   k_mlp_reduce_adam<<<(np + 255) / 256, 256, 0, s>>>(np, nt, partials, grads, params, m1, m2,
                                                      lr, b1, b2, 1e-8f, c1, c2);
   rc = launch_status();
   if (!rc && lr > 0.f) rc = pack(s);
   if (!rc && loss_out) {
      std::vector<float> h(nt);
      cudaMemcpyAsync(h.data(), losspart, sizeof(float) * nt, cudaMemcpyDeviceToHost, s);
      if (cudaStreamSynchronize(s) != cudaSuccess) return AMPE_ERR_CUDA;
      double acc = 0;
      for (int q = 0; q < nt; q++) acc += h[q];
      *loss_out = (float)(acc / B);
   }
   return rc;
}

int Mlp::infer(const Grid& g, const double* phi, const double* conc,
               const double* tfield, float* gl, float* gs, bool tensor,
               cudaStream_t s)
{
   if (tensor) {
      const int smem = (int)sizeof(MlpSmem) + 1024;
      static std::atomic<unsigned long long> attr{0};
      if (first_on_device(attr))
         cudaFuncSetAttribute(k_mlp_infer_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
      // 42 KB of shared memory and 64 TMEM columns per CTA: five CTAs per SM
      long long tiles = (g.cells() + 127) / 128;
      int blocks = (int)(tiles < max_blocks(5) ? tiles : max_blocks(5));
      k_mlp_infer_tc<<<blocks, 128, smem, s>>>(m, g, norm, (const __nv_bfloat16*)packed,
                                               bias_cat, phi, conc, tfield, gl, gs, err,
                                               wait_limit, skip_issue);
   } else {
      long long b = (g.cells() + 127) / 128;
      if (b > max_blocks(16)) b = max_blocks(16);
      k_mlp_infer_simt<<<(unsigned)b, 128, 0, s>>>(m, g, norm, W(0), W(1), W(2), W(3),
                                                   bias_cat, phi, conc, tfield, gl, gs);
   }
   return launch_status();
}

int Mlp::generate(long long n, uint32_t seed, double tlo, double thi, double clo,
                  double chi, cudaStream_t s)
{
   if (samples_x) cudaFree(samples_x);
   if (samples_t) cudaFree(samples_t);
   samples_x = samples_t = nullptr;
   if (cudaMalloc(&samples_x, sizeof(float) * 4 * n) ||
       cudaMalloc(&samples_t, sizeof(float) * 2 * n))
      return AMPE_ERR_CUDA;
   nsamples = n;
   norm.t_mid = 0.5 * (tlo + thi);
   norm.t_inv_half = thi > tlo ? 2.0 / (thi - tlo) : 0.0;
   unsigned long long* fails;
   cudaMalloc(&fails, sizeof(*fails));
   cudaMemsetAsync(fails, 0, sizeof(*fails), s);
   long long b = (n + 255) / 256;
   if (b > max_blocks(16)) b = max_blocks(16);
   k_gen_samples<<<(unsigned)b, 256, 0, s>>>(m, norm, seed, n, tlo, thi, clo, chi,
                                             samples_x, samples_t, fails);
   unsigned long long hf = 0;
   cudaMemcpyAsync(&hf, fails, sizeof(hf), cudaMemcpyDeviceToHost, s);
   cudaStreamSynchronize(s);
   cudaFree(fails);
   gen_fails = (long long)hf;
   return launch_status();
}

}  // namespace ampe

// ---------------------------------------------------------------------------
// C-ABI
// ---------------------------------------------------------------------------
using namespace ampe;

extern "C" {

int ampe_mlp_create(const ampe_model_t* m, int batch, unsigned seed, void** handle)
{
   if (!handle || check_model(m) || batch < 1) return AMPE_ERR_INVALID;
   *handle = nullptr;
   if (ampe_device_count() < 1) return AMPE_ERR_NO_DEVICE;
   Mlp* M = new Mlp;
   int rc = M->create(*m, batch);
   if (!rc) rc = M->init_weights(seed);
   if (!rc) rc = M->pack(nullptr);
   if (!rc && cudaDeviceSynchronize() != cudaSuccess) rc = AMPE_ERR_CUDA;
   if (rc) {
      M->release();
      delete M;
      return rc;
   }
   *handle = M;
   return AMPE_OK;
}

int ampe_mlp_destroy(void* h)
{
   Mlp* M = (Mlp*)h;
   if (!M) return AMPE_ERR_INVALID;
   cudaDeviceSynchronize();
   M->release();
   if (M->bias_cat) cudaFree(M->bias_cat);
   delete M;
   return AMPE_OK;
}

int ampe_mlp_nparams(void* h) { return h ? ((Mlp*)h)->nparams() : 0; }

int ampe_mlp_generate(void* h, long long n, unsigned seed, double t_lo,
                      double t_hi, double c_lo, double c_hi,
                      long long* newton_failures)
{
   Mlp* M = (Mlp*)h;
   if (!M || n < 1 || !(t_hi >= t_lo) || !(c_lo > 0.0) || !(c_hi < 1.0))
      return AMPE_ERR_INVALID;
   int rc = M->generate(n, seed, t_lo, t_hi, c_lo, c_hi, nullptr);
   if (newton_failures) *newton_failures = M->gen_fails;
   return rc;
}

int ampe_mlp_train(void* h, int steps, int batch, float lr0, float* final_loss)
{
   Mlp* M = (Mlp*)h;
   if (!M || steps < 0 || batch < 1 || batch > M->batch || M->nsamples < batch)
      return AMPE_ERR_INVALID;
   float loss = 0.f;
   const long long nb = M->nsamples / batch;
   for (int s = 0; s < steps; s++) {
      const long long off = (long long)(s % nb) * batch;
      const bool last = s == steps - 1;
      // cosine decay from lr0 to lr0/20
      const float lr = lr0 * (0.05f + 0.95f * 0.5f * (1.f + std::cos(3.14159265f * s / steps)));
      const int rc = M->step_tc(M->samples_x + 4 * off, M->samples_t + 2 * off, batch, lr,
                                nullptr, last ? &loss : nullptr);
      if (rc) return rc;
   }
   int rc = M->pack(nullptr);
   if (cudaDeviceSynchronize() != cudaSuccess) return AMPE_ERR_CUDA;
   if (final_loss) *final_loss = loss;
   return rc;
}

int ampe_mlp_grad(void* h, const float* x, const float* target, int batch,
                  float* loss)
{
   Mlp* M = (Mlp*)h;
   if (!M || !x || !target || batch < 1 || batch > M->batch) return AMPE_ERR_INVALID;
   int rc = M->step_tc(x, target, batch, 0.f, nullptr, loss);
   if (cudaDeviceSynchronize() != cudaSuccess) return AMPE_ERR_CUDA;
   return rc;
}

int ampe_mlp_get(void* h, float* params, float* grads, int host)
{
   Mlp* M = (Mlp*)h;
   if (!M) return AMPE_ERR_INVALID;
   const cudaMemcpyKind k = host ? cudaMemcpyDeviceToHost : cudaMemcpyDeviceToDevice;
   const size_t bytes = sizeof(float) * M->nparams();
   if (params) cudaMemcpy(params, M->params, bytes, k);
   if (grads) cudaMemcpy(grads, M->grads, bytes, k);
   return cudaGetLastError() == cudaSuccess ? AMPE_OK : AMPE_ERR_CUDA;
}

int ampe_mlp_set(void* h, const float* params, int host)
{
   Mlp* M = (Mlp*)h;
   if (!M || !params) return AMPE_ERR_INVALID;
   const cudaMemcpyKind k = host ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToDevice;
   cudaMemcpy(M->params, params, sizeof(float) * M->nparams(), k);
   int rc = M->pack(nullptr);
   if (cudaDeviceSynchronize() != cudaSuccess) return AMPE_ERR_CUDA;
   return rc;
}

int ampe_mlp_set_normalization(void* h, double t_lo, double t_hi)
{
   Mlp* M = (Mlp*)h;
   if (!M || !(t_hi >= t_lo)) return AMPE_ERR_INVALID;
   M->norm.t_mid = 0.5 * (t_lo + t_hi);
   M->norm.t_inv_half = t_hi > t_lo ? 2.0 / (t_hi - t_lo) : 0.0;
   return AMPE_OK;
}

int ampe_mlp_infer(void* h, const ampe_model_t* grid, const double* phi,
                   const double* conc, const double* temp, float* guess_l,
                   float* guess_s, int tensor_cores, void* stream)
{
   Mlp* M = (Mlp*)h;
   if (!M || check_model(grid) || !phi || !conc || !guess_l || !guess_s)
      return AMPE_ERR_INVALID;
   if (grid->temp_mode == AMPE_TEMP_FIELD && !temp) return AMPE_ERR_INVALID;
   ampe_model_t mm = *grid;
   M->m.temp_mode = mm.temp_mode;
   M->m.T0 = mm.T0;
   M->m.gradT = mm.gradT;
   for (int d = 0; d < 3; d++) M->m.dx[d] = mm.dx[d];
   return M->infer(make_grid(mm), phi, conc, temp, guess_l, guess_s,
                   tensor_cores != 0, (cudaStream_t)stream);
}

int ampe_mlp_set_wait_limit(void* h, int wait_limit, int skip_issue)
{
   Mlp* M = (Mlp*)h;
   if (!M || wait_limit < 1) return AMPE_ERR_INVALID;
   M->wait_limit = wait_limit;
   M->skip_issue = skip_issue ? 1 : 0;
   return AMPE_OK;
}

int ampe_mlp_clear_status(void* h)
{
   Mlp* M = (Mlp*)h;
   if (!M) return AMPE_ERR_INVALID;
   return cudaMemset(M->err, 0, sizeof(int)) == cudaSuccess ? AMPE_OK : AMPE_ERR_CUDA;
}

int ampe_mlp_status(void* h)
{
   Mlp* M = (Mlp*)h;
   if (!M) return AMPE_ERR_INVALID;
   int e = 0;
   cudaMemcpy(&e, M->err, sizeof(int), cudaMemcpyDeviceToHost);
   return e ? AMPE_ERR_NOT_CONVERGED : AMPE_OK;
}

}  // extern "C"
