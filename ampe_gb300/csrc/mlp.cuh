// Surrogate MLP (mlp.cu): parameters, training buffers and kernels.
#pragma once

#include <stdint.h>

#include "common.cuh"

namespace ampe {

struct MlpNorm {
   double t_mid = 1500.0, t_inv_half = 0.005;  // T -> (T - mid) * inv_half
};

struct Mlp {
   ampe_model_t m;
   MlpNorm norm;
   int batch = 0, step = 0;
   float* params = nullptr;  // FP32 master [W0 b0 W1 b1 W2 b2 W3 b3]
   float *grads = nullptr, *m1 = nullptr, *m2 = nullptr;
   void* packed = nullptr;      // BF16 canonical operands for tcgen05
   float* bias_cat = nullptr;   // [64 | 64 | 64 | 2]
   int ntiles = 0;               // 128-sample tiles of the largest batch
   float* partials = nullptr;    // [ntiles][nparams] gradient partials
   float* losspart = nullptr;    // [ntiles]
   int* err = nullptr;
   // bound of the tensor-core kernels' mbarrier waits, and the test switch
   // that makes their issuing thread commit nothing (the timeout path)
   int wait_limit = 1 << 22, skip_issue = 0;
   float *samples_x = nullptr, *samples_t = nullptr;
   long long nsamples = 0, gen_fails = 0;

   int nparams() const;
   int create(const ampe_model_t& model, int batch_max);
   void release();
   float* W(int l) const;
   float* b(int l) const;
   float* gW(int l) const;
   float* gb(int l) const;
   int init_weights(uint32_t seed);
   int pack(cudaStream_t s);
   int step_tc(const float* x, const float* target, int B, float lr, cudaStream_t s,
               float* loss_out);
   int infer(const Grid& g, const double* phi, const double* conc,
             const double* tfield, float* gl, float* gs, bool tensor,
             cudaStream_t s);
   int generate(long long n, uint32_t seed, double tlo, double thi,
                double clo, double chi, cudaStream_t s);
};

}  // namespace ampe
