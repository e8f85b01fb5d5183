// Mixed-precision kernels (mixed.cu) used by the stepper.
#pragma once

#include "common.cuh"

namespace ampe {

// FP32 copy of ThermoCoef for the mixed kernels
struct CoefF {
   float RT, iRT, dG[2], GB[2], L[2][4];
};

int build_coef_f(const ThermoCoef* tab, CoefF* tabf, int n, cudaStream_t s);

// FP32 constants of the mixed kernels, computed once on the host so that no
// kernel spends FP64-pipe cycles on per-thread divisions or conversions
struct MixParams {
   float dxi[3];       // 1/dx
   float flux_dinv[3]; // eps^2/dx (simple) or eps^2/(12 dx) (isotropic)
   float w, Mphi, Mc, Dl, Ds, qlR, qsR, ivm;
   int tdep, iso;
};
MixParams make_mix_params(const ampe_model_t& m);
int kks_mixed(const ampe_model_t& m, const MixParams& mp, const Grid& g,
              const ThermoCoef* tab, const CoefF* tabf, const double* tfield,
              const double* phi,
              const double* conc, const float* guess_l, const float* guess_s,
              const float* clr, const float* csr, float* cl, float* cs,
              float* dF, unsigned long long* counters, cudaStream_t s);
int rhs_mixed(const ampe_model_t& m, const MixParams& mp, const Grid& g,
              const double* tfield,
              const double* phi, float* pf, const float* cl, const float* cs,
              const float* dF, double* phi_rhs, double* conc_rhs,
              cudaStream_t s);
int jv_mixed(const ampe_model_t& m, const MixParams& mp, const Grid& g,
             const CoefF* tabf,
             const double* tfield, const float* pf, const float* cl,
             const float* cs, const float* dF, const double* v, double gamma,
             float* dphi, float* da, float* db, double* out, cudaStream_t s);

}  // namespace ampe
