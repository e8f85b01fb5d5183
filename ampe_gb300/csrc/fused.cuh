// Fused hot-path kernels (fused.cu) used by the stepper.
#pragma once

#include "common.cuh"

namespace ampe {

int build_thermo_table(const ampe_model_t& m, ThermoCoef* tab, int n,
                       cudaStream_t s);
int kks_interior(const ampe_model_t& m, const Grid& g, const ThermoCoef* tab,
                 const double* tfield, const double* phi, const double* conc,
                 const double* clr, const double* csr, double* cl, double* cs,
                 double* dF, unsigned long long* counters, cudaStream_t s);
int rhs_fused(const ampe_model_t& m, const Grid& g, const double* phi,
              const double* quat, const double* tfield, const ThermoCoef* tab,
              const double* cl, const double* cs, const double* dF,
              const double* phid, const double* ogm, const double* conc,
              const double* cld, const double* csd, double* phi_rhs,
              double* conc_rhs, cudaStream_t s);

}  // namespace ampe
