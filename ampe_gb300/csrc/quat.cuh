// Quaternion orientation kernels (quat.cu) used by the stepper.
#pragma once

#include "common.cuh"

namespace ampe {

template <class R>
int quat_grad_modulus(const ampe_model_t& m, const Grid& g, const R* q, R* ogm,
                      cudaStream_t s);
template <class R>
int quat_mobility(const ampe_model_t& m, const Grid& g, const double* phi, R* mq,
                  cudaStream_t s);
// fc = scale (-grad_normi 2H T p1(phibar) - eps_q^2 p2(phibar)) on every face
template <class QT, class R>
int quat_face_coef(const ampe_model_t& m, const Grid& g, const double* phi,
                   const double* tfield, const QT* qlag, double scale, R* fc0,
                   R* fc1, R* fc2, cudaStream_t s);
template <class R>
int quat_rhs(const ampe_model_t& m, const Grid& g, const R* fc0, const R* fc1,
             const R* fc2, const R* mq, const R* q, double* out, cudaStream_t s);
int quat_project(long long N, double* q, cudaStream_t s);

}  // namespace ampe
