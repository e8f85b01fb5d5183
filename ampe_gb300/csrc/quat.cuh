// Quaternion orientation kernels (quat.cu) used by the stepper, and the
// device helpers shared with the FP32 kernels of the mixed path (mixed.cu).
#pragma once

#include "common.cuh"

namespace ampe {

// 1/dx per direction, computed on the host (0 beyond dim)
template <class R>
struct Inv3 {
   R v[3];
};
template <class R>
inline Inv3<R> inv_spacing(const ampe_model_t& m)
{
   Inv3<R> r;
   for (int d = 0; d < 3; d++) r.v[d] = d < m.dim ? (R)(1.0 / m.dx[d]) : R(0);
   return r;
}

// eval_grad_normi (quat.f:1497-1537): 1/|grad q| regularised by the floor
// ('m' max, 't' tanh with its Taylor branch, 's' smooth)
__device__ __forceinline__ double eval_grad_normi(double g2, char type,
                                                  double floor2, double maxi)
{
   if (type == 'm') return g2 > floor2 ? pow(g2, -0.5) : maxi;
   if (type == 't') {
      const double gng2 = g2 * maxi * maxi;
      if (gng2 > 0.01) {
         const double gn = sqrt(g2);
         return tanh(maxi * gn) / gn;
      }
      return maxi * (1.0 - gng2 * (5.0 - 2.0 * gng2) / 15.0);
   }
   return pow(g2 + floor2, -0.5);
}

__device__ __forceinline__ float eval_grad_normi(float g2, char type,
                                                 float floor2, float maxi)
{
   if (type == 'm') return g2 > floor2 ? rsqrtf(g2) : maxi;
   if (type == 't') {
      const float gng2 = g2 * maxi * maxi;
      if (gng2 > 0.01f) {
         const float gn = sqrtf(g2);
         return tanhf(maxi * gn) / gn;
      }
      return maxi * (1.f - gng2 * (5.f - 2.f * gng2) * (1.f / 15.f));
   }
   return rsqrtf(g2 + floor2);
}

// squared norm over components and directions of the side gradient of q on
// face `dir` whose upper cell is (i,j,k): QUATGRAD_SIDE (3d/quatgrad.m4:
// 213-335) -- normal difference, tangential average of four differences --
// summed as in COMPUTE_FACE_COEF3D (3d/quatfacops.m4:14-155)
template <int DIM, class R>
__device__ __forceinline__ R face_grad_norm2(const Grid& g, const R* dinv,
                                             const R* q, int dir, int i, int j,
                                             int k)
{
   const long long qs = g.cells_ghost();
   const int ei = dir == 0, ej = dir == 1, ek = dir == 2;
   R gsum[3][4];
#pragma unroll
   for (int m = 0; m < 4; m++) {
      const R* Q = q + m * qs;
#pragma unroll
      for (int n = 0; n < DIM; n++) {
         if (n == dir) {
            gsum[n][m] = dinv[n] * (Q[g.c(i, j, k)] - Q[g.c(i - ei, j - ej, k - ek)]);
            continue;
         }
         const int fi = n == 0, fj = n == 1, fk = n == 2;
         auto D = [&](int a, int b, int c) {
            return Q[g.c(a, b, c)] - Q[g.c(a - fi, b - fj, c - fk)];
         };
         const R p25 = (R)0.25 * dinv[n];
         gsum[n][m] = p25 * (D(i - ei + fi, j - ej + fj, k - ek + fk) + D(i - ei, j - ej, k - ek) +
                             D(i + fi, j + fj, k + fk) + D(i, j, k));
      }
   }
   R s = 0;
#pragma unroll
   for (int n = 0; n < DIM; n++)
#pragma unroll
      for (int m = 0; m < 4; m++) s += gsum[n][m] * gsum[n][m];
   return s;
}

// face index t over [x faces | y faces | z faces] -> (dir, i, j, k)
__device__ __forceinline__ void face_of(const Grid& g, long long t, int& dir,
                                        int& i, int& j, int& k)
{
   const long long nx = g.nfx(), ny = g.nfy();
   long long r = t;
   if (r < nx) {
      dir = 0;
      g.split(r, g.fd0p, g.fd1, i, j, k);
   } else if ((r -= nx) < ny) {
      dir = 1;
      g.split(r, g.fd0, g.fd1p, i, j, k);
   } else {
      r -= ny;
      dir = 2;
      g.ijk(r, i, j, k);
   }
}

template <class R>
int quat_grad_modulus(const ampe_model_t& m, const Grid& g, const R* q, R* ogm,
                      cudaStream_t s);
template <class R>
int quat_mobility(const ampe_model_t& m, const Grid& g, const double* phi, R* mq,
                  cudaStream_t s);
// fc = scale (-grad_normi 2H T p1(phibar) - eps_q^2 p2(phibar)) on every
// face, FP64
int quat_face_coef(const ampe_model_t& m, const Grid& g, const double* phi,
                   const double* tfield, const double* qlag, double scale,
                   double* fc0, double* fc1, double* fc2, cudaStream_t s);
template <class R>
int quat_rhs(const ampe_model_t& m, const Grid& g, const R* fc0, const R* fc1,
             const R* fc2, const R* mq, const R* q, double* out, cudaStream_t s);
int quat_project(long long N, double* q, cudaStream_t s);

}  // namespace ampe
