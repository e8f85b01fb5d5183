// Phase flux on one face for the three reference discretisations:
// gradient_flux (3d/quatrhs.m4:12-65), compute_flux_isotropic
// (2d/quatrhs.m4:106-151) and anisotropic_gradient_flux
// (2d/quatrhs.m4:154-256, 3d/quatrhs.m4:180-349, compute_dgamma :149-177).
// Shared by the leaf kernel (one face per thread) and the fused RHS kernel.
#pragma once

#include "common.cuh"

namespace ampe {

__device__ __forceinline__ void qmul(const double* a, const double* b,
                                     double* q)
{
   // quat.f:867-894 (Hamilton product)
   q[0] = a[0] * b[0] - a[1] * b[1] - a[2] * b[2] - a[3] * b[3];
   q[1] = a[0] * b[1] + a[1] * b[0] + a[2] * b[3] - a[3] * b[2];
   q[2] = a[0] * b[2] + a[2] * b[0] + a[3] * b[1] - a[1] * b[3];
   q[3] = a[0] * b[3] + a[3] * b[0] + a[1] * b[2] - a[2] * b[1];
}

// compute_dgamma, 3d/quatrhs.m4:149-177
__device__ __forceinline__ void dgamma_of(const double* q, const double* n,
                                          double* dg, double* n4)
{
   double qp[4] = {q[0], -q[1], -q[2], -q[3]}, tmp[4], np[4];
   qmul(n, qp, tmp);
   qmul(q, tmp, np);
   *n4 = np[1] * np[1] * np[1] * np[1] + np[2] * np[2] * np[2] * np[2] +
         np[3] * np[3] * np[3] * np[3];
   double d[4] = {0.0, np[1] * (np[1] * np[1] - *n4),
                  np[2] * (np[2] * np[2] - *n4),
                  np[3] * (np[3] * np[3] - *n4)};
   qmul(d, q, tmp);
   qmul(qp, tmp, dg);
}

// Flux on face `dir` whose upper cell is (i,j,k); shared by the leaf and the
// fused kernels.  phase(a,b,c) accessor P, quaternion accessor Q(comp,a,b,c).
template <class PF, class QF>
__device__ __forceinline__ double phase_face_flux(const ampe_model_t& m,
                                                  int dim, int dir, int i,
                                                  int j, int k, PF P, QF Q)
{
   const double eps = m.epsilon_phi, eps2 = eps * eps;
   const double fthr = (double)1.e-12f;  // REAL literal in the reference
   if (m.flux_type == AMPE_FLUX_SIMPLE) {
      const double dinv = eps2 / m.dx[dir];
      if (dir == 0) return (P(i, j, k) - P(i - 1, j, k)) * dinv;
      if (dir == 1) return (P(i, j, k) - P(i, j - 1, k)) * dinv;
      return (P(i, j, k) - P(i, j, k - 1)) * dinv;
   }
   if (m.flux_type == AMPE_FLUX_ISOTROPIC) {
      const double dinv = (1.0 / 12.0) * eps2 / m.dx[dir];
      if (dir == 0)
         return dinv * ((P(i, j - 1, k) - P(i - 1, j - 1, k)) +
                        (P(i, j, k) - P(i - 1, j, k)) * 10.0 +
                        (P(i, j + 1, k) - P(i - 1, j + 1, k)));
      return dinv * ((P(i - 1, j, k) - P(i - 1, j - 1, k)) +
                     (P(i, j, k) - P(i, j - 1, k)) * 10.0 +
                     (P(i + 1, j, k) - P(i + 1, j - 1, k)));
   }
   const double dxi = 1.0 / m.dx[0], dyi = 1.0 / m.dx[1];
   if (dim == 2) {
      const double pi = 4.0 * atan(1.0);
      const double nu = m.aniso_eps, kn = (double)m.aniso_k;
      double dpx, dpy, q;
      if (dir == 0) {
         dpx = (P(i, j, k) - P(i - 1, j, k)) * dxi;
         dpy = 0.25 * (P(i - 1, j + 1, k) - P(i - 1, j - 1, k) + P(i, j + 1, k) -
                       P(i, j - 1, k)) * dyi;
         q = 0.5 * (Q(0, i - 1, j, k) + Q(0, i, j, k));
      } else {
         dpx = 0.25 * (P(i + 1, j - 1, k) - P(i - 1, j - 1, k) + P(i + 1, j, k) -
                       P(i - 1, j, k)) * dxi;
         dpy = (P(i, j, k) - P(i, j - 1, k)) * dyi;
         q = 0.5 * (Q(0, i, j - 1, k) + Q(0, i, j, k));
      }
      const double theta = fabs(dpx) > fthr ? atan(dpy / dpx) : 0.5 * pi;
      if (q > 1.0) q = 1.0;
      if (q < -1.0) q = -1.0;
      const double phi = (m.qlen == 4) ? 2.0 * acos(q) : acos(q);
      const double et = eps * (1.0 + nu * cos(kn * (theta - phi)));
      const double de = -kn * eps * nu * sin(kn * (theta - phi));
      if (dir == 0) return et * et * dpx - et * de * dpy;
      return et * et * dpy + et * de * dpx;
   }
   const double dzi = 1.0 / m.dx[2];
   const double e4 = m.aniso_eps;
   const double factor = 4.0 * e4 / (1.0 - 3.0 * e4);
   double g[3];
   if (dir == 0) {
      g[0] = (P(i, j, k) - P(i - 1, j, k)) * dxi;
      g[1] = 0.25 * (P(i - 1, j + 1, k) - P(i - 1, j - 1, k) + P(i, j + 1, k) -
                     P(i, j - 1, k)) * dyi;
      g[2] = 0.25 * (P(i - 1, j, k + 1) - P(i - 1, j, k - 1) + P(i, j, k + 1) -
                     P(i, j, k - 1)) * dzi;
   } else if (dir == 1) {
      g[0] = 0.25 * (P(i + 1, j - 1, k) - P(i - 1, j - 1, k) + P(i + 1, j, k) -
                     P(i - 1, j, k)) * dxi;
      g[1] = (P(i, j, k) - P(i, j - 1, k)) * dyi;
      g[2] = 0.25 * (P(i, j - 1, k + 1) - P(i, j - 1, k - 1) + P(i, j, k + 1) -
                     P(i, j, k - 1)) * dzi;
   } else {
      g[0] = 0.25 * (P(i + 1, j, k - 1) - P(i - 1, j, k - 1) + P(i + 1, j, k) -
                     P(i - 1, j, k)) * dxi;
      g[1] = 0.25 * (P(i, j + 1, k - 1) - P(i, j - 1, k - 1) + P(i, j + 1, k) -
                     P(i, j - 1, k)) * dyi;
      g[2] = (P(i, j, k) - P(i, j, k - 1)) * dzi;
   }
   const double gphi2 = g[0] * g[0] + g[1] * g[1] + g[2] * g[2];
   double dg[4], n4;
   if (fabs(gphi2) > fthr) {
      const double nni = 1.0 / sqrt(gphi2);
      const double n[4] = {0.0, g[0] * nni, g[1] * nni, g[2] * nni};
      const int ei = dir == 0, ej = dir == 1, ek = dir == 2;
      double q[4];
      for (int c = 0; c < 4; c++)
         q[c] = 0.5 * (Q(c, i - ei, j - ej, k - ek) + Q(c, i, j, k));
      dgamma_of(q, n, dg, &n4);
   } else {
      dg[0] = dg[1] = 0.0;
      dg[2] = dir == 2 ? 1.0 : 0.0;
      dg[3] = dir == 2 ? 0.0 : 1.0;
      n4 = 0.0;
   }
   const double gamma = eps * (1.0 - 3.0 * e4) * (1.0 + factor * n4);
   return gamma * gamma * g[dir] +
          16.0 * eps * gamma * e4 * sqrt(gphi2) * dg[dir + 1];
}

}  // namespace ampe
