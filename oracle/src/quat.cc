// CPU restatement of the quaternion orientation kernels on the hot path.
// TEST INFRASTRUCTURE ONLY.  q is stored as 4 ghosted cell fields back to
// back (SAMRAI CellData depth 4).
//   quatdiffs + quatgrad_side          3d/quatdiffs.m4:70-128, 3d/quatgrad.m4:213-335
//   quatgrad_modulus_from_sides_compact 3d/quatgrad.m4:725-790
//   quatmobility                       3d/mobility.m4:13-95
//   compute_face_coef3d, eval_grad_normi 3d/quatfacops.m4:14-155, quat.f:1497-1537
//   compute_flux3d + add_quat_op3d     3d/quatfacops.m4:227-311, 596-657
//   project3d                          3d/quatfacops.m4:1022-1075
#include <cstring>

#include "oracle_api.h"
#include "oracle_common.h"

using namespace orc;

namespace {

double eval_grad_normi(double g2, char type, double floor2, double maxi)
{
   if (type == 'm') return g2 > floor2 ? std::pow(g2, -0.5) : maxi;
   if (type == 't') {
      const double tol_taylor2 = 0.01;
      const double gng2 = g2 * maxi * maxi;
      if (gng2 > tol_taylor2) {
         const double gn = std::sqrt(g2);
         return std::tanh(maxi * gn) / gn;
      }
      return maxi * (1.0 - gng2 * (5.0 - 2.0 * gng2) / 15.0);
   }
   return std::pow(g2 + floor2, -0.5);  // 's'
}

// squared L2 norm over components and directions of the side gradient on
// face `dir` whose upper cell is (i,j,k) (quatgrad_side, then the loop of
// compute_face_coef3d: n outer, m inner)
double face_grad_norm2(const Layout& L, const double* dx, const double* q,
                       int dir, int i, int j, int k)
{
   const long qs = L.cells_ghost();
   auto Q = [&](int m, int a, int b, int c) { return q[m * qs + L.c(a, b, c)]; };
   const int ei = dir == 0, ej = dir == 1, ek = dir == 2;
   double g[3][4];
   for (int m = 0; m < 4; m++) {
      for (int n = 0; n < L.dim; n++) {
         const double dinv = 1.0 / dx[n];
         if (n == dir) {
            g[n][m] = dinv * (Q(m, i, j, k) - Q(m, i - ei, j - ej, k - ek));
            continue;
         }
         // tangential: average of the 4 differences along n around the face
         const int fi = n == 0, fj = n == 1, fk = n == 2;
         auto D = [&](int a, int b, int c) {  // diff along n ending at (a,b,c)
            return Q(m, a, b, c) - Q(m, a - fi, b - fj, c - fk);
         };
         const double p25 = 0.25 * dinv;
         g[n][m] = p25 * (D(i - ei + fi, j - ej + fj, k - ek + fk) + D(i - ei, j - ej, k - ek) +
                          D(i + fi, j + fj, k + fk) + D(i, j, k));
      }
   }
   double s = 0.0;
   for (int n = 0; n < L.dim; n++)
      for (int m = 0; m < 4; m++) s += g[n][m] * g[n][m];
   return s;
}

}  // namespace

extern "C" {

// |grad q| at cells from the normal differences on the cell's faces
void orc_quat_grad_modulus(const ampe_model_t* m, const double* q, double* ogm)
{
   Layout L(*m);
   const long qs = L.cells_ghost();
#pragma omp parallel for collapse(2) schedule(static)
   for (int k = 0; k < L.n2; k++)
      for (int j = 0; j < L.n1; j++)
         for (int i = 0; i < L.n0; i++) {
            double s = 0.0;
            for (int d = 0; d < L.dim; d++) {
               const int ei = d == 0, ej = d == 1, ek = d == 2;
               const double dinv = 1.0 / m->dx[d];
               for (int side = 0; side < 2; side++)
                  for (int c = 0; c < 4; c++) {
                     const double* qc = q + c * qs;
                     const double gd =
                         dinv * (qc[L.c(i + side * ei, j + side * ej, k + side * ek)] -
                                 qc[L.c(i + side * ei - ei, j + side * ej - ej,
                                        k + side * ek - ek)]);
                     s += gd * gd;
                  }
            }
            ogm[L.interior(i, j, k)] = std::sqrt(0.5 * s);
         }
}

// M_q(phi) on the interior (ghosted output layout)
void orc_quat_mobility(const ampe_model_t* m, const double* phi, double* mq)
{
   Layout L(*m);
   for (int k = 0; k < L.n2; k++)
      for (int j = 0; j < L.n1; j++)
         for (int i = 0; i < L.n0; i++) {
            double p = phi[L.c(i, j, k)];
            p = std::fmax(0.0, std::fmin(1.0, p));
            const double qf = 1.0 - p * p * p * (10.0 - 15.0 * p + 6.0 * p * p);
            mq[L.c(i, j, k)] =
                m->min_quat_mobility + (m->quat_mobility - m->min_quat_mobility) * qf;
         }
}

// face coefficients fc = -grad_normi * 2H Tbar p1(phibar) - eps_q^2 p2(phibar)
void orc_quat_face_coef(const ampe_model_t* m, const double* phi,
                        const double* temp, const double* qlag, double* fc0,
                        double* fc1, double* fc2)
{
   Layout L(*m);
   const double floor2 = m->quat_grad_floor * m->quat_grad_floor;
   const double maxi = 1.0 / m->quat_grad_floor;
   const double eps2 = m->epsilon_q * m->epsilon_q;
   for (int dir = 0; dir < L.dim; dir++) {
      const int ei = dir == 0, ej = dir == 1, ek = dir == 2;
      double* fc = dir == 0 ? fc0 : (dir == 1 ? fc1 : fc2);
#pragma omp parallel for collapse(2) schedule(static)
      for (int k = 0; k < L.n2 + ek; k++)
         for (int j = 0; j < L.n1 + ej; j++)
            for (int i = 0; i < L.n0 + ei; i++) {
               const double phia = average_func(phi[L.c(i - ei, j - ej, k - ek)],
                                                phi[L.c(i, j, k)], m->avg_type);
               const double tempa =
                   0.5 * (temperature_at(*m, temp, L, i - ei, j - ej, k - ek) +
                          temperature_at(*m, temp, L, i, j, k));
               const double diff = m->misorientation_factor * tempa *
                                   interp_func(phia, m->orient_interp1);
               const double hphi2 = interp_func(phia, m->orient_interp2);
               const double g2 = face_grad_norm2(L, m->dx, qlag, dir, i, j, k);
               const double gni = eval_grad_normi(g2, m->quat_floor_type, floor2, maxi);
               const long f = dir == 0 ? L.fx(i, j, k) : (dir == 1 ? L.fy(i, j, k) : L.fz(i, j, k));
               fc[f] = -gni * diff - eps2 * hphi2;
            }
   }
}

// q' = -M_q div(fc grad q) for the 4 components (interior output, 4N)
void orc_quat_rhs(const ampe_model_t* m, const double* fc0, const double* fc1,
                  const double* fc2, const double* mq, const double* q,
                  double* out)
{
   Layout L(*m);
   const long qs = L.cells_ghost(), N = L.cells();
   const double hinv[3] = {1.0 / m->dx[0], 1.0 / m->dx[1],
                           L.dim == 3 ? 1.0 / m->dx[2] : 0.0};
   for (int c = 0; c < 4; c++) {
      const double* qc = q + c * qs;
#pragma omp parallel for collapse(2) schedule(static)
      for (int k = 0; k < L.n2; k++)
         for (int j = 0; j < L.n1; j++)
            for (int i = 0; i < L.n0; i++) {
               auto flux = [&](int dir, int a, int b, int cc) {
                  const int ei = dir == 0, ej = dir == 1, ek = dir == 2;
                  const double f = dir == 0 ? fc0[L.fx(a, b, cc)]
                                            : (dir == 1 ? fc1[L.fy(a, b, cc)] : fc2[L.fz(a, b, cc)]);
                  return f * hinv[dir] * (qc[L.c(a, b, cc)] - qc[L.c(a - ei, b - ej, cc - ek)]);
               };
               double div = (flux(0, i + 1, j, k) - flux(0, i, j, k)) * hinv[0] +
                            (flux(1, i, j + 1, k) - flux(1, i, j, k)) * hinv[1];
               if (L.dim == 3) div += (flux(2, i, j, k + 1) - flux(2, i, j, k)) * hinv[2];
               out[c * N + L.interior(i, j, k)] = 0.0 - mq[L.c(i, j, k)] * div;
            }
   }
}

// project q (interior 4N) onto unit quaternions
void orc_quat_project(long ncells, double* q)
{
   for (long t = 0; t < ncells; t++) {
      double s = 0.0;
      for (int c = 0; c < 4; c++) s += q[c * ncells + t] * q[c * ncells + t];
      const double f = 1.0 / std::sqrt(s);
      for (int c = 0; c < 4; c++) q[c * ncells + t] *= f;
   }
}

}  // extern "C"
