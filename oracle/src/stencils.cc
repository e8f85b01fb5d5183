// CPU restatement of the phase / composition right-hand-side kernels.
// TEST INFRASTRUCTURE ONLY.  Loops and expression order follow the
// reference Fortran cited at each function.
#include <cstring>

#include "oracle_common.h"
#include "oracle_api.h"

using namespace orc;

extern "C" {

// SAMRAI periodic ghost fill of a cell field (all faces, edges, corners).
void orc_fill_ghosts(const ampe_model_t* m, double* f)
{
   Layout L(*m);
   for (int k = -L.gz; k < L.n2 + L.gz; k++)
      for (int j = -L.ng; j < L.n1 + L.ng; j++)
         for (int i = -L.ng; i < L.n0 + L.ng; i++) {
            const bool in = i >= 0 && i < L.n0 && j >= 0 && j < L.n1 &&
                            k >= 0 && k < L.n2;
            if (in) continue;
            const int iw = ((i % L.n0) + L.n0) % L.n0;
            const int jw = ((j % L.n1) + L.n1) % L.n1;
            const int kw = ((k % L.n2) + L.n2) % L.n2;
            f[L.c(i, j, k)] = f[L.c(iw, jw, kw)];
         }
}

// gradient_flux (2d/quatrhs.m4:12-53, 3d/quatrhs.m4:12-65),
// compute_flux_isotropic (2d/quatrhs.m4:106-151),
// anisotropic_gradient_flux (2d/quatrhs.m4:154-256, 3d/quatrhs.m4:180-349).
static void quat_mult(const double* a, const double* b, double* q)
{
   // quat.f:867-894
   q[0] = a[0] * b[0] - a[1] * b[1] - a[2] * b[2] - a[3] * b[3];
   q[1] = a[0] * b[1] + a[1] * b[0] + a[2] * b[3] - a[3] * b[2];
   q[2] = a[0] * b[2] + a[2] * b[0] + a[3] * b[1] - a[1] * b[3];
   q[3] = a[0] * b[3] + a[3] * b[0] + a[1] * b[2] - a[2] * b[1];
}

// compute_dgamma, 3d/quatrhs.m4:149-177
static void compute_dgamma(const double* q, const double* n, double* dg,
                           double* n4)
{
   double qp[4] = {q[0], -q[1], -q[2], -q[3]}, tmp[4], np[4];
   quat_mult(n, qp, tmp);
   quat_mult(q, tmp, np);
   *n4 = np[1] * np[1] * np[1] * np[1] + np[2] * np[2] * np[2] * np[2] +
         np[3] * np[3] * np[3] * np[3];
   double d[4] = {0.0, np[1] * (np[1] * np[1] - *n4),
                  np[2] * (np[2] * np[2] - *n4),
                  np[3] * (np[3] * np[3] - *n4)};
   quat_mult(d, q, tmp);
   quat_mult(qp, tmp, dg);
}

void orc_phase_flux(const ampe_model_t* m, const double* ph,
                    const double* quat, double* f0, double* f1, double* f2)
{
   Layout L(*m);
   const double* dx = m->dx;
   const double eps = m->epsilon_phi, eps2 = eps * eps;
   const long qs = L.cells_ghost();
   const double fthr = (double)1.e-12f;  // REAL literal in the reference
   if (m->flux_type == AMPE_FLUX_SIMPLE) {
      const double dxi = eps2 / dx[0], dyi = eps2 / dx[1];
      #pragma omp parallel for collapse(2) schedule(static)
      for (int k = 0; k < L.n2; k++)
         for (int j = 0; j < L.n1; j++)
            for (int i = 0; i <= L.n0; i++)
               f0[L.fx(i, j, k)] = (ph[L.c(i, j, k)] - ph[L.c(i - 1, j, k)]) * dxi;
      #pragma omp parallel for collapse(2) schedule(static)
      for (int k = 0; k < L.n2; k++)
         for (int j = 0; j <= L.n1; j++)
            for (int i = 0; i < L.n0; i++)
               f1[L.fy(i, j, k)] = (ph[L.c(i, j, k)] - ph[L.c(i, j - 1, k)]) * dyi;
      if (L.dim == 3) {
         const double dzi = eps2 / dx[2];
         #pragma omp parallel for collapse(2) schedule(static)
         for (int k = 0; k <= L.n2; k++)
            for (int j = 0; j < L.n1; j++)
               for (int i = 0; i < L.n0; i++)
                  f2[L.fz(i, j, k)] =
                      (ph[L.c(i, j, k)] - ph[L.c(i, j, k - 1)]) * dzi;
      }
      return;
   }
   if (m->flux_type == AMPE_FLUX_ISOTROPIC) {
      // 2D only: the 3D variant stops in the reference (3d/quatrhs.m4:90-92)
      const double dxi = (1.0 / 12.0) * eps2 / dx[0];
      const double dyi = (1.0 / 12.0) * eps2 / dx[1];
      const int k = 0;
      for (int j = 0; j < L.n1; j++)
         for (int i = 0; i <= L.n0; i++)
            f0[L.fx(i, j, k)] =
                dxi * ((ph[L.c(i, j - 1, k)] - ph[L.c(i - 1, j - 1, k)]) +
                       (ph[L.c(i, j, k)] - ph[L.c(i - 1, j, k)]) * 10.0 +
                       (ph[L.c(i, j + 1, k)] - ph[L.c(i - 1, j + 1, k)]));
      for (int j = 0; j <= L.n1; j++)
         for (int i = 0; i < L.n0; i++)
            f1[L.fy(i, j, k)] =
                dyi * ((ph[L.c(i - 1, j, k)] - ph[L.c(i - 1, j - 1, k)]) +
                       (ph[L.c(i, j, k)] - ph[L.c(i, j - 1, k)]) * 10.0 +
                       (ph[L.c(i + 1, j, k)] - ph[L.c(i + 1, j - 1, k)]));
      return;
   }
   // anisotropic
   const double dxi = 1.0 / dx[0], dyi = 1.0 / dx[1];
   if (L.dim == 2) {
      const double pi = 4.0 * std::atan(1.0);
      const double nu = m->aniso_eps;
      const double kn = (double)m->aniso_k;
      const int k = 0;
      for (int j = 0; j < L.n1; j++)
         for (int i = 0; i <= L.n0; i++) {
            const double dpx = (ph[L.c(i, j, k)] - ph[L.c(i - 1, j, k)]) * dxi;
            const double dpy =
                0.25 * (ph[L.c(i - 1, j + 1, k)] - ph[L.c(i - 1, j - 1, k)] +
                        ph[L.c(i, j + 1, k)] - ph[L.c(i, j - 1, k)]) * dyi;
            const double theta =
                std::fabs(dpx) > fthr ? std::atan(dpy / dpx) : 0.5 * pi;
            double q = 0.5 * (quat[L.c(i - 1, j, k)] + quat[L.c(i, j, k)]);
            if (q > 1.0) q = 1.0;
            if (q < -1.0) q = -1.0;
            const double phi = (m->qlen == 4) ? 2.0 * std::acos(q) : std::acos(q);
            const double et = eps * (1.0 + nu * std::cos(kn * (theta - phi)));
            const double de = -kn * eps * nu * std::sin(kn * (theta - phi));
            f0[L.fx(i, j, k)] = et * et * dpx - et * de * dpy;
         }
      for (int j = 0; j <= L.n1; j++)
         for (int i = 0; i < L.n0; i++) {
            const double dpx =
                0.25 * (ph[L.c(i + 1, j - 1, k)] - ph[L.c(i - 1, j - 1, k)] +
                        ph[L.c(i + 1, j, k)] - ph[L.c(i - 1, j, k)]) * dxi;
            const double dpy = (ph[L.c(i, j, k)] - ph[L.c(i, j - 1, k)]) * dyi;
            const double theta =
                std::fabs(dpx) > fthr ? std::atan(dpy / dpx) : 0.5 * pi;
            double q = 0.5 * (quat[L.c(i, j - 1, k)] + quat[L.c(i, j, k)]);
            if (q > 1.0) q = 1.0;
            if (q < -1.0) q = -1.0;
            const double phi = (m->qlen == 4) ? 2.0 * std::acos(q) : std::acos(q);
            const double et = eps * (1.0 + nu * std::cos(kn * (theta - phi)));
            const double de = -kn * eps * nu * std::sin(kn * (theta - phi));
            f1[L.fy(i, j, k)] = et * et * dpy + et * de * dpx;
         }
      return;
   }
   const double dzi = 1.0 / dx[2];
   const double e4 = m->aniso_eps;
   const double factor = 4.0 * e4 / (1.0 - 3.0 * e4);
   for (int dir = 0; dir < 3; dir++) {
      const int ei = dir == 0, ej = dir == 1, ek = dir == 2;
      const int ni = L.n0 + ei, nj = L.n1 + ej, nk = L.n2 + ek;
#pragma omp parallel for collapse(2) schedule(static)
      for (int k = 0; k < nk; k++)
         for (int j = 0; j < nj; j++)
            for (int i = 0; i < ni; i++) {
               // neighbour cell across the face is (i-ei, j-ej, k-ek)
               double g[3];
               auto P = [&](int a, int b, int c) { return ph[L.c(a, b, c)]; };
               if (dir == 0) {
                  g[0] = (P(i, j, k) - P(i - 1, j, k)) * dxi;
                  g[1] = 0.25 * (P(i - 1, j + 1, k) - P(i - 1, j - 1, k) +
                                 P(i, j + 1, k) - P(i, j - 1, k)) * dyi;
                  g[2] = 0.25 * (P(i - 1, j, k + 1) - P(i - 1, j, k - 1) +
                                 P(i, j, k + 1) - P(i, j, k - 1)) * dzi;
               } else if (dir == 1) {
                  g[0] = 0.25 * (P(i + 1, j - 1, k) - P(i - 1, j - 1, k) +
                                 P(i + 1, j, k) - P(i - 1, j, k)) * dxi;
                  g[1] = (P(i, j, k) - P(i, j - 1, k)) * dyi;
                  g[2] = 0.25 * (P(i, j - 1, k + 1) - P(i, j - 1, k - 1) +
                                 P(i, j, k + 1) - P(i, j, k - 1)) * dzi;
               } else {
                  g[0] = 0.25 * (P(i + 1, j, k - 1) - P(i - 1, j, k - 1) +
                                 P(i + 1, j, k) - P(i - 1, j, k)) * dxi;
                  g[1] = 0.25 * (P(i, j + 1, k - 1) - P(i, j - 1, k - 1) +
                                 P(i, j + 1, k) - P(i, j - 1, k)) * dyi;
                  g[2] = (P(i, j, k) - P(i, j, k - 1)) * dzi;
               }
               const double gphi2 = g[0] * g[0] + g[1] * g[1] + g[2] * g[2];
               double dg[4], n4;
               if (std::fabs(gphi2) > fthr) {
                  const double nni = 1.0 / std::sqrt(gphi2);
                  const double n[4] = {0.0, g[0] * nni, g[1] * nni, g[2] * nni};
                  double q[4];
                  for (int c = 0; c < 4; c++)
                     q[c] = 0.5 * (quat[c * qs + L.c(i - ei, j - ej, k - ek)] +
                                   quat[c * qs + L.c(i, j, k)]);
                  compute_dgamma(q, n, dg, &n4);
               } else {
                  // reference defaults: (0,0,0,1) on x,y faces, (0,0,1,0) on z
                  dg[0] = dg[1] = 0.0;
                  dg[2] = dir == 2 ? 1.0 : 0.0;
                  dg[3] = dir == 2 ? 0.0 : 1.0;
                  n4 = 0.0;
               }
               const double gamma = eps * (1.0 - 3.0 * e4) * (1.0 + factor * n4);
               const double v = gamma * gamma * g[dir] +
                                16.0 * eps * gamma * e4 * std::sqrt(gphi2) *
                                    dg[dir + 1];
               if (dir == 0) f0[L.fx(i, j, k)] = v;
               if (dir == 1) f1[L.fy(i, j, k)] = v;
               if (dir == 2) f2[L.fz(i, j, k)] = v;
            }
   }
}

// computerhspbg (2d/quatrhs.m4:264-405, 3d/quatrhs.m4:357-512), two phases
void orc_computerhspbg(const ampe_model_t* m, const double* f0,
                       const double* f1, const double* f2, const double* temp,
                       const double* phi, const double* ogm, double* rhs)
{
   Layout L(*m);
   const double dxi = 1.0 / m->dx[0], dyi = 1.0 / m->dx[1];
   const double dzi = L.dim == 3 ? 1.0 / m->dx[2] : 0.0;
   const double eq2 = 0.5 * m->epsilon_q * m->epsilon_q;
#pragma omp parallel for collapse(2) schedule(static)
   for (int k = 0; k < L.n2; k++)
      for (int j = 0; j < L.n1; j++)
         for (int i = 0; i < L.n0; i++) {
            double d = (f0[L.fx(i + 1, j, k)] - f0[L.fx(i, j, k)]) * dxi +
                       (f1[L.fy(i, j + 1, k)] - f1[L.fy(i, j, k)]) * dyi;
            if (L.dim == 3)
               d = (f0[L.fx(i + 1, j, k)] - f0[L.fx(i, j, k)]) * dxi +
                   (f1[L.fy(i, j + 1, k)] - f1[L.fy(i, j, k)]) * dyi +
                   (f2[L.fz(i, j, k + 1)] - f2[L.fz(i, j, k)]) * dzi;
            const double p = phi[L.c(i, j, k)];
            double r = d - m->phase_well_scale * deriv_well_func(p, m->well_type);
            if (m->with_orient) {
               const double p1 = deriv_interp_func(p, m->orient_interp1);
               const double p2 = deriv_interp_func(p, m->orient_interp2);
               const double g = ogm[L.interior(i, j, k)];
               const double T = temperature_at(*m, temp, L, i, j, k);
               r = r - m->misorientation_factor * T * p1 * g - p2 * eq2 * g * g;
            }
            rhs[L.interior(i, j, k)] = r;
         }
}

// KKSdiluteBinary.cc:507-626 / CALPHADFreeEnergyStrategyBinary.cc:521-670
void orc_add_driving_force(const ampe_model_t* m, const double* temp,
                           const double* phi, const double* cl,
                           const double* cs, double* rhs)
{
   Layout L(*m);
#pragma omp parallel for collapse(2) schedule(static)
   for (int k = 0; k < L.n2; k++)
      for (int j = 0; j < L.n1; j++)
         for (int i = 0; i < L.n0; i++) {
            const long ci = L.c(i, j, k);
            const double T = temperature_at(*m, temp, L, i, j, k);
            ThermoT th = thermo_at(*m, T);
            const double a = cl[ci], b = cs[ci];
            const double fl = free_energy(th, a, 0) * m->inv_molar_volume[0];
            const double fa = free_energy(th, b, 1) * m->inv_molar_volume[1];
            const double mu = dfdc(th, b, 1) * m->inv_molar_volume[1];
            const double hp = deriv_interp_func(phi[ci], m->energy_interp);
            rhs[L.interior(i, j, k)] += hp * ((fl - fa) - mu * (a - b));
         }
}

// PhaseConcentrationsStrategy::computePhaseConcentrationsOnPatch over the
// ghost box (CALPHADequilibriumPhaseConcentrationsStrategy.cc:325-452).
// Returns the summed iterations; *nfail receives failed cells.
long orc_phase_concentrations(const ampe_model_t* m, const double* temp,
                              const double* phi, const double* conc,
                              const double* clr, const double* csr,
                              double* cl, double* cs, long* nfail)
{
   Layout L(*m);
   long nits = 0, fails = 0;
#pragma omp parallel for collapse(2) reduction(+ : nits, fails) schedule(static)
   for (int k = -L.gz; k < L.n2 + L.gz; k++)
      for (int j = -L.ng; j < L.n1 + L.ng; j++)
         for (int i = -L.ng; i < L.n0 + L.ng; i++) {
            const long ci = L.c(i, j, k);
            const double T = temperature_at(*m, temp, L, i, j, k);
            ThermoT th = thermo_at(*m, T);
            const double h = interp_func(phi[ci], m->conc_interp);
            double x[2] = {clr[ci], csr[ci]};
            const int it = kks_newton(*m, th, h, conc[ci], x);
            if (it < 0) {
               fails++;
               nits += m->newton_max_its;
            } else {
               nits += it;
            }
            cl[ci] = x[0];
            cs[ci] = x[1];
         }
   if (nfail) *nfail = fails;
   return nits;
}

// concentration_pfmdiffusion_of_temperature (3d/concentrationdiffusion.m4:
// 310-428) on interior faces.
void orc_conc_diffusion(const ampe_model_t* m, const double* phi,
                        const double* temp, double* dl0, double* dl1,
                        double* dl2, double* ds0, double* ds1, double* ds2)
{
   Layout L(*m);
   const double qlR = m->Q_liquid / kGasR, qsR = m->Q_solid / kGasR;
   for (int dir = 0; dir < L.dim; dir++) {
      const int ei = dir == 0, ej = dir == 1, ek = dir == 2;
#pragma omp parallel for collapse(2) schedule(static)
      for (int k = 0; k < L.n2 + ek; k++)
         for (int j = 0; j < L.n1 + ej; j++)
            for (int i = 0; i < L.n0 + ei; i++) {
               const double vphi = average_func(phi[L.c(i - ei, j - ej, k - ek)],
                                                phi[L.c(i, j, k)], m->avg_type);
               const double hphi = interp_func(vphi, m->diff_interp);
               const double invT =
                   2.0 / (temperature_at(*m, temp, L, i - ei, j - ej, k - ek) +
                          temperature_at(*m, temp, L, i, j, k));
               const double dlq = m->D_liquid * std::exp(-qlR * invT);
               const double dsq = m->D_solid * std::exp(-qsR * invT);
               const long f = dir == 0 ? L.fx(i, j, k)
                                       : (dir == 1 ? L.fy(i, j, k) : L.fz(i, j, k));
               double* DL = dir == 0 ? dl0 : (dir == 1 ? dl1 : dl2);
               double* DS = dir == 0 ? ds0 : (dir == 1 ? ds1 : ds2);
               DL[f] = (1.0 - hphi) * dlq;
               DS[f] = hphi * dsq;
            }
   }
}

// Composition flux of the "kks" form (KKSCompositionRHSStrategy.cc:98-441):
// D0 = (1-h) D_L + h D_S with h = energy_interp(phibar) and T-dependent
// D_L, D_S (concentration_pfmdiffusion, 3d/concentrationdiffusion.m4:
// 14-128), the coupling D_phi = D0 h'(phibar) (cLbar - cSbar) with
// arithmetic means of cL, cS over the face (setDiffCoeffForPhaseOnPatch,
// KKSCompositionRHSStrategy.cc:166-310), and
// flux = (D0 (c_up - c_lo) + D_phi (phi_up - phi_lo)) / dx
// (concentrationflux, 3d/concentrationrhs.m4:14-104).  phid, cld, csd give
// the coefficients (lagged in finite-difference evaluations), phi and conc
// the differences.
void orc_conc_flux_kks(const ampe_model_t* m, const double* phid, const double* cld,
                       const double* csd, const double* temp, const double* phi,
                       const double* conc, double* f0, double* f1, double* f2)
{
   Layout L(*m);
   const double qlR = m->Q_liquid / kGasR, qsR = m->Q_solid / kGasR;
   for (int dir = 0; dir < L.dim; dir++) {
      const int ei = dir == 0, ej = dir == 1, ek = dir == 2;
      const double dinv = 1.0 / m->dx[dir];
#pragma omp parallel for collapse(2) schedule(static)
      for (int k = 0; k < L.n2 + ek; k++)
         for (int j = 0; j < L.n1 + ej; j++)
            for (int i = 0; i < L.n0 + ei; i++) {
               const long lo = L.c(i - ei, j - ej, k - ek), up = L.c(i, j, k);
               const double vphi = average_func(phid[lo], phid[up], m->avg_type);
               const double hphi = interp_func(vphi, m->energy_interp);
               const double invT =
                   2.0 / (temperature_at(*m, temp, L, i - ei, j - ej, k - ek) +
                          temperature_at(*m, temp, L, i, j, k));
               const double dlq = m->D_liquid * std::exp(-qlR * invT);
               const double dsq = m->D_solid * std::exp(-qsR * invT);
               const double d0 = (1.0 - hphi) * dlq + hphi * dsq;
               const double clb = 0.5 * (cld[up] + cld[lo]);
               const double csb = 0.5 * (csd[up] + csd[lo]);
               const double dphi = d0 * deriv_interp_func(vphi, m->energy_interp) * (clb - csb);
               const long f = dir == 0 ? L.fx(i, j, k)
                                       : (dir == 1 ? L.fy(i, j, k) : L.fz(i, j, k));
               double* F = dir == 0 ? f0 : (dir == 1 ? f1 : f2);
               F[f] = dinv * (d0 * (conc[up] - conc[lo]) + dphi * (phi[up] - phi[lo]));
            }
   }
}

// add_flux (2d/flux.m4:11-58, 3d/flux.m4:15-100), depth 1
void orc_add_flux(const ampe_model_t* m, const double* u, const double* d0,
                  const double* d1, const double* d2, double* f0, double* f1,
                  double* f2)
{
   Layout L(*m);
   const double dxi = 1.0 / m->dx[0], dyi = 1.0 / m->dx[1];
   #pragma omp parallel for collapse(2) schedule(static)
   for (int k = 0; k < L.n2; k++)
      for (int j = 0; j < L.n1; j++)
         for (int i = 0; i <= L.n0; i++) {
            const long f = L.fx(i, j, k);
            f0[f] = f0[f] + dxi * d0[f] * (u[L.c(i, j, k)] - u[L.c(i - 1, j, k)]);
         }
   #pragma omp parallel for collapse(2) schedule(static)
   for (int k = 0; k < L.n2; k++)
      for (int j = 0; j <= L.n1; j++)
         for (int i = 0; i < L.n0; i++) {
            const long f = L.fy(i, j, k);
            f1[f] = f1[f] + dyi * d1[f] * (u[L.c(i, j, k)] - u[L.c(i, j - 1, k)]);
         }
   if (L.dim == 3) {
      const double dzi = 1.0 / m->dx[2];
      #pragma omp parallel for collapse(2) schedule(static)
      for (int k = 0; k <= L.n2; k++)
         for (int j = 0; j < L.n1; j++)
            for (int i = 0; i < L.n0; i++) {
               const long f = L.fz(i, j, k);
               f2[f] = f2[f] + dzi * d2[f] * (u[L.c(i, j, k)] - u[L.c(i, j, k - 1)]);
            }
   }
}

// computerhsconcentration (3d/concentrationrhs.m4:412-456)
void orc_computerhsconcentration(const ampe_model_t* m, const double* f0,
                                 const double* f1, const double* f2,
                                 double* rhs)
{
   Layout L(*m);
   const double dxi = 1.0 / m->dx[0], dyi = 1.0 / m->dx[1];
   const double dzi = L.dim == 3 ? 1.0 / m->dx[2] : 0.0;
#pragma omp parallel for collapse(2) schedule(static)
   for (int k = 0; k < L.n2; k++)
      for (int j = 0; j < L.n1; j++)
         for (int i = 0; i < L.n0; i++) {
            double s = dxi * (f0[L.fx(i + 1, j, k)] - f0[L.fx(i, j, k)]) +
                       dyi * (f1[L.fy(i, j + 1, k)] - f1[L.fy(i, j, k)]);
            if (L.dim == 3)
               s = dxi * (f0[L.fx(i + 1, j, k)] - f0[L.fx(i, j, k)]) +
                   dyi * (f1[L.fy(i, j + 1, k)] - f1[L.fy(i, j, k)]) +
                   dzi * (f2[L.fz(i, j, k + 1)] - f2[L.fz(i, j, k)]);
            rhs[L.interior(i, j, k)] = m->conc_mobility * s;
         }
}

// Whole phi + c right-hand side for given (ghost-filled) phi, cl, cs:
// PhaseRHSStrategyWithQ::evaluateRHS (.cc:90-313) followed by
// QuatIntegrator::evaluateConcentrationRHS (QuatIntegrator.cc:2578-2689).
// phi_d: phase field used for the face diffusivities (lagged in
// finite-difference Jacobian evaluations); outputs are interior arrays.
void orc_rhs_phase_conc(const ampe_model_t* m, const double* phi,
                        const double* quat, const double* temp,
                        const double* cl, const double* cs,
                        const double* phi_d, double* phi_rhs,
                        double* conc_rhs)
{
   ampe_model_t mm = *m;
   mm.with_orient = 0;
   orc_rhs_phase_conc_q(&mm, phi, quat, temp, cl, cs, phi_d, nullptr, phi_rhs,
                        conc_rhs);
}

// as orc_rhs_phase_conc, with the orientation term of COMPUTERHSPBG
// (3d/quatrhs.m4:481-509) from the cell modulus |grad q| when with_orient
void orc_rhs_phase_conc_q(const ampe_model_t* m, const double* phi,
                          const double* quat, const double* temp,
                          const double* cl, const double* cs,
                          const double* phi_d, const double* ogm,
                          double* phi_rhs, double* conc_rhs)
{
   orc_rhs_phase_conc_qd(m, phi, quat, temp, cl, cs, phi_d, cl, cs, ogm, phi_rhs,
                         conc_rhs);
}

// QuatModel.cc:375-395 / CompositionDiffusionStrategyFactory.h:36-95: the
// "ebs" form's diffusivities, temperature_dependent or composition_dependent
void orc_conc_diffusion_model(const ampe_model_t* m, const double* phi,
                              const double* temp, const double* cl_d,
                              const double* cs_d, double* dl0, double* dl1,
                              double* dl2, double* ds0, double* ds1, double* ds2)
{
   if (m->conc_diffusion == AMPE_DIFF_MOBILITY)
      orc_conc_diffusion_mobility(m, &m->mobility, phi, temp, cl_d, cs_d, dl0, dl1, dl2,
                                  ds0, ds1, ds2, nullptr, nullptr, nullptr, nullptr,
                                  nullptr, nullptr);
   else
      orc_conc_diffusion(m, phi, temp, dl0, dl1, dl2, ds0, ds1, ds2);
}

void orc_rhs_phase_conc_qd(const ampe_model_t* m, const double* phi,
                           const double* quat, const double* temp,
                           const double* cl, const double* cs,
                           const double* phi_d, const double* cl_d,
                           const double* cs_d, const double* ogm,
                           double* phi_rhs, double* conc_rhs)
{
   Layout L(*m);
   std::vector<double> f0(L.nfx()), f1(L.nfy()), f2(L.dim == 3 ? L.nfz() : 1);
   orc_phase_flux(m, phi, quat, f0.data(), f1.data(), f2.data());
   orc_computerhspbg(m, f0.data(), f1.data(), f2.data(), temp, phi, ogm,
                     phi_rhs);
   orc_add_driving_force(m, temp, phi, cl, cs, phi_rhs);
   const long N = L.cells();
   for (long c = 0; c < N; c++) phi_rhs[c] *= m->phase_mobility;

   std::vector<double> dl0(L.nfx()), dl1(L.nfy()), dl2(f2.size());
   std::vector<double> ds0(L.nfx()), ds1(L.nfy()), ds2(f2.size());
   orc_conc_diffusion_model(m, phi_d ? phi_d : phi, temp, cl_d, cs_d, dl0.data(),
                            dl1.data(), dl2.data(), ds0.data(), ds1.data(), ds2.data());
   std::fill(f0.begin(), f0.end(), 0.0);
   std::fill(f1.begin(), f1.end(), 0.0);
   std::fill(f2.begin(), f2.end(), 0.0);
   orc_add_flux(m, cl, dl0.data(), dl1.data(), dl2.data(), f0.data(),
                f1.data(), f2.data());
   orc_add_flux(m, cs, ds0.data(), ds1.data(), ds2.data(), f0.data(),
                f1.data(), f2.data());
   orc_computerhsconcentration(m, f0.data(), f1.data(), f2.data(), conc_rhs);
}

// Analytic Jacobian-vector product of the phi + c right-hand side at the
// state (phi, cL, cS) (ghosted) with the face diffusivities held fixed:
//   J [da; db] = [dc - (b - a) h_c'(phi) dphi; 0]            (KKS split)
//   d(phi') = M [div(eps^2 grad dphi) - w g'' dphi + h_e'' dF dphi
//                + h_e' (-f_S''(b) (a - b)) db]
//   d(c')   = M_c div(D_L grad da + D_S grad db)
// out = v - gamma J v; v, out interior [dphi | dc].  Simple / isotropic
// flux only.
void orc_jv_analytic(const ampe_model_t* m, const double* phi,
                     const double* cl, const double* cs, const double* v,
                     double gamma, double* out)
{
   Layout L(*m);
   const long N = L.cells(), NG = L.cells_ghost();
   std::vector<double> dp(NG), da(NG), db(NG);
#pragma omp parallel for collapse(2) schedule(static)
   for (int k = 0; k < L.n2; k++)
      for (int j = 0; j < L.n1; j++)
         for (int i = 0; i < L.n0; i++) {
            const long c = L.c(i, j, k), t = L.interior(i, j, k);
            ThermoT th = thermo_at(*m, temperature_at(*m, nullptr, L, i, j, k));
            const double a = cl[c], b = cs[c], p = phi[c];
            const double h = interp_func(p, m->conc_interp);
            const double J00 = 1.0 - h, J01 = h;
            const double J10 = 1.0 / (a * (1.0 - a)) + dxi(th, a, 0) / th.RT;
            const double J11 = -1.0 / (b * (1.0 - b)) - dxi(th, b, 1) / th.RT;
            const double det = J00 * J11 - J01 * J10;
            const double r0 = v[t + N] - (b - a) * deriv_interp_func(p, m->conc_interp) * v[t];
            dp[c] = v[t];
            da[c] = J11 * r0 / det;
            db[c] = -J10 * r0 / det;
         }
   orc_fill_ghosts(m, dp.data());
   orc_fill_ghosts(m, da.data());
   orc_fill_ghosts(m, db.data());
   // phase part: linear flux of dphi + pointwise terms.  The product is
   // defined for the linear (simple, isotropic) fluxes only: for the
   // anisotropic flux the phase rows are NaN (not available) and the
   // composition rows are still formed.
   const bool linear_flux = m->flux_type != AMPE_FLUX_ANISOTROPIC;
   std::vector<double> f0(L.nfx()), f1(L.nfy()), f2(L.dim == 3 ? L.nfz() : 1);
   if (linear_flux) orc_phase_flux(m, dp.data(), nullptr, f0.data(), f1.data(), f2.data());
   std::vector<double> lap(N);
   ampe_model_t m0 = *m;
   m0.phase_well_scale = 0.0;
   m0.with_orient = 0;
   orc_computerhspbg(&m0, f0.data(), f1.data(), f2.data(), nullptr, dp.data(),
                     nullptr, lap.data());
   // composition part
   std::vector<double> l0(L.nfx()), l1(L.nfy()), l2(f2.size());
   std::vector<double> s0(L.nfx()), s1(L.nfy()), s2(f2.size());
   orc_conc_diffusion_model(m, phi, nullptr, cl, cs, l0.data(), l1.data(), l2.data(),
                            s0.data(), s1.data(), s2.data());
   std::fill(f0.begin(), f0.end(), 0.0);
   std::fill(f1.begin(), f1.end(), 0.0);
   std::fill(f2.begin(), f2.end(), 0.0);
   orc_add_flux(m, da.data(), l0.data(), l1.data(), l2.data(), f0.data(),
                f1.data(), f2.data());
   orc_add_flux(m, db.data(), s0.data(), s1.data(), s2.data(), f0.data(),
                f1.data(), f2.data());
   if (m->conc_form == AMPE_CONC_KKS) {
      // "kks" form: flux linear in (c, phi) with the coefficients held
      std::vector<double> dcv(NG);
      for (int k = 0; k < L.n2; k++)
         for (int j = 0; j < L.n1; j++)
            for (int i = 0; i < L.n0; i++)
               dcv[L.c(i, j, k)] = v[L.interior(i, j, k) + N];
      orc_fill_ghosts(m, dcv.data());
      orc_conc_flux_kks(m, phi, cl, cs, nullptr, dp.data(), dcv.data(), f0.data(), f1.data(),
                        f2.data());
   }
   std::vector<double> jc(N);
   orc_computerhsconcentration(m, f0.data(), f1.data(), f2.data(), jc.data());
#pragma omp parallel for collapse(2) schedule(static)
   for (int k = 0; k < L.n2; k++)
      for (int j = 0; j < L.n1; j++)
         for (int i = 0; i < L.n0; i++) {
            const long c = L.c(i, j, k), t = L.interior(i, j, k);
            ThermoT th = thermo_at(*m, temperature_at(*m, nullptr, L, i, j, k));
            const double a = cl[c], b = cs[c], p = phi[c];
            const double fl = free_energy(th, a, 0) * m->inv_molar_volume[0];
            const double fa = free_energy(th, b, 1) * m->inv_molar_volume[1];
            const double mu = dfdc(th, b, 1) * m->inv_molar_volume[1];
            const double dF = (fl - fa) - mu * (a - b);
            const double ddF = -d2fdc2(th, b, 1) * (a - b) * m->inv_molar_volume[1] * db[c];
            const double jp =
                m->phase_mobility *
                (lap[t] - m->phase_well_scale * second_deriv_well_func(p, m->well_type) * v[t] +
                 second_deriv_interp_func(p, m->energy_interp) * dF * v[t] +
                 deriv_interp_func(p, m->energy_interp) * ddF);
            out[t] = linear_flux ? v[t] - gamma * jp : std::nan("");
            out[t + N] = v[t + N] - gamma * jc[t];
         }
}


// addconcentrationfluxfromgradt (3d/concentrationrhs.m4:460-535,
// 2d/concentrationrhs.m4:369-437): loops of the reference, one face
// direction after the other
void orc_add_flux_from_grad_t(const ampe_model_t* m, const double* T, const double* q0,
                              const double* q1, const double* q2, double* f0, double* f1,
                              double* f2)
{
   Layout L(*m);
   const double dxinv = 1.0 / m->dx[0], dyinv = 1.0 / m->dx[1];
   for (int k = 0; k < L.n2; k++)
      for (int j = 0; j < L.n1; j++)
         for (int i = 0; i <= L.n0; i++) {
            const double sideT = average_func(T[L.c(i - 1, j, k)], T[L.c(i, j, k)], m->avg_type);
            const long f = L.fx(i, j, k);
            f0[f] = f0[f] - dxinv * q0[f] * ((T[L.c(i, j, k)] - T[L.c(i - 1, j, k)]) / sideT);
         }
   for (int k = 0; k < L.n2; k++)
      for (int j = 0; j <= L.n1; j++)
         for (int i = 0; i < L.n0; i++) {
            const double sideT = average_func(T[L.c(i, j - 1, k)], T[L.c(i, j, k)], m->avg_type);
            const long f = L.fy(i, j, k);
            f1[f] = f1[f] - dyinv * q1[f] * ((T[L.c(i, j, k)] - T[L.c(i, j - 1, k)]) / sideT);
         }
   if (L.dim == 3) {
      const double dzinv = 1.0 / m->dx[2];
      for (int k = 0; k <= L.n2; k++)
         for (int j = 0; j < L.n1; j++)
            for (int i = 0; i < L.n0; i++) {
               const double sideT =
                   average_func(T[L.c(i, j, k - 1)], T[L.c(i, j, k)], m->avg_type);
               const long f = L.fz(i, j, k);
               f2[f] = f2[f] - dzinv * q2[f] * ((T[L.c(i, j, k)] - T[L.c(i, j, k - 1)]) / sideT);
            }
   }
}

// addconcentrationfluxfromantitrapping, one composition
// (3d/concentrationrhs.m4:537-700, 2d/concentrationrhs.m4:439-527)
void orc_add_flux_from_antitrapping(const ampe_model_t* m, const double* phase,
                                    const double* cl, const double* ca, const double* dphidt,
                                    double alpha, double* f0, double* f1, double* f2)
{
   Layout L(*m);
   const bool d3 = L.dim == 3;
   const double tol = (double)1.e-8f, tol2 = tol * tol;
   const double dxinv = 1.0 / m->dx[0], dyinv = 1.0 / m->dx[1];
   const double dzinv = d3 ? 1.0 / m->dx[2] : 0.0;
   auto P = [&](int i, int j, int k) { return phase[L.c(i, j, k)]; };
   auto add = [&](double* F, long f, long cm, long c, double dn, double d2) {
      if (std::fabs(d2) > tol2) {
         const double dphin = std::sqrt(d2);
         const double dpdt = 0.5 * (dphidt[cm] + dphidt[c]);
         const double acl = 0.5 * (cl[cm] + cl[c]);
         const double aca = 0.5 * (ca[cm] + ca[c]);
         F[f] = F[f] + alpha * (dn / dphin) * (acl - aca) * dpdt;
      }
   };
   for (int k = 0; k < L.n2; k++)
      for (int j = 0; j < L.n1; j++)
         for (int i = 0; i <= L.n0; i++) {
            const double dphix = dxinv * (P(i, j, k) - P(i - 1, j, k));
            double dphiy, dphiz = 0.0;
            if (d3) {
               dphiy = dyinv * 0.25 * (P(i, j + 1, k) - P(i, j - 1, k) + P(i - 1, j + 1, k) -
                                       P(i - 1, j - 1, k));
               dphiz = dzinv * 0.25 * (P(i, j, k + 1) - P(i, j, k - 1) + P(i - 1, j, k + 1) -
                                       P(i - 1, j, k - 1));
            } else {
               dphiy = dyinv * 0.25 * (P(i - 1, j + 1, k) - P(i - 1, j - 1, k) + P(i, j + 1, k) -
                                       P(i, j - 1, k));
            }
            const double d2 = d3 ? dphix * dphix + dphiy * dphiy + dphiz * dphiz
                                 : dphix * dphix + dphiy * dphiy;
            add(f0, L.fx(i, j, k), L.c(i - 1, j, k), L.c(i, j, k), dphix, d2);
         }
   for (int k = 0; k < L.n2; k++)
      for (int j = 0; j <= L.n1; j++)
         for (int i = 0; i < L.n0; i++) {
            const double dphiy = dyinv * (P(i, j, k) - P(i, j - 1, k));
            const double dphix = dxinv * 0.25 * (P(i + 1, j - 1, k) - P(i - 1, j - 1, k) +
                                                  P(i + 1, j, k) - P(i - 1, j, k));
            double dphiz = 0.0;
            if (d3)
               dphiz = dzinv * 0.25 * (P(i, j - 1, k + 1) - P(i, j - 1, k - 1) + P(i, j, k + 1) -
                                       P(i, j, k - 1));
            const double d2 = d3 ? dphix * dphix + dphiy * dphiy + dphiz * dphiz
                                 : dphix * dphix + dphiy * dphiy;
            add(f1, L.fy(i, j, k), L.c(i, j - 1, k), L.c(i, j, k), dphiy, d2);
         }
   if (d3) {
      for (int k = 0; k <= L.n2; k++)
         for (int j = 0; j < L.n1; j++)
            for (int i = 0; i < L.n0; i++) {
               const double dphiz = dzinv * (P(i, j, k) - P(i, j, k - 1));
               const double dphix = dxinv * 0.25 * (P(i + 1, j, k - 1) - P(i - 1, j, k - 1) +
                                                     P(i + 1, j, k) - P(i - 1, j, k));
               const double dphiy = dyinv * 0.25 * (P(i, j + 1, k - 1) - P(i, j - 1, k - 1) +
                                                     P(i, j + 1, k) - P(i, j - 1, k));
               const double d2 = dphix * dphix + dphiy * dphiy + dphiz * dphiz;
               add(f2, L.fz(i, j, k), L.c(i, j, k - 1), L.c(i, j, k), dphiz, d2);
            }
   }
}

// KimMobilityStrategyInfMob::evaluateMobility (KimMobilityStrategyInfMob.cc:
// 49-80) with kks_mobility_factor (KKStools.cc:13-30), binary, over the
// ghost box (KimMobilityStrategy.cc:204-300); factor given by the caller
void orc_kim_mobility(const ampe_model_t* m, const double* tfield, const double* cl,
                      const double* cs, double factor, double D0, double Q0, double mv,
                      double* mob)
{
   Layout L(*m);
   for (int k = -L.gz; k < L.n2 + L.gz; k++)
      for (int j = -L.ng; j < L.n1 + L.ng; j++)
         for (int i = -L.ng; i < L.n0 + L.ng; i++) {
            const long c = L.c(i, j, k);
            const double T = temperature_at(*m, tfield, L, i, j, k);
            const double d2f = d2fdc2(thermo_at(*m, T), cl[c], 0);
            const double DL = D0 * std::exp(-Q0 / (kGasR * T));
            double zeta = (cl[c] - cs[c]) * d2f * (cl[c] - cs[c]);
            zeta = zeta / DL;
            zeta *= 1.e-6 / mv;
            mob[c] = factor / zeta;
         }
}


// Composition-dependent diffusion from CALPHAD atomic mobilities, binary
// (MobilityCompositionDiffusionStrategy.cc:180-611 setDiffCoeffInEachPhase-
// OnPatch and setPFMDiffOnPatch; mobility matrix of
// computeDiffusionMobilityBinaryPhase, CALPHADMobility.cc:196-215; atomic
// mobility and dG of CALPHADMobility.h:70-115 and .cc:152-162; the
// diffusion matrix is the mobility times the J/mol free-energy curvature,
// computeLocalDiffusionMatrixL/A, .cc:46-80).
static double orc_mob_q(const double* a, double T)
{
   return a[0] + kGasR * T * std::log(a[1]) + a[2] * T * std::log(T) + a[3] / T;
}

static double orc_mob_qq(const double* a, double T)
{
   return a[0] + kGasR * T * std::log(a[1]);
}

static double orc_atomic_mobility(const ampe_mobility_t& mb, int s, int p, double c0,
                                  double c1, double T)
{
   const double dc = c0 - c1;
   const double dG =
       c0 * orc_mob_q(mb.q[s][p][0], T) + c1 * orc_mob_q(mb.q[s][p][1], T) +
       c0 * c1 *
           (orc_mob_qq(mb.qq[s][p][0], T) +
            dc * (orc_mob_qq(mb.qq[s][p][1], T) +
                  dc * (orc_mob_qq(mb.qq[s][p][2], T) + dc * orc_mob_qq(mb.qq[s][p][3], T))));
   const double rtinv = 1.0 / (kGasR * T);
   return std::exp(dG * rtinv) * rtinv;
}

double orc_phase_diffusion_mobility(const ampe_model_t* m, const ampe_mobility_t* mb, int p,
                                    double c, double T)
{
   const double c1 = 1.0 - c;
   const double m0 = orc_atomic_mobility(*mb, 0, p, c, c1, T);
   const double m1 = orc_atomic_mobility(*mb, 1, p, c, c1, T);
   const double mm = c * m1 + c1 * m0;
   return c * c1 * mm * 1.e12 * d2fdc2(thermo_at(*m, T), c, p);
}

void orc_conc_diffusion_mobility(const ampe_model_t* m, const ampe_mobility_t* mb,
                                 const double* phi, const double* temp, const double* cl,
                                 const double* cs, double* dl0, double* dl1, double* dl2,
                                 double* ds0, double* ds1, double* ds2, double* el0,
                                 double* el1, double* el2, double* es0, double* es1,
                                 double* es2)
{
   Layout L(*m);
   for (int dir = 0; dir < L.dim; dir++) {
      const int ei = dir == 0, ej = dir == 1, ek = dir == 2;
      double* DL = dir == 0 ? dl0 : (dir == 1 ? dl1 : dl2);
      double* DS = dir == 0 ? ds0 : (dir == 1 ? ds1 : ds2);
      double* EL = dir == 0 ? el0 : (dir == 1 ? el1 : el2);
      double* ES = dir == 0 ? es0 : (dir == 1 ? es1 : es2);
#pragma omp parallel for collapse(2) schedule(static)
      for (int k = 0; k < L.n2 + ek; k++)
         for (int j = 0; j < L.n1 + ej; j++)
            for (int i = 0; i < L.n0 + ei; i++) {
               const long hi = L.c(i, j, k), lo = L.c(i - ei, j - ej, k - ek);
               const double T = 0.5 * (temperature_at(*m, temp, L, i, j, k) +
                                       temperature_at(*m, temp, L, i - ei, j - ej, k - ek));
               const double dlc = orc_phase_diffusion_mobility(m, mb, 0,
                                                               0.5 * (cl[hi] + cl[lo]), T);
               const double dsc = orc_phase_diffusion_mobility(m, mb, 1,
                                                               0.5 * (cs[hi] + cs[lo]), T);
               const double hphi =
                   interp_func(average_func(phi[hi], phi[lo], m->avg_type), m->diff_interp);
               const long f = dir == 0 ? L.fx(i, j, k)
                                       : (dir == 1 ? L.fy(i, j, k) : L.fz(i, j, k));
               DL[f] = (1.0 - hphi) * dlc;
               DS[f] = hphi * dsc;
               if (EL) EL[f] = dlc;
               if (ES) ES[f] = dsc;
            }
   }
}

}  // extern "C"
