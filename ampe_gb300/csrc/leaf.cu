// Leaf kernels of libampe_gb300: one CUDA kernel per reference Fortran /
// C++ routine that the C-ABI replaces (see include/ampe_gb300.h for the
// reference file:line of each).  They keep the reference's data layout
// (ghosted cell arrays, ghost-free side arrays) so that a SAMRAI adapter can
// hand them patch data directly.  The fused hot-path kernels live in
// fused.cu; these are the drop-in / parity surface.
#include <atomic>
#include <cstdio>

#include "common.cuh"
#include "fac.cuh"
#include "phase_flux.cuh"

namespace ampe {

long long g_launches = 0;

int device_sms()
{
   constexpr int kDevs = 64;
   static std::atomic<int> sms[kDevs];
   int dev = 0;
   if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kDevs) dev = -1;
   if (dev >= 0) {
      const int v = sms[dev].load(std::memory_order_relaxed);
      if (v > 0) return v;
   }
   int n = 0;
   if (dev < 0 || cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) !=
                      cudaSuccess || n < 1)
      return 152;  // no device to ask: the GB300's count (launches fail anyway)
   sms[dev].store(n, std::memory_order_relaxed);
   return n;
}

int check_model(const ampe_model_t* m)
{
   if (!m) return AMPE_ERR_INVALID;
   if (m->dim != 2 && m->dim != 3) return AMPE_ERR_INVALID;
   if (m->ng < 1) return AMPE_ERR_INVALID;
   const int nd = m->dim;
   for (int d = 0; d < nd; d++)
      if (m->n[d] < 2 * m->ng || m->dx[d] <= 0.0) return AMPE_ERR_INVALID;
   if (m->dim == 2 && m->n[2] != 1) return AMPE_ERR_INVALID;
   if (m->flux_type == AMPE_FLUX_ISOTROPIC && m->dim == 3)
      return AMPE_ERR_INVALID;  // 3d/quatrhs.m4:90-92 stops: no 3D variant
   // kernels split linear cell and face indices with 31-bit arithmetic
   const long long lim = (1LL << 31) - 1;
   const long long e0 = m->n[0], e1 = m->n[1], e2 = m->dim == 3 ? m->n[2] : 1;
   const long long gz = m->dim == 3 ? m->ng : 0;
   const long long ghost = (e0 + 2 * m->ng) * (e1 + 2 * m->ng) * (e2 + 2 * gz);
   if (m->ng_side < 0) return AMPE_ERR_INVALID;
   const long long s = m->ng_side, sz = m->dim == 3 ? s : 0;
   const long long faces = (e0 + 1 + 2 * s) * (e1 + 2 * s) * (e2 + 2 * sz) +
                           (e0 + 2 * s) * (e1 + 1 + 2 * s) * (e2 + 2 * sz) +
                           (e0 + 2 * s) * (e1 + 2 * s) * (e2 + 1 + 2 * sz);
   if (ghost > lim || faces > lim) return AMPE_ERR_TOO_LARGE;
   if (m->conc_diffusion != AMPE_DIFF_ARRHENIUS && m->conc_diffusion != AMPE_DIFF_MOBILITY)
      return AMPE_ERR_INVALID;
   if (m->conc_diffusion == AMPE_DIFF_MOBILITY && check_mobility(&m->mobility))
      return AMPE_ERR_INVALID;
   return AMPE_OK;
}

// the logarithms of the mobility terms need a1 > 0
int check_mobility(const ampe_mobility_t* mob)
{
   if (!mob) return AMPE_ERR_INVALID;
   for (int s = 0; s < 2; s++)
      for (int p = 0; p < 2; p++) {
         for (int i = 0; i < 2; i++)
            if (!(mob->q[s][p][i][1] > 0.0)) return AMPE_ERR_INVALID;  // ln(a1)
         for (int n = 0; n < 4; n++)
            if (!(mob->qq[s][p][n][1] > 0.0)) return AMPE_ERR_INVALID;
      }
   return AMPE_OK;
}

// ---------------------------------------------------------------------------
// periodic ghost fill
// ---------------------------------------------------------------------------
int fill_ghosts(const Grid& g, double* f, cudaStream_t s)
{
   return fill_ghosts_t<double>(g, f, s);
}

// ---------------------------------------------------------------------------
// phase fluxes
// ---------------------------------------------------------------------------
__global__ void k_phase_flux(ampe_model_t m, Grid g, const double* ph,
                             const double* quat, double* f0, double* f1,
                             double* f2)
{
   const long long qs = g.cells_ghost();
   auto P = [&](int a, int b, int c) { return ph[g.c(a, b, c)]; };
   auto Q = [&](int comp, int a, int b, int c) {
      return quat[comp * qs + g.c(a, b, c)];
   };
   const long long nx = g.nfx(), ny = g.nfy();
   const long long nz = g.dim == 3 ? g.nfz() : 0;
   const long long tot = nx + ny + nz;
   for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
        t < tot; t += (long long)gridDim.x * blockDim.x) {
      int dir, i, j, k;
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
      const double v = phase_face_flux(m, g.dim, dir, i, j, k, P, Q);
      if (dir == 0) f0[g.fx(i, j, k)] = v;
      if (dir == 1) f1[g.fy(i, j, k)] = v;
      if (dir == 2) f2[g.fz(i, j, k)] = v;
   }
}

// ---------------------------------------------------------------------------
// computerhspbg, driving force, composition kernels
// ---------------------------------------------------------------------------
__global__ void k_computerhspbg(ampe_model_t m, Grid g, const double* f0,
                                const double* f1, const double* f2,
                                const double* temp, const double* phi,
                                const double* ogm, double* rhs)
{
   const double dxi = 1.0 / m.dx[0], dyi = 1.0 / m.dx[1];
   const double dzi = g.dim == 3 ? 1.0 / m.dx[2] : 0.0;
   const double eq2 = 0.5 * m.epsilon_q * m.epsilon_q;
   for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
        t < g.cells(); t += (long long)gridDim.x * blockDim.x) {
      int i, j, k;
      g.ijk(t, i, j, k);
      double d = (f0[g.fx(i + 1, j, k)] - f0[g.fx(i, j, k)]) * dxi +
                 (f1[g.fy(i, j + 1, k)] - f1[g.fy(i, j, k)]) * dyi;
      if (g.dim == 3) d = d + (f2[g.fz(i, j, k + 1)] - f2[g.fz(i, j, k)]) * dzi;
      const double p = phi[g.c(i, j, k)];
      double r = d - m.phase_well_scale * deriv_well_func(p, m.well_type);
      if (m.with_orient) {
         const double p1 = deriv_interp_func(p, m.orient_interp1);
         const double p2 = deriv_interp_func(p, m.orient_interp2);
         const double gm = ogm[t];
         const double T = temperature_at(m, g, temp, i, j, k);
         r = r - m.misorientation_factor * T * p1 * gm - p2 * eq2 * gm * gm;
      }
      rhs[t] = r;
   }
}

__global__ void k_add_driving_force(ampe_model_t m, Grid g,
                                    const double* temp, const double* phi,
                                    const double* cl, const double* cs,
                                    double* rhs)
{
   for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
        t < g.cells(); t += (long long)gridDim.x * blockDim.x) {
      int i, j, k;
      g.ijk(t, i, j, k);
      const long long ci = g.c(i, j, k);
      const ThermoCoef th = thermo_coef(m, temperature_at(m, g, temp, i, j, k));
      const double a = cl[ci], b = cs[ci];
      const double fl = free_energy_of(th, a, 0) * m.inv_molar_volume[0];
      const double fa = free_energy_of(th, b, 1) * m.inv_molar_volume[1];
      const double mu = dfdc_of(th, b, 1) * m.inv_molar_volume[1];
      const double hp = deriv_interp_func(phi[ci], m.energy_interp);
      rhs[t] += hp * ((fl - fa) - mu * (a - b));
   }
}

// per-cell KKS solve over the ghost box (reference loop bounds)
__global__ void k_phase_conc_ghostbox(ampe_model_t m, Grid g,
                                      const double* temp, const double* phi,
                                      const double* conc, const double* clr,
                                      const double* csr, double* cl,
                                      double* cs, unsigned long long* counters)
{
   const int ex = g.n0 + 2 * g.ng, ey = g.n1 + 2 * g.ng;
   const long long tot = g.cells_ghost();
   unsigned long long its = 0, fails = 0;
   for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
        t < tot; t += (long long)gridDim.x * blockDim.x) {
      const int i = (int)(t % ex) - g.ng;
      const int j = (int)((t / ex) % ey) - g.ng;
      const int k = (int)(t / ((long long)ex * ey)) - g.gz;
      const long long ci = g.c(i, j, k);
      const ThermoCoef th = thermo_coef(m, temperature_at(m, g, temp, i, j, k));
      const double h = interp_func(phi[ci], m.conc_interp);
      double x[2] = {clr[ci], csr[ci]};
      const int it = kks_newton(th, h, conc[ci], x, m.newton_max_its,
                                m.newton_tol);
      if (it < 0) {
         fails++;
         its += m.newton_max_its;
      } else {
         its += it;
      }
      cl[ci] = x[0];
      cs[ci] = x[1];
   }
   if (counters) {
      atomicAdd(&counters[0], its);
      atomicAdd(&counters[1], fails);
   }
}

// "kks" composition flux: concentration_pfmdiffusion (3d/concentrationdiffusion.m4:
// 14-128, energy interpolation of KKSCompositionRHSStrategy.cc:111), the
// coupling D0 h'(phibar)(cLbar - cSbar) (KKSCompositionRHSStrategy.cc:
// 166-310) and concentrationflux (3d/concentrationrhs.m4:14-104), fused
__global__ void k_conc_flux_kks(ampe_model_t m, Grid g, const double* phi,
                                const double* temp, const double* conc,
                                const double* cl, const double* cs, double* f0,
                                double* f1, double* f2)
{
   const double qlR = m.Q_liquid / kGasR, qsR = m.Q_solid / kGasR;
   const long long tot = g.nfx() + g.nfy() + (g.dim == 3 ? g.nfz() : 0);
   for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < tot;
        t += (long long)gridDim.x * blockDim.x) {
      int dir, i, j, k;
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
      const int ei = dir == 0, ej = dir == 1, ek = dir == 2;
      const long long lo = g.c(i - ei, j - ej, k - ek), up = g.c(i, j, k);
      const double vphi = average_func(phi[lo], phi[up], m.avg_type);
      const double hphi = interp_func(vphi, m.energy_interp);
      const double invT = 2.0 / (temperature_at(m, g, temp, i - ei, j - ej, k - ek) +
                                 temperature_at(m, g, temp, i, j, k));
      const double dlq = m.D_liquid * exp(-qlR * invT);
      const double dsq = m.D_solid * exp(-qsR * invT);
      const double d0 = (1.0 - hphi) * dlq + hphi * dsq;
      const double clb = 0.5 * (cl[up] + cl[lo]);
      const double csb = 0.5 * (cs[up] + cs[lo]);
      const double dph = d0 * deriv_interp_func(vphi, m.energy_interp) * (clb - csb);
      const double dinv = 1.0 / m.dx[dir];
      const double v = dinv * (d0 * (conc[up] - conc[lo]) + dph * (phi[up] - phi[lo]));
      if (dir == 0) f0[g.fx(i, j, k)] = v;
      if (dir == 1) f1[g.fy(i, j, k)] = v;
      if (dir == 2) f2[g.fz(i, j, k)] = v;
   }
}

__global__ void k_conc_diffusion(ampe_model_t m, Grid g, const double* phi,
                                 const double* temp, double* dl0, double* dl1,
                                 double* dl2, double* ds0, double* ds1,
                                 double* ds2)
{
   const double qlR = m.Q_liquid / kGasR, qsR = m.Q_solid / kGasR;
   const long long nx = g.nfx(), ny = g.nfy();
   const long long nz = g.dim == 3 ? g.nfz() : 0;
   for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
        t < nx + ny + nz; t += (long long)gridDim.x * blockDim.x) {
      int dir, i, j, k;
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
      const int ei = dir == 0, ej = dir == 1, ek = dir == 2;
      const double vphi = average_func(phi[g.c(i - ei, j - ej, k - ek)],
                                       phi[g.c(i, j, k)], m.avg_type);
      const double hphi = interp_func(vphi, m.diff_interp);
      const double invT = 2.0 / (temperature_at(m, g, temp, i - ei, j - ej, k - ek) +
                                 temperature_at(m, g, temp, i, j, k));
      const double dlq = m.D_liquid * exp(-qlR * invT);
      const double dsq = m.D_solid * exp(-qsR * invT);
      if (dir == 0) {
         dl0[g.fx(i, j, k)] = (1.0 - hphi) * dlq;
         ds0[g.fx(i, j, k)] = hphi * dsq;
      } else if (dir == 1) {
         dl1[g.fy(i, j, k)] = (1.0 - hphi) * dlq;
         ds1[g.fy(i, j, k)] = hphi * dsq;
      } else {
         dl2[g.fz(i, j, k)] = (1.0 - hphi) * dlq;
         ds2[g.fz(i, j, k)] = hphi * dsq;
      }
   }
}

__global__ void k_add_flux(ampe_model_t m, Grid g, const double* u,
                           const double* d0, const double* d1,
                           const double* d2, double* f0, double* f1,
                           double* f2)
{
   const long long nx = g.nfx(), ny = g.nfy();
   const long long nz = g.dim == 3 ? g.nfz() : 0;
   for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
        t < nx + ny + nz; t += (long long)gridDim.x * blockDim.x) {
      long long r = t;
      if (r < nx) {
         int i, j, k;
         g.split(r, g.fd0p, g.fd1, i, j, k);
         const int f = g.fx(i, j, k);
         f0[f] = f0[f] + (1.0 / m.dx[0]) * d0[f] *
                             (u[g.c(i, j, k)] - u[g.c(i - 1, j, k)]);
      } else if ((r -= nx) < ny) {
         int i, j, k;
         g.split(r, g.fd0, g.fd1p, i, j, k);
         const int f = g.fy(i, j, k);
         f1[f] = f1[f] + (1.0 / m.dx[1]) * d1[f] *
                             (u[g.c(i, j, k)] - u[g.c(i, j - 1, k)]);
      } else {
         r -= ny;
         int i, j, k;
         g.ijk(r, i, j, k);
         const int f = g.fz(i, j, k);
         f2[f] = f2[f] + (1.0 / m.dx[2]) * d2[f] *
                             (u[g.c(i, j, k)] - u[g.c(i, j, k - 1)]);
      }
   }
}

__global__ void k_rhs_conc(ampe_model_t m, Grid g, const double* f0,
                           const double* f1, const double* f2, double* rhs)
{
   const double dxi = 1.0 / m.dx[0], dyi = 1.0 / m.dx[1];
   const double dzi = g.dim == 3 ? 1.0 / m.dx[2] : 0.0;
   for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
        t < g.cells(); t += (long long)gridDim.x * blockDim.x) {
      int i, j, k;
      g.ijk(t, i, j, k);
      double s = dxi * (f0[g.fx(i + 1, j, k)] - f0[g.fx(i, j, k)]) +
                 dyi * (f1[g.fy(i, j + 1, k)] - f1[g.fy(i, j, k)]);
      if (g.dim == 3) s = s + dzi * (f2[g.fz(i, j, k + 1)] - f2[g.fz(i, j, k)]);
      rhs[t] = m.conc_mobility * s;
   }
}

// ADDCONCENTRATIONFLUXFROMGRADT (3d/concentrationrhs.m4:460-535,
// 2d/concentrationrhs.m4:369-437): the thermal-diffusion part of the flux,
// flux_d -= (1/dx_d) Mq_d ((T_i - T_{i-1}) / Tbar), Tbar the face average of
// T (average_func, avg_type)
__global__ void k_flux_grad_t(ampe_model_t m, Grid g, const double* T, const double* q0,
                              const double* q1, const double* q2, double* f0, double* f1,
                              double* f2)
{
   const long long nx = g.nfx(), ny = g.nfy();
   const long long nz = g.dim == 3 ? g.nfz() : 0;
   for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < nx + ny + nz;
        t += (long long)gridDim.x * blockDim.x) {
      long long r = t;
      int i, j, k, dir;
      if (r < nx) {
         g.split(r, g.fd0p, g.fd1, i, j, k);
         dir = 0;
      } else if ((r -= nx) < ny) {
         g.split(r, g.fd0, g.fd1p, i, j, k);
         dir = 1;
      } else {
         g.ijk(r - ny, i, j, k);
         dir = 2;
      }
      const int c = g.c(i, j, k);
      const int cm = dir == 0 ? g.c(i - 1, j, k) : (dir == 1 ? g.c(i, j - 1, k) : g.c(i, j, k - 1));
      const double sideT = average_func(T[cm], T[c], m.avg_type);
      const double dxi = 1.0 / m.dx[dir];
      double* F = dir == 0 ? f0 : (dir == 1 ? f1 : f2);
      const double* Q = dir == 0 ? q0 : (dir == 1 ? q1 : q2);
      const int f = dir == 0 ? g.fx(i, j, k) : (dir == 1 ? g.fy(i, j, k) : g.fz(i, j, k));
      F[f] = F[f] - dxi * Q[f] * ((T[c] - T[cm]) / sideT);
   }
}

// ADDCONCENTRATIONFLUXFROMANTITRAPPING for one composition
// (3d/concentrationrhs.m4:537-700, 2d/concentrationrhs.m4:439-527): on faces
// where |grad phi| > 1e-8, flux += alpha (dphi_n / |grad phi|) (cLbar -
// cSbar) dphidt_bar, the normal difference across the face and the
// tangential ones as the mean of the two cells' centred differences, in the
// reference's order of terms
__global__ void k_flux_antitrapping(ampe_model_t m, Grid g, const double* P,
                                    const double* cl, const double* cs, const double* dpdt,
                                    double alpha, double* f0, double* f1, double* f2)
{
   const long long nx = g.nfx(), ny = g.nfy();
   const long long nz = g.dim == 3 ? g.nfz() : 0;
   const double dxi = 1.0 / m.dx[0], dyi = 1.0 / m.dx[1];
   const double dzi = g.dim == 3 ? 1.0 / m.dx[2] : 0.0;
   const double tol = (double)1.e-8f;  // a default-real constant in the reference
   const double tol2 = tol * tol;
   for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < nx + ny + nz;
        t += (long long)gridDim.x * blockDim.x) {
      long long r = t;
      int i, j, k, dir;
      if (r < nx) {
         g.split(r, g.fd0p, g.fd1, i, j, k);
         dir = 0;
      } else if ((r -= nx) < ny) {
         g.split(r, g.fd0, g.fd1p, i, j, k);
         dir = 1;
      } else {
         g.ijk(r - ny, i, j, k);
         dir = 2;
      }
      auto p = [&](int a, int b, int cc) { return P[g.c(a, b, cc)]; };
      double gx, gy, gz = 0.0, gn;
      int cm;
      if (dir == 0) {
         gx = dxi * (p(i, j, k) - p(i - 1, j, k));
         if (g.dim == 3) {
            gy = dyi * 0.25 * (p(i, j + 1, k) - p(i, j - 1, k) + p(i - 1, j + 1, k) -
                               p(i - 1, j - 1, k));
            gz = dzi * 0.25 * (p(i, j, k + 1) - p(i, j, k - 1) + p(i - 1, j, k + 1) -
                               p(i - 1, j, k - 1));
         } else {
            gy = dyi * 0.25 * (p(i - 1, j + 1, k) - p(i - 1, j - 1, k) + p(i, j + 1, k) -
                               p(i, j - 1, k));
         }
         gn = gx;
         cm = g.c(i - 1, j, k);
      } else if (dir == 1) {
         gy = dyi * (p(i, j, k) - p(i, j - 1, k));
         gx = dxi * 0.25 * (p(i + 1, j - 1, k) - p(i - 1, j - 1, k) + p(i + 1, j, k) -
                            p(i - 1, j, k));
         if (g.dim == 3)
            gz = dzi * 0.25 * (p(i, j - 1, k + 1) - p(i, j - 1, k - 1) + p(i, j, k + 1) -
                               p(i, j, k - 1));
         gn = gy;
         cm = g.c(i, j - 1, k);
      } else {
         gz = dzi * (p(i, j, k) - p(i, j, k - 1));
         gx = dxi * 0.25 * (p(i + 1, j, k - 1) - p(i - 1, j, k - 1) + p(i + 1, j, k) -
                            p(i - 1, j, k));
         gy = dyi * 0.25 * (p(i, j + 1, k - 1) - p(i, j - 1, k - 1) + p(i, j + 1, k) -
                            p(i, j - 1, k));
         gn = gz;
         cm = g.c(i, j, k - 1);
      }
      double g2 = gx * gx + gy * gy;
      if (g.dim == 3) g2 = g2 + gz * gz;
      if (fabs(g2) > tol2) {
         const int c = g.c(i, j, k);
         const double dn = sqrt(g2);
         const double dt = 0.5 * (dpdt[cm] + dpdt[c]);
         const double acl = 0.5 * (cl[cm] + cl[c]);
         const double aca = 0.5 * (cs[cm] + cs[c]);
         double* F = dir == 0 ? f0 : (dir == 1 ? f1 : f2);
         const int f = dir == 0 ? g.fx(i, j, k) : (dir == 1 ? g.fy(i, j, k) : g.fz(i, j, k));
         F[f] = F[f] + alpha * (gn / dn) * (acl - aca) * dt;
      }
   }
}

// KimMobilityStrategyInfMob::evaluateMobility (KimMobilityStrategyInfMob.cc:
// 49-80) for a binary alloy, per cell of the ghost box
// (KimMobilityStrategy::update, KimMobilityStrategy.cc:204-300):
// M_phi = factor / zeta, zeta = (cL - cS)^2 f_L''(cL) / D_L(T) x 1e-6 / Vm,
// D_L(T) = D0 exp(-Q0 / (R T)), factor = 16 w / (3 eps^2 a2)
// (kks_mobility_factor, KKStools.cc:13-30)
__global__ void k_kim_mobility(ampe_model_t m, Grid g, const double* tfield, const double* cl,
                               const double* cs, double factor, double D0, double Q0,
                               double ivm, double* mob)
{
   const int SX = g.n0 + 2 * g.ng, SY = g.n1 + 2 * g.ng;
   for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < g.cells_ghost();
        t += (long long)gridDim.x * blockDim.x) {
      const int i = (int)(t % SX) - g.ng;
      const int j = (int)((t / SX) % SY) - g.ng;
      const int k = (int)(t / ((long long)SX * SY)) - g.gz;
      const double T = temperature_at(m, g, tfield, i, j, k);
      const ThermoCoef th = thermo_coef(m, T);
      const double a = cl[t], b = cs[t];
      const double d2f = th.RT / (a * (1.0 - a)) + dxi_of(th, a, 0);
      const double DL = D0 * exp(-Q0 / (kGasR * T));
      double zeta = (a - b) * d2f * (a - b);
      zeta = zeta / DL;
      zeta *= ivm;
      mob[t] = factor / zeta;
   }
}

__global__ void k_conc_diffusion_mobility(ampe_model_t m, ampe_mobility_t mb, Grid g,
                                          const double* phi, const double* temp,
                                          const double* cl, const double* cs, double* dl0,
                                          double* dl1, double* dl2, double* ds0, double* ds1,
                                          double* ds2, double* el0, double* el1, double* el2,
                                          double* es0, double* es1, double* es2)
{
   const long long nx = g.nfx(), ny = g.nfy();
   const long long nz = g.dim == 3 ? g.nfz() : 0;
   for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < nx + ny + nz;
        t += (long long)gridDim.x * blockDim.x) {
      int dir, i, j, k;
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
      const int ei = dir == 0, ej = dir == 1, ek = dir == 2;
      const long long lo = g.c(i - ei, j - ej, k - ek), hi = g.c(i, j, k);
      const double T = 0.5 * (temperature_at(m, g, temp, i, j, k) +
                              temperature_at(m, g, temp, i - ei, j - ej, k - ek));
      const double DL = phase_diffusion(m, mb, 0, 0.5 * (cl[hi] + cl[lo]), T);
      const double DS = phase_diffusion(m, mb, 1, 0.5 * (cs[hi] + cs[lo]), T);
      const double hphi = interp_func(average_func(phi[hi], phi[lo], m.avg_type), m.diff_interp);
      const long long f = dir == 0 ? g.fx(i, j, k) : (dir == 1 ? g.fy(i, j, k) : g.fz(i, j, k));
      double* DLo = dir == 0 ? dl0 : (dir == 1 ? dl1 : dl2);
      double* DSo = dir == 0 ? ds0 : (dir == 1 ? ds1 : ds2);
      double* ELo = dir == 0 ? el0 : (dir == 1 ? el1 : el2);
      double* ESo = dir == 0 ? es0 : (dir == 1 ? es1 : es2);
      DLo[f] = (1.0 - hphi) * DL;
      DSo[f] = hphi * DS;
      if (ELo) ELo[f] = DL;
      if (ESo) ESo[f] = DS;
   }
}

}  // namespace ampe

using namespace ampe;

static cudaStream_t S(void* s) { return (cudaStream_t)s; }
static unsigned blocks_for(long long n)
{
   long long b = (n + 255) / 256;
   if (b > max_blocks(64)) b = max_blocks(64);
   return (unsigned)(b < 1 ? 1 : b);
}

extern "C" {

const char* ampe_version(void) { return "ampe_gb300 1.0 (sm_103a)"; }

int ampe_device_count(void)
{
   int n = 0;
   if (cudaGetDeviceCount(&n) != cudaSuccess) return 0;
   return n;
}

int ampe_fill_ghosts(const ampe_model_t* m, double* field, void* stream)
{
   if (check_model(m) || !field) return AMPE_ERR_INVALID;
   return fill_ghosts(make_grid(*m), field, S(stream));
}

int ampe_phase_flux(const ampe_model_t* m, const double* phase,
                    const double* quat, double* flux0, double* flux1,
                    double* flux2, void* stream)
{
   if (check_model(m) || !phase || !flux0 || !flux1) return AMPE_ERR_INVALID;
   if (m->dim == 3 && !flux2) return AMPE_ERR_INVALID;
   if (m->flux_type == AMPE_FLUX_ANISOTROPIC && !quat) return AMPE_ERR_INVALID;
   Grid g = make_grid(*m);
   const long long tot = g.nfx() + g.nfy() + (g.dim == 3 ? g.nfz() : 0);
   k_phase_flux<<<blocks_for(tot), 256, 0, S(stream)>>>(*m, g, phase, quat,
                                                        flux0, flux1, flux2);
   return launch_status();
}

int ampe_computerhspbg(const ampe_model_t* m, const double* flux0,
                       const double* flux1, const double* flux2,
                       const double* temp, const double* phi,
                       const double* ogm, double* rhs, void* stream)
{
   if (check_model(m) || !flux0 || !flux1 || !phi || !rhs)
      return AMPE_ERR_INVALID;
   if (m->with_orient && !ogm) return AMPE_ERR_INVALID;
   if (m->temp_mode == AMPE_TEMP_FIELD && m->with_orient && !temp)
      return AMPE_ERR_INVALID;
   Grid g = make_grid(*m);
   k_computerhspbg<<<blocks_for(g.cells()), 256, 0, S(stream)>>>(
       *m, g, flux0, flux1, flux2, temp, phi, ogm, rhs);
   return launch_status();
}

int ampe_add_driving_force(const ampe_model_t* m, const double* temp,
                           const double* phi, const double* cl,
                           const double* cs, double* rhs, void* stream)
{
   if (check_model(m) || !phi || !cl || !cs || !rhs) return AMPE_ERR_INVALID;
   if (m->temp_mode == AMPE_TEMP_FIELD && !temp) return AMPE_ERR_INVALID;
   Grid g = make_grid(*m);
   k_add_driving_force<<<blocks_for(g.cells()), 256, 0, S(stream)>>>(
       *m, g, temp, phi, cl, cs, rhs);
   return launch_status();
}

int ampe_phase_concentrations(const ampe_model_t* m, const double* temp,
                              const double* phi, const double* conc,
                              const double* cl_ref, const double* cs_ref,
                              double* cl, double* cs,
                              unsigned long long* counters, void* stream)
{
   if (check_model(m) || !phi || !conc || !cl_ref || !cs_ref || !cl || !cs)
      return AMPE_ERR_INVALID;
   if (m->temp_mode == AMPE_TEMP_FIELD && !temp) return AMPE_ERR_INVALID;
   if (m->newton_max_its < 1) return AMPE_ERR_INVALID;
   Grid g = make_grid(*m);
   k_phase_conc_ghostbox<<<blocks_for(g.cells_ghost()), 256, 0, S(stream)>>>(
       *m, g, temp, phi, conc, cl_ref, cs_ref, cl, cs, counters);
   return launch_status();
}

int ampe_conc_diffusion(const ampe_model_t* m, const double* phi,
                        const double* temp, double* dl0, double* dl1,
                        double* dl2, double* ds0, double* ds1, double* ds2,
                        void* stream)
{
   if (check_model(m) || !phi || !dl0 || !dl1 || !ds0 || !ds1)
      return AMPE_ERR_INVALID;
   if (m->dim == 3 && (!dl2 || !ds2)) return AMPE_ERR_INVALID;
   if (m->temp_mode == AMPE_TEMP_FIELD && !temp) return AMPE_ERR_INVALID;
   Grid g = make_grid(*m);
   const long long tot = g.nfx() + g.nfy() + (g.dim == 3 ? g.nfz() : 0);
   k_conc_diffusion<<<blocks_for(tot), 256, 0, S(stream)>>>(
       *m, g, phi, temp, dl0, dl1, dl2, ds0, ds1, ds2);
   return launch_status();
}

int ampe_conc_flux_kks(const ampe_model_t* m, const double* phi, const double* temp,
                       const double* conc, const double* cl, const double* cs,
                       double* flux0, double* flux1, double* flux2, void* stream)
{
   if (check_model(m) || !phi || !conc || !cl || !cs || !flux0 || !flux1)
      return AMPE_ERR_INVALID;
   if (m->dim == 3 && !flux2) return AMPE_ERR_INVALID;
   if (m->temp_mode == AMPE_TEMP_FIELD && !temp) return AMPE_ERR_INVALID;
   Grid g = make_grid(*m);
   const long long tot = g.nfx() + g.nfy() + (g.dim == 3 ? g.nfz() : 0);
   k_conc_flux_kks<<<blocks_for(tot), 256, 0, S(stream)>>>(*m, g, phi, temp, conc, cl, cs,
                                                           flux0, flux1, flux2);
   return launch_status();
}

int ampe_add_flux_from_grad_t(const ampe_model_t* m, const double* temp, const double* mq0,
                              const double* mq1, const double* mq2, double* flux0,
                              double* flux1, double* flux2, void* stream)
{
   if (check_model(m) || !temp || !mq0 || !mq1 || !flux0 || !flux1) return AMPE_ERR_INVALID;
   if (m->dim == 3 && (!mq2 || !flux2)) return AMPE_ERR_INVALID;
   Grid g = make_grid(*m);
   const long long tot = g.nfx() + g.nfy() + (g.dim == 3 ? g.nfz() : 0);
   k_flux_grad_t<<<blocks_for(tot), 256, 0, S(stream)>>>(*m, g, temp, mq0, mq1, mq2, flux0,
                                                         flux1, flux2);
   return launch_status();
}

int ampe_kim_mobility(const ampe_model_t* m, const double* temp, const double* cl,
                      const double* cs, double D0, double Q0, double molar_volume,
                      double* mobility, void* stream)
{
   if (check_model(m) || !cl || !cs || !mobility || !(molar_volume > 0.0) || !(D0 > 0.0))
      return AMPE_ERR_INVALID;
   if (m->temp_mode == AMPE_TEMP_FIELD && !temp) return AMPE_ERR_INVALID;
   double a2;
   if (m->energy_interp == 'p')
      a2 = 47.0 / 60.0;
   else if (m->energy_interp == 'h')
      a2 = 0.5;
   else
      return AMPE_ERR_INVALID;  // kks_mobility_factor: other types refused
   if (!(m->epsilon_phi > 0.0)) return AMPE_ERR_INVALID;
   const double factor =
       16.0 * m->phase_well_scale / (3.0 * m->epsilon_phi * m->epsilon_phi * a2);
   Grid g = make_grid(*m);
   k_kim_mobility<<<blocks_for(g.cells_ghost()), 256, 0, S(stream)>>>(
       *m, g, temp, cl, cs, factor, D0, Q0, 1.0e-6 / molar_volume, mobility);
   return launch_status();
}

int ampe_conc_diffusion_mobility(const ampe_model_t* m, const ampe_mobility_t* mob,
                                 const double* phi, const double* temp,
                                 const double* cl, const double* cs, double* dl0,
                                 double* dl1, double* dl2, double* ds0, double* ds1,
                                 double* ds2, double* coef_l0, double* coef_l1,
                                 double* coef_l2, double* coef_s0, double* coef_s1,
                                 double* coef_s2, void* stream)
{
   if (check_model(m) || !mob || !phi || !cl || !cs || !dl0 || !dl1 || !ds0 || !ds1)
      return AMPE_ERR_INVALID;
   if (m->dim == 3 && (!dl2 || !ds2)) return AMPE_ERR_INVALID;
   if (m->temp_mode == AMPE_TEMP_FIELD && !temp) return AMPE_ERR_INVALID;
   if (check_mobility(mob)) return AMPE_ERR_INVALID;
   Grid g = make_grid(*m);
   const long long tot = g.nfx() + g.nfy() + (g.dim == 3 ? g.nfz() : 0);
   k_conc_diffusion_mobility<<<blocks_for(tot), 256, 0, S(stream)>>>(
       *m, *mob, g, phi, temp, cl, cs, dl0, dl1, dl2, ds0, ds1, ds2, coef_l0, coef_l1,
       coef_l2, coef_s0, coef_s1, coef_s2);
   return launch_status();
}

int ampe_add_flux_from_antitrapping(const ampe_model_t* m, const double* phi,
                                    const double* cl, const double* cs, const double* dphidt,
                                    double alpha, double* flux0, double* flux1,
                                    double* flux2, void* stream)
{
   if (check_model(m) || !phi || !cl || !cs || !dphidt || !flux0 || !flux1)
      return AMPE_ERR_INVALID;
   if (m->dim == 3 && !flux2) return AMPE_ERR_INVALID;
   Grid g = make_grid(*m);
   const long long tot = g.nfx() + g.nfy() + (g.dim == 3 ? g.nfz() : 0);
   k_flux_antitrapping<<<blocks_for(tot), 256, 0, S(stream)>>>(*m, g, phi, cl, cs, dphidt,
                                                               alpha, flux0, flux1, flux2);
   return launch_status();
}

int ampe_add_flux(const ampe_model_t* m, const double* u, const double* d0,
                  const double* d1, const double* d2, double* flux0,
                  double* flux1, double* flux2, void* stream)
{
   if (check_model(m) || !u || !d0 || !d1 || !flux0 || !flux1)
      return AMPE_ERR_INVALID;
   if (m->dim == 3 && (!d2 || !flux2)) return AMPE_ERR_INVALID;
   Grid g = make_grid(*m);
   const long long tot = g.nfx() + g.nfy() + (g.dim == 3 ? g.nfz() : 0);
   k_add_flux<<<blocks_for(tot), 256, 0, S(stream)>>>(*m, g, u, d0, d1, d2,
                                                      flux0, flux1, flux2);
   return launch_status();
}

int ampe_computerhsconcentration(const ampe_model_t* m, const double* flux0,
                                 const double* flux1, const double* flux2,
                                 double* rhs, void* stream)
{
   if (check_model(m) || !flux0 || !flux1 || !rhs) return AMPE_ERR_INVALID;
   if (m->dim == 3 && !flux2) return AMPE_ERR_INVALID;
   Grid g = make_grid(*m);
   k_rhs_conc<<<blocks_for(g.cells()), 256, 0, S(stream)>>>(*m, g, flux0,
                                                            flux1, flux2, rhs);
   return launch_status();
}

}  // extern "C"
