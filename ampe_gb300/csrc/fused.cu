// Fused hot-path kernels of the phi + c implicit step (FP64 path).
//
//  k_kks_interior : per-cell KKS Newton for (cL, cS) on interior cells,
//                   written through to the periodic ghost images, plus the
//                   chemical driving force dF = (fL - fS) - muS (cL - cS)
//                   (PhaseConcentrationsStrategy + FreeEnergyStrategy::
//                   addDrivingForce, fused).
//  k_rhs_fused    : PhaseRHSStrategyWithQ::evaluateRHS (flux + well +
//                   h'(phi) dF, times M_phi) and the EBS composition RHS
//                   M_c div(D_L grad cL + D_S grad cS) in one pass.
#include "common.cuh"
#include "fused.cuh"
#include "phase_flux.cuh"

namespace ampe {

__global__ void k_thermo_table(ampe_model_t m, int n, ThermoCoef* tab)
{
   const int i = blockIdx.x * blockDim.x + threadIdx.x;
   if (i >= n) return;
   double T = m.T0;
   if (m.temp_mode == AMPE_TEMP_GRADIENT)
      T = m.T0 + m.gradT * ((double)i + 0.5) * m.dx[0];
   tab[i] = thermo_coef(m, T);
}

int build_thermo_table(const ampe_model_t& m, ThermoCoef* tab, int n,
                       cudaStream_t s)
{
   k_thermo_table<<<(n + 127) / 128, 128, 0, s>>>(m, n, tab);
   return launch_status();
}

__device__ __forceinline__ ThermoCoef coef_at(const ampe_model_t& m,
                                              const Grid& g,
                                              const ThermoCoef* tab,
                                              const double* tfield, int i,
                                              int j, int k)
{
   if (tab) return tab[m.temp_mode == AMPE_TEMP_GRADIENT ? i : 0];
   return thermo_coef(m, temperature_at(m, g, tfield, i, j, k));
}

// (fL(a) - fS(b)) - muS(b) (a - b) in J/mol, ideal-mixing part written as
// RT[a ln(a/b) + (1-a) ln((1-a)/(1-b))] (two logarithms instead of five).
__device__ __forceinline__ double driving_force_molar(const ThermoCoef& th,
                                                      double a, double b)
{
   const double ua = 2.0 * a - 1.0, ub = 2.0 * b - 1.0;
   double SLa, S1La, S2La, SSb, S1Sb, S2Sb;
   rk_sums(th.L[0], ua, SLa, S1La, S2La);
   rk_sums(th.L[1], ub, SSb, S1Sb, S2Sb);
   const double ideal = th.RT * (a * log(a / b) + (1.0 - a) * log((1.0 - a) / (1.0 - b)));
   const double fl = a * th.dG[0] + th.GB[0] + a * (1.0 - a) * SLa;
   const double fs = b * th.dG[1] + th.GB[1] + b * (1.0 - b) * SSb;
   const double xs = th.dG[1] - ub * SSb + b * (1.0 - b) * 2.0 * S1Sb;
   return ideal + (fl - fs) - xs * (a - b);
}

__device__ __forceinline__ double driving_force_scaled(const ampe_model_t& m,
                                                       const ThermoCoef& th,
                                                       double a, double b)
{
   if (m.inv_molar_volume[0] == m.inv_molar_volume[1])
      return driving_force_molar(th, a, b) * m.inv_molar_volume[1];
   const double fl = free_energy_of(th, a, 0) * m.inv_molar_volume[0];
   const double fa = free_energy_of(th, b, 1) * m.inv_molar_volume[1];
   const double mu = dfdc_of(th, b, 1) * m.inv_molar_volume[1];
   return (fl - fa) - mu * (a - b);
}

__global__ void k_kks_interior(ampe_model_t m, Grid g, const ThermoCoef* tab,
                               const double* tfield, const double* phi,
                               const double* conc, const double* clr,
                               const double* csr, double* cl, double* cs,
                               double* dF, unsigned long long* counters)
{
   unsigned long long its = 0, fails = 0;
   for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
        t < g.cells(); t += (long long)gridDim.x * blockDim.x) {
      int i, j, k;
      g.ijk(t, i, j, k);
      const long long ci = g.c(i, j, k);
      const ThermoCoef th = coef_at(m, g, tab, tfield, i, j, k);
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
      const double a = x[0], b = x[1];
      cl[ci] = a;
      cs[ci] = b;
      for_each_image(g, i, j, k, [&](long long idx) {
         cl[idx] = a;
         cs[idx] = b;
      });
      if (dF) dF[t] = driving_force_scaled(m, th, a, b);
   }
   if (counters) {
      for (int o = 16; o > 0; o >>= 1) {
         its += __shfl_xor_sync(0xffffffffu, its, o);
         fails += __shfl_xor_sync(0xffffffffu, fails, o);
      }
      if ((threadIdx.x & 31) == 0) {
         atomicAdd(&counters[0], its);
         if (fails) atomicAdd(&counters[1], fails);
      }
   }
}

int kks_interior(const ampe_model_t& m, const Grid& g, const ThermoCoef* tab,
                 const double* tfield, const double* phi, const double* conc,
                 const double* clr, const double* csr, double* cl, double* cs,
                 double* dF, unsigned long long* counters, cudaStream_t s)
{
   long long b = (g.cells() + 255) / 256;
   if (b > max_blocks(16)) b = max_blocks(16);
   k_kks_interior<<<(unsigned)b, 256, 0, s>>>(m, g, tab, tfield, phi, conc,
                                              clr, csr, cl, cs, dF, counters);
   return launch_status();
}

// ---------------------------------------------------------------------------
// fused right-hand side
// ---------------------------------------------------------------------------
template <bool HAS_Q, bool MOB>
__global__ void k_rhs_fused(ampe_model_t m, Grid g, const double* phi,
                            const double* quat, const double* tfield,
                            const ThermoCoef* tab, const double* cl,
                            const double* cs, const double* dF,
                            const double* phid, const double* ogm, const double* conc,
                            const double* cld, const double* csd, double* phi_rhs,
                            double* conc_rhs)
{
   const long long qs = g.cells_ghost();
   const double eq2 = 0.5 * m.epsilon_q * m.epsilon_q;
   auto P = [&](int a, int b, int c) { return phi[g.c(a, b, c)]; };
   auto Q = [&](int comp, int a, int b, int c) {
      return HAS_Q ? quat[comp * qs + g.c(a, b, c)] : 0.0;
   };
   const double dxi[3] = {1.0 / m.dx[0], 1.0 / m.dx[1],
                          g.dim == 3 ? 1.0 / m.dx[2] : 0.0};
   const double qlR = m.Q_liquid / kGasR, qsR = m.Q_solid / kGasR;
   const bool tdep = (m.Q_liquid != 0.0 || m.Q_solid != 0.0);
   for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
        t < g.cells(); t += (long long)gridDim.x * blockDim.x) {
      int i, j, k;
      g.ijk(t, i, j, k);
      const long long c = g.c(i, j, k);
      // ---- phase ----
      double diff = 0.0;
      for (int d = 0; d < g.dim; d++) {
         const int ei = d == 0, ej = d == 1, ek = d == 2;
         const double fm = phase_face_flux(m, g.dim, d, i, j, k, P, Q);
         const double fp =
             phase_face_flux(m, g.dim, d, i + ei, j + ej, k + ek, P, Q);
         diff = diff + (fp - fm) * dxi[d];
      }
      const double p = phi[c];
      double r = diff - m.phase_well_scale * deriv_well_func(p, m.well_type);
      double df;
      if (dF) {
         df = dF[t];
      } else {
         const ThermoCoef th = coef_at(m, g, tab, tfield, i, j, k);
         df = driving_force_scaled(m, th, cl[c], cs[c]);
      }
      if (ogm) {  // orientation term of COMPUTERHSPBG, 3d/quatrhs.m4:481-509
         const double p1 = deriv_interp_func(p, m.orient_interp1);
         const double p2 = deriv_interp_func(p, m.orient_interp2);
         const double gm = ogm[t];
         const double T = temperature_at(m, g, tfield, i, j, k);
         r = r - m.misorientation_factor * T * p1 * gm - p2 * eq2 * gm * gm;
      }
      r += deriv_interp_func(p, m.energy_interp) * df;
      phi_rhs[t] = r * m.phase_mobility;
      // ---- composition ----
      double div = 0.0;
      for (int d = 0; d < g.dim; d++) {
         const int ei = d == 0, ej = d == 1, ek = d == 2;
         double fl[2];
         for (int side = 0; side < 2; side++) {
            // face between (a-e) and (a)
            const int a0 = i + side * ei, a1 = j + side * ej, a2 = k + side * ek;
            const long long up = g.c(a0, a1, a2);
            const long long lo = g.c(a0 - ei, a1 - ej, a2 - ek);
            const double vphi = average_func(phid[lo], phid[up], m.avg_type);
            const bool kksf = m.conc_form == AMPE_CONC_KKS;
            const double hphi = interp_func(vphi, kksf ? m.energy_interp : m.diff_interp);
            double dlq = m.D_liquid, dsq = m.D_solid;
            if (MOB) {
               // composition-dependent D_L, D_S from the atomic mobilities at
               // the face means of the lagged cL, cS and of T
               // (MobilityCompositionDiffusionStrategy.cc:83-611)
               const double T = 0.5 * (temperature_at(m, g, tfield, a0, a1, a2) +
                                       temperature_at(m, g, tfield, a0 - ei, a1 - ej, a2 - ek));
               dlq = phase_diffusion(m, m.mobility, 0, 0.5 * (cld[up] + cld[lo]), T);
               dsq = phase_diffusion(m, m.mobility, 1, 0.5 * (csd[up] + csd[lo]), T);
            } else if (tdep) {
               const double invT =
                   2.0 / (temperature_at(m, g, tfield, a0 - ei, a1 - ej, a2 - ek) +
                          temperature_at(m, g, tfield, a0, a1, a2));
               dlq = m.D_liquid * exp(-qlR * invT);
               dsq = m.D_solid * exp(-qsR * invT);
            }
            if (kksf) {
               // "kks" form (KKSCompositionRHSStrategy.cc:98-441): D0 grad c +
               // D0 h'(phibar)(cLbar - cSbar) grad phi, coefficients from the
               // lagged phi, cL, cS
               const double d0 = (1.0 - hphi) * dlq + hphi * dsq;
               const double clb = 0.5 * (cld[up] + cld[lo]);
               const double csb = 0.5 * (csd[up] + csd[lo]);
               const double dph = d0 * deriv_interp_func(vphi, m.energy_interp) * (clb - csb);
               fl[side] = dxi[d] * (d0 * (conc[up] - conc[lo]) + dph * (phi[up] - phi[lo]));
               continue;
            }
            const double DL = (1.0 - hphi) * dlq, DS = hphi * dsq;
            double f = 0.0;
            f = f + dxi[d] * DL * (cl[up] - cl[lo]);
            f = f + dxi[d] * DS * (cs[up] - cs[lo]);
            fl[side] = f;
         }
         div = div + dxi[d] * (fl[1] - fl[0]);
      }
      conc_rhs[t] = m.conc_mobility * div;
   }
}

int rhs_fused(const ampe_model_t& m, const Grid& g, const double* phi,
              const double* quat, const double* tfield, const ThermoCoef* tab,
              const double* cl, const double* cs, const double* dF,
              const double* phid, const double* ogm, const double* conc,
              const double* cld, const double* csd, double* phi_rhs,
              double* conc_rhs, cudaStream_t s)
{
   if (m.conc_form == AMPE_CONC_KKS && (!conc || !cld || !csd)) return AMPE_ERR_INVALID;
   const bool mob = m.conc_diffusion == AMPE_DIFF_MOBILITY;
   if (mob && (m.conc_form != AMPE_CONC_EBS || !cld || !csd)) return AMPE_ERR_INVALID;
   long long b = (g.cells() + 255) / 256;
   if (b > max_blocks()) b = max_blocks();
#define AMPE_FUSED(Q, M)                                                                     \
   k_rhs_fused<Q, M><<<(unsigned)b, 256, 0, s>>>(m, g, phi, quat, tfield, tab, cl, cs, dF,   \
                                                 phid, ogm, conc, cld, csd, phi_rhs, conc_rhs)
   if (quat) {
      if (mob)
         AMPE_FUSED(true, true);
      else
         AMPE_FUSED(true, false);
   } else {
      if (mob)
         AMPE_FUSED(false, true);
      else
         AMPE_FUSED(false, false);
   }
#undef AMPE_FUSED
   return launch_status();
}

}  // namespace ampe

using namespace ampe;

extern "C" int ampe_rhs_phase_conc(const ampe_model_t* m, const double* phi,
                                   const double* quat, const double* temp,
                                   const double* cl, const double* cs,
                                   double* phi_rhs, double* conc_rhs,
                                   void* stream)
{
   if (check_model(m) || !phi || !cl || !cs || !phi_rhs || !conc_rhs)
      return AMPE_ERR_INVALID;
   if (m->flux_type == AMPE_FLUX_ANISOTROPIC && !quat) return AMPE_ERR_INVALID;
   if (m->temp_mode == AMPE_TEMP_FIELD && !temp) return AMPE_ERR_INVALID;
   if (m->conc_form == AMPE_CONC_KKS) return AMPE_ERR_INVALID;  // needs c: ampe_conc_flux_kks
   // the diffusivities (either model) at this phi, cL, cS
   return rhs_fused(*m, make_grid(*m), phi, quat, temp, nullptr, cl, cs,
                    nullptr, phi, nullptr, nullptr, cl, cs, phi_rhs, conc_rhs,
                    (cudaStream_t)stream);
}
