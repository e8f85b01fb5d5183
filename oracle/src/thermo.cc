// CPU restatement of the binary KKS thermodynamics used on the hot path.
// TEST INFRASTRUCTURE ONLY.
//
// CALPHAD binary (doc/latex/manual/appendix.tex:517-596):
//   f^i(c) = c G_A^i + (1-c) G_B^i + RT[c ln c + (1-c) ln(1-c)]
//            + c(1-c) sum_k L_k^i (2c-1)^k,        L_k = a_k + b_k T
//   df/dc  = RT ln(c/(1-c)) + xi_i(c)
// with the species G(T) of thermodynamic_data/calphadAuNi.dat:1-49.
//
// KKS dilute binary.  The reference delegates this model to Thermo4PFM
// (KKSFreeEnergyFunctionDiluteBinary, not in the reference tree).  It is
// restated here as ideal solutions whose reference energies reproduce the
// linearised phase diagram given by the reference inputs meltingT, liquidus
// slope m and keq (tests/KKSdiluteBinaryKKS/test.input:12-17):
//   cLe = (T - Tm)/m,  cSe = k cLe,
//   f^L(c) = RT[c ln c + (1-c) ln(1-c)]
//   f^S(c) = (1-c) fA + c fB + RT[c ln c + (1-c) ln(1-c)],
//   fA = RT ln((1-cLe)/(1-cSe)),  fB = -RT ln k,
// so that (cLe, cSe) is the exact common tangent (the property pinned by
// tests/testKKSdiluteBinaryEquilibrium.cc:97-130).
#include <algorithm>

#include "oracle_common.h"

namespace orc {

static double xlogx(double x) { return x > 0.0 ? x * std::log(x) : 0.0; }

// calphadAuNi.dat:5 "G = a + b*T + c*T*ln(T)+sum_i di*T^i"
double gterm(const ampe_gterm_t& g, double T)
{
   if (g.nseg <= 0) return 0.0;
   int s = 0;
   while (s < g.nseg - 1 && T >= g.tc[s + 1]) s++;
   const double T2 = T * T, T3 = T2 * T, T4 = T2 * T2, T7 = T4 * T3;
   const double iT = 1.0 / T, iT9 = std::pow(iT, 9);
   return g.a[s] + g.b[s] * T + g.c[s] * T * std::log(T) + g.d2[s] * T2 +
          g.d3[s] * T3 + g.d4[s] * T4 + g.d7[s] * T7 + g.dm1[s] * iT +
          g.dm9[s] * iT9;
}

ThermoT thermo_at(const ampe_model_t& m, double T)
{
   ThermoT th;
   th.T = T;
   th.RT = kGasR * T;
   for (int p = 0; p < 2; p++)
      for (int k = 0; k < 4; k++) th.p[p].L[k] = 0.0;
   if (m.thermo == AMPE_THERMO_CALPHAD) {
      for (int p = 0; p < 2; p++) {
         const double GA = gterm(m.g[0][p], T);
         const double GB = gterm(m.g[1][p], T);
         th.p[p].dG = GA - GB;
         th.p[p].GB = GB;
         for (int k = 0; k < 4; k++)
            th.p[p].L[k] = m.L[p][k][0] + m.L[p][k][1] * T;
      }
   } else {
      const double cLe = (T - m.dilute_Tm) / m.dilute_m;
      const double cSe = m.dilute_k * cLe;
      const double fA = th.RT * std::log((1.0 - cLe) / (1.0 - cSe));
      const double fB = -th.RT * std::log(m.dilute_k);
      th.p[0].dG = 0.0;
      th.p[0].GB = 0.0;
      th.p[1].dG = fB - fA;
      th.p[1].GB = fA;
   }
   return th;
}

static void rk_sums(const double* L, double u, double& S, double& S1,
                    double& S2)
{
   // S = sum L_k u^k, S1 = sum k L_k u^(k-1), S2 = sum k(k-1) L_k u^(k-2)
   S = L[0] + u * (L[1] + u * (L[2] + u * L[3]));
   S1 = L[1] + u * (2.0 * L[2] + u * 3.0 * L[3]);
   S2 = 2.0 * L[2] + u * 6.0 * L[3];
}

double free_energy(const ThermoT& th, double c, int phase)
{
   const PhaseCoef& p = th.p[phase];
   double S, S1, S2;
   rk_sums(p.L, 2.0 * c - 1.0, S, S1, S2);
   return c * p.dG + p.GB + th.RT * (xlogx(c) + xlogx(1.0 - c)) +
          c * (1.0 - c) * S;
}

double xi(const ThermoT& th, double c, int phase)
{
   const PhaseCoef& p = th.p[phase];
   const double u = 2.0 * c - 1.0;
   double S, S1, S2;
   rk_sums(p.L, u, S, S1, S2);
   return p.dG - u * S + c * (1.0 - c) * 2.0 * S1;
}

double dxi(const ThermoT& th, double c, int phase)
{
   const PhaseCoef& p = th.p[phase];
   const double u = 2.0 * c - 1.0;
   double S, S1, S2;
   rk_sums(p.L, u, S, S1, S2);
   return -2.0 * S - 4.0 * u * S1 + 4.0 * c * (1.0 - c) * S2;
}

double dfdc(const ThermoT& th, double c, int phase)
{
   return th.RT * std::log(c / (1.0 - c)) + xi(th, c, phase);
}

double d2fdc2(const ThermoT& th, double c, int phase)
{
   return th.RT / (c * (1.0 - c)) + dxi(th, c, phase);
}

// Newton for c = (1-h) cL + h cS, muL(cL) = muS(cS).  Residual scaled by
// 1/RT; chemical-potential equality written with a single logarithm.
// Iterates are projected into (0,1) by halving the distance to the bound.
// Returns the number of iterations (>=1), or -1 if not converged.
int kks_newton(const ampe_model_t& m, const ThermoT& th, double h, double c,
               double x[2])
{
   if (!(x[0] > 0.0 && x[0] < 1.0)) x[0] = c;
   if (!(x[1] > 0.0 && x[1] < 1.0)) x[1] = c;
   const double iRT = 1.0 / th.RT;
   for (int it = 1; it <= m.newton_max_its; it++) {
      const double a = x[0], b = x[1];
      const double F0 = (1.0 - h) * a + h * b - c;
      const double F1 = std::log(a * (1.0 - b) / ((1.0 - a) * b)) +
                        (xi(th, a, 0) - xi(th, b, 1)) * iRT;
      const double J00 = 1.0 - h, J01 = h;
      const double J10 = 1.0 / (a * (1.0 - a)) + dxi(th, a, 0) * iRT;
      const double J11 = -1.0 / (b * (1.0 - b)) - dxi(th, b, 1) * iRT;
      const double det = J00 * J11 - J01 * J10;
      const double d0 = (F0 * J11 - F1 * J01) / det;
      const double d1 = (J00 * F1 - J10 * F0) / det;
      double na = a - d0, nb = b - d1;
      if (na <= 0.0) na = 0.5 * a;
      if (na >= 1.0) na = 0.5 * (1.0 + a);
      if (nb <= 0.0) nb = 0.5 * b;
      if (nb >= 1.0) nb = 0.5 * (1.0 + b);
      x[0] = na;
      x[1] = nb;
      if (std::fmax(std::fabs(d0), std::fabs(d1)) < m.newton_tol) return it;
      if (!(std::isfinite(na) && std::isfinite(nb))) return -1;
   }
   return -1;
}

// Common tangent (computeCeqT role): muL(cL) = muS(cS) and equal grand
// potentials fL - mu cL = fS - mu cS, Newton in units of RT.
int ceq_newton(const ampe_model_t& m, const ThermoT& th, double x[2])
{
   const double iRT = 1.0 / th.RT;
   for (int it = 1; it <= std::max(m.newton_max_its, 50); it++) {
      const double a = x[0], b = x[1];
      const double mL = dfdc(th, a, 0) * iRT, mS = dfdc(th, b, 1) * iRT;
      const double kL = d2fdc2(th, a, 0) * iRT, kS = d2fdc2(th, b, 1) * iRT;
      const double gL = free_energy(th, a, 0) * iRT;
      const double gS = free_energy(th, b, 1) * iRT;
      const double F0 = mL - mS;
      const double F1 = gL - gS - mL * (a - b);
      const double J00 = kL, J01 = -kS;
      const double J10 = -kL * (a - b), J11 = mL - mS;
      const double det = J00 * J11 - J01 * J10;
      const double d0 = (F0 * J11 - F1 * J01) / det;
      const double d1 = (J00 * F1 - J10 * F0) / det;
      double na = a - d0, nb = b - d1;
      if (na <= 0.0) na = 0.5 * a;
      if (na >= 1.0) na = 0.5 * (1.0 + a);
      if (nb <= 0.0) nb = 0.5 * b;
      if (nb >= 1.0) nb = 0.5 * (1.0 + b);
      x[0] = na;
      x[1] = nb;
      if (std::fmax(std::fabs(d0), std::fabs(d1)) < 1.0e-14) return it;
      if (!(std::isfinite(na) && std::isfinite(nb))) return -1;
   }
   return -1;
}

double temperature_at(const ampe_model_t& m, const double* tfield,
                      const Layout& L, int i, int j, int k)
{
   if (m.temp_mode == AMPE_TEMP_CONSTANT) return m.T0;
   if (m.temp_mode == AMPE_TEMP_GRADIENT) {
      const int iw = ((i % L.n0) + L.n0) % L.n0;
      return m.T0 + m.gradT * ((double)iw + 0.5) * m.dx[0];
   }
   return tfield[L.c(i, j, k)];
}

}  // namespace orc
