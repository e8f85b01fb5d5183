// Oracle-internal helpers.  TEST INFRASTRUCTURE ONLY: the oracle is the
// CPU checker of libampe_gb300; nothing in the product links it.
#ifndef AMPE_ORACLE_COMMON_H
#define AMPE_ORACLE_COMMON_H

#include <cmath>
#include <cstddef>
#include <vector>

#include "ampe_gb300.h"

namespace orc {

constexpr double kGasR = 8.314472;  // J/(K mol), KKSdiluteBinary.cc:45

// ---- layout -------------------------------------------------------------
struct Layout {
   int dim, n0, n1, n2, ng, gz;
   long sx, sy;  // strides in elements: sx = row pitch, sy = plane pitch
   explicit Layout(const ampe_model_t& m)
       : dim(m.dim), n0(m.n[0]), n1(m.n[1]), n2(m.dim == 3 ? m.n[2] : 1),
         ng(m.ng), gz(m.dim == 3 ? m.ng : 0)
   {
      sx = n0 + 2 * ng;
      sy = sx * (n1 + 2 * ng);
   }
   long cells_ghost() const { return sy * (n2 + 2 * gz); }
   long cells() const { return (long)n0 * n1 * n2; }
   // (i,j,k) interior coordinates, may be in [-ng, n+ng)
   long c(int i, int j, int k) const
   {
      return ((long)(k + gz) * (n1 + 2 * ng) + (j + ng)) * sx + (i + ng);
   }
   long fx(int i, int j, int k) const
   {
      return ((long)k * n1 + j) * (n0 + 1) + i;
   }
   long fy(int i, int j, int k) const
   {
      return ((long)k * (n1 + 1) + j) * n0 + i;
   }
   long fz(int i, int j, int k) const { return ((long)k * n1 + j) * n0 + i; }
   long nfx() const { return (long)(n0 + 1) * n1 * n2; }
   long nfy() const { return (long)n0 * (n1 + 1) * n2; }
   long nfz() const { return (long)n0 * n1 * (n2 + 1); }
   long interior(int i, int j, int k) const
   {
      return ((long)k * n1 + j) * n0 + i;
   }
};

// ---- functions.f restatement --------------------------------------------
double interp_func(double phi, char type);
double deriv_interp_func(double phi, char type);
double second_deriv_interp_func(double phi, char type);
double well_func(double phi, char type);
double deriv_well_func(double phi, char type);
double second_deriv_well_func(double phi, char type);
double average_func(double a, double b, char type);

// ---- thermodynamics ------------------------------------------------------
double gterm(const ampe_gterm_t& g, double T);
struct PhaseCoef {  // mu_i(c)/RT = ln(c/(1-c)) + xi_i(c)/RT
   double dG;       // G_A - G_B (J/mol)
   double GB;       // G_B (J/mol)
   double L[4];     // Redlich-Kister L_k(T)
};
struct ThermoT {
   double T, RT;
   PhaseCoef p[2];  // liquid, solid
};
ThermoT thermo_at(const ampe_model_t& m, double T);
double free_energy(const ThermoT& th, double c, int phase);  // J/mol
double dfdc(const ThermoT& th, double c, int phase);          // J/mol
double d2fdc2(const ThermoT& th, double c, int phase);        // J/mol
double xi(const ThermoT& th, double c, int phase);            // J/mol
double dxi(const ThermoT& th, double c, int phase);
int kks_newton(const ampe_model_t& m, const ThermoT& th, double h, double c,
               double x[2]);
int ceq_newton(const ampe_model_t& m, const ThermoT& th, double x[2]);

double temperature_at(const ampe_model_t& m, const double* tfield,
                      const Layout& L, int i, int j, int k);

}  // namespace orc

#endif
