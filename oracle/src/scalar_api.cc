// extern "C" wrappers of the oracle's scalar functions.  TEST INFRASTRUCTURE.
#include "oracle_api.h"
#include "oracle_common.h"

using namespace orc;

extern "C" {

double orc_interp_func(double phi, char t) { return interp_func(phi, t); }
double orc_deriv_interp_func(double phi, char t)
{
   return deriv_interp_func(phi, t);
}
double orc_second_deriv_interp_func(double phi, char t)
{
   return second_deriv_interp_func(phi, t);
}
double orc_well_func(double phi, char t) { return well_func(phi, t); }
double orc_deriv_well_func(double phi, char t)
{
   return deriv_well_func(phi, t);
}
double orc_second_deriv_well_func(double phi, char t)
{
   return second_deriv_well_func(phi, t);
}
double orc_average_func(double a, double b, char t)
{
   return average_func(a, b, t);
}

double orc_free_energy(const ampe_model_t* m, double T, double c, int phase)
{
   return free_energy(thermo_at(*m, T), c, phase);
}
double orc_dfdc(const ampe_model_t* m, double T, double c, int phase)
{
   return dfdc(thermo_at(*m, T), c, phase);
}
double orc_d2fdc2(const ampe_model_t* m, double T, double c, int phase)
{
   return d2fdc2(thermo_at(*m, T), c, phase);
}
double orc_gterm(const ampe_gterm_t* g, double T) { return gterm(*g, T); }

int orc_kks_cell(const ampe_model_t* m, double T, double h, double c,
                 double* x)
{
   return kks_newton(*m, thermo_at(*m, T), h, c, x);
}

int orc_ceq(const ampe_model_t* m, double T, double* x)
{
   return ceq_newton(*m, thermo_at(*m, T), x);
}

}  // extern "C"
