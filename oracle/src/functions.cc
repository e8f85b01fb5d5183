// CPU restatement of AMPE's scalar interpolation, well and average
// functions (source/fortran/functions.f:17-406).  TEST INFRASTRUCTURE.
#include "oracle_common.h"

namespace orc {

static double clamp01(double p) { return std::fmax(0.0, std::fmin(1.0, p)); }

// functions.f:17-89
double interp_func(double phi, char type)
{
   const double gamma = 10.0;
   double p;
   switch (type) {
      case 'q':
         p = std::fmax(0.0, phi);
         return p * p;
      case 'p':
         p = clamp01(phi);
         return p * p * p * (10.0 - 15.0 * p + 6.0 * p * p);
      case 'h':
         p = clamp01(phi);
         return p * p * (3.0 - 2.0 * p);
      case 'w':
         p = std::fmax(0.0, phi);
         return p * p * (2.0 - p);
      case 'l':
         return clamp01(phi);
      case 'm':
         p = clamp01(phi);
         return p * p / (2.0 * p * (p - 1.0) + 1.0);
      case '3':
         p = std::fmax(0.0, phi);
         return p * p * p;
      case 's':
         return std::log(std::cosh(gamma * phi)) / std::log(std::cosh(gamma));
      case 'c':
         return 1.0;
      default:
         return NAN;
   }
}

// functions.f:95-170
double deriv_interp_func(double phi, char type)
{
   const double gamma = 10.0;
   double p, t;
   switch (type) {
      case 'q':
         return 2.0 * std::fmax(0.0, phi);
      case 'p':
         p = clamp01(phi);
         return 30.0 * p * p * (1.0 - p) * (1.0 - p);
      case 'h':
         p = clamp01(phi);
         return 6.0 * p * (1.0 - p);
      case 'w':
         p = std::fmax(0.0, phi);
         return p * (4.0 - 3.0 * p);
      case 'l':
         // the reference tests (phi > 0 .or. phi < 1), true for every phi
         return (phi > 0.0 || phi < 1.0) ? 1.0 : 0.0;
      case 'm':
         p = clamp01(phi);
         t = 2.0 * p * (p - 1.0) + 1.0;
         return 2.0 * p * (1.0 - p) / (t * t);
      case '3':
         p = std::fmax(0.0, phi);
         return 3.0 * p * p;
      case 's':
         p = std::fmax(0.0, phi);
         return gamma * std::tanh(gamma * p) / std::log(std::cosh(gamma));
      case 'c':
         return 0.0;
      default:
         return NAN;
   }
}

// functions.f:176-243
double second_deriv_interp_func(double phi, char type)
{
   double p;
   switch (type) {
      case 'q':
         return phi >= 0.0 ? 2.0 : 0.0;
      case 'p':
         p = clamp01(phi);
         return 60.0 * p * (1.0 - 3.0 * p + 2.0 * p * p);
      case 'h':
         p = clamp01(phi);
         return 6.0 * (1.0 - 2.0 * p);
      case 'w':
         p = std::fmax(0.0, phi);
         return 4.0 - 6.0 * p;
      case 'l':
      case 'c':
         return 0.0;
      default:
         return NAN;
   }
}

// functions.f:246-270
double well_func(double phi, char type)
{
   if (type == 'd') return 16.0 * phi * phi * (1.0 - phi) * (1.0 - phi);
   if (type == 's') return (1.0 - phi) * (1.0 - phi);
   return NAN;
}

// functions.f:275-300
double deriv_well_func(double phi, char type)
{
   if (type == 'd') return 32.0 * phi * (1.0 - phi) * (1.0 - 2.0 * phi);
   if (type == 's') return 2.0 * (phi - 1.0);
   return NAN;
}

// functions.f:304-330
double second_deriv_well_func(double phi, char type)
{
   if (type == 'd') return 32.0 * (1.0 + 6.0 * phi * (phi - 1.0));
   if (type == 's') return 2.0;
   return NAN;
}

// functions.f:333-369
double average_func(double a, double b, char type)
{
   const double threshold = 1.0e-16;
   if (type == 'a') return 0.5 * (a + b);
   if (type == 'h') {
      if (a < threshold || b < threshold) return 0.0;
      return 2.0 / (1.0 / a + 1.0 / b);
   }
   return NAN;
}

}  // namespace orc
