// Device-side building blocks shared by every kernel of libampe_gb300:
// grid layout, periodic ghost images, the scalar interpolation/well
// functions of AMPE (source/fortran/functions.f:17-406) and the binary KKS
// thermodynamics (doc/latex/manual/appendix.tex:517-596 for CALPHAD; the
// dilute model is the ideal-solution form calibrated on meltingT,
// liquidus_slope and keq).
#pragma once

#include <atomic>
#include <cuda_runtime.h>
#include <stdint.h>

#include "ampe_gb300.h"
#include "bitconv.h"
#include "fastdiv.h"

#define AMPE_HD __host__ __device__ __forceinline__

namespace ampe {

constexpr double kGasR = 8.314472;  // J/(K mol), KKSdiluteBinary.cc:45

// ---------------------------------------------------------------------------
// layout of a ghosted cell field (SAMRAI CellData ghost box, x fastest)
// ---------------------------------------------------------------------------
struct Grid {
   // Index math is 32-bit: ghost boxes and face sets stay below 2^31
   // entries (enforced by check_model).
   int dim, n0, n1, n2, ng, gz;
   int sx, sy;  // row and plane pitch of the ghosted layout
   int gs, gsz;  // ghost width of side (face) arrays, in-plane and along z
   // divisors of the index decompositions: n0, n1, n0+1, n1+1, (n0+1)/2
   FastDiv fd0, fd1, fd0p, fd1p, fdh;
   // linear index t < 2^31 over an (a.d x b.d x *) box -> (i, j, k)
   AMPE_HD void split(long long t, const FastDiv& a, const FastDiv& b, int& i,
                      int& j, int& k) const
   {
      const unsigned u = (unsigned)t;
      const unsigned q = a.div(u);
      i = (int)(u - q * a.d);
      const unsigned kk = b.div(q);
      j = (int)(q - kk * b.d);
      k = (int)kk;
   }
   // interior cell of linear index t (x fastest)
   AMPE_HD void ijk(long long t, int& i, int& j, int& k) const
   {
      split(t, fd0, fd1, i, j, k);
   }
   AMPE_HD int c(int i, int j, int k) const
   {
      return ((k + gz) * (n1 + 2 * ng) + (j + ng)) * sx + (i + ng);
   }
   AMPE_HD int interior(int i, int j, int k) const { return (k * n1 + j) * n0 + i; }
   // side arrays (SAMRAI SideData of ghost width gs): normal d has extent
   // n_d + 1 + 2 gs along d and n_e + 2 gs along the others (no z ghosts
   // in 2D)
   AMPE_HD int fx(int i, int j, int k) const
   {
      return ((k + gsz) * (n1 + 2 * gs) + (j + gs)) * (n0 + 1 + 2 * gs) + (i + gs);
   }
   AMPE_HD int fy(int i, int j, int k) const
   {
      return ((k + gsz) * (n1 + 1 + 2 * gs) + (j + gs)) * (n0 + 2 * gs) + (i + gs);
   }
   AMPE_HD int fz(int i, int j, int k) const
   {
      return ((k + gsz) * (n1 + 2 * gs) + (j + gs)) * (n0 + 2 * gs) + (i + gs);
   }
   // index distance to the next y face (y-side arrays) and z face (z-side)
   AMPE_HD int fys() const { return n0 + 2 * gs; }
   AMPE_HD int fzs() const { return (n0 + 2 * gs) * (n1 + 2 * gs); }
   AMPE_HD long long cells() const { return (long long)n0 * n1 * n2; }
   AMPE_HD long long cells_ghost() const { return (long long)sy * (n2 + 2 * gz); }
   // interior faces of each normal (the faces the kernels compute)
   AMPE_HD long long nfx() const { return (long long)(n0 + 1) * n1 * n2; }
   AMPE_HD long long nfy() const { return (long long)n0 * (n1 + 1) * n2; }
   AMPE_HD long long nfz() const { return (long long)n0 * n1 * (n2 + 1); }
};

inline Grid make_grid(const ampe_model_t& m)
{
   Grid g;
   g.dim = m.dim;
   g.n0 = m.n[0];
   g.n1 = m.n[1];
   g.n2 = m.dim == 3 ? m.n[2] : 1;
   g.ng = m.ng;
   g.gz = m.dim == 3 ? m.ng : 0;
   g.sx = g.n0 + 2 * g.ng;
   g.sy = g.sx * (g.n1 + 2 * g.ng);
   g.gs = m.ng_side;
   g.gsz = m.dim == 3 ? m.ng_side : 0;
   g.fd0 = FastDiv((unsigned)g.n0);
   g.fd1 = FastDiv((unsigned)g.n1);
   g.fd0p = FastDiv((unsigned)(g.n0 + 1));
   g.fd1p = FastDiv((unsigned)(g.n1 + 1));
   g.fdh = FastDiv((unsigned)((g.n0 + 1) / 2));
   return g;
}

// Call f(index) for every periodic ghost image of interior cell (i,j,k):
// the ghost-box positions that a SAMRAI periodic fill would copy it to.
template <class F>
__device__ __forceinline__ void for_each_image(const Grid& g, int i, int j,
                                               int k, F f)
{
   if (i >= g.ng && i < g.n0 - g.ng && j >= g.ng && j < g.n1 - g.ng &&
       (g.dim != 3 || (k >= g.ng && k < g.n2 - g.ng)))
      return;  // interior cell: no image
   int si[2] = {0, 0}, sj[2] = {0, 0}, sk[2] = {0, 0};
   int ni = 1, nj = 1, nk = 1;
   if (i < g.ng)
      si[ni++] = g.n0;
   else if (i >= g.n0 - g.ng)
      si[ni++] = -g.n0;
   if (j < g.ng)
      sj[nj++] = g.n1;
   else if (j >= g.n1 - g.ng)
      sj[nj++] = -g.n1;
   if (g.dim == 3) {
      if (k < g.ng)
         sk[nk++] = g.n2;
      else if (k >= g.n2 - g.ng)
         sk[nk++] = -g.n2;
   }
   for (int c = 0; c < nk; c++)
      for (int b = 0; b < nj; b++)
         for (int a = 0; a < ni; a++)
            if (a | b | c) f(g.c(i + si[a], j + sj[b], k + sk[c]));
}

// ---------------------------------------------------------------------------
// functions.f restatement (same branch structure, device versions)
// ---------------------------------------------------------------------------
template <class R>
AMPE_HD R clamp01(R p)
{
   return p < R(0) ? R(0) : (p > R(1) ? R(1) : p);
}

template <class R>
__device__ __forceinline__ R interp_func(R phi, char type)
{
   R p;
   switch (type) {
      case 'q':
         p = phi > R(0) ? phi : R(0);
         return p * p;
      case 'p':
         p = clamp01(phi);
         return p * p * p * (R(10) - R(15) * p + R(6) * p * p);
      case 'h':
         p = clamp01(phi);
         return p * p * (R(3) - R(2) * p);
      case 'w':
         p = phi > R(0) ? phi : R(0);
         return p * p * (R(2) - p);
      case 'l':
         return clamp01(phi);
      case 'm':
         p = clamp01(phi);
         return p * p / (R(2) * p * (p - R(1)) + R(1));
      case '3':
         p = phi > R(0) ? phi : R(0);
         return p * p * p;
      case 's':
         return log(cosh(R(10) * phi)) / log(cosh(R(10)));
      case 'c':
         return R(1);
      default:
         return R(NAN);
   }
}

template <class R>
__device__ __forceinline__ R deriv_interp_func(R phi, char type)
{
   R p, t;
   switch (type) {
      case 'q':
         return R(2) * (phi > R(0) ? phi : R(0));
      case 'p':
         p = clamp01(phi);
         return R(30) * p * p * (R(1) - p) * (R(1) - p);
      case 'h':
         p = clamp01(phi);
         return R(6) * p * (R(1) - p);
      case 'w':
         p = phi > R(0) ? phi : R(0);
         return p * (R(4) - R(3) * p);
      case 'l':
         return (phi > R(0) || phi < R(1)) ? R(1) : R(0);
      case 'm':
         p = clamp01(phi);
         t = R(2) * p * (p - R(1)) + R(1);
         return R(2) * p * (R(1) - p) / (t * t);
      case '3':
         p = phi > R(0) ? phi : R(0);
         return R(3) * p * p;
      case 's':
         p = phi > R(0) ? phi : R(0);
         return R(10) * tanh(R(10) * p) / log(cosh(R(10)));
      case 'c':
         return R(0);
      default:
         return R(NAN);
   }
}

template <class R>
__device__ __forceinline__ R deriv_well_func(R phi, char type)
{
   if (type == 'd') return R(32) * phi * (R(1) - phi) * (R(1) - R(2) * phi);
   if (type == 's') return R(2) * (phi - R(1));
   return R(NAN);
}

template <class R>
__device__ __forceinline__ R second_deriv_well_func(R phi, char type)
{
   if (type == 'd') return R(32) * (R(1) + R(6) * phi * (phi - R(1)));
   if (type == 's') return R(2);
   return R(NAN);
}

template <class R>
__device__ __forceinline__ R average_func(R a, R b, char type)
{
   if (type == 'a') return R(0.5) * (a + b);
   if (type == 'h') {
      const R thr = R(1.0e-16);
      if (a < thr || b < thr) return R(0);
      return R(2) / (R(1) / a + R(1) / b);
   }
   return R(NAN);
}

// ---------------------------------------------------------------------------
// thermodynamics: per-temperature coefficients of
//   mu_i(c)/RT = ln(c/(1-c)) + xi_i(c)/RT,
//   xi_i(c) = dG_i - u S_i(u) + 2 c (1-c) S_i'(u),  u = 2c-1,
//   S_i(u) = sum_k L_k^i u^k.
// ---------------------------------------------------------------------------
struct ThermoCoef {
   double RT, iRT;
   double dG[2], GB[2];
   double L[2][4];
};

__host__ __device__ inline double gterm_eval(const ampe_gterm_t& g, double T)
{
   if (g.nseg <= 0) return 0.0;
   int s = 0;
   while (s < g.nseg - 1 && T >= g.tc[s + 1]) s++;
   const double T2 = T * T, T3 = T2 * T, T4 = T2 * T2, T7 = T4 * T3;
   const double iT = 1.0 / T, iT3 = iT * iT * iT, iT9 = iT3 * iT3 * iT3;
   return g.a[s] + g.b[s] * T + g.c[s] * T * log(T) + g.d2[s] * T2 +
          g.d3[s] * T3 + g.d4[s] * T4 + g.d7[s] * T7 + g.dm1[s] * iT +
          g.dm9[s] * iT9;
}

__host__ __device__ inline ThermoCoef thermo_coef(const ampe_model_t& m,
                                                  double T)
{
   ThermoCoef th;
   th.RT = kGasR * T;
   th.iRT = 1.0 / th.RT;
   for (int p = 0; p < 2; p++)
      for (int k = 0; k < 4; k++) th.L[p][k] = 0.0;
   if (m.thermo == AMPE_THERMO_CALPHAD) {
      for (int p = 0; p < 2; p++) {
         const double GA = gterm_eval(m.g[0][p], T);
         const double GB = gterm_eval(m.g[1][p], T);
         th.dG[p] = GA - GB;
         th.GB[p] = GB;
         for (int k = 0; k < 4; k++)
            th.L[p][k] = m.L[p][k][0] + m.L[p][k][1] * T;
      }
   } else {
      const double cLe = (T - m.dilute_Tm) / m.dilute_m;
      const double cSe = m.dilute_k * cLe;
      const double fA = th.RT * log((1.0 - cLe) / (1.0 - cSe));
      const double fB = -th.RT * log(m.dilute_k);
      th.dG[0] = 0.0;
      th.GB[0] = 0.0;
      th.dG[1] = fB - fA;
      th.GB[1] = fA;
   }
   return th;
}

template <class R>
__device__ __forceinline__ void rk_sums(const double* L, R u, R& S, R& S1,
                                        R& S2)
{
   const R L0 = R(L[0]), L1 = R(L[1]), L2 = R(L[2]), L3 = R(L[3]);
   S = L0 + u * (L1 + u * (L2 + u * L3));
   S1 = L1 + u * (R(2) * L2 + u * R(3) * L3);
   S2 = R(2) * L2 + u * R(6) * L3;
}

template <class R>
__device__ __forceinline__ R xi_of(const ThermoCoef& th, R c, int p)
{
   const R u = R(2) * c - R(1);
   R S, S1, S2;
   rk_sums(th.L[p], u, S, S1, S2);
   return R(th.dG[p]) - u * S + c * (R(1) - c) * R(2) * S1;
}

template <class R>
__device__ __forceinline__ R dxi_of(const ThermoCoef& th, R c, int p)
{
   const R u = R(2) * c - R(1);
   R S, S1, S2;
   rk_sums(th.L[p], u, S, S1, S2);
   return -R(2) * S - R(4) * u * S1 + R(4) * c * (R(1) - c) * S2;
}

// Q_i(T) and the interaction terms of one species' mobility in one phase
// (CALPHADMobility.h getQ, getQQ0..3)
__device__ __forceinline__ double mob_q(const double* a, double T)
{
   return a[0] + kGasR * T * log(a[1]) + a[2] * T * log(T) + a[3] / T;
}

__device__ __forceinline__ double mob_qq(const double* a, double T)
{
   return a[0] + kGasR * T * log(a[1]);
}

// atomic mobility of species s in phase p at composition (c0, c1 = 1 - c0)
// (CALPHADMobility::getAtomicMobility and getDeltaG, binary form)
__device__ __forceinline__ double atomic_mobility(const ampe_mobility_t& mb, int s, int p,
                                                  double c0, double c1, double T)
{
   const double dc = c0 - c1;
   const double dG =
       c0 * mob_q(mb.q[s][p][0], T) + c1 * mob_q(mb.q[s][p][1], T) +
       c0 * c1 *
           (mob_qq(mb.qq[s][p][0], T) +
            dc * (mob_qq(mb.qq[s][p][1], T) +
                  dc * (mob_qq(mb.qq[s][p][2], T) + dc * mob_qq(mb.qq[s][p][3], T))));
   const double rtinv = 1.0 / (kGasR * T);
   return exp(dG * rtinv) * rtinv;
}

// D_p = (mobility matrix) x (free-energy curvature), 1x1 for a binary
// (computeLocalDiffusionMatrixL/A with computeDiffusionMobilityBinaryPhase)
__device__ __forceinline__ double phase_diffusion(const ampe_model_t& m,
                                                  const ampe_mobility_t& mb, int p, double c,
                                                  double T)
{
   const double c1 = 1.0 - c;
   const double m0 = atomic_mobility(mb, 0, p, c, c1, T);
   const double m1 = atomic_mobility(mb, 1, p, c, c1, T);
   const double mm = c * m1 + c1 * m0;
   const double mob = c * c1 * mm * 1.e12;
   const ThermoCoef th = thermo_coef(m, T);
   const double curv = th.RT / (c * (1.0 - c)) + dxi_of(th, c, p);
   return mob * curv;
}

__device__ __forceinline__ double xlogx(double x)
{
   return x > 0.0 ? x * log(x) : 0.0;
}

__device__ __forceinline__ double free_energy_of(const ThermoCoef& th,
                                                 double c, int p)
{
   const double u = 2.0 * c - 1.0;
   double S, S1, S2;
   rk_sums(th.L[p], u, S, S1, S2);
   return c * th.dG[p] + th.GB[p] + th.RT * (xlogx(c) + xlogx(1.0 - c)) +
          c * (1.0 - c) * S;
}

__device__ __forceinline__ double dfdc_of(const ThermoCoef& th, double c,
                                          int p)
{
   return th.RT * log(c / (1.0 - c)) + xi_of(th, c, p);
}

// The KKS Newton of the oracle (same update, projection and stop test).
// Returns iterations >= 1, or -1 when not converged.
__device__ __forceinline__ int kks_newton(const ThermoCoef& th, double h,
                                          double c, double x[2], int max_its,
                                          double tol)
{
   if (!(x[0] > 0.0 && x[0] < 1.0)) x[0] = c;
   if (!(x[1] > 0.0 && x[1] < 1.0)) x[1] = c;
   for (int it = 1; it <= max_its; it++) {
      const double a = x[0], b = x[1];
      const double F0 = (1.0 - h) * a + h * b - c;
      const double F1 = log(a * (1.0 - b) / ((1.0 - a) * b)) +
                        (xi_of(th, a, 0) - xi_of(th, b, 1)) * th.iRT;
      const double J00 = 1.0 - h, J01 = h;
      const double J10 = 1.0 / (a * (1.0 - a)) + dxi_of(th, a, 0) * th.iRT;
      const double J11 = -1.0 / (b * (1.0 - b)) - dxi_of(th, b, 1) * th.iRT;
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
      if (fmax(fabs(d0), fabs(d1)) < tol) return it;
      if (!(isfinite(na) && isfinite(nb))) return -1;
   }
   return -1;
}

// Temperature of cell (i,j,k) (ghost cells take their periodic image).
__device__ __forceinline__ double temperature_at(const ampe_model_t& m,
                                                 const Grid& g,
                                                 const double* tfield, int i,
                                                 int j, int k)
{
   if (m.temp_mode == AMPE_TEMP_CONSTANT) return m.T0;
   if (m.temp_mode == AMPE_TEMP_GRADIENT) {
      const int iw = i < 0 ? i + g.n0 : (i >= g.n0 ? i - g.n0 : i);
      return m.T0 + m.gradT * ((double)iw + 0.5) * m.dx[0];
   }
   return tfield[g.c(i, j, k)];
}

// value conversion between the FP64 and FP32 arrays of the stepper (integer
// pipe for the float <-> double cases, see bitconv.h)
template <class D, class S>
__device__ __forceinline__ D cvt(S x)
{
   return (D)x;
}
template <>
__device__ __forceinline__ float cvt<float, double>(double x)
{
   return d2f(x);
}
template <>
__device__ __forceinline__ double cvt<double, float>(float x)
{
   return f2d(x);
}

}  // namespace ampe

// ---------------------------------------------------------------------------
// host-side helpers
// ---------------------------------------------------------------------------
namespace ampe {
int check_model(const ampe_model_t* m);
int check_mobility(const ampe_mobility_t* mob);
extern long long g_launches;  // kernels launched through this library
inline int launch_status()
{
   g_launches++;
   cudaError_t e = cudaGetLastError();
   return e == cudaSuccess ? AMPE_OK : AMPE_ERR_CUDA;
}
// multiprocessor count of the current device (queried once per device)
int device_sms();
// true on the first call with this flag on the current device: for one-time
// set-up that applies to one device only (cudaFuncSetAttribute)
inline bool first_on_device(std::atomic<unsigned long long>& seen)
{
   int dev = 0;
   if (cudaGetDevice(&dev) != cudaSuccess) return true;
   const unsigned long long bit = 1ull << (dev & 63);
   return !(seen.fetch_or(bit) & bit);
}
// grid cap of the grid-stride kernels: per_sm blocks (32 by default, of 256
// threads) per SM of the current device.  Threads then loop over several
// items and set up their per-thread constants once (measured faster than one
// thread per item for the stencil kernels, whose setup includes FP64 work;
// the smoother colour and residual kernels run one thread per item instead)
inline long long max_blocks(int per_sm = 32)
{
   return (long long)device_sms() * per_sm;
}
inline unsigned grid_for(long long n, int block)
{
   return (unsigned)((n + block - 1) / block);
}
}  // namespace ampe
