// CPU restatement of the implicit step (FP64): fixed-step BDF(<=2),
// Newton with CVODE's convergence/divergence tests, left-preconditioned
// GMRES (modified Gram-Schmidt, no restarts) with WRMS scaling and
// finite-difference Jacobian-vector products, and the block-diagonal
// phase / composition FAC preconditioner.  TEST INFRASTRUCTURE ONLY.
//
// Reference roles: QuatIntegrator::evaluateRHSFunction (QuatIntegrator.cc:
// 3134-3295), CVSpgmrPrecondSet (:3300-3375), CVSpgmrPrecondSolve
// (:3666-3769), CVODESolver (samrai/CVODESolver.cc:112-258; SUNDIALS
// CVODE 5.7.0 cvNls / SPGMR algorithms restated from their published
// descriptions).
#include <algorithm>
#include <cstring>
#include <vector>

#include "oracle_api.h"
#include "oracle_common.h"

using namespace orc;

namespace {

struct OStepper {
   ampe_model_t m;
   ampe_step_params_t p;
   long N, NG;  // interior cells, ghost-box cells
   int nb = 2;  // scalar fields in y: phi, c (+ q0..q3)
   long NY = 0; // nb * N
   std::vector<double> q_g, q_lag, ogm, mq, fcq[3], Dq[3];
   // static orientation field of the anisotropic phase flux (qlen ghosted
   // components; evolve_quat models use q_g instead)
   std::vector<double> qorient;
   void* fac_quat = nullptr;
   std::vector<double> phi_g, c_g, cl, cs, clr, csr, temp, phi_lag;
   std::vector<double> cl_nf, cs_nf;  // cL, cS of the last f(y) with fd_flag=0
   std::vector<double> yn, ynm1;  // NY: [phi | c | q0..q3]
   std::vector<double> Cphi, Dc[3];
   void* fac_phi = nullptr;
   void* fac_conc = nullptr;
   int nsteps_done = 0;
   int hist = 0;  // 1 when ynm1 is one step of size dt behind yn
   // variable-step BDF (params adaptive = 1): y_{n-2}, the last two step
   // sizes, the next step's size and order, steps before an order change
   // is considered, the growth cap, the number of valid back values
   std::vector<double> ynm2;
   double h_next = 0.0, h1 = 0.0, h2 = 0.0, eta_max = 1.0e4;
   int q_next = 1, qwait = 2, nhist = 0;
   double t = 0.0;
   double T_start = 0.0;  // T0 at t = 0 of a model with dTdt != 0
   ampe_step_stats_t st{};
};

// QuatIntegrator::setTemperatureField before every f(t, y)
// (QuatIntegrator.cc:3191): T0(t) of ScalarTemperatureStrategy::
// getCurrentTemperature (ScalarTemperatureStrategy.cc:57-73), or T0 + dTdt t
// of GradientTemperatureStrategy.cc:124-131 without a moving frame
void at_time(OStepper& s, double t)
{
   if (s.m.dTdt == 0.0 || s.m.temp_mode == AMPE_TEMP_FIELD) return;
   double T = s.T_start + s.m.dTdt * t;
   if (s.m.temp_mode == AMPE_TEMP_CONSTANT) {
      if (s.m.dTdt < 0.0 && T < s.m.T_target)
         T = s.m.T_target;
      else if (s.m.T_target > 0.0 && s.m.dTdt > 0.0 && T > s.m.T_target)
         T = s.m.T_target;
   }
   s.m.T0 = T;
}

void to_ghosted(const OStepper& s, const double* src, std::vector<double>& g)
{
   Layout L(s.m);
   for (int k = 0; k < L.n2; k++)
      for (int j = 0; j < L.n1; j++)
         for (int i = 0; i < L.n0; i++)
            g[L.c(i, j, k)] = src[L.interior(i, j, k)];
   orc_fill_ghosts(&s.m, g.data());
}

void from_ghosted(const OStepper& s, const std::vector<double>& g, double* dst)
{
   Layout L(s.m);
   for (int k = 0; k < L.n2; k++)
      for (int j = 0; j < L.n1; j++)
         for (int i = 0; i < L.n0; i++)
            dst[L.interior(i, j, k)] = g[L.c(i, j, k)];
}

const double* temp_ptr(const OStepper& s)
{
   return s.m.temp_mode == AMPE_TEMP_FIELD ? s.temp.data() : nullptr;
}

// f(y): fd_flag != 0 lags the face diffusivities (QuatIntegrator.cc:3189,
// 3262-3263).
void eval_rhs(OStepper& s, const double* y, double* fy, int fd_flag)
{
   to_ghosted(s, y, s.phi_g);
   to_ghosted(s, y + s.N, s.c_g);
   const bool quat = s.m.evolve_quat != 0;
   if (quat)
      for (int c = 0; c < 4; c++) {
         std::vector<double> tmp(s.NG);
         to_ghosted(s, y + (2 + c) * s.N, tmp);
         std::copy(tmp.begin(), tmp.end(), s.q_g.begin() + c * s.NG);
      }
   long nfail = 0;
   long its = orc_phase_concentrations(&s.m, temp_ptr(s), s.phi_g.data(),
                                       s.c_g.data(), s.clr.data(),
                                       s.csr.data(), s.cl.data(), s.cs.data(),
                                       &nfail);
   s.st.kks_iters += its;
   s.st.kks_fail += nfail;
   if (!fd_flag) {
      s.phi_lag = s.phi_g;
      s.cl_nf = s.cl;
      s.cs_nf = s.cs;
      if (quat) {  // QuatIntegrator::computeQuatGradients, lagged in FD calls
         s.q_lag = s.q_g;
         orc_quat_grad_modulus(&s.m, s.q_lag.data(), s.ogm.data());
      }
   }
   const double* qflux = nullptr;
   if (s.m.flux_type == AMPE_FLUX_ANISOTROPIC)
      qflux = quat ? s.q_g.data() : s.qorient.data();
   orc_rhs_phase_conc_qd(&s.m, s.phi_g.data(), qflux, temp_ptr(s), s.cl.data(),
                         s.cs.data(), s.phi_lag.data(), s.cl_nf.data(), s.cs_nf.data(),
                         quat ? s.ogm.data() : nullptr, fy, fy + s.N);
   if (s.m.conc_form == AMPE_CONC_KKS) {
      // "kks" composition form: coefficients from the lagged phi, cL, cS
      // (QuatIntegrator.cc:3266-3267), differences of the current phi and c
      Layout L(s.m);
      std::vector<double> f0(L.nfx()), f1(L.nfy()), f2(L.dim == 3 ? L.nfz() : 1);
      orc_conc_flux_kks(&s.m, s.phi_lag.data(), s.cl_nf.data(), s.cs_nf.data(), temp_ptr(s),
                        s.phi_g.data(), s.c_g.data(), f0.data(), f1.data(), f2.data());
      orc_computerhsconcentration(&s.m, f0.data(), f1.data(), f2.data(), fy + s.N);
   }
   if (quat) {
      orc_quat_mobility(&s.m, s.phi_g.data(), s.mq.data());
      orc_quat_face_coef(&s.m, s.phi_g.data(), temp_ptr(s), s.q_lag.data(),
                         s.fcq[0].data(), s.fcq[1].data(), s.fcq[2].data());
      orc_quat_rhs(&s.m, s.fcq[0].data(), s.fcq[1].data(), s.fcq[2].data(),
                   s.mq.data(), s.q_g.data(), fy + 2 * s.N);
   }
   s.st.rhs_evals++;
}

double wrms(const OStepper& s, const double* v, const double* w)
{
   double acc = 0.0;
   #pragma omp parallel for reduction(+ : acc) schedule(static)
   for (long c = 0; c < s.NY; c++) {
      const double x = v[c] * w[c];
      acc += x * x;
   }
   return std::sqrt(acc / (double)s.NY);
}

// PhaseFACOps::setOperatorCoefficients + ConcFACOps::setOperatorCoefficients
// at the state whose phi is in s.phi_g (C) and s.phi_lag (face D).
void precond_setup(OStepper& s, double gamma)
{
   Layout L(s.m);
   orc_phase_fac_set_c(&s.m, s.phi_g.data(), gamma, s.Cphi.data());
   orc_fill_ghosts(&s.m, s.Cphi.data());
   const double eps2 = s.m.epsilon_phi * s.m.epsilon_phi;
   orc_fac_set_operator(s.fac_phi, nullptr, nullptr, nullptr, -gamma * eps2,
                        s.Cphi.data(), 0.0, nullptr, s.m.phase_mobility);
   // composition: D = -gamma (D_L + D_S), C = 1, M = M_c
   std::vector<double> l0(L.nfx()), l1(L.nfy()), l2(L.dim == 3 ? L.nfz() : 1);
   std::vector<double> s0(L.nfx()), s1(L.nfy()), s2(l2.size());
   ampe_model_t mp = s.m;  // the "kks" form's D0 uses the energy interpolation
   if (s.m.conc_form == AMPE_CONC_KKS) mp.diff_interp = s.m.energy_interp;
   orc_conc_diffusion_model(&mp, s.phi_lag.data(), temp_ptr(s), s.cl_nf.data(),
                            s.cs_nf.data(), l0.data(), l1.data(), l2.data(), s0.data(),
                            s1.data(), s2.data());
   for (long f = 0; f < L.nfx(); f++) s.Dc[0][f] = -gamma * (l0[f] + s0[f]);
   for (long f = 0; f < L.nfy(); f++) s.Dc[1][f] = -gamma * (l1[f] + s1[f]);
   if (L.dim == 3)
      for (long f = 0; f < L.nfz(); f++) s.Dc[2][f] = -gamma * (l2[f] + s2[f]);
   orc_fac_set_operator(s.fac_conc, s.Dc[0].data(), s.Dc[1].data(),
                        L.dim == 3 ? s.Dc[2].data() : nullptr, 0.0, nullptr,
                        1.0, nullptr, s.m.conc_mobility);
   if (s.m.evolve_quat) {
      // QuatFACOps::setOperatorCoefficients: C = 1, M = M_q(phi),
      // D = gamma fc (face coefficients of the lagged gradients)
      orc_quat_mobility(&s.m, s.phi_g.data(), s.mq.data());
      orc_fill_ghosts(&s.m, s.mq.data());
      orc_quat_face_coef(&s.m, s.phi_g.data(), temp_ptr(s), s.q_lag.data(),
                         s.Dq[0].data(), s.Dq[1].data(), s.Dq[2].data());
      for (int d = 0; d < L.dim; d++)
         for (auto& x : s.Dq[d]) x *= gamma;
      orc_fac_set_operator(s.fac_quat, s.Dq[0].data(), s.Dq[1].data(),
                           L.dim == 3 ? s.Dq[2].data() : nullptr, 0.0, nullptr,
                           1.0, s.mq.data(), 0.0);
   }
   s.st.precond_setups++;
}

void precond_solve(OStepper& s, const double* r, double* z, double delta)
{
   if (s.p.precond == 0) {
      std::copy(r, r + s.NY, z);
      return;
   }
   Layout L(s.m);
   std::vector<double> fg(s.NG, 0.0), ug(s.NG, 0.0);
   for (int blk = 0; blk < s.nb; blk++) {
      to_ghosted(s, r + blk * s.N, fg);
      double res;
      void* fac = blk == 0 ? s.fac_phi : (blk == 1 ? s.fac_conc : s.fac_quat);
      int cyc = orc_fac_solve(fac, &s.p, s.p.precond, fg.data(), ug.data(),
                              delta, &res);
      s.st.fac_cycles += cyc;
      from_ghosted(s, ug, z + blk * s.N);
   }
   s.st.precond_solves++;
}

// A v = v - gamma (f(y + sig v) - f(y)) / sig, sig = 1/WRMS(v)
void matvec(OStepper& s, const double* y, const double* fy, const double* w,
            double gamma, const double* v, double* out)
{
   const long n2 = s.NY;
   const double sig = 1.0 / wrms(s, v, w);
   std::vector<double> yp(n2), fp(n2);
   for (long c = 0; c < n2; c++) yp[c] = y[c] + sig * v[c];
   eval_rhs(s, yp.data(), fp.data(), 1);
   #pragma omp parallel for schedule(static)
   for (long c = 0; c < n2; c++)
      out[c] = v[c] - gamma * (fp[c] - fy[c]) / sig;
}

// Left-preconditioned scaled GMRES, x0 = 0.  Returns iterations.
int gmres(OStepper& s, const double* y, const double* fy, const double* w,
          double gamma, const double* b, double* x, double tol)
{
   const long n2 = s.NY;
   const int maxl = s.p.max_krylov;
   const double sqrtN = std::sqrt((double)n2);
   std::vector<std::vector<double>> V(maxl + 1, std::vector<double>(n2));
   std::vector<double> H((maxl + 1) * maxl, 0.0), g(maxl + 1, 0.0);
   std::vector<double> cs(maxl), sn(maxl), tmp(n2), av(n2);
   std::fill(x, x + n2, 0.0);
   precond_solve(s, b, tmp.data(), tol * sqrtN);
   for (long c = 0; c < n2; c++) V[0][c] = w[c] * tmp[c];
   double beta = 0.0;
   for (long c = 0; c < n2; c++) beta += V[0][c] * V[0][c];
   beta = std::sqrt(beta);
   if (beta / sqrtN <= tol) return 0;
   for (long c = 0; c < n2; c++) V[0][c] /= beta;
   g[0] = beta;
   int l = 0;
   for (; l < maxl; l++) {
      for (long c = 0; c < n2; c++) tmp[c] = V[l][c] / w[c];
      matvec(s, y, fy, w, gamma, tmp.data(), av.data());
      precond_solve(s, av.data(), tmp.data(), tol * sqrtN);
      for (long c = 0; c < n2; c++) V[l + 1][c] = w[c] * tmp[c];
      for (int i = 0; i <= l; i++) {  // modified Gram-Schmidt
         double h = 0.0;
         for (long c = 0; c < n2; c++) h += V[i][c] * V[l + 1][c];
         H[i * maxl + l] = h;
         for (long c = 0; c < n2; c++) V[l + 1][c] -= h * V[i][c];
      }
      double hn = 0.0;
      for (long c = 0; c < n2; c++) hn += V[l + 1][c] * V[l + 1][c];
      hn = std::sqrt(hn);
      H[(l + 1) * maxl + l] = hn;
      if (hn > 0.0)
         for (long c = 0; c < n2; c++) V[l + 1][c] /= hn;
      // apply previous Givens rotations to column l
      for (int i = 0; i < l; i++) {
         const double a = H[i * maxl + l], bb = H[(i + 1) * maxl + l];
         H[i * maxl + l] = cs[i] * a + sn[i] * bb;
         H[(i + 1) * maxl + l] = -sn[i] * a + cs[i] * bb;
      }
      const double a = H[l * maxl + l], bb = H[(l + 1) * maxl + l];
      const double rr = std::sqrt(a * a + bb * bb);
      cs[l] = a / rr;
      sn[l] = bb / rr;
      H[l * maxl + l] = rr;
      H[(l + 1) * maxl + l] = 0.0;
      g[l + 1] = -sn[l] * g[l];
      g[l] = cs[l] * g[l];
      if (std::fabs(g[l + 1]) / sqrtN <= tol || hn == 0.0) {
         l++;
         break;
      }
   }
   const int k = std::min(l, maxl);
   std::vector<double> yk(k, 0.0);
   for (int i = k - 1; i >= 0; i--) {
      double acc = g[i];
      for (int j = i + 1; j < k; j++) acc -= H[i * maxl + j] * yk[j];
      yk[i] = acc / H[i * maxl + i];
   }
   for (int i = 0; i < k; i++)
      for (long c = 0; c < n2; c++) x[c] += yk[i] * V[i][c];
   for (long c = 0; c < n2; c++) x[c] /= w[c];
   return k;
}

// Newton iteration of one BDF step, y - gamma f(y) = a, from the predictor
// in y; convergence test del min(1, crate) <= newton_coef.  0 on
// convergence (result in ynew), 1 on Newton failure.  w receives the WRMS
// weights of y_n.
int bdf_newton(OStepper& s, const std::vector<double>& a, std::vector<double>& y,
               double gamma, double newton_coef, std::vector<double>& w,
               std::vector<double>& ynew)
{
   const long n2 = s.NY;
   std::vector<double> fy(n2), b(n2), d(n2);
   w.resize(n2);
   #pragma omp parallel for schedule(static)
   for (long c = 0; c < n2; c++)
      w[c] = 1.0 / (s.p.rtol * std::fabs(s.yn[c]) + s.p.atol);
   double crate = 1.0, delp = 0.0;
   const double lintol = s.p.lin_coef * newton_coef;
   for (int it = 0; it < s.p.max_newton; it++) {
      eval_rhs(s, y.data(), fy.data(), 0);
      if (it == 0 && s.p.precond) precond_setup(s, gamma);
      for (long c = 0; c < n2; c++) b[c] = -(y[c] - gamma * fy[c] - a[c]);
      const int li = gmres(s, y.data(), fy.data(), w.data(), gamma, b.data(),
                           d.data(), lintol);
      s.st.gmres_iters += li;
      s.st.newton_iters++;
      for (long c = 0; c < n2; c++) y[c] += d[c];
      const double del = wrms(s, d.data(), w.data());
      if (it > 0) crate = std::max(0.3 * crate, del / delp);
      const double dcon = del * std::min(1.0, crate) / newton_coef;
      if (dcon <= 1.0) {
         ynew = y;
         // projection of the accepted state (QuatIntegrator::applyProjection,
         // QuatIntegrator.cc:3911-3940; project3d)
         if (s.m.evolve_quat) orc_quat_project(s.N, ynew.data() + 2 * s.N);
         return 0;
      }
      if (it >= 1 && del > 2.0 * delp) break;
      delp = del;
   }
   s.st.newton_fail++;
   return 1;
}

// One BDF step of size h and order q from yn (and ynm1 for q=2), ending at
// t_end; constant-step coefficients, linear-extrapolation predictor.
// Returns 0 on convergence, 1 on Newton failure.
int bdf_step(OStepper& s, double t_end, double h, int q, std::vector<double>& ynew)
{
   at_time(s, t_end);
   const long n2 = s.NY;
   std::vector<double> a(n2), y(n2), w;
   double gamma;
   if (q == 1) {
      gamma = h;
      #pragma omp parallel for schedule(static)
      for (long c = 0; c < n2; c++) {
         a[c] = s.yn[c];
         y[c] = s.yn[c];
      }
   } else {
      gamma = 2.0 * h / 3.0;
      #pragma omp parallel for schedule(static)
      for (long c = 0; c < n2; c++) {
         a[c] = (4.0 * s.yn[c] - s.ynm1[c]) / 3.0;
         y[c] = 2.0 * s.yn[c] - s.ynm1[c];
      }
   }
   return bdf_newton(s, a, y, gamma, s.p.newton_coef, w, ynew);
}

// ---- variable-step BDF of orders 1 and 2 with CVODE's error control ----
// (the GPU stepper's adaptive mode restated; the rules are SUNDIALS CVODE
// 5.7.0's published ones: error test dsm = c ||y_{n+1} - pred||_WRMS <= 1,
// Newton test with 0.1 / c, eta = 1/((6 dsm)^(1/(q+1)) + 1e-6), order
// candidates every q+1 steps with biases 6 and 10, threshold 1.5, growth
// caps 1e4 / 10 / 1 after failures, error-test failures eta >= 0.1, <= 0.2
// from the second, order 1 from the third, 7 at most; Newton failures
// eta = 0.25, 10 at most.)

// the predictor pred = k0 y_n + k1 y_{n-1} + k2 y_{n-2} + k3 f(y_n) and the
// error constant c of LTE ~ c (y_{n+1} - pred): explicit Euler without
// history (c = 1/2); linear extrapolation for order 1 (c = w / (2w+1),
// w = h / h_{n-1}); quadratic extrapolation for order 2 (c = A / (P + A),
// A = h^3 (1+w)^2 / (w (1+2w)), P = h (h+h1)(h+h1+h2))
struct OPred {
   double k0, k1, k2, k3, c;
};
OPred predictor(const OStepper& s, double h, int q)
{
   OPred P{1.0, 0.0, 0.0, 0.0, 0.5};
   if (s.nhist == 0) {
      P.k3 = h;
      return P;
   }
   const double h1 = s.h1, w = h / h1;
   if (q == 1) {
      P.k0 = 1.0 + w;
      P.k1 = -w;
      P.c = w / (2.0 * w + 1.0);
      return P;
   }
   const double h2 = s.h2;
   P.k0 = (h + h1) * (h + h1 + h2) / (h1 * (h1 + h2));
   P.k1 = -h * (h + h1 + h2) / (h1 * h2);
   P.k2 = h * (h + h1) / ((h1 + h2) * h2);
   const double A = h * h * h * (1.0 + w) * (1.0 + w) / (w * (1.0 + 2.0 * w));
   const double Pp = h * (h + h1) * (h + h1 + h2);
   P.c = A / (Pp + A);
   return P;
}

double wrms_comb(const OStepper& s, const std::vector<double>& w, const double* v0,
                 double c0, const double* v1, double c1, const double* v2, double c2,
                 const double* v3, double c3)
{
   std::vector<double> x(s.NY);
   for (long t = 0; t < s.NY; t++) {
      double v = c0 * v0[t] + c1 * v1[t];
      if (v2) v += c2 * v2[t];
      if (v3) v += c3 * v3[t];
      x[t] = v;
   }
   return wrms(s, x.data(), w.data());
}

void restart_history(OStepper& s)
{
   s.nhist = 0;
   s.q_next = 1;
   s.qwait = 2;
   s.h_next = s.p.dt;
   s.h1 = s.h2 = 0.0;
   s.eta_max = 1.0e4;
}

// one accepted variable step, not past t_stop (> t); 0 ok, 1 failed
int adaptive_step(OStepper& s, double t_stop)
{
   const long n2 = s.NY;
   const double hmax = s.p.h_max > 0.0 ? s.p.h_max : 1.0e300;
   std::vector<double> fn;
   if (s.nhist == 0) {
      fn.resize(n2);
      at_time(s, s.t);
      eval_rhs(s, s.yn.data(), fn.data(), 0);
   }
   std::vector<double> a(n2), y(n2), w, ynew;
   int nef = 0, ncf = 0;
   for (;;) {
      int q = std::min(s.q_next, std::min(2, s.p.max_order));
      if (s.nhist < q) q = s.nhist < 1 ? 1 : s.nhist;
      double h = std::min(s.h_next, hmax);
      if (t_stop > s.t && s.t + h > t_stop - 1e-12 * std::fabs(t_stop)) h = t_stop - s.t;
      const OPred P = predictor(s, h, q);
      double gamma = h, a0 = 1.0, a1 = 0.0;
      if (q == 2) {
         const double wr = h / s.h1;
         a0 = (1.0 + wr) * (1.0 + wr) / (1.0 + 2.0 * wr);
         a1 = -wr * wr / (1.0 + 2.0 * wr);
         gamma = h * (1.0 + wr) / (1.0 + 2.0 * wr);
      }
      for (long t = 0; t < n2; t++) {
         double pr = P.k0 * s.yn[t];
         if (s.nhist >= 1) pr += P.k1 * s.ynm1[t];
         if (q == 2) pr += P.k2 * s.ynm2[t];
         if (s.nhist == 0) pr += P.k3 * fn[t];
         y[t] = pr;
         a[t] = q == 2 ? a0 * s.yn[t] + a1 * s.ynm1[t] : s.yn[t];
      }
      at_time(s, s.t + h);
      if (bdf_newton(s, a, y, gamma, 0.1 / P.c, w, ynew)) {
         ncf++;
         if (ncf >= 10 || h <= s.p.h_min) return 1;
         s.h_next = h * 0.25;
         s.eta_max = 1.0;
         continue;
      }
      const double dsm =
          P.c * wrms_comb(s, w, ynew.data(), 1.0, s.yn.data(), -P.k0,
                          s.nhist >= 1 ? s.ynm1.data() : nullptr, -P.k1,
                          q == 2 ? s.ynm2.data() : (s.nhist == 0 ? fn.data() : nullptr),
                          q == 2 ? -P.k2 : -P.k3);
      if (dsm > 1.0) {
         nef++;
         s.st.err_test_fails++;
         if (nef >= 7 || h <= s.p.h_min) return 1;
         double eta = 1.0 / (std::pow(6.0 * dsm, 1.0 / (q + 1)) + 1.0e-6);
         eta = std::max(0.1, eta);
         if (nef >= 2) eta = std::min(eta, 0.2);
         if (nef >= 3) s.q_next = 1;
         s.h_next = h * eta;
         s.eta_max = 1.0;
         continue;
      }
      double eta = 1.0 / (std::pow(6.0 * dsm, 1.0 / (q + 1)) + 1.0e-6);
      int qn = q;
      if (--s.qwait <= 0) {
         if (q == 2) {
            const double h1 = s.h1;
            const double ca = 1.0 / (h * (h + h1)), cb = 1.0 / (h1 * (h + h1));
            const double dsm1 = wrms_comb(s, w, ynew.data(), h * h * ca, s.yn.data(),
                                          -h * h * (ca + cb), s.ynm1.data(), h * h * cb,
                                          nullptr, 0.0);
            const double em = 1.0 / (std::pow(6.0 * dsm1, 0.5) + 1.0e-6);
            if (em > eta) {
               eta = em;
               qn = 1;
            }
         } else if (s.p.max_order >= 2 && s.nhist >= 2) {
            const double h1 = s.h1, h2 = s.h2;
            const double t0 = h, t1 = 0.0, t2 = -h1, t3 = -h1 - h2;
            const double w0 = 1.0 / ((t0 - t1) * (t0 - t2) * (t0 - t3));
            const double w1 = 1.0 / ((t1 - t0) * (t1 - t2) * (t1 - t3));
            const double w2 = 1.0 / ((t2 - t0) * (t2 - t1) * (t2 - t3));
            const double w3 = 1.0 / ((t3 - t0) * (t3 - t1) * (t3 - t2));
            const double k = 4.0 / 3.0 * h * h * h;
            const double dsm2 = wrms_comb(s, w, ynew.data(), k * w0, s.yn.data(), k * w1,
                                          s.ynm1.data(), k * w2, s.ynm2.data(), k * w3);
            const double ep = 1.0 / (std::pow(10.0 * dsm2, 1.0 / 3.0) + 1.0e-6);
            if (ep > eta) {
               eta = ep;
               qn = 2;
            }
         }
         s.qwait = qn + 1;
      }
      if (eta < 1.5) {
         eta = 1.0;
         qn = q;
      } else {
         eta = std::min(eta, s.eta_max);
      }
      if (nef || ncf) eta = std::min(eta, 1.0);
      s.eta_max = 10.0;
      s.h_next = std::min(h * eta, hmax);
      s.q_next = qn;
      s.ynm2.swap(s.ynm1);
      s.ynm1.swap(s.yn);
      s.yn.swap(ynew);
      s.h2 = s.h1;
      s.h1 = h;
      s.nhist = std::min(s.nhist + 1, 2);
      s.t += h;
      s.st.h_last = h;
      s.st.q_last = q;
      return 0;
   }
}

}  // namespace

extern "C" {

void* orc_stepper_create(const ampe_model_t* m, const ampe_step_params_t* p)
{
   OStepper* s = new OStepper;
   s->m = *m;
   s->T_start = m->T0;
   s->p = *p;
   Layout L(*m);
   s->N = L.cells();
   s->NG = L.cells_ghost();
   for (auto* v : {&s->phi_g, &s->c_g, &s->cl, &s->cs, &s->clr, &s->csr,
                   &s->phi_lag, &s->Cphi})
      v->assign(s->NG, 0.0);
   s->temp.assign(s->NG, m->T0);
   s->Dc[0].assign(L.nfx(), 0.0);
   s->Dc[1].assign(L.nfy(), 0.0);
   s->Dc[2].assign(L.dim == 3 ? L.nfz() : 1, 0.0);
   s->nb = m->evolve_quat ? 6 : 2;
   if (m->flux_type == AMPE_FLUX_ANISOTROPIC && !m->evolve_quat) {
      // default orientation: q = (1, 0, ...), angle 0
      s->qorient.assign((size_t)m->qlen * s->NG, 0.0);
      std::fill(s->qorient.begin(), s->qorient.begin() + s->NG, 1.0);
   }
   s->NY = s->nb * s->N;
   s->yn.assign(s->NY, 0.0);
   s->ynm1.assign(s->NY, 0.0);
   s->ynm2.assign(s->NY, 0.0);
   s->h_next = p->dt;
   const int nl = p->precond == 2 ? p->mg_levels : 1;
   s->fac_phi = orc_fac_create(m, nl);
   s->fac_conc = orc_fac_create(m, nl);
   if (m->evolve_quat) {
      s->q_g.assign(4 * s->NG, 0.0);
      s->q_lag.assign(4 * s->NG, 0.0);
      s->ogm.assign(s->N, 0.0);
      s->mq.assign(s->NG, 0.0);
      const long nf[3] = {L.nfx(), L.nfy(), L.dim == 3 ? L.nfz() : 1};
      for (int d = 0; d < 3; d++) {
         s->fcq[d].assign(nf[d], 0.0);
         s->Dq[d].assign(nf[d], 0.0);
      }
      s->fac_quat = orc_fac_create(m, nl);
   }
   return s;
}

void orc_stepper_destroy(void* h)
{
   OStepper* s = (OStepper*)h;
   orc_fac_destroy(s->fac_phi);
   orc_fac_destroy(s->fac_conc);
   if (s->fac_quat) orc_fac_destroy(s->fac_quat);
   delete s;
}

void orc_stepper_set_state(void* h, const double* phi, const double* conc,
                           const double* cl, const double* cs,
                           const double* temp)
{
   OStepper* s = (OStepper*)h;
   std::copy(phi, phi + s->N, s->yn.begin());
   std::copy(conc, conc + s->N, s->yn.begin() + s->N);
   if (s->m.evolve_quat)  // default orientation (1,0,0,0) until set_quat
      for (int c = 0; c < 4; c++)
         std::fill(s->yn.begin() + (2 + c) * s->N, s->yn.begin() + (3 + c) * s->N,
                   c == 0 ? 1.0 : 0.0);
   s->ynm1 = s->yn;
   to_ghosted(*s, cl ? cl : conc, s->clr);
   to_ghosted(*s, cs ? cs : conc, s->csr);
   s->cl = s->clr;
   s->cs = s->csr;
   s->cl_nf = s->clr;
   s->cs_nf = s->csr;
   s->hist = 0;
   restart_history(*s);
   if (temp) to_ghosted(*s, temp, s->temp);
   s->nsteps_done = 0;
   s->t = 0.0;
}

void orc_stepper_get_state(void* h, double* phi, double* conc, double* cl,
                           double* cs)
{
   OStepper* s = (OStepper*)h;
   if (phi) std::copy(s->yn.begin(), s->yn.begin() + s->N, phi);
   if (conc) std::copy(s->yn.begin() + s->N, s->yn.begin() + 2 * s->N, conc);
   if (cl) from_ghosted(*s, s->clr, cl);
   if (cs) from_ghosted(*s, s->csr, cs);
}

void orc_stepper_set_quat(void* h, const double* q)
{
   OStepper* s = (OStepper*)h;
   if (!s->m.evolve_quat) return;
   std::copy(q, q + 4 * s->N, s->yn.begin() + 2 * s->N);
   std::copy(q, q + 4 * s->N, s->ynm1.begin() + 2 * s->N);
   s->hist = 0;
   restart_history(*s);
}

// static orientation (qlen interior components) of the anisotropic flux
void orc_stepper_set_orientation(void* h, const double* q)
{
   OStepper* s = (OStepper*)h;
   if (s->qorient.empty()) return;
   std::vector<double> tmp(s->NG);
   for (int c = 0; c < s->m.qlen; c++) {
      to_ghosted(*s, q + c * s->N, tmp);
      std::copy(tmp.begin(), tmp.end(), s->qorient.begin() + c * s->NG);
   }
}

void orc_stepper_get_quat(void* h, double* q)
{
   OStepper* s = (OStepper*)h;
   if (s->m.evolve_quat) std::copy(s->yn.begin() + 2 * s->N, s->yn.end(), q);
}

void orc_stepper_eval_rhs(void* h, double* phi_rhs, double* conc_rhs)
{
   OStepper* s = (OStepper*)h;
   std::vector<double> fy(s->NY);
   at_time(*s, s->t);
   eval_rhs(*s, s->yn.data(), fy.data(), 0);
   std::copy(fy.begin(), fy.begin() + s->N, phi_rhs);
   std::copy(fy.begin() + s->N, fy.begin() + 2 * s->N, conc_rhs);
}

// f(y_n) over the whole state vector (NY doubles)
void orc_stepper_eval_rhs_full(void* h, double* out)
{
   OStepper* s = (OStepper*)h;
   at_time(*s, s->t);
   eval_rhs(*s, s->yn.data(), out, 0);
}

long orc_stepper_size(void* h) { return ((OStepper*)h)->NY; }

// Advance nsteps accepted steps.  Returns 0, or 1 if a step failed after
// max_retries step-size halvings.
// variable steps until t_stop (if > t) or max_steps; 0 ok, 1 failed
static int advance_adaptive(OStepper* s, double t_stop, int max_steps)
{
   // a stop time not in the past (at t already: no step); earlier: none
   const double eps = 1e-12 * std::fabs(t_stop);
   const bool has_stop = t_stop >= s->t - eps;
   for (int n = 0; n < max_steps; n++) {
      if (has_stop && s->t >= t_stop - eps) break;
      if (adaptive_step(*s, t_stop)) return 1;
      s->clr = s->cl_nf;  // QuatModel::resetRefPhaseConcentrations
      s->csr = s->cs_nf;
      s->nsteps_done++;
      s->st.steps++;
   }
   return 0;
}

int orc_stepper_advance_to(void* h, double t_stop, int max_steps, ampe_step_stats_t* stats)
{
   OStepper* s = (OStepper*)h;
   const int rc = advance_adaptive(s, t_stop, max_steps);
   s->st.t = s->t;
   s->st.h_next = s->h_next;
   s->st.q_next = s->q_next;
   if (stats) *stats = s->st;
   return rc;
}

void orc_stepper_set_temperature(void* h, double T0, double gradT)
{
   OStepper* s = (OStepper*)h;
   if (s->m.dTdt != 0.0) return;  // T follows the model's T0(t)
   s->m.T0 = T0;
   s->m.gradT = gradT;
}

int orc_stepper_advance(void* h, int nsteps, ampe_step_stats_t* stats)
{
   OStepper* s = (OStepper*)h;
   if (s->p.adaptive) return orc_stepper_advance_to(h, -1.0e300, nsteps, stats);
   std::vector<double> ynew;
   int ret = 0;
   for (int n = 0; n < nsteps; n++) {
      double hstep = s->p.dt;
      int q = s->hist ? std::min(2, s->p.max_order) : 1;
      int fail = bdf_step(*s, s->t + hstep, hstep, q, ynew);
      int retries = 0;
      if (fail) {
         // order-1 sub-steps: after each failure halve the sub-step and go
         // on from the last accepted sub-step until the whole step is
         // covered; if the retries run out, the step's start is restored
         const std::vector<double> ysave = s->yn, ym1save = s->ynm1;
         double done = 0.0, hsub = hstep;
         while (fail && retries < s->p.max_retries) {
            retries++;
            s->st.step_retries++;
            hsub *= 0.5;
            fail = 0;
            while (done < hstep * (1.0 - 1e-12)) {
               const double hh = std::min(hsub, hstep - done);
               if (bdf_step(*s, s->t + done + hh, hh, 1, ynew)) {
                  fail = 1;
                  break;
               }
               done += hh;
               if (done < hstep * (1.0 - 1e-12)) {  // accept the sub-step
                  s->ynm1 = s->yn;
                  s->yn = ynew;
               }
            }
         }
         if (fail) {
            s->yn = ysave;
            s->ynm1 = ym1save;
         }
      }
      if (fail) {
         ret = 1;
         break;
      }
      s->hist = retries == 0 ? 1 : 0;
      s->ynm1 = s->yn;
      s->yn = ynew;
      s->clr = s->cl_nf;  // QuatModel::resetRefPhaseConcentrations
      s->csr = s->cs_nf;
      s->nsteps_done++;
      s->t += s->p.dt;
      s->st.steps++;
      s->st.h_last = s->p.dt;
      s->st.q_last = q;
   }
   s->st.t = s->t;
   s->st.h_next = s->p.dt;
   s->st.q_next = s->hist ? std::min(2, s->p.max_order) : 1;
   if (stats) *stats = s->st;
   return ret;
}

// out = v - gamma J v at the current state y_n: finite differences of f
// (analytic = 0, the CVODE product) or the analytic linearisation.
void orc_stepper_jv(void* h, const double* v, double gamma, double* out,
                    int analytic)
{
   OStepper* s = (OStepper*)h;
   const long n2 = s->NY;
   std::vector<double> fy(n2), w(n2);
   at_time(*s, s->t);
   eval_rhs(*s, s->yn.data(), fy.data(), 0);
   for (long c = 0; c < n2; c++)
      w[c] = 1.0 / (s->p.rtol * std::fabs(s->yn[c]) + s->p.atol);
   if (analytic)
      orc_jv_analytic(&s->m, s->phi_g.data(), s->cl.data(), s->cs.data(), v,
                      gamma, out);
   else
      matvec(*s, s->yn.data(), fy.data(), w.data(), gamma, v, out);
}

}  // extern "C"
