// Mixed-precision kernels of the phi + c implicit step.
//
// The outer Newton residual G(y) = y - gamma f(y) - a, the Krylov vectors,
// their inner products and the WRMS norms stay FP64 (stepper.cu).  Inside:
//  k_kks_f32 /   per-cell KKS Newton in FP32 (logf, FP32 Redlich-Kister
//  k_kks_polish64 polynomials); cells whose solution lies within 1e-4 of
//                c = 0 or 1 (or that FP32 did not converge) are listed and
//                get an FP64 Newton polish from the FP32 result (and an FP64
//                driving force) in a second kernel over the list.  Optional
//                initial guess from the surrogate MLP; cells not converged
//                within 3 iterations from it restart from the plain warm
//                start.
//  k_rhs_mixed   the fused phase + composition right-hand side in FP32
//                arithmetic, FP64 in/out.
//  k_jv_point /  the Jacobian-vector product of f written out analytically
//  k_jv_stencil  (linearised KKS split from its own 2x2 Jacobian, the
//                chemical driving force, the well, the flux stencils with
//                the diffusivities held fixed as the reference's
//                finite-difference products hold them, QuatIntegrator.cc:
//                3189, 3262-3263), in FP32.
//  k_quat_cells_f32 / k_quat_faces_f32 / k_jv_quat
//                the quaternion equation of evolve_quat models in FP32:
//                |grad q|, M_q, the face coefficients and their phi
//                derivative, and the q rows of the Jacobian-vector product
//                (gradients lagged as in the finite-difference products).
#include "common.cuh"
#include "mixed.cuh"
#include "phase_flux.cuh"
#include "quat.cuh"

namespace ampe {

__device__ __forceinline__ CoefF to_f(const ThermoCoef& t)
{
   CoefF f;
   f.RT = (float)t.RT;
   f.iRT = (float)t.iRT;
   for (int p = 0; p < 2; p++) {
      f.dG[p] = (float)t.dG[p];
      f.GB[p] = (float)t.GB[p];
      for (int k = 0; k < 4; k++) f.L[p][k] = (float)t.L[p][k];
   }
   return f;
}

__device__ __forceinline__ void rk_f(const float* L, float u, float& S,
                                     float& S1, float& S2)
{
   S = L[0] + u * (L[1] + u * (L[2] + u * L[3]));
   S1 = L[1] + u * (2.f * L[2] + u * 3.f * L[3]);
   S2 = 2.f * L[2] + u * 6.f * L[3];
}

__device__ __forceinline__ float xi_f(const CoefF& th, float c, int p)
{
   const float u = 2.f * c - 1.f;
   float S, S1, S2;
   rk_f(th.L[p], u, S, S1, S2);
   return th.dG[p] - u * S + c * (1.f - c) * 2.f * S1;
}

__device__ __forceinline__ float dxi_f(const CoefF& th, float c, int p)
{
   const float u = 2.f * c - 1.f;
   float S, S1, S2;
   rk_f(th.L[p], u, S, S1, S2);
   return -2.f * S - 4.f * u * S1 + 4.f * c * (1.f - c) * S2;
}

constexpr float kEdge = 1.0e-4f;  // FP64 polish within this of c = 0 or 1

__device__ __forceinline__ bool near_bound(float a)
{
   return a < kEdge || a > 1.f - kEdge;
}

// FP32 Newton; returns iterations (>0) or -1 when not converged within
// max_its (or a non-finite iterate).
__device__ __forceinline__ int kks_newton_f32(const CoefF& th, float h,
                                              float c, float x[2],
                                              int max_its)
{
   for (int it = 1; it <= max_its; it++) {
      const float a = x[0], b = x[1];
      const float F0 = (1.f - h) * a + h * b - c;
      const float F1 = logf(a * (1.f - b) / ((1.f - a) * b)) +
                       (xi_f(th, a, 0) - xi_f(th, b, 1)) * th.iRT;
      const float J00 = 1.f - h, J01 = h;
      const float J10 = 1.f / (a * (1.f - a)) + dxi_f(th, a, 0) * th.iRT;
      const float J11 = -1.f / (b * (1.f - b)) - dxi_f(th, b, 1) * th.iRT;
      const float idet = 1.f / (J00 * J11 - J01 * J10);
      const float d0 = (F0 * J11 - F1 * J01) * idet;
      const float d1 = (J00 * F1 - J10 * F0) * idet;
      float na = a - d0, nb = b - d1;
      if (na <= 0.f) na = 0.5f * a;
      if (na >= 1.f) na = 0.5f * (1.f + a);
      if (nb <= 0.f) nb = 0.5f * b;
      if (nb >= 1.f) nb = 0.5f * (1.f + b);
      x[0] = na;
      x[1] = nb;
      if (fmaxf(fabsf(d0), fabsf(d1)) < 2.0e-6f) return it;
      if (!(isfinite(na) && isfinite(nb))) return -1;
   }
   return -1;
}

__device__ __forceinline__ double driving_force_scaled(const ampe_model_t& m,
                                                       const ThermoCoef& th,
                                                       double a, double b)
{
   // (fL - fS) - muS (a - b) in FP64 (fused.cu writes the same quantity)
   const double fl = free_energy_of(th, a, 0) * m.inv_molar_volume[0];
   const double fa = free_energy_of(th, b, 1) * m.inv_molar_volume[1];
   const double mu = dfdc_of(th, b, 1) * m.inv_molar_volume[1];
   return (fl - fa) - mu * (a - b);
}

__device__ __forceinline__ float driving_force_f32(const CoefF& th, float a,
                                                   float b)
{
   const float ua = 2.f * a - 1.f, ub = 2.f * b - 1.f;
   float SLa, S1La, S2La, SSb, S1Sb, S2Sb;
   rk_f(th.L[0], ua, SLa, S1La, S2La);
   rk_f(th.L[1], ub, SSb, S1Sb, S2Sb);
   // ln(a/b) = log1p((a-b)/b) and ln((1-a)/(1-b)) = log1p((b-a)/(1-b)): the
   // arguments of the logarithms are near one for a ~ b and for dilute
   // compositions; log1p of the exactly formed difference keeps FP32
   // relative accuracy there
   const float ideal =
       th.RT * (a * log1pf((a - b) / b) + (1.f - a) * log1pf((b - a) / (1.f - b)));
   const float fl = a * th.dG[0] + th.GB[0] + a * (1.f - a) * SLa;
   const float fs = b * th.dG[1] + th.GB[1] + b * (1.f - b) * SSb;
   const float xs = th.dG[1] - ub * SSb + b * (1.f - b) * 2.f * S1Sb;
   return ideal + (fl - fs) - xs * (a - b);
}

__global__ void k_build_coef_f(int n, const ThermoCoef* tab, CoefF* tabf)
{
   const int i = blockIdx.x * blockDim.x + threadIdx.x;
   if (i < n) tabf[i] = to_f(tab[i]);
}

__device__ __forceinline__ CoefF coef_f_at(const ampe_model_t& m,
                                          const Grid& g, const CoefF* tabf,
                                          const double* tfield, int i, int j,
                                          int k)
{
   if (tabf) return tabf[m.temp_mode == AMPE_TEMP_GRADIENT ? i : 0];
   return to_f(thermo_coef(m, temperature_at(m, g, tfield, i, j, k)));
}

// FP32 pass over every cell.  Cells whose FP32 Newton converged away from
// c = 0 and 1 are finished here (cL, cS with images, dF); the others are
// appended to `list` (interior index t, bit 31 set when the FP32 iterate is
// converged and is the FP64 start) for k_kks_polish64.  The rare FP64 path
// stays out of this kernel, so it runs at the FP32 path's register count.
__global__ void __launch_bounds__(256, 4)
    k_kks_f32(ampe_model_t m, MixParams mp, Grid g, const CoefF* tabf, const double* tfield,
              const double* __restrict__ phi, const double* __restrict__ conc,
              const float* __restrict__ guess_l, const float* __restrict__ guess_s,
              const float* __restrict__ clr, const float* __restrict__ csr, float* cl,
              float* cs, float* __restrict__ dF, int* __restrict__ list,
              unsigned long long* counters)
{
   // counters: [0] FP32 iterations, [3] surrogate fallbacks
   unsigned long long it32 = 0, nfb = 0;
   const float ivm = mp.ivm;
   int* const nlist = list + g.cells();
   for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
        t < g.cells(); t += (long long)gridDim.x * blockDim.x) {
      int i, j, k;
      g.ijk(t, i, j, k);
      const int ci = g.c(i, j, k);
      const CoefF tf = coef_f_at(m, g, tabf, tfield, i, j, k);
      const float h = interp_func(d2f(phi[ci]), m.conc_interp);
      const float c = d2f(conc[ci]);
      float x[2];
      int st = -1;
      if (guess_l) {
         x[0] = guess_l[t];
         x[1] = guess_s[t];
         if (!(x[0] > 0.f && x[0] < 1.f)) x[0] = c;
         if (!(x[1] > 0.f && x[1] < 1.f)) x[1] = c;
         st = kks_newton_f32(tf, h, c, x, 3);
         if (st > 0) it32 += st;
         if (st < 0) {
            it32 += 3;
            nfb++;
         }
      }
      if (st < 0) {  // plain warm start
         x[0] = clr[ci];
         x[1] = csr[ci];
         if (!(x[0] > 0.f && x[0] < 1.f)) x[0] = c;
         if (!(x[1] > 0.f && x[1] < 1.f)) x[1] = c;
         st = kks_newton_f32(tf, h, c, x, 12);
         it32 += st > 0 ? st : 12;
      }
      const float a = x[0], b = x[1];
      if (st > 0 && !near_bound(a) && !near_bound(b)) {
         cl[ci] = a;
         cs[ci] = b;
         for_each_image(g, i, j, k, [&](int idx) {
            cl[idx] = a;
            cs[idx] = b;
         });
         dF[t] = driving_force_f32(tf, a, b) * ivm;
      } else {
         if (st > 0) {  // the FP32 iterate is the FP64 polish's start
            cl[ci] = a;
            cs[ci] = b;
         }
         const int q = atomicAdd(nlist, 1);
         list[q] = (int)t | (st > 0 ? (int)0x80000000 : 0);
      }
   }
   if (counters) {
      unsigned long long v[2] = {it32, nfb};
      const int slot[2] = {0, 3};
      for (int q = 0; q < 2; q++) {
         unsigned long long x = v[q];
         for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
         if ((threadIdx.x & 31) == 0 && x) atomicAdd(&counters[slot[q]], x);
      }
   }
}

// FP64 Newton for the listed cells near c = 0 or 1, or not converged in
// FP32: from the FP32 iterate when it converged, else from the warm start
// (full FP64 Newton); FP64 driving force.
__global__ void __launch_bounds__(128)
    k_kks_polish64(ampe_model_t m, Grid g, const ThermoCoef* tab, const double* tfield,
                   const double* __restrict__ phi, const double* __restrict__ conc,
                   const float* __restrict__ clr, const float* __restrict__ csr, float* cl,
                   float* cs, float* __restrict__ dF, const int* __restrict__ list,
                   unsigned long long* counters)
{
   // counters: [1] failed cells, [2] FP64-polished cells, [4] FP64 iterations
   unsigned long long fails = 0, n64 = 0, it64 = 0;
   const int n = list[g.cells()];
   for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < n; q += gridDim.x * blockDim.x) {
      const int e = list[q];
      const int t = e & 0x7fffffff;
      int i, j, k;
      g.ijk(t, i, j, k);
      const int ci = g.c(i, j, k);
      n64++;
      const ThermoCoef th = tab ? tab[m.temp_mode == AMPE_TEMP_GRADIENT ? i : 0]
                                : thermo_coef(m, temperature_at(m, g, tfield, i, j, k));
      double xd[2];
      if (e < 0) {
         xd[0] = cl[ci];
         xd[1] = cs[ci];
      } else {
         xd[0] = clr[ci];
         xd[1] = csr[ci];
      }
      const double hd = interp_func(phi[ci], m.conc_interp);
      const int s64 = kks_newton(th, hd, conc[ci], xd, m.newton_max_its, 1.0e-10);
      if (s64 < 0) {
         fails++;
         it64 += m.newton_max_its;
      } else {
         it64 += s64;
      }
      const float a = (float)xd[0], b = (float)xd[1];
      cl[ci] = a;
      cs[ci] = b;
      for_each_image(g, i, j, k, [&](int idx) {
         cl[idx] = a;
         cs[idx] = b;
      });
      dF[t] = (float)driving_force_scaled(m, th, xd[0], xd[1]);
   }
   if (counters) {
      unsigned long long v[3] = {fails, n64, it64};
      const int slot[3] = {1, 2, 4};
      for (int q = 0; q < 3; q++) {
         unsigned long long x = v[q];
         for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
         if ((threadIdx.x & 31) == 0 && x) atomicAdd(&counters[slot[q]], x);
      }
   }
}

int build_coef_f(const ThermoCoef* tab, CoefF* tabf, int n, cudaStream_t s)
{
   k_build_coef_f<<<(n + 127) / 128, 128, 0, s>>>(n, tab, tabf);
   return launch_status();
}

int kks_mixed(const ampe_model_t& m, const MixParams& mp, const Grid& g,
              const ThermoCoef* tab, const CoefF* tabf, const double* tfield,
              const double* phi, const double* conc, const float* guess_l, const float* guess_s,
              const float* clr, const float* csr, float* cl, float* cs,
              float* dF, int* list, unsigned long long* counters, cudaStream_t s)
{
   cudaMemsetAsync(list + g.cells(), 0, sizeof(int), s);
   long long b = (g.cells() + 255) / 256;
   if (b > max_blocks(16)) b = max_blocks(16);
   k_kks_f32<<<(unsigned)b, 256, 0, s>>>(m, mp, g, tabf, tfield, phi, conc, guess_l, guess_s,
                                         clr, csr, cl, cs, dF, list, counters);
   const int rc = launch_status();
   if (rc) return rc;
   k_kks_polish64<<<(unsigned)max_blocks(4), 128, 0, s>>>(m, g, tab, tfield, phi, conc, clr,
                                                          csr, cl, cs, dF, list, counters);
   return launch_status();
}

MixParams make_mix_params(const ampe_model_t& m)
{
   MixParams p;
   const double eps2 = m.epsilon_phi * m.epsilon_phi;
   const bool iso = m.flux_type == AMPE_FLUX_ISOTROPIC && m.dim == 2;
   for (int d = 0; d < 3; d++) {
      const double dx = d < m.dim ? m.dx[d] : 1.0;
      p.dxi[d] = d < m.dim ? (float)(1.0 / dx) : 0.f;
      p.flux_dinv[d] = (float)((iso ? 1.0 / 12.0 : 1.0) * eps2 / dx);
   }
   p.w = (float)m.phase_well_scale;
   p.Mphi = (float)m.phase_mobility;
   p.Mc = (float)m.conc_mobility;
   p.Dl = (float)m.D_liquid;
   p.Ds = (float)m.D_solid;
   p.qlR = (float)(m.Q_liquid / kGasR);
   p.qsR = (float)(m.Q_solid / kGasR);
   p.ivm = (float)m.inv_molar_volume[1];
   p.tdep = (m.Q_liquid != 0.0 || m.Q_solid != 0.0) ? 1 : 0;
   p.iso = iso ? 1 : 0;
   p.misor = (float)m.misorientation_factor;
   p.eq2h = (float)(0.5 * m.epsilon_q * m.epsilon_q);
   p.epsq2 = (float)(m.epsilon_q * m.epsilon_q);
   p.qM = (float)m.quat_mobility;
   p.qMmin = (float)m.min_quat_mobility;
   p.qfloor2 = (float)(m.quat_grad_floor * m.quat_grad_floor);
   p.qmaxi = m.quat_grad_floor > 0.0 ? (float)(1.0 / m.quat_grad_floor) : 0.f;
   p.T0 = (float)m.T0;
   p.gdx = (float)(m.gradT * m.dx[0]);
   p.qfloor = m.quat_floor_type;
   p.eps = (float)m.epsilon_phi;
   p.nu = (float)m.aniso_eps;
   p.kn = (float)m.aniso_k;
   p.qlen4 = m.qlen == 4 ? 1 : 0;
   p.kksc = m.conc_form == AMPE_CONC_KKS ? 1 : 0;
   p.dq = nullptr;
   p.pb = (m.avg_type == 'a' && m.diff_interp == 'p' && m.energy_interp == 'p' &&
           m.conc_interp == 'p' && m.well_type == 'd' && m.orient_interp1 == 'p' &&
           m.orient_interp2 == 'p')
              ? 1
              : 0;
   return p;
}

// ---------------------------------------------------------------------------
// FP32 stencil helpers (DIM known at compile time)
// ---------------------------------------------------------------------------
// The functions.f type codes of the model; PB: the common set ('a' face
// average, 'p' interpolation everywhere, 'd' double well) as compile-time
// constants, so that the type dispatch folds away.
template <bool PB>
struct Types {
   char avg, diff, energy, conc, well, o1, o2;
   __device__ __forceinline__ explicit Types(const ampe_model_t& m)
       : avg(PB ? 'a' : m.avg_type),
         diff(PB ? 'p' : m.diff_interp),
         energy(PB ? 'p' : m.energy_interp),
         conc(PB ? 'p' : m.conc_interp),
         well(PB ? 'd' : m.well_type),
         o1(PB ? 'p' : m.orient_interp1),
         o2(PB ? 'p' : m.orient_interp2)
   {
   }
};
template <int DIM>
__device__ __forceinline__ float face_flux_lin(const MixParams& mp, int d,
                                               const float* pf, const Grid& g,
                                               int i, int j, int k)
{
   // linear phase flux on face d whose upper cell is (i,j,k)
   if (DIM == 3 || !mp.iso) {
      const int ei = d == 0, ej = d == 1, ek = d == 2;
      return (pf[g.c(i, j, k)] - pf[g.c(i - ei, j - ej, k - ek)]) * mp.flux_dinv[d];
   }
   auto P = [&](int a, int b) { return pf[g.c(a, b, 0)]; };
   const float dinv = mp.flux_dinv[d];
   if (d == 0)
      return dinv * ((P(i, j - 1) - P(i - 1, j - 1)) + (P(i, j) - P(i - 1, j)) * 10.f +
                     (P(i, j + 1) - P(i - 1, j + 1)));
   return dinv * ((P(i - 1, j) - P(i - 1, j - 1)) + (P(i, j) - P(i, j - 1)) * 10.f +
                  (P(i + 1, j) - P(i + 1, j - 1)));
}

// ---------------------------------------------------------------------------
// 2D anisotropic flux (anisotropic_gradient_flux, 2d/quatrhs.m4:154-256) in
// FP32 with its Jacobian.  theta = atan(dpy/dpx) (pi/2 when |dpx| <= 1e-12),
// orientation phi_o = acos(q0) (2 acos for four-component q),
// eps(theta) = eps (1 + nu cos k(theta - phi_o)), e' = d eps / d theta:
//   x faces: F = e^2 dpx - e e' dpy,   y faces: F = e^2 dpy + e e' dpx,
// and dF/d(dpx), dF/d(dpy) through theta's derivatives
// (-dpy, dpx) / (dpx^2 + dpy^2).
// ---------------------------------------------------------------------------
__global__ void k_aniso_faces_f32(MixParams mp, Grid g, const double* ph, const double* q,
                                  AnisoF a)
{
   const long long nx = g.nfx(), tot = nx + g.nfy();
   const float fthr = 1.e-12f;
   const float half_pi = 1.5707963267948966f;
   for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < tot;
        t += (long long)gridDim.x * blockDim.x) {
      int dir, i, j, k;
      face_of(g, t, dir, i, j, k);
      // neighbour differences of the FP64 phase, rounded once
      auto D = [&](int x, int y, int x2, int y2) {
         return d2f(ph[g.c(x, y, 0)] - ph[g.c(x2, y2, 0)]);
      };
      float dpx, dpy, po;
      if (dir == 0) {
         dpx = D(i, j, i - 1, j) * mp.dxi[0];
         dpy = 0.25f * (D(i - 1, j + 1, i - 1, j - 1) + D(i, j + 1, i, j - 1)) * mp.dxi[1];
         po = a.PO[0][g.fx(i, j, 0)];
      } else {
         dpx = 0.25f * (D(i + 1, j - 1, i - 1, j - 1) + D(i + 1, j, i - 1, j)) * mp.dxi[0];
         dpy = D(i, j, i, j - 1) * mp.dxi[1];
         po = a.PO[1][g.fy(i, j, 0)];
      }
      const bool steep = fabsf(dpx) > fthr;
      const float theta = steep ? atanf(dpy / dpx) : half_pi;
      float sn, cs;
      sincosf(mp.kn * (theta - po), &sn, &cs);
      const float e = mp.eps * (1.f + mp.nu * cs);
      const float de = -mp.kn * mp.eps * mp.nu * sn;
      const float dde = -mp.kn * mp.kn * mp.eps * mp.nu * cs;
      float tx = 0.f, ty = 0.f;
      const float r2 = dpx * dpx + dpy * dpy;
      if (steep && r2 > 0.f) {
         tx = -dpy / r2;
         ty = dpx / r2;
      }
      float F, JA, JB;
      if (dir == 0) {
         F = e * e * dpx - e * de * dpy;
         const float dFdt = 2.f * e * de * dpx - (de * de + e * dde) * dpy;
         JA = e * e + dFdt * tx;
         JB = -e * de + dFdt * ty;
         const int f = g.fx(i, j, 0);
         a.F[0][f] = F;
         a.JA[0][f] = JA;
         a.JB[0][f] = JB;
      } else {
         F = e * e * dpy + e * de * dpx;
         const float dFdt = 2.f * e * de * dpy + (de * de + e * dde) * dpx;
         JA = e * de + dFdt * tx;
         JB = e * e + dFdt * ty;
         const int f = g.fy(i, j, 0);
         a.F[1][f] = F;
         a.JA[1][f] = JA;
         a.JB[1][f] = JB;
      }
   }
}

__global__ void k_aniso_orientation(Grid g, int qlen4, const double* q, AnisoF a)
{
   const long long nx = g.nfx(), tot = nx + g.nfy();
   for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < tot;
        t += (long long)gridDim.x * blockDim.x) {
      int dir, i, j, k;
      face_of(g, t, dir, i, j, k);
      double qa = dir == 0 ? 0.5 * (q[g.c(i - 1, j, 0)] + q[g.c(i, j, 0)])
                           : 0.5 * (q[g.c(i, j - 1, 0)] + q[g.c(i, j, 0)]);
      qa = fmin(1.0, fmax(-1.0, qa));
      const double po = qlen4 ? 2.0 * acos(qa) : acos(qa);
      if (dir == 0)
         a.PO[0][g.fx(i, j, 0)] = (float)po;
      else
         a.PO[1][g.fy(i, j, 0)] = (float)po;
   }
}

// ---------------------------------------------------------------------------
// 3D anisotropic flux (anisotropic_gradient_flux, 3d/quatrhs.m4:180-355,
// with compute_dgamma, 3d/quatrhs.m4:149-177) in FP32, and its gradient with
// respect to the face gradient g of phi by forward-mode differentiation:
// every quantity carries its value and its three partial derivatives.
//   n = g/|g|, n' = q n q*, n4 = sum n'_i^4,
//   dg = q* (n'_i (n'_i^2 - n4))_i q,
//   gamma = eps (1 - 3 e4)(1 + 4 e4/(1 - 3 e4) n4),
//   F_d = gamma^2 g_d + 16 eps gamma e4 |g| dg_d,
// q the (unnormalised) face mean of the orientation quaternion; below
// |g|^2 = 1e-12 the reference's constant dg and n4 = 0 are used.
// ---------------------------------------------------------------------------
struct Dual3 {
   float v, d[3];
};

__device__ __forceinline__ Dual3 dconst(float v) { return {v, {0.f, 0.f, 0.f}}; }
__device__ __forceinline__ Dual3 operator+(const Dual3& a, const Dual3& b)
{
   return {a.v + b.v, {a.d[0] + b.d[0], a.d[1] + b.d[1], a.d[2] + b.d[2]}};
}
__device__ __forceinline__ Dual3 operator-(const Dual3& a, const Dual3& b)
{
   return {a.v - b.v, {a.d[0] - b.d[0], a.d[1] - b.d[1], a.d[2] - b.d[2]}};
}
__device__ __forceinline__ Dual3 operator*(const Dual3& a, const Dual3& b)
{
   return {a.v * b.v,
           {a.d[0] * b.v + a.v * b.d[0], a.d[1] * b.v + a.v * b.d[1],
            a.d[2] * b.v + a.v * b.d[2]}};
}
__device__ __forceinline__ Dual3 operator*(float a, const Dual3& b)
{
   return {a * b.v, {a * b.d[0], a * b.d[1], a * b.d[2]}};
}
__device__ __forceinline__ Dual3 dsqrt(const Dual3& a)
{
   const float r = sqrtf(a.v);
   const float h = r > 0.f ? 0.5f / r : 0.f;  // zero at a flat face: the term it scales is zero
   return {r, {h * a.d[0], h * a.d[1], h * a.d[2]}};
}
__device__ __forceinline__ Dual3 drcp(const Dual3& a)
{
   const float r = 1.f / a.v, r2 = -r * r;
   return {r, {r2 * a.d[0], r2 * a.d[1], r2 * a.d[2]}};
}

// quaternion product on Dual3 components (quatmult4 order)
__device__ __forceinline__ void dqmul(const Dual3* a, const Dual3* b, Dual3* q)
{
   q[0] = a[0] * b[0] - a[1] * b[1] - a[2] * b[2] - a[3] * b[3];
   q[1] = a[0] * b[1] + a[1] * b[0] + a[2] * b[3] - a[3] * b[2];
   q[2] = a[0] * b[2] + a[2] * b[0] + a[3] * b[1] - a[1] * b[3];
   q[3] = a[0] * b[3] + a[3] * b[0] + a[1] * b[2] - a[2] * b[1];
}

// F and dF/dg on face dir from the face gradient gv (values) and the face
// quaternion qf
__device__ __forceinline__ Dual3 aniso3d_flux(const MixParams& mp, int dir, const float* gv,
                                              const float* qf)
{
   const float eps = mp.eps, e4 = mp.nu;
   const float factor = 4.f * e4 / (1.f - 3.f * e4);
   Dual3 gd[3];
   for (int a = 0; a < 3; a++) {
      gd[a] = dconst(gv[a]);
      gd[a].d[a] = 1.f;
   }
   const Dual3 gphi2 = gd[0] * gd[0] + gd[1] * gd[1] + gd[2] * gd[2];
   Dual3 dg[4], n4;
   if (fabsf(gphi2.v) > 1.e-12f) {
      const Dual3 nni = drcp(dsqrt(gphi2));
      const Dual3 n[4] = {dconst(0.f), gd[0] * nni, gd[1] * nni, gd[2] * nni};
      const Dual3 q[4] = {dconst(qf[0]), dconst(qf[1]), dconst(qf[2]), dconst(qf[3])};
      const Dual3 qp[4] = {q[0], dconst(-qf[1]), dconst(-qf[2]), dconst(-qf[3])};
      Dual3 tmp[4], np[4];
      dqmul(n, qp, tmp);
      dqmul(q, tmp, np);
      const Dual3 p1 = np[1] * np[1], p2 = np[2] * np[2], p3 = np[3] * np[3];
      n4 = p1 * p1 + p2 * p2 + p3 * p3;
      const Dual3 dd[4] = {dconst(0.f), np[1] * (p1 - n4), np[2] * (p2 - n4),
                           np[3] * (p3 - n4)};
      dqmul(dd, q, tmp);
      dqmul(qp, tmp, dg);
   } else {
      dg[0] = dg[1] = dconst(0.f);
      dg[2] = dconst(dir == 2 ? 1.f : 0.f);
      dg[3] = dconst(dir == 2 ? 0.f : 1.f);
      n4 = dconst(0.f);
   }
   const Dual3 gamma = (eps * (1.f - 3.f * e4)) * (dconst(1.f) + factor * n4);
   return gamma * gamma * gd[dir] + (16.f * eps * e4) * (gamma * dsqrt(gphi2) * dg[dir + 1]);
}

// face gradient of a cell field on face dir whose upper cell is (i, j, k),
// the stencil of the 3D anisotropic flux; D(a, b) = field(a) - field(b)
template <class DF>
__device__ __forceinline__ void aniso3d_face_grad(const MixParams& mp, const Grid& g, int dir,
                                                  int i, int j, int k, DF D, float* gv)
{
   auto C = [&](int a, int b, int c) { return g.c(a, b, c); };
   if (dir == 0) {
      gv[0] = D(C(i, j, k), C(i - 1, j, k)) * mp.dxi[0];
      gv[1] = 0.25f * (D(C(i - 1, j + 1, k), C(i - 1, j - 1, k)) +
                       D(C(i, j + 1, k), C(i, j - 1, k))) * mp.dxi[1];
      gv[2] = 0.25f * (D(C(i - 1, j, k + 1), C(i - 1, j, k - 1)) +
                       D(C(i, j, k + 1), C(i, j, k - 1))) * mp.dxi[2];
   } else if (dir == 1) {
      gv[0] = 0.25f * (D(C(i + 1, j - 1, k), C(i - 1, j - 1, k)) +
                       D(C(i + 1, j, k), C(i - 1, j, k))) * mp.dxi[0];
      gv[1] = D(C(i, j, k), C(i, j - 1, k)) * mp.dxi[1];
      gv[2] = 0.25f * (D(C(i, j - 1, k + 1), C(i, j - 1, k - 1)) +
                       D(C(i, j, k + 1), C(i, j, k - 1))) * mp.dxi[2];
   } else {
      gv[0] = 0.25f * (D(C(i + 1, j, k - 1), C(i - 1, j, k - 1)) +
                       D(C(i + 1, j, k), C(i - 1, j, k))) * mp.dxi[0];
      gv[1] = 0.25f * (D(C(i, j + 1, k - 1), C(i, j - 1, k - 1)) +
                       D(C(i, j + 1, k), C(i, j - 1, k))) * mp.dxi[1];
      gv[2] = D(C(i, j, k), C(i, j, k - 1)) * mp.dxi[2];
   }
}

__device__ __forceinline__ long long face_index(const Grid& g, int dir, int i, int j, int k)
{
   return dir == 0 ? g.fx(i, j, k) : (dir == 1 ? g.fy(i, j, k) : g.fz(i, j, k));
}

__global__ void k_aniso3d_faces_f32(MixParams mp, Grid g, const double* ph, const double* q,
                                    AnisoF a)
{
   const long long tot = g.nfx() + g.nfy() + g.nfz();
   const long long qs = g.cells_ghost();
   for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < tot;
        t += (long long)gridDim.x * blockDim.x) {
      int dir, i, j, k;
      face_of(g, t, dir, i, j, k);
      float gv[3];
      // neighbour differences of the FP64 phase, rounded once
      aniso3d_face_grad(mp, g, dir, i, j, k,
                        [&](long long u, long long l) { return d2f(ph[u] - ph[l]); }, gv);
      const int ei = dir == 0, ej = dir == 1, ek = dir == 2;
      const long long lo = g.c(i - ei, j - ej, k - ek), up = g.c(i, j, k);
      float qf[4];
      for (int c = 0; c < 4; c++) qf[c] = d2f(0.5 * (q[c * qs + lo] + q[c * qs + up]));
      const Dual3 F = aniso3d_flux(mp, dir, gv, qf);
      const long long f = face_index(g, dir, i, j, k);
      a.F[dir][f] = F.v;
      a.JA[dir][f] = F.d[0];
      a.JB[dir][f] = F.d[1];
      a.JC[dir][f] = F.d[2];
   }
}

int aniso_orientation_f32(const ampe_model_t& m, const Grid& g, const double* q,
                          AnisoF& a, cudaStream_t s)
{
   const long long tot = g.nfx() + g.nfy();
   long long b = (tot + 255) / 256;
   if (b > max_blocks()) b = max_blocks();
   k_aniso_orientation<<<(unsigned)b, 256, 0, s>>>(g, m.qlen == 4 ? 1 : 0, q, a);
   return launch_status();
}

int aniso_faces_f32(const ampe_model_t& m, const MixParams& mp, const Grid& g,
                    const double* ph, const double* q, AnisoF& a, cudaStream_t s)
{
   (void)m;
   const long long tot = g.nfx() + g.nfy() + (g.dim == 3 ? g.nfz() : 0);
   long long b = (tot + 255) / 256;
   if (b > max_blocks()) b = max_blocks();
   if (g.dim == 3)
      k_aniso3d_faces_f32<<<(unsigned)b, 256, 0, s>>>(mp, g, ph, q, a);
   else
      k_aniso_faces_f32<<<(unsigned)b, 256, 0, s>>>(mp, g, ph, q, a);
   return launch_status();
}

// linearised 3D anisotropic flux on face d whose upper cell is (i, j, k)
__device__ __forceinline__ float aniso3d_dflux(const MixParams& mp, const AnisoF& a, int d,
                                               const float* dp, const Grid& g, int i, int j,
                                               int k)
{
   float gv[3];
   aniso3d_face_grad(mp, g, d, i, j, k, [&](long long u, long long l) { return dp[u] - dp[l]; },
                     gv);
   const long long f = face_index(g, d, i, j, k);
   return a.JA[d][f] * gv[0] + a.JB[d][f] * gv[1] + a.JC[d][f] * gv[2];
}

// linearised anisotropic flux on face d whose upper cell is (i, j): the face
// gradient of dphi (the stencil of the flux) through the face's Jacobian
__device__ __forceinline__ float aniso_dflux(const MixParams& mp, const AnisoF& a, int d,
                                             const float* dp, const Grid& g, int i, int j)
{
   auto P = [&](int x, int y) { return dp[g.c(x, y, 0)]; };
   if (d == 0) {
      const float gx = (P(i, j) - P(i - 1, j)) * mp.dxi[0];
      const float gy =
          0.25f * (P(i - 1, j + 1) - P(i - 1, j - 1) + P(i, j + 1) - P(i, j - 1)) * mp.dxi[1];
      const int f = g.fx(i, j, 0);
      return a.JA[0][f] * gx + a.JB[0][f] * gy;
   }
   const float gx =
       0.25f * (P(i + 1, j - 1) - P(i - 1, j - 1) + P(i + 1, j) - P(i - 1, j)) * mp.dxi[0];
   const float gy = (P(i, j) - P(i, j - 1)) * mp.dxi[1];
   const int f = g.fy(i, j, 0);
   return a.JA[1][f] * gx + a.JB[1][f] * gy;
}

// "kks" composition form on the face lo|up (KKSCompositionRHSStrategy.cc:
// 98-441): D0 = (1-h) D_L + h D_S with h = energy_interp(phibar), and the
// coupling D_phi = D0 h'(phibar)(cLbar - cSbar)
// (D_L, D_S) of the face between cells (a0-ei, ...) and (a0, a1, a2):
// D^0 exp(-Q / (R Tbar)), Tbar the mean of the two cells' temperatures
__device__ __forceinline__ float2 face_dq(const ampe_model_t& m, const MixParams& mp,
                                          const Grid& g, const double* tfield, int a0,
                                          int a1, int a2, int ei, int ej, int ek)
{
   const float invT = 2.f / (float)(temperature_at(m, g, tfield, a0 - ei, a1 - ej, a2 - ek) +
                                    temperature_at(m, g, tfield, a0, a1, a2));
   return make_float2(mp.Dl * expf(-mp.qlR * invT), mp.Ds * expf(-mp.qsR * invT));
}

__device__ __forceinline__ float2 face_dq_at(const ampe_model_t& m, const MixParams& mp,
                                             const Grid& g, const double* tfield, int a0,
                                             int a1, int a2, int ei, int ej, int ek)
{
   if (!mp.tdep) return make_float2(mp.Dl, mp.Ds);
   if (mp.dq) return mp.dq[ei ? a0 : g.n0 + 1 + a0];
   return face_dq(m, mp, g, tfield, a0, a1, a2, ei, ej, ek);
}

__global__ void k_diff_table(ampe_model_t m, MixParams mp, Grid g, float2* dq)
{
   const int t = blockIdx.x * blockDim.x + threadIdx.x;
   if (t <= g.n0)
      dq[t] = face_dq(m, mp, g, nullptr, t, 0, 0, 1, 0, 0);
   else if (t < 2 * g.n0 + 1)
      dq[t] = face_dq(m, mp, g, nullptr, t - g.n0 - 1, 0, 0, 0, 1, 0);
}

int build_diff_table(const ampe_model_t& m, const MixParams& mp, const Grid& g,
                     float2* dq, cudaStream_t s)
{
   if (m.temp_mode == AMPE_TEMP_FIELD || !mp.tdep) return AMPE_ERR_INVALID;
   const int n = 2 * g.n0 + 1;
   k_diff_table<<<(n + 127) / 128, 128, 0, s>>>(m, mp, g, dq);
   return launch_status();
}

template <int DIM, bool PB>
__device__ __forceinline__ void kks_face_coef(const ampe_model_t& m, const MixParams& mp,
                                              const Grid& g, const double* tfield,
                                              const float* pf, const float* cl,
                                              const float* cs, long long lo, long long up,
                                              int a0, int a1, int a2, int ei, int ej, int ek,
                                              float& D0, float& Dp)
{
   const Types<PB> ty(m);
   const float vphi = average_func(pf[lo], pf[up], ty.avg);
   const float h = interp_func(vphi, ty.energy);
   const float2 dq = face_dq_at(m, mp, g, tfield, a0, a1, a2, ei, ej, ek);
   D0 = (1.f - h) * dq.x + h * dq.y;
   Dp = D0 * deriv_interp_func(vphi, ty.energy) *
        (0.5f * (cl[up] + cl[lo]) - 0.5f * (cs[up] + cs[lo]));
}

// the same flux from the FP64 phase: each neighbour difference is formed in
// FP64 and rounded once (phi ~ 1 rounded to FP32 first would leave the
// difference of two rounded numbers: ~6e-8 absolute, about 1e-6 relative to
// an interface gradient)
template <int DIM>
__device__ __forceinline__ float face_flux_lin64(const MixParams& mp, int d,
                                                 const double* ph, const Grid& g,
                                                 int i, int j, int k)
{
   if (DIM == 3 || !mp.iso) {
      const int ei = d == 0, ej = d == 1, ek = d == 2;
      return d2f(ph[g.c(i, j, k)] - ph[g.c(i - ei, j - ej, k - ek)]) * mp.flux_dinv[d];
   }
   auto D = [&](int a, int b, int a2, int b2) {
      return d2f(ph[g.c(a, b, 0)] - ph[g.c(a2, b2, 0)]);
   };
   const float dinv = mp.flux_dinv[d];
   if (d == 0)
      return dinv * (D(i, j - 1, i - 1, j - 1) + D(i, j, i - 1, j) * 10.f +
                     D(i, j + 1, i - 1, j + 1));
   return dinv * (D(i - 1, j, i - 1, j - 1) + D(i, j, i, j - 1) * 10.f +
                  D(i + 1, j, i + 1, j - 1));
}

// face weights (1-h) D_L, h D_S from the phases of the two cells
template <int DIM, bool PB = false>
__device__ __forceinline__ void face_diff(const ampe_model_t& m,
                                          const MixParams& mp, const Grid& g,
                                          const double* tfield, const float* pf,
                                          long long lo, long long up, int a0,
                                          int a1, int a2, int ei, int ej,
                                          int ek, float& DL, float& DS)
{
   const Types<PB> ty(m);
   const float vphi = average_func(pf[lo], pf[up], ty.avg);
   const float hphi = interp_func(vphi, ty.diff);
   const float2 dq = face_dq_at(m, mp, g, tfield, a0, a1, a2, ei, ej, ek);
   DL = (1.f - hphi) * dq.x;
   DS = hphi * dq.y;
}

// face weights with the composition-dependent D_L, D_S of the atomic
// mobilities, evaluated in FP64 at the face means of the FP32 cL, cS of this
// f(y) (MobilityCompositionDiffusionStrategy.cc:83-611) and rounded once
template <int DIM, bool PB = false>
__device__ __forceinline__ void face_diff_mob(const ampe_model_t& m, const Grid& g,
                                              const double* tfield, const float* pf,
                                              const float* cl, const float* cs,
                                              long long lo, long long up, int a0,
                                              int a1, int a2, int ei, int ej, int ek,
                                              float& DL, float& DS)
{
   const Types<PB> ty(m);
   const float vphi = average_func(pf[lo], pf[up], ty.avg);
   const float hphi = interp_func(vphi, ty.diff);
   const double T = 0.5 * (temperature_at(m, g, tfield, a0, a1, a2) +
                           temperature_at(m, g, tfield, a0 - ei, a1 - ej, a2 - ek));
   const double cL = 0.5 * ((double)cl[up] + (double)cl[lo]);
   const double cS = 0.5 * ((double)cs[up] + (double)cs[lo]);
   DL = (1.f - hphi) * d2f(phase_diffusion(m, m.mobility, 0, cL, T));
   DS = hphi * d2f(phase_diffusion(m, m.mobility, 1, cS, T));
}

// temperature of cell (i,j,k) in FP32 (ghost cells take their periodic image)
__device__ __forceinline__ float temp_f(const ampe_model_t& m, const MixParams& mp,
                                        const Grid& g, const double* tfield, int i,
                                        int j, int k)
{
   if (m.temp_mode == AMPE_TEMP_CONSTANT) return mp.T0;
   if (m.temp_mode == AMPE_TEMP_GRADIENT) {
      const int iw = i < 0 ? i + g.n0 : (i >= g.n0 ? i - g.n0 : i);
      return mp.T0 + mp.gdx * ((float)iw + 0.5f);
   }
   return (float)tfield[g.c(i, j, k)];
}

__global__ void k_phi_to_f32(Grid g, const double* phi, float* pf)
{
   for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
        t < g.cells_ghost(); t += (long long)gridDim.x * blockDim.x)
      pf[t] = d2f(phi[t]);
}

// weights of the lower (m) and upper (p) face of cell (i,j,k) along d
__device__ __forceinline__ void face_w(const FaceW& fw, const Grid& g, int d, int i, int j,
                                       int k, float& Am, float& Bm, float& Ap, float& Bp)
{
   int f, step;
   if (d == 0) {
      f = g.fx(i, j, k);
      step = 1;
   } else if (d == 1) {
      f = g.fy(i, j, k);
      step = g.n0;
   } else {
      f = g.fz(i, j, k);
      step = g.n0 * g.n1;
   }
   Am = fw.A[d][f];
   Bm = fw.B[d][f];
   Ap = fw.A[d][f + step];
   Bp = fw.B[d][f + step];
}

template <int DIM, bool PB, bool ANISO>
__global__ void k_rhs_mixed(ampe_model_t m, MixParams mp, Grid g, AnisoF an, FaceW fw,
                            const double* tfield, const double* ph, const double* cc,
                            const float* pf,
                            const float* cl, const float* cs, const float* dF,
                            const float* ogm, double* phi_rhs, double* conc_rhs)
{
   for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
        t < g.cells(); t += (long long)gridDim.x * blockDim.x) {
      int i, j, k;
      g.ijk(t, i, j, k);
      const long long c = g.c(i, j, k);
      float diff = 0.f, div = 0.f;
#pragma unroll
      for (int d = 0; d < DIM; d++) {
         const int ei = d == 0, ej = d == 1, ek = d == 2;
         float fm, fp;
         if (ANISO) {  // precomputed face fluxes
            fm = an.F[d][face_index(g, d, i, j, k)];
            fp = an.F[d][face_index(g, d, i + ei, j + ej, k + ek)];
         } else {
            fm = face_flux_lin64<DIM>(mp, d, ph, g, i, j, k);
            fp = face_flux_lin64<DIM>(mp, d, ph, g, i + ei, j + ej, k + ek);
         }
         diff += (fp - fm) * mp.dxi[d];
         const long long up = g.c(i + ei, j + ej, k + ek);
         const long long lo = g.c(i - ei, j - ej, k - ek);
         float Am, Bm, Ap, Bp;
         face_w(fw, g, d, i, j, k, Am, Bm, Ap, Bp);
         float flm, flp;
         if (mp.kksc) {  // "kks" form: c and phi differences in FP64, rounded once
            flm = mp.dxi[d] * (Am * d2f(cc[c] - cc[lo]) + Bm * d2f(ph[c] - ph[lo]));
            flp = mp.dxi[d] * (Ap * d2f(cc[up] - cc[c]) + Bp * d2f(ph[up] - ph[c]));
         } else {
            flm = mp.dxi[d] * (Am * (cl[c] - cl[lo]) + Bm * (cs[c] - cs[lo]));
            flp = mp.dxi[d] * (Ap * (cl[up] - cl[c]) + Bp * (cs[up] - cs[c]));
         }
         div += mp.dxi[d] * (flp - flm);
      }
      const Types<PB> ty(m);
      const float p = pf[c];
      float r = diff - mp.w * deriv_well_func(p, ty.well);
      if (ogm) {  // orientation term, 3d/quatrhs.m4:481-509
         const float gm = ogm[t];
         const float T = temp_f(m, mp, g, tfield, i, j, k);
         r = r - mp.misor * T * deriv_interp_func(p, ty.o1) * gm -
             deriv_interp_func(p, ty.o2) * mp.eq2h * gm * gm;
      }
      r += deriv_interp_func(p, ty.energy) * dF[t];
      phi_rhs[t] = f2d(r * mp.Mphi);
      conc_rhs[t] = f2d(mp.Mc * div);
   }
}

// composition flux weights of every face (EBS: (1-h) D_L, h D_S with h =
// diff_interp; "kks": D0, D_phi).  One thread per point (i, j, k) of the box
// [0, n0] x [0, n1] x [0, n2] computes the lower x, y and z faces of cell
// (i, j, k) that exist, sharing the cell's index math and loads.  MOB: the
// atomic-mobility diffusivities (their FP64 arithmetic in an instantiation
// of its own, so the others keep their registers).
template <int DIM, bool PB, bool MOB>
__global__ void k_face_weights(ampe_model_t m, MixParams mp, Grid g, const double* tfield,
                               const float* __restrict__ pf, const float* __restrict__ cl,
                               const float* __restrict__ cs, FaceW fw)
{
   const long long tot = (long long)(g.n0 + 1) * (g.n1 + 1) * (DIM == 3 ? g.n2 + 1 : 1);
   for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < tot;
        t += (long long)gridDim.x * blockDim.x) {
      int i, j, k;
      g.split(t, g.fd0p, g.fd1p, i, j, k);
      const long long up = g.c(i, j, k);
#pragma unroll
      for (int dir = 0; dir < DIM; dir++) {
         const bool has = dir == 0 ? (j < g.n1 && k < g.n2)
                                   : (dir == 1 ? (i < g.n0 && k < g.n2) : (i < g.n0 && j < g.n1));
         if (!has) continue;
         const int ei = dir == 0, ej = dir == 1, ek = dir == 2;
         const long long lo = g.c(i - ei, j - ej, k - ek);
         float a, b;
         if (mp.kksc)
            kks_face_coef<DIM, PB>(m, mp, g, tfield, pf, cl, cs, lo, up, i, j, k, ei, ej, ek, a,
                                   b);
         else if (MOB)
            face_diff_mob<DIM, PB>(m, g, tfield, pf, cl, cs, lo, up, i, j, k, ei, ej, ek, a, b);
         else
            face_diff<DIM, PB>(m, mp, g, tfield, pf, lo, up, i, j, k, ei, ej, ek, a, b);
         const int f = dir == 0 ? g.fx(i, j, k) : (dir == 1 ? g.fy(i, j, k) : g.fz(i, j, k));
         fw.A[dir][f] = a;
         fw.B[dir][f] = b;
      }
   }
}

int rhs_mixed(const ampe_model_t& m, const MixParams& mp, const Grid& g,
              const double* tfield, const double* phi, float* pf,
              const float* cl, const float* cs, const float* dF,
              const float* ogm, const double* q, AnisoF* an, const double* cc,
              const FaceW& fw, double* phi_rhs, double* conc_rhs, cudaStream_t s)
{
   if (mp.kksc && !cc) return AMPE_ERR_INVALID;
   long long b = (g.cells_ghost() + 255) / 256;
   if (b > max_blocks()) b = max_blocks();
   k_phi_to_f32<<<(unsigned)b, 256, 0, s>>>(g, phi, pf);
   launch_status();
   {
      const long long tot =
          (long long)(g.n0 + 1) * (g.n1 + 1) * (g.dim == 3 ? g.n2 + 1 : 1);
      long long bf = (tot + 255) / 256;
      if (bf > max_blocks()) bf = max_blocks();
      const bool mob = !mp.kksc && m.conc_diffusion == AMPE_DIFF_MOBILITY;
#define AMPE_FW(D, P, M) \
   k_face_weights<D, P, M><<<(unsigned)bf, 256, 0, s>>>(m, mp, g, tfield, pf, cl, cs, fw)
      if (mob) {
         if (g.dim == 3)
            AMPE_FW(3, false, true);
         else
            AMPE_FW(2, false, true);
      } else if (g.dim == 3) {
         if (mp.pb)
            AMPE_FW(3, true, false);
         else
            AMPE_FW(3, false, false);
      } else {
         if (mp.pb)
            AMPE_FW(2, true, false);
         else
            AMPE_FW(2, false, false);
      }
#undef AMPE_FW
      launch_status();
   }
   b = (g.cells() + 255) / 256;
   if (b > max_blocks()) b = max_blocks();
   const bool aniso = m.flux_type == AMPE_FLUX_ANISOTROPIC;
   if (aniso) {
      if (!q || !an) return AMPE_ERR_INVALID;
      aniso_faces_f32(m, mp, g, phi, q, *an, s);
   }
   const AnisoF a0 = an ? *an : AnisoF();
#define AMPE_RHS(D, P)                                                                      \
   k_rhs_mixed<D, P, false><<<(unsigned)b, 256, 0, s>>>(m, mp, g, a0, fw, tfield, phi, cc, pf, \
                                                        cl, cs, dF, ogm, phi_rhs, conc_rhs)
   if (aniso && g.dim == 3) {
      if (mp.pb)
         k_rhs_mixed<3, true, true><<<(unsigned)b, 256, 0, s>>>(m, mp, g, a0, fw, tfield, phi,
                                                               cc, pf, cl, cs, dF, ogm,
                                                               phi_rhs, conc_rhs);
      else
         k_rhs_mixed<3, false, true><<<(unsigned)b, 256, 0, s>>>(m, mp, g, a0, fw, tfield, phi,
                                                                cc, pf, cl, cs, dF, ogm,
                                                                phi_rhs, conc_rhs);
   } else if (aniso) {
      if (mp.pb)
         k_rhs_mixed<2, true, true><<<(unsigned)b, 256, 0, s>>>(m, mp, g, a0, fw, tfield, phi,
                                                               cc, pf, cl, cs, dF, ogm,
                                                               phi_rhs, conc_rhs);
      else
         k_rhs_mixed<2, false, true><<<(unsigned)b, 256, 0, s>>>(m, mp, g, a0, fw, tfield, phi,
                                                                cc, pf, cl, cs, dF, ogm,
                                                                phi_rhs, conc_rhs);
   } else if (g.dim == 3) {
      if (mp.pb)
         AMPE_RHS(3, true);
      else
         AMPE_RHS(3, false);
   } else {
      if (mp.pb)
         AMPE_RHS(2, true);
      else
         AMPE_RHS(2, false);
   }
#undef AMPE_RHS
   return launch_status();
}

// ---------------------------------------------------------------------------
// analytic Jacobian-vector product
// ---------------------------------------------------------------------------
// pointwise: dphi, and the linearised KKS split (da, db) solving
//   J [da; db] = [dc - (b - a) h_c'(phi) dphi; 0]
template <bool PB>
__global__ void k_jv_point(ampe_model_t m, Grid g, const CoefF* tabf,
                           const double* tfield, const float* pf,
                           const float* cl, const float* cs, const float* v,
                           float* dphi, float* da, float* db, float* dcv, float* dq)
{
   const long long N = g.cells(), NG = g.cells_ghost();
   for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < N;
        t += (long long)gridDim.x * blockDim.x) {
      int i, j, k;
      g.ijk(t, i, j, k);
      const long long c = g.c(i, j, k);
      const CoefF tf = coef_f_at(m, g, tabf, tfield, i, j, k);
      const Types<PB> ty(m);
      const float p = pf[c], a = cl[c], b = cs[c];
      const float h = interp_func(p, ty.conc);
      const float vp = v[t], vc = v[t + N];
      const float J00 = 1.f - h, J01 = h;
      const float J10 = 1.f / (a * (1.f - a)) + dxi_f(tf, a, 0) * tf.iRT;
      const float J11 = -1.f / (b * (1.f - b)) - dxi_f(tf, b, 1) * tf.iRT;
      const float idet = 1.f / (J00 * J11 - J01 * J10);
      const float r0 = vc - (b - a) * deriv_interp_func(p, ty.conc) * vp;
      const float xa = J11 * r0 * idet, xb = -J10 * r0 * idet;
      dphi[c] = vp;
      da[c] = xa;
      db[c] = xb;
      for_each_image(g, i, j, k, [&](long long idx) {
         dphi[idx] = vp;
         da[idx] = xa;
         db[idx] = xb;
      });
      if (dcv) {  // the c part of v, ghosted ("kks" composition form)
         dcv[c] = vc;
         for_each_image(g, i, j, k, [&](long long idx) { dcv[idx] = vc; });
      }
      if (dq) {
#pragma unroll
         for (int q = 0; q < 4; q++) {
            const float x = v[t + (2 + q) * N];
            float* dqq = dq + q * NG;
            dqq[c] = x;
            for_each_image(g, i, j, k, [&](long long idx) { dqq[idx] = x; });
         }
      }
   }
}

__device__ __forceinline__ float second_deriv_interp_f(float phi, char type)
{
   float p;
   switch (type) {
      case 'p':
         p = clamp01(phi);
         return 60.f * p * (1.f - 3.f * p + 2.f * p * p);
      case 'h':
         p = clamp01(phi);
         return 6.f * (1.f - 2.f * p);
      case 'q':
         return phi >= 0.f ? 2.f : 0.f;
      case 'w':
         p = phi > 0.f ? phi : 0.f;
         return 4.f - 6.f * p;
      case '3':
         p = phi > 0.f ? phi : 0.f;
         return 6.f * p;
      case 'm': {
         p = clamp01(phi);
         const float t = 2.f * p * (p - 1.f) + 1.f;
         return 2.f * (1.f - 2.f * p) / (t * t) -
                4.f * p * (1.f - p) * (4.f * p - 2.f) / (t * t * t);
      }
      case 's': {
         p = phi > 0.f ? phi : 0.f;
         const float th = tanhf(10.f * p);
         return 100.f * (1.f - th * th) / logf(coshf(10.f));
      }
      default:  // 'l', 'c': piecewise linear / constant
         return 0.f;
   }
}

// out = v - gamma J v
template <int DIM, bool PB, bool ANISO>
__global__ void k_jv_stencil(ampe_model_t m, MixParams mp, Grid g, AnisoF an, FaceW fw,
                             const CoefF* tabf, const double* tfield,
                             const float* pf, const float* cl, const float* cs,
                             const float* dF, const float* dphi,
                             const float* da, const float* db, const float* dcv,
                             const float* v, const float* ogm, float gamma, float* out)
{
   const long long N = g.cells();
   for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < N;
        t += (long long)gridDim.x * blockDim.x) {
      int i, j, k;
      g.ijk(t, i, j, k);
      const long long c = g.c(i, j, k);
      float diff = 0.f, div = 0.f;
#pragma unroll
      for (int d = 0; d < DIM; d++) {
         const int ei = d == 0, ej = d == 1, ek = d == 2;
         float fm, fp;
         if (ANISO && DIM == 3) {  // linearised anisotropic flux on the two faces
            fm = aniso3d_dflux(mp, an, d, dphi, g, i, j, k);
            fp = aniso3d_dflux(mp, an, d, dphi, g, i + ei, j + ej, k + ek);
         } else if (ANISO) {
            fm = aniso_dflux(mp, an, d, dphi, g, i, j);
            fp = aniso_dflux(mp, an, d, dphi, g, i + ei, j + ej);
         } else {
            fm = face_flux_lin<DIM>(mp, d, dphi, g, i, j, k);
            fp = face_flux_lin<DIM>(mp, d, dphi, g, i + ei, j + ej, k + ek);
         }
         diff += (fp - fm) * mp.dxi[d];
         const long long up = g.c(i + ei, j + ej, k + ek);
         const long long lo = g.c(i - ei, j - ej, k - ek);
         float Am, Bm, Ap, Bp;
         face_w(fw, g, d, i, j, k, Am, Bm, Ap, Bp);
         // "kks" form: linear in (c, phi) with the weights held; EBS: in the
         // linearised split (dcL, dcS)
         const float* xa = mp.kksc ? dcv : da;
         const float* xb = mp.kksc ? dphi : db;
         const float flm = mp.dxi[d] * (Am * (xa[c] - xa[lo]) + Bm * (xb[c] - xb[lo]));
         const float flp = mp.dxi[d] * (Ap * (xa[up] - xa[c]) + Bp * (xb[up] - xb[c]));
         div += mp.dxi[d] * (flp - flm);
      }
      const Types<PB> ty(m);
      const CoefF tf = coef_f_at(m, g, tabf, tfield, i, j, k);
      const float p = pf[c], a = cl[c], b = cs[c], vp = dphi[c];
      // d(dF)/db = -f_S''(b) (a - b), d(dF)/da = muL - muS = 0
      const float fS2 = tf.RT / (b * (1.f - b)) + dxi_f(tf, b, 1);
      const float ddF = -fS2 * (a - b) * mp.ivm * db[c];
      float orient = 0.f;
      if (ogm) {  // phi-derivative of the orientation term at lagged |grad q|
         const float gm = ogm[t];
         const float T = temp_f(m, mp, g, tfield, i, j, k);
         orient = (mp.misor * T * second_deriv_interp_f(p, ty.o1) * gm +
                   second_deriv_interp_f(p, ty.o2) * mp.eq2h * gm * gm) *
                  vp;
      }
      const float jp = mp.Mphi * (diff - mp.w * second_deriv_well_func(p, ty.well) * vp -
                                  orient +
                                  second_deriv_interp_f(p, ty.energy) * dF[t] * vp +
                                  deriv_interp_func(p, ty.energy) * ddF);
      const float jc = mp.Mc * div;
      out[t] = v[t] - gamma * jp;
      out[t + N] = v[t + N] - gamma * jc;
   }
}

// ---------------------------------------------------------------------------
// quaternion equation, FP32
// ---------------------------------------------------------------------------
template <int DIM>
__global__ void k_quat_cells_f32(MixParams mp, Grid g, const double* phi,
                                 const float* q, float* ogm, float* mq)
{
   const long long qs = g.cells_ghost();
   for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
        t < g.cells(); t += (long long)gridDim.x * blockDim.x) {
      int i, j, k;
      g.ijk(t, i, j, k);
      const long long c = g.c(i, j, k);
      const long long st[3] = {1, g.sx, g.sy};
      float s = 0.f;
#pragma unroll
      for (int d = 0; d < DIM; d++)
#pragma unroll
         for (int comp = 0; comp < 4; comp++) {
            const float* qc = q + comp * qs;
            const float a = mp.dxi[d] * (qc[c] - qc[c - st[d]]);
            const float b = mp.dxi[d] * (qc[c + st[d]] - qc[c]);
            s += a * a + b * b;
         }
      ogm[t] = sqrtf(0.5f * s);
      mq[c] = mp.qMmin + (mp.qM - mp.qMmin) * (1.f - interp_func(d2f(phi[c]), 'p'));
   }
}

struct FacePtrs {
   float* fc[3];
   float* dfc[3];
};

template <int DIM>
__global__ void k_quat_faces_f32(ampe_model_t m, MixParams mp, Grid g,
                                 const double* tfield, const float* pf,
                                 const float* q, float scale, FacePtrs f)
{
   const long long tot = g.nfx() + g.nfy() + (DIM == 3 ? g.nfz() : 0);
   for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < tot;
        t += (long long)gridDim.x * blockDim.x) {
      int dir, i, j, k;
      face_of(g, t, dir, i, j, k);
      const int ei = dir == 0, ej = dir == 1, ek = dir == 2;
      const float phia = average_func(pf[g.c(i - ei, j - ej, k - ek)], pf[g.c(i, j, k)],
                                      m.avg_type);
      const float tempa = 0.5f * (temp_f(m, mp, g, tfield, i - ei, j - ej, k - ek) +
                                  temp_f(m, mp, g, tfield, i, j, k));
      const float g2 = face_grad_norm2<DIM, float>(g, mp.dxi, q, dir, i, j, k);
      const float gni = eval_grad_normi(g2, mp.qfloor, mp.qfloor2, mp.qmaxi);
      const float a1 = gni * mp.misor * tempa;
      const float v = scale * (-a1 * interp_func(phia, m.orient_interp1) -
                               mp.epsq2 * interp_func(phia, m.orient_interp2));
      const long long fi = dir == 0 ? g.fx(i, j, k) : (dir == 1 ? g.fy(i, j, k) : g.fz(i, j, k));
      f.fc[dir][fi] = v;
      if (f.dfc[0])
         f.dfc[dir][fi] = -a1 * deriv_interp_func(phia, m.orient_interp1) -
                          mp.epsq2 * deriv_interp_func(phia, m.orient_interp2);
   }
}

// composition preconditioner faces from the face weights of the last f
// evaluation: D = -gamma (A + B) for EBS ((1-h) D_L + h D_S), -gamma A for
// the "kks" form (D0)
__global__ void k_conc_faces_f32(long long nx, long long ny, long long nz, FaceW fw,
                                 float gamma, int kksc, FacePtrs f)
{
   for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < nx + ny + nz;
        t += (long long)gridDim.x * blockDim.x) {
      const int dir = t < nx ? 0 : (t < nx + ny ? 1 : 2);
      const long long fi = t - (dir == 0 ? 0 : (dir == 1 ? nx : nx + ny));
      const float a = fw.A[dir][fi];
      f.fc[dir][fi] = kksc ? -gamma * a : -gamma * (a + fw.B[dir][fi]);
   }
}

// derivative of the face average of phi along (da, db)
__device__ __forceinline__ float d_average_f(float a, float b, float da, float db,
                                             char type)
{
   if (type == 'a') return 0.5f * (da + db);
   if (a < 1.0e-16f || b < 1.0e-16f) return 0.f;  // harmonic
   const float s = a + b;
   return 2.f * (b * b * da + a * a * db) / (s * s);
}

// q rows of v - gamma J v:
//   J_q dq = -M_q div(fc grad dq) - dM_q div(fc grad q) - M_q div(dfc grad q)
// with dM_q = M_q'(phi) dphi and dfc = (d fc / d phibar) dphibar at each face
template <int DIM>
__global__ void k_jv_quat(ampe_model_t m, MixParams mp, Grid g, const float* pf,
                          const float* dphi, QuatF32 qf, const float* v,
                          float gamma, float* out)
{
   const long long N = g.cells(), qs = g.cells_ghost();
   const float gm = gamma;
   for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < N;
        t += (long long)gridDim.x * blockDim.x) {
      int i, j, k;
      g.ijk(t, i, j, k);
      const long long c = g.c(i, j, k);
      const long long st[3] = {1, g.sx, g.sy};
      // per face (d, side): fc, and dfc * dphibar
      float F[3][2], dF[3][2];
#pragma unroll
      for (int d = 0; d < DIM; d++)
#pragma unroll
         for (int side = 0; side < 2; side++) {
            const int ii = i + (d == 0 ? side : 0), jj = j + (d == 1 ? side : 0),
                      kk = k + (d == 2 ? side : 0);
            const long long fi = d == 0 ? g.fx(ii, jj, kk)
                                        : (d == 1 ? g.fy(ii, jj, kk) : g.fz(ii, jj, kk));
            const long long up = c + side * st[d], lo = up - st[d];
            F[d][side] = qf.fc[d][fi];
            dF[d][side] = qf.dfc[d][fi] *
                          d_average_f(pf[lo], pf[up], dphi[lo], dphi[up], m.avg_type);
         }
      const float p = pf[c];
      const float mqc = qf.mq[c];
      const float dmq = -(mp.qM - mp.qMmin) * deriv_interp_func(p, 'p') * dphi[c];
#pragma unroll
      for (int comp = 0; comp < 4; comp++) {
         const float* qc = qf.q + comp * qs;
         const float* dqc = qf.dq + comp * qs;
         float A = 0.f, B = 0.f, Cc = 0.f;
#pragma unroll
         for (int d = 0; d < DIM; d++) {
            const float h = mp.dxi[d];
            const float gqm = h * (qc[c] - qc[c - st[d]]), gqp = h * (qc[c + st[d]] - qc[c]);
            const float gdm = h * (dqc[c] - dqc[c - st[d]]),
                        gdp = h * (dqc[c + st[d]] - dqc[c]);
            A += h * (F[d][1] * gdp - F[d][0] * gdm);
            B += h * (F[d][1] * gqp - F[d][0] * gqm);
            Cc += h * (dF[d][1] * gqp - dF[d][0] * gqm);
         }
         const float jq = -(mqc * (A + Cc) + dmq * B);
         const long long o = t + (2 + comp) * N;
         out[o] = v[o] - gm * jq;
      }
   }
}

int jv_mixed(const ampe_model_t& m, const MixParams& mp, const Grid& g,
             const CoefF* tabf, const double* tfield, const float* pf,
             const float* cl, const float* cs, const float* dF, const float* v,
             double gamma, float* dphi, float* da, float* db, float* dcv,
             const QuatF32* qf, const AnisoF* an, const FaceW& fw, float* out,
             cudaStream_t s)
{
   if (mp.kksc && !dcv) return AMPE_ERR_INVALID;
   long long b = (g.cells() + 255) / 256;
   if (b > max_blocks()) b = max_blocks();
   float* dq = qf ? qf->dq : nullptr;
   if (mp.pb)
      k_jv_point<true><<<(unsigned)b, 256, 0, s>>>(m, g, tabf, tfield, pf, cl, cs, v, dphi, da,
                                                   db, mp.kksc ? dcv : nullptr, dq);
   else
      k_jv_point<false><<<(unsigned)b, 256, 0, s>>>(m, g, tabf, tfield, pf, cl, cs, v, dphi,
                                                    da, db, mp.kksc ? dcv : nullptr, dq);
   launch_status();
   const float* ogm = (qf && m.with_orient) ? qf->ogm : nullptr;
   const AnisoF a0 = an ? *an : AnisoF();
#define AMPE_JV(D, P)                                                                          \
   k_jv_stencil<D, P, false><<<(unsigned)b, 256, 0, s>>>(m, mp, g, a0, fw, tabf, tfield, pf, cl, cs, \
                                                         dF, dphi, da, db, dcv, v, ogm,          \
                                                         (float)gamma, out)
   if (m.flux_type == AMPE_FLUX_ANISOTROPIC && g.dim == 3) {
      if (!an) return AMPE_ERR_INVALID;
      if (mp.pb)
         k_jv_stencil<3, true, true><<<(unsigned)b, 256, 0, s>>>(
             m, mp, g, a0, fw, tabf, tfield, pf, cl, cs, dF, dphi, da, db, dcv, v, ogm,
             (float)gamma, out);
      else
         k_jv_stencil<3, false, true><<<(unsigned)b, 256, 0, s>>>(
             m, mp, g, a0, fw, tabf, tfield, pf, cl, cs, dF, dphi, da, db, dcv, v, ogm,
             (float)gamma, out);
   } else if (m.flux_type == AMPE_FLUX_ANISOTROPIC) {
      if (!an) return AMPE_ERR_INVALID;
      if (mp.pb)
         k_jv_stencil<2, true, true><<<(unsigned)b, 256, 0, s>>>(
             m, mp, g, a0, fw, tabf, tfield, pf, cl, cs, dF, dphi, da, db, dcv, v, ogm,
             (float)gamma, out);
      else
         k_jv_stencil<2, false, true><<<(unsigned)b, 256, 0, s>>>(
             m, mp, g, a0, fw, tabf, tfield, pf, cl, cs, dF, dphi, da, db, dcv, v, ogm,
             (float)gamma, out);
   } else if (g.dim == 3) {
      if (mp.pb)
         AMPE_JV(3, true);
      else
         AMPE_JV(3, false);
   } else {
      if (mp.pb)
         AMPE_JV(2, true);
      else
         AMPE_JV(2, false);
   }
#undef AMPE_JV
   int rc = launch_status();
   if (qf && !rc) {
      if (g.dim == 3)
         k_jv_quat<3><<<(unsigned)b, 256, 0, s>>>(m, mp, g, pf, dphi, *qf, v, (float)gamma, out);
      else
         k_jv_quat<2><<<(unsigned)b, 256, 0, s>>>(m, mp, g, pf, dphi, *qf, v, (float)gamma, out);
      rc = launch_status();
   }
   return rc;
}

int quat_cells_f32(const ampe_model_t& m, const MixParams& mp, const Grid& g,
                   const double* phi, QuatF32& qf, cudaStream_t s)
{
   long long b = (g.cells() + 255) / 256;
   if (b > max_blocks()) b = max_blocks();
   if (g.dim == 3)
      k_quat_cells_f32<3><<<(unsigned)b, 256, 0, s>>>(mp, g, phi, qf.q, qf.ogm, qf.mq);
   else
      k_quat_cells_f32<2><<<(unsigned)b, 256, 0, s>>>(mp, g, phi, qf.q, qf.ogm, qf.mq);
   return launch_status();
}

int conc_faces_f32(const ampe_model_t& m, const MixParams& mp, const Grid& g,
                   const FaceW& fw, double gamma, float* const D[3], cudaStream_t s)
{
   (void)m;
   const long long nz = g.dim == 3 ? g.nfz() : 0;
   const long long tot = g.nfx() + g.nfy() + nz;
   long long b = (tot + 255) / 256;
   if (b > max_blocks()) b = max_blocks();
   FacePtrs f;
   for (int d = 0; d < 3; d++) {
      f.fc[d] = D[d];
      f.dfc[d] = nullptr;
   }
   k_conc_faces_f32<<<(unsigned)b, 256, 0, s>>>(g.nfx(), g.nfy(), nz, fw, (float)gamma,
                                                mp.kksc, f);
   return launch_status();
}

int quat_faces_f32(const ampe_model_t& m, const MixParams& mp, const Grid& g,
                   const double* tfield, const float* pf, const float* q,
                   double scale, float* const fc[3], float* const dfc[3],
                   cudaStream_t s)
{
   const long long tot = g.nfx() + g.nfy() + (g.dim == 3 ? g.nfz() : 0);
   long long b = (tot + 255) / 256;
   if (b > max_blocks()) b = max_blocks();
   FacePtrs f;
   for (int d = 0; d < 3; d++) {
      f.fc[d] = fc[d];
      f.dfc[d] = dfc ? dfc[d] : nullptr;
   }
   if (g.dim == 3)
      k_quat_faces_f32<3><<<(unsigned)b, 256, 0, s>>>(m, mp, g, tfield, pf, q, (float)scale, f);
   else
      k_quat_faces_f32<2><<<(unsigned)b, 256, 0, s>>>(m, mp, g, tfield, pf, q, (float)scale, f);
   return launch_status();
}

}  // namespace ampe
