// CPU restatement of AMPE's multi-level (AMR) FAC on a two-level composite
// grid: a periodic coarse level and one fine box refined by 2.
// TEST INFRASTRUCTURE ONLY (the checker of ampe_fac2_*).
//   solveSystem / computeFullCompositeResidual / facCycle_Recursive
//       samrai/FACPreconditioner.cc:267-464, 661-683
//   computeCompositeResidualOnLevel     EllipticFACOps.cc:1593-1758
//   computeFluxOnPatch, ewingFixFlux    EllipticFACOps.cc:1947-2029, 1239-1347
//   smoothErrorByRedBlack               EllipticFACOps.cc:1067-1230
//   restrictSolution/Residual, prolongErrorAndCorrect  EllipticFACOps.cc:948-1045
//   solveCoarsestLevel ("redblack")     EllipticFACOps.cc:1356-1384
//   efo_compfluxvardc3d, efo_compresvarsca3d, efo_rbgswithfluxmax*3d,
//   efo_ewingfixflux*3d                 3d/ellipticfacops.m4:16-82, 83-447,
//                                       448-512, 697-1105
// Ghost cells of the fine level come from the coarse level by constant
// refinement (the "Ewing" coarse-fine discretisation's ghost fill); the
// volume- and area-weighted averages are SAMRAI's conservative coarsening
// of cell and side data, written as (sum of fine value x fine measure) /
// coarse measure in (k, j, i) order.
#include <cmath>
#include <cstring>
#include <vector>

#include "oracle_api.h"
#include "oracle_common.h"

using namespace orc;

namespace {

struct Level {
   ampe_model_t m;
   const double* D[3];
   const double* C;
   const double* M;
   double dc, cc, mc;
   double D_at(int d, long f) const { return D[d] ? D[d][f] : dc; }
   double C_at(long c) const { return C ? C[c] : cc; }
   double M_at(long c) const { return M ? M[c] : mc; }
};

struct Two {
   const ampe_fac2_t* p;
   Level c, f;
   double flux_dinv_c[3], flux_dinv_f[3];  // 1/dx used for fluxes
   double ewing_h[3];                      // h of the Ewing correction
   double tranwt, longwt;
};

int fdiv(int a, int b) { return a >= 0 ? a / b : -((-a + b - 1) / b); }
int wrapi(int a, int n) { return ((a % n) + n) % n; }

long faces(const Layout& L, int d)
{
   return d == 0 ? L.nfx() : (d == 1 ? L.nfy() : L.nfz());
}
long face(const Layout& L, int d, int i, int j, int k)
{
   return d == 0 ? L.fx(i, j, k) : (d == 1 ? L.fy(i, j, k) : L.fz(i, j, k));
}

// fine ghost cells <- the coarse cell they lie in (CONSTANT_REFINE)
void cf_fill(const Two& T, const double* uc, double* uf)
{
   Layout Lc(T.c.m), Lf(T.f.m);
   const ampe_fac2_t& p = *T.p;
   for (int k = -Lf.gz; k < Lf.n2 + Lf.gz; k++)
      for (int j = -Lf.ng; j < Lf.n1 + Lf.ng; j++)
         for (int i = -Lf.ng; i < Lf.n0 + Lf.ng; i++) {
            if (i >= 0 && i < Lf.n0 && j >= 0 && j < Lf.n1 && k >= 0 && k < Lf.n2) continue;
            const int I = wrapi(p.lo[0] + fdiv(i, 2), Lc.n0);
            const int J = wrapi(p.lo[1] + fdiv(j, 2), Lc.n1);
            const int K = wrapi(p.lo[2] + fdiv(k, 2), Lc.n2);
            uf[Lf.c(i, j, k)] = uc[Lc.c(I, J, K)];
         }
}

// efo_compfluxvardc3d on every interior face
void comp_flux(const Level& lv, const double* dinv, const double* u, double* const* flux)
{
   Layout L(lv.m);
   for (int d = 0; d < 3; d++) {
      const int ei = d == 0, ej = d == 1, ek = d == 2;
      for (int k = 0; k < L.n2 + ek; k++)
         for (int j = 0; j < L.n1 + ej; j++)
            for (int i = 0; i < L.n0 + ei; i++) {
               const long f = face(L, d, i, j, k);
               flux[d][f] = dinv[d] * lv.D_at(d, f) *
                            (u[L.c(i, j, k)] - u[L.c(i - ei, j - ej, k - ek)]);
            }
   }
}

// efo_ewingfixflux*3d on the six sides of the fine box
void ewing(const Two& T, const double* u, double* const* flux)
{
   Layout L(T.f.m);
   const int n[3] = {L.n0, L.n1, L.n2};
   for (int loc = 0; loc < 6; loc++) {
      const int d = loc / 2, hi = loc % 2;
      const int cell = hi ? n[d] - 1 : 0, bnd = hi ? n[d] : 0;
      const double sgn = hi ? -1.0 : 1.0;
      // the reference's loop nests: x sides (k, j), y sides (i, k), z sides (i, j)
      const int outer = d == 0 ? 2 : 0, inner = d == 0 ? 1 : (d == 1 ? 2 : 1);
      for (int o = 0; o < n[outer]; o += 2)
         for (int q = 0; q < n[inner]; q += 2)
            for (int op = 0; op < 2; op++)
               for (int qp = 0; qp < 2; qp++) {
                  const int oq = 1 - op, qq = 1 - qp;
                  int at[3], opp[3];
                  at[d] = opp[d] = cell;
                  at[outer] = o + op;
                  at[inner] = q + qp;
                  opp[outer] = o + oq;
                  opp[inner] = q + qq;
                  int fi[3] = {at[0], at[1], at[2]};
                  fi[d] = bnd;
                  const long f = face(L, d, fi[0], fi[1], fi[2]);
                  const double diff = u[L.c(opp[0], opp[1], opp[2])] - u[L.c(at[0], at[1], at[2])];
                  flux[d][f] = T.longwt * flux[d][f] +
                               sgn * (T.tranwt * T.f.D_at(d, f) * diff / T.ewing_h[d]);
               }
   }
}

// efo_compresvarsca3d
void comp_res(const Level& lv, double* const* flux, const double* u, const double* rhs,
              double* r)
{
   Layout L(lv.m);
   const double dxi = 1.0 / lv.m.dx[0], dyi = 1.0 / lv.m.dx[1], dzi = 1.0 / lv.m.dx[2];
   for (int k = 0; k < L.n2; k++)
      for (int j = 0; j < L.n1; j++)
         for (int i = 0; i < L.n0; i++) {
            const long c = L.c(i, j, k);
            r[c] = rhs[c] -
                   lv.M_at(c) * (dxi * (flux[0][L.fx(i + 1, j, k)] - flux[0][L.fx(i, j, k)]) +
                                 dyi * (flux[1][L.fy(i, j + 1, k)] - flux[1][L.fy(i, j, k)]) +
                                 dzi * (flux[2][L.fz(i, j, k + 1)] - flux[2][L.fz(i, j, k)])) -
                   lv.C_at(c) * u[c];
         }
}

// efo_rbgswithfluxmax*3d, one colour (offset 0 red, 1 black)
void rbgs_flux(const Level& lv, double* const* flux, const double* rhs, double* u, int offset)
{
   Layout L(lv.m);
   const double dxi = 1.0 / lv.m.dx[0], dyi = 1.0 / lv.m.dx[1], dzi = 1.0 / lv.m.dx[2];
   const double dxi2 = dxi * dxi, dyi2 = dyi * dyi, dzi2 = dzi * dzi;
   for (int k = 0; k < L.n2; k++)
      for (int j = 0; j < L.n1; j++) {
         const int io = ((j + k) % 2 != offset) ? 1 : 0;
         for (int i = io; i < L.n0; i += 2) {
            const long c = L.c(i, j, k);
            const double m = lv.M_at(c);
            const double res =
                rhs[c] -
                m * (dxi * (flux[0][L.fx(i + 1, j, k)] - flux[0][L.fx(i, j, k)]) +
                     dyi * (flux[1][L.fy(i, j + 1, k)] - flux[1][L.fy(i, j, k)]) +
                     dzi * (flux[2][L.fz(i, j, k + 1)] - flux[2][L.fz(i, j, k)])) -
                lv.C_at(c) * u[c];
            const double dudr =
                1.0 / (m * (dxi2 * (lv.D_at(0, L.fx(i + 1, j, k)) + lv.D_at(0, L.fx(i, j, k))) +
                            dyi2 * (lv.D_at(1, L.fy(i, j + 1, k)) + lv.D_at(1, L.fy(i, j, k))) +
                            dzi2 * (lv.D_at(2, L.fz(i, j, k + 1)) + lv.D_at(2, L.fz(i, j, k)))) -
                       lv.C_at(c));
            const double du = -res * dudr;
            u[c] = u[c] + du * 1.0;
         }
      }
}

// smoothErrorByRedBlack with a fixed number of sweeps
void smooth(const Two& T, bool fine, double* e, const double* r, int sweeps, double* const* flux,
            const double* ec)
{
   const Level& lv = fine ? T.f : T.c;
   if (fine) cf_fill(T, ec, e);  // one-time transfer from the coarser level
   else orc_fill_ghosts(&lv.m, e);
   for (int s = 0; s < sweeps; s++)
      for (int off = 0; off < 2; off++) {
         if (!fine) orc_fill_ghosts(&lv.m, e);
         comp_flux(lv, fine ? T.flux_dinv_f : T.flux_dinv_c, e, flux);
         if (fine) ewing(T, e, flux);
         rbgs_flux(lv, flux, r, e, off);
      }
   if (!fine) orc_fill_ghosts(&lv.m, e);
}

// conservative coarsening of cell data into the coarse cells under the box
void restrict_cells(const Two& T, const double* vf, double* vc)
{
   Layout Lc(T.c.m), Lf(T.f.m);
   const ampe_fac2_t& p = *T.p;
   const double dvf = T.f.m.dx[0] * T.f.m.dx[1] * T.f.m.dx[2];
   const double dvc = T.c.m.dx[0] * T.c.m.dx[1] * T.c.m.dx[2];
   for (int K = 0; K < p.nbox[2]; K++)
      for (int J = 0; J < p.nbox[1]; J++)
         for (int I = 0; I < p.nbox[0]; I++) {
            double s = 0.0;
            for (int kr = 0; kr < 2; kr++)
               for (int jr = 0; jr < 2; jr++)
                  for (int ir = 0; ir < 2; ir++)
                     s += vf[Lf.c(2 * I + ir, 2 * J + jr, 2 * K + kr)] * dvf;
            vc[Lc.c(wrapi(p.lo[0] + I, Lc.n0), wrapi(p.lo[1] + J, Lc.n1),
                    wrapi(p.lo[2] + K, Lc.n2))] = s / dvc;
         }
}

// conservative coarsening of the fine fluxes on the box's boundary faces
// onto the coarse faces there (xeqScheduleFluxCoarsen of the outer fluxes)
void coarsen_boundary_flux(const Two& T, double* const* ff, double* const* fc)
{
   Layout Lc(T.c.m), Lf(T.f.m);
   const ampe_fac2_t& p = *T.p;
   const double* dxf = T.f.m.dx;
   const double* dxc = T.c.m.dx;
   for (int d = 0; d < 3; d++) {
      const int a = d == 0 ? 1 : 0, b = d == 2 ? 1 : 2;
      const double daf = dxf[a] * dxf[b], dac = dxc[a] * dxc[b];
      for (int side = 0; side < 2; side++) {
         const int Fn = side ? p.nbox[d] : 0;  // coarse face index relative to lo
         for (int B = 0; B < p.nbox[b]; B++)
            for (int A = 0; A < p.nbox[a]; A++) {
               double s = 0.0;
               for (int br = 0; br < 2; br++)
                  for (int ar = 0; ar < 2; ar++) {
                     int fi[3];
                     fi[d] = 2 * Fn;
                     fi[a] = 2 * A + ar;
                     fi[b] = 2 * B + br;
                     s += ff[d][face(Lf, d, fi[0], fi[1], fi[2])] * daf;
                  }
               int ci[3];
               ci[d] = p.lo[d] + Fn;
               ci[a] = p.lo[a] + A;
               ci[b] = p.lo[b] + B;
               // coarse face index: faces 0..n_d; the wrapped image of n_d is 0
               const int n[3] = {Lc.n0, Lc.n1, Lc.n2};
               for (int e = 0; e < 3; e++)
                  if (e != d) ci[e] = wrapi(ci[e], n[e]);
               ci[d] = wrapi(ci[d], n[d]);
               fc[d][face(Lc, d, ci[0], ci[1], ci[2])] = s / dac;
               if (ci[d] == 0) fc[d][face(Lc, d, ci[0] + (d == 0) * n[0], ci[1] + (d == 1) * n[1],
                                          ci[2] + (d == 2) * n[2])] = s / dac;
            }
      }
   }
}

// computeFullCompositeResidual: fine residual, u_f restricted, coarse
// residual with the fine boundary fluxes, fine residual restricted
double composite_residual(const Two& T, const double* fcr, const double* ffr, double* uc,
                          double* uf, double* rc, double* rf, double* const* fluxc,
                          double* const* fluxf)
{
   cf_fill(T, uc, uf);
   comp_flux(T.f, T.flux_dinv_f, uf, fluxf);
   ewing(T, uf, fluxf);
   comp_res(T.f, fluxf, uf, ffr, rf);
   restrict_cells(T, uf, uc);
   orc_fill_ghosts(&T.c.m, uc);
   comp_flux(T.c, T.flux_dinv_c, uc, fluxc);
   coarsen_boundary_flux(T, fluxf, fluxc);
   comp_res(T.c, fluxc, uc, fcr, rc);
   restrict_cells(T, rf, rc);
   // weighted RMS: fine cells, coarse cells outside the box
   Layout Lc(T.c.m), Lf(T.f.m);
   const double dvf = T.f.m.dx[0] * T.f.m.dx[1] * T.f.m.dx[2];
   const double dvc = T.c.m.dx[0] * T.c.m.dx[1] * T.c.m.dx[2];
   double num = 0.0;
   long ncoarse = 0;
   for (int k = 0; k < Lf.n2; k++)
      for (int j = 0; j < Lf.n1; j++)
         for (int i = 0; i < Lf.n0; i++) {
            const double v = rf[Lf.c(i, j, k)];
            num += dvf * v * v;
         }
   const ampe_fac2_t& p = *T.p;
   for (int k = 0; k < Lc.n2; k++)
      for (int j = 0; j < Lc.n1; j++)
         for (int i = 0; i < Lc.n0; i++) {
            const bool under = wrapi(i - p.lo[0], Lc.n0) < p.nbox[0] &&
                               wrapi(j - p.lo[1], Lc.n1) < p.nbox[1] &&
                               wrapi(k - p.lo[2], Lc.n2) < p.nbox[2];
            if (under) continue;
            const double v = rc[Lc.c(i, j, k)];
            num += dvc * v * v;
            ncoarse++;
         }
   const double den = (double)Lf.cells() * dvf + (double)ncoarse * dvc;
   return std::sqrt(num / den);
}

bool setup(Two& T, const ampe_fac2_t* p, const ampe_fac2_level_t* lc, const ampe_fac2_level_t* lf)
{
   if (!p || p->coarse.dim != 3 || p->ng_fine < 1 || p->coarse.ng < 1) return false;
   for (int d = 0; d < 3; d++)
      if (p->nbox[d] < 2 || p->nbox[d] > p->coarse.n[d]) return false;
   T.p = p;
   T.c.m = p->coarse;
   T.c.m.ng_side = 0;
   T.f.m = p->coarse;
   T.f.m.ng = p->ng_fine;
   T.f.m.ng_side = 0;
   for (int d = 0; d < 3; d++) {
      T.f.m.n[d] = 2 * p->nbox[d];
      T.f.m.dx[d] = 0.5 * p->coarse.dx[d];
   }
   const ampe_fac2_level_t* src[2] = {lc, lf};
   Level* dst[2] = {&T.c, &T.f};
   for (int l = 0; l < 2; l++) {
      for (int d = 0; d < 3; d++) dst[l]->D[d] = src[l] ? src[l]->D[d] : nullptr;
      dst[l]->C = src[l] ? src[l]->C : nullptr;
      dst[l]->M = src[l] ? src[l]->M : nullptr;
      dst[l]->dc = p->d_const;
      dst[l]->cc = p->c_const;
      dst[l]->mc = p->m_const;
   }
   for (int d = 0; d < 3; d++) {
      T.flux_dinv_c[d] = 1.0 / p->coarse.dx[d];
      // the reference: the grid geometry's (level 0) spacing on every level
      T.flux_dinv_f[d] = 1.0 / (p->level_dx ? T.f.m.dx[d] : p->coarse.dx[d]);
      T.ewing_h[d] = p->level_dx ? T.f.m.dx[d] : p->coarse.dx[d];
   }
   // 1.0/(1+ratio): a single-precision quotient in the reference
   T.tranwt = (double)(1.0f / (float)(1 + 2));
   T.longwt = 2 * T.tranwt;
   return true;
}

}  // namespace

extern "C" {

long long orc_fac2_work_doubles(const ampe_fac2_t* p)
{
   Two T;
   if (!setup(T, p, nullptr, nullptr)) return -1;
   Layout Lc(T.c.m), Lf(T.f.m);
   long long n = 2 * (long long)Lc.cells_ghost() + 3 * (long long)Lf.cells_ghost();
   for (int d = 0; d < 3; d++) n += faces(Lc, d) + faces(Lf, d);
   return n;
}

double orc_fac2_composite_residual(const ampe_fac2_t* p, const ampe_fac2_level_t* lc,
                                   const ampe_fac2_level_t* lf, const double* fc,
                                   const double* ff, double* uc, double* uf, double* rc,
                                   double* rf)
{
   Two T;
   if (!setup(T, p, lc, lf)) return -1.0;
   Layout Lc(T.c.m), Lf(T.f.m);
   std::vector<double> fxc[3], fxf[3];
   double *pc[3], *pf[3];
   for (int d = 0; d < 3; d++) {
      fxc[d].assign(faces(Lc, d), 0.0);
      fxf[d].assign(faces(Lf, d), 0.0);
      pc[d] = fxc[d].data();
      pf[d] = fxf[d].data();
   }
   return composite_residual(T, fc, ff, uc, uf, rc, rf, pc, pf);
}

int orc_fac2_solve(const ampe_fac2_t* p, const ampe_fac2_level_t* lc,
                   const ampe_fac2_level_t* lf, const double* fc, const double* ff,
                   double* uc, double* uf, int max_cycles, double tol, double* norms)
{
   Two T;
   if (!setup(T, p, lc, lf)) return -1;
   Layout Lc(T.c.m), Lf(T.f.m);
   std::vector<double> rc(Lc.cells_ghost(), 0.0), rf(Lf.cells_ghost(), 0.0);
   std::vector<double> ec(Lc.cells_ghost()), ef(Lf.cells_ghost()), tf(Lf.cells_ghost(), 0.0);
   std::vector<double> fxc[3], fxf[3];
   double *pc[3], *pf[3];
   for (int d = 0; d < 3; d++) {
      fxc[d].assign(faces(Lc, d), 0.0);
      fxf[d].assign(faces(Lf, d), 0.0);
      pc[d] = fxc[d].data();
      pf[d] = fxf[d].data();
   }
   double norm = composite_residual(T, fc, ff, uc, uf, rc.data(), rf.data(), pc, pf);
   if (norms) norms[0] = norm;
   int it = 0;
   while (it < max_cycles && !(norm <= tol)) {
      std::fill(ec.begin(), ec.end(), 0.0);
      std::fill(ef.begin(), ef.end(), 0.0);
      // facCycle_Recursive, ln = 1
      smooth(T, true, ef.data(), rf.data(), p->presweeps, pf, ec.data());
      cf_fill(T, ec.data(), ef.data());
      comp_flux(T.f, T.flux_dinv_f, ef.data(), pf);
      ewing(T, ef.data(), pf);
      comp_res(T.f, pf, ef.data(), rf.data(), tf.data());
      restrict_cells(T, tf.data(), rc.data());
      // ln = 0: solveCoarsestLevel
      smooth(T, false, ec.data(), rc.data(), p->coarse_sweeps, pc, nullptr);
      // prolongErrorAndCorrect (constant refinement into the fine interior)
      for (int k = 0; k < Lf.n2; k++)
         for (int j = 0; j < Lf.n1; j++)
            for (int i = 0; i < Lf.n0; i++) {
               const long cf = Lf.c(i, j, k);
               ef[cf] = ef[cf] + ec[Lc.c(wrapi(p->lo[0] + i / 2, Lc.n0),
                                         wrapi(p->lo[1] + j / 2, Lc.n1),
                                         wrapi(p->lo[2] + k / 2, Lc.n2))];
            }
      smooth(T, true, ef.data(), rf.data(), p->postsweeps, pf, ec.data());
      // u += e on both levels' interiors, then u_c <- R u_f under the box
      for (int k = 0; k < Lc.n2; k++)
         for (int j = 0; j < Lc.n1; j++)
            for (int i = 0; i < Lc.n0; i++) uc[Lc.c(i, j, k)] += ec[Lc.c(i, j, k)];
      for (int k = 0; k < Lf.n2; k++)
         for (int j = 0; j < Lf.n1; j++)
            for (int i = 0; i < Lf.n0; i++) uf[Lf.c(i, j, k)] += ef[Lf.c(i, j, k)];
      restrict_cells(T, uf, uc);
      norm = composite_residual(T, fc, ff, uc, uf, rc.data(), rf.data(), pc, pf);
      it++;
      if (norms) norms[it] = norm;
   }
   return it;
}

}  // extern "C"
