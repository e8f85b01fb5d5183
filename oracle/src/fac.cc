// CPU restatement of the single-level FAC operator kernels and of the
// within-level multigrid that replaces the reference's hypre coarse solve.
// TEST INFRASTRUCTURE ONLY.
//
// Operator (EllipticFACOps, doc/latex/manual/algorithm.tex:193-250):
//   A u = C u + M div(D grad u)
// red-black update  (3d/ellipticfacops.m4:83-177, 267-359)
//   r    = f - M sum_d dxi_d (flux_d(+) - flux_d(-)) - C u,
//   flux = dxi_d D (u - u_nbr)
//   u   += r / (C - M sum_d dxi_d^2 (D(+) + D(-)))
// on cells with (i+j+k) % 2 == offset, ghosts refilled between colours.
#include <algorithm>
#include <cstring>

#include "oracle_api.h"
#include "oracle_common.h"

using namespace orc;

namespace {

struct Op {
   ampe_model_t m;  // grid part used: dim, n, ng, dx
   const double* D[3];
   double Dc;
   const double* C;
   double Cc;
   const double* M;
   double Mc;
};

double faceD(const Op& op, const Layout& L, int dir, int i, int j, int k)
{
   if (!op.D[0]) return op.Dc;
   if (dir == 0) return op.D[0][L.fx(i, j, k)];
   if (dir == 1) return op.D[1][L.fy(i, j, k)];
   return op.D[2][L.fz(i, j, k)];
}

double cellM(const Op& op, const Layout& L, int i, int j, int k)
{
   return op.M ? op.M[L.c(i, j, k)] : op.Mc;
}
double cellC(const Op& op, const Layout& L, int i, int j, int k)
{
   return op.C ? op.C[L.c(i, j, k)] : op.Cc;
}

// residual r = f - A u at one cell; also returns the diagonal inverse
double cell_residual(const Op& op, const Layout& L, const double* f,
                     const double* u, int i, int j, int k, double* dudr)
{
   const double* dx = op.m.dx;
   const double dxi[3] = {1.0 / dx[0], 1.0 / dx[1],
                          L.dim == 3 ? 1.0 / dx[2] : 0.0};
   const long c = L.c(i, j, k);
   double div = 0.0, dsum = 0.0;
   for (int d = 0; d < L.dim; d++) {
      const int ei = d == 0, ej = d == 1, ek = d == 2;
      const double Dm = faceD(op, L, d, i, j, k);
      const double Dp = faceD(op, L, d, i + ei, j + ej, k + ek);
      const double fm = dxi[d] * Dm * (u[c] - u[L.c(i - ei, j - ej, k - ek)]);
      const double fp = dxi[d] * Dp * (u[L.c(i + ei, j + ej, k + ek)] - u[c]);
      div += dxi[d] * (fp - fm);
      dsum += dxi[d] * dxi[d] * (Dp + Dm);
   }
   const double M = cellM(op, L, i, j, k), C = cellC(op, L, i, j, k);
   if (dudr) *dudr = 1.0 / (M * dsum - C);
   return f[c] - M * div - C * u[c];
}

}  // namespace

extern "C" {

// One colour of EFO_RBGSWITHFLUXMAX*; returns max |residual| of the colour.
double orc_efo_rbgs(const ampe_model_t* m, const double* d0, const double* d1,
                    const double* d2, double dc, const double* ccell,
                    double cc, const double* mcell, double mc,
                    const double* f, double* u, int offset)
{
   Layout L(*m);
   Op op{*m, {d0, d1, d2}, dc, ccell, cc, mcell, mc};
   double maxres = 0.0;
#pragma omp parallel for collapse(2) reduction(max : maxres) schedule(static)
   for (int k = 0; k < L.n2; k++)
      for (int j = 0; j < L.n1; j++)
         for (int i = 0; i < L.n0; i++) {
            if (((i + j + k) & 1) != offset) continue;
            double dudr;
            const double r = cell_residual(op, L, f, u, i, j, k, &dudr);
            u[L.c(i, j, k)] += -r * dudr;
            maxres = std::max(maxres, std::fabs(r));
         }
   return maxres;
}

void orc_efo_residual(const ampe_model_t* m, const double* d0,
                      const double* d1, const double* d2, double dc,
                      const double* ccell, double cc, const double* mcell,
                      double mc, const double* f, const double* u, double* res)
{
   Layout L(*m);
   Op op{*m, {d0, d1, d2}, dc, ccell, cc, mcell, mc};
#pragma omp parallel for collapse(2) schedule(static)
   for (int k = 0; k < L.n2; k++)
      for (int j = 0; j < L.n1; j++)
         for (int i = 0; i < L.n0; i++)
            res[L.c(i, j, k)] = cell_residual(op, L, f, u, i, j, k, nullptr);
}

// PhaseFACOps::setCOnPatchPrivate (PhaseFACOps.cc:101-183)
void orc_phase_fac_set_c(const ampe_model_t* m, const double* phi,
                         double gamma, double* ccell)
{
   Layout L(*m);
   for (int k = 0; k < L.n2; k++)
      for (int j = 0; j < L.n1; j++)
         for (int i = 0; i < L.n0; i++) {
            const long c = L.c(i, j, k);
            const double g2 = second_deriv_well_func(phi[c], m->well_type);
            const double gm = gamma * m->phase_mobility;
            ccell[c] = 1.0 + gm * m->phase_well_scale * g2;
         }
}

double orc_rms_interior(const ampe_model_t* m, const double* v)
{
   Layout L(*m);
   double s = 0.0;
#pragma omp parallel for collapse(2) reduction(+ : s) schedule(static)
   for (int k = 0; k < L.n2; k++)
      for (int j = 0; j < L.n1; j++)
         for (int i = 0; i < L.n0; i++) {
            const double x = v[L.c(i, j, k)];
            s += x * x;
         }
   return std::sqrt(s / (double)L.cells());
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Multigrid hierarchy: level l has n/2^l cells and spacing dx*2^l; C, M
// and face D are averages of the finer level's children; restriction is the
// mean of the 2^d children; prolongation is piecewise constant.
// ---------------------------------------------------------------------------
namespace orc {

struct MGLevel {
   ampe_model_t m;
   std::vector<double> D[3], C, M, u, f, r;
   bool hasD = false, hasC = false, hasM = false;
   double Dc = 0, Cc = 0, Mc = 0;
};

struct FacSolver {
   std::vector<MGLevel> lev;
};

}  // namespace orc

namespace {

void ghosted_alloc(MGLevel& l)
{
   Layout L(l.m);
   l.u.assign(L.cells_ghost(), 0.0);
   l.f.assign(L.cells_ghost(), 0.0);
   l.r.assign(L.cells_ghost(), 0.0);
}

Op level_op(const MGLevel& l)
{
   Op op{l.m,
         {l.hasD ? l.D[0].data() : nullptr, l.hasD ? l.D[1].data() : nullptr,
          (l.hasD && l.m.dim == 3) ? l.D[2].data() : nullptr},
         l.Dc,
         l.hasC ? l.C.data() : nullptr,
         l.Cc,
         l.hasM ? l.M.data() : nullptr,
         l.Mc};
   return op;
}

void rb_sweep(MGLevel& l, double* red_max, double* blk_max)
{
   Op op = level_op(l);
   const double* D0 = op.D[0];
   double mr = orc_efo_rbgs(&l.m, D0, op.D[1], op.D[2], op.Dc, op.C, op.Cc,
                            op.M, op.Mc, l.f.data(), l.u.data(), 0);
   orc_fill_ghosts(&l.m, l.u.data());
   double mb = orc_efo_rbgs(&l.m, D0, op.D[1], op.D[2], op.Dc, op.C, op.Cc,
                            op.M, op.Mc, l.f.data(), l.u.data(), 1);
   orc_fill_ghosts(&l.m, l.u.data());
   if (red_max) *red_max = mr;
   if (blk_max) *blk_max = mb;
}

void residual(MGLevel& l)
{
   Op op = level_op(l);
   orc_efo_residual(&l.m, op.D[0], op.D[1], op.D[2], op.Dc, op.C, op.Cc, op.M,
                    op.Mc, l.f.data(), l.u.data(), l.r.data());
}

void restrict_to(const MGLevel& fine, const std::vector<double>& src,
                 MGLevel& coarse, std::vector<double>& dst)
{
   Layout Lf(fine.m), Lc(coarse.m);
   const int dz = Lf.dim == 3 ? 2 : 1;
   const double w = Lf.dim == 3 ? 0.125 : 0.25;
#pragma omp parallel for collapse(2) schedule(static)
   for (int k = 0; k < Lc.n2; k++)
      for (int j = 0; j < Lc.n1; j++)
         for (int i = 0; i < Lc.n0; i++) {
            double s = 0.0;
            for (int c = 0; c < dz; c++)
               for (int b = 0; b < 2; b++)
                  for (int a = 0; a < 2; a++)
                     s += src[Lf.c(2 * i + a, 2 * j + b, dz * k + c)];
            dst[Lc.c(i, j, k)] = w * s;
         }
}

void prolong_add(const MGLevel& coarse, MGLevel& fine)
{
   Layout Lf(fine.m), Lc(coarse.m);
   const int dz = Lf.dim == 3 ? 2 : 1;
#pragma omp parallel for collapse(2) schedule(static)
   for (int k = 0; k < Lf.n2; k++)
      for (int j = 0; j < Lf.n1; j++)
         for (int i = 0; i < Lf.n0; i++)
            fine.u[Lf.c(i, j, k)] += coarse.u[Lc.c(i / 2, j / 2, k / dz)];
}

void vcycle(FacSolver& s, int l, const ampe_step_params_t& p)
{
   MGLevel& L = s.lev[l];
   std::fill(L.u.begin(), L.u.end(), 0.0);
   if (l == (int)s.lev.size() - 1) {
      for (int it = 0; it < p.mg_coarse_sweeps; it++) rb_sweep(L, 0, 0);
      return;
   }
   for (int it = 0; it < p.mg_pre; it++) rb_sweep(L, 0, 0);
   residual(L);
   MGLevel& C = s.lev[l + 1];
   restrict_to(L, L.r, C, C.f);
   vcycle(s, l + 1, p);
   orc_fill_ghosts(&C.m, C.u.data());
   prolong_add(C, L);
   orc_fill_ghosts(&L.m, L.u.data());
   for (int it = 0; it < p.mg_post; it++) rb_sweep(L, 0, 0);
}

}  // namespace

extern "C" {

void* orc_fac_create(const ampe_model_t* m, int nlevels)
{
   FacSolver* s = new FacSolver;
   ampe_model_t mm = *m;
   for (int l = 0; l < nlevels; l++) {
      MGLevel lv;
      lv.m = mm;
      ghosted_alloc(lv);
      s->lev.push_back(lv);
      const int dz = mm.dim == 3 ? 2 : 1;
      if (mm.n[0] % 2 || mm.n[1] % 2 || (mm.dim == 3 && mm.n[2] % 2)) break;
      mm.n[0] /= 2;
      mm.n[1] /= 2;
      if (mm.dim == 3) mm.n[2] /= dz;
      for (int d = 0; d < 3; d++) mm.dx[d] *= 2.0;
   }
   return s;
}

void orc_fac_destroy(void* h) { delete (FacSolver*)h; }

// Set the fine-level operator: D faces (NULL -> constant dc), C, M cell
// arrays in the ghosted layout (NULL -> constants), and build the coarse
// levels by averaging.
void orc_fac_set_operator(void* h, const double* d0, const double* d1,
                          const double* d2, double dc, const double* ccell,
                          double cc, const double* mcell, double mc)
{
   FacSolver* s = (FacSolver*)h;
   for (size_t l = 0; l < s->lev.size(); l++) {
      MGLevel& lv = s->lev[l];
      Layout L(lv.m);
      lv.hasD = d0 != nullptr;
      lv.hasC = ccell != nullptr;
      lv.hasM = mcell != nullptr;
      lv.Dc = dc;
      lv.Cc = cc;
      lv.Mc = mc;
      if (l == 0) {
         if (lv.hasD) {
            lv.D[0].assign(d0, d0 + L.nfx());
            lv.D[1].assign(d1, d1 + L.nfy());
            if (L.dim == 3) lv.D[2].assign(d2, d2 + L.nfz());
         }
         if (lv.hasC) lv.C.assign(ccell, ccell + L.cells_ghost());
         if (lv.hasM) lv.M.assign(mcell, mcell + L.cells_ghost());
         continue;
      }
      const MGLevel& fl = s->lev[l - 1];
      Layout Lf(fl.m);
      const int dz = L.dim == 3 ? 2 : 1;
      const double w = L.dim == 3 ? 0.125 : 0.25;
      if (lv.hasC) {
         lv.C.assign(L.cells_ghost(), 0.0);
         restrict_to(fl, fl.C, lv, lv.C);
      }
      if (lv.hasM) {
         lv.M.assign(L.cells_ghost(), 0.0);
         restrict_to(fl, fl.M, lv, lv.M);
      }
      if (lv.hasD) {
         const double wf = L.dim == 3 ? 0.25 : 0.5;
         lv.D[0].assign(L.nfx(), 0.0);
         lv.D[1].assign(L.nfy(), 0.0);
         if (L.dim == 3) lv.D[2].assign(L.nfz(), 0.0);
         for (int k = 0; k < L.n2; k++)
            for (int j = 0; j < L.n1; j++)
               for (int i = 0; i <= L.n0; i++) {
                  double s2 = 0.0;
                  for (int c = 0; c < dz; c++)
                     for (int b = 0; b < 2; b++)
                        s2 += fl.D[0][Lf.fx(2 * i, 2 * j + b, dz * k + c)];
                  lv.D[0][L.fx(i, j, k)] = wf * s2;
               }
         for (int k = 0; k < L.n2; k++)
            for (int j = 0; j <= L.n1; j++)
               for (int i = 0; i < L.n0; i++) {
                  double s2 = 0.0;
                  for (int c = 0; c < dz; c++)
                     for (int a = 0; a < 2; a++)
                        s2 += fl.D[1][Lf.fy(2 * i + a, 2 * j, dz * k + c)];
                  lv.D[1][L.fy(i, j, k)] = wf * s2;
               }
         if (L.dim == 3)
            for (int k = 0; k <= L.n2; k++)
               for (int j = 0; j < L.n1; j++)
                  for (int i = 0; i < L.n0; i++) {
                     double s2 = 0.0;
                     for (int b = 0; b < 2; b++)
                        for (int a = 0; a < 2; a++)
                           s2 += fl.D[2][Lf.fz(2 * i + a, 2 * j + b, 2 * k)];
                     lv.D[2][L.fz(i, j, k)] = wf * s2;
                  }
      }
      (void)w;
   }
   for (auto& lv : s->lev) {
      if (lv.hasC) orc_fill_ghosts(&lv.m, lv.C.data());
      if (lv.hasM) orc_fill_ghosts(&lv.m, lv.M.data());
   }
}

// FACPreconditioner::solveSystem (samrai/FACPreconditioner.cc:267-416) for a
// single level: u = 0, cycles of (e = cycle(r); u += e; r = f - A u) until
// RMS(r) <= tol or max_cycles.  mode 1: a cycle is rb_sweeps red-black
// sweeps with early exit on max residual <= rb_tol (solveCoarsestLevel
// "redblack", EllipticFACOps.cc:1356-1385, 1067-1230); mode 2: one V-cycle.
// f, u: ghosted layout of the fine level.  Returns cycles used; *res gets
// the final RMS residual.
int orc_fac_solve(void* h, const ampe_step_params_t* p, int mode,
                  const double* f, double* u, double tol, double* res)
{
   FacSolver* s = (FacSolver*)h;
   MGLevel& F = s->lev[0];
   Layout L(F.m);
   const long ng = L.cells_ghost();
   std::vector<double> sol(ng, 0.0), rr(ng, 0.0);
   // residual of u = 0 is f
   for (long c = 0; c < ng; c++) rr[c] = f[c];
   Op op = level_op(F);
   double norm = orc_rms_interior(&F.m, rr.data());
   int it = 0;
   do {
      // cycle on the error equation A e = rr
      std::copy(rr.begin(), rr.end(), F.f.begin());
      if (mode == 2 && s->lev.size() > 1) {
         vcycle(*s, 0, *p);
      } else {
         std::fill(F.u.begin(), F.u.end(), 0.0);
         int not_conv = 1;
         for (int sw = 0; sw < p->rb_sweeps && not_conv; sw++) {
            double rm, bm;
            rb_sweep(F, &rm, &bm);
            if (p->rb_tol >= 0.0) not_conv = std::max(rm, bm) > p->rb_tol;
         }
      }
      for (long c = 0; c < ng; c++) sol[c] += F.u[c];
      orc_fill_ghosts(&F.m, sol.data());
      // rr = f - A sol
      std::vector<double> fcopy(f, f + ng);
      orc_efo_residual(&F.m, op.D[0], op.D[1], op.D[2], op.Dc, op.C, op.Cc,
                       op.M, op.Mc, fcopy.data(), sol.data(), rr.data());
      norm = orc_rms_interior(&F.m, rr.data());
      it++;
   } while (norm > tol && it < p->fac_max_cycles);
   std::copy(sol.begin(), sol.end(), u);
   if (res) *res = norm;
   return it;
}

}  // extern "C"
