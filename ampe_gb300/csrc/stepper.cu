// Device-resident implicit stepper: fixed-step BDF(<=2), Newton with
// CVODE's convergence (crate, dcon) and divergence tests, left-
// preconditioned scaled GMRES (modified Gram-Schmidt, no restarts) with
// finite-difference Jacobian-vector products, and the block-diagonal
// phase / composition FAC preconditioner (single-level red-black sweeps or
// a within-level multigrid V-cycle).
//
// Roles replaced: QuatIntegrator::evaluateRHSFunction (QuatIntegrator.cc:
// 3134-3295), CVSpgmrPrecondSet (:3300-3375), CVSpgmrPrecondSolve
// (:3666-3769) with PhasePrecondSolve / ConcentrationPrecondSolve
// (:3391-3560), FACPreconditioner::solveSystem (samrai/
// FACPreconditioner.cc:267-416) and the CVODE BDF/SPGMR driver
// (samrai/CVODESolver.cc:112-258).
//
// All state lives in HBM; the host only runs the scalar control flow
// (Newton/GMRES bookkeeping, Givens rotations) and reads back one reduced
// scalar at a time.  Every device buffer is allocated in
// ampe_stepper_create; ampe_stepper_advance allocates nothing.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <new>
#include <vector>

#include "common.cuh"
#include "devvec.cuh"
#include "fac.cuh"
#include "fused.cuh"
#include "mixed.cuh"
#include "mlp.cuh"
#include "quat.cuh"

namespace ampe {

// ---------------------------------------------------------------------------
// templated ghost fill / transfers for the preconditioner's arithmetic type
// ---------------------------------------------------------------------------
// dst(ghosted, with ghost images) = src + sig * v   (v may be null)
template <class R>
__global__ void k_to_ghosted(Grid g, const double* src, const double* v,
                             double sig, R* dst)
{
   for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
        t < g.cells(); t += (long long)gridDim.x * blockDim.x) {
      int i, j, k;
      g.ijk(t, i, j, k);
      const R x = cvt<R, double>(v ? src[t] + sig * v[t] : src[t]);
      dst[g.c(i, j, k)] = x;
      for_each_image(g, i, j, k, [&](long long idx) { dst[idx] = x; });
   }
}

template <class R>
int to_ghosted(const Grid& g, const double* src, const double* v, double sig,
               R* dst, cudaStream_t s)
{
   k_to_ghosted<R><<<map_blocks(g.cells()), 256, 0, s>>>(g, src, v, sig, dst);
   return launch_status();
}

template <class R, class D>
__global__ void k_from_ghosted(Grid g, const R* src, D* dst)
{
   for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
        t < g.cells(); t += (long long)gridDim.x * blockDim.x) {
      int i, j, k;
      g.ijk(t, i, j, k);
      dst[t] = cvt<D, R>(src[g.c(i, j, k)]);
   }
}

// cell-average restriction of interior values (2^d children)
template <class R>
__global__ void k_restrict(Grid gf, Grid gc, const R* src, R* dst)
{
   const int dz = gf.dim == 3 ? 2 : 1;
   const R w = gf.dim == 3 ? R(0.125) : R(0.25);
   for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
        t < gc.cells(); t += (long long)gridDim.x * blockDim.x) {
      int i, j, k;
      gc.ijk(t, i, j, k);
      R s = R(0);
      for (int c = 0; c < dz; c++)
         for (int b = 0; b < 2; b++)
            for (int a = 0; a < 2; a++)
               s += src[gf.c(2 * i + a, 2 * j + b, dz * k + c)];
      dst[gc.c(i, j, k)] = w * s;
   }
}

// fine u += coarse u (piecewise constant), written through to the fine
// level's periodic ghost images
template <class R>
__global__ void k_prolong_add(Grid gf, Grid gc, const R* cu, R* fu)
{
   const int dz = gf.dim == 3 ? 2 : 1;
   for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
        t < gf.cells(); t += (long long)gridDim.x * blockDim.x) {
      int i, j, k;
      gf.ijk(t, i, j, k);
      const long long c = gf.c(i, j, k);
      const R v = fu[c] + cu[gc.c(i / 2, j / 2, k / dz)];
      fu[c] = v;
      for_each_image(gf, i, j, k, [&](long long idx) { fu[idx] = v; });
   }
}

// coarse face D = mean of the fine faces lying on it
template <class R>
__global__ void k_coarsen_faces(Grid gf, Grid gc, int dir, const R* src,
                                R* dst)
{
   const int dz = gf.dim == 3 ? 2 : 1;
   const R w = gf.dim == 3 ? R(0.25) : R(0.5);
   const int ni = gc.n0 + (dir == 0), nj = gc.n1 + (dir == 1),
             nk = gc.n2 + (dir == 2);
   const long long tot = (long long)ni * nj * nk;
   for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
        t < tot; t += (long long)gridDim.x * blockDim.x) {
      int i, j, k;
      gc.split(t, dir == 0 ? gc.fd0p : gc.fd0, dir == 1 ? gc.fd1p : gc.fd1, i, j, k);
      R s = R(0);
      if (dir == 0) {
         for (int c = 0; c < dz; c++)
            for (int b = 0; b < 2; b++) s += src[gf.fx(2 * i, 2 * j + b, dz * k + c)];
         dst[gc.fx(i, j, k)] = w * s;
      } else if (dir == 1) {
         for (int c = 0; c < dz; c++)
            for (int a = 0; a < 2; a++) s += src[gf.fy(2 * i + a, 2 * j, dz * k + c)];
         dst[gc.fy(i, j, k)] = w * s;
      } else {
         for (int b = 0; b < 2; b++)
            for (int a = 0; a < 2; a++) s += src[gf.fz(2 * i + a, 2 * j + b, 2 * k)];
         dst[gc.fz(i, j, k)] = w * s;
      }
   }
}

// composition preconditioner faces: D = -gamma (D_L + D_S) at the faces
// (EBSCompositionRHSStrategy::setDiffusionCoeffForPreconditioner,
// EBSCompositionRHSStrategy.cc:330-420, then ConcFACOps.cc:28-60)
template <class R, bool MOB>
__global__ void k_conc_precond_faces(ampe_model_t m, Grid g, const double* phi,
                                     const double* cld, const double* csd,
                                     const double* tfield, double gamma,
                                     R* D0, R* D1, R* D2)
{
   const double qlR = m.Q_liquid / kGasR, qsR = m.Q_solid / kGasR;
   const bool tdep = m.Q_liquid != 0.0 || m.Q_solid != 0.0;
   const long long nz = g.dim == 3 ? g.nfz() : 0;
   for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
        t < g.nfx() + g.nfy() + nz; t += (long long)gridDim.x * blockDim.x) {
      int dir, i, j, k;
      face_of(g, t, dir, i, j, k);
      const int ei = dir == 0, ej = dir == 1, ek = dir == 2;
      const double vphi = average_func(phi[g.c(i - ei, j - ej, k - ek)],
                                       phi[g.c(i, j, k)], m.avg_type);
      // the "kks" composition form's D0 uses the energy interpolation
      const double hphi = interp_func(
          vphi, m.conc_form == AMPE_CONC_KKS ? m.energy_interp : m.diff_interp);
      double dlq = m.D_liquid, dsq = m.D_solid;  // exp(0) = 1 exactly
      if (MOB) {
         const long long up = g.c(i, j, k), lo = g.c(i - ei, j - ej, k - ek);
         const double T = 0.5 * (temperature_at(m, g, tfield, i, j, k) +
                                 temperature_at(m, g, tfield, i - ei, j - ej, k - ek));
         dlq = phase_diffusion(m, m.mobility, 0, 0.5 * (cld[up] + cld[lo]), T);
         dsq = phase_diffusion(m, m.mobility, 1, 0.5 * (csd[up] + csd[lo]), T);
      } else if (tdep) {
         const double invT = 2.0 / (temperature_at(m, g, tfield, i - ei, j - ej, k - ek) +
                                    temperature_at(m, g, tfield, i, j, k));
         dlq = m.D_liquid * exp(-qlR * invT);
         dsq = m.D_solid * exp(-qsR * invT);
      }
      const double v = -gamma * ((1.0 - hphi) * dlq + hphi * dsq);
      if (dir == 0) D0[g.fx(i, j, k)] = (R)v;
      if (dir == 1) D1[g.fy(i, j, k)] = (R)v;
      if (dir == 2) D2[g.fz(i, j, k)] = (R)v;
   }
}

// ---------------------------------------------------------------------------
// FAC / multigrid on the device
// ---------------------------------------------------------------------------
template <class R>
struct DevLevel {
   Grid g;
   double dx[3];
   R *u = nullptr, *f = nullptr, *r = nullptr, *C = nullptr, *M = nullptr;
   // single-pass z-marching sweep (3D levels that qualify): u -> u2, then
   // the two pointers swap
   bool zsweep = false;
   ZShape zs;
   R* u2 = nullptr;
   R* D[3] = {nullptr, nullptr, nullptr};
   bool hasC = false, hasD = false, hasM = false;
   R cc = 0, dc = 0, mc = 0;
   FacOp<R> op() const
   {
      FacOp<R> o;
      if (hasD) {
         o.D0 = D[0];
         o.D1 = D[1];
         o.D2 = D[2];
      }
      o.dc = dc;
      o.C = hasC ? C : nullptr;
      o.cc = cc;
      o.M = hasM ? M : nullptr;
      o.mc = mc;
      for (int d = 0; d < 3; d++) o.dxi[d] = d < g.dim ? R(1.0 / dx[d]) : R(0);
      o.f_interior = true;  // right-hand sides: interior arrays
      return o;
   }
};

template <class R>
struct DevFac {
   std::vector<DevLevel<R>> lev;
   R *sol = nullptr, *rr = nullptr;
   double* maxres = nullptr;  // device [2]: red, black
};

template <class R>
static void* dalloc(std::vector<void*>& pool, long long n, int* err)
{
   void* p = nullptr;
   if (n < 1) n = 1;
   if (cudaMalloc(&p, sizeof(R) * (size_t)n) != cudaSuccess) {
      *err = AMPE_ERR_CUDA;
      return nullptr;
   }
   cudaMemset(p, 0, sizeof(R) * (size_t)n);
   pool.push_back(p);
   return p;
}

template <class R>
int fac_create(DevFac<R>& F, const ampe_model_t& m, int nlevels, bool hasD,
               bool hasC, std::vector<void*>& pool, bool hasM = false)
{
   int err = AMPE_OK;
   ampe_model_t mm = m;
   for (int l = 0; l < nlevels; l++) {
      DevLevel<R> L;
      L.g = make_grid(mm);
      for (int d = 0; d < 3; d++) L.dx[d] = mm.dx[d];
      const long long ng = L.g.cells_ghost();
      L.u = (R*)dalloc<R>(pool, ng, &err);
      L.zsweep = sweep_z_ok<R>(L.g, &L.zs);
      if (L.zsweep) L.u2 = (R*)dalloc<R>(pool, ng, &err);
      L.f = (R*)dalloc<R>(pool, ng, &err);
      L.r = (R*)dalloc<R>(pool, ng, &err);
      L.hasC = hasC;
      L.hasD = hasD;
      if (hasC) L.C = (R*)dalloc<R>(pool, ng, &err);
      L.hasM = hasM;
      if (hasM) L.M = (R*)dalloc<R>(pool, ng, &err);
      if (hasD) {
         L.D[0] = (R*)dalloc<R>(pool, L.g.nfx(), &err);
         L.D[1] = (R*)dalloc<R>(pool, L.g.nfy(), &err);
         if (L.g.dim == 3) L.D[2] = (R*)dalloc<R>(pool, L.g.nfz(), &err);
      }
      F.lev.push_back(L);
      if (mm.n[0] % 2 || mm.n[1] % 2 || (mm.dim == 3 && mm.n[2] % 2)) break;
      if (mm.n[0] / 2 < 2 * mm.ng || mm.n[1] / 2 < 2 * mm.ng ||
          (mm.dim == 3 && mm.n[2] / 2 < 2 * mm.ng))
         break;
      mm.n[0] /= 2;
      mm.n[1] /= 2;
      if (mm.dim == 3) mm.n[2] /= 2;
      for (int d = 0; d < 3; d++) mm.dx[d] *= 2.0;
   }
   const long long ng0 = F.lev[0].g.cells_ghost();
   F.sol = (R*)dalloc<R>(pool, ng0, &err);
   F.rr = (R*)dalloc<R>(pool, ng0, &err);
   F.maxres = (double*)dalloc<double>(pool, 2, &err);
   return err;
}

// after level 0's C / D are set: build the coarse operators
template <class R>
void fac_coarsen_operator(DevFac<R>& F, cudaStream_t s)
{
   for (size_t l = 1; l < F.lev.size(); l++) {
      DevLevel<R>& c = F.lev[l];
      const DevLevel<R>& f = F.lev[l - 1];
      c.cc = f.cc;
      c.dc = f.dc;
      c.mc = f.mc;
      if (c.hasC) {
         k_restrict<R><<<map_blocks(c.g.cells()), 256, 0, s>>>(f.g, c.g, f.C, c.C);
         launch_status();
         fill_ghosts_t(c.g, c.C, s);
      }
      if (c.hasM) {
         k_restrict<R><<<map_blocks(c.g.cells()), 256, 0, s>>>(f.g, c.g, f.M, c.M);
         launch_status();
         fill_ghosts_t(c.g, c.M, s);
      }
      if (c.hasD)
         for (int d = 0; d < c.g.dim; d++) {
            const long long nf = d == 0 ? c.g.nfx() : (d == 1 ? c.g.nfy() : c.g.nfz());
            k_coarsen_faces<R><<<map_blocks(nf), 256, 0, s>>>(f.g, c.g, d, f.D[d], c.D[d]);
            launch_status();
         }
   }
}

struct Ctx {
   cudaStream_t s;
   Reducer* red;
   const ampe_step_params_t* p;
   ampe_step_stats_t* st;
   // optional timing hook around the finest level's smoother sweeps
   void (*mark)(void* owner, bool begin) = nullptr;
   void* owner = nullptr;
};

template <class R>
double rms_interior(Ctx& cx, const Grid& g, const R* v)
{
   const double ss = cx.red->sum(g.cells(), [=] __device__(long long t) {
      int i, j, k;
      g.ijk(t, i, j, k);
      const double x = (double)v[g.c(i, j, k)];
      return x * x;
   });
   return sqrt(ss / (double)g.cells());
}

// red then black.  first: the sweep starts from u = 0.  Levels that take
// the single-pass z-marching sweep run it (u -> u2, pointers swapped) unless
// the residual maxima are wanted; otherwise two colour launches in place,
// each writing through to the ghost images (the one-launch box sweep
// k_rb_sweep is reachable only through the leaf entry ampe_efo_rbgs_sweep).
template <class R>
void rb_sweep(Ctx& cx, DevLevel<R>& L, double* maxres, bool first = false)
{
   FacOp<R> op = L.op();
   if (L.zsweep && !maxres) {
      sweep_z(op, L.g, L.zs, L.f, first ? nullptr : L.u, L.u2, nullptr, (const R*)nullptr, cx.s);
      std::swap(L.u, L.u2);
      return;
   }
   if (first) cudaMemsetAsync(L.u, 0, sizeof(R) * L.g.cells_ghost(), cx.s);
   if (maxres) cudaMemsetAsync(maxres, 0, 2 * sizeof(double), cx.s);
   rbgs_color(op, L.g, L.f, L.u, 0, maxres, cx.s, true);
   rbgs_color(op, L.g, L.f, L.u, 1, maxres ? maxres + 1 : nullptr, cx.s, true);
}

template <class R>
void vcycle(Ctx& cx, DevFac<R>& F, int l)
{
   DevLevel<R>& L = F.lev[l];
   const long long ng = L.g.cells_ghost();
   if (l == (int)F.lev.size() - 1) {
      if (cx.p->mg_coarse_sweeps < 1) cudaMemsetAsync(L.u, 0, sizeof(R) * ng, cx.s);
      for (int it = 0; it < cx.p->mg_coarse_sweeps; it++) rb_sweep(cx, L, nullptr, it == 0);
      return;
   }
   if (cx.p->mg_pre < 1) cudaMemsetAsync(L.u, 0, sizeof(R) * ng, cx.s);
   if (l == 0 && cx.mark) cx.mark(cx.owner, true);
   for (int it = 0; it < cx.p->mg_pre; it++) rb_sweep(cx, L, nullptr, it == 0);
   if (l == 0 && cx.mark) cx.mark(cx.owner, false);
   DevLevel<R>& C = F.lev[l + 1];
   residual_restrict(L.op(), L.g, C.g, L.f, L.u, C.f, cx.s);
   vcycle(cx, F, l + 1);
   if (l == 0 && cx.mark) cx.mark(cx.owner, true);
   int it = 0;
   if (cx.p->mg_post > 0 && L.zsweep) {
      // prolongation fused into the first post-sweep (u + P e staged)
      sweep_z(L.op(), L.g, L.zs, L.f, L.u, L.u2, &C.g, C.u, cx.s);
      std::swap(L.u, L.u2);
      it = 1;
   } else if (cx.p->mg_post > 0) {
      // prolongation fused into the first post-sweep's two colours
      const FacOp<R> op = L.op();
      if (rbgs_color_prolong(op, L.g, L.f, L.u, 0, C.g, C.u, cx.s) == AMPE_OK) {
         rbgs_color_prolong(op, L.g, L.f, L.u, 1, C.g, C.u, cx.s);
         it = 1;
      }
   }
   if (it == 0) {
      k_prolong_add<R><<<map_blocks(L.g.cells()), 256, 0, cx.s>>>(L.g, C.g, C.u, L.u);
      launch_status();
   }
   for (; it < cx.p->mg_post; it++) rb_sweep(cx, L, nullptr);
   if (l == 0 && cx.mark) cx.mark(cx.owner, false);
}

// FACPreconditioner::solveSystem on one level.  r: interior block of the
// Krylov vector; z: interior output (FP64 path: double, mixed path: float).
template <class R>
int fac_solve(Ctx& cx, DevFac<R>& F, int mode, const R* r, R* z, double tol)
{
   DevLevel<R>& L0 = F.lev[0];
   const Grid g = L0.g;
   const long long ng = g.cells_ghost();
   FacOp<R> op = L0.op();
   R* const f_own = L0.f;
   double norm = 0.0;
   int it = 0;
   do {
      // cycle 0 solves with the right-hand side r itself (interior layout,
      // zero initial guess) and its result becomes sol; later cycles correct
      // sol with u from the residual rr.  Level 0's f is only read.
      L0.f = it == 0 ? const_cast<R*>(r) : F.rr;
      if (mode == 2 && F.lev.size() > 1) {
         vcycle(cx, F, 0);
      } else {
         if (cx.p->rb_sweeps < 1) cudaMemsetAsync(L0.u, 0, sizeof(R) * ng, cx.s);
         int not_conv = 1;
         for (int sw = 0; sw < cx.p->rb_sweeps && not_conv; sw++) {
            const bool early = cx.p->rb_tol >= 0.0;
            rb_sweep(cx, L0, early ? F.maxres : nullptr, sw == 0);
            if (early) {
               double h[2];
               cudaMemcpyAsync(h, F.maxres, 2 * sizeof(double),
                               cudaMemcpyDeviceToHost, cx.s);
               cudaStreamSynchronize(cx.s);
               not_conv = std::max(h[0], h[1]) > cx.p->rb_tol;
            }
         }
      }
      if (it == 0) {
         std::swap(F.sol, L0.u);  // the cycle's result buffer becomes sol
      } else {  // ghosts included: u's ghosts are current
         R* sol = F.sol;
         const R* u = L0.u;
         map(ng, [=] __device__(long long t) { sol[t] += u[t]; }, cx.s);
      }
      // the norm of r - A sol, and sol's interior into z; the residual
      // itself is stored only when another cycle needs it (most solves end
      // after one cycle)
      int nblk = 0;
      residual_partial(op, g, r, F.sol, (R*)nullptr, cx.red->part, &nblk, z, cx.s);
      k_finish<<<1, 1024, 0, cx.s>>>(cx.red->part, nblk, cx.red->dres, 0);
      g_launches++;
      norm = sqrt(cx.red->fetch(1)[0] / (double)g.cells());
      it++;
      if (norm > tol && it < cx.p->fac_max_cycles)
         residual_partial(op, g, r, F.sol, F.rr, cx.red->part, &nblk, (R*)nullptr, cx.s);
   } while (norm > tol && it < cx.p->fac_max_cycles);
   L0.f = f_own;
   cx.st->fac_cycles += it;
   return it;
}

// ---------------------------------------------------------------------------
// the stepper
// ---------------------------------------------------------------------------
struct Stepper {
   ampe_model_t m;
   ampe_step_params_t p;
   Grid g;
   long long N = 0, NG = 0, NY = 0;
   int nb = 2;  // scalar fields in y: phi, c (+ q0..q3 when evolve_quat)
   cudaStream_t s = nullptr;      // the stream every launch and copy goes to
   cudaStream_t own_s = nullptr;  // the stepper's private stream
   Reducer red;
   std::vector<void*> pool;
   // ghosted FP64 scratch
   double *phi_g, *c_g, *cl, *cs, *clr, *csr, *cl_nf, *cs_nf, *phi_lag, *tfield;
   double* dF;                 // interior driving force
   ThermoCoef* tab = nullptr;  // per-x (or single) thermodynamic table
   CoefF* tabf = nullptr;      // its FP32 copy (mixed path)
   float2* dqtab = nullptr;    // (D_L, D_S) per x index (mixed path, analytic T)
   MixParams mp;               // FP32 constants of the mixed kernels
   unsigned long long* counters;
   // 2N interior vectors
   double *yn, *ynm1, *ynew, *a, *y, *fy, *b, *d, *w, *wi, *tmp, *av, *fp;
   double *ysave, *ym1save;  // y_n, y_{n-1} at the start of a step being retried
   std::vector<double*> V;
   // mixed path Krylov vectors (FP32) and FP32 copies of the WRMS weights
   std::vector<float*> Vf;
   float *tmpf = nullptr, *avf = nullptr, *bf = nullptr, *w32 = nullptr, *wi32 = nullptr;
   // mixed path (FP32 working copies)
   float *cl32 = nullptr, *cs32 = nullptr, *clr32 = nullptr, *csr32 = nullptr;
   float *dF32 = nullptr, *pf32 = nullptr, *dphi32 = nullptr, *da32 = nullptr,
         *db32 = nullptr, *dc32 = nullptr;
   float *guess_l = nullptr, *guess_s = nullptr;  // surrogate initial guess
   // no converged phase concentrations to warm-start from yet (set_state
   // without cl / cs, until the first accepted step): the surrogate's guess
   // is used only then, since a converged warm start from the previous step
   // needs fewer Newton iterations than the network's guess
   bool cold = true;
   Mlp* mlp = nullptr;                            // attached surrogate
   unsigned long long* mcount = nullptr;          // mixed KKS counters [5]
   int* kks_list = nullptr;  // cells for the FP64 polish (N + 1 ints, mixed path)
   // quaternion fields: ghosted q (4 NG) and its lagged copy, the cell
   // modulus |grad q| of the lagged copy, M_q(phi), face coefficients
   double *q_g = nullptr, *q_lag = nullptr, *ogm = nullptr, *mq = nullptr;
   double* fcq[3] = {nullptr, nullptr, nullptr};
   QuatF32 qf32;  // FP32 quaternion working set (mixed path)
   // orientation of the anisotropic phase flux: qlen ghosted FP64 components
   // (static; evolve_quat models use the evolving q instead)
   double* qorient = nullptr;
   AnisoF an;  // FP32 anisotropic face fluxes and Jacobians (2D mixed path)
   FaceW fw;   // FP32 composition flux weights per face (mixed path)
   // preconditioner (FP64 or FP32)
   DevFac<double> facp64, facc64, facq64;
   DevFac<float> facp32, facc32, facq32;
   int hist = 0;
   // variable-step BDF (params adaptive = 1): y_{n-2}, f(y_n) for the
   // explicit-Euler predictor of a first step, the sizes of the last two
   // accepted steps, the next step's size and order, the accepted steps
   // before an order change is considered, the growth cap of the next step
   // size, how many back values (y_{n-1}, y_{n-2}) are valid
   double *ynm2 = nullptr, *fn = nullptr;
   double h_next = 0.0, h1 = 0.0, h2 = 0.0, eta_max = 1.0e4;
   int q_next = 1, qwait = 2, nhist = 0;
   bool fn_valid = false;
   double T_start = 0.0;  // T0 at t = 0 of a model with dTdt != 0
   double t = 0.0;
   ampe_step_stats_t st;
   // optional per-kernel CUDA-event timing on the stepper's stream
   bool prof = false;
   std::vector<cudaEvent_t> ev_pool;
   size_t ev_next = 0;
   std::vector<std::pair<int, std::pair<cudaEvent_t, cudaEvent_t>>> pending;
   double kms[8] = {0, 0, 0, 0, 0, 0, 0, 0};
   long long kcount[8] = {0, 0, 0, 0, 0, 0, 0, 0};

   cudaEvent_t smooth_a = nullptr;  // open KT_SMOOTH interval
   Ctx ctx();
};

constexpr int kMaxKrylov = 16;  // Krylov dimension limit of the stepper

// coefficients and basis vectors of the GMRES update, passed by value
struct KrylovComb {
   const double* v[kMaxKrylov];
   double c[kMaxKrylov];
};
struct KrylovCombF {
   const float* v[kMaxKrylov];
   float c[kMaxKrylov];
};

// kernel classes timed in profiling mode
enum {
   KT_KKS = 0,
   KT_RHS = 1,
   KT_JV = 2,
   KT_MLP = 3,
   KT_QUAT = 4,
   KT_PREC = 5,    // whole preconditioner solve (all blocks)
   KT_PSET = 6,    // preconditioner setup
   KT_SMOOTH = 7,  // red-black sweeps on the finest multigrid level
   KT_NKINDS = 8
};

static cudaEvent_t prof_event(Stepper& S)
{
   if (S.ev_next >= S.ev_pool.size()) return nullptr;
   return S.ev_pool[S.ev_next++];
}

struct ProfScope {
   Stepper& S;
   int kind;
   cudaEvent_t a = nullptr, b = nullptr;
   ProfScope(Stepper& s_, int k) : S(s_), kind(k)
   {
      if (!S.prof) return;
      a = prof_event(S);
      b = prof_event(S);
      if (a && b) cudaEventRecord(a, S.s);
   }
   ~ProfScope()
   {
      if (a && b) {
         cudaEventRecord(b, S.s);
         S.pending.push_back({kind, {a, b}});
      }
   }
};

// Ctx hook: time the finest level's sweeps (KT_SMOOTH) in profiling mode
static void smooth_mark(void* owner, bool begin)
{
   Stepper& S = *(Stepper*)owner;
   if (!S.prof) return;
   if (begin) {
      S.smooth_a = prof_event(S);
      if (S.smooth_a) cudaEventRecord(S.smooth_a, S.s);
      return;
   }
   cudaEvent_t b = S.smooth_a ? prof_event(S) : nullptr;
   if (b) {
      cudaEventRecord(b, S.s);
      S.pending.push_back({KT_SMOOTH, {S.smooth_a, b}});
   }
   S.smooth_a = nullptr;
}

Ctx Stepper::ctx()
{
   Ctx c{s, &red, &p, &st};
   c.mark = smooth_mark;
   c.owner = this;
   return c;
}

// fold finished event pairs into the totals (stream must be idle)
static void prof_collect(Stepper& S)
{
   for (auto& e : S.pending) {
      float ms = 0.f;
      if (cudaEventElapsedTime(&ms, e.second.first, e.second.second) == cudaSuccess) {
         S.kms[e.first] += ms;
         S.kcount[e.first]++;
      }
   }
   S.pending.clear();
   S.ev_next = 0;
}

static double* dvec(Stepper& S, long long n, int* err)
{
   return (double*)dalloc<double>(S.pool, n, err);
}

static void eval_rhs(Stepper& S, const double* y, const double* v, double sig,
                     double* out, int fd_flag)
{
   to_ghosted<double>(S.g, y, v, sig, S.phi_g, S.s);
   to_ghosted<double>(S.g, y + S.N, v ? v + S.N : nullptr, sig, S.c_g, S.s);
   const double* tf = S.m.temp_mode == AMPE_TEMP_FIELD ? S.tfield : nullptr;
   const bool quat = S.nb == 6;
   if (quat && S.p.precision == 1) {
      for (int c = 0; c < 4; c++)
         to_ghosted<float>(S.g, y + (2 + c) * S.N, v ? v + (2 + c) * S.N : nullptr, sig,
                           S.qf32.q + c * S.NG, S.s);
      ProfScope ps(S, KT_QUAT);
      quat_cells_f32(S.m, S.mp, S.g, S.phi_g, S.qf32, S.s);
   } else if (quat) {
      for (int c = 0; c < 4; c++)
         to_ghosted<double>(S.g, y + (2 + c) * S.N, v ? v + (2 + c) * S.N : nullptr,
                            sig, S.q_g + c * S.NG, S.s);
      // QuatIntegrator::computeQuatGradients; the finite-difference calls
      // keep the gradients of the last f(y) (QuatIntegrator.cc:3189)
      if (!fd_flag) {
         cudaMemcpyAsync(S.q_lag, S.q_g, sizeof(double) * 4 * (size_t)S.NG,
                         cudaMemcpyDeviceToDevice, S.s);
         quat_grad_modulus<double>(S.m, S.g, S.q_lag, S.ogm, S.s);
      }
   }
   if (S.p.precision == 1) {
      // surrogate = 1: the network's guess while no converged warm start
      // exists (a cold start); 2: for every KKS solve (the warm start is
      // then only the fallback)
      const bool sur = S.p.surrogate && S.mlp && (S.cold || S.p.surrogate == 2);
      if (sur) {
         ProfScope ps(S, KT_MLP);
         S.mlp->infer(S.g, S.phi_g, S.c_g, tf, S.guess_l, S.guess_s, true, S.s);
      }
      {
         ProfScope ps(S, KT_KKS);
         kks_mixed(S.m, S.mp, S.g, S.tab, S.tabf, tf, S.phi_g, S.c_g,
                   sur ? S.guess_l : nullptr, sur ? S.guess_s : nullptr, S.clr32, S.csr32,
                   S.cl32, S.cs32, S.dF32, S.kks_list, S.mcount, S.s);
      }
      {
         ProfScope ps(S, KT_RHS);
         rhs_mixed(S.m, S.mp, S.g, tf, S.phi_g, S.pf32, S.cl32, S.cs32, S.dF32,
                   quat && S.m.with_orient ? S.qf32.ogm : nullptr, S.qorient, &S.an, S.c_g,
                   S.fw, out, out + S.N, S.s);
      }
      if (quat) {
         ProfScope ps(S, KT_QUAT);
         quat_faces_f32(S.m, S.mp, S.g, tf, S.pf32, S.qf32.q, 1.0, S.qf32.fc, S.qf32.dfc,
                        S.s);
         quat_rhs<float>(S.m, S.g, S.qf32.fc[0], S.qf32.fc[1], S.qf32.fc[2], S.qf32.mq,
                         S.qf32.q, out + 2 * S.N, S.s);
      }
      S.st.rhs_evals++;
      return;
   }
   {
      ProfScope ps(S, KT_KKS);
      kks_interior(S.m, S.g, S.tab, tf, S.phi_g, S.c_g, S.clr, S.csr, S.cl,
                   S.cs, S.dF, S.counters, S.s);
   }
   if (!fd_flag) {
      const size_t bytes = sizeof(double) * (size_t)S.NG;
      cudaMemcpyAsync(S.phi_lag, S.phi_g, bytes, cudaMemcpyDeviceToDevice, S.s);
      cudaMemcpyAsync(S.cl_nf, S.cl, bytes, cudaMemcpyDeviceToDevice, S.s);
      cudaMemcpyAsync(S.cs_nf, S.cs, bytes, cudaMemcpyDeviceToDevice, S.s);
   }
   {
      ProfScope ps(S, KT_RHS);
      const double* qflux = nullptr;
      if (S.m.flux_type == AMPE_FLUX_ANISOTROPIC) qflux = quat ? S.q_g : S.qorient;
      rhs_fused(S.m, S.g, S.phi_g, qflux, tf, S.tab, S.cl, S.cs, S.dF,
                S.phi_lag, quat && S.m.with_orient ? S.ogm : nullptr, S.c_g, S.cl_nf,
                S.cs_nf, out, out + S.N, S.s);
   }
   if (quat) {
      ProfScope ps(S, KT_QUAT);
      quat_mobility<double>(S.m, S.g, S.phi_g, S.mq, S.s);
      quat_face_coef(S.m, S.g, S.phi_g, tf, S.q_lag, 1.0, S.fcq[0], S.fcq[1],
                             S.fcq[2], S.s);
      quat_rhs<double>(S.m, S.g, S.fcq[0], S.fcq[1], S.fcq[2], S.mq, S.q_g,
                       out + 2 * S.N, S.s);
   }
   S.st.rhs_evals++;
}

static double wrms(Stepper& S, const double* v, const double* w)
{
   const long long ny = S.NY;
   const double ss = S.red.sum(ny, [=] __device__(long long t) {
      const double x = v[t] * w[t];
      return x * x;
   });
   return sqrt(ss / (double)ny);
}

static double dot(Stepper& S, const double* a, const double* b)
{
   return S.red.sum(S.NY, [=] __device__(long long t) { return a[t] * b[t]; });
}

// composition block faces D = -gamma (D_L + D_S): FP64 at the lagged phi, or
// FP32 from the FP32 phi copy of the last f(y) (mixed path)
static void conc_precond_faces(Stepper& S, const double* tf, double gamma,
                               DevLevel<double>& C0)
{
   const long long nf = S.g.nfx() + S.g.nfy() + (S.g.dim == 3 ? S.g.nfz() : 0);
   if (S.m.conc_diffusion == AMPE_DIFF_MOBILITY)
      k_conc_precond_faces<double, true><<<map_blocks(nf), 256, 0, S.s>>>(
          S.m, S.g, S.phi_lag, S.cl_nf, S.cs_nf, tf, gamma, C0.D[0], C0.D[1], C0.D[2]);
   else
      k_conc_precond_faces<double, false><<<map_blocks(nf), 256, 0, S.s>>>(
          S.m, S.g, S.phi_lag, S.cl_nf, S.cs_nf, tf, gamma, C0.D[0], C0.D[1], C0.D[2]);
   launch_status();
}

static void conc_precond_faces(Stepper& S, const double* tf, double gamma,
                               DevLevel<float>& C0)
{
   (void)tf;
   conc_faces_f32(S.m, S.mp, S.g, S.fw, gamma, C0.D, S.s);
}

// D = gamma fc of the quaternion block: FP64 from the lagged q, or FP32 from
// the FP32 working copy (mixed path)
static void quat_precond_faces(Stepper& S, const double* tf, double gamma,
                               DevLevel<double>& Q0)
{
   quat_face_coef(S.m, S.g, S.phi_g, tf, S.q_lag, gamma, Q0.D[0], Q0.D[1], Q0.D[2], S.s);
}

static void quat_precond_faces(Stepper& S, const double* tf, double gamma,
                               DevLevel<float>& Q0)
{
   quat_faces_f32(S.m, S.mp, S.g, tf, S.pf32, S.qf32.q, gamma, Q0.D, nullptr, S.s);
}

template <class R>
static void precond_setup_t(Stepper& S, DevFac<R>& fp, DevFac<R>& fc,
                            DevFac<R>& fq, double gamma)
{
   const double* tf = S.m.temp_mode == AMPE_TEMP_FIELD ? S.tfield : nullptr;
   DevLevel<R>& P0 = fp.lev[0];
   phase_set_c<R>(S.m, S.g, S.phi_g, gamma, P0.C, S.s);
   fill_ghosts_t(S.g, P0.C, S.s);
   const double eps2 = S.m.epsilon_phi * S.m.epsilon_phi;
   for (auto& L : fp.lev) {
      L.dc = (R)(-gamma * eps2);
      L.cc = 0;
      L.mc = (R)S.m.phase_mobility;
   }
   fac_coarsen_operator(fp, S.s);
   conc_precond_faces(S, tf, gamma, fc.lev[0]);
   for (auto& L : fc.lev) {
      L.dc = 0;
      L.cc = (R)1.0;
      L.mc = (R)S.m.conc_mobility;
   }
   fac_coarsen_operator(fc, S.s);
   if (S.nb == 6) {
      // QuatFACOps::setOperatorCoefficients: C = 1, M = M_q(phi) per cell,
      // D = gamma fc at the faces (lagged gradients)
      DevLevel<R>& Q0 = fq.lev[0];
      quat_mobility<R>(S.m, S.g, S.phi_g, Q0.M, S.s);
      fill_ghosts_t(S.g, Q0.M, S.s);
      quat_precond_faces(S, tf, gamma, Q0);
      for (auto& L : fq.lev) {
         L.dc = 0;
         L.cc = (R)1.0;
         L.mc = 0;
      }
      fac_coarsen_operator(fq, S.s);
   }
}

static void precond_setup(Stepper& S, double gamma)
{
   ProfScope ps(S, KT_PSET);
   if (S.p.precision == 1)
      precond_setup_t(S, S.facp32, S.facc32, S.facq32, gamma);
   else
      precond_setup_t(S, S.facp64, S.facc64, S.facq64, gamma);
   S.st.precond_setups++;
}

// z = P^-1 r, one FAC solve per block (FP64 path)
static void precond_solve(Stepper& S, const double* r, double* z,
                          double delta)
{
   if (S.p.precond == 0) {
      cudaMemcpyAsync(z, r, sizeof(double) * S.NY, cudaMemcpyDeviceToDevice,
                      S.s);
      return;
   }
   ProfScope ps(S, KT_PREC);
   Ctx cx = S.ctx();
   for (int blk = 0; blk < S.nb; blk++)
      fac_solve(cx, blk == 0 ? S.facp64 : (blk == 1 ? S.facc64 : S.facq64), S.p.precond,
                r + blk * S.N, z + blk * S.N, delta);
   S.st.precond_solves++;
}

// the same with FP32 Krylov vectors and FP32 FAC blocks (mixed path)
static void precond_solve(Stepper& S, const float* r, float* z, double delta)
{
   if (S.p.precond == 0) {
      cudaMemcpyAsync(z, r, sizeof(float) * S.NY, cudaMemcpyDeviceToDevice, S.s);
      return;
   }
   ProfScope ps(S, KT_PREC);
   Ctx cx = S.ctx();
   for (int blk = 0; blk < S.nb; blk++)
      fac_solve(cx, blk == 0 ? S.facp32 : (blk == 1 ? S.facc32 : S.facq32), S.p.precond,
                r + blk * S.N, z + blk * S.N, delta);
   S.st.precond_solves++;
}

// out = v - gamma (f(y + sig v) - f(y)) / sig, sig = 1 / WRMS(v)
static void matvec(Stepper& S, const double* y, const double* fy,
                   const double* w, double gamma, const double* v,
                   double* out)
{
   const double wn = wrms(S, v, w);
   const double sig = 1.0 / wn;
   eval_rhs(S, y, v, sig, S.fp, 1);
   const double* fp = S.fp;
   map(S.NY, [=] __device__(long long t) {
      out[t] = v[t] - gamma * (fp[t] - fy[t]) * wn;
   }, S.s);
}

static int gmres(Stepper& S, const double* y, const double* fy,
                 const double* w, double gamma, const double* b, double* x,
                 double tol)
{
   const long long ny = S.NY;
   const int maxl = S.p.max_krylov;
   const double sqrtN = std::sqrt((double)ny);
   std::vector<double> H((maxl + 1) * maxl, 0.0), gv(maxl + 1, 0.0), cs(maxl),
       sn(maxl);
   double* tmp = S.tmp;
   double* av = S.av;
   const double* wi = S.wi;  // 1 / w
   precond_solve(S, b, tmp, tol * sqrtN);
   double* V0 = S.V[0];
   // V0 = w P^-1 b and |V0|^2 in one pass
   double beta = std::sqrt(S.red.sum(ny, [=] __device__(long long t) {
      const double xv = w[t] * tmp[t];
      V0[t] = xv;
      return xv * xv;
   }));
   if (beta / sqrtN <= tol) {
      cudaMemsetAsync(x, 0, sizeof(double) * ny, S.s);
      return 0;
   }
   {
      const double ib = 1.0 / beta;
      map(ny, [=] __device__(long long t) { V0[t] *= ib; }, S.s);
   }
   gv[0] = beta;
   int l = 0;
   for (; l < maxl; l++) {
      double* Vl = S.V[l];
      double* Vn = S.V[l + 1];
      map(ny, [=] __device__(long long t) { tmp[t] = Vl[t] * wi[t]; }, S.s);
      matvec(S, y, fy, w, gamma, tmp, av);
      precond_solve(S, av, tmp, tol * sqrtN);
      // modified Gram-Schmidt; every projection pass also forms the next
      // inner product (with V_{i+1}, or |Vn|^2 after the last one)
      double h = S.red.sum(ny, [=] __device__(long long t) {
         const double xv = w[t] * tmp[t];
         Vn[t] = xv;
         return V0[t] * xv;
      });
      double hn2 = 0.0;
      for (int i = 0; i <= l; i++) {
         H[i * maxl + l] = h;
         const double* Vi = S.V[i];
         const double hh = h;
         if (i < l) {
            const double* Vj = S.V[i + 1];
            h = S.red.sum(ny, [=] __device__(long long t) {
               const double xv = Vn[t] - hh * Vi[t];
               Vn[t] = xv;
               return Vj[t] * xv;
            });
         } else {
            hn2 = S.red.sum(ny, [=] __device__(long long t) {
               const double xv = Vn[t] - hh * Vi[t];
               Vn[t] = xv;
               return xv * xv;
            });
         }
      }
      const double hn = std::sqrt(hn2);
      H[(l + 1) * maxl + l] = hn;
      if (hn > 0.0) {
         const double ih = 1.0 / hn;
         map(ny, [=] __device__(long long t) { Vn[t] *= ih; }, S.s);
      }
      for (int i = 0; i < l; i++) {
         const double aa = H[i * maxl + l], bb = H[(i + 1) * maxl + l];
         H[i * maxl + l] = cs[i] * aa + sn[i] * bb;
         H[(i + 1) * maxl + l] = -sn[i] * aa + cs[i] * bb;
      }
      const double aa = H[l * maxl + l], bb = H[(l + 1) * maxl + l];
      const double rr = std::sqrt(aa * aa + bb * bb);
      cs[l] = aa / rr;
      sn[l] = bb / rr;
      H[l * maxl + l] = rr;
      H[(l + 1) * maxl + l] = 0.0;
      gv[l + 1] = -sn[l] * gv[l];
      gv[l] = cs[l] * gv[l];
      if (std::fabs(gv[l + 1]) / sqrtN <= tol || hn == 0.0) {
         l++;
         break;
      }
   }
   const int k = std::min(l, maxl);
   std::vector<double> yk(k, 0.0);
   for (int i = k - 1; i >= 0; i--) {
      double acc = gv[i];
      for (int j = i + 1; j < k; j++) acc -= H[i * maxl + j] * yk[j];
      yk[i] = acc / H[i * maxl + i];
   }
   // x = (sum_i yk_i V_i) / w in one pass (same summation order)
   KrylovComb cb;
   for (int i = 0; i < k; i++) {
      cb.v[i] = S.V[i];
      cb.c[i] = yk[i];
   }
   map(ny, [=] __device__(long long t) {
      double acc = 0.0;
      for (int i = 0; i < k; i++) acc += cb.c[i] * cb.v[i][t];
      x[t] = acc * wi[t];
   }, S.s);
   return k;
}

// out = v - gamma J v with the analytic FP32 product at the state of the
// last f(y) (mixed path)
static void matvec32(Stepper& S, double gamma, const float* v, float* out)
{
   const double* tf = S.m.temp_mode == AMPE_TEMP_FIELD ? S.tfield : nullptr;
   ProfScope ps(S, KT_JV);
   jv_mixed(S.m, S.mp, S.g, S.tabf, tf, S.pf32, S.cl32, S.cs32, S.dF32, v, gamma, S.dphi32,
            S.da32, S.db32, S.dc32, S.nb == 6 ? &S.qf32 : nullptr, &S.an, S.fw, out, S.s);
}

// GMRES of the mixed path: the same algorithm as gmres() (left
// preconditioning, WRMS scaling, modified Gram-Schmidt) on FP32 Krylov
// vectors.  Inner products: FP32 products, compensated FP32 sums per thread,
// FP64 across threads and blocks.  b and the correction x are FP64.
static int gmres32(Stepper& S, double gamma, const float* bf, double* x,
                   double tol)
{
   const long long ny = S.NY;
   const int maxl = S.p.max_krylov;
   const double sqrtN = std::sqrt((double)ny);
   std::vector<double> H((maxl + 1) * maxl, 0.0), gv(maxl + 1, 0.0), cs(maxl),
       sn(maxl);
   float* tmp = S.tmpf;
   float* av = S.avf;
   const float* w = S.w32;
   const float* wi = S.wi32;
   precond_solve(S, bf, tmp, tol * sqrtN);
   float* V0 = S.Vf[0];
   double beta = std::sqrt(S.red.sumf(ny, [=] __device__(long long t) {
      const float xv = w[t] * tmp[t];
      V0[t] = xv;
      return xv * xv;
   }));
   if (beta / sqrtN <= tol) {
      cudaMemsetAsync(x, 0, sizeof(double) * ny, S.s);
      return 0;
   }
   {
      const float ib = (float)(1.0 / beta);
      map(ny, [=] __device__(long long t) { V0[t] *= ib; }, S.s);
   }
   gv[0] = beta;
   int l = 0;
   for (; l < maxl; l++) {
      float* Vl = S.Vf[l];
      float* Vn = S.Vf[l + 1];
      map(ny, [=] __device__(long long t) { tmp[t] = Vl[t] * wi[t]; }, S.s);
      matvec32(S, gamma, tmp, av);
      precond_solve(S, av, tmp, tol * sqrtN);
      double h = S.red.sumf(ny, [=] __device__(long long t) {
         const float xv = w[t] * tmp[t];
         Vn[t] = xv;
         return V0[t] * xv;
      });
      double hn2 = 0.0;
      for (int i = 0; i <= l; i++) {
         H[i * maxl + l] = h;
         const float* Vi = S.Vf[i];
         const float hh = (float)h;
         if (i < l) {
            const float* Vj = S.Vf[i + 1];
            h = S.red.sumf(ny, [=] __device__(long long t) {
               const float xv = Vn[t] - hh * Vi[t];
               Vn[t] = xv;
               return Vj[t] * xv;
            });
         } else {
            hn2 = S.red.sumf(ny, [=] __device__(long long t) {
               const float xv = Vn[t] - hh * Vi[t];
               Vn[t] = xv;
               return xv * xv;
            });
         }
      }
      const double hn = std::sqrt(hn2);
      H[(l + 1) * maxl + l] = hn;
      if (hn > 0.0) {
         const float ih = (float)(1.0 / hn);
         map(ny, [=] __device__(long long t) { Vn[t] *= ih; }, S.s);
      }
      for (int i = 0; i < l; i++) {
         const double aa = H[i * maxl + l], bb = H[(i + 1) * maxl + l];
         H[i * maxl + l] = cs[i] * aa + sn[i] * bb;
         H[(i + 1) * maxl + l] = -sn[i] * aa + cs[i] * bb;
      }
      const double aa = H[l * maxl + l], bb = H[(l + 1) * maxl + l];
      const double rr = std::sqrt(aa * aa + bb * bb);
      cs[l] = aa / rr;
      sn[l] = bb / rr;
      H[l * maxl + l] = rr;
      H[(l + 1) * maxl + l] = 0.0;
      gv[l + 1] = -sn[l] * gv[l];
      gv[l] = cs[l] * gv[l];
      if (std::fabs(gv[l + 1]) / sqrtN <= tol || hn == 0.0) {
         l++;
         break;
      }
   }
   const int k = std::min(l, maxl);
   std::vector<double> yk(k, 0.0);
   for (int i = k - 1; i >= 0; i--) {
      double acc = gv[i];
      for (int j = i + 1; j < k; j++) acc -= H[i * maxl + j] * yk[j];
      yk[i] = acc / H[i * maxl + i];
   }
   KrylovCombF cb;
   for (int i = 0; i < k; i++) {
      cb.v[i] = S.Vf[i];
      cb.c[i] = (float)yk[i];
   }
   map(ny, [=] __device__(long long t) {
      float acc = 0.f;
      for (int i = 0; i < k; i++) acc += cb.c[i] * cb.v[i][t];
      x[t] = f2d(acc * wi[t]);
   }, S.s);
   return k;
}

// the temperature-dependent state after a change of S.m.T0 / gradT: the
// FP32 constants, the per-x thermodynamic and diffusivity tables, the
// network's copy of the model (launches on the stepper's stream, no wait)
static int apply_temperature(Stepper& S)
{
   const float2* dq = S.mp.dq;
   S.mp = make_mix_params(S.m);
   S.mp.dq = dq;
   const int nt = S.m.temp_mode == AMPE_TEMP_GRADIENT ? S.m.n[0] : 1;
   int err = AMPE_OK;
   if (S.tab) err = build_thermo_table(S.m, S.tab, nt, S.s);
   if (!err && S.tabf) err = build_coef_f(S.tab, S.tabf, nt, S.s);
   if (!err && S.dqtab) err = build_diff_table(S.m, S.mp, S.g, S.dqtab, S.s);
   if (S.mlp) {  // the network sees the stepper's temperature field
      S.mlp->m.T0 = S.m.T0;
      S.mlp->m.gradT = S.m.gradT;
   }
   return err;
}

// QuatIntegrator::setTemperatureField before every f(t, y)
// (QuatIntegrator.cc:3191): the model's T0(t)
// (ScalarTemperatureStrategy::getCurrentTemperature,
// ScalarTemperatureStrategy.cc:57-73; GradientTemperatureStrategy.cc:
// 124-131 without a moving frame)
static void at_time(Stepper& S, double t)
{
   const ampe_model_t& m = S.m;
   if (m.dTdt == 0.0 || m.temp_mode == AMPE_TEMP_FIELD) return;
   double T = S.T_start + m.dTdt * t;
   if (m.temp_mode == AMPE_TEMP_CONSTANT) {
      if (m.dTdt < 0.0 && T < m.T_target)
         T = m.T_target;
      else if (m.T_target > 0.0 && m.dTdt > 0.0 && T > m.T_target)
         T = m.T_target;
   }
   if (T == m.T0) return;
   S.m.T0 = T;
   apply_temperature(S);
}

// Newton iteration of one BDF step: y - gamma f(y) = a from the predictor
// in S.y, convergence test del min(1, crate) <= newton_coef; result in
// S.ynew.  0 = converged.
static int bdf_newton(Stepper& S, double gamma, double newton_coef)
{
   const long long ny = S.NY;
   double *a = S.a, *y = S.y, *yn = S.yn, *w = S.w;
   double *fy = S.fy, *b = S.b, *d = S.d;
   const double rtol = S.p.rtol, atol = S.p.atol;
   double* wi = S.wi;
   if (S.p.precision == 1) {
      // FP32 weights (no FP64 division per element); the FP64 copy used by
      // the Newton test holds the same values exactly
      float *w32 = S.w32, *wi32 = S.wi32;
      const float rtf = (float)rtol, atf = (float)atol;
      map(ny, [=] __device__(long long t) {
         const float e = rtf * fabsf(d2f(yn[t])) + atf;
         const float wv = 1.f / e;
         w32[t] = wv;
         wi32[t] = e;
         w[t] = f2d(wv);
      }, S.s);
   } else {
      map(ny, [=] __device__(long long t) {
         const double e = rtol * fabs(yn[t]) + atol;
         w[t] = 1.0 / e;
         wi[t] = e;
      }, S.s);
   }
   double crate = 1.0, delp = 0.0;
   const double lintol = S.p.lin_coef * newton_coef;
   for (int it = 0; it < S.p.max_newton; it++) {
      eval_rhs(S, y, nullptr, 0.0, fy, 0);
      if (it == 0 && S.p.precond) precond_setup(S, gamma);
      const double gm = gamma;
      int li;
      if (S.p.precision == 1) {  // the Newton right-hand side straight to FP32
         float* bf = S.bf;
         map(ny, [=] __device__(long long t) { bf[t] = d2f(-(y[t] - gm * fy[t] - a[t])); },
             S.s);
         li = gmres32(S, gamma, bf, d, lintol);
      } else {
         map(ny, [=] __device__(long long t) { b[t] = -(y[t] - gm * fy[t] - a[t]); },
             S.s);
         li = gmres(S, y, fy, w, gamma, b, d, lintol);
      }
      S.st.gmres_iters += li;
      S.st.newton_iters++;
      // y += d and WRMS(d) in one pass
      const double del = std::sqrt(S.red.sum(ny, [=] __device__(long long t) {
         y[t] += d[t];
         const double xv = d[t] * w[t];
         return xv * xv;
      }) / (double)ny);
      if (it > 0) crate = std::max(0.3 * crate, del / delp);
      const double dcon = del * std::min(1.0, crate) / newton_coef;
      if (dcon <= 1.0) {
         cudaMemcpyAsync(S.ynew, y, sizeof(double) * ny,
                         cudaMemcpyDeviceToDevice, S.s);
         // QuatIntegrator::applyProjection (QuatIntegrator.cc:3911-3940)
         if (S.nb == 6) quat_project(S.N, S.ynew + 2 * S.N, S.s);
         return 0;
      }
      if (it >= 1 && del > 2.0 * delp) break;
      delp = del;
   }
   S.st.newton_fail++;
   return 1;
}

// one fixed-size BDF step of size h, order q, ending at t_end
// (constant-step coefficients, linear-extrapolation predictor); result in
// S.ynew.  0 = converged.
static int bdf_step(Stepper& S, double t_end, double h, int q)
{
   at_time(S, t_end);
   const long long ny = S.NY;
   double *a = S.a, *y = S.y, *yn = S.yn, *ynm1 = S.ynm1;
   double gamma;
   if (q == 1) {
      gamma = h;
      map(ny, [=] __device__(long long t) {
         a[t] = yn[t];
         y[t] = yn[t];
      }, S.s);
   } else {
      gamma = 2.0 * h / 3.0;
      const double third = 1.0 / 3.0;
      map(ny, [=] __device__(long long t) {
         a[t] = (4.0 * yn[t] - ynm1[t]) * third;
         y[t] = 2.0 * yn[t] - ynm1[t];
      }, S.s);
   }
   return bdf_newton(S, gamma, S.p.newton_coef);
}

static void swap_ptr(double*& a, double*& b)
{
   double* t = a;
   a = b;
   b = t;
}

// KKS warm starts of the next step: the accepted step's phase
// concentrations (QuatModel::resetRefPhaseConcentrations, QuatModel.cc:5218)
static void keep_warm_start(Stepper& S)
{
   const size_t gb = sizeof(double) * (size_t)S.NG;
   if (S.p.precision == 1) {
      const size_t gf = sizeof(float) * (size_t)S.NG;
      cudaMemcpyAsync(S.clr32, S.cl32, gf, cudaMemcpyDeviceToDevice, S.s);
      cudaMemcpyAsync(S.csr32, S.cs32, gf, cudaMemcpyDeviceToDevice, S.s);
   } else {
      cudaMemcpyAsync(S.clr, S.cl_nf, gb, cudaMemcpyDeviceToDevice, S.s);
      cudaMemcpyAsync(S.csr, S.cs_nf, gb, cudaMemcpyDeviceToDevice, S.s);
   }
}

// Variable-step BDF predictor of the next step (size h, order q, from the
// accepted history): pred = k0 y_n + k1 y_{n-1} + k2 y_{n-2} + k3 f(y_n).
// Also the error constant c of the estimate LTE ~ c (y_{n+1} - pred):
//  - no history: explicit Euler y_n + h f(y_n); the BDF1 error h^2 y''/2
//    against the predictor's h^2 y'': c = 1/2;
//  - order 1: linear extrapolation through y_n, y_{n-1}, ratio
//    w = h / h_{n-1}: c = w / (2w + 1) (1/3 at constant steps);
//  - order 2: quadratic extrapolation through y_n, y_{n-1}, y_{n-2}; the
//    variable-coefficient BDF2 error A y3/6 with A = h^3 (1+w)^2 /
//    (w (1+2w)) against the predictor's P y3/6 with P = h (h+h1)(h+h1+h2)
//    (y3 the third derivative): c = A / (P + A) (2/11 at constant steps).
struct Pred {
   double k0, k1, k2, k3, c;
};
static Pred predictor(const Stepper& S, double h, int q)
{
   Pred P{1.0, 0.0, 0.0, 0.0, 0.5};
   if (S.nhist == 0) {
      P.k3 = h;
      return P;
   }
   const double h1 = S.h1, w = h / h1;
   if (q == 1) {
      P.k0 = 1.0 + w;
      P.k1 = -w;
      P.c = w / (2.0 * w + 1.0);
      return P;
   }
   const double h2 = S.h2;
   P.k0 = (h + h1) * (h + h1 + h2) / (h1 * (h1 + h2));
   P.k1 = -h * (h + h1 + h2) / (h1 * h2);
   P.k2 = h * (h + h1) / ((h1 + h2) * h2);
   const double A = h * h * h * (1.0 + w) * (1.0 + w) / (w * (1.0 + 2.0 * w));
   const double Pp = h * (h + h1) * (h + h1 + h2);
   P.c = A / (Pp + A);
   return P;
}

// WRMS norm (weights S.w) of c0 v0 + c1 v1 (+ c2 v2) (+ c3 v3)
static double wrms_comb(Stepper& S, const double* v0, double c0, const double* v1, double c1,
                        const double* v2, double c2, const double* v3, double c3)
{
   const double* w = S.w;
   const double ss = S.red.sum(S.NY, [=] __device__(long long t) {
      double x = c0 * v0[t] + c1 * v1[t];
      if (v2) x += c2 * v2[t];
      if (v3) x += c3 * v3[t];
      x *= w[t];
      return x * x;
   });
   return std::sqrt(ss / (double)S.NY);
}

// One accepted step of a variable-step BDF of orders 1 and 2 with CVODE's
// local error test and step-size / order selection (SUNDIALS CVODE 5.7.0
// as configured by CVODESolver::initializeCVODE, samrai/CVODESolver.cc:
// 112-258, and driven in CV_ONE_STEP mode, QuatIntegrator.cc:1571-1596).
// Its published rules: error test dsm = c ||y_{n+1} - pred||_WRMS <= 1;
// Newton test del min(1, crate) c <= 0.1; after a step
// eta = 1 / ((6 dsm)^(1/(q+1)) + 1e-6), and every q+1 steps the order-(q-1)
// and order-(q+1) candidates (bias 6 and 10); no change below eta 1.5;
// growth capped at 1e4 on the first step and 10 afterwards, at 1 after a
// step with failures; after an error-test failure eta = max(0.1, ...), at
// most 0.2 from the second failure, order 1 from the third, 7 failures at
// most; after a Newton failure eta = 0.25, 10 failures at most.  The
// corrector is a variable-coefficient BDF with extrapolation predictors
// instead of CVODE's Nordsieck array, so the step sequence is this
// algorithm's, not CVODE's own.  The step ends at t_stop at the latest
// (when t_stop > t).  0 = accepted, 1 = failed (state unchanged).
static int adaptive_step(Stepper& S, double t_stop)
{
   const long long ny = S.NY;
   const double hmax = S.p.h_max > 0.0 ? S.p.h_max : 1.0e300;
   int nef = 0, ncf = 0;
   for (;;) {
      int q = std::min(S.q_next, std::min(2, S.p.max_order));
      if (S.nhist < q) q = S.nhist < 1 ? 1 : S.nhist;
      double h = std::min(S.h_next, hmax);
      if (t_stop > S.t && S.t + h > t_stop - 1e-12 * std::fabs(t_stop)) h = t_stop - S.t;
      if (S.nhist == 0 && !S.fn_valid) {
         at_time(S, S.t);
         eval_rhs(S, S.yn, nullptr, 0.0, S.fn, 0);
         S.fn_valid = true;
      }
      const Pred P = predictor(S, h, q);
      double gamma = h, a0 = 1.0, a1 = 0.0;
      if (q == 2) {
         const double w = h / S.h1;
         a0 = (1.0 + w) * (1.0 + w) / (1.0 + 2.0 * w);
         a1 = -w * w / (1.0 + 2.0 * w);
         gamma = h * (1.0 + w) / (1.0 + 2.0 * w);
      }
      {
         double *a = S.a, *y = S.y;
         const double *yn = S.yn, *y1 = S.ynm1, *y2 = S.ynm2, *fn = S.fn;
         const Pred Q = P;
         const bool use1 = S.nhist >= 1, use2 = q == 2, usef = S.nhist == 0;
         map(ny, [=] __device__(long long t) {
            double pr = Q.k0 * yn[t];
            if (use1) pr += Q.k1 * y1[t];
            if (use2) pr += Q.k2 * y2[t];
            if (usef) pr += Q.k3 * fn[t];
            y[t] = pr;
            a[t] = use2 ? a0 * yn[t] + a1 * y1[t] : yn[t];
         }, S.s);
      }
      at_time(S, S.t + h);
      if (bdf_newton(S, gamma, 0.1 / P.c)) {
         ncf++;
         if (ncf >= 10 || h <= S.p.h_min) return 1;
         S.h_next = h * 0.25;
         S.eta_max = 1.0;
         continue;
      }
      // local error estimate from the predictor-corrector difference
      const double dsm =
          P.c * wrms_comb(S, S.ynew, 1.0, S.yn, -P.k0, S.nhist >= 1 ? S.ynm1 : nullptr, -P.k1,
                          q == 2 ? S.ynm2 : (S.nhist == 0 ? S.fn : nullptr),
                          q == 2 ? -P.k2 : -P.k3);
      if (dsm > 1.0) {
         nef++;
         S.st.err_test_fails++;
         if (nef >= 7 || h <= S.p.h_min) return 1;
         double eta = 1.0 / (std::pow(6.0 * dsm, 1.0 / (q + 1)) + 1.0e-6);
         eta = std::max(0.1, eta);
         if (nef >= 2) eta = std::min(eta, 0.2);
         if (nef >= 3) S.q_next = 1;
         S.h_next = h * eta;
         S.eta_max = 1.0;
         continue;
      }
      // accepted: the next step's size and order
      double eta = 1.0 / (std::pow(6.0 * dsm, 1.0 / (q + 1)) + 1.0e-6);
      int qn = q;
      if (--S.qwait <= 0) {
         if (q == 2) {  // order 1: h^2 times the second divided difference
            const double h1 = S.h1;
            const double ca = 1.0 / (h * (h + h1)), cb = 1.0 / (h1 * (h + h1));
            const double dsm1 = wrms_comb(S, S.ynew, h * h * ca, S.yn, -h * h * (ca + cb),
                                          S.ynm1, h * h * cb, nullptr, 0.0);
            const double em = 1.0 / (std::pow(6.0 * dsm1, 0.5) + 1.0e-6);
            if (em > eta) {
               eta = em;
               qn = 1;
            }
         } else if (S.p.max_order >= 2 && S.nhist >= 2) {
            // order 2: (4/3) h^3 times the third divided difference
            // y[t_{n+1}, t_n, t_{n-1}, t_{n-2}] = sum_i y_i / prod_{j!=i}(t_i - t_j)
            const double h1 = S.h1, h2 = S.h2;
            const double t0 = h, t1 = 0.0, t2 = -h1, t3 = -h1 - h2;
            const double w0 = 1.0 / ((t0 - t1) * (t0 - t2) * (t0 - t3));
            const double w1 = 1.0 / ((t1 - t0) * (t1 - t2) * (t1 - t3));
            const double w2 = 1.0 / ((t2 - t0) * (t2 - t1) * (t2 - t3));
            const double w3 = 1.0 / ((t3 - t0) * (t3 - t1) * (t3 - t2));
            const double k = 4.0 / 3.0 * h * h * h;
            const double dsm2 = wrms_comb(S, S.ynew, k * w0, S.yn, k * w1, S.ynm1, k * w2,
                                          S.ynm2, k * w3);
            const double ep = 1.0 / (std::pow(10.0 * dsm2, 1.0 / 3.0) + 1.0e-6);
            if (ep > eta) {
               eta = ep;
               qn = 2;
            }
         }
         S.qwait = qn + 1;
      }
      if (eta < 1.5) {
         eta = 1.0;
         qn = q;
      } else {
         eta = std::min(eta, S.eta_max);
      }
      if (nef || ncf) eta = std::min(eta, 1.0);
      S.eta_max = 10.0;
      S.h_next = std::min(h * eta, hmax);
      S.q_next = qn;
      // history shift: y_{n-2} <- y_{n-1} <- y_n <- y_{n+1}
      double* old2 = S.ynm2;
      S.ynm2 = S.ynm1;
      S.ynm1 = S.yn;
      S.yn = S.ynew;
      S.ynew = old2;
      S.h2 = S.h1;
      S.h1 = h;
      S.nhist = std::min(S.nhist + 1, 2);
      S.fn_valid = false;
      S.t += h;
      S.st.h_last = h;
      S.st.q_last = q;
      return 0;
   }
}

// a new start for the variable-step BDF: first step of size dt, order 1
static void restart_history(Stepper& S)
{
   S.nhist = 0;
   S.q_next = 1;
   S.qwait = 2;
   S.h_next = S.p.dt;
   S.h1 = S.h2 = 0.0;
   S.eta_max = 1.0e4;
   S.fn_valid = false;
}

// bookkeeping after an accepted step (either mode)
static void step_accepted(Stepper& S)
{
   S.cold = false;
   keep_warm_start(S);
   S.st.steps++;
   if (S.prof) {
      cudaStreamSynchronize(S.s);
      prof_collect(S);
   }
}

// counters of the KKS kernels and the history into the stats
static int finish_stats(Stepper& S, ampe_step_stats_t* stats)
{
   unsigned long long c[2] = {0, 0}, mc[5] = {0, 0, 0, 0, 0};
   cudaMemcpyAsync(c, S.counters, sizeof(c), cudaMemcpyDeviceToHost, S.s);
   if (S.mcount) cudaMemcpyAsync(mc, S.mcount, sizeof(mc), cudaMemcpyDeviceToHost, S.s);
   if (cudaStreamSynchronize(S.s) != cudaSuccess) return AMPE_ERR_CUDA;
   S.st.kks_iters = (long long)(c[0] + mc[0] + mc[4]);
   S.st.kks_fail = (long long)(c[1] + mc[1]);
   S.st.kks_fp64_cells = (long long)mc[2];
   S.st.kks_fallback = (long long)mc[3];
   S.st.t = S.t;
   S.st.h_next = S.p.adaptive ? S.h_next : S.p.dt;
   S.st.q_next = S.p.adaptive ? S.q_next : (S.hist ? std::min(2, S.p.max_order) : 1);
   if (stats) *stats = S.st;
   return AMPE_OK;
}

// accepted variable steps until t_stop (if > t) or max_steps
static int advance_adaptive(Stepper& S, double t_stop, int max_steps)
{
   // a stop time not in the past (at t already: no step, as CVODE's
   // CV_TSTOP_RETURN); anything earlier means none
   const double eps = 1e-12 * std::fabs(t_stop);
   const bool has_stop = t_stop >= S.t - eps;
   for (int n = 0; n < max_steps; n++) {
      if (has_stop && S.t >= t_stop - eps) break;
      if (adaptive_step(S, t_stop)) return AMPE_ERR_NOT_CONVERGED;
      step_accepted(S);
   }
   return AMPE_OK;
}

}  // namespace ampe

using namespace ampe;

// Host <-> device copies of the state for callers that hand the fields in
// and out every step.  Pinned host memory is mapped into the device's
// address space (unified addressing); there a grid of 16-byte loads and
// stores over the host link moves the data faster than one copy engine, so
// mapped buffers are copied by a kernel and anything else (pageable memory,
// a buffer not mapped) by cudaMemcpyAsync.
static const double* mapped_host(const double* p)
{
   cudaPointerAttributes a;
   if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
      cudaGetLastError();  // an unregistered pointer: clear the query's error
      return nullptr;
   }
   if (a.type == cudaMemoryTypeHost && a.devicePointer)
      return static_cast<const double*>(a.devicePointer);
   return nullptr;
}

__global__ void k_copy_f64(const double* __restrict__ src, double* __restrict__ dst,
                           long long n)
{
   const long long n2 = n / 2;
   const double2* s2 = reinterpret_cast<const double2*>(src);
   double2* d2 = reinterpret_cast<double2*>(dst);
   for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < n2;
        t += (long long)gridDim.x * blockDim.x)
      d2[t] = s2[t];
   if (blockIdx.x == 0 && threadIdx.x == 0 && (n & 1)) dst[n - 1] = src[n - 1];
}

// copy n doubles between the host and the device on stream s (host -> device
// if to_device); the kernel path needs both pointers 16-byte aligned
static int copy_host(double* dst, const double* src, long long n, bool to_device, cudaStream_t s)
{
   const double* hp = to_device ? src : dst;
   const double* mp = mapped_host(hp);
   const bool aligned = ((reinterpret_cast<uintptr_t>(dst) | reinterpret_cast<uintptr_t>(src)) & 15) == 0;
   if (mp && aligned && n >= 2) {
      const double* from = to_device ? mp : src;
      double* to = to_device ? dst : const_cast<double*>(mp);
      k_copy_f64<<<(unsigned)max_blocks(8), 256, 0, s>>>(from, to, n);
      g_launches++;
      return cudaGetLastError() == cudaSuccess ? AMPE_OK : AMPE_ERR_CUDA;
   }
   return cudaMemcpyAsync(dst, src, sizeof(double) * (size_t)n,
                          to_device ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToHost, s) ==
                  cudaSuccess
              ? AMPE_OK
              : AMPE_ERR_CUDA;
}

extern "C" {

int ampe_stepper_create(const ampe_model_t* m, const ampe_step_params_t* p,
                        void** handle)
{
   if (!handle || !p || check_model(m)) return AMPE_ERR_INVALID;
   *handle = nullptr;
   if (p->dt <= 0.0 || p->max_krylov < 1 || p->max_newton < 1 ||
       p->max_order < 1 || p->atol <= 0.0)
      return AMPE_ERR_INVALID;
   if (p->precond < 0 || p->precond > 2 || p->precision < 0 ||
       p->precision > 1 || p->max_krylov > kMaxKrylov)
      return AMPE_ERR_INVALID;
   if (p->adaptive < 0 || p->adaptive > 1 || p->h_min < 0.0) return AMPE_ERR_INVALID;
   if (p->surrogate < 0 || p->surrogate > 2) return AMPE_ERR_INVALID;
   if (m->flux_type == AMPE_FLUX_ANISOTROPIC) {
      if (m->qlen != 2 && m->qlen != 4) return AMPE_ERR_INVALID;
      if (m->evolve_quat && m->qlen != 4) return AMPE_ERR_INVALID;
      // the mixed path linearises the anisotropic flux for a static
      // orientation field (no evolve_quat)
      if (p->precision == 1 && m->evolve_quat) return AMPE_ERR_INVALID;
   }
   if (m->evolve_quat && (m->quat_mobility_type != 'p' || !(m->quat_grad_floor > 0.0)))
      return AMPE_ERR_INVALID;
   if (!std::isfinite(m->dTdt) || (m->dTdt != 0.0 && m->temp_mode == AMPE_TEMP_FIELD))
      return AMPE_ERR_INVALID;
   // the mobility diffusivities belong to the "ebs" form and take the
   // CALPHAD free-energy curvature
   if (m->conc_diffusion == AMPE_DIFF_MOBILITY &&
       (m->conc_form != AMPE_CONC_EBS || m->thermo != AMPE_THERMO_CALPHAD))
      return AMPE_ERR_INVALID;
   if (ampe_device_count() < 1) return AMPE_ERR_NO_DEVICE;
   Stepper* S = new (std::nothrow) Stepper;
   if (!S) return AMPE_ERR_INVALID;
   S->m = *m;
   S->T_start = m->T0;
   S->m.ng_side = 0;  // the stepper's own face arrays carry no ghosts
   m = &S->m;
   S->p = *p;
   S->g = make_grid(*m);
   S->N = S->g.cells();
   S->NG = S->g.cells_ghost();
   S->nb = m->evolve_quat ? 6 : 2;
   S->NY = S->nb * S->N;
   S->mp = make_mix_params(*m);
   std::memset(&S->st, 0, sizeof(S->st));
   int err = AMPE_OK;
   if (cudaStreamCreateWithFlags(&S->s, cudaStreamNonBlocking) != cudaSuccess)
      err = AMPE_ERR_CUDA;
   S->own_s = S->s;
   if (!err) err = S->red.init(S->s);
   double** gh[] = {&S->phi_g, &S->c_g, &S->cl, &S->cs, &S->clr,
                    &S->csr, &S->cl_nf, &S->cs_nf, &S->phi_lag, &S->tfield};
   for (double** q : gh) *q = dvec(*S, S->NG, &err);
   S->dF = dvec(*S, S->N, &err);
   double** vv[] = {&S->yn, &S->ynm1, &S->ynew, &S->a,   &S->y,  &S->fy, &S->b,  &S->d,
                    &S->w,  &S->wi,   &S->tmp,  &S->av, &S->fp, &S->ysave, &S->ym1save};
   for (double** q : vv) *q = dvec(*S, S->NY, &err);
   if (p->adaptive) {
      S->ynm2 = dvec(*S, S->NY, &err);
      S->fn = dvec(*S, S->NY, &err);
   }
   S->h_next = p->dt;
   if (p->precision == 1) {
      for (int l = 0; l <= p->max_krylov; l++)
         S->Vf.push_back((float*)dalloc<float>(S->pool, S->NY, &err));
      float** fv[] = {&S->tmpf, &S->avf, &S->bf, &S->w32, &S->wi32};
      for (float** q : fv) *q = (float*)dalloc<float>(S->pool, S->NY, &err);
   } else {
      for (int l = 0; l <= p->max_krylov; l++) S->V.push_back(dvec(*S, S->NY, &err));
   }
   S->counters = (unsigned long long*)dalloc<unsigned long long>(S->pool, 2, &err);
   if (m->flux_type == AMPE_FLUX_ANISOTROPIC && !m->evolve_quat) {
      S->qorient = dvec(*S, (long long)m->qlen * S->NG, &err);
      if (p->precision == 1) {
         for (int d = 0; d < m->dim; d++) {
            const long long nf = d == 0 ? S->g.nfx() : (d == 1 ? S->g.nfy() : S->g.nfz());
            S->an.F[d] = (float*)dalloc<float>(S->pool, nf, &err);
            S->an.JA[d] = (float*)dalloc<float>(S->pool, nf, &err);
            S->an.JB[d] = (float*)dalloc<float>(S->pool, nf, &err);
            if (m->dim == 3)
               S->an.JC[d] = (float*)dalloc<float>(S->pool, nf, &err);
            else
               S->an.PO[d] = (float*)dalloc<float>(S->pool, nf, &err);
         }
      }
   }
   if (S->nb == 6) {
      S->q_g = dvec(*S, 4 * S->NG, &err);
      S->q_lag = dvec(*S, 4 * S->NG, &err);
      S->ogm = dvec(*S, S->N, &err);
      S->mq = dvec(*S, S->NG, &err);
      S->fcq[0] = dvec(*S, S->g.nfx(), &err);
      S->fcq[1] = dvec(*S, S->g.nfy(), &err);
      if (S->g.dim == 3) S->fcq[2] = dvec(*S, S->g.nfz(), &err);
   }
   if (p->precision == 1) {
      float** f32g[] = {&S->cl32, &S->cs32, &S->clr32, &S->csr32, &S->pf32,
                        &S->dphi32, &S->da32, &S->db32};
      for (float** q : f32g) *q = (float*)dalloc<float>(S->pool, S->NG, &err);
      S->dF32 = (float*)dalloc<float>(S->pool, S->N, &err);
      if (m->conc_form == AMPE_CONC_KKS)
         S->dc32 = (float*)dalloc<float>(S->pool, S->NG, &err);
      const long long nfd[3] = {S->g.nfx(), S->g.nfy(), S->g.dim == 3 ? S->g.nfz() : 0};
      for (int d = 0; d < S->g.dim; d++) {
         S->fw.A[d] = (float*)dalloc<float>(S->pool, nfd[d], &err);
         S->fw.B[d] = (float*)dalloc<float>(S->pool, nfd[d], &err);
      }
      S->mcount = (unsigned long long*)dalloc<unsigned long long>(S->pool, 5, &err);
      S->kks_list = (int*)dalloc<int>(S->pool, S->N + 1, &err);
      if (p->surrogate) {
         S->guess_l = (float*)dalloc<float>(S->pool, S->N, &err);
         S->guess_s = (float*)dalloc<float>(S->pool, S->N, &err);
      }
      if (S->nb == 6) {
         QuatF32& Q = S->qf32;
         Q.q = (float*)dalloc<float>(S->pool, 4 * S->NG, &err);
         Q.dq = (float*)dalloc<float>(S->pool, 4 * S->NG, &err);
         Q.ogm = (float*)dalloc<float>(S->pool, S->N, &err);
         Q.mq = (float*)dalloc<float>(S->pool, S->NG, &err);
         const long long nf[3] = {S->g.nfx(), S->g.nfy(), S->g.dim == 3 ? S->g.nfz() : 0};
         for (int d = 0; d < S->g.dim; d++) {
            Q.fc[d] = (float*)dalloc<float>(S->pool, nf[d], &err);
            Q.dfc[d] = (float*)dalloc<float>(S->pool, nf[d], &err);
         }
      }
   }
   const int nt = m->temp_mode == AMPE_TEMP_GRADIENT ? m->n[0] : 1;
   if (m->temp_mode != AMPE_TEMP_FIELD) {
      S->tab = (ThermoCoef*)dalloc<ThermoCoef>(S->pool, nt, &err);
      if (p->precision == 1) S->tabf = (CoefF*)dalloc<CoefF>(S->pool, nt, &err);
      if (p->precision == 1 && S->mp.tdep)
         S->dqtab = (float2*)dalloc<float2>(S->pool, 2LL * m->n[0] + 1, &err);
   }
   const int nl = p->precond == 2 ? std::max(1, p->mg_levels) : 1;
   if (!err && p->precond) {
      if (p->precision == 1) {
         err = fac_create(S->facp32, *m, nl, false, true, S->pool);
         if (!err) err = fac_create(S->facc32, *m, nl, true, false, S->pool);
         if (!err && S->nb == 6)
            err = fac_create(S->facq32, *m, nl, true, false, S->pool, true);
      } else {
         err = fac_create(S->facp64, *m, nl, false, true, S->pool);
         if (!err) err = fac_create(S->facc64, *m, nl, true, false, S->pool);
         if (!err && S->nb == 6)
            err = fac_create(S->facq64, *m, nl, true, false, S->pool, true);
      }
   }
   // the zero fills of dalloc run on the legacy stream, which does not
   // order with the non-blocking stepper stream: finish them first
   if (!err && cudaDeviceSynchronize() != cudaSuccess) err = AMPE_ERR_CUDA;
   if (!err && S->qorient) {  // default orientation: angle 0, q = (1, 0, ...)
      double* q0 = S->qorient;
      const long long ng = S->NG;
      map(ng, [=] __device__(long long t) { q0[t] = 1.0; }, S->s);
      if (S->an.PO[0]) aniso_orientation_f32(*m, S->g, S->qorient, S->an, S->s);
   }
   if (!err && S->tab) err = build_thermo_table(*m, S->tab, nt, S->s);
   if (!err && S->tabf) err = build_coef_f(S->tab, S->tabf, nt, S->s);
   if (!err && S->dqtab) {
      err = build_diff_table(*m, S->mp, S->g, S->dqtab, S->s);
      S->mp.dq = S->dqtab;
   }
   if (!err && cudaStreamSynchronize(S->s) != cudaSuccess) err = AMPE_ERR_CUDA;
   if (err) {
      ampe_stepper_destroy(S);
      return err;
   }
   *handle = S;
   return AMPE_OK;
}

int ampe_stepper_destroy(void* h)
{
   Stepper* S = (Stepper*)h;
   if (!S) return AMPE_ERR_INVALID;
   if (S->s) cudaStreamSynchronize(S->s);
   for (cudaEvent_t e : S->ev_pool) cudaEventDestroy(e);
   for (void* q : S->pool) cudaFree(q);
   S->red.release();
   if (S->own_s) cudaStreamDestroy(S->own_s);
   delete S;
   return AMPE_OK;
}

int ampe_stepper_set_state(void* h, const double* phi, const double* conc,
                           const double* cl, const double* cs,
                           const double* temp, int host)
{
   Stepper* S = (Stepper*)h;
   if (!S || !phi || !conc) return AMPE_ERR_INVALID;
   if (S->m.temp_mode == AMPE_TEMP_FIELD && !temp) return AMPE_ERR_INVALID;
   const cudaMemcpyKind kind = host ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToDevice;
   const size_t bytes = sizeof(double) * (size_t)S->N;
   cudaMemcpyAsync(S->yn, phi, bytes, kind, S->s);
   cudaMemcpyAsync(S->yn + S->N, conc, bytes, kind, S->s);
   if (S->nb == 6) {  // orientation (1, 0, 0, 0) until ampe_stepper_set_quat
      double* q = S->yn + 2 * S->N;
      const long long n4 = 4 * S->N, N = S->N;
      map(n4, [=] __device__(long long t) { q[t] = t < N ? 1.0 : 0.0; }, S->s);
   }
   cudaMemcpyAsync(S->ynm1, S->yn, S->nb * bytes, cudaMemcpyDeviceToDevice, S->s);
   // warm starts (interior) -> ghosted refs; default (c, c)
   double* stage = S->tmp;
   cudaMemcpyAsync(stage, cl ? cl : conc, bytes, cl ? kind : kind, S->s);
   cudaMemcpyAsync(stage + S->N, cs ? cs : conc, bytes, kind, S->s);
   to_ghosted<double>(S->g, stage, nullptr, 0.0, S->clr, S->s);
   to_ghosted<double>(S->g, stage + S->N, nullptr, 0.0, S->csr, S->s);
   const size_t gb = sizeof(double) * (size_t)S->NG;
   cudaMemcpyAsync(S->cl, S->clr, gb, cudaMemcpyDeviceToDevice, S->s);
   cudaMemcpyAsync(S->cs, S->csr, gb, cudaMemcpyDeviceToDevice, S->s);
   cudaMemcpyAsync(S->cl_nf, S->clr, gb, cudaMemcpyDeviceToDevice, S->s);
   cudaMemcpyAsync(S->cs_nf, S->csr, gb, cudaMemcpyDeviceToDevice, S->s);
   if (S->p.precision == 1) {
      to_ghosted<float>(S->g, stage, nullptr, 0.0, S->clr32, S->s);
      to_ghosted<float>(S->g, stage + S->N, nullptr, 0.0, S->csr32, S->s);
      const size_t gf = sizeof(float) * (size_t)S->NG;
      cudaMemcpyAsync(S->cl32, S->clr32, gf, cudaMemcpyDeviceToDevice, S->s);
      cudaMemcpyAsync(S->cs32, S->csr32, gf, cudaMemcpyDeviceToDevice, S->s);
   }
   if (temp) {
      cudaMemcpyAsync(stage, temp, bytes, kind, S->s);
      to_ghosted<double>(S->g, stage, nullptr, 0.0, S->tfield, S->s);
   }
   S->hist = 0;
   restart_history(*S);
   S->t = 0.0;
   S->cold = !(cl && cs);
   if (cudaStreamSynchronize(S->s) != cudaSuccess) return AMPE_ERR_CUDA;
   return AMPE_OK;
}

int ampe_stepper_get_state(void* h, double* phi, double* conc, double* cl,
                           double* cs, int host)
{
   Stepper* S = (Stepper*)h;
   if (!S) return AMPE_ERR_INVALID;
   const cudaMemcpyKind kind = host ? cudaMemcpyDeviceToHost : cudaMemcpyDeviceToDevice;
   const size_t bytes = sizeof(double) * (size_t)S->N;
   if (host) {
      if (phi && copy_host(phi, S->yn, S->N, false, S->s)) return AMPE_ERR_CUDA;
      if (conc && copy_host(conc, S->yn + S->N, S->N, false, S->s)) return AMPE_ERR_CUDA;
   } else {
      if (phi) cudaMemcpyAsync(phi, S->yn, bytes, kind, S->s);
      if (conc) cudaMemcpyAsync(conc, S->yn + S->N, bytes, kind, S->s);
   }
   if (cl || cs) {
      if (S->p.precision == 1) {
         k_from_ghosted<float, double><<<map_blocks(S->N), 256, 0, S->s>>>(S->g, S->clr32,
                                                                           S->tmp);
         k_from_ghosted<float, double><<<map_blocks(S->N), 256, 0, S->s>>>(S->g, S->csr32,
                                                                           S->tmp + S->N);
      } else {
         k_from_ghosted<double, double><<<map_blocks(S->N), 256, 0, S->s>>>(S->g, S->clr,
                                                                            S->tmp);
         k_from_ghosted<double, double><<<map_blocks(S->N), 256, 0, S->s>>>(S->g, S->csr,
                                                                            S->tmp + S->N);
      }
      g_launches += 2;
      if (cl) cudaMemcpyAsync(cl, S->tmp, bytes, kind, S->s);
      if (cs) cudaMemcpyAsync(cs, S->tmp + S->N, bytes, kind, S->s);
   }
   if (cudaStreamSynchronize(S->s) != cudaSuccess) return AMPE_ERR_CUDA;
   return AMPE_OK;
}

int ampe_stepper_eval_rhs(void* h, double* phi_rhs, double* conc_rhs, int host)
{
   Stepper* S = (Stepper*)h;
   if (!S || !phi_rhs || !conc_rhs) return AMPE_ERR_INVALID;
   at_time(*S, S->t);
   eval_rhs(*S, S->yn, nullptr, 0.0, S->fy, 0);
   const cudaMemcpyKind kind = host ? cudaMemcpyDeviceToHost : cudaMemcpyDeviceToDevice;
   const size_t bytes = sizeof(double) * (size_t)S->N;
   cudaMemcpyAsync(phi_rhs, S->fy, bytes, kind, S->s);
   cudaMemcpyAsync(conc_rhs, S->fy + S->N, bytes, kind, S->s);
   if (cudaStreamSynchronize(S->s) != cudaSuccess) return AMPE_ERR_CUDA;
   return AMPE_OK;
}

int ampe_stepper_advance(void* h, int nsteps, ampe_step_stats_t* stats)
{
   Stepper* S = (Stepper*)h;
   if (!S || nsteps < 0) return AMPE_ERR_INVALID;
   if (S->p.adaptive) {
      const int rc = advance_adaptive(*S, -1.0e300, nsteps);
      const int rs = finish_stats(*S, stats);
      return rc ? rc : rs;
   }
   int ret = AMPE_OK;
   const size_t b2 = sizeof(double) * (size_t)S->NY;
   for (int n = 0; n < nsteps; n++) {
      double hstep = S->p.dt;
      const int q = S->hist ? std::min(2, S->p.max_order) : 1;
      int fail = bdf_step(*S, S->t + hstep, hstep, q);
      int retries = 0;
      if (fail) {
         // order-1 sub-steps: after each failure halve the sub-step and go
         // on from the last accepted sub-step until the whole step is
         // covered; if the retries run out, the step's start is restored
         cudaMemcpyAsync(S->ysave, S->yn, b2, cudaMemcpyDeviceToDevice, S->s);
         cudaMemcpyAsync(S->ym1save, S->ynm1, b2, cudaMemcpyDeviceToDevice, S->s);
         double done = 0.0, hsub = hstep;
         while (fail && retries < S->p.max_retries) {
            retries++;
            S->st.step_retries++;
            hsub *= 0.5;
            fail = 0;
            while (done < hstep * (1.0 - 1e-12)) {
               const double hh = std::min(hsub, hstep - done);
               if (bdf_step(*S, S->t + done + hh, hh, 1)) {
                  fail = 1;
                  break;
               }
               done += hh;
               if (done < hstep * (1.0 - 1e-12)) {  // accept the sub-step
                  cudaMemcpyAsync(S->ynm1, S->yn, b2, cudaMemcpyDeviceToDevice, S->s);
                  cudaMemcpyAsync(S->yn, S->ynew, b2, cudaMemcpyDeviceToDevice, S->s);
               }
            }
         }
         if (fail) {
            cudaMemcpyAsync(S->yn, S->ysave, b2, cudaMemcpyDeviceToDevice, S->s);
            cudaMemcpyAsync(S->ynm1, S->ym1save, b2, cudaMemcpyDeviceToDevice, S->s);
         }
      }
      if (fail) {
         ret = AMPE_ERR_NOT_CONVERGED;
         break;
      }
      S->hist = retries == 0 ? 1 : 0;
      swap_ptr(S->ynm1, S->yn);  // ynm1 <- yn
      swap_ptr(S->yn, S->ynew);  // yn <- ynew
      S->t += S->p.dt;
      S->st.h_last = S->p.dt;
      S->st.q_last = q;
      step_accepted(*S);
   }
   const int rs = finish_stats(*S, stats);
   return ret ? ret : rs;
}

int ampe_stepper_advance_to(void* h, double t_stop, int max_steps, ampe_step_stats_t* stats)
{
   Stepper* S = (Stepper*)h;
   if (!S || max_steps < 0 || !S->p.adaptive) return AMPE_ERR_INVALID;
   const int rc = advance_adaptive(*S, t_stop, max_steps);
   const int rs = finish_stats(*S, stats);
   return rc ? rc : rs;
}

int ampe_stepper_set_temperature(void* h, double T0, double gradT)
{
   Stepper* S = (Stepper*)h;
   if (!S || !(T0 > 0.0) || S->m.temp_mode == AMPE_TEMP_FIELD) return AMPE_ERR_INVALID;
   if (S->m.temp_mode == AMPE_TEMP_CONSTANT && gradT != 0.0) return AMPE_ERR_INVALID;
   if (S->m.dTdt != 0.0) return AMPE_ERR_INVALID;  // T follows the model's T0(t)
   S->m.T0 = T0;
   S->m.gradT = gradT;
   int err = apply_temperature(*S);
   S->fn_valid = false;
   if (!err && cudaStreamSynchronize(S->s) != cudaSuccess) err = AMPE_ERR_CUDA;
   return err;
}

long long ampe_stepper_kernel_launches(void* h)
{
   (void)h;
   return g_launches;
}

int ampe_stepper_attach_surrogate(void* h, void* mlp)
{
   Stepper* S = (Stepper*)h;
   if (!S || !mlp || !S->guess_l) return AMPE_ERR_INVALID;
   Mlp* M = (Mlp*)mlp;
   // the network sees the stepper's temperature field
   M->m.temp_mode = S->m.temp_mode;
   M->m.T0 = S->m.T0;
   M->m.gradT = S->m.gradT;
   for (int d = 0; d < 3; d++) M->m.dx[d] = S->m.dx[d];
   S->mlp = M;
   return AMPE_OK;
}

int ampe_stepper_set_stream(void* h, void* stream)
{
   Stepper* S = (Stepper*)h;
   if (!S) return AMPE_ERR_INVALID;
   if (cudaStreamSynchronize(S->s) != cudaSuccess) return AMPE_ERR_CUDA;
   S->s = stream ? (cudaStream_t)stream : S->own_s;
   S->red.s = S->s;
   return AMPE_OK;
}

void* ampe_stepper_stream(void* h)
{
   Stepper* S = (Stepper*)h;
   return S ? (void*)S->s : nullptr;
}

int ampe_stepper_profile(void* h, int enable)
{
   Stepper* S = (Stepper*)h;
   if (!S) return AMPE_ERR_INVALID;
   if (enable && S->ev_pool.empty()) {
      S->ev_pool.resize(8192);
      for (auto& e : S->ev_pool)
         if (cudaEventCreate(&e) != cudaSuccess) return AMPE_ERR_CUDA;
   }
   cudaStreamSynchronize(S->s);
   prof_collect(*S);
   for (int k = 0; k < 8; k++) {
      S->kms[k] = 0.0;
      S->kcount[k] = 0;
   }
   S->prof = enable != 0;
   return AMPE_OK;
}

int ampe_stepper_kernel_time(void* h, int kind, double* total_ms,
                             long long* launches)
{
   Stepper* S = (Stepper*)h;
   if (!S || kind < 0 || kind >= KT_NKINDS) return AMPE_ERR_INVALID;
   cudaStreamSynchronize(S->s);
   prof_collect(*S);
   if (total_ms) *total_ms = S->kms[kind];
   if (launches) *launches = S->kcount[kind];
   return AMPE_OK;
}

int ampe_stepper_jv(void* h, const double* v, double gamma, double* out,
                    int host)
{
   Stepper* S = (Stepper*)h;
   if (!S || !v || !out) return AMPE_ERR_INVALID;
   const cudaMemcpyKind in = host ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToDevice;
   const cudaMemcpyKind ot = host ? cudaMemcpyDeviceToHost : cudaMemcpyDeviceToDevice;
   const size_t b2 = sizeof(double) * (size_t)S->NY;
   double *w = S->w, *yn = S->yn;
   const double rtol = S->p.rtol, atol = S->p.atol;
   double* wi = S->wi;
   map(S->NY, [=] __device__(long long t) {
      const double e = rtol * fabs(yn[t]) + atol;
      w[t] = 1.0 / e;
      wi[t] = e;
   }, S->s);
   at_time(*S, S->t);
   eval_rhs(*S, S->yn, nullptr, 0.0, S->fy, 0);
   cudaMemcpyAsync(S->b, v, b2, in, S->s);
   if (S->p.precision == 1) {
      const double* bd = S->b;
      double* dd = S->d;
      float *bf = S->bf, *of = S->avf;
      map(S->NY, [=] __device__(long long t) { bf[t] = d2f(bd[t]); }, S->s);
      matvec32(*S, gamma, bf, of);
      map(S->NY, [=] __device__(long long t) { dd[t] = f2d(of[t]); }, S->s);
   } else {
      matvec(*S, S->yn, S->fy, S->w, gamma, S->b, S->d);
   }
   cudaMemcpyAsync(out, S->d, b2, ot, S->s);
   if (cudaStreamSynchronize(S->s) != cudaSuccess) return AMPE_ERR_CUDA;
   return AMPE_OK;
}

int ampe_stepper_set_quat(void* h, const double* q, int host)
{
   Stepper* S = (Stepper*)h;
   if (!S || !q || S->nb != 6) return AMPE_ERR_INVALID;
   const cudaMemcpyKind kind = host ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToDevice;
   const size_t b4 = sizeof(double) * 4 * (size_t)S->N;
   cudaMemcpyAsync(S->yn + 2 * S->N, q, b4, kind, S->s);
   cudaMemcpyAsync(S->ynm1 + 2 * S->N, S->yn + 2 * S->N, b4, cudaMemcpyDeviceToDevice,
                   S->s);
   S->hist = 0;
   restart_history(*S);
   if (cudaStreamSynchronize(S->s) != cudaSuccess) return AMPE_ERR_CUDA;
   return AMPE_OK;
}

int ampe_stepper_set_orientation(void* h, const double* q, int host)
{
   Stepper* S = (Stepper*)h;
   if (!S || !q || !S->qorient) return AMPE_ERR_INVALID;
   const cudaMemcpyKind kind = host ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToDevice;
   const size_t bytes = sizeof(double) * (size_t)S->N;
   for (int c = 0; c < S->m.qlen; c++) {
      cudaMemcpyAsync(S->tmp, q + c * S->N, bytes, kind, S->s);
      to_ghosted<double>(S->g, S->tmp, nullptr, 0.0, S->qorient + c * S->NG, S->s);
   }
   if (S->an.PO[0]) aniso_orientation_f32(S->m, S->g, S->qorient, S->an, S->s);
   if (cudaStreamSynchronize(S->s) != cudaSuccess) return AMPE_ERR_CUDA;
   return AMPE_OK;
}

int ampe_stepper_get_quat(void* h, double* q, int host)
{
   Stepper* S = (Stepper*)h;
   if (!S || !q || S->nb != 6) return AMPE_ERR_INVALID;
   const cudaMemcpyKind kind = host ? cudaMemcpyDeviceToHost : cudaMemcpyDeviceToDevice;
   cudaMemcpyAsync(q, S->yn + 2 * S->N, sizeof(double) * 4 * (size_t)S->N, kind, S->s);
   if (cudaStreamSynchronize(S->s) != cudaSuccess) return AMPE_ERR_CUDA;
   return AMPE_OK;
}

int ampe_stepper_eval_rhs_full(void* h, double* out, int host)
{
   Stepper* S = (Stepper*)h;
   if (!S || !out) return AMPE_ERR_INVALID;
   at_time(*S, S->t);
   eval_rhs(*S, S->yn, nullptr, 0.0, S->fy, 0);
   const cudaMemcpyKind kind = host ? cudaMemcpyDeviceToHost : cudaMemcpyDeviceToDevice;
   cudaMemcpyAsync(out, S->fy, sizeof(double) * (size_t)S->NY, kind, S->s);
   if (cudaStreamSynchronize(S->s) != cudaSuccess) return AMPE_ERR_CUDA;
   return AMPE_OK;
}

long long ampe_stepper_size(void* h)
{
   Stepper* S = (Stepper*)h;
   return S ? S->NY : 0;
}

int ampe_stepper_load_y(void* h, const double* phi, const double* conc,
                        int host)
{
   Stepper* S = (Stepper*)h;
   if (!S || !phi || !conc) return AMPE_ERR_INVALID;
   const cudaMemcpyKind kind = host ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToDevice;
   const size_t bytes = sizeof(double) * (size_t)S->N;
   if (host) {
      if (copy_host(S->yn, phi, S->N, true, S->s) ||
          copy_host(S->yn + S->N, conc, S->N, true, S->s))
         return AMPE_ERR_CUDA;
      return AMPE_OK;
   }
   cudaMemcpyAsync(S->yn, phi, bytes, kind, S->s);
   cudaMemcpyAsync(S->yn + S->N, conc, bytes, kind, S->s);
   return cudaGetLastError() == cudaSuccess ? AMPE_OK : AMPE_ERR_CUDA;
}

}  // extern "C"
