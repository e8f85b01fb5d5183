// Two-level composite FAC (AMR): a periodic coarse level and one fine box
// refined by 2, for A u = M div(D grad u) + C u = f (C a scalar field, <= 0
// for a definite operator).  The cycle and the composite residual follow
// FACPreconditioner's default recursive cycle and solveSystem
// (samrai/FACPreconditioner.cc:267-464, 661-683) over EllipticFACOps
// (EllipticFACOps.cc:948-2029):
//   k_cf_fill        fine ghost cells <- the coarse cell they lie in
//                    (constant refinement, the "Ewing" ghost fill)
//   k_comp_flux      efo_compfluxvardc3d (3d/ellipticfacops.m4:16-82)
//   k_ewing          efo_ewingfixflux*3d (3d/ellipticfacops.m4:697-1105) on
//                    the fine box's six sides
//   k_comp_res       efo_compresvarsca3d (3d/ellipticfacops.m4:448-512)
//   k_rbgs_flux      efo_rbgswithfluxmax*3d (3d/ellipticfacops.m4:83-447)
//   k_restrict, k_coarsen_flux   conservative (volume / area weighted)
//                    coarsening of cells under the box and of the fine
//                    fluxes on its boundary faces
//   k_prolong_add    constant refinement of the coarse error, added
// One thread per cell or face; the level data are small next to the
// single-level hot path, so the kernels are written for clarity and the
// host loop mirrors the reference's call sequence.
#include <cmath>
#include <vector>

#include "common.cuh"
#include "fac.cuh"

namespace ampe {

struct FacLevel {
   const double* D[3];
   const double* C;
   const double* M;
   double dc, cc, mc;
   double dx[3];  // the level's own spacing (divergence and smoother)
   __device__ double D_at(int d, long long f) const { return D[d] ? D[d][f] : dc; }
   __device__ double C_at(long long c) const { return C ? C[c] : cc; }
   __device__ double M_at(long long c) const { return M ? M[c] : mc; }
};

struct Box {
   int lo[3], nb[3];
};

namespace {

__device__ __forceinline__ int fdiv2(int a) { return a >= 0 ? a / 2 : -((-a + 1) / 2); }
__device__ __forceinline__ int wrapn(int a, int n) { return ((a % n) + n) % n; }

__device__ __forceinline__ long long face_at(const Grid& g, int d, int i, int j, int k)
{
   return d == 0 ? g.fx(i, j, k) : (d == 1 ? g.fy(i, j, k) : g.fz(i, j, k));
}

__device__ __forceinline__ void face_split(const Grid& g, long long t, int& d, int& i, int& j,
                                           int& k)
{
   const long long nx = g.nfx(), ny = g.nfy();
   long long r = t;
   if (r < nx) {
      d = 0;
      g.split(r, g.fd0p, g.fd1, i, j, k);
   } else if ((r -= nx) < ny) {
      d = 1;
      g.split(r, g.fd0, g.fd1p, i, j, k);
   } else {
      d = 2;
      g.ijk(r - ny, i, j, k);
   }
}

#define GRID_STRIDE(t, n)                                                                   \
   for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < (n);           \
        t += (long long)gridDim.x * blockDim.x)

}  // namespace

__global__ void k_cf_fill(Grid gc, Grid gf, Box b, const double* uc, double* uf)
{
   const long long SX = gf.n0 + 2 * gf.ng, SY = gf.n1 + 2 * gf.ng;
   GRID_STRIDE(t, gf.cells_ghost())
   {
      const int i = (int)(t % SX) - gf.ng;
      const int j = (int)((t / SX) % SY) - gf.ng;
      const int k = (int)(t / (SX * SY)) - gf.gz;
      if (i >= 0 && i < gf.n0 && j >= 0 && j < gf.n1 && k >= 0 && k < gf.n2) continue;
      const int I = wrapn(b.lo[0] + fdiv2(i), gc.n0);
      const int J = wrapn(b.lo[1] + fdiv2(j), gc.n1);
      const int K = wrapn(b.lo[2] + fdiv2(k), gc.n2);
      uf[t] = uc[gc.c(I, J, K)];
   }
}

__global__ void k_comp_flux(Grid g, FacLevel lv, double dx0, double dx1, double dx2,
                            const double* u, double* f0, double* f1, double* f2)
{
   const double dinv[3] = {dx0, dx1, dx2};
   GRID_STRIDE(t, g.nfx() + g.nfy() + g.nfz())
   {
      int d, i, j, k;
      face_split(g, t, d, i, j, k);
      const int ei = d == 0, ej = d == 1, ek = d == 2;
      const long long f = face_at(g, d, i, j, k);
      double* out = d == 0 ? f0 : (d == 1 ? f1 : f2);
      out[f] = dinv[d] * lv.D_at(d, f) * (u[g.c(i, j, k)] - u[g.c(i - ei, j - ej, k - ek)]);
   }
}

// the faces of the fine box's six sides: side s = 2 d + hi
__global__ void k_ewing(Grid g, FacLevel lv, double h0, double h1, double h2, double tranwt,
                        double longwt, const double* u, double* f0, double* f1, double* f2)
{
   const int n[3] = {g.n0, g.n1, g.n2};
   const double h[3] = {h0, h1, h2};
   const long long per[3] = {(long long)n[1] * n[2], (long long)n[0] * n[2],
                             (long long)n[0] * n[1]};
   GRID_STRIDE(t, 2 * (per[0] + per[1] + per[2]))
   {
      long long r = t;
      int d = 0;
      while (r >= 2 * per[d]) r -= 2 * per[d++];
      const int hi = r >= per[d];
      if (hi) r -= per[d];
      // transverse axes (ascending) and the face's position in them
      const int a = d == 0 ? 1 : 0, b = d == 2 ? 1 : 2;
      const int ta = (int)(r % n[a]), tb = (int)(r / n[a]);
      int at[3], opp[3];
      at[d] = opp[d] = hi ? n[d] - 1 : 0;
      at[a] = ta;
      at[b] = tb;
      // the diametrically opposite fine cell within the coarse face
      opp[a] = (ta & ~1) + (1 - (ta & 1));
      opp[b] = (tb & ~1) + (1 - (tb & 1));
      int fi[3] = {at[0], at[1], at[2]};
      fi[d] = hi ? n[d] : 0;
      const long long f = face_at(g, d, fi[0], fi[1], fi[2]);
      double* out = d == 0 ? f0 : (d == 1 ? f1 : f2);
      const double diff = u[g.c(opp[0], opp[1], opp[2])] - u[g.c(at[0], at[1], at[2])];
      const double corr = tranwt * lv.D_at(d, f) * diff / h[d];
      out[f] = hi ? longwt * out[f] - corr : longwt * out[f] + corr;
   }
}

__device__ __forceinline__ double div_flux(const Grid& g, const double* f0, const double* f1,
                                           const double* f2, double dxi, double dyi,
                                           double dzi, int i, int j, int k)
{
   return dxi * (f0[g.fx(i + 1, j, k)] - f0[g.fx(i, j, k)]) +
          dyi * (f1[g.fy(i, j + 1, k)] - f1[g.fy(i, j, k)]) +
          dzi * (f2[g.fz(i, j, k + 1)] - f2[g.fz(i, j, k)]);
}

__global__ void k_comp_res(Grid g, FacLevel lv, const double* f0, const double* f1,
                           const double* f2, const double* u, const double* rhs, double* r)
{
   const double dxi = 1.0 / lv.dx[0], dyi = 1.0 / lv.dx[1], dzi = 1.0 / lv.dx[2];
   GRID_STRIDE(t, g.cells())
   {
      int i, j, k;
      g.ijk(t, i, j, k);
      const long long c = g.c(i, j, k);
      r[c] = rhs[c] - lv.M_at(c) * div_flux(g, f0, f1, f2, dxi, dyi, dzi, i, j, k) -
             lv.C_at(c) * u[c];
   }
}

__global__ void k_rbgs_flux(Grid g, FacLevel lv, const double* f0, const double* f1,
                            const double* f2, const double* rhs, double* u, int offset)
{
   const double dxi = 1.0 / lv.dx[0], dyi = 1.0 / lv.dx[1], dzi = 1.0 / lv.dx[2];
   const double dxi2 = dxi * dxi, dyi2 = dyi * dyi, dzi2 = dzi * dzi;
   GRID_STRIDE(t, g.cells())
   {
      int i, j, k;
      g.ijk(t, i, j, k);
      if (((i + j + k) & 1) != offset) continue;
      const long long c = g.c(i, j, k);
      const double m = lv.M_at(c);
      const double res = rhs[c] - m * div_flux(g, f0, f1, f2, dxi, dyi, dzi, i, j, k) -
                         lv.C_at(c) * u[c];
      const double dudr =
          1.0 / (m * (dxi2 * (lv.D_at(0, g.fx(i + 1, j, k)) + lv.D_at(0, g.fx(i, j, k))) +
                      dyi2 * (lv.D_at(1, g.fy(i, j + 1, k)) + lv.D_at(1, g.fy(i, j, k))) +
                      dzi2 * (lv.D_at(2, g.fz(i, j, k + 1)) + lv.D_at(2, g.fz(i, j, k)))) -
                 lv.C_at(c));
      u[c] = u[c] + (-res * dudr) * 1.0;
   }
}

__global__ void k_restrict(Grid gc, Grid gf, Box b, double dvf, double dvc, const double* vf,
                           double* vc)
{
   GRID_STRIDE(t, (long long)b.nb[0] * b.nb[1] * b.nb[2])
   {
      const int I = (int)(t % b.nb[0]), J = (int)((t / b.nb[0]) % b.nb[1]);
      const int K = (int)(t / ((long long)b.nb[0] * b.nb[1]));
      double s = 0.0;
      for (int kr = 0; kr < 2; kr++)
         for (int jr = 0; jr < 2; jr++)
            for (int ir = 0; ir < 2; ir++)
               s += vf[gf.c(2 * I + ir, 2 * J + jr, 2 * K + kr)] * dvf;
      vc[gc.c(wrapn(b.lo[0] + I, gc.n0), wrapn(b.lo[1] + J, gc.n1), wrapn(b.lo[2] + K, gc.n2))] =
          s / dvc;
   }
}

__global__ void k_coarsen_flux(Grid gc, Grid gf, Box b, double daf0, double daf1, double daf2,
                               double dac0, double dac1, double dac2, const double* ff0,
                               const double* ff1, const double* ff2, double* fc0, double* fc1,
                               double* fc2)
{
   const double daf[3] = {daf0, daf1, daf2}, dac[3] = {dac0, dac1, dac2};
   const int nc[3] = {gc.n0, gc.n1, gc.n2};
   const long long per[3] = {(long long)b.nb[1] * b.nb[2], (long long)b.nb[0] * b.nb[2],
                             (long long)b.nb[0] * b.nb[1]};
   GRID_STRIDE(t, 2 * (per[0] + per[1] + per[2]))
   {
      long long r = t;
      int d = 0;
      while (r >= 2 * per[d]) r -= 2 * per[d++];
      const int side = r >= per[d];
      if (side) r -= per[d];
      const int a = d == 0 ? 1 : 0, bb = d == 2 ? 1 : 2;
      const int A = (int)(r % b.nb[a]), B = (int)(r / b.nb[a]);
      const int Fn = side ? b.nb[d] : 0;
      const double* ff = d == 0 ? ff0 : (d == 1 ? ff1 : ff2);
      double* fc = d == 0 ? fc0 : (d == 1 ? fc1 : fc2);
      double s = 0.0;
      for (int br = 0; br < 2; br++)
         for (int ar = 0; ar < 2; ar++) {
            int fi[3];
            fi[d] = 2 * Fn;
            fi[a] = 2 * A + ar;
            fi[bb] = 2 * B + br;
            s += ff[face_at(gf, d, fi[0], fi[1], fi[2])] * daf[d];
         }
      int ci[3];
      ci[d] = wrapn(b.lo[d] + Fn, nc[d]);
      ci[a] = wrapn(b.lo[a] + A, nc[a]);
      ci[bb] = wrapn(b.lo[bb] + B, nc[bb]);
      const double v = s / dac[d];
      fc[face_at(gc, d, ci[0], ci[1], ci[2])] = v;
      if (ci[d] == 0) {  // the periodic image of face 0
         ci[d] = nc[d];
         fc[face_at(gc, d, ci[0], ci[1], ci[2])] = v;
      }
   }
}

__global__ void k_prolong_add(Grid gc, Grid gf, Box b, const double* ec, double* ef)
{
   GRID_STRIDE(t, gf.cells())
   {
      int i, j, k;
      gf.ijk(t, i, j, k);
      const long long cf = gf.c(i, j, k);
      ef[cf] = ef[cf] + ec[gc.c(wrapn(b.lo[0] + i / 2, gc.n0), wrapn(b.lo[1] + j / 2, gc.n1),
                                wrapn(b.lo[2] + k / 2, gc.n2))];
   }
}

__global__ void k_add_interior(Grid g, const double* e, double* u)
{
   GRID_STRIDE(t, g.cells())
   {
      int i, j, k;
      g.ijk(t, i, j, k);
      const long long c = g.c(i, j, k);
      u[c] += e[c];
   }
}

// sum of w r^2: fine cells (weight dvf) and coarse cells outside the box
// (dvc), one partial per block
__global__ void k_wnorm(Grid gc, Grid gf, Box b, double dvc, double dvf, const double* rc,
                        const double* rf, double* part)
{
   __shared__ double sh[256];
   double s = 0.0;
   const long long nf = gf.cells(), nc = gc.cells();
   GRID_STRIDE(t, nf + nc)
   {
      int i, j, k;
      if (t < nf) {
         gf.ijk(t, i, j, k);
         const double v = rf[gf.c(i, j, k)];
         s += dvf * v * v;
      } else {
         gc.ijk(t - nf, i, j, k);
         const bool under = wrapn(i - b.lo[0], gc.n0) < b.nb[0] &&
                            wrapn(j - b.lo[1], gc.n1) < b.nb[1] &&
                            wrapn(k - b.lo[2], gc.n2) < b.nb[2];
         if (under) continue;
         const double v = rc[gc.c(i, j, k)];
         s += dvc * v * v;
      }
   }
   sh[threadIdx.x] = s;
   __syncthreads();
   for (int w = blockDim.x / 2; w > 0; w >>= 1) {
      if ((int)threadIdx.x < w) sh[threadIdx.x] += sh[threadIdx.x + w];
      __syncthreads();
   }
   if (threadIdx.x == 0) part[blockIdx.x] = sh[0];
}

namespace {

constexpr int kNormBlocks = 304;

struct Fac2 {
   ampe_fac2_t p;
   Grid gc, gf;
   Box b;
   FacLevel c, f;
   double flux_dinv_c[3], flux_dinv_f[3], ewing_h[3], tranwt, longwt;
   double dvc, dvf, den;
   // workspace
   double *ec, *rcw, *ef, *rfw, *tf, *fc[3], *ff[3], *part;
   cudaStream_t s;
};

unsigned nblk(long long n)
{
   long long b = (n + 255) / 256;
   if (b > max_blocks(32)) b = max_blocks(32);
   return (unsigned)(b < 1 ? 1 : b);
}

long long faces_of(const Grid& g) { return g.nfx() + g.nfy() + g.nfz(); }

int setup(Fac2& F, const ampe_fac2_t* p, const ampe_fac2_level_t* lc, const ampe_fac2_level_t* lf)
{
   if (!p || p->coarse.dim != 3 || p->coarse.ng < 1 || p->ng_fine < 1) return AMPE_ERR_INVALID;
   if (p->presweeps < 0 || p->postsweeps < 0 || p->coarse_sweeps < 0) return AMPE_ERR_INVALID;
   ampe_model_t mc = p->coarse;
   mc.ng_side = 0;
   if (check_model(&mc)) return AMPE_ERR_INVALID;
   ampe_model_t mf = mc;
   mf.ng = p->ng_fine;
   for (int d = 0; d < 3; d++) {
      if (p->nbox[d] < 2 || p->nbox[d] > mc.n[d]) return AMPE_ERR_INVALID;
      if (p->lo[d] < 0 || p->lo[d] >= mc.n[d]) return AMPE_ERR_INVALID;
      mf.n[d] = 2 * p->nbox[d];
      mf.dx[d] = 0.5 * mc.dx[d];
   }
   if (check_model(&mf)) return AMPE_ERR_INVALID;
   F.p = *p;
   F.gc = make_grid(mc);
   F.gf = make_grid(mf);
   for (int d = 0; d < 3; d++) {
      F.b.lo[d] = p->lo[d];
      F.b.nb[d] = p->nbox[d];
      F.flux_dinv_c[d] = 1.0 / mc.dx[d];
      F.flux_dinv_f[d] = 1.0 / (p->level_dx ? mf.dx[d] : mc.dx[d]);
      F.ewing_h[d] = p->level_dx ? mf.dx[d] : mc.dx[d];
   }
   F.tranwt = (double)(1.0f / (float)(1 + 2));  // REAL quotient in the reference
   F.longwt = 2 * F.tranwt;
   const ampe_fac2_level_t* src[2] = {lc, lf};
   FacLevel* dst[2] = {&F.c, &F.f};
   for (int l = 0; l < 2; l++) {
      for (int d = 0; d < 3; d++) dst[l]->D[d] = src[l] ? src[l]->D[d] : nullptr;
      dst[l]->C = src[l] ? src[l]->C : nullptr;
      dst[l]->M = src[l] ? src[l]->M : nullptr;
      dst[l]->dc = p->d_const;
      dst[l]->cc = p->c_const;
      dst[l]->mc = p->m_const;
      for (int d = 0; d < 3; d++) dst[l]->dx[d] = l ? mf.dx[d] : mc.dx[d];
   }
   F.dvc = mc.dx[0] * mc.dx[1] * mc.dx[2];
   F.dvf = mf.dx[0] * mf.dx[1] * mf.dx[2];
   // the sum of the weights: fine cells, and coarse cells outside the box
   const long long under = (long long)p->nbox[0] * p->nbox[1] * p->nbox[2];
   F.den = (double)F.gf.cells() * F.dvf + (double)(F.gc.cells() - under) * F.dvc;
   return AMPE_OK;
}

long long work_doubles(const Fac2& F)
{
   return 2 * F.gc.cells_ghost() + 3 * F.gf.cells_ghost() + faces_of(F.gc) + faces_of(F.gf) +
          kNormBlocks;
}

void carve(Fac2& F, double* w)
{
   F.ec = w;
   w += F.gc.cells_ghost();
   F.rcw = w;
   w += F.gc.cells_ghost();
   F.ef = w;
   w += F.gf.cells_ghost();
   F.rfw = w;
   w += F.gf.cells_ghost();
   F.tf = w;
   w += F.gf.cells_ghost();
   const long long fcn[3] = {F.gc.nfx(), F.gc.nfy(), F.gc.nfz()};
   const long long ffn[3] = {F.gf.nfx(), F.gf.nfy(), F.gf.nfz()};
   for (int d = 0; d < 3; d++) {
      F.fc[d] = w;
      w += fcn[d];
   }
   for (int d = 0; d < 3; d++) {
      F.ff[d] = w;
      w += ffn[d];
   }
   F.part = w;
}

void cf_fill(Fac2& F, const double* uc, double* uf)
{
   k_cf_fill<<<nblk(F.gf.cells_ghost()), 256, 0, F.s>>>(F.gc, F.gf, F.b, uc, uf);
}

void flux_fine(Fac2& F, const double* u)
{
   k_comp_flux<<<nblk(faces_of(F.gf)), 256, 0, F.s>>>(F.gf, F.f, F.flux_dinv_f[0],
                                                       F.flux_dinv_f[1], F.flux_dinv_f[2], u,
                                                       F.ff[0], F.ff[1], F.ff[2]);
   const long long nb = 2LL * (F.gf.n1 * (long long)F.gf.n2 + F.gf.n0 * (long long)F.gf.n2 +
                               F.gf.n0 * (long long)F.gf.n1);
   k_ewing<<<nblk(nb), 256, 0, F.s>>>(F.gf, F.f, F.ewing_h[0], F.ewing_h[1], F.ewing_h[2],
                                      F.tranwt, F.longwt, u, F.ff[0], F.ff[1], F.ff[2]);
}

void flux_coarse(Fac2& F, const double* u)
{
   k_comp_flux<<<nblk(faces_of(F.gc)), 256, 0, F.s>>>(F.gc, F.c, F.flux_dinv_c[0],
                                                       F.flux_dinv_c[1], F.flux_dinv_c[2], u,
                                                       F.fc[0], F.fc[1], F.fc[2]);
}

void restrict_cells(Fac2& F, const double* vf, double* vc)
{
   k_restrict<<<nblk((long long)F.b.nb[0] * F.b.nb[1] * F.b.nb[2]), 256, 0, F.s>>>(
       F.gc, F.gf, F.b, F.dvf, F.dvc, vf, vc);
}

void smooth(Fac2& F, bool fine, double* e, const double* r, int sweeps)
{
   const Grid& g = fine ? F.gf : F.gc;
   if (fine)
      cf_fill(F, F.ec, e);
   else
      fill_ghosts(g, e, F.s);
   for (int sw = 0; sw < sweeps; sw++)
      for (int off = 0; off < 2; off++) {
         double* const* fl;
         if (fine) {
            flux_fine(F, e);
            fl = F.ff;
         } else {
            fill_ghosts(g, e, F.s);
            flux_coarse(F, e);
            fl = F.fc;
         }
         k_rbgs_flux<<<nblk(g.cells()), 256, 0, F.s>>>(g, fine ? F.f : F.c, fl[0], fl[1], fl[2],
                                                      r, e, off);
      }
   if (!fine) fill_ghosts(g, e, F.s);
}

int norm_of(Fac2& F, const double* rc, const double* rf, double* out)
{
   k_wnorm<<<kNormBlocks, 256, 0, F.s>>>(F.gc, F.gf, F.b, F.dvc, F.dvf, rc, rf, F.part);
   std::vector<double> h(kNormBlocks);
   if (cudaMemcpyAsync(h.data(), F.part, kNormBlocks * sizeof(double), cudaMemcpyDeviceToHost,
                       F.s) != cudaSuccess ||
       cudaStreamSynchronize(F.s) != cudaSuccess)
      return AMPE_ERR_CUDA;
   double num = 0.0;
   for (double v : h) num += v;
   *out = std::sqrt(num / F.den);
   return AMPE_OK;
}

int composite_residual(Fac2& F, const double* fcr, const double* ffr, double* uc, double* uf,
                       double* rc, double* rf, double* norm)
{
   cf_fill(F, uc, uf);
   flux_fine(F, uf);
   k_comp_res<<<nblk(F.gf.cells()), 256, 0, F.s>>>(F.gf, F.f, F.ff[0], F.ff[1], F.ff[2], uf,
                                                   ffr, rf);
   restrict_cells(F, uf, uc);
   fill_ghosts(F.gc, uc, F.s);
   flux_coarse(F, uc);
   const double* dxf = F.f.dx;
   const double* dxc = F.c.dx;
   k_coarsen_flux<<<nblk(2 * (F.b.nb[1] * F.b.nb[2] + F.b.nb[0] * F.b.nb[2] +
                              F.b.nb[0] * F.b.nb[1])),
                    256, 0, F.s>>>(F.gc, F.gf, F.b, dxf[1] * dxf[2], dxf[0] * dxf[2],
                                   dxf[0] * dxf[1], dxc[1] * dxc[2], dxc[0] * dxc[2],
                                   dxc[0] * dxc[1], F.ff[0], F.ff[1], F.ff[2], F.fc[0], F.fc[1],
                                   F.fc[2]);
   k_comp_res<<<nblk(F.gc.cells()), 256, 0, F.s>>>(F.gc, F.c, F.fc[0], F.fc[1], F.fc[2], uc,
                                                   fcr, rc);
   restrict_cells(F, rf, rc);
   int rcode = launch_status();
   if (rcode) return rcode;
   return norm ? norm_of(F, rc, rf, norm) : AMPE_OK;
}

}  // namespace

}  // namespace ampe

using namespace ampe;

extern "C" {

long long ampe_fac2_work_doubles(const ampe_fac2_t* p)
{
   Fac2 F;
   if (setup(F, p, nullptr, nullptr)) return AMPE_ERR_INVALID;
   return work_doubles(F);
}

int ampe_fac2_composite_residual(const ampe_fac2_t* p, const ampe_fac2_level_t* coarse,
                                 const ampe_fac2_level_t* fine, const double* fc,
                                 const double* ff, double* uc, double* uf, double* rc,
                                 double* rf, double* work, double* norm, void* stream)
{
   Fac2 F;
   int e = setup(F, p, coarse, fine);
   if (e) return e;
   if (!fc || !ff || !uc || !uf || !rc || !rf || !work) return AMPE_ERR_INVALID;
   F.s = (cudaStream_t)stream;
   carve(F, work);
   return composite_residual(F, fc, ff, uc, uf, rc, rf, norm);
}

int ampe_fac2_solve(const ampe_fac2_t* p, const ampe_fac2_level_t* coarse,
                    const ampe_fac2_level_t* fine, const double* fc, const double* ff,
                    double* uc, double* uf, int max_cycles, double tol, double* work,
                    double* norms, void* stream)
{
   Fac2 F;
   int e = setup(F, p, coarse, fine);
   if (e) return e;
   if (!fc || !ff || !uc || !uf || !work || max_cycles < 0) return AMPE_ERR_INVALID;
   F.s = (cudaStream_t)stream;
   carve(F, work);
   double norm = 0.0;
   if ((e = composite_residual(F, fc, ff, uc, uf, F.rcw, F.rfw, &norm))) return e;
   if (norms) norms[0] = norm;
   int it = 0;
   const size_t bc = F.gc.cells_ghost() * sizeof(double), bf = F.gf.cells_ghost() * sizeof(double);
   while (it < max_cycles && !(norm <= tol)) {
      if (cudaMemsetAsync(F.ec, 0, bc, F.s) != cudaSuccess ||
          cudaMemsetAsync(F.ef, 0, bf, F.s) != cudaSuccess)
         return AMPE_ERR_CUDA;
      // facCycle_Recursive: fine presmoothing, fine residual restricted into
      // the coarse right-hand side, coarse sweeps, prolongation, postsmoothing
      smooth(F, true, F.ef, F.rfw, p->presweeps);
      cf_fill(F, F.ec, F.ef);
      flux_fine(F, F.ef);
      k_comp_res<<<nblk(F.gf.cells()), 256, 0, F.s>>>(F.gf, F.f, F.ff[0], F.ff[1], F.ff[2],
                                                      F.ef, F.rfw, F.tf);
      restrict_cells(F, F.tf, F.rcw);
      smooth(F, false, F.ec, F.rcw, p->coarse_sweeps);
      k_prolong_add<<<nblk(F.gf.cells()), 256, 0, F.s>>>(F.gc, F.gf, F.b, F.ec, F.ef);
      smooth(F, true, F.ef, F.rfw, p->postsweeps);
      k_add_interior<<<nblk(F.gc.cells()), 256, 0, F.s>>>(F.gc, F.ec, uc);
      k_add_interior<<<nblk(F.gf.cells()), 256, 0, F.s>>>(F.gf, F.ef, uf);
      restrict_cells(F, uf, uc);
      if ((e = composite_residual(F, fc, ff, uc, uf, F.rcw, F.rfw, &norm))) return e;
      it++;
      if (norms) norms[it] = norm;
   }
   return it;
}

}  // extern "C"
