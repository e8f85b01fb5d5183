// FAC operator kernels: red-black Gauss-Seidel colour update, residual and
// the phase operator's C coefficient (EllipticFACOps / PhaseFACOps,
// 3d/ellipticfacops.m4:16-575).  Operator  A u = C u + M div(D grad u);
// cell arrays ghosted (width g.ng), face D arrays ghost-free.
// Templated on the arithmetic type R so that the mixed-precision
// preconditioner runs the same code in FP32.
#include <type_traits>

#include "common.cuh"
#include "devvec.cuh"
#include "fac.cuh"

namespace ampe {

template <class R>
__device__ __forceinline__ R face_d(const FacOp<R>& op, const Grid& g,
                                    int dir, int i, int j, int k)
{
   if (!op.D0) return op.dc;
   if (dir == 0) return op.D0[g.fx(i, j, k)];
   if (dir == 1) return op.D1[g.fy(i, j, k)];
   return op.D2[g.fz(i, j, k)];
}

// r = f - A u at (i,j,k) and 1/(M sum D/h^2 - C) (expression order of
// efo_rbgswithfluxmaxvardcvarsf3d, 3d/ellipticfacops.m4:153-172)
template <class R>
__device__ __forceinline__ R cell_residual(const FacOp<R>& op, const Grid& g,
                                           const R* f, const R* u, int i,
                                           int j, int k, R* dudr)
{
   const long long c = g.c(i, j, k);
   const R uc = u[c];
   R div = R(0), dsum = R(0);
#pragma unroll
   for (int d = 0; d < 3; d++) {
      if (d >= g.dim) break;
      const int ei = d == 0, ej = d == 1, ek = d == 2;
      const R dxi = op.dxi[d];
      const R Dm = face_d(op, g, d, i, j, k);
      const R Dp = face_d(op, g, d, i + ei, j + ej, k + ek);
      const R fm = dxi * Dm * (uc - u[g.c(i - ei, j - ej, k - ek)]);
      const R fp = dxi * Dp * (u[g.c(i + ei, j + ej, k + ek)] - uc);
      div += dxi * (fp - fm);
      dsum += dxi * dxi * (Dp + Dm);
   }
   const R M = op.M ? op.M[c] : op.mc;
   const R C = op.C ? op.C[c] : op.cc;
   if (dudr) *dudr = R(1) / (M * dsum - C);
   return f[c] - M * div - C * uc;
}

// cell_residual specialised on the dimension and on which coefficients are
// arrays (HD: face D, HC: cell C, HM: cell M); c = g.c(i,j,k).  Neighbours
// and upper faces by their constant offsets.  Same expression order as
// cell_residual.
// U(index, di, dj, dk) loads u at the neighbour (di, dj, dk) of the cell.
template <class R, int DIM, bool HD, bool HC, bool HM, class UL>
__device__ __forceinline__ R op_residual_u(const FacOp<R>& op, const Grid& g,
                                           const R* __restrict__ f, const UL& U, int i,
                                           int j, int k, int c, R* dudr)
{
   const R uc = U(c, 0, 0, 0);
   R div = R(0), dsum = R(0);
   {
      const R dxi = op.dxi[0];
      R Dm = op.dc, Dp = op.dc;
      if (HD) {
         const int fi = g.fx(i, j, k);
         Dm = op.D0[fi];
         Dp = op.D0[fi + 1];
      }
      const R fm = dxi * Dm * (uc - U(c - 1, -1, 0, 0));
      const R fp = dxi * Dp * (U(c + 1, 1, 0, 0) - uc);
      div += dxi * (fp - fm);
      dsum += dxi * dxi * (Dp + Dm);
   }
   {
      const R dxi = op.dxi[1];
      R Dm = op.dc, Dp = op.dc;
      if (HD) {
         const int fi = g.fy(i, j, k);
         Dm = op.D1[fi];
         Dp = op.D1[fi + g.fys()];
      }
      const R fm = dxi * Dm * (uc - U(c - g.sx, 0, -1, 0));
      const R fp = dxi * Dp * (U(c + g.sx, 0, 1, 0) - uc);
      div += dxi * (fp - fm);
      dsum += dxi * dxi * (Dp + Dm);
   }
   if (DIM == 3) {
      const R dxi = op.dxi[2];
      R Dm = op.dc, Dp = op.dc;
      if (HD) {
         const int fi = g.fz(i, j, k);
         Dm = op.D2[fi];
         Dp = op.D2[fi + g.fzs()];
      }
      const R fm = dxi * Dm * (uc - U(c - g.sy, 0, 0, -1));
      const R fp = dxi * Dp * (U(c + g.sy, 0, 0, 1) - uc);
      div += dxi * (fp - fm);
      dsum += dxi * dxi * (Dp + Dm);
   }
   const R M = HM ? op.M[c] : op.mc;
   const R C = HC ? op.C[c] : op.cc;
   if (dudr) *dudr = R(1) / (M * dsum - C);
   const R fv = op.f_interior ? f[g.interior(i, j, k)] : f[c];
   return fv - M * div - C * uc;
}

template <class R>
struct PlainU {
   const R* u;
   __device__ __forceinline__ R operator()(int c, int, int, int) const { return u[c]; }
};

template <class R, int DIM, bool HD, bool HC, bool HM>
__device__ __forceinline__ R op_residual(const FacOp<R>& op, const Grid& g,
                                         const R* __restrict__ f, const R* u, int i,
                                         int j, int k, int c, R* dudr)
{
   return op_residual_u<R, DIM, HD, HC, HM>(op, g, f, PlainU<R>{u}, i, j, k, c, dudr);
}

// u plus the piecewise-constant coarse correction e of the next coarser
// level (coarse ghosts current), at the cell and, with NB, at its
// neighbours: the value k_prolong_add would have stored there
template <class R, bool NB>
struct ProlongU {
   const R* u;
   const R* e;
   Grid gc;
   int i, j, k, zs;
   __device__ __forceinline__ R operator()(int c, int di, int dj, int dk) const
   {
      const R v = u[c];
      if (!NB && (di | dj | dk)) return v;
      return v + e[gc.c((i + di) >> 1, (j + dj) >> 1, (k + dk) >> zs)];
   }
};

// call F<DIM, HD, HC, HM>() for the operator's shape
template <class R, class F>
void dispatch_op(const FacOp<R>& op, int dim, F&& fn)
{
   const bool hd = op.D0 != nullptr, hc = op.C != nullptr, hm = op.M != nullptr;
#define AMPE_OP_CASE(D, A, B, C_)                                               \
   if (dim == D && hd == A && hc == B && hm == C_) {                            \
      fn(std::integral_constant<int, D>(), std::integral_constant<bool, A>(),   \
         std::integral_constant<bool, B>(), std::integral_constant<bool, C_>()); \
      return;                                                                  \
   }
   AMPE_OP_CASE(3, false, true, false)  // phase block
   AMPE_OP_CASE(3, true, false, false)  // composition block
   AMPE_OP_CASE(3, true, false, true)   // quaternion block
   AMPE_OP_CASE(2, false, true, false)
   AMPE_OP_CASE(2, true, false, false)
   AMPE_OP_CASE(2, true, false, true)
   AMPE_OP_CASE(3, false, false, false)
   AMPE_OP_CASE(3, false, false, true)
   AMPE_OP_CASE(3, false, true, true)
   AMPE_OP_CASE(3, true, true, false)
   AMPE_OP_CASE(3, true, true, true)
   AMPE_OP_CASE(2, false, false, false)
   AMPE_OP_CASE(2, false, false, true)
   AMPE_OP_CASE(2, false, true, true)
   AMPE_OP_CASE(2, true, true, false)
   AMPE_OP_CASE(2, true, true, true)
#undef AMPE_OP_CASE
}

__device__ __forceinline__ void atomic_max_nonneg(double* a, double v)
{
   atomicMax((unsigned long long*)a, (unsigned long long)__double_as_longlong(v));
}

// periodic ghost fill as a gather: every ghost cell copies its wrapped
// interior source (the same values as a SAMRAI periodic fill).  Threads run
// over the ghost layers only: z slabs, then y slabs, then x columns.
template <class R>
__global__ void k_fill_ghosts_gather(Grid g, R* f)
{
   const int ng = g.ng;
   const long long SX = g.n0 + 2 * ng, SY = g.n1 + 2 * ng;
   const long long nzs = 2LL * g.gz * SX * SY;
   const long long nys = (long long)g.n2 * 2 * ng * SX;
   const long long nxs = (long long)g.n2 * g.n1 * 2 * ng;
   for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
        t < nzs + nys + nxs; t += (long long)gridDim.x * blockDim.x) {
      int i, j, k;
      long long r = t;
      if (r < nzs) {
         i = (int)(r % SX) - ng;
         r /= SX;
         j = (int)(r % SY) - ng;
         const int l = (int)(r / SY);
         k = l < g.gz ? l - g.gz : g.n2 + l - g.gz;
      } else if ((r -= nzs) < nys) {
         i = (int)(r % SX) - ng;
         r /= SX;
         const int l = (int)(r % (2 * ng));
         j = l < ng ? l - ng : g.n1 + l - ng;
         k = (int)(r / (2 * ng));
      } else {
         r -= nys;
         const int l = (int)(r % (2 * ng));
         i = l < ng ? l - ng : g.n0 + l - ng;
         r /= 2 * ng;
         k = (int)g.fd1.div((unsigned)r);
         j = (int)r - k * g.n1;
      }
      const int si = i < 0 ? i + g.n0 : (i >= g.n0 ? i - g.n0 : i);
      const int sj = j < 0 ? j + g.n1 : (j >= g.n1 ? j - g.n1 : j);
      const int sk = k < 0 ? k + g.n2 : (k >= g.n2 ? k - g.n2 : k);
      f[g.c(i, j, k)] = f[g.c(si, sj, sk)];
   }
}

template <class R>
int fill_ghosts_t(const Grid& g, R* f, cudaStream_t s)
{
   const long long SX = g.n0 + 2 * g.ng, SY = g.n1 + 2 * g.ng;
   const long long tot = 2LL * g.gz * SX * SY + (long long)g.n2 * 2 * g.ng * SX +
                         (long long)g.n2 * g.n1 * 2 * g.ng;
   long long b = (tot + 255) / 256;
   if (b > max_blocks()) b = max_blocks();
   k_fill_ghosts_gather<R><<<(unsigned)(b < 1 ? 1 : b), 256, 0, s>>>(g, f);
   return launch_status();
}

// One colour of the red-black sweep.  images: also write each updated value
// to its periodic ghost images, so that no ghost fill is needed between
// colours (the stepper's smoother); the leaf entry point updates the
// interior only.
template <class R, int DIM, bool HD, bool HC, bool HM>
__global__ void __launch_bounds__(256)
    k_rbgs_color(FacOp<R> op, Grid g, const R* __restrict__ f, R* u, int offset,
                 double* maxres, bool images)
{
   // one thread per cell of the colour, i = 2*ih + parity(j,k): every cell's
   // loads are in flight at once (no grid-stride loop that would serialise
   // them behind the in-place stores)
   const int nh = (g.n0 + 1) / 2;
   const long long tot = (long long)nh * g.n1 * g.n2;
   R mres = R(0);
   const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
   if (t < tot) {
      int ih, j, k;
      g.split(t, g.fdh, g.fd1, ih, j, k);
      const int i = 2 * ih + ((j + k + offset) & 1);
      if (i < g.n0) {
         R dudr;
         const int c = g.c(i, j, k);
         const R r = op_residual<R, DIM, HD, HC, HM>(op, g, f, u, i, j, k, c, &dudr);
         const R un = u[c] + -r * dudr;
         u[c] = un;
         if (images) for_each_image(g, i, j, k, [&](long long idx) { u[idx] = un; });
         if (maxres) mres = fmax(mres, fabs(r));
      }
   }
   if (maxres) {
      double mr = (double)mres;
      for (int o = 16; o > 0; o >>= 1)
         mr = fmax(mr, __shfl_xor_sync(0xffffffffu, mr, o));
      if ((threadIdx.x & 31) == 0) atomic_max_nonneg(maxres, mr);
   }
}

// One colour of the first post-smoothing sweep with the prolongation of the
// coarse correction e fused in (u += e is never stored separately): the red
// pass reads u + e at the cell and its black neighbours, the black pass at
// the cell (its red neighbours already hold their final values).  Every
// value equals the one k_prolong_add followed by k_rbgs_color computes.
template <class R, int DIM, bool HD, bool HC, bool HM, bool RED>
__global__ void __launch_bounds__(256)
    k_rbgs_color_prolong(FacOp<R> op, Grid g, const R* __restrict__ f, R* u,
                         Grid gc, const R* __restrict__ e)
{
   const int nh = (g.n0 + 1) / 2;
   const long long tot = (long long)nh * g.n1 * g.n2;
   const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
   if (t >= tot) return;
   int ih, j, k;
   g.split(t, g.fdh, g.fd1, ih, j, k);
   const int i = 2 * ih + ((j + k + (RED ? 0 : 1)) & 1);
   if (i >= g.n0) return;
   R dudr;
   const int c = g.c(i, j, k);
   const ProlongU<R, RED> U{u, e, gc, i, j, k, DIM == 3 ? 1 : 0};
   const R r = op_residual_u<R, DIM, HD, HC, HM>(op, g, f, U, i, j, k, c, &dudr);
   const R un = U(c, 0, 0, 0) + -r * dudr;
   u[c] = un;
   for_each_image(g, i, j, k, [&](long long idx) { u[idx] = un; });
}

// ---------------------------------------------------------------------------
// One whole red-black sweep (red, then black) in one launch.
//
// Each block owns a box of cells (32 x 8 x 4 in 3D, 32 x 16 in 2D).  It
// stages u over the box plus a halo of two cells, and f, C, M over the box
// plus one, in shared memory with dense coalesced loads; updates the red
// cells of the box plus its halo of one (neighbouring blocks repeat those
// halo updates on identical inputs), then the black cells of the box, and
// writes the box to uout with its periodic ghost images.  u is read from uin
// and written to uout, so no block reads values another block has written
// and the result is the two colour passes' result, bit for bit: every update
// evaluates cell_residual's expression in the same order.  Colours follow
// (i + j + k) % 2 of the interior index, which requires even extents.
// ---------------------------------------------------------------------------
template <int DIM>
struct SweepBox {
   static constexpr int TX = 32, TY = DIM == 3 ? 8 : 16, TZ = DIM == 3 ? 4 : 1;
   static constexpr int BX = TX + 4, BY = TY + 4, BZ = DIM == 3 ? TZ + 4 : 1;  // u, halo 2
   static constexpr int CX = TX + 2, CY = TY + 2, CZ = DIM == 3 ? TZ + 2 : 1;  // halo 1
   static constexpr int NU = BX * BY * BZ, NC = CX * CY * CZ;
};

template <class R>
size_t rb_sweep_smem(const FacOp<R>& op, int dim)
{
   const int nu = dim == 3 ? SweepBox<3>::NU : SweepBox<2>::NU;
   const int nc = dim == 3 ? SweepBox<3>::NC : SweepBox<2>::NC;
   return sizeof(R) * (size_t)(nu + nc * (1 + (op.C ? 1 : 0) + (op.M ? 1 : 0)));
}

// periodic wrap of an index a >= -2 into [0, n); extents below the halo
// reach take the modulo
__device__ __forceinline__ int wrap_idx(int a, int n)
{
   return a < 0 ? (a + n) % n : (a >= n ? (a - n < n ? a - n : a % n) : a);
}

// blockDim (32, 8): lane x along rows, warp y over rows
template <class R, int DIM, bool ZERO>
__global__ void __launch_bounds__(256)
    k_rb_sweep(FacOp<R> op, Grid g, const R* __restrict__ f, const R* __restrict__ uin,
               R* __restrict__ uout)
{
   using B = SweepBox<DIM>;
   extern __shared__ __align__(16) unsigned char sweep_smem[];
   R* U = (R*)sweep_smem;
   R* Fs = U + B::NU;
   R* Cs = Fs + B::NC;
   R* Ms = Cs + (op.C ? B::NC : 0);
   const int tx = threadIdx.x, ty = threadIdx.y;
   const int i0 = blockIdx.x * B::TX, j0 = blockIdx.y * B::TY, k0 = blockIdx.z * B::TZ;
   const int pitch_z = g.sy, pitch_y = g.sx;
   // address of cell (i, 0, 0) minus i for row (j, k): c = rowc + i
   auto rowc = [&](int j, int k) { return g.c(0, j, k); };
   const int ia = wrap_idx(i0 + tx - 2, g.n0);            // x of lane tx in the u box
   const int ib = tx < 4 ? wrap_idx(i0 + tx + 30, g.n0) : 0;  // x of lane tx + 32
   const int ic = wrap_idx(i0 + tx - 1, g.n0);            // x of lane tx in the f box
   const int id = tx < 2 ? wrap_idx(i0 + tx + 31, g.n0) : 0;
   (void)pitch_z;
   (void)pitch_y;
   if (!ZERO) {
      for (int z = 0; z < B::BZ; z++) {
         const int kw = DIM == 3 ? wrap_idx(k0 + z - 2, g.n2) : 0;
         for (int y = ty; y < B::BY; y += 8) {
            const int rc = rowc(wrap_idx(j0 + y - 2, g.n1), kw);
            R* dst = U + (z * B::BY + y) * B::BX;
            dst[tx] = uin[rc + ia];
            if (tx < 4) dst[tx + 32] = uin[rc + ib];
         }
      }
   } else {
      for (int p = ty * 32 + tx; p < B::NU; p += 256) U[p] = R(0);
   }
   for (int z = 0; z < B::CZ; z++) {
      const int kw = DIM == 3 ? wrap_idx(k0 + z - 1, g.n2) : 0;
      for (int y = ty; y < B::CY; y += 8) {
         const int rc = rowc(wrap_idx(j0 + y - 1, g.n1), kw);
         const int o = (z * B::CY + y) * B::CX;
         Fs[o + tx] = f[rc + ic];
         if (tx < 2) Fs[o + tx + 32] = f[rc + id];
         if (op.C) {
            Cs[o + tx] = op.C[rc + ic];
            if (tx < 2) Cs[o + tx + 32] = op.C[rc + id];
         }
         if (op.M) {
            Ms[o + tx] = op.M[rc + ic];
            if (tx < 2) Ms[o + tx + 32] = op.M[rc + id];
         }
      }
   }
   __syncthreads();
   // one colour on the u-box rows [lo, hiy) x [lo, hiz) (3D), lanes along x
   auto colour = [&](int col, int lo, int nxh, int hiy, int hiz) {
      const int zlo = DIM == 3 ? lo : 0, zhi = DIM == 3 ? hiz : 1;
      const int ny = hiy - lo;
      for (int rr = ty; rr < ny * (zhi - zlo); rr += 8) {
         const int z = zlo + rr / ny, y = lo + rr % ny;
         if (tx >= nxh) continue;
         const int jg = j0 + y - 2, kg = DIM == 3 ? k0 + z - 2 : 0;
         const int q = (col + i0 + jg + kg) & 1;  // parity of x for this colour
         const int x = lo + ((q + lo) & 1) + 2 * tx;
         const int u0 = (z * B::BY + y) * B::BX + x;
         const int c0 = ((DIM == 3 ? z - 1 : 0) * B::CY + (y - 1)) * B::CX + (x - 1);
         const R uc = U[u0];
         R div = R(0), dsum = R(0);
         int iw = 0, jw = 0, kw = 0;
         if (op.D0) {
            iw = wrap_idx(i0 + x - 2, g.n0);
            jw = wrap_idx(jg, g.n1);
            kw = DIM == 3 ? wrap_idx(kg, g.n2) : 0;
         }
         {
            const R dxi = op.dxi[0];
            const R Dm = op.D0 ? op.D0[g.fx(iw, jw, kw)] : op.dc;
            const R Dp = op.D0 ? op.D0[g.fx(iw + 1, jw, kw)] : op.dc;
            const R fm = dxi * Dm * (uc - U[u0 - 1]);
            const R fp = dxi * Dp * (U[u0 + 1] - uc);
            div += dxi * (fp - fm);
            dsum += dxi * dxi * (Dp + Dm);
         }
         {
            const R dxi = op.dxi[1];
            const R Dm = op.D0 ? op.D1[g.fy(iw, jw, kw)] : op.dc;
            const R Dp = op.D0 ? op.D1[g.fy(iw, jw + 1, kw)] : op.dc;
            const R fm = dxi * Dm * (uc - U[u0 - B::BX]);
            const R fp = dxi * Dp * (U[u0 + B::BX] - uc);
            div += dxi * (fp - fm);
            dsum += dxi * dxi * (Dp + Dm);
         }
         if (DIM == 3) {
            const R dxi = op.dxi[2];
            const R Dm = op.D0 ? op.D2[g.fz(iw, jw, kw)] : op.dc;
            const R Dp = op.D0 ? op.D2[g.fz(iw, jw, kw + 1)] : op.dc;
            const R fm = dxi * Dm * (uc - U[u0 - B::BX * B::BY]);
            const R fp = dxi * Dp * (U[u0 + B::BX * B::BY] - uc);
            div += dxi * (fp - fm);
            dsum += dxi * dxi * (Dp + Dm);
         }
         const R M = op.M ? Ms[c0] : op.mc;
         const R C = op.C ? Cs[c0] : op.cc;
         const R dudr = R(1) / (M * dsum - C);
         const R r = Fs[c0] - M * div - C * uc;
         U[u0] = uc + -r * dudr;
      }
   };
   colour(0, 1, B::CX / 2, B::BY - 1, B::BZ - 1);  // red: box + halo 1
   __syncthreads();
   colour(1, 2, B::TX / 2, B::BY - 2, B::BZ - 2);  // black: the box
   __syncthreads();
   const int i = i0 + tx;
   if (i >= g.n0) return;
   for (int zz = 0; zz < B::TZ; zz++) {
      const int k = k0 + zz;
      if (DIM == 3 && k >= g.n2) break;
      for (int yy = ty; yy < B::TY; yy += 8) {
         const int j = j0 + yy;
         if (j >= g.n1) break;
         const R v = U[((DIM == 3 ? zz + 2 : 0) * B::BY + yy + 2) * B::BX + tx + 2];
         uout[g.c(i, j, k)] = v;
         for_each_image(g, i, j, k, [&](long long idx) { uout[idx] = v; });
      }
   }
}

template <class R>
bool rb_sweep_fusable(const Grid& g)
{
   return g.n0 % 2 == 0 && g.n1 % 2 == 0 && (g.dim == 2 || g.n2 % 2 == 0) && g.n0 >= 4 &&
          g.n1 >= 4 && (g.dim == 2 || g.n2 >= 4);
}

template <class R, int DIM, bool ZERO>
static int launch_sweep(const FacOp<R>& op, const Grid& g, const R* f, const R* uin, R* uout,
                        cudaStream_t s)
{
   using B = SweepBox<DIM>;
   const size_t smem = rb_sweep_smem(op, DIM);
   // opt in to more than 48 KB once per instantiation and device
   static std::atomic<unsigned long long> attr{0};
   if (first_on_device(attr)) {
      const int most = (int)(sizeof(R) * (size_t)(B::NU + 3 * B::NC));  // f, C and M staged
      cudaFuncSetAttribute(k_rb_sweep<R, DIM, ZERO>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           most);
   }
   const dim3 grid((g.n0 + B::TX - 1) / B::TX, (g.n1 + B::TY - 1) / B::TY,
                   DIM == 3 ? (g.n2 + B::TZ - 1) / B::TZ : 1);
   k_rb_sweep<R, DIM, ZERO><<<grid, dim3(32, 8), smem, s>>>(op, g, f, uin, uout);
   return launch_status();
}

template <class R>
int rb_sweep_fused(const FacOp<R>& op, const Grid& g, const R* f, const R* uin, R* uout,
                   cudaStream_t s)
{
   if (op.f_interior) return AMPE_ERR_INVALID;  // stages f with ghosted indexing
   if (g.dim == 3)
      return uin ? launch_sweep<R, 3, false>(op, g, f, uin, uout, s)
                 : launch_sweep<R, 3, true>(op, g, f, uin, uout, s);
   return uin ? launch_sweep<R, 2, false>(op, g, f, uin, uout, s)
              : launch_sweep<R, 2, true>(op, g, f, uin, uout, s);
}

// res = f - A u and part[block] = sum over the block's cells of res^2
// (fixed grid, fixed order: deterministic with the finishing pass)
template <class R, int DIM, bool HD, bool HC, bool HM>
__global__ void k_residual_part(FacOp<R> op, Grid g, const R* __restrict__ f,
                                const R* __restrict__ u, R* __restrict__ res, double* part,
                                R* __restrict__ z)
{
   __shared__ double sh[32];
   R accr = R(0);  // per-thread sum in R (FP32 in the mixed path)
#pragma unroll 4
   for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
        t < g.cells(); t += (long long)gridDim.x * blockDim.x) {
      int i, j, k;
      g.ijk(t, i, j, k);
      const int c = g.c(i, j, k);
      const R r = op_residual<R, DIM, HD, HC, HM>(op, g, f, u, i, j, k, c, (R*)nullptr);
      if (res) res[t] = r;
      if (z) z[t] = u[c];
      accr += r * r;
   }
   double acc = block_sum<NoOp>((double)accr, sh);
   if (threadIdx.x == 0) part[blockIdx.x] = acc;
}

template <class R, int DIM, bool HD, bool HC, bool HM>
__global__ void k_residual(FacOp<R> op, Grid g, const R* __restrict__ f,
                           const R* __restrict__ u, R* __restrict__ res)
{
   for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
        t < g.cells(); t += (long long)gridDim.x * blockDim.x) {
      int i, j, k;
      g.ijk(t, i, j, k);
      const int c = g.c(i, j, k);
      res[c] = op_residual<R, DIM, HD, HC, HM>(op, g, f, u, i, j, k, c, (R*)nullptr);
   }
}

template <class R>
__global__ void k_phase_set_c(Grid g, const double* phi, double gamma,
                              double mobility, double well_scale, char wt,
                              R* ccell)
{
   for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
        t < g.cells(); t += (long long)gridDim.x * blockDim.x) {
      int i, j, k;
      g.ijk(t, i, j, k);
      const long long c = g.c(i, j, k);
      const double g2 = second_deriv_well_func(phi[c], wt);
      const double gm = gamma * mobility;
      ccell[c] = (R)(1.0 + gm * well_scale * g2);
   }
}

static unsigned nblocks(long long n)
{
   long long b = (n + 255) / 256;
   if (b > max_blocks()) b = max_blocks();
   return (unsigned)(b < 1 ? 1 : b);
}

template <class R>
int rbgs_color(const FacOp<R>& op, const Grid& g, const R* f, R* u,
               int offset, double* maxres, cudaStream_t s, bool images)
{
   const long long tot = (long long)((g.n0 + 1) / 2) * g.n1 * g.n2;
   const unsigned nb = (unsigned)((tot + 255) / 256);
   dispatch_op(op, g.dim, [&](auto D, auto HD, auto HC, auto HM) {
      k_rbgs_color<R, decltype(D)::value, decltype(HD)::value, decltype(HC)::value,
                   decltype(HM)::value><<<nb, 256, 0, s>>>(op, g, f, u, offset, maxres, images);
   });
   return launch_status();
}

template <class R>
int rbgs_color_prolong(const FacOp<R>& op, const Grid& g, const R* f, R* u, int offset,
                       const Grid& gc, const R* e, cudaStream_t s)
{
   const long long tot = (long long)((g.n0 + 1) / 2) * g.n1 * g.n2;
   const unsigned nb = (unsigned)((tot + 255) / 256);
   const bool hd = op.D0 != nullptr, hc = op.C != nullptr, hm = op.M != nullptr;
#define AMPE_PROL(D, A, B, C_)                                                          \
   if (g.dim == D && hd == A && hc == B && hm == C_) {                                   \
      if (offset == 0)                                                                  \
         k_rbgs_color_prolong<R, D, A, B, C_, true><<<nb, 256, 0, s>>>(op, g, f, u, gc, e);  \
      else                                                                              \
         k_rbgs_color_prolong<R, D, A, B, C_, false><<<nb, 256, 0, s>>>(op, g, f, u, gc, e); \
      return launch_status();                                                           \
   }
   AMPE_PROL(3, false, true, false)  // phase block
   AMPE_PROL(3, true, false, false)  // composition block
   AMPE_PROL(3, true, false, true)   // quaternion block
   AMPE_PROL(2, false, true, false)
   AMPE_PROL(2, true, false, false)
   AMPE_PROL(2, true, false, true)
#undef AMPE_PROL
   return AMPE_ERR_INVALID;
}

// coarse cell (ic,jc,kc): w * sum of the residuals of its 2^d children, in
// the order of k_restrict (z, then y, then x)
template <class R, int DIM, bool HD, bool HC, bool HM>
__global__ void k_residual_restrict(FacOp<R> op, Grid gf, Grid gc, const R* __restrict__ f,
                                    const R* __restrict__ u, R* __restrict__ fc)
{
   const R w = DIM == 3 ? R(0.125) : R(0.25);
   const int dz = DIM == 3 ? 2 : 1;
   for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < gc.cells();
        t += (long long)gridDim.x * blockDim.x) {
      int i, j, k;
      gc.ijk(t, i, j, k);
      R s = R(0);
      for (int cz = 0; cz < dz; cz++)
         for (int b = 0; b < 2; b++)
            for (int a = 0; a < 2; a++) {
               const int fi = 2 * i + a, fj = 2 * j + b, fk = dz * k + cz;
               s += op_residual<R, DIM, HD, HC, HM>(op, gf, f, u, fi, fj, fk,
                                                    gf.c(fi, fj, fk), (R*)nullptr);
            }
      fc[t] = w * s;
   }
}

template <class R>
int residual_restrict(const FacOp<R>& op, const Grid& gf, const Grid& gc, const R* f,
                      const R* u, R* fc, cudaStream_t s)
{
   const unsigned nb = (unsigned)((gc.cells() + 255) / 256);
   dispatch_op(op, gf.dim, [&](auto D, auto HD, auto HC, auto HM) {
      k_residual_restrict<R, decltype(D)::value, decltype(HD)::value, decltype(HC)::value,
                          decltype(HM)::value><<<nb, 256, 0, s>>>(op, gf, gc, f, u, fc);
   });
   return launch_status();
}

template <class R>
int residual_partial(const FacOp<R>& op, const Grid& g, const R* f, const R* u,
                     R* res, double* part, int* nblk, R* z, cudaStream_t s)
{
   const long long n = g.cells();
   long long nb = (n + kRedThreads - 1) / kRedThreads;
   const int blocks = (int)(nb < kRedBlocks ? (nb < 1 ? 1 : nb) : kRedBlocks);
   *nblk = blocks;
   dispatch_op(op, g.dim, [&](auto D, auto HD, auto HC, auto HM) {
      k_residual_part<R, decltype(D)::value, decltype(HD)::value, decltype(HC)::value,
                      decltype(HM)::value><<<blocks, kRedThreads, 0, s>>>(op, g, f, u, res,
                                                                         part, z);
   });
   return launch_status();
}

template <class R>
int residual(const FacOp<R>& op, const Grid& g, const R* f, const R* u,
             R* res, cudaStream_t s)
{
   const unsigned nb = (unsigned)((g.cells() + 255) / 256);
   dispatch_op(op, g.dim, [&](auto D, auto HD, auto HC, auto HM) {
      k_residual<R, decltype(D)::value, decltype(HD)::value, decltype(HC)::value,
                 decltype(HM)::value><<<nb, 256, 0, s>>>(op, g, f, u, res);
   });
   return launch_status();
}

template <class R>
int phase_set_c(const ampe_model_t& m, const Grid& g, const double* phi,
                double gamma, R* ccell, cudaStream_t s)
{
   k_phase_set_c<R><<<nblocks(g.cells()), 256, 0, s>>>(
       g, phi, gamma, m.phase_mobility, m.phase_well_scale, m.well_type,
       ccell);
   return launch_status();
}

template int rbgs_color<double>(const FacOp<double>&, const Grid&,
                                const double*, double*, int, double*,
                                cudaStream_t, bool);
template int rbgs_color<float>(const FacOp<float>&, const Grid&, const float*,
                               float*, int, double*, cudaStream_t, bool);
template int rbgs_color_prolong<double>(const FacOp<double>&, const Grid&, const double*,
                                        double*, int, const Grid&, const double*,
                                        cudaStream_t);
template int rbgs_color_prolong<float>(const FacOp<float>&, const Grid&, const float*, float*,
                                       int, const Grid&, const float*, cudaStream_t);
template int residual_partial<double>(const FacOp<double>&, const Grid&, const double*,
                                      const double*, double*, double*, int*, double*,
                                      cudaStream_t);
template int residual_partial<float>(const FacOp<float>&, const Grid&, const float*,
                                     const float*, float*, double*, int*, float*,
                                     cudaStream_t);
template int residual_restrict<double>(const FacOp<double>&, const Grid&, const Grid&,
                                       const double*, const double*, double*, cudaStream_t);
template int residual_restrict<float>(const FacOp<float>&, const Grid&, const Grid&,
                                      const float*, const float*, float*, cudaStream_t);
template int fill_ghosts_t<double>(const Grid&, double*, cudaStream_t);
template bool rb_sweep_fusable<double>(const Grid&);
template bool rb_sweep_fusable<float>(const Grid&);
template int rb_sweep_fused<double>(const FacOp<double>&, const Grid&, const double*,
                                    const double*, double*, cudaStream_t);
template int rb_sweep_fused<float>(const FacOp<float>&, const Grid&, const float*,
                                   const float*, float*, cudaStream_t);
template int fill_ghosts_t<float>(const Grid&, float*, cudaStream_t);
template int residual<double>(const FacOp<double>&, const Grid&, const double*,
                              const double*, double*, cudaStream_t);
template int residual<float>(const FacOp<float>&, const Grid&, const float*,
                             const float*, float*, cudaStream_t);
template int phase_set_c<double>(const ampe_model_t&, const Grid&,
                                 const double*, double, double*, cudaStream_t);
template int phase_set_c<float>(const ampe_model_t&, const Grid&,
                                const double*, double, float*, cudaStream_t);

// sum of squares of the interior of a ghosted field -> sqrt(sum / cells)
__global__ void k_rms_finish(const double* part, int np, double inv_cells,
                             double* out)
{
   __shared__ double sh[32];
   double acc = 0.0;
   for (int t = threadIdx.x; t < np; t += blockDim.x) acc += part[t];
   acc = block_sum<NoOp>(acc, sh);
   if (threadIdx.x == 0) *out = sqrt(acc * inv_cells);
}

long long residual_rms_scratch_doubles(const Grid& g)
{
   // residual field (ghost box), then kRedBlocks partial sums
   return g.cells_ghost() + kRedBlocks;
}

// res = f - A u into scratch, then its interior RMS into *rms (device);
// deterministic: fixed block count, fixed summation order.
int residual_rms_into(const FacOp<double>& op, const Grid& g, const double* f,
                      const double* u, double* scratch, double* rms,
                      cudaStream_t s)
{
   double* res = scratch;
   double* part = scratch + g.cells_ghost();
   int rc = residual(op, g, f, u, res, s);
   if (rc) return rc;
   const long long n = g.cells();
   long long nb = (n + kRedThreads - 1) / kRedThreads;
   const int blocks = (int)(nb < kRedBlocks ? (nb < 1 ? 1 : nb) : kRedBlocks);
   const Grid gg = g;
   auto sq = [=] __device__(long long t) {
      int i, j, k;
      gg.ijk(t, i, j, k);
      const double x = res[gg.c(i, j, k)];
      return x * x;
   };
   k_partial<<<blocks, kRedThreads, 0, s>>>(n, sq, part);
   g_launches++;
   k_rms_finish<<<1, 1024, 0, s>>>(part, blocks, 1.0 / (double)n, rms);
   return launch_status();
}

}  // namespace ampe

using namespace ampe;

static FacOp<double> make_op(const ampe_model_t* m, const double* d0,
                             const double* d1, const double* d2, double dc,
                             const double* cc, double cconst, const double* mm,
                             double mconst)
{
   FacOp<double> op;
   op.D0 = d0;
   op.D1 = d1;
   op.D2 = d2;
   op.dc = dc;
   op.C = cc;
   op.cc = cconst;
   op.M = mm;
   op.mc = mconst;
   for (int d = 0; d < 3; d++) op.dxi[d] = d < m->dim ? 1.0 / m->dx[d] : 0.0;
   return op;
}

extern "C" {

int ampe_efo_rbgs(const ampe_model_t* m, const double* dface0,
                  const double* dface1, const double* dface2, double d_const,
                  const double* ccell, double c_const, const double* mcell,
                  double m_const, const double* rhs, double* u, int offset,
                  double* maxres, void* stream)
{
   if (check_model(m) || !rhs || !u || (offset != 0 && offset != 1))
      return AMPE_ERR_INVALID;
   if (dface0 && (!dface1 || (m->dim == 3 && !dface2))) return AMPE_ERR_INVALID;
   FacOp<double> op = make_op(m, dface0, dface1, dface2, d_const, ccell,
                              c_const, mcell, m_const);
   return rbgs_color(op, make_grid(*m), rhs, u, offset, maxres,
                     (cudaStream_t)stream, false);
}

int ampe_efo_rbgs_sweep(const ampe_model_t* m, const double* dface0,
                        const double* dface1, const double* dface2, double d_const,
                        const double* ccell, double c_const, const double* mcell,
                        double m_const, const double* rhs, const double* u_in,
                        double* u_out, void* stream)
{
   if (check_model(m) || !rhs || !u_out || u_in == u_out) return AMPE_ERR_INVALID;
   if (dface0 && (!dface1 || (m->dim == 3 && !dface2))) return AMPE_ERR_INVALID;
   const Grid g = make_grid(*m);
   if (!rb_sweep_fusable<double>(g)) return AMPE_ERR_INVALID;
   FacOp<double> op = make_op(m, dface0, dface1, dface2, d_const, ccell, c_const, mcell,
                              m_const);
   // the z-marching sweep for the operator shapes of the phase, composition
   // and quaternion blocks on large 3D levels, else the box sweep
   ZShape zs;
   if (sweep_z_ok<double>(g, &zs)) {
      const int rc = sweep_z(op, g, zs, rhs, u_in, u_out, nullptr, (const double*)nullptr,
                             (cudaStream_t)stream);
      if (rc != AMPE_ERR_INVALID) return rc;
   }
   return rb_sweep_fused(op, g, rhs, u_in, u_out, (cudaStream_t)stream);
}

int ampe_efo_residual(const ampe_model_t* m, const double* dface0,
                      const double* dface1, const double* dface2,
                      double d_const, const double* ccell, double c_const,
                      const double* mcell, double m_const, const double* rhs,
                      const double* u, double* res, void* stream)
{
   if (check_model(m) || !rhs || !u || !res) return AMPE_ERR_INVALID;
   if (dface0 && (!dface1 || (m->dim == 3 && !dface2))) return AMPE_ERR_INVALID;
   FacOp<double> op = make_op(m, dface0, dface1, dface2, d_const, ccell,
                              c_const, mcell, m_const);
   return residual(op, make_grid(*m), rhs, u, res, (cudaStream_t)stream);
}

size_t ampe_efo_residual_rms_scratch_doubles(const ampe_model_t* m)
{
   if (check_model(m)) return 0;
   return (size_t)residual_rms_scratch_doubles(make_grid(*m));
}

int ampe_efo_residual_rms(const ampe_model_t* m, const double* dface0,
                          const double* dface1, const double* dface2,
                          double d_const, const double* ccell, double c_const,
                          const double* mcell, double m_const,
                          const double* rhs, const double* u, double* scratch,
                          double* rms, void* stream)
{
   if (check_model(m) || !rhs || !u || !scratch || !rms)
      return AMPE_ERR_INVALID;
   if (dface0 && (!dface1 || (m->dim == 3 && !dface2))) return AMPE_ERR_INVALID;
   FacOp<double> op = make_op(m, dface0, dface1, dface2, d_const, ccell,
                              c_const, mcell, m_const);
   return residual_rms_into(op, make_grid(*m), rhs, u, scratch, rms,
                            (cudaStream_t)stream);
}

int ampe_phase_fac_set_c(const ampe_model_t* m, const double* phi,
                         double gamma, double* ccell, void* stream)
{
   if (check_model(m) || !phi || !ccell) return AMPE_ERR_INVALID;
   return phase_set_c(*m, make_grid(*m), phi, gamma, ccell,
                      (cudaStream_t)stream);
}

}  // extern "C"
