// One whole red-black Gauss-Seidel sweep of a 3D FAC level in a single pass
// that marches along z (EllipticFACOps::smoothErrorByRedBlack,
// EllipticFACOps.cc:1067-1230: all red cells, then all black cells, with
// the update of efo_rbgswithfluxmaxvardcvarsf3d, 3d/ellipticfacops.m4:
// 153-172).
//
// Two colour passes over the level read every array twice (each pass
// touches whole cache lines of both colours).  Here each block owns a tile
// of TY rows (y) x the whole x extent and a chunk of KZ planes (z).  It
// stages u plane by plane in a shared-memory ring (cp.async, two planes
// ahead), and at step w updates the red cells of plane w on the tile plus
// one halo row on each side, then the black cells of plane w-1 on the tile
// (whose red neighbours at w-2, w-1 and w are final by then), and writes
// plane w-1 to the output buffer with its periodic ghost images.  The halo
// rows and the two extra red planes at the chunk ends repeat, on identical
// inputs, updates that the neighbouring blocks also make, so every block
// reads only the input u (u_in -> u_out, never in place) and the result is
// the two colour passes' result: every update evaluates the colour kernel's
// expression in the same order.  f, C, M and the face coefficients are read
// from global memory at the cell, once per sweep from DRAM.
//
// The ring stores each row colour-split (red half, black half, padded so
// that the two halves sit 16 banks apart): an update reads its own value and
// its six neighbours from consecutive words across the warp.
#include <algorithm>
#include <cstdint>

#include "common.cuh"
#include "fac.cuh"

namespace ampe {

namespace {

constexpr int kZRing = kZRingPlanes;  // w-2 .. w+1 in use, w+2, w+3 in flight
constexpr int kZPrefetch = 2;  // planes loaded ahead of the one needed next
constexpr int kZThreads = 256;

__device__ __forceinline__ uint32_t smem_addr(const void* p)
{
   return (uint32_t)__cvta_generic_to_shared(p);
}

template <int BYTES>
__device__ __forceinline__ void cp_async(void* dst, const void* src)
{
   asm volatile("cp.async.ca.shared.global [%0], [%1], %2;" ::"r"(smem_addr(dst)), "l"(src),
                "n"(BYTES)
                : "memory");
}

__device__ __forceinline__ void cp_commit()
{
   asm volatile("cp.async.commit_group;" ::: "memory");
}

// wait until at most n of the most recent groups are pending (n <= 2)
__device__ __forceinline__ void cp_wait(int n)
{
   if (n <= 0)
      asm volatile("cp.async.wait_group 0;" ::: "memory");
   else if (n == 1)
      asm volatile("cp.async.wait_group 1;" ::: "memory");
   else
      asm volatile("cp.async.wait_group 2;" ::: "memory");
}

__device__ __forceinline__ int wrap(int a, int n)
{
   return a < 0 ? a + n : (a >= n ? a - n : a);
}

}  // namespace

// MODE 0: sweep from u_in; 1: from u = 0 (u_in unused); 2: from u_in + P e
// (e the next coarser level's correction, piecewise constant: the first
// post-smoothing sweep with the prolongation fused in)
// per-cell coefficients of one update (members the operator shape does not
// use stay unset)
template <class R>
struct Coef {
   R f, c, m;
   R d[6];  // faces x-, x+, y-, y+, z-, z+
};

// CAPR / CAPB: red / black cells per thread and step (at least
// (ty+2) nh / 256 and ty nh / 256)
template <class R, bool HD, bool HC, bool HM, int MODE, int CAPR, int CAPB>
__global__ void __launch_bounds__(kZThreads, 2)
    k_sweep_z(FacOp<R> op, Grid g, ZShape zs, const R* __restrict__ f,
              const R* __restrict__ uin, R* __restrict__ uout, Grid gc,
              const R* __restrict__ e)
{
   extern __shared__ __align__(16) unsigned char zsm[];
   R* const S = reinterpret_cast<R*>(zsm);
   const int tid = threadIdx.x;
   const int j0 = blockIdx.x * zs.ty;
   const int k0 = blockIdx.y * zs.kz;
   const int k1 = k0 + zs.kz;
   const int nh = zs.nh, hs = zs.hs, rs = 2 * zs.hs, rows = zs.ty + 4;
   const int ps = rows * rs;
   auto slot = [&](int p) { return S + ((p - k0 + 2) % kZRing) * ps; };

   // stage plane p (rows j0-2 .. j0+ty+1, every x) in its ring slot
   auto load_plane = [&](int p) {
      R* dst = slot(p);
      const int kw = wrap(p, g.n2);
      const int n = rows * g.n0;
      for (int t = tid; t < n; t += kZThreads) {
         const int r = (int)g.fd0.div((unsigned)t);
         const int i = t - r * g.n0;
         const int j = j0 - 2 + r;
         const int col = (i + j + p) & 1;
         R* d = dst + r * rs + col * hs + (i >> 1);
         if (MODE == 1)
            *d = R(0);
         else
            cp_async<sizeof(R)>(d, uin + g.c(i, wrap(j, g.n1), kw));
      }
   };
   // MODE 2: add the coarse correction to the values this thread staged
   auto add_correction = [&](int p) {
      R* dst = slot(p);
      const int kw = wrap(p, g.n2);
      const int n = rows * g.n0;
      for (int t = tid; t < n; t += kZThreads) {
         const int r = (int)g.fd0.div((unsigned)t);
         const int i = t - r * g.n0;
         const int j = j0 - 2 + r;
         const int col = (i + j + p) & 1;
         R* d = dst + r * rs + col * hs + (i >> 1);
         *d = *d + e[gc.c(i >> 1, wrap(j, g.n1) >> 1, kw >> 1)];
      }
   };
   // cell m of this thread in colour col of plane p on ring rows
   // [r_lo, r_lo + nr): t = tid + 256 m < nr * nh
   struct Cell {
      int r, j, jw, i, hx, q;
   };
   auto cell = [&](int p, int col, int r_lo, int t) {
      Cell e;
      const int rr = (int)g.fdh.div((unsigned)t);
      e.hx = t - rr * nh;
      e.r = r_lo + rr;
      e.j = j0 - 2 + e.r;
      e.jw = wrap(e.j, g.n1);
      e.q = (col + e.j + p) & 1;  // x parity of this colour in the row
      e.i = 2 * e.hx + e.q;
      return e;
   };
   // the cell's coefficients (f, C, M, face D) from global memory: every
   // load of a step is issued before any update of the step computes
   auto gather = [&](int p, int col, int r_lo, int nr, int m, Coef<R>& cf) {
      const int t = tid + m * kZThreads;
      if (t >= nr * nh) return;
      const int kw = wrap(p, g.n2);
      const Cell e = cell(p, col, r_lo, t);
      const int c = g.c(e.i, e.jw, kw);
      cf.f = __ldg(f + (op.f_interior ? g.interior(e.i, e.jw, kw) : c));
      if (HC) cf.c = __ldg(op.C + c);
      if (HM) cf.m = __ldg(op.M + c);
      if (HD) {
         const int fx = g.fx(e.i, e.jw, kw), fy = g.fy(e.i, e.jw, kw), fz = g.fz(e.i, e.jw, kw);
         cf.d[0] = __ldg(op.D0 + fx);
         cf.d[1] = __ldg(op.D0 + fx + 1);
         cf.d[2] = __ldg(op.D1 + fy);
         cf.d[3] = __ldg(op.D1 + fy + g.fys());
         cf.d[4] = __ldg(op.D2 + fz);
         cf.d[5] = __ldg(op.D2 + fz + g.fzs());
      }
   };
   // update cell m of colour col of plane p from the staged u and its
   // gathered coefficients
   auto update = [&](int p, int col, int r_lo, int nr, int m, const Coef<R>& cf) {
      const int t = tid + m * kZThreads;
      if (t >= nr * nh) return;
      R* P = slot(p);
      const R* Pm = slot(p - 1);
      const R* Pp = slot(p + 1);
      const int oth = (1 - col) * hs;
      const Cell e = cell(p, col, r_lo, t);
      const int hx = e.hx, r = e.r;
      int hm = hx - 1 + e.q;
      if (hm < 0) hm = nh - 1;
      int hp = hx + e.q;
      if (hp == nh) hp = 0;
      R* own = P + r * rs + col * hs + hx;
      const R uc = *own;
      const R uxm = P[r * rs + oth + hm], uxp = P[r * rs + oth + hp];
      const R uym = P[(r - 1) * rs + oth + hx], uyp = P[(r + 1) * rs + oth + hx];
      const R uzm = Pm[r * rs + oth + hx], uzp = Pp[r * rs + oth + hx];
      // expression order of op_residual_u (the colour kernel's)
      R div = R(0), dsum = R(0);
      {
         const R dxi = op.dxi[0];
         const R Dm = HD ? cf.d[0] : op.dc, Dp = HD ? cf.d[1] : op.dc;
         const R fm = dxi * Dm * (uc - uxm);
         const R fp = dxi * Dp * (uxp - uc);
         div += dxi * (fp - fm);
         dsum += dxi * dxi * (Dp + Dm);
      }
      {
         const R dxi = op.dxi[1];
         const R Dm = HD ? cf.d[2] : op.dc, Dp = HD ? cf.d[3] : op.dc;
         const R fm = dxi * Dm * (uc - uym);
         const R fp = dxi * Dp * (uyp - uc);
         div += dxi * (fp - fm);
         dsum += dxi * dxi * (Dp + Dm);
      }
      {
         const R dxi = op.dxi[2];
         const R Dm = HD ? cf.d[4] : op.dc, Dp = HD ? cf.d[5] : op.dc;
         const R fm = dxi * Dm * (uc - uzm);
         const R fp = dxi * Dp * (uzp - uc);
         div += dxi * (fp - fm);
         dsum += dxi * dxi * (Dp + Dm);
      }
      const R M = HM ? cf.m : op.mc;
      const R C = HC ? cf.c : op.cc;
      const R dudr = R(1) / (M * dsum - C);
      const R res = cf.f - M * div - C * uc;
      *own = uc + -res * dudr;
   };
   // the block's rows of plane p (final values) -> u_out and its images
   auto store = [&](int p) {
      const R* P = slot(p);
      const int n = zs.ty * g.n0;
      for (int t = tid; t < n; t += kZThreads) {
         const int rr = (int)g.fd0.div((unsigned)t);
         const int i = t - rr * g.n0;
         const int j = j0 + rr;
         const int col = (i + j + p) & 1;
         const R v = P[(rr + 2) * rs + col * hs + (i >> 1)];
         uout[g.c(i, j, p)] = v;
         for_each_image(g, i, j, p, [&](int idx) { uout[idx] = v; });
      }
   };

   int next = k0 - 2;  // next plane to stage
   for (int w = k0 - 1; w <= k1; w++) {
      const int want = min(w + 1 + kZPrefetch, k1 + 1);
      for (; next <= want; next++) {
         load_plane(next);
         cp_commit();
      }
      // plane w+1 and all older ones have landed
      cp_wait(next - (w + 2));
      if (MODE == 2) {
         // every plane gets its correction once, when it is first needed
         if (w == k0 - 1) {
            add_correction(k0 - 2);
            add_correction(k0 - 1);
         }
         add_correction(w + 1);
      }
      // coefficients of both updates of this step (red at w on the tile
      // and one halo row each side, black at w-1 on the tile)
      Coef<R> cr[CAPR], cb[CAPB];
#pragma unroll
      for (int m = 0; m < CAPR; m++) gather(w, 0, 1, zs.ty + 2, m, cr[m]);
      if (w > k0) {
#pragma unroll
         for (int m = 0; m < CAPB; m++) gather(w - 1, 1, 2, zs.ty, m, cb[m]);
      }
      __syncthreads();
#pragma unroll
      for (int m = 0; m < CAPR; m++) update(w, 0, 1, zs.ty + 2, m, cr[m]);
      __syncthreads();
      if (w > k0) {
#pragma unroll
         for (int m = 0; m < CAPB; m++) update(w - 1, 1, 2, zs.ty, m, cb[m]);
         __syncthreads();
         store(w - 1);
      }
   }
}

template <class R>
static ZShape choose_zshape(const Grid& g)
{
   ZShape zs;
   zs.nh = g.n0 / 2;
   // colour halves 16 banks apart: hs * sizeof(R) / 4 = 16 (mod 32)
   const int unit = (int)sizeof(R) / 4;
   const int mod = 32 / unit, want = 16 / unit;
   zs.hs = zs.nh + ((want - zs.nh % mod) % mod + mod) % mod;
   zs.ty = 8;
   while (zs.ty > 2 && zsweep_smem_bytes<R>(zs) > 112 * 1024) zs.ty /= 2;
   // planes per block: the most that still give every SM a block, at least
   // 8 (each chunk stages 4 planes and updates 2 red planes twice)
   const int by = g.n1 / zs.ty;
   const int target = device_sms();
   int best = g.n2;
   for (int kz = g.n2; kz >= 8; kz--) {
      if (g.n2 % kz) continue;
      best = kz;
      if ((long long)by * (g.n2 / kz) >= target) break;
   }
   zs.kz = best;
   return zs;
}

template <class R>
bool sweep_z_ok(const Grid& g, ZShape* out)
{
   if (g.dim != 3 || g.ng < 1) return false;
   if (g.n0 % 2 || g.n1 % 2 || g.n2 % 2) return false;
   if (g.cells() < (1LL << 21)) return false;  // small levels: colour kernels
   const ZShape zs = choose_zshape<R>(g);
   if (g.n1 % zs.ty || g.n2 % zs.kz || zs.kz < 8) return false;
   if (zsweep_smem_bytes<R>(zs) > 200 * 1024) return false;
   // the cells per thread and step the kernels are built for
   if ((zs.ty + 2) * zs.nh > 6 * kZThreads || zs.ty * zs.nh > 4 * kZThreads) return false;
   if (out) *out = zs;
   return true;
}

template <class R, bool HD, bool HC, bool HM, int MODE, int CAPR, int CAPB>
static int launch_caps(const FacOp<R>& op, const Grid& g, const ZShape& zs, const R* f,
                       const R* uin, R* uout, const Grid& gc, const R* e, cudaStream_t s)
{
   const int smem = (int)zsweep_smem_bytes<R>(zs);
   static std::atomic<unsigned long long> attr{0};
   if (first_on_device(attr))
      cudaFuncSetAttribute(k_sweep_z<R, HD, HC, HM, MODE, CAPR, CAPB>,
                           cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
   const dim3 grid(g.n1 / zs.ty, g.n2 / zs.kz);
   k_sweep_z<R, HD, HC, HM, MODE, CAPR, CAPB>
       <<<grid, kZThreads, smem, s>>>(op, g, zs, f, uin, uout, gc, e);
   return launch_status();
}

template <class R, bool HD, bool HC, bool HM, int MODE>
static int launch_z(const FacOp<R>& op, const Grid& g, const ZShape& zs, const R* f,
                    const R* uin, R* uout, const Grid& gc, const R* e, cudaStream_t s)
{
   const int red = (zs.ty + 2) * zs.nh, black = zs.ty * zs.nh;
   if (red <= 3 * kZThreads && black <= 2 * kZThreads)
      return launch_caps<R, HD, HC, HM, MODE, 3, 2>(op, g, zs, f, uin, uout, gc, e, s);
   if (red <= 6 * kZThreads && black <= 4 * kZThreads)
      return launch_caps<R, HD, HC, HM, MODE, 6, 4>(op, g, zs, f, uin, uout, gc, e, s);
   return AMPE_ERR_INVALID;
}

template <class R, int MODE>
static int dispatch_z(const FacOp<R>& op, const Grid& g, const ZShape& zs, const R* f,
                      const R* uin, R* uout, const Grid& gc, const R* e, cudaStream_t s)
{
   const bool hd = op.D0 != nullptr, hc = op.C != nullptr, hm = op.M != nullptr;
   if (!hd && hc && !hm) return launch_z<R, false, true, false, MODE>(op, g, zs, f, uin, uout, gc, e, s);
   if (hd && !hc && !hm) return launch_z<R, true, false, false, MODE>(op, g, zs, f, uin, uout, gc, e, s);
   if (hd && !hc && hm) return launch_z<R, true, false, true, MODE>(op, g, zs, f, uin, uout, gc, e, s);
   return AMPE_ERR_INVALID;
}

template <class R>
int sweep_z(const FacOp<R>& op, const Grid& g, const ZShape& zs, const R* f, const R* uin,
            R* uout, const Grid* gc, const R* e, cudaStream_t s)
{
   if (uin == uout) return AMPE_ERR_INVALID;
   if (e) return dispatch_z<R, 2>(op, g, zs, f, uin, uout, *gc, e, s);
   if (!uin) return dispatch_z<R, 1>(op, g, zs, f, uin, uout, g, e, s);
   return dispatch_z<R, 0>(op, g, zs, f, uin, uout, g, e, s);
}

template bool sweep_z_ok<double>(const Grid&, ZShape*);
template bool sweep_z_ok<float>(const Grid&, ZShape*);
template int sweep_z<double>(const FacOp<double>&, const Grid&, const ZShape&, const double*,
                             const double*, double*, const Grid*, const double*, cudaStream_t);
template int sweep_z<float>(const FacOp<float>&, const Grid&, const ZShape&, const float*,
                            const float*, float*, const Grid*, const float*, cudaStream_t);

}  // namespace ampe
