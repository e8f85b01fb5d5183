// One whole red-black Gauss-Seidel sweep of a 3D FAC level in a single pass
// that marches along z (EllipticFACOps::smoothErrorByRedBlack,
// EllipticFACOps.cc:1067-1230: all red cells, then all black cells, with
// the update of efo_rbgswithfluxmaxvardcvarsf3d, 3d/ellipticfacops.m4:
// 153-172).
//
// Two colour passes over the level read every array twice (each pass
// touches whole cache lines of both colours).  Here a block owns TY rows
// (y) x the whole x extent (one thread per x column) and a chunk of KZ
// planes (z).  It stages u plane by plane in a shared-memory ring (cp.async,
// two planes ahead), and at step w updates the red cells of plane w on its
// rows plus one halo row on each side, then the black cells of plane w-1 on
// its rows (whose red neighbours at w-2, w-1 and w are final by then), and
// writes plane w-1 to the output buffer with its periodic ghost images.
// The halo rows and the two extra red planes at the chunk ends repeat, on
// identical inputs, updates that the neighbouring blocks also make, so every
// block reads only the input u (u_in -> u_out, never in place) and the
// result is the two colour passes' result: every update evaluates the colour
// kernel's expression in the same order.  f, C, M and the face coefficients
// are read from global memory at the cell, once per sweep from DRAM; the
// coefficient loads of a colour stage are all issued before its first
// update.
//
// Each thread keeps its x column, its neighbours' columns and the block's
// rows for the whole kernel, so per cell the index work is a few integer
// operations; in a warp the even and odd lanes update cells of one colour in
// adjacent rows, so the row-major ring is read without bank conflicts.
#include <algorithm>
#include <cstdint>

#include "common.cuh"
#include "fac.cuh"

namespace ampe {

namespace {

constexpr int kZRing = kZRingPlanes;  // w-2 .. w+1 in use, w+2, w+3 in flight
constexpr int kZPrefetch = 2;         // planes loaded ahead of the one needed next

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

// per-cell coefficients of one update (members the operator shape does not
// use stay unset)
template <class R>
struct Coef {
   R f, c, m;
   R d[6];  // faces x-, x+, y-, y+, z-, z+
};

// MODE 0: sweep from u_in; 1: from u = 0 (u_in unused); 2: from u_in + P e
// (e the next coarser level's correction, piecewise constant: the first
// post-smoothing sweep with the prolongation fused in).  blockDim.x = n0
// (<= 256).  The ring's rows are kZRowStride elements apart whatever n0,
// so every shared-memory access of a cell update has a constant offset from
// one of a few per-step base pointers.
template <class R, bool HD, bool HC, bool HM, int MODE, int TY>
__global__ void __launch_bounds__(256, (sizeof(R) == 4 && !HD && MODE != 2) ? 3 : 2)
    k_sweep_z(FacOp<R> op, Grid g, int kz, const R* __restrict__ f,
              const R* __restrict__ uin, R* __restrict__ uout, Grid gc,
              const R* __restrict__ e)
{
   constexpr int ROWS = TY + 4;
   constexpr int HS = kZRowStride, PS = ROWS * HS;
   constexpr int NRED = (TY + 2) / 2, NBLACK = TY / 2;
   // software-pipelined coefficient loads where they fit the registers (the
   // phase operator: f and C per cell)
   constexpr bool PIPE = !HD;
   // FP32 (the mixed path's preconditioner): the update in its Jacobi form
   // with an approximate reciprocal, three blocks per SM for the cell-C
   // operator (the face-D operators keep two: their coefficients need the
   // registers); FP64 keeps the colour kernel's expression order and rounding
   constexpr bool FAST = sizeof(R) == 4;
   float w2[3] = {0.f, 0.f, 0.f}, dsum_c = 0.f;
   if constexpr (FAST) {
      for (int d = 0; d < 3; d++) w2[d] = (float)op.dxi[d] * (float)op.dxi[d];
      if constexpr (!HD) {
         for (int d = 0; d < 3; d++) w2[d] *= (float)op.dc;
         dsum_c = 2.f * (w2[0] + w2[1] + w2[2]);
      }
   }
   extern __shared__ __align__(16) unsigned char zsm[];
   R* const S = reinterpret_cast<R*>(zsm);
   const int n0 = g.n0, x = threadIdx.x;
   const int dxm = x == 0 ? n0 - 1 : -1;  // offsets of the periodic x neighbours
   const int dxp = x == n0 - 1 ? 1 - n0 : 1;
   const int j0 = blockIdx.x * TY;
   // the last chunk may be shorter (launches sized to one wave of blocks)
   const int k0 = blockIdx.y * kz, k1 = min(k0 + kz, g.n2);
   // wrapped y index of ring row r (the block's rows and two halo rows on
   // each side) and its ghosted row offset, formed where they are used (a
   // few integer operations, no registers held and no load in front of the
   // load that needs them)
   auto jw = [&](int r) { return wrap(j0 - 2 + r, g.n1); };
   auto rowg = [&](int r) { return (jw(r) + g.ng) * g.sx; };
   const bool xedge = x < g.ng || x >= n0 - g.ng;
   // ring slot of plane p (p >= k0 - 2), this column
   auto slot_of = [&](int p) { return (p - k0 + 2) % kZRing; };
   auto colp = [&](int sl) { return S + sl * PS + x; };
   // ghosted offset of this column in plane kk
   auto gplane = [&](int kk) { return (kk + g.gz) * g.sy + g.ng + x; };

   auto load_plane = [&](int p) {
      R* dst = colp(slot_of(p));
      const R* src = uin + gplane(wrap(p, g.n2));
#pragma unroll
      for (int r = 0; r < ROWS; r++) {
         if (MODE == 1)
            dst[r * HS] = R(0);
         else
            cp_async<sizeof(R)>(dst + r * HS, src + rowg(r));
      }
   };
   // MODE 2: add the coarse correction to the values this thread staged
   auto add_correction = [&](int p) {
      R* dst = colp(slot_of(p));
      const R* ep = e + (((wrap(p, g.n2) >> 1) + gc.gz) * gc.sy + gc.ng + (x >> 1));
#pragma unroll
      for (int r = 0; r < ROWS; r++)
         dst[r * HS] = dst[r * HS] + ep[((jw(r) >> 1) + gc.ng) * gc.sx];
   };
   // this column's cells of colour col in plane p from ring row rlo on sit
   // at rows rlo + par + 2m, par = 0 or 1 by the column's parity
   auto par_of = [&](int p, int col, int rlo) { return (x + j0 - 2 + rlo + p + col) & 1; };
   // coefficients of ring row rr of plane p
   auto gather = [&](int kw, int cplane, int fplane, int jj, Coef<R>& cf) {
      const int c = cplane + (jj + g.ng) * g.sx;
      cf.f = __ldg(f + (op.f_interior ? fplane + jj * n0 : c));
      if (HC) cf.c = __ldg(op.C + c);
      if (HM) cf.m = __ldg(op.M + c);
      if (HD) {
         const int fx = g.fx(x, jj, kw), fy = g.fy(x, jj, kw), fz = g.fz(x, jj, kw);
         cf.d[0] = __ldg(op.D0 + fx);
         cf.d[1] = __ldg(op.D0 + fx + 1);
         cf.d[2] = __ldg(op.D1 + fy);
         cf.d[3] = __ldg(op.D1 + fy + g.fys());
         cf.d[4] = __ldg(op.D2 + fz);
         cf.d[5] = __ldg(op.D2 + fz + g.fzs());
      }
   };
   // one update at ring row offset o (a compile-time multiple of HS) from
   // the column bases of its plane (P), the x neighbours' (P + dxm, P + dxp)
   // and the planes below and above (Pm, Pp)
   auto update = [&](R* P, const R* Pm, const R* Pp, int o, const Coef<R>& cf) {
      const R uc = P[o];
      const R uxm = P[o + dxm], uxp = P[o + dxp];
      const R uym = P[o - HS], uyp = P[o + HS];
      const R uzm = Pm[o], uzp = Pp[o];
      if constexpr (FAST) {
         // u <- (M nb - f) / (M dsum - C): the same update, with
         // nb = sum_d dxi_d^2 (D- u- + D+ u+), dsum = sum_d dxi_d^2 (D- + D+)
         (void)uc;
         float nb, dsum;
         if constexpr (HD) {
            nb = w2[0] * (cf.d[0] * uxm + cf.d[1] * uxp);
            nb = fmaf(w2[1], cf.d[2] * uym + cf.d[3] * uyp, nb);
            nb = fmaf(w2[2], cf.d[4] * uzm + cf.d[5] * uzp, nb);
            dsum = w2[0] * (cf.d[0] + cf.d[1]);
            dsum = fmaf(w2[1], cf.d[2] + cf.d[3], dsum);
            dsum = fmaf(w2[2], cf.d[4] + cf.d[5], dsum);
         } else {
            nb = w2[0] * (uxm + uxp);
            nb = fmaf(w2[1], uym + uyp, nb);
            nb = fmaf(w2[2], uzm + uzp, nb);
            dsum = dsum_c;
         }
         const float M = HM ? cf.m : op.mc;
         const float C = HC ? cf.c : op.cc;
         P[o] = __fdividef(fmaf(M, nb, -cf.f), fmaf(M, dsum, -C));
         return;
      }
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
      P[o] = uc + -res * dudr;
   };
   // the block's rows of plane p (final values, column base P) -> u_out
   // and its images
   auto store = [&](int p, const R* P) {
      const int dbase = gplane(p);
      const bool pedge = p < g.ng || p >= g.n2 - g.ng;
#pragma unroll
      for (int r = 2; r < TY + 2; r++) {
         const int j = j0 + r - 2;
         const R v = P[r * HS];
         uout[dbase + (j + g.ng) * g.sx] = v;
         if (xedge || pedge || j < g.ng || j >= g.n1 - g.ng)
            for_each_image(g, x, j, p, [&](int idx) { uout[idx] = v; });
      }
   };

   // the coefficients of one step: red at w on the rows and one halo row
   // each side (ring rows 1 .. TY+2), black at w-1 on the rows (ring rows
   // 2 .. TY+1)
   auto gather_step = [&](int w, Coef<R>* cr, Coef<R>* cb) {
      {
         const int kw = wrap(w, g.n2);
         const int cpl = gplane(kw), fpl = kw * g.n1 * n0 + x;
         const int pr = par_of(w, 0, 1);
#pragma unroll
         for (int m = 0; m < NRED; m++) {
            const int r = 1 + 2 * m;
            gather(kw, cpl, fpl, jw(r + pr), cr[m]);
         }
      }
      if (w > k0) {
         const int kw = wrap(w - 1, g.n2);
         const int cpl = gplane(kw), fpl = kw * g.n1 * n0 + x;
         const int pb = par_of(w - 1, 1, 2);
#pragma unroll
         for (int m = 0; m < NBLACK; m++) {
            const int r = 2 + 2 * m;
            gather(kw, cpl, fpl, jw(r + pb), cb[m]);
         }
      }
   };
   int next = k0 - 2;  // next plane to stage
   // One step; with PIPE the coefficients of step w come in cur (gathered
   // during step w-1) and those of step w+1 are gathered into nxt after
   // this step's updates, so their loads overlap the store and the next
   // step's wait.  Two barriers per step.  The first makes plane w+1
   // (every thread's copies) and the previous step's black updates visible;
   // only then is plane w+3 issued, into the slot of plane w-3, which the
   // previous step's black updates were the last to read.  The second
   // orders the red updates of plane w before the black ones of plane w-1.
   // Each thread updates and stores only its own column, so the store of
   // plane w-1 needs no barrier.
   auto step = [&](int w, Coef<R>* cr, Coef<R>* cb, Coef<R>* nr, Coef<R>* nb) {
      // plane w+1 and all older ones have landed (this thread's copies)
      cp_wait(next - (w + 2));
      if (MODE == 2) {
         // every plane gets its correction once, when it is first needed
         if (w == k0 - 1) {
            add_correction(k0 - 2);
            add_correction(k0 - 1);
         }
         add_correction(w + 1);
      }
      if (!PIPE) gather_step(w, cr, cb);
      __syncthreads();
      const int want = min(w + 1 + kZPrefetch, k1 + 1);
      for (; next <= want; next++) {
         load_plane(next);
         cp_commit();
      }
      // slots of planes w-2 .. w+1
      const int s0 = slot_of(w);
      const int sm1 = s0 == 0 ? kZRing - 1 : s0 - 1;
      const int sm2 = sm1 == 0 ? kZRing - 1 : sm1 - 1;
      const int sp1 = s0 == kZRing - 1 ? 0 : s0 + 1;
      R* const Pw = colp(s0);
      R* const Pw1 = colp(sm1);
      {
         const int pr = par_of(w, 0, 1);
         R* const P = Pw + pr * HS;
         const R* const Pm = Pw1 + pr * HS;
         const R* const Pp = colp(sp1) + pr * HS;
#pragma unroll
         for (int m = 0; m < NRED; m++) update(P, Pm, Pp, (1 + 2 * m) * HS, cr[m]);
      }
      __syncthreads();
      if (w > k0) {
         const int pb = par_of(w - 1, 1, 2);
         R* const P = Pw1 + pb * HS;
         const R* const Pm = colp(sm2) + pb * HS;
         const R* const Pp = Pw + pb * HS;
#pragma unroll
         for (int m = 0; m < NBLACK; m++) update(P, Pm, Pp, (2 + 2 * m) * HS, cb[m]);
      }
      if (PIPE && w < k1) gather_step(w + 1, nr, nb);
      if (w > k0) store(w - 1, Pw1);
   };
   // prologue: the planes the first step reads (k0-2 .. k0) and one ahead
   for (; next <= min(k0 + 1, k1 + 1); next++) {
      load_plane(next);
      cp_commit();
   }
   if constexpr (PIPE) {
      Coef<R> ar[NRED], ab[NBLACK], br[NRED], bb[NBLACK];
      gather_step(k0 - 1, ar, ab);
      for (int w = k0 - 1; w <= k1; w += 2) {
         step(w, ar, ab, br, bb);
         if (w + 1 <= k1) step(w + 1, br, bb, ar, ab);
      }
   } else {
      Coef<R> cr[NRED], cb[NBLACK];
      for (int w = k0 - 1; w <= k1; w++) step(w, cr, cb, cr, cb);
   }
}

// planes per z chunk so that the launch's n1/ty x ceil(n2/kz) blocks fill the
// SMs' resident slots (bps blocks per SM) in one wave: a second, partly
// filled wave would leave most SMs idle for its whole duration.  Chunks of
// at least 8 planes (each stages 4 planes and updates 2 red planes more
// than it stores); the last chunk takes the remainder.
static int wave_kz(const Grid& g, int ty, int bps)
{
   const long long by = g.n1 / ty;
   const long long slots = (long long)device_sms() * std::max(1, bps);
   long long nz = std::max(1LL, slots / by);
   nz = std::min(nz, (long long)std::max(1, g.n2 / 8));
   return (int)((g.n2 + nz - 1) / nz);
}

template <class R>
static ZShape choose_zshape(const Grid& g)
{
   ZShape zs;
   zs.nh = g.n0 / 2;
   zs.hs = kZRowStride;  // row stride of the ring (one x column per thread)
   // 8 rows per block in FP32 (<= 74 KB of ring per block), 4 in FP64 (the
   // coefficients of 8 rows do not fit the register budget)
   zs.ty = sizeof(R) == 4 ? 8 : 4;
   if (zsweep_smem_bytes<R>(zs) > 74 * 1024) zs.ty = 4;
   // planes per block: a default for two resident blocks per SM; each
   // launch sizes its chunks to the blocks its kernel keeps resident
   zs.kz = wave_kz(g, zs.ty, 2);
   return zs;
}

template <class R>
bool sweep_z_ok(const Grid& g, ZShape* out)
{
   if (g.dim != 3 || g.ng < 1) return false;
   if (g.n0 % 32 || g.n0 > 256 || g.n1 % 2 || g.n2 % 2) return false;
   if (g.cells() < (1LL << 21)) return false;  // small levels: colour kernels
   const ZShape zs = choose_zshape<R>(g);
   if (g.n1 % zs.ty) return false;
   if (zsweep_smem_bytes<R>(zs) > 200 * 1024) return false;
   if (out) *out = zs;
   return true;
}

template <class R, bool HD, bool HC, bool HM, int MODE, int TY>
static int launch_ty(const FacOp<R>& op, const Grid& g, const ZShape& zs, const R* f,
                     const R* uin, R* uout, const Grid& gc, const R* e, cudaStream_t s)
{
   const int smem = (int)zsweep_smem_bytes<R>(zs);
   auto* fn = k_sweep_z<R, HD, HC, HM, MODE, TY>;
   static std::atomic<unsigned long long> attr{0};
   if (first_on_device(attr))
      cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
   // resident blocks per SM of this instance at this block size (queried
   // once per device and block size)
   constexpr int kDevs = 64;
   static std::atomic<int> bps_of[kDevs];
   int dev = 0;
   if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kDevs) dev = 0;
   int packed = bps_of[dev].load(std::memory_order_relaxed);
   int bps = packed & 0xff;
   if (!packed || (packed >> 8) != g.n0) {
      if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, fn, g.n0, smem) != cudaSuccess ||
          bps < 1)
         bps = 1;
      bps_of[dev].store((g.n0 << 8) | std::min(bps, 255), std::memory_order_relaxed);
   }
   const int kz = wave_kz(g, TY, bps);
   const dim3 grid(g.n1 / TY, (g.n2 + kz - 1) / kz);
   fn<<<grid, g.n0, smem, s>>>(op, g, kz, f, uin, uout, gc, e);
   return launch_status();
}

template <class R, bool HD, bool HC, bool HM, int MODE>
static int launch_z(const FacOp<R>& op, const Grid& g, const ZShape& zs, const R* f,
                    const R* uin, R* uout, const Grid& gc, const R* e, cudaStream_t s)
{
   if (zs.ty == 8) return launch_ty<R, HD, HC, HM, MODE, 8>(op, g, zs, f, uin, uout, gc, e, s);
   if (zs.ty == 4) return launch_ty<R, HD, HC, HM, MODE, 4>(op, g, zs, f, uin, uout, gc, e, s);
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
