// FAC operator descriptor shared by fac.cu and the stepper.
#pragma once

#include "common.cuh"

namespace ampe {

// A u = C u + M div(D grad u); null pointers select the constants.
template <class R>
struct FacOp {
   const R* D0 = nullptr;
   const R* D1 = nullptr;
   const R* D2 = nullptr;
   R dc = 0;
   const R* C = nullptr;
   R cc = 0;
   const R* M = nullptr;
   R mc = 0;
   R dxi[3] = {0, 0, 0};
   // the right-hand side f is an interior array (no ghosts: it is only read
   // at the cell itself); false: ghosted like u (the leaf entry points)
   bool f_interior = false;
};

template <class R>
int rbgs_color(const FacOp<R>& op, const Grid& g, const R* f, R* u,
               int offset, double* maxres, cudaStream_t s, bool images);
// one colour of a sweep on u + P e (e: the next coarser level's correction,
// ghosts current, P piecewise constant), u updated in place with images:
// the red (offset 0) then black pass equal k_prolong_add followed by a sweep.
// Phase, composition and quaternion operator shapes only.
template <class R>
int rbgs_color_prolong(const FacOp<R>& op, const Grid& g, const R* f, R* u, int offset,
                       const Grid& gc, const R* e, cudaStream_t s);
// res = f - A u (interior layout; optional) and per-block sums of res^2
// into part (*nblk blocks); z (optional) receives u's interior values
template <class R>
int residual_partial(const FacOp<R>& op, const Grid& g, const R* f, const R* u,
                     R* res, double* part, int* nblk, R* z, cudaStream_t s);
// coarse f (interior layout) = cell average of the fine residual f - A u
template <class R>
int residual_restrict(const FacOp<R>& op, const Grid& gf, const Grid& gc, const R* f,
                      const R* u, R* fc, cudaStream_t s);
template <class R>
int fill_ghosts_t(const Grid& g, R* f, cudaStream_t s);
// one red + black sweep in one launch, uin -> uout (ghost images written);
// uin null: zero initial guess.  Requires even extents (rb_sweep_fusable).
template <class R>
bool rb_sweep_fusable(const Grid& g);
template <class R>
int rb_sweep_fused(const FacOp<R>& op, const Grid& g, const R* f, const R* uin, R* uout,
                   cudaStream_t s);
template <class R>
int residual(const FacOp<R>& op, const Grid& g, const R* f, const R* u,
             R* res, cudaStream_t s);
template <class R>
int phase_set_c(const ampe_model_t& m, const Grid& g, const double* phi,
                double gamma, R* ccell, cudaStream_t s);

// One red-black sweep of a 3D level in a single z-marching pass (sweep_z.cu):
// blocks of ty rows x the whole x extent (one thread per column) x a chunk
// of planes (kz here for two resident blocks per SM; each launch re-sizes
// the chunks to its kernel's resident blocks, one wave), u staged in a ring
// of kZRingPlanes shared-memory planes of (ty + 4) rows of hs elements.
constexpr int kZRingPlanes = 6;
constexpr int kZRowStride = 256;  // ring row stride (n0 <= 256)
struct ZShape {
   int ty = 0, kz = 0, nh = 0, hs = 0;
};
template <class R>
inline size_t zsweep_smem_bytes(const ZShape& z)
{
   return sizeof(R) * (size_t)kZRingPlanes * (size_t)(z.ty + 4) * (size_t)z.hs;
}
// whether the level takes the single-pass sweep (3D, n0 a multiple of 32 up
// to 256, even extents, at least 2^21 cells, shape fits in shared memory);
// the chosen shape into *out
template <class R>
bool sweep_z_ok(const Grid& g, ZShape* out);
// uin -> uout (uin != uout; ghost images of uout written).  uin null: start
// from u = 0.  e non-null: start from uin + P e, e the correction on the
// next coarser level gc (ghosts current), P piecewise constant.  The result
// equals two rbgs_color passes (red, black) on the same start.
template <class R>
int sweep_z(const FacOp<R>& op, const Grid& g, const ZShape& zs, const R* f, const R* uin,
            R* uout, const Grid* gc, const R* e, cudaStream_t s);

int fill_ghosts(const Grid& g, double* f, cudaStream_t s);
long long residual_rms_scratch_doubles(const Grid& g);
int residual_rms_into(const FacOp<double>& op, const Grid& g, const double* f,
                      const double* u, double* scratch, double* rms,
                      cudaStream_t s);

}  // namespace ampe
