// Symmetry-aware quaternion kernels for 3D, qlen 4 (cubic crystal
// symmetry: the 48 unit quaternions of the double cover of the cubic
// rotation group).
//   k_quat_symm_rotation   QUAT_SYMM_ROTATION (3d/quatrotation.m4:12-91) with
//                          quatfindsymm4 (quat.f:73-163): per face, the
//                          rotation of the lower cell's q closest to the
//                          upper cell's q, searched from the face's previous
//                          index
//   k_quat_fundamental     QUAT_FUNDAMENTAL (3d/quatrotation.m4:93-147): each
//                          interior q mapped to the rotation closest to 1
//   k_quat_diffs_symm      QUATDIFFS_SYMM (3d/quatdiffs.m4:131-219)
//   k_quat_grad_side_symm  QUATGRAD_SIDE_SYMM (3d/quatgrad.m4:376-679)
// The products, norms and differences use explicitly rounded operations
// (no fused multiply-add), in the reference's order of operations, so that
// the discrete choices (the rotation index of each face) and the values are
// those of the CPU evaluation of the same formulas.
#include <cmath>

#include "common.cuh"

namespace ampe {

// the 48 rotations in quat.f setqr's order, normalised as quatset does,
// and the index (0-based) of each one's conjugate
struct SymmTable {
   double qr[48][4];
   int conj[48];
   double thr;  // (2 sin(pi/16))^2: a rotation this close ends the search
};

namespace {

__device__ __forceinline__ double M(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double A(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double S(double a, double b) { return __dsub_rn(a, b); }

// quatmult4 (quat.f:867-896)
__device__ __forceinline__ void qmult(const double* a, const double* b, double* q)
{
   q[0] = S(S(S(M(a[0], b[0]), M(a[1], b[1])), M(a[2], b[2])), M(a[3], b[3]));
   q[1] = S(A(A(M(a[0], b[1]), M(a[1], b[0])), M(a[2], b[3])), M(a[3], b[2]));
   q[2] = S(A(A(M(a[0], b[2]), M(a[2], b[0])), M(a[3], b[1])), M(a[1], b[3]));
   q[3] = S(A(A(M(a[0], b[3]), M(a[3], b[0])), M(a[1], b[2])), M(a[2], b[1]));
}

// quatnorm4 with quatmaginv4 (quat.f:997-1085): 0 below a magnitude of 1e-15
__device__ __forceinline__ void qnorm(double* q)
{
   const double m =
       __dsqrt_rn(A(A(A(M(q[0], q[0]), M(q[1], q[1])), M(q[2], q[2])), M(q[3], q[3])));
   const double minv = m < 1.e-15 ? 0.0 : __ddiv_rn(1.0, m);
   for (int c = 0; c < 4; c++) q[c] = M(q[c], minv);
}

// quatdiffsq4 (quat.f:1171-1199): |q2/|q2| - q1/|q1||^2
__device__ __forceinline__ double qdiffsq(const double* q1, const double* q2)
{
   double a[4], b[4];
   for (int c = 0; c < 4; c++) {
      a[c] = q1[c];
      b[c] = q2[c];
   }
   qnorm(a);
   qnorm(b);
   double d[4];
   for (int c = 0; c < 4; c++) d[c] = S(b[c], a[c]);
   return A(A(A(M(d[0], d[0]), M(d[1], d[1])), M(d[2], d[2])), M(d[3], d[3]));
}

// quatsymmrotate4 (quat.f:290-341); iq 1-based, negative: the conjugate.
// Returns false for an index out of range (the reference stops there).
__device__ __forceinline__ bool qrotate(const SymmTable& T, const double* q, int iq,
                                        double* qp)
{
   if (iq == 0 || iq > 48 || iq < -48) return false;
   if (iq < 0) iq = T.conj[-iq - 1] + 1;
   if (iq == 1) {
      for (int c = 0; c < 4; c++) qp[c] = q[c];
   } else {
      qmult(q, T.qr[iq - 1], qp);
   }
   return true;
}

// quatfindsymm4 (quat.f:73-163): iq in/out (1-based)
__device__ __forceinline__ void qfindsymm(const SymmTable& T, const double* q1,
                                          const double* q2, int& iq, double* q2p)
{
   if (iq == 0 || iq > 48 || iq < -48) iq = 1;
   if (iq < 0) iq = T.conj[-iq - 1] + 1;
   double dsq;
   if (iq == 1) {
      for (int c = 0; c < 4; c++) q2p[c] = q2[c];
   } else {
      qmult(q2, T.qr[iq - 1], q2p);
   }
   dsq = qdiffsq(q1, q2p);
   if (dsq <= T.thr) return;
   double min_dsq = dsq, minq[4];
   int min_iq = iq;
   for (int c = 0; c < 4; c++) minq[c] = q2p[c];
   for (int nn = 1; nn <= 48; nn++) {
      if (nn == iq) continue;
      double t[4];
      if (nn == 1) {
         for (int c = 0; c < 4; c++) t[c] = q2[c];
      } else {
         qmult(q2, T.qr[nn - 1], t);
      }
      dsq = qdiffsq(q1, t);
      if (dsq < min_dsq) {
         min_dsq = dsq;
         min_iq = nn;
         for (int c = 0; c < 4; c++) minq[c] = t[c];
      }
      if (dsq <= T.thr) break;
   }
   for (int c = 0; c < 4; c++) q2p[c] = minq[c];
   iq = min_iq;
}

__device__ __forceinline__ void load_q(const Grid& g, const double* q, long long qs, int i,
                                       int j, int k, double* v)
{
   const long long c = g.c(i, j, k);
   for (int m = 0; m < 4; m++) v[m] = q[m * qs + c];
}

// faces of normal d with one transverse ghost layer (the loops of
// QUAT_SYMM_ROTATION and QUATDIFFS_SYMM): counts and decomposition
__device__ __forceinline__ void face_ext(const Grid& g, int d, int& e0, int& e1, int& e2)
{
   e0 = g.n0 + (d == 0 ? 1 : 2);
   e1 = g.n1 + (d == 1 ? 1 : 2);
   e2 = g.n2 + (d == 2 ? 1 : 2);
}

__device__ __forceinline__ long long side_index(const Grid& g, int d, int i, int j, int k)
{
   return d == 0 ? g.fx(i, j, k) : (d == 1 ? g.fy(i, j, k) : g.fz(i, j, k));
}

__device__ __forceinline__ long long side_size(const Grid& g, int d)
{
   const long long a = g.n0 + 2 * g.gs + (d == 0), b = g.n1 + 2 * g.gs + (d == 1);
   const long long c = g.n2 + 2 * g.gsz + (d == 2);
   return a * b * c;
}

}  // namespace

__global__ void k_quat_symm_rotation(Grid g, SymmTable T, const double* q, int* r0, int* r1,
                                     int* r2)
{
   const long long qs = g.cells_ghost();
   long long tot[3];
   for (int d = 0; d < 3; d++) {
      int e0, e1, e2;
      face_ext(g, d, e0, e1, e2);
      tot[d] = (long long)e0 * e1 * e2;
   }
   for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
        t < tot[0] + tot[1] + tot[2]; t += (long long)gridDim.x * blockDim.x) {
      int d = 0;
      long long r = t;
      while (r >= tot[d]) r -= tot[d++];
      int e0, e1, e2;
      face_ext(g, d, e0, e1, e2);
      const int i = (int)(r % e0) - (d != 0);
      const int j = (int)((r / e0) % e1) - (d != 1);
      const int k = (int)(r / ((long long)e0 * e1)) - (d != 2);
      const int ei = d == 0, ej = d == 1, ek = d == 2;
      double q1[4], q2[4], q2p[4];
      load_q(g, q, qs, i, j, k, q1);
      load_q(g, q, qs, i - ei, j - ej, k - ek, q2);
      int* rot = d == 0 ? r0 : (d == 1 ? r1 : r2);
      const long long f = side_index(g, d, i, j, k);
      int iq = rot[f];
      qfindsymm(T, q1, q2, iq, q2p);
      rot[f] = iq;
   }
}

__global__ void k_quat_fundamental(Grid g, SymmTable T, double* q)
{
   const long long qs = g.cells_ghost();
   double q1[4] = {1.0, 0.0, 0.0, 0.0};
   qnorm(q1);
   for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < g.cells();
        t += (long long)gridDim.x * blockDim.x) {
      int i, j, k;
      g.ijk(t, i, j, k);
      double q2[4], q2p[4];
      load_q(g, q, qs, i, j, k, q2);
      int iq = 1;
      qfindsymm(T, q1, q2, iq, q2p);
      const long long c = g.c(i, j, k);
      for (int m = 0; m < 4; m++) q[m * qs + c] = q2p[m];
   }
}

__global__ void k_quat_diffs_symm(Grid g, SymmTable T, const double* q, const int* r0,
                                  const int* r1, const int* r2, double* d0, double* d1,
                                  double* d2)
{
   const long long qs = g.cells_ghost();
   long long tot[3], ss[3];
   for (int d = 0; d < 3; d++) {
      int e0, e1, e2;
      face_ext(g, d, e0, e1, e2);
      tot[d] = (long long)e0 * e1 * e2;
      ss[d] = side_size(g, d);
   }
   for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
        t < tot[0] + tot[1] + tot[2]; t += (long long)gridDim.x * blockDim.x) {
      int d = 0;
      long long r = t;
      while (r >= tot[d]) r -= tot[d++];
      int e0, e1, e2;
      face_ext(g, d, e0, e1, e2);
      const int i = (int)(r % e0) - (d != 0);
      const int j = (int)((r / e0) % e1) - (d != 1);
      const int k = (int)(r / ((long long)e0 * e1)) - (d != 2);
      const int ei = d == 0, ej = d == 1, ek = d == 2;
      double q1[4], q2[4], q2p[4];
      load_q(g, q, qs, i, j, k, q1);
      load_q(g, q, qs, i - ei, j - ej, k - ek, q2);
      const int* rot = d == 0 ? r0 : (d == 1 ? r1 : r2);
      double* out = d == 0 ? d0 : (d == 1 ? d1 : d2);
      const long long f = side_index(g, d, i, j, k);
      if (!qrotate(T, q2, rot[f], q2p))
         for (int m = 0; m < 4; m++) q2p[m] = NAN;  // invalid rotation index
      for (int m = 0; m < 4; m++) out[m * ss[d] + f] = S(q1[m], q2p[m]);
   }
}

// QUATGRAD_SIDE_SYMM: on the faces of normal d, the normal component is
// diff / h; a tangential component e averages the four e-differences
// around the face, the two on the upper cell's side rotated back by their
// faces' rotations (-iq) and the sum of the two on the lower side's
// neighbour faces rotated into the face's frame (iq of the face).
__global__ void k_quat_grad_side_symm(Grid g, SymmTable T, double hx, double hy, double hz,
                                      const double* d0, const double* d1, const double* d2,
                                      const int* r0, const int* r1, const int* r2,
                                      double* gxx, double* gyx, double* gzx, double* gxy,
                                      double* gyy, double* gzy, double* gxz, double* gyz,
                                      double* gzz)
{
   const double inv[3] = {__ddiv_rn(1.0, hx), __ddiv_rn(1.0, hy), __ddiv_rn(1.0, hz)};
   const double p25[3] = {M(0.25, inv[0]), M(0.25, inv[1]), M(0.25, inv[2])};
   const double* diff[3] = {d0, d1, d2};
   const int* rot[3] = {r0, r1, r2};
   double* out[3][3] = {{gxx, gyx, gzx}, {gxy, gyy, gzy}, {gxz, gyz, gzz}};  // [side][comp]
   long long ss[3];
   for (int d = 0; d < 3; d++) ss[d] = side_size(g, d);
   const long long nx = g.nfx(), ny = g.nfy(), nz = g.nfz();
   for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < nx + ny + nz;
        t += (long long)gridDim.x * blockDim.x) {
      int d, i, j, k;
      long long r = t;
      if (r < nx) {
         d = 0;
         g.split(r, g.fd0p, g.fd1, i, j, k);
      } else if ((r -= nx) < ny) {
         d = 1;
         g.split(r, g.fd0, g.fd1p, i, j, k);
      } else {
         r -= ny;
         d = 2;
         g.ijk(r, i, j, k);
      }
      const long long f = side_index(g, d, i, j, k);
      const int iqf = rot[d][f];
      for (int m = 0; m < 4; m++)
         out[d][d][m * ss[d] + f] = M(inv[d], diff[d][m * ss[d] + f]);
      // the two tangential directions, in the reference's order
      for (int e = 0; e < 3; e++) {
         if (e == d) continue;
         // offsets: +1 along e on this face's cell; -1 along d (lower cell)
         const int ue[3] = {e == 0, e == 1, e == 2};
         const int ld[3] = {d == 0, d == 1, d == 2};
         // d1: e-face of the upper cell's +e neighbour face; d2: the lower
         // cell's +e face; d3: the lower cell's e-face
         const int a1[3] = {i + ue[0], j + ue[1], k + ue[2]};
         const int a2[3] = {a1[0] - ld[0], a1[1] - ld[1], a1[2] - ld[2]};
         const int a3[3] = {i - ld[0], j - ld[1], k - ld[2]};
         const long long f1 = side_index(g, e, a1[0], a1[1], a1[2]);
         const long long f2 = side_index(g, e, a2[0], a2[1], a2[2]);
         const long long f3 = side_index(g, e, a3[0], a3[1], a3[2]);
         const long long fo = side_index(g, e, i, j, k);
         double v1[4], v2[4], v3[4], v1p[4], v2p[4], v4[4], v4p[4];
         for (int m = 0; m < 4; m++) {
            v1[m] = diff[e][m * ss[e] + f1];
            v2[m] = diff[e][m * ss[e] + f2];
            v3[m] = diff[e][m * ss[e] + f3];
         }
         bool ok = qrotate(T, v1, -rot[e][f1], v1p);
         ok = qrotate(T, v2, -rot[e][f2], v2p) && ok;
         for (int m = 0; m < 4; m++) v4[m] = A(v2p[m], v3[m]);
         ok = qrotate(T, v4, iqf, v4p) && ok;
         for (int m = 0; m < 4; m++) {
            const double v =
                ok ? M(p25[e], A(A(v4p[m], v1p[m]), diff[e][m * ss[e] + fo])) : NAN;
            out[d][e][m * ss[d] + f] = v;
         }
      }
   }
}

// host: the rotation table, built by rule in setqr's order
static SymmTable make_symm_table()
{
   SymmTable T;
   int n = 0;
   auto put = [&](double w, double x, double y, double z) {
      double* q = T.qr[n++];
      q[0] = w;
      q[1] = x;
      q[2] = y;
      q[3] = z;
      const double m = std::sqrt(w * w + x * x + y * y + z * z);
      const double minv = 1.0 / m;
      for (int c = 0; c < 4; c++) q[c] = q[c] * minv;
   };
   // +1, +i, +j, +k, then their negatives
   for (int s = 0; s < 2; s++)
      for (int a = 0; a < 4; a++) {
         double v[4] = {0, 0, 0, 0};
         v[a] = s ? -1.0 : 1.0;
         put(v[0], v[1], v[2], v[3]);
      }
   // two non-zero components: sign patterns (+,+), (-,+), (+,-), (-,-),
   // each over the pairs (0,1), (0,2), (0,3), (1,2), (1,3), (2,3)
   const double sg[4][2] = {{1, 1}, {-1, 1}, {1, -1}, {-1, -1}};
   for (int s = 0; s < 4; s++)
      for (int a = 0; a < 4; a++)
         for (int b = a + 1; b < 4; b++) {
            double v[4] = {0, 0, 0, 0};
            v[a] = sg[s][0];
            v[b] = sg[s][1];
            put(v[0], v[1], v[2], v[3]);
         }
   // four non-zero components: no minus, one minus (at 0..3), two minuses
   // (pairs in order), three minuses (the plus at 0..3), all minus
   put(1, 1, 1, 1);
   for (int a = 0; a < 4; a++) {
      double v[4] = {1, 1, 1, 1};
      v[a] = -1;
      put(v[0], v[1], v[2], v[3]);
   }
   for (int a = 0; a < 4; a++)
      for (int b = a + 1; b < 4; b++) {
         double v[4] = {1, 1, 1, 1};
         v[a] = v[b] = -1;
         put(v[0], v[1], v[2], v[3]);
      }
   for (int a = 0; a < 4; a++) {
      double v[4] = {-1, -1, -1, -1};
      v[a] = 1;
      put(v[0], v[1], v[2], v[3]);
   }
   put(-1, -1, -1, -1);
   for (int a = 0; a < 48; a++) {
      T.conj[a] = -1;
      for (int b = 0; b < 48; b++)
         if (T.qr[b][0] == T.qr[a][0] && T.qr[b][1] == -T.qr[a][1] &&
             T.qr[b][2] == -T.qr[a][2] && T.qr[b][3] == -T.qr[a][3])
            T.conj[a] = b;
   }
   const double pi = std::acos(-1.0);
   const double t = 2.0 * std::sin(pi / 16.0);
   T.thr = t * t;
   return T;
}

static const SymmTable& symm_table()
{
   static const SymmTable T = make_symm_table();
   return T;
}

}  // namespace ampe

using namespace ampe;

static unsigned symm_blocks(long long n)
{
   long long b = (n + 127) / 128;
   if (b > max_blocks(64)) b = max_blocks(64);
   return (unsigned)(b < 1 ? 1 : b);
}

static int check_symm_model(const ampe_model_t* m)
{
   if (check_model(m)) return AMPE_ERR_INVALID;
   if (m->dim != 3 || m->ng_side < 1) return AMPE_ERR_INVALID;
   return AMPE_OK;
}

extern "C" {

int ampe_quat_symm_table(double* qr, int* conj)
{
   const SymmTable& T = symm_table();
   for (int a = 0; a < 48; a++) {
      for (int c = 0; c < 4 && qr; c++) qr[4 * a + c] = T.qr[a][c];
      if (conj) conj[a] = T.conj[a] + 1;
   }
   return AMPE_OK;
}

int ampe_quat_symm_rotation(const ampe_model_t* m, const double* q, int* rot0, int* rot1,
                            int* rot2, void* stream)
{
   if (check_symm_model(m) || !q || !rot0 || !rot1 || !rot2) return AMPE_ERR_INVALID;
   const Grid g = make_grid(*m);
   const long long tot = (long long)(g.n0 + 1) * (g.n1 + 2) * (g.n2 + 2) +
                         (long long)(g.n0 + 2) * (g.n1 + 1) * (g.n2 + 2) +
                         (long long)(g.n0 + 2) * (g.n1 + 2) * (g.n2 + 1);
   k_quat_symm_rotation<<<symm_blocks(tot), 128, 0, (cudaStream_t)stream>>>(
       g, symm_table(), q, rot0, rot1, rot2);
   return launch_status();
}

int ampe_quat_fundamental(const ampe_model_t* m, double* q, void* stream)
{
   if (check_model(m) || m->dim != 3 || !q) return AMPE_ERR_INVALID;
   const Grid g = make_grid(*m);
   k_quat_fundamental<<<symm_blocks(g.cells()), 128, 0, (cudaStream_t)stream>>>(
       g, symm_table(), q);
   return launch_status();
}

int ampe_quat_diffs_symm(const ampe_model_t* m, const double* q, const int* rot0,
                         const int* rot1, const int* rot2, double* diff0, double* diff1,
                         double* diff2, void* stream)
{
   if (check_symm_model(m) || !q || !rot0 || !rot1 || !rot2 || !diff0 || !diff1 || !diff2)
      return AMPE_ERR_INVALID;
   const Grid g = make_grid(*m);
   const long long tot = (long long)(g.n0 + 1) * (g.n1 + 2) * (g.n2 + 2) +
                         (long long)(g.n0 + 2) * (g.n1 + 1) * (g.n2 + 2) +
                         (long long)(g.n0 + 2) * (g.n1 + 2) * (g.n2 + 1);
   k_quat_diffs_symm<<<symm_blocks(tot), 128, 0, (cudaStream_t)stream>>>(
       g, symm_table(), q, rot0, rot1, rot2, diff0, diff1, diff2);
   return launch_status();
}

int ampe_quat_grad_side_symm(const ampe_model_t* m, const double* diff0, const double* diff1,
                             const double* diff2, const int* rot0, const int* rot1,
                             const int* rot2, double* grad_x_xside, double* grad_y_xside,
                             double* grad_z_xside, double* grad_x_yside, double* grad_y_yside,
                             double* grad_z_yside, double* grad_x_zside, double* grad_y_zside,
                             double* grad_z_zside, void* stream)
{
   if (check_symm_model(m) || !diff0 || !diff1 || !diff2 || !rot0 || !rot1 || !rot2)
      return AMPE_ERR_INVALID;
   double* outs[9] = {grad_x_xside, grad_y_xside, grad_z_xside, grad_x_yside, grad_y_yside,
                      grad_z_yside, grad_x_zside, grad_y_zside, grad_z_zside};
   for (double* p : outs)
      if (!p) return AMPE_ERR_INVALID;
   const Grid g = make_grid(*m);
   const long long tot = g.nfx() + g.nfy() + g.nfz();
   k_quat_grad_side_symm<<<symm_blocks(tot), 128, 0, (cudaStream_t)stream>>>(
       g, symm_table(), m->dx[0], m->dx[1], m->dx[2], diff0, diff1, diff2, rot0, rot1, rot2,
       grad_x_xside, grad_y_xside, grad_z_xside, grad_x_yside, grad_y_yside, grad_z_yside,
       grad_x_zside, grad_y_zside, grad_z_zside);
   return launch_status();
}

}  // extern "C"
