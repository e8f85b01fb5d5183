// CPU restatement of the quaternion orientation kernels on the hot path.
// TEST INFRASTRUCTURE ONLY.  q is stored as 4 ghosted cell fields back to
// back (SAMRAI CellData depth 4).
//   quatdiffs + quatgrad_side          3d/quatdiffs.m4:70-128, 3d/quatgrad.m4:213-335
//   quatgrad_modulus_from_sides_compact 3d/quatgrad.m4:725-790
//   quatmobility                       3d/mobility.m4:13-95
//   compute_face_coef3d, eval_grad_normi 3d/quatfacops.m4:14-155, quat.f:1497-1537
//   compute_flux3d + add_quat_op3d     3d/quatfacops.m4:227-311, 596-657
//   project3d                          3d/quatfacops.m4:1022-1075
#include <cstring>

#include "oracle_api.h"
#include "oracle_common.h"

using namespace orc;

namespace {

double eval_grad_normi(double g2, char type, double floor2, double maxi)
{
   if (type == 'm') return g2 > floor2 ? std::pow(g2, -0.5) : maxi;
   if (type == 't') {
      const double tol_taylor2 = 0.01;
      const double gng2 = g2 * maxi * maxi;
      if (gng2 > tol_taylor2) {
         const double gn = std::sqrt(g2);
         return std::tanh(maxi * gn) / gn;
      }
      return maxi * (1.0 - gng2 * (5.0 - 2.0 * gng2) / 15.0);
   }
   return std::pow(g2 + floor2, -0.5);  // 's'
}

// squared L2 norm over components and directions of the side gradient on
// face `dir` whose upper cell is (i,j,k) (quatgrad_side, then the loop of
// compute_face_coef3d: n outer, m inner)
double face_grad_norm2(const Layout& L, const double* dx, const double* q,
                       int dir, int i, int j, int k)
{
   const long qs = L.cells_ghost();
   auto Q = [&](int m, int a, int b, int c) { return q[m * qs + L.c(a, b, c)]; };
   const int ei = dir == 0, ej = dir == 1, ek = dir == 2;
   double g[3][4];
   for (int m = 0; m < 4; m++) {
      for (int n = 0; n < L.dim; n++) {
         const double dinv = 1.0 / dx[n];
         if (n == dir) {
            g[n][m] = dinv * (Q(m, i, j, k) - Q(m, i - ei, j - ej, k - ek));
            continue;
         }
         // tangential: average of the 4 differences along n around the face
         const int fi = n == 0, fj = n == 1, fk = n == 2;
         auto D = [&](int a, int b, int c) {  // diff along n ending at (a,b,c)
            return Q(m, a, b, c) - Q(m, a - fi, b - fj, c - fk);
         };
         const double p25 = 0.25 * dinv;
         g[n][m] = p25 * (D(i - ei + fi, j - ej + fj, k - ek + fk) + D(i - ei, j - ej, k - ek) +
                          D(i + fi, j + fj, k + fk) + D(i, j, k));
      }
   }
   double s = 0.0;
   for (int n = 0; n < L.dim; n++)
      for (int m = 0; m < 4; m++) s += g[n][m] * g[n][m];
   return s;
}

}  // namespace

extern "C" {

// |grad q| at cells from the normal differences on the cell's faces
void orc_quat_grad_modulus(const ampe_model_t* m, const double* q, double* ogm)
{
   Layout L(*m);
   const long qs = L.cells_ghost();
#pragma omp parallel for collapse(2) schedule(static)
   for (int k = 0; k < L.n2; k++)
      for (int j = 0; j < L.n1; j++)
         for (int i = 0; i < L.n0; i++) {
            double s = 0.0;
            for (int d = 0; d < L.dim; d++) {
               const int ei = d == 0, ej = d == 1, ek = d == 2;
               const double dinv = 1.0 / m->dx[d];
               for (int side = 0; side < 2; side++)
                  for (int c = 0; c < 4; c++) {
                     const double* qc = q + c * qs;
                     const double gd =
                         dinv * (qc[L.c(i + side * ei, j + side * ej, k + side * ek)] -
                                 qc[L.c(i + side * ei - ei, j + side * ej - ej,
                                        k + side * ek - ek)]);
                     s += gd * gd;
                  }
            }
            ogm[L.interior(i, j, k)] = std::sqrt(0.5 * s);
         }
}

// M_q(phi) on the interior (ghosted output layout)
void orc_quat_mobility(const ampe_model_t* m, const double* phi, double* mq)
{
   Layout L(*m);
   for (int k = 0; k < L.n2; k++)
      for (int j = 0; j < L.n1; j++)
         for (int i = 0; i < L.n0; i++) {
            double p = phi[L.c(i, j, k)];
            p = std::fmax(0.0, std::fmin(1.0, p));
            const double qf = 1.0 - p * p * p * (10.0 - 15.0 * p + 6.0 * p * p);
            mq[L.c(i, j, k)] =
                m->min_quat_mobility + (m->quat_mobility - m->min_quat_mobility) * qf;
         }
}

// face coefficients fc = -grad_normi * 2H Tbar p1(phibar) - eps_q^2 p2(phibar)
void orc_quat_face_coef(const ampe_model_t* m, const double* phi,
                        const double* temp, const double* qlag, double* fc0,
                        double* fc1, double* fc2)
{
   Layout L(*m);
   const double floor2 = m->quat_grad_floor * m->quat_grad_floor;
   const double maxi = 1.0 / m->quat_grad_floor;
   const double eps2 = m->epsilon_q * m->epsilon_q;
   for (int dir = 0; dir < L.dim; dir++) {
      const int ei = dir == 0, ej = dir == 1, ek = dir == 2;
      double* fc = dir == 0 ? fc0 : (dir == 1 ? fc1 : fc2);
#pragma omp parallel for collapse(2) schedule(static)
      for (int k = 0; k < L.n2 + ek; k++)
         for (int j = 0; j < L.n1 + ej; j++)
            for (int i = 0; i < L.n0 + ei; i++) {
               const double phia = average_func(phi[L.c(i - ei, j - ej, k - ek)],
                                                phi[L.c(i, j, k)], m->avg_type);
               const double tempa =
                   0.5 * (temperature_at(*m, temp, L, i - ei, j - ej, k - ek) +
                          temperature_at(*m, temp, L, i, j, k));
               const double diff = m->misorientation_factor * tempa *
                                   interp_func(phia, m->orient_interp1);
               const double hphi2 = interp_func(phia, m->orient_interp2);
               const double g2 = face_grad_norm2(L, m->dx, qlag, dir, i, j, k);
               const double gni = eval_grad_normi(g2, m->quat_floor_type, floor2, maxi);
               const long f = dir == 0 ? L.fx(i, j, k) : (dir == 1 ? L.fy(i, j, k) : L.fz(i, j, k));
               fc[f] = -gni * diff - eps2 * hphi2;
            }
   }
}

// q' = -M_q div(fc grad q) for the 4 components (interior output, 4N)
void orc_quat_rhs(const ampe_model_t* m, const double* fc0, const double* fc1,
                  const double* fc2, const double* mq, const double* q,
                  double* out)
{
   Layout L(*m);
   const long qs = L.cells_ghost(), N = L.cells();
   const double hinv[3] = {1.0 / m->dx[0], 1.0 / m->dx[1],
                           L.dim == 3 ? 1.0 / m->dx[2] : 0.0};
   for (int c = 0; c < 4; c++) {
      const double* qc = q + c * qs;
#pragma omp parallel for collapse(2) schedule(static)
      for (int k = 0; k < L.n2; k++)
         for (int j = 0; j < L.n1; j++)
            for (int i = 0; i < L.n0; i++) {
               auto flux = [&](int dir, int a, int b, int cc) {
                  const int ei = dir == 0, ej = dir == 1, ek = dir == 2;
                  const double f = dir == 0 ? fc0[L.fx(a, b, cc)]
                                            : (dir == 1 ? fc1[L.fy(a, b, cc)] : fc2[L.fz(a, b, cc)]);
                  return f * hinv[dir] * (qc[L.c(a, b, cc)] - qc[L.c(a - ei, b - ej, cc - ek)]);
               };
               double div = (flux(0, i + 1, j, k) - flux(0, i, j, k)) * hinv[0] +
                            (flux(1, i, j + 1, k) - flux(1, i, j, k)) * hinv[1];
               if (L.dim == 3) div += (flux(2, i, j, k + 1) - flux(2, i, j, k)) * hinv[2];
               out[c * N + L.interior(i, j, k)] = 0.0 - mq[L.c(i, j, k)] * div;
            }
   }
}

// project q (interior 4N) onto unit quaternions
void orc_quat_project(long ncells, double* q)
{
   for (long t = 0; t < ncells; t++) {
      double s = 0.0;
      for (int c = 0; c < 4; c++) s += q[c * ncells + t] * q[c * ncells + t];
      const double f = 1.0 / std::sqrt(s);
      for (int c = 0; c < 4; c++) q[c * ncells + t] *= f;
   }
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Symmetry-aware orientation, cubic symmetry, qlen 4 (quat.f:73-341,
// 3d/quatrotation.m4:12-147, 3d/quatdiffs.m4:131-219, 3d/quatgrad.m4:
// 376-679).  Side arrays here carry the ghost width m->ng_side (>= 1).
// ---------------------------------------------------------------------------
namespace {

// setqr (quat.f:165-288): the 48 rotations, (w, x, y, z) before quatset's
// normalisation, and the conjugate table
const double kQR[48][4] = {
    {1, 0, 0, 0},   {0, 1, 0, 0},   {0, 0, 1, 0},   {0, 0, 0, 1},   {-1, 0, 0, 0},
    {0, -1, 0, 0},  {0, 0, -1, 0},  {0, 0, 0, -1},  {1, 1, 0, 0},   {1, 0, 1, 0},
    {1, 0, 0, 1},   {0, 1, 1, 0},   {0, 1, 0, 1},   {0, 0, 1, 1},   {-1, 1, 0, 0},
    {-1, 0, 1, 0},  {-1, 0, 0, 1},  {0, -1, 1, 0},  {0, -1, 0, 1},  {0, 0, -1, 1},
    {1, -1, 0, 0},  {1, 0, -1, 0},  {1, 0, 0, -1},  {0, 1, -1, 0},  {0, 1, 0, -1},
    {0, 0, 1, -1},  {-1, -1, 0, 0}, {-1, 0, -1, 0}, {-1, 0, 0, -1}, {0, -1, -1, 0},
    {0, -1, 0, -1}, {0, 0, -1, -1}, {1, 1, 1, 1},   {-1, 1, 1, 1},  {1, -1, 1, 1},
    {1, 1, -1, 1},  {1, 1, 1, -1},  {-1, -1, 1, 1}, {-1, 1, -1, 1}, {-1, 1, 1, -1},
    {1, -1, -1, 1}, {1, -1, 1, -1}, {1, 1, -1, -1}, {1, -1, -1, -1}, {-1, 1, -1, -1},
    {-1, -1, 1, -1}, {-1, -1, -1, 1}, {-1, -1, -1, -1}};
const int kConj[48] = {1,  6,  7,  8,  5,  2,  3,  4,  21, 22, 23, 30, 31, 32, 27, 28,
                       29, 24, 25, 26, 9,  10, 11, 18, 19, 20, 15, 16, 17, 12, 13, 14,
                       44, 48, 43, 42, 41, 45, 46, 47, 37, 36, 35, 33, 38, 39, 40, 34};

void qnorm4(double* q)
{
   const double m = std::sqrt(q[0] * q[0] + q[1] * q[1] + q[2] * q[2] + q[3] * q[3]);
   double minv = 0.0;
   if (!(m < 1.e-15)) minv = 1.0 / m;
   for (int c = 0; c < 4; c++) q[c] = q[c] * minv;
}

struct Rotations {
   double qr[48][4];
   double thr;
   Rotations()
   {
      for (int a = 0; a < 48; a++) {
         for (int c = 0; c < 4; c++) qr[a][c] = kQR[a][c];
         qnorm4(qr[a]);
      }
      const double pi = std::acos(-1.0);
      const double t = 2.0 * std::sin(pi / 16.0);
      thr = t * t;
   }
};

const Rotations& rotations()
{
   static const Rotations R;
   return R;
}

void qmult4(const double* a, const double* b, double* q)
{
   q[0] = a[0] * b[0] - a[1] * b[1] - a[2] * b[2] - a[3] * b[3];
   q[1] = a[0] * b[1] + a[1] * b[0] + a[2] * b[3] - a[3] * b[2];
   q[2] = a[0] * b[2] + a[2] * b[0] + a[3] * b[1] - a[1] * b[3];
   q[3] = a[0] * b[3] + a[3] * b[0] + a[1] * b[2] - a[2] * b[1];
}

double qdiffsq4(const double* q1, const double* q2)
{
   double a[4], b[4], d[4];
   std::memcpy(a, q1, sizeof(a));
   std::memcpy(b, q2, sizeof(b));
   qnorm4(a);
   qnorm4(b);
   for (int c = 0; c < 4; c++) d[c] = b[c] - a[c];
   return d[0] * d[0] + d[1] * d[1] + d[2] * d[2] + d[3] * d[3];
}

// quatsymmrotate4; false where the reference stops (index out of range)
bool symm_rotate(const double* q, int iq, double* qp)
{
   if (iq == 0 || iq > 48 || iq < -48) return false;
   if (iq < 0) iq = kConj[-iq - 1];
   if (iq == 1)
      std::memcpy(qp, q, 4 * sizeof(double));
   else
      qmult4(q, rotations().qr[iq - 1], qp);
   return true;
}

// quatfindsymm4
void find_symm(const double* q1, const double* q2, int& iq, double* q2p)
{
   const Rotations& R = rotations();
   if (iq == 0 || iq > 48 || iq < -48) iq = 1;
   if (iq < 0) iq = kConj[-iq - 1];
   if (iq == 1)
      std::memcpy(q2p, q2, 4 * sizeof(double));
   else
      qmult4(q2, R.qr[iq - 1], q2p);
   double dsq = qdiffsq4(q1, q2p);
   if (dsq <= R.thr) return;
   double min_dsq = dsq, min_q[4];
   int min_iq = iq;
   std::memcpy(min_q, q2p, sizeof(min_q));
   for (int nn = 1; nn <= 48; nn++) {
      if (nn == iq) continue;
      if (nn == 1)
         std::memcpy(q2p, q2, 4 * sizeof(double));
      else
         qmult4(q2, R.qr[nn - 1], q2p);
      dsq = qdiffsq4(q1, q2p);
      if (dsq < min_dsq) {
         min_dsq = dsq;
         min_iq = nn;
         std::memcpy(min_q, q2p, sizeof(min_q));
      }
      if (dsq <= R.thr) break;
   }
   std::memcpy(q2p, min_q, sizeof(min_q));
   iq = min_iq;
}

// SIDE3d<d>(lo, hi, g) layout of the side arrays
struct SideLayout {
   int n0, n1, n2, g;
   long ext(int d, int a) const
   {
      const int n = a == 0 ? n0 : (a == 1 ? n1 : n2);
      return n + 2 * g + (a == d);
   }
   long size(int d) const { return ext(d, 0) * ext(d, 1) * ext(d, 2); }
   long at(int d, int i, int j, int k) const
   {
      return ((long)(k + g) * ext(d, 1) + (j + g)) * ext(d, 0) + (i + g);
   }
};

}  // namespace

extern "C" {

void orc_quat_symm_table(double* qr, int* conj)
{
   for (int a = 0; a < 48; a++) {
      for (int c = 0; c < 4; c++) qr[4 * a + c] = rotations().qr[a][c];
      conj[a] = kConj[a];
   }
}

// quatfindsymm4 for one pair (iq in/out), for tests of the search itself
int orc_quat_find_symm(const double* q1, const double* q2, int iq, double* q2p)
{
   find_symm(q1, q2, iq, q2p);
   return iq;
}

void orc_quat_symm_rotation(const ampe_model_t* m, const double* q, int* rot0, int* rot1,
                            int* rot2)
{
   Layout L(*m);
   const SideLayout S{L.n0, L.n1, L.n2, m->ng_side};
   const long qs = L.cells_ghost();
   int* rot[3] = {rot0, rot1, rot2};
   for (int d = 0; d < 3; d++) {
      const int ei = d == 0, ej = d == 1, ek = d == 2;
      for (int k = -1 + ek; k <= L.n2; k++)
         for (int j = -1 + ej; j <= L.n1; j++)
            for (int i = -1 + ei; i <= L.n0; i++) {
               double q1[4], q2[4], q2p[4];
               for (int c = 0; c < 4; c++) {
                  q1[c] = q[c * qs + L.c(i, j, k)];
                  q2[c] = q[c * qs + L.c(i - ei, j - ej, k - ek)];
               }
               int& iq = rot[d][S.at(d, i, j, k)];
               find_symm(q1, q2, iq, q2p);
            }
   }
}

void orc_quat_fundamental(const ampe_model_t* m, double* q)
{
   Layout L(*m);
   const long qs = L.cells_ghost();
   double q1[4] = {1.0, 0.0, 0.0, 0.0};
   qnorm4(q1);
   for (int k = 0; k < L.n2; k++)
      for (int j = 0; j < L.n1; j++)
         for (int i = 0; i < L.n0; i++) {
            double q2[4], q2p[4];
            for (int c = 0; c < 4; c++) q2[c] = q[c * qs + L.c(i, j, k)];
            int iq = 1;
            find_symm(q1, q2, iq, q2p);
            for (int c = 0; c < 4; c++) q[c * qs + L.c(i, j, k)] = q2p[c];
         }
}

void orc_quat_diffs_symm(const ampe_model_t* m, const double* q, const int* rot0,
                         const int* rot1, const int* rot2, double* diff0, double* diff1,
                         double* diff2)
{
   Layout L(*m);
   const SideLayout S{L.n0, L.n1, L.n2, m->ng_side};
   const long qs = L.cells_ghost();
   const int* rot[3] = {rot0, rot1, rot2};
   double* diff[3] = {diff0, diff1, diff2};
   for (int d = 0; d < 3; d++) {
      const int ei = d == 0, ej = d == 1, ek = d == 2;
      const long ss = S.size(d);
      for (int k = -1 + ek; k <= L.n2; k++)
         for (int j = -1 + ej; j <= L.n1; j++)
            for (int i = -1 + ei; i <= L.n0; i++) {
               double q2[4], q2p[4];
               for (int c = 0; c < 4; c++) q2[c] = q[c * qs + L.c(i - ei, j - ej, k - ek)];
               const long f = S.at(d, i, j, k);
               if (!symm_rotate(q2, rot[d][f], q2p))
                  for (int c = 0; c < 4; c++) q2p[c] = std::nan("");
               for (int c = 0; c < 4; c++)
                  diff[d][c * ss + f] = q[c * qs + L.c(i, j, k)] - q2p[c];
            }
   }
}

void orc_quat_grad_side_symm(const ampe_model_t* m, const double* diff0, const double* diff1,
                             const double* diff2, const int* rot0, const int* rot1,
                             const int* rot2, double* gxx, double* gyx, double* gzx,
                             double* gxy, double* gyy, double* gzy, double* gxz, double* gyz,
                             double* gzz)
{
   Layout L(*m);
   const SideLayout S{L.n0, L.n1, L.n2, m->ng_side};
   const double dinv[3] = {1.0 / m->dx[0], 1.0 / m->dx[1], 1.0 / m->dx[2]};
   const double p25[3] = {0.25 * dinv[0], 0.25 * dinv[1], 0.25 * dinv[2]};
   const double* diff[3] = {diff0, diff1, diff2};
   const int* rot[3] = {rot0, rot1, rot2};
   double* grad[3][3] = {{gxx, gyx, gzx}, {gxy, gyy, gzy}, {gxz, gyz, gzz}};  // [side][comp]
   for (int d = 0; d < 3; d++) {
      const int ld[3] = {d == 0, d == 1, d == 2};
      const long sd = S.size(d);
      for (int k = 0; k < L.n2 + ld[2]; k++)
         for (int j = 0; j < L.n1 + ld[1]; j++)
            for (int i = 0; i < L.n0 + ld[0]; i++) {
               const long f = S.at(d, i, j, k);
               for (int c = 0; c < 4; c++) grad[d][d][c * sd + f] = dinv[d] * diff[d][c * sd + f];
               for (int e = 0; e < 3; e++) {
                  if (e == d) continue;
                  const int ue[3] = {e == 0, e == 1, e == 2};
                  const long se = S.size(e);
                  // d1 = diff_e at (cell + e), d2 = diff_e at (cell + e - d),
                  // d3 = diff_e at (cell - d)
                  const long f1 = S.at(e, i + ue[0], j + ue[1], k + ue[2]);
                  const long f2 = S.at(e, i + ue[0] - ld[0], j + ue[1] - ld[1], k + ue[2] - ld[2]);
                  const long f3 = S.at(e, i - ld[0], j - ld[1], k - ld[2]);
                  const long fo = S.at(e, i, j, k);
                  double d1[4], d2[4], d1p[4], d2p[4], d4[4], d4p[4];
                  for (int c = 0; c < 4; c++) {
                     d1[c] = diff[e][c * se + f1];
                     d2[c] = diff[e][c * se + f2];
                  }
                  bool ok = symm_rotate(d1, -rot[e][f1], d1p);
                  ok = symm_rotate(d2, -rot[e][f2], d2p) && ok;
                  for (int c = 0; c < 4; c++) d4[c] = d2p[c] + diff[e][c * se + f3];
                  ok = symm_rotate(d4, rot[d][f], d4p) && ok;
                  for (int c = 0; c < 4; c++)
                     grad[d][e][c * sd + f] =
                         ok ? p25[e] * (d4p[c] + d1p[c] + diff[e][c * se + fo]) : std::nan("");
               }
            }
   }
}

}  // extern "C"
