// Quaternion orientation kernels (evolve_quat models).  q is stored as 4
// ghosted cell fields back to back (SAMRAI CellData depth 4).
//   k_quat_grad_modulus  QUATGRAD_MODULUS_FROM_SIDES_COMPACT (3d/quatgrad.m4:725-790)
//                        on the normal differences of QUATDIFFS/QUATGRAD_SIDE
//   k_quat_mobility      QUATMOBILITY 'p' (3d/mobility.m4:13-95)
//   k_quat_face_coef     COMPUTE_FACE_COEF3D (3d/quatfacops.m4:14-155) with the
//                        side gradients of QUATGRAD_SIDE (3d/quatgrad.m4:213-335)
//                        and eval_grad_normi (quat.f:1497-1537)
//   k_quat_rhs           COMPUTE_FLUX3D + ADD_QUAT_OP3D (3d/quatfacops.m4:227-311,
//                        596-657): q' = -M_q div(fc grad q)
//   k_quat_project       PROJECT3D (3d/quatfacops.m4:1022-1075) on the state
#include "common.cuh"
#include "quat.cuh"

namespace ampe {

__device__ __forceinline__ double eval_grad_normi(double g2, char type,
                                                  double floor2, double maxi)
{
   if (type == 'm') return g2 > floor2 ? pow(g2, -0.5) : maxi;
   if (type == 't') {
      const double gng2 = g2 * maxi * maxi;
      if (gng2 > 0.01) {
         const double gn = sqrt(g2);
         return tanh(maxi * gn) / gn;
      }
      return maxi * (1.0 - gng2 * (5.0 - 2.0 * gng2) / 15.0);
   }
   return pow(g2 + floor2, -0.5);
}

template <class R>
__device__ __forceinline__ R face_grad_norm2(const Grid& g, const double* dx,
                                             const R* q, int dir, int i,
                                             int j, int k)
{
   const long long qs = g.cells_ghost();
   const int ei = dir == 0, ej = dir == 1, ek = dir == 2;
   R gsum[3][4];
   for (int m = 0; m < 4; m++) {
      const R* Q = q + m * qs;
      for (int n = 0; n < g.dim; n++) {
         const R dinv = (R)(1.0 / dx[n]);
         if (n == dir) {
            gsum[n][m] = dinv * (Q[g.c(i, j, k)] - Q[g.c(i - ei, j - ej, k - ek)]);
            continue;
         }
         const int fi = n == 0, fj = n == 1, fk = n == 2;
         auto D = [&](int a, int b, int c) {
            return Q[g.c(a, b, c)] - Q[g.c(a - fi, b - fj, c - fk)];
         };
         const R p25 = (R)0.25 * dinv;
         gsum[n][m] = p25 * (D(i - ei + fi, j - ej + fj, k - ek + fk) + D(i - ei, j - ej, k - ek) +
                             D(i + fi, j + fj, k + fk) + D(i, j, k));
      }
   }
   R s = 0;
   for (int n = 0; n < g.dim; n++)
      for (int m = 0; m < 4; m++) s += gsum[n][m] * gsum[n][m];
   return s;
}

template <class R>
__global__ void k_quat_grad_modulus(Grid g, double dx0, double dx1, double dx2,
                                    const R* q, R* ogm)
{
   const long long qs = g.cells_ghost();
   const double dxs[3] = {dx0, dx1, dx2};
   for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
        t < g.cells(); t += (long long)gridDim.x * blockDim.x) {
      const int i = (int)(t % g.n0);
      const int j = (int)((t / g.n0) % g.n1);
      const int k = (int)(t / ((long long)g.n0 * g.n1));
      R s = 0;
      for (int d = 0; d < g.dim; d++) {
         const int ei = d == 0, ej = d == 1, ek = d == 2;
         const R dinv = (R)(1.0 / dxs[d]);
         for (int side = 0; side < 2; side++)
            for (int c = 0; c < 4; c++) {
               const R* qc = q + c * qs;
               const R gd = dinv * (qc[g.c(i + side * ei, j + side * ej, k + side * ek)] -
                                    qc[g.c(i + side * ei - ei, j + side * ej - ej,
                                           k + side * ek - ek)]);
               s += gd * gd;
            }
      }
      ogm[t] = sqrt((R)0.5 * s);
   }
}

template <class R>
__global__ void k_quat_mobility(Grid g, double mmin, double mscale,
                                const double* phi, R* mq)
{
   for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
        t < g.cells(); t += (long long)gridDim.x * blockDim.x) {
      const int i = (int)(t % g.n0);
      const int j = (int)((t / g.n0) % g.n1);
      const int k = (int)(t / ((long long)g.n0 * g.n1));
      const long long c = g.c(i, j, k);
      double p = phi[c];
      p = fmax(0.0, fmin(1.0, p));
      const double qf = 1.0 - p * p * p * (10.0 - 15.0 * p + 6.0 * p * p);
      mq[c] = (R)(mmin + (mscale - mmin) * qf);
   }
}

template <class QT, class R>
__global__ void k_quat_face_coef(ampe_model_t m, Grid g, const double* phi,
                                 const double* tfield, const QT* qlag,
                                 double scale, R* fc0, R* fc1, R* fc2)
{
   const double floor2 = m.quat_grad_floor * m.quat_grad_floor;
   const double maxi = 1.0 / m.quat_grad_floor;
   const double eps2 = m.epsilon_q * m.epsilon_q;
   const long long nx = g.nfx(), ny = g.nfy();
   const long long nz = g.dim == 3 ? g.nfz() : 0;
   for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
        t < nx + ny + nz; t += (long long)gridDim.x * blockDim.x) {
      int dir, i, j, k;
      long long r = t;
      if (r < nx) {
         dir = 0;
         i = (int)(r % (g.n0 + 1));
         j = (int)((r / (g.n0 + 1)) % g.n1);
         k = (int)(r / ((long long)(g.n0 + 1) * g.n1));
      } else if ((r -= nx) < ny) {
         dir = 1;
         i = (int)(r % g.n0);
         j = (int)((r / g.n0) % (g.n1 + 1));
         k = (int)(r / ((long long)g.n0 * (g.n1 + 1)));
      } else {
         r -= ny;
         dir = 2;
         i = (int)(r % g.n0);
         j = (int)((r / g.n0) % g.n1);
         k = (int)(r / ((long long)g.n0 * g.n1));
      }
      const int ei = dir == 0, ej = dir == 1, ek = dir == 2;
      const double phia = average_func(phi[g.c(i - ei, j - ej, k - ek)], phi[g.c(i, j, k)],
                                       m.avg_type);
      const double tempa = 0.5 * (temperature_at(m, g, tfield, i - ei, j - ej, k - ek) +
                                  temperature_at(m, g, tfield, i, j, k));
      const double diff = m.misorientation_factor * tempa * interp_func(phia, m.orient_interp1);
      const double hphi2 = interp_func(phia, m.orient_interp2);
      const double g2 = (double)face_grad_norm2<QT>(g, m.dx, qlag, dir, i, j, k);
      const double gni = eval_grad_normi(g2, m.quat_floor_type, floor2, maxi);
      const R v = (R)(scale * (-gni * diff - eps2 * hphi2));
      if (dir == 0) fc0[g.fx(i, j, k)] = v;
      if (dir == 1) fc1[g.fy(i, j, k)] = v;
      if (dir == 2) fc2[g.fz(i, j, k)] = v;
   }
}

template <class R>
__global__ void k_quat_rhs(Grid g, double dx0, double dx1, double dx2,
                           const R* fc0, const R* fc1, const R* fc2,
                           const R* mq, const R* q, double* out)
{
   const long long qs = g.cells_ghost(), N = g.cells();
   const R hinv[3] = {(R)(1.0 / dx0), (R)(1.0 / dx1), g.dim == 3 ? (R)(1.0 / dx2) : (R)0};
   for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < 4 * N;
        t += (long long)gridDim.x * blockDim.x) {
      const int c = (int)(t / N);
      const long long tt = t - c * N;
      const int i = (int)(tt % g.n0);
      const int j = (int)((tt / g.n0) % g.n1);
      const int k = (int)(tt / ((long long)g.n0 * g.n1));
      const R* qc = q + c * qs;
      auto flux = [&](int dir, int a, int b, int cc) {
         const int ei = dir == 0, ej = dir == 1, ek = dir == 2;
         const R f = dir == 0 ? fc0[g.fx(a, b, cc)]
                              : (dir == 1 ? fc1[g.fy(a, b, cc)] : fc2[g.fz(a, b, cc)]);
         return f * hinv[dir] * (qc[g.c(a, b, cc)] - qc[g.c(a - ei, b - ej, cc - ek)]);
      };
      R div = (flux(0, i + 1, j, k) - flux(0, i, j, k)) * hinv[0] +
              (flux(1, i, j + 1, k) - flux(1, i, j, k)) * hinv[1];
      if (g.dim == 3) div = div + (flux(2, i, j, k + 1) - flux(2, i, j, k)) * hinv[2];
      out[c * N + tt] = (double)((R)0 - mq[g.c(i, j, k)] * div);
   }
}

__global__ void k_quat_project(long long N, double* q)
{
   for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < N;
        t += (long long)gridDim.x * blockDim.x) {
      double s = 0.0;
      for (int c = 0; c < 4; c++) s += q[c * N + t] * q[c * N + t];
      const double f = 1.0 / sqrt(s);
      for (int c = 0; c < 4; c++) q[c * N + t] *= f;
   }
}

static unsigned nb(long long n)
{
   long long b = (n + 255) / 256;
   if (b > 152 * 32) b = 152 * 32;
   return (unsigned)(b < 1 ? 1 : b);
}

template <class R>
int quat_grad_modulus(const ampe_model_t& m, const Grid& g, const R* q, R* ogm,
                      cudaStream_t s)
{
   k_quat_grad_modulus<R><<<nb(g.cells()), 256, 0, s>>>(g, m.dx[0], m.dx[1], m.dx[2], q, ogm);
   return launch_status();
}

template <class R>
int quat_mobility(const ampe_model_t& m, const Grid& g, const double* phi, R* mq,
                  cudaStream_t s)
{
   k_quat_mobility<R><<<nb(g.cells()), 256, 0, s>>>(g, m.min_quat_mobility, m.quat_mobility,
                                                    phi, mq);
   return launch_status();
}

template <class QT, class R>
int quat_face_coef(const ampe_model_t& m, const Grid& g, const double* phi,
                   const double* tfield, const QT* qlag, double scale, R* fc0,
                   R* fc1, R* fc2, cudaStream_t s)
{
   const long long tot = g.nfx() + g.nfy() + (g.dim == 3 ? g.nfz() : 0);
   k_quat_face_coef<QT, R><<<nb(tot), 256, 0, s>>>(m, g, phi, tfield, qlag, scale, fc0, fc1, fc2);
   return launch_status();
}

template <class R>
int quat_rhs(const ampe_model_t& m, const Grid& g, const R* fc0, const R* fc1,
             const R* fc2, const R* mq, const R* q, double* out, cudaStream_t s)
{
   k_quat_rhs<R><<<nb(4 * g.cells()), 256, 0, s>>>(g, m.dx[0], m.dx[1], m.dx[2], fc0, fc1,
                                                   fc2, mq, q, out);
   return launch_status();
}

int quat_project(long long N, double* q, cudaStream_t s)
{
   k_quat_project<<<nb(N), 256, 0, s>>>(N, q);
   return launch_status();
}

#define INST(R)                                                                      \
   template int quat_grad_modulus<R>(const ampe_model_t&, const Grid&, const R*, R*, \
                                     cudaStream_t);                                  \
   template int quat_mobility<R>(const ampe_model_t&, const Grid&, const double*, R*, \
                                 cudaStream_t);                                      \
   template int quat_rhs<R>(const ampe_model_t&, const Grid&, const R*, const R*,    \
                            const R*, const R*, const R*, double*, cudaStream_t);
INST(double)
INST(float)
#undef INST
template int quat_face_coef<double, double>(const ampe_model_t&, const Grid&, const double*,
                                            const double*, const double*, double, double*,
                                            double*, double*, cudaStream_t);
template int quat_face_coef<double, float>(const ampe_model_t&, const Grid&, const double*,
                                           const double*, const double*, double, float*,
                                           float*, float*, cudaStream_t);

}  // namespace ampe

using namespace ampe;

extern "C" {

int ampe_quat_grad_modulus(const ampe_model_t* m, const double* q, double* ogm,
                           void* stream)
{
   if (check_model(m) || !q || !ogm) return AMPE_ERR_INVALID;
   return quat_grad_modulus<double>(*m, make_grid(*m), q, ogm, (cudaStream_t)stream);
}

int ampe_quat_mobility(const ampe_model_t* m, const double* phi, double* mq,
                       void* stream)
{
   if (check_model(m) || !phi || !mq) return AMPE_ERR_INVALID;
   if (m->quat_mobility_type != 'p') return AMPE_ERR_INVALID;
   return quat_mobility<double>(*m, make_grid(*m), phi, mq, (cudaStream_t)stream);
}

int ampe_quat_face_coef(const ampe_model_t* m, const double* phi,
                        const double* temp, const double* q, double* fc0,
                        double* fc1, double* fc2, void* stream)
{
   if (check_model(m) || !phi || !q || !fc0 || !fc1 || (m->dim == 3 && !fc2))
      return AMPE_ERR_INVALID;
   if (m->temp_mode == AMPE_TEMP_FIELD && !temp) return AMPE_ERR_INVALID;
   if (!(m->quat_grad_floor > 0.0)) return AMPE_ERR_INVALID;
   return quat_face_coef<double, double>(*m, make_grid(*m), phi, temp, q, 1.0, fc0, fc1, fc2,
                                 (cudaStream_t)stream);
}

int ampe_quat_rhs(const ampe_model_t* m, const double* fc0, const double* fc1,
                  const double* fc2, const double* mq, const double* q,
                  double* out, void* stream)
{
   if (check_model(m) || !fc0 || !fc1 || !mq || !q || !out || (m->dim == 3 && !fc2))
      return AMPE_ERR_INVALID;
   return quat_rhs<double>(*m, make_grid(*m), fc0, fc1, fc2, mq, q, out,
                           (cudaStream_t)stream);
}

}  // extern "C"
