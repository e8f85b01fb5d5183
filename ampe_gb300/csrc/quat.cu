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
// The FP32 face coefficients of the mixed path live in mixed.cu.
#include "common.cuh"
#include "quat.cuh"

namespace ampe {

template <int DIM, class R>
__global__ void k_quat_grad_modulus(Grid g, Inv3<R> dinv, const R* q, R* ogm)
{
   const long long qs = g.cells_ghost();
   for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
        t < g.cells(); t += (long long)gridDim.x * blockDim.x) {
      int i, j, k;
      g.ijk(t, i, j, k);
      R s = 0;
#pragma unroll
      for (int d = 0; d < DIM; d++) {
         const int ei = d == 0, ej = d == 1, ek = d == 2;
#pragma unroll
         for (int side = 0; side < 2; side++)
#pragma unroll
            for (int c = 0; c < 4; c++) {
               const R* qc = q + c * qs;
               const R gd = dinv.v[d] * (qc[g.c(i + side * ei, j + side * ej, k + side * ek)] -
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
      int i, j, k;
      g.ijk(t, i, j, k);
      const long long c = g.c(i, j, k);
      double p = phi[c];
      p = fmax(0.0, fmin(1.0, p));
      const double qf = 1.0 - p * p * p * (10.0 - 15.0 * p + 6.0 * p * p);
      mq[c] = (R)(mmin + (mscale - mmin) * qf);
   }
}

template <int DIM>
__global__ void k_quat_face_coef(ampe_model_t m, Grid g, Inv3<double> dinv,
                                 const double* phi, const double* tfield,
                                 const double* qlag, double scale, double* fc0,
                                 double* fc1, double* fc2)
{
   const double floor2 = m.quat_grad_floor * m.quat_grad_floor;
   const double maxi = 1.0 / m.quat_grad_floor;
   const double eps2 = m.epsilon_q * m.epsilon_q;
   const long long tot = g.nfx() + g.nfy() + (DIM == 3 ? g.nfz() : 0);
   for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < tot;
        t += (long long)gridDim.x * blockDim.x) {
      int dir, i, j, k;
      face_of(g, t, dir, i, j, k);
      const int ei = dir == 0, ej = dir == 1, ek = dir == 2;
      const double phia = average_func(phi[g.c(i - ei, j - ej, k - ek)], phi[g.c(i, j, k)],
                                       m.avg_type);
      const double tempa = 0.5 * (temperature_at(m, g, tfield, i - ei, j - ej, k - ek) +
                                  temperature_at(m, g, tfield, i, j, k));
      const double diff = m.misorientation_factor * tempa * interp_func(phia, m.orient_interp1);
      const double hphi2 = interp_func(phia, m.orient_interp2);
      const double g2 = face_grad_norm2<DIM, double>(g, dinv.v, qlag, dir, i, j, k);
      const double gni = eval_grad_normi(g2, m.quat_floor_type, floor2, maxi);
      const double v = scale * (-gni * diff - eps2 * hphi2);
      if (dir == 0) fc0[g.fx(i, j, k)] = v;
      if (dir == 1) fc1[g.fy(i, j, k)] = v;
      if (dir == 2) fc2[g.fz(i, j, k)] = v;
   }
}

template <int DIM, class R>
__global__ void k_quat_rhs(Grid g, Inv3<R> hinv, const R* fc0, const R* fc1,
                           const R* fc2, const R* mq, const R* q, double* out)
{
   const long long qs = g.cells_ghost(), N = g.cells();
   for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < N;
        t += (long long)gridDim.x * blockDim.x) {
      int i, j, k;
      g.ijk(t, i, j, k);
      // the six face coefficients are shared by the four components
      const R fxm = fc0[g.fx(i, j, k)], fxp = fc0[g.fx(i + 1, j, k)];
      const R fym = fc1[g.fy(i, j, k)], fyp = fc1[g.fy(i, j + 1, k)];
      R fzm = 0, fzp = 0;
      if (DIM == 3) {
         fzm = fc2[g.fz(i, j, k)];
         fzp = fc2[g.fz(i, j, k + 1)];
      }
      const long long cc = g.c(i, j, k);
      const R mqc = mq[cc];
#pragma unroll
      for (int c = 0; c < 4; c++) {
         const R* qc = q + c * qs;
         const R q0 = qc[cc];
         auto flux = [&](R f, int dir, R qa, R qb) { return f * hinv.v[dir] * (qa - qb); };
         R div = (flux(fxp, 0, qc[cc + 1], q0) - flux(fxm, 0, q0, qc[cc - 1])) * hinv.v[0] +
                 (flux(fyp, 1, qc[cc + g.sx], q0) - flux(fym, 1, q0, qc[cc - g.sx])) * hinv.v[1];
         if (DIM == 3)
            div = div + (flux(fzp, 2, qc[cc + g.sy], q0) - flux(fzm, 2, q0, qc[cc - g.sy])) *
                            hinv.v[2];
         out[c * N + t] = cvt<double, R>((R)0 - mqc * div);
      }
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
   if (b > max_blocks()) b = max_blocks();
   return (unsigned)(b < 1 ? 1 : b);
}

template <class R>
int quat_grad_modulus(const ampe_model_t& m, const Grid& g, const R* q, R* ogm,
                      cudaStream_t s)
{
   const Inv3<R> dinv = inv_spacing<R>(m);
   if (g.dim == 3)
      k_quat_grad_modulus<3, R><<<nb(g.cells()), 256, 0, s>>>(g, dinv, q, ogm);
   else
      k_quat_grad_modulus<2, R><<<nb(g.cells()), 256, 0, s>>>(g, dinv, q, ogm);
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

int quat_face_coef(const ampe_model_t& m, const Grid& g, const double* phi,
                   const double* tfield, const double* qlag, double scale,
                   double* fc0, double* fc1, double* fc2, cudaStream_t s)
{
   const long long tot = g.nfx() + g.nfy() + (g.dim == 3 ? g.nfz() : 0);
   const Inv3<double> dinv = inv_spacing<double>(m);
   if (g.dim == 3)
      k_quat_face_coef<3><<<nb(tot), 256, 0, s>>>(m, g, dinv, phi, tfield, qlag, scale, fc0,
                                                  fc1, fc2);
   else
      k_quat_face_coef<2><<<nb(tot), 256, 0, s>>>(m, g, dinv, phi, tfield, qlag, scale, fc0,
                                                  fc1, fc2);
   return launch_status();
}

template <class R>
int quat_rhs(const ampe_model_t& m, const Grid& g, const R* fc0, const R* fc1,
             const R* fc2, const R* mq, const R* q, double* out, cudaStream_t s)
{
   const Inv3<R> hinv = inv_spacing<R>(m);
   if (g.dim == 3)
      k_quat_rhs<3, R><<<nb(g.cells()), 256, 0, s>>>(g, hinv, fc0, fc1, fc2, mq, q, out);
   else
      k_quat_rhs<2, R><<<nb(g.cells()), 256, 0, s>>>(g, hinv, fc0, fc1, fc2, mq, q, out);
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
   return quat_face_coef(*m, make_grid(*m), phi, temp, q, 1.0, fc0, fc1, fc2,
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
