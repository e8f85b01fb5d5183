// Allocation-free residual RMS norm (ampe_efo_residual_rms_noalloc).
//
// Some callers cannot allocate device memory: a host framework that manages
// every GPU byte through its own pool and hands this library a fixed budget,
// or a solver loop that must not call cudaMalloc/cudaFree because they
// synchronise the device.  For them this entry point takes no scratch
// argument and allocates nothing: its working memory (the residual field and
// the reduction partials) lives in one file-scope device array that each GPU
// loading the library keeps until exit.
#include <mutex>

#include "common.cuh"
#include "devvec.cuh"
#include "fac.cuh"

namespace {

// The library-owned working buffer.  In host code `g_rms_scratch` only names
// the symbol; its device address comes from cudaGetSymbolAddress.
static __device__ __align__(256) double g_rms_scratch[AMPE_NOALLOC_SCRATCH_DOUBLES];

constexpr int kMaxDevices = 64;
std::mutex g_mu;
double* g_dev_addr[kMaxDevices] = {nullptr};

// Device address of the buffer on the current device; looked up once per
// device (on its first call, which therefore must not be inside a stream
// capture) and kept for the life of the process, so it does not survive a
// cudaDeviceReset of that device.
int scratch_on_current_device(double** out)
{
   int dev = -1;
   if (cudaGetDevice(&dev) != cudaSuccess) return AMPE_ERR_CUDA;
   if (dev < 0 || dev >= kMaxDevices) return AMPE_ERR_INVALID;
   std::lock_guard<std::mutex> lock(g_mu);
   if (!g_dev_addr[dev]) {
      void* p = nullptr;
      if (cudaGetSymbolAddress(&p, g_rms_scratch) != cudaSuccess || !p)
         return AMPE_ERR_CUDA;
      g_dev_addr[dev] = (double*)p;
   }
   *out = g_dev_addr[dev];
   return AMPE_OK;
}

}  // namespace

using namespace ampe;

extern "C" int ampe_efo_residual_rms_noalloc(
    const ampe_model_t* m, const double* dface0, const double* dface1,
    const double* dface2, double d_const, const double* ccell, double c_const,
    const double* mcell, double m_const, const double* rhs, const double* u,
    double* rms, void* stream)
{
   if (check_model(m) || !rhs || !u || !rms) return AMPE_ERR_INVALID;
   if (dface0 && (!dface1 || (m->dim == 3 && !dface2))) return AMPE_ERR_INVALID;
   const Grid g = make_grid(*m);
   if (residual_rms_scratch_doubles(g) > (long long)AMPE_NOALLOC_SCRATCH_DOUBLES)
      return AMPE_ERR_TOO_LARGE;
   double* scratch = nullptr;
   const int rc = scratch_on_current_device(&scratch);
   if (rc) return rc;
   FacOp<double> op;
   op.D0 = dface0;
   op.D1 = dface1;
   op.D2 = dface2;
   op.dc = d_const;
   op.C = ccell;
   op.cc = c_const;
   op.M = mcell;
   op.mc = m_const;
   for (int d = 0; d < 3; d++) op.dxi[d] = d < m->dim ? 1.0 / m->dx[d] : 0.0;
   // every byte this call reads from the buffer it first writes itself:
   // the residual on all interior cells, then the partial sums of the blocks
   // it launches, so nothing has to be cleared between calls
   return residual_rms_into(op, g, rhs, u, scratch, rms, (cudaStream_t)stream);
}
