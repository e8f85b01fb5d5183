// Mixed-precision kernels (mixed.cu) used by the stepper.
#pragma once

#include "common.cuh"

namespace ampe {

// FP32 copy of ThermoCoef for the mixed kernels
struct CoefF {
   float RT, iRT, dG[2], GB[2], L[2][4];
};

int build_coef_f(const ThermoCoef* tab, CoefF* tabf, int n, cudaStream_t s);

// FP32 constants of the mixed kernels, computed once on the host so that no
// kernel spends FP64-pipe cycles on per-thread divisions or conversions
struct MixParams {
   float dxi[3];       // 1/dx
   float flux_dinv[3]; // eps^2/dx (simple) or eps^2/(12 dx) (isotropic)
   float w, Mphi, Mc, Dl, Ds, qlR, qsR, ivm;
   int tdep, iso;
   // orientation term and quaternion equation
   float misor;        // 2H
   float eq2h, epsq2;  // eps_q^2 / 2, eps_q^2
   float qM, qMmin;    // M_q scale and floor
   float qfloor2, qmaxi;  // grad floor^2, 1/floor
   float T0, gdx;      // T = T0 (+ gdx (i + 1/2) for a gradient along x)
   char qfloor;        // eval_grad_normi type
   int pb;             // common type codes ('a', 'p', 'd'): specialised kernels
   // 2D anisotropic phase flux
   float eps, nu, kn;
   int qlen4;
   int kksc;  // "kks" composition flux form
   // T-dependent diffusivities per x index for analytic temperatures:
   // dq[i] = (D_L, D_S) at x-face i (0..n0, T averaged over cells i-1, i),
   // dq[n0 + 1 + i] = (D_L, D_S) at cell column i (y and z faces); null
   // with a stored temperature field or T-independent diffusion
   const float2* dq;
};

// composition flux weights per face, computed once per f evaluation and
// read by the RHS, the Jacobian-vector products and the composition
// preconditioner: EBS form A = (1-h) D_L, B = h D_S (flux = A grad cL +
// B grad cS); "kks" form A = D0, B = D_phi (flux = A grad c + B grad phi)
struct FaceW {
   float* A[3] = {nullptr, nullptr, nullptr};
   float* B[3] = {nullptr, nullptr, nullptr};
};

// 2D anisotropic phase flux per face and its Jacobian with respect to the
// face gradient (dphi/dx, dphi/dy): F[d], JA[d] = dF/d(dphi/dx),
// JB[d] = dF/d(dphi/dy) for x (d = 0) and y (d = 1) faces
// anisotropic phase flux per face (normal d) at the last f evaluation and
// its derivatives with respect to the face gradient of phi: JA = dF/dgx,
// JB = dF/dgy, JC = dF/dgz (3D)
struct AnisoF {
   float* F[3] = {nullptr, nullptr, nullptr};
   float* JA[3] = {nullptr, nullptr, nullptr};
   float* JB[3] = {nullptr, nullptr, nullptr};
   float* JC[3] = {nullptr, nullptr, nullptr};
   float* PO[2] = {nullptr, nullptr};  // 2D: orientation angle phi_o per face
};
// phi_o = acos(qbar) (2 acos for four-component q) per face, in FP64, once
// per orientation field: acos is ill-conditioned at qbar ~ +-1, where an
// FP32 qbar would cost up to ~1e-3 rad
// fills mp.dq (2 n0 + 1 entries) for analytic temperatures
int build_diff_table(const ampe_model_t& m, const MixParams& mp, const Grid& g,
                     float2* dq, cudaStream_t s);
int aniso_orientation_f32(const ampe_model_t& m, const Grid& g, const double* q,
                          AnisoF& a, cudaStream_t s);
// fill an AnisoF from the FP64 phase (differences formed in FP64, rounded
// once) and the orientation q (component 0, ghosted FP64), 2D only
int aniso_faces_f32(const ampe_model_t& m, const MixParams& mp, const Grid& g,
                    const double* ph, const double* q, AnisoF& a, cudaStream_t s);

// FP32 working set of the quaternion equation in the mixed path
struct QuatF32 {
   float* q = nullptr;    // ghosted q, 4 components
   float* dq = nullptr;   // ghosted q-part of a Jv direction, 4 components
   float* ogm = nullptr;  // |grad q| at cells (interior)
   float* mq = nullptr;   // M_q(phi) (ghosted layout)
   float* fc[3] = {nullptr, nullptr, nullptr};   // face coefficients
   float* dfc[3] = {nullptr, nullptr, nullptr};  // d fc / d phibar
};
MixParams make_mix_params(const ampe_model_t& m);
// guess_l / guess_s (may be null): surrogate initial guesses (3 FP32
// iterations from them, then the warm start clr / csr as fallback).
// list: cells + 1 ints of workspace (the cells for the FP64 polish and
// their count).
int kks_mixed(const ampe_model_t& m, const MixParams& mp, const Grid& g,
              const ThermoCoef* tab, const CoefF* tabf, const double* tfield,
              const double* phi,
              const double* conc, const float* guess_l, const float* guess_s,
              const float* clr, const float* csr, float* cl, float* cs,
              float* dF, int* list, unsigned long long* counters, cudaStream_t s);
// q: orientation of the 2D anisotropic flux (null otherwise); its face
// fluxes and Jacobians go to *an for the Jacobian-vector products
int rhs_mixed(const ampe_model_t& m, const MixParams& mp, const Grid& g,
              const double* tfield,
              const double* phi, float* pf, const float* cl, const float* cs,
              const float* dF, const float* ogm, const double* q, AnisoF* an,
              const double* cc, const FaceW& fw, double* phi_rhs, double* conc_rhs,
              cudaStream_t s);
// out = v - gamma J v; qf (null without quaternions) adds the q rows and
// the orientation term of the phase row
int jv_mixed(const ampe_model_t& m, const MixParams& mp, const Grid& g,
             const CoefF* tabf,
             const double* tfield, const float* pf, const float* cl,
             const float* cs, const float* dF, const float* v, double gamma,
             float* dphi, float* da, float* db, float* dcv, const QuatF32* qf,
             const AnisoF* an, const FaceW& fw, float* out, cudaStream_t s);
// composition preconditioner faces D = -gamma ((1-h) D_L + h D_S), FP32
int conc_faces_f32(const ampe_model_t& m, const MixParams& mp, const Grid& g,
                   const FaceW& fw, double gamma, float* const D[3], cudaStream_t s);
// |grad q| (from qf.q) and M_q(phi) at cells
int quat_cells_f32(const ampe_model_t& m, const MixParams& mp, const Grid& g,
                   const double* phi, QuatF32& qf, cudaStream_t s);
// fc = scale (-grad_normi 2H T p1 - eps_q^2 p2) into fc[], and (when dfc is
// non-null) d fc / d phibar at scale 1
int quat_faces_f32(const ampe_model_t& m, const MixParams& mp, const Grid& g,
                   const double* tfield, const float* pf, const float* q,
                   double scale, float* const fc[3], float* const dfc[3],
                   cudaStream_t s);

}  // namespace ampe
