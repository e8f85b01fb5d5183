/*
 * ampe_gb300.h -- C-ABI of the GB300 implicit-step library (libampe_gb300.so).
 *
 * The library implements, for ONE uniform patch level on ONE GPU, the
 * per-level implicit step of AMPE's QuatModel with phase phi, binary
 * composition c and (optionally) a quaternion orientation field:
 *   - the phase right-hand side (PhaseFluxStrategy fluxes + COMPUTERHSPBG +
 *     FreeEnergyStrategy::addDrivingForce),
 *   - the per-cell KKS phase-concentration Newton solve
 *     (PhaseConcentrationsStrategy::computePhaseConcentrationsOnPatch),
 *   - the composition right-hand side (EBSCompositionRHSStrategy fluxes with
 *     temperature dependent or atomic-mobility diffusivities; the "kks"
 *     form),
 *   - the quaternion orientation equation (gradients, mobility, face
 *     coefficients, the symmetry-aware variants),
 *   - the Phase/Conc FAC operators (red-black Gauss-Seidel smoother,
 *     residual, within-level restrict/prolong),
 *   - a BDF Newton-GMRES stepper that plays the role of CVODE (fixed or
 *     variable steps, the temperature history evaluated at every f(t, y)),
 *   - a two-level composite FAC operator and solve (one refined box).
 *
 * Conventions shared by every entry point:
 *   - every array pointer is a DEVICE pointer unless the name says "host";
 *   - `stream` is a cudaStream_t passed as void* (NULL = legacy default);
 *   - a cell field is stored like a SAMRAI CellData<double> of depth 1 over
 *     its ghost box: x fastest, ghost width `ng` on both sides of every
 *     active direction (no z ghosts in 2D); strides sx=1, sy=n0+2ng,
 *     sz=(n0+2ng)*(n1+2ng);
 *   - a side (face) field with normal d is stored like a SAMRAI SideData with
 *     ghost width m->ng_side (0 by default): extent n_d+1+2g along d,
 *     n_e+2g along the others (no z ghosts in 2D), x fastest;
 *   - return value: 0 success, <0 error (AMPE_ERR_*), >0 a count of cells
 *     or cycles that did not converge (never an abort).
 * Device memory is allocated only by ampe_stepper_create (the stepper's
 * whole workspace), ampe_mlp_create (the network and its training buffers)
 * and ampe_mlp_generate (the sample set); every other entry point works in
 * the caller's buffers (or, for ampe_efo_residual_rms_noalloc, in one
 * library-owned static buffer).
 */
#ifndef AMPE_GB300_H
#define AMPE_GB300_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

#define AMPE_OK 0
#define AMPE_ERR_INVALID (-1)
#define AMPE_ERR_CUDA (-2)
#define AMPE_ERR_NOT_CONVERGED (-3)
#define AMPE_ERR_NO_DEVICE (-4)
#define AMPE_ERR_TOO_LARGE (-5) /* level too large for a fixed-size buffer */

/* phase flux discretisations (PhaseFluxStrategyFactory.h:12-40) */
#define AMPE_FLUX_SIMPLE 0      /* gradient_flux, quatrhs.m4 */
#define AMPE_FLUX_ISOTROPIC 1   /* compute_flux_isotropic, 2d/quatrhs.m4:106 */
#define AMPE_FLUX_ANISOTROPIC 2 /* anisotropic_gradient_flux 2d:154 / 3d:180 */

/* free-energy models (FreeEnergyStrategyFactory.h:46-250) */
#define AMPE_THERMO_DILUTE 0  /* KKSdiluteBinary */
#define AMPE_THERMO_CALPHAD 1 /* CALPHADFreeEnergyStrategyBinary */

/* composition flux forms: EBSCompositionRHSStrategy (M_c div((1-h)D_L grad cL
 * + h D_S grad cS), h = diff_interp) and KKSCompositionRHSStrategy (M_c
 * div(D0 grad c + D0 h'(phibar)(cLbar - cSbar) grad phi), D0 = (1-h)D_L +
 * h D_S, h = energy_interp; KKSCompositionRHSStrategy.cc:98-441) */
#define AMPE_CONC_EBS 0
#define AMPE_CONC_KKS 1

#define AMPE_DIFF_ARRHENIUS 0
#define AMPE_DIFF_MOBILITY 1

/* temperature sources */
#define AMPE_TEMP_CONSTANT 0 /* T = T0 everywhere */
#define AMPE_TEMP_GRADIENT 1 /* T = T0 + gradT * (i + 0.5) * dx[0], analytic */
#define AMPE_TEMP_FIELD 2    /* T read from a cell field */

#define AMPE_MAX_TSEG 6

/* Pure-species Gibbs energy G(T) in J/mol, piecewise in T
 * (thermodynamic_data/calphadAuNi.dat:1-49):
 *   G = a + b T + c T ln T + d2 T^2 + d3 T^3 + d4 T^4 + d7 T^7
 *       + dm1 / T + dm9 / T^9   on [tc[s], tc[s+1]). */
typedef struct ampe_gterm {
   int nseg;
   double tc[AMPE_MAX_TSEG + 1];
   double a[AMPE_MAX_TSEG], b[AMPE_MAX_TSEG], c[AMPE_MAX_TSEG];
   double d2[AMPE_MAX_TSEG], d3[AMPE_MAX_TSEG], d4[AMPE_MAX_TSEG];
   double d7[AMPE_MAX_TSEG], dm1[AMPE_MAX_TSEG], dm9[AMPE_MAX_TSEG];
} ampe_gterm_t;

/* CALPHAD atomic mobilities of a binary alloy, one set per species and phase
 * (CALPHADMobility::initialize, CALPHADMobility.cc:17-150: the
 * MobilityParameters block of a thermodynamic database).  For species s in
 * phase p (0 liquid "PhaseL", 1 solid "PhaseA"):
 *   q[s][p][i]  = (a0, a1, a2, a3) of qA (i = 0) and qB (i = 1):
 *                 Q_i(T) = a0 + R T ln(a1) + a2 T ln(T) + a3 / T
 *                 (a2 = a3 = 0 when the database gives two values);
 *   qq[s][p][n] = (a0, a1) of q<n>AB, n = 0..3: a0 + R T ln(a1), (0, 1)
 *                 when absent. */
typedef struct ampe_mobility {
   double q[2][2][2][4];
   double qq[2][2][4][2];
} ampe_mobility_t;

typedef struct ampe_model {
   /* ---- grid: one uniform periodic patch level ---- */
   int dim;      /* 2 or 3 */
   int n[3];     /* interior cells; n[2]=1 in 2D */
   int ng;       /* ghost width of cell fields (>=1) */
   double dx[3]; /* mesh spacing */

   /* ---- phase equation (QuatModelParameters, PhaseRHSStrategyWithQ) ---- */
   int flux_type;       /* AMPE_FLUX_* */
   double epsilon_phi;  /* gradient energy coefficient epsilon */
   double aniso_eps;    /* 2D: nu of eps(1+nu cos k(theta-phi)); 3D: eps4 */
   int aniso_k;         /* 2D anisotropy fold knumber */
   int qlen;            /* quaternion components seen by the flux (2 or 4) */
   double phase_well_scale; /* w of -w g'(phi) */
   double phase_mobility;   /* constant M_phi */
   char well_type;      /* 'd' double well 16 phi^2 (1-phi)^2, 's' single */
   char energy_interp;  /* h(phi) of the driving force, functions.f types */
   char conc_interp;    /* h(phi) of c=(1-h)cL+h cS */
   char diff_interp;    /* h(phi) weighting the phase diffusivities */
   char avg_type;       /* 'a' arithmetic, 'h' harmonic face average of phi */
   char orient_interp1, orient_interp2; /* p1, p2 of the orientation term */
   char pad0;
   int with_orient;     /* add -2H T p1'|grad q| - p2' eps_q^2/2 |grad q|^2 */
   double misorientation_factor; /* 2 H */
   double epsilon_q;

   /* ---- composition equation (EBSCompositionRHSStrategy) ---- */
   double conc_mobility; /* M_c */
   double D_liquid, Q_liquid, D_solid, Q_solid; /* D0 exp(-Q/RT) */

   /* ---- thermodynamics ---- */
   int thermo;                 /* AMPE_THERMO_* */
   double inv_molar_volume[2]; /* 1e-6/Vm for liquid, solid (J/mol->pJ/um^3) */
   double dilute_Tm, dilute_m, dilute_k; /* meltingT, liquidus_slope, keq */
   ampe_gterm_t g[2][2];       /* [species A,B][phase L,S] */
   double L[2][4][2];          /* [phase L,S][RK order k][a,b]: Lk=a+b T */
   int newton_max_its;
   double newton_tol;          /* on |dx| of the (cL,cS) Newton update */

   /* ---- temperature ---- */
   int temp_mode;  /* AMPE_TEMP_* */
   double T0;
   double gradT;   /* K per unit length along x */

   /* ---- quaternion orientation field (QuatFACOps, QuatModelParameters) ---- */
   int evolve_quat;          /* 1: q (4 components) is part of the state */
   double quat_mobility;     /* orient_mobility (scale of M_q) */
   double min_quat_mobility; /* min_orient_mobility (1e-6 default) */
   double quat_grad_floor;   /* orient_grad_floor (1e-2 default) */
   char quat_floor_type;     /* 'm' max, 's' smooth, 't' tanh (quat.f:1497) */
   char quat_mobility_type;  /* 'p' 1 - pbg(phi) (3d/mobility.m4:13-95) */
   char pad1[6];

   /* ---- composition flux form (QuatModelParameters.cc:203-222 rhs_form) ---- */
   int conc_form;  /* AMPE_CONC_EBS or AMPE_CONC_KKS */
   /* ghost width of the side (face) arrays the leaf entry points take and
    * return (SAMRAI SideData ghost width, passed by the reference per array,
    * e.g. fluxng beside phaseng in GRADIENT_FLUX, QuatFort.h:50-61); 0 by
    * default.  Only interior faces are read or written.  The stepper keeps
    * its own face arrays and ignores it. */
   int ng_side;

   /* ---- composition diffusivities of the "ebs" form (diffusion_type,
    * QuatModelParameters.cc:238-249; the strategy QuatModel.cc:375-395 and
    * CompositionDiffusionStrategyFactory.h:36-95 build) ---- */
   int conc_diffusion; /* AMPE_DIFF_ARRHENIUS: D_liquid, D_solid above
                        * (temperature_dependent); AMPE_DIFF_MOBILITY: from
                        * `mobility` at the face means of cL, cS and T
                        * (composition_dependent, the reference's default for
                        * "ebs"; see ampe_conc_diffusion_mobility) */
   int pad2;
   ampe_mobility_t mobility;

   /* ---- temperature in time (ScalarTemperatureStrategy::
    * getCurrentTemperature, ScalarTemperatureStrategy.cc:57-73;
    * GradientTemperatureStrategy.cc:124-131), set at every f(t, y) as
    * QuatIntegrator::evaluateRHSFunction does (QuatIntegrator.cc:3191):
    * T0(t) = T0 + dTdt t with T0 the temperature at t = 0; in
    * AMPE_TEMP_CONSTANT held at T_target once past it (dTdt < 0: below
    * it; dTdt > 0 and T_target > 0: above it).  The stepper evaluates
    * each BDF step's Newton iterations at the step's end time and f(y_n)
    * at its start.  dTdt = 0: T0 fixed (ampe_stepper_set_temperature
    * changes it; with dTdt != 0 that call is refused). */
   double dTdt;
   double T_target;
} ampe_model_t;

/* Integrator / preconditioner controls (QuatIntegrator.cc:278-301,
 * samrai/FACPreconditioner.cc:79-106, EllipticFACOps.cc:282-286). */
typedef struct ampe_step_params {
   double dt;          /* fixed step size */
   int max_order;      /* 1 or 2 (BDF order after the first step) */
   double atol, rtol;  /* WRMS weights 1/(rtol |y| + atol) */
   int max_newton;     /* Newton corrections per step (CVODE maxcor=3) */
   double newton_coef; /* Newton test: del*min(1,crate) <= newton_coef */
   int max_krylov;     /* GMRES Krylov dimension (5), no restarts */
   double lin_coef;    /* GMRES test: WRMS(P^-1 r) <= lin_coef*newton_coef */
   int precond;        /* 0 none, 1 single-level red-black, 2 multigrid */
   int fac_max_cycles; /* FAC cycles per block solve (10) */
   int rb_sweeps;      /* red-black sweeps per cycle (coarse solve) */
   double rb_tol;      /* red-black early-exit tolerance (<0 = never) */
   int mg_levels;      /* multigrid levels incl. the fine one */
   int mg_pre, mg_post, mg_coarse_sweeps;
   int precision;      /* 0 FP64, 1 mixed (FP32 preconditioner + Jv) */
   int surrogate;      /* MLP initial guess for the cL,cS Newton: 1 on cold
                        * starts only, 2 for every solve (0: none) */
   int max_retries;    /* step-size halvings after a Newton failure */
   /* 0: fixed steps of size dt.  1: variable steps chosen by CVODE's local
    * error test and step-size / order rules (CVODESolver.cc:112-258 with
    * CVodeSStolerances(rtol, atol), CVodeSetMaxOrd(max_order),
    * CVodeSetInitStep(dt), CVodeSetMaxStep(h_max), CVodeSetMinStep(h_min);
    * QuatIntegrator.cc:1571-1596), orders 1 and 2. */
   int adaptive;
   double h_max;       /* largest step (<= 0: none) */
   double h_min;       /* smallest step before a failure is final (>= 0) */
} ampe_step_params_t;

typedef struct ampe_step_stats {
   long long steps, newton_iters, gmres_iters, rhs_evals, precond_solves,
       precond_setups, fac_cycles, newton_fail, kks_iters, kks_fallback,
       kks_fail, step_retries, kks_fp64_cells;
   double t;
   /* variable steps: local error test failures, the last accepted step's
    * size and order, the next step's size and order */
   long long err_test_fails;
   double h_last, h_next;
   int q_last, q_next;
} ampe_step_stats_t;

/* ---------------------------------------------------------------------
 * Leaf kernels (one per reference Fortran/C++ routine they replace).
 * ------------------------------------------------------------------- */

/* Periodic ghost fill of one cell field (SAMRAI RefineSchedule::fillData for
 * a periodic level, QuatIntegrator.cc:2948-2954). */
int ampe_fill_ghosts(const ampe_model_t* m, double* field, void* stream);

/* Replaces GRADIENT_FLUX (QuatFort.h:50, 3d/quatrhs.m4:12-66),
 * COMPUTE_FLUX_ISOTROPIC (QuatFort.h:62, 2d/quatrhs.m4:106-151) and
 * ANISOTROPIC_GRADIENT_FLUX (QuatFort.h:75, 2d/quatrhs.m4:154-256,
 * 3d/quatrhs.m4:180-349) selected by m->flux_type.  quat: qlen cell fields
 * back to back (may be NULL unless anisotropic). */
int ampe_phase_flux(const ampe_model_t* m, const double* phase,
                    const double* quat, double* flux0, double* flux1,
                    double* flux2, void* stream);

/* Replaces COMPUTERHSPBG (QuatFort.h:90, 3d/quatrhs.m4:357-512) with
 * three_phase=0; temp and orient_grad_mod may be NULL when with_orient=0.
 * rhs has ghost width 0. */
int ampe_computerhspbg(const ampe_model_t* m, const double* flux0,
                       const double* flux1, const double* flux2,
                       const double* temp, const double* phi,
                       const double* orient_grad_mod, double* rhs,
                       void* stream);

/* Replaces KKSdiluteBinary::addDrivingForceOnPatch (KKSdiluteBinary.cc:
 * 507-626) and CALPHADFreeEnergyStrategyBinary::addDrivingForce (.cc:
 * 521-670, two phases): rhs += h'(phi)[(fL - fS) - muS(cS)(cL - cS)]. */
int ampe_add_driving_force(const ampe_model_t* m, const double* temp,
                           const double* phi, const double* cl,
                           const double* cs, double* rhs, void* stream);

/* Replaces PhaseConcentrationsStrategy::computePhaseConcentrationsOnPatch
 * (PhaseConcentrationsStrategy.h:27-35; CALPHAD .cc:162-454, dilute
 * KKSdiluteEquilibriumPhaseConcentrationsStrategy.cc:41-190): per cell of
 * the ghost box solve c=(1-h)cL+h cS, muL(cL)=muS(cS), starting from
 * (cl_ref, cs_ref).  counters (device, may be NULL): [0] += Newton
 * iterations, [1] += cells not converged. */
int ampe_phase_concentrations(const ampe_model_t* m, const double* temp,
                              const double* phi, const double* conc,
                              const double* cl_ref, const double* cs_ref,
                              double* cl, double* cs,
                              unsigned long long* counters, void* stream);

/* Replaces CONCENTRATION_PFMDIFFUSION_OF_TEMPERATURE (ConcFort.h:223,
 * 3d/concentrationdiffusion.m4:310-428) on interior faces: face D_L, D_S. */
int ampe_conc_diffusion(const ampe_model_t* m, const double* phi,
                        const double* temp, double* dl0, double* dl1,
                        double* dl2, double* ds0, double* ds1, double* ds2,
                        void* stream);

/* Composition flux of the "kks" form (AMPE's default rhs_form,
 * KKSCompositionRHSStrategy.cc:98-441): CONCENTRATION_PFMDIFFUSION
 * (ConcFort.h, 3d/concentrationdiffusion.m4:14-128; h = energy_interp) for
 * D0, the coupling D0 h'(phibar)(cLbar - cSbar) of
 * setDiffCoeffForPhaseOnPatch (:166-310) and CONCENTRATIONFLUX
 * (ConcFort.h:16, 3d/concentrationrhs.m4:14-104), fused:
 * flux = (D0 (c_up - c_lo) + D_phi (phi_up - phi_lo)) / dx on every face.
 * phi, conc, cl, cs ghosted; flux side arrays.  Then
 * ampe_computerhsconcentration gives c'. */
int ampe_conc_flux_kks(const ampe_model_t* m, const double* phi,
                       const double* temp, const double* conc, const double* cl,
                       const double* cs, double* flux0, double* flux1,
                       double* flux2, void* stream);

/* Replaces ADD_FLUX (ConcFort.h:139, 3d/flux.m4:15-100) for depth 1:
 * flux_d += D_d * (u_i - u_{i-1}) / dx_d. */
int ampe_add_flux(const ampe_model_t* m, const double* u, const double* d0,
                  const double* d1, const double* d2, double* flux0,
                  double* flux1, double* flux2, void* stream);

/* Replaces ADDCONCENTRATIONFLUXFROMGRADT (3d/concentrationrhs.m4:460-535,
 * 2d:369-437; EBSCompositionRHSStrategyWithGradT::addFluxFromGradTonPatch,
 * EBSCompositionRHSStrategyWithGradT.cc:488-525, called by
 * QuatIntegrator::evaluateConcentrationRHS, QuatIntegrator.cc:2604-2607):
 * flux_d -= Mq_d (T_i - T_{i-1}) / (dx_d Tbar), Tbar = average_func of the
 * two cells (avg_type).  temp ghosted; mq0..2 side arrays (the thermal-
 * diffusion mobility of the strategy); flux side arrays, updated. */
int ampe_add_flux_from_grad_t(const ampe_model_t* m, const double* temp,
                              const double* mq0, const double* mq1,
                              const double* mq2, double* flux0, double* flux1,
                              double* flux2, void* stream);

/* Replaces ADDCONCENTRATIONFLUXFROMANTITRAPPING for one composition
 * (3d/concentrationrhs.m4:537-700, 2d:439-527;
 * EBSCompositionRHSStrategy::addFluxFromAntitrappingonPatch,
 * EBSCompositionRHSStrategy.cc:441-520, QuatIntegrator.cc:2608-2612): on
 * faces with |grad phi| > 1e-8, flux += alpha (dphi_n / |grad phi|)
 * (cLbar - cSbar) dphidt_bar.  phi, cl, cs, dphidt ghosted (corner ghosts
 * filled); flux side arrays, updated. */
int ampe_add_flux_from_antitrapping(const ampe_model_t* m, const double* phi,
                                    const double* cl, const double* cs,
                                    const double* dphidt, double alpha,
                                    double* flux0, double* flux1,
                                    double* flux2, void* stream);

/* Phase mobility of the Kim model with infinite interface mobility,
 * binary alloy (KimMobilityStrategyInfMob::evaluateMobility,
 * KimMobilityStrategyInfMob.cc:49-80, on every cell of the ghost box as
 * KimMobilityStrategy::update, KimMobilityStrategy.cc:204-300, with the
 * zeta of the liquid phase computed, i.e. no zeta factor given):
 * M = factor / zeta, zeta = (cL - cS)^2 f_L''(cL) / (D0 exp(-Q0/(R T)))
 * x 1e-6 / molar_volume, factor = 16 w / (3 eps^2 a2), a2 = 47/60 for
 * energy_interp 'p', 1/2 for 'h' (kks_mobility_factor, KKStools.cc:13-30;
 * other types AMPE_ERR_INVALID).  cl, cs, temp (AMPE_TEMP_FIELD only) and
 * mobility ghosted.  The finite-mobility variant
 * (KimMobilityStrategyFiniteMob.cc) is the constant mu / (3 sqrt(2) xi),
 * xi = eps / sqrt(16 w). */
int ampe_kim_mobility(const ampe_model_t* m, const double* temp,
                      const double* cl, const double* cs, double D0,
                      double Q0, double molar_volume, double* mobility,
                      void* stream);

/* Composition-dependent diffusion from atomic mobilities, binary alloy
 * (MobilityCompositionDiffusionStrategy::setDiffusion,
 * MobilityCompositionDiffusionStrategy.cc:83-611, with
 * computeDiffusionMobilityBinaryPhase, CALPHADMobility.cc:196-215): on every
 * interior face, with T, cL and cS the arithmetic means of the two cells,
 *   D_p = c(1-c) (c M_1 + (1-c) M_0) 1e12 * f_p''(c)   (c = cL or cS),
 *   M_s = exp(dG_s / (R T)) / (R T),
 *   dG_s = c Q_A + (1-c) Q_B + c (1-c) sum_n q_n (2c-1)^n,
 * f_p'' the phase's free-energy curvature in J/mol, and
 *   dl = (1 - h) D_L,  ds = h D_S,  h = diff_interp(avg_type(phi, phi')).
 * Optional coef_l0..2, coef_s0..2 (may be NULL) receive D_L and D_S
 * themselves (the reference's diffusion_coeff side data).  Cell fields
 * ghosted with m->ng, side fields with m->ng_side; temp is read only for
 * AMPE_TEMP_FIELD. */
int ampe_conc_diffusion_mobility(const ampe_model_t* m, const ampe_mobility_t* mob,
                                 const double* phi, const double* temp,
                                 const double* cl, const double* cs, double* dl0,
                                 double* dl1, double* dl2, double* ds0, double* ds1,
                                 double* ds2, double* coef_l0, double* coef_l1,
                                 double* coef_l2, double* coef_s0, double* coef_s1,
                                 double* coef_s2, void* stream);

/* Replaces COMPUTERHSCONCENTRATION (ConcFort.h:419,
 * 3d/concentrationrhs.m4:412-456): rhs = M_c div(flux). */
int ampe_computerhsconcentration(const ampe_model_t* m, const double* flux0,
                                 const double* flux1, const double* flux2,
                                 double* rhs, void* stream);

/* ---------------------------------------------------------------------
 * Fused hot-path kernels.
 * ------------------------------------------------------------------- */

/* Whole phi+c right-hand side of QuatIntegrator::evaluateRHSFunction
 * (QuatIntegrator.cc:3134-3295) for given cL, cS (already computed on the
 * ghost box): phase flux + well + driving force times M_phi, and
 * composition M_c div(D_L grad cL + D_S grad cS), D_L and D_S of the
 * model's conc_diffusion (AMPE_DIFF_MOBILITY: at the face means of these
 * cL, cS).  phi, cl, cs, temp with ghosts filled; outputs with ghost
 * width 0. */
int ampe_rhs_phase_conc(const ampe_model_t* m, const double* phi,
                        const double* quat, const double* temp,
                        const double* cl, const double* cs, double* phi_rhs,
                        double* conc_rhs, void* stream);

/* ---------------------------------------------------------------------
 * FAC operator kernels, A u = C u + M div(D grad u)
 * (EllipticFACOps, 3d/ellipticfacops.m4).  Cell arrays have ghost width
 * m->ng; dface0..2 are side arrays (NULL -> constant d_const); mcell /
 * ccell NULL -> constants m_const / c_const.
 * ------------------------------------------------------------------- */

/* One colour of EFO_RBGSWITHFLUXMAX* (3d/ellipticfacops.m4:83-177,
 * 267-359; EllipticFACOps.cc:2294-2515): flux from the current u, then
 * u += r/diag on cells of colour `offset` ((i+j+k)%2 == offset).  If
 * maxres (device double) is non-NULL it receives max|r| over the colour. */
int ampe_efo_rbgs(const ampe_model_t* m, const double* dface0,
                  const double* dface1, const double* dface2, double d_const,
                  const double* ccell, double c_const, const double* mcell,
                  double m_const, const double* rhs, double* u, int offset,
                  double* maxres, void* stream);

/* One whole red-black sweep of EllipticFACOps::smoothErrorByRedBlack
 * (EllipticFACOps.cc:1067-1230: red cells, then black cells) in a single
 * launch, reading u_in and writing u_out (interior and periodic ghost
 * images); u_in NULL starts from u = 0.  The result equals two
 * ampe_efo_rbgs colour calls with a ghost fill between them.  Requires
 * even extents (AMPE_ERR_INVALID otherwise) and u_in != u_out.  3D levels of
 * at least 2^21 cells with the phase (cell C), composition (face D) or
 * quaternion (face D, cell M) operator shape take the z-marching sweep that
 * the stepper's multigrid runs. */
int ampe_efo_rbgs_sweep(const ampe_model_t* m, const double* dface0,
                        const double* dface1, const double* dface2,
                        double d_const, const double* ccell, double c_const,
                        const double* mcell, double m_const, const double* rhs,
                        const double* u_in, double* u_out, void* stream);

/* EFO_COMPRES* (3d/ellipticfacops.m4:448-575): res = f - A u. */
int ampe_efo_residual(const ampe_model_t* m, const double* dface0,
                      const double* dface1, const double* dface2,
                      double d_const, const double* ccell, double c_const,
                      const double* mcell, double m_const, const double* rhs,
                      const double* u, double* res, void* stream);

/* Residual res = f - A u (EFO_COMPRES*) and its RMS over the interior cells
 * (EllipticFACOps::computeResidualNorm, EllipticFACOps.cc:1760-1786, the
 * norm the FAC loop tests after every cycle, samrai/FACPreconditioner.cc:
 * 365-416).  `scratch` is caller-allocated device memory of
 * ampe_efo_residual_rms_scratch_doubles(m) doubles (the residual field and
 * the partial sums of a deterministic two-pass reduction); *rms is a device
 * double written asynchronously on `stream`. */
size_t ampe_efo_residual_rms_scratch_doubles(const ampe_model_t* m);
int ampe_efo_residual_rms(const ampe_model_t* m, const double* dface0,
                          const double* dface1, const double* dface2,
                          double d_const, const double* ccell, double c_const,
                          const double* mcell, double m_const,
                          const double* rhs, const double* u, double* scratch,
                          double* rms, void* stream);

/* Same result as ampe_efo_residual_rms, without any device allocation and
 * without a scratch argument.  No counterpart in the reference: it exists for
 * callers that cannot allocate device memory themselves -- a host framework
 * that owns all GPU memory through its own pool and gives this library a
 * fixed budget, or code that must not call cudaMalloc/cudaFree because those
 * calls synchronise the device (a latency-critical solver loop).  Its
 * working memory is one library-owned buffer of AMPE_NOALLOC_SCRATCH_DOUBLES
 * doubles (4 MiB) that every GPU which loads the library keeps until the
 * process exits; levels whose ghost box plus the reduction partials do not
 * fit (ghost box above ~523,000 cells, e.g. 80^3) are refused with
 * AMPE_ERR_TOO_LARGE before any launch.  The first call on a device looks up
 * the buffer's device address (cudaGetSymbolAddress), so make that first call
 * outside any CUDA stream capture.  That address is kept for the life of the
 * process: after cudaDeviceReset (or any other teardown of the device's
 * primary context) it is stale, so do not call this entry point on a device
 * that has been reset.  All calls share the one buffer: calls
 * whose work overlaps on the GPU (different streams, or different host
 * threads) race and give wrong norms -- serialise them.  No part of the
 * buffer has to start at zero: each call overwrites what it reads. */
#define AMPE_NOALLOC_SCRATCH_DOUBLES (1 << 19)
int ampe_efo_residual_rms_noalloc(const ampe_model_t* m, const double* dface0,
                                  const double* dface1, const double* dface2,
                                  double d_const, const double* ccell,
                                  double c_const, const double* mcell,
                                  double m_const, const double* rhs,
                                  const double* u, double* rms, void* stream);

/* ---------------------------------------------------------------------
 * Two-level composite FAC (AMR): a periodic coarse level and one fine box
 * refined by 2 in every direction, for  A u = M div(D grad u) - C u = f
 * (EllipticFACOps with FACPreconditioner's default recursive cycle,
 * samrai/FACPreconditioner.cc:267-464, EllipticFACOps.cc:948-1758 and
 * 1947-2029; ellipticfacops.m4 efo_compfluxvardc3d, efo_compresvarsca3d,
 * efo_rbgswithfluxmax*, efo_ewingfixfluxvardc3d):
 *   - fine ghost cells from the coarse level by constant refinement, the
 *     coarse-fine face fluxes by Ewing's correction (weights 2/3 and 1/3
 *     with the reference's single-precision 1/3);
 *   - coarse faces on the fine box's boundary take the mean of the four
 *     fine face fluxes, coarse cells under the box the mean of the fine
 *     solution / residual (volume-weighted averages);
 *   - a cycle: presweeps red-black sweeps on the fine level (flux form),
 *     the fine residual restricted into the coarse right-hand side,
 *     coarse_sweeps sweeps on the coarse level, the coarse error prolonged
 *     (constant) and added, postsweeps fine sweeps;
 *   - the norm: RMS of the composite residual weighted by cell volume,
 *     coarse cells under the box weight 0.
 * The reference computes face fluxes and the Ewing correction with the
 * level-0 spacing on every level (EllipticFACOps.cc:1253,1961: the grid
 * geometry's dx) and the divergence and smoother with the level's own
 * spacing; level_dx = 0 reproduces that, level_dx = 1 uses each level's own
 * spacing throughout (the consistent operator).
 * Arrays (device): coarse cells ghosted with coarse.ng, fine cells with
 * ng_fine, face coefficients ghost-free (D0, D1, D2 per level; NULL:
 * d_const); C and M cell arrays or NULL (c_const, m_const).  3D only. */
typedef struct ampe_fac2 {
   ampe_model_t coarse; /* dim 3, n, ng >= 1, dx */
   int lo[3];           /* fine box lower corner (coarse cells) */
   int nbox[3];         /* fine box size in coarse cells (>= 2 each) */
   int ng_fine;         /* ghost width of fine cell arrays (>= 1) */
   int level_dx;        /* 0: reference spacing rule, 1: per-level spacing */
   int presweeps, postsweeps, coarse_sweeps;
   double d_const, c_const, m_const;
} ampe_fac2_t;

typedef struct ampe_fac2_level {
   const double* D[3]; /* face coefficients (NULL: d_const) */
   const double* C;    /* cell (NULL: c_const) */
   const double* M;    /* cell (NULL: m_const) */
} ampe_fac2_level_t;

/* doubles of workspace ampe_fac2_solve and ampe_fac2_composite_residual
 * need */
long long ampe_fac2_work_doubles(const ampe_fac2_t* p);
/* composite residual r = f - A u on both levels (computeFullCompositeResidual,
 * FACPreconditioner.cc:661-683): also restricts u_f into the coarse cells
 * under the box.  norm (host, may be NULL): the weighted RMS. */
int ampe_fac2_composite_residual(const ampe_fac2_t* p, const ampe_fac2_level_t* coarse,
                                 const ampe_fac2_level_t* fine, const double* fc,
                                 const double* ff, double* uc, double* uf, double* rc,
                                 double* rf, double* work, double* norm, void* stream);
/* FAC iterations (solveSystem, FACPreconditioner.cc:267-420): at most
 * max_cycles, stopping once the norm is <= tol.  norms (host, max_cycles+1
 * entries): the norm before the first cycle and after each one.  Returns
 * the number of cycles taken (>= 0) or an AMPE_ERR_*. */
int ampe_fac2_solve(const ampe_fac2_t* p, const ampe_fac2_level_t* coarse,
                    const ampe_fac2_level_t* fine, const double* fc, const double* ff,
                    double* uc, double* uf, int max_cycles, double tol, double* work,
                    double* norms, void* stream);

/* ---------------------------------------------------------------------
 * Quaternion orientation kernels (evolve_quat models).  q is 4 ghosted
 * cell fields back to back (CellData depth 4), ghosts filled.
 * ------------------------------------------------------------------- */

/* |grad q| at cells from the normal differences on the cell's faces:
 * QUATDIFFS (3d/quatdiffs.m4:70-128) + QUATGRAD_MODULUS_FROM_SIDES_COMPACT
 * (3d/quatgrad.m4:725-790), the path of QuatModel::computeQuatGradients.
 * ogm: interior (ghost width 0). */
int ampe_quat_grad_modulus(const ampe_model_t* m, const double* q,
                           double* ogm, void* stream);
/* QUATMOBILITY (3d/mobility.m4:13-95, quat_mobility_type 'p'):
 * M_q = min + (M - min)(1 - p(phi)) on interior cells of mq (ghost width
 * m->ng). */
int ampe_quat_mobility(const ampe_model_t* m, const double* phi, double* mq,
                       void* stream);
/* COMPUTE_FACE_COEF3D (3d/quatfacops.m4:14-155) with the side gradients of
 * QUATGRAD_SIDE (3d/quatgrad.m4:213-335) and the floor types of
 * eval_grad_normi (quat.f:1497-1537): fc = -2H T p1(phibar) / |grad q|_f
 * - eps_q^2 p2(phibar) on every face (side arrays). */
int ampe_quat_face_coef(const ampe_model_t* m, const double* phi,
                        const double* temp, const double* q, double* fc0,
                        double* fc1, double* fc2, void* stream);
/* COMPUTE_FLUX3D + ADD_QUAT_OP3D (3d/quatfacops.m4:227-311, 596-657) as
 * used by QuatModel's RHS: out_c = -M_q div(fc grad q_c), c = 0..3,
 * interior output 4N (component-major). */
int ampe_quat_rhs(const ampe_model_t* m, const double* fc0, const double* fc1,
                  const double* fc2, const double* mq, const double* q,
                  double* out, void* stream);

/* Symmetry-aware orientation (cubic symmetry, 3D, qlen 4), the path of
 * QuatModel::computeSymmetryRotations and makeQuatFundamental
 * (QuatModel.cc:4978-5105) and of the symmetric differences and side
 * gradients.  Side arrays (int rotation indices, depth-4 differences and
 * gradients, component-major) have ghost width m->ng_side >= 1: the
 * rotations and differences cover the faces of the interior plus one
 * transverse ghost layer, as the reference's loops do.  Rotation indices
 * are 1-based into the 48 unit quaternions of quat.f setqr (quat.f:
 * 165-288), negative for the conjugate.  Products and norms are evaluated
 * without fused multiply-add, in the reference's order. */

/* The 48 rotations (qr: 48 x 4, w x y z) and each one's conjugate index
 * (1-based), as the kernels use them (host only). */
int ampe_quat_symm_table(double* qr, int* conj);
/* QUAT_SYMM_ROTATION (3d/quatrotation.m4:12-91) with quatfindsymm4
 * (quat.f:73-163): for every face, the rotation r minimising
 * |q_lo r / |q_lo r| - q_hi / |q_hi||^2, searched from the index already in
 * rot (0 or out of range: 1), ending at the first rotation within
 * (2 sin(pi/16))^2.  rot0..2 in/out. */
int ampe_quat_symm_rotation(const ampe_model_t* m, const double* q, int* rot0,
                            int* rot1, int* rot2, void* stream);
/* QUAT_FUNDAMENTAL (3d/quatrotation.m4:93-147): every interior q replaced
 * by its rotation closest to the identity (search from rotation 1). */
int ampe_quat_fundamental(const ampe_model_t* m, double* q, void* stream);
/* QUATDIFFS_SYMM (3d/quatdiffs.m4:131-219): diff = q_hi - q_lo r(rot) on the
 * faces of QUAT_SYMM_ROTATION.  An index out of range gives NaN. */
int ampe_quat_diffs_symm(const ampe_model_t* m, const double* q, const int* rot0,
                         const int* rot1, const int* rot2, double* diff0,
                         double* diff1, double* diff2, void* stream);
/* QUATGRAD_SIDE_SYMM (3d/quatgrad.m4:376-679) on interior faces:
 * grad_<c>_<d>side, component c of grad q on the faces of normal d. */
int ampe_quat_grad_side_symm(const ampe_model_t* m, const double* diff0,
                             const double* diff1, const double* diff2,
                             const int* rot0, const int* rot1, const int* rot2,
                             double* grad_x_xside, double* grad_y_xside,
                             double* grad_z_xside, double* grad_x_yside,
                             double* grad_y_yside, double* grad_z_yside,
                             double* grad_x_zside, double* grad_y_zside,
                             double* grad_z_zside, void* stream);

/* PhaseFACOps::setCOnPatchPrivate (PhaseFACOps.cc:101-183):
 * C = 1 + gamma M_phi w g''(phi) on interior cells (ghost width m->ng). */
int ampe_phase_fac_set_c(const ampe_model_t* m, const double* phi,
                         double gamma, double* ccell, void* stream);

/* ---------------------------------------------------------------------
 * Surrogate MLP for the KKS initial guess: (phi, c, T) -> (cL, cS),
 * 3 -> 64 -> 64 -> 64 -> 2, SiLU, BF16 weights, FP32 accumulation.  No
 * counterpart in the reference (its Newton starts from the previous step's
 * cL, cS, QuatModel.cc:5218-5231).  Trained on samples labelled by the FP64
 * KKS Newton of the model given at create; inference on the tensor cores.
 * ------------------------------------------------------------------- */
int ampe_mlp_create(const ampe_model_t* m, int batch, unsigned seed,
                    void** handle);
int ampe_mlp_destroy(void* handle);
int ampe_mlp_nparams(void* handle);
/* n samples phi~U[0,1], c~U[c_lo,c_hi], T~U[t_lo,t_hi], labelled by the
 * FP64 Newton from (c, c); sets the T normalisation to [t_lo, t_hi]. */
int ampe_mlp_generate(void* handle, long long n, unsigned seed, double t_lo,
                      double t_hi, double c_lo, double c_hi,
                      long long* newton_failures);
/* Adam on minibatches of the generated samples (loss: 1/2 mean squared
 * error of the two logits): each step is one tcgen05 forward + backward
 * launch (one CTA per 128 samples) and one reduction + FP32 Adam launch;
 * repacks the BF16 tensor-core operands. */
int ampe_mlp_train(void* handle, int steps, int batch, float lr,
                   float* final_loss);
/* gradient of the loss on one batch (x: [batch][4] encoded inputs, target:
 * [batch][2] logits; device pointers) into the handle's gradient buffer,
 * formed as the training steps form it: the tensor-core forward and
 * backward products (BF16 operands, FP32 accumulation; the weight
 * gradients of the 128-sample tiles summed in a fixed order). */
int ampe_mlp_grad(void* handle, const float* x, const float* target,
                  int batch, float* loss);
int ampe_mlp_get(void* handle, float* params, float* grads, int host);
int ampe_mlp_set(void* handle, const float* params, int host);
int ampe_mlp_set_normalization(void* handle, double t_lo, double t_hi);
/* guesses for the interior cells of `grid` (phi, conc ghosted FP64);
 * tensor_cores=1: tcgen05 kernel, 0: CUDA-core reference kernel. */
int ampe_mlp_infer(void* handle, const ampe_model_t* grid, const double* phi,
                   const double* conc, const double* temp, float* guess_l,
                   float* guess_s, int tensor_cores, void* stream);
/* AMPE_OK, or AMPE_ERR_NOT_CONVERGED if a tensor-core wait timed out. */
int ampe_mlp_status(void* handle);
int ampe_mlp_clear_status(void* handle);
/* Bound (polls, >= 1; default 2^22) of the tensor-core kernels' mbarrier
 * waits.  skip_issue != 0 is a test of the timeout path: the issuing thread
 * commits no MMA, so each kernel's first wait runs out with nothing in
 * flight, sets the status and frees its tensor memory. */
int ampe_mlp_set_wait_limit(void* handle, int wait_limit, int skip_issue);

/* ---------------------------------------------------------------------
 * Implicit stepper (CVODEAbstractFunctions + CVODESolver role,
 * samrai/CVODEAbstractFunctions.h:61-90, QuatIntegrator.cc:2096-3906).
 * Allocates all its device workspace here, never in ampe_stepper_advance.
 * ------------------------------------------------------------------- */
int ampe_stepper_create(const ampe_model_t* m, const ampe_step_params_t* p,
                        void** handle);
int ampe_stepper_destroy(void* handle);
/* Copy the state in.  host!=0: pointers are host memory.  phi, conc and
 * (CALPHAD) cl, cs warm starts are interior arrays n0*n1*n2 (no ghosts);
 * temp may be NULL unless temp_mode==AMPE_TEMP_FIELD. */
int ampe_stepper_set_state(void* handle, const double* phi,
                           const double* conc, const double* cl,
                           const double* cs, const double* temp, int host);
int ampe_stepper_get_state(void* handle, double* phi, double* conc,
                           double* cl, double* cs, int host);
/* Advance nsteps accepted steps: of size p->dt, or (p->adaptive) of the
 * sizes the error control chooses. */
int ampe_stepper_advance(void* handle, int nsteps, ampe_step_stats_t* stats);
/* p->adaptive: accepted steps until t reaches t_stop (the last step ends at
 * t_stop exactly) or max_steps steps were taken; max_steps = 1 is CVODE's
 * CV_ONE_STEP mode with a stop time, as QuatModel drives it (one internal
 * step per QuatIntegrator::Advance, QuatIntegrator.cc:2096-2104).  A
 * t_stop the stepper has reached takes no step; one before the current t
 * sets no stop time.  The history (step sizes, order, back values) carries
 * over between calls. */
int ampe_stepper_advance_to(void* handle, double t_stop, int max_steps,
                            ampe_step_stats_t* stats);
/* Temperature of the following steps (TemperatureStrategy role: a scalar
 * T0 with an optional x gradient, set from the host between steps); the
 * per-x thermodynamic tables are rebuilt, the BDF history is kept.  Models
 * with temp_mode AMPE_TEMP_FIELD take their field via set_state; models
 * with dTdt != 0 follow their T0(t) and refuse this call. */
int ampe_stepper_set_temperature(void* handle, double T0, double gradT);
/* Evaluate f(y) of the current state (fd_flag=0 path): outputs interior. */
int ampe_stepper_eval_rhs(void* handle, double* phi_rhs, double* conc_rhs,
                          int host);
/* out = v - gamma J v at the current state (J the Jacobian of f): the
 * finite-difference product of CVODE (QuatIntegrator::
 * evaluateJTimesRHSFunction role) on the FP64 path, the analytic FP32
 * linearisation on the mixed path.  v, out: [phi | conc] interior. */
int ampe_stepper_jv(void* handle, const double* v, double gamma, double* out,
                    int host);
/* Replace the current state y_n (phi, conc interior arrays) keeping the BDF
 * history and the Newton warm starts: for callers that own the fields in
 * host memory and hand them in every step (a SAMRAI patch adapter).
 * host != 0 here and in ampe_stepper_get_state: pinned host buffers that
 * the device can address (cudaHostAlloc / cudaHostRegister under unified
 * addressing) are copied by a kernel over the host link, other host memory
 * by cudaMemcpyAsync; both on the stepper's stream. */
int ampe_stepper_load_y(void* handle, const double* phi, const double* conc,
                        int host);
/* evolve_quat models: the orientation part of y_n, 4N doubles (component-
 * major interior arrays, unit quaternions).  set_state initialises it to
 * (1, 0, 0, 0); set_quat replaces it and restarts the BDF history.
 * Accepted steps are projected onto unit quaternions
 * (QuatIntegrator::applyProjection, QuatIntegrator.cc:3911-3940). */
int ampe_stepper_set_quat(void* handle, const double* q, int host);
/* Anisotropic flux models without evolve_quat: the static orientation field
 * read by the phase flux (PhaseFluxStrategyAnisotropy, quat_id of
 * PhaseFluxStrategy::computeFluxes, PhaseFluxStrategy.h:25-27), qlen
 * component-major interior arrays; 2D qlen 2 gives phi_o = acos q0.
 * Default after create: q = (1, 0, ...), angle 0. */
int ampe_stepper_set_orientation(void* handle, const double* q, int host);
int ampe_stepper_get_quat(void* handle, double* q, int host);
/* Length of the stepper's state vector y: 2N, or 6N with quaternions. */
long long ampe_stepper_size(void* handle);
/* f(y_n) for the whole state vector (ampe_stepper_size doubles). */
int ampe_stepper_eval_rhs_full(void* handle, double* out, int host);
/* Use a trained surrogate (ampe_mlp_*) for the KKS initial guesses of the
 * mixed path (params surrogate=1) while no converged phase concentrations
 * exist (after ampe_stepper_set_state without cl / cs, until the first
 * accepted step): each cell starts from the network's guess and falls back
 * to the stored values when 3 FP32 Newton iterations do not converge.
 * Afterwards the previous step's values are the starting point.  The handle
 * must outlive the stepper. */
int ampe_stepper_attach_surrogate(void* handle, void* mlp);
/* Launches of library kernels in this process (launch accounting). */
long long ampe_stepper_kernel_launches(void* handle);
/* Run the stepper's work on the caller's stream (cudaStream_t; NULL: back to
 * the stepper's private stream) from the next call on: every launch and copy
 * of the following calls is ordered on it, after the caller's earlier work
 * there (CVODE's callbacks run in the caller's order, samrai/
 * CVODEAbstractFunctions.h:61-90).  The stepper still waits on that stream
 * where the Newton / GMRES control reads a reduced value, and it waits for
 * its previous stream before switching.  The stream must outlive its use. */
int ampe_stepper_set_stream(void* handle, void* stream);
/* The stepper's CUDA stream (cudaStream_t), for events around advance. */
void* ampe_stepper_stream(void* handle);
/* Per-kernel CUDA-event timing on the stepper stream.  kind: 0 KKS Newton,
 * 1 fused RHS, 2 analytic Jacobian-vector product (mixed path), 3 surrogate
 * inference, 4 quaternion RHS (mobility, face coefficients, divergence),
 * 5 preconditioner solves (all blocks, FAC cycles included), 6
 * preconditioner setups, 7 red-black sweeps on the finest multigrid level
 * (one interval per pre- or post-smoothing, two colour launches per sweep).
 * Enabling resets the totals. */
int ampe_stepper_profile(void* handle, int enable);
int ampe_stepper_kernel_time(void* handle, int kind, double* total_ms,
                             long long* launches);

/* Library identification. */
const char* ampe_version(void);
int ampe_device_count(void);

#ifdef __cplusplus
}
#endif
#endif
