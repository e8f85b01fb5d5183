/* C-ABI of the CPU oracle (liborc_ampe.so).  TEST INFRASTRUCTURE ONLY:
 * loaded by tests/, __graft_entry__.smoke() and bench.py's CPU-baseline
 * leg as the checker of libampe_gb300; never part of the product path.
 * Arrays are host arrays in the layouts of include/ampe_gb300.h. */
#ifndef AMPE_ORACLE_API_H
#define AMPE_ORACLE_API_H

#include "ampe_gb300.h"

#ifdef __cplusplus
extern "C" {
#endif

/* scalar functions (functions.f) */
double orc_interp_func(double phi, char type);
double orc_deriv_interp_func(double phi, char type);
double orc_second_deriv_interp_func(double phi, char type);
double orc_well_func(double phi, char type);
double orc_deriv_well_func(double phi, char type);
double orc_second_deriv_well_func(double phi, char type);
double orc_average_func(double a, double b, char type);

/* thermodynamics at one temperature (J/mol) */
double orc_free_energy(const ampe_model_t* m, double T, double c, int phase);
double orc_dfdc(const ampe_model_t* m, double T, double c, int phase);
double orc_d2fdc2(const ampe_model_t* m, double T, double c, int phase);
double orc_gterm(const ampe_gterm_t* g, double T);
int orc_kks_cell(const ampe_model_t* m, double T, double h, double c,
                 double* x);
int orc_ceq(const ampe_model_t* m, double T, double* x);

/* stencils */
void orc_fill_ghosts(const ampe_model_t* m, double* f);
void orc_phase_flux(const ampe_model_t* m, const double* ph,
                    const double* quat, double* f0, double* f1, double* f2);
void orc_computerhspbg(const ampe_model_t* m, const double* f0,
                       const double* f1, const double* f2, const double* temp,
                       const double* phi, const double* ogm, double* rhs);
void orc_add_driving_force(const ampe_model_t* m, const double* temp,
                           const double* phi, const double* cl,
                           const double* cs, double* rhs);
long orc_phase_concentrations(const ampe_model_t* m, const double* temp,
                              const double* phi, const double* conc,
                              const double* clr, const double* csr,
                              double* cl, double* cs, long* nfail);
void orc_conc_diffusion(const ampe_model_t* m, const double* phi,
                        const double* temp, double* dl0, double* dl1,
                        double* dl2, double* ds0, double* ds1, double* ds2);
void orc_conc_flux_kks(const ampe_model_t* m, const double* phid, const double* cld,
                       const double* csd, const double* temp, const double* phi,
                       const double* conc, double* f0, double* f1, double* f2);
void orc_add_flux(const ampe_model_t* m, const double* u, const double* d0,
                  const double* d1, const double* d2, double* f0, double* f1,
                  double* f2);
void orc_computerhsconcentration(const ampe_model_t* m, const double* f0,
                                 const double* f1, const double* f2,
                                 double* rhs);
void orc_rhs_phase_conc(const ampe_model_t* m, const double* phi,
                        const double* quat, const double* temp,
                        const double* cl, const double* cs,
                        const double* phi_d, double* phi_rhs,
                        double* conc_rhs);

void orc_rhs_phase_conc_q(const ampe_model_t* m, const double* phi,
                          const double* quat, const double* temp,
                          const double* cl, const double* cs,
                          const double* phi_d, const double* ogm,
                          double* phi_rhs, double* conc_rhs);
/* as orc_rhs_phase_conc_q with the face diffusivities at (phi_d, cl_d, cs_d)
 * (the lagged fields of finite-difference Jacobian evaluations) */
void orc_rhs_phase_conc_qd(const ampe_model_t* m, const double* phi,
                           const double* quat, const double* temp,
                           const double* cl, const double* cs,
                           const double* phi_d, const double* cl_d,
                           const double* cs_d, const double* ogm,
                           double* phi_rhs, double* conc_rhs);
/* the face diffusivities of the model's conc_diffusion: Arrhenius
 * (orc_conc_diffusion) or the atomic mobilities at the face means of
 * cl_d, cs_d (orc_conc_diffusion_mobility) */
void orc_conc_diffusion_model(const ampe_model_t* m, const double* phi,
                              const double* temp, const double* cl_d,
                              const double* cs_d, double* dl0, double* dl1,
                              double* dl2, double* ds0, double* ds1, double* ds2);
/* quaternion kernels (quat.cc) */
void orc_quat_grad_modulus(const ampe_model_t* m, const double* q, double* ogm);
void orc_quat_mobility(const ampe_model_t* m, const double* phi, double* mq);
void orc_quat_face_coef(const ampe_model_t* m, const double* phi,
                        const double* temp, const double* qlag, double* fc0,
                        double* fc1, double* fc2);
void orc_quat_rhs(const ampe_model_t* m, const double* fc0, const double* fc1,
                  const double* fc2, const double* mq, const double* q,
                  double* out);
void orc_quat_project(long ncells, double* q);

void orc_jv_analytic(const ampe_model_t* m, const double* phi,
                     const double* cl, const double* cs, const double* v,
                     double gamma, double* out);

/* FAC operator */
double orc_efo_rbgs(const ampe_model_t* m, const double* d0, const double* d1,
                    const double* d2, double dc, const double* ccell,
                    double cc, const double* mcell, double mc,
                    const double* f, double* u, int offset);
void orc_efo_residual(const ampe_model_t* m, const double* d0,
                      const double* d1, const double* d2, double dc,
                      const double* ccell, double cc, const double* mcell,
                      double mc, const double* f, const double* u,
                      double* res);
void orc_phase_fac_set_c(const ampe_model_t* m, const double* phi,
                         double gamma, double* ccell);
double orc_rms_interior(const ampe_model_t* m, const double* v);
void* orc_fac_create(const ampe_model_t* m, int nlevels);
void orc_fac_destroy(void* h);
void orc_fac_set_operator(void* h, const double* d0, const double* d1,
                          const double* d2, double dc, const double* ccell,
                          double cc, const double* mcell, double mc);
int orc_fac_solve(void* h, const ampe_step_params_t* p, int mode,
                  const double* f, double* u, double tol, double* res);

void orc_add_flux_from_grad_t(const ampe_model_t* m, const double* T, const double* q0,
                              const double* q1, const double* q2, double* f0, double* f1,
                              double* f2);
void orc_add_flux_from_antitrapping(const ampe_model_t* m, const double* phase,
                                    const double* cl, const double* ca, const double* dphidt,
                                    double alpha, double* f0, double* f1, double* f2);
void orc_kim_mobility(const ampe_model_t* m, const double* tfield, const double* cl,
                      const double* cs, double factor, double D0, double Q0, double mv,
                      double* mob);
double orc_phase_diffusion_mobility(const ampe_model_t* m, const ampe_mobility_t* mb, int p,
                                    double c, double T);
void orc_conc_diffusion_mobility(const ampe_model_t* m, const ampe_mobility_t* mb,
                                 const double* phi, const double* temp, const double* cl,
                                 const double* cs, double* dl0, double* dl1, double* dl2,
                                 double* ds0, double* ds1, double* ds2, double* el0,
                                 double* el1, double* el2, double* es0, double* es1,
                                 double* es2);
/* symmetry-aware orientation (cubic, qlen 4; side arrays of ghost width m->ng_side) */
void orc_quat_symm_table(double* qr, int* conj);
int orc_quat_find_symm(const double* q1, const double* q2, int iq, double* q2p);
void orc_quat_symm_rotation(const ampe_model_t* m, const double* q, int* rot0, int* rot1,
                            int* rot2);
void orc_quat_fundamental(const ampe_model_t* m, double* q);
void orc_quat_diffs_symm(const ampe_model_t* m, const double* q, const int* rot0,
                         const int* rot1, const int* rot2, double* diff0, double* diff1,
                         double* diff2);
void orc_quat_grad_side_symm(const ampe_model_t* m, const double* diff0, const double* diff1,
                             const double* diff2, const int* rot0, const int* rot1,
                             const int* rot2, double* gxx, double* gyx, double* gzx,
                             double* gxy, double* gyy, double* gzy, double* gxz, double* gyz,
                             double* gzz);
/* two-level composite FAC */
long long orc_fac2_work_doubles(const ampe_fac2_t* p);
double orc_fac2_composite_residual(const ampe_fac2_t* p, const ampe_fac2_level_t* lc,
                                   const ampe_fac2_level_t* lf, const double* fc,
                                   const double* ff, double* uc, double* uf, double* rc,
                                   double* rf);
int orc_fac2_solve(const ampe_fac2_t* p, const ampe_fac2_level_t* lc,
                   const ampe_fac2_level_t* lf, const double* fc, const double* ff,
                   double* uc, double* uf, int max_cycles, double tol, double* norms);
/* implicit stepper */
void* orc_stepper_create(const ampe_model_t* m, const ampe_step_params_t* p);
void orc_stepper_destroy(void* h);
void orc_stepper_set_state(void* h, const double* phi, const double* conc,
                           const double* cl, const double* cs,
                           const double* temp);
/* q: 4 interior component arrays back to back (evolve_quat models) */
void orc_stepper_set_quat(void* h, const double* q);
void orc_stepper_get_quat(void* h, double* q);
void orc_stepper_get_state(void* h, double* phi, double* conc, double* cl,
                           double* cs);
void orc_stepper_eval_rhs(void* h, double* phi_rhs, double* conc_rhs);
void orc_stepper_eval_rhs_full(void* h, double* out);
void orc_stepper_set_orientation(void* h, const double* q);
long orc_stepper_size(void* h);
int orc_stepper_advance(void* h, int nsteps, ampe_step_stats_t* stats);
int orc_stepper_advance_to(void* h, double t_stop, int max_steps, ampe_step_stats_t* stats);
void orc_stepper_set_temperature(void* h, double T0, double gradT);
void orc_stepper_jv(void* h, const double* v, double gamma, double* out,
                    int analytic);

#ifdef __cplusplus
}
#endif
#endif
