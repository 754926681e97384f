/*
 * salsa_ref.h -- CPU oracle of the SALSA microphysics step.
 *
 * TEST INFRASTRUCTURE ONLY.  This is a plain-C FP64 restatement of the
 * reference Fortran path run_SALSA -> salsa (UCLALES-SALSA
 * src/src_salsa/mo_salsa_driver.f90:112-435, mo_salsa.f90:45-153 and the
 * process modules), used by the tests as the parity checker and by bench.py as
 * the timed CPU baseline.  The product library never links or calls it.
 *
 * Parity status: the reference is Fortran and no Fortran compiler exists in
 * this environment, and the reference ships no tests, golden vectors or
 * fixtures for this path.  The restatement is therefore "parity unpinned"
 * against the real Fortran; it is checked instead by second, independent numpy
 * restatements of the Fortran in tests/ (every process of the step, composed
 * into whole steps of the workload configurations, the secondary-ice schemes,
 * sedimentation and the post-step diagnostics), by closed-form checks
 * (flux-matching limits, semi-implicit single-pair update, Koehler equilibrium,
 * water conservation by construction) and by committed golden vectors of its
 * own outputs (tests/golden/).
 *
 * Interface: same structs as the product C-ABI (include/salsa_gb300.h).
 */
#ifndef SALSA_REF_H
#define SALSA_REF_H
#include "../include/salsa_gb300.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct salsa_ref_ctx salsa_ref_ctx_t;

int salsa_ref_create(const salsa_config_t *cfg, salsa_ref_ctx_t **out);

/* Test infrastructure: move every exp/log/log10/pow/erf/cos result of the following runs
 * by two ulps, up (1), down (-1) or in a direction from the argument's bits (2 and above,
 * one pattern per mode); 0 turns it off.  The parity tests take the oracle's response as part of their envelope. */
void salsa_ref_set_libm_perturbation(int mode);
void salsa_ref_destroy(salsa_ref_ctx_t *ctx);

/* Same argument meaning as salsa_gb300_run; host pointers only.
 * nthreads <= 0: use all OpenMP threads.  carry_over != 0 reproduces the
 * reference's serial module-state carry-over between cells (allSALSA keeps the
 * previous cell's derived diameters); 0 resets them per cell (the GPU
 * semantics, every cell sees the post-initialisation module state). */
/* tend_constrain2 and SALSA_diagnostics (src/src_LES/constrain_SALSA.f90), same
 * arguments as salsa_gb300_tend_constrain / salsa_gb300_diagnostics; host pointers. */
int salsa_ref_tend_constrain(salsa_ref_ctx_t *ctx, int nzp, int nxp, int nyp, double dtlt,
                             const salsa_post_fields_t *f);
int salsa_ref_diagnostics(salsa_ref_ctx_t *ctx, int nzp, int nxp, int nyp, int only_diag, int lcharge,
                          const salsa_post_fields_t *f);

/* sedim_SALSA (src/src_LES/mcrp.f90:745-1275); arguments as salsa_gb300_sedimentation. */
int salsa_ref_sedimentation(salsa_ref_ctx_t *ctx, int nzp, int nxp, int nyp, double dtlt, const int sed[4],
                            const salsa_sedim_fields_t *f);

int salsa_ref_run(salsa_ref_ctx_t *ctx, int nzp, int nxp, int nyp, int ns,
                  double tstep, double time, int istp, int level, int lcharge,
                  int initialize, const salsa_fields_t *f, salsa_status_t *st,
                  int nthreads, int carry_over);

int salsa_ref_layout(const salsa_ref_ctx_t *ctx, int *nbins, int *ncld, int *nprc,
                     int *nice, int *nwet, double *lolim_diam);

/* Work-unit counters accumulated over the last run: [0] coagc evaluations,
 * [1] acth2o calls, [2] J_imm evaluations, [3] equilibration iterations,
 * [4] condensation substeps. */
void salsa_ref_counters(const salsa_ref_ctx_t *ctx, long long out[5]);

/* Process states after the last run (set_SALSA_runtime): lscoag, lscnd, lsauto,
 * lsactiv, lsicenucl, lsicemelt, lssecice, the three secondary-ice schemes,
 * lsfreeRH, lsFreeTheta. */
void salsa_ref_states(const salsa_ref_ctx_t *ctx, int out[12]);

/* Single-function probes used by the closed-form tests. */
double salsa_ref_terminal_vel(double diam, double rhop, double rhoa, double visc,
                              double beta, int flag);
double salsa_ref_coagc_pair(const salsa_ref_ctx_t *ctx, int b1, int b2,
                            double numc1, double dwet1, double numc2,
                            double dwet2, double temp, double pres);
double salsa_ref_coagc_sections(const salsa_ref_ctx_t *ctx, int b1, double numc1,
                                const double *volc1, int b2, double numc2,
                                const double *volc2, double temp, double pres);
void salsa_ref_ice_shape(const salsa_ref_ctx_t *ctx, double mpri, double mrim, double numc,
                         double out[5]);
double salsa_ref_nucleation_rate(const salsa_ref_ctx_t *ctx, int kind, double theta,
                                 double Tk, double Din, double S);
double salsa_ref_freezing_fraction(const salsa_ref_ctx_t *ctx, int mode, double Tk, double S,
                                   double th00, double thm, double ths, double dins,
                                   double tstep);
double salsa_ref_sweq(const salsa_ref_ctx_t *ctx, int b, double numc, const double *volc,
                      double T);

#ifdef __cplusplus
}
#endif
#endif
