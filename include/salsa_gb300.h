/*
 * salsa_gb300.h -- C-ABI of the GB300 SALSA microphysics step.
 *
 * This library replaces the body of UCLALES-SALSA's per-grid-cell microphysics
 * driver, src/src_salsa/mo_salsa_driver.f90:112-435 (SUBROUTINE run_SALSA), and
 * everything it calls below it (mo_salsa.f90:45-153 SUBROUTINE salsa and the
 * process modules).  The arrays keep run_SALSA's layout: every field is a
 * column-major (Fortran order) array with z fastest,
 *     index(kk, ii, jj, b) = kk + nzp*(ii + nxp*(jj + nyp*b))      (0-based)
 * and a per-species mass array of a category with nb bins stores bin b of
 * species s at last index s*nb + b  (util.f90:955-961 getMassIndex, 0-based).
 * Only interior cells are touched: kk = 1..nzp-2, ii = 2..nxp-3, jj = 2..nyp-3
 * (0-based; mo_salsa_driver.f90:180-182 loops jj=3..nyp-2, ii=3..nxp-2,
 * kk=nzp-1..2 in 1-based indexing).
 *
 * Units at the boundary are those of the LES: numbers #/kg, masses kg/kg,
 * pressure Pa, temperature K, mixing ratios kg/kg, air density kg/m3.
 *
 * Every pointer in salsa_fields_t may point to host memory or to device memory
 * of the handle's GPU (all pointers of one call must be on the same side).  For
 * host pointers the library copies the fields to the GPU and the results back
 * inside the call.  The call is synchronous.
 *
 * Threading: a handle is not reentrant; distinct handles are independent (no
 * global mutable state).  The reference module state (allSALSA, zcc**, rateDiag)
 * lives per cell on the GPU.
 */
#ifndef SALSA_GB300_H
#define SALSA_GB300_H

#ifdef __cplusplus
extern "C" {
#endif

/* Limits of the bin layout supported by one handle. */
#define SALSA_MAXSPEC 7      /* dry species (classSpecies.f90 maxspec) */
#define SALSA_MAXNSP 9       /* dry + H2O + rime */
#define SALSA_MAXBINS 96     /* ntotal = nbins + ncld + nprc + nice */

/* Diagnostic process-rate fields, in the order of mo_salsa_driver.f90:392-411. */
enum {
  SALSA_DIAG_AUTOC = 0,    /* s_m_autoc      */
  SALSA_DIAG_AUTOC80,      /* s_m_autoc80    */
  SALSA_DIAG_AUTOC50,      /* s_m_autoc50    */
  SALSA_DIAG_ACCR,         /* s_m_accr       */
  SALSA_DIAG_ACCR80,       /* s_m_accr80     */
  SALSA_DIAG_ACCR50,       /* s_m_accr50     */
  SALSA_DIAG_ACCOLL,       /* s_m_ACcoll_dry */
  SALSA_DIAG_APCOLL,       /* s_m_APcoll_dry */
  SALSA_DIAG_ACTIV,        /* s_n_activ      */
  SALSA_DIAG_CONDA,        /* s_m_conda      */
  SALSA_DIAG_CONDC,        /* s_m_condc      */
  SALSA_DIAG_CONDP,        /* s_m_condp      */
  SALSA_DIAG_AICOLL,       /* s_m_AIcoll_dry (level 5) */
  SALSA_DIAG_ICEHOM,       /* s_n_icehom     (level 5) */
  SALSA_DIAG_ICEDEP,       /* s_n_icedep     (level 5) */
  SALSA_DIAG_ICEIMM,       /* s_n_iceimm     (level 5) */
  SALSA_DIAG_CONDI,        /* s_m_condi      (level 5) */
  SALSA_DIAG_SIPDRFR,      /* s_n_sipdrfr    (level 5, lssecice; :412-416) */
  SALSA_DIAG_SIPRMSPL,     /* s_n_siprmspl   (level 5, lssecice) */
  SALSA_DIAG_SIPIIBR,      /* s_n_sipiibr    (level 5, lssecice) */
  SALSA_NDIAG
};

/* ProcessSwitch (classProcessSwitch.f90:5-14): state is derived per call. */
typedef struct {
  int sw;          /* %switch */
  double delay;    /* %delay [s] */
  int mode;        /* %mode */
} salsa_switch_t;

/* POD mirror of the &salsa NAMELIST (mo_salsa_init.f90:522-600) plus the
 * arguments of define_salsa(level) and salsa_initialize(chargeTmax,
 * chargeCollEnh) (mo_salsa_init.f90:465, 792).  Defaults: salsa_gb300_default_config. */
typedef struct {
  int level;                                  /* thermodynamic level, 4 or 5 */
  salsa_switch_t lscoag, lscnd, lsauto, lsactiv, lsicenucl, lsicemelt, lssecice;
  int lscgaa, lscgcc, lscgca, lscgpc, lscgpa, lscgpp, lscgia, lscgic, lscgii, lscgip;
  double Eiagg_max, Eiagg_min;
  double cgintvl;
  int lscndgas, lscndh2oae, lscndh2ocl, lscndh2oic;
  int lsicehom, lsiceimm, lsicedep;
  int ice_theta_dist;
  salsa_switch_t lsFreeTheta;
  double initMinTheta;
  double mean_theta_imm, sigma_theta_imm, mean_theta_dep, sigma_theta_dep;
  double iceShapeAlpha, iceShapeBeta, iceShapeGamma, iceShapeSigma;
  int lsdistupdate;
  int lscheckarrays;
  double fixinc;
  salsa_switch_t lsfreeRH;
  double rhlim;
  double eddy_dis;
  int nsnucl, nj3;
  double act_coeff;
  /* bin layout: aerosol regimes (mo_submctl.f90:208-212), precip and ice BinLayout */
  int nbin[2];
  double reglim[4];
  int prc_nbins;  double prc_dlo, prc_vol_ratio;
  int ice_nbins;  double ice_dlo, ice_vol_ratio;
  /* species: nspec_dry names out of SO4 OC BC DU SS NO NH, in mass-array order */
  int nspec_dry;
  char listspec[SALSA_MAXSPEC][4];
  /* salsa_initialize arguments */
  double chargeTMax, chargeCollEnh;
  /* secondary-ice subprocess switches (lssub, mo_salsa_init.f90:493-494, 675-677) */
  salsa_switch_t lssiprimespln, lssipdropfrac, lssipicecollbreak;
  /* ---- GB300 extensions (no counterpart in the reference) ---- */
  int precision;     /* 0: FP64 (parity form); 1: FP32-mixed form */
  int diagnostics;   /* 1: accumulate process-rate diagnostics; 0: skip them */
} salsa_config_t;

/* Array arguments of run_SALSA (mo_salsa_driver.f90:112-133) after the Diag/Prog
 * getData lookups (:481-561).  "t" suffix = tendency (time level 2), in/out:
 * the library ADDS (new-old)/tstep to it.  NULL is allowed for arrays that the
 * configuration does not use (rsi/nice/mice/micet/indef at level 4, chargeTime
 * without lcharge, gaero/gaerot without lscndgas, wp without cloud-base activation,
 * any diag entry).  With lscndgas, gaero holds the five gases in #/kg (SO4, HNO3,
 * NH3, non-volatile OC, semi-volatile OC; mo_salsa_driver.f90:285-290) and gaerot
 * receives their tendencies. */
typedef struct {
  const double *press, *temp, *rsl, *rsi, *dn;    /* (nzp,nxp,nyp) */
  const double *rp;  double *rpt;                 /* water vapour mixing ratio and its tendency */
  const double *wp;                               /* vertical velocity */
  const double *naero, *ncloud, *nprecp, *nice;   /* (...,nbins|ncld|nprc|nice) #/kg */
  double *naerot, *ncloudt, *nprecpt, *nicet;
  const double *maero, *mcloud, *mprecp, *mice;   /* (...,nwet*nb | (nwet+1)*nice) kg/kg */
  double *maerot, *mcloudt, *mprecpt, *micet;
  double *indef;        /* (...,nliquid) in/out: IN nucleated fraction (level 5, ice_theta_dist) */
  double *chargeTime;   /* (...,nliquid) in/out: charging time tracer (lcharge) */
  const double *gaero;  double *gaerot;           /* (...,5) gases #/kg */
  double *pa_nactd;     /* (...,ncld) out */
  double *pa_vactd;     /* (...,ns*ncld) out */
  double *diag[SALSA_NDIAG];                      /* (nzp,nxp,nyp) out */
  /* GB300 extension: per-cell hygroscopicity override (NULL = species tables) */
  const double *kappa;
  /* secondary-ice tracers (level 5 with lssecice, required then): crystals produced by
   * drop fracturing, rime splintering and ice-ice breakup, per ice bin, #/kg, updated
   * in place (Prog sipdrfr, siprmspl, sipiibr; mo_salsa_driver.f90:259-261, 346-348) */
  double *sipdrfr, *siprmspl, *sipiibr;           /* (...,nice) */
} salsa_fields_t;

/* Per-call status.  The reference STOPs or prints in these situations; the
 * library records them per cell, finishes the step and returns nonzero. */
typedef struct {
  int code;                       /* 0 ok, else SALSA_E_* */
  long long n_cells;              /* interior cells processed */
  long long n_equil_nonconv;      /* equilibration > 100 iterations (mo_salsa_properties.f90:242,356) */
  long long n_distr_nonconv;      /* distr_update > 100 passes (mo_salsa_update.f90:138,231,329,424) */
  long long n_distr_negfrac;      /* zvfrac < 0 (mo_salsa_update.f90:111,204,302,397) */
  long long n_cond_substeps;      /* > 100 condensation substeps (mo_salsa_dynamics.f90:1051) */
  long long n_negative;           /* numc < -1e-6 after coagulation (mo_salsa_dynamics.f90:192) */
  long long n_nonfinite;          /* NaN/Inf in the new state */
} salsa_status_t;

enum {
  SALSA_OK = 0,
  SALSA_E_ARG = 1,          /* NULL pointer / bad dimension / bad config value */
  SALSA_E_UNSUPPORTED = 2,  /* configuration outside what this build implements */
  SALSA_E_CUDA = 3,         /* CUDA runtime error */
  SALSA_E_NUMERIC = 4,      /* a per-cell condition above occurred */
  SALSA_E_NODEV = 5         /* no usable GPU */
};

typedef struct salsa_handle salsa_handle_t;

/* Fill *cfg with the reference defaults (mo_submctl.f90, mo_ice_shape.f90,
 * classProcessSwitch.f90, mo_salsa_init.f90:687-695). */
void salsa_gb300_default_config(salsa_config_t *cfg);

/* Replaces define_salsa(level) + salsa_initialize(chargeTmax, chargeCollEnh)
 * (mo_salsa_init.f90:465-637, 792-858): builds species and bin tables on the
 * host and uploads them to the current CUDA device. */
int salsa_gb300_init(const salsa_config_t *cfg, salsa_handle_t **out);

/* Replaces run_SALSA(Diag, Prog, nzp, nxp, nyp, ns, wp, pa_nactd, pa_vactd,
 * tstep, time, istp, level, lcharge, initialize)  (mo_salsa_driver.f90:112-435). */
int salsa_gb300_run(salsa_handle_t *h, int nzp, int nxp, int nyp, int ns,
                    double tstep, double time, int istp, int level, int lcharge,
                    int initialize, const salsa_fields_t *f, salsa_status_t *st);

/* Same as salsa_gb300_run but enqueued on the caller's CUDA stream (a
 * cudaStream_t passed as void*); all field pointers must be device pointers.
 * Status counters are written to st after the stream reaches the end of the
 * step only if sync != 0. */
int salsa_gb300_run_async(salsa_handle_t *h, int nzp, int nxp, int nyp, int ns,
                          double tstep, double time, int istp, int level, int lcharge,
                          int initialize, const salsa_fields_t *f, void *stream,
                          int sync, salsa_status_t *st);

/* No counterpart in the reference.  The step for callers that must not allocate GPU
 * memory: a model that gives all free device memory to its own pool at start-up (a
 * later cudaMalloc then fails), or one whose time loop cannot afford the
 * device-wide synchronisation that cudaMalloc and cudaFree imply.  Same arguments
 * and results as salsa_gb300_run_async (device pointers only), but the scratch the
 * step needs -- the cell-order list and the status counters -- sits in a static
 * device array of the library: 8 MiB, enough for SALSA_NOALLOC_MAXCELLS =
 * 2,097,152 interior cells (larger grids return SALSA_E_ARG).  Every GPU that loads
 * the library holds that array until the process exits.  The array keeps the last
 * call's contents; each call clears the status counters on its stream and rewrites
 * the whole order list.  salsa_gb300_init, not the first call, loads the step's
 * kernel modules on the handle's device (the array is part of one of them: with lazy
 * module loading a module's device memory is taken when it loads) and looks up the
 * array's device address there (cudaGetSymbolAddress); so create the handle before
 * the caller's pool takes the free memory.  All calls on one device share the array: calls that overlap
 * on the GPU (other streams, other handles on that device) race on it, so the
 * caller must serialise them. */
#define SALSA_NOALLOC_MAXCELLS 2097152
int salsa_gb300_run_noalloc(salsa_handle_t *h, int nzp, int nxp, int nyp, int ns,
                            double tstep, double time, int istp, int level, int lcharge,
                            int initialize, const salsa_fields_t *f, void *stream,
                            int sync, salsa_status_t *st);

/* Bin layout queries (mo_submctl.f90 nbins/ncld/nprc/nice and the diameter
 * limit tables aerobins/cloudbins/precpbins/icebins, mo_salsa_init.f90:236-239). */
int salsa_gb300_layout(const salsa_handle_t *h, int *nbins, int *ncld, int *nprc,
                       int *nice, int *nwet, double *lolim_diam /* ntotal or NULL */);

/* Number of kernel launches the last run issued (for launch accounting). */
int salsa_gb300_last_launches(const salsa_handle_t *h);

/* Device time in ms of the last run's kernels (cell-order pre-pass and step kernel). */
double salsa_gb300_last_kernel_ms(const salsa_handle_t *h);

void salsa_gb300_finalize(salsa_handle_t *h);

const char *salsa_gb300_version(void);

/* ---- LES-side constraints after the step (src/src_LES/constrain_SALSA.f90) ----
 * t_step (step.f90:330-334) follows run_SALSA with tend_constrain2, the scalar
 * update, tend0 and SALSA_diagnostics; the two SALSA routines are here, on the same
 * arrays as run_SALSA.  Value arrays (time level 1) and tendencies (level 2) of the
 * SALSA_4d tracers (mo_progn_state.f90:165-333: naero, maero, ncloud, mcloud, nprecp,
 * mprecp, gaero, nice, mice), the IN deficit and the charge time are in/out; rh and
 * rhi (relative humidities over water and ice), temp and rp are the thermodynamic
 * diagnostics SALSA_diagnostics reads, and rc, srp, snrp, rtot, ri, riri the
 * diagnostic mixing ratios it writes (mo_diag_state.f90).  Arrays the level or
 * configuration does not use may be NULL.  Device pointers only: these routines serve
 * an LES whose fields live on the GPU.  Calls are asynchronous on `stream` (the
 * library stream when NULL). */
typedef struct {
  double *naero, *ncloud, *nprecp, *nice;           /* (nzp,nxp,nyp,nb) #/kg */
  double *maero, *mcloud, *mprecp, *mice;           /* (...,nspec*nb) kg/kg */
  double *gaero;                                    /* (...,5) #/kg */
  double *indef;                                    /* (...,nliquid) */
  double *chargeTime;                               /* (...,nliquid) */
  double *naerot, *ncloudt, *nprecpt, *nicet;       /* tendencies of the above */
  double *maerot, *mcloudt, *mprecpt, *micet, *gaerot;
  const double *rh, *rhi, *temp, *rp;               /* (nzp,nxp,nyp) */
  double *rc, *srp, *snrp, *rtot, *ri, *riri;       /* (nzp,nxp,nyp) */
} salsa_post_fields_t;

/* tend_constrain2 (constrain_SALSA.f90:18-35): every tendency element of the SALSA_4d
 * tracers becomes at least (-1 + 1e-8) * value / dtlt, so that one step of length dtlt
 * leaves a value above zero; with ice_theta_dist at level 5 the IN deficit is
 * clipped to [0, 1]. */
int salsa_gb300_tend_constrain(salsa_handle_t *h, int nzp, int nxp, int nyp, double dtlt,
                               const salsa_post_fields_t *f, void *stream);

/* SALSA_diagnostics (constrain_SALSA.f90:52-370, findDry4Wet :376-463): negative
 * values to zero; unless only_diag, particles with number but no mass are removed,
 * evaporating cloud droplets, drops and ice return their number and mass to the
 * aerosol bins, and aerosol bins below 0.1 nm dry diameter are emptied (their
 * volatile species to the gases when gas condensation is on); then the water
 * diagnostics rc, srp, snrp, rtot (and ri, riri at level 5) are recomputed. */
int salsa_gb300_diagnostics(salsa_handle_t *h, int nzp, int nxp, int nyp, int only_diag, int lcharge,
                            const salsa_post_fields_t *f, void *stream);

/* ---- Sedimentation and deposition of the bins (src/src_LES/mcrp.f90:745-1275) ----
 * sedim_SALSA, called by micro after the step (step.f90:342): DepositionSlow for the
 * aerosol and cloud bins (flux divergence of the fall speed, dry deposition on the
 * lowest level) and DepositionFast for precipitation and ice (each parcel falls the
 * distance of one time step, which may cross several levels).  Values are read; the
 * tendencies, the liquid water potential temperature tendency tlt, the precipitation
 * and ice fluxes rrate/irate (nzp,nxp,nyp) and sfcrrate/sfcirate (nxp,nyp) and the
 * terminal velocities VtPrc/VtIce (nzp,nxp,nyp,nprc|nice) are written (the rates and
 * velocities are overwritten, the tendencies and tlt added to).  tk, th and adn are the
 * absolute and potential temperature and the air density; ustar (nxp,nyp) is the
 * friction velocity and dzt (nzp) the inverse level thickness.  sed[0..3] switch the
 * aerosol, cloud, precipitation and ice parts (sed_aero .. sed_ice); ice only at level
 * 5.  Device pointers; asynchronous on `stream` (the library stream when NULL). */
typedef struct {
  const double *naero, *ncloud, *nprecp, *nice;       /* (nzp,nxp,nyp,nb) #/kg */
  const double *maero, *mcloud, *mprecp, *mice;       /* (...,nspec*nb) kg/kg */
  double *naerot, *ncloudt, *nprecpt, *nicet;         /* tendencies, added to */
  double *maerot, *mcloudt, *mprecpt, *micet;
  const double *tk, *th, *adn;                        /* (nzp,nxp,nyp) */
  const double *ustar;                                /* (nxp,nyp) */
  const double *dzt;                                  /* (nzp) */
  double *tlt;                                        /* (nzp,nxp,nyp), added to */
  double *rrate, *irate;                              /* (nzp,nxp,nyp) W/m2 */
  double *sfcrrate, *sfcirate;                        /* (nxp,nyp) W/m2 */
  double *VtPrc, *VtIce;                              /* (nzp,nxp,nyp,nprc|nice) m/s */
} salsa_sedim_fields_t;

int salsa_gb300_sedimentation(salsa_handle_t *h, int nzp, int nxp, int nyp, double dtlt, const int sed[4],
                              const salsa_sedim_fields_t *f, void *stream);

/* ---- Gradient harness (no counterpart in the reference, which has no adjoint) ----
 * A chain advances ncell independent warm cells (a level-4 handle) through nsub
 * steps of length dt.  Each step is the coagulation (mo_salsa_dynamics.f90:92-202)
 * followed by the water condensation (mo_salsa_dynamics.f90:691-1125 with the water
 * uptake of mo_salsa_properties.f90:73-380); precipitation bins must stay empty
 * (no autoconversion, activation or redistribution in the chain).  At the start of
 * every step the vapour is imposed as rv = rs (1 + ssat), and the solute term of the
 * water activity is kappa * V_soluble.
 * The state of a cell is nstate = nliquid * (1 + nwet) doubles: the numbers of the
 * liquid bins [#/kg], then the masses m[s][b] [kg/kg] (species-major, liquid bins
 * fastest).  x arrays are [ncell][nstate]; all pointers are device pointers.
 * Calls are synchronous on the library stream (or on `stream` when not NULL). */
typedef struct {
  int ncell;
  int nsub;
  double dt;                                      /* s, at most 1.2 */
  const double *temp, *press, *rs, *dn;           /* [ncell]: K, Pa, kg/kg, kg/m3 */
  const double *kappa;                            /* [ncell] solute hygroscopicity */
  const double *ssat;                             /* [ncell] imposed supersaturation */
} salsa_chain_t;

/* nstate of the handle's layout (0 when the handle is not level 4). */
int salsa_gb300_chain_state_size(const salsa_handle_t *h);

/* Device memory in bytes that a forward + adjoint pair with checkpoint spacing
 * ckpt_every takes beyond its input and output arrays: the checkpoints, the per-cell
 * tape of one step, the states of one checkpoint segment (ckpt_every > 1) and the
 * work counters (-1 for a bad argument or a handle that is not level 4).  No
 * counterpart in the reference: it lets the caller choose the spacing that fits. */
long long salsa_gb300_chain_adjoint_bytes(const salsa_handle_t *h, int ncell, int nsub, double dt,
                                          int ckpt_every);

/* xN = chain(x0).  ckpt (NULL or [ceil(nsub/ckpt_every)][ncell][nstate]) receives
 * the states entering steps 0, ckpt_every, 2 ckpt_every, ... in SALSA units (#/m3,
 * m3/m3), the form in which the adjoint restarts from them. */
int salsa_gb300_chain_forward(salsa_handle_t *h, const salsa_chain_t *c, const double *x0, double *xN,
                              double *ckpt, int ckpt_every, void *stream);

/* Tangent-linear model: xN and dxN = J (dx0, dkappa, dssat); the d* inputs may be NULL (zero). */
int salsa_gb300_chain_tlm(salsa_handle_t *h, const salsa_chain_t *c, const double *x0, const double *dx0,
                          const double *dkappa, const double *dssat, double *xN, double *dxN, void *stream);

/* Adjoint: xbar0 = J_x^T xbarN, kappabar = J_kappa^T xbarN, ssatbar = J_ssat^T xbarN.
 * ckpt holds the states written by salsa_gb300_chain_forward with the same
 * ckpt_every; the states between checkpoints are recomputed. */
int salsa_gb300_chain_adjoint(salsa_handle_t *h, const salsa_chain_t *c, const double *ckpt, int ckpt_every,
                              const double *xbarN, double *xbar0, double *kappabar, double *ssatbar,
                              void *stream);

#ifdef __cplusplus
}
#endif
#endif
