/*
 * salsa_ref.c -- CPU oracle: FP64 restatement of UCLALES-SALSA run_SALSA/salsa.
 *
 * TEST INFRASTRUCTURE ONLY (parity checker and timed CPU baseline); see
 * salsa_ref.h for the parity status ("parity unpinned" against the Fortran,
 * which cannot be compiled here).
 *
 * Structure follows the reference modules one routine per Fortran routine, with
 * 0-based bin and species indices.  Every routine cites the reference lines it
 * restates (paths relative to the UCLALES-SALSA tree).  Build with
 * -ffp-contract=off so no fused multiply-add changes the rounding of the
 * Fortran expressions (the reference is built for x86-64 SSE2, no FMA).
 */
#include <math.h>
#include <float.h>
#include <stddef.h>
#include <stdlib.h>
#include <string.h>
#include <stdio.h>
#ifdef _OPENMP
#include <omp.h>
#endif
#include "salsa_ref.h"

/* ---- rounding perturbation of the library functions (test infrastructure) ----
 * Two correct FP64 implementations of this path differ in how their exp, log, pow and
 * cube roots round (glibc here, CUDA's functions on the GPU): by one or two ulps.  The
 * parity tests measure the oracle's own response to that difference: with a mode set,
 * every result of those functions moves by two ulps, up (+1), down (-1), or in a
 * direction taken from the bits of the argument (modes 2 and above, one pattern each).
 * sqrt rounds correctly on both sides and is left alone.  Mode 0 (the default) leaves
 * every result as it is. */
static int g_libm_pert = 0;
void salsa_ref_set_libm_perturbation(int mode) { g_libm_pert = mode; }
static inline double pert_ulp(double r, double x) {
  if (!g_libm_pert || !isfinite(r) || r == 0.) return r;
  int up = g_libm_pert > 0;
  if (g_libm_pert >= 2) {
    unsigned long long b;
    memcpy(&b, &x, sizeof b);
    b += 0x9e3779b97f4a7c15ULL * (unsigned long long)g_libm_pert;   /* one direction pattern per mode */
    b ^= b >> 29;
    b *= 0xbf58476d1ce4e5b9ULL;
    b ^= b >> 32;
    up = (int)(b & 1u);
  }
  /* two ulps: the documented bound of CUDA's pow (exp, log and cbrt are within one) */
  const double dir = up ? INFINITY : -INFINITY;
  return nextafter(nextafter(r, dir), dir);
}
#define exp(x) pert_ulp(exp(x), (x))
#define log(x) pert_ulp(log(x), (x))
#define log10(x) pert_ulp(log10(x), (x))
#define pow(x, y) pert_ulp(pow((x), (y)), (x) + (y))
#define erf(x) pert_ulp(erf(x), (x))
#define cos(x) pert_ulp(cos(x), (x))

/* ---- constants: src/src_shared/mo_submctl.f90:253-338 (truncated as written) ---- */
#define AVOG   6.0221e+23
#define BOLTZ  1.3807e-23
#define PLANCK 6.626070040e-34
#define GRAV   9.81
#define PSTAND 1.01325e+5
#define RG     8.314
#define PI     3.1415927
#define PI6    0.5235988
#define MAIR   28.97e-3
#define CPA    1005.
#define EPSR   DBL_EPSILON
#define RD     287.04
#define ALV    2.5e6
#define ALS    2.834e6
#define SURFW0 0.073
#define SURFI0 0.105
#define EPSOC  0.15
#define NLIM   1.0
#define PRLIM  1.e-6
#define DLAERO  30.e-6
#define DLCLOUD 100.e-6
#define DLPRECP 5.e-3
#define DLICE   10.e-3
#define MWA_C   18.016e-3
#define RHOWA_C 1000.
#define MVWA   (MWA_C/AVOG/RHOWA_C)
/* condensing vapours (mo_submctl.f90:284-322) */
#define MSU_C  98.08e-3
#define MOC_C  150.e-3
#define RHOSU_C 1830.
#define RHOOC_C 1400.
#define MVSU   (MSU_C/AVOG/RHOSU_C)
#define MVOC   (MOC_C/AVOG/RHOOC_C)
#define D_SA   5.539376964394570e-10
#define N3     158.79
/* math_functions.f90:7 uses full-precision pi */
#define PI_FULL 3.14159265358979323846264338327

#define MAXB SALSA_MAXBINS
#define DLLIQ_RS 24.0e-6   /* mo_salsa_SIP_RS.f90:17: smallest drop that splinters on riming */
#define DSPLINT 10.e-6     /* :21: splinter diameter */
#define DLLIQ_DF 100.e-6   /* mo_salsa_SIP_DF.f90:18: smallest drop that fractures on freezing */
#define NSP  SALSA_MAXNSP

static inline double sq(double x) { return x * x; }
static inline double cube(double x) { return x * x * x; }
static inline double fmaxd(double a, double b) { return a > b ? a : b; }
static inline double fmind(double a, double b) { return a < b ? a : b; }

/* ---- Section (classSection.f90:5-50) ---- */
typedef struct {
  double vhilim, vlolim, vratiohi, vratiolo, dmid;
  double dwet, ddry, dins, dnsp, numc, core;
  double volc[NSP];
  double rhomean, rhoeff;
  int phase;
  double nlim, dlim;
  double INdef, chargeTime, chargeTimeMax, chargeCollEnh;
  double sip[3];   /* SIP_drfr, SIP_rmspl, SIP_iibr (:42-44): crystals from each scheme */
} Section;

/* Rate (classProcessRates.f90:37-41) */
typedef struct { double volc[NSP]; double numc; } Rate;
enum { R_AUTOC = 0, R_AUTOC50, R_AUTOC80, R_ACCR, R_ACCR50, R_ACCR80, R_ACCOLL, R_APCOLL,
       R_AICOLL, R_ACTIV, R_ICEHOM, R_ICEIMM, R_ICEDEP, R_CONDA, R_CONDC, R_CONDP, R_CONDI,
       R_SIPDRFR, R_SIPRMSPL, R_SIPIIBR, R_N };

typedef struct { double alpha, beta, gamma, sigma; } Shape;   /* mo_ice_shape.f90:33-35 */

struct salsa_ref_ctx {
  salsa_config_t cfg;
  /* species (classSpecies.f90:167-244) */
  int nused, ndry, nwet, iwa, irim;
  double rholiq[NSP], rhoice[NSP], MM[NSP], diss[NSP];
  int nsoluble, ninsoluble, ind_soluble[5], ind_insoluble[2];
  int idx_name[9];    /* mass-array index of SO4 OC BC DU SS NO NH H2O rime, -1 if unused */
  double rhosu, rhooc, rhono, rhoss, msu, moc, mno, mss;   /* spec%rho**, spec%m** pointers */
  double rhoic, rhori, rhowa, mwa;
  /* bins (mo_salsa_init.f90:148-450) */
  int nbins, ncld, nprc, nice, ntotal, nliquid;
  int in1a, fn1a, in2a, fn2a, in2b, fn2b;
  int ica_cur, ica_par, fca_cur, fca_par, icb_cur, icb_par, fcb_cur, fcb_par;
  Section tmpl[MAXB];
  double precpbins[MAXB], icebins[MAXB];
  double massacc[MAXB];
  /* sticky switch states (mo_salsa_driver.f90:445-474) */
  int st_coag, st_cnd, st_auto, st_activ, st_icenucl, st_icemelt, st_secice, st_freeRH,
      st_freeTheta, lcgupdt;
  int st_siprs, st_sipdf, st_sipib;   /* lssiprimespln, lssipdropfrac, lssipicecollbreak states
                                          (lssub, mo_salsa_driver.f90:458-461) */
  long long counters[5];
  Section carry[MAXB];
  int carry_valid;
  /* kernel storage of lscoag%mode = 2 (mo_salsa_driver.f90:52-55, 601-697): per interior
     cell the ten kernel arrays, zero until first stored */
  double *kcache;
  long long kcache_cells;
};

/* Per-cell working state: the module arrays allSALSA, zcc**, rateDiag. */
typedef struct {
  const salsa_ref_ctx_t *c;
  Section all[MAXB];
  Section *aero, *cloud, *precp, *ice, *liquid;
  /* kernels, laid out as buildKernel writes them: zcc[i*n2 + j] = coagc(cat1 i, cat2 j) */
  double zccaa[MAXB * MAXB], zcccc[MAXB * MAXB], zccpp[MAXB * MAXB], zccii[MAXB * MAXB];
  double zccca[MAXB * MAXB], zccpa[MAXB * MAXB], zccia[MAXB * MAXB];
  double zccpc[MAXB * MAXB], zccic[MAXB * MAXB], zccip[MAXB * MAXB];
  /* rime-splintering tallies nfrzn_rs / mfrzn_rs (mo_salsa_SIP_RS.f90:14), (nprc, nice):
     number and mass of drops frozen onto each ice bin; cleared per cell */
  double nfrzn_rs[MAXB * MAXB], mfrzn_rs[MAXB * MAXB];
  double nfrzn_df[MAXB * MAXB], mfrzn_df[MAXB * MAXB];   /* drop fracturing's (mo_salsa_SIP_DF.f90:15) */
  double nii_ibr[MAXB * MAXB], mii_ibr[MAXB * MAXB];     /* ice-ice breakup's (mo_salsa_SIP_IIBR.f90:15), (nice, nice) */
  Rate rate[R_N];
  int lcharge, level;
  /* status flags */
  int f_equil, f_distr, f_negfrac, f_cond, f_neg;
  long long cnt[5];
  const double *kappa;   /* NULL or per-cell kappa override */
  double kappa_cell;
  long long cell;        /* interior cell index (kernel storage) */
} Cell;

static void rate_acc_n(Rate *r, double n) { r->numc += n; }
static void rate_acc_v(Rate *r, const double *v, int nv) { for (int i = 0; i < nv; i++) r->volc[i] += v[i]; }

/* ======================================================================
 * Section type-bound procedures: classSection.f90:91-224
 * ====================================================================== */

/* mo_ice_shape.f90:104-107 */
static double getBulkRho(const salsa_ref_ctx_t *c, double Fr) { return Fr * c->rhori + (1. - Fr) * c->rhoic; }

/* mo_ice_shape.f90:46-91 getDiameter */
static double getDiameter(const salsa_ref_ctx_t *c, double mpri, double mrim, double numc) {
  const salsa_config_t *g = &c->cfg;
  double res = 1.e-9;
  if (numc < 1.e-6) return res;
  double Mtot = (mpri + mrim) / numc;
  double Fr = fmaxd(fmind(mrim / (Mtot * numc), 0.9999), 0.0001);
  double rho_b = getBulkRho(c, Fr);
  double Dth = pow(PI6 * c->rhoic / g->iceShapeAlpha, 1. / (g->iceShapeBeta - 3.));
  double Dgr = pow(g->iceShapeAlpha / (PI6 * rho_b), 1. / (3. - g->iceShapeBeta));
  double Dcr = pow((1. / (1. - Fr)) * g->iceShapeAlpha / (PI6 * rho_b), 1. / (3. - g->iceShapeBeta));
  double Mth = c->rhoic * PI6 * cube(Dth);
  double Mgr = rho_b * PI6 * cube(Dgr);
  double Mcr = rho_b * PI6 * cube(Dcr);
  if (Mtot < Mth) {
    res = pow(Mtot / (PI6 * c->rhoic), 1. / 3.);               /* D_spherical :137-141 */
  } else if (Mtot >= Mth && Mtot < Mgr) {
    res = pow(Mtot / g->iceShapeAlpha, 1. / g->iceShapeBeta);  /* D_nonsphericalIce :114-117 */
  } else if (Mtot >= Mgr && Mtot < Mcr) {
    res = pow(Mtot / (PI6 * rho_b), 1. / 3.);
  } else if (Mtot >= Mcr) {
    double hlp = 1. / (1. - Fr);                               /* D_nonsphericalRimed :123-129 */
    res = pow(Mtot / (hlp * g->iceShapeAlpha), 1. / g->iceShapeBeta);
  }
  return res;
}

/* mo_ice_shape.f90:145-191 getShapeCoefficients */
static void getShapeCoefficients(const salsa_ref_ctx_t *c, Shape *s, double mpri, double mrim, double numc) {
  const salsa_config_t *g = &c->cfg;
  s->alpha = PI6 * c->rhoic;
  s->beta = 3.;
  s->gamma = PI / 4.;
  s->sigma = 2.;
  if (numc < 1.e-6) return;
  double Mtot = (mpri + mrim) / numc;
  double Fr = fmaxd(fmind(mrim / (Mtot * numc), 0.9999), 0.0001);
  double rho_b = getBulkRho(c, Fr);
  double Dth = pow(PI6 * c->rhoic / g->iceShapeAlpha, 1. / (g->iceShapeBeta - 3.));
  double Dgr = pow(g->iceShapeAlpha / (PI6 * rho_b), 1. / (3. - g->iceShapeBeta));
  double Dcr = pow((1. / (1. - Fr)) * g->iceShapeAlpha / (PI6 * rho_b), 1. / (3. - g->iceShapeBeta));
  double Mth = c->rhoic * PI6 * cube(Dth);
  double Mgr = rho_b * PI6 * cube(Dgr);
  double Mcr = rho_b * PI6 * cube(Dcr);
  if (Mtot >= Mth && Mtot < Mgr) {
    s->alpha = g->iceShapeAlpha;
    s->beta = g->iceShapeBeta;
    s->gamma = g->iceShapeGamma;
    s->sigma = g->iceShapeSigma;
  } else if (Mtot > Mcr) {
    double hlp = 1. / (1. - Fr);
    s->alpha = g->iceShapeAlpha * hlp;
    s->beta = g->iceShapeBeta;
    s->gamma = g->iceShapeGamma * (1. - Fr) + PI / 4. * Fr;
    s->sigma = g->iceShapeSigma * (1. - Fr) + 2. * Fr;
  }
}

enum { T_WET = 1, T_DRY = 2, T_INS = 4, T_NSP = 8, T_ALL = 15 };

/* classSection.f90:91-159 updateDiameter */
static void updateDiameter(const salsa_ref_ctx_t *c, Section *s, int limit, int type) {
  int nwet = c->nwet, ndry = c->ndry, nnsp = c->nused;
  if (s->numc > s->nlim) {
    if (type & T_NSP) {
      s->dnsp = 1.e-10;
      if (s->phase == 4) {
        double mpri = 0.;
        for (int i = 0; i < nwet; i++) mpri += s->volc[i] * c->rhoice[i];
        double mrim = s->volc[nnsp - 1] * c->rhori;
        s->dnsp = getDiameter(c, mpri, mrim, s->numc);
      }
    }
    if (type & T_WET) {
      double v = 0.;
      for (int i = 0; i < NSP; i++) v += s->volc[i];   /* SUM(volc(:)) over all 9 */
      s->dwet = pow(v / s->numc / PI6, 1. / 3.);
    }
    if (type & T_DRY) {
      double v = 0.;
      for (int i = 0; i < ndry; i++) v += s->volc[i];
      s->ddry = pow(v / s->numc / PI6, 1. / 3.);
    }
    if (type & T_INS) {   /* ALL(ind_insoluble > 0) is true for an empty list: dins = 0 then */
      double v = 0.;
      for (int i = 0; i < c->ninsoluble; i++) v += s->volc[c->ind_insoluble[i]];
      s->dins = pow(v / s->numc / PI6, 1. / 3.);
    }
  } else {
    if (type & T_NSP) s->dnsp = s->dmid;
    if (type & T_WET) s->dwet = s->dmid;
    if (type & T_DRY) s->ddry = s->dmid;
    if (type & T_INS) s->dins = s->dmid;
  }
  if (limit) {
    if (type & T_NSP) s->dnsp = fmind(s->dwet, s->dlim);
    if (type & T_WET) s->dwet = fmind(s->dwet, s->dlim);
    if (type & T_DRY) s->ddry = fmind(s->ddry, s->dlim);
    if (type & T_INS) s->dins = fmind(s->dins, s->dlim);
  }
}

/* classSection.f90:169-195 updateRhomean */
static void updateRhomean(const salsa_ref_ctx_t *c, Section *s) {
  s->rhomean = c->rhowa;
  if (s->phase > 3) {
    if (s->numc > s->nlim) {
      double mass_p = c->rhoic * s->volc[c->iwa];
      double mass_r = c->rhori * s->volc[c->irim];
      double mass_t = mass_p + mass_r;
      s->rhomean = (mass_p * c->rhoic + mass_r * c->rhori) / fmaxd(mass_t, 7.e-25);
      s->rhomean = fmind(s->rhomean, c->rhoic);
    } else {
      s->rhomean = c->rhoic;
    }
  } else {
    s->rhomean = c->rhowa;
  }
}

/* classSection.f90:202-224 getRimeFraction */
static double getRimeFraction(const salsa_ref_ctx_t *c, const Section *s) {
  double r = 0.;
  if (s->phase == 4 && s->volc[c->iwa] > 1.e-23 && s->volc[c->irim] > 1.e-23 && s->numc > s->nlim)
    r = s->volc[c->irim] * c->rhori / (s->volc[c->iwa] * c->rhoic + s->volc[c->irim] * c->rhori);
  return r;
}

/* ======================================================================
 * Terminal velocity: mo_particle_external_properties.f90:237-352
 * ====================================================================== */
static double kc1213(double X) { const double c1 = 0.0902; return sqrt(1. + c1 * sqrt(X)); }
static double kcbre(double X) {
  const double c1 = 0.0902;
  double r = 0.5 * c1 * sqrt(X);
  r = r / (kc1213(X) - 1.);
  r = r / kc1213(X);
  return r;
}
static double kcare(double X) {
  const double delta0 = 9.06;
  double bre = kcbre(X);
  double r = 0.25 * sq(delta0);
  r = r * sq(kc1213(X) - 1.);
  r = r / pow(X, bre);
  return r;
}
static double kcAv(const Shape *s, double X, double visc, double rhoa) {
  double are = kcare(X), bre = kcbre(X);
  double r = are * pow(visc, 1. - 2. * bre);
  r = r * pow((2. * s->alpha * GRAV) / (rhoa * s->gamma), bre);
  return r;
}
static double kcBv(const Shape *s, double X) { double bre = kcbre(X); return bre * (s->beta - s->sigma + 2.) - 1.; }
static double kcVt(const Shape *s, double D, double X, double visc, double rhoa) {
  double Av = kcAv(s, X, visc, rhoa), Bv = kcBv(s, X);
  return Av * pow(D, Bv);
}

static double terminal_vel(double diam, double rhop, double rhoa, double visc, double beta, int flag,
                           const Shape *shape, double dnsp) {
  const double rhoa_ref = 1.225; (void)rhoa_ref;
  double tv = 0.;
  if (flag == 1 || flag == 2 || flag == 3) {
    if (diam <= 19E-6) {
      tv = sq(diam) * (rhop - rhoa) * GRAV * beta / (18. * visc);
    } else if (diam > 19E-6 && diam < 1.07E-3) {
      double NDa = 4. / 3. * pow(diam, 3.) * GRAV * (rhop - rhoa) * rhoa / pow(visc, 2.);
      double X = log(NDa);
      double Y = -0.318657E1 + 0.992696 * X - 0.153193E-2 * sq(X) - 0.987059E-3 * cube(X)
                 - 0.578878E-3 * sq(sq(X)) + 0.855176E-4 * sq(sq(X)) * X - 0.327815E-5 * cube(sq(X));
      double Re2 = beta * exp(Y);
      tv = visc / rhoa / diam * Re2;
    } else {
      double Np = pow(SURFW0, 3.) * pow(rhoa, 2.) / (pow(visc, 4.) * (rhop - rhoa) * GRAV);
      double Bo = 4. / 3. * (rhop - rhoa) * GRAV / SURFW0 * pow(diam, 2.);
      double X3 = log(Bo * pow(Np, 1. / 6.));
      double Y3 = -0.500015E1 + 0.523778E1 * X3 - 0.204914E1 * sq(X3) + 0.475294 * cube(X3)
                  - 0.542819E-1 * sq(sq(X3)) + 0.238449E-2 * sq(sq(X3)) * X3;
      double Re3 = pow(Np, 1. / 6.) * exp(Y3);
      tv = fmind(visc / rhoa / diam * Re3, 9.2);
    }
  } else if (flag == 4) {
    double Vb = PI6 * cube(diam);
    double Ap = shape->gamma * pow(dnsp, shape->sigma);
    double X = (2. * Vb * (rhop - rhoa) * GRAV * sq(dnsp)) / (Ap * rhoa * sq(visc));
    tv = kcVt(shape, dnsp, X, visc, rhoa);
  }
  return tv;
}

double salsa_ref_terminal_vel(double diam, double rhop, double rhoa, double visc, double beta, int flag) {
  return terminal_vel(diam, rhop, rhoa, visc, beta, flag, NULL, 0.);
}

/* ======================================================================
 * Coagulation kernels: mo_salsa_coagulation_kernels.f90
 * ====================================================================== */

/* :185-420 coagc (kernel == 2 is the only variant called) */
static double coagc(const salsa_ref_ctx_t *c, const Section *pp1, const Section *pp2, double temp,
                    double pres, int lcharge) {
  const salsa_config_t *g = &c->cfg;
  int ns = c->nused;
  double diam1 = (pp1->phase == 4) ? pp1->dnsp : pp1->dwet;
  double diam2 = (pp2->phase == 4) ? pp2->dnsp : pp2->dwet;
  double dsph1 = pp1->dwet, dsph2 = pp2->dwet;
  double mass1 = pp1->rhomean * PI6 * cube(dsph1);
  double mass2 = pp2->rhomean * PI6 * cube(dsph2);
  if (fabs(pp1->dmid - pp2->dmid) / pp1->dmid < 1.e-2) {
    diam1 = 1.1 * diam2;
    mass1 = 1.33 * mass2;
  }
  double diam[2] = {diam1, diam2}, mpart[2] = {mass1, mass2};
  double visc = (7.44523e-3 * sqrt(cube(temp))) / (5093. * (temp + 110.4));
  double mfp = (1.656e-10 * temp + 1.828e-8) * PSTAND / pres;
  double knud[2], beta[2], dfpart[2], mtvel[2], omega[2], tva[2], flux[2], termv[2], zrhop[2];
  for (int i = 0; i < 2; i++) {
    knud[i] = 2. * mfp / diam[i];
    beta[i] = 1. + knud[i] * (1.142 + 0.558 * exp(-0.999 / knud[i]));
    dfpart[i] = beta[i] * BOLTZ * temp / (3. * PI * visc * diam[i]);
    mtvel[i] = sqrt((8. * BOLTZ * temp) / (PI * mpart[i]));
    omega[i] = 8. * dfpart[i] / (PI * mtvel[i]);
  }
  double mdiam = 0.5 * (diam[0] + diam[1]);
  flux[0] = 4. * PI * mdiam * (dfpart[0] + dfpart[1]);
  flux[1] = PI * sqrt(sq(mtvel[0]) + sq(mtvel[1])) * sq(mdiam);
  for (int i = 0; i < 2; i++)
    tva[i] = (cube(mdiam + omega[i]) - (sq(mdiam) + sq(omega[i])) * sqrt(sq(mdiam) + sq(omega[i]))) /
                 (3. * mdiam * omega[i]) - mdiam;
  double fmdist = sqrt(sq(tva[0]) + sq(tva[1]));

  int sml = 0, lrg = 1;
  if (diam[0] >= diam[1]) { lrg = 0; sml = 1; }
  Shape shape1 = {0, 0, 0, 0}, shape2 = {0, 0, 0, 0};
  if (pp1->phase == 4) {
    double mp = 0.;
    for (int i = 0; i < ns - 1; i++) mp += pp1->volc[i] * c->rhoic;
    getShapeCoefficients(c, &shape1, mp, pp1->volc[ns - 1] * c->rhori, pp1->numc);
  }
  if (pp2->phase == 4) {
    double mp = 0.;
    for (int i = 0; i < ns - 1; i++) mp += pp2->volc[i] * c->rhoic;
    getShapeCoefficients(c, &shape2, mp, pp2->volc[ns - 1] * c->rhori, pp2->numc);
  }
  double zrhoa = pres / (RD * temp);
  for (int i = 0; i < 2; i++) zrhop[i] = mpart[i] / (PI6 * cube(diam[i]));
  (void)zrhop;
  double vkin = visc / zrhoa;
  if (pp1->phase < 4) termv[0] = terminal_vel(diam1, pp1->rhomean, zrhoa, visc, beta[0], pp1->phase, NULL, 0.);
  else termv[0] = terminal_vel(dsph1, pp1->rhomean, zrhoa, visc, beta[0], pp1->phase, &shape1, diam1);
  if (pp2->phase < 4) termv[1] = terminal_vel(diam2, pp2->rhomean, zrhoa, visc, beta[1], pp2->phase, NULL, 0.);
  else termv[1] = terminal_vel(dsph2, pp2->rhomean, zrhoa, visc, beta[1], pp2->phase, &shape2, diam2);

  double reyn[2], schm[2];
  for (int i = 0; i < 2; i++) { reyn[i] = diam[i] * termv[i] / vkin; schm[i] = vkin / dfpart[i]; }
  double stok = 2. * termv[sml] * fabs(termv[0] - termv[1]) / (diam[lrg] * GRAV);
  double zbrown = flux[0] / (mdiam / (mdiam + fmdist) + flux[0] / flux[1]);
  double zbrconv = 0.;
  if (reyn[lrg] <= 1.) zbrconv = 0.45 * zbrown * pow(reyn[lrg] * schm[sml], 1. / 3.);
  else if (reyn[lrg] > 1.) zbrconv = 0.45 * zbrown * sqrt(reyn[lrg]) * pow(schm[sml], 1. / 3.);
  double ztshear = sqrt(8. * PI * g->eddy_dis / (15. * vkin)) * cube(0.5 * (diam[0] + diam[1]));
  double zturbinert = PI * pow(g->eddy_dis, 0.75) / (GRAV * sqrt(sqrt(vkin))) * sq(0.5 * (diam[0] + diam[1])) *
                      fabs(termv[0] - termv[1]);
  double zea = sq(stok) / sq(stok + 0.5);
  double zev = 0.;
  if (stok > 1.214) {
    zev = 0.75 * log(2. * stok) / (stok - 1.214);
    zev = 1. / sq(1. + zev);
  } else if (stok <= 1.214) {
    zev = 0.;
  }
  double zecoll = (60. * zev + zea * reyn[lrg]) / (60. + reyn[lrg]);
  double zgrav = zecoll * PI * sq(mdiam);
  zgrav = zgrav * fabs(termv[0] - termv[1]);
  double r = zbrown + zbrconv + sqrt(sq(zgrav) + sq(ztshear) + sq(zturbinert));
  if (lcharge)
    r = r + r * pp1->chargeCollEnh * 0.5 * (pp1->chargeTime + pp2->chargeTime) / pp1->chargeTimeMax;
  return r;
}

/* :94-133 buildKernelSelf */
static void buildKernelSelf(Cell *w, int nb1, Section *p1, double *zcc, double T, double P) {
  const salsa_ref_ctx_t *c = w->c;
  for (int i = 0; i < nb1 * nb1; i++) zcc[i] = 0.;
  for (int mm = 0; mm < nb1; mm++) { updateDiameter(c, &p1[mm], 1, T_ALL); updateRhomean(c, &p1[mm]); }
  for (int mm = 0; mm < nb1; mm++) {
    if (p1[mm].numc < p1[mm].nlim) continue;
    for (int nn = mm; nn < nb1; nn++) {
      if (p1[nn].numc < p1[nn].nlim) continue;
      zcc[mm * nb1 + nn] = coagc(c, &p1[mm], &p1[nn], T, P, w->lcharge);
      zcc[nn * nb1 + mm] = zcc[mm * nb1 + nn];
      w->cnt[0]++;
    }
  }
}

/* :137-180 buildKernel; zcc stored [mm*nb2 + nn] */
static void buildKernel(Cell *w, int nb1, Section *p1, int nb2, Section *p2, double *zcc, double T, double P) {
  const salsa_ref_ctx_t *c = w->c;
  for (int i = 0; i < nb1 * nb2; i++) zcc[i] = 0.;
  for (int mm = 0; mm < nb1; mm++) { updateDiameter(c, &p1[mm], 1, T_ALL); updateRhomean(c, &p1[mm]); }
  for (int nn = 0; nn < nb2; nn++) { updateDiameter(c, &p2[nn], 1, T_ALL); updateRhomean(c, &p2[nn]); }
  for (int mm = 0; mm < nb1; mm++) {
    if (p1[mm].numc < p1[mm].nlim) continue;
    for (int nn = 0; nn < nb2; nn++) {
      if (p2[nn].numc < p2[nn].nlim) continue;
      zcc[mm * nb2 + nn] = coagc(c, &p1[mm], &p2[nn], T, P, w->lcharge);
      w->cnt[0]++;
    }
  }
}

/* :24-90 update_coagulation_kernels */
static void update_coagulation_kernels(Cell *w, double P, double T) {
  const salsa_ref_ctx_t *c = w->c;
  const salsa_config_t *g = &c->cfg;
  if (g->lscgaa) buildKernelSelf(w, c->nbins, w->aero, w->zccaa, T, P);
  if (g->lscgcc) buildKernelSelf(w, c->ncld, w->cloud, w->zcccc, T, P);
  if (g->lscgpp) buildKernelSelf(w, c->nprc, w->precp, w->zccpp, T, P);
  if (g->lscgii) buildKernelSelf(w, c->nice, w->ice, w->zccii, T, P);
  if (g->lscgca) buildKernel(w, c->nbins, w->aero, c->ncld, w->cloud, w->zccca, T, P);
  if (g->lscgpa) buildKernel(w, c->nbins, w->aero, c->nprc, w->precp, w->zccpa, T, P);
  if (g->lscgia) buildKernel(w, c->nbins, w->aero, c->nice, w->ice, w->zccia, T, P);
  if (g->lscgpc) buildKernel(w, c->ncld, w->cloud, c->nprc, w->precp, w->zccpc, T, P);
  if (g->lscgic) buildKernel(w, c->ncld, w->cloud, c->nice, w->ice, w->zccic, T, P);
  if (g->lscgip) buildKernel(w, c->nprc, w->precp, c->nice, w->ice, w->zccip, T, P);
}

double salsa_ref_coagc_pair(const salsa_ref_ctx_t *c, int b1, int b2, double numc1, double dwet1, double numc2,
                            double dwet2, double temp, double pres) {
  Section s1 = c->tmpl[b1], s2 = c->tmpl[b2];
  s1.numc = numc1; s2.numc = numc2;
  s1.volc[c->iwa] = numc1 * PI6 * cube(dwet1);
  s2.volc[c->iwa] = numc2 * PI6 * cube(dwet2);
  updateDiameter(c, &s1, 1, T_ALL); updateRhomean(c, &s1);
  updateDiameter(c, &s2, 1, T_ALL); updateRhomean(c, &s2);
  return coagc(c, &s1, &s2, temp, pres, 0);
}

/* single-function probe of coagc for two bins given their number concentrations and
   the volume concentrations of all c->nused species (dry, water, then rime for ice),
   with the diameters and mean densities updated as buildKernel updates them */
double salsa_ref_coagc_sections(const salsa_ref_ctx_t *c, int b1, double numc1, const double *volc1, int b2,
                                double numc2, const double *volc2, double temp, double pres) {
  Section s1 = c->tmpl[b1], s2 = c->tmpl[b2];
  s1.numc = numc1; s2.numc = numc2;
  for (int i = 0; i < NSP; i++) {
    s1.volc[i] = i < c->nused ? volc1[i] : 0.;
    s2.volc[i] = i < c->nused ? volc2[i] : 0.;
  }
  updateDiameter(c, &s1, 1, T_ALL); updateRhomean(c, &s1);
  updateDiameter(c, &s2, 1, T_ALL); updateRhomean(c, &s2);
  return coagc(c, &s1, &s2, temp, pres, 0);
}

/* single-function probe of getShapeCoefficients and getDiameter for primary ice mass
   mpri, rime mass mrim and number numc: out = alpha, beta, gamma, sigma, diameter */
void salsa_ref_ice_shape(const salsa_ref_ctx_t *c, double mpri, double mrim, double numc, double out[5]) {
  Shape s;
  getShapeCoefficients(c, &s, mpri, mrim, numc);
  out[0] = s.alpha; out[1] = s.beta; out[2] = s.gamma; out[3] = s.sigma;
  out[4] = getDiameter(c, mpri, mrim, numc);
}

/* ======================================================================
 * Coagulation processes: mo_salsa_coagulation_processes.f90
 * Kernel access helpers follow the dummy-argument shapes of the reference:
 *   KS(z, nb_second, i, j) = zcc(i, j) of an array written by buildKernel
 *   with (nb1 = first, nb2 = second).
 * ====================================================================== */
#define KIDX(z, n2, i, j) ((z)[(i) * (n2) + (j)])

/* :707-1020 accumulateSink.  zcc(nbtrgt, nbcoll): value zcc(itrgt, ll). */
static void accumulateSink(Cell *w, int nbcoll, int itrgt, int istr, int iend, const double *zcc,
                           const Section *coll, double *sink, int trgtphase, double xx) {
  const salsa_ref_ctx_t *c = w->c;
  const salsa_config_t *g = &c->cfg;
  double nrate = 0., nrate50 = 0., nrate80 = 0., nrate_au50 = 0., nrate_au80 = 0.;
  double Eagg[MAXB];
  for (int ll = 0; ll < nbcoll; ll++) Eagg[ll] = 1.;
  if (coll[0].phase == 4 && trgtphase == 4) {
    for (int ll = istr; ll <= iend; ll++) {
      double rimfr = fmaxd(getRimeFraction(c, &coll[ll]), getRimeFraction(c, &coll[itrgt]));
      Eagg[ll] = g->Eiagg_max - rimfr * (g->Eiagg_max - g->Eiagg_min);
    }
  }
  for (int ll = istr; ll <= iend; ll++) {
    double dnum = Eagg[ll] * xx * KIDX(zcc, nbcoll, itrgt, ll) * coll[ll].numc;
    *sink += dnum;
    nrate += dnum;
  }
  if (coll[0].phase == 3) {
    int nprc = c->nprc;
    int cnt80 = 0, cnt50 = 0;
    for (int i = 0; i < nprc; i++) { if (c->precpbins[i] < 80.e-6) cnt80++; if (c->precpbins[i] < 50.e-6) cnt50++; }
    int it_cl = itrgt < nprc - 1 ? itrgt : nprc - 1;   /* MIN(itrgt,nprc) */
    double D = 0.;
    if (trgtphase == 2 || (trgtphase == 3 && c->precpbins[it_cl] < 80.e-6)) {
      for (int ll = cnt80; ll <= iend; ll++)           /* ix = COUNT+1 (1-based) */
        nrate80 += Eagg[ll] * xx * KIDX(zcc, nbcoll, itrgt, ll) * coll[ll].numc;
      int ex = istr > cnt80 - 1 ? istr : cnt80 - 1;     /* MAX(istr, COUNT) (1-based) */
      if (trgtphase == 2) D = w->cloud[itrgt].dwet;
      else if (trgtphase == 3) D = w->precp[itrgt].dwet;
      for (int ll = istr; ll <= ex; ll++)
        if (cube(D) + cube(coll[ll].dwet) >= cube(80.e-6))
          nrate_au80 += Eagg[ll] * xx * KIDX(zcc, nbcoll, itrgt, ll) * coll[ll].numc;
    }
    if (trgtphase == 2 || (trgtphase == 3 && c->precpbins[it_cl] < 50.e-6)) {
      for (int ll = cnt50; ll <= iend; ll++)
        nrate50 += Eagg[ll] * xx * KIDX(zcc, nbcoll, itrgt, ll) * coll[ll].numc;
      int ex = istr > cnt50 - 1 ? istr : cnt50 - 1;
      if (trgtphase == 2) D = w->cloud[itrgt].dwet;
      else if (trgtphase == 3) D = w->precp[itrgt].dwet;
      for (int ll = istr; ll <= ex; ll++)
        if (cube(D) + cube(coll[ll].dwet) >= cube(50.e-6))
          nrate_au50 += Eagg[ll] * xx * KIDX(zcc, nbcoll, itrgt, ll) * coll[ll].numc;
    }
  }
  /* secondary-ice tallies (:863-977) with ice collectors; of them drop fracturing's and
     rime splintering's frozen-drop numbers, per (precipitation bin, ice bin); drops
     collected from cloud bins all count in row 1 */
  if (coll[0].phase == 4 && c->st_secice) {
    double sum = 0.;
    for (int l = 0; l < c->nice; l++) sum += KIDX(zcc, nbcoll, itrgt, l) * coll[l].numc;
    const double fix_coag = fmaxd(1. - sum, 0.1);
    /* ice-ice breakup (:881-896): collisions of the smaller target with larger crystals */
    if (c->st_sipib && trgtphase == 4)
      for (int ll = istr; ll <= iend; ll++)
        if (w->ice[itrgt].dnsp < coll[ll].dnsp && w->ice[itrgt].numc > w->ice[itrgt].nlim && coll[ll].numc > coll[ll].nlim)
          w->nii_ibr[ll * c->nice + itrgt] += Eagg[ll] * KIDX(zcc, nbcoll, ll, itrgt) * coll[ll].numc *
                                               w->ice[itrgt].numc * fix_coag;
    /* drop fracturing (:899-944): drops larger than the collecting crystal (mode 4 would
       count the others too); the drop bin's own numbers are tested twice, as written */
    if (c->st_sipdf && (trgtphase == 3 || trgtphase == 2)) {
      const Section *t = trgtphase == 3 ? &w->precp[itrgt] : &w->cloud[itrgt];
      const int row = trgtphase == 3 ? itrgt : 0;
      for (int ll = istr; ll <= iend; ll++) {
        if (coll[ll].numc > coll[ll].nlim && coll[ll].dwet < t->dwet && t->dwet > DLLIQ_DF && t->numc > t->nlim &&
            coll[ll].numc > coll[ll].nlim)
          w->nfrzn_df[row * c->nice + ll] += Eagg[ll] * KIDX(zcc, nbcoll, itrgt, ll) * coll[ll].numc * t->numc * fix_coag;
        /* :916-921, :936-941: Phillips' full scheme also counts drops collected by larger crystals */
        if (g->lssipdropfrac.mode == 4 && coll[ll].numc > coll[ll].nlim && coll[ll].dwet >= t->dwet &&
            t->dwet > DLLIQ_DF && t->numc > t->nlim)
          w->nfrzn_df[row * c->nice + ll] += Eagg[ll] * KIDX(zcc, nbcoll, itrgt, ll) * coll[ll].numc * t->numc * fix_coag;
      }
    }
    if (c->st_siprs && (trgtphase == 3 || trgtphase == 2)) {
      const Section *t = trgtphase == 3 ? &w->precp[itrgt] : &w->cloud[itrgt];
      const int row = trgtphase == 3 ? itrgt : 0;
      for (int ll = istr; ll <= iend; ll++)
        if (coll[ll].dwet >= t->dwet && t->dwet > DLLIQ_RS && t->numc > t->nlim && coll[ll].numc > coll[ll].nlim)
          w->nfrzn_rs[row * c->nice + ll] += Eagg[ll] * KIDX(zcc, nbcoll, itrgt, ll) * coll[ll].numc * t->numc * fix_coag;
    }
  }
  if (trgtphase == 2) {
    double n = w->cloud[itrgt].numc;
    rate_acc_n(&w->rate[R_ACCR80], nrate80 * n);
    rate_acc_n(&w->rate[R_ACCR50], nrate50 * n);
    rate_acc_n(&w->rate[R_AUTOC80], nrate_au80 * n);
    rate_acc_n(&w->rate[R_AUTOC50], nrate_au50 * n);
  } else if (trgtphase == 3) {
    double n = w->precp[itrgt].numc;
    rate_acc_n(&w->rate[R_ACCR80], nrate80 * n);
    rate_acc_n(&w->rate[R_ACCR50], nrate50 * n);
    rate_acc_n(&w->rate[R_AUTOC80], nrate_au80 * n);
    rate_acc_n(&w->rate[R_AUTOC50], nrate_au50 * n);
  }
  if (coll[0].phase == 3 && trgtphase == 2) rate_acc_n(&w->rate[R_ACCR], nrate * w->cloud[itrgt].numc);
  else if (coll[0].phase == 2 && trgtphase == 1) rate_acc_n(&w->rate[R_ACCOLL], nrate * w->aero[itrgt].numc);
  else if (coll[0].phase == 3 && trgtphase == 1) rate_acc_n(&w->rate[R_APCOLL], nrate * w->aero[itrgt].numc);
  else if (coll[0].phase == 4 && trgtphase == 1) rate_acc_n(&w->rate[R_AICOLL], nrate * w->aero[itrgt].numc);
}

/* :1023-1045 accumulateSinkReverse.  zcc(nbcoll, nbtrgt): value zcc(ll, itrgt). */
static void accumulateSinkReverse(int nbtrgt, int itrgt, int istr, int iend, const double *zcc,
                                  const Section *coll, double *sink) {
  for (int ll = istr; ll <= iend; ll++) *sink += KIDX(zcc, nbtrgt, ll, itrgt) * coll[ll].numc;
}

/* :1049-1217 accumulateSource.  zcc(nbcoll, nbtrgt): value zcc(ll, itrgt). */
static void accumulateSource(Cell *w, int nbtrgt, int nspec, int itrgt, int istr, int iend, const double *zcc,
                             const Section *coll, double *source, int trgtphase) {
  const salsa_ref_ctx_t *c = w->c;
  double vrate[NSP] = {0}, vrate80[NSP] = {0}, vrate50[NSP] = {0}, vau80[NSP] = {0}, vau50[NSP] = {0};
  for (int ll = istr; ll <= iend; ll++) {
    double k = KIDX(zcc, nbtrgt, ll, itrgt);
    for (int s = 0; s < nspec; s++) {
      double dv = k * coll[ll].volc[s];
      vrate[s] += dv;
      source[s] += dv;
    }
  }
  int cnt80 = 0, cnt50 = 0;
  for (int i = 0; i < c->nprc; i++) { if (c->precpbins[i] < 80.e-6) cnt80++; if (c->precpbins[i] < 50.e-6) cnt50++; }
  int cp = coll[0].phase;
  /* autoconversion past 80 um (:1088-1113) */
  {
    double D = 0.;
    int ex = iend;
    if (trgtphase == 3) D = w->precp[itrgt].dwet;
    if (cp == 2) ex = iend;
    else if (cp == 3) ex = iend < cnt80 - 1 ? iend : cnt80 - 1;
    if (D > 0. && D < 80.e-6 && (cp == 2 || cp == 3))
      for (int ll = istr; ll <= ex; ll++)
        if (cube(D) + cube(coll[ll].dwet) > cube(80.e-6)) {
          double k = KIDX(zcc, nbtrgt, ll, itrgt);
          for (int s = 0; s < nspec; s++) vau80[s] += k * coll[ll].volc[s];
        }
  }
  {
    double D = 0.;
    int ex = iend;
    if (trgtphase == 3) D = w->precp[itrgt].dwet;
    if (cp == 2) ex = iend;
    else if (cp == 3) ex = iend < cnt50 - 1 ? iend : cnt50 - 1;
    if (D > 0. && D < 50.e-6 && (cp == 2 || cp == 3))
      for (int ll = istr; ll <= ex; ll++)
        if (cube(D) + cube(coll[ll].dwet) > cube(50.e-6)) {
          double k = KIDX(zcc, nbtrgt, ll, itrgt);
          for (int s = 0; s < nspec; s++) vau50[s] += k * coll[ll].volc[s];
        }
  }
  if (trgtphase == 3 && c->precpbins[itrgt] > 80.e-6) {
    int ex = iend;
    if (cp == 3) ex = iend < cnt80 - 1 ? iend : cnt80 - 1;
    if (cp == 2 || cp == 3)
      for (int ll = istr; ll <= ex; ll++) {
        double k = KIDX(zcc, nbtrgt, ll, itrgt);
        for (int s = 0; s < nspec; s++) vrate80[s] += k * coll[ll].volc[s];
      }
  }
  if (trgtphase == 3 && c->precpbins[itrgt] > 50.e-6) {
    int ex = iend;
    if (cp == 3) ex = iend < cnt50 - 1 ? iend : cnt50 - 1;
    if (cp == 2 || cp == 3)
      for (int ll = istr; ll <= ex; ll++) {
        double k = KIDX(zcc, nbtrgt, ll, itrgt);
        for (int s = 0; s < nspec; s++) vrate50[s] += k * coll[ll].volc[s];
      }
  }
  if (trgtphase == 3) {
    double n = w->precp[itrgt].numc;
    for (int s = 0; s < nspec; s++) { vrate80[s] *= n; vrate50[s] *= n; vau80[s] *= n; vau50[s] *= n; }
    rate_acc_v(&w->rate[R_ACCR80], vrate80, nspec);
    rate_acc_v(&w->rate[R_ACCR50], vrate50, nspec);
    rate_acc_v(&w->rate[R_AUTOC80], vau80, nspec);
    rate_acc_v(&w->rate[R_AUTOC50], vau50, nspec);
  }
  int rid = -1; double n = 0.;
  if (trgtphase == 3 && cp == 2) { rid = R_ACCR; n = w->precp[itrgt].numc; }
  else if (trgtphase == 2 && cp == 1) { rid = R_ACCOLL; n = w->cloud[itrgt].numc; }
  else if (trgtphase == 3 && cp == 1) { rid = R_APCOLL; n = w->precp[itrgt].numc; }
  else if (trgtphase == 4 && cp == 1) { rid = R_AICOLL; n = w->ice[itrgt].numc; }
  if (rid >= 0) {
    for (int s = 0; s < nspec; s++) vrate[s] *= n;
    rate_acc_v(&w->rate[rid], vrate, nspec);
  }
}

/* :1219-1242 accumulateSourceReverse.  zcc(nbtrgt, nbcoll): value zcc(itrgt, ll). */
static void accumulateSourceReverse(int nbcoll, int nspec, int itrgt, int istr, int iend, const double *zcc,
                                    const Section *coll, double *source) {
  for (int ll = istr; ll <= iend; ll++) {
    double k = KIDX(zcc, nbcoll, itrgt, ll);
    for (int s = 0; s < nspec; s++) source[s] += k * coll[ll].volc[s];
  }
}

/* :1244-1381 accumulateSourcePhaseChange.  zcc(nbcoll, nbtrgt): zcc(ll, itrgt). */
static void accumulateSourcePhaseChange(Cell *w, int nbtrgt, int iice, int iwa, int itrgt, int istr, int iend,
                                        double rhotrgt, double rhocoll, const double *zcc, const Section *coll,
                                        double *source) {
  const salsa_ref_ctx_t *c = w->c;
  int ndry = c->ndry;
  for (int ll = istr; ll <= iend; ll++) {
    double k = KIDX(zcc, nbtrgt, ll, itrgt);
    for (int s = 0; s < ndry; s++) source[s] += k * coll[ll].volc[s];
    source[iice] += k * coll[ll].volc[iwa] * rhocoll / rhotrgt;
  }
  /* secondary-ice tallies (:1285-1378).  With lssecice on, the ice target's diameters are
     updated here (:1291-1308), whichever scheme runs; of the tallies, rime splintering's
     frozen-drop masses (:1354-1375), where drops collected from cloud bins use the kernel
     of cloud bin 1 (ix = 1), as written */
  if (c->st_secice) {
    double fix_coag = 1.;
    const int nb = coll[0].phase == 2 ? c->ncld : (coll[0].phase == 3 ? c->nprc : (coll[0].phase == 4 ? c->nice : 0));
    if (nb > 0) {
      double sum = 0.;
      for (int l = 0; l < nb; l++) sum += KIDX(zcc, nbtrgt, l, itrgt) * coll[l].numc;
      fix_coag = fmaxd(1. - sum, 0.1);
      updateDiameter(c, &w->ice[itrgt], 1, T_ALL);
    }
    if (c->st_sipdf)   /* :1312-1346: drops larger than the crystal */
      for (int ll = istr; ll <= iend; ll++) {
        const int ph = coll[ll].phase;
        if (ph != 2 && ph != 3) continue;
        if (w->ice[itrgt].dnsp < coll[ll].dwet && coll[ll].dwet > DLLIQ_DF && w->ice[itrgt].numc > w->ice[itrgt].nlim &&
            coll[ll].numc > coll[ll].nlim) {
          const int ix = ph == 3 ? ll : 0;
          w->mfrzn_df[ix * c->nice + itrgt] +=
              KIDX(zcc, nbtrgt, ix, itrgt) * coll[ll].volc[iwa] * w->ice[itrgt].numc * rhocoll * fix_coag;
        }
        /* :1331-1343: Phillips' full scheme, drops collected by more massive crystals */
        if (c->cfg.lssipdropfrac.mode == 4 && w->ice[itrgt].dnsp >= coll[ll].dwet && coll[ll].dwet > DLLIQ_DF &&
            coll[ll].numc > coll[ll].nlim && w->ice[itrgt].numc > w->ice[itrgt].nlim) {
          const int ix = ph == 3 ? ll : 0;
          w->mfrzn_df[ix * c->nice + itrgt] +=
              KIDX(zcc, nbtrgt, ix, itrgt) * coll[ll].volc[iwa] * w->ice[itrgt].numc * rhocoll * fix_coag;
        }
      }
    if (c->st_siprs)
      for (int ll = istr; ll <= iend; ll++) {
        const int ph = coll[ll].phase;
        if (ph != 2 && ph != 3) continue;
        if (coll[ll].dwet >= DLLIQ_RS && coll[ll].dwet < w->ice[itrgt].dnsp) {
          const int ix = ph == 3 ? ll : 0;
          w->mfrzn_rs[ix * c->nice + itrgt] +=
              KIDX(zcc, nbtrgt, ix, itrgt) * coll[ll].volc[iwa] * w->ice[itrgt].numc * rhocoll * fix_coag;
        }
      }
  }
}

/* :1385-1452 accumulateSourceIce.  zcc(nbcoll, nbtrgt): zcc(ll, itrgt). */
static void accumulateSourceIce(Cell *w, int nbtrgt, int nspec, int itrgt, int istr, int iend, const double *zcc,
                                const Section *coll, double *source) {
  const salsa_ref_ctx_t *c = w->c;
  const salsa_config_t *g = &c->cfg;
  double Eagg[MAXB];
  for (int ll = istr; ll <= iend; ll++) {
    double rimfr = fmaxd(getRimeFraction(c, &coll[ll]), getRimeFraction(c, &coll[itrgt]));
    Eagg[ll] = g->Eiagg_max - rimfr * (g->Eiagg_max - g->Eiagg_min);
  }
  for (int ll = istr; ll <= iend; ll++) {
    double k = KIDX(zcc, nbtrgt, ll, itrgt);
    for (int s = 0; s < nspec; s++) source[s] += Eagg[ll] * k * coll[ll].volc[s];
  }
  /* :1429-1447 ice-ice breakup: ice mass collected from the smaller bins; the target's
     diameters are updated first, for every smaller bin */
  if (c->st_secice && c->st_sipib)
    for (int ll = istr; ll <= iend; ll++) {
      updateDiameter(c, &w->ice[itrgt], 1, T_ALL);
      if (w->ice[itrgt].dnsp > coll[ll].dnsp && w->ice[itrgt].numc > w->ice[itrgt].nlim && coll[ll].numc > coll[ll].nlim)
        w->mii_ibr[itrgt * c->nice + ll] +=
            Eagg[ll] * KIDX(zcc, nbtrgt, itrgt, ll) *
            (coll[ll].volc[nspec - 2] * c->rhoic + coll[ll].volc[nspec - 1] * c->rhori) * coll[itrgt].numc;
    }
}

/* :1457-1584 accumulatePrecipFormation (cloud-cloud; zcc symmetric, (ncld,ncld)) */
static void accumulatePrecipFormation(Cell *w, int nspec, int itrgt, int istr, int iend, double fix_coag,
                                      const double *zcc, double *source, double *sink, double *volsink_slf,
                                      double *vol_prc, double *num_prc, double *INF_prc) {
  const salsa_ref_ctx_t *c = w->c;
  int ncld = c->ncld, nprc = c->nprc;
  Section *cl = w->cloud;
  int selfcoll = (itrgt == istr && itrgt == iend);
  for (int ll = istr; ll <= iend; ll++) {
    double D_new = pow(cube(cl[itrgt].dwet) + cube(cl[ll].dwet), 1. / 3.);
    int cnt = 0;
    for (int i = 0; i < nprc; i++) if (D_new > c->precpbins[i]) cnt++;
    int tp = cnt - 1;   /* 0-based trgt_prc */
    double dvol[NSP] = {0}, dnum = 0.;
    double kli = KIDX(zcc, ncld, ll, itrgt), kil = KIDX(zcc, ncld, itrgt, ll);
    if (D_new > c->precpbins[0]) {
      if (selfcoll) {
        for (int s = 0; s < nspec; s++) {
          dvol[s] = cl[ll].volc[s] * cl[itrgt].numc * kli * fix_coag;
          vol_prc[tp * NSP + s] += dvol[s];
        }
        dnum = (0.5 * kli * cl[ll].numc * cl[itrgt].numc) * fix_coag;
        num_prc[tp] += dnum;
        if (num_prc[tp] > 0.)
          INF_prc[tp] = (INF_prc[tp] * (num_prc[tp] - dnum) + cl[ll].INdef * dnum) / num_prc[tp];
      } else {
        for (int s = 0; s < nspec; s++) {
          dvol[s] = (cl[ll].volc[s] * cl[itrgt].numc + cl[itrgt].volc[s] * cl[ll].numc) * kli * fix_coag;
          vol_prc[tp * NSP + s] += dvol[s];
        }
        dnum = (kli * cl[ll].numc * cl[itrgt].numc) * fix_coag;
        num_prc[tp] += dnum;
        if (num_prc[tp] > 0.)
          INF_prc[tp] = (INF_prc[tp] * (num_prc[tp] - dnum) + 0.5 * (cl[ll].INdef + cl[itrgt].INdef) * dnum) /
                        num_prc[tp];
      }
      rate_acc_n(&w->rate[R_AUTOC], dnum); rate_acc_v(&w->rate[R_AUTOC], dvol, nspec);
      if (D_new > 50.e-6) { rate_acc_n(&w->rate[R_AUTOC50], dnum); rate_acc_v(&w->rate[R_AUTOC50], dvol, nspec); }
      if (D_new > 80.e-6) { rate_acc_n(&w->rate[R_AUTOC80], dnum); rate_acc_v(&w->rate[R_AUTOC80], dvol, nspec); }
      if (selfcoll) {
        for (int s = 0; s < nspec; s++) volsink_slf[s] += cl[ll].volc[s] * cl[itrgt].numc * kli * fix_coag;
        *sink += 0.5 * kli * cl[itrgt].numc;
      } else {
        *sink += kil * cl[ll].numc;
      }
    } else {
      if (selfcoll) {
        *sink += 0.5 * kil * cl[ll].numc;
      } else {
        for (int s = 0; s < nspec; s++) source[s] += kli * cl[ll].volc[s];
      }
    }
  }
}

/* :1588-1611 precipSelfCoag */
static void precipSelfCoag(Cell *w, int nspec, int ibin, const double *zcc, double *num_slf, double *vol_slf) {
  int nprc = w->c->nprc;
  Section *p = w->precp;
  double k = KIDX(zcc, nprc, ibin, ibin);
  for (int s = 0; s < nspec; s++) vol_slf[s] += p[ibin].volc[s] * p[ibin].numc * k;
  *num_slf += (0.5 * k * p[ibin].numc * p[ibin].numc);
}

/* :539-559 applyCoag */
static void applyCoag(int nspec, Section *t, double dt, const double *source, double sink, double sink_self) {
  for (int s = 0; s < nspec; s++) t->volc[s] = (t->volc[s] + dt * source[s] * t->numc) / (1. + dt * sink);
  t->numc = t->numc / (1. + dt * (sink + sink_self));
}

/* :563-601 applyCoagPrecp */
static void applyCoagPrecp(Cell *w, int nspec, int itrgt, double dt, const double *source, double sink,
                           double sink_self, double num_slf, const double *vol_slf) {
  Section *p = w->precp;
  int nb = w->c->nprc;
  for (int s = 0; s < nspec; s++)
    p[itrgt].volc[s] = (p[itrgt].volc[s] + dt * source[s] * p[itrgt].numc) / (1. + dt * sink);
  p[itrgt].numc = p[itrgt].numc / (1. + dt * (sink + sink_self));
  if (itrgt < nb - 1) {
    for (int s = 0; s < nspec; s++) p[itrgt + 1].volc[s] = p[itrgt + 1].volc[s] + dt * vol_slf[s];
    p[itrgt + 1].numc = p[itrgt + 1].numc + dt * num_slf;
    for (int s = 0; s < nspec; s++) p[itrgt].volc[s] = p[itrgt].volc[s] - dt * vol_slf[s];
    p[itrgt].numc = p[itrgt].numc - dt * num_slf;
  }
}

/* :605-651 applyCoagIce */
static void applyCoagIce(Cell *w, int iwa, int irim, int itrgt, double dt, const double *source, double sink,
                         double sink_self) {
  Section *t = &w->ice[itrgt];
  int ndry = w->c->ndry;
  for (int s = 0; s < ndry; s++) t->volc[s] = (t->volc[s] + dt * source[s] * t->numc) / (1. + dt * sink);
  t->volc[irim] = (t->volc[irim] + dt * source[irim] * t->numc) / (1. + dt * sink);
  t->volc[iwa] = (t->volc[iwa] + dt * source[iwa] * t->numc) / (1. + dt * sink);
  t->numc = t->numc / (1. + dt * (sink + sink_self));
  updateRhomean(w->c, t);
}

/* :654-702 applyCoagPrecipFormation */
static void applyCoagPrecipFormation(Cell *w, int nspec, int itrgt, double dt, const double *volsink_slf,
                                     const double *vol_prc, const double *num_prc, const double *INF_prc) {
  Section *cl = w->cloud, *p = w->precp;
  for (int s = 0; s < nspec; s++) cl[itrgt].volc[s] = cl[itrgt].volc[s] - dt * volsink_slf[s];
  for (int cc = 0; cc < w->c->nprc; cc++) {
    for (int s = 0; s < nspec; s++) p[cc].volc[s] = p[cc].volc[s] + dt * vol_prc[cc * NSP + s];
    double nrate = num_prc[cc];
    p[cc].numc = p[cc].numc + dt * nrate;
    if (p[cc].numc > p[cc].nlim)
      p[cc].INdef = (p[cc].INdef * (p[cc].numc - dt * nrate) + INF_prc[cc] * dt * nrate) / p[cc].numc;
  }
}

static int all_below(const Section *s) { return s->numc < s->nlim; }

/* :24-215 coag_aero */
static void coag_aero(Cell *w, int nspec, double dt) {
  const salsa_ref_ctx_t *c = w->c;
  const salsa_config_t *g = &c->cfg;
  Section *ae = w->aero;
  double plus[NSP], minus, mself;
  /* regime 1a */
  for (int kk = c->in1a; kk <= c->fn1a; kk++) {
    if (all_below(&ae[kk])) continue;
    int icla = c->ica_cur + (kk - c->ica_par > 0 ? kk - c->ica_par : 0);
    int iclb = c->icb_cur + (icla - c->ica_cur);
    memset(plus, 0, sizeof plus); minus = 0.; mself = 0.;
    if (g->lscgaa) {
      accumulateSink(w, c->nbins, kk, kk + 1, c->fn2b, w->zccaa, ae, &minus, 1, 1.0);
      accumulateSink(w, c->nbins, kk, kk, kk, w->zccaa, ae, &mself, 1, 0.5);
    }
    if (g->lscgca) {
      accumulateSink(w, c->ncld, kk, icla, c->fca_cur, w->zccca, w->cloud, &minus, 1, 1.0);
      accumulateSink(w, c->ncld, kk, iclb, c->fcb_cur, w->zccca, w->cloud, &minus, 1, 1.0);
    }
    if (g->lscgpa) accumulateSink(w, c->nprc, kk, 0, c->nprc - 1, w->zccpa, w->precp, &minus, 1, 1.0);
    if (g->lscgia) accumulateSink(w, c->nice, kk, 0, c->nice - 1, w->zccia, w->ice, &minus, 1, 1.0);
    if (g->lscgaa && kk > c->in1a)
      accumulateSource(w, c->nbins, nspec, kk, c->in1a, kk - 1, w->zccaa, ae, plus, 1);
    if (g->lscgca) {
      icla = c->ica_cur + (kk - c->ica_par) - 1;
      iclb = c->icb_cur + (icla - c->ica_cur);
      if (icla >= c->ica_cur) accumulateSourceReverse(c->ncld, nspec, kk, c->ica_cur, icla, w->zccca, w->cloud, plus);
      if (iclb >= c->icb_cur) accumulateSourceReverse(c->ncld, nspec, kk, c->icb_cur, iclb, w->zccca, w->cloud, plus);
    }
    applyCoag(nspec, &ae[kk], dt, plus, minus, mself);
  }
  /* regime 2a */
  for (int kk = c->in2a; kk <= c->fn2a; kk++) {
    if (all_below(&ae[kk])) continue;
    int index_b = c->in2b + (kk - c->in2a);
    int icla = c->ica_cur + (kk - c->ica_par > 0 ? kk - c->ica_par : 0);
    int iclb = c->icb_cur + (kk - c->ica_par > 0 ? kk - c->ica_par : 0);
    memset(plus, 0, sizeof plus); minus = 0.; mself = 0.;
    if (g->lscgaa) {
      if (kk < c->fn2a) {
        accumulateSink(w, c->nbins, kk, kk + 1, c->fn2a, w->zccaa, ae, &minus, 1, 1.0);
        accumulateSink(w, c->nbins, kk, index_b, c->fn2b, w->zccaa, ae, &minus, 1, 1.0);
      }
      accumulateSink(w, c->nbins, kk, kk, kk, w->zccaa, ae, &mself, 1, 0.5);
    }
    if (g->lscgca) {
      accumulateSink(w, c->ncld, kk, icla, c->fca_cur, w->zccca, w->cloud, &minus, 1, 1.0);
      accumulateSink(w, c->ncld, kk, iclb, c->fcb_cur, w->zccca, w->cloud, &minus, 1, 1.0);
    }
    if (g->lscgpa) accumulateSink(w, c->nprc, kk, 0, c->nprc - 1, w->zccpa, w->precp, &minus, 1, 1.0);
    if (g->lscgia) accumulateSink(w, c->nice, kk, 0, c->nice - 1, w->zccia, w->ice, &minus, 1, 1.0);
    if (g->lscgaa) {
      accumulateSource(w, c->nbins, nspec, kk, c->in1a, kk - 1, w->zccaa, ae, plus, 1);
      accumulateSource(w, c->nbins, nspec, kk, c->in2b, index_b, w->zccaa, ae, plus, 1);
    }
    if (g->lscgca) {
      icla = c->ica_cur + (kk - c->ica_par) - 1;
      iclb = c->icb_cur + (icla - c->ica_cur);
      if (icla >= c->ica_cur) accumulateSourceReverse(c->ncld, nspec, kk, c->ica_cur, icla, w->zccca, w->cloud, plus);
      if (iclb >= c->icb_cur) accumulateSourceReverse(c->ncld, nspec, kk, c->icb_cur, iclb, w->zccca, w->cloud, plus);
    }
    applyCoag(nspec, &ae[kk], dt, plus, minus, mself);
  }
  /* regime 2b */
  for (int kk = c->in2b; kk <= c->fn2b; kk++) {
    if (all_below(&ae[kk])) continue;
    int index_a = c->in2a + (kk - c->in2b);
    int icla = c->ica_cur + (kk - c->icb_par > 0 ? kk - c->icb_par : 0);
    int iclb = c->icb_cur + (kk - c->icb_par > 0 ? kk - c->icb_par : 0);
    memset(plus, 0, sizeof plus); minus = 0.; mself = 0.;
    if (g->lscgaa) {
      if (kk < c->fn2b) {
        accumulateSink(w, c->nbins, kk, kk + 1, c->fn2b, w->zccaa, ae, &minus, 1, 1.0);
        accumulateSink(w, c->nbins, kk, index_a, c->fn2a, w->zccaa, ae, &minus, 1, 1.0);
      }
      accumulateSink(w, c->nbins, kk, kk, kk, w->zccaa, ae, &mself, 1, 0.5);
    }
    if (g->lscgca) {
      accumulateSink(w, c->ncld, kk, icla, c->fca_cur, w->zccca, w->cloud, &minus, 1, 1.0);
      accumulateSink(w, c->ncld, kk, iclb, c->fcb_cur, w->zccca, w->cloud, &minus, 1, 1.0);
    }
    if (g->lscgpa) accumulateSink(w, c->nprc, kk, 0, c->nprc - 1, w->zccpa, w->precp, &minus, 1, 1.0);
    if (g->lscgia) accumulateSink(w, c->nice, kk, 0, c->nice - 1, w->zccia, w->ice, &minus, 1, 1.0);
    if (g->lscgaa) {
      accumulateSource(w, c->nbins, nspec, kk, c->in2b, kk - 1, w->zccaa, ae, plus, 1);
      accumulateSource(w, c->nbins, nspec, kk, c->in1a, index_a, w->zccaa, ae, plus, 1);
    }
    if (g->lscgca) {
      iclb = c->icb_cur + (kk - c->icb_par) - 1;
      icla = c->ica_cur + (iclb - c->icb_cur);
      if (icla >= c->ica_cur) accumulateSourceReverse(c->ncld, nspec, kk, c->ica_cur, icla, w->zccca, w->cloud, plus);
      if (iclb >= c->icb_cur) accumulateSourceReverse(c->ncld, nspec, kk, c->icb_cur, iclb, w->zccca, w->cloud, plus);
    }
    applyCoag(nspec, &ae[kk], dt, plus, minus, mself);
  }
}

/* :221-412 coag_cloud */
static void coag_cloud(Cell *w, int nspec, double dt) {
  const salsa_ref_ctx_t *c = w->c;
  const salsa_config_t *g = &c->cfg;
  Section *cl = w->cloud;
  int autoc1 = c->st_auto && g->lsauto.mode == 1;
  double plus[NSP], minus, mself, volsink_slf[NSP], vol_prc[MAXB * NSP], num_prc[MAXB], INF_prc[MAXB];
  for (int reg = 0; reg < 2; reg++) {
    int kfirst = reg == 0 ? c->ica_cur : c->icb_cur;
    int klast = reg == 0 ? c->fca_cur : c->fcb_cur;
    for (int kk = kfirst; kk <= klast; kk++) {
      if (all_below(&cl[kk])) continue;
      memset(plus, 0, sizeof plus); minus = 0.; mself = 0.;
      memset(volsink_slf, 0, sizeof volsink_slf); memset(vol_prc, 0, sizeof vol_prc);
      memset(num_prc, 0, sizeof num_prc); memset(INF_prc, 0, sizeof INF_prc);
      /* the parallel bin in the other regime */
      int other = reg == 0 ? c->icb_cur + (kk - c->ica_cur) : c->ica_cur + (kk - c->icb_cur);
      int rel = kk - kfirst;
      if (g->lscgca && kk < klast) {
        int iaa = c->ica_par + rel + 1, iab = c->icb_par + rel + 1;
        accumulateSinkReverse(c->ncld, kk, iaa, c->fn2a, w->zccca, w->aero, &minus);
        accumulateSinkReverse(c->ncld, kk, iab, c->fn2b, w->zccca, w->aero, &minus);
      }
      if (g->lscgcc) {
        if (kk < klast) {
          accumulateSink(w, c->ncld, kk, kk + 1, klast, w->zcccc, cl, &minus, 2, 1.0);
          accumulateSink(w, c->ncld, kk, other, reg == 0 ? c->fcb_cur : c->fca_cur, w->zcccc, cl, &minus, 2, 1.0);
        }
        if (autoc1) {
          double fix = fmaxd(1. - dt * (0.5 * KIDX(w->zcccc, c->ncld, kk, kk) * sq(cl[kk].numc) / (cl[kk].numc)), 0.1);
          accumulatePrecipFormation(w, nspec, kk, kk, kk, fix, w->zcccc, plus, &mself, volsink_slf, vol_prc, num_prc,
                                    INF_prc);
        } else {
          accumulateSink(w, c->ncld, kk, kk, kk, w->zcccc, cl, &mself, 2, 0.5);
        }
      }
      if (g->lscgpc) accumulateSink(w, c->nprc, kk, 0, c->nprc - 1, w->zccpc, w->precp, &minus, 2, 1.0);
      if (g->lscgic) accumulateSink(w, c->nice, kk, 0, c->nice - 1, w->zccic, w->ice, &minus, 2, 1.0);
      if (g->lscgca) {
        int iaa = c->ica_par + rel, iab = c->icb_par + rel;
        accumulateSource(w, c->ncld, nspec, kk, c->in1a, iaa, w->zccca, w->aero, plus, 2);
        accumulateSource(w, c->ncld, nspec, kk, c->in2b, iab, w->zccca, w->aero, plus, 2);
      }
      if (g->lscgcc && kk > kfirst) {
        /* regime a: own regime ica..kk-1 then regime b icb..index_b;
           regime b: own regime icb..kk-1 then regime a ica..index_a */
        int o_first = reg == 0 ? c->icb_cur : c->ica_cur;
        int o_last_full = reg == 0 ? c->fcb_cur : c->fca_cur;
        if (autoc1) {
          double s1 = 0.;
          for (int i = kfirst; i <= klast; i++) s1 += KIDX(w->zcccc, c->ncld, kk, i) * cl[i].numc;
          double fix = fmaxd(1. - dt * s1, 0.1);
          accumulatePrecipFormation(w, nspec, kk, kfirst, kk - 1, fix, w->zcccc, plus, &minus, volsink_slf, vol_prc,
                                    num_prc, INF_prc);
          double s2 = 0.;
          for (int i = o_first; i <= o_last_full; i++) s2 += KIDX(w->zcccc, c->ncld, kk, i) * cl[i].numc;
          fix = fmaxd(1. - dt * s2, 0.1);
          accumulatePrecipFormation(w, nspec, kk, o_first, other, fix, w->zcccc, plus, &minus, volsink_slf, vol_prc,
                                    num_prc, INF_prc);
        } else {
          accumulateSource(w, c->ncld, nspec, kk, kfirst, kk - 1, w->zcccc, cl, plus, 2);
          accumulateSource(w, c->ncld, nspec, kk, o_first, other, w->zcccc, cl, plus, 2);
        }
      }
      applyCoag(nspec, &cl[kk], dt, plus, minus, mself);
      if (autoc1) applyCoagPrecipFormation(w, nspec, kk, dt, volsink_slf, vol_prc, num_prc, INF_prc);
    }
  }
}

/* :418-470 coag_precp */
static void coag_precp(Cell *w, int nspec, double dt) {
  const salsa_ref_ctx_t *c = w->c;
  const salsa_config_t *g = &c->cfg;
  Section *p = w->precp;
  int nprc = c->nprc;
  double plus[NSP], minus, mself, num_slf, vol_slf[NSP];
  for (int kk = 0; kk < nprc; kk++) {
    if (all_below(&p[kk])) continue;
    memset(plus, 0, sizeof plus); minus = 0.; mself = 0.; num_slf = 0.; memset(vol_slf, 0, sizeof vol_slf);
    if (g->lscgpp) {
      if (kk < nprc - 1) {
        accumulateSink(w, nprc, kk, kk + 1, nprc - 1, w->zccpp, p, &minus, 3, 1.0);
        precipSelfCoag(w, nspec, kk, w->zccpp, &num_slf, vol_slf);
      } else {
        accumulateSink(w, nprc, kk, kk, kk, w->zccpp, p, &mself, 3, 0.5);
      }
    }
    if (g->lscgip) accumulateSink(w, c->nice, kk, 0, c->nice - 1, w->zccip, w->ice, &minus, 3, 1.0);
    if (g->lscgpa) accumulateSource(w, nprc, nspec, kk, c->in1a, c->fn2b, w->zccpa, w->aero, plus, 3);
    if (g->lscgpc) accumulateSource(w, nprc, nspec, kk, 0, c->ncld - 1, w->zccpc, w->cloud, plus, 3);
    if (g->lscgpp && kk > 0) accumulateSource(w, nprc, nspec, kk, 0, kk - 1, w->zccpp, p, plus, 3);
    applyCoagPrecp(w, nspec, kk, dt, plus, minus, mself, num_slf, vol_slf);
  }
}

/* :476-535 coag_ice */
static void coag_ice(Cell *w, int nspec, double dt) {
  const salsa_ref_ctx_t *c = w->c;
  const salsa_config_t *g = &c->cfg;
  Section *ic = w->ice;
  int nice = c->nice, iwa = c->iwa, irim = c->irim;
  double plus[NSP], minus, mself;
  for (int kk = 0; kk < nice; kk++) {
    if (all_below(&ic[kk])) continue;
    memset(plus, 0, sizeof plus); minus = 0.; mself = 0.;
    if (g->lscgii) {
      if (kk < nice - 1) accumulateSink(w, nice, kk, kk + 1, nice - 1, w->zccii, ic, &minus, 4, 1.0);
      accumulateSink(w, nice, kk, kk, kk, w->zccii, ic, &mself, 4, 0.5);
    }
    if (g->lscgia)
      accumulateSourcePhaseChange(w, nice, iwa, iwa, kk, c->in1a, c->fn2b, c->rhoic, c->rhowa, w->zccia, w->aero, plus);
    if (g->lscgic)
      accumulateSourcePhaseChange(w, nice, irim, iwa, kk, c->ica_cur, c->fcb_cur, c->rhori, c->rhowa, w->zccic,
                                  w->cloud, plus);
    if (g->lscgip)
      accumulateSourcePhaseChange(w, nice, irim, iwa, kk, 0, c->nprc - 1, c->rhori, c->rhowa, w->zccip, w->precp, plus);
    if (g->lscgii && kk > 0) accumulateSourceIce(w, nice, nspec, kk, 0, kk - 1, w->zccii, ic, plus);
    applyCoagIce(w, iwa, irim, kk, dt, plus, minus, mself);
  }
}

/* the ten kernel arrays of a cell in the storage of lscoag%mode = 2, in the order aa cc pp
   ii ca pa ia pc ic ip (store_coag / fetch_coag, mo_salsa_driver.f90:655-697) */
static long long kc_cell_doubles(const salsa_ref_ctx_t *c) {
  const long long a = c->nbins, k = c->ncld, p = c->nprc, i = c->nice;
  return a * a + k * k + p * p + i * i + a * k + a * p + a * i + k * p + k * i + p * i;
}
static void kc_copy(Cell *w, int store) {
  const salsa_ref_ctx_t *c = w->c;
  const int a = c->nbins, k = c->ncld, p = c->nprc, i = c->nice;
  double *arr[10] = {w->zccaa, w->zcccc, w->zccpp, w->zccii, w->zccca, w->zccpa, w->zccia, w->zccpc, w->zccic,
                     w->zccip};
  const int n[10] = {a * a, k * k, p * p, i * i, a * k, a * p, a * i, k * p, k * i, p * i};
  double *sto = c->kcache + w->cell * kc_cell_doubles(c);
  for (int q = 0; q < 10; q++) {
    if (store) memcpy(sto, arr[q], sizeof(double) * n[q]);
    else memcpy(arr[q], sto, sizeof(double) * n[q]);
    sto += n[q];
  }
}

/* Per-cell reset of the working state.  The kernel arrays are cleared over the bins
   of the layout only, as the reference's kernel arrays of those sizes are: clearing
   their full MAXB x MAXB extent would cost more than the rest of a cell's work. */
static void cell_clear(Cell *w, const salsa_ref_ctx_t *c) {
  memset(w, 0, offsetof(Cell, zccaa));
  memset(w->rate, 0, sizeof(Cell) - offsetof(Cell, rate));
  const int a = c->nbins, k = c->ncld, p = c->nprc, i = c->nice;
  double *arr[10] = {w->zccaa, w->zcccc, w->zccpp, w->zccii, w->zccca, w->zccpa, w->zccia, w->zccpc, w->zccic,
                     w->zccip};
  const int n[10] = {a * a, k * k, p * p, i * i, a * k, a * p, a * i, k * p, k * i, p * i};
  for (int q = 0; q < 10; q++) memset(arr[q], 0, sizeof(double) * n[q]);
  memset(w->nfrzn_rs, 0, sizeof(double) * p * i);
  memset(w->mfrzn_rs, 0, sizeof(double) * p * i);
  memset(w->nfrzn_df, 0, sizeof(double) * p * i);
  memset(w->mfrzn_df, 0, sizeof(double) * p * i);
  memset(w->nii_ibr, 0, sizeof(double) * i * i);
  memset(w->mii_ibr, 0, sizeof(double) * i * i);
}

/* mo_salsa_dynamics.f90:92-202 coagulation */
static void coagulation(Cell *w, double dt, double T, double P) {
  const salsa_ref_ctx_t *c = w->c;
  const salsa_config_t *g = &c->cfg;
  for (int bb = 0; bb < c->ntotal; bb++) updateDiameter(c, &w->all[bb], 1, T_ALL);
  if (g->lscoag.mode == 1 || c->lcgupdt) update_coagulation_kernels(w, P, T);
  else if (g->lscoag.mode == 2) kc_copy(w, 0);   /* fetch_coag (mo_salsa_driver.f90:297-298) */
  int any_aero = g->lscgaa || g->lscgca || g->lscgpa || g->lscgia;
  int any_cloud = g->lscgcc || g->lscgca || g->lscgpc || g->lscgic;
  int any_precp = g->lscgpp || g->lscgpa || g->lscgpc || g->lscgip;
  int any_ice = g->lscgii || g->lscgia || g->lscgic || g->lscgip;
  if (any_ice && T < 273.15) coag_ice(w, c->nused, dt);
  int nspec = c->nwet;
  if (any_precp) coag_precp(w, nspec, dt);
  if (any_aero) coag_aero(w, nspec, dt);
  if (any_cloud) coag_cloud(w, nspec, dt);
  for (int bb = 0; bb < c->ntotal; bb++) {
    if (w->all[bb].numc < -1.e-6) w->f_neg = 1;
    w->all[bb].numc = fmaxd(0., w->all[bb].numc);
    for (int s = 0; s < NSP; s++) w->all[bb].volc[s] = fmaxd(0., w->all[bb].volc[s]);
  }
}

/* ======================================================================
 * Water uptake: mo_salsa_properties.f90:73-380 equilibration
 * ====================================================================== */
static void equilibration(Cell *w, double prh, double ptemp, int init) {
  const salsa_ref_ctx_t *c = w->c;
  Section *ae = w->aero;
  double zvolc[MAXB][7];
  for (int kk = c->in1a; kk <= c->fn2b; kk++)
    for (int cc = 0; cc < 7; cc++) zvolc[kk][cc] = 0.;
  for (int cc = 0; cc < 5; cc++) {
    int dd = c->idx_name[cc];
    if (dd >= 0)
      for (int kk = c->in1a; kk <= c->fn2b; kk++) zvolc[kk][cc] = ae[kk].volc[dd];
  }
  double zvpart[7] = {0}, zbinmol[7];
  double zke, zaw, zlwc = 0., zdold, zrh, zcore = 0., zdwet = 0.;
  zke = 1.001;
  for (int kk = c->in1a; kk <= c->fn1a; kk++) {
    for (int i = 0; i < 7; i++) zbinmol[i] = 0.;
    zdold = 1.;
    if (ae[kk].numc > NLIM) {
      zvpart[0] = zvolc[kk][0] / ae[kk].numc;
      zvpart[1] = zvolc[kk][1] / ae[kk].numc;
      zvpart[5] = zvolc[kk][5] / ae[kk].numc;
      zvpart[6] = zvolc[kk][6] / ae[kk].numc;
      zcore = zvpart[0] + zvpart[1];
      zdwet = ae[kk].dwet;
      zrh = prh;
      zrh = fmaxd(zrh, 0.05);
      zrh = fmind(zrh, 0.98);
      int count = 0;
      while (fabs(zdwet / zdold - 1.) > 1.e-2) {
        zdold = fmaxd(zdwet, 1.e-20);
        zaw = zrh / zke;
        zbinmol[0] = +1.1065495e+2 - 3.6759197e+2 * zaw + 5.0462934e+2 * sq(zaw) - 3.1543839e+2 * cube(zaw) +
                     6.770824e+1 * sq(sq(zaw));
        zbinmol[1] = 1. / (zaw * c->mwa) - 1. / c->mwa;
        zbinmol[5] = +2.306844303e+1 - 3.563608869e+1 * zaw - 6.210577919e+1 * sq(zaw) + 5.510176187e+2 * cube(zaw) -
                     1.460055286e+3 * sq(sq(zaw)) + 1.894467542e+3 * sq(sq(zaw)) * zaw -
                     1.220611402e+3 * cube(sq(zaw)) + 3.098597737e+2 * cube(sq(zaw)) * zaw;
        zlwc = (zvolc[kk][0] * (c->rhosu / c->msu)) / zbinmol[0] +
               EPSOC * zvolc[kk][1] * (c->rhooc / c->moc) / zbinmol[1] +
               (zvolc[kk][5] * (c->rhono / c->mno)) / zbinmol[5];
        zdwet = pow(zlwc / ae[kk].numc / c->rhowa / PI6 + (zvpart[5] + zvpart[6]) / PI6 + zcore / PI6, 1. / 3.);
        zke = exp(2. * SURFW0 * MVWA / (BOLTZ * ptemp * zdwet));
        count++;
        w->cnt[3]++;
        if (count > 100) { w->f_equil = 1; break; }
      }
      ae[kk].volc[c->iwa] = zlwc / c->rhowa;
      if (init) { ae[kk].dwet = zdwet; ae[kk].core = zcore; }
    } else {
      if (init) { ae[kk].dwet = ae[kk].dmid; ae[kk].core = PI6 * cube(ae[kk].dmid); }
    }
  }
  if (init) {
    for (int kk = c->in2a; kk <= c->fn2b; kk++) {
      zke = 1.02;
      for (int i = 0; i < 7; i++) zbinmol[i] = 0.;
      zdold = 1.;
      if (ae[kk].numc > NLIM) {
        for (int i = 0; i < 7; i++) zvpart[i] = zvolc[kk][i] / ae[kk].numc;
        zcore = zvpart[0] + zvpart[1] + zvpart[2] + zvpart[3] + zvpart[4];
        zdwet = ae[kk].dwet;
        zrh = prh;
        zrh = fmaxd(zrh, 0.37);
        zrh = fmind(zrh, 0.98);
        int count = 0;
        while (fabs(zdwet / zdold - 1.) > 1.e-12) {
          zdold = fmaxd(zdwet, 1.e-20);
          zaw = zrh / zke;
          zbinmol[0] = +1.1065495e+2 - 3.6759197e+2 * zaw + 5.0462934e+2 * sq(zaw) - 3.1543839e+2 * cube(zaw) +
                       6.770824e+1 * sq(sq(zaw));
          zbinmol[1] = 1. / (zaw * c->mwa) - 1. / c->mwa;
          zbinmol[5] = +2.306844303e+1 - 3.563608869e+1 * zaw - 6.210577919e+1 * sq(zaw) +
                       5.510176187e+2 * cube(zaw) - 1.460055286e+3 * sq(sq(zaw)) +
                       1.894467542e+3 * sq(sq(zaw)) * zaw - 1.220611402e+3 * cube(sq(zaw)) +
                       3.098597737e+2 * cube(sq(zaw)) * zaw;
          zbinmol[4] = +5.875248e+1 - 1.8781997e+2 * zaw + 2.7211377e+2 * sq(zaw) - 1.8458287e+2 * cube(zaw) +
                       4.153689e+1 * sq(sq(zaw));
          zlwc = (zvolc[kk][0] * (c->rhosu / c->msu)) / zbinmol[0] +
                 EPSOC * (zvolc[kk][1] * (c->rhooc / c->moc)) / zbinmol[1] +
                 (zvolc[kk][5] * (c->rhono / c->mno)) / zbinmol[5] + (zvolc[kk][4] * (c->rhoss / c->mss)) / zbinmol[4];
          zdwet = pow(zlwc / ae[kk].numc / c->rhowa / PI6 + (zvpart[5] + zvpart[6]) / PI6 + zcore / PI6, 1. / 3.);
          zke = exp(2. * SURFW0 * MVWA / (BOLTZ * ptemp * zdwet));
          count++;
          w->cnt[3]++;
          if (count > 100) { w->f_equil = 1; break; }
        }
        ae[kk].volc[c->iwa] = zlwc / c->rhowa;
        ae[kk].dwet = zdwet;
        ae[kk].core = zcore;
      } else {
        ae[kk].dwet = ae[kk].dmid;
        ae[kk].core = PI6 * cube(ae[kk].dmid);
      }
    }
  }
}

/* ======================================================================
 * Condensation: mo_salsa_dynamics.f90
 * ====================================================================== */

/* :1127-1157 acth2o (+ per-cell kappa override: the solute moles are replaced by
 * kappa * V_soluble * rho_w / M_w, the kappa-Koehler form of the same ratio) */
static double acth2o(Cell *w, const Section *pp, int has_pcw, double pcw) {
  const salsa_ref_ctx_t *c = w->c;
  double zns = 0., znw;
  w->cnt[1]++;
  if (w->kappa) {
    double vs = 0.;
    for (int nn = 0; nn < c->ndry; nn++) if (c->diss[nn] > 0.) vs += pp->volc[nn];
    zns = w->kappa_cell * vs * c->rhowa / c->mwa;
  } else {
    for (int nn = 0; nn < c->ndry; nn++) zns = zns + c->diss[nn] * pp->volc[nn] * c->rholiq[nn] / c->MM[nn];
  }
  if (has_pcw) znw = pcw;
  else znw = pp->volc[c->iwa] * c->rholiq[c->iwa] / c->MM[c->iwa];
  return fmaxd(0.1, znw / fmaxd(EPSR, (znw + zns)));
}

static double zbeta_of(double zknud, double massacc) {
  return (zknud + 1.) / (0.377 * zknud + 1. + 4. / (3. * massacc) * (zknud + sq(zknud)));
}

/* :691-1125 gpparth2o */
static void gpparth2o(Cell *w, double ptemp, double ppres, double prs, double prsi, double *prv, double ptstep) {
  const salsa_ref_ctx_t *c = w->c;
  const salsa_config_t *g = &c->cfg;
  int nbins = c->nbins, ncld = c->ncld, nprc = c->nprc, nice = c->nice;
  Section *ae = w->aero, *cl = w->cloud, *pr = w->precp, *ic = w->ice;
  double zrh = *prv / prs;
  int iwa = c->iwa, irim = c->irim, nspec = c->nused;
  int nstr = c->in2a;
  double zaelwc1 = 0., zaelwc2 = 0.;
  for (int k = c->in1a; k <= c->fn2b; k++) zaelwc1 += ae[k].volc[iwa];
  zaelwc1 *= c->rhowa;
  equilibration(w, zrh, ptemp, 0);
  if (zrh < 0.98 || !g->lscndh2oae) equilibration(w, zrh, ptemp, 1);
  for (int k = c->in1a; k <= c->fn2b; k++) zaelwc2 += ae[k].volc[iwa];
  zaelwc2 *= c->rhowa;
  *prv = *prv - (zaelwc2 - zaelwc1) / (ppres * MAIR / (RG * ptemp));

  int anycl = 0, anypr = 0, anyic = 0, anyae = 0;
  for (int k = 0; k < ncld; k++) if (cl[k].numc > NLIM) anycl = 1;
  for (int k = 0; k < nprc; k++) if (pr[k].numc > PRLIM) anypr = 1;
  for (int k = 0; k < nice; k++) if (ic[k].numc > PRLIM) anyic = 1;
  for (int k = 0; k < nbins; k++) if (ae[k].numc > NLIM) anyae = 1;
  if (!((anycl || (anypr && g->lscndh2ocl)) || (anyic && g->lscndh2oic) || (anyae && zrh > 0.98 && g->lscndh2oae)))
    return;

  double rhoair = MAIR * ppres / (RG * ptemp);
  double zdfh2o = (5. / (16. * AVOG * rhoair * 1.e-3 * sq(3.11e-8))) *
                  sqrt(RG * 1.e7 * ptemp * MAIR * 1.e3 * (c->mwa + MAIR) * 1.e3 / (2. * PI * c->mwa * 1.e3));
  zdfh2o = zdfh2o * 1.e-4;
  double zmfph2o = 3. * zdfh2o * sqrt(PI * c->mwa / (8. * RG * ptemp));
  double zthcond = 0.023807 + 7.1128e-5 * (ptemp - 273.16);

  double zkelvin[MAXB], zkelvincd[MAXB], zkelvinpd[MAXB], zkelvinic[MAXB];
  double zcwsurfae[MAXB], zcwsurfcd[MAXB], zcwsurfpd[MAXB], zcwsurfic[MAXB];
  double zmtae[MAXB], zmtcd[MAXB], zmtpd[MAXB], zmtic[MAXB];
  double zwsatae[MAXB], zwsatcd[MAXB], zwsatpd[MAXB], zwsatic[MAXB];
  double zcwcae[MAXB], zcwccd[MAXB], zcwcpd[MAXB], zcwcit[MAXB];
  double zcwintae[MAXB], zcwintcd[MAXB], zcwintpd[MAXB], zcwintit[MAXB];
  double zorgic[MAXB], zorgri[MAXB];
  for (int k = 0; k < MAXB; k++) {
    zkelvin[k] = zkelvincd[k] = zkelvinpd[k] = zkelvinic[k] = 1.;
    zcwsurfae[k] = zcwsurfcd[k] = zcwsurfpd[k] = zcwsurfic[k] = 0.;
    zmtae[k] = zmtcd[k] = zmtpd[k] = zmtic[k] = 0.;
    zwsatae[k] = zwsatcd[k] = zwsatpd[k] = zwsatic[k] = 0.;
  }
  for (int cc = 0; cc < c->ntotal; cc++) { updateDiameter(c, &w->all[cc], 1, T_ALL); updateRhomean(c, &w->all[cc]); }

  for (int cc = 0; cc < ncld; cc++) {
    if (cl[cc].numc > cl[cc].nlim && g->lscndh2ocl) {
      double dwet = cl[cc].dwet;
      double zact = acth2o(w, &cl[cc], 0, 0.);
      zkelvincd[cc] = exp(4. * SURFW0 * c->mwa / (RG * ptemp * c->rhowa * dwet));
      zcwsurfcd[cc] = prs * rhoair / c->mwa;
      zwsatcd[cc] = zact * zkelvincd[cc];
      double zknud = 2. * zmfph2o / dwet;
      double zbeta = zbeta_of(zknud, 1.);
      double h1 = cl[cc].numc * 2. * PI * dwet * zdfh2o * zbeta;
      double h2 = c->mwa * zdfh2o * ALV * zwsatcd[cc] * zcwsurfcd[cc] / (zthcond * ptemp);
      double h3 = ((ALV * c->mwa) / (RG * ptemp)) - 1.;
      zmtcd[cc] = h1 / (h2 * h3 + 1.);
    }
  }
  for (int cc = 0; cc < nprc; cc++) {
    if (pr[cc].numc > pr[cc].nlim && g->lscndh2ocl) {
      double dwet = pr[cc].dwet;
      double zact = acth2o(w, &pr[cc], 0, 0.);
      zkelvinpd[cc] = exp(4. * SURFW0 * c->mwa / (RG * ptemp * c->rhowa * dwet));
      zcwsurfpd[cc] = prs * rhoair / c->mwa;
      zwsatpd[cc] = zact * zkelvinpd[cc];
      double zknud = 2. * zmfph2o / dwet;
      double zbeta = zbeta_of(zknud, 1.);
      double h1 = pr[cc].numc * 2. * PI * dwet * zdfh2o * zbeta;
      double h2 = c->mwa * zdfh2o * ALV * zwsatpd[cc] * zcwsurfpd[cc] / (zthcond * ptemp);
      double h3 = ((ALV * c->mwa) / (RG * ptemp)) - 1.;
      zmtpd[cc] = h1 / (h2 * h3 + 1.);
    }
  }
  for (int cc = 0; cc < nice; cc++) {
    if (ic[cc].numc > ic[cc].nlim && g->lscndh2oic && ptemp < 273.15) {
      double dwet = ic[cc].dnsp;
      double cap = 0.5 * dwet;
      double zact = 1.0;
      zkelvinic[cc] = exp(4. * SURFI0 * c->mwa / (RG * ptemp * c->rhowa * dwet));
      zcwsurfic[cc] = prsi * rhoair / c->mwa;
      zwsatic[cc] = zact * zkelvinic[cc];
      double zknud = 2. * zmfph2o / dwet;
      double zbeta = zbeta_of(zknud, 1.);
      double h1 = ic[cc].numc * 4. * PI * cap * zdfh2o * zbeta;
      double h2 = c->mwa * zdfh2o * ALS * zwsatic[cc] * zcwsurfic[cc] / (zthcond * ptemp);
      double h3 = ((ALS * c->mwa) / (RG * ptemp)) - 1.;
      zmtic[cc] = h1 / (h2 * h3 + 1.);
    }
  }
  for (int cc = 0; cc < nbins; cc++) {
    if (ae[cc].numc > ae[cc].nlim && zrh > 0.98 && g->lscndh2oae) {
      double dwet = ae[cc].dwet;
      double zact = acth2o(w, &ae[cc], 0, 0.);
      zkelvin[cc] = exp(4. * SURFW0 * c->mwa / (RG * ptemp * c->rhowa * dwet));
      zcwsurfae[cc] = prs * rhoair / c->mwa;
      zwsatae[cc] = zact * zkelvin[cc];
      double zknud = 2. * zmfph2o / dwet;
      double zbeta = zbeta_of(zknud, c->massacc[cc]);
      double h1 = ae[cc].numc * 2. * PI * dwet * zdfh2o * zbeta;
      double h2 = c->mwa * zdfh2o * ALV * zwsatae[cc] * zcwsurfae[cc] / (zthcond * ptemp);
      double h3 = ((ALV * c->mwa) / (RG * ptemp)) - 1.;
      zmtae[cc] = h1 / (h2 * h3 + 1.);
    }
  }
  double zcwc = *prv * rhoair / c->mwa;
  for (int k = 0; k < nbins; k++) zcwcae[k] = ae[k].volc[iwa] * c->rhowa / c->mwa;
  for (int k = 0; k < ncld; k++) zcwccd[k] = cl[k].volc[iwa] * c->rhowa / c->mwa;
  for (int k = 0; k < nprc; k++) zcwcpd[k] = pr[k].volc[iwa] * c->rhowa / c->mwa;
  for (int k = 0; k < nice; k++) {
    zcwcit[k] = ic[k].volc[iwa] * c->rhoic / c->mwa;
    zcwcit[k] = zcwcit[k] + ic[k].volc[irim] * c->rhori / c->mwa;
    zorgic[k] = ic[k].volc[iwa] * c->rhoic / c->mwa;
    zorgri[k] = ic[k].volc[irim] * c->rhori / c->mwa;
  }
  double sae = 0., scd = 0., spd = 0., sit = 0.;
  for (int k = 0; k < nbins; k++) sae += zcwcae[k];
  for (int k = 0; k < ncld; k++) scd += zcwccd[k];
  for (int k = 0; k < nprc; k++) spd += zcwcpd[k];
  for (int k = 0; k < nice; k++) sit += zcwcit[k];
  double zcwtot = zcwc + sae + scd + spd + sit;
  double ttot = 0.;
  for (int k = 0; k < nbins; k++) zcwintae[k] = zcwcae[k];
  for (int k = 0; k < ncld; k++) zcwintcd[k] = zcwccd[k];
  for (int k = 0; k < nprc; k++) zcwintpd[k] = zcwcpd[k];
  for (int k = 0; k < nice; k++) zcwintit[k] = zcwcit[k];

  int anyae_nl = 0, anycl_nl = 0, anypr_nl = 0, anyic_nl = 0;
  for (int k = 0; k < nbins; k++) if (ae[k].numc > ae[k].nlim) anyae_nl = 1;
  for (int k = 0; k < ncld; k++) if (cl[k].numc > cl[k].nlim) anycl_nl = 1;
  for (int k = 0; k < nprc; k++) if (pr[k].numc > pr[k].nlim) anypr_nl = 1;
  for (int k = 0; k < nice; k++) if (ic[k].numc > ic[k].nlim) anyic_nl = 1;

  double zcwint = 0.;
  int counter = 0;
  while (ttot < ptstep) {
    double adt = 2.e-2;
    double s1 = 0., s2 = 0., s3 = 0., s4 = 0.;
    for (int k = nstr; k < nbins; k++) s1 += zmtae[k] * zwsatae[k] * zcwsurfae[k];
    for (int k = 0; k < ncld; k++) s2 += zmtcd[k] * zwsatcd[k] * zcwsurfcd[k];
    for (int k = 0; k < nprc; k++) s3 += zmtpd[k] * zwsatpd[k] * zcwsurfpd[k];
    for (int k = 0; k < nice; k++) s4 += zmtic[k] * zwsatic[k] * zcwsurfic[k];
    double zhlp1 = zcwc + adt * (s1 + s2 + s3 + s4);
    double m1 = 0., m2 = 0., m3 = 0., m4 = 0.;
    for (int k = nstr; k < nbins; k++) m1 += zmtae[k];
    for (int k = 0; k < ncld; k++) m2 += zmtcd[k];
    for (int k = 0; k < nprc; k++) m3 += zmtpd[k];
    for (int k = 0; k < nice; k++) m4 += zmtic[k];
    double zhlp2 = 1. + adt * (m1 + m2 + m3 + m4);
    zcwint = zhlp1 / zhlp2;
    zcwint = fmind(zcwint, zcwtot);
    if (anyae_nl && zrh > 0.98) {
      for (int cc = nstr; cc < nbins; cc++) {
        zcwintae[cc] = zcwcae[cc] + fmind(fmaxd(adt * zmtae[cc] * (zcwint - zwsatae[cc] * zcwsurfae[cc]),
                                                -1.e-1 * zcwcae[cc]), 1.e-1 * zcwcae[cc]);
        zwsatae[cc] = acth2o(w, &ae[cc], 1, zcwintae[cc]) * zkelvin[cc];
      }
    }
    if (anycl_nl) {
      for (int cc = 0; cc < ncld; cc++) {
        zcwintcd[cc] = zcwccd[cc] + fmind(fmaxd(adt * zmtcd[cc] * (zcwint - zwsatcd[cc] * zcwsurfcd[cc]),
                                                -1.e-1 * zcwccd[cc]), 1.e-1 * zcwccd[cc]);
        zwsatcd[cc] = acth2o(w, &cl[cc], 1, zcwintcd[cc]) * zkelvincd[cc];
      }
    }
    if (anypr_nl) {
      for (int cc = 0; cc < nprc; cc++) {
        zcwintpd[cc] = zcwcpd[cc] + fmind(fmaxd(adt * zmtpd[cc] * (zcwint - zwsatpd[cc] * zcwsurfpd[cc]),
                                                -1.e-1 * zcwcpd[cc]), 1.e-1 * zcwcpd[cc]);
        zwsatpd[cc] = acth2o(w, &pr[cc], 1, zcwintpd[cc]) * zkelvinpd[cc];
      }
    }
    if (anyic_nl) {
      for (int cc = 0; cc < nice; cc++) {
        zcwintit[cc] = zcwcit[cc] + fmind(fmaxd(adt * zmtic[cc] * (zcwint - zwsatic[cc] * zcwsurfic[cc]),
                                                -1.e-1 * zcwcit[cc]), 1.e-1 * zcwcit[cc]);
        zwsatic[cc] = zkelvinic[cc];
      }
    }
    for (int k = nstr; k < nbins; k++) zcwintae[k] = fmaxd(zcwintae[k], 0.);
    for (int k = 0; k < ncld; k++) zcwintcd[k] = fmaxd(zcwintcd[k], 0.);
    for (int k = 0; k < nprc; k++) zcwintpd[k] = fmaxd(zcwintpd[k], 0.);
    for (int k = 0; k < nice; k++) zcwintit[k] = fmaxd(zcwintit[k], 0.);
    double t1 = 0., t2 = 0., t3 = 0., t4 = 0.;
    for (int k = 0; k < nbins; k++) t1 += zcwintae[k];
    for (int k = 0; k < ncld; k++) t2 += zcwintcd[k];
    for (int k = 0; k < nprc; k++) t3 += zcwintpd[k];
    for (int k = 0; k < nice; k++) t4 += zcwintit[k];
    zcwint = zcwtot - t1 - t2 - t3 - t4;
    for (int k = 0; k < nbins; k++) zcwcae[k] = zcwintae[k];
    for (int k = 0; k < ncld; k++) zcwccd[k] = zcwintcd[k];
    for (int k = 0; k < nprc; k++) zcwcpd[k] = zcwintpd[k];
    for (int k = 0; k < nice; k++) zcwcit[k] = zcwintit[k];
    zcwc = zcwint;
    ttot = ttot + adt;
    counter++;
    w->cnt[4]++;
    if (counter > 100) w->f_cond = 1;
  }
  double zcwn = zcwint;
  *prv = zcwn * c->mwa / rhoair;
  double vrate[NSP];
  memset(vrate, 0, sizeof vrate);
  for (int cc = 0; cc < nbins; cc++) {
    vrate[iwa] = fmaxd(0., zcwintae[cc] * c->mwa / c->rhowa) - ae[cc].volc[iwa];
    rate_acc_v(&w->rate[R_CONDA], vrate, nspec);
    ae[cc].volc[iwa] = fmaxd(0., zcwintae[cc] * c->mwa / c->rhowa);
  }
  memset(vrate, 0, sizeof vrate);
  for (int cc = 0; cc < ncld; cc++) {
    vrate[iwa] = fmaxd(0., zcwintcd[cc] * c->mwa / c->rhowa) - cl[cc].volc[iwa];
    rate_acc_v(&w->rate[R_CONDC], vrate, nspec);
    cl[cc].volc[iwa] = fmaxd(0., zcwintcd[cc] * c->mwa / c->rhowa);
  }
  memset(vrate, 0, sizeof vrate);
  for (int cc = 0; cc < nprc; cc++) {
    vrate[iwa] = fmaxd(0., zcwintpd[cc] * c->mwa / c->rhowa) - pr[cc].volc[iwa];
    rate_acc_v(&w->rate[R_CONDP], vrate, nspec);
    pr[cc].volc[iwa] = fmaxd(0., zcwintpd[cc] * c->mwa / c->rhowa);
  }
  memset(vrate, 0, sizeof vrate);
  for (int cc = 0; cc < nice; cc++) {
    double dvitot = zcwintit[cc] - (zorgic[cc] + zorgri[cc]);
    if (dvitot > 0.) {
      double dvice = dvitot;
      ic[cc].volc[iwa] = ic[cc].volc[iwa] + dvice * c->mwa / c->rhoic;
      vrate[iwa] = dvice * c->mwa / c->rhoic;
      rate_acc_v(&w->rate[R_CONDI], vrate, nspec);
    } else if (dvitot < 0.) {
      double dvice = (zcwintit[cc] / (zorgic[cc] + zorgri[cc])) - 1.;
      dvice = dvice * zorgic[cc];
      double dvrime = (zcwintit[cc] / (zorgic[cc] + zorgri[cc])) - 1.;
      dvrime = dvrime * zorgri[cc];
      vrate[iwa] = dvice * c->mwa / c->rhoic;
      vrate[irim] = dvrime * c->mwa / c->rhori;
      rate_acc_v(&w->rate[R_CONDI], vrate, nspec);
      ic[cc].volc[iwa] = ic[cc].volc[iwa] + dvice * c->mwa / c->rhoic;
      ic[cc].volc[irim] = ic[cc].volc[irim] + dvrime * c->mwa / c->rhori;
    }
  }
  for (int cc = 0; cc < c->ntotal; cc++)
    if (w->all[cc].numc > w->all[cc].nlim) updateRhomean(c, &w->all[cc]);
}

/* ======================================================================
 * Cloud activation and autoconversion: mo_salsa_cloud.f90
 * ====================================================================== */
static double intgN(double ikk, double icc, double ilow, double ihigh) {   /* :1381-1388 */
  return 0.5 * ikk * fmaxd(sq(ihigh) - sq(ilow), 0.) + icc * fmaxd(ihigh - ilow, 0.);
}
static double intgV(double ikk, double icc, double ilow, double ihigh) {   /* :1391-1398 */
  return (1. / 3.) * ikk * fmaxd(cube(ihigh) - cube(ilow), 0.) + 0.5 * icc * fmaxd(sq(ihigh) - sq(ilow), 0.);
}

/* :116-157 getSolute: moles of dissolved solute per particle of each aerosol bin */
static void getSolute(const Cell *w, double *pns) {
  const salsa_ref_ctx_t *c = w->c;
  for (int kk = 0; kk <= c->fn2b; kk++) {
    pns[kk] = 0.;
    const Section *a = &w->aero[kk];
    if (a->numc > a->nlim) {
      for (int nn = 0; nn < c->ndry; nn++) pns[kk] = pns[kk] + c->diss[nn] * a->volc[nn] * c->rholiq[nn] / c->MM[nn];
      pns[kk] = pns[kk] / a->numc;
    }
  }
}

/* :1199-1378 activate3: number and volume of the activated droplets of every cloud bin,
   from piecewise-linear number densities in dry volume integrated above the critical
   volume.  The state is not changed; only pactd (actd_n, actd_v) is. */
static void activate3(Cell *w, int bcrita, const double *pdcrit, const double *pdcrlo, const double *pdcrhi,
                      double pdcstar, double *actd_n, double *actd_v) {
  const salsa_ref_ctx_t *c = w->c;
  const Section *ae = w->aero;
  const int ndry = c->ndry, nwet = c->nwet, iwa = c->iwa;
  int all_small = 1;
  for (int k = 0; k <= c->fn2b; k++) if (!(pdcrit[k] < EPSR)) all_small = 0;
  if (all_small) return;
  double zvcstar = 0., Vmid, Vhi, Vlo, zhlp;
  const Section *bc = &ae[bcrita];
  if (bc->numc < bc->nlim) {
    Vmid = PI6 * cube(bc->dmid);
  } else {
    double sd = 0.;
    for (int i = 0; i < ndry; i++) sd += bc->volc[i];
    Vmid = sd / fmaxd(bc->nlim, bc->numc);
  }
  Vhi = bc->vhilim;
  Vlo = bc->vlolim;
  if (pdcstar >= pdcrit[bcrita]) {
    zhlp = (PI6 * cube(pdcstar) - PI6 * cube(pdcrit[bcrita])) /
           fmaxd(EPSR, PI6 * cube(pdcrhi[bcrita]) - PI6 * cube(pdcrit[bcrita]));
    zvcstar = Vmid + zhlp * (Vhi - Vmid);
  } else if (pdcstar < pdcrit[bcrita]) {
    zhlp = (PI6 * cube(pdcrit[bcrita]) - PI6 * cube(pdcstar)) /
           fmaxd(EPSR, PI6 * cube(pdcrit[bcrita]) - PI6 * cube(pdcrlo[bcrita]));
    zvcstar = Vmid - zhlp * (Vmid - Vlo);
  }
  zvcstar = fmaxd(zvcstar, bc->vlolim);
  zvcstar = fmind(zvcstar, bc->vhilim);
  for (int cb = c->ica_cur; cb <= c->fcb_cur; cb++) {
    const int ab = cb <= c->fca_cur ? c->ica_par + (cb - c->ica_cur) : c->icb_par + (cb - c->icb_cur);
    const Section *a = &ae[ab];
    if (a->numc < a->nlim) continue;
    double Nmid = fmaxd(a->numc, a->nlim), sd = 0.;
    for (int i = 0; i < ndry; i++) sd += a->volc[i];
    Vmid = sd / Nmid;
    Vlo = a->vlolim;
    Vhi = a->vhilim;
    double Nim1, Vim1, Vlom1, Vhim1, Nip1, Vip1, Vlop1, Vhip1;
    if (ab == c->in1a || ab == c->in2b) {
      Nim1 = a->nlim;
      Vim1 = Vlo / 2.;
      Vlom1 = 0.;
      Vhim1 = Vlo;
    } else {
      const Section *m = &ae[ab - 1];
      Nim1 = fmaxd(m->numc, m->nlim);
      if (Nim1 > m->nlim) {
        double v = 0.;
        for (int i = 0; i < ndry; i++) v += m->volc[i];
        Vim1 = v / Nim1;
      } else {
        Vim1 = PI6 * cube(m->dmid);
      }
      Vlom1 = m->vlolim;
      Vhim1 = m->vhilim;
    }
    if (ab == c->fn2a || ab == c->fn2b) {
      Nip1 = a->nlim;
      Vip1 = Vhi + 0.5 * (Vhi - Vlo);
      Vlop1 = Vhi;
      Vhip1 = Vhi + (Vhi - Vlo);
    } else {
      const Section *q = &ae[ab + 1];
      Nip1 = fmaxd(q->numc, q->nlim);
      if (Nip1 > q->nlim) {
        double v = 0.;
        for (int i = 0; i < ndry; i++) v += q->volc[i];
        Vip1 = v / Nip1;
      } else {
        Vip1 = PI6 * cube(q->dmid);
      }
      Vlop1 = q->vlolim;
      Vhip1 = q->vhilim;
    }
    Vip1 = fmaxd(Vlop1, fmind(Vip1, Vhip1));
    Vim1 = fmaxd(Vlom1, fmind(Vim1, Vhim1));
    const double dNim1 = Nim1 / (Vhim1 - Vlom1), dNip1 = Nip1 / (Vhip1 - Vlop1), dNmid = Nmid / (Vhi - Vlo);
    const double zs1 = (dNmid - dNim1) / (Vmid - Vim1), zs2 = (dNip1 - dNmid) / (Vip1 - Vmid);
    const double N01 = dNmid - zs1 * Vmid, N02 = dNip1 - zs2 * Vip1;
    const double Nnorm = intgN(zs1, N01, Vlo, Vmid) + intgN(zs2, N02, Vmid, Vhi);
    const double Vnorm = intgV(zs1, N01, Vlo, Vmid) + intgV(zs2, N02, Vmid, Vhi);
    double nact = 0., zactvol = 0.;
    int set = 0;
    if (zvcstar < Vmid) {
      const double zvcint = fmaxd(zvcstar, Vlo);
      nact = (Nmid / Nnorm) * (intgN(zs1, N01, zvcint, Vmid) + intgN(zs2, N02, Vmid, Vhi));
      zactvol = (Nmid * Vmid / Vnorm) * (intgV(zs1, N01, zvcint, Vmid) + intgV(zs2, N02, Vmid, Vhi));
      set = 1;
    } else if (zvcstar >= Vmid) {
      const double zvcint = fmind(zvcstar, Vhi);
      nact = (Nmid / Nnorm) * (intgN(zs2, N02, zvcint, Vhi));
      zactvol = (Nmid * Vmid / Vnorm) * (intgV(zs2, N02, zvcint, Vhi));
      set = 1;
    }
    double *av = actd_v + cb * NSP;
    if (set) {
      actd_n[cb] = nact;
      for (int ss = 0; ss < nwet; ss++) av[ss] = zactvol * (a->volc[ss] / (Vmid * Nmid));
    }
    actd_n[cb] = fmaxd(0., actd_n[cb]);
    for (int ss = 0; ss < nwet; ss++) av[ss] = fmaxd(0., av[ss]);
    av[iwa] = actd_n[cb] * PI6 * cube(pdcrit[ab]) * fmind(2., sq(3.e-6 / fmaxd(EPSR, pdcrit[ab])));
  }
}

/* :161-375 ActCloudBase (Abdul-Razzak & Ghan 2002, sectional form): maximum parcel
   supersaturation at cloud base from the updraft, critical diameters per bin, then
   activate3 */
static void ActCloudBase(Cell *w, double pres, double temp, double wvel, double *actd_n, double *actd_v) {
  const salsa_ref_ctx_t *c = w->c;
  const Section *ae = w->aero;
  const int in1a = c->in1a, fn2a = c->fn2a, in2b = c->in2b, fn2b = c->fn2b;
  const double mwa = c->mwa, rhowa = c->rhowa;
  const double bb = 6. * mwa / (PI * rhowa);
  double ns[MAXB], scrit[MAXB], frac[MAXB], zdcrit[MAXB], zdcrlo[MAXB], zdcrhi[MAXB];
  for (int k = 0; k < MAXB; k++) frac[k] = zdcrit[k] = zdcrlo[k] = zdcrhi[k] = 0.;
  int bcrita = fn2a, bcritb = fn2b;
  double zdcstar = 0.;
  getSolute(w, ns);
  if (wvel > 0.) {
    const double aa = 4. * mwa * SURFW0 / (RG * rhowa * temp);
    const double x = 4. * cube(aa) / (27. * bb);
    for (int k = in1a; k <= fn2b; k++) scrit[k] = exp(sqrt(x / fmaxd(EPSR, ns[k]))) - 1.;
    double ntot = 0., sum1 = 0.;
    for (int k = in1a; k <= fn2b; k++) ntot += ae[k].numc;
    for (int k = in1a; k <= fn2b; k++) sum1 += ae[k].numc / pow(scrit[k], 2. / 3.);
    if (!(ntot < ae[0].nlim)) {
      const double V = wvel;
      const double L = 2.501e6 - 2370. * (temp - 273.15);
      const double a1 = 1. - (373.15 / temp);
      const double ps = 101325. * exp(13.3185 * a1 - 1.976 * sq(a1) - 0.6445 * cube(a1) - 0.1299 * sq(sq(a1)));
      const double alpha = GRAV * mwa * L / (CPA * RG * sq(temp)) - GRAV * MAIR / (RG * temp);
      const double gamma = RG * temp / (ps * mwa) + mwa * sq(L) / (CPA * pres * MAIR * temp);
      const double x1 = pres / 101325.;
      const double dv1 = 1.e-4 * (0.211 / x1) * pow(temp / 273., 1.94);
      const double ka1 = 1.e-3 * (4.39 + 0.071 * temp);
      const double Gc = 1. / (rhowa * RG * temp / (ps * dv1 * mwa) + L * rhowa / (ka1 * temp) * (L * mwa / (temp * RG) - 1.));
      const double s_eff = sqrt(cube(ntot / sum1));
      const double theta = (sqrt(cube(alpha * V / Gc))) / (2. * PI * rhowa * gamma * ntot);
      const double khi = (2. / 3.) * aa * sqrt(alpha * V / Gc);
      const double s_max = s_eff / sqrt(0.5 * sqrt(cube(khi / theta)) + pow(sq(s_eff) / (theta + 3. * khi), 0.75));
      zdcstar = 2. * aa / (3. * s_max);
      for (int kk = in1a; kk <= fn2b; kk++) {
        if (ae[kk].numc < ae[kk].nlim) continue;
        const double nshi = ns[kk] * ae[kk].vratiohi;
        const double sil = exp(sqrt(x / nshi)) - 1.;
        if (s_max < sil) continue;
        const double nslo = ns[kk] * ae[kk].vratiolo;
        const double siu = exp(sqrt(x / nslo)) - 1.;
        frac[kk] = fmind(1., log(s_max / sil) / log(siu / sil));
        zdcrlo[kk] = 2. * sqrt(3. * nslo * bb / aa);
        zdcrhi[kk] = 2. * sqrt(3. * nshi * bb / aa);
        zdcrit[kk] = 2. * sqrt(3. * ns[kk] * bb / aa);
      }
      for (int kk = in1a; kk <= fn2a; kk++)
        if (frac[kk] < 1. && frac[kk] > 0.) { bcrita = kk; break; }
      for (int kk = in2b; kk <= fn2b; kk++)
        if (frac[kk] < 1. && frac[kk] > 0.) { bcritb = kk; break; }
    }
  }
  (void)bcritb;   /* computed by the reference, never read by activate3 */
  activate3(w, bcrita, zdcrit, zdcrlo, zdcrhi, zdcstar, actd_n, actd_v);
}

/* :859-1195 actInterst */
static void actInterst(Cell *w, double prv, double prs, double temp) {
  const salsa_ref_ctx_t *c = w->c;
  const double THvol = 1.e-28;
  int ndry = c->ndry, nwet = c->nwet, iwa = c->iwa;
  Section *ae = w->aero, *cl = w->cloud;
  if (prv / prs <= 1.000) return;
  double zkelvin = 4. * c->mwa * SURFW0 / (RG * c->rhowa * temp);
  double zdcstar = 2. * zkelvin / (3. * ((prv / prs) - 1.));
  double zvcstar = PI6 * cube(zdcstar);
  double act_n[MAXB], act_v[MAXB][NSP];
  for (int cb = c->ica_cur; cb <= c->fcb_cur; cb++) {
    int ab = (cb <= c->fca_cur) ? c->ica_par + (cb - c->ica_cur) : c->icb_par + (cb - c->icb_cur);
    act_n[cb] = 0.;
    for (int s = 0; s < NSP; s++) act_v[cb][s] = 0.;
    double vol_sol = 0., vol_insol = 0.;
    for (int i = 0; i < c->nsoluble; i++) vol_sol += ae[ab].volc[c->ind_soluble[i]];
    for (int i = 0; i < c->ninsoluble; i++) vol_insol += ae[ab].volc[c->ind_insoluble[i]];
    (void)vol_insol;
    if (ae[ab].numc < ae[ab].nlim) continue;
    if (vol_sol < ae[ab].numc * THvol) continue;
    if (ae[ab].volc[iwa] < ae[ab].numc * THvol) continue;
    int intr[4] = {0, 0, 0, 0};
    double Nmid = ae[ab].numc;
    double Vwmid = 0., Vmid = 0.;
    for (int s = 0; s < nwet; s++) Vwmid += ae[ab].volc[s];
    Vwmid /= Nmid;
    for (int s = 0; s < ndry; s++) Vmid += ae[ab].volc[s];
    Vmid /= Nmid;
    double Vlo = Vmid * ae[ab].vratiolo, Vhi = Vmid * ae[ab].vratiohi;
    double Nim1, Vim1, Vlom1, Vhim1, Vwim1, Nip1, Vip1, Vlop1, Vhip1, Vwip1;
    if (ab == c->in1a || ab == c->in2b) {
      Nim1 = ae[ab].nlim; Vim1 = Vlo / 2.; Vlom1 = 0.; Vhim1 = Vlo; Vwim1 = Vim1;
    } else {
      Nim1 = ae[ab - 1].numc;
      if (Nim1 > ae[ab - 1].nlim) {
        double vd = 0., vw = 0.;
        for (int s = 0; s < ndry; s++) vd += ae[ab - 1].volc[s];
        for (int s = 0; s < nwet; s++) vw += ae[ab - 1].volc[s];
        Vim1 = vd / Nim1; Vwim1 = vw / Nim1;
      } else {
        Vim1 = PI6 * cube(ae[ab - 1].dmid);
        Vwim1 = PI6 * cube(ae[ab - 1].dmid);
      }
      Vlom1 = Vim1 * ae[ab - 1].vratiolo;
      Vhim1 = Vim1 * ae[ab - 1].vratiohi;
    }
    if (ab == c->fn2a || ab == c->fn2b) {
      Nip1 = ae[ab].nlim; Vip1 = Vhi + 0.5 * (Vhi - Vlo); Vlop1 = Vhi; Vhip1 = Vhi + (Vhi - Vlo); Vwip1 = Vip1;
    } else {
      Nip1 = ae[ab + 1].numc;
      if (Nip1 > ae[ab + 1].nlim) {
        double vd = 0., vw = 0.;
        for (int s = 0; s < ndry; s++) vd += ae[ab + 1].volc[s];
        for (int s = 0; s < nwet; s++) vw += ae[ab + 1].volc[s];
        Vip1 = vd / Nip1; Vwip1 = vw / Nip1;
      } else {
        Vip1 = PI6 * cube(ae[ab + 1].dmid);
        Vwip1 = PI6 * cube(ae[ab + 1].dmid);
      }
      Vlop1 = Vip1 * ae[ab + 1].vratiolo;
      Vhip1 = Vip1 * ae[ab + 1].vratiohi;
    }
    Vip1 = fmaxd(Vhi, Vip1);
    Vim1 = fmind(Vlo, Vim1);
    double zs1 = (Vwmid - fmaxd(Vwim1, 0.)) / (Vmid - Vim1);
    double zs2 = (fmaxd(Vwip1, 0.) - Vwmid) / (Vip1 - Vmid);
    double V01 = Vwmid - zs1 * Vmid, V02 = Vwmid - zs2 * Vmid;
    double Vwlo = fmaxd(V01 + zs1 * Vlo, Vlo);
    double Vwhi = fmaxd(V02 + zs2 * Vhi, Vhi);
    double vint1, vint2, vcut;
    if (zvcstar < Vwlo && zvcstar < Vwmid && zvcstar < Vwhi) {
      vint1 = Vlo; vint2 = Vhi;
      intr[0] = intr[1] = intr[2] = intr[3] = 1;
    } else if (zvcstar > Vwlo && zvcstar > Vwmid && zvcstar > Vwhi) {
      vint1 = 999.; vint2 = 999.;
    } else {
      vcut = (zvcstar - V01) / zs1;
      if (vcut < Vlo || vcut > Vmid) vint1 = Vlo; else vint1 = vcut;
      vcut = (zvcstar - V02) / zs2;
      if (vcut < Vmid || vcut > Vhi) vint2 = Vmid; else vint2 = vcut;
      intr[0] = (Vwlo > zvcstar);
      intr[1] = (Vwmid > zvcstar);
      intr[2] = (Vwmid > zvcstar);
      intr[3] = (Vwhi > zvcstar);
    }
    double dNim1 = Nim1 / (Vhim1 - Vlom1);
    double dNip1 = Nip1 / (Vhip1 - Vlop1);
    double dNmid = Nmid / (Vhi - Vlo);
    zs1 = (dNmid - dNim1) / (Vmid - Vim1);
    zs2 = (dNip1 - dNmid) / (Vip1 - Vmid);
    double N01 = dNmid - zs1 * Vmid, N02 = dNmid - zs2 * Vmid;
    double Nnorm = intgN(zs1, N01, Vlo, Vmid) + intgN(zs2, N02, Vmid, Vhi);
    double Vnorm = intgV(zs1, N01, Vlo, Vmid) + intgV(zs2, N02, Vmid, Vhi);
    double zactvol = 0., Nact = 0.;
    if (intr[0]) { Nact += (Nmid / Nnorm) * intgN(zs1, N01, Vlo, vint1); zactvol += (Nmid * Vmid / Vnorm) * intgV(zs1, N01, Vlo, vint1); }
    if (intr[1]) { Nact += (Nmid / Nnorm) * intgN(zs1, N01, vint1, Vmid); zactvol += (Nmid * Vmid / Vnorm) * intgV(zs1, N01, vint1, Vmid); }
    if (intr[2]) { Nact += (Nmid / Nnorm) * intgN(zs2, N02, Vmid, vint2); zactvol += (Nmid * Vmid / Vnorm) * intgV(zs2, N02, Vmid, vint2); }
    if (intr[3]) { Nact += (Nmid / Nnorm) * intgN(zs2, N02, vint2, Vhi); zactvol += (Nmid * Vmid / Vnorm) * intgV(zs2, N02, vint2, Vhi); }
    double Vact[NSP];
    for (int ss = 0; ss < nwet; ss++) Vact[ss] = zactvol * (ae[ab].volc[ss] / (Vmid * Nmid));
    act_n[cb] = fmind(Nact, Nmid);
    for (int ss = 0; ss < nwet; ss++) act_v[cb][ss] = fmind(Vact[ss], ae[ab].volc[ss]);
    rate_acc_n(&w->rate[R_ACTIV], act_n[cb]);
    rate_acc_v(&w->rate[R_ACTIV], act_v[cb], nwet);
  }
  for (int cb = c->ica_cur; cb <= c->fcb_cur; cb++) {
    int ab = c->ica_par + (cb - c->ica_cur);   /* zaer => aero(ica%par:fcb%par), 1:1 */
    Section *za = &ae[ab], *zc = &cl[cb];
    if (act_n[cb] > 0.)
      zc->chargeTime = (act_n[cb] * za->chargeTimeMax + zc->numc * zc->chargeTime) / (act_n[cb] + zc->numc);
    za->numc = fmaxd(0., za->numc - act_n[cb]);
    zc->numc = zc->numc + act_n[cb];
    for (int ss = 0; ss < nwet; ss++) {
      za->volc[ss] = fmaxd(0., za->volc[ss] - act_v[cb][ss]);
      zc->volc[ss] = zc->volc[ss] + act_v[cb][ss];
    }
    if (zc->numc > 0.) zc->INdef = (zc->INdef * (zc->numc - act_n[cb]) + za->INdef * act_n[cb]) / zc->numc;
  }
}

/* math_functions.f90:543-555 cumlognorm */
static double cumlognorm(double dg, double sigmag, double dpart) {
  double hlp1 = (log(dpart) - log(dg));
  double hlp2 = sqrt(2.) * log(sigmag);
  return 0.5 + 0.5 * erf(hlp1 / hlp2);
}

/* mo_salsa_cloud.f90:1401-1477 autoconv2 */
static void autoconv2(Cell *w, double ptstep) {
  const salsa_ref_ctx_t *c = w->c;
  const double zd0 = 50.e-6, sigmag = 1.2, max_rate_autoc = 1.0e10;
  int nwet = c->nwet, ndry = c->ndry, iwa = c->iwa;
  Section *cl = w->cloud, *pr = w->precp;
  double tot = 0.;
  for (int cc = c->ncld - 1; cc >= 0; cc--) {
    tot = 0.;
    double Ntot = cl[cc].numc, Vtot = 0.;
    for (int s = 0; s < nwet; s++) Vtot += cl[cc].volc[s];
    if (Ntot > cl[cc].nlim && Vtot > 0.) {
      double dvg = pow(Vtot / Ntot / PI6, 1. / 3.) * exp((3. * sq(log(sigmag))) / 2.);
      double dg = dvg * exp(-3. * sq(log(sigmag)));
      double Vrem = Vtot * (1. - cumlognorm(dvg, sigmag, zd0));
      double Nrem = Ntot * (1. - cumlognorm(dg, sigmag, zd0));
      if (Vrem > 0. && Nrem > pr[0].nlim) {
        for (int ss = 0; ss < ndry; ss++) {
          pr[0].volc[ss] = pr[0].volc[ss] + cl[cc].volc[ss] * (Nrem / Ntot);
          cl[cc].volc[ss] = cl[cc].volc[ss] * (1. - (Nrem / Ntot));
        }
        pr[0].volc[iwa] = pr[0].volc[iwa] + cl[cc].volc[iwa] * (Vrem / Vtot);
        cl[cc].volc[iwa] = cl[cc].volc[iwa] * (1. - (Vrem / Vtot));
        pr[0].numc = pr[0].numc + Nrem;
        cl[cc].numc = cl[cc].numc - Nrem;
        tot = tot + Nrem;
        if (tot > max_rate_autoc * ptstep) break;
      }
    }
  }
}

/* ======================================================================
 * Ice nucleation (contact-angle distribution): mo_salsa_cloud_ice_SE.f90
 * ====================================================================== */

/* mo_particle_external_properties.f90:402-447 calcSweq (+ kappa override as in acth2o) */
static double calcSweq(Cell *w, const Section *part, double T) {
  const salsa_ref_ctx_t *c = w->c;
  int iwa = c->iwa, ndry = c->ndry;
  if (part->numc < part->nlim) return 0.;
  double v = 0.;
  for (int i = 0; i < NSP; i++) v += part->volc[i];
  double dwet = pow(v / part->numc / PI6, 1. / 3.);
  double znw = part->volc[iwa] * c->rhowa / c->mwa;
  double zvw = part->volc[iwa];
  double zns = 0., zvs = 0., zvtot = 0.;
  for (int i = 0; i < ndry; i++) {
    zns = zns + c->diss[i] * part->volc[i] * c->rholiq[i] / c->MM[i];
    zvs = zvs + fmind(1., c->diss[i]) * part->volc[i];
    zvtot = zvtot + part->volc[i];
  }
  if (w->kappa) {
    double vs = 0.;
    for (int i = 0; i < ndry; i++) if (c->diss[i] > 0.) vs += part->volc[i];
    zns = w->kappa_cell * vs * c->rhowa / c->mwa;
  }
  double kel = exp(4. * SURFW0 * c->mwa / (RG * T * c->rhowa * dwet));
  if (zvw > 1.e-28 * part->numc || zvs > 1.e-28 * part->numc) return (znw / (zns + znw)) * kel;
  else if (zvtot - zvs > 1.e-28 * part->numc) return kel;
  return (znw / (EPSR + zns + znw)) * kel;
}

/* single-function probe of calcSweq for the closed-form tests: the equilibrium
   saturation ratio of liquid bin b holding numc particles with the volume
   concentrations volc[0..nwet-1] (dry species, then water) at temperature T */
double salsa_ref_sweq(const salsa_ref_ctx_t *c, int b, double numc, const double *volc, double T) {
  Cell *w = (Cell *)malloc(sizeof(Cell));
  if (!w) return -1.;
  cell_clear(w, c);
  w->c = c;
  Section s = c->tmpl[b];
  s.numc = numc;
  for (int i = 0; i < NSP; i++) s.volc[i] = i < c->nwet ? volc[i] : 0.;
  const double r = calcSweq(w, &s, T);
  free(w);
  return r;
}

/* math_functions.f90:494-510 erfm1 */
static double erfm1(double x) {
  const double a = 0.140012;
  double sgn = 1.;
  if (x < 0.) sgn = -1.;
  double xx = fmaxd(1.e-20, 1. - sq(x));
  double t1 = log(xx);
  double t2 = 2. / (PI_FULL * a);
  double t3 = t2 + 0.5 * t1;
  double t4 = t1 / a;
  double t5 = t2 + 0.5 * t1;
  return sgn * sqrt(sqrt(sq(t3) - t4) - t5);
}

/* math_functions.f90:515-524 f_gauss */
static double f_gauss(double x, double sig, double mean) {
  double a = sqrt(2. * PI_FULL) * sig;
  double b = sq(x - mean);
  b = b / sq(sig);
  return (1. / a) * exp(-0.5 * b);
}

/* mo_salsa_cloud_ice_SE.f90:375-390 het_sf (also mo_salsa_cloud_ice.f90:293-308) */
static double het_sf(double x, double mis) {
  if (x > 100.) return (cube(mis) - 3. * mis + 2.) / 4.;
  double fii = sqrt(1. - 2. * mis * x + sq(x));
  double fpsi = (x - mis) / fii;
  return 0.5 * (1. + cube((1. - mis * x) / fii) + (2. - 3. * fpsi + cube(fpsi)) * cube(x) + 3. * mis * (fpsi - 1.) * sq(x));
}

/* :210-278 J_imm */
static double J_imm(const salsa_ref_ctx_t *c, double theta, double Tk, double Din, double Seq) {
  const double C = 1.7e10, rho_ice = 900., c_1s = 1.e19, T0 = 273.15, epsi = 0., alpha = 0.0;
  if (Din < 1e-10) return 0.;
  double Tc = Tk - T0;
  double act_energy = RG * Tk * (347. / (Tk - 177.) - log(4.14 / 349.)) / AVOG;
  double sigma_is = 28.e-3 + 0.25e-3 * Tc;
  double Lefm = (79.7 + 0.708 * Tc - 2.5e-3 * sq(Tc)) * 4.1868e3;
  double GG = RG * Tk / c->mwa / Lefm;
  if ((T0 / Tk) * pow(Seq, GG) < 1.0001) return 0.;
  double d_g = 4. * sigma_is / (rho_ice * Lefm * log((T0 / Tk) * pow(Seq, GG)) - C * sq(epsi));
  if (d_g <= 1e-10) return 0.;
  double thrad = theta * PI / 180.;
  double costh = cos(thrad);
  double sf = het_sf(Din / d_g, costh);
  double crit_energy = (PI / 3.) * sigma_is * sq(d_g) * sf - (1. / 4.) * alpha * (1. - costh) * sq(Din);
  return (BOLTZ * Tk / PLANCK) * c_1s * PI * sq(Din) * exp(-(act_energy + crit_energy) / (BOLTZ * Tk));
}

/* :282-331 J_dep */
static double J_dep(const salsa_ref_ctx_t *c, double theta, double Tk, double Din, double Seq) {
  const double C = 1.7e10, epsi = 0.;
  if (Din < 1e-10 || Seq < 1.0001) return 0.;
  double Tc = Tk - 273.15;
  double act_energy = 0.;
  double sigma_iv = ((76.1 - 0.155 * Tc) + (28.5 + 0.25 * Tc)) * 1.e-3;
  double d_g = 4. * sigma_iv / (RG * c->rhoic / c->mwa * Tk * log(Seq) - C * sq(epsi));
  if (d_g <= 1e-10) return 0.;
  double thrad = theta * PI / 180.;
  double costh = cos(thrad);
  double sf = het_sf(Din / d_g, costh);
  double crit_energy = (PI / 3.) * sigma_iv * sq(d_g) * sf;
  return (1. / 4.) * 1.e30 * sq(Din) * exp(-(act_energy + crit_energy) / (BOLTZ * Tk));
}

/* :335-371 J_hf */
static double J_hf(const salsa_ref_ctx_t *c, double Tk, double Sw) {
  const double Nc = 5.85e16, T0 = 273.15;
  double Tc = Tk - T0;
  double act_energy = 0.694e-19 * (1. + 0.027 * (Tc + 30.));
  double Lefm = (79.7 + 0.708 * Tc - 2.5e-3 * sq(Tc)) * 4.1868e3;
  double GG = RG * Tk / Lefm / c->mwa;
  if ((T0 / Tk) * pow(Sw, GG) < 1.0001) return 0.;
  double sigma_is = 28.e-3 + 0.25e-3 * Tc;
  double d_g = 4. * sigma_is / (c->rhoic * Lefm * log((T0 / Tk) * pow(Sw, GG)));
  if (d_g <= 1e-10) return 0.;
  double crit_energy = (PI / 3.) * sigma_is * sq(d_g);
  return 2.0 * Nc * (c->rhowa * BOLTZ * Tk / c->rhoic / PLANCK) * sqrt(sigma_is / BOLTZ / Tk) *
         exp(-(crit_energy + act_energy) / (BOLTZ * Tk));
}

/* single-function probe of the nucleation rates for the closed-form tests: kind 1 J_imm,
   2 J_dep (theta, Tk, Din, S), 3 J_hf (Tk, S) */
double salsa_ref_nucleation_rate(const salsa_ref_ctx_t *c, int kind, double theta, double Tk, double Din,
                                 double S) {
  if (kind == 1) return J_imm(c, theta, Tk, Din, S);
  if (kind == 2) return J_dep(c, theta, Tk, Din, S);
  if (kind == 3) return J_hf(c, Tk, S);
  return 0.;
}

static const double GL_X[10] = {-0.973908239224106, -0.865060566454542, -0.679410688379483, -0.433395397408358,
                                -0.148874339007507, 0.148874339007507,  0.433395397408358,  0.679410688379483,
                                0.865060566454542,  0.973908239224106};
static const double GL_W[10] = {0.066667031481273176, 0.14945422671662059, 0.21908574324601154, 0.26926671836765848,
                                0.29552422471242434,  0.29552422471242434, 0.26926671836765848, 0.21908574324601154,
                                0.14945422671662059,  0.066667031481273176};

/* :131-206 gauss_legendre */
static void gauss_legendre(Cell *w, double Tk, const double *Seq, const double *th00, double thm, double ths,
                           double tstep, const int *mask, int mode, double *frac) {
  const salsa_ref_ctx_t *c = w->c;
  double thmax = 180.;
  for (int kk = 0; kk < c->nliquid; kk++) {
    frac[kk] = 0.;
    if (!mask[kk] || Tk > 273.15 || w->liquid[kk].numc < w->liquid[kk].nlim) continue;
    double thmin = th00[kk];
    double dins = w->liquid[kk].ddry;
    for (int i = 0; i < 10; i++) {
      double th1 = 0.5 * (thmax - thmin) * GL_X[i] + 0.5 * (thmax + thmin);
      double J = 0.;
      if (mode == 1) J = J_imm(c, th1, Tk, dins, Seq[kk]);
      else if (mode == 2) J = J_dep(c, th1, Tk, dins, Seq[kk]);
      w->cnt[2]++;
      double ftheta = (th1 > thmin) ? f_gauss(th1, ths, thm) : 0.;
      frac[kk] = frac[kk] + ftheta * GL_W[i] * (1. - exp(-J * tstep));
    }
    frac[kk] = 0.5 * (thmax - thmin) * frac[kk];
  }
}

/* :394-417 low_theta */
static void low_theta(Cell *w, double *th00, double thmean, double thstd) {
  const salsa_ref_ctx_t *c = w->c;
  const double sqrt2 = sqrt(2.);
  for (int nb = 0; nb < c->nliquid; nb++) {
    double indef = w->liquid[nb].INdef;
    th00[nb] = thmean + sqrt2 * thstd * erfm1(2. * indef - 1.);
    th00[nb] = fmind(fmaxd(th00[nb], 0.), 180.);
    if (!c->st_freeTheta) th00[nb] = fmaxd(c->cfg.initMinTheta, th00[nb]);
  }
}

/* single-function probe of the contact-angle quadrature for the closed-form tests: the
   frozen fraction of one liquid bin (the cloud bins' first) with insoluble diameter dins,
   from gauss_legendre with mode 1 (immersion) or 2 (deposition) */
double salsa_ref_freezing_fraction(const salsa_ref_ctx_t *c, int mode, double Tk, double S, double th00, double thm,
                                   double ths, double dins, double tstep) {
  Cell *w = (Cell *)malloc(sizeof(Cell));
  if (!w) return -1.;
  cell_clear(w, c);
  w->c = c;
  memcpy(w->all, c->tmpl, sizeof(Section) * c->ntotal);
  w->liquid = &w->all[0];
  double Seq[MAXB], th[MAXB], frac[MAXB];
  int mask[MAXB];
  for (int k = 0; k < c->nliquid; k++) { Seq[k] = S; th[k] = th00; mask[k] = 0; frac[k] = 0.; }
  const int kk = c->nbins;   /* first cloud bin */
  w->liquid[kk].numc = 1.e6;
  w->liquid[kk].ddry = dins;
  mask[kk] = 1;
  gauss_legendre(w, Tk, Seq, th, thm, ths, tstep, mask, mode, frac);
  const double r = frac[kk];
  free(w);
  return r;
}

/* :542-555 getIceBin */
static int getIceBin(const Cell *w, double ldwet) {
  const salsa_ref_ctx_t *c = w->c;
  double vol = PI6 * cube(ldwet);
  vol = vol * c->rhowa / c->rhoic;
  int ii = 0;
  for (int k = 0; k < c->nice; k++) if (w->ice[k].vlolim < vol) ii++;
  if (ii < 1) ii = 1;
  if (ii > c->nice) ii = c->nice;
  return ii - 1;
}

/* :559-573 getPrecipBin */
static int getPrecipBin(const Cell *w, double idwet, double idens) {
  const salsa_ref_ctx_t *c = w->c;
  double vol = PI6 * cube(idwet);
  vol = vol * idens / c->rhowa;
  int ii = 0;
  for (int k = 0; k < c->nprc; k++) if (w->precp[k].vlolim < vol) ii++;
  if (ii < 1) ii = 1;
  if (ii > c->nprc) ii = c->nprc;
  return ii - 1;
}

/* :421-538 iceNucleation (SE variant) */
static void iceNucleation_SE(Cell *w, const double *frac) {
  const salsa_ref_ctx_t *c = w->c;
  const double minVin = PI6 * cube(1.e-8);
  int ndry = c->ndry, iwa = c->iwa, irim = c->irim, I_DU = c->idx_name[3];
  for (int kk = 0; kk < c->nliquid; kk++) {
    Section *L = &w->liquid[kk];
    if (L->numc < L->nlim) continue;
    double vins = 0.;
    for (int i = 0; i < c->ninsoluble; i++) vins += L->volc[c->ind_insoluble[i]];
    if (vins < minVin) continue;
    double dwet = L->dwet;
    int bb = getIceBin(w, dwet);
    Section *I = &w->ice[bb];
    double vdry = 0.;
    for (int s = 0; s < ndry; s++) vdry += L->volc[s];
    double V_tot = frac[kk] * vdry;
    double frac_DU = L->volc[I_DU] / vdry;
    double frac2, ncur0;
    if (frac_DU <= 0.1) { frac2 = frac[kk] * frac_DU; ncur0 = L->numc * frac_DU; }
    else { frac2 = frac[kk]; ncur0 = L->numc; }
    double nnuc_new = frac2 * L->numc;
    double f0 = L->INdef;
    double f1 = nnuc_new + (ncur0 - nnuc_new) * f0;
    f1 = f1 / ncur0;
    f1 = fmind(fmaxd(f1, 0.), 1. - 1.e-20);
    L->INdef = f1;
    if (frac_DU <= 0.1) {
      if (c->st_icenucl) I->volc[I_DU] = fmaxd(0., I->volc[I_DU] + V_tot * frac_DU);
      L->volc[I_DU] = fmaxd(0., L->volc[I_DU] - V_tot * frac_DU);
    } else {
      for (int ss = 0; ss < ndry; ss++) {
        if (c->st_icenucl) I->volc[ss] = fmaxd(0., I->volc[ss] + L->volc[ss] * frac2);
        L->volc[ss] = fmaxd(0., L->volc[ss] * (1. - frac2));
      }
    }
    if (L->phase == 1 || L->phase == 2) {
      if (c->st_icenucl) I->volc[iwa] = fmaxd(0., I->volc[iwa] + L->volc[iwa] * frac2 * c->rhowa / c->rhoic);
      L->volc[iwa] = fmaxd(0., L->volc[iwa] * (1. - frac2));
    } else if (L->phase == 3) {
      if (c->st_icenucl) I->volc[irim] = fmaxd(0., I->volc[irim] + L->volc[iwa] * frac2 * c->rhowa / c->rhori);
      L->volc[iwa] = fmaxd(0., L->volc[iwa] * (1. - frac2));
    }
    if (c->st_icenucl) I->numc = fmaxd(0., I->numc + L->numc * frac2);
    L->numc = fmaxd(0., L->numc * (1. - frac2));
  }
}

/* :28-127 ice_nucl_driver (SE) */
static void ice_nucl_SE(Cell *w, double ptemp, double prv, double prs, double prsi, double tstep) {
  const salsa_ref_ctx_t *c = w->c;
  const salsa_config_t *g = &c->cfg;
  const double dmin = 1.e-10, tmax_homog = 237.9;
  int nl = c->nliquid;
  if (c->ninsoluble <= 0) return;
  double f_dep[MAXB], f_imm[MAXB], f_hom[MAXB], Seq[MAXB], Si[MAXB], th00[MAXB], frac[MAXB];
  int mask[MAXB];
  for (int kk = 0; kk < nl; kk++) {
    f_dep[kk] = f_imm[kk] = f_hom[kk] = 0.;
    Seq[kk] = calcSweq(w, &w->liquid[kk], ptemp);
    Si[kk] = prv / prsi;
    updateDiameter(c, &w->liquid[kk], 1, T_ALL);
    double dwet = w->liquid[kk].dwet, dins = w->liquid[kk].ddry;
    if (dwet - dins > dmin && ptemp < tmax_homog && g->lsicehom) {
      double Jhom = J_hf(c, ptemp, Seq[kk]);
      f_hom[kk] = 1. - exp(-Jhom * PI6 * (cube(dwet) - cube(dins)) * tstep);
    }
  }
  if (g->lsiceimm) {
    low_theta(w, th00, g->mean_theta_imm, g->sigma_theta_imm);
    for (int kk = 0; kk < nl; kk++)
      mask[kk] = (w->liquid[kk].phase == 2 || w->liquid[kk].phase == 3) && (w->liquid[kk].dins > dmin);
    gauss_legendre(w, ptemp, Seq, th00, g->mean_theta_imm, g->sigma_theta_imm, tstep, mask, 1, f_imm);
  }
  if (g->lsicedep) {
    low_theta(w, th00, g->mean_theta_dep, g->sigma_theta_dep);
    for (int kk = 0; kk < nl; kk++)
      mask[kk] = (w->liquid[kk].phase == 1 && prv / prs < 1.0) && (w->liquid[kk].dwet - w->liquid[kk].dins < dmin) &&
                 (w->liquid[kk].dins > dmin);
    gauss_legendre(w, ptemp, Si, th00, g->mean_theta_dep, g->sigma_theta_dep, tstep, mask, 2, f_dep);
  }
  /* iceDiagnostics :577-594 */
  for (int kk = 0; kk < nl; kk++) {
    rate_acc_n(&w->rate[R_ICEHOM], w->liquid[kk].numc * f_hom[kk]);
    rate_acc_n(&w->rate[R_ICEDEP], w->liquid[kk].numc * f_dep[kk]);
    rate_acc_n(&w->rate[R_ICEIMM], w->liquid[kk].numc * f_imm[kk]);
  }
  for (int kk = 0; kk < nl; kk++)
    frac[kk] = fmaxd(0., fmind(0.99, f_imm[kk] + f_hom[kk] + f_dep[kk] - (f_imm[kk] + f_dep[kk]) * f_hom[kk]));
  iceNucleation_SE(w, frac);
}

/* ======================================================================
 * Classic ice nucleation and melting: mo_salsa_cloud_ice.f90
 * ====================================================================== */
static double calc_Jhet(const salsa_ref_ctx_t *c, double rn, double temp, double Sw) {   /* :146-207 */
  const double C = 1.7e10, rho_ice = 900., c_1s = 1e32, T0 = 273.15, epsi = 0., alpha = 0.0, mis = 0.5;
  if (rn < 1e-10) return 0.;
  double Tc = temp - T0;
  double act_energy = RG * temp * (347. / (temp - 177.) - log(4.14 / 349.)) / AVOG;
  double Lefm = (79.7 + 0.708 * Tc - 2.5e-3 * sq(Tc)) * 4.1868e3;
  double GG = RG * temp / c->mwa / Lefm;
  if ((T0 / temp) * pow(Sw, GG) < 1.0001) return 0.;
  double sigma_is = 28.e-3 + 0.25e-3 * Tc;
  double r_g = 4. * sigma_is / (rho_ice * Lefm * log((T0 / temp) * pow(Sw, GG)) - C * sq(epsi));
  if (r_g <= 1e-10) return 0.;
  double sf = het_sf(rn / r_g, mis);
  double crit_energy = (PI / 3.) * sigma_is * sq(r_g) * sf - (1. / 4.) * alpha * (1. - mis) * sq(rn);
  return BOLTZ * temp / PLANCK * c_1s * PI * sq(rn) * exp((-act_energy - crit_energy) / (BOLTZ * temp));
}
static double calc_Jdep(const salsa_ref_ctx_t *c, double rn, double temp, double Si) {   /* :210-255 */
  const double C = 1.7e10, rho_ice = 900., epsi = 0., mis = 0.5;
  if (rn < 1e-10 || Si < 1.0001) return 0.;
  double Tc = temp - 273.15;
  double act_energy = 0.;
  double sigma_iv = ((76.1 - 0.155 * Tc) + (28.5 + 0.25 * Tc)) * 1e-3;
  double r_g = 4. * sigma_iv / (RG * rho_ice / c->mwa * temp * log(Si) - C * sq(epsi));
  if (r_g <= 1e-10) return 0.;
  double sf = het_sf(rn / r_g, mis);
  double crit_energy = (PI / 3.) * sigma_iv * sq(r_g) * sf;
  return (1. / 4.) * 1.e30 * sq(rn) * exp((-act_energy - crit_energy) / (BOLTZ * temp));
}
static double calc_Jhf(const salsa_ref_ctx_t *c, double temp, double Sw) {   /* :257-291 */
  const double Nc = 5.85e16, rho_ice = 900., T0 = 273.15;
  double Tc = temp - T0;
  double act_energy = 0.694e-19 * (1. + 0.027 * (Tc + 30.));
  double Lefm = (79.7 + 0.708 * Tc - 2.5e-3 * sq(Tc)) * 4.1868e3;
  double GG = RG * temp / Lefm / c->mwa;
  if ((T0 / temp) * pow(Sw, GG) < 1.0001) return 0.;
  double sigma_is = 28.e-3 + 0.25e-3 * Tc;
  double r_g = 2. * sigma_is / (rho_ice * Lefm * log((T0 / temp) * pow(Sw, GG)));
  if (r_g <= 1e-10) return 0.;
  double crit_energy = 4. * PI / 3. * sigma_is * sq(r_g);
  return 2.0 * Nc * (c->rhowa * BOLTZ * temp / rho_ice / PLANCK) * sqrt(sigma_is / BOLTZ / temp) *
         exp((-crit_energy - act_energy) / (BOLTZ * temp));
}

/* :498-531 iceNucleation (classic) */
static void iceNucleation_classic(Cell *w, int iice, Section *L, double frac) {
  const salsa_ref_ctx_t *c = w->c;
  Section *I = &w->ice[iice];
  int ndry = c->ndry, iwa = c->iwa, irim = c->irim;
  for (int ss = 0; ss < ndry; ss++) {
    if (c->st_icenucl) I->volc[ss] = fmaxd(0., I->volc[ss] + L->volc[ss] * frac);
    L->volc[ss] = fmaxd(0., L->volc[ss] * (1. - frac));
  }
  if (L->phase == 1 || L->phase == 2) {
    if (c->st_icenucl) I->volc[iwa] = fmaxd(0., I->volc[iwa] + L->volc[iwa] * frac * c->rhowa / c->rhoic);
    L->volc[iwa] = fmaxd(0., L->volc[iwa] * (1. - frac));
  } else if (L->phase == 3) {
    if (c->st_icenucl) I->volc[irim] = fmaxd(0., I->volc[irim] + L->volc[iwa] * frac * c->rhowa / c->rhori);
    L->volc[iwa] = fmaxd(0., L->volc[iwa] * (1. - frac));
  }
  if (c->st_icenucl) I->numc = fmaxd(0., I->numc + L->numc * frac);
  L->numc = fmaxd(0., L->numc * (1. - frac));
}

/* :26-140 ice_nucl_driver (classic) */
static void ice_nucl_classic(Cell *w, double ptemp, double prv, double prs, double prsi, double ptstep) {
  const salsa_ref_ctx_t *c = w->c;
  const salsa_config_t *g = &c->cfg;
  const double tmax_homog = 237.9, dmin = 1.e-10;
  for (int kk = 0; kk < c->nliquid; kk++) {
    Section *L = &w->liquid[kk];
    if (ptemp > 273.15) continue;
    if (L->numc < L->nlim) continue;
    int phase = L->phase;
    updateDiameter(c, L, 1, T_ALL);
    double dins = L->dins, dwet = L->dwet;
    double Sw_eq = calcSweq(w, L, ptemp);
    double pf_imm = 0., pf_dep = 0., pf_hom = 0.;
    if (dins > dmin && g->lsiceimm && (phase == 2 || phase == 3)) {
      double jf = calc_Jhet(c, dins, ptemp, Sw_eq);
      pf_imm = 1. - exp(-jf * ptstep);
    }
    if (dins > dmin && dwet - dins < dmin && prv / prs < 1.0 && phase == 1 && g->lsicedep) {
      double Si = prv / prsi;
      double jf = calc_Jdep(c, dins, ptemp, Si);
      pf_dep = 1. - exp(-jf * ptstep);
    }
    if (dwet - dins > dmin && ptemp < tmax_homog && g->lsicehom) {
      double jf = calc_Jhf(c, ptemp, Sw_eq);
      pf_hom = 1. - exp(-jf * PI6 * (cube(dwet) - cube(dins)) * ptstep);
    }
    double frac = fmaxd(0., fmind(0.99, pf_imm + pf_hom + pf_dep - (pf_imm + pf_dep) * pf_hom));
    int bb = getIceBin(w, dwet);
    iceNucleation_classic(w, bb, L, frac);
    rate_acc_n(&w->rate[R_ICEHOM], L->numc * pf_hom);
    rate_acc_n(&w->rate[R_ICEDEP], L->numc * pf_dep);
    rate_acc_n(&w->rate[R_ICEIMM], L->numc * pf_imm);
    updateRhomean(c, &w->ice[bb]);
  }
}

/* :393-462 ice_melt */
static void ice_melt(Cell *w, double ptemp) {
  const salsa_ref_ctx_t *c = w->c;
  const double maxfrac = 0.999;
  int ndry = c->ndry, iwa = c->iwa, irim = c->irim;
  if (ptemp < 273.15) return;
  for (int kk = 0; kk < c->nice; kk++) {
    Section *I = &w->ice[kk];
    if (I->numc < I->nlim) continue;
    updateDiameter(c, I, 1, T_WET);
    double dwet = I->dwet;
    updateRhomean(c, I);
    double rhomean = I->rhomean;
    int bb = getPrecipBin(w, dwet, rhomean);
    Section *P = &w->precp[bb];
    for (int ss = 0; ss < ndry; ss++) {
      P->volc[ss] = P->volc[ss] + maxfrac * I->volc[ss];
      I->volc[ss] = (1. - maxfrac) * I->volc[ss];
    }
    double liqvol = (I->volc[iwa] * c->rhoic + I->volc[irim] * c->rhori) / c->rhowa;
    P->numc = P->numc + maxfrac * I->numc;
    I->numc = (1. - maxfrac) * I->numc;
    P->volc[iwa] = P->volc[iwa] + maxfrac * liqvol;
    I->volc[iwa] = (1. - maxfrac) * I->volc[iwa];
    I->volc[irim] = (1. - maxfrac) * I->volc[irim];
    for (int k = 0; k < 3; k++) I->sip[k] = (1. - maxfrac) * I->sip[k];   /* :453-456 */
  }
}

/* ======================================================================
 * Bin redistribution: mo_salsa_update.f90:21-433 distr_update
 * ====================================================================== */
static void distr_update(Cell *w, int level) {
  const salsa_ref_ctx_t *c = w->c;
  int zndry = c->ndry, znwet = c->nwet, znnsp = c->nused;
  Section *ae = w->aero, *cl = w->cloud, *pr = w->precp, *ic = w->ice;
  double zvpart, znfrac, zvfrac, zVrat, zVilo, zVihi, zVexc, zvdec;
  int within_bins, count, mm;
  /* aerosols */
  within_bins = 0; count = 0;
  while (!within_bins) {
    within_bins = 1;
    for (int kk = c->fn2b - 1; kk >= c->in1a; kk--) {
      mm = 0;
      if (ae[kk].numc > NLIM) {
        if (kk == c->fn2a) continue;
        double sd = 0.;
        for (int s = 0; s < zndry; s++) sd += ae[kk].volc[s];
        zvpart = sd / ae[kk].numc;
        if (ae[kk].vlolim > zvpart && kk == c->in1a) continue;
        if (ae[kk].vlolim > zvpart) {
          mm = kk - 1;
          if (kk == c->in2b) mm = c->fn1a;
          ae[mm].numc = ae[mm].numc + ae[kk].numc;
          ae[kk].numc = 0.;
          for (int s = 0; s < znwet; s++) { ae[mm].volc[s] = ae[mm].volc[s] + ae[kk].volc[s]; ae[kk].volc[s] = 0.; }
          continue;
        }
        if (zvpart <= PI6 * cube(ae[kk].dmid)) continue;
        zVrat = ae[kk].vhilim / ae[kk].vlolim;
        zVilo = 2. * zvpart / (1. + zVrat);
        zVihi = zVrat * zVilo;
        zVexc = 0.5 * (zVihi + ae[kk].vhilim);
        znfrac = fmind(1., (zVihi - ae[kk].vhilim) / (zVihi - zVilo));
        zvfrac = fmind(0.99, znfrac * zVexc / zvpart);
        if (zvfrac < 0.) w->f_negfrac = 1;
        mm = kk + 1;
        double sdry = 0.;
        for (int s = 0; s < zndry; s++) sdry += ae[kk].volc[s];
        double vold[NSP];
        for (int s = 0; s < znwet; s++) vold[s] = ae[kk].volc[s];
        for (int s = 0; s < znwet; s++)
          ae[mm].volc[s] = ae[mm].volc[s] + znfrac * ae[kk].numc * zVexc * vold[s] / sdry;
        for (int s = 0; s < znwet; s++)
          ae[kk].volc[s] = ae[kk].volc[s] - znfrac * ae[kk].numc * zVexc * vold[s] / sdry;
        ae[mm].numc = ae[mm].numc + znfrac * ae[kk].numc;
        ae[kk].numc = ae[kk].numc * (1. - znfrac);
      }
      if (ae[kk].numc > NLIM) {
        double sd = 0.;
        for (int s = 0; s < zndry; s++) sd += ae[kk].volc[s];
        zvpart = sd / ae[kk].numc;
        within_bins = (ae[kk].vlolim < zvpart && zvpart < ae[kk].vhilim);
      }
    }
    count++;
    if (count > 100) { w->f_distr = 1; break; }
  }
  /* cloud droplets */
  within_bins = 0; count = 0;
  while (!within_bins) {
    within_bins = 1;
    for (int kk = c->ncld - 1; kk >= c->ica_cur; kk--) {
      mm = 0;
      double sd = 0.;
      for (int s = 0; s < zndry; s++) sd += cl[kk].volc[s];
      if (cl[kk].numc > NLIM && sd > 1.e-30) {
        zvpart = sd / cl[kk].numc;
        zVrat = cl[kk].vhilim / cl[kk].vlolim;
        zVilo = 2. * zvpart / (1. + zVrat);
        zVihi = zVrat * zVilo;
        if (zvpart < cl[kk].vlolim && (kk != c->ica_cur && kk != c->icb_cur)) {
          zVexc = 0.5 * (zVilo + cl[kk].vlolim);
          znfrac = fmind(1., (cl[kk].vlolim - zVilo) / (zVihi - zVilo));
          mm = kk - 1;
        } else if (zvpart > cl[kk].vhilim && (kk != c->fca_cur && kk != c->fcb_cur)) {
          zVexc = 0.5 * (zVihi + cl[kk].vhilim);
          znfrac = fmind(1., (zVihi - cl[kk].vhilim) / (zVihi - zVilo));
          mm = kk + 1;
        } else {
          continue;
        }
        zvfrac = fmind(0.99, znfrac * zVexc / zvpart);
        if (zvfrac < 0.) w->f_negfrac = 1;
        for (int s = 0; s < znwet; s++) {
          cl[mm].volc[s] = cl[mm].volc[s] + zvfrac * cl[kk].volc[s];
          cl[kk].volc[s] = cl[kk].volc[s] - zvfrac * cl[kk].volc[s];
        }
        cl[mm].numc = cl[mm].numc + znfrac * cl[kk].numc;
        cl[kk].numc = cl[kk].numc - znfrac * cl[kk].numc;
      }
      sd = 0.;
      for (int s = 0; s < zndry; s++) sd += cl[kk].volc[s];
      if (cl[kk].numc > NLIM && sd > 1.e-30) {
        zvpart = sd / cl[kk].numc;
        within_bins = (cl[kk].vlolim < zvpart && zvpart < cl[kk].vhilim);
      }
    }
    count++;
    if (count > 100) { w->f_distr = 1; break; }
  }
  /* rain drops */
  within_bins = 0; count = 0;
  while (!within_bins) {
    within_bins = 1;
    for (int kk = c->nprc - 1; kk >= 0; kk--) {
      mm = 0;
      if (pr[kk].numc > PRLIM) {
        double sw = 0.;
        for (int s = 0; s < znwet; s++) sw += pr[kk].volc[s];
        zvpart = sw / pr[kk].numc;
        zVrat = pr[kk].vhilim / pr[kk].vlolim;
        zVilo = 2. * zvpart / (1. + zVrat);
        zVihi = zVrat * zVilo;
        zvdec = (PI6 * cube(pr[kk].dmid)) - 0.2 * ((PI6 * cube(pr[kk].dmid)) - pr[kk].vlolim);
        if (zvpart < zvdec && kk != 0) {
          zVexc = 0.5 * (zVilo + pr[kk].vlolim);
          znfrac = fmind(1., (pr[kk].vlolim - zVilo) / (zVihi - zVilo));
          mm = kk - 1;
        } else if (zvpart > PI6 * cube(pr[kk].dmid) && kk != c->nprc - 1) {
          zVexc = 0.5 * (zVihi + pr[kk].vhilim);
          znfrac = fmind(.99, (zVihi - pr[kk].vhilim) / (zVihi - zVilo));
          mm = kk + 1;
        } else {
          continue;
        }
        zvfrac = fmind(0.99, znfrac * zVexc / zvpart);
        if (zvfrac < 0.) w->f_negfrac = 1;
        for (int s = 0; s < znwet; s++) {
          pr[mm].volc[s] = pr[mm].volc[s] + zvfrac * pr[kk].volc[s];
          pr[kk].volc[s] = pr[kk].volc[s] - zvfrac * pr[kk].volc[s];
        }
        pr[mm].numc = pr[mm].numc + znfrac * pr[kk].numc;
        pr[kk].numc = pr[kk].numc - znfrac * pr[kk].numc;
      }
      if (pr[kk].numc > PRLIM) {
        double sw = 0.;
        for (int s = 0; s < znwet; s++) sw += pr[kk].volc[s];
        zvpart = sw / pr[kk].numc;
        within_bins = (pr[kk].vlolim < zvpart && zvpart < pr[kk].vhilim);
      }
    }
    count++;
    if (count > 100) { w->f_distr = 1; break; }
  }
  if (level < 5) return;
  /* ice */
  within_bins = 0; count = 0;
  while (!within_bins) {
    within_bins = 1;
    for (int kk = c->nice - 1; kk >= 0; kk--) {
      mm = 0;
      if (ic[kk].numc > ic[kk].nlim) {
        double st = 0.;
        for (int s = 0; s < znnsp; s++) st += ic[kk].volc[s];
        zvpart = st / ic[kk].numc;
        zVrat = ic[kk].vhilim / ic[kk].vlolim;
        zVilo = 2. * zvpart / (1. + zVrat);
        zVihi = zVrat * zVilo;
        zvdec = (PI6 * cube(ic[kk].dmid)) - 0.2 * ((PI6 * cube(ic[kk].dmid)) - ic[kk].vlolim);
        if (zvpart < zvdec && kk != 0) {
          zVexc = 0.5 * (zVilo + ic[kk].vlolim);
          znfrac = fmind(1.0, (ic[kk].vlolim - zVilo) / (zVihi - zVilo));
          mm = kk - 1;
        } else if (zvpart > PI6 * cube(ic[kk].dmid) && kk != c->nice - 1) {
          zVexc = 0.5 * (zVihi + ic[kk].vhilim);
          znfrac = fmind(0.99, (zVihi - ic[kk].vhilim) / (zVihi - zVilo));
          mm = kk + 1;
        } else {
          continue;
        }
        zvfrac = fmind(0.99, znfrac * zVexc / zvpart);
        if (zvfrac < 0.) w->f_negfrac = 1;
        for (int s = 0; s < znnsp; s++) {
          ic[mm].volc[s] = ic[mm].volc[s] + zvfrac * ic[kk].volc[s];
          ic[kk].volc[s] = ic[kk].volc[s] - zvfrac * ic[kk].volc[s];
        }
        ic[mm].numc = ic[mm].numc + znfrac * ic[kk].numc;
        ic[kk].numc = ic[kk].numc - znfrac * ic[kk].numc;
      }
      double st = 0.;
      for (int s = 0; s < znnsp; s++) st += ic[kk].volc[s];
      if (ic[kk].numc > ic[kk].nlim && st > 1.e-30) {
        zvpart = st / ic[kk].numc;
        within_bins = (ic[kk].vlolim < zvpart && zvpart < ic[kk].vhilim);
      }
    }
    count++;
    if (count > 100) { w->f_distr = 1; break; }
  }
}

/* ======================================================================
 * mo_salsa_dynamics.f90:348-685 condgas: H2SO4 and organic vapours onto every bin
 * (Fuchs-Sutugin collision rates, implicit gas-phase update).  The nucleation terms of
 * the smallest bin (Jacobson 16.73, 16.75) read condgas's own zj3n3 and zxocnv, which
 * it declares locally and zeroes (:433-444), so they vanish whatever nucleation
 * computed; zxsa (the H2SO4 fraction of the 3 nm clusters) only multiplies such a zero.
 * ====================================================================== */
static void condgas(Cell *w, double *pcsa, double *pcocnv, double *pcocsv, double zxsa, double ptemp, double ppres,
                    double ptstep) {
  const salsa_ref_ctx_t *c = w->c;
  Section *ae = w->aero, *cl = w->cloud, *pr = w->precp, *ic = w->ice;
  const int in1a = c->in1a, in2a = c->in2a, fn2b = c->fn2b, ncld = c->ncld, nprc = c->nprc, nice = c->nice;
  const int ioc = c->idx_name[1], iso4 = c->idx_name[0];
  const double zj3n3[2] = {0., 0.}, zxocnv = 0.;
  double zdvolsa[MAXB], zdvoloc[MAXB], zn_vs_c = 0.;
  for (int k = 0; k < MAXB; k++) zdvolsa[k] = zdvoloc[k] = 0.;
  for (int bb = 0; bb < c->ntotal; bb++) updateDiameter(c, &w->all[bb], 1, T_WET);
  /* 1) air and vapour properties */
  const double zvisc = (7.44523e-3 * sqrt(cube(ptemp))) / (5093. * (ptemp + 110.4));
  const double zdfvap = 5.1111e-10 * pow(ptemp, 1.75) * PSTAND / ppres;
  const double zmfp = 3. * zdfvap * sqrt(PI * c->msu / (8. * RG * ptemp));
  /* 2) Knudsen numbers and transition-regime corrections; 3) collision rates */
  double zknud[MAXB], zbeta[MAXB], zcolrate[MAXB], zcolrateca[MAXB], zcolratepa[MAXB], zcolrateia[MAXB];
  for (int k = in1a; k <= fn2b; k++) {
    zknud[k] = k <= in1a + 1 ? 2. * zmfp / (ae[k].dwet + D_SA) : 2. * zmfp / ae[k].dwet;
    zbeta[k] = (zknud[k] + 1.) / (0.377 * zknud[k] + 1. + 4. / (3. * c->massacc[k]) * (zknud[k] + sq(zknud[k])));
  }
  for (int k = in1a; k <= fn2b; k++) {
    zcolrate[k] = 0.;
    if (k <= in1a + 1) {
      const double zdfpart = BOLTZ * ptemp * zbeta[k] / (3. * PI * zvisc * ae[k].dwet);
      if (ae[k].numc > NLIM) zcolrate[k] = 2. * PI * (ae[k].dwet + D_SA) * (zdfvap + zdfpart) * zbeta[k] * ae[k].numc;
    } else if (ae[k].numc > NLIM) {
      zcolrate[k] = 2. * PI * ae[k].dwet * zdfvap * zbeta[k] * ae[k].numc;
    }
  }
  /* hydrometeors: beta = 1 / (1 + Kn (1.33 + 0.71/Kn) / (1 + 1/Kn)) */
  Section *hs[3] = {cl, pr, ic};
  double *hr[3] = {zcolrateca, zcolratepa, zcolrateia};
  const int hn[3] = {ncld, nprc, nice};
  const double hl[3] = {NLIM, PRLIM, PRLIM};
  for (int h = 0; h < 3; h++)
    for (int k = 0; k < hn[h]; k++) {
      const double kn = 2. * zmfp / hs[h][k].dwet;
      double b = 1. + kn * (1.33 + (0.71 / kn)) / (1. + (1. / kn));
      b = 1. / b;
      hr[h][k] = hs[h][k].numc > hl[h] ? 2. * PI * hs[h][k].dwet * zdfvap * b * hs[h][k].numc : 0.;
    }
  /* 4) condensation sink (Fortran SUM: in order) */
  double sa = 0., sca = 0., spa = 0., sia = 0., sa2 = 0.;
  for (int k = in1a; k <= fn2b; k++) sa += zcolrate[k];
  for (int k = 0; k < ncld; k++) sca += zcolrateca[k];
  for (int k = 0; k < nprc; k++) spa += zcolratepa[k];
  for (int k = 0; k < nice; k++) sia += zcolrateia[k];
  for (int k = in2a; k <= fn2b; k++) sa2 += zcolrate[k];
  const double zcs_tot = sa + sca + spa + sia;
  /* 5.1.1) non-volatile organics onto every bin */
  if (*pcocnv > 1.e-10 && zcs_tot > 1.e-30 && ioc >= 0) {
    zn_vs_c = 0.;
    if (zj3n3[1] > 1.) zn_vs_c = zj3n3[1] / (zj3n3[1] + *pcocnv * zcolrate[in1a]);
    double zcolrate_ocnv[MAXB];
    for (int k = in1a; k <= fn2b; k++) zcolrate_ocnv[k] = zcolrate[k];
    zcolrate_ocnv[in1a] = zcolrate_ocnv[in1a] + zj3n3[1] / *pcocnv;
    const double zcs_ocnv = zcs_tot + zj3n3[1] / *pcocnv;
    const double zcvap_new2 = *pcocnv / (1. + ptstep * zcs_ocnv);
    const double zdvap2 = *pcocnv - zcvap_new2;
    *pcocnv = zcvap_new2;
    for (int k = in1a; k <= fn2b; k++) zdvoloc[k] = zcolrate_ocnv[k] / zcs_ocnv * MVOC * zdvap2;
    for (int k = in1a; k <= fn2b; k++) ae[k].volc[ioc] = ae[k].volc[ioc] + zdvoloc[k];
    for (int k = 0; k < ncld; k++) cl[k].volc[ioc] = cl[k].volc[ioc] + zcolrateca[k] / zcs_ocnv * MVOC * zdvap2;
    for (int k = 0; k < nprc; k++) pr[k].volc[ioc] = pr[k].volc[ioc] + zcolratepa[k] / zcs_ocnv * MVOC * zdvap2;
    for (int k = 0; k < nice; k++) ic[k].volc[ioc] = ic[k].volc[ioc] + zcolrateia[k] / zcs_ocnv * MVOC * zdvap2;
    if (zxocnv > 0.) ae[in1a].numc = ae[in1a].numc + zn_vs_c * zdvoloc[in1a] / MVOC / (N3 * zxocnv);
  }
  /* 5.1.2) semi-volatile organics onto regimes 2a/2b and the hydrometeors.  The aerosol
     update adds all of zdvoloc, which still holds the non-volatile increments of 5.1.1. */
  const double zcs_ocsv = sa2 + sca + spa + sia;
  if (*pcocsv > 1.e-10 && zcs_ocsv > 1.e-30 && ioc >= 0) {
    const double zcvap_new3 = *pcocsv / (1. + ptstep * zcs_ocsv);
    const double zdvap3 = *pcocsv - zcvap_new3;
    *pcocsv = zcvap_new3;
    for (int k = in2a; k <= fn2b; k++) zdvoloc[k] = zdvoloc[k] + zcolrate[k] / zcs_ocsv * MVOC * zdvap3;
    for (int k = in1a; k <= fn2b; k++) ae[k].volc[ioc] = ae[k].volc[ioc] + zdvoloc[k];
    for (int k = 0; k < ncld; k++) cl[k].volc[ioc] = cl[k].volc[ioc] + zcolrateca[k] / zcs_ocsv * MVOC * zdvap3;
    for (int k = 0; k < nprc; k++) pr[k].volc[ioc] = pr[k].volc[ioc] + zcolratepa[k] / zcs_ocsv * MVOC * zdvap3;
    for (int k = 0; k < nice; k++) ic[k].volc[ioc] = ic[k].volc[ioc] + zcolrateia[k] / zcs_ocsv * MVOC * zdvap3;
  }
  /* 5.2) sulphuric acid onto every bin */
  if (*pcsa > 1.e-10 && zcs_tot > 1.e-30 && iso4 >= 0) {
    zn_vs_c = 0.;
    if (zj3n3[0] > 1.) zn_vs_c = zj3n3[0] / (zj3n3[0] + *pcsa * zcolrate[in1a]);
    zcolrate[in1a] = zcolrate[in1a] + zj3n3[0] / *pcsa;
    const double zcs_su = zcs_tot + zj3n3[0] / *pcsa;
    const double zcvap_new1 = *pcsa / (1. + ptstep * zcs_su);
    const double zdvap1 = *pcsa - zcvap_new1;
    *pcsa = zcvap_new1;
    for (int k = in1a; k <= fn2b; k++) zdvolsa[k] = zcolrate[k] / zcs_su * MVSU * zdvap1;
    for (int k = in1a; k <= fn2b; k++) ae[k].volc[iso4] = ae[k].volc[iso4] + zdvolsa[k];
    for (int k = 0; k < ncld; k++) cl[k].volc[iso4] = cl[k].volc[iso4] + zcolrateca[k] / zcs_su * MVSU * zdvap1;
    for (int k = 0; k < nprc; k++) pr[k].volc[iso4] = pr[k].volc[iso4] + zcolratepa[k] / zcs_su * MVSU * zdvap1;
    for (int k = 0; k < nice; k++) ic[k].volc[iso4] = ic[k].volc[iso4] + zcolrateia[k] / zcs_su * MVSU * zdvap1;
    if (zxsa > 0.) ae[in1a].numc = ae[in1a].numc + zn_vs_c * zdvolsa[in1a] / MVSU / (N3 * zxsa);
  }
}

/* ======================================================================
 * Secondary ice: mo_salsa_secondary_ice.f90:6-40 -> rime splintering,
 * mo_salsa_SIP_RS.f90:28-215 (Hallett and Mossop 1974; Mossop 1976)
 * ====================================================================== */
/* :247-270 rs_halletmossop (splinters per kg of rime) and :276-299 rs_mossop (per frozen
   drop), with dltemp_rs = 5: no temperature dependence */
static double rs_splinters(int mode, double mfrzn, double nfrzn) {
  return mode == 1 ? 3.5E8 * mfrzn : 4.0E-3 * nfrzn;
}

static void rimesplintering(Cell *w, double ptemp, double ptstep) {
  const salsa_ref_ctx_t *c = w->c;
  const int nprc = c->nprc, nice = c->nice, nspec = c->nused, mode = c->cfg.lssiprimespln.mode;
  const double tmin = 238.15, tmax = 273.15;
  const double v_i = 3.405365461487051e-16;   /* a 10 um hexagonal column of bulk ice */
  Section *ice = w->ice;
  int splbin = 0;                             /* :72, 1-based */
  for (int bb = 0; bb < nice; bb++) splbin += c->icebins[bb] < DSPLINT;
  if (splbin < 1) splbin = 1;
  for (int e = 0; e < nprc * nice; e++) {
    w->mfrzn_rs[e] = w->mfrzn_rs[e] * ptstep;
    w->nfrzn_rs[e] = w->nfrzn_rs[e] * ptstep;
  }
  double fragvolc[MAXB][NSP], sinkvolc[MAXB][NSP], fragnumc[MAXB], sinknumc[MAXB], sinkv[NSP];
  memset(fragvolc, 0, sizeof fragvolc); memset(sinkvolc, 0, sizeof sinkvolc);
  memset(fragnumc, 0, sizeof fragnumc); memset(sinknumc, 0, sizeof sinknumc);
  for (int bb = 0; bb < nice; bb++) {
    double vall = 0.;
    for (int s = 0; s < NSP; s++) vall += ice[bb].volc[s];
    for (int cc = 0; cc < nprc; cc++) {
      const double nf = w->nfrzn_rs[cc * nice + bb], mf = w->mfrzn_rs[cc * nice + bb];
      if (ptemp < tmin || ptemp > tmax || nf < 1.e-12 || vall < 1.e-15 || ice[bb].numc < ice[bb].nlim ||
          bb + 1 < splbin + 2)
        continue;
      const double ddmean = pow(mf / nf / c->rhowa / PI6, 1. / 3.);
      if (ddmean < DLLIQ_RS) continue;
      const double dN = rs_splinters(mode, mf, nf);
      const double dV = dN * v_i;
      fragnumc[splbin - 1] = fragnumc[splbin - 1] + dN;
      double sv = 0.;
      for (int s = 0; s < nspec; s++) sv += ice[bb].volc[s];
      for (int s = 0; s < nspec; s++)
        fragvolc[splbin - 1][s] = fragvolc[splbin - 1][s] + ice[bb].volc[s] * fmind(dV / sv, 1.);
      for (int s = 0; s < nspec; s++) sinkv[s] = ice[bb].volc[s] * fmind(dV / sv, 1.0);
      for (int s = 0; s < nspec; s++) sinkvolc[bb][s] = sinkvolc[bb][s] + sinkv[s];
      double ss = 0.;
      for (int s = 0; s < nspec; s++) ss += sinkv[s];
      sinknumc[bb] = sinknumc[bb] + ss / (PI6 * pow(ddmean, 3.0));
      ice[splbin - 1].sip[1] = ice[splbin - 1].sip[1] + dN;   /* :134-136 */
      rate_acc_n(&w->rate[R_SIPRMSPL], dN / ptstep);
    }
    if (ice[bb].numc < sinknumc[bb]) {                       /* :152-158 */
      sinknumc[bb] = ice[bb].numc;
      for (int s = 0; s < nspec; s++) sinkvolc[bb][s] = ice[bb].volc[s];
    }
    double ssk = 0., sv = 0.;                                /* :160-168: the fragments keep their volume */
    for (int s = 0; s < nspec; s++) { ssk += sinkvolc[bb][s]; sv += ice[bb].volc[s]; }
    if (ssk > sv) {
      const double frconst = 0.99 * sv / ssk;
      for (int s = 0; s < nspec; s++) sinkvolc[bb][s] = sinkvolc[bb][s] * frconst;
      sinknumc[bb] = sinknumc[bb] * frconst;
      sinknumc[bb] = fmind(sinknumc[bb], 0.99 * ice[bb].numc);
    }
  }
  for (int bb = 0; bb < nice; bb++) {                        /* :194-201 */
    ice[bb].numc = ice[bb].numc + fragnumc[bb];
    ice[bb].numc = ice[bb].numc - sinknumc[bb];
    ice[bb].numc = fmaxd(0., ice[bb].numc);
    for (int s = 0; s < nspec; s++) {
      ice[bb].volc[s] = ice[bb].volc[s] + fragvolc[bb][s];
      ice[bb].volc[s] = ice[bb].volc[s] - sinkvolc[bb][s];
      ice[bb].volc[s] = fmaxd(0., ice[bb].volc[s]);
    }
  }
}

/* mo_salsa_SIP_DF.f90:370-398 df_lawson (mode 1), df_sullivan (mode 2), df_phillips_simple
   (mode 3): fragments from nfrzn frozen drops of mean diameter ddmean */
static double df_fragments(int mode, double T, double nfrzn, double ddmean) {
  if (mode == 1) return nfrzn * 2.5e-11 * pow(fmind(ddmean, 3.e-3) * 1.e6, 4.);
  if (mode == 2) {
    const double hT = f_gauss(T, 10., 258.) / f_gauss(258., 10., 258.);
    return nfrzn * 0.2 * hT * 2.5e-11 * pow(fmind(ddmean, 3.e-3) * 1.e6, 4.);
  }
  const double tl[5] = {-24. + 273.15, -20. + 273.15, -16. + 273.15, -10. + 273.15, -6. + 273.15};
  const double hv[5] = {0.6, 0.24, 2.6, 0.43, 0.35};
  double hT = 0.;
  if (T >= tl[0] && T < tl[1]) hT = (hv[1] - hv[0]) * ((T - tl[0]) / 4.) + hv[0];
  else if (T >= tl[1] && T < tl[2]) hT = (hv[2] - hv[1]) * ((T - tl[2]) / 4.) + hv[2];
  else if (T >= tl[2] && T < tl[3]) hT = (hv[3] - hv[2]) * ((T - tl[3]) / 6.) + hv[3];
  else if (T >= tl[3] && T < tl[4]) hT = (hv[4] - hv[3]) * ((T - tl[4]) / 4.) + hv[4];
  return nfrzn * ((4. / 9.) * 1.e4 * hT * ddmean);
}

/* mo_salsa_SIP_DF.f90:534-608: Phillips et al. (2018) fits in x = log10 of the drop
   diameter in mm, limited to 0.06-1.6 mm (beta: 0 below 0.4 mm, upper limit only) */
static double ph_x(double d) { return log10(fmaxd(fmind(d * 1.e3, 1.6), 0.06)); }
static double ph_cubic(double x, double c1, double c2, double c3, double c4) {
  return (c1 * cube(x)) + (c2 * sq(x)) + (c3 * x) + c4;
}
static double ph_beta(double d) {
  if (d < 0.4e-3) return 0.;
  const double x = log10(fmind(d * 1.e3, 1.6));
  return (-0.1839 * sq(x)) + (-0.2017 * x) + -0.0512;
}
/* :431-451 fragments per frozen drop, mode 1 (drop heavier than the crystal), eq. 1 */
static double df_phillips_mode1_total(double d, double T) {
  const double tc = T - 273.15, x = ph_x(d);
  const double T0 = ph_cubic(x, -1.3999, -5.3285, -3.9847, -15.0332);
  const double zeta = pow(10., ph_cubic(x, 2.4268, 3.3274, 2.0783, 1.2927));
  const double eta = pow(10., ph_cubic(x, 0.1242, -0.2316, -0.9874, -0.0827));
  return ph_beta(d) * tc + (zeta * sq(eta)) / (sq(tc - T0) + sq(eta));
}
/* :479-532 mode 2 (crystal heavier than the drop), eq. 7: from the collision's kinetic
   energy over the drop's surface energy */
static double df_phillips_mode2(const salsa_ref_ctx_t *c, double p, double T, double d, double disph, double dinsph,
                                double mrim, double mpri, double ncice, double rhoip) {
  const double rhoa = p / (RD * T);
  const double visc = (7.44523e-3 * sqrt(cube(T))) / (5093. * (T + 110.4));
  const double mfp = (1.656e-10 * T + 1.828e-8) * PSTAND / p;
  double knud = 2. * mfp / dinsph;
  double beta = 1. + knud * (1.142 + 0.558 * exp(-0.999 / knud));
  Shape ish;
  getShapeCoefficients(c, &ish, mpri, mrim, ncice);
  const double vti = terminal_vel(disph, rhoip, rhoa, visc, beta, 4, &ish, dinsph);
  knud = 2. * mfp / d;
  beta = 1. + knud * (1.142 + 0.558 * exp(-0.999 / knud));
  const double vtd = terminal_vel(d, c->rhowa, rhoa, visc, beta, 3, &ish, d);
  const double mip = (mrim + mpri) / ncice, mdp = c->rhowa * PI6 * cube(d);
  const double K0 = 0.5 * (mip * mdp / (mdp + mip)) * sq(vtd - vti);
  const double DE = K0 / (SURFW0 * PI * sq(d));
  const double fT = -4200. * (T - 273.15) / 3.3e5;   /* cwa, alf (mo_submctl.f90:268, 281) */
  return 3. * fmind(4. * fT, 1.) * (1. - fT) * fmaxd(DE - 0.2, 0.);
}
/* :313-372 df_phillips_full_total: the regime by the masses of drop and crystal */
static double df_phillips_full_total(const salsa_ref_ctx_t *c, double p, double T, double d, const Section *ice,
                                     double nf) {
  const int nspec = c->nused;
  double sv = 0.;
  for (int s = 0; s < nspec - 1; s++) sv += ice->volc[s];
  const double mrim = ice->volc[nspec - 1] * c->rhori, mpri = sv * c->rhoic, ncice = ice->numc;
  const double mip = (mrim + mpri) / ncice, mdp = c->rhowa * PI6 * cube(d);
  if (mdp > mip) {
    if (d < 50.e-6 && T > 267.15) return 0.;
    return fmind(df_phillips_mode1_total(d, T), 100.) * nf;
  }
  if (d < 150.e-6) return 0.;
  const double rhoip = (mrim * c->rhori + mpri * c->rhoic) / (mrim + mpri);
  return fmind(df_phillips_mode2(c, p, T, d, ice->dwet, ice->dnsp, mrim, mpri, ncice, rhoip), 100.) * nf;
}

/* mo_salsa_SIP_DF.f90:29-260 dropfracturing (per cell): the fragments of each frozen
   drop size go to the ice bins below it with a d^-3 number distribution */
static void dropfracturing(Cell *w, double ppres, double ptemp, double ptstep) {
  const salsa_ref_ctx_t *c = w->c;
  const int nprc = c->nprc, nice = c->nice, nspec = c->nused, mode = c->cfg.lssipdropfrac.mode;
  const double tmin = 248.15, tmax = 271.15;
  Section *ice = w->ice;
  double icediams[MAXB], icebw[MAXB];
  for (int bb = 0; bb < nice; bb++) {
    icediams[bb] = ice[bb].dmid;
    icebw[bb] = pow(ice[bb].vhilim / PI6, 1. / 3) - pow(ice[bb].vlolim / PI6, 1. / 3);
  }
  for (int e = 0; e < nprc * nice; e++) {
    w->mfrzn_df[e] = w->mfrzn_df[e] * ptstep;
    w->nfrzn_df[e] = w->nfrzn_df[e] * ptstep;
  }
  double fragvolc[MAXB][NSP], sinkvolc[MAXB][NSP], fragnumc[MAXB], sinknumc[MAXB];
  double fragv_loc[MAXB][NSP], fragn_loc[MAXB], sinkv[NSP], dNb[MAXB], dVb[MAXB];
  memset(fragvolc, 0, sizeof fragvolc); memset(sinkvolc, 0, sizeof sinkvolc);
  memset(fragnumc, 0, sizeof fragnumc); memset(sinknumc, 0, sizeof sinknumc);
  for (int bb = 0; bb < nice; bb++) {
    memset(fragv_loc, 0, sizeof fragv_loc); memset(fragn_loc, 0, sizeof fragn_loc);
    double vall = 0.;
    for (int s = 0; s < NSP; s++) vall += ice[bb].volc[s];
    for (int cc = 0; cc < nprc; cc++) {
      const double nf = w->nfrzn_df[cc * nice + bb], mf = w->mfrzn_df[cc * nice + bb];
      if (ptemp < tmin || ptemp > tmax || nf < 1.e-12 || vall < 1.e-15 || ice[bb].numc < ice[bb].nlim) continue;
      const double ddmean = pow(mf / nf / c->rhowa / PI6, 1. / 3.);
      if (ddmean < DLLIQ_DF) continue;
      int npmax = 0;                                        /* :122, 1-based count */
      for (int k = 0; k < nice; k++) npmax += icediams[k] <= ddmean;
      npmax = npmax - 1 > 1 ? npmax - 1 : 1;
      if (npmax <= 2) continue;
      const double dN = mode == 4 ? df_phillips_full_total(c, ppres, ptemp, ddmean, &ice[bb], nf)
                                  : df_fragments(mode, ptemp, nf, ddmean);
      for (int k = 0; k < nice; k++) dNb[k] = dVb[k] = 0.;
      double Nnorm = 0.;
      for (int k = 0; k < npmax; k++) dNb[k] = 1. / cube(icediams[k]);
      for (int k = 0; k < npmax; k++) Nnorm += dNb[k] * icebw[k];
      for (int k = 0; k < npmax; k++) dNb[k] = dN * dNb[k] * icebw[k] / Nnorm;
      for (int k = 0; k < npmax; k++) dVb[k] = dNb[k] * PI6 * cube(icediams[k]);
      double sv = 0., sdv = 0.;
      for (int s = 0; s < nspec; s++) sv += ice[bb].volc[s];
      for (int k = 0; k < npmax; k++) sdv += dVb[k];
      for (int k = 0; k < npmax; k++) {
        fragn_loc[k] = fragn_loc[k] + dNb[k];
        for (int s = 0; s < nspec; s++) fragv_loc[k][s] = fragv_loc[k][s] + ice[bb].volc[s] * (dVb[k] / sv);
      }
      for (int s = 0; s < nspec; s++) sinkv[s] = ice[bb].volc[s] * sdv / sv;
      for (int s = 0; s < nspec; s++) sinkvolc[bb][s] = sinkvolc[bb][s] + sinkv[s];
      const double v_i = mf / nf / c->rhowa;
      double ss = 0.;
      for (int s = 0; s < nspec; s++) ss += sinkv[s];
      sinknumc[bb] = sinknumc[bb] + ss / v_i;
      double sdn = 0.;                                      /* :165-167 */
      for (int k = 0; k < npmax; k++) ice[k].sip[0] = ice[k].sip[0] + dNb[k];
      for (int k = 0; k < nice; k++) sdn += dNb[k];
      rate_acc_n(&w->rate[R_SIPDRFR], sdn / ptstep);
    }
    for (int k = 0; k < nice; k++) {                        /* :175-176, before the safeguard */
      fragnumc[k] = fragnumc[k] + fragn_loc[k];
      for (int s = 0; s < NSP; s++) fragvolc[k][s] = fragvolc[k][s] + fragv_loc[k][s];
    }
    if (ice[bb].numc < sinknumc[bb]) {                      /* :183-189 */
      sinknumc[bb] = ice[bb].numc;
      for (int s = 0; s < nspec; s++) sinkvolc[bb][s] = ice[bb].volc[s];
    }
    double ssk = 0., sv = 0.;                               /* :191-199: fragments already added */
    for (int s = 0; s < nspec; s++) { ssk += sinkvolc[bb][s]; sv += ice[bb].volc[s]; }
    if (ssk > sv) {
      const double frconst = 0.99 * sv / ssk;
      for (int s = 0; s < nspec; s++) sinkvolc[bb][s] = sinkvolc[bb][s] * frconst;
      sinknumc[bb] = sinknumc[bb] * frconst;
      sinknumc[bb] = fmind(sinknumc[bb], 0.99 * ice[bb].numc);
    }
  }
  for (int bb = 0; bb < nice; bb++) {                       /* :230-237 */
    ice[bb].numc = ice[bb].numc + fragnumc[bb];
    ice[bb].numc = ice[bb].numc - sinknumc[bb];
    ice[bb].numc = fmaxd(0., ice[bb].numc);
    for (int s = 0; s < nspec; s++) {
      ice[bb].volc[s] = ice[bb].volc[s] + fragvolc[bb][s];
      ice[bb].volc[s] = ice[bb].volc[s] - sinkvolc[bb][s];
      ice[bb].volc[s] = fmaxd(0., ice[bb].volc[s]);
    }
  }
}

/* mo_salsa_SIP_IIBR.f90:262-291 imf_sullivan (mode 1), imf_sotiropoulou (mode 2):
   fragments per collision, at most 100 */
static double iibr_imf(int mode, double T, double dmin) {
  const double fbr = 280., Tmin = 252., D0 = 0.02;
  double imf;
  if (mode == 1) imf = T < Tmin ? 0. : fmaxd(0., fbr * pow(T - Tmin, 1.2) * exp(-(T - Tmin) / 5.));
  else imf = T <= Tmin ? 0. : fmaxd(0., fbr * pow(T - Tmin, 1.2) * exp(-(T - Tmin) / 5.) * dmin / D0);
  return fmind(imf, 100.0);
}

/* mo_salsa_SIP_IIBR.f90:588-607 mip and :552-585 getvelocity: mean crystal mass of an ice
   bin, and its fall speed with the bin's shape coefficients and rime-weighted density */
static void iibr_masses(const salsa_ref_ctx_t *c, const Section *s, double *mrim, double *mpri) {
  double v = 0.;
  for (int k = 0; k <= c->iwa; k++) v += s->volc[k];
  *mrim = s->volc[c->irim] * c->rhori;
  *mpri = v * c->rhoic;
}
static double iibr_mip(const salsa_ref_ctx_t *c, const Section *s) {
  double mrim, mpri;
  iibr_masses(c, s, &mrim, &mpri);
  return (mrim + mpri) / s->numc;
}
static double iibr_velocity(const salsa_ref_ctx_t *c, const Section *s, double visc, double rhoa, double mfp) {
  const double knud = 2. * mfp / s->dnsp;
  const double beta = 1. + knud * (1.142 + 0.558 * exp(-0.999 / knud));
  double mrim, mpri;
  iibr_masses(c, s, &mrim, &mpri);
  const double rhoip = (mrim * c->rhori + mpri * c->rhoic) / (mrim + mpri);
  Shape sh;
  getShapeCoefficients(c, &sh, mpri, mrim, s->numc);
  return terminal_vel(s->dwet, rhoip, rhoa, visc, beta, 4, &sh, s->dnsp);
}
/* :505-548 kinetic_collision_energy of two ice bins */
static double iibr_k0(const salsa_ref_ctx_t *c, double p, double T, const Section *a, const Section *b) {
  const double rhoa = p / (RD * T);
  const double visc = (7.44523e-3 * sqrt(cube(T))) / (5093. * (T + 110.4));
  const double mfp = (1.656e-10 * T + 1.828e-8) * PSTAND / p;
  const double v1 = iibr_velocity(c, a, visc, rhoa, mfp), m1 = iibr_mip(c, a);
  const double v2 = iibr_velocity(c, b, visc, rhoa, mfp), m2 = iibr_mip(c, b);
  return (m1 * m2 / (m1 + m2)) * (1.7 * sq(v1 - v2) + 0.3 * v1 * v2);
}
/* :323-401 imf_phillips_mod: Phillips et al. (2017) breakup with the corrections of
   Sotiropoulou et al. (2020); asperity parameters by the rime fraction of `small`, the
   supersaturation over ice ssi and the distance from -15 C */
static double imf_phillips_mod(const salsa_ref_ctx_t *c, double p, double T, const Section *large,
                               const Section *small, double disphmin, double ssi) {
  const double T0 = 258.15;
  double mrim, mpri;
  iibr_masses(c, small, &mrim, &mpri);
  const double rimfrac = mrim / (mrim + mpri);
  double a0, C, g, Nmax;
  if (rimfrac > 0.5) {
    a0 = exp(14.74 * ssi + 14.28);
    C = exp(20.15 * ssi + 13.78);
    g = ssi + 0.55;
    Nmax = 600.;
  } else {
    a0 = 4.75E7;
    C = 1.0E08;
    g = 0.78;
    Nmax = 500.;
  }
  const double Am = a0 / 3. + fmaxd(2. / 3. * a0 - 1. / 9. * a0 * fabs(T - T0), 0.);
  const double alpha = PI * sq(disphmin);
  const double K0 = iibr_k0(c, p, T, large, small);
  return fmind(alpha * Am * (1 - exp(-pow(C * K0 / alpha / Am, g))), Nmax);
}

/* mo_salsa_SIP_IIBR.f90:23-258 iceicecollbreak (per cell): each pair (smaller bb, larger cc)
   breaks the smaller crystal into fragments spread over the bins below it as d^-3 */
static void iceicecollbreak(Cell *w, double ppres, double ptemp, double ptstep, double prv, double prsi) {
  const salsa_ref_ctx_t *c = w->c;
  const int nice = c->nice, nspec = c->nused, mode = c->cfg.lssipicecollbreak.mode;
  const double tmin = 248.15, tmax = 270.15;
  Section *ice = w->ice;
  double icediams[MAXB], icebw[MAXB];
  for (int bb = 0; bb < nice; bb++) {
    icediams[bb] = ice[bb].dmid;
    icebw[bb] = pow(ice[bb].vhilim / PI6, 1. / 3) - pow(ice[bb].vlolim / PI6, 1. / 3);
  }
  for (int e = 0; e < nice * nice; e++) {
    w->mii_ibr[e] = w->mii_ibr[e] * ptstep;
    w->nii_ibr[e] = w->nii_ibr[e] * ptstep;
  }
  double fragvolc[MAXB][NSP], sinkvolc[MAXB][NSP], fragnumc[MAXB], sinknumc[MAXB];
  double fragv_loc[MAXB][NSP], fragn_loc[MAXB], sinkv[NSP], dNb[MAXB], dVb[MAXB];
  memset(fragvolc, 0, sizeof fragvolc); memset(sinkvolc, 0, sizeof sinkvolc);
  memset(fragnumc, 0, sizeof fragnumc); memset(sinknumc, 0, sizeof sinknumc);
  for (int bb = 0; bb < nice; bb++) {
    memset(fragv_loc, 0, sizeof fragv_loc); memset(fragn_loc, 0, sizeof fragn_loc);
    for (int cc = bb; cc < nice; cc++) {
      const double nii = w->nii_ibr[cc * nice + bb], mii = w->mii_ibr[cc * nice + bb];
      double vb = 0., vc = 0.;
      for (int s = 0; s < NSP; s++) { vb += ice[bb].volc[s]; vc += ice[cc].volc[s]; }
      if (ptemp < tmin || ptemp > tmax || nii < 1.e-12 || mii < 1.e-15 || vb < 1.e-15 || ice[bb].numc < ice[bb].nlim ||
          vc < 1.e-15 || ice[cc].numc < ice[cc].nlim)
        continue;
      updateDiameter(c, &ice[bb], 1, T_ALL);
      const double v_i = mii / nii / ice[bb].rhomean;
      const double dinsphmin = pow(v_i / PI6, 1. / 3.);
      int npmax = 0;
      for (int k = 0; k < nice; k++) npmax += icediams[k] <= dinsphmin;
      npmax = npmax - 1;
      if (npmax <= 2) continue;
      double dN;
      if (mode == 3) {   /* :148-155: bb passes as the larger crystal, as the reference writes it */
        const double disphmin = pow((mii / nii / ice[bb].rhomean) / PI6, 1. / 3.);
        const double ssi = fmaxd(0., prv / prsi - 1.0);
        dN = fmind(imf_phillips_mod(c, ppres, ptemp, &ice[bb], &ice[cc], disphmin, ssi), 600.0) * nii;
      } else {
        dN = iibr_imf(mode, ptemp, dinsphmin) * nii;
      }
      for (int k = 0; k < nice; k++) dNb[k] = dVb[k] = 0.;
      double Nnorm = 0.;
      for (int k = 0; k < npmax; k++) dNb[k] = 1. / cube(icediams[k]);
      for (int k = 0; k < npmax; k++) Nnorm += dNb[k] * icebw[k];
      for (int k = 0; k < npmax; k++) dNb[k] = dN * dNb[k] * icebw[k] / Nnorm;
      for (int k = 0; k < npmax; k++) dVb[k] = dNb[k] * PI6 * cube(icediams[k]);
      double sv = 0., sdv = 0.;
      for (int s = 0; s < nspec; s++) sv += ice[bb].volc[s];
      for (int k = 0; k < npmax; k++) sdv += dVb[k];
      for (int k = 0; k < npmax; k++) {
        fragn_loc[k] = fragn_loc[k] + dNb[k];
        for (int s = 0; s < nspec; s++) fragv_loc[k][s] = fragv_loc[k][s] + ice[bb].volc[s] * (dVb[k] / sv);
      }
      for (int s = 0; s < nspec; s++) sinkv[s] = ice[bb].volc[s] * sdv / sv;
      for (int s = 0; s < nspec; s++) sinkvolc[bb][s] = sinkvolc[bb][s] + sinkv[s];
      double ss = 0.;
      for (int s = 0; s < nspec; s++) ss += sinkv[s];
      sinknumc[bb] = sinknumc[bb] + ss / v_i;
      double sdn = 0.;                                      /* :187-189 */
      for (int k = 0; k < npmax; k++) ice[k].sip[2] = ice[k].sip[2] + dNb[k];
      for (int k = 0; k < nice; k++) sdn += dNb[k];
      rate_acc_n(&w->rate[R_SIPIIBR], sdn / ptstep);
    }
    for (int k = 0; k < nice; k++) {                        /* :187-188, before the safeguard */
      fragnumc[k] = fragnumc[k] + fragn_loc[k];
      for (int s = 0; s < NSP; s++) fragvolc[k][s] = fragvolc[k][s] + fragv_loc[k][s];
    }
    if (ice[bb].numc < sinknumc[bb]) {
      sinknumc[bb] = ice[bb].numc;
      for (int s = 0; s < nspec; s++) sinkvolc[bb][s] = ice[bb].volc[s];
    }
    double ssk = 0., sv = 0.;
    for (int s = 0; s < nspec; s++) { ssk += sinkvolc[bb][s]; sv += ice[bb].volc[s]; }
    if (ssk > sv) {
      const double frconst = 0.99 * sv / ssk;
      for (int s = 0; s < nspec; s++) sinkvolc[bb][s] = sinkvolc[bb][s] * frconst;
      sinknumc[bb] = sinknumc[bb] * frconst;
      sinknumc[bb] = fmind(sinknumc[bb], 0.99 * ice[bb].numc);
    }
  }
  for (int bb = 0; bb < nice; bb++) {
    ice[bb].numc = ice[bb].numc + fragnumc[bb];
    ice[bb].numc = ice[bb].numc - sinknumc[bb];
    ice[bb].numc = fmaxd(0., ice[bb].numc);
    for (int s = 0; s < nspec; s++) {
      ice[bb].volc[s] = ice[bb].volc[s] + fragvolc[bb][s];
      ice[bb].volc[s] = ice[bb].volc[s] - sinkvolc[bb][s];
      ice[bb].volc[s] = fmaxd(0., ice[bb].volc[s]);
    }
  }
}

/* ======================================================================
 * mo_salsa.f90:45-153 salsa
 * ====================================================================== */
static void salsa_cell(Cell *w, double ppres, double *prv, double prs, double prsi, double ptemp, double ptstep,
                       double pw, int level, double *actd_n, double *actd_v, double *zg) {
  const salsa_ref_ctx_t *c = w->c;
  const salsa_config_t *g = &c->cfg;
  if (c->st_coag) coagulation(w, ptstep, ptemp, ppres);
  if (c->st_secice) {                                                   /* :98-99 */
    if (c->st_siprs) rimesplintering(w, ptemp, ptstep);
    if (c->st_sipdf) dropfracturing(w, ppres, ptemp, ptstep);
    if (c->st_sipib) iceicecollbreak(w, ppres, ptemp, ptstep, *prv, prsi);
  }
  if (c->st_cnd) {
    /* condensation :276-342.  nucleation (mo_salsa_nucleation.f90:72-625) only returns the
       3 nm formation rates, which condgas does not read (see condgas), and the H2SO4
       fraction of the clusters: 1 for the H2SO4 schemes nsnucl = 1-3; for the mixed
       schemes 5-9 it only multiplies condgas's vanishing nucleation term, and 1 stands in. */
    const double zxsa = g->nsnucl > 0 ? 1. : 0.;
    if (g->lscndgas) condgas(w, &zg[0], &zg[3], &zg[4], zxsa, ptemp, ppres, ptstep);
    if (g->lscndh2ocl || g->lscndh2oae || g->lscndh2oic) gpparth2o(w, ptemp, ppres, prs, prsi, prv, ptstep);
  }
  if (c->st_auto && g->lsauto.mode == 2) autoconv2(w, ptstep);
  if (c->st_activ) {
    for (int k = 0; k < c->ncld; k++) { actd_n[k] = 0.; for (int s = 0; s < NSP; s++) actd_v[k * NSP + s] = 0.; }
    if (g->lsactiv.mode == 1) actInterst(w, *prv, prs, ptemp);
    if (g->lsactiv.mode == 2) ActCloudBase(w, ppres, ptemp, pw, actd_n, actd_v);
  }
  if (c->st_icenucl || g->lsicenucl.mode == 2) {
    if (g->lsicehom || g->lsiceimm || g->lsicedep) {
      if (g->ice_theta_dist) ice_nucl_SE(w, ptemp, *prv, prs, prsi, ptstep);
      else ice_nucl_classic(w, ptemp, *prv, prs, prsi, ptstep);
    }
  }
  if (c->st_icemelt) ice_melt(w, ptemp);
  if (g->lsdistupdate) distr_update(w, level);
}

/* ======================================================================
 * Setup: classSpecies.f90:167-341, mo_salsa_init.f90:148-450, 792-858
 * ====================================================================== */
static const char *ALLNAMES[9] = {"SO4", "OC", "BC", "DU", "SS", "NO", "NH", "H2O", "rime"};
static const double ALLMM[9] = {98.08e-3, 150.e-3, 12.e-3, 100.e-3, 58.44e-3, 62.01e-3, 18.04e-3, 18.016e-3, 18.016e-3};
static const double ALLRHO[9] = {1830., 1400., 2000., 2650., 2165., 1479., 1530., 1000., 400.};
static const double ALLDISS[9] = {3., 1., 0., 0., 2., 1., 1., 1., 1.};

static int name_eq(const char *a, const char *b) {
  /* Fortran blank-padded comparison of up to 4 characters */
  char x[5] = {0}, y[5] = {0};
  strncpy(x, a, 4); strncpy(y, b, 4);
  for (int i = 3; i >= 0 && (x[i] == ' ' || x[i] == 0); i--) x[i] = 0;
  for (int i = 3; i >= 0 && (y[i] == ' ' || y[i] == 0); i--) y[i] = 0;
  return strcmp(x, y) == 0;
}

static void make_section(Section *s, int phase, double nlim, double dlim, double ctmax, double cenh) {
  memset(s, 0, sizeof *s);
  s->phase = phase; s->nlim = nlim; s->dlim = dlim;
  s->chargeTimeMax = ctmax; s->chargeCollEnh = cenh;
}

static void set_bin(Section *s, double vlo, double vhi) {
  s->vlolim = vlo; s->vhilim = vhi;
  s->dmid = pow((s->vhilim + s->vlolim) / (2. * PI6), 1. / 3.);
  s->vratiohi = s->vhilim / (PI6 * cube(s->dmid));
  s->vratiolo = s->vlolim / (PI6 * cube(s->dmid));
  s->dwet = s->dmid;
}

int salsa_ref_create(const salsa_config_t *cfg, salsa_ref_ctx_t **out) {
  if (!cfg || !out) return SALSA_E_ARG;
  if (cfg->nbin[0] < 1 || cfg->nbin[1] < 4 || cfg->prc_nbins < 1 || cfg->ice_nbins < 1) return SALSA_E_ARG;
  if (cfg->nspec_dry < 1 || cfg->nspec_dry > SALSA_MAXSPEC) return SALSA_E_ARG;
  /* secondary ice (mo_salsa_secondary_ice.f90:6-40): rime splintering (mo_salsa_SIP_RS.f90)
     in its two modes, drop fracturing (mo_salsa_SIP_DF.f90) in modes 1-3 and ice-ice
     breakup (mo_salsa_SIP_IIBR.f90) in modes 1-2; Phillips' schemes (drop fracturing
     mode 4, breakup mode 3) are not restated */
  if (cfg->lssecice.sw && cfg->level == 5 &&
      ((cfg->lssipicecollbreak.sw && (cfg->lssipicecollbreak.mode < 1 || cfg->lssipicecollbreak.mode > 3)) ||
       (cfg->lssiprimespln.sw && cfg->lssiprimespln.mode != 1 && cfg->lssiprimespln.mode != 2) ||
       (cfg->lssipdropfrac.sw && (cfg->lssipdropfrac.mode < 1 || cfg->lssipdropfrac.mode > 4))))
    return SALSA_E_UNSUPPORTED;
  /* nucleation: the ternary scheme STOPs in the reference (mo_salsa_nucleation.f90:236-238);
     nj3 outside 1-3 STOPs once a cell nucleates (:600-602) */
  if (cfg->nsnucl == 4 || cfg->nsnucl < 0 || (cfg->nsnucl > 0 && (cfg->nj3 < 1 || cfg->nj3 > 3)))
    return SALSA_E_UNSUPPORTED;
  if (cfg->level == 5 && cfg->fixinc > 0. && !(cfg->lsicehom || cfg->lsiceimm || cfg->lsicedep))
    return SALSA_E_UNSUPPORTED;   /* ice_fixed_NC: marked broken in the reference (mo_salsa_cloud_ice.f90:321) */
  int ntot = cfg->nbin[0] + 2 * cfg->nbin[1] + 2 * cfg->nbin[1] + cfg->prc_nbins + cfg->ice_nbins;
  if (ntot > MAXB) return SALSA_E_ARG;
  salsa_ref_ctx_t *c = (salsa_ref_ctx_t *)calloc(1, sizeof *c);
  if (!c) return SALSA_E_ARG;
  c->cfg = *cfg;
  /* species */
  int allInd[9], used[9];
  for (int i = 0; i < 9; i++) { allInd[i] = -1; used[i] = 0; }
  for (int i = 0; i < cfg->nspec_dry; i++)
    for (int k = 0; k < SALSA_MAXSPEC; k++)
      if (name_eq(ALLNAMES[k], cfg->listspec[i])) { allInd[k] = i; used[k] = 1; }
  int nlist = cfg->nspec_dry;
  for (int k = 0; k < SALSA_MAXSPEC; k++) if (used[k]) {
    int cnt = 0; for (int j = 0; j < SALSA_MAXSPEC; j++) cnt += used[j];
    (void)cnt;
  }
  {
    int cnt = 0; for (int j = 0; j < SALSA_MAXSPEC; j++) cnt += used[j];
    if (cnt != nlist) { free(c); return SALSA_E_ARG; }   /* unknown or repeated name */
  }
  allInd[7] = nlist; used[7] = 1;
  allInd[8] = nlist + 1; used[8] = 1;
  c->nused = nlist + 2; c->ndry = nlist; c->nwet = nlist + 1; c->iwa = nlist; c->irim = nlist + 1;
  for (int k = 0; k < 9; k++) c->idx_name[k] = used[k] ? allInd[k] : -1;
  for (int k = 0; k < 9; k++) if (used[k]) {
    int j = allInd[k];
    c->rholiq[j] = ALLRHO[k];
    c->rhoice[j] = (k == 7) ? 917. : ALLRHO[k];
    c->MM[j] = ALLMM[k];
    c->diss[j] = ALLDISS[k];
  }
  c->nsoluble = c->ninsoluble = 0;
  for (int j = 0; j < c->nused; j++) {   /* PACK in mass-array order */
    for (int k = 0; k < 9; k++) if (used[k] && allInd[k] == j) {
      if (k == 0 || k == 1 || k == 4 || k == 5 || k == 6) c->ind_soluble[c->nsoluble++] = j;
      if (k == 2 || k == 3) c->ind_insoluble[c->ninsoluble++] = j;
    }
  }
  if (cfg->level == 5 && cfg->ice_theta_dist && (cfg->lsicehom || cfg->lsiceimm || cfg->lsicedep) &&
      c->idx_name[3] < 0) { free(c); return SALSA_E_UNSUPPORTED; }   /* iceNucleation indexes DU */
  c->rhosu = ALLRHO[0]; c->rhooc = ALLRHO[1]; c->rhono = ALLRHO[5]; c->rhoss = ALLRHO[4];
  c->msu = ALLMM[0]; c->moc = ALLMM[1]; c->mno = ALLMM[5]; c->mss = ALLMM[4];
  c->rhoic = 917.; c->rhori = 400.; c->rhowa = 1000.; c->mwa = ALLMM[7];
  /* bins */
  c->in1a = 0; c->in2a = c->in1a + cfg->nbin[0]; c->in2b = c->in2a + cfg->nbin[1];
  c->fn1a = c->in2a - 1; c->fn2a = c->fn1a + cfg->nbin[1]; c->fn2b = c->fn2a + cfg->nbin[1];
  c->nbins = c->fn2b + 1;
  int nba = c->fn2a - c->in2a + 1, nbb = nba;
  c->ica_cur = 0; c->ica_par = c->in2a;
  c->fca_cur = c->ica_cur + nba - 1; c->fca_par = c->ica_par + nba - 1;
  c->icb_cur = c->fca_cur + 1; c->icb_par = c->fn2b - nbb + 1;
  c->fcb_cur = c->icb_cur + nbb - 1; c->fcb_par = c->icb_par + nbb - 1;
  c->ncld = c->fcb_cur + 1;
  c->nprc = cfg->prc_nbins; c->nice = cfg->ice_nbins;
  c->ntotal = c->nbins + c->ncld + c->nprc + c->nice;
  c->nliquid = c->nbins + c->ncld + c->nprc;
  Section *ae = &c->tmpl[0], *cl = &c->tmpl[c->nbins], *pr = &c->tmpl[c->nbins + c->ncld],
          *ic = &c->tmpl[c->nbins + c->ncld + c->nprc];
  for (int i = 0; i < c->nbins; i++) make_section(&ae[i], 1, NLIM, DLAERO, cfg->chargeTMax, cfg->chargeCollEnh);
  for (int i = 0; i < c->ncld; i++) make_section(&cl[i], 2, NLIM, DLCLOUD, cfg->chargeTMax, cfg->chargeCollEnh);
  for (int i = 0; i < c->nprc; i++) make_section(&pr[i], 3, PRLIM, DLPRECP, cfg->chargeTMax, cfg->chargeCollEnh);
  for (int i = 0; i < c->nice; i++) make_section(&ic[i], 4, PRLIM, DLICE, cfg->chargeTMax, cfg->chargeCollEnh);
  {
    const double *rl = cfg->reglim;
    double ratio = rl[1] / rl[0];
    for (int cc = c->in1a; cc <= c->fn1a; cc++)
      set_bin(&ae[cc], PI6 * cube(rl[0] * pow(ratio, (double)(cc) / cfg->nbin[0])),
              PI6 * cube(rl[0] * pow(ratio, (double)(cc + 1) / cfg->nbin[0])));
    int nbin2 = 4, nbin3 = cfg->nbin[1] - nbin2;
    ratio = rl[2] / rl[1];
    for (int dd = c->in2a; dd <= c->in2a + nbin2 - 1; dd++) {
      int cc = dd - c->in2a;
      set_bin(&ae[dd], PI6 * cube(rl[1] * pow(ratio, (double)cc / nbin2)),
              PI6 * cube(rl[1] * pow(ratio, (double)(cc + 1) / nbin2)));
    }
    ratio = rl[3] / rl[2];
    for (int dd = c->in2a + nbin2; dd <= c->fn2a; dd++) {
      int cc = dd - (c->fn2a - (nbin3 - 1));
      set_bin(&ae[dd], PI6 * cube(rl[2] * pow(ratio, (double)cc / nbin3)),
              PI6 * cube(rl[2] * pow(ratio, (double)(cc + 1) / nbin3)));
    }
    for (int i = 0; i < cfg->nbin[1]; i++) {
      Section *b = &ae[c->in2b + i], *a = &ae[c->in2a + i];
      b->vlolim = a->vlolim; b->vhilim = a->vhilim; b->dmid = a->dmid; b->vratiohi = a->vratiohi;
      b->vratiolo = a->vratiolo; b->dwet = b->dmid;
    }
    for (int i = 0; i < c->nbins; i++) ae[i].dwet = ae[i].dmid;
  }
  for (int i = 0; i < nba; i++) {
    Section *a = &ae[c->ica_par + i], *b = &cl[c->ica_cur + i];
    b->vhilim = a->vhilim; b->vlolim = a->vlolim; b->vratiohi = a->vratiohi; b->vratiolo = a->vratiolo; b->dmid = a->dmid;
    a = &ae[c->icb_par + i]; b = &cl[c->icb_cur + i];
    b->vhilim = a->vhilim; b->vlolim = a->vlolim; b->vratiohi = a->vratiohi; b->vratiolo = a->vratiolo; b->dmid = a->dmid;
  }
  for (int i = 0; i < c->ncld; i++) cl[i].dwet = cl[i].dmid;
  {
    /* buildBinLimits :429-450 */
    double r = pow(cfg->prc_vol_ratio, 1. / 3.), lo = cfg->prc_dlo, hi = cfg->prc_dlo * pow(cfg->prc_vol_ratio, 1. / 3.);
    for (int i = 0; i < c->nprc; i++) {
      if (i > 0) { lo = lo * pow(cfg->prc_vol_ratio, 1. / 3.); hi = lo * pow(cfg->prc_vol_ratio, 1. / 3.); }
      set_bin(&pr[i], PI6 * cube(lo), PI6 * cube(hi));
      pr[i].dmid = pow((pr[i].vlolim + pr[i].vhilim) / (2. * PI6), 1. / 3.);
      pr[i].dwet = pr[i].dmid;
    }
    (void)r;
    lo = cfg->ice_dlo; hi = cfg->ice_dlo * pow(cfg->ice_vol_ratio, 1. / 3.);
    for (int i = 0; i < c->nice; i++) {
      if (i > 0) { lo = lo * pow(cfg->ice_vol_ratio, 1. / 3.); hi = lo * pow(cfg->ice_vol_ratio, 1. / 3.); }
      set_bin(&ic[i], PI6 * cube(lo), PI6 * cube(hi));
      ic[i].dwet = ic[i].dmid;
    }
  }
  for (int i = 0; i < c->nprc; i++) c->precpbins[i] = pow(pr[i].vlolim / PI6, 1. / 3.);
  for (int i = 0; i < c->nice; i++) c->icebins[i] = pow(ic[i].vlolim / PI6, 1. / 3.);   /* set_icebins :420-423 */
  for (int i = 0; i < c->nbins; i++) c->massacc[i] = 1.;
  *out = c;
  return SALSA_OK;
}

void salsa_ref_destroy(salsa_ref_ctx_t *ctx) {
  if (ctx) free(ctx->kcache);
  free(ctx);
}

int salsa_ref_layout(const salsa_ref_ctx_t *c, int *nbins, int *ncld, int *nprc, int *nice, int *nwet,
                     double *lolim) {
  if (!c) return SALSA_E_ARG;
  if (nbins) *nbins = c->nbins;
  if (ncld) *ncld = c->ncld;
  if (nprc) *nprc = c->nprc;
  if (nice) *nice = c->nice;
  if (nwet) *nwet = c->nwet;
  if (lolim)
    for (int i = 0; i < c->ntotal; i++) lolim[i] = pow(c->tmpl[i].vlolim / PI6, 1. / 3.);
  return SALSA_OK;
}

void salsa_ref_counters(const salsa_ref_ctx_t *c, long long out[5]) {
  for (int i = 0; i < 5; i++) out[i] = c->counters[i];
}

/* The sticky process states set_SALSA_runtime keeps (mo_salsa_driver.f90:445-474). */
void salsa_ref_states(const salsa_ref_ctx_t *c, int out[12]) {
  const int v[12] = {c->st_coag, c->st_cnd, c->st_auto, c->st_activ, c->st_icenucl, c->st_icemelt,
                     c->st_secice, c->st_siprs, c->st_sipdf, c->st_sipib, c->st_freeRH, c->st_freeTheta};
  for (int i = 0; i < 12; i++) out[i] = v[i];
}

/* ======================================================================
 * mo_salsa_driver.f90:112-435 run_SALSA (+ set_SALSA_runtime :445-474)
 * ====================================================================== */
int salsa_ref_run(salsa_ref_ctx_t *c, int nzp, int nxp, int nyp, int ns, double tstep, double time, int istp,
                  int level, int lcharge, int initialize, const salsa_fields_t *f, salsa_status_t *st,
                  int nthreads, int carry_over) {
  if (!c || !f) return SALSA_E_ARG;
  const salsa_config_t *g = &c->cfg;
  if (nzp < 3 || nxp < 5 || nyp < 5 || tstep <= 0. || level != g->level) return SALSA_E_ARG;
  if (ns < c->nwet) return SALSA_E_ARG;
  if (!f->press || !f->temp || !f->rsl || !f->dn || !f->rp || !f->rpt || !f->naero || !f->ncloud || !f->nprecp ||
      !f->naerot || !f->ncloudt || !f->nprecpt || !f->maero || !f->mcloud || !f->mprecp || !f->maerot ||
      !f->mcloudt || !f->mprecpt || !f->pa_nactd || !f->pa_vactd)
    return SALSA_E_ARG;
  if (level == 5 && (!f->rsi || !f->nice || !f->mice || !f->nicet || !f->micet)) return SALSA_E_ARG;
  if (level == 5 && g->ice_theta_dist && !f->indef) return SALSA_E_ARG;
  if (level == 5 && g->lssecice.sw && (!f->sipdrfr || !f->siprmspl || !f->sipiibr)) return SALSA_E_ARG;
  if (lcharge && !f->chargeTime) return SALSA_E_ARG;
  if (g->lscndgas && (!f->gaero || !f->gaerot)) return SALSA_E_ARG;
  if (g->lsactiv.sw && g->lsactiv.mode == 2 && !f->wp) return SALSA_E_ARG;
  /* set_SALSA_runtime (sticky states) */
  const salsa_switch_t *ms[7] = {&g->lscoag, &g->lscnd, &g->lsauto, &g->lsactiv, &g->lsicenucl, &g->lsicemelt,
                                 &g->lssecice};
  int *sts[7] = {&c->st_coag, &c->st_cnd, &c->st_auto, &c->st_activ, &c->st_icenucl, &c->st_icemelt, &c->st_secice};
  int lvl4 = (level == 4);
  for (int i = 0; i < 7; i++) {
    int sw = ms[i]->sw;
    if (lvl4 && (i == 4 || i == 5 || i == 6)) sw = 0;    /* define_salsa :615-635 */
    if (sw && time >= ms[i]->delay) *sts[i] = 1;
  }
  /* subprocess switches; define_salsa switches them off at level 4 (:631-633) */
  if (!lvl4 && g->lssiprimespln.sw && time >= g->lssiprimespln.delay) c->st_siprs = 1;
  if (!lvl4 && g->lssipdropfrac.sw && time >= g->lssipdropfrac.delay) c->st_sipdf = 1;
  if (!lvl4 && g->lssipicecollbreak.sw && time >= g->lssipicecollbreak.delay) c->st_sipib = 1;
  if (g->lsfreeRH.sw && time > g->lsfreeRH.delay) c->st_freeRH = 1;
  if (g->lsFreeTheta.sw && time > g->lsFreeTheta.delay) c->st_freeTheta = 1;
  c->lcgupdt = (c->st_coag && g->lscoag.mode == 2 && (fmod(time, g->cgintvl) < tstep || istp <= 1));
  (void)istp;
  /* level 4 forces the ice sub-switches off (define_salsa :615-635) */
  salsa_ref_ctx_t cl4;
  const salsa_ref_ctx_t *cc = c;
  if (lvl4) {
    cl4 = *c;
    cl4.cfg.lscgia = cl4.cfg.lscgic = cl4.cfg.lscgii = cl4.cfg.lscgip = 0;
    cl4.cfg.lscndh2oic = 0;
    cl4.cfg.ice_theta_dist = 0;
    cl4.cfg.lsicehom = cl4.cfg.lsiceimm = cl4.cfg.lsicedep = 0;
    cc = &cl4;
  }
  long long plane = (long long)nzp * nxp * nyp;
  int nbins = c->nbins, ncld = c->ncld, nprc = c->nprc, nice = c->nice, nwet = c->nwet, ndry = c->ndry;
  int iwa = c->iwa, irim = c->irim;
  long long s_eq = 0, s_di = 0, s_nf = 0, s_co = 0, s_ng = 0, s_nan = 0, ncell = 0;
  long long cnt[5] = {0, 0, 0, 0, 0};
  int nint_z = nzp - 2, nint_x = nxp - 4, nint_y = nyp - 4;
  long long ncells = (long long)nint_z * nint_x * nint_y;
  if (carry_over) nthreads = 1;
#ifdef _OPENMP
  int nt = nthreads > 0 ? nthreads : omp_get_max_threads();
#else
  int nt = 1; (void)nthreads;
#endif
  const double *nin[4] = {f->naero, f->ncloud, f->nprecp, f->nice};
  double *nten[4] = {f->naerot, f->ncloudt, f->nprecpt, f->nicet};
  const double *min_[4] = {f->maero, f->mcloud, f->mprecp, f->mice};
  double *mten[4] = {f->maerot, f->mcloudt, f->mprecpt, f->micet};
  int bstart[4] = {0, nbins, nbins + ncld, nbins + ncld + nprc};
  int bnum[4] = {nbins, ncld, nprc, nice};
  if (!carry_over) c->carry_valid = 0;
  /* initialize_coagstorage (mo_salsa_driver.f90:601-650): zero storage for the grid */
  if (g->lscoag.mode == 2 && (!c->kcache || c->kcache_cells != ncells)) {
    free(c->kcache);
    c->kcache = (double *)calloc((size_t)(ncells * kc_cell_doubles(c)), sizeof(double));
    c->kcache_cells = c->kcache ? ncells : 0;
    if (!c->kcache) return SALSA_E_ARG;
  }
  if (lvl4) { cl4.kcache = c->kcache; cl4.kcache_cells = c->kcache_cells; }

#pragma omp parallel num_threads(nt) reduction(+ : s_eq, s_di, s_nf, s_co, s_ng, s_nan, ncell, cnt[:5])
  {
    Cell *w = (Cell *)malloc(sizeof(Cell));
    double actd_n[MAXB], actd_v[MAXB * NSP];
#pragma omp for schedule(dynamic, 64)
    for (long long q = 0; q < ncells; q++) {
      /* reference loop order: jj outer, ii, kk = nzp-1..2 descending */
      long long r = q;
      int kq = (int)(r % nint_z); r /= nint_z;
      int iq = (int)(r % nint_x); r /= nint_x;
      int jq = (int)r;
      int kk = nzp - 2 - kq, ii = 2 + iq, jj = 2 + jq;
      long long p = kk + (long long)nzp * (ii + (long long)nxp * jj);
      cell_clear(w, cc);
      w->c = cc;
      w->lcharge = lcharge;
      w->level = level;
      if (carry_over && c->carry_valid) memcpy(w->all, c->carry, sizeof(Section) * c->ntotal);
      else memcpy(w->all, c->tmpl, sizeof(Section) * c->ntotal);
      w->aero = &w->all[0]; w->cloud = &w->all[nbins]; w->precp = &w->all[nbins + ncld];
      w->ice = &w->all[nbins + ncld + nprc]; w->liquid = &w->all[0];
      w->kappa = f->kappa;
      if (f->kappa) w->kappa_cell = f->kappa[p];
      w->cell = q;
      double in_p = f->press[p], in_t = f->temp[p], in_rs = f->rsl[p];
      double in_rsi = (level == 5) ? f->rsi[p] : 0.;
      double in_w = f->wp ? f->wp[p] : 0.;
      double in_rv = c->st_freeRH ? f->rp[p] : fmind(f->rp[p], f->rsl[p] * g->rhlim);
      double rv_old = in_rv;
      double dn = f->dn[p];
      for (int nb = 0; nb < c->ntotal; nb++) {
        Section *s = &w->all[nb];
        int icat = s->phase - 1;
        if (icat == 3 && level < 5) break;
        int nbloc = nb - bstart[icat], cat_nb = bnum[icat];
        if (icat < 3) {
          for (int nc = 0; nc < nwet; nc++)
            s->volc[nc] = min_[icat][p + plane * (nc * cat_nb + nbloc)] * dn / c->rholiq[nc];
          if (level == 5 && g->ice_theta_dist) s->INdef = f->indef[p + plane * nb];
          if (lcharge) s->chargeTime = f->chargeTime[p + plane * nb];
        } else {
          for (int nc = 0; nc < nwet; nc++)
            s->volc[nc] = min_[icat][p + plane * (nc * cat_nb + nbloc)] * dn / c->rhoice[nc];
          s->volc[irim] = min_[icat][p + plane * (irim * cat_nb + nbloc)] * dn / c->rhori;
          if (g->lssecice.sw) {                                            /* :258-262 */
            s->sip[0] = f->sipdrfr[p + plane * nbloc] * dn;
            s->sip[1] = f->siprmspl[p + plane * nbloc] * dn;
            s->sip[2] = f->sipiibr[p + plane * nbloc] * dn;
          }
        }
        s->numc = nin[icat][p + plane * nbloc] * dn;
        updateRhomean(cc, s);
        if (s->numc > s->nlim) {
          double sd = 0.;
          for (int i = 0; i < ndry; i++) sd += s->volc[i];
          s->core = sd / s->numc;
        } else {
          s->core = PI6 * cube(s->dmid);
        }
      }
      if (initialize) equilibration(w, 0.3, in_t, 1);
      /* gases in #/m3 (mo_salsa_driver.f90:285-290): SO4, HNO3, NH3, OC non-volatile, OC semi-volatile */
      double zg[5] = {0., 0., 0., 0., 0.};
      if (f->gaero)
        for (int i = 0; i < 5; i++) zg[i] = f->gaero[p + plane * i] * dn;
      for (int k = 0; k < ncld; k++) { actd_n[k] = 0.; for (int s2 = 0; s2 < NSP; s2++) actd_v[k * NSP + s2] = 0.; }
      salsa_cell(w, in_p, &in_rv, in_rs, in_rsi, in_t, tstep, in_w, level, actd_n, actd_v, zg);
      if (g->lscoag.mode == 2 && c->lcgupdt) kc_copy(w, 1);   /* store_coag (:421-423) */
      for (int nb = 0; nb < c->ntotal; nb++) {
        Section *s = &w->all[nb];
        int icat = s->phase - 1;
        if (icat == 3 && level < 5) break;
        int nbloc = nb - bstart[icat], cat_nb = bnum[icat];
        if (icat < 3) {
          for (int nc = 0; nc < nwet; nc++) {
            long long str = p + plane * (nc * cat_nb + nbloc);
            mten[icat][str] = mten[icat][str] + ((s->volc[nc] * c->rholiq[nc] / dn) - min_[icat][str]) / tstep;
          }
          if (level == 5 && g->ice_theta_dist) f->indef[p + plane * nb] = s->INdef;
          if (lcharge) f->chargeTime[p + plane * nb] = s->chargeTime;
        } else {
          for (int nc = 0; nc < nwet; nc++) {
            long long str = p + plane * (nc * cat_nb + nbloc);
            mten[icat][str] = mten[icat][str] + ((s->volc[nc] * c->rhoice[nc] / dn) - min_[icat][str]) / tstep;
          }
          long long str = p + plane * (irim * cat_nb + nbloc);
          mten[icat][str] = mten[icat][str] + ((s->volc[irim] * c->rhori / dn) - min_[icat][str]) / tstep;
          if (g->lssecice.sw) {                                            /* :345-349 */
            f->sipdrfr[p + plane * nbloc] = s->sip[0] / dn;
            f->siprmspl[p + plane * nbloc] = s->sip[1] / dn;
            f->sipiibr[p + plane * nbloc] = s->sip[2] / dn;
          }
        }
        nten[icat][p + plane * nbloc] = nten[icat][p + plane * nbloc] + ((s->numc / dn) - nin[icat][p + plane * nbloc]) / tstep;
        if (!isfinite(s->numc)) s_nan++;
      }
      for (int k = 0; k < ncld; k++) f->pa_nactd[p + plane * k] = actd_n[k] / dn;
      for (int nc = 0; nc < nwet; nc++)
        for (int k = 0; k < ncld; k++)
          f->pa_vactd[p + plane * (nc * ncld + k)] = actd_v[k * NSP + nc] * c->rholiq[nc] / dn;
      f->rpt[p] = f->rpt[p] + (in_rv - rv_old) / tstep;
      if (g->lscndgas)   /* :369-384 */
        for (int i = 0; i < 5; i++)
          f->gaerot[p + plane * i] = f->gaerot[p + plane * i] + ((zg[i] / dn) - f->gaero[p + plane * i]) / tstep;
      if (g->diagnostics) {
        double d[SALSA_NDIAG];
        const Rate *R = w->rate;
        d[SALSA_DIAG_AUTOC] = R[R_AUTOC].volc[iwa] * c->rhowa / dn;
        d[SALSA_DIAG_AUTOC80] = R[R_AUTOC80].volc[iwa] * c->rhowa / dn;
        d[SALSA_DIAG_AUTOC50] = R[R_AUTOC50].volc[iwa] * c->rhowa / dn;
        d[SALSA_DIAG_ACCR] = R[R_ACCR].volc[iwa] * c->rhowa / dn;
        d[SALSA_DIAG_ACCR80] = R[R_ACCR80].volc[iwa] * c->rhowa / dn;
        d[SALSA_DIAG_ACCR50] = R[R_ACCR50].volc[iwa] * c->rhowa / dn;
        double a1 = 0., a2 = 0., a3 = 0.;
        for (int i = 0; i < ndry; i++) {
          a1 += R[R_ACCOLL].volc[i] * c->rholiq[i];
          a2 += R[R_APCOLL].volc[i] * c->rholiq[i];
          a3 += R[R_AICOLL].volc[i] * c->rhoice[i];
        }
        d[SALSA_DIAG_ACCOLL] = a1 / dn;
        d[SALSA_DIAG_APCOLL] = a2 / dn;
        d[SALSA_DIAG_ACTIV] = R[R_ACTIV].numc / dn;
        d[SALSA_DIAG_CONDA] = R[R_CONDA].volc[iwa] / dn;
        d[SALSA_DIAG_CONDC] = R[R_CONDC].volc[iwa] / dn;
        d[SALSA_DIAG_CONDP] = R[R_CONDP].volc[iwa] / dn;
        d[SALSA_DIAG_AICOLL] = a3 / dn;
        d[SALSA_DIAG_ICEHOM] = R[R_ICEHOM].numc / dn;
        d[SALSA_DIAG_ICEDEP] = R[R_ICEDEP].numc / dn;
        d[SALSA_DIAG_ICEIMM] = R[R_ICEIMM].numc / dn;
        d[SALSA_DIAG_CONDI] = (R[R_CONDI].volc[iwa] * c->rhoic + R[R_CONDI].volc[irim] * c->rhori) / dn;
        d[SALSA_DIAG_SIPDRFR] = R[R_SIPDRFR].numc / dn;                     /* :412-416 */
        d[SALSA_DIAG_SIPRMSPL] = R[R_SIPRMSPL].numc / dn;
        d[SALSA_DIAG_SIPIIBR] = R[R_SIPIIBR].numc / dn;
        int nd = (level == 5) ? (g->lssecice.sw ? SALSA_NDIAG : SALSA_DIAG_CONDI + 1) : SALSA_DIAG_AICOLL;
        for (int i = 0; i < nd; i++) if (f->diag[i]) f->diag[i][p] = d[i];
      }
      if (carry_over) { memcpy(c->carry, w->all, sizeof(Section) * c->ntotal); c->carry_valid = 1; }
      s_eq += w->f_equil; s_di += w->f_distr; s_nf += w->f_negfrac; s_co += w->f_cond; s_ng += w->f_neg;
      for (int i = 0; i < 5; i++) cnt[i] += w->cnt[i];
      ncell++;
    }
    free(w);
  }
  for (int i = 0; i < 5; i++) c->counters[i] = cnt[i];
  salsa_status_t loc;
  memset(&loc, 0, sizeof loc);
  loc.n_cells = ncell; loc.n_equil_nonconv = s_eq; loc.n_distr_nonconv = s_di; loc.n_distr_negfrac = s_nf;
  loc.n_cond_substeps = s_co; loc.n_negative = s_ng; loc.n_nonfinite = s_nan;
  loc.code = (s_eq || s_di || s_nf || s_nan) ? SALSA_E_NUMERIC : SALSA_OK;
  if (st) *st = loc;
  return loc.code;
}

/* ======================================================================
 * LES-side constraints after the step: src/src_LES/constrain_SALSA.f90
 * ====================================================================== */

/* tend_constrain2 (:18-35) over every element of the SALSA_4d tracers (halos included) */
int salsa_ref_tend_constrain(salsa_ref_ctx_t *c, int nzp, int nxp, int nyp, double dtlt,
                             const salsa_post_fields_t *f) {
  if (!c || !f || nzp < 3 || nxp < 5 || nyp < 5 || !(dtlt > 0.)) return SALSA_E_ARG;
  const salsa_config_t *g = &c->cfg;
  const long long plane = (long long)nzp * nxp * nyp;
  const int nw = c->nwet, lvl5 = g->level == 5;
  double *vp[9] = {f->naero, f->maero, f->ncloud, f->mcloud, f->nprecp, f->mprecp, f->gaero,
                   lvl5 ? f->nice : NULL, lvl5 ? f->mice : NULL};
  double *vt[9] = {f->naerot, f->maerot, f->ncloudt, f->mcloudt, f->nprecpt, f->mprecpt, f->gaerot,
                   lvl5 ? f->nicet : NULL, lvl5 ? f->micet : NULL};
  const long long np[9] = {c->nbins, (long long)nw * c->nbins, c->ncld, (long long)nw * c->ncld, c->nprc,
                           (long long)nw * c->nprc, 5, c->nice, (long long)(nw + 1) * c->nice};
  for (int a = 0; a < 9; a++) {
    if (!vp[a] || !vt[a]) continue;
    const long long n = np[a] * plane;
    for (long long e = 0; e < n; e++) vt[a][e] = fmaxd((-1. + 1.e-8) * vp[a][e] / dtlt, vt[a][e]);
  }
  if (g->ice_theta_dist && g->level > 4 && f->indef) {
    const long long n = (long long)c->nliquid * plane;
    for (long long e = 0; e < n; e++) f->indef[e] = fmind(fmaxd(f->indef[e], 0.), 1.);
  }
  return SALSA_OK;
}

/* util.f90:1005-1024 calc_correlation, as written: sxy keeps only the last product */
static double calc_correlation(const double *x, const double *y, int n) {
  const double eps = EPSR;
  double sx = 0., sy = 0., sx2 = 0., sy2 = 0., sxy = 0.;
  for (int i = 0; i < n; i++) {
    sx = sx + x[i];
    sy = sy + y[i];
    sx2 = sx2 + sq(x[i]);
    sy2 = sy2 + sq(y[i]);
    sxy = x[i] * y[i];
  }
  if (sx2 * n - sq(sx) < eps || sy2 * n - sq(sy) < eps) return 0.;
  return (sxy * n - sx * sy) / (sqrt(sx2 * n - sq(sx)) * sqrt(sy2 * n - sq(sy)));
}

/* :376-463 findDry4Wet: the aerosol bin for evaporating drops or ice of bin ib at point p
   (mevap species-major with nb bins).  The b bin is taken as fn2a + (ba - in2a), as the
   reference writes it. */
static int findDry4Wet(const salsa_ref_ctx_t *c, const double *aetot, const double *nevap, const double *mevap,
                       int nb, int ib, long long p, long long plane, const double *naero, const double *maero) {
  const int ndry = c->ndry, nbins = c->nbins, in2a = c->in2a, fn2a = c->fn2a;
  double cd = 0.;
  for (int s = 0; s < ndry; s++) cd += mevap[p + plane * ((long long)s * nb + ib)] / c->rholiq[s];
  cd = cd / nevap[p + plane * ib];
  cd = pow(cd / PI6, 1. / 3.);
  int cnt = 0;
  for (int b = in2a; b <= fn2a; b++) cnt += cd > aetot[b];
  int ba = in2a + cnt - 1;
  if (ba < in2a) ba = in2a;
  if (ba > fn2a) ba = fn2a;
  const int bb = fn2a + (ba - in2a);
  if (naero[p + plane * bb] <= NLIM) return ba;
  if (naero[p + plane * ba] <= NLIM) return bb;
  double xa[NSP], xb[NSP], y[NSP];
  for (int s = 0; s < ndry; s++) {
    xa[s] = maero[p + plane * ((long long)s * nbins + ba)];
    xb[s] = maero[p + plane * ((long long)s * nbins + bb)];
    y[s] = mevap[p + plane * ((long long)s * nb + ib)];
  }
  const double ra = calc_correlation(xa, y, ndry), rb = calc_correlation(xb, y, ndry);
  return ra < rb ? bb : ba;
}

/* :52-370 SALSA_diagnostics */
int salsa_ref_diagnostics(salsa_ref_ctx_t *c, int nzp, int nxp, int nyp, int only_diag, int lcharge,
                          const salsa_post_fields_t *f) {
  if (!c || !f || nzp < 3 || nxp < 5 || nyp < 5) return SALSA_E_ARG;
  const salsa_config_t *g = &c->cfg;
  const int lvl5 = g->level == 5;
  if (!f->naero || !f->ncloud || !f->nprecp || !f->maero || !f->mcloud || !f->mprecp || !f->rp || !f->rc ||
      !f->srp || !f->snrp || !f->rtot)
    return SALSA_E_ARG;
  if (lvl5 && (!f->nice || !f->mice || !f->ri || !f->riri)) return SALSA_E_ARG;
  if (!only_diag && (!f->rh || !f->temp || (lvl5 && !f->rhi) || (lcharge && !f->chargeTime) ||
                     (g->lscndgas && !f->gaero)))
    return SALSA_E_ARG;
  const long long plane = (long long)nzp * nxp * nyp;
  const int nbins = c->nbins, ncld = c->ncld, nprc = c->nprc, nice = c->nice, nspec = c->nwet, ndry = c->ndry;
  const int iwa = c->iwa, irim = c->irim;
  const double massTH = 1.e-25;
  double aetot[MAXB];
  for (int b = 0; b < nbins; b++) aetot[b] = pow(c->tmpl[b].vlolim / PI6, 1. / 3.);   /* aerobins */
  double *na = f->naero, *nc = f->ncloud, *np = f->nprecp, *ni = f->nice;
  double *ma = f->maero, *mc = f->mcloud, *mp = f->mprecp, *mi = f->mice;
#define AT(arr, nb, s, b) (arr)[p + plane * ((long long)(s) * (nb) + (b))]
  /* remove negative values */
  {
    double *arr[8] = {na, nc, np, ma, mc, mp, lvl5 ? ni : NULL, lvl5 ? mi : NULL};
    const long long n[8] = {nbins, ncld, nprc, (long long)nspec * nbins, (long long)nspec * ncld,
                            (long long)nspec * nprc, nice, (long long)(nspec + 1) * nice};
    for (int a = 0; a < 8; a++)
      if (arr[a])
        for (long long e = 0; e < n[a] * plane; e++) arr[a][e] = fmaxd(0., arr[a][e]);
  }
  if (!only_diag) {
    for (int j = 2; j <= nyp - 3; j++)
      for (int i = 2; i <= nxp - 3; i++)
        for (int k = 0; k < nzp; k++) {
          const long long p = k + (long long)nzp * (i + (long long)nxp * j);
          /* particles with number but no mass */
          for (int bc = 0; bc < nbins; bc++) {
            double sm = 0.;
            for (int s = 0; s < nspec; s++) sm += AT(ma, nbins, s, bc);
            if (na[p + plane * bc] > 0. && sm <= 0.) {
              na[p + plane * bc] = 0.;
              for (int s = 0; s < nspec; s++) AT(ma, nbins, s, bc) = 0.;
              if (lcharge) f->chargeTime[p + plane * bc] = 0.;
            }
          }
          for (int bc = 0; bc < ncld; bc++) {
            double sm = 0.;
            for (int s = 0; s < nspec; s++) sm += AT(mc, ncld, s, bc);
            if (nc[p + plane * bc] > 0. && sm <= 0.) {
              nc[p + plane * bc] = 0.;
              for (int s = 0; s < nspec; s++) AT(mc, ncld, s, bc) = 0.;
              if (lcharge) f->chargeTime[p + plane * (nbins + bc)] = 0.;
            }
          }
          for (int bc = 0; bc < nprc; bc++) {
            if (np[p + plane * bc] > 0. && AT(mp, nprc, iwa, bc) <= 0.) {
              np[p + plane * bc] = 0.;
              for (int s = 0; s < nspec; s++) AT(mp, nprc, s, bc) = 0.;
              if (lcharge) f->chargeTime[p + plane * (nbins + ncld + bc)] = 0.;
            }
          }
          if (lvl5)
            for (int bc = 0; bc < nice; bc++) {
              const double mt = AT(mi, nice, iwa, bc) + AT(mi, nice, irim, bc);
              if (ni[p + plane * bc] > 0. && mt < massTH) {
                ni[p + plane * bc] = 0.;
                for (int s = 0; s < nspec + 1; s++) AT(mi, nice, s, bc) = 0.;
              }
            }
          const double T = f->temp[p], rh = f->rh[p];
          /* evaporating cloud droplets */
          for (int bc = c->ica_cur; bc <= c->fcb_cur; bc++) {
            const double n_ = nc[p + plane * bc];
            if (n_ > NLIM && rh < 0.999 && AT(mc, ncld, iwa, bc) < 1.e-5) {
              double ns = 0.;
              for (int s = 0; s < nspec - 1; s++) ns += c->diss[s] * AT(mc, ncld, s, bc) / c->MM[s];
              ns = ns / n_;
              const double zbb = 6. * c->mwa * ns / (PI * c->rhowa);
              const double zaa = 4. * c->mwa * SURFW0 / (RG * c->rhowa * T);
              const double cdcld = sqrt(3. * zbb / zaa);
              double zvol = 0.;
              for (int s = 0; s < nspec; s++) zvol += AT(mc, ncld, s, bc) / c->rholiq[s];
              zvol = zvol / n_;
              const double zdh2o = pow(zvol / PI6, 1. / 3.);
              if (zdh2o < fmind(0.7 * cdcld, 1.3e-5) || AT(mc, ncld, iwa, bc) < massTH * n_) {
                const int ba = bc <= c->fca_cur ? c->ica_par + (bc - c->ica_cur) : c->icb_par + (bc - c->icb_cur);
                na[p + plane * ba] = na[p + plane * ba] + n_;
                nc[p + plane * bc] = 0.;
                for (int s = 0; s < nspec; s++) {
                  AT(ma, nbins, s, ba) = AT(ma, nbins, s, ba) + AT(mc, ncld, s, bc);
                  AT(mc, ncld, s, bc) = 0.;
                }
                if (lcharge) f->chargeTime[p + plane * (nbins + bc)] = 0.;
              }
            }
          }
          /* evaporating drops */
          for (int bc = 0; bc < nprc; bc++) {
            const double n_ = np[p + plane * bc];
            if (n_ > PRLIM && rh < 0.999 && AT(mp, nprc, iwa, bc) < 1.e-6) {
              double ns = 0.;
              for (int s = 0; s < nspec - 1; s++) ns += c->diss[s] * AT(mp, nprc, s, bc) / c->MM[s];
              ns = ns / n_;
              const double zbb = 6. * c->mwa * ns / (PI * c->rhowa);
              const double zaa = 4. * c->mwa * SURFW0 / (RG * c->rhowa * T);
              const double cdprc = sqrt(3. * zbb / zaa);
              double zvol = 0.;
              for (int s = 0; s < nspec; s++) zvol += AT(mp, nprc, s, bc) / c->rholiq[s];
              zvol = zvol / n_;
              const double zdh2o = pow(zvol / PI6, 1. / 3.);
              if (zdh2o < fmind(0.2 * cdprc, 10.e-6) || AT(mp, nprc, iwa, bc) < massTH * n_) {
                const int ba = findDry4Wet(c, aetot, np, mp, nprc, bc, p, plane, na, ma);
                na[p + plane * ba] = na[p + plane * ba] + n_;
                np[p + plane * bc] = 0.;
                for (int s = 0; s < nspec; s++) {
                  AT(ma, nbins, s, ba) = AT(ma, nbins, s, ba) + AT(mp, nprc, s, bc);
                  AT(mp, nprc, s, bc) = 0.;
                }
                if (lcharge) f->chargeTime[p + plane * (nbins + ncld + bc)] = 0.;
              }
            }
          }
          /* evaporating ice */
          if (lvl5)
            for (int bc = 0; bc < nice; bc++) {
              const double mt = AT(mi, nice, iwa, bc) + AT(mi, nice, irim, bc);
              double vt = 0.;
              for (int s = 0; s < nspec + 1; s++) vt += AT(mi, nice, s, bc) / c->rhoice[s];
              const double n_ = ni[p + plane * bc];
              if (n_ > PRLIM && f->rhi[p] < 0.999 && mt < 1.e-15) {
                double cdice = vt / n_;
                cdice = pow(cdice / PI6, 1. / 3.);
                double zdrms = 0., zwams = 0.;
                for (int s = 0; s < ndry; s++) zdrms += AT(mi, nice, s, bc);
                for (int s = 0; s < nspec + 1; s++) zwams += AT(mi, nice, s, bc);
                const double zvol = zdrms / zwams;
                if (zvol > 0.5 || cdice < 2.e-6) {
                  const int ba = findDry4Wet(c, aetot, ni, mi, nice, bc, p, plane, na, ma);
                  na[p + plane * ba] = na[p + plane * ba] + n_;
                  ni[p + plane * bc] = 0.;
                  for (int s = 0; s < nspec; s++) {
                    AT(ma, nbins, s, ba) = AT(ma, nbins, s, ba) + AT(mi, nice, s, bc);
                    AT(mi, nice, s, bc) = 0.;
                  }
                  AT(ma, nbins, iwa, ba) = AT(ma, nbins, iwa, ba) + AT(mi, nice, irim, bc);
                  AT(mi, nice, irim, bc) = 0.;
                }
              }
            }
          /* aerosol bins below 0.1 nm dry diameter */
          for (int ba = 0; ba < nbins; ba++) {
            const double n_ = na[p + plane * ba];
            if (n_ > NLIM) {
              double zvol = 0.;
              for (int s = 0; s < nspec - 1; s++) zvol += AT(ma, nbins, s, ba) / c->rholiq[s];
              zvol = zvol / n_;
              if (zvol < PI6 * cube(1.e-10)) {
                if (g->lscndgas) {
                  const int ix[4] = {c->idx_name[0], c->idx_name[1], c->idx_name[5], c->idx_name[6]};
                  const int gi[4] = {0, 4, 1, 2};   /* SO4 -> 1, OC -> 5, NO -> 2, NH -> 3 */
                  for (int q = 0; q < 4; q++)
                    if (ix[q] >= 0)
                      f->gaero[p + plane * gi[q]] = f->gaero[p + plane * gi[q]] + AT(ma, nbins, ix[q], ba) / c->MM[ix[q]] * AVOG;
                }
                for (int s = 0; s < nspec; s++) AT(ma, nbins, s, ba) = 0.;
                na[p + plane * ba] = 0.;
              }
            }
          }
        }
  }
  /* water diagnostics, every point */
  for (long long p = 0; p < plane; p++) {
    double rc = 0., srp = 0., snrp = 0.;
    for (int b = c->in1a; b <= c->fn2b; b++) rc += AT(ma, nbins, iwa, b);
    double rcc = 0.;
    for (int b = c->ica_cur; b <= c->fcb_cur; b++) rcc += AT(mc, ncld, iwa, b);
    rc = rc + rcc;
    for (int b = 0; b < nprc; b++) srp += AT(mp, nprc, iwa, b);
    for (int b = 0; b < nprc; b++) snrp += np[p + plane * b];
    f->rc[p] = rc;
    f->srp[p] = srp;
    f->snrp[p] = snrp;
    double rt = rc + srp + f->rp[p];
    if (lvl5) {
      double ri = 0., riri = 0.;
      for (int b = 0; b < nice; b++) ri += AT(mi, nice, iwa, b);
      for (int b = 0; b < nice; b++) riri += AT(mi, nice, irim, b);
      f->ri[p] = ri;
      f->riri[p] = riri;
      rt = rt + ri + riri;
    }
    f->rtot[p] = rt;
  }
#undef AT
  return SALSA_OK;
}

/* ======================================================================
 * Sedimentation: src/src_LES/mcrp.f90:745-1275 (sedim_SALSA, DepositionSlow,
 * DepositionFast).  Indices below are 0-based: level kc is the reference's k = kc + 1.
 * The LES constants of defs.f90 (full-precision pi among them) sit beside the SALSA
 * ones (pi6 of mo_submctl) as in the reference.
 * ====================================================================== */
#define LES_ALVL 2.5e+06
#define LES_ALVI 2.834e+06
#define LES_CP   1005.
#define LES_G    9.81
#define LES_KB   1.3807e-23
#define SED_M    4.8096e-26
#define SED_A    1.249
#define SED_B    0.42
#define SED_C    0.87

/* calcDiamLES (mo_particle_external_properties.f90:169-201), spherical */
static double calc_diam_les(const salsa_ref_ctx_t *c, int ns, double numc, const double *mass, int flag) {
  if (numc < 1.e-15) return 0.;
  double v = 0.;
  for (int s = 0; s < ns; s++) v += mass[s] / (flag == 4 ? c->rhoice[s] : c->rholiq[s]);
  return pow(v / numc / PI6, 1. / 3.);
}

/* per-level air properties (atm modelling eq. 4.54) */
static void sed_air(double T, double adn, double *avis, double *kvis, double *lambda) {
  *avis = 1.8325e-5 * (416.16 / (T + 120.0)) * pow(T / 296.16, 1.5);
  *kvis = *avis / adn;
  const double va = sqrt(8. * LES_KB * T / (PI_FULL * SED_M));
  *lambda = 2. * *avis / (adn * va);
}

/* DepositionSlow (:926-1069) for nb bins of ns species; tendencies, tlt and the rates
   are updated as sedim_SALSA does after the call (:790-835) */
static void dep_slow(const salsa_ref_ctx_t *c, int nzp, int nxp, int nyp, double dtlt, int nb, int ns, int flag,
                     const double *numc, const double *mass, double *tn, double *tm, const salsa_sedim_fields_t *f) {
  const long long plane = (long long)nzp * nxp * nyp;
  const double clim = (flag == 3 || flag == 4) ? PRLIM : NLIM;
  const int iw = ns - 1;   /* water: the last of the wet species */
  double *rflm = (double *)calloc((size_t)nzp * nb * ns, sizeof(double));
  double *rfln = (double *)calloc((size_t)nzp * nb, sizeof(double));
  double *divm = (double *)calloc((size_t)nzp * nb * ns, sizeof(double));
  double *divn = (double *)calloc((size_t)nzp * nb, sizeof(double));
  double pmass[NSP];
  for (int j = 2; j <= nyp - 3; j++)
    for (int i = 2; i <= nxp - 3; i++) {
      memset(rflm, 0, sizeof(double) * nzp * nb * ns);
      memset(rfln, 0, sizeof(double) * nzp * nb);
      memset(divm, 0, sizeof(double) * nzp * nb * ns);
      memset(divn, 0, sizeof(double) * nzp * nb);
      const long long col = (long long)nzp * (i + (long long)nxp * j);
      for (int kc = nzp - 2; kc >= 1; kc--) {
        const long long p = col + kc;
        const int kp1 = kc + 1;
        const double T = f->tk[p], ad = f->adn[p];
        double avis, kvis, lambda;
        sed_air(T, ad, &avis, &kvis, &lambda);
        for (int bin = 0; bin < nb; bin++) {
          const double n = numc[p + plane * bin];
          if (n < clim) continue;
          for (int s = 0; s < ns; s++) pmass[s] = mass[p + plane * ((long long)s * nb + bin)];
          const double dwet = calc_diam_les(c, ns, n, pmass, flag);
          double sm = 0.;
          for (int s = 0; s < ns; s++) sm += pmass[s];
          const double zdn = sm / n / (PI6 * cube(dwet));
          const double Kn = 2. * lambda / dwet;
          const double GG = 1. + Kn * (SED_A + SED_B * exp(-SED_C / Kn));
          double vc = terminal_vel(dwet, zdn, ad, avis, GG, flag, NULL, 0.);
          vc = fmind(vc, fmind(0.5 * (1. / f->dzt[kc]) / dtlt, 2.0));
          if (kc == 1) {   /* the level just above the surface */
            const double mdiff = (LES_KB * T * GG) / (3.0 * PI_FULL * avis * dwet);
            const double Sc = kvis / mdiff;
            double St = vc * pow(f->ustar[i + (long long)nxp * j], 2.0) / LES_G * kvis;
            if (St < 0.01) St = 0.01;
            const double rt = 1.0 / fmaxd(EPSR, (f->ustar[i + (long long)nxp * j] *
                                                 (pow(Sc, -2.0 / 3.0) + pow(10., -3.0 / St))));
            vc = (1. / rt) + vc;
          }
          for (int s = 0; s < ns; s++) rflm[(long long)kc * nb * ns + s * nb + bin] = -pmass[s] * vc;
          rfln[kc * nb + bin] = -n * vc;
        }
        const double adp = f->adn[p + 1];
        for (int e = 0; e < nb * ns; e++)
          divm[(long long)kc * nb * ns + e] = (rflm[(long long)kp1 * nb * ns + e] * adp - rflm[(long long)kc * nb * ns + e] * ad) *
                                              f->dzt[kc] / ad;
        for (int e = 0; e < nb; e++)
          divn[kc * nb + e] = (rfln[kp1 * nb + e] * adp - rfln[kc * nb + e] * ad) * f->dzt[kc] / ad;
        double sw = 0.;   /* SUM(rflm(k,(ns-1)*nb:ns*nb)), 1-based as written */
        for (int e = iw * nb - 1; e <= ns * nb - 1; e++) sw += rflm[(long long)kc * nb * ns + e];
        f->rrate[p] = f->rrate[p] - sw * ad * LES_ALVL;
      }
      {
        double sw = 0.;
        for (int e = iw * nb - 1; e <= ns * nb - 1; e++) sw += rflm[(long long)1 * nb * ns + e];
        const long long q = i + (long long)nxp * j;
        f->sfcrrate[q] = f->sfcrrate[q] - sw * f->adn[col + 1] * LES_ALVL;
      }
      for (int kc = 1; kc <= nzp - 2; kc++) {
        const long long p = col + kc;
        for (int b = 0; b < nb; b++) tn[p + plane * b] = tn[p + plane * b] - divn[kc * nb + b];
        for (int e = 0; e < nb * ns; e++) tm[p + plane * e] = tm[p + plane * e] - divm[(long long)kc * nb * ns + e];
      }
      for (int kc = 1; kc <= nzp - 1; kc++) {   /* k = 2 .. nzp */
        const long long p = col + kc;
        double sw = 0.;
        for (int b = 0; b < nb; b++) sw += divm[(long long)kc * nb * ns + iw * nb + b];
        f->tlt[p] = f->tlt[p] + sw * (LES_ALVL / LES_CP) * f->th[p] / f->tk[p];
      }
    }
  free(rflm); free(rfln); free(divm); free(divn);
}

/* DepositionFast (:1073-1275) for nb bins of ns species, then sedim_SALSA's updates
   (:840-905): tendencies += change / dtlt over the whole arrays, tlt */
static void dep_fast(const salsa_ref_ctx_t *c, int nzp, int nxp, int nyp, double dtlt, int nb, int ns, int flag,
                     const double *numc, const double *mass, double *tn, double *tm, double *rate, double *srate,
                     double *Vt, const salsa_sedim_fields_t *f) {
  const long long plane = (long long)nzp * nxp * nyp;
  const double clim = (flag == 3 || flag == 4) ? PRLIM : NLIM;
  double *prnt = (double *)calloc((size_t)(plane * nb), sizeof(double));
  double *prvt = (double *)calloc((size_t)(plane * nb * ns), sizeof(double));
  double *prnchg = (double *)calloc((size_t)nzp * nb, sizeof(double));
  double *prvchg = (double *)calloc((size_t)nzp * nb * ns, sizeof(double));
  double *remprc = (double *)calloc((size_t)nb * ns, sizeof(double));
  double pmass[NSP];
  for (long long e = 0; e < plane * nb; e++) Vt[e] = 0.;
  for (int j = 2; j <= nyp - 3; j++)
    for (int i = 2; i <= nxp - 3; i++) {
      memset(prnchg, 0, sizeof(double) * nzp * nb);
      memset(prvchg, 0, sizeof(double) * nzp * nb * ns);
      memset(remprc, 0, sizeof(double) * nb * ns);
      const long long col = (long long)nzp * (i + (long long)nxp * j);
      for (int kc = nzp - 2; kc >= 1; kc--) {
        const long long p = col + kc;
        const double T = f->tk[p], ad = f->adn[p];
        double avis, kvis, lambda;
        sed_air(T, ad, &avis, &kvis, &lambda);
        (void)kvis;
        for (int bin = 0; bin < nb; bin++) {
          const double n = numc[p + plane * bin];
          if (n < clim) continue;
          for (int s = 0; s < ns; s++) pmass[s] = mass[p + plane * ((long long)s * nb + bin)];
          const double dwet = calc_diam_les(c, ns, n, pmass, flag);
          double dnsp = 0.;
          Shape shape;
          if (flag == 4) {
            double mp = 0.;
            for (int s = 0; s < ns - 1; s++) mp += pmass[s];
            dnsp = getDiameter(c, mp, pmass[ns - 1], n);   /* calcDiamLES(sph=.FALSE.) */
            getShapeCoefficients(c, &shape, mp, pmass[ns - 1], n);
          }
          double sm = 0.;
          for (int s = 0; s < ns; s++) sm += pmass[s];
          const double zdn = sm / n / (PI6 * cube(dwet));
          const double Kn = 2. * lambda / dwet;
          const double GG = 1. + Kn * (SED_A + SED_B * exp(-SED_C / Kn));
          const double vc = flag < 4 ? terminal_vel(dwet, zdn, ad, avis, GG, flag, NULL, 0.)
                                     : terminal_vel(dwet, zdn, ad, avis, GG, flag, &shape, dnsp);
          Vt[p + plane * bin] = vc;
          const double fdmax = dtlt * vc;
          double fd = 0.;
          int fi = 0, prcdep = 0;
          while (fd < fdmax) {
            fd = fd + (1. / f->dzt[kc - fi]);
            fi = fi + 1;
            if (kc - fi <= 0) { prcdep = 1; break; }
          }
          fi = fi - 1;
          const int kf = kc - fi;
          fd = fd - (1. / f->dzt[kf]);
          const double fdos = fmind(fmaxd(fdmax - fd, 0.), 1. / f->dzt[kf]);
          const double prnumc = n;
          prnchg[kc * nb + bin] = prnchg[kc * nb + bin] - prnumc;
          for (int ni = 0; ni < ns; ni++) {
            pmass[ni] = mass[p + plane * ((long long)ni * nb + bin)];
            prvchg[((long long)kc * nb + bin) * ns + ni] = prvchg[((long long)kc * nb + bin) * ns + ni] - pmass[ni];
          }
          if (prcdep)
            for (int ni = 0; ni < ns; ni++) remprc[ni * nb + bin] = remprc[ni * nb + bin] + pmass[ni] * ad * vc;
          if (flag == 4)
            rate[p] = rate[p] + (mass[p + plane * ((long long)(ns - 2) * nb + bin)] +
                                 mass[p + plane * ((long long)(ns - 1) * nb + bin)]) * ad * vc * LES_ALVI;
          else
            rate[p] = rate[p] + mass[p + plane * ((long long)(ns - 1) * nb + bin)] * ad * vc * LES_ALVL;
          if (fdos * f->dzt[kf] > 0.5) {
            prnchg[(kf - 1) * nb + bin] = prnchg[(kf - 1) * nb + bin] + prnumc * f->dzt[kf - 1] / f->dzt[kc];
            for (int ni = 0; ni < ns; ni++) {
              double *q = &prvchg[((long long)(kf - 1) * nb + bin) * ns + ni];
              *q = *q + pmass[ni] * f->dzt[kf - 1] / f->dzt[kc];
            }
          } else {
            prnchg[(kf - 1) * nb + bin] = prnchg[(kf - 1) * nb + bin] + (fdos * f->dzt[kf]) * prnumc * f->dzt[kf - 1] / f->dzt[kf];
            prnchg[kf * nb + bin] = prnchg[kf * nb + bin] + (1. - fdos * f->dzt[kf]) * prnumc;
            for (int ni = 0; ni < ns; ni++) {
              double *q1 = &prvchg[((long long)(kf - 1) * nb + bin) * ns + ni];
              double *q0 = &prvchg[((long long)kf * nb + bin) * ns + ni];
              *q1 = *q1 + (fdos * f->dzt[kf]) * pmass[ni] * f->dzt[kf - 1] / f->dzt[kf];
              *q0 = *q0 + (1. - fdos * f->dzt[kf]) * pmass[ni];
            }
          }
        }
      }
      {
        const long long q = i + (long long)nxp * j;
        double sw = 0.;
        const int e0 = (flag == 4 ? (ns - 2) * nb : (ns - 1) * nb) - 1;
        for (int e = e0; e <= ns * nb - 1; e++) sw += remprc[e];
        srate[q] = srate[q] + sw * (flag == 4 ? LES_ALVI : LES_ALVL);
      }
      for (int kc = 0; kc < nzp; kc++) {
        const long long p = col + kc;
        for (int b = 0; b < nb; b++) prnt[p + plane * b] = prnt[p + plane * b] + prnchg[kc * nb + b];
        for (int ni = 0; ni < ns; ni++)
          for (int b = 0; b < nb; b++)
            prvt[p + plane * ((long long)ni * nb + b)] = prvt[p + plane * ((long long)ni * nb + b)] +
                                                          prvchg[((long long)kc * nb + b) * ns + ni];
      }
    }
  for (long long e = 0; e < plane * nb; e++) tn[e] = tn[e] + prnt[e] / dtlt;
  for (long long e = 0; e < plane * nb * ns; e++) tm[e] = tm[e] + prvt[e] / dtlt;
  const int w0 = (flag == 4 ? ns - 2 : ns - 1) * nb, w1 = ns * nb;   /* water (and rime) bins */
  const double lat = flag == 4 ? LES_ALVI : LES_ALVL;
  for (int j = 2; j <= nyp - 3; j++)
    for (int i = 2; i <= nxp - 3; i++)
      for (int kc = 0; kc <= nzp - 2; kc++) {
        const long long p = kc + (long long)nzp * (i + (long long)nxp * j);
        double sw = 0.;
        for (int e = w0; e < w1; e++) sw += prvt[p + plane * e];
        f->tlt[p] = f->tlt[p] - (sw / dtlt) * (lat / LES_CP) * f->th[p] / f->tk[p];
      }
  free(prnt); free(prvt); free(prnchg); free(prvchg); free(remprc);
}

int salsa_ref_sedimentation(salsa_ref_ctx_t *c, int nzp, int nxp, int nyp, double dtlt, const int sed[4],
                            const salsa_sedim_fields_t *f) {
  if (!c || !f || !sed || nzp < 3 || nxp < 5 || nyp < 5 || !(dtlt > 0.)) return SALSA_E_ARG;
  const int lvl5 = c->cfg.level == 5, nspec = c->nwet;
  if (!f->tk || !f->th || !f->adn || !f->ustar || !f->dzt || !f->tlt || !f->rrate || !f->sfcrrate) return SALSA_E_ARG;
  if ((sed[0] && (!f->naero || !f->maero || !f->naerot || !f->maerot)) ||
      (sed[1] && (!f->ncloud || !f->mcloud || !f->ncloudt || !f->mcloudt)) ||
      (sed[2] && (!f->nprecp || !f->mprecp || !f->nprecpt || !f->mprecpt || !f->VtPrc)) ||
      (sed[3] && lvl5 && (!f->nice || !f->mice || !f->nicet || !f->micet || !f->VtIce)))
    return SALSA_E_ARG;
  const long long plane = (long long)nzp * nxp * nyp, area = (long long)nxp * nyp;
  for (long long e = 0; e < plane; e++) f->rrate[e] = 0.;
  for (long long e = 0; e < area; e++) f->sfcrrate[e] = 0.;
  if (lvl5) {
    if (!f->irate || !f->sfcirate) return SALSA_E_ARG;
    for (long long e = 0; e < plane; e++) f->irate[e] = 0.;
    for (long long e = 0; e < area; e++) f->sfcirate[e] = 0.;
  }
  if (sed[0]) dep_slow(c, nzp, nxp, nyp, dtlt, c->nbins, nspec, 1, f->naero, f->maero, f->naerot, f->maerot, f);
  if (sed[1]) dep_slow(c, nzp, nxp, nyp, dtlt, c->ncld, nspec, 2, f->ncloud, f->mcloud, f->ncloudt, f->mcloudt, f);
  if (sed[2])
    dep_fast(c, nzp, nxp, nyp, dtlt, c->nprc, nspec, 3, f->nprecp, f->mprecp, f->nprecpt, f->mprecpt, f->rrate,
             f->sfcrrate, f->VtPrc, f);
  if (sed[3] && lvl5)
    dep_fast(c, nzp, nxp, nyp, dtlt, c->nice, nspec + 1, 4, f->nice, f->mice, f->nicet, f->micet, f->irate,
             f->sfcirate, f->VtIce, f);
  return SALSA_OK;
}
