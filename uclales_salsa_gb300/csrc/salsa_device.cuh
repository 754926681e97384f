// salsa_device.cuh -- device-side definitions of the GB300 SALSA step.
//
// One warp advances one grid cell through the SALSA process chain of
// UCLALES-SALSA (src/src_salsa/mo_salsa.f90:45-153); lanes split the bins and
// the bin pairs.  A block of SALSA_CPG warps owns SALSA_CPG consecutive cells so
// that every 32-byte sector of the bin-major input planes is used in full.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

#define SALSA_CPG 4                 // cells (= warps) per block
#define SALSA_THREADS (32 * SALSA_CPG)
#define SALSA_NSV 7                 // volume slots per bin (dry species + water + rime)
#define SALSA_MAXNB 96

// ---- constants: src/src_shared/mo_submctl.f90:253-338 (truncated values as written) ----
#define K_AVOG 6.0221e+23
#define K_BOLTZ 1.3807e-23
#define K_PLANCK 6.626070040e-34
#define K_GRAV 9.81
#define K_PSTAND 1.01325e+5
#define K_RG 8.314
#define K_PI 3.1415927
#define K_PI6 0.5235988
#define K_MAIR 28.97e-3
#define K_CPA 1005.
#define K_EPS 2.220446049250313e-16
#define K_RD 287.04
#define K_ALV 2.5e6
#define K_ALS 2.834e6
#define K_SURFW0 0.073
#define K_SURFI0 0.105
#define K_EPSOC 0.15
#define K_NLIM 1.0
#define K_PRLIM 1.e-6
#define K_MWA 18.016e-3
#define K_RHOWA 1000.
#define K_RHOIC 917.
#define K_RHORI 400.
#define K_MVWA (K_MWA / K_AVOG / K_RHOWA)
#define K_PI_FULL 3.14159265358979323846
// condensing vapours (mo_submctl.f90:284-322): molar masses, densities, molecular volumes
#define K_MSU 98.08e-3
#define K_MVSU (98.08e-3 / K_AVOG / 1830.)
#define K_MVOC (150.e-3 / K_AVOG / 1400.)
#define K_DSA 5.539376964394570e-10
#define K_N3 158.79
#define K_MASSACC 1.   // mass accommodation coefficient of every aerosol bin (mo_salsa_init.f90:818-820)

namespace salsa {

// input field ids (index into DevParams::fin)
enum {
  FI_PRESS = 0, FI_TEMP, FI_RSL, FI_RSI, FI_RP, FI_DN, FI_WP, FI_KAPPA,
  FI_NAERO, FI_NCLOUD, FI_NPRECP, FI_NICE, FI_MAERO, FI_MCLOUD, FI_MPRECP, FI_MICE,
  FI_INDEF, FI_CHARGE, FI_GAERO, FI_SIPDRFR, FI_SIPRMSPL, FI_SIPIIBR, FI_N
};
// output field ids (index into DevParams::fout)
enum {
  FO_RPT = 0, FO_NAEROT, FO_NCLOUDT, FO_NPRECPT, FO_NICET, FO_MAEROT, FO_MCLOUDT, FO_MPRECPT, FO_MICET,
  FO_INDEF, FO_CHARGE, FO_NACT, FO_VACT, FO_GAEROT, FO_SIPDRFR, FO_SIPRMSPL, FO_SIPIIBR, FO_DIAG0,
  FO_N = FO_DIAG0 + 20   // the diagnostics of the header's enum, the secondary-ice rates last
};
// row modes
enum { ROW_IN = 0, ROW_TEND = 1, ROW_INOUT = 2, ROW_OUT = 3 };

// raw slots of the thermodynamic inputs
enum { RW_P = 0, RW_T, RW_RS, RW_RSI, RW_RV, RW_DN, RW_W, RW_KAPPA, RW_NTHERMO };

// diagnostic accumulators (ordering follows include/salsa_gb300.h)
enum {
  DG_AUTOC = 0, DG_AUTOC80, DG_AUTOC50, DG_ACCR, DG_ACCR80, DG_ACCR50, DG_ACCOLL, DG_APCOLL, DG_ACTIV,
  DG_CONDA, DG_CONDC, DG_CONDP, DG_AICOLL, DG_ICEHOM, DG_ICEDEP, DG_ICEIMM, DG_CONDI, DG_N
};

// status counters
enum { ST_CELLS = 0, ST_EQUIL, ST_DISTR, ST_NEGFRAC, ST_COND, ST_NEG, ST_NONFINITE,
       ST_ORDER_CLEAR, ST_ORDER_CLOUDY,   // fill counters of the cell order list
       ST_N };

struct Row {
  int16_t fin;     // input field id or -1
  int16_t fout;    // output field id or -1
  int16_t idx;     // last-dimension index inside the field
  int16_t mode;    // ROW_*
};

struct DevParams {
  // grid
  int nzp, nxp, nyp, nz_int, nx_int;
  long long ncells, plane, ngroups;
  int level, lcharge, initialize;
  double dt;
  double inv_dt;   // 1/dt when dt is a power of two (the product then equals the quotient), else 0
  // layout
  int nbins, ncld, nprc, nice, ntotal, nliquid, nused, ndry, nwet, iwa, irim, nb_pad;
  int in1a, fn1a, in2a, fn2a, in2b, fn2b;
  int ica_cur, ica_par, fca_cur, icb_cur, icb_par, fcb_cur;
  int nsoluble, ninsoluble, ind_soluble[5], ind_insoluble[2];
  int ix_so4, ix_oc, ix_bc, ix_du, ix_ss, ix_no, ix_nh;
  double rholiq[9], rhoice[9], MM[9], diss[9];
  double irholiq[9], irhoice[9];   // reciprocal densities (the unit conversions multiply)
  int cnt80, cnt50;
  // effective switches for this call
  int st_coag, st_cnd, st_auto, st_activ, st_icenucl, st_icemelt, st_freeRH, st_freeTheta;
  int coag_mode, auto_mode, activ_mode, icenucl_mode;
  int lscgaa, lscgcc, lscgca, lscgpc, lscgpa, lscgpp, lscgia, lscgic, lscgii, lscgip;
  int lscndh2oae, lscndh2ocl, lscndh2oic, lsicehom, lsiceimm, lsicedep, ice_theta_dist, lsdistupdate;
  int has_kappa;
  int lscndgas, nsnucl;   // gas condensation; nucleation scheme (0: off)
  // kernel storage of lscoag%mode = 2: 0 compute, 1 compute and store, 2 fetch
  int kc_mode, kc_stride;  // kc_stride: kernel-type entries per cell (the kernel triangle)
  long long kc_base;       // storage index of the call's first cell (host-buffer slabs)
  void *kcache;
  double Eiagg_max, Eiagg_min, eddy_dis, rhlim, initMinTheta, chargeTimeMax, chargeCollEnh;
  double mean_theta_imm, sigma_theta_imm, mean_theta_dep, sigma_theta_dep;
  double iceShapeAlpha, iceShapeBeta, iceShapeGamma, iceShapeSigma;
  // workspace layout (doubles)
  int raw_num, raw_mbase[4], raw_indef, raw_charge, raw_nact, raw_vact, raw_diag, nraw;
  int raw_gas;         // first of the five gas rows (SO4, HNO3, NH3, OC non-volatile, OC semi-volatile), or -1
  int nrows;           // rows in the row table
  int npairs;          // collision pairs in the pair table
  int npairs_plain;    // pairs before the equal-size (self-coagulation offset) section
  int ws_doubles;      // per-warp workspace size
  int tab_doubles;     // per-block table size
  int list_off;        // offset (doubles) of the int16 partner lists inside the block table
  // pointers
  const double *fin[FI_N];
  double *fout[FO_N];
  const Row *rows;
  const double *tables;     // bin tables (see TAB_* offsets)
  const int *pairs;         // packed pair list (i | j << 8)
  unsigned long long *status;
  const int *order;         // processing order of the cells (clear cells first), or null
  unsigned long long *stage_clocks;   // per-stage clock sums (instrumented builds only)
  // secondary ice (mo_salsa_secondary_ice.f90): states of lssecice and the three schemes,
  // the schemes' modes, the first splinter bin (1-based, mo_salsa_SIP_RS.f90:72) and the
  // offset of the tally region inside each warp's workspace (doubles)
  int st_secice, st_siprs, st_sipdf, st_sipib;
  int sip_rs_mode, sip_df_mode, sip_ib_mode, sip_splbin, sip_off;
  int raw_sip;   // first of the 3 x nice tracer rows (sipdrfr, siprmspl, sipiibr), or -1
};

// block table layout (per bin, padded to nb_pad): offsets in units of nb_pad
enum { TAB_VLO = 0, TAB_VHI, TAB_VRLO, TAB_VRHI, TAB_DMID, TAB_PRECPBINS, TAB_N };

__device__ __forceinline__ double sq(double x) { return x * x; }
__device__ __forceinline__ float sq(float x) { return x * x; }
__device__ __forceinline__ double cube(double x) { return x * x * x; }
__device__ __forceinline__ float cube(float x) { return x * x * x; }

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}
__device__ __forceinline__ float warp_sum(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}
__device__ __forceinline__ int warp_any(bool b) { return __any_sync(0xffffffffu, b); }

// offset of interior cell q (z fastest, then x, then y) inside a (nyp, nxp, nzp) plane
__device__ __forceinline__ long long cell_offset(const DevParams &P, long long q) {
  long long kq = q % P.nz_int, r = q / P.nz_int;
  long long iq = r % P.nx_int, jq = r / P.nx_int;
  return (1 + kq) + (long long)P.nzp * ((2 + iq) + (long long)P.nxp * (2 + jq));
}
__device__ __forceinline__ long long cell_at(const DevParams &P, long long i) { return P.order ? P.order[i] : i; }

}  // namespace salsa
