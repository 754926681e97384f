// salsa_capi.cu -- host side of the C-ABI in include/salsa_gb300.h.
//
// salsa_gb300_init replaces define_salsa + salsa_initialize
// (src/src_salsa/mo_salsa_init.f90:465-637, 792-858): it validates the &salsa
// configuration, builds the species tables (src/src_shared/classSpecies.f90:167-341)
// and the bin layout (mo_salsa_init.f90:148-450), and uploads the per-block tables,
// the I/O row table and the collision-pair table to the GPU.
// salsa_gb300_run replaces run_SALSA (mo_salsa_driver.f90:112-435): it resolves the
// process-switch states (set_SALSA_runtime :445-474), stages host arrays when the
// caller passes host memory, and launches the fused step kernel.
#include <cuda_runtime.h>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <algorithm>
#include <cstring>
#include <vector>

#include "../../include/salsa_gb300.h"
#include "salsa_device.cuh"
#include "salsa_internal.h"

namespace salsa {
cudaError_t launch_d0(const DevParams &, cudaStream_t, int);
cudaError_t launch_d1(const DevParams &, cudaStream_t, int);
cudaError_t launch_f0(const DevParams &, cudaStream_t, int);
cudaError_t launch_f1(const DevParams &, cudaStream_t, int);
int blocks_per_sm_d0(const DevParams &);
int blocks_per_sm_d1(const DevParams &);
int blocks_per_sm_f0(const DevParams &);
int blocks_per_sm_f1(const DevParams &);
cudaError_t launch_ds(const DevParams &, cudaStream_t, int);
cudaError_t launch_fs(const DevParams &, cudaStream_t, int);
int blocks_per_sm_ds(const DevParams &);
int blocks_per_sm_fs(const DevParams &);
}  // namespace salsa

using salsa::DevParams;
using salsa::Row;

// Scratch of salsa_gb300_run_noalloc, the step for callers that cannot allocate GPU
// memory (their own pool holds it, or cudaMalloc's device-wide synchronisation would
// stall their time loop): the cell-order list and the status counters live in module
// memory.  SALSA_NOALLOC_MAXCELLS (header) bounds the interior cells of one call.
// Host code must not take these names as device addresses: salsa_gb300_init looks the
// addresses up with cudaGetSymbolAddress on the handle's device.
static __device__ __align__(256) int g_na_order[SALSA_NOALLOC_MAXCELLS];
static __device__ __align__(256) unsigned long long g_na_status[salsa::ST_N];

// Cell order of one step: cells whose cloud, precipitation and ice bins are all below
// the population limits fill the list from the front, the others from the back, so
// that the four cells of a block (which meet at barriers) take the same code path.
// Each warp claims its slots with one atomic per class; the order of the claims does
// not affect any result, since every cell is computed independently.
__global__ void salsa_order_kernel(const DevParams P, int *order) {
  const unsigned F = 0xffffffffu;
  const int lane = threadIdx.x & 31;
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long base = (long long)blockIdx.x * blockDim.x; base < P.ncells; base += stride) {
    const long long q = base + threadIdx.x;
    const bool act = q < P.ncells;
    bool cloudy = false;
    if (act) {
      const long long off = salsa::cell_offset(P, q);
      const double dn = __ldg(P.fin[salsa::FI_DN] + off);
      const int cat[3] = {salsa::FI_NCLOUD, salsa::FI_NPRECP, salsa::FI_NICE};
      const int nbc[3] = {P.ncld, P.nprc, P.level == 5 ? P.nice : 0};
      const double lim[3] = {K_NLIM, K_PRLIM, K_PRLIM};
      for (int c = 0; c < 3 && !cloudy; c++) {
        const double *f = P.fin[cat[c]];
        if (!f) continue;
        for (int b = 0; b < nbc[c]; b++)
          if (__ldg(f + off + P.plane * b) * dn >= lim[c]) { cloudy = true; break; }
      }
    }
    const unsigned mc = __ballot_sync(F, act && cloudy), ma = __ballot_sync(F, act && !cloudy);
    unsigned long long b0 = 0, b1 = 0;
    if (lane == 0) {
      if (ma) b0 = atomicAdd(P.status + salsa::ST_ORDER_CLEAR, (unsigned long long)__popc(ma));
      if (mc) b1 = atomicAdd(P.status + salsa::ST_ORDER_CLOUDY, (unsigned long long)__popc(mc));
    }
    b0 = __shfl_sync(F, b0, 0);
    b1 = __shfl_sync(F, b1, 0);
    const unsigned lt = (1u << lane) - 1u;
    if (act) {
      if (cloudy) order[P.ncells - 1 - (long long)(b1 + __popc(mc & lt))] = (int)q;
      else order[b0 + __popc(ma & lt)] = (int)q;
    }
  }
}

namespace {

const double PI6 = 0.5235988;   // mo_submctl.f90:266
const char *ALLNAMES[9] = {"SO4", "OC", "BC", "DU", "SS", "NO", "NH", "H2O", "rime"};
const double ALLMM[9] = {98.08e-3, 150.e-3, 12.e-3, 100.e-3, 58.44e-3, 62.01e-3, 18.04e-3, 18.016e-3, 18.016e-3};
const double ALLRHO[9] = {1830., 1400., 2000., 2650., 2165., 1479., 1530., 1000., 400.};
const double ALLDISS[9] = {3., 1., 0., 0., 2., 1., 1., 1., 1.};

bool name_eq(const char *a, const char *b) {
  char x[5] = {0}, y[5] = {0};
  strncpy(x, a, 4);
  strncpy(y, b, 4);
  for (int i = 3; i >= 0 && (x[i] == ' ' || x[i] == 0); i--) x[i] = 0;
  for (int i = 3; i >= 0 && (y[i] == ' ' || y[i] == 0); i--) y[i] = 0;
  return strcmp(x, y) == 0;
}

struct BinTab {
  std::vector<double> vlo, vhi, vrlo, vrhi, dmid;
};

void set_bin(BinTab &t, int b, double vlo, double vhi) {
  t.vlo[b] = vlo;
  t.vhi[b] = vhi;
  t.dmid[b] = std::pow((vhi + vlo) / (2. * PI6), 1. / 3.);
  double v = PI6 * t.dmid[b] * t.dmid[b] * t.dmid[b];
  t.vrhi[b] = vhi / v;
  t.vrlo[b] = vlo / v;
}

double hcube(double x) { return x * x * x; }

}  // namespace

// host-buffer pipeline: staging slots and the number of y-slabs a grid is cut into
#define SALSA_PIPE_SLOTS 3
#define SALSA_PIPE_SLABS 16

struct salsa_handle {
  salsa_config_t cfg;
  int device = 0, nsm = 0;
  DevParams base;               // layout part of the kernel parameters
  double *d_tables = nullptr;
  Row *d_rows = nullptr;
  int *d_pairs = nullptr;
  unsigned long long *d_status = nullptr;
  unsigned long long *h_status = nullptr;
  cudaStream_t stream = nullptr;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  std::vector<double> lolim_diam;
  // sticky switch states (set_SALSA_runtime)
  int st[7] = {0, 0, 0, 0, 0, 0, 0};
  int st_freeRH = 0, st_freeTheta = 0;
  int st_sip[3] = {0, 0, 0};    // lssiprimespln, lssipdropfrac, lssipicecollbreak
  // staging buffers for host-pointer calls
  void *stage = nullptr;
  size_t stage_bytes = 0;
  void *kcache = nullptr;       // kernel storage of lscoag%mode = 2
  size_t kcache_bytes = 0;
  cudaStream_t s_in = nullptr, s_out = nullptr;     // copy streams of the host-buffer pipeline
  cudaEvent_t pev[3 * SALSA_PIPE_SLOTS + 2] = {};   // its slot and start/end events
  int *d_order = nullptr;       // cell order list (salsa_order_kernel)
  long long order_cap = 0;
  int *na_order = nullptr;      // module scratch of salsa_gb300_run_noalloc on this handle's device
  unsigned long long *na_status = nullptr;
  void *scratch[4] = {nullptr, nullptr, nullptr, nullptr};   // gradient-chain buffers
  size_t scratch_bytes[4] = {0, 0, 0, 0};
  int last_launches = 0;
  double last_kernel_ms = 0.;
  unsigned long long *d_stage = nullptr;   // instrumented builds only
};

extern "C" {

const char *salsa_gb300_version(void) { return "salsa_gb300 1.0 (sm_103a)"; }

void salsa_gb300_default_config(salsa_config_t *c) {
  if (!c) return;
  memset(c, 0, sizeof *c);
  c->level = 5;
  salsa_switch_t off = {0, 0., 1};
  c->lscoag = c->lscnd = c->lsauto = c->lsactiv = c->lsicenucl = c->lsicemelt = c->lssecice = off;
  c->lsFreeTheta = c->lsfreeRH = off;
  c->lssiprimespln = c->lssipdropfrac = c->lssipicecollbreak = off;
  c->lscgaa = c->lscgcc = c->lscgca = c->lscgpc = c->lscgpa = c->lscgpp = 1;
  c->lscgia = c->lscgic = c->lscgii = c->lscgip = 1;
  c->Eiagg_max = 0.3;
  c->Eiagg_min = 0.05;
  c->cgintvl = 10.;
  c->lscndgas = 0;
  c->lscndh2oae = c->lscndh2ocl = c->lscndh2oic = 1;
  c->ice_theta_dist = 1;
  c->mean_theta_imm = 132.;
  c->sigma_theta_imm = 20.;
  c->mean_theta_dep = 15.5;
  c->sigma_theta_dep = 1.4;
  c->iceShapeAlpha = 15.56999e-3;
  c->iceShapeBeta = 2.02;
  c->iceShapeGamma = 0.55;
  c->iceShapeSigma = 1.97;
  c->lsdistupdate = 1;
  c->fixinc = -1.;
  c->rhlim = 1.20;
  c->eddy_dis = 0.001;
  c->nj3 = 1;
  c->act_coeff = 1.e-7;
  c->nbin[0] = 3;
  c->nbin[1] = 8;
  c->reglim[0] = 3.e-9;
  c->reglim[1] = 4.e-8;
  c->reglim[2] = 7.e-7;
  c->reglim[3] = 1.5e-5;
  c->prc_nbins = 20;
  c->prc_dlo = 20.e-6;
  c->prc_vol_ratio = 2.;
  c->ice_nbins = 20;
  c->ice_dlo = 20.e-6;
  c->ice_vol_ratio = 2.;
  c->nspec_dry = 1;
  strcpy(c->listspec[0], "SO4");
  c->chargeTMax = 1000.;
  c->chargeCollEnh = 0.;
  c->precision = 0;
  c->diagnostics = 1;
}

int salsa_gb300_init(const salsa_config_t *cfg, salsa_handle_t **out) {
  if (!cfg || !out) return SALSA_E_ARG;
  *out = nullptr;
  const salsa_config_t &g = *cfg;
  if (g.level != 4 && g.level != 5) return SALSA_E_ARG;
  if (g.nbin[0] < 1 || g.nbin[1] < 4 || g.prc_nbins < 1 || g.ice_nbins < 1) return SALSA_E_ARG;
  if (g.nspec_dry < 1 || g.nspec_dry > SALSA_MAXSPEC) return SALSA_E_ARG;
  if (g.nspec_dry > 5) return SALSA_E_UNSUPPORTED;   // SALSA_NSV volume slots per bin
  if (g.precision != 0 && g.precision != 1) return SALSA_E_ARG;
  // the secondary-ice modes of the reference: rime splintering 1-2, drop fracturing 1-4,
  // ice-ice breakup 1-3
  if (g.lssecice.sw) {
    const salsa_switch_t &rs = g.lssiprimespln, &df = g.lssipdropfrac, &ib = g.lssipicecollbreak;
    if (rs.sw && (rs.mode < 1 || rs.mode > 2)) return SALSA_E_UNSUPPORTED;
    if (df.sw && (df.mode < 1 || df.mode > 4)) return SALSA_E_UNSUPPORTED;
    if (ib.sw && (ib.mode < 1 || ib.mode > 3)) return SALSA_E_UNSUPPORTED;
  }
  if (g.lscoag.mode == 2 && !(g.cgintvl > 0.)) return SALSA_E_ARG;
  // nucleation: the ternary scheme STOPs in the reference (mo_salsa_nucleation.f90:236-238);
  // nj3 outside 1-3 STOPs once a cell nucleates (:600-602)
  if (g.nsnucl == 4 || g.nsnucl < 0 || (g.nsnucl > 0 && (g.nj3 < 1 || g.nj3 > 3))) return SALSA_E_UNSUPPORTED;
  if (g.level == 5 && g.fixinc > 0. && !(g.lsicehom || g.lsiceimm || g.lsicedep)) return SALSA_E_UNSUPPORTED;
  if (g.prc_nbins > 20) return SALSA_E_UNSUPPORTED;   // precipitation-formation accumulators
  int nb1 = g.nbin[0], nb2 = g.nbin[1];
  int nbins = nb1 + 2 * nb2, ncld = 2 * nb2, nprc = g.prc_nbins, nice = g.ice_nbins;
  int ntotal = nbins + ncld + nprc + nice;
  if (ntotal > SALSA_MAXNB || ntotal > 255) return SALSA_E_ARG;

  // ---- species (classSpecies.f90:167-244, sortProperties :247-272, defineSubsets :275-341) ----
  int allInd[9], used[9];
  for (int i = 0; i < 9; i++) { allInd[i] = -1; used[i] = 0; }
  for (int i = 0; i < g.nspec_dry; i++)
    for (int k = 0; k < SALSA_MAXSPEC; k++)
      if (name_eq(ALLNAMES[k], g.listspec[i])) { allInd[k] = i; used[k] = 1; }
  int cnt = 0;
  for (int k = 0; k < SALSA_MAXSPEC; k++) cnt += used[k];
  if (cnt != g.nspec_dry) return SALSA_E_ARG;
  int nlist = g.nspec_dry;
  allInd[7] = nlist; used[7] = 1;
  allInd[8] = nlist + 1; used[8] = 1;
  DevParams B;
  memset(&B, 0, sizeof B);
  B.nused = nlist + 2; B.ndry = nlist; B.nwet = nlist + 1; B.iwa = nlist; B.irim = nlist + 1;
  for (int k = 0; k < 9; k++) if (used[k]) {
    int j = allInd[k];
    B.rholiq[j] = ALLRHO[k];
    B.rhoice[j] = (k == 7) ? 917. : ALLRHO[k];
    B.MM[j] = ALLMM[k];
    B.diss[j] = ALLDISS[k];
    B.irholiq[j] = 1. / B.rholiq[j];
    B.irhoice[j] = 1. / B.rhoice[j];
  }
  for (int j = 0; j < B.nused; j++)
    for (int k = 0; k < 9; k++) if (used[k] && allInd[k] == j) {
      if (k == 0 || k == 1 || k == 4 || k == 5 || k == 6) B.ind_soluble[B.nsoluble++] = j;
      if (k == 2 || k == 3) B.ind_insoluble[B.ninsoluble++] = j;
    }
  B.ix_so4 = allInd[0]; B.ix_oc = allInd[1]; B.ix_bc = allInd[2]; B.ix_du = allInd[3];
  B.ix_ss = allInd[4]; B.ix_no = allInd[5]; B.ix_nh = allInd[6];
  if (g.level == 5 && g.ice_theta_dist && (g.lsicehom || g.lsiceimm || g.lsicedep) && B.ix_du < 0)
    return SALSA_E_UNSUPPORTED;   // iceNucleation (mo_salsa_cloud_ice_SE.f90:439) indexes DU

  // ---- bins (mo_salsa_init.f90:148-450, salsa_initialize :806-814) ----
  B.in1a = 0; B.in2a = B.in1a + nb1; B.in2b = B.in2a + nb2;
  B.fn1a = B.in2a - 1; B.fn2a = B.fn1a + nb2; B.fn2b = B.fn2a + nb2;
  B.nbins = nbins; B.ncld = ncld; B.nprc = nprc; B.nice = nice; B.ntotal = ntotal;
  B.nliquid = nbins + ncld + nprc;
  B.ica_cur = 0; B.ica_par = B.in2a; B.fca_cur = nb2 - 1;
  B.icb_cur = nb2; B.icb_par = B.in2b; B.fcb_cur = ncld - 1;
  BinTab t;
  t.vlo.assign(ntotal, 0.); t.vhi.assign(ntotal, 0.); t.vrlo.assign(ntotal, 0.); t.vrhi.assign(ntotal, 0.);
  t.dmid.assign(ntotal, 0.);
  {
    const double *rl = g.reglim;
    double ratio = rl[1] / rl[0];
    for (int cc = B.in1a; cc <= B.fn1a; cc++)
      set_bin(t, cc, PI6 * hcube(rl[0] * std::pow(ratio, (double)cc / nb1)),
              PI6 * hcube(rl[0] * std::pow(ratio, (double)(cc + 1) / nb1)));
    int nbin2 = 4, nbin3 = nb2 - nbin2;
    ratio = rl[2] / rl[1];
    for (int dd = B.in2a; dd <= B.in2a + nbin2 - 1; dd++) {
      int cc = dd - B.in2a;
      set_bin(t, dd, PI6 * hcube(rl[1] * std::pow(ratio, (double)cc / nbin2)),
              PI6 * hcube(rl[1] * std::pow(ratio, (double)(cc + 1) / nbin2)));
    }
    ratio = rl[3] / rl[2];
    for (int dd = B.in2a + nbin2; dd <= B.fn2a; dd++) {
      int cc = dd - (B.fn2a - (nbin3 - 1));
      set_bin(t, dd, PI6 * hcube(rl[2] * std::pow(ratio, (double)cc / nbin3)),
              PI6 * hcube(rl[2] * std::pow(ratio, (double)(cc + 1) / nbin3)));
    }
    for (int i = 0; i < nb2; i++) {
      int a = B.in2a + i, b = B.in2b + i;
      t.vlo[b] = t.vlo[a]; t.vhi[b] = t.vhi[a]; t.dmid[b] = t.dmid[a]; t.vrlo[b] = t.vrlo[a]; t.vrhi[b] = t.vrhi[a];
    }
    // cloud bins parallel to 2a and 2b (set_cloudbins :311-324)
    for (int i = 0; i < nb2; i++) {
      for (int r = 0; r < 2; r++) {
        int a = (r == 0 ? B.in2a : B.in2b) + i, c = nbins + r * nb2 + i;
        t.vlo[c] = t.vlo[a]; t.vhi[c] = t.vhi[a]; t.dmid[c] = t.dmid[a]; t.vrlo[c] = t.vrlo[a]; t.vrhi[c] = t.vrhi[a];
      }
    }
    // buildBinLimits :429-450
    auto blo = [&](int n, double dlo, double vr, int off) {
      double r = std::pow(vr, 1. / 3.);
      double lo = dlo, hi = dlo * r;
      for (int i = 0; i < n; i++) {
        if (i > 0) { lo = lo * r; hi = lo * r; }
        set_bin(t, off + i, PI6 * hcube(lo), PI6 * hcube(hi));
      }
    };
    blo(nprc, g.prc_dlo, g.prc_vol_ratio, nbins + ncld);
    blo(nice, g.ice_dlo, g.ice_vol_ratio, B.nliquid);
  }
  std::vector<double> precpbins(nprc);
  for (int i = 0; i < nprc; i++) precpbins[i] = std::pow(t.vlo[nbins + ncld + i] / PI6, 1. / 3.);
  B.cnt80 = B.cnt50 = 0;
  for (int i = 0; i < nprc; i++) { B.cnt80 += precpbins[i] < 80.e-6; B.cnt50 += precpbins[i] < 50.e-6; }

  // ---- per-block tables ----
  int nbp = ntotal;
  B.nb_pad = nbp;
  std::vector<double> tab((size_t)salsa::TAB_N * nbp, 0.);
  for (int b = 0; b < ntotal; b++) {
    tab[salsa::TAB_VLO * nbp + b] = t.vlo[b];
    tab[salsa::TAB_VHI * nbp + b] = t.vhi[b];
    tab[salsa::TAB_VRLO * nbp + b] = t.vrlo[b];
    tab[salsa::TAB_VRHI * nbp + b] = t.vrhi[b];
    tab[salsa::TAB_DMID * nbp + b] = t.dmid[b];
  }
  for (int i = 0; i < nprc; i++) tab[salsa::TAB_PRECPBINS * nbp + i] = precpbins[i];
  B.tab_doubles = (int)tab.size();

  // ---- I/O rows: thermodynamics, numbers, masses, IN deficit, charge time, outputs ----
  std::vector<Row> rows;
  auto add = [&](int fin, int fout, int idx, int mode) {
    Row r;
    r.fin = (int16_t)fin; r.fout = (int16_t)fout; r.idx = (int16_t)idx; r.mode = (int16_t)mode;
    rows.push_back(r);
  };
  add(salsa::FI_PRESS, -1, 0, salsa::ROW_IN);
  add(salsa::FI_TEMP, -1, 0, salsa::ROW_IN);
  add(salsa::FI_RSL, -1, 0, salsa::ROW_IN);
  add(salsa::FI_RSI, -1, 0, salsa::ROW_IN);
  add(salsa::FI_RP, salsa::FO_RPT, 0, salsa::ROW_TEND);
  add(salsa::FI_DN, -1, 0, salsa::ROW_IN);
  add(salsa::FI_WP, -1, 0, salsa::ROW_IN);
  add(salsa::FI_KAPPA, -1, 0, salsa::ROW_IN);
  // gases (mo_salsa_driver.f90:285-290, tendencies :369-384) only with gas condensation
  B.raw_gas = -1;
  if (g.lscndgas) {
    B.raw_gas = (int)rows.size();
    for (int i = 0; i < 5; i++) add(salsa::FI_GAERO, salsa::FO_GAEROT, i, salsa::ROW_TEND);
  }
  B.lscndgas = g.lscndgas;
  B.nsnucl = g.nsnucl;
  B.kc_mode = 0;
  B.kc_stride = 0;
  B.kc_base = 0;
  B.kcache = nullptr;
  int ncat = (g.level == 5) ? 4 : 3;
  const int catnb[4] = {nbins, ncld, nprc, nice};
  B.raw_num = (int)rows.size();
  for (int c = 0; c < ncat; c++)
    for (int b = 0; b < catnb[c]; b++) add(salsa::FI_NAERO + c, salsa::FO_NAEROT + c, b, salsa::ROW_TEND);
  for (int c = 0; c < 4; c++) B.raw_mbase[c] = 0;
  for (int c = 0; c < ncat; c++) {
    B.raw_mbase[c] = (int)rows.size();
    int nsp = (c == 3) ? B.nwet + 1 : B.nwet;
    for (int s = 0; s < nsp; s++)
      for (int b = 0; b < catnb[c]; b++) add(salsa::FI_MAERO + c, salsa::FO_MAEROT + c, s * catnb[c] + b, salsa::ROW_TEND);
  }
  B.raw_indef = -1;
  if (g.level == 5 && g.ice_theta_dist) {
    B.raw_indef = (int)rows.size();
    for (int b = 0; b < B.nliquid; b++) add(salsa::FI_INDEF, salsa::FO_INDEF, b, salsa::ROW_INOUT);
  }
  B.raw_charge = (int)rows.size();
  for (int b = 0; b < B.nliquid; b++) add(salsa::FI_CHARGE, salsa::FO_CHARGE, b, salsa::ROW_INOUT);
  B.raw_nact = (int)rows.size();
  for (int k = 0; k < ncld; k++) add(-1, salsa::FO_NACT, k, salsa::ROW_OUT);
  B.raw_vact = (int)rows.size();
  for (int s = 0; s < B.nwet; s++)
    for (int k = 0; k < ncld; k++) add(-1, salsa::FO_VACT, s * ncld + k, salsa::ROW_OUT);
  B.raw_diag = (int)rows.size();
  // the secondary-ice rates follow the level-5 diagnostics when lssecice is on
  const bool sipsw = g.level == 5 && g.lssecice.sw;
  int ndiag = (g.level == 5) ? (sipsw ? SALSA_NDIAG : SALSA_DIAG_CONDI + 1) : SALSA_DIAG_AICOLL;
  for (int i = 0; i < ndiag; i++) add(-1, salsa::FO_DIAG0 + i, 0, salsa::ROW_OUT);
  // the secondary-ice tracers, per ice bin, in and out in place (mo_salsa_driver.f90:259-261, 346-348)
  B.raw_sip = -1;
  if (sipsw) {
    B.raw_sip = (int)rows.size();
    for (int k = 0; k < 3; k++)
      for (int b = 0; b < nice; b++) add(salsa::FI_SIPDRFR + k, salsa::FO_SIPDRFR + k, b, salsa::ROW_INOUT);
  }
  B.nrows = (int)rows.size();
  B.nraw = B.nrows;

  // ---- collision pairs i <= j of enabled category pairs (mo_salsa_coagulation_kernels.f90:24-90) ----
  salsa_config_t e = g;
  if (g.level == 4) { e.lscgia = e.lscgic = e.lscgii = e.lscgip = 0; }
  auto cat_of = [&](int b) { return b < nbins ? 0 : (b < nbins + ncld ? 1 : (b < B.nliquid ? 2 : 3)); };
  auto pair_on = [&](int ci, int cj) -> bool {
    if (ci > cj) { int x = ci; ci = cj; cj = x; }
    if (ci == 0 && cj == 0) return e.lscgaa;
    if (ci == 1 && cj == 1) return e.lscgcc;
    if (ci == 2 && cj == 2) return e.lscgpp;
    if (ci == 3 && cj == 3) return e.lscgii;
    if (ci == 0 && cj == 1) return e.lscgca;
    if (ci == 0 && cj == 2) return e.lscgpa;
    if (ci == 0 && cj == 3) return e.lscgia;
    if (ci == 1 && cj == 2) return e.lscgpc;
    if (ci == 1 && cj == 3) return e.lscgic;
    return e.lscgip;
  };
  // pairs of (nearly) equal bin sizes take the self-coagulation offset of coagc
  // (mo_salsa_coagulation_kernels.f90:273-276); they are listed after the others
  std::vector<int> pairs, pairs_eq;
  for (int i = 0; i < ntotal; i++)
    for (int j = i; j < ntotal; j++)
      if (pair_on(cat_of(i), cat_of(j))) {
        bool eq = std::fabs(t.dmid[i] - t.dmid[j]) / t.dmid[i] < 1.e-2;
        (eq ? pairs_eq : pairs).push_back(i | (j << 8));
      }
  B.npairs_plain = (int)pairs.size();
  pairs.insert(pairs.end(), pairs_eq.begin(), pairs_eq.end());
  B.npairs = (int)pairs.size();

  // ---- per-target partner lists of the plain sink and source sums of the coagulation
  // update (the partner ranges of mo_salsa_coagulation_processes.f90:24-430 for aerosol,
  // cloud and precipitation targets; self terms and weighted sums stay in the kernel) ----
  {
    std::vector<int16_t> hdr(4 * (size_t)ntotal, 0), ent;
    auto rng = [&](std::vector<int16_t> &v, int g0, int a, int b) {
      for (int x = a; x <= b; x++) v.push_back((int16_t)(g0 + x));
    };
    const int C0 = nbins, P0 = nbins + ncld, I0 = B.nliquid;
    for (int t = 0; t < ntotal; t++) {
      std::vector<int16_t> sk, sr;
      int cat = cat_of(t);
      if (cat == 0) {
        int kk = t;
        int reg = kk <= B.fn1a ? 0 : (kk <= B.fn2a ? 1 : 2);
        if (reg == 0) {
          int icla = B.ica_cur + std::max(kk - B.ica_par, 0);
          int iclb = B.icb_cur + (icla - B.ica_cur);
          if (e.lscgaa) rng(sk, 0, kk + 1, B.fn2b);
          if (e.lscgca) { rng(sk, C0, icla, B.fca_cur); rng(sk, C0, iclb, B.fcb_cur); }
          if (e.lscgaa && kk > B.in1a) rng(sr, 0, B.in1a, kk - 1);
        } else if (reg == 1) {
          int index_b = B.in2b + (kk - B.in2a);
          int icla = B.ica_cur + std::max(kk - B.ica_par, 0);
          int iclb = B.icb_cur + std::max(kk - B.ica_par, 0);
          if (e.lscgaa && kk < B.fn2a) { rng(sk, 0, kk + 1, B.fn2a); rng(sk, 0, index_b, B.fn2b); }
          if (e.lscgca) { rng(sk, C0, icla, B.fca_cur); rng(sk, C0, iclb, B.fcb_cur); }
          if (e.lscgaa) { rng(sr, 0, B.in1a, kk - 1); rng(sr, 0, B.in2b, index_b); }
        } else {
          int index_a = B.in2a + (kk - B.in2b);
          int icla = B.ica_cur + std::max(kk - B.icb_par, 0);
          int iclb = B.icb_cur + std::max(kk - B.icb_par, 0);
          if (e.lscgaa && kk < B.fn2b) { rng(sk, 0, kk + 1, B.fn2b); rng(sk, 0, index_a, B.fn2a); }
          if (e.lscgca) { rng(sk, C0, icla, B.fca_cur); rng(sk, C0, iclb, B.fcb_cur); }
          if (e.lscgaa) { rng(sr, 0, B.in2b, kk - 1); rng(sr, 0, B.in1a, index_a); }
        }
        if (e.lscgpa) rng(sk, P0, 0, nprc - 1);
        if (e.lscgia) rng(sk, I0, 0, nice - 1);
        if (e.lscgca) {
          int icla, iclb;
          if (reg < 2) { icla = B.ica_cur + (kk - B.ica_par) - 1; iclb = B.icb_cur + (icla - B.ica_cur); }
          else { iclb = B.icb_cur + (kk - B.icb_par) - 1; icla = B.ica_cur + (iclb - B.icb_cur); }
          if (icla >= B.ica_cur) rng(sr, C0, B.ica_cur, icla);
          if (iclb >= B.icb_cur) rng(sr, C0, B.icb_cur, iclb);
        }
      } else if (cat == 1) {
        int kk = t - C0;
        bool ra = kk <= B.fca_cur;
        int kfirst = ra ? B.ica_cur : B.icb_cur, klast = ra ? B.fca_cur : B.fcb_cur;
        int o_first = ra ? B.icb_cur : B.ica_cur, o_last = ra ? B.fcb_cur : B.fca_cur;
        int rel = kk - kfirst, other = o_first + rel;
        if (e.lscgca && kk < klast) { rng(sk, 0, B.ica_par + rel + 1, B.fn2a); rng(sk, 0, B.icb_par + rel + 1, B.fn2b); }
        if (e.lscgcc && kk < klast) { rng(sk, C0, kk + 1, klast); rng(sk, C0, other, o_last); }
        if (e.lscgpc) rng(sk, P0, 0, nprc - 1);
        if (e.lscgic) rng(sk, I0, 0, nice - 1);
      } else if (cat == 2) {
        int kk = t - P0;
        if (e.lscgpp && kk < nprc - 1) rng(sk, P0, kk + 1, nprc - 1);
        if (e.lscgip) rng(sk, I0, 0, nice - 1);
      }
      hdr[4 * t] = (int16_t)(4 * ntotal + ent.size());
      hdr[4 * t + 1] = (int16_t)sk.size();
      ent.insert(ent.end(), sk.begin(), sk.end());
      hdr[4 * t + 2] = (int16_t)(4 * ntotal + ent.size());
      hdr[4 * t + 3] = (int16_t)sr.size();
      ent.insert(ent.end(), sr.begin(), sr.end());
    }
    hdr.insert(hdr.end(), ent.begin(), ent.end());
    while (hdr.size() % 4) hdr.push_back(0);
    B.list_off = (int)tab.size();
    size_t nd = hdr.size() / 4;
    tab.resize(tab.size() + nd, 0.);
    std::memcpy(tab.data() + B.list_off, hdr.data(), hdr.size() * sizeof(int16_t));
    B.tab_doubles = (int)tab.size();
  }

  salsa_handle *h = new salsa_handle();
  h->cfg = g;
  if (cudaGetDevice(&h->device) != cudaSuccess) { delete h; return SALSA_E_NODEV; }
  cudaDeviceProp prop;
  if (cudaGetDeviceProperties(&prop, h->device) != cudaSuccess) { delete h; return SALSA_E_NODEV; }
  h->nsm = prop.multiProcessorCount;
  int kt_bytes = g.precision == 0 ? 8 : 4;
  {
    size_t tri_n = (size_t)nbp * (nbp + 1) / 2;
    // the kernel triangle; after the coagulation the ice nucleation keeps 8 doubles per liquid bin there
    size_t kd = std::max((tri_n * kt_bytes + 7) / 8, (size_t)8 * B.nliquid);
    size_t n = ((B.nraw + 1) & ~1) + nbp + SALSA_NSV * nbp + 7 * nbp + 13 * nbp + 336 + 64 + kd;
    if (g.lssecice.sw && g.level == 5) {
      // the secondary-ice tallies and the schemes' scratch after the kernel triangle
      n = (n + 1) & ~(size_t)1;
      B.sip_off = (int)n;
      n += 4 * (size_t)nprc * nice + 2 * (size_t)nice * nice + 7 * (size_t)nice + 3 * (size_t)nice * SALSA_NSV +
           4 * (size_t)nice + 4;
      int spl = 0;   // mo_salsa_SIP_RS.f90:72: ice bins whose lower limit is below the 10 um splinters
      for (int bb = 0; bb < nice; bb++) spl += std::pow(t.vlo[B.nliquid + bb] / PI6, 1. / 3.) < 10.e-6;
      B.sip_splbin = spl < 1 ? 1 : spl;
      B.sip_rs_mode = g.lssiprimespln.mode;
      B.sip_df_mode = g.lssipdropfrac.mode;
      B.sip_ib_mode = g.lssipicecollbreak.mode;
    }
    B.ws_doubles = (int)((n + 1) & ~(size_t)1);
  }
  size_t smem = sizeof(double) * ((size_t)B.tab_doubles + (size_t)SALSA_CPG * B.ws_doubles);
  if (smem > (size_t)prop.sharedMemPerBlockOptin) { delete h; return SALSA_E_UNSUPPORTED; }
  bool ok = cudaMalloc(&h->d_tables, tab.size() * sizeof(double)) == cudaSuccess &&
            cudaMalloc(&h->d_rows, rows.size() * sizeof(Row)) == cudaSuccess &&
            cudaMalloc(&h->d_pairs, (pairs.size() + 1) * sizeof(int)) == cudaSuccess &&
            cudaMalloc(&h->d_status, salsa::ST_N * sizeof(unsigned long long)) == cudaSuccess &&
            cudaMallocHost(&h->h_status, salsa::ST_N * sizeof(unsigned long long)) == cudaSuccess &&
            // a blocking stream: the synchronous entries then start after the work the
            // caller queued on the legacy default stream (e.g. the copies that filled the
            // fields), as a synchronous call should
            cudaStreamCreate(&h->stream) == cudaSuccess &&
            cudaEventCreate(&h->ev0) == cudaSuccess && cudaEventCreate(&h->ev1) == cudaSuccess;
  if (ok)
    ok = cudaMemcpy(h->d_tables, tab.data(), tab.size() * sizeof(double), cudaMemcpyHostToDevice) == cudaSuccess &&
         cudaMemcpy(h->d_rows, rows.data(), rows.size() * sizeof(Row), cudaMemcpyHostToDevice) == cudaSuccess &&
         (pairs.empty() ||
          cudaMemcpy(h->d_pairs, pairs.data(), pairs.size() * sizeof(int), cudaMemcpyHostToDevice) == cudaSuccess);
  if (!ok) {
    salsa_gb300_finalize(h);
    return SALSA_E_CUDA;
  }
  B.tables = h->d_tables;
  B.rows = h->d_rows;
  B.pairs = h->d_pairs;
  B.status = h->d_status;
#ifdef SALSA_STAGE_TIMERS
  cudaMalloc(&h->d_stage, 16 * sizeof(unsigned long long));
  cudaMemset(h->d_stage, 0, 16 * sizeof(unsigned long long));
  B.stage_clocks = h->d_stage;
#endif
  B.Eiagg_max = g.Eiagg_max; B.Eiagg_min = g.Eiagg_min; B.eddy_dis = g.eddy_dis; B.rhlim = g.rhlim;
  B.initMinTheta = g.initMinTheta; B.chargeTimeMax = g.chargeTMax; B.chargeCollEnh = g.chargeCollEnh;
  B.mean_theta_imm = g.mean_theta_imm; B.sigma_theta_imm = g.sigma_theta_imm;
  B.mean_theta_dep = g.mean_theta_dep; B.sigma_theta_dep = g.sigma_theta_dep;
  B.iceShapeAlpha = g.iceShapeAlpha; B.iceShapeBeta = g.iceShapeBeta;
  B.iceShapeGamma = g.iceShapeGamma; B.iceShapeSigma = g.iceShapeSigma;
  B.level = g.level;
  h->base = B;
  // Load, on the handle's device, every module a step of this handle can launch, and
  // resolve the module scratch of salsa_gb300_run_noalloc: under lazy module loading a
  // module (and its static device arrays) is loaded on first use, and for callers of
  // the no-alloc step that first use must not come after their pool has taken the
  // free memory.
  {
    void *po = nullptr, *ps = nullptr;
    cudaFuncAttributes fa;
    const bool sip = g.lssecice.sw && g.level == 5;
    const int bps = sip ? (g.precision == 0 ? salsa::blocks_per_sm_ds(B) : salsa::blocks_per_sm_fs(B))
                        : (g.precision == 0 ? (g.diagnostics ? salsa::blocks_per_sm_d1(B) : salsa::blocks_per_sm_d0(B))
                                            : (g.diagnostics ? salsa::blocks_per_sm_f1(B) : salsa::blocks_per_sm_f0(B)));
    if (bps <= 0 || cudaFuncGetAttributes(&fa, salsa_order_kernel) != cudaSuccess ||
        cudaGetSymbolAddress(&po, g_na_order) != cudaSuccess || cudaGetSymbolAddress(&ps, g_na_status) != cudaSuccess) {
      salsa_gb300_finalize(h);
      return SALSA_E_CUDA;
    }
    h->na_order = static_cast<int *>(po);
    h->na_status = static_cast<unsigned long long *>(ps);
  }
  h->lolim_diam.resize(ntotal);
  for (int b = 0; b < ntotal; b++) h->lolim_diam[b] = std::pow(t.vlo[b] / PI6, 1. / 3.);
  *out = h;
  return SALSA_OK;
}

void salsa_gb300_finalize(salsa_handle_t *h) {
  if (!h) return;
  if (h->d_tables) cudaFree(h->d_tables);
  if (h->d_rows) cudaFree(h->d_rows);
  if (h->d_pairs) cudaFree(h->d_pairs);
  if (h->d_order) cudaFree(h->d_order);
  for (int i = 0; i < 4; i++)
    if (h->scratch[i]) cudaFree(h->scratch[i]);
  if (h->d_status) cudaFree(h->d_status);
  if (h->h_status) cudaFreeHost(h->h_status);
  if (h->stage) cudaFree(h->stage);
  if (h->kcache) cudaFree(h->kcache);
  for (auto e : h->pev)
    if (e) cudaEventDestroy(e);
  if (h->s_in) cudaStreamDestroy(h->s_in);
  if (h->s_out) cudaStreamDestroy(h->s_out);
  if (h->ev0) cudaEventDestroy(h->ev0);
  if (h->ev1) cudaEventDestroy(h->ev1);
  if (h->stream) cudaStreamDestroy(h->stream);
  delete h;
}

int salsa_gb300_layout(const salsa_handle_t *h, int *nbins, int *ncld, int *nprc, int *nice, int *nwet,
                       double *lolim) {
  if (!h) return SALSA_E_ARG;
  if (nbins) *nbins = h->base.nbins;
  if (ncld) *ncld = h->base.ncld;
  if (nprc) *nprc = h->base.nprc;
  if (nice) *nice = h->base.nice;
  if (nwet) *nwet = h->base.nwet;
  if (lolim) for (int b = 0; b < h->base.ntotal; b++) lolim[b] = h->lolim_diam[b];
  return SALSA_OK;
}

int salsa_gb300_last_launches(const salsa_handle_t *h) { return h ? h->last_launches : 0; }
double salsa_gb300_last_kernel_ms(const salsa_handle_t *h) { return h ? h->last_kernel_ms : 0.; }

}  // extern "C"

namespace {

// Field bookkeeping: (pointer slot in salsa_fields_t, role, number of planes)
struct FieldRef {
  const double **in;   // for inputs
  double **inout;      // for tendencies / outputs
  int planes;
  int is_output;       // needs device->host copy back
  int is_input;        // needs host->device copy
};

int resolve_side(const void *p, int *side) {
  if (!p) return 0;
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();
    return SALSA_E_ARG;
  }
  int s = (a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged) ? 1 : 0;
  if (*side < 0) *side = s;
  else if (*side != s) return SALSA_E_ARG;
  return 0;
}

int run_impl(salsa_handle_t *h, int nzp, int nxp, int nyp, int ns, double tstep, double time, int istp, int level,
             int lcharge, int initialize, const salsa_fields_t *f, cudaStream_t stream, int sync, salsa_status_t *st,
             int allow_host, int noalloc = 0) {
  if (!h || !f) return SALSA_E_ARG;
  const salsa_config_t &g = h->cfg;
  if (level != g.level || nzp < 3 || nxp < 5 || nyp < 5 || !(tstep > 0.) || !(tstep <= 600.) || ns < h->base.nwet)
    return SALSA_E_ARG;   // tstep <= 600 s keeps the 0.02 s condensation substep loop bounded
  if (!f->press || !f->temp || !f->rsl || !f->dn || !f->rp || !f->rpt || !f->naero || !f->ncloud || !f->nprecp ||
      !f->naerot || !f->ncloudt || !f->nprecpt || !f->maero || !f->mcloud || !f->mprecp || !f->maerot || !f->mcloudt ||
      !f->mprecpt || !f->pa_nactd || !f->pa_vactd)
    return SALSA_E_ARG;
  if (level == 5 && (!f->rsi || !f->nice || !f->mice || !f->nicet || !f->micet)) return SALSA_E_ARG;
  if (level == 5 && g.ice_theta_dist && !f->indef) return SALSA_E_ARG;
  if (lcharge && !f->chargeTime) return SALSA_E_ARG;
  if (level == 5 && g.lssecice.sw && (!f->sipdrfr || !f->siprmspl || !f->sipiibr)) return SALSA_E_ARG;
  if (g.lscndgas && (!f->gaero || !f->gaerot)) return SALSA_E_ARG;
  if (g.lsactiv.sw && g.lsactiv.mode == 2 && !f->wp) return SALSA_E_ARG;
  if (cudaSetDevice(h->device) != cudaSuccess) return SALSA_E_NODEV;

  // set_SALSA_runtime (mo_salsa_driver.f90:445-474): states switch on once and stay on
  const salsa_switch_t *ms[7] = {&g.lscoag, &g.lscnd, &g.lsauto, &g.lsactiv, &g.lsicenucl, &g.lsicemelt, &g.lssecice};
  for (int i = 0; i < 7; i++) {
    int sw = ms[i]->sw;
    if (level == 4 && i >= 4) sw = 0;   // define_salsa :615-635
    if (sw && time >= ms[i]->delay) h->st[i] = 1;
  }
  const salsa_switch_t *sips[3] = {&g.lssiprimespln, &g.lssipdropfrac, &g.lssipicecollbreak};
  for (int i = 0; i < 3; i++)
    if (level == 5 && sips[i]->sw && time >= sips[i]->delay) h->st_sip[i] = 1;
  if (g.lsfreeRH.sw && time > g.lsfreeRH.delay) h->st_freeRH = 1;
  if (g.lsFreeTheta.sw && time > g.lsFreeTheta.delay) h->st_freeTheta = 1;
  (void)istp;

  DevParams P = h->base;
  P.nzp = nzp; P.nxp = nxp; P.nyp = nyp;
  P.nz_int = nzp - 2; P.nx_int = nxp - 4;
  P.ncells = (long long)(nzp - 2) * (nxp - 4) * (nyp - 4);
  P.plane = (long long)nzp * nxp * nyp;
  P.ngroups = (P.ncells + SALSA_CPG - 1) / SALSA_CPG;
  P.level = level; P.lcharge = lcharge; P.initialize = initialize;
  P.dt = tstep;
  {
    int ex = 0;
    P.inv_dt = std::frexp(tstep, &ex) == 0.5 ? 1. / tstep : 0.;   // exact reciprocal of a power of two
  }
  P.st_coag = h->st[0]; P.st_cnd = h->st[1]; P.st_auto = h->st[2]; P.st_activ = h->st[3];
  P.st_icenucl = h->st[4]; P.st_icemelt = h->st[5];
  P.st_freeRH = h->st_freeRH; P.st_freeTheta = h->st_freeTheta;
  P.st_secice = h->st[6] && h->base.sip_off > 0;
  P.st_siprs = h->st_sip[0]; P.st_sipdf = h->st_sip[1]; P.st_sipib = h->st_sip[2];
  P.coag_mode = g.lscoag.mode; P.auto_mode = g.lsauto.mode; P.activ_mode = g.lsactiv.mode;
  P.icenucl_mode = (level == 4) ? 1 : g.lsicenucl.mode;
  P.lscgaa = g.lscgaa; P.lscgcc = g.lscgcc; P.lscgca = g.lscgca; P.lscgpc = g.lscgpc; P.lscgpa = g.lscgpa;
  P.lscgpp = g.lscgpp; P.lscgia = g.lscgia; P.lscgic = g.lscgic; P.lscgii = g.lscgii; P.lscgip = g.lscgip;
  P.lscndh2oae = g.lscndh2oae; P.lscndh2ocl = g.lscndh2ocl; P.lscndh2oic = g.lscndh2oic;
  P.lsicehom = g.lsicehom; P.lsiceimm = g.lsiceimm; P.lsicedep = g.lsicedep;
  P.ice_theta_dist = g.ice_theta_dist; P.lsdistupdate = g.lsdistupdate;
  if (level == 4) {
    P.lscgia = P.lscgic = P.lscgii = P.lscgip = 0;
    P.lscndh2oic = 0;
    P.ice_theta_dist = 0;
    P.lsicehom = P.lsiceimm = P.lsicedep = 0;
  }
  P.has_kappa = f->kappa != nullptr;
  // low-frequency kernel update (lscoag%mode = 2, set_SALSA_runtime :469-470): kernels are
  // computed and stored on update steps and fetched from the storage on the others; the
  // storage starts at zero (initialize_coagstorage :601-650)
  if (g.lscoag.mode == 2 && P.st_coag && P.ncells > 0) {
    if (noalloc) return SALSA_E_UNSUPPORTED;
    const bool upd = std::fmod(time, g.cgintvl) < tstep || istp <= 1;
    P.kc_mode = upd ? 1 : 2;
    P.kc_stride = h->base.nb_pad * (h->base.nb_pad + 1) / 2;
    const size_t bytes = (size_t)P.ncells * P.kc_stride * (g.precision == 0 ? 8 : 4);
    if (bytes != h->kcache_bytes) {
      if (h->kcache) cudaFree(h->kcache);
      h->kcache = nullptr;
      h->kcache_bytes = 0;
      if (cudaMalloc(&h->kcache, bytes) != cudaSuccess) return SALSA_E_CUDA;
      if (cudaMemset(h->kcache, 0, bytes) != cudaSuccess) return SALSA_E_CUDA;
      h->kcache_bytes = bytes;
    }
    P.kcache = h->kcache;
  }
  int nliq = h->base.nliquid;
  const int nb[4] = {h->base.nbins, h->base.ncld, h->base.nprc, h->base.nice};
  const int nw = h->base.nwet;
  // field table: pointer, planes, direction
  struct F { const double *src; double *dst; long long planes; int in, out, fi, fo; };
  std::vector<F> fl;
  auto fin = [&](const double *p, long long planes, int fi) { fl.push_back({p, nullptr, planes, 1, 0, fi, -1}); };
  auto fio = [&](double *p, long long planes, int fo, int in) { fl.push_back({p, p, planes, in, 1, -1, fo}); };
  fin(f->press, 1, salsa::FI_PRESS); fin(f->temp, 1, salsa::FI_TEMP); fin(f->rsl, 1, salsa::FI_RSL);
  fin(level == 5 ? f->rsi : nullptr, 1, salsa::FI_RSI);
  fin(f->rp, 1, salsa::FI_RP); fin(f->dn, 1, salsa::FI_DN); fin(f->wp, 1, salsa::FI_WP);
  fin(f->kappa, 1, salsa::FI_KAPPA);
  fin(f->naero, nb[0], salsa::FI_NAERO); fin(f->ncloud, nb[1], salsa::FI_NCLOUD); fin(f->nprecp, nb[2], salsa::FI_NPRECP);
  fin(level == 5 ? f->nice : nullptr, nb[3], salsa::FI_NICE);
  fin(f->maero, (long long)nw * nb[0], salsa::FI_MAERO); fin(f->mcloud, (long long)nw * nb[1], salsa::FI_MCLOUD);
  fin(f->mprecp, (long long)nw * nb[2], salsa::FI_MPRECP);
  fin(level == 5 ? f->mice : nullptr, (long long)(nw + 1) * nb[3], salsa::FI_MICE);
  fin(g.lscndgas ? f->gaero : nullptr, 5, salsa::FI_GAERO);
  bool use_indef = level == 5 && g.ice_theta_dist;
  fio(f->rpt, 1, salsa::FO_RPT, 1);
  fio(f->naerot, nb[0], salsa::FO_NAEROT, 1); fio(f->ncloudt, nb[1], salsa::FO_NCLOUDT, 1);
  fio(f->nprecpt, nb[2], salsa::FO_NPRECPT, 1);
  fio(level == 5 ? f->nicet : nullptr, nb[3], salsa::FO_NICET, 1);
  fio(f->maerot, (long long)nw * nb[0], salsa::FO_MAEROT, 1); fio(f->mcloudt, (long long)nw * nb[1], salsa::FO_MCLOUDT, 1);
  fio(f->mprecpt, (long long)nw * nb[2], salsa::FO_MPRECPT, 1);
  fio(level == 5 ? f->micet : nullptr, (long long)(nw + 1) * nb[3], salsa::FO_MICET, 1);
  fio(use_indef ? f->indef : nullptr, nliq, salsa::FO_INDEF, 1);
  fio(lcharge ? f->chargeTime : nullptr, nliq, salsa::FO_CHARGE, 1);
  fio(f->pa_nactd, nb[1], salsa::FO_NACT, 0);
  fio(f->pa_vactd, (long long)nw * nb[1], salsa::FO_VACT, 0);
  fio(g.lscndgas ? f->gaerot : nullptr, 5, salsa::FO_GAEROT, 1);
  const bool sipsw = level == 5 && g.lssecice.sw;
  int ndiag = (level == 5) ? (sipsw ? SALSA_NDIAG : SALSA_DIAG_CONDI + 1) : SALSA_DIAG_AICOLL;
  for (int i = 0; i < ndiag; i++) fio(g.diagnostics ? f->diag[i] : nullptr, 1, salsa::FO_DIAG0 + i, 0);
  fio(sipsw ? f->sipdrfr : nullptr, nb[3], salsa::FO_SIPDRFR, 1);
  fio(sipsw ? f->siprmspl : nullptr, nb[3], salsa::FO_SIPRMSPL, 1);
  fio(sipsw ? f->sipiibr : nullptr, nb[3], salsa::FO_SIPIIBR, 1);

  int side = -1;
  for (auto &x : fl) {
    const void *p = x.src ? (const void *)x.src : (const void *)x.dst;
    if (resolve_side(p, &side)) return SALSA_E_ARG;
  }
  bool host = side == 0;
  if (host && !allow_host) return SALSA_E_ARG;
  cudaStream_t s = stream ? stream : h->stream;
  int launches = 0;
  for (int i = 0; i < salsa::FI_N; i++) P.fin[i] = nullptr;
  for (int i = 0; i < salsa::FO_N; i++) P.fout[i] = nullptr;
  if (noalloc && P.ncells > SALSA_NOALLOC_MAXCELLS) return SALSA_E_ARG;
  unsigned long long *d_status = noalloc ? h->na_status : h->d_status;
  P.status = d_status;
  const int prec = g.precision, dg = g.diagnostics ? 1 : 0;
  auto bind = [&](DevParams &Q, const F &x, double *dp) {
    if (x.fi >= 0) Q.fin[x.fi] = dp;
    if (x.fo >= 0) {
      Q.fout[x.fo] = dp;
      if (x.fo == salsa::FO_INDEF) Q.fin[salsa::FI_INDEF] = dp;
      if (x.fo == salsa::FO_CHARGE) Q.fin[salsa::FI_CHARGE] = dp;
      if (x.fo >= salsa::FO_SIPDRFR && x.fo <= salsa::FO_SIPIIBR) Q.fin[salsa::FI_SIPDRFR + (x.fo - salsa::FO_SIPDRFR)] = dp;
    }
  };
  // order pre-pass and step kernel over the cells of Q, on stream s
  auto launch = [&](DevParams &Q, int *order) -> int {
    const bool sip = Q.st_secice != 0;
    int bps = sip ? (prec == 0 ? salsa::blocks_per_sm_ds(Q) : salsa::blocks_per_sm_fs(Q))
                  : prec == 0 ? (dg ? salsa::blocks_per_sm_d1(Q) : salsa::blocks_per_sm_d0(Q))
                              : (dg ? salsa::blocks_per_sm_f1(Q) : salsa::blocks_per_sm_f0(Q));
    if (bps <= 0) return SALSA_E_CUDA;
    long long grid = (long long)bps * h->nsm * 8;
    if (grid > Q.ngroups) grid = Q.ngroups;
    Q.order = order;
    if (order) {
      // the order list's fill counters start at zero for every launch (a call may launch
      // several, one per slab)
      if (cudaMemsetAsync(Q.status + salsa::ST_ORDER_CLEAR, 0, 2 * sizeof(unsigned long long), s) != cudaSuccess)
        return SALSA_E_CUDA;
      long long og = (Q.ncells + 255) / 256;
      if (og > (long long)h->nsm * 16) og = (long long)h->nsm * 16;
      salsa_order_kernel<<<(int)og, 256, 0, s>>>(Q, order);
      if (cudaGetLastError() != cudaSuccess) return SALSA_E_CUDA;
      launches++;
    }
    cudaError_t e = sip ? (prec == 0 ? salsa::launch_ds(Q, s, (int)grid) : salsa::launch_fs(Q, s, (int)grid))
                    : prec == 0 ? (dg ? salsa::launch_d1(Q, s, (int)grid) : salsa::launch_d0(Q, s, (int)grid))
                                : (dg ? salsa::launch_f1(Q, s, (int)grid) : salsa::launch_f0(Q, s, (int)grid));
    if (e != cudaSuccess) return SALSA_E_CUDA;
    launches++;
    return SALSA_OK;
  };
  // the cell order list (clear cells first) for up to n cells
  auto order_for = [&](long long n) -> int * {
    if (noalloc) return h->na_order;
    if (n > 0x7fffffffLL) return nullptr;
    if (n > h->order_cap) {
      if (h->d_order) cudaFree(h->d_order);
      h->d_order = nullptr;
      h->order_cap = 0;
      if (cudaMalloc(&h->d_order, (size_t)n * sizeof(int)) != cudaSuccess) return nullptr;
      h->order_cap = n;
    }
    return h->d_order;
  };
  if (P.ncells > 0 && cudaMemsetAsync(d_status, 0, salsa::ST_N * sizeof(unsigned long long), s) != cudaSuccess)
    return SALSA_E_CUDA;
  if (!host) {
    for (auto &x : fl) {
      const double *hp = x.src ? x.src : x.dst;
      if (hp) bind(P, x, const_cast<double *>(hp));
    }
    if (P.ncells > 0) {
      int *order = order_for(P.ncells);
      if (!order && P.ncells <= 0x7fffffffLL) return SALSA_E_CUDA;
      cudaEventRecord(h->ev0, s);
      int rc = launch(P, order);
      cudaEventRecord(h->ev1, s);
      if (rc) return rc;
    }
  } else if (P.ncells > 0) {
    // Host arrays: the interior y rows travel in slabs through a ring of staging slots.
    // Slab k is copied in on h->s_in, computed on s and copied out on h->s_out, so the
    // copies of neighbouring slabs overlap the computation; a slot is refilled once the
    // slab it held has been copied out.  Every array is copied in, outputs included, so
    // the values outside the interior cells come back unchanged.
    const int NS = SALSA_PIPE_SLOTS;
    const long long nyi = nyp - 4, rowd = (long long)nxp * nzp;
    const long long R = (nyi + SALSA_PIPE_SLABS - 1) / SALSA_PIPE_SLABS;
    const int nslab = (int)((nyi + R - 1) / R);
    const long long plane_s = (R + 4) * rowd;
    size_t per_slot = 0;
    for (auto &x : fl)
      if (x.src || x.dst) per_slot += (size_t)(x.planes * plane_s) * sizeof(double);
    if ((size_t)NS * per_slot > h->stage_bytes) {
      if (h->stage) cudaFree(h->stage);
      h->stage = nullptr;
      h->stage_bytes = 0;
      if (cudaMalloc(&h->stage, (size_t)NS * per_slot) != cudaSuccess) return SALSA_E_CUDA;
      h->stage_bytes = (size_t)NS * per_slot;
    }
    if (!h->s_in) {
      if (cudaStreamCreateWithFlags(&h->s_in, cudaStreamNonBlocking) != cudaSuccess ||
          cudaStreamCreateWithFlags(&h->s_out, cudaStreamNonBlocking) != cudaSuccess)
        return SALSA_E_CUDA;
      for (int i = 0; i < 3 * NS + 2; i++)
        if (cudaEventCreateWithFlags(&h->pev[i], cudaEventDisableTiming) != cudaSuccess) return SALSA_E_CUDA;
    }
    cudaEvent_t *ev_in = h->pev, *ev_k = h->pev + NS, *ev_out = h->pev + 2 * NS;
    cudaEvent_t ev_start = h->pev[3 * NS], ev_end = h->pev[3 * NS + 1];
    int *order = order_for((long long)R * P.nz_int * P.nx_int);
    if (!order) return SALSA_E_CUDA;
    if (cudaEventRecord(ev_start, s) != cudaSuccess || cudaStreamWaitEvent(h->s_in, ev_start, 0) != cudaSuccess)
      return SALSA_E_CUDA;
    const size_t prow = (size_t)P.plane * sizeof(double), srow = (size_t)plane_s * sizeof(double);
    for (int k = 0; k < nslab; k++) {
      const int slot = k % NS;
      char *base = static_cast<char *>(h->stage) + (size_t)slot * per_slot;
      const long long j0 = 2 + (long long)k * R, rs = std::min(R, nyi - (long long)k * R);
      const size_t width = (size_t)(rs * rowd) * sizeof(double);
      if (k >= NS && cudaStreamWaitEvent(h->s_in, ev_out[slot], 0) != cudaSuccess) return SALSA_E_CUDA;
      DevParams Q = P;
      Q.nyp = (int)(rs + 4);
      Q.plane = plane_s;
      Q.ncells = (long long)P.nz_int * P.nx_int * rs;
      Q.ngroups = (Q.ncells + SALSA_CPG - 1) / SALSA_CPG;
      Q.kc_base = (long long)k * R * P.nz_int * P.nx_int;
      size_t off = 0;
      for (auto &x : fl) {
        const double *hp = x.src ? x.src : x.dst;
        if (!hp) continue;
        double *dp = reinterpret_cast<double *>(base + off);
        off += (size_t)(x.planes * plane_s) * sizeof(double);
        bind(Q, x, dp);
        if (cudaMemcpy2DAsync(dp + 2 * rowd, srow, hp + j0 * rowd, prow, width, (size_t)x.planes,
                              cudaMemcpyHostToDevice, h->s_in) != cudaSuccess)
          return SALSA_E_CUDA;
      }
      if (cudaEventRecord(ev_in[slot], h->s_in) != cudaSuccess || cudaStreamWaitEvent(s, ev_in[slot], 0) != cudaSuccess)
        return SALSA_E_CUDA;
      if (k == 0) cudaEventRecord(h->ev0, s);
      int rc = launch(Q, order);
      if (rc) return rc;
      if (k == nslab - 1) cudaEventRecord(h->ev1, s);
      if (cudaEventRecord(ev_k[slot], s) != cudaSuccess || cudaStreamWaitEvent(h->s_out, ev_k[slot], 0) != cudaSuccess)
        return SALSA_E_CUDA;
      off = 0;
      for (auto &x : fl) {
        const double *hp = x.src ? x.src : x.dst;
        if (!hp) continue;
        double *dp = reinterpret_cast<double *>(base + off);
        off += (size_t)(x.planes * plane_s) * sizeof(double);
        if (x.out && cudaMemcpy2DAsync(x.dst + j0 * rowd, prow, dp + 2 * rowd, srow, width, (size_t)x.planes,
                                       cudaMemcpyDeviceToHost, h->s_out) != cudaSuccess)
          return SALSA_E_CUDA;
      }
      if (cudaEventRecord(ev_out[slot], h->s_out) != cudaSuccess) return SALSA_E_CUDA;
    }
    if (cudaEventRecord(ev_end, h->s_out) != cudaSuccess || cudaStreamWaitEvent(s, ev_end, 0) != cudaSuccess)
      return SALSA_E_CUDA;
  }
  if (P.ncells > 0 &&
      cudaMemcpyAsync(h->h_status, d_status, salsa::ST_N * sizeof(unsigned long long), cudaMemcpyDeviceToHost, s) !=
          cudaSuccess)
    return SALSA_E_CUDA;
  h->last_launches = launches;
  if (!sync && !host) {
    if (st) memset(st, 0, sizeof *st);
    return SALSA_OK;
  }
  if (cudaStreamSynchronize(s) != cudaSuccess) return SALSA_E_CUDA;
  float kms = 0.f;
  if (P.ncells > 0 && cudaEventElapsedTime(&kms, h->ev0, h->ev1) == cudaSuccess) h->last_kernel_ms = kms;
  salsa_status_t loc;
  memset(&loc, 0, sizeof loc);
  if (P.ncells > 0) {
    loc.n_cells = (long long)h->h_status[salsa::ST_CELLS];
    loc.n_equil_nonconv = (long long)h->h_status[salsa::ST_EQUIL];
    loc.n_distr_nonconv = (long long)h->h_status[salsa::ST_DISTR];
    loc.n_distr_negfrac = (long long)h->h_status[salsa::ST_NEGFRAC];
    loc.n_cond_substeps = (long long)h->h_status[salsa::ST_COND];
    loc.n_negative = (long long)h->h_status[salsa::ST_NEG];
    loc.n_nonfinite = (long long)h->h_status[salsa::ST_NONFINITE];
  }
  loc.code = (loc.n_equil_nonconv || loc.n_distr_nonconv || loc.n_distr_negfrac || loc.n_nonfinite) ? SALSA_E_NUMERIC
                                                                                                      : SALSA_OK;
  if (st) *st = loc;
  return loc.code;
}

}  // namespace

#ifdef SALSA_STAGE_TIMERS
extern "C" int salsa_gb300_stage_clocks(salsa_handle_t *h, unsigned long long *out16) {
  cudaDeviceSynchronize();
  cudaMemcpy(out16, h->d_stage, 16 * sizeof(unsigned long long), cudaMemcpyDeviceToHost);
  cudaMemset(h->d_stage, 0, 16 * sizeof(unsigned long long));
  return 0;
}
#endif

extern "C" int salsa_gb300_run(salsa_handle_t *h, int nzp, int nxp, int nyp, int ns, double tstep, double time,
                               int istp, int level, int lcharge, int initialize, const salsa_fields_t *f,
                               salsa_status_t *st) {
  return run_impl(h, nzp, nxp, nyp, ns, tstep, time, istp, level, lcharge, initialize, f, nullptr, 1, st, 1);
}

extern "C" int salsa_gb300_run_async(salsa_handle_t *h, int nzp, int nxp, int nyp, int ns, double tstep, double time,
                                     int istp, int level, int lcharge, int initialize, const salsa_fields_t *f,
                                     void *stream, int sync, salsa_status_t *st) {
  return run_impl(h, nzp, nxp, nyp, ns, tstep, time, istp, level, lcharge, initialize, f, (cudaStream_t)stream, sync,
                  st, 0);
}

extern "C" int salsa_gb300_run_noalloc(salsa_handle_t *h, int nzp, int nxp, int nyp, int ns, double tstep,
                                       double time, int istp, int level, int lcharge, int initialize,
                                       const salsa_fields_t *f, void *stream, int sync, salsa_status_t *st) {
  if (!h || !h->na_order || !h->na_status) return SALSA_E_ARG;   // both resolved by salsa_gb300_init
  return run_impl(h, nzp, nxp, nyp, ns, tstep, time, istp, level, lcharge, initialize, f, (cudaStream_t)stream, sync,
                  st, 0, 1);
}

// ---- handle internals for the other translation units (C++ linkage, not part of the C-ABI) ----
namespace salsa {
bool handle_params(const salsa_handle_t *h, DevParams *base, cudaStream_t *stream, int *device, int *nsm) {
  if (!h) return false;
  *base = h->base;
  *stream = h->stream;
  *device = h->device;
  *nsm = h->nsm;
  return true;
}
const salsa_config_t *handle_config(const salsa_handle_t *h) { return h ? &h->cfg : nullptr; }
bool device_ptrs(std::initializer_list<const void *> ps) {
  for (const void *p : ps) {
    if (!p) continue;
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) { cudaGetLastError(); return false; }
    if (a.type != cudaMemoryTypeDevice && a.type != cudaMemoryTypeManaged) return false;
  }
  return true;
}
void *handle_scratch(salsa_handle_t *h, int slot, size_t bytes) {
  if (!h || slot < 0 || slot >= 4) return nullptr;
  if (bytes > h->scratch_bytes[slot]) {
    if (h->scratch[slot]) cudaFree(h->scratch[slot]);
    h->scratch[slot] = nullptr;
    h->scratch_bytes[slot] = 0;
    if (cudaMalloc(&h->scratch[slot], bytes) != cudaSuccess) return nullptr;
    h->scratch_bytes[slot] = bytes;
  }
  return h->scratch[slot];
}
}  // namespace salsa
