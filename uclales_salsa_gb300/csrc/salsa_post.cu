// salsa_post.cu -- the LES-side constraints that follow a SALSA step
// (src/src_LES/constrain_SALSA.f90): tend_constrain2 and SALSA_diagnostics, on the
// arrays of run_SALSA (device pointers).
//
// Both are memory-bound passes over the bin-major fields.  tend_constrain2 is an
// element-wise clamp of every tendency of the SALSA_4d tracers.  SALSA_diagnostics
// runs one thread per grid point (z fastest, so a warp's loads of one bin plane are
// contiguous) through the reference's steps in order: negative values, particles with
// number but no mass, evaporating droplets / drops / ice returned to the aerosol bins,
// vanishing aerosol bins, and the water diagnostics.  Each point only reads and writes
// its own values, so the reference's bin-outer loops give the same result point by
// point.  Values are written only where they change.
//
// FP64 is the scarce pipe on this GPU, so the decisions are taken on the bit patterns
// where that is exact: a sign test, or the order of non-negative doubles (which is the
// order of their bits as integers), or an exponent bound that settles all but the cases
// near the threshold, which then take the FP64 comparison.  FP64 arithmetic remains
// where a value is produced.
//
// sedim_SALSA (src/src_LES/mcrp.f90:745-1275) runs one warp per column with the lanes
// over the levels; see the comment above sedimentation_kernel.
#include <cuda_runtime.h>
#include <algorithm>
#include <cstring>
#include <vector>
#include "../../include/salsa_gb300.h"
#include "salsa_kernel_impl.cuh"
#include "salsa_internal.h"

namespace salsa {
namespace {

struct PostArgs {
  long long plane;
  int nzp, nxp, nyp, level, only_diag, lcharge, lscndgas;
  int nbins, ncld, nprc, nice, nspec, ndry, iwa, irim, in1a, in2a, fn2a, fn2b;
  int ica_cur, fca_cur, ica_par, icb_cur, icb_par, fcb_cur;
  int gas_ix[4];                  // mass index of SO4, OC, NO, NH (or -1)
  double rholiq[9], rhoice[9], MM[9], diss[9];
  double aetot[SALSA_MAXBINS];    // aerosol bin lower limits, dry diameter (aerobins)
  salsa_post_fields_t f;
};

// ---- tend_constrain2 (:18-35) ----
struct ClampArgs {
  double *p[9], *t[9];
  long long n[9];
  double dtlt;
  double rdt;           // 1 / dtlt when dtlt is a power of two (the quotient is then a product), else 0
  int be_dt;            // biased exponent of dtlt
  double *indef;
  long long nindef;
};

constexpr long long ABS_MASK = 0x7fffffffffffffffLL, INF_BITS = 0x7ff0000000000000LL;
__device__ __forceinline__ long long bits_of(double x) { return __double_as_longlong(x); }
__device__ __forceinline__ int bexp(long long b) { return (int)((b >> 52) & 0x7ff); }
// x < 0 (false for -0 and NaN)
__device__ __forceinline__ bool neg_bits(long long b) { return b < 0 && (b & ABS_MASK) != 0 && (b & ABS_MASK) <= INF_BITS; }
// for x >= 0 (either zero) or NaN of either sign, and c > 0 finite: x > c, x < c, x <= 0
__device__ __forceinline__ bool gt_bits(long long b, long long bc) { return b > bc && b <= INF_BITS; }
__device__ __forceinline__ bool lt_bits(long long b, long long bc) { return (b & ABS_MASK) < bc; }
__device__ __forceinline__ bool le0_bits(long long b) { return (b & ABS_MASK) == 0; }

// t = MAX((-1 + 1e-8) * p / dtlt, t).  For p = +-0 the limit is the zero of the other
// sign (a finite positive dtlt).  The limit is < 0 for a normal p > 0, so a tendency with
// its sign bit clear never moves; for t < 0 the exponents settle |t| < |lo| whenever
// |t| dtlt < p / 4; the rest compute lo in FP64.
__device__ __forceinline__ void clamp_tendency(double p, double t, double *tp, double dtlt, double rdt, int be_dt) {
  const long long bp = bits_of(p), bt = bits_of(t);
  if ((bp & ABS_MASK) == 0) {          // p = +-0: lo is the zero of the other sign
    if (neg_bits(bt)) *tp = bp == 0 ? -0. : 0.;
    return;
  }
  if (bp >= 0 && bexp(bp) != 0 && bexp(bp) != 0x7ff) {
    if (bt >= 0) return;
    if (bexp(bt) + be_dt + 3 - 1023 <= bexp(bp)) return;
  }
  const double q = (-1. + 1.e-8) * p;
  const double lo = rdt != 0. ? q * rdt : q / dtlt;   // the same rounding of the same quotient
  if (lo > t) *tp = lo;
}

__global__ void __launch_bounds__(256) tend_constrain_kernel(const ClampArgs A) {
  const long long stride = (long long)gridDim.x * blockDim.x;
  const long long i0 = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  constexpr int B = 4;   // elements per thread and pass, loaded before any store
  for (int a = 0; a < 9; a++) {
    const double *__restrict__ p = A.p[a];
    double *__restrict__ t = A.t[a];
    if (!p || !t) continue;
    const long long n = A.n[a];
    for (long long e0 = i0; e0 < n; e0 += B * stride) {
      double vp[B], vt[B];
#pragma unroll
      for (int u = 0; u < B; u++) {
        const long long e = e0 + u * stride;
        vp[u] = e < n ? __ldg(p + e) : 0.;
        vt[u] = e < n ? t[e] : 0.;
      }
#pragma unroll
      for (int u = 0; u < B; u++) {
        const long long e = e0 + u * stride;
        if (e < n) clamp_tendency(vp[u], vt[u], t + e, A.dtlt, A.rdt, A.be_dt);
      }
    }
  }
  if (A.indef)
    for (long long e = i0; e < A.nindef; e += stride) {
      const double v = A.indef[e];
      const double c = fmin(fmax(v, 0.), 1.);
      if (c != v) A.indef[e] = c;
    }
}

// util.f90:1005-1024 calc_correlation, as written (sxy keeps the last product only)
__device__ double calc_correlation(const double *x, const double *y, int n) {
  double sx = 0., sy = 0., sx2 = 0., sy2 = 0., sxy = 0.;
  for (int i = 0; i < n; i++) {
    sx = sx + x[i];
    sy = sy + y[i];
    sx2 = sx2 + sq(x[i]);
    sy2 = sy2 + sq(y[i]);
    sxy = x[i] * y[i];
  }
  if (sx2 * n - sq(sx) < K_EPS || sy2 * n - sq(sy) < K_EPS) return 0.;
  return (sxy * n - sx * sy) / (sqrt(sx2 * n - sq(sx)) * sqrt(sy2 * n - sq(sy)));
}

// findDry4Wet (:376-463): aerosol bin for evaporating drops or ice of bin ib (mevap with
// nb bins); the b bin is fn2a + (ba - in2a), as the reference writes it
__device__ int find_dry4wet(const PostArgs &A, const double *nevap, const double *mevap, int nb, int ib,
                            long long p) {
  const long long pl = A.plane;
  const double *na = A.f.naero, *ma = A.f.maero;
  double cd = 0.;
  for (int s = 0; s < A.ndry; s++) cd += mevap[p + pl * ((long long)s * nb + ib)] / A.rholiq[s];
  cd = cd / nevap[p + pl * ib];
  cd = pow(cd / K_PI6, 1. / 3.);
  int cnt = 0;
  for (int b = A.in2a; b <= A.fn2a; b++) cnt += cd > A.aetot[b];
  int ba = A.in2a + cnt - 1;
  ba = ba < A.in2a ? A.in2a : (ba > A.fn2a ? A.fn2a : ba);
  const int bb = A.fn2a + (ba - A.in2a);
  if (na[p + pl * bb] <= K_NLIM) return ba;
  if (na[p + pl * ba] <= K_NLIM) return bb;
  double xa[9], xb[9], y[9];
  for (int s = 0; s < A.ndry; s++) {
    xa[s] = ma[p + pl * ((long long)s * A.nbins + ba)];
    xb[s] = ma[p + pl * ((long long)s * A.nbins + bb)];
    y[s] = mevap[p + pl * ((long long)s * nb + ib)];
  }
  const double ra = calc_correlation(xa, y, A.ndry), rb = calc_correlation(xb, y, A.ndry);
  return ra < rb ? bb : ba;
}

// moves the number and the first nsp species of bin bc of a hydrometeor category to
// aerosol bin ba
__device__ __forceinline__ void to_aerosol(const PostArgs &A, double *nh, double *mh, int nbh, int bc, int ba,
                                           long long p) {
  const long long pl = A.plane;
  double *na = A.f.naero, *ma = A.f.maero;
  na[p + pl * ba] = na[p + pl * ba] + nh[p + pl * bc];
  nh[p + pl * bc] = 0.;
  for (int s = 0; s < A.nspec; s++) {
    double *dst = ma + p + pl * ((long long)s * A.nbins + ba), *src = mh + p + pl * ((long long)s * nbh + bc);
    *dst = *dst + *src;
    *src = 0.;
  }
}

// negative values of n planes of one point to zero; the loads of a batch are issued
// before any store, so they are in flight together
__device__ __forceinline__ void clamp_neg(double *a, long long p, long long pl, int n) {
  constexpr int B = 8;
  for (int e0 = 0; e0 < n; e0 += B) {
    double v[B];
#pragma unroll
    for (int u = 0; u < B; u++) v[u] = e0 + u < n ? a[p + pl * (e0 + u)] : 0.;
#pragma unroll
    for (int u = 0; u < B; u++)
      if (neg_bits(bits_of(v[u]))) a[p + pl * (e0 + u)] = 0.;
  }
}

// ---- SALSA_diagnostics (:52-370) ----
__global__ void __launch_bounds__(128) diagnostics_kernel(const PostArgs A) {
  const long long pl = A.plane;
  const salsa_post_fields_t &f = A.f;
  double *na = f.naero, *nc = f.ncloud, *np = f.nprecp, *ni = f.nice;
  double *ma = f.maero, *mc = f.mcloud, *mp = f.mprecp, *mi = f.mice;
  const int nbins = A.nbins, ncld = A.ncld, nprc = A.nprc, nice = A.nice, nspec = A.nspec;
  const int iwa = A.iwa, irim = A.irim;
  const bool lvl5 = A.level == 5;
  const double massTH = 1.e-25;
  const long long BITS_MASSTH = bits_of(1.e-25), BITS_NLIM = bits_of(K_NLIM), BITS_PRLIM = bits_of(K_PRLIM);
  const long long BITS_1EM5 = bits_of(1.e-5), BITS_1EM6 = bits_of(1.e-6), BITS_1EM15 = bits_of(1.e-15);
  for (long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x; p < pl; p += (long long)gridDim.x * blockDim.x) {
#define AT(arr, nb, s, b) (arr)[p + pl * ((long long)(s) * (nb) + (b))]
    // negative values (whole arrays)
    clamp_neg(na, p, pl, nbins);
    clamp_neg(nc, p, pl, ncld);
    clamp_neg(np, p, pl, nprc);
    clamp_neg(ma, p, pl, nspec * nbins);
    clamp_neg(mc, p, pl, nspec * ncld);
    clamp_neg(mp, p, pl, nspec * nprc);
    if (lvl5) {
      clamp_neg(ni, p, pl, nice);
      clamp_neg(mi, p, pl, (nspec + 1) * nice);
    }
    const long long r = p / A.nzp;
    const int i = (int)(r % A.nxp), j = (int)(r / A.nxp);
    if (!A.only_diag && i >= 2 && i <= A.nxp - 3 && j >= 2 && j <= A.nyp - 3) {
      // particles with number but no mass
      // (the values are >= 0 or NaN now: a sum of them is <= 0 exactly when every term
      // is +-0, and x > 0 is a bit test)
      for (int bc = 0; bc < nbins; bc++) {
        bool empty = true;
        for (int s = 0; s < nspec; s++) empty &= le0_bits(bits_of(AT(ma, nbins, s, bc)));
        if (empty && gt_bits(bits_of(na[p + pl * bc]), 0)) {
          na[p + pl * bc] = 0.;
          for (int s = 0; s < nspec; s++) AT(ma, nbins, s, bc) = 0.;
          if (A.lcharge) f.chargeTime[p + pl * bc] = 0.;
        }
      }
      for (int bc = 0; bc < ncld; bc++) {
        bool empty = true;
        for (int s = 0; s < nspec; s++) empty &= le0_bits(bits_of(AT(mc, ncld, s, bc)));
        if (empty && gt_bits(bits_of(nc[p + pl * bc]), 0)) {
          nc[p + pl * bc] = 0.;
          for (int s = 0; s < nspec; s++) AT(mc, ncld, s, bc) = 0.;
          if (A.lcharge) f.chargeTime[p + pl * (nbins + bc)] = 0.;
        }
      }
      for (int bc = 0; bc < nprc; bc++)
        if (le0_bits(bits_of(AT(mp, nprc, iwa, bc))) && gt_bits(bits_of(np[p + pl * bc]), 0)) {
          np[p + pl * bc] = 0.;
          for (int s = 0; s < nspec; s++) AT(mp, nprc, s, bc) = 0.;
          if (A.lcharge) f.chargeTime[p + pl * (nbins + ncld + bc)] = 0.;
        }
      if (lvl5)
        for (int bc = 0; bc < nice; bc++) {
          if (!gt_bits(bits_of(ni[p + pl * bc]), 0)) continue;
          const double w_ = AT(mi, nice, iwa, bc), r_ = AT(mi, nice, irim, bc);
          if (!lt_bits(bits_of(w_), BITS_MASSTH) || !lt_bits(bits_of(r_), BITS_MASSTH)) continue;
          if (w_ + r_ < massTH) {
            ni[p + pl * bc] = 0.;
            for (int s = 0; s < nspec + 1; s++) AT(mi, nice, s, bc) = 0.;
          }
        }
      const double T = f.temp[p];
      const bool dry = f.rh[p] < 0.999;
      const double zaa = 4. * K_MWA * K_SURFW0 / (K_RG * K_RHOWA * T);
      // evaporating cloud droplets: back to the parallel aerosol bin
      for (int bc = A.ica_cur; bc <= A.fcb_cur; bc++) {
        const double n_ = nc[p + pl * bc];
        if (dry && gt_bits(bits_of(n_), BITS_NLIM) && lt_bits(bits_of(AT(mc, ncld, iwa, bc)), BITS_1EM5)) {
          double ns = 0., zvol = 0.;
          for (int s = 0; s < nspec - 1; s++) ns += A.diss[s] * AT(mc, ncld, s, bc) / A.MM[s];
          ns = ns / n_;
          const double zbb = 6. * K_MWA * ns / (K_PI * K_RHOWA);
          const double cdcld = sqrt(3. * zbb / zaa);
          for (int s = 0; s < nspec; s++) zvol += AT(mc, ncld, s, bc) / A.rholiq[s];
          zvol = zvol / n_;
          const double zdh2o = pow(zvol / K_PI6, 1. / 3.);
          if (zdh2o < fmin(0.7 * cdcld, 1.3e-5) || AT(mc, ncld, iwa, bc) < massTH * n_) {
            const int ba = bc <= A.fca_cur ? A.ica_par + (bc - A.ica_cur) : A.icb_par + (bc - A.icb_cur);
            to_aerosol(A, nc, mc, ncld, bc, ba, p);
            if (A.lcharge) f.chargeTime[p + pl * (nbins + bc)] = 0.;
          }
        }
      }
      // evaporating drops: to the aerosol bin of the closest dry size and composition
      for (int bc = 0; bc < nprc; bc++) {
        const double n_ = np[p + pl * bc];
        if (dry && gt_bits(bits_of(n_), BITS_PRLIM) && lt_bits(bits_of(AT(mp, nprc, iwa, bc)), BITS_1EM6)) {
          double ns = 0., zvol = 0.;
          for (int s = 0; s < nspec - 1; s++) ns += A.diss[s] * AT(mp, nprc, s, bc) / A.MM[s];
          ns = ns / n_;
          const double zbb = 6. * K_MWA * ns / (K_PI * K_RHOWA);
          const double cdprc = sqrt(3. * zbb / zaa);
          for (int s = 0; s < nspec; s++) zvol += AT(mp, nprc, s, bc) / A.rholiq[s];
          zvol = zvol / n_;
          const double zdh2o = pow(zvol / K_PI6, 1. / 3.);
          if (zdh2o < fmin(0.2 * cdprc, 10.e-6) || AT(mp, nprc, iwa, bc) < massTH * n_) {
            const int ba = find_dry4wet(A, np, mp, nprc, bc, p);
            to_aerosol(A, np, mp, nprc, bc, ba, p);
            if (A.lcharge) f.chargeTime[p + pl * (nbins + ncld + bc)] = 0.;
          }
        }
      }
      // evaporating ice (rime goes to the aerosol water)
      if (lvl5 && f.rhi[p] < 0.999)
        for (int bc = 0; bc < nice; bc++) {
          const double n_ = ni[p + pl * bc];
          if (!gt_bits(bits_of(n_), BITS_PRLIM)) continue;
          const double w_ = AT(mi, nice, iwa, bc), r_ = AT(mi, nice, irim, bc);
          if (!lt_bits(bits_of(w_), BITS_1EM15) || !lt_bits(bits_of(r_), BITS_1EM15)) continue;
          if (w_ + r_ < 1.e-15) {
            double vt = 0.;
            for (int s = 0; s < nspec + 1; s++) vt += AT(mi, nice, s, bc) / A.rhoice[s];
            double cdice = vt / n_;
            cdice = pow(cdice / K_PI6, 1. / 3.);
            double zdrms = 0., zwams = 0.;
            for (int s = 0; s < A.ndry; s++) zdrms += AT(mi, nice, s, bc);
            for (int s = 0; s < nspec + 1; s++) zwams += AT(mi, nice, s, bc);
            if (zdrms / zwams > 0.5 || cdice < 2.e-6) {
              const int ba = find_dry4wet(A, ni, mi, nice, bc, p);
              to_aerosol(A, ni, mi, nice, bc, ba, p);
              double *dst = ma + p + pl * ((long long)iwa * nbins + ba), *src = mi + p + pl * ((long long)irim * nice + bc);
              *dst = *dst + *src;
              *src = 0.;
            }
          }
        }
      // aerosol bins below 0.1 nm dry diameter vanish; volatile species to the gases
      for (int ba = 0; ba < nbins; ba++) {
        const double n_ = na[p + pl * ba];
        if (gt_bits(bits_of(n_), BITS_NLIM)) {
          // the dry volume per particle is at least m_s / 2650 for every dry species s
          // (no density is larger): when the largest m_s is 2^88 times below n, the
          // particle is above 0.1 nm (pi/6 1e-30 * 2650 < 2^-88) and the sum is not needed
          long long mx = 0;
          for (int s = 0; s < nspec - 1; s++) mx = max(mx, bits_of(AT(ma, nbins, s, ba)));
          if (mx <= INF_BITS && bexp(mx) != 0 && bexp(mx) + 88 >= bexp(bits_of(n_))) continue;
          double zvol = 0.;
          for (int s = 0; s < nspec - 1; s++) zvol += AT(ma, nbins, s, ba) / A.rholiq[s];
          zvol = zvol / n_;
          if (zvol < K_PI6 * cube(1.e-10)) {
            if (A.lscndgas) {
              const int gi[4] = {0, 4, 1, 2};   // SO4 -> 1, OC -> 5, NO -> 2, NH -> 3
              for (int q = 0; q < 4; q++) {
                const int ix = A.gas_ix[q];
                if (ix >= 0) {
                  double *gq = f.gaero + p + pl * gi[q];
                  *gq = *gq + AT(ma, nbins, ix, ba) / A.MM[ix] * K_AVOG;
                }
              }
            }
            for (int s = 0; s < nspec; s++) AT(ma, nbins, s, ba) = 0.;
            na[p + pl * ba] = 0.;
          }
        }
      }
    }
    // water diagnostics
    double rc = 0., rcc = 0., srp = 0., snrp = 0.;
    for (int b = A.in1a; b <= A.fn2b; b++) rc += AT(ma, nbins, iwa, b);
    for (int b = A.ica_cur; b <= A.fcb_cur; b++) rcc += AT(mc, ncld, iwa, b);
    rc = rc + rcc;
    for (int b = 0; b < nprc; b++) srp += AT(mp, nprc, iwa, b);
    for (int b = 0; b < nprc; b++) snrp += np[p + pl * b];
    f.rc[p] = rc;
    f.srp[p] = srp;
    f.snrp[p] = snrp;
    double rt = rc + srp + f.rp[p];
    if (lvl5) {
      double ri = 0., riri = 0.;
      for (int b = 0; b < nice; b++) ri += AT(mi, nice, iwa, b);
      for (int b = 0; b < nice; b++) riri += AT(mi, nice, irim, b);
      f.ri[p] = ri;
      f.riri[p] = riri;
      rt = rt + ri + riri;
    }
    f.rtot[p] = rt;
#undef AT
  }
}

// ---- sedim_SALSA (src/src_LES/mcrp.f90:745-1275) ----
// One warp per column (0-based level kc is the reference's k = kc + 1).  The air
// properties of every level are computed once per column into shared memory; then,
// in the reference's order:
//   DepositionSlow (:926-1069) for the aerosol and then the cloud bins.  Per bin, a
//     ballot pass lists the levels whose number reaches the limit; the lanes take
//     those levels for the fall speed (so a sparse bin costs only its populated
//     levels), then the levels whose own or upper flux is non-zero for the flux
//     divergence, which is subtracted from the tendency in place;
//   DepositionFast (:1073-1275) for precipitation and then ice.  Per bin, pass A gives
//     each populated source level its fall speed and the level kf its parcel reaches
//     and marks the levels it changes; pass B gathers, for every marked level, the
//     contributions of the sources in the order the reference adds them (sources from
//     the top down, a level's removal of its own parcel before its re-deposit).
// Levels and bins that the reference visits only to add a zero are skipped.  The sums
// over bins (rrate, tlt, the surface rates) run in the reference's index order,
// including the range (ns-1)*nb:ns*nb of its water sums, which starts at the last bin
// of the species before water; the ice tlt sum adds the rime changes as one partial
// sum after the water changes (the reference adds them one by one).  Quotients by a
// density, by the number, by the diameter, by the level's air density and by dtlt are
// taken as products with a reciprocal, which moves results by an ulp or so.  Halo
// columns only get their rates and fall speeds zeroed, as the reference's whole-array
// assignments do (its zero change to their tendencies is not repeated).
constexpr double LES_ALVL = 2.5e+06, LES_ALVI = 2.834e+06, LES_CP = 1005., LES_G = 9.81, LES_KB = 1.3807e-23;
constexpr double LES_PI = 3.14159265358979323846;   // defs.f90 pi (the SALSA pi6 stays truncated)
constexpr double SED_M = 4.8096e-26, SED_A = 1.249, SED_B = 0.42, SED_C = 0.87;
constexpr double EPS_REAL = 2.220446049250313e-16;   // epsilon(1.0) of the 8-byte default real
constexpr double R_PI6 = 1. / K_PI6;
constexpr int SED_KF = 0xffff, SED_BR = 1 << 16, SED_DEP = 1 << 17;   // pass-A code: kf | branch | deposited
constexpr int SED_NS = SALSA_MAXSPEC + 2;   // species slots of a bin (wet species and rime)
// per-warp shared arrays of nzp doubles
enum { W_AD = 0, W_AVIS, W_LAM, W_ILAM, W_TLT, W_RR, W_IR, W_VC, W_P0, W_P1, W_P2, W_P3, W_N };

struct SedArgs {
  DevParams P;                    // densities and ice shape parameters
  long long plane;
  int nzp, nxp, nyp, nspec, lvl5;
  int sed[4];
  int off_int, off_rem, off_sr, warp_doubles;   // per-warp shared layout (doubles)
  double dtlt, rdtlt;
  double rrholiq[9], rrhoice[9];  // reciprocal densities
  salsa_sedim_fields_t f;
};

// mo_ice_shape.f90:46-91 getDiameter (the maximum dimension of a non-spherical crystal)
__device__ double ice_diameter(const DevParams &P, double mpri, double mrim, double numc) {
  double res = 1.e-9;
  if (numc < 1.e-6) return res;
  const double Mtot = (mpri + mrim) / numc;
  const double Fr = fmax(fmin(mrim / (Mtot * numc), 0.9999), 0.0001);
  const double rho_b = Fr * K_RHORI + (1. - Fr) * K_RHOIC;
  const double Dth = pow(K_PI6 * K_RHOIC / P.iceShapeAlpha, 1. / (P.iceShapeBeta - 3.));
  const double Dgr = pow(P.iceShapeAlpha / (K_PI6 * rho_b), 1. / (3. - P.iceShapeBeta));
  const double Dcr = pow((1. / (1. - Fr)) * P.iceShapeAlpha / (K_PI6 * rho_b), 1. / (3. - P.iceShapeBeta));
  const double Mth = K_RHOIC * K_PI6 * cube(Dth), Mgr = rho_b * K_PI6 * cube(Dgr), Mcr = rho_b * K_PI6 * cube(Dcr);
  if (Mtot < Mth) res = cbrt(Mtot / (K_PI6 * K_RHOIC));
  else if (Mtot >= Mth && Mtot < Mgr) res = pow(Mtot / P.iceShapeAlpha, 1. / P.iceShapeBeta);
  else if (Mtot >= Mgr && Mtot < Mcr) res = cbrt(Mtot / (K_PI6 * rho_b));
  else if (Mtot >= Mcr) res = pow(Mtot / ((1. / (1. - Fr)) * P.iceShapeAlpha), 1. / P.iceShapeBeta);
  return res;
}

// fall speed of one bin at one level (:999-1011, :1148-1173): wet diameter
// (calcDiamLES), particle density, slip correction GG and terminal_vel
__device__ __forceinline__ double sed_vel(const SedArgs &A, int flag, int ns, double n, const double (&m)[SED_NS],
                                          double ad, double avis, double lam, double ilam, double &dwet, double &GG) {
  double v = 0., sm = 0.;
#pragma unroll
  for (int s = 0; s < SED_NS; s++)
    if (s < ns) {
      v += m[s] * (flag == 4 ? A.rrhoice[s] : A.rrholiq[s]);
      sm += m[s];
    }
  const double rn = 1. / n;
  dwet = n < 1.e-15 ? 0. : cbrt(v * rn * R_PI6);
  const double rd = 1. / dwet;
  Shape<double> sh{0., 0., 0., 0.};
  double dnsp = 0.;
  if (flag == 4) {
    double mp = 0., mr = 0.;
#pragma unroll
    for (int s = 0; s < SED_NS; s++) {
      if (s < ns - 1) mp += m[s];
      if (s == ns - 1) mr = m[s];
    }
    dnsp = n < 1.e-15 ? 0. : ice_diameter(A.P, mp, mr, n);   // calcDiamLES, non-spherical
    shape_coeffs<double>(A.P, sh, mp, mr, n);
  }
  const double zdn = sm * rn * (rd * rd * rd) * R_PI6;
  const double Kn = 2. * lam * rd;                            // 2 lambda / dwet
  GG = 1. + Kn * (SED_A + SED_B * exp(-SED_C * 0.5 * dwet * ilam));
  return terminal_vel<double>(dwet, zdn, ad, avis, GG, flag, sh, dnsp);
}

__device__ __forceinline__ bool act_bit(const unsigned *w, int k) { return (w[k >> 5] >> (k & 31)) & 1u; }
__device__ __forceinline__ unsigned lanes_below(int lane) { return (1u << lane) - 1u; }

// one bin: activity bits of the levels 1..nzp-2 (a number that is not below the limit)
// and the ascending list of the active levels; zeroes the fall speed of the others
__device__ int sed_activity(int nzp, const double *ncol, double clim, unsigned *actw, int *la, double *vt, int lane) {
  const int R = (nzp + 31) >> 5;
  int cnt = 0;
  for (int r = 0; r < R; r++) {
    const int kc = r * 32 + lane;
    const bool inr = kc >= 1 && kc <= nzp - 2;
    const bool act = inr && !(ncol[kc] < clim);
    const unsigned w = __ballot_sync(0xffffffffu, act);
    if (lane == 0) actw[r] = w;
    if (act) la[cnt + __popc(w & lanes_below(lane))] = kc;
    if (vt && !act && kc < nzp) vt[kc] = 0.;
    cnt += __popc(w);
  }
  __syncwarp();
  return cnt;
}

// DepositionSlow for one part of one column, with sedim_SALSA's tendency and tlt
// updates (:799-843)
__device__ void sed_slow(const SedArgs &A, double *sm, const double *blk, long long col, long long c2, int nb,
                         int flag, const double *numc, const double *mass, double *tn, double *tm, int lane) {
  const int nzp = A.nzp, ns = A.nspec, R = (nzp + 31) >> 5;
  const long long pl = A.plane, ps = pl * nb;
  const double *ad_s = sm + W_AD * nzp, *avis_s = sm + W_AVIS * nzp, *lam_s = sm + W_LAM * nzp,
               *ilam_s = sm + W_ILAM * nzp;
  double *tlt_s = sm + W_TLT * nzp, *rr_s = sm + W_RR * nzp, *vc_s = sm + W_VC * nzp;
  double *rs_s = sm + W_P0 * nzp, *ts_s = sm + W_P1 * nzp, *wr_s = sm + W_P2 * nzp, *wd_s = sm + W_P3 * nzp;
  int *la = (int *)(sm + A.off_int), *lf = la + nzp;
  unsigned *actw = (unsigned *)(lf + nzp);
  double *sr_s = sm + A.off_sr;
  const double *dzt_b = blk, *vmax_b = blk + 2 * nzp;
  for (int e = lane; e < nzp; e += 32) rs_s[e] = ts_s[e] = wr_s[e] = wd_s[e] = 0.;
  for (int bi = 0; bi < nb; bi++) {
    const int b = bi == 0 ? nb - 1 : bi - 1;   // the last bin first: it opens the water sum
    const double *ncol = numc + col + pl * b, *mcol = mass + col + pl * b;
    const int na = sed_activity(nzp, ncol, K_NLIM, actw, la, nullptr, lane);
    if (na == 0) continue;   // no flux anywhere in the column
    // fall speeds of the populated levels (:990-1028)
    for (int i = lane; i < ((na + 31) & ~31); i += 32) {
      if (i >= na) continue;
      const int k = la[i];
      const double n = ncol[k];
      double m[SED_NS];
#pragma unroll
      for (int s = 0; s < SED_NS; s++) m[s] = s < ns ? mcol[k + ps * s] : 0.;
      double dwet, GG;
      double vc = sed_vel(A, flag, ns, n, m, ad_s[k], avis_s[k], lam_s[k], ilam_s[k], dwet, GG);
      vc = fmin(vc, vmax_b[k]);
      if (k == 1) {   // the level just above the surface (:1020-1028)
        const double T = A.f.tk[col + 1], us = A.f.ustar[c2], avis = avis_s[1];
        const double kvis = avis / ad_s[1];
        const double mdiff = (LES_KB * T * GG) / (3.0 * LES_PI * avis * dwet);
        const double Sc = kvis / mdiff;
        double St = vc * (us * us) / LES_G * kvis;
        if (St < 0.01) St = 0.01;
        const double rt = 1.0 / fmax(EPS_REAL, (us * (pow(Sc, -2.0 / 3.0) + pow(10., -3.0 / St))));
        vc = (1. / rt) + vc;
      }
      vc_s[k] = vc;
    }
    // the levels with a non-zero divergence: own or upper level populated
    int nf = 0;
    for (int r = 0; r < R; r++) {
      const int kc = r * 32 + lane;
      const bool f = kc >= 1 && kc <= nzp - 2 && (act_bit(actw, kc) || act_bit(actw, kc + 1));
      const unsigned w = __ballot_sync(0xffffffffu, f);
      if (f) lf[nf + __popc(w & lanes_below(lane))] = kc;
      nf += __popc(w);
    }
    __syncwarp();
    // flux divergence (:1040-1048), number then the species in mass-index order
    for (int i = lane; i < ((nf + 31) & ~31); i += 32) {
      if (i >= nf) continue;
      const int k = lf[i];
      const bool a0 = act_bit(actw, k), a1 = act_bit(actw, k + 1);
      const double v0 = a0 ? vc_s[k] : 0., v1 = a1 ? vc_s[k + 1] : 0.;
      const double ad = ad_s[k], adp = ad_s[k + 1], q = dzt_b[k] / ad;
#pragma unroll
      for (int s = -1; s < SED_NS; s++) {
        if (s >= ns) continue;
        const double *src = s < 0 ? ncol : mcol + ps * s;
        const double rf0 = a0 ? -src[k] * v0 : 0., rf1 = a1 ? -src[k + 1] * v1 : 0.;
        const double d = (rf1 * adp - rf0 * ad) * q;
        double *t = s < 0 ? tn + col + pl * b + k : tm + col + pl * b + ps * s + k;
        *t = *t - d;
        if (s == ns - 2 && bi == 0) rs_s[k] = 0. + rf0;   // rflm(k,(ns-1)*nb) opens the sum
        if (s == ns - 1) {
          if (bi == 0) { wr_s[k] = rf0; wd_s[k] = d; }
          else { rs_s[k] += rf0; ts_s[k] += d; }
        }
      }
    }
    __syncwarp();
  }
  for (int r = 0; r < R; r++) {
    const int kc = r * 32 + lane;
    if (kc < 1 || kc > nzp - 1) continue;
    if (kc <= nzp - 2) {
      const double rsum = rs_s[kc] + wr_s[kc];
      rr_s[kc] = rr_s[kc] - rsum * ad_s[kc] * LES_ALVL;
      if (kc == 1) sr_s[0] = sr_s[0] - rsum * ad_s[kc] * LES_ALVL;
    }
    const double tsum = ts_s[kc] + wd_s[kc];
    tlt_s[kc] = tlt_s[kc] + tsum * (LES_ALVL / LES_CP) * A.f.th[col + kc] / A.f.tk[col + kc];
  }
  __syncwarp();
}

// DepositionFast for one part of one column, with sedim_SALSA's tendency and tlt
// updates (:847-905)
__device__ void sed_fast(const SedArgs &A, double *sm, const double *blk, long long col, int nb, int ns, int flag,
                         const double *numc, const double *mass, double *tn, double *tm, double *Vt, double *rate_s,
                         double *srate_s, int lane) {
  const int nzp = A.nzp, R = (nzp + 31) >> 5;
  const long long pl = A.plane, ps = pl * nb;
  const double alv = flag == 4 ? LES_ALVI : LES_ALVL;
  const int iw = flag == 4 ? ns - 2 : ns - 1;   // water; for ice the rime follows it
  const double *ad_s = sm + W_AD * nzp, *avis_s = sm + W_AVIS * nzp, *lam_s = sm + W_LAM * nzp,
               *ilam_s = sm + W_ILAM * nzp;
  double *tlt_s = sm + W_TLT * nzp, *vc_s = sm + W_VC * nzp, *f1_s = sm + W_P0 * nzp, *ws_s = sm + W_P2 * nzp,
         *wq_s = sm + W_P3 * nzp;
  int *kf_s = (int *)(sm + W_P1 * nzp), *tg_s = kf_s + nzp;
  int *la = (int *)(sm + A.off_int), *lt = la + nzp;
  unsigned *actw = (unsigned *)(lt + nzp);
  double *rem_s = sm + A.off_rem;
  const double *dzt_b = blk, *dzl_b = blk + nzp;
  for (int e = lane; e < nzp; e += 32) ws_s[e] = wq_s[e] = 0.;
  for (int e = lane; e < 1 + 2 * nb; e += 32) rem_s[e] = 0.;
  for (int b = 0; b < nb; b++) {
    const double *ncol = numc + col + pl * b, *mcol = mass + col + pl * b;
    double *vt = Vt + col + pl * b;
    const int na = sed_activity(nzp, ncol, K_PRLIM, actw, la, vt, lane);
    if (na == 0) continue;
    for (int e = lane; e < nzp; e += 32) tg_s[e] = 0;
    __syncwarp();
    // pass A: fall speed and destination of each populated source level (:1140-1216)
    int span = -1;
    for (int i = lane; i < ((na + 31) & ~31); i += 32) {
      if (i >= na) continue;
      const int kc = la[i];
      const double n = ncol[kc];
      double m[SED_NS];
#pragma unroll
      for (int s = 0; s < SED_NS; s++) m[s] = s < ns ? mcol[kc + ps * s] : 0.;
      const double ad = ad_s[kc];
      double dwet, GG;
      const double vc = sed_vel(A, flag, ns, n, m, ad, avis_s[kc], lam_s[kc], ilam_s[kc], dwet, GG);
      vt[kc] = vc;
      const double fdmax = A.dtlt * vc;
      double fd = 0.;
      int fi = 0;
      bool dep = false;
      while (fd < fdmax) {   // at most kc passes
        fd = fd + dzl_b[kc - fi];
        fi = fi + 1;
        if (kc - fi <= 0) { dep = true; break; }
      }
      fi = fi - 1;
      const int kf = kc - fi;
      fd = fd - dzl_b[kf];
      const double fdos = fmin(fmax(fdmax - fd, 0.), dzl_b[kf]);
      const double f1 = fdos * dzt_b[kf];
      const bool br = f1 > 0.5;
      kf_s[kc] = kf | (br ? SED_BR : 0) | (dep ? SED_DEP : 0);
      f1_s[kc] = f1;
      vc_s[kc] = vc;
      tg_s[kc] = 1;
      tg_s[kf - 1] = 1;
      if (!br) tg_s[kf] = 1;
      span = max(span, kc - kf);
      double mw = 0.;
#pragma unroll
      for (int s = 0; s < SED_NS; s++) if (s == iw) mw = m[s];
      if (flag == 4) {
        double mr = 0.;
#pragma unroll
        for (int s = 0; s < SED_NS; s++) if (s == ns - 1) mr = m[s];
        mw = mw + mr;
      }
      rate_s[kc] = rate_s[kc] + mw * ad * vc * alv;
    }
    const int F = __reduce_max_sync(0xffffffffu, span);
    __syncwarp();
    // removal statistics of the parcels that reach the surface (:1197-1202), for the
    // elements that the surface rate sums
    if (lane < 3) {
      int s = -1, pos = 0;
      if (lane == 0 && b == nb - 1) { s = iw - 1; pos = 0; }
      if (lane == 1) { s = iw; pos = 1 + b; }
      if (lane == 2 && flag == 4) { s = ns - 1; pos = 1 + nb + b; }
      if (s >= 0) {
        double acc = 0.;
        for (int i = na - 1; i >= 0; i--) {
          const int kc = la[i];
          if (kf_s[kc] & SED_DEP) acc = acc + mcol[kc + ps * s] * ad_s[kc] * vc_s[kc];
        }
        rem_s[pos] = acc;
      }
    }
    // the levels that change
    int nt = 0;
    for (int r = 0; r < R; r++) {
      const int L = r * 32 + lane;
      const bool t = L < nzp && tg_s[L];
      const unsigned w = __ballot_sync(0xffffffffu, t);
      if (t) lt[nt + __popc(w & lanes_below(lane))] = L;
      nt += __popc(w);
    }
    __syncwarp();
    // pass B: each changed level gathers its change (:1218-1250), number then species
    for (int i = lane; i < ((nt + 31) & ~31); i += 32) {
      if (i >= nt) continue;
      const int L = lt[i];
      const int k0 = min(nzp - 2, L + 1 + F), k1 = max(1, L - 1);
#pragma unroll 1
      for (int s = -1; s < ns; s++) {
        const double *src = s < 0 ? ncol : mcol + ps * s;
        double acc = 0.;
        for (int k = k0; k >= k1; k--) {
          if (!act_bit(actw, k)) continue;
          const int code = kf_s[k];
          const int kf = code & SED_KF;
          if (k != L && kf - 1 != L && kf != L) continue;
          const double v = src[k];
          if (k == L) acc = acc - v;
          if (kf - 1 == L) {
            if (code & SED_BR) acc = acc + v * dzt_b[kf - 1] / dzt_b[k];
            else acc = acc + (f1_s[k] * v) * dzt_b[kf - 1] / dzt_b[kf];
          } else if (kf == L && !(code & SED_BR)) {
            acc = acc + (1. - f1_s[k]) * v;
          }
        }
        const double val = 0. + acc;
        double *t = s < 0 ? tn + col + pl * b + L : tm + col + pl * b + ps * s + L;
        *t = *t + val * A.rdtlt;
        if (s == iw) ws_s[L] += val;
        if (flag == 4 && s == ns - 1) wq_s[L] += val;
      }
    }
    __syncwarp();
  }
  // surface rate (:1252-1257) and tlt (:867-876, :893-902)
  if (lane == 0) {
    double S = 0.;
    const int npos = flag == 4 ? 1 + 2 * nb : 1 + nb;
    for (int e = 0; e < npos; e++) S += rem_s[e];
    srate_s[0] = srate_s[0] + S * alv;
  }
  for (int r = 0; r < R; r++) {
    const int L = r * 32 + lane;
    if (L > nzp - 2) continue;
    const double S = flag == 4 ? ws_s[L] + wq_s[L] : ws_s[L];
    tlt_s[L] = tlt_s[L] - (S * A.rdtlt) * (alv / LES_CP) * A.f.th[col + L] / A.f.tk[col + L];
  }
  __syncwarp();
}

__global__ void __launch_bounds__(128) sedimentation_kernel(const SedArgs A) {
  extern __shared__ double sed_smem[];
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5, nzp = A.nzp;
  // per block: dzt, 1/dzt and the slow fall-speed cap 0.5*(1/dzt)/dtlt (at most 2 m/s)
  double *blk = sed_smem;
  for (int k = threadIdx.x; k < nzp; k += blockDim.x) {
    const double dz = A.f.dzt[k], dzl = 1. / dz;
    blk[k] = dz;
    blk[nzp + k] = dzl;
    blk[2 * nzp + k] = fmin(0.5 * dzl / A.dtlt, 2.0);
  }
  __syncthreads();
  const long long c2 = (long long)blockIdx.x * (blockDim.x >> 5) + wib;   // column i + nxp*j
  if (c2 >= (long long)A.nxp * A.nyp) return;
  const int i = (int)(c2 % A.nxp), j = (int)(c2 / A.nxp);
  const long long col = (long long)nzp * c2, pl = A.plane;
  const bool fprc = A.sed[2], fice = A.sed[3] && A.lvl5;
  if (i < 2 || i > A.nxp - 3 || j < 2 || j > A.nyp - 3) {   // halo: the whole-array zeroing only
    for (int k = lane; k < nzp; k += 32) {
      A.f.rrate[col + k] = 0.;
      if (A.lvl5) A.f.irate[col + k] = 0.;
      if (fprc) for (int b = 0; b < A.P.nprc; b++) A.f.VtPrc[col + k + pl * b] = 0.;
      if (fice) for (int b = 0; b < A.P.nice; b++) A.f.VtIce[col + k + pl * b] = 0.;
    }
    if (lane == 0) {
      A.f.sfcrrate[c2] = 0.;
      if (A.lvl5) A.f.sfcirate[c2] = 0.;
    }
    return;
  }
  double *sm = sed_smem + 3 * nzp + (size_t)wib * A.warp_doubles;
  double *ad_s = sm + W_AD * nzp, *avis_s = sm + W_AVIS * nzp, *lam_s = sm + W_LAM * nzp, *ilam_s = sm + W_ILAM * nzp;
  double *tlt_s = sm + W_TLT * nzp, *rr_s = sm + W_RR * nzp, *ir_s = sm + W_IR * nzp, *sr_s = sm + A.off_sr;
  // air properties per level, atm modelling eq. 4.54 (:986-989)
  for (int k = lane; k < nzp; k += 32) {
    const long long p = col + k;
    const double ad = A.f.adn[p];
    ad_s[k] = ad;
    double avis = 0., lam = 0., ilam = 0.;
    if (k >= 1 && k <= nzp - 2) {
      const double T = A.f.tk[p], x = T / 296.16;
      avis = 1.8325e-5 * (416.16 / (T + 120.0)) * (x * sqrt(x));
      const double va = sqrt(8. * LES_KB * T / (LES_PI * SED_M));
      lam = 2. * avis / (ad * va);
      ilam = 1. / lam;
    }
    avis_s[k] = avis;
    lam_s[k] = lam;
    ilam_s[k] = ilam;
    tlt_s[k] = A.f.tlt[p];
    rr_s[k] = 0.;
    ir_s[k] = 0.;
  }
  if (lane == 0) sr_s[0] = sr_s[1] = 0.;
  __syncwarp();
  if (A.sed[0]) sed_slow(A, sm, blk, col, c2, A.P.nbins, 1, A.f.naero, A.f.maero, A.f.naerot, A.f.maerot, lane);
  if (A.sed[1]) sed_slow(A, sm, blk, col, c2, A.P.ncld, 2, A.f.ncloud, A.f.mcloud, A.f.ncloudt, A.f.mcloudt, lane);
  if (fprc)
    sed_fast(A, sm, blk, col, A.P.nprc, A.nspec, 3, A.f.nprecp, A.f.mprecp, A.f.nprecpt, A.f.mprecpt, A.f.VtPrc,
             rr_s, sr_s, lane);
  if (fice)
    sed_fast(A, sm, blk, col, A.P.nice, A.nspec + 1, 4, A.f.nice, A.f.mice, A.f.nicet, A.f.micet, A.f.VtIce, ir_s,
             sr_s + 1, lane);
  for (int k = lane; k < nzp; k += 32) {
    A.f.tlt[col + k] = tlt_s[k];
    A.f.rrate[col + k] = rr_s[k];
    if (A.lvl5) A.f.irate[col + k] = ir_s[k];
  }
  if (lane == 0) {
    A.f.sfcrrate[c2] = sr_s[0];
    if (A.lvl5) A.f.sfcirate[c2] = sr_s[1];
  }
}

// every non-NULL pointer must be device (or managed) memory
bool device_ptrs(std::initializer_list<const void *> ps) {
  for (const void *p : ps) {
    if (!p) continue;
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) { cudaGetLastError(); return false; }
    if (a.type != cudaMemoryTypeDevice && a.type != cudaMemoryTypeManaged) return false;
  }
  return true;
}

}  // namespace
}  // namespace salsa

extern "C" {

int salsa_gb300_tend_constrain(salsa_handle_t *h, int nzp, int nxp, int nyp, double dtlt,
                               const salsa_post_fields_t *f, void *stream) {
  salsa::DevParams P;
  cudaStream_t hs;
  int dev = 0, nsm = 0;
  if (!f || !salsa::handle_params(h, &P, &hs, &dev, &nsm)) return SALSA_E_ARG;
  if (nzp < 3 || nxp < 5 || nyp < 5 || !(dtlt > 0.)) return SALSA_E_ARG;
  const salsa_config_t *g = salsa::handle_config(h);
  const bool lvl5 = g->level == 5;
  salsa::ClampArgs A;
  const long long plane = (long long)nzp * nxp * nyp, nw = P.nwet;
  double *vp[9] = {f->naero, f->maero, f->ncloud, f->mcloud, f->nprecp, f->mprecp, f->gaero,
                   lvl5 ? f->nice : nullptr, lvl5 ? f->mice : nullptr};
  double *vt[9] = {f->naerot, f->maerot, f->ncloudt, f->mcloudt, f->nprecpt, f->mprecpt, f->gaerot,
                   lvl5 ? f->nicet : nullptr, lvl5 ? f->micet : nullptr};
  const long long np_[9] = {P.nbins, nw * P.nbins, P.ncld, nw * P.ncld, P.nprc, nw * P.nprc, 5, P.nice,
                            (nw + 1) * P.nice};
  for (int a = 0; a < 9; a++) { A.p[a] = vp[a]; A.t[a] = vt[a]; A.n[a] = np_[a] * plane; }
  A.dtlt = dtlt;
  long long bdt;
  memcpy(&bdt, &dtlt, sizeof bdt);
  A.be_dt = (int)((bdt >> 52) & 0x7ff);
  // a normal power of two with a normal reciprocal: mantissa zero
  const bool pow2 = (bdt & 0x000fffffffffffffLL) == 0 && A.be_dt > 1 && A.be_dt < 2045;
  A.rdt = pow2 ? 1. / dtlt : 0.;
  A.indef = (g->ice_theta_dist && g->level > 4) ? f->indef : nullptr;
  A.nindef = (long long)P.nliquid * plane;
  if (!salsa::device_ptrs({vp[0], vp[1], vp[2], vp[3], vp[4], vp[5], vp[6], vp[7], vp[8], vt[0], vt[1], vt[2], vt[3],
                           vt[4], vt[5], vt[6], vt[7], vt[8], A.indef}))
    return SALSA_E_ARG;
  if (cudaSetDevice(dev) != cudaSuccess) return SALSA_E_NODEV;
  cudaStream_t s = stream ? (cudaStream_t)stream : hs;
  salsa::tend_constrain_kernel<<<nsm * 8, 256, 0, s>>>(A);
  return cudaGetLastError() == cudaSuccess ? SALSA_OK : SALSA_E_CUDA;
}

int salsa_gb300_diagnostics(salsa_handle_t *h, int nzp, int nxp, int nyp, int only_diag, int lcharge,
                            const salsa_post_fields_t *f, void *stream) {
  salsa::DevParams P;
  cudaStream_t hs;
  int dev = 0, nsm = 0;
  if (!f || !salsa::handle_params(h, &P, &hs, &dev, &nsm)) return SALSA_E_ARG;
  if (nzp < 3 || nxp < 5 || nyp < 5) return SALSA_E_ARG;
  const salsa_config_t *g = salsa::handle_config(h);
  const bool lvl5 = g->level == 5;
  if (!f->naero || !f->ncloud || !f->nprecp || !f->maero || !f->mcloud || !f->mprecp || !f->rp || !f->rc ||
      !f->srp || !f->snrp || !f->rtot)
    return SALSA_E_ARG;
  if (lvl5 && (!f->nice || !f->mice || !f->ri || !f->riri)) return SALSA_E_ARG;
  if (!only_diag && (!f->rh || !f->temp || (lvl5 && !f->rhi) || (lcharge && !f->chargeTime) ||
                     (P.lscndgas && !f->gaero)))
    return SALSA_E_ARG;
  if (!salsa::device_ptrs({f->naero, f->ncloud, f->nprecp, f->nice, f->maero, f->mcloud, f->mprecp, f->mice, f->gaero,
                           f->chargeTime, f->rh, f->rhi, f->temp, f->rp, f->rc, f->srp, f->snrp, f->rtot, f->ri,
                           f->riri}))
    return SALSA_E_ARG;
  salsa::PostArgs A;
  A.plane = (long long)nzp * nxp * nyp;
  A.nzp = nzp; A.nxp = nxp; A.nyp = nyp;
  A.level = g->level; A.only_diag = only_diag; A.lcharge = lcharge; A.lscndgas = P.lscndgas;
  A.nbins = P.nbins; A.ncld = P.ncld; A.nprc = P.nprc; A.nice = P.nice;
  A.nspec = P.nwet; A.ndry = P.ndry; A.iwa = P.iwa; A.irim = P.irim;
  A.in1a = P.in1a; A.in2a = P.in2a; A.fn2a = P.fn2a; A.fn2b = P.fn2b;
  A.ica_cur = P.ica_cur; A.fca_cur = P.fca_cur; A.ica_par = P.ica_par;
  A.icb_cur = P.icb_cur; A.icb_par = P.icb_par; A.fcb_cur = P.fcb_cur;
  A.gas_ix[0] = P.ix_so4; A.gas_ix[1] = P.ix_oc; A.gas_ix[2] = P.ix_no; A.gas_ix[3] = P.ix_nh;
  for (int s = 0; s < 9; s++) {
    A.rholiq[s] = P.rholiq[s]; A.rhoice[s] = P.rhoice[s]; A.MM[s] = P.MM[s]; A.diss[s] = P.diss[s];
  }
  std::vector<double> lolim(P.ntotal);
  int nb = 0, ncl = 0, npr = 0, nic = 0, nwt = 0;
  if (salsa_gb300_layout(h, &nb, &ncl, &npr, &nic, &nwt, lolim.data()) != SALSA_OK || nb > SALSA_MAXBINS)
    return SALSA_E_ARG;
  for (int b = 0; b < nb; b++) A.aetot[b] = lolim[b];
  A.f = *f;
  if (cudaSetDevice(dev) != cudaSuccess) return SALSA_E_NODEV;
  cudaStream_t s = stream ? (cudaStream_t)stream : hs;
  long long grid = (A.plane + 127) / 128;
  if (grid > (long long)nsm * 16) grid = (long long)nsm * 16;
  salsa::diagnostics_kernel<<<(int)grid, 128, 0, s>>>(A);
  return cudaGetLastError() == cudaSuccess ? SALSA_OK : SALSA_E_CUDA;
}

int salsa_gb300_sedimentation(salsa_handle_t *h, int nzp, int nxp, int nyp, double dtlt, const int sed[4],
                              const salsa_sedim_fields_t *f, void *stream) {
  salsa::DevParams P;
  cudaStream_t hs;
  int dev = 0, nsm = 0;
  if (!f || !sed || !salsa::handle_params(h, &P, &hs, &dev, &nsm)) return SALSA_E_ARG;
  if (nzp < 3 || nxp < 5 || nyp < 5 || !(dtlt > 0.)) return SALSA_E_ARG;
  const salsa_config_t *g = salsa::handle_config(h);
  const bool lvl5 = g->level == 5;
  const int s0 = sed[0] != 0, s1 = sed[1] != 0, s2 = sed[2] != 0, s3 = sed[3] != 0 && lvl5;
  if (!f->tk || !f->th || !f->adn || !f->ustar || !f->dzt || !f->tlt || !f->rrate || !f->sfcrrate) return SALSA_E_ARG;
  if (lvl5 && (!f->irate || !f->sfcirate)) return SALSA_E_ARG;
  if ((s0 && (!f->naero || !f->maero || !f->naerot || !f->maerot)) ||
      (s1 && (!f->ncloud || !f->mcloud || !f->ncloudt || !f->mcloudt)) ||
      (s2 && (!f->nprecp || !f->mprecp || !f->nprecpt || !f->mprecpt || !f->VtPrc)) ||
      (s3 && (!f->nice || !f->mice || !f->nicet || !f->micet || !f->VtIce)))
    return SALSA_E_ARG;
  if (!salsa::device_ptrs({f->naero, f->ncloud, f->nprecp, f->nice, f->maero, f->mcloud, f->mprecp, f->mice,
                           f->naerot, f->ncloudt, f->nprecpt, f->nicet, f->maerot, f->mcloudt, f->mprecpt, f->micet,
                           f->tk, f->th, f->adn, f->ustar, f->dzt, f->tlt, f->rrate, f->irate, f->sfcrrate,
                           f->sfcirate, f->VtPrc, f->VtIce}))
    return SALSA_E_ARG;
  if (nzp > salsa::SED_KF || P.nwet < 2) return SALSA_E_UNSUPPORTED;
  salsa::SedArgs A;
  A.P = P;
  A.plane = (long long)nzp * nxp * nyp;
  A.nzp = nzp; A.nxp = nxp; A.nyp = nyp; A.nspec = P.nwet; A.lvl5 = lvl5;
  A.sed[0] = s0; A.sed[1] = s1; A.sed[2] = s2; A.sed[3] = s3;
  A.dtlt = dtlt;
  A.rdtlt = 1. / dtlt;
  for (int s = 0; s < 9; s++) {
    A.rrholiq[s] = P.rholiq[s] > 0. ? 1. / P.rholiq[s] : 0.;
    A.rrhoice[s] = P.rhoice[s] > 0. ? 1. / P.rhoice[s] : 0.;
  }
  A.f = *f;
  // shared layout: per block dzt, 1/dzt and the slow cap (3 nzp doubles); per warp the
  // per-level arrays (W_N nzp doubles), three int arrays (two level lists of nzp and
  // the activity words), the surface removal elements and the two surface rates
  const int nb_fast = std::max(s2 ? P.nprc : 0, s3 ? P.nice : 0);
  const int R = (nzp + 31) / 32;
  A.off_int = salsa::W_N * nzp;
  A.off_rem = A.off_int + (2 * nzp + R + 1) / 2;
  A.off_sr = A.off_rem + 1 + 2 * nb_fast;
  A.warp_doubles = A.off_sr + 2;
  const size_t wbytes = (size_t)A.warp_doubles * sizeof(double), bbytes = (size_t)3 * nzp * sizeof(double);
  int warps = 4;
  while (warps > 1 && bbytes + warps * wbytes > 100u * 1024u) warps >>= 1;
  const size_t smem = bbytes + warps * wbytes;
  if (smem > 200u * 1024u) return SALSA_E_UNSUPPORTED;
  if (cudaSetDevice(dev) != cudaSuccess) return SALSA_E_NODEV;
  if (smem > 48u * 1024u &&
      cudaFuncSetAttribute(salsa::sedimentation_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) !=
          cudaSuccess)
    return SALSA_E_CUDA;
  cudaStream_t s = stream ? (cudaStream_t)stream : hs;
  const long long cols = (long long)nxp * nyp, grid = (cols + warps - 1) / warps;
  salsa::sedimentation_kernel<<<(unsigned)grid, 32 * warps, smem, s>>>(A);
  return cudaGetLastError() == cudaSuccess ? SALSA_OK : SALSA_E_CUDA;
}

}  // extern "C"
