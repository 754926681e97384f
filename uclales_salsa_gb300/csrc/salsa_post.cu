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
#include <cuda_runtime.h>
#include <cstring>
#include <vector>
#include "../../include/salsa_gb300.h"
#include "salsa_device.cuh"
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
  int pow2;             // dtlt is a power of two
  int be_dt;            // biased exponent of dtlt
  unsigned long long cm;   // significand of |-1 + 1e-8| with its leading bit
  int ce;                  // biased exponent of |-1 + 1e-8|
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

// |(-1 + 1e-8) p| / dtlt for p > 0 normal and dtlt = 2^(1023 - dk) a power of two, as the
// bit pattern of a positive double, from the integer product of the significands rounded
// to nearest even: the bits of the FP64 product and power-of-two quotient whenever the
// result is normal, which is then exact.  Returns -1 where it would not be normal.
__device__ __forceinline__ long long mag_lo_bits(long long bp, unsigned long long cm, int ce, int dk) {
  const unsigned long long mp = ((unsigned long long)bp & 0x000fffffffffffffULL) | (1ULL << 52);
  const unsigned long long hi = __umul64hi(mp, cm), lo = mp * cm;   // product in [2^104, 2^106)
  const int ep = bexp(bp);
  unsigned long long m, r, half;
  int e;
  if (hi >> 41) { m = (hi << 11) | (lo >> 53); r = lo & ((1ULL << 53) - 1); half = 1ULL << 52; e = ep + ce - 1022; }
  else { m = (hi << 12) | (lo >> 52); r = lo & ((1ULL << 52) - 1); half = 1ULL << 51; e = ep + ce - 1023; }
  if (r > half || (r == half && (m & 1ULL))) {
    m++;
    if (m >> 53) { m >>= 1; e++; }
  }
  e += dk;
  if (e <= 0 || e >= 2047) return -1;
  return ((long long)e << 52) | (long long)(m & 0x000fffffffffffffULL);
}

// t = MAX((-1 + 1e-8) * p / dtlt, t), from the bit patterns bp, bt of p and t (the
// values are loaded as integers, so no FP64 compare is formed for the decisions taken on
// bits).  For p = +-0 the limit is the zero of the other sign (a finite positive dtlt).
// The limit is < 0 for a normal p > 0, so a tendency with its sign bit clear never moves;
// for t < 0 the exponents settle |t| < |lo| whenever |t| dtlt < p / 4.  The rest form lo:
// with a power-of-two dtlt from the integer product (mag_lo_bits) and compare magnitudes
// as integers (both negative), otherwise in FP64.
__device__ __forceinline__ void clamp_tendency(long long bp, long long bt, long long *tp, const ClampArgs &A) {
  if ((bp & ABS_MASK) == 0) {          // p = +-0: lo is the zero of the other sign
    if (neg_bits(bt)) *tp = bp == 0 ? (long long)0x8000000000000000ULL : 0LL;
    return;
  }
  if (bp >= 0 && bexp(bp) != 0 && bexp(bp) != 0x7ff) {
    if (bt >= 0) return;
    if (bexp(bt) + A.be_dt + 3 - 1023 <= bexp(bp)) return;
    if (A.pow2 && (bt & ABS_MASK) <= INF_BITS) {
      const long long ml = mag_lo_bits(bp, A.cm, A.ce, 1023 - A.be_dt);
      if (ml >= 0) {
        // lo = -|lo| > t  <=>  |lo| < |t| (t < 0, not NaN)
        if (ml < (bt & ABS_MASK)) *tp = ml | (long long)0x8000000000000000ULL;
        return;
      }
    }
  }
  const double q = (-1. + 1.e-8) * __longlong_as_double(bp);
  const double lo = A.pow2 ? q * A.rdt : q / A.dtlt;   // the same rounding of the same quotient
  if (lo > __longlong_as_double(bt)) *tp = __double_as_longlong(lo);
}

__global__ void __launch_bounds__(256) tend_constrain_kernel(const ClampArgs A) {
  const long long stride = (long long)gridDim.x * blockDim.x;
  const long long i0 = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  constexpr int B = 4;   // elements per thread and pass, loaded before any store
  for (int a = 0; a < 9; a++) {
    const long long *__restrict__ p = reinterpret_cast<const long long *>(A.p[a]);
    long long *__restrict__ t = reinterpret_cast<long long *>(A.t[a]);
    if (!p || !t) continue;
    const long long n = A.n[a];
    for (long long e0 = i0; e0 < n; e0 += B * stride) {
      long long vp[B], vt[B];
#pragma unroll
      for (int u = 0; u < B; u++) {
        const long long e = e0 + u * stride;
        vp[u] = e < n ? __ldg(p + e) : 0LL;
        vt[u] = e < n ? t[e] : 0LL;
      }
#pragma unroll
      for (int u = 0; u < B; u++) {
        const long long e = e0 + u * stride;
        if (e < n) clamp_tendency(vp[u], vt[u], t + e, A);
      }
    }
  }
  // the IN deficit to [0, 1] (MIN(MAX(v, 0), 1)), decided on the bits: NaN and v < 0
  // become 0, v > 1 becomes 1; -0 and values inside stay as they are
  if (A.indef) {
    const long long ONE = 0x3ff0000000000000LL;
    long long *in = reinterpret_cast<long long *>(A.indef);
    for (long long e = i0; e < A.nindef; e += stride) {
      const long long b = in[e], m = b & ABS_MASK;
      if (m > INF_BITS || neg_bits(b)) in[e] = 0LL;
      else if (b > ONE) in[e] = ONE;
    }
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
// at most 64 registers (8 blocks of 128 threads per SM): a point's passes over its bins
// are dependent loads, so the kernel is bound by latency and gains from warps in flight
__global__ void __launch_bounds__(128, 8) diagnostics_kernel(const PostArgs A) {
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
  A.pow2 = pow2 ? 1 : 0;
  {
    const double c = -1. + 1.e-8;   // the factor of the limit, as tend_constrain2 writes it
    const double cabs = -c;
    long long bc;
    memcpy(&bc, &cabs, sizeof bc);
    A.cm = ((unsigned long long)bc & 0x000fffffffffffffULL) | (1ULL << 52);
    A.ce = (int)((bc >> 52) & 0x7ff);
  }
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

}  // extern "C"
