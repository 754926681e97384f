// salsa_sedim.cu -- bin sedimentation after a SALSA step: sedim_SALSA
// (src/src_LES/mcrp.f90:745-1275, DepositionSlow and DepositionFast) on the arrays of
// the LES, device pointers.  Compiled with multiply-add contraction: the kernel is
// bound by the FP64 pipe, and its parity bound is a tolerance, not the last bit.
#include <cuda_runtime.h>
#include <algorithm>
#include <cstring>
#include "../../include/salsa_gb300.h"
#include "salsa_kernel_impl.cuh"
#include "salsa_internal.h"

namespace salsa {
namespace {

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
// taken as products with a reciprocal, and products and sums contract to fused
// multiply-adds, which moves results by an ulp or so.  Halo
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
enum { W_AD = 0, W_AVIS, W_LAM, W_ILAM, W_R18, W_Q, W_TLT, W_RR, W_IR, W_VC, W_P0, W_P1, W_P2, W_P3, W_N };

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
                                          double ad, double avis, double lam, double ilam, double r18v, double &dwet,
                                          double &GG) {
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
  if (flag <= 3 && dwet <= 19E-6) return sq(dwet) * (zdn - ad) * K_GRAV * GG * r18v;   // Stokes, eq. 3.21
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
               *ilam_s = sm + W_ILAM * nzp, *r18_s = sm + W_R18 * nzp, *q_s = sm + W_Q * nzp;
  double *tlt_s = sm + W_TLT * nzp, *rr_s = sm + W_RR * nzp, *vc_s = sm + W_VC * nzp;
  double *rs_s = sm + W_P0 * nzp, *ts_s = sm + W_P1 * nzp, *wr_s = sm + W_P2 * nzp, *wd_s = sm + W_P3 * nzp;
  int *la = (int *)(sm + A.off_int), *lf = la + nzp;
  unsigned *actw = (unsigned *)(lf + nzp);
  double *sr_s = sm + A.off_sr;
  const double *vmax_b = blk + 2 * nzp;
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
      double vc = sed_vel(A, flag, ns, n, m, ad_s[k], avis_s[k], lam_s[k], ilam_s[k], r18_s[k], dwet, GG);
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
      const double ad = ad_s[k], adp = ad_s[k + 1], q = q_s[k];
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
               *ilam_s = sm + W_ILAM * nzp, *r18_s = sm + W_R18 * nzp;
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
      const double vc = sed_vel(A, flag, ns, n, m, ad, avis_s[kc], lam_s[kc], ilam_s[kc], r18_s[kc], dwet, GG);
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
  double *ad_s = sm + W_AD * nzp, *avis_s = sm + W_AVIS * nzp, *lam_s = sm + W_LAM * nzp, *ilam_s = sm + W_ILAM * nzp,
         *r18_s = sm + W_R18 * nzp, *q_s = sm + W_Q * nzp;
  double *tlt_s = sm + W_TLT * nzp, *rr_s = sm + W_RR * nzp, *ir_s = sm + W_IR * nzp, *sr_s = sm + A.off_sr;
  // air properties per level, atm modelling eq. 4.54 (:986-989)
  for (int k = lane; k < nzp; k += 32) {
    const long long p = col + k;
    const double ad = A.f.adn[p];
    ad_s[k] = ad;
    double avis = 0., lam = 0., ilam = 0., r18 = 0., q = 0.;
    if (k >= 1 && k <= nzp - 2) {
      const double T = A.f.tk[p], x = T / 296.16;
      avis = 1.8325e-5 * (416.16 / (T + 120.0)) * (x * sqrt(x));
      const double va = sqrt(8. * LES_KB * T / (LES_PI * SED_M));
      lam = 2. * avis / (ad * va);
      ilam = 1. / lam;
      r18 = 1. / (18. * avis);
      q = A.f.dzt[k] / ad;
    }
    avis_s[k] = avis;
    lam_s[k] = lam;
    ilam_s[k] = ilam;
    r18_s[k] = r18;
    q_s[k] = q;
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

}  // namespace
}  // namespace salsa

extern "C" {

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
