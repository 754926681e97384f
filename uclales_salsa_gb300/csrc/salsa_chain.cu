// salsa_chain.cu -- gradient harness: chains of coagulation + condensation steps.
//
// A chain advances independent cells through nsub steps of length dt.  Each step is
// the coagulation (mo_salsa_dynamics.f90:92-202 with the kernels and the update of
// mo_salsa_coagulation_kernels.f90 / mo_salsa_coagulation_processes.f90) followed by
// the water condensation (gpparth2o, mo_salsa_dynamics.f90:691-1125, with the
// aerosol water uptake of mo_salsa_properties.f90:73-380), in warm (level 4) cells
// whose precipitation bins stay empty, with no autoconversion, activation or bin
// redistribution.  The water vapour is imposed at the start of every step,
// rv = rs (1 + s), and the solute term of the water activity is kappa * V_soluble.
//
// Three kernels share one generic step, chain_step<R>:
//   * chain_forward_kernel  (R = double): the chain, with optional checkpoints;
//   * chain_tlm_kernel      (R = Dual<1>): the tangent-linear model of the chain;
//   * the adjoint (R = double), hand-written, run step by step from the last step:
//     chain_taped_kernel recomputes the step of every cell from its checkpoint (or
//     from the states chain_seg_kernel recomputed inside a checkpoint segment) and
//     tapes the intermediate states, the condensation substep history and the
//     collision kernels with their diameter derivatives; chain_rev_kernel then runs
//     the adjoint of each stage in reverse order.  Local partial derivatives of the
//     collision kernel, the mass-transfer coefficients and one water-uptake
//     iteration come from dual-number evaluations of the same code.
// One warp owns one cell; lanes split bins and bin pairs as in the step kernel.
#include <cuda_runtime.h>
#include <type_traits>
#include "../../include/salsa_gb300.h"
#include "salsa_kernel_impl.cuh"
#include "salsa_dual.cuh"
#include "salsa_internal.h"

// Sub-stage clocks of the instrumented build (stage_profile --chain): a warp adds the
// clock64() delta since the previous mark to counter k.
#ifdef SALSA_STAGE_TIMERS
#define SUB_BEGIN() long long t_sub = clock64()
#define SUB_MARK(k)                                                                               \
  do {                                                                                            \
    long long t_ = clock64();                                                                     \
    if (lane == 0 && P.stage_clocks) atomicAdd(P.stage_clocks + (k), (unsigned long long)(t_ - t_sub)); \
    t_sub = t_;                                                                                   \
  } while (0)
#else
#define SUB_BEGIN() do { } while (0)
#define SUB_MARK(k) do { } while (0)
#endif

namespace salsa {
namespace {

// dual-number forms of the math templates used by bin_props / coag_pair / terminal_vel
template <> __device__ __forceinline__ Dual<1> t_exp<Dual<1>>(Dual<1> x) { return d_exp(x); }
template <> __device__ __forceinline__ Dual<1> t_log<Dual<1>>(Dual<1> x) { return d_log(x); }
template <> __device__ __forceinline__ Dual<1> t_sqrt<Dual<1>>(Dual<1> x) { return d_sqrt(x); }
template <> __device__ __forceinline__ Dual<1> t_cbrt<Dual<1>>(Dual<1> x) { return d_cbrt(x); }
template <> __device__ __forceinline__ Dual<1> t_pow<Dual<1>>(Dual<1> x, Dual<1> y) { return d_pow(x, y); }
template <> __device__ __forceinline__ Dual<2> t_exp<Dual<2>>(Dual<2> x) { return d_exp(x); }
template <> __device__ __forceinline__ Dual<2> t_log<Dual<2>>(Dual<2> x) { return d_log(x); }
template <> __device__ __forceinline__ Dual<2> t_sqrt<Dual<2>>(Dual<2> x) { return d_sqrt(x); }
template <> __device__ __forceinline__ Dual<2> t_cbrt<Dual<2>>(Dual<2> x) { return d_cbrt(x); }
template <> __device__ __forceinline__ Dual<2> t_pow<Dual<2>>(Dual<2> x, Dual<2> y) { return d_pow(x, y); }

// generic math for the step (double or dual)
__device__ __forceinline__ double g_cbrt(double x) { return cbrt(x); }
__device__ __forceinline__ double g_exp(double x) { return exp(x); }
template <int N> __device__ __forceinline__ Dual<N> g_cbrt(const Dual<N> &x) { return d_cbrt(x); }
template <int N> __device__ __forceinline__ Dual<N> g_exp(const Dual<N> &x) { return d_exp(x); }
__device__ __forceinline__ double g_fma(double a, double b, double c) { return fma(a, b, c); }
// the value rounds once, as fma(double) does, so a dual run's values equal the plain run's
template <int N>
__device__ __forceinline__ Dual<N> g_fma(const Dual<N> &a, const Dual<N> &b, const Dual<N> &c) {
  Dual<N> r;
  r.v = fma(a.v, b.v, c.v);
#pragma unroll
  for (int i = 0; i < N; i++) r.d[i] = fma(a.d[i], b.v, fma(a.v, b.d[i], c.d[i]));
  return r;
}
template <typename R> __device__ __forceinline__ R g_wsum(R v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += shfl_xor(v, o);
  return v;
}
template <typename R> __device__ __forceinline__ R g_acth2o(R znw, R zns) {   // acth2o_w
  return fmax(R(0.1), znw / fmax(R(K_EPS), znw + zns));
}

// ---- per-cell constants of a chain ----
template <typename R>
struct ChainCell {
  double T, pres, prs, dn, rhoair;
  R kappa, prv0;     // solute hygroscopicity; imposed vapour rs (1 + s)
};

// ---- per-warp workspace (shared memory) of the generic step ----
//   n[NL], v[NW][NL]  state in SALSA units (#/m3, m3/m3); bins 0..NL-1 are the liquid bins
//   dw[NL]            diameters at the start of the coagulation
//   K[NL (NL+1)/2]    collision kernels of the liquid bins (i <= j)
//   S[9][NL]          per-bin collision properties
//   kel, surf, mt, wsat, cw, zns [NL]  condensation coefficients and substep state
template <typename R>
struct CW {
  R *n, *v, *dw, *K, *S, *kel, *surf, *mt, *wsat, *cw, *zns;
  int *pbuf;
  int NL;
  __device__ __forceinline__ R &V(int s, int b) const { return v[s * NL + b]; }
  __device__ __forceinline__ R &Kij(int i, int j) const { return i <= j ? K[tri(i, j, NL)] : K[tri(j, i, NL)]; }
};

__host__ __device__ __forceinline__ int chain_tri(int NL) { return NL * (NL + 1) / 2; }
// R-typed entries of the workspace, then 64 ints of compaction buffer
__host__ __device__ __forceinline__ int chain_ws_entries(int NL, int NW) {
  return NL + NW * NL + NL + chain_tri(NL) + 9 * NL + 6 * NL;
}

template <typename R>
__device__ __forceinline__ CW<R> make_cw(R *base, int NL, int NW) {
  CW<R> w;
  w.NL = NL;
  R *p = base;
  w.n = p; p += NL;
  w.v = p; p += NW * NL;
  w.dw = p; p += NL;
  w.K = p; p += chain_tri(NL);
  w.S = p; p += 9 * NL;
  w.kel = p; p += NL;
  w.surf = p; p += NL;
  w.mt = p; p += NL;
  w.wsat = p; p += NL;
  w.cw = p; p += NL;
  w.zns = p; p += NL;
  w.pbuf = reinterpret_cast<int *>(p);
  return w;
}

// ---- tape of one step (global memory, doubles, per cell) ----
enum { TP_MAXEQ = 104 };
struct TapeLayout {
  int x_in, x_pre, x_mid, x_eq, sums, K, dki, dkj, eq, hist_zc, hist_c, hist_w, nit, maxit, total;
};
// maxit: substep rows of the condensation history (the loop count plus the final row)
__host__ __device__ __forceinline__ TapeLayout tape_layout(int NL, int NW, int n1a, int maxit) {
  TapeLayout t;
  const int ns = NL * (1 + NW), tr = NL * (NL + 1) / 2;
  t.maxit = maxit;
  t.x_in = 0;
  t.x_pre = t.x_in + ns;                    // after the coagulation sweep, before the clamp
  t.x_mid = t.x_pre + ns;
  t.x_eq = t.x_mid + ns;
  t.sums = t.x_eq + ns;                     // per coagulation target: sink, self, src[NSV]
  t.K = t.sums + NL * (2 + SALSA_NSV);      // collision kernels of the step
  t.dki = t.K + tr;                         // dK/dd_i and dK/dd_j of every pair (i <= j)
  t.dkj = t.dki + tr;
  t.eq = t.dkj + tr;                        // per 1a bin: [count, zke_0 .. zke_count]
  t.hist_zc = t.eq + n1a * TP_MAXEQ;        // per substep: zcwc entering it
  t.hist_c = t.hist_zc + maxit;             // per substep: c of every bin entering it
  t.hist_w = t.hist_c + maxit * NL;         // per substep: wsat of every bin entering it
  t.nit = t.hist_w + maxit * NL;            // number of substeps; then the cell's void flag
  t.total = t.nit + 2;
  return t;
}
__host__ __device__ __forceinline__ int tape_maxit(double dt) { return (int)(dt / 2.e-2) + 3; }

__device__ __forceinline__ void state_to_tape(double *dst, const double *n, const double *v, int NL, int NW, int lane) {
  for (int e = lane; e < NL * (1 + NW); e += 32) dst[e] = e < NL ? n[e] : v[e - NL];
}
__device__ __forceinline__ void tape_to_state(const double *src, double *n, double *v, int NL, int NW, int lane) {
  for (int e = lane; e < NL * (1 + NW); e += 32) {
    if (e < NL) n[e] = src[e];
    else v[e - NL] = src[e];
  }
}

// ---------------------------------------------------------------------------------------
// Generic step (R = double or Dual<1>).  Each stage restates the step kernel's code for
// the liquid bins with the same operation order, so the R = double chain reproduces the
// step kernel's coagulation + condensation bit for bit.
// ---------------------------------------------------------------------------------------
template <typename R>
__device__ __forceinline__ R liquid_dwet(const DevParams &P, const CW<R> &w, const double *dmid, int b) {
  // updateDiameterAll, wet diameter of a liquid bin (classSection.f90:91-159)
  const int ph = phase_of(P, b);
  R dw;
  if (val(w.n[b]) > nlim_of(ph)) {
    R vs = R(0.);
    for (int s = 0; s < P.nwet; s++) vs += w.V(s, b);
    dw = g_cbrt(vs * (R(1.) / (w.n[b] * K_PI6)));   // as the step kernel's updateDiameterAll
  } else {
    dw = R(dmid[b]);
  }
  return fmin(dw, R(dlim_of(ph)));
}

template <typename R>
__device__ __forceinline__ CoagCell<R> chain_coagcell(double T, double pres, const DevParams &P) {
  const double visc = (7.44523e-3 * sqrt(cube(T))) / (5093. * (T + 110.4));
  const double mfp = (1.656e-10 * T + 1.828e-8) * K_PSTAND / pres;
  const double zrhoa = pres / (K_RD * T);
  const double vkin = visc / zrhoa;
  CoagCell<R> c;
  c.T_ = R(T); c.visc = R(visc); c.mfp = R(mfp); c.zrhoa = R(zrhoa); c.vkin = R(vkin);
  c.shearA = R(sqrt(8. * K_PI * P.eddy_dis / (15. * vkin)));
  c.turbB = R(K_PI * pow(P.eddy_dis, 0.75) / (K_GRAV * sqrt(sqrt(vkin))));
  return c;
}

template <typename R>
__device__ __forceinline__ void chain_store_props(R *S, int NL, int b, const BinProps<R> &o) {
  const R *po = &o.diam;
#pragma unroll
  for (int k = 0; k < 9; k++) S[k * NL + b] = po[k];
}
template <typename R>
__device__ __forceinline__ void chain_load_props(const R *S, int NL, int b, BinProps<R> &o) {
  R *po = &o.diam;
#pragma unroll
  for (int k = 0; k < 9; k++) po[k] = S[k * NL + b];
}

// Populated bins (number at or above the bin's limit), compacted into pbuf in bin order;
// returns their count.  Bins below the limit have no collision properties and every
// pair with such a bin has K = 0 (the step kernel's build_kernels does the same).
template <typename R>
__device__ __forceinline__ int chain_active_bins(const DevParams &P, const CW<R> &w, int lane) {
  const unsigned lt = (1u << lane) - 1u;
  int nact = 0;
  for (int base = 0; base < w.NL; base += 32) {
    const int b = base + lane;
    const bool act = b < w.NL && val(w.n[b]) >= nlim_of(phase_of(P, b));
    const unsigned bal = __ballot_sync(0xffffffffu, act);
    if (act) w.pbuf[nact + __popc(bal & lt)] = b;
    nact += __popc(bal);
  }
  __syncwarp();
  return nact;
}

// Scans the pair table section by section (pairs of unequal, then of equal bin sizes),
// compacts the pairs of two populated bins into pbuf and calls f(sec, pair) for 32 of
// them at a time, one per lane, then for the rest; zero(pair) is called for the pairs
// with an empty bin.  Lanes never idle on an empty pair.
template <typename R, typename F, typename Z>
__device__ __forceinline__ void chain_pairs(const DevParams &P, const CW<R> &w, int lane, F f, Z zero) {
  const unsigned lt = (1u << lane) - 1u;
  for (int sec = 0; sec < 2; sec++) {
    const int p0 = sec == 0 ? 0 : P.npairs_plain, p1 = sec == 0 ? P.npairs_plain : P.npairs;
    int nbuf = 0;
    for (int base = p0; base < p1; base += 32) {
      const int t = base + lane;
      bool act = false;
      int pk = 0;
      if (t < p1) {
        pk = __ldg(P.pairs + t);
        const int i = pk & 0xff, j = (pk >> 8) & 0xff;
        act = val(w.n[i]) >= nlim_of(phase_of(P, i)) && val(w.n[j]) >= nlim_of(phase_of(P, j));
        if (!act) zero(pk);
      }
      const unsigned bal = __ballot_sync(0xffffffffu, act);
      if (act) w.pbuf[nbuf + __popc(bal & lt)] = pk;
      nbuf += __popc(bal);
      __syncwarp();
      if (nbuf >= 32) {
        f(sec, w.pbuf[nbuf - 32 + lane]);
        nbuf -= 32;
        __syncwarp();
      }
    }
    if (lane < nbuf) f(sec, w.pbuf[lane]);
    __syncwarp();
  }
}

// Collision properties of populated bin b, and the kernel of its pairs of equal bin size
// (coagc :273-276: the first particle of such a pair is taken 1.1 times larger and 1.33
// times heavier).  For liquid bins that first particle's properties depend on bin j of
// the pair alone: terminal_vel takes the same branch for every liquid phase and the
// sphere-equivalent diameter enters only for ice.  So every equal-size pair (i, j) of the
// chain's liquid bins has the kernel of bin j, evaluated once per bin here.
template <typename R>
__device__ __forceinline__ R chain_bin_props(const DevParams &P, const CoagCell<R> &cc, int b, R d, BinProps<R> &o) {
  Shape<R> sh;
  sh.alpha = sh.beta = sh.gamma = sh.sigma = R(0.);
  const R mass = R(K_RHOWA * K_PI6) * cube(d);
  bin_props<R>(cc, phase_of(P, b), d, d, mass, R(K_RHOWA), sh, o);
  BinProps<R> big;
  bin_props<R>(cc, phase_of(P, b), R(1.1) * d, d, R(1.33) * mass, R(K_RHOWA), sh, big);
  return coag_pair<R>(cc, big, o);
}

// diameters at the start of the coagulation, collision properties and kernels
template <typename R>
__device__ void chain_kernels(const DevParams &P, const CW<R> &w, const double *tb, double T, double pres, int lane) {
  const int NL = w.NL;
  const double *dmid = tb + TAB_DMID * P.nb_pad;
  const CoagCell<R> cc = chain_coagcell<R>(T, pres, P);
  for (int b = lane; b < NL; b += 32) w.dw[b] = liquid_dwet(P, w, dmid, b);
  __syncwarp();
  R *keq = w.kel;   // equal-size kernel per bin (the condensation rows are free here)
  const int nact = chain_active_bins(P, w, lane);
  for (int e = lane; e < nact; e += 32) {
    const int b = w.pbuf[e];
    BinProps<R> o;
    keq[b] = chain_bin_props<R>(P, cc, b, w.dw[b], o);
    chain_store_props<R>(w.S, NL, b, o);
  }
  __syncwarp();
  chain_pairs(
      P, w, lane,
      [&](int sec, int pk) {
        const int i = pk & 0xff, j = (pk >> 8) & 0xff;
        if (sec == 1) {
          w.K[tri(i, j, NL)] = keq[j];
          return;
        }
        BinProps<R> a, bb;
        chain_load_props<R>(w.S, NL, i, a);
        chain_load_props<R>(w.S, NL, j, bb);
        w.K[tri(i, j, NL)] = coag_pair<R>(cc, a, bb);
      },
      [&](int pk) { w.K[tri(pk & 0xff, (pk >> 8) & 0xff, NL)] = R(0.); });
  __syncwarp();
}

// semi-implicit update of one target from its reduced sums (applyCoag, :539-559)
template <typename R>
__device__ __forceinline__ void chain_apply(const CW<R> &w, int t, int nspec, double dt, R (&src)[SALSA_NSV], R sink,
                                            R self, int lane) {
  R my = R(0.);
#pragma unroll
  for (int s = 0; s < SALSA_NSV; s++)
    if (lane == s) my = src[s];
  const R n = w.n[t];
  const bool vol = lane < nspec;
  const R num = vol ? w.V(lane, t) + dt * my * n : n;
  const R den = vol ? 1. + dt * sink : 1. + dt * (sink + self);
  const R q = num / den;
  __syncwarp();
  if (vol) w.V(lane, t) = q;
  else if (lane == nspec) w.n[t] = q;
  __syncwarp();
}

// warp totals of the sums of one target; in FP64 the eight sums share one transposed
// butterfly (warp_sum8: the same addition tree as g_wsum, so the same totals)
template <typename R>
__device__ __forceinline__ void chain_reduce(R (&src)[SALSA_NSV], R &sink, R &self, int lane) {
  static_assert(SALSA_NSV == 7, "src and sink fill the eight slots of warp_sum8");
  if constexpr (std::is_same<R, double>::value) {
    double v[8];
#pragma unroll
    for (int s = 0; s < 7; s++) v[s] = src[s];
    v[7] = sink;
    warp_sum8(v, lane);
#pragma unroll
    for (int s = 0; s < 7; s++) src[s] = v[s];
    sink = v[7];
  } else {
#pragma unroll
    for (int s = 0; s < SALSA_NSV; s++) src[s] = g_wsum(src[s]);
    sink = g_wsum(sink);
  }
  self = shfl_idx(self, 0);
}

// Sources of cloud target tg (coag_cloud, :320-420 without precipitation formation):
// aerosol bins in1a..iaa and in2b..iab, then cloud bins kfirst..kk-1 and o_first..other.
// f(g) is called for every partner g of this lane, in the step kernel's lane order.
template <typename F>
__device__ __forceinline__ void cloud_sources(const DevParams &P, int kk, int kfirst, int o_first, int lane, F f) {
  const int C0 = P.nbins, rel = kk - kfirst, other = o_first + rel;
  if (P.lscgca) {
    const int iaa = P.ica_par + rel, iab = P.icb_par + rel;
    for (int ll = P.in1a + lane; ll <= iaa; ll += 32) f(ll);
    for (int ll = P.in2b + lane; ll <= iab; ll += 32) f(ll);
  }
  if (P.lscgcc && kk > kfirst) {
    for (int ll = kfirst + lane; ll <= kk - 1; ll += 32) f(C0 + ll);
    for (int ll = o_first + lane; ll <= other; ll += 32) f(C0 + ll);
  }
}

// Gauss-Seidel coagulation update of the aerosol, then the cloud targets
// (mo_salsa_dynamics.f90:160-186); chain_coag_clamp is the clamp of :188-197.
template <typename R>
__device__ __forceinline__ void tape_sums(double *ts, int t, const R (&src)[SALSA_NSV], R sink, R self, int lane) {
  if (ts && lane == 0) {
    double *o = ts + t * (2 + SALSA_NSV);
    o[0] = val(sink); o[1] = val(self);
    for (int s = 0; s < SALSA_NSV; s++) o[2 + s] = val(src[s]);
  }
}

template <typename R>
__device__ void chain_coag_update(const DevParams &P, const CW<R> &w, const double *tb, double dt, int lane,
                                  double *ts = nullptr) {
  const int nspec = P.nwet;
  const int16_t *L = partner_lists(P, tb);
  for (int kk = P.in1a; kk <= P.fn2b; kk++) {
    if (val(w.n[kk]) < K_NLIM) continue;
    R src[SALSA_NSV], sink = R(0.), self = R(0.);
#pragma unroll
    for (int s = 0; s < SALSA_NSV; s++) src[s] = R(0.);
    if (P.lscgaa && lane == 0) self = 0.5 * w.Kij(kk, kk) * w.n[kk];
    {
      const int off = L[4 * kk], n = L[4 * kk + 1];
      for (int e = lane; e < n; e += 32) { const int g = L[off + e]; sink += w.Kij(kk, g) * w.n[g]; }
    }
    {
      const int off = L[4 * kk + 2], n = L[4 * kk + 3];
      for (int e = lane; e < n; e += 32) {
        const int g = L[off + e];
        const R k = w.Kij(g, kk);
#pragma unroll
        for (int s = 0; s < SALSA_NSV; s++)
          if (s < nspec) src[s] += k * w.V(s, g);
      }
    }
    chain_reduce(src, sink, self, lane);
    tape_sums(ts, kk, src, sink, self, lane);
    chain_apply(w, kk, nspec, dt, src, sink, self, lane);
  }
  const int C0 = P.nbins;
  for (int reg = 0; reg < 2; reg++) {
    const int kfirst = reg == 0 ? P.ica_cur : P.icb_cur, klast = reg == 0 ? P.fca_cur : P.fcb_cur;
    const int o_first = reg == 0 ? P.icb_cur : P.ica_cur;
    for (int kk = kfirst; kk <= klast; kk++) {
      const int tg = C0 + kk;
      if (val(w.n[tg]) < K_NLIM) continue;
      R src[SALSA_NSV], sink = R(0.), self = R(0.);
#pragma unroll
      for (int s = 0; s < SALSA_NSV; s++) src[s] = R(0.);
      {
        const int off = L[4 * tg], n = L[4 * tg + 1];
        for (int e = lane; e < n; e += 32) { const int g = L[off + e]; sink += w.Kij(tg, g) * w.n[g]; }
      }
      if (P.lscgcc && lane == 0) self += 0.5 * w.Kij(tg, tg) * w.n[tg];
      cloud_sources(P, kk, kfirst, o_first, lane, [&](int g) {
        const R k = w.Kij(g, tg);
#pragma unroll
        for (int s = 0; s < SALSA_NSV; s++)
          if (s < nspec) src[s] += k * w.V(s, g);
      });
      chain_reduce(src, sink, self, lane);
      tape_sums(ts, tg, src, sink, self, lane);
      chain_apply(w, tg, nspec, dt, src, sink, self, lane);
    }
  }
}

template <typename R>
__device__ void chain_coag_clamp(const DevParams &P, const CW<R> &w, int lane) {
  for (int b = lane; b < w.NL; b += 32) {
    w.n[b] = fmax(R(0.), w.n[b]);
    for (int s = 0; s < P.nwet; s++) w.V(s, b) = fmax(R(0.), w.V(s, b));
  }
  __syncwarp();
}

// ---- condensation (gpparth2o) ----
template <typename R>
__device__ __forceinline__ R chain_zvolc(const DevParams &P, const CW<R> &w, int which, int b) {
  const int ix[7] = {P.ix_so4, P.ix_oc, P.ix_bc, P.ix_du, P.ix_ss, P.ix_no, P.ix_nh};
  const int d = ix[which];
  return (d >= 0 && which < 5) ? w.V(d, b) : R(0.);
}

// one iteration of the regime-1a water uptake (equil_iterate, :196-245) in the form of
// the step kernel's eq_step, operation for operation: izke = 1/zke -> (zlwc, zdwet, izke')
template <typename R>
__device__ __forceinline__ void eq1a_iter(R zrh, R &izke, R zv0, R zv1, R numc, R zvp56, R zcore, double T, R &zlwc,
                                          R &zdwet) {
  const double rhosu_msu = 1830. / 98.08e-3, rhooc_moc = 1400. / 150.e-3;
  const double ckt = 2. * K_SURFW0 * K_MVWA / (K_BOLTZ * T);
  R zaw = zrh * izke;
  R a2 = zaw * zaw, a3 = a2 * zaw, a4 = a2 * a2;
  R bm1 = +1.1065495e+2 - 3.6759197e+2 * zaw + 5.0462934e+2 * a2 - 3.1543839e+2 * a3 + 6.770824e+1 * a4;
  R bm2 = 1. / (zaw * K_MWA) - 1. / K_MWA;
  R q0 = zv0 * rhosu_msu, q1 = K_EPSOC * zv1 * rhooc_moc;
  zlwc = g_fma(q1, bm1, q0 * bm2) / (bm1 * bm2);
  R rinv = 1. / (numc * (K_RHOWA * K_PI6));
  zdwet = g_cbrt(g_fma(zlwc, rinv, zvp56 / K_PI6) + zcore / K_PI6);
  izke = g_exp(-(ckt / zdwet));
}

// the regime-1a chain of the non-initialising equilibration (:160-250), on every lane
template <typename R>
__device__ void chain_equil_1a(const DevParams &P, const CW<R> &w, R prh, double T, double *tp_eq, int lane) {
  R izke = R(1. / 1.001);   // 1/zke, carried from bin to bin
  const R zrh = fmin(fmax(prh, R(0.05)), R(0.98));
  for (int kk = P.in1a; kk <= P.fn1a; kk++) {
    double *te = tp_eq ? tp_eq + (kk - P.in1a) * TP_MAXEQ : nullptr;
    if (!(val(w.n[kk]) > K_NLIM)) {
      if (te && lane == 0) te[0] = -1.;
      continue;
    }
    const R numc = w.n[kk];
    const R zv0 = chain_zvolc(P, w, 0, kk), zv1 = chain_zvolc(P, w, 1, kk);
    R zvp[7];
    for (int i = 0; i < 7; i++) zvp[i] = chain_zvolc(P, w, i, kk) / numc;
    const R zcore = zvp[0] + zvp[1];
    const R zvp56 = zvp[5] + zvp[6];
    double zdwet = val(w.dw[kk]), zdold = 1.;
    R zlwc = R(0.);
    int count = 0;
    if (te && lane == 0) te[1] = val(izke);
    while (fabs(zdwet - zdold) > 1.e-2 * zdold) {   // |zdwet/zdold - 1| > 1e-2, zdold > 0
      zdold = fmax(zdwet, 1.e-20);
      R zd;
      eq1a_iter(zrh, izke, zv0, zv1, numc, zvp56, zcore, T, zlwc, zd);
      zdwet = val(zd);
      count++;
      if (te && lane == 0 && count + 1 < TP_MAXEQ) te[count + 1] = val(izke);
      if (count > 100) break;
    }
    if (te && lane == 0) te[0] = (double)count;
    __syncwarp();
    if (lane == 0) w.V(P.iwa, kk) = zlwc / K_RHOWA;
    __syncwarp();
  }
}

// per-bin condensation coefficients (:819-955) for the liquid bins
template <typename R>
__device__ __forceinline__ void cond_coeffs(R n, R dwet, R znw, R zns, double T, double prs, double rhoair, double zdfh2o,
                                            double zmfph2o, double zthcond, R &k_, R &sf, R &ws, R &m) {
  R zact = g_acth2o(znw, zns);
  k_ = g_exp(4. * K_SURFW0 * K_MWA / (K_RG * T * K_RHOWA * dwet));
  sf = R(prs * rhoair / K_MWA);
  ws = zact * k_;
  R zknud = 2. * zmfph2o / dwet;
  R zbeta = (zknud + 1.) / (0.377 * zknud + 1. + 4. / (3. * 1.) * (zknud + zknud * zknud));
  R h1 = n * 2. * K_PI * dwet * zdfh2o * zbeta;
  R h2 = K_MWA * zdfh2o * K_ALV * ws * sf / (zthcond * T);
  R h3 = R(((K_ALV * K_MWA) / (K_RG * T)) - 1.);
  m = h1 / (h2 * h3 + 1.);
}

struct CondConst { double rhoair, zdfh2o, zmfph2o, zthcond; };
__device__ __forceinline__ CondConst cond_const(double T, double pres) {
  CondConst c;
  c.rhoair = K_MAIR * pres / (K_RG * T);
  double zdfh2o = (5. / (16. * K_AVOG * c.rhoair * 1.e-3 * sq(3.11e-8))) *
                  sqrt(K_RG * 1.e7 * T * K_MAIR * 1.e3 * (K_MWA + K_MAIR) * 1.e3 / (2. * K_PI * K_MWA * 1.e3));
  c.zdfh2o = zdfh2o * 1.e-4;
  c.zmfph2o = 3. * c.zdfh2o * sqrt(K_PI * K_MWA / (8. * K_RG * T));
  c.zthcond = 0.023807 + 7.1128e-5 * (T - 273.16);
  return c;
}

template <typename R>
__device__ __forceinline__ R chain_solute(const DevParams &P, const CW<R> &w, int b, R kappa) {
  R vs = R(0.);
  for (int nn = 0; nn < P.ndry; nn++)
    if (P.diss[nn] > 0.) vs += w.V(nn, b);
  return kappa * vs * K_RHOWA / K_MWA;
}

// gpparth2o for warm cells (level 4).  Returns the substep count.
template <typename R>
__device__ int chain_condensation(const DevParams &P, const CW<R> &w, const double *tb, const ChainCell<R> &c,
                                  double dt, double *tp, const TapeLayout &tl, int lane) {
  const int NL = w.NL, iwa = P.iwa;
  const double *dmid = tb + TAB_DMID * P.nb_pad;
  const double T = c.T, pres = c.pres, prs = c.prs;
  SUB_BEGIN();
  R prv = c.prv0;
  const R zrh = prv / prs;
  R l1 = R(0.);
  for (int b = lane; b <= P.fn2b; b += 32) l1 += w.V(iwa, b);
  const R zaelwc1 = g_wsum(l1) * K_RHOWA;
  chain_equil_1a(P, w, zrh, T, tp ? tp + tl.eq : nullptr, lane);
  if (tp) { state_to_tape(tp + tl.x_eq, (double *)w.n, (double *)w.v, NL, P.nwet, lane); }
  R l2 = R(0.);
  for (int b = lane; b <= P.fn2b; b += 32) l2 += w.V(iwa, b);
  const R zaelwc2 = g_wsum(l2) * K_RHOWA;
  prv = prv - (zaelwc2 - zaelwc1) / (pres * K_MAIR / (K_RG * T));

  bool anycl = false, anypr = false, anyae = false;
  for (int b = lane; b < NL; b += 32) {
    const int ph = phase_of(P, b);
    const double n = val(w.n[b]);
    if (ph == 1) anyae |= n > K_NLIM;
    else if (ph == 2) anycl |= n > K_NLIM;
    else anypr |= n > K_PRLIM;
  }
  anyae = warp_any(anyae); anycl = warp_any(anycl); anypr = warp_any(anypr);
  if (tp && lane == 0) tp[tl.nit] = -1.;
  if (!((anycl || (anypr && P.lscndh2ocl)) || (anyae && val(zrh) > 0.98 && P.lscndh2oae))) return 0;

  const CondConst cc = cond_const(T, pres);
  for (int b = lane; b < NL; b += 32) {
    const int ph = phase_of(P, b);
    const R dwet = liquid_dwet(P, w, dmid, b);
    const R n = w.n[b];
    R k_ = R(1.), sf = R(0.), m = R(0.), ws = R(0.);
    const R ns_ = chain_solute(P, w, b, c.kappa);
    bool act;
    if (ph == 1) act = val(n) > K_NLIM && val(zrh) > 0.98 && P.lscndh2oae;
    else if (ph == 2) act = val(n) > K_NLIM && P.lscndh2ocl;
    else act = val(n) > K_PRLIM && P.lscndh2ocl;
    if (act) {
      const R znw = w.V(iwa, b) * P.rholiq[iwa] / P.MM[iwa];
      cond_coeffs(n, dwet, znw, ns_, T, prs, cc.rhoair, cc.zdfh2o, cc.zmfph2o, cc.zthcond, k_, sf, ws, m);
    }
    w.kel[b] = k_; w.surf[b] = sf; w.mt[b] = m; w.wsat[b] = ws; w.zns[b] = ns_;
    w.cw[b] = w.V(iwa, b) * K_RHOWA / K_MWA;
  }
  __syncwarp();
  SUB_MARK(5);
  bool a = false, cl = false, pr = false;
  for (int b = lane; b < NL; b += 32) {
    const int ph = phase_of(P, b);
    const double n = val(w.n[b]);
    if (ph == 1) a |= n > K_NLIM; else if (ph == 2) cl |= n > K_NLIM; else pr |= n > K_PRLIM;
  }
  const bool upd_ae = warp_any(a) && val(zrh) > 0.98, upd_cl = warp_any(cl), upd_pr = warp_any(pr);
  R zcwc = prv * cc.rhoair / K_MWA;
  R tsum = R(0.), msum = R(0.);
  for (int b = lane; b < NL; b += 32) {
    tsum += w.cw[b];
    if (b >= P.in2a) msum += w.mt[b];
  }
  const R zcwtot = zcwc + g_wsum(tsum);
  const R mtot = g_wsum(msum);
  double ttot = 0.;
  R zcwint = R(0.);
  int counter = 0;
  // the step kernel's form of the substeps (gpparth2o): the sum of mt*wsat*surf that
  // opens a substep is formed at the end of the previous one, with the same lane
  // partial sums (lane l: bins l, l+32)
  const double adt = 2.e-2;
  R spsum;
  {
    R sp = R(0.);
    for (int b = lane; b < NL; b += 32)
      if (b >= P.in2a) sp += w.mt[b] * w.wsat[b] * w.surf[b];
    spsum = g_wsum(sp);
  }
  while (ttot < dt) {
    if (tp && counter < tl.maxit) {
      if (lane == 0) tp[tl.hist_zc + counter] = val(zcwc);
      for (int b = lane; b < NL; b += 32) {
        tp[tl.hist_c + counter * NL + b] = val(w.cw[b]);
        tp[tl.hist_w + counter * NL + b] = val(w.wsat[b]);
      }
    }
    const R zhlp1 = zcwc + adt * spsum;
    const R zhlp2 = 1. + adt * mtot;
    zcwint = fmin(zhlp1 / zhlp2, zcwtot);
    R cs = R(0.), sp = R(0.);
    for (int b = lane; b < NL; b += 32) {
      const int ph = phase_of(P, b);
      R cc_ = w.cw[b];
      const bool upd = (ph == 1) ? (upd_ae && b >= P.in2a) : (ph == 2 ? upd_cl : upd_pr);
      if (upd) {
        const R ci = cc_ + fmin(fmax(adt * w.mt[b] * (zcwint - w.wsat[b] * w.surf[b]), -1.e-1 * cc_), 1.e-1 * cc_);
        w.wsat[b] = g_acth2o(ci, w.zns[b]) * w.kel[b];
        cc_ = fmax(ci, R(0.));
      }
      w.cw[b] = cc_;
      cs += cc_;
      if (b >= P.in2a) sp += w.mt[b] * w.wsat[b] * w.surf[b];
    }
    zcwint = zcwtot - g_wsum(cs);
    spsum = g_wsum(sp);
    zcwc = zcwint;
    ttot = ttot + adt;
    counter++;
    if (counter >= 200000) break;
  }
  if (tp) {
    if (lane == 0) tp[tl.nit] = (double)counter;
    if (counter < tl.maxit)
      for (int b = lane; b < NL; b += 32) tp[tl.hist_c + counter * NL + b] = val(w.cw[b]);
  }
  __syncwarp();
  for (int b = lane; b < NL; b += 32) w.V(iwa, b) = fmax(R(0.), w.cw[b] * K_MWA / K_RHOWA);
  __syncwarp();
  SUB_MARK(6);
  return counter;
}

// Collision kernels of a taped step (FP64): the values as chain_kernels<double>, plus
// dK/dd_i and dK/dd_j of every pair from dual numbers.  drow (9 NL) receives the
// diameter derivatives of the per-bin properties; the kernels and their derivatives
// go to the tape (tri layout, zero for pairs that are not active).
__device__ void chain_kernels_taped(const DevParams &P, const CW<double> &w, const double *tb, double T, double pres,
                                    double *drow, double *Kt, double *dki, double *dkj, int lane) {
  const int NL = w.NL;
  const double *dmid = tb + TAB_DMID * P.nb_pad;
  const CoagCell<Dual<1>> c1 = chain_coagcell<Dual<1>>(T, pres, P);
  const CoagCell<Dual<2>> c2 = chain_coagcell<Dual<2>>(T, pres, P);
  for (int b = lane; b < NL; b += 32) w.dw[b] = liquid_dwet(P, w, dmid, b);
  for (int e = lane; e < chain_tri(NL); e += 32) { dki[e] = 0.; dkj[e] = 0.; }
  __syncwarp();
  double *keq = w.kel, *dkeq = w.surf;   // equal-size kernel per bin and its d-derivative
  const int nact = chain_active_bins(P, w, lane);
  for (int e = lane; e < nact; e += 32) {
    const int b = w.pbuf[e];
    Dual<1> d(w.dw[b]);
    d.d[0] = 1.;
    BinProps<Dual<1>> o;
    const Dual<1> k = chain_bin_props<Dual<1>>(P, c1, b, d, o);
    keq[b] = k.v;
    dkeq[b] = k.d[0];
    const Dual<1> *po = &o.diam;
    for (int k = 0; k < 9; k++) { w.S[k * NL + b] = po[k].v; drow[k * NL + b] = po[k].d[0]; }
  }
  __syncwarp();
  auto lift = [&](int b, int dir, BinProps<Dual<2>> &o) {
    Dual<2> *po = &o.diam;
    for (int k = 0; k < 9; k++) {
      Dual<2> x(w.S[k * NL + b]);
      x.d[dir] = drow[k * NL + b];
      po[k] = x;
    }
  };
  chain_pairs(
      P, w, lane,
      [&](int sec, int pk) {
        const int i = pk & 0xff, j = (pk >> 8) & 0xff;
        const int ti = tri(i, j, NL);
        if (sec == 1) {   // the equal-size kernel depends on bin j alone
          w.K[ti] = keq[j];
          dki[ti] = 0.;
          dkj[ti] = dkeq[j];
          return;
        }
        BinProps<Dual<2>> A_, B_;
        lift(i, 0, A_);
        lift(j, 1, B_);
        const Dual<2> k = coag_pair<Dual<2>>(c2, A_, B_);
        w.K[ti] = k.v;
        dki[ti] = k.d[0];
        dkj[ti] = k.d[1];
      },
      [&](int pk) { w.K[tri(pk & 0xff, (pk >> 8) & 0xff, NL)] = 0.; });
  __syncwarp();
  for (int e = lane; e < chain_tri(NL); e += 32) Kt[e] = w.K[e];
  __syncwarp();
}

// ---- one step of the chain ----
template <typename R>
__device__ int chain_step(const DevParams &P, const CW<R> &w, const double *tb, const ChainCell<R> &c, double dt,
                          double *tp, const TapeLayout &tl, int lane, double *drow = nullptr) {
  const int NL = w.NL, NW = P.nwet;
  if (tp) state_to_tape(tp + tl.x_in, (const double *)w.n, nullptr, NL * (1 + NW), 0, lane);
  // the chain's domain: empty precipitation bins, vapour at or above 98 % of saturation
  // (the non-initialising branch of the water uptake, mo_salsa_dynamics.f90:797-801)
  bool pr = false;
  for (int b = P.nbins + P.ncld + lane; b < NL; b += 32) pr |= val(w.n[b]) >= K_PRLIM;
  if (warp_any(pr) || !(val(c.prv0) / c.prs >= 0.98)) return 1;
#ifdef SALSA_STAGE_TIMERS
  long long t_stage = clock64();
#endif
  if constexpr (std::is_same<R, double>::value) {
    if (tp) chain_kernels_taped(P, w, tb, c.T, c.pres, drow, tp + tl.K, tp + tl.dki, tp + tl.dkj, lane);
    else chain_kernels<R>(P, w, tb, c.T, c.pres, lane);
  } else {
    chain_kernels<R>(P, w, tb, c.T, c.pres, lane);
  }
  STAGE_MARK(11);
  chain_coag_update<R>(P, w, tb, dt, lane, tp ? tp + tl.sums : nullptr);
  __syncwarp();
  if (tp) state_to_tape(tp + tl.x_pre, (const double *)w.n, nullptr, NL * (1 + NW), 0, lane);
  chain_coag_clamp<R>(P, w, lane);
  if (tp) state_to_tape(tp + tl.x_mid, (const double *)w.n, nullptr, NL * (1 + NW), 0, lane);
  __syncwarp();
  STAGE_MARK(12);
  chain_condensation<R>(P, w, tb, c, dt, tp, tl, lane);
  STAGE_MARK(13);
  return 0;
}

struct ChainArgs {
  int ncell, nsub, every, NL, NW, nstate, ws_doubles, n1a;
  double dt;
  const double *temp, *press, *rs, *dn, *kappa, *ssat;
  const double *x0;
  double *xN, *ckpt;
  const double *dx0, *dkappa, *dssat;
  double *dxN;
  const double *xbarN;
  double *xbar0, *kappabar, *ssatbar;
  double *seg, *tape;
  unsigned long long *err;
};

__device__ __forceinline__ void set_tangent(double &, double) {}
__device__ __forceinline__ void set_tangent(Dual<1> &x, double t) { x.d[0] = t; }
__device__ __forceinline__ double tangent(double) { return 0.; }
__device__ __forceinline__ double tangent(const Dual<1> &x) { return x.d[0]; }

// boundary units (#/kg, kg/kg) <-> SALSA units (#/m3, m3/m3), as the step kernel's unpack
template <typename R>
__device__ void chain_load(const DevParams &P, const CW<R> &w, const double *x, const double *dx, double dn, int lane) {
  const int NL = w.NL;
  for (int e = lane; e < NL * (1 + P.nwet); e += 32) {
    if (e < NL) {
      w.n[e] = R(x[e] * dn);
      if (dx) set_tangent(w.n[e], dx[e] * dn);
    } else {
      const int s = (e - NL) / NL, b = (e - NL) - s * NL;
      w.V(s, b) = R(x[e] * dn * P.irholiq[s]);   // as the step kernel's unpacking
      if (dx) set_tangent(w.V(s, b), dx[e] * dn * P.irholiq[s]);
    }
  }
  __syncwarp();
}
template <typename R>
__device__ void chain_store(const DevParams &P, const CW<R> &w, double *x, double *dx, double dn, int lane) {
  const int NL = w.NL;
  __syncwarp();
  for (int e = lane; e < NL * (1 + P.nwet); e += 32) {
    if (e < NL) {
      x[e] = val(w.n[e]) / dn;
      if (dx) dx[e] = tangent(w.n[e]) / dn;
    } else {
      const int s = (e - NL) / NL, b = (e - NL) - s * NL;
      x[e] = val(w.V(s, b)) * P.rholiq[s] / dn;
      if (dx) dx[e] = tangent(w.V(s, b)) * P.rholiq[s] / dn;
    }
  }
  __syncwarp();
}

template <typename R>
__device__ __forceinline__ ChainCell<R> chain_cell(const ChainArgs &A, long long q, bool tlm) {
  ChainCell<R> c;
  c.T = A.temp[q]; c.pres = A.press[q]; c.prs = A.rs[q]; c.dn = A.dn[q];
  c.rhoair = K_MAIR * c.pres / (K_RG * c.T);
  c.kappa = R(A.kappa[q]);
  c.prv0 = R(A.rs[q] * (1.0 + A.ssat[q]));
  if (tlm) {
    set_tangent(c.kappa, A.dkappa ? A.dkappa[q] : 0.);
    set_tangent(c.prv0, A.dssat ? A.rs[q] * A.dssat[q] : 0.);
  }
  return c;
}

__device__ __forceinline__ void chain_tables(const DevParams &P, double *tb) {
  for (int i = threadIdx.x; i < P.tab_doubles; i += blockDim.x) tb[i] = P.tables[i];
  __syncthreads();
}

// forward chain (R = double) and tangent-linear chain (R = Dual<1>); one warp per cell
template <typename R, bool TLM>
__global__ void __launch_bounds__(128, 2) chain_fwd_kernel(const DevParams P, const ChainArgs A) {
  extern __shared__ double smem[];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, wpb = blockDim.x >> 5;
  double *tb = smem;
  chain_tables(P, tb);
  CW<R> w = make_cw<R>(reinterpret_cast<R *>(smem + P.tab_doubles + (size_t)warp * A.ws_doubles), A.NL, A.NW);
  TapeLayout tl = tape_layout(A.NL, A.NW, A.n1a, tape_maxit(A.dt));
  unsigned long long nerr = 0;
  for (long long q = (long long)blockIdx.x * wpb + warp; q < A.ncell; q += (long long)gridDim.x * wpb) {
    const ChainCell<R> c = chain_cell<R>(A, q, TLM);
    chain_load<R>(P, w, A.x0 + q * A.nstate, TLM ? (A.dx0 ? A.dx0 + q * A.nstate : nullptr) : nullptr, c.dn, lane);
    int bad = 0;
    for (int k = 0; k < A.nsub && !bad; k++) {
      if (!TLM && A.ckpt && k % A.every == 0) {
        double *dst = A.ckpt + ((long long)(k / A.every) * A.ncell + q) * A.nstate;
        for (int e = lane; e < A.nstate; e += 32) dst[e] = val(w.n[e]);   // n then v: SALSA units
      }
      bad = chain_step<R>(P, w, tb, c, A.dt, nullptr, tl, lane);
    }
    nerr += bad;
    chain_store<R>(P, w, A.xN + q * A.nstate, TLM ? A.dxN + q * A.nstate : nullptr, c.dn, lane);
  }
  if (lane == 0 && nerr) atomicAdd(A.err, nerr);
}


// =======================================================================================
// Adjoint (R = double).  Shared-memory adjoint workspace per warp:
//   an[NL], av[NW][NL]   adjoint of the state (the "new" slot during the coagulation reverse)
//   on[NL], ov[NW][NL]   adjoint of the state entering the coagulation sweep ("old" slot)
//   Kb[tri]              adjoint of K; then K-bar * dK/dd_i per pair
//   cb, wb, mtb, kelb, znsb [NL]   adjoints of the condensation quantities
// =======================================================================================
struct AW {
  double *an, *av, *on, *ov, *Kb, *cb, *wb, *mtb, *kelb, *znsb;
  int NL;
  __device__ __forceinline__ double &AV(int s, int b) const { return av[s * NL + b]; }
  __device__ __forceinline__ double &OV(int s, int b) const { return ov[s * NL + b]; }
};
__host__ __device__ __forceinline__ int adj_ws_doubles(int NL, int NW) {
  return 2 * (NL + NW * NL) + chain_tri(NL) + 5 * NL;
}
__device__ __forceinline__ AW make_aw(double *p, int NL, int NW) {
  AW a;
  a.NL = NL;
  a.an = p; p += NL;
  a.av = p; p += NW * NL;
  a.on = p; p += NL;
  a.ov = p; p += NW * NL;
  a.Kb = p; p += chain_tri(NL);
  a.cb = p; p += NL;
  a.wb = p; p += NL;
  a.mtb = p; p += NL;
  a.kelb = p; p += NL;
  a.znsb = p; p += NL;
  return a;
}

__device__ __forceinline__ double wsum(double v) { return g_wsum(v); }

// ---- condensation reverse: adjoint of the state after condensation -> after the
// coagulation (x_mid); adds to kbar (kappa) and pbar (imposed vapour) ----
__device__ void cond_reverse(const DevParams &P, const CW<double> &w, const AW &a, const double *tb,
                             const ChainCell<double> &c, double dt, const double *tp, const TapeLayout &tl,
                             double &kbar, double &pbar, int lane) {
  const int NL = w.NL, NW = P.nwet, iwa = P.iwa;
  const double *dmid = tb + TAB_DMID * P.nb_pad;
  const double T = c.T, pres = c.pres, prs = c.prs;
  const double D = pres * K_MAIR / (K_RG * T);
  const int nit = (int)tp[tl.nit];
  SUB_BEGIN();
  // state after the water uptake (x_eq)
  tape_to_state(tp + tl.x_eq, w.n, w.v, NL, NW, lane);
  __syncwarp();
  const double zrh = c.prv0 / prs;
  double prv_adj_bar = 0.;
  const CondConst cc = cond_const(T, pres);
  if (nit >= 0) {
    // recompute the coefficients of the substep loop
    for (int b = lane; b < NL; b += 32) {
      const int ph = phase_of(P, b);
      const double dwet = liquid_dwet(P, w, dmid, b);
      const double n = w.n[b];
      double k_ = 1., sf = 0., m = 0., ws = 0.;
      const double ns_ = chain_solute(P, w, b, c.kappa);
      bool act;
      if (ph == 1) act = n > K_NLIM && zrh > 0.98 && P.lscndh2oae;
      else if (ph == 2) act = n > K_NLIM && P.lscndh2ocl;
      else act = n > K_PRLIM && P.lscndh2ocl;
      if (act) {
        const double znw = w.V(iwa, b) * P.rholiq[iwa] / P.MM[iwa];
        cond_coeffs(n, dwet, znw, ns_, T, prs, cc.rhoair, cc.zdfh2o, cc.zmfph2o, cc.zthcond, k_, sf, ws, m);
      }
      w.kel[b] = k_; w.surf[b] = sf; w.mt[b] = m; w.zns[b] = ns_;
      a.cb[b] = 0.; a.wb[b] = 0.; a.mtb[b] = 0.; a.kelb[b] = 0.; a.znsb[b] = 0.;
    }
    __syncwarp();
    bool ae = false, cl = false, pr = false;
    for (int b = lane; b < NL; b += 32) {
      const int ph = phase_of(P, b);
      const double n = w.n[b];
      if (ph == 1) ae |= n > K_NLIM; else if (ph == 2) cl |= n > K_NLIM; else pr |= n > K_PRLIM;
    }
    const bool upd_ae = warp_any(ae) && zrh > 0.98, upd_cl = warp_any(cl), upd_pr = warp_any(pr);
    double tsum = 0., msum = 0.;
    for (int b = lane; b < NL; b += 32) {
      tsum += w.V(iwa, b) * K_RHOWA / K_MWA;
      if (b >= P.in2a) msum += w.mt[b];
    }
    const double zcwtot = tp[tl.hist_zc] + wsum(tsum);
    const double mtot = wsum(msum);
    // write-back: V_w = max(0, c_final MWA / RHOWA)
    for (int b = lane; b < NL; b += 32) {
      const double cf = tp[tl.hist_c + nit * NL + b];
      const double y = cf * K_MWA / K_RHOWA;
      a.cb[b] = y > 0. ? a.AV(iwa, b) * K_MWA / K_RHOWA : 0.;
      a.AV(iwa, b) = 0.;
    }
    __syncwarp();
    double zcb = 0., zcwtotb = 0., mtotb = 0.;
    const double adt = 2.e-2;
    const double izh2 = 1. / (1. + adt * mtot);   // the substeps' constant denominator
    for (int it = nit - 1; it >= 0; it--) {
      const double zc_in = tp[tl.hist_zc + it];
      const double *cin = tp + tl.hist_c + it * NL, *win = tp + tl.hist_w + it * NL;
      double sp = 0.;
      for (int b = lane; b < NL; b += 32)
        if (b >= P.in2a) sp += w.mt[b] * win[b] * w.surf[b];
      const double zhlp1 = zc_in + adt * wsum(sp);
      const double zhlp2 = 1. + adt * mtot;
      const double q = zhlp1 / zhlp2;
      const double zcwint = fmin(q, zcwtot);
      // zcwc_out = zcwtot - sum c_out
      zcwtotb += zcb;
      double zib = 0.;   // adjoint of zcwint (this lane's share)
      for (int b = lane; b < NL; b += 32) {
        a.cb[b] -= zcb;
        const int ph = phase_of(P, b);
        const bool upd = (ph == 1) ? (upd_ae && b >= P.in2a) : (ph == 2 ? upd_cl : upd_pr);
        if (!upd) continue;
        const double c0 = cin[b], w0 = win[b], mt = w.mt[b], sf = w.surf[b], kel = w.kel[b], zns = w.zns[b];
        const double arg = adt * mt * (zcwint - w0 * sf);
        const double lo = -1.e-1 * c0, hi = 1.e-1 * c0;
        const double a1 = fmax(arg, lo);
        const double cl_ = fmin(a1, hi);
        const double ci = c0 + cl_;
        double cib = ci > 0. ? a.cb[b] : 0.;
        // wsat_out = acth2o(ci, zns) * kel
        const double gw = a.wb[b];
        const double den = fmax(K_EPS, ci + zns);
        const double r = ci / den;
        const double act = fmax(0.1, r);
        a.kelb[b] += gw * act;
        const double ab = gw * kel;
        if (r > 0.1) {
          if (ci + zns > K_EPS) {
            const double id = 1. / (ci + zns), q2 = ab * id * id;
            cib += q2 * zns;
            a.znsb[b] += -q2 * ci;
          } else {
            cib += ab / K_EPS;
          }
        }
        double c0b = cib, a1b = 0.;
        if (hi < a1) c0b += 1.e-1 * cib; else a1b = cib;
        double argb = 0.;
        if (lo > arg) c0b += -1.e-1 * a1b; else argb = a1b;
        a.mtb[b] += argb * adt * (zcwint - w0 * sf);
        zib += argb * adt * mt;
        a.cb[b] = c0b;
        a.wb[b] = -argb * adt * mt * sf;
      }
      const double zcwintb = wsum(zib);
      double qb = 0.;
      if (zcwtot < q) zcwtotb += zcwintb; else qb = zcwintb;
      const double zhlp1b = qb * izh2;
      const double zhlp2b = -qb * q * izh2;
      mtotb += zhlp2b * adt;
      zcb = zhlp1b;
      const double spb = zhlp1b * adt;
      for (int b = P.in2a + lane; b < NL; b += 32) {
        a.mtb[b] += spb * win[b] * w.surf[b];
        a.wb[b] += spb * w.mt[b] * w.surf[b];
      }
      __syncwarp();
    }
    // loop set-up: mtot, zcwtot = zcwc0 + sum cw0, zcwc0 = prv_adj rhoair / MWA
    for (int b = lane; b < NL; b += 32) {
      if (b >= P.in2a) a.mtb[b] += mtotb;
      a.cb[b] += zcwtotb;
    }
    zcb += zcwtotb;
    prv_adj_bar = zcb * cc.rhoair / K_MWA;
    __syncwarp();
    SUB_MARK(0);
    // coefficients (x_eq state): cw0, zns, and kel/ws/mt through dual numbers
    double kb_l = 0.;
    for (int b = lane; b < NL; b += 32) {
      const int ph = phase_of(P, b);
      a.AV(iwa, b) += a.cb[b] * K_RHOWA / K_MWA;
      const double n = w.n[b];
      bool act;
      if (ph == 1) act = n > K_NLIM && zrh > 0.98 && P.lscndh2oae;
      else if (ph == 2) act = n > K_NLIM && P.lscndh2ocl;
      else act = n > K_PRLIM && P.lscndh2ocl;
      double znsb = a.znsb[b];
      if (act) {
        // inputs: 0 n, 1 dwet, 2 znw, 3 zns
        Dual<4> dn_(n), dd(liquid_dwet(P, w, dmid, b)), dz(w.V(iwa, b) * P.rholiq[iwa] / P.MM[iwa]), ds(w.zns[b]);
        dn_.d[0] = 1.; dd.d[1] = 1.; dz.d[2] = 1.; ds.d[3] = 1.;
        Dual<4> k_, sf, ws, m;
        cond_coeffs(dn_, dd, dz, ds, T, prs, cc.rhoair, cc.zdfh2o, cc.zmfph2o, cc.zthcond, k_, sf, ws, m);
        double g[4];
        for (int i = 0; i < 4; i++) g[i] = a.kelb[b] * k_.d[i] + a.wb[b] * ws.d[i] + a.mtb[b] * m.d[i];
        a.an[b] += g[0];
        a.AV(iwa, b) += g[2] * P.rholiq[iwa] / P.MM[iwa];
        znsb += g[3];
        // wet diameter of x_eq
        if (n > nlim_of(ph)) {
          double vs = 0.;
          for (int s = 0; s < NW; s++) vs += w.V(s, b);
          const double dw = cbrt(vs / n / K_PI6);
          if (!(dlim_of(ph) < dw)) {
            for (int s = 0; s < NW; s++) a.AV(s, b) += g[1] * dw / (3. * vs);
            a.an[b] += -g[1] * dw / (3. * n);
          }
        }
      }
      // zns = kappa * V_soluble * RHOWA / MWA
      double vsol = 0.;
      for (int nn = 0; nn < P.ndry; nn++)
        if (P.diss[nn] > 0.) vsol += w.V(nn, b);
      kb_l += znsb * vsol * K_RHOWA / K_MWA;
      for (int nn = 0; nn < P.ndry; nn++)
        if (P.diss[nn] > 0.) a.AV(nn, b) += znsb * c.kappa * K_RHOWA / K_MWA;
    }
    kbar += wsum(kb_l);
    __syncwarp();
    SUB_MARK(1);
  }
  // prv_adj = prv0 - (zaelwc2 - zaelwc1) / D
  pbar += prv_adj_bar;
  const double zael2b = -prv_adj_bar / D, zael1b = prv_adj_bar / D;
  for (int b = lane; b <= P.fn2b; b += 32) a.AV(iwa, b) += zael2b * K_RHOWA;
  __syncwarp();
  // Regime-1a water uptake reverse.  The forward iterates zke_{i+1} = f(zke_i; bin) through
  // the 1a bins in order, carrying zke from bin to bin; the tape holds every iterate.  The
  // local partials of the iterations are independent of one another, so lanes evaluate
  // them in parallel (Dual<5>, 32 iterations at a time, in reverse order: bins fn1a ..
  // in1a, iterations cnt .. 1).  The adjoint of zke then runs through each chunk serially,
  // and the input adjoints of every bin are warp sums of its iterations' terms.
  {
    const int n1a = P.fn1a - P.in1a + 1;
    const double *xm = tp + tl.x_mid;
    const Dual<5> zrhd(fmin(fmax(zrh, 0.05), 0.98));
    auto eq_of = [&](int r) { return tp + tl.eq + (P.fn1a - r - P.in1a) * TP_MAXEQ; };
    int total = 0;
    for (int r = 0; r < n1a; r++) total += eq_of(r)[0] > 0. ? (int)eq_of(r)[0] : 0;
    double tot[4] = {0., 0., 0., 0.};   // lane r < n1a: sums for bin fn1a - r (zv0, zv1, numc, zcore)
    double zkeb = 0.;
    for (int base = 0; base < total; base += 32) {
      const int f = base + lane;
      int r = -1;
      double p[5] = {0., 0., 0., 0., 0.}, q[5] = {0., 0., 0., 0., 0.};
      if (f < total) {
        int rem = f, cnt = 0;
        for (r = 0; r < n1a; r++) {
          cnt = eq_of(r)[0] > 0. ? (int)eq_of(r)[0] : 0;
          if (rem < cnt) break;
          rem -= cnt;
        }
        const int i = cnt - rem, kk = P.fn1a - r;
        const double *te = eq_of(r);
        const double numc = xm[kk];
        const double zv0 = P.ix_so4 >= 0 ? xm[NL + P.ix_so4 * NL + kk] : 0.;
        const double zv1 = P.ix_oc >= 0 ? xm[NL + P.ix_oc * NL + kk] : 0.;
        const double zcore = zv0 / numc + zv1 / numc;
        Dual<5> izke(te[i]), d0(zv0), d1(zv1), dnm(numc), dco(zcore);
        izke.d[0] = 1.; d0.d[1] = 1.; d1.d[2] = 1.; dnm.d[3] = 1.; dco.d[4] = 1.;
        Dual<5> zlwc, zd;
        eq1a_iter(zrhd, izke, d0, d1, dnm, Dual<5>(0.), dco, T, zlwc, zd);   // izke is now 1/zke_i
        const double lb = (i == cnt) ? a.AV(iwa, kk) / K_RHOWA : 0.;
        for (int k = 0; k < 5; k++) { p[k] = izke.d[k]; q[k] = lb * zlwc.d[k]; }
      }
      // the zke adjoint entering each iteration, serially through the chunk
      const int n = min(32, total - base);
      double myz = 0.;
      for (int l = 0; l < n; l++) {
        const double q0 = shfl_idx(q[0], l), p0 = shfl_idx(p[0], l);
        if (lane == l) myz = zkeb;
        zkeb = q0 + zkeb * p0;
      }
      double g[4];
      for (int k = 0; k < 4; k++) g[k] = q[k + 1] + myz * p[k + 1];
      // per-bin sums, two bins per transposed butterfly
      for (int r0 = 0; r0 < n1a; r0 += 2) {
        double v[8];
        for (int k = 0; k < 4; k++) { v[k] = r == r0 ? g[k] : 0.; v[4 + k] = r == r0 + 1 ? g[k] : 0.; }
        warp_sum8(v, lane);
        for (int k = 0; k < 4; k++) {
          if (lane == r0) tot[k] += v[k];
          if (lane == r0 + 1) tot[k] += v[4 + k];
        }
      }
    }
    __syncwarp();
    if (lane < n1a) {
      const int kk = P.fn1a - lane;
      const double *te = eq_of(lane);
      if (te[0] >= 0.) {
        a.AV(iwa, kk) = 0.;
        if (te[0] > 0.) {
          const double numc = xm[kk];
          const double zv0 = P.ix_so4 >= 0 ? xm[NL + P.ix_so4 * NL + kk] : 0.;
          const double zv1 = P.ix_oc >= 0 ? xm[NL + P.ix_oc * NL + kk] : 0.;
          double zv0b = tot[0], zv1b = tot[1], numcb = tot[2];
          const double zcoreb = tot[3];
          zv0b += zcoreb / numc;
          zv1b += zcoreb / numc;
          numcb += -zcoreb * zv0 / (numc * numc) - zcoreb * zv1 / (numc * numc);
          if (P.ix_so4 >= 0) a.AV(P.ix_so4, kk) += zv0b;
          if (P.ix_oc >= 0) a.AV(P.ix_oc, kk) += zv1b;
          a.an[kk] += numcb;
        }
      }
    }
  }
  __syncwarp();
  for (int b = lane; b <= P.fn2b; b += 32) a.AV(iwa, b) += zael1b * K_RHOWA;
  __syncwarp();
  SUB_MARK(2);
}

// ---- coagulation reverse: adjoint of x_mid (after the clamp) -> adjoint of x_in ----
// Values a target saw: a partner updated earlier in the sweep (lower index, processed)
// shows its new value (x_pre), any other its old value (x_in).
// w.n / w.v hold x_in, xpre the state after the sweep and w.K the step's kernels (shared
// memory copies of the tape's rows).
__device__ void coag_reverse(const DevParams &P, const CW<double> &w, const AW &a, const double *tb, double dt,
                             const double *tp, const TapeLayout &tl, const double *xpre, int lane) {
  const int NL = w.NL, NW = P.nwet, C0 = P.nbins;
  const double *xin = w.n, *xmid = tp + tl.x_mid;
  const int16_t *L = partner_lists(P, tb);
  // clamp: pass where the clamped value is positive
  for (int e = lane; e < NL * (1 + NW); e += 32) {
    double *slot = e < NL ? a.an + e : a.av + (e - NL);
    if (!(xmid[e] > 0.)) *slot = 0.;
  }
  for (int e = lane; e < NL * (1 + NW); e += 32) (e < NL ? a.on[e] : a.ov[e - NL]) = 0.;
  for (int e = lane; e < chain_tri(NL); e += 32) a.Kb[e] = 0.;
  __syncwarp();
  auto processed = [&](int b) -> bool {
    return ((b >= P.in1a && b <= P.fn2b) || (b >= C0 && b < C0 + P.ncld)) && xin[b] >= K_NLIM;
  };
  // value of partner g and its adjoint slot as seen by target t
  auto nval = [&](int g, int t) -> double { return (processed(g) && g < t) ? xpre[g] : xin[g]; };
  auto vval = [&](int s, int g, int t) -> double {
    return (processed(g) && g < t) ? xpre[NL + s * NL + g] : xin[NL + s * NL + g];
  };
  auto nslot = [&](int g, int t) -> double & { return (processed(g) && g < t) ? a.an[g] : a.on[g]; };
  auto vslot = [&](int s, int g, int t) -> double & { return (processed(g) && g < t) ? a.AV(s, g) : a.OV(s, g); };
  // K at the step's start state lives in w.K (recomputed by the caller)
  for (int t = C0 + P.ncld - 1; t >= P.in1a; t--) {
    if (!processed(t)) continue;
    const bool isc = t >= C0;
    int kk = 0, kfirst = 0, o_first = 0;
    if (isc) {
      kk = t - C0;
      const bool ra = kk <= P.fca_cur;
      kfirst = ra ? P.ica_cur : P.icb_cur;
      o_first = ra ? P.icb_cur : P.ica_cur;
    }
    // the target's sums, taped by the forward sweep
    const double *tsum = tp + tl.sums + t * (2 + SALSA_NSV);
    double src[SALSA_NSV];
    const double sink = tsum[0], self = tsum[1];
    for (int s = 0; s < SALSA_NSV; s++) src[s] = tsum[2 + s];
    const int soff = L[4 * t], sn = L[4 * t + 1];
    const bool has_self = isc ? P.lscgcc : P.lscgaa;
    const double nt = xin[t];
    // the two denominators of the update, as reciprocals (the partials divide by them)
    const double r1 = 1. / (1. + dt * sink), r2 = 1. / (1. + dt * (sink + self));
    // adjoints of the outputs (new slot of t)
    double vbar[SALSA_NSV];
    for (int s = 0; s < SALSA_NSV; s++) vbar[s] = s < NW ? a.AV(s, t) : 0.;
    const double nbar = a.an[t];
    const double nnew = xpre[t];
    double srcb[SALSA_NSV], ntb = nbar * r2, sinkb = -nbar * nnew * dt * r2;
    const double selfb = sinkb;
    for (int s = 0; s < SALSA_NSV; s++) {
      srcb[s] = 0.;
      if (s < NW) {
        const double vn = xpre[NL + s * NL + t], vr = vbar[s] * dt * r1;
        srcb[s] = vr * nt;
        ntb += vr * src[s];
        sinkb += -vr * vn;
      }
    }
    __syncwarp();
    if (lane == 0) {
      for (int s = 0; s < NW; s++) { a.OV(s, t) += vbar[s] * r1; a.AV(s, t) = 0.; }
      if (has_self) {
        a.Kb[tri(t, t, NL)] += selfb * 0.5 * nt;
        ntb += selfb * 0.5 * w.Kij(t, t);
      }
      a.on[t] += ntb;
      a.an[t] = 0.;
    }
    __syncwarp();
    // partners (distinct bins per lane)
    for (int e = lane; e < sn; e += 32) {
      const int g = L[soff + e];
      a.Kb[g < t ? tri(g, t, NL) : tri(t, g, NL)] += sinkb * nval(g, t);
      nslot(g, t) += sinkb * w.Kij(t, g);
    }
    __syncwarp();
    auto src_rev = [&](int g) {
      const double k = w.Kij(g, t);
      double kb = 0.;
      for (int s = 0; s < NW; s++) {
        kb += srcb[s] * vval(s, g, t);
        vslot(s, g, t) += srcb[s] * k;
      }
      a.Kb[g < t ? tri(g, t, NL) : tri(t, g, NL)] += kb;
    };
    if (isc) {
      cloud_sources(P, kk, kfirst, o_first, lane, src_rev);
    } else {
      const int roff = L[4 * t + 2], rn = L[4 * t + 3];
      for (int e = lane; e < rn; e += 32) src_rev(L[roff + e]);
    }
    __syncwarp();
  }
  // adjoint of x_in: old slot, plus the new slot of the bins the sweep did not update
  for (int e = lane; e < NL * (1 + NW); e += 32) {
    const int b = e < NL ? e : (e - NL) % NL;
    double &nw_ = e < NL ? a.an[e] : a.av[e - NL];
    const double o = e < NL ? a.on[e] : a.ov[e - NL];
    nw_ = (processed(b) ? 0. : nw_) + o;
  }
  __syncwarp();
}

// ---- collision-kernel reverse: K-bar and the taped dK/dd -> x_in adjoint ----
__device__ void kernel_reverse(const DevParams &P, const AW &a, const double *xin, const double *dki,
                               const double *dkj, double *Pj, int NL, int NW, int lane) {
  for (int e = lane; e < chain_tri(NL); e += 32) {
    const double kb = a.Kb[e];
    a.Kb[e] = kb * dki[e];
    Pj[e] = kb * dkj[e];
  }
  __syncwarp();
  // gather per bin in a fixed order, then through the wet diameter of x_in
  for (int b = lane; b < NL; b += 32) {
    double g = 0.;
    for (int j = b; j < NL; j++) g += a.Kb[tri(b, j, NL)];
    for (int i = 0; i <= b; i++) g += Pj[tri(i, b, NL)];
    const int ph = phase_of(P, b);
    const double n = xin[b];
    if (n > nlim_of(ph) && g != 0.) {
      double vs = 0.;
      for (int s = 0; s < NW; s++) vs += xin[NL + s * NL + b];
      const double dw = cbrt(vs / n / K_PI6);
      if (!(dlim_of(ph) < dw)) {
        for (int s = 0; s < NW; s++) a.AV(s, b) += g * dw / (3. * vs);
        a.an[b] += -g * dw / (3. * n);
      }
    }
  }
  __syncwarp();
}

// ---- adjoint kernels; the host runs them step by step, last step first ----
// Cells are handed to warps one at a time from a counter of the launch (zero before it),
// so that warps drawing cheap cells take more of them and the launch ends evenly.
__device__ __forceinline__ long long next_cell(unsigned *ctr, int lane) {
  unsigned q = 0;
  if (lane == 0) q = atomicAdd(ctr, 1u);
  return (long long)__shfl_sync(0xffffffffu, q, 0);
}

// Segment recompute: the states entering steps k0+1 .. k1-1 of a checkpoint segment.
__global__ void __launch_bounds__(128, 2) chain_seg_kernel(const DevParams P, const ChainArgs A, int sg,
                                                           unsigned *ctr) {
  extern __shared__ double smem[];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, wpb = blockDim.x >> 5;
  double *tb = smem;
  chain_tables(P, tb);
  const int NL = A.NL, NW = A.NW, ns = A.nstate;
  CW<double> w = make_cw<double>(smem + P.tab_doubles + (size_t)warp * A.ws_doubles, NL, NW);
  const TapeLayout tl = tape_layout(NL, NW, A.n1a, tape_maxit(A.dt));
  const int k0 = sg * A.every, k1 = min(A.nsub, k0 + A.every);
  unsigned long long nerr = 0;
  for (long long q = next_cell(ctr, lane); q < A.ncell; q = next_cell(ctr, lane)) {
    const ChainCell<double> c = chain_cell<double>(A, q, false);
    tape_to_state(A.ckpt + ((long long)sg * A.ncell + q) * ns, w.n, w.v, NL, NW, lane);
    __syncwarp();
    int bad = 0;
    for (int k = k0; k < k1 - 1 && !bad; k++) {
      bad = chain_step<double>(P, w, tb, c, A.dt, nullptr, tl, lane);
      __syncwarp();
      double *dst = A.seg + ((long long)(k + 1 - k0) * A.ncell + q) * ns;
      for (int e = lane; e < ns; e += 32) dst[e] = w.n[e];
      __syncwarp();
    }
    nerr += bad;
  }
  if (lane == 0 && nerr) atomicAdd(A.err, nerr);
}

// Taped step: recompute step k of every cell from the state entering it, taping.
__global__ void __launch_bounds__(128, 2) chain_taped_kernel(const DevParams P, const ChainArgs A, const double *src,
                                                             unsigned *ctr) {
  extern __shared__ double smem[];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, wpb = blockDim.x >> 5;
  double *tb = smem;
  chain_tables(P, tb);
  const int NL = A.NL, NW = A.NW, ns = A.nstate;
  double *base = smem + P.tab_doubles + (size_t)warp * A.ws_doubles;
  CW<double> w = make_cw<double>(base, NL, NW);
  double *drow = base + chain_ws_entries(NL, NW) + 32;
  const TapeLayout tl = tape_layout(NL, NW, A.n1a, tape_maxit(A.dt));
  unsigned long long nerr = 0;
  for (long long q = next_cell(ctr, lane); q < A.ncell; q = next_cell(ctr, lane)) {
    const ChainCell<double> c = chain_cell<double>(A, q, false);
    tape_to_state(src + q * ns, w.n, w.v, NL, NW, lane);
    __syncwarp();
    double *tp = A.tape + q * (long long)tl.total;
    const int bad = chain_step<double>(P, w, tb, c, A.dt, tp, tl, lane, drow);
    nerr += bad;
    if (lane == 0) tp[tl.nit + 1] = bad ? 1. : 0.;   // 1: the cell's adjoint is void
    __syncwarp();
  }
  if (lane == 0 && nerr) atomicAdd(A.err, nerr);
}

// Reverse of step k of every cell; the running adjoint of the state (SALSA units) is
// kept in xbar0, the kappa and supersaturation adjoints accumulate in place.
__global__ void __launch_bounds__(128, 2) chain_rev_kernel(const DevParams P, const ChainArgs A, unsigned *ctr) {
  extern __shared__ double smem[];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, wpb = blockDim.x >> 5;
  double *tb = smem;
  chain_tables(P, tb);
  const int NL = A.NL, NW = A.NW, ns = A.nstate;
  double *base = smem + P.tab_doubles + (size_t)warp * A.ws_doubles;
  // condensation-reverse workspace: state and six per-bin rows; then the adjoint
  // workspace, and copies of the tape's x_pre and K for the coagulation reverse (K's
  // rows take K-bar * dK/dd_j in the kernel reverse)
  CW<double> w;
  w.NL = NL;
  w.n = base; w.v = base + NL;
  w.kel = base + ns; w.surf = w.kel + NL; w.mt = w.surf + NL; w.wsat = w.mt + NL; w.cw = w.wsat + NL;
  w.zns = w.cw + NL;
  w.dw = nullptr; w.S = nullptr; w.pbuf = nullptr; w.K = nullptr;
  AW a = make_aw(base + ns + 6 * NL, NL, NW);
  double *xpre_s = base + ns + 6 * NL + adj_ws_doubles(NL, NW), *K_s = xpre_s + ns;
  const TapeLayout tl = tape_layout(NL, NW, A.n1a, tape_maxit(A.dt));
  for (long long q = next_cell(ctr, lane); q < A.ncell; q = next_cell(ctr, lane)) {
    double *tp = A.tape + q * (long long)tl.total;
    if (tp[tl.nit + 1] != 0.) continue;
    const ChainCell<double> c = chain_cell<double>(A, q, false);
    double *xb = A.xbar0 + q * ns;
    for (int e = lane; e < ns; e += 32) { if (e < NL) a.an[e] = xb[e]; else a.av[e - NL] = xb[e]; }
    __syncwarp();
    double kbar = 0., pbar = 0.;
#ifdef SALSA_STAGE_TIMERS
    long long t_stage = clock64();
#endif
    cond_reverse(P, w, a, tb, c, A.dt, tp, tl, kbar, pbar, lane);
    STAGE_MARK(14);
    tape_to_state(tp + tl.x_in, w.n, w.v, NL, NW, lane);
    for (int e = lane; e < ns; e += 32) xpre_s[e] = tp[tl.x_pre + e];
    for (int e = lane; e < chain_tri(NL); e += 32) K_s[e] = tp[tl.K + e];
    w.K = K_s;
    __syncwarp();
    coag_reverse(P, w, a, tb, A.dt, tp, tl, xpre_s, lane);
    STAGE_MARK(15);
    kernel_reverse(P, a, w.n, tp + tl.dki, tp + tl.dkj, K_s, NL, NW, lane);
    STAGE_MARK(3);
    for (int e = lane; e < ns; e += 32) xb[e] = e < NL ? a.an[e] : a.av[e - NL];
    if (lane == 0) {
      A.kappabar[q] += kbar;
      A.ssatbar[q] += pbar * c.prs;
    }
    __syncwarp();
  }
}

// Unit conversions of the adjoint between the boundary (#/kg, kg/kg) and SALSA units.
__global__ void chain_adj_units(const DevParams P, const ChainArgs A, int to_salsa) {
  const long long n = (long long)A.ncell * A.nstate;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const long long q = i / A.nstate;
    const int e = (int)(i - q * A.nstate);
    const double dn = A.dn[q];
    const double rho = e < A.NL ? 1. : P.rholiq[(e - A.NL) / A.NL];
    if (to_salsa) {
      A.xbar0[i] = A.xbarN[i] * rho / dn;
      if (e == 0) { A.kappabar[q] = 0.; A.ssatbar[q] = 0.; }
    } else {
      A.xbar0[i] = A.xbar0[i] * dn / rho;
    }
  }
}

}  // namespace
}  // namespace salsa

// =======================================================================================
// C-ABI entry points of the chain
// =======================================================================================
namespace {
using salsa::DevParams;
using salsa::ChainArgs;

int chain_params(salsa_handle_t *h, const salsa_chain_t *c, DevParams *P, ChainArgs *A, cudaStream_t *st, void *stream,
                 int *nsm) {
  int dev = 0;
  cudaStream_t hs;
  if (!h || !c || !salsa::handle_params(h, P, &hs, &dev, nsm)) return SALSA_E_ARG;
  const salsa_config_t *g = salsa::handle_config(h);
  if (g->level != 4) return SALSA_E_UNSUPPORTED;
  if (c->ncell <= 0 || c->nsub <= 0 || !(c->dt > 0.) || c->dt > 1.2) return SALSA_E_ARG;
  if (!c->temp || !c->press || !c->rs || !c->dn || !c->kappa || !c->ssat) return SALSA_E_ARG;
  if (cudaSetDevice(dev) != cudaSuccess) return SALSA_E_NODEV;
  *st = stream ? (cudaStream_t)stream : hs;
  P->level = 4; P->lcharge = 0; P->initialize = 0; P->dt = c->dt; P->has_kappa = 1;
  P->lscgaa = g->lscgaa; P->lscgcc = g->lscgcc; P->lscgca = g->lscgca; P->lscgpc = g->lscgpc; P->lscgpa = g->lscgpa;
  P->lscgpp = g->lscgpp; P->lscgia = P->lscgic = P->lscgii = P->lscgip = 0;
  P->lscndh2oae = g->lscndh2oae; P->lscndh2ocl = g->lscndh2ocl; P->lscndh2oic = 0;
  memset(A, 0, sizeof *A);
  A->ncell = c->ncell; A->nsub = c->nsub; A->dt = c->dt;
  A->NL = P->nliquid; A->NW = P->nwet; A->nstate = A->NL * (1 + A->NW); A->n1a = P->fn1a - P->in1a + 1;
  A->temp = c->temp; A->press = c->press; A->rs = c->rs; A->dn = c->dn; A->kappa = c->kappa; A->ssat = c->ssat;
  A->every = 1;
  unsigned long long *err = (unsigned long long *)salsa::handle_scratch(h, 3, 64);
  if (!err) return SALSA_E_CUDA;
  A->err = err;
  if (cudaMemsetAsync(err, 0, sizeof(unsigned long long), *st) != cudaSuccess) return SALSA_E_CUDA;
  return SALSA_OK;
}

template <typename R>
int ws_doubles(int NL, int NW) {
  return (int)(((size_t)salsa::chain_ws_entries(NL, NW) * sizeof(R) + 7) / 8) + 32;
}

template <typename K>
int launch_chain(K kernel, const DevParams &P, const ChainArgs &A, cudaStream_t st, int nsm, int wpb) {
  size_t smem = sizeof(double) * ((size_t)P.tab_doubles + (size_t)wpb * A.ws_doubles);
  if (cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess)
    return SALSA_E_CUDA;
  int bps = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, kernel, 32 * wpb, smem) != cudaSuccess || bps <= 0)
    return SALSA_E_CUDA;
  long long grid = (long long)bps * nsm * 4;
  long long need = (A.ncell + wpb - 1) / wpb;
  if (grid > need) grid = need;
  kernel<<<(int)grid, 32 * wpb, smem, st>>>(P, A);
  return cudaGetLastError() == cudaSuccess ? SALSA_OK : SALSA_E_CUDA;
}

int chain_finish(const ChainArgs &A, cudaStream_t st) {
  unsigned long long nerr = 0;
  if (cudaMemcpyAsync(&nerr, A.err, sizeof nerr, cudaMemcpyDeviceToHost, st) != cudaSuccess) return SALSA_E_CUDA;
  if (cudaStreamSynchronize(st) != cudaSuccess) return SALSA_E_CUDA;
  return nerr ? SALSA_E_NUMERIC : SALSA_OK;
}
}  // namespace

extern "C" {

int salsa_gb300_chain_state_size(const salsa_handle_t *h) {
  DevParams P;
  cudaStream_t s;
  int dev, nsm;
  if (!salsa::handle_params(h, &P, &s, &dev, &nsm)) return 0;
  return salsa::handle_config(h)->level == 4 ? P.nliquid * (1 + P.nwet) : 0;
}

long long salsa_gb300_chain_adjoint_bytes(const salsa_handle_t *h, int ncell, int nsub, double dt,
                                          int ckpt_every) {
  DevParams P;
  cudaStream_t s;
  int dev, nsm;
  if (!salsa::handle_params(h, &P, &s, &dev, &nsm) || salsa::handle_config(h)->level != 4) return -1;
  if (ncell <= 0 || nsub <= 0 || ckpt_every <= 0 || !(dt > 0.)) return -1;
  const long long ns = (long long)P.nliquid * (1 + P.nwet);
  const salsa::TapeLayout tl = salsa::tape_layout(P.nliquid, P.nwet, P.fn1a - P.in1a + 1, salsa::tape_maxit(dt));
  const long long nseg = (nsub + ckpt_every - 1) / ckpt_every;
  long long d = nseg * ncell * ns + (long long)ncell * tl.total;   // checkpoints, tape
  if (ckpt_every > 1) d += (long long)ckpt_every * ncell * ns;      // states of one segment
  return d * (long long)sizeof(double) + (nseg + 2LL * nsub) * (long long)sizeof(unsigned) + 64;
}

int salsa_gb300_chain_forward(salsa_handle_t *h, const salsa_chain_t *c, const double *x0, double *xN, double *ckpt,
                              int ckpt_every, void *stream) {
  DevParams P;
  ChainArgs A;
  cudaStream_t st;
  int nsm = 0;
  int rc = chain_params(h, c, &P, &A, &st, stream, &nsm);
  if (rc) return rc;
  if (!x0 || !xN || (ckpt && ckpt_every <= 0)) return SALSA_E_ARG;
  A.x0 = x0; A.xN = xN; A.ckpt = ckpt; A.every = ckpt ? ckpt_every : 1;
  A.ws_doubles = ws_doubles<double>(A.NL, A.NW);
  rc = launch_chain(salsa::chain_fwd_kernel<double, false>, P, A, st, nsm, 4);
  if (rc) return rc;
  return chain_finish(A, st);
}

int salsa_gb300_chain_tlm(salsa_handle_t *h, const salsa_chain_t *c, const double *x0, const double *dx0,
                          const double *dkappa, const double *dssat, double *xN, double *dxN, void *stream) {
  DevParams P;
  ChainArgs A;
  cudaStream_t st;
  int nsm = 0;
  int rc = chain_params(h, c, &P, &A, &st, stream, &nsm);
  if (rc) return rc;
  if (!x0 || !xN || !dxN) return SALSA_E_ARG;
  A.x0 = x0; A.xN = xN; A.dx0 = dx0; A.dkappa = dkappa; A.dssat = dssat; A.dxN = dxN;
  A.ws_doubles = ws_doubles<salsa::Dual<1>>(A.NL, A.NW);
  rc = launch_chain(salsa::chain_fwd_kernel<salsa::Dual<1>, true>, P, A, st, nsm, 4);
  if (rc) return rc;
  return chain_finish(A, st);
}

int salsa_gb300_chain_adjoint(salsa_handle_t *h, const salsa_chain_t *c, const double *ckpt, int ckpt_every,
                              const double *xbarN, double *xbar0, double *kappabar, double *ssatbar, void *stream) {
  DevParams P;
  ChainArgs A;
  cudaStream_t st;
  int nsm = 0;
  int rc = chain_params(h, c, &P, &A, &st, stream, &nsm);
  if (rc) return rc;
  if (!ckpt || ckpt_every <= 0 || !xbarN || !xbar0 || !kappabar || !ssatbar) return SALSA_E_ARG;
  A.ckpt = const_cast<double *>(ckpt); A.every = ckpt_every;
  A.xbarN = xbarN; A.xbar0 = xbar0; A.kappabar = kappabar; A.ssatbar = ssatbar;
  const int NL = A.NL, NW = A.NW, ns = A.nstate, wpb = 4;
  const salsa::TapeLayout tl = salsa::tape_layout(NL, NW, A.n1a, salsa::tape_maxit(A.dt));
  A.tape = (double *)salsa::handle_scratch(h, 0, (size_t)A.ncell * tl.total * sizeof(double));
  A.seg = ckpt_every > 1
              ? (double *)salsa::handle_scratch(h, 1, (size_t)ckpt_every * A.ncell * ns * sizeof(double))
              : nullptr;
  if (!A.tape || (ckpt_every > 1 && !A.seg)) return SALSA_E_CUDA;
  // one work counter per launch: segment recomputes, then a taped and a reverse step each
  const int nseg = (A.nsub + A.every - 1) / A.every;
  const size_t nctr = (size_t)nseg + 2 * (size_t)A.nsub;
  unsigned *ctr = (unsigned *)salsa::handle_scratch(h, 2, nctr * sizeof(unsigned));
  if (!ctr || cudaMemsetAsync(ctr, 0, nctr * sizeof(unsigned), st) != cudaSuccess) return SALSA_E_CUDA;
  // per-kernel shared memory (doubles per warp) and grids
  const int ws_fwd = salsa::chain_ws_entries(NL, NW) + 32;
  const int ws_tap = ws_fwd + 9 * NL;
  const int ws_rev = ns + 6 * NL + salsa::adj_ws_doubles(NL, NW) + ns + salsa::chain_tri(NL);
  auto config = [&](auto kernel, int wsd, int *grid, size_t *smem) -> bool {
    *smem = sizeof(double) * ((size_t)P.tab_doubles + (size_t)wpb * wsd);
    if (cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)*smem) != cudaSuccess)
      return false;
    int bps = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, kernel, 32 * wpb, *smem) != cudaSuccess || bps <= 0)
      return false;
    long long g = (long long)bps * nsm, need = (A.ncell + wpb - 1) / wpb;
    *grid = (int)(g < need ? g : need);
    return true;
  };
  int g_seg = 0, g_tap = 0, g_rev = 0;
  size_t s_seg = 0, s_tap = 0, s_rev = 0;
  if (!config(salsa::chain_seg_kernel, ws_fwd, &g_seg, &s_seg) ||
      !config(salsa::chain_taped_kernel, ws_tap, &g_tap, &s_tap) ||
      !config(salsa::chain_rev_kernel, ws_rev, &g_rev, &s_rev))
    return SALSA_E_CUDA;
  salsa::chain_adj_units<<<4 * nsm, 256, 0, st>>>(P, A, 1);
  for (int sg = nseg - 1; sg >= 0; sg--) {
    const int k0 = sg * A.every, k1 = A.nsub < k0 + A.every ? A.nsub : k0 + A.every;
    if (k1 - k0 > 1) {
      A.ws_doubles = ws_fwd;
      salsa::chain_seg_kernel<<<g_seg, 32 * wpb, s_seg, st>>>(P, A, sg, ctr + sg);
    }
    for (int k = k1 - 1; k >= k0; k--) {
      const double *src = k == k0 ? A.ckpt + (size_t)sg * A.ncell * ns : A.seg + (size_t)(k - k0) * A.ncell * ns;
      A.ws_doubles = ws_tap;
      unsigned *c_k = ctr + nseg + 2 * k;
      salsa::chain_taped_kernel<<<g_tap, 32 * wpb, s_tap, st>>>(P, A, src, c_k);
      A.ws_doubles = ws_rev;
      salsa::chain_rev_kernel<<<g_rev, 32 * wpb, s_rev, st>>>(P, A, c_k + 1);
    }
  }
  salsa::chain_adj_units<<<4 * nsm, 256, 0, st>>>(P, A, 0);
  if (cudaGetLastError() != cudaSuccess) return SALSA_E_CUDA;
  return chain_finish(A, st);
}

}  // extern "C"
