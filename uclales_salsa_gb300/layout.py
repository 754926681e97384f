"""Bin layout of the SALSA size distribution (host side).

Restates src/src_salsa/mo_salsa_init.f90:148-450 (set_aerobins, set_cloudbins,
set_icebins, buildBinLimits) and the index bookkeeping of salsa_initialize
(:806-814) with 0-based indices.  Used by the synthetic-input generator and by
the tests that compare the device tables with the oracle's.
"""
from dataclasses import dataclass, field
import math

PI6 = 0.5235988          # mo_submctl.f90:266 (truncated as written)
ALLNAMES = ["SO4", "OC", "BC", "DU", "SS", "NO", "NH"]
ALLMM = {"SO4": 98.08e-3, "OC": 150.e-3, "BC": 12.e-3, "DU": 100.e-3, "SS": 58.44e-3,
         "NO": 62.01e-3, "NH": 18.04e-3, "H2O": 18.016e-3, "rime": 18.016e-3}
ALLRHO = {"SO4": 1830., "OC": 1400., "BC": 2000., "DU": 2650., "SS": 2165.,
          "NO": 1479., "NH": 1530., "H2O": 1000., "rime": 400.}
ALLDISS = {"SO4": 3., "OC": 1., "BC": 0., "DU": 0., "SS": 2., "NO": 1., "NH": 1., "H2O": 1., "rime": 1.}
RHO_ICE = 917.
RHO_RIME = 400.


@dataclass
class Layout:
    nbins: int
    ncld: int
    nprc: int
    nice: int
    in1a: int
    fn1a: int
    in2a: int
    fn2a: int
    in2b: int
    fn2b: int
    species: list
    vlolim: list = field(default_factory=list)
    vhilim: list = field(default_factory=list)
    dmid: list = field(default_factory=list)
    phase: list = field(default_factory=list)

    @property
    def ntotal(self):
        return self.nbins + self.ncld + self.nprc + self.nice

    @property
    def nliquid(self):
        return self.nbins + self.ncld + self.nprc

    @property
    def ndry(self):
        return len(self.species)

    @property
    def nwet(self):
        return len(self.species) + 1

    def cloud_parallel(self, cb):
        """Aerosol bin parallel to cloud bin cb (mo_salsa_init.f90:279-282)."""
        return self.in2a + cb

    def rholiq(self):
        return [ALLRHO[s] for s in self.species] + [ALLRHO["H2O"]]

    def rhoice(self):
        return [ALLRHO[s] for s in self.species] + [RHO_ICE, RHO_RIME]


def _set_bin(vlo, vhi):
    dmid = ((vhi + vlo) / (2. * PI6)) ** (1. / 3.)
    return vlo, vhi, dmid


def build_layout(cfg):
    n1, n2 = cfg.nbin[0], cfg.nbin[1]
    rl = list(cfg.reglim)
    in1a = 0
    in2a = in1a + n1
    in2b = in2a + n2
    fn1a = in2a - 1
    fn2a = fn1a + n2
    fn2b = fn2a + n2
    nbins = fn2b + 1
    ncld = 2 * n2
    lay = Layout(nbins=nbins, ncld=ncld, nprc=cfg.prc_nbins, nice=cfg.ice_nbins, in1a=in1a, fn1a=fn1a,
                 in2a=in2a, fn2a=fn2a, in2b=in2b, fn2b=fn2b, species=cfg.species())
    aero = [None] * nbins
    ratio = rl[1] / rl[0]
    for cc in range(in1a, fn1a + 1):
        aero[cc] = _set_bin(PI6 * (rl[0] * ratio ** (cc / n1)) ** 3, PI6 * (rl[0] * ratio ** ((cc + 1) / n1)) ** 3)
    nbin2, nbin3 = 4, n2 - 4
    ratio = rl[2] / rl[1]
    for dd in range(in2a, in2a + nbin2):
        cc = dd - in2a
        aero[dd] = _set_bin(PI6 * (rl[1] * ratio ** (cc / nbin2)) ** 3, PI6 * (rl[1] * ratio ** ((cc + 1) / nbin2)) ** 3)
    ratio = rl[3] / rl[2]
    for dd in range(in2a + nbin2, fn2a + 1):
        cc = dd - (fn2a - (nbin3 - 1))
        aero[dd] = _set_bin(PI6 * (rl[2] * ratio ** (cc / nbin3)) ** 3, PI6 * (rl[2] * ratio ** ((cc + 1) / nbin3)) ** 3)
    for i in range(n2):
        aero[in2b + i] = aero[in2a + i]
    cloud = [aero[in2a + i] for i in range(n2)] + [aero[in2b + i] for i in range(n2)]

    def blo(n, dlo, vr):
        r = vr ** (1. / 3.)
        out = []
        lo = dlo
        hi = dlo * r
        for i in range(n):
            if i > 0:
                lo = lo * r
                hi = lo * r
            out.append(_set_bin(PI6 * lo ** 3, PI6 * hi ** 3))
        return out

    prc = blo(cfg.prc_nbins, cfg.prc_dlo, cfg.prc_vol_ratio)
    ice = blo(cfg.ice_nbins, cfg.ice_dlo, cfg.ice_vol_ratio)
    for ph, group in ((1, aero), (2, cloud), (3, prc), (4, ice)):
        for vlo, vhi, dmid in group:
            lay.vlolim.append(vlo)
            lay.vhilim.append(vhi)
            lay.dmid.append(dmid)
            lay.phase.append(ph)
    return lay


def lolim_diameters(lay):
    return [(v / PI6) ** (1. / 3.) for v in lay.vlolim]


def rslf(p, t):
    """Liquid saturation mixing ratio, src/src_LES/thrm.f90:345-364."""
    c = (0.6105851e+03, 0.4440316e+02, 0.1430341e+01, 0.2641412e-01, 0.2995057e-03,
         0.2031998e-05, 0.6936113e-08, 0.2564861e-11, -.3704404e-13)
    x = (t - 273.16).clamp(-80., 50.) if hasattr(t, "clamp") else min(max(-80., t - 273.16), 50.)
    esl = c[0] + x * (c[1] + x * (c[2] + x * (c[3] + x * (c[4] + x * (c[5] + x * (c[6] + x * (c[7] + x * c[8])))))))
    return .622 * esl / (p - esl)


def rsif(p, t):
    """Ice saturation mixing ratio, src/src_LES/thrm.f90:370-386."""
    c = (0.6114327e+03, 0.5027041e+02, 0.1875982e+01, 0.4158303e-01, 0.5992408e-03,
         0.5743775e-05, 0.3566847e-07, 0.1306802e-09, 0.2152144e-12)
    x = (t - 273.16).clamp(-80., 0.) if hasattr(t, "clamp") else min(max(-80., t - 273.16), 0.)
    esi = c[0] + x * (c[1] + x * (c[2] + x * (c[3] + x * (c[4] + x * (c[5] + x * (c[6] + x * (c[7] + x * c[8])))))))
    return .622 * esi / (p - esi)


def lognormal_bin_fractions(lay, dg, sigmag, nstr, nend):
    """Fraction of a lognormal number mode in each aerosol bin, with the
    10-sub-interval quadrature of src/src_salsa/mo_salsa_sizedist.f90:6-75."""
    out = [0.0] * lay.nbins
    for kk in range(nstr, nend + 1):
        d1b = (lay.vlolim[kk] / PI6) ** (1. / 3.)
        d2b = (lay.vhilim[kk] / PI6) ** (1. / 3.)
        dd = (d2b - d1b) / 10
        acc = 0.0
        for ib in range(1, 11):
            d1 = d1b + (ib - 1.) * dd
            d2 = d1 + dd
            dm = (d1 + d2) / 2
            dlnd = math.log(d2 / d1)
            acc += dlnd / (math.sqrt(2. * math.pi) * math.log(sigmag)) * \
                math.exp(-math.log(dm / dg) ** 2 / (2. * math.log(sigmag) ** 2))
        out[kk] = acc
    return out
