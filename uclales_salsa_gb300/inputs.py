"""Seeded synthetic inputs in run_SALSA's array layout.

No public dataset is involved: the reference's own case inputs (aerosol_in.nc,
soundings) are replaced by seeded synthetic fields with the shapes, sizes and
value ranges of the measured workloads.  Arrays are halo-padded exactly as
run_SALSA sees them (mo_salsa_driver.f90:180-182): for an interior X x Y x Z
block, nxp = X+4, nyp = Y+4, nzp = Z+2; halo cells are zero and never read.

A field of the reference, Fortran shape (nzp, nxp, nyp, nb), is held as a
contiguous torch tensor of shape (nb, nyp, nxp, nzp): the same bytes.

Construction of the fields:
  * aerosol number per bin from lognormal modes with the 10-sub-interval
    quadrature of mo_salsa_sizedist.f90:6-75, a per-cell random fraction moved
    to the parallel 2b regime;
  * dry masses N * pi6 * dmid^3 * rho_s * f_s as in aerosol_init/setAeroMass
    (src/src_LES/init.f90:940-1048) with seeded random volume fractions;
  * aerosol water from a kappa-Koehler estimate at min(RH, 0.95);
  * rs, rsi from rslf/rsif (src/src_LES/thrm.f90:345-386), rv = RH * rs,
    air density p / (Rd T).
"""
import math
from dataclasses import dataclass, field

import torch

from .config import workload_config
from .layout import build_layout, lognormal_bin_fractions, rslf, rsif, PI6, ALLRHO, RHO_ICE, RHO_RIME

RD = 287.04

WORKLOADS = {
    # 16x16x40, dt = 1 s, level 4: coagulation, condensation, activation
    "grid16x16x40": dict(X=16, Y=16, Z=40, level=4, T=(280., 295.), p=(90.e3, 101.e3),
                         rh_clear=(0.90, 1.01), cloudy=0.0, pattern="none", ice=False, seed=0, dt=1.0),
    # 256x256x128, level 5, 30 % cloudy cells
    "grid256x256x128": dict(X=256, Y=256, Z=128, level=5, T=(240., 275.), p=(90.e3, 101.e3),
                            rh_clear=(0.90, 1.01), rh_cloud=(1.0, 1.01), cloudy=0.30, pattern="random",
                            ice=False, seed=1, dt=1.0),
    # 65,536 independent cells as a 1-D batch (nxp = nyp = 5), kappa and supersaturation per cell
    "batch65536": dict(X=1, Y=1, Z=65536, level=4, T=(280., 295.), p=(90.e3, 101.e3),
                       rh_clear=(1.0, 1.01), cloudy=0.0, pattern="none", ice=False, seed=3, dt=0.5,
                       kappa=(0.1, 1.2), supersat=(0.0, 0.01)),
    # gradient workload: 65,536 independent warm cells, every cell holding the cloud
    # droplet distribution (and no precipitation), kappa and an imposed supersaturation
    "chain65536": dict(X=1, Y=1, Z=65536, level=4, T=(280., 295.), p=(90.e3, 101.e3),
                       rh_clear=(1.0, 1.01), rh_cloud=(1.0, 1.01), cloudy=1.0, pattern="random", ice=False,
                       precip=False, seed=5, dt=0.5, kappa=(0.1, 1.2), supersat=(0.0, 0.01)),
    # 384x384x160, level 5, 10 % cloudy as convective columns with ice, 90 % clear at RH 40-85 %
    "grid384x384x160": dict(X=384, Y=384, Z=160, level=5, T=(235., 270.), p=(90.e3, 101.e3),
                            rh_clear=(0.40, 0.85), rh_cloud=(1.0, 1.01), cloudy=0.10, pattern="columns",
                            ice=True, seed=4, dt=1.0),
}

SOLUBLE_KAPPA = {"SO4": 1.0, "OC": 0.17, "BC": 0.0, "DU": 0.0, "SS": 1.3, "NO": 1.0, "NH": 1.0}
# composition weights (volume) of the 1a, 2a and 2b regimes
W_1A = {"SO4": 1.0, "OC": 0.5}
W_2A = {"SO4": 1.0, "OC": 0.6, "BC": 0.1, "DU": 0.15, "SS": 0.3}
W_2B = {"SO4": 0.3, "OC": 0.3, "BC": 0.3, "DU": 1.0, "SS": 0.3}


@dataclass
class SalsaInputs:
    name: str
    cfg: object
    layout: object
    nzp: int
    nxp: int
    nyp: int
    ns: int
    dt: float
    level: int
    fields: dict = field(default_factory=dict)

    @property
    def ncells(self):
        return (self.nzp - 2) * (self.nxp - 4) * (self.nyp - 4)

    def plane(self):
        return self.nzp * self.nxp * self.nyp


def _u(gen, n, lo, hi, device):
    return lo + (hi - lo) * torch.rand(n, generator=gen, device=device, dtype=torch.float64)


def _comp(gen, n, species, weights, device):
    """Random volume fractions (weighted unit exponentials, normalised) per cell."""
    cols = []
    for s in species:
        w = weights.get(s, 0.0)
        e = -torch.log(torch.rand(n, generator=gen, device=device, dtype=torch.float64).clamp_min(1e-12))
        cols.append(w * e)
    f = torch.stack(cols, 0)
    return f / f.sum(0, keepdim=True).clamp_min(1e-300)


def _cloud_mask(spec, gen, X, Y, Z, device):
    n = X * Y * Z
    if spec["cloudy"] <= 0.0:
        return torch.zeros(n, dtype=torch.bool, device=device)
    if spec["pattern"] == "random":
        return torch.rand(n, generator=gen, device=device, dtype=torch.float64) < spec["cloudy"]
    # vertical convective columns of radius 4-12 cells around seeded centres, spanning
    # the lower 70 % of the domain; columns are added until the cloudy fraction is reached
    zc = torch.arange(Z, device=device)
    zmask = zc < int(0.7 * Z)
    yy, xx = torch.meshgrid(torch.arange(Y, device=device), torch.arange(X, device=device), indexing="ij")
    col = torch.zeros((Y, X), dtype=torch.bool, device=device)
    target = spec["cloudy"] / 0.7
    cg = torch.Generator(device="cpu")
    cg.manual_seed(spec["seed"] * 7919 + 11)
    while col.double().mean().item() < target:
        cy = int(torch.randint(0, Y, (1,), generator=cg))
        cx = int(torch.randint(0, X, (1,), generator=cg))
        r = float(torch.randint(4, 13, (1,), generator=cg))
        dy = torch.minimum((yy - cy).abs(), Y - (yy - cy).abs())
        dx = torch.minimum((xx - cx).abs(), X - (xx - cx).abs())
        col |= (dy * dy + dx * dx).double() <= r * r
    # cell order inside the interior block: (y, x, z) with z fastest
    m = col[:, :, None] & zmask[None, None, :]
    return m.reshape(-1)


def make_inputs(name, device="cpu", X=None, Y=None, Z=None, precision=0, diagnostics=1, seed=None, gases=False,
                overrides=None):
    """Build the fields of workload `name` (optionally with a smaller interior).

    overrides: entries of the workload's description to replace (e.g. cloudy=0.0 for
    clear cells only, or cloudy=1.0 with pattern="random" for cloudy cells only).

    gases: seeded condensing-vapour concentrations in gaero (H2SO4 and non-volatile
    organics 1e5-1e7 /cm3, semi-volatile organics 1e6-1e8 /cm3, HNO3 and NH3 1e8-1e9
    /cm3, log-uniform) and gas condensation switched on; otherwise gaero is zero."""
    spec = dict(WORKLOADS[name])
    if X is not None:
        spec["X"], spec["Y"], spec["Z"] = X, Y, Z
    if seed is not None:
        spec["seed"] = seed
    if overrides:
        spec.update(overrides)
    X, Y, Z = spec["X"], spec["Y"], spec["Z"]
    level = spec["level"]
    cfg = workload_config(level, precision=precision, diagnostics=diagnostics)
    lay = build_layout(cfg)
    if spec.get("pattern") == "none" and X == 1 and Y == 1:
        nxp = nyp = 5
    else:
        nxp, nyp = X + 4, Y + 4
    nzp = Z + 2
    ncell = X * Y * Z
    dev = torch.device(device)
    gen = torch.Generator(device=dev)
    gen.manual_seed(1000003 * spec["seed"] + 17)
    species = lay.species
    ndry, nwet = lay.ndry, lay.nwet
    rhol = lay.rholiq()
    f64 = dict(dtype=torch.float64, device=dev)

    T = _u(gen, ncell, *spec["T"], dev)
    P = _u(gen, ncell, *spec["p"], dev)
    cloudy = _cloud_mask(spec, gen, X, Y, Z, dev)
    RH = _u(gen, ncell, *spec["rh_clear"], dev)
    if spec["cloudy"] > 0:
        RH = torch.where(cloudy, _u(gen, ncell, *spec["rh_cloud"], dev), RH)
    dn = P / (RD * T)
    rs = rslf(P, T)
    rsi = rsif(P, T)
    if "supersat" in spec:
        s = _u(gen, ncell, *spec["supersat"], dev)
        rv = rs * (1.0 + s)
    else:
        rv = RH * rs
    wvel = _u(gen, ncell, -1.0, 1.0, dev)

    # aerosol number [#/m3] per bin
    nb = lay.nbins
    f_ait = lognormal_bin_fractions(lay, 40.e-9, 1.6, lay.in1a, lay.fn2a)
    f_acc = lognormal_bin_fractions(lay, 150.e-9, 1.5, lay.in1a, lay.fn2a)
    s_ait = _u(gen, ncell, 0.8, 1.2, dev) * 300.e6
    s_acc = _u(gen, ncell, 0.8, 1.2, dev) * 150.e6
    fb = _u(gen, ncell, 0.1, 0.3, dev)
    naer = torch.zeros((nb, ncell), **f64)
    for b in range(lay.in1a, lay.fn2a + 1):
        naer[b] = s_ait * f_ait[b] + s_acc * f_acc[b]
    for i in range(lay.fn2a - lay.in2a + 1):
        naer[lay.in2b + i] = fb * naer[lay.in2a + i]
        naer[lay.in2a + i] = (1.0 - fb) * naer[lay.in2a + i]
    c1a = _comp(gen, ncell, species, W_1A, dev)
    c2a = _comp(gen, ncell, species, W_2A, dev)
    c2b = _comp(gen, ncell, species, W_2B, dev)
    kap = {k: torch.zeros(ncell, **f64) for k in ("1a", "2a", "2b")}
    for i, s in enumerate(species):
        kap["1a"] += c1a[i] * SOLUBLE_KAPPA[s]
        kap["2a"] += c2a[i] * SOLUBLE_KAPPA[s]
        kap["2b"] += c2b[i] * SOLUBLE_KAPPA[s]
    aw = RH.clamp(0.3, 0.95)
    vaer = torch.zeros((nwet, nb, ncell), **f64)     # volume concentration [m3/m3]
    for b in range(nb):
        reg = "1a" if b <= lay.fn1a else ("2a" if b <= lay.fn2a else "2b")
        comp = {"1a": c1a, "2a": c2a, "2b": c2b}[reg]
        vdry = naer[b] * PI6 * lay.dmid[b] ** 3
        for i in range(ndry):
            vaer[i, b] = vdry * comp[i]
        vaer[ndry, b] = vdry * kap[reg] * aw / (1.0 - aw)

    ncl, npr, nic = lay.ncld, lay.nprc, lay.nice
    ncld_ = torch.zeros((ncl, ncell), **f64)
    vcld = torch.zeros((nwet, ncl, ncell), **f64)
    nprc_ = torch.zeros((npr, ncell), **f64)
    vprc = torch.zeros((nwet, npr, ncell), **f64)
    nice_ = torch.zeros((nic, ncell), **f64)
    vice = torch.zeros((nwet + 1, nic, ncell), **f64)
    if spec["cloudy"] > 0:
        cm = cloudy.double()
        na = ncl // 2
        w = torch.tensor([f_acc[lay.in2a + i] for i in range(na)], **f64)
        w = w / w.sum()
        cum = torch.cumsum(w, 0) - 0.5 * w
        z = math.sqrt(2.0) * torch.erfinv(2.0 * cum - 1.0)
        dwet = 15.e-6 * (1.3 ** z)
        ntot = 100.e6 * cm
        for i in range(na):
            for reg, frac, comp, cb in (("a", 1.0 - fb, c2a, i), ("b", fb, c2b, na + i)):
                ncld_[cb] = ntot * frac * w[i]
                dm = lay.dmid[lay.nbins + cb]
                vd = PI6 * dm ** 3
                vw = PI6 * float(dwet[i]) ** 3 - vd
                for k in range(ndry):
                    vcld[k, cb] = ncld_[cb] * vd * comp[k]
                vcld[ndry, cb] = ncld_[cb] * vw
        for j in range(npr if spec.get("precip", True) else 0):
            nprc_[j] = 1000.0 / npr * cm
            dm = lay.dmid[lay.nbins + ncl + j]
            v = PI6 * dm ** 3
            for k in range(ndry):
                vprc[k, j] = nprc_[j] * 1.e-3 * v * c2a[k]
            vprc[ndry, j] = nprc_[j] * (1.0 - 1.e-3) * v
        if spec["ice"] and level == 5:
            for j in range(nic):
                nice_[j] = 5000.0 / nic * cm
                dm = lay.dmid[lay.nbins + ncl + npr + j]
                v = PI6 * dm ** 3
                for k in range(ndry):
                    vice[k, j] = nice_[j] * 1.e-3 * v * c2b[k]
                vice[ndry, j] = nice_[j] * 0.8 * v
                vice[ndry + 1, j] = nice_[j] * 0.2 * v

    def pad(vals, nbv):
        out = torch.zeros((nbv, nyp, nxp, nzp), **f64)
        out[:, 2:2 + Y, 2:2 + X, 1:1 + Z] = vals.reshape(nbv, Y, X, Z)
        return out

    fields = {}
    fields["press"] = pad(P[None], 1)[0]
    fields["temp"] = pad(T[None], 1)[0]
    fields["rsl"] = pad(rs[None], 1)[0]
    fields["dn"] = pad(dn[None], 1)[0]
    fields["rp"] = pad(rv[None], 1)[0]
    fields["wp"] = pad(wvel[None], 1)[0]
    fields["naero"] = pad(naer / dn, nb)
    fields["ncloud"] = pad(ncld_ / dn, ncl)
    fields["nprecp"] = pad(nprc_ / dn, npr)
    fields["maero"] = pad(torch.stack([vaer[k] * rhol[k] / dn for k in range(nwet)]).reshape(nwet * nb, ncell), nwet * nb)
    fields["mcloud"] = pad(torch.stack([vcld[k] * rhol[k] / dn for k in range(nwet)]).reshape(nwet * ncl, ncell), nwet * ncl)
    fields["mprecp"] = pad(torch.stack([vprc[k] * rhol[k] / dn for k in range(nwet)]).reshape(nwet * npr, ncell), nwet * npr)
    fields["gaero"] = torch.zeros((5, nyp, nxp, nzp), **f64)
    if level == 5:
        rhoi = lay.rhoice()
        fields["rsi"] = pad(rsi[None], 1)[0]
        fields["nice"] = pad(nice_ / dn, nic)
        fields["mice"] = pad(torch.stack([vice[k] * rhoi[k] / dn for k in range(nwet + 1)]).reshape((nwet + 1) * nic, ncell),
                             (nwet + 1) * nic)
        fields["indef"] = pad(_u(gen, lay.nliquid * ncell, 0.0, 0.05, dev).reshape(lay.nliquid, ncell), lay.nliquid)
    if "kappa" in spec:
        fields["kappa"] = pad(_u(gen, ncell, *spec["kappa"], dev)[None], 1)[0]
    if gases:
        lo = torch.tensor([1.e5, 1.e8, 1.e8, 1.e5, 1.e6], **f64).log()
        hi = torch.tensor([1.e7, 1.e9, 1.e9, 1.e7, 1.e8], **f64).log()
        u = torch.rand((5, ncell), generator=gen, **f64)
        conc = torch.exp(lo[:, None] + (hi - lo)[:, None] * u) * 1.e6     # #/m3
        fields["gaero"] = pad(conc / dn, 5)
        cfg.lscndgas = 1
    return SalsaInputs(name=name, cfg=cfg, layout=lay, nzp=nzp, nxp=nxp, nyp=nyp, ns=nwet, dt=spec["dt"],
                       level=level, fields=fields)


def make_outputs(inp, device=None, with_diag=True):
    """Zeroed tendency and output arrays for one call."""
    lay = inp.layout
    dev = device or inp.fields["press"].device
    shp = (inp.nyp, inp.nxp, inp.nzp)
    z = lambda n: torch.zeros((n,) + shp, dtype=torch.float64, device=dev)
    out = {
        "rpt": torch.zeros(shp, dtype=torch.float64, device=dev),
        "naerot": z(lay.nbins), "ncloudt": z(lay.ncld), "nprecpt": z(lay.nprc),
        "maerot": z(lay.nwet * lay.nbins), "mcloudt": z(lay.nwet * lay.ncld), "mprecpt": z(lay.nwet * lay.nprc),
        "pa_nactd": z(lay.ncld), "pa_vactd": z(inp.ns * lay.ncld),
    }
    if inp.level == 5:
        out["nicet"] = z(lay.nice)
        out["micet"] = z((lay.nwet + 1) * lay.nice)
    if with_diag:
        nd = (20 if inp.cfg.lssecice.sw else 17) if inp.level == 5 else 12
        out["diag"] = z(nd)
    if inp.cfg.lscndgas:
        out["gaerot"] = z(5)
    return out
