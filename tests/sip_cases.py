"""States for the secondary-ice (rime splintering, drop fracturing) oracle tests.

A block of the 256x256x128 workload (cloud droplets and drops in 30 % of the cells,
T 240-275 K) with ice seeded in the cloudy cells.  The ice bins take the reference's
layout style, diameters from 20 um doubling per bin, so that crystals large enough to
rime drops above 24 um exist; the splinters (10 um) then go to the first ice bin.
"""
import torch

from uclales_salsa_gb300.inputs import make_inputs, PI6
from uclales_salsa_gb300.layout import build_layout


def sip_state(mode, splinter=True, coag_only=True, seed=7, X=6, Y=6, Z=8, scheme="lssiprimespln"):
    inp = make_inputs("grid256x256x128", "cpu", X=X, Y=Y, Z=Z)
    cfg = inp.cfg
    cfg.ice_nbins, cfg.ice_dlo, cfg.ice_vol_ratio = 7, 20e-6, 8.0
    lay = build_layout(cfg)
    inp.layout = lay
    f = inp.fields
    g = torch.Generator().manual_seed(seed)
    dn = torch.where(f["dn"] > 0, f["dn"], torch.ones_like(f["dn"]))
    cm = (f["ncloud"].sum(0) > 0).double()
    nw, nic, nd = lay.nwet, lay.nice, lay.ndry
    rhoi = lay.rhoice()
    f["nice"] = torch.zeros((nic,) + tuple(dn.shape), dtype=torch.float64)
    f["mice"] = torch.zeros(((nw + 1) * nic,) + tuple(dn.shape), dtype=torch.float64)
    mi = f["mice"].view(nw + 1, nic, *dn.shape)
    for j in range(nic):
        n = 2000.0 / nic * cm * (0.5 + torch.rand(dn.shape, generator=g, dtype=torch.float64))
        v = PI6 * lay.dmid[lay.nbins + lay.ncld + lay.nprc + j] ** 3
        f["nice"][j] = n / dn
        for k in range(nd):
            mi[k, j] = n * 1.e-3 * v / nd * rhoi[k] / dn
        mi[nd, j] = n * 0.5 * v * rhoi[nd] / dn           # pristine ice
        mi[nd + 1, j] = n * 0.5 * v * rhoi[nd + 1] / dn   # rime
    # the secondary-ice tracers (#/kg per ice bin), seeded so that their passage through
    # the step (x dn on the way in, / dn on the way out, melting) shows
    for name in ("sipdrfr", "siprmspl", "sipiibr"):
        f[name] = f["nice"] * 0.1 * torch.rand(f["nice"].shape, generator=g, dtype=torch.float64)
    if coag_only:
        for sw in (cfg.lscnd, cfg.lsauto, cfg.lsactiv, cfg.lsicenucl, cfg.lsicemelt):
            sw.sw = 0
    cfg.lssecice.sw = int(splinter)
    sw = getattr(cfg, scheme)
    sw.sw = int(splinter)
    sw.mode = mode
    return inp
