"""States for the sedim_SALSA tests (src/src_LES/mcrp.f90:745-1275).

The bins come from a workload's initial state (aerosol everywhere, cloud droplets,
drops and at level 5 ice in the cloudy cells).  The LES fields around them are
seeded: temperature, pressure (giving the air density and the potential
temperature) at every point including the halo, the friction velocity per column,
and level thicknesses that vary from level to level (or one thickness for the
conservation checks).  The tendencies and tlt start from seeded values, so the
test sees that they are added to; the rates and fall speeds start from a fill
value, so it sees that they are overwritten.
"""
import torch

from uclales_salsa_gb300.inputs import make_inputs, RD, PI6

BINS = ("aero", "cloud", "precp", "ice")
VALUE = {"aero": ("naero", "maero"), "cloud": ("ncloud", "mcloud"), "precp": ("nprecp", "mprecp"),
         "ice": ("nice", "mice")}
TEND = {"aero": ("naerot", "maerot"), "cloud": ("ncloudt", "mcloudt"), "precp": ("nprecpt", "mprecpt"),
        "ice": ("nicet", "micet")}
FILL = 123.0


def sedim_state(workload, seed=5, dz=(3.0, 40.0), **kw):
    """(inputs, arrays): arrays maps SedimFields names to CPU tensors.

    dz: (lo, hi) for seeded level thicknesses, or one thickness for all levels."""
    inp = make_inputs(workload, "cpu", **kw)
    f = inp.fields
    g = torch.Generator().manual_seed(seed)
    f64 = dict(dtype=torch.float64)
    shp = f["press"].shape
    nyp, nxp, nzp = shp
    u = lambda size, lo, hi: lo + (hi - lo) * torch.rand(size, generator=g, **f64)
    lay = inp.layout
    if inp.level == 5 and float(f["nice"].abs().sum()) == 0:
        _seed_ice(inp, g)
    a = {}
    for part in BINS:
        v, t = VALUE[part], TEND[part]
        if v[0] not in f:
            continue
        a[v[0]] = f[v[0]].clone()
        a[v[1]] = f[v[1]].clone()
        a[t[0]] = torch.randn(a[v[0]].shape, generator=g, **f64) * 1e-3 * a[v[0]].abs().mean()
        a[t[1]] = torch.randn(a[v[1]].shape, generator=g, **f64) * 1e-3 * a[v[1]].abs().mean()
    T = u(shp, 240.0, 295.0)
    p = u(shp, 7.0e4, 1.01e5)
    a["tk"] = T
    a["adn"] = p / (RD * T)
    a["th"] = T * (1.0e5 / p) ** (RD / 1005.0)
    a["ustar"] = u((nyp, nxp), 0.05, 0.8)
    if isinstance(dz, tuple):
        a["dzt"] = 1.0 / u((nzp,), *dz)
    else:
        a["dzt"] = torch.full((nzp,), 1.0 / dz, **f64)
    a["tlt"] = torch.randn(shp, generator=g, **f64) * 1e-4
    for k in ("rrate", "irate"):
        a[k] = torch.full(shp, FILL, **f64)
    for k in ("sfcrrate", "sfcirate"):
        a[k] = torch.full((nyp, nxp), FILL, **f64)
    a["VtPrc"] = torch.full((lay.nprc,) + tuple(shp), FILL, **f64)
    if inp.level == 5:
        a["VtIce"] = torch.full((lay.nice,) + tuple(shp), FILL, **f64)
    return inp, a


def _seed_ice(inp, g):
    """Ice in the cloudy cells of a workload that starts without it: 5000 /m3 over the
    ice bins at their mid diameters, 80 % pristine ice, 20 % rime, a little dry matter."""
    f, lay = inp.fields, inp.layout
    nw, nic, nd = lay.nwet, lay.nice, lay.ndry
    dn = torch.where(f["dn"] > 0, f["dn"], torch.ones_like(f["dn"]))
    cm = (f["ncloud"].sum(0) > 0).double()
    rhoi = lay.rhoice()
    mi = f["mice"].view(nw + 1, nic, *dn.shape)
    for j in range(nic):
        n = 5000.0 / nic * cm * (0.5 + torch.rand(dn.shape, generator=g, dtype=torch.float64))
        v = PI6 * lay.dmid[lay.nbins + lay.ncld + lay.nprc + j] ** 3
        f["nice"][j] = n / dn
        for k in range(nd):
            mi[k, j] = n * 1.e-3 * v / nd * rhoi[k] / dn
        mi[nd, j] = n * 0.8 * v * rhoi[nd] / dn
        mi[nd + 1, j] = n * 0.2 * v * rhoi[nd + 1] / dn
