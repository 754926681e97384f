"""Post-step states for the tend_constrain2 / SALSA_diagnostics tests.

A block of a workload takes one oracle step; its tendencies and the updated values
are then perturbed so that every branch of constrain_SALSA.f90 is taken somewhere:
tendencies that would empty a bin, negative values, cloud droplets and drops that have
lost their water, ice without mass, and aerosol bins below 0.1 nm dry diameter.
"""
import torch

from uclales_salsa_gb300.inputs import make_inputs, make_outputs
from oracle_ref import Oracle

VALUES = ["naero", "ncloud", "nprecp", "nice", "maero", "mcloud", "mprecp", "mice", "gaero", "indef"]
TENDS = {"naero": "naerot", "ncloud": "ncloudt", "nprecp": "nprecpt", "nice": "nicet", "maero": "maerot",
         "mcloud": "mcloudt", "mprecp": "mprecpt", "mice": "micet", "gaero": "gaerot"}


def post_state(workload, seed=3, **kw):
    """(inputs, arrays): arrays maps PostFields names to CPU tensors."""
    inp = make_inputs(workload, "cpu", gases=True, **kw)
    f = {k: v.clone() for k, v in inp.fields.items()}
    out = make_outputs(inp)
    rc, _ = Oracle(inp.cfg).run(inp, f, out, time=1.0)
    assert rc == 0
    g = torch.Generator().manual_seed(seed)
    lay = inp.layout
    a = {}
    for v, t in TENDS.items():
        if v in f and t in out:
            a[v] = f[v].clone()
            a[t] = out[t].clone()
    if "indef" in f:
        a["indef"] = f["indef"].clone() * 40 - 0.5          # values outside [0, 1] too
    dt = inp.dt

    def pick(shape, frac):
        return torch.rand(shape, generator=g, dtype=torch.float64) < frac

    # tendencies that would take a value below zero in one step
    for v, t in TENDS.items():
        if t in a:
            m = pick(a[t].shape, 0.05)
            a[t] = torch.where(m, -3.0 * a[v].abs() / dt - 1.0, a[t])
    # updated values, then the states that SALSA_diagnostics repairs
    for v, t in TENDS.items():
        if t in a:
            a[v] = a[v] + a[t] * dt * 0.5
    nw = lay.nwet
    iw = nw - 1
    for name, nb in (("mcloud", lay.ncld), ("mprecp", lay.nprc)):
        m = a[name].view(nw, nb, *a[name].shape[1:])
        sel = pick((nb,) + tuple(m.shape[2:]), 0.3)
        m[iw] = torch.where(sel, m[iw] * 1e-7, m[iw])
    ma = a["maero"].view(nw, lay.nbins, *a["maero"].shape[1:])
    sel = pick((lay.nbins,) + tuple(ma.shape[2:]), 0.02)
    for s in range(nw):
        ma[s] = torch.where(sel, ma[s] * 1e-20, ma[s])
    if "mice" in a:
        mi = a["mice"].view(nw + 1, lay.nice, *a["mice"].shape[1:])
        sel = pick((lay.nice,) + tuple(mi.shape[2:]), 0.3)
        mi[iw] = torch.where(sel, mi[iw] * 1e-12, mi[iw])
        mi[iw + 1] = torch.where(sel, mi[iw + 1] * 1e-12, mi[iw + 1])
    for name in ("naero", "maero", "ncloud", "mcloud"):
        a[name] = torch.where(pick(a[name].shape, 0.01), -a[name] * 1e-3, a[name])
    rs = f["rsl"].clamp(min=1e-12)
    a["rh"] = f["rp"] / rs * torch.where(pick(rs.shape, 0.5), 0.97, 1.0)
    if "rsi" in f:
        a["rhi"] = f["rp"] / f["rsi"].clamp(min=1e-12) * torch.where(pick(rs.shape, 0.5), 0.9, 1.0)
    a["temp"] = f["temp"].clone()
    a["rp"] = f["rp"].clone()
    shp = f["press"].shape
    for d in ("rc", "srp", "snrp", "rtot", "ri", "riri"):
        a[d] = torch.zeros(shp, dtype=torch.float64)
    return inp, a
