"""sedim_SALSA (src/src_LES/mcrp.f90:745-1275) in the oracle: the budgets that the
reference's deposition schemes close, and the overwrite / add-to semantics of its
outputs."""
import torch

from oracle_ref import Oracle
from parity import interior
from sedim_cases import sedim_state, VALUE, TEND, FILL

ALVL = 2.5e6


def _run(inp, a, dtlt, sed):
    b = {k: v.clone() for k, v in a.items()}
    assert Oracle(inp.cfg).sedimentation(inp.nzp, inp.nxp, inp.nyp, dtlt, sed, b) == 0
    return b


def _cols(t, inp):
    """Interior columns (all levels) of a (..., nyp, nxp, nzp) tensor."""
    return t[..., 2:inp.nyp - 2, 2:inp.nxp - 2, :]


def test_fast_fall_moves_parcels_without_loss():
    """With one level thickness, DepositionFast only moves number and mass down the
    column (parcels that reach the ground go to the lowest level)."""
    for dtlt in (1.0, 4.0):
        inp, a = sedim_state("grid256x256x128", X=4, Y=4, Z=40, dz=4.0)
        b = _run(inp, a, dtlt, (0, 0, 1, 1))
        for part in ("precp", "ice"):
            for v, t in zip(VALUE[part], TEND[part]):
                d = _cols(b[t] - a[t], inp) * dtlt
                tot = d.sum(-1)
                scale = _cols(a[v], inp).abs().sum(-1).clamp(min=1e-300)
                assert float((tot.abs() / scale).max()) < 1e-12, (part, v)
                assert float(d.abs().max()) > 0, (part, v)
        # some parcels cross more than one level at dtlt = 4 s (up to 9.2 m/s x 4 s over 4 m levels)
        vt = interior(b["VtPrc"], inp.nzp, inp.nxp, inp.nyp)
        if dtlt == 4.0:
            assert float(vt.max()) * dtlt > 2 * 4.0


def test_slow_divergence_equals_surface_deposition():
    """DepositionSlow's flux divergence telescopes: the column's water loss equals the
    surface flux, which the reference reports in sfcrrate (its sum also takes in the
    last bin of the species before water, set to zero here)."""
    inp, a = sedim_state("grid16x16x40", X=4, Y=4, Z=24)
    lay = inp.layout
    nw = lay.nwet
    for part, nb in (("aero", lay.nbins), ("cloud", lay.ncld)):
        m = a[VALUE[part][1]].view(nw, nb, *a[VALUE[part][1]].shape[1:])
        m[nw - 2, nb - 1] = 0.0
    b = _run(inp, a, 1.0, (1, 1, 0, 0))
    adn, dzt = a["adn"], a["dzt"]
    lost = 0
    for part, nb in (("aero", lay.nbins), ("cloud", lay.ncld)):
        t = TEND[part][1]
        d = (b[t] - a[t]).view(nw, nb, *a[t].shape[1:])[nw - 1].sum(0)      # water, all bins
        lost = lost + (_cols(d * adn / dzt, inp)).sum(-1)
    sfc = b["sfcrrate"][2:inp.nyp - 2, 2:inp.nxp - 2]
    assert float(sfc.min()) > 0
    assert torch.allclose(-lost * ALVL, sfc, rtol=1e-9, atol=0)


def test_rates_and_fall_speeds():
    inp, a = sedim_state("grid256x256x128", X=4, Y=4, Z=20)
    lay = inp.layout
    b = _run(inp, a, 1.0, (0, 0, 1, 0))
    vt = b["VtPrc"]
    n = a["nprecp"]
    I = lambda x: interior(x, inp.nzp, inp.nxp, inp.nyp)
    act = I(n) >= 1e-6
    assert int(act.sum()) > 0
    assert float(I(vt)[act].min()) > 0 and float(I(vt)[act].max()) <= 9.2
    assert float(I(vt)[~act].abs().max()) == 0
    # halo columns and the outer levels: zero, as after the reference's whole-array zeroing
    assert float(vt[..., :2, :, :].abs().max()) == 0 and float(vt[..., :, :, 0].abs().max()) == 0
    # rrate is the downward water flux of the bins, sum over bins in bin order
    nw = lay.nwet
    mw = a["mprecp"].view(nw, lay.nprc, *n.shape[1:])[nw - 1]
    rr = torch.zeros_like(b["rrate"])
    for bb in range(lay.nprc):
        rr = rr + mw[bb] * a["adn"] * vt[bb] * ALVL
    assert torch.allclose(b["rrate"], rr, rtol=1e-14, atol=0)
    assert float(b["irate"].abs().max()) == 0 and float(b["sfcirate"].abs().max()) == 0
    # tendencies and tlt of the halo are untouched; rates overwritten everywhere
    assert torch.equal(b["nprecpt"][..., :2, :, :], a["nprecpt"][..., :2, :, :])
    assert float((b["rrate"] == FILL).sum()) == 0 and float((b["sfcrrate"] == FILL).sum()) == 0


def test_switches_and_arguments():
    inp, a = sedim_state("grid16x16x40", X=3, Y=3, Z=8)
    b = _run(inp, a, 1.0, (0, 0, 0, 0))
    for k in ("naerot", "maerot", "ncloudt", "mcloudt", "nprecpt", "mprecpt", "tlt", "VtPrc"):
        assert torch.equal(a[k], b[k]), k
    assert float(b["rrate"].abs().max()) == 0
    # a missing array of a switched-on part is an argument error (SALSA_E_ARG)
    c = {k: v.clone() for k, v in a.items() if k != "mcloudt"}
    assert Oracle(inp.cfg).sedimentation(inp.nzp, inp.nxp, inp.nyp, 1.0, (0, 1, 0, 0), c) == 1
    assert Oracle(inp.cfg).sedimentation(inp.nzp, inp.nxp, inp.nyp, 0.0, (1, 1, 1, 1), a) == 1


def test_long_step_deposits_every_drop():
    """With dtlt = 1e5 s every populated precipitation parcel falls through the column:
    it leaves its level and lands on the lowest one (one level thickness, so without
    rescaling), and the surface rate is the water flux of all those parcels."""
    inp, a = sedim_state("grid256x256x128", X=4, Y=4, Z=12, dz=5.0)
    lay = inp.layout
    dtlt = 1.0e5   # 20 um drops fall ~1 cm/s: 1 km in that time, the column is 60 m
    b = _run(inp, a, dtlt, (0, 0, 1, 0))
    n = a["nprecp"]
    act = n >= 1e-6
    d = (b["nprecpt"] - a["nprecpt"]) * dtlt
    cols = _cols(d, inp)
    nc = _cols(n * act, inp)
    assert int(act.sum()) > 10
    # levels 1..nzp-2 lose their parcel; level 0 gains the column's total
    assert torch.allclose(cols[..., 1:-1], -nc[..., 1:-1], rtol=1e-12, atol=0)
    assert torch.allclose(cols[..., 0], nc[..., 1:-1].sum(-1), rtol=1e-12, atol=0)
    # surface rate: sum over the reference's range (last bin of the species before
    # water, then the water bins) of m * adn * Vt over the column, times alvl
    nw, nb = lay.nwet, lay.nprc
    m = a["mprecp"].view(nw, nb, *n.shape[1:])
    vt = b["VtPrc"]
    terms = [m[nw - 2, nb - 1] * a["adn"] * vt[nb - 1]] + [m[nw - 1, k] * a["adn"] * vt[k] for k in range(nb)]
    sfc = sum(_cols(t, inp)[..., 1:-1].sum(-1) for t in terms) * ALVL
    got = b["sfcrrate"][2:inp.nyp - 2, 2:inp.nxp - 2]
    assert float(got.max()) > 0
    assert torch.allclose(got, sfc, rtol=1e-12, atol=0)


def test_nothing_to_sediment():
    """Empty bins everywhere: tendencies and tlt unchanged, rates and fall speeds zero."""
    inp, a = sedim_state("grid16x16x40", X=3, Y=3, Z=6)
    for k in ("naero", "ncloud", "nprecp", "maero", "mcloud", "mprecp"):
        a[k] = torch.zeros_like(a[k])
    b = _run(inp, a, 1.0, (1, 1, 1, 1))
    for k in ("naerot", "maerot", "ncloudt", "mcloudt", "nprecpt", "mprecpt", "tlt"):
        assert torch.equal(b[k], a[k]), k
    for k in ("rrate", "sfcrrate", "VtPrc"):
        assert float(b[k].abs().max()) == 0, k
