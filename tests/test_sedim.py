"""sedim_SALSA (src/src_LES/mcrp.f90:745-1275) in the oracle: the budgets that the
reference's deposition schemes close, and the overwrite / add-to semantics of its
outputs."""
import math

import numpy as np
import pytest
import torch

from fall_speed import terminal_vel_numpy, ice_shape_numpy, ice_terminal_vel_numpy
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


def sedim_numpy(inp, a, dtlt, sed):
    """Independent restatement of sedim_SALSA, DepositionSlow and DepositionFast
    (src/src_LES/mcrp.f90:745-1275) on numpy copies of the arrays, levels 0-based (the
    reference's k = level + 1).  Slow particles (aerosol, cloud): the flux -x vc of
    every level from the top interior level down, vc the fall speed capped at half a
    level per step and 2 m/s, plus the dry-deposition velocity 1/rt at the level above
    the surface; the tendency takes the flux divergence.  Fast particles
    (precipitation, ice): each parcel falls dtlt vc, is removed from its level and put
    into the level it reaches and the one below (by the overshoot, or all into the one
    below when that is more than half the level), parcels that reach the lowest
    interior level landing on level 0.  rrate / irate take the water fluxes,
    sfcrrate / sfcirate the surface fluxes over the reference's index ranges (which
    start at the last bin of the species before water), tlt the latent heat, VtPrc /
    VtIce the fall speeds."""
    lay = inp.layout
    r = {k: v.numpy().copy() for k, v in a.items()}
    nyp, nxp, nzp = inp.nyp, inp.nxp, inp.nzp
    pi_les, kb, g, alvl, alvi, cp = 3.14159265358979323846264338327, 1.3807e-23, 9.81, 2.5e6, 2.834e6, 1005.
    pi6, A, B, Cc, M = 0.5235988, 1.249, 0.42, 0.87, 4.8096e-26
    tk, adn, th, dzt, ustar = r["tk"], r["adn"], r["th"], r["dzt"], r["ustar"]
    nw = lay.nwet
    lvl5 = inp.level == 5
    r["rrate"][...] = 0.
    r["sfcrrate"][...] = 0.
    if lvl5:
        r["irate"][...] = 0.
        r["sfcirate"][...] = 0.

    def air(q):
        T = tk[q]
        avis = 1.8325e-5 * (416.16 / (T + 120.0)) * (T / 296.16) ** 1.5
        va = math.sqrt(8. * kb * T / (pi_les * M))
        return avis, avis / adn[q], 2. * avis / (adn[q] * va)

    def particle(m, n, b, flag, rho, q):
        """dwet (sphere of the bin's volume), density, slip factor and, for ice, the
        maximum dimension and the shape coefficients."""
        pm = [float(m[s][b][q]) for s in range(len(m))]
        nn = float(n[b][q])
        dwet = (sum(x / rh for x, rh in zip(pm, rho)) / nn / pi6) ** (1. / 3.)
        zdn = sum(pm) / nn / (pi6 * dwet ** 3)
        shape, dnsp = None, None
        if flag == 4:
            shape, dnsp, _ = ice_shape_numpy(sum(pm[:-1]), pm[-1], nn)
        return pm, dwet, zdn, shape, dnsp

    def fall(dwet, zdn, q, avis, lam, flag, shape, dnsp):
        kn = 2. * lam / dwet
        gg = 1. + kn * (A + B * math.exp(-Cc / kn))
        if flag < 4:
            return terminal_vel_numpy(dwet, zdn, adn[q], avis, gg), gg
        return ice_terminal_vel_numpy(dwet, dnsp, zdn, adn[q], avis, shape), gg

    def slow(nk, mk, tk_, nb, flag):
        n, m = r[nk], r[mk].reshape(nw, nb, nyp, nxp, nzp)
        rho = lay.rholiq()
        clim = 1.
        divn = np.zeros_like(n)
        divm = np.zeros((nw, nb, nyp, nxp, nzp))
        for j in range(2, nyp - 2):
            for i in range(2, nxp - 2):
                rflm = np.zeros((nzp, nw, nb))
                rfln = np.zeros((nzp, nb))
                for k in range(nzp - 2, 0, -1):
                    q = (j, i, k)
                    avis, kvis, lam = air(q)
                    for b in range(nb):
                        if n[b][q] < clim:
                            continue
                        pm, dwet, zdn, _, _ = particle(m, n, b, flag, rho, q)
                        vc, gg = fall(dwet, zdn, q, avis, lam, flag, None, None)
                        vc = min(vc, min(0.5 * (1. / dzt[k]) / dtlt, 2.0))
                        if k == 1:
                            mdiff = kb * tk[q] * gg / (3.0 * pi_les * avis * dwet)
                            sc = kvis / mdiff
                            st = max(vc * ustar[j, i] ** 2.0 / g * kvis, 0.01)
                            rt = 1.0 / max(np.finfo(float).eps, ustar[j, i] * (sc ** (-2.0 / 3.0) + 10. ** (-3.0 / st)))
                            vc = 1. / rt + vc
                        for s in range(nw):
                            rflm[k, s, b] = -m[s][b][q] * vc
                        rfln[k, b] = -n[b][q] * vc
                    for s in range(nw):
                        for b in range(nb):
                            divm[s, b, j, i, k] = (rflm[k + 1, s, b] * adn[j, i, k + 1] - rflm[k, s, b] * adn[q]) * \
                                dzt[k] / adn[q]
                    for b in range(nb):
                        divn[b, j, i, k] = (rfln[k + 1, b] * adn[j, i, k + 1] - rfln[k, b] * adn[q]) * dzt[k] / adn[q]
                    # the reference's range: the last bin of the species before water, then water
                    r["rrate"][q] = r["rrate"][q] - (rflm[k, nw - 2, nb - 1] + rflm[k, nw - 1].sum()) * adn[q] * alvl
                r["sfcrrate"][j, i] = r["sfcrrate"][j, i] - (rflm[1, nw - 2, nb - 1] + rflm[1, nw - 1].sum()) * \
                    adn[j, i, 1] * alvl
        r[tk_[0]] -= divn
        r[tk_[1]] -= divm.reshape(nw * nb, nyp, nxp, nzp)
        for j in range(2, nyp - 2):
            for i in range(2, nxp - 2):
                for k in range(1, nzp):
                    r["tlt"][j, i, k] += divm[nw - 1, :, j, i, k].sum() * (alvl / cp) * th[j, i, k] / tk[j, i, k]

    def fast(nk, mk, tk_, nb, ns, flag, vt, rate, srate, rho, lat):
        n, m = r[nk], r[mk].reshape(ns, nb, nyp, nxp, nzp)
        r[vt][...] = 0.
        prnt = np.zeros((nb, nyp, nxp, nzp))
        prvt = np.zeros((ns, nb, nyp, nxp, nzp))
        for j in range(2, nyp - 2):
            for i in range(2, nxp - 2):
                rem = np.zeros((ns, nb))
                for k in range(nzp - 2, 0, -1):
                    q = (j, i, k)
                    avis, _, lam = air(q)
                    for b in range(nb):
                        if n[b][q] < 1.e-6:
                            continue
                        pm, dwet, zdn, shape, dnsp = particle(m, n, b, flag, rho, q)
                        vc, _ = fall(dwet, zdn, q, avis, lam, flag, shape, dnsp)
                        r[vt][b][q] = vc
                        fdmax = dtlt * vc
                        fd, fi, dep = 0., 0, False
                        while fd < fdmax:
                            fd = fd + 1. / dzt[k - fi]
                            fi = fi + 1
                            if k - fi <= 0:
                                dep = True
                                break
                        fi = fi - 1
                        kf = k - fi
                        fd = fd - 1. / dzt[kf]
                        fdos = min(max(fdmax - fd, 0.), 1. / dzt[kf])
                        num = n[b][q]
                        prnt[b, j, i, k] -= num
                        for s in range(ns):
                            prvt[s, b, j, i, k] -= pm[s]
                        if dep:
                            for s in range(ns):
                                rem[s, b] += pm[s] * adn[q] * vc
                        water = pm[ns - 2] + pm[ns - 1] if flag == 4 else pm[ns - 1]
                        r[rate][q] += water * adn[q] * vc * lat
                        if fdos * dzt[kf] > 0.5:
                            prnt[b, j, i, kf - 1] += num * dzt[kf - 1] / dzt[k]
                            for s in range(ns):
                                prvt[s, b, j, i, kf - 1] += pm[s] * dzt[kf - 1] / dzt[k]
                        else:
                            f = fdos * dzt[kf]
                            prnt[b, j, i, kf - 1] += f * num * dzt[kf - 1] / dzt[kf]
                            prnt[b, j, i, kf] += (1. - f) * num
                            for s in range(ns):
                                prvt[s, b, j, i, kf - 1] += f * pm[s] * dzt[kf - 1] / dzt[kf]
                                prvt[s, b, j, i, kf] += (1. - f) * pm[s]
                # the reference's range starts one bin early (the last bin of the species before)
                first = ns - 3 if flag == 4 else ns - 2
                r[srate][j, i] += (rem[first, nb - 1] + rem[first + 1:].sum()) * lat
        r[tk_[0]] += prnt / dtlt
        r[tk_[1]] += prvt.reshape(ns * nb, nyp, nxp, nzp) / dtlt
        lo = ns - 2 if flag == 4 else ns - 1
        for j in range(2, nyp - 2):
            for i in range(2, nxp - 2):
                for k in range(0, nzp - 1):
                    r["tlt"][j, i, k] -= (prvt[lo:, :, j, i, k].sum() / dtlt) * (lat / cp) * th[j, i, k] / tk[j, i, k]

    if sed[0]:
        slow("naero", "maero", TEND["aero"], lay.nbins, 1)
    if sed[1]:
        slow("ncloud", "mcloud", TEND["cloud"], lay.ncld, 2)
    if sed[2]:
        fast("nprecp", "mprecp", TEND["precp"], lay.nprc, nw, 3, "VtPrc", "rrate", "sfcrrate", lay.rholiq(), alvl)
    if sed[3] and lvl5:
        fast("nice", "mice", TEND["ice"], lay.nice, nw + 1, 4, "VtIce", "irate", "sfcirate", lay.rhoice(), alvi)
    return r


def test_sedimentation_matches_independent_restatement():
    """sedim_SALSA in the oracle against the restatement above, all four parts on,
    for both workloads with level thicknesses that vary from level to level and a
    step that carries the largest drops and crystals over several levels, and with
    levels thin enough for the cap of half a level per step to bind: every tendency,
    tlt, the rates and the fall speeds (1e-12).  A parcel that partly stays
    on its level leaves a small difference of two moved amounts there, so the
    tendencies of the fast parts are held to 1e-14 of the largest amount in their
    column (times the largest ratio of level thicknesses, by which a landing parcel
    is scaled) rather than to their own size."""
    cases = (("grid16x16x40", dict(X=3, Y=3, Z=24), 1.0), ("grid256x256x128", dict(X=3, Y=3, Z=40), 3.0),
             ("grid256x256x128", dict(X=3, Y=3, Z=16, dz=(0.005, 0.05)), 2.0))   # thin levels: the slow cap binds
    for wl, kw, dtlt in cases:
        inp, a = sedim_state(wl, **kw)
        want = sedim_numpy(inp, a, dtlt, (1, 1, 1, 1))
        b = _run(inp, a, dtlt, (1, 1, 1, 1))
        value = {t: v for part in VALUE for v, t in zip(VALUE[part], TEND[part])}
        for k, w in want.items():
            tol = 1e-300
            if k in value and k in a:
                stretch = float(a["dzt"].max() / a["dzt"].min())     # a parcel lands scaled by dzt ratios
                tol = 1e-14 * stretch * a[value[k]].abs().amax(-1, keepdim=True).numpy() / dtlt + 1e-300
            got = b[k].numpy()
            bad = np.abs(got - w) > np.maximum(1e-12 * np.abs(w), tol)
            assert not bad.any(), (wl, k, np.argwhere(bad)[:3], got[bad][:3], w[bad][:3])
