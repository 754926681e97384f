"""tend_constrain2 and SALSA_diagnostics (src/src_LES/constrain_SALSA.f90) in the
oracle: the properties the LES relies on after a SALSA step."""
import math

import numpy as np
import pytest
import torch

from oracle_ref import Oracle
from parity import interior
from post_cases import post_state, TENDS
from uclales_salsa_gb300.layout import lolim_diameters


def test_tend_constrain_keeps_values_positive():
    for wl in ("grid16x16x40", "grid256x256x128"):
        inp, a = post_state(wl, X=6, Y=6, Z=6)
        before = {k: v.clone() for k, v in a.items()}
        assert Oracle(inp.cfg).tend_constrain(inp.nzp, inp.nxp, inp.nyp, inp.dt, a) == 0
        for v, t in TENDS.items():
            if t not in a:
                continue
            new = a[v] + a[t] * inp.dt      # at least 1e-8 of the value, up to rounding
            assert float((new - 1e-8 * a[v] + 1e-15 * a[v].abs()).min()) >= 0, v
            lo = (-1. + 1.e-8) * a[v] / inp.dt
            keep = before[t] >= lo
            assert torch.equal(a[t][keep], before[t][keep]), t
            assert torch.equal(a[t][~keep], lo[~keep]), t
        if inp.level == 5:
            assert float(a["indef"].min()) >= 0 and float(a["indef"].max()) <= 1


def test_diagnostics_move_mass_and_report_water():
    for wl in ("grid16x16x40", "grid256x256x128"):
        inp, a = post_state(wl, X=6, Y=6, Z=6)
        lay = inp.layout
        before = {k: v.clone() for k, v in a.items()}
        assert Oracle(inp.cfg).diagnostics(inp.nzp, inp.nxp, inp.nyp, a) == 0
        I = lambda t: interior(t, inp.nzp, inp.nxp, inp.nyp)
        for k in ("naero", "ncloud", "nprecp", "maero", "mcloud", "mprecp"):
            assert float(a[k].min()) >= 0, k
        # evaporated droplets and drops went to the aerosol bins: the total of each dry
        # species over all categories only loses the removed tiny aerosol bins
        nw, iw = lay.nwet, lay.nwet - 1
        cats = [("maero", lay.nbins, nw), ("mcloud", lay.ncld, nw), ("mprecp", lay.nprc, nw)]
        if inp.level == 5:
            cats.append(("mice", lay.nice, nw + 1))
        moved = int((I(before["ncloud"]) > 1).sum() - (I(a["ncloud"]) > 1).sum())
        assert moved > 0
        for s in range(lay.ndry):
            tot = lambda d: sum(d[k].clamp(min=0).view(n, nb, *d[k].shape[1:])[s].sum(0) for k, nb, n in cats)
            t0, t1 = I(tot(before)), I(tot(a))
            assert float((t1 - t0).max()) <= 1e-12 * float(t0.max())
            assert float(((t0 - t1) / t0.clamp(min=1e-30)).median()) < 1e-14
        # water diagnostics
        mc = a["mcloud"].view(nw, lay.ncld, *a["mcloud"].shape[1:])[iw].sum(0)
        ma = a["maero"].view(nw, lay.nbins, *a["maero"].shape[1:])[iw].sum(0)
        mp = a["mprecp"].view(nw, lay.nprc, *a["mprecp"].shape[1:])[iw].sum(0)
        assert torch.allclose(a["rc"], ma + mc, rtol=1e-14, atol=0)
        assert torch.allclose(a["srp"], mp, rtol=1e-14, atol=0)
        rt = a["rc"] + a["srp"] + a["rp"]
        if inp.level == 5:
            rt = rt + a["ri"] + a["riri"]
        assert torch.allclose(a["rtot"], rt, rtol=1e-14, atol=0)


def test_diagnostics_only_diag_changes_no_values_but_negatives():
    inp, a = post_state("grid256x256x128", X=6, Y=6, Z=6)
    before = {k: v.clone() for k, v in a.items()}
    assert Oracle(inp.cfg).diagnostics(inp.nzp, inp.nxp, inp.nyp, a, only_diag=1) == 0
    for k in ("naero", "ncloud", "nprecp", "maero", "mcloud", "mprecp", "nice", "mice", "gaero"):
        assert torch.equal(a[k], before[k].clamp(min=0) if k != "gaero" else before[k]), k


def mag_lo_bits(bp, cm, ce, dk):
    """The integer form of |(-1 + 1e-8) p| / dtlt that tend_constrain_kernel uses for a
    power-of-two dtlt (csrc/salsa_post.cu mag_lo_bits), restated on Python integers:
    the 106-bit product of the significands rounded to nearest even, with the exponents
    added; -1 where the result would not be normal."""
    mp = (bp & ((1 << 52) - 1)) | (1 << 52)
    prod = mp * cm
    ep = (bp >> 52) & 0x7ff
    if prod >> 105:
        m, r, half, e = prod >> 53, prod & ((1 << 53) - 1), 1 << 52, ep + ce - 1022
    else:
        m, r, half, e = prod >> 52, prod & ((1 << 52) - 1), 1 << 51, ep + ce - 1023
    if r > half or (r == half and (m & 1)):
        m += 1
        if m >> 53:
            m >>= 1
            e += 1
    e += dk
    if e <= 0 or e >= 2047:
        return -1
    return (e << 52) | (m & ((1 << 52) - 1))


def test_integer_limit_equals_the_fp64_product():
    """For every normal p > 0 and power-of-two time step, the integer limit has the bits
    of the FP64 expression (-1 + 1e-8) * p / dtlt that tend_constrain2 writes (sign
    aside), including mantissas next to the rounding boundaries; outside the normal range
    it reports -1, and the kernel then takes the FP64 path."""
    import random
    import struct
    bits = lambda x: struct.unpack("<q", struct.pack("<d", x))[0]
    c = -1. + 1.e-8
    cb = bits(-c)
    cm, ce = (cb & ((1 << 52) - 1)) | (1 << 52), (cb >> 52) & 0x7ff
    rng = random.Random(17)
    checked = 0
    for n in range(200000):
        if n % 4 == 0:
            # a mantissa whose product with cm lands next to a rounding boundary
            t = rng.getrandbits(52) | (1 << 52)
            q, rem = divmod((t << 52) + rng.choice((-2, -1, 0, 1, 2)) + (1 << 51), cm)
            mp = q if (1 << 52) <= q < (1 << 53) else (rng.getrandbits(52) | (1 << 52))
            bp = (rng.randrange(1, 2046) << 52) | (mp & ((1 << 52) - 1))
        else:
            bp = (rng.randrange(1, 2046) << 52) | rng.getrandbits(52)
        dtlt = 2.0 ** rng.randrange(-8, 9)
        dk = 1023 - ((bits(dtlt) >> 52) & 0x7ff)
        p = struct.unpack("<d", struct.pack("<q", bp))[0]
        want = abs(c * p / dtlt)
        got = mag_lo_bits(bp, cm, ce, dk)
        wb = bits(want)
        normal = 0 < (wb >> 52) < 2047
        if normal and got >= 0:
            assert got == wb, (p, dtlt)
            checked += 1
        else:
            assert got == -1 or not normal, (p, dtlt)
    assert checked > 150000


DISS = {"SO4": 3., "OC": 1., "BC": 0., "DU": 0., "SS": 2.}
MMOL = {"SO4": 98.08e-3, "OC": 150.e-3, "BC": 12.e-3, "DU": 100.e-3, "SS": 58.44e-3}


def correlation_numpy(x, y):
    """calc_correlation (src/src_LES/util.f90:1005-1024) as the reference writes it:
    the cross term keeps only the last product, and nearly constant vectors (variance
    term below the FP64 epsilon) give 0."""
    n = len(x)
    sx, sy = sum(x), sum(y)
    sx2, sy2 = sum(v * v for v in x), sum(v * v for v in y)
    sxy = x[-1] * y[-1]
    if sx2 * n - sx * sx < np.finfo(float).eps or sy2 * n - sy * sy < np.finfo(float).eps:
        return 0.
    return (sxy * n - sx * sy) / (math.sqrt(sx2 * n - sx * sx) * math.sqrt(sy2 * n - sy * sy))


def diagnostics_numpy(inp, a, lscndgas):
    """Independent restatement of SALSA_diagnostics with findDry4Wet
    (src/src_LES/constrain_SALSA.f90:50-470) on numpy copies of the arrays: negatives
    to zero everywhere; on the horizontal interior, every level, bins with number but
    no mass emptied, then evaporated cloud droplets (below 0.7 of the critical diameter
    or 13 um) to their parallel aerosol bin, drops (below 0.2 of it or 10 um) and dry or
    small ice to the aerosol bin of matching dry size, the b bin taken as fn2a + (ba -
    in2a) as the reference writes it and chosen by composition when both are
    populated, and aerosol bins below 0.1 nm dry diameter removed, their sulphate and
    organics to the gas phase; then the water mixing ratios at every point."""
    lay = inp.layout
    sp = lay.species
    nb, nc, npr, ni, nd = lay.nbins, lay.ncld, lay.nprc, lay.nice, lay.ndry
    nsp = nd + 1
    iwa, irim = nd, nd + 1
    pi, pi6, rg, surfw0, mwa, rhowa, avog = 3.1415927, 0.5235988, 8.314, 0.073, 18.016e-3, 1000., 6.0221e+23
    rhol, rhoi = lay.rholiq(), lay.rhoice()
    aetot = lolim_diameters(lay)
    r = {k: v.numpy().copy() for k, v in a.items()}
    sh = r["naero"].shape[1:]
    lvl5 = inp.level == 5
    if not lvl5:
        ni = 0
    na, nc_, np_ = r["naero"], r["ncloud"], r["nprecp"]
    ma = r["maero"].reshape(nsp, nb, *sh)
    mc = r["mcloud"].reshape(nsp, nc, *sh)
    mp = r["mprecp"].reshape(nsp, npr, *sh)
    ni_ = r["nice"] if lvl5 else None
    mi = r["mice"].reshape(nsp + 1, ni, *sh) if lvl5 else None
    for arr in (na, nc_, np_, ni_, ma, mc, mp, mi):
        if arr is not None:
            np.maximum(arr, 0., out=arr)

    def dry4wet(n, m, ib, q):
        cd = sum(m[s][ib][q] / rhol[s] for s in range(nd)) / n[ib][q]
        cd = (cd / pi6) ** (1. / 3.)
        ba = min(max(lay.in2a + sum(cd > aetot[b] for b in range(lay.in2a, lay.fn2a + 1)) - 1, lay.in2a), lay.fn2a)
        bb = lay.fn2a + (ba - lay.in2a)
        if na[bb][q] <= 1.:
            return ba
        if na[ba][q] <= 1.:
            return bb
        y = [m[s][ib][q] for s in range(nd)]
        ra = correlation_numpy([ma[s][ba][q] for s in range(nd)], y)
        rb = correlation_numpy([ma[s][bb][q] for s in range(nd)], y)
        return bb if ra < rb else ba

    def move(n, m, nsrc, b, ba, q):
        na[ba][q] = na[ba][q] + n[b][q]
        n[b][q] = 0.
        for s in range(nsrc):
            ma[s][ba][q] = ma[s][ba][q] + m[s][b][q]
            m[s][b][q] = 0.

    def critical_diameter(m, b, n, T):
        ns = sum(DISS[sp[s]] * m[s][b] / MMOL[sp[s]] for s in range(nd)) / n
        zbb = 6. * mwa * ns / (pi * rhowa)
        with np.errstate(divide="ignore"):
            zaa = 4. * mwa * surfw0 / (rg * rhowa * T)
        return float(np.sqrt(3. * zbb / zaa))

    for j in range(2, inp.nyp - 2):
        for i in range(2, inp.nxp - 2):
            for k in range(inp.nzp):
                q = (j, i, k)
                for n, m, nbn in ((na, ma, nb), (nc_, mc, nc)):
                    for b in range(nbn):
                        if n[b][q] > 0. and sum(m[s][b][q] for s in range(nsp)) <= 0.:
                            n[b][q] = 0.
                            for s in range(nsp):
                                m[s][b][q] = 0.
                for b in range(npr):
                    if np_[b][q] > 0. and mp[iwa][b][q] <= 0.:
                        np_[b][q] = 0.
                        for s in range(nsp):
                            mp[s][b][q] = 0.
                for b in range(ni):
                    if ni_[b][q] > 0. and mi[iwa][b][q] + mi[irim][b][q] < 1.e-25:
                        ni_[b][q] = 0.
                        for s in range(nsp + 1):
                            mi[s][b][q] = 0.
                T, rh = np.float64(r["temp"][q]), float(r["rh"][q])     # IEEE division at T = 0
                rhi = float(r["rhi"][q]) if lvl5 else 1.
                for b in range(nc):
                    n = nc_[b][q]
                    if n > 1. and rh < 0.999 and mc[iwa][b][q] < 1.e-5:
                        cd = critical_diameter([[mc[s][bb][q] for bb in range(nc)] for s in range(nd)], b, n, T)
                        d = (sum(mc[s][b][q] / rhol[s] for s in range(nsp)) / n / pi6) ** (1. / 3.)
                        if d < min(0.7 * cd, 1.3e-5) or mc[iwa][b][q] < 1.e-25 * n:
                            move(nc_, mc, nsp, b, lay.cloud_parallel(b), q)
                for b in range(npr):
                    n = np_[b][q]
                    if n > 1.e-6 and rh < 0.999 and mp[iwa][b][q] < 1.e-6:
                        cd = critical_diameter([[mp[s][bb][q] for bb in range(npr)] for s in range(nd)], b, n, T)
                        d = (sum(mp[s][b][q] / rhol[s] for s in range(nsp)) / n / pi6) ** (1. / 3.)
                        if d < min(0.2 * cd, 10.e-6) or mp[iwa][b][q] < 1.e-25 * n:
                            move(np_, mp, nsp, b, dry4wet(np_, mp, b, q), q)
                for b in range(ni):
                    n = ni_[b][q]
                    if n > 1.e-6 and rhi < 0.999 and mi[iwa][b][q] + mi[irim][b][q] < 1.e-15:
                        d = (sum(mi[s][b][q] / rhoi[s] for s in range(nsp + 1)) / n / pi6) ** (1. / 3.)
                        dry = sum(mi[s][b][q] for s in range(nd)) / sum(mi[s][b][q] for s in range(nsp + 1))
                        if dry > 0.5 or d < 2.e-6:
                            ba = dry4wet(ni_, mi, b, q)
                            rime = mi[irim][b][q]
                            move(ni_, mi, nsp, b, ba, q)
                            ma[iwa][ba][q] = ma[iwa][ba][q] + rime
                            mi[irim][b][q] = 0.
                for b in range(nb):
                    n = na[b][q]
                    if n > 1. and sum(ma[s][b][q] / rhol[s] for s in range(nd)) / n < pi6 * 1.e-10 ** 3:
                        if lscndgas:
                            for name, g in (("SO4", 0), ("OC", 4)):
                                if name in sp:
                                    s = sp.index(name)
                                    r["gaero"][g][q] = r["gaero"][g][q] + ma[s][b][q] / MMOL[name] * avog
                        for s in range(nsp):
                            ma[s][b][q] = 0.
                        na[b][q] = 0.
    r["rc"] = ma[iwa][lay.in1a:lay.fn2b + 1].sum(0) + mc[iwa].sum(0)
    r["srp"] = mp[iwa].sum(0)
    r["snrp"] = np_.sum(0)
    r["rtot"] = r["rc"] + r["srp"] + r["rp"]
    if lvl5:
        r["ri"] = mi[iwa].sum(0)
        r["riri"] = mi[irim].sum(0)
        r["rtot"] = r["rtot"] + r["ri"] + r["riri"]
    return r


def test_diagnostics_match_independent_restatement():
    """SALSA_diagnostics in the oracle against the restatement above on perturbed
    post-step states of both workloads, every branch taken somewhere: each number
    and mass array, the gas concentrations and the water mixing ratios (1e-14; the
    bin moves themselves agree exactly)."""
    moves = dict(ncloud=0, nprecp=0, nice=0, gaero=0)
    for wl in ("grid16x16x40", "grid256x256x128"):
        inp, a = post_state(wl, X=6, Y=6, Z=6)
        want = diagnostics_numpy(inp, a, bool(inp.cfg.lscndgas))
        before = {k: v.clone() for k, v in a.items()}
        assert Oracle(inp.cfg).diagnostics(inp.nzp, inp.nxp, inp.nyp, a) == 0
        for k, w in want.items():
            got = a[k].numpy()
            assert got == pytest.approx(w, rel=1e-14, abs=0.), (wl, k)
        # count the moves: cloud, drops and ice to aerosol, tiny aerosol to gas
        for k, lim in (("ncloud", 1.), ("nprecp", 1.e-6), ("nice", 1.e-6)):
            if k in a:
                moves[k] += int((before[k] > lim).sum() - (a[k] > lim).sum())
        moves["gaero"] += int((a["gaero"] != before["gaero"]).sum())
    assert min(moves.values()) > 0, moves


def test_diagnostics_choose_the_aerosol_bin_by_composition():
    """Evaporating drops and dry ice crystals into populated a and b aerosol bins of
    random composition, so that findDry4Wet decides by calc_correlation (both
    outcomes occur), the ice carrying rime that goes to the aerosol water: the oracle
    against the restatement above.  calc_correlation returns 0 when a variance term
    is below the FP64 epsilon, which mass mixing ratios of realistic aerosol (1e-9
    kg/kg) always are, so the masses here are raised to 1e-6 kg/kg and more for the
    composition to decide."""
    inp, a = post_state("grid256x256x128", X=6, Y=6, Z=6)
    lay = inp.layout
    nd, nsp = lay.ndry, lay.nwet
    rng = np.random.default_rng(23)
    sh = a["naero"].shape[1:]
    ma = a["maero"].view(nsp, lay.nbins, *sh)
    mp = a["mprecp"].view(nsp, lay.nprc, *sh)
    mi = a["mice"].view(nsp + 1, lay.nice, *sh)
    rho = lay.rholiq()
    aetot = lolim_diameters(lay)
    for j in range(2, inp.nyp - 2):
        for i in range(2, inp.nxp - 2):
            for k in range(inp.nzp):
                a["rh"][j, i, k] = a["rhi"][j, i, k] = 0.9
                big = (i + j + k) % 3 != 0           # else realistic masses: no composition choice
                for b in range(lay.nbins):
                    a["naero"][b, j, i, k] = 10. ** rng.uniform(2., 8.)
                    for s in range(nd):
                        ma[s, b, j, i, k] = float(rng.uniform(0., 1.)) * (1.e-5 if big else 1.e-9)
                for m, n, nb, extra in ((mp, a["nprecp"], lay.nprc, ()), (mi, a["nice"], lay.nice, (nsp,))):
                    for b in range(nb):
                        n[b, j, i, k] = num = 10. ** rng.uniform(12., 14.) * (1. if big else 1.e-5)
                        # dry diameter inside the 2a range, random composition
                        d = float(np.exp(rng.uniform(np.log(aetot[lay.in2a]), np.log(1.5 * aetot[lay.fn2a]))))
                        w = rng.uniform(0., 1., nd)
                        v = num * 0.5235988 * d ** 3
                        for s in range(nd):
                            m[s, b, j, i, k] = v * w[s] / w.sum() * rho[s]
                        m[nsp - 1, b, j, i, k] = 1.e-30 * num
                        for s in extra:
                            m[s, b, j, i, k] = 3.e-30 * num
    calls = []

    def corr(x, y):
        r = correlation_numpy(x, y)
        calls.append(r)
        return r
    g = dict(globals())
    g["correlation_numpy"] = corr
    restated = type(diagnostics_numpy)(diagnostics_numpy.__code__, g)
    want = restated(inp, a, bool(inp.cfg.lscndgas))
    before = {k: v.clone() for k, v in a.items()}
    assert Oracle(inp.cfg).diagnostics(inp.nzp, inp.nxp, inp.nyp, a) == 0
    for k, w in want.items():
        assert a[k].numpy() == pytest.approx(w, rel=1e-14, abs=0.), k
    pairs = list(zip(calls[0::2], calls[1::2]))
    assert sum(ra < rb for ra, rb in pairs) > 20 and sum(ra > rb for ra, rb in pairs) > 20
    assert sum(ra == rb == 0. for ra, rb in pairs) > 20
    assert int((a["nice"] < before["nice"]).sum()) > 100 and int((a["nprecp"] < before["nprecp"]).sum()) > 100
