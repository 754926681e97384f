"""tend_constrain2 and SALSA_diagnostics (src/src_LES/constrain_SALSA.f90) in the
oracle: the properties the LES relies on after a SALSA step."""
import torch

from oracle_ref import Oracle
from parity import interior
from post_cases import post_state, TENDS


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
