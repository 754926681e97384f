"""Rime splintering (mo_salsa_SIP_RS.f90), drop fracturing (mo_salsa_SIP_DF.f90) and
ice-ice collisional breakup (mo_salsa_SIP_IIBR.f90), through mo_salsa_secondary_ice.f90,
in the oracle: the properties of the reference's schemes (budgets, temperature ranges and
tracers).  tests/test_gpu_sip.py compares the GPU form with the oracle."""
import pytest
import torch

from uclales_salsa_gb300.inputs import make_outputs
from oracle_ref import Oracle
from parity import interior
from sip_cases import sip_state


def _step(inp):
    f = {k: v.clone() for k, v in inp.fields.items()}
    out = make_outputs(inp)
    rc, st = Oracle(inp.cfg).run(inp, f, out, time=1.0)
    assert rc == 0, st.as_dict()
    I = lambda t: interior(t, inp.nzp, inp.nxp, inp.nyp)
    new = {k: I(f[k] + out[t] * inp.dt) for k, t in (("nice", "nicet"), ("mice", "micet"), ("nprecp", "nprecpt"),
                                                    ("ncloud", "ncloudt"))}
    return new, I(inp.fields["temp"])


@pytest.mark.parametrize("mode", [1, 2])
def test_splinters_conserve_ice_volume_and_add_crystals(mode):
    """With coagulation alone, the scheme moves rime-ice volume from the riming bins to
    the splinter bin (ice volume per species conserved) and adds crystals."""
    a, T = _step(sip_state(mode, splinter=False))
    b, _ = _step(sip_state(mode, splinter=True))
    inp = sip_state(mode)
    lay = inp.layout
    nw1, nic = lay.nwet + 1, lay.nice
    ma = a["mice"].view(nw1, nic, *a["mice"].shape[1:]).sum(1)
    mb = b["mice"].view(nw1, nic, *b["mice"].shape[1:]).sum(1)
    scale = ma.abs().amax(0).clamp(min=1e-30)
    assert float(((mb - ma).abs() / scale).max()) < 1e-12
    dn = b["nice"].sum(0) - a["nice"].sum(0)
    assert float(dn.min()) >= -1e-12 * float(a["nice"].sum(0).max())
    assert int((dn > 0).sum()) > 5
    # the splinters land in the first ice bin (10 um is below every bin's lower limit)
    assert float((b["nice"][0] - a["nice"][0]).max()) > 0
    # the other categories are untouched by the scheme itself
    assert torch.equal(a["nprecp"], b["nprecp"]) and torch.equal(a["ncloud"], b["ncloud"])


def test_no_splinters_outside_the_temperature_range():
    """Rime splintering acts between 238.15 K and 273.15 K only (:64-66)."""
    a, T = _step(sip_state(1, splinter=False))
    b, _ = _step(sip_state(1, splinter=True))
    out = (T < 238.15) | (T > 273.15)
    assert int(out.sum()) > 0
    for k in ("nice", "mice"):
        assert torch.equal(a[k][:, out], b[k][:, out]), k


def test_hallett_mossop_counts_rime_mass_and_mossop_counts_drops():
    """Mode 1 makes 3.5e8 splinters per kg of rime, mode 2 one per 250 frozen drops:
    for the same collisions mode 1 gives far more splinters here (drops of ~1e-9 kg)."""
    a, _ = _step(sip_state(1, splinter=False))
    d1 = _step(sip_state(1))[0]["nice"].sum(0) - a["nice"].sum(0)
    d2 = _step(sip_state(2))[0]["nice"].sum(0) - a["nice"].sum(0)
    assert float(d1.sum()) > 100 * float(d2.sum()) > 0


@pytest.mark.parametrize("mode", [1, 2, 3, 4])
def test_drop_fracturing_conserves_ice_volume_and_adds_small_crystals(mode):
    """Frozen drops above 100 um shatter into fragments spread over the ice bins below
    their size: ice volume per species conserved, crystals added, small bins gain."""
    kw = dict(scheme="lssipdropfrac")
    a, T = _step(sip_state(mode, splinter=False, **kw))
    b, _ = _step(sip_state(mode, **kw))
    lay = sip_state(mode, **kw).layout
    nw1, nic = lay.nwet + 1, lay.nice
    ma = a["mice"].view(nw1, nic, *a["mice"].shape[1:]).sum(1)
    mb = b["mice"].view(nw1, nic, *b["mice"].shape[1:]).sum(1)
    scale = ma.abs().amax(0).clamp(min=1e-30)
    assert float(((mb - ma).abs() / scale).max()) < 1e-12
    dn = b["nice"].sum(0) - a["nice"].sum(0)
    assert int((dn > 0).sum()) > 5
    assert float((b["nice"][0] - a["nice"][0]).max()) > 0
    out = (T < 248.15) | (T > 271.15)             # the scheme's range (:56)
    assert int(out.sum()) > 0
    assert torch.equal(a["nice"][:, out], b["nice"][:, out])


@pytest.mark.parametrize("mode", [1, 2, 3])
def test_ice_ice_breakup_conserves_ice_volume_and_adds_fragments(mode):
    """Collisions of a crystal with larger ones break it into fragments spread over the
    bins below its size (Sullivan; Sotiropoulou): volume conserved, crystals added, and
    nothing outside 248.15-270.15 K."""
    kw = dict(scheme="lssipicecollbreak")
    a, T = _step(sip_state(mode, splinter=False, **kw))
    b, _ = _step(sip_state(mode, **kw))
    lay = sip_state(mode, **kw).layout
    nw1, nic = lay.nwet + 1, lay.nice
    ma = a["mice"].view(nw1, nic, *a["mice"].shape[1:]).sum(1)
    mb = b["mice"].view(nw1, nic, *b["mice"].shape[1:]).sum(1)
    scale = ma.abs().amax(0).clamp(min=1e-30)
    assert float(((mb - ma).abs() / scale).max()) < 1e-12
    dn = b["nice"].sum(0) - a["nice"].sum(0)
    assert int((dn > 0).sum()) > 5
    out = (T < 248.15) | (T > 270.15)
    assert int(out.sum()) > 0
    assert torch.equal(a["nice"][:, out], b["nice"][:, out])


@pytest.mark.parametrize("scheme,mode,tracer,rate", [("lssiprimespln", 1, "siprmspl", 18),
                                                      ("lssipdropfrac", 1, "sipdrfr", 17),
                                                      ("lssipicecollbreak", 1, "sipiibr", 19)])
def test_tracers_gain_what_the_rates_report(scheme, mode, tracer, rate):
    """Each scheme adds its fragments to its tracer (per ice bin, mo_salsa_SIP_*.f90) and
    to its rate diagnostic (per second, run_SALSA :412-416): summed over the ice bins,
    the tracer's gain is the rate times the time step."""
    inp = sip_state(mode, scheme=scheme)
    before = inp.fields[tracer].clone()
    f = {k: v.clone() for k, v in inp.fields.items()}
    out = make_outputs(inp)
    rc, _ = Oracle(inp.cfg).run(inp, f, out, time=1.0)
    assert rc == 0
    gain = (f[tracer] - before).sum(0)
    expect = out["diag"][rate] * inp.dt
    assert float(expect.max()) > 0
    assert float((gain - expect).abs().max()) <= 1e-12 * float(expect.abs().max())
    others = [t for t in ("sipdrfr", "siprmspl", "sipiibr") if t != tracer]
    for t in others:                          # the other schemes are off: their tracers pass through
        assert float((f[t] - inp.fields[t]).abs().max()) <= 1e-15 * float(inp.fields[t].abs().max())
