"""GPU parity of the step's secondary-ice form (rime splintering, drop fracturing,
ice-ice breakup) against the oracle, with the step's parity criterion.
"""
import pytest

from sip_cases import sip_state
from test_gpu_parity import oracle_run, gpu_run, envelope, check, VIOL_FRAC, FRAC_WITHIN

pytestmark = pytest.mark.gpu

SCHEMES = [("lssiprimespln", 1), ("lssiprimespln", 2), ("lssipdropfrac", 1), ("lssipdropfrac", 2),
           ("lssipdropfrac", 3), ("lssipdropfrac", 4), ("lssipicecollbreak", 1), ("lssipicecollbreak", 2),
           ("lssipicecollbreak", 3)]


def _parity(inp, rtol, eps):
    fg, gpu = gpu_run(inp)
    fr, ref = oracle_run(inp)
    env = envelope(inp, ref, eps)
    rep = check(inp, gpu, ref, env, rtol)
    print(rep)
    for k, r in rep.items():
        assert r["violations"] <= VIOL_FRAC * r["n"], (k, r)
        assert r["frac_within"] >= FRAC_WITHIN, (k, r)
    # the tracers (updated in place) and the three rate diagnostics, relative to each
    # field's largest value
    pairs = [(fg[k].cpu(), fr[k]) for k in ("sipdrfr", "siprmspl", "sipiibr")]
    pairs += [(gpu["diag"][i], ref["diag"][i]) for i in (17, 18, 19)]
    for a, b in pairs:
        scale = float(b.abs().max())    # zero for the rates of schemes that are off
        assert float((a - b).abs().max()) <= 1e-6 * scale
    return ref


@pytest.mark.parametrize("scheme,mode", SCHEMES)
def test_secondary_ice_fp64_parity(scheme, mode):
    """Coagulation and one scheme: the GPU step matches the oracle, and the scheme
    changes the ice numbers by far more than the tolerance (the test sees it)."""
    inp = sip_state(mode, scheme=scheme)
    ref = _parity(inp, 1e-10, 2.2e-16)
    _, off = oracle_run(sip_state(mode, splinter=False, scheme=scheme))
    d = (ref["nicet"] - off["nicet"]).abs().max()
    assert float(d) > 1e-6 * float(ref["nicet"].abs().max())


def test_secondary_ice_all_processes_fp64_parity():
    """All processes with the three schemes on (the secondary_ice_sub fixture's setup)."""
    inp = sip_state(1, coag_only=False)
    for sw in (inp.cfg.lssipdropfrac, inp.cfg.lssipicecollbreak):
        sw.sw, sw.mode = 1, 1
    _parity(inp, 1e-10, 2.2e-16)


def test_secondary_ice_mixed_error_bound():
    inp = sip_state(1, coag_only=False)
    for sw in (inp.cfg.lssipdropfrac, inp.cfg.lssipicecollbreak):
        sw.sw, sw.mode = 1, 1
    inp.cfg.precision = 1
    _parity(inp, 1e-6, 1e-7)
