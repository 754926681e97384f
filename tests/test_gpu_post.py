"""tend_constrain2 and SALSA_diagnostics on the GPU (salsa_gb300_tend_constrain,
salsa_gb300_diagnostics) against the oracle on the same post-step states.  The
arithmetic is the same operation for operation; only pow(x, 1/3) comes from two
libraries, so every array must agree to the last bit outside a rare branch flip."""
import pytest
import torch

from uclales_salsa_gb300.api import SalsaStep
from oracle_ref import Oracle
from post_cases import post_state

pytestmark = pytest.mark.gpu
CASES = [("grid16x16x40", dict(X=8, Y=8, Z=16)), ("grid256x256x128", dict(X=8, Y=8, Z=16)),
         ("grid384x384x160", dict(X=12, Y=12, Z=8))]


def _compare(a, b):
    bad = {}
    for k in a:
        x, y = a[k], b[k].cpu()
        n = int((x != y).sum())
        if n:
            bad[k] = n
    return bad


@pytest.mark.parametrize("wl,kw", CASES, ids=[c[0] for c in CASES])
@pytest.mark.parametrize("lcharge,dtlt", [(0, None), (1, 0.7)])
def test_post_step_matches_oracle(wl, kw, lcharge, dtlt):
    inp, a = post_state(wl, **kw)
    if lcharge:
        g = torch.Generator().manual_seed(8)
        lay = inp.layout
        a["chargeTime"] = torch.rand((lay.nbins + lay.ncld + lay.nprc,) + tuple(a["rp"].shape), generator=g,
                                     dtype=torch.float64)
    dtlt = dtlt or inp.dt          # a power of two (product path) and a general step (quotient path)
    ref = {k: v.clone() for k, v in a.items()}
    o = Oracle(inp.cfg)
    assert o.tend_constrain(inp.nzp, inp.nxp, inp.nyp, dtlt, ref) == 0
    assert o.diagnostics(inp.nzp, inp.nxp, inp.nyp, ref, lcharge=lcharge) == 0
    dev = {k: v.clone().cuda() for k, v in a.items()}
    step = SalsaStep(inp.cfg)
    step.tend_constrain(inp.nzp, inp.nxp, inp.nyp, dtlt, dev)
    step.diagnostics(inp.nzp, inp.nxp, inp.nyp, dev, lcharge=lcharge)
    torch.cuda.synchronize()
    step.close()
    bad = _compare(ref, dev)
    n = sum(v.numel() for v in ref.values())
    assert sum(bad.values()) <= 1e-6 * n, bad
    changed = sum(int((ref[k] != a[k]).sum()) for k in ref)
    assert changed > 1000     # the cases do exercise the repairs


def test_only_diag_and_errors():
    inp, a = post_state("grid256x256x128", X=6, Y=6, Z=6)
    ref = {k: v.clone() for k, v in a.items()}
    assert Oracle(inp.cfg).diagnostics(inp.nzp, inp.nxp, inp.nyp, ref, only_diag=1) == 0
    dev = {k: v.clone().cuda() for k, v in a.items()}
    step = SalsaStep(inp.cfg)
    step.diagnostics(inp.nzp, inp.nxp, inp.nyp, dev, only_diag=1)
    torch.cuda.synchronize()
    assert _compare(ref, dev) == {}
    with pytest.raises(Exception):   # host arrays are refused
        step.diagnostics(inp.nzp, inp.nxp, inp.nyp, a)
    step.close()
