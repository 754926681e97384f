"""GPU parity of the step's less common paths (FP64 form against the oracle).

Each case changes one part of the configuration or of the call on a small block of
a workload: the classic ice nucleation (mo_salsa_cloud_ice.f90:26-140), every SE
freezing mode, ice melting (mo_salsa_cloud_ice.f90:393-462), the second
autoconversion mode (mo_salsa_cloud.f90 autoconv2), the charging enhancement of the
collision kernels (mo_salsa_coagulation_kernels.f90:411-416), the initialising call
(run_SALSA with initialize=.TRUE.), a step without coagulation, gas condensation with
nucleation switched on (mo_salsa_dynamics.f90:276-685) and cloud-base activation
(mo_salsa_cloud.f90:161-375, 1199-1378), the last two at levels 5 and 4.  The
activated-droplet outputs are checked as well.  The criterion is
the one of test_gpu_parity.py.
"""
import pytest
import torch

from uclales_salsa_gb300.inputs import make_inputs, make_outputs
from uclales_salsa_gb300.api import SalsaStep
from oracle_ref import Oracle
from test_gpu_parity import check, assert_fp64, VIOL_FRAC, FRAC_WITHIN, PERTURBED, LIBM_MODES
from parity import FLOOR, interior

pytestmark = pytest.mark.gpu


def _classic_ice(inp, f):
    c = inp.cfg
    c.ice_theta_dist = 0
    c.lsicehom = c.lsiceimm = c.lsicedep = 1


def _se_all_modes(inp, f):
    c = inp.cfg
    c.lsicehom = c.lsiceimm = c.lsicedep = 1


def _melting(inp, f):
    f["temp"] += 12.0          # part of the ice now sits above 273.15 K
    inp.cfg.lsicemelt.sw = 1


def _autoconv2(inp, f):
    inp.cfg.lsauto.mode = 2


def _no_coag(inp, f):
    inp.cfg.lscoag.sw = 0


def _nucleation(inp, f):
    inp.cfg.nsnucl = 1     # binary nucleation; gas condensation comes with the gas fields


def _cloudbase(inp, f):
    inp.cfg.lsactiv.mode = 2


def _charge(inp, f):
    lay = inp.layout
    g = torch.Generator().manual_seed(5)
    shp = (lay.nbins + lay.ncld + lay.nprc,) + tuple(f["press"].shape)
    f["chargeTime"] = torch.rand(shp, generator=g, dtype=torch.float64) * inp.cfg.chargeTMax
    inp.cfg.chargeCollEnh = 2.0   # the default 0 would switch the enhancement off


CASES = [
    ("classic_ice", "grid384x384x160", dict(X=12, Y=12, Z=8), _classic_ice, {}),
    ("se_all_modes", "grid384x384x160", dict(X=12, Y=12, Z=8), _se_all_modes, {}),
    ("melting", "grid384x384x160", dict(X=12, Y=12, Z=8), _melting, {}),
    ("autoconv2", "grid256x256x128", dict(X=8, Y=8, Z=16), _autoconv2, {}),
    ("no_coagulation", "grid256x256x128", dict(X=8, Y=8, Z=16), _no_coag, {}),
    ("charge", "grid256x256x128", dict(X=8, Y=8, Z=16), _charge, dict(lcharge=1)),
    ("initialize", "grid16x16x40", dict(X=8, Y=8, Z=16), lambda inp, f: None, dict(initialize=1)),
    ("gas_condensation", "grid256x256x128", dict(X=8, Y=8, Z=16, gases=True), _nucleation, {}),
    ("gas_condensation_level4", "grid16x16x40", dict(X=8, Y=8, Z=16, gases=True), _nucleation, {}),
    ("cloudbase_activation", "grid384x384x160", dict(X=12, Y=12, Z=8), _cloudbase, {}),
    ("cloudbase_activation_level4", "grid16x16x40", dict(X=8, Y=8, Z=16), _cloudbase, {}),
]


def check_activation(inp, gpu, ref, env, rtol):
    """The activated-droplet outputs (per kg of air) under the criterion of check()."""
    rep = {}
    I = lambda t: interior(t, inp.nzp, inp.nxp, inp.nyp)
    for k, fl in (("pa_nactd", FLOOR["n"]), ("pa_vactd", FLOOR["m"])):
        a, b, e = I(gpu[k]), I(ref[k]), I(env[k])
        scale = b.abs().clamp(min=fl)
        err = (a - b).abs()
        rel = err / scale
        rep[k] = dict(max_rel=float(rel.max()), frac_within=float((rel <= rtol).double().mean()),
                      violations=int((err > torch.maximum(rtol * scale, 10.0 * e)).sum()), n=rel.numel())
    return rep


def _oracle(inp, fields, kw, pf=None, eps=0.0, libm=0, variant="plain"):
    f = {k: v.clone() for k, v in fields.items()}
    if pf:
        f[pf] = f[pf] * (1 + eps)
    out = make_outputs(inp)
    rc, st = Oracle(inp.cfg, variant=variant).run(inp, f, out, time=1.0, libm=libm, **kw)
    assert rc == 0, st.as_dict()
    return out


@pytest.mark.parametrize("name,wl,kw,mod,call", CASES, ids=[c[0] for c in CASES])
def test_variant_parity(name, wl, kw, mod, call):
    inp = make_inputs(wl, "cpu", precision=0, **kw)
    fields = {k: v.clone() for k, v in inp.fields.items()}
    mod(inp, fields)
    inp.fields = fields
    ref = _oracle(inp, fields, call)
    env = {k: torch.zeros_like(v) for k, v in ref.items()}
    runs = [dict(pf=pf, eps=sgn * 2.2e-16) for pf in PERTURBED if pf in fields for sgn in (1.0, -1.0)]
    runs += [dict(libm=m) for m in LIBM_MODES] + [dict(variant="contract")]
    for r in runs:
        o = _oracle(inp, fields, call, **r)
        for k in env:
            env[k] = torch.maximum(env[k], (o[k] - ref[k]).abs())
    f = {k: v.clone().cuda() for k, v in fields.items()}
    out = {k: v.cuda() for k, v in make_outputs(inp).items()}
    step = SalsaStep(inp.cfg)
    rc, st = step.run(inp, f, out, time=1.0, **call)
    torch.cuda.synchronize()
    assert rc == 0, (name, st.as_dict())
    gpu = {k: v.cpu() for k, v in out.items()}
    step.close()
    rep = check(inp, gpu, ref, env, 1e-10)
    rep.update(check_activation(inp, gpu, ref, env, 1e-10))
    print(name, rep)
    assert_fp64(rep)


@pytest.mark.parametrize("host", [False, True])
def test_low_frequency_kernels(host):
    """lscoag%mode = 2 over three steps (update, fetch with a changed state, update at a
    multiple of cgintvl) against the oracle; with host arrays the slabs address the
    storage by their first cell."""
    inp = make_inputs("grid256x256x128", "cpu", precision=0, X=8, Y=8, Z=16)
    inp.cfg.lscoag.mode, inp.cfg.cgintvl = 2, 10.
    o = Oracle(inp.cfg)
    step = SalsaStep(inp.cfg)
    fields = {k: v.clone() for k, v in inp.fields.items()}
    fields0 = {k: v.clone() for k, v in inp.fields.items()}    # the state the first (update) step stores
    for time, istp in ((1.0, 1), (2.0, 2), (10.0, 10)):
        ref = make_outputs(inp)
        rc, _ = o.run(inp, {k: v.clone() for k, v in fields.items()}, ref, time=time, istp=istp)
        assert rc == 0
        env = {k: torch.zeros_like(v) for k, v in ref.items()}
        for pf in PERTURBED:
            for sgn in (1.0, -1.0):
                f2 = {k: v.clone() for k, v in fields.items()}
                f2[pf] = f2[pf] * (1 + sgn * 2.2e-16)
                o2 = Oracle(inp.cfg)       # same storage state: replay the update step first
                if istp > 1:
                    warm = make_outputs(inp)
                    o2.run(inp, {k: v.clone() for k, v in fields0.items()}, warm, time=1.0, istp=1)
                out2 = make_outputs(inp)
                o2.run(inp, f2, out2, time=time, istp=istp)
                for k in env:
                    env[k] = torch.maximum(env[k], (out2[k] - ref[k]).abs())
        if host:
            f = {k: v.clone().pin_memory() for k, v in fields.items()}
            out = {k: v.pin_memory() for k, v in make_outputs(inp).items()}
        else:
            f = {k: v.clone().cuda() for k, v in fields.items()}
            out = {k: v.cuda() for k, v in make_outputs(inp).items()}
        rc, st = step.run(inp, f, out, time=time, istp=istp)
        torch.cuda.synchronize()
        assert rc == 0
        inp.fields = fields
        rep = check(inp, {k: v.cpu() for k, v in out.items()}, ref, env, 1e-10)
        for k, r in rep.items():
            assert r["violations"] <= VIOL_FRAC * r["n"], (time, k, r)
            assert r["frac_within"] >= FRAC_WITHIN, (time, k, r)
        # the next step starts from the new state
        for t, v in (("naerot", "naero"), ("ncloudt", "ncloud"), ("nprecpt", "nprecp"), ("nicet", "nice"),
                     ("maerot", "maero"), ("mcloudt", "mcloud"), ("mprecpt", "mprecp"), ("micet", "mice")):
            fields[v] = (fields[v] + ref[t] * inp.dt).clamp(min=0)
    step.close()
