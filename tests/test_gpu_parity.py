"""GPU parity tests: the CUDA step (through the C-ABI) against the CPU oracle.

Criterion.  For every bin value of the new state x = x_old + tendency * dt:
    |x_gpu - x_oracle| <= max(RTOL * max(|x_oracle|, |x_old|, floor), C_ENV * envelope)
where `envelope` is the oracle's own response to the rounding differences between two
correct FP64 implementations of the path: one-ulp perturbations (both signs) of its
inputs (T, p, rv, rsi, every bin and the IN deficit), two-ulp changes of every result of
its library functions (exp, log, pow, ...: up, down, and four patterns taken from the
argument's bits), and multiply-add contraction (the same source built with contraction).
The reference's explicit, clamped condensation substep loop and its freezing
probabilities 1 - exp(-J dt) amplify such differences by many orders of magnitude
(tests/test_oracle.py), so no implementation that is not bit-identical, libm included,
can meet RTOL there.  Where a value is well conditioned the envelope is ~1e-16 of it and
the bound is RTOL; C_ENV = 100 covers the new ice of freezing drops in supersaturated
cells, whose difference reaches 10-50 times the envelope (relative 1e-9).
FP64 form: RTOL = 1e-10, no value may exceed the bound, and at least FRAC_WITHIN of
the values of every field lie within RTOL.  FP32-mixed form: RTOL = 1e-6 with the
envelope taken from float-sized (1e-7) input perturbations; up to VIOL_FRAC of the
values may exceed that bound.
"""
import pytest
import torch

from uclales_salsa_gb300.inputs import make_inputs, make_outputs
from uclales_salsa_gb300.api import SalsaStep
from uclales_salsa_gb300 import capi
from oracle_ref import Oracle
from parity import STATE_OF, NUMBER_FIELDS, FLOOR, floor_of, interior, output_errors

pytestmark = pytest.mark.gpu
C_ENV = 100.0
VIOL_FRAC = 1e-3
FRAC_WITHIN = 0.99
PERTURBED = ("temp", "press", "rp", "rsi", "maero", "naero", "mcloud", "ncloud", "mprecp", "nprecp", "mice", "nice",
             "indef")
LIBM_MODES = (1, -1, 2, 3, 4, 5)
CASES = [("grid16x16x40", {}), ("grid256x256x128", dict(X=8, Y=8, Z=16)), ("grid384x384x160", dict(X=16, Y=16, Z=12))]
# 131,072-cell blocks of the two large workloads
LARGE = [("grid256x256x128", dict(X=64, Y=64, Z=32)), ("grid384x384x160", dict(X=64, Y=64, Z=32))]
# a cell count that is not a multiple of the cells one block stages, and a single cell
RAGGED = [("grid256x256x128", dict(X=5, Y=3, Z=7)), ("grid384x384x160", dict(X=1, Y=1, Z=1))]


def oracle_run(inp, fields=None, scale=None, pert_eps=0.0, pert_field=None, libm=0, variant="plain"):
    f = {k: v.clone() for k, v in (fields or inp.fields).items()}
    if pert_field:
        f[pert_field] = f[pert_field] * (1 + pert_eps)
    out = make_outputs(inp)
    rc, st = Oracle(inp.cfg, variant=variant).run(inp, f, out, time=1.0, libm=libm)
    assert rc == 0, st.as_dict()
    return f, out


def gpu_run(inp, fields=None, host=False, diag=True):
    src = fields or inp.fields
    if host:
        f = {k: v.clone().pin_memory() for k, v in src.items()}
        out = {k: v.pin_memory() for k, v in make_outputs(inp, with_diag=diag).items()}
    else:
        f = {k: v.clone().cuda() for k, v in src.items()}
        out = {k: v.cuda() for k, v in make_outputs(inp, with_diag=diag).items()}
    step = SalsaStep(inp.cfg)
    rc, st = step.run(inp, f, out, time=1.0)
    torch.cuda.synchronize()
    assert rc == 0, st.as_dict()
    assert st.n_cells == inp.ncells
    step.close()
    return f, {k: v.cpu() for k, v in out.items()}


def envelope(inp, base, eps):
    """Largest change of each output under the perturbations of the module docstring;
    eps is the relative size of the input perturbations.  The library-function and
    contraction runs belong to the FP64 form only (eps at the FP64 epsilon)."""
    env = {k: torch.zeros_like(v) for k, v in base.items()}

    def add(o):
        for k in env:
            env[k] = torch.maximum(env[k], (o[k] - base[k]).abs())

    for pf in PERTURBED:
        if pf not in inp.fields:
            continue
        for sgn in (1.0, -1.0):
            add(oracle_run(inp, pert_eps=sgn * eps, pert_field=pf)[1])
    if eps < 1e-15:
        for mode in LIBM_MODES:
            add(oracle_run(inp, libm=mode)[1])
        add(oracle_run(inp, variant="contract")[1])
    return env


def check(inp, gpu, ref, env, rtol):
    report = {}
    for name, st in STATE_OF.items():
        if name not in ref:
            continue
        dt = inp.dt
        I = lambda t: interior(t, inp.nzp, inp.nxp, inp.nyp)
        old = I(inp.fields[st])
        a, b = old + I(gpu[name]) * dt, old + I(ref[name]) * dt
        e = I(env[name]) * dt
        fl = floor_of(name)
        scale = torch.maximum(b.abs(), old.abs()).clamp(min=fl)
        err = (a - b).abs()
        bound = torch.maximum(rtol * scale, C_ENV * e)
        rel = err / scale
        report[name] = dict(max_rel=float(rel.max()), frac_within=float((rel <= rtol).double().mean()),
                            violations=int((err > bound).sum()), n=rel.numel())
    return report


def assert_fp64(rep):
    for k, r in rep.items():
        assert r["violations"] == 0, (k, r)
        assert r["frac_within"] >= FRAC_WITHIN, (k, r)


def assert_mixed(rep):
    for k, r in rep.items():
        assert r["violations"] <= VIOL_FRAC * r["n"], (k, r)
        assert r["frac_within"] >= FRAC_WITHIN, (k, r)


@pytest.mark.parametrize("name,kw", CASES)
def test_fp64_parity(name, kw):
    inp = make_inputs(name, "cpu", precision=0, **kw)
    _, ref = oracle_run(inp)
    _, gpu = gpu_run(inp)
    env = envelope(inp, ref, 2.2e-16)
    rep = check(inp, gpu, ref, env, 1e-10)
    print(name, rep)
    assert_fp64(rep)


@pytest.mark.parametrize("name,kw", LARGE)
def test_fp64_parity_large_block(name, kw):
    """The FP64 criterion on 131,072-cell blocks of the two large workloads: every bin
    value within the bound; the per-field maximum error and the fraction within 1e-10
    are printed."""
    inp = make_inputs(name, "cpu", precision=0, **kw)
    _, ref = oracle_run(inp)
    _, gpu = gpu_run(inp)
    rep = check(inp, gpu, ref, envelope(inp, ref, 2.2e-16), 1e-10)
    for k, r in rep.items():
        print(f"{name} {k:8s} max rel {r['max_rel']:.3e}  within 1e-10 {100 * r['frac_within']:.4f} %  "
              f"beyond the bound {r['violations']} of {r['n']}")
    assert_fp64(rep)


@pytest.mark.parametrize("precision", [0, 1])
@pytest.mark.parametrize("name,kw", RAGGED)
def test_ragged_and_single_cell_blocks(name, kw, precision):
    """105 interior cells (the last block stages a partial group) and a single cell:
    every bin value within the bound of its form."""
    inp = make_inputs(name, "cpu", precision=precision, **kw)
    _, ref = oracle_run(inp)
    _, gpu = gpu_run(inp)
    eps, rtol = (2.2e-16, 1e-10) if precision == 0 else (1e-7, 1e-6)
    rep = check(inp, gpu, ref, envelope(inp, ref, eps), rtol)
    print(name, precision, rep)
    for k, r in rep.items():
        assert r["violations"] == 0, (k, r)


@pytest.mark.parametrize("name,kw", CASES)
def test_fp32_mixed_error_bound(name, kw):
    inp = make_inputs(name, "cpu", precision=1, **kw)
    _, ref = oracle_run(inp)
    _, gpu = gpu_run(inp)
    env = envelope(inp, ref, 1e-7)
    rep = check(inp, gpu, ref, env, 1e-6)
    print(name, rep)
    assert_mixed(rep)


def test_diagnostics_and_outputs_match():
    inp = make_inputs("grid384x384x160", "cpu", precision=0, X=12, Y=12, Z=8)
    _, ref = oracle_run(inp)
    _, gpu = gpu_run(inp)
    errs = output_errors(inp, gpu, ref)
    print(errs)
    for k, v in errs.items():
        assert v < 1e-6, (k, v)   # relative to the field's largest value
    assert float(gpu["pa_nactd"].abs().max()) == 0.0   # interstitial activation leaves them zero


def test_in_deficit_fraction_matches():
    inp = make_inputs("grid384x384x160", "cpu", precision=0, X=12, Y=12, Z=8)
    fr, _ = oracle_run(inp)
    fg, _ = gpu_run(inp)
    a, b = fg["indef"].cpu(), fr["indef"]
    assert float((a - b).abs().max()) < 1e-9


def test_host_and_device_pointers_agree():
    """Host arrays go through the slab pipeline (ragged last slab, more slabs than
    staging slots); the results equal the device-pointer call's, and values outside the
    interior cells (halo columns, levels 1 and nzp, halo rows) come back unchanged in
    every output, the outputs that are only written included."""
    inp = make_inputs("grid256x256x128", "cpu", precision=0, X=8, Y=21, Z=8)
    fh, oh = gpu_run(inp, host=True)
    fd, od = gpu_run(inp, host=False)
    for k in oh:
        assert torch.equal(oh[k], od[k]), k
    assert torch.equal(fh["indef"].cpu(), fd["indef"].cpu())
    g = torch.Generator().manual_seed(11)
    pre = {k: torch.rand(v.shape, generator=g, dtype=torch.float64) for k, v in make_outputs(inp).items()}
    res = {}
    for host in (True, False):
        f = {k: (v.clone().pin_memory() if host else v.clone().cuda()) for k, v in inp.fields.items()}
        out = {k: (v.clone().pin_memory() if host else v.clone().cuda()) for k, v in pre.items()}
        step = SalsaStep(inp.cfg)
        rc, st = step.run(inp, f, out, time=1.0)
        torch.cuda.synchronize()
        step.close()
        assert rc == 0
        res[host] = {k: v.cpu() for k, v in out.items()}
    for k in pre:
        assert torch.equal(res[True][k], res[False][k]), k
        m = torch.ones_like(pre[k], dtype=torch.bool)
        interior(m, inp.nzp, inp.nxp, inp.nyp).fill_(False)
        assert torch.equal(res[True][k][m], pre[k][m]), k


def test_deterministic_and_diagnostics_do_not_change_state():
    inp = make_inputs("grid384x384x160", "cpu", precision=0, X=12, Y=12, Z=8)
    _, a = gpu_run(inp)
    _, b = gpu_run(inp)
    for k in a:
        assert torch.equal(a[k], b[k]), k
    inp.cfg.diagnostics = 0
    _, c = gpu_run(inp, diag=False)
    for k in c:
        assert torch.equal(a[k], c[k]), k


def test_async_entry_on_caller_stream():
    inp = make_inputs("grid384x384x160", "cuda", precision=1, X=8, Y=8, Z=8)
    out = make_outputs(inp)
    step = SalsaStep(inp.cfg)
    s = torch.cuda.Stream()
    f = {k: v.clone() for k, v in inp.fields.items()}
    rc, st = step.run(inp, f, out, stream=s)
    s.synchronize()
    assert rc == 0 and st.n_cells == inp.ncells
    out2 = make_outputs(inp)
    f2 = {k: v.clone() for k, v in inp.fields.items()}
    step.run(inp, f2, out2)
    for k in out:
        assert torch.equal(out[k], out2[k]), k


def test_error_codes():
    import ctypes as C
    from uclales_salsa_gb300 import api
    inp = make_inputs("grid16x16x40", "cuda", X=4, Y=4, Z=4)
    step = SalsaStep(inp.cfg)
    out = make_outputs(inp)
    f = capi.make_fields(inp.fields, out)
    st = capi.Status()
    L = api.library()
    run = lambda *a: L.salsa_gb300_run(step.h, *a, C.byref(f), C.byref(st))
    assert run(inp.nzp, inp.nxp, inp.nyp, inp.ns, 1.0, 1.0, 1, 5, 0, 0) == capi.SALSA_E_ARG    # level mismatch
    assert run(inp.nzp, 4, inp.nyp, inp.ns, 1.0, 1.0, 1, 4, 0, 0) == capi.SALSA_E_ARG         # nxp < 5
    assert run(inp.nzp, inp.nxp, inp.nyp, inp.ns, 1e4, 1.0, 1, 4, 0, 0) == capi.SALSA_E_ARG   # tstep bound
    assert run(inp.nzp, inp.nxp, inp.nyp, 2, 1.0, 1.0, 1, 4, 0, 0) == capi.SALSA_E_ARG        # ns < nwet
    assert run(inp.nzp, inp.nxp, inp.nyp, inp.ns, 1.0, 1.0, 1, 4, 1, 0) == capi.SALSA_E_ARG   # lcharge w/o array
    f.press = capi.ptr_of(0)
    assert run(inp.nzp, inp.nxp, inp.nyp, inp.ns, 1.0, 1.0, 1, 4, 0, 0) == capi.SALSA_E_ARG   # NULL input
    cfg = inp.cfg
    cfg.nsnucl = 4          # ternary nucleation STOPs in the reference
    h = C.c_void_p()
    assert L.salsa_gb300_init(C.byref(cfg), C.byref(h)) == capi.SALSA_E_UNSUPPORTED
    cfg.nsnucl = 0
    cfg.lscndgas = 1        # gas condensation needs the gas tendency array
    f.press = capi.ptr_of(inp.fields["press"].data_ptr())
    f.gaerot = capi.ptr_of(0)
    g = SalsaStep(cfg)
    assert L.salsa_gb300_run(g.h, inp.nzp, inp.nxp, inp.nyp, inp.ns, 1.0, 1.0, 1, 4, 0, 0, C.byref(f),
                             C.byref(st)) == capi.SALSA_E_ARG
    g.close()


def test_full_size_invariants():
    """256x256x128 (8.4M cells): finite, non-negative state and a closed water budget
    for condensation + activation (size-independent properties of the step)."""
    inp = make_inputs("grid256x256x128", "cuda", precision=0, diagnostics=0)
    inp.cfg.lscoag.sw = 0
    inp.cfg.lsicenucl.sw = 0
    out = make_outputs(inp, with_diag=False)
    step = SalsaStep(inp.cfg)
    f = {k: v.clone() for k, v in inp.fields.items()}
    rc, st = step.run(inp, f, out, time=1.0)
    torch.cuda.synchronize()
    assert rc == 0 and st.n_cells == inp.ncells and st.n_nonfinite == 0
    lay, dt = inp.layout, inp.dt
    I = lambda t: interior(t, inp.nzp, inp.nxp, inp.nyp)
    for name, s in STATE_OF.items():
        if name in out:
            new = I(inp.fields[s]) + I(out[name]) * dt
            assert bool(torch.isfinite(new).all()), name
            fl = floor_of(name)
            assert float(new.min()) > -1e-12 * (float(I(inp.fields[s]).abs().max()) + fl), name
    dn, T, p = I(inp.fields["dn"]), I(inp.fields["temp"]), I(inp.fields["press"])
    rhoair = 28.97e-3 * p / (8.314 * T)
    iw = lay.nwet - 1
    dm = torch.zeros_like(dn)
    for t, nb in (("maerot", lay.nbins), ("mcloudt", lay.ncld), ("mprecpt", lay.nprc)):
        dm += I(out[t])[iw * nb:(iw + 1) * nb].sum(0) * dn
    dm += I(out["micet"])[iw * lay.nice:(iw + 2) * lay.nice].sum(0) * dn
    dv = I(out["rpt"]) * rhoair
    total = I(inp.fields["rp"]) * rhoair / dt
    assert float(((dm + dv).abs() / total).max()) < 1e-9
