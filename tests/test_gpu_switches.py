"""Process-switch delays on the GPU (set_SALSA_runtime, mo_salsa_driver.f90:453-466).

A handle keeps the switch states as the reference keeps them: a master switch takes
effect once time >= delay and then stays on, also for a later call at an earlier time.
A delayed coagulation therefore gives, bit for bit, the handle's step without
coagulation before its delay and the step with it from then on (the oracle's own
sequence is checked in tests/test_oracle.py; both steps are checked against the
oracle in tests/test_gpu_parity.py and tests/test_gpu_variants.py).
"""
import pytest
import torch

from uclales_salsa_gb300.inputs import make_inputs, make_outputs
from uclales_salsa_gb300.api import SalsaStep

pytestmark = pytest.mark.gpu


def _gpu(step, inp, time):
    f = {k: v.clone().cuda() for k, v in inp.fields.items()}
    out = {k: v.cuda() for k, v in make_outputs(inp).items()}
    rc, st = step.run(inp, f, out, time=time)
    torch.cuda.synchronize()
    assert rc == 0, st.as_dict()
    return {k: v.cpu() for k, v in out.items()}


def _same(a, b):
    return all(torch.equal(a[k], b[k]) for k in a)


def test_delayed_coagulation_switches_on_at_its_delay_and_stays_on():
    inp = make_inputs("grid256x256x128", "cpu", precision=0, X=8, Y=8, Z=8)
    inp.cfg.lscoag.sw = 0
    s = SalsaStep(inp.cfg)
    no_coag = _gpu(s, inp, 1.0)
    s.close()
    inp.cfg.lscoag.sw, inp.cfg.lscoag.delay = 1, 0.0
    s = SalsaStep(inp.cfg)
    with_coag = _gpu(s, inp, 1.0)
    s.close()
    assert not _same(no_coag, with_coag)
    inp.cfg.lscoag.delay = 5.0
    s = SalsaStep(inp.cfg)
    for time, expect in ((1.0, no_coag), (4.999, no_coag), (5.0, with_coag), (2.0, with_coag)):
        assert _same(_gpu(s, inp, time), expect), time
    s.close()
