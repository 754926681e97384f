"""salsa_gb300_run_noalloc: the step for callers that cannot allocate GPU memory.

An LES that hands its GPU memory to its own pool, or whose time loop cannot take
the synchronisation of cudaMalloc, calls this entry point; it keeps its scratch in
a static device array of the library instead of allocating.  Two calls in a row on
the same inputs must reproduce salsa_gb300_run_async bit for bit (outputs,
in-place IN deficit and status counts); the second call checks that the counters
and the order list left by the first call do not leak into it.  A call on a fresh
handle, over a larger grid than any call before it, must leave the device's free
memory unchanged.  The file is collected last so that it also runs after every
other GPU test in one session.
"""
import ctypes as C

import pytest
import torch

from uclales_salsa_gb300 import api, capi
from uclales_salsa_gb300.inputs import make_inputs, make_outputs

pytestmark = pytest.mark.gpu


def _call(fn, step, inp, fields, out, stream):
    f = capi.make_fields(fields, out)
    st = capi.Status()
    rc = fn(step.h, inp.nzp, inp.nxp, inp.nyp, inp.ns, inp.dt, 1.0, 1, inp.level, 0, 0, C.byref(f),
            C.c_void_p(stream.cuda_stream), 1, C.byref(st))
    return rc, st


def test_noalloc_matches_run_async_on_two_calls():
    L = api.library()
    L.salsa_gb300_run_noalloc.argtypes = L.salsa_gb300_run_async.argtypes
    L.salsa_gb300_run_noalloc.restype = C.c_int
    inp = make_inputs("grid384x384x160", "cuda", precision=0, X=24, Y=24, Z=16)
    stream = torch.cuda.Stream()
    res = {}
    for name, fn in (("async", L.salsa_gb300_run_async), ("noalloc", L.salsa_gb300_run_noalloc)):
        step = api.SalsaStep(inp.cfg)
        runs = []
        for _ in range(2):
            f = {k: v.clone() for k, v in inp.fields.items()}
            out = make_outputs(inp)
            rc, st = _call(fn, step, inp, f, out, stream)
            stream.synchronize()
            assert rc == 0, (name, rc, st.as_dict())
            runs.append((out, f["indef"], st.as_dict()))
        step.close()
        res[name] = runs
    for i in range(2):
        oa, ia, sa = res["async"][i]
        on, ina, sn = res["noalloc"][i]
        for k in oa:
            assert torch.equal(oa[k], on[k]), (i, k)
        assert torch.equal(ia, ina)
        assert sa == sn and sn["n_cells"] == inp.ncells


def test_noalloc_rejects_grids_beyond_its_scratch():
    L = api.library()
    L.salsa_gb300_run_noalloc.argtypes = L.salsa_gb300_run_async.argtypes
    L.salsa_gb300_run_noalloc.restype = C.c_int
    inp = make_inputs("grid16x16x40", "cuda", X=4, Y=4, Z=4)
    step = api.SalsaStep(inp.cfg)
    out = make_outputs(inp)
    f = capi.make_fields(inp.fields, out)
    st = capi.Status()
    stream = torch.cuda.Stream()
    big = 2097152 // (4 * 4) + 8     # interior cells = 4 * 4 * (nzp - 2) > SALSA_NOALLOC_MAXCELLS
    rc = L.salsa_gb300_run_noalloc(step.h, big + 2, inp.nxp, inp.nyp, inp.ns, inp.dt, 1.0, 1, inp.level, 0, 0,
                                   C.byref(f), C.c_void_p(stream.cuda_stream), 1, C.byref(st))
    assert rc == capi.SALSA_E_ARG
    step.close()


def test_noalloc_call_leaves_free_device_memory_unchanged():
    """The property the entry point exists for: after the handle is made (init loads
    the kernels and resolves the module scratch), a call takes no device memory, even
    on a grid larger than any earlier call's.  Any cudaMalloc would move the free
    memory by at least one 2 MiB page."""
    L = api.library()
    L.salsa_gb300_run_noalloc.argtypes = L.salsa_gb300_run_async.argtypes
    L.salsa_gb300_run_noalloc.restype = C.c_int
    stream = torch.cuda.Stream()
    small = make_inputs("grid384x384x160", "cuda", precision=0, X=8, Y=8, Z=8)
    step = api.SalsaStep(small.cfg)
    rc, st = _call(L.salsa_gb300_run_noalloc, step, small, {k: v.clone() for k, v in small.fields.items()},
                   make_outputs(small), stream)
    stream.synchronize()
    assert rc == 0, st.as_dict()
    step.close()
    inp = make_inputs("grid384x384x160", "cuda", precision=0, X=48, Y=48, Z=20)
    f = {k: v.clone() for k, v in inp.fields.items()}
    out = make_outputs(inp)
    fresh = api.SalsaStep(inp.cfg)
    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info()[0]
    rc, st = _call(L.salsa_gb300_run_noalloc, fresh, inp, f, out, stream)
    stream.synchronize()
    free1 = torch.cuda.mem_get_info()[0]
    assert rc == 0 and st.as_dict()["n_cells"] == inp.ncells, st.as_dict()
    assert free1 == free0, (free0, free1)
    fresh.close()


def test_noalloc_refuses_the_low_frequency_kernel_storage():
    """lscoag mode 2 keeps one kernel triangle per cell in memory the library must
    allocate, so the no-alloc step answers SALSA_E_UNSUPPORTED for it."""
    L = api.library()
    L.salsa_gb300_run_noalloc.argtypes = L.salsa_gb300_run_async.argtypes
    L.salsa_gb300_run_noalloc.restype = C.c_int
    inp = make_inputs("grid16x16x40", "cuda", X=4, Y=4, Z=4)
    inp.cfg.lscoag.mode, inp.cfg.cgintvl = 2, 10.0
    step = api.SalsaStep(inp.cfg)
    stream = torch.cuda.Stream()
    rc, _ = _call(L.salsa_gb300_run_noalloc, step, inp, {k: v.clone() for k, v in inp.fields.items()},
                  make_outputs(inp), stream)
    assert rc == capi.SALSA_E_UNSUPPORTED
    step.close()
