"""The LES-side constraints after a step (tend_constrain2 + SALSA_diagnostics) on a
block of a workload, resident on the GPU (for timing and profiling).

    python -m uclales_salsa_gb300.post_case --workload grid256x256x128 --X 128 --Y 128 --Z 64 --reps 3

Runs one SALSA step to obtain tendencies, then times `reps` calls of each routine with
CUDA events on one stream and prints their device times and the bytes each call reads
and writes at least once (the values and tendencies it must inspect).
"""
import argparse
import json

import torch

from .api import SalsaStep
from .inputs import make_inputs, make_outputs

TRACERS = [("naero", "naerot"), ("maero", "maerot"), ("ncloud", "ncloudt"), ("mcloud", "mcloudt"),
           ("nprecp", "nprecpt"), ("mprecp", "mprecpt"), ("nice", "nicet"), ("mice", "micet")]


def post_arrays(inp, fields, outs):
    """PostFields arrays from the fields and tendencies of a step (device tensors)."""
    a = {}
    for v, t in TRACERS:
        if v in fields and t in outs:
            a[v], a[t] = fields[v], outs[t]
    if "indef" in fields:
        a["indef"] = fields["indef"]
    a["rh"] = fields["rp"] / fields["rsl"]
    if "rsi" in fields:
        a["rhi"] = fields["rp"] / fields["rsi"]
    a["temp"], a["rp"] = fields["temp"], fields["rp"]
    names = ("rc", "srp", "snrp", "rtot") + (("ri", "riri") if inp.level == 5 else ())
    for d in names:
        a[d] = torch.zeros_like(fields["press"])
    return a


def post_bytes(a, level):
    """Bytes each routine reads or writes at least once per call."""
    b = lambda k: a[k].numel() * 8 if k in a else 0
    tc = sum(b(v) + b(t) for v, t in TRACERS) + b("indef")
    dg = sum(b(v) for v, _ in TRACERS) + b("rh") + b("temp") + b("rp") + (b("rhi") if level == 5 else 0)
    dg += sum(b(d) for d in ("rc", "srp", "snrp", "rtot", "ri", "riri"))
    return tc, dg


def time_post(step, inp, a, stream, reps):
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(3)]
    with torch.cuda.stream(stream):
        step.tend_constrain(inp.nzp, inp.nxp, inp.nyp, inp.dt, a, stream=stream)     # warm-up
        step.diagnostics(inp.nzp, inp.nxp, inp.nyp, a, stream=stream)
        ev[0].record(stream)
        for _ in range(reps):
            step.tend_constrain(inp.nzp, inp.nxp, inp.nyp, inp.dt, a, stream=stream)
        ev[1].record(stream)
        for _ in range(reps):
            step.diagnostics(inp.nzp, inp.nxp, inp.nyp, a, stream=stream)
        ev[2].record(stream)
    torch.cuda.synchronize()
    return ev[0].elapsed_time(ev[1]) / reps, ev[1].elapsed_time(ev[2]) / reps


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--workload", default="grid256x256x128")
    ap.add_argument("--X", type=int)
    ap.add_argument("--Y", type=int)
    ap.add_argument("--Z", type=int)
    ap.add_argument("--reps", type=int, default=3)
    a_ = ap.parse_args()
    inp = make_inputs(a_.workload, "cuda", X=a_.X, Y=a_.Y, Z=a_.Z, diagnostics=0)
    step = SalsaStep(inp.cfg)
    fields = {k: v.clone() for k, v in inp.fields.items()}
    outs = make_outputs(inp, with_diag=False)
    step.run(inp, fields, outs, time=1.0)
    a = post_arrays(inp, fields, outs)
    s = torch.cuda.Stream()
    tc_ms, dg_ms = time_post(step, inp, a, s, a_.reps)
    tcb, dgb = post_bytes(a, inp.level)
    print(json.dumps({"workload": a_.workload, "points": inp.nzp * inp.nxp * inp.nyp,
                      "tend_constrain_ms": tc_ms, "diagnostics_ms": dg_ms,
                      "tend_constrain_gbs": tcb / tc_ms / 1e6, "diagnostics_gbs": dgb / dg_ms / 1e6}))
    step.close()


if __name__ == "__main__":
    main()
