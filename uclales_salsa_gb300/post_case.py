"""The LES-side routines around a step (tend_constrain2, SALSA_diagnostics and the
bin sedimentation sedim_SALSA) on a block of a workload, resident on the GPU (for
timing and profiling).

    python -m uclales_salsa_gb300.post_case --workload grid256x256x128 --X 128 --Y 128 --Z 64 --reps 3

Runs one SALSA step to obtain tendencies, then times `reps` calls of each routine with
CUDA events on one stream and prints their device times and the bytes each call reads
and writes at least once (the values and tendencies it must inspect).  The
sedimentation runs with all four parts on, level thickness 20 m, friction velocity
0.3 m/s and dtlt = the step length.
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


SEDIM_PARTS = [("naero", "maero", "naerot", "maerot"), ("ncloud", "mcloud", "ncloudt", "mcloudt"),
               ("nprecp", "mprecp", "nprecpt", "mprecpt"), ("nice", "mice", "nicet", "micet")]


def sedim_arrays(inp, fields, outs, dz=20.0, ustar=0.3):
    """SedimFields arrays from the fields and tendencies of a step (device tensors)."""
    a = {}
    for n, m, nt, mt in SEDIM_PARTS:
        if n in fields and nt in outs:
            a[n], a[m], a[nt], a[mt] = fields[n], fields[m], outs[nt], outs[mt]
    t, p = fields["temp"], fields["press"]
    tk = torch.where(t > 0, t, torch.full_like(t, 280.0))
    pr = torch.where(p > 0, p, torch.full_like(p, 9.0e4))
    a["tk"] = tk
    a["adn"] = pr / (287.04 * tk)
    a["th"] = tk * (1.0e5 / pr) ** (287.04 / 1005.0)
    a["ustar"] = torch.full((inp.nyp, inp.nxp), ustar, dtype=torch.float64, device=t.device)
    a["dzt"] = torch.full((inp.nzp,), 1.0 / dz, dtype=torch.float64, device=t.device)
    a["tlt"] = torch.zeros_like(t)
    for k in ("rrate", "irate"):
        a[k] = torch.zeros_like(t)
    for k in ("sfcrrate", "sfcirate"):
        a[k] = torch.zeros_like(a["ustar"])
    lay = inp.layout
    a["VtPrc"] = torch.zeros((lay.nprc,) + tuple(t.shape), dtype=torch.float64, device=t.device)
    if inp.level == 5:
        a["VtIce"] = torch.zeros((lay.nice,) + tuple(t.shape), dtype=torch.float64, device=t.device)
    return a


def sedim_bytes(a):
    """Bytes sedim_SALSA reads or writes at least once per call: the bin values, the
    tendencies (read and written), tk, th, adn, tlt (read and written), the rates and
    the fall speeds."""
    b = lambda k: a[k].numel() * 8 if k in a else 0
    tot = 0
    for n, m, nt, mt in SEDIM_PARTS:
        tot += b(n) + b(m) + 2 * (b(nt) + b(mt))
    tot += b("tk") + b("th") + b("adn") + 2 * b("tlt") + b("rrate") + b("irate") + b("VtPrc") + b("VtIce")
    return tot


def time_sedim(step, inp, a, stream, reps, sed=(1, 1, 1, 1)):
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
    with torch.cuda.stream(stream):
        step.sedimentation(inp.nzp, inp.nxp, inp.nyp, inp.dt, sed, a, stream=stream)     # warm-up
        ev[0].record(stream)
        for _ in range(reps):
            step.sedimentation(inp.nzp, inp.nxp, inp.nyp, inp.dt, sed, a, stream=stream)
        ev[1].record(stream)
    torch.cuda.synchronize()
    return ev[0].elapsed_time(ev[1]) / reps


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
    sa = sedim_arrays(inp, fields, outs)
    sd_ms = time_sedim(step, inp, sa, s, a_.reps)
    sdb = sedim_bytes(sa)
    print(json.dumps({"workload": a_.workload, "points": inp.nzp * inp.nxp * inp.nyp,
                      "tend_constrain_ms": tc_ms, "diagnostics_ms": dg_ms, "sedimentation_ms": sd_ms,
                      "tend_constrain_gbs": tcb / tc_ms / 1e6, "diagnostics_gbs": dgb / dg_ms / 1e6,
                      "sedimentation_gbs": sdb / sd_ms / 1e6}))
    step.close()


if __name__ == "__main__":
    main()
