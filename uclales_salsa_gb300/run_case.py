"""Run the SALSA step on a synthetic workload (used for profiling and quick checks).

    python -m uclales_salsa_gb300.run_case --workload grid384x384x160 --X 64 --Y 64 --Z 32 \
        --precision 0 --steps 2 [--cgintvl 10]
"""
import argparse
import json

import torch

from .api import SalsaStep
from .inputs import make_inputs, make_outputs


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--workload", default="grid384x384x160")
    ap.add_argument("--X", type=int)
    ap.add_argument("--Y", type=int)
    ap.add_argument("--Z", type=int)
    ap.add_argument("--precision", type=int, default=0)
    ap.add_argument("--diagnostics", type=int, default=1)
    ap.add_argument("--steps", type=int, default=2)
    ap.add_argument("--cgintvl", type=float, default=0.,
                    help="> 0: low-frequency kernels (lscoag mode 2) updated every cgintvl s; step k runs at time k")
    a = ap.parse_args()
    inp = make_inputs(a.workload, "cuda", X=a.X, Y=a.Y, Z=a.Z, precision=a.precision, diagnostics=a.diagnostics)
    if a.cgintvl > 0:
        inp.cfg.lscoag.mode, inp.cfg.cgintvl = 2, a.cgintvl
    step = SalsaStep(inp.cfg)
    outs = make_outputs(inp)
    res = []
    for k in range(a.steps):
        f = {k_: v.clone() for k_, v in inp.fields.items()}
        rc, st = step.run(inp, f, outs, time=float(k + 1), istp=k + 1)
        res.append(dict(rc=rc, kernel_ms=step.last_kernel_ms(), **st.as_dict()))
    torch.cuda.synchronize()
    print(json.dumps({"workload": a.workload, "cells": inp.ncells, "precision": a.precision, "runs": res}))


if __name__ == "__main__":
    main()
