"""One forward + adjoint run of the gradient harness (for profiling and timing).

    python -m uclales_salsa_gb300.chain_case --cells 16384 --steps 10

Builds `cells` cells of the chain65536 workload, runs the forward chain with a
checkpoint every step and the adjoint of the final cloud numbers and masses, and
prints the two device times.
"""
import argparse
import json

import torch

from .inputs import make_inputs
from .chain import SalsaChain, chain_config, pack_state


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--cells", type=int, default=16384)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--ckpt-every", type=int, default=1)
    a = ap.parse_args()
    inp = make_inputs("chain65536", "cuda", X=1, Y=1, Z=a.cells)
    inp.cfg = chain_config()
    x, th, k, s = pack_state(inp)
    ch = SalsaChain(inp.cfg)
    lay = inp.layout
    nl = lay.nbins + lay.ncld + lay.nprc
    yb = torch.zeros_like(x)
    for b in range(lay.nbins, lay.nbins + lay.ncld):
        yb[:, b] = 1.0
        for sp in range(lay.nwet):
            yb[:, nl + sp * nl + b] = 1.0
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(3)]
    ev[0].record()
    xN, ck = ch.forward(x, th, k, s, a.steps, inp.dt, ckpt_every=a.ckpt_every)
    ev[1].record()
    xb, kb, sb = ch.adjoint(ck, a.ckpt_every, th, k, s, a.steps, inp.dt, yb / xN.abs().clamp(min=1e-30))
    ev[2].record()
    torch.cuda.synchronize()
    print(json.dumps({"cells": a.cells, "steps": a.steps, "forward_ms": ev[0].elapsed_time(ev[1]),
                      "adjoint_ms": ev[1].elapsed_time(ev[2]),
                      "finite": bool(torch.isfinite(xb).all() and torch.isfinite(kb).all() and torch.isfinite(sb).all())}))
    ch.close()


if __name__ == "__main__":
    main()
