"""Per-stage clock breakdown of the SALSA step.

Builds an instrumented copy of the library (-DSALSA_STAGE_TIMERS: every warp adds
clock64() deltas of the process stages of its cell to a device counter array) into
_build/stages/, runs one step of each form on a block of the workloads and prints
each stage's share.  With --chain it runs the gradient harness instead (cells of the
chain65536 workload, --steps steps) and prints the stage clocks of the forward chain,
of the adjoint's taped recompute and of its reverse sweep.  The instrumented library
is separate from the product build.

    python -m uclales_salsa_gb300.stage_profile [--X 96 --Y 96 --Z 32] [--classes]
    python -m uclales_salsa_gb300.stage_profile --chain [--cells 16384 --steps 10]
"""
import argparse
import ctypes as C
import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

from . import build as B
from . import api

STAGES = ["unpack", "coag(update)", "condensation", "activation", "ice nucl+melt", "distr_update", "output", "-",
          "coag kernels", "cond substeps", "equilibration"]
# stages 8-10 are parts of stages 1 and 2
CHAIN_STAGES = {11: "collision kernels", 12: "coagulation update", 13: "condensation", 14: "reverse condensation",
                15: "reverse coagulation", 3: "reverse collision kernels"}
# sub-stages (indented in the print-out) of the chain's condensation and its reverse
CHAIN_SUB = {13: [(5, "1a uptake + coefficients"), (6, "substeps")],
             14: [(0, "coefficients + substeps"), (1, "coefficient partials"), (2, "1a uptake")]}


def build_instrumented():
    out = os.path.join(B.BUILD, "stages")
    os.makedirs(out, exist_ok=True)

    def comp(u):
        obj = os.path.join(out, u.replace(".cu", ".o"))
        extra = ["-fmad=false"] if u in B.FP64_UNITS else []
        subprocess.run([B.nvcc()] + B.ARCH + ["-O3", "-std=c++17", "-Xcompiler", "-fPIC", "-DSALSA_STAGE_TIMERS"] +
                       extra + ["-c", os.path.join(B.CSRC, u), "-o", obj], check=True)
        return obj

    with ThreadPoolExecutor(len(B.UNITS)) as ex:
        objs = list(ex.map(comp, B.UNITS))
    lib = os.path.join(out, "libsalsa_stages.so")
    subprocess.run([B.nvcc()] + B.ARCH + ["-shared", "-o", lib] + objs + ["-lcudart"], check=True)
    return lib


def chain_stages(L, cells, steps):
    import torch
    from .inputs import make_inputs
    from .chain import SalsaChain, chain_config, pack_state
    inp = make_inputs("chain65536", "cuda", X=1, Y=1, Z=cells)
    inp.cfg = chain_config()
    x, th, k, s = pack_state(inp)
    ch = SalsaChain(inp.cfg)
    yb = torch.ones_like(x)
    arr = (C.c_ulonglong * 16)()
    _, ck = ch.forward(x, th, k, s, 2, inp.dt)          # warm-up
    ch.adjoint(ck, 1, th, k, s, 2, inp.dt, yb)
    L.salsa_gb300_stage_clocks(ch.step.h, arr)
    _, ck = ch.forward(x, th, k, s, steps, inp.dt)
    L.salsa_gb300_stage_clocks(ch.step.h, arr)
    fwd = [arr[i] for i in range(16)]
    ch.adjoint(ck, 1, th, k, s, steps, inp.dt, yb)
    L.salsa_gb300_stage_clocks(ch.step.h, arr)
    adj = [arr[i] for i in range(16)]
    ch.close()
    norm = cells * steps
    print(f"chain65536 block: {cells} cells x {steps} steps (warp clocks per cell-step)")
    def show(arr, stages):
        for i in stages:
            print(f"     {CHAIN_STAGES[i]:32s} {arr[i] / norm:10.0f}")
            for j, name in CHAIN_SUB.get(i, []):
                print(f"       {name:30s} {arr[j] / norm:10.0f}")
        print(f"     {'total':32s} {sum(arr[i] for i in stages) / norm:10.0f}")

    print("   forward:")
    show(fwd, (11, 12, 13))
    print("   adjoint (taped recompute, then reverse):")
    show(adj, (11, 12, 13, 14, 15, 3))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--X", type=int, default=96)
    ap.add_argument("--Y", type=int, default=96)
    ap.add_argument("--Z", type=int, default=32)
    ap.add_argument("--chain", action="store_true")
    ap.add_argument("--cells", type=int, default=16384)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--classes", action="store_true",
                    help="also profile grid384x384x160 with clear cells only and with cloudy cells only")
    a = ap.parse_args()
    lib = build_instrumented()
    B.LIB = lib
    api._lib = None
    L = api.library()
    L.salsa_gb300_stage_clocks.argtypes = [C.c_void_p, C.POINTER(C.c_ulonglong)]
    if a.chain:
        chain_stages(L, a.cells, a.steps)
        return
    import torch
    from .inputs import make_inputs, make_outputs
    cases = [("grid256x256x128", None), ("grid384x384x160", None)]
    if a.classes:
        cases += [("grid384x384x160", dict(cloudy=0.0)), ("grid384x384x160", dict(cloudy=1.0, pattern="random"))]
    for wl, ov in cases:
        for prec in (0, 1):
            inp = make_inputs(wl, "cuda", precision=prec, diagnostics=0, X=a.X, Y=a.Y, Z=a.Z, overrides=ov)
            s = api.SalsaStep(inp.cfg)
            outs = make_outputs(inp, with_diag=False)
            arr = (C.c_ulonglong * 16)()
            f = {k: v.clone() for k, v in inp.fields.items()}
            s.run(inp, f, outs)                      # warm-up
            L.salsa_gb300_stage_clocks(s.h, arr)     # reads and clears the counters
            f = {k: v.clone() for k, v in inp.fields.items()}
            s.run(inp, f, outs)
            L.salsa_gb300_stage_clocks(s.h, arr)
            tot = sum(arr[i] for i in range(7))
            print(wl, ov or "", "precision", prec, "cells", inp.ncells, "kernel ms", round(s.last_kernel_ms(), 2))
            for i, n in enumerate(STAGES):
                if n != "-":
                    print(f"   {n:16s} {100.0 * arr[i] / tot:6.2f} %   ({arr[i] / inp.ncells:.0f} warp-clk/cell)")
            sys.stdout.flush()
            s.close()
            del f, outs, inp
            torch.cuda.empty_cache()


if __name__ == "__main__":
    main()
