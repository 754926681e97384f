"""Per-stage clock breakdown of the SALSA step.

Builds an instrumented copy of the library (-DSALSA_STAGE_TIMERS: every warp adds
clock64() deltas of the process stages of its cell to a device counter array) into
_build/stages/, runs one step of each form on a block of the workloads and prints
each stage's share.  The instrumented library is separate from the product build.

    python -m uclales_salsa_gb300.stage_profile [--X 96 --Y 96 --Z 32]
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


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--X", type=int, default=96)
    ap.add_argument("--Y", type=int, default=96)
    ap.add_argument("--Z", type=int, default=32)
    a = ap.parse_args()
    lib = build_instrumented()
    B.LIB = lib
    api._lib = None
    L = api.library()
    L.salsa_gb300_stage_clocks.argtypes = [C.c_void_p, C.POINTER(C.c_ulonglong)]
    import torch
    from .inputs import make_inputs, make_outputs
    for wl in ("grid256x256x128", "grid384x384x160"):
        for prec in (0, 1):
            inp = make_inputs(wl, "cuda", precision=prec, diagnostics=0, X=a.X, Y=a.Y, Z=a.Z)
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
            print(wl, "precision", prec, "cells", inp.ncells, "kernel ms", round(s.last_kernel_ms(), 2))
            for i, n in enumerate(STAGES):
                if n != "-":
                    print(f"   {n:16s} {100.0 * arr[i] / tot:6.2f} %   ({arr[i] / inp.ncells:.0f} warp-clk/cell)")
            sys.stdout.flush()
            s.close()
            del f, outs, inp
            torch.cuda.empty_cache()


if __name__ == "__main__":
    main()
