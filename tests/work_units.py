"""Work per cell-step, counted in the oracle (measurement script, not a test).

Runs one SALSA step of each workload's sample block in the FP64 oracle and prints the
oracle's work-unit counters per cell: collision-kernel (coagc) evaluations, water
activity (acth2o) calls, immersion/deposition nucleation rate (J_imm, J_dep)
evaluations at the Gauss-Legendre nodes, equilibration iterations and condensation
substeps.  The grid384x384x160 sample is also split into its clear and its cloudy
cells.

    python tests/work_units.py
"""
import os
import sys
import time

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))
sys.path.insert(0, HERE)

from uclales_salsa_gb300.inputs import make_inputs, make_outputs  # noqa: E402

UNITS = ("coagc evaluations", "acth2o calls", "J_imm / J_dep evaluations", "equilibration iterations",
         "condensation substeps")

# (label, workload, interior X Y Z or None for the whole grid, overrides)
SAMPLES = [
    ("grid16x16x40 (whole grid, level 4)", "grid16x16x40", None, None),
    ("grid256x256x128, 64x64x16 block", "grid256x256x128", (64, 64, 16), None),
    ("grid384x384x160, 64x64x16 block", "grid384x384x160", (64, 64, 16), None),
    ("grid384x384x160, clear cells", "grid384x384x160", (64, 64, 16), dict(cloudy=0.0)),
    ("grid384x384x160, cloudy cells", "grid384x384x160", (64, 64, 16), dict(cloudy=1.0, pattern="random")),
]


def count(name, box, overrides):
    from oracle_ref import Oracle
    kw = dict(X=box[0], Y=box[1], Z=box[2]) if box else {}
    inp = make_inputs(name, "cpu", precision=0, diagnostics=0, overrides=overrides, **kw)
    o = Oracle(inp.cfg)
    out = make_outputs(inp, with_diag=False)
    t0 = time.perf_counter()
    rc, st = o.run(inp, {k: v.clone() for k, v in inp.fields.items()}, out, time=1.0, istp=1)
    secs = time.perf_counter() - t0
    assert rc in (0, 4), st.as_dict()
    return inp.ncells, [c / inp.ncells for c in o.counters()], secs


def main():
    print("| sample | cells | " + " | ".join(UNITS) + " |")
    print("|---|---|" + "---|" * len(UNITS))
    for label, name, box, ov in SAMPLES:
        n, per, secs = count(name, box, ov)
        print(f"| {label} | {n} | " + " | ".join(f"{x:.1f}" for x in per) + " |", flush=True)
    print(f"\nper cell-step, one step of 1 s from the initial state; oracle on {os.cpu_count()} threads")


if __name__ == "__main__":
    main()
