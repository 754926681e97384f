"""Error tables of the FP32-mixed form over many steps (measurement script, not a test).

Advances the whole workload (default: the 256x256x128 grid, 8,388,608 cells) for
`steps` SALSA steps twice on the GPU, in the FP64 form and in the FP32-mixed form,
and a 262,144-cell sub-block of the same fields in the FP64 oracle.  Every step adds
the tendencies to the prognostic fields (numbers, masses, water vapour; the IN deficit
is updated in place), as the LES time step does.  After the last step it prints, per
bin, the maximum and RMS relative error of the number and of the total mass (all
species) of the mixed form against the FP64 form over every cell, the same for both GPU
forms against the oracle on the sub-block, and the change of each species' total mass
over the run.  Relative errors use the floors of the parity tests (numbers 1e-3 /kg,
masses 1e-24 kg/kg).

    python tests/mixed_precision_tables.py --workload grid256x256x128 --steps 100
"""
import argparse
import os
import sys
import time

import torch

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))
sys.path.insert(0, HERE)

from uclales_salsa_gb300.inputs import make_inputs, make_outputs  # noqa: E402
from uclales_salsa_gb300.api import SalsaStep  # noqa: E402

PROG = {"naerot": "naero", "ncloudt": "ncloud", "nprecpt": "nprecp", "nicet": "nice", "maerot": "maero",
        "mcloudt": "mcloud", "mprecpt": "mprecp", "micet": "mice", "rpt": "rp"}
FLOOR_N, FLOOR_M = 1.e-3, 1.e-24


def sub_block(inp, X, Y, Z):
    """The first X x Y x Z interior cells of `inp` as inputs of their own (halo rows and
    columns are the neighbours' values; the step never reads them)."""
    from copy import copy
    s = copy(inp)
    s.fields = {k: v[..., :Y + 4, :X + 4, :Z + 2].contiguous() for k, v in inp.fields.items()}
    s.nyp, s.nxp, s.nzp = Y + 4, X + 4, Z + 2
    return s


def advance_gpu(inp, fields, steps):
    """Every step: zero the tendencies, one synchronous SALSA call, add the tendencies
    (torch's stream and the library's are ordered by the synchronisations)."""
    step = SalsaStep(inp.cfg)
    out = make_outputs(inp, with_diag=False)
    for k in range(steps):
        for v in out.values():
            v.zero_()
        torch.cuda.synchronize()
        rc, st = step.run(inp, fields, out, time=float(k + 1), istp=k + 1)
        assert rc in (0, 4), st.as_dict()
        for t, f in PROG.items():
            if t in out:
                fields[f].add_(out[t], alpha=inp.dt)
    torch.cuda.synchronize()
    step.close()
    return fields


def advance_oracle(inp, fields, steps):
    from oracle_ref import Oracle
    o = Oracle(inp.cfg)
    for k in range(steps):
        out = make_outputs(inp, with_diag=False)
        rc, st = o.run(inp, fields, out, time=float(k + 1), istp=k + 1)
        assert rc in (0, 4), st.as_dict()
        for t, f in PROG.items():
            if t in out:
                fields[f] += out[t] * inp.dt
    return fields


def interior(inp, t, X=None, Y=None, Z=None):
    Y = Y or inp.nyp - 4
    X = X or inp.nxp - 4
    Z = Z or inp.nzp - 2
    v = t[..., 2:2 + Y, 2:2 + X, 1:1 + Z]
    return v.reshape(v.shape[0], -1)


def categories(inp):
    lay = inp.layout
    cats = [("aerosol", "naero", "maero", lay.nbins, lay.nwet), ("cloud", "ncloud", "mcloud", lay.ncld, lay.nwet),
            ("precipitation", "nprecp", "mprecp", lay.nprc, lay.nwet)]
    if inp.level == 5:
        cats.append(("ice", "nice", "mice", lay.nice, lay.nwet + 1))
    return cats


def bin_table(inp, a, b, title, box=(None, None, None)):
    """Per-bin errors of state a against state b (number and total mass)."""
    X, Y, Z = box
    print(f"### {title}\n")
    print("| category | bin | N max rel | N RMS rel | M max rel | M RMS rel |")
    print("|---|---|---|---|---|---|")
    worst = [0., 0.]
    for cname, nk, mk, nb, nsp in categories(inp):
        n_a, n_b = interior(inp, a[nk], X, Y, Z).double(), interior(inp, b[nk], X, Y, Z).double()
        m_a = interior(inp, a[mk], X, Y, Z).double().reshape(nsp, nb, -1).sum(0)
        m_b = interior(inp, b[mk], X, Y, Z).double().reshape(nsp, nb, -1).sum(0)
        for i in range(nb):
            en = (n_a[i] - n_b[i]).abs() / n_b[i].abs().clamp(min=FLOOR_N)
            em = (m_a[i] - m_b[i]).abs() / m_b[i].abs().clamp(min=FLOOR_M)
            worst[0] = max(worst[0], float(en.max()))
            worst[1] = max(worst[1], float(em.max()))
            print(f"| {cname} | {i} | {float(en.max()):.2e} | {float(en.pow(2).mean().sqrt()):.2e} | "
                  f"{float(em.max()):.2e} | {float(em.pow(2).mean().sqrt()):.2e} |")
    print(f"\nworst bin: number {worst[0]:.2e}, mass {worst[1]:.2e}\n")


def species_table(inp, init, states, names):
    lay = inp.layout
    print("| species | " + " | ".join(f"total change, {n}" for n in names) + " | mixed - FP64 (relative) |")
    print("|---|" + "---|" * (len(names) + 1))
    for s, sp in enumerate(lay.species + ["H2O"]):
        def tot(d):
            return sum(float(interior(inp, d[mk]).double().reshape(nsp, nb, -1)[s].sum())
                       for _, _, mk, nb, nsp in categories(inp))
        t0 = tot(init)
        tt = [tot(d) for d in states]
        cells = " | ".join(f"{(t - t0) / max(abs(t0), 1e-300):+.3e}" for t in tt)
        print(f"| {sp} | {cells} | {(tt[1] - tt[0]) / max(abs(tt[0]), 1e-300):+.3e} |")
    print()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--workload", default="grid256x256x128")
    ap.add_argument("--steps", type=int, default=100)
    ap.add_argument("--sub", type=int, nargs=3, default=[64, 64, 64], help="oracle sub-block X Y Z")
    a = ap.parse_args()
    X, Y, Z = a.sub
    inp = make_inputs(a.workload, "cuda", precision=0, diagnostics=0)
    init = {k: v.clone() for k, v in inp.fields.items()}
    res, secs = {}, {}
    for prec in (0, 1):
        inp.cfg.precision = prec
        t0 = time.perf_counter()
        res[prec] = advance_gpu(inp, {k: v.clone() for k, v in init.items()}, a.steps)
        secs[prec] = time.perf_counter() - t0
    inp.cfg.precision = 0
    sub = sub_block(inp, X, Y, Z)
    sub.fields = {k: v.cpu() for k, v in sub.fields.items()}
    t0 = time.perf_counter()
    ref = advance_oracle(sub, {k: v.clone() for k, v in sub.fields.items()}, a.steps)
    secs["oracle"] = time.perf_counter() - t0
    print(f"# {a.workload} ({inp.ncells} cells), {a.steps} steps of {inp.dt} s\n")
    print(f"GPU: FP64 form {secs[0]:.0f} s, mixed form {secs[1]:.0f} s for the run; oracle sub-block "
          f"{X}x{Y}x{Z} ({X * Y * Z} cells) {secs['oracle']:.0f} s on {os.cpu_count()} threads.\n")
    bin_table(inp, res[1], res[0], "FP32-mixed form against the FP64 form, every cell")
    cpu = lambda d: {k: v[..., :Y + 4, :X + 4, :Z + 2].cpu() for k, v in d.items()}
    bin_table(sub, cpu(res[0]), ref, f"FP64 form against the oracle, {X}x{Y}x{Z} sub-block", (X, Y, Z))
    bin_table(sub, cpu(res[1]), ref, f"FP32-mixed form against the oracle, {X}x{Y}x{Z} sub-block", (X, Y, Z))
    print("### Species totals over the run, every cell\n")
    species_table(inp, init, [res[0], res[1]], ["FP64 form", "mixed form"])


if __name__ == "__main__":
    main()
