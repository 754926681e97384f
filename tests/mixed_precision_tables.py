"""Error tables of the FP32-mixed form over many steps (measurement script, not a test).

Advances the whole workload (default: the 256x256x128 grid, 8,388,608 cells) for
`steps` SALSA steps twice on the GPU, in the FP64 form and in the FP32-mixed form,
and a 262,144-cell sub-block of the same fields in the FP64 oracle, once as built for
parity (no multiply-add contraction) and once built with contraction.  Every step adds
the tendencies to the prognostic fields (numbers, masses, water vapour; the IN deficit
is updated in place), as the LES time step does.

After the last step it prints, per bin, the errors of the number and of the total mass
(all species) of one state against another: the mixed form against the FP64 form over
every cell, both GPU forms against the oracle on the sub-block, and the contracted
oracle against the oracle on the sub-block.  The last comparison is the spread of two
correct FP64 builds of the same code after the same steps, the yardstick for the
others.  Per bin:

- max and RMS of the relative difference |a - b| / max(|a|, |b|, floor), floors
  1e-3 /kg for numbers and 1e-24 kg/kg for masses (a bin empty in one state and
  populated in the other counts 1); a bin's mass in a cell where it holds fewer
  particles than the number floor in both states is the residue of an emptied bin and
  is not counted;
- the number of cells beyond 1e-3;
- the largest |a - b| over the cells, relative to the bin's largest value.

Then a summary per category and comparison, the step times and the change of each
species' total mass over the run.

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
    secs = []
    for k in range(steps):
        for v in out.values():
            v.zero_()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        rc, st = step.run(inp, fields, out, time=float(k + 1), istp=k + 1)
        secs.append(time.perf_counter() - t0)
        assert rc in (0, 4), st.as_dict()
        for t, f in PROG.items():
            if t in out:
                fields[f].add_(out[t], alpha=inp.dt)
    torch.cuda.synchronize()
    step.close()
    return fields, secs


def advance_oracle(inp, fields, steps, variant="plain"):
    from oracle_ref import Oracle
    o = Oracle(inp.cfg, variant=variant)
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


def bin_errors(inp, a, b, box=(None, None, None)):
    """Per category and bin, the errors of state a against state b: for the number and
    for the total mass, (max rel, RMS rel, cells beyond 1e-3, max abs / bin max)."""
    X, Y, Z = box
    res = []
    for cname, nk, mk, nb, nsp in categories(inp):
        n_a, n_b = interior(inp, a[nk], X, Y, Z).double(), interior(inp, b[nk], X, Y, Z).double()
        m_a = interior(inp, a[mk], X, Y, Z).double().reshape(nsp, nb, -1).sum(0)
        m_b = interior(inp, b[mk], X, Y, Z).double().reshape(nsp, nb, -1).sum(0)
        for i in range(nb):
            row = []
            held = torch.maximum(n_a[i].abs(), n_b[i].abs()) > FLOOR_N
            for xa, xb, floor in ((n_a[i], n_b[i], FLOOR_N), (m_a[i], m_b[i], FLOOR_M)):
                d = (xa - xb).abs()
                r = d / torch.maximum(xa.abs(), xb.abs()).clamp(min=floor)
                if floor == FLOOR_M:
                    r = torch.where(held, r, torch.zeros_like(r))
                big = float(xb.abs().max())
                row.append((float(r.max()), float(r.pow(2).mean().sqrt()), int((r > 1e-3).sum()),
                            float(d.max()) / big if big > 0 else 0.))
            res.append((cname, i, row))
    return res


def bin_table(title, errs):
    print(f"### {title}\n")
    print("| category | bin | N max rel | N RMS rel | N cells > 1e-3 | N max abs / bin max "
          "| M max rel | M RMS rel | M cells > 1e-3 | M max abs / bin max |")
    print("|---|---|---|---|---|---|---|---|---|---|")
    for cname, i, row in errs:
        cols = " | ".join(f"{mx:.2e} | {rms:.2e} | {cnt} | {ab:.2e}" for mx, rms, cnt, ab in row)
        print(f"| {cname} | {i} | {cols} |")
    print()


def summary_table(rows, ncells):
    """One line per comparison and category: the largest RMS relative difference and
    the largest count of cells beyond 1e-3 over the category's bins (number or mass),
    and the largest max-abs / bin-max."""
    print("| comparison | cells | category | largest RMS rel | most cells > 1e-3 in a bin | largest max abs / bin max |")
    print("|---|---|---|---|---|---|")
    for name, errs in rows:
        for cname in dict.fromkeys(c for c, _, _ in errs):
            sel = [row for c, _, row in errs if c == cname]
            rms = max(max(q[1] for q in r) for r in sel)
            cnt = max(max(q[2] for q in r) for r in sel)
            ab = max(max(q[3] for q in r) for r in sel)
            print(f"| {name} | {ncells[name]} | {cname} | {rms:.2e} | {cnt} | {ab:.2e} |")
    print()


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
    res, secs, steps = {}, {}, {}
    for prec in (0, 1):
        inp.cfg.precision = prec
        t0 = time.perf_counter()
        res[prec], steps[prec] = advance_gpu(inp, {k: v.clone() for k, v in init.items()}, a.steps)
        secs[prec] = time.perf_counter() - t0
    inp.cfg.precision = 0
    sub = sub_block(inp, X, Y, Z)
    sub.fields = {k: v.cpu() for k, v in sub.fields.items()}
    ref = {}
    for var in ("plain", "contract"):
        t0 = time.perf_counter()
        ref[var] = advance_oracle(sub, {k: v.clone() for k, v in sub.fields.items()}, a.steps, var)
        secs[var] = time.perf_counter() - t0
    nsub = X * Y * Z
    print(f"# {a.workload} ({inp.ncells} cells), {a.steps} steps of {inp.dt} s\n")
    print(f"GPU: FP64 form {secs[0]:.0f} s, mixed form {secs[1]:.0f} s for the run; oracle sub-block "
          f"{X}x{Y}x{Z} ({nsub} cells) {secs['plain']:.0f} s, contracted build {secs['contract']:.0f} s, "
          f"on {os.cpu_count()} threads.\n")
    q = lambda v, k: v[min(k, len(v) - 1)]
    print("Step times on the GPU (s), first / 10th / 50th / last step: FP64 form "
          + " / ".join(f"{q(steps[0], k):.2f}" for k in (0, 9, 49, a.steps - 1)) + "; mixed form "
          + " / ".join(f"{q(steps[1], k):.2f}" for k in (0, 9, 49, a.steps - 1)) + ".\n")
    cpu = lambda d: {k: v[..., :Y + 4, :X + 4, :Z + 2].cpu() for k, v in d.items()}
    box = (X, Y, Z)
    rows = [("mixed vs FP64, every cell", bin_errors(inp, res[1], res[0])),
            ("FP64 vs oracle, sub-block", bin_errors(sub, cpu(res[0]), ref["plain"], box)),
            ("mixed vs oracle, sub-block", bin_errors(sub, cpu(res[1]), ref["plain"], box)),
            ("contracted oracle vs oracle, sub-block", bin_errors(sub, ref["contract"], ref["plain"], box))]
    ncells = {rows[0][0]: inp.ncells, rows[1][0]: nsub, rows[2][0]: nsub, rows[3][0]: nsub}
    print("### Summary\n")
    summary_table(rows, ncells)
    for name, errs in rows:
        bin_table(name, errs)
    print("### Species totals over the run, every cell\n")
    species_table(inp, init, [res[0], res[1]], ["FP64 form", "mixed form"])


if __name__ == "__main__":
    main()
