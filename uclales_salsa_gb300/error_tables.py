"""Error tables of the FP32-mixed form over many steps.

Runs the same seeded block of a workload for `steps` SALSA steps in three ways:
the FP64 CPU oracle (the reference restatement), the FP64 GPU form and the
FP32-mixed GPU form.  Every step adds the tendencies to the prognostic fields
(numbers, masses, water vapour, IN deficit), as the LES time step would.  After
the last step it prints, per bin, the maximum and the RMS relative error of the
number and of the total mass (all species) of the mixed form against the oracle,
and the drift of the total mass of each species.  Relative errors use the floors
of the parity tests (numbers 1e-3 /kg, masses 1e-24 kg/kg).

    python -m uclales_salsa_gb300.error_tables --workload grid256x256x128 --X 16 --Y 16 --Z 16 --steps 100
"""
import argparse
import os
import sys

import torch

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, os.path.join(ROOT, "tests"))

from .inputs import make_inputs, make_outputs  # noqa: E402
from .api import SalsaStep  # noqa: E402

PROG = {"naerot": "naero", "ncloudt": "ncloud", "nprecpt": "nprecp", "nicet": "nice", "maerot": "maero",
        "mcloudt": "mcloud", "mprecpt": "mprecp", "micet": "mice", "rpt": "rp"}
FLOOR_N, FLOOR_M = 1.e-3, 1.e-24


def advance(run, inp, fields, steps):
    for k in range(steps):
        out = make_outputs(inp, device=fields["press"].device, with_diag=False)
        run(fields, out, float(k + 1))
        for t, f in PROG.items():
            if t in out:
                fields[f] += out[t] * inp.dt
    return fields


def interior(inp, t):
    v = t[..., 2:inp.nyp - 2, 2:inp.nxp - 2, 1:inp.nzp - 1]
    return v.reshape(v.shape[0], -1)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--workload", default="grid256x256x128")
    ap.add_argument("--X", type=int, default=16)
    ap.add_argument("--Y", type=int, default=16)
    ap.add_argument("--Z", type=int, default=16)
    ap.add_argument("--steps", type=int, default=100)
    a = ap.parse_args()
    from oracle_ref import Oracle
    inp = make_inputs(a.workload, "cpu", X=a.X, Y=a.Y, Z=a.Z, precision=0, diagnostics=0)
    lay = inp.layout
    init = {k: v.clone() for k, v in inp.fields.items()}

    orc = Oracle(inp.cfg)

    def run_oracle(f, out, time):
        rc, st = orc.run(inp, f, out, time=time)
        assert rc == 0, st.as_dict()

    ref = advance(run_oracle, inp, {k: v.clone() for k, v in init.items()}, a.steps)
    res = {}
    for prec in (0, 1):
        inp.cfg.precision = prec
        step = SalsaStep(inp.cfg)

        def run_gpu(f, out, time):
            step.run(inp, f, out, time=time)

        g = advance(run_gpu, inp, {k: v.clone().cuda() for k, v in init.items()}, a.steps)
        res[prec] = {k: v.cpu() for k, v in g.items()}
        step.close()
    cats = [("aerosol", "naero", "maero", lay.nbins, lay.nwet), ("cloud", "ncloud", "mcloud", lay.ncld, lay.nwet),
            ("precipitation", "nprecp", "mprecp", lay.nprc, lay.nwet)]
    if inp.level == 5:
        cats.append(("ice", "nice", "mice", lay.nice, lay.nwet + 1))
    print(f"# {a.workload} block {a.X}x{a.Y}x{a.Z} ({inp.ncells} cells), {a.steps} steps of {inp.dt} s\n")
    for prec, name in ((1, "FP32-mixed"), (0, "FP64 GPU")):
        print(f"## {name} form against the FP64 oracle\n")
        print("| category | bin | N max rel | N RMS rel | M max rel | M RMS rel |")
        print("|---|---|---|---|---|---|")
        worst = [0., 0.]
        for cname, nk, mk, nb, nsp in cats:
            n_r, n_g = interior(inp, ref[nk]), interior(inp, res[prec][nk])
            m_r = interior(inp, ref[mk]).reshape(nsp, nb, -1).sum(0)
            m_g = interior(inp, res[prec][mk]).reshape(nsp, nb, -1).sum(0)
            for b in range(nb):
                en = (n_g[b] - n_r[b]).abs() / n_r[b].abs().clamp(min=FLOOR_N)
                em = (m_g[b] - m_r[b]).abs() / m_r[b].abs().clamp(min=FLOOR_M)
                worst[0] = max(worst[0], float(en.max()))
                worst[1] = max(worst[1], float(em.max()))
                print(f"| {cname} | {b} | {float(en.max()):.2e} | {float(en.pow(2).mean().sqrt()):.2e} | "
                      f"{float(em.max()):.2e} | {float(em.pow(2).mean().sqrt()):.2e} |")
        print(f"\nworst bin: number {worst[0]:.2e}, mass {worst[1]:.2e}\n")
        print("| species | total mass change over the run (oracle) | relative difference to the oracle |")
        print("|---|---|---|")
        for s, sp in enumerate(lay.species + ["H2O"]):
            tot = lambda d: sum(float(interior(inp, d[mk]).reshape(nsp, nb, -1)[s].sum())
                                for _, _, mk, nb, nsp in cats)
            t0, tr, tg = tot(init), tot(ref), tot(res[prec])
            print(f"| {sp} | {(tr - t0) / max(abs(t0), 1e-300):+.3e} | {(tg - tr) / max(abs(tr), 1e-300):+.3e} |")
        print()


if __name__ == "__main__":
    main()
