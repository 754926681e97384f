"""Generate the golden fixtures of the CPU oracle.

The reference ships no tests or golden data for this path and cannot be
compiled here (no Fortran compiler), so these fixtures pin the oracle's own
outputs: every test re-runs the oracle on the same seeded inputs and checks it
reproduces them.  Regenerate only when the oracle is deliberately changed:
    python tests/golden/make_golden.py [tag ...]
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
sys.path.insert(0, os.path.dirname(HERE))

from uclales_salsa_gb300.inputs import make_inputs, make_outputs  # noqa: E402
from oracle_ref import Oracle  # noqa: E402

CASES = {
    "grid16x16x40_sub": dict(name="grid16x16x40", X=4, Y=4, Z=8),
    "grid256x256x128_sub": dict(name="grid256x256x128", X=4, Y=4, Z=8),
    "grid384x384x160_sub": dict(name="grid384x384x160", X=8, Y=8, Z=4),
    # all processes and the three secondary-ice schemes (tests/sip_cases.py state)
    "secondary_ice_sub": dict(name="sip", X=4, Y=4, Z=8),
}


def sip_inputs(X, Y, Z):
    from sip_cases import sip_state
    inp = sip_state(1, coag_only=False, X=X, Y=Y, Z=Z)
    for sw in (inp.cfg.lssipdropfrac, inp.cfg.lssipicecollbreak):
        sw.sw, sw.mode = 1, 1
    return inp


def run_case(spec):
    kw = dict(spec)
    name = kw.pop("name")
    inp = sip_inputs(**kw) if name == "sip" else make_inputs(name, "cpu", **kw)
    fields = {k: v.clone() for k, v in inp.fields.items()}
    out = make_outputs(inp)
    rc, st = Oracle(inp.cfg).run(inp, fields, out, time=1.0, nthreads=1)
    return inp, fields, out, rc


def main(tags):
    for tag, spec in CASES.items():
        if tags and tag not in tags:
            continue
        inp, fields, out, rc = run_case(spec)
        assert rc == 0
        arrays = {f"out_{k}": v.numpy() for k, v in out.items()}
        if "indef" in fields:
            arrays["indef_after"] = fields["indef"].numpy()
        for k in ("sipdrfr", "siprmspl", "sipiibr"):
            if k in fields:
                arrays[f"{k}_after"] = fields[k].numpy()
        np.savez_compressed(os.path.join(HERE, f"{tag}.npz"), **arrays)
        print("wrote", tag, sorted(arrays))


if __name__ == "__main__":
    main(sys.argv[1:])   # tags to write (default: all)
