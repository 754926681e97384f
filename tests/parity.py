"""Comparison helpers for the parity tests (GPU step vs the CPU oracle)."""
import torch

NUMBER_FIELDS = ["naerot", "ncloudt", "nprecpt", "nicet"]
MASS_FIELDS = ["maerot", "mcloudt", "mprecpt", "micet"]
STATE_OF = {"naerot": "naero", "ncloudt": "ncloud", "nprecpt": "nprecp", "nicet": "nice",
            "maerot": "maero", "mcloudt": "mcloud", "mprecpt": "mprecp", "micet": "mice", "rpt": "rp",
            "gaerot": "gaero"}
# absolute floors below which a value is physically empty: numbers in #/kg, masses in kg/kg,
# gas molecules in #/kg
FLOOR = {"n": 1.e-3, "m": 1.e-24, "rp": 1.e-12, "g": 1.0}


def floor_of(name):
    if name == "rpt":
        return FLOOR["rp"]
    if name == "gaerot":
        return FLOOR["g"]
    return FLOOR["n"] if name in NUMBER_FIELDS else FLOOR["m"]


def interior(t, nzp, nxp, nyp):
    """View of the interior cells of a (..., nyp, nxp, nzp) tensor."""
    return t[..., 2:nyp - 2, 2:nxp - 2, 1:nzp - 1]


def state_errors(inp, fields, out_a, out_b, tol=1e-6):
    """Max relative error of the NEW state (old + tendency * dt) per output field.

    The error of a bin value is measured relative to the scale of its update,
    max(|new_ref|, |old|, floor): when a process empties a bin completely the
    result is the difference of two equal magnitudes and its rounding is relative
    to the old value.  Returns {field: (max_rel, n_over_tol, n)}."""
    res = {}
    dt = inp.dt
    for name, st in STATE_OF.items():
        if name not in out_a or name not in out_b:
            continue
        old = fields[st].double().cpu()
        a = old + out_a[name].double().cpu() * dt
        b = old + out_b[name].double().cpu() * dt
        a = interior(a, inp.nzp, inp.nxp, inp.nyp)
        b = interior(b, inp.nzp, inp.nxp, inp.nyp)
        fl = floor_of(name)
        o = interior(old, inp.nzp, inp.nxp, inp.nyp)
        scale = torch.maximum(b.abs(), o.abs()).clamp(min=fl)
        rel = (a - b).abs() / scale
        res[name] = (float(rel.max()), int((rel > tol).sum()), rel.numel())
    return res


def output_errors(inp, out_a, out_b, names=("pa_nactd", "pa_vactd", "diag")):
    res = {}
    for name in names:
        if name not in out_a:
            continue
        a = interior(out_a[name].double().cpu(), inp.nzp, inp.nxp, inp.nyp)
        b = interior(out_b[name].double().cpu(), inp.nzp, inp.nxp, inp.nyp)
        if name == "diag":
            for i in range(a.shape[0]):
                scale = float(b[i].abs().max())
                res[f"diag{i}"] = float((a[i] - b[i]).abs().max()) / max(scale, 1e-300)
        else:
            res[name] = float((a - b).abs().max())
    return res
