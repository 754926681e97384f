"""CPU tests of the per-bin metric of the many-step error tables
(tests/mixed_precision_tables.py): bounded relative differences, the count of cells
beyond 1e-3, the largest difference over the bin's largest value, and mass residues of
emptied bins left out."""
import os
import sys

import torch

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)

import mixed_precision_tables as T  # noqa: E402
from uclales_salsa_gb300.inputs import make_inputs  # noqa: E402


def _state():
    inp = make_inputs("grid256x256x128", "cpu", X=4, Y=4, Z=4, precision=0, diagnostics=0)
    return inp, {k: v.clone() for k, v in inp.fields.items()}


def _errs(inp, a, b, cat, i):
    for cname, bi, row in T.bin_errors(inp, a, b):
        if cname == cat and bi == i:
            return row
    raise KeyError((cat, i))


def test_identical_states_have_no_error():
    inp, a = _state()
    for cname, _, row in T.bin_errors(inp, a, {k: v.clone() for k, v in a.items()}):
        for mx, rms, cnt, ab in row:
            assert mx == 0. and rms == 0. and cnt == 0 and ab == 0., cname


def test_a_bin_empty_in_one_state_counts_one_and_its_cells():
    inp, a = _state()
    b = {k: v.clone() for k, v in a.items()}
    # cloud bin 3, one interior cell: populated in b, empty in a
    b["ncloud"][3, 2, 2, 1] = 5.e6
    a["ncloud"][3, 2, 2, 1] = 0.
    (n_mx, n_rms, n_cnt, n_ab), _ = _errs(inp, a, b, "cloud", 3)
    assert n_mx == 1.
    assert n_cnt == 1
    assert 0. < n_rms <= 1.
    assert abs(n_ab - 5.e6 / float(T.interior(inp, b["ncloud"])[3].abs().max())) < 1e-12


def test_mass_residue_of_a_bin_empty_in_both_states_is_not_counted():
    inp, a = _state()
    b = {k: v.clone() for k, v in a.items()}
    lay = inp.layout
    a["naero"][4, 2, 2, 1] = b["naero"][4, 2, 2, 1] = 0.
    for s in range(lay.nwet):
        a["maero"][s * lay.nbins + 4, 2, 2, 1] = 0.
        b["maero"][s * lay.nbins + 4, 2, 2, 1] = 3.e-24 * (s + 1)
    _, (m_mx, m_rms, m_cnt, m_ab) = _errs(inp, a, b, "aerosol", 4)
    assert m_mx == 0. and m_cnt == 0
    # the same residue next to a populated bin is counted
    a["naero"][4, 2, 2, 1] = b["naero"][4, 2, 2, 1] = 1.e2
    _, (m_mx, m_rms, m_cnt, m_ab) = _errs(inp, a, b, "aerosol", 4)
    assert m_mx == 1. and m_cnt == 1


def test_summary_takes_the_largest_figure_of_each_category(capsys):
    inp, a = _state()
    b = {k: v.clone() for k, v in a.items()}
    b["nprecp"][1, 2, 3, 1] = a["nprecp"][1, 2, 3, 1] * 1.01 + 1.
    errs = T.bin_errors(inp, a, b)
    T.summary_table([("x vs y", errs)], {"x vs y": inp.ncells})
    out = capsys.readouterr().out
    line = [ln for ln in out.splitlines() if "| precipitation |" in ln][0]
    cells = [c.strip() for c in line.strip("|").split("|")]
    assert cells[0] == "x vs y" and int(cells[1]) == inp.ncells
    assert int(cells[4]) == 1
    assert float(cells[3]) > 0.
    assert torch.isfinite(torch.tensor(float(cells[5])))
