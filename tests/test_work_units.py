"""CPU tests of the oracle's work-unit counters (tests/work_units.py): clear cells take
no condensation substeps and no water-activity calls; every count per cell stays
within the bounds of the bin layout."""
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)

import work_units as W  # noqa: E402


def test_clear_cells_take_no_substeps_and_no_activity_calls():
    n, per, _ = W.count("grid384x384x160", (8, 8, 4), dict(cloudy=0.0))
    assert n == 256
    coagc, acth2o, jimm, equil, substeps = per
    assert acth2o == 0. and substeps == 0.
    assert 0. < coagc <= 1035.
    assert equil > 0.


def test_cloudy_cells_count_every_unit_within_the_layout_bounds():
    n, per, _ = W.count("grid384x384x160", (8, 8, 4), dict(cloudy=1.0, pattern="random"))
    coagc, acth2o, jimm, equil, substeps = per
    assert 0. < coagc <= 1035.          # at most one evaluation per bin pair (45 bins at level 5)
    assert substeps > 0. and acth2o > 0.
    assert jimm == 0. or jimm >= 10.    # 10 Gauss-Legendre nodes per bin that can freeze
