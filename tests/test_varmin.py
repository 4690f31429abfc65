"""Variance-minimisation driver, host side: the grids and parameter mapping
of JastrowOptimizer::optimize (src/sampling/optimize.rs:210-304)."""
import numpy as np

import rust_qmc_gb300 as Q
from rust_qmc_gb300 import varmin as V


def test_coarse_grid_order():
    g = V.coarse_grid()
    assert len(g) == 42
    assert g[0] == (0.5, 1.0) and g[1] == (0.5, 2.0) and g[6] == (1.0, 1.0) and g[-1] == (5.0, 6.0)


def test_fine_grid_clamps():
    g = V.fine_grid((0.5, 1.0))
    assert len(g) == 49
    b_ee = sorted(set(p[0] for p in g))
    b_en = sorted(set(p[1] for p in g))
    assert b_ee == [0.25, 0.5, 0.75, 1.0, 1.25]          # 0.5 - 0.75 and 0.5 - 0.5 clamp to 0.25
    assert b_en == [0.5, 0.75, 1.0, 1.25, 1.5, 1.75]
    assert g[0] == (0.25, 0.5) and g[-1] == (1.25, 1.75)
    g2 = V.fine_grid((3.0, 4.0))
    assert g2[0] == (2.25, 3.25) and g2[24] == (3.0, 4.0) and g2[-1] == (3.75, 4.75)


def test_with_jastrow_sets_both_classes():
    s = Q.methane_minimal()
    t = V.with_jastrow(s, 2.5, 3.5)
    assert t.jas[0] == t.jas[1] == 2.5 and t.jas[4] == t.jas[5] == 3.5
    np.testing.assert_array_equal(t.jas[[2, 3, 6, 7]], s.jas[[2, 3, 6, 7]])
    np.testing.assert_array_equal(t.rot_angle, s.rot_angle)
