"""Geometry optimisation (rust_qmc_gb300/geometry.py) against the
reference's rules (src/sampling/geometry_opt.rs:176-309).

CPU: the steepest-descent step (charge-weighted mean force removed,
displacement capped at 0.02 bohr).
GPU: the bare and zero-variance mean forces from the device batches equal the
reference's estimators evaluated on the oracle's F_HF, Omega and E_L of the
same configurations (1e-9 relative), and a stretched H2 relaxes inward.
"""
import numpy as np
import pytest

import rust_qmc_gb300 as Q
from rust_qmc_gb300 import geometry as G
from tests.helpers import random_configs


def test_steepest_descent_step_projects_and_caps():
    R = np.array([[0.0, 0.0, -0.7], [0.0, 0.0, 0.7], [1.0, 0.0, 0.0]])
    Z = np.array([1.0, 1.0, 6.0])
    F = np.array([[0.0, 0.0, 1.0], [0.0, 0.0, -1.0], [0.5, 0.0, 0.0]])
    R2 = G.steepest_descent_step(R, Z, F, 0.005)
    com = (F * Z[:, None]).sum(0) / Z.sum()
    d = R2 - R
    want = 0.005 * (F - com)
    for i in range(3):
        n = np.linalg.norm(want[i])
        np.testing.assert_allclose(d[i], want[i] * (0.02 / n) if n > 0.02 else want[i], atol=1e-15)
    R3 = G.steepest_descent_step(R, Z, 100.0 * F, 1.0)
    assert np.all(np.linalg.norm(R3 - R, axis=1) <= 0.02 + 1e-15)


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["h2", "ch4_min"])
def test_mean_forces_match_reference_estimators(ctx, oracle, name):
    spec = {"h2": Q.h2_mo, "ch4_min": Q.methane_minimal}[name]()
    sysh = Q.System(ctx, spec)
    cfg = random_configs(spec, 400, seed=41)
    F_o, Om_o = oracle.forces(spec, cfg)
    E_o = oracle.evaluate(spec, cfg)["e_local"]
    n = len(E_o)
    e_mean = E_o.sum() / n
    bare_ref = F_o.sum(0) / n
    zv_ref = bare_ref - 2.0 * ((E_o[:, None, None] * Om_o).sum(0) / n - e_mean * Om_o.sum(0) / n)
    for est, ref in (("bare", bare_ref), ("zv", zv_ref)):
        f, em, _, _ = G.mean_forces(sysh, cfg, est)
        assert abs(em - e_mean) < 1e-9 * max(1.0, abs(e_mean))
        assert np.max(np.abs(f - ref)) < 1e-9 * max(1.0, np.max(np.abs(ref)))


@pytest.mark.gpu
def test_stretched_h2_relaxes_inward(ctx):
    spec = Q.h2_mo()
    R0 = spec.nuc_pos.copy()
    R0[:, 2] = [-0.9, 0.9]                             # bond stretched from 1.4 to 1.8 bohr
    sysh = Q.System(ctx, spec.with_nuclei(R0.reshape(-1)))
    res = G.optimize(sysh, n_samples=65536, n_walkers=8192, n_equilibrate=100, step_size=0.05, max_iterations=3,
                     force_threshold=1e-6, mc_step_size=0.5, estimator="zv", seed=3)
    R = res["final_nuclei"]
    assert R[1, 2] - R[0, 2] < 1.8 - 0.02                # moved inward by more than one capped step
    np.testing.assert_allclose(R.mean(0), R0.mean(0), atol=1e-12)   # no rigid translation
    assert len(res["geometry_history"]) == 4 and np.isfinite(res["final_energy"])
