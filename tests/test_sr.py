"""Stochastic reconfiguration driver (rust_qmc_gb300/sr.py) against the
reference's update rules (src/sampling/sr_optimize.rs:176-307).

CPU: the host update (regularised solve, step clamp, parameter bounds).
GPU: the direction computed from the device SR sums equals the reference's
compute_sr_update restated on the oracle's E_L and O_p of the same
configurations (1e-8 relative), and a short optimisation runs end to end.
"""
import numpy as np
import pytest

import rust_qmc_gb300 as Q
from rust_qmc_gb300 import _lib as L
from rust_qmc_gb300 import sr
from tests.helpers import random_configs


def reference_sr_update(E, O, eps):
    """compute_sr_update (sr_optimize.rs:176-246): returns (dp, e_mean, variance)."""
    n = len(E)
    e_mean = E.sum() / n
    variance = ((E - e_mean) ** 2).sum() / n
    o_mean = O.sum(0) / n
    S = O.T @ O / n - np.outer(o_mean, o_mean) + eps * np.eye(O.shape[1])
    f = (E[:, None] * O).sum(0) / n - e_mean * o_mean
    try:
        dp = np.linalg.solve(S, -f)
    except np.linalg.LinAlgError:
        dp = -f
    return dp, e_mean, variance


def test_apply_update_clamps_like_the_reference():
    p = np.array([1.0, 0.06, 9.9, 2.0, 1.0, 1.0, 1.0, 1.0, 0.2, -0.1])
    dp = np.array([100.0, -100.0, 100.0, 1.0, 0, 0, 0, 0, -100.0, 3.0])
    q = sr.apply_update(p, dp, 0.05)
    assert q[0] == pytest.approx(1.3)            # step clamped to +0.3
    assert q[1] == pytest.approx(0.05)           # bound
    assert q[2] == pytest.approx(10.0)           # bound
    assert q[3] == pytest.approx(2.05)
    assert q[8] == pytest.approx(-0.1)           # rotation angle: step clamped, no bound
    assert q[9] == pytest.approx(0.05)


def test_sr_direction_solves_and_falls_back():
    rng = np.random.default_rng(0)
    A = rng.standard_normal((5, 5))
    S = A @ A.T
    f = rng.standard_normal(5)
    dp = sr.sr_direction(S, f, 1e-3)
    np.testing.assert_allclose((S + 1e-3 * np.eye(5)) @ dp, -f, atol=1e-10)
    assert np.array_equal(sr.sr_direction(-1e-3 * np.eye(5), f, 1e-3), -f)


@pytest.mark.gpu
def test_sr_direction_from_device_sums_matches_reference_rule(ctx, oracle):
    spec = Q.methane_minimal()
    spec = spec.with_params(np.concatenate([spec.jas, [0.1, -0.2, 0.05, 0.3]]))
    sysh = Q.System(ctx, spec)
    cfg = random_configs(spec, 600, seed=31)
    _, E, S, f, em = sysh.logderiv_batch(cfg, sums=True)
    dp = sr.sr_direction(S, f, 1e-3)
    Eo = oracle.evaluate(spec, cfg)["e_local"]
    Oo = oracle.log_derivatives(spec, cfg)
    dp_ref, em_ref, var_ref = reference_sr_update(Eo, Oo, 1e-3)
    assert abs(em - em_ref) < 1e-9 * max(1.0, abs(em_ref))
    assert np.max(np.abs(dp - dp_ref)) < 1e-8 * max(1.0, np.max(np.abs(dp_ref)))
    assert float(np.mean((E - em) ** 2)) == pytest.approx(var_ref, rel=1e-9)


@pytest.mark.gpu
def test_sr_optimize_runs(ctx):
    sysh = Q.System(ctx, Q.methane_minimal())
    p0 = sysh.get_params()
    res = sr.sr_optimize(sysh, n_samples=4096, n_walkers=1024, n_equilibrate=40, max_iterations=3,
                         learning_rate=0.05, step_size=0.3, seed=5)
    assert len(res["energy_history"]) == 3 and len(res["param_history"]) == 4
    assert np.all(np.isfinite(res["energy_history"])) and np.isfinite(res["final_energy"])
    p = res["final_params"]
    assert np.all(p[:8] >= 0.05) and np.all(p[:8] <= 10.0)
    assert np.max(np.abs(p - p0)) <= 3 * 0.3 + 1e-12
    assert not np.allclose(p, p0)
