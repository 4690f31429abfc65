"""Twist-averaged electron gas on the device: every Monkhorst-Pack twist runs
as one system of an uneven batch; the averages follow examples/heg_vmc.rs:
178-186.  (Twisted evaluation against the oracle is in test_gpu_parity.)"""
import math

import numpy as np
import pytest

import rust_qmc_gb300 as Q
from rust_qmc_gb300 import _lib as L
from rust_qmc_gb300.twist import twist_average

pytestmark = pytest.mark.gpu


def test_twist_average_2x2x2(ctx):
    r = twist_average(ctx, 2, walkers_per_twist=128, n_steps=128, n_burnin=32, refresh_every=16, seed=3)
    runs = r["runs"]
    assert len(runs) == 8 and r["twists"].shape == (8, 3)
    e = np.array([x["energy"] for x in runs])
    s = np.array([x["error"] for x in runs])
    assert np.all(np.isfinite(e)) and np.all(s >= 0)
    assert all(x["status_flags"] == 0 for x in runs)
    assert r["energy"] == e.sum() / 8
    assert r["error"] == math.sqrt((s * s).sum() / 8)


def test_twist_run_equals_standalone_system(ctx):
    """Twist i of the batch follows the standalone VMC run of that twisted
    system keyed by qmc_batch_system_seed(seed, i)."""
    r = twist_average(ctx, 2, walkers_per_twist=96, n_steps=16, n_burnin=8, refresh_every=16, seed=11)
    th = r["twists"][5]
    sysh = Q.System(ctx, Q.electron_gas(twist=th))
    alone = Q.vmc_run(sysh, n_walkers=96, n_steps=16, n_burnin=8, move_kind=L.QMC_MOVE_ONE_GAUSS, step=2.0,
                      precision=L.QMC_FP32_REFINE, refresh_every=16, seed=Q.batch_system_seed(11, 5))
    assert alone["energy"] == r["runs"][5]["energy"]
    np.testing.assert_array_equal(alone["energies"], r["runs"][5]["energies"])
