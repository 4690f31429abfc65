"""Step-size and time-step adaptation of the VMC samplers on the device.

MCMCSimulation::adapt_step_size (src/sampling/vmc.rs:122-128) and
DriftDiffusionVMC::adapt_time_step (vmc.rs:397-402) run every
adaptation_interval steps through burn-in and production (vmc.rs:85-88,
423-428, 458-463).  qmc_vmc_run applies them on the host between launches from
the device's acceptance counts.  The replays below drive the same kernels
through the public walker API, apply the reference's rule in Python to the
acceptance each window returns, and must reproduce the driver's energy series
and final step exactly."""
import math

import numpy as np
import pytest

import rust_qmc_gb300 as Q
from rust_qmc_gb300 import _lib as L

pytestmark = pytest.mark.gpu


def mcmc_rule(step, rate, target, lo, hi):
    """vmc.rs:122-128."""
    return min(hi, max(lo, step * math.sqrt(rate / target)))


def drift_rule(tau, rate, target, lo, hi):
    """vmc.rs:397-402 (gentle factor clamped to [0.8, 1.2])."""
    return min(hi, max(lo, tau * min(1.2, max(0.8, math.sqrt(rate / target)))))


def test_mcmc_step_adaptation_replays_reference_rule(ctx):
    sysh = Q.System(ctx, Q.h2_mo())
    W, n, burn, iv = 512, 600, 200, 100
    r = Q.vmc_run(sysh, n_walkers=W, n_steps=n, n_burnin=burn, move_kind=L.QMC_MOVE_ALL_GAUSS, step=0.2, seed=9,
                  target_acceptance=0.5, adaptation_interval=iv, min_step=0.1, max_step=3.0)
    wk = Q.Walkers(sysh, W, L.QMC_FP64)
    wk.init(seed=9)
    wk.refresh()
    step, window, series, steps = 0.2, 0, [], []
    for t in range(burn + n):
        window += wk.sweep(L.QMC_MOVE_ALL_GAUSS, 1, t, seed=9, step=step)
        if t >= burn:
            series.append(wk.state()[2].mean())
        if (t + 1) % iv == 0:
            step = mcmc_rule(step, window / float(iv * W), 0.5, 0.1, 3.0)
            steps.append(step)
            window = 0
    assert len(set(np.round(steps, 12))) > 1                  # the step really moved
    assert r["final_step"] == pytest.approx(step, rel=1e-14)
    np.testing.assert_allclose(r["energies"], series, rtol=1e-12, atol=1e-12)
    wk.close()


def test_drift_time_step_adaptation_replays_reference_rule(ctx):
    sysh = Q.System(ctx, Q.methane_minimal())
    W, n, burn, iv, every = 1024, 240, 120, 40, 8
    kw = dict(n_walkers=W, n_steps=n, n_burnin=burn, move_kind=L.QMC_MOVE_ONE_DRIFT, tau=0.02, max_drift=1.0,
              precision=L.QMC_FP64, refresh_every=every, seed=21, target_acceptance=0.5, adaptation_interval=iv)
    r = Q.vmc_run(sysh, **kw)
    wk = Q.Walkers(sysh, W, L.QMC_FP64)
    wk.init(seed=21)
    wk.refresh()
    N = sysh.spec.n_elec
    tau, window, series, t, since = 0.02, 0, [], 0, 0
    total = burn + n
    while t < total:
        end = min(total, burn if t < burn else total, t + (every - since), (t // iv + 1) * iv)
        window += wk.sweep(L.QMC_MOVE_ONE_DRIFT, end - t, t, seed=21, step=1.0, tau=tau, max_drift=1.0)
        since += end - t
        t = end
        if since == every or t == burn or t == total:
            e_sum = wk.refresh()
            if t > burn:
                series.append(e_sum / W)
            since = 0
        if t % iv == 0:
            tau = drift_rule(tau, window / float(iv * N * W), 0.5, 0.001, 0.05)
            window = 0
    assert r["final_step"] == pytest.approx(tau, rel=1e-14)
    np.testing.assert_allclose(r["energies"], series, rtol=1e-12, atol=1e-12)
    wk.close()


def test_adaptation_drives_acceptance_to_target(ctx):
    """The adapted width of single-electron Gaussian moves brings the
    production acceptance of CH4 to the 0.5 target from a start at 0.05 bohr
    (acceptance near 1), and the all-electron Li step (the reference's
    main.rs:51-59 settings) likewise."""
    sysh = Q.System(ctx, Q.methane_minimal())
    r = Q.vmc_run(sysh, n_walkers=4096, n_steps=400, n_burnin=400, move_kind=L.QMC_MOVE_ONE_GAUSS, step=0.05,
                  precision=L.QMC_FP32_REFINE, refresh_every=8, seed=4, target_acceptance=0.5,
                  adaptation_interval=20, min_step=0.01, max_step=3.0)
    assert abs(r["acceptance_rate"] - 0.5) < 0.03, r["acceptance_rate"]
    assert r["final_step"] > 0.05
    li = Q.System(ctx, Q.lithium_atom(reference_quirks=True))
    r2 = Q.vmc_run(li, n_walkers=4096, n_steps=1000, n_burnin=500, move_kind=L.QMC_MOVE_ALL_GAUSS, step=1.0,
                   seed=6, target_acceptance=0.5, adaptation_interval=100, min_step=0.2, max_step=2.0)
    assert abs(r2["acceptance_rate"] - 0.5) < 0.03, r2["acceptance_rate"]
