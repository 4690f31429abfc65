"""Variance minimisation on the device (JastrowOptimizer::optimize,
src/sampling/optimize.rs:210-304): grid points sampled as walker sets of one
batch give the statistics of standalone runs, and the optimiser keeps the
first point of least variance."""
import numpy as np
import pytest

import rust_qmc_gb300 as Q
from rust_qmc_gb300 import _lib as L
from rust_qmc_gb300 import varmin as V

pytestmark = pytest.mark.gpu


def standalone_stats(ctx, spec, i, *, n_walkers, n_samples, n_equilibrate, sweeps_per_sample, step, precision, seed):
    key = Q.batch_system_seed(seed, i)
    sysh = Q.System(ctx, spec)
    wk = Q.Walkers(sysh, n_walkers, precision)
    wk.init(seed=key)
    wk.refresh()
    step0 = 0
    for _ in range(-(-n_equilibrate // 32)):
        wk.sweep(L.QMC_MOVE_ONE_GAUSS, 32, step0, seed=key, step=step, count=False)
        wk.refresh()
        step0 += 32
    s1 = s2 = 0.0
    rounds = max(1, n_samples // n_walkers)
    for _ in range(rounds):
        wk.sweep(L.QMC_MOVE_ONE_GAUSS, sweeps_per_sample, step0, seed=key, step=step, count=False)
        _, el = wk.refresh(want_energies=True)
        step0 += sweeps_per_sample
        s1 += el.sum()
        s2 += (el * el).sum()
    sysh.close()
    n = rounds * n_walkers
    e = s1 / n
    return e, max(s2 / n - e * e, 0.0)


def test_batched_points_equal_standalone_runs(ctx):
    base = Q.methane_minimal()
    pts = [(1.0, 2.0), (3.0, 1.0), (1.5, 4.0)]
    kw = dict(n_walkers=128, n_samples=512, n_equilibrate=40, sweeps_per_sample=2, step=0.3,
              precision=L.QMC_FP32_REFINE, seed=9)
    got = V.sample_stats(ctx, [V.with_jastrow(base, *p) for p in pts], **kw)
    for i, p in enumerate(pts):
        e, var = standalone_stats(ctx, V.with_jastrow(base, *p), i, **kw)
        assert got[i]["n_samples"] == 512
        assert abs(got[i]["energy"] - e) <= 1e-12 * abs(e)
        assert abs(got[i]["variance"] - var) <= 1e-9 * var
    # different Jastrow factors give different variances
    assert len(set(round(g["variance"], 6) for g in got)) == 3


def test_optimize_scans_both_grids(ctx):
    r = V.optimize(ctx, Q.methane_minimal(), n_walkers=64, n_samples=128, n_equilibrate=32, seed=4)
    vh = np.array(r["variance_history"])
    assert len(vh) == 42 + 49 and len(r["energy_history"]) == 91
    assert np.all(np.isfinite(vh)) and np.all(vh > 0)
    k = int(np.argmin(vh))                      # first occurrence, as the strict < of the reference
    pts = V.coarse_grid() + V.fine_grid(V.coarse_grid()[int(np.argmin(vh[:42]))])
    assert (r["params"]["b_ee"], r["params"]["b_en"]) == pts[k]
    assert r["best_scan_variance"] == vh[k]
    assert np.isfinite(r["final_energy"]) and r["final_variance"] > 0
