"""DMC force estimators (qmc_dmc_run_forces) against replays through the
public walker API (src/sampling/is_dmc.rs:303-380, 479-485, 520-534):

  * forces_mixed equals <F_HF> over the populations that qmc_walkers_dmc_step
    produces step by step with the driver's E_ref feedback;
  * forces_vmc equals <F_HF> over the configurations of the same VMC
    schedule (min(n_walkers, 50) walkers, Gaussian width 0.5, equilibration,
    rounds of five steps);
  * forces_extrapolated = 2 forces_mixed - forces_vmc.

F_HF is the reference's hellmann_feynman_force (src/systems/methane.rs:
1241-1272), restated below in numpy.
"""
import numpy as np
import pytest

import rust_qmc_gb300 as Q
from rust_qmc_gb300 import _lib as L

pytestmark = pytest.mark.gpu

VMC_KEY = 0xD1B54A32D192ED03


def hf_force(pos, R, Z):
    """[W][n_nuc][3] Hellmann-Feynman forces in the reference's convention."""
    W, n = pos.shape[0], len(Z)
    F = np.zeros((W, n, 3))
    for I in range(n):
        d = pos - R[I]
        r = np.linalg.norm(d, axis=2)
        far = r > 1e-10
        inv3 = np.where(far, 1.0 / np.where(far, r, 1.0) ** 3, 0.0)
        F[:, I, :] += Z[I] * (d * inv3[..., None]).sum(1)
        for J in range(n):
            if J != I:
                dr = R[I] - R[J]
                F[:, I, :] -= Z[I] * Z[J] * dr / np.linalg.norm(dr) ** 3
    return F


def replay_dmc(sysh, prec, target, n_steps, n_burnin, tau, every, seed, R, Z):
    wk = Q.Walkers(sysh, target, prec, capacity=4 * target)
    wk.init(seed=seed)
    e_ref = wk.refresh() / target
    total, samples = np.zeros((len(Z), 3)), 0
    for t in range(n_burnin + n_steps):
        n, em = wk.dmc_step(tau, e_ref, seed=seed, step=t, max_drift=1.0, fixed_node=True,
                            fp64_measure=((t + 1) % every) == 0)
        assert n > 0
        if t >= n_burnin:
            total += hf_force(wk.get_positions(), R, Z).sum(0)
            samples += n
        e_ref = em - 0.5 * np.log(n / target) / tau
    wk.close()
    return total / samples


def replay_vmc(sysh, prec, n_walkers, n_equil, n_samples, seed, all_electron, R, Z):
    W = min(n_walkers, 50)
    rounds = max(1, n_samples // W)
    key = seed ^ VMC_KEY
    wk = Q.Walkers(sysh, W, prec)
    wk.init(seed=key)
    wk.refresh()
    mk = L.QMC_MOVE_ALL_GAUSS if all_electron else L.QMC_MOVE_ONE_GAUSS
    step = [0]

    def advance(n):
        if n > 0:
            wk.sweep(mk, n, step[0], seed=key, step=0.5, count=False)
            step[0] += n
            if not all_electron:
                wk.refresh()

    advance(n_equil)
    total = np.zeros((len(Z), 3))
    for _ in range(rounds):
        advance(5)
        total += hf_force(wk.get_positions(), R, Z).sum(0)
    wk.close()
    return total / (rounds * W)


CASES = {
    "h2": (lambda: Q.h2_mo(), L.QMC_FP64, True, 64, 12),
    "ch4_min": (lambda: Q.methane_minimal(), L.QMC_FP32_REFINE, True, 64, 8),
    "c6h6": (lambda: Q.benzene_minimal(), L.QMC_FP32_REFINE, False, 16, 3),
}


@pytest.mark.parametrize("name", sorted(CASES))
def test_dmc_forces_match_replay(ctx, name):
    build, prec, all_electron, target, n_steps = CASES[name]
    spec = build()
    sysh = Q.System(ctx, spec)
    R, Z = np.asarray(spec.nuc_pos, dtype=float), np.asarray(spec.nuc_charge, dtype=float)
    n_burnin, tau, every, seed = 2, 0.01, 2, 2024
    n_equil, n_samples = 6, 120
    got = Q.dmc_run_forces(sysh, n_walkers=target, n_steps=n_steps, n_burnin=n_burnin, tau=tau, precision=prec,
                           refresh_every=every, n_vmc_equilibrate=n_equil, n_vmc_force_samples=n_samples, seed=seed)
    assert got["n_samples"] == n_steps and got["status_flags"] == 0
    plain = Q.dmc_run(sysh, n_walkers=target, n_steps=n_steps, n_burnin=n_burnin, tau=tau, precision=prec,
                      refresh_every=every, seed=seed)
    assert got["energy"] == plain["energy"]
    mixed = replay_dmc(sysh, prec, target, n_steps, n_burnin, tau, every, seed, R, Z)
    vmc = replay_vmc(sysh, prec, target, n_equil, n_samples, seed, all_electron, R, Z)
    scale = np.abs(mixed).max()
    assert np.abs(got["forces_mixed"] - mixed).max() <= 1e-10 * scale
    assert np.abs(got["forces_vmc"] - vmc).max() <= 1e-10 * np.abs(vmc).max()
    assert np.array_equal(got["forces_extrapolated"], 2.0 * got["forces_mixed"] - got["forces_vmc"])

