"""Stochastic reconfiguration driver: SROptimizer::optimize
(src/sampling/sr_optimize.rs:252-349) on the device.

Sampling (sr_optimize.rs:104-171) runs as resident walkers on the GPU: n_walkers
chains, all-electron Gaussian proposals of width step_size, n_equilibrate steps,
then n_samples / n_walkers rounds of five steps, each round recording every
walker's configuration.  One batched call evaluates E_L and the parameter
log-derivatives O_p of all recorded configurations and reduces the SR sums
(S = <O O^T> - <O><O>^T, f = <E O> - <E><O>) in compensated FP64 on the device.
The host part is the reference's: S + eps I, dp = -(S + eps I)^-1 f by LU
(falling back to dp = -f), p += clamp(lr dp, -0.3, 0.3), convergence when
|dE| < tolerance after the sixth iteration, and a final sampling pass.

The reference bounds every parameter to [0.05, 10] (sr_optimize.rs:303-305); its
four parameters are Jastrow b and a values.  Here the bound applies to the eight
Jastrow parameters that generalise them; MO rotation angles are not bounded.
"""
import numpy as np

from . import _lib as L
from .api import Walkers

N_JASTROW = 8
PARAM_LO, PARAM_HI, STEP_CLAMP = 0.05, 10.0, 0.3


def sr_direction(S, f, eps):
    """dp solving (S + eps I) dp = -f (sr_optimize.rs:217-241); -f if singular."""
    S = np.asarray(S, dtype=np.float64)
    f = np.asarray(f, dtype=np.float64)
    A = S + eps * np.eye(len(f))
    try:
        return np.linalg.solve(A, -f)
    except np.linalg.LinAlgError:
        return -f


def apply_update(params, dp, learning_rate, n_bounded=N_JASTROW):
    """p += clamp(lr dp, -0.3, 0.3); the first n_bounded parameters are then
    clamped to [0.05, 10] (sr_optimize.rs:296-307)."""
    p = np.array(params, dtype=np.float64, copy=True)
    p += np.clip(learning_rate * np.asarray(dp), -STEP_CLAMP, STEP_CLAMP)
    p[:n_bounded] = np.clip(p[:n_bounded], PARAM_LO, PARAM_HI)
    return p


def sample_configurations(system, n_walkers, n_samples, n_equilibrate, step_size, seed, precision=L.QMC_FP64,
                          steps_between=5):
    """Configurations recorded as sr_optimize.rs:104-171 records them:
    (n_samples // n_walkers) rounds x n_walkers walkers."""
    wk = Walkers(system, n_walkers, precision)
    try:
        wk.init(seed=seed)
        wk.refresh()
        if n_equilibrate:
            wk.sweep(L.QMC_MOVE_ALL_GAUSS, n_equilibrate, 0, seed=seed, step=step_size, count=False)
        rounds = max(1, n_samples // n_walkers)
        out = np.empty((rounds, n_walkers, system.N, 3))
        step0 = n_equilibrate
        for r in range(rounds):
            wk.sweep(L.QMC_MOVE_ALL_GAUSS, steps_between, step0, seed=seed, step=step_size, count=False)
            step0 += steps_between
            out[r] = wk.get_positions()
        return out.reshape(rounds * n_walkers, system.N, 3)
    finally:
        wk.close()


def sr_optimize(system, *, n_samples=5000, n_walkers=20, n_equilibrate=500, max_iterations=50, learning_rate=0.05,
                sr_epsilon=1e-3, tolerance=1e-5, step_size=0.5, seed=1, precision=L.QMC_FP64, verbose=False):
    """Optimise the system's parameters in place; returns the SRResult fields
    (sr_optimize.rs:352-366) as a dict."""
    energy_history, variance_history, param_history = [], [], [system.get_params()]
    prev_energy = np.inf
    for it in range(max_iterations):
        cfg = sample_configurations(system, n_walkers, n_samples, n_equilibrate, step_size,
                                    seed + 7919 * (it + 1), precision)
        _, E, S, f, e_mean = system.logderiv_batch(cfg, sums=True)
        variance = float(np.mean((E - e_mean) ** 2))
        dp = sr_direction(S, f, sr_epsilon)
        energy_history.append(e_mean)
        variance_history.append(variance)
        params = apply_update(system.get_params(), dp, learning_rate)
        system.set_params(params)
        param_history.append(params)
        if verbose:
            print("  Iter %3d: E = %10.5f +/- %.4f Ha, var = %.3f" % (it + 1, e_mean, np.sqrt(variance / len(E)),
                                                                     variance), flush=True)
        if it > 5 and abs(e_mean - prev_energy) < tolerance:
            break
        prev_energy = e_mean
    cfg = sample_configurations(system, n_walkers, n_samples, n_equilibrate, step_size, seed, precision)
    _, E = system.logderiv_batch(cfg)
    final_energy = float(np.mean(E))
    return dict(final_params=system.get_params(), final_energy=final_energy,
                final_variance=float(np.mean((E - final_energy) ** 2)), energy_history=energy_history,
                variance_history=variance_history, param_history=param_history)
