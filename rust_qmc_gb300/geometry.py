"""Geometry optimisation with VMC forces: GeometryOptimizer::optimize
(src/sampling/geometry_opt.rs:105-347) on the device.

Sampling is the reference's (geometry_opt.rs:114-172): n_walkers chains of
all-electron Gaussian proposals (width mc_step_size), n_equilibrate steps, then
n_samples / n_walkers rounds of five steps, each round recording every walker.
Hellmann-Feynman forces, the nuclear log-derivatives Omega_I = d ln|psi| / dR_I
and E_L of all recorded configurations come from two batched device calls.

Estimators (geometry_opt.rs:176-216, force_variance.rs):
  bare  F_I = <F_I^HF>;
  zero variance (Assaraf-Caffarel)  F_I = <F_I^HF> - 2 (<E_L Omega_I> - <E_L><Omega_I>).
Step (geometry_opt.rs:284-309): the charge-weighted mean force is removed,
R_I += step_size F_I with each displacement capped at 0.02 bohr; converged when
max |F_I| < force_threshold.  A final sampling pass gives the final energy.
"""
import numpy as np

from . import _lib as L
from .sr import sample_configurations

MAX_DISPLACEMENT = 0.02


def mean_forces(system, cfg, estimator="zv"):
    """(mean forces [n_nuc][3], mean E_L, error of E_L, force variance [n_nuc])
    over configurations cfg (geometry_opt.rs:176-216)."""
    f_hf, omega = system.forces_batch(cfg)
    E = system.eval_batch(cfg, L.QMC_FP64)["e_local"]
    n = len(E)
    e_mean = E.sum() / n
    e_var = (E * E).sum() / n - e_mean * e_mean
    error = np.sqrt(max(e_var, 0.0) / n)
    f_mean = f_hf.sum(0) / n
    if estimator == "zv":
        cov = (E[:, None, None] * omega).sum(0) / n - e_mean * omega.sum(0) / n
        forces = f_mean - 2.0 * cov
    elif estimator == "bare":
        forces = f_mean
    else:
        raise ValueError("estimator must be 'zv' or 'bare'")
    f_var = np.maximum((f_hf * f_hf).sum(2).sum(0) / n - (f_mean * f_mean).sum(1), 0.0)
    return forces, e_mean, error, f_var


def steepest_descent_step(nuclei, charges, forces, step_size):
    """R_I += alpha (F_I - F_com), |displacement| <= 0.02 bohr (geometry_opt.rs:284-309)."""
    R = np.array(nuclei, dtype=np.float64, copy=True).reshape(-1, 3)
    Z = np.asarray(charges, dtype=np.float64)
    F = np.asarray(forces, dtype=np.float64).reshape(-1, 3)
    com = (F * Z[:, None]).sum(0) / Z.sum()
    for i in range(len(R)):
        d = step_size * (F[i] - com)
        norm = np.linalg.norm(d)
        R[i] += d * (MAX_DISPLACEMENT / norm) if norm > MAX_DISPLACEMENT else d
    return R


def optimize(system, *, n_samples=5000, n_walkers=20, n_equilibrate=500, step_size=0.005, max_iterations=50,
             force_threshold=0.05, mc_step_size=0.5, estimator="zv", seed=1, precision=L.QMC_FP64, verbose=False):
    """Relax the system's nuclei in place; returns the GeometryOptResult fields
    (geometry_opt.rs:311-334) as a dict."""
    energy_history, force_history = [], []
    geometry_history = [system.get_nuclei().reshape(-1, 3).copy()]
    for it in range(max_iterations):
        cfg = sample_configurations(system, n_walkers, n_samples, n_equilibrate, mc_step_size,
                                    seed + 104729 * (it + 1), precision)
        forces, e_mean, error, _ = mean_forces(system, cfg, estimator)
        max_force = float(np.max(np.linalg.norm(forces, axis=1)))
        energy_history.append(e_mean)
        force_history.append(max_force)
        if verbose:
            print("  Step %3d: E = %10.5f +/- %.4f Ha, max|F| = %.4f Ha/Bohr" % (it + 1, e_mean, error, max_force),
                  flush=True)
        if max_force < force_threshold:
            break
        R = steepest_descent_step(system.get_nuclei(), system.get_charges(), forces, step_size)
        system.set_nuclei(R)
        geometry_history.append(R)
    cfg = sample_configurations(system, n_walkers, n_samples, n_equilibrate, mc_step_size, seed, precision)
    _, final_energy, _, _ = mean_forces(system, cfg, estimator)
    return dict(final_nuclei=system.get_nuclei().reshape(-1, 3), final_energy=final_energy,
                final_max_force=force_history[-1] if force_history else 0.0, energy_history=energy_history,
                force_history=force_history, geometry_history=geometry_history, force_estimator=estimator)
