"""Twist-averaged boundary conditions for the electron gas: the twist loop of
examples/heg_vmc.rs:114-187 over HomogeneousElectronGas::new_with_twist_and_form
(src/systems/heg.rs:131-232), on the device.

Every Monkhorst-Pack twist is its own system (its orbital wave vectors shifted
by theta 2 pi / L); all of them run as one uneven batch (qmc_batch_run: one
sweep and one refresh per step over every twist's walker tiles), so a 3x3x3 grid
costs one set of launches, not 27 runs.  The reference runs each twist with
its all-electron MCMCSimulation; the electron gas kernels here move one
electron at a time, with Gaussian proposals of width ``step``.

Averages are the reference's (heg_vmc.rs:178-186): E = sum_t E_t / n and the
quoted error sqrt(sum_t err_t^2 / n); ``error_of_mean`` adds the standard
error of the twist average, sqrt(sum_t err_t^2) / n.
"""
import math

import numpy as np

from . import _lib as L
from .api import System, batch_run
from .systems import electron_gas, monkhorst_pack_grid


def hartree_fock_energy(rs):
    """Hartree-Fock energy per electron of the paramagnetic electron gas
    (HomogeneousElectronGas::hartree_fock_energy, src/systems/heg.rs:819-831):
    (3/5) k_F^2 / 2 - 3 k_F / (4 pi) with k_F = (9 pi / 4)^(1/3) / r_s."""
    kf = (9.0 * math.pi / 4.0) ** (1.0 / 3.0) / rs
    return 0.3 * kf * kf - 3.0 * kf / (4.0 * math.pi)


def correlation_energy(rs):
    """Perdew-Zunger fit of the Ceperley-Alder correlation energy per electron
    (paramagnetic), the reference value the twist example prints
    (src/systems/heg.rs:834-849): gamma / (1 + beta1 sqrt(r_s) + beta2 r_s)
    for r_s >= 1, A ln r_s + B + C r_s ln r_s + D r_s below."""
    if rs >= 1.0:
        return -0.1423 / (1.0 + 1.0529 * math.sqrt(rs) + 0.3334 * rs)
    return 0.0311 * math.log(rs) - 0.048 + 0.0020 * rs * math.log(rs) - 0.0116 * rs


def average_twists(energies, errors):
    """(E, reference error, standard error of the mean) over the twists."""
    e = np.asarray(energies, dtype=np.float64)
    s = np.asarray(errors, dtype=np.float64)
    n = len(e)
    if n == 0:
        raise ValueError("no twists")
    total_var = float((s * s).sum())
    return float(e.sum() / n), math.sqrt(total_var / n), math.sqrt(total_var) / n


def twist_average(ctx, n_grid, *, walkers_per_twist, n_steps, n_burnin=0, step=2.0, precision=L.QMC_FP32_REFINE,
                  refresh_every=16, seed=1, n_elec=54, **gas):
    """VMC of the electron gas averaged over an n_grid^3 Monkhorst-Pack grid.

    ``gas`` passes through to ``electron_gas`` (rs, F, form, reference_quirks,
    alpha_L, kmax).  Returns the averages, per-electron values, the twists
    and each twist's run result."""
    twists = monkhorst_pack_grid(n_grid)
    systems = [System(ctx, electron_gas(n_elec=n_elec, twist=t, **gas)) for t in twists]
    try:
        runs = batch_run(ctx, systems, [walkers_per_twist] * len(systems), n_steps=n_steps, n_burnin=n_burnin,
                         move_kind=L.QMC_MOVE_ONE_GAUSS, step=step, precision=precision,
                         refresh_every=refresh_every, seed=seed)
    finally:
        for s in systems:
            s.close()
    e, err, err_mean = average_twists([r["energy"] for r in runs], [r["error"] for r in runs])
    rs = gas.get("rs", 4.0)
    # the reference values printed beside the result (heg_vmc.rs:137-145)
    e_hf, e_c = hartree_fock_energy(rs), correlation_energy(rs)
    return dict(energy=e, error=err, error_of_mean=err_mean, energy_per_electron=e / n_elec,
                error_per_electron=err / n_elec, twists=twists, runs=runs,
                hartree_fock_per_electron=e_hf, correlation_per_electron=e_c,
                expected_total_per_electron=e_hf + e_c)
