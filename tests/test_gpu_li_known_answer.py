"""The reference's one published full local-energy answer, reproduced on the
device: the Li atom, STO-7G determinant (src/wavefunction/slater.rs:48-145)
times Jastrow2 with F = 1 (src/main.rs:34-49), sampled by MCMCSimulation's
all-electron Gaussian moves with step adaptation (target acceptance 0.5,
every 100 steps, step in [0.2, 2.0], start 1.0: main.rs:51-59).  The
reference's README (README.md:34-44) reports -2.029792 +- 0.000148 Ha and, on
a second run, -2.029456 +- 0.000148 Ha, both with its Jastrow2 Laplacian
without cross terms (quirk B), which lithium_atom(reference_quirks=True)
reproduces."""
import numpy as np
import pytest

import rust_qmc_gb300 as Q
from rust_qmc_gb300 import _lib as L

pytestmark = pytest.mark.gpu

README_E, README_SIGMA = -2.0298, 1.48e-4


def test_li_vmc_energy_matches_reference_readme(ctx):
    sysh = Q.System(ctx, Q.lithium_atom(reference_quirks=True))
    r = Q.vmc_run(sysh, n_walkers=131072, n_steps=4000, n_burnin=1000, move_kind=L.QMC_MOVE_ALL_GAUSS, step=1.0,
                  seed=2024, target_acceptance=0.5, adaptation_interval=100, min_step=0.2, max_step=2.0)
    assert 0 < r["error"] <= 1.5e-4, r
    assert abs(r["acceptance_rate"] - 0.5) < 0.05, r
    assert abs(r["energy"] - README_E) < 3 * np.hypot(r["error"], README_SIGMA), r
