"""The Li atom of the reference's main program on the device: STO-7G
determinant (src/wavefunction/slater.rs:48-145) times Jastrow2 with F = 1
(src/main.rs:34-49), sampled by MCMCSimulation's all-electron Gaussian moves
with the main program's step adaptation (target acceptance 0.5 every 100
steps, step in [0.2, 2.0] from 1.0: main.rs:51-59), E_L with the reference's
Jastrow2 Laplacian without cross terms (quirk B, reproduced by
lithium_atom(reference_quirks=True)).

The reference's README (README.md:34-44) reports -2.029792 +- 0.000148 Ha
for this run.  The reference's code as it stands gives a different energy:
its E_L and its all-electron Markov chain are reproduced here configuration
for configuration (the trajectory test below against the oracle, whose E_L
formulas are pinned to the reference's Jastrow2 and STO expressions and to
finite differences), and the sampled energy comes out near -2.99 Ha.  The
README's output block is not the current main program's output either (it
prints "Final energy" and a "Binding energy" of (E + 1 Ha) in eV; the
program prints "Energy" in Ha and E x 27.211 eV), so it records an earlier
version of the code.  The energy test therefore pins the sampler's
behaviour (adapted acceptance, error bar) and a band around the value the
reference's current code gives, and does not compare with the README."""
import numpy as np
import pytest

import rust_qmc_gb300 as Q
from rust_qmc_gb300 import _lib as L
from tests.test_gpu_parity import assert_same_chain

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("move", [L.QMC_MOVE_ALL_GAUSS, L.QMC_MOVE_ALL_BOX])
def test_li_all_electron_chain_matches_oracle(ctx, oracle, move):
    spec = Q.lithium_atom(reference_quirks=True)
    sysh = Q.System(ctx, spec)
    W, n = 256, 30
    wk = Q.Walkers(sysh, W, L.QMC_FP64)
    wk.init(seed=31)
    wk.refresh()
    pos0 = wk.get_positions()
    acc = wk.sweep(move, n, 0, seed=515, step=0.7)
    got = wk.get_positions()
    want, acc_o, el_o, mg = oracle.sweeps(spec, pos0, n, 0, move, 515, step=0.7, want_margin=True)
    same = assert_same_chain(got, want, mg, acc, acc_o)
    _, _, el = wk.state()
    np.testing.assert_allclose(el[same], el_o[same], rtol=1e-10, atol=1e-10)


def test_li_vmc_with_reference_main_settings(ctx):
    sysh = Q.System(ctx, Q.lithium_atom(reference_quirks=True))
    r = Q.vmc_run(sysh, n_walkers=131072, n_steps=4000, n_burnin=1000, move_kind=L.QMC_MOVE_ALL_GAUSS, step=1.0,
                  seed=2024, target_acceptance=0.5, adaptation_interval=100, min_step=0.2, max_step=2.0)
    assert abs(r["acceptance_rate"] - 0.5) < 0.01, r
    assert 0.2 <= r["final_step"] <= 2.0
    assert 0 < r["error"] <= 5e-4, r
    assert -3.05 < r["energy"] < -2.93, r
