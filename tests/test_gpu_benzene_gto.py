"""The reference's own BenzeneGTO (src/systems/benzene.rs:48-860): 66-AO
6-31G basis, the hand-built MO table, C-H 2.042 bohr, through the warp
kernels on the device.  Tolerances as in test_gpu_parity: FP64 1e-10
relative (1e-9 for gradients and Laplacians), FP32 walkers' refresh E_L
within 1e-6 Ha, trajectories on the oracle's chain."""
import numpy as np
import pytest

import rust_qmc_gb300 as Q
from rust_qmc_gb300 import _lib as L
from tests.helpers import random_configs
from tests.test_gpu_parity import assert_same_chain, rel

pytestmark = pytest.mark.gpu


def test_benzene_gto_eval_matches_oracle(ctx, oracle):
    spec = Q.benzene_gto()
    sysh = Q.System(ctx, spec)
    cfg = oracle.init_positions(spec, 33, seed=3)
    g = sysh.eval_batch(cfg, L.QMC_FP64)
    o = oracle.evaluate(spec, cfg)
    assert np.array_equal(g["sign"], o["sign"])
    assert rel(g["logabs"], o["logabs"]) < 1e-10
    assert rel(g["grad"], o["grad"]) < 1e-9
    assert rel(g["lap"], o["lap"]) < 1e-9
    assert rel(g["e_local"], o["e_local"]) < 1e-10


def test_benzene_gto_log_derivatives_forces(ctx, oracle):
    """OptimizableWfn (benzene.rs:726-756) and ForceCalculator
    (benzene.rs:811-858) at BenzeneGTO::new(2.0, 3.0), the parameters of the
    reference's log-derivative test (benzene.rs:976-1006)."""
    spec = Q.benzene_gto(2.0, 3.0)
    sysh = Q.System(ctx, spec)
    cfg = oracle.init_positions(spec, 24, seed=4)
    O, E, dE = sysh.logderiv_batch(cfg, el_derivs=True)
    assert rel(O, oracle.log_derivatives(spec, cfg)) < 1e-10
    assert rel(E, oracle.evaluate(spec, cfg)["e_local"]) < 1e-9
    assert rel(dE, oracle.el_derivatives(spec, cfg)) < 1e-9
    F, _ = sysh.forces_batch(cfg, omega=False)
    assert rel(F, oracle.forces(spec, cfg)[0]) < 1e-12


@pytest.mark.parametrize("move", [L.QMC_MOVE_ONE_GAUSS, L.QMC_MOVE_ONE_DRIFT])
def test_benzene_gto_fp64_trajectory_matches_oracle(ctx, oracle, move):
    spec = Q.benzene_gto()
    sysh = Q.System(ctx, spec)
    W, n = 128, 2
    wk = Q.Walkers(sysh, W, L.QMC_FP64)
    wk.init(seed=7)
    wk.refresh()
    pos0 = wk.get_positions()
    np.testing.assert_allclose(pos0, oracle.init_positions(spec, W, seed=7), atol=1e-12)
    acc = wk.sweep(move, n, 1, seed=707, step=0.3, tau=0.005, max_drift=1.0)
    got = wk.get_positions()
    want, acc_o, _, mg = oracle.sweeps(spec, pos0, n, 1, move, 707, step=0.3, tau=0.005, max_drift=1.0,
                                       want_energy=False, want_margin=True)
    assert_same_chain(got, want, mg, acc, acc_o)


def test_benzene_gto_fp32_refresh_energy_within_1e6(ctx, oracle):
    spec = Q.benzene_gto()
    sysh = Q.System(ctx, spec)
    wk = Q.Walkers(sysh, 256, L.QMC_FP32_REFINE)
    wk.init(seed=8)
    wk.refresh()
    assert wk.sweep(L.QMC_MOVE_ONE_GAUSS, 8, 0, seed=9, step=0.3) > 0
    _, el = wk.refresh(want_energies=True)
    la, sg, _ = wk.state()
    o = oracle.evaluate(spec, wk.get_positions())
    assert np.max(np.abs(el - o["e_local"])) <= 1e-6
    assert rel(la, o["logabs"]) < 1e-10
    assert np.array_equal(sg, o["sign"])
