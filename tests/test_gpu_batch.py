"""Uneven batches (qmc_batch_*): many systems of different shapes, precisions
and walker counts advanced by persistent class launches and CUDA graphs.

Parity bar:
  * a batched sweep of walker set i is bit-identical to the standalone
    qmc_walkers_sweep of that set with Philox key qmc_batch_system_seed(seed, i)
    (same kernels' arithmetic, same counters);
  * the per-set mean E_L of a batched refresh equals the standalone refresh to
    1e-13 relative (the two sum the same per-walker FP64 energies in a
    different order);
  * qmc_batch_run of system i reproduces qmc_vmc_run of that system with its
    batch key, measurement by measurement, to 1e-12 relative;
  * one FP64 member is checked directly against the oracle's sweeps.
"""
import numpy as np
import pytest

import rust_qmc_gb300 as Q
from rust_qmc_gb300 import _lib as L

pytestmark = pytest.mark.gpu

# (builder, walkers): uneven sizes with partial tiles in every class
MEMBERS = [
    ("h2", lambda: Q.h2_mo(), 70),
    ("li_ref", lambda: Q.lithium_atom(reference_quirks=True), 64),
    ("ch4_min", lambda: Q.methane_minimal(), 130),
    ("ch4_gto", lambda: Q.methane_gto(), 65),
    ("c6h6", lambda: Q.benzene_minimal(), 9),
    ("heg", lambda: Q.electron_gas(), 6),
    ("h2_b", lambda: Q.h2_mo(), 1),
]


def _make_sets(ctx, prec, init_seed=21):
    systems, a, b = [], [], []
    for i, (_, build, W) in enumerate(MEMBERS):
        sysh = Q.System(ctx, build())
        systems.append(sysh)
        for group in (a, b):
            wk = Q.Walkers(sysh, W, prec)
            wk.init(seed=init_seed + i)
            wk.refresh()
            group.append(wk)
    return systems, a, b


@pytest.mark.parametrize("prec", [L.QMC_FP64, L.QMC_FP32_REFINE])
@pytest.mark.parametrize("move", [L.QMC_MOVE_ONE_GAUSS, L.QMC_MOVE_ONE_DRIFT])
def test_batch_sweep_matches_standalone(ctx, prec, move):
    systems, a, b = _make_sets(ctx, prec)
    batch = Q.Batch(ctx, a)
    seed, step0, n = 9001, 7, 3
    kw = dict(step=0.3, tau=0.02, max_drift=1.0)
    batch.sweep(move, n, step0, seed, **kw)
    for i, wk in enumerate(b):
        wk.sweep(move, n, step0, seed=Q.batch_system_seed(seed, i), count=False, **kw)
    for i, (wa, wb) in enumerate(zip(a, b)):
        pa, pb = wa.get_positions(), wb.get_positions()
        assert np.array_equal(pa, pb), MEMBERS[i][0]
        assert np.array_equal(wa.state()[1], wb.state()[1]), MEMBERS[i][0]
    e_batch = batch.refresh()
    e_single = np.array([wk.refresh() / wk.W for wk in b])
    np.testing.assert_allclose(e_batch, e_single, rtol=1e-13, atol=0)
    for i, (wa, wb) in enumerate(zip(a, b)):
        la, sa, ea = wa.state()
        lb, sb, eb = wb.state()
        assert np.array_equal(ea, eb) and np.array_equal(la, lb) and np.array_equal(sa, sb), MEMBERS[i][0]
    batch.close()


def test_batch_member_matches_oracle(ctx, oracle):
    """The FP64 CH4 member of a batch against the oracle's reference sweeps."""
    systems, a, _ = _make_sets(ctx, L.QMC_FP64)
    k = [m[0] for m in MEMBERS].index("ch4_min")
    spec = systems[k].spec
    pos0 = a[k].get_positions()
    batch = Q.Batch(ctx, a)
    seed = 4242
    batch.sweep(L.QMC_MOVE_ONE_GAUSS, 2, 10, seed, step=0.3)
    got = a[k].get_positions()
    want, _, _ = oracle.sweeps(spec, pos0, 2, 10, L.QMC_MOVE_ONE_GAUSS, Q.batch_system_seed(seed, k), step=0.3,
                               want_energy=False)
    same = np.all(np.abs(got - want) < 1e-9, axis=(1, 2))
    assert same.mean() >= 0.98, same.mean()
    batch.close()


@pytest.mark.parametrize("prec", [L.QMC_FP64, L.QMC_FP32_REFINE])
def test_batch_graph_steps_match_eager(ctx, prec):
    """Graph-captured steps (device control block, concurrent class branches)
    equal the eager sweep + refresh sequence."""
    systems, a, b = _make_sets(ctx, prec)
    ga, gb = Q.Batch(ctx, a), Q.Batch(ctx, b)
    seed, step0, per, steps = 77, 3, 2, 4
    series = ga.run_steps(L.QMC_MOVE_ONE_DRIFT, steps, per, step0, seed, tau=0.02, max_drift=1.0)
    eager = []
    for k in range(steps):
        gb.sweep(L.QMC_MOVE_ONE_DRIFT, per, step0 + k * per, seed, tau=0.02, max_drift=1.0)
        eager.append(gb.refresh())
    eager = np.array(eager)
    np.testing.assert_array_equal(series, eager)
    for wa, wb in zip(a, b):
        assert np.array_equal(wa.get_positions(), wb.get_positions())
    # a second call replays the cached graph from a new step counter
    s2 = ga.run_steps(L.QMC_MOVE_ONE_DRIFT, 2, per, step0 + steps * per, seed, tau=0.02, max_drift=1.0)
    for k in range(2):
        gb.sweep(L.QMC_MOVE_ONE_DRIFT, per, step0 + (steps + k) * per, seed, tau=0.02, max_drift=1.0)
        np.testing.assert_array_equal(s2[k], gb.refresh())
    ga.close()
    gb.close()


@pytest.mark.parametrize("prec", [L.QMC_FP64, L.QMC_FP32_REFINE])
def test_batch_run_matches_vmc_run(ctx, prec):
    names = ["h2", "li_ref", "ch4_min", "heg"]
    builders = {m[0]: m[1] for m in MEMBERS}
    systems = [Q.System(ctx, builders[n]()) for n in names]
    W = [96, 64, 150, 5]
    kw = dict(n_steps=10, n_burnin=5, move_kind=L.QMC_MOVE_ONE_DRIFT, tau=0.02, max_drift=1.0, precision=prec,
              refresh_every=4)
    seed = 1234
    res = Q.batch_run(ctx, systems, W, seed=seed, **kw)
    for i, (sysh, w) in enumerate(zip(systems, W)):
        single = Q.vmc_run(sysh, n_walkers=w, seed=Q.batch_system_seed(seed, i), **kw)
        assert res[i]["n_samples"] == single["n_samples"] == 3
        np.testing.assert_allclose(res[i]["energies"], single["energies"], rtol=1e-12, atol=0)
        assert res[i]["acceptance_rate"] == single["acceptance_rate"]
        assert res[i]["status_flags"] == 0


def test_batch_binding_defers_walker_release(ctx, qmc_lib):
    systems, a, _ = _make_sets(ctx, L.QMC_FP64)
    batch = Q.Batch(ctx, a[:3])
    victim = a[1]
    assert qmc_lib.qmc_walkers_destroy(victim.h) == L.QMC_OK      # bound: release deferred
    victim.h = None
    batch.sweep(L.QMC_MOVE_ONE_GAUSS, 1, 0, 5, step=0.3)
    e = batch.refresh()
    assert np.all(np.isfinite(e))
    batch.close()                                                 # frees the released set


def test_batch_rejects_bad_arguments(ctx):
    systems, a, _ = _make_sets(ctx, L.QMC_FP64)
    with pytest.raises(Q.QMCError):
        Q.Batch(ctx, [a[0], a[0]])
    batch = Q.Batch(ctx, a[:2])
    with pytest.raises(Q.QMCError):
        batch.sweep(L.QMC_MOVE_ALL_GAUSS, 1, 0, 1, step=0.3)
    with pytest.raises(Q.QMCError):
        batch.sweep(L.QMC_MOVE_ONE_DRIFT, 1, 0, 1, tau=0.0)
    batch.close()
