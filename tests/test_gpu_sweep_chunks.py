"""The chunked single-electron sweep of the thread-per-walker shapes
(k_sweep_chunks: taken for FP32 walker sets that give every SM sub-partition
three warps; each 32-walker group's sweeps move between warps every 8 sweeps)
against the one-warp-per-group kernel.  A walker's stream depends only on its
index, so the first 32 768 walkers of a 65 536-walker set (chunked) must end,
bit for bit, where a 32 768-walker set from the same seed ends (one warp per
group for the whole launch)."""
import numpy as np
import pytest

import rust_qmc_gb300 as Q
from rust_qmc_gb300 import _lib as L

pytestmark = pytest.mark.gpu

BIG, SMALL, SWEEPS = 65536, 32768, 24


@pytest.fixture(scope="module")
def ctx():
    c = Q.Context(0)
    yield c
    c.close()


def _run(sysh, W, move, fixed_node=False):
    wk = Q.Walkers(sysh, W, L.QMC_FP32_REFINE)
    wk.init(17)
    wk.refresh()
    acc = wk.sweep(move, SWEEPS, 0, 23, step=0.3, tau=0.01, max_drift=1.0)
    pos = wk.get_positions()
    status = wk.status()
    wk.refresh()
    la, sg, el = wk.state()
    wk.close()
    return acc, pos, sg, status


SYSTEMS = {
    "ch4_min": (lambda: Q.methane_minimal(), 10),
    "ch4_gto": (lambda: Q.methane_gto(), 10),
    "li_ref": (lambda: Q.lithium_atom(reference_quirks=True), 3),
    "h2": (lambda: Q.h2_mo(), 2),
}


@pytest.mark.parametrize("name,move", [("ch4_min", L.QMC_MOVE_ONE_GAUSS), ("ch4_min", L.QMC_MOVE_ONE_DRIFT),
                                       ("ch4_gto", L.QMC_MOVE_ONE_GAUSS), ("li_ref", L.QMC_MOVE_ONE_GAUSS),
                                       ("h2", L.QMC_MOVE_ONE_GAUSS)])
def test_chunked_sweep_matches_one_warp_per_group(ctx, name, move):
    build, n_elec = SYSTEMS[name]
    sysh = Q.System(ctx, build())
    acc_b, pos_b, sg_b, st_b = _run(sysh, BIG, move)
    acc_s, pos_s, sg_s, st_s = _run(sysh, SMALL, move)
    assert st_b == 0 and st_s == 0, (st_b, st_s)          # no flag, no wait that gave up
    assert np.array_equal(pos_b[:SMALL], pos_s)
    assert np.array_equal(sg_b[:SMALL], sg_s)
    # acceptance of the two halves of the big set agree with the small set's rate
    rate_b = acc_b / float(BIG * n_elec * SWEEPS)
    rate_s = acc_s / float(SMALL * n_elec * SWEEPS)
    assert abs(rate_b - rate_s) < 0.01, (rate_b, rate_s)
    assert 0.05 < rate_b < 0.999
