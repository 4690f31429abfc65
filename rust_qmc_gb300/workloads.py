"""Named single-GPU workloads of the walker kernels, for timing and profiling.

    python -m rust_qmc_gb300.workloads refresh --system ch4_min --walkers 65536
    python -m rust_qmc_gb300.workloads sweeps  --system heg --walkers 16384 --sweeps 8
    python -m rust_qmc_gb300.workloads batch   --systems 512 --sweeps 8
    python -m rust_qmc_gb300.workloads dmc     --system c6h6 --walkers 16384 --sweeps 4

Each run creates one walker set of the chosen system and precision, seeds it,
refreshes it once (inverse, log|psi| and E_L from the positions), then times
the requested operation with CUDA events on the context stream and prints one
line per repetition.  The first kernel launches of a run are the initial
refresh, which is what a profiler capture with a launch-count limit sees first.
``batch`` instead binds the uneven mix of ``batch_mix`` (one walker set per
system) into one batch and times graph-captured steps of qmc_batch_run_steps;
``dmc`` equilibrates ``--walkers`` with 128 Gaussian sweeps, then times
``--sweeps`` IS-DMC steps (drift-diffusion sweep, E_L, branching and
compaction) per repetition.
"""
import argparse
import sys

import numpy as np

from . import _lib as L
from .api import Batch, Context, System, Walkers
from . import systems as S

SYSTEMS = {
    "h2": lambda: S.h2_mo(),
    "li": lambda: S.lithium_atom(reference_quirks=True),
    "ch4_min": lambda: S.methane_minimal(),
    "ch4_gto": lambda: S.methane_gto(),
    "c6h6": lambda: S.benzene_minimal(),
    "heg": lambda: S.electron_gas(),
}
MOVES = {"gauss": L.QMC_MOVE_ONE_GAUSS, "drift": L.QMC_MOVE_ONE_DRIFT, "all": L.QMC_MOVE_ALL_GAUSS}
BATCH_KINDS = ("h2", "li", "ch4_min", "c6h6", "heg")


def batch_mix(n, seed=5, kinds=BATCH_KINDS):
    """The uneven-batch workload: n systems cycling over H2, Li, CH4 (9 AO),
    benzene and the 54-electron gas (or the given subset), walker counts drawn
    from U{256..4096} by a seeded generator."""
    rng = np.random.default_rng(seed)
    kinds = [kinds[i % len(kinds)] for i in range(n)]
    walkers = [int(w) for w in rng.integers(256, 4097, size=n)]
    return kinds, walkers


def run_dmc(a, ctx, sysh, prec):
    W = a.walkers
    wk = Walkers(sysh, W, prec, capacity=4 * W)
    wk.init(seed=3)
    wk.refresh()
    # VMC equilibration first (the initial Gaussian clouds give E_L spread so
    # wide that branching would empty most of the population)
    for k in range(4):
        wk.sweep(L.QMC_MOVE_ONE_GAUSS, 32, 32 * k, seed=2, step=0.3, count=False)
        wk.refresh()
    e_ref = wk.refresh() / W
    t = 0
    for i in range(a.repeat):
        ctx.synchronize()
        ctx.record(0)
        n_moves = 0
        for _ in range(a.sweeps):
            n_before = wk.W
            n, em = wk.dmc_step(0.005, e_ref, seed=1, step=t, fp64_measure=True, branch_cut=2.0 / np.sqrt(0.005))
            t += 1
            n_moves += n_before * sysh.N
            e_ref = em - 0.5 * np.log(n / W) / 0.005
        ctx.record(1)
        ms = ctx.elapsed_ms(0, 1)
        print("dmc %s W=%d %s: %.3f ms for %d steps  %.3e moves/s  population %d"
              % (a.system, W, a.precision, ms, a.sweeps, n_moves / ms * 1e3, wk.W), flush=True)
    wk.close()


def run_batch(a, ctx, prec):
    kinds, walkers = batch_mix(a.systems, kinds=tuple(a.kinds.split(",")) if a.kinds else BATCH_KINDS)
    specs = {k: SYSTEMS[k]() for k in set(kinds)}
    handles = {k: System(ctx, specs[k]) for k in specs}
    sets = []
    for k, W in zip(kinds, walkers):
        wk = Walkers(handles[k], W, prec)
        wk.init(seed=len(sets) + 1)
        wk.refresh()
        sets.append(wk)
    batch = Batch(ctx, sets)
    moves = sum(W * specs[k].n_elec for k, W in zip(kinds, walkers)) * a.sweeps
    step0 = 0
    for i in range(a.repeat + 1):                  # the first step captures the graph
        ctx.synchronize()
        ctx.record(0)
        batch.run_steps(MOVES[a.move], 1, a.sweeps, step0, seed=1, step=0.3, tau=0.02)
        ctx.record(1)
        step0 += a.sweeps
        ms = ctx.elapsed_ms(0, 1)
        print("batch %d systems, %d walkers, %s: %.3f ms per step (%d sweeps + refresh)  %.3e moves/s%s"
              % (a.systems, sum(walkers), a.precision, ms, a.sweeps, moves / ms * 1e3,
                 "  (graph capture)" if i == 0 else ""), flush=True)
    batch.close()
    for wk in sets:
        wk.close()
    for h in handles.values():
        h.close()


def main(argv=None):
    p = argparse.ArgumentParser(description=__doc__.splitlines()[0])
    p.add_argument("what", choices=["refresh", "sweeps", "batch", "dmc"])
    p.add_argument("--system", choices=sorted(SYSTEMS), default="ch4_min")
    p.add_argument("--walkers", type=int, default=65536)
    p.add_argument("--precision", choices=["fp32", "fp64"], default="fp32")
    p.add_argument("--sweeps", type=int, default=8, help="sweeps per timed call (sweeps)")
    p.add_argument("--move", choices=sorted(MOVES), default="gauss")
    p.add_argument("--repeat", type=int, default=3)
    p.add_argument("--systems", type=int, default=512, help="systems in the uneven batch (batch)")
    p.add_argument("--kinds", default="", help="comma-separated subset of %s (batch)" % ",".join(BATCH_KINDS))
    a = p.parse_args(argv)
    prec = L.QMC_FP32_REFINE if a.precision == "fp32" else L.QMC_FP64
    ctx = Context(0)
    if a.what == "batch":
        run_batch(a, ctx, prec)
        ctx.close()
        return 0
    spec = SYSTEMS[a.system]()
    sysh = System(ctx, spec)
    if a.what == "dmc":
        run_dmc(a, ctx, sysh, prec)
        sysh.close()
        ctx.close()
        return 0
    wk = Walkers(sysh, a.walkers, prec)
    wk.init(seed=3)
    wk.refresh()
    for i in range(a.repeat):
        ctx.synchronize()
        ctx.record(0)
        if a.what == "refresh":
            wk.refresh()
        else:
            wk.sweep(MOVES[a.move], a.sweeps, 1 + i * a.sweeps, seed=1, step=0.3, tau=0.02, count=False)
        ctx.record(1)
        ms = ctx.elapsed_ms(0, 1)
        extra = ""
        if a.what == "sweeps":
            extra = "  %.3e moves/s" % (a.walkers * spec.n_elec * a.sweeps / ms * 1e3)
        print("%s %s W=%d %s: %.3f ms%s" % (a.what, a.system, a.walkers, a.precision, ms, extra), flush=True)
    wk.close()
    sysh.close()
    ctx.close()
    return 0


if __name__ == "__main__":
    sys.exit(main())
