"""Named single-GPU workloads of the walker kernels, for timing and profiling.

    python -m rust_qmc_gb300.workloads refresh --system ch4_min --walkers 65536
    python -m rust_qmc_gb300.workloads sweeps  --system heg --walkers 16384 --sweeps 8

Each run creates one walker set of the chosen system and precision, seeds it,
refreshes it once (inverse, log|psi| and E_L from the positions), then times
the requested operation with CUDA events on the context stream and prints one
line per repetition.  The first kernel launches of a run are the initial
refresh, which is what a profiler capture with a launch-count limit sees first.
"""
import argparse
import sys

from . import _lib as L
from .api import Context, System, Walkers
from . import systems as S

SYSTEMS = {
    "h2": lambda: S.h2_mo(),
    "li": lambda: S.lithium_atom(reference_quirks=True),
    "ch4_min": lambda: S.methane_minimal(),
    "ch4_gto": lambda: S.methane_gto(),
    "c6h6": lambda: S.benzene_minimal(),
    "heg": lambda: S.electron_gas(),
}
MOVES = {"gauss": L.QMC_MOVE_ONE_GAUSS, "drift": L.QMC_MOVE_ONE_DRIFT}


def main(argv=None):
    p = argparse.ArgumentParser(description=__doc__.splitlines()[0])
    p.add_argument("what", choices=["refresh", "sweeps"])
    p.add_argument("--system", choices=sorted(SYSTEMS), default="ch4_min")
    p.add_argument("--walkers", type=int, default=65536)
    p.add_argument("--precision", choices=["fp32", "fp64"], default="fp32")
    p.add_argument("--sweeps", type=int, default=8, help="sweeps per timed call (sweeps)")
    p.add_argument("--move", choices=sorted(MOVES), default="gauss")
    p.add_argument("--repeat", type=int, default=3)
    a = p.parse_args(argv)
    prec = L.QMC_FP32_REFINE if a.precision == "fp32" else L.QMC_FP64
    ctx = Context(0)
    spec = SYSTEMS[a.system]()
    sysh = System(ctx, spec)
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
