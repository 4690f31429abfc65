"""Jastrow variance minimisation: JastrowOptimizer::optimize
(src/sampling/optimize.rs:210-304) on the device.

The reference scores every (b_ee, b_en) point of a 7 x 6 coarse grid and then
of a 7 x 7 fine grid (step 0.25 around the best point, b_ee >= 0.25,
b_en >= 0.5) by the variance of E_L over a VMC sample (optimize.rs:110-178:
n_walkers chains, n_equilibrate steps, then n_samples / n_walkers steps that
each record every walker's E_L; population variance), keeps the first point
of least variance and samples it once more.

Here the points of a phase are the walker sets of one batch (qmc_batch_*):
one sweep and one refresh per step advance all of them, the FP64 refresh that
ends each step gives every walker's E_L, and each point's mean, variance and
error over its recorded samples are reduced on the host.  The batch moves
electrons one at a time (Gaussian proposals of width ``step``) where the
reference moves all electrons at once (width 0.5); the sampled distribution,
|psi|^2, is the same.
"""
import numpy as np

from . import _lib as L
from .api import Batch, System, Walkers, batch_system_seed

COARSE_B_EE = (0.5, 1.0, 1.5, 2.0, 3.0, 4.0, 5.0)
COARSE_B_EN = (1.0, 2.0, 3.0, 4.0, 5.0, 6.0)
FINE_STEP = 0.25


def coarse_grid():
    """(b_ee, b_en) points of phase 1 in the reference's loop order (optimize.rs:222-230)."""
    return [(b_ee, b_en) for b_ee in COARSE_B_EE for b_en in COARSE_B_EN]


def fine_grid(best):
    """Phase-2 points around best (optimize.rs:258-265): offsets -3..3 steps of
    0.25, b_ee clamped to >= 0.25 and b_en to >= 0.5."""
    b_ee = [max(best[0] + i * FINE_STEP, 0.25) for i in range(-3, 4)]
    b_en = [max(best[1] + i * FINE_STEP, 0.5) for i in range(-3, 4)]
    return [(x, y) for x in b_ee for y in b_en]


def with_jastrow(spec, b_ee, b_en):
    """MethaneGTO::with_jastrow_params: both spin classes take b_ee, both
    species take b_en; the amplitudes are kept."""
    p = np.asarray(spec.jas, dtype=np.float64).copy()
    p[0] = p[1] = b_ee
    p[4] = p[5] = b_en
    return spec.with_params(np.concatenate([p, np.asarray(spec.rot_angle, dtype=np.float64)]))


def sample_stats(ctx, specs, *, n_walkers=256, n_samples=5000, n_equilibrate=64, sweeps_per_sample=2, step=0.3,
                 precision=L.QMC_FP32_REFINE, seed=1):
    """SamplingStats (energy, variance, error, n_samples) of every system in
    `specs`, all sampled in one batch.  Walker set i is seeded and moved with
    the key qmc_batch_system_seed(seed, i)."""
    systems = [System(ctx, s) for s in specs]
    batch = None
    try:
        wks = [Walkers(s, n_walkers, precision) for s in systems]
        for i, w in enumerate(wks):
            w.init(seed=batch_system_seed(seed, i))
            w.refresh()
        batch = Batch(ctx, wks)
        step0 = 0
        eq_per_step = 32
        n_eq_steps = -(-n_equilibrate // eq_per_step)
        if n_eq_steps:
            batch.run_steps(L.QMC_MOVE_ONE_GAUSS, n_eq_steps, eq_per_step, step0, seed, step=step)
            step0 += n_eq_steps * eq_per_step
        rounds = max(1, n_samples // n_walkers)
        s1 = np.zeros(len(wks))
        s2 = np.zeros(len(wks))
        for _ in range(rounds):
            batch.run_steps(L.QMC_MOVE_ONE_GAUSS, 1, sweeps_per_sample, step0, seed, step=step)
            step0 += sweeps_per_sample
            for i, w in enumerate(wks):
                el = w.state()[2]
                s1[i] += el.sum()
                s2[i] += (el * el).sum()
        n = rounds * n_walkers
        out = []
        for i in range(len(wks)):
            e = s1[i] / n
            var = max(s2[i] / n - e * e, 0.0)
            out.append(dict(energy=e, variance=var, error=float(np.sqrt(var / n)), n_samples=n))
        return out
    finally:
        if batch is not None:
            batch.close()
        for s in systems:
            s.close()


def optimize(ctx, spec, *, n_walkers=256, n_samples=5000, n_equilibrate=64, sweeps_per_sample=2, step=0.3,
             precision=L.QMC_FP32_REFINE, seed=1, verbose=False):
    """OptimizationResult fields (optimize.rs:29-40) as a dict; `spec` is a
    Jastrow3 system (methane_gto / methane_minimal) whose (b_ee, b_en) are varied."""
    kw = dict(n_walkers=n_walkers, n_samples=n_samples, n_equilibrate=n_equilibrate,
              sweeps_per_sample=sweeps_per_sample, step=step, precision=precision)
    energy_history, variance_history = [], []
    best, best_var, best_e = (float(spec.jas[0]), float(spec.jas[4])), np.inf, 0.0
    for phase, points in (("coarse", coarse_grid()), ("fine", None)):
        if points is None:
            points = fine_grid(best)
        stats = sample_stats(ctx, [with_jastrow(spec, *p) for p in points], seed=seed + (0 if phase == "coarse" else 1),
                             **kw)
        for p, st in zip(points, stats):
            energy_history.append(st["energy"])
            variance_history.append(st["variance"])
            if verbose:
                print("  b_ee=%.2f, b_en=%.2f: E=%8.4f +/- %.4f, var=%.2f" % (p[0], p[1], st["energy"], st["error"],
                                                                          st["variance"]), flush=True)
            if st["variance"] < best_var:
                best, best_var, best_e = p, st["variance"], st["energy"]
    final = sample_stats(ctx, [with_jastrow(spec, *best)], seed=seed + 2, **kw)[0]
    return dict(params=dict(b_ee=best[0], b_en=best[1]), final_energy=final["energy"],
                final_variance=final["variance"], energy_history=energy_history, variance_history=variance_history,
                best_scan_energy=best_e, best_scan_variance=best_var)
