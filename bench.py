#!/usr/bin/env python3
"""Walker-moves/s of the CH4 single-electron VMC workload on one GB300.

Workload (one "step"): 65 536 walkers of the 9-function CH4 system
(10 electrons, 5x5 spin determinants, Jastrow with one-body term), 64 sweeps
of single-electron Gaussian moves of width 0.3 bohr (640 proposals per
walker) followed by the FP64 refresh: inverse Slater matrices and log|psi|
rebuilt in FP64 and the FP64 local energy of every walker, reduced with a
compensated sum.  The headline form keeps walkers in FP32 (FP32+refine);
the plain FP64 form runs the same schedule with FP64 walkers.

value  = walker-moves/s with walker state resident in HBM, timed by CUDA
         events around each step (L2 flushed between steps, outside timing)
e2e    = same metric through the C ABI with host buffers: every step uploads
         the walkers' positions from pinned host memory, rebuilds their
         inverse Slater matrices (qmc_walkers_rebuild_inverse), sweeps, and
         reads back the refreshed E_L of every walker.
--impl reference times the oracle's restatement of the reference algorithm
(full re-evaluation of psi per proposal) on the host cores.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "walker-moves/s on 1 GB300, FP32+refine vs plain FP64, at <=1e-6 Ha E_L error"
UNIT = "walker-moves/s"
N_ELEC, N_UP, N_NUC = 10, 5, 5


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=10)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    p.add_argument("--walkers", type=int, default=65536)
    p.add_argument("--sweeps", type=int, default=64, help="sweeps per step (= FP64 refresh period)")
    p.add_argument("--step-size", type=float, default=0.3)
    p.add_argument("--fp64-steps", type=int, default=0, help="steps of the plain FP64 form (0: --steps)")
    p.add_argument("--no-fp64-form", action="store_true")
    p.add_argument("--no-configs", action="store_true", help="skip the other workloads (H2, CH4 SR, benzene, batch)")
    p.add_argument("--batch-systems", type=int, default=512)
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--cpu-seconds", type=float, default=12.0)
    return p.parse_args()


def dist_env():
    return int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")), int(os.environ.get("LOCAL_RANK", "0"))


class Replicas:
    """The host-side exchange of an N-replica run (one process per GPU, each
    advancing its own walkers): a gloo group used only for the barriers
    around the timed region, the max-over-ranks time and the summed move
    counts.  The walkers themselves never cross ranks (no data-path
    collective)."""

    def __init__(self, world):
        self.pg = None
        if world > 1:
            import torch.distributed as dist
            dist.init_process_group("gloo")
            self.pg = dist

    def barrier(self):
        if self.pg:
            self.pg.barrier()

    def _reduce(self, x, op):
        if not self.pg:
            return x
        import torch
        t = torch.tensor([x], dtype=torch.float64)
        self.pg.all_reduce(t, op=op)
        return float(t.item())

    def max(self, x):
        return self._reduce(x, self.pg.ReduceOp.MAX if self.pg else None)

    def sum(self, x):
        return self._reduce(x, self.pg.ReduceOp.SUM if self.pg else None)

    def close(self):
        if self.pg:
            self.pg.destroy_process_group()
            self.pg = None


def replica_seed(base, rank):
    """Disjoint Philox keys per replica."""
    return base + 2 + 1000 * rank


def whole_job_rate(moves_this_rank, seconds_this_rank, group):
    """Moves of all ranks over the slowest rank's time."""
    return group.sum(moves_this_rank) / group.max(seconds_this_rank)


class ClockSampler:
    """nvidia-smi sampling of SM clocks and throttle reasons during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu):
        self.gpu, self.rows, self.proc = gpu, [], None

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.Q,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([x.strip() for x in line.split(",")])

    def stop(self):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
        out = {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": len(self.rows)}
        sm, mx = [], []
        reasons = set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in self.rows:
            try:
                sm.append(float(r[1]))
                mx.append(float(r[2]))
                for n, v in zip(names, r[5:9]):
                    if v.strip().lower() == "active":
                        reasons.add(n)
            except (ValueError, IndexError):
                pass
        if sm:
            out["sm_mhz"] = statistics.median(sm)
            out["sm_max_mhz"] = max(mx)
        out["reasons"] = sorted(reasons)
        return out


def measured_peak_hbm():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        d = json.load(open(p))
        for k in ("hbm_gbs", "hbm_GBps", "hbm"):
            if k in d:
                v = d[k]
                return float(v["value"] if isinstance(v, dict) else v), "measured"
    except Exception:
        pass
    return 6800.0, "fallback"


def cpu_baseline(spec, seconds, threads=1, walkers_hint=8):
    """Oracle (reference algorithm) single-electron sweeps on the host."""
    from oracle import oracle as O
    import numpy as np
    pos = O.init_positions(spec, max(walkers_hint, threads), seed=1)
    t0 = time.perf_counter()
    O.sweeps(spec, pos, 1, 0, 2, 3, step=0.3, threads=threads, want_energy=False)
    dt = time.perf_counter() - t0
    per_walker = dt / pos.shape[0]
    W = max(threads, int(seconds / max(per_walker, 1e-9)))
    pos = O.init_positions(spec, W, seed=2)
    t0 = time.perf_counter()
    O.sweeps(spec, pos, 1, 0, 2, 3, step=0.3, threads=threads, want_energy=False)
    dt = time.perf_counter() - t0
    moves = W * N_ELEC
    return moves / dt, W, dt


def held_out_accuracy(spec, pos, el_dev):
    """Per-configuration E_L error of the device path: the oracle's FP64 E_L
    at the held-out (FP32-valued) configurations against the device's."""
    from oracle import oracle as O
    import numpy as np
    t0 = time.perf_counter()
    ref = O.evaluate(spec, pos)["e_local"]
    dt = time.perf_counter() - t0
    err = np.abs(el_dev - ref)
    return {"configurations": int(len(pos)), "max_abs_dEL_Ha": float(err.max()),
            "median_abs_dEL_Ha": float(np.median(err)), "within_1e-6_Ha": bool(err.max() <= 1e-6),
            "oracle_eval_s": dt}


def oracle_sweep_rate(spec, move_kind, seconds, step=0.3, tau=0.005, threads=1, seed=1):
    """Bounded sample of the oracle's reference-algorithm sweeps (full psi
    re-evaluation per proposal): single-electron moves/s, or all-electron
    walker steps/s for move kinds 0 and 1."""
    from oracle import oracle as O
    per = spec.n_elec if move_kind >= 2 else 1
    pos = O.init_positions(spec, max(2, threads), seed=seed)
    t0 = time.perf_counter()
    O.sweeps(spec, pos, 1, 0, move_kind, 3, step=step, tau=tau, threads=threads, want_energy=False)
    dt = time.perf_counter() - t0
    W = max(threads, int(seconds / max(dt / pos.shape[0], 1e-9)))
    pos = O.init_positions(spec, W, seed=seed + 1)
    t0 = time.perf_counter()
    O.sweeps(spec, pos, 1, 0, move_kind, 3, step=step, tau=tau, threads=threads, want_energy=False)
    dt = time.perf_counter() - t0
    return {"value": W * per / dt, "cores": threads, "kind": "port",
            "sample": "%d walkers x 1 %s, %.2f s" % (W, "sweep" if move_kind >= 2 else "step", dt)}


def _events_ms(ctx, fn):
    ctx.synchronize()
    ctx.record(5)
    fn()
    ctx.record(6)
    return ctx.elapsed_ms(5, 6)


def other_configs(ctx, args, fp32_peak, fp64_peak, cpu=True, cpu_seconds=2.0):
    """The other workloads of the scope, one key each, with device time from
    CUDA events on the context stream (end-to-end host time for the SR batch,
    whose C call takes host buffers), a roofline fraction from the library's
    algorithmic counts and a bounded oracle CPU sample beside it."""
    import numpy as np
    import rust_qmc_gb300 as Q
    from rust_qmc_gb300 import _lib as L
    from rust_qmc_gb300.workloads import batch_mix, SYSTEMS
    out = {}

    # H2 all-electron VMC: 4096 walkers, uniform box of 1.0 bohr, 500 + 2000 steps, FP64
    spec = Q.h2_mo()
    sysh = Q.System(ctx, spec)
    wk = Q.Walkers(sysh, 4096, L.QMC_FP64)
    wk.init(seed=0x51A7E5 + 1)
    wk.refresh()
    wk.sweep(L.QMC_MOVE_ALL_BOX, 500, 0, seed=0x51A7E5 + 1, step=1.0, count=False)
    ms = _events_ms(ctx, lambda: wk.sweep(L.QMC_MOVE_ALL_BOX, 2000, 500, seed=0x51A7E5 + 1, step=1.0, count=False))
    wk.close()
    r = Q.vmc_run(sysh, n_walkers=4096, n_steps=2000, n_burnin=500, move_kind=L.QMC_MOVE_ALL_BOX, step=1.0,
                  seed=0x51A7E5 + 1)
    c = Q.roofline_model(spec, L.QMC_FP64, r["acceptance_rate"])
    v = 4096 * 2000 / (ms / 1e3)
    tf = v * c["refresh_flops"] / 1e12
    out["h2_vmc"] = {"workload": "H2 LCAO-Jastrow, 4096 walkers, 2000 all-electron box steps of 1.0 bohr after 500, "
                                 "FP64", "value": v, "unit": "walker-moves/s (all-electron proposals)",
                     "electron_moves_per_s": 2 * v, "ms": ms, "energy": r["energy"], "error": r["error"],
                     "acceptance": r["acceptance_rate"],
                     "roofline": {"bound": "fp64_simt", "achieved": tf, "peak": fp64_peak, "unit": "TFLOP/s",
                                  "frac": tf / fp64_peak if fp64_peak else None,
                                  "flops_per_move": c["refresh_flops"]}}
    if cpu:
        out["h2_vmc"]["cpu_baseline"] = oracle_sweep_rate(spec, L.QMC_MOVE_ALL_BOX, cpu_seconds, step=1.0)
    sysh.close()

    # CH4 SR gradient batch: 65536 walkers, P = 12, O, E_L, dE_L/dp and the SR sums
    spec = Q.methane_minimal()
    spec = spec.with_params(np.concatenate([spec.jas, [0.1, -0.2, 0.05, 0.3]]))
    sysh = Q.System(ctx, spec)
    wk = Q.Walkers(sysh, 65536, L.QMC_FP32_REFINE)
    wk.init(seed=0x51A7E5 + 3)
    wk.refresh()
    wk.sweep(L.QMC_MOVE_ONE_GAUSS, 64, 0, seed=0x51A7E5 + 3, step=0.3, count=False)
    pos = wk.get_positions()
    wk.close()
    sysh.logderiv_batch(pos, sums=True, el_derivs=True)
    ts = []
    for _ in range(3):
        t0 = time.perf_counter()
        sysh.logderiv_batch(pos, sums=True, el_derivs=True)
        ts.append(time.perf_counter() - t0)
    t = min(ts)
    c = Q.roofline_model(spec, L.QMC_FP64, 0.5)
    tf = 65536 * c["refresh_flops"] / t / 1e12
    out["ch4_sr"] = {"workload": "CH4 9-AO SR gradient batch: 65536 walkers, P = 12 (8 Jastrow + 4 MO rotations): "
                                 "O_p, E_L, dE_L/dp, S (12x12) and f in FP64, through qmc_logderiv_batch with host "
                                 "buffers", "value": 65536 / t, "unit": "walkers/s", "ms": 1e3 * t,
                     "h2d_bytes": int(pos.nbytes), "d2h_bytes": int(65536 * 12 * 16 + 65536 * 8),
                     "roofline": {"bound": "fp64_simt", "achieved": tf, "peak": fp64_peak, "unit": "TFLOP/s",
                                  "frac": tf / fp64_peak if fp64_peak else None,
                                  "note": "evaluation flops only (values, gradients, Laplacians, inverse, E_L); "
                                          "the derivative work is extra, so the fraction is a lower bound"}}
    if cpu:
        from oracle import oracle as O
        n = 64
        t0 = time.perf_counter()
        O.evaluate(spec, pos[:n], threads=1)
        O.log_derivatives(spec, pos[:n], threads=1)
        O.el_derivatives(spec, pos[:n], threads=1)
        dt = time.perf_counter() - t0
        out["ch4_sr"]["cpu_baseline"] = {"value": n / dt, "unit": "walkers/s", "cores": 1, "kind": "port",
                                         "sample": "%d walkers: E_L, O_p and dE_L/dp, %.2f s" % (n, dt)}
    sysh.close()

    # benzene VMC and DMC: 16384 walkers, FP32+refine
    spec = Q.benzene_minimal()
    sysh = Q.System(ctx, spec)
    W = 16384
    wk = Q.Walkers(sysh, W, L.QMC_FP32_REFINE, capacity=4 * W)
    wk.init(seed=0x51A7E5 + 4)
    wk.refresh()
    for k in range(4):
        wk.sweep(L.QMC_MOVE_ONE_GAUSS, 32, 32 * k, seed=0x51A7E5 + 4, step=0.3, count=False)
        wk.refresh()
    acc = wk.sweep(L.QMC_MOVE_ONE_GAUSS, 64, 128, seed=0x51A7E5 + 4, step=0.3) / float(W * 42 * 64)
    wk.refresh()
    sw, rf = [], []
    s0 = 192
    for _ in range(3):
        sw.append(_events_ms(ctx, lambda: wk.sweep(L.QMC_MOVE_ONE_GAUSS, 64, s0, seed=0x51A7E5 + 4, step=0.3,
                                                   count=False)))
        rf.append(_events_ms(ctx, wk.refresh_async))
        s0 += 64
    moves = W * 42 * 64
    c = Q.roofline_model(spec, L.QMC_FP32_REFINE, acc)
    tf = moves * c["sweep_flops_per_move"] / (statistics.mean(sw) / 1e3) / 1e12
    out["c6h6_vmc"] = {"workload": "benzene 36-AO, 16384 walkers, 64 single-electron Gaussian sweeps of 0.3 bohr "
                                   "+ FP64-class refresh per step, FP32+refine",
                       "value": moves / ((statistics.mean(sw) + statistics.mean(rf)) / 1e3), "unit": UNIT,
                       "sweep_moves_per_s": moves / (statistics.mean(sw) / 1e3), "sweep_ms": statistics.mean(sw),
                       "refresh_ms": statistics.mean(rf), "acceptance": acc,
                       "roofline": {"bound": "fp32_simt", "kernel": "kw_sweep", "achieved": tf, "peak": fp32_peak,
                                    "unit": "TFLOP/s", "frac": tf / fp32_peak if fp32_peak else None,
                                    "flops_per_move": c["sweep_flops_per_move"]}}
    e_ref = wk.refresh() / W
    cut = 2.0 / np.sqrt(0.005)
    step = 0
    for _ in range(5):
        n, em = wk.dmc_step(0.005, e_ref, seed=0x51A7E5 + 4, step=step, fp64_measure=True, branch_cut=cut)
        step += 1
        e_ref = em - 0.5 * np.log(n / W) / 0.005
    ctx.synchronize()
    t0 = time.perf_counter()
    dmoves, pops = 0, []
    ctx.record(5)
    for _ in range(20):
        nb = wk.W
        n, em = wk.dmc_step(0.005, e_ref, seed=0x51A7E5 + 4, step=step, fp64_measure=True, branch_cut=cut)
        step += 1
        dmoves += nb * 42
        pops.append(n)
        e_ref = em - 0.5 * np.log(n / W) / 0.005
    ctx.record(6)
    dms = ctx.elapsed_ms(5, 6)
    out["c6h6_dmc"] = {"workload": "benzene IS-DMC, target 16384, tau 0.005: drift-diffusion sweep with fixed-node "
                                   "rejection, FP64-class E_L, FP64 log-weight branching (branching energy clamped "
                                   "to E_ref +- 2/sqrt(tau)) and on-device compaction per step (FP32 walkers)", "value": dmoves / (dms / 1e3), "unit": UNIT,
                       "ms_per_step": dms / 20, "population": [min(pops), max(pops)]}
    wk.close()
    if cpu:
        out["c6h6_vmc"]["cpu_baseline"] = oracle_sweep_rate(spec, L.QMC_MOVE_ONE_GAUSS, cpu_seconds)
        out["c6h6_dmc"]["cpu_baseline"] = oracle_sweep_rate(spec, L.QMC_MOVE_ONE_DRIFT, cpu_seconds)
    sysh.close()

    # uneven batch: systems cycling H2, Li, CH4, benzene, HEG-54; W ~ U{256..4096}
    kinds, walkers = batch_mix(args.batch_systems)
    specs = {k: SYSTEMS[k]() for k in set(kinds)}
    handles = {k: Q.System(ctx, specs[k]) for k in specs}
    sets = []
    for k, Wk in zip(kinds, walkers):
        w = Q.Walkers(handles[k], Wk, L.QMC_FP32_REFINE)
        w.init(seed=len(sets) + 1)
        w.refresh()
        sets.append(w)
    batch = Q.Batch(ctx, sets)
    sweeps = 8
    moves = sum(Wk * specs[k].n_elec for k, Wk in zip(kinds, walkers)) * sweeps
    batch.run_steps(L.QMC_MOVE_ONE_GAUSS, 1, sweeps, 0, seed=1, step=0.3)       # captures the graph
    bms = []
    for i in range(3):
        bms.append(_events_ms(ctx, lambda: batch.run_steps(L.QMC_MOVE_ONE_GAUSS, 1, sweeps, sweeps * (i + 1),
                                                           seed=1, step=0.3)))
    out["batch"] = {"workload": "%d systems (H2, Li, CH4 9-AO, benzene, HEG-54 cycling), %d walkers (U{256..4096} "
                                "each), one CUDA-graph step = %d Gaussian sweeps + refresh of every system, FP32+refine"
                                % (len(kinds), sum(walkers), sweeps),
                    "value": moves / (statistics.mean(bms) / 1e3), "unit": UNIT, "ms_per_step": statistics.mean(bms)}
    batch.close()
    for w in sets:
        w.close()
    if cpu:
        est = 0.0
        for k in sorted(specs):
            rk = oracle_sweep_rate(specs[k], L.QMC_MOVE_ONE_GAUSS, cpu_seconds / 4, step=1.0 if k == "heg" else 0.3)
            est += sum(Wk * specs[k].n_elec for kk, Wk in zip(kinds, walkers) if kk == k) * sweeps / rk["value"]
        out["batch"]["cpu_baseline"] = {"value": moves / est, "unit": UNIT, "cores": 1, "kind": "port",
                                        "sample": "per-kind oracle sweep rates (bounded samples) applied to the "
                                                  "batch's moves"}
    for h in handles.values():
        h.close()
    return out


def run_reference(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return
    import rust_qmc_gb300.systems as S
    from oracle import oracle as O
    spec = S.methane_minimal()
    threads = os.cpu_count() or 1
    # size one step to a bounded sample of about 3 s on all host threads
    v, W, dt = cpu_baseline(spec, 3.0 * threads, threads=threads, walkers_hint=threads * 2)
    pos = O.init_positions(spec, W, seed=5)
    for i in range(args.warmup):
        O.sweeps(spec, pos[: max(threads, W // 8)], 1, i, 2, 3, step=0.3, threads=threads, want_energy=False)
    times = []
    for i in range(args.steps):
        t0 = time.perf_counter()
        pos, _, _ = O.sweeps(spec, pos, 1, 100 + i, 2, 3, step=0.3, threads=threads, want_energy=False)
        times.append(time.perf_counter() - t0)
    moves = W * N_ELEC
    value = moves * len(times) / sum(times)
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * sum(times) / len(times),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded CH4 configurations)",
        "config": {"workload": "CH4 9-AO single-electron VMC, reference algorithm (full psi re-evaluation "
                               "per proposal), bounded sample", "walkers_per_step": W, "sweeps_per_step": 1,
                   "step_bohr": 0.3},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
                         "sample": "%d walkers x 1 sweep (10 proposals each) per step" % W},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
        return
    rank, world, local = dist_env()
    import numpy as np
    import rust_qmc_gb300 as Q
    from rust_qmc_gb300 import _lib as L

    group = Replicas(world)
    barrier, max_over_ranks, sum_over_ranks = group.barrier, group.max, group.sum

    ctx = Q.Context(local)
    spec = Q.methane_minimal()
    sysh = Q.System(ctx, spec)
    W, SW = args.walkers, args.sweeps
    seed = replica_seed(Q.SEED_BASE, rank)
    moves_per_step = W * N_ELEC * SW

    def make(prec):
        wk = Q.Walkers(sysh, W, prec)
        wk.init(seed)
        wk.refresh()
        return wk

    # ---------------- headline: FP32 walkers + FP64 refresh -----------------
    wk = make(L.QMC_FP32_REFINE)
    step_idx = 0
    acc = 0
    for _ in range(args.warmup):
        acc = wk.sweep(L.QMC_MOVE_ONE_GAUSS, SW, step_idx, seed, step=args.step_size)
        step_idx += SW
        wk.refresh_async()
    ctx.synchronize()
    acc_rate = acc / float(moves_per_step)

    clocks = ClockSampler(local)
    clocks.start()
    time.sleep(0.3)
    barrier()
    ctx.synchronize()
    launches0 = ctx.launch_count()
    step_ms, sweep_ms, refresh_ms = [], [], []
    for _ in range(args.steps):
        ctx.flush_l2()
        ctx.record(0)
        wk.sweep(L.QMC_MOVE_ONE_GAUSS, SW, step_idx, seed, step=args.step_size, count=False)
        ctx.record(1)
        wk.refresh_async()
        ctx.record(2)
        step_idx += SW
        step_ms.append(ctx.elapsed_ms(0, 2))
        sweep_ms.append(ctx.elapsed_ms(0, 1))
        refresh_ms.append(ctx.elapsed_ms(1, 2))
    ctx.synchronize()
    barrier()
    clk = clocks.stop()
    flush_launches = args.steps
    gpu_launches = ctx.launch_count() - launches0 - flush_launches
    value = whole_job_rate(moves_per_step * args.steps, sum(step_ms) / 1e3, group)
    e_sum, el_dev = wk.refresh(want_energies=True)
    e_mean = e_sum / W
    flags = wk.status()
    # held-out configurations for the accuracy condition of the metric: the
    # first 4096 walkers of the ensemble after the timed steps, with their
    # device E_L from the refresh (checked against the oracle on the host)
    held_pos, held_el = wk.get_positions()[:4096], el_dev[:4096]

    # ---------------- plain FP64 form (same schedule) -------------------------
    fp64 = None
    if not args.no_fp64_form:
        wk64 = make(L.QMC_FP64)
        s64 = 0
        wk64.sweep(L.QMC_MOVE_ONE_GAUSS, SW, s64, seed, step=args.step_size, count=False)
        wk64.refresh_async()
        s64 += SW
        t64 = []
        for _ in range(max(1, args.fp64_steps or args.steps)):
            ctx.flush_l2()
            ctx.record(3)
            wk64.sweep(L.QMC_MOVE_ONE_GAUSS, SW, s64, seed, step=args.step_size, count=False)
            wk64.refresh_async()
            ctx.record(4)
            s64 += SW
            t64.append(ctx.elapsed_ms(3, 4))
        v64 = sum_over_ranks(moves_per_step * len(t64)) / max_over_ranks(sum(t64) / 1e3)
        fp64 = {"value": v64, "unit": UNIT, "ms_per_step": sum(t64) / len(t64), "steps": len(t64),
                "speedup_fp32_refine_over_fp64": value / v64}
        wk64.close()

    # ---------------- end to end through the C ABI, host buffers --------------
    pin_pos = Q.PinnedArray(ctx.lib, (W, N_ELEC, 3))
    pin_el = Q.PinnedArray(ctx.lib, (W,))
    pin_pos.array[:] = wk.get_positions()
    import ctypes as C
    el_ptr = C.cast(pin_el.ptr, C.POINTER(C.c_double))
    wk_e2e = Q.Walkers(sysh, W, L.QMC_FP32_REFINE)
    e2e_times = []
    for i in range(args.warmup + args.steps):
        ctx.synchronize()
        t0 = time.perf_counter()
        wk_e2e.set_positions_ptr(pin_pos.ptr)          # H2D of the step's configurations
        wk_e2e.rebuild_inverse()                        # FP64 inverse and log|psi| of the uploaded walkers
        wk_e2e.sweep(L.QMC_MOVE_ONE_GAUSS, SW, 10 ** 6 + i * SW, seed, step=args.step_size, count=False)
        L.check(ctx.lib.qmc_walkers_refresh(wk_e2e.h, el_ptr, None), "qmc_walkers_refresh")  # D2H E_L
        t1 = time.perf_counter()
        if i >= args.warmup:
            e2e_times.append(t1 - t0)
    e2e_value = sum_over_ranks(moves_per_step * len(e2e_times)) / max_over_ranks(sum(e2e_times))
    e2e = {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": W * N_ELEC * 3 * 8,
           "d2h_bytes_per_step": W * 8}
    assert np.all(np.isfinite(pin_el.array)), "non-finite E_L in the end-to-end run"
    wk_e2e.close()
    pin_pos.free()
    pin_el.free()

    # ---------------- roofline of the dominant kernel (the sweep) -------------
    # algorithmic counts from the library's formulas (qmc_roofline_model)
    counts = Q.roofline_model(spec, L.QMC_FP32_REFINE, acc_rate)
    launch_s = statistics.mean(sweep_ms) / 1e3
    bytes_launch = W * counts["sweep_state_bytes"]
    achieved_gbs = bytes_launch / launch_s / 1e9
    peak_hbm, peak_kind = measured_peak_hbm()
    fp32_peak, fp64_peak = ctx.measure_peaks()
    flops_launch = moves_per_step * counts["sweep_flops_per_move"]
    achieved_tf = flops_launch / launch_s / 1e12
    # the library takes the chunked sweep (k_sweep_chunks) for sets that give
    # every SM sub-partition three warps, as 65 536 walkers do on 152 SMs
    traffic, sweep_kernel = None, "k_sweep_chunks<ShapeCH4Min,float,ONE_GAUSS,64>"
    tpath = os.path.join(ROOT, "profiles", "traffic_ch4_sweep.json")
    if os.path.exists(tpath):
        try:
            tj = json.load(open(tpath))
            traffic = tj.get("bytes_per_launch_65536_walkers")
            sweep_kernel = tj.get("kernel", sweep_kernel)
        except Exception:
            traffic = None
    # the sweep keeps its walkers in shared memory for all 64 sweeps: FP32 issue
    # (FMA + MUFU) bounds it, so the binding roofline is the FP32 one; the HBM
    # figure (state bytes per launch) is kept beside it
    roofline = {"bound": "fp32_simt", "achieved": achieved_tf, "peak": fp32_peak, "unit": "TFLOP/s",
                "frac": achieved_tf / fp32_peak if fp32_peak else None, "traffic": traffic,
                "peak_source": "measured FMA-chain kernel on this GPU (qmc_ctx_measure_peaks)",
                "kernel": sweep_kernel,
                "flops_per_move": counts["sweep_flops_per_move"],
                "traffic_source": "dram__bytes_read.sum + dram__bytes_write.sum per launch, one ncu capture "
                                  "(profiles/traffic_ch4_sweep.json)"}
    roofline_hbm = {"bound": "hbm", "achieved": achieved_gbs, "peak": peak_hbm, "unit": "GB/s",
                    "frac": achieved_gbs / peak_hbm, "peak_source": peak_kind + " (MEASURED_PEAKS.json hbm_gbs)",
                    "note": "walker state bytes per launch / launch time"}

    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": statistics.mean(step_ms), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32 (moves) + f64-class float-float (refresh, E_L)",
        "data": "synthetic (seeded CH4, QR-orthonormal MOs)",
        "config": {"workload": "CH4 9-AO single-electron VMC, FP32+refine", "walkers": W,
                   "sweeps_per_step": SW, "refresh_every": SW, "moves_per_step": moves_per_step,
                   "step_bohr": args.step_size, "parallelism": "replicas" if world > 1 else "single",
                   "l2": "flushed between steps (256 MB write, outside timing)"},
        "sweep_ms": statistics.mean(sweep_ms), "refresh_ms": statistics.mean(refresh_ms),
        "acceptance": acc_rate, "mean_energy": e_mean, "status_flags": flags,
        "fp64_form": fp64,
        "e2e": e2e,
        "roofline": roofline, "roofline_hbm": roofline_hbm,
        "peaks_measured": {"fp32_tflops": fp32_peak, "fp64_tflops": fp64_peak},
        "clocks": clk,
        "gpu_launches": gpu_launches,
    }
    if not args.no_configs:
        line["configs"] = other_configs(ctx, args, fp32_peak, fp64_peak, cpu=rank == 0 and not args.no_cpu_baseline)
    if rank == 0 and not args.no_cpu_baseline:
        try:
            v, Wc, dt = cpu_baseline(spec, args.cpu_seconds, threads=1)
            line["cpu_baseline"] = {"value": v, "unit": UNIT, "cores": 1, "kind": "port",
                                    "sample": "%d walkers x 1 sweep (10 proposals), reference algorithm, %.1f s"
                                              % (Wc, dt)}
        except Exception as e:  # the baseline is reported, never required
            line["cpu_baseline"] = {"value": None, "unit": UNIT, "cores": 1, "kind": "port",
                                    "sample": "failed: %s" % e}
        # the metric's accuracy condition: the oracle's FP64 E_L of the 4096
        # held-out configurations against the device's (refresh) E_L
        line["accuracy"] = held_out_accuracy(spec, held_pos, held_el)
        line["max_abs_dEL_Ha"] = line["accuracy"]["max_abs_dEL_Ha"]
        if not line["accuracy"]["within_1e-6_Ha"]:
            line["status"] = "E_L error above 1e-6 Ha"
    if rank == 0:
        print(json.dumps(line), flush=True)
    wk.close()
    sysh.close()
    ctx.close()
    group.close()


if __name__ == "__main__":
    main()
