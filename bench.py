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
    p.add_argument("--fp64-steps", type=int, default=2)
    p.add_argument("--no-fp64-form", action="store_true")
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
    e_mean = wk.refresh() / W
    flags = wk.status()

    # ---------------- plain FP64 form (same schedule) -------------------------
    fp64 = None
    if not args.no_fp64_form:
        wk64 = make(L.QMC_FP64)
        s64 = 0
        wk64.sweep(L.QMC_MOVE_ONE_GAUSS, SW, s64, seed, step=args.step_size, count=False)
        wk64.refresh_async()
        s64 += SW
        t64 = []
        for _ in range(max(1, args.fp64_steps)):
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
    traffic = None
    tpath = os.path.join(ROOT, "profiles", "traffic_ch4_sweep.json")
    if os.path.exists(tpath):
        try:
            traffic = json.load(open(tpath)).get("bytes_per_launch_65536_walkers")
        except Exception:
            traffic = None
    roofline = {"bound": "hbm", "achieved": achieved_gbs, "peak": peak_hbm, "unit": "GB/s",
                "frac": achieved_gbs / peak_hbm, "traffic": traffic, "peak_source": peak_kind,
                "kernel": "k_sweep_one<ShapeCH4Min,float,ONE_GAUSS,64>",
                "note": "state bytes per launch / launch time; the kernel keeps walkers in shared memory "
                        "for all 64 sweeps and is bound by FP32/SFU issue, see roofline_fp32"}
    roofline_fp32 = {"bound": "fp32_simt", "achieved": achieved_tf, "peak": fp32_peak, "unit": "TFLOP/s",
                     "frac": achieved_tf / fp32_peak if fp32_peak else None,
                     "peak_source": "measured FMA-chain kernel on this GPU",
                     "flops_per_move": counts["sweep_flops_per_move"]}

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
        "roofline": roofline, "roofline_fp32": roofline_fp32,
        "peaks_measured": {"fp32_tflops": fp32_peak, "fp64_tflops": fp64_peak},
        "clocks": clk,
        "gpu_launches": gpu_launches,
    }
    if rank == 0 and not args.no_cpu_baseline:
        try:
            v, Wc, dt = cpu_baseline(spec, args.cpu_seconds, threads=1)
            line["cpu_baseline"] = {"value": v, "unit": UNIT, "cores": 1, "kind": "port",
                                    "sample": "%d walkers x 1 sweep (10 proposals), reference algorithm, %.1f s"
                                              % (Wc, dt)}
        except Exception as e:  # the baseline is reported, never required
            line["cpu_baseline"] = {"value": None, "unit": UNIT, "cores": 1, "kind": "port",
                                    "sample": "failed: %s" % e}
    if rank == 0:
        print(json.dumps(line), flush=True)
    wk.close()
    sysh.close()
    ctx.close()
    group.close()


if __name__ == "__main__":
    main()
