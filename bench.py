#!/usr/bin/env python3
"""Benchmark: WLS state-estimation hot-start solves on one GB300 per rank.

Workload (the configuration the headline metric is quoted on): the seeded
10,000-bus / 14,000-branch synthetic grid (|V| at 30 % of buses, P+Q
injection at 60 %, both-end P+Q flows on 70 % of branches, plus the pseudo
flows that restore observability), plain FP64.  A flat-start solve brings the
state to the operating point; each step is then one telemetry update that
re-noises 1 % of the rows followed by a hot-start Gauss-Newton solve to
max|dx| < 1e-6 (sle_SolveWithConfig, PRECISION mode, refactorised gain).

  value   solves/s with the telemetry snapshots already resident in device
          memory (device-to-device copy into the engine, then the solve),
          timed with CUDA events on the engine's stream;
  e2e     the same metric through the reference-facing C ABI with host
          buffers: sle_UpdateTelemetry (host -> device) + sle_SolveWithConfig
          + sle_GetVoltageMagnitudes / sle_GetVoltageAngles (device -> host),
          wall-clock per step;
L2 is flushed (256 MiB write on the engine's stream) before every timed step
in both legs.  With torchrun (N > 1) every rank solves its own replica (the
path does not shard; there is no collective); value = all ranks' solves / the
slowest rank's time.

--impl reference times the reference's algorithm on the host cores instead:
the reference has no CPU implementation and its GPU path cannot run, so this
arm runs the CPU FP64 oracle (the restatement of the reference's
Gauss-Newton WLS) on the same workload.
"""
import argparse
import ctypes
import json
import os
import subprocess
import sys
import tempfile
import time

import numpy as np

REPO = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, REPO)

METRIC = "solves/s & p50/p99 latency, served mixed-prec vs plain FP64, ≤1e-6 state err"
UNIT = "solves/s"
WORKLOAD = "grid10k"
FLUSH_BYTES = 256 << 20


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=100)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--cpu-seconds", type=float, default=15.0, help="bounded CPU-baseline sample")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    return ap.parse_args()


def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("gloo")
    return world, rank, local


def allreduce_max(x, world):
    if world == 1:
        return x
    import torch
    import torch.distributed as dist

    t = torch.tensor([float(x)], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def barrier(world):
    if world > 1:
        import torch.distributed as dist

        dist.barrier()


class ClockSampler:
    """nvidia-smi clock / throttle sampling during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu):
        self.gpu = gpu
        self.proc = None
        self.path = None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.FIELDS, "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        with open(self.path) as fh:
            for line in fh:
                p = [x.strip() for x in line.split(",")]
                if len(p) < 9:
                    continue
                try:
                    sm.append(float(p[1]))
                    mx.append(float(p[2]))
                except ValueError:
                    continue
                for nm, v in zip(names, p[5:9]):
                    if v.lower() == "active":
                        reasons.add(nm)
        os.unlink(self.path)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def load_peaks():
    try:
        with open(os.path.join(REPO, "MEASURED_PEAKS.json")) as fh:
            p = json.load(fh)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def profile_traffic(kernel):
    """DRAM bytes per launch from a committed ncu summary, if one exists."""
    path = os.path.join(REPO, "profiles", "%s.md" % kernel)
    try:
        with open(path) as fh:
            for line in fh:
                if line.strip().startswith("traffic_bytes_per_launch:"):
                    return float(line.split(":", 1)[1])
    except OSError:
        pass
    return None


def stage_bytes(info, g, vb=8):
    """Algorithmic DRAM bytes per call of each stage (vb-byte factor values,
    FP64 vectors, int32 indices)."""
    m, n, ns = info.n_meas, info.n_bus, info.n_state
    nnz_h = info.nnz_h
    n_inj = int(np.isin(g.m_type, (2, 3, 7, 8)).sum())
    n_flow = int(np.isin(g.m_type, (4, 5, 6)).sum())
    avg_y = info.nnz_ybus / max(n, 1)
    return {
        # row metadata + z, w, sigma in; h, r, w_eff, w*r and H values out; state and Ybus gathers
        "evaluate": 72.0 * m + 8.0 * nnz_h + 16.0 * n + 28.0 * n_inj * avg_y + 48.0 * n_flow,
        # gain pairs + targets + H / weights in; L panels out; update matrices written and read once
        "factor": 8.0 * info.n_gain_pairs + 12.0 * info.n_gain_targets + vb * nnz_h + 8.0 * m
                  + vb * info.lx_size + 2.0 * vb * info.u_size,
        # column gather lists + H + w*r in, b out
        "rhs": 16.0 * nnz_h + 8.0 * m + 8.0 * ns,
        # L read by the forward and the backward sweep; vectors
        "solve": 2.0 * vb * info.lx_size + 32.0 * ns,
        "update": 48.0 * n,
    }


def run_leg(args, g, snaps, local, mixed, world):
    """One precision form: device-resident leg, end-to-end leg, profiled pass."""
    from state_estimation_with_cuda_gb300 import Estimator, native
    from state_estimation_with_cuda_gb300.api import MODE_PRECISION

    cfg = native.SLE_Config()
    est0 = Estimator()
    lib = est0.lib
    lib.sle_GetConfig(est0.h, ctypes.byref(cfg))
    est0.close()
    cfg.device_id = local
    cfg.use_double_precision = 0 if mixed else 1
    est = Estimator(cfg)
    est.load_network(g, z=g.z)
    est.upload_model()
    rc, res = est.solve_with(max_iterations=30, tolerance=1e-6, flat_start=True)
    assert res.status == 0, "flat-start solve did not converge (status %d)" % res.status
    info = est.plan_info()
    for i, z in enumerate(snaps):
        est._check(lib.sle_ExStageTelemetry(est.h, z.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), g.n_meas, i))
    scfg = native.SLE_SolverConfig(MODE_PRECISION, 20, 1e-6, 1.5, 0, 0, 0.0)
    r = native.SLE_Result()
    ms = ctypes.c_double()

    def device_step(i):
        est._check(lib.sle_ExFlushL2(est.h, FLUSH_BYTES))
        est._check(lib.sle_ExTimer(est.h, 0, None))
        est._check(lib.sle_ExUseTelemetry(est.h, i))
        rc = lib.sle_SolveWithConfig(est.h, ctypes.byref(scfg), ctypes.byref(r))
        est._check(lib.sle_ExTimer(est.h, 1, ctypes.byref(ms)))
        if rc != 0:
            raise RuntimeError("hot-start solve failed: status %d" % r.status)
        return ms.value, r.iterations

    # ---- device-resident leg -------------------------------------------------------
    for i in range(args.warmup):
        device_step(i)
    clocks = ClockSampler(local)
    st0 = native.SLE_ExStats()
    lib.sle_ExGetStats(est.h, ctypes.byref(st0))
    barrier(world)
    clocks.start()
    times, iters = [], []
    for k in range(args.steps):
        t, it = device_step(args.warmup + k)
        times.append(t)
        iters.append(it)
    clk = clocks.stop()
    st1 = native.SLE_ExStats()
    lib.sle_ExGetStats(est.h, ctypes.byref(st1))
    barrier(world)
    total_ms = allreduce_max(sum(times), world)
    launches = st1.total_launches - st0.total_launches
    v_dev = np.empty(g.n_bus)
    t_dev = np.empty(g.n_bus)
    dp = ctypes.POINTER(ctypes.c_double)
    est._check(lib.sle_GetVoltageMagnitudes(est.h, v_dev.ctypes.data_as(dp), g.n_bus))
    est._check(lib.sle_GetVoltageAngles(est.h, t_dev.ctypes.data_as(dp), g.n_bus))

    # ---- end-to-end leg through the C ABI with host buffers ---------------------------
    vbuf = np.empty(g.n_bus)
    tbuf = np.empty(g.n_bus)
    e2e_times = []
    for k in range(args.warmup + args.steps):
        z = snaps[k]
        est._check(lib.sle_ExFlushL2(est.h, FLUSH_BYTES))
        t0 = time.perf_counter()
        est._check(lib.sle_UpdateTelemetry(est.h, z.ctypes.data_as(dp), g.n_meas))
        rc = lib.sle_SolveWithConfig(est.h, ctypes.byref(scfg), ctypes.byref(r))
        est._check(lib.sle_GetVoltageMagnitudes(est.h, vbuf.ctypes.data_as(dp), g.n_bus))
        est._check(lib.sle_GetVoltageAngles(est.h, tbuf.ctypes.data_as(dp), g.n_bus))
        t1 = time.perf_counter()
        if rc != 0:
            raise RuntimeError("e2e solve failed: status %d" % r.status)
        if k >= args.warmup:
            e2e_times.append((t1 - t0) * 1e3)
    barrier(world)
    e2e_total = allreduce_max(sum(e2e_times), world)

    # ---- per-stage event timing for the roofline (separate pass, profiling on) --------------
    cfg.enable_profiling = 1
    est._check(lib.sle_SetConfig(est.h, ctypes.byref(cfg)))
    lib.sle_ExResetStats(est.h)
    for k in range(args.steps):
        device_step(args.warmup + k)
    prof = native.SLE_ExStats()
    lib.sle_ExGetStats(est.h, ctypes.byref(prof))
    est.close()
    names = ["evaluate", "factor", "rhs", "solve", "update", "final"]
    return dict(
        times=times, iters=iters, total_ms=total_ms, launches=launches, clk=clk, e2e_times=e2e_times,
        e2e_total=e2e_total, info=info, v=v_dev, th=t_dev,
        stage_ms={names[i]: prof.ms[i] for i in range(6)},
        stage_launch={names[i]: prof.launches[i] for i in range(6)},
        stage_calls={names[i]: prof.calls[i] for i in range(6)})


def roofline(leg, g, mixed):
    info = leg["info"]
    dom = max(("evaluate", "factor", "rhs", "solve", "update"), key=lambda s: leg["stage_ms"][s])
    sb = stage_bytes(info, g, 4 if mixed else 8)
    peak, peak_kind = load_peaks()
    per_call_ms = leg["stage_ms"][dom] / max(leg["stage_calls"][dom], 1)
    achieved = sb[dom] / (per_call_ms * 1e-3) / 1e9 if per_call_ms > 0 else 0.0
    kernel = {"evaluate": "k_evaluate", "factor": "front_factorisation", "rhs": "k_rhs", "solve": "front_solves",
              "update": "k_update"}[dom]
    return {"bound": "hbm", "kernel": kernel, "achieved": round(achieved, 2), "peak": peak, "peak_kind": peak_kind,
            "unit": "GB/s", "frac": round(achieved / peak, 5), "traffic": profile_traffic(kernel),
            "algorithmic_bytes_per_call": int(sb[dom])}


def run_gb300(args, world, rank, local):
    from state_estimation_with_cuda_gb300 import workloads

    g = workloads.make(WORKLOAD)
    snaps = [g.renoise(u).copy() for u in range(args.warmup + args.steps)]
    mixed = run_leg(args, g, snaps, local, True, world)
    fp64 = run_leg(args, g, snaps, local, False, world)
    out = None
    if rank == 0:
        def summary(leg):
            lat = np.array(leg["times"])
            return {"value": round(world * args.steps / (leg["total_ms"] * 1e-3), 3),
                    "ms_per_step": round(leg["total_ms"] / args.steps, 5),
                    "latency_ms": {"p50": round(float(np.percentile(lat, 50)), 4),
                                   "p99": round(float(np.percentile(lat, 99)), 4)},
                    "e2e": {"value": round(world * args.steps / (leg["e2e_total"] * 1e-3), 3), "unit": UNIT,
                            "h2d_bytes_per_step": 8 * g.n_meas, "d2h_bytes_per_step": 16 * g.n_bus,
                            "latency_ms": {"p50": round(float(np.percentile(leg["e2e_times"], 50)), 4),
                                           "p99": round(float(np.percentile(leg["e2e_times"], 99)), 4)}},
                    "iterations_per_solve": round(float(np.mean(leg["iters"])), 3),
                    "gpu_launches": int(leg["launches"]),
                    "stages_ms_per_solve": {k: round(v / max(args.steps, 1), 5) for k, v in leg["stage_ms"].items()},
                    "stage_launches_per_solve": {k: round(v / max(args.steps, 1), 2)
                                                 for k, v in leg["stage_launch"].items()}}
        sm, sf = summary(mixed), summary(fp64)
        err = float(max(np.abs(mixed["v"] - fp64["v"]).max(), np.abs(mixed["th"] - fp64["th"]).max()))
        info = mixed["info"]
        out = {
            "metric": METRIC, "value": sm["value"], "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": sm["ms_per_step"], "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32 gain/factor + f64 residual/refinement/state",
            "data": "synthetic (seeded generator)",
            "config": {
                "workload": "grid10k hot-start solves: %d buses, %d branches, %d rows, %d states; 1%% of rows "
                            "re-noised per step; tol 1e-6, gain refactorised every iteration; mixed precision "
                            "(value) and plain FP64 (fp64)" % (g.n_bus, g.n_branch, g.n_meas, 2 * g.n_bus - 1),
                "l2": "flushed before every timed step (256 MiB write)",
                "parallelism": "replicas" if world > 1 else "single",
                "iterations_per_solve": sm["iterations_per_solve"],
            },
            "latency_ms": sm["latency_ms"],
            "e2e": sm["e2e"],
            "gpu_launches": sm["gpu_launches"],
            "roofline": roofline(mixed, g, True),
            "stages_ms_per_solve": sm["stages_ms_per_solve"],
            "stage_launches_per_solve": sm["stage_launches_per_solve"],
            "fp64": dict(sf, roofline=roofline(fp64, g, False)),
            "mixed_vs_fp64_max_state_err": err,
            "clocks": mixed["clk"],
            "plan": {"nnz_l": info.nnz_l, "n_super": info.n_super, "levels": info.n_levels,
                     "max_front": info.max_front, "factor_flops": info.factor_flops},
        }
    return out, g


def cpu_hot_start(g, seconds, min_solves=3, max_solves=None):
    """Oracle hot-start solves of the same workload for about `seconds`."""
    from oracle.binding import Oracle, threads

    o = Oracle(g)
    v, th, res, _ = o.wls(g.z, g.v_setpoint, np.zeros(g.n_bus), max_iterations=30, tolerance=1e-6)
    assert res.status == 0
    times = []
    u = 0
    t_start = time.perf_counter()
    while True:
        z = g.renoise(10000 + u)
        t0 = time.perf_counter()
        v, th, res, _ = o.wls(z, v, th, max_iterations=20, tolerance=1e-6, flat_start=False)
        times.append(time.perf_counter() - t0)
        u += 1
        if max_solves is not None and u >= max_solves:
            break
        if u >= min_solves and time.perf_counter() - t_start > seconds:
            break
    o.close()
    return len(times) / sum(times), times, threads()


def main():
    args = parse()
    world, rank, local = dist_setup()
    if args.impl == "reference":
        if rank != 0:
            return
        from state_estimation_with_cuda_gb300 import workloads

        g = workloads.make(WORKLOAD)
        # warm-up solves (untimed), then exactly `steps` timed hot-start solves
        _, _, _ = cpu_hot_start(g, 0.0, min_solves=max(args.warmup, 1), max_solves=max(args.warmup, 1))
        value, times, cores = cpu_hot_start(g, 0.0, min_solves=args.steps, max_solves=args.steps)
        line = {
            "metric": METRIC, "value": round(value, 3), "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": round(1e3 * float(np.mean(times)), 4), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded generator)",
            "config": {"workload": "grid10k hot-start solves (as the gb300 arm)", "l2": "n/a (host)"},
            "impl": "reference",
            "cpu_baseline": {"value": round(value, 3), "unit": UNIT, "cores": cores, "kind": "port",
                             "sample": "%d hot-start solves of grid10k (1%% re-noise each)" % len(times)},
            "e2e": {"value": round(value, 3), "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        }
        print(json.dumps(line))
        return
    out, g = run_gb300(args, world, rank, local)
    if rank == 0:
        if world == 1 and not args.no_cpu_baseline:
            value, times, cores = cpu_hot_start(g, args.cpu_seconds)
            out["cpu_baseline"] = {"value": round(value, 3), "unit": UNIT, "cores": cores, "kind": "port",
                                   "sample": "%d hot-start solves of grid10k (1%% re-noise each), %.1f s"
                                             % (len(times), sum(times))}
        print(json.dumps(out))
    if world > 1:
        import torch.distributed as dist

        dist.destroy_process_group()


if __name__ == "__main__":
    main()
