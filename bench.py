#!/usr/bin/env python3
"""Benchmark: WLS state-estimation solves on one GB300 per rank.

Headline workload (the serving form): a resident fleet of 200 seeded
synthetic grids with Zipf(1.2) sizes over 30..200,000 buses (1.4 branches per
bus; |V| at 30 % of buses, P+Q injection at 60 %, both-end P+Q flows on 70 %
of branches, plus the pseudo flows that restore observability).  Requests
arrive as a Poisson stream at 2,000 requests/s, each a fresh FP64
measurement snapshot for a uniformly chosen grid (0.5 % also open or close a
non-bridge branch), hot-started from the grid's last estimate, max|dx| < 1e-6.

One step = one window of 150 consecutive requests of the stream (75 ms of
arrivals).  W warm-up windows are served and drained, then K windows are
timed, from the first submission to the last completion, through the C ABI
with host buffers: sle_ExServerSubmitEx copies the snapshot host -> device
and, when the request completes, the grid's |V| and theta device -> host;
sle_ExServerWait returns the result record.

  value            requests completed per second, mixed-precision server
                   (FP32 gain / factor / solves, FP64 residual, gradient and
                   state), latency_ms p50 / p99 from submit to result;
  served_fp64      the same stream through a plain-FP64 server;
  per_grid_fp64    the plain FP64 per-grid path on the same requests: one
                   engine per grid (sle_UpdateTelemetry + sle_SolveWithConfig
                   + sle_GetVoltage*), one request at a time;
  state_err_vs_oracle  served states of a seeded sample of the timed
                   requests against the CPU FP64 oracle's converged estimate.

Secondary configurations print one JSON line each before the final line:
grid200k (cold and warm flat starts, Huber, errors against the oracle),
grid10k (100 hot-start updates, device-resident and e2e legs, per-stage
roofline), batch512, the loaded-pass roofline and the CPU baselines of every
configuration.

With torchrun (N > 1) every rank serves its own replica of the fleet (grids
do not shard across GPUs; no collective); value = all ranks' requests / the
slowest rank's time.

--impl reference times the reference's algorithm on the host cores instead:
the reference has no CPU implementation and its GPU path cannot run, so this
arm runs the CPU FP64 oracle (the restatement of the reference's
Gauss-Newton WLS) on a bounded sample of each window of the same stream.
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


LAMBDA = 2000.0
FLEET = 200
SNAPS_PER_GRID = 4
BREAKER_FRAC = 0.005
STEP_REQUESTS = 150   # requests per step (one window of the stream)
COLD_STARTS = 3  # grid200k cold flat starts per precision (the median is reported)
HUBER_STALL = 1e-5    # the grid200k leg's Huber stall safeguard (option huber_stall)
REF_STEP_SECONDS = 4.0  # CPU seconds of each window the host-core reference arm spends


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20, help="timed steps (windows of %d requests)" % STEP_REQUESTS)
    ap.add_argument("--warmup", type=int, default=5, help="warm-up steps")
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--cpu-seconds", type=float, default=10.0, help="bounded CPU-baseline sample of the stream")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--grid10k-steps", type=int, default=100, help="hot-start updates of the grid10k leg")
    ap.add_argument("--skip-extra", action="store_true", help="headline legs only")
    ap.add_argument("--union-passes", type=int, default=3, help="profiled passes of the batch roofline leg")
    ap.add_argument("--only", choices=["batch512", "grid200k", "grid10k", "union_roofline"],
                    help="run one secondary configuration alone and print its object (for profiling)")
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
    """grid10k, one precision form: device-resident leg, end-to-end leg,
    profiled pass (args.steps / args.warmup here are the grid10k counts)."""
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
    if info.n_bus > 100000:  # the batch union: its own committed summary
        kernel = "union_" + kernel
    return {"bound": "hbm", "kernel": kernel, "achieved": round(achieved, 2), "peak": peak, "peak_kind": peak_kind,
            "unit": "GB/s", "frac": round(achieved / peak, 5), "traffic": profile_traffic(kernel),
            "algorithmic_bytes_per_call": int(sb[dom])}


class Stream:
    """The serving workload: fleet, per-grid snapshots, seeded request stream."""

    def __init__(self, n_req):
        from state_estimation_with_cuda_gb300 import workloads

        self.grids = workloads.fleet_grids(FLEET)
        self.snaps = [[g.renoise(u).copy() for u in range(SNAPS_PER_GRID)] for g in self.grids]
        rng = np.random.default_rng(0x5E04 + 1)
        self.arrival = np.cumsum(rng.exponential(1.0 / LAMBDA, n_req))
        self.target = rng.integers(0, FLEET, n_req)
        self.breaker = rng.random(n_req) < BREAKER_FRAC
        # snapshot index per request: a grid's k-th request uses its snapshot k mod SNAPS_PER_GRID
        seen = np.zeros(FLEET, np.int64)
        self.snap = np.empty(n_req, np.int64)
        for i, g in enumerate(self.target):
            self.snap[i] = seen[g] % SNAPS_PER_GRID
            seen[g] += 1
        # breaker edits: open a non-bridge branch, close it again at the grid's next edit
        self.branch = np.full(n_req, -1, np.int64)
        self.closed = np.ones(n_req, np.int64)
        opened = {}
        for i in np.nonzero(self.breaker)[0]:
            g = int(self.target[i])
            if g in opened:
                self.branch[i], self.closed[i] = opened.pop(g), 1
            else:
                k = self.grids[g]._lib.segen_pick_nonbridge(self.grids[g]._h, int(i))
                if k >= 0:
                    self.branch[i], self.closed[i] = k, 0
                    opened[g] = k
        self.n_req = n_req

    def z(self, i):
        return self.snaps[int(self.target[i])][int(self.snap[i])]

    def sample(self, lo, hi, n_small=10, n_mid=2):
        """Seeded timed requests whose served state is checked against the
        oracle: grids without breaker edits in the stream, n_small of at most
        5,000 buses and n_mid of 5,000..60,000 buses."""
        edited = set(int(self.target[i]) for i in np.nonzero(self.branch >= 0)[0])
        rng = np.random.default_rng(0x5E04 + 2)
        order = rng.permutation(np.arange(lo, hi))
        small, mid = [], []
        for i in order:
            g = int(self.target[i])
            if g in edited:
                continue
            n = self.grids[g].n_bus
            if n <= 5000 and len(small) < n_small:
                small.append(int(i))
            elif 5000 < n <= 60000 and len(mid) < n_mid:
                mid.append(int(i))
        return sorted(small + mid)

    def describe(self):
        n = [g.n_bus for g in self.grids]
        return {"grids": FLEET, "buses_min": int(min(n)), "buses_max": int(max(n)), "buses_total": int(sum(n)),
                "rows_total": int(sum(g.n_meas for g in self.grids)), "lambda_per_s": LAMBDA,
                "breaker_fraction": BREAKER_FRAC}


def run_served(args, stream, mixed, local, lo, hi, clocks=None, sample=()):
    """Requests [lo, hi) of the stream paced at their arrival offsets through a
    Server; warm-up requests [0, lo) are served and drained first.  Every
    request's |V| and theta come back to host buffers (per grid; the sampled
    requests get their own) before its ticket completes."""
    import threading

    from state_estimation_with_cuda_gb300 import Server, native

    t0 = time.perf_counter()
    srv = Server(mixed=mixed, device_id=local)
    lib = srv.lib
    for g in stream.grids:
        srv.add_grid(g)
    srv.start()
    t_start = time.perf_counter() - t0
    grid_out = [(np.empty(g.n_bus), np.empty(g.n_bus)) for g in stream.grids]
    sample_out = {i: (np.empty(stream.grids[int(stream.target[i])].n_bus),
                      np.empty(stream.grids[int(stream.target[i])].n_bus)) for i in sample}

    def serve(a, b):
        tickets = [None] * (b - a)

        def submitter():
            base = time.perf_counter()
            off = stream.arrival[a]
            for i in range(a, b):
                dt = (stream.arrival[i] - off) - (time.perf_counter() - base)
                if dt > 0:
                    time.sleep(dt)
                g = int(stream.target[i])
                out = sample_out.get(i, grid_out[g])
                tickets[i - a] = srv.submit(g, stream.z(i), int(stream.branch[i]), int(stream.closed[i]), out=out)

        th = threading.Thread(target=submitter)
        th.start()
        out = []
        for k in range(b - a):
            while tickets[k] is None:
                time.sleep(0.0002)
            out.append(srv.wait(tickets[k], 3.6e6))
        th.join()
        return out

    serve(0, lo)
    stats = native.SLE_ExStats()
    from state_estimation_with_cuda_gb300 import Estimator

    est = Estimator()
    lib.sle_ExGetStats(est.h, ctypes.byref(stats))
    l0 = stats.total_launches
    if clocks:
        clocks.start()
    res = serve(lo, hi)
    clk = clocks.stop() if clocks else None
    lib.sle_ExGetStats(est.h, ctypes.byref(stats))
    launches = stats.total_launches - l0
    est.close()
    st = srv.stats()
    srv.close()
    lat = np.array([(r.t_done_ns - r.t_submit_ns) / 1e6 for r in res])
    t_first = min(r.t_submit_ns for r in res)
    t_last = max(r.t_done_ns for r in res)
    nb = np.array([stream.grids[int(stream.target[i])].n_bus for i in range(lo, hi)])
    nm = np.array([stream.grids[int(stream.target[i])].n_meas for i in range(lo, hi)])
    big = nb >= 20000
    return {
        "elapsed_s": (t_last - t_first) / 1e9, "lat": lat, "ok": int(sum(r.status == 0 for r in res)),
        "iters": float(np.mean([r.iterations for r in res])), "batch": float(np.mean([r.batch_size for r in res])),
        "units": st.units, "device_bytes": int(st.device_bytes), "start_s": t_start, "launches": int(launches),
        "clk": clk, "lat_small": lat[~big], "lat_big": lat[big],
        # per request: the snapshot in; the state (2 x n_bus doubles) and the result record out
        "h2d_total": int(8 * nm.sum()), "d2h_total": int(16 * nb.sum() + 56 * len(nb)),
        "states": {i: sample_out[i] for i in sample},
        "evictions": int(st.evictions),
        "status_counts": {str(k): int(v) for k, v in zip(*np.unique([r.status for r in res], return_counts=True))},
        "not_ok_breaker": int(sum(r.status != 0 and stream.branch[lo + k] >= 0 for k, r in enumerate(res))),
    }


def served_state_error(stream, states):
    """Max |V| / theta difference between served states and the oracle's
    estimate of the same snapshot (flat start, converged to 1e-10)."""
    from oracle.binding import Oracle

    worst = 0.0
    for i, (v, th) in states.items():
        grid = stream.grids[int(stream.target[i])]
        o = Oracle(grid)
        ov, oth, res, _ = o.wls(stream.z(i), grid.v_setpoint, np.zeros(grid.n_bus), max_iterations=40,
                                tolerance=1e-10)
        o.close()
        if res.status != 0:
            return None
        worst = max(worst, float(np.abs(v - ov).max()), float(np.abs(th - oth).max()))
    return worst


def run_per_grid_fp64(stream, local, lo, hi):
    """Plain FP64 per-grid path: one engine per grid, requests one at a time
    (breaker requests are served as plain snapshots here: no re-analysis)."""
    from state_estimation_with_cuda_gb300 import Estimator

    engines = {}
    for i in range(lo, hi):
        g = int(stream.target[i])
        if g not in engines:
            e = Estimator()
            e.load_network(stream.grids[g])
            e.upload_model()
            e.solve_with(max_iterations=20, tolerance=1e-6, flat_start=True)
            engines[g] = e
    lat = []
    t0 = time.perf_counter()
    for i in range(lo, hi):
        e = engines[int(stream.target[i])]
        ts = time.perf_counter()
        e.update_telemetry(stream.z(i))
        rc, r = e.solve_with(max_iterations=20, tolerance=1e-6)
        e.voltages()  # the state back to the host, as the served legs return it
        lat.append((time.perf_counter() - ts) * 1e3)
    dt = time.perf_counter() - t0
    for e in engines.values():
        e.close()
    return {"value": round((hi - lo) / dt, 3), "service_ms": {"p50": round(float(np.percentile(lat, 50)), 3),
                                                              "p99": round(float(np.percentile(lat, 99)), 3)},
            "note": "one engine per grid, one request at a time, state read back; breaker requests served as "
                    "plain snapshots"}


def run_batch512():
    """Batched form with the autotuned schedule (tuned.json: size buckets solved
    concurrently, phase-A width); falls back to one bucket of all grids."""
    from state_estimation_with_cuda_gb300 import workloads
    from state_estimation_with_cuda_gb300.tune import BatchSet, tuned_config

    best = tuned_config().get("batch", {}).get("best", {})
    bounds = tuple(best.get("bucket_bus", ()))
    width = best.get("flow_small_f")
    grids = workloads.batch_grids(512)
    snaps = [[g.renoise(u).copy() for g in grids] for u in range(3)]
    out = {}
    for mixed in (True, False):
        # the tuned phase-A width is the mixed form's; FP64 keeps the engine's default
        b = BatchSet(grids, bounds, mixed=mixed, flow_small_f=width if mixed else None)
        b.solve(flat_start=True)
        times, its = [], []
        for u in range(3):
            t0 = time.perf_counter()
            for i in range(len(grids)):
                b.set_telemetry(i, snaps[u][i])
            res = b.solve(flat_start=False)
            times.append(time.perf_counter() - t0)
            its += [r.iterations for r in res]
            assert all(r.status == 0 for r in res)
        b.close()
        out["mixed" if mixed else "fp64"] = {"value": round(3 * len(grids) / sum(times), 1),
                                             "ms_per_batch": round(1e3 * float(np.mean(times)), 2),
                                             "iterations_mean": round(float(np.mean(its)), 3),
                                             "iterations_max": int(max(its))}
    out["config"] = ("512 grids, log-uniform 30..5000 buses (%d buses, %d rows); hot start after a 1%% re-noise; "
                     "size buckets %s (one batch each, solved concurrently), phase-A width %s (mixed; FP64 64); "
                     "wall clock including the telemetry copies"
                     % (sum(g.n_bus for g in grids), sum(g.n_meas for g in grids), list(bounds) or "[all]",
                        width or 64))
    out["unit"] = "solves/s"
    out["schedule_source"] = "tuned.json" if best else "defaults"
    return out


def run_union_roofline(local, passes=3):
    """Throughput-regime roofline: one Gauss-Newton pass of the 512-grid batch
    with every grid taking the step (flat start), stages timed with CUDA events
    (profiling on, so no graphs), L2 flushed before the pass; the dominant
    stage against its algorithmic bytes on the union's plan.  The single
    grid10k leg keeps its own roofline: one grid of that size is bound by the
    elimination tree's serial chain, not by HBM."""
    from state_estimation_with_cuda_gb300 import BatchEstimator, native, workloads

    grids = workloads.batch_grids(512)
    b = BatchEstimator(mixed=True)
    b.set_config(enable_profiling=1, device_id=local)
    for g in grids:
        b.add_grid(g)
    b.upload_model()
    b.solve(flat_start=True, max_iterations=1)  # warm-up
    lib = b.lib
    names = ["evaluate", "factor", "rhs", "solve", "update", "final"]
    best = None
    for _ in range(passes):
        b._check(lib.sle_ExFlushL2(b.h, FLUSH_BYTES))
        lib.sle_ExResetStats(b.h)
        b.solve(flat_start=True, max_iterations=1)
        st = native.SLE_ExStats()
        lib.sle_ExGetStats(b.h, ctypes.byref(st))
        leg = {"stage_ms": {names[i]: st.ms[i] for i in range(6)},
               "stage_calls": {names[i]: st.calls[i] for i in range(6)},
               "stage_launches": {names[i]: st.launches[i] for i in range(6)}}
        if best is None or sum(leg["stage_ms"].values()) < sum(best["stage_ms"].values()):
            best = leg
    best["info"] = b.plan_info()
    b.close()
    union = argparse.Namespace(m_type=np.concatenate([g.m_type for g in grids]))
    r = roofline(best, union, True)
    r["workload"] = ("one Gauss-Newton pass of the 512-grid batch (%d buses, %d rows), every grid active, mixed "
                     "precision, L2 flushed before the pass" % (sum(g.n_bus for g in grids),
                                                               sum(g.n_meas for g in grids)))
    r["stages_ms"] = {k: round(v, 4) for k, v in best["stage_ms"].items()}
    r["stage_launches"] = best["stage_launches"]
    return r


def run_grid200k(oracle_state=None):
    """Config 2: the 200,000-bus grid.  Cold flat start = wall clock of load ->
    symbolic analysis -> upload -> solve through the C ABI (each precision on
    a fresh handle, the process's CUDA context already up); warm flat start = the solve alone on the uploaded model
    with its graphs captured.  Plain WLS as the reference runs it with robust
    estimation off; then the Huber solve (gamma 1.5) with the reference's
    weights, and with the stall safeguard on the Huber objective.  Errors against
    the oracle's converged estimate when it is given."""
    from state_estimation_with_cuda_gb300 import Estimator, workloads

    g = workloads.make("grid200k")
    out, states = {}, {}
    # the process's CUDA context and its kernels (loaded at first launch) come
    # up first, on a 20k-bus grid in both precisions (tiled fronts included):
    # a cold flat start times the grid's own work, not the process's
    wg = workloads.SyntheticGrid(20000, 28000, 5)
    for wm in (0, 1):
        w = Estimator()
        w.set_option("use_double_precision", wm)
        w.load_network(wg)
        w.upload_model()
        w.solve_with(max_iterations=3, tolerance=1e-6, flat_start=True)
        w.close()

    def cold_flat_start(mixed):
        """One cold flat start on a fresh handle: its wall time, its host
        phases (upload = analysis + schedule + arena and copies) and the handle."""
        t0 = time.perf_counter()
        e = Estimator()
        e.set_option("use_double_precision", 0 if mixed else 1)
        e.load_network(g)
        t_load = time.perf_counter()
        e.upload_model()
        t_up = time.perf_counter()
        e.solve_with(max_iterations=30, tolerance=1e-6, flat_start=True)
        cold = time.perf_counter() - t0
        st = e.stats()
        phases = {"handle_and_load": round((t_load - t0) * 1e3, 1), "analysis": round(st.analysis_ms, 1),
                  "schedule": round(st.schedule_ms, 1), "arena_and_copies": round(st.upload_ms, 1),
                  "upload_total": round((t_up - t_load) * 1e3, 1),
                  "first_solve": round((t0 + cold - t_up) * 1e3, 1), "graph_capture_in_solve": round(st.capture_ms, 1)}
        return cold, phases, e

    for mixed in (True, False):
        # three cold starts, each on a fresh handle; the median one is reported
        runs = []
        for k in range(COLD_STARTS):
            cold, phases, e = cold_flat_start(mixed)
            runs.append((cold, phases))
            if k + 1 < COLD_STARTS:
                e.close()
        cold_samples = [round(c * 1e3, 1) for c, _ in runs]
        cold, phases = sorted(runs, key=lambda r: r[0])[COLD_STARTS // 2]
        e.solve_with(max_iterations=2, tolerance=1e-6, flat_start=True)  # graphs of both iteration kinds
        t0 = time.perf_counter()
        rc, r = e.solve_with(max_iterations=30, tolerance=1e-6, flat_start=True)
        dt = time.perf_counter() - t0
        states[mixed] = e.voltages()
        t0 = time.perf_counter()
        rc, rh = e.solve_with(max_iterations=100, tolerance=1e-6, flat_start=True, robust=True, huber_gamma=1.5)
        th_ref = time.perf_counter() - t0
        huber = {"status": rh.status, "iterations": rh.iterations, "ms": round(th_ref * 1e3, 1)}
        # the stall safeguard: also stop once an iteration lowers the Huber objective by <= 1e-5 of it
        e.set_option("huber_stall", HUBER_STALL)
        t0 = time.perf_counter()
        rc, rs = e.solve_with(max_iterations=100, tolerance=1e-6, flat_start=True, robust=True, huber_gamma=1.5)
        huber["stall_%g" % HUBER_STALL] = {"status": rs.status, "iterations": rs.iterations,
                                           "ms": round((time.perf_counter() - t0) * 1e3, 1)}
        e.close()
        out["mixed" if mixed else "fp64"] = {
            "cold_flat_start_ms": round(cold * 1e3, 1), "cold_samples_ms": cold_samples, "cold_phases_ms": phases,
            "flat_start_ms": round(dt * 1e3, 2),
            "iterations": r.iterations, "status": r.status, "huber": huber}
    out["mixed_vs_fp64_max_state_err"] = float(max(np.abs(states[True][0] - states[False][0]).max(),
                                                   np.abs(states[True][1] - states[False][1]).max()))
    if oracle_state is not None:
        ov, oth, iters = oracle_state
        for mixed in (True, False):
            err = float(max(np.abs(states[mixed][0] - ov).max(), np.abs(states[mixed][1] - oth).max()))
            out["%s_vs_oracle_max_state_err" % ("mixed" if mixed else "fp64")] = err
        out["oracle_iterations"] = iters
    out["config"] = ("%d buses, %d branches, %d rows, 2%% gross errors on telemetry rows; flat start, "
                     "max|dx| < 1e-6; cold = load + analysis + upload + solve on a fresh handle, median of %d"
                     % (g.n_bus, g.n_branch, g.n_meas, COLD_STARTS))
    return out


def cpu_baselines(budget_each=30.0):
    """The CPU FP64 oracle on every configuration (host cores; OpenMP in the
    evaluation, the ordering and Cholesky single-threaded): config 0 and 2
    flat starts, config 1 flat start plus 100 hot-start updates (each from
    the oracle's own previous estimate), config 3 on a seeded sample of the
    512 grids.  Returns (summary, grid200k oracle state)."""
    from oracle.binding import Oracle, threads
    from state_estimation_with_cuda_gb300 import workloads

    out = {"cores": threads(), "kind": "port", "unit": "solves/s"}
    g = workloads.make("grid14")
    o = Oracle(g)
    t0 = time.perf_counter()
    reps = 0
    while time.perf_counter() - t0 < 1.0:
        o.wls(g.z, g.v_setpoint, np.zeros(g.n_bus), max_iterations=20, tolerance=1e-6)
        reps += 1
    out["grid14_flat_start"] = round(reps / (time.perf_counter() - t0), 2)
    o.close()
    g = workloads.make("grid10k")
    o = Oracle(g)
    t0 = time.perf_counter()
    v, th, r, _ = o.wls(g.z, g.v_setpoint, np.zeros(g.n_bus), max_iterations=20, tolerance=1e-6)
    t_flat = time.perf_counter() - t0
    t0 = time.perf_counter()
    n_up = 0
    for u in range(100):
        v, th, r, _ = o.wls(g.renoise(u), v, th, max_iterations=20, tolerance=1e-6, flat_start=False)
        n_up += 1
        if time.perf_counter() - t0 > budget_each:
            break
    t_up = time.perf_counter() - t0
    out["grid10k_flat_start_ms"] = round(t_flat * 1e3, 1)
    out["grid10k_hot_start"] = round(n_up / t_up, 2)
    out["grid10k_updates"] = n_up
    o.close()
    grids = workloads.batch_grids(512)
    rng = np.random.default_rng(3)
    pick = rng.choice(len(grids), 48, replace=False)
    t0 = time.perf_counter()
    for i in pick:
        gg = grids[int(i)]
        oo = Oracle(gg)
        oo.wls(gg.z, gg.v_setpoint, np.zeros(gg.n_bus), max_iterations=20, tolerance=1e-6)
        oo.close()
    out["batch512_flat_start_sample"] = round(len(pick) / (time.perf_counter() - t0), 2)
    g = workloads.make("grid200k")
    o = Oracle(g)
    t0 = time.perf_counter()
    v, th, r, _ = o.wls(g.z, g.v_setpoint, np.zeros(g.n_bus), max_iterations=20, tolerance=1e-6)
    out["grid200k_flat_start_ms"] = round((time.perf_counter() - t0) * 1e3, 1)
    out["grid200k_iterations"] = r.iterations
    o.close()
    out["note"] = ("oracle timings per configuration; batch512 on 48 seeded grids of the 512 (flat start each); "
                   "grid10k updates re-noise 1% of rows and hot-start from the previous estimate")
    return out, (v, th, r.iterations)


def oracle_served(stream, lo, hi, step_seconds):
    """The CPU FP64 oracle on the windows of [lo, hi) of the stream: in each
    window, requests in arrival order, one at a time, until the window's
    `step_seconds` of solve time are spent (at least one request a window).
    A grid's first request starts from the grid's true state (a per-grid
    flat-start estimate first would take minutes of host time on the large
    grids); its later requests start from the oracle's own previous
    estimate, as the served arms do.  The oracle's symbolic analysis of a
    grid (done once, like the GPU server's at start) is outside the timing."""
    from oracle.binding import Oracle, threads

    cache, state = {}, {}
    times = []
    for w in range(lo, hi, STEP_REQUESTS):
        spent = 0.0
        for i in range(w, min(w + STEP_REQUESTS, hi)):
            g = int(stream.target[i])
            grid = stream.grids[g]
            if g not in cache:
                cache[g] = Oracle(grid)
                cache[g].wls(stream.z(i), grid.v_true, grid.theta_true, max_iterations=0, flat_start=False)
                state[g] = (grid.v_true.copy(), grid.theta_true.copy())
            v0, th0 = state[g]
            t0 = time.perf_counter()
            v, th, _, _ = cache[g].wls(stream.z(i), v0, th0, max_iterations=20, tolerance=1e-6, flat_start=False)
            dt = time.perf_counter() - t0
            times.append(dt)
            spent += dt
            state[g] = (v, th)
            if spent >= step_seconds:
                break
    for o in cache.values():
        o.close()
    return len(times) / sum(times), times, threads()


def emit(obj):
    print(json.dumps(obj), flush=True)


def pct(a, q):
    return round(float(np.percentile(a, q)), 3) if len(a) else None


def run_gb300(args, world, rank, local):
    lo, hi = args.warmup * STEP_REQUESTS, (args.warmup + args.steps) * STEP_REQUESTS
    stream = Stream(hi)
    sample = stream.sample(lo, hi)
    clocks = ClockSampler(local)
    barrier(world)
    sm = run_served(args, stream, True, local, lo, hi, clocks, sample)
    barrier(world)
    sf = run_served(args, stream, False, local, lo, hi, sample=sample)
    elapsed = allreduce_max(sm["elapsed_s"], world)
    out = None
    if rank == 0:
        per_grid = run_per_grid_fp64(stream, local, lo, hi)
        err_mixed = served_state_error(stream, sm["states"])
        err_fp64 = served_state_error(stream, sf["states"])
        union = None
        if not args.skip_extra:
            ostate = None
            if not args.no_cpu_baseline:
                cpu, ostate = cpu_baselines()
                emit({"leg": "cpu_baselines", **cpu})
            emit({"leg": "grid200k", **run_grid200k(ostate)})
            emit({"leg": "batch512", **run_batch512()})
            union = run_union_roofline(local)
            emit({"leg": "union_roofline", **union})
    if not args.skip_extra:
        from state_estimation_with_cuda_gb300 import workloads

        a10 = argparse.Namespace(**vars(args))
        a10.steps, a10.warmup = args.grid10k_steps, 3
        g10 = workloads.make("grid10k")
        snaps10 = [g10.renoise(u).copy() for u in range(a10.warmup + a10.steps)]
        m10 = run_leg(a10, g10, snaps10, local, True, world)
        f10 = run_leg(a10, g10, snaps10, local, False, world)
        if rank == 0:
            emit({"leg": "grid10k", **summarize_leg(m10, f10, g10, a10, world)})
    if rank == 0:
        value = round(world * (hi - lo) / elapsed, 3)
        pg = per_grid["value"]
        out = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": round(1e3 * elapsed / args.steps, 4), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32 gain/factor/solves + f64 residual/gradient/state",
            "data": "synthetic (seeded generator)",
            "config": {"workload": "serving form: 200 resident grids, Zipf(1.2) over 30..200000 buses, Poisson "
                                   "2000 req/s, 0.5% breaker edits, hot start, max|dx| < 1e-6",
                       "step": "%d requests" % STEP_REQUESTS, "timed_requests": hi - lo,
                       "buses_total": int(sum(g.n_bus for g in stream.grids)),
                       "parallelism": "replicas" if world > 1 else "single",
                       "l2": "fleet working set %.1f GB > L2" % (sm["device_bytes"] / 1e9)},
            "latency_ms": {"p50": pct(sm["lat"], 50), "p99": pct(sm["lat"], 99),
                           "p50_below_20k": pct(sm["lat_small"], 50), "p99_below_20k": pct(sm["lat_small"], 99),
                           "p50_20k_plus": pct(sm["lat_big"], 50), "p99_20k_plus": pct(sm["lat_big"], 99)},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": sm["h2d_total"] // args.steps,
                    "d2h_bytes_per_step": sm["d2h_total"] // args.steps},
            "gpu_launches": sm["launches"],
            "served_fp64": {"value": round((hi - lo) / sf["elapsed_s"], 3), "p50": pct(sf["lat"], 50),
                            "p99": pct(sf["lat"], 99)},
            "per_grid_fp64": {"value": pg, "p50": per_grid["service_ms"]["p50"],
                              "p99": per_grid["service_ms"]["p99"]},
            "served_mixed_vs_per_grid_fp64": round(value / pg, 3) if pg else None,
            "state_err_vs_oracle": {"mixed": err_mixed, "fp64": err_fp64, "requests": len(sample)},
            "served": {"ok": sm["ok"], "status_counts": sm["status_counts"], "not_ok_breaker": sm["not_ok_breaker"],
                       "iterations_mean": round(sm["iters"], 3), "mean_batch": round(sm["batch"], 2)},
            "clocks": sm["clk"],
        }
        if union:
            out["roofline"] = {k: union[k] for k in ("bound", "kernel", "achieved", "peak", "unit", "frac", "traffic")}
            out["roofline"]["workload"] = "one loaded Gauss-Newton pass of the 512-grid batch (factorisation stage)"
    return out, stream, (lo, hi)


def summarize_leg(mixed, fp64, g, a, world):
    def summary(leg):
        lat = np.array(leg["times"])
        return {"value": round(world * a.steps / (leg["total_ms"] * 1e-3), 3),
                "ms_per_step": round(leg["total_ms"] / a.steps, 5),
                "latency_ms": {"p50": round(float(np.percentile(lat, 50)), 4),
                               "p99": round(float(np.percentile(lat, 99)), 4)},
                "e2e": {"value": round(world * a.steps / (leg["e2e_total"] * 1e-3), 3), "unit": UNIT,
                        "h2d_bytes_per_step": 8 * g.n_meas, "d2h_bytes_per_step": 16 * g.n_bus},
                "iterations_per_solve": round(float(np.mean(leg["iters"])), 3),
                "gpu_launches": int(leg["launches"]),
                "stages_ms_per_solve": {k: round(v / max(a.steps, 1), 5) for k, v in leg["stage_ms"].items()}}
    sm, sf = summary(mixed), summary(fp64)
    err = float(max(np.abs(mixed["v"] - fp64["v"]).max(), np.abs(mixed["th"] - fp64["th"]).max()))
    info = mixed["info"]
    return {
        "config": "grid10k hot-start solves: %d buses, %d branches, %d rows, %d states; 1%% of rows re-noised per "
                  "step; device-resident telemetry, L2 flushed (256 MiB write) before every step"
                  % (g.n_bus, g.n_branch, g.n_meas, 2 * g.n_bus - 1),
        "mixed": dict(sm, roofline=roofline(mixed, g, True)),
        "fp64": dict(sf, roofline=roofline(fp64, g, False)),
        "mixed_vs_fp64_max_state_err": err,
        "plan": {"nnz_l": info.nnz_l, "n_super": info.n_super, "levels": info.n_levels,
                 "max_front": info.max_front, "factor_flops": info.factor_flops},
    }


def main():
    args = parse()
    world, rank, local = dist_setup()
    if args.only:
        if args.only == "batch512":
            out = run_batch512()
        elif args.only == "union_roofline":
            out = run_union_roofline(local, args.union_passes)
        elif args.only == "grid200k":
            out = run_grid200k()
        else:
            from state_estimation_with_cuda_gb300 import workloads

            a10 = argparse.Namespace(**vars(args))
            a10.steps, a10.warmup = args.grid10k_steps, 3
            g10 = workloads.make("grid10k")
            snaps10 = [g10.renoise(u).copy() for u in range(a10.warmup + a10.steps)]
            out = summarize_leg(run_leg(a10, g10, snaps10, local, True, world),
                                run_leg(a10, g10, snaps10, local, False, world), g10, a10, world)
        if rank == 0:
            print(json.dumps({"only": args.only, **out}))
        return
    if args.impl == "reference":
        if rank != 0:
            return
        lo, hi = args.warmup * STEP_REQUESTS, (args.warmup + args.steps) * STEP_REQUESTS
        stream = Stream(hi)
        oracle_served(stream, 0, min(lo, STEP_REQUESTS), 0.5)  # warm-up (untimed)
        value, times, cores = oracle_served(stream, lo, hi, REF_STEP_SECONDS)
        line = {
            "metric": METRIC, "value": round(value, 4), "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": round(1e3 * STEP_REQUESTS / value, 3), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded generator)",
            "config": {"workload": "serving form (as the gb300 arm): the CPU FP64 oracle serves every "
                                   "%d-request window in arrival order, one request at a time, for %.0f s of "
                                   "solves a window" % (STEP_REQUESTS, REF_STEP_SECONDS),
                       "step": "%d requests" % STEP_REQUESTS},
            "impl": "reference",
            "cpu_baseline": {"value": round(value, 4), "unit": UNIT, "cores": cores, "kind": "port",
                             "sample": "%d requests (the first of each window, %.0f s of solves a window; %.1f s "
                                       "in all); a grid's first request starts from its true state, later ones "
                                       "from the previous estimate" % (len(times), REF_STEP_SECONDS, sum(times))},
            "e2e": {"value": round(value, 4), "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        }
        print(json.dumps(line))
        return
    out, stream, (lo, hi) = run_gb300(args, world, rank, local)
    if rank == 0:
        if world == 1 and not args.no_cpu_baseline:
            value, times, cores = oracle_served(stream, lo, hi, args.cpu_seconds / max(args.steps, 1))
            out["cpu_baseline"] = {"value": round(value, 4), "unit": UNIT, "cores": cores, "kind": "port",
                                   "sample": "%d requests of the timed windows (the first of each, %.1f s of solves "
                                             "a window; %.1f s in all)"
                                             % (len(times), args.cpu_seconds / max(args.steps, 1), sum(times))}
        print(json.dumps(out))
    if world > 1:
        import torch.distributed as dist

        dist.destroy_process_group()


if __name__ == "__main__":
    main()
