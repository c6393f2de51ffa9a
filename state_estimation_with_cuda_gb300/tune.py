"""Autotuner for the batched and served forms.

It measures candidate schedules on the device and keeps the fastest:

* batched form: the supernode-width threshold of the high-occupancy dataflow
  phase (``flow_small_f``: fronts whose subtree is at most this wide are
  factorised several CTAs per SM) and the size buckets the grids are split
  into (each bucket one batch, its own CUDA graph per Gauss-Newton step,
  buckets solved concurrently);
* served form: the bus-count bounds of the serving units (``bucket_bus``) and
  the size at which a grid gets a unit of its own (``own_unit_bus``); the
  highest throughput among the candidates whose median latency is within
  1.5x of the best median.

Usage (on a GPU host)::

    python -m state_estimation_with_cuda_gb300.tune --out tuned.json

The result is a JSON object; ``tuned_config()`` reads the copy shipped in
this package (``tuned.json``), which Server and BatchSet use as defaults.
"""
import argparse
import json
import os
import threading
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
TUNED = os.path.join(HERE, "tuned.json")

BATCH_WIDTHS = (32, 64, 96, 128)
SERVE_CANDIDATES = (
    {"bucket_bus": (300, 2000, 20000, 0), "own_unit_bus": 1 << 30},
    {"bucket_bus": (300, 2000, 0, 0), "own_unit_bus": 1 << 30},
    {"bucket_bus": (300, 2000, 20000, 80000), "own_unit_bus": 1 << 30},
    {"bucket_bus": (500, 5000, 50000, 0), "own_unit_bus": 1 << 30},
    {"bucket_bus": (500, 5000, 0, 0), "own_unit_bus": 1 << 30},
    {"bucket_bus": (300, 2000, 10000, 50000), "own_unit_bus": 1 << 30},
    {"bucket_bus": (300, 2000, 20000, 0), "own_unit_bus": 100000},
)


def tuned_config():
    """The shipped tuning result ({} when absent)."""
    try:
        with open(TUNED) as fh:
            return json.load(fh)
    except (OSError, ValueError):
        return {}


class BatchSet:
    """Grids split into size buckets, one BatchEstimator per bucket, buckets
    solved concurrently (one host thread each; ctypes releases the GIL)."""

    def __init__(self, grids, bounds, mixed=True, flow_small_f=None):
        from .api import BatchEstimator

        self.bounds = sorted(b for b in bounds if b > 0)
        self.buckets = []  # (estimator, [global grid ids])
        groups = {}
        for i, g in enumerate(grids):
            k = 0
            while k < len(self.bounds) and g.n_bus > self.bounds[k]:
                k += 1
            groups.setdefault(k, []).append(i)
        self.where = {}
        for k in sorted(groups):
            b = BatchEstimator(mixed=mixed)
            if flow_small_f:
                b.set_option("flow_small_f", flow_small_f)
            for j, i in enumerate(groups[k]):
                b.add_grid(grids[i])
                self.where[i] = (len(self.buckets), j)
            self.buckets.append((b, groups[k]))
        for b, _ in self.buckets:
            b.upload_model()

    def set_telemetry(self, i, z):
        k, j = self.where[i]
        self.buckets[k][0].set_telemetry(j, z)

    def solve(self, flat_start=False, **kw):
        out = [None] * len(self.buckets)

        def run(k):
            out[k] = self.buckets[k][0].solve(flat_start=flat_start, **kw)

        th = [threading.Thread(target=run, args=(k,)) for k in range(len(self.buckets))]
        for t in th:
            t.start()
        for t in th:
            t.join()
        res = {}
        for k, (_, ids) in enumerate(self.buckets):
            for j, i in enumerate(ids):
                res[i] = out[k][j]
        return [res[i] for i in sorted(res)]

    def close(self):
        for b, _ in self.buckets:
            b.close()


def time_batch(grids, snaps, bounds, width, mixed=True):
    bs = BatchSet(grids, bounds, mixed=mixed, flow_small_f=width)
    bs.solve(flat_start=True)
    times = []
    for u in range(len(snaps)):
        t0 = time.perf_counter()
        for i in range(len(grids)):
            bs.set_telemetry(i, snaps[u][i])
        res = bs.solve()
        times.append(time.perf_counter() - t0)
        assert all(r.status == 0 for r in res)
    bs.close()
    return len(grids) * len(times) / sum(times)


def tune_batch(count=512, rounds=2):
    from .workloads import batch_grids

    grids = batch_grids(count)
    snaps = [[g.renoise(u).copy() for g in grids] for u in range(rounds)]
    sizes = np.array(sorted(g.n_bus for g in grids))
    splits = {"1": (), "2": (int(np.median(sizes)),),
              "3": (int(np.percentile(sizes, 33)), int(np.percentile(sizes, 67)))}
    trials = []
    for w in BATCH_WIDTHS:
        for name, b in splits.items():
            v = time_batch(grids, snaps, b, w)
            trials.append({"flow_small_f": w, "bucket_bus": list(b), "solves_per_s": round(v, 1)})
            print("batch", trials[-1], flush=True)
    best = max(trials, key=lambda t: t["solves_per_s"])
    return best, trials


def tune_serving(n_req=800, warm=100):
    from .api import Server
    from .workloads import fleet_grids

    grids = fleet_grids(200)
    snaps = [[g.renoise(u).copy() for u in range(2)] for g in grids]
    rng = np.random.default_rng(0x5E04 + 7)
    arrival = np.cumsum(rng.exponential(1.0 / 2000.0, n_req))
    target = rng.integers(0, len(grids), n_req)
    trials = []
    for cand in SERVE_CANDIDATES:
        s = Server(mixed=True, bucket_bus=cand["bucket_bus"], own_unit_bus=cand["own_unit_bus"])
        for g in grids:
            s.add_grid(g)
        s.start()
        tickets = [None] * n_req

        def submit():
            base = time.perf_counter()
            for i in range(n_req):
                dt = arrival[i] - (time.perf_counter() - base)
                if dt > 0:
                    time.sleep(dt)
                tickets[i] = s.submit(int(target[i]), snaps[int(target[i])][i % 2])

        th = threading.Thread(target=submit)
        th.start()
        res = []
        for i in range(n_req):
            while tickets[i] is None:
                time.sleep(0.0002)
            res.append(s.wait(tickets[i], 3.6e6))
        th.join()
        s.close()
        res = res[warm:]
        el = (max(r.t_done_ns for r in res) - min(r.t_submit_ns for r in res)) / 1e9
        lat = [(r.t_done_ns - r.t_submit_ns) / 1e6 for r in res]
        trials.append({"bucket_bus": list(cand["bucket_bus"]), "own_unit_bus": cand["own_unit_bus"],
                       "solves_per_s": round(len(res) / el, 1), "p50_ms": round(float(np.percentile(lat, 50)), 2),
                       "p99_ms": round(float(np.percentile(lat, 99)), 2)})
        print("serve", trials[-1], flush=True)
    # throughput, among the candidates whose median latency stays within 1.5x
    # of the best median (a schedule that buys throughput with latency loses)
    p50_floor = min(t["p50_ms"] for t in trials)
    ok = [t for t in trials if t["p50_ms"] <= 1.5 * p50_floor]
    best = max(ok, key=lambda t: (t["solves_per_s"], -t["p99_ms"]))
    return best, trials


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--out", default=TUNED)
    ap.add_argument("--skip-serving", action="store_true")
    args = ap.parse_args()
    from .api import Estimator

    e = Estimator()
    e.initialize()
    info = e.lib.sle_GetDeviceInfo(e.h)
    e.close()
    result = {"device": info.decode() if info else "unknown"}
    best, trials = tune_batch()
    result["batch"] = {"best": best, "trials": trials}
    if not args.skip_serving:
        best, trials = tune_serving()
        result["serving"] = {"best": best, "trials": trials}
    with open(args.out, "w") as fh:
        json.dump(result, fh, indent=1)
    print(json.dumps(result))


if __name__ == "__main__":
    main()
