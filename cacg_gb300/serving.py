"""Open-loop load driver for the solve server (cacg_server_*).

Serving workload: a stream of SPD requests with Poisson arrivals, each a 2-D
5-point or 3-D 7-point Laplacian (50/50) with n log-uniform in [1e3, 1e6], a
diagonal shift U[0, 0.1], 1-16 right-hand sides (uniform integer) of N(0, 1)
values, all drawn from one seeded generator.

Latency of a request = its completion time - its scheduled arrival time, so
it includes queueing, admission under the memory budget, the host<->device
copies and the solve.  Requests are built on a producer thread ahead of their
arrival (building is the client's work, not the server's), submitted at their
arrival times, and a poller thread timestamps completions.
"""
from __future__ import annotations

import math
import queue
import threading
import time

import numpy as np

from . import solver as S


def request_specs(count: int, seed: int = 4, nmin: float = 1e3, nmax: float = 1e6):
    """Request shapes of the serving workload (kind, grid edge, shift, RHS, RHS seed)."""
    rng = np.random.default_rng(seed)
    specs = []
    for _ in range(count):
        kind = "lap2d" if rng.random() < 0.5 else "lap3d7"
        n_target = math.exp(rng.uniform(math.log(nmin), math.log(nmax)))
        N = max(2, int(round(n_target ** (0.5 if kind == "lap2d" else 1.0 / 3.0))))
        specs.append(dict(kind=kind, N=N, shift=float(rng.uniform(0.0, 0.1)),
                          m=int(rng.integers(1, 17)), seed=int(rng.integers(1, 2 ** 31 - 1))))
    return specs


def build_request(spec):
    rp, ci, v = S.gen_matrix(spec["kind"], spec["N"], shift=spec["shift"])
    B = S.gen_rhs("normal", len(rp) - 1, spec["m"], spec["seed"])
    return rp, ci, v, B


def _percentile(x, q):
    return float(np.percentile(np.asarray(x, np.float64), q)) if len(x) else None


def run(specs, params: S.Params, rate: float | None, mem_budget: int, max_active: int,
        prefetch: int = 16, poll_interval: float = 2e-4, arrival_seed: int = 12345,
        engine: str = "batched", batch_max_rows: int = 0, prebuild: bool = False):
    """Drive the server with `specs`.  rate = requests/s of the Poisson
    arrivals, or None for a closed burst (everything arrives at t = 0).
    prebuild: every request is built before the clock starts (otherwise a
    producer thread builds them at most `prefetch` ahead of submission).
    Returns a dict of latencies (s), throughput and per-request outcomes."""
    srv = S.Server(mem_budget, max_active, engine=engine, batch_max_rows=batch_max_rows)
    built: queue.Queue = queue.Queue(maxsize=len(specs) if prebuild else prefetch)

    def producer():
        for sp in specs:
            built.put(build_request(sp))

    if prebuild:
        producer()
    else:
        threading.Thread(target=producer, daemon=True).start()
    K = len(specs)
    if rate:
        gaps = np.random.default_rng(arrival_seed).exponential(1.0 / rate, K)
        sched = np.concatenate([[0.0], np.cumsum(gaps)[:-1]])
    else:
        sched = np.zeros(K)
    outstanding: dict[int, int] = {}
    done: dict[int, tuple[float, dict]] = {}
    lock = threading.Lock()
    submitted_all = threading.Event()
    errors: list[BaseException] = []

    def poller():
        try:
            while True:
                with lock:
                    items = list(outstanding.items())
                    if submitted_all.is_set() and not items:
                        return
                for t, i in items:
                    r = srv.poll(t)
                    if r is not None:
                        now = time.perf_counter()
                        with lock:
                            outstanding.pop(t)
                            done[i] = (now, r[1])
                time.sleep(poll_interval)
        except BaseException as e:  # surfaced to the caller
            errors.append(e)

    # the first request is built before the clock starts
    first = built.get()
    pol = threading.Thread(target=poller, daemon=True)
    pol.start()
    t0 = time.perf_counter()
    try:
        for i in range(K):
            rp, ci, v, B = first if i == 0 else built.get()
            target = t0 + sched[i]
            while True:
                d = target - time.perf_counter()
                if d <= 0:
                    break
                time.sleep(min(d, 5e-4))
            t = srv.submit(rp, ci, v, B, params)
            with lock:
                outstanding[t] = i
    finally:
        submitted_all.set()
        pol.join()
        engine_stats = srv.engine_stats()
        srv.close()
    if errors:
        raise errors[0]
    lat = [done[i][0] - (t0 + sched[i]) for i in range(K)]
    end = max(done[i][0] for i in range(K))
    infos = [done[i][1] for i in range(K)]
    rhs = sum(sp["m"] for sp in specs)
    return {"latency_s": lat, "makespan_s": end - t0, "requests_per_s": K / (end - t0),
            "rhs_per_s": rhs / (end - t0), "infos": infos, "engine": engine_stats}


def summarize(res, specs, tol):
    lat_ms = [1e3 * x for x in res["latency_s"]]
    st = [i["status"] for i in res["infos"]]
    rr = [i["true_relres_max"] for i in res["infos"]]
    return {"requests": len(specs), "p50_ms": _percentile(lat_ms, 50),
            "p99_ms": _percentile(lat_ms, 99), "mean_ms": float(np.mean(lat_ms)),
            "max_ms": float(np.max(lat_ms)), "rhs_per_s": res["rhs_per_s"],
            "requests_per_s": res["requests_per_s"],
            "all_converged": all(s == 0 for s in st) and max(rr) <= tol,
            "true_relres_max": float(max(rr))}


def main(argv=None):
    """Command line: one run of the serving stream's first `--requests`
    requests (a closed burst, or Poisson arrivals at `--rate` requests/s),
    printing the latency summary and the engine's counters as one JSON line.
    Example: python -m cacg_gb300.serving --requests 64 --max-rows 65536 --prebuild"""
    import argparse
    import json

    ap = argparse.ArgumentParser(prog="python -m cacg_gb300.serving")
    ap.add_argument("--requests", type=int, default=64)
    ap.add_argument("--precision", choices=["mixed", "fp64"], default="mixed")
    ap.add_argument("--engine", choices=["batched", "streams"], default="batched")
    ap.add_argument("--rate", type=float, default=None, help="requests/s (default: closed burst)")
    ap.add_argument("--max-active", type=int, default=32)
    ap.add_argument("--max-rows", type=float, default=1e6,
                    help="largest request size of the stream (n log-uniform in [1e3, this])")
    ap.add_argument("--budget-gb", type=int, default=120)
    ap.add_argument("--seed", type=int, default=4)
    ap.add_argument("--prebuild", action="store_true",
                    help="build every request before the clock starts")
    a = ap.parse_args(argv)
    specs = request_specs(a.requests, seed=a.seed, nmax=a.max_rows)
    p = S.Params(s=4, bounds="gerschgorin", tol=1e-8, maxit=3000, precision=a.precision,
                 rr_period=5)
    res = run(specs, p, a.rate, a.budget_gb << 30, a.max_active, engine=a.engine,
              prebuild=a.prebuild)
    out = summarize(res, specs, 1e-8)
    out.update(engine=a.engine, precision=a.precision, engine_stats=res["engine"])
    print(json.dumps(out))


if __name__ == "__main__":
    main()
