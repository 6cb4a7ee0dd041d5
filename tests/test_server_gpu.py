"""Serving loop: requests admitted under a device-memory budget run
concurrently; each result is bit-identical to the same request solved alone,
and meets its tolerance."""
import numpy as np
import pytest

import cacg_gb300 as cg
import oracle as O

pytestmark = pytest.mark.gpu


def _requests():
    reqs = []
    specs = [("lap2d", 40, 3, "fp64"), ("lap3d7", 14, 8, "mixed"), ("lap2d", 70, 1, "fp64"),
             ("lap3d7", 18, 5, "fp64"), ("lap2d", 33, 16, "mixed"), ("lap3d7", 10, 2, "mixed")]
    for i, (kind, N, m, prec) in enumerate(specs):
        rp, ci, v = cg.gen_matrix(kind, N, shift=0.01 * (i + 1))
        B = cg.gen_rhs("normal", len(rp) - 1, m, 100 + i)
        p = cg.Params(s=4, bounds="gerschgorin", tol=1e-8, maxit=500, precision=prec)
        reqs.append((rp, ci, v, B, p))
    return reqs


def test_results_identical_alone_and_in_mix(lib):
    reqs = _requests()
    alone = []
    srv = cg.Server(mem_budget_bytes=2 << 30, max_active=1)
    for r in reqs:
        t = srv.submit(*r)
        alone.append(srv.wait(t))
    srv.close()
    srv = cg.Server(mem_budget_bytes=2 << 30, max_active=4)
    tickets = [srv.submit(*r) for r in reqs]
    mixed = [srv.wait(t) for t in tickets]
    srv.close()
    for (rp, ci, v, B, p), (Xa, ia), (Xm, im) in zip(reqs, alone, mixed):
        assert ia["status"] == 0 and im["status"] == 0
        assert np.array_equal(Xa, Xm)
        assert ia["iterations"] == im["iterations"]
        assert O.port_true_relres(rp, ci, v, B, Xm).max() <= 1e-8


def test_admission_respects_budget(lib):
    reqs = _requests()
    need = max(cg.lib().cacg_workspace_bytes(len(r[0]) - 1, r[3].shape[1], 4, 0)
               for r in reqs)
    srv = cg.Server(mem_budget_bytes=int(need * 1.6) + (64 << 20), max_active=4)
    tickets = [srv.submit(*r) for r in reqs]
    peak = 0
    done = {}
    while len(done) < len(tickets):
        st = srv.stats()
        peak = max(peak, st["bytes_in_use"])
        for t in tickets:
            if t not in done:
                r = srv.poll(t)
                if r is not None:
                    done[t] = r
    srv.close()
    assert peak <= int(need * 1.6) + (64 << 20)
    assert all(r[1]["status"] == 0 for r in done.values())


def test_oversized_request_refused(lib):
    rp, ci, v = cg.gen_matrix("lap2d", 64)
    B = np.ones((4096, 4))
    srv = cg.Server(mem_budget_bytes=1 << 20, max_active=1)
    with pytest.raises(cg.CacgError) as e:
        srv.submit(rp, ci, v, B, cg.Params())
    srv.close()
    assert e.value.code == -7


def test_open_loop_driver_small_stream(lib):
    """The load driver: Poisson arrivals of small serving-workload requests,
    every request converges and gets a latency >= its own solve time."""
    from cacg_gb300 import serving as SV

    specs = SV.request_specs(16, seed=7, nmin=1e3, nmax=2e4)
    p = cg.Params(s=4, bounds="gerschgorin", tol=1e-8, maxit=3000, precision="mixed")
    res = SV.run(specs, p, rate=200.0, mem_budget=4 << 30, max_active=4)
    summ = SV.summarize(res, specs, 1e-8)
    assert summ["all_converged"], summ
    assert len(res["latency_s"]) == 16
    for lat, info in zip(res["latency_s"], res["infos"]):
        assert lat >= info["seconds"] * 0.99
    assert summ["p99_ms"] >= summ["p50_ms"] > 0
