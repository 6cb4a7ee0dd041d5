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


@pytest.mark.parametrize("engine", ["batched", "streams"])
def test_results_identical_alone_and_in_mix(lib, engine):
    reqs = _requests()
    alone = []
    srv = cg.Server(mem_budget_bytes=2 << 30, max_active=1, engine=engine)
    for r in reqs:
        t = srv.submit(*r)
        alone.append(srv.wait(t))
    srv.close()
    srv = cg.Server(mem_budget_bytes=2 << 30, max_active=4, engine=engine)
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


def test_batched_fp64_matches_reference(lib):
    """The batched engine's FP64 requests with the reference's stopping test
    (||R(:,0)|| < eps, Gerschgorin bounds) against the reference bcbcg_v1 /
    cbcg_v1 on the same inputs: outer iterations within +-1, solution within
    1e-6, while sharing every launch with other requests."""
    specs = [("lap2d", 48, 4, 4), ("lap3d7", 16, 8, 4), ("lap2d", 64, 1, 4), ("lap3d7", 12, 3, 5),
             ("lap2d", 40, 16, 4)]
    reqs = []
    for i, (kind, N, m, s_) in enumerate(specs):
        rp, ci, v = cg.gen_matrix(kind, N, shift=0.02 * i)
        B = cg.gen_rhs("normal", len(rp) - 1, m, 200 + i)
        eps = 1e-8 * float(np.linalg.norm(B[:, 0]))
        p = cg.Params(s=s_, bounds="gerschgorin", tol=eps, tol_mode="abs_col0", maxit=1000,
                      precision="fp64")
        reqs.append((rp, ci, v, B, p))
    srv = cg.Server(mem_budget_bytes=2 << 30, max_active=8)
    tickets = [srv.submit(*r) for r in reqs]
    outs = [srv.wait(t) for t in tickets]
    st = srv.engine_stats()
    srv.close()
    assert st["steps"] > 0 and st["graph_replays"] == st["steps"]
    for (rp, ci, v, B, p), (X, info) in zip(reqs, outs):
        if O.ref_available():
            Xr, itr, _, _ = O.ref_solve(rp, ci, v, B, np.zeros_like(B), p.s, p.tol, None, 1000)
        else:
            Xr, itr, _ = O.port_solve(rp, ci, v, B, np.zeros_like(B), p.s, p.tol, None, 1000)
        assert info["status"] == 0
        assert abs(info["iterations"] - itr) <= 1, (info["iterations"], itr)
        assert np.linalg.norm(X - Xr) / np.linalg.norm(Xr) <= 1e-6


def test_batched_edge_shapes(lib):
    """Shapes at the batched kernels' edges, all in one batch: one partial row
    tile (n = 81), k not a multiple of 4 (21, 25, 51), m = 1 and m = 32, k = 64
    (at m = 32 the Gram's tile count exceeds the block and takes two passes),
    and a request of many Gram pieces (n = 40,000).  FP64 requests against the
    oracle's bcbcg (outer iterations within +-1, solution within 1e-6); mixed
    requests reach the tolerance on the true residual."""
    specs = [("lap2d", 9, 1, 2), ("lap3d7", 10, 32, 2), ("lap2d", 30, 8, 8), ("lap2d", 37, 7, 3),
             ("lap3d7", 13, 5, 5), ("lap2d", 200, 3, 4), ("lap3d7", 11, 17, 3)]
    reqs = []
    for i, (kind, N, m, s_) in enumerate(specs):
        rp, ci, v = cg.gen_matrix(kind, N, shift=0.05 + 0.01 * i)
        B = cg.gen_rhs("normal", len(rp) - 1, m, 300 + i)
        eps = 1e-8 * float(np.linalg.norm(B[:, 0]))
        p64 = cg.Params(s=s_, bounds="gerschgorin", tol=eps, tol_mode="abs_col0", maxit=1000,
                        precision="fp64")
        pmx = cg.Params(s=s_, bounds="gerschgorin", tol=1e-8, maxit=1000, precision="mixed")
        reqs.append((rp, ci, v, B, p64))
        reqs.append((rp, ci, v, B, pmx))
    srv = cg.Server(mem_budget_bytes=4 << 30, max_active=16)
    tickets = [srv.submit(*r) for r in reqs]
    outs = [srv.wait(t) for t in tickets]
    st = srv.engine_stats()
    srv.close()
    assert st["steps"] > 0
    for (rp, ci, v, B, p), (X, info) in zip(reqs, outs):
        assert info["status"] == 0, (len(rp) - 1, B.shape, p.s, p.precision)
        if p.precision == "fp64":
            if O.ref_available():
                Xr, itr, _, _ = O.ref_solve(rp, ci, v, B, np.zeros_like(B), p.s, p.tol, None, 1000)
            else:
                Xr, itr, _ = O.port_solve(rp, ci, v, B, np.zeros_like(B), p.s, p.tol, None, 1000)
            assert abs(info["iterations"] - itr) <= 1, (info["iterations"], itr)
            assert np.linalg.norm(X - Xr) / np.linalg.norm(Xr) <= 1e-6
        else:
            assert O.port_true_relres(rp, ci, v, B, X).max() <= 1e-8


def test_batched_graph_replay_equals_direct_launches(lib):
    """Replaying the captured step and launching it directly give the same
    bits (FP64 and mixed requests in one batch)."""
    reqs = _requests()
    res = []
    for graphs in (True, False):
        srv = cg.Server(mem_budget_bytes=2 << 30, max_active=6, graphs=graphs)
        tickets = [srv.submit(*r) for r in reqs]
        res.append([srv.wait(t) for t in tickets])
        st = srv.engine_stats()
        srv.close()
        assert (st["graph_replays"] > 0) == graphs
    for (Xa, ia), (Xb, ib) in zip(*res):
        assert np.array_equal(Xa, Xb) and ia["iterations"] == ib["iterations"]


def test_autotuner_choices(lib):
    srv = cg.Server(mem_budget_bytes=1 << 30, max_active=2)
    r = _requests()[1]  # a mixed request: tunes the FP32 class
    srv.wait(srv.submit(*r))
    st = srv.engine_stats()
    srv.close()
    assert all(v in (1, 2, 4, 8) for v in st["blocks_per_sm"]["fp32"].values())


def test_requests_beyond_batched_limits_run_on_stream_worker(lib):
    """k = s m > 64, Lanczos bounds and more rows than batch_max_rows leave
    the batched kernels; such requests still complete, next to batched ones."""
    rp, ci, v = cg.gen_matrix("lap2d", 40, shift=0.01)
    B = cg.gen_rhs("normal", 1600, 20, 5)
    big = cg.Params(s=4, bounds="gerschgorin", tol=1e-8, maxit=500, precision="fp64")  # k = 80
    lz = cg.Params(s=4, bounds=("lanczos", 30), tol=1e-8, maxit=500, precision="mixed")
    srv = cg.Server(mem_budget_bytes=2 << 30, max_active=4, batch_max_rows=1000)
    t1 = srv.submit(rp, ci, v, B, big)
    t2 = srv.submit(rp, ci, v, B[:, :4].copy(), lz)
    t3 = srv.submit(*_requests()[0])  # 1600 rows > batch_max_rows
    t4 = srv.submit(*_requests()[5])  # 1000 rows: batched
    outs = [srv.wait(t) for t in (t1, t2, t3, t4)]
    st = srv.engine_stats()
    srv.close()
    assert st["steps"] > 0
    for X, info in outs:
        assert info["status"] == 0 and info["true_relres_max"] <= 1e-8
    assert O.port_true_relres(rp, ci, v, B, outs[0][0]).max() <= 1e-8
