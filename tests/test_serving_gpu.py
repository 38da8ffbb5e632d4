"""Serving (continuous batching): every job's result equals the same job run
alone, whether it runs alone on the server or mixed with other jobs that
arrive while it is on the GPU (MI and GC bit-exact; APSP bit-exact)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _alone(req):
    from netsci_gb300 import serving
    res, _ = serving.run_plain([serving.Request(0.0, req.kind, req.params, req.data)])
    return res[0]


def test_results_same_alone_and_in_the_mix():
    from netsci_gb300 import serving
    trace = serving.c5_trace(14, seed=11, rate=400.0, scale=0.12)
    kinds = {r.kind for r in trace}
    assert {"gc", "mi"} <= kinds
    with serving.Server(budget_bytes=4 << 30, tick_ops=2e9) as srv:
        mixed, summary = serving.run_served(srv, trace)
        stats = srv.stats()
    assert stats["jobs_done"] == len(trace)
    # small ticks: several jobs must have shared ticks
    assert stats["ticks"] >= 2
    for r, got in zip(trace, mixed):
        want = _alone(r)
        assert np.array_equal(got, want), r.kind
    assert summary["p99_ms"] >= summary["p50_ms"] > 0


def test_server_one_job_each_kind_and_budget():
    from netsci_gb300 import serving, synthetic
    X, _ = synthetic.protein_trajectory(9, 700, seed=2)
    x, y = synthetic.gaussian_pair(1500, 0.6, seed=3)
    A = synthetic.random_geometric_graph(150, 8, seed=4, integer_weights=True)
    with serving.Server(budget_bytes=1 << 30) as srv:
        t = srv.register_trajectory(X, 3)
        jg = srv.submit_gc(t, 9, 6)
        jm = srv.submit_mi(x, y, 1, 4)
        ja = srv.submit_apsp(A, 150)
        gc, mi, H = srv.wait(jg), srv.wait(jm), srv.wait(ja)
        info = srv.info(jg)
    assert info["done"] >= info["admit"] >= info["submit"] > 0
    import oracle
    assert np.array_equal(gc, oracle.pairs(X, 700, 3, synthetic.all_pairs(9), 6, gc=True,
                                           threads=4)) or \
        np.max(np.abs(gc - oracle.pairs(X, 700, 3, synthetic.all_pairs(9), 6, gc=True,
                                        threads=4))) <= 1e-6
    assert float(mi[0]) == oracle.mi_pair(x, y, 1500, 4, 1)
    Ho, _, _ = oracle.apsp_lengths(A, 150)
    assert np.array_equal(H, Ho)


def test_grid_ticks_match_plans():
    """Jobs large enough for the cell-grid search (m >= 2048) share ticks
    with each other and with a small job; every result equals the same job
    run alone through a plan."""
    import torch
    from netsci_gb300 import device, serving, synthetic
    X1, _ = synthetic.protein_trajectory(6, 3000, seed=21)
    X2, _ = synthetic.protein_trajectory(5, 2500, seed=22)
    X3, _ = synthetic.protein_trajectory(4, 600, seed=23)
    x, y = synthetic.gaussian_pair(4000, 0.5, seed=24)

    def alone_gc(X):
        Xd, m = device.pack_trajectory(X, 3)
        pairs = device.make_pairs(Xd, m, synthetic.all_pairs(X.shape[0]))
        g = torch.empty(len(pairs), device="cuda")
        device.ksg_pairs(pairs, 6, 3, gc=g)
        return g.cpu().numpy()

    with serving.Server(budget_bytes=4 << 30, tick_ops=5e9) as srv:
        ts = [srv.register_trajectory(X, 3) for X in (X1, X2, X3)]
        jobs = [srv.submit_gc(t, X.shape[0], 6) for t, X in zip(ts, (X1, X2, X3))]
        jm = srv.submit_mi(x, y, 1, 4)
        got = [srv.wait(j) for j in jobs]
        mi = srv.wait(jm)
        assert srv.stats()["ticks"] >= 2
    for g, X in zip(got, (X1, X2, X3)):
        assert np.array_equal(g, alone_gc(X))
    import oracle
    assert float(mi[0]) == oracle.mi_pair(x, y, 4000, 4, 1)
