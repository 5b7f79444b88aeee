"""Serving loop on the GPU: jobs admitted by HBM budget, advanced together
while others arrive, each result equal to the same job run alone within the
mixed form's tolerance (1e-4 of its displacement / velocity scales)."""
import numpy as np
import pytest

from openradioss_gb300 import model as M

pytestmark = pytest.mark.gpu


def test_served_results_equal_alone():
    from openradioss_gb300.engine import Engine
    from openradioss_gb300.serving import Server, estimate_device_bytes
    jobs = [(0, M.crash_box(n_side=5, n_len=10, seed=11), 120, 0.0),
            (1, M.hexa_impact_block(2500, seed=12, law="law1"), 90, 0.0),
            (2, M.crash_box(n_side=7, n_len=8, seed=13, thk=1.5e-3), 60, 0.05),
            (3, M.hexa_impact_block(1800, seed=14, law="law2"), 150, 0.1),
            (4, M.crash_box(n_side=4, n_len=16, seed=15, v0=19.0), 80, 0.1)]
    # budget for about two jobs at a time: admission must wait for retirements
    need = sorted(estimate_device_bytes(m, 1) for _, m, _, _ in jobs)
    budget = need[-1] + need[-2]
    srv = Server(budget, max_jobs=8, precision=1, step_cycles=25, keep_results=True,
                 executor="batch")
    stats = srv.run(jobs)
    srv.close()
    assert stats["jobs"] == 5 and len(srv.done) == 5
    assert stats["max_used_bytes"] <= budget
    for rec in srv.done:
        _, m, n, _ = jobs[rec.key]
        assert rec.device_bytes <= estimate_device_bytes(m, 1)
        ref = Engine(m, precision=1)
        ref.cycle(n)
        nd = ref.nodes()
        assert rec.result["time"]["ncycle"] == n
        sd = np.max(np.abs(nd["X"] - m.X))
        assert np.max(np.abs(rec.result["X"] - nd["X"])) <= 1e-4 * sd, rec.key
        assert np.max(np.abs(rec.result["V"] - nd["V"])) <= 1e-4 * np.max(np.abs(nd["V"])), rec.key
        assert rec.result["status"] == 0
    assert stats["p99_latency_s"] >= stats["p50_latency_s"] > 0.0


def test_streams_executor_results_equal_alone_bitwise():
    """The streams executor runs each job's own single-model graph on the
    job's own stream: a served job ends bit for bit where the same job run
    alone ends, whatever runs beside it."""
    from openradioss_gb300.engine import Engine
    from openradioss_gb300.serving import Server, estimate_device_bytes
    jobs = [(0, M.crash_box(n_side=5, n_len=10, seed=11), 130, 0.0),
            (1, M.hexa_impact_block(2500, seed=12, law="law2"), 90, 0.0),
            (2, M.crash_box(n_side=7, n_len=8, seed=13, thk=1.5e-3), 70, 0.05),
            (3, M.hexa_impact_block(1800, seed=14, law="law2"), 150, 0.1)]
    need = sorted(estimate_device_bytes(m, 1) for _, m, _, _ in jobs)
    budget = need[-1] + need[-2]
    for prec in (1, 0):
        srv = Server(budget, max_jobs=8, precision=prec, step_cycles=40, keep_results=True,
                     executor="streams")
        stats = srv.run(jobs)
        srv.close()
        assert stats["completed"] == 4 and stats["max_used_bytes"] <= budget
        for rec in srv.done:
            _, m, n, _ = jobs[rec.key]
            ref = Engine(m, precision=prec)
            ref.cycle(n)
            nd = ref.nodes()
            assert rec.result["time"]["ncycle"] == n
            assert np.array_equal(rec.result["X"], nd["X"]), rec.key
            assert np.array_equal(rec.result["V"], nd["V"]), rec.key
            assert rec.result["status"] == 0
