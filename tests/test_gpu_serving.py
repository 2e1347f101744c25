"""Continuous batching of independent trajectories (the serving ensemble).

Each request's result (final sigma and lead currents) computed in a mix of
overlapping trajectories must equal the result computed alone; the stated
tolerance is 1e-12 (max abs), and the kernels are deterministic so the
results are expected to be identical.  Admission respects the HBM budget.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_results_same_alone_and_in_the_mix():
    import torch
    assert torch.cuda.is_available()
    from zandpack_gb300.serve import Server, c4_estimate
    from zandpack_gb300.workloads import c4_requests, c4_workload
    reqs = c4_requests(12, rate=400.0, seed=77, t_span=0.3)
    mix, stats = Server(c4_workload, c4_estimate, max_slots=6).run(reqs)
    assert stats["completed"] == len(reqs), [r.error for r in mix if r.error]
    assert stats["p99_latency_s"] >= stats["p50_latency_s"] > 0
    alone, _ = Server(c4_workload, c4_estimate, max_slots=1).run(reqs, time_scale=0.0)
    a = {r.id: r for r in alone}
    for r in mix:
        s = a[r.id]
        assert r.attempts == s.attempts and abs(r.t_end - s.t_end) == 0.0
        assert np.abs(r.sigma - s.sigma).max() <= 1e-12
        assert np.abs(r.currents - s.currents).max() <= 1e-12


def test_admission_by_footprint():
    """With a budget for about two trajectories, the server never reserves
    more than the budget and still completes every request."""
    from zandpack_gb300.serve import Server, c4_estimate
    from zandpack_gb300.workloads import c4_requests, c4_workload
    reqs = c4_requests(6, rate=1000.0, seed=78, t_span=0.1)
    budget = 2 * max(c4_estimate(r, "mixed") for r in reqs)
    srv = Server(c4_workload, c4_estimate, max_slots=6, hbm_budget=budget)
    res, stats = srv.run(reqs)
    assert stats["completed"] == len(reqs)
    assert stats["peak_hbm_reserved"] <= budget


def test_graph_mode_matches_host_mode():
    """Graph-launched attempts (controller on the device) serve the same
    results as one zg_attempt call per attempt: same attempt counts, sigma and
    currents to 1e-10 (device and host libm may differ in the last place of
    the bias and the step-size update)."""
    from zandpack_gb300.serve import Server, c4_estimate
    from zandpack_gb300.workloads import c4_requests, c4_workload
    reqs = c4_requests(8, rate=400.0, seed=79, t_span=0.3)
    g, gs = Server(c4_workload, c4_estimate, max_slots=4, attempt_mode="graph").run(reqs, time_scale=0.0)
    h, hs = Server(c4_workload, c4_estimate, max_slots=4, attempt_mode="host").run(reqs, time_scale=0.0)
    assert gs["completed"] == hs["completed"] == len(reqs), [r.error for r in g + h if r.error]
    hm = {r.id: r for r in h}
    for r in g:
        s = hm[r.id]
        assert r.attempts == s.attempts and r.accepted == s.accepted
        assert abs(r.t_end - s.t_end) <= 1e-9 * abs(s.t_end)
        assert np.abs(r.sigma - s.sigma).max() <= 1e-10
        assert np.abs(r.currents - s.currents).max() <= 1e-10
