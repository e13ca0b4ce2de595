"""Routing of a request stream over serving slots (host logic, no GPU)."""
from omega_h_gb300.serve import route, summary


def test_route_balances_work_per_dimension():
    dims = [3, 2, 3, 3, 2, 3, 2, 2]
    work = [8, 5, 1, 1, 1, 6, 1, 1]
    where = route(dims, work, {2: 2, 3: 2})
    assert where == [0, 0, 1, 1, 1, 1, 1, 1]
    load = {(d, s): 0 for d in (2, 3) for s in (0, 1)}
    for d, w, s in zip(dims, work, where):
        load[(d, s)] += w
    assert load == {(3, 0): 8, (3, 1): 8, (2, 0): 5, (2, 1): 3}


def test_route_single_slot():
    assert route([2, 3, 2], [1, 2, 3], {2: 1, 3: 1}) == [0, 0, 0]


class _R:
    def __init__(self, arrival, done, ep):
        self.arrival, self.done, self.element_passes = arrival, done, ep


def test_summary_percentiles_and_rate():
    reqs = [_R(0.0, 0.010, 100), _R(0.001, 0.021, 100), _R(0.002, 0.032, 200)]
    s = summary(reqs)
    assert s["requests"] == 3 and abs(s["p50_ms"] - 20.0) < 1e-9 and abs(s["p99_ms"] - 30.0) < 1e-9
    assert abs(s["elements_per_s"] - 400 / 0.032) < 1e-6
