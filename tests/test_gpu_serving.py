"""The serving loop (cupic_gb300.serve) on the GPU.

Requests arriving while others run are admitted into the running batch by
footprint; each request's result (the time-averaged probe current) must be
the one it gets when run alone with the plain one-at-a-time method, exactly.
"""
import copy

import pytest

import cupic_gb300 as cg
from cupic_gb300 import serve
from cupic_gb300.params import bias_instances, footprint_bytes

pytestmark = pytest.mark.gpu


def requests(n=10, rate=400.0, steps=200, window=100):
    ps = bias_instances(n, seed=7, sweeps=50, sizes=(32, 64))
    t = serve.poisson_arrivals(n, rate, seed=3)
    return [serve.Request(k, p, float(t[k]), steps=steps, window=window) for k, p in enumerate(ps)]


@pytest.mark.parametrize("budget_fraction", [1.0, 0.3])
def test_each_result_is_the_same_alone_and_in_the_mix(gpu_lib, budget_fraction):
    reqs = requests()
    budget = int(budget_fraction * sum(footprint_bytes(r.params) for r in reqs))
    budget = max(budget, max(footprint_bytes(r.params) for r in reqs))
    mixed = serve.serve_batched(copy.deepcopy(reqs), budget_bytes=budget, tick=20)
    alone = serve.serve_plain(copy.deepcopy(reqs))
    for m, a in zip(sorted(mixed, key=lambda r: r.rid), sorted(alone, key=lambda r: r.rid)):
        assert m.current == a.current, f"request {m.rid}"
        assert m.finish >= m.start >= m.arrival
    s = serve.summary(mixed)
    assert s["solves"] == len(reqs) and s["p99_ms"] >= s["p50_ms"] > 0


def test_a_failing_request_leaves_alone(gpu_lib):
    """A request whose electrons the probe drives across two rows in one
    step (a bias of -5000 Te/e) fails with its device flag, in the batch and
    alone; every other request gets the result it gets alone."""
    reqs = requests()
    bad = reqs[3]
    bad.params.phi_p = -5000.0
    mixed = serve.serve_batched(copy.deepcopy(reqs), tick=20)
    alone = serve.serve_plain(copy.deepcopy(reqs))
    for m, a in zip(sorted(mixed, key=lambda r: r.rid), sorted(alone, key=lambda r: r.rid)):
        if m.rid == bad.rid:
            assert m.error and a.error and m.current is None and a.current is None
        else:
            assert m.error is None and m.current == a.current, f"request {m.rid}"
    s = serve.summary(mixed)
    assert s["failed"] == 1 and s["solves"] == len(reqs) - 1
