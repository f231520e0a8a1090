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
