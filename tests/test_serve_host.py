"""Host-side logic of the serving loop and the bias-point workload, on CPU:
arrival streams, admission footprints, the instance generator and the
summary of a finished stream (failed requests included)."""
import numpy as np
import pytest

from cupic_gb300 import serve
from cupic_gb300.params import bias_instances, footprint_bytes


def test_poisson_arrivals_are_seeded_and_increasing():
    a = serve.poisson_arrivals(1000, 100.0, seed=3)
    b = serve.poisson_arrivals(1000, 100.0, seed=3)
    np.testing.assert_array_equal(a, b)
    assert np.all(np.diff(a) > 0)
    # mean gap 1/rate within 10% over 1000 arrivals
    assert np.mean(np.diff(a)) == pytest.approx(0.01, rel=0.1)


def test_footprint_is_16_bytes_per_particle_and_12_per_cell():
    p = bias_instances(1, seed=2)[0]
    particles = 2 * p.ppr * p.ncy
    assert footprint_bytes(p) == 16 * particles + 12 * p.ncx * p.ncy


def test_bias_instances_follow_the_drawn_distribution():
    ps = bias_instances(256, seed=2)
    assert {p.ncx for p in ps} <= {32, 64, 128, 256}
    assert all(p.ncy == 4 * p.ncx for p in ps)
    ppc = [p.n * p.ds ** 3 for p in ps]
    assert min(ppc) >= 10 - 1e-9 and max(ppc) <= 50 + 1e-9
    assert all(-10.0 <= p.phi_p <= 2.0 for p in ps)
    assert all(p.mi == 1836.0 and p.kti == pytest.approx(0.1) for p in ps)
    assert all(p.min_sweeps == p.max_sweeps == 200 for p in ps)
    assert len({p.seed for p in ps}) == 256
    # the same seed draws the same instances
    again = bias_instances(256, seed=2)
    assert [(p.ncx, p.ppr, p.phi_p) for p in ps] == [(q.ncx, q.ppr, q.phi_p) for q in again]


def request(rid, arrival, start, finish, error=None):
    r = serve.Request(rid, None, arrival)
    r.start, r.finish, r.error = start, finish, error
    r.current = None if error else 0.0
    return r


def test_summary_counts_failed_requests_apart():
    reqs = [request(0, 0.0, 0.0, 1.0), request(1, 0.5, 0.5, 2.0),
            request(2, 1.0, 1.0, 1.5, error="device flags 0x1"), request(3, 1.0, 1.2, 4.0)]
    s = serve.summary(reqs)
    assert s["solves"] == 3 and s["failed"] == 1
    assert s["seconds"] == pytest.approx(4.0)
    assert s["solves_per_s"] == pytest.approx(3 / 4.0)
    lat = np.array([1.0, 1.5, 3.0])
    assert s["p50_ms"] == pytest.approx(1e3 * np.percentile(lat, 50))
    assert s["p99_ms"] == pytest.approx(1e3 * np.percentile(lat, 99))


def test_summary_of_a_stream_where_every_request_failed():
    s = serve.summary([request(0, 0.0, 0.0, 1.0, error="device flags 0x4")])
    assert s["solves"] == 0 and s["failed"] == 1 and s["solves_per_s"] == 0.0


class FakeSim:
    """Stands in for a context: `fail_at` steps in, its rows cannot grow,
    which the library reports as CUPIC_FLAG_CAPACITY (0x2) on the context."""

    def __init__(self, params, device=0):
        self.p = params
        self.done = 0
        self.fail_at = getattr(params, "fail_at", None)

    def init_plasma(self, wait=True):
        pass

    def sync(self):
        pass

    def failed(self):
        return self.fail_at is not None and self.done >= self.fail_at

    def flags(self):
        return 0x2 if self.failed() else 0

    def probe_current(self, window):
        return float(self.p.rid)

    def close(self):
        pass


class FakeBatch:
    def __init__(self, sims=(), device=0):
        self.members = list(sims)

    def set(self, sims):
        self.members = list(sims)

    def step(self, n=1, sync=True):
        for s in self.members:
            s.done += n

    def sync(self):
        if any(s.failed() for s in self.members):
            from cupic_gb300 import CupicError
            raise CupicError(5, "batch_sync")

    def close(self):
        pass


class FakeParams:
    def __init__(self, rid, fail_at=None):
        self.rid, self.fail_at = rid, fail_at
        self.ncx, self.ncy, self.ppr = 32, 128, 320
        self.check_every = self.max_sweeps = self.init_max_sweeps = 200


def test_a_request_whose_rows_cannot_grow_fails_alone(monkeypatch):
    """A member whose halted run cannot grow its rows reports the capacity
    flag; the serving loop ends that request with its error and finishes
    the others with their own results."""
    monkeypatch.setattr(serve, "Sim", FakeSim)
    monkeypatch.setattr(serve, "Batch", FakeBatch)
    monkeypatch.setattr(serve, "reserve", lambda *a, **k: None)
    reqs = [serve.Request(k, FakeParams(k, fail_at=30 if k == 1 else None), 0.0, steps=100,
                          window=50) for k in range(3)]
    out = serve.serve_batched(reqs, tick=20)
    byid = {r.rid: r for r in out}
    assert byid[1].error == "device flags 0x2" and byid[1].current is None
    assert byid[0].current == 0.0 and byid[2].current == 2.0
    assert byid[0].error is None and byid[2].error is None
