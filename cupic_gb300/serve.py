"""Serving loop for bias-point requests, and the plain one-at-a-time loop it
is measured against.  There is no counterpart in the reference, which runs
one simulation per process.

A request is one probe-bias instance (a Params set) to run for `steps`
steps; its result is the time-averaged probe current over the last `window`
steps: the net charge absorbed by the probe per step, ions minus electrons.

Continuous batching (``serve_batched``): requests that have arrived are
admitted while their footprint (16 B per particle plus 12 B per cell) fits
the HBM budget and a slot is free; their state is created and initialised
on the device while the running members step (creation and initialisation
are enqueued on the request's own stream and never wait for the device),
and they join the batch at the next tick.  A tick is one ``Batch.step`` of all members (at most `tick`
steps, never past a member's last step); members that finish leave the
batch and free their footprint.  A member's result is bit-identical to the
one it gets alone, because batched and solo steps compute the same thing.
A request whose context reports an error (a device flag: a particle that
crossed two rows, a full staging row, a non-finite coordinate) fails alone:
it leaves with its error and the others run on.
"""
import collections
import dataclasses
import time

import numpy as np

from . import Batch, CupicError, Sim, reserve
from .params import footprint_bytes


@dataclasses.dataclass
class Request:
    rid: int
    params: object
    arrival: float          # seconds after the start of the run
    steps: int = 2000
    window: int = 1000
    start: float = None     # admission time
    finish: float = None    # result time
    current: float = None   # mean net absorbed charge per step over the window
    error: str = None       # why the request failed (it then has no current)

    @property
    def latency(self):
        return self.finish - self.arrival


def poisson_arrivals(n, rate, seed=3):
    """Arrival times of n requests of a Poisson stream of `rate` per second."""
    rng = np.random.default_rng(seed)
    return np.cumsum(rng.exponential(1.0 / rate, size=n))


def probe_current(sim, window):
    return sim.probe_current(window)


def warm_plans(requests, device=0):
    """Creates one context per distinct mesh shape so that the solver layout
    of each shape is tuned (and cached) before the clock starts."""
    seen = set()
    for r in requests:
        p = r.params
        key = (p.ncx, p.ncy, p.check_every, p.max_sweeps, p.init_max_sweeps)
        if key not in seen:
            seen.add(key)
            Sim(p, device=device).close()


def serve_batched(requests, budget_bytes=96 << 30, max_slots=512, tick=50, device=0,
                  clock=time.perf_counter):
    """Runs the requests with continuous batching in real time; fills in
    start, finish and current of every request and returns them."""
    warm_plans(requests, device)
    # the memory pool holds what the admitted requests can use at once (a
    # context takes about three times its admission footprint: row slack,
    # staging rows, mesh arrays) and the kept streams serve as many
    # contexts, so that admissions during the run neither map new pages nor
    # create streams
    need = sum(sorted((footprint_bytes(r.params) for r in requests), reverse=True)[:max_slots])
    reserve(min(budget_bytes, 3 * need), min(max_slots, len(requests)), device)
    pending = collections.deque(sorted(requests, key=lambda r: r.arrival))
    queue = collections.deque()
    active = []   # [request, sim, steps done]
    joining = []
    used = 0
    batch = Batch(device=device)
    t0 = clock()
    try:
        while pending or queue or active or joining:
            stepping = bool(active)
            k = 0
            if stepping:
                k = min(tick, min(r.steps - d for r, _, d in active))
                batch.step(k, sync=False)
            now = clock() - t0
            while pending and pending[0].arrival <= now:
                queue.append(pending.popleft())
            while queue and len(active) + len(joining) < max_slots:
                fp = footprint_bytes(queue[0].params)
                if used + fp > budget_bytes:
                    if not active and not joining:
                        raise RuntimeError(f"request {queue[0].rid} exceeds the HBM budget")
                    break
                r = queue.popleft()
                sim = Sim(r.params, device=device)
                sim.init_plasma(wait=False)  # on its own stream, beside the batch
                r.start = clock() - t0
                joining.append([r, sim, 0])
                used += fp
            failed = []
            if stepping:
                try:
                    batch.sync()
                except CupicError:
                    # every member was waited for; those with a device flag
                    # leave with their error, the others ran their k steps
                    failed = [a for a in active if a[1].flags()]
                    if not failed:
                        raise
                for a in active:
                    a[2] += k
                for r, sim, _ in failed:
                    r.error = f"device flags {sim.flags():#x}"
                    r.finish = clock() - t0
                gone = {id(a) for a in failed}
                active = [a for a in active if id(a) not in gone]
            done = [a for a in active if a[2] >= a[0].steps]
            for r, sim, _ in done:
                r.current = probe_current(sim, r.window)
                r.finish = clock() - t0
            if done or joining or failed:
                for a in joining:
                    a[1].sync()  # its initialisation is complete before the batch uses it
                active = [a for a in active if a[2] < a[0].steps] + joining
                joining = []
                batch.set([a[1] for a in active])
            for r, sim, _ in done + failed:
                sim.close()
                used -= footprint_bytes(r.params)
            if not active and not queue and pending:
                time.sleep(max(0.0, pending[0].arrival - (clock() - t0)))
    finally:
        batch.close()
        for a in active + joining:
            a[1].close()
    return requests


def serve_plain(requests, device=0, clock=time.perf_counter):
    """The plain method: one request at a time in arrival order, each stepped
    alone (cupic_step), in real time."""
    warm_plans(requests, device)
    t0 = clock()
    for r in sorted(requests, key=lambda q: q.arrival):
        wait = r.arrival - (clock() - t0)
        if wait > 0:
            time.sleep(wait)
        r.start = clock() - t0
        sim = Sim(r.params, device=device)
        try:
            sim.init_plasma()
            sim.step(r.steps)
            r.current = probe_current(sim, r.window)
        except CupicError:
            if not sim.flags():
                raise
            r.error = f"device flags {sim.flags():#x}"
        finally:
            sim.close()
        r.finish = clock() - t0
    return requests


def summary(requests):
    """Solves/s and latency percentiles of the requests that succeeded; the
    span runs from the first arrival to the last finish of any request."""
    ok = [r for r in requests if r.error is None]
    lat = np.array([r.latency for r in ok]) if ok else np.zeros(1)
    span = max(r.finish for r in requests) - min(r.arrival for r in requests)
    return {"solves": len(ok), "failed": len(requests) - len(ok), "seconds": span,
            "solves_per_s": len(ok) / span,
            "p50_ms": 1e3 * float(np.percentile(lat, 50)),
            "p99_ms": 1e3 * float(np.percentile(lat, 99))}
