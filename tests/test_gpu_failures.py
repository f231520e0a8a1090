"""Failure detection on the GPU, without a GPU fault.

Each case makes the failure on purpose from the host side or with a wait
that nothing satisfies, and checks that the device raises its sticky flag,
that the call returns the matching status, and that the context keeps
working after cupic_clear_flags.  No case faults, traps or hangs the GPU:
every index the kernels use is clamped, and every wait is bounded.
"""
import math

import numpy as np
import pytest

import cupic_gb300 as cg

pytestmark = pytest.mark.gpu

CFL, CAPACITY, STAGE, NONFINITE, TIMEOUT = 1, 2, 4, 8, 16


def plasma(p, rng, rows, per_row, vy=0.0):
    """per_row particles in each of `rows`, at rest in x, moving vy in y."""
    out = []
    for j in rows:
        x = rng.uniform(0, p.ncx * p.ds, per_row)
        y = (j + rng.uniform(0.2, 0.3, per_row)) * p.ds
        out.append(np.stack([x, y, np.zeros(per_row), np.full(per_row, vy)], axis=1))
    return np.concatenate(out)


def stepped(sim):
    with pytest.raises(cg.CupicError) as e:
        sim.step(1)
    return e.value.status


def recovers(sim, p, rng):
    """After clear_flags, a clean plasma steps without flags."""
    sim.clear_flags()
    sim.load(0, plasma(p, rng, range(8, 12), 20))
    sim.step(2)
    assert sim.flags() == 0


@pytest.fixture
def tiny(gpu_lib):
    p = cg.workload_params("tiny", row_slack=0.0)
    sim = cg.Sim(p)
    sim.init_plasma()
    yield p, sim
    sim.close()


def test_bounded_wait_gives_up_and_reports_timeout(tiny):
    p, sim = tiny
    rc = sim.L.cupic_test_bounded_wait(sim.h)
    assert rc == 9  # CUPIC_ERR_TIMEOUT
    assert sim.flags() & TIMEOUT
    recovers(sim, p, np.random.default_rng(0))


def test_particle_crossing_rows_in_one_step_is_flagged(tiny):
    p, sim = tiny
    rng = np.random.default_rng(1)
    e = plasma(p, rng, range(8, 12), 20)
    e[0, 3] = 30.0  # 1.5 length units per step: three cell rows
    sim.load(0, e)
    assert stepped(sim) == 6  # CUPIC_ERR_CFL
    assert sim.flags() & CFL
    recovers(sim, p, rng)


def test_nonfinite_particle_is_removed_and_flagged(tiny):
    p, sim = tiny
    rng = np.random.default_rng(2)
    e = plasma(p, rng, range(8, 12), 20)
    e[5, 2] = math.nan
    sim.load(0, e)
    n0 = sim.counts()[0]
    assert stepped(sim) == 7  # CUPIC_ERR_NONFINITE
    assert sim.flags() & NONFINITE
    assert not np.isnan(sim.particles(0)).any()
    assert sim.stats(1)[0]["removed"][0] >= 1 and sim.counts()[0] < n0 + sim.stats(1)[0]["injected"][0]
    recovers(sim, p, rng)


def test_full_row_grows_instead_of_overflowing(tiny):
    """A row that cannot take its arrivals is grown by the room check and the
    host before any particle is written: no particle is lost, no flag."""
    p, sim = tiny
    rng = np.random.default_rng(3)
    # row 10 full at its capacity; row 9 sends all its particles up into it
    cap = (int(math.ceil(p.ppr)) + 7) // 8 * 8 + 64
    e = np.concatenate([plasma(p, rng, [10], cap - 8), plasma(p, rng, [9], 40, vy=10.0)])
    sim.load(0, e)
    sim.step(1)
    assert sim.flags() == 0
    rows = sim.row_counts(0)
    assert rows[10] == cap - 8 + 40 and rows[9] == 0


def test_staging_overflow_is_flagged(tiny):
    p, sim = tiny
    rng = np.random.default_rng(4)
    # 200 particles of row 9 move up in one step; loading them gives row 9
    # 264 places and the staging rows 136, so 64 movers find no staging slot
    sim.load(0, plasma(p, rng, [9], 200, vy=10.0))
    assert stepped(sim) == 5  # CUPIC_ERR_CAPACITY
    assert sim.flags() & STAGE
    recovers(sim, p, rng)
