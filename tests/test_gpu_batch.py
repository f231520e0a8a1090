"""The batched form (cupic_batch_*) on the GPU.

Contexts of uneven sizes stepped together in one launch per kernel must
give, bit for bit, what each gets when stepped alone: particles (order
included), phi, E and every per-step counter.  One member is large enough
that its solve takes a group of many CTAs inside the batched launch.
"""
import numpy as np
import pytest

import cupic_gb300 as cg
from oracle.oracle import Oracle
from parity import check_state, check_stats

pytestmark = pytest.mark.gpu

FIXED = dict(tol=0.0, check_every=100, min_sweeps=100, max_sweeps=100, init_tol=0.0,
             init_min_sweeps=100, init_max_sweeps=100)
MEMBERS = [
    ("tiny", {}),
    ("tiny", dict(seed=11, phi_p=2.0)),
    ("small", dict(ncx=32, ncy=128, n=40.0, eps0=40.0, seed=3, **FIXED)),
    ("small", dict(ncx=64, ncy=256, n=80.0, eps0=80.0, seed=4, mi=1836.0, kti=0.1, **FIXED)),
    ("small", dict(ncx=256, ncy=1024, n=40.0, eps0=40.0, seed=5, phi_p=-10.0, **FIXED)),
]


def make_all(**extra):
    out = []
    for name, over in MEMBERS:
        s = cg.Sim(cg.workload_params(name, **over, **extra))
        s.init_plasma()
        out.append(s)
    return out


def compare(a, b, what):
    for sp in (0, 1):
        np.testing.assert_array_equal(a.particles(sp), b.particles(sp), err_msg=f"{what} species {sp}")
    np.testing.assert_array_equal(a.phi(), b.phi(), err_msg=f"{what} phi")
    for x, y in zip(a.efield(), b.efield()):
        np.testing.assert_array_equal(x, y, err_msg=f"{what} E")
    np.testing.assert_array_equal(a.rho_fixed(0), b.rho_fixed(0), err_msg=f"{what} rho")


def test_batch_equals_members_alone(gpu_lib):
    alone, batched = make_all(), make_all()
    steps = 6
    try:
        for s in alone:
            s.step(steps)
        with cg.Batch(batched) as b:
            b.step(2)
            b.step(steps - 2)
        for k, (a, m) in enumerate(zip(alone, batched)):
            compare(a, m, f"member {k}")
            assert a.stats(steps) == m.stats(steps), f"member {k} stats"
            assert m.flags() == 0
    finally:
        for s in alone + batched:
            s.close()


def test_membership_changes_between_steps(gpu_lib):
    """Members leave and join between batched steps (continuous batching);
    each one's state still equals its solo run."""
    batched = make_all()
    try:
        with cg.Batch(batched[:2]) as b:
            b.step(1)
            b.set(batched[:4])       # two join
            b.step(1)
            b.set(batched[1:])       # one leaves, the large one joins
            b.step(1)
            b.set([batched[4], batched[2]])
            b.step(1)
            b.set([batched[3], batched[4]])
            b.step(1)
            b.set([batched[4]])
            b.step(2)
        # steps taken: member0 2, member1 3, member2 3, member3 3, member4 5
        for k, n in enumerate((2, 3, 3, 3, 5)):
            ref = cg.Sim(batched[k].p)
            ref.init_plasma()
            ref.step(n)
            compare(ref, batched[k], f"member {k}")
            ref.close()
    finally:
        for s in batched:
            s.close()


def test_members_whose_rows_fill_up(gpu_lib):
    """Members without row slack halt alone when a row runs out of room;
    the batch's sync grows their rows and completes their steps, the next
    batched step runs on the new buffers, and every member still equals its
    solo run."""
    alone, batched = make_all(row_slack=0.0), make_all(row_slack=0.0)
    caps = [(int(np.ceil(s.p.ppr)) + 7) // 8 * 8 + 64 for s in batched]
    steps, tick = 24, 4
    most = [0] * len(batched)
    try:
        for s in alone:
            s.step(steps)
        with cg.Batch(batched) as b:
            for _ in range(steps // tick):
                b.step(tick)
                for k, m in enumerate(batched):
                    most[k] = max(most[k], int(m.row_counts(0).max()), int(m.row_counts(1).max()))
        for k, (a, m) in enumerate(zip(alone, batched)):
            compare(a, m, f"member {k}")
            assert a.stats(steps) == m.stats(steps), f"member {k} stats"
            assert m.flags() == 0
        # the 64x256 member (pushed from the work list) and the 256x1024 one
        # (pushed by the single-context kernel) outgrow their rows
        assert most[3] > caps[3] and most[4] > caps[4], (most, caps)
    finally:
        for s in alone + batched:
            s.close()


def test_member_reloaded_between_steps(gpu_lib):
    """A member whose electrons are reloaded between batched steps, with rows
    fuller than their capacity (so they are laid out anew): the next batched
    step deposits its charge, takes its new buffers, and it still equals its
    solo run."""
    alone, batched = make_all(), make_all()
    try:
        for s in alone:
            s.step(2)
        with cg.Batch(batched) as b:
            b.step(2)
            for s in (alone[2], batched[2]):
                e = s.particles(0)
                rows = np.floor(e[:, 1] / s.p.ds).astype(int)
                extra = e[rows == rows.max()]
                extra = np.concatenate([extra] * 3)  # the top row three times over
                s.load(0, np.concatenate([e, extra]))
            for s in alone:
                s.step(3)
            b.step(3)
        for k, (a, m) in enumerate(zip(alone, batched)):
            compare(a, m, f"member {k}")
            assert a.stats(3) == m.stats(3), f"member {k} stats"
            assert m.flags() == 0
    finally:
        for s in alone + batched:
            s.close()


def test_batched_large_member_matches_oracle(gpu_lib):
    """The 256x1024 member, solved by a group of CTAs inside the batched
    launch and pushed by the batched kernels, equals the FP32 oracle bit for
    bit (particles, rows, charge, potential, field, counters), not only its
    own solo run."""
    members = make_all()
    big = members[4]
    assert (big.p.ncx, big.p.ncy) == (256, 1024)
    ora = Oracle(big.p, fp64=False)
    ora.init_plasma()
    try:
        with cg.Batch(members) as b:
            for _ in range(3):
                b.step(1)
                b.sync()
                ora.step(1)
                check_stats(big.stats(1)[0], ora.stats())
        check_state(big, ora)
    finally:
        ora.close()
        for s in members:
            s.close()


def test_tuned_batch_equals_members_alone(gpu_lib, monkeypatch):
    """A set of 18 members is large enough for the batched-solve autotuner:
    it times its candidate layouts on the members' own meshes, restores
    their potential, field and solver status, and the members still get
    their solo results bit for bit.  A second batch of the same mix takes
    the cached pick; CUPIC_BATCH_TUNE=0 takes the default layout."""
    from cupic_gb300.params import bias_instances
    monkeypatch.delenv("CUPIC_BATCH_TUNE", raising=False)
    ps = bias_instances(18, seed=5, sizes=(32, 64))

    def make():
        out = []
        for p in ps:
            s = cg.Sim(p)
            s.init_plasma()
            out.append(s)
        return out

    alone, batched = make(), make()
    try:
        phi0 = [s.phi() for s in batched]
        with cg.Batch(batched) as b:
            depth, mult, ctas = b.plan()
            assert depth in (1, 2, 4, 8) and mult in (1, 2) and ctas > 0
            # the trials left every member's potential as it was
            for k, s in enumerate(batched):
                np.testing.assert_array_equal(s.phi(), phi0[k], err_msg=f"member {k} phi after tuning")
                assert s.flags() == 0
            b.step(4)
        for s in alone:
            s.step(4)
        for k, (a, m) in enumerate(zip(alone, batched)):
            compare(a, m, f"member {k}")
            assert a.stats(4) == m.stats(4), f"member {k} stats"
        with cg.Batch(batched) as b2:
            assert b2.plan()[:2] == (depth, mult)
        monkeypatch.setenv("CUPIC_BATCH_TUNE", "0")
        with cg.Batch(batched) as b3:
            assert b3.plan()[:2] == (4, 1)
    finally:
        for s in alone + batched:
            s.close()
