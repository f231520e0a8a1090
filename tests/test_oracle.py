"""Known-answer tests of the CPU oracle (no GPU).

The reference ships no tests or golden vectors, so the oracle's arithmetic
is pinned by analytic answers, published test vectors of the generator, and
(test_ref_pin.py) the reference's own config getters compiled from source.
"""
import math

import numpy as np
import pytest

from cupic_gb300.params import workload_params


@pytest.fixture(scope="module")
def O(oracle_mod):
    return oracle_mod


# ---- generator ---------------------------------------------------------------

def test_philox_published_vectors(O):
    # Salmon et al. (SC'11) Philox4x32-10 known-answer vectors
    assert O.philox([0, 0, 0, 0], [0, 0]) == [0x6627e8d5, 0xe169c58d, 0xbc57ac4c, 0x9b00dbd8]
    assert O.philox([0xffffffff] * 4, [0xffffffff] * 2) == [
        0x408f276d, 0x41c83b0e, 0xa20bc7c6, 0x6d5451fd]
    assert O.philox([0x243f6a88, 0x85a308d3, 0x13198a2e, 0x03707344],
                    [0xa4093822, 0x299f31d0]) == [0xd16cfe09, 0x94fdcceb, 0x5001e420, 0x24126ea1]


def test_log_and_sincos_accuracy(O):
    xs = np.concatenate([np.geomspace(1e-300, 1.0, 2000), np.linspace(0.5, 2.0, 2000)])
    for x in xs:
        ref = math.log(x)
        assert abs(O.olog(x) - ref) <= 4e-16 * max(1.0, abs(ref))
    for u in np.linspace(0.0, 1.0, 4001)[:-1]:
        s, c = O.osincos2pi(u)
        assert abs(s - math.sin(2 * math.pi * u)) < 2e-15
        assert abs(c - math.cos(2 * math.pi * u)) < 2e-15


# ---- helpers -------------------------------------------------------------------

def one_particle_state(O, x, y, species=1, name="tiny", fp64=True, **over):
    p = workload_params(name, **over)
    o = O.Oracle(p, fp64=fp64)
    o.load(species, np.array([[x, y, 0.0, 0.0]]))
    o.load(1 - species, np.zeros((0, 4)))
    return p, o


# ---- deposition (mesh.cu:196-240) ----------------------------------------------

@pytest.mark.parametrize("fp64", [True, False])
def test_single_particle_cic_weights(O, fp64):
    p, o = one_particle_state(O, 2.125, 3.375, fp64=fp64)  # ds=0.5 -> cell (4,6), fx=.25 fy=.75
    rho = o.rho() * p.ds ** 3
    nnx = p.nnx
    w = {(4, 6): 0.75 * 0.25, (5, 6): 0.25 * 0.25, (4, 7): 0.75 * 0.75, (5, 7): 0.25 * 0.75}
    for (i, j), v in w.items():
        assert rho[j, i] == pytest.approx(v, abs=1e-12)
    rho2 = rho.copy()
    for (i, j) in w:
        rho2[j, i] = 0
    assert np.all(rho2 == 0)
    if not fp64:
        acc = o.rho_fixed()
        assert acc.sum() == 2 ** 32  # exactly one unit of charge
        assert acc[6, 4] == int(0.75 * 0.25 * 2 ** 32)


def test_seam_fold_x0_and_xLx(O):
    p, o = one_particle_state(O, 7.875, 5.25, fp64=True)  # ic = ncx-1, fx = .75
    rho = o.rho() * p.ds ** 3
    nx = p.ncx
    # node ncx (x=Lx) is the same node as 0: both carry the folded value
    assert rho[10, 0] == rho[10, nx] == pytest.approx(0.75 * 0.5)
    assert rho[10, nx - 1] == pytest.approx(0.25 * 0.5)


def test_dirichlet_rows_use_half_volume(O):
    p, o = one_particle_state(O, 1.0, 0.0, fp64=True)
    rho = o.rho()
    assert rho[0, 2] == pytest.approx(1.0 / (0.5 * p.ds ** 3))


def test_charge_is_conserved_exactly(O):
    p = workload_params("tiny")
    o = O.Oracle(p, fp64=False)
    o.init_plasma()
    for _ in range(3):
        o.step(1)
        ne, ni = o.counts()
        acc = o.rho_fixed()
        assert acc.sum() == (ni - ne) * 2 ** 32


# ---- Jacobi (mesh.cu:327-369) and field (mesh.cu:413-468) ------------------------

@pytest.mark.parametrize("fp64", [True, False])
def test_linear_potential_is_a_fixed_point(O, fp64):
    """init.cu:235-241's linear profile solves the charge-free problem."""
    p = workload_params("tiny")
    o = O.Oracle(p, fp64=fp64)
    for s in (0, 1):
        o.load(s, np.zeros((0, 4)))
    j = np.arange(p.nny)[:, None]
    phi0 = (1.0 - j / p.ncy) * p.phi_p * np.ones((1, p.nnx))
    o.set_phi(phi0)
    sweeps, res = o.solve(1e-12, 1, 50, 1)
    assert sweeps == 1 or res < 1e-5
    np.testing.assert_allclose(o.phi(), phi0, atol=2e-6)
    o.field()
    ex, ey = o.efield()
    np.testing.assert_allclose(ey, p.phi_p / (p.ncy * p.ds), rtol=2e-5)
    assert np.all(ex[[0, -1]] == 0.0)
    np.testing.assert_allclose(ex, 0.0, atol=2e-5)


def test_jacobi_converges_to_discrete_solution(O):
    """A point charge: the converged phi satisfies the 5-point equations."""
    p = workload_params("tiny", max_sweeps=20000)
    p, o = one_particle_state(O, 4.1, 8.2, max_sweeps=20000)
    o.set_phi(np.zeros((p.nny, p.nnx)))
    sweeps, res = o.solve(1e-13, 1, 20000, 1)
    phi = o.phi()
    rho = o.rho(1)
    ds = p.ds
    lap = (phi[1:-1, :-2] + phi[1:-1, 2:] + phi[:-2, 1:-1] + phi[2:, 1:-1] - 4 * phi[1:-1, 1:-1])
    lap = lap / ds ** 2
    np.testing.assert_allclose(lap, -rho[1:-1, 1:-1] / p.eps0, atol=1e-8)


def test_jacobi_stop_rule(O):
    p = workload_params("tiny")
    o = O.Oracle(p, fp64=True)
    o.init_plasma()
    # min sweeps forces at least that many; max caps it
    s, _ = o.solve(1.0, 37, 100, 1)
    assert s == 37
    s, r = o.solve(0.0, 1, 23, 1)
    assert s == 23
    # check_every: stops only on a checked sweep
    s, _ = o.solve(1.0, 1, 100, 8)
    assert s == 8


# ---- push (particles.cu:145-225, init.cu:825-826) -------------------------------

def test_leapfrog_in_uniform_field_closed_form(O):
    """With the linear potential, E = (0, phi_p/Ly) everywhere: an ion at
    rest moves y(n) = y0 + a dt^2 n(n+1)/2 after the velocity half-step."""
    p = workload_params("tiny", phi_p=-2.0)
    o = O.Oracle(p, fp64=True)
    y0 = 9.1
    o.load(1, np.array([[3.3, y0, 0.0, 0.0]]))
    o.load(0, np.zeros((0, 4)))
    j = np.arange(p.nny)[:, None]
    o.set_phi((1.0 - j / p.ncy) * p.phi_p * np.ones((1, p.nnx)))
    o.field()
    a = (p.qi / p.mi) * p.phi_p / (p.ncy * p.ds)
    o.push(1)  # v(-dt/2) = -a dt/2
    vy = o.particles(1)[0, 3]
    assert vy == pytest.approx(-0.5 * a * p.dt, rel=1e-12)
    for n in range(1, 6):
        o.push(0)
        y = o.particles(1)[0, 1]
        # y(t) = y0 + a t^2 / 2 at t = n dt, exactly the uniform-acceleration path
        assert y == pytest.approx(y0 + 0.5 * a * (n * p.dt) ** 2, rel=1e-12)
        v_expect = a * p.dt * (n - 0.5)
        assert o.particles(1)[0, 3] == pytest.approx(v_expect, rel=1e-9)


def test_periodic_wrap_maps_into_0_Lx(O):
    p = workload_params("tiny")
    o = O.Oracle(p, fp64=False)
    lx = p.ds * p.ncx
    o.load(1, np.array([[0.01, 5.0, -1.0, 0.0], [lx - 0.01, 5.0, 1.0, 0.0]]))
    o.load(0, np.zeros((0, 4)))
    o.field()
    o.push(0)
    x = o.particles(1)[:, 0]
    assert np.all(x >= 0) and np.all(x < lx)
    assert x[0] == pytest.approx(lx - 0.04, abs=1e-5)
    assert x[1] == pytest.approx(0.04, abs=1e-5)


def test_binning_order_is_stable(O):
    """row d = stayers + up-movers from d-1 + down-movers from d+1, each in
    previous order (the build's deterministic replacement of cc.cu:303-772)."""
    p = workload_params("tiny", dt=1.0)
    o = O.Oracle(p, fp64=True)
    ds = p.ds
    parts = np.array([
        [1.0, 2.2 * ds, 0.0, 0.0],   # row 2 stays
        [2.0, 1.9 * ds, 0.0, 0.2],   # row 1 -> 2 (up)
        [3.0, 2.5 * ds, 0.0, 0.0],   # row 2 stays
        [4.0, 3.1 * ds, 0.0, -0.1],  # row 3 -> 2 (down)
        [5.0, 2.9 * ds, 0.0, 0.0],   # row 2 stays
        [6.0, 1.5 * ds, 0.0, 0.3],   # row 1 -> 2 (up)
    ])
    o.load(1, parts)
    o.load(0, np.zeros((0, 4)))
    o.push(0)
    got = o.particles(1)
    assert list(got[:, 0]) == [1.0, 3.0, 5.0, 2.0, 6.0, 4.0]
    assert list(o.row_counts(1)[:4]) == [0, 0, 6, 0]


def test_absorption_and_removal_counts(O):
    p = workload_params("tiny", dt=1.0)
    o = O.Oracle(p, fp64=True)
    ly = p.ds * p.ncy
    o.load(0, np.array([[1.0, 0.1, 0.0, -0.5], [2.0, 0.2, 0.0, -0.1], [1.0, ly - 0.1, 0.0, 0.5]]))
    o.load(1, np.array([[1.0, 0.05, 0.0, -0.2]]))
    o.push(0)
    st = o.stats()
    assert st["absorbed"] == [1, 1] and st["removed"] == [1, 0]
    assert o.counts() == (1, 0)


# ---- injection (cc.cu:179-256) --------------------------------------------------

def test_injection_counts_follow_tin_dtin(O):
    p = workload_params("small")
    o = O.Oracle(p, fp64=False)
    lx = p.ds * p.ncx
    dtin_e = math.sqrt(2 * math.pi) / (p.n * lx * p.ds)
    dtin_i = math.sqrt(2 * math.pi * p.mi / p.kti) / (p.n * lx * p.ds)
    for s in (0, 1):
        o.load(s, np.zeros((0, 4)))
    t = p.dt
    tin = [t + dtin_e, t + dtin_i]
    tot = [0, 0]
    for k in range(20):
        o.inject(t)
        st = o.stats()
        fpt = t + p.dt
        for s, dtin in enumerate((dtin_e, dtin_i)):
            n = 1 + int((fpt - tin[s]) / dtin) if tin[s] < fpt else 0
            for _ in range(n):
                tin[s] += dtin
            assert st["injected"][s] == n
            tot[s] += n
        t += p.dt
    assert o.counts() == tuple(tot)
    parts = o.particles(0)
    assert np.all(parts[:, 3] < 0)  # injected inward
    assert np.all(parts[:, 1] <= p.ds * p.ncy)


def test_injected_velocity_distribution(O):
    """vx ~ N(0, sqrt(kT/m)), -vy ~ Rayleigh(sqrt(kT/m)) (cc.cu:218-219)."""
    p = workload_params("small", dt=2.0)
    o = O.Oracle(p, fp64=True)
    for s in (0, 1):
        o.load(s, np.zeros((0, 4)))
    t = p.dt
    for _ in range(40):
        o.inject(t)
        t += p.dt
    v = o.particles(0)
    assert v.shape[0] > 3000
    assert np.mean(v[:, 2]) == pytest.approx(0.0, abs=0.06)
    assert np.std(v[:, 2]) == pytest.approx(1.0, rel=0.05)
    assert np.mean(-v[:, 3]) == pytest.approx(math.sqrt(math.pi / 2), rel=0.05)


# ---- whole cycle ------------------------------------------------------------------

def test_initial_plasma_shape(O):
    p = workload_params("small")
    o = O.Oracle(p, fp64=False)
    o.init_plasma()
    assert o.counts() == (p.ppr * p.ncy, p.ppr * p.ncy)
    rc = o.row_counts(0)
    assert np.all(rc == p.ppr)
    e = o.particles(0)
    assert np.std(e[:, 2]) == pytest.approx(1.0, rel=0.02)
    i = o.particles(1)
    assert np.std(i[:, 2]) == pytest.approx(math.sqrt(p.kti / p.mi), rel=0.02)


def test_fp32_tracks_fp64(O):
    p = workload_params("tiny")
    a = O.Oracle(p, fp64=False)
    b = O.Oracle(p, fp64=True)
    a.init_plasma()
    b.init_plasma()
    a.step(5)
    b.step(5)
    np.testing.assert_allclose(a.phi(), b.phi(), atol=2e-3)
    ca, cb = a.counts(), b.counts()
    assert abs(ca[0] - cb[0]) <= 3 and abs(ca[1] - cb[1]) <= 3


def test_thread_count_does_not_change_fp32_results(O):
    p = workload_params("tiny")
    outs = []
    for n in (1, 4):
        O.set_threads(n)
        o = O.Oracle(p, fp64=False)
        o.init_plasma()
        o.step(3)
        outs.append((o.particles(0), o.phi(), o.rho_fixed()))
    import os
    O.set_threads(os.cpu_count())
    for x, y in zip(outs[0], outs[1]):
        np.testing.assert_array_equal(x, y)
