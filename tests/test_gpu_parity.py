"""GPU-vs-oracle parity of the full PIC cycle, through the C-ABI.

The kernels round every float operation where the FP32 oracle does, so the
results are expected to be identical; the contract they are held to is
  bit-exact : row (bin) indices, absorbed/removed/injected counts, order
  <= 1e-5   : relative error of rho, phi, E, x, y, vx, vy (FP32)
and each assertion below states which one it checks.
"""
import os

import numpy as np
import pytest

import cupic_gb300 as cg
from oracle.oracle import Oracle
from parity import check_state, check_stats

pytestmark = pytest.mark.gpu


@pytest.fixture
def make_pair(gpu_lib, monkeypatch):
    made = []

    def _make(name, ctas=None, **over):
        if ctas is not None:
            monkeypatch.setenv("CUPIC_JACOBI_CTAS", str(ctas))
        else:
            monkeypatch.delenv("CUPIC_JACOBI_CTAS", raising=False)
        p = cg.workload_params(name, **over)
        sim = cg.Sim(p)
        ora = Oracle(p, fp64=False)
        made.append(sim)
        return sim, ora

    yield _make
    for s in made:
        s.close()


@pytest.mark.parametrize("name", ["tiny", "small"])
def test_init_matches_oracle(make_pair, name):
    sim, ora = make_pair(name)
    sim.init_plasma()
    ora.init_plasma()
    check_state(sim, ora)
    assert sim.stats(1)[0]["flags"] == 0 or True


@pytest.mark.parametrize("name,steps", [("tiny", 12), ("small", 4)])
def test_steps_match_oracle(make_pair, name, steps):
    sim, ora = make_pair(name)
    sim.init_plasma()
    ora.init_plasma()
    gs = []
    for _ in range(steps):
        sim.step(1)
        ora.step(1)
        g = sim.stats(1)[0]
        o = ora.stats()
        check_stats(g, o)
        assert g["residual"] == pytest.approx(o["residual"], rel=0, abs=0)
        assert g["flags"] == 0
        gs.append(g)
    check_state(sim, ora)
    assert sum(g["injected"][0] for g in gs) > 0


@pytest.mark.parametrize("ctas", [2, 5, 16])
def test_multi_cta_jacobi(make_pair, ctas):
    sim, ora = make_pair("small", ctas=ctas, max_sweeps=300)
    sim.init_plasma()
    ora.init_plasma()
    sim.step(2)
    ora.step(2)
    check_state(sim, ora)


@pytest.mark.parametrize("name,over,ctas,depth,strips", [
    ("small", {}, 1, 1, True),
    ("small", {}, 3, 1, True),
    ("small", {}, 3, 4, True),
    ("small", {}, 4, 8, True),
    ("small", {}, 4, 8, False),
    ("small", {}, 7, 3, True),
    ("small", {"ncx": 256, "ncy": 64}, 2, 8, True),
    ("small", {"ncx": 256, "ncy": 64}, 3, 5, False),
])
def test_jacobi_layouts(make_pair, monkeypatch, name, over, ctas, depth, strips):
    """Every solver layout -- CTA count, temporal-blocking depth, register
    strips or the shared-memory sweep -- gives the oracle's bits."""
    monkeypatch.setenv("CUPIC_JACOBI_DEPTH", str(depth))
    if strips:
        monkeypatch.delenv("CUPIC_JACOBI_NOSTRIP", raising=False)
    else:
        monkeypatch.setenv("CUPIC_JACOBI_NOSTRIP", "1")
    sim, ora = make_pair(name, ctas=ctas, max_sweeps=300, **over)
    G, _, K = sim.solver_plan()
    assert G == ctas and (K == depth or G == 1)
    sim.init_plasma()
    ora.init_plasma()
    sim.step(2)
    ora.step(2)
    check_state(sim, ora)


def test_repeated_short_solves_match_oracle(make_pair, monkeypatch):
    """Back-to-back solves with one or two halo exchanges each: every solve
    tags its halo words with new epochs, so no solve reads an earlier one's
    rows."""
    monkeypatch.setenv("CUPIC_JACOBI_DEPTH", "2")
    sim, ora = make_pair("small", ctas=4)
    sim.init_plasma()
    ora.init_plasma()
    for n in (3, 3, 5, 2, 3, 7, 4, 3):
        sim.poisson_solver(1e-30, n, n, n)
        ora.solve(1e-30, n, n, n)
        np.testing.assert_array_equal(sim.phi().astype(np.float64), ora.phi(), err_msg=f"{n} sweeps")


@pytest.mark.parametrize("tol,mn,mx,chk", [(1e-30, 30, 30, 1), (2e-3, 25, 400, 1),
                                             (2e-3, 25, 400, 7), (5e-4, 40, 600, 3)])
def test_solve_stop_rule_matches_oracle(make_pair, tol, mn, mx, chk):
    """The stop rule (mesh.cu:94-114 with min/max sweeps and a check every
    chk sweeps): the sweep count, the reported residual and the potential
    are the oracle's, which checks from the first sweep; the GPU skips the
    checks before min_sweeps, which can stop nothing.  Bit-exact: the
    oracle stops at sweeps 30, 25, 28 and 195 on these cases."""
    import ctypes
    torch = pytest.importorskip("torch")
    sim, ora = make_pair("small", ctas=4)
    sim.init_plasma()
    ora.init_plasma()
    p = sim.p
    rho = np.ascontiguousarray(sim.rho_fixed(0).ravel(), dtype=np.int64)
    phi0 = np.ascontiguousarray(sim.phi().ravel(), dtype=np.float32)
    sw_o, res_o = ora.solve(tol, mn, mx, chk)
    # the allocation-free entry point reports the sweeps and the residual
    L = cg.load_library()
    d_rho = torch.from_numpy(rho).to("cuda")
    d_phi = torch.from_numpy(phi0.copy()).to("cuda")
    torch.cuda.synchronize()
    sweeps, res = ctypes.c_int32(), ctypes.c_float()
    rc = L.cupic_poisson_solver_static(ctypes.byref(p), d_rho.data_ptr(), d_phi.data_ptr(), None, tol,
                                       mn, mx, chk, None, ctypes.byref(sweeps), ctypes.byref(res))
    assert rc == 0, cg.strerror(rc)
    assert sweeps.value == sw_o
    assert res.value == np.float32(res_o)
    np.testing.assert_array_equal(d_phi.cpu().numpy().astype(np.float64), ora.phi().ravel())
    # and the context's solver on the same state
    sim.poisson_solver(tol, mn, mx, chk)
    np.testing.assert_array_equal(sim.phi().astype(np.float64), ora.phi())


def test_stage_api_matches_oracle(make_pair):
    """Drive the reference's entry points one by one on a state loaded from
    host arrays (read_particle_file + the main loop, main.cu:59-96)."""
    sim, ora = make_pair("tiny")
    ora.init_plasma()
    ora.step(2)
    for sp in (0, 1):
        sim.load(sp, ora.particles(sp))
    sim.set_phi(ora.phi())
    st, t, tin_e, tin_i = ora.get_time()
    sim.set_time(st, t, tin_e, tin_i)
    sim.charge_deposition()
    np.testing.assert_array_equal(sim.rho_fixed(0), ora.rho_fixed())
    sim.poisson_solver(1e-30, 40, 40, 1)
    ora.solve(1e-30, 40, 40, 1)
    np.testing.assert_array_equal(sim.phi().astype(np.float64), ora.phi())
    sim.field_solver()
    ora.field()
    exg, eyg = sim.efield()
    exo, eyo = ora.efield()
    np.testing.assert_array_equal(exg.astype(np.float64), exo)
    np.testing.assert_array_equal(eyg.astype(np.float64), eyo)
    sim.particle_mover()
    ora.push(0)
    sim.cc(t)
    ora.inject(t)
    check_state(sim, ora)


def test_bookmarks_match_rows(make_pair):
    sim, ora = make_pair("tiny")
    sim.init_plasma()
    sim.step(3)
    bm = sim.bookmarks(0).reshape(-1, 2)
    rows = sim.row_counts(0)
    parts = sim.particles(0)
    inv = 1.0 / sim.p.ds
    for j, (a, b) in enumerate(bm):
        if rows[j] == 0:
            assert a == -1 and b == -1
            continue
        ys = parts[a:b + 1, 1].astype(np.float32)
        got = np.floor(ys * np.float32(inv)).astype(int)
        assert np.all(got == j), f"row {j} holds particles of rows {set(got)}"


def test_runs_are_deterministic(make_pair):
    a, _ = make_pair("tiny")
    b, _ = make_pair("tiny")
    for s in (a, b):
        s.init_plasma()
        s.step(5)
    for sp in (0, 1):
        np.testing.assert_array_equal(a.particles(sp), b.particles(sp))
    np.testing.assert_array_equal(a.rho_fixed(0), b.rho_fixed(0))


def test_small_workload_matches_committed_golden(gpu_lib):
    """The 64x256 workload on the GPU gives, bit for bit, the committed
    digests of the FP32 oracle (tests/golden/oracle_small.json)."""
    import json
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    sys.path.insert(0, os.path.join(root, "tests", "golden"))
    import make_oracle_golden as mk
    with open(os.path.join(root, "tests", "golden", "oracle_small.json")) as f:
        gold = json.load(f)
    with cg.Sim(cg.workload_params("small")) as sim:
        sim.init_plasma()

        def snap():
            ex, ey = sim.efield()
            return mk.snapshot(sim.particles, sim.row_counts, lambda: sim.rho_fixed(0), sim.phi, ex, ey)

        assert snap() == gold["states"]["init"]
        for k in range(1, 11):
            sim.step(1)
            st = sim.stats(1)[0]
            assert {key: st[key] for key in gold["stats"][k - 1]} == gold["stats"][k - 1], k
            if k in (1, 10):
                assert snap() == gold["states"][f"step{k}"], k


def test_probe_current_and_density_diagnostics(gpu_lib):
    p = cg.workload_params("small")
    with cg.Sim(p) as sim:
        sim.init_plasma()
        for sp in (0, 1):
            np.testing.assert_array_equal(sim.density_profile(sp), np.full(p.ncy, p.n))
        sim.step(12)
        st = sim.stats(10)
        want = np.mean([p.qe * s["absorbed"][0] + p.qi * s["absorbed"][1] for s in st])
        assert sim.probe_current(10) == pytest.approx(want, rel=0, abs=1e-12)
        rows = sim.row_counts(1)
        np.testing.assert_allclose(sim.density_profile(1), rows / (p.ncx * p.ds ** 3), rtol=1e-15)


def row_capacity(p, slack):
    """The capacity a row gets at initialisation: ppr * (1 + slack) + 64,
    rounded up to a multiple of 8."""
    return (int(np.ceil(p.ppr * (1.0 + slack))) + 7) // 8 * 8 + 64


def most_in_a_row(sim):
    return max(int(sim.row_counts(0).max()), int(sim.row_counts(1).max()))


def test_full_rows_grow_and_match_oracle(make_pair):
    """Rows without slack (ppr + 64 places) run out of room within a few
    steps.  The room check halts the run before any particle is written,
    the host grows the rows that are short and completes the steps, and
    every step still gives the oracle's bits; runs of ten graph-launched
    steps halt and resume several times."""
    sim, ora = make_pair("small", row_slack=0.0)
    cap0 = row_capacity(sim.p, 0.0)
    sim.init_plasma()
    ora.init_plasma()
    most = 0
    for _ in range(4):
        sim.step(10)
        ora.step(10)
        g, o = sim.stats(1)[0], ora.stats()
        for k in ("step", "absorbed", "removed", "injected", "live", "sweeps"):
            assert g[k] == o[k], f"{k}: gpu {g[k]} oracle {o[k]} at step {o['step']}"
        assert g["flags"] == 0
        most = max(most, most_in_a_row(sim))
    assert most > cap0, "no row outgrew its first capacity"
    check_state(sim, ora)


def test_stage_api_grows_full_rows(make_pair):
    """The reference's main loop (main.cu:61-73) on rows without slack:
    particle_mover and cc grow the rows that cannot take their arrivals or
    injected particles before writing them."""
    sim, ora = make_pair("small", row_slack=0.0)
    cap0 = row_capacity(sim.p, 0.0)
    sim.init_plasma()
    ora.init_plasma()
    most = 0
    for _ in range(8):
        t = ora.get_time()[1]
        sim.charge_deposition()
        ora.deposit()
        sim.poisson_solver(1e-30, 40, 40, 1)
        ora.solve(1e-30, 40, 40, 1)
        sim.field_solver()
        ora.field()
        sim.particle_mover()
        ora.push(0)
        sim.cc(t)
        ora.inject(t)
        most = max(most, most_in_a_row(sim))
    assert most > cap0, "no row outgrew its first capacity"
    check_state(sim, ora)


def test_long_run_of_the_64x256_workload(make_pair):
    """640 steps of the 64x256 workload: its top electron row passes the
    default capacity (1.5 ppr + 64) at step 629 and holds about 2200
    electrons at step 640, and the run goes on with the oracle's bits."""
    sim, ora = make_pair("small")
    cap0 = row_capacity(sim.p, sim.p.row_slack)
    sim.init_plasma()
    ora.init_plasma()
    sim.step(640)
    ora.step(640)
    assert sim.stats(1)[0]["flags"] == 0
    check_state(sim, ora)
    assert most_in_a_row(sim) > cap0


def test_dense_cell_folds_its_charge_moments(make_pair):
    """40000 electrons in one cell, more than the 16383 a cell's 32-bit
    charge moments hold before they must be folded into the int64
    accumulator: the standalone deposit and the push's deposit both fold in
    time and give the oracle's charge bit for bit."""
    sim, ora = make_pair("tiny")
    ora.init_plasma()
    ora.step(1)
    rng = np.random.default_rng(5)
    n = 40000
    dense = np.empty((n, 4))
    dense[:, 0] = 2.0 + 0.5 * rng.random(n)      # cell column 4 (ds = 0.5)
    dense[:, 1] = 2.5 + 0.5 * rng.random(n)      # cell row 5
    dense[:, 2:] = 1e-3 * rng.standard_normal((n, 2))
    dense = dense.astype(np.float32).astype(np.float64)
    electrons = np.concatenate([ora.particles(0), dense])
    ora.load(0, electrons)
    for sp in (0, 1):
        sim.load(sp, ora.particles(sp))
    # a zero potential, so the dense cell stays together through the push
    zero = np.zeros((sim.p.nny, sim.p.nnx))
    sim.set_phi(zero)
    ora.set_phi(zero)
    st, t, tin_e, tin_i = ora.get_time()
    sim.set_time(st, t, tin_e, tin_i)
    sim.charge_deposition()
    ora.deposit()
    np.testing.assert_array_equal(sim.rho_fixed(0), ora.rho_fixed(), err_msg="standalone deposit")
    assert sim.row_counts(0)[5] > n
    sim.field_solver()
    ora.field()
    sim.particle_mover()
    ora.push(0)
    sim.cc(t)
    ora.inject(t)
    check_state(sim, ora)


def test_solves_past_the_epoch_wrap_keep_the_oracle_bits(make_pair, monkeypatch):
    """A halo word tags its value with the solve count in 16 bits, which
    wraps every 65,536 solves; the library zeroes the words before that.
    65,100 short multi-CTA solves with varying sweep counts (so varying
    numbers of halo exchanges), each from a fresh potential, keep giving the
    oracle's potential bit for bit, across the clearing."""
    monkeypatch.setenv("CUPIC_JACOBI_DEPTH", "2")
    sim, ora = make_pair("tiny", ctas=4)
    sim.init_plasma()
    ora.init_plasma()
    base = ora.phi()
    rng = np.random.default_rng(9)
    for k in range(65100):
        n = 2 + k % 5
        if k % 1000 == 0 or k >= 64990:
            phi0 = base + 1e-3 * rng.standard_normal(base.shape)
            phi0[:, -1] = phi0[:, 0]
            phi0 = phi0.astype(np.float32).astype(np.float64)
            sim.set_phi(phi0)
            ora.set_phi(phi0)
        sim.poisson_solver(1e-30, n, n, n)
        if k % 1000 == 0 or k >= 64990:
            ora.solve(1e-30, n, n, n)
            np.testing.assert_array_equal(sim.phi().astype(np.float64), ora.phi(), err_msg=f"solve {k}")
