"""The Poisson solve that allocates nothing (cupic_poisson_solver_static).

Some callers of this library cannot allocate device memory at the moment they
need a solve:
- real-time loops that forbid allocation after start-up, since an allocation
  can block for an unbounded time;
- applications whose device memory all comes from their own pool.
They pass their own charge, potential and field buffers, and the solver's
scratch is a static device array inside the library.

Each case checks, through the C-ABI, two calls in a row of the static entry
point against the context's own solver (cupic_poisson_solver +
cupic_field_solver) on the same charge and starting potential. The
tolerance is the 1e-5 relative one the parity tests use. Both paths run the
same kernel, so they also agree bit for bit.
"""
import ctypes

import numpy as np
import pytest

import cupic_gb300 as cg

pytestmark = pytest.mark.gpu

RTOL = 1e-5


def rel_err(got, ref):
    got = np.asarray(got, dtype=np.float64)
    ref = np.asarray(ref, dtype=np.float64)
    return float(np.abs(got - ref).max() / max(np.abs(ref).max(), 1e-30))


CASES = [
    # (workload, overrides, forced CTA count): one CTA, a few CTAs, and the
    # default many-CTA plan with temporal blocking
    ("tiny", {}, None),
    ("small", {}, "6"),
    ("small", {"ncx": 128, "ncy": 512, "n": 16.0, "eps0": 16.0, "max_sweeps": 300}, None),
]


@pytest.mark.parametrize("name,over,ctas", CASES)
def test_static_solve_matches_context_solver(gpu_lib, monkeypatch, name, over, ctas):
    torch = pytest.importorskip("torch")
    if ctas:
        monkeypatch.setenv("CUPIC_JACOBI_CTAS", ctas)
    else:
        monkeypatch.delenv("CUPIC_JACOBI_CTAS", raising=False)
    L = cg.load_library()
    p = cg.workload_params(name, **over)
    sim = cg.Sim(p)
    try:
        sim.init_plasma()
        sim.step(2)
        nn = p.nnx * p.nny
        rho = np.ascontiguousarray(sim.rho_fixed(0).ravel(), dtype=np.int64)
        phi = np.ascontiguousarray(sim.phi().ravel(), dtype=np.float32)
        d_rho = torch.from_numpy(rho).to("cuda")
        d_phi = torch.from_numpy(phi.copy()).to("cuda")
        d_e = torch.zeros(2 * nn, dtype=torch.float32, device="cuda")
        torch.cuda.synchronize()
        tol, mn, mx, chk = p.tol, p.min_sweeps, min(p.max_sweeps, 300), p.check_every
        for call in range(2):
            sweeps, res = ctypes.c_int32(), ctypes.c_float()
            rc = L.cupic_poisson_solver_static(
                ctypes.byref(p), d_rho.data_ptr(), d_phi.data_ptr(), d_e.data_ptr(), tol, mn, mx,
                chk, None, ctypes.byref(sweeps), ctypes.byref(res))
            assert rc == 0, f"call {call}: {cg.strerror(rc)}"
            assert 1 <= sweeps.value <= mx
            sim.poisson_solver(tol, mn, mx, chk)
            sim.field_solver()
            ref_phi = sim.phi().ravel()
            ref_ex, ref_ey = sim.efield()
            got_phi = d_phi.cpu().numpy()
            got_e = d_e.cpu().numpy().reshape(-1, 2)
            assert rel_err(got_phi, ref_phi) <= RTOL, f"phi, call {call}"
            assert rel_err(got_e[:, 0], ref_ex.ravel()) <= RTOL, f"Ex, call {call}"
            assert rel_err(got_e[:, 1], ref_ey.ravel()) <= RTOL, f"Ey, call {call}"
            np.testing.assert_array_equal(got_phi, ref_phi)
    finally:
        sim.close()


def test_static_solve_rejects_meshes_beyond_its_scratch(gpu_lib):
    """A mesh whose exchange scratch exceeds the static 8 MiB is refused
    before anything runs on the device."""
    torch = pytest.importorskip("torch")
    L = cg.load_library()
    p = cg.workload_params("tiny", ncx=4096, ncy=200)
    nn = p.nnx * p.nny
    d_rho = torch.zeros(nn, dtype=torch.int64, device="cuda")
    d_phi = torch.zeros(nn, dtype=torch.float32, device="cuda")
    rc = L.cupic_poisson_solver_static(ctypes.byref(p), d_rho.data_ptr(), d_phi.data_ptr(), None,
                                       1e-6, 1, 10, 1, None, None, None)
    assert rc == 5  # CUPIC_ERR_CAPACITY
