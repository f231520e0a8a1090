"""The FP32 path against FP64 arithmetic on identical inputs.

The parity tests hold the GPU to the FP32 oracle, which shares the GPU's
quantisation: 18-bit fixed-point CIC weights per axis and FP32 Jacobi
sweeps.  Here one state -- the GPU's own after set-up and two steps -- goes
into the FP64 oracle, which computes with the reference's arithmetic (exact
CIC weights as in mesh.cu:196-240, FP64 Jacobi as in mesh.cu:327-350, FP64
field and push as in mesh.cu:413-468 and particles.cu:145-225), and one
cycle's stages run on both:
  charge deposition           -> rho
  S Jacobi sweeps from the same potential -> phi
  field derivation            -> Ex, Ey
  one push (gather + leapfrog + wrap + row binning) -> x, y, vx, vy
Errors are normwise, max |gpu - fp64| / max |fp64| over each array.  The
pushed particles are paired row by row; a particle within rounding of a row
boundary can be binned into the next row in the other run, so each
particle is paired with its nearest neighbour among its row and the two
beside it (parity.pair_rows): every row of the 64x256 workload, and 32 rows
spread over the 2048 of the 512x2048 one (1.6 million particles per
species).

The contract is 1e-5.  Charge, potential, positions and velocities meet it
on both workloads.  The field of the plain FP32 path meets it on the
64x256 workload, but not on the 512x2048 one: there the potential spans
|phi_p| = 5 Te/e over 2048 rows, so E is small (|E| < 0.1) while every
stored FP32 potential carries a rounding error near ulp(5)/2 = 2.4e-7, which
the central difference turns into an absolute field error of the same size
-- a few 1e-5 of |E|, whatever the solver does.  The precision form, which
holds phi in FP64 and derives E in FP64, meets the contract there
(test_precision_form_meets_the_field_contract).  Every measured error is
printed.
"""
import numpy as np
import pytest

import cupic_gb300 as cg
from oracle.oracle import Oracle
from parity import RTOL, pair_rows, rel_err

pytestmark = pytest.mark.gpu

# field error of the plain FP32 path at 512x2048: FP32 storage of phi bounds
# it (see above); measured 2-3e-5
E_BOUND_FP32_LARGE = 1e-4


def run_stages(sim, o64, sweeps, tag, rows=None):
    """Deposit, solve, field and push on both sides from one state; returns
    {quantity: relative error}.  rows: the rows whose pushed particles are
    compared (all by default)."""
    err = {}
    sim.charge_deposition()
    o64.deposit()
    err["rho"] = rel_err(sim.rho(0), o64.rho(0))
    sim.poisson_solver(0.0, sweeps, sweeps, sweeps)
    o64.solve(0.0, sweeps, sweeps, sweeps)
    err["phi"] = rel_err(sim.phi(), o64.phi())
    sim.field_solver()
    o64.field()
    (gx, gy), (ox, oy) = sim.efield(), o64.efield()
    err["Ex"] = rel_err(gx, ox)
    err["Ey"] = rel_err(gy, oy)
    mag = float(np.sqrt(ox ** 2 + oy ** 2).max())
    err["E"] = float(max(np.abs(gx - ox).max(), np.abs(gy - oy).max()) / mag)
    del gx, gy, ox, oy
    sim.particle_mover()
    o64.push(0)
    for sp in (0, 1):
        g, o = pair_rows(sim.particles(sp), sim.row_counts(sp), o64.particles(sp),
                         o64.row_counts(sp), rows)
        for c, name in enumerate(("x", "y", "vx", "vy")):
            err[f"{name}{sp}"] = rel_err(g[:, c], o[:, c])
        del g, o
    print(f"\n{tag}: " + ", ".join(f"{k} {v:.2e}" for k, v in err.items()))
    return err


@pytest.mark.parametrize("name,sweeps", [("small", 400), ("large", 200)])
def test_fp32_path_against_fp64_arithmetic(gpu_lib, name, sweeps):
    pytest.importorskip("scipy")
    p = cg.workload_params(name)
    with cg.Sim(p) as sim:
        sim.init_plasma()
        sim.step(2)
        o64 = Oracle(p, fp64=True)
        for sp in (0, 1):
            o64.load(sp, sim.particles(sp))
        o64.set_phi(sim.phi().astype(np.float64))
        rows = None if p.ncy <= 256 else np.linspace(0, p.ncy - 1, 32).astype(int)
        err = run_stages(sim, o64, sweeps, f"{name} FP32 path vs FP64", rows)
        o64.close()
    for k in ("rho", "phi", "x0", "y0", "vx0", "vy0", "x1", "y1", "vx1", "vy1"):
        assert err[k] <= RTOL, f"{k}: {err[k]:.3e}"
    if name == "small":
        for k in ("Ex", "Ey"):
            assert err[k] <= RTOL, f"{k}: {err[k]:.3e}"
    else:
        assert err["E"] <= E_BOUND_FP32_LARGE, f"E: {err['E']:.3e}"


def test_precision_form_meets_the_field_contract(gpu_lib):
    """The precision form (FP32 sweeps on a correction, FP64 residual and
    update every 32 sweeps, FP64 potential, field derived in FP64) at
    512x2048: after 320 sweeps from one state its potential and field agree
    with 320 plain FP64 Jacobi sweeps to well within 1e-5."""
    pytest.importorskip("scipy")
    p = cg.workload_params("precision")
    with cg.Sim(p) as sim:
        sim.init_plasma()
        sim.step(1)
        o64 = Oracle(p, fp64=True)
        for sp in (0, 1):
            o64.load(sp, sim.particles(sp))
        phi0 = sim.phi64()
        sim.set_phi(phi0)
        o64.set_phi(phi0)
        sim.charge_deposition()
        o64.deposit()
        sim.poisson_solver(0.0, 320, 320, 32)
        o64.solve(0.0, 320, 320, 32)
        e_phi = rel_err(sim.phi64(), o64.phi())
        sim.field_solver()
        o64.field()
        (gx, gy), (ox, oy) = sim.efield(), o64.efield()
        e_ex, e_ey = rel_err(gx, ox), rel_err(gy, oy)
        o64.close()
    print(f"\nprecision form vs FP64 at 512x2048: phi {e_phi:.2e}, Ex {e_ex:.2e}, Ey {e_ey:.2e}")
    assert e_phi <= RTOL and e_ex <= RTOL and e_ey <= RTOL
